// Entry points whose implementation is still being written.
#include "../../include/clue.h"
#include "clue_runtime.h"

using clue::set_error;

extern "C" {

void clue3d_default_params(clue3d_params* p) {
  p->n_layers = 94;
  p->density_sibling_layers = 3;
  p->density_xy_distance_sqr = 3.24f;
  p->kernel_density_factor = 0.2f;
  p->density_on_same_layer = 0;
  p->nh_sibling_layers = 3;
  p->nh_on_same_layer = 0;
  p->critical_xy_distance = 1.8f;
  p->critical_z_distance_lyr = 5.f;
  p->critical_density = 0.6f;
  p->critical_self_density = 0.15f;
  p->outlier_multiplier = 2.f;
}

int clue3d_run_batch(clue_handle*, const clue3d_params*, int32_t, const int64_t*, const clue3d_inputs*,
                     const clue3d_outputs*, int32_t*, int) {
  return set_error(CLUE_EINVAL, "clue3d_run_batch: not available in this build");
}

int clue_server_create(const clue_params*, const clue_server_config*, clue_server**) {
  return set_error(CLUE_EINVAL, "serving: not available in this build");
}
int clue_server_destroy(clue_server*) { return CLUE_OK; }
int clue_server_submit(clue_server*, int32_t, const float*, const float*, const int32_t*, const float*,
                       const clue_outputs*, int64_t*) {
  return set_error(CLUE_EINVAL, "serving: not available in this build");
}
int clue_server_poll(clue_server*, int64_t, int32_t, double*) { return set_error(CLUE_EINVAL, "serving"); }
int clue_server_drain(clue_server*, int32_t) { return set_error(CLUE_EINVAL, "serving"); }
int clue_server_get_stats(clue_server*, clue_server_stats*) { return set_error(CLUE_EINVAL, "serving"); }
int clue_server_reset_stats(clue_server*) { return set_error(CLUE_EINVAL, "serving"); }

}  // extern "C"
