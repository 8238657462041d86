// Entry points whose implementation is still being written.
#include "../../include/clue.h"
#include "clue_runtime.h"

using clue::set_error;

extern "C" {

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
