// Stress test of the resident host-copy pool: several threads run copy sets
// of random sizes (below and above the parallel threshold) and functions over
// numbered pieces at once; every byte must arrive, every piece must run
// exactly once, and every run must return.
#include <cstdio>
#include <atomic>
#include <cstdlib>
#include <random>
#include <thread>
#include <vector>

#include "copy_pool.h"

int main(int argc, char** argv) {
  const int iters = argc > 1 ? std::atoi(argv[1]) : 1000;
  const int helpers = argc > 2 ? std::atoi(argv[2]) : 7;
  clue::CopyPool pool;
  pool.start(helpers);
  std::atomic<int> bad{0};
  auto client = [&](int seed) {
    std::mt19937 rng(seed);
    for (int it = 0; it < iters; ++it) {
      const int nt = 1 + (int)(rng() % 6);
      std::vector<std::vector<char>> src(nt), dst(nt);
      std::vector<clue::CopyTask> tasks;
      for (int k = 0; k < nt; ++k) {
        const size_t n = (rng() % 4) == 0 ? rng() % 3000000 : rng() % 200000;
        src[k].resize(n);
        dst[k].assign(n, 0);
        for (size_t b = 0; b < n; b += 4093) src[k][b] = (char)(b * 7 + k + it);
        tasks.push_back({dst[k].data(), src[k].data(), n});
      }
      pool.run(tasks);
      for (int k = 0; k < nt; ++k)
        if (src[k] != dst[k]) bad++;
      // a function over numbered pieces: every piece runs exactly once
      const size_t np = rng() % 300;
      std::vector<std::atomic<int>> hits(np);
      for (auto& hh : hits) hh = 0;
      pool.for_pieces(np, [&](size_t i) { hits[i].fetch_add(1); });
      for (auto& hh : hits)
        if (hh.load() != 1) bad++;
    }
  };
  std::vector<std::thread> th;
  for (int c = 0; c < 3; ++c) th.emplace_back(client, c + 1);
  for (auto& t : th) t.join();
  pool.stop();
  std::printf("mismatches %d\n", bad.load());
  return bad.load() != 0;
}
