// Launch-shape autotuner.
//
// Some kernels have several launch shapes that compute exactly the same
// values: the tile shape of the matrix-free operator (each node's sum runs
// over the same cells and corners in the same order whatever the tile), and
// the shared-memory budget per block of the Galerkin row products (each row
// node's products run in one warp in the same order whatever the warps per
// block).  For those, the tuner times every variant on the problem's own data
// with CUDA events the first time a shape key is seen, keeps the fastest, and
// reuses the choice for later launches with the same key.  Because the
// variants agree bit for bit, tuning changes the speed, never the results.
//
// Choices live in a process-wide table; with the environment variable
// SIMP_TUNE_CACHE naming a file they are also read from and appended to it,
// so later processes skip the timing.  Tuning launches are never issued
// inside a stream capture.
#pragma once

#include "common.h"

#include <functional>
#include <string>
#include <vector>

namespace simp {

struct TuneRecord {
  std::string key;
  int chosen = 0;
  std::vector<double> ms;  // per variant (empty when the choice came from the cache file)
};

// Index of the fastest of `count` variants for `key`; `run(v)` launches
// variant v on `stream`.  Each variant runs once untimed and `reps` times
// timed.  Disabled tuning (set_enabled(false)) returns `fallback`.
int tune_pick(const std::string& key, int count, const std::function<void(int)>& run, cudaStream_t stream,
              int fallback, int reps = 3);

// Records `variant` as the choice for `key` (replacing a tuned one).
void tune_set(const std::string& key, int variant);
void tune_set_enabled(bool on);
bool tune_enabled();
std::vector<TuneRecord> tune_records();

}  // namespace simp
