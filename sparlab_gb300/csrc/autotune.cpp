// Launch-shape autotuner (see autotune.h).
#include "autotune.h"

#include <atomic>
#include <cstdlib>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>

namespace simp {
namespace {

std::mutex g_mu;
std::map<std::string, TuneRecord> g_table;
bool g_file_read = false;
std::atomic<bool> g_enabled{true};

const char* cache_path() { return std::getenv("SIMP_TUNE_CACHE"); }

void read_file_locked() {
  if (g_file_read) return;
  g_file_read = true;
  const char* path = cache_path();
  if (!path) return;
  std::ifstream in(path);
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream ls(line);
    std::string key;
    int v = -1;
    if (ls >> key >> v && v >= 0) {
      TuneRecord r;
      r.key = key;
      r.chosen = v;
      g_table[key] = r;
    }
  }
}

void append_file(const std::string& key, int v) {
  const char* path = cache_path();
  if (!path) return;
  std::ofstream out(path, std::ios::app);
  out << key << ' ' << v << '\n';
}

}  // namespace

void tune_set_enabled(bool on) { g_enabled = on; }

void tune_set(const std::string& key, int variant) {
  std::lock_guard<std::mutex> lock(g_mu);
  read_file_locked();
  TuneRecord r;
  r.key = key;
  r.chosen = variant;
  g_table[key] = r;
}
bool tune_enabled() { return g_enabled; }

std::vector<TuneRecord> tune_records() {
  std::lock_guard<std::mutex> lock(g_mu);
  std::vector<TuneRecord> out;
  for (const auto& kv : g_table) out.push_back(kv.second);
  return out;
}

int tune_pick(const std::string& key, int count, const std::function<void(int)>& run, cudaStream_t stream,
              int fallback, int reps) {
  if (!g_enabled || count <= 1) return fallback;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    read_file_locked();
    auto it = g_table.find(key);
    if (it != g_table.end() && it->second.chosen < count) return it->second.chosen;
  }
  // never time inside a stream capture (the launches would only be recorded)
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  SIMP_CUDA(cudaStreamIsCapturing(stream, &cs));
  if (cs != cudaStreamCaptureStatusNone) return fallback;
  TuneRecord rec;
  rec.key = key;
  cudaEvent_t e0, e1;
  SIMP_CUDA(cudaEventCreate(&e0));
  SIMP_CUDA(cudaEventCreate(&e1));
  double best = 0.0;
  for (int v = 0; v < count; ++v) {
    run(v);  // untimed first launch
    SIMP_CUDA(cudaEventRecord(e0, stream));
    for (int r = 0; r < reps; ++r) run(v);
    SIMP_CUDA(cudaEventRecord(e1, stream));
    SIMP_CUDA(cudaEventSynchronize(e1));
    float ms = 0.0f;
    SIMP_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    const double per = static_cast<double>(ms) / reps;
    rec.ms.push_back(per);
    if (v == 0 || per < best) {
      best = per;
      rec.chosen = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  {
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_table.find(key);
    if (it != g_table.end()) return it->second.chosen;  // another thread tuned it meanwhile
    g_table[key] = rec;
  }
  append_file(key, rec.chosen);
  return rec.chosen;
}

}  // namespace simp
