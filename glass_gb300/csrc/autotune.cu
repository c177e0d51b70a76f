// Launch-shape autotuner (see autotune.cuh).
#include "autotune.cuh"

#include <cstdlib>
#include <cstring>
#include <mutex>

namespace gg {

namespace {

struct Entry {
  std::string kernel, shape;
  std::vector<std::string> names;
  std::vector<float> ms;
  int choice = 0;
};

std::mutex g_mutex;
std::vector<Entry> g_entries;
int g_enabled = -1;  // -1: not read from the environment yet

bool enabled_locked() {
  if (g_enabled < 0) {
    const char* env = std::getenv("GG_AUTOTUNE");
    g_enabled = (env && std::strcmp(env, "0") == 0) ? 0 : 1;
  }
  return g_enabled != 0;
}

Entry* find_locked(const std::string& kernel, const std::string& shape) {
  for (Entry& e : g_entries)
    if (e.kernel == kernel && e.shape == shape) return &e;
  return nullptr;
}

}  // namespace

int autotune_choose(const std::string& kernel, const std::string& shape, const std::vector<std::string>& names,
                    int fallback, cudaStream_t stream, const std::function<void(int)>& launch) {
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (const Entry* e = find_locked(kernel, shape)) return e->choice;
    if (!enabled_locked() || names.size() < 2) return fallback;
  }
  cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
  check_cuda(cudaStreamIsCapturing(stream, &capture), "cudaStreamIsCapturing");
  if (capture != cudaStreamCaptureStatusNone) return fallback;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  check_cuda(cudaEventCreate(&e0), "cudaEventCreate(autotune)");
  check_cuda(cudaEventCreate(&e1), "cudaEventCreate(autotune)");
  Entry entry;
  entry.kernel = kernel;
  entry.shape = shape;
  entry.names = names;
  try {
    for (int i = 0; i < static_cast<int>(names.size()); ++i) {
      launch(i);  // warm: instruction cache, L2, clocks
      check_cuda(cudaEventRecord(e0, stream), "cudaEventRecord(autotune)");
      launch(i);
      launch(i);
      check_cuda(cudaEventRecord(e1, stream), "cudaEventRecord(autotune)");
      check_cuda(cudaEventSynchronize(e1), "cudaEventSynchronize(autotune)");
      float ms = 0.0f;
      check_cuda(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime(autotune)");
      entry.ms.push_back(ms / 2.0f);
    }
  } catch (...) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    throw;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  int best = 0;
  for (int i = 1; i < static_cast<int>(entry.ms.size()); ++i)
    if (entry.ms[i] < entry.ms[best]) best = i;
  entry.choice = best;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (const Entry* e = find_locked(kernel, shape)) return e->choice;
  g_entries.push_back(entry);
  return best;
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_autotune_set_enabled(int enabled) {
  std::lock_guard<std::mutex> lock(g_mutex);
  g_enabled = enabled ? 1 : 0;
  return GG_OK;
}

int gg_autotune_clear(void) {
  std::lock_guard<std::mutex> lock(g_mutex);
  g_entries.clear();
  return GG_OK;
}

int gg_autotune_count(int32_t* out) {
  if (!out) return GG_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(g_mutex);
  *out = static_cast<int32_t>(g_entries.size());
  return GG_OK;
}

int gg_autotune_entry(int32_t index, char* kernel, size_t kernel_len, char* shape, size_t shape_len,
                      char* choice, size_t choice_len, float* best_ms, int32_t* candidates) {
  std::lock_guard<std::mutex> lock(g_mutex);
  if (index < 0 || index >= static_cast<int32_t>(g_entries.size())) return GG_ERR_OUT_OF_RANGE;
  const Entry& e = g_entries[static_cast<size_t>(index)];
  auto put = [](char* dst, size_t len, const std::string& src) {
    if (!dst || len == 0) return;
    const size_t n = std::min(len - 1, src.size());
    std::memcpy(dst, src.data(), n);
    dst[n] = '\0';
  };
  put(kernel, kernel_len, e.kernel);
  put(shape, shape_len, e.shape);
  put(choice, choice_len, e.names[static_cast<size_t>(e.choice)]);
  if (best_ms) *best_ms = e.ms[static_cast<size_t>(e.choice)];
  if (candidates) *candidates = static_cast<int32_t>(e.names.size());
  return GG_OK;
}

}  // extern "C"
