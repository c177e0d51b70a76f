// Resident stack lifecycle, host<->device transfers and the library-level
// entry points of the C ABI (include/glass_gb300.h).
//
// Reference counterparts: the pybind11 class ResidentCalibratedStack
// (cpp/src/native_bindings.cpp:2915-3080 ctor/dtor/accounting, 15118-15130
// index/loaded checks, 5979-8865 calibration entry points) and the module
// functions cuda_available / get_device_info / host_pinned_empty_*.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <mutex>

#include "sampling.cuh"
#include "stack.cuh"

namespace gg {

namespace {
thread_local int g_last_code = GG_OK;
thread_local std::string g_last_message;
}  // namespace

void set_last_error(int code, const char* msg) {
  g_last_code = code;
  g_last_message = msg ? msg : "";
}

static std::atomic<long long> g_launches{0};
void note_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

namespace {
template <unsigned BYTES>
struct ParamBlock {
  unsigned char* dst;
  unsigned bytes;
  alignas(16) unsigned char data[BYTES];
};

// Writes the block carried in the launch parameters to its destination;
// whole 32-bit words when the destination and the size allow it.
template <unsigned BYTES>
__global__ void __launch_bounds__(256) param_block_kernel(const __grid_constant__ ParamBlock<BYTES> b) {
  if ((reinterpret_cast<uintptr_t>(b.dst) & 3u) == 0 && (b.bytes & 3u) == 0) {
    const unsigned* src = reinterpret_cast<const unsigned*>(b.data);
    unsigned* dst = reinterpret_cast<unsigned*>(b.dst);
    for (unsigned i = threadIdx.x; i < b.bytes / 4; i += blockDim.x) dst[i] = src[i];
  } else {
    for (unsigned i = threadIdx.x; i < b.bytes; i += blockDim.x) b.dst[i] = b.data[i];
  }
}

template <unsigned BYTES>
void launch_param_block(cudaStream_t stream, unsigned char* dst, const unsigned char* src, unsigned bytes,
                        const char* what) {
  ParamBlock<BYTES> b;
  b.dst = dst;
  b.bytes = bytes;
  std::memcpy(b.data, src, bytes);
  note_launch();
  param_block_kernel<BYTES><<<1, 256, 0, stream>>>(b);
  check_cuda(cudaGetLastError(), what);
}
}  // namespace

void upload_params(cudaStream_t stream, void* dst, const void* src, std::size_t bytes, const char* what) {
  if (bytes == 0) return;
  if (bytes > kParamUploadMax) {
    check_cuda(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream), what);
    return;
  }
  // 16 KB blocks stay well inside the 32,764-byte kernel parameter limit
  constexpr unsigned kLarge = 16384, kSmall = 1024;
  auto* d = static_cast<unsigned char*>(dst);
  const auto* h = static_cast<const unsigned char*>(src);
  for (std::size_t off = 0; off < bytes; off += kLarge) {
    const unsigned n = static_cast<unsigned>(std::min<std::size_t>(kLarge, bytes - off));
    if (n <= kSmall) launch_param_block<kSmall>(stream, d + off, h + off, n, what);
    else launch_param_block<kLarge>(stream, d + off, h + off, n, what);
  }
}

int sm_count() {
  static int cached = 0;
  if (cached == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 148;
    cached = n;
  }
  return cached;
}

void stack_activate(gg_stack* s) { check_cuda(cudaSetDevice(s->device), "cudaSetDevice"); }

void stack_require_index(const gg_stack* s, int64_t index) {
  if (index < 0 || index >= s->frames) fail(GG_ERR_OUT_OF_RANGE, "resident frame index is out of range");
}

void stack_require_loaded(const gg_stack* s, int64_t index, const char* what) {
  stack_require_index(s, index);
  if (!s->loaded[static_cast<size_t>(index)]) {
    fail(GG_ERR_RUNTIME, std::string("resident frame must be loaded before ") + what);
  }
}

void stack_require_all_loaded(const gg_stack* s, const char* what) {
  if (s->loaded_count != s->frames) {
    fail(GG_ERR_RUNTIME, std::string("all resident frames must be loaded before ") + what);
  }
}

void stack_mark_loaded(gg_stack* s, int64_t index) {
  if (!s->loaded[static_cast<size_t>(index)]) {
    s->loaded[static_cast<size_t>(index)] = 1;
    ++s->loaded_count;
  }
}

void stack_read_slots(gg_stack* s, std::vector<int>& out) {
  out.resize(static_cast<size_t>(s->frames));
  check_cuda(cudaMemcpyAsync(s->h_slot_table_pinned, s->d_slot_of_frame, sizeof(int) * s->frames,
                             cudaMemcpyDeviceToHost, s->stream),
             "cudaMemcpyAsync(slot table)");
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(slot table)");
  std::copy(s->h_slot_table_pinned, s->h_slot_table_pinned + s->frames, out.begin());
}

static void* device_alloc(gg_stack* s, size_t bytes, const char* what) {
  void* p = nullptr;
  const cudaError_t err = cudaMalloc(&p, bytes);
  if (err != cudaSuccess) {
    cudaGetLastError();
    fail(GG_ERR_OUT_OF_MEMORY, std::string("cudaMalloc(") + what + ") of " + std::to_string(bytes) +
                                   " bytes failed: " + cudaGetErrorString(err));
  }
  s->bytes_allocated += static_cast<int64_t>(bytes);
  return p;
}

static void* pinned_alloc(gg_stack* s, size_t bytes, const char* what) {
  void* p = nullptr;
  check_cuda(cudaHostAlloc(&p, bytes, cudaHostAllocPortable), what);
  s->host_pinned_bytes += static_cast<int64_t>(bytes);
  return p;
}

void stack_ensure_maps(gg_stack* s) {
  if (s->d_master != nullptr) return;
  const size_t p = static_cast<size_t>(s->pixels);
  s->d_master = static_cast<float*>(device_alloc(s, p * 4, "master map"));
  s->d_weight = static_cast<float*>(device_alloc(s, p * 4, "weight map"));
  s->d_coverage = device_alloc(s, p * 4, "coverage map");
  s->d_low = device_alloc(s, p * 4, "low rejection map");
  s->d_high = device_alloc(s, p * 4, "high rejection map");
  s->d_dq = static_cast<int16_t*>(device_alloc(s, p * 2, "dq map"));
}

void stack_check_device_error(gg_stack* s) {
  int err = 0;
  check_cuda(cudaMemcpyAsync(&err, s->d_error, sizeof(int), cudaMemcpyDeviceToHost, s->stream),
             "cudaMemcpyAsync(device error)");
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(device error)");
  if (err != 0) {
    check_cuda(cudaMemsetAsync(s->d_error, 0, sizeof(int), s->stream), "cudaMemsetAsync(device error)");
    check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(device error)");
    fail(GG_ERR_TIMEOUT, "a device-side wait ran out of its iteration limit (result of the last batch is invalid)");
  }
}

void stack_ensure_partials(gg_stack* s, size_t doubles) {
  if (s->partial_capacity >= doubles) return;
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(partials)");
  if (s->d_partials) {
    cudaFree(s->d_partials);
    s->bytes_allocated -= static_cast<int64_t>(s->partial_capacity * sizeof(double));
  }
  if (s->h_partials_pinned) {
    cudaFreeHost(s->h_partials_pinned);
    s->host_pinned_bytes -= static_cast<int64_t>(s->partial_capacity * sizeof(double));
  }
  s->d_partials = nullptr;
  s->h_partials_pinned = nullptr;
  s->partial_capacity = 0;
  s->d_partials = static_cast<double*>(device_alloc(s, doubles * sizeof(double), "reduction partials"));
  s->h_partials_pinned = static_cast<double*>(pinned_alloc(s, doubles * sizeof(double), "cudaHostAlloc(partials)"));
  s->partial_capacity = doubles;
}

static void stack_free(gg_stack* s) {
  if (!s) return;
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->copy_stream) cudaStreamSynchronize(s->copy_stream);
  if (s->star_scratch && s->star_scratch_free) s->star_scratch_free(s->star_scratch);
  if (s->reg_scratch && s->reg_scratch_free) s->reg_scratch_free(s->reg_scratch);
  if (s->metric_scratch && s->metric_scratch_free) s->metric_scratch_free(s->metric_scratch);
  if (s->gn_scratch && s->gn_scratch_free) s->gn_scratch_free(s->gn_scratch);
  if (s->step_graph && s->step_graph_free) s->step_graph_free(s->step_graph);
  if (s->ln_scratch && s->ln_scratch_free) s->ln_scratch_free(s->ln_scratch);
  if (s->raw_stage && s->raw_stage_free) s->raw_stage_free(s->raw_stage);
  void* dev_ptrs[] = {s->d_slots,    s->d_slot_of_frame, s->d_spare_slot, s->d_frame_nonfinite,
                      s->d_bias,     s->d_dark,          s->d_flat,       s->d_master,
                      s->d_weight,   s->d_coverage,      s->d_low,        s->d_high,
                      s->d_dq,       s->d_warp_coverage, s->d_weights,    s->d_partials,
                      s->d_raw_lane[0], s->d_raw_lane[1], s->d_warp_items, s->d_error,
                      s->d_cat_xy,   s->d_cat_n,         s->d_fused_frames, s->d_fused_counts,
                      s->d_fused_geometric};
  for (void* p : dev_ptrs) {
    if (p) cudaFree(p);
  }
  if (s->warp_items_free) cudaEventDestroy(s->warp_items_free);
  void* host_ptrs[] = {s->h_pinned_lane[0], s->h_pinned_lane[1], s->h_weights_pinned, s->h_partials_pinned,
                       s->h_slot_table_pinned, s->h_warp_items};
  for (void* p : host_ptrs) {
    if (p) cudaFreeHost(p);
  }
  for (int i = 0; i < gg_stack::kLanes; ++i) {
    if (s->lane_free[i]) cudaEventDestroy(s->lane_free[i]);
    if (s->lane_ready[i]) cudaEventDestroy(s->lane_ready[i]);
  }
  if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
  if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
  delete s;
}

__global__ void init_slot_tables_kernel(int* slot_of_frame, int frames, int* spare, int spares) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < frames) slot_of_frame[i] = i;
  if (i < spares) spare[i] = frames + i;
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_version(int* version) {
  GG_API_BEGIN
  require(version != nullptr, "version pointer is null");
  *version = 10000;
  GG_API_END
}

int gg_kernel_launches(int64_t* count) {
  GG_API_BEGIN
  require(count != nullptr, "count pointer is null");
  *count = static_cast<int64_t>(g_launches.load(std::memory_order_relaxed));
  GG_API_END
}

int gg_last_error(char* buf, size_t cap) {
  if (buf && cap > 0) {
    const size_t n = std::min(cap - 1, g_last_message.size());
    std::memcpy(buf, g_last_message.data(), n);
    buf[n] = '\0';
  }
  return g_last_code;
}

int gg_cuda_available(int* available) {
  GG_API_BEGIN
  require(available != nullptr, "available pointer is null");
  int n = 0;
  const cudaError_t err = cudaGetDeviceCount(&n);
  if (err != cudaSuccess) cudaGetLastError();
  *available = (err == cudaSuccess && n > 0) ? 1 : 0;
  GG_API_END
}

int gg_device_count(int* count) {
  GG_API_BEGIN
  require(count != nullptr, "count pointer is null");
  int n = 0;
  const cudaError_t err = cudaGetDeviceCount(&n);
  if (err != cudaSuccess) {
    cudaGetLastError();
    n = 0;
  }
  *count = n;
  GG_API_END
}

int gg_device_info(int device, gg_device_info_t* info) {
  GG_API_BEGIN
  require(info != nullptr, "info pointer is null");
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    fail(GG_ERR_NO_DEVICE, "no CUDA device is available");
  }
  if (device < 0 || device >= n) fail(GG_ERR_OUT_OF_RANGE, "device index is out of range");
  cudaDeviceProp prop{};
  check_cuda(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
  std::memset(info, 0, sizeof(*info));
  std::snprintf(info->name, sizeof(info->name), "%s", prop.name);
  info->major = prop.major;
  info->minor = prop.minor;
  info->multiprocessor_count = prop.multiProcessorCount;
  info->total_global_mem = static_cast<int64_t>(prop.totalGlobalMem);
  info->l2_cache_bytes = static_cast<int64_t>(prop.l2CacheSize);
  info->shared_mem_per_block_optin = static_cast<int64_t>(prop.sharedMemPerBlockOptin);
  GG_API_END
}

int gg_host_alloc_pinned(size_t bytes, void** host_ptr) {
  GG_API_BEGIN
  require(host_ptr != nullptr, "host_ptr is null");
  *host_ptr = nullptr;
  check_cuda(cudaHostAlloc(host_ptr, bytes > 0 ? bytes : 1, cudaHostAllocPortable), "cudaHostAlloc");
  GG_API_END
}

int gg_host_free_pinned(void* host_ptr) {
  GG_API_BEGIN
  if (host_ptr) check_cuda(cudaFreeHost(host_ptr), "cudaFreeHost");
  GG_API_END
}

int gg_stack_create(int64_t frame_count, int64_t height, int64_t width, gg_stack** out) {
  GG_API_BEGIN
  require(out != nullptr, "out pointer is null");
  *out = nullptr;
  require(frame_count > 0, "frame_count must be positive");
  require(height > 0 && width > 0, "height and width must be positive");
  require(frame_count < (1 << 20), "frame_count is too large");
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    fail(GG_ERR_NO_DEVICE, "no CUDA device is available");
  }
  gg_stack* s = new gg_stack();
  try {
    check_cuda(cudaGetDevice(&s->device), "cudaGetDevice");
    s->frames = frame_count;
    s->height = height;
    s->width = width;
    s->pixels = height * width;
    s->stride = (s->pixels + 63) / 64 * 64;
    // Spare slots receive warp outputs.  Small stacks get one spare per frame
    // (a whole stack warps in one launch); large stacks cap the spare memory.
    const int64_t frame_bytes = s->stride * 4;
    int64_t spares = std::min<int64_t>(frame_count, 16);
    if (frame_bytes * frame_count <= (int64_t(2) << 30)) spares = frame_count;
    s->spares = std::max<int64_t>(spares, 1);
    s->slots = s->frames + s->spares;
    s->loaded.assign(static_cast<size_t>(frame_count), 0);

    check_cuda(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    s->own_stream = true;
    check_cuda(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking), "cudaStreamCreate(copy)");
    for (int i = 0; i < gg_stack::kLanes; ++i) {
      check_cuda(cudaEventCreateWithFlags(&s->lane_free[i], cudaEventDisableTiming), "cudaEventCreate");
      check_cuda(cudaEventCreateWithFlags(&s->lane_ready[i], cudaEventDisableTiming), "cudaEventCreate");
    }

    const size_t slot_bytes = static_cast<size_t>(s->slots) * static_cast<size_t>(s->stride) * 4;
    s->d_slots = static_cast<float*>(device_alloc(s, slot_bytes, "resident stack slots"));
    s->d_slot_of_frame = static_cast<int*>(device_alloc(s, sizeof(int) * frame_count, "slot table"));
    s->d_spare_slot = static_cast<int*>(device_alloc(s, sizeof(int) * s->spares, "spare slot table"));
    s->d_frame_nonfinite = static_cast<unsigned*>(device_alloc(s, sizeof(unsigned) * frame_count, "nonfinite counters"));
    s->d_weights = static_cast<float*>(device_alloc(s, sizeof(float) * frame_count, "weights"));
    s->h_weights_pinned = static_cast<float*>(pinned_alloc(s, sizeof(float) * frame_count, "cudaHostAlloc(weights)"));
    s->h_slot_table_pinned = static_cast<int*>(pinned_alloc(s, sizeof(int) * frame_count, "cudaHostAlloc(slots)"));
    s->d_error = static_cast<int*>(device_alloc(s, sizeof(int), "device error word"));
    check_cuda(cudaMemsetAsync(s->d_error, 0, sizeof(int), s->stream), "cudaMemsetAsync(error)");
    check_cuda(cudaEventCreateWithFlags(&s->warp_items_free, cudaEventDisableTiming), "cudaEventCreate");
    s->has_slot_tmap = (s->width % 4 == 0) && make_slot_tensor_map(s, kBoxW, kBoxH);

    check_cuda(cudaMemsetAsync(s->d_slots, 0, slot_bytes, s->stream), "cudaMemsetAsync(stack)");
    check_cuda(cudaMemsetAsync(s->d_frame_nonfinite, 0, sizeof(unsigned) * frame_count, s->stream),
               "cudaMemsetAsync(nonfinite)");
    const int64_t m = std::max(frame_count, s->spares);
    note_launch();
    init_slot_tables_kernel<<<static_cast<unsigned>((m + 255) / 256), 256, 0, s->stream>>>(
        s->d_slot_of_frame, static_cast<int>(frame_count), s->d_spare_slot, static_cast<int>(s->spares));
    check_cuda(cudaGetLastError(), "init_slot_tables_kernel launch");
    check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(create)");
  } catch (...) {
    stack_free(s);
    throw;
  }
  *out = s;
  GG_API_END
}

int gg_stack_destroy(gg_stack* stack) {
  GG_API_BEGIN
  stack_free(stack);
  GG_API_END
}

int gg_stack_info(const gg_stack* s, gg_stack_info_t* info) {
  GG_API_BEGIN
  require(s != nullptr && info != nullptr, "null argument");
  std::memset(info, 0, sizeof(*info));
  info->frame_count = s->frames;
  info->height = s->height;
  info->width = s->width;
  info->pixels_per_frame = s->pixels;
  info->frame_stride = s->stride;
  info->slot_count = s->slots;
  info->loaded_count = s->loaded_count;
  info->bytes_allocated = s->bytes_allocated;
  info->warp_scratch_bytes = s->spares * s->stride * 4;
  info->host_pinned_bytes = s->host_pinned_bytes;
  info->calibration_lane_count = s->d_raw_lane[0] ? gg_stack::kLanes : 0;
  info->warp_coverage_frame_count = s->warp_coverage_frames;
  info->has_bias = s->has_bias;
  info->has_dark = s->has_dark;
  info->has_flat = s->has_flat;
  GG_API_END
}

int gg_stack_set_stream(gg_stack* s, void* cuda_stream) {
  GG_API_BEGIN
  require(s != nullptr, "stack is null");
  stack_activate(s);
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(set_stream)");
  if (cuda_stream == nullptr) {
    if (!s->own_stream) {
      check_cuda(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "cudaStreamCreate");
      s->own_stream = true;
    }
  } else {
    if (s->own_stream) cudaStreamDestroy(s->stream);
    s->stream = static_cast<cudaStream_t>(cuda_stream);
    s->own_stream = false;
  }
  GG_API_END
}

int gg_stack_synchronize(gg_stack* s) {
  GG_API_BEGIN
  require(s != nullptr, "stack is null");
  stack_activate(s);
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
  stack_check_device_error(s);
  GG_API_END
}

int gg_stack_set_masters(gg_stack* s, const float* host_bias, const float* host_dark, const float* host_flat) {
  GG_API_BEGIN
  require(s != nullptr, "stack is null");
  stack_activate(s);
  const size_t bytes = static_cast<size_t>(s->pixels) * 4;
  struct Item {
    const float* src;
    float** dst;
    bool* has;
    const char* name;
  } items[] = {{host_bias, &s->d_bias, &s->has_bias, "master bias"},
               {host_dark, &s->d_dark, &s->has_dark, "master dark"},
               {host_flat, &s->d_flat, &s->has_flat, "master flat"}};
  for (auto& it : items) {
    if (it.src == nullptr) {
      *it.has = false;
      continue;
    }
    if (*it.dst == nullptr) *it.dst = static_cast<float*>(device_alloc(s, bytes, it.name));
    check_cuda(cudaMemcpyAsync(*it.dst, it.src, bytes, cudaMemcpyHostToDevice, s->stream), "cudaMemcpyAsync(master)");
    *it.has = true;
  }
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(masters)");
  GG_API_END
}

int gg_stack_upload_frame(gg_stack* s, int64_t index, const float* host_frame) {
  GG_API_BEGIN
  require(s != nullptr && host_frame != nullptr, "null argument");
  stack_require_index(s, index);
  stack_activate(s);
  std::vector<int> slots;
  stack_read_slots(s, slots);
  float* dst = s->d_slots + static_cast<size_t>(slots[static_cast<size_t>(index)]) * s->stride;
  check_cuda(cudaMemcpyAsync(dst, host_frame, static_cast<size_t>(s->pixels) * 4, cudaMemcpyHostToDevice, s->stream),
             "cudaMemcpyAsync(upload frame)");
  launch_count_nonfinite(s, index);
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(upload)");
  stack_mark_loaded(s, index);
  GG_API_END
}

int gg_stack_download_frames_tile(gg_stack* s, const int64_t* indices, int64_t count, int64_t x0, int64_t y0,
                                  int64_t x1, int64_t y1, float* host_out) {
  GG_API_BEGIN
  require(s != nullptr && indices != nullptr && host_out != nullptr, "null argument");
  require(count > 0, "indices must contain at least one frame index");
  require(0 <= x0 && x0 < x1 && x1 <= s->width && 0 <= y0 && y0 < y1 && y1 <= s->height,
          "tile bounds are outside the resident frame");
  stack_activate(s);
  std::vector<int> slots;
  stack_read_slots(s, slots);
  const size_t tw = static_cast<size_t>(x1 - x0);
  const size_t th = static_cast<size_t>(y1 - y0);
  for (int64_t k = 0; k < count; ++k) {
    stack_require_loaded(s, indices[k], "download");
    const float* src = s->d_slots + static_cast<size_t>(slots[static_cast<size_t>(indices[k])]) * s->stride +
                       static_cast<size_t>(y0) * s->width + static_cast<size_t>(x0);
    check_cuda(cudaMemcpy2DAsync(host_out + static_cast<size_t>(k) * tw * th, tw * 4, src,
                                 static_cast<size_t>(s->width) * 4, tw * 4, th, cudaMemcpyDeviceToHost, s->stream),
               "cudaMemcpy2DAsync(download tile)");
  }
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(download)");
  GG_API_END
}

int gg_stack_download_frame_tile(gg_stack* s, int64_t index, int64_t x0, int64_t y0, int64_t x1, int64_t y1,
                                 float* host_out) {
  return gg_stack_download_frames_tile(s, &index, 1, x0, y0, x1, y1, host_out);
}

int gg_stack_device_ptrs(gg_stack* s, gg_stack_device_ptrs_t* out) {
  GG_API_BEGIN
  require(s != nullptr && out != nullptr, "null argument");
  std::memset(out, 0, sizeof(*out));
  out->slots = s->d_slots;
  out->slot_of_frame = s->d_slot_of_frame;
  out->master = s->d_master;
  out->weight = s->d_weight;
  out->coverage = s->d_coverage;
  out->low = s->d_low;
  out->high = s->d_high;
  out->dq = s->d_dq;
  out->warp_coverage = s->d_warp_coverage;
  GG_API_END
}

int gg_stack_download_weights(gg_stack* s, float* host_out) {
  GG_API_BEGIN
  require(s != nullptr && host_out != nullptr, "null argument");
  stack_activate(s);
  check_cuda(cudaMemcpyAsync(s->h_weights_pinned, s->d_weights, sizeof(float) * s->frames, cudaMemcpyDeviceToHost,
                             s->stream),
             "cudaMemcpyAsync(weights)");
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(weights)");
  std::copy(s->h_weights_pinned, s->h_weights_pinned + s->frames, host_out);
  GG_API_END
}

int gg_stack_frame_device_ptr(gg_stack* s, int64_t index, float** out) {
  GG_API_BEGIN
  require(s != nullptr && out != nullptr, "null argument");
  stack_require_loaded(s, index, "frame_device_ptr");
  stack_activate(s);
  std::vector<int> slots;
  stack_read_slots(s, slots);  // synchronises the stack's stream
  *out = s->d_slots + static_cast<int64_t>(slots[static_cast<size_t>(index)]) * s->stride;
  GG_API_END
}

}  // extern "C"
