// Frame statistics for callers that must not allocate device memory.
//
// gg_frames_stats_f32_noalloc computes the same per-frame mean / std / valid
// count as gg_stack_frame_stats (the simple_snr weight inputs), for frames
// that already live in device memory the caller owns.  Some callers cannot
// call cudaMalloc at all: plugins whose host application owns every device
// allocation through its own pool, and real-time loops that forbid allocation
// after start-up.  This entry point therefore uses no allocation of any kind:
// its reduction scratch is a file-scope __device__ array of fixed size
// (kNoAllocMaxFrames x kNoAllocBlocks partial sums plus one folded triple per
// frame, 193.5 KiB), which every GPU that loads this library keeps reserved
// until the process exits.
//
// Rules for callers:
//   - at most kNoAllocMaxFrames (64) frames per call; more is rejected with
//     GG_ERR_INVALID_ARGUMENT;
//   - the first call on each device resolves the device address of the
//     scratch array (cudaGetSymbolAddress) and caches it per device ordinal;
//     after cudaDeviceReset (or any reset of the primary context) that cached
//     address is stale, so do not call this entry point again in a process
//     that has reset the device;
//   - `stream` must belong to the device the frames live on (the device is
//     taken from the stream; the legacy default stream means the current
//     device);
//   - the call copies its results to the host and synchronises `stream`, so
//     it cannot run while `stream` is being captured into a CUDA graph: such
//     a call is rejected with GG_ERR_INVALID_ARGUMENT before anything is
//     enqueued, and the caller's capture stays valid;
//   - all calls share the one scratch array, so calls whose work overlaps on
//     the GPU (different streams or host threads) race; serialise them.  Every
//     call rewrites every partial and result it reads, so nothing needs
//     clearing between calls.
#include <cmath>
#include <mutex>

#include "stack.cuh"

namespace gg {

constexpr int kNoAllocMaxFrames = 64;
constexpr int kNoAllocBlocks = 128;  // CTAs per frame

// [frame][block][sum, sum2, count], then [frame][sum, sum2, count] folded
constexpr int kNoAllocPartials = kNoAllocMaxFrames * kNoAllocBlocks * 3;
static __device__ __align__(256) double g_noalloc_partials[kNoAllocPartials + kNoAllocMaxFrames * 3];

__global__ void __launch_bounds__(256) noalloc_frame_stats_kernel(const float* frames, int64_t pixels,
                                                                  int64_t frame_stride, double* partials) {
  const float* src = frames + static_cast<int64_t>(blockIdx.y) * frame_stride;
  FF s1, s2;
  unsigned count = 0;
  for (int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; p < pixels; p += int64_t(gridDim.x) * blockDim.x) {
    const float v = src[p];
    if (isfinite(v)) {
      s1.add(v);
      s2.add_prod(v, v);
      ++count;
    }
  }
  // Each warp folds its float-float sums in double (exact for these sizes).
  double d1 = static_cast<double>(s1.hi) + static_cast<double>(s1.lo);
  double d2 = static_cast<double>(s2.hi) + static_cast<double>(s2.lo);
  double dn = static_cast<double>(count);
  for (int off = 16; off > 0; off >>= 1) {
    d1 += __shfl_xor_sync(0xffffffffu, d1, off);
    d2 += __shfl_xor_sync(0xffffffffu, d2, off);
    dn += __shfl_xor_sync(0xffffffffu, dn, off);
  }
  __shared__ double sh[3][8];
  const int warp = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    sh[0][warp] = d1;
    sh[1][warp] = d2;
    sh[2][warp] = dn;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double t = 0.0;
    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) t += sh[threadIdx.x][w];
    partials[(static_cast<int64_t>(blockIdx.y) * gridDim.x + blockIdx.x) * 3 + threadIdx.x] = t;
  }
}

// One warp per frame folds the CTA partials into (sum, sum2, count) and
// writes them to the frame's triple in the compact result region `folded`.
__global__ void noalloc_fold_kernel(const double* partials, int blocks, int count, double* folded) {
  const int frame = blockIdx.x;
  const int lane = threadIdx.x;
  if (frame >= count) return;
  double s = 0.0, s2 = 0.0, n = 0.0;
  for (int b = lane; b < blocks; b += 32) {
    const double* q = partials + (static_cast<int64_t>(frame) * blocks + b) * 3;
    s += q[0];
    s2 += q[1];
    n += q[2];
  }
  for (int off = 16; off > 0; off >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, off);
    s2 += __shfl_xor_sync(0xffffffffu, s2, off);
    n += __shfl_xor_sync(0xffffffffu, n, off);
  }
  __syncwarp();
  if (lane == 0) {
    double* q = folded + static_cast<int64_t>(frame) * 3;
    q[0] = s;
    q[1] = s2;
    q[2] = n;
  }
}

// Device address of g_noalloc_partials, resolved once per device.  Host code
// must not pass the symbol itself to a kernel: on the host it names a shadow
// variable, not device memory.
static double* noalloc_scratch(int device) {
  static std::mutex mu;
  static double* addr[64] = {nullptr};
  if (device < 0 || device >= 64) fail(GG_ERR_INVALID_ARGUMENT, "device index out of range for the no-alloc path");
  std::lock_guard<std::mutex> lock(mu);
  if (addr[device] == nullptr) {
    void* p = nullptr;
    check_cuda(cudaGetSymbolAddress(&p, g_noalloc_partials), "cudaGetSymbolAddress(no-alloc scratch)");
    addr[device] = static_cast<double*>(p);
  }
  return addr[device];
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_frames_stats_f32_noalloc(const float* dev_frames, int64_t frame_count, int64_t pixels, int64_t frame_stride,
                                void* cuda_stream, gg_frame_stats_t* out) {
  GG_API_BEGIN
  require(dev_frames != nullptr && out != nullptr, "null argument");
  require(frame_count >= 1, "frame_count must be at least 1");
  require(frame_count <= kNoAllocMaxFrames,
          "gg_frames_stats_f32_noalloc handles at most 64 frames per call (fixed scratch size)");
  require(pixels >= 1, "pixels must be positive");
  require(frame_stride >= pixels, "frame_stride must be at least pixels");
  auto stream = static_cast<cudaStream_t>(cuda_stream);
  // The results are copied back and the stream synchronised, neither of which
  // a capturing stream allows: refuse before enqueuing anything so that the
  // caller's capture is not invalidated.
  cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
  check_cuda(cudaStreamIsCapturing(stream, &capture), "cudaStreamIsCapturing");
  require(capture == cudaStreamCaptureStatusNone,
          "gg_frames_stats_f32_noalloc cannot run on a stream that is being captured");
  int device = 0;
  if (stream != nullptr) {
    check_cuda(cudaStreamGetDevice(stream, &device), "cudaStreamGetDevice");
  } else {
    check_cuda(cudaGetDevice(&device), "cudaGetDevice");
  }
  int current = 0;
  check_cuda(cudaGetDevice(&current), "cudaGetDevice");
  require(device == current, "the stream of gg_frames_stats_f32_noalloc must belong to the current device");
  double* scratch = noalloc_scratch(device);
  double* folded = scratch + kNoAllocPartials;
  note_launch();
  noalloc_frame_stats_kernel<<<dim3(kNoAllocBlocks, static_cast<unsigned>(frame_count)), 256, 0, stream>>>(
      dev_frames, pixels, frame_stride, scratch);
  check_cuda(cudaGetLastError(), "noalloc_frame_stats launch");
  note_launch();
  noalloc_fold_kernel<<<static_cast<unsigned>(frame_count), 32, 0, stream>>>(scratch, kNoAllocBlocks,
                                                                           static_cast<int>(frame_count), folded);
  check_cuda(cudaGetLastError(), "noalloc_fold launch");
  double sums[kNoAllocMaxFrames * 3];
  check_cuda(cudaMemcpyAsync(sums, folded, static_cast<size_t>(frame_count) * 3 * sizeof(double),
                             cudaMemcpyDeviceToHost, stream),
             "cudaMemcpyAsync(no-alloc statistics)");
  check_cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize(no-alloc statistics)");
  for (int64_t k = 0; k < frame_count; ++k) {
    const double n = sums[k * 3 + 2];
    const double mean = n > 0 ? sums[k * 3] / n : 0.0;
    double var = n > 0 ? sums[k * 3 + 1] / n - mean * mean : 0.0;
    if (var < 0.0) var = 0.0;
    out[k].mean = mean;
    out[k].std = std::sqrt(var);
    out[k].valid_pixels = static_cast<int64_t>(n);
    out[k].total_pixels = pixels;
  }
  GG_API_END
}

}  // extern "C"
