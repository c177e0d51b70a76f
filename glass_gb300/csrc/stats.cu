// Frame statistics (frame weights) and the standalone DQ-map builder.
//
// frame_global_stats: mean/std/valid count of the finite samples of a frame
// (reference: native_bindings.cpp:10569-10640 over
// local_norm_kernels.cu:73-117, float64 sums).  Used for the simple_snr frame
// weight |mean|/std (resident_cuda.py:1948-1956).  Here every thread keeps
// float-float sums of v and v^2 (TwoSum/TwoProd), a warp folds them with
// shuffles, and each CTA writes one (sum, sum2, count) triple of doubles; the
// host adds the partials.  One launch covers all requested frames
// (grid.y = frame).
#include <cmath>
#include <vector>

#include "stack.cuh"

namespace gg {

__device__ __forceinline__ void ff_merge(FF& a, const FF& b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  a.hi = s;
  a.lo = __fadd_rn(__fadd_rn(a.lo, b.lo), e);
}

__global__ void __launch_bounds__(256) frame_stats_kernel(const float* slots, const int* slot_of_frame, int64_t stride,
                                                          int64_t pixels, const int* frames, double* partials) {
  const int frame = frames[blockIdx.y];
  const float* src = slots + static_cast<int64_t>(slot_of_frame[frame]) * stride;
  // Two independent accumulator pairs over float4 loads (slots are 256 B
  // aligned), then the scalar tail.
  FF s1, s2, t1, t2;
  unsigned count = 0;
  const int64_t quads = pixels / 4;
  const float4* src4 = reinterpret_cast<const float4*>(src);
  for (int64_t q = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; q < quads; q += int64_t(gridDim.x) * blockDim.x) {
    const float4 v = __ldcs(src4 + q);
    if (isfinite(v.x)) { s1.add(v.x); s2.add_prod(v.x, v.x); ++count; }
    if (isfinite(v.y)) { t1.add(v.y); t2.add_prod(v.y, v.y); ++count; }
    if (isfinite(v.z)) { s1.add(v.z); s2.add_prod(v.z, v.z); ++count; }
    if (isfinite(v.w)) { t1.add(v.w); t2.add_prod(v.w, v.w); ++count; }
  }
  for (int64_t p = quads * 4 + blockIdx.x * int64_t(blockDim.x) + threadIdx.x; p < pixels;
       p += int64_t(gridDim.x) * blockDim.x) {
    const float v = src[p];
    if (isfinite(v)) { s1.add(v); s2.add_prod(v, v); ++count; }
  }
  ff_merge(s1, t1);
  ff_merge(s2, t2);
  for (int off = 16; off > 0; off >>= 1) {
    FF o1, o2;
    o1.hi = __shfl_xor_sync(0xffffffffu, s1.hi, off);
    o1.lo = __shfl_xor_sync(0xffffffffu, s1.lo, off);
    o2.hi = __shfl_xor_sync(0xffffffffu, s2.hi, off);
    o2.lo = __shfl_xor_sync(0xffffffffu, s2.lo, off);
    count += __shfl_xor_sync(0xffffffffu, count, off);
    ff_merge(s1, o1);
    ff_merge(s2, o2);
  }
  __shared__ double sh[3][8];
  const int warp = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    sh[0][warp] = static_cast<double>(s1.hi) + static_cast<double>(s1.lo);
    sh[1][warp] = static_cast<double>(s2.hi) + static_cast<double>(s2.lo);
    sh[2][warp] = static_cast<double>(count);
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double t = 0.0;
    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) t += sh[threadIdx.x][w];
    partials[(static_cast<int64_t>(blockIdx.y) * gridDim.x + blockIdx.x) * 3 + threadIdx.x] = t;
  }
}

// simple_snr weights from the per-CTA partials (resident_cuda.py:1948-1956):
//   valid == 0 -> 0;  std <= eps -> 1/eps;  else max(|mean|/std, eps)
// A frame whose prior weight is not finite and positive keeps weight 0
// (zero-weight frames are skipped, resident_cuda.py:12766-12770); otherwise
// the prior multiplies the SNR weight in float64 (the registration-agreement
// multiplier, resident_cuda.py:12800-12804).
// One warp per frame: lanes fold the CTA partials, then a shuffle reduction.
__global__ void snr_weights_kernel(const double* partials, int blocks, const int* frames, int count,
                                   const float* prior, float eps, int mode, float* weights) {
  const int k = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (k >= count) return;
  const int f = frames[k];
  const float pw = prior ? prior[k] : 1.0f;
  if (!(isfinite(pw) && pw > 0.0f) || mode == 0) {
    if (lane == 0) weights[f] = (isfinite(pw) && pw > 0.0f) ? pw : 0.0f;
    return;
  }
  double sum = 0.0, sum2 = 0.0, n = 0.0;
  for (int b = lane; b < blocks; b += 32) {
    const double* q = partials + (static_cast<int64_t>(k) * blocks + b) * 3;
    sum += q[0];
    sum2 += q[1];
    n += q[2];
  }
  for (int off = 16; off > 0; off >>= 1) {
    sum += __shfl_xor_sync(0xffffffffu, sum, off);
    sum2 += __shfl_xor_sync(0xffffffffu, sum2, off);
    n += __shfl_xor_sync(0xffffffffu, n, off);
  }
  if (lane != 0) return;
  if (n <= 0.0) {
    weights[f] = 0.0f;
    return;
  }
  const double mean = sum / n;
  double var = sum2 / n - mean * mean;
  if (var < 0.0) var = 0.0;
  const double sd = sqrt(var);
  const double e = static_cast<double>(eps);
  const double w = sd <= e ? 1.0 / e : fmax(fabs(mean) / sd, e);
  weights[f] = static_cast<float>(w * static_cast<double>(pw));
}

// Per-CTA (sum, sum2, count) partials of the given frames (device frame list).
void launch_frame_stats_partials(gg_stack* s, const int* d_frames, int count, int blocks, double* partials) {
  note_launch();
  frame_stats_kernel<<<dim3(blocks, static_cast<unsigned>(count)), 256, 0, s->stream>>>(
      s->d_slots, s->d_slot_of_frame, s->stride, s->pixels, d_frames, partials);
  check_cuda(cudaGetLastError(), "frame_stats kernel launch");
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_stack_compute_weights(gg_stack* s, int mode, const float* host_prior, float eps, float* host_weights_out) {
  GG_API_BEGIN
  require(s != nullptr, "stack is null");
  require(mode == GG_WEIGHTS_PRIOR || mode == GG_WEIGHTS_SIMPLE_SNR, "unsupported weighting mode");
  require(eps > 0.0f && std::isfinite(eps), "eps must be positive");
  stack_require_all_loaded(s, "frame weighting");
  stack_activate(s);
  const int64_t count = s->frames;
  const int blocks = static_cast<int>(std::min<int64_t>(sm_count() * 2, (s->pixels + 255) / 256));
  const size_t partial_doubles = static_cast<size_t>(count) * blocks * 3;
  // partials | frame list (ints) | prior weights (floats)
  stack_ensure_partials(s, partial_doubles + static_cast<size_t>(count));
  int* d_frames = reinterpret_cast<int*>(s->d_partials + partial_doubles);
  float* d_prior = reinterpret_cast<float*>(d_frames + count);
  int* h_frames = reinterpret_cast<int*>(s->h_partials_pinned + partial_doubles);
  float* h_prior = reinterpret_cast<float*>(h_frames + count);
  for (int64_t k = 0; k < count; ++k) {
    h_frames[k] = static_cast<int>(k);
    h_prior[k] = host_prior ? host_prior[k] : 1.0f;
  }
  upload_params(s->stream, d_frames, h_frames, sizeof(int) * count * 2, "cudaMemcpyAsync(weights frames)");
  if (mode == GG_WEIGHTS_SIMPLE_SNR) {
    note_launch();
    frame_stats_kernel<<<dim3(blocks, static_cast<unsigned>(count)), 256, 0, s->stream>>>(
        s->d_slots, s->d_slot_of_frame, s->stride, s->pixels, d_frames, s->d_partials);
    check_cuda(cudaGetLastError(), "frame_stats kernel launch");
  }
  note_launch();
  snr_weights_kernel<<<static_cast<unsigned>((count + 3) / 4), 128, 0, s->stream>>>(
      s->d_partials, blocks, d_frames, static_cast<int>(count), d_prior, eps, mode, s->d_weights);
  check_cuda(cudaGetLastError(), "snr_weights kernel launch");
  if (host_weights_out) {
    check_cuda(cudaMemcpyAsync(s->h_weights_pinned, s->d_weights, sizeof(float) * count, cudaMemcpyDeviceToHost,
                               s->stream),
               "cudaMemcpyAsync(weights out)");
    check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(weights)");
    std::copy(s->h_weights_pinned, s->h_weights_pinned + count, host_weights_out);
  }
  GG_API_END
}

int gg_stack_frame_stats(gg_stack* s, const int64_t* indices, int64_t count, gg_frame_stats_t* out) {
  GG_API_BEGIN
  require(s != nullptr && indices != nullptr && out != nullptr, "null argument");
  require(count > 0 && count <= 65535, "frame count for statistics must be in [1, 65535]");
  for (int64_t k = 0; k < count; ++k) stack_require_loaded(s, indices[k], "global frame statistics");
  stack_activate(s);
  const int blocks = static_cast<int>(std::min<int64_t>(sm_count() * 2, (s->pixels + 255) / 256));
  const size_t need = static_cast<size_t>(count) * blocks * 3 + static_cast<size_t>(count);
  stack_ensure_partials(s, need);
  // Frame list goes in the tail of the partial buffer (as ints).
  int* d_frames = reinterpret_cast<int*>(s->d_partials + static_cast<size_t>(count) * blocks * 3);
  std::vector<int> frames(static_cast<size_t>(count));
  for (int64_t k = 0; k < count; ++k) frames[static_cast<size_t>(k)] = static_cast<int>(indices[k]);
  int* h_frames = reinterpret_cast<int*>(s->h_partials_pinned + static_cast<size_t>(count) * blocks * 3);
  std::copy(frames.begin(), frames.end(), h_frames);
  upload_params(s->stream, d_frames, h_frames, sizeof(int) * count, "cudaMemcpyAsync(stats frames)");
  note_launch();
  frame_stats_kernel<<<dim3(blocks, static_cast<unsigned>(count)), 256, 0, s->stream>>>(
      s->d_slots, s->d_slot_of_frame, s->stride, s->pixels, d_frames, s->d_partials);
  check_cuda(cudaGetLastError(), "frame_stats kernel launch");
  check_cuda(cudaMemcpyAsync(s->h_partials_pinned, s->d_partials, sizeof(double) * count * blocks * 3,
                             cudaMemcpyDeviceToHost, s->stream),
             "cudaMemcpyAsync(stats partials)");
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(stats)");
  for (int64_t k = 0; k < count; ++k) {
    double sum = 0.0, sum2 = 0.0, n = 0.0;
    for (int b = 0; b < blocks; ++b) {
      const double* q = s->h_partials_pinned + (static_cast<size_t>(k) * blocks + b) * 3;
      sum += q[0];
      sum2 += q[1];
      n += q[2];
    }
    const double mean = n > 0 ? sum / n : 0.0;
    double var = 0.0;
    if (n > 0) {
      var = sum2 / n - mean * mean;
      if (var < 0.0) var = 0.0;
    }
    out[k].mean = mean;
    out[k].std = std::sqrt(var);
    out[k].valid_pixels = static_cast<int64_t>(n);
    out[k].total_pixels = s->pixels;
  }
  GG_API_END
}

int gg_dq_map_i16(const float* host_master, const float* host_weight, const float* host_coverage,
                  const float* host_low, const float* host_high, const float* host_geometric, int64_t n,
                  int64_t active_frame_count, int16_t* host_dq) {
  GG_API_BEGIN
  // Host routine: the maps are already on the host when the caller asks for a
  // DQ map (resident_cuda.py:3110-3297); the fused device version runs inside
  // the integrator.
  require(host_master != nullptr && host_weight != nullptr && host_dq != nullptr, "null argument");
  require(n >= 0, "n must be non-negative");
  for (int64_t i = 0; i < n; ++i) {
    int bits = 0;
    const float m = host_master[i], w = host_weight[i];
    bool invalid = !std::isfinite(m) || !std::isfinite(w) || !(w > 0.0f);
    if (host_coverage) {
      const float c = host_coverage[i];
      if (!std::isfinite(c) || c <= 0.5f) {
        bits |= 64;
        invalid = true;
      }
    }
    if (host_geometric) {
      const float g = host_geometric[i];
      if (!std::isfinite(g) || g <= 0.5f) {
        bits |= 64;
        invalid = true;
      } else if (active_frame_count > 0 && g < static_cast<float>(static_cast<double>(active_frame_count) - 0.5)) {
        bits |= 64;
      }
    }
    if (invalid) bits |= 1;
    if (host_low && std::isfinite(host_low[i]) && host_low[i] > 0.0f) bits |= 256;
    if (host_high && std::isfinite(host_high[i]) && host_high[i] > 0.0f) bits |= 512;
    host_dq[i] = static_cast<int16_t>(bits);
  }
  GG_API_END
}

}  // extern "C"
