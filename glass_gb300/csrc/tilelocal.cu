// Tile-local weighted integration: integrate_tile_local_mean and
// integrate_tile_local_sigma_clip (integration_kernels.cu:1658-1711,
// 3622-3796; native_bindings.cpp:12998-13210, 14337-14630).
//
// Per pixel, the weight of every target frame is multiplied by the
// multiplier of the first (tiles do not overlap) tile whose half-open extent
// [x0, x1) x [y0, y1) contains the pixel (1 outside every tile).  A sample
// takes part when its effective weight is > 0 and finite and the sample is
// finite.
//   mean:        master = sum(w v) / sum(w), weight = sum(w)
//   sigma clip:  mean / population std of the taking-part samples
//                (unweighted); winsorized: the mean / std of the samples
//                clipped to mean -/+ k std replace them; samples outside
//                centre -/+ k scale are rejected (low / high counts), the
//                rest are averaged with their weights.
// Arithmetic is float32 in frame order, one rounding per operation (the
// reference's CUDA kernels may contract a += b * c into one fused
// multiply-add; the restatement in oracle/tile_local.py is this sequence).
//
// GB300 layout: one thread per pixel, the pixel's column staged once in
// shared memory ([frame][thread], bank-conflict free) so the up to five
// passes of the sigma clip read on-chip memory instead of re-reading HBM
// (the reference streams the column from global memory on every pass).
#include <cmath>
#include <cstring>
#include <vector>

#include "stack.cuh"

namespace gg {

constexpr int kTlThreads = 128;
constexpr int kTlMaxFrames = 128;
constexpr int kTlMaxTiles = 2048;

struct TileLocalArgs {
  const float* slots;
  const int* slot_of_frame;
  int64_t stride;
  int width, height, frames;
  const float* weights;          // [frames]
  const unsigned char* target;   // [frames]
  const int4* tiles;             // [tile_count] (x0, y0, x1, y1)
  const float* multipliers;      // [tile_count]
  int tile_count;
  int mode;                      // 0 mean, 1 sigma clip, 2 winsorized sigma clip
  float low_sigma, high_sigma;
  float *master, *weight, *coverage, *low, *high;
};

__global__ void __launch_bounds__(kTlThreads) tile_local_kernel(TileLocalArgs a) {
  extern __shared__ float col[];  // [frames][kTlThreads]
  __shared__ float s_w[kTlMaxFrames];
  __shared__ unsigned char s_t[kTlMaxFrames];
  __shared__ const float* s_base[kTlMaxFrames];
  for (int f = threadIdx.x; f < a.frames; f += blockDim.x) {
    s_w[f] = a.weights[f];
    s_t[f] = a.target[f];
    s_base[f] = a.slots + static_cast<int64_t>(a.slot_of_frame[f]) * a.stride;
  }
  __syncthreads();
  const int tid = threadIdx.x;
  float* C = col + tid;
  const int64_t P = static_cast<int64_t>(a.width) * a.height;
  for (int64_t p = static_cast<int64_t>(blockIdx.x) * kTlThreads + tid; p < P;
       p += static_cast<int64_t>(gridDim.x) * kTlThreads) {
    const int y = static_cast<int>(p / a.width), x = static_cast<int>(p - static_cast<int64_t>(y) * a.width);
    float mult = 1.0f;
    for (int t = 0; t < a.tile_count; ++t) {
      const int4 e = __ldg(a.tiles + t);
      if (x >= e.x && x < e.z && y >= e.y && y < e.w) {
        mult = __ldg(a.multipliers + t);
        break;
      }
    }
    // stage the column; a NaN marks a sample that does not take part
    const float kNaN = __int_as_float(0x7fc00000);
    for (int f = 0; f < a.frames; ++f) {
      const float w = s_t[f] ? __fmul_rn(s_w[f], mult) : s_w[f];
      const float v = __ldcs(s_base[f] + p);
      C[f * kTlThreads] = (w > 0.0f && isfinite(w) && isfinite(v)) ? v : kNaN;
    }
    float master = 0.0f, wsum = 0.0f, cov = 0.0f, lowc = 0.0f, highc = 0.0f;
    float lt = -__int_as_float(0x7f800000), ht = __int_as_float(0x7f800000);
    bool ok = true;
    if (a.mode != 0) {
      float mean = 0.0f, count = 0.0f;
      for (int f = 0; f < a.frames; ++f) {
        const float v = C[f * kTlThreads];
        if (v == v) {
          mean = __fadd_rn(mean, v);
          count = __fadd_rn(count, 1.0f);
        }
      }
      if (count <= 0.0f) {
        ok = false;
      } else {
        mean = __fdiv_rn(mean, count);
        float var = 0.0f;
        for (int f = 0; f < a.frames; ++f) {
          const float v = C[f * kTlThreads];
          if (v == v) {
            const float d = __fsub_rn(v, mean);
            var = __fadd_rn(var, __fmul_rn(d, d));
          }
        }
        float center = mean, scale = __fsqrt_rn(__fdiv_rn(var, count));
        lt = __fsub_rn(center, __fmul_rn(a.low_sigma, scale));
        ht = __fadd_rn(center, __fmul_rn(a.high_sigma, scale));
        if (a.mode == 2) {
          float wm = 0.0f;
          for (int f = 0; f < a.frames; ++f) {
            float v = C[f * kTlThreads];
            if (v == v) wm = __fadd_rn(wm, v < lt ? lt : (v > ht ? ht : v));
          }
          wm = __fdiv_rn(wm, count);
          float wv = 0.0f;
          for (int f = 0; f < a.frames; ++f) {
            float v = C[f * kTlThreads];
            if (v == v) {
              const float d = __fsub_rn(v < lt ? lt : (v > ht ? ht : v), wm);
              wv = __fadd_rn(wv, __fmul_rn(d, d));
            }
          }
          center = wm;
          scale = __fsqrt_rn(__fdiv_rn(wv, count));
          lt = __fsub_rn(center, __fmul_rn(a.low_sigma, scale));
          ht = __fadd_rn(center, __fmul_rn(a.high_sigma, scale));
        }
      }
    }
    if (ok) {
      float sum = 0.0f;
      for (int f = 0; f < a.frames; ++f) {
        const float v = C[f * kTlThreads];
        if (!(v == v)) continue;
        if (a.mode != 0) {
          if (v < lt) {
            lowc = __fadd_rn(lowc, 1.0f);
            continue;
          }
          if (v > ht) {
            highc = __fadd_rn(highc, 1.0f);
            continue;
          }
        }
        const float w = s_t[f] ? __fmul_rn(s_w[f], mult) : s_w[f];
        sum = __fadd_rn(sum, __fmul_rn(v, w));
        wsum = __fadd_rn(wsum, w);
        cov = __fadd_rn(cov, 1.0f);
      }
      master = wsum > 0.0f ? __fdiv_rn(sum, wsum) : 0.0f;
    }
    a.master[p] = master;
    a.weight[p] = wsum;
    if (a.mode != 0) {
      a.coverage[p] = cov;
      a.low[p] = lowc;
      a.high[p] = highc;
    }
  }
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_stack_integrate_tile_local(gg_stack* s, int mode, const float* host_weights,
                                  const uint8_t* host_target_mask, const int32_t* host_tile_extents,
                                  const float* host_multipliers, int32_t tile_count, float low_sigma,
                                  float high_sigma) {
  GG_API_BEGIN
  require(s != nullptr && host_target_mask != nullptr && host_tile_extents != nullptr && host_multipliers != nullptr,
          "null argument");
  require(mode >= 0 && mode <= 2, "mode must be 0 (mean), 1 (sigma clip) or 2 (winsorized sigma clip)");
  require(s->frames <= kTlMaxFrames, "tile-local integration takes at most 128 frames");
  require(s->width <= (int64_t{1} << 30) && s->height <= (int64_t{1} << 30),
          "resident tile-local integration requires image dimensions within int range");
  stack_require_all_loaded(s, "tile-local integration");
  if (mode != 0) require(low_sigma > 0.0f && high_sigma > 0.0f, "sigma thresholds must be positive");
  int targets = 0;
  for (int64_t f = 0; f < s->frames; ++f) targets += host_target_mask[f] != 0;
  require(targets > 0, "target_mask must select at least one resident frame");
  require(tile_count >= 1 && tile_count <= kTlMaxTiles, "tile_extents must contain between 1 and 2048 tiles");
  for (int t = 0; t < tile_count; ++t) {
    const int32_t* e = host_tile_extents + 4 * t;
    require(e[0] >= 0 && e[1] >= 0 && e[2] > e[0] && e[3] > e[1] && e[2] <= s->width && e[3] <= s->height,
            "tile_extents must be positive half-open rectangles inside the image");
    require(std::isfinite(host_multipliers[t]) && host_multipliers[t] >= 0.0f,
            "tile_multipliers must be finite non-negative values");
    for (int u = 0; u < t; ++u) {
      const int32_t* o = host_tile_extents + 4 * u;
      require(!(std::max(e[0], o[0]) < std::min(e[2], o[2]) && std::max(e[1], o[1]) < std::min(e[3], o[3])),
              "tile_extents must not overlap for deterministic tile-local integration");
    }
  }
  stack_activate(s);
  stack_ensure_maps(s);
  const int n = static_cast<int>(s->frames);
  // small per-call parameter block in stream-ordered memory
  const size_t bytes = sizeof(float) * n + n + sizeof(int4) * tile_count + sizeof(float) * tile_count + 64;
  std::vector<unsigned char> host(bytes, 0);
  size_t off_w = 0, off_t = sizeof(float) * n;
  size_t off_e = (off_t + n + 15) & ~size_t(15);
  size_t off_m = off_e + sizeof(int4) * tile_count;
  for (int f = 0; f < n; ++f) {
    const float w = host_weights ? host_weights[f] : 1.0f;
    std::memcpy(host.data() + off_w + sizeof(float) * f, &w, sizeof(float));
    host[off_t + f] = host_target_mask[f] ? 1 : 0;
  }
  std::memcpy(host.data() + off_e, host_tile_extents, sizeof(int4) * tile_count);
  std::memcpy(host.data() + off_m, host_multipliers, sizeof(float) * tile_count);
  unsigned char* dev = nullptr;
  check_cuda(cudaMallocAsync(reinterpret_cast<void**>(&dev), bytes, s->stream), "cudaMallocAsync(tile-local params)");
  upload_params(s->stream, dev, host.data(), bytes, "cudaMemcpyAsync(tile-local params)");
  TileLocalArgs a{};
  a.slots = s->d_slots;
  a.slot_of_frame = s->d_slot_of_frame;
  a.stride = s->stride;
  a.width = static_cast<int>(s->width);
  a.height = static_cast<int>(s->height);
  a.frames = n;
  a.weights = reinterpret_cast<const float*>(dev + off_w);
  a.target = dev + off_t;
  a.tiles = reinterpret_cast<const int4*>(dev + off_e);
  a.multipliers = reinterpret_cast<const float*>(dev + off_m);
  a.tile_count = tile_count;
  a.mode = mode;
  a.low_sigma = low_sigma;
  a.high_sigma = high_sigma;
  a.master = s->d_master;
  a.weight = s->d_weight;
  a.coverage = static_cast<float*>(s->d_coverage);
  a.low = static_cast<float*>(s->d_low);
  a.high = static_cast<float*>(s->d_high);
  const size_t smem = sizeof(float) * n * kTlThreads;
  check_cuda(cudaFuncSetAttribute(tile_local_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(smem)),
             "cudaFuncSetAttribute(tile-local)");
  int per_sm = 0;
  check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tile_local_kernel, kTlThreads, smem),
             "occupancy");
  note_launch();
  tile_local_kernel<<<grid_for(static_cast<size_t>(s->pixels), kTlThreads, std::max(per_sm, 1)), kTlThreads, smem,
                      s->stream>>>(a);
  check_cuda(cudaGetLastError(), "tile_local launch");
  check_cuda(cudaFreeAsync(dev, s->stream), "cudaFreeAsync(tile-local params)");
  s->last_count_dtype = GG_COUNT_F32;
  GG_API_END
}

}  // extern "C"
