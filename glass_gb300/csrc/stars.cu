// Star detection on resident frames: robust background, threshold,
// local-maximum candidates, windowed moments, flux-ordered de-duplication.
//
// Semantics: src/glass/cpu/star_detect.py:29-168 (detect_stars):
//   median / MAD of the finite pixels (exact order statistics; an even count
//   takes the float32 mean of the two middle values, as np.median does),
//   noise = 1.4826 * MAD (float64; falls back to the pixel std, then 1),
//   threshold = median + k * max(noise, 1e-6) (float64, compared against the
//   float32 pixels after rounding to float32 - NumPy's scalar promotion),
//   candidate = interior pixel, finite, > threshold, >= its 8 neighbours,
//   measurement in a (2r+1)^2 window clipped to the image with float64
//   moments of max(v - background, 0) (star_detect.py:45-100),
//   greedy de-duplication in flux order (stable: raster order breaks ties,
//   star_detect.py:103-118), then the brightest `max_stars`.
//
// GB300 layout:
//   - order statistics by a 3-pass radix select over the frame (11+11+10 key
//     bits, per-CTA shared-memory histograms fed by per-thread run-length
//     counters and folded with global atomics); the MAD reuses it with key
//     |v - median|;
//   - candidates are appended with one atomic per warp, then one CTA per
//     frame sorts them into raster order in shared memory, measures flux and
//     centroid one warp per candidate, resolves the flux-ordered
//     de-duplication with a row-range neighbour search (centroids stay within
//     the window of their peak) and selects the brightest by an 8-bit radix
//     select on the flux bits; second moments (fwhm, eccentricity) are
//     measured only for the selected stars;
//   - the first 80 selected stars (optionally only those passing a shape
//     filter) stay on the device as the frame's registration catalog.
#include <cmath>
#include <cstring>
#include <vector>

#include <math_constants.h>

#include "stack.cuh"

namespace gg {

constexpr int kSelBins = 2048;
constexpr int kMaxCandidates = 32768;  // per frame (shared-memory sort capacity)

// Per-frame detection state on the device.
struct StarFrameState {
  unsigned count;        // valid (finite) pixels
  unsigned candidates;   // appended candidates (may exceed capacity)
  unsigned overflow;
  unsigned pad;
  unsigned prefix[2];    // radix-select prefix per requested rank
  unsigned residual[2];  // rank remaining inside the prefix bucket
  float median;
  float mad;
  double noise;
  double threshold;
  float threshold_f32;
  float background_f32;
  double background;
  int kept;
  int pad2;
  // sample-bracket selection (per mode: 0 median, 1 MAD)
  unsigned band_lo, band_hi;  // inclusive key band from the sample
  unsigned below;             // finite keys under band_lo
  unsigned inside;            // keys in the band (appended, may exceed capacity)
  int resolved[2];            // 1: the order statistic came from the band
  // radix select inside the band (bracket_band_* kernels)
  unsigned band_prefix[2], band_rank[2];
  int band_ok, band_shift;
};

__device__ __forceinline__ unsigned float_key(float v) {
  const unsigned b = __float_as_uint(v);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float key_float(unsigned k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

struct SelectArgs {
  const float* slots;
  const int* slot_of_frame;
  int64_t stride;
  int64_t pixels;
  const int* frames;   // [count]
  StarFrameState* state;
  unsigned* hist;      // [count][2][kSelBins]
  int pass;            // 0, 1, 2
  int mode;            // 0: v, 1: |v - median|
};

// Histogram pass: digit of `pass` for keys matching each rank's prefix.
// Sky pixels share their leading digits, so each thread keeps a run-length
// counter per histogram (last digit, count) and only touches shared memory
// when the digit changes; four pixels per float4 load.  When both ranks
// share their prefix (the usual case: the two middle values of an even
// count lie in one bucket) only the first histogram is built and copied.
template <int PASS>
__global__ void __launch_bounds__(256) select_hist_kernel(SelectArgs a) {
  __shared__ unsigned h[2][kSelBins];
  __shared__ unsigned s_valid;
  const int k = blockIdx.y;
  if (a.state[k].resolved[a.mode]) return;  // the sample bracket found it
  for (int i = threadIdx.x; i < 2 * kSelBins; i += blockDim.x) (&h[0][0])[i] = 0u;
  if (threadIdx.x == 0) s_valid = 0;
  __syncthreads();
  const unsigned p0 = a.state[k].prefix[0], p1 = a.state[k].prefix[1];
  const bool shared_prefix = p0 == p1;
  const float median = a.state[k].median;
  const bool absdev = a.mode == 1;
  const float* src = a.slots + static_cast<int64_t>(a.slot_of_frame[a.frames[k]]) * a.stride;
  constexpr int kShift = PASS == 0 ? 21 : (PASS == 1 ? 10 : 0);
  constexpr unsigned kMask = PASS == 2 ? 1023u : 2047u;
  constexpr int kPrefixShift = PASS == 1 ? 21 : 10;
  unsigned valid = 0;
  unsigned d0 = 0xffffffffu, n0 = 0u, d1 = 0xffffffffu, n1 = 0u;
  auto add = [&](float v) {
    if (!isfinite(v)) return;
    ++valid;
    if (absdev) v = fabsf(__fsub_rn(v, median));
    const unsigned key = float_key(v);
    const unsigned digit = (key >> kShift) & kMask;
    bool in0 = true, in1 = false;
    if constexpr (PASS != 0) {
      const unsigned hp = key >> kPrefixShift;
      in0 = hp == p0;
      in1 = !shared_prefix && hp == p1;
    }
    if (in0) {
      if (digit == d0) {
        ++n0;
      } else {
        if (n0) atomicAdd(&h[0][d0], n0);
        d0 = digit;
        n0 = 1u;
      }
    }
    if (in1) {
      if (digit == d1) {
        ++n1;
      } else {
        if (n1) atomicAdd(&h[1][d1], n1);
        d1 = digit;
        n1 = 1u;
      }
    }
  };
  const int64_t gtid = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  const int64_t gstride = int64_t(gridDim.x) * blockDim.x;
  const int64_t n4 = a.pixels / 4;  // slots start on 256-byte boundaries
  const float4* src4 = reinterpret_cast<const float4*>(src);
  for (int64_t i = gtid; i < n4; i += gstride) {
    const float4 q = __ldg(src4 + i);
    add(q.x);
    add(q.y);
    add(q.z);
    add(q.w);
  }
  for (int64_t p = n4 * 4 + gtid; p < a.pixels; p += gstride) add(__ldg(src + p));
  if (n0) atomicAdd(&h[0][d0], n0);
  if (n1) atomicAdd(&h[1][d1], n1);
  if (PASS == 0) {
    valid = __reduce_add_sync(0xffffffffu, valid);
    if ((threadIdx.x & 31) == 0 && valid) atomicAdd(&s_valid, valid);
  }
  __syncthreads();
  unsigned* g = a.hist + static_cast<int64_t>(k) * 2 * kSelBins;
  const int nh = PASS == 0 ? 1 : 2;
  for (int i = threadIdx.x; i < nh * kSelBins; i += blockDim.x) {
    const unsigned v = (shared_prefix && i >= kSelBins) ? h[0][i - kSelBins] : (&h[0][0])[i];
    if (v) atomicAdd(g + i, v);
  }
  if (PASS == 0 && a.mode == 0 && threadIdx.x == 0 && s_valid) atomicAdd(&a.state[k].count, s_valid);
}

// One block per frame: locate each rank's bucket in the histogram (copied to
// shared memory, then a warp prefix scan over 32 runs of bins).
// ranks: pass 0 sets them from the valid count (median of n: n//2 and
// n//2 - 1 when n is even, both n//2 when odd).
__global__ void __launch_bounds__(256) select_scan_kernel(SelectArgs a, int frames) {
  __shared__ unsigned hs[2][kSelBins];
  __shared__ unsigned s_bucket[2], s_rem[2];
  const int k = blockIdx.x;
  if (k >= frames) return;
  StarFrameState& st = a.state[k];
  if (st.resolved[a.mode]) return;  // the sample bracket found it
  const unsigned* g = a.hist + static_cast<int64_t>(k) * 2 * kSelBins;
  const int nbins = a.pass == 2 ? 1024 : kSelBins;
  const int nh = a.pass == 0 ? 1 : 2;
  for (int i = threadIdx.x; i < nh * kSelBins; i += blockDim.x) (&hs[0][0])[i] = g[i];
  if (threadIdx.x == 0 && a.pass == 0) {
    const unsigned n = st.count;
    const unsigned hi = n / 2;
    const unsigned lo = (n & 1u) ? hi : (hi > 0 ? hi - 1 : 0);
    st.residual[0] = lo;
    st.residual[1] = hi;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    const int per = nbins / 32;
    for (int r = 0; r < 2; ++r) {
      const unsigned* hr = hs[a.pass == 0 ? 0 : r];
      const unsigned rem = st.residual[r];
      unsigned loc = 0;
      for (int b = 0; b < per; ++b) loc += hr[lane * per + b];
      unsigned incl = loc;
      for (int off = 1; off < 32; off <<= 1) {
        const unsigned v = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += v;
      }
      const unsigned excl = incl - loc;
      if (lane == 0) {  // empty frame (rank past the end): keeps the state defined
        s_bucket[r] = static_cast<unsigned>(nbins - 1);
        s_rem[r] = 0u;
      }
      __syncwarp();
      if (excl <= rem && rem < incl) {
        unsigned left = rem - excl;
        int b = lane * per;
        while (left >= hr[b]) {
          left -= hr[b];
          ++b;
        }
        s_bucket[r] = static_cast<unsigned>(b);
        s_rem[r] = left;
      }
      __syncwarp();
    }
    if (lane == 0) {
      const int bits = a.pass == 2 ? 10 : 11;
      for (int r = 0; r < 2; ++r) {
        const unsigned prev = a.pass == 0 ? 0u : st.prefix[r];
        st.prefix[r] = (prev << bits) | s_bucket[r];
        st.residual[r] = s_rem[r];
      }
    }
  }
  if (threadIdx.x == 0) {
    if (a.pass == 2) {
      // Both keys are complete: value = mean of the two middle values.
      const float lo = key_float(st.prefix[0]);
      const float hi = key_float(st.prefix[1]);
      const float med = st.count ? __fmul_rn(__fadd_rn(lo, hi), 0.5f) : 0.0f;
      if (a.mode == 0) st.median = med; else st.mad = med;
    }
  }
}

// ---- order statistics by a sample bracket ------------------------------------
// One pass over the frame instead of three: a sample of kBracketSamples
// evenly spaced pixels is sorted in shared memory and gives a key band that
// holds the wanted ranks (the middle ranks of the finite pixels) with a
// seven-sigma margin; the pass counts the finite keys below the band and
// copies the keys inside it to a per-frame buffer, where a radix select over
// the band's key range finds the exact order statistics.  A frame whose band
// misses the ranks or overflows the buffer (heavily tied data) keeps
// resolved = 0 and goes through the three-pass radix select above.
constexpr int kBracketSamples = 32768;

struct BracketArgs {
  const float* slots;
  const int* slot_of_frame;
  int64_t stride;
  int64_t pixels;
  const int* frames;
  StarFrameState* state;
  unsigned* band;      // [count][band_cap]
  int64_t band_cap;
  int mode;            // 0: v, 1: |v - median|
  unsigned* ghist;     // [count][2][256] band histograms (zero between passes)
  int pass;            // radix pass of the band select (0..3)
  int count_frames;
};

__device__ __forceinline__ bool bracket_key(float v, int mode, float median, unsigned& key) {
  if (!isfinite(v)) return false;
  key = float_key(mode == 1 ? fabsf(__fsub_rn(v, median)) : v);
  return true;
}

__global__ void __launch_bounds__(1024) bracket_sample_kernel(BracketArgs a) {
  extern __shared__ unsigned keys[];  // kBracketSamples (or pixels, if fewer)
  __shared__ unsigned s_valid;
  const int k = blockIdx.x;
  StarFrameState& st = a.state[k];
  const float* src = a.slots + static_cast<int64_t>(a.slot_of_frame[a.frames[k]]) * a.stride;
  const int n = static_cast<int>(a.pixels < kBracketSamples ? a.pixels : static_cast<int64_t>(kBracketSamples));
  int m = 1;
  while (m < n) m <<= 1;
  if (threadIdx.x == 0) s_valid = 0u;
  __syncthreads();
  unsigned valid = 0;
  const float median = st.median;
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    unsigned key = 0xffffffffu;
    if (i < n) {
      const int64_t pos = ((2 * static_cast<int64_t>(i) + 1) * a.pixels) / (2 * static_cast<int64_t>(n));
      if (bracket_key(__ldg(src + pos), a.mode, median, key)) ++valid;
      else key = 0xffffffffu;
    }
    keys[i] = key;
  }
  valid = __reduce_add_sync(0xffffffffu, valid);
  if ((threadIdx.x & 31) == 0 && valid) atomicAdd(&s_valid, valid);
  __syncthreads();
  for (int size = 2; size <= m; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const int j = i ^ stride;
        if (j > i) {
          const unsigned x = keys[i], y = keys[j];
          if (((i & size) == 0) == (x > y)) {
            keys[i] = y;
            keys[j] = x;
          }
        }
      }
      __syncthreads();
    }
  }
  if (threadIdx.x == 0) {
    const int sv = static_cast<int>(s_valid);
    // middle of the finite samples +- 7 binomial sigma (+8 for small samples)
    const int margin = static_cast<int>(ceilf(3.5f * sqrtf(static_cast<float>(sv)))) + 8;
    const int c = sv / 2;
    st.band_lo = sv > 0 ? keys[max(0, c - margin)] : 0u;
    st.band_hi = sv > 0 ? keys[min(sv - 1, c + margin)] : 0u;
    st.below = 0u;
    st.inside = 0u;
    if (a.mode == 0) st.count = 0u;
  }
}

// One pass over a frame: the finite samples below the band and the band's
// keys (appended to the frame's band buffer in no particular order).  Each
// block iteration covers 16 samples per thread (four float4 loads issued
// first) and reserves the band slots of all its in-band samples with one
// atomic, so the per-frame counter sees one atomic per 4096 samples.  The
// per-sample tests are unsigned range checks on the order-preserving keys:
// a finite float32 has a key in [0x00800000, 0xff7fffff] (float_key), so
// mode 0 needs no separate isfinite; mode 1 (|v - median|) tests the sample
// itself.
constexpr int kBracketThreads = 256;

template <int MODE>
__global__ void __launch_bounds__(kBracketThreads) bracket_pass_kernel(BracketArgs a) {
  __shared__ unsigned s_warp[kBracketThreads / 32];
  __shared__ unsigned s_base;
  const int k = blockIdx.y;
  StarFrameState& st = a.state[k];
  const unsigned lo = st.band_lo, hi = st.band_hi;
  const unsigned span = hi - lo;  // the band is [lo, lo + span]
  constexpr unsigned kFiniteLo = 0x00800000u, kFiniteSpan = 0xff7fffffu - 0x00800000u;
  // mode 0: key < lo for a finite key <=> (key - kFiniteLo) < (lo - kFiniteLo),
  // nothing is below a band that starts below the finite keys
  const unsigned lo_f = lo >= kFiniteLo ? lo - kFiniteLo : 0u;
  const float median = st.median;
  const float* src = a.slots + static_cast<int64_t>(a.slot_of_frame[a.frames[k]]) * a.stride;
  unsigned* band = a.band + static_cast<int64_t>(k) * a.band_cap;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned below = 0, valid = 0;
  constexpr int kLoads = 4;
  const int64_t n4 = a.pixels / 4;
  const float4* src4 = reinterpret_cast<const float4*>(src);
  const int64_t gstride = int64_t(gridDim.x) * blockDim.x * kLoads;
  // every thread of the block runs the same trip count (the barriers need them all)
  for (int64_t base = blockIdx.x * int64_t(blockDim.x) * kLoads; base < n4; base += gstride) {
    float4 q[kLoads];
#pragma unroll
    for (int u = 0; u < kLoads; ++u) {
      const int64_t i = base + u * int64_t(blockDim.x) + threadIdx.x;
      q[u] = i < n4 ? __ldg(src4 + i) : make_float4(CUDART_INF_F, CUDART_INF_F, CUDART_INF_F, CUDART_INF_F);
    }
    unsigned key[4 * kLoads];
    unsigned in_mask = 0u;
#pragma unroll
    for (int u = 0; u < kLoads; ++u) {
      const float v4[4] = {q[u].x, q[u].y, q[u].z, q[u].w};
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int j = 4 * u + c;
        bool fin;
        if constexpr (MODE == 0) {
          const unsigned bits = __float_as_uint(v4[c]);
          key[j] = bits ^ (static_cast<unsigned>(static_cast<int>(bits) >> 31) | 0x80000000u);  // float_key
          const unsigned kf = key[j] - kFiniteLo;
          fin = kf <= kFiniteSpan;
          valid += fin ? 1u : 0u;
          below += (kf < lo_f) ? 1u : 0u;  // implies finite
        } else {
          fin = (__float_as_uint(v4[c]) & 0x7f800000u) != 0x7f800000u;
          key[j] = __float_as_uint(fabsf(__fsub_rn(v4[c], median))) | 0x80000000u;  // float_key of a |d|
          below += (fin && key[j] < lo) ? 1u : 0u;
        }
        in_mask |= (fin && key[j] - lo <= span) ? (1u << j) : 0u;
      }
    }
    // block-wide exclusive prefix of the in-band counts, one reservation
    const unsigned mine = __popc(in_mask);
    unsigned incl = mine;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const unsigned n = __shfl_up_sync(0xffffffffu, incl, off);
      if (lane >= off) incl += n;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned total = 0;
#pragma unroll
      for (int w = 0; w < kBracketThreads / 32; ++w) {
        const unsigned c = s_warp[w];
        s_warp[w] = total;
        total += c;
      }
      s_base = total ? atomicAdd(&st.inside, total) : 0u;
    }
    __syncthreads();
    int64_t pos = static_cast<int64_t>(s_base) + s_warp[warp] + (incl - mine);
    while (in_mask) {
      const int j = __ffs(in_mask) - 1;
      in_mask &= in_mask - 1u;
      if (pos < a.band_cap) band[pos] = key[j];
      ++pos;
    }
    __syncthreads();  // s_warp and s_base are rewritten by the next iteration
  }
  // the last pixels % 4 samples: one warp, one atomic per in-band sample
  if (blockIdx.x == 0 && threadIdx.x < 32) {
    for (int64_t p = n4 * 4 + threadIdx.x; p < a.pixels; p += 32) {
      unsigned key = 0u;
      const bool fin = bracket_key(__ldg(src + p), MODE, median, key);
      valid += fin ? 1u : 0u;
      below += (fin && key < lo) ? 1u : 0u;
      if (fin && key >= lo && key <= hi) {
        const unsigned at = atomicAdd(&st.inside, 1u);
        if (at < a.band_cap) band[at] = key;
      }
    }
  }
  below = __reduce_add_sync(0xffffffffu, below);
  valid = __reduce_add_sync(0xffffffffu, valid);
  if (lane == 0) {
    if (below) atomicAdd(&st.below, below);
    if (MODE == 0 && valid) atomicAdd(&st.count, valid);
  }
}

// The two middle ranks' keys inside the band by an MSB-first radix select
// over key - band_lo (8 bits per pass), then the median / MAD as the float32
// mean of the two middle values (np.median).  The band of a 9600 x 6422
// frame holds ~1.6 M keys, so each pass spreads it over several CTAs per
// frame (shared histograms merged into a per-frame global histogram) and one
// warp per frame picks the digit:
//   bracket_band_init   the ranks inside the band (or no band select when
//                       the order statistics lie outside it: the radix
//                       fallback then takes the frame), passes from the
//                       bits of the band's key range
//   bracket_band_hist   per pass, CTAs x frames
//   bracket_band_digit  per pass, one warp per frame
//   bracket_band_finish the value of the two ranks
__global__ void bracket_band_init_kernel(BracketArgs a) {
  const int k = blockIdx.x;
  StarFrameState& st = a.state[k];
  unsigned* g = a.ghist + static_cast<int64_t>(k) * 512;
  for (int i = threadIdx.x; i < 512; i += blockDim.x) g[i] = 0u;
  if (threadIdx.x != 0) return;
  const unsigned n = st.count;
  const unsigned rhi = n / 2, rlo = (n & 1u) ? rhi : (rhi > 0 ? rhi - 1 : 0);
  const bool ok = n > 0 && static_cast<int64_t>(st.inside) <= a.band_cap && st.below <= rlo &&
                  rhi < st.below + st.inside;
  st.band_ok = ok ? 1 : 0;
  st.band_rank[0] = ok ? rlo - st.below : 0u;
  st.band_rank[1] = ok ? rhi - st.below : 0u;
  st.band_prefix[0] = st.band_prefix[1] = 0u;
  st.resolved[a.mode] = 0;
  if (!ok && a.mode == 0) st.count = 0u;  // the radix passes count the finite pixels again
  const unsigned range = st.band_hi - st.band_lo;
  int top = 0;  // bits of the key range
  while (top < 32 && (range >> top) != 0u) ++top;
  st.band_shift = ((top + 7) / 8) * 8 - 8;  // first pass's digit shift (< 0: a one-value band)
}

__global__ void __launch_bounds__(256) bracket_band_hist_kernel(BracketArgs a) {
  __shared__ unsigned hist[2][256];
  const int k = blockIdx.y;
  const StarFrameState& st = a.state[k];
  const int shift = st.band_shift - 8 * a.pass;
  if (!st.band_ok || shift < 0) return;
  for (int i = threadIdx.x; i < 512; i += blockDim.x) (&hist[0][0])[i] = 0u;
  __syncthreads();
  const unsigned lo = st.band_lo, pre0 = st.band_prefix[0], pre1 = st.band_prefix[1];
  const int hi_shift = shift + 8;
  const unsigned* band = a.band + static_cast<int64_t>(k) * a.band_cap;
  const int64_t m = st.inside;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < m; i += int64_t(gridDim.x) * blockDim.x) {
    const unsigned d = band[i] - lo;
    const unsigned hp = hi_shift >= 32 ? 0u : (d >> hi_shift);
    const unsigned digit = (d >> shift) & 255u;
    if (hp == pre0) atomicAdd(&hist[0][digit], 1u);
    if (hp == pre1 && pre1 != pre0) atomicAdd(&hist[1][digit], 1u);
  }
  __syncthreads();
  unsigned* g = a.ghist + static_cast<int64_t>(k) * 512;
  for (int i = threadIdx.x; i < 512; i += blockDim.x) {
    const unsigned c = (&hist[0][0])[i];
    if (c) atomicAdd(g + i, c);
  }
}

__global__ void bracket_band_digit_kernel(BracketArgs a) {
  const int k = blockIdx.x;
  StarFrameState& st = a.state[k];
  const int shift = st.band_shift - 8 * a.pass;
  if (!st.band_ok || shift < 0) return;
  unsigned* g = a.ghist + static_cast<int64_t>(k) * 512;
  if (threadIdx.x < 2) {
    const int r = threadIdx.x;
    const unsigned* h = (r == 1 && st.band_prefix[1] == st.band_prefix[0]) ? g : g + 256 * r;
    unsigned rank = st.band_rank[r];
    int b = 0;
    while (b < 255 && rank >= h[b]) {
      rank -= h[b];
      ++b;
    }
    __syncwarp(0x3u);
    st.band_rank[r] = rank;
    st.band_prefix[r] = (st.band_prefix[r] << 8) | static_cast<unsigned>(b);
  }
  __syncwarp();
  for (int i = threadIdx.x; i < 512; i += blockDim.x) g[i] = 0u;  // ready for the next pass
}

__global__ void bracket_band_finish_kernel(BracketArgs a) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.count_frames) return;
  StarFrameState& st = a.state[k];
  if (!st.band_ok) return;
  const float vlo = key_float(st.band_lo + st.band_prefix[0]);
  const float vhi = key_float(st.band_lo + st.band_prefix[1]);
  const float med = __fmul_rn(__fadd_rn(vlo, vhi), 0.5f);
  if (a.mode == 0) st.median = med; else st.mad = med;
  st.resolved[a.mode] = 1;
}

// Threshold from median / MAD (star_detect.py:29-43, 133-137).
__global__ void star_threshold_kernel(StarFrameState* state, int frames, float k_sigma, int has_background,
                                      float background, int has_noise, float noise, const double* rms) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= frames) return;
  StarFrameState& st = state[k];
  double med = st.count ? static_cast<double>(st.median) : 0.0;
  double nz = st.count ? 1.4826 * static_cast<double>(st.mad) : 1.0;
  if (st.count && !(nz > 0.0)) nz = rms ? rms[k] : 0.0;
  if (!(nz > 0.0)) nz = 1.0;
  if (has_background) med = static_cast<double>(background);
  if (has_noise) nz = static_cast<double>(noise);
  st.noise = nz;
  st.threshold = med + static_cast<double>(k_sigma) * fmax(nz, 1.0e-6);
  st.threshold_f32 = static_cast<float>(st.threshold);
  st.background_f32 = static_cast<float>(med);
  st.background = med;
}

// ---- background mesh (no reference counterpart) ------------------------------
// Cells of `cell` x `cell` pixels from the top-left corner (edge cells
// smaller).  Each cell's finite pixels give the float64 median (an even count
// takes 0.5 * (a + b) of the two middle values) and noise 1.4826 * MAD (1
// when the MAD is 0; NaN median and noise without finite pixels).  Values at
// a pixel interpolate bilinearly between cell centres, u = (x + 0.5) / cell -
// 0.5, clamped at the first and last centre, in float64 without fused
// multiply-adds (the oracle evaluates the same operations in NumPy).
constexpr int kMeshMaxCell = 64;
constexpr int kMeshElems = kMeshMaxCell * kMeshMaxCell;

struct MeshView {
  const double* bg;  // [count][ny * nx] or nullptr (global statistics)
  const double* nz;
  int cell, nx, ny;
};

__device__ __forceinline__ void mesh_axis(int coord, int cell, int n, int& i0, int& i1, double& f) {
  const double u = __dsub_rn(__ddiv_rn(__dadd_rn(static_cast<double>(coord), 0.5), static_cast<double>(cell)), 0.5);
  const double fl = floor(u);
  if (fl < 0.0) {
    i0 = 0;
    f = 0.0;
  } else if (fl >= static_cast<double>(n - 1)) {
    i0 = n - 1;
    f = 0.0;
  } else {
    i0 = static_cast<int>(fl);
    f = __dsub_rn(u, fl);
  }
  i1 = min(i0 + 1, n - 1);
}

__device__ __forceinline__ double mesh_lerp(const double* m, int nx, int i0, int i1, int j0, int j1, double fx,
                                            double fy) {
  const double gx = __dsub_rn(1.0, fx), gy = __dsub_rn(1.0, fy);
  const double top = __dadd_rn(__dmul_rn(gx, m[j0 * nx + i0]), __dmul_rn(fx, m[j0 * nx + i1]));
  const double bot = __dadd_rn(__dmul_rn(gx, m[j1 * nx + i0]), __dmul_rn(fx, m[j1 * nx + i1]));
  return __dadd_rn(__dmul_rn(gy, top), __dmul_rn(fy, bot));
}

// Interpolated background and noise of frame k at pixel (x, y).
__device__ __forceinline__ void mesh_at(const MeshView& m, int k, int x, int y, double& bg, double& nz) {
  int i0, i1, j0, j1;
  double fx, fy;
  mesh_axis(x, m.cell, m.nx, i0, i1, fx);
  mesh_axis(y, m.cell, m.ny, j0, j1, fy);
  const int64_t off = static_cast<int64_t>(k) * m.nx * m.ny;
  bg = mesh_lerp(m.bg + off, m.nx, i0, i1, j0, j1, fx, fy);
  nz = mesh_lerp(m.nz + off, m.nx, i0, i1, j0, j1, fx, fy);
}

__device__ void bitonic_sort_shared(double* v, int n) {
  for (int k = 2; k <= n; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const bool up = (i & k) == 0;
          const double a = v[i], b = v[ixj];
          if ((a > b) == up) {
            v[i] = b;
            v[ixj] = a;
          }
        }
      }
      __syncthreads();
    }
}

__device__ __forceinline__ double median_sorted(const double* v, int n) {
  const int m = n / 2;
  return (n & 1) ? v[m] : __dmul_rn(__dadd_rn(v[m - 1], v[m]), 0.5);
}

struct MeshArgs {
  const float* slots;
  const int* slot_of_frame;
  int64_t stride;
  int width, height;
  const int* frames;
  double* bg;
  double* nz;
  int cell, nx, ny;
};

// One CTA per (cell, frame): gather the finite pixels, sort, median; sort the
// absolute deviations, MAD.
__global__ void __launch_bounds__(1024) mesh_stats_kernel(MeshArgs a) {
  __shared__ double v[kMeshElems];
  __shared__ int s_n;
  __shared__ double s_med;
  const int c = blockIdx.x, k = blockIdx.y;
  const int cx = c % a.nx, cy = c / a.nx;
  const int x0 = cx * a.cell, y0 = cy * a.cell;
  const int w = min(a.cell, a.width - x0), h = min(a.cell, a.height - y0);
  const float* img = a.slots + static_cast<int64_t>(a.slot_of_frame[a.frames[k]]) * a.stride;
  if (threadIdx.x == 0) s_n = 0;
  __syncthreads();
  for (int q = threadIdx.x; q < w * h; q += blockDim.x) {
    const float val = __ldg(img + static_cast<int64_t>(y0 + q / w) * a.width + x0 + q % w);
    if (isfinite(val)) v[atomicAdd(&s_n, 1)] = static_cast<double>(val);
  }
  __syncthreads();
  const int n = s_n;
  const int64_t out = static_cast<int64_t>(k) * a.nx * a.ny + c;
  if (n == 0) {
    if (threadIdx.x == 0) a.bg[out] = a.nz[out] = __longlong_as_double(0x7ff8000000000000LL);
    return;
  }
  int p2 = 1;
  while (p2 < n) p2 <<= 1;
  const double inf = __longlong_as_double(0x7ff0000000000000LL);
  for (int q = n + threadIdx.x; q < p2; q += blockDim.x) v[q] = inf;
  __syncthreads();
  bitonic_sort_shared(v, p2);
  if (threadIdx.x == 0) s_med = median_sorted(v, n);
  __syncthreads();
  const double med = s_med;
  for (int q = threadIdx.x; q < n; q += blockDim.x) v[q] = fabs(__dsub_rn(v[q], med));
  __syncthreads();
  bitonic_sort_shared(v, p2);
  if (threadIdx.x == 0) {
    const double mad = median_sorted(v, n);
    a.bg[out] = med;
    a.nz[out] = mad > 0.0 ? __dmul_rn(1.4826, mad) : 1.0;
  }
}

struct DetectArgs {
  const float* slots;
  const int* slot_of_frame;
  int64_t stride;
  int width, height;
  const int* frames;
  StarFrameState* state;
  unsigned* cand;  // [count][kMaxCandidates] raster indices
  MeshView mesh;
  double k_sigma;
};

// Local-maximum candidates (star_detect.py:142-151).  Rows are dealt to
// blocks, columns to the block's threads (coalesced, no division), kPer
// columns per thread and pass with all their loads issued first.  Every
// thread of a row pass runs the same trip count, so the warp ballot always
// sees the full warp.  MESH: per-pixel threshold from the background mesh
// (float64), else the frame's float32 threshold.
template <bool MESH>
__global__ void __launch_bounds__(256) star_detect_kernel(DetectArgs a) {
  const int k = blockIdx.y;
  const float* img = a.slots + static_cast<int64_t>(a.slot_of_frame[a.frames[k]]) * a.stride;
  const float thr = a.state[k].threshold_f32;
  const int W = a.width, H = a.height;
  unsigned* out = a.cand + static_cast<int64_t>(k) * kMaxCandidates;
  const int lane = threadIdx.x & 31;
  constexpr int kPer = MESH ? 4 : 8;
  const int span = static_cast<int>(blockDim.x) * kPer;
  const int passes = (W - 2 + span - 1) / span;
  for (int y = 1 + static_cast<int>(blockIdx.x); y < H - 1; y += static_cast<int>(gridDim.x)) {
    const float* row = img + static_cast<int64_t>(y) * W;
    for (int pass = 0; pass < passes; ++pass) {
      const int x0 = 1 + pass * span + static_cast<int>(threadIdx.x);
      float c[kPer];
#pragma unroll
      for (int u = 0; u < kPer; ++u) {
        const int x = x0 + u * static_cast<int>(blockDim.x);
        c[u] = x <= W - 2 ? __ldg(row + x) : 0.0f;
      }
      // threshold first: most passes hold no candidate in the whole warp
      unsigned above_bits = 0u;
#pragma unroll
      for (int u = 0; u < kPer; ++u) {
        const int x = x0 + u * static_cast<int>(blockDim.x);
        bool above = false;
        if constexpr (MESH) {
          if (x <= W - 2) {  // the mesh is read inside the frame only
            double bg, nz;
            mesh_at(a.mesh, k, x, y, bg, nz);
            const double nzc = (nz >= 1.0e-6 || isnan(nz)) ? nz : 1.0e-6;  // np.maximum keeps NaN
            above = static_cast<double>(c[u]) > __dadd_rn(bg, __dmul_rn(a.k_sigma, nzc));
          }
        } else {
          above = c[u] > thr;
        }
        above_bits |= (x <= W - 2 && isfinite(c[u]) && above) ? (1u << u) : 0u;
      }
      if (!__any_sync(0xffffffffu, above_bits != 0u)) continue;
      // every column's 3 x 3 test first (their loads all in flight
      // together), then one ballot per column
      unsigned hit_bits = 0u;
#pragma unroll
      for (int u = 0; u < kPer; ++u) {
        if ((above_bits >> u) & 1u) {
          const float* p = row + x0 + u * static_cast<int>(blockDim.x);
          bool hit = true;
#pragma unroll
          for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
            for (int dx = -1; dx <= 1; ++dx)
              if (dx || dy) hit &= (c[u] >= __ldg(p + static_cast<int64_t>(dy) * W + dx));
          hit_bits |= hit ? (1u << u) : 0u;
        }
      }
#pragma unroll
      for (int u = 0; u < kPer; ++u) {
        const int x = x0 + u * static_cast<int>(blockDim.x);
        const bool hit = (hit_bits >> u) & 1u;
        const unsigned mask = __ballot_sync(0xffffffffu, hit);
        if (mask) {
          const int leader = __ffs(mask) - 1;
          unsigned base = 0;
          if (lane == leader) base = atomicAdd(&a.state[k].candidates, static_cast<unsigned>(__popc(mask)));
          base = __shfl_sync(0xffffffffu, base, leader);
          if (hit) {
            const unsigned pos = base + __popc(mask & ((1u << lane) - 1u));
            if (pos < static_cast<unsigned>(kMaxCandidates))
              out[pos] = static_cast<unsigned>(static_cast<int64_t>(y) * W + x);
          }
        }
      }
    }
  }
}

// Measured star (float64 fields as the CPU's Python floats).
// Float-float sum of the whole warp (TwoSum butterfly), in every lane.
__device__ __forceinline__ void ff_warp_sum(FF& s) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, s.hi, off);
    const float ol = __shfl_xor_sync(0xffffffffu, s.lo, off);
    float h, e;
    two_sum(s.hi, oh, h, e);
    s.hi = h;
    s.lo = __fadd_rn(__fadd_rn(s.lo, ol), e);
  }
}

// (n.hi + n.lo) / (d.hi + d.lo) to about 46 bits, returned as a double.
__device__ __forceinline__ double ff_quotient_f64(const FF& n, const FF& d) {
  const float q = __fdiv_rn(n.hi, d.hi);
  float r = __fmaf_rn(-q, d.hi, n.hi);
  r = __fadd_rn(r, n.lo);
  r = __fmaf_rn(-q, d.lo, r);
  return static_cast<double>(q) + static_cast<double>(__fdiv_rn(r, d.hi));
}

struct StarRec {
  double x, y, flux, peak, fwhm, ecc, snr, sharpness;
  int npix;
  int valid;
};

struct CatalogArgs {
  const float* slots;
  const int* slot_of_frame;
  int64_t stride;
  int width, height;
  const int* frames;
  StarFrameState* state;
  unsigned* cand;   // [count][kMaxCandidates]
  StarRec* recs;    // [count][kMaxCandidates]
  int* kept;        // [count][kMaxCandidates] flags / order
  gg_star_t* out;   // [count][max_stars]
  int max_stars;
  int radius;
  double min_sep;
  int* error;
  double* cat_xy;  // [frames][kCatalogPoints][2]: brightest stars, for registration
  int* cat_n;      // [frames]
  MeshView mesh;   // local background / noise per star when mesh.bg is set
};

// Sort candidate raster indices ascending (one CTA per frame, bitonic in
// shared memory, padded with 0xffffffff).
__global__ void __launch_bounds__(1024) star_sort_kernel(CatalogArgs a) {
  extern __shared__ unsigned keys[];
  const int k = blockIdx.x;
  StarFrameState& st = a.state[k];
  const unsigned n = min(st.candidates, static_cast<unsigned>(kMaxCandidates));
  if (threadIdx.x == 0 && st.candidates > static_cast<unsigned>(kMaxCandidates)) st.overflow = 1u;
  unsigned m = 1;
  while (m < n) m <<= 1;
  unsigned* cand = a.cand + static_cast<int64_t>(k) * kMaxCandidates;
  for (unsigned i = threadIdx.x; i < m; i += blockDim.x) keys[i] = i < n ? cand[i] : 0xffffffffu;
  __syncthreads();
  for (unsigned size = 2; size <= m; size <<= 1) {
    for (unsigned stride = size >> 1; stride > 0; stride >>= 1) {
      for (unsigned i = threadIdx.x; i < m; i += blockDim.x) {
        const unsigned j = i ^ stride;
        if (j > i) {
          const bool up = (i & size) == 0;
          const unsigned ki = keys[i], kj = keys[j];
          if ((ki > kj) == up) {
            keys[i] = kj;
            keys[j] = ki;
          }
        }
      }
      __syncthreads();
    }
  }
  for (unsigned i = threadIdx.x; i < n; i += blockDim.x) cand[i] = keys[i];
}

// One warp per candidate: windowed moments (star_detect.py:45-100).
__global__ void __launch_bounds__(256) star_measure_kernel(CatalogArgs a) {
  const int k = blockIdx.y;
  const StarFrameState& st = a.state[k];
  const int n = static_cast<int>(min(st.candidates, static_cast<unsigned>(kMaxCandidates)));
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const float* img = a.slots + static_cast<int64_t>(a.slot_of_frame[a.frames[k]]) * a.stride;
  const unsigned* cand = a.cand + static_cast<int64_t>(k) * kMaxCandidates;
  StarRec* recs = a.recs + static_cast<int64_t>(k) * kMaxCandidates;
  const int W = a.width, H = a.height, r = a.radius;
  for (int c = warp; c < n; c += nwarps) {
    const unsigned idx = cand[c];
    const int x = static_cast<int>(idx % static_cast<unsigned>(W));
    const int y = static_cast<int>(idx / static_cast<unsigned>(W));
    double bg = st.background, noise = st.noise;
    if (a.mesh.bg) mesh_at(a.mesh, k, x, y, bg, noise);
    const float bg32 = a.mesh.bg ? __double2float_rn(bg) : st.background_f32;
    (void)noise;
    const int x0 = max(0, x - r), x1 = min(W, x + r + 1);
    const int y0 = max(0, y - r), y1 = min(H, y + r + 1);
    const int ww = x1 - x0, npx = ww * (y1 - y0);
    // float-float sums (about 48 bits; the weights are float32 and the
    // coordinate products exact): float64 is scarce on this part
    FF f, sx, sy;
    int fin = 0, pos = 0;
    for (int q = lane; q < npx; q += 32) {
      const int row = q / ww;
      const int xx = x0 + (q - row * ww), yy = y0 + row;
      const float v = __ldg(img + static_cast<int64_t>(yy) * W + xx);
      if (!isfinite(v)) continue;
      ++fin;
      const float wv = fmaxf(__fsub_rn(v, bg32), 0.0f);
      pos += wv > 0.0f;
      f.add(wv);
      sx.add_prod(static_cast<float>(xx), wv);
      sy.add_prod(static_cast<float>(yy), wv);
    }
    ff_warp_sum(f);
    ff_warp_sum(sx);
    ff_warp_sum(sy);
    fin = __reduce_add_sync(0xffffffffu, fin);
    pos = __reduce_add_sync(0xffffffffu, pos);
    StarRec rec{};
    rec.valid = (fin > 0 && f.hi > 0.0f) ? 1 : 0;
    if (rec.valid && lane == 0) {
      // second moments, snr and sharpness are filled in for the selected
      // stars only (star_select_kernel, star_moments_kernel)
      rec.x = ff_quotient_f64(sx, f);
      rec.y = ff_quotient_f64(sy, f);
      rec.flux = static_cast<double>(f.hi) + static_cast<double>(f.lo);
      const float center = __ldg(img + static_cast<int64_t>(y) * W + x);
      rec.peak = fmax(static_cast<double>(center) - bg, 0.0);
      rec.npix = pos;
    }
    if (lane == 0) recs[c] = rec;
  }
}

// Priority: higher flux first, then lower raster index (stable sort order).
__device__ __forceinline__ bool higher_priority(double fj, unsigned rj, double fi, unsigned ri) {
  return fj > fi || (fj == fi && rj < ri);
}

__device__ __forceinline__ unsigned long long flux_key(double f) {
  return static_cast<unsigned long long>(__double_as_longlong(f));  // f > 0: bit order = value order
}

// One CTA per frame: flux-ordered greedy de-duplication and top-N selection.
__global__ void __launch_bounds__(1024) star_select_kernel(CatalogArgs a) {
  extern __shared__ unsigned char sm[];
  const int k = blockIdx.x;
  StarFrameState& st = a.state[k];
  const int n = static_cast<int>(min(st.candidates, static_cast<unsigned>(kMaxCandidates)));
  const unsigned* cand = a.cand + static_cast<int64_t>(k) * kMaxCandidates;
  const StarRec* recs = a.recs + static_cast<int64_t>(k) * kMaxCandidates;
  int* state = a.kept + static_cast<int64_t>(k) * kMaxCandidates;  // -1 undecided, 0 dropped, 1 kept
  const int W = a.width;
  const int reach = static_cast<int>(ceil(a.min_sep)) + 2 * a.radius;
  const double sep2 = a.min_sep * a.min_sep;
  const bool dedupe = a.min_sep > 0.0;
  // 1) initial state: invalid stars drop out; others undecided
  for (int i = threadIdx.x; i < n; i += blockDim.x) state[i] = recs[i].valid ? -1 : 0;
  __syncthreads();
  // 2) rounds: a star is kept when no higher-priority conflicting star can be
  //    kept; dropped when a higher-priority conflicting star is kept.
  __shared__ int s_changed, s_undecided;
  for (int round = 0; round < n + 1; ++round) {
    if (threadIdx.x == 0) {
      s_changed = 0;
      s_undecided = 0;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      if (state[i] != -1) continue;
      const StarRec ri = recs[i];
      const unsigned ci = cand[i];
      int verdict = 1;  // kept unless a conflict says otherwise
      if (dedupe) {
        const int py = static_cast<int>(ci / static_cast<unsigned>(W));
        const int px = static_cast<int>(ci % static_cast<unsigned>(W));
        const unsigned lo_key = static_cast<unsigned>(max(0, py - reach)) * static_cast<unsigned>(W);
        int lo = 0, hi = n;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (cand[mid] < lo_key) lo = mid + 1; else hi = mid;
        }
        for (int j = lo; j < n; ++j) {
          const unsigned cj = cand[j];
          const int qy = static_cast<int>(cj / static_cast<unsigned>(W));
          if (qy > py + reach) break;
          if (j == i || abs(static_cast<int>(cj % static_cast<unsigned>(W)) - px) > reach) continue;
          const int sj = state[j];
          if (sj == 0) continue;
          const StarRec rj = recs[j];
          if (!higher_priority(rj.flux, cj, ri.flux, ci)) continue;
          const double dx = ri.x - rj.x, dy = ri.y - rj.y;
          if (dx * dx + dy * dy < sep2) {
            if (sj == 1) {
              verdict = 0;
              break;
            }
            verdict = -1;  // waits for the brighter neighbour
          }
        }
      }
      if (verdict != -1) {
        state[i] = verdict;
        s_changed = 1;
      } else {
        s_undecided = 1;
      }
    }
    __syncthreads();
    const bool done = s_undecided == 0 || s_changed == 0;
    __syncthreads();
    if (done) break;
  }
  // 3) the max_stars-th largest kept flux: radix select (8-bit digits, most
  //    significant first) of rank total_kept - take in ascending key order
  __shared__ int s_count;
  __shared__ unsigned s_hist[256];
  __shared__ unsigned long long s_prefix;
  __shared__ int s_rank;
  int total_kept = 0;
  {
    int c = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) c += state[i] == 1;
    if (threadIdx.x == 0) s_count = 0;
    __syncthreads();
    atomicAdd(&s_count, c);
    __syncthreads();
    total_kept = s_count;
  }
  const int take = min(total_kept, a.max_stars);
  unsigned long long t = 0;  // keep fluxes with key > t, plus ties at t
  if (take < total_kept) {
    unsigned long long prefix = 0ull, mask = 0ull;
    int rank = total_kept - take;
    for (int shift = 56; shift >= 0; shift -= 8) {
      for (int i = threadIdx.x; i < 256; i += blockDim.x) s_hist[i] = 0u;
      __syncthreads();
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        if (state[i] != 1) continue;
        const unsigned long long key = flux_key(recs[i].flux);
        if ((key & mask) == prefix) atomicAdd(&s_hist[(key >> shift) & 255u], 1u);
      }
      __syncthreads();
      if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        unsigned loc = 0;
        for (int b = 0; b < 8; ++b) loc += s_hist[lane * 8 + b];
        unsigned incl = loc;
        for (int off = 1; off < 32; off <<= 1) {
          const unsigned v = __shfl_up_sync(0xffffffffu, incl, off);
          if (lane >= off) incl += v;
        }
        const unsigned excl = incl - loc;
        if (excl <= static_cast<unsigned>(rank) && static_cast<unsigned>(rank) < incl) {
          unsigned r = static_cast<unsigned>(rank) - excl;
          int b = lane * 8;
          while (r >= s_hist[b]) {
            r -= s_hist[b];
            ++b;
          }
          s_prefix = prefix | (static_cast<unsigned long long>(b) << shift);
          s_rank = static_cast<int>(r);
        }
      }
      __syncthreads();
      prefix = s_prefix;
      rank = s_rank;
      mask |= 0xffull << shift;
      __syncthreads();
    }
    t = prefix;
  }
  // 4) gather the selected stars (key > t and all ties key == t) and sort
  //    them by priority in shared memory: the first `take` are the answer
  //    (ties at t come out in raster order).
  struct Sel {
    double flux;
    unsigned raster;
    int idx;
  };
  Sel* sel = reinterpret_cast<Sel*>(sm);
  __shared__ int s_n;
  if (threadIdx.x == 0) s_n = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    if (state[i] == 1 && (take == total_kept || flux_key(recs[i].flux) >= t)) {
      const int p = atomicAdd(&s_n, 1);
      if (p < 4096) sel[p] = {recs[i].flux, cand[i], i};
    }
  }
  __syncthreads();
  const int m0 = min(s_n, 4096);
  int m = 1;
  while (m < m0) m <<= 1;
  for (int i = threadIdx.x + m0; i < m; i += blockDim.x) sel[i] = {-1.0, 0xffffffffu, -1};
  __syncthreads();
  for (int size = 2; size <= m; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const int j = i ^ stride;
        if (j > i) {
          const bool up = (i & size) == 0;  // "up" = priority order
          const Sel si = sel[i], sj = sel[j];
          const bool j_first = higher_priority(sj.flux, sj.raster, si.flux, si.raster);
          if (j_first == up) {
            sel[i] = sj;
            sel[j] = si;
          }
        }
      }
      __syncthreads();
    }
  }
  gg_star_t* out = a.out + static_cast<int64_t>(k) * a.max_stars;
  const int nout = min(take, m0);
  int* chosen = a.kept + static_cast<int64_t>(k) * kMaxCandidates;  // dedupe states are no longer read
  for (int i = threadIdx.x; i < nout; i += blockDim.x) {
    const StarRec r = recs[sel[i].idx];
    gg_star_t s;
    s.x = r.x;
    s.y = r.y;
    s.flux = r.flux;
    s.peak = r.peak;
    s.fwhm = nan("");  // star_moments_kernel
    s.eccentricity = nan("");
    double noise = st.noise;
    if (a.mesh.bg) {
      const unsigned idx = a.cand[static_cast<int64_t>(k) * kMaxCandidates + sel[i].idx];
      double bg_unused;
      mesh_at(a.mesh, k, static_cast<int>(idx % static_cast<unsigned>(a.width)),
              static_cast<int>(idx / static_cast<unsigned>(a.width)), bg_unused, noise);
    }
    s.snr = r.flux / fmax(noise * sqrt(static_cast<double>(max(r.npix, 1))), 1.0e-6);
    s.sharpness = r.peak / fmax(r.flux, 1.0e-6);
    s.npix = r.npix;
    s.pad = 0;
    out[i] = s;
    chosen[i] = sel[i].idx;
  }
  if (threadIdx.x == 0) st.kept = nout;
}

// Registration catalog of each frame: the first kCatalogPoints output stars
// (brightest first, cpu/registration.py:37-39) that pass the optional shape
// filter.  One warp per frame, order-preserving ballot compaction.
__global__ void star_catalog_kernel(CatalogArgs a, float min_fwhm, float max_ecc) {
  const int k = blockIdx.x;
  const int lane = threadIdx.x;
  const int nout = a.state[k].kept;
  const gg_star_t* out = a.out + static_cast<int64_t>(k) * a.max_stars;
  const int frame = a.frames[k];
  double* dst = a.cat_xy + static_cast<int64_t>(frame) * kCatalogPoints * 2;
  const bool test_fwhm = min_fwhm > 0.0f, test_ecc = max_ecc < 1.0f;
  int taken = 0;
  for (int base = 0; base < nout && taken < kCatalogPoints; base += 32) {
    const int i = base + lane;
    bool pass = false;
    double x = 0.0, y = 0.0;
    if (i < nout) {
      const gg_star_t s = out[i];
      pass = (!test_fwhm || s.fwhm >= static_cast<double>(min_fwhm)) &&
             (!test_ecc || s.eccentricity <= static_cast<double>(max_ecc));
      x = s.x;
      y = s.y;
    }
    const unsigned mask = __ballot_sync(0xffffffffu, pass);
    const int pos = taken + __popc(mask & ((1u << lane) - 1u));
    if (pass && pos < kCatalogPoints) {
      dst[2 * pos] = x;
      dst[2 * pos + 1] = y;
    }
    taken += __popc(mask);
  }
  if (lane == 0) a.cat_n[frame] = min(taken, kCatalogPoints);
}

// Second moments of the selected stars (star_detect.py:83-99): intensity
// weighted about the centroid, fwhm from the mean of the principal
// variances, eccentricity from their ratio.  One warp per star.
__global__ void __launch_bounds__(256) star_moments_kernel(CatalogArgs a) {
  const int k = blockIdx.y;
  const StarFrameState& st = a.state[k];
  const int nout = st.kept;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const float* img = a.slots + static_cast<int64_t>(a.slot_of_frame[a.frames[k]]) * a.stride;
  const unsigned* cand = a.cand + static_cast<int64_t>(k) * kMaxCandidates;
  const StarRec* recs = a.recs + static_cast<int64_t>(k) * kMaxCandidates;
  const int* chosen = a.kept + static_cast<int64_t>(k) * kMaxCandidates;
  gg_star_t* out = a.out + static_cast<int64_t>(k) * a.max_stars;
  const int W = a.width, H = a.height, r = a.radius;
  for (int i = warp; i < nout; i += nwarps) {
    const int c = chosen[i];
    const StarRec rec = recs[c];
    const unsigned idx = cand[c];
    const int x = static_cast<int>(idx % static_cast<unsigned>(W));
    const int y = static_cast<int>(idx / static_cast<unsigned>(W));
    float bg32 = st.background_f32;
    if (a.mesh.bg) {
      double bg, noise;
      mesh_at(a.mesh, k, x, y, bg, noise);
      bg32 = __double2float_rn(bg);
    }
    const int x0 = max(0, x - r), x1 = min(W, x + r + 1);
    const int y0 = max(0, y - r), y1 = min(H, y + r + 1);
    const int ww = x1 - x0, npx = ww * (y1 - y0);
    const double cx = rec.x, cy = rec.y, f = rec.flux;
    double mxx = 0.0, myy = 0.0, mxy = 0.0;
    for (int q = lane; q < npx; q += 32) {
      const int xx = x0 + q % ww, yy = y0 + q / ww;
      const float v = __ldg(img + static_cast<int64_t>(yy) * W + xx);
      if (!isfinite(v)) continue;
      const double wd = static_cast<double>(fmaxf(__fsub_rn(v, bg32), 0.0f));
      const double dx = static_cast<double>(xx) - cx, dy = static_cast<double>(yy) - cy;
      mxx += dx * dx * wd;
      myy += dy * dy * wd;
      mxy += dx * dy * wd;
    }
    for (int off = 16; off > 0; off >>= 1) {
      mxx += __shfl_xor_sync(0xffffffffu, mxx, off);
      myy += __shfl_xor_sync(0xffffffffu, myy, off);
      mxy += __shfl_xor_sync(0xffffffffu, mxy, off);
    }
    mxx /= f;
    myy /= f;
    mxy /= f;
    const double trace = fmax(mxx + myy, 0.0);
    const double det = fmax((mxx - myy) * (mxx - myy) + 4.0 * mxy * mxy, 0.0);
    const double root = sqrt(det);
    const double major = fmax((trace + root) / 2.0, 0.0);
    const double minor = fmax((trace - root) / 2.0, 0.0);
    const double mean_sigma = sqrt(fmax((major + minor) / 2.0, 0.0));
    if (lane == 0) {
      out[i].fwhm = mean_sigma > 0.0 ? 2.354820045 * mean_sigma : nan("");
      out[i].eccentricity = major > 0.0 ? sqrt(fmax(0.0, 1.0 - minor / major)) : nan("");
    }
  }
}

// ---- np.std of the finite pixels, bit-exact (fallback noise, MAD == 0) -----
// NumPy sums a contiguous float32 array pairwise: blocks of <= 128 use eight
// interleaved accumulators, longer runs split at n/2 rounded down to a
// multiple of 8 (verified against np.sum).  np.std(finite) is
// sqrt(pairwise((x - m)^2) / n) with m = pairwise(x) / n, all float32.  The
// finite pixels form a compacted sequence; a per-1024-pixel finite-count
// prefix maps a compacted index back to raster order.  One CTA walks the
// frames of the batch in turn and only works on frames whose MAD is zero.
constexpr int kPwBlock = 1024;

struct PwArgs {
  const float* slots;
  const int* slot_of_frame;
  int64_t stride;
  int64_t pixels;
  const int* frames;
  int count;
  StarFrameState* state;
  double* rms;     // [count]
  int* prefix;     // [pixels / kPwBlock + 2]
  int2* leaves;    // [pixels / 64 + 2]
  float* leaf_sum; // [pixels / 64 + 2]
};

// Position of the `c`-th finite pixel (compacted index) in raster order.
__device__ int64_t finite_position(const float* src, const int* prefix, int nblocks, int64_t pixels, int64_t c,
                                   bool dense) {
  if (dense) return c;
  int lo = 0, hi = nblocks;  // last block with prefix <= c
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (prefix[mid] <= c) lo = mid; else hi = mid;
  }
  int64_t p = static_cast<int64_t>(lo) * kPwBlock;
  int64_t seen = prefix[lo];
  for (; p < pixels; ++p) {
    if (isfinite(src[p])) {
      if (seen == c) return p;
      ++seen;
    }
  }
  return pixels;
}

__device__ float pw_leaf(const float* src, const int* prefix, int nblocks, int64_t pixels, bool dense, int64_t off,
                         int len, bool square, float mean) {
  int64_t p = finite_position(src, prefix, nblocks, pixels, off, dense);
  auto next = [&]() -> float {
    while (!isfinite(src[p])) ++p;
    float v = src[p++];
    if (square) {
      const float d = __fsub_rn(v, mean);
      v = __fmul_rn(d, d);
    }
    return v;
  };
  if (len < 8) {
    float r = 0.0f;
    for (int i = 0; i < len; ++i) r = __fadd_rn(r, next());
    return r;
  }
  float r[8];
  for (int j = 0; j < 8; ++j) r[j] = next();
  int i = 8;
  for (; i < len - (len % 8); i += 8)
    for (int j = 0; j < 8; ++j) r[j] = __fadd_rn(r[j], next());
  float res = __fadd_rn(__fadd_rn(__fadd_rn(r[0], r[1]), __fadd_rn(r[2], r[3])),
                        __fadd_rn(__fadd_rn(r[4], r[5]), __fadd_rn(r[6], r[7])));
  for (; i < len; ++i) res = __fadd_rn(res, next());
  return res;
}

__device__ __forceinline__ int64_t pw_split(int64_t n) {
  int64_t n2 = n / 2;
  return n2 - n2 % 8;
}

// Thread 0: leaves of the pairwise tree in left-to-right order.
__device__ int pw_leaves(int64_t n, int2* leaves) {
  int64_t st_off[96], st_n[96];
  int top = 0, count = 0;
  st_off[0] = 0;
  st_n[0] = n;
  top = 1;
  while (top > 0) {
    --top;
    const int64_t off = st_off[top], m = st_n[top];
    if (m <= 128) {
      leaves[count++] = make_int2(static_cast<int>(off), static_cast<int>(m));
    } else {
      const int64_t m2 = pw_split(m);
      st_off[top] = off + m2;
      st_n[top] = m - m2;
      ++top;
      st_off[top] = off;
      st_n[top] = m2;
      ++top;
    }
  }
  return count;
}

// Thread 0: fold the leaf sums in the tree's order (left + right at each node).
__device__ float pw_fold(int64_t n, const float* leaf_sum) {
  int64_t node_n[96];
  int node_state[96];
  float vals[96];
  int top = 1, vtop = 0, next = 0;
  node_n[0] = n;
  node_state[0] = 0;
  while (top > 0) {
    const int64_t m = node_n[top - 1];
    if (m <= 128) {
      --top;
      vals[vtop++] = leaf_sum[next++];
    } else if (node_state[top - 1] == 0) {
      node_state[top - 1] = 1;
      const int64_t m2 = pw_split(m);
      node_n[top] = m - m2;
      node_state[top] = 0;
      ++top;
      node_n[top] = m2;
      node_state[top] = 0;
      ++top;
    } else {
      --top;
      const float b = vals[--vtop];
      const float a = vals[--vtop];
      vals[vtop++] = __fadd_rn(a, b);
    }
  }
  return vals[0];
}

__global__ void __launch_bounds__(1024) pairwise_std_kernel(PwArgs a) {
  __shared__ int s_leaves;
  __shared__ float s_mean;
  const int nblocks = static_cast<int>((a.pixels + kPwBlock - 1) / kPwBlock);
  for (int k = 0; k < a.count; ++k) {
    const StarFrameState& st = a.state[k];
    if (st.count == 0 || !(1.4826 * static_cast<double>(st.mad) <= 0.0)) continue;  // uniform branch
    const float* src = a.slots + static_cast<int64_t>(a.slot_of_frame[a.frames[k]]) * a.stride;
    const bool dense = static_cast<int64_t>(st.count) == a.pixels;
    if (!dense) {
      // finite counts per block, then an exclusive prefix (thread 0)
      for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
        int c = 0;
        const int64_t p1 = min(a.pixels, static_cast<int64_t>(b + 1) * kPwBlock);
        for (int64_t p = static_cast<int64_t>(b) * kPwBlock; p < p1; ++p) c += isfinite(src[p]) ? 1 : 0;
        a.prefix[b + 1] = c;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        a.prefix[0] = 0;
        for (int b = 1; b <= nblocks; ++b) a.prefix[b] += a.prefix[b - 1];
      }
    }
    const int64_t n = st.count;
    if (threadIdx.x == 0) s_leaves = pw_leaves(n, a.leaves);
    __syncthreads();
    const int L = s_leaves;
    for (int pass = 0; pass < 2; ++pass) {
      const float mean = pass ? s_mean : 0.0f;
      for (int l = threadIdx.x; l < L; l += blockDim.x) {
        const int2 lf = a.leaves[l];
        a.leaf_sum[l] = pw_leaf(src, a.prefix, nblocks, a.pixels, dense, lf.x, lf.y, pass == 1, mean);
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        const float total = pw_fold(n, a.leaf_sum);
        const float fn = static_cast<float>(n);
        if (pass == 0) {
          s_mean = __fdiv_rn(total, fn);
        } else {
          a.rms[k] = static_cast<double>(__fsqrt_rn(__fdiv_rn(total, fn)));
        }
      }
      __syncthreads();
    }
  }
}

// ---- host side -------------------------------------------------------------------
void ensure_catalog_storage(gg_stack* s) {
  if (s->d_cat_xy) return;
  check_cuda(cudaMalloc(&s->d_cat_xy, sizeof(double) * 2 * kCatalogPoints * s->frames), "cudaMalloc(catalogs)");
  check_cuda(cudaMalloc(&s->d_cat_n, sizeof(int) * s->frames), "cudaMalloc(catalog counts)");
  check_cuda(cudaMemsetAsync(s->d_cat_n, 0, sizeof(int) * s->frames, s->stream), "cudaMemsetAsync(catalogs)");
  s->bytes_allocated += static_cast<int64_t>(sizeof(double) * 2 * kCatalogPoints * s->frames + sizeof(int) * s->frames);
}

struct StarScratch {
  StarFrameState* state = nullptr;
  unsigned* hist = nullptr;
  unsigned* cand = nullptr;
  StarRec* recs = nullptr;
  int* kept = nullptr;
  gg_star_t* out = nullptr;
  int* frames = nullptr;
  double* rms = nullptr;
  int* pw_prefix = nullptr;
  int2* pw_leaves = nullptr;
  float* pw_sums = nullptr;
  int64_t pw_pixels = 0;
  int capacity_frames = 0;
  int max_stars = 0;
  double* mesh_bg = nullptr;  // [frames][cells]
  double* mesh_nz = nullptr;
  int64_t mesh_cap = 0;       // doubles per array
  unsigned* band = nullptr;   // sample-bracket key buffers
  int64_t band_elems = 0;
};

static void free_star_scratch(StarScratch& s) {
  void* ps[] = {s.state,  s.hist,      s.cand,      s.recs,    s.kept,    s.out,    s.frames,
                s.rms,    s.pw_prefix, s.pw_leaves, s.pw_sums, s.mesh_bg, s.mesh_nz, s.band};
  for (void* p : ps)
    if (p) cudaFree(p);
  s = StarScratch{};
}

static void ensure_star_scratch(StarScratch& s, int frames, int max_stars) {
  if (s.capacity_frames >= frames && s.max_stars >= max_stars) return;
  free_star_scratch(s);
  const size_t f = static_cast<size_t>(frames);
  check_cuda(cudaMalloc(&s.state, sizeof(StarFrameState) * f), "cudaMalloc(star state)");
  check_cuda(cudaMalloc(&s.hist, sizeof(unsigned) * f * 2 * kSelBins), "cudaMalloc(star hist)");
  check_cuda(cudaMalloc(&s.cand, sizeof(unsigned) * f * kMaxCandidates), "cudaMalloc(star candidates)");
  check_cuda(cudaMalloc(&s.recs, sizeof(StarRec) * f * kMaxCandidates), "cudaMalloc(star records)");
  check_cuda(cudaMalloc(&s.kept, sizeof(int) * f * kMaxCandidates), "cudaMalloc(star kept)");
  check_cuda(cudaMalloc(&s.out, sizeof(gg_star_t) * f * static_cast<size_t>(max_stars)), "cudaMalloc(star out)");
  check_cuda(cudaMalloc(&s.frames, sizeof(int) * f), "cudaMalloc(star frames)");
  check_cuda(cudaMalloc(&s.rms, sizeof(double) * f), "cudaMalloc(star rms)");
  s.capacity_frames = frames;
  s.max_stars = max_stars;
}

// Scratch lives with the stack (freed by gg_stack_destroy through the hook).
static StarScratch& star_scratch(gg_stack* s) {
  if (!s->star_scratch) {
    s->star_scratch = new StarScratch();
    s->star_scratch_free = [](void* p) {
      auto* sc = static_cast<StarScratch*>(p);
      free_star_scratch(*sc);
      delete sc;
    };
  }
  return *static_cast<StarScratch*>(s->star_scratch);
}

__global__ void star_rms_kernel(const double* partials, int blocks, int count, double* rms) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  double s1 = 0.0, s2 = 0.0, n = 0.0;
  for (int b = 0; b < blocks; ++b) {
    const double* q = partials + (static_cast<int64_t>(k) * blocks + b) * 3;
    s1 += q[0];
    s2 += q[1];
    n += q[2];
  }
  const double mean = n > 0 ? s1 / n : 0.0;
  const double var = n > 0 ? fmax(s2 / n - mean * mean, 0.0) : 0.0;
  rms[k] = sqrt(var);
}

void launch_frame_stats_partials(gg_stack* s, const int* d_frames, int count, int blocks, double* partials);

void detect_stars(gg_stack* s, const int64_t* indices, int count, const gg_star_params_t& p) {
  StarScratch& sc = star_scratch(s);
  ensure_star_scratch(sc, count, p.max_stars);
  std::vector<int> frames(static_cast<size_t>(count));
  for (int k = 0; k < count; ++k) frames[static_cast<size_t>(k)] = static_cast<int>(indices[k]);
  upload_params(s->stream, sc.frames, frames.data(), sizeof(int) * count, "cudaMemcpyAsync(star frames)");
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(star frames)");
  check_cuda(cudaMemsetAsync(sc.state, 0, sizeof(StarFrameState) * count, s->stream), "cudaMemsetAsync(state)");
  const bool need_stats = !std::isfinite(p.background) || !std::isfinite(p.noise);
  SelectArgs sa{};
  sa.slots = s->d_slots;
  sa.slot_of_frame = s->d_slot_of_frame;
  sa.stride = s->stride;
  sa.pixels = s->pixels;
  sa.frames = sc.frames;
  sa.state = sc.state;
  sa.hist = sc.hist;
  const unsigned per_frame =
      std::max(1u, std::min<unsigned>(static_cast<unsigned>((s->pixels + 255) / 256),
                                      std::max(1u, static_cast<unsigned>(sm_count() * 8 / std::max(count, 1)))));
  double* rms = nullptr;
  if (need_stats) {
    // band buffers of the sample-bracket selection: a sixteenth of the frame
    // (the band holds ~2.5 % of a 9600 x 6422 frame's pixels)
    const int64_t band_cap = std::min<int64_t>(s->pixels, std::max<int64_t>(65536, s->pixels / 16));
    if (sc.band_elems < band_cap * count) {
      if (sc.band) cudaFree(sc.band);
      sc.band = nullptr;
      sc.band_elems = 0;
      check_cuda(cudaMalloc(&sc.band, sizeof(unsigned) * band_cap * count), "cudaMalloc(bracket band)");
      sc.band_elems = band_cap * count;
    }
    BracketArgs ba{s->d_slots, s->d_slot_of_frame, s->stride, s->pixels, sc.frames, sc.state, sc.band, band_cap, 0};
    ba.ghist = sc.hist;  // [count][2][kSelBins] >= 512 words per frame; the radix fallback zeroes it again
    ba.count_frames = count;
    // CTAs per frame for the band histograms: about eight waves of the GPU's SMs over all frames
    const unsigned band_ctas = static_cast<unsigned>(std::max(1, std::min(64, sm_count() * 8 / std::max(count, 1))));
    const int samples = static_cast<int>(std::min<int64_t>(kBracketSamples, s->pixels));
    int sample_pow2 = 1;
    while (sample_pow2 < samples) sample_pow2 <<= 1;
    const size_t sample_smem = sizeof(unsigned) * static_cast<size_t>(sample_pow2);
    check_cuda(cudaFuncSetAttribute(bracket_sample_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(sample_smem)),
               "cudaFuncSetAttribute(bracket sample)");
    for (int mode = 0; mode < 2; ++mode) {
      sa.mode = mode;
      ba.mode = mode;
      note_launch(3);
      bracket_sample_kernel<<<static_cast<unsigned>(count), 1024, sample_smem, s->stream>>>(ba);
      if (mode == 0)
        bracket_pass_kernel<0><<<dim3(per_frame, static_cast<unsigned>(count)), kBracketThreads, 0, s->stream>>>(ba);
      else
        bracket_pass_kernel<1><<<dim3(per_frame, static_cast<unsigned>(count)), kBracketThreads, 0, s->stream>>>(ba);
      check_cuda(cudaGetLastError(), "bracket select launch");
      note_launch(2);
      bracket_band_init_kernel<<<static_cast<unsigned>(count), 32, 0, s->stream>>>(ba);
      for (int pass = 0; pass < 4; ++pass) {
        ba.pass = pass;
        note_launch(2);
        bracket_band_hist_kernel<<<dim3(band_ctas, static_cast<unsigned>(count)), 256, 0, s->stream>>>(ba);
        bracket_band_digit_kernel<<<static_cast<unsigned>(count), 32, 0, s->stream>>>(ba);
      }
      bracket_band_finish_kernel<<<(count + 127) / 128, 128, 0, s->stream>>>(ba);
      check_cuda(cudaGetLastError(), "bracket band select launch");
      // frames the bracket could not settle: three-pass radix select
      for (int pass = 0; pass < 3; ++pass) {
        sa.pass = pass;
        check_cuda(cudaMemsetAsync(sc.hist, 0, sizeof(unsigned) * count * 2 * kSelBins, s->stream),
                   "cudaMemsetAsync(hist)");
        note_launch();
        const dim3 hist_grid(per_frame, static_cast<unsigned>(count));
        if (pass == 0) select_hist_kernel<0><<<hist_grid, 256, 0, s->stream>>>(sa);
        else if (pass == 1) select_hist_kernel<1><<<hist_grid, 256, 0, s->stream>>>(sa);
        else select_hist_kernel<2><<<hist_grid, 256, 0, s->stream>>>(sa);
        check_cuda(cudaGetLastError(), "select_hist launch");
        note_launch();
        select_scan_kernel<<<static_cast<unsigned>(count), 256, 0, s->stream>>>(sa, count);
        check_cuda(cudaGetLastError(), "select_scan launch");
      }
    }
    // np.std of the finite pixels, the fallback noise when the MAD is zero
    // (star_detect.py:35-41); computed only for such frames.
    if (sc.pw_pixels != s->pixels) {
      if (sc.pw_prefix) cudaFree(sc.pw_prefix);
      if (sc.pw_leaves) cudaFree(sc.pw_leaves);
      if (sc.pw_sums) cudaFree(sc.pw_sums);
      const size_t nb = static_cast<size_t>(s->pixels / kPwBlock + 2);
      // leaves hold >= 57 elements once n > 128 (split at n/2 rounded down to 8)
      const size_t nl = static_cast<size_t>(s->pixels / 32 + 2);
      check_cuda(cudaMalloc(&sc.pw_prefix, sizeof(int) * nb), "cudaMalloc(pairwise prefix)");
      check_cuda(cudaMalloc(&sc.pw_leaves, sizeof(int2) * nl), "cudaMalloc(pairwise leaves)");
      check_cuda(cudaMalloc(&sc.pw_sums, sizeof(float) * nl), "cudaMalloc(pairwise sums)");
      sc.pw_pixels = s->pixels;
    }
    PwArgs pa{};
    pa.slots = s->d_slots;
    pa.slot_of_frame = s->d_slot_of_frame;
    pa.stride = s->stride;
    pa.pixels = s->pixels;
    pa.frames = sc.frames;
    pa.count = count;
    pa.state = sc.state;
    pa.rms = sc.rms;
    pa.prefix = sc.pw_prefix;
    pa.leaves = sc.pw_leaves;
    pa.leaf_sum = sc.pw_sums;
    rms = sc.rms;
    note_launch();
    pairwise_std_kernel<<<1, 1024, 0, s->stream>>>(pa);
    check_cuda(cudaGetLastError(), "pairwise_std launch");
  }
  note_launch();
  star_threshold_kernel<<<(count + 127) / 128, 128, 0, s->stream>>>(
      sc.state, count, p.threshold_sigma, std::isfinite(p.background) ? 1 : 0, p.background,
      std::isfinite(p.noise) ? 1 : 0, p.noise, rms);
  check_cuda(cudaGetLastError(), "star_threshold launch");
  if (s->width < 3 || s->height < 3) return;  // no interior (star_detect.py:140-141)
  DetectArgs da{};
  da.slots = s->d_slots;
  da.slot_of_frame = s->d_slot_of_frame;
  da.stride = s->stride;
  da.width = static_cast<int>(s->width);
  da.height = static_cast<int>(s->height);
  da.frames = sc.frames;
  da.state = sc.state;
  da.cand = sc.cand;
  da.k_sigma = static_cast<double>(p.threshold_sigma);
  if (p.mesh_cell > 0) {
    MeshArgs ma{};
    ma.cell = p.mesh_cell;
    ma.nx = static_cast<int>((s->width + p.mesh_cell - 1) / p.mesh_cell);
    ma.ny = static_cast<int>((s->height + p.mesh_cell - 1) / p.mesh_cell);
    const int64_t need = static_cast<int64_t>(ma.nx) * ma.ny * count;
    if (sc.mesh_cap < need) {
      if (sc.mesh_bg) cudaFree(sc.mesh_bg);
      if (sc.mesh_nz) cudaFree(sc.mesh_nz);
      sc.mesh_bg = sc.mesh_nz = nullptr;
      sc.mesh_cap = 0;
      check_cuda(cudaMalloc(&sc.mesh_bg, sizeof(double) * need), "cudaMalloc(background mesh)");
      check_cuda(cudaMalloc(&sc.mesh_nz, sizeof(double) * need), "cudaMalloc(noise mesh)");
      sc.mesh_cap = need;
    }
    ma.slots = s->d_slots;
    ma.slot_of_frame = s->d_slot_of_frame;
    ma.stride = s->stride;
    ma.width = static_cast<int>(s->width);
    ma.height = static_cast<int>(s->height);
    ma.frames = sc.frames;
    ma.bg = sc.mesh_bg;
    ma.nz = sc.mesh_nz;
    note_launch();
    mesh_stats_kernel<<<dim3(static_cast<unsigned>(ma.nx * ma.ny), static_cast<unsigned>(count)), 1024, 0,
                        s->stream>>>(ma);
    check_cuda(cudaGetLastError(), "mesh_stats launch");
    da.mesh = MeshView{sc.mesh_bg, sc.mesh_nz, ma.cell, ma.nx, ma.ny};
  }
  note_launch();
  const unsigned detect_rows = static_cast<unsigned>(std::max<int64_t>(
      1, std::min<int64_t>(s->height - 2, std::max<int64_t>(1, sm_count() * 8 / std::max(count, 1)))));
  if (da.mesh.bg)
    star_detect_kernel<true><<<dim3(detect_rows, static_cast<unsigned>(count)), 256, 0, s->stream>>>(da);
  else
    star_detect_kernel<false><<<dim3(detect_rows, static_cast<unsigned>(count)), 256, 0, s->stream>>>(da);
  check_cuda(cudaGetLastError(), "star_detect launch");
  CatalogArgs ca{};
  ca.slots = s->d_slots;
  ca.slot_of_frame = s->d_slot_of_frame;
  ca.stride = s->stride;
  ca.width = da.width;
  ca.height = da.height;
  ca.frames = sc.frames;
  ca.state = sc.state;
  ca.cand = sc.cand;
  ca.recs = sc.recs;
  ca.kept = sc.kept;
  ca.out = sc.out;
  ca.max_stars = p.max_stars;
  ca.radius = std::max(1, p.window_radius);
  ca.min_sep = p.min_separation_px;
  ca.error = s->d_error;
  ensure_catalog_storage(s);
  ca.cat_xy = s->d_cat_xy;
  ca.cat_n = s->d_cat_n;
  ca.mesh = da.mesh;
  const size_t sort_smem = sizeof(unsigned) * kMaxCandidates;
  check_cuda(cudaFuncSetAttribute(star_sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(sort_smem)),
             "cudaFuncSetAttribute(star sort)");
  note_launch();
  star_sort_kernel<<<static_cast<unsigned>(count), 1024, sort_smem, s->stream>>>(ca);
  check_cuda(cudaGetLastError(), "star_sort launch");
  note_launch();
  star_measure_kernel<<<dim3(64, static_cast<unsigned>(count)), 256, 0, s->stream>>>(ca);
  check_cuda(cudaGetLastError(), "star_measure launch");
  const size_t sel_smem = 16 * 4096;
  check_cuda(cudaFuncSetAttribute(star_select_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(sel_smem)),
             "cudaFuncSetAttribute(star select)");
  note_launch();
  star_select_kernel<<<static_cast<unsigned>(count), 1024, sel_smem, s->stream>>>(ca);
  check_cuda(cudaGetLastError(), "star_select launch");
  const unsigned mom_blocks = static_cast<unsigned>(std::max(1, std::min(64, (p.max_stars * 32 + 255) / 256)));
  note_launch();
  star_moments_kernel<<<dim3(mom_blocks, static_cast<unsigned>(count)), 256, 0, s->stream>>>(ca);
  check_cuda(cudaGetLastError(), "star_moments launch");
  note_launch();
  star_catalog_kernel<<<static_cast<unsigned>(count), 32, 0, s->stream>>>(ca, p.catalog_min_fwhm,
                                                                           p.catalog_max_eccentricity);
  check_cuda(cudaGetLastError(), "star_catalog launch");
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_stack_detect_stars(gg_stack* s, const int64_t* indices, int64_t count, const gg_star_params_t* params,
                          gg_star_t* host_stars, int32_t* host_counts, gg_star_frame_info_t* host_info) {
  GG_API_BEGIN
  require(s != nullptr && indices != nullptr && params != nullptr, "null argument");
  require(count > 0 && count <= 65535, "frame count must be in [1, 65535]");
  const gg_star_params_t& p = *params;
  require(p.max_stars >= 1 && p.max_stars <= 4096, "max_stars must be in [1, 4096]");
  require(p.window_radius >= 0 && p.window_radius <= 16, "window_radius must be in [0, 16]");
  require(std::isfinite(p.threshold_sigma), "threshold_sigma must be finite");
  require(std::isfinite(p.min_separation_px), "min_separation_px must be finite");
  require(std::isfinite(p.catalog_min_fwhm) && std::isfinite(p.catalog_max_eccentricity),
          "catalog filter thresholds must be finite");
  require(p.mesh_cell == 0 || (p.mesh_cell >= 8 && p.mesh_cell <= kMeshMaxCell), "mesh_cell must be 0 or in [8, 64]");
  require(p.mesh_cell == 0 || (std::isnan(p.background) && std::isnan(p.noise)),
          "a background mesh estimates background and noise itself (pass NaN)");
  for (int64_t k = 0; k < count; ++k) stack_require_loaded(s, indices[k], "star detection");
  stack_activate(s);
  detect_stars(s, indices, static_cast<int>(count), p);
  StarScratch& sc = star_scratch(s);
  std::vector<StarFrameState> st(static_cast<size_t>(count));
  check_cuda(cudaMemcpyAsync(st.data(), sc.state, sizeof(StarFrameState) * count, cudaMemcpyDeviceToHost, s->stream),
             "cudaMemcpyAsync(star state)");
  if (host_stars) {
    check_cuda(cudaMemcpyAsync(host_stars, sc.out, sizeof(gg_star_t) * count * p.max_stars, cudaMemcpyDeviceToHost,
                               s->stream),
               "cudaMemcpyAsync(stars)");
  }
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(stars)");
  stack_check_device_error(s);
  for (int64_t k = 0; k < count; ++k) {
    const StarFrameState& f = st[static_cast<size_t>(k)];
    if (f.overflow) fail(GG_ERR_RUNTIME, "more than 32768 star candidates in one frame; raise threshold_sigma");
    if (host_counts) host_counts[k] = (s->width < 3 || s->height < 3) ? 0 : f.kept;
    if (host_info) {
      host_info[k].median = f.median;
      host_info[k].mad = f.mad;
      host_info[k].noise = f.noise;
      host_info[k].threshold = f.threshold;
      host_info[k].candidates = static_cast<int64_t>(f.candidates);
      host_info[k].valid_pixels = static_cast<int64_t>(f.count);
    }
  }
  GG_API_END
}

}  // extern "C"

// ---- isolated cosmetic defects (source DQ) ------------------------------------
// cpu/cosmetic.py:97-307 on resident frames: a finite pixel is a hot (cold)
// candidate when it exceeds float32(median + k_hot sigma) (is below
// float32(median - k_cold sigma)) and its distance to the float32 median of
// its finite 8-neighbours (edge-clamped; float32 (a + b) / 2 for an even
// count; the global median without any) exceeds float32(k sigma); it is a
// defect when fewer than min_support neighbours pass float32(median -/+
// max(0, structure_sigma) sigma) on the same side; the protected variant
// keeps defects inside the radius of catalog stars with npix >= min_pixels
// and sharpness <= max_sharpness.  median and sigma are the frame's star-
// detection statistics (the same robust_background).  Defects become NaN
// (resident_source_dq.py:825-925: no replacement).
namespace gg {

struct CosmeticArgs {
  const float* slots;
  const int* slot_of_frame;
  int64_t stride;
  int width, height;
  const int* frames;
  const StarFrameState* state;
  const gg_star_t* stars;  // [count][max_stars] (protected variant)
  int max_stars;
  unsigned* hot_bits;      // [count][words]
  unsigned* cold_bits;
  int64_t words;
  unsigned long long* counts;  // [count][8]
  double hot_sigma, cold_sigma, support_sigma;
  int min_support;
  int protect;
  int min_pixels;
  double max_sharpness, radius_sq;
};

__device__ __forceinline__ bool star_protected(const CosmeticArgs& a, int k, int x, int y) {
  const int n = a.state[k].kept;
  const gg_star_t* st = a.stars + static_cast<int64_t>(k) * a.max_stars;
  for (int i = 0; i < n; ++i) {
    const gg_star_t s = st[i];
    if (s.npix < a.min_pixels || s.sharpness > a.max_sharpness) continue;
    if (!isfinite(s.x) || !isfinite(s.y)) continue;
    const double dx = static_cast<double>(x) - s.x, dy = static_cast<double>(y) - s.y;
    if (__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)) <= a.radius_sq) return true;
  }
  return false;
}

__global__ void __launch_bounds__(256) cosmetic_classify_kernel(CosmeticArgs a) {
  __shared__ unsigned long long s_counts[8];
  if (threadIdx.x < 8) s_counts[threadIdx.x] = 0;
  __syncthreads();
  const int k = blockIdx.y;
  const float* img = a.slots + static_cast<int64_t>(a.slot_of_frame[a.frames[k]]) * a.stride;
  const StarFrameState& st = a.state[k];
  const double med = static_cast<double>(st.median), sigma = st.noise;
  const float medf = st.median;
  const float hot_limit = __double2float_rn(__dadd_rn(med, __dmul_rn(a.hot_sigma, sigma)));
  const float cold_limit = __double2float_rn(__dsub_rn(med, __dmul_rn(a.cold_sigma, sigma)));
  const float hot_delta = __double2float_rn(__dmul_rn(a.hot_sigma, sigma));
  const float cold_delta = __double2float_rn(__dmul_rn(a.cold_sigma, sigma));
  const float sup_hi = __double2float_rn(__dadd_rn(med, __dmul_rn(a.support_sigma, sigma)));
  const float sup_lo = __double2float_rn(__dsub_rn(med, __dmul_rn(a.support_sigma, sigma)));
  const int W = a.width, H = a.height;
  const int64_t P = static_cast<int64_t>(W) * H;
  unsigned c_hot = 0, c_cold = 0, c_cand_hot = 0, c_cand_cold = 0, c_prot_hot = 0, c_prot_cold = 0;
  for (int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; p < P;
       p += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const float v = __ldg(img + p);
    if (!isfinite(v) || !(v > hot_limit || v < cold_limit)) continue;  // only global outliers go on
    const int y = static_cast<int>(p / W), x = static_cast<int>(p - static_cast<int64_t>(y) * W);
    float nb[8];
    int n = 0, hs = 0, cs = 0;
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
      for (int dx = -1; dx <= 1; ++dx) {
        if (!dx && !dy) continue;
        const int yy = min(max(y + dy, 0), H - 1), xx = min(max(x + dx, 0), W - 1);
        const float u = __ldg(img + static_cast<int64_t>(yy) * W + xx);
        if (isfinite(u)) {
          nb[n++] = u;
          hs += u > sup_hi;
          cs += u < sup_lo;
        }
      }
    for (int i = 1; i < n; ++i) {  // insertion sort of <= 8 values
      const float t = nb[i];
      int j = i - 1;
      while (j >= 0 && nb[j] > t) {
        nb[j + 1] = nb[j];
        --j;
      }
      nb[j + 1] = t;
    }
    const float lmed = n == 0 ? medf : ((n & 1) ? nb[n / 2] : __fmul_rn(__fadd_rn(nb[n / 2 - 1], nb[n / 2]), 0.5f));
    const bool cand_hot = v > hot_limit && __fsub_rn(v, lmed) > hot_delta;
    const bool cand_cold = v < cold_limit && __fsub_rn(lmed, v) > cold_delta;
    c_cand_hot += cand_hot;
    c_cand_cold += cand_cold;
    bool hot = cand_hot && hs < a.min_support;
    bool cold = cand_cold && cs < a.min_support;
    if ((hot || cold) && a.protect && star_protected(a, k, x, y)) {
      c_prot_hot += hot;
      c_prot_cold += cold;
      hot = cold = false;
    }
    const int64_t word = static_cast<int64_t>(k) * a.words + (p >> 5);
    const unsigned bit = 1u << (p & 31);
    if (hot) {
      ++c_hot;
      atomicOr(a.hot_bits + word, bit);
    }
    if (cold) {
      ++c_cold;
      atomicOr(a.cold_bits + word, bit);
    }
  }
  const unsigned vals[6] = {c_hot, c_cold, c_cand_hot, c_cand_cold, c_prot_hot, c_prot_cold};
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    unsigned v = vals[i];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(&s_counts[i], static_cast<unsigned long long>(v));
  }
  __syncthreads();
  if (threadIdx.x < 6 && s_counts[threadIdx.x])
    atomicAdd(a.counts + static_cast<int64_t>(k) * 8 + threadIdx.x, s_counts[threadIdx.x]);
}

// Defects -> NaN; the frame's non-finite counter grows by the pixels set.
__global__ void __launch_bounds__(256) cosmetic_apply_kernel(CosmeticArgs a, unsigned* frame_nonfinite) {
  const int k = blockIdx.y;
  float* img = const_cast<float*>(a.slots) + static_cast<int64_t>(a.slot_of_frame[a.frames[k]]) * a.stride;
  const int64_t P = static_cast<int64_t>(a.width) * a.height;
  unsigned added = 0;
  for (int64_t w = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; w < a.words;
       w += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    unsigned bits = a.hot_bits[static_cast<int64_t>(k) * a.words + w] | a.cold_bits[static_cast<int64_t>(k) * a.words + w];
    while (bits) {
      const int b = __ffs(bits) - 1;
      bits &= bits - 1;
      const int64_t p = w * 32 + b;
      if (p < P) {
        img[p] = __int_as_float(0x7fc00000);
        ++added;
      }
    }
  }
  for (int off = 16; off > 0; off >>= 1) added += __shfl_xor_sync(0xffffffffu, added, off);
  if ((threadIdx.x & 31) == 0 && added) atomicAdd(frame_nonfinite + a.frames[k], added);
}

}  // namespace gg

extern "C" int gg_stack_cosmetic_mask(gg_stack* s, const int64_t* indices, int64_t count,
                                      const gg_cosmetic_params_t* params, gg_cosmetic_result_t* host_out) {
  using namespace gg;
  GG_API_BEGIN
  require(s != nullptr && indices != nullptr && params != nullptr, "null argument");
  require(count > 0 && count <= 65535, "frame count must be in [1, 65535]");
  const gg_cosmetic_params_t& p = *params;
  require(std::isfinite(p.hot_sigma) && std::isfinite(p.cold_sigma) && std::isfinite(p.structure_sigma),
          "cosmetic sigmas must be finite");
  require(!p.star_protection || (std::isfinite(p.star_protection_radius_px) && std::isfinite(p.star_threshold_sigma) &&
                                 std::isfinite(p.star_max_sharpness)),
          "star protection parameters must be finite");
  for (int64_t k = 0; k < count; ++k) stack_require_loaded(s, indices[k], "cosmetic defect detection");
  stack_activate(s);
  gg_star_params_t sp{};
  sp.threshold_sigma = p.star_threshold_sigma;
  sp.max_stars = 500;
  sp.window_radius = 4;
  sp.min_separation_px = std::max(2.0f, p.star_protection_radius_px * 0.5f);
  sp.background = std::nanf("");
  sp.noise = std::nanf("");
  sp.catalog_min_fwhm = 0.0f;
  sp.catalog_max_eccentricity = 1.0f;
  sp.mesh_cell = 0;
  detect_stars(s, indices, static_cast<int>(count), sp);
  StarScratch& sc = star_scratch(s);
  const int64_t words = (s->pixels + 31) / 32;
  unsigned* bits = nullptr;
  unsigned long long* counts = nullptr;
  check_cuda(cudaMallocAsync(reinterpret_cast<void**>(&bits), sizeof(unsigned) * words * count * 2, s->stream),
             "cudaMallocAsync(cosmetic bits)");
  check_cuda(cudaMallocAsync(reinterpret_cast<void**>(&counts), sizeof(unsigned long long) * 8 * count, s->stream),
             "cudaMallocAsync(cosmetic counts)");
  check_cuda(cudaMemsetAsync(bits, 0, sizeof(unsigned) * words * count * 2, s->stream), "cudaMemsetAsync(bits)");
  check_cuda(cudaMemsetAsync(counts, 0, sizeof(unsigned long long) * 8 * count, s->stream), "cudaMemsetAsync(counts)");
  CosmeticArgs a{};
  a.slots = s->d_slots;
  a.slot_of_frame = s->d_slot_of_frame;
  a.stride = s->stride;
  a.width = static_cast<int>(s->width);
  a.height = static_cast<int>(s->height);
  a.frames = sc.frames;
  a.state = sc.state;
  a.stars = sc.out;
  a.max_stars = sp.max_stars;
  a.hot_bits = bits;
  a.cold_bits = bits + words * count;
  a.words = words;
  a.counts = counts;
  a.hot_sigma = p.hot_sigma;
  a.cold_sigma = p.cold_sigma;
  a.support_sigma = std::max(0.0, static_cast<double>(p.structure_sigma));
  a.min_support = std::max(0, p.min_neighbor_support);
  a.protect = p.star_protection ? 1 : 0;
  a.min_pixels = p.star_min_pixels;
  a.max_sharpness = p.star_max_sharpness;
  const double r = std::max(0.0, static_cast<double>(p.star_protection_radius_px));
  a.radius_sq = r * r;
  if (!(r > 0.0)) a.protect = 0;
  const unsigned per_frame = grid_for(static_cast<size_t>(s->pixels), 256, std::max(1, 8 / static_cast<int>(std::min<int64_t>(count, 8))));
  note_launch();
  cosmetic_classify_kernel<<<dim3(per_frame, static_cast<unsigned>(count)), 256, 0, s->stream>>>(a);
  check_cuda(cudaGetLastError(), "cosmetic_classify launch");
  if (p.apply) {
    note_launch();
    cosmetic_apply_kernel<<<dim3(std::max(1u, static_cast<unsigned>(std::min<int64_t>((words + 255) / 256, 1024))),
                                 static_cast<unsigned>(count)), 256, 0, s->stream>>>(a, s->d_frame_nonfinite);
    check_cuda(cudaGetLastError(), "cosmetic_apply launch");
  }
  std::vector<unsigned long long> host(static_cast<size_t>(8 * count));
  std::vector<StarFrameState> states(static_cast<size_t>(count));
  check_cuda(cudaMemcpyAsync(host.data(), counts, sizeof(unsigned long long) * 8 * count, cudaMemcpyDeviceToHost,
                             s->stream),
             "cudaMemcpyAsync(cosmetic counts)");
  check_cuda(cudaMemcpyAsync(states.data(), sc.state, sizeof(StarFrameState) * count, cudaMemcpyDeviceToHost, s->stream),
             "cudaMemcpyAsync(cosmetic state)");
  check_cuda(cudaFreeAsync(bits, s->stream), "cudaFreeAsync(cosmetic bits)");
  check_cuda(cudaFreeAsync(counts, s->stream), "cudaFreeAsync(cosmetic counts)");
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(cosmetic)");
  if (host_out) {
    for (int64_t k = 0; k < count; ++k) {
      gg_cosmetic_result_t& r = host_out[k];
      const unsigned long long* c = host.data() + 8 * k;
      r.hot_pixels = static_cast<int64_t>(c[0]);
      r.cold_pixels = static_cast<int64_t>(c[1]);
      r.candidate_hot_pixels = static_cast<int64_t>(c[2]);
      r.candidate_cold_pixels = static_cast<int64_t>(c[3]);
      r.star_protected_hot_pixels = static_cast<int64_t>(c[4]);
      r.star_protected_cold_pixels = static_cast<int64_t>(c[5]);
      r.median = static_cast<double>(states[static_cast<size_t>(k)].median);
      r.sigma = states[static_cast<size_t>(k)].noise;
      r.star_count = states[static_cast<size_t>(k)].kept;
      r.pad = 0;
    }
  }
  GG_API_END
}

namespace gg {

// Source-DQ invalid mask (glass_apply_invalid_mask_f32_kernel semantics):
// non-zero mask bytes make the sample NaN; the frame's non-finite counter
// counts the samples that were finite before.
__global__ void __launch_bounds__(256) invalid_mask_kernel(float* img, const unsigned char* mask, int64_t n,
                                                           unsigned* nonfinite) {
  unsigned added = 0;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (mask[i] && isfinite(img[i])) {
      img[i] = __int_as_float(0x7fc00000);
      ++added;
    }
  }
  for (int off = 16; off > 0; off >>= 1) added += __shfl_xor_sync(0xffffffffu, added, off);
  if ((threadIdx.x & 31) == 0 && added) atomicAdd(nonfinite, added);
}

}  // namespace gg

extern "C" int gg_stack_apply_invalid_mask(gg_stack* s, int64_t index, const uint8_t* host_mask,
                                           int64_t* host_invalid_samples) {
  using namespace gg;
  GG_API_BEGIN
  require(s != nullptr && host_mask != nullptr, "null argument");
  stack_require_loaded(s, index, "source-DQ invalid mask");
  stack_activate(s);
  std::vector<int> slots;
  stack_read_slots(s, slots);
  unsigned char* d_mask = nullptr;
  check_cuda(cudaMallocAsync(reinterpret_cast<void**>(&d_mask), static_cast<size_t>(s->pixels), s->stream),
             "cudaMallocAsync(invalid mask)");
  check_cuda(cudaMemcpyAsync(d_mask, host_mask, static_cast<size_t>(s->pixels), cudaMemcpyHostToDevice, s->stream),
             "cudaMemcpyAsync(invalid mask)");
  float* img = s->d_slots + static_cast<int64_t>(slots[static_cast<size_t>(index)]) * s->stride;
  note_launch();
  invalid_mask_kernel<<<grid_for(static_cast<size_t>(s->pixels), 256), 256, 0, s->stream>>>(
      img, d_mask, s->pixels, s->d_frame_nonfinite + index);
  check_cuda(cudaGetLastError(), "invalid_mask launch");
  check_cuda(cudaFreeAsync(d_mask, s->stream), "cudaFreeAsync(invalid mask)");
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(invalid mask)");
  if (host_invalid_samples) {
    int64_t n = 0;
    for (int64_t i = 0; i < s->pixels; ++i) n += host_mask[i] != 0;
    *host_invalid_samples = n;
  }
  GG_API_END
}

namespace gg {

// Threshold-only cosmetic mask (apply / count_cosmetic_threshold_mask_frame(s)
// semantics, integration_kernels.cu:181-232, 266-330): per listed frame a
// sample is non-finite, hot (> high) or cold (< low), tested in that order;
// with `apply` all three become NaN and the frame's non-finite counter grows
// by the hot and cold samples (a non-finite sample was already counted).
// float4 grid-stride loop per frame (slots start 256-byte aligned), one
// store per quad that changed, counts folded per warp.
struct ThresholdFrame {
  int frame;
  float low, high;
  int pad;
};

__device__ __forceinline__ bool threshold_classify(float& x, float low, float high, bool apply, unsigned& hot,
                                                   unsigned& cold, unsigned& nonfinite) {
  bool hit = true;
  if (!isfinite(x)) ++nonfinite;
  else if (x > high) ++hot;
  else if (x < low) ++cold;
  else hit = false;
  if (hit && apply) x = __int_as_float(0x7fc00000);
  return hit && apply;
}

__global__ void __launch_bounds__(256) cosmetic_threshold_kernel(float* slots, const int* slot_of_frame, int64_t stride,
                                                                 int64_t pixels, const ThresholdFrame* frames,
                                                                 int apply, unsigned long long* counts,
                                                                 unsigned* frame_nonfinite) {
  const int k = blockIdx.y;
  const ThresholdFrame tf = frames[k];
  float* img = slots + static_cast<int64_t>(slot_of_frame[tf.frame]) * stride;
  const bool ap = apply != 0;
  unsigned hot = 0, cold = 0, nonf = 0;
  const int64_t quads = pixels / 4;
  const int64_t t0 = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t step = static_cast<int64_t>(gridDim.x) * blockDim.x;
  float4* img4 = reinterpret_cast<float4*>(img);
  for (int64_t q = t0; q < quads; q += step) {
    float4 v = img4[q];
    bool changed = threshold_classify(v.x, tf.low, tf.high, ap, hot, cold, nonf);
    changed |= threshold_classify(v.y, tf.low, tf.high, ap, hot, cold, nonf);
    changed |= threshold_classify(v.z, tf.low, tf.high, ap, hot, cold, nonf);
    changed |= threshold_classify(v.w, tf.low, tf.high, ap, hot, cold, nonf);
    if (changed) img4[q] = v;
  }
  for (int64_t p = quads * 4 + t0; p < pixels; p += step) {
    float x = img[p];
    if (threshold_classify(x, tf.low, tf.high, ap, hot, cold, nonf)) img[p] = x;
  }
  for (int off = 16; off > 0; off >>= 1) {
    hot += __shfl_xor_sync(0xffffffffu, hot, off);
    cold += __shfl_xor_sync(0xffffffffu, cold, off);
    nonf += __shfl_xor_sync(0xffffffffu, nonf, off);
  }
  if ((threadIdx.x & 31) == 0) {
    unsigned long long* c = counts + static_cast<int64_t>(k) * 3;
    if (hot) atomicAdd(c, static_cast<unsigned long long>(hot));
    if (cold) atomicAdd(c + 1, static_cast<unsigned long long>(cold));
    if (nonf) atomicAdd(c + 2, static_cast<unsigned long long>(nonf));
    if (ap && hot + cold) atomicAdd(frame_nonfinite + tf.frame, hot + cold);
  }
}

}  // namespace gg

extern "C" int gg_stack_cosmetic_threshold(gg_stack* s, const int64_t* indices, int64_t count,
                                           const float* low_thresholds, const float* high_thresholds, int32_t apply,
                                           int64_t* host_counts) {
  using namespace gg;
  GG_API_BEGIN
  require(s != nullptr && indices != nullptr && low_thresholds != nullptr && high_thresholds != nullptr,
          "null argument");
  require(count > 0 && count <= 65535, "batch cosmetic threshold application supports at most 65535 frames per launch");
  std::vector<ThresholdFrame> frames(static_cast<size_t>(count));
  for (int64_t k = 0; k < count; ++k) {
    const float lo = low_thresholds[k], hi = high_thresholds[k];
    require(!std::isnan(lo) && !std::isnan(hi) && lo <= hi,
            "cosmetic thresholds must be finite-or-infinite values with low <= high");
    stack_require_loaded(s, indices[k], "source-DQ cosmetic threshold mask");
    frames[static_cast<size_t>(k)] = ThresholdFrame{static_cast<int>(indices[k]), lo, hi, 0};
  }
  stack_activate(s);
  const size_t count_bytes = sizeof(unsigned long long) * 3 * static_cast<size_t>(count);
  const size_t frame_bytes = sizeof(ThresholdFrame) * static_cast<size_t>(count);
  unsigned char* buf = nullptr;
  check_cuda(cudaMallocAsync(reinterpret_cast<void**>(&buf), count_bytes + frame_bytes, s->stream),
             "cudaMallocAsync(cosmetic threshold)");
  auto* d_counts = reinterpret_cast<unsigned long long*>(buf);
  auto* d_frames = reinterpret_cast<ThresholdFrame*>(buf + count_bytes);
  check_cuda(cudaMemsetAsync(d_counts, 0, count_bytes, s->stream), "cudaMemsetAsync(cosmetic threshold counts)");
  upload_params(s->stream, d_frames, frames.data(), frame_bytes, "cudaMemcpyAsync(cosmetic threshold frames)");
  const unsigned per_frame = grid_for(static_cast<size_t>((s->pixels + 3) / 4), 256,
                                      std::max(1, 8 / static_cast<int>(std::min<int64_t>(count, 8))));
  note_launch();
  cosmetic_threshold_kernel<<<dim3(per_frame, static_cast<unsigned>(count)), 256, 0, s->stream>>>(
      s->d_slots, s->d_slot_of_frame, s->stride, s->pixels, d_frames, apply ? 1 : 0, d_counts, s->d_frame_nonfinite);
  check_cuda(cudaGetLastError(), "cosmetic_threshold launch");
  std::vector<unsigned long long> host(3 * static_cast<size_t>(count));
  check_cuda(cudaMemcpyAsync(host.data(), d_counts, count_bytes, cudaMemcpyDeviceToHost, s->stream),
             "cudaMemcpyAsync(cosmetic threshold counts)");
  check_cuda(cudaFreeAsync(buf, s->stream), "cudaFreeAsync(cosmetic threshold)");
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(cosmetic threshold)");
  if (host_counts)
    for (size_t i = 0; i < host.size(); ++i) host_counts[i] = static_cast<int64_t>(host[i]);
  GG_API_END
}
