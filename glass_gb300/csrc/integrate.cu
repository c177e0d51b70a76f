// Per-pixel rejection and weighted integration into the six output maps.
//
// Semantics are those of the CPU oracle, cpu/integration.py:36-118 with the
// per-pixel statistics of engine/rejection.py:31-66, 219-366:
//   valid      = finite(sample) & finite(w) & (w > 0)
//   winsorized = median / IQR/1.349 (fallback std) -> clip -> mean / std
//                (fallback first scale) -> reject outside mean -/+ k*std
//   sigma_clip = median centre, std scale (NumPy nanmedian / nanstd)
//   guard      = cancel a pixel's rejections when fewer than min_samples
//                remain or the rejected fraction exceeds max_reject_fraction
//   master     = sum(w*v) / sum(w) over kept samples; weight = sum(w)
// NumPy evaluates two formula families depending on whether the *whole* stack
// is valid (rejection.py:39-44 vs :54-60).  The stack keeps a per-frame count
// of non-finite samples (maintained by every kernel that writes a frame), so
// the kernel knows which family applies without another pass over HBM.
//
// Arithmetic: float64 sums of the CPU path are reproduced with float-float
// (TwoSum/TwoProd) accumulators; float32 steps are spelled out with _rn
// intrinsics so no FMA contraction changes a rounding.  Order statistics come
// from a sorting network over the pixel's column held in registers.
//
// GB300 layout: one thread per output pixel; a warp covers 32 consecutive
// pixels, so every per-frame load is one coalesced 128 B line and the column
// lives in registers (N <= 64) or in a [rank][thread] shared-memory tile
// (N > 64), which is bank-conflict free for any per-thread rank index.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "autotune.cuh"
#include "sampling.cuh"
#include "stack.cuh"

namespace gg {

// Fused warp (integrate_matrix_warped_*): a frame's samples come from its
// source pixels through the inverse of its matrix instead of from the stack.
struct FusedFrame {
  float m[9][2];  // inverse, float-float
  int affine;
  unsigned src_nonfinite;  // non-finite source pixels of the frame
  int pad[2];
};

struct IntegrateArgs {
  const float* slots;
  const int* slot_of_frame;
  int64_t stride;
  int64_t pixels;
  int frames;
  const float* weights;  // device [frames], raw values
  const unsigned* nonfinite;
  int rejection;
  float low_sigma;
  float high_sigma;
  int min_samples;
  float max_frac;
  int lfc_iterations;
  float* master;
  float* weight;
  void* coverage;
  void* low;
  void* high;
  int16_t* dq;
  int count_u16;
  const float* geometric;  // optional warp coverage (float32 per pixel)
  // fused warp only
  const FusedFrame* fused;
  int width, height;
  float clamp;
  float* geometric_out;  // frames with a geometrically valid sample, per pixel
  int tile_w, tile_h;    // fused path: 2-D pixel tiles (tile_w * tile_h == threads), 0 = rows
  int64_t tiles_x;       // tiles per image row
  int64_t tile_slots;    // tiles * threads
};

// One fused sample of frame f at output pixel (x, y): the value the warp
// kernel would have written (NaN fill when invalid); `geo` counts the
// samples the warp would have marked covered.
template <int INTERP>
__device__ __forceinline__ float fused_sample_inline(const IntegrateArgs& a, const float* src, const FusedFrame& fz,
                                                     int x, int y, int& geo) {
  const float nan = __int_as_float(0x7fc00000);
  FFv sx, sy;
  if (!source_coord(fz, static_cast<float>(x), static_cast<float>(y), sx, sy)) return nan;
  const float W = static_cast<float>(a.width), H = static_cast<float>(a.height);
  const bool valid = INTERP == GG_INTERP_BILINEAR
                         ? (ff_ge(sx, 0.0f) && ff_le(sx, W - 1.0f) && ff_ge(sy, 0.0f) && ff_le(sy, H - 1.0f))
                         : (ff_ge(sx, 2.0f) && ff_lt(sx, W - 3.0f) && ff_ge(sy, 2.0f) && ff_lt(sy, H - 3.0f));
  if (!valid) return nan;
  int x0, y0;
  float tx, ty;
  ff_floor_frac(sx, x0, tx);
  ff_floor_frac(sy, y0, ty);
  TapSource ts;
  ts.tile = nullptr;
  ts.src = src;
  ts.bx = ts.by = 0;
  ts.width = a.width;
  float v;
  if (INTERP == GG_INTERP_BILINEAR) {
    v = sample_bilinear(ts, x0, y0, tx, ty, a.width, a.height);
  } else if (!sample_lanczos3(ts, x0, y0, tx, ty, fz.src_nonfinite == 0u, a.clamp, v)) {
    return nan;
  }
  ++geo;
  return v;
}

// Out-of-line copy for the column kernel, which keeps the sampler out of its
// unrolled register code; the warp-per-pixel tile fill inlines it.
template <int INTERP>
__device__ __noinline__ float fused_sample(const IntegrateArgs& a, const float* src, const FusedFrame& fz, int x,
                                           int y, int& geo) {
  return fused_sample_inline<INTERP>(a, src, fz, x, y, geo);
}

constexpr float kInf = __builtin_huge_valf();

// ---- sorting network (Batcher odd-even merge sort, fully unrolled) --------
// Loop counters are kept additive (log2 of p and k) so that nvcc unrolls the
// whole network and v[] stays in registers.
template <int N>
__device__ __forceinline__ void sort_network(float (&v)[N]) {
  constexpr int LOG2N = (N <= 1) ? 0 : (N <= 2) ? 1 : (N <= 4) ? 2 : (N <= 8) ? 3 : (N <= 16) ? 4 : (N <= 32) ? 5 : 6;
  static_assert((1 << LOG2N) == N, "sort_network needs a power-of-two size up to 64");
#pragma unroll
  for (int lp = 0; lp < LOG2N; ++lp) {
#pragma unroll
    for (int lk = lp; lk >= 0; --lk) {
#pragma unroll
      for (int a = 0; a < N; ++a) {
        // Comparator (a, a+k) of stage (p, k); all conditions fold at compile time.
        const int p = 1 << lp, k = 1 << lk, j0 = k % p;
        if (a >= j0 && a + k < N && ((a - j0) % (2 * k)) < k && (a / (2 * p)) == ((a + k) / (2 * p))) {
          const float lo = fminf(v[a], v[a + k]);
          const float hi = fmaxf(v[a], v[a + k]);
          v[a] = lo;
          v[a + k] = hi;
        }
      }
    }
  }
}

// ---- percentiles ------------------------------------------------------------
// engine/rejection.py:299-321: per-pixel valid count, lo*(1-t) + hi*t.
__device__ __forceinline__ float percentile_valid(const float* S, int T, int cnt, float fraction) {
  if (cnt <= 0) return 0.0f;
  const float pos = __fmul_rn(static_cast<float>(cnt - 1), fraction);
  const int lower = static_cast<int>(floorf(pos));
  const int upper = min(lower + 1, cnt - 1);
  const float t = __fsub_rn(pos, static_cast<float>(lower));
  const float lv = S[lower * T];
  const float uv = S[upper * T];
  return __fadd_rn(__fmul_rn(lv, __fsub_rn(1.0f, t)), __fmul_rn(uv, t));
}

// engine/rejection.py:352-366: whole-stack frame count, lo + (hi-lo)*f.
// `fraction` is float32(percent / 100): the callers' 0.25, 0.5 and 0.75 are
// exactly the quotients of 25, 50 and 75 by 100.
__device__ __forceinline__ float percentile_all(const float* S, int T, int n, float fraction) {
  if (n == 1) return S[0];
  const float pos = __fmul_rn(fraction, static_cast<float>(n - 1));
  const int lower = static_cast<int>(floorf(pos));
  const int upper = static_cast<int>(ceilf(pos));
  const float f = __fsub_rn(pos, static_cast<float>(lower));
  const float lv = S[lower * T];
  if (upper == lower) return lv;
  const float uv = S[upper * T];
  return __fadd_rn(lv, __fmul_rn(__fsub_rn(uv, lv), f));
}

__device__ __forceinline__ float clipf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

// ---- output ---------------------------------------------------------------
// DQ bits: contracts.py:77-88; rules: resident_cuda.py:3110-3297.
__device__ __forceinline__ void write_outputs(const IntegrateArgs& a, int64_t p, float master, float weight, int cov,
                                              int nlow, int nhigh, int active_frames) {
  a.master[p] = master;
  a.weight[p] = weight;
  if (a.count_u16) {
    static_cast<uint16_t*>(a.coverage)[p] = static_cast<uint16_t>(min(cov, 65535));
    static_cast<uint16_t*>(a.low)[p] = static_cast<uint16_t>(min(nlow, 65535));
    static_cast<uint16_t*>(a.high)[p] = static_cast<uint16_t>(min(nhigh, 65535));
  } else {
    static_cast<float*>(a.coverage)[p] = static_cast<float>(cov);
    static_cast<float*>(a.low)[p] = static_cast<float>(nlow);
    static_cast<float*>(a.high)[p] = static_cast<float>(nhigh);
  }
  if (a.dq) {
    int bits = 0;
    bool invalid = !isfinite(master) || !isfinite(weight) || !(weight > 0.0f);
    if (cov <= 0) {
      bits |= 64;
      invalid = true;
    }
    if (a.geometric) {
      const float g = a.geometric[p];
      if (!isfinite(g) || g <= 0.5f) {
        bits |= 64;
        invalid = true;
      } else if (active_frames > 0 && g < static_cast<float>(active_frames) - 0.5f) {
        bits |= 64;
      }
    }
    if (invalid) bits |= 1;
    if (nlow > 0) bits |= 256;
    if (nhigh > 0) bits |= 512;
    a.dq[p] = static_cast<int16_t>(bits);
  }
}

// ---- per-pixel statistics over a column ------------------------------------
// The column is reachable two ways: `sorted` holds the valid samples in
// ascending order at ranks [0, cnt) with stride T (+inf beyond), and the
// frame-order view is provided by the caller's RawView.
struct CenterScale {
  float center;
  float scale;
};

// Fallback scale: std of the valid samples (rejection.py:231 all-valid,
// rejection.py:323-349 otherwise).
template <class Sorted>
__device__ __forceinline__ float std_of_valid(const Sorted& sorted, int cnt, bool allvalid) {
  FF s1;
  for (int i = 0; i < cnt; ++i) s1.add(sorted(i));
  float mh, ml;
  if (allvalid) {
    ff_div_pair(s1.hi, s1.lo, static_cast<float>(cnt), mh, ml);
  } else {
    mh = ff_div_f32(s1.hi, s1.lo, static_cast<float>(cnt));
    ml = 0.0f;
  }
  FF v;
  for (int i = 0; i < cnt; ++i) ff_add_sqdev(v, sorted(i), mh, ml);
  float q, ql;
  ff_div_pair(v.hi, v.lo, static_cast<float>(cnt), q, ql);
  return ff_sqrt_f32(q, ql);
}

// Winsorized sigma centre/scale (rejection.py:219-297).
template <class Sorted>
__device__ __forceinline__ CenterScale winsorized_stats(const Sorted& sorted, const float* S, int T, int cnt,
                                                        int nframes, bool allvalid, float ls, float hs) {
  CenterScale r{0.0f, 0.0f};
  if (cnt <= 0) return r;
  float med, q25, q75;
  if (allvalid) {
    med = percentile_all(S, T, nframes, 0.5f);
    q25 = percentile_all(S, T, nframes, 0.25f);
    q75 = percentile_all(S, T, nframes, 0.75f);
  } else {
    med = percentile_valid(S, T, cnt, 0.5f);
    q25 = percentile_valid(S, T, cnt, 0.25f);
    q75 = percentile_valid(S, T, cnt, 0.75f);
  }
  float scale1 = __fdiv_rn(__fsub_rn(q75, q25), 1.349f);
  const bool ok1 = allvalid ? (scale1 > 0.0f) : (scale1 > 0.0f && isfinite(scale1));
  if (!ok1) scale1 = std_of_valid(sorted, cnt, allvalid);
  const float lo1 = __fsub_rn(med, __fmul_rn(ls, scale1));
  const float hi1 = __fadd_rn(med, __fmul_rn(hs, scale1));
  FF sw;
  for (int i = 0; i < cnt; ++i) sw.add(clipf(sorted(i), lo1, hi1));
  float mh, ml;
  if (allvalid) {
    ff_div_pair(sw.hi, sw.lo, static_cast<float>(cnt), mh, ml);
    r.center = __fadd_rn(mh, ml);
  } else {
    r.center = ff_div_f32(sw.hi, sw.lo, static_cast<float>(cnt));
    mh = r.center;
    ml = 0.0f;
  }
  FF sv;
  for (int i = 0; i < cnt; ++i) ff_add_sqdev(sv, clipf(sorted(i), lo1, hi1), mh, ml);
  float q, ql;
  ff_div_pair(sv.hi, sv.lo, static_cast<float>(cnt), q, ql);
  float scale = ff_sqrt_f32(q, ql);
  const bool ok2 = allvalid ? (scale > 0.0f) : (scale > 0.0f && isfinite(scale));
  r.scale = ok2 ? scale : scale1;
  return r;
}

// Sigma-clip centre/scale: nanmedian + nanstd in float32, frame order
// (rejection.py:46-49; NumPy masked median and _nanvar).
template <class Raw>
__device__ __forceinline__ CenterScale sigma_stats(const Raw& raw, const float* S, int T, int cnt, int nframes) {
  CenterScale r{0.0f, 0.0f};
  if (cnt <= 0) return r;
  const int h = cnt / 2;
  const int l = (cnt & 1) ? h : h - 1;
  r.center = __fmul_rn(__fadd_rn(S[l * T], S[h * T]), 0.5f);
  float sum = 0.0f;
  for (int f = 0; f < nframes; ++f) {
    float x;
    if (raw(f, x)) sum = __fadd_rn(sum, x);
  }
  const float mean = __fdiv_rn(sum, static_cast<float>(cnt));
  float v = 0.0f;
  for (int f = 0; f < nframes; ++f) {
    float x;
    if (raw(f, x)) {
      const float d = __fsub_rn(x, mean);
      v = __fadd_rn(v, __fmul_rn(d, d));
    }
  }
  r.scale = __fsqrt_rn(__fdiv_rn(v, static_cast<float>(cnt)));
  return r;
}

// Linear-fit clipping.  The reference has no implementation of it; this
// library defines it (and oracle/integration.py restates it in float64):
//   1. fit v = a + b*(r - c) by least squares to the kept sorted samples,
//      r = rank within the kept range, c = (n-1)/2;
//   2. sigma = mean |v - fit|;
//   3. walk up from the lowest kept rank while v < fit - k_lo*sigma and down
//      from the highest while v > fit + k_hi*sigma; samples equal in value to
//      the first kept one are kept too, so the kept set is a value interval;
//   4. repeat on the kept range until it stops changing or `iterations` runs.
// On return [keep_lo, keep_hi) is the kept rank range.
template <class Sorted>
__device__ __forceinline__ void linear_fit_clip(const Sorted& sorted, int cnt, float ls, float hs, int iterations,
                                                int& keep_lo, int& keep_hi) {
  keep_lo = 0;
  keep_hi = cnt;  // exclusive
  for (int it = 0; it < iterations; ++it) {
    const int n = keep_hi - keep_lo;
    if (n < 3) break;
    const float fn = static_cast<float>(n);
    const float c = 0.5f * static_cast<float>(n - 1);
    FF sy, sry;
    for (int i = keep_lo; i < keep_hi; ++i) {
      const float y = sorted(i);
      sy.add(y);
      sry.add_prod(__fsub_rn(static_cast<float>(i - keep_lo), c), y);
    }
    // sum of squared centred ranks n(n^2-1)/12, exact in float for n <= 512.
    const float srr = fn * (fn * fn - 1.0f) / 12.0f;
    const float a0 = ff_div_f32(sy.hi, sy.lo, fn);
    const float b = __fdiv_rn(sry.value_f32(), srr);
    FF sad;
    for (int i = keep_lo; i < keep_hi; ++i) {
      const float fit = __fmaf_rn(b, __fsub_rn(static_cast<float>(i - keep_lo), c), a0);
      sad.add(fabsf(__fsub_rn(sorted(i), fit)));
    }
    const float sigma = ff_div_f32(sad.hi, sad.lo, fn);
    int new_lo = keep_lo, new_hi = keep_hi;
    while (new_lo < keep_hi) {
      const float fit = __fmaf_rn(b, __fsub_rn(static_cast<float>(new_lo - keep_lo), c), a0);
      if (sorted(new_lo) < __fsub_rn(fit, __fmul_rn(ls, sigma))) ++new_lo; else break;
    }
    while (new_hi > new_lo) {
      const float fit = __fmaf_rn(b, __fsub_rn(static_cast<float>(new_hi - 1 - keep_lo), c), a0);
      if (sorted(new_hi - 1) > __fadd_rn(fit, __fmul_rn(hs, sigma))) --new_hi; else break;
    }
    if (new_hi <= new_lo) break;  // never reject everything
    while (new_lo > keep_lo && sorted(new_lo - 1) == sorted(new_lo)) --new_lo;
    while (new_hi < keep_hi && sorted(new_hi) == sorted(new_hi - 1)) ++new_hi;
    if (new_lo == keep_lo && new_hi == keep_hi) break;
    keep_lo = new_lo;
    keep_hi = new_hi;
  }
}

// Rejection, guard and final weighted sums for one pixel.  `sorted` gives the
// valid samples in ascending order, `raw(f, x)` the frame-order view.
template <class Sorted, class Raw>
__device__ __forceinline__ void finish_pixel(const IntegrateArgs& a, int64_t p, const Sorted& sorted, const float* S,
                                             int T, const Raw& raw, const float* s_w, int cnt, bool allvalid,
                                             bool unit_weights, int active) {
  const float ls = a.low_sigma, hs = a.high_sigma;
  int nl = 0, nh = 0;
  float lt = -kInf, ht = kInf;
  bool use_thresholds = false;
  if (a.rejection == GG_REJECT_WINSORIZED || a.rejection == GG_REJECT_SIGMA_CLIP) {
    const CenterScale cs = (a.rejection == GG_REJECT_WINSORIZED)
                               ? winsorized_stats(sorted, S, T, cnt, a.frames, allvalid, ls, hs)
                               : sigma_stats(raw, S, T, cnt, a.frames);
    lt = __fsub_rn(cs.center, __fmul_rn(ls, cs.scale));
    ht = __fadd_rn(cs.center, __fmul_rn(hs, cs.scale));
    for (int i = 0; i < cnt; ++i) {
      const float x = sorted(i);
      nl += (x < lt);
      nh += (x > ht);
    }
    use_thresholds = true;
  } else if (a.rejection == GG_REJECT_LINEAR_FIT && cnt > 0) {
    int lfc_lo = 0, lfc_hi = cnt;
    linear_fit_clip(sorted, cnt, ls, hs, a.lfc_iterations, lfc_lo, lfc_hi);
    nl = lfc_lo;
    nh = cnt - lfc_hi;
    // The kept set is the value interval [sorted(lo), sorted(hi-1)].
    lt = sorted(lfc_lo);
    ht = sorted(lfc_hi - 1);
    use_thresholds = true;
  }
  if (nl + nh > 0) {
    // cpu/integration.py:85-99
    const int rej = nl + nh;
    const float frac = __fdiv_rn(static_cast<float>(rej), static_cast<float>(cnt));
    const bool allowed = (cnt - rej >= a.min_samples) && (frac <= a.max_frac);
    if (!allowed) {
      nl = nh = 0;
      use_thresholds = false;
    }
  }
  float master = 0.0f, weight = 0.0f;
  int kept = 0;
  if (unit_weights && a.rejection != GG_REJECT_NONE) {
    // Unit weights: sum the kept samples straight from the sorted column
    // (without rejection the column is not sorted and the frame loop runs).
    FF ws;
    for (int i = 0; i < cnt; ++i) {
      const float x = sorted(i);
      if (use_thresholds && (x < lt || x > ht)) continue;
      ws.add(x);
      ++kept;
    }
    if (kept > 0) {
      master = ff_div_f32(ws.hi, ws.lo, static_cast<float>(kept));
      weight = static_cast<float>(kept);
    }
  } else {
    FF ws, wsum;
    for (int f = 0; f < a.frames; ++f) {
      float x;
      if (!raw(f, x)) continue;
      if (use_thresholds && (x < lt || x > ht)) continue;
      ws.add_prod(x, s_w[f]);
      wsum.add(s_w[f]);
      ++kept;
    }
    if (kept > 0 && wsum.hi > 0.0f) {
      master = ff_div_ff(ws.hi, ws.lo, wsum.hi, wsum.lo);
      weight = wsum.value_f32();
    }
  }
  write_outputs(a, p, master, weight, kept, nl, nh, active);
}

// ---- CTA prologue: weights, frame bases, all-valid flag --------------------
// Both flags are derived here from the device weights, so weights computed on
// the GPU (frame statistics) feed the integrator without a host round trip.
template <int MAXF>
struct FrameTable {
  float w[MAXF];
  const float* base[MAXF];
  int allvalid;  // every weight valid and no non-finite sample anywhere
  int unit;      // every valid weight is exactly 1
  int active;    // frames with a valid weight
};

template <int MAXF>
__device__ __forceinline__ void load_frame_table(const IntegrateArgs& a, FrameTable<MAXF>& t) {
  for (int f = threadIdx.x; f < a.frames; f += blockDim.x) {
    const float w = a.weights ? a.weights[f] : 1.0f;
    t.w[f] = (isfinite(w) && w > 0.0f) ? w : 0.0f;
    t.base[f] = a.slots + static_cast<int64_t>(a.slot_of_frame[f]) * a.stride;
  }
  if (threadIdx.x < 32) {
    unsigned bad = 0, invalid_w = 0, non_unit = 0, active = 0;
    for (int f = threadIdx.x; f < a.frames; f += 32) {
      bad |= a.nonfinite[f];
      const float w = a.weights ? a.weights[f] : 1.0f;
      const bool ok = isfinite(w) && w > 0.0f;
      invalid_w |= ok ? 0u : 1u;
      non_unit |= (ok && w != 1.0f) ? 1u : 0u;
      active += ok ? 1u : 0u;
    }
    bad = __reduce_or_sync(0xffffffffu, bad);
    invalid_w = __reduce_or_sync(0xffffffffu, invalid_w);
    non_unit = __reduce_or_sync(0xffffffffu, non_unit);
    active = __reduce_add_sync(0xffffffffu, active);
    if (threadIdx.x == 0) {
      t.allvalid = (invalid_w == 0u && bad == 0u) ? 1 : 0;
      t.unit = non_unit == 0u ? 1 : 0;
      t.active = static_cast<int>(active);
    }
  }
  __syncthreads();
}

// ---- kernel F: N <= NB <= 32, specialised per rejection mode ----------------
// The frame-order column x[] stays in registers (for the weighted sum); a
// sorted copy goes through a register sorting network into shared memory
// S[rank][thread] (conflict-free for any per-thread rank).  The statistics
// passes are compact rolled loops over S, so the code fits the instruction
// cache, and they use the magnitude order the sort provides: summing
// same-sign values from the largest magnitude down makes Fast2Sum (3 flops)
// error-free, and squared deviations are summed from both ends of the sorted
// column inwards for the same reason.  Rejection counts are binary searches.

__device__ __forceinline__ void ff_merge2(FF& a, const FF& b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  a.hi = s;
  a.lo = __fadd_rn(__fadd_rn(a.lo, b.lo), e);
}

// Fast2Sum: error-free when |a.hi| >= |x| (or a.hi == 0).
__device__ __forceinline__ void ff_add_fast(FF& a, float x) {
  const float s = __fadd_rn(a.hi, x);
  const float e = __fsub_rn(x, __fsub_rn(s, a.hi));
  a.hi = s;
  a.lo = __fadd_rn(a.lo, e);
}

// True when every value in [lo, hi] lies within a factor of two of c (same
// sign), so x - c is exact in float32 (Sterbenz).
__device__ __forceinline__ bool sterbenz_interval(float lo, float hi, float c) {
  if (c > 0.0f) return lo >= 0.5f * c && hi <= 2.0f * c;
  if (c < 0.0f) return hi <= 0.5f * c && lo >= 2.0f * c;
  return false;
}

// Number of sorted valid values < t (strict) or <= t.
__device__ __forceinline__ int count_below(const float* S, int T, int cnt, float t, bool inclusive) {
  int lo = 0, hi = cnt;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    const float v = S[mid * T];
    if (inclusive ? (v <= t) : (v < t)) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Sum of S[i0..i1) (clipped to [lo, hi]) without rounding error loss.
__device__ __forceinline__ FF sum_sorted(const float* S, int T, int i0, int i1, float lo, float hi) {
  FF acc;
  if (i1 <= i0) return acc;
  const float first = clipf(S[i0 * T], lo, hi);
  const float last = clipf(S[(i1 - 1) * T], lo, hi);
  if (first >= 0.0f) {
#pragma unroll 4
    for (int i = i1 - 1; i >= i0; --i) ff_add_fast(acc, clipf(S[i * T], lo, hi));
  } else if (last <= 0.0f) {
#pragma unroll 4
    for (int i = i0; i < i1; ++i) ff_add_fast(acc, clipf(S[i * T], lo, hi));
  } else {
    FF b;
#pragma unroll 2
    for (int i = i0; i < i1; i += 2) {
      acc.add(clipf(S[i * T], lo, hi));
      if (i + 1 < i1) b.add(clipf(S[(i + 1) * T], lo, hi));
    }
    ff_merge2(acc, b);
  }
  return acc;
}

// Sum of squared deviations of clip(S[0..cnt)) from (mh + ml).
__device__ __forceinline__ FF sqdev_sorted(const float* S, int T, int cnt, float lo, float hi, float mh, float ml) {
  FF left, right;
  const float vlo = clipf(S[0], lo, hi);
  const float vhi = clipf(S[(cnt - 1) * T], lo, hi);
  if (sterbenz_interval(vlo, vhi, mh)) {
    // Values <= mh from the bottom up and values > mh from the top down:
    // both sequences have non-increasing |deviation|, so Fast2Sum is exact.
    const int nl = count_below(S, T, cnt, mh, true);
    const int nr = cnt - nl;
    const int steps = max(nl, nr);
    const float m2 = __fmul_rn(-2.0f, ml);
#pragma unroll 2
    for (int k = 0; k < steps; ++k) {
      if (k < nl) {
        const float d = __fsub_rn(clipf(S[k * T], lo, hi), mh);
        const float p = __fmul_rn(d, d);
        ff_add_fast(left, p);
        left.lo = __fadd_rn(left.lo, __fmaf_rn(m2, d, __fmaf_rn(d, d, -p)));
      }
      if (k < nr) {
        const float d = __fsub_rn(clipf(S[(cnt - 1 - k) * T], lo, hi), mh);
        const float p = __fmul_rn(d, d);
        ff_add_fast(right, p);
        right.lo = __fadd_rn(right.lo, __fmaf_rn(m2, d, __fmaf_rn(d, d, -p)));
      }
    }
  } else {
#pragma unroll 2
    for (int i = 0; i < cnt; i += 2) {
      ff_add_sqdev(left, clipf(S[i * T], lo, hi), mh, ml);
      if (i + 1 < cnt) ff_add_sqdev(right, clipf(S[(i + 1) * T], lo, hi), mh, ml);
    }
  }
  ff_merge2(left, right);
  return left;
}

// Winsorized centre/scale over the sorted column (rejection.py:219-297).
__device__ __forceinline__ CenterScale winsorized_sorted(const float* S, int T, int cnt, int nframes, bool allvalid,
                                                         float ls, float hs) {
  CenterScale r{0.0f, 0.0f};
  if (cnt <= 0) return r;
  float med, q25, q75;
  if (allvalid) {
    med = percentile_all(S, T, nframes, 0.5f);
    q25 = percentile_all(S, T, nframes, 0.25f);
    q75 = percentile_all(S, T, nframes, 0.75f);
  } else {
    med = percentile_valid(S, T, cnt, 0.5f);
    q25 = percentile_valid(S, T, cnt, 0.25f);
    q75 = percentile_valid(S, T, cnt, 0.75f);
  }
  float scale1 = __fdiv_rn(__fsub_rn(q75, q25), 1.349f);
  const bool ok1 = allvalid ? (scale1 > 0.0f) : (scale1 > 0.0f && isfinite(scale1));
  if (!ok1) {
    // Fallback std of the valid samples (rejection.py:231 / :323-349).
    const FF s1 = sum_sorted(S, T, 0, cnt, -kInf, kInf);
    float mh, ml;
    if (allvalid) {
      ff_div_pair(s1.hi, s1.lo, static_cast<float>(cnt), mh, ml);
    } else {
      mh = ff_div_f32(s1.hi, s1.lo, static_cast<float>(cnt));
      ml = 0.0f;
    }
    const FF v = sqdev_sorted(S, T, cnt, -kInf, kInf, mh, ml);
    float q, ql;
    ff_div_pair(v.hi, v.lo, static_cast<float>(cnt), q, ql);
    scale1 = ff_sqrt_f32(q, ql);
  }
  const float lo1 = __fsub_rn(med, __fmul_rn(ls, scale1));
  const float hi1 = __fadd_rn(med, __fmul_rn(hs, scale1));
  const FF sw = sum_sorted(S, T, 0, cnt, lo1, hi1);
  float mh, ml;
  if (allvalid) {
    ff_div_pair(sw.hi, sw.lo, static_cast<float>(cnt), mh, ml);
    r.center = __fadd_rn(mh, ml);
  } else {
    r.center = ff_div_f32(sw.hi, sw.lo, static_cast<float>(cnt));
    mh = r.center;
    ml = 0.0f;
  }
  const FF sv = sqdev_sorted(S, T, cnt, lo1, hi1, mh, ml);
  float q, ql;
  ff_div_pair(sv.hi, sv.lo, static_cast<float>(cnt), q, ql);
  const float scale = ff_sqrt_f32(q, ql);
  const bool ok2 = allvalid ? (scale > 0.0f) : (scale > 0.0f && isfinite(scale));
  r.scale = ok2 ? scale : scale1;
  return r;
}

// WARP = 0 reads the stack; GG_INTERP_BILINEAR / GG_INTERP_LANCZOS3 sample
// every frame through its inverse matrix (fused warp + integration).
// One CTA's share (block `bid` of `nblocks`) of one stack's pixels.
template <int NB, int T, int MODE, int WARP>
__device__ __forceinline__ void integrate_col_run(const IntegrateArgs& a, int bid, int nblocks) {
  extern __shared__ float smem[];
  float* S = smem;  // [NB][T] ascending valid samples
  __shared__ FrameTable<NB> tab;
  __shared__ float s_wtot[2];
  __shared__ FusedFrame fz[WARP ? NB : 1];
  if constexpr (WARP != 0)
    for (int f = threadIdx.x; f < a.frames; f += blockDim.x) fz[f] = a.fused[f];
  load_frame_table<NB>(a, tab);
  if (threadIdx.x == 0) {
    FF wt;
    for (int f = 0; f < a.frames; ++f)
      if (tab.w[f] > 0.0f) wt.add(tab.w[f]);
    s_wtot[0] = wt.hi;
    s_wtot[1] = wt.lo;
  }
  __syncthreads();
  const bool allvalid = tab.allvalid != 0;
  const bool unit = tab.unit != 0;
  const int tid = threadIdx.x;
  const int N = a.frames;
  const int64_t P = a.pixels;
  const float ls = a.low_sigma, hs = a.high_sigma;
  float* St = S + tid;
  // The fused path may walk the image in tiles of tile_w x tile_h pixels
  // (one tile per CTA iteration; neighbouring rows share Lanczos taps in L1);
  // otherwise a CTA covers T consecutive pixels.
  const bool tiled = WARP != 0 && a.tile_w > 0;
  const int64_t Q = tiled ? a.tile_slots : P;
  for (int64_t q = static_cast<int64_t>(bid) * T + tid; q < Q; q += static_cast<int64_t>(nblocks) * T) {
    int64_t p = q;
    if (tiled) {
      const int64_t t = q / T;
      const int px0 = static_cast<int>(t % a.tiles_x) * a.tile_w + tid % a.tile_w;
      const int py0 = static_cast<int>(t / a.tiles_x) * a.tile_h + tid / a.tile_w;
      if (px0 >= a.width || py0 >= a.height) continue;
      p = static_cast<int64_t>(py0) * a.width + px0;
    }
    float x[NB];
    if constexpr (WARP == 0) {
#pragma unroll
      for (int f = 0; f < NB; ++f) x[f] = (f < N) ? __ldcs(tab.base[f] + p) : kInf;
    } else {
      // samples staged through this thread's own shared-memory column (the
      // sampler stays out of the unrolled register code)
      const int py = static_cast<int>(p / a.width), px = static_cast<int>(p - static_cast<int64_t>(py) * a.width);
      int geo = 0;
#pragma unroll 1
      for (int f = 0; f < N; ++f) St[f * T] = fused_sample<WARP>(a, tab.base[f], fz[f], px, py, geo);
#pragma unroll
      for (int f = 0; f < NB; ++f) x[f] = (f < N) ? St[f * T] : kInf;
      a.geometric_out[p] = static_cast<float>(geo);
    }
    int cnt = 0;
    int nl = 0, nh = 0;
    float lt = -kInf, ht = kInf;
    bool thresholds = false;
    if (MODE != GG_REJECT_NONE) {
      float s[NB];
#pragma unroll
      for (int f = 0; f < NB; ++f) {
        const bool ok = (f < N) && tab.w[f] > 0.0f && isfinite(x[f]);
        s[f] = ok ? x[f] : kInf;
        cnt += ok ? 1 : 0;
      }
      sort_network<NB>(s);
#pragma unroll
      for (int f = 0; f < NB; ++f) St[f * T] = s[f];
      if (cnt > 0) {
        if (MODE == GG_REJECT_LINEAR_FIT) {
          auto sorted = [&](int i) -> float { return St[i * T]; };
          int lo = 0, hi = cnt;
          linear_fit_clip(sorted, cnt, ls, hs, a.lfc_iterations, lo, hi);
          nl = lo;
          nh = cnt - hi;
          lt = sorted(lo);
          ht = sorted(hi - 1);
        } else {
          CenterScale cs{0.0f, 0.0f};
          if (MODE == GG_REJECT_WINSORIZED) {
            cs = winsorized_sorted(St, T, cnt, N, allvalid, ls, hs);
          } else {
            // NumPy nanmedian + float32 nanstd in frame order (sigma_stats).
            const int h = cnt / 2;
            const int l = (cnt & 1) ? h : h - 1;
            cs.center = __fmul_rn(__fadd_rn(St[l * T], St[h * T]), 0.5f);
            float sum = 0.0f;
#pragma unroll
            for (int f = 0; f < NB; ++f)
              if (f < N && tab.w[f] > 0.0f && isfinite(x[f])) sum = __fadd_rn(sum, x[f]);
            const float mean = __fdiv_rn(sum, static_cast<float>(cnt));
            float v = 0.0f;
#pragma unroll
            for (int f = 0; f < NB; ++f) {
              if (f < N && tab.w[f] > 0.0f && isfinite(x[f])) {
                const float d = __fsub_rn(x[f], mean);
                v = __fadd_rn(v, __fmul_rn(d, d));
              }
            }
            cs.scale = __fsqrt_rn(__fdiv_rn(v, static_cast<float>(cnt)));
          }
          lt = __fsub_rn(cs.center, __fmul_rn(ls, cs.scale));
          ht = __fadd_rn(cs.center, __fmul_rn(hs, cs.scale));
          nl = count_below(St, T, cnt, lt, false);
          nh = cnt - count_below(St, T, cnt, ht, true);
        }
        if (nl + nh > 0) {
          const int rej = nl + nh;
          const float frac = __fdiv_rn(static_cast<float>(rej), static_cast<float>(cnt));
          thresholds = (cnt - rej >= a.min_samples) && (frac <= a.max_frac);
          if (!thresholds) nl = nh = 0;
        }
      }
    } else {
#pragma unroll
      for (int f = 0; f < NB; ++f) cnt += ((f < N) && tab.w[f] > 0.0f && isfinite(x[f])) ? 1 : 0;
    }
    float master = 0.0f, weight = 0.0f;
    int kept = 0;
    if (MODE != GG_REJECT_NONE && unit) {
      // Kept samples are the contiguous sorted range [nl, cnt - nh).
      kept = cnt - nl - nh;
      if (kept > 0) {
        const FF ws = sum_sorted(St, T, nl, cnt - nh, -kInf, kInf);
        master = ff_div_f32(ws.hi, ws.lo, static_cast<float>(kept));
        weight = static_cast<float>(kept);
      }
    } else if (cnt == N && !thresholds) {
      // Every frame valid, nothing rejected: sum(w*x) over all frames and the
      // CTA-wide weight total.
      FF w0, w1;
#pragma unroll
      for (int f = 0; f < NB; f += 2) {
        if (f < N) w0.add_prod(x[f], tab.w[f]);
        if (f + 1 < N) w1.add_prod(x[f + 1], tab.w[f + 1]);
      }
      ff_merge2(w0, w1);
      kept = N;
      if (s_wtot[0] > 0.0f) {
        master = ff_div_ff(w0.hi, w0.lo, s_wtot[0], s_wtot[1]);
        weight = __fadd_rn(s_wtot[0], s_wtot[1]);
      }
    } else {
      FF ws, wsum;
#pragma unroll
      for (int f = 0; f < NB; ++f) {
        const bool ok = (f < N) && tab.w[f] > 0.0f && isfinite(x[f]) && !(thresholds && (x[f] < lt || x[f] > ht));
        if (ok) {
          ws.add_prod(x[f], tab.w[f]);
          wsum.add(tab.w[f]);
          ++kept;
        }
      }
      if (kept > 0 && wsum.hi > 0.0f) {
        master = ff_div_ff(ws.hi, ws.lo, wsum.hi, wsum.lo);
        weight = wsum.value_f32();
      }
    }
    write_outputs(a, p, master, weight, kept, nl, nh, tab.active);
  }
}

// MINB > 1 asks the compiler for MINB resident CTAs per SM (a register cap:
// more warps to hide the sort network's dependent latencies, against a few
// spilled registers); the autotuner picks per problem shape.
template <int NB, int T, int MODE, int WARP = 0, int MINB = 1>
__global__ void __launch_bounds__(T, MINB) integrate_col_kernel(IntegrateArgs a) {
  integrate_col_run<NB, T, MODE, WARP>(a, blockIdx.x, gridDim.x);
}

// Several stacks (of different frame counts and shapes, each with its own
// maps and weights) in one launch: CTAs [start[k], start[k+1]) work on stack
// k, so a CTA loads one frame table and never mixes stacks.
constexpr int kMaxBatchStacks = 64;
struct BatchTable {
  int start[kMaxBatchStacks + 1];
  int stacks;
};

template <int NB, int T, int MODE, int MINB = 1>
__global__ void __launch_bounds__(T, MINB) integrate_batch_kernel(const IntegrateArgs* args, BatchTable bt) {
  int k = 0;
  while (k + 1 < bt.stacks && static_cast<int>(blockIdx.x) >= bt.start[k + 1]) ++k;
  const IntegrateArgs a = args[k];
  integrate_col_run<NB, T, MODE, 0>(a, static_cast<int>(blockIdx.x) - bt.start[k], bt.start[k + 1] - bt.start[k]);
}

// ---- kernel A: N <= NB <= 64, column in registers ----------------------------
template <int NB, int T>
__global__ void __launch_bounds__(T) integrate_reg_kernel(IntegrateArgs a) {
  extern __shared__ float smem[];
  float* R = smem;            // [NB][T] frame order (raw)
  float* S = smem + NB * T;   // [NB][T] ascending valid samples
  __shared__ FrameTable<NB> tab;
  load_frame_table<NB>(a, tab);
  const bool allvalid = tab.allvalid != 0;
  const int tid = threadIdx.x;
  const int N = a.frames;
  const int64_t P = a.pixels;
  for (int64_t p = static_cast<int64_t>(blockIdx.x) * T + tid; p < P; p += static_cast<int64_t>(gridDim.x) * T) {
    float s[NB];
    int cnt = 0;
#pragma unroll
    for (int f = 0; f < NB; ++f) {
      float x = kInf;
      if (f < N) {
        x = __ldcs(tab.base[f] + p);
        R[f * T + tid] = x;
      }
      const bool ok = (f < N) && tab.w[f] > 0.0f && isfinite(x);
      s[f] = ok ? x : kInf;
      cnt += ok ? 1 : 0;
    }
    auto raw = [&](int f, float& x) -> bool {
      x = R[f * T + tid];
      return tab.w[f] > 0.0f && isfinite(x);
    };
    if (a.rejection != GG_REJECT_NONE) {
      sort_network<NB>(s);
#pragma unroll
      for (int f = 0; f < NB; ++f) S[f * T + tid] = s[f];
    }
    auto sorted = [&](int i) -> float { return S[i * T + tid]; };
    finish_pixel(a, p, sorted, S + tid, T, raw, tab.w, cnt, allvalid, tab.unit != 0, tab.active);
  }
}

// ---- kernel B: N > 64, chunk-sorted column in shared memory ------------------
// Each thread sorts its column in chunks of 32 (registers), then streams a
// k-way merge of the chunks (k <= MR heads in registers) into the sorted
// buffer.  Frame-order values are re-read from global memory (the CTA's tile
// is L2 resident) by the raw view.
template <int MR, int T>
__global__ void __launch_bounds__(T) integrate_smem_kernel(IntegrateArgs a) {
  constexpr int MAXF = MR * 32;
  extern __shared__ float smem[];
  float* A = smem;               // [MAXF][T] chunk-sorted
  float* S = smem + MAXF * T;    // [MAXF][T] merged
  __shared__ FrameTable<MAXF> tab;
  load_frame_table<MAXF>(a, tab);
  const bool allvalid = tab.allvalid != 0;
  const int tid = threadIdx.x;
  const int N = a.frames;
  const int chunks = (N + 31) / 32;
  const int64_t P = a.pixels;
  for (int64_t p = static_cast<int64_t>(blockIdx.x) * T + tid; p < P; p += static_cast<int64_t>(gridDim.x) * T) {
    int cnt = 0;
    for (int c = 0; c < chunks; ++c) {
      float v[32];
#pragma unroll
      for (int k = 0; k < 32; ++k) {
        const int f = c * 32 + k;
        float x = kInf;
        if (f < N) x = __ldcs(tab.base[f] + p);
        const bool ok = (f < N) && tab.w[f] > 0.0f && isfinite(x);
        v[k] = ok ? x : kInf;
        cnt += ok ? 1 : 0;
      }
      if (a.rejection != GG_REJECT_NONE) sort_network<32>(v);
#pragma unroll
      for (int k = 0; k < 32; ++k) A[(c * 32 + k) * T + tid] = v[k];
    }
    auto raw = [&](int f, float& x) -> bool {
      x = tab.base[f][p];
      return tab.w[f] > 0.0f && isfinite(x);
    };
    if (a.rejection != GG_REJECT_NONE) {
      // k-way merge of the sorted chunks: heads in registers.
      float head[MR];
      int pos[MR];
#pragma unroll
      for (int r = 0; r < MR; ++r) {
        pos[r] = 0;
        head[r] = (r < chunks) ? A[(r * 32) * T + tid] : kInf;
      }
      for (int out = 0; out < cnt; ++out) {
        float best = head[0];
        int br = 0;
#pragma unroll
        for (int r = 1; r < MR; ++r) {
          if (head[r] < best) {
            best = head[r];
            br = r;
          }
        }
        S[out * T + tid] = best;
#pragma unroll
        for (int r = 0; r < MR; ++r) {
          if (r == br) {
            const int np = pos[r] + 1;
            pos[r] = np;
            head[r] = (np < 32) ? A[(r * 32 + np) * T + tid] : kInf;
          }
        }
      }
    } else {
      for (int i = 0; i < chunks * 32; ++i) S[i * T + tid] = A[i * T + tid];
    }
    auto sorted = [&](int i) -> float { return S[i * T + tid]; };
    finish_pixel(a, p, sorted, S + tid, T, raw, tab.w, cnt, allvalid, tab.unit != 0, tab.active);
  }
}

// ---- kernel W: 32 < N <= 32 * NPL, one warp per pixel ------------------------
// A CTA stages a tile of kWarpTilePx consecutive pixels of every frame in
// shared memory ([frame][pixel], rows padded to kWarpTilePx + 1 floats so a
// warp reading one pixel's column is bank-conflict free; every frame row is
// one coalesced 128 B load), then each warp takes one pixel at a time.  The
// column is spread over the lanes (NPL values per lane), sorted by a
// warp-wide bitonic network (in-register steps within a lane, shuffles
// across lanes), and every sum of the statistics and of the integration is a
// per-lane float-float sum combined across the warp.  The shared-memory cost
// is 4 * 33 B per frame instead of a sorted column per thread, so an SM keeps
// tens of warps in flight at N = 200.  WARP = GG_INTERP_* fills the tile by
// sampling every frame through its inverse matrix (fused warp + integration
// of more than 32 frames) and counts each pixel's geometrically valid
// samples in shared memory.
constexpr int kWarpTilePx = 32;
constexpr int kWarpTileRow = kWarpTilePx + 1;
constexpr int kWarpThreads = 256;

// (hi, lo) float-float sum over each segment of LANES lanes (the whole warp
// by default), in every lane of the segment.  TwoSum is exact and
// symmetric, so both partners of each butterfly step hold the same pair.
template <int LANES = 32>
__device__ __forceinline__ void ff_warp_reduce(FF& s) {
#pragma unroll
  for (int off = LANES / 2; off > 0; off >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, s.hi, off);
    const float ol = __shfl_xor_sync(0xffffffffu, s.lo, off);
    float h, e;
    two_sum(s.hi, oh, h, e);
    s.hi = h;
    s.lo = __fadd_rn(__fadd_rn(s.lo, ol), e);
  }
}

// Integer sum over each segment of LANES lanes, in every lane of it.
template <int LANES>
__device__ __forceinline__ int seg_sum(int x) {
  if constexpr (LANES == 32) {
    return __reduce_add_sync(0xffffffffu, x);
  } else {
#pragma unroll
    for (int off = LANES / 2; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
    return x;
  }
}

// Ascending bitonic sort of the warp's 32 * NPL values; rank e lives in lane
// e / NPL, register e % NPL.  Steps with partner distance >= NPL exchange
// across lanes (shuffles); the shorter ones stay in a lane.  From merge size
// NPL up, a lane's direction is the same for all its registers, so its
// in-register steps always sort ascending (compile-time directions: a min
// and a max per pair) and a lane whose block sorts descending reverses its
// registers afterwards; below NPL the direction of a pair is a compile-time
// function of its register index.
// With LANES = 16 the two half-warps sort two columns of 16 * NPL values
// independently (every partner distance stays below 16); `lane` is then the
// lane within the half.
template <int NPL, int LANES = 32>
__device__ __forceinline__ void warp_bitonic_sort(float (&v)[NPL], int lane) {
  constexpr int M = LANES * NPL;
  constexpr int LOGM = (M == 64) ? 6 : (M == 128) ? 7 : (M == 256) ? 8 : 9;
  static_assert(M == (1 << LOGM) && NPL >= 2 && NPL <= 16, "LANES * NPL must be 64 .. 512");
#pragma unroll
  for (int ls = 1; ls <= LOGM; ++ls) {
    const int size = 1 << ls;
#pragma unroll
    for (int lj = ls - 1; lj >= 0; --lj) {
      const int j = 1 << lj;
      if (j >= NPL) {
        const int lm = j / NPL;
        const bool up = ((lane * NPL) & size) == 0;  // always true in the last merge
        const bool keep_min = ((lane & lm) == 0) == up;
#pragma unroll
        for (int k = 0; k < NPL; ++k) {
          const float o = __shfl_xor_sync(0xffffffffu, v[k], lm);
          v[k] = keep_min ? fminf(v[k], o) : fmaxf(v[k], o);
        }
      } else if (size < NPL) {
#pragma unroll
        for (int k = 0; k < NPL; ++k) {
          if ((k ^ j) > k) {
            const int q = k ^ j;
            const float lo = fminf(v[k], v[q]), hi = fmaxf(v[k], v[q]);
            const bool up = (k & size) == 0;  // compile time: lane * NPL has no bit below NPL
            v[k] = up ? lo : hi;
            v[q] = up ? hi : lo;
          }
        }
      } else {
#pragma unroll
        for (int k = 0; k < NPL; ++k) {
          if ((k ^ j) > k) {
            const int q = k ^ j;
            const float lo = fminf(v[k], v[q]), hi = fmaxf(v[k], v[q]);
            v[k] = lo;
            v[q] = hi;
          }
        }
      }
    }
    if (size >= NPL && size < M) {
      // descending blocks of this merge: reverse the ascending registers
      if (((lane * NPL) & size) != 0) {
#pragma unroll
        for (int k = 0; k < NPL / 2; ++k) {
          const float t = v[k];
          v[k] = v[NPL - 1 - k];
          v[NPL - 1 - k] = t;
        }
      }
    }
  }
}

// Value of warp-uniform rank i; the register index i % NPL is warp-uniform,
// so a switch on it (uniform branch) replaces a per-lane select chain.
template <int NPL, int LANES = 32>
__device__ __forceinline__ float warp_rank(const float (&v)[NPL], int i, int seg = 0) {
  float t = v[0];
  switch (i & (NPL - 1)) {
    case 0: if constexpr (0 < NPL) t = v[0]; break;
    case 1: if constexpr (1 < NPL) t = v[1]; break;
    case 2: if constexpr (2 < NPL) t = v[2]; break;
    case 3: if constexpr (3 < NPL) t = v[3]; break;
    case 4: if constexpr (4 < NPL) t = v[4]; break;
    case 5: if constexpr (5 < NPL) t = v[5]; break;
    case 6: if constexpr (6 < NPL) t = v[6]; break;
    case 7: if constexpr (7 < NPL) t = v[7]; break;
    case 8: if constexpr (8 < NPL) t = v[8]; break;
    case 9: if constexpr (9 < NPL) t = v[9]; break;
    case 10: if constexpr (10 < NPL) t = v[10]; break;
    case 11: if constexpr (11 < NPL) t = v[11]; break;
    case 12: if constexpr (12 < NPL) t = v[12]; break;
    case 13: if constexpr (13 < NPL) t = v[13]; break;
    case 14: if constexpr (14 < NPL) t = v[14]; break;
    case 15: if constexpr (15 < NPL) t = v[15]; break;
  }
  return __shfl_sync(0xffffffffu, t, seg * LANES + i / NPL);
}

// percentile_valid / percentile_all on the warp's sorted column.  With
// LANES = 16 the two halves rank their own columns; the shuffles run in
// every lane whatever the counts (a half with no samples gets 0).
template <int NPL, int LANES = 32>
__device__ __forceinline__ float warp_percentile_valid(const float (&v)[NPL], int cnt, float fraction, int seg = 0) {
  const int c = cnt > 0 ? cnt : 1;
  const float pos = __fmul_rn(static_cast<float>(c - 1), fraction);
  const int lower = static_cast<int>(floorf(pos));
  const int upper = min(lower + 1, c - 1);
  const float t = __fsub_rn(pos, static_cast<float>(lower));
  const float lv = warp_rank<NPL, LANES>(v, lower, seg);
  const float uv = warp_rank<NPL, LANES>(v, upper, seg);
  if (cnt <= 0) return 0.0f;
  return __fadd_rn(__fmul_rn(lv, __fsub_rn(1.0f, t)), __fmul_rn(uv, t));
}

template <int NPL, int LANES = 32>
__device__ __forceinline__ float warp_percentile_all(const float (&v)[NPL], int n, float fraction, int seg = 0) {
  if (n == 1) return warp_rank<NPL, LANES>(v, 0, seg);
  const float pos = __fmul_rn(fraction, static_cast<float>(n - 1));
  const int lower = static_cast<int>(floorf(pos));
  const int upper = static_cast<int>(ceilf(pos));
  const float f = __fsub_rn(pos, static_cast<float>(lower));
  const float lv = warp_rank<NPL, LANES>(v, lower, seg);
  if (upper == lower) return lv;
  const float uv = warp_rank<NPL, LANES>(v, upper, seg);
  return __fadd_rn(lv, __fmul_rn(__fsub_rn(uv, lv), f));
}

// Mean (hi, lo) and float-float squared deviations of the valid ranks after
// clipping to [lo, hi] (+-inf: no clipping); the two passes of std_of_valid
// and winsorized_stats.
template <int NPL, int LANES = 32>
__device__ __forceinline__ float warp_clipped_std(const float (&v)[NPL], int lane, int cnt, bool allvalid, float lo,
                                                  float hi, float& mean_out) {
  FF s1;
#pragma unroll
  for (int k = 0; k < NPL; ++k)
    if (lane * NPL + k < cnt) s1.add(clipf(v[k], lo, hi));
  ff_warp_reduce<LANES>(s1);
  float mh, ml;
  if (allvalid) {
    ff_div_pair(s1.hi, s1.lo, static_cast<float>(cnt), mh, ml);
    mean_out = __fadd_rn(mh, ml);
  } else {
    mh = ff_div_f32(s1.hi, s1.lo, static_cast<float>(cnt));
    ml = 0.0f;
    mean_out = mh;
  }
  FF sv;
#pragma unroll
  for (int k = 0; k < NPL; ++k)
    if (lane * NPL + k < cnt) ff_add_sqdev(sv, clipf(v[k], lo, hi), mh, ml);
  ff_warp_reduce<LANES>(sv);
  float q, ql;
  ff_div_pair(sv.hi, sv.lo, static_cast<float>(cnt), q, ql);
  return ff_sqrt_f32(q, ql);
}

__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(dst))),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(PENDING) : "memory");
}

// PIPE (resident frames only): two tile buffers; the copies of the next tile
// (cp.async, one 4-byte sample per thread and step) are in flight while the
// warps integrate the current one.
// LANES = 16: two pixels per warp, one per half (columns of at most
// 16 * NPL frames): the per-pixel scalar work and the butterfly reductions
// are shared by two pixels.
template <int NPL, int WARP, bool PIPE = false, int LANES = 32>
__global__ void __launch_bounds__(kWarpThreads, LANES == 16 ? (NPL >= 16 ? 3 : 4) : 1)
    integrate_warp_kernel(IntegrateArgs a) {
  extern __shared__ float smem_tiles[];  // [frames][kWarpTileRow] (x2 with PIPE), then (fused) [frames] FusedFrame
  __shared__ FrameTable<32 * NPL> tab;
  __shared__ int s_geo[kWarpTilePx];
  static_assert(!(PIPE && WARP != 0), "the pipelined tile copy serves resident frames only");
  FusedFrame* fz = reinterpret_cast<FusedFrame*>(smem_tiles + a.frames * kWarpTileRow);
  if constexpr (WARP != 0)
    for (int f = threadIdx.x; f < a.frames; f += blockDim.x) fz[f] = a.fused[f];
  load_frame_table<32 * NPL>(a, tab);
  const bool allvalid = tab.allvalid != 0;
  const bool unit = tab.unit != 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int hl = lane & (LANES - 1), seg = lane / LANES;
  const int N = a.frames;
  const int64_t P = a.pixels;
  const int64_t tiles = (P + kWarpTilePx - 1) / kWarpTilePx;
  const float ls = a.low_sigma, hs = a.high_sigma;
  auto fill_async = [&](int64_t tt, float* dst) {
    const int64_t q0 = tt * kWarpTilePx;
    for (int i = threadIdx.x; i < N * kWarpTilePx; i += kWarpThreads) {
      const int f = i / kWarpTilePx, px = i - f * kWarpTilePx;
      if (q0 + px < P) cp_async4(dst + f * kWarpTileRow + px, tab.base[f] + q0 + px);
      else dst[f * kWarpTileRow + px] = 0.0f;
    }
    cp_async_commit();
  };
  if constexpr (PIPE) {
    if (blockIdx.x < tiles) fill_async(blockIdx.x, smem_tiles);
  }
  int buf = 0;
  for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x, buf ^= 1) {
    const int64_t p0 = t * kWarpTilePx;
    float* tile = smem_tiles;
    if constexpr (PIPE) {
      tile = smem_tiles + buf * (N * kWarpTileRow);
      if (t + gridDim.x < tiles) {
        fill_async(t + gridDim.x, smem_tiles + (buf ^ 1) * (N * kWarpTileRow));
        cp_async_wait<1>();
      } else {
        cp_async_wait<0>();
      }
    } else {
      __syncthreads();  // the previous tile's columns are consumed
      if constexpr (WARP != 0) {
        if (threadIdx.x < kWarpTilePx) s_geo[threadIdx.x] = 0;
        __syncthreads();
      }
      for (int i = threadIdx.x; i < N * kWarpTilePx; i += kWarpThreads) {
        const int f = i / kWarpTilePx, px = i - f * kWarpTilePx;
        const int64_t p = p0 + px;
        float v = 0.0f;
        if constexpr (WARP == 0) {
          if (p < P) v = __ldcs(tab.base[f] + p);
        } else if (p < P) {
          const int py = static_cast<int>(p / a.width),
                    pxx = static_cast<int>(p - static_cast<int64_t>(py) * a.width);
          int geo = 0;
          v = fused_sample_inline<WARP>(a, tab.base[f], fz[f], pxx, py, geo);
          if (geo) atomicAdd(&s_geo[px], 1);
        }
        tile[f * kWarpTileRow + px] = v;
      }
    }
    __syncthreads();
    // LANES = 32: one warp per pixel; LANES = 16: each half-warp takes a
    // pixel, the halves 16 tile columns apart (their column loads fall in
    // disjoint shared-memory banks).  Every shuffle below runs in all 32
    // lanes; a half whose pixel lies past the frame works on the tile's zero
    // padding and writes nothing.
    constexpr int kPixelsPerPass = 32 / LANES;
    for (int pb = warp; pb < kWarpTilePx / kPixelsPerPass; pb += kWarpThreads / 32) {
      const int px = pb + seg * (kWarpTilePx / kPixelsPerPass);
      const int64_t p = p0 + px;
      const bool in_frame = p < P;
      if (!__any_sync(0xffffffffu, in_frame)) break;
      const float* col = tile + px;
      // column: lane l of the segment holds frames l, l + LANES, ... (+inf when invalid)
      float v[NPL];
      int c = 0;
#pragma unroll
      for (int k = 0; k < NPL; ++k) {
        const int f = k * LANES + hl;
        const float x = f < N ? col[f * kWarpTileRow] : kInf;
        const bool ok = in_frame && f < N && tab.w[f] > 0.0f && isfinite(x);
        v[k] = ok ? x : kInf;
        c += ok ? 1 : 0;
      }
      const int cnt = seg_sum<LANES>(c);
      int nl = 0, nh = 0;
      float lt = -kInf, ht = kInf;
      bool use_thresholds = false;
      if (a.rejection != GG_REJECT_NONE) {
        warp_bitonic_sort<NPL, LANES>(v, hl);
        CenterScale cs{0.0f, 0.0f};
        if (a.rejection == GG_REJECT_WINSORIZED) {
          float med, q25, q75;
          if (allvalid) {
            med = warp_percentile_all<NPL, LANES>(v, N, 0.5f, seg);
            q25 = warp_percentile_all<NPL, LANES>(v, N, 0.25f, seg);
            q75 = warp_percentile_all<NPL, LANES>(v, N, 0.75f, seg);
          } else {
            med = warp_percentile_valid<NPL, LANES>(v, cnt, 0.5f, seg);
            q25 = warp_percentile_valid<NPL, LANES>(v, cnt, 0.25f, seg);
            q75 = warp_percentile_valid<NPL, LANES>(v, cnt, 0.75f, seg);
          }
          float scale1 = __fdiv_rn(__fsub_rn(q75, q25), 1.349f);
          const bool ok1 = allvalid ? (scale1 > 0.0f) : (scale1 > 0.0f && isfinite(scale1));
          if (__any_sync(0xffffffffu, !ok1)) {
            float unused;
            const float sd = warp_clipped_std<NPL, LANES>(v, hl, cnt, allvalid, -kInf, kInf, unused);
            if (!ok1) scale1 = sd;
          }
          const float lo1 = __fsub_rn(med, __fmul_rn(ls, scale1));
          const float hi1 = __fadd_rn(med, __fmul_rn(hs, scale1));
          const float scale = warp_clipped_std<NPL, LANES>(v, hl, cnt, allvalid, lo1, hi1, cs.center);
          const bool ok2 = allvalid ? (scale > 0.0f) : (scale > 0.0f && isfinite(scale));
          cs.scale = ok2 ? scale : scale1;
          if (cnt <= 0) cs = CenterScale{0.0f, 0.0f};
        } else {
          // sigma clip: median, then float32 frame-order sums (sequential, as
          // NumPy reduces over the frame axis)
          const int cc = cnt > 0 ? cnt : 1;
          const int h = cc / 2;
          const int l = (cc & 1) ? h : h - 1;
          const float ml = warp_rank<NPL, LANES>(v, l, seg), mh = warp_rank<NPL, LANES>(v, h, seg);
          float scale = 0.0f;
          if (hl == 0 && cnt > 0) {
            float sum = 0.0f;
            for (int f = 0; f < N; ++f) {
              const float x = col[f * kWarpTileRow];
              if (tab.w[f] > 0.0f && isfinite(x)) sum = __fadd_rn(sum, x);
            }
            const float mean = __fdiv_rn(sum, static_cast<float>(cnt));
            float var = 0.0f;
            for (int f = 0; f < N; ++f) {
              const float x = col[f * kWarpTileRow];
              if (tab.w[f] > 0.0f && isfinite(x)) {
                const float d = __fsub_rn(x, mean);
                var = __fadd_rn(var, __fmul_rn(d, d));
              }
            }
            scale = __fsqrt_rn(__fdiv_rn(var, static_cast<float>(cnt)));
          }
          scale = __shfl_sync(0xffffffffu, scale, seg * LANES);
          if (cnt > 0) {
            cs.center = __fmul_rn(__fadd_rn(ml, mh), 0.5f);
            cs.scale = scale;
          }
        }
        lt = __fsub_rn(cs.center, __fmul_rn(ls, cs.scale));
        ht = __fadd_rn(cs.center, __fmul_rn(hs, cs.scale));
        int cl = 0, ch = 0;
#pragma unroll
        for (int k = 0; k < NPL; ++k) {
          if (hl * NPL + k < cnt) {
            cl += v[k] < lt;
            ch += v[k] > ht;
          }
        }
        nl = seg_sum<LANES>(cl);
        nh = seg_sum<LANES>(ch);
        use_thresholds = true;
        if (nl + nh > 0) {
          // cpu/integration.py:85-99
          const int rej = nl + nh;
          const float frac = __fdiv_rn(static_cast<float>(rej), static_cast<float>(cnt));
          if (!((cnt - rej >= a.min_samples) && (frac <= a.max_frac))) {
            nl = nh = 0;
            use_thresholds = false;
          }
        }
      }
      float master = 0.0f, weight = 0.0f;
      int kept = 0;
      if (unit && a.rejection != GG_REJECT_NONE) {
        FF ws;
#pragma unroll
        for (int k = 0; k < NPL; ++k) {
          const float x = v[k];
          if (hl * NPL + k < cnt && !(use_thresholds && (x < lt || x > ht))) {
            ws.add(x);
            ++kept;
          }
        }
        ff_warp_reduce<LANES>(ws);
        kept = seg_sum<LANES>(kept);
        if (kept > 0) {
          master = ff_div_f32(ws.hi, ws.lo, static_cast<float>(kept));
          weight = static_cast<float>(kept);
        }
      } else {
        FF ws, wsum;
#pragma unroll
        for (int k = 0; k < NPL; ++k) {
          const int f = k * LANES + hl;
          if (in_frame && f < N) {
            const float x = col[f * kWarpTileRow];
            const float w = tab.w[f];
            if (w > 0.0f && isfinite(x) && !(use_thresholds && (x < lt || x > ht))) {
              ws.add_prod(x, w);
              wsum.add(w);
              ++kept;
            }
          }
        }
        ff_warp_reduce<LANES>(ws);
        ff_warp_reduce<LANES>(wsum);
        kept = seg_sum<LANES>(kept);
        if (kept > 0 && wsum.hi > 0.0f) {
          master = ff_div_ff(ws.hi, ws.lo, wsum.hi, wsum.lo);
          weight = wsum.value_f32();
        }
      }
      if (hl == 0 && in_frame) {
        if constexpr (WARP != 0) a.geometric_out[p] = static_cast<float>(s_geo[px]);
        write_outputs(a, p, master, weight, kept, nl, nh, tab.active);
      }
    }
    if constexpr (PIPE) __syncthreads();  // this buffer is refilled by the next iteration's prefetch
  }
}

template <int NPL, int WARP = 0, int LANES = 32>
static void launch_warp(const IntegrateArgs& args, cudaStream_t stream) {
  const size_t tile_bytes = static_cast<size_t>(args.frames) * kWarpTileRow * sizeof(float);
  // resident frames: double-buffered tiles while two of them stay under 100 KB
  constexpr bool kCanPipe = WARP == 0;
  const bool pipe = kCanPipe && 2 * tile_bytes <= 100 * 1024;
  const size_t smem = tile_bytes * (pipe ? 2 : 1) +
                      (WARP != 0 ? static_cast<size_t>(args.frames) * sizeof(FusedFrame) : 0);
  auto kern = pipe ? integrate_warp_kernel<NPL, WARP, kCanPipe, LANES> : integrate_warp_kernel<NPL, WARP, false, LANES>;
  check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)),
             "cudaFuncSetAttribute(integrate_warp)");
  int per_sm = 0;
  check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWarpThreads, smem), "occupancy");
  const int64_t tiles = (args.pixels + kWarpTilePx - 1) / kWarpTilePx;
  const int64_t resident = static_cast<int64_t>(std::max(per_sm, 1)) * sm_count();
  const unsigned grid = static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>(tiles, resident)));
  note_launch();
  kern<<<grid, kWarpThreads, smem, stream>>>(args);
  check_cuda(cudaGetLastError(), "integrate_warp launch");
}

template <int NB>
static void launch_reg(const IntegrateArgs& args, cudaStream_t stream) {
  constexpr int T = 128;
  const size_t smem = size_t(2) * NB * T * sizeof(float);
  auto kern = integrate_reg_kernel<NB, T>;
  check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)),
             "cudaFuncSetAttribute(integrate)");
  int per_sm = 0;
  check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, T, smem), "occupancy");
  const unsigned grid = grid_for(static_cast<size_t>(args.pixels), T, std::max(per_sm, 1));
  note_launch();
  kern<<<grid, T, smem, stream>>>(args);
  check_cuda(cudaGetLastError(), "integrate kernel launch");
}

template <int NB, int MODE>
static void launch_col(const IntegrateArgs& args, cudaStream_t stream) {
  constexpr int T = 128;
  const size_t smem = size_t(NB) * T * sizeof(float);
  auto run_kernel = [&](auto kern) {
    check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)),
               "cudaFuncSetAttribute(integrate)");
    int per_sm = 0;
    check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, T, smem), "occupancy");
    const unsigned grid = grid_for(static_cast<size_t>(args.pixels), T, std::max(per_sm, 1));
    note_launch();
    kern<<<grid, T, smem, stream>>>(args);
    check_cuda(cudaGetLastError(), "integrate kernel launch");
  };
  if constexpr (NB == 32 && MODE != GG_REJECT_NONE) {
    auto run = [&](int c) {
      if (c == 0) run_kernel(integrate_col_kernel<NB, T, MODE, 0, 1>);
      else run_kernel(integrate_col_kernel<NB, T, MODE, 0, 4>);
    };
    const std::string shape = std::to_string(args.frames) + " frames x " + std::to_string(args.pixels) +
                              " px mode" + std::to_string(MODE);
    run(autotune_choose("integrate_col registers", shape, {"unbounded", "4 CTAs/SM"}, 0, stream, run));
  } else {
    run_kernel(integrate_col_kernel<NB, T, MODE>);
  }
}

// Non-finite warped samples per frame for the fused path: the count the warp
// kernel would have left in the frame's counter (it selects the integrator's
// all-valid formulas).  Frames without non-finite source pixels only need
// the validity test; the others evaluate the sample.
template <int INTERP>
__global__ void __launch_bounds__(256) fused_nonfinite_kernel(IntegrateArgs a, unsigned* counts) {
  const int f = blockIdx.y;
  __shared__ FusedFrame fz;
  __shared__ const float* base;
  if (threadIdx.x == 0) {
    fz = a.fused[f];
    base = a.slots + static_cast<int64_t>(a.slot_of_frame[f]) * a.stride;
  }
  __syncthreads();
  const bool src_finite = fz.src_nonfinite == 0u;
  const float W = static_cast<float>(a.width), H = static_cast<float>(a.height);
  unsigned bad = 0;
  for (int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; p < a.pixels; p += int64_t(gridDim.x) * blockDim.x) {
    const int py = static_cast<int>(p / a.width), px = static_cast<int>(p - static_cast<int64_t>(py) * a.width);
    bool nan_out;
    if (src_finite) {
      FFv sx, sy;
      if (!source_coord(fz, static_cast<float>(px), static_cast<float>(py), sx, sy)) {
        nan_out = true;
      } else if (INTERP == GG_INTERP_BILINEAR) {
        nan_out = !(ff_ge(sx, 0.0f) && ff_le(sx, W - 1.0f) && ff_ge(sy, 0.0f) && ff_le(sy, H - 1.0f));
      } else if (!(ff_ge(sx, 2.0f) && ff_lt(sx, W - 3.0f) && ff_ge(sy, 2.0f) && ff_lt(sy, H - 3.0f))) {
        nan_out = true;
      } else {
        // all taps finite: the sample is invalid only for a vanishing weight sum
        int x0, y0;
        float tx, ty;
        ff_floor_frac(sx, x0, tx);
        ff_floor_frac(sy, y0, ty);
        float wx[6], wy[6];
        lanczos3_weights(tx, wx);
        lanczos3_weights(ty, wy);
        float sxw = 0.0f, syw = 0.0f;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
          sxw += wx[i];
          syw += wy[i];
        }
        nan_out = !(fabsf(sxw * syw) > 1.0e-12f);
      }
    } else {
      int geo = 0;
      nan_out = !isfinite(fused_sample<INTERP>(a, base, fz, px, py, geo));
    }
    bad += nan_out ? 1u : 0u;
  }
  bad = __reduce_add_sync(0xffffffffu, bad);
  if ((threadIdx.x & 31) == 0 && bad) atomicAdd(counts + f, bad);
}

template <int MR>
static void launch_smem(const IntegrateArgs& args, cudaStream_t stream) {
  constexpr int T = 32;
  const size_t smem = size_t(2) * MR * 32 * T * sizeof(float);
  auto kern = integrate_smem_kernel<MR, T>;
  check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)),
             "cudaFuncSetAttribute(integrate)");
  int per_sm = 0;
  check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, T, smem), "occupancy");
  const unsigned grid = grid_for(static_cast<size_t>(args.pixels), T, std::max(per_sm, 1));
  note_launch();
  kern<<<grid, T, smem, stream>>>(args);
  check_cuda(cudaGetLastError(), "integrate kernel launch");
}

static void validate_integrate(const gg_integrate_params_t& p) {
  require(p.rejection >= GG_REJECT_NONE && p.rejection <= GG_REJECT_LINEAR_FIT, "unsupported rejection mode");
  require(p.count_dtype == GG_COUNT_F32 || p.count_dtype == GG_COUNT_U16, "count_map_dtype must be float32 or uint16");
  if (p.rejection != GG_REJECT_NONE) {
    require(p.low_sigma > 0.0f && p.high_sigma > 0.0f, "sigma thresholds must be positive");
    require(p.min_samples >= 1, "min_samples must be at least 1");
    require(p.max_reject_fraction >= 0.0f && p.max_reject_fraction <= 1.0f,
            "max_reject_fraction must be between 0 and 1");
  }
}

static IntegrateArgs integrate_args(gg_stack* s, const float* d_weights, const gg_integrate_params_t& p);

void launch_integrate(gg_stack* s, const float* d_weights, const gg_integrate_params_t& p) {
  const IntegrateArgs a = integrate_args(s, d_weights, p);
  const int n = a.frames;
  if (n <= 32) {
    switch (p.rejection) {
      case GG_REJECT_NONE:
        n <= 8 ? launch_col<8, GG_REJECT_NONE>(a, s->stream)
               : n <= 16 ? launch_col<16, GG_REJECT_NONE>(a, s->stream) : launch_col<32, GG_REJECT_NONE>(a, s->stream);
        break;
      case GG_REJECT_SIGMA_CLIP:
        n <= 8 ? launch_col<8, GG_REJECT_SIGMA_CLIP>(a, s->stream)
               : n <= 16 ? launch_col<16, GG_REJECT_SIGMA_CLIP>(a, s->stream)
                         : launch_col<32, GG_REJECT_SIGMA_CLIP>(a, s->stream);
        break;
      case GG_REJECT_WINSORIZED:
        n <= 8 ? launch_col<8, GG_REJECT_WINSORIZED>(a, s->stream)
               : n <= 16 ? launch_col<16, GG_REJECT_WINSORIZED>(a, s->stream)
                         : launch_col<32, GG_REJECT_WINSORIZED>(a, s->stream);
        break;
      default:
        n <= 8 ? launch_col<8, GG_REJECT_LINEAR_FIT>(a, s->stream)
               : n <= 16 ? launch_col<16, GG_REJECT_LINEAR_FIT>(a, s->stream)
                         : launch_col<32, GG_REJECT_LINEAR_FIT>(a, s->stream);
        break;
    }
  }
  else if (p.rejection != GG_REJECT_LINEAR_FIT && n <= 512) {
    // one warp per pixel (the linear fit's serial rank walks stay below)
    // two pixels per warp up to 256 frames (16 lanes x NPL values each)
    if (n <= 64) launch_warp<4, 0, 16>(a, s->stream);
    else if (n <= 128) launch_warp<8, 0, 16>(a, s->stream);
    else if (n <= 256) launch_warp<16, 0, 16>(a, s->stream);
    else launch_warp<16>(a, s->stream);
  }
  else if (n <= 64) launch_reg<64>(a, s->stream);
  else if (n <= 128) launch_smem<4>(a, s->stream);
  else if (n <= 256) launch_smem<8>(a, s->stream);
  else if (n <= 512) launch_smem<16>(a, s->stream);
  else fail(GG_ERR_INVALID_ARGUMENT, "frame_count above 512 is not supported by the resident integrator");
  s->last_count_dtype = p.count_dtype;
}

// Several stacks of at most 32 frames in one launch of the column kernel
// (NB = the largest frame count's bucket); CTAs are shared out in proportion
// to each stack's samples (pixels x frames), at least one per stack.
template <int MODE>
static void launch_batch(std::vector<gg_stack*>& stacks, const std::vector<IntegrateArgs>& args, int nb,
                         IntegrateArgs* d_args) {
  constexpr int T = 128;
  cudaStream_t stream = stacks[0]->stream;
  BatchTable bt{};
  bt.stacks = static_cast<int>(stacks.size());
  auto launch = [&](auto kern, int NBv) {
    const size_t smem = size_t(NBv) * T * sizeof(float);
    check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)),
               "cudaFuncSetAttribute(integrate batch)");
    int per_sm = 0;
    check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, T, smem), "occupancy");
    const double budget = static_cast<double>(sm_count()) * std::max(per_sm, 1);
    double work = 0.0;
    for (const IntegrateArgs& a : args) work += static_cast<double>(a.pixels) * a.frames;
    bt.start[0] = 0;
    for (size_t k = 0; k < args.size(); ++k) {
      const int64_t most = (args[k].pixels + T - 1) / T;
      const int64_t share = static_cast<int64_t>(budget * static_cast<double>(args[k].pixels) * args[k].frames / work);
      bt.start[k + 1] = bt.start[k] + static_cast<int>(std::max<int64_t>(1, std::min(most, share)));
    }
    note_launch();
    kern<<<static_cast<unsigned>(bt.start[args.size()]), T, smem, stream>>>(d_args, bt);
    check_cuda(cudaGetLastError(), "integrate batch launch");
  };
  if (nb <= 8) launch(integrate_batch_kernel<8, T, MODE>, 8);
  else if (nb <= 16) launch(integrate_batch_kernel<16, T, MODE>, 16);
  else launch(integrate_batch_kernel<32, T, MODE, MODE == GG_REJECT_NONE ? 1 : 4>, 32);
}

static IntegrateArgs integrate_args(gg_stack* s, const float* d_weights, const gg_integrate_params_t& p) {
  stack_ensure_maps(s);
  IntegrateArgs a{};
  a.slots = s->d_slots;
  a.slot_of_frame = s->d_slot_of_frame;
  a.stride = s->stride;
  a.pixels = s->pixels;
  a.frames = static_cast<int>(s->frames);
  a.weights = d_weights;
  a.nonfinite = s->d_frame_nonfinite;
  a.rejection = p.rejection;
  a.low_sigma = p.low_sigma;
  a.high_sigma = p.high_sigma;
  a.min_samples = p.min_samples;
  a.max_frac = p.max_reject_fraction;
  a.lfc_iterations = p.linear_fit_iterations > 0 ? p.linear_fit_iterations : 5;
  a.master = s->d_master;
  a.weight = s->d_weight;
  a.coverage = s->d_coverage;
  a.low = s->d_low;
  a.high = s->d_high;
  a.dq = s->d_dq;
  a.count_u16 = p.count_dtype == GG_COUNT_U16;
  a.geometric = (s->d_warp_coverage && s->warp_coverage_frames > 0) ? s->d_warp_coverage : nullptr;
  return a;
}

// Integrates `count` stacks (same device, each at most 32 frames, each with
// its own device weights) in one launch on the first stack's stream; the
// other stacks' streams are joined before and after it.
static void integrate_batch(std::vector<gg_stack*>& stacks, const gg_integrate_params_t& p) {
  const int count = static_cast<int>(stacks.size());
  // one launch per frame-count bucket (8 / 16 / 32): a stack never pays for
  // a larger sorting network than its own
  auto bucket = [](int n) { return n <= 8 ? 0 : (n <= 16 ? 1 : 2); };
  std::vector<IntegrateArgs> args;
  int bucket_start[4] = {0, 0, 0, 0};
  for (int b = 0; b < 3; ++b) {
    bucket_start[b] = static_cast<int>(args.size());
    for (gg_stack* s : stacks)
      if (bucket(static_cast<int>(s->frames)) == b) args.push_back(integrate_args(s, s->d_weights, p));
  }
  bucket_start[3] = static_cast<int>(args.size());
  gg_stack* lead = stacks[0];
  // join: the lead stream waits for every stack's queued work
  std::vector<cudaEvent_t> events;
  auto cleanup = [&]() {
    for (cudaEvent_t e : events) cudaEventDestroy(e);
  };
  try {
    for (int k = 1; k < count; ++k) {
      cudaEvent_t e = nullptr;
      check_cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate(batch)");
      events.push_back(e);
      check_cuda(cudaEventRecord(e, stacks[static_cast<size_t>(k)]->stream), "cudaEventRecord(batch)");
      check_cuda(cudaStreamWaitEvent(lead->stream, e, 0), "cudaStreamWaitEvent(batch)");
    }
    IntegrateArgs* d_args = nullptr;
    check_cuda(cudaMallocAsync(reinterpret_cast<void**>(&d_args), sizeof(IntegrateArgs) * count, lead->stream),
               "cudaMallocAsync(batch args)");
    upload_params(lead->stream, d_args, args.data(), sizeof(IntegrateArgs) * count, "cudaMemcpyAsync(batch args)");
    for (int b = 0; b < 3; ++b) {
      if (bucket_start[b + 1] == bucket_start[b]) continue;
      const std::vector<IntegrateArgs> sub(args.begin() + bucket_start[b], args.begin() + bucket_start[b + 1]);
      const int nb = b == 0 ? 8 : (b == 1 ? 16 : 32);
      IntegrateArgs* d_sub = d_args + bucket_start[b];
      switch (p.rejection) {
        case GG_REJECT_NONE: launch_batch<GG_REJECT_NONE>(stacks, sub, nb, d_sub); break;
        case GG_REJECT_SIGMA_CLIP: launch_batch<GG_REJECT_SIGMA_CLIP>(stacks, sub, nb, d_sub); break;
        case GG_REJECT_WINSORIZED: launch_batch<GG_REJECT_WINSORIZED>(stacks, sub, nb, d_sub); break;
        default: launch_batch<GG_REJECT_LINEAR_FIT>(stacks, sub, nb, d_sub); break;
      }
    }
    check_cuda(cudaFreeAsync(d_args, lead->stream), "cudaFreeAsync(batch args)");
    // the other stacks' later work waits for the batch
    cudaEvent_t done = nullptr;
    check_cuda(cudaEventCreateWithFlags(&done, cudaEventDisableTiming), "cudaEventCreate(batch)");
    events.push_back(done);
    check_cuda(cudaEventRecord(done, lead->stream), "cudaEventRecord(batch)");
    for (int k = 1; k < count; ++k)
      check_cuda(cudaStreamWaitEvent(stacks[static_cast<size_t>(k)]->stream, done, 0), "cudaStreamWaitEvent(batch)");
  } catch (...) {
    cleanup();
    throw;
  }
  cleanup();
  for (gg_stack* s : stacks) s->last_count_dtype = p.count_dtype;
}

__global__ void fused_prepare_kernel(FusedFrame* fused, const unsigned* src_nonfinite, unsigned* counts, int frames) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= frames) return;
  fused[f].src_nonfinite = src_nonfinite[f];
  counts[f] = 0u;
}

template <int MODE, int INTERP>
static void launch_fused(const IntegrateArgs& a, cudaStream_t stream) {
  constexpr int T = 128;
  const size_t smem = size_t(32) * T * sizeof(float);
  auto kern = integrate_col_kernel<32, T, MODE, INTERP>;
  check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)),
             "cudaFuncSetAttribute(fused integrate)");
  int per_sm = 0;
  check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, T, smem), "occupancy");
  // pixel tile shape (tile_w x tile_h = T): wider tiles coalesce the map
  // writes, taller ones share the Lanczos / bilinear source rows in L1
  static const int kTiles[3][2] = {{128, 1}, {64, 2}, {32, 4}};
  auto run = [&](int c) {
    IntegrateArgs b = a;
    b.tile_w = kTiles[c][0];
    b.tile_h = kTiles[c][1];
    b.tiles_x = (a.width + b.tile_w - 1) / b.tile_w;
    b.tile_slots = b.tiles_x * ((a.height + b.tile_h - 1) / b.tile_h) * T;
    const unsigned grid = grid_for(static_cast<size_t>(b.tile_slots), T, std::max(per_sm, 1));
    note_launch();
    kern<<<grid, T, smem, stream>>>(b);
    check_cuda(cudaGetLastError(), "fused integrate launch");
  };
  const std::string shape = std::to_string(a.frames) + "x" + std::to_string(a.height) + "x" +
                            std::to_string(a.width) + (INTERP == GG_INTERP_LANCZOS3 ? " lanczos3" : " bilinear") +
                            " mode" + std::to_string(MODE);
  run(autotune_choose("fused_warp_integrate tile", shape, {"128x1", "64x2", "32x4"}, 0, stream, run));
}

// integrate_matrix_warped_{mean,sigma_clip} (integration_kernels.cu:3840-4123):
// the result of warping every frame through its matrix (NaN fill) and
// integrating, without writing the warped frames.
static void validate_fused(gg_stack* s, int interp, const gg_integrate_params_t& p) {
  require(s->frames <= 512, "fused warp-integration supports at most 512 frames");
  require(p.rejection == GG_REJECT_NONE || p.rejection == GG_REJECT_SIGMA_CLIP || p.rejection == GG_REJECT_WINSORIZED,
          "fused warp-integration supports the mean, sigma-clip and winsorized sigma-clip rejections");
  require(interp == GG_INTERP_BILINEAR || interp == GG_INTERP_LANCZOS3,
          "fused matrix-warped interpolation must be bilinear or lanczos3");
}

// Float-float inverse coefficients of every frame's forward matrix.
static std::vector<FusedFrame> fused_frames_host(const double* fwd, int n) {
  std::vector<FusedFrame> frames(static_cast<size_t>(n));
  for (int f = 0; f < n; ++f) {
    const double* m = fwd + 9 * f;
    for (int q = 0; q < 9; ++q)
      if (!std::isfinite(m[q])) fail(GG_ERR_INVALID_ARGUMENT, "warp matrix must be finite");
    FusedFrame& ff = frames[static_cast<size_t>(f)];
    std::memset(&ff, 0, sizeof(ff));
    if (!inverse_coefficients(m, ff.m, ff.affine)) fail(GG_ERR_INVALID_ARGUMENT, "warp matrix is singular");
  }
  return frames;
}

static void ensure_fused_buffers(gg_stack* s) {
  stack_ensure_maps(s);
  const int n = static_cast<int>(s->frames);
  if (!s->d_fused_frames) {
    check_cuda(cudaMalloc(&s->d_fused_frames, sizeof(FusedFrame) * n), "cudaMalloc(fused frames)");
    check_cuda(cudaMalloc(&s->d_fused_counts, sizeof(unsigned) * n), "cudaMalloc(fused counts)");
    check_cuda(cudaMalloc(&s->d_fused_geometric, sizeof(float) * s->pixels), "cudaMalloc(fused coverage)");
    s->bytes_allocated += static_cast<int64_t>(sizeof(FusedFrame) + sizeof(unsigned)) * n + 4 * s->pixels;
  }
}

// The device part of the fused warp-integration: every argument already on
// the device, nothing but kernel launches on the stack's stream (so it can
// be captured into a CUDA graph).
static void launch_fused_sequence(gg_stack* s, FusedFrame* d_frames, int interp, float clamp, const float* d_weights,
                                  const gg_integrate_params_t& p) {
  const int n = static_cast<int>(s->frames);
  note_launch();
  fused_prepare_kernel<<<(n + 127) / 128, 128, 0, s->stream>>>(d_frames, s->d_frame_nonfinite, s->d_fused_counts, n);
  check_cuda(cudaGetLastError(), "fused_prepare launch");
  IntegrateArgs a{};
  a.slots = s->d_slots;
  a.slot_of_frame = s->d_slot_of_frame;
  a.stride = s->stride;
  a.pixels = s->pixels;
  a.frames = n;
  a.weights = d_weights;
  a.nonfinite = s->d_fused_counts;
  a.rejection = p.rejection;
  a.low_sigma = p.low_sigma;
  a.high_sigma = p.high_sigma;
  a.min_samples = p.min_samples;
  a.max_frac = p.max_reject_fraction;
  a.lfc_iterations = 5;
  a.master = s->d_master;
  a.weight = s->d_weight;
  a.coverage = s->d_coverage;
  a.low = s->d_low;
  a.high = s->d_high;
  a.dq = s->d_dq;
  a.count_u16 = p.count_dtype == GG_COUNT_U16;
  a.fused = d_frames;
  a.width = static_cast<int>(s->width);
  a.height = static_cast<int>(s->height);
  a.clamp = clamp;
  a.geometric_out = s->d_fused_geometric;
  a.geometric = s->d_fused_geometric;
  const dim3 count_grid(static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>((s->pixels + 255) / 256,
                                                                                      sm_count() * 8 / n + 1))),
                        static_cast<unsigned>(n));
  note_launch();
  if (interp == GG_INTERP_BILINEAR)
    fused_nonfinite_kernel<GG_INTERP_BILINEAR><<<count_grid, 256, 0, s->stream>>>(a, s->d_fused_counts);
  else
    fused_nonfinite_kernel<GG_INTERP_LANCZOS3><<<count_grid, 256, 0, s->stream>>>(a, s->d_fused_counts);
  check_cuda(cudaGetLastError(), "fused_nonfinite launch");
  if (n > 32) {  // one warp per pixel over a sampled [frame][32 px] tile
    auto run = [&](auto tag) {
      constexpr int I = decltype(tag)::value;
      if (n <= 64) launch_warp<2, I>(a, s->stream);
      else if (n <= 128) launch_warp<4, I>(a, s->stream);
      else if (n <= 256) launch_warp<8, I>(a, s->stream);
      else launch_warp<16, I>(a, s->stream);
    };
    if (interp == GG_INTERP_BILINEAR) run(std::integral_constant<int, GG_INTERP_BILINEAR>{});
    else run(std::integral_constant<int, GG_INTERP_LANCZOS3>{});
  } else if (interp == GG_INTERP_BILINEAR) {
    if (p.rejection == GG_REJECT_NONE) launch_fused<GG_REJECT_NONE, GG_INTERP_BILINEAR>(a, s->stream);
    else if (p.rejection == GG_REJECT_SIGMA_CLIP) launch_fused<GG_REJECT_SIGMA_CLIP, GG_INTERP_BILINEAR>(a, s->stream);
    else launch_fused<GG_REJECT_WINSORIZED, GG_INTERP_BILINEAR>(a, s->stream);
  } else {
    if (p.rejection == GG_REJECT_NONE) launch_fused<GG_REJECT_NONE, GG_INTERP_LANCZOS3>(a, s->stream);
    else if (p.rejection == GG_REJECT_SIGMA_CLIP) launch_fused<GG_REJECT_SIGMA_CLIP, GG_INTERP_LANCZOS3>(a, s->stream);
    else launch_fused<GG_REJECT_WINSORIZED, GG_INTERP_LANCZOS3>(a, s->stream);
  }
  s->last_count_dtype = p.count_dtype;
  s->has_fused_geometric = true;
}

static void integrate_warped(gg_stack* s, const double* fwd, int interp, float clamp, const float* d_weights,
                             const gg_integrate_params_t& p) {
  validate_fused(s, interp, p);
  const std::vector<FusedFrame> frames = fused_frames_host(fwd, static_cast<int>(s->frames));
  ensure_fused_buffers(s);
  auto* d_frames = static_cast<FusedFrame*>(s->d_fused_frames);
  upload_params(s->stream, d_frames, frames.data(), sizeof(FusedFrame) * frames.size(),
                "cudaMemcpyAsync(fused frames)");
  launch_fused_sequence(s, d_frames, interp, clamp, d_weights, p);
}

// ---- CUDA graph of the resident step with fixed matrices ---------------------
// calibrate (uint16 frames already on the device) -> frame weights -> fused
// warp + rejection + integration.  The graph owns its inverse-coefficient
// buffer; it reads the raw frames from the device pointer given at capture
// and writes the stack's maps at every replay.
struct StepGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  FusedFrame* d_frames = nullptr;
  int kernels = 0;
};

static void step_graph_release(StepGraph& g) {
  if (g.exec) cudaGraphExecDestroy(g.exec);
  if (g.graph) cudaGraphDestroy(g.graph);
  if (g.d_frames) cudaFree(g.d_frames);
  g = StepGraph{};
}

static StepGraph& step_graph(gg_stack* s) {
  if (!s->step_graph) {
    s->step_graph = new StepGraph();
    s->step_graph_free = [](void* q) {
      auto* g = static_cast<StepGraph*>(q);
      step_graph_release(*g);
      delete g;
    };
  }
  return *static_cast<StepGraph*>(s->step_graph);
}

static void run_step_sequence(gg_stack* s, const void* dev_raw, const std::vector<int64_t>& idx,
                              const gg_calib_params_t& calib, int weighting, FusedFrame* d_frames, int interp,
                              float clamp, const gg_integrate_params_t& p) {
  int rc = gg_stack_calibrate_u16_device(s, idx.data(), static_cast<int64_t>(idx.size()), dev_raw, 0, &calib);
  if (rc != GG_OK) fail(rc, "step graph: calibration failed");
  rc = gg_stack_compute_weights(s, weighting, nullptr, 1.0e-6f, nullptr);
  if (rc != GG_OK) fail(rc, "step graph: frame weighting failed");
  launch_fused_sequence(s, d_frames, interp, clamp, s->d_weights, p);
}

}  // namespace gg

extern "C" int gg_stack_graph_capture_step(gg_stack* s, const void* dev_raw, const double* host_matrices,
                                           int interpolation, float clamping_threshold, int weighting,
                                           const gg_calib_params_t* calib, const gg_integrate_params_t* params) {
  using namespace gg;
  GG_API_BEGIN
  require(s != nullptr && dev_raw != nullptr && host_matrices != nullptr && calib != nullptr && params != nullptr,
          "null argument");
  require(weighting == GG_WEIGHTS_PRIOR || weighting == GG_WEIGHTS_SIMPLE_SNR, "unsupported weighting mode");
  validate_integrate(*params);
  validate_fused(s, interpolation, *params);
  stack_activate(s);
  const std::vector<FusedFrame> frames = fused_frames_host(host_matrices, static_cast<int>(s->frames));
  StepGraph& g = step_graph(s);
  step_graph_release(g);
  check_cuda(cudaMalloc(&g.d_frames, sizeof(FusedFrame) * frames.size()), "cudaMalloc(step graph frames)");
  check_cuda(cudaMemcpy(g.d_frames, frames.data(), sizeof(FusedFrame) * frames.size(), cudaMemcpyHostToDevice),
             "cudaMemcpy(step graph frames)");
  ensure_fused_buffers(s);
  std::vector<int64_t> idx(static_cast<size_t>(s->frames));
  for (int64_t k = 0; k < s->frames; ++k) idx[static_cast<size_t>(k)] = k;
  // one eager pass: validates the inputs, sizes every lazily allocated
  // buffer, so the capture only records launches and stream-ordered copies
  run_step_sequence(s, dev_raw, idx, *calib, weighting, g.d_frames, interpolation, clamping_threshold, *params);
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(step graph warm-up)");
  const int64_t before = gg::launch_count();
  check_cuda(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeRelaxed), "cudaStreamBeginCapture");
  try {
    run_step_sequence(s, dev_raw, idx, *calib, weighting, g.d_frames, interpolation, clamping_threshold, *params);
  } catch (...) {
    cudaGraph_t broken = nullptr;
    cudaStreamEndCapture(s->stream, &broken);
    if (broken) cudaGraphDestroy(broken);
    note_launch(static_cast<int>(before - gg::launch_count()));
    throw;
  }
  check_cuda(cudaStreamEndCapture(s->stream, &g.graph), "cudaStreamEndCapture");
  g.kernels = static_cast<int>(gg::launch_count() - before);
  note_launch(-g.kernels);  // recorded, not executed
  check_cuda(cudaGraphInstantiate(&g.exec, g.graph, 0), "cudaGraphInstantiate");
  GG_API_END
}

// ---- several stacks in one graph ------------------------------------------------
namespace gg {
void* warp_items_device(gg_stack* s, const int64_t* indices, int64_t count, const double* fwd);
void launch_warp_items_device(gg_stack* s, void* d_items, int64_t count, int interp, float fill, float clamp);
}  // namespace gg

struct gg_stacks_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t stream = nullptr;
  int device = 0;
  std::vector<void*> items;       // per step: device warp descriptors (or null)
  std::vector<int64_t> warped;    // per step: descriptor count
  int kernels = 0;
};

namespace gg {

static void stacks_graph_free(gg_stacks_graph* g) {
  if (!g) return;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  for (void* p : g->items)
    if (p) cudaFree(p);
  delete g;
}

// One stack's step on its (current) stream: decode + calibration of every
// frame, frame weights, the warp of every frame whose matrix is not the
// identity, rejection + integration with the device weights.
static void run_stack_step(const gg_stack_step_t& st, void* d_items, int64_t warped) {
  gg_stack* s = st.stack;
  std::vector<int64_t> idx(static_cast<size_t>(s->frames));
  for (int64_t k = 0; k < s->frames; ++k) idx[static_cast<size_t>(k)] = k;
  int rc = gg_stack_calibrate_u16_device(s, idx.data(), s->frames, st.dev_raw, 0, &st.calib);
  if (rc != GG_OK) fail(rc, "stacks graph: calibration failed");
  rc = gg_stack_compute_weights(s, st.weighting, nullptr, 1.0e-6f, nullptr);
  if (rc != GG_OK) fail(rc, "stacks graph: frame weighting failed");
  if (warped > 0) launch_warp_items_device(s, d_items, warped, st.interpolation, NAN, st.clamping_threshold);
  launch_integrate(s, s->d_weights, st.integrate);
}

}  // namespace gg

extern "C" int gg_stacks_graph_capture(const gg_stack_step_t* steps, int32_t count, void* cuda_stream,
                                       gg_stacks_graph** out) {
  using namespace gg;
  GG_API_BEGIN
  require(steps != nullptr && out != nullptr, "null argument");
  require(count >= 1 && count <= kMaxBatchStacks, "stack count must be in [1, 64]");
  *out = nullptr;
  for (int k = 0; k < count; ++k) {
    const gg_stack_step_t& st = steps[k];
    require(st.stack != nullptr && st.dev_raw != nullptr && st.host_matrices != nullptr, "null argument");
    require(st.stack->device == steps[0].stack->device, "stacks of one graph must live on one device");
    for (int j = 0; j < k; ++j) require(steps[j].stack != st.stack, "a stack appears twice in the graph");
    require(st.interpolation == GG_INTERP_BILINEAR || st.interpolation == GG_INTERP_LANCZOS3,
            "interpolation must be bilinear or lanczos3");
    require(st.weighting == GG_WEIGHTS_PRIOR || st.weighting == GG_WEIGHTS_SIMPLE_SNR, "unsupported weighting mode");
    validate_integrate(st.integrate);
    require(st.stack->width < (1 << 24) && st.stack->height < (1 << 24), "frame too large for float coordinates");
  }
  gg_stack* first = steps[0].stack;
  stack_activate(first);
  auto* g = new gg_stacks_graph();
  struct Guard {
    gg_stacks_graph*& g;
    std::vector<cudaStream_t> saved;
    const gg_stack_step_t* steps;
    int count;
    ~Guard() {
      for (int k = 0; k < static_cast<int>(saved.size()); ++k) steps[k].stack->stream = saved[k];
      if (g) stacks_graph_free(g);
    }
  } guard{g, {}, steps, count};
  g->device = first->device;
  g->stream = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : first->stream;
  for (int k = 0; k < count; ++k) {
    const gg_stack_step_t& st = steps[k];
    std::vector<int64_t> idx;
    std::vector<double> mats;
    for (int64_t f = 0; f < st.stack->frames; ++f) {
      const double* m = st.host_matrices + 9 * f;
      const bool identity = m[0] == 1.0 && m[1] == 0.0 && m[2] == 0.0 && m[3] == 0.0 && m[4] == 1.0 &&
                            m[5] == 0.0 && m[6] == 0.0 && m[7] == 0.0 && m[8] == 1.0;
      if (identity) continue;
      idx.push_back(f);
      mats.insert(mats.end(), m, m + 9);
    }
    // the frames must hold data for the descriptor checks; the warm-up
    // calibration below loads them, so calibrate first
    guard.saved.push_back(st.stack->stream);
    st.stack->stream = g->stream;
    std::vector<int64_t> all(static_cast<size_t>(st.stack->frames));
    for (int64_t f = 0; f < st.stack->frames; ++f) all[static_cast<size_t>(f)] = f;
    const int rc = gg_stack_calibrate_u16_device(st.stack, all.data(), st.stack->frames, st.dev_raw, 0, &st.calib);
    if (rc != GG_OK) fail(rc, "stacks graph: calibration failed");
    g->items.push_back(idx.empty() ? nullptr : warp_items_device(st.stack, idx.data(), static_cast<int64_t>(idx.size()),
                                                                  mats.data()));
    g->warped.push_back(static_cast<int64_t>(idx.size()));
  }
  // one eager pass sizes every lazily allocated buffer and settles the
  // autotuner, so the capture records launches and stream-ordered copies only
  for (int k = 0; k < count; ++k) run_stack_step(steps[k], g->items[k], g->warped[k]);
  check_cuda(cudaStreamSynchronize(g->stream), "cudaStreamSynchronize(stacks graph warm-up)");
  const int64_t before = gg::launch_count();
  check_cuda(cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeRelaxed), "cudaStreamBeginCapture");
  try {
    for (int k = 0; k < count; ++k) run_stack_step(steps[k], g->items[k], g->warped[k]);
  } catch (...) {
    cudaGraph_t broken = nullptr;
    cudaStreamEndCapture(g->stream, &broken);
    if (broken) cudaGraphDestroy(broken);
    note_launch(static_cast<int>(before - gg::launch_count()));
    throw;
  }
  check_cuda(cudaStreamEndCapture(g->stream, &g->graph), "cudaStreamEndCapture");
  g->kernels = static_cast<int>(gg::launch_count() - before);
  note_launch(-g->kernels);  // recorded, not executed
  check_cuda(cudaGraphInstantiate(&g->exec, g->graph, 0), "cudaGraphInstantiate");
  *out = g;
  g = nullptr;  // owned by the caller now
  GG_API_END
}

extern "C" int gg_stacks_graph_launch(gg_stacks_graph* g) {
  using namespace gg;
  GG_API_BEGIN
  require(g != nullptr && g->exec != nullptr, "null graph");
  check_cuda(cudaSetDevice(g->device), "cudaSetDevice");
  check_cuda(cudaGraphLaunch(g->exec, g->stream), "cudaGraphLaunch");
  note_launch(g->kernels);
  GG_API_END
}

extern "C" int gg_stacks_graph_kernel_count(gg_stacks_graph* g, int32_t* out) {
  using namespace gg;
  GG_API_BEGIN
  require(g != nullptr && out != nullptr, "null argument");
  *out = g->kernels;
  GG_API_END
}

extern "C" int gg_stacks_graph_destroy(gg_stacks_graph* g) {
  using namespace gg;
  GG_API_BEGIN
  if (g) {
    check_cuda(cudaSetDevice(g->device), "cudaSetDevice");
    stacks_graph_free(g);
  }
  GG_API_END
}

extern "C" int gg_stack_graph_launch(gg_stack* s) {
  using namespace gg;
  GG_API_BEGIN
  require(s != nullptr, "null argument");
  require(s->step_graph && static_cast<StepGraph*>(s->step_graph)->exec, "no step graph has been captured");
  stack_activate(s);
  StepGraph& g = *static_cast<StepGraph*>(s->step_graph);
  check_cuda(cudaGraphLaunch(g.exec, s->stream), "cudaGraphLaunch");
  note_launch(g.kernels);
  GG_API_END
}

extern "C" int gg_stack_graph_kernel_count(gg_stack* s, int* out) {
  using namespace gg;
  GG_API_BEGIN
  require(s != nullptr && out != nullptr, "null argument");
  *out = s->step_graph ? static_cast<StepGraph*>(s->step_graph)->kernels : 0;
  GG_API_END
}

extern "C" int gg_stack_graph_destroy(gg_stack* s) {
  using namespace gg;
  GG_API_BEGIN
  require(s != nullptr, "null argument");
  if (s->step_graph) step_graph_release(*static_cast<StepGraph*>(s->step_graph));
  GG_API_END
}

using namespace gg;

extern "C" {

int gg_stack_integrate(gg_stack* s, const float* host_weights, const gg_integrate_params_t* params) {
  GG_API_BEGIN
  require(s != nullptr && params != nullptr, "null argument");
  validate_integrate(*params);
  stack_require_all_loaded(s, "integration");
  stack_activate(s);
  for (int64_t f = 0; f < s->frames; ++f) s->h_weights_pinned[f] = host_weights ? host_weights[f] : 1.0f;
  upload_params(s->stream, s->d_weights, s->h_weights_pinned, sizeof(float) * s->frames, "cudaMemcpyAsync(weights)");
  launch_integrate(s, s->d_weights, *params);
  GG_API_END
}

int gg_stack_integrate_device_weights(gg_stack* s, const void* dev_weights, const gg_integrate_params_t* params) {
  GG_API_BEGIN
  require(s != nullptr && params != nullptr, "null argument");
  validate_integrate(*params);
  stack_require_all_loaded(s, "integration");
  stack_activate(s);
  launch_integrate(s, dev_weights ? static_cast<const float*>(dev_weights) : s->d_weights, *params);
  GG_API_END
}

int gg_stacks_integrate_batch(gg_stack* const* stacks, int32_t count, const gg_integrate_params_t* params) {
  GG_API_BEGIN
  require(stacks != nullptr && params != nullptr, "null argument");
  require(count >= 1 && count <= kMaxBatchStacks, "stack count must be in [1, 64]");
  validate_integrate(*params);
  std::vector<gg_stack*> v(static_cast<size_t>(count));
  for (int k = 0; k < count; ++k) {
    gg_stack* s = stacks[k];
    require(s != nullptr, "null stack");
    require(s->device == stacks[0]->device, "batched stacks must live on one device");
    require(s->frames <= 32, "batched integration takes stacks of at most 32 frames");
    for (int j = 0; j < k; ++j) require(stacks[j] != s, "a stack appears twice in the batch");
    stack_require_all_loaded(s, "batched integration");
    v[static_cast<size_t>(k)] = s;
  }
  stack_activate(stacks[0]);
  integrate_batch(v, *params);
  GG_API_END
}

int gg_stack_integrate_warped(gg_stack* s, const double* host_matrices, int interpolation, float clamping_threshold,
                              const float* host_weights, const gg_integrate_params_t* params) {
  GG_API_BEGIN
  require(s != nullptr && host_matrices != nullptr && params != nullptr, "null argument");
  validate_integrate(*params);
  stack_require_all_loaded(s, "fused warp-integration");
  stack_activate(s);
  for (int64_t f = 0; f < s->frames; ++f) s->h_weights_pinned[f] = host_weights ? host_weights[f] : 1.0f;
  upload_params(s->stream, s->d_weights, s->h_weights_pinned, sizeof(float) * s->frames, "cudaMemcpyAsync(weights)");
  integrate_warped(s, host_matrices, interpolation, clamping_threshold, s->d_weights, *params);
  GG_API_END
}

int gg_stack_integrate_warped_device_weights(gg_stack* s, const double* host_matrices, int interpolation,
                                             float clamping_threshold, const gg_integrate_params_t* params) {
  GG_API_BEGIN
  require(s != nullptr && host_matrices != nullptr && params != nullptr, "null argument");
  validate_integrate(*params);
  stack_require_all_loaded(s, "fused warp-integration");
  stack_activate(s);
  integrate_warped(s, host_matrices, interpolation, clamping_threshold, s->d_weights, *params);
  GG_API_END
}

int gg_stack_download_fused_coverage(gg_stack* s, float* host_out) {
  GG_API_BEGIN
  require(s != nullptr && host_out != nullptr, "null argument");
  if (!s->has_fused_geometric) fail(GG_ERR_RUNTIME, "no fused warp-integration has been run");
  stack_activate(s);
  check_cuda(cudaMemcpyAsync(host_out, s->d_fused_geometric, sizeof(float) * s->pixels, cudaMemcpyDeviceToHost,
                             s->stream),
             "cudaMemcpyAsync(fused coverage)");
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(fused coverage)");
  GG_API_END
}

int gg_stack_download_maps(gg_stack* s, float* host_master, float* host_weight, void* host_coverage, void* host_low,
                           void* host_high, int16_t* host_dq) {
  GG_API_BEGIN
  require(s != nullptr, "stack is null");
  if (s->d_master == nullptr || s->last_count_dtype < 0) fail(GG_ERR_RUNTIME, "no integration has been run");
  stack_activate(s);
  const size_t p = static_cast<size_t>(s->pixels);
  const size_t cb = s->last_count_dtype == GG_COUNT_U16 ? 2 : 4;
  struct Item {
    void* dst;
    const void* src;
    size_t bytes;
  } items[] = {{host_master, s->d_master, p * 4}, {host_weight, s->d_weight, p * 4},
               {host_coverage, s->d_coverage, p * cb}, {host_low, s->d_low, p * cb},
               {host_high, s->d_high, p * cb}, {host_dq, s->d_dq, p * 2}};
  for (auto& it : items) {
    if (!it.dst) continue;
    check_cuda(cudaMemcpyAsync(it.dst, it.src, it.bytes, cudaMemcpyDeviceToHost, s->stream),
               "cudaMemcpyAsync(download maps)");
  }
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(download maps)");
  GG_API_END
}

}  // extern "C"
