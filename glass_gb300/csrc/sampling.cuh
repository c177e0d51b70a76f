// Source sampling shared by the warps and the fused warp-integration:
// bilinear and Lanczos3 taps read from a shared-memory box or from global
// memory (engine/warp.py:99-152; warp_kernels.cu:371-777).
#pragma once

#include "geometry.cuh"

namespace gg {

constexpr float kInfF = __builtin_huge_valf();
// Shared-memory source box of the tiled warp (columns x rows).
constexpr int kBoxW = 80;
constexpr int kBoxH = 64;

// sin(pi u) for |u| <= 1/2 and sin / cos of |x| <= pi/3 by their Taylor
// series (truncation below 1e-9 on these ranges), evaluated by Horner.
__device__ __forceinline__ float sin_taylor(float z) {
  const float z2 = z * z;
  float p = 1.0f / 6227020800.0f;
  p = __fmaf_rn(p, z2, -1.0f / 39916800.0f);
  p = __fmaf_rn(p, z2, 1.0f / 362880.0f);
  p = __fmaf_rn(p, z2, -1.0f / 5040.0f);
  p = __fmaf_rn(p, z2, 1.0f / 120.0f);
  p = __fmaf_rn(p, z2, -1.0f / 6.0f);
  return __fmaf_rn(p * z2, z, z);
}

__device__ __forceinline__ float cos_taylor(float z) {
  const float z2 = z * z;
  float p = -1.0f / 87178291200.0f;
  p = __fmaf_rn(p, z2, 1.0f / 479001600.0f);
  p = __fmaf_rn(p, z2, -1.0f / 3628800.0f);
  p = __fmaf_rn(p, z2, 1.0f / 40320.0f);
  p = __fmaf_rn(p, z2, -1.0f / 720.0f);
  p = __fmaf_rn(p, z2, 1.0f / 24.0f);
  p = __fmaf_rn(p, z2, -0.5f);
  return __fmaf_rn(p, z2, 1.0f);
}

constexpr float kPiF = 3.14159265358979323846f;

// Lanczos3 weights of taps k = -2..3 at fractional offset t in [0, 1): the
// tap at distance d = t - k weighs L(d) = sinc(d) sinc(d / 3).  With
// u = t - 1/2 the taps pair up as L(c + u), L(c - u) for c = 1/2 (k = 0, 1),
// 3/2 (k = -1, 2) and 5/2 (k = -2, 3); each pair is E_c(u) +- O_c(u) with
// E_c even and O_c odd, evaluated as degree-5 polynomials in u^2 (fit error
// below 3e-10, coefficients from glass_gb300/lanczos_poly.py), so the six
// weights cost 36 FMAs and no transcendental or division.  Each weight is
// within 1.3e-7 of the exact value (float32 rounding included); callers
// that need the exact weights 0, 0, 1, 0, 0, 0 of an integer coordinate
// (exact integer translations) take the source sample directly.
// pair A (c = 0.5): max fit error 7.3e-11
__device__ __forceinline__ float l3_even_a(float x) {
  float p = 1.680220594e-03f;
  p = __fmaf_rn(p, x, -9.777043946e-03f);
  p = __fmaf_rn(p, x, 2.186747268e-02f);
  p = __fmaf_rn(p, x, 6.364143640e-02f);
  p = __fmaf_rn(p, x, -4.488392770e-01f);
  return __fmaf_rn(p, x, 6.079270840e-01f);
}
__device__ __forceinline__ float l3_odd_a(float x) {
  float p = 2.676349832e-03f;
  p = __fmaf_rn(p, x, -2.544626780e-02f);
  p = __fmaf_rn(p, x, 1.599001437e-01f);
  p = __fmaf_rn(p, x, -6.481293440e-01f);
  p = __fmaf_rn(p, x, 1.468628168e+00f);
  return __fmaf_rn(p, x, -1.329050660e+00f);
}
// pair B (c = 1.5): max fit error 1.8e-10
__device__ __forceinline__ float l3_even_b(float x) {
  float p = -4.255278502e-03f;
  p = __fmaf_rn(p, x, 2.526676841e-02f);
  p = __fmaf_rn(p, x, -6.422392279e-02f);
  p = __fmaf_rn(p, x, -6.639494002e-02f);
  p = __fmaf_rn(p, x, 5.606142282e-01f);
  return __fmaf_rn(p, x, -1.350949109e-01f);
}
__device__ __forceinline__ float l3_odd_b(float x) {
  float p = -1.830645255e-03f;
  p = __fmaf_rn(p, x, 1.821853220e-02f);
  p = __fmaf_rn(p, x, -1.171571687e-01f);
  p = __fmaf_rn(p, x, 4.563217461e-01f);
  p = __fmaf_rn(p, x, -8.275418282e-01f);
  return __fmaf_rn(p, x, 1.801265478e-01f);
}
// pair C (c = 2.5): max fit error 2.1e-10
__device__ __forceinline__ float l3_even_c(float x) {
  float p = 4.921542015e-03f;
  p = __fmaf_rn(p, x, -3.034376726e-02f);
  p = __fmaf_rn(p, x, 9.083209187e-02f);
  p = __fmaf_rn(p, x, -6.445738673e-02f);
  p = __fmaf_rn(p, x, -8.637610078e-02f);
  return __fmaf_rn(p, x, 2.431708388e-02f);
}
__device__ __forceinline__ float l3_odd_c(float x) {
  float p = 5.886373110e-04f;
  p = __fmaf_rn(p, x, -7.546908688e-03f);
  p = __fmaf_rn(p, x, 5.576262996e-02f);
  p = __fmaf_rn(p, x, -2.164693773e-01f);
  p = __fmaf_rn(p, x, 3.049877286e-01f);
  return __fmaf_rn(p, x, -6.355997920e-02f);
}

__device__ __forceinline__ void lanczos3_weights(float t, float (&w)[6]) {
  const float u = __fsub_rn(t, 0.5f);
  const float x = __fmul_rn(u, u);
  const float ea = l3_even_a(x), oa = __fmul_rn(u, l3_odd_a(x));
  const float eb = l3_even_b(x), ob = __fmul_rn(u, l3_odd_b(x));
  const float ec = l3_even_c(x), oc = __fmul_rn(u, l3_odd_c(x));
  w[0] = __fadd_rn(ec, oc);
  w[1] = __fadd_rn(eb, ob);
  w[2] = __fadd_rn(ea, oa);
  w[3] = __fsub_rn(ea, oa);
  w[4] = __fsub_rn(eb, ob);
  w[5] = __fsub_rn(ec, oc);
}

// Lanczos3 weights with relative (not only absolute) accuracy, for the
// renormalised sums over the finite taps: at fractional offset t in [0, 1)
// (d = t - k): w = sinc(d) sinc(d/3) = 3 sin(pi d) sin(pi d / 3) / (pi d)^2,
// with sin(pi d) = (-1)^k sin(pi t) and sin(pi d / 3) from the angle sum, so
// one sin(pi t) and one sin/cos(pi t / 3) serve all six taps.  |d| < 1e-6
// gives 1, as the reference's sinc does.
__device__ __forceinline__ void lanczos3_weights_trig(float t, float (&w)[6]) {
  const float u = t <= 0.5f ? t : 1.0f - t;
  const float s = sin_taylor(kPiF * u);
  const float x3 = t * (kPiF / 3.0f);
  const float s3 = sin_taylor(x3), c3 = cos_taylor(x3);
  const float ck[6] = {-0.5f, 0.5f, 1.0f, 0.5f, -0.5f, -1.0f};
  const float sk[6] = {-0.86602540378443865f, -0.86602540378443865f, 0.0f, 0.86602540378443865f,
                       0.86602540378443865f, 0.0f};
  constexpr float k3_over_pi2 = 0.30396355092701331f;  // 3 / pi^2
  // Tap k = 1 (d = t - 1 in [-1, 0)) would lose its small sin(pi d / 3) to
  // cancellation in the angle sum near t = 1: evaluate it directly.
  const float s3_k1 = sin_taylor((kPiF / 3.0f) * (t - 1.0f));
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const float d = t - static_cast<float>(j - 2);
    const float s1 = ((j - 2) & 1) ? -s : s;
    const float s3d = (j == 3) ? s3_k1 : __fmaf_rn(s3, ck[j], -c3 * sk[j]);
    const float wv = k3_over_pi2 * s1 * s3d * __fdividef(1.0f, d * d);
    w[j] = fabsf(d) < 1.0e-6f ? 1.0f : wv;
  }
}

// Tap reader: shared-memory tile (origin bx, by) or global frame.
struct TapSource {
  const float* tile;  // nullptr -> global
  const float* src;
  int bx, by, width;
  __device__ __forceinline__ float at(int x, int y) const {
    return tile ? tile[(y - by) * kBoxW + (x - bx)] : __ldg(src + static_cast<int64_t>(y) * width + x);
  }
};

__device__ __forceinline__ float sample_bilinear(const TapSource& ts, int x0, int y0, float tx, float ty, int W,
                                                 int H) {
  const int x1 = min(x0 + 1, W - 1);
  const int y1 = min(y0 + 1, H - 1);
  const float v00 = ts.at(x0, y0), v01 = ts.at(x1, y0), v10 = ts.at(x0, y1), v11 = ts.at(x1, y1);
  const float ox = __fsub_rn(1.0f, tx), oy = __fsub_rn(1.0f, ty);
  const float top = __fadd_rn(__fmul_rn(v00, ox), __fmul_rn(v01, tx));
  const float bottom = __fadd_rn(__fmul_rn(v10, ox), __fmul_rn(v11, tx));
  return __fadd_rn(__fmul_rn(top, oy), __fmul_rn(bottom, ty));
}

// Non-finite taps present: skip them and renormalise.  Dropping taps can
// leave a small weight sum (lobes cancel), which amplifies rounding, so the
// sums are float-float here.  Kept out of line: it is the rare path.  Its
// arguments and result are plain values (registers): a reference argument
// would make every caller keep the tap source in local memory.
struct L3Renorm {
  float value, vmin, vmax;
  int ok;
};

static __device__ __noinline__ L3Renorm lanczos3_nonfinite(const float* tile, const float* src, int bx, int by,
                                                           int width, int x0, int y0, float tx, float ty) {
  TapSource ts;
  ts.tile = tile;
  ts.src = src;
  ts.bx = bx;
  ts.by = by;
  ts.width = width;
  // Dropped taps can leave a small sum, so the weights here carry relative
  // accuracy (the polynomial pairs are accurate to ~1e-7 absolute only).
  float wx[6], wy[6];
  lanczos3_weights_trig(tx, wx);
  lanczos3_weights_trig(ty, wy);
  FF facc, fw;
  L3Renorm r{0.0f, kInfF, -kInfF, 0};
  for (int j = 0; j < 6; ++j) {
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      const float v = ts.at(x0 - 2 + i, y0 - 2 + j);
      if (isfinite(v)) {
        const float w = wy[j] * wx[i];
        facc.add_prod(w, v);
        fw.add(w);
        r.vmin = fminf(r.vmin, v);
        r.vmax = fmaxf(r.vmax, v);
      }
    }
  }
  if (!(fabsf(__fadd_rn(fw.hi, fw.lo)) > 1.0e-12f)) return r;
  r.value = ff_div_ff(facc.hi, facc.lo, fw.hi, fw.lo);
  r.ok = 1;
  return r;
}

// Returns false when the tap weights sum to (almost) zero.  CLAMP = false
// compiles the window loops without the min/max tracking (clamp < 0);
// FINITE = 1 compiles only the all-finite branch (a frame known to hold no
// non-finite sample), 0 both, chosen by all_finite.
template <bool CLAMP, int FINITE = 0>
__device__ __forceinline__ bool sample_lanczos3_impl(const TapSource& ts, int x0, int y0, float tx, float ty,
                                                     bool all_finite, float clamp, float& out) {
  if (FINITE) all_finite = true;
  float wx[6], wy[6];
  lanczos3_weights(tx, wx);
  lanczos3_weights(ty, wy);
  float acc = 0.0f, wsum = 0.0f;
  float vmin = kInfF, vmax = -kInfF;
  if (all_finite) {
    float sx = 0.0f, sy = 0.0f;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      sx += wx[i];
      sy += wy[i];
    }
    if (ts.tile) {
      // 6x6 window at constant offsets from one shared-memory row pointer.
      const float* r0 = ts.tile + (y0 - 2 - ts.by) * kBoxW + (x0 - 2 - ts.bx);
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        float row = 0.0f;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
          const float v = r0[j * kBoxW + i];
          row = __fmaf_rn(wx[i], v, row);
          if (CLAMP) {
            vmin = fminf(vmin, v);
            vmax = fmaxf(vmax, v);
          }
        }
        acc = __fmaf_rn(wy[j], row, acc);
      }
    } else {
#pragma unroll 1
      for (int j = 0; j < 6; ++j) {
        float row = 0.0f;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
          const float v = ts.at(x0 - 2 + i, y0 - 2 + j);
          row = __fmaf_rn(wx[i], v, row);
          if (CLAMP) {
            vmin = fminf(vmin, v);
            vmax = fmaxf(vmax, v);
          }
        }
        acc = __fmaf_rn(wy[j], row, acc);
      }
    }
    wsum = sx * sy;
  } else if (!FINITE) {
    const L3Renorm r = lanczos3_nonfinite(ts.tile, ts.src, ts.bx, ts.by, ts.width, x0, y0, tx, ty);
    if (!r.ok) return false;
    acc = r.value;
    vmin = r.vmin;
    vmax = r.vmax;
    wsum = 1.0f;
  }
  if (!(fabsf(wsum) > 1.0e-12f)) return false;
  // all-finite sums lie within a few per cent of 1: the fast reciprocal is
  // within 2 ulp; renormalised partial sums take the exact division
  float value = all_finite ? __fdividef(acc, wsum) : __fdiv_rn(acc, wsum);
  if (CLAMP && vmin <= vmax) {
    const float range = vmax - vmin;
    value = fminf(vmax + clamp * range, fmaxf(vmin - clamp * range, value));
  }
  out = value;
  return true;
}

// clamp >= 0: clamp to [min - clamp * range, max + clamp * range] of the taps.
__device__ __forceinline__ bool sample_lanczos3(const TapSource& ts, int x0, int y0, float tx, float ty,
                                                bool all_finite, float clamp, float& out) {
  return clamp >= 0.0f ? sample_lanczos3_impl<true>(ts, x0, y0, tx, ty, all_finite, clamp, out)
                       : sample_lanczos3_impl<false>(ts, x0, y0, tx, ty, all_finite, clamp, out);
}

// The same for a source frame known to hold only finite samples.
__device__ __forceinline__ bool sample_lanczos3_finite(const TapSource& ts, int x0, int y0, float tx, float ty,
                                                       float clamp, float& out) {
  return clamp >= 0.0f ? sample_lanczos3_impl<true, 1>(ts, x0, y0, tx, ty, true, clamp, out)
                       : sample_lanczos3_impl<false, 1>(ts, x0, y0, tx, ty, true, clamp, out);
}

}  // namespace gg
