// Position derivatives of the bilinear and Lanczos3 samplers, shared by the
// warp adjoint (adjoint.cu) and the Gauss-Newton registration refinement
// (gnrefine.cu).  The weights and their derivatives are recomputed per
// sample, never stored.
//
// Lanczos3: w(d) = f(d) f(d/3) with f(d) = sin(pi d) / (pi d), so
// w'(d) = f'(d) f(d/3) + f(d) f'(d/3) / 3, f'(d) = pi dsinc(pi d),
// dsinc(a) = (a cos a - sin a) / a^2.  The sampled value over a window whose
// taps are all finite is O = N / D (N = sum w_i w_j S_ij, D = sum w_i w_j),
// and dO/dsx = (N_x - O D_x) / D with N_x, D_x the same sums with w_i
// replaced by w'_i (likewise for y).
#pragma once

#include <cmath>
#include <cstring>

#include "sampling.cuh"

namespace gg {

// Inverse affine map (output -> source) as float-float coefficients, in the
// layout source_coord() reads: rows 0-1 the two affine rows, row 2 (0, 0, 1).
struct AffineCoef {
  float m[9][2];
  int affine;
};

inline AffineCoef affine_coef_from(const double* theta) {
  AffineCoef c;
  std::memset(&c, 0, sizeof(c));
  for (int q = 0; q < 6; ++q) {
    const float hi = static_cast<float>(theta[q]);
    c.m[q][0] = hi;
    c.m[q][1] = static_cast<float>(theta[q] - static_cast<double>(hi));
  }
  c.m[8][0] = 1.0f;
  c.affine = 1;
  return c;
}

__device__ __forceinline__ AffineCoef affine_coef_device(const double* theta) {
  AffineCoef c;
#pragma unroll
  for (int q = 0; q < 9; ++q) c.m[q][0] = c.m[q][1] = 0.0f;
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    const float hi = __double2float_rn(theta[q]);
    c.m[q][0] = hi;
    c.m[q][1] = __double2float_rn(theta[q] - static_cast<double>(hi));
  }
  c.m[8][0] = 1.0f;
  c.affine = 1;
  return c;
}

// sin and cos of pi t for t in [0, 1) from the Taylor helpers (|pi u| <= pi/2).
__device__ __forceinline__ void sincospi01(float t, float& s, float& c) {
  const float u = t <= 0.5f ? t : 1.0f - t;
  s = sin_taylor(kPiF * u);
  const float cu = cos_taylor(kPiF * u);
  c = t <= 0.5f ? cu : -cu;
}

// d/da [sin(a) / a] = (a cos a - sin a) / a^2.  Below |a| = 1 the difference
// cancels, so the Maclaurin series sum_{n>=1} (-1)^n 2n a^(2n-1) / (2n+1)!
// (truncated after a^9; remainder < 2e-9) is used instead.
__device__ __forceinline__ float dsinc_arg(float a, float s, float c) {
  if (fabsf(a) < 1.0f) {
    const float a2 = a * a;
    float p = -1.0f / 3991680.0f;
    p = __fmaf_rn(p, a2, 1.0f / 45360.0f);
    p = __fmaf_rn(p, a2, -1.0f / 840.0f);
    p = __fmaf_rn(p, a2, 1.0f / 30.0f);
    p = __fmaf_rn(p, a2, -1.0f / 3.0f);
    return p * a;
  }
  return (c * a - s) / (a * a);
}

// Lanczos3 weights w(t - k) and derivatives w'(t - k), k = -2..3.
__device__ __forceinline__ void lanczos3_weights_grad(float t, float (&w)[6], float (&dw)[6]) {
  float s, c;
  sincospi01(t, s, c);
  const float x3 = t * (kPiF / 3.0f);
  const float s3 = sin_taylor(x3), c3 = cos_taylor(x3);
  const float ck[6] = {-0.5f, 0.5f, 1.0f, 0.5f, -0.5f, -1.0f};
  const float sk[6] = {-0.86602540378443865f, -0.86602540378443865f, 0.0f, 0.86602540378443865f,
                       0.86602540378443865f, 0.0f};
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const float d = t - static_cast<float>(j - 2);
    const bool odd = ((j - 2) & 1) != 0;
    const float s1 = odd ? -s : s, c1 = odd ? -c : c;  // sin / cos (pi d)
    // sin / cos (pi d / 3) by the angle sum with pi k / 3 (k = j - 2)
    float sd3 = __fmaf_rn(s3, ck[j], -c3 * sk[j]);
    const float cd3 = __fmaf_rn(c3, ck[j], s3 * sk[j]);
    if (j == 3) sd3 = sin_taylor((kPiF / 3.0f) * (t - 1.0f));  // small near t = 1: direct
    if (fabsf(d) < 1.0e-6f) {
      w[j] = 1.0f;
      dw[j] = 0.0f;
      continue;
    }
    // one correctly rounded reciprocal per tap serves f, g and both
    // derivative quotients (1 / a3 = 3 / a)
    const float a = kPiF * d, a3 = a * (1.0f / 3.0f);
    const float ia = __frcp_rn(a), ia3 = 3.0f * ia;
    const float f = s1 * ia, g = sd3 * ia3;
    const float fp = kPiF * (fabsf(a) < 1.0f ? dsinc_arg(a, s1, c1) : (c1 * a - s1) * ia * ia);
    const float gp = (kPiF / 3.0f) * (fabsf(a3) < 1.0f ? dsinc_arg(a3, sd3, cd3) : (cd3 * a3 - sd3) * ia3 * ia3);
    w[j] = f * g;
    dw[j] = fp * g + f * gp;
  }
}

// Lanczos3 value and its derivatives with respect to the sample position
// over a window whose 36 taps are all finite; false when a tap is not finite
// or the weights cancel (|D| <= 1e-12).
// UNROLL = true issues all 36 tap loads of the window at once (more loads in
// flight, more registers); false walks it row by row.
template <bool UNROLL = false>
__device__ __forceinline__ bool lanczos3_value_grad(const float* src, int W, int x0, int y0, float tx, float ty,
                                                    float& O, float& Ox, float& Oy) {
  float wx[6], wy[6], dwx[6], dwy[6];
  lanczos3_weights_grad(tx, wx, dwx);
  lanczos3_weights_grad(ty, wy, dwy);
  float sx = 0.0f, sy = 0.0f, dsx = 0.0f, dsy = 0.0f;
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    sx += wx[i];
    sy += wy[i];
    dsx += dwx[i];
    dsy += dwy[i];
  }
  float N = 0.0f, Nx = 0.0f, Ny = 0.0f;
  bool finite = true;
#pragma unroll(UNROLL ? 6 : 1)
  for (int j = 0; j < 6; ++j) {
    const float* row = src + static_cast<int64_t>(y0 - 2 + j) * W + (x0 - 2);
    float r = 0.0f, rx = 0.0f;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      const float v = __ldg(row + i);
      finite = finite && isfinite(v);
      r = __fmaf_rn(wx[i], v, r);
      rx = __fmaf_rn(dwx[i], v, rx);
    }
    N = __fmaf_rn(wy[j], r, N);
    Nx = __fmaf_rn(wy[j], rx, Nx);
    Ny = __fmaf_rn(dwy[j], r, Ny);
  }
  // all taps finite: D = (sum wx)(sum wy), D_x = (sum wx')(sum wy), D_y = (sum wx)(sum wy')
  const float D = sx * sy;
  if (!finite || !(fabsf(D) > 1.0e-12f)) return false;
  O = N / D;
  Ox = (Nx - O * (dsx * sy)) / D;
  Oy = (Ny - O * (sx * dsy)) / D;
  return true;
}

// Bilinear value and position derivatives (engine/warp.py:99-119 sampling);
// false when a tap is not finite.
__device__ __forceinline__ bool bilinear_value_grad(const float* src, int W, int H, int x0, int y0, float tx, float ty,
                                                    float& O, float& Ox, float& Oy) {
  const int x1 = min(x0 + 1, W - 1), y1 = min(y0 + 1, H - 1);
  const float s00 = __ldg(src + static_cast<int64_t>(y0) * W + x0);
  const float s01 = __ldg(src + static_cast<int64_t>(y0) * W + x1);
  const float s10 = __ldg(src + static_cast<int64_t>(y1) * W + x0);
  const float s11 = __ldg(src + static_cast<int64_t>(y1) * W + x1);
  if (!(isfinite(s00) && isfinite(s01) && isfinite(s10) && isfinite(s11))) return false;
  const float ox = 1.0f - tx, oy = 1.0f - ty;
  const float top = ox * s00 + tx * s01, bottom = ox * s10 + tx * s11;
  O = oy * top + ty * bottom;
  Ox = oy * (s01 - s00) + ty * (s11 - s10);
  Oy = bottom - top;
  return true;
}

}  // namespace gg
