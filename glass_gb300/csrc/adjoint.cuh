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

// Derivatives d/dx of the paired Lanczos3 polynomials of sampling.cuh
// (printed by glass_gb300/lanczos_poly.py --derivatives from the same
// float32 coefficients).
__device__ __forceinline__ float l3_even_a_dx(float x) {
  float p = 8.401103318e-03f;
  p = __fmaf_rn(p, x, -3.910817578e-02f);
  p = __fmaf_rn(p, x, 6.560242176e-02f);
  p = __fmaf_rn(p, x, 1.272828728e-01f);
  return __fmaf_rn(p, x, -4.488392770e-01f);
}
__device__ __forceinline__ float l3_odd_a_dx(float x) {
  float p = 1.338174939e-02f;
  p = __fmaf_rn(p, x, -1.017850712e-01f);
  p = __fmaf_rn(p, x, 4.797004461e-01f);
  p = __fmaf_rn(p, x, -1.296258688e+00f);
  return __fmaf_rn(p, x, 1.468628168e+00f);
}
__device__ __forceinline__ float l3_even_b_dx(float x) {
  float p = -2.127639204e-02f;
  p = __fmaf_rn(p, x, 1.010670736e-01f);
  p = __fmaf_rn(p, x, -1.926717758e-01f);
  p = __fmaf_rn(p, x, -1.327898800e-01f);
  return __fmaf_rn(p, x, 5.606142282e-01f);
}
__device__ __forceinline__ float l3_odd_b_dx(float x) {
  float p = -9.153226390e-03f;
  p = __fmaf_rn(p, x, 7.287412882e-02f);
  p = __fmaf_rn(p, x, -3.514715135e-01f);
  p = __fmaf_rn(p, x, 9.126434922e-01f);
  return __fmaf_rn(p, x, -8.275418282e-01f);
}
__device__ __forceinline__ float l3_even_c_dx(float x) {
  float p = 2.460771054e-02f;
  p = __fmaf_rn(p, x, -1.213750690e-01f);
  p = __fmaf_rn(p, x, 2.724962831e-01f);
  p = __fmaf_rn(p, x, -1.289147735e-01f);
  return __fmaf_rn(p, x, -8.637610078e-02f);
}
__device__ __forceinline__ float l3_odd_c_dx(float x) {
  float p = 2.943186555e-03f;
  p = __fmaf_rn(p, x, -3.018763475e-02f);
  p = __fmaf_rn(p, x, 1.672878861e-01f);
  p = __fmaf_rn(p, x, -4.329387546e-01f);
  return __fmaf_rn(p, x, 3.049877286e-01f);
}

// Lanczos3 weights and their t-derivatives from the paired polynomials the
// warp samples with: with u = t - 1/2 and x = u^2 each pair is E(u) +- O(u),
// E = P_e(x), O = u P_o(x), so dE/dt = 2u P_e'(x) and
// dO/dt = P_o(x) + 2x P_o'(x).  Absolute accuracy (about 1e-7), enough for
// sums over windows whose taps are all finite.
__device__ __forceinline__ void lanczos3_weights_grad_poly(float t, float (&w)[6], float (&dw)[6]) {
  const float u = __fsub_rn(t, 0.5f);
  const float x = __fmul_rn(u, u);
  const float u2 = __fadd_rn(u, u), x2 = __fadd_rn(x, x);
  const float ea = l3_even_a(x), pa = l3_odd_a(x), oa = __fmul_rn(u, pa);
  const float eb = l3_even_b(x), pb = l3_odd_b(x), ob = __fmul_rn(u, pb);
  const float ec = l3_even_c(x), pc = l3_odd_c(x), oc = __fmul_rn(u, pc);
  const float dea = __fmul_rn(u2, l3_even_a_dx(x)), doa = __fmaf_rn(x2, l3_odd_a_dx(x), pa);
  const float deb = __fmul_rn(u2, l3_even_b_dx(x)), dob = __fmaf_rn(x2, l3_odd_b_dx(x), pb);
  const float dec = __fmul_rn(u2, l3_even_c_dx(x)), doc = __fmaf_rn(x2, l3_odd_c_dx(x), pc);
  w[0] = __fadd_rn(ec, oc);
  w[1] = __fadd_rn(eb, ob);
  w[2] = __fadd_rn(ea, oa);
  w[3] = __fsub_rn(ea, oa);
  w[4] = __fsub_rn(eb, ob);
  w[5] = __fsub_rn(ec, oc);
  dw[0] = __fadd_rn(dec, doc);
  dw[1] = __fadd_rn(deb, dob);
  dw[2] = __fadd_rn(dea, doa);
  dw[3] = __fsub_rn(dea, doa);
  dw[4] = __fsub_rn(deb, dob);
  dw[5] = __fsub_rn(dec, doc);
}

// Lanczos3 value and its derivatives with respect to the sample position
// over a window whose 36 taps are all finite (the warp's polynomial weights
// and their exact derivatives); false when a tap is not finite or the
// weights cancel (|D| <= 1e-12).
// UNROLL = true issues all 36 tap loads of the window at once (more loads in
// flight, more registers); false walks it row by row.
template <bool UNROLL = false>
__device__ __forceinline__ bool lanczos3_value_grad(const float* src, int W, int x0, int y0, float tx, float ty,
                                                    float& O, float& Ox, float& Oy) {
  float wx[6], wy[6], dwx[6], dwy[6];
  lanczos3_weights_grad_poly(tx, wx, dwx);
  lanczos3_weights_grad_poly(ty, wy, dwy);
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
