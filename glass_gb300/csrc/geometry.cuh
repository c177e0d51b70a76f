// Source-coordinate geometry shared by the warps and the alignment metrics.
//
// An output pixel (x, y) samples the source at M^-1 (x, y, 1) with the
// inverse evaluated in float64 by the reference (engine/warp.py:155-227).
// The device evaluates it in float-float: the float64 inverse is split into
// (hi, lo) float pairs and a*x + b*y + c is formed with TwoProd/TwoSum, so
// floor and validity decisions agree with float64 without float64 arithmetic.
#pragma once

#include <cmath>

#include "common.cuh"

namespace gg {

struct FFv {
  float hi, lo;
};

// a*x + b*y + c with (hi, lo) coefficients; x, y exact small integers.  Split
// into the part that does not depend on c (shared by transforms that differ
// only in their translation) and the rest; ff_lin is the two in sequence.
struct FFPre {
  float s, t, e;
};

__device__ __forceinline__ FFPre ff_lin_pre(float a_hi, float b_hi, float x, float y) {
  const float p1 = __fmul_rn(a_hi, x);
  const float e1 = __fmaf_rn(a_hi, x, -p1);
  const float p2 = __fmul_rn(b_hi, y);
  const float e2 = __fmaf_rn(b_hi, y, -p2);
  FFPre r;
  two_sum(p1, p2, r.s, r.t);
  r.e = __fadd_rn(e1, e2);
  return r;
}

__device__ __forceinline__ FFv ff_lin_finish(const FFPre& p, float a_lo, float b_lo, float x, float y, float c_hi,
                                             float c_lo) {
  float s2, t2;
  two_sum(p.s, c_hi, s2, t2);
  float lo = __fadd_rn(p.t, t2);
  lo = __fadd_rn(lo, p.e);
  lo = __fmaf_rn(a_lo, x, lo);
  lo = __fmaf_rn(b_lo, y, lo);
  lo = __fadd_rn(lo, c_lo);
  const float h = __fadd_rn(s2, lo);
  return {h, __fsub_rn(lo, __fsub_rn(h, s2))};
}

__device__ __forceinline__ FFv ff_lin(const float (*r)[2], float x, float y) {
  return ff_lin_finish(ff_lin_pre(r[0][0], r[1][0], x, y), r[0][1], r[1][1], x, y, r[2][0], r[2][1]);
}

__device__ __forceinline__ FFv ff_div(FFv n, FFv d) {
  const float q = __fdiv_rn(n.hi, d.hi);
  float r = __fmaf_rn(-q, d.hi, n.hi);
  r = __fadd_rn(r, n.lo);
  r = __fmaf_rn(-q, d.lo, r);
  const float ql = __fdiv_rn(r, d.hi);
  const float h = __fadd_rn(q, ql);
  return {h, __fsub_rn(ql, __fsub_rn(h, q))};
}

// v + (b_hi, b_lo), renormalised.
__device__ __forceinline__ FFv ff_add_ff(FFv v, float b_hi, float b_lo) {
  float s, e;
  two_sum(v.hi, b_hi, s, e);
  const float lo = __fadd_rn(__fadd_rn(v.lo, b_lo), e);
  const float h = __fadd_rn(s, lo);
  return {h, __fsub_rn(lo, __fsub_rn(h, s))};
}

__device__ __forceinline__ bool ff_ge(FFv v, float b) { return v.hi > b || (v.hi == b && v.lo >= 0.0f); }
__device__ __forceinline__ bool ff_le(FFv v, float b) { return v.hi < b || (v.hi == b && v.lo <= 0.0f); }
__device__ __forceinline__ bool ff_lt(FFv v, float b) { return v.hi < b || (v.hi == b && v.lo < 0.0f); }

// floor and float32(v - floor(v)) of a float-float value.
__device__ __forceinline__ void ff_floor_frac(FFv v, int& i, float& frac) {
  float f = floorf(v.hi);
  if (v.hi == f && v.lo < 0.0f) f -= 1.0f;
  i = static_cast<int>(f);
  frac = __fadd_rn(__fsub_rn(v.hi, f), v.lo);
}

// Source coordinate of output pixel (x, y) for an inverse with members
// m[9][2] (row-major (hi, lo)) and affine; returns false when the projective
// denominator vanishes (|w| <= 1e-12, engine/warp.py:178-191).
template <class C>
__device__ __forceinline__ bool source_coord(const C& it, float x, float y, FFv& sx, FFv& sy) {
  const float (*m)[2] = it.m;
  const float rx[3][2] = {{m[0][0], m[0][1]}, {m[1][0], m[1][1]}, {m[2][0], m[2][1]}};
  const float ry[3][2] = {{m[3][0], m[3][1]}, {m[4][0], m[4][1]}, {m[5][0], m[5][1]}};
  sx = ff_lin(rx, x, y);
  sy = ff_lin(ry, x, y);
  if (it.affine) return true;
  const float rw[3][2] = {{m[6][0], m[6][1]}, {m[7][0], m[7][1]}, {m[8][0], m[8][1]}};
  const FFv w = ff_lin(rw, x, y);
  if (!(fabsf(w.hi) > 1.0e-12f)) return false;
  sx = ff_div(sx, w);
  sy = ff_div(sy, w);
  return true;
}

// Bilinear sample at (x0 + tx, y0 + ty) of a row-major float32 image
// (engine/warp.py:99-119): x1 = min(x0 + 1, W - 1), float32 arithmetic.
__device__ __forceinline__ float bilinear_at(const float* img, int W, int H, int x0, int y0, float tx, float ty) {
  const int x1 = min(x0 + 1, W - 1);
  const int y1 = min(y0 + 1, H - 1);
  const float* r0 = img + static_cast<int64_t>(y0) * W;
  const float* r1 = img + static_cast<int64_t>(y1) * W;
  const float v00 = __ldg(r0 + x0), v01 = __ldg(r0 + x1), v10 = __ldg(r1 + x0), v11 = __ldg(r1 + x1);
  const float ox = __fsub_rn(1.0f, tx), oy = __fsub_rn(1.0f, ty);
  const float top = __fadd_rn(__fmul_rn(v00, ox), __fmul_rn(v01, tx));
  const float bottom = __fadd_rn(__fmul_rn(v10, ox), __fmul_rn(v11, tx));
  return __fadd_rn(__fmul_rn(top, oy), __fmul_rn(bottom, ty));
}

// ---- host -----------------------------------------------------------------------
// 3x3 inverse by cofactors in float64; false for singular or non-finite.
inline bool invert3(const double* m, double* inv) {
  const double a = m[0], b = m[1], c = m[2], d = m[3], e = m[4], f = m[5], g = m[6], h = m[7], i = m[8];
  const double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
  const double det = a * A + b * B + c * C;
  if (!(std::fabs(det) > 0.0) || !std::isfinite(det)) return false;
  const double r = 1.0 / det;
  inv[0] = A * r;
  inv[1] = -(b * i - c * h) * r;
  inv[2] = (b * f - c * e) * r;
  inv[3] = B * r;
  inv[4] = (a * i - c * g) * r;
  inv[5] = -(a * f - c * d) * r;
  inv[6] = C * r;
  inv[7] = -(a * h - b * g) * r;
  inv[8] = (a * e - b * d) * r;
  for (int k = 0; k < 9; ++k)
    if (!std::isfinite(inv[k])) return false;
  return true;
}

// Float-float coefficients (and the affine flag) of the inverse of a forward
// matrix; false when the matrix is singular.
inline bool inverse_coefficients(const double* fwd, float (*m)[2], int& affine) {
  double inv[9];
  if (!invert3(fwd, inv)) return false;
  // An affine matrix has an affine inverse; the cofactor formula leaves
  // inv[8] = det * (1 / det), which may round to 1 - 2^-53 and would send
  // every sample through the projective division for a 1e-16 relative change.
  if (fwd[6] == 0.0 && fwd[7] == 0.0 && fwd[8] == 1.0) {
    inv[6] = 0.0;
    inv[7] = 0.0;
    inv[8] = 1.0;
  }
  affine = (inv[6] == 0.0 && inv[7] == 0.0 && inv[8] == 1.0) ? 1 : 0;
  for (int q = 0; q < 9; ++q) {
    const float hi = static_cast<float>(inv[q]);
    m[q][0] = hi;
    m[q][1] = static_cast<float>(inv[q] - static_cast<double>(hi));
  }
  return true;
}

}  // namespace gg
