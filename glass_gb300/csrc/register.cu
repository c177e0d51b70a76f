// Triangle-asterism registration of star catalogs on the device.
//
// Semantics follow the reference's CPU estimator, src/glass/cpu/registration.py:
//   _local_triangle_descriptors  :273-303  k nearest neighbours per anchor
//        (stable distance order), every 3-subset in combination order, first
//        occurrence of each vertex set, area >= 2, area-descending stable
//        order, first max_descriptors
//   _ordered_triangle_by_sides   :242-270  vertex order from the side lengths,
//        descriptor (longest/middle, middle/shortest)
//   estimate_triangle_asterism_transform :361-475  matches within the
//        descriptor radius sorted by distance (stable), first max_candidates,
//        two reference orientations per match, best = most pairs then
//        smallest rms (first wins), three guarded refits
//   _fit_similarity_matrix       :140-162  Procrustes fit
//   _fit_affine_matrix           :106-119  least-squares affine fit (the
//        transform_model = "affine" estimator: 3-point affine hypotheses,
//        affine refits)
//   _greedy_pairs / _score_matrix :177-215 pairs within tolerance, greedy by
//        distance, rms of the residuals
// and, in descriptor-list mode, the reference's similarity-from-descriptors
// fallback (src/glass_cuda.py:2097-2140: every reference x moving descriptor
// pair within the radius in reference-major order, float32 descriptor
// distance, no truncation, no refit).
//
// The 2x2 SVD of the Procrustes fit is replaced by its closed form: rotation
// angle atan2(C01 - C10, C00 + C11) and sum of singular values max(E, F) with
// E = |(C00 + C11, C01 - C10)|, F = |(C00 - C11, C01 + C10)|.  Matrices agree
// with the reference to rounding; pair sets and inlier counts exactly.
//
// GB300 mapping: FP64 is scarce on this part, so every all-pairs loop filters
// in cheap arithmetic first (per-component descriptor bounds, float32
// transformed coordinates) and evaluates the float64 distance only for
// survivors.  One CTA per catalog builds descriptors in shared memory, one
// CTA per frame pair selects matches, one warp per candidate transform fits
// and scores it, one warp per frame pair picks the best and refits.
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "stack.cuh"

namespace gg {

constexpr int kRegPts = kCatalogPoints;  // points per catalog row (80)
constexpr int kMaxNeighbors = 6;
constexpr int kMaxCombos = 20;  // C(6, 3)
constexpr int kMaxTri = kRegPts * kMaxCombos;
constexpr int kMaxDesc = kMaxTri;
constexpr int kMaxSel = 2048;  // max_candidates ceiling of the estimator
constexpr int kPairCap = 512;  // point pairs within tolerance per candidate
constexpr int kStackMatchCap = 65536;
constexpr int kListMatchCap = 262144;

enum RegMode { kEstimator = 0, kDescriptorList = 1 };

struct Desc {
  double d0, d1, area;
  int v[3];
  int pad;
};

struct TriCand {
  double d0, d1, area;
  int key;     // sorted vertex set, 7 bits per vertex
  int packed;  // ordered vertices (7 bits each), bit 31 = kept
};

struct RegJob {
  int ref_row;
  int mov_row;
};

struct Cand {
  double m[6];
  double rms;
  long long order;
  int count;
  int valid;
};

struct RegResult {
  double m[9];
  double rms;
  long long best_order;
  int inliers;
  int status;
  int ndesc_ref;
  int ndesc_mov;
  int matches;
  int pad;
};

struct RegArgs {
  const double* pts;  // [rows][kRegPts][2]
  const int* npts;    // [rows]
  Desc* desc;         // [rows][kMaxDesc]
  int* ndesc;         // [rows]
  const RegJob* jobs;
  double* match_dist;    // [jobs][match_cap]
  int* match_key;        // [jobs][match_cap]
  int2* sel;             // [jobs][sel_cap]  (moving, reference) descriptor indices
  long long* sel_order;  // [jobs][sel_cap]
  int* nsel;             // [jobs]
  Cand* cands;           // [jobs][2 * sel_cap]
  RegResult* out;        // [jobs]
  short2* pairs;         // [jobs][kRegPts]
  int* overflow;
  double tol;
  double radius;
  int match_cap;
  int sel_cap;
  int mode;
  int neighbors;
  int max_stars;
  int max_desc;
  int max_cand;
  int min_inliers;
  int model;  // GG_TRANSFORM_SIMILARITY or GG_TRANSFORM_AFFINE
};

// ---- float64 arithmetic rounded step by step like NumPy ---------------------
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
// sqrt(dx^2 + dy^2) as an elementwise square-and-sum (np.sum(d ** 2, axis=-1))
__device__ __forceinline__ double hyp_sum(double dx, double dy) { return sqrt(dadd(dmul(dx, dx), dmul(dy, dy))); }
// np.linalg.norm of a 2-vector: a dot product whose second term is fused
__device__ __forceinline__ double hyp_dot(double dx, double dy) { return sqrt(__fma_rn(dy, dy, dmul(dx, dx))); }
// Order-preserving bits of a non-negative double.
__device__ __forceinline__ unsigned long long dbits_of(double d) {
  return static_cast<unsigned long long>(__double_as_longlong(d));
}

// NumPy's pairwise sum of a contiguous float64 array (eight interleaved
// accumulators per block of <= 128, longer runs split at n/2 rounded down to
// a multiple of 8).
__device__ double pw_block(const double* v, int n) {
  if (n < 8) {
    double r = 0.0;
    for (int i = 0; i < n; ++i) r = dadd(r, v[i]);
    return r;
  }
  double r[8];
  for (int j = 0; j < 8; ++j) r[j] = v[j];
  int i = 8;
  for (; i < n - (n % 8); i += 8)
    for (int j = 0; j < 8; ++j) r[j] = dadd(r[j], v[i + j]);
  double res = dadd(dadd(dadd(r[0], r[1]), dadd(r[2], r[3])), dadd(dadd(r[4], r[5]), dadd(r[6], r[7])));
  for (; i < n; ++i) res = dadd(res, v[i]);
  return res;
}
__device__ double pw_sum(const double* v, int n) {
  if (n <= 128) return pw_block(v, n);
  int n2 = n / 2;
  n2 -= n2 % 8;
  return dadd(pw_block(v, n2), pw_block(v + n2, n - n2));  // n <= 160 here: both halves <= 128
}

// Similarity fit of n >= 2 point pairs (registration.py:140-162).  mx/my are
// moving coordinates, rx/ry reference; scratch holds 2n doubles.
__device__ bool fit_similarity(const double* mx, const double* my, const double* rx, const double* ry, int n,
                               double* scratch, double (&m)[6]) {
  if (n < 2) return false;
  double smx = 0.0, smy = 0.0, srx = 0.0, sry = 0.0;
  for (int i = 0; i < n; ++i) {  // np.mean(axis=0): rows added in order
    smx = dadd(smx, mx[i]);
    smy = dadd(smy, my[i]);
    srx = dadd(srx, rx[i]);
    sry = dadd(sry, ry[i]);
  }
  const double dn = static_cast<double>(n);
  const double mmx = __ddiv_rn(smx, dn), mmy = __ddiv_rn(smy, dn);
  const double mrx = __ddiv_rn(srx, dn), mry = __ddiv_rn(sry, dn);
  for (int i = 0; i < n; ++i) {
    const double cx = dsub(mx[i], mmx), cy = dsub(my[i], mmy);
    scratch[2 * i] = dmul(cx, cx);
    scratch[2 * i + 1] = dmul(cy, cy);
  }
  const double variance = pw_sum(scratch, 2 * n);
  if (!(variance > 1.0e-12)) return false;
  double c00 = 0.0, c01 = 0.0, c10 = 0.0, c11 = 0.0;
  for (int i = 0; i < n; ++i) {
    const double ax = dsub(mx[i], mmx), ay = dsub(my[i], mmy);
    const double bx = dsub(rx[i], mrx), by = dsub(ry[i], mry);
    c00 = dadd(c00, dmul(ax, bx));
    c01 = dadd(c01, dmul(ax, by));
    c10 = dadd(c10, dmul(ay, bx));
    c11 = dadd(c11, dmul(ay, by));
  }
  const double e = hyp_sum(dadd(c00, c11), dsub(c01, c10));
  const double f = hyp_sum(dsub(c00, c11), dadd(c01, c10));
  double cs = 1.0, sn = 0.0;
  if (e > 0.0) {
    cs = __ddiv_rn(dadd(c00, c11), e);
    sn = __ddiv_rn(dsub(c01, c10), e);
  }
  const double scale = __ddiv_rn(fmax(e, f), variance);
  const double l00 = dmul(scale, cs), l01 = dmul(scale, -sn), l10 = dmul(scale, sn), l11 = dmul(scale, cs);
  m[0] = l00;
  m[1] = l01;
  m[2] = dsub(mrx, dadd(dmul(mmx, l00), dmul(mmy, l01)));
  m[3] = l10;
  m[4] = l11;
  m[5] = dsub(mry, dadd(dmul(mmx, l10), dmul(mmy, l11)));
  return true;
}

// Affine fit of n >= 3 point pairs (registration.py:106-119: the least-squares
// solution of the 2n x 6 system).  The same solution from the normal
// equations about the means, which decouple the translation: with centred
// moving (a) and reference (b) coordinates,
//   [Sxx Sxy; Sxy Syy] (l00, l01) = (S(ax bx), S(ay bx)), likewise for row 1,
// solved by Cramer's rule; t = mean(b) - L mean(a).  False for fewer than 3
// pairs or a (numerically) singular system — collinear moving points, where
// the reference returns the minimum-norm solution instead; the descriptor
// filter (area >= 2 px^2) keeps those out of the 3-point fits.
struct AffineSums {
  double mmx, mmy, mrx, mry, sxx, sxy, syy, sxr, syr, sxs, sys;
};

__device__ __forceinline__ bool affine_from_sums(const AffineSums& q, double (&m)[6]) {
  const double det = dsub(dmul(q.sxx, q.syy), dmul(q.sxy, q.sxy));
  if (!(q.sxx > 0.0 && q.syy > 0.0 && det > dmul(1.0e-12, dmul(q.sxx, q.syy)))) return false;
  const double l00 = __ddiv_rn(dsub(dmul(q.sxr, q.syy), dmul(q.syr, q.sxy)), det);
  const double l01 = __ddiv_rn(dsub(dmul(q.syr, q.sxx), dmul(q.sxr, q.sxy)), det);
  const double l10 = __ddiv_rn(dsub(dmul(q.sxs, q.syy), dmul(q.sys, q.sxy)), det);
  const double l11 = __ddiv_rn(dsub(dmul(q.sys, q.sxx), dmul(q.sxs, q.sxy)), det);
  m[0] = l00;
  m[1] = l01;
  m[2] = dsub(q.mrx, dadd(dmul(l00, q.mmx), dmul(l01, q.mmy)));
  m[3] = l10;
  m[4] = l11;
  m[5] = dsub(q.mry, dadd(dmul(l10, q.mmx), dmul(l11, q.mmy)));
  return true;
}

__device__ bool fit_affine(const double* mx, const double* my, const double* rx, const double* ry, int n,
                           double (&m)[6]) {
  if (n < 3) return false;
  AffineSums q{};
  double smx = 0.0, smy = 0.0, srx = 0.0, sry = 0.0;
  for (int i = 0; i < n; ++i) {
    smx = dadd(smx, mx[i]);
    smy = dadd(smy, my[i]);
    srx = dadd(srx, rx[i]);
    sry = dadd(sry, ry[i]);
  }
  const double dn = static_cast<double>(n);
  q.mmx = __ddiv_rn(smx, dn);
  q.mmy = __ddiv_rn(smy, dn);
  q.mrx = __ddiv_rn(srx, dn);
  q.mry = __ddiv_rn(sry, dn);
  for (int i = 0; i < n; ++i) {
    const double ax = dsub(mx[i], q.mmx), ay = dsub(my[i], q.mmy);
    const double bx = dsub(rx[i], q.mrx), by = dsub(ry[i], q.mry);
    q.sxx = dadd(q.sxx, dmul(ax, ax));
    q.sxy = dadd(q.sxy, dmul(ax, ay));
    q.syy = dadd(q.syy, dmul(ay, ay));
    q.sxr = dadd(q.sxr, dmul(ax, bx));
    q.syr = dadd(q.syr, dmul(ay, bx));
    q.sxs = dadd(q.sxs, dmul(ax, by));
    q.sys = dadd(q.sys, dmul(ay, by));
  }
  return affine_from_sums(q, m);
}

// ---- point pairs of a transform (registration.py:177-215) ------------------------
// The reference catalog of a frame pair is bucketed into a uniform grid of at
// most 8 x 8 cells (at least 2 * (tol + 0.5) px wide), so a transformed
// moving star only visits the reference stars of <= 2 x 2 cells instead of
// all of them.
constexpr int kGrid = 8;

struct JobPoints {
  double mx[kRegPts], my[kRegPts], rx[kRegPts], ry[kRegPts];
  float mx32[kRegPts], my32[kRegPts], rx32[kRegPts], ry32[kRegPts];
  unsigned char cell_start[kGrid * kGrid + 1];
  unsigned char cell_pt[kRegPts];
  float gx0, gy0, ginv;
  int gnx, gny;
  float cmax;  // max |x| + |y| of the moving stars
  float rmax;  // max |x|, |y| of the reference stars
  int nm, nr;
};

struct WarpScratch {
  double tx[kRegPts], ty[kRegPts];
  float tx32[kRegPts], ty32[kRegPts];
  unsigned long long key[kPairCap];  // distance bits of the pairs within tolerance
  int idx[kPairCap];                 // (moving << 8) | reference: row-major order
  int acc[kRegPts];                  // accepted entries in greedy order
  double res[kRegPts];
  unsigned used_r[3];
  int count;
};

// Reference stars within `r` of (x, y) in grid order; calls f(j).
template <class F>
__device__ __forceinline__ void grid_visit(const JobPoints& jp, float x, float y, float r, F&& f) {
  if (!(fabsf(x) < 3.0e38f && fabsf(y) < 3.0e38f) || jp.gnx == 0) return;
  const float fx0 = (x - r - jp.gx0) * jp.ginv, fx1 = (x + r - jp.gx0) * jp.ginv;
  const float fy0 = (y - r - jp.gy0) * jp.ginv, fy1 = (y + r - jp.gy0) * jp.ginv;
  if (fx1 < 0.0f || fy1 < 0.0f || fx0 >= static_cast<float>(jp.gnx) || fy0 >= static_cast<float>(jp.gny)) return;
  const int cx0 = max(0, static_cast<int>(floorf(fmaxf(fx0, -1.0f))));
  const int cx1 = min(jp.gnx - 1, static_cast<int>(floorf(fminf(fx1, static_cast<float>(jp.gnx)))));
  const int cy0 = max(0, static_cast<int>(floorf(fmaxf(fy0, -1.0f))));
  const int cy1 = min(jp.gny - 1, static_cast<int>(floorf(fminf(fy1, static_cast<float>(jp.gny)))));
  for (int cy = cy0; cy <= cy1; ++cy)
    for (int cx = cx0; cx <= cx1; ++cx) {
      const int c = cy * kGrid + cx;
      for (int k = jp.cell_start[c]; k < jp.cell_start[c + 1]; ++k) f(static_cast<int>(jp.cell_pt[k]));
    }
}

// NumPy pairwise sum of v[0..n) (n <= 128) by lanes 0..7 of the warp: lane j
// runs accumulator j; every lane returns the sum.
__device__ double warp_pw_sum(const double* v, int n) {
  const int lane = threadIdx.x & 31;
  double r = 0.0;
  if (n >= 8 && lane < 8) {
    r = v[lane];
    for (int i = lane + 8; i < n - (n % 8); i += 8) r = dadd(r, v[i]);
  }
  double out = 0.0;
  const double r1 = __shfl_down_sync(0xffffffffu, r, 1);
  const double r2 = __shfl_down_sync(0xffffffffu, r, 2);
  const double r3 = __shfl_down_sync(0xffffffffu, r, 3);
  const double r4 = __shfl_down_sync(0xffffffffu, r, 4);
  const double r5 = __shfl_down_sync(0xffffffffu, r, 5);
  const double r6 = __shfl_down_sync(0xffffffffu, r, 6);
  const double r7 = __shfl_down_sync(0xffffffffu, r, 7);
  if (lane == 0) {
    if (n < 8) {
      for (int i = 0; i < n; ++i) out = dadd(out, v[i]);
    } else {
      out = dadd(dadd(dadd(r, r1), dadd(r2, r3)), dadd(dadd(r4, r5), dadd(r6, r7)));
      for (int i = n - (n % 8); i < n; ++i) out = dadd(out, v[i]);
    }
  }
  return __shfl_sync(0xffffffffu, out, 0);
}

// Exact scoring: every lane returns the greedy pair count and rms (+inf
// without pairs); the pairs (moving, reference) go to `pairs` when not null.
__device__ void warp_score_exact(const double (&m)[6], const JobPoints& jp, double tol, WarpScratch& w,
                                 int& npairs, double& rms, short2* pairs, int* overflow) {
  const int lane = threadIdx.x & 31;
  const int nm = jp.nm;
  for (int i = lane; i < nm; i += 32) {
    const double x = dadd(dadd(dmul(jp.mx[i], m[0]), dmul(jp.my[i], m[1])), m[2]);
    const double y = dadd(dadd(dmul(jp.mx[i], m[3]), dmul(jp.my[i], m[4])), m[5]);
    w.tx[i] = x;
    w.ty[i] = y;
    w.tx32[i] = static_cast<float>(x);
    w.ty32[i] = static_cast<float>(y);
  }
  if (lane == 0) w.count = 0;
  __syncwarp();
  // pairs within tolerance (float32 prefilter with a 0.5 px margin, then the
  // float64 distance); any order, sorted below
  const float r = static_cast<float>(tol + 0.5);
  const float pre = r * r;
  for (int i = lane; i < nm; i += 32) {
    const float x = w.tx32[i], y = w.ty32[i];
    grid_visit(jp, x, y, r, [&](int j) {
      const float fx = x - jp.rx32[j], fy = y - jp.ry32[j];
      if (fx * fx + fy * fy > pre) return;
      const double d = hyp_sum(dsub(w.tx[i], jp.rx[j]), dsub(w.ty[i], jp.ry[j]));
      if (!(d <= tol)) return;
      const int pos = atomicAdd(&w.count, 1);
      if (pos < kPairCap) {
        w.key[pos] = dbits_of(d);
        w.idx[pos] = (i << 8) | j;
      }
    });
  }
  __syncwarp();
  int L = w.count;
  if (L > kPairCap) {
    if (lane == 0) atomicExch(overflow, 1);
    L = kPairCap;
  }
  // sort by (distance, row-major index): the stable distance sort of the
  // row-major candidate list
  int mlen = 1;
  while (mlen < L) mlen <<= 1;
  for (int t = L + lane; t < mlen; t += 32) {
    w.key[t] = ~0ull;
    w.idx[t] = 0x7fffffff;
  }
  __syncwarp();
  for (int size = 2; size <= mlen; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int t = lane; t < mlen; t += 32) {
        const int u = t ^ stride;
        if (u > t) {
          const bool up = (t & size) == 0;
          const unsigned long long kt = w.key[t], ku = w.key[u];
          const int it = w.idx[t], iu = w.idx[u];
          const bool gt = kt > ku || (kt == ku && it > iu);
          if (gt == up) {
            w.key[t] = ku;
            w.key[u] = kt;
            w.idx[t] = iu;
            w.idx[u] = it;
          }
        }
      }
      __syncwarp();
    }
  }
  // greedy one-to-one pairing in distance order
  int n = 0;
  if (lane == 0) {
    unsigned used_m[3] = {0u, 0u, 0u}, used_r[3] = {0u, 0u, 0u};
    for (int a = 0; a < L; ++a) {
      const int i = w.idx[a] >> 8, j = w.idx[a] & 255;
      if ((used_m[i >> 5] >> (i & 31)) & 1u) continue;
      if ((used_r[j >> 5] >> (j & 31)) & 1u) continue;
      used_m[i >> 5] |= 1u << (i & 31);
      used_r[j >> 5] |= 1u << (j & 31);
      w.acc[n++] = a;
    }
  }
  n = __shfl_sync(0xffffffffu, n, 0);
  __syncwarp();
  for (int t = lane; t < n; t += 32) {
    const int a = w.acc[t];
    const double d = __longlong_as_double(static_cast<long long>(w.key[a]));
    w.res[t] = dmul(d, d);
    if (pairs) pairs[t] = make_short2(static_cast<short>(w.idx[a] >> 8), static_cast<short>(w.idx[a] & 255));
  }
  __syncwarp();
  const double s = warp_pw_sum(w.res, n);
  npairs = n;
  rms = n > 0 ? sqrt(__ddiv_rn(s, static_cast<double>(n))) : __longlong_as_double(0x7ff0000000000000ll);
  __syncwarp();
}

// Fast scoring for ranking: the exact pair count when no moving or reference
// star has two partners within tolerance (then greedy pairing keeps every
// pair), and the sum of squared residuals in any order.  Membership is
// decided in float32 outside a band of +-delta around the tolerance (delta
// bounds the float32 transform error) and in float64 inside it.  `conflict`
// reports that the exact scorer is needed.
__device__ void warp_score_fast(const double (&m)[6], const JobPoints& jp, double tol, WarpScratch& w, int& count,
                                double& sum_d2, bool& conflict) {
  const int lane = threadIdx.x & 31;
  const float m0 = static_cast<float>(m[0]), m1 = static_cast<float>(m[1]), m2 = static_cast<float>(m[2]);
  const float m3 = static_cast<float>(m[3]), m4 = static_cast<float>(m[4]), m5 = static_cast<float>(m[5]);
  const double lin = fmax(fmax(fabs(m[0]), fabs(m[1])), fmax(fabs(m[3]), fabs(m[4])));
  const double trn = fmax(fabs(m[2]), fabs(m[5]));
  const double eps = 5.9604644775390625e-08;  // 2^-24
  const double delta = 2.0 * (1.5 * (6.0 * eps * (lin * jp.cmax + trn) + eps * jp.rmax) + 4.0 * eps * (tol + 1.0)) +
                       1.0e-6;
  const double lo = tol - delta;
  const float lo2 = lo > 0.0 ? static_cast<float>(lo * lo) : -1.0f;
  const float hi2 = static_cast<float>((tol + delta) * (tol + delta));
  const float r = static_cast<float>(tol + delta);
  if (lane < 3) w.used_r[lane] = 0u;
  __syncwarp();
  int cnt = 0;
  double acc = 0.0;
  bool conf = false;
  for (int i = lane; i < jp.nm; i += 32) {
    const float x = __fadd_rn(__fadd_rn(__fmul_rn(m0, jp.mx32[i]), __fmul_rn(m1, jp.my32[i])), m2);
    const float y = __fadd_rn(__fadd_rn(__fmul_rn(m3, jp.mx32[i]), __fmul_rn(m4, jp.my32[i])), m5);
    int hits = 0;
    bool have64 = false;
    double x64 = 0.0, y64 = 0.0;
    grid_visit(jp, x, y, r, [&](int j) {
      const float fx = x - jp.rx32[j], fy = y - jp.ry32[j];
      const float d2 = fx * fx + fy * fy;
      if (d2 > hi2) return;
      if (!have64) {
        x64 = dadd(dadd(dmul(jp.mx[i], m[0]), dmul(jp.my[i], m[1])), m[2]);
        y64 = dadd(dadd(dmul(jp.mx[i], m[3]), dmul(jp.my[i], m[4])), m[5]);
        have64 = true;
      }
      const double ex = dsub(x64, jp.rx[j]), ey = dsub(y64, jp.ry[j]);
      const double dd2 = dadd(dmul(ex, ex), dmul(ey, ey));
      if (!(d2 <= lo2) && !(sqrt(dd2) <= tol)) return;
      ++hits;
      acc = dadd(acc, dd2);
      const unsigned bit = 1u << (j & 31);
      if (atomicOr(&w.used_r[j >> 5], bit) & bit) conf = true;
    });
    if (hits > 1) conf = true;
    cnt += hits;
  }
  for (int off = 16; off > 0; off >>= 1) {
    cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
    acc = dadd(acc, __shfl_xor_sync(0xffffffffu, acc, off));
  }
  conflict = __any_sync(0xffffffffu, conf);
  count = cnt;
  sum_d2 = acc;
  __syncwarp();
}

// Warp-cooperative similarity fit of n <= 80 pairs: the same arithmetic as
// fit_similarity with the independent sums on separate lanes.  Every lane
// returns the result.
__device__ bool warp_fit_similarity(const double* mx, const double* my, const double* rx, const double* ry, int n,
                                    double* sq, double (&m)[6]) {
  const int lane = threadIdx.x & 31;
  if (n < 2) return false;
  double s = 0.0;
  if (lane < 4) {
    const double* v = lane == 0 ? mx : (lane == 1 ? my : (lane == 2 ? rx : ry));
    for (int i = 0; i < n; ++i) s = dadd(s, v[i]);
  }
  const double dn = static_cast<double>(n);
  const double mmx = __ddiv_rn(__shfl_sync(0xffffffffu, s, 0), dn);
  const double mmy = __ddiv_rn(__shfl_sync(0xffffffffu, s, 1), dn);
  const double mrx = __ddiv_rn(__shfl_sync(0xffffffffu, s, 2), dn);
  const double mry = __ddiv_rn(__shfl_sync(0xffffffffu, s, 3), dn);
  for (int i = lane; i < n; i += 32) {
    const double cx = dsub(mx[i], mmx), cy = dsub(my[i], mmy);
    sq[2 * i] = dmul(cx, cx);
    sq[2 * i + 1] = dmul(cy, cy);
  }
  __syncwarp();
  double variance;
  if (2 * n <= 128) {
    variance = warp_pw_sum(sq, 2 * n);
  } else {
    int n2 = n;  // (2n) / 2
    n2 -= n2 % 8;
    variance = dadd(warp_pw_sum(sq, n2), warp_pw_sum(sq + n2, 2 * n - n2));
  }
  if (!(variance > 1.0e-12)) return false;
  double c = 0.0;
  if (lane < 4) {
    for (int i = 0; i < n; ++i) {
      const double a = lane < 2 ? dsub(mx[i], mmx) : dsub(my[i], mmy);
      const double b = (lane & 1) == 0 ? dsub(rx[i], mrx) : dsub(ry[i], mry);
      c = dadd(c, dmul(a, b));
    }
  }
  const double c00 = __shfl_sync(0xffffffffu, c, 0), c01 = __shfl_sync(0xffffffffu, c, 1);
  const double c10 = __shfl_sync(0xffffffffu, c, 2), c11 = __shfl_sync(0xffffffffu, c, 3);
  const double e = hyp_sum(dadd(c00, c11), dsub(c01, c10));
  const double f = hyp_sum(dsub(c00, c11), dadd(c01, c10));
  double cs = 1.0, sn = 0.0;
  if (e > 0.0) {
    cs = __ddiv_rn(dadd(c00, c11), e);
    sn = __ddiv_rn(dsub(c01, c10), e);
  }
  const double scale = __ddiv_rn(fmax(e, f), variance);
  const double l00 = dmul(scale, cs), l01 = dmul(scale, -sn), l10 = dmul(scale, sn), l11 = dmul(scale, cs);
  m[0] = l00;
  m[1] = l01;
  m[2] = dsub(mrx, dadd(dmul(mmx, l00), dmul(mmy, l01)));
  m[3] = l10;
  m[4] = l11;
  m[5] = dsub(mry, dadd(dmul(mmx, l10), dmul(mmy, l11)));
  return true;
}

// Warp-cooperative affine fit of n <= 80 pairs: fit_affine's sums, one per
// lane (each in pair order).  Every lane returns the result.
__device__ bool warp_fit_affine(const double* mx, const double* my, const double* rx, const double* ry, int n,
                                double (&m)[6]) {
  const int lane = threadIdx.x & 31;
  if (n < 3) return false;
  double s = 0.0;
  if (lane < 4) {
    const double* v = lane == 0 ? mx : (lane == 1 ? my : (lane == 2 ? rx : ry));
    for (int i = 0; i < n; ++i) s = dadd(s, v[i]);
  }
  const double dn = static_cast<double>(n);
  AffineSums q{};
  q.mmx = __ddiv_rn(__shfl_sync(0xffffffffu, s, 0), dn);
  q.mmy = __ddiv_rn(__shfl_sync(0xffffffffu, s, 1), dn);
  q.mrx = __ddiv_rn(__shfl_sync(0xffffffffu, s, 2), dn);
  q.mry = __ddiv_rn(__shfl_sync(0xffffffffu, s, 3), dn);
  double c = 0.0;
  if (lane < 7) {
    // lane: 0 ax ax, 1 ax ay, 2 ay ay, 3 ax bx, 4 ay bx, 5 ax by, 6 ay by
    for (int i = 0; i < n; ++i) {
      const double ax = dsub(mx[i], q.mmx), ay = dsub(my[i], q.mmy);
      const double u = (lane == 0 || lane == 1 || lane == 3 || lane == 5) ? ax : ay;
      const double v = lane == 0 ? ax : (lane <= 2 ? ay : (lane <= 4 ? dsub(rx[i], q.mrx) : dsub(ry[i], q.mry)));
      c = dadd(c, dmul(u, v));
    }
  }
  q.sxx = __shfl_sync(0xffffffffu, c, 0);
  q.sxy = __shfl_sync(0xffffffffu, c, 1);
  q.syy = __shfl_sync(0xffffffffu, c, 2);
  q.sxr = __shfl_sync(0xffffffffu, c, 3);
  q.syr = __shfl_sync(0xffffffffu, c, 4);
  q.sxs = __shfl_sync(0xffffffffu, c, 5);
  q.sys = __shfl_sync(0xffffffffu, c, 6);
  return affine_from_sums(q, m);
}

// ---- K1: triangle descriptors, one CTA per catalog row ----------------------------------
__device__ __forceinline__ double row_x(const RegArgs& a, int row, int i) {
  return a.pts[(static_cast<int64_t>(row) * kRegPts + i) * 2];
}
__device__ __forceinline__ double row_y(const RegArgs& a, int row, int i) {
  return a.pts[(static_cast<int64_t>(row) * kRegPts + i) * 2 + 1];
}

__global__ void __launch_bounds__(1024) reg_desc_kernel(RegArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  TriCand* tri = reinterpret_cast<TriCand*>(smem);
  __shared__ double px[kRegPts], py[kRegPts];
  __shared__ int nb[kRegPts][kMaxNeighbors];
  __shared__ int s_kept;
  const int row = blockIdx.x;
  const int n = min(a.npts[row], a.max_stars);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    px[i] = row_x(a, row, i);
    py[i] = row_y(a, row, i);
  }
  if (threadIdx.x == 0) s_kept = 0;
  __syncthreads();
  if (n < 3) {
    if (threadIdx.x == 0) a.ndesc[row] = 0;
    return;
  }
  const int k = min(n, max(3, a.neighbors));
  // k nearest points of each anchor (the anchor itself first), index order on ties
  for (int an = threadIdx.x; an < n; an += blockDim.x) {
    double bd[kMaxNeighbors];
    int bi[kMaxNeighbors];
    int cnt = 0;
    for (int j = 0; j < n; ++j) {
      const double d = hyp_sum(dsub(px[j], px[an]), dsub(py[j], py[an]));
      if (cnt == k && !(d < bd[k - 1])) continue;
      int pos = cnt < k ? cnt : k - 1;
      while (pos > 0 && bd[pos - 1] > d) {
        bd[pos] = bd[pos - 1];
        bi[pos] = bi[pos - 1];
        --pos;
      }
      bd[pos] = d;
      bi[pos] = j;
      if (cnt < k) ++cnt;
    }
    for (int q = 0; q < k; ++q) nb[an][q] = bi[q];
  }
  __syncthreads();
  int combo[kMaxCombos][3];
  int ncomb = 0;
  for (int i0 = 0; i0 < k; ++i0)
    for (int i1 = i0 + 1; i1 < k; ++i1)
      for (int i2 = i1 + 1; i2 < k; ++i2) {
        combo[ncomb][0] = i0;
        combo[ncomb][1] = i1;
        combo[ncomb][2] = i2;
        ++ncomb;
      }
  const int T = n * ncomb;
  for (int t = threadIdx.x; t < T; t += blockDim.x) {
    const int an = t / ncomb, c = t - (t / ncomb) * ncomb;
    const int r[3] = {nb[an][combo[c][0]], nb[an][combo[c][1]], nb[an][combo[c][2]]};
    int s0 = r[0], s1 = r[1], s2 = r[2];
    if (s0 > s1) { const int q = s0; s0 = s1; s1 = q; }
    if (s1 > s2) { const int q = s1; s1 = s2; s2 = q; }
    if (s0 > s1) { const int q = s0; s0 = s1; s1 = q; }
    TriCand tc;
    tc.key = (s0 << 14) | (s1 << 7) | s2;
    tc.packed = 0;
    tc.d0 = tc.d1 = 0.0;
    const double ex = dsub(px[r[1]], px[r[0]]), ey = dsub(py[r[1]], py[r[0]]);
    const double fx = dsub(px[r[2]], px[r[0]]), fy = dsub(py[r[2]], py[r[0]]);
    tc.area = dmul(fabs(dsub(dmul(ex, fy), dmul(ey, fx))), 0.5);
    if (tc.area >= 2.0) {
      const int pa[3] = {0, 1, 2}, pb[3] = {1, 2, 0};
      double side[3];
      for (int q = 0; q < 3; ++q)
        side[q] = hyp_dot(dsub(px[r[pa[q]]], px[r[pb[q]]]), dsub(py[r[pa[q]]], py[r[pb[q]]]));
      double lo = side[0], mid = side[1], hi = side[2];
      if (lo > mid) { const double q = lo; lo = mid; mid = q; }
      if (mid > hi) { const double q = mid; mid = hi; hi = q; }
      if (lo > mid) { const double q = lo; lo = mid; mid = q; }
      if (lo > 1.0e-6 && mid > 1.0e-6) {
        int iarg = 0;  // first maximum
        for (int q = 1; q < 3; ++q)
          if (side[q] > side[iarg]) iarg = q;
        int first = pa[iarg], second = pb[iarg];
        const int third = 3 - first - second;
        const double dft = hyp_dot(dsub(px[r[first]], px[r[third]]), dsub(py[r[first]], py[r[third]]));
        const double dst = hyp_dot(dsub(px[r[second]], px[r[third]]), dsub(py[r[second]], py[r[third]]));
        if (dft < dst) {
          const int q = first;
          first = second;
          second = q;
        }
        tc.packed = static_cast<int>(0x80000000u |
                                     static_cast<unsigned>(r[first] | (r[second] << 7) | (r[third] << 14)));
        tc.d0 = __ddiv_rn(hi, mid);
        tc.d1 = __ddiv_rn(mid, lo);
      }
    }
    tri[t] = tc;
  }
  __syncthreads();
  // keep the first occurrence of each vertex set (whatever its validity)
  for (int t = threadIdx.x; t < T; t += blockDim.x) {
    if (tri[t].packed >= 0) continue;
    const int key = tri[t].key;
    bool keep = true;
    for (int q = 0; q < t && keep; ++q)
      if (tri[q].key == key) keep = false;
    if (!keep) tri[t].packed &= 0x7fffffff;
  }
  __syncthreads();
  // stable area-descending rank
  for (int t = threadIdx.x; t < T; t += blockDim.x) {
    if (tri[t].packed >= 0) continue;
    const double ar = tri[t].area;
    int rank = 0;
    for (int q = 0; q < T; ++q)
      if (tri[q].packed < 0 && (tri[q].area > ar || (tri[q].area == ar && q < t))) ++rank;
    if (rank < a.max_desc) {
      Desc d;
      d.d0 = tri[t].d0;
      d.d1 = tri[t].d1;
      d.area = ar;
      const int p = tri[t].packed;
      d.v[0] = p & 127;
      d.v[1] = (p >> 7) & 127;
      d.v[2] = (p >> 14) & 127;
      d.pad = 0;
      a.desc[static_cast<int64_t>(row) * kMaxDesc + rank] = d;
    }
    atomicAdd(&s_kept, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) a.ndesc[row] = min(s_kept, a.max_desc);
}

// ---- K2: descriptor matches, one CTA per frame pair -----------------------------------
__device__ __forceinline__ unsigned long long dbits(double d) {
  return static_cast<unsigned long long>(__double_as_longlong(d));
}

struct SelEntry {
  double d;
  int key;
  int pad;
};

__global__ void __launch_bounds__(1024) reg_match_kernel(RegArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  double2* rdd = reinterpret_cast<double2*>(smem);              // [kMaxDesc]
  double2* mdd = rdd + kMaxDesc;                                // [kMaxDesc]
  SelEntry* sel = reinterpret_cast<SelEntry*>(mdd + kMaxDesc);  // [kMaxSel]
  float2* rdf = reinterpret_cast<float2*>(sel + kMaxSel);       // [kMaxDesc]
  float2* mdf = rdf + kMaxDesc;                                 // [kMaxDesc]
  __shared__ unsigned s_count;
  __shared__ int s_c, s_n;
  __shared__ unsigned s_hist[256];
  __shared__ unsigned long long s_prefix;
  __shared__ int s_rank, s_eq;
  const int j = blockIdx.x;
  const RegJob job = a.jobs[j];
  const Desc* rd = a.desc + static_cast<int64_t>(job.ref_row) * kMaxDesc;
  const Desc* md = a.desc + static_cast<int64_t>(job.mov_row) * kMaxDesc;
  const int nr = a.ndesc[job.ref_row], nm = a.ndesc[job.mov_row];
  for (int i = threadIdx.x; i < nr; i += blockDim.x) {
    rdd[i] = make_double2(rd[i].d0, rd[i].d1);
    rdf[i] = make_float2(static_cast<float>(rd[i].d0), static_cast<float>(rd[i].d1));
  }
  for (int i = threadIdx.x; i < nm; i += blockDim.x) {
    mdd[i] = make_double2(md[i].d0, md[i].d1);
    mdf[i] = make_float2(static_cast<float>(md[i].d0), static_cast<float>(md[i].d1));
  }
  double* mdist = a.match_dist + static_cast<int64_t>(j) * a.match_cap;
  int* mkey = a.match_key + static_cast<int64_t>(j) * a.match_cap;
  if (threadIdx.x == 0) s_count = 0;
  __syncthreads();
  const int total = nm * nr;
  const double radius = a.radius;
  const double bound = radius * 1.000001 + 1.0e-300;
  const float radf = static_cast<float>(radius) * 1.000001f + 1.0e-30f;
  const bool list_mode = a.mode == kDescriptorList;
  // descriptor distance of flat index q = moving * nr + reference; false when
  // the pair is outside the radius
  auto match_dist = [&](int q, double& d) -> bool {
    const int mi = q / nr, ri = q - (q / nr) * nr;
    const float2 rf = rdf[ri], mf = mdf[mi];
    if (list_mode) {
      const float e0 = __fsub_rn(rf.x, mf.x);
      const float e1 = __fsub_rn(rf.y, mf.y);
      const float df = sqrtf(__fadd_rn(__fmul_rn(e0, e0), __fmul_rn(e1, e1)));
      d = static_cast<double>(df);
      return d <= radius;
    }
    // float32 bounds per component (conversion error <= 2^-24 relative),
    // then the float64 distance
    if (fabsf(rf.x - mf.x) > radf + 3.0e-7f * (fabsf(rf.x) + fabsf(mf.x))) return false;
    if (fabsf(rf.y - mf.y) > radf + 3.0e-7f * (fabsf(rf.y) + fabsf(mf.y))) return false;
    const double2 r = rdd[ri], m = mdd[mi];
    const double e0 = dsub(r.x, m.x);
    if (fabs(e0) > bound) return false;
    const double e1 = dsub(r.y, m.y);
    if (fabs(e1) > bound) return false;
    d = hyp_sum(e0, e1);
    return d <= radius;
  };
  for (int q = threadIdx.x; q < total; q += blockDim.x) {
    double d;
    if (match_dist(q, d)) {
      const unsigned pos = atomicAdd(&s_count, 1u);
      if (pos < static_cast<unsigned>(a.match_cap)) {
        mdist[pos] = d;
        mkey[pos] = q;
      }
    }
  }
  __syncthreads();
  const int n = static_cast<int>(s_count);
  const bool stored_all = n <= a.match_cap;
  int2* out = a.sel + static_cast<int64_t>(j) * a.sel_cap;
  long long* out_order = a.sel_order + static_cast<int64_t>(j) * a.sel_cap;
  if (list_mode) {
    // every match is a candidate; order = reference-major enumeration index
    const bool fits = stored_all && n <= a.sel_cap;
    if (fits) {
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int q = mkey[i];
        const int mi = q / nr, ri = q - (q / nr) * nr;
        out[i] = make_int2(mi, ri);
        out_order[i] = static_cast<long long>(ri) * nm + mi;
      }
    }
    if (threadIdx.x == 0) {
      if (!fits) atomicExch(a.overflow, 1);
      a.nsel[j] = fits ? n : 0;
      a.out[j].matches = n;
      a.out[j].ndesc_ref = nr;
      a.out[j].ndesc_mov = nm;
    }
    return;
  }
  // block-wide count of matches satisfying pred(distance bits, flat index)
  auto block_count = [&](auto pred) -> int {
    int c = 0;
    if (stored_all) {
      for (int q = threadIdx.x; q < n; q += blockDim.x) c += pred(dbits(mdist[q]), mkey[q]) ? 1 : 0;
    } else {
      for (int q = threadIdx.x; q < total; q += blockDim.x) {
        double d;
        if (match_dist(q, d)) c += pred(dbits(d), q) ? 1 : 0;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) s_c = 0;
    __syncthreads();
    if (c) atomicAdd(&s_c, c);
    __syncthreads();
    const int r = s_c;
    __syncthreads();
    return r;
  };
  const int take = min(n, a.max_cand);
  // the take smallest (distance, index) pairs: distance threshold t, then the
  // index threshold K among the matches at exactly distance t
  unsigned long long t = dbits(radius);
  int K = total;
  if (take == 0) {
    t = 0ull;
    K = -1;  // keeps nothing: distances are never below +0
  } else if (take < n) {
    int need = 0, equal = 0;
    if (stored_all) {
      // radix select (8-bit digits, most significant first) of the
      // (take - 1)-th smallest distance among the stored matches
      unsigned long long prefix = 0ull, mask = 0ull;
      int rank = take - 1;
      for (int shift = 56; shift >= 0; shift -= 8) {
        for (int i = threadIdx.x; i < 256; i += blockDim.x) s_hist[i] = 0u;
        __syncthreads();
        for (int q = threadIdx.x; q < n; q += blockDim.x) {
          const unsigned long long k = dbits(mdist[q]);
          if ((k & mask) == prefix) atomicAdd(&s_hist[(k >> shift) & 255u], 1u);
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
          const bool here = excl <= static_cast<unsigned>(rank) && static_cast<unsigned>(rank) < incl;
          if (here) {
            unsigned r = static_cast<unsigned>(rank) - excl;
            int b = lane * 8;
            while (r >= s_hist[b]) {
              r -= s_hist[b];
              ++b;
            }
            s_prefix = prefix | (static_cast<unsigned long long>(b) << shift);
            s_rank = static_cast<int>(r);
            s_eq = static_cast<int>(s_hist[b]);
          }
        }
        __syncthreads();
        prefix = s_prefix;
        rank = s_rank;
        mask |= 0xffull << shift;
        __syncthreads();
      }
      t = prefix;
      need = rank + 1;  // entries at exactly distance t to keep
      equal = s_eq;     // entries at exactly distance t
    } else {
      unsigned long long lo = 0ull, hi = dbits(radius);
      while (lo < hi) {
        const unsigned long long mid = lo + (hi - lo) / 2;
        if (block_count([&](unsigned long long b, int) { return b <= mid; }) >= take) hi = mid;
        else lo = mid + 1;
      }
      t = lo;
      const int below = t == 0 ? 0 : block_count([&](unsigned long long b, int) { return b < t; });
      need = take - below;
      equal = block_count([&](unsigned long long b, int) { return b == t; });
    }
    if (need < equal) {  // ties at the cut: the smallest flat indices win
      int klo = 0, khi = total - 1;
      while (klo < khi) {
        const int mid = klo + (khi - klo) / 2;
        if (block_count([&](unsigned long long b, int q) { return b == t && q <= mid; }) >= need) khi = mid;
        else klo = mid + 1;
      }
      K = klo;
    }
  }
  if (threadIdx.x == 0) s_n = 0;
  __syncthreads();
  auto keep = [&](unsigned long long b, int q) { return b < t || (b == t && q <= K); };
  if (stored_all) {
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
      if (keep(dbits(mdist[q]), mkey[q])) {
        const int p = atomicAdd(&s_n, 1);
        if (p < kMaxSel) sel[p] = {mdist[q], mkey[q], 0};
      }
    }
  } else {
    for (int q = threadIdx.x; q < total; q += blockDim.x) {
      double d;
      if (match_dist(q, d) && keep(dbits(d), q)) {
        const int p = atomicAdd(&s_n, 1);
        if (p < kMaxSel) sel[p] = {d, q, 0};
      }
    }
  }
  __syncthreads();
  const int ns = min(s_n, kMaxSel);
  int m = 1;
  while (m < ns) m <<= 1;
  for (int i = ns + threadIdx.x; i < m; i += blockDim.x)
    sel[i] = {__longlong_as_double(0x7ff0000000000000ll), 0x7fffffff, 0};
  __syncthreads();
  for (int size = 2; size <= m; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const int jj = i ^ stride;
        if (jj > i) {
          const bool up = (i & size) == 0;
          const SelEntry si = sel[i], sj = sel[jj];
          const bool gt = si.d > sj.d || (si.d == sj.d && si.key > sj.key);
          if (gt == up) {
            sel[i] = sj;
            sel[jj] = si;
          }
        }
      }
      __syncthreads();
    }
  }
  for (int i = threadIdx.x; i < ns; i += blockDim.x) {
    const int q = sel[i].key;
    out[i] = make_int2(q / nr, q - (q / nr) * nr);
    out_order[i] = i;
  }
  if (threadIdx.x == 0) {
    a.nsel[j] = ns;
    a.out[j].matches = ns;
    a.out[j].ndesc_ref = nr;
    a.out[j].ndesc_mov = nm;
  }
}

// ---- K3: candidate transforms ---------------------------------------------------------
// Loads the two catalogs of a job and buckets the reference stars (block-wide;
// the caller synchronises afterwards).
__device__ void load_job_points(const RegArgs& a, const RegJob& job, JobPoints& jp, double tol) {
  const int nm = min(a.npts[job.mov_row], a.max_stars);
  const int nr = min(a.npts[job.ref_row], a.max_stars);
  for (int i = threadIdx.x; i < kRegPts; i += blockDim.x) {
    if (i < nm) {
      jp.mx[i] = row_x(a, job.mov_row, i);
      jp.my[i] = row_y(a, job.mov_row, i);
      jp.mx32[i] = static_cast<float>(jp.mx[i]);
      jp.my32[i] = static_cast<float>(jp.my[i]);
    }
    if (i < nr) {
      jp.rx[i] = row_x(a, job.ref_row, i);
      jp.ry[i] = row_y(a, job.ref_row, i);
      jp.rx32[i] = static_cast<float>(jp.rx[i]);
      jp.ry32[i] = static_cast<float>(jp.ry[i]);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    jp.nm = nm;
    jp.nr = nr;
    float cmax = 0.0f, rmax = 0.0f;
    for (int i = 0; i < nm; ++i) cmax = fmaxf(cmax, fabsf(jp.mx32[i]) + fabsf(jp.my32[i]));
    float x0 = 3.0e38f, x1 = -3.0e38f, y0 = 3.0e38f, y1 = -3.0e38f;
    for (int i = 0; i < nr; ++i) {
      x0 = fminf(x0, jp.rx32[i]);
      x1 = fmaxf(x1, jp.rx32[i]);
      y0 = fminf(y0, jp.ry32[i]);
      y1 = fmaxf(y1, jp.ry32[i]);
      rmax = fmaxf(rmax, fmaxf(fabsf(jp.rx32[i]), fabsf(jp.ry32[i])));
    }
    jp.cmax = cmax * 1.0001f + 1.0f;
    jp.rmax = rmax * 1.0001f + 1.0f;
    for (int c = 0; c <= kGrid * kGrid; ++c) jp.cell_start[c] = 0;
    if (nr == 0) {
      jp.gnx = jp.gny = 0;
      jp.gx0 = jp.gy0 = 0.0f;
      jp.ginv = 1.0f;
    } else {
      // cells at least 2 * (tol + 0.5) wide (> the widest search radius) so
      // a search touches <= 2 x 2 cells
      const float reach = static_cast<float>(2.0 * (tol + 0.5)) + 1.0f;
      const float cell = fmaxf(fmaxf(x1 - x0, y1 - y0) / static_cast<float>(kGrid), reach);
      jp.gx0 = x0;
      jp.gy0 = y0;
      if (cell < 1.0e30f) {
        jp.ginv = 1.0f / cell;
        jp.gnx = min(kGrid, static_cast<int>((x1 - x0) * jp.ginv) + 1);
        jp.gny = min(kGrid, static_cast<int>((y1 - y0) * jp.ginv) + 1);
      } else {  // one cell holding every star
        jp.ginv = 0.0f;
        jp.gnx = jp.gny = 1;
      }
      unsigned char cnt[kGrid * kGrid];
      for (int c = 0; c < kGrid * kGrid; ++c) cnt[c] = 0;
      int cellof[kRegPts];
      for (int i = 0; i < nr; ++i) {
        const int cx = min(jp.gnx - 1, max(0, static_cast<int>((jp.rx32[i] - x0) * jp.ginv)));
        const int cy = min(jp.gny - 1, max(0, static_cast<int>((jp.ry32[i] - y0) * jp.ginv)));
        cellof[i] = cy * kGrid + cx;
        ++cnt[cellof[i]];
      }
      int run = 0;
      for (int c = 0; c < kGrid * kGrid; ++c) {
        jp.cell_start[c] = static_cast<unsigned char>(run);
        run += cnt[c];
      }
      jp.cell_start[kGrid * kGrid] = static_cast<unsigned char>(run);
      for (int c = 0; c < kGrid * kGrid; ++c) cnt[c] = jp.cell_start[c];
      for (int i = 0; i < nr; ++i) jp.cell_pt[cnt[cellof[i]]++] = static_cast<unsigned char>(i);
    }
  }
}

constexpr int kScoreWarps = 4;

// Cand::valid bits: 1 = fit succeeded, 2 = count and rms are exact.
template <int MODEL>
__global__ void __launch_bounds__(32 * kScoreWarps) reg_score_kernel(RegArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  WarpScratch* ws = reinterpret_cast<WarpScratch*>(smem);
  __shared__ JobPoints jp;
  __shared__ double cm[kScoreWarps][32][6];
  __shared__ int cok[kScoreWarps][32];
  const int j = blockIdx.y;
  const RegJob job = a.jobs[j];
  load_job_points(a, job, jp, a.tol);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ncand = 2 * a.nsel[j];
  const Desc* rd = a.desc + static_cast<int64_t>(job.ref_row) * kMaxDesc;
  const Desc* md = a.desc + static_cast<int64_t>(job.mov_row) * kMaxDesc;
  const int2* sel = a.sel + static_cast<int64_t>(j) * a.sel_cap;
  const long long* order = a.sel_order + static_cast<int64_t>(j) * a.sel_cap;
  Cand* cands = a.cands + static_cast<int64_t>(j) * 2 * a.sel_cap;
  for (int base = (blockIdx.x * kScoreWarps + warp) * 32; base < ncand; base += gridDim.x * kScoreWarps * 32) {
    // one 3-point fit per lane
    const int c = base + lane;
    int ok = 0;
    if (c < ncand) {
      const int2 s = sel[c >> 1];
      const Desc dm = md[s.x], dr = rd[s.y];
      int rv0 = dr.v[0], rv1 = dr.v[1];
      if (c & 1) {  // reference triangle in the order [1, 0, 2]
        const int q = rv0;
        rv0 = rv1;
        rv1 = q;
      }
      const double tmx[3] = {jp.mx[dm.v[0]], jp.mx[dm.v[1]], jp.mx[dm.v[2]]};
      const double tmy[3] = {jp.my[dm.v[0]], jp.my[dm.v[1]], jp.my[dm.v[2]]};
      const double trx[3] = {jp.rx[rv0], jp.rx[rv1], jp.rx[dr.v[2]]};
      const double try_[3] = {jp.ry[rv0], jp.ry[rv1], jp.ry[dr.v[2]]};
      double scratch[6];
      double m[6];
      if constexpr (MODEL == GG_TRANSFORM_AFFINE)
        ok = fit_affine(tmx, tmy, trx, try_, 3, m) ? 1 : 0;
      else
        ok = fit_similarity(tmx, tmy, trx, try_, 3, scratch, m) ? 1 : 0;
      Cand& cd = cands[c];
      for (int q = 0; q < 6; ++q) {
        cm[warp][lane][q] = ok ? m[q] : 0.0;
        cd.m[q] = ok ? m[q] : 0.0;
      }
      cd.order = 2 * order[c >> 1] + (c & 1);
    }
    cok[warp][lane] = ok;
    __syncwarp();
    // score the chunk one candidate at a time with the whole warp
    const int nb = min(32, ncand - base);
    for (int t = 0; t < nb; ++t) {
      int count = 0, exact = 0;
      double rms = __longlong_as_double(0x7ff0000000000000ll);
      if (cok[warp][t]) {
        double m[6];
        for (int q = 0; q < 6; ++q) m[q] = cm[warp][t][q];
        double sum_d2;
        bool conflict;
        warp_score_fast(m, jp, a.tol, ws[warp], count, sum_d2, conflict);
        if (conflict) {
          warp_score_exact(m, jp, a.tol, ws[warp], count, rms, nullptr, a.overflow);
          exact = 1;
        } else if (count > 0) {
          rms = sqrt(__ddiv_rn(sum_d2, static_cast<double>(count)));
        }
      }
      if (lane == 0) {
        Cand& cd = cands[base + t];
        cd.count = count;
        cd.rms = rms;
        cd.valid = cok[warp][t] ? (1 | (exact << 1)) : 0;
      }
    }
    __syncwarp();
  }
}

// ---- K4: best candidate and guarded refits, one warp per frame pair --------------------
// The reference keeps the first candidate with the most pairs and, among
// those, the smallest rms.  Counts are exact for every candidate; the fast
// rms differs from the exact one by < 1e-13 relative, so every candidate that
// can win lies in the window rms <= min * (1 + 1e-12) and only those are
// re-scored exactly (usually one).
constexpr int kWindowCap = 1024;

__global__ void __launch_bounds__(32) reg_best_kernel(RegArgs a) {
  __shared__ JobPoints jp;
  __shared__ WarpScratch ws;
  __shared__ double fx[kRegPts], fy[kRegPts], gx[kRegPts], gy[kRegPts], buf[2 * kRegPts];
  __shared__ short2 prs[kRegPts], prs2[kRegPts];
  __shared__ int window[kWindowCap];
  const int j = blockIdx.x;
  const int lane = threadIdx.x;
  const RegJob job = a.jobs[j];
  load_job_points(a, job, jp, a.tol);
  __syncthreads();
  const int ncand = 2 * a.nsel[j];
  const Cand* cs = a.cands + static_cast<int64_t>(j) * 2 * a.sel_cap;
  const double inf = __longlong_as_double(0x7ff0000000000000ll);
  // most pairs
  int bn = 0;
  for (int c = lane; c < ncand; c += 32)
    if ((cs[c].valid & 1) && cs[c].count > bn) bn = cs[c].count;
  for (int off = 16; off > 0; off >>= 1) bn = max(bn, __shfl_xor_sync(0xffffffffu, bn, off));
  // smallest (fast) rms among them
  double rmin = inf;
  if (bn > 0) {
    for (int c = lane; c < ncand; c += 32)
      if ((cs[c].valid & 1) && cs[c].count == bn) rmin = fmin(rmin, cs[c].rms);
    for (int off = 16; off > 0; off >>= 1) rmin = fmin(rmin, __shfl_xor_sync(0xffffffffu, rmin, off));
  }
  const double thr = rmin + rmin * 1.0e-12;
  // window members in candidate order
  int nw = 0;
  if (bn > 0) {
    for (int base = 0; base < ncand; base += 32) {
      const int c = base + lane;
      const bool in = c < ncand && (cs[c].valid & 1) && cs[c].count == bn && cs[c].rms <= thr;
      const unsigned mask = __ballot_sync(0xffffffffu, in);
      if (in) {
        const int pos = nw + __popc(mask & ((1u << lane) - 1u));
        if (pos < kWindowCap) window[pos] = c;
      }
      nw += __popc(mask);
    }
  }
  if (nw > kWindowCap) {
    if (lane == 0) atomicExch(a.overflow, 1);
    nw = kWindowCap;
  }
  __syncwarp();
  // exact rms of the window members: smallest wins, earliest order on ties
  int bc = -1;
  double br = inf;
  long long bo = -1;
  for (int w = 0; w < nw; ++w) {
    const int c = window[w];
    double r = cs[c].rms;
    if (!(cs[c].valid & 2)) {
      double m[6];
      for (int q = 0; q < 6; ++q) m[q] = cs[c].m[q];
      int n;
      warp_score_exact(m, jp, a.tol, ws, n, r, nullptr, a.overflow);
    }
    const long long o = cs[c].order;
    if (bc < 0 || r < br || (r == br && o < bo)) {
      bc = c;
      br = r;
      bo = o;
    }
  }
  double best[6] = {1.0, 0.0, 0.0, 0.0, 1.0, 0.0};
  int best_n = 0;
  double best_rms = inf;
  if (bc >= 0) {
    for (int q = 0; q < 6; ++q) best[q] = cs[bc].m[q];
    warp_score_exact(best, jp, a.tol, ws, best_n, best_rms, prs, a.overflow);
  }
  __syncwarp();
  const int iterations = a.mode == kEstimator ? 3 : 0;
  for (int it = 0; it < iterations; ++it) {
    if (best_n < 3) break;
    for (int q = lane; q < best_n; q += 32) {
      fx[q] = jp.mx[prs[q].x];
      fy[q] = jp.my[prs[q].x];
      gx[q] = jp.rx[prs[q].y];
      gy[q] = jp.ry[prs[q].y];
    }
    __syncwarp();
    double m[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    const bool fitted = a.model == GG_TRANSFORM_AFFINE ? warp_fit_affine(fx, fy, gx, gy, best_n, m)
                                                       : warp_fit_similarity(fx, fy, gx, gy, best_n, buf, m);
    if (!fitted) break;
    int n2;
    double r2;
    warp_score_exact(m, jp, a.tol, ws, n2, r2, prs2, a.overflow);
    if (n2 > best_n || (n2 == best_n && r2 <= best_rms)) {
      for (int q = 0; q < 6; ++q) best[q] = m[q];
      for (int q = lane; q < n2; q += 32) prs[q] = prs2[q];
      best_n = n2;
      best_rms = r2;
    }
    __syncwarp();
  }
  if (lane == 0) {
    RegResult& r = a.out[j];
    for (int q = 0; q < 6; ++q) r.m[q] = best[q];
    r.m[6] = 0.0;
    r.m[7] = 0.0;
    r.m[8] = 1.0;
    r.rms = best_rms;
    r.best_order = bo;
    r.inliers = best_n;
    r.status = a.mode == kEstimator ? (best_n >= a.min_inliers ? 1 : 0) : (best_n > 0 ? 1 : 0);
  }
  for (int q = lane; q < kRegPts; q += 32)
    a.pairs[static_cast<int64_t>(j) * kRegPts + q] = q < best_n ? prs[q] : make_short2(-1, -1);
}

__global__ void reg_copy_catalogs_kernel(const double* cat_xy, const int* cat_n, const int* row_frames, int rows,
                                         double* pts, int* npts) {
  const int row = blockIdx.x;
  if (row >= rows) return;
  const int f = row_frames[row];
  for (int i = threadIdx.x; i < kRegPts * 2; i += blockDim.x)
    pts[static_cast<int64_t>(row) * kRegPts * 2 + i] = cat_xy[static_cast<int64_t>(f) * kRegPts * 2 + i];
  if (threadIdx.x == 0) npts[row] = cat_n[f];
}

// ---- host side ------------------------------------------------------------------
struct RegScratch {
  double* pts = nullptr;
  int* npts = nullptr;
  Desc* desc = nullptr;
  int* ndesc = nullptr;
  RegJob* jobs = nullptr;
  int* row_frames = nullptr;
  double* match_dist = nullptr;
  int* match_key = nullptr;
  int2* sel = nullptr;
  long long* sel_order = nullptr;
  int* nsel = nullptr;
  Cand* cands = nullptr;
  RegResult* out = nullptr;
  short2* pairs = nullptr;
  int* overflow = nullptr;
  int rows = 0;
  int jobs_cap = 0;
  int match_cap = 0;
  int sel_cap = 0;
  int device = -1;
};

static void reg_scratch_release(RegScratch& r) {
  void* ps[] = {r.pts, r.npts,      r.desc, r.ndesc, r.jobs, r.row_frames, r.match_dist, r.match_key,
                r.sel, r.sel_order, r.nsel, r.cands, r.out,  r.pairs,      r.overflow};
  for (void* p : ps)
    if (p) cudaFree(p);
  r = RegScratch{};
}

static int64_t reg_scratch_bytes(const RegScratch& r) {
  if (r.device < 0) return 0;
  const int64_t R = r.rows, J = r.jobs_cap, M = r.match_cap, S = r.sel_cap;
  return R * (16 * kRegPts + 12 + static_cast<int64_t>(sizeof(Desc)) * kMaxDesc) +
         J * (8 + 12 * M + 16 * S + 4 + 2 * static_cast<int64_t>(sizeof(Cand)) * S +
              static_cast<int64_t>(sizeof(RegResult)) + 4 * kRegPts) +
         4;
}

static void reg_scratch_ensure(RegScratch& r, int rows, int jobs, int match_cap, int sel_cap) {
  int dev = 0;
  check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  if (r.device == dev && r.rows >= rows && r.jobs_cap >= jobs && r.match_cap >= match_cap && r.sel_cap >= sel_cap)
    return;
  if (r.device == dev) {
    rows = std::max(rows, r.rows);
    jobs = std::max(jobs, r.jobs_cap);
    match_cap = std::max(match_cap, r.match_cap);
    sel_cap = std::max(sel_cap, r.sel_cap);
  }
  reg_scratch_release(r);
  const size_t R = static_cast<size_t>(rows), J = static_cast<size_t>(jobs);
  const size_t M = static_cast<size_t>(match_cap), S = static_cast<size_t>(sel_cap);
  check_cuda(cudaMalloc(&r.pts, sizeof(double) * 2 * kRegPts * R), "cudaMalloc(registration points)");
  check_cuda(cudaMalloc(&r.npts, sizeof(int) * R), "cudaMalloc(registration counts)");
  check_cuda(cudaMalloc(&r.desc, sizeof(Desc) * kMaxDesc * R), "cudaMalloc(registration descriptors)");
  check_cuda(cudaMalloc(&r.ndesc, sizeof(int) * R), "cudaMalloc(registration descriptor counts)");
  check_cuda(cudaMalloc(&r.row_frames, sizeof(int) * R), "cudaMalloc(registration rows)");
  check_cuda(cudaMalloc(&r.jobs, sizeof(RegJob) * J), "cudaMalloc(registration jobs)");
  check_cuda(cudaMalloc(&r.match_dist, sizeof(double) * M * J), "cudaMalloc(registration matches)");
  check_cuda(cudaMalloc(&r.match_key, sizeof(int) * M * J), "cudaMalloc(registration match keys)");
  check_cuda(cudaMalloc(&r.sel, sizeof(int2) * S * J), "cudaMalloc(registration selection)");
  check_cuda(cudaMalloc(&r.sel_order, sizeof(long long) * S * J), "cudaMalloc(registration order)");
  check_cuda(cudaMalloc(&r.nsel, sizeof(int) * J), "cudaMalloc(registration selection counts)");
  check_cuda(cudaMalloc(&r.cands, sizeof(Cand) * 2 * S * J), "cudaMalloc(registration candidates)");
  check_cuda(cudaMalloc(&r.out, sizeof(RegResult) * J), "cudaMalloc(registration results)");
  check_cuda(cudaMalloc(&r.pairs, sizeof(short2) * kRegPts * J), "cudaMalloc(registration pairs)");
  check_cuda(cudaMalloc(&r.overflow, sizeof(int)), "cudaMalloc(registration overflow)");
  r.rows = rows;
  r.jobs_cap = jobs;
  r.match_cap = match_cap;
  r.sel_cap = sel_cap;
  r.device = dev;
}

static void validate_reg(const gg_register_params_t& p) {
  require(p.transform_model == GG_TRANSFORM_SIMILARITY || p.transform_model == GG_TRANSFORM_AFFINE,
          "triangle asterism registration supports similarity or affine transforms");
  require(std::isfinite(p.tolerance_px) && p.tolerance_px >= 0.0, "tolerance_px must be non-negative");
  require(std::isfinite(p.descriptor_radius) && p.descriptor_radius >= 0.0, "descriptor_radius must be non-negative");
  require(p.neighbors <= kMaxNeighbors, "neighbors must be at most 6");
  require(p.max_stars >= 0 && p.max_stars <= kRegPts, "max_stars must be in [0, 80]");
  require(p.max_descriptors >= 0, "max_descriptors must be non-negative");
  require(p.max_candidates >= 0 && p.max_candidates <= kMaxSel, "max_candidates must be in [0, 2048]");
}

static RegArgs make_args(RegScratch& r, int mode, double tol, double radius) {
  RegArgs a{};
  a.pts = r.pts;
  a.npts = r.npts;
  a.desc = r.desc;
  a.ndesc = r.ndesc;
  a.jobs = r.jobs;
  a.match_dist = r.match_dist;
  a.match_key = r.match_key;
  a.sel = r.sel;
  a.sel_order = r.sel_order;
  a.nsel = r.nsel;
  a.cands = r.cands;
  a.out = r.out;
  a.pairs = r.pairs;
  a.overflow = r.overflow;
  a.tol = tol;
  a.radius = radius;
  a.match_cap = r.match_cap;
  a.sel_cap = r.sel_cap;
  a.mode = mode;
  a.max_stars = kRegPts;
  a.neighbors = 5;
  a.max_desc = kMaxDesc;
  a.max_cand = kMaxSel;
  a.min_inliers = 0;
  a.model = GG_TRANSFORM_SIMILARITY;  // the descriptor-list fallback fits similarities
  return a;
}

static void apply_params(RegArgs& a, const gg_register_params_t& p) {
  a.max_stars = p.max_stars;
  a.neighbors = p.neighbors;
  a.max_desc = std::min(p.max_descriptors, kMaxDesc);
  a.max_cand = p.max_candidates;
  a.min_inliers = p.min_inliers;
  a.model = p.transform_model;
}

static void launch_desc(const RegArgs& a, int rows, cudaStream_t stream) {
  const size_t smem = sizeof(TriCand) * kMaxTri;
  check_cuda(cudaFuncSetAttribute(reg_desc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(smem)),
             "cudaFuncSetAttribute(reg_desc)");
  note_launch();
  reg_desc_kernel<<<rows, 1024, smem, stream>>>(a);
  check_cuda(cudaGetLastError(), "reg_desc launch");
}

static void launch_match_score_best(const RegArgs& a, int njobs, int64_t max_sel, cudaStream_t stream) {
  const size_t smem = (sizeof(double2) + sizeof(float2)) * 2 * kMaxDesc + sizeof(SelEntry) * kMaxSel;
  check_cuda(cudaFuncSetAttribute(reg_match_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(smem)),
             "cudaFuncSetAttribute(reg_match)");
  note_launch();
  reg_match_kernel<<<njobs, 1024, smem, stream>>>(a);
  check_cuda(cudaGetLastError(), "reg_match launch");
  const int64_t per_job = (2 * max_sel + 32 * kScoreWarps - 1) / (32 * kScoreWarps);
  const unsigned gx = static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>(per_job, 1024)));
  const size_t score_smem = sizeof(WarpScratch) * kScoreWarps;
  auto score = a.model == GG_TRANSFORM_AFFINE ? reg_score_kernel<GG_TRANSFORM_AFFINE>
                                              : reg_score_kernel<GG_TRANSFORM_SIMILARITY>;
  check_cuda(cudaFuncSetAttribute(score, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(score_smem)),
             "cudaFuncSetAttribute(reg_score)");
  note_launch();
  score<<<dim3(gx, static_cast<unsigned>(njobs)), 32 * kScoreWarps, score_smem, stream>>>(a);
  check_cuda(cudaGetLastError(), "reg_score launch");
  note_launch();
  reg_best_kernel<<<njobs, 32, 0, stream>>>(a);
  check_cuda(cudaGetLastError(), "reg_best launch");
}

static void fill_result(const RegResult& q, gg_registration_t& o) {
  std::memcpy(o.matrix, q.m, sizeof(q.m));
  o.rms_px = std::isfinite(q.rms) ? q.rms : std::nan("");
  o.best_candidate = q.best_order;
  o.inliers = q.inliers;
  o.status = q.status;
  o.descriptors_reference = q.ndesc_ref;
  o.descriptors_moving = q.ndesc_mov;
  o.matches = q.matches;
  o.pad = 0;
}

static void copy_pairs(const RegScratch& r, int32_t* host_pairs) {
  if (!host_pairs) return;
  std::vector<short2> prs(kRegPts);
  check_cuda(cudaMemcpy(prs.data(), r.pairs, sizeof(short2) * kRegPts, cudaMemcpyDeviceToHost),
             "cudaMemcpy(registration pairs)");
  for (int i = 0; i < kRegPts; ++i) {
    host_pairs[2 * i] = prs[static_cast<size_t>(i)].x;
    host_pairs[2 * i + 1] = prs[static_cast<size_t>(i)].y;
  }
}

// Process-wide scratch for the point-list entry points (calls are serialised).
static std::mutex g_list_mu;
static RegScratch g_list_scratch;

static void require_device() {
  int devs = 0;
  if (cudaGetDeviceCount(&devs) != cudaSuccess || devs <= 0) {
    cudaGetLastError();
    fail(GG_ERR_NO_DEVICE, "no CUDA device is available");
  }
}

static void upload_points(RegScratch& r, int row, const double* xy, int n) {
  std::vector<double> pts(2 * kRegPts, 0.0);
  for (int i = 0; i < 2 * n; ++i) pts[static_cast<size_t>(i)] = xy[i];
  check_cuda(cudaMemcpy(r.pts + static_cast<size_t>(row) * 2 * kRegPts, pts.data(), sizeof(double) * pts.size(),
                        cudaMemcpyHostToDevice),
             "cudaMemcpy(points)");
  check_cuda(cudaMemcpy(r.npts + row, &n, sizeof(int), cudaMemcpyHostToDevice), "cudaMemcpy(point count)");
}

static void check_overflow(const RegScratch& r, cudaStream_t stream) {
  int overflow = 0;
  check_cuda(cudaMemcpyAsync(&overflow, r.overflow, sizeof(int), cudaMemcpyDeviceToHost, stream),
             "cudaMemcpyAsync(overflow)");
  check_cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize(registration)");
  if (overflow) fail(GG_ERR_RUNTIME, "registration buffers overflowed (too many descriptor matches or point pairs)");
}

// Pixel coordinates: finite and within +-1e15 (float32-representable with
// room for the transform error bound).
static void require_finite_points(const double* xy, int64_t n) {
  for (int64_t i = 0; i < 2 * n; ++i)
    require(std::isfinite(xy[i]) && std::fabs(xy[i]) <= 1.0e15, "star coordinates must be finite and within 1e15");
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_triangle_descriptors(const double* host_xy, int64_t n, int32_t max_stars, int32_t neighbors,
                            int32_t max_descriptors, double* host_descriptors, int32_t* host_indices,
                            double* host_areas, int64_t capacity, int64_t* count) {
  GG_API_BEGIN
  require(count != nullptr, "null count");
  require(n >= 0 && (n == 0 || host_xy != nullptr), "invalid point list");
  require(max_stars >= 0 && max_stars <= kRegPts, "max_stars must be in [0, 80]");
  require(neighbors <= kMaxNeighbors, "neighbors must be at most 6");
  require(max_descriptors >= 0, "max_descriptors must be non-negative");
  require(capacity >= 0, "capacity must be non-negative");
  const int np = static_cast<int>(std::min<int64_t>(n, max_stars));
  require_finite_points(host_xy, np);
  require_device();
  std::lock_guard<std::mutex> lock(g_list_mu);
  RegScratch& r = g_list_scratch;
  reg_scratch_ensure(r, 2, 1, kStackMatchCap, kMaxSel);
  upload_points(r, 0, host_xy, np);
  RegArgs a = make_args(r, kEstimator, 0.0, 0.0);
  a.max_stars = max_stars;
  a.neighbors = neighbors;
  a.max_desc = std::min(max_descriptors, kMaxDesc);
  launch_desc(a, 1, nullptr);
  int nd = 0;
  check_cuda(cudaMemcpy(&nd, r.ndesc, sizeof(int), cudaMemcpyDeviceToHost), "cudaMemcpy(descriptor count)");
  *count = nd;
  const bool want = host_descriptors || host_indices || host_areas;
  if (want && capacity < nd) fail(GG_ERR_OUT_OF_RANGE, "output capacity is smaller than the descriptor count");
  if (nd > 0 && want) {
    std::vector<Desc> d(static_cast<size_t>(nd));
    check_cuda(cudaMemcpy(d.data(), r.desc, sizeof(Desc) * nd, cudaMemcpyDeviceToHost), "cudaMemcpy(descriptors)");
    for (int i = 0; i < nd; ++i) {
      const Desc& q = d[static_cast<size_t>(i)];
      if (host_descriptors) {
        host_descriptors[2 * i] = q.d0;
        host_descriptors[2 * i + 1] = q.d1;
      }
      if (host_indices)
        for (int k = 0; k < 3; ++k) host_indices[3 * i + k] = q.v[k];
      if (host_areas) host_areas[i] = q.area;
    }
  }
  GG_API_END
}

int gg_register_star_lists(const double* host_ref_xy, int64_t n_ref, const double* host_mov_xy, int64_t n_mov,
                           const gg_register_params_t* params, gg_registration_t* host_out, int32_t* host_pairs) {
  GG_API_BEGIN
  require(params != nullptr && host_out != nullptr, "null argument");
  require(n_ref >= 0 && n_mov >= 0, "point counts must be non-negative");
  require((n_ref == 0 || host_ref_xy) && (n_mov == 0 || host_mov_xy), "null point list");
  validate_reg(*params);
  const int nr = static_cast<int>(std::min<int64_t>(n_ref, params->max_stars));
  const int nm = static_cast<int>(std::min<int64_t>(n_mov, params->max_stars));
  require_finite_points(host_ref_xy, nr);
  require_finite_points(host_mov_xy, nm);
  require_device();
  std::lock_guard<std::mutex> lock(g_list_mu);
  RegScratch& r = g_list_scratch;
  reg_scratch_ensure(r, 2, 1, kStackMatchCap, kMaxSel);
  upload_points(r, 0, host_ref_xy, nr);
  upload_points(r, 1, host_mov_xy, nm);
  const RegJob job{0, 1};
  check_cuda(cudaMemcpy(r.jobs, &job, sizeof(job), cudaMemcpyHostToDevice), "cudaMemcpy(job)");
  check_cuda(cudaMemset(r.overflow, 0, sizeof(int)), "cudaMemset(overflow)");
  RegArgs a = make_args(r, kEstimator, params->tolerance_px, params->descriptor_radius);
  apply_params(a, *params);
  launch_desc(a, 2, nullptr);
  launch_match_score_best(a, 1, params->max_candidates, nullptr);
  check_overflow(r, nullptr);
  RegResult res;
  check_cuda(cudaMemcpy(&res, r.out, sizeof(res), cudaMemcpyDeviceToHost), "cudaMemcpy(registration result)");
  fill_result(res, *host_out);
  if (nr < 3 || nm < 3) {
    host_out->descriptors_reference = 0;
    host_out->descriptors_moving = 0;
    host_out->matches = 0;
  }
  copy_pairs(r, host_pairs);
  GG_API_END
}

int gg_similarity_from_descriptors(const double* host_ref_xy, int64_t n_ref, const double* host_mov_xy,
                                   int64_t n_mov, const float* host_ref_desc, const int32_t* host_ref_idx,
                                   int64_t n_ref_desc, const float* host_mov_desc, const int32_t* host_mov_idx,
                                   int64_t n_mov_desc, double tolerance_px, double descriptor_radius,
                                   gg_registration_t* host_out, int32_t* host_pairs) {
  GG_API_BEGIN
  require(host_out != nullptr, "null output");
  require(std::isfinite(tolerance_px) && tolerance_px >= 0.0, "tolerance_px must be non-negative");
  require(std::isfinite(descriptor_radius) && descriptor_radius >= 0.0, "descriptor_radius must be non-negative");
  require(n_ref >= 0 && n_mov >= 0 && n_ref_desc >= 0 && n_mov_desc >= 0, "counts must be non-negative");
  if (n_ref > kRegPts || n_mov > kRegPts) fail(GG_ERR_OUT_OF_RANGE, "catalogs are limited to 80 stars");
  if (n_ref_desc > kMaxDesc || n_mov_desc > kMaxDesc)
    fail(GG_ERR_OUT_OF_RANGE, "descriptor lists are limited to 1600 rows");
  require((n_ref == 0 || host_ref_xy) && (n_mov == 0 || host_mov_xy), "null point list");
  require((n_ref_desc == 0 || (host_ref_desc && host_ref_idx)) && (n_mov_desc == 0 || (host_mov_desc && host_mov_idx)),
          "null descriptor list");
  for (int64_t i = 0; i < 3 * n_ref_desc; ++i)
    if (host_ref_idx[i] < 0 || host_ref_idx[i] >= n_ref)
      fail(GG_ERR_OUT_OF_RANGE, "reference triangle index out of range");
  for (int64_t i = 0; i < 3 * n_mov_desc; ++i)
    if (host_mov_idx[i] < 0 || host_mov_idx[i] >= n_mov) fail(GG_ERR_OUT_OF_RANGE, "moving triangle index out of range");
  require_finite_points(host_ref_xy, n_ref);
  require_finite_points(host_mov_xy, n_mov);
  require_device();
  std::lock_guard<std::mutex> lock(g_list_mu);
  RegScratch& r = g_list_scratch;
  reg_scratch_ensure(r, 2, 1, kListMatchCap, kListMatchCap);
  upload_points(r, 0, host_ref_xy, static_cast<int>(n_ref));
  upload_points(r, 1, host_mov_xy, static_cast<int>(n_mov));
  auto upload_desc = [&](int row, const float* dv, const int32_t* iv, int64_t nd) {
    std::vector<Desc> d(static_cast<size_t>(nd));
    for (int64_t i = 0; i < nd; ++i) {
      Desc& q = d[static_cast<size_t>(i)];
      q.d0 = dv[2 * i];
      q.d1 = dv[2 * i + 1];
      q.area = 0.0;
      for (int k = 0; k < 3; ++k) q.v[k] = iv[3 * i + k];
      q.pad = 0;
    }
    if (nd > 0)
      check_cuda(cudaMemcpy(r.desc + static_cast<size_t>(row) * kMaxDesc, d.data(), sizeof(Desc) * nd,
                            cudaMemcpyHostToDevice),
                 "cudaMemcpy(descriptors)");
    const int n32 = static_cast<int>(nd);
    check_cuda(cudaMemcpy(r.ndesc + row, &n32, sizeof(int), cudaMemcpyHostToDevice), "cudaMemcpy(descriptor count)");
  };
  upload_desc(0, host_ref_desc, host_ref_idx, n_ref_desc);
  upload_desc(1, host_mov_desc, host_mov_idx, n_mov_desc);
  const RegJob job{0, 1};
  check_cuda(cudaMemcpy(r.jobs, &job, sizeof(job), cudaMemcpyHostToDevice), "cudaMemcpy(job)");
  check_cuda(cudaMemset(r.overflow, 0, sizeof(int)), "cudaMemset(overflow)");
  RegArgs a = make_args(r, kDescriptorList, tolerance_px, descriptor_radius);
  const int64_t max_sel = std::max<int64_t>(1, std::min<int64_t>(n_ref_desc * n_mov_desc, kListMatchCap));
  launch_match_score_best(a, 1, max_sel, nullptr);
  check_overflow(r, nullptr);
  RegResult res;
  check_cuda(cudaMemcpy(&res, r.out, sizeof(res), cudaMemcpyDeviceToHost), "cudaMemcpy(registration result)");
  fill_result(res, *host_out);
  copy_pairs(r, host_pairs);
  GG_API_END
}

int gg_stack_register_frames(gg_stack* s, int64_t reference_index, const int64_t* indices, int64_t count,
                             const gg_register_params_t* params, gg_registration_t* host_out) {
  GG_API_BEGIN
  require(s != nullptr && indices != nullptr && params != nullptr && host_out != nullptr, "null argument");
  require(count > 0, "indices must contain at least one frame index");
  validate_reg(*params);
  stack_require_index(s, reference_index);
  for (int64_t k = 0; k < count; ++k) stack_require_index(s, indices[k]);
  if (!s->d_cat_xy) fail(GG_ERR_RUNTIME, "detect stars on the frames before registering them");
  stack_activate(s);
  if (!s->reg_scratch) {
    s->reg_scratch = new RegScratch();
    s->reg_scratch_free = [](void* q) {
      auto* r = static_cast<RegScratch*>(q);
      reg_scratch_release(*r);
      delete r;
    };
  }
  RegScratch& r = *static_cast<RegScratch*>(s->reg_scratch);
  const int64_t before = reg_scratch_bytes(r);
  const int rows = static_cast<int>(count) + 1;
  reg_scratch_ensure(r, rows, static_cast<int>(count), kStackMatchCap, kMaxSel);
  s->bytes_allocated += reg_scratch_bytes(r) - before;
  // row 0 = reference catalog, row k + 1 = moving catalog k; job k = (0, k + 1)
  std::vector<int> row_frames(static_cast<size_t>(rows));
  std::vector<RegJob> jobs(static_cast<size_t>(count));
  row_frames[0] = static_cast<int>(reference_index);
  for (int64_t k = 0; k < count; ++k) {
    row_frames[static_cast<size_t>(k + 1)] = static_cast<int>(indices[k]);
    jobs[static_cast<size_t>(k)] = RegJob{0, static_cast<int>(k + 1)};
  }
  upload_params(s->stream, r.row_frames, row_frames.data(), sizeof(int) * rows, "cudaMemcpyAsync(registration rows)");
  upload_params(s->stream, r.jobs, jobs.data(), sizeof(RegJob) * count, "cudaMemcpyAsync(registration jobs)");
  check_cuda(cudaMemsetAsync(r.overflow, 0, sizeof(int), s->stream), "cudaMemsetAsync(overflow)");
  note_launch();
  reg_copy_catalogs_kernel<<<rows, 128, 0, s->stream>>>(s->d_cat_xy, s->d_cat_n, r.row_frames, rows, r.pts, r.npts);
  check_cuda(cudaGetLastError(), "reg_copy_catalogs launch");
  RegArgs a = make_args(r, kEstimator, params->tolerance_px, params->descriptor_radius);
  apply_params(a, *params);
  launch_desc(a, rows, s->stream);
  launch_match_score_best(a, static_cast<int>(count), params->max_candidates, s->stream);
  std::vector<RegResult> res(static_cast<size_t>(count));
  check_cuda(cudaMemcpyAsync(res.data(), r.out, sizeof(RegResult) * count, cudaMemcpyDeviceToHost, s->stream),
             "cudaMemcpyAsync(registration results)");
  check_overflow(r, s->stream);  // synchronises the stack stream
  for (int64_t k = 0; k < count; ++k) fill_result(res[static_cast<size_t>(k)], host_out[k]);
  GG_API_END
}

}  // extern "C"
