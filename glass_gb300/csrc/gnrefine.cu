// Batched Gauss-Newton registration refinement on resident frames.
//
// For every (reference, moving) frame pair the parameters of the inverse
// affine map theta (reference pixel -> moving pixel) and a photometric match
// (alpha, beta) minimise the masked sum of squares
//     sum_p m_p (O_p(theta) - alpha a_p - beta)^2
// over the reference pixels p on a sample grid (every row_stride-th row and
// every sample_stride-th column of it; row_stride 0 means sample_stride, a
// square grid, and whole rows - sample_stride 1 - keep the loads of a warp
// contiguous on large frames), where O_p is the moving frame sampled at theta(p) (bilinear or
// Lanczos3, engine/warp.py:99-152 sampling) and a_p the reference pixel.  The
// mask m_p drops invalid samples (outside the sampler's valid range or a
// non-finite tap or reference pixel) and single-frame outliers (cosmic rays,
// hot pixels): |r_p| > clip_sigma * sigma + mask_shift_px * min(|alpha| |grad a|,
// |grad O|) is excluded, i.e. more than the noise plus what a misregistration
// of mask_shift_px pixels of the smoother of the two frames can explain, and
// so is |grad O| > 2 |alpha| |grad a| + 3 sigma: structure in the moving frame
// that the reference lacks (the Lanczos ringing around a cosmic ray has small
// residuals but large Jacobians and would bias the step).  sigma is
// 1.4826 * median |r| of the previous pass.
//
// The reference's refinement is a grid search over translations
// (registration_kernels.cu:127-233; glass_cuda.py:771-1030); this replaces
// it with a gradient method: the Jacobian of O_p with respect to theta is the
// sampler's position derivative (adjoint.cuh, the same derivative the warp
// adjoint uses) times (x, y, 1).  Everything stays on the device:
//   gn_accumulate_kernel  one pass over the samples of every job: J^T J
//                         (upper triangle of the model's columns, projected
//                         in the kernel, or all 8 for the affine model),
//                         J^T r, r^2 and the count of kept samples, float32
//                         per thread, float64 across threads and blocks
//                         (fixed order); statistics passes keep only sum r,
//                         sum r^2 and the count;
//   gn_solve_kernel       one warp per job in float64: reduce the block
//                         partials, then either update (beta, sigma) from the
//                         kept residuals (statistics passes) or solve the
//                         damped normal equations projected on the transform
//                         model by Cholesky and apply the step.
// The host uploads the start states once and reads the results once; the
// launch sequence has no host synchronisation, so it can be captured in a
// CUDA graph.  The Jacobian uses centred, scaled coordinates
// ((x - cx) / R, (y - cy) / R), R = max(W, H) / 2, so that a unit step of
// every parameter moves the image corners by about one pixel.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include "adjoint.cuh"
#include "autotune.cuh"
#include "stack.cuh"

namespace gg {

constexpr int kGnThreads = 256;
constexpr int kGnSamplesPerThread = 64;
constexpr int kGnMaxBlocksPerJob = 64;
constexpr int kGnSums = 48;  // 36 (J^T J upper) + 8 (J^T r) + sum r^2 + count, padded
constexpr int kGnUsed = 46;
// Residual scale: sigma = 1.4826 * median |r| over the valid samples (robust
// to the cosmic rays and their interpolation ringing, which an RMS of the
// kept residuals is not), from a histogram of log2 |r| with 8 bins per octave
// over [2^-10, 2^22).
constexpr int kGnBins = 256;
constexpr float kGnBinsPerOctave = 8.0f;
constexpr float kGnLog2Min = -10.0f;
// Photometric start, two coarse passes before the statistics passes:
//  1. histograms of log2 v (32 bins per octave over [2^-2, 2^22)) of the
//     sampled reference and moving values give each frame's median m and a
//     noise scale s = m - (15.87th percentile), which stars and cosmic rays
//     (both on the bright side) do not move;
//  2. alpha = median of (O - m_O) / (a - m_a) over the samples bright in both
//     frames (more than 10 s above m): star pixels, which scale with alpha;
//     a cosmic ray is bright in one frame only.  beta = m_O - alpha m_a.
// The ratio histogram has 21.3 bins per octave over [2^-6, 2^6).
constexpr int kGnVBins = 768;
constexpr float kGnVBinsPerOctave = 32.0f;
constexpr float kGnVLog2Min = -2.0f;
constexpr int kGnRBins = 256;
constexpr float kGnRBinsPerOctave = 256.0f / 12.0f;
constexpr float kGnRLog2Min = -6.0f;
constexpr double kGnNoiseQuantile = 0.15865525393145707;  // Phi(-1)
constexpr float kGnBrightSigmas = 10.0f;
constexpr int kGnHistWords = kGnBins + 2 * kGnVBins;  // per job: residual, reference, moving
// Gradient consistency: keep a sample only while |grad O| <= 2 |alpha| |grad a| + 3 sigma.
constexpr float kGnGradFactor = 2.0f;
constexpr float kGnGradSigmas = 3.0f;

__device__ __forceinline__ int ratio_bin(float q) {
  const float b = (log2f(q) - kGnRLog2Min) * kGnRBinsPerOctave;
  return b < 0.0f ? 0 : (b >= static_cast<float>(kGnRBins - 1) ? kGnRBins - 1 : static_cast<int>(b));
}

__device__ __forceinline__ int value_bin(float v) {
  if (!(v > 0.0f)) return 0;
  const float b = (log2f(v) - kGnVLog2Min) * kGnVBinsPerOctave;
  return b < 0.0f ? 0 : (b >= static_cast<float>(kGnVBins - 1) ? kGnVBins - 1 : static_cast<int>(b));
}

__device__ __forceinline__ int residual_bin(float r) {
  const float l = log2f(fabsf(r));  // -inf for 0: first bin
  const float b = (l - kGnLog2Min) * kGnBinsPerOctave;
  return b < 0.0f ? 0 : (b >= static_cast<float>(kGnBins - 1) ? kGnBins - 1 : static_cast<int>(b));
}

struct GnState {
  double theta[6];  // inverse map in pixel units
  double alpha, beta, sigma;
  double rms;       // residual RMS over the kept samples (last pass)
  double step_px;   // corner displacement of the last step
  double samples;   // kept samples (last pass)
  double med_ref, med_mov;  // photometric start: medians and brightness thresholds
  double thr_ref, thr_mov;
  int iterations;
  int status;       // 0 running, 1 converged, 2 iteration cap, -1 too few samples, -2 singular
};

struct GnArgs {
  const float* slots;
  const int* slot_of_frame;
  int64_t stride;
  const int2* jobs;  // (reference frame, moving frame)
  GnState* state;
  double* partials;  // [job][block][kGnSums]
  double* sums_out;  // [job][kGnSums] (normal-equation export) or nullptr
  unsigned* hist;    // [job][kGnHistWords] residual magnitude and value histograms, zeroed by the solve
  int width, height;
  int sample_stride, row_stride, nsx, nsy;
  int blocks_per_job;
  int phase;  // 1, 2: the photometric-start passes (value, ratio histograms)
  float clip_sigma, shift_px;
  float cx, cy, inv_r;
};

// Accumulators of one pass.  K = 0: statistics pass (sum r, sum r^2, count);
// K = 4 / 6: the translation / similarity Jacobian columns, projected in the
// kernel (x shift, y shift[, scale, rotation], alpha, beta); K = 8: all eight
// columns (affine model, normal-equation export).  Slots of the 48 sums: the
// packed upper triangle of J^T J at [0, K(K+1)/2), J^T r at [36, 36 + K),
// sum r^2 at 44, the count at 45; the statistics pass keeps J_beta^T r =
// -sum r at 43.
template <int K>
struct GnLayout {
  static constexpr int kTri = K * (K + 1) / 2;
  static constexpr int kAcc = K == 0 ? 3 : kTri + K + 2;
  __host__ __device__ static constexpr int slot(int q) {
    return K == 0 ? 43 + q : (q < kTri ? q : (q < kTri + K ? 36 + (q - kTri) : 44 + (q - kTri - K)));
  }
};

// One reference-frame sample of a pass: its residual goes into the
// histogram, and unless the mask drops it, into the pass's accumulators.
template <int INTERP, int K, bool UNROLL>
__device__ __forceinline__ void gn_sample(const GnArgs& a, const AffineCoef& coef, const float* ref, const float* mov,
                                          int x, int y, float alpha, float beta, float clip, float sigma,
                                          unsigned* s_hist, unsigned* s_vhist, const float* s_start,
                                          float (&acc)[GnLayout<K>::kAcc]) {
  const int W = a.width, H = a.height;
  const float fW = static_cast<float>(W), fH = static_cast<float>(H);
  const float* rp = ref + static_cast<int64_t>(y) * W + x;
  const float av = __ldg(rp);
  if (!isfinite(av)) return;
  FFv sx, sy;
  source_coord(coef, static_cast<float>(x), static_cast<float>(y), sx, sy);
  const bool inside = INTERP == GG_INTERP_BILINEAR
                          ? (ff_ge(sx, 0.0f) && ff_le(sx, fW - 1.0f) && ff_ge(sy, 0.0f) && ff_le(sy, fH - 1.0f))
                          : (ff_ge(sx, 2.0f) && ff_lt(sx, fW - 3.0f) && ff_ge(sy, 2.0f) && ff_lt(sy, fH - 3.0f));
  if (!inside) return;
  int x0, y0;
  float tx, ty;
  ff_floor_frac(sx, x0, tx);
  ff_floor_frac(sy, y0, ty);
  float O, Ox, Oy;
  bool ok;
  if constexpr (INTERP == GG_INTERP_BILINEAR)
    ok = bilinear_value_grad(mov, W, H, x0, y0, tx, ty, O, Ox, Oy);
  else
    ok = lanczos3_value_grad<UNROLL>(mov, W, x0, y0, tx, ty, O, Ox, Oy);
  if (!ok) return;
  if constexpr (K == 0) {
    if (a.phase == 1) {
      atomicAdd(&s_vhist[value_bin(av)], 1u);
      atomicAdd(&s_vhist[kGnVBins + value_bin(O)], 1u);
    } else if (a.phase == 2) {
      const float da = av - s_start[0], dm = O - s_start[1];
      if (da > s_start[2] && dm > s_start[3]) atomicAdd(&s_vhist[ratio_bin(dm / da)], 1u);
    }
  }
  const float r = O - alpha * av - beta;
  atomicAdd(&s_hist[residual_bin(r)], 1u);
  float ga = 0.0f;
  if (x > 0 && x < W - 1 && y > 0 && y < H - 1) {
    ga = 0.5f * fmaxf(fabsf(__ldg(rp + 1) - __ldg(rp - 1)), fabsf(__ldg(rp + W) - __ldg(rp - W)));
    if (!isfinite(ga)) ga = 0.0f;
  }
  const float gb = fmaxf(fabsf(Ox), fabsf(Oy));
  const float allow = clip + a.shift_px * fminf(fabsf(alpha) * ga, gb);
  if (!(fabsf(r) <= allow)) return;
  // structure the reference lacks (a cosmic ray's interpolation ringing:
  // small residual, large Jacobian) fails the gradient-consistency test
  if (!(gb <= kGnGradFactor * fabsf(alpha) * ga + kGnGradSigmas * sigma)) return;
  if constexpr (K == 0) {
    acc[0] = __fmaf_rn(-1.0f, r, acc[0]);
    acc[1] = __fmaf_rn(r, r, acc[1]);
    acc[2] += 1.0f;
  } else {
    const float xt = (static_cast<float>(x) - a.cx) * a.inv_r, yt = (static_cast<float>(y) - a.cy) * a.inv_r;
    float J[K];
    if constexpr (K == 8) {
      J[0] = Ox * xt, J[1] = Ox * yt, J[2] = Ox, J[3] = Oy * xt, J[4] = Oy * yt, J[5] = Oy;
    } else if constexpr (K == 6) {
      J[0] = Ox, J[1] = Oy;
      J[2] = __fmaf_rn(Oy, yt, Ox * xt);   // scale: columns 0 + 4
      J[3] = __fmaf_rn(Oy, xt, -Ox * yt);  // rotation: columns 3 - 1
    } else {
      J[0] = Ox, J[1] = Oy;
    }
    J[K - 2] = -av;
    J[K - 1] = -1.0f;
    int q = 0;
#pragma unroll
    for (int i = 0; i < K; ++i)
#pragma unroll
      for (int j = i; j < K; ++j) {
        acc[q] = __fmaf_rn(J[i], J[j], acc[q]);
        ++q;
      }
#pragma unroll
    for (int i = 0; i < K; ++i) acc[GnLayout<K>::kTri + i] = __fmaf_rn(J[i], r, acc[GnLayout<K>::kTri + i]);
    acc[GnLayout<K>::kTri + K] = __fmaf_rn(r, r, acc[GnLayout<K>::kTri + K]);
    acc[GnLayout<K>::kTri + K + 1] += 1.0f;
  }
}

// Three CTAs per SM for the statistics and projected passes (at most a few
// bytes of spills); the 46 accumulators of the full pass keep the compiler's
// register count.
template <int INTERP, int K, bool UNROLL>
__global__ void __launch_bounds__(kGnThreads, K == 8 ? 1 : 3) gn_accumulate_kernel(GnArgs a) {
  using L = GnLayout<K>;
  __shared__ AffineCoef s_coef;
  __shared__ float s_phot[3];
  __shared__ float s_start[4];
  __shared__ int s_run;
  __shared__ double s_red[kGnThreads / 32][L::kAcc];
  __shared__ unsigned s_hist[kGnBins];
  __shared__ unsigned s_vhist[K == 0 ? 2 * kGnVBins : 1];
  const int job = blockIdx.y;
  for (int b = threadIdx.x; b < kGnBins; b += blockDim.x) s_hist[b] = 0u;
  if constexpr (K == 0)
    for (int b = threadIdx.x; b < 2 * kGnVBins; b += blockDim.x) s_vhist[b] = 0u;
  if (threadIdx.x == 0) {
    const GnState& st = a.state[job];
    s_run = st.status == 0;
    s_coef = affine_coef_device(st.theta);
    s_phot[0] = static_cast<float>(st.alpha);
    s_phot[1] = static_cast<float>(st.beta);
    s_phot[2] = static_cast<float>(st.sigma);
    s_start[0] = static_cast<float>(st.med_ref);
    s_start[1] = static_cast<float>(st.med_mov);
    s_start[2] = static_cast<float>(st.thr_ref);
    s_start[3] = static_cast<float>(st.thr_mov);
  }
  __syncthreads();
  if (!s_run) return;
  const int2 jb = a.jobs[job];
  const float* ref = a.slots + static_cast<int64_t>(a.slot_of_frame[jb.x]) * a.stride;
  const float* mov = a.slots + static_cast<int64_t>(a.slot_of_frame[jb.y]) * a.stride;
  const float alpha = s_phot[0], beta = s_phot[1], sigma = s_phot[2];
  const float clip = a.clip_sigma * sigma;  // +inf in the first statistics pass
  float acc[L::kAcc];
#pragma unroll
  for (int q = 0; q < L::kAcc; ++q) acc[q] = 0.0f;
  const int64_t items = static_cast<int64_t>(a.nsx) * a.nsy;
  for (int64_t it = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; it < items;
       it += static_cast<int64_t>(a.blocks_per_job) * blockDim.x) {
    const int iy = static_cast<int>(it / a.nsx), ix = static_cast<int>(it - static_cast<int64_t>(iy) * a.nsx);
    gn_sample<INTERP, K, UNROLL>(a, s_coef, ref, mov, ix * a.sample_stride, iy * a.row_stride, alpha, beta,
                                 clip, sigma, s_hist, s_vhist, s_start, acc);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < L::kAcc; ++q) {
    double d = static_cast<double>(acc[q]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) d += __shfl_xor_sync(0xffffffffu, d, off);
    if (lane == 0) s_red[warp][q] = d;
  }
  __syncthreads();
  if (threadIdx.x < L::kAcc) {
    double t = 0.0;
#pragma unroll
    for (int w = 0; w < kGnThreads / 32; ++w) t += s_red[w][threadIdx.x];
    a.partials[(static_cast<int64_t>(job) * a.blocks_per_job + blockIdx.x) * kGnSums + L::slot(threadIdx.x)] = t;
  }
  for (int b = threadIdx.x; b < kGnBins; b += blockDim.x)
    if (s_hist[b]) atomicAdd(&a.hist[static_cast<int64_t>(job) * kGnHistWords + b], s_hist[b]);
  if constexpr (K == 0) {
    if (a.phase != 0)
      for (int b = threadIdx.x; b < 2 * kGnVBins; b += blockDim.x)
        if (s_vhist[b]) atomicAdd(&a.hist[static_cast<int64_t>(job) * kGnHistWords + kGnBins + b], s_vhist[b]);
  }
}

// Quantile q of a log2 value histogram (log-linear inside the bin).
__device__ double histogram_quantile(const unsigned* h, int bins, double q, double log2min, double per_octave) {
  unsigned long long total = 0;
  for (int b = 0; b < bins; ++b) total += h[b];
  if (total == 0) return 0.0;
  const double want = q * static_cast<double>(total);
  double cum = 0.0;
  for (int b = 0; b < bins; ++b) {
    const double c = static_cast<double>(h[b]);
    if (cum + c >= want && c > 0.0) return exp2(log2min + (b + (want - cum) / c) / per_octave);
    cum += c;
  }
  return exp2(log2min + bins / per_octave);
}

// 1.4826 * median |r| from the job's histogram (log-linear inside the bin).
__device__ double histogram_sigma(const unsigned* h) {
  unsigned long long total = 0;
  for (int b = 0; b < kGnBins; ++b) total += h[b];
  if (total == 0) return 0.0;
  const double half = 0.5 * static_cast<double>(total);
  double cum = 0.0;
  for (int b = 0; b < kGnBins; ++b) {
    const double c = static_cast<double>(h[b]);
    if (cum + c >= half && c > 0.0) {
      const double f = (half - cum) / c;
      const double l = kGnLog2Min + (b + f) / kGnBinsPerOctave;
      return 1.4826 * exp2(l);
    }
    cum += c;
  }
  return 1.4826 * exp2(kGnLog2Min + kGnBins / kGnBinsPerOctave);
}

// Columns of the model projection P (8 x k): the parameters the solve
// updates, as combinations of the 8 Jacobian columns
// (t0', t1', t2', t3', t4', t5', alpha, beta) in centred units.
__device__ __forceinline__ int model_columns(int model, float (&P)[8][8]) {
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) P[i][j] = 0.0f;
  if (model == GG_TRANSFORM_AFFINE) {
#pragma unroll
    for (int i = 0; i < 8; ++i) P[i][i] = 1.0f;
    return 8;
  }
  int k = 0;
  P[2][k++] = 1.0f;  // x shift
  P[5][k++] = 1.0f;  // y shift
  if (model == GG_TRANSFORM_SIMILARITY) {
    P[0][k] = 1.0f;  // scale
    P[4][k++] = 1.0f;
    P[1][k] = -1.0f;  // rotation
    P[3][k++] = 1.0f;
  }
  P[6][k++] = 1.0f;  // alpha
  P[7][k++] = 1.0f;  // beta
  return k;
}

// mode 0: statistics pass (beta, sigma); 1: Gauss-Newton step; 2: export sums;
// 3, 4: photometric start (medians and thresholds; alpha, beta).
__global__ void gn_solve_kernel(GnArgs a, int mode, int model, double min_samples, double tol_px, double max_step_px,
                                int last) {
  __shared__ double s[kGnSums];
  const int job = blockIdx.x, lane = threadIdx.x;
  GnState& st = a.state[job];
  if (mode != 2 && st.status != 0) return;
  for (int q = lane; q < kGnUsed; q += 32) {
    double t = 0.0;
    for (int b = 0; b < a.blocks_per_job; ++b)
      t += a.partials[(static_cast<int64_t>(job) * a.blocks_per_job + b) * kGnSums + q];
    s[q] = t;
  }
  __syncwarp();
  unsigned* hist = a.hist + static_cast<int64_t>(job) * kGnHistWords;
  double robust_sigma = 0.0;
  if (lane == 0) robust_sigma = histogram_sigma(hist);
  __syncwarp();
  for (int b = lane; b < kGnBins; b += 32) hist[b] = 0u;  // ready for the next pass
  if (mode == 3 || mode == 4) {  // photometric start
    unsigned* vh = hist + kGnBins;
    if (lane == 0 && mode == 3) {
      const double ma = histogram_quantile(vh, kGnVBins, 0.5, kGnVLog2Min, kGnVBinsPerOctave);
      const double la = histogram_quantile(vh, kGnVBins, kGnNoiseQuantile, kGnVLog2Min, kGnVBinsPerOctave);
      const double mo = histogram_quantile(vh + kGnVBins, kGnVBins, 0.5, kGnVLog2Min, kGnVBinsPerOctave);
      const double lo = histogram_quantile(vh + kGnVBins, kGnVBins, kGnNoiseQuantile, kGnVLog2Min, kGnVBinsPerOctave);
      st.med_ref = ma;
      st.med_mov = mo;
      // +inf (no ratio samples, alpha stays) when a frame has no spread
      st.thr_ref = ma > la ? kGnBrightSigmas * (ma - la) : HUGE_VAL;
      st.thr_mov = mo > lo ? kGnBrightSigmas * (mo - lo) : HUGE_VAL;
    } else if (lane == 0) {
      unsigned long long n = 0;
      for (int b = 0; b < kGnRBins; ++b) n += vh[b];
      if (n >= 16) {
        const double alpha = histogram_quantile(vh, kGnRBins, 0.5, kGnRLog2Min, kGnRBinsPerOctave);
        st.alpha = alpha;
        st.beta = st.med_mov - alpha * st.med_ref;
      }
    }
    __syncwarp();
    for (int b = lane; b < 2 * kGnVBins; b += 32) vh[b] = 0u;
    return;
  }
  if (lane != 0) return;
  if (mode == 2) {
    for (int q = 0; q < kGnSums; ++q) a.sums_out[static_cast<int64_t>(job) * kGnSums + q] = q < kGnUsed ? s[q] : 0.0;
    return;
  }
  const double n = s[45], srr = s[44];
  st.samples = n;
  if (!(n >= min_samples)) {
    st.status = -1;
    return;
  }
  st.rms = sqrt(srr / n);
  if (mode == 0) {
    const double mean = -s[43] / n;  // J_beta = -1
    st.beta += mean;
    st.sigma = robust_sigma + 1.0e-12;
    return;
  }
  // unpack J^T J and J^T r: already projected on the model's k columns by
  // the pass (translation, similarity), or all 8 columns (affine: P = I)
  float P[8][8];
  const int k = model_columns(model, P);
  const int kc = model == GG_TRANSFORM_AFFINE ? 8 : k;
  double H[8][8], g[8];
  int q = 0;
  for (int i = 0; i < kc; ++i)
    for (int j = i; j < kc; ++j) {
      H[i][j] = s[q];
      H[j][i] = s[q];
      ++q;
    }
  for (int i = 0; i < kc; ++i) g[i] = s[36 + i];
  double A[8][8], b[8];
  for (int i = 0; i < k; ++i) {
    b[i] = -g[i];
    for (int j = 0; j < k; ++j) A[i][j] = H[i][j];
  }
  // damped Cholesky solve (A + 1e-10 diag(A)) d = b
  for (int i = 0; i < k; ++i) A[i][i] *= 1.0 + 1.0e-10;
  double L[8][8];
  for (int i = 0; i < k; ++i)
    for (int j = 0; j <= i; ++j) {
      double t = A[i][j];
      for (int u = 0; u < j; ++u) t -= L[i][u] * L[j][u];
      if (i == j) {
        if (!(t > 0.0)) {
          st.status = -2;
          return;
        }
        L[i][i] = sqrt(t);
      } else {
        L[i][j] = t / L[j][j];
      }
    }
  double d[8];
  for (int i = 0; i < k; ++i) {
    double t = b[i];
    for (int u = 0; u < i; ++u) t -= L[i][u] * d[u];
    d[i] = t / L[i][i];
  }
  for (int i = k - 1; i >= 0; --i) {
    double t = d[i];
    for (int u = i + 1; u < k; ++u) t -= L[u][i] * d[u];
    d[i] = t / L[i][i];
  }
  double dt[8];
  for (int u = 0; u < 8; ++u) {
    double t = 0.0;
    for (int i = 0; i < k; ++i) t += P[u][i] * d[i];
    dt[u] = t;
  }
  // largest displacement of the four corners (centred units span +-ex, +-ey)
  const double ex = (a.width - 1) * 0.5 * a.inv_r, ey = (a.height - 1) * 0.5 * a.inv_r;
  double step = 0.0;
  for (int c = 0; c < 4; ++c) {
    const double xc = (c & 1) ? ex : -ex, yc = (c & 2) ? ey : -ey;
    const double dx = dt[0] * xc + dt[1] * yc + dt[2], dy = dt[3] * xc + dt[4] * yc + dt[5];
    step = fmax(step, sqrt(dx * dx + dy * dy));
  }
  if (step > max_step_px) {
    const double f = max_step_px / step;
    for (int u = 0; u < 8; ++u) dt[u] *= f;
    step = max_step_px;
  }
  // centred -> pixel parameters: t0 = t0' / R, t2 = t2' - (t0' cx + t1' cy) / R
  const double ir = a.inv_r, cx = a.cx, cy = a.cy;
  st.theta[0] += dt[0] * ir;
  st.theta[1] += dt[1] * ir;
  st.theta[2] += dt[2] - (dt[0] * cx + dt[1] * cy) * ir;
  st.theta[3] += dt[3] * ir;
  st.theta[4] += dt[4] * ir;
  st.theta[5] += dt[5] - (dt[3] * cx + dt[4] * cy) * ir;
  st.alpha += dt[6];
  st.beta += dt[7];
  st.sigma = robust_sigma + 1.0e-12;
  st.step_px = step;
  st.iterations += 1;
  if (step < tol_px)
    st.status = 1;
  else if (last)
    st.status = 2;
}

struct GnScratch {
  int2* jobs = nullptr;
  GnState* state = nullptr;
  double* partials = nullptr;
  double* sums = nullptr;
  unsigned* hist = nullptr;
  GnState* h_state = nullptr;  // pinned
  int job_cap = 0;
  int block_cap = 0;
};

static void gn_scratch_release(GnScratch& g) {
  if (g.jobs) cudaFree(g.jobs);
  if (g.state) cudaFree(g.state);
  if (g.partials) cudaFree(g.partials);
  if (g.sums) cudaFree(g.sums);
  if (g.hist) cudaFree(g.hist);
  if (g.h_state) cudaFreeHost(g.h_state);
  g = GnScratch{};
}

static GnScratch& gn_scratch(gg_stack* s, int jobs, int blocks) {
  if (!s->gn_scratch) {
    s->gn_scratch = new GnScratch();
    s->gn_scratch_free = [](void* q) {
      auto* g = static_cast<GnScratch*>(q);
      gn_scratch_release(*g);
      delete g;
    };
  }
  GnScratch& g = *static_cast<GnScratch*>(s->gn_scratch);
  if (g.job_cap < jobs || g.block_cap < blocks) {
    auto bytes = [](int64_t jc, int64_t bc) {
      return jc * static_cast<int64_t>(sizeof(int2) + sizeof(GnState) + sizeof(double) * kGnSums * (bc + 1) +
                                          sizeof(unsigned) * kGnHistWords);
    };
    const int64_t before = bytes(g.job_cap, g.block_cap);
    check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(gradient refine scratch)");
    const int jc = std::max(jobs, g.job_cap), bc = std::max(blocks, g.block_cap);
    gn_scratch_release(g);
    check_cuda(cudaMalloc(&g.jobs, sizeof(int2) * jc), "cudaMalloc(gradient refine jobs)");
    check_cuda(cudaMalloc(&g.state, sizeof(GnState) * jc), "cudaMalloc(gradient refine state)");
    check_cuda(cudaMalloc(&g.partials, sizeof(double) * kGnSums * static_cast<size_t>(jc) * bc),
               "cudaMalloc(gradient refine partials)");
    check_cuda(cudaMalloc(&g.sums, sizeof(double) * kGnSums * static_cast<size_t>(jc)),
               "cudaMalloc(gradient refine sums)");
    check_cuda(cudaMalloc(&g.hist, sizeof(unsigned) * kGnHistWords * static_cast<size_t>(jc)),
               "cudaMalloc(gradient refine histogram)");
    check_cuda(cudaHostAlloc(reinterpret_cast<void**>(&g.h_state), sizeof(GnState) * jc, cudaHostAllocDefault),
               "cudaHostAlloc(gradient refine state)");
    g.job_cap = jc;
    g.block_cap = bc;
    s->bytes_allocated += bytes(jc, bc) - before;
  }
  return g;
}

// Blocks per job: about kGnSamplesPerThread samples per thread, or more
// when that leaves the GPU short of two waves of three CTAs per SM; at least
// two samples per thread, at most kGnMaxBlocksPerJob blocks and 2^18 block
// partials over all jobs.  A launch is then many short CTAs, so its time
// follows the jobs still running: the CTAs of converged jobs return at once,
// where a few long CTAs per job would keep every iteration as long as the
// first.  On frames large enough to fill the GPU (the c5 stack: 1 M samples
// per frame) the count depends on the samples alone, so a job's sums do not
// depend on which frames share its launch.
static int gn_blocks_per_job(int64_t samples, int jobs) {
  constexpr int64_t per_block = int64_t{kGnThreads} * kGnSamplesPerThread;
  const int64_t j = std::max(jobs, 1);
  const int64_t by_samples = (samples + per_block - 1) / per_block;
  const int64_t by_fill = (int64_t{6} * sm_count() + j - 1) / j;
  const int64_t floor_cap = std::max<int64_t>(1, (samples + 2 * kGnThreads - 1) / (2 * kGnThreads));
  const int64_t cap = std::min<int64_t>({kGnMaxBlocksPerJob, floor_cap, std::max<int64_t>(1, (int64_t{1} << 18) / j)});
  return static_cast<int>(std::max<int64_t>(1, std::min(std::max(by_samples, by_fill), cap)));
}

static void validate_params(const gg_gradient_refine_params_t& p) {
  require(p.transform_model == GG_TRANSFORM_TRANSLATION || p.transform_model == GG_TRANSFORM_SIMILARITY ||
              p.transform_model == GG_TRANSFORM_AFFINE,
          "transform_model must be translation, similarity or affine");
  require(p.interpolation == GG_INTERP_BILINEAR || p.interpolation == GG_INTERP_LANCZOS3,
          "interpolation must be bilinear or lanczos3");
  require(p.sample_stride >= 1 && p.sample_stride <= 64, "sample_stride must be in [1, 64]");
  require(p.row_stride >= 0 && p.row_stride <= 4096, "row_stride must be in [0, 4096] (0: sample_stride)");
  require(p.stats_passes >= 1 && p.stats_passes <= 16, "stats_passes must be in [1, 16]");
  require(p.iterations >= 1 && p.iterations <= 100, "iterations must be in [1, 100]");
  require(p.min_samples >= 16, "min_samples must be at least 16");
  require(std::isfinite(p.clip_sigma) && p.clip_sigma > 0.0f, "clip_sigma must be positive");
  require(std::isfinite(p.mask_shift_px) && p.mask_shift_px >= 0.0f, "mask_shift_px must be non-negative");
  require(std::isfinite(p.tolerance_px) && p.tolerance_px >= 0.0, "tolerance_px must be non-negative");
  require(std::isfinite(p.max_step_px) && p.max_step_px > 0.0, "max_step_px must be positive");
}

// Column and row steps of a sample grid.  The fine grid is the caller's; the
// photometric and statistics passes use one twice as coarse (both steps of a
// square grid, the row step of a whole-row grid).
struct SampleGrid {
  int cols, rows;
};

static SampleGrid fine_grid(const gg_gradient_refine_params_t& p) {
  return {p.sample_stride, p.row_stride > 0 ? p.row_stride : p.sample_stride};
}

static SampleGrid coarse_grid(const gg_gradient_refine_params_t& p) {
  if (p.row_stride > 0) return {p.sample_stride, std::min(2 * p.row_stride, 8192)};
  const int c = std::min(2 * p.sample_stride, 64);
  return {c, c};
}

// Shared setup: jobs, start states (theta from forward matrices or given
// directly), launch geometry.
struct GnPlan {
  GnArgs args{};
  int jobs = 0;
  int interp = 0;
};

static GnPlan gn_prepare(gg_stack* s, int64_t reference_index, const int64_t* moving, int64_t count,
                         const std::vector<GnState>& states, int interp, int sample_stride, int row_stride,
                         float clip_sigma, float shift_px) {
  stack_require_loaded(s, reference_index, "gradient refinement");
  for (int64_t k = 0; k < count; ++k) stack_require_loaded(s, moving[k], "gradient refinement");
  require(s->pixels <= (int64_t{1} << 31) - 1, "gradient refinement supports frames of fewer than 2^31 pixels");
  stack_activate(s);
  GnPlan plan;
  plan.jobs = static_cast<int>(count);
  plan.interp = interp;
  const int64_t nsx = (s->width + sample_stride - 1) / sample_stride;
  const int64_t nsy = (s->height + row_stride - 1) / row_stride;
  // partial sums for the sample grid given here (the finest one a call uses)
  const int bpj = gn_blocks_per_job(nsx * nsy, plan.jobs);
  GnScratch& g = gn_scratch(s, plan.jobs, bpj);
  std::vector<int2> jobs(static_cast<size_t>(count));
  for (int64_t k = 0; k < count; ++k) jobs[k] = make_int2(static_cast<int>(reference_index), static_cast<int>(moving[k]));
  std::memcpy(g.h_state, states.data(), sizeof(GnState) * states.size());
  upload_params(s->stream, g.jobs, jobs.data(), sizeof(int2) * count, "cudaMemcpyAsync(gradient refine jobs)");
  upload_params(s->stream, g.state, g.h_state, sizeof(GnState) * count, "cudaMemcpyAsync(gradient refine state)");
  GnArgs& a = plan.args;
  a.slots = s->d_slots;
  a.slot_of_frame = s->d_slot_of_frame;
  a.stride = s->stride;
  a.jobs = g.jobs;
  a.state = g.state;
  a.partials = g.partials;
  a.sums_out = g.sums;
  a.hist = g.hist;
  check_cuda(cudaMemsetAsync(g.hist, 0, sizeof(unsigned) * kGnHistWords * count, s->stream),
             "cudaMemsetAsync(gradient refine histogram)");
  a.width = static_cast<int>(s->width);
  a.height = static_cast<int>(s->height);
  a.sample_stride = sample_stride;
  a.row_stride = row_stride;
  a.nsx = static_cast<int>(nsx);
  a.nsy = static_cast<int>(nsy);
  a.blocks_per_job = bpj;
  a.clip_sigma = clip_sigma;
  a.shift_px = shift_px;
  a.cx = static_cast<float>((s->width - 1) * 0.5);
  a.cy = static_cast<float>((s->height - 1) * 0.5);
  a.inv_r = static_cast<float>(2.0 / static_cast<double>(std::max(s->width, s->height)));
  return plan;
}

using GnKernelFn = void (*)(GnArgs);

template <int K>
static GnKernelFn gn_kernel_k(int interp, bool unroll) {
  if (interp == GG_INTERP_BILINEAR) return gn_accumulate_kernel<GG_INTERP_BILINEAR, K, false>;
  return unroll ? gn_accumulate_kernel<GG_INTERP_LANCZOS3, K, true> : gn_accumulate_kernel<GG_INTERP_LANCZOS3, K, false>;
}

static GnKernelFn gn_kernel(int interp, int K, bool unroll) {
  switch (K) {
    case 0: return gn_kernel_k<0>(interp, unroll);
    case 4: return gn_kernel_k<4>(interp, unroll);
    case 6: return gn_kernel_k<6>(interp, unroll);
    default: return gn_kernel_k<8>(interp, unroll);
  }
}


// One pass over the samples: K = 0 statistics, else the model's projected
// columns (see GnLayout).  Lanczos3 passes tune row-by-row against
// whole-window tap loads per shape.
static void gn_accumulate(gg_stack* s, GnPlan& plan, SampleGrid grid_step, int K, int phase = 0) {
  GnArgs a = plan.args;
  a.sample_stride = grid_step.cols;
  a.row_stride = grid_step.rows;
  a.phase = phase;
  a.nsx = static_cast<int>((s->width + grid_step.cols - 1) / grid_step.cols);
  a.nsy = static_cast<int>((s->height + grid_step.rows - 1) / grid_step.rows);
  const int64_t samples = static_cast<int64_t>(a.nsx) * a.nsy;
  GnScratch& g = *static_cast<GnScratch*>(s->gn_scratch);
  auto run = [&](int variant) {
    GnKernelFn fn = gn_kernel(plan.interp, K, variant == 1);
    a.blocks_per_job = std::min(gn_blocks_per_job(samples, plan.jobs), g.block_cap);
    check_cuda(cudaMemsetAsync(g.hist, 0, sizeof(unsigned) * kGnHistWords * plan.jobs, s->stream),
               "cudaMemsetAsync(gradient refine histogram)");
    const dim3 grid(static_cast<unsigned>(a.blocks_per_job), static_cast<unsigned>(plan.jobs));
    note_launch();
    fn<<<grid, kGnThreads, 0, s->stream>>>(a);
    check_cuda(cudaGetLastError(), "gn_accumulate launch");
  };
  int variant = 0;
  if (plan.interp == GG_INTERP_LANCZOS3) {
    const std::string shape = std::to_string(plan.jobs) + " jobs x " + std::to_string(samples) + " samples, " +
                              std::to_string(K) + " columns" + (phase ? ", start pass " + std::to_string(phase) : "");
    variant = autotune_choose("gn_accumulate taps", shape, {"rows", "window"}, 0, s->stream, run);
  }
  run(variant);
  plan.args.blocks_per_job = a.blocks_per_job;
}

static void gn_solve(gg_stack* s, const GnPlan& plan, int mode, int model, int min_samples, double tol,
                     double max_step, int last) {
  note_launch();
  gn_solve_kernel<<<plan.jobs, 32, 0, s->stream>>>(plan.args, mode, model, static_cast<double>(min_samples), tol,
                                                   max_step, last);
  check_cuda(cudaGetLastError(), "gn_solve launch");
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_stack_refine_gradient(gg_stack* s, int64_t reference_index, const int64_t* moving, int64_t count,
                             const double* host_matrices, const gg_gradient_refine_params_t* params,
                             gg_gradient_refine_result_t* host_out) {
  GG_API_BEGIN
  require(s != nullptr && moving != nullptr && host_matrices != nullptr && params != nullptr && host_out != nullptr,
          "null argument");
  require(count > 0 && count <= (int64_t{1} << 20), "indices must contain between 1 and 2^20 frame indices");
  const gg_gradient_refine_params_t& p = *params;
  validate_params(p);
  std::vector<GnState> states(static_cast<size_t>(count));
  for (int64_t k = 0; k < count; ++k) {
    const double* m = host_matrices + 9 * k;
    for (int q = 0; q < 9; ++q) require(std::isfinite(m[q]), "refine matrix must be finite");
    require(m[6] == 0.0 && m[7] == 0.0 && m[8] == 1.0, "refine matrix must be affine (last row 0, 0, 1)");
    double inv[9];
    require(invert3(m, inv), "refine matrix is singular");
    GnState& st = states[static_cast<size_t>(k)];
    std::memset(&st, 0, sizeof(st));
    for (int q = 0; q < 6; ++q) st.theta[q] = inv[q];
    st.alpha = 1.0;
    st.beta = 0.0;
    st.sigma = std::numeric_limits<double>::infinity();
  }
  const SampleGrid fine = fine_grid(p), coarse = coarse_grid(p);
  GnPlan plan = gn_prepare(s, reference_index, moving, count, states, p.interpolation, fine.cols, fine.rows,
                           p.clip_sigma, p.mask_shift_px);
  const int model_k = p.transform_model == GG_TRANSFORM_TRANSLATION ? 4
                      : p.transform_model == GG_TRANSFORM_SIMILARITY ? 6
                                                                      : 8;
  // photometric start (alpha, beta), then statistics passes (offset and
  // noise), all on the coarse grid
  gn_accumulate(s, plan, coarse, 0, 1);
  gn_solve(s, plan, 3, p.transform_model, p.min_samples, p.tolerance_px, p.max_step_px, 0);
  gn_accumulate(s, plan, coarse, 0, 2);
  gn_solve(s, plan, 4, p.transform_model, p.min_samples, p.tolerance_px, p.max_step_px, 0);
  for (int k = 0; k < p.stats_passes; ++k) {
    gn_accumulate(s, plan, coarse, 0);
    gn_solve(s, plan, 0, p.transform_model, p.min_samples, p.tolerance_px, p.max_step_px, 0);
  }
  for (int k = 0; k < p.iterations; ++k) {
    gn_accumulate(s, plan, fine, model_k);
    gn_solve(s, plan, 1, p.transform_model, p.min_samples, p.tolerance_px, p.max_step_px,
             k == p.iterations - 1 ? 1 : 0);
  }
  GnScratch& g = *static_cast<GnScratch*>(s->gn_scratch);
  check_cuda(cudaMemcpyAsync(g.h_state, g.state, sizeof(GnState) * count, cudaMemcpyDeviceToHost, s->stream),
             "cudaMemcpyAsync(gradient refine results)");
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(gradient refine)");
  for (int64_t k = 0; k < count; ++k) {
    const GnState& st = g.h_state[k];
    gg_gradient_refine_result_t& r = host_out[k];
    std::memset(&r, 0, sizeof(r));
    const double inv[9] = {st.theta[0], st.theta[1], st.theta[2], st.theta[3], st.theta[4], st.theta[5],
                           0.0, 0.0, 1.0};
    double fwd[9];
    if (st.status >= 1 && invert3(inv, fwd)) {
      fwd[6] = 0.0;
      fwd[7] = 0.0;
      fwd[8] = 1.0;
      std::memcpy(r.matrix, fwd, sizeof(fwd));
    } else {
      std::memcpy(r.matrix, host_matrices + 9 * k, sizeof(double) * 9);
      if (st.status >= 1) r.status = -2;
    }
    r.alpha = st.alpha;
    r.beta = st.beta;
    r.sigma = st.sigma;
    r.rms = st.rms;
    r.last_step_px = st.step_px;
    r.samples = static_cast<int64_t>(st.samples);
    r.iterations = st.iterations;
    if (r.status == 0) r.status = st.status;
  }
  GG_API_END
}

int gg_stack_gradient_normal_equations(gg_stack* s, int64_t reference_index, const int64_t* moving, int64_t count,
                                       const double* host_theta, const double* host_photometric,
                                       const gg_gradient_refine_params_t* params, double* host_sums) {
  GG_API_BEGIN
  require(s != nullptr && moving != nullptr && host_theta != nullptr && host_photometric != nullptr &&
              params != nullptr && host_sums != nullptr,
          "null argument");
  require(count > 0 && count <= (int64_t{1} << 20), "indices must contain between 1 and 2^20 frame indices");
  validate_params(*params);
  std::vector<GnState> states(static_cast<size_t>(count));
  for (int64_t k = 0; k < count; ++k) {
    GnState& st = states[static_cast<size_t>(k)];
    std::memset(&st, 0, sizeof(st));
    for (int q = 0; q < 6; ++q) {
      require(std::isfinite(host_theta[6 * k + q]), "theta must be finite");
      st.theta[q] = host_theta[6 * k + q];
    }
    st.alpha = host_photometric[3 * k];
    st.beta = host_photometric[3 * k + 1];
    st.sigma = host_photometric[3 * k + 2];
    require(std::isfinite(st.alpha) && std::isfinite(st.beta) && !(st.sigma < 0.0),
            "alpha and beta must be finite and sigma non-negative");
  }
  const SampleGrid fine = fine_grid(*params);
  GnPlan plan = gn_prepare(s, reference_index, moving, count, states, params->interpolation, fine.cols, fine.rows,
                           params->clip_sigma, params->mask_shift_px);
  gn_accumulate(s, plan, fine, 8);
  gn_solve(s, plan, 2, params->transform_model, params->min_samples, 0.0, 1.0, 0);
  GnScratch& g = *static_cast<GnScratch*>(s->gn_scratch);
  check_cuda(cudaMemcpyAsync(host_sums, g.sums, sizeof(double) * kGnSums * count, cudaMemcpyDeviceToHost, s->stream),
             "cudaMemcpyAsync(gradient normal equations)");
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(gradient normal equations)");
  GG_API_END
}

}  // extern "C"
