// Alignment metrics of candidate transforms and sub-pixel translation
// refinement of resident frames.
//
// Semantics (reference NumPy paths of src/glass_cuda.py):
//   matrix_alignment_metrics_f32 :706-768  warp the moving frame bilinearly
//        (fill 0) through M; sample every `stride`-th row and column; valid =
//        covered & finite(reference) & finite(warped); float64 statistics:
//        rms = sqrt(mean(d^2)), mean_abs_diff = mean(|d|), d = warped - ref,
//        ncc = sum(rc * wc) / sqrt(sum(rc^2) sum(wc^2)) about the means
//        (NaN when <= 1 valid sample or a zero denominator).
//   refine_matrix_translation_with_metrics_f32 :771-900  translation offsets
//        on a coarse grid (np.arange(-r, r + step/2, step) in float32, dx
//        outer, dy inner) added in float32 to the float32 matrix, best by the
//        key (rms, -ncc), first wins; then a fine grid around the best at the
//        final stride (or one re-score at the final stride).
//   estimate_translation_subpixel_ncc_f32 :1131-1245  translations center +
//        (ox, oy) * step (oy outer), score = ncc (-inf when <= 1 valid sample
//        or a zero denominator), best by strictly greater score.
// The resident reference evaluates the same grids with its own kernels
// (native_bindings.cpp:10186-10417, warp_kernels.cu:1198-1323).
//
// GB300 mapping: one CTA per (job, sample band).  A warp takes a chunk of
// 32 x 4 samples, keeps the reference samples (and the candidate-independent
// part of the float-float coordinates) in registers and scores every
// candidate of the job on it; the chunk's moving-frame taps stay in L1 across
// candidates, so HBM sees one pass over the sampled pixels per job instead of
// one per candidate.  Per-lane float32 sums about a centring constant, one
// transposing butterfly reduction (8 statistics, 9 shuffles) per candidate
// and chunk, float64 across warps and bands.
#include <array>
#include <cmath>
#include <cstring>
#include <vector>

#include "autotune.cuh"
#include "sampling.cuh"
#include "stack.cuh"

namespace gg {

constexpr int kMetricThreads = 256;
constexpr int kMetricWarps = kMetricThreads / 32;
constexpr int kMaxJobCands = 128;    // candidates of one job per launch
constexpr int kMetricStats = 7;      // sum r, sum w, sum d^2, sum |d|, sum r^2, sum w^2, sum r w

struct MetricCand {
  float m[9][2];  // inverse, float-float
  int affine;
  int pad[3];
};

struct MetricJob {
  int ref_frame;
  int mov_frame;
  int cand_begin;
  int cand_count;  // <= kMaxJobCands
};

struct MetricArgs {
  const float* slots;
  const int* slot_of_frame;
  int64_t stride;
  int width, height;
  int sample_stride;
  int bands;  // CTAs per job
  const MetricJob* jobs;
  const MetricCand* cands;
  double* partial;  // [cand][bands][8]: n, 7 sums
};

struct MetricShared {
  float acc[kMetricWarps][kMaxJobCands][8];  // per-warp sums: n, 7 statistics
  MetricCand sc[kMaxJobCands];
};

constexpr int kChunkK = 4;  // samples per lane per chunk

// Sums v[0..7] over the warp and leaves the sum of v[(lane >> 2) & 7] in
// every lane: a transposing butterfly (4 + 2 + 1 + 1 + 1 shuffles instead
// of 5 per value).
__device__ __forceinline__ float warp_sum8_transposed(const float (&v)[8], int lane) {
  const bool b4 = (lane >> 4) & 1, b3 = (lane >> 3) & 1, b2 = (lane >> 2) & 1;
  float u[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float send = b4 ? v[i] : v[i + 4];
    const float keep = b4 ? v[i + 4] : v[i];
    u[i] = __fadd_rn(keep, __shfl_xor_sync(0xffffffffu, send, 16));
  }
  float w[2];
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const float send = b3 ? u[i] : u[i + 2];
    const float keep = b3 ? u[i + 2] : u[i];
    w[i] = __fadd_rn(keep, __shfl_xor_sync(0xffffffffu, send, 8));
  }
  float z = __fadd_rn(b2 ? w[1] : w[0], __shfl_xor_sync(0xffffffffu, b2 ? w[0] : w[1], 4));
  z = __fadd_rn(z, __shfl_xor_sync(0xffffffffu, z, 2));
  z = __fadd_rn(z, __shfl_xor_sync(0xffffffffu, z, 1));
  return z;
}

__global__ void __launch_bounds__(kMetricThreads) metric_partials_kernel(MetricArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  MetricShared& sh_ = *reinterpret_cast<MetricShared*>(smem);
  auto& acc = sh_.acc;
  auto& sc = sh_.sc;
  __shared__ int s_shared;
  __shared__ float s_urange[4];  // min/max translation (hi) over the candidates: x0, x1, y0, y1
  const MetricJob job = a.jobs[blockIdx.y];
  const int nc = job.cand_count;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < nc; i += blockDim.x) sc[i] = a.cands[job.cand_begin + i];
  for (int i = threadIdx.x; i < kMetricWarps * kMaxJobCands * 8; i += blockDim.x) (&acc[0][0][0])[i] = 0.0f;
  __syncthreads();
  if (threadIdx.x == 0) {
    // Candidates that differ only in their translation (a translation grid
    // around one matrix) share the x/y products of the source coordinate.
    int shared = 1;
    for (int c = 0; c < nc && shared; ++c) {
      const MetricCand& q = sc[c];
      shared = q.affine && q.m[0][0] == sc[0].m[0][0] && q.m[0][1] == sc[0].m[0][1] &&
               q.m[1][0] == sc[0].m[1][0] && q.m[1][1] == sc[0].m[1][1] && q.m[3][0] == sc[0].m[3][0] &&
               q.m[3][1] == sc[0].m[3][1] && q.m[4][0] == sc[0].m[4][0] && q.m[4][1] == sc[0].m[4][1];
    }
    s_shared = shared;
    float ux0 = kInfF, ux1 = -kInfF, uy0 = kInfF, uy1 = -kInfF;
    for (int c = 0; c < nc; ++c) {
      ux0 = fminf(ux0, sc[c].m[2][0]);
      ux1 = fmaxf(ux1, sc[c].m[2][0]);
      uy0 = fminf(uy0, sc[c].m[5][0]);
      uy1 = fmaxf(uy1, sc[c].m[5][0]);
    }
    s_urange[0] = ux0;
    s_urange[1] = ux1;
    s_urange[2] = uy0;
    s_urange[3] = uy1;
  }
  __syncthreads();
  const int W = a.width, H = a.height, st = a.sample_stride;
  const float* ref = a.slots + static_cast<int64_t>(a.slot_of_frame[job.ref_frame]) * a.stride;
  const float* mov = a.slots + static_cast<int64_t>(a.slot_of_frame[job.mov_frame]) * a.stride;
  // centring constant shared by every CTA of the job
  float shift = __ldg(ref + static_cast<int64_t>(H / 2) * W + W / 2);
  if (!isfinite(shift)) shift = 0.0f;
  const int sw = (W + st - 1) / st, sh = (H + st - 1) / st;
  const int64_t total = static_cast<int64_t>(sw) * sh;
  const int64_t begin = total * blockIdx.x / a.bands, end = total * (blockIdx.x + 1) / a.bands;
  const float Wm1 = static_cast<float>(W - 1), Hm1 = static_cast<float>(H - 1);
  const bool shared = s_shared != 0;
  const int slot = (lane >> 2) & 7;  // statistic this lane holds after the reduction
  constexpr int kChunk = 32 * kChunkK;
  // a chunk of 128 samples per warp: its reference samples and moving-frame
  // taps are loaded once (registers / L1) and scored for every candidate
  for (int64_t c0 = begin + static_cast<int64_t>(warp) * kChunk; c0 < end; c0 += kMetricWarps * kChunk) {
    float rv[kChunkK];
    int xs[kChunkK], ys[kChunkK];
    bool rok[kChunkK];
#pragma unroll
    for (int k = 0; k < kChunkK; ++k) {
      const int64_t t = c0 + lane + 32 * k;
      rok[k] = false;
      xs[k] = ys[k] = 0;
      rv[k] = 0.0f;
      if (t < end) {
        const int row = static_cast<int>(t / sw), col = static_cast<int>(t - static_cast<int64_t>(row) * sw);
        xs[k] = col * st;
        ys[k] = row * st;
        rv[k] = __ldg(ref + static_cast<int64_t>(ys[k]) * W + xs[k]);
        rok[k] = isfinite(rv[k]);
      }
    }
    FFPre px[kChunkK], py[kChunkK];
    bool inside = false;
    if (shared) {
      float lo_x = kInfF, hi_x = -kInfF, lo_y = kInfF, hi_y = -kInfF;
#pragma unroll
      for (int k = 0; k < kChunkK; ++k) {
        px[k] = ff_lin_pre(sc[0].m[0][0], sc[0].m[1][0], static_cast<float>(xs[k]), static_cast<float>(ys[k]));
        py[k] = ff_lin_pre(sc[0].m[3][0], sc[0].m[4][0], static_cast<float>(xs[k]), static_cast<float>(ys[k]));
        if (rok[k]) {
          lo_x = fminf(lo_x, px[k].s);
          hi_x = fmaxf(hi_x, px[k].s);
          lo_y = fminf(lo_y, py[k].s);
          hi_y = fmaxf(hi_y, py[k].s);
        }
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        lo_x = fminf(lo_x, __shfl_xor_sync(0xffffffffu, lo_x, off));
        hi_x = fmaxf(hi_x, __shfl_xor_sync(0xffffffffu, hi_x, off));
        lo_y = fminf(lo_y, __shfl_xor_sync(0xffffffffu, lo_y, off));
        hi_y = fmaxf(hi_y, __shfl_xor_sync(0xffffffffu, hi_y, off));
      }
      // Every candidate's source coordinate of every sample of the chunk lies
      // inside [0, W-2] x [0, H-2] with a margin above the float-float low
      // parts (a few float32 ulps of the coordinate): skip the per-sample
      // validity tests and the edge clamps of the bilinear taps.
      const float margin = 0.01f + 1.0e-6f * (Wm1 + Hm1);
      inside = lo_x + s_urange[0] >= margin && hi_x + s_urange[1] <= Wm1 - 1.0f - margin &&
               lo_y + s_urange[2] >= margin && hi_y + s_urange[3] <= Hm1 - 1.0f - margin;
    }
    if (inside) {
      for (int c = 0; c < nc; ++c) {
        float s[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};  // n, 7 statistics
        const MetricCand& cd = sc[c];
#pragma unroll
        for (int k = 0; k < kChunkK; ++k) {
          if (!rok[k]) continue;
          const float xf = static_cast<float>(xs[k]), yf = static_cast<float>(ys[k]);
          const FFv sx = ff_lin_finish(px[k], cd.m[0][1], cd.m[1][1], xf, yf, cd.m[2][0], cd.m[2][1]);
          const FFv sy = ff_lin_finish(py[k], cd.m[3][1], cd.m[4][1], xf, yf, cd.m[5][0], cd.m[5][1]);
          int x0, y0;
          float tx, ty;
          ff_floor_frac(sx, x0, tx);
          ff_floor_frac(sy, y0, ty);
          const float* r0 = mov + y0 * W + x0;  // y0 * W < 2^31 (checked on the host)
          const float v00 = __ldg(r0), v01 = __ldg(r0 + 1), v10 = __ldg(r0 + W), v11 = __ldg(r0 + W + 1);
          const float ox = __fsub_rn(1.0f, tx), oy = __fsub_rn(1.0f, ty);
          const float top = __fadd_rn(__fmul_rn(v00, ox), __fmul_rn(v01, tx));
          const float bottom = __fadd_rn(__fmul_rn(v10, ox), __fmul_rn(v11, tx));
          const float w = __fadd_rn(__fmul_rn(top, oy), __fmul_rn(bottom, ty));
          if (!isfinite(w)) continue;
          const float r = rv[k];
          const float rc = __fsub_rn(r, shift), wc = __fsub_rn(w, shift), d = __fsub_rn(w, r);
          s[0] = __fadd_rn(s[0], 1.0f);
          s[1] = __fadd_rn(s[1], rc);
          s[2] = __fadd_rn(s[2], wc);
          s[3] = __fmaf_rn(d, d, s[3]);
          s[4] = __fadd_rn(s[4], fabsf(d));
          s[5] = __fmaf_rn(rc, rc, s[5]);
          s[6] = __fmaf_rn(wc, wc, s[6]);
          s[7] = __fmaf_rn(rc, wc, s[7]);
        }
        const float z = warp_sum8_transposed(s, lane);
        if ((lane & 3) == 0) acc[warp][c][slot] = __fadd_rn(acc[warp][c][slot], z);
      }
      continue;
    }
    for (int c = 0; c < nc; ++c) {
      float s[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};  // n, 7 statistics
      const MetricCand& cd = sc[c];
#pragma unroll
      for (int k = 0; k < kChunkK; ++k) {
        if (!rok[k]) continue;
        FFv sx, sy;
        const float xf = static_cast<float>(xs[k]), yf = static_cast<float>(ys[k]);
        if (shared) {
          sx = ff_lin_finish(px[k], cd.m[0][1], cd.m[1][1], xf, yf, cd.m[2][0], cd.m[2][1]);
          sy = ff_lin_finish(py[k], cd.m[3][1], cd.m[4][1], xf, yf, cd.m[5][0], cd.m[5][1]);
        } else if (!source_coord(cd, xf, yf, sx, sy)) {
          continue;
        }
        if (!(ff_ge(sx, 0.0f) && ff_le(sx, Wm1) && ff_ge(sy, 0.0f) && ff_le(sy, Hm1))) continue;
        int x0, y0;
        float tx, ty;
        ff_floor_frac(sx, x0, tx);
        ff_floor_frac(sy, y0, ty);
        const float w = bilinear_at(mov, W, H, x0, y0, tx, ty);
        if (!isfinite(w)) continue;
        const float r = rv[k];
        const float rc = __fsub_rn(r, shift), wc = __fsub_rn(w, shift), d = __fsub_rn(w, r);
        s[0] = __fadd_rn(s[0], 1.0f);
        s[1] = __fadd_rn(s[1], rc);
        s[2] = __fadd_rn(s[2], wc);
        s[3] = __fmaf_rn(d, d, s[3]);
        s[4] = __fadd_rn(s[4], fabsf(d));
        s[5] = __fmaf_rn(rc, rc, s[5]);
        s[6] = __fmaf_rn(wc, wc, s[6]);
        s[7] = __fmaf_rn(rc, wc, s[7]);
      }
      const float z = warp_sum8_transposed(s, lane);
      if ((lane & 3) == 0) acc[warp][c][slot] = __fadd_rn(acc[warp][c][slot], z);
    }
  }
  __syncthreads();
  for (int c = threadIdx.x; c < nc; c += blockDim.x) {
    double out[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int w = 0; w < kMetricWarps; ++w)
      for (int q = 0; q < 8; ++q) out[q] += static_cast<double>(acc[w][c][q]);
    double* dst = a.partial + (static_cast<int64_t>(job.cand_begin + c) * a.bands + blockIdx.x) * 8;
    for (int q = 0; q < 8; ++q) dst[q] = out[q];
  }
}

// Sum the band partials of every candidate in band order.  The statistics
// stay about the centring constant: the metrics only use differences and
// central moments, in which it cancels.
__global__ void metric_reduce_kernel(const double* partial, int ncand, int bands, double* sums) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncand) return;
  double out[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int b = 0; b < bands; ++b)
    for (int q = 0; q < 8; ++q) out[q] += partial[(static_cast<int64_t>(c) * bands + b) * 8 + q];
  for (int q = 0; q < 8; ++q) sums[static_cast<int64_t>(c) * 8 + q] = out[q];
}

struct Metrics {
  int64_t valid = 0;
  int64_t sampled = 0;
  double rms = NAN;
  double mad = NAN;
  double ncc = NAN;
};

// Statistics about the centring constant -> metrics (the constant cancels).
static Metrics metrics_from_sums(const double* s, int64_t sampled) {
  Metrics m;
  m.sampled = sampled;
  const double n = s[0];
  m.valid = static_cast<int64_t>(n);
  if (m.valid == 0) return m;
  m.rms = std::sqrt(s[3] / n);
  m.mad = s[4] / n;
  if (m.valid <= 1) return m;
  const double mr = s[1] / n, mw = s[2] / n;
  const double srr = s[5] - n * mr * mr, sww = s[6] - n * mw * mw, srw = s[7] - n * mr * mw;
  const double den = std::sqrt(std::max(srr, 0.0) * std::max(sww, 0.0));
  m.ncc = den > 0.0 ? srw / den : NAN;
  return m;
}

struct MetricScratch {
  MetricJob* jobs = nullptr;
  MetricCand* cands = nullptr;
  double* partial = nullptr;
  double* sums = nullptr;
  int job_cap = 0;
  int cand_cap = 0;
  int bands_cap = 0;
};

static void metric_scratch_release(MetricScratch& m) {
  if (m.jobs) cudaFree(m.jobs);
  if (m.cands) cudaFree(m.cands);
  if (m.partial) cudaFree(m.partial);
  if (m.sums) cudaFree(m.sums);
  m = MetricScratch{};
}

static MetricScratch& metric_scratch(gg_stack* s) {
  if (!s->metric_scratch) {
    s->metric_scratch = new MetricScratch();
    s->metric_scratch_free = [](void* q) {
      auto* m = static_cast<MetricScratch*>(q);
      metric_scratch_release(*m);
      delete m;
    };
  }
  return *static_cast<MetricScratch*>(s->metric_scratch);
}

// A candidate list for one (reference, moving) frame pair.
struct PairCands {
  int ref_frame;
  int mov_frame;
  std::vector<MetricCand> cands;
};

// Evaluates every candidate of every pair at `stride`; returns the eight
// statistics per candidate (pair-major).
static std::vector<double> evaluate_candidates(gg_stack* s, const std::vector<PairCands>& pairs, int stride) {
  std::vector<MetricJob> jobs;
  std::vector<MetricCand> cands;
  for (const PairCands& p : pairs) {
    const int base = static_cast<int>(cands.size());
    cands.insert(cands.end(), p.cands.begin(), p.cands.end());
    for (int c0 = 0; c0 < static_cast<int>(p.cands.size()); c0 += kMaxJobCands)
      jobs.push_back(MetricJob{p.ref_frame, p.mov_frame, base + c0,
                               std::min(kMaxJobCands, static_cast<int>(p.cands.size()) - c0)});
  }
  std::vector<double> sums(cands.size() * 8, 0.0);
  if (jobs.empty()) return sums;
  const int64_t sw = (s->width + stride - 1) / stride, sh = (s->height + stride - 1) / stride;
  require(s->pixels <= (int64_t{1} << 31) - 1, "alignment metrics support frames of fewer than 2^31 pixels");
  // bands: enough CTAs to fill the GPU (2, 4 or 8 per SM over all jobs,
  // picked by the autotuner), at least 2048 samples each
  const int64_t samples = sw * sh;
  int band_options[3];
  for (int i = 0; i < 3; ++i) {
    const int want = std::max(1, (sm_count() * (2 << i) + static_cast<int>(jobs.size()) - 1) /
                                     static_cast<int>(jobs.size()));
    band_options[i] = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(want, (samples + 2047) / 2048)));
  }
  const int bands = std::max(band_options[0], std::max(band_options[1], band_options[2]));  // capacity
  MetricScratch& m = metric_scratch(s);
  const int nj = static_cast<int>(jobs.size()), ncand = static_cast<int>(cands.size());
  if (m.job_cap < nj || m.cand_cap < ncand || m.bands_cap < bands) {
    auto bytes = [](int64_t jc, int64_t cc, int64_t bc) {
      return jc * static_cast<int64_t>(sizeof(MetricJob)) + cc * static_cast<int64_t>(sizeof(MetricCand)) +
             64 * cc * bc + 64 * cc;
    };
    const int64_t before = bytes(m.job_cap, m.cand_cap, m.bands_cap);
    check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(metric scratch)");
    const int jc = std::max(nj, m.job_cap), cc = std::max(ncand, m.cand_cap), bc = std::max(bands, m.bands_cap);
    metric_scratch_release(m);
    check_cuda(cudaMalloc(&m.jobs, sizeof(MetricJob) * jc), "cudaMalloc(metric jobs)");
    check_cuda(cudaMalloc(&m.cands, sizeof(MetricCand) * cc), "cudaMalloc(metric candidates)");
    check_cuda(cudaMalloc(&m.partial, sizeof(double) * 8 * static_cast<size_t>(cc) * bc), "cudaMalloc(metric partials)");
    check_cuda(cudaMalloc(&m.sums, sizeof(double) * 8 * static_cast<size_t>(cc)), "cudaMalloc(metric sums)");
    m.job_cap = jc;
    m.cand_cap = cc;
    m.bands_cap = bc;
    s->bytes_allocated += bytes(jc, cc, bc) - before;
  }
  upload_params(s->stream, m.jobs, jobs.data(), sizeof(MetricJob) * nj, "cudaMemcpyAsync(metric jobs)");
  upload_params(s->stream, m.cands, cands.data(), sizeof(MetricCand) * ncand, "cudaMemcpyAsync(metric candidates)");
  MetricArgs a{};
  a.slots = s->d_slots;
  a.slot_of_frame = s->d_slot_of_frame;
  a.stride = s->stride;
  a.width = static_cast<int>(s->width);
  a.height = static_cast<int>(s->height);
  a.sample_stride = stride;
  a.jobs = m.jobs;
  a.cands = m.cands;
  a.partial = m.partial;
  check_cuda(cudaFuncSetAttribute(metric_partials_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(sizeof(MetricShared))),
             "cudaFuncSetAttribute(metric_partials)");
  auto run = [&](int c) {
    MetricArgs b = a;
    b.bands = band_options[c];
    note_launch();
    metric_partials_kernel<<<dim3(b.bands, nj), kMetricThreads, sizeof(MetricShared), s->stream>>>(b);
    check_cuda(cudaGetLastError(), "metric_partials launch");
    note_launch();
    metric_reduce_kernel<<<(ncand + 127) / 128, 128, 0, s->stream>>>(m.partial, ncand, b.bands, m.sums);
    check_cuda(cudaGetLastError(), "metric_reduce launch");
  };
  const std::string shape = std::to_string(nj) + " jobs x " + std::to_string(ncand / std::max(nj, 1)) +
                            " candidates x " + std::to_string(samples) + " samples";
  run(autotune_choose("metric_partials bands", shape, {"2/SM", "4/SM", "8/SM"}, 1, s->stream, run));
  check_cuda(cudaMemcpyAsync(sums.data(), m.sums, sizeof(double) * 8 * ncand, cudaMemcpyDeviceToHost, s->stream),
             "cudaMemcpyAsync(metric sums)");
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(metrics)");
  return sums;
}

static MetricCand candidate_from_forward(const double* fwd) {
  MetricCand c;
  std::memset(&c, 0, sizeof(c));
  for (int q = 0; q < 9; ++q)
    if (!std::isfinite(fwd[q])) fail(GG_ERR_INVALID_ARGUMENT, "alignment matrix must be finite");
  if (!inverse_coefficients(fwd, c.m, c.affine)) fail(GG_ERR_INVALID_ARGUMENT, "alignment matrix is singular");
  return c;
}

// float32 matrix with (dx, dy) added in float32 to the translation terms.
static void shifted_matrix32(const float* base, float dx, float dy, float* out32, double* out64) {
  for (int q = 0; q < 9; ++q) out32[q] = base[q];
  out32[2] = base[2] + dx;
  out32[5] = base[5] + dy;
  for (int q = 0; q < 9; ++q) out64[q] = static_cast<double>(out32[q]);
}

// np.arange(start, stop, step, dtype=np.float32) with Python-float bounds:
// length ceil((stop - start) / step); the first two values rounded from
// float64, the rest start + i * (second - first) in float32.
static std::vector<float> arange_f32(double start, double stop, double step) {
  std::vector<float> v;
  const double len_d = std::ceil((stop - start) / step);
  if (!(len_d > 0.0)) return v;
  require(len_d <= 1.0e6, "translation search grid is too large");
  const int64_t len = static_cast<int64_t>(len_d);
  v.resize(static_cast<size_t>(len));
  v[0] = static_cast<float>(start);
  if (len > 1) v[1] = static_cast<float>(start + step);
  const float delta = len > 1 ? v[1] - v[0] : 0.0f;
  for (int64_t i = 2; i < len; ++i) {
    volatile float prod = static_cast<float>(i) * delta;  // no fused multiply-add
    v[static_cast<size_t>(i)] = v[0] + prod;
  }
  return v;
}

// Python tuple comparison (rms, -ncc) < (rms', -ncc') with NaN compares false.
static bool key_less(double r1, double n1, double r2, double n2) {
  if (r1 != r2) return r1 < r2;
  return -n1 < -n2;
}

static void fill_metrics(const Metrics& m, int stride, gg_alignment_metrics_t& o) {
  o.valid_pixels = m.valid;
  o.sampled_pixels = m.sampled;
  o.sample_stride = stride;
  o.pad = 0;
  o.rms = m.rms;
  o.mean_abs_diff = m.mad;
  o.ncc = m.ncc;
}

static int64_t sampled_count(const gg_stack* s, int stride) {
  return ((s->width + stride - 1) / stride) * ((s->height + stride - 1) / stride);
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_stack_alignment_metrics(gg_stack* s, int64_t reference_index, const int64_t* indices, int64_t count,
                               const double* host_matrices, int32_t sample_stride, gg_alignment_metrics_t* host_out) {
  GG_API_BEGIN
  require(s != nullptr && indices != nullptr && host_matrices != nullptr && host_out != nullptr, "null argument");
  require(count > 0, "indices must contain at least one frame index");
  require(sample_stride > 0, "sample_stride must be positive");
  stack_require_loaded(s, reference_index, "alignment metrics");
  std::vector<PairCands> pairs(static_cast<size_t>(count));
  for (int64_t k = 0; k < count; ++k) {
    stack_require_loaded(s, indices[k], "alignment metrics");
    pairs[static_cast<size_t>(k)].ref_frame = static_cast<int>(reference_index);
    pairs[static_cast<size_t>(k)].mov_frame = static_cast<int>(indices[k]);
    pairs[static_cast<size_t>(k)].cands.push_back(candidate_from_forward(host_matrices + 9 * k));
  }
  stack_activate(s);
  const std::vector<double> sums = evaluate_candidates(s, pairs, sample_stride);
  const int64_t sampled = sampled_count(s, sample_stride);
  for (int64_t k = 0; k < count; ++k)
    fill_metrics(metrics_from_sums(&sums[static_cast<size_t>(k) * 8], sampled), sample_stride, host_out[k]);
  GG_API_END
}

int gg_stack_refine_translation(gg_stack* s, int64_t reference_index, const int64_t* indices, int64_t count,
                                const double* host_matrices, const gg_refine_params_t* params,
                                gg_refine_result_t* host_out) {
  GG_API_BEGIN
  require(s != nullptr && indices != nullptr && host_matrices != nullptr && params != nullptr && host_out != nullptr,
          "null argument");
  require(count > 0, "indices must contain at least one frame index");
  const gg_refine_params_t& p = *params;
  require(std::isfinite(p.search_radius_px) && p.search_radius_px >= 0.0, "search_radius_px must be non-negative");
  require(std::isfinite(p.coarse_step_px) && p.coarse_step_px > 0.0, "coarse_step_px must be positive");
  require(std::isfinite(p.fine_radius_px) && p.fine_radius_px >= 0.0, "fine_radius_px must be non-negative");
  require(std::isfinite(p.fine_step_px) && p.fine_step_px > 0.0, "fine_step_px must be positive");
  require(p.coarse_sample_stride > 0 && p.final_sample_stride > 0, "sample strides must be positive");
  stack_require_loaded(s, reference_index, "translation refinement");
  for (int64_t k = 0; k < count; ++k) stack_require_loaded(s, indices[k], "translation refinement");
  stack_activate(s);
  const size_t n = static_cast<size_t>(count);
  std::vector<std::array<float, 9>> base(n);
  for (size_t k = 0; k < n; ++k)
    for (int q = 0; q < 9; ++q) {
      if (!std::isfinite(host_matrices[9 * k + q])) fail(GG_ERR_INVALID_ARGUMENT, "refine matrix must be finite");
      base[k][q] = static_cast<float>(host_matrices[9 * k + q]);
    }
  // coarse grid (glass_cuda.py:823-843)
  const double r = p.search_radius_px, cs = p.coarse_step_px;
  const std::vector<float> coarse = arange_f32(-r, r + cs * 0.5, cs);
  require(!coarse.empty(), "empty coarse translation grid");
  std::vector<PairCands> pairs(n);
  for (size_t k = 0; k < n; ++k) {
    pairs[k].ref_frame = static_cast<int>(reference_index);
    pairs[k].mov_frame = static_cast<int>(indices[k]);
    for (float dx : coarse)
      for (float dy : coarse) {
        float m32[9];
        double m64[9];
        shifted_matrix32(base[k].data(), dx, dy, m32, m64);
        pairs[k].cands.push_back(candidate_from_forward(m64));
      }
  }
  const int64_t coarse_sampled = sampled_count(s, p.coarse_sample_stride);
  std::vector<double> sums = evaluate_candidates(s, pairs, p.coarse_sample_stride);
  std::vector<float> best_dx(n, 0.0f), best_dy(n, 0.0f);
  std::vector<Metrics> best_m(n);
  size_t off = 0;
  for (size_t k = 0; k < n; ++k) {
    bool have = false;
    for (float dx : coarse)
      for (float dy : coarse) {
        const Metrics m = metrics_from_sums(&sums[off * 8], coarse_sampled);
        ++off;
        if (!have || key_less(m.rms, m.ncc, best_m[k].rms, best_m[k].ncc)) {
          have = true;
          best_m[k] = m;
          best_dx[k] = dx;
          best_dy[k] = dy;
        }
      }
  }
  int best_stride = p.coarse_sample_stride;
  std::vector<int> fine_count(n, 0);
  if (p.fine_radius_px > 0.0 || p.final_sample_stride != p.coarse_sample_stride) {
    // fine grid around the coarse best (glass_cuda.py:845-871), or one
    // re-score of the coarse best at the final stride
    std::vector<std::vector<float>> fx(n), fy(n);
    for (size_t k = 0; k < n; ++k) {
      pairs[k].cands.clear();
      if (p.fine_radius_px > 0.0) {
        const double bx = best_dx[k], by = best_dy[k], fr = p.fine_radius_px, fs = p.fine_step_px;
        fx[k] = arange_f32(bx - fr, bx + fr + fs * 0.5, fs);
        fy[k] = arange_f32(by - fr, by + fr + fs * 0.5, fs);
      } else {
        fx[k] = {best_dx[k]};
        fy[k] = {best_dy[k]};
      }
      for (float dx : fx[k])
        for (float dy : fy[k]) {
          float m32[9];
          double m64[9];
          shifted_matrix32(base[k].data(), dx, dy, m32, m64);
          pairs[k].cands.push_back(candidate_from_forward(m64));
        }
    }
    const int64_t fine_sampled = sampled_count(s, p.final_sample_stride);
    sums = evaluate_candidates(s, pairs, p.final_sample_stride);
    off = 0;
    for (size_t k = 0; k < n; ++k) {
      bool have = false;
      for (float dx : fx[k])
        for (float dy : fy[k]) {
          const Metrics m = metrics_from_sums(&sums[off * 8], fine_sampled);
          ++off;
          if (p.fine_radius_px > 0.0) ++fine_count[k];
          if (!have || key_less(m.rms, m.ncc, best_m[k].rms, best_m[k].ncc)) {
            have = true;
            best_m[k] = m;
            best_dx[k] = dx;
            best_dy[k] = dy;
          }
        }
    }
    best_stride = p.final_sample_stride;
  }
  for (size_t k = 0; k < n; ++k) {
    gg_refine_result_t& o = host_out[k];
    float m32[9];
    double m64[9];
    shifted_matrix32(base[k].data(), best_dx[k], best_dy[k], m32, m64);
    for (int q = 0; q < 9; ++q) o.matrix[q] = m64[q];
    o.dx_correction = best_dx[k];
    o.dy_correction = best_dy[k];
    fill_metrics(best_m[k], best_stride, o.metrics);
    o.coarse_candidates = static_cast<int32_t>(coarse.size() * coarse.size());
    o.fine_candidates = fine_count[k];
  }
  GG_API_END
}

int gg_stack_translation_ncc(gg_stack* s, int64_t reference_index, int64_t moving_index, double center_dx,
                             double center_dy, int32_t radius_steps, double step, int32_t sample_stride,
                             gg_translation_ncc_t* host_out) {
  GG_API_BEGIN
  require(s != nullptr && host_out != nullptr, "null argument");
  require(sample_stride > 0, "sample_stride must be positive");
  require(radius_steps >= 0, "radius_steps must be non-negative");
  require(radius_steps <= 512, "radius_steps must be at most 512");
  require(std::isfinite(step) && step > 0.0, "step must be positive");
  require(std::isfinite(center_dx) && std::isfinite(center_dy), "center must be finite");
  stack_require_loaded(s, reference_index, "translation ncc");
  stack_require_loaded(s, moving_index, "translation ncc");
  stack_activate(s);
  std::vector<PairCands> pairs(1);
  pairs[0].ref_frame = static_cast<int>(reference_index);
  pairs[0].mov_frame = static_cast<int>(moving_index);
  std::vector<double> dxs, dys;
  for (int oy = -radius_steps; oy <= radius_steps; ++oy)
    for (int ox = -radius_steps; ox <= radius_steps; ++ox) {
      const double dx = center_dx + ox * step, dy = center_dy + oy * step;
      const double fwd[9] = {1.0, 0.0, dx, 0.0, 1.0, dy, 0.0, 0.0, 1.0};
      pairs[0].cands.push_back(candidate_from_forward(fwd));
      dxs.push_back(dx);
      dys.push_back(dy);
    }
  const std::vector<double> sums = evaluate_candidates(s, pairs, sample_stride);
  const int64_t sampled = sampled_count(s, sample_stride);
  double best = -HUGE_VAL;
  host_out->dx = center_dx;
  host_out->dy = center_dy;
  for (size_t c = 0; c < dxs.size(); ++c) {
    const Metrics m = metrics_from_sums(&sums[c * 8], sampled);
    const double score = (m.valid <= 1 || std::isnan(m.ncc)) ? -HUGE_VAL : m.ncc;
    if (score > best) {
      best = score;
      host_out->dx = dxs[c];
      host_out->dy = dys[c];
    }
  }
  host_out->score = best;
  host_out->candidate_count = static_cast<int64_t>(dxs.size());
  GG_API_END
}

}  // extern "C"
