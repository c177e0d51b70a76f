// Matrix warps of resident frames: bilinear and Lanczos3, TMA-staged.
//
// Semantics (CPU oracle): output pixel (x, y) samples the source at
// M^-1 (x, y, 1) (float64 in the reference: engine/warp.py:155-227,
// tests/test_gpu_warp_vs_cpu.py:34-128; reference kernels
// warp_kernels.cu:206-777).
//   bilinear: valid iff 0 <= sx <= W-1 and 0 <= sy <= H-1; x1 = min(x0+1, W-1);
//             tx = float32(sx - x0); top/bottom/result in float32 arithmetic.
//   lanczos3: valid iff 2 <= sx < W-3 and 2 <= sy < H-3; 6x6 taps from
//             (x0-2, y0-2); w = sinc(d) sinc(d/3); non-finite taps are skipped
//             and the sum is renormalised; |sum w| <= 1e-12 -> invalid; an
//             optional clamp to [min - c*range, max + c*range] of the taps.
//   invalid pixels get `fill` and coverage 0.
//
// GB300 design
//   - source coordinates are evaluated in float-float (TwoProd/TwoSum) from
//     the float64 inverse, so floor/validity decisions agree with the float64
//     reference without float64 arithmetic on the device;
//   - each CTA owns a 64x48 output tile; its source footprint (an 80x64 box
//     for the small rotations registration produces) is copied to shared
//     memory by one cp.async.bulk.tensor (TMA) load, double-buffered against
//     the previous tile's compute.  Footprints that do not fit the box (large
//     rotation/scale) and image widths that TMA cannot describe (W % 4 != 0)
//     read the taps straight from global memory instead;
//   - output goes to a spare slot; a follow-up kernel swaps the frame->slot
//     table, so nothing is copied back (8 B/pixel instead of 16 B);
//   - Lanczos3 weights are paired even/odd polynomials in (t - 1/2)^2
//     (sampling.cuh); interior tiles of finite frames run a straight-line
//     form without per-pixel tests.
#include <cmath>
#include <cstring>
#include <vector>

#include <cudaTypedefs.h>

#include "sampling.cuh"
#include "stack.cuh"

namespace gg {

constexpr int kTileW = 64;
constexpr int kTileH = 48;
constexpr int kWarpThreads = 256;  // 64 x 4; each thread covers kTileH / 4 rows
constexpr int kRowsPerThread = kTileH / 4;
// Affine source coordinates are stepped by 4 output rows in float-float and
// evaluated afresh every kFreshRows rows: at most three steps of rounding
// separate a coordinate from the float64-faithful evaluation, so floor and
// fraction decisions stay those of a direct evaluation.
constexpr int kFreshRows = 4;

struct WarpItem {
  int frame;
  int src_slot;     // filled on the device
  int dst_slot;     // filled on the device
  unsigned src_nonfinite;
  int affine;
  int int_shift;  // inverse is an exact integer translation
  int pad[2];
  float m[9][2];  // inverse matrix, float-float (hi, lo), row-major
};

struct WarpArgs {
  float* slots;
  int* slot_of_frame;
  int* spare_slot;
  unsigned* nonfinite;
  WarpItem* items;
  int item_count;
  int64_t stride;
  int width;
  int height;
  int tiles_x;
  int tiles_y;
  int interp;
  float fill;
  float clamp;
  float* coverage;  // optional accumulator (+1 per covered pixel)
  int* error;
};

// ---- PTX helpers -------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: gives up after `limit` polls (each poll may suspend briefly).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, int limit) {
  for (int i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tma_load_3d(float* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(smem_addr(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

// Register copy of one item's inverse matrix (loaded once per work item so
// that output stores cannot force re-reads of the descriptor).
struct Coef {
  float m[9][2];
  int affine;
};

__device__ __forceinline__ Coef load_coef(const WarpItem* p) {
  Coef c;
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    c.m[q][0] = __ldg(&p->m[q][0]);
    c.m[q][1] = __ldg(&p->m[q][1]);
  }
  c.affine = __ldg(&p->affine);
  return c;
}

// Tile plan: box origin for the source footprint of output tile (tx, ty).
struct TilePlan {
  int bx, by, fits, interior;
};

// interior: an affine map sends the whole tile at least one pixel inside the
// valid source range (valid_lo <= s <= valid_hi on both axes), so no pixel
// of the tile needs its own validity test.
__device__ __forceinline__ TilePlan plan_tile(const Coef& it, int tile_x, int tile_y, int radius, float valid_lo,
                                              float valid_hi_x, float valid_hi_y) {
  const float x0 = static_cast<float>(tile_x * kTileW), y0 = static_cast<float>(tile_y * kTileH);
  const float cx[4] = {x0, x0 + kTileW - 1, x0, x0 + kTileW - 1};
  const float cy[4] = {y0, y0, y0 + kTileH - 1, y0 + kTileH - 1};
  float minx = kInfF, maxx = -kInfF, miny = kInfF, maxy = -kInfF;
  bool ok = true;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    FFv sx, sy;
    ok &= source_coord(it, cx[c], cy[c], sx, sy);
    minx = fminf(minx, sx.hi);
    maxx = fmaxf(maxx, sx.hi);
    miny = fminf(miny, sy.hi);
    maxy = fmaxf(maxy, sy.hi);
  }
  TilePlan p{0, 0, 0, 0};
  if (!ok || !(maxx - minx < 1.0e6f) || !(maxy - miny < 1.0e6f) || fabsf(minx) > 1.0e8f || fabsf(miny) > 1.0e8f)
    return p;
  // taps span [floor(s) - (radius-1), floor(s) + radius]; one pixel of margin.
  const int lo_x = static_cast<int>(floorf(minx)) - radius;
  const int hi_x = static_cast<int>(floorf(maxx)) + radius + 1;  // inclusive
  const int lo_y = static_cast<int>(floorf(miny)) - radius;
  const int hi_y = static_cast<int>(floorf(maxy)) + radius + 1;
  p.bx = lo_x >= 0 ? (lo_x & ~3) : -((-lo_x + 3) & ~3);  // 16-byte aligned x (TMA rule)
  p.by = lo_y;
  p.fits = (hi_x - p.bx < kBoxW) && (hi_y - p.by < kBoxH);
  p.interior = it.affine && minx >= valid_lo + 1.0f && maxx <= valid_hi_x - 1.0f && miny >= valid_lo + 1.0f &&
               maxy <= valid_hi_y - 1.0f;
  return p;
}

// The output rows of one thread in a 64 x 48 tile (rows ly, ly + 4, ...).
// FINITE: the source frame holds no non-finite sample (every Lanczos3 window
// takes the plain normalised sum); returns the count of non-finite outputs.
template <int INTERP, bool FINITE>
__device__ __forceinline__ unsigned warp_tile_rows(const WarpArgs& a, const Coef& co, const TapSource& ts, float* dst,
                                                   int tile_x, int tile_y, int lx, int ly, bool interior,
                                                   bool int_shift) {
  constexpr int radius = (INTERP == GG_INTERP_LANCZOS3) ? 3 : 1;
  const int ox = tile_x * kTileW + lx;
  unsigned bad = 0;
  // Affine source coordinates step by 4 output rows: (sx, sy) += 4 (b, e)
  // in float-float (exact scaling by 4, one TwoSum per axis), with a fresh
  // evaluation every kFreshRows rows.
  FFv sx_row{0.0f, 0.0f}, sy_row{0.0f, 0.0f};
  bool row_ok = false;
  const float step_x_hi = 4.0f * co.m[1][0], step_x_lo = 4.0f * co.m[1][1];
  const float step_y_hi = 4.0f * co.m[4][0], step_y_lo = 4.0f * co.m[4][1];
#pragma unroll 1
  for (int r = 0; r < kRowsPerThread; ++r) {
    const int oy = tile_y * kTileH + ly + 4 * r;
    const bool inside = ox < a.width && oy < a.height;
    bool valid = false;
    float value = a.fill;
    if (co.affine) {
      if (r % kFreshRows == 0) {
        row_ok = source_coord(co, static_cast<float>(ox), static_cast<float>(oy), sx_row, sy_row);
      } else {
        sx_row = ff_add_ff(sx_row, step_x_hi, step_x_lo);
        sy_row = ff_add_ff(sy_row, step_y_hi, step_y_lo);
      }
    }
    if (inside) {
      FFv sx = sx_row, sy = sy_row;
      if (co.affine ? row_ok : source_coord(co, static_cast<float>(ox), static_cast<float>(oy), sx, sy)) {
        const float W = static_cast<float>(a.width), H = static_cast<float>(a.height);
        if (interior)
          valid = true;
        else if (INTERP != GG_INTERP_LANCZOS3)
          valid = ff_ge(sx, 0.0f) && ff_le(sx, W - 1.0f) && ff_ge(sy, 0.0f) && ff_le(sy, H - 1.0f);
        else
          valid = ff_ge(sx, 2.0f) && ff_lt(sx, W - 3.0f) && ff_ge(sy, 2.0f) && ff_lt(sy, H - 3.0f);
        if (valid) {
          int x0, y0;
          float tx, ty;
          ff_floor_frac(sx, x0, tx);
          ff_floor_frac(sy, y0, ty);
          if (INTERP == GG_INTERP_NEAREST) {
            // np.rint: round half to even (engine/warp.py:87-96).
            if (tx > 0.5f || (tx == 0.5f && (x0 & 1))) ++x0;
            if (ty > 0.5f || (ty == 0.5f && (y0 & 1))) ++y0;
          }
          TapSource src = ts;
          // Any tap outside the staged box reads global memory instead
          // (an affine tile that fits the box keeps every tap inside it).
          if (src.tile && !co.affine &&
              (x0 - (radius - 1) < src.bx || x0 + radius >= src.bx + kBoxW || y0 - (radius - 1) < src.by ||
               y0 + radius >= src.by + kBoxH))
            src.tile = nullptr;
          if (INTERP == GG_INTERP_NEAREST) {
            value = src.at(x0, y0);
          } else if (INTERP == GG_INTERP_BILINEAR) {
            value = sample_bilinear(src, x0, y0, tx, ty, a.width, a.height);
          } else if (int_shift) {
            // exact weights 0, 0, 1, 0, 0, 0: the source sample itself, or
            // no sample when it is not finite (nothing left to normalise)
            value = src.at(x0, y0);
            if (!isfinite(value)) {
              valid = false;
              value = a.fill;
            }
          } else {
            valid = FINITE ? sample_lanczos3_finite(src, x0, y0, tx, ty, a.clamp, value)
                           : sample_lanczos3(src, x0, y0, tx, ty, false, a.clamp, value);
            if (!valid) value = a.fill;
          }
        }
      }
      dst[static_cast<int64_t>(oy) * a.width + ox] = value;
      if (a.coverage && valid) atomicAdd(a.coverage + static_cast<int64_t>(oy) * a.width + ox, 1.0f);
      bad += isfinite(value) ? 0u : 1u;
    }
  }
  return bad;
}

// The common Lanczos3 tile in straight-line form: an affine map, the whole
// 64 x 48 tile inside the output and mapped at least one pixel inside the
// valid source range, its footprint staged in the shared-memory box, a source
// frame without non-finite samples, no clamp and no coverage map.  Every
// pixel is then valid and takes the plain normalised 6 x 6 sum, so the rows
// need no per-pixel tests (same arithmetic as the general path).
__device__ __forceinline__ unsigned warp_tile_rows_fast(const WarpArgs& a, const Coef& co, const float* box, int bx,
                                                        int by, float* dst, int ox, int oy0) {
  FFv sx, sy;
  const float step_x_hi = 4.0f * co.m[1][0], step_x_lo = 4.0f * co.m[1][1];
  const float step_y_hi = 4.0f * co.m[4][0], step_y_lo = 4.0f * co.m[4][1];
  float* out = dst + static_cast<int64_t>(oy0) * a.width + ox;
  const int64_t out_step = 4 * static_cast<int64_t>(a.width);
  unsigned bad = 0;
#pragma unroll 1
  for (int r = 0; r < kRowsPerThread; ++r) {
    if (r % kFreshRows == 0) {
      source_coord(co, static_cast<float>(ox), static_cast<float>(oy0 + 4 * r), sx, sy);
    } else {
      sx = ff_add_ff(sx, step_x_hi, step_x_lo);
      sy = ff_add_ff(sy, step_y_hi, step_y_lo);
    }
    int x0, y0;
    float tx, ty;
    ff_floor_frac(sx, x0, tx);
    ff_floor_frac(sy, y0, ty);
    float wx[6], wy[6];
    lanczos3_weights(tx, wx);
    lanczos3_weights(ty, wy);
    float swx = 0.0f, swy = 0.0f;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      swx += wx[i];
      swy += wy[i];
    }
    const float* r0 = box + (y0 - 2 - by) * kBoxW + (x0 - 2 - bx);
    float acc = 0.0f;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      float row = 0.0f;
#pragma unroll
      for (int i = 0; i < 6; ++i) row = __fmaf_rn(wx[i], r0[j * kBoxW + i], row);
      acc = __fmaf_rn(wy[j], row, acc);
    }
    const float wsum = swx * swy;
    const float value = fabsf(wsum) > 1.0e-12f ? __fdividef(acc, wsum) : a.fill;
    out[r * out_step] = value;
    bad += isfinite(value) ? 0u : 1u;
  }
  return bad;
}

template <int INTERP, bool USE_TMA>
__global__ void __launch_bounds__(kWarpThreads, 3) warp_tiles_kernel(const __grid_constant__ CUtensorMap tmap,
                                                                  WarpArgs a) {
  __shared__ alignas(128) float tile[2][kBoxH * kBoxW];
  __shared__ alignas(8) uint64_t bar[2];
  __shared__ int s_bx[2], s_by[2], s_fit[2], s_interior[2];
  __shared__ int s_abort;
  constexpr int radius = (INTERP == GG_INTERP_LANCZOS3) ? 3 : 1;
  const int tid = threadIdx.x;
  const int lx = tid & 63, ly = tid >> 6;
  const int tiles = a.tiles_x * a.tiles_y;
  const int items = a.item_count * tiles;
  if (tid == 0) {
    s_abort = 0;
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  auto issue = [&](int item, int buf) {
    // thread 0 only
    const WarpItem* ip = a.items + item / tiles;
    const int t = item % tiles;
    // validity ranges: bilinear 0 <= s <= W - 1; Lanczos3 2 <= s < W - 3
    const float vlo = INTERP == GG_INTERP_LANCZOS3 ? 2.0f : 0.0f;
    const float vhx = static_cast<float>(a.width) - (INTERP == GG_INTERP_LANCZOS3 ? 3.0f : 1.0f);
    const float vhy = static_cast<float>(a.height) - (INTERP == GG_INTERP_LANCZOS3 ? 3.0f : 1.0f);
    TilePlan p = plan_tile(load_coef(ip), t % a.tiles_x, t / a.tiles_x, radius, vlo, vhx, vhy);
    if (!USE_TMA) p.fits = 0;
    s_interior[buf] = p.interior;
    s_bx[buf] = p.bx;
    s_by[buf] = p.by;
    s_fit[buf] = p.fits;
    if (p.fits) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_expect_tx(&bar[buf], kBoxW * kBoxH * 4);
      tma_load_3d(tile[buf], &tmap, p.bx, p.by, __ldg(&ip->src_slot), &bar[buf]);
    }
  };

  unsigned phase[2] = {0u, 0u};
  int item = blockIdx.x;
  if (tid == 0 && item < items) issue(item, 0);
  __syncthreads();
  for (int i = 0; item < items; ++i, item += gridDim.x) {
    const int buf = i & 1;
    const int next = item + gridDim.x;
    if (tid == 0 && next < items) issue(next, buf ^ 1);
    const int item_index = item / tiles;
    const WarpItem* ip = a.items + item_index;
    const Coef co = load_coef(ip);
    const int it_frame = __ldg(&ip->frame);
    const int it_src = __ldg(&ip->src_slot);
    const int it_dst = __ldg(&ip->dst_slot);
    const unsigned it_nonfinite = __ldg(&ip->src_nonfinite);
    const bool int_shift = __ldg(&ip->int_shift) != 0;
    const int t = item - item_index * tiles;
    const int tile_x = t % a.tiles_x, tile_y = t / a.tiles_x;
    const bool fit = s_fit[buf] != 0;
    const bool interior = s_interior[buf] != 0;
    if (fit) {
      // Bounded wait: on expiry flag the error, give the copy one more
      // bounded wait to land, finish this item (its output is discarded by
      // the host) and leave the loop with the whole CTA.
      if (!mbar_wait_bounded(&bar[buf], phase[buf], 1 << 24)) {
        atomicExch(a.error, 1);
        s_abort = 1;
        mbar_wait_bounded(&bar[buf], phase[buf], 1 << 24);
      }
      phase[buf] ^= 1u;
    }
    {
      TapSource ts;
      ts.tile = fit ? tile[buf] : nullptr;
      ts.src = a.slots + static_cast<int64_t>(it_src) * a.stride;
      ts.bx = s_bx[buf];
      ts.by = s_by[buf];
      ts.width = a.width;
      float* dst = a.slots + static_cast<int64_t>(it_dst) * a.stride;
      // the renormalising path (and its out-of-line call) only for frames
      // that hold non-finite samples; the straight-line form for the common
      // interior tile
      const bool full_tile = (tile_x + 1) * kTileW <= a.width && (tile_y + 1) * kTileH <= a.height;
      unsigned bad;
      if (INTERP == GG_INTERP_LANCZOS3 && fit && interior && co.affine && it_nonfinite == 0u && !int_shift &&
          a.clamp < 0.0f && a.coverage == nullptr && full_tile)
        bad = warp_tile_rows_fast(a, co, ts.tile, ts.bx, ts.by, dst, tile_x * kTileW + lx, tile_y * kTileH + ly);
      else if (INTERP == GG_INTERP_LANCZOS3 && it_nonfinite == 0u)
        bad = warp_tile_rows<INTERP, true>(a, co, ts, dst, tile_x, tile_y, lx, ly, interior, int_shift);
      else
        bad = warp_tile_rows<INTERP, false>(a, co, ts, dst, tile_x, tile_y, lx, ly, interior, int_shift);
      const unsigned warp_bad = __reduce_add_sync(0xffffffffu, bad);
      if ((tid & 31) == 0 && warp_bad) atomicAdd(a.nonfinite + it_frame, warp_bad);
    }
    __syncthreads();
    if (s_abort) {
      // Let the prefetch already issued for the next item land before exit.
      if (next < items && s_fit[buf ^ 1]) mbar_wait_bounded(&bar[buf ^ 1], phase[buf ^ 1], 1 << 24);
      break;
    }
  }
}

// Resolve slots for the batch and move the source non-finite counts aside.
__global__ void warp_prepare_kernel(WarpItem* items, int count, const int* slot_of_frame, const int* spare,
                                    unsigned* nonfinite) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const int f = items[k].frame;
  items[k].src_slot = slot_of_frame[f];
  items[k].dst_slot = spare[k];
  items[k].src_nonfinite = nonfinite[f];
  nonfinite[f] = 0u;
}

// The warped frame now lives in the spare slot; the old slot becomes spare.
__global__ void warp_finish_kernel(const WarpItem* items, int count, int* slot_of_frame, int* spare) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  slot_of_frame[items[k].frame] = items[k].dst_slot;
  spare[k] = items[k].src_slot;
}

__global__ void fill_kernel(float* p, int64_t n, float v) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    p[i] = v;
}

__global__ void add_scalar_kernel(float* p, int64_t n, float v) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    p[i] += v;
}

// ---- host side -------------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    else
      cudaGetLastError();
  }
  return fn;
}

bool make_slot_tensor_map(gg_stack* s, int box_w, int box_h) {
  auto fn = encode_fn();
  if (!fn) return false;
  if ((s->width * 4) % 16 != 0 || (s->stride * 4) % 16 != 0) return false;
  const cuuint64_t dims[3] = {static_cast<cuuint64_t>(s->width), static_cast<cuuint64_t>(s->height),
                              static_cast<cuuint64_t>(s->slots)};
  const cuuint64_t strides[2] = {static_cast<cuuint64_t>(s->width) * 4, static_cast<cuuint64_t>(s->stride) * 4};
  const cuuint32_t box[3] = {static_cast<cuuint32_t>(box_w), static_cast<cuuint32_t>(box_h), 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  std::memset(&s->slot_tmap, 0, sizeof(s->slot_tmap));
  const CUresult r = fn(&s->slot_tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, s->d_slots, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// float64 3x3 inverse (np.linalg.inv of the float32 matrix promoted to float64).
static void ensure_warp_items(gg_stack* s, int64_t count) {
  if (s->warp_item_capacity >= count) return;
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(warp items)");
  if (s->d_warp_items) cudaFree(s->d_warp_items);
  if (s->h_warp_items) cudaFreeHost(s->h_warp_items);
  s->d_warp_items = nullptr;
  s->h_warp_items = nullptr;
  const size_t bytes = sizeof(WarpItem) * static_cast<size_t>(count);
  check_cuda(cudaMalloc(&s->d_warp_items, bytes), "cudaMalloc(warp items)");
  check_cuda(cudaHostAlloc(&s->h_warp_items, bytes, cudaHostAllocPortable), "cudaHostAlloc(warp items)");
  s->warp_item_capacity = count;
}

static void ensure_warp_coverage(gg_stack* s) {
  if (s->d_warp_coverage) return;
  check_cuda(cudaMalloc(reinterpret_cast<void**>(&s->d_warp_coverage), sizeof(float) * s->pixels),
             "cudaMalloc(warp coverage)");
  s->bytes_allocated += static_cast<int64_t>(sizeof(float) * s->pixels);
  check_cuda(cudaMemsetAsync(s->d_warp_coverage, 0, sizeof(float) * s->pixels, s->stream), "cudaMemsetAsync");
}

template <int INTERP>
static void launch_warp_tiles(gg_stack* s, const WarpArgs& args, bool use_tma) {
  int per_sm = 0;
  auto kern = use_tma ? warp_tiles_kernel<INTERP, true> : warp_tiles_kernel<INTERP, false>;
  check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWarpThreads, 0), "occupancy(warp)");
  const int64_t items = static_cast<int64_t>(args.item_count) * args.tiles_x * args.tiles_y;
  const unsigned grid =
      static_cast<unsigned>(std::min<int64_t>(items, static_cast<int64_t>(sm_count()) * std::max(per_sm, 1)));
  note_launch();
  kern<<<grid, kWarpThreads, 0, s->stream>>>(s->slot_tmap, args);
  check_cuda(cudaGetLastError(), "warp kernel launch");
}

// Host descriptors of a warp batch (validated; inverse coefficients).
static std::vector<WarpItem> warp_items_host(gg_stack* s, const int64_t* indices, int64_t count, const double* fwd) {
  std::vector<WarpItem> items(static_cast<size_t>(count));
  for (int64_t k = 0; k < count; ++k) {
    stack_require_loaded(s, indices[k], "warp");
    for (int64_t j = 0; j < k; ++j)
      if (indices[j] == indices[k]) fail(GG_ERR_INVALID_ARGUMENT, "frame indices of a warp batch must be unique");
    const double* m = fwd + 9 * k;
    for (int q = 0; q < 9; ++q)
      if (!std::isfinite(m[q])) fail(GG_ERR_INVALID_ARGUMENT, "warp matrix must be finite");
    WarpItem& it = items[static_cast<size_t>(k)];
    std::memset(&it, 0, sizeof(it));
    it.frame = static_cast<int>(indices[k]);
    if (!inverse_coefficients(m, it.m, it.affine)) fail(GG_ERR_INVALID_ARGUMENT, "warp matrix is singular");
    // an exact integer translation (identity linear part, integer shifts):
    // its inverse is one too and every source coordinate is an integer
    it.int_shift = (m[0] == 1.0 && m[1] == 0.0 && m[3] == 0.0 && m[4] == 1.0 && m[6] == 0.0 && m[7] == 0.0 &&
                    m[8] == 1.0 && m[2] == std::floor(m[2]) && m[5] == std::floor(m[5]) && std::fabs(m[2]) < 1.0e7 &&
                    std::fabs(m[5]) < 1.0e7)
                       ? 1
                       : 0;
  }
  return items;
}

// The kernels of a warp batch whose descriptors are already in device
// memory (d_items, `count` of them): per group of at most `spares` frames,
// resolve slots, warp into the spare slots, swap the slot table.  Only
// launches on the stack's stream (safe inside a stream capture).
static void launch_warp_items(gg_stack* s, WarpItem* d_items, int64_t count, int interp, float fill, float clamp,
                              bool track_coverage) {
  const bool use_tma = s->has_slot_tmap;
  for (int64_t k0 = 0; k0 < count; k0 += s->spares) {
    const int nb = static_cast<int>(std::min<int64_t>(s->spares, count - k0));
    note_launch();
    warp_prepare_kernel<<<(nb + 127) / 128, 128, 0, s->stream>>>(d_items + k0, nb, s->d_slot_of_frame,
                                                                 s->d_spare_slot, s->d_frame_nonfinite);
    check_cuda(cudaGetLastError(), "warp_prepare launch");
    WarpArgs a{};
    a.slots = s->d_slots;
    a.slot_of_frame = s->d_slot_of_frame;
    a.spare_slot = s->d_spare_slot;
    a.nonfinite = s->d_frame_nonfinite;
    a.items = d_items + k0;
    a.item_count = nb;
    a.stride = s->stride;
    a.width = static_cast<int>(s->width);
    a.height = static_cast<int>(s->height);
    a.tiles_x = static_cast<int>((s->width + kTileW - 1) / kTileW);
    a.tiles_y = static_cast<int>((s->height + kTileH - 1) / kTileH);
    a.interp = interp;
    a.fill = fill;
    a.clamp = clamp;
    a.coverage = track_coverage ? s->d_warp_coverage : nullptr;
    a.error = s->d_error;
    if (interp == GG_INTERP_NEAREST)
      launch_warp_tiles<GG_INTERP_NEAREST>(s, a, use_tma);
    else if (interp == GG_INTERP_BILINEAR)
      launch_warp_tiles<GG_INTERP_BILINEAR>(s, a, use_tma);
    else
      launch_warp_tiles<GG_INTERP_LANCZOS3>(s, a, use_tma);
    note_launch();
    warp_finish_kernel<<<(nb + 127) / 128, 128, 0, s->stream>>>(d_items + k0, nb, s->d_slot_of_frame,
                                                                s->d_spare_slot);
    check_cuda(cudaGetLastError(), "warp_finish launch");
  }
}

void warp_frames(gg_stack* s, const int64_t* indices, int64_t count, const double* fwd, int interp, float fill,
                 float clamp, bool track_coverage) {
  const std::vector<WarpItem> items = warp_items_host(s, indices, count, fwd);
  ensure_warp_items(s, std::max<int64_t>(count, s->spares));
  if (track_coverage) ensure_warp_coverage(s);
  // The staging buffer may still feed the previous call's copy.
  check_cuda(cudaEventSynchronize(s->warp_items_free), "cudaEventSynchronize(warp items)");
  std::memcpy(s->h_warp_items, items.data(), sizeof(WarpItem) * items.size());
  upload_params(s->stream, s->d_warp_items, s->h_warp_items, sizeof(WarpItem) * items.size(),
                "cudaMemcpyAsync(warp items)");
  check_cuda(cudaEventRecord(s->warp_items_free, s->stream), "cudaEventRecord(warp items)");
  launch_warp_items(s, static_cast<WarpItem*>(s->d_warp_items), count, interp, fill, clamp, track_coverage);
  if (track_coverage) s->warp_coverage_frames += count;
}

// Warp descriptors in a caller-owned device buffer (for captured graphs):
// returns the device pointer (cudaMalloc, the caller frees it with cudaFree)
// and their count through `count_out`.
void* warp_items_device(gg_stack* s, const int64_t* indices, int64_t count, const double* fwd) {
  const std::vector<WarpItem> items = warp_items_host(s, indices, count, fwd);
  void* d = nullptr;
  check_cuda(cudaMalloc(&d, sizeof(WarpItem) * items.size()), "cudaMalloc(graph warp items)");
  const cudaError_t err = cudaMemcpy(d, items.data(), sizeof(WarpItem) * items.size(), cudaMemcpyHostToDevice);
  if (err != cudaSuccess) {
    cudaFree(d);
    check_cuda(err, "cudaMemcpy(graph warp items)");
  }
  return d;
}

void launch_warp_items_device(gg_stack* s, void* d_items, int64_t count, int interp, float fill, float clamp) {
  launch_warp_items(s, static_cast<WarpItem*>(d_items), count, interp, fill, clamp, false);
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_stack_warp_frames(gg_stack* s, const int64_t* indices, int64_t count, const double* host_matrices,
                         int interpolation, float fill, float clamping_threshold, int track_coverage) {
  GG_API_BEGIN
  require(s != nullptr && indices != nullptr && host_matrices != nullptr, "null argument");
  require(count > 0, "indices must contain at least one frame index");
  require(interpolation == GG_INTERP_NEAREST || interpolation == GG_INTERP_BILINEAR ||
              interpolation == GG_INTERP_LANCZOS3,
          "interpolation must be nearest, bilinear or lanczos3");
  require(s->width < (1 << 24) && s->height < (1 << 24), "frame too large for float coordinates");
  stack_activate(s);
  warp_frames(s, indices, count, host_matrices, interpolation, fill, clamping_threshold, track_coverage != 0);
  GG_API_END
}

int gg_stack_reset_warp_coverage(gg_stack* s) {
  GG_API_BEGIN
  require(s != nullptr, "stack is null");
  stack_activate(s);
  ensure_warp_coverage(s);
  check_cuda(cudaMemsetAsync(s->d_warp_coverage, 0, sizeof(float) * s->pixels, s->stream), "cudaMemsetAsync");
  s->warp_coverage_frames = 0;
  GG_API_END
}

int gg_stack_accumulate_full_warp_coverage_frame(gg_stack* s) {
  GG_API_BEGIN
  require(s != nullptr, "stack is null");
  stack_activate(s);
  ensure_warp_coverage(s);
  note_launch();
  add_scalar_kernel<<<grid_for(static_cast<size_t>(s->pixels), 256, 4), 256, 0, s->stream>>>(s->d_warp_coverage,
                                                                                            s->pixels, 1.0f);
  check_cuda(cudaGetLastError(), "add_scalar launch");
  s->warp_coverage_frames += 1;
  GG_API_END
}

int gg_stack_download_warp_coverage(gg_stack* s, float* host_out) {
  GG_API_BEGIN
  require(s != nullptr && host_out != nullptr, "null argument");
  stack_activate(s);
  ensure_warp_coverage(s);
  check_cuda(cudaMemcpyAsync(host_out, s->d_warp_coverage, sizeof(float) * s->pixels, cudaMemcpyDeviceToHost,
                             s->stream),
             "cudaMemcpyAsync(warp coverage)");
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(warp coverage)");
  stack_check_device_error(s);
  GG_API_END
}

int gg_stack_tma_enabled(gg_stack* s, int* enabled) {
  GG_API_BEGIN
  require(s != nullptr && enabled != nullptr, "null argument");
  *enabled = s->has_slot_tmap ? 1 : 0;
  GG_API_END
}

int gg_warp_matrix_f32(const float* host_in, int64_t height, int64_t width, const double* host_matrix,
                       int interpolation, float fill, float clamping_threshold, float* host_out,
                       float* host_coverage) {
  GG_API_BEGIN
  require(host_in != nullptr && host_matrix != nullptr && host_out != nullptr, "null argument");
  gg_stack* s = nullptr;
  int rc = gg_stack_create(1, height, width, &s);
  if (rc != GG_OK) fail(rc, "temporary stack: create failed");
  struct Guard {
    gg_stack* s;
    ~Guard() { gg_stack_destroy(s); }
  } guard{s};
  rc = gg_stack_upload_frame(s, 0, host_in);
  if (rc != GG_OK) fail(rc, "temporary stack: upload failed");
  const int64_t idx = 0;
  if (host_coverage) {
    rc = gg_stack_reset_warp_coverage(s);
    if (rc != GG_OK) fail(rc, "temporary stack: coverage reset failed");
  }
  warp_frames(s, &idx, 1, host_matrix, interpolation, fill, clamping_threshold, host_coverage != nullptr);
  rc = gg_stack_download_frame_tile(s, 0, 0, 0, width, height, host_out);
  if (rc != GG_OK) fail(rc, "temporary stack: download failed");
  if (host_coverage) {
    rc = gg_stack_download_warp_coverage(s, host_coverage);
    if (rc != GG_OK) fail(rc, "temporary stack: coverage download failed");
  }
  GG_API_END
}

}  // extern "C"
