// Affine warp of one device image and its adjoint (reverse-mode derivative)
// with respect to the source image and the six affine parameters.
//
// The forward is the warp of warp_tiles_kernel (engine/warp.py:99-152
// semantics; bilinear or Lanczos3 without the overshoot clamp): output pixel
// (x, y) samples the source at (sx, sy) = (t0 x + t1 y + t2, t3 x + t4 y + t5),
// where t are the parameters of the inverse (output -> source) map.
//
// Adjoint, per output pixel with incoming gradient g (zero where the sample
// is invalid or the loss ignores it):
//   bilinear   O = sum_ij wx_i wy_j S_ij, dO/dtx = (1-ty)(S01-S00) + ty(S11-S10),
//              dO/dty = ((1-tx)S10 + tx S11) - ((1-tx)S00 + tx S01);
//   Lanczos3   O = N / D over the finite taps, N = sum wx_i wy_j S_ij,
//              D = sum wx_i wy_j; dO/dtx = (N_x - O D_x) / D with N_x, D_x
//              the same sums with wx replaced by its derivative w'(t - k);
//   grad S_ij += g * wx_i wy_j / D            (scatter, float atomics);
//   grad t    += g * (dO/dsx (x, y, 1), dO/dsy (x, y, 1)).
// Weights and their derivatives are recomputed, never stored.
// w(d) = sinc(d) sinc(d/3), w'(d) = f'(d) g(d) + f(d) g'(d) with
// f(d) = sin(pi d)/(pi d), g(d) = f(d/3), f'(d) = pi (cos(pi d) pi d - sin(pi d)) / (pi d)^2.
#include <cmath>
#include <cstring>

#include "adjoint.cuh"
#include "stack.cuh"

namespace gg {

struct AdjointArgs {
  const float* src;
  float* out;
  const float* grad_out;
  float* grad_src;
  double* partials;  // [blocks][6]
  AffineCoef coef;
  int width, height;
  float fill;
  int src_finite;
};

__device__ __forceinline__ bool sample_coords(const AdjointArgs& a, int x, int y, int interp, int& x0, int& y0,
                                              float& tx, float& ty) {
  FFv sx, sy;
  if (!source_coord(a.coef, static_cast<float>(x), static_cast<float>(y), sx, sy)) return false;
  const float W = static_cast<float>(a.width), H = static_cast<float>(a.height);
  const bool valid = interp == GG_INTERP_BILINEAR
                         ? (ff_ge(sx, 0.0f) && ff_le(sx, W - 1.0f) && ff_ge(sy, 0.0f) && ff_le(sy, H - 1.0f))
                         : (ff_ge(sx, 2.0f) && ff_lt(sx, W - 3.0f) && ff_ge(sy, 2.0f) && ff_lt(sy, H - 3.0f));
  if (!valid) return false;
  ff_floor_frac(sx, x0, tx);
  ff_floor_frac(sy, y0, ty);
  return true;
}

template <int INTERP>
__global__ void __launch_bounds__(256) affine_forward_kernel(AdjointArgs a) {
  const int64_t P = static_cast<int64_t>(a.width) * a.height;
  for (int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; p < P; p += int64_t(gridDim.x) * blockDim.x) {
    const int y = static_cast<int>(p / a.width), x = static_cast<int>(p - static_cast<int64_t>(y) * a.width);
    int x0, y0;
    float tx, ty;
    float v = a.fill;
    if (sample_coords(a, x, y, INTERP, x0, y0, tx, ty)) {
      TapSource ts;
      ts.tile = nullptr;
      ts.src = a.src;
      ts.bx = ts.by = 0;
      ts.width = a.width;
      if (INTERP == GG_INTERP_BILINEAR) {
        v = sample_bilinear(ts, x0, y0, tx, ty, a.width, a.height);
      } else if (!sample_lanczos3(ts, x0, y0, tx, ty, a.src_finite != 0, -1.0f, v)) {
        v = a.fill;
      }
    }
    a.out[p] = v;
  }
}

template <int INTERP>
__global__ void __launch_bounds__(256) affine_backward_kernel(AdjointArgs a) {
  __shared__ double red[8][6];
  const int64_t P = static_cast<int64_t>(a.width) * a.height;
  float acc[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
  const int W = a.width;
  for (int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; p < P; p += int64_t(gridDim.x) * blockDim.x) {
    const float g = a.grad_out[p];
    if (!(g != 0.0f) || !isfinite(g)) continue;
    const int y = static_cast<int>(p / W), x = static_cast<int>(p - static_cast<int64_t>(y) * W);
    int x0, y0;
    float tx, ty;
    if (!sample_coords(a, x, y, INTERP, x0, y0, tx, ty)) continue;
    float gsx = 0.0f, gsy = 0.0f;  // g * dO/dsx, g * dO/dsy
    if (INTERP == GG_INTERP_BILINEAR) {
      const int x1 = min(x0 + 1, W - 1), y1 = min(y0 + 1, a.height - 1);
      const float s00 = __ldg(a.src + static_cast<int64_t>(y0) * W + x0);
      const float s01 = __ldg(a.src + static_cast<int64_t>(y0) * W + x1);
      const float s10 = __ldg(a.src + static_cast<int64_t>(y1) * W + x0);
      const float s11 = __ldg(a.src + static_cast<int64_t>(y1) * W + x1);
      if (!(isfinite(s00) && isfinite(s01) && isfinite(s10) && isfinite(s11))) continue;  // NaN output
      const float ox = 1.0f - tx, oy = 1.0f - ty;
      gsx = g * (oy * (s01 - s00) + ty * (s11 - s10));
      gsy = g * ((ox * s10 + tx * s11) - (ox * s00 + tx * s01));
      if (a.grad_src) {
        atomicAdd(a.grad_src + static_cast<int64_t>(y0) * W + x0, g * ox * oy);
        atomicAdd(a.grad_src + static_cast<int64_t>(y0) * W + x1, g * tx * oy);
        atomicAdd(a.grad_src + static_cast<int64_t>(y1) * W + x0, g * ox * ty);
        atomicAdd(a.grad_src + static_cast<int64_t>(y1) * W + x1, g * tx * ty);
      }
    } else if (float Os, Osx, Osy;
               !a.grad_src && lanczos3_value_grad<true>(a.src, W, x0, y0, tx, ty, Os, Osx, Osy)) {
      // parameter gradient only over a window of finite taps: the separable
      // sums with the warp's polynomial weights and their exact derivatives
      gsx = g * Osx;
      gsy = g * Osy;
    } else {
      // source gradient, or non-finite taps (renormalised over the finite ones)
      float wx[6], wy[6], dwx[6], dwy[6];
      lanczos3_weights_grad(tx, wx, dwx);
      lanczos3_weights_grad(ty, wy, dwy);
      float N = 0.0f, D = 0.0f, Nx = 0.0f, Dx = 0.0f, Ny = 0.0f, Dy = 0.0f;
      for (int j = 0; j < 6; ++j) {
        const float* row = a.src + static_cast<int64_t>(y0 - 2 + j) * W + (x0 - 2);
#pragma unroll
        for (int i = 0; i < 6; ++i) {
          const float v = __ldg(row + i);
          if (!isfinite(v)) continue;
          const float w = wx[i] * wy[j], wxd = dwx[i] * wy[j], wyd = wx[i] * dwy[j];
          N = __fmaf_rn(w, v, N);
          D += w;
          Nx = __fmaf_rn(wxd, v, Nx);
          Dx += wxd;
          Ny = __fmaf_rn(wyd, v, Ny);
          Dy += wyd;
        }
      }
      if (!(fabsf(D) > 1.0e-12f)) continue;  // invalid sample
      const float O = N / D;
      gsx = g * (Nx - O * Dx) / D;
      gsy = g * (Ny - O * Dy) / D;
      if (a.grad_src) {
        const float gd = g / D;
        for (int j = 0; j < 6; ++j) {
          float* grow = a.grad_src + static_cast<int64_t>(y0 - 2 + j) * W + (x0 - 2);
          const float* row = a.src + static_cast<int64_t>(y0 - 2 + j) * W + (x0 - 2);
#pragma unroll
          for (int i = 0; i < 6; ++i)
            if (isfinite(__ldg(row + i))) atomicAdd(grow + i, gd * wx[i] * wy[j]);
        }
      }
    }
    const float xf = static_cast<float>(x), yf = static_cast<float>(y);
    acc[0] = __fmaf_rn(gsx, xf, acc[0]);
    acc[1] = __fmaf_rn(gsx, yf, acc[1]);
    acc[2] += gsx;
    acc[3] = __fmaf_rn(gsy, xf, acc[3]);
    acc[4] = __fmaf_rn(gsy, yf, acc[4]);
    acc[5] += gsy;
  }
  // block reduction in float64
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double d[6];
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    d[q] = static_cast<double>(acc[q]);
    for (int off = 16; off > 0; off >>= 1) d[q] += __shfl_xor_sync(0xffffffffu, d[q], off);
  }
  if (lane == 0)
    for (int q = 0; q < 6; ++q) red[warp][q] = d[q];
  __syncthreads();
  if (threadIdx.x < 6) {
    double s = 0.0;
    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) s += red[w][threadIdx.x];
    a.partials[static_cast<int64_t>(blockIdx.x) * 6 + threadIdx.x] = s;
  }
}

__global__ void affine_reduce_kernel(const double* partials, int blocks, double* grad_theta) {
  const int q = threadIdx.x;
  if (q >= 6) return;
  double s = 0.0;
  for (int b = 0; b < blocks; ++b) s += partials[static_cast<int64_t>(b) * 6 + q];
  grad_theta[q] = s;
}

static AffineCoef affine_coef(const double* theta) {
  for (int q = 0; q < 6; ++q) require(std::isfinite(theta[q]), "affine parameters must be finite");
  return affine_coef_from(theta);
}

static unsigned affine_grid(int64_t pixels) {
  return static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>((pixels + 255) / 256, sm_count() * 8)));
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_warp_affine_f32_device(const float* dev_src, int64_t height, int64_t width, const double* host_theta,
                              int interpolation, float fill, int src_all_finite, float* dev_out,
                              void* cuda_stream) {
  GG_API_BEGIN
  require(dev_src != nullptr && dev_out != nullptr && host_theta != nullptr, "null argument");
  require(height > 0 && width > 0 && height * width < (int64_t{1} << 31), "invalid image shape");
  require(interpolation == GG_INTERP_BILINEAR || interpolation == GG_INTERP_LANCZOS3,
          "interpolation must be bilinear or lanczos3");
  AdjointArgs a{};
  a.src = dev_src;
  a.out = dev_out;
  a.coef = affine_coef(host_theta);
  a.width = static_cast<int>(width);
  a.height = static_cast<int>(height);
  a.fill = fill;
  a.src_finite = src_all_finite;
  auto stream = static_cast<cudaStream_t>(cuda_stream);
  note_launch();
  if (interpolation == GG_INTERP_BILINEAR)
    affine_forward_kernel<GG_INTERP_BILINEAR><<<affine_grid(height * width), 256, 0, stream>>>(a);
  else
    affine_forward_kernel<GG_INTERP_LANCZOS3><<<affine_grid(height * width), 256, 0, stream>>>(a);
  check_cuda(cudaGetLastError(), "affine_forward launch");
  GG_API_END
}

int gg_warp_affine_backward_f32_device(const float* dev_src, int64_t height, int64_t width, const double* host_theta,
                                       int interpolation, const float* dev_grad_out, float* dev_grad_src,
                                       double* dev_grad_theta, void* cuda_stream) {
  GG_API_BEGIN
  require(dev_src != nullptr && dev_grad_out != nullptr && host_theta != nullptr, "null argument");
  require(height > 0 && width > 0 && height * width < (int64_t{1} << 31), "invalid image shape");
  require(interpolation == GG_INTERP_BILINEAR || interpolation == GG_INTERP_LANCZOS3,
          "interpolation must be bilinear or lanczos3");
  AdjointArgs a{};
  a.src = dev_src;
  a.grad_out = dev_grad_out;
  a.grad_src = dev_grad_src;
  a.coef = affine_coef(host_theta);
  a.width = static_cast<int>(width);
  a.height = static_cast<int>(height);
  auto stream = static_cast<cudaStream_t>(cuda_stream);
  const unsigned blocks = affine_grid(height * width);
  double* partials = nullptr;
  check_cuda(cudaMallocAsync(reinterpret_cast<void**>(&partials), sizeof(double) * 6 * blocks, stream),
             "cudaMallocAsync(adjoint partials)");
  a.partials = partials;
  note_launch();
  if (interpolation == GG_INTERP_BILINEAR)
    affine_backward_kernel<GG_INTERP_BILINEAR><<<blocks, 256, 0, stream>>>(a);
  else
    affine_backward_kernel<GG_INTERP_LANCZOS3><<<blocks, 256, 0, stream>>>(a);
  check_cuda(cudaGetLastError(), "affine_backward launch");
  if (dev_grad_theta) {
    note_launch();
    affine_reduce_kernel<<<1, 32, 0, stream>>>(partials, static_cast<int>(blocks), dev_grad_theta);
    check_cuda(cudaGetLastError(), "affine_reduce launch");
  }
  check_cuda(cudaFreeAsync(partials, stream), "cudaFreeAsync(adjoint partials)");
  GG_API_END
}

}  // extern "C"
