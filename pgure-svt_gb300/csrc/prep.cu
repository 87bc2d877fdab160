// prep.cu — input conversion, frame maxima and per-window normalisation.
//
// Reference: pguresvt.hpp:87 (conv_to<Cube<double>>), :100-120 (window slice
// [t-fw, t+fw] clamped at the sequence ends, divided by its maximum).
#include <algorithm>

#include "pgsvt_internal.h"

namespace pgsvt {

template <typename T>
__global__ void k_convert(const T* __restrict__ X, size_t n, float* __restrict__ xs,
                          double* __restrict__ x64) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (; i < n; i += stride) {
    const T v = X[i];
    xs[i] = (float)v;
    if (x64) x64[i] = (double)v;
  }
}

cudaError_t launch_convert(const void* X, int dtype, size_t n, float* xs, double* x64,
                           cudaStream_t s) {
  const int threads = 256;
  const int blocks = (int)std::min<size_t>((n + threads - 1) / threads, 152 * 16);
  switch (dtype) {
    case 0: k_convert<uint8_t><<<blocks, threads, 0, s>>>((const uint8_t*)X, n, xs, nullptr); break;
    case 1: k_convert<uint16_t><<<blocks, threads, 0, s>>>((const uint16_t*)X, n, xs, nullptr); break;
    case 2: k_convert<float><<<blocks, threads, 0, s>>>((const float*)X, n, xs, nullptr); break;
    default: k_convert<double><<<blocks, threads, 0, s>>>((const double*)X, n, xs, x64); break;
  }
  return cudaGetLastError();
}

// Per input frame: maximum (exact), a flag for negative / non-finite values
// and (fint, optional) whether every value is an integer <= 2^19.
__global__ void k_frame_max(const float* __restrict__ xs, const double* __restrict__ x64,
                            size_t F, double* __restrict__ fmx, int* __restrict__ fint) {
  const int f = blockIdx.x;
  double m = -INFINITY;
  bool bad = false, nonint = false;
  for (size_t i = threadIdx.x; i < F; i += blockDim.x) {
    const double v = x64 ? x64[f * F + i] : (double)xs[f * F + i];
    bad |= !(v >= 0.0) || isinf(v);  // NaN, negative or infinite
    nonint |= !(v <= 524288.0) || v != floor(v);
    m = fmax(m, v);
  }
  __shared__ double sm[32];
  __shared__ int sbad, snon;
  if (threadIdx.x == 0) {
    sbad = 0;
    snon = 0;
  }
  __syncthreads();
  if (bad) atomicOr(&sbad, 1);
  if (nonint) atomicOr(&snon, 1);
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = (threadIdx.x < blockDim.x / 32) ? sm[threadIdx.x] : -INFINITY;
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) {
      fmx[f] = sbad ? -1.0 : m;  // -1 marks an invalid frame
      if (fint) fint[f] = snon ? 0 : 1;
    }
  }
}

cudaError_t launch_frame_max(const float* xs, const double* x64, int nimg, size_t F,
                             double* fmax, cudaStream_t s, int* fint) {
  k_frame_max<<<nimg, 512, 0, s>>>(xs, x64, F, fmax, fint);
  return cudaGetLastError();
}

// ---- median pre-filter of the ARPS input (pguresvt.hpp:69-84)
//
// The reference converts each frame to uint16 (arma::conv_to; taken here as
// C's truncation toward zero, clamped to [0, 65535]) and filters it with
// ConstantTimeMedianFilter (medfilter.hpp:478-541) of radius r, which is the
// exact median of the (2r+1)^2 window with coordinates clamped to the frame.
// GB300 form: one thread per output pixel of a 32 x 8 tile, the tile and its
// halo staged in shared memory as uint16; the median is found by a 16-step
// binary search on the value (the largest v with #{x < v} <= n/2), each step
// one counting pass over the window.
__device__ __forceinline__ uint16_t to_u16(double v) {
  if (!(v > 0.0)) return 0;
  if (v >= 65535.0) return 65535;
  return (uint16_t)v;
}

template <bool F64>
__global__ void __launch_bounds__(256) k_median(const float* __restrict__ xs,
                                                const double* __restrict__ x64, int S, int r,
                                                float* __restrict__ zs) {
  extern __shared__ uint16_t tile[];
  const size_t base = (size_t)blockIdx.z * S * S;
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 8;  // x: the fast axis
  const int TW = 32 + 2 * r, TH = 8 + 2 * r;
  for (int i = threadIdx.x; i < TW * TH; i += blockDim.x) {
    const int gx = min(max(x0 + i % TW - r, 0), S - 1);
    const int gy = min(max(y0 + i / TW - r, 0), S - 1);
    const size_t k = base + gx + (size_t)gy * S;
    tile[i] = to_u16(F64 ? x64[k] : (double)xs[k]);
  }
  __syncthreads();
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  if (x0 + tx >= S || y0 + ty >= S) return;
  const int d = 2 * r + 1, half = (d * d) / 2;
  uint32_t ans = 0;
  for (int b = 15; b >= 0; --b) {
    const uint32_t cand = ans | (1u << b);
    int cnt = 0;
    for (int dy = 0; dy < d; ++dy) {
      const uint16_t* row = tile + (ty + dy) * TW + tx;
      for (int dx = 0; dx < d; ++dx) cnt += (uint32_t)row[dx] < cand;
    }
    if (cnt <= half) ans = cand;
  }
  zs[base + (x0 + tx) + (size_t)(y0 + ty) * S] = (float)ans;
}

cudaError_t launch_median(const float* xs, const double* x64, int nimg, int S, int r, float* zs,
                          cudaStream_t s) {
  if (r < 0 || r > kMaxMedian) return cudaErrorInvalidValue;
  const dim3 grid((S + 31) / 32, (S + 7) / 8, nimg);
  const size_t shm = (size_t)(32 + 2 * r) * (8 + 2 * r) * sizeof(uint16_t);
  if (x64) k_median<true><<<grid, 256, shm, s>>>(xs, x64, S, r, zs);
  else k_median<false><<<grid, 256, shm, s>>>(xs, x64, S, r, zs);
  return cudaGetLastError();
}

// Window constants and the normalised window u = x / umax.
__global__ void k_window_const(Problem pb, DeviceBuffers d) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= pb.W) return;
  const Geometry& g = pb.g;
  const int t = d.win0 + w;
  int s0;
  if (t < g.fw) s0 = 0;
  else if (t >= g.nimg - g.fw) s0 = g.nimg - 2 * g.fw - 1;
  else s0 = t - g.fw;
  double umax = d.fmax[s0];
  for (int k = 1; k < g.nwin; ++k) umax = fmax(umax, d.fmax[s0 + k]);
  WinConst c;
  c.umax = umax;
  c.unorm = umax > 0.0 ? umax : 1.0;
  c.wnorm = c.unorm;
  if (d.zs) {
    double wm = d.zmax[s0];
    for (int k = 1; k < g.nwin; ++k) wm = fmax(wm, d.zmax[s0 + k]);
    c.wnorm = wm > 0.0 ? wm : 1.0;
  }
  c.t = t;
  c.s0 = s0;
  if (t < g.fw) {
    c.out_slice = t;
    c.ref = t;
  } else if (t >= g.nimg - g.fw) {
    c.out_slice = t - (g.nimg - g.Ntc);      // pguresvt.hpp:161
    c.ref = t - (g.nimg - g.nwin);            // arps.hpp:82
  } else {
    c.out_slice = g.fw;
    c.ref = g.fw;
  }
  c.est_alpha = pb.alpha_c;  // replaced by noise.cu when estimated
  c.est_mu = pb.mu_c;
  c.est_sigma = pb.sigma_c;
  // PGURE(u, p, alpha, sigma, mu, ...) binds to the ctor's (alpha, mu, sigma)
  c.alpha = pb.alpha_c;
  if (pb.compat & 0x1) {
    c.mu = pb.sigma_c;
    c.sigma = pb.mu_c;
  } else {
    c.mu = pb.mu_c;
    c.sigma = pb.sigma_c;
  }
  // max(U) of the normalised window is umax/umax (pgure.hpp:72-73)
  const double umaxn = umax > 0.0 ? umax / umax : 1.0;
  c.eps1 = umaxn * 0.0001;
  c.eps2 = 100 * c.eps1;
  c.sum_u = 0.0;
  c.start = 0.0;
  c.upper = 100.0;
  d.wc[w] = c;
}

template <bool F64>
__global__ void k_window_norm(Problem pb, DeviceBuffers d) {
  const Geometry& g = pb.g;
  const int w = blockIdx.y;
  const size_t C = g.cube();
  const WinConst& c = d.wc[w];
  const size_t base = (size_t)c.s0 * g.F();
  float* u = d.u + (size_t)w * C;
  const float um = (float)c.unorm;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < C;
       i += (size_t)gridDim.x * blockDim.x) {
    if (F64) u[i] = (float)(d.x64[base + i] / c.unorm);
    else u[i] = __fdiv_rn(d.xs[base + i], um);  // exact operands: correctly rounded
  }
  if (d.zs) {  // ARPS input from the median-filtered sequence
    float* wz = d.wz + (size_t)w * C;
    double* w64 = d.w64 + (size_t)w * C;
    const float wn = (float)c.wnorm;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < C;
         i += (size_t)gridDim.x * blockDim.x) {
      wz[i] = __fdiv_rn(d.zs[base + i], wn);
      w64[i] = (double)d.zs[base + i] / c.wnorm;  // pguresvt.hpp:117-120
    }
  }
}

cudaError_t launch_window_setup(const Problem& pb, const DeviceBuffers& d, cudaStream_t s) {
  k_window_const<<<(pb.W + 63) / 64, 64, 0, s>>>(pb, d);
  return launch_window_norm_only(pb, d, s);
}

cudaError_t launch_window_norm_only(const Problem& pb, const DeviceBuffers& d, cudaStream_t s) {
  const size_t C = pb.g.cube();
  dim3 grid((unsigned)std::min<size_t>((C + 255) / 256, 1024), pb.W);
  if (d.x64) k_window_norm<true><<<grid, 256, 0, s>>>(pb, d);
  else k_window_norm<false><<<grid, 256, 0, s>>>(pb, d);
  return cudaGetLastError();
}

}  // namespace pgsvt
