// hotpixel.cu — the reference's hot-pixel filter (HotPixelFilter,
// hotpixel.hpp:19-64) on the GPU, applied by the command-line tool before
// denoising.
//
// Per uint16 frame: med = median of the column medians; mad = median of the
// column medians of |frame - med| times 1/0.6745; every pixel with
// |x - med| > threshold * mad (converted to uint16) is an outlier.  Outliers are then replaced in
// column-major order, in place: an interior one by the mean of the 4th and
// 5th of its 8 sorted neighbours (as they are at that moment, so earlier
// replacements feed later ones), an edge one by med, both truncated to uint16.
//
// Reproduced from the reference's element types (Armadillo 9.880.1, absent
// from the reference tree, restated from its documented behaviour): the
// medians of uint16 data are uint16 (an even count gives lo + (hi - lo) / 2
// in integer arithmetic); `frame - med` converts med to uint16 and subtracts
// in uint16, so values below med wrap around modulo 65536 (abs() of an
// unsigned value is the value).
//
// GB300 mapping: one CTA per (frame, column) for the column medians (radix
// selection on 16-bit keys in shared memory), one CTA per frame for the
// median of medians and the outlier flags, and one thread per frame for the
// order-dependent replacement pass (outliers are sparse).
#include "pgsvt.h"
#include "pgsvt_internal.h"

namespace pgsvt {
namespace {

// k-th smallest of n uint16 values val(i) (two 8-bit radix passes)
template <class F>
__device__ uint32_t select16(F val, int n, int k, unsigned* hist, int* sh) {
  uint32_t prefix = 0u, mask = 0u;
  for (int shift = 8; shift >= 0; shift -= 8) {
    for (int i = threadIdx.x; i < 256; i += blockDim.x) hist[i] = 0u;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const uint32_t v = val(i);
      if ((v & mask) == prefix) atomicAdd(&hist[(v >> shift) & 255u], 1u);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int acc = 0, dg = 0;
      for (; dg < 255; ++dg) {
        if (acc + (int)hist[dg] > k) break;
        acc += (int)hist[dg];
      }
      sh[0] = dg;
      sh[1] = k - acc;
    }
    __syncthreads();
    prefix |= (uint32_t)sh[0] << shift;
    mask |= 255u << shift;
    k = sh[1];
    __syncthreads();
  }
  return prefix;
}

// Armadillo median() of n uint16 values: the middle one, or lo + (hi - lo)/2
template <class F>
__device__ uint32_t median16(F val, int n, unsigned* hist, int* sh) {
  if (n % 2) return select16(val, n, n / 2, hist, sh);
  const uint32_t lo = select16(val, n, n / 2 - 1, hist, sh);
  const uint32_t hi = select16(val, n, n / 2, hist, sh);
  return lo + (hi - lo) / 2u;
}

// pass 0: column medians of the frame; pass 1: of |frame - med| (uint16 wrap)
__global__ void __launch_bounds__(256) k_col_median(const uint16_t* seq, int nr, int nc,
                                                    const uint32_t* med, int pass,
                                                    uint16_t* colmed) {
  const int c = blockIdx.x, f = blockIdx.y;
  __shared__ unsigned hist[256];
  __shared__ int sh[2];
  const uint16_t* col = seq + ((size_t)f * nc + c) * nr;
  const uint16_t m = pass ? (uint16_t)med[f] : 0;
  auto val = [&](int i) -> uint32_t {
    return pass ? (uint16_t)(col[i] - m) : col[i];
  };
  const uint32_t v = median16(val, nr, hist, sh);
  if (threadIdx.x == 0) colmed[(size_t)f * nc + c] = (uint16_t)v;
}

// median of a frame's column medians
__global__ void __launch_bounds__(256) k_frame_median(const uint16_t* colmed, int nc,
                                                      uint32_t* out) {
  const int f = blockIdx.x;
  __shared__ unsigned hist[256];
  __shared__ int sh[2];
  const uint16_t* cm = colmed + (size_t)f * nc;
  const uint32_t v = median16([&](int i) -> uint32_t { return cm[i]; }, nc, hist, sh);
  if (threadIdx.x == 0) out[f] = v;
}

// outlier flags from the unmodified frame; the comparison converts
// threshold * mad to uint16 (Armadillo's relational operators take the
// element type)
__global__ void k_hot_flags(const uint16_t* seq, size_t F, int nimg, const uint32_t* med,
                            const uint32_t* madm, double thr, uint8_t* flag) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < F * nimg;
       i += (size_t)gridDim.x * blockDim.x) {
    const size_t f = i / F;
    const double t = thr * ((double)madm[f] * (1.0 / 0.6745));
    const uint16_t tu = !(t > 0.0) ? 0 : (t >= 65535.0 ? 65535 : (uint16_t)t);
    const uint16_t d = (uint16_t)(seq[i] - (uint16_t)med[f]);
    flag[i] = d > tu ? 1 : 0;
  }
}

// order-dependent replacement, one thread per frame (column-major order)
__global__ void k_hot_replace(uint16_t* seq, int nr, int nc, int nimg, const uint32_t* med,
                              const uint8_t* flag) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nimg) return;
  uint16_t* a = seq + (size_t)f * nr * nc;
  const uint8_t* fl = flag + (size_t)f * nr * nc;
  for (size_t i = 0; i < (size_t)nr * nc; ++i) {
    if (!fl[i]) continue;
    const int r = (int)(i % nr), c = (int)(i / nr);
    if (r > 0 && r < nr - 1 && c > 0 && c < nc - 1) {
      double w[8] = {(double)a[(r - 1) + (size_t)(c - 1) * nr], (double)a[(r - 1) + (size_t)c * nr],
                     (double)a[(r - 1) + (size_t)(c + 1) * nr], (double)a[r + (size_t)(c - 1) * nr],
                     (double)a[r + (size_t)(c + 1) * nr], (double)a[(r + 1) + (size_t)(c - 1) * nr],
                     (double)a[(r + 1) + (size_t)c * nr], (double)a[(r + 1) + (size_t)(c + 1) * nr]};
      for (int p = 1; p < 8; ++p)  // insertion sort of the 8 neighbours
        for (int q = p; q > 0 && w[q - 1] > w[q]; --q) {
          const double t = w[q];
          w[q] = w[q - 1];
          w[q - 1] = t;
        }
      a[i] = (uint16_t)(0.5 * (w[3] + w[4]));
    } else {
      a[i] = (uint16_t)(double)med[f];
    }
  }
}

}  // namespace

cudaError_t launch_hot_pixel(uint16_t* seq, int nr, int nc, int nimg, double thr, uint16_t* colmed,
                             uint32_t* med, uint32_t* madm, uint8_t* flag, cudaStream_t s) {
  k_col_median<<<dim3(nc, nimg), 256, 0, s>>>(seq, nr, nc, nullptr, 0, colmed);
  k_frame_median<<<nimg, 256, 0, s>>>(colmed, nc, med);
  k_col_median<<<dim3(nc, nimg), 256, 0, s>>>(seq, nr, nc, med, 1, colmed);
  k_frame_median<<<nimg, 256, 0, s>>>(colmed, nc, madm);
  k_hot_flags<<<1024, 256, 0, s>>>(seq, (size_t)nr * nc, nimg, med, madm, thr, flag);
  k_hot_replace<<<(nimg + 63) / 64, 64, 0, s>>>(seq, nr, nc, nimg, med, flag);
  return cudaGetLastError();
}

}  // namespace pgsvt
