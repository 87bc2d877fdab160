// noise.cu — the reference's noise estimator (NoiseEstimator::Estimate,
// noise.hpp:36-152) on the GPU.
//
// The reference estimates (alpha, mu, sigma) on every normalised window u
// when PGURE optimisation is on (pguresvt.hpp:122-127): per slice a
// quadtree of F-tested blocks (noise.hpp:181-222, 411-453), per leaf a
// robust mean (IRLS with Huber weights, noise.hpp:239-270) and a robust
// variance of the Laplacian-filtered block (1.4826 MAD, noise.hpp:232-236,
// 386-409), then an IRLS straight-line fit var = alpha * mean + beta over
// all leaves of the window (noise.hpp:310-357).  Noise method 4 takes
// mu = the smallest leaf mean, method 3 the mode of the leaf means; sigma =
// sqrt(|beta + alpha * mu|).
//
// GB300 mapping.  The split decisions and the leaf variances are
// scale-equivariant, so they are computed once per input frame on the raw
// values and rescaled per window (var_u = var_x / umax^2); the robust means
// (whose stopping tolerance is absolute) and the fit run per window:
//   k_quad_decide   one CTA per (frame, block of side > 8): the F statistic
//   k_quad_tree     one thread per frame: replays the reference's recursion
//                   over the decision table, including its quirks (the
//                   node that was last before a split is re-visited, the
//                   fourth child is not; the smallest split index, the root,
//                   stays a leaf), and lists the leaves in its order
//   k_leaf_stats    one CTA per (frame, leaf): order statistics by 8-bit
//                   radix selection (IQD bounds, Laplacian median and MAD)
//   k_leaf_mean     one warp per (window, slice, leaf of side <= 32, values
//                   staged in shared memory), one CTA per larger leaf: the
//                   IRLS robust mean; the recursion lists most blocks twice,
//                   and every repeated block reuses the first one's results
//   k_noise_fit     one cluster of 8 CTAs per window (distributed shared
//                   memory for the sums and the radix selections): the IRLS
//                   fit, mu, sigma
// All arithmetic is FP64.
#include <cooperative_groups.h>

#include "pgsvt.h"
#include "pgsvt_internal.h"

namespace pgsvt {

namespace {

// 2.5% points of F(N^2 - 1, N^2 - 1) for N = 2, 4, ..., 4096, to six digits as
// the reference tabulates them (noise.hpp:167-178)
__constant__ double kF0025[12] = {15.4392, 2.86209, 1.64602, 1.27893, 1.13046, 1.06318,
                                  1.03110, 1.01543, 1.00769, 1.00384, 1.00192, 1.00096};
constexpr int kLeafMin = 8;        // NoiseEstimator's minimum block size
constexpr double kTol = 1e-6, kEps = 1e-12;
constexpr int kMaxIter = 10000;

__device__ __forceinline__ unsigned long long okey(double v) {  // order-preserving bits
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double ovalue(unsigned long long k) {
  const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)b);
}

// k-th smallest (0-based) of the n values val(i), by 8-bit radix digits of
// their ordered bit patterns.  Called by every thread of the block.
template <class F>
__device__ double block_select(F val, int n, int k, unsigned* hist, int* sh) {
  unsigned long long prefix = 0ull, mask = 0ull;
  for (int shift = 56; shift >= 0; shift -= 8) {
    for (int i = threadIdx.x; i < 256; i += blockDim.x) hist[i] = 0u;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const unsigned long long kv = okey(val(i));
      if ((kv & mask) == prefix) atomicAdd(&hist[(unsigned)(kv >> shift) & 255u], 1u);
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
    prefix |= (unsigned long long)sh[0] << shift;
    mask |= 255ull << shift;
    k = sh[1];
    __syncthreads();
  }
  return ovalue(prefix);
}

__device__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[wid] = v;
  __syncthreads();
  double t = 0.0;
  for (int q = 0; q < nw; ++q) t += red[q];
  return t;
}

__device__ double block_max(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[wid] = v;
  __syncthreads();
  double t = red[0];
  for (int q = 1; q < nw; ++q) t = fmax(t, red[q]);
  return t;
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double huber(double x) {  // WeightFunction type 0
  const double ax = fabs(x);
  return ax < 0.75 ? 1.0 : 0.75 / ax;
}

// Blocks of one frame: levels l = 0.. with side S >> l, 4^l blocks each,
// block (bi, bj) of level l at index (4^l - 1)/3 + bi + bj * 2^l.
__host__ __device__ inline int level_off(int l) { return ((1 << (2 * l)) - 1) / 3; }

struct FrameSrc {
  const float* xs;
  const double* x64;
  int S;
  __device__ double at(size_t f, int r, int c) const {
    const size_t k = f * (size_t)S * S + r + (size_t)c * S;
    return x64 ? x64[k] : (double)xs[k];
  }
};

// border indexing of noise.hpp:184-190 and 393-397
__device__ __forceinline__ int nxt(int x, int N) { return (x + 1 == N) ? 1 : x + 1; }
__device__ __forceinline__ int prv(int x, int N) { return (x == 0) ? N - 2 : x - 1; }

// SplitBlockQ (noise.hpp:181-222): the F statistic of block b of frame f
// (level l: side S >> l), computed by `step` cooperating threads (a warp for
// sides 16 and 32, a CTA above).
template <bool BLOCK>
__device__ void decide_block(const FrameSrc& src, int f, int b, int nlev, uint8_t* split,
                             double* red) {
  int l = 0;
  while (l + 1 < nlev && b >= level_off(l + 1)) ++l;
  const int N = src.S >> l, nb = 1 << l, loc = b - level_off(l);
  const int i0 = (loc % nb) * N, j0 = (loc / nb) * N;
  const size_t R = (size_t)N * N;
  const int lane = BLOCK ? threadIdx.x : (threadIdx.x & 31);
  const int step = BLOCK ? blockDim.x : 32;
  const double sq30 = sqrt(30.0);  // sqrt(l*l + l), l = 5
  auto A = [&](int r, int c) { return src.at(f, i0 + r, j0 + c); };
  auto res = [&](size_t e) {
    const int y = (int)(e % N), x = (int)(e / N);
    const double s4 = ((A(nxt(y, N), x) + A(prv(y, N), x)) + A(y, prv(x, N))) + A(y, nxt(x, N));
    return (5.0 * A(y, x) - s4) / sq30;
  };
  auto sum = [&](double v) { return BLOCK ? block_sum(v, red) : warp_sum(v); };
  double sa = 0.0, sr = 0.0;
  for (size_t e = lane; e < R; e += step) {
    sa += A((int)(e % N), (int)(e / N));
    sr += res(e);
  }
  const double mz = sum(sa) / (double)R;
  const double mr = sum(sr) / (double)R;
  double qa = 0.0, qr = 0.0;
  for (size_t e = lane; e < R; e += step) {
    const double da = A((int)(e % N), (int)(e / N)) - mz, dr = res(e) - mr;
    qa += da * da;
    qr += dr * dr;
  }
  const double Sz = sum(qa) / (double)(R - 1);
  const double Se = sum(qr) / (double)(R - 1);
  if (lane == 0) {
    const double stat = (Sz > Se) ? Sz / Se : Se / Sz;
    const int li = 31 - __clz(N) - 1;  // N = 2^(li+1)
    split[(size_t)f * level_off(nlev) + b] = (li >= 0 && li < 12 && stat > kF0025[li]) ? 1 : 0;
  }
}

// blocks of side >= 64: one CTA each (levels [0, lbig))
__global__ void __launch_bounds__(256) k_quad_decide_big(FrameSrc src, int nlev, uint8_t* split) {
  __shared__ double red[32];
  decide_block<true>(src, blockIdx.y, blockIdx.x, nlev, split, red);
}

// blocks of sides 32 and 16: one warp each (levels [lbig, nlev))
__global__ void __launch_bounds__(256) k_quad_decide_small(FrameSrc src, int nlev, int lbig,
                                                           uint8_t* split) {
  const int b = level_off(lbig) + blockIdx.x * 8 + (threadIdx.x >> 5);
  if (b >= level_off(nlev)) return;
  decide_block<false>(src, blockIdx.y, b, nlev, split, nullptr);
}

// QuadTree (noise.hpp:411-453) replayed over the decision table; writes the
// leaves (row, col, side) in the reference's order.
__global__ void k_quad_tree(const uint8_t* split, int nimg, int S, int nlev, int maxNodes,
                            int4* nodes, uint8_t* isdel, int4* leaf, int* nleaf, int* dup,
                            int* first, int* err) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nimg) return;
  const uint8_t* sp = split + (size_t)f * level_off(nlev);
  int4* nd = nodes + (size_t)f * maxNodes;
  uint8_t* dl = isdel + (size_t)f * maxNodes;
  int len = 1, minDel = maxNodes, top = 0;
  nd[0] = make_int4(0, 0, S, 0);
  dl[0] = 0;
  int stk_n[32], stk_it[32];
  bool bad = false;
  auto try_split = [&](int part) {
    const int4 q = nd[part];
    if (q.z <= kLeafMin) return;
    const int l = 31 - __clz(S / q.z), nb = 1 << l;
    if (!sp[level_off(l) + q.x / q.z + (q.y / q.z) * nb]) return;
    if (len + 4 > maxNodes || top >= 32) {
      bad = true;
      return;
    }
    const int h = q.z / 2, n = len - 1;
    nd[len] = make_int4(q.x, q.y, h, 0);
    nd[len + 1] = make_int4(q.x + h, q.y, h, 0);
    nd[len + 2] = make_int4(q.x, q.y + h, h, 0);
    nd[len + 3] = make_int4(q.x + h, q.y + h, h, 0);
    for (int k = 0; k < 4; ++k) dl[len + k] = 0;
    len += 4;
    dl[part] = 1;
    minDel = min(minDel, part);
    stk_n[top] = n;
    stk_it[top] = n;
    ++top;
  };
  try_split(0);
  while (top > 0 && !bad) {
    const int t = top - 1;
    if (stk_it[t] > stk_n[t] + 3) {
      --top;
      continue;
    }
    try_split(stk_it[t]++);
  }
  // leaves in node order; the recursion lists most blocks twice, and a
  // repeated block (same row, column, side) reuses the first one's statistics
  int* fi = first + (size_t)f * level_off(nlev + 1);
  for (int b = 0; b < level_off(nlev + 1); ++b) fi[b] = -1;
  int nl = 0;
  for (int k = 0; k < len; ++k) {
    if (dl[k] && k != minDel) continue;
    const int4 q = nd[k];
    const int l = 31 - __clz(S / q.z);
    const int id = level_off(l) + q.x / q.z + (q.y / q.z) * (1 << l);
    dup[(size_t)f * maxNodes + nl] = fi[id];
    if (fi[id] < 0) fi[id] = nl;
    leaf[(size_t)f * maxNodes + nl++] = q;
  }
  nleaf[f] = bad ? 0 : nl;
  if (bad) atomicExch(err, 1);
}

// ConvolveFIR (noise.hpp:386-409) value at e = x + y*N of the N x N block:
// in(x, y) - (its 8 neighbours) / 8, in the order of the reference's 3x3
// product with two interleaved accumulators.
template <class A_t>
__device__ __forceinline__ double lap_at(A_t A, int e, int N) {
  const int x = e % N, y = e / N;
  const int xp = nxt(x, N), xm = prv(x, N), yp = nxt(y, N), ym = prv(y, N);
  const double nb[9] = {A(xm, ym), A(xm, y), A(xm, yp), A(x, ym), A(x, y),
                        A(x, yp), A(xp, ym), A(xp, y), A(xp, yp)};
  double v1 = 0.0, v2 = 0.0;
#pragma unroll
  for (int k = 0; k < 8; k += 2) {
    v1 = __dadd_rn(v1, __dmul_rn(nb[k], k == 4 ? 1.0 : -0.125));
    v2 = __dadd_rn(v2, __dmul_rn(nb[k + 1], -0.125));
  }
  v1 = __dadd_rn(v1, __dmul_rn(nb[8], -0.125));
  return __dadd_rn(v1, v2);
}

__device__ __forceinline__ int iqd_m(int n) { return ((n + 1) / 2 + 1) / 2; }  // noise.hpp:227

// Bitonic sort of n2 (power of two) ordered keys in shared memory by one warp.
__device__ void warp_sort(unsigned long long* buf, int n2) {
  const int lane = threadIdx.x & 31;
  for (int k = 2; k <= n2; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < n2; i += 32) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const unsigned long long a = buf[i], b = buf[ixj];
          if ((a > b) == ((i & k) == 0)) {
            buf[i] = b;
            buf[ixj] = a;
          }
        }
      }
      __syncwarp();
    }
}

// Per (frame, leaf of side <= 32): IQD order statistics and the robust
// variance of the Laplacian (raw scale): stats = (a_lo, a_hi, var).  One warp
// per leaf, three sorts of at most 1024 keys in shared memory.
__global__ void __launch_bounds__(128) k_leaf_stats_small(FrameSrc src, const int4* leaf,
                                                          const int* nleaf, const int* dup,
                                                          int maxNodes, double* stats) {
  __shared__ unsigned long long sbuf[4][1024];
  const int f = blockIdx.y, wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int li = blockIdx.x * 4 + wib;
  if (li >= nleaf[f] || dup[(size_t)f * maxNodes + li] >= 0) return;
  const int4 q = leaf[(size_t)f * maxNodes + li];
  if (q.z > 32) return;  // k_leaf_stats_big
  const int N = q.z, n = N * N;
  int n2 = 1;
  while (n2 < n) n2 <<= 1;
  unsigned long long* buf = sbuf[wib];
  auto A = [&](int r, int c) { return src.at(f, q.x + r, q.y + c); };
  auto sort_vals = [&](auto fv) {
    for (int i = lane; i < n2; i += 32) buf[i] = i < n ? okey(fv(i)) : ~0ull;
    __syncwarp();
    warp_sort(buf, n2);
  };
  auto median_sorted = [&]() {  // Armadillo median(): lo + (hi - lo) / 2 for even n
    if (n % 2) return ovalue(buf[n / 2]);
    const double lo = ovalue(buf[n / 2 - 1]), hi = ovalue(buf[n / 2]);
    return lo + (hi - lo) / 2.0;
  };
  sort_vals([&](int e) { return A(e % N, e / N); });
  const int m = iqd_m(n);
  const double alo = ovalue(buf[m - 1]), ahi = ovalue(buf[n - m - 1]);
  __syncwarp();
  sort_vals([&](int e) { return lap_at(A, e, N); });
  const double med = median_sorted();
  __syncwarp();
  // |lap - med| of the sorted values (the order does not matter)
  for (int i = lane; i < n; i += 32) buf[i] = okey(fabs(ovalue(buf[i]) - med));
  __syncwarp();
  warp_sort(buf, n2);
  const double mad = median_sorted();
  if (lane == 0) {
    const double sig = 1.4826 * mad;
    double* o = stats + ((size_t)f * maxNodes + li) * 3;
    o[0] = alo;
    o[1] = ahi;
    o[2] = sig * sig;
  }
}

// The same for leaves of side > 32: one CTA per leaf, radix selection.
__global__ void __launch_bounds__(256) k_leaf_stats_big(FrameSrc src, const int4* leaf,
                                                        const int* big, const int* nbig,
                                                        const int* dup, int maxNodes,
                                                        double* stats) {
  const int f = blockIdx.y;
  if ((int)blockIdx.x >= nbig[f]) return;
  const int li = big[(size_t)f * maxNodes + blockIdx.x];
  if (dup[(size_t)f * maxNodes + li] >= 0) return;
  const int4 q = leaf[(size_t)f * maxNodes + li];
  const int N = q.z, n = N * N;
  __shared__ unsigned hist[256];
  __shared__ int sh[2];
  auto A = [&](int r, int c) { return src.at(f, q.x + r, q.y + c); };
  auto aval = [&](int e) { return A(e % N, e / N); };
  const int m = iqd_m(n);
  const double alo = block_select(aval, n, m - 1, hist, sh);
  const double ahi = block_select(aval, n, n - m - 1, hist, sh);
  auto lap = [&](int e) { return lap_at(A, e, N); };
  auto median_of = [&](auto fv) {
    if (n % 2) return block_select(fv, n, n / 2, hist, sh);
    const double lo = block_select(fv, n, n / 2 - 1, hist, sh);
    const double hi = block_select(fv, n, n / 2, hist, sh);
    return lo + (hi - lo) / 2.0;
  };
  const double med = median_of(lap);
  auto dev = [&](int e) { return fabs(lap(e) - med); };
  const double mad = median_of(dev);
  if (threadIdx.x == 0) {
    const double sig = 1.4826 * mad;
    double* o = stats + ((size_t)f * maxNodes + li) * 3;
    o[0] = alo;
    o[1] = ahi;
    o[2] = sig * sig;
  }
}

struct MeanArgs {
  FrameSrc src;
  const int4* leaf;
  const int* nleaf;
  const int* dup;
  const double* stats;
  int maxNodes, nwin;
  double* mean;  // [W][nwin][maxNodes]
};

// RobustMeanEstimate (noise.hpp:239-270) of one leaf of window w, slice k.
// The weights of an iteration come from the previous (m, 1/d), so nothing
// is stored per element; the IQD of r = u - m is (u_hi - m) - (u_lo - m)
// from the leaf's order statistics.  `val(e)` is the leaf's e-th u value;
// `lane`/`step`/`sum` describe the cooperating threads (a warp or a CTA).
template <class V, class R>
__device__ double robust_mean(V val, int n, double ulo, double uhi, int lane, int step, R sum) {
  double m = 0.0, m0 = 1e12, mprev = 0.0, inv = 0.0;
  for (int it = 0; it < kMaxIter; ++it) {
    double sw = 0.0, swa = 0.0;
    for (int e = lane; e < n; e += step) {
      const double x = val(e);
      const double w = it == 0 ? 1.0 : huber((x - mprev) * inv);
      sw += w;
      swa += w * x;
    }
    sw = sum(sw);
    swa = sum(swa);
    m = (fabs(sw) < kEps) ? m0 : swa / sw;
    double se = 0.0;
    for (int e = lane; e < n; e += step) se += fabs(val(e) - m);
    se = sum(se);
    if (fabs(m0 - m) < kTol || se / (double)n < kTol) break;
    m0 = m;
    const double d = ((uhi - m) - (ulo - m)) + kEps;
    mprev = m;
    inv = 1.0 / d;
  }
  return m;
}

// leaves of side <= 32: one warp each, the leaf's u values (x / umax, as the
// reference normalises) staged once in shared memory
__global__ void __launch_bounds__(128) k_leaf_mean_warp(Problem pb, DeviceBuffers d, MeanArgs a) {
  __shared__ double sbuf[4][1024];
  const int w = blockIdx.z, k = blockIdx.y, wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int li = blockIdx.x * 4 + wib;
  const WinConst& wc = d.wc[w];
  const size_t f = (size_t)(wc.s0 + k);
  if (li >= a.nleaf[f] || a.dup[f * a.maxNodes + li] >= 0) return;
  const int4 q = a.leaf[f * a.maxNodes + li];
  if (q.z > 32) return;  // k_leaf_mean_block
  const int N = q.z, n = N * N;
  const double um = wc.unorm;
  double* buf = sbuf[wib];
  for (int e = lane; e < n; e += 32) buf[e] = a.src.at(f, q.x + e % N, q.y + e / N) / um;
  __syncwarp();
  const double* st = a.stats + (f * a.maxNodes + li) * 3;
  const double m = robust_mean([&](int e) { return buf[e]; }, n, st[0] / um, st[1] / um, lane,
                               32, [](double v) { return warp_sum(v); });
  if (lane == 0) a.mean[((size_t)w * a.nwin + k) * a.maxNodes + li] = m;
}

// leaves of side > 32: one CTA each
__global__ void __launch_bounds__(256) k_leaf_mean_block(Problem pb, DeviceBuffers d, MeanArgs a,
                                                         const int* big, const int* nbig) {
  const int w = blockIdx.z, k = blockIdx.y;
  const WinConst& wc = d.wc[w];
  const size_t f = (size_t)(wc.s0 + k);
  if ((int)blockIdx.x >= nbig[f]) return;
  const int li = big[f * a.maxNodes + blockIdx.x];
  if (a.dup[f * a.maxNodes + li] >= 0) return;
  const int4 q = a.leaf[f * a.maxNodes + li];
  const int N = q.z;
  const double um = wc.unorm;
  __shared__ double red[32];
  const double* st = a.stats + (f * a.maxNodes + li) * 3;
  const double m = robust_mean(
      [&](int e) { return a.src.at(f, q.x + e % N, q.y + e / N) / um; }, N * N, st[0] / um,
      st[1] / um, threadIdx.x, blockDim.x, [&](double v) { return block_sum(v, red); });
  if (threadIdx.x == 0) a.mean[((size_t)w * a.nwin + k) * a.maxNodes + li] = m;
}

// Leaves of side > 32 of each frame (for k_leaf_mean_block / k_leaf_stats_big).
__global__ void k_big_leaves(const int4* leaf, const int* nleaf, int nimg, int maxNodes, int* big,
                             int* nbig) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nimg) return;
  int c = 0;
  for (int li = 0; li < nleaf[f]; ++li)
    if (leaf[(size_t)f * maxNodes + li].z > 32) big[(size_t)f * maxNodes + c++] = li;
  nbig[f] = c;
}

struct FitArgs {
  const int* nleaf;
  const int* dup;
  const double* stats;
  const double* mean;
  int maxNodes, nwin, method;
  double* x;        // [W][nwin * maxNodes] leaf means of the window
  double* y;        // leaf variances of the window
  unsigned long long* key;  // ordered bits of the residuals
  int* hist;        // [W][nwin * maxNodes + 1] mode counts (method 3)
};

constexpr int kFitCtas = 8;       // CTAs of the cluster that fits one window
constexpr int kFitThreads = 512;
constexpr int kDigitBits = 11, kDigits = 1 << kDigitBits;

namespace cg = cooperative_groups;

__device__ double cluster_max(cg::cluster_group& cl, double v, double* red, double* part) {
  v = block_max(v, red);
  if (threadIdx.x == 0) *part = v;
  cl.sync();
  double t = *cl.map_shared_rank(part, 0);
  for (int r = 1; r < kFitCtas; ++r) t = fmax(t, *cl.map_shared_rank(part, r));
  cl.sync();
  return t;
}

// Sum over the cluster of one value per CTA thread; every thread of every
// CTA gets the same total (the CTAs' partials added in rank order).
__device__ double cluster_sum(cg::cluster_group& cl, double v, double* red, double* part) {
  v = block_sum(v, red);
  if (threadIdx.x == 0) *part = v;
  cl.sync();
  double t = 0.0;
  for (int r = 0; r < kFitCtas; ++r) t += *cl.map_shared_rank(part, r);
  cl.sync();  // the partials may be overwritten afterwards
  return t;
}

// k-th smallest (0-based) of the window's N residual keys, 11 bits per pass;
// each CTA histograms its slice, every CTA adds the cluster's histograms.
__device__ unsigned long long cluster_select(cg::cluster_group& cl, const unsigned long long* key,
                                             int lo, int hi, int k, unsigned* hist,
                                             unsigned* tot) {
  unsigned long long prefix = 0ull, mask = 0ull;
  for (int shift = 64 - kDigitBits; shift > -kDigitBits; shift -= kDigitBits) {
    const int sh = shift < 0 ? 0 : shift;
    const int bits = shift < 0 ? kDigitBits + shift : kDigitBits;
    const unsigned dmask = (1u << bits) - 1u;
    for (int i = threadIdx.x; i < kDigits; i += blockDim.x) hist[i] = 0u;
    __syncthreads();
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      const unsigned long long kv = key[i];
      if ((kv & mask) == prefix) atomicAdd(&hist[(unsigned)(kv >> sh) & dmask], 1u);
    }
    cl.sync();
    for (int i = threadIdx.x; i < kDigits; i += blockDim.x) {
      unsigned t = 0u;
      for (int r = 0; r < kFitCtas; ++r) t += cl.map_shared_rank(hist, r)[i];
      tot[i] = t;
    }
    cl.sync();  // every CTA has read every histogram
    __shared__ int s_dg, s_k;
    if (threadIdx.x == 0) {
      int acc = 0, dg = 0;
      for (; dg < (int)dmask; ++dg) {
        if (acc + (int)tot[dg] > k) break;
        acc += (int)tot[dg];
      }
      s_dg = dg;
      s_k = k - acc;
    }
    __syncthreads();
    prefix |= (unsigned long long)s_dg << sh;
    mask |= (unsigned long long)dmask << sh;
    k = s_k;
    __syncthreads();
  }
  return prefix;
}

// WLSFit (noise.hpp:302-358) and the method's mu / sigma for one window, by a
// cluster of kFitCtas CTAs (distributed shared memory for the reductions);
// the results go to the window constants (caller-side values, then the
// risk's binding).
__global__ void __cluster_dims__(kFitCtas, 1, 1) __launch_bounds__(kFitThreads)
    k_noise_fit(Problem pb, DeviceBuffers d, FitArgs a) {
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int w = blockIdx.y;
  WinConst& wc = d.wc[w];
  __shared__ double red[32];
  __shared__ double part;
  __shared__ unsigned hist[kDigits], tot[kDigits];
  __shared__ int base[32];
  const int nwin = a.nwin;
  if (threadIdx.x == 0) {
    int t = 0;
    for (int k = 0; k < nwin; ++k) {
      base[k] = t;
      t += a.nleaf[wc.s0 + k];
    }
    base[nwin] = t;
  }
  __syncthreads();
  const int N = base[nwin];
  const int lo = (int)((long long)N * rank / kFitCtas), hi = (int)((long long)N * (rank + 1) / kFitCtas);
  double* X = a.x + (size_t)w * nwin * a.maxNodes;
  double* Y = a.y + (size_t)w * nwin * a.maxNodes;
  unsigned long long* K = a.key + (size_t)w * nwin * a.maxNodes;
  const double um2 = wc.unorm * wc.unorm;
  for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    int k = 0;
    while (k + 1 < nwin && i >= base[k + 1]) ++k;
    const size_t f = (size_t)(wc.s0 + k);
    const int li = i - base[k];
    const int dp = a.dup[f * a.maxNodes + li];
    const int src = dp >= 0 ? dp : li;
    X[i] = a.mean[((size_t)w * nwin + k) * a.maxNodes + src];
    Y[i] = a.stats[(f * a.maxNodes + src) * 3 + 2] / um2;
  }
  cl.sync();
  const int mq = ((N + 1) / 2 + 1) / 2;
  double a0 = 1e12, b0 = 1e12, p0 = 0.0, p1 = 0.0, q0 = 0.0, q1 = 0.0, dd = 1.0;
  for (int it = 0; it < kMaxIter; ++it) {
    double s[5] = {0, 0, 0, 0, 0};
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      const double xi = X[i], yi = Y[i];
      const double wt = it == 0 ? 1.0 : huber((yi - (xi * q0 + q1)) / dd);
      const double w2 = wt * wt;
      s[0] += w2;
      s[1] += w2 * xi;
      s[2] += w2 * yi;
      s[3] += w2 * (xi * yi);
      s[4] += w2 * (xi * xi);
    }
    for (int k = 0; k < 5; ++k) s[k] = cluster_sum(cl, s[k], red, &part);
    p0 = s[0] * s[3] - s[1] * s[2];
    const double aux = s[0] * s[4] - s[1] * s[1];
    p0 = (fabs(aux) < kEps) ? a0 : p0 / aux;
    p1 = s[2] - p0 * s[1];
    p1 = (fabs(aux) < kEps) ? b0 : p1 / s[0];
    double se = 0.0;
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      const double r = Y[i] - (X[i] * p0 + p1);
      se += fabs(r);
      K[i] = okey(r);
    }
    se = cluster_sum(cl, se, red, &part) / (double)N;  // its syncs also publish K
    if ((fabs(a0 - p0) < kTol && fabs(b0 - p1) < kTol) || se < kTol) break;
    a0 = p0;
    b0 = p1;
    const double rlo = ovalue(cluster_select(cl, K, lo, hi, mq - 1, hist, tot));
    const double rhi = ovalue(cluster_select(cl, K, lo, hi, N - mq - 1, hist, tot));
    q0 = p0;
    q1 = p1;
    dd = (rhi - rlo) + kEps;
  }
  // mu: smallest leaf mean (method 4) or the mode of the leaf means (3)
  double mn = 1e300, mx = -1e300;
  for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    mn = fmin(mn, X[i]);
    mx = fmax(mx, X[i]);
  }
  mn = -cluster_max(cl, -mn, red, &part);
  mx = cluster_max(cl, mx, red, &part);
  double mode = 0.0;
  if (a.method == 3) {  // ComputeMode (noise.hpp:272-297) of the leaf means
    int* h = a.hist + (size_t)w * (nwin * a.maxNodes + 1);
    const double dyn = (double)N;
    for (int i = lo + threadIdx.x; i <= (rank + 1 == kFitCtas ? N : hi - 1); i += blockDim.x) h[i] = 0;
    cl.sync();
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      const double r = round(X[i] * dyn / mx);
      atomicAdd(&h[(int)fmin(fmax(r, 0.0), dyn)], 1);
    }
    cl.sync();
    __shared__ double s_mode;
    if (threadIdx.x == 0) {  // most frequent rounded value; ties: the smallest
      int best = 0, bc = -1;
      for (int i = 0; i <= N; ++i)
        if (h[i] > bc) {
          bc = h[i];
          best = i;
        }
      s_mode = (double)best * mx / dyn;
    }
    __syncthreads();
    mode = s_mode;
  }
  if (rank == 0 && threadIdx.x == 0) {
    const double alpha = pb.alpha_c >= 0 ? pb.alpha_c : p0;
    const double mu = pb.mu_c >= 0 ? pb.mu_c : (a.method == 3 ? mode : mn);
    const double sigma = pb.sigma_c >= 0 ? pb.sigma_c : sqrt(fabs(p1 + p0 * mu));
    wc.est_alpha = alpha;
    wc.est_mu = mu;
    wc.est_sigma = sigma;
    wc.alpha = alpha;  // PGURE(u, p, alpha, sigma, mu, ...) binding (pgure.hpp:26-30)
    if (pb.compat & PGSVT_COMPAT_SWAP_MU_SIGMA) {
      wc.mu = sigma;
      wc.sigma = mu;
    } else {
      wc.mu = mu;
      wc.sigma = sigma;
    }
  }
}

}  // namespace

// ---- host side

int noise_levels(int S) {
  int nlev = 0;
  for (int s = S; s > kLeafMin; s >>= 1) ++nlev;
  return nlev;
}
int noise_blocks(int nlev) { return level_off(nlev); }

cudaError_t launch_noise_frames(const float* xs, const double* x64, int nimg, int S,
                                const NoiseFrames& nf, cudaStream_t s) {
  const FrameSrc src{xs, x64, S};
  const int nlev = nf.nlev, lbig = nlev > 2 ? nlev - 2 : 0;
  const int nsmall = level_off(nlev) - level_off(lbig);
  if (lbig > 0) k_quad_decide_big<<<dim3(level_off(lbig), nimg), 256, 0, s>>>(src, nlev, nf.split);
  if (nsmall > 0)
    k_quad_decide_small<<<dim3((nsmall + 7) / 8, nimg), 256, 0, s>>>(src, nlev, lbig, nf.split);
  k_quad_tree<<<(nimg + 63) / 64, 64, 0, s>>>(nf.split, nimg, S, nlev, nf.maxNodes, nf.nodes,
                                              nf.isdel, nf.leaf, nf.nleaf, nf.dup, nf.first,
                                              nf.err);
  k_big_leaves<<<(nimg + 63) / 64, 64, 0, s>>>(nf.leaf, nf.nleaf, nimg, nf.maxNodes, nf.big,
                                               nf.nbig);
  k_leaf_stats_small<<<dim3((nf.maxNodes + 3) / 4, nimg), 128, 0, s>>>(src, nf.leaf, nf.nleaf,
                                                                       nf.dup, nf.maxNodes,
                                                                       nf.stats);
  k_leaf_stats_big<<<dim3(nf.maxBig, nimg), 256, 0, s>>>(src, nf.leaf, nf.big, nf.nbig, nf.dup,
                                                         nf.maxNodes, nf.stats);
  return cudaGetLastError();
}

cudaError_t launch_noise_windows(const Problem& pb, const DeviceBuffers& d, const NoiseFrames& nf,
                                 const NoiseWindows& nw, cudaStream_t s) {
  const Geometry& g = pb.g;
  MeanArgs ma{FrameSrc{d.xs, d.x64, g.S}, nf.leaf, nf.nleaf, nf.dup, nf.stats, nf.maxNodes,
              g.nwin, nw.mean};
  k_leaf_mean_warp<<<dim3((nf.maxNodes + 3) / 4, g.nwin, pb.W), 128, 0, s>>>(pb, d, ma);
  k_leaf_mean_block<<<dim3(nf.maxBig, g.nwin, pb.W), 256, 0, s>>>(pb, d, ma, nf.big, nf.nbig);
  FitArgs fa{nf.nleaf, nf.dup, nf.stats, nw.mean, nf.maxNodes, g.nwin, nw.method, nw.x, nw.y,
             nw.key, nw.hist};
  k_noise_fit<<<dim3(kFitCtas, pb.W), kFitThreads, 0, s>>>(pb, d, fa);
  return cudaGetLastError();
}

}  // namespace pgsvt
