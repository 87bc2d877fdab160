// noise.cu — the reference's noise estimator (NoiseEstimator::Estimate,
// noise.hpp:36-152) on the GPU.
//
// The reference estimates (alpha, mu, sigma) on every normalised window u
// when PGURE optimisation is on (pguresvt.hpp:122-127): per slice a
// quadtree of F-tested blocks (noise.hpp:181-222, 411-453), per leaf a
// robust mean (IRLS with Huber weights, noise.hpp:239-270) and a robust
// variance of the Laplacian-filtered block (1.4826 MAD, noise.hpp:232-236,
// 386-409), then an IRLS straight-line fit var = alpha * mean + beta over
// all leaves of the window (noise.hpp:310-357).  The leaves taken in
// ascending mean order, mu and sigma follow the method (noise.hpp:115-147):
//   1  modes of the means and of the variances of the first
//      round(0.05 * floor(Nx Ny / leaves)) + 1 leaves; sigma = sqrt(var mode)
//   2  mu = mode of all means; v = mode of all variances;
//      sigma = sqrt(max(v, beta + alpha v, 0))
//   3  mu = mode of all means; sigma = sqrt(|beta + alpha mu|)
//   4  mu = the smallest mean; sigma = sqrt(|beta + alpha mu|)
// A mode (ComputeMode, noise.hpp:272-297) is the most frequent value of
// round(v n / max v), ties going to the one met first in that order.
//
// GB300 mapping.  The split decisions and the leaf variances are
// scale-equivariant, so they are computed once per input frame on the raw
// values and rescaled per window (var_u = var_x / umax^2); the robust means
// depend on the window only through its maximum (their stopping tolerance is
// absolute), so they run once per (frame, distinct window maximum) pair, and
// every window then fits its own line:
//   k_quad_decide   one CTA per (frame, block of side > 8): the F statistic
//   k_quad_tree     one thread per frame: replays the reference's recursion
//                   over the decision table, including its quirks (the
//                   node that was last before a split is re-visited, the
//                   fourth child is not; the smallest split index, the root,
//                   stays a leaf), and lists the leaves in its order
//   k_leaf_stats    per (frame, unique leaf): order statistics (IQD bounds,
//                   Laplacian median and MAD) by warp bitonic sorts in shared
//                   memory (sides <= 32) or by a cluster of 8 CTAs with
//                   11-bit radix selection over distributed shared memory
//   k_leaf_mean     per (frame, window maximum) pair: one warp per leaf of
//                   side <= 32, one cluster of 8 CTAs per larger leaf: the
//                   IRLS robust mean, on the raw values with the absolute
//                   tolerances scaled by the window maximum; the recursion
//                   lists most blocks twice, and every repeated block reuses
//                   the first one's results
//   k_noise_fit     one cluster of 8 CTAs per window, all windows in one
//                   launch (distributed shared memory for the sums and the
//                   radix selections): the IRLS fit, mu, sigma; modes over
//                   all leaves by a histogram of the n + 1 rounded values
//                   with first-occurrence keys, method 1's few leaves by
//                   a radix selection and the reference's O(n^2) count
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

// ---- cluster helpers (distributed shared memory across kCl CTAs)

constexpr int kCl = 8;            // CTAs per cluster
constexpr int kClThreads = 512;
constexpr int kDigitBits = 11, kDigits = 1 << kDigitBits;

namespace cg = cooperative_groups;

struct ClusterSmem {
  double red[32];
  double part[8];
  unsigned h[2][kDigits];   // this CTA's histograms
  unsigned t[2][kDigits];   // the cluster's
  int dg[2], kk[2];
  int scan[kClThreads / 32 + 1];
};

// Sums over the cluster of up to 8 values per thread; every thread of every
// CTA gets the same totals (the CTAs' partials added in rank order).
template <int NV>
__device__ void cluster_sums(cg::cluster_group& cl, double (&v)[NV], ClusterSmem& sm) {
  for (int k = 0; k < NV; ++k) {
    const double b = block_sum(v[k], sm.red);
    if (threadIdx.x == 0) sm.part[k] = b;
  }
  cl.sync();
  for (int k = 0; k < NV; ++k) {
    double t = 0.0;
    for (int r = 0; r < kCl; ++r) t += cl.map_shared_rank(sm.part, r)[k];
    v[k] = t;
  }
  cl.sync();  // the partials may be overwritten afterwards
}

__device__ double cluster_max(cg::cluster_group& cl, double v, ClusterSmem& sm) {
  const double b = block_max(v, sm.red);
  if (threadIdx.x == 0) sm.part[0] = b;
  cl.sync();
  double t = *cl.map_shared_rank(sm.part, 0);
  for (int r = 1; r < kCl; ++r) t = fmax(t, cl.map_shared_rank(sm.part, r)[0]);
  cl.sync();
  return t;
}

// The digit of the k-th smallest key among the counts t[0..nb): a block-wide
// prefix scan (each thread owns nb / blockDim consecutive bins).
__device__ void find_digit(const unsigned* t, int nb, int k, int* out_dg, int* out_k, int* scan) {
  const int per = (nb + blockDim.x - 1) / blockDim.x;
  const int b0 = threadIdx.x * per;
  int loc = 0;
  for (int b = b0; b < b0 + per && b < nb; ++b) loc += (int)t[b];
  // exclusive scan of loc over the block
  int inc = loc;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) scan[wid] = inc;
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
      const int v = scan[q];
      scan[q] = acc;
      acc += v;
    }
  }
  __syncthreads();
  int before = scan[wid] + inc - loc;
  if (before <= k && k < before + loc) {
    for (int b = b0; b < b0 + per && b < nb; ++b) {
      if (before + (int)t[b] > k) {
        *out_dg = b;
        *out_k = k - before;
        break;
      }
      before += (int)t[b];
    }
  }
  __syncthreads();
}

// The k0-th and k1-th smallest of the n keys key(i) spread over the cluster
// (this CTA holds the indices [lo, hi)), 11 bits per pass.
template <class K>
__device__ void cluster_select2(cg::cluster_group& cl, K key, int lo, int hi, int k0, int k1,
                                ClusterSmem& sm, unsigned long long& v0, unsigned long long& v1) {
  unsigned long long pre[2] = {0ull, 0ull}, mask = 0ull;
  int k[2] = {k0, k1};
  for (int shift = 64 - kDigitBits; shift > -kDigitBits; shift -= kDigitBits) {
    const int sh = shift < 0 ? 0 : shift;
    const int bits = shift < 0 ? kDigitBits + shift : kDigitBits;
    const unsigned dm = (1u << bits) - 1u;
    for (int b = threadIdx.x; b < kDigits; b += blockDim.x) sm.h[0][b] = sm.h[1][b] = 0u;
    __syncthreads();
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      const unsigned long long kv = key(i);
      const unsigned dgt = (unsigned)(kv >> sh) & dm;
      if ((kv & mask) == pre[0]) atomicAdd(&sm.h[0][dgt], 1u);
      if ((kv & mask) == pre[1]) atomicAdd(&sm.h[1][dgt], 1u);
    }
    cl.sync();
    for (int b = threadIdx.x; b <= (int)dm; b += blockDim.x) {
      unsigned t0 = 0u, t1 = 0u;
      for (int r = 0; r < kCl; ++r) {
        const ClusterSmem* rs = cl.map_shared_rank(&sm, r);
        t0 += rs->h[0][b];
        t1 += rs->h[1][b];
      }
      sm.t[0][b] = t0;
      sm.t[1][b] = t1;
    }
    cl.sync();  // every CTA has read every histogram
    for (int q = 0; q < 2; ++q) find_digit(sm.t[q], (int)dm + 1, k[q], &sm.dg[q], &sm.kk[q], sm.scan);
    for (int q = 0; q < 2; ++q) {
      pre[q] |= (unsigned long long)sm.dg[q] << sh;
      k[q] = sm.kk[q];
    }
    mask |= (unsigned long long)dm << sh;
    __syncthreads();
  }
  v0 = pre[0];
  v1 = pre[1];
}

// Armadillo median() from the two middle keys of an even count
__device__ __forceinline__ double median_from(unsigned long long lo, unsigned long long hi, int n) {
  if (n % 2) return ovalue(hi);
  const double a = ovalue(lo), b = ovalue(hi);
  return a + (b - a) / 2.0;
}

// Per (frame, unique leaf of side > 32): the leaf statistics of
// k_leaf_stats_small by one cluster per leaf.
__global__ void __cluster_dims__(kCl, 1, 1) __launch_bounds__(kClThreads)
    k_leaf_stats_big(FrameSrc src, const int4* leaf, const int* big, const int* nbig,
                     const int* dup, int maxNodes, double* stats) {
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank(), bi = blockIdx.x / kCl, f = blockIdx.y;
  __shared__ ClusterSmem sm;
  const bool valid = bi < nbig[f];  // uniform over the cluster
  if (!valid) return;
  const int li = big[(size_t)f * maxNodes + bi];
  if (dup[(size_t)f * maxNodes + li] >= 0) return;
  const int4 q = leaf[(size_t)f * maxNodes + li];
  const int N = q.z, n = N * N;
  const int lo = (int)((long long)n * rank / kCl), hi = (int)((long long)n * (rank + 1) / kCl);
  auto A = [&](int r, int c) { return src.at(f, q.x + r, q.y + c); };
  const int m = iqd_m(n);
  unsigned long long a0, a1, l0, l1, d0, d1;
  cluster_select2(cl, [&](int e) { return okey(A(e % N, e / N)); }, lo, hi, m - 1, n - m - 1, sm,
                  a0, a1);
  const int mlo = n % 2 ? n / 2 : n / 2 - 1;
  cluster_select2(cl, [&](int e) { return okey(lap_at(A, e, N)); }, lo, hi, mlo, n / 2, sm, l0, l1);
  const double med = median_from(l0, l1, n);
  cluster_select2(cl, [&](int e) { return okey(fabs(lap_at(A, e, N) - med)); }, lo, hi, mlo,
                  n / 2, sm, d0, d1);
  const double mad = median_from(d0, d1, n);
  if (rank == 0 && threadIdx.x == 0) {
    const double sig = 1.4826 * mad;
    double* o = stats + ((size_t)f * maxNodes + li) * 3;
    o[0] = ovalue(a0);
    o[1] = ovalue(a1);
    o[2] = sig * sig;
  }
}

// RobustMeanEstimate (noise.hpp:239-270) of one leaf, run on the raw values
// x = u * um: with u = x / um every step is the same up to rounding when the
// absolute constants scale with um (tol, eps; the weights are scale-free),
// so m_u = m_x / um without dividing every element.  The weights of an
// iteration come from the previous (m, 1/d), so nothing is stored per
// element; the IQD of r = x - m is (x_hi - m) - (x_lo - m) from the leaf's
// order statistics.  `sum(a, b, c)` reduces three values over the
// cooperating threads (a warp, or a cluster).
template <class V, class R>
__device__ double robust_mean(V val, int lo, int hi, int n, double xlo, double xhi, double um,
                              int lane, int step, R sum) {
  const double tol = kTol * um, eps = kEps * um;
  double m = 0.0, m0 = 1e12 * um, mprev = 0.0, inv = 0.0;
  for (int it = 0; it < kMaxIter; ++it) {
    double sw = 0.0, swa = 0.0;
    for (int e = lo + lane; e < hi; e += step) {
      const double x = val(e);
      const double w = it == 0 ? 1.0 : huber((x - mprev) * inv);
      sw += w;
      swa += w * x;
    }
    double se = 0.0;
    // e = mean |x - m| needs m first: a second pass after the reduction
    sum(sw, swa, se, false);
    m = (fabs(sw) < kEps) ? m0 : swa / sw;
    for (int e = lo + lane; e < hi; e += step) se += fabs(val(e) - m);
    sum(sw, swa, se, true);
    if (fabs(m0 - m) < tol || se / (double)n < tol) break;
    m0 = m;
    const double d = ((xhi - m) - (xlo - m)) + eps;
    mprev = m;
    inv = 1.0 / d;
  }
  return m / um;
}

struct PairArgs {
  FrameSrc src;
  const int4* leaf;
  const int* nleaf;
  const int* dup;
  const int* big;
  const int* nbig;
  const double* stats;
  int maxNodes;
  const int* pair_frame;     // [npairs]
  const double* pair_norm;   // [npairs] normalisation of the pair (window maximum)
  double* mean;              // [npairs][maxNodes]
};

// robust means of the leaves of side <= 32 of every (frame, normalisation)
// pair: one warp per leaf
__global__ void __launch_bounds__(128) k_leaf_mean_warp(PairArgs a) {
  const int pr = blockIdx.y, lane = threadIdx.x & 31;
  const int li = blockIdx.x * 4 + (threadIdx.x >> 5);
  const size_t f = (size_t)a.pair_frame[pr];
  if (li >= a.nleaf[f] || a.dup[f * a.maxNodes + li] >= 0) return;
  const int4 q = a.leaf[f * a.maxNodes + li];
  if (q.z > 32) return;  // k_leaf_mean_big
  const int N = q.z;
  const double um = a.pair_norm[pr];
  const double* st = a.stats + (f * a.maxNodes + li) * 3;
  const double m = robust_mean(
      [&](int e) { return a.src.at(f, q.x + e % N, q.y + e / N); }, 0, N * N, N * N, st[0], st[1],
      um, lane, 32, [](double& x, double& y, double& z, bool zonly) {
        if (zonly) {
          z = warp_sum(z);
        } else {
          x = warp_sum(x);
          y = warp_sum(y);
        }
      });
  if (lane == 0) a.mean[(size_t)pr * a.maxNodes + li] = m;
}

// ... and of the leaves of side > 32: one cluster per leaf
__global__ void __cluster_dims__(kCl, 1, 1) __launch_bounds__(kClThreads)
    k_leaf_mean_big(PairArgs a) {
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank(), bi = blockIdx.x / kCl, pr = blockIdx.y;
  const size_t f = (size_t)a.pair_frame[pr];
  if (bi >= a.nbig[f]) return;  // uniform over the cluster
  const int li = a.big[f * a.maxNodes + bi];
  if (a.dup[f * a.maxNodes + li] >= 0) return;
  __shared__ ClusterSmem sm;
  const int4 q = a.leaf[f * a.maxNodes + li];
  const int N = q.z, n = N * N;
  const int lo = (int)((long long)n * rank / kCl), hi = (int)((long long)n * (rank + 1) / kCl);
  const double* st = a.stats + (f * a.maxNodes + li) * 3;
  const double m = robust_mean(
      [&](int e) { return a.src.at(f, q.x + e % N, q.y + e / N); }, lo, hi, n, st[0], st[1],
      a.pair_norm[pr], threadIdx.x, blockDim.x, [&](double& x, double& y, double& z, bool zonly) {
        if (zonly) {
          double v[1] = {z};
          cluster_sums(cl, v, sm);
          z = v[0];
        } else {
          double v[2] = {x, y};
          cluster_sums(cl, v, sm);
          x = v[0];
          y = v[1];
        }
      });
  if (rank == 0 && threadIdx.x == 0) a.mean[(size_t)pr * a.maxNodes + li] = m;
}

// Leaves of side > 32 of each frame.
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
  const double* mean;        // [npairs][maxNodes]
  const int* win_pair;       // [nwindows][nwin] pair of (window, slice)
  const int* win_s0;         // [nwindows] first frame of the window
  const double* win_norm;    // [nwindows] window normalisation
  int maxNodes, nwin, method;
  double alpha_c, mu_c, sigma_c;  // caller values (< 0: estimate)
  double* x;                 // [nwindows][nwin * maxNodes] scratch
  double* y;
  unsigned long long* key;
  int* hist;                 // [nwindows][nwin * maxNodes + 1]
  unsigned long long* fkey;  // [nwindows][nwin * maxNodes + 1] first-occurrence keys
  int* fidx;                 // [nwindows][nwin * maxNodes + 1]
  double* est;               // [nwindows][3] caller-side (alpha, mu, sigma)
  int nx;                    // frame side
};

// WLSFit (noise.hpp:302-358) and the method's mu / sigma for every window:
// one cluster per window.
__global__ void __cluster_dims__(kCl, 1, 1) __launch_bounds__(kClThreads) k_noise_fit(FitArgs a) {
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank(), w = blockIdx.y;
  __shared__ ClusterSmem sm;
  __shared__ int base[32];
  const int nwin = a.nwin, s0 = a.win_s0[w];
  if (threadIdx.x == 0) {
    int t = 0;
    for (int k = 0; k < nwin; ++k) {
      base[k] = t;
      t += a.nleaf[s0 + k];
    }
    base[nwin] = t;
  }
  __syncthreads();
  const int N = base[nwin];
  const int lo = (int)((long long)N * rank / kCl), hi = (int)((long long)N * (rank + 1) / kCl);
  const size_t per = (size_t)nwin * a.maxNodes;
  double* X = a.x + (size_t)w * per;
  double* Y = a.y + (size_t)w * per;
  unsigned long long* K = a.key + (size_t)w * per;
  const double um = a.win_norm[w], um2 = um * um;
  for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    int k = 0;
    while (k + 1 < nwin && i >= base[k + 1]) ++k;
    const size_t f = (size_t)(s0 + k);
    const int li = i - base[k];
    const int dp = a.dup[f * a.maxNodes + li];
    const int src = dp >= 0 ? dp : li;
    X[i] = a.mean[(size_t)a.win_pair[(size_t)w * nwin + k] * a.maxNodes + src];
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
    cluster_sums(cl, s, sm);
    p0 = s[0] * s[3] - s[1] * s[2];
    const double aux = s[0] * s[4] - s[1] * s[1];
    p0 = (fabs(aux) < kEps) ? a0 : p0 / aux;
    p1 = s[2] - p0 * s[1];
    p1 = (fabs(aux) < kEps) ? b0 : p1 / s[0];
    double se[1] = {0.0};
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      const double r = Y[i] - (X[i] * p0 + p1);
      se[0] += fabs(r);
      K[i] = okey(r);
    }
    cluster_sums(cl, se, sm);  // its syncs also publish K
    if ((fabs(a0 - p0) < kTol && fabs(b0 - p1) < kTol) || se[0] / (double)N < kTol) break;
    a0 = p0;
    b0 = p1;
    unsigned long long r0, r1;
    cluster_select2(cl, [&](int i) { return K[i]; }, lo, hi, mq - 1, N - mq - 1, sm, r0, r1);
    q0 = p0;
    q1 = p1;
    dd = (ovalue(r1) - ovalue(r0)) + kEps;
  }
  // mu: smallest leaf mean (method 4) or the mode of the leaf means (3)
  double mn = 1e300, mx = -1e300;
  for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    mn = fmin(mn, X[i]);
    mx = fmax(mx, X[i]);
  }
  mn = -cluster_max(cl, -mn, sm);
  mx = cluster_max(cl, mx, sm);
  // mu and sigma by the noise method (noise.hpp:115-147)
  int* h = a.hist + (size_t)w * (per + 1);
  unsigned long long* fk = a.fkey + (size_t)w * (per + 1);
  int* fi = a.fidx + (size_t)w * (per + 1);
  __shared__ double s_res[2];
  // ComputeMode (noise.hpp:272-297) of all N values v(i) taken in the
  // means-sorted order: the most frequent rounded value round(v N / max),
  // ties going to the value whose first occurrence (least (mean, index))
  // comes first.  A histogram over the N + 1 rounded values.
  auto mode_all = [&](auto v, double vmax, bool by_value) -> double {
    const double dyn = (double)N;
    for (int t = lo + threadIdx.x; t < (rank + 1 == kCl ? N + 1 : hi); t += blockDim.x) {
      h[t] = 0;
      fk[t] = ~0ull;
      fi[t] = 0x7fffffff;
    }
    __threadfence();
    cl.sync();
    auto bin = [&](int t) { return (int)fmin(fmax(round(v(t) * dyn / vmax), 0.0), dyn); };
    for (int t = lo + threadIdx.x; t < hi; t += blockDim.x) {
      const int b = bin(t);
      atomicAdd(&h[b], 1);
      if (!by_value) atomicMin(&fk[b], okey(X[t]));
    }
    __threadfence();
    cl.sync();
    if (!by_value) {
      for (int t = lo + threadIdx.x; t < hi; t += blockDim.x) {
        const int b = bin(t);
        if (okey(X[t]) == fk[b]) atomicMin(&fi[b], t);
      }
      __threadfence();
      cl.sync();
    }
    if (threadIdx.x == 0) {
      int best = 0, bc = -1;
      for (int t = 0; t <= N; ++t) {
        // by value (sorted values): the smallest of the most frequent;
        // else the one whose first occurrence comes first
        const bool better = h[t] > bc ||
                            (!by_value && h[t] == bc && bc > 0 &&
                             (fk[t] < fk[best] || (fk[t] == fk[best] && fi[t] < fi[best])));
        if (better) {
          bc = h[t];
          best = t;
        }
      }
      s_res[0] = (double)best * vmax / dyn;
    }
    __syncthreads();
    const double r = s_res[0];
    cl.sync();  // the scratch is reused by the next call
    return r;
  };
  double mu = a.mu_c, sigma = a.sigma_c;
  if (a.method == 1) {
    // the K = round(0.05 L) + 1 leaves of least mean (L = Nx Ny / N, integer
    // division), modes of their means and of their variances; K is clamped to
    // N (beyond N the reference reads past its arrays)
    const int L = (int)(((long long)a.nx * a.nx) / N);
    const int K = min(N, (int)llround(0.05 * L) + 1);
    unsigned long long tk, tk2;
    cluster_select2(cl, [&](int t) { return okey(X[t]); }, lo, hi, K - 1, K - 1, sm, tk, tk2);
    int* cnt = fi;  // count of candidates, then their indices
    if (rank == 0 && threadIdx.x == 0) cnt[0] = 0;
    __threadfence();
    cl.sync();
    for (int t = lo + threadIdx.x; t < hi; t += blockDim.x)
      if (okey(X[t]) <= tk) {
        const int slot = atomicAdd(&cnt[0], 1);
        if (slot < (int)per) cnt[1 + slot] = t;
      }
    __threadfence();
    cl.sync();
    if (rank == 0 && threadIdx.x == 0) {
      const int nc = min(cnt[0], (int)per);
      int* idx = cnt + 1;
      for (int p = 1; p < nc; ++p)  // order by (mean, index)
        for (int q = p; q > 0; --q) {
          const unsigned long long ka = okey(X[idx[q - 1]]), kb = okey(X[idx[q]]);
          if (ka < kb || (ka == kb && idx[q - 1] < idx[q])) break;
          const int t = idx[q];
          idx[q] = idx[q - 1];
          idx[q - 1] = t;
        }
      auto mode_small = [&](auto v, int n) {  // ComputeMode as written, O(n^2)
        double M = v(0);
        for (int t = 1; t < n; ++t) M = fmax(M, v(t));
        const double dyn = (double)n;
        int maxCount = 0;
        double maxValue = 0.0;
        for (int t = 0; t < n; ++t) {
          const double at = round(v(t) * dyn / M);
          int c = 0;
          for (int u = 0; u < n; ++u) c += round(v(u) * dyn / M) == at;
          if (c > maxCount) {
            maxCount = c;
            maxValue = at;
          }
        }
        return maxValue * M / dyn;
      };
      const int n = min(K, nc);
      s_res[0] = mode_small([&](int t) { return X[idx[t]]; }, n);
      s_res[1] = mode_small([&](int t) { return Y[idx[t]]; }, n);
    }
    __syncthreads();
    if (mu < 0) mu = s_res[0];
    if (sigma < 0) sigma = sqrt(s_res[1]);
  } else if (a.method == 2) {
    double ymx = -1e300;
    for (int t = lo + threadIdx.x; t < hi; t += blockDim.x) ymx = fmax(ymx, Y[t]);
    ymx = cluster_max(cl, ymx, sm);
    const double mmode = mode_all([&](int t) { return X[t]; }, mx, true);
    const double dSi = mode_all([&](int t) { return Y[t]; }, ymx, false);
    if (mu < 0) mu = mmode;
    if (sigma < 0) sigma = sqrt(fmax(dSi, fmax(p1 + p0 * dSi, 0.0)));
  } else if (a.method == 3) {
    const double mmode = mode_all([&](int t) { return X[t]; }, mx, true);
    if (mu < 0) mu = mmode;
    if (sigma < 0) sigma = sqrt(fabs(p1 + p0 * mu));
  } else {
    if (mu < 0) mu = mn;
    if (sigma < 0) sigma = sqrt(fabs(p1 + p0 * mu));
  }
  if (rank == 0 && threadIdx.x == 0) {
    const double alpha = a.alpha_c >= 0 ? a.alpha_c : p0;
    a.est[(size_t)w * 3] = alpha;
    a.est[(size_t)w * 3 + 1] = mu;
    a.est[(size_t)w * 3 + 2] = sigma;
  }
}

// The estimates of a window batch into its window constants: caller-side
// values, then the risk's binding PGURE(u, p, alpha, sigma, mu, ...)
// (pgure.hpp:26-30).
__global__ void k_noise_apply(Problem pb, DeviceBuffers d, const double* est, int win0) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= pb.W) return;
  WinConst& wc = d.wc[w];
  const double* e = est + (size_t)(wc.t - win0) * 3;
  wc.est_alpha = e[0];
  wc.est_mu = e[1];
  wc.est_sigma = e[2];
  wc.alpha = e[0];
  if (pb.compat & PGSVT_COMPAT_SWAP_MU_SIGMA) {
    wc.mu = e[2];
    wc.sigma = e[1];
  } else {
    wc.mu = e[1];
    wc.sigma = e[2];
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
  k_leaf_stats_big<<<dim3(kCl * nf.maxBig, nimg), kClThreads, 0, s>>>(
      src, nf.leaf, nf.big, nf.nbig, nf.dup, nf.maxNodes, nf.stats);
  return cudaGetLastError();
}

cudaError_t launch_noise_pass(const NoiseFrames& nf, const NoisePass& np, const float* xs,
                              const double* x64, int S, cudaStream_t s) {
  PairArgs pa{FrameSrc{xs, x64, S}, nf.leaf, nf.nleaf, nf.dup, nf.big, nf.nbig, nf.stats,
              nf.maxNodes, np.pair_frame, np.pair_norm, np.mean};
  if (np.npairs > 0) {
    k_leaf_mean_warp<<<dim3((nf.maxNodes + 3) / 4, np.npairs), 128, 0, s>>>(pa);
    k_leaf_mean_big<<<dim3(kCl * nf.maxBig, np.npairs), kClThreads, 0, s>>>(pa);
  }
  FitArgs fa{nf.nleaf, nf.dup, nf.stats, np.mean, np.win_pair, np.win_s0, np.win_norm,
             nf.maxNodes, np.nwin, np.method, np.alpha_c, np.mu_c, np.sigma_c, np.x, np.y,
             np.key, np.hist, np.fkey, np.fidx, np.est, S};
  k_noise_fit<<<dim3(kCl, np.nwindows), kClThreads, 0, s>>>(fa);
  return cudaGetLastError();
}

cudaError_t launch_noise_apply(const Problem& pb, const DeviceBuffers& d, const double* est,
                               int win0, cudaStream_t s) {
  k_noise_apply<<<(pb.W + 63) / 64, 64, 0, s>>>(pb, d, est, win0);
  return cudaGetLastError();
}

}  // namespace pgsvt
