// eval.cu — singular-value thresholding, overlap averaging and the PGURE risk.
//
// Reference: SVT::Reconstruct (svt.hpp:121-167), PGURE::CalculatePGURE
// (pgure.hpp:120-137) and the lambda search driven by PGURE::Optimize
// (pgure.hpp:197-237).
//
// The risk of one window at lambda is
//   R = (1/N) [ sum (Uh-U)^2 - (a+m) sum U + (2/e1) sum d1 (aU-am+s^2)(U1-Uh)
//               - (2 s^2 a / e2^2) sum d2 (U2p - 2 Uh + U2m) + 2 m sum Uh + m ] - s^2
// (a, m, s are PGURE's alpha, mu, sigma members).  Every term except the first
// is linear in a reconstructed cube, and each reconstructed cube is an
// overlap average Uc = (sum_p scatter(R_p)) / cnt with R_p = sum_i g_i u_i v_i^T.
// Hence  sum_x L(x) Uc(x) = sum_p sum_i g_i (u_i^T G_p v_i)  with the
// lambda-independent field G = L / cnt gathered along patch p's trajectory:
// the SVD epilogue stores h_i = u_i^T G_p v_i once, and a lambda evaluation
// needs only sum_i g_i(lambda) h_i per patch and copy.  Only sum (Uh-U)^2 needs
// the clean reconstruction voxel by voxel: copy 0 is rebuilt and scattered
// into a fixed-point accumulator (int32 at 2^-20, or int64 at 2^-32 when one
// voxel can collect every patch, as with the zero-motion quirk), which makes
// the sums independent of the order of the atomics, so the whole search is
// deterministic.
#include <algorithm>

#include <map>
#include <mutex>
#include <utility>

#include "pgsvt_internal.h"

namespace pgsvt {

namespace {

__device__ __forceinline__ double warp_sum_d(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---- coverage counts (weights in svt.hpp:157-159)
//
// A warp's 32 patches are half of an 8 x 8 tile of grid positions (the
// processing order), so their blocks in slice k overlap: the warp counts them
// in a shared-memory tile and adds the tile with one global atomic per
// touched pixel (plain global atomics when the footprint does not fit).
constexpr int kCountTile = 512;

__global__ void __launch_bounds__(128) k_counts(Problem pb, DeviceBuffers d) {
  const Geometry& g = pb.g;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y, w = blockIdx.z;
  const int lane = threadIdx.x & 31;
  __shared__ int tiles[4][kCountTile];
  int* tile = tiles[threadIdx.x >> 5];
  const bool live = p < g.NP;
  int y = 0, x = 0;
  if (live) {
    const uint32_t pc = d.pos[((size_t)w * g.nwin + k) * g.P + d.plist[p]];
    y = pc & 0xffffu;
    x = pc >> 16;
  }
  const int y0 = __reduce_min_sync(0xffffffffu, live ? y : 0x7fffffff);
  const int y1 = __reduce_max_sync(0xffffffffu, live ? y : -1);
  const int x0 = __reduce_min_sync(0xffffffffu, live ? x : 0x7fffffff);
  const int x1 = __reduce_max_sync(0xffffffffu, live ? x : -1);
  if (y1 < 0) return;  // no live patch in this warp (warp-uniform)
  int32_t* c = d.cnt + (size_t)w * g.cube() + (size_t)k * g.F();
  const int th = y1 - y0 + g.bs, tw = x1 - x0 + g.bs;
  if (th * tw > kCountTile) {  // warp-uniform
    if (live)
      for (int cc = 0; cc < g.bs; ++cc)
        for (int r = 0; r < g.bs; ++r) atomicAdd(c + (y + r) + (size_t)(x + cc) * g.S, 1);
    return;
  }
  for (int i = lane; i < th * tw; i += 32) tile[i] = 0;
  __syncwarp();
  if (live)
    for (int cc = 0; cc < g.bs; ++cc)
      for (int r = 0; r < g.bs; ++r) atomicAdd(tile + (y - y0 + r) + (x - x0 + cc) * th, 1);
  __syncwarp();
  for (int i = lane; i < th * tw; i += 32) {
    const int v = tile[i];
    if (v) atomicAdd(c + (y0 + i % th) + (size_t)(x0 + i / th) * g.S, v);
  }
}

// ---- lambda-independent fields and sum(U)
__global__ void k_fields(Problem pb, DeviceBuffers d) {
  const Geometry& g = pb.g;
  const int w = blockIdx.y;
  const size_t C = g.cube();
  const WinConst& wc = d.wc[w];
  const float* u = d.u + (size_t)w * C;
  const int32_t* cnt = d.cnt + (size_t)w * C;
  const double a = wc.alpha, m = wc.mu, s2 = wc.sigma * wc.sigma;
  const double c2 = 2 * s2 * a / (wc.eps2 * wc.eps2);
  const bool intd1 = pb.compat & 0x4;
  const int8_t* d1 = d.d1 + (size_t)w * d.probe_stride;
  const int8_t* d2c = d.d2code + (size_t)w * d.probe_stride;
  double su = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < C;
       i += (size_t)gridDim.x * blockDim.x) {
    const double uv = u[i];
    su += uv;
    if (!pb.optimize) continue;
    const int n = cnt[i];
    const double ic = n > 0 ? 1.0 / n : 0.0;
    const double dl2 = d2c[i] ? d.d2neg : d.d2pos;
    double l0 = 2 * c2 * dl2 + 2 * m;
    if (!intd1) {
      const double l1 = (2 / wc.eps1) * d1[i] * ((a * uv - a * m) + s2);
      l0 -= l1;
      d.fld1[(size_t)w * C + i] = (float)(l1 * ic);
    }
    d.fld0[(size_t)w * C + i] = (float)(l0 * ic);
    d.fld2[(size_t)w * C + i] = (float)(-c2 * dl2 * ic);
  }
  su = warp_sum_d(su);
  __shared__ double sm[32];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = su;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += sm[q];
    d.part_mse[(size_t)w * gridDim.x + blockIdx.x] = t;  // reused as scratch
  }
}

__global__ void k_sum_u(Problem pb, DeviceBuffers d, int nblk) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= pb.W) return;
  double t = 0.0;
  for (int b = 0; b < nblk; ++b) t += d.part_mse[(size_t)w * nblk + b];
  d.wc[w].sum_u = t;
}

// ---- search state machine (one thread per window)
//
// Bracketed batch grid search, identical to the oracle's: round 0 places K
// points geometrically over [lo, hi]; each later round places K/2 points
// evenly inside the bracket formed by the neighbours of the best point so far
// (K points in a narrow search, or when the bracket reaches down to zero).  A
// hint (a given or learned proposal) runs a narrow search first: hint_K
// points over [hint/span, hint*span] and hint_rounds refinements.  When the
// best point of its grid lies on an edge and the neighbouring point's risk
// is more than hint_flat (relative) above it, the plain search runs instead
// and the better of the two results is kept.

struct Sch {
  __device__ static void grid(SearchState& s, double lo, double hi) {
    const int K = s.K;
    for (int j = 0; j < K; ++j)
      s.next[j] = (K == 1) ? hi : lo * pow(hi / lo, (double)j / (double)(K - 1));
    s.nnext = K;
    s.first = 1;
  }
  // batch_search's set-up: K shrinks to the evaluation budget
  __device__ static void phase(SearchState& s, int ph, int K0, int max_eval, int rounds,
                               int zero_lo) {
    s.phase = ph;
    s.K = (max_eval < K0) ? max(1, max_eval) : K0;
    s.max_eval = max_eval;
    s.rounds = rounds;
    s.zero_lo = zero_lo;
    s.rd = 0;
    s.evals_phase = 0;
    s.npts = 0;
    s.best = 0;
    s.nsent = 0;
    s.sent_risk = INFINITY;
  }
  __device__ static int best(const SearchState& s) {
    int b = 0;
    for (int i = 1; i < s.npts; ++i)
      if (s.risk[i] < s.risk[b]) b = i;
    return b;
  }
};

// The narrow grid inherits the plain search's bounds: a grid reaching below
// the plain grid's bottom (upper * 1e-4) may refine down to 0 as the plain
// search does, and a grid clipped at `upper` ends there as the plain one
// does; a best point on such a bound is a result, not a miss.  Its first
// round also evaluates the plain grid's ends that it does not reach
// (sentinels, kept out of the point list): one of them below the narrow
// grid's best sends the search to the plain grid.
__device__ void start_narrow(SearchState& s, const Problem& pb, double upper, double hint) {
  const double h = fmin(hint, upper);
  const double lo = h / pb.hint_span, hi = fmin(upper, h * pb.hint_span);
  Sch::phase(s, 1, pb.hint_K, pb.max_evals, pb.hint_rounds, lo <= upper * 1e-4 ? 1 : 0);
  Sch::grid(s, lo, hi);
  const int room = min(pb.K - s.nnext, pb.max_evals - s.nnext);
  if (room > 0 && lo > upper * 1e-4) s.next[s.nnext + s.nsent++] = upper * 1e-4;
  if (room > s.nsent && hi < upper) s.next[s.nnext + s.nsent++] = upper;
  s.nnext += s.nsent;
}

__global__ void k_search_init(Problem pb, DeviceBuffers d) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= pb.W) return;
  const Geometry& g = pb.g;
  WinConst& wc = d.wc[w];
  SearchState& s = d.st[w];
  s.npts = 0;
  s.nnext = 0;
  s.evals_total = 0;
  s.best = 0;
  s.final_lambda = pb.lambda_user;
  s.final_risk = 0.0;
  s.hint_lambda = s.hint_risk = 0.0;
  s.nsent = 0;
  s.sent_risk = INFINITY;
  if (!pb.optimize) {
    s.done = 1;
    return;
  }
  // pguresvt.hpp:139-141
  const double OoN = 1.0 / (double)((uint32_t)g.S * (uint32_t)g.S * (uint32_t)g.Ntc);
  double start = (pb.lambda_user >= 0.0) ? pb.lambda_user : wc.sum_u * OoN;
  start = fmax(0.0, start);
  wc.start = start;
  wc.upper = fmax(100.0, start);
  s.done = 0;
  if (pb.nfixed > 0) {  // a given list: one round, no refinement
    Sch::phase(s, 0, pb.nfixed, pb.nfixed, 0, 0);
    for (int j = 0; j < pb.nfixed; ++j) s.next[j] = pb.fixed[j];
    s.nnext = pb.nfixed;
    s.first = 1;
  } else if (pb.hint > 0) {
    start_narrow(s, pb, wc.upper, pb.hint);
  } else {
    Sch::phase(s, 0, pb.K, pb.max_evals, pb.rounds, 1);
    Sch::grid(s, wc.upper * 1e-4, wc.upper);
  }
}

// Narrow searches around the learned proposals y = log10(lambda/upper).
__global__ void k_search_hint(Problem pb, DeviceBuffers d) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= pb.W) return;
  SearchState& s = d.st[w];
  if (s.done) return;
  const double upper = d.wc[w].upper;
  const double y = fmin(0.0, fmax(-6.0, (double)d.prop[w]));  // NaN -> -6
  start_narrow(s, pb, upper, upper * pow(10.0, y));
}

__device__ void search_finish(SearchState& s, unsigned long long* counters) {
  atomicAdd(counters + 3, (unsigned long long)s.evals_total);
  const int b = s.best;
  double lam = s.lam[b], risk = s.risk[b];
  if (s.phase == 2 && !(risk < s.hint_risk)) {
    lam = s.hint_lambda;
    risk = s.hint_risk;
  }
  s.final_lambda = lam;
  s.final_risk = risk;
  s.done = 1;
  s.nnext = 0;
}

// Risk of lambda slot j of window w (pgure.hpp:136) from the block
// partials, reduced by the calling block in a fixed order.
__device__ double block_sum(const double* v, int n, double* red) {
  double t = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) t += v[i];
  red[threadIdx.x] = t;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  const double r = red[0];
  __syncthreads();
  return r;
}

// Merge the risks of the pending round and schedule the next one.
// One block per window: the partial sums are reduced in parallel, thread 0
// advances the search state.
__global__ void __launch_bounds__(256) k_search_step(Problem pb, DeviceBuffers d) {
  const int w = blockIdx.x;
  SearchState& s = d.st[w];
  if (s.done) return;
  __shared__ double red[256];
  __shared__ double risk[kMaxK];
  const Geometry& g = pb.g;
  const WinConst& wc = d.wc[w];
  const double N = (double)g.S * g.S * g.nwin;
  const double a = wc.alpha, m = wc.mu, s2 = wc.sigma * wc.sigma;
  const int nn = s.nnext;
  for (int j = 0; j < nn; ++j) {
    const double lin = block_sum(d.part_lin + ((size_t)w * pb.K + j) * d.nblk_eval, d.nblk_eval, red);
    const double mse = block_sum(d.part_mse + ((size_t)w * pb.K + j) * d.nblk_mse, d.nblk_mse, red);
    if (threadIdx.x == 0) risk[j] = (1.0 / N) * (mse + lin - (a + m) * wc.sum_u + m) - s2;  // pgure.hpp:136
  }
  if (threadIdx.x != 0) return;
  const double prev_best = s.npts > 0 ? s.risk[s.best] : 0.0;
  for (int j = nn - s.nsent; j < nn; ++j) s.sent_risk = fmin(s.sent_risk, risk[j]);
  for (int j = 0; j < nn - s.nsent; ++j) {
    int pos = s.npts;  // keep lambda ascending, new points after equal ones
    while (pos > 0 && s.lam[pos - 1] > s.next[j]) {
      s.lam[pos] = s.lam[pos - 1];
      s.risk[pos] = s.risk[pos - 1];
      --pos;
    }
    s.lam[pos] = s.next[j];
    s.risk[pos] = risk[j];
    ++s.npts;
  }
  s.evals_phase += s.nnext;
  s.evals_total += s.nnext;
  s.nnext = 0;
  const int b = Sch::best(s);
  s.best = b;
  const bool grid_round = s.first != 0;
  if (s.first) {
    s.first = 0;
    const bool bound = (b == 0 && s.zero_lo) || (b == s.npts - 1 && s.lam[b] >= wc.upper);
    const bool edge = (b == 0 || b == s.npts - 1) && !bound;
    bool steep = edge;
    if (edge && s.npts >= 2) {
      const int nb = (b == 0) ? 1 : s.npts - 2;
      steep = !(s.risk[nb] - s.risk[b] <= pb.hint_flat * fabs(s.risk[b]));
    }
    const bool beaten = s.sent_risk < s.risk[b];  // a plain-grid end does better
    s.nsent = 0;
    if (s.phase == 1 && (steep || beaten)) {  // proposal not bracketed: plain search
      s.hint_lambda = s.lam[b];
      s.hint_risk = s.risk[b];
      const int left = pb.max_evals > s.evals_phase ? pb.max_evals - s.evals_phase : 1;
      Sch::phase(s, 2, pb.K, left, pb.rounds, 1);
      Sch::grid(s, wc.upper * 1e-4, wc.upper);
      return;
    }
  } else {
    ++s.rd;
  }
  const double blo = (b > 0) ? s.lam[b - 1] : (s.zero_lo ? 0.0 : s.lam[b]);
  const double bhi = (b + 1 < s.npts) ? s.lam[b + 1] : s.lam[b];
  if (!grid_round && prev_best - s.risk[b] <= pb.tol * fabs(s.risk[b]) &&
      bhi - blo <= kNarrowBracket * s.lam[b]) {
    search_finish(s, d.counters);  // no progress and a narrow bracket
    return;
  }
  // refinement rounds of the plain search place half the grid's points,
  // unless the bracket reaches down to the zero bound
  const int Kr = (s.phase == 1 || (b == 0 && s.zero_lo)) ? s.K : max(2, s.K / 2);
  if (s.rd >= s.rounds || s.evals_phase + Kr > s.max_eval) {
    search_finish(s, d.counters);
    return;
  }
  if (!(bhi > blo)) {
    search_finish(s, d.counters);
    return;
  }
  for (int i = 0; i < Kr; ++i)
    s.next[i] = blo + (bhi - blo) * (double)(i + 1) / (double)(Kr + 1);
  s.nnext = Kr;
}

// ---- fixed-point accumulators
template <typename T>
struct Acc;
template <>
struct Acc<int> {  // 2^-20: one voxel holds |sum| < 2048
  static constexpr float kScale = 1048576.f;
  __device__ static int fix(float v) { return __float2int_rn(v * kScale); }
  __device__ static float unfix(int a) { return (float)a * (1.f / kScale); }
  __device__ static int from_tile(int t) { return t; }
  __device__ static void add(int* p, int v) { atomicAdd(p, v); }
};
template <>
struct Acc<unsigned long long> {  // 2^-32
  __device__ static long long fix(float v) { return fix32(v); }
  __device__ static float unfix(unsigned long long a) { return unfix32((long long)a); }
  __device__ static long long from_tile(int t) { return (long long)t * 4096; }
  __device__ static void add(unsigned long long* p, long long v) {
    atomicAdd(p, (unsigned long long)v);
  }
};

// ---- one evaluation round: shrink, linear terms, rebuild + scatter of copy 0
//
// Block = 32 kept patches (an 8 x 4 half of an 8 x 8 tile of grid positions,
// see the patch order in capi.cu; one per lane) x nwin warps, small enough
// (at most about 100 KB of shared memory, 64 registers) for two blocks per
// SM when nwin <= 16.  Phase A spreads the (lambda, copy) pairs over all
// warps: the shrunk singular values g_i (svt.hpp:135-143) of copy 0 go to
// shared memory and sum_i g_i h_i of every copy to per-lane partials.
// Phase B: warp k rebuilds column k (trajectory slice k) of its lanes'
// patches from the live singular triplets.  The 32 rebuilt blocks of one
// slice overlap heavily, so each warp sums them into a shared-memory tile in
// int32 fixed point (2^-20, order-free) and adds the tile to the accumulator
// with one atomic per touched pixel.

constexpr int kTileMax = 512;      // pixels of a warp's shared-memory tile
constexpr float kTileBound = 60.f; // |value| above this bypasses the tile (32 x 60 < 2048)

// launch bounds of k_eval: a block is 32 x nwin threads, nwin <= MAXW;
// windows up to 16 frames run two blocks per SM

template <int BS, typename AccT, bool STAGE = false, int MAXW = 21>
__global__ void __launch_bounds__(32 * MAXW, MAXW <= 16 ? 2 : 1)
    k_eval(Problem pb, DeviceBuffers d, int final_pass) {
  const int nb = BS > 0 ? BS : pb.g.bs;  // BS == 0: any side (9..16)
  const int M = nb * nb;
  constexpr int PB = kEvalPatches;  // patches per block
  constexpr int H = PB / 32;         // patches per lane
  const Geometry& g = pb.g;
  const int w = blockIdx.y;
  const SearchState& st = d.st[w];
  const int nl = final_pass ? 1 : st.nnext;
  if (!final_pass && (st.done || nl == 0)) return;
  const int lane = threadIdx.x & 31, k = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  const int NC = g.NC;
  const size_t NP = g.NP;
  const bool lin_terms = pb.optimize && !final_pass;
  const int ncp = lin_terms ? d.ncopies : 1;
  extern __shared__ float sg[];  // g of copy 0 [nl][NC][PB], lin [nl][4][PB], tiles
  float* slin = sg + (size_t)nl * NC * PB;
  int* tiles = (int*)(slin + (size_t)nl * 4 * PB);
  __shared__ int srmax[kMaxK];
  const WinConst& wc = d.wc[w];
  int* tile = tiles + (size_t)k * kTileMax;
  for (int i = lane; i < kTileMax; i += 32) tile[i] = 0;
  if (threadIdx.x < kMaxK) srmax[threadIdx.x] = 0;
  __syncthreads();
  // phase A: (lambda, copy, half) tasks over all warps
  for (int task = k; task < nl * ncp * H; task += nwarps) {
    const int h = task % H, jc = task / H;
    const int j = jc / ncp, c = jc % ncp;
    const int slot = h * 32 + lane;
    const int p = blockIdx.x * PB + slot;
    const bool live = p < g.NP;
    const float lam = (float)(final_pass ? st.final_lambda : st.next[j]);
    const float* sv = d.sv + ((size_t)w * 4 + c) * NC * NP;
    const float* hv = d.hv + ((size_t)w * 4 + c) * NC * NP;
    const float smax = live ? sv[p] : 0.f;  // sorted: column 0 is the largest
    float lin = 0.f;
    int r0 = 0;
    for (int i = 0; i < NC; ++i) {
      const float s = live ? sv[(size_t)i * NP + p] : 0.f;
      float th;
      if (pb.expw) th = fabsf(smax * expf(-0.5f * lam * (s * s)));  // svt.hpp:137
      else th = lam;                                                // svt.hpp:142
      const float gi = fmaxf(fabsf(s) - th, 0.f);
      if (c == 0) {
        sg[((size_t)j * NC + i) * PB + slot] = gi;
        r0 += gi > 0.f;
      }
      if (lin_terms && live) lin = fmaf(gi, hv[(size_t)i * NP + p], lin);
    }
    slin[((size_t)j * 4 + c) * PB + slot] = lin;
    if (c == 0) {
      for (int o = 16; o > 0; o >>= 1) r0 = max(r0, __shfl_xor_sync(0xffffffffu, r0, o));
      if (lane == 0) atomicMax(&srmax[j], r0);
    }
  }
  __syncthreads();
  // patches of at most 16 rows: the left singular vectors of the block's
  // patches, up to the largest rank any lambda of the round keeps, staged in
  // shared memory once ([i][e][PB]); every slice warp and every lambda reads
  // them there instead of through L1
  constexpr bool kStage = STAGE && BS > 0 && BS * BS <= 16;
  float* Us = (float*)(tiles + (size_t)nwarps * kTileMax);
  if constexpr (kStage) {
    int R = 0;
    for (int j = 0; j < nl; ++j) R = max(R, srmax[j]);
    const float* U0w = d.U0 + (size_t)w * NC * M * NP;
    for (int t = threadIdx.x; t < R * M * PB; t += blockDim.x) {
      const int slot = t % PB, ie = t / PB;  // ie = i * M + e
      const int p = blockIdx.x * PB + slot;
      Us[t] = p < g.NP ? __ldg(U0w + (size_t)ie * NP + p) : 0.f;
    }
    __syncthreads();
  }
  if (lin_terms)
    for (int j = k; j < nl; j += nwarps) {
      float lin = 0.f;
      for (int h = 0; h < H; ++h)
        for (int c = 0; c < ncp; ++c) lin += slin[((size_t)j * 4 + c) * PB + h * 32 + lane];
      const double t = warp_sum_d((double)lin);
      if (lane == 0) d.part_lin[((size_t)w * pb.K + j) * d.nblk_eval + blockIdx.x] = t;
    }
  if (k >= g.nwin) return;
  if (final_pass == 1 && k != wc.out_slice) return;  // 2: every slice
  int y[H], x[H], nlive[H];
  bool live[H];
  int y0 = 1 << 30, y1 = -1, x0 = 1 << 30, x1 = -1;
#pragma unroll
  for (int h = 0; h < H; ++h) {
    const int p = blockIdx.x * PB + h * 32 + lane;
    live[h] = p < g.NP;
    y[h] = x[h] = nlive[h] = 0;
    if (live[h]) {
      const uint32_t pc = d.pos[((size_t)w * g.nwin + k) * g.P + d.plist[p]];
      y[h] = pc & 0xffffu;
      x[h] = pc >> 16;
      nlive[h] = d.nlive0[(size_t)w * NP + p];
      y0 = min(y0, y[h]);
      y1 = max(y1, y[h]);
      x0 = min(x0, x[h]);
      x1 = max(x1, x[h]);
    }
  }
  // the warp's footprint in this slice
  for (int o = 16; o > 0; o >>= 1) {
    y0 = min(y0, __shfl_xor_sync(0xffffffffu, y0, o));
    y1 = max(y1, __shfl_xor_sync(0xffffffffu, y1, o));
    x0 = min(x0, __shfl_xor_sync(0xffffffffu, x0, o));
    x1 = max(x1, __shfl_xor_sync(0xffffffffu, x1, o));
  }
  // Two lambda values per pass share every load of the left and right
  // vectors (patches of at most 16 rows, whose left vectors are staged in
  // shared memory; the larger forms keep one value per pass within their
  // registers); each has its own half of the warp's tile.  The tile's column
  // stride is padded to 8 (mod 16) where the footprint allows it, so that
  // the warp's four 8-row lane groups (one grid column each) start 0, 8, 16,
  // 24 (or 0, 24, 16, 8) banks apart.
  const int th = y1 - y0 + nb, tw = x1 - x0 + nb;
  constexpr int kHalfTile = kTileMax / 2;
  int ths = th <= 8 ? 8 : 8 + 16 * ((th - 8 + 15) / 16);
  if (ths * tw > kHalfTile) ths = th;
  const bool use_tile = (y1 >= 0) && ths * tw <= kHalfTile;
  const float* U0 = d.U0 + (size_t)w * NC * M * NP;
  const float* V0 = d.V0 + (size_t)w * NC * g.nwin * NP;
  AccT* accw = (AccT*)d.acc;
  constexpr int CH = (BS > 0 && BS * BS < 16) ? BS * BS : 16;  // rows rebuilt per pass
  constexpr bool kPair = kStage;
  for (int j0 = 0; j0 < nl; j0 += kPair ? 2 : 1) {
    const bool two = kPair && j0 + 1 < nl;
    AccT* acc[2];
    int* tl[2] = {tile, tile + kHalfTile};
#pragma unroll
    for (int jj = 0; jj < 2; ++jj)
      acc[jj] = accw + (((size_t)w * pb.K + (two ? j0 + jj : j0)) * g.nwin + k) * g.F();
    const int rj = max(srmax[j0], two ? srmax[j0 + 1] : 0);
#pragma unroll 1
    for (int h = 0; h < H; ++h) {
      if (!live[h]) continue;
      const int p = blockIdx.x * PB + h * 32 + lane;
      const int rm = min(rj, nlive[h]);
      const float* sg0 = sg + (size_t)j0 * NC * PB + h * 32 + lane;
      const float* sg1 = sg + (size_t)(two ? j0 + 1 : j0) * NC * PB + h * 32 + lane;
#pragma unroll 1
      for (int e0 = 0; e0 < M; e0 += CH) {
        float col[2][CH];
#pragma unroll
        for (int e = 0; e < CH; ++e) col[0][e] = col[1][e] = 0.f;
        for (int i = 0; i < rm; ++i) {
          const float v = V0[((size_t)i * g.nwin + k) * NP + p];
          const float c0 = sg0[(size_t)i * PB] * v;
          const float c1 = two ? sg1[(size_t)i * PB] * v : 0.f;
          if (c0 == 0.f && c1 == 0.f) continue;
          if constexpr (kStage) {
            const float* ui = Us + ((size_t)i * M + e0) * PB + h * 32 + lane;
#pragma unroll
            for (int e = 0; e < CH; ++e)
              if (e0 + e < M) {
                const float u = ui[e * PB];
                col[0][e] = fmaf(c0, u, col[0][e]);
                col[1][e] = fmaf(c1, u, col[1][e]);
              }
          } else {
            const float* ui = U0 + ((size_t)i * M + e0) * NP + p;
#pragma unroll
            for (int e = 0; e < CH; ++e)
              if (e0 + e < M) {
                const float u = __ldg(ui + (size_t)e * NP);
                col[0][e] = fmaf(c0, u, col[0][e]);
                col[1][e] = fmaf(c1, u, col[1][e]);
              }
          }
        }
#pragma unroll
        for (int jj = 0; jj < 2; ++jj) {
          if (jj == 1 && !two) break;
#pragma unroll
          for (int e = 0; e < CH; ++e) {
            const int ee = e0 + e;
            const float val = col[jj][e];
            if (ee >= M || val == 0.f) continue;
            const int er = ee % nb, ec = ee / nb;
            if (use_tile && fabsf(val) <= kTileBound)
              atomicAdd(tl[jj] + (y[h] - y0 + er) + (x[h] - x0 + ec) * ths,
                        __float2int_rn(val * 1048576.f));
            else
              Acc<AccT>::add(acc[jj] + (y[h] + er) + (size_t)(x[h] + ec) * g.S, Acc<AccT>::fix(val));
          }
        }
      }
    }
    if (use_tile) {
      __syncwarp();
#pragma unroll
      for (int jj = 0; jj < 2; ++jj) {
        if (jj == 1 && !two) break;
        for (int t = lane; t < ths * tw; t += 32) {
          const int v = tl[jj][t];
          if (v != 0) {
            tl[jj][t] = 0;
            Acc<AccT>::add(acc[jj] + (y0 + t % ths) + (size_t)(x0 + t / ths) * g.S,
                           Acc<AccT>::from_tile(v));
          }
        }
      }
      __syncwarp();
    }
  }
}

// ---- sum over voxels of (Uh - U)^2 for every lambda of the round; clears acc
template <typename AccT, int KT>
__global__ void __launch_bounds__(256) k_mse(Problem pb, DeviceBuffers d) {
  const Geometry& g = pb.g;
  const int w = blockIdx.y;
  const SearchState& st = d.st[w];
  if (st.done || st.nnext == 0) return;
  const int nl = st.nnext;
  const size_t C = g.cube();
  const float* u = d.u + (size_t)w * C;
  const int32_t* cnt = d.cnt + (size_t)w * C;
  AccT* acc = (AccT*)d.acc + (size_t)w * pb.K * C;
  float part[KT];  // a thread sees about 16 voxels: FP32 partials, FP64 beyond
#pragma unroll
  for (int j = 0; j < KT; ++j) part[j] = 0.f;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < C;
       i += (size_t)gridDim.x * blockDim.x) {
    const int n = __ldg(cnt + i);
    const float uv = __ldg(u + i);
    const float inv = n > 0 ? 1.f / (float)n : 0.f;
    AccT av[KT];  // every load first: the clears below could alias them
#pragma unroll
    for (int j = 0; j < KT; ++j) av[j] = (j < nl) ? __ldcs(acc + (size_t)j * C + i) : (AccT)0;
#pragma unroll
    for (int j = 0; j < KT; ++j)
      if (j < nl) __stcs(acc + (size_t)j * C + i, (AccT)0);
#pragma unroll
    for (int j = 0; j < KT; ++j) {
      const float df = Acc<AccT>::unfix(av[j]) * inv - uv;
      if (j < nl) part[j] = fmaf(df, df, part[j]);
    }
  }
  __shared__ double sm[KT][8];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int j = 0; j < KT; ++j) {
    if (j >= nl) break;
    const double t = warp_sum_d((double)part[j]);
    if (lane == 0) sm[j][wid] = t;
  }
  __syncthreads();
  if (threadIdx.x < nl) {
    const int j = threadIdx.x;
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += sm[j][q];
    d.part_mse[((size_t)w * pb.K + j) * d.nblk_mse + blockIdx.x] = t;
  }
}

// ---- output slice and estimates (pguresvt.hpp:146-166)
template <typename AccT>
__global__ void k_output(Problem pb, DeviceBuffers d) {
  const Geometry& g = pb.g;
  const int w = blockIdx.y;
  const WinConst& wc = d.wc[w];
  const size_t F = g.F();
  AccT* acc = (AccT*)d.acc + ((size_t)w * pb.K * g.nwin + wc.out_slice) * F;
  const int32_t* cnt = d.cnt + (size_t)w * g.cube() + (size_t)wc.out_slice * F;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < F;
       i += (size_t)gridDim.x * blockDim.x) {
    const AccT a = acc[i];
    acc[i] = 0;
    const int n = cnt[i];
    double v = n > 0 ? (double)Acc<AccT>::unfix(a) / n : 0.0;
    if (!isfinite(v)) v = 0.0;
    d.Y[(size_t)wc.t * F + i] = v * wc.umax;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const int n = g.nimg;
    if (d.risk_out) d.risk_out[wc.t] = d.st[w].final_risk;
    if (pb.fixed_risk) {  // risks of the given list, in its order
      const SearchState& s = d.st[w];
      for (int j = 0; j < pb.nfixed; ++j) {
        double r = NAN;
        for (int i = 0; i < s.npts; ++i)
          if (s.lam[i] == pb.fixed[j]) r = s.risk[i];
        pb.fixed_risk[(size_t)wc.t * pb.nfixed + j] = r;
      }
    }
    if (d.evals_out) d.evals_out[wc.t] = (uint32_t)d.st[w].evals_total;
    d.est[wc.t] = d.st[w].final_lambda;
    d.est[wc.t + n] = wc.est_alpha;
    d.est[wc.t + 2 * (size_t)n] = wc.est_mu;
    d.est[wc.t + 3 * (size_t)n] = wc.est_sigma;
  }
}

// ---- whole reconstructed window v = acc / cnt (svt.hpp:163-164), window 0
template <typename AccT>
__global__ void k_cube_out(Problem pb, DeviceBuffers d, double* v) {
  const Geometry& g = pb.g;
  const size_t C = g.cube();
  AccT* acc = (AccT*)d.acc;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < C;
       i += (size_t)gridDim.x * blockDim.x) {
    const AccT a = acc[i];
    acc[i] = 0;
    const int n = d.cnt[i];
    double q = n > 0 ? (double)Acc<AccT>::unfix(a) / n : 0.0;
    v[i] = isfinite(q) ? q : 0.0;
  }
}

// ---- risks of the pending round without searching (component entry point)
__global__ void k_risk_collect(Problem pb, DeviceBuffers d, double* out) {
  const int w = 0;
  SearchState& s = d.st[w];
  const Geometry& g = pb.g;
  const WinConst& wc = d.wc[w];
  const double N = (double)g.S * g.S * g.nwin;
  const double a = wc.alpha, m = wc.mu, s2 = wc.sigma * wc.sigma;
  const int j = threadIdx.x;
  if (j < s.nnext) {
    double lin = 0.0, mse = 0.0;
    const double* pl = d.part_lin + ((size_t)w * pb.K + j) * d.nblk_eval;
    const double* pm = d.part_mse + ((size_t)w * pb.K + j) * d.nblk_mse;
    for (int b = 0; b < d.nblk_eval; ++b) lin += pl[b];
    for (int b = 0; b < d.nblk_mse; ++b) mse += pm[b];
    out[j] = (1.0 / N) * (mse + lin - (a + m) * wc.sum_u + m) - s2;
  }
}

// shared memory of a k_eval block; stage: the left vectors fit beside it
size_t eval_smem(const Geometry& g, int nl, int& stage) {
  const size_t base = (size_t)nl * (g.NC + 4) * kEvalPatches * sizeof(float) +
                      (size_t)g.nwin * kTileMax * sizeof(int);
  const size_t staged = g.bs <= 4 ? (size_t)g.NC * g.M * kEvalPatches * sizeof(float) : 0;
  stage = (staged > 0 && base + staged <= 227 * 1024) ? 1 : 0;
  return base + (stage ? staged : 0);
}

// Raise, never lower, a kernel's dynamic shared-memory limit on the current
// device.  k_eval's footprint depends on the lambda count of the round, and
// concurrent callers (pgsvt_denoise_batch runs sequences on several host
// threads) must not shrink the limit under another thread's launch.
void allow_dynamic_smem(const void* kernel, size_t shm) {
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, size_t> limit;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  size_t& cur = limit[{dev, kernel}];
  if (shm > cur && cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)shm) == cudaSuccess)
    cur = shm;
}

template <int BS, typename AccT>
void launch_k_eval_bs(dim3 grid, int threads, size_t shm, cudaStream_t s, const Problem& pb,
                      const DeviceBuffers& d, int final_pass, int stage) {
  if constexpr (BS > 0 && BS * BS <= 16) {
    if (stage && threads <= 32 * 16) {  // two blocks per SM
      allow_dynamic_smem((const void*)k_eval<BS, AccT, true, 16>, shm);
      k_eval<BS, AccT, true, 16><<<grid, threads, shm, s>>>(pb, d, final_pass);
      return;
    }
    if (stage) {  // the left vectors staged in shared memory
      allow_dynamic_smem((const void*)k_eval<BS, AccT, true>, shm);
      k_eval<BS, AccT, true><<<grid, threads, shm, s>>>(pb, d, final_pass);
      return;
    }
  }
  if (threads <= 32 * 16) {  // two blocks per SM
    allow_dynamic_smem((const void*)k_eval<BS, AccT, false, 16>, shm);
    k_eval<BS, AccT, false, 16><<<grid, threads, shm, s>>>(pb, d, final_pass);
    return;
  }
  allow_dynamic_smem((const void*)k_eval<BS, AccT>, shm);
  k_eval<BS, AccT><<<grid, threads, shm, s>>>(pb, d, final_pass);
}

template <typename AccT>
void launch_k_eval_t(int bs, dim3 grid, int threads, size_t shm, cudaStream_t s,
                     const Problem& pb, const DeviceBuffers& d, int final_pass, int stage) {
  switch (bs) {
    case 2: launch_k_eval_bs<2, AccT>(grid, threads, shm, s, pb, d, final_pass, stage); break;
    case 3: launch_k_eval_bs<3, AccT>(grid, threads, shm, s, pb, d, final_pass, stage); break;
    case 4: launch_k_eval_bs<4, AccT>(grid, threads, shm, s, pb, d, final_pass, stage); break;
    case 5: launch_k_eval_bs<5, AccT>(grid, threads, shm, s, pb, d, final_pass, stage); break;
    case 6: launch_k_eval_bs<6, AccT>(grid, threads, shm, s, pb, d, final_pass, stage); break;
    case 7: launch_k_eval_bs<7, AccT>(grid, threads, shm, s, pb, d, final_pass, stage); break;
    case 8: launch_k_eval_bs<8, AccT>(grid, threads, shm, s, pb, d, final_pass, stage); break;
    default: launch_k_eval_bs<0, AccT>(grid, threads, shm, s, pb, d, final_pass, stage); break;
  }
}

void launch_k_eval(const Problem& pb, const DeviceBuffers& d, int final_pass, int nl,
                   cudaStream_t s) {
  const Geometry& g = pb.g;
  int stage = 0;
  const size_t shm = eval_smem(g, nl, stage);
  const dim3 grid(d.nblk_eval, pb.W);
  if (pb.acc64)
    launch_k_eval_t<unsigned long long>(g.bs, grid, 32 * g.nwin, shm, s, pb, d, final_pass, stage);
  else launch_k_eval_t<int>(g.bs, grid, 32 * g.nwin, shm, s, pb, d, final_pass, stage);
}

void launch_k_mse(const Problem& pb, const DeviceBuffers& d, cudaStream_t s) {
  const dim3 grid(d.nblk_mse, pb.W);
  if (pb.K <= 8) {
    if (pb.acc64) k_mse<unsigned long long, 8><<<grid, 256, 0, s>>>(pb, d);
    else k_mse<int, 8><<<grid, 256, 0, s>>>(pb, d);
  } else {
    if (pb.acc64) k_mse<unsigned long long, kMaxK><<<grid, 256, 0, s>>>(pb, d);
    else k_mse<int, kMaxK><<<grid, 256, 0, s>>>(pb, d);
  }
}

}  // namespace

int eval_blocks(const Geometry& g) { return (g.NP + kEvalPatches - 1) / kEvalPatches; }
int mse_blocks(const Geometry& g) {
  return (int)std::max<size_t>(32, std::min<size_t>(1024, g.cube() / 4096));
}

cudaError_t launch_fields(const Problem& pb, const DeviceBuffers& d, cudaStream_t s) {
  const Geometry& g = pb.g;
  cudaMemsetAsync(d.cnt, 0, sizeof(int32_t) * g.cube() * pb.W, s);
  dim3 gc((g.NP + 127) / 128, g.nwin, pb.W);
  k_counts<<<gc, 128, 0, s>>>(pb, d);
  const int nb = 256;
  k_fields<<<dim3(nb, pb.W), 256, 0, s>>>(pb, d);
  k_sum_u<<<(pb.W + 63) / 64, 64, 0, s>>>(pb, d, nb);
  return cudaGetLastError();
}

cudaError_t launch_search_init(const Problem& pb, const DeviceBuffers& d, cudaStream_t s) {
  k_search_init<<<(pb.W + 63) / 64, 64, 0, s>>>(pb, d);
  return cudaGetLastError();
}

cudaError_t launch_search_hint(const Problem& pb, const DeviceBuffers& d, cudaStream_t s) {
  k_search_hint<<<(pb.W + 63) / 64, 64, 0, s>>>(pb, d);
  return cudaGetLastError();
}

cudaError_t launch_eval_round(const Problem& pb, const DeviceBuffers& d, int final_pass,
                              cudaStream_t s) {
  launch_k_eval(pb, d, final_pass, final_pass ? 1 : pb.K, s);
  if (final_pass) return cudaGetLastError();
  launch_k_mse(pb, d, s);
  k_search_step<<<pb.W, 256, 0, s>>>(pb, d);
  return cudaGetLastError();
}

cudaError_t launch_cube_out(const Problem& pb, const DeviceBuffers& d, double* v,
                            cudaStream_t s) {
  if (pb.acc64) k_cube_out<unsigned long long><<<512, 256, 0, s>>>(pb, d, v);
  else k_cube_out<int><<<512, 256, 0, s>>>(pb, d, v);
  return cudaGetLastError();
}

cudaError_t launch_risk_round(const Problem& pb, const DeviceBuffers& d, double* out,
                              cudaStream_t s) {
  launch_k_eval(pb, d, 0, pb.K, s);
  launch_k_mse(pb, d, s);
  k_risk_collect<<<1, kMaxK, 0, s>>>(pb, d, out);
  return cudaGetLastError();
}

cudaError_t launch_output(const Problem& pb, const DeviceBuffers& d, cudaStream_t s) {
  const Geometry& g = pb.g;
  dim3 go((unsigned)std::min<size_t>((g.F() + 255) / 256, 512), pb.W);
  if (pb.acc64) k_output<unsigned long long><<<go, 256, 0, s>>>(pb, d);
  else k_output<int><<<go, 256, 0, s>>>(pb, d);
  return cudaGetLastError();
}

}  // namespace pgsvt
