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
// into a fixed-point (2^-32) int64 accumulator, which makes the sums
// independent of the order of the atomics, so the whole search is
// deterministic.
#include <algorithm>

#include "pgsvt_internal.h"

namespace pgsvt {

namespace {

constexpr int kMseBlocks = 128;

__device__ __forceinline__ double warp_sum_d(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---- coverage counts (weights in svt.hpp:157-159)
__global__ void k_counts(Problem pb, DeviceBuffers d) {
  const Geometry& g = pb.g;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y, w = blockIdx.z;
  if (p >= g.NP) return;
  const uint32_t pc = d.pos[((size_t)w * g.nwin + k) * g.P + d.plist[p]];
  const int y = pc & 0xffffu, x = pc >> 16;
  int32_t* c = d.cnt + (size_t)w * g.cube() + (size_t)k * g.F();
  for (int cc = 0; cc < g.bs; ++cc)
    for (int r = 0; r < g.bs; ++r) atomicAdd(c + (y + r) + (size_t)(x + cc) * g.S, 1);
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
// points geometrically over [lo, hi]; each later round places K points evenly
// inside the bracket formed by the neighbours of the best point so far.  A
// hint (learned proposal) searches [hint/span, hint*span] first and falls back
// to the plain search when its best point lies on that grid's edge.

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
  }
  __device__ static int best(const SearchState& s) {
    int b = 0;
    for (int i = 1; i < s.npts; ++i)
      if (s.risk[i] < s.risk[b]) b = i;
    return b;
  }
};

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
  if (pb.hint > 0) {
    Sch::phase(s, 1, pb.K, pb.max_evals, max(1, pb.rounds / 2), 0);
    Sch::grid(s, pb.hint / pb.hint_span, fmin(wc.upper, pb.hint * pb.hint_span));
  } else {
    Sch::phase(s, 0, pb.K, pb.max_evals, pb.rounds, 1);
    Sch::grid(s, wc.upper * 1e-4, wc.upper);
  }
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

// Merge the risks of the pending round and schedule the next one.
__global__ void k_search_step(Problem pb, DeviceBuffers d) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= pb.W) return;
  SearchState& s = d.st[w];
  if (s.done) return;
  const Geometry& g = pb.g;
  const WinConst& wc = d.wc[w];
  const double N = (double)g.S * g.S * g.nwin;
  const double a = wc.alpha, m = wc.mu, s2 = wc.sigma * wc.sigma;
  const int nbe = d.nblk_eval, nbm = d.nblk_mse;
  const double prev_best = s.npts > 0 ? s.risk[s.best] : 0.0;
  for (int j = 0; j < s.nnext; ++j) {
    double lin = 0.0, mse = 0.0;
    const double* pl = d.part_lin + ((size_t)w * pb.K + j) * nbe;
    const double* pm = d.part_mse + ((size_t)w * pb.K + j) * nbm;
    for (int b = 0; b < nbe; ++b) lin += pl[b];
    for (int b = 0; b < nbm; ++b) mse += pm[b];
    // pgure.hpp:136
    const double r = (1.0 / N) * (mse + lin - (a + m) * wc.sum_u + m) - s2;
    int pos = s.npts;  // keep lambda ascending, new points after equal ones
    while (pos > 0 && s.lam[pos - 1] > s.next[j]) {
      s.lam[pos] = s.lam[pos - 1];
      s.risk[pos] = s.risk[pos - 1];
      --pos;
    }
    s.lam[pos] = s.next[j];
    s.risk[pos] = r;
    ++s.npts;
  }
  s.evals_phase += s.nnext;
  s.evals_total += s.nnext;
  s.nnext = 0;
  const int b = Sch::best(s);
  s.best = b;
  if (s.first) {
    s.first = 0;
    const bool edge = (b == 0 || b == s.npts - 1);
    if (s.phase == 1 && edge) {  // proposal not bracketed: plain search
      s.hint_lambda = s.lam[b];
      s.hint_risk = s.risk[b];
      const int left = pb.max_evals > s.evals_phase ? pb.max_evals - s.evals_phase : 1;
      Sch::phase(s, 2, pb.K, left, pb.rounds, 1);
      Sch::grid(s, wc.upper * 1e-4, wc.upper);
      return;
    }
  } else {
    ++s.rd;
    if (prev_best - s.risk[b] <= pb.tol * fabs(s.risk[b])) {
      search_finish(s, d.counters);
      return;
    }
  }
  if (s.rd >= s.rounds || s.evals_phase + s.K > s.max_eval) {
    search_finish(s, d.counters);
    return;
  }
  const double blo = (b > 0) ? s.lam[b - 1] : (s.zero_lo ? 0.0 : s.lam[b]);
  const double bhi = (b + 1 < s.npts) ? s.lam[b + 1] : s.lam[b];
  if (!(bhi > blo)) {
    search_finish(s, d.counters);
    return;
  }
  for (int i = 0; i < s.K; ++i)
    s.next[i] = blo + (bhi - blo) * (double)(i + 1) / (double)(s.K + 1);
  s.nnext = s.K;
}

// ---- one evaluation round: shrink, linear terms, rebuild + scatter of copy 0
//
// Block = 32 consecutive kept patches x nwin warps; warp k rebuilds column k
// (trajectory slice k) of its lanes' patches.
template <int BS>
__global__ void k_eval(Problem pb, DeviceBuffers d, int final_pass) {
  constexpr int M = BS * BS;
  const Geometry& g = pb.g;
  const int w = blockIdx.y;
  const SearchState& st = d.st[w];
  const int nl = final_pass ? 1 : st.nnext;
  if (!final_pass && (st.done || nl == 0)) return;
  const int lane = threadIdx.x & 31, k = threadIdx.x >> 5;
  const int p = blockIdx.x * 32 + lane;
  const bool live = p < g.NP;
  const int NC = g.NC;
  const size_t NP = g.NP;
  extern __shared__ float sg[];             // [nl][NC][32]
  __shared__ int srmax[kMaxK];
  const WinConst& wc = d.wc[w];
  const int ncp = d.ncopies;
  // phase A: warp j < nl computes g for lambda j
  for (int j = k; j < nl; j += blockDim.x >> 5) {
    const double lamd = final_pass ? st.final_lambda : st.next[j];
    const float lam = (float)lamd;
    float lin = 0.f;
    int r0 = 0;
    for (int c = 0; c < 4; ++c) {
      if (c >= ncp && !(c == 3 && ncp == 4)) continue;
      if (c > 0 && (final_pass || !pb.optimize)) break;
      const float* sv = d.sv + ((size_t)w * 4 + c) * NC * NP;
      const float* hv = d.hv + ((size_t)w * 4 + c) * NC * NP;
      const float smax = live ? sv[p] : 0.f;  // sorted: column 0 is the largest
      for (int i = 0; i < NC; ++i) {
        const float s = live ? sv[(size_t)i * NP + p] : 0.f;
        float th;
        if (pb.expw) th = fabsf(smax * expf(-0.5f * lam * (s * s)));  // svt.hpp:137
        else th = lam;                                                // svt.hpp:142
        const float gi = fmaxf(fabsf(s) - th, 0.f);
        if (c == 0) {
          sg[((size_t)j * NC + i) * 32 + lane] = gi;
          r0 += gi > 0.f;
        }
        if (pb.optimize && !final_pass && live) lin = fmaf(gi, hv[(size_t)i * NP + p], lin);
      }
    }
    if (!final_pass && pb.optimize) {
      const double t = warp_sum_d((double)lin);
      if (lane == 0) d.part_lin[((size_t)w * pb.K + j) * d.nblk_eval + blockIdx.x] = t;
    }
    for (int o = 16; o > 0; o >>= 1) r0 = max(r0, __shfl_xor_sync(0xffffffffu, r0, o));
    if (lane == 0) srmax[j] = r0;
  }
  __syncthreads();
  if (!live || k >= g.nwin) return;
  if (final_pass == 1 && k != wc.out_slice) return;  // 2: every slice
  const uint32_t pc = d.pos[((size_t)w * g.nwin + k) * g.P + d.plist[p]];
  const int y = pc & 0xffffu, x = pc >> 16;
  const float* U0 = d.U0 + (size_t)w * NC * M * NP;
  const float* V0 = d.V0 + (size_t)w * NC * g.nwin * NP;
  float col[M];
  for (int j = 0; j < nl; ++j) {
#pragma unroll
    for (int e = 0; e < M; ++e) col[e] = 0.f;
    const int rm = srmax[j];
    for (int i = 0; i < rm; ++i) {
      const float coef = sg[((size_t)j * NC + i) * 32 + lane] * V0[((size_t)i * g.nwin + k) * NP + p];
      if (coef == 0.f) continue;
      const float* ui = U0 + (size_t)i * M * NP + p;
#pragma unroll
      for (int e = 0; e < M; ++e) col[e] = fmaf(coef, __ldg(ui + (size_t)e * NP), col[e]);
    }
    unsigned long long* acc = d.acc + (((size_t)w * pb.K + j) * g.nwin + k) * g.F();
#pragma unroll
    for (int e = 0; e < M; ++e) {
      const long long q = __float2ll_rn(col[e] * 4294967296.0f);
      if (q != 0) atomicAdd(acc + (y + e % BS) + (size_t)(x + e / BS) * g.S, (unsigned long long)q);
    }
  }
}

// ---- sum over voxels of (Uh - U)^2 for each lambda of the round; clears acc
__global__ void k_mse(Problem pb, DeviceBuffers d) {
  const Geometry& g = pb.g;
  const int w = blockIdx.z, j = blockIdx.y;
  const SearchState& st = d.st[w];
  if (st.done || j >= st.nnext) return;
  const size_t C = g.cube();
  const float* u = d.u + (size_t)w * C;
  const int32_t* cnt = d.cnt + (size_t)w * C;
  unsigned long long* acc = d.acc + ((size_t)w * pb.K + j) * C;
  double tot = 0.0;
  for (size_t i0 = blockIdx.x * (size_t)blockDim.x * 4 + threadIdx.x; i0 < C;
       i0 += (size_t)gridDim.x * blockDim.x * 4) {
    float part = 0.f;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const size_t i = i0 + (size_t)q * blockDim.x;
      if (i >= C) break;
      const long long a = (long long)acc[i];
      acc[i] = 0ull;
      const int n = cnt[i];
      const float uh = n > 0 ? (float)((double)a * (1.0 / 4294967296.0)) / (float)n : 0.f;
      const float df = uh - u[i];
      part = fmaf(df, df, part);
    }
    tot += part;
  }
  tot = warp_sum_d(tot);
  __shared__ double sm[32];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = tot;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += sm[q];
    d.part_mse[((size_t)w * pb.K + j) * d.nblk_mse + blockIdx.x] = t;
  }
}

// ---- output slice and estimates (pguresvt.hpp:146-166)
__global__ void k_output(Problem pb, DeviceBuffers d) {
  const Geometry& g = pb.g;
  const int w = blockIdx.y;
  const WinConst& wc = d.wc[w];
  const size_t F = g.F();
  const size_t off = ((size_t)w * pb.K * g.nwin + wc.out_slice) * F;
  const int32_t* cnt = d.cnt + (size_t)w * g.cube() + (size_t)wc.out_slice * F;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < F;
       i += (size_t)gridDim.x * blockDim.x) {
    const long long a = (long long)d.acc[off + i];
    d.acc[off + i] = 0ull;
    const int n = cnt[i];
    double v = n > 0 ? ((double)a * (1.0 / 4294967296.0)) / n : 0.0;
    if (!isfinite(v)) v = 0.0;
    d.Y[(size_t)wc.t * F + i] = v * wc.umax;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const int n = g.nimg;
    d.est[wc.t] = d.st[w].final_lambda;
    d.est[wc.t + n] = pb.alpha_c;
    d.est[wc.t + 2 * (size_t)n] = pb.mu_c;
    d.est[wc.t + 3 * (size_t)n] = pb.sigma_c;
  }
}

// ---- whole reconstructed window v = acc / cnt (svt.hpp:163-164), window 0
__global__ void k_cube_out(Problem pb, DeviceBuffers d, double* v) {
  const Geometry& g = pb.g;
  const size_t C = g.cube();
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < C;
       i += (size_t)gridDim.x * blockDim.x) {
    const long long a = (long long)d.acc[i];
    d.acc[i] = 0ull;
    const int n = d.cnt[i];
    double q = n > 0 ? ((double)a * (1.0 / 4294967296.0)) / n : 0.0;
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

template <typename... A>
void launch_k_eval(int bs, dim3 grid, int threads, size_t shm, cudaStream_t s, A... a) {
  switch (bs) {
    case 2: k_eval<2><<<grid, threads, shm, s>>>(a...); break;
    case 3: k_eval<3><<<grid, threads, shm, s>>>(a...); break;
    case 4: k_eval<4><<<grid, threads, shm, s>>>(a...); break;
    case 5: k_eval<5><<<grid, threads, shm, s>>>(a...); break;
    case 6: k_eval<6><<<grid, threads, shm, s>>>(a...); break;
    case 7: k_eval<7><<<grid, threads, shm, s>>>(a...); break;
    default: k_eval<8><<<grid, threads, shm, s>>>(a...); break;
  }
}

}  // namespace

int eval_blocks(const Geometry& g) { return (g.NP + 31) / 32; }
int mse_blocks(const Geometry&) { return kMseBlocks; }

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

cudaError_t launch_eval_round(const Problem& pb, const DeviceBuffers& d, int final_pass,
                              cudaStream_t s) {
  const Geometry& g = pb.g;
  const int nl = final_pass ? 1 : pb.K;
  const size_t shm = (size_t)nl * g.NC * 32 * sizeof(float);
  dim3 ge(d.nblk_eval, pb.W);
  launch_k_eval(g.bs, ge, 32 * g.nwin, shm, s, pb, d, final_pass);
  if (final_pass) return cudaGetLastError();
  dim3 gm(d.nblk_mse, pb.K, pb.W);
  k_mse<<<gm, 256, 0, s>>>(pb, d);
  k_search_step<<<(pb.W + 63) / 64, 64, 0, s>>>(pb, d);
  return cudaGetLastError();
}

cudaError_t launch_cube_out(const Problem& pb, const DeviceBuffers& d, double* v,
                            cudaStream_t s) {
  k_cube_out<<<512, 256, 0, s>>>(pb, d, v);
  return cudaGetLastError();
}

cudaError_t launch_risk_round(const Problem& pb, const DeviceBuffers& d, double* out,
                              cudaStream_t s) {
  const Geometry& g = pb.g;
  const size_t shm = (size_t)pb.K * g.NC * 32 * sizeof(float);
  launch_k_eval(g.bs, dim3(d.nblk_eval, 1), 32 * g.nwin, shm, s, pb, d, 0);
  k_mse<<<dim3(d.nblk_mse, pb.K, 1), 256, 0, s>>>(pb, d);
  k_risk_collect<<<1, kMaxK, 0, s>>>(pb, d, out);
  return cudaGetLastError();
}

cudaError_t launch_output(const Problem& pb, const DeviceBuffers& d, cudaStream_t s) {
  const Geometry& g = pb.g;
  dim3 go((unsigned)std::min<size_t>((g.F() + 255) / 256, 512), pb.W);
  k_output<<<go, 256, 0, s>>>(pb, d);
  return cudaGetLastError();
}

}  // namespace pgsvt
