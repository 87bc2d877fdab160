// arps.cu — ARPS block matching on the GPU with motion vectors identical to
// the reference's FP64 MotionEstimator (arps.hpp:52-375).
//
// One thread runs one motion-slot chain (<= 2 frame pairs that share a slot of
// the reference's `motions` cube, arps.hpp:121-130) for one grid position.
// Block costs (mean squared difference, arps.hpp:148-151) are computed in FP32
// from the normalised window together with a rigorous bound on their distance
// to the FP64 value; whenever the FP32 argmin of a diamond step is not certain
// under those bounds, every candidate of that step is recomputed exactly as the
// reference does (FP64 x/umax, FP64 squares, Armadillo's two-accumulator
// accu(), no fused multiply-add) and the FP64 argmin is taken.  The decisions,
// hence the motion vectors, are therefore the FP64 ones.
#include "pgsvt_internal.h"

namespace pgsvt {

namespace {


struct ArpsCtx {
  bool integer;       // integer-valued input below 2^19: exact integer costs
  const float* fa1;   // normalised window slice a1
  const float* fa2;   // normalised window slice a2
  const float* xa1;   // input frames (exact f32 values) for the FP64 path
  const float* xa2;
  const double* xa1d; // input frames when the input is f64
  const double* xa2d;
  const double* pa1;  // FP64 normalised slices when precomputed (median
  const double* pa2;  // pre-filter: ties are frequent), else null
  double umax;
  int S;
  int mw;
  int bs;             // patch side (used when the kernel is not specialised)
};

// The reference block of one position.  BS > 0: its values in registers;
// BS == 0 (patch sides above 8): read from the frame where needed.
template <int BS>
struct Block {
  float ref[BS > 0 ? BS * BS : 1];  // normalised values, or the raw integers in integer mode
  const float* src = nullptr;       // BS == 0: the block's first element
  int S = 0;

  __device__ __forceinline__ float at(int e, int nb) const {
    if constexpr (BS > 0) return ref[e];
    else return __ldg(src + (e % nb) + (size_t)(e / nb) * S);
  }

  __device__ void load(const ArpsCtx& c, int i, int j) {
    const float* sp = c.integer ? c.xa1 : c.fa1;
    if constexpr (BS > 0) {
#pragma unroll
      for (int cc = 0; cc < BS; ++cc)
#pragma unroll
        for (int r = 0; r < BS; ++r) ref[r + cc * BS] = __ldg(sp + (i + r) + (size_t)(j + cc) * c.S);
    } else {
      src = sp + i + (size_t)j * c.S;
      S = c.S;
    }
  }

  // Integer mode: the exact sum of squared differences D.  The reference's
  // FP64 cost is D / (umax^2 m) up to an absolute error below
  // (m + 7) 2^-53 (values <= 1 after normalisation), while two different D
  // differ by at least 1 / (umax^2 m) > 2 (m + 7) 2^-53 for umax <= 2^19 and
  // m <= 64, or umax <= 2^17 and m <= 256 (the host enables the mode only
  // then): comparing D decides exactly as the reference does, except for
  // equal D.
  __device__ unsigned long long ssd(const ArpsCtx& c, int y, int x) const {
    const int nb = BS > 0 ? BS : c.bs;
    unsigned long long acc = 0ull;
#pragma unroll
    for (int cc = 0; cc < nb; ++cc)
#pragma unroll
      for (int r = 0; r < nb; ++r) {
        const int a = (int)at(r + cc * nb, nb);
        const int b = (int)__ldg(c.xa2 + (y + r) + (size_t)(x + cc) * c.S);
        const unsigned d = (unsigned)abs(a - b);  // < 2^19
        acc += (unsigned long long)d * d;
      }
    return acc;
  }

  // the candidate block at (y, x) equals the one at (y2, x2), element by element
  __device__ bool same(const ArpsCtx& c, int y, int x, int y2, int x2) const {
    const int nb = BS > 0 ? BS : c.bs;
    bool eq = true;
#pragma unroll
    for (int cc = 0; cc < nb; ++cc)
#pragma unroll
      for (int r = 0; r < nb; ++r)
        eq &= __ldg(c.xa2 + (y + r) + (size_t)(x + cc) * c.S) ==
              __ldg(c.xa2 + (y2 + r) + (size_t)(x2 + cc) * c.S);
    return eq;
  }

  // cost of the candidate at (y, x): FP32 with an error bound, or exact D
  __device__ void cost(const ArpsCtx& c, int y, int x, float& cf, float& err,
                       unsigned long long& cd) const {
    if (c.integer) {
      cd = ssd(c, y, x);
      cf = 0.f;
      err = 0.f;
    } else {
      cost32(c, y, x, cf, err);
      cd = 0ull;
    }
  }

  // FP32 cost and a bound on |cost32 - cost64| (u = 2^-24, m = bs^2): the
  // FP32 operands differ from the reference's FP64 ones by <= 2u|a| (the
  // normalisation divides by the FP32-rounded maximum), so every difference
  // by <= 3u(|a|+|b|) and every square by <= 6u(|a|+|b|)^2; the m-term FMA
  // sum adds <= m u sum d^2 = m^2 u cost.  With margin:
  //   err = u * (8 * sum_e (|a_e|+|b_e|)^2 / m + (m + 4) * cost)
  __device__ void cost32(const ArpsCtx& c, int y, int x, float& cost, float& err) const {
    const int nb = BS > 0 ? BS : c.bs;
    float acc = 0.f, sb = 0.f;
#pragma unroll
    for (int cc = 0; cc < nb; ++cc)
#pragma unroll
      for (int r = 0; r < nb; ++r) {
        const float a = at(r + cc * nb, nb);
        const float b = __ldg(c.fa2 + (y + r) + (size_t)(x + cc) * c.S);
        const float d = a - b;
        acc = fmaf(d, d, acc);
        const float s = fabsf(a) + fabsf(b);
        sb = fmaf(s, s, sb);
      }
    const float m = (float)(nb * nb);
    const float oo = 1.0f / m;
    cost = acc * oo;
    err = 5.9604645e-8f * (8.f * sb * oo + (m + 4.f) * cost);
  }
};

__device__ __forceinline__ double src64(const ArpsCtx& c, const float* xf, const double* xd,
                                        size_t idx) {
  return xd ? xd[idx] : (double)xf[idx];
}

// Per-warp scratch of the exact (FP64) decisions.
template <int BS>
struct ArpsWarp {
  static constexpr int kSq = 256;  // squared differences per pass
  double sq[kSq];
  double cst[32 * 6];     // exact cost per (lane, slot)
  uint32_t pos[32 * 6];   // candidate (y, x) per (lane, slot), 16 bits each
  uint32_t blk[32];       // reference block (i, j) per lane, 16 bits each
  uint16_t cand[32 * 6];  // the warp's candidates to evaluate: lane * 6 + slot
};

// Exact reference costs (arps.hpp:148-151 as the reference evaluates them:
// FP64 x/umax, FP64 squares, Armadillo's two-accumulator accu(), no fused
// multiply-add) of every slot in `em` of every lane, computed by the whole
// warp at once: the squared differences of all candidate blocks are spread
// over the lanes, and the even- and odd-element accumulators of every
// candidate are summed in element order by two lanes.  The FP64 pipe runs a
// warp instruction at a fraction of the FP32 rate whatever its active lanes,
// so this takes a small part of the FP64 instructions (and of the latency) of
// per-thread evaluations.  Results in ws.cst[lane * 6 + slot].
template <int BS>
__device__ void warp_cost64(const ArpsCtx& c, ArpsWarp<BS>& ws, unsigned em, int i, int j,
                            int y, int x, const int (*off)[2], int nslot) {
  const int lane = threadIdx.x & 31;
  const int nb = BS > 0 ? BS : c.bs;
  const int m = nb * nb;
  const double oo = 1.0 / (double)m;
  // this lane's candidates, and their place in the warp's list
  const int mine = __popc(em);
  int first = mine;
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, first, o);
    if (lane >= o) first += t;
  }
  const int total = __shfl_sync(0xffffffffu, first, 31);
  first -= mine;
  if (em) {
    ws.blk[lane] = ((uint32_t)i & 0xffffu) | ((uint32_t)j << 16);
    int r = first;
    for (int k = 0; k < nslot; ++k) {
      if (!((em >> k) & 1u)) continue;
      ws.pos[lane * 6 + k] = ((uint32_t)(y + off[k][1]) & 0xffffu) | ((uint32_t)(x + off[k][0]) << 16);
      ws.cand[r++] = (uint16_t)(lane * 6 + k);
    }
  }
  __syncwarp();
  const int per = min(16, ArpsWarp<BS>::kSq / m);  // two summing lanes per candidate
  for (int c0 = 0; c0 < total; c0 += per) {
    const int cn = min(per, total - c0);
    for (int t = lane; t < cn * m; t += 32) {
      const int cd = ws.cand[c0 + t / m];
      const int e = t % m, r = e % nb, cc = e / nb;
      const uint32_t pb = ws.blk[cd / 6], pk = ws.pos[cd];
      const int bi = (int)(pb & 0xffffu), bj = (int)(pb >> 16);
      const int py = (int)(pk & 0xffffu), px = (int)(pk >> 16);
      const size_t ka = (bi + r) + (size_t)(bj + cc) * c.S;
      const size_t kb = (py + r) + (size_t)(px + cc) * c.S;
      const double a = c.pa1 ? c.pa1[ka] : __ddiv_rn(src64(c, c.xa1, c.xa1d, ka), c.umax);
      const double b = c.pa2 ? c.pa2[kb] : __ddiv_rn(src64(c, c.xa2, c.xa2d, kb), c.umax);
      const double d = __dsub_rn(a, b);
      ws.sq[t] = __dmul_rn(d, d);
    }
    __syncwarp();
    double v = 0.0;
    if (lane < 2 * cn) {
      const double* q = ws.sq + (lane >> 1) * m;
      for (int e = lane & 1; e < m; e += 2) v = __dadd_rn(v, q[e]);
    }
    const double v2 = __shfl_down_sync(0xffffffffu, v, 1);
    if (lane < 2 * cn && !(lane & 1))
      ws.cst[ws.cand[c0 + (lane >> 1)]] = __dmul_rn(__dadd_rn(v, v2), oo);
    __syncwarp();
  }
}

// The slot chosen from the exact costs of the slots em: integer mode, the
// first of the least cost among the tied slots; otherwise the first index of
// the minimum over every evaluated slot (unevaluated ones count as 1e9).
__device__ int resolve_exact(bool integer, const double* cst, unsigned em, int nslot) {
  if (integer) {
    int kb = -1;
    double mm = 0.0;
    for (int k = 0; k < nslot; ++k) {
      if (!((em >> k) & 1u)) continue;
      if (kb < 0 || cst[k] < mm) {
        mm = cst[k];
        kb = k;
      }
    }
    return kb;
  }
  double c64[6];
  for (int k = 0; k < nslot; ++k) c64[k] = ((em >> k) & 1u) ? cst[k] : 1e9;
  double mm = c64[0];
  for (int k = 1; k < nslot; ++k) mm = fmin(mm, c64[k]);
  for (int k = 0; k < nslot; ++k)
    if (c64[k] == mm) return k;
  return 2;
}

// Integer mode: first index of the least D; equal D decided as the
// reference does: identical candidate blocks have identical FP64 costs (the
// first one wins), otherwise the FP64 costs of the tied candidates decide
// (returns -1 with those slots in em).
template <int BS>
__device__ int decide_int(const ArpsCtx& c, const Block<BS>& blk, const unsigned long long* cd,
                          const bool* ev, const int (*off)[2], int nslot, int y, int x,
                          unsigned& em) {
  int ks = 2;
  unsigned long long best = cd[2];
  for (int k = 0; k < nslot; ++k)
    if (ev[k] && (cd[k] < best || (cd[k] == best && k < ks))) {
      best = cd[k];
      ks = k;
    }
  unsigned tied = 1u << ks;
  bool distinct = false;
  for (int k = 0; k < nslot; ++k) {
    if (!ev[k] || k == ks || cd[k] != best) continue;
    tied |= 1u << k;
    if (!blk.same(c, y + off[k][1], x + off[k][0], y + off[ks][1], x + off[ks][0])) distinct = true;
  }
  if (!distinct) return ks;
  em = tied;
  return -1;
}

// First index of the minimum among evaluated slots when the FP32 decision is
// certain under the error bounds; else -1 with every evaluated slot in em.
__device__ int decide_f32(const float* cs, const float* es, const bool* ev, int nslot,
                          unsigned& em) {
  int ks = 2;
  float best = cs[2];
  for (int k = 0; k < nslot; ++k)
    if (ev[k] && (cs[k] < best || (cs[k] == best && k < ks))) {
      best = cs[k];
      ks = k;
    }
  bool certain = true;
  const float hi = cs[ks] + es[ks];
  for (int k = 0; k < nslot; ++k) {
    if (!ev[k] || k == ks) continue;
    const float lo = cs[k] - es[k];
    if (k < ks ? !(lo > hi) : !(lo >= hi)) certain = false;
  }
  if (certain) return ks;
  em = 0u;
  for (int k = 0; k < nslot; ++k)
    if (ev[k]) em |= 1u << k;
  return -1;
}

// ARPSMotionEstimation (arps.hpp:153-375) for one position of one frame pair.
// (my, mx) holds the predictor slot on entry and the new motion on exit.
// The lanes of a warp step through the diamond searches together (a lane
// whose search ended, or that holds no position, idles), so that the exact
// decisions any of them needs are taken by the whole warp.
template <int BS>
__device__ void arps_pair(const ArpsCtx& c, bool live, int it, int& my, int& mx, int& oy,
                          int& ox, ArpsWarp<BS>& ws, unsigned& nexact) {
  const int lane = threadIdx.x & 31;
  const int S = c.S, M = c.mw, Wd = 2 * M + 1;
  const int nb = BS > 0 ? BS : c.bs;
  const int n1 = S - nb + 1;
  const int i = it % n1, j = it / n1;
  Block<BS> blk;
  blk.load(c, i, j);
  uint32_t seen[(2 * kMaxMW + 1) * (2 * kMaxMW + 1) / 32 + 1];
  const int nw = (Wd * Wd + 31) / 32;
  for (int q = 0; q < nw; ++q) seen[q] = 0u;
  auto mark = [&](int dy, int dx) {
    if (dy < -M || dy > M || dx < -M || dx > M) return;  // cannot occur for mw >= 2
    const int b = (dy + M) * Wd + (dx + M);
    seen[b >> 5] |= 1u << (b & 31);
  };
  auto is_seen = [&](int dy, int dx) {
    const int b = (dy + M) * Wd + (dx + M);
    return (seen[b >> 5] >> (b & 31)) & 1u;
  };
  int x = j, y = i;
  float cs[6], es[6];
  unsigned long long cd[6];
  bool ev[6];
  float curC, curE;
  unsigned long long curD;
  blk.cost(c, i, j, curC, curE, curD);
  mark(0, 0);
  int step, nld;
  int LD[6][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}};
  if (j == 0) {
    step = 2;
    nld = 5;
  } else {
    const int ay = abs(my), ax = abs(mx);
    step = (ax <= ay) ? ay : ax;
    if ((ay == 0 && ax == step) || (ax == 0 && ay == step)) {
      nld = 5;
    } else {
      nld = 6;
      LD[5][0] = mx;
      LD[5][1] = my;
    }
  }
  LD[0][1] = -step;
  LD[1][0] = -step;
  LD[3][0] = step;
  LD[4][1] = step;
  // LDSP candidates (arps.hpp:247-287)
  for (int k = 0; k < 6; ++k) ev[k] = false;
  ev[2] = true;
  cs[2] = curC;
  es[2] = curE;
  cd[2] = curD;
  if (live)
    for (int k = 0; k < nld; ++k) {
      if (k == 2 || step == 0) continue;
      const int vy = y + LD[k][1], hx = x + LD[k][0];
      if (hx < 0 || vy < 0 || hx + nb - 1 >= S || vy + nb - 1 >= S) continue;
      blk.cost(c, vy, hx, cs[k], es[k], cd[k]);
      ev[k] = true;
      mark(LD[k][1], LD[k][0]);
    }
  // step 0 decides the LDSP (arps.hpp:289-294), steps 1.. the SDSP
  // (arps.hpp:299-368); every SDSP move enters an unvisited cell, so a search
  // ends within Wd*Wd moves.
  const int SD[5][2] = {{0, -1}, {-1, 0}, {0, 0}, {1, 0}, {0, 1}};
  bool done = !live;
  for (int n = 0; n <= Wd * Wd + 1; ++n) {
    const int (*off)[2] = (n == 0) ? LD : SD;
    const int nslot = (n == 0) ? 6 : 5;
    if (n > 0 && !done) {
      for (int k = 0; k < 6; ++k) ev[k] = false;
      ev[2] = true;
      cs[2] = curC;
      es[2] = curE;
      cd[2] = curD;
      for (int k = 0; k < 5; ++k) {
        if (k == 2) continue;
        const int vy = y + SD[k][1], hx = x + SD[k][0];
        if (hx < 0 || vy < 0 || hx + nb - 1 >= S || vy + nb - 1 >= S) continue;
        if (hx < j - M || hx > j + M || vy < i - M || vy > i + M) continue;
        if (is_seen(vy - i, hx - j)) continue;
        blk.cost(c, vy, hx, cs[k], es[k], cd[k]);
        ev[k] = true;
        mark(vy - i, hx - j);
      }
    }
    int ks = 2;
    unsigned em = 0u;
    if (!done)
      ks = c.integer ? decide_int<BS>(c, blk, cd, ev, off, nslot, y, x, em)
                     : decide_f32(cs, es, ev, nslot, em);
    if (__any_sync(0xffffffffu, em != 0u)) {
      warp_cost64<BS>(c, ws, em, i, j, y, x, off, nslot);
      if (em) {
        ks = resolve_exact(c.integer, ws.cst + lane * 6, em, nslot);
        ++nexact;
      }
      __syncwarp();
    }
    if (!done) {
      x += off[ks][0];
      y += off[ks][1];
      curC = cs[ks];
      curE = es[ks];
      curD = cd[ks];
      if (n > 0 && ks == 2) done = true;
    }
    if (!__any_sync(0xffffffffu, !done)) break;
  }
  my = y - i;
  mx = x - j;
  oy = y;
  ox = x;
}

// five blocks per SM: 96 registers, no spills (128 at the default bound)
template <int BS>
__global__ void __launch_bounds__(128, 5) k_arps(Problem pb, DeviceBuffers d) {
  const Geometry& g = pb.g;
  const int it0 = blockIdx.x * blockDim.x + threadIdx.x;
  const int ch = blockIdx.y, w = blockIdx.z;
  const ArpsChain cn = d.chains[w * d.nchains + ch];
  if (cn.npairs == 0) return;  // uniform over the block
  const bool live = it0 < g.P;
  const int it = live ? it0 : 0;
  __shared__ ArpsWarp<BS> wsh[4];
  ArpsWarp<BS>& ws = wsh[threadIdx.x >> 5];
  const WinConst& wc = d.wc[w];
  const size_t F = g.F();
  // ARPS input: the median-filtered window when the pre-filter is on
  // (its values are integers, exact in FP32), else the window itself
  const bool med = d.zs != nullptr;
  const float* fw = med ? d.wz : d.u;
  const float* xw = med ? d.zs : d.xs;
  const double* xd = med ? nullptr : d.x64;
  ArpsCtx c;
  c.bs = g.bs;
  c.integer = med || d.int_input;
  c.umax = med ? wc.wnorm : wc.unorm;
  c.S = g.S;
  c.mw = g.mw;
  int my = 0, mx = 0;
  unsigned nexact = 0u;
  for (int q = 0; q < cn.npairs; ++q) {
    const int a1 = cn.a1[q], a2 = cn.a2[q];
    c.fa1 = fw + ((size_t)w * g.nwin + a1) * F;
    c.fa2 = fw + ((size_t)w * g.nwin + a2) * F;
    c.xa1 = xw + (size_t)(wc.s0 + a1) * F;
    c.xa2 = xw + (size_t)(wc.s0 + a2) * F;
    c.xa1d = xd ? xd + (size_t)(wc.s0 + a1) * F : nullptr;
    c.xa2d = xd ? xd + (size_t)(wc.s0 + a2) * F : nullptr;
    c.pa1 = d.w64 ? d.w64 + ((size_t)w * g.nwin + a1) * F : nullptr;
    c.pa2 = d.w64 ? d.w64 + ((size_t)w * g.nwin + a2) * F : nullptr;
    int oy, ox;
    arps_pair<BS>(c, live, it, my, mx, oy, ox, ws, nexact);
    if (live) d.pos[((size_t)w * g.nwin + a2) * g.P + it] = (uint32_t)oy | ((uint32_t)ox << 16);
  }
  for (int o = 16; o > 0; o >>= 1) nexact += __shfl_xor_sync(0xffffffffu, nexact, o);
  if ((threadIdx.x & 31) == 0 && nexact) atomicAdd(d.counters, (unsigned long long)nexact);
}

// Reference slice (always) and, without motion estimation, the other slices:
// (0,0) in compat mode (arps.hpp:42), else the grid position.
__global__ void k_grid(Problem pb, DeviceBuffers d) {
  const Geometry& g = pb.g;
  const int it = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y, w = blockIdx.z;
  if (it >= g.P) return;
  const int ref = d.wc[w].ref;
  const int n1 = g.S - g.bs + 1;
  const uint32_t grid = (uint32_t)(it % n1) | ((uint32_t)(it / n1) << 16);
  uint32_t v;
  if (k == ref) v = grid;
  else if (pb.motion) return;  // written by k_arps
  else v = (pb.compat & 0x2) ? 0u : grid;
  d.pos[((size_t)w * g.nwin + k) * g.P + it] = v;
}

}  // namespace

cudaError_t launch_arps(const Problem& pb, const DeviceBuffers& d, cudaStream_t s) {
  const Geometry& g = pb.g;
  const int threads = 128;
  dim3 gg((g.P + threads - 1) / threads, g.nwin, pb.W);
  k_grid<<<gg, threads, 0, s>>>(pb, d);
  if (!pb.motion || d.nchains == 0) return cudaGetLastError();
  dim3 ga((g.P + threads - 1) / threads, d.nchains, pb.W);
  switch (g.bs) {
    case 2: k_arps<2><<<ga, threads, 0, s>>>(pb, d); break;
    case 3: k_arps<3><<<ga, threads, 0, s>>>(pb, d); break;
    case 4: k_arps<4><<<ga, threads, 0, s>>>(pb, d); break;
    case 5: k_arps<5><<<ga, threads, 0, s>>>(pb, d); break;
    case 6: k_arps<6><<<ga, threads, 0, s>>>(pb, d); break;
    case 7: k_arps<7><<<ga, threads, 0, s>>>(pb, d); break;
    case 8: k_arps<8><<<ga, threads, 0, s>>>(pb, d); break;
    default: k_arps<0><<<ga, threads, 0, s>>>(pb, d); break;  // sides 9..16
  }
  return cudaGetLastError();
}

}  // namespace pgsvt
