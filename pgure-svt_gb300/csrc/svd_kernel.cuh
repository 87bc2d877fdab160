// svd_kernel.cuh — the batched one-sided Jacobi kernel template (see svd.cu).
#ifndef PGSVT_SVD_KERNEL_CUH
#define PGSVT_SVD_KERNEL_CUH

#include "pgsvt_internal.h"

namespace pgsvt {
namespace svdk {

constexpr int kMaxSweeps = 16;
constexpr float kTol = 1e-6f;     // rotate while |a_i.a_j| > kTol |a_i| |a_j|
constexpr float kBand = 4.f;      // near-degenerate pairs below kBand*kTol: FP64 decides
constexpr float kDegen = 1e-3f;   // |a_i|^2 and |a_j|^2 within 0.1%: near-degenerate
constexpr float kStopRel = 1e-3f; // owner form: a sweep whose rotations were all below
                                  // this relative inner product is the last

// Round-robin ordering with a fixed pairing pattern in register space: the
// pad column (always zero, nwin < NC) sits at position NC-1 and meets
// position 0 (a skipped, trivial pair); positions k and NC-1-k (k >= 1) are
// paired; after each round positions 0..NC-2 shift by one.  NC-1 rounds pair
// every two columns once and bring every column back to its position.

// A lane's RPL rows of the NC columns in registers.  With an even RPL the rows
// are packed in pairs (float2) so that a rotation updates two rows per
// packed FP32x2 instruction; the results are those of the scalar FMAs.
template <int RPL, int NC, bool PACK = (RPL % 2 == 0)>
struct RegCols {
  float2 v[RPL / 2][NC];
  __device__ __forceinline__ float& operator()(int r, int k) {
    return (r & 1) ? v[r >> 1][k].y : v[r >> 1][k].x;
  }
  // columns i, j <- (c a_i - s a_j, s a_i + c a_j)
  __device__ __forceinline__ void rotate(int i, int j, float cs, float sn) {
    const float2 c2 = make_float2(cs, cs), s2 = make_float2(sn, sn), n2 = make_float2(-sn, -sn);
#pragma unroll
    for (int r = 0; r < RPL / 2; ++r) {
      const float2 a = v[r][i], b = v[r][j];
      v[r][i] = __ffma2_rn(c2, a, __fmul2_rn(n2, b));
      v[r][j] = __ffma2_rn(s2, a, __fmul2_rn(c2, b));
    }
  }
  // positions 0..NC-2 move down by one, position 0 to NC-2
  __device__ __forceinline__ void shift() {
#pragma unroll
    for (int r = 0; r < RPL / 2; ++r) {
      const float2 t = v[r][0];
#pragma unroll
      for (int k = 0; k < NC - 2; ++k) v[r][k] = v[r][k + 1];
      v[r][NC - 2] = t;
    }
  }
};
template <int RPL, int NC>
struct RegCols<RPL, NC, false> {
  float v[RPL][NC];
  __device__ __forceinline__ float& operator()(int r, int k) { return v[r][k]; }
  __device__ __forceinline__ void rotate(int i, int j, float cs, float sn) {
#pragma unroll
    for (int r = 0; r < RPL; ++r) {
      const float a = v[r][i], b = v[r][j];
      v[r][i] = fmaf(cs, a, -sn * b);
      v[r][j] = fmaf(sn, a, cs * b);
    }
  }
  __device__ __forceinline__ void shift() {
#pragma unroll
    for (int r = 0; r < RPL; ++r) {
      const float t = v[r][0];
#pragma unroll
      for (int k = 0; k < NC - 2; ++k) v[r][k] = v[r][k + 1];
      v[r][NC - 2] = t;
    }
  }
};

template <int NC>
__device__ __forceinline__ void shift_norms(float (&nrm)[NC]) {
  const float t = nrm[0];
#pragma unroll
  for (int k = 0; k < NC - 2; ++k) nrm[k] = nrm[k + 1];
  nrm[NC - 2] = t;
}

template <int LANES>
__device__ __forceinline__ float lanes_sum(float v) {
#pragma unroll
  for (int o = 1; o < LANES; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int LANES>
__device__ __forceinline__ double lanes_sum_d(double v) {
#pragma unroll
  for (int o = 1; o < LANES; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Can singular value s (largest smax) survive the threshold for some lambda
// of the search (svt.hpp:135-143)?  Conservative: columns reported dead have
// g = 0 for every lambda the search evaluates, with margin for FP32 rounding.
__device__ __forceinline__ bool can_survive(const Problem& pb, float s, float smax,
                                            float upper) {
  if (!(s > 0.f)) return false;
  if (!pb.optimize) {
    const float lam = (float)pb.lambda_user;
    const float th = pb.expw ? fabsf(smax * expf(-0.5f * lam * (s * s))) : lam;
    return s * 1.0001f > th;
  }
  if (!pb.expw) return true;  // lambda may approach 0
  return 2.f * logf(smax / s) < 1.05f * upper * (s * s) + 1e-6f;
}

// Rotation of one pair from the half-angle identities: with d = be - al,
// r = sqrt(d^2 + 4g^2), cos 2th = |d| / r and sin 2th = 2 g sign(d) / r (the
// smaller of the two orthogonalising angles, sign(0) = +1): cos th =
// sqrt((1 + cos 2th) / 2), sin th = sin 2th / (2 cos th).  Flags whether the
// pair was near-degenerate within the FP64 band.
__device__ __forceinline__ void rotation(float al, float be, float gv, float g2, float ab,
                                         float& cs, float& sn, bool& definite, bool& band) {
  const bool degen = fabsf(be - al) <= kDegen * (al + be);
  if (degen && g2 <= (kBand * kBand * kTol * kTol) * ab) band = true;
  else definite = true;
  const float dd = be - al;
  const float ir = rsqrtf(fmaf(dd, dd, 4.f * g2));
  const float hh = fmaf(0.5f * fabsf(dd), ir, 0.5f);  // (1 + cos 2th) / 2
  const float rh = rsqrtf(hh);
  cs = hh * rh;
  sn = (dd >= 0.f ? gv : -gv) * ir * rh;
}

// |c a - s b|^2 and |s a + c b|^2 from al = |a|^2, be = |b|^2, g = a.b
__device__ __forceinline__ void rotated_norms(float al, float be, float gv, float cs, float sn,
                                              float& ni, float& nj) {
  const float c2 = cs * cs, s2 = sn * sn, csg = 2.f * cs * sn * gv;
  ni = fmaf(c2, al, fmaf(s2, be, -csg));
  nj = fmaf(s2, al, fmaf(c2, be, csg));
}

// RPL consecutive floats of one lane (16-byte vectors when RPL % 4 == 0)
template <int RPL>
__device__ __forceinline__ void load_rows(const float* p, float (&v)[RPL]) {
  if constexpr (RPL % 4 == 0) {
#pragma unroll
    for (int r = 0; r < RPL; r += 4) {
      const float4 t = *reinterpret_cast<const float4*>(p + r);
      v[r] = t.x;
      v[r + 1] = t.y;
      v[r + 2] = t.z;
      v[r + 3] = t.w;
    }
  } else {
#pragma unroll
    for (int r = 0; r < RPL; ++r) v[r] = p[r];
  }
}
template <int RPL>
__device__ __forceinline__ void store_rows(float* p, const float (&v)[RPL]) {
  if constexpr (RPL % 4 == 0) {
#pragma unroll
    for (int r = 0; r < RPL; r += 4)
      *reinterpret_cast<float4*>(p + r) = make_float4(v[r], v[r + 1], v[r + 2], v[r + 3]);
  } else {
#pragma unroll
    for (int r = 0; r < RPL; ++r) p[r] = v[r];
  }
}

// Rounds unrolled per loop iteration (code size vs register moves of the
// round shift) and the residency target of the launch bounds.
#ifndef PGSVT_SVD_UNROLL
#define PGSVT_SVD_UNROLL 1
#endif
#ifndef PGSVT_SVD_MINBLOCKS
#define PGSVT_SVD_MINBLOCKS 3
#endif
#ifndef PGSVT_SVD_MINBLOCKS_SM
#define PGSVT_SVD_MINBLOCKS_SM 4
#endif

// Shared-memory footprint of one patch: SM keeps the columns there during the
// sweeps ([NC][MP] plus NC norms, the patch stride an odd multiple of 16
// floats so the two 4-lane patches of a quarter-warp use disjoint banks);
// otherwise the epilogue's staging copy ([NC][MP+1]).
template <int RPL, int LANES, int NC, bool SM>
struct SvdSmem {
  static constexpr int MP = RPL * LANES;
  static constexpr int CS = SM ? MP : MP + 1;  // column stride
  static constexpr int NRM = ((NC + 15) / 16) * 16;
  static constexpr int BASE = NC * MP + NRM;
  static constexpr int STRIDE = SM ? ((LANES == 4 && BASE % 32 == 0) ? BASE + 16 : BASE)
                                   : NC * (MP + 1) + 4;
};

// residency target: the shared-memory form holds a round's column pairs in
// registers, (NC/2) * 2 * RPL floats; the register form holds RPL * NC
// floats twice over (sweeps, then the epilogue's fresh gather)
template <int RPL, int NC, bool SM>
constexpr int svd_minblocks() {
  return SM ? ((NC / 2) * 2 * RPL <= 64 ? PGSVT_SVD_MINBLOCKS_SM
                                        : ((NC / 2) * 2 * RPL <= 128 ? 2 : 1))
            : (RPL * NC >= 128 ? 2 : PGSVT_SVD_MINBLOCKS);
}

// Only near-degenerate pairs moved, by amounts at the FP32 noise level of
// their inner products: decide convergence from FP64 inner products of the
// current columns (exact products of the FP32 entries) staged in As
// ([NC][CS], this lane's RPL rows at q * RPL).  fp64_tests counts these
// decisions (one per patch and check).
template <int RPL, int LANES, int CS>
__device__ bool fp64_check(const float* As, int q, int nwin, unsigned& fp64_tests) {
  ++fp64_tests;
  bool again = false;
  for (int i = 0; i < nwin; ++i) {
    for (int j = i + 1; j < nwin; ++j) {
      float gi = 0.f, ai = 0.f, aj = 0.f;
#pragma unroll
      for (int r = 0; r < RPL; ++r) {
        const float x = As[i * CS + q * RPL + r], y = As[j * CS + q * RPL + r];
        gi = fmaf(x, y, gi);
        ai = fmaf(x, x, ai);
        aj = fmaf(y, y, aj);
      }
      gi = lanes_sum<LANES>(gi);
      ai = lanes_sum<LANES>(ai);
      aj = lanes_sum<LANES>(aj);
      const float sc = sqrtf(ai * aj);
      const bool cand = fabsf(gi) > 0.5f * kTol * sc && fabsf(aj - ai) <= kDegen * (ai + aj);
      if (__any_sync(0xffffffffu, cand)) {
        double g64 = 0.0;
#pragma unroll
        for (int r = 0; r < RPL; ++r)
          g64 = fma((double)As[i * CS + q * RPL + r], (double)As[j * CS + q * RPL + r], g64);
        g64 = lanes_sum_d<LANES>(g64);
        if (cand && fabs(g64) > (double)kTol * (double)sc) again = true;
      }
    }
  }
  __syncwarp();
  return __any_sync(0xffffffffu, again);
}

// Patches of 4 lanes x 4 rows and at most 16 columns take the owner form of
// the sweeps (below), unrolled three rounds per loop iteration where the
// round count allows (PGSVT_SVD_OWNER_UNROLL).
template <int RPL, int LANES, int NC>
constexpr bool kOwnerForm =
#ifdef PGSVT_SVD_REPLICATED
    false;
#else
    RPL == 4 && LANES == 4 && NC <= 16;
#endif
#ifndef PGSVT_SVD_OWNER_UNROLL
#define PGSVT_SVD_OWNER_UNROLL 3
#endif
template <int NC>
constexpr int kOwnerUnroll = ((NC - 1) % PGSVT_SVD_OWNER_UNROLL == 0) ? PGSVT_SVD_OWNER_UNROLL : 1;

// Lane q's copy of one of four per-lane candidates (q = 0..3), from registers
// with compile-time indices.
__device__ __forceinline__ float sel4(int q, float a, float b, float c, float d) {
  return (q & 2) ? ((q & 1) ? d : c) : ((q & 1) ? b : a);
}

// Jacobi sweeps for patches held by 4 lanes x 4 rows, with each pair's
// rotation computed once per patch instead of in all four lanes.  The lanes
// reduce-scatter the round's inner products (two exchange steps) so that lane
// q holds the complete inner products of pairs q and q + 4 (pair 0 is the
// zero pad column's); it computes those pairs' rotations and rotated norms
// and broadcasts them, and every lane applies every rotation to its rows.
// The pairs, the rotation formulas and the convergence rules are those of
// register_sweeps; pairs no patch of the warp needs to rotate are skipped
// warp-uniformly (a patch that does not need a rotated pair applies the
// identity, which leaves its columns and norms unchanged).
template <int NC, int CS, int U>
__device__ int owner_sweeps(RegCols<4, NC>& A, float* As, int q, int nwin,
                            unsigned& fp64_tests) {
  constexpr int NP = NC / 2;  // pairs per round, pair 0 included
  static_assert(NP <= 8, "each lane owns two pairs");
  const int gbase = (threadIdx.x & 31) & ~3;
  const int up = gbase | ((q + 1) & 3), dn = gbase | ((q + 3) & 3);
  const bool b1 = (q & 2) != 0, b0 = (q & 1) != 0;
  int sweeps = 0;
#pragma unroll 1
  for (; sweeps < kMaxSweeps; ++sweeps) {
    // squared norms of the owned pairs' columns: L[i] of position q + 4i,
    // R[i] of position NC - 1 - q - 4i (the pad column's is 0)
    float L[2], R[2];
    {
      float nrm[NC];
#pragma unroll
      for (int k = 0; k < NC - 1; ++k) {
        float t = 0.f;
#pragma unroll
        for (int r = 0; r < 4; ++r) t = fmaf(A(r, k), A(r, k), t);
        nrm[k] = lanes_sum<4>(t);
      }
      nrm[NC - 1] = 0.f;
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        L[i] = sel4(q, nrm[(4 * i) % NC], nrm[(4 * i + 1) % NC], nrm[(4 * i + 2) % NC],
                    nrm[(4 * i + 3) % NC]);
        R[i] = sel4(q, nrm[NC - 1 - 4 * i], nrm[NC - 2 - 4 * i], nrm[NC - 3 - 4 * i],
                    nrm[NC - 4 - 4 * i]);
      }
    }
    bool definite = false, band = false, big = false;
#pragma unroll U
    for (int rd = 0; rd < NC - 1; ++rd) {
      // this lane's partial inner products of the round's pairs
      float gm[8];
#pragma unroll
      for (int pp = 0; pp < 8; ++pp) {
        if (pp >= 1 && pp < NP) {
          float2 t = __fmul2_rn(A.v[0][pp], A.v[0][NC - 1 - pp]);
          t = __ffma2_rn(A.v[1][pp], A.v[1][NC - 1 - pp], t);
          gm[pp] = t.x + t.y;
        } else {
          gm[pp] = 0.f;
        }
      }
      // reduce-scatter: across lanes q, q^2 keep the pairs whose bit 1 is
      // q's (pp = 2*b1 + {0, 1, 4, 5}), then across q, q^1 those whose bit
      // 0 is q's: the inner product of pair q + 4i
      float h[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int lo = (j & 1) | ((j >> 1) << 2);
        const float keep = b1 ? gm[lo + 2] : gm[lo];
        const float send = b1 ? gm[lo] : gm[lo + 2];
        h[j] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
      }
      float cs_[2], sn_[2];
      bool need_[2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const float keep = b0 ? h[2 * i + 1] : h[2 * i];
        const float send = b0 ? h[2 * i] : h[2 * i + 1];
        const float gv = keep + __shfl_xor_sync(0xffffffffu, send, 1);
        const int po = q + 4 * i;  // the owned pair
        const float al = L[i], be = R[i];
        const float g2 = gv * gv, ab = al * be;
        need_[i] = po >= 1 && po < NP && g2 > (kTol * kTol) * ab;
        cs_[i] = 1.f;
        sn_[i] = 0.f;
        if (need_[i]) {
          rotation(al, be, gv, g2, ab, cs_[i], sn_[i], definite, band);
          big |= g2 > (kStopRel * kStopRel) * ab;
          rotated_norms(al, be, gv, cs_[i], sn_[i], L[i], R[i]);
        }
      }
      const unsigned m0 = __ballot_sync(0xffffffffu, need_[0]);
      const unsigned m1 = __ballot_sync(0xffffffffu, need_[1]);
#pragma unroll
      for (int pp = 1; pp < NP; ++pp) {
        const int i = pp >> 2;
        if (!((i ? m1 : m0) & (0x11111111u << (pp & 3)))) continue;  // warp-uniform
        const int src = gbase | (pp & 3);
        const float cs = __shfl_sync(0xffffffffu, cs_[i], src);
        const float sn = __shfl_sync(0xffffffffu, sn_[i], src);
        A.rotate(pp, NC - 1 - pp, cs, sn);
      }
      A.shift();
      // the norms follow their columns to the next round's owners: the new
      // left member of pair p is the old left member of pair p + 1 (for the
      // last pair, its own old right member), the new right member of pair p
      // the old right member of pair p - 1 (for pair 1, the old left member
      // of pair 0; for pair 0, the pad)
      float nl[2], nr[2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const float vl = (q == 0) ? L[(i + 1) & 1] : L[i];
        const float vr = (q == 3) ? (i == 0 ? 0.f : R[0]) : ((q == 0 && i == 0) ? L[0] : R[i]);
        nl[i] = __shfl_sync(0xffffffffu, vl, up);
        nr[i] = __shfl_sync(0xffffffffu, vr, dn);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        L[i] = (q + 4 * i == NP - 1) ? R[i] : nl[i];
        R[i] = nr[i];
      }
    }
    if (__any_sync(0xffffffffu, definite)) {
      // every rotation of the sweep was smaller than kStopRel: convergence is
      // quadratic, so the inner products it leaves are of order kStopRel^2,
      // the rotation threshold, and the next sweep would be the last
      if (!__any_sync(0xffffffffu, band) && !__any_sync(0xffffffffu, big)) break;
      continue;
    }
    if (!__any_sync(0xffffffffu, band)) break;
#pragma unroll
    for (int k = 0; k < NC; ++k)
#pragma unroll
      for (int r = 0; r < 4; ++r) As[k * CS + q * 4 + r] = A(r, k);
    __syncwarp();
    if (!fp64_check<4, 4, CS>(As, q, nwin, fp64_tests)) break;
  }
  return sweeps;
}

// Jacobi sweeps with the columns in registers: the round-robin moves them one
// position per round.  Column norms are recomputed exactly at every sweep's
// start and updated in closed form after each rotation.  Returns the sweeps
// with rotations; As ([NC][CS]) stages the columns for the FP64 check.
// Patches of 4 lanes x 4 rows take the owner form above.
template <int RPL, int LANES, int NC, int CS, int U>
__device__ int register_sweeps(RegCols<RPL, NC>& A, float* As, int q, int nwin,
                               unsigned& fp64_tests) {
  if constexpr (kOwnerForm<RPL, LANES, NC>)
    return owner_sweeps<NC, CS, kOwnerUnroll<NC>>(A, As, q, nwin, fp64_tests);
  int sweeps = 0;
  float nrm[NC];
#pragma unroll 1
  for (; sweeps < kMaxSweeps; ++sweeps) {
#pragma unroll
    for (int k = 0; k < NC - 1; ++k) {
      float s = 0.f;
#pragma unroll
      for (int r = 0; r < RPL; ++r) s = fmaf(A(r, k), A(r, k), s);
      nrm[k] = lanes_sum<LANES>(s);
    }
    nrm[NC - 1] = 0.f;
    bool definite = false, band = false;
#pragma unroll U
    for (int rd = 0; rd < NC - 1; ++rd) {
      float gm[NC / 2];
#pragma unroll
      for (int pp = 1; pp < NC / 2; ++pp) {
        float s = 0.f;
#pragma unroll
        for (int r = 0; r < RPL; ++r) s = fmaf(A(r, pp), A(r, NC - 1 - pp), s);
        gm[pp] = s;
      }
#pragma unroll
      for (int o = 1; o < LANES; o <<= 1)
#pragma unroll
        for (int pp = 1; pp < NC / 2; ++pp) gm[pp] += __shfl_xor_sync(0xffffffffu, gm[pp], o);
#pragma unroll
      for (int pp = 1; pp < NC / 2; ++pp) {
        const int pi = pp, pj = NC - 1 - pp;
        const float al = nrm[pi], be = nrm[pj], gv = gm[pp];
        const float g2 = gv * gv, ab = al * be;
        const bool need = g2 > (kTol * kTol) * ab;
        if (!__any_sync(0xffffffffu, need)) continue;  // converged pair in every lane
        if (need) {
          float cs, sn;
          rotation(al, be, gv, g2, ab, cs, sn, definite, band);
          A.rotate(pi, pj, cs, sn);
          rotated_norms(al, be, gv, cs, sn, nrm[pi], nrm[pj]);
        }
      }
      A.shift();
      shift_norms<NC>(nrm);
    }
    if (__any_sync(0xffffffffu, definite)) continue;
    if (!__any_sync(0xffffffffu, band)) break;
#pragma unroll
    for (int k = 0; k < NC; ++k)
#pragma unroll
      for (int r = 0; r < RPL; ++r) As[k * CS + q * RPL + r] = A(r, k);
    __syncwarp();
    if (!fp64_check<RPL, LANES, CS>(As, q, nwin, fp64_tests)) break;
  }
  return sweeps;
}

template <int RPL, int LANES, int NC, bool SM = false>
__global__ void __launch_bounds__(128, (svd_minblocks<RPL, NC, SM>()))
    k_svd(Problem pb, DeviceBuffers d, int nitems) {
  constexpr int GROUPS = 32 / LANES;
  constexpr int GSTRIDE = SvdSmem<RPL, LANES, NC, SM>::STRIDE;  // smem floats per patch
  constexpr int CS = SvdSmem<RPL, LANES, NC, SM>::CS;
  constexpr int U = ((NC - 1) % PGSVT_SVD_UNROLL == 0) ? PGSVT_SVD_UNROLL : 1;
  const Geometry& g = pb.g;
  const int lane = threadIdx.x & 31;
  const int q = lane % LANES;     // row block of this lane
  const int grp = lane / LANES;   // patch slot in the warp
  const int wib = threadIdx.x >> 5;
  const int gid = (blockIdx.x * (blockDim.x >> 5) + wib) * GROUPS + grp;
  const bool live = gid < nitems;
  int p, c, w;
  {
    const int gg = live ? gid : 0;
    p = gg % g.NP;
    const int r = gg / g.NP;
    c = r % d.ncopies;
    w = r / d.ncopies;
  }
  const WinConst& wc = d.wc[w];
  const size_t F = g.F();
  const float* uw = d.u + (size_t)w * g.cube();
  const int posidx = d.plist[p];
  const uint32_t* posw = d.pos + (size_t)w * g.nwin * g.P;
  const size_t poff = (size_t)w * d.probe_stride;
  const int nwin = g.nwin;

  // offsets of this lane's rows inside a frame (row e of the Casorati matrix
  // is pixel (e % bs, e / bs) of the patch, svt.hpp:105-108); -1: padding row
  int roff[RPL];
#pragma unroll
  for (int r = 0; r < RPL; ++r) {
    const int e = q * RPL + r;
    roff[r] = (live && e < g.M) ? (e % g.bs) + (e / g.bs) * g.S : -1;
  }
  // perturbation of copy c (pgure.hpp:80-82), precomputed in FP32
  float pa = 0.f, pb0 = 0.f;
  if (c == 1 || c == 2) {
    const double sg = (c == 1) ? 1.0 : -1.0;
    pa = (float)(sg * d.d2neg * wc.eps2);  // delta2 code 1
    pb0 = (float)(sg * d.d2pos * wc.eps2); // delta2 code 0
  } else if (c == 3) {
    pa = (float)wc.eps1;                   // delta1 = +1 (times eps1)
  }
  auto value = [&](size_t kidx) -> float {
    float v = __ldg(uw + kidx);
    if (c == 1 || c == 2) v += __ldg(d.d2code + poff + kidx) ? pa : pb0;
    else if (c == 3) v += (float)__ldg(d.d1 + poff + kidx) * pa;
    return v;
  };

  extern __shared__ float smem[];
  float* As = smem + (size_t)(wib * GROUPS + grp) * GSTRIDE;  // [NC][CS]

  // ---- gather B (svt.hpp:101-109)
  RegCols<RPL, NC> A;
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    size_t base = 0;
    const bool colok = live && k < nwin;
    if (colok) {
      const uint32_t pc = __ldg(posw + (size_t)k * g.P + posidx);
      base = (size_t)k * F + (pc & 0xffffu) + (size_t)(pc >> 16) * g.S;
    }
#pragma unroll
    for (int r = 0; r < RPL; ++r) {
      const float v = (colok && roff[r] >= 0) ? value(base + roff[r]) : 0.f;
      if constexpr (SM) As[k * CS + q * RPL + r] = v;
      else A(r, k) = v;
    }
  }

  // ---- Jacobi sweeps
  int sweeps = 0;
  unsigned fp64_tests = 0;
  auto fp64_again = [&]() { return fp64_check<RPL, LANES, CS>(As, q, nwin, fp64_tests); };
  if constexpr (!SM) {
    sweeps = register_sweeps<RPL, LANES, NC, CS, U>(A, As, q, nwin, fp64_tests);
  } else {
    // columns in shared memory, addressed by the same round-robin schedule
    // (position k of round rd holds column (k + rd) mod (NC-1)): the same
    // rotations in the same order, without moving data
    float* nrs = As + NC * CS;  // column norms
#pragma unroll 1
    for (; sweeps < kMaxSweeps; ++sweeps) {
#pragma unroll
      for (int k = 0; k < NC - 1; ++k) {
        float s = 0.f;
#pragma unroll
        for (int r = 0; r < RPL; ++r) {
          const float x = As[k * CS + q * RPL + r];
          s = fmaf(x, x, s);
        }
        s = lanes_sum<LANES>(s);
        if (q == 0) nrs[k] = s;
      }
      if (q == 0) nrs[NC - 1] = 0.f;
      __syncwarp();
      bool definite = false, band = false, big = false;
#pragma unroll 1
      for (int rd = 0; rd < NC - 1; ++rd) {
        float va[NC / 2][RPL], vb[NC / 2][RPL], gm[NC / 2];
        int ca[NC / 2], cb[NC / 2];
#pragma unroll
        for (int pp = 1; pp < NC / 2; ++pp) {
          int ia = pp + rd, ib = NC - 1 - pp + rd;
          if (ia >= NC - 1) ia -= NC - 1;
          if (ib >= NC - 1) ib -= NC - 1;
          ca[pp] = ia;
          cb[pp] = ib;
          load_rows<RPL>(As + ia * CS + q * RPL, va[pp]);
          load_rows<RPL>(As + ib * CS + q * RPL, vb[pp]);
          float s = 0.f;
#pragma unroll
          for (int r = 0; r < RPL; ++r) s = fmaf(va[pp][r], vb[pp][r], s);
          gm[pp] = s;
        }
        if constexpr (kOwnerForm<RPL, LANES, NC>) {
          // the owner form's order of operations (owner_sweeps): packed
          // partial products, the reduce-scatter, one rotation per pair
          // computed by its owner lane and broadcast; identical results
#pragma unroll
          for (int pp = 1; pp < NC / 2; ++pp) {
            float p0 = va[pp][0] * vb[pp][0], p1 = va[pp][1] * vb[pp][1];
            p0 = fmaf(va[pp][2], vb[pp][2], p0);
            p1 = fmaf(va[pp][3], vb[pp][3], p1);
            gm[pp] = p0 + p1;
          }
          float g8[8];
#pragma unroll
          for (int pp = 0; pp < 8; ++pp) g8[pp] = (pp >= 1 && pp < NC / 2) ? gm[pp] : 0.f;
          const bool b1 = (q & 2) != 0, b0 = (q & 1) != 0;
          float h[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int lo = (j & 1) | ((j >> 1) << 2);
            const float keep = b1 ? g8[lo + 2] : g8[lo];
            const float send = b1 ? g8[lo] : g8[lo + 2];
            h[j] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
          }
          float cs_[2], sn_[2];
          bool need_[2];
#pragma unroll
          for (int i = 0; i < 2; ++i) {
            const float keep = b0 ? h[2 * i + 1] : h[2 * i];
            const float send = b0 ? h[2 * i] : h[2 * i + 1];
            const float gv = keep + __shfl_xor_sync(0xffffffffu, send, 1);
            const int po = q + 4 * i;
            int ia = po + rd, ib = NC - 1 - po + rd;
            if (ia >= NC - 1) ia -= NC - 1;
            if (ib >= NC - 1) ib -= NC - 1;
            const bool valid = po >= 1 && po < NC / 2;
            const float al = valid ? nrs[ia] : 0.f, be = valid ? nrs[ib] : 0.f;
            const float g2 = gv * gv, ab = al * be;
            need_[i] = valid && g2 > (kTol * kTol) * ab;
            cs_[i] = 1.f;
            sn_[i] = 0.f;
            if (need_[i]) {
              rotation(al, be, gv, g2, ab, cs_[i], sn_[i], definite, band);
              big |= g2 > (kStopRel * kStopRel) * ab;
              float ni, nj;
              rotated_norms(al, be, gv, cs_[i], sn_[i], ni, nj);
              nrs[ia] = ni;
              nrs[ib] = nj;
            }
          }
          const unsigned m0 = __ballot_sync(0xffffffffu, need_[0]);
          const unsigned m1 = __ballot_sync(0xffffffffu, need_[1]);
          const int gbase = lane & ~3;
#pragma unroll
          for (int pp = 1; pp < NC / 2; ++pp) {
            const int i = pp >> 2;
            if (!((i ? m1 : m0) & (0x11111111u << (pp & 3)))) continue;  // warp-uniform
            const float cs = __shfl_sync(0xffffffffu, cs_[i], gbase | (pp & 3));
            const float sn = __shfl_sync(0xffffffffu, sn_[i], gbase | (pp & 3));
#pragma unroll
            for (int r = 0; r < RPL; ++r) {
              const float a = va[pp][r], b = vb[pp][r];
              va[pp][r] = fmaf(cs, a, -sn * b);
              vb[pp][r] = fmaf(sn, a, cs * b);
            }
            store_rows<RPL>(As + ca[pp] * CS + q * RPL, va[pp]);
            store_rows<RPL>(As + cb[pp] * CS + q * RPL, vb[pp]);
          }
        } else {
#pragma unroll
        for (int o = 1; o < LANES; o <<= 1)
#pragma unroll
          for (int pp = 1; pp < NC / 2; ++pp) gm[pp] += __shfl_xor_sync(0xffffffffu, gm[pp], o);
#pragma unroll
        for (int pp = 1; pp < NC / 2; ++pp) {
          const float al = nrs[ca[pp]], be = nrs[cb[pp]], gv = gm[pp];
          const float g2 = gv * gv, ab = al * be;
          const bool need = g2 > (kTol * kTol) * ab;
          if (!__any_sync(0xffffffffu, need)) continue;
          if (need) {
            float cs, sn;
            rotation(al, be, gv, g2, ab, cs, sn, definite, band);
#pragma unroll
            for (int r = 0; r < RPL; ++r) {
              const float a = va[pp][r], b = vb[pp][r];
              va[pp][r] = fmaf(cs, a, -sn * b);
              vb[pp][r] = fmaf(sn, a, cs * b);
            }
            store_rows<RPL>(As + ca[pp] * CS + q * RPL, va[pp]);
            store_rows<RPL>(As + cb[pp] * CS + q * RPL, vb[pp]);
            float ni, nj;
            rotated_norms(al, be, gv, cs, sn, ni, nj);
            if (q == 0) {
              nrs[ca[pp]] = ni;
              nrs[cb[pp]] = nj;
            }
          }
        }
        }
        __syncwarp();
      }
      if (__any_sync(0xffffffffu, definite)) {
        if constexpr (kOwnerForm<RPL, LANES, NC>)  // the owner form's stopping rule
          if (!__any_sync(0xffffffffu, band) && !__any_sync(0xffffffffu, big)) break;
        continue;
      }
      if (!__any_sync(0xffffffffu, band)) break;
      if (!fp64_again()) break;
    }
  }
  if (lane == 0) atomicAdd(d.counters + 1, (unsigned long long)(sweeps + 1));
  if (q == 0 && fp64_tests) atomicAdd(d.counters + 2, (unsigned long long)fp64_tests);

  // ---- epilogue
  // singular values and their order
  float sv[NC];
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    float s = 0.f;
#pragma unroll
    for (int r = 0; r < RPL; ++r) {
      if constexpr (SM) {
        const float x = As[k * CS + q * RPL + r];
        s = fmaf(x, x, s);
      } else {
        s = fmaf(A(r, k), A(r, k), s);
        As[k * CS + q * RPL + r] = A(r, k);
      }
    }
    sv[k] = sqrtf(lanes_sum<LANES>(s));
  }
  __syncwarp();
  float smax = sv[0];
#pragma unroll
  for (int k = 1; k < NC; ++k) smax = fmaxf(smax, sv[k]);
  const size_t NP = g.NP;
  const int NCg = g.NC;
  const int cslot = c;
  float* svo = d.sv + (((size_t)w * 4 + cslot) * NCg) * NP + p;
  float* hvo = d.hv + (((size_t)w * 4 + cslot) * NCg) * NP + p;
  // column of rank t: walk the columns in decreasing order (ties by index)
  int nl = 0;
#pragma unroll
  for (int k = 0; k < NC; ++k) nl += can_survive(pb, sv[k], smax, (float)wc.upper);
  int nl_max = nl;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) nl_max = max(nl_max, __shfl_xor_sync(0xffffffffu, nl_max, o));
  if (c == 0 && live && q == 0) d.nlive0[(size_t)w * NP + p] = nl;

  // B again (the Jacobi overwrote it) and the lambda-independent field G
  const float* fld = (c == 0) ? d.fld0 : (c == 3 ? d.fld1 : d.fld2);
  const float* fw_ = (pb.optimize && fld) ? fld + (size_t)w * g.cube() : nullptr;
  float B[RPL][NC];
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    size_t base = 0;
    const bool colok = live && k < nwin && nl_max > 0;
    if (colok) {
      const uint32_t pc = __ldg(posw + (size_t)k * g.P + posidx);
      base = (size_t)k * F + (pc & 0xffffu) + (size_t)(pc >> 16) * g.S;
    }
#pragma unroll
    for (int r = 0; r < RPL; ++r) B[r][k] = (colok && roff[r] >= 0) ? value(base + roff[r]) : 0.f;
  }
  int prev = -1;
  float prev_s = INFINITY;
  for (int t = 0; t < NC; ++t) {
    // next column in decreasing singular-value order
    int ct = 0;
    float st = -1.f;
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      const float s = sv[k];
      const bool after = (s < prev_s) || (s == prev_s && k > prev);
      if (after && (s > st)) {
        st = s;
        ct = k;
      }
    }
    prev = ct;
    prev_s = st;
    const bool use = t < nl;
    if (live && q == 0) {
      svo[(size_t)t * NP] = st;
      if (!use) hvo[(size_t)t * NP] = 0.f;
    }
    if (t >= nl_max) continue;  // warp-uniform
    const float inv = st > 0.f ? 1.f / st : 0.f;
    float a[RPL];
#pragma unroll
    for (int r = 0; r < RPL; ++r) a[r] = As[ct * CS + q * RPL + r] * inv;  // u_t rows
    if (c == 0 && live && use && d.U0) {
#pragma unroll
      for (int r = 0; r < RPL; ++r)
        if (roff[r] >= 0) d.U0[(((size_t)w * NCg + t) * g.M + q * RPL + r) * NP + p] = a[r];
    }
    // v_t = B^T u_t / s_t and h_t = u_t^T G v_t = sum_k v_k (G_k . u_t),
    // the latter from the lanes' partial sums with one reduction
    float h = 0.f;
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      if (k >= nwin) break;  // uniform: keeps B[][k] in registers
      float bu = 0.f;
#pragma unroll
      for (int r = 0; r < RPL; ++r) bu = fmaf(B[r][k], a[r], bu);
      bu = lanes_sum<LANES>(bu);
      const float vk = bu * inv;
      if (c == 0 && live && use && (k % LANES) == q && d.V0)
        d.V0[(((size_t)w * NCg + t) * nwin + k) * NP + p] = vk;
      if (fw_ && live && use) {
        const uint32_t pc = __ldg(posw + (size_t)k * g.P + posidx);
        const size_t base = (size_t)k * F + (pc & 0xffffu) + (size_t)(pc >> 16) * g.S;
        float gu = 0.f;
#pragma unroll
        for (int r = 0; r < RPL; ++r)
          if (roff[r] >= 0) gu = fmaf(__ldg(fw_ + base + roff[r]), a[r], gu);
        h = fmaf(vk, gu, h);
      }
    }
    if (fw_) h = lanes_sum<LANES>(h);
    if (live && use && q == 0) hvo[(size_t)t * NP] = h;
  }
}

template <int RPL, int LANES, int NC, bool SM>
cudaError_t run_svd(const Problem& pb, const DeviceBuffers& d, cudaStream_t s) {
  constexpr int GROUPS = 32 / LANES;
  constexpr int GSTRIDE = SvdSmem<RPL, LANES, NC, SM>::STRIDE;
  const int nitems = pb.W * d.ncopies * pb.g.NP;
  const int warps = (nitems + GROUPS - 1) / GROUPS;
  const int wpb = 4;
  const size_t shm = (size_t)wpb * GROUPS * GSTRIDE * sizeof(float);
  cudaError_t e = cudaFuncSetAttribute(k_svd<RPL, LANES, NC, SM>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  if (e != cudaSuccess) return e;
  k_svd<RPL, LANES, NC, SM><<<(warps + wpb - 1) / wpb, wpb * 32, shm, s>>>(pb, d, nitems);
  return cudaGetLastError();
}

}  // namespace svdk
}  // namespace pgsvt

#define PGSVT_INSTANTIATE_SVD_SM(RPL, LANES, NC, SM)                               \
  template cudaError_t pgsvt::svdk::run_svd<RPL, LANES, NC, SM>(                    \
      const pgsvt::Problem&, const pgsvt::DeviceBuffers&, cudaStream_t);
#define PGSVT_INSTANTIATE_SVD(RPL, LANES, NC) PGSVT_INSTANTIATE_SVD_SM(RPL, LANES, NC, false)

#endif
