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

// Round-robin ordering with a fixed pairing pattern in register space: the
// pad column (always zero, nwin < NC) sits at position NC-1 and meets
// position 0 (a skipped, trivial pair); positions k and NC-1-k (k >= 1) are
// paired; after each round positions 0..NC-2 shift by one.  NC-1 rounds pair
// every two columns once and bring every column back to its position.

template <int RPL, int NC>
__device__ __forceinline__ void shift_round(float (&A)[RPL][NC], float (&nrm)[NC]) {
#pragma unroll
  for (int r = 0; r < RPL; ++r) {
    const float t = A[r][0];
#pragma unroll
    for (int k = 0; k < NC - 2; ++k) A[r][k] = A[r][k + 1];
    A[r][NC - 2] = t;
  }
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

// Rounds unrolled per loop iteration (code size vs register moves of the
// round shift) and the residency target of the launch bounds.
#ifndef PGSVT_SVD_UNROLL
#define PGSVT_SVD_UNROLL 1
#endif
#ifndef PGSVT_SVD_MINBLOCKS
#define PGSVT_SVD_MINBLOCKS 3
#endif

template <int RPL, int LANES, int NC>
__global__ void __launch_bounds__(128, PGSVT_SVD_MINBLOCKS) k_svd(Problem pb, DeviceBuffers d,
                                                                  int nitems) {
  constexpr int GROUPS = 32 / LANES;
  constexpr int MP = RPL * LANES;               // padded rows
  constexpr int GSTRIDE = NC * (MP + 1) + 4;    // smem floats per patch
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

  // ---- gather B (svt.hpp:101-109)
  float A[RPL][NC];
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    size_t base = 0;
    const bool colok = live && k < nwin;
    if (colok) {
      const uint32_t pc = __ldg(posw + (size_t)k * g.P + posidx);
      base = (size_t)k * F + (pc & 0xffffu) + (size_t)(pc >> 16) * g.S;
    }
#pragma unroll
    for (int r = 0; r < RPL; ++r) A[r][k] = (colok && roff[r] >= 0) ? value(base + roff[r]) : 0.f;
  }

  extern __shared__ float smem[];
  float* As = smem + (size_t)(wib * GROUPS + grp) * GSTRIDE;  // [NC][MP+1]

  // ---- Jacobi sweeps
  float nrm[NC];
  int sweeps = 0;
  unsigned fp64_tests = 0;
#pragma unroll 1
  for (; sweeps < kMaxSweeps; ++sweeps) {
#pragma unroll
    for (int k = 0; k < NC - 1; ++k) {
      float s = 0.f;
#pragma unroll
      for (int r = 0; r < RPL; ++r) s = fmaf(A[r][k], A[r][k], s);
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
        for (int r = 0; r < RPL; ++r) s = fmaf(A[r][pp], A[r][NC - 1 - pp], s);
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
          const bool degen = fabsf(be - al) <= kDegen * (al + be);
          if (degen && g2 <= (kBand * kBand * kTol * kTol) * ab) band = true;
          else definite = true;
          // Rotation angle from the half-angle identities: with d = be - al,
          // r = sqrt(d^2 + 4g^2), cos 2th = |d| / r and sin 2th = 2 g sign(d) / r
          // (the smaller of the two orthogonalising angles, sign(0) = +1):
          // cos th = sqrt((1 + cos 2th) / 2), sin th = sin 2th / (2 cos th).
          const float dd = be - al;
          const float ir = rsqrtf(fmaf(dd, dd, 4.f * g2));
          const float hh = fmaf(0.5f * fabsf(dd), ir, 0.5f);  // (1 + cos 2th) / 2
          const float rh = rsqrtf(hh);
          const float cs = hh * rh;
          const float sn = (dd >= 0.f ? gv : -gv) * ir * rh;
#pragma unroll
          for (int r = 0; r < RPL; ++r) {
            const float a = A[r][pi], b = A[r][pj];
            A[r][pi] = fmaf(cs, a, -sn * b);
            A[r][pj] = fmaf(sn, a, cs * b);
          }
          // |c a - s b|^2 and |s a + c b|^2 from al, be, g
          const float c2 = cs * cs, s2 = sn * sn, csg = 2.f * cs * sn * gv;
          nrm[pi] = fmaf(c2, al, fmaf(s2, be, -csg));
          nrm[pj] = fmaf(s2, al, fmaf(c2, be, csg));
        }
      }
      shift_round<RPL, NC>(A, nrm);
    }
    if (__any_sync(0xffffffffu, definite)) continue;
    if (!__any_sync(0xffffffffu, band)) break;
    // Only near-degenerate pairs moved, by amounts at the FP32 noise level of
    // their inner products: decide convergence from FP64 inner products of
    // the current columns (exact products of the FP32 entries).
#pragma unroll
    for (int k = 0; k < NC; ++k)
#pragma unroll
      for (int r = 0; r < RPL; ++r) As[k * (MP + 1) + q * RPL + r] = A[r][k];
    __syncwarp();
    bool again = false;
    for (int i = 0; i < nwin; ++i) {
      for (int j = i + 1; j < nwin; ++j) {
        float gi = 0.f, ai = 0.f, aj = 0.f;
#pragma unroll
        for (int r = 0; r < RPL; ++r) {
          const float x = As[i * (MP + 1) + q * RPL + r], y = As[j * (MP + 1) + q * RPL + r];
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
            g64 = fma((double)As[i * (MP + 1) + q * RPL + r], (double)As[j * (MP + 1) + q * RPL + r], g64);
          g64 = lanes_sum_d<LANES>(g64);
          if (cand) {
            ++fp64_tests;
            if (fabs(g64) > (double)kTol * (double)sc) again = true;
          }
        }
      }
    }
    __syncwarp();
    if (!__any_sync(0xffffffffu, again)) break;
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
      s = fmaf(A[r][k], A[r][k], s);
      As[k * (MP + 1) + q * RPL + r] = A[r][k];
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
    for (int r = 0; r < RPL; ++r) a[r] = As[ct * (MP + 1) + q * RPL + r] * inv;  // u_t rows
    if (c == 0 && live && use) {
#pragma unroll
      for (int r = 0; r < RPL; ++r)
        if (roff[r] >= 0) d.U0[(((size_t)w * NCg + t) * g.M + q * RPL + r) * NP + p] = a[r];
    }
    // v_t = B^T u_t / s_t and h_t = u_t^T G v_t, summed over the lanes' rows
    float h = 0.f;
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      if (k >= nwin) break;  // uniform: keeps B[][k] in registers
      float bu = 0.f;
#pragma unroll
      for (int r = 0; r < RPL; ++r) bu = fmaf(B[r][k], a[r], bu);
      bu = lanes_sum<LANES>(bu);
      const float vk = bu * inv;
      if (c == 0 && live && use && (k % LANES) == q)
        d.V0[(((size_t)w * NCg + t) * nwin + k) * NP + p] = vk;
      if (fw_) {
        float gu = 0.f;
        if (live && use) {
          const uint32_t pc = __ldg(posw + (size_t)k * g.P + posidx);
          const size_t base = (size_t)k * F + (pc & 0xffffu) + (size_t)(pc >> 16) * g.S;
#pragma unroll
          for (int r = 0; r < RPL; ++r)
            if (roff[r] >= 0) gu = fmaf(__ldg(fw_ + base + roff[r]), a[r], gu);
        }
        h = fmaf(vk, lanes_sum<LANES>(gu), h);
      }
    }
    if (live && use && q == 0) hvo[(size_t)t * NP] = h;
  }
}

template <int RPL, int LANES, int NC>
cudaError_t run_svd(const Problem& pb, const DeviceBuffers& d, cudaStream_t s) {
  constexpr int GROUPS = 32 / LANES, MP = RPL * LANES;
  constexpr int GSTRIDE = NC * (MP + 1) + 4;
  const int nitems = pb.W * d.ncopies * pb.g.NP;
  const int warps = (nitems + GROUPS - 1) / GROUPS;
  const int wpb = 4;
  const size_t shm = (size_t)wpb * GROUPS * GSTRIDE * sizeof(float);
  cudaError_t e = cudaFuncSetAttribute(k_svd<RPL, LANES, NC>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  if (e != cudaSuccess) return e;
  k_svd<RPL, LANES, NC><<<(warps + wpb - 1) / wpb, wpb * 32, shm, s>>>(pb, d, nitems);
  return cudaGetLastError();
}

}  // namespace svdk
}  // namespace pgsvt

#define PGSVT_INSTANTIATE_SVD(RPL, LANES, NC) \
  template cudaError_t pgsvt::svdk::run_svd<RPL, LANES, NC>(const pgsvt::Problem&, \
                                                          const pgsvt::DeviceBuffers&, cudaStream_t);

#endif
