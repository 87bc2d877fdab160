// svd_kernel.cuh — the batched one-sided Jacobi kernel template (see svd.cu).
#ifndef PGSVT_SVD_KERNEL_CUH
#define PGSVT_SVD_KERNEL_CUH

#include "pgsvt_internal.h"

namespace pgsvt {
namespace svdk {

constexpr int kMaxSweeps = 16;
constexpr float kTol = 1e-6f;

// round-robin (circle method) schedule: player NC-1 fixed
template <int NC>
__device__ __forceinline__ constexpr int rr_i(int rd, int pp) {
  return pp == 0 ? rd : (rd + pp) % (NC - 1);
}
template <int NC>
__device__ __forceinline__ constexpr int rr_j(int rd, int pp) {
  return pp == 0 ? NC - 1 : (rd - pp + (NC - 1)) % (NC - 1);
}

struct Item {
  int w, c, p;  // window, copy, kept patch
  bool live;
};

// value of the copy-c matrix at voxel idx of slice k
// (pgure.hpp:80-82: U1 = U + delta1*eps1, U2p = U + delta2*eps2, U2m = U - delta2*eps2)
__device__ __forceinline__ float perturbed(const DeviceBuffers& d, const WinConst& wc, int c,
                                           const float* u, size_t kidx, size_t poff) {
  const float v = u[kidx];
  if (c == 0) return v;
  if (c == 3) return v + (float)((double)d.d1[poff + kidx] * wc.eps1);
  const double dl = d.d2code[poff + kidx] ? d.d2neg : d.d2pos;
  return (c == 1) ? v + (float)(dl * wc.eps2) : v - (float)(dl * wc.eps2);
}

template <int RPL, int LANES, int NC>
__global__ void __launch_bounds__(128) k_svd(Problem pb, DeviceBuffers d, int nitems) {
  constexpr int GROUPS = 32 / LANES;
  constexpr int MP = RPL * LANES;  // padded rows
  const Geometry& g = pb.g;
  const int lane = threadIdx.x & 31;
  const int q = lane % LANES;       // row block of this lane
  const int grp = lane / LANES;     // patch slot in the warp
  const int warp_in_blk = threadIdx.x >> 5;
  const int gid = (blockIdx.x * (blockDim.x >> 5) + warp_in_blk) * GROUPS + grp;
  Item it;
  it.live = gid < nitems;
  {
    const int gg = it.live ? gid : 0;
    it.p = gg % g.NP;
    const int r = gg / g.NP;
    it.c = r % d.ncopies;
    it.w = r / d.ncopies;
  }
  const WinConst& wc = d.wc[it.w];
  const size_t F = g.F();
  const float* uw = d.u + (size_t)it.w * g.cube();
  const int posidx = d.plist[it.p];
  const uint32_t* posw = d.pos + (size_t)it.w * g.nwin * g.P;
  const size_t poff = (size_t)it.w * d.probe_stride;

  // ---- gather B (svt.hpp:101-109)
  float A[RPL][NC];
#pragma unroll
  for (int r = 0; r < RPL; ++r) {
    const int e = q * RPL + r;
    const int er = e % g.bs, ec = e / g.bs;
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      float v = 0.f;
      if (it.live && e < g.M && k < g.nwin) {
        const uint32_t pc = __ldg(posw + (size_t)k * g.P + posidx);
        const size_t kidx = (size_t)k * F + ((pc & 0xffffu) + er) + (size_t)((pc >> 16) + ec) * g.S;
        v = perturbed(d, wc, it.c, uw, kidx, poff);
      }
      A[r][k] = v;
    }
  }

  // ---- Jacobi sweeps
  float nrm[NC];
  int sweeps = 0;
#pragma unroll 1
  for (; sweeps < kMaxSweeps; ++sweeps) {
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      float s = 0.f;
#pragma unroll
      for (int r = 0; r < RPL; ++r) s = fmaf(A[r][k], A[r][k], s);
#pragma unroll
      for (int o = 1; o < LANES; o <<= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      nrm[k] = s;
    }
    bool unconverged = false;
#pragma unroll
    for (int rd = 0; rd < NC - 1; ++rd) {
      float gm[NC / 2];
#pragma unroll
      for (int pp = 0; pp < NC / 2; ++pp) {
        const int pi = rr_i<NC>(rd, pp), pj = rr_j<NC>(rd, pp);
        float s = 0.f;
#pragma unroll
        for (int r = 0; r < RPL; ++r) s = fmaf(A[r][pi], A[r][pj], s);
        gm[pp] = s;
      }
#pragma unroll
      for (int o = 1; o < LANES; o <<= 1)
#pragma unroll
        for (int pp = 0; pp < NC / 2; ++pp) gm[pp] += __shfl_xor_sync(0xffffffffu, gm[pp], o);
#pragma unroll
      for (int pp = 0; pp < NC / 2; ++pp) {
        const int pi = rr_i<NC>(rd, pp), pj = rr_j<NC>(rd, pp);
        const float al = nrm[pi], be = nrm[pj], gv = gm[pp];
        const float scale = sqrtf(al * be);
        const float ratio = fabsf(gv);
        bool doit = ratio > kTol * scale;
        // near-degenerate pair close to the threshold: decide in FP64
        const bool amb = ratio > 0.5f * kTol * scale && ratio <= 2.f * kTol * scale &&
                         fabsf(be - al) <= 1e-3f * (al + be);
        if (__any_sync(0xffffffffu, amb)) {
          double g64 = 0.0, a64 = 0.0, b64 = 0.0;
#pragma unroll
          for (int r = 0; r < RPL; ++r) {
            const double x = A[r][pi], y = A[r][pj];
            g64 = fma(x, y, g64);
            a64 = fma(x, x, a64);
            b64 = fma(y, y, b64);
          }
#pragma unroll
          for (int o = 1; o < LANES; o <<= 1) {
            g64 += __shfl_xor_sync(0xffffffffu, g64, o);
            a64 += __shfl_xor_sync(0xffffffffu, a64, o);
            b64 += __shfl_xor_sync(0xffffffffu, b64, o);
          }
          if (amb) {
            doit = fabs(g64) > (double)kTol * sqrt(a64 * b64);
            if (it.live && q == 0) atomicAdd(d.counters + 2, 1ull);
          }
        }
        if (doit) {
          unconverged = true;
          const float dd = be - al;
          const float rr = sqrtf(fmaf(dd, dd, 4.f * gv * gv));
          const float tt = __fdividef(copysignf(2.f * gv, dd == 0.f ? 1.f : dd), fabsf(dd) + rr);
          const float cs = rsqrtf(fmaf(tt, tt, 1.f));
          const float sn = cs * tt;
#pragma unroll
          for (int r = 0; r < RPL; ++r) {
            const float a = A[r][pi], b = A[r][pj];
            A[r][pi] = fmaf(cs, a, -sn * b);
            A[r][pj] = fmaf(sn, a, cs * b);
          }
          nrm[pi] = fmaf(-tt, gv, al);
          nrm[pj] = fmaf(tt, gv, be);
        }
      }
    }
    if (!__any_sync(0xffffffffu, unconverged)) break;
  }
  if (lane == 0) atomicAdd(d.counters + 1, (unsigned long long)(sweeps + 1));  // per warp

  // ---- epilogue: norms, order, U, V = B^T U S^-1, projections h
  extern __shared__ float smem[];
  float* As = smem + (size_t)warp_in_blk * (GROUPS * NC * MP + GROUPS * NC);
  float* Ss = As + GROUPS * NC * MP;
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    float s = 0.f;
#pragma unroll
    for (int r = 0; r < RPL; ++r) {
      s = fmaf(A[r][k], A[r][k], s);
      As[(grp * NC + k) * MP + q * RPL + r] = A[r][k];
    }
#pragma unroll
    for (int o = 1; o < LANES; o <<= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (q == 0) Ss[grp * NC + k] = sqrtf(s);
  }
  __syncwarp();
  if (!it.live) return;
  const float* fld = (it.c == 0) ? d.fld0 : (it.c == 3 ? d.fld1 : d.fld2);
  const float* fw_ = fld ? fld + (size_t)it.w * g.cube() : nullptr;
  const size_t NP = g.NP;
  const size_t wbase = (size_t)it.w;
  for (int i = q; i < NC; i += LANES) {
    const float s = Ss[grp * NC + i];
    int rank = 0;
    for (int jj = 0; jj < NC; ++jj) {
      const float t = Ss[grp * NC + jj];
      rank += (t > s) || (t == s && jj < i);
    }
    const float* a = As + (grp * NC + i) * MP;
    const float inv = s > 0.f ? 1.f / s : 0.f;
    float h = 0.f;
    for (int k = 0; k < g.nwin; ++k) {
      const uint32_t pc = __ldg(posw + (size_t)k * g.P + posidx);
      const int y = pc & 0xffffu, x = pc >> 16;
      float bu = 0.f, gu = 0.f;
      for (int e = 0; e < g.M; ++e) {
        const size_t kidx = (size_t)k * F + (y + e % g.bs) + (size_t)(x + e / g.bs) * g.S;
        const float ue = a[e] * inv;
        bu = fmaf(perturbed(d, wc, it.c, uw, kidx, poff), ue, bu);
        if (fw_) gu = fmaf(__ldg(fw_ + kidx), ue, gu);
      }
      const float vk = bu * inv;
      h = fmaf(vk, gu, h);
      if (it.c == 0) d.V0[((wbase * NC + rank) * g.nwin + k) * NP + it.p] = vk;
    }
    if (it.c == 0)
      for (int e = 0; e < g.M; ++e) d.U0[((wbase * NC + rank) * g.M + e) * NP + it.p] = a[e] * inv;
    const int cslot = it.c == 3 ? 3 : it.c;
    d.sv[((wbase * 4 + cslot) * NC + rank) * NP + it.p] = s;
    d.hv[((wbase * 4 + cslot) * NC + rank) * NP + it.p] = h;
  }
}

template <int RPL, int LANES, int NC>
cudaError_t run_svd(const Problem& pb, const DeviceBuffers& d, cudaStream_t s) {
  constexpr int GROUPS = 32 / LANES, MP = RPL * LANES;
  const int nitems = pb.W * d.ncopies * pb.g.NP;
  const int warps = (nitems + GROUPS - 1) / GROUPS;
  const int wpb = 4;
  const size_t shm = (size_t)wpb * (GROUPS * NC * MP + GROUPS * NC) * sizeof(float);
  k_svd<RPL, LANES, NC><<<(warps + wpb - 1) / wpb, wpb * 32, shm, s>>>(pb, d, nitems);
  return cudaGetLastError();
}

}  // namespace svdk
}  // namespace pgsvt

#define PGSVT_INSTANTIATE_SVD(RPL, LANES, NC) \
  template cudaError_t pgsvt::svdk::run_svd<RPL, LANES, NC>(const pgsvt::Problem&, \
                                                          const pgsvt::DeviceBuffers&, cudaStream_t);

#endif
