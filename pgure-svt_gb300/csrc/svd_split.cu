// svd_split.cu — SVD forms that run as several kernels, each with a small
// code footprint (one kernel holding all phases thrashed the instruction
// cache) and its own register budget:
//
// QR-preconditioned form, Casorati matrices of 17..64 rows (patch sides
// 5..8) and windows of up to 15 frames.  A one-sided Jacobi sweep costs work
// proportional to the rows of the matrix it orthogonalises.  For an m x n
// Casorati matrix B with m > n the kernels first reduce B to the n x n
// triangle R of its Householder QR factorisation (B = Q R), then run the
// Jacobi sweeps on X = R^T, whose rotated columns X W = U_X S give the right
// singular vectors of B directly (R = W S U_X^T, so B = (Q W) S U_X^T):
// v_t = U_X e_t, and the left ones follow from B itself, u_t = B v_t / s_t.
// Q and W are never formed.
//   k_qr      16 lanes per patch: B staged in shared memory, Householder
//             reflections in a runtime loop; X = R^T to a scratch array
//   k_xsweep  4 lanes x (NC/4) rows per patch, eight patches per warp: the
//             register-form Jacobi sweeps of svd_kernel.cuh (same rotations,
//             same convergence rules) on X; rotated columns and their norms
//             back to the scratch
//   k_qr_out  16 lanes x 4 rows per patch: u_t = B v_t / s_t, the stored
//             factors and the risk projections h_t = u_t^T G v_t.
//
// Two-kernel register form, at most 16 rows and windows of up to 15 frames
// (the default for patch sides 2..4): k_bsweep runs the register form's
// sweeps on B at four resident blocks per SM, k_bout the factors, exactly as
// the single-kernel form computes them.
#include <cuda.h>

#include <cstring>

#include "svd_kernel.cuh"

namespace pgsvt {
namespace svdk {

// Tensor maps of the factors kernel's staged tiles: the normalised windows,
// the risk fields of copies 0 and 1/2, and the probe codes of copies 1/2.
struct BoutMaps {
  CUtensorMap u, f0, f2, d2;
};

namespace {

constexpr int kQL = 16;  // lanes per patch in the QR and the epilogue
constexpr int kQR = 4;   // rows per lane there

template <int NC>
struct QrDims {
  static constexpr int RX = (NC + 3) / 4;  // rows of X per lane in the sweeps
  static constexpr int XR = 4 * RX;        // rows of X (NC rounded up to 4)
  static constexpr int CS = XR + 1;        // column stride of X staged in shared memory
  static constexpr int MS = 68;            // column stride of B in shared memory (64 rows)
};

// One patch's source: window, trajectory and the perturbation of its copy.
struct PatchSrc {
  const float* uw;
  const uint32_t* posw;
  const int8_t* d1;
  const int8_t* d2code;
  size_t poff, F;
  int posidx, P, S, c;
  float pa, pb0;
  __device__ void init(const Problem& pb, const DeviceBuffers& d, int p, int c_, int w) {
    const Geometry& g = pb.g;
    const WinConst& wc = d.wc[w];
    F = g.F();
    P = g.P;
    S = g.S;
    c = c_;
    uw = d.u + (size_t)w * g.cube();
    posidx = d.plist[p];
    posw = d.pos + (size_t)w * g.nwin * g.P;
    poff = (size_t)w * d.probe_stride;
    d1 = d.d1;
    d2code = d.d2code;
    pa = pb0 = 0.f;
    if (c == 1 || c == 2) {  // pgure.hpp:80-82
      const double sg = (c == 1) ? 1.0 : -1.0;
      pa = (float)(sg * d.d2neg * wc.eps2);
      pb0 = (float)(sg * d.d2pos * wc.eps2);
    } else if (c == 3) {
      pa = (float)wc.eps1;
    }
  }
  __device__ size_t base(int k) const {  // slice k of the trajectory
    const uint32_t pc = __ldg(posw + (size_t)k * P + posidx);
    return (size_t)k * F + (pc & 0xffffu) + (size_t)(pc >> 16) * S;
  }
  __device__ float value(size_t kidx) const {
    float v = __ldg(uw + kidx);
    if (c == 1 || c == 2) v += __ldg(d2code + poff + kidx) ? pa : pb0;
    else if (c == 3) v += (float)__ldg(d1 + poff + kidx) * pa;
    return v;
  }
};

__device__ __forceinline__ float half_sum(float v) {  // over the 16 lanes of a half-warp
#pragma unroll
  for (int o = 1; o < kQL; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---- TMA staging of frame tiles (k_bout<NC, true>)
//
// The 32 patches of a factors block are 8 x 4 neighbouring grid positions
// (the tile order of the kept patches), so in every slice of the window their
// trajectory positions fall in a small box.  One thread of the block loads,
// per slice, a tile of the normalised window, of the risk field and of the
// probe codes around that box with cp.async.bulk.tensor into the block's own
// shared memory (one mbarrier, bounded wait); the lanes then assemble their
// Casorati rows from shared memory.  Slices whose box does not fit a tile,
// and blocks that straddle two windows or copies, read global memory as the
// unstaged kernel does.  The tensor maps cover this device's buffers only.
constexpr int kTR = 24, kTC = 12;  // fp32 tile: rows (inner, 96 bytes) x columns
constexpr int kTRP = 32;           // probe-code tile rows (uint8, 32 bytes)
constexpr int kTile = kTR * kTC, kPTile = kTRP * kTC;
constexpr unsigned kSpinPolls = 1u << 22;  // bounded mbarrier polls

__device__ __forceinline__ uint32_t smem_addr(const void* ptr) {
  return (uint32_t)__cvta_generic_to_shared(ptr);
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (unsigned it = 0; it < kSpinPolls; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void tma_tile3(uint32_t dst, const CUtensorMap* map, int x, int y, int z,
                                          uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];"
      :: "r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

// ---- Householder QR of every patch's Casorati matrix, X = R^T to xq
// ([item][NC][XR]; column k of X = row k of R).  B in shared memory, one
// reflection per column in a runtime loop, four rows per lane.
template <int NC>
__global__ void __launch_bounds__(128) k_qr(Problem pb, DeviceBuffers d, int nitems) {
  using D = QrDims<NC>;
  const Geometry& g = pb.g;
  const int lane = threadIdx.x & 31, l16 = lane & (kQL - 1);
  const int slot = threadIdx.x >> 4;  // patch of the block (8 per block)
  const int gid = blockIdx.x * 8 + slot;
  const bool live = gid < nitems;
  const int nwin = g.nwin, M = g.M;
  __shared__ __align__(16) float Bs[8][NC * D::MS];
  float* B = Bs[slot];
  int p, c, w;
  {
    const int gg = live ? gid : 0;
    p = gg % g.NP;
    const int r = gg / g.NP;
    c = r % d.ncopies;
    w = r / d.ncopies;
  }
  PatchSrc src;
  src.init(pb, d, p, c, w);
  // gather B (svt.hpp:101-109): rows l16*4 .. +3 of every column
  for (int k = 0; k < NC; ++k) {
    const bool colok = live && k < nwin;
    const size_t b = colok ? src.base(k) : 0;
    float4 v;
    float* vp = &v.x;
#pragma unroll
    for (int r = 0; r < kQR; ++r) {
      const int e = l16 * kQR + r;
      vp[r] = (colok && e < M) ? src.value(b + (e % g.bs) + (size_t)(e / g.bs) * g.S) : 0.f;
    }
    *reinterpret_cast<float4*>(B + k * D::MS + l16 * kQR) = v;
  }
  __syncwarp();
  const int r0 = l16 * kQR;
  for (int jj = 0; jj < nwin; ++jj) {
    const float4 x4 = *reinterpret_cast<const float4*>(B + jj * D::MS + r0);
    const float* xp = &x4.x;
    float ss = 0.f;  // |rows >= jj of column jj|^2
#pragma unroll
    for (int r = 0; r < kQR; ++r)
      if (r0 + r >= jj) ss = fmaf(xp[r], xp[r], ss);
    ss = half_sum(ss);
    const float xj = B[jj * D::MS + jj];
    const float alpha = xj >= 0.f ? -sqrtf(ss) : sqrtf(ss);
    const float vtv = 2.f * (ss - xj * alpha);  // |x - alpha e_jj|^2
    const float beta = vtv > 0.f ? 2.f / vtv : 0.f;
    float v[kQR];
#pragma unroll
    for (int r = 0; r < kQR; ++r) {
      const int e = r0 + r;
      v[r] = e > jj ? xp[r] : (e == jj ? xj - alpha : 0.f);
    }
#pragma unroll 4
    for (int kk = jj + 1; kk < nwin; ++kk) {
      float4 b4 = *reinterpret_cast<const float4*>(B + kk * D::MS + r0);
      float* bp = &b4.x;
      float t = 0.f;
#pragma unroll
      for (int r = 0; r < kQR; ++r) t = fmaf(v[r], bp[r], t);
      const float f = beta * half_sum(t);
#pragma unroll
      for (int r = 0; r < kQR; ++r) bp[r] = fmaf(-f, v[r], bp[r]);
      *reinterpret_cast<float4*>(B + kk * D::MS + r0) = b4;
    }
    __syncwarp();
    float4 o4 = x4;
    float* op = &o4.x;
#pragma unroll
    for (int r = 0; r < kQR; ++r) {
      const int e = r0 + r;
      if (e == jj) op[r] = alpha;
      else if (e > jj) op[r] = 0.f;
    }
    *reinterpret_cast<float4*>(B + jj * D::MS + r0) = o4;
    __syncwarp();
  }
  // X column k = row k of R (rows >= nwin of R are zero)
  if (live && l16 < NC) {
    float* xo = d.xq + ((size_t)gid * NC + l16) * D::XR;
#pragma unroll
    for (int j = 0; j < D::XR; j += 4) {
      float4 t;
      t.x = j + 0 < NC ? B[(j + 0) * D::MS + l16] : 0.f;
      t.y = j + 1 < NC ? B[(j + 1) * D::MS + l16] : 0.f;
      t.z = j + 2 < NC ? B[(j + 2) * D::MS + l16] : 0.f;
      t.w = j + 3 < NC ? B[(j + 3) * D::MS + l16] : 0.f;
      *reinterpret_cast<float4*>(xo + j) = t;
    }
  }
}

// ---- Jacobi sweeps on X, four lanes per patch, eight patches per warp
template <int NC>
__global__ void __launch_bounds__(128, 4) k_xsweep(Problem pb, DeviceBuffers d, int nitems) {
  using D = QrDims<NC>;
  constexpr int RX = D::RX, CS = D::CS;
  const int lane = threadIdx.x & 31, q = lane & 3;
  const int slot = threadIdx.x >> 2;  // patch of the block (32 per block)
  const int gid = blockIdx.x * 32 + slot;
  const bool live = gid < nitems;
  __shared__ float Xs[32][NC * CS];
  float* X = Xs[slot];
  const float* xi = d.xq + (size_t)(live ? gid : 0) * NC * D::XR;
  RegCols<RX, NC> A;
#pragma unroll
  for (int k = 0; k < NC; ++k)
#pragma unroll
    for (int r = 0; r < RX; ++r) A(r, k) = live ? __ldg(xi + k * D::XR + q * RX + r) : 0.f;
  unsigned fp64_tests = 0;
  const int sweeps = register_sweeps<RX, 4, NC, CS, 1>(A, X, q, pb.g.nwin, fp64_tests);
  if (lane == 0) atomicAdd(d.counters + 1, (unsigned long long)(sweeps + 1));
  if (q == 0 && fp64_tests) atomicAdd(d.counters + 2, (unsigned long long)fp64_tests);
  // column norms (the singular values), then the rotated columns of those
  // triplets that can survive the threshold (the only ones k_qr_out reads)
  float sv[NC];
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    float t = 0.f;
#pragma unroll
    for (int r = 0; r < RX; ++r) t = fmaf(A(r, k), A(r, k), t);
    sv[k] = sqrtf(lanes_sum<4>(t));  // every lane takes part
  }
  if (!live) return;
  float smax = sv[0];
#pragma unroll
  for (int k = 1; k < NC; ++k) smax = fmaxf(smax, sv[k]);
  const float upper = (float)d.wc[(gid / pb.g.NP) / d.ncopies].upper;
  float* xo = d.xq + (size_t)gid * NC * D::XR;
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    if (q == 0) d.xqn[(size_t)gid * NC + k] = sv[k];
    if (can_survive(pb, sv[k], smax, upper))
#pragma unroll
      for (int r = 0; r < RX; ++r) xo[k * D::XR + q * RX + r] = A(r, k);
  }
}

// ---- the factors: u_t = B v_t / s_t, h_t = u_t^T G v_t, sorted by s
template <int NC>
__global__ void __launch_bounds__(128) k_qr_out(Problem pb, DeviceBuffers d, int nitems) {
  using D = QrDims<NC>;
  const Geometry& g = pb.g;
  const int lane = threadIdx.x & 31, l16 = lane & (kQL - 1);
  const int gid = blockIdx.x * 8 + (threadIdx.x >> 4);
  const bool live = gid < nitems;
  const int nwin = g.nwin, M = g.M;
  int p, c, w;
  {
    const int gg = live ? gid : 0;
    p = gg % g.NP;
    const int r = gg / g.NP;
    c = r % d.ncopies;
    w = r / d.ncopies;
  }
  const WinConst& wc = d.wc[w];
  const float* X = d.xq + (size_t)(live ? gid : 0) * NC * D::XR;
  int roff[kQR];
#pragma unroll
  for (int r = 0; r < kQR; ++r) {
    const int e = l16 * kQR + r;
    roff[r] = e < M ? (e % g.bs) + (e / g.bs) * g.S : -1;
  }
  float sv[NC];
#pragma unroll
  for (int k = 0; k < NC; ++k) sv[k] = live ? __ldg(d.xqn + (size_t)gid * NC + k) : 0.f;
  float smax = sv[0];
#pragma unroll
  for (int k = 1; k < NC; ++k) smax = fmaxf(smax, sv[k]);
  const size_t NP = g.NP;
  const int NCg = g.NC;
  float* svo = d.sv + (((size_t)w * 4 + c) * NCg) * NP + p;
  float* hvo = d.hv + (((size_t)w * 4 + c) * NCg) * NP + p;
  int nl = 0;
#pragma unroll
  for (int k = 0; k < NC; ++k) nl += can_survive(pb, sv[k], smax, (float)wc.upper);
  int nl_max = nl;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) nl_max = max(nl_max, __shfl_xor_sync(0xffffffffu, nl_max, o));
  if (c == 0 && live && l16 == 0) d.nlive0[(size_t)w * NP + p] = nl;
  const float* fld = (c == 0) ? d.fld0 : (c == 3 ? d.fld1 : d.fld2);
  const float* fw_ = (pb.optimize && fld) ? fld + (size_t)w * g.cube() : nullptr;
  PatchSrc src;
  src.init(pb, d, p, c, w);
  float B[kQR][NC];
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    const bool colok = live && k < nwin && nl_max > 0;
    const size_t b = colok ? src.base(k) : 0;
#pragma unroll
    for (int r = 0; r < kQR; ++r)
      B[r][k] = (colok && roff[r] >= 0) ? src.value(b + roff[r]) : 0.f;
  }
  int prev = -1;
  float prev_s = INFINITY;
  for (int t = 0; t < NC; ++t) {
    // next column in decreasing singular-value order (ties by index)
    int ct = 0;
    float st = -1.f;
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      const float sk = sv[k];
      const bool after = (sk < prev_s) || (sk == prev_s && k > prev);
      if (after && (sk > st)) {
        st = sk;
        ct = k;
      }
    }
    prev = ct;
    prev_s = st;
    const bool use = t < nl;
    if (live && l16 == 0) {
      svo[(size_t)t * NP] = st;
      if (!use) hvo[(size_t)t * NP] = 0.f;
    }
    if (t >= nl_max) continue;  // warp-uniform
    const float inv = st > 0.f ? 1.f / st : 0.f;
    const float* xc = X + ct * D::XR;  // v_t = X's rotated column ct times inv
    float a[kQR];                      // u_t rows
#pragma unroll
    for (int r = 0; r < kQR; ++r) a[r] = 0.f;
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      const float vk = (live && k < nwin) ? __ldg(xc + k) * inv : 0.f;
#pragma unroll
      for (int r = 0; r < kQR; ++r) a[r] = fmaf(B[r][k], vk, a[r]);
    }
#pragma unroll
    for (int r = 0; r < kQR; ++r) a[r] *= inv;
    if (c == 0 && live && use && d.U0 && d.V0) {
#pragma unroll
      for (int r = 0; r < kQR; ++r)
        if (roff[r] >= 0) d.U0[(((size_t)w * NCg + t) * g.M + l16 * kQR + r) * NP + p] = a[r];
      if (l16 < nwin)
        d.V0[(((size_t)w * NCg + t) * nwin + l16) * NP + p] = __ldg(xc + l16) * inv;
    }
    if (fw_) {
      // h_t = sum_k v_k (G_k . u_t): the lanes' partial sums, one reduction
      float h = 0.f;
      if (live && use) {
#pragma unroll
        for (int k = 0; k < NC; ++k) {
          if (k >= nwin) break;
          const size_t b = src.base(k);
          float gu = 0.f;
#pragma unroll
          for (int r = 0; r < kQR; ++r)
            if (roff[r] >= 0) gu = fmaf(__ldg(fw_ + b + roff[r]), a[r], gu);
          h = fmaf(__ldg(xc + k) * inv, gu, h);
        }
      }
      h = half_sum(h);
      if (live && use && l16 == 0) hvo[(size_t)t * NP] = h;
    }
  }
}

// ---- the same two-kernel split without the QR, for patches of at most 16
// rows (sides 2..4): the sweeps on B itself at four resident blocks per SM,
// then the factors from the rotated columns (u_t = a_t / s_t, v_t = B^T u_t
// / s_t), exactly as the single-kernel register form computes them: the same
// operations in the same order, so the results are identical to it.
template <int NC>
__global__ void __launch_bounds__(128, 4) k_bsweep(Problem pb, DeviceBuffers d, int nitems) {
  constexpr int RX = 4, XR = 16, CS = XR + 1;
  const Geometry& g = pb.g;
  const int lane = threadIdx.x & 31, q = lane & 3;
  const int slot = threadIdx.x >> 2;  // patch of the block (32 per block)
  const int gid = blockIdx.x * 32 + slot;
  const bool live = gid < nitems;
  const int nwin = g.nwin, M = g.M;
  __shared__ float Xs[32][NC * CS];
  float* X = Xs[slot];
  int p, c, w;
  {
    const int gg = live ? gid : 0;
    p = gg % g.NP;
    const int r = gg / g.NP;
    c = r % d.ncopies;
    w = r / d.ncopies;
  }
  PatchSrc src;
  src.init(pb, d, p, c, w);
  int roff[RX];
#pragma unroll
  for (int r = 0; r < RX; ++r) {
    const int e = q * RX + r;
    roff[r] = (live && e < M) ? (e % g.bs) + (e / g.bs) * g.S : -1;
  }
  RegCols<RX, NC> A;
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    const bool colok = live && k < nwin;
    const size_t b = colok ? src.base(k) : 0;
#pragma unroll
    for (int r = 0; r < RX; ++r) A(r, k) = (colok && roff[r] >= 0) ? src.value(b + roff[r]) : 0.f;
  }
  unsigned fp64_tests = 0;
  const int sweeps = register_sweeps<RX, 4, NC, CS, 1>(A, X, q, nwin, fp64_tests);
  if (lane == 0) atomicAdd(d.counters + 1, (unsigned long long)(sweeps + 1));
  if (q == 0 && fp64_tests) atomicAdd(d.counters + 2, (unsigned long long)fp64_tests);
  // column norms (the singular values), then the rotated columns of those
  // triplets that can survive the threshold (the only ones k_bout reads)
  float sv[NC];
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    float t = 0.f;
#pragma unroll
    for (int r = 0; r < RX; ++r) t = fmaf(A(r, k), A(r, k), t);
    sv[k] = sqrtf(lanes_sum<4>(t));  // every lane takes part
  }
  if (!live) return;
  float smax = sv[0];
#pragma unroll
  for (int k = 1; k < NC; ++k) smax = fmaxf(smax, sv[k]);
  const float upper = (float)d.wc[w].upper;
  float* xo = d.xq + (size_t)gid * NC * XR;
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    if (q == 0) d.xqn[(size_t)gid * NC + k] = sv[k];
    if (can_survive(pb, sv[k], smax, upper))
#pragma unroll
      for (int r = 0; r < RX; ++r) xo[k * XR + q * RX + r] = A(r, k);
  }
}

template <int NC, bool TMA>
__global__ void __launch_bounds__(128, 4)
    k_bout(Problem pb, DeviceBuffers d, int nitems, const __grid_constant__ BoutMaps tm) {
  constexpr int RX = 4, XR = 16;
  const Geometry& g = pb.g;
  const int lane = threadIdx.x & 31, q = lane & 3;
  const int gid = blockIdx.x * 32 + (threadIdx.x >> 2);
  const bool live = gid < nitems;
  const int nwin = g.nwin, M = g.M;
  int p, c, w;
  {
    const int gg = live ? gid : 0;
    p = gg % g.NP;
    const int r = gg / g.NP;
    c = r % d.ncopies;
    w = r / d.ncopies;
  }
  const WinConst& wc = d.wc[w];
  const float* X = d.xq + (size_t)(live ? gid : 0) * NC * XR;
  int roff[RX];
#pragma unroll
  for (int r = 0; r < RX; ++r) {
    const int e = q * RX + r;
    roff[r] = (live && e < M) ? (e % g.bs) + (e / g.bs) * g.S : -1;
  }
  float sv[NC];
#pragma unroll
  for (int k = 0; k < NC; ++k) sv[k] = live ? __ldg(d.xqn + (size_t)gid * NC + k) : 0.f;
  float smax = sv[0];
#pragma unroll
  for (int k = 1; k < NC; ++k) smax = fmaxf(smax, sv[k]);
  const size_t NP = g.NP;
  const int NCg = g.NC;
  float* svo = d.sv + (((size_t)w * 4 + c) * NCg) * NP + p;
  float* hvo = d.hv + (((size_t)w * 4 + c) * NCg) * NP + p;
  int nl = 0;
#pragma unroll
  for (int k = 0; k < NC; ++k) nl += can_survive(pb, sv[k], smax, (float)wc.upper);
  int nl_max = nl;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) nl_max = max(nl_max, __shfl_xor_sync(0xffffffffu, nl_max, o));
  if (c == 0 && live && q == 0) d.nlive0[(size_t)w * NP + p] = nl;
  const float* fld = (c == 0) ? d.fld0 : (c == 3 ? d.fld1 : d.fld2);
  const float* fw_ = (pb.optimize && fld) ? fld + (size_t)w * g.cube() : nullptr;
  PatchSrc src;
  src.init(pb, d, p, c, w);
  // B again and, in shared memory, this lane's rows of the field G along the
  // trajectory (each lane reads back only what it wrote)
  float B[RX][NC];
  float* gs;
  if constexpr (!TMA) {
    __shared__ __align__(16) float Gs[32][NC][4 * RX];
    gs = &Gs[threadIdx.x >> 2][0][q * RX];
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      const bool colok = live && k < nwin && nl_max > 0;
      const size_t b = colok ? src.base(k) : 0;
#pragma unroll
      for (int r = 0; r < RX; ++r) B[r][k] = (colok && roff[r] >= 0) ? src.value(b + roff[r]) : 0.f;
      if (fw_) {
        float4 g4 = make_float4(0.f, 0.f, 0.f, 0.f);
        float* gp = &g4.x;
#pragma unroll
        for (int r = 0; r < RX; ++r)
          if (colok && roff[r] >= 0) gp[r] = __ldg(fw_ + b + roff[r]);
        *reinterpret_cast<float4*>(gs + k * 4 * RX) = g4;
      }
    }
  } else {
    // dynamic shared memory: [Gs (padded rows) | field tiles]; the window
    // and probe tiles share the Gs region, which is written only after
    // every lane has assembled B
    constexpr int GSS = NC * 4 * RX + 16;  // Gs floats per patch (+16: no bank conflicts)
    constexpr int GS_BYTES = 32 * GSS * 4;
    static_assert(NC * (kTile * 4 + kPTile) <= GS_BYTES, "window tiles must fit the Gs region");
    extern __shared__ unsigned char dyn_smem[];
    unsigned char* sbase = (unsigned char*)(((uintptr_t)dyn_smem + 127) & ~(uintptr_t)127);
    float* gsm = (float*)sbase;
    float* ut = (float*)sbase;
    uint8_t* ptl = sbase + NC * kTile * 4;
    float* ftl = (float*)(sbase + GS_BYTES);
    __shared__ __align__(8) unsigned long long bar;
    __shared__ int fymin[NC], fymax[NC], fxmin[NC], fxmax[NC], fy0[NC], fyp0[NC], fx0[NC];
    __shared__ int cta_ok;
    const int tid = threadIdx.x;
    const uint32_t bara = smem_addr(&bar);
    const bool probes = (c == 1 || c == 2);
    if (tid < NC) {
      fymin[tid] = fxmin[tid] = 0x7fffffff;
      fymax[tid] = fxmax[tid] = -1;
    }
    if (tid == 0) {
      const int g0 = blockIdx.x * 32, g1 = min(nitems, g0 + 32) - 1;
      const int r0 = g0 / g.NP, r1 = g1 / g.NP;  // (window, copy) of the first and last item
      cta_ok = (r0 == r1) && (r0 % d.ncopies) <= 2;
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(bara), "r"(1) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // trajectory position of slice k of this patch (row | col << 16)
    auto posk = [&](int k) -> uint32_t {
      return (live && k < nwin) ? __ldg(src.posw + (size_t)k * src.P + src.posidx) : 0u;
    };
    if (cta_ok) {
#pragma unroll 1
      for (int k = 0; k < nwin; ++k) {
        const uint32_t pc = posk(k);
        const int y = (int)(pc & 0xffffu), x = (int)(pc >> 16);
        const int ylo = __reduce_min_sync(0xffffffffu, live ? y : 0x7fffffff);
        const int yhi = __reduce_max_sync(0xffffffffu, live ? y : -1);
        const int xlo = __reduce_min_sync(0xffffffffu, live ? x : 0x7fffffff);
        const int xhi = __reduce_max_sync(0xffffffffu, live ? x : -1);
        if (lane == 0) {
          atomicMin(&fymin[k], ylo);
          atomicMax(&fymax[k], yhi);
          atomicMin(&fxmin[k], xlo);
          atomicMax(&fxmax[k], xhi);
        }
      }
    }
    __syncthreads();
    if (tid == 0) {
      unsigned bytes = 0;
      for (int k = 0; k < NC; ++k) {
        fy0[k] = -1;
        if (!cta_ok || k >= nwin || fymin[k] > fymax[k]) continue;
        const int y0 = fymin[k] & ~3, yp0 = fymin[k] & ~15, x0 = fxmin[k];
        bool fit = fymax[k] + g.bs - y0 <= kTR && fxmax[k] + g.bs - x0 <= kTC;
        if (probes) fit = fit && fymax[k] + g.bs - yp0 <= kTRP;
        if (!fit) continue;
        fy0[k] = y0;
        fyp0[k] = yp0;
        fx0[k] = x0;
        bytes += kTile * 4 + (fw_ ? kTile * 4 : 0) + (probes ? kPTile : 0);
      }
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                   :: "r"(bara), "r"(bytes) : "memory");
      const int zp = d.probe_stride ? w * nwin : 0;
      for (int k = 0; k < NC; ++k) {
        if (k >= nwin || fy0[k] < 0) continue;
        tma_tile3(smem_addr(ut + k * kTile), &tm.u, fy0[k], fx0[k], w * nwin + k, bara);
        if (fw_)
          tma_tile3(smem_addr(ftl + k * kTile), c == 0 ? &tm.f0 : &tm.f2, fy0[k], fx0[k],
                    w * nwin + k, bara);
        if (probes) tma_tile3(smem_addr(ptl + k * kPTile), &tm.d2, fyp0[k], fx0[k], zp + k, bara);
      }
    }
    __syncthreads();
    const bool ok = mbar_wait(bara, 0);
    if (__syncthreads_or(!ok)) {  // a copy did not land in time: report, drain, stop
      if (tid == 0) atomicAdd(d.counters + 4, 1ull);
      mbar_wait(bara, 0);
      return;
    }
    // tile offsets of this lane's rows (row e of the Casorati matrix is pixel
    // (e % bs, e / bs) of the patch)
    int toff[RX], poff[RX];
#pragma unroll
    for (int r = 0; r < RX; ++r) {
      const int e = q * RX + r;
      toff[r] = e % g.bs + (e / g.bs) * kTR;
      poff[r] = e % g.bs + (e / g.bs) * kTRP;
    }
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      const bool colok = live && k < nwin && nl_max > 0;
      const uint32_t pc = colok ? posk(k) : 0u;
      const int y = (int)(pc & 0xffffu), x = (int)(pc >> 16);
      if (colok && fy0[k] >= 0) {
        const float* ub = ut + k * kTile + (y - fy0[k]) + (x - fx0[k]) * kTR;
        const uint8_t* pbs = ptl + k * kPTile + (y - fyp0[k]) + (x - fx0[k]) * kTRP;
#pragma unroll
        for (int r = 0; r < RX; ++r) {
          float v = 0.f;
          if (roff[r] >= 0) {
            v = ub[toff[r]];
            if (probes) v += pbs[poff[r]] ? src.pa : src.pb0;
          }
          B[r][k] = v;
        }
      } else {
        const size_t b = colok ? (size_t)k * src.F + y + (size_t)x * src.S : 0;
#pragma unroll
        for (int r = 0; r < RX; ++r) B[r][k] = (colok && roff[r] >= 0) ? src.value(b + roff[r]) : 0.f;
      }
    }
    __syncthreads();  // the window and probe tiles are dead: Gs takes their place
    gs = gsm + (size_t)(threadIdx.x >> 2) * GSS + q * RX;
    if (fw_) {
#pragma unroll
      for (int k = 0; k < NC; ++k) {
        const bool colok = live && k < nwin && nl_max > 0;
        const uint32_t pc = colok ? posk(k) : 0u;
        const int y = (int)(pc & 0xffffu), x = (int)(pc >> 16);
        float4 g4 = make_float4(0.f, 0.f, 0.f, 0.f);
        float* gp = &g4.x;
        if (colok && fy0[k] >= 0) {
          const float* fb = ftl + k * kTile + (y - fy0[k]) + (x - fx0[k]) * kTR;
#pragma unroll
          for (int r = 0; r < RX; ++r)
            if (roff[r] >= 0) gp[r] = fb[toff[r]];
        } else if (colok) {
          const size_t b = (size_t)k * src.F + y + (size_t)x * src.S;
#pragma unroll
          for (int r = 0; r < RX; ++r)
            if (roff[r] >= 0) gp[r] = __ldg(fw_ + b + roff[r]);
        }
        *reinterpret_cast<float4*>(gs + k * 4 * RX) = g4;
      }
    }
  }
  int prev = -1;
  float prev_s = INFINITY;
  for (int t = 0; t < NC; ++t) {
    // next column in decreasing singular-value order (ties by index)
    int ct = 0;
    float st = -1.f;
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      const float sk = sv[k];
      const bool after = (sk < prev_s) || (sk == prev_s && k > prev);
      if (after && (sk > st)) {
        st = sk;
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
    float a[RX];  // u_t rows
#pragma unroll
    for (int r = 0; r < RX; ++r) a[r] = (live ? __ldg(X + ct * XR + q * RX + r) : 0.f) * inv;
    if (c == 0 && live && use && d.U0 && d.V0) {
#pragma unroll
      for (int r = 0; r < RX; ++r)
        if (roff[r] >= 0) d.U0[(((size_t)w * NCg + t) * g.M + q * RX + r) * NP + p] = a[r];
    }
    // v_t = B^T u_t / s_t and h_t = u_t^T G v_t = sum_k v_k (G_k . u_t)
    float h = 0.f;
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      if (k >= nwin) break;  // uniform: keeps B[][k] in registers
      float bu = 0.f;
#pragma unroll
      for (int r = 0; r < RX; ++r) bu = fmaf(B[r][k], a[r], bu);
      bu = lanes_sum<4>(bu);
      const float vk = bu * inv;
      if (c == 0 && live && use && (k % 4) == q && d.V0)
        d.V0[(((size_t)w * NCg + t) * nwin + k) * NP + p] = vk;
      if (fw_ && live && use) {
        const float4 g4 = *reinterpret_cast<const float4*>(gs + k * 4 * RX);
        const float* gp = &g4.x;
        float gu = 0.f;
#pragma unroll
        for (int r = 0; r < RX; ++r)
          if (roff[r] >= 0) gu = fmaf(gp[r], a[r], gu);
        h = fmaf(vk, gu, h);
      }
    }
    if (fw_) h = lanes_sum<4>(h);
    if (live && use && q == 0) hvo[(size_t)t * NP] = h;
  }
}

}  // namespace

template <int NC>
cudaError_t run_svd_qr(const Problem& pb, const DeviceBuffers& d, cudaStream_t s) {
  if (!d.xq || !d.xqn) return cudaErrorInvalidValue;
  const int nitems = pb.W * d.ncopies * pb.g.NP;
  k_qr<NC><<<(nitems + 7) / 8, 128, 0, s>>>(pb, d, nitems);
  k_xsweep<NC><<<(nitems + 31) / 32, 128, 0, s>>>(pb, d, nitems);
  k_qr_out<NC><<<(nitems + 7) / 8, 128, 0, s>>>(pb, d, nitems);
  return cudaGetLastError();
}

template cudaError_t run_svd_qr<10>(const Problem&, const DeviceBuffers&, cudaStream_t);
template cudaError_t run_svd_qr<16>(const Problem&, const DeviceBuffers&, cudaStream_t);

namespace {

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled through the runtime's driver entry point (no libcuda link)
EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess || q != cudaDriverEntryPointSuccess)
      return (EncodeTiledFn) nullptr;
    return (EncodeTiledFn)f;
  }();
  return fn;
}

// A 3-D map over `frames` column-major S x S frames (rows innermost) with a
// box of box_rows x box_cols x 1; a null buffer gives an unused zero map.
bool frame_map(CUtensorMap* m, CUtensorMapDataType dt, size_t esize, const void* base, int S,
               int frames, int box_rows, int box_cols) {
  std::memset(m, 0, sizeof(*m));
  if (!base) return true;
  const EncodeTiledFn enc = encode_tiled();
  if (!enc) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)S, (cuuint64_t)S, (cuuint64_t)frames};
  const cuuint64_t strides[2] = {(cuuint64_t)S * esize, (cuuint64_t)S * S * esize};
  const cuuint32_t box[3] = {(cuuint32_t)box_rows, (cuuint32_t)box_cols, 1};
  const cuuint32_t es[3] = {1, 1, 1};
  return enc(m, dt, 3, const_cast<void*>(base), dims, strides, box, es,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

template <int NC>
cudaError_t run_svd_split(const Problem& pb, const DeviceBuffers& d, cudaStream_t s, bool staged) {
  if (!d.xq || !d.xqn) return cudaErrorInvalidValue;
  const int nitems = pb.W * d.ncopies * pb.g.NP;
  const int S = pb.g.S, nwin = pb.g.nwin;
  k_bsweep<NC><<<(nitems + 31) / 32, 128, 0, s>>>(pb, d, nitems);
  // the factors from shared-memory tiles staged by TMA (when asked for and
  // every map's row stride is a multiple of 16 bytes), else from global
  // memory; the same values either way, so identical results
  BoutMaps tm;
  bool tma = staged && S % 16 == 0 && d.counters != nullptr;
  if (tma) {
    const int pframes = d.probe_stride ? pb.W * nwin : nwin;
    tma = frame_map(&tm.u, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, d.u, S, pb.W * nwin, kTR, kTC) &&
          frame_map(&tm.f0, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, pb.optimize ? d.fld0 : nullptr, S,
                    pb.W * nwin, kTR, kTC) &&
          frame_map(&tm.f2, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, pb.optimize ? d.fld2 : nullptr, S,
                    pb.W * nwin, kTR, kTC) &&
          frame_map(&tm.d2, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, d.ncopies > 1 ? d.d2code : nullptr,
                    S, pframes, kTRP, kTC);
  }
  if (tma) {
    constexpr int GSS = NC * 16 + 16;
    const size_t shm = (size_t)32 * GSS * 4 + (size_t)NC * kTile * 4 + 128;
    const cudaError_t e = cudaFuncSetAttribute(
        k_bout<NC, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
    if (e != cudaSuccess) return e;
    k_bout<NC, true><<<(nitems + 31) / 32, 128, shm, s>>>(pb, d, nitems, tm);
  } else {
    std::memset(&tm, 0, sizeof(tm));
    k_bout<NC, false><<<(nitems + 31) / 32, 128, 0, s>>>(pb, d, nitems, tm);
  }
  return cudaGetLastError();
}

template cudaError_t run_svd_split<10>(const Problem&, const DeviceBuffers&, cudaStream_t, bool);
template cudaError_t run_svd_split<16>(const Problem&, const DeviceBuffers&, cudaStream_t, bool);

}  // namespace svdk
}  // namespace pgsvt
