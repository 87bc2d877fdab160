// svd.cu — batched one-sided Jacobi SVD of the Casorati matrices.
//
// Reference: SVT::Decompose (svt.hpp:58-118) gathers, for every kept patch,
// the m x n Casorati matrix B (column k = the bs x bs patch of slice k at its
// trajectory position, column-major within the patch) and calls
// arma::svd_econ.  PGURE decomposes up to three more copies of the window
// (pgure.hpp:62-91): U +/- eps2*delta2 and, without the integer-delta1 quirk,
// U + eps1*delta1.
//
// GB300 mapping: one patch is held in the registers of LANES lanes, each lane
// owning RPL consecutive rows of all NC (even, >= n) columns; 32/LANES patches
// share a warp.  A sweep applies the NC-1 rounds of the round-robin ordering,
// each round NC/2 disjoint Hestenes rotations; the only cross-lane traffic is
// the butterfly sum of the column inner products.  Column norms are updated in
// closed form during a sweep and recomputed exactly at its start.  A pair is
// rotated when |a_i.a_j| > tol*|a_i||a_j|; for near-degenerate pairs close to
// the threshold the inner product is re-evaluated in FP64 (exact products of
// the FP32 entries) so that FP32 rounding cannot decide convergence.
//
// The epilogue needs no V accumulation: with u_i = a_i/s_i, the right vectors
// are v_i = B^T u_i / s_i from a fresh gather of B, and the risk projections
// h_i = u_i^T G v_i use the lambda-independent fields G (eval.cu).  Singular
// triplets are stored sorted by decreasing s.
#include "pgsvt_internal.h"

namespace pgsvt {
namespace svdk {
template <int RPL, int LANES, int NC, bool SM>
cudaError_t run_svd(const Problem& pb, const DeviceBuffers& d, cudaStream_t s);
template <int NC>
cudaError_t run_svd_qr(const Problem& pb, const DeviceBuffers& d, cudaStream_t s);
template <int NC>
cudaError_t run_svd_split(const Problem& pb, const DeviceBuffers& d, cudaStream_t s, bool tma);
}

int svd_columns(int nwin) {
  if (nwin <= 10) return 10;
  if (nwin <= 16) return 16;
  if (nwin <= 22) return 22;
  return 0;
}

bool svd_supported(int bs, int nwin) {
  // bs <= 4 clamps the window to bs*bs-1 <= 15 frames
  return bs >= 2 && bs <= 16 && svd_columns(nwin) > 0;
}

// Kernel forms: rows per lane x lanes per patch covers bs*bs rows; the
// instantiations live in svd_i*.cu / svd_s*.cu so that they compile in
// parallel.  Variant 0 is the default shape with the columns in registers
// (moved one position per round), variant 1 spreads a patch over more lanes
// (fewer registers per lane, more shuffles per inner product), variant 2 is the
// default shape with the columns in shared memory (addressed by the round's
// schedule, no moves), variant 3 holds 8 rows per lane in fewer lanes (the
// per-pair rotation arithmetic, replicated in every lane of a patch, is shared
// by twice the rows; 2 resident blocks per SM instead of 3), variant 4
// (patches of 17..64 rows, windows <= 15) sweeps the triangle of B's QR
// factorisation instead of B (svd_split.cu), variant 5 is the two-kernel
// register form with the factors kernel reading TMA-staged frame tiles
// (svd_split.cu; measured slower than variant 0's global-memory gather, so
// it is a candidate of the autotuner only).  For patches of at most 16 rows
// and windows of at most 15 frames variant 0 runs its sweeps and its factors
// in two kernels (svd_split.cu; the sweeps without the factors' registers fit
// four resident blocks per SM instead of three), with identical results,
// wherever the caller provides the scratch (not in the allocation-free entry).  Variants 0 and 2 apply the same
// rotations in the same order; all agree to FP32 rounding.  The autotuner
// (capi.cu) times them on the caller's data and keeps the fastest.
bool svd_variant_ok(int M, int NC, int v) {
  if (M > 64) return v == 0;  // patch sides 9..16: the shared-memory form only
  if (v == 0 || v == 2) return true;
  if (v == 1) return !(M > 16 && M <= 32);  // 5x5 patches have no variant 1
  if (v == 3) return NC <= 16 && (M <= 16 || M > 40);  // 8 x 2 and 8 x 8 lanes
  if (v == 4) return svd_qr_form(M, NC);                 // QR-preconditioned
  if (v == 5) return M <= 16 && NC <= 16;                // two-kernel form, TMA-staged factors
  return false;
}
bool svd_qr_form(int M, int NC) { return M > 16 && M <= 64 && NC <= 16; }
bool svd_split_scratch(int M, int NC) { return svd_qr_form(M, NC) || (M <= 16 && NC <= 16); }
// the untuned shape: the QR-preconditioned form for 7x7 and 8x8 patches
// (2.2x faster than their 64-row register form on 512^2 windows), else 0
int svd_default_variant(int M, int NC) { return (M > 40 && svd_qr_form(M, NC)) ? 4 : 0; }
int svd_variants(int M, int NC) {
  int n = 0;
  for (int v = 0; v < kSvdVariants; ++v) n += svd_variant_ok(M, NC, v);
  return n;
}

template <int RPL, int LANES, int NC>
cudaError_t run_pair(const Problem& pb, const DeviceBuffers& d, cudaStream_t s) {
  return pb.svd_variant == 2 ? svdk::run_svd<RPL, LANES, NC, true>(pb, d, s)
                             : svdk::run_svd<RPL, LANES, NC, false>(pb, d, s);
}

cudaError_t launch_svd(const Problem& pb, const DeviceBuffers& d, cudaStream_t s) {
  using namespace svdk;
  const int M = pb.g.M, NC = pb.g.NC;
  const bool alt = pb.svd_variant == 1;
  if (pb.svd_variant == 4 && M > 16 && M <= 64) {  // QR-preconditioned
    if (NC == 10) return run_svd_qr<10>(pb, d, s);
    if (NC == 16) return run_svd_qr<16>(pb, d, s);
  }
  if ((pb.svd_variant == 0 || pb.svd_variant == 5) && M <= 16 && d.xq && d.xqn) {
    // sweeps and factors in two kernels; variant 5 stages the factors' frame
    // tiles with TMA
    if (NC == 10) return run_svd_split<10>(pb, d, s, pb.svd_variant == 5);
    if (NC == 16) return run_svd_split<16>(pb, d, s, pb.svd_variant == 5);
  }
  if (pb.svd_variant == 3 && NC <= 16) {  // 8 rows per lane
    if (M <= 16) {
      if (NC == 10) return run_svd<8, 2, 10, false>(pb, d, s);
      if (NC == 16) return run_svd<8, 2, 16, false>(pb, d, s);
    } else if (M > 40 && M <= 64) {
      if (NC == 10) return run_svd<8, 8, 10, false>(pb, d, s);
      if (NC == 16) return run_svd<8, 8, 16, false>(pb, d, s);
    }
  }
  if (M <= 16) {  // bs 2..4
    if (alt) {
      if (NC == 10) return run_svd<2, 8, 10, false>(pb, d, s);
      if (NC == 16) return run_svd<2, 8, 16, false>(pb, d, s);
    }
    if (NC == 10) return run_pair<4, 4, 10>(pb, d, s);
    if (NC == 16) return run_pair<4, 4, 16>(pb, d, s);
  } else if (M <= 32) {  // bs 5
    if (NC == 10) return run_pair<4, 8, 10>(pb, d, s);
    if (NC == 16) return run_pair<4, 8, 16>(pb, d, s);
    if (NC == 22) return run_pair<4, 8, 22>(pb, d, s);
  } else if (M <= 40) {  // bs 6
    if (alt) {
      if (NC == 10) return run_svd<3, 16, 10, false>(pb, d, s);
      if (NC == 16) return run_svd<3, 16, 16, false>(pb, d, s);
      if (NC == 22) return run_svd<3, 16, 22, false>(pb, d, s);
    }
    if (NC == 10) return run_pair<5, 8, 10>(pb, d, s);
    if (NC == 16) return run_pair<5, 8, 16>(pb, d, s);
    if (NC == 22) return run_pair<5, 8, 22>(pb, d, s);
  } else if (M > 64) {  // bs 9..16: 8 rows x 32 lanes, columns in shared memory
    if (NC == 10) return run_svd<8, 32, 10, true>(pb, d, s);
    if (NC == 16) return run_svd<8, 32, 16, true>(pb, d, s);
    if (NC == 22) return run_svd<8, 32, 22, true>(pb, d, s);
  } else {  // bs 7, 8
    if (alt) {
      if (NC == 10) return run_svd<2, 32, 10, false>(pb, d, s);
      if (NC == 16) return run_svd<2, 32, 16, false>(pb, d, s);
      if (NC == 22) return run_svd<2, 32, 22, false>(pb, d, s);
    }
    if (NC == 10) return run_pair<4, 16, 10>(pb, d, s);
    if (NC == 16) return run_pair<4, 16, 16>(pb, d, s);
    if (NC == 22) return run_pair<4, 16, 22>(pb, d, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace pgsvt
