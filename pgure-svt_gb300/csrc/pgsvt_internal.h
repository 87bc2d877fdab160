// pgsvt_internal.h — device-side data layout and kernel launchers of libpgsvt.
//
// One "window" is the reference's per-output-frame work item
// (pguresvt.hpp:90-167): nwin = 2*fw+1 frames of an S x S sequence,
// normalised by their maximum.  Windows are processed in batches of W on one
// device; every buffer below holds W windows back to back.
//
// Layout in HBM (all column-major like the reference's Armadillo cubes):
//   xs      f32 [nimg][S*S]       the input sequence, converted once
//   x64     f64 [nimg][S*S]       only for f64 input: exact values for the
//                                 FP64 ARPS tie-break path
//   u       f32 [W][nwin][S*S]    normalised windows (u = x / umax)
//   pos     u32 [W][nwin][P]      trajectory table: row | col << 16, where
//                                 P = (S-bs+1)^2 ARPS positions (arps.hpp:42)
//   cnt     i32 [W][nwin][S*S]    patch coverage per voxel (svt.hpp:157-159)
//   fld0,2  f32 [W][nwin][S*S]    lambda-independent risk fields (see eval.cu)
//   U0      f32 [W][NC][M][NP]    left singular vectors of copy 0 (patch
//                                 fastest), columns sorted by singular value
//   V0      f32 [W][NC][N][NP]    right singular vectors of copy 0
//   sv,hv   f32 [W][4][NC][NP]    singular values and risk projections of
//                                 copies 0 (clean), 1 (+eps2*delta2),
//                                 2 (-eps2*delta2), 3 (+eps1*delta1)
//   acc     i32 [W][K][nwin][S*S] fixed-point (2^-20) scatter accumulators
//           (i64 at 2^-32 when a voxel can collect every patch)
// NP is the number of kept patches (svt.hpp:61-94), M = bs*bs, N = nwin,
// NC = N rounded up to the kernel's even column count.
#ifndef PGSVT_INTERNAL_H
#define PGSVT_INTERNAL_H

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <string>
#include <vector>

namespace pgsvt {

// Kept patches (svt.hpp:61-94): the row-major-looking index i*nyMbs + j of the
// first loop is reproduced as written, then the right and bottom edges are
// added and the set is sorted and made unique.  Every entry point builds its
// patch list here, so all of them keep the same patches in the same order.
inline std::vector<int32_t> kept_patches(int S, int bs, int ov) {
  const int64_t nMbs = S - bs;
  std::vector<int64_t> v;
  for (int64_t i = 0; i < 1 + nMbs; i += ov)
    for (int64_t j = 0; j < 1 + nMbs; j += ov) v.push_back(i * nMbs + j);
  for (int64_t i = 0; i < 1 + nMbs; i += ov) v.push_back((nMbs + 1) * i + nMbs);
  for (int64_t i = 0; i < 1 + nMbs; i += ov) v.push_back((nMbs + 1) * nMbs + i);
  std::sort(v.begin(), v.end());
  v.erase(std::unique(v.begin(), v.end()), v.end());
  return std::vector<int32_t>(v.begin(), v.end());
}

constexpr int kMaxK = 16;          // lambda values per evaluation round
constexpr int kMaxPts = 160;       // evaluated points kept per window
// The lambda search stops after a refinement round without progress only
// when the bracket around its best point is narrower than this fraction of
// the point (else it refines again, within its round and evaluation limits).
constexpr double kNarrowBracket = 0.25;
constexpr int kMaxMW = 15;         // motion window supported by ARPS
constexpr int kEvalPatches = 32;   // kept patches per lambda-evaluation block (8 x 4 half tile)
constexpr double kFixScale = 4294967296.0;  // 2^32 fixed-point scale

// round(v * 2^32) toward zero as an int64, with integer instructions only
// (float <-> 64-bit integer conversions run on the FP64 unit)
__device__ __forceinline__ long long fix32(float v) {
  const int b = __float_as_int(v);
  const int ex = ((b >> 23) & 0xff) - 127;
  if (ex < -33) return 0;  // |v| < 2^-33 (also +-0, denormals)
  const long long m = (long long)((b & 0x7fffff) | 0x800000);
  const int sh = ex + 9;   // v * 2^32 = m * 2^(ex - 23 + 32)
  const long long r = sh >= 0 ? (m << sh) : (m >> (-sh));
  return b < 0 ? -r : r;
}

// int64 fixed-point value (2^-32) to float, with 32-bit conversions only
__device__ __forceinline__ float unfix32(long long a) {
  const int hi = (int)(a >> 32);
  const unsigned lo = (unsigned)(a & 0xffffffffll);
  return (float)hi + (float)lo * 2.3283064365386963e-10f;
}

// Per-window constants, computed on the device.
struct WinConst {
  double umax;     // window maximum (pguresvt.hpp:116)
  double wnorm;    // maximum of the median-filtered window (ARPS input
                   // scale, pguresvt.hpp:117; 1 when it is 0)
  double unorm;    // divisor of the normalisation: umax, or 1 for an all-zero
                   // window (the reference's 0/0 ends as a zero output frame)
  double sum_u;    // accu(u)
  double alpha, mu, sigma;  // PGURE members (after the argument binding)
  double est_alpha, est_mu, est_sigma;  // caller-side values (estimates(t, 1..3))
  double eps1, eps2;
  double start, upper;      // lambda search start point / upper bound
  int32_t t;                // output frame index
  int32_t s0;               // first sequence frame of the window
  int32_t out_slice;        // window slice copied to the output
  int32_t ref;              // ARPS reference slice
};

// Search state of one window (device-resident, advanced by k_search_step).
// Phases: 0 = plain search, 1 = hinted search, 2 = plain search after a
// hint whose best point fell on the edge of its grid.
struct SearchState {
  double lam[kMaxPts];
  double risk[kMaxPts];
  double next[kMaxK];   // lambda values of the pending round
  double hint_lambda, hint_risk;
  double final_lambda, final_risk;
  double sent_risk;     // least risk of the narrow search's sentinel points
  int32_t nsent;        // sentinels at the end of the pending round's list
  int32_t npts, nnext, done, best;
  int32_t phase, K, max_eval, rounds, zero_lo, rd, evals_phase, evals_total, first;
};

// ARPS chain table: for each window, up to 2*fw chains of <=2 frame pairs
// (pairs sharing a motion slot, arps.hpp:121-130), executed in order.
struct ArpsChain {
  int8_t npairs;
  int8_t a1[2], a2[2];
};

struct Geometry {
  int S;        // frame side
  int bs;       // patch side
  int M;        // bs*bs
  int nwin;     // window length
  int fw;       // frame window
  int Ntc;      // clamped trajectory length (pguresvt.hpp:57)
  int P;        // ARPS positions
  int NP;       // kept patches
  int NC;       // padded column count of the SVD kernel
  int mw;       // motion window
  int nimg;
  __host__ __device__ size_t F() const { return (size_t)S * S; }
  __host__ __device__ size_t cube() const { return F() * nwin; }
};

struct Problem {
  Geometry g;
  int W;                 // windows in this batch
  int K;                 // lambda values per round
  int optimize, expw, motion, compat;
  double alpha_c, mu_c, sigma_c;  // caller-side noise parameters
  double lambda_user;
  double tol;
  int max_evals, rounds;
  double hint, hint_span;
  int hint_K, hint_rounds;  // narrow search: points per round, refinements
  double hint_flat;         // relative risk within which an edge best is kept
  int acc64;             // accumulators int64 at 2^-32 (else int32 at 2^-20)
  int svd_variant;       // kernel shape of the SVD (svd.cu)
  const double* fixed;   // device list of lambda values evaluated once per
  int nfixed;            // window instead of a search (null / 0: search)
  double* fixed_risk;    // optional out [nimg][nfixed], frame-major
};

struct DeviceBuffers {
  const float* xs;
  const double* x64;
  const double* fmax;      // per input frame maximum
  const float* zs;         // median-filtered sequence (null: no pre-filter)
  const double* zmax;      // its per-frame maxima
  float* wz;               // [W][nwin][S*S] ARPS input zs / wnorm
  double* w64;             // [W][nwin][S*S] the same in FP64 (the reference's values)
  int int_input;           // every input value an integer <= 2^19 (ARPS integer mode)
  float* u;
  uint32_t* pos;
  const int32_t* plist;    // kept patch -> position index
  int32_t* pidx;           // position -> kept patch index (-1 if not kept)
  int32_t* cnt;
  float* fld0;
  float* fld1;             // first-order field (only without the int-delta1 quirk)
  float* fld2;
  const int8_t* d1;        // probes, nwin*S*S per set
  const int8_t* d2code;    // 1 -> -sqrt(vQ/vP), 0 -> sqrt(vP/vQ)
  size_t probe_stride;     // 0: one set for all windows (seed >= 0), else per window
  double d2neg, d2pos;     // the two delta2 values (pgure.hpp:173-183)
  float* U0;
  float* V0;
  float* sv;
  float* hv;
  float* xq;               // split SVD forms' scratch: [items][NC][X rows] (svd_split.cu)
  float* xqn;              // its column norms [items][NC]
  int32_t* nlive0;         // [W][NP] singular triplets of copy 0 that can survive
  void* acc;               // [W][K][nwin][S*S] int32 or int64 fixed point
  double* part_lin;        // [W][K][nblk_eval]
  double* part_mse;        // [W][K][nblk_mse]
  WinConst* wc;
  SearchState* st;
  const ArpsChain* chains; // [W][2*fw]
  int nchains;
  double* Y;               // output [nimg][S*S] (double)
  double* est;             // output estimates (nimg x 4)
  unsigned long long* counters;  // [0] ARPS FP64 steps, [1] SVD warp-sweeps,
                                 // [2] FP64 convergence decisions, [3] risk
                                 // evaluations, [4] expired staged-copy waits
  // learned lambda proposal
  const int32_t* feat_slots;  // sampled kept-patch slots of the features
  int nfeat_slots;
  float* feat;             // [W][67] window features
  float* prop;             // [W] proposals y = log10(lambda/upper)
  const float* model;      // FP32 model (null: no proposal)
  const void* model_bf16;  // its bf16 shadow
  float* feat_out;         // optional per-frame outputs (device, frame-indexed)
  float* prop_out;
  double* risk_out;
  uint32_t* evals_out;
  int win0;                // first window (output frame) of this batch
  int ncopies;             // SVD copies decomposed (1, 3 or 4)
  int nblk_eval, nblk_mse;
};

// launchers (each returns cudaGetLastError())
cudaError_t launch_convert(const void* X, int dtype, size_t n, float* xs, double* x64,
                           cudaStream_t s);
cudaError_t launch_frame_max(const float* xs, const double* x64, int nimg, size_t F,
                             double* fmax, cudaStream_t s, int* fint = nullptr);
cudaError_t launch_median(const float* xs, const double* x64, int nimg, int S, int r, float* zs,
                          cudaStream_t s);
constexpr int kMaxMedian = 15;     // median pre-filter radius supported
cudaError_t launch_window_setup(const Problem& pb, const DeviceBuffers& d, cudaStream_t s);
cudaError_t launch_window_norm_only(const Problem& pb, const DeviceBuffers& d, cudaStream_t s);
cudaError_t launch_arps(const Problem& pb, const DeviceBuffers& d, cudaStream_t s);
cudaError_t launch_fields(const Problem& pb, const DeviceBuffers& d, cudaStream_t s);
cudaError_t launch_svd(const Problem& pb, const DeviceBuffers& d, cudaStream_t s);
cudaError_t launch_search_init(const Problem& pb, const DeviceBuffers& d, cudaStream_t s);
cudaError_t launch_eval_round(const Problem& pb, const DeviceBuffers& d, int final_pass,
                              cudaStream_t s);
cudaError_t launch_output(const Problem& pb, const DeviceBuffers& d, cudaStream_t s);
cudaError_t launch_cube_out(const Problem& pb, const DeviceBuffers& d, double* v,
                            cudaStream_t s);
cudaError_t launch_risk_round(const Problem& pb, const DeviceBuffers& d, double* out,
                              cudaStream_t s);

// noise estimation (noise.cu): per input frame ...
struct NoiseFrames {
  int nlev, maxNodes, maxBig;
  uint8_t* split;   // [nimg][blocks of side > 8] F-test decisions
  int4* nodes;      // [nimg][maxNodes] quadtree replay scratch
  uint8_t* isdel;   // [nimg][maxNodes]
  int4* leaf;       // [nimg][maxNodes] leaves (row, col, side) in the reference's order
  int* nleaf;       // [nimg]
  int* big;         // [nimg][maxNodes] indices of leaves of side > 32
  int* nbig;        // [nimg]
  double* stats;    // [nimg][maxNodes][3] (a_lo, a_hi, var), raw scale
  int* dup;         // [nimg][maxNodes] earlier leaf with the same block, or -1
  int* first;       // [nimg][blocks of side >= 8] scratch of the duplicate search
  int* err;         // replay overflow flag
};
// ... and the windows' estimates, before the denoising batches
struct NoisePass {
  int method, npairs, nwindows, nwin;
  double alpha_c, mu_c, sigma_c;  // caller values (< 0: estimate)
  const int* pair_frame;     // [npairs] frame of each (frame, window maximum) pair
  const double* pair_norm;   // [npairs] its window maximum
  double* mean;              // [npairs][maxNodes] robust leaf means (normalised)
  const int* win_pair;       // [nwindows][nwin] pair of each (window, slice)
  const int* win_s0;         // [nwindows] first frame
  const double* win_norm;    // [nwindows] window maximum
  double* x;                 // [nwindows][nwin * maxNodes] fit scratch
  double* y;
  unsigned long long* key;
  int* hist;                 // [nwindows][nwin * maxNodes + 1]
  unsigned long long* fkey;  // [nwindows][nwin * maxNodes + 1] mode scratch
  int* fidx;                 // [nwindows][nwin * maxNodes + 1]
  double* est;               // [nwindows][3] (alpha, mu, sigma), caller-side
};
int noise_levels(int S);
int noise_blocks(int nlev);
cudaError_t launch_noise_frames(const float* xs, const double* x64, int nimg, int S,
                                const NoiseFrames& nf, cudaStream_t s);
cudaError_t launch_noise_pass(const NoiseFrames& nf, const NoisePass& np, const float* xs,
                              const double* x64, int S, cudaStream_t s);
cudaError_t launch_noise_apply(const Problem& pb, const DeviceBuffers& d, const double* est,
                               int win0, cudaStream_t s);

// hot-pixel filter (hotpixel.cu)
cudaError_t launch_hot_pixel(uint16_t* seq, int nr, int nc, int nimg, double thr, uint16_t* colmed,
                             uint32_t* med, uint32_t* madm, uint8_t* flag, cudaStream_t s);

// learned lambda proposal (lambda.cu)
struct LambdaTrain {
  float* m;            // FP32 model (PGSVT_LAMBDA_MODEL_FLOATS)
  void* wbf;           // bf16 shadow
  float *mom1, *mom2;  // Adam moments (PGSVT_LAMBDA_PARAMS)
  const float* feat;   // [n][67]
  const float* target; // [n]
  const int32_t* perm; // [epochs][n] sample order
  int* epoch;          // device epoch counter
  float* part;         // [batch/32][PGSVT_LAMBDA_PARAMS] gradient partials
  float* loss_acc;     // [steps][batch/32]
  float* epoch_loss;   // [epochs]
  int n, batch, steps, total_steps;
  float lr, lr_final, wd, b1, b2, eps;
};
cudaError_t launch_lambda_features(const Problem& pb, const DeviceBuffers& d, cudaStream_t s);
cudaError_t launch_lambda_propose(const Problem& pb, const DeviceBuffers& d, cudaStream_t s);
cudaError_t launch_search_hint(const Problem& pb, const DeviceBuffers& d, cudaStream_t s);
cudaError_t lambda_shadow(const float* m, void* wbf, cudaStream_t s);
cudaError_t lambda_forward(const float* m, const void* wbf, const float* feat, int n, float* y,
                           cudaStream_t s);
cudaError_t lambda_grad(const float* m, const void* wbf, const float* feat, const float* target,
                        int n, float* part, float* part_loss, float* grad, cudaStream_t s);
cudaError_t lambda_train_epoch(const LambdaTrain& t, cudaStream_t s);
cudaError_t lambda_attrs();

// message returned by pgsvt_last_error() on the calling thread
void set_last_error(const std::string& m);

int eval_blocks(const Geometry& g);
int mse_blocks(const Geometry& g);
int svd_columns(int nwin);
constexpr int kSvdVariants = 6;
int svd_variants(int M, int NC);
bool svd_qr_form(int M, int NC);  // the QR-preconditioned SVD applies (its scratch is needed)
int svd_default_variant(int M, int NC);
bool svd_split_scratch(int M, int NC);  // a split SVD form applies (xq, xqn needed)
bool svd_variant_ok(int M, int NC, int v);
bool svd_supported(int bs, int nwin);

}  // namespace pgsvt

#endif
