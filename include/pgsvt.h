/*
 * pgsvt.h — C ABI of the GB300 PGURE-SVT denoiser (libpgsvt.so).
 *
 * This is the drop-in boundary for the reference's denoising entry point
 *
 *   template <typename T1, typename T2>
 *   uint32_t PGURESVT(arma::Cube<T2>& Y, arma::Mat<T2>& estimates,
 *                     const arma::Cube<T1>& X, uint32_t trajLength,
 *                     uint32_t blockSize, uint32_t blockOverlap,
 *                     uint32_t motionWindow, int64_t medianSize,
 *                     uint32_t noiseMethod, uint32_t maxIter, int64_t nJobs,
 *                     int64_t randomSeed, bool optimizePGURE, bool expWeighting,
 *                     bool motionEstimation, double lambdaEst, double alphaEst,
 *                     double muEst, double sigmaEst, double tol, bool verbose)
 *     (src/pguresvt.hpp:17-38; bound from Python in pguresvt/_pguresvt.pyx:143-148)
 *
 * Plain pointers and sizes only: no Armadillo, no torch types.  All arrays are
 * column-major exactly like the reference's Armadillo cubes: element
 * (r, c, t) of an nrows x ncols x nframes cube sits at r + c*nrows + t*nrows*ncols.
 * `estimates` is the reference's Mat<double>(nframes, 4): element (t, j) at
 * t + j*nframes, columns (lambda, alpha, mu, sigma) as in pguresvt.hpp:150-153.
 *
 * Every call computes on one CUDA device (the current one) with hand-written
 * sm_103a kernels.  There is no CPU fallback: if no device is usable the call
 * fails with PGSVT_ERR_CUDA.
 */
#ifndef PGSVT_H
#define PGSVT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PGSVT_ABI_VERSION 1

/* Input element types: the reference instantiates PGURESVT for uint8, uint16,
 * float and double inputs (pguresvt/_pguresvt.pyx:151,210,269,328). */
typedef enum {
  PGSVT_U8 = 0,
  PGSVT_U16 = 1,
  PGSVT_F32 = 2,
  PGSVT_F64 = 3
} pgsvt_dtype;

typedef enum {
  PGSVT_OK = 0,
  PGSVT_ERR_INVALID_ARG = 1,   /* bad size / parameter (message says which) */
  PGSVT_ERR_UNSUPPORTED = 2,   /* a reference feature this build does not run */
  PGSVT_ERR_CUDA = 3,          /* CUDA runtime error or no usable device */
  PGSVT_ERR_OOM = 4,           /* device allocation failed */
  PGSVT_ERR_TIMEOUT = 5,       /* a bounded device wait expired */
  PGSVT_ERR_NONFINITE = 6      /* input holds NaN / Inf */
} pgsvt_status_code;

/* Reference behaviours that are reproduced by default (parity mode).  Clearing
 * a bit selects the evidently intended behaviour instead.                     */
/* PGURE(u,p,alpha,sigma,mu,...) binds to the ctor's (alpha,mu,sigma): inside the
 * risk mu and sigma are swapped (pguresvt.hpp:133 vs pgure.hpp:26-30).         */
#define PGSVT_COMPAT_SWAP_MU_SIGMA 0x1u
/* With motion estimation off, frames other than the reference frame keep
 * trajectory coordinates (0,0) (arps.hpp:42,60-64).  Cleared: every frame uses
 * the patch's own grid position.                                               */
#define PGSVT_COMPAT_ZERO_MOTION 0x2u
/* delta1 is an integer cube, so delta1*eps1 truncates eps1 to 0 and U1 == U
 * (pgure.hpp:80,167-183): the first-order divergence term vanishes.  Cleared:
 * U1 = U + eps1*delta1 is decomposed and the term is evaluated.               */
#define PGSVT_COMPAT_INT_DELTA1 0x4u
#define PGSVT_COMPAT_ALL 0x7u

/* Parameters of PGURESVT (pguresvt.hpp:17-38), same names and sentinels:
 * negative lambda/alpha/mu/sigma mean "estimate", random_seed < 0 seeds from
 * std::random_device, median_size <= 0 disables the median pre-filter.      */
typedef struct {
  uint32_t traj_length;     /* trajLength   (Python: trajectory_length) */
  uint32_t block_size;      /* blockSize    (patch_size)                */
  uint32_t block_overlap;   /* blockOverlap (patch_overlap)             */
  uint32_t motion_window;   /* motionWindow (motion_window)             */
  int64_t median_size;      /* medianSize   (motion_filter)             */
  uint32_t noise_method;    /* noiseMethod  (noise_method)              */
  uint32_t max_iter;        /* maxIter: cap on risk evaluations/window  */
  int64_t n_jobs;           /* nJobs: host threads (staging only)       */
  int64_t random_seed;      /* randomSeed                               */
  int32_t optimize_pgure;   /* optimizePGURE                            */
  int32_t exp_weighting;    /* expWeighting                             */
  int32_t motion_estimation;/* motionEstimation                         */
  int32_t verbose;          /* verbose                                  */
  double lambda;            /* lambdaEst (start point when optimising)  */
  double alpha;             /* alphaEst                                 */
  double mu;                /* muEst                                    */
  double sigma;             /* sigmaEst                                 */
  double tol;               /* tol (ftol of the lambda search)          */
  uint32_t compat_flags;    /* PGSVT_COMPAT_* (default PGSVT_COMPAT_ALL)*/
  uint32_t search_points;   /* grid points; K/2 per refinement (0: 8)   */
  uint32_t search_rounds;   /* refinement rounds after the grid (0: 4)  */
  uint32_t window_batch;    /* windows in flight on the device (0: auto)*/
  double lambda_hint;       /* >0: narrow search around this proposal   */
  double hint_span;         /* bracket [hint/span, hint*span] (0: 2.0)  */
  uint32_t frame_begin;     /* output frames [frame_begin, frame_end) are */
  uint32_t frame_end;       /* computed (0,0: all); others are left zero  */
  /* Learned lambda proposal (not in the reference): a host array of
   * PGSVT_LAMBDA_MODEL_FLOATS floats (see pgsvt_lambda_train), NULL: off.
   * Each window's proposal replaces lambda_hint for that window.  A model
   * serves the patch size and window length it was trained on: the shipped
   * one (lambda_mlp.npz) covers 4x4 patches and 15-frame windows.          */
  const float* lambda_model;
  uint32_t hint_points;     /* lambda values per narrow-search round (0: 4) */
  uint32_t hint_rounds;     /* refinement rounds of the narrow search (0: 2) */
  double hint_flat;         /* a best point on the narrow grid's edge is kept
                               when its neighbour's risk is within this
                               relative amount (0: 1e-3); else the plain
                               search runs                                   */
  uint32_t autotune;        /* 1: time the SVD kernel shapes on the first
                               window batch of each patch size / window
                               length seen by the process and keep the
                               fastest (results agree to FP32 rounding);
                               0: the default shape (the QR-preconditioned
                               form for 7x7 and 8x8 patches and windows
                               <= 15 frames, else the register form);
                               2: more lanes per patch where the patch size
                               has that form; 3: the register form with
                               its columns in shared memory; 4: 8 rows per
                               lane (patch sides <= 4 and 7..8, windows
                               <= 15); 5: the QR-preconditioned form (patch
                               sides 5..8, windows <= 15); 6: the two-kernel
                               register form with the factors assembled from
                               TMA-staged frame tiles (patch sides <= 4,
                               windows <= 15)                                */
} pgsvt_params;

/* Optional per-frame outputs of pgsvt_denoise_ex / pgsvt_denoise_device_ex
 * (host memory for the former, device memory for the latter; any member may
 * be NULL).                                                                  */
typedef struct {
  float* lambda_features;   /* nframes x PGSVT_LAMBDA_FEATURES, row t at
                               t*PGSVT_LAMBDA_FEATURES                      */
  float* lambda_proposals;  /* nframes: model output log10(lambda/upper)
                               (NaN without a model)                       */
  double* risk;             /* nframes: PGURE risk at the returned lambda
                               (0 when not optimising)                     */
  uint32_t* risk_evals;     /* nframes: lambda values evaluated            */
} pgsvt_outputs;

/* Per-call report.  All times are wall seconds measured by the library. */
typedef struct {
  int32_t code;             /* pgsvt_status_code of the call              */
  int32_t cuda_error;       /* last cudaError_t seen (0 if none)          */
  uint64_t windows;         /* windows (output frames) processed          */
  uint64_t risk_evals;      /* lambda values evaluated over all windows   */
  uint64_t kernel_launches; /* kernels launched by the call               */
  uint64_t h2d_bytes;       /* host->device bytes copied                  */
  uint64_t d2h_bytes;       /* device->host bytes copied                  */
  double seconds;           /* whole call                                 */
  /* device time per stage (CUDA events on the call's stream):
   * [0] convert + frame maxima  [1] window normalisation  [2] ARPS
   * [3] coverage + risk fields  [4] SVD  [5] lambda search rounds
   * [6] final reconstruction + output  [7] uploads between batches       */
  double stage_seconds[8];
  uint64_t svd_launches;    /* launches of the SVD kernel                 */
  uint64_t svd_matrices;    /* Casorati matrices decomposed               */
  uint64_t arps_exact_steps;/* ARPS diamond steps decided in FP64         */
  uint64_t svd_fp64_tests;  /* Jacobi convergence decisions taken from    *
                             * FP64 inner products (per patch and check)  */
  uint64_t svd_warp_sweeps; /* Jacobi sweeps summed over warps            */
  char message[256];        /* human-readable error / note                */
  int32_t svd_variant;      /* SVD kernel shape used (0: default)         */
  int32_t svd_tuned;        /* 1 if this call ran the autotuner           */
} pgsvt_status;

/* Fill *p with the reference defaults (pguresvt/_pguresvt.pyx:151-168 and
 * pguresvt/svt.py:172-191): T=15, patch 4, overlap 1, motion window 7,
 * median 5, noise method 4, max_iter 500, n_jobs -1, seed -1, optimise,
 * exponential weighting, motion estimation on, lambda/alpha/mu/sigma -1,
 * tol 1e-7, compat PGSVT_COMPAT_ALL.                                       */
int pgsvt_default_params(pgsvt_params* p);

/* Denoise an image sequence: the replacement for PGURESVT<T1,double>
 * (pguresvt.hpp:17-172).  X is host memory (nrows x ncols x nframes, dtype
 * `dtype`), Y (same shape, double) and estimates (nframes x 4, double) are
 * host memory owned by the caller.  Returns a pgsvt_status_code; `st` may be
 * NULL.  Frames must be square (the reference's ARPS indexing assumes it,
 * arps.hpp:186-187) and nframes >= the clamped trajectory length.          */
int pgsvt_denoise(const void* X, int32_t dtype, uint32_t nrows, uint32_t ncols,
                  uint32_t nframes, double* Y, double* estimates,
                  const pgsvt_params* p, pgsvt_status* st);

/* Same as pgsvt_denoise with X, Y, estimates already in device memory of the
 * current device; `stream` is a cudaStream_t (NULL: the library's stream).
 * The call returns after the work has completed.                          */
int pgsvt_denoise_device(const void* X_dev, int32_t dtype, uint32_t nrows,
                         uint32_t ncols, uint32_t nframes, double* Y_dev,
                         double* estimates_dev, const pgsvt_params* p,
                         void* stream, pgsvt_status* st);

/* pgsvt_denoise / pgsvt_denoise_device plus the optional per-frame outputs
 * listed in a pgsvt_outputs struct; `out` may be NULL.                      */
int pgsvt_denoise_ex(const void* X, int32_t dtype, uint32_t nrows, uint32_t ncols,
                     uint32_t nframes, double* Y, double* estimates,
                     const pgsvt_params* p, const pgsvt_outputs* out,
                     pgsvt_status* st);
int pgsvt_denoise_device_ex(const void* X_dev, int32_t dtype, uint32_t nrows,
                            uint32_t ncols, uint32_t nframes, double* Y_dev,
                            double* estimates_dev, const pgsvt_params* p,
                            const pgsvt_outputs* out_dev, void* stream,
                            pgsvt_status* st);

/* --- Batches of sequences (config of uneven sizes; not in the reference) ---
 *
 * One sequence of a batch.  X, Y and estimates are host memory as in
 * pgsvt_denoise.  With `lambdas` (nlambdas <= 16 values), every window
 * evaluates the PGURE risk of exactly those values (one round, together)
 * and is reconstructed at the one of least risk; `risks` (optional,
 * nframes x nlambdas, row t at t*nlambdas) receives them.  Without a list
 * the window runs the lambda search of `params`.  `status` (optional)
 * receives the sequence's own report.                                       */
typedef struct {
  const void* X;
  int32_t dtype;
  uint32_t nrows, ncols, nframes;
  double* Y;
  double* estimates;
  const pgsvt_params* params;
  const double* lambdas;
  uint32_t nlambdas;
  double* risks;
  pgsvt_status* status;
} pgsvt_sequence;

/* Denoise nseq sequences of any sizes, patch sizes and trajectory lengths on
 * the current device.  A host work queue hands the sequences, largest first,
 * to `slots` concurrent workers (0: 2), each with its own stream, so that
 * one sequence's uploads, ARPS and search overlap another's SVD.  `st`
 * (optional) receives the totals; the return value is the first failing
 * sequence's code (PGSVT_OK if none).                                       */
int pgsvt_denoise_batch(const pgsvt_sequence* seqs, uint32_t nseq, uint32_t slots,
                        pgsvt_status* st);

/* --- Learned lambda proposal (not in the reference) ---
 *
 * A window's features are the three noise parameters as its risk uses them
 * (after the PGSVT_COMPAT_SWAP_MU_SIGMA binding), each as asinh(1000 v)/8,
 * and a 64-bin histogram of log10 of the singular values of 4096 of its
 * kept patches (stratified, seeded choice; all patches when fewer), bins of
 * width 6/64 over [-4, 2), clamped at both ends, counts divided by the
 * number of values.  The MLP maps them to y = log10(lambda/upper):
 *   x0 = (f - mean) * scale
 *   a1 = gelu(W1 x0 + b1), a2 = gelu(W2 a1 + b2), a3 = gelu(W3 a2 + b3)
 *   y  = (W4 a3 + b4) * y_scale + y_mean
 * with gelu(z) = z/2 (1 + erf(z/sqrt 2)).  W1..W4 are used rounded to bf16
 * (round to nearest even); biases, activations and sums are FP32.
 * Model array (floats): mean[67] scale[67] W1[128][67] b1[128] W2[128][128]
 * b2[128] W3[128][128] b3[128] W4[128] b4 y_mean y_scale.  The trainable
 * parameters are the PGSVT_LAMBDA_PARAMS floats from W1 to b4.            */
#define PGSVT_LAMBDA_FEATURES 67
#define PGSVT_LAMBDA_HIDDEN 128
#define PGSVT_LAMBDA_SAMPLES 4096
#define PGSVT_LAMBDA_MODEL_FLOATS 41993
#define PGSVT_LAMBDA_PARAM_OFFSET 134
#define PGSVT_LAMBDA_PARAMS 41857

/* Model outputs y for n feature rows (host buffers). */
int pgsvt_lambda_predict(const float* model, const float* features, uint32_t n, float* y);

/* Gradient of the loss L = (1/n) sum_i (o_i - t_i)^2, o_i the network output
 * before the y_scale/y_mean map and t_i = (target_i - y_mean)/y_scale, with
 * respect to the PGSVT_LAMBDA_PARAMS trainable floats (taken at their bf16
 * values for the weights).  Host buffers; *loss receives L.               */
int pgsvt_lambda_grad(const float* model, const float* features, const float* targets,
                      uint32_t n, float* grad, double* loss);

typedef struct {
  uint32_t epochs;          /* passes over the samples                     */
  uint32_t batch;           /* samples per step (multiple of 32)           */
  float lr, lr_final;       /* AdamW step size, cosine-decayed to lr_final */
  float weight_decay;       /* decoupled decay (weights only)              */
  float beta1, beta2, eps;  /* Adam moments                                */
  uint64_t seed;            /* shuffling                                   */
} pgsvt_train_params;

/* Train the model in place on the device (FP32 master weights, bf16 weights
 * in the forward and backward passes, AdamW), one CUDA graph per epoch.
 * `model` holds the initial values, including mean/scale/y_mean/y_scale,
 * which training keeps.  epoch_loss (may be NULL) receives the mean loss of
 * each epoch.                                                               */
int pgsvt_lambda_train(float* model, const float* features, const float* targets,
                       uint32_t n, const pgsvt_train_params* tp, float* epoch_loss,
                       pgsvt_status* st);

/* --- Component entry points (one reference stage each, host buffers) --- */

/* ARPS block matching for one window (MotionEstimator::Estimate,
 * arps.hpp:52-134).  `w` is the max-normalised window (double, nrows x nrows
 * x nwin with nwin = 2*(T/2)+1); time_iter / frame_window / nimages are the
 * reference's timeIter / timeWindow / nImages.  Writes the trajectory table
 * (the reference's icube patches(2, P, nwin)) as rows[k*P+it], cols[k*P+it].*/
int pgsvt_arps_window(const double* w, uint32_t nrows, uint32_t nwin,
                      uint32_t block_size, uint32_t motion_window,
                      uint32_t time_iter, uint32_t frame_window,
                      uint32_t nimages, int32_t motion_estimation,
                      uint32_t compat_flags, int32_t* rows, int32_t* cols);

/* Singular values of every kept patch's Casorati matrix for one window
 * (SVT::Decompose, svt.hpp:58-118).  `u` is the normalised window, rows/cols
 * the trajectory table.  S is npatch x nwin (descending per patch);
 * *npatch receives the number of kept patches (svt.hpp:61-94).            */
int pgsvt_svd_window(const double* u, uint32_t nrows, uint32_t nwin,
                     uint32_t block_size, uint32_t block_overlap,
                     const int32_t* rows, const int32_t* cols, float* S,
                     uint32_t* npatch);

/* pgsvt_svd_window that also fills `st` (may be NULL): svd_matrices,
 * svd_warp_sweeps and svd_fp64_tests, the Jacobi convergence decisions taken
 * from FP64 inner products when a sweep rotated only near-degenerate pairs. */
int pgsvt_svd_window_ex(const double* u, uint32_t nrows, uint32_t nwin,
                        uint32_t block_size, uint32_t block_overlap,
                        const int32_t* rows, const int32_t* cols, float* S,
                        uint32_t* npatch, pgsvt_status* st);

/* Singular-value thresholding reconstruction of one window at `lambda`
 * (SVT::Reconstruct, svt.hpp:121-167): v is nrows x nrows x nwin double. */
int pgsvt_reconstruct_window(const double* u, uint32_t nrows, uint32_t nwin,
                             uint32_t block_size, uint32_t block_overlap,
                             int32_t exp_weighting, const int32_t* rows,
                             const int32_t* cols, double lambda, double* v);

/* PGURE risk of one window at `nl` lambda values (PGURE ctor + CalculatePGURE,
 * pgure.hpp:26-137).  alpha/mu/sigma are the caller-side values passed to
 * PGURE (the swap of PGSVT_COMPAT_SWAP_MU_SIGMA is applied inside).         */
int pgsvt_risk_window(const double* u, uint32_t nrows, uint32_t nwin,
                      uint32_t block_size, uint32_t block_overlap,
                      int32_t exp_weighting, const int32_t* rows,
                      const int32_t* cols, double alpha, double mu,
                      double sigma, int64_t random_seed, uint32_t compat_flags,
                      const double* lambdas, uint32_t nl, double* risk);

/* Median pre-filter of the ARPS input for `nframes` uint16 frames
 * (ConstantTimeMedianFilter, medfilter.hpp:478-541, as called in
 * pguresvt.hpp:69-80): the median of the (2r+1)^2 window with coordinates
 * clamped to the frame.  src and dst are host arrays of nrows x ncols x
 * nframes (column-major); 1 <= r <= 15 and 2r+1 <= min(nrows, ncols).     */
int pgsvt_median_filter(const uint16_t* src, uint16_t* dst, uint32_t nrows, uint32_t ncols,
                        uint32_t nframes, uint32_t r);

/* Hot-pixel filter of the command-line tool (HotPixelFilter,
 * hotpixel.hpp:19-64, applied by PGURE-SVT.cpp:170-176 when `hot_pixel` is
 * set), in place on `nframes` uint16 frames (host, nrows x ncols x nframes,
 * column-major): per frame, pixels farther than threshold x MAD (median
 * absolute deviation / 0.6745) from the median are replaced by the mean of
 * the middle two of their 8 neighbours, or by the median at the frame edge. */
int pgsvt_hot_pixel_filter(uint16_t* frames, uint32_t nrows, uint32_t ncols, uint32_t nframes,
                           double threshold);

/* Singular values of one window without any device allocation.
 *
 * This entry point has no counterpart in the reference.  It serves callers
 * that cannot allocate device memory while they work: acquisition loops that
 * reserved their memory up front, code running under an allocator that owns
 * the whole device, or processes that must avoid cudaMalloc/cudaFree because
 * those calls synchronise the device.  Inputs and outputs are caller-owned
 * device memory: u_dev is the normalised window (float, nrows x nrows x nwin,
 * column-major), rows_dev/cols_dev the trajectory table (int32, nwin x P as in
 * pgsvt_arps_window), S_dev receives npatch x nwin singular values (descending
 * per patch, patches in the reference's sorted order; NULL: only *npatch is
 * set).  Intermediates live in a fixed static device array (about 1 MB, held
 * by every GPU that loads the library until the process exits), so windows
 * are limited to nrows <= PGSVT_NOALLOC_MAX_SIDE, nwin <= PGSVT_NOALLOC_MAX_NWIN
 * and block_size <= 4; larger ones are rejected with PGSVT_ERR_INVALID_ARG.
 * The first call on a device looks up that device's copy of the array (make
 * it before any stream capture); the first call after a cudaDeviceReset
 * looks it up again.  Non-finite or huge pixel values give non-finite
 * singular values, never a fault.  All calls share the array and it keeps the
 * previous call's contents: calls whose GPU work overlaps race, so serialise
 * them.  Runs on `stream` (a cudaStream_t, NULL: default stream) and returns
 * once the work has completed: it copies the patch list from pageable host
 * memory and synchronises the stream, so no call can be captured into a
 * CUDA graph.  Calls no allocating routine.                                  */
#define PGSVT_NOALLOC_MAX_SIDE 64
#define PGSVT_NOALLOC_MAX_NWIN 15
int pgsvt_svd_window_noalloc(const float* u_dev, uint32_t nrows, uint32_t nwin,
                             uint32_t block_size, uint32_t block_overlap,
                             const int32_t* rows_dev, const int32_t* cols_dev,
                             float* S_dev, uint32_t* npatch, void* stream);

/* Message of the last failing call on this thread ("" if none). */
const char* pgsvt_last_error(void);

/* Library version string, e.g. "pgsvt-gb300 0.1.0 (sm_103a)". */
const char* pgsvt_version(void);

#ifdef __cplusplus
}
#endif

#endif /* PGSVT_H */
