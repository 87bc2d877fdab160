/*
 * pgsvt_oracle.h — C API of the CPU oracle (test infrastructure only).
 *
 * The oracle is an FP64 restatement of the reference's denoising path
 * (src/pguresvt.hpp, src/arps.hpp, src/svt.hpp, src/pgure.hpp,
 * src/utils.hpp of tjof2/pgure-svt 0.6.4).  It is the parity checker for the
 * CUDA library and the timed CPU baseline; nothing in the product links it.
 * The SVD is LAPACK dgesdd (the routine behind arma::svd_econ's default "dc"
 * method), supplied at run time as a function pointer (orc_set_dgesdd).
 */
#ifndef PGSVT_ORACLE_H
#define PGSVT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef void (*orc_dgesdd_fn)(char* jobz, int* m, int* n, double* a, int* lda,
                              double* s, double* u, int* ldu, double* vt,
                              int* ldvt, double* work, int* lwork, int* iwork,
                              int* info);

/* Same fields, order and meaning as pgsvt_params (include/pgsvt.h). */
typedef struct {
  uint32_t traj_length, block_size, block_overlap, motion_window;
  int64_t median_size;
  uint32_t noise_method, max_iter;
  int64_t n_jobs, random_seed;
  int32_t optimize_pgure, exp_weighting, motion_estimation, verbose;
  double lambda, alpha, mu, sigma, tol;
  uint32_t compat_flags, search_points, search_rounds, window_batch;
  double lambda_hint, hint_span;
  uint32_t frame_begin, frame_end;
  const float* lambda_model;  /* unused by the oracle (layout only) */
  uint32_t hint_points, hint_rounds;
  double hint_flat;
  uint32_t autotune;  /* unused by the oracle (layout only) */
  /* oracle only: per-frame narrow-search centres (NULL: lambda_hint for all)
   * and per-frame outputs (NULL: not written) */
  const double* lambda_hints;
  double* risk_out;
  uint32_t* evals_out;
  /* oracle only: threads inside each window (ARPS positions, SVD patches,
   * reconstruction frames); results do not depend on it.  0 or 1: one. */
  uint32_t window_threads;
} orc_params;

typedef struct {
  uint64_t windows;
  uint64_t risk_evals;
  double seconds;
} orc_report;

void orc_set_dgesdd(orc_dgesdd_fn fn);

/* Threads used inside one window by orc_arps_window, orc_svd_window,
 * orc_reconstruct_window and orc_risk_window (default 1; results do not
 * depend on it). */
void orc_set_threads(uint32_t n);

/* PGURE probes (pgure.hpp:167-186): delta1 (+-1) then delta2, n each. */
int orc_probes(int64_t seed, uint64_t n, int8_t* d1, double* d2);

/* Kept patch indices (svt.hpp:61-94), sorted unique.  out may be NULL to
 * query the count only. */
int orc_patch_list(uint32_t side, uint32_t bs, uint32_t ov, int64_t* out,
                   uint64_t* count);

int orc_arps_window(const double* w, uint32_t side, uint32_t nwin, uint32_t bs,
                    uint32_t mw, uint32_t time_iter, uint32_t frame_window,
                    uint32_t nimages, int32_t motion, uint32_t compat,
                    int32_t* rows, int32_t* cols);

int orc_svd_window(const double* u, uint32_t side, uint32_t nwin, uint32_t bs,
                   uint32_t ov, const int32_t* rows, const int32_t* cols,
                   double* S, uint64_t* npatch);

int orc_reconstruct_window(const double* u, uint32_t side, uint32_t nwin,
                           uint32_t bs, uint32_t ov, int32_t expw,
                           const int32_t* rows, const int32_t* cols,
                           double lambda, double* v);

int orc_risk_window(const double* u, uint32_t side, uint32_t nwin, uint32_t bs,
                    uint32_t ov, int32_t expw, const int32_t* rows,
                    const int32_t* cols, double alpha, double mu, double sigma,
                    int64_t seed, uint32_t compat, const double* lambdas,
                    uint32_t nl, double* risk);

/* Noise parameters of a normalised window (NoiseEstimator::Estimate,
 * noise.hpp:36-152): u is nrows x ncols x nslices; alpha/mu/sigma hold the
 * user values (< 0: estimate) on entry and the results on exit. */
int orc_noise_estimate(const double* u, uint32_t nrows, uint32_t ncols, uint32_t nslices,
                       uint32_t method, double* alpha, double* mu, double* sigma);

/* Hot-pixel filter (hotpixel.hpp:19-64), in place on uint16 frames. */
int orc_hot_pixel(uint16_t* seq, uint32_t nrows, uint32_t ncols, uint32_t nframes,
                  double threshold);

/* Median of the (2r+1)^2 window with clamped coordinates (the reference's
 * ConstantTimeMedianFilter, medfilter.hpp:478-541); nx is the fast axis. */
int orc_median_filter(const uint16_t* src, uint16_t* dst, uint32_t nx, uint32_t ny,
                      uint32_t r);

/* Whole sequence (PGURESVT<T1,double>, pguresvt.hpp:17-172); X is FP64. */
int orc_denoise(const double* X, uint32_t nrows, uint32_t ncols,
                uint32_t nimages, const orc_params* p, double* Y,
                double* estimates, orc_report* rep);

const char* orc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
