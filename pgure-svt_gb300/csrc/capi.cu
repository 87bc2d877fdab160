// capi.cu — host orchestration and the C ABI of libpgsvt (include/pgsvt.h).
//
// pgsvt_denoise replaces PGURESVT<T1,double> (pguresvt.hpp:17-172).  Instead of
// the reference's std::thread fan-out over output frames (utils.hpp:108-168),
// windows are processed W at a time on one device: every kernel of the
// per-window pipeline runs over the whole batch, and the lambda search is a
// device-resident state machine, so a batch is one fixed, synchronisation-free
// launch sequence on one stream.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <atomic>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "pgsvt.h"
#include "pgsvt_internal.h"

using namespace pgsvt;

namespace {

thread_local std::string g_err;

struct Fail : std::runtime_error {
  int code;
  int cuda;
  Fail(int c, const std::string& m, int ce = 0) : std::runtime_error(m), code(c), cuda(ce) {}
};

#define PGSVT_CK(x)                                                                  \
  do {                                                                               \
    cudaError_t e_ = (x);                                                            \
    if (e_ != cudaSuccess)                                                           \
      throw Fail(e_ == cudaErrorMemoryAllocation ? PGSVT_ERR_OOM : PGSVT_ERR_CUDA,   \
                 std::string(#x) + ": " + cudaGetErrorString(e_), (int)e_);          \
  } while (0)

// ---------------------------------------------------------------------------
// Probes: pcg64 (O'Neill's PCG, 128-bit LCG with XSL-RR output, seeded as the
// reference's RNG.seed(randomSeed), pgure.hpp:52-59) feeding
// std::bernoulli_distribution semantics (one 64-bit draw scaled by 2^-64,
// true when below p), in column-major cube order, delta1 then delta2
// (pgure.hpp:167-186).
class Pcg64 {
 public:
  using u128 = unsigned __int128;
  explicit Pcg64(u128 seed) {
    inc_ = ((u128)6364136223846793005ULL << 64) | 1442695040888963407ULL;
    state_ = (seed + inc_) * mult() + inc_;
  }
  uint64_t operator()() {
    state_ = state_ * mult() + inc_;
    const uint64_t hi = (uint64_t)(state_ >> 64), lo = (uint64_t)state_;
    const unsigned rot = (unsigned)(hi >> 58);
    const uint64_t x = hi ^ lo;
    return (x >> rot) | (x << ((64u - rot) & 63u));
  }

 private:
  static u128 mult() { return ((u128)2549297995355413924ULL << 64) | 4865540595714422341ULL; }
  u128 state_, inc_;
};

bool draw(Pcg64& g, double p) {
  double u = (double)g() / 18446744073709551616.0;
  if (u >= 1.0) u = std::nextafter(1.0, 0.0);
  return u < p;
}

double probe_vp() {
  const double kappa = 1.0;
  return 0.5 + 0.5 * kappa / std::sqrt(kappa * kappa + 4);
}

void make_probes(int64_t seed, size_t n, int8_t* d1, int8_t* d2code) {
  Pcg64::u128 s;
  if (seed >= 0) {
    s = (Pcg64::u128)(uint64_t)seed;
  } else {
    std::random_device rd;
    s = ((Pcg64::u128)(((uint64_t)rd() << 32) | rd()) << 64) | (((uint64_t)rd() << 32) | rd());
  }
  Pcg64 g(s);
  const double vP = probe_vp();
  for (size_t i = 0; i < n; ++i) d1[i] = draw(g, 0.5) ? -1 : 1;
  for (size_t i = 0; i < n; ++i) d2code[i] = draw(g, vP) ? 1 : 0;
}

// ---------------------------------------------------------------------------
std::vector<int32_t> patch_list(int S, int bs, int ov) { return kept_patches(S, bs, ov); }

// Processing order of the kept patches: 8 x 8 tiles of grid positions (rows
// fastest), so the 32 patches of a lambda-evaluation block (half a tile)
// cover a compact region of every slice and their rebuilt blocks overlap
// (k_eval).  The
// order has no effect on the results: the overlap sums are integer sums.
std::vector<int32_t> tile_order(const std::vector<int32_t>& plist, int S, int bs) {
  const int n1 = S - bs + 1, ti = (n1 + 7) / 8;
  std::vector<std::pair<int64_t, int32_t>> key;
  key.reserve(plist.size());
  for (int32_t it : plist) {
    const int i = it % n1, j = it / n1;
    const int64_t tk = ((int64_t)(j / 8) * ti + i / 8) * 64 + (j % 8) * 8 + (i % 8);
    key.push_back({tk, it});
  }
  std::sort(key.begin(), key.end());
  std::vector<int32_t> out;
  out.reserve(key.size());
  for (auto& kv : key) out.push_back(kv.second);
  return out;
}

// Kept patches whose singular values make up a window's lambda features: a
// stratified choice of PGSVT_LAMBDA_SAMPLES of them (all of them when fewer)
// in the reference's sorted order, sample i drawn from stratum i at an
// offset given by the lowbias32 integer hash (C. Wellons) of i.  Returned as
// processing slots.
uint32_t lowbias32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

std::vector<int32_t> feature_slots(const std::vector<int32_t>& sorted,
                                   const std::vector<int32_t>& plist, int P) {
  const uint64_t NP = sorted.size();
  const uint64_t ns = std::min<uint64_t>(NP, PGSVT_LAMBDA_SAMPLES);
  std::vector<int32_t> slot_of(P, -1);
  for (size_t k = 0; k < plist.size(); ++k) slot_of[plist[k]] = (int32_t)k;
  std::vector<int32_t> out(ns);
  for (uint64_t i = 0; i < ns; ++i) {
    const uint64_t h = lowbias32((uint32_t)i ^ 0x5eed1234u);
    const uint64_t k = (i * NP + ((h * NP) >> 32)) / ns;
    out[i] = slot_of[sorted[k]];
  }
  return out;
}

// Frame pairs of MotionEstimator::Estimate (arps.hpp:52-134) grouped into
// chains of pairs that share a motion slot (the only data dependence).
std::vector<ArpsChain> chains_for(int t, int tw, int nimg, int nwin) {
  struct Pr { int a1, a2, a3; };
  std::vector<Pr> prs;
  if (t < tw) {
    const int loopEnd = nwin - t - 1;
    for (int i = 0; i < loopEnd; ++i) prs.push_back({t + i, t + i + 1, t + i});
    for (int i = 0; i < t; ++i) prs.push_back({t - i, t - i - 1, t - i});
  } else if (t >= nimg - tw) {
    const int e = t - (nimg - nwin), loopEnd = 2 * tw - e;
    for (int i = 0; i < loopEnd; ++i) prs.push_back({e + i, e + i + 1, e + i});
    for (int i = 0; i < e; ++i) {
      if (2 * tw == e) prs.push_back({e - i, e - i - 1, e - i - 1});
      else prs.push_back({e - i, e - i - 1, e - i});
    }
  } else {
    for (int i = 0; i < tw; ++i) prs.push_back({tw + i, tw + i + 1, tw + i});
    for (int i = 0; i < tw; ++i) prs.push_back({tw - i, tw - i - 1, tw - i});
  }
  std::vector<ArpsChain> out(2 * tw);
  std::vector<int> slot_of(2 * tw + 1, -1);
  int n = 0;
  for (const Pr& p : prs) {
    int& c = slot_of[p.a3];
    if (c < 0) c = n++;
    ArpsChain& ch = out[c];
    if (ch.npairs >= 2) throw Fail(PGSVT_ERR_INVALID_ARG, "ARPS chain longer than 2 pairs");
    ch.a1[ch.npairs] = (int8_t)p.a1;
    ch.a2[ch.npairs] = (int8_t)p.a2;
    ch.npairs++;
  }
  return out;
}

struct DevMem {
  std::vector<void*> ptrs;
  void* get(size_t bytes) {
    void* p = nullptr;
    if (bytes == 0) bytes = 16;
    PGSVT_CK(cudaMalloc(&p, bytes));
    ptrs.push_back(p);
    return p;
  }
  template <typename T>
  T* arr(size_t n) { return (T*)get(n * sizeof(T)); }
  ~DevMem() {
    for (void* p : ptrs) cudaFree(p);
  }
};

struct Stats {
  uint64_t launches = 0, h2d = 0, d2h = 0, evals = 0, windows = 0;
  uint64_t svd_launches = 0, svd_matrices = 0, arps_exact = 0, svd_fp64 = 0, svd_sweeps = 0;
  int svd_variant = 0, svd_tuned = 0;
  double stage[8] = {0, 0, 0, 0, 0, 0, 0, 0};
};

// Device time per pipeline stage: an event is recorded on the stream at each
// stage boundary and the intervals are summed once the stream is drained.
class StageClock {
 public:
  explicit StageClock(cudaStream_t s) : s_(s) {}
  ~StageClock() {
    for (auto& m : marks_) cudaEventDestroy(m.ev);
  }
  void mark(int stage) {  // the interval from the previous mark belongs to `stage`
    cudaEvent_t e;
    PGSVT_CK(cudaEventCreate(&e));
    PGSVT_CK(cudaEventRecord(e, s_));
    marks_.push_back({e, stage});
  }
  void accumulate(double* out) const {
    for (size_t i = 1; i < marks_.size(); ++i) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, marks_[i - 1].ev, marks_[i].ev) == cudaSuccess && ms > 0)
        out[marks_[i].stage] += ms * 1e-3;
    }
  }

 private:
  struct Mark { cudaEvent_t ev; int stage; };
  cudaStream_t s_;
  std::vector<Mark> marks_;
};

void check_launch(cudaError_t e, Stats& s, int n = 1) {
  s.launches += n;
  PGSVT_CK(e);
}

// Validation mirroring pguresvt/svt.py:212-271 and the limits of this build.
void validate(const pgsvt_params& p, uint32_t nr, uint32_t nc, uint32_t nimg) {
  if (nr == 0 || nc == 0 || nimg == 0) throw Fail(PGSVT_ERR_INVALID_ARG, "empty input");
  if (nr != nc)
    throw Fail(PGSVT_ERR_INVALID_ARG, "frames must be square (the reference's ARPS indexing, "
                                      "arps.hpp:186-187, assumes nrows == ncols)");
  if (nr > 32767) throw Fail(PGSVT_ERR_UNSUPPORTED, "frame side above 32767");
  if (p.block_size < 2 || p.block_size > 16)
    throw Fail(PGSVT_ERR_UNSUPPORTED, "block_size must be in [2, 16] in this build");
  if (p.block_size > nr) throw Fail(PGSVT_ERR_INVALID_ARG, "block_size larger than the frame");
  if (p.block_overlap < 1 || p.block_overlap > p.block_size)
    throw Fail(PGSVT_ERR_INVALID_ARG, "Invalid patch_overlap parameter: must be in [1, block_size]");
  if (p.traj_length < 1) throw Fail(PGSVT_ERR_INVALID_ARG, "Invalid trajectory_length parameter");
  const uint32_t Ntc = (p.block_size * p.block_size < p.traj_length)
                           ? p.block_size * p.block_size - 1 : p.traj_length;
  const uint32_t nwin = 2 * (Ntc / 2) + 1;
  if (nimg < nwin) throw Fail(PGSVT_ERR_INVALID_ARG, "sequence shorter than the trajectory");
  if (!svd_supported((int)p.block_size, (int)nwin))
    throw Fail(PGSVT_ERR_UNSUPPORTED, "trajectory window above 21 frames in this build");
  if (p.motion_estimation && (p.motion_window < 2 || p.motion_window > (uint32_t)kMaxMW))
    throw Fail(PGSVT_ERR_INVALID_ARG, "Invalid motion_window parameter: must be in [2, 15]");
  if (p.median_size > kMaxMedian)
    throw Fail(PGSVT_ERR_UNSUPPORTED, "motion_filter (median radius) above 15 in this build");
  if (p.median_size > 0 && 2 * p.median_size + 1 > (int64_t)nr)
    throw Fail(PGSVT_ERR_INVALID_ARG, "motion_filter window wider than the frame");
  if (p.optimize_pgure && (p.alpha < 0 || p.mu < 0 || p.sigma < 0)) {  // noise estimation
    if (nr > 8 && (nr & (nr - 1)))
      throw Fail(PGSVT_ERR_UNSUPPORTED, "noise estimation needs power-of-two frames "
                                        "(noise.hpp:216 has F-test values for 2^k blocks only); "
                                        "give alpha, mu and sigma");
    if (nr < 4) throw Fail(PGSVT_ERR_INVALID_ARG, "noise estimation needs frames of side >= 4");
    if (p.noise_method < 1 || p.noise_method > 4)
      throw Fail(PGSVT_ERR_INVALID_ARG, "noise_method must be 1, 2, 3 or 4");
  }
  if (!p.optimize_pgure && !(p.lambda >= 0))
    throw Fail(PGSVT_ERR_INVALID_ARG, "Invalid lambda1 parameter: must be >= 0 without optimisation");
  if (p.search_points > (uint32_t)kMaxK)
    throw Fail(PGSVT_ERR_INVALID_ARG, "search_points above 16");
}

struct Setup {
  Geometry g;
  int K, rounds, max_rounds;
  std::vector<int32_t> sorted;  // kept patches in the reference's (sorted) order
  std::vector<int32_t> plist;   // processing order
};

Setup make_setup(const pgsvt_params& p, int S, int nimg, int nfixed = 0) {
  Setup s;
  Geometry& g = s.g;
  g.S = S;
  g.bs = (int)p.block_size;
  g.M = g.bs * g.bs;
  g.Ntc = (g.M < (int)p.traj_length) ? g.M - 1 : (int)p.traj_length;  // pguresvt.hpp:57
  g.fw = g.Ntc / 2;                                                   // pguresvt.hpp:58
  g.nwin = 2 * g.fw + 1;
  g.P = (S - g.bs + 1) * (S - g.bs + 1);
  s.sorted = patch_list(S, g.bs, (int)p.block_overlap);
  s.plist = tile_order(s.sorted, S, g.bs);
  g.NP = (int)s.plist.size();
  g.NC = svd_columns(g.nwin);
  g.mw = (int)p.motion_window;
  g.nimg = nimg;
  s.K = p.search_points ? (int)p.search_points : 8;
  s.rounds = p.search_rounds ? (int)p.search_rounds : 4;
  // bound the points a window keeps
  while (s.K * (1 + s.rounds) > kMaxPts && s.rounds > 0) --s.rounds;
  // plain: 1 grid + rounds refinements; narrow (hinted or learned): 1 grid +
  // hint_rounds refinements, then possibly the plain search
  const int hr = p.hint_rounds ? (int)p.hint_rounds : 2;
  const bool narrow = p.lambda_hint > 0 || (p.lambda_model && p.optimize_pgure);
  s.max_rounds = narrow ? (1 + hr) + (1 + s.rounds) : 1 + s.rounds;
  if (nfixed > 0) {  // one round over a given lambda list
    s.K = nfixed;
    s.rounds = 0;
    s.max_rounds = 1;
  }
  return s;
}

Problem make_problem(const pgsvt_params& p, const Setup& su) {
  Problem pb;
  pb.g = su.g;
  pb.W = 0;
  pb.K = su.K;
  pb.optimize = p.optimize_pgure ? 1 : 0;
  pb.expw = p.exp_weighting ? 1 : 0;
  pb.motion = p.motion_estimation ? 1 : 0;
  pb.compat = (int)p.compat_flags;
  pb.alpha_c = p.alpha;
  pb.mu_c = p.mu;
  pb.sigma_c = p.sigma;
  pb.lambda_user = p.lambda;
  pb.tol = p.tol;
  pb.max_evals = std::max<int>(1, (int)p.max_iter);
  pb.rounds = su.rounds;
  pb.hint = p.lambda_hint;
  pb.hint_span = p.hint_span > 1.0 ? p.hint_span : 2.0;
  pb.hint_K = std::min(su.K, p.hint_points ? (int)p.hint_points : 4);
  pb.hint_rounds = p.hint_rounds ? (int)p.hint_rounds : 2;
  pb.hint_flat = p.hint_flat > 0 ? p.hint_flat : 1e-3;
  pb.acc64 = 0;
  pb.svd_variant = svd_default_variant(pb.g.M, pb.g.NC);
  pb.fixed = nullptr;
  pb.nfixed = 0;
  pb.fixed_risk = nullptr;
  return pb;
}

// Bytes of device memory one window of a batch needs.
size_t window_bytes(const Problem& pb) {
  const Geometry& g = pb.g;
  const size_t C = g.cube(), NP = g.NP, NC = g.NC;
  size_t b = 0;
  b += C * 4;                       // u
  b += C * 12;                      // wz, w64 (median pre-filter; counted always)
  b += (size_t)g.nwin * g.P * 4;    // pos
  b += C * 4;                       // cnt
  b += C * 4 * 3;                   // fields
  b += NC * g.M * NP * 4;           // U0
  b += NC * g.nwin * NP * 4;        // V0
  b += 2 * 4 * NC * NP * 4 + NP * 4;  // sv, hv, nlive0
  if (svd_split_scratch(g.M, g.NC)) b += 4 * NP * NC * (16 + 1) * 4;  // xq, xqn
  b += (size_t)pb.K * C * (pb.acc64 ? 8 : 4);  // acc
  b += (size_t)pb.K * ((NP + 31) / 32 + mse_blocks(g)) * 8 + 256 * 8;  // partials
  b += sizeof(WinConst) + sizeof(SearchState) + 2 * (size_t)g.fw * sizeof(ArpsChain);
  return b;
}

// Batch buffers and bookkeeping of one stream.
struct Lane {
  cudaStream_t s = nullptr;
  bool own = false;
  DeviceBuffers d{};
  std::vector<int8_t> hp1, hp2;
  int8_t* pd1 = nullptr;
  int8_t* pd2 = nullptr;
  std::unique_ptr<StageClock> clk;
};

// The per-sequence engine.  X_dev holds the input (dtype) on the device.
// Windows are processed in batches of W; batches go round-robin to NS
// streams, so one batch's lambda search overlaps another batch's SVD.
// SVD kernel shape chosen by the autotuner per (patch rows, padded columns),
// process-wide.
std::mutex g_tune_mu;
std::map<std::pair<int, int>, int> g_tuned;

// Time every SVD kernel shape of this geometry on the batch at hand (second
// of two runs each) and keep the fastest; leaves the outputs of the chosen
// shape in place.
int tune_svd(Problem& pb, const DeviceBuffers& d, cudaStream_t s, Stats& stats) {
  const int nv = kSvdVariants;
  cudaEvent_t e0, e1;
  PGSVT_CK(cudaEventCreate(&e0));
  PGSVT_CK(cudaEventCreate(&e1));
  struct EG { cudaEvent_t a, b; ~EG() { cudaEventDestroy(a); cudaEventDestroy(b); } } eg{e0, e1};
  int best = 0, last = 0;
  float best_ms = 0.f;
  for (int v = 0; v < nv; ++v) {
    if (!svd_variant_ok(pb.g.M, pb.g.NC, v)) continue;
    pb.svd_variant = v;
    float ms = 0.f;
    for (int rep = 0; rep < 2; ++rep) {
      PGSVT_CK(cudaEventRecord(e0, s));
      check_launch(launch_svd(pb, d, s), stats);
      PGSVT_CK(cudaEventRecord(e1, s));
      PGSVT_CK(cudaEventSynchronize(e1));
      PGSVT_CK(cudaEventElapsedTime(&ms, e0, e1));
    }
    last = v;
    if (best_ms == 0.f || ms < best_ms) {
      best_ms = ms;
      best = v;
    }
  }
  pb.svd_variant = best;
  if (best != last) check_launch(launch_svd(pb, d, s), stats);
  return best;
}

void run_sequence(const void* X_dev, int dtype, int S, int nimg, double* Y_dev, double* est_dev,
                  const pgsvt_params& p, const pgsvt_outputs* out, cudaStream_t s, Stats& stats,
                  const double* fixed = nullptr, int nfixed = 0, double* fixed_risk = nullptr) {
  Setup su = make_setup(p, S, nimg, nfixed);
  Problem pb = make_problem(p, su);
  DevMem mem0;
  if (nfixed > 0) {
    double* f = mem0.arr<double>(nfixed);
    PGSVT_CK(cudaMemcpyAsync(f, fixed, sizeof(double) * nfixed, cudaMemcpyHostToDevice, s));
    PGSVT_CK(cudaStreamSynchronize(s));
    stats.h2d += sizeof(double) * nfixed;
    pb.fixed = f;
    pb.nfixed = nfixed;
    pb.fixed_risk = fixed_risk;
  }
  // SVD kernel shape: tuned once per process and geometry when asked
  const std::pair<int, int> tkey(pb.g.M, pb.g.NC);
  bool tune = false;
  if (p.autotune >= 2) {  // forced: shape autotune - 1 where the patch size has it
    const int v = (int)p.autotune - 1;
    pb.svd_variant = svd_variant_ok(pb.g.M, pb.g.NC, v) ? v : svd_default_variant(pb.g.M, pb.g.NC);
  } else if (p.autotune) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find(tkey);
    if (it != g_tuned.end()) pb.svd_variant = it->second;
    else tune = svd_variants(pb.g.M, pb.g.NC) > 1;
  }
  stats.svd_variant = pb.svd_variant;
  const Geometry& g = pb.g;
  DevMem mem;
  const size_t F = g.F(), C = g.cube();
  // sequence buffers
  float* xs = mem.arr<float>((size_t)nimg * F);
  double* x64 = (dtype == PGSVT_F64) ? mem.arr<double>((size_t)nimg * F) : nullptr;
  double* fmx = mem.arr<double>(nimg);
  StageClock clk0(s);
  clk0.mark(0);
  check_launch(launch_convert(X_dev, dtype, (size_t)nimg * F, xs, x64, s), stats);
  int* fint = mem.arr<int>(nimg);
  check_launch(launch_frame_max(xs, x64, nimg, F, fmx, s, fint), stats);
  clk0.mark(0);
  std::vector<double> hmax(nimg);
  std::vector<int> hint(nimg);
  PGSVT_CK(cudaMemcpyAsync(hmax.data(), fmx, sizeof(double) * nimg, cudaMemcpyDeviceToHost, s));
  PGSVT_CK(cudaMemcpyAsync(hint.data(), fint, sizeof(int) * nimg, cudaMemcpyDeviceToHost, s));
  PGSVT_CK(cudaStreamSynchronize(s));
  stats.d2h += (sizeof(double) + sizeof(int)) * nimg;
  int int_input = 1;  // ARPS integer mode for integer-valued inputs (arps.cu)
  for (int v : hint) int_input &= v;
  if (g.M > 64)
    for (double v : hmax) int_input &= (v <= 131072.0) ? 1 : 0;
  for (double v : hmax)
    if (v < 0) throw Fail(PGSVT_ERR_NONFINITE, "input holds negative, NaN or infinite values");
  // noise estimation tables per input frame (noise.cu)
  const bool estimate = pb.optimize && (p.alpha < 0 || p.mu < 0 || p.sigma < 0);
  NoiseFrames nf{};
  if (estimate) {
    nf.nlev = noise_levels(S);
    const int B = noise_blocks(nf.nlev);
    nf.maxNodes = 1 + 8 * B;
    int lbig = 0;  // levels of side >= 128, whose children can exceed 32
    for (int sz = S; sz >= 128; sz >>= 1) ++lbig;
    nf.maxBig = 1 + 8 * noise_blocks(lbig);
    const size_t nn = (size_t)nimg * nf.maxNodes;
    nf.split = mem.arr<uint8_t>(std::max<size_t>(1, (size_t)nimg * B));
    nf.nodes = mem.arr<int4>(nn);
    nf.isdel = mem.arr<uint8_t>(nn);
    nf.leaf = mem.arr<int4>(nn);
    nf.nleaf = mem.arr<int>(nimg);
    nf.big = mem.arr<int>(nn);
    nf.nbig = mem.arr<int>(nimg);
    nf.stats = mem.arr<double>(nn * 3);
    nf.dup = mem.arr<int>(nn);
    nf.first = mem.arr<int>((size_t)nimg * noise_blocks(nf.nlev + 1));
    nf.err = mem.arr<int>(1);
    PGSVT_CK(cudaMemsetAsync(nf.err, 0, sizeof(int), s));
    check_launch(launch_noise_frames(xs, x64, nimg, S, nf, s), stats, 6);
    int herr = 0;
    PGSVT_CK(cudaMemcpyAsync(&herr, nf.err, sizeof(int), cudaMemcpyDeviceToHost, s));
    PGSVT_CK(cudaStreamSynchronize(s));
    if (herr) throw Fail(PGSVT_ERR_CUDA, "noise estimation: quadtree replay overflow");
  }
  // median pre-filter of the ARPS input (pguresvt.hpp:69-84)
  float* zs = nullptr;
  double* zmx = nullptr;
  if (p.median_size > 0) {
    zs = mem.arr<float>((size_t)nimg * F);
    zmx = mem.arr<double>(nimg);
    check_launch(launch_median(xs, x64, nimg, S, (int)p.median_size, zs, s), stats);
    check_launch(launch_frame_max(zs, nullptr, nimg, F, zmx, s), stats);
  }

  const int ncopies = !pb.optimize ? 1 : ((pb.compat & PGSVT_COMPAT_INT_DELTA1) ? 3 : 4);
  // zero-motion quirk: every patch lands on the (0,0) block of the other
  // slices, beyond the int32 range
  pb.acc64 = (!pb.motion && (pb.compat & PGSVT_COMPAT_ZERO_MOTION)) ? 1 : 0;
  int fb = (int)p.frame_begin, fe = (int)p.frame_end;
  if (fb == 0 && fe == 0) fe = nimg;
  if (fb < 0 || fe > nimg || fb >= fe) throw Fail(PGSVT_ERR_INVALID_ARG, "bad frame range");
  const int nwinds = fe - fb;
  // noise estimates of every window before the batches (noise.cu): leaf
  // means once per (frame, window maximum) pair, then one fit per window
  double* est_win = nullptr;
  if (estimate) {
    std::vector<int> win_s0(nwinds), win_pair((size_t)nwinds * g.nwin), pair_frame;
    std::vector<double> win_norm(nwinds), pair_norm;
    std::map<std::pair<int, double>, int> pid;
    for (int k = 0; k < nwinds; ++k) {
      const int t = fb + k;
      const int s0 = t < g.fw ? 0 : (t >= nimg - g.fw ? nimg - 2 * g.fw - 1 : t - g.fw);
      double um = hmax[s0];
      for (int q = 1; q < g.nwin; ++q) um = std::max(um, hmax[s0 + q]);
      um = um > 0.0 ? um : 1.0;  // the window's normalisation (WinConst::unorm)
      win_s0[k] = s0;
      win_norm[k] = um;
      for (int q = 0; q < g.nwin; ++q) {
        const auto key = std::make_pair(s0 + q, um);
        auto it = pid.find(key);
        if (it == pid.end()) {
          it = pid.emplace(key, (int)pair_frame.size()).first;
          pair_frame.push_back(s0 + q);
          pair_norm.push_back(um);
        }
        win_pair[(size_t)k * g.nwin + q] = it->second;
      }
    }
    NoisePass np{};
    np.method = (int)p.noise_method;
    np.npairs = (int)pair_frame.size();
    np.nwin = g.nwin;
    np.alpha_c = p.alpha;
    np.mu_c = p.mu;
    np.sigma_c = p.sigma;
    auto up = [&](const auto& v) {
      using T = typename std::decay_t<decltype(v)>::value_type;
      T* dptr = mem.arr<T>(v.size());
      PGSVT_CK(cudaMemcpyAsync(dptr, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, s));
      stats.h2d += sizeof(T) * v.size();
      return dptr;
    };
    np.pair_frame = up(pair_frame);
    np.pair_norm = up(pair_norm);
    np.mean = mem.arr<double>((size_t)np.npairs * nf.maxNodes);
    int* d_win_pair = up(win_pair);
    int* d_win_s0 = up(win_s0);
    double* d_win_norm = up(win_norm);
    est_win = mem.arr<double>((size_t)nwinds * 3);
    // windows in chunks, the fit scratch reused
    const int chunk = std::min(nwinds, 64);
    const size_t per_w = (size_t)g.nwin * nf.maxNodes;
    np.x = mem.arr<double>(chunk * per_w);
    np.y = mem.arr<double>(chunk * per_w);
    np.key = mem.arr<unsigned long long>(chunk * per_w);
    np.hist = mem.arr<int>(chunk * (per_w + 1));
    np.fkey = mem.arr<unsigned long long>(chunk * (per_w + 1));
    np.fidx = mem.arr<int>(chunk * (per_w + 1));
    for (int k0 = 0; k0 < nwinds; k0 += chunk) {
      NoisePass npc = np;
      npc.nwindows = std::min(chunk, nwinds - k0);
      npc.win_pair = d_win_pair + (size_t)k0 * g.nwin;
      npc.win_s0 = d_win_s0 + k0;
      npc.win_norm = d_win_norm + k0;
      npc.est = est_win + (size_t)k0 * 3;
      if (k0 > 0) npc.npairs = 0;  // the leaf means are computed once
      check_launch(launch_noise_pass(nf, npc, xs, x64, S, s), stats, k0 > 0 ? 1 : 3);
    }
    PGSVT_CK(cudaStreamSynchronize(s));  // the host vectors go out of scope
  }
  // batch size: about half a million kept patches per batch
  int W = p.window_batch ? (int)p.window_batch
                         : (int)std::max<int64_t>(1, (500000 + g.NP - 1) / (int64_t)g.NP);
  W = std::max(1, std::min({W, nwinds, 32}));
  const int nbatches = (nwinds + W - 1) / W;
  int NS = std::min(3, nbatches);
  size_t freeb = 0, totb = 0;
  PGSVT_CK(cudaMemGetInfo(&freeb, &totb));
  const size_t per = window_bytes(pb);
  while (NS > 1 && (size_t)NS * W * per > freeb / 2) --NS;
  while (W > 1 && (size_t)NS * W * per > freeb / 2) --W;
  if ((size_t)NS * W * per > freeb) throw Fail(PGSVT_ERR_OOM, "not enough device memory for one window");

  // sequence-level tables shared by the streams
  int32_t* plist = mem.arr<int32_t>(g.NP);
  PGSVT_CK(cudaMemcpyAsync(plist, su.plist.data(), sizeof(int32_t) * g.NP, cudaMemcpyHostToDevice, s));
  stats.h2d += sizeof(int32_t) * g.NP;
  const int nchains = 2 * g.fw;
  std::vector<ArpsChain> hch((size_t)nimg * nchains);
  for (int t = 0; t < nimg; ++t) {
    auto c = chains_for(t, g.fw, nimg, g.nwin);
    std::copy(c.begin(), c.end(), hch.begin() + (size_t)t * nchains);
  }
  ArpsChain* dch = mem.arr<ArpsChain>(hch.size());
  PGSVT_CK(cudaMemcpyAsync(dch, hch.data(), sizeof(ArpsChain) * hch.size(), cudaMemcpyHostToDevice, s));
  stats.h2d += sizeof(ArpsChain) * hch.size();
  unsigned long long* counters = mem.arr<unsigned long long>(5);
  PGSVT_CK(cudaMemsetAsync(counters, 0, 5 * sizeof(unsigned long long), s));
  const double vP = probe_vp();
  const bool shared_probes = p.random_seed >= 0;
  int8_t* sp1 = nullptr;
  int8_t* sp2 = nullptr;
  if (pb.optimize && shared_probes) {  // one probe set for every window (pgure.hpp:52-59)
    std::vector<int8_t> h1(C), h2(C);
    make_probes(p.random_seed, C, h1.data(), h2.data());
    sp1 = mem.arr<int8_t>(C);
    sp2 = mem.arr<int8_t>(C);
    PGSVT_CK(cudaMemcpyAsync(sp1, h1.data(), C, cudaMemcpyHostToDevice, s));
    PGSVT_CK(cudaMemcpyAsync(sp2, h2.data(), C, cudaMemcpyHostToDevice, s));
    PGSVT_CK(cudaStreamSynchronize(s));  // h1/h2 go out of scope
    stats.h2d += 2 * C;
  }
  if (fb > 0 || fe < nimg) {
    PGSVT_CK(cudaMemsetAsync(Y_dev, 0, sizeof(double) * (size_t)nimg * F, s));
    PGSVT_CK(cudaMemsetAsync(est_dev, 0, sizeof(double) * (size_t)nimg * 4, s));
  }
  // learned lambda proposal: model, its bf16 shadow, the sampled patch slots
  const bool use_model = pb.optimize && p.lambda_model && pb.nfixed == 0;
  const bool want_feat = use_model || (out && out->lambda_features);
  float* dmodel = nullptr;
  void* dmodel_bf = nullptr;
  int32_t* fslots = nullptr;
  int nfslots = 0;
  if (use_model) {
    dmodel = mem.arr<float>(PGSVT_LAMBDA_MODEL_FLOATS);
    dmodel_bf = mem.get(PGSVT_LAMBDA_MODEL_FLOATS * 2);
    PGSVT_CK(cudaMemcpyAsync(dmodel, p.lambda_model, sizeof(float) * PGSVT_LAMBDA_MODEL_FLOATS,
                             cudaMemcpyHostToDevice, s));
    stats.h2d += sizeof(float) * PGSVT_LAMBDA_MODEL_FLOATS;
    check_launch(lambda_shadow(dmodel, dmodel_bf, s), stats);
    PGSVT_CK(lambda_attrs());
  }
  if (want_feat) {
    const std::vector<int32_t> fs = feature_slots(su.sorted, su.plist, g.P);
    nfslots = (int)fs.size();
    fslots = mem.arr<int32_t>(fs.size());
    PGSVT_CK(cudaMemcpyAsync(fslots, fs.data(), sizeof(int32_t) * fs.size(), cudaMemcpyHostToDevice, s));
    PGSVT_CK(cudaStreamSynchronize(s));  // fs goes out of scope
    stats.h2d += sizeof(int32_t) * fs.size();
  }
  if (out && out->lambda_proposals && !use_model)  // all-ones bytes: NaN
    PGSVT_CK(cudaMemsetAsync(out->lambda_proposals, 0xff, sizeof(float) * nimg, s));
  cudaEvent_t ready;
  PGSVT_CK(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
  struct EvGuard { cudaEvent_t e; ~EvGuard() { cudaEventDestroy(e); } } evg{ready};
  PGSVT_CK(cudaEventRecord(ready, s));

  std::vector<Lane> lanes(NS);
  struct LaneGuard {
    std::vector<Lane>& l;
    ~LaneGuard() {
      for (auto& x : l) {
        x.clk.reset();
        if (x.own && x.s) cudaStreamDestroy(x.s);
      }
    }
  } lg{lanes};
  for (int li = 0; li < NS; ++li) {
    Lane& L = lanes[li];
    if (li == 0) {
      L.s = s;
    } else {
      PGSVT_CK(cudaStreamCreateWithFlags(&L.s, cudaStreamNonBlocking));
      L.own = true;
      PGSVT_CK(cudaStreamWaitEvent(L.s, ready, 0));
    }
    L.clk.reset(new StageClock(L.s));
    DeviceBuffers& d = L.d;
    d.xs = xs;
    d.x64 = x64;
    d.fmax = fmx;
    d.zs = zs;
    d.zmax = zmx;
    d.int_input = int_input;
    if (zs) {
      d.wz = mem.arr<float>((size_t)W * C);
      d.w64 = mem.arr<double>((size_t)W * C);
    }
    d.plist = plist;
    d.counters = counters;
    d.Y = Y_dev;
    d.est = est_dev;
    d.ncopies = ncopies;
    d.nchains = nchains;
    d.d2neg = -1 * std::sqrt((1 - vP) / vP);
    d.d2pos = std::sqrt(vP / (1 - vP));
    d.u = mem.arr<float>((size_t)W * C);
    d.pos = mem.arr<uint32_t>((size_t)W * g.nwin * g.P);
    d.cnt = mem.arr<int32_t>((size_t)W * C);
    if (pb.optimize) {
      d.fld0 = mem.arr<float>((size_t)W * C);
      d.fld2 = mem.arr<float>((size_t)W * C);
      d.fld1 = (ncopies == 4) ? mem.arr<float>((size_t)W * C) : nullptr;
    }
    d.U0 = mem.arr<float>((size_t)W * g.NC * g.M * g.NP);
    d.V0 = mem.arr<float>((size_t)W * g.NC * g.nwin * g.NP);
    d.sv = mem.arr<float>((size_t)W * 4 * g.NC * g.NP);
    d.hv = mem.arr<float>((size_t)W * 4 * g.NC * g.NP);
    d.nlive0 = mem.arr<int32_t>((size_t)W * g.NP);
    if (svd_split_scratch(g.M, g.NC)) {
      const size_t items = (size_t)W * ncopies * g.NP;
      d.xq = mem.arr<float>(items * g.NC * 16);
      d.xqn = mem.arr<float>(items * g.NC);
    }
    PGSVT_CK(cudaMemsetAsync(d.hv, 0, sizeof(float) * (size_t)W * 4 * g.NC * g.NP, L.s));
    const size_t accb = (size_t)W * pb.K * C * (pb.acc64 ? 8 : 4);
    d.acc = mem.get(accb);
    PGSVT_CK(cudaMemsetAsync(d.acc, 0, accb, L.s));
    d.nblk_eval = eval_blocks(g);
    d.nblk_mse = mse_blocks(g);
    d.part_lin = mem.arr<double>((size_t)W * pb.K * d.nblk_eval);
    d.part_mse = mem.arr<double>(std::max<size_t>((size_t)W * pb.K * d.nblk_mse, (size_t)W * 256));
    d.wc = mem.arr<WinConst>(W);
    d.st = mem.arr<SearchState>(W);

    d.model = dmodel;
    d.model_bf16 = dmodel_bf;
    d.feat_slots = fslots;
    d.nfeat_slots = nfslots;
    if (want_feat) {
      d.feat = mem.arr<float>((size_t)W * PGSVT_LAMBDA_FEATURES);
      d.prop = mem.arr<float>(W);
    }
    if (out) {
      d.feat_out = out->lambda_features;
      d.prop_out = use_model ? out->lambda_proposals : nullptr;
      d.risk_out = out->risk;
      d.evals_out = out->risk_evals;
    }
    if (pb.optimize) {
      if (shared_probes) {
        d.d1 = sp1;
        d.d2code = sp2;
        d.probe_stride = 0;
      } else {  // fresh entropy per window (pgure.hpp:54-55)
        L.pd1 = mem.arr<int8_t>((size_t)W * C);
        L.pd2 = mem.arr<int8_t>((size_t)W * C);
        L.hp1.resize((size_t)W * C);
        L.hp2.resize((size_t)W * C);
        d.d1 = L.pd1;
        d.d2code = L.pd2;
        d.probe_stride = C;
      }
    }
  }

  int bi = 0;
  for (int win0 = fb; win0 < fe; win0 += W, ++bi) {
    Lane& L = lanes[bi % NS];
    DeviceBuffers& d = L.d;
    Problem pbb = pb;
    pbb.W = std::min(W, fe - win0);
    d.win0 = win0;
    d.chains = dch + (size_t)win0 * nchains;
    StageClock& clk = *L.clk;
    if (pb.optimize && !shared_probes) {
      PGSVT_CK(cudaStreamSynchronize(L.s));  // the lane's host buffers are reused
      for (int w = 0; w < pbb.W; ++w)
        make_probes(-1, C, L.hp1.data() + (size_t)w * C, L.hp2.data() + (size_t)w * C);
      PGSVT_CK(cudaMemcpyAsync(L.pd1, L.hp1.data(), (size_t)pbb.W * C, cudaMemcpyHostToDevice, L.s));
      PGSVT_CK(cudaMemcpyAsync(L.pd2, L.hp2.data(), (size_t)pbb.W * C, cudaMemcpyHostToDevice, L.s));
      stats.h2d += 2 * (size_t)pbb.W * C;
    }
    clk.mark(7);  // probe uploads and other gaps
    check_launch(launch_window_setup(pbb, d, L.s), stats, 2);
    if (estimate) check_launch(launch_noise_apply(pbb, d, est_win, fb, L.s), stats);
    clk.mark(1);
    check_launch(launch_arps(pbb, d, L.s), stats, pbb.motion ? 2 : 1);
    clk.mark(2);
    check_launch(launch_fields(pbb, d, L.s), stats, 4);
    check_launch(launch_search_init(pbb, d, L.s), stats);  // sets the lambda range
    clk.mark(3);
    if (tune) {
      const int v = tune_svd(pbb, d, L.s, stats);
      pb.svd_variant = v;
      stats.svd_variant = v;
      stats.svd_tuned = 1;
      tune = false;
      std::lock_guard<std::mutex> lk(g_tune_mu);
      g_tuned[tkey] = v;
    } else {
      check_launch(launch_svd(pbb, d, L.s), stats);
    }
    clk.mark(4);
    stats.svd_launches += 1;
    stats.svd_matrices += (uint64_t)pbb.W * ncopies * g.NP;
    stats.windows += pbb.W;
    if (want_feat) {
      check_launch(launch_lambda_features(pbb, d, L.s), stats);
      if (d.feat_out)
        PGSVT_CK(cudaMemcpyAsync(d.feat_out + (size_t)win0 * PGSVT_LAMBDA_FEATURES, d.feat,
                                 sizeof(float) * PGSVT_LAMBDA_FEATURES * pbb.W,
                                 cudaMemcpyDeviceToDevice, L.s));
    }
    if (use_model) {
      check_launch(launch_lambda_propose(pbb, d, L.s), stats);
      check_launch(launch_search_hint(pbb, d, L.s), stats);
    }
    if (pbb.optimize)
      for (int r = 0; r < su.max_rounds; ++r) check_launch(launch_eval_round(pbb, d, 0, L.s), stats, 3);
    clk.mark(5);
    check_launch(launch_eval_round(pbb, d, 1, L.s), stats);
    check_launch(launch_output(pbb, d, L.s), stats);
    clk.mark(6);
  }
  // the caller's stream completes after every lane
  for (int li = 1; li < NS; ++li) {
    cudaEvent_t e;
    PGSVT_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    PGSVT_CK(cudaEventRecord(e, lanes[li].s));
    PGSVT_CK(cudaStreamWaitEvent(s, e, 0));
    cudaEventDestroy(e);
  }
  unsigned long long cnt[5];
  PGSVT_CK(cudaMemcpyAsync(cnt, counters, sizeof(cnt), cudaMemcpyDeviceToHost, s));
  PGSVT_CK(cudaStreamSynchronize(s));
  stats.d2h += sizeof(cnt);
  if (cnt[4])
    throw Fail(PGSVT_ERR_TIMEOUT, "SVD factors: a staged tile copy did not complete in time");
  stats.evals += cnt[3];
  stats.arps_exact += cnt[0];
  stats.svd_sweeps += cnt[1];
  stats.svd_fp64 += cnt[2];
  clk0.accumulate(stats.stage);
  for (auto& L : lanes) L.clk->accumulate(stats.stage);
  if (p.verbose)
    std::fprintf(stderr, "pgsvt: %dx%dx%d, bs=%d, nwin=%d, patches=%d, batch=%d x %d streams, "
                         "arps fp64 steps=%llu, svd warp-sweeps=%llu, fp64 tests=%llu\n",
                 S, S, nimg, g.bs, g.nwin, g.NP, W, NS, cnt[0], cnt[1], cnt[2]);
}

template <typename Fn>
int guarded(pgsvt_status* st, Fn&& fn) {
  const auto t0 = std::chrono::steady_clock::now();
  Stats stats;
  int code = PGSVT_OK, cuda = 0;
  g_err.clear();
  try {
    fn(stats);
  } catch (const Fail& f) {
    code = f.code;
    cuda = f.cuda;
    g_err = f.what();
  } catch (const std::exception& e) {
    code = PGSVT_ERR_CUDA;
    g_err = e.what();
  }
  if (st) {
    st->code = code;
    st->cuda_error = cuda;
    st->kernel_launches = stats.launches;
    st->h2d_bytes = stats.h2d;
    st->d2h_bytes = stats.d2h;
    st->risk_evals = stats.evals;
    st->windows = stats.windows;
    for (int i = 0; i < 8; ++i) st->stage_seconds[i] = stats.stage[i];
    st->svd_launches = stats.svd_launches;
    st->svd_matrices = stats.svd_matrices;
    st->arps_exact_steps = stats.arps_exact;
    st->svd_fp64_tests = stats.svd_fp64;
    st->svd_warp_sweeps = stats.svd_sweeps;
    st->svd_variant = stats.svd_variant;
    st->svd_tuned = stats.svd_tuned;
    st->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::snprintf(st->message, sizeof(st->message), "%s", g_err.c_str());
  }
  return code;
}

size_t dtype_size(int dtype) {
  switch (dtype) {
    case PGSVT_U8: return 1;
    case PGSVT_U16: return 2;
    case PGSVT_F32: return 4;
    case PGSVT_F64: return 8;
    default: throw Fail(PGSVT_ERR_INVALID_ARG, "Invalid dtype");
  }
}

void need_device() {
  int n = 0;
  const cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0)
    throw Fail(PGSVT_ERR_CUDA, "no CUDA device available (this library has no CPU path)", (int)e);
}

// Host-memory denoise of one sequence on its own stream (pgsvt_denoise_ex and
// the batch workers).  `fixed`/`nfixed`: a lambda list evaluated instead of
// the search, `risks` its per-frame risks (host, nframes x nfixed).
void denoise_host(const void* X, int32_t dtype, uint32_t nrows, uint32_t ncols, uint32_t nframes,
                  double* Y, double* estimates, const pgsvt_params& p, const pgsvt_outputs* out,
                  const double* fixed, int nfixed, double* risks, Stats& stats) {
  const size_t es = dtype_size(dtype);
  validate(p, nrows, ncols, nframes);
  if (nfixed > 0 && !p.optimize_pgure)
    throw Fail(PGSVT_ERR_INVALID_ARG, "a lambda list needs optimize_pgure (its risks are PGURE)");
  if (nfixed > kMaxK) throw Fail(PGSVT_ERR_INVALID_ARG, "more than 16 lambda values");
  const size_t n = (size_t)nrows * ncols * nframes;
  DevMem mem;
  cudaStream_t s;
  PGSVT_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct SG { cudaStream_t s; ~SG() { cudaStreamDestroy(s); } } sg{s};
  void* Xd = mem.get(n * es);
  double* Yd = mem.arr<double>(n);
  double* Ed = mem.arr<double>((size_t)nframes * 4);
  pgsvt_outputs od{};  // device twins of the requested per-frame outputs
  const size_t nf = nframes, nfe = nf * PGSVT_LAMBDA_FEATURES;
  if (out) {
    if (out->lambda_features) od.lambda_features = mem.arr<float>(nfe);
    if (out->lambda_proposals) od.lambda_proposals = mem.arr<float>(nf);
    if (out->risk) od.risk = mem.arr<double>(nf);
    if (out->risk_evals) od.risk_evals = mem.arr<uint32_t>(nf);
    if (od.lambda_features) PGSVT_CK(cudaMemsetAsync(od.lambda_features, 0, nfe * 4, s));
    if (od.risk) PGSVT_CK(cudaMemsetAsync(od.risk, 0, nf * 8, s));
    if (od.risk_evals) PGSVT_CK(cudaMemsetAsync(od.risk_evals, 0, nf * 4, s));
    if (od.lambda_proposals) PGSVT_CK(cudaMemsetAsync(od.lambda_proposals, 0xff, nf * 4, s));
  }
  double* rd = nullptr;
  if (risks && nfixed > 0) {
    rd = mem.arr<double>(nf * nfixed);
    PGSVT_CK(cudaMemsetAsync(rd, 0, nf * nfixed * 8, s));
  }
  PGSVT_CK(cudaMemcpyAsync(Xd, X, n * es, cudaMemcpyHostToDevice, s));
  stats.h2d += n * es;
  run_sequence(Xd, dtype, (int)nrows, (int)nframes, Yd, Ed, p, out ? &od : nullptr, s, stats,
               fixed, nfixed, rd);
  PGSVT_CK(cudaMemcpyAsync(Y, Yd, n * sizeof(double), cudaMemcpyDeviceToHost, s));
  PGSVT_CK(cudaMemcpyAsync(estimates, Ed, (size_t)nframes * 4 * sizeof(double),
                           cudaMemcpyDeviceToHost, s));
  stats.d2h += n * sizeof(double) + (size_t)nframes * 4 * sizeof(double);
  auto back = [&](void* h, const void* d, size_t b) {
    if (!h) return;
    PGSVT_CK(cudaMemcpyAsync(h, d, b, cudaMemcpyDeviceToHost, s));
    stats.d2h += b;
  };
  if (out) {
    back(out->lambda_features, od.lambda_features, nfe * 4);
    back(out->lambda_proposals, od.lambda_proposals, nf * 4);
    back(out->risk, od.risk, nf * 8);
    back(out->risk_evals, od.risk_evals, nf * 4);
  }
  if (rd) back(risks, rd, nf * nfixed * 8);
  PGSVT_CK(cudaStreamSynchronize(s));
}

// ---------------------------------------------------------------------------
// Single-window pipeline for the component entry points: the window itself is
// uploaded as an FP64 "sequence" of nwin slices, and the window constants come
// from the host.

struct OneWindow {
  DevMem mem;
  Problem pb;
  DeviceBuffers d{};
  Setup su;
  cudaStream_t s = nullptr;
  Stats stats;

  OneWindow(const double* u, uint32_t S, uint32_t nwin, const pgsvt_params& p, int ref,
            int out_slice) {
    need_device();
    if (nwin % 2 == 0 || nwin < 1) throw Fail(PGSVT_ERR_INVALID_ARG, "nwin must be odd");
    if (S < p.block_size || p.block_size < 2 || p.block_size > 8)
      throw Fail(PGSVT_ERR_INVALID_ARG, "bad block size");
    if (!svd_supported((int)p.block_size, (int)nwin))
      throw Fail(PGSVT_ERR_UNSUPPORTED, "window above 21 frames");
    pgsvt_params q = p;
    q.traj_length = nwin;  // the caller gives the window directly
    if (p.block_size * p.block_size <= nwin) throw Fail(PGSVT_ERR_INVALID_ARG, "window too long for bs");
    su = make_setup(q, (int)S, (int)nwin);
    pb = make_problem(q, su);
    pb.W = 1;
    PGSVT_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    const Geometry& g = pb.g;
    const size_t C = g.cube();
    double* x64 = mem.arr<double>(C);
    float* xs = mem.arr<float>(C);
    PGSVT_CK(cudaMemcpyAsync(x64, u, C * sizeof(double), cudaMemcpyHostToDevice, s));
    check_launch(launch_convert(x64, PGSVT_F64, C, xs, nullptr, s), stats);
    d.xs = xs;
    d.x64 = x64;
    double umax = u[0];
    for (size_t i = 1; i < C; ++i) umax = std::max(umax, u[i]);
    WinConst wc{};
    wc.umax = umax;
    wc.unorm = umax > 0 ? umax : 1.0;
    wc.t = 0;
    wc.s0 = 0;
    wc.ref = ref;
    wc.out_slice = out_slice;
    wc.alpha = p.alpha;
    if (p.compat_flags & PGSVT_COMPAT_SWAP_MU_SIGMA) {
      wc.mu = p.sigma;
      wc.sigma = p.mu;
    } else {
      wc.mu = p.mu;
      wc.sigma = p.sigma;
    }
    wc.eps1 = (umax > 0 ? umax / umax : 1.0) * 0.0001;
    wc.eps2 = 100 * wc.eps1;
    d.wc = mem.arr<WinConst>(1);
    PGSVT_CK(cudaMemcpyAsync(d.wc, &wc, sizeof(wc), cudaMemcpyHostToDevice, s));
    d.u = mem.arr<float>(C);
    d.pos = mem.arr<uint32_t>((size_t)g.nwin * g.P);
    int32_t* plist = mem.arr<int32_t>(g.NP);
    PGSVT_CK(cudaMemcpyAsync(plist, su.plist.data(), sizeof(int32_t) * g.NP, cudaMemcpyHostToDevice, s));
    d.plist = plist;
    d.cnt = mem.arr<int32_t>(C);
    d.counters = mem.arr<unsigned long long>(5);
    PGSVT_CK(cudaMemsetAsync(d.counters, 0, 5 * sizeof(unsigned long long), s));
    d.nchains = 2 * g.fw;
    const double vP = probe_vp();
    d.d2neg = -1 * std::sqrt((1 - vP) / vP);
    d.d2pos = std::sqrt(vP / (1 - vP));
    d.nblk_eval = eval_blocks(g);
    d.nblk_mse = mse_blocks(g);
    check_launch(launch_window_norm_only(pb, d, s), stats);
  }
  ~OneWindow() {
    if (s) cudaStreamDestroy(s);
  }

  void set_positions(const int32_t* rows, const int32_t* cols) {
    const Geometry& g = pb.g;
    std::vector<uint32_t> h((size_t)g.nwin * g.P);
    for (size_t i = 0; i < h.size(); ++i) {
      if (rows[i] < 0 || cols[i] < 0 || rows[i] + g.bs > g.S || cols[i] + g.bs > g.S)
        throw Fail(PGSVT_ERR_INVALID_ARG, "trajectory position outside the frame");
      h[i] = (uint32_t)rows[i] | ((uint32_t)cols[i] << 16);
    }
    PGSVT_CK(cudaMemcpyAsync(d.pos, h.data(), h.size() * 4, cudaMemcpyHostToDevice, s));
    PGSVT_CK(cudaStreamSynchronize(s));
  }

  void alloc_factors(int ncopies) {
    const Geometry& g = pb.g;
    d.ncopies = ncopies;
    d.U0 = mem.arr<float>((size_t)g.NC * g.M * g.NP);
    d.V0 = mem.arr<float>((size_t)g.NC * g.nwin * g.NP);
    d.sv = mem.arr<float>((size_t)4 * g.NC * g.NP);
    d.hv = mem.arr<float>((size_t)4 * g.NC * g.NP);
    d.nlive0 = mem.arr<int32_t>(g.NP);
    if (svd_split_scratch(g.M, g.NC)) {
      d.xq = mem.arr<float>((size_t)ncopies * g.NP * g.NC * 16);
      d.xqn = mem.arr<float>((size_t)ncopies * g.NP * g.NC);
    }
    PGSVT_CK(cudaMemsetAsync(d.hv, 0, sizeof(float) * 4 * g.NC * g.NP, s));
    pb.acc64 = 1;  // a caller-given trajectory table may stack any number of patches
    d.acc = mem.get(sizeof(unsigned long long) * pb.K * g.cube());
    PGSVT_CK(cudaMemsetAsync(d.acc, 0, sizeof(unsigned long long) * pb.K * g.cube(), s));
    d.part_lin = mem.arr<double>((size_t)pb.K * d.nblk_eval);
    d.part_mse = mem.arr<double>(std::max<size_t>((size_t)pb.K * d.nblk_mse, 256));
    d.st = mem.arr<SearchState>(1);
  }
};

}  // namespace

namespace pgsvt {
void set_last_error(const std::string& m) { g_err = m; }
}  // namespace pgsvt

extern "C" {

int pgsvt_default_params(pgsvt_params* p) {
  if (!p) return PGSVT_ERR_INVALID_ARG;
  std::memset(p, 0, sizeof(*p));
  p->traj_length = 15;
  p->block_size = 4;
  p->block_overlap = 1;
  p->motion_window = 7;
  p->median_size = 5;
  p->noise_method = 4;
  p->max_iter = 500;
  p->n_jobs = -1;
  p->random_seed = -1;
  p->optimize_pgure = 1;
  p->exp_weighting = 1;
  p->motion_estimation = 1;
  p->verbose = 0;
  p->lambda = -1.0;
  p->alpha = -1.0;
  p->mu = -1.0;
  p->sigma = -1.0;
  p->tol = 1e-7;
  p->compat_flags = PGSVT_COMPAT_ALL;
  p->search_points = 8;
  p->search_rounds = 4;
  p->window_batch = 0;
  p->lambda_hint = -1.0;
  p->hint_span = 2.0;
  p->frame_begin = 0;
  p->frame_end = 0;
  p->lambda_model = nullptr;
  p->hint_points = 4;
  p->hint_rounds = 2;
  p->hint_flat = 1e-3;
  p->autotune = 0;
  return PGSVT_OK;
}

int pgsvt_denoise_device_ex(const void* X_dev, int32_t dtype, uint32_t nrows, uint32_t ncols,
                            uint32_t nframes, double* Y_dev, double* est_dev,
                            const pgsvt_params* p, const pgsvt_outputs* out_dev, void* stream,
                            pgsvt_status* st) {
  return guarded(st, [&](Stats& stats) {
    if (!X_dev || !Y_dev || !est_dev || !p) throw Fail(PGSVT_ERR_INVALID_ARG, "null pointer");
    need_device();
    dtype_size(dtype);
    validate(*p, nrows, ncols, nframes);
    cudaStream_t s = (cudaStream_t)stream;
    run_sequence(X_dev, dtype, (int)nrows, (int)nframes, Y_dev, est_dev, *p, out_dev, s, stats);
  });
}

int pgsvt_denoise_device(const void* X_dev, int32_t dtype, uint32_t nrows, uint32_t ncols,
                         uint32_t nframes, double* Y_dev, double* est_dev, const pgsvt_params* p,
                         void* stream, pgsvt_status* st) {
  return pgsvt_denoise_device_ex(X_dev, dtype, nrows, ncols, nframes, Y_dev, est_dev, p, nullptr,
                                 stream, st);
}

int pgsvt_denoise_ex(const void* X, int32_t dtype, uint32_t nrows, uint32_t ncols,
                     uint32_t nframes, double* Y, double* estimates, const pgsvt_params* p,
                     const pgsvt_outputs* out, pgsvt_status* st) {
  return guarded(st, [&](Stats& stats) {
    if (!X || !Y || !estimates || !p) throw Fail(PGSVT_ERR_INVALID_ARG, "null pointer");
    need_device();
    denoise_host(X, dtype, nrows, ncols, nframes, Y, estimates, *p, out, nullptr, 0, nullptr,
                 stats);
  });
}

int pgsvt_denoise(const void* X, int32_t dtype, uint32_t nrows, uint32_t ncols, uint32_t nframes,
                  double* Y, double* estimates, const pgsvt_params* p, pgsvt_status* st) {
  return pgsvt_denoise_ex(X, dtype, nrows, ncols, nframes, Y, estimates, p, nullptr, st);
}

int pgsvt_denoise_batch(const pgsvt_sequence* seqs, uint32_t nseq, uint32_t slots,
                        pgsvt_status* st) {
  return guarded(st, [&](Stats& total) {
    if (!seqs && nseq) throw Fail(PGSVT_ERR_INVALID_ARG, "null pointer");
    for (uint32_t i = 0; i < nseq; ++i)
      if (!seqs[i].X || !seqs[i].Y || !seqs[i].estimates || !seqs[i].params)
        throw Fail(PGSVT_ERR_INVALID_ARG, "null pointer in sequence " + std::to_string(i));
    if (nseq == 0) return;
    need_device();
    int dev = 0;
    PGSVT_CK(cudaGetDevice(&dev));
    // largest first, so the queue's tail holds the short sequences
    std::vector<uint32_t> order(nseq);
    for (uint32_t i = 0; i < nseq; ++i) order[i] = i;
    auto cost = [&](uint32_t i) {
      const pgsvt_sequence& q = seqs[i];
      return (double)q.nrows * q.ncols * q.nframes * (double)q.params->block_size;
    };
    std::stable_sort(order.begin(), order.end(),
                     [&](uint32_t a, uint32_t b) { return cost(a) > cost(b); });
    const int nw = (int)std::min<uint32_t>(nseq, slots ? slots : 2);
    std::atomic<uint32_t> next{0};
    std::vector<Stats> part(nw);
    std::vector<int> codes(nseq, PGSVT_OK), cudas(nseq, 0);
    std::vector<std::string> msgs(nseq);
    auto worker = [&](int wi) {
      cudaSetDevice(dev);
      for (;;) {
        const uint32_t k = next.fetch_add(1);
        if (k >= nseq) break;
        const uint32_t i = order[k];
        const pgsvt_sequence& q = seqs[i];
        const int rc = guarded(q.status, [&](Stats& stats) {
          denoise_host(q.X, q.dtype, q.nrows, q.ncols, q.nframes, q.Y, q.estimates, *q.params,
                       nullptr, q.lambdas, (int)q.nlambdas, q.risks, stats);
          Stats& P = part[wi];
          P.launches += stats.launches;
          P.h2d += stats.h2d;
          P.d2h += stats.d2h;
          P.evals += stats.evals;
          P.windows += stats.windows;
          P.svd_launches += stats.svd_launches;
          P.svd_matrices += stats.svd_matrices;
          P.arps_exact += stats.arps_exact;
          P.svd_fp64 += stats.svd_fp64;
          P.svd_sweeps += stats.svd_sweeps;
          P.svd_tuned |= stats.svd_tuned;
          for (int j = 0; j < 8; ++j) P.stage[j] += stats.stage[j];
        });
        codes[i] = rc;
        if (rc != PGSVT_OK) msgs[i] = "sequence " + std::to_string(i) + ": " + g_err;
      }
    };
    std::vector<std::thread> th;
    for (int wi = 1; wi < nw; ++wi) th.emplace_back(worker, wi);
    worker(0);
    for (auto& t : th) t.join();
    for (const Stats& P : part) {
      total.launches += P.launches;
      total.h2d += P.h2d;
      total.d2h += P.d2h;
      total.evals += P.evals;
      total.windows += P.windows;
      total.svd_launches += P.svd_launches;
      total.svd_matrices += P.svd_matrices;
      total.arps_exact += P.arps_exact;
      total.svd_fp64 += P.svd_fp64;
      total.svd_sweeps += P.svd_sweeps;
      total.svd_tuned |= P.svd_tuned;
      for (int j = 0; j < 8; ++j) total.stage[j] += P.stage[j];
    }
    for (uint32_t i = 0; i < nseq; ++i)
      if (codes[i] != PGSVT_OK) throw Fail(codes[i], msgs[i]);
  });
}

// ---- learned lambda proposal: inference, gradient and training on the device

int pgsvt_lambda_predict(const float* model, const float* features, uint32_t n, float* y) {
  return guarded(nullptr, [&](Stats& stats) {
    if (!model || !features || !y) throw Fail(PGSVT_ERR_INVALID_ARG, "null pointer");
    if (n == 0) return;
    need_device();
    DevMem mem;
    cudaStream_t s;
    PGSVT_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct SG { cudaStream_t s; ~SG() { cudaStreamDestroy(s); } } sg{s};
    float* m = mem.arr<float>(PGSVT_LAMBDA_MODEL_FLOATS);
    void* wbf = mem.get(PGSVT_LAMBDA_MODEL_FLOATS * 2);
    float* f = mem.arr<float>((size_t)n * PGSVT_LAMBDA_FEATURES);
    float* yd = mem.arr<float>(n);
    PGSVT_CK(cudaMemcpyAsync(m, model, sizeof(float) * PGSVT_LAMBDA_MODEL_FLOATS, cudaMemcpyHostToDevice, s));
    PGSVT_CK(cudaMemcpyAsync(f, features, sizeof(float) * n * PGSVT_LAMBDA_FEATURES,
                             cudaMemcpyHostToDevice, s));
    PGSVT_CK(lambda_attrs());
    check_launch(lambda_shadow(m, wbf, s), stats);
    check_launch(lambda_forward(m, wbf, f, (int)n, yd, s), stats);
    PGSVT_CK(cudaMemcpyAsync(y, yd, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
    PGSVT_CK(cudaStreamSynchronize(s));
  });
}

int pgsvt_lambda_grad(const float* model, const float* features, const float* targets, uint32_t n,
                      float* grad, double* loss) {
  return guarded(nullptr, [&](Stats& stats) {
    if (!model || !features || !targets || !grad) throw Fail(PGSVT_ERR_INVALID_ARG, "null pointer");
    if (n == 0) throw Fail(PGSVT_ERR_INVALID_ARG, "no samples");
    need_device();
    DevMem mem;
    cudaStream_t s;
    PGSVT_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct SG { cudaStream_t s; ~SG() { cudaStreamDestroy(s); } } sg{s};
    const int nblk = ((int)n + 31) / 32;
    float* m = mem.arr<float>(PGSVT_LAMBDA_MODEL_FLOATS);
    void* wbf = mem.get(PGSVT_LAMBDA_MODEL_FLOATS * 2);
    float* f = mem.arr<float>((size_t)n * PGSVT_LAMBDA_FEATURES);
    float* t = mem.arr<float>(n);
    float* part = mem.arr<float>((size_t)nblk * PGSVT_LAMBDA_PARAMS);
    float* pl = mem.arr<float>(nblk);
    float* g = mem.arr<float>(PGSVT_LAMBDA_PARAMS);
    PGSVT_CK(cudaMemcpyAsync(m, model, sizeof(float) * PGSVT_LAMBDA_MODEL_FLOATS, cudaMemcpyHostToDevice, s));
    PGSVT_CK(cudaMemcpyAsync(f, features, sizeof(float) * n * PGSVT_LAMBDA_FEATURES,
                             cudaMemcpyHostToDevice, s));
    PGSVT_CK(cudaMemcpyAsync(t, targets, sizeof(float) * n, cudaMemcpyHostToDevice, s));
    PGSVT_CK(lambda_attrs());
    check_launch(lambda_shadow(m, wbf, s), stats);
    check_launch(lambda_grad(m, wbf, f, t, (int)n, part, pl, g, s), stats, 2);
    std::vector<float> hl(nblk);
    PGSVT_CK(cudaMemcpyAsync(grad, g, sizeof(float) * PGSVT_LAMBDA_PARAMS, cudaMemcpyDeviceToHost, s));
    PGSVT_CK(cudaMemcpyAsync(hl.data(), pl, sizeof(float) * nblk, cudaMemcpyDeviceToHost, s));
    PGSVT_CK(cudaStreamSynchronize(s));
    if (loss) {
      double L = 0.0;
      for (float v : hl) L += v;
      *loss = L / n;
    }
  });
}

int pgsvt_lambda_train(float* model, const float* features, const float* targets, uint32_t n,
                       const pgsvt_train_params* tp, float* epoch_loss, pgsvt_status* st) {
  return guarded(st, [&](Stats& stats) {
    if (!model || !features || !targets || !tp) throw Fail(PGSVT_ERR_INVALID_ARG, "null pointer");
    const int batch = (int)tp->batch;
    if (batch < 32 || batch % 32 != 0 || batch > 8192)
      throw Fail(PGSVT_ERR_INVALID_ARG, "batch must be a multiple of 32 in [32, 8192]");
    if (n < (uint32_t)batch) throw Fail(PGSVT_ERR_INVALID_ARG, "fewer samples than one batch");
    if (tp->epochs < 1 || (uint64_t)tp->epochs * n > (1ull << 31))
      throw Fail(PGSVT_ERR_INVALID_ARG, "epochs x samples must be in [1, 2^31]");
    need_device();
    DevMem mem;
    cudaStream_t s;
    PGSVT_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct SG { cudaStream_t s; ~SG() { cudaStreamDestroy(s); } } sg{s};
    LambdaTrain t{};
    t.n = (int)n;
    t.batch = batch;
    t.steps = (int)n / batch;
    t.total_steps = t.steps * (int)tp->epochs;
    t.lr = tp->lr;
    t.lr_final = tp->lr_final;
    t.wd = tp->weight_decay;
    t.b1 = tp->beta1;
    t.b2 = tp->beta2;
    t.eps = tp->eps;
    const int nblk = batch / 32;
    t.m = mem.arr<float>(PGSVT_LAMBDA_MODEL_FLOATS);
    t.wbf = mem.get(PGSVT_LAMBDA_MODEL_FLOATS * 2);
    t.mom1 = mem.arr<float>(PGSVT_LAMBDA_PARAMS);
    t.mom2 = mem.arr<float>(PGSVT_LAMBDA_PARAMS);
    float* feat = mem.arr<float>((size_t)n * PGSVT_LAMBDA_FEATURES);
    float* target = mem.arr<float>(n);
    int32_t* perm = mem.arr<int32_t>((size_t)tp->epochs * n);
    t.feat = feat;
    t.target = target;
    t.perm = perm;
    t.epoch = mem.arr<int>(1);
    t.part = mem.arr<float>((size_t)nblk * PGSVT_LAMBDA_PARAMS);
    t.loss_acc = mem.arr<float>((size_t)t.steps * nblk);
    t.epoch_loss = mem.arr<float>(tp->epochs);
    // sample order of every epoch: Fisher-Yates shuffles from a pcg64 stream
    std::vector<int32_t> hp((size_t)tp->epochs * n);
    Pcg64 rng((Pcg64::u128)tp->seed);
    for (uint32_t e = 0; e < tp->epochs; ++e) {
      int32_t* q = hp.data() + (size_t)e * n;
      for (uint32_t i = 0; i < n; ++i) q[i] = (int32_t)i;
      for (uint32_t i = n - 1; i > 0; --i) {
        const uint32_t j = (uint32_t)(((unsigned __int128)rng() * (i + 1)) >> 64);
        std::swap(q[i], q[j]);
      }
    }
    PGSVT_CK(cudaMemcpyAsync(t.m, model, sizeof(float) * PGSVT_LAMBDA_MODEL_FLOATS, cudaMemcpyHostToDevice, s));
    PGSVT_CK(cudaMemcpyAsync(feat, features, sizeof(float) * n * PGSVT_LAMBDA_FEATURES,
                             cudaMemcpyHostToDevice, s));
    PGSVT_CK(cudaMemcpyAsync(target, targets, sizeof(float) * n, cudaMemcpyHostToDevice, s));
    PGSVT_CK(cudaMemcpyAsync(perm, hp.data(), sizeof(int32_t) * hp.size(), cudaMemcpyHostToDevice, s));
    stats.h2d += sizeof(float) * (PGSVT_LAMBDA_MODEL_FLOATS + (size_t)n * (PGSVT_LAMBDA_FEATURES + 1)) +
                 sizeof(int32_t) * hp.size();
    PGSVT_CK(cudaMemsetAsync(t.mom1, 0, sizeof(float) * PGSVT_LAMBDA_PARAMS, s));
    PGSVT_CK(cudaMemsetAsync(t.mom2, 0, sizeof(float) * PGSVT_LAMBDA_PARAMS, s));
    PGSVT_CK(cudaMemsetAsync(t.epoch, 0, sizeof(int), s));
    PGSVT_CK(lambda_attrs());
    check_launch(lambda_shadow(t.m, t.wbf, s), stats);
    // one epoch = steps x (gradient, AdamW) + epoch bookkeeping, as a graph
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    PGSVT_CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    const cudaError_t ce = lambda_train_epoch(t, s);
    const cudaError_t ee = cudaStreamEndCapture(s, &graph);
    struct GG {
      cudaGraph_t& g;
      cudaGraphExec_t& x;
      ~GG() {
        if (x) cudaGraphExecDestroy(x);
        if (g) cudaGraphDestroy(g);
      }
    } gg{graph, exec};
    PGSVT_CK(ce);
    PGSVT_CK(ee);
    PGSVT_CK(cudaGraphInstantiate(&exec, graph, 0));
    for (uint32_t e = 0; e < tp->epochs; ++e) {
      PGSVT_CK(cudaGraphLaunch(exec, s));
      stats.launches += 2 * (uint64_t)t.steps + 1;
    }
    PGSVT_CK(cudaMemcpyAsync(model, t.m, sizeof(float) * PGSVT_LAMBDA_MODEL_FLOATS, cudaMemcpyDeviceToHost, s));
    if (epoch_loss)
      PGSVT_CK(cudaMemcpyAsync(epoch_loss, t.epoch_loss, sizeof(float) * tp->epochs,
                               cudaMemcpyDeviceToHost, s));
    PGSVT_CK(cudaStreamSynchronize(s));
    stats.d2h += sizeof(float) * (PGSVT_LAMBDA_MODEL_FLOATS + (epoch_loss ? tp->epochs : 0));
  });
}

int pgsvt_median_filter(const uint16_t* src, uint16_t* dst, uint32_t nrows, uint32_t ncols,
                        uint32_t nframes, uint32_t r) {
  return guarded(nullptr, [&](Stats& stats) {
    if (!src || !dst) throw Fail(PGSVT_ERR_INVALID_ARG, "null pointer");
    if (nrows != ncols) throw Fail(PGSVT_ERR_INVALID_ARG, "frames must be square");
    if (r < 1 || r > (uint32_t)kMaxMedian || 2 * r + 1 > nrows)
      throw Fail(PGSVT_ERR_INVALID_ARG, "median radius must be in [1, 15] and 2r+1 <= frame side");
    if (nframes == 0) return;
    need_device();
    const size_t F = (size_t)nrows * ncols, n = F * nframes;
    DevMem mem;
    cudaStream_t s;
    PGSVT_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct SG { cudaStream_t s; ~SG() { cudaStreamDestroy(s); } } sg{s};
    uint16_t* in = mem.arr<uint16_t>(n);
    float* xs = mem.arr<float>(n);
    float* zs = mem.arr<float>(n);
    PGSVT_CK(cudaMemcpyAsync(in, src, n * 2, cudaMemcpyHostToDevice, s));
    check_launch(launch_convert(in, PGSVT_U16, n, xs, nullptr, s), stats);
    check_launch(launch_median(xs, nullptr, (int)nframes, (int)nrows, (int)r, zs, s), stats);
    std::vector<float> h(n);
    PGSVT_CK(cudaMemcpyAsync(h.data(), zs, n * 4, cudaMemcpyDeviceToHost, s));
    PGSVT_CK(cudaStreamSynchronize(s));
    for (size_t i = 0; i < n; ++i) dst[i] = (uint16_t)h[i];
  });
}

int pgsvt_hot_pixel_filter(uint16_t* frames, uint32_t nrows, uint32_t ncols, uint32_t nframes,
                           double threshold) {
  return guarded(nullptr, [&](Stats& stats) {
    if (!frames) throw Fail(PGSVT_ERR_INVALID_ARG, "null pointer");
    if (!(threshold >= 0.0)) throw Fail(PGSVT_ERR_INVALID_ARG, "threshold must be >= 0");
    if (nrows == 0 || ncols == 0 || nframes == 0) return;
    need_device();
    const size_t F = (size_t)nrows * ncols, n = F * nframes;
    DevMem mem;
    cudaStream_t s;
    PGSVT_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct SG { cudaStream_t s; ~SG() { cudaStreamDestroy(s); } } sg{s};
    uint16_t* seq = mem.arr<uint16_t>(n);
    uint16_t* colmed = mem.arr<uint16_t>((size_t)ncols * nframes);
    uint32_t* med = mem.arr<uint32_t>(nframes);
    uint32_t* madm = mem.arr<uint32_t>(nframes);
    uint8_t* flag = mem.arr<uint8_t>(n);
    PGSVT_CK(cudaMemcpyAsync(seq, frames, n * 2, cudaMemcpyHostToDevice, s));
    check_launch(launch_hot_pixel(seq, (int)nrows, (int)ncols, (int)nframes, threshold, colmed,
                                  med, madm, flag, s), stats, 6);
    PGSVT_CK(cudaMemcpyAsync(frames, seq, n * 2, cudaMemcpyDeviceToHost, s));
    PGSVT_CK(cudaStreamSynchronize(s));
  });
}

int pgsvt_arps_window(const double* w, uint32_t nrows, uint32_t nwin, uint32_t block_size,
                      uint32_t motion_window, uint32_t time_iter, uint32_t frame_window,
                      uint32_t nimages, int32_t motion_estimation, uint32_t compat_flags,
                      int32_t* rows, int32_t* cols) {
  return guarded(nullptr, [&](Stats&) {
    if (!w || !rows || !cols) throw Fail(PGSVT_ERR_INVALID_ARG, "null pointer");
    if (nwin != 2 * frame_window + 1) throw Fail(PGSVT_ERR_INVALID_ARG, "nwin must be 2*frame_window+1");
    if (nimages < nwin || time_iter >= nimages) throw Fail(PGSVT_ERR_INVALID_ARG, "bad time index");
    if (motion_estimation && (motion_window < 2 || motion_window > (uint32_t)kMaxMW))
      throw Fail(PGSVT_ERR_INVALID_ARG, "motion_window must be in [2, 15]");
    pgsvt_params p;
    pgsvt_default_params(&p);
    p.block_size = block_size;
    p.motion_window = motion_window;
    p.motion_estimation = motion_estimation;
    p.compat_flags = compat_flags;
    const int t = (int)time_iter, tw = (int)frame_window, ni = (int)nimages;
    int ref;
    if (t < tw) ref = t;
    else if (t >= ni - tw) ref = t - (ni - (int)nwin);
    else ref = tw;
    OneWindow ow(w, nrows, nwin, p, ref, ref);
    const Geometry& g = ow.pb.g;
    auto ch = chains_for(t, tw, ni, (int)nwin);
    ArpsChain* dch = ow.mem.arr<ArpsChain>(ch.size());
    PGSVT_CK(cudaMemcpyAsync(dch, ch.data(), sizeof(ArpsChain) * ch.size(), cudaMemcpyHostToDevice, ow.s));
    ow.d.chains = dch;
    PGSVT_CK(launch_arps(ow.pb, ow.d, ow.s));
    std::vector<uint32_t> h((size_t)g.nwin * g.P);
    PGSVT_CK(cudaMemcpyAsync(h.data(), ow.d.pos, h.size() * 4, cudaMemcpyDeviceToHost, ow.s));
    PGSVT_CK(cudaStreamSynchronize(ow.s));
    for (size_t i = 0; i < h.size(); ++i) {
      rows[i] = (int32_t)(h[i] & 0xffffu);
      cols[i] = (int32_t)(h[i] >> 16);
    }
  });
}

int pgsvt_svd_window_ex(const double* u, uint32_t nrows, uint32_t nwin, uint32_t block_size,
                        uint32_t block_overlap, const int32_t* rows, const int32_t* cols,
                        float* S, uint32_t* npatch, pgsvt_status* st) {
  return guarded(st, [&](Stats& stats) {
    if (!u || !rows || !cols || !npatch) throw Fail(PGSVT_ERR_INVALID_ARG, "null pointer");
    pgsvt_params p;
    pgsvt_default_params(&p);
    p.block_size = block_size;
    p.block_overlap = block_overlap;
    p.optimize_pgure = 0;
    p.lambda = 0.0;
    OneWindow ow(u, nrows, nwin, p, (int)nwin / 2, (int)nwin / 2);
    const Geometry& g = ow.pb.g;
    ow.set_positions(rows, cols);
    ow.alloc_factors(1);
    PGSVT_CK(launch_svd(ow.pb, ow.d, ow.s));
    *npatch = (uint32_t)g.NP;
    unsigned long long c[5];
    PGSVT_CK(cudaMemcpyAsync(c, ow.d.counters, sizeof(c), cudaMemcpyDeviceToHost, ow.s));
    PGSVT_CK(cudaStreamSynchronize(ow.s));
    if (c[4])
      throw Fail(PGSVT_ERR_TIMEOUT, "SVD factors: a staged tile copy did not complete in time");
    stats.svd_launches = 1;
    stats.svd_matrices = (uint64_t)g.NP;
    stats.svd_sweeps = c[1];
    stats.svd_fp64 = c[2];
    stats.svd_variant = ow.pb.svd_variant;
    if (S) {
      std::vector<float> h((size_t)g.NC * g.NP);
      PGSVT_CK(cudaMemcpyAsync(h.data(), ow.d.sv, h.size() * 4, cudaMemcpyDeviceToHost, ow.s));
      PGSVT_CK(cudaStreamSynchronize(ow.s));
      // back to the reference's patch order (sorted position index)
      const std::vector<int32_t>& so = ow.su.sorted;
      for (int pi = 0; pi < g.NP; ++pi) {
        const int32_t pos = ow.su.plist[pi];
        const size_t out = std::lower_bound(so.begin(), so.end(), pos) - so.begin();
        for (int i = 0; i < g.nwin; ++i) S[out * g.nwin + i] = h[(size_t)i * g.NP + pi];
      }
    }
  });
}

int pgsvt_svd_window(const double* u, uint32_t nrows, uint32_t nwin, uint32_t block_size,
                     uint32_t block_overlap, const int32_t* rows, const int32_t* cols, float* S,
                     uint32_t* npatch) {
  return pgsvt_svd_window_ex(u, nrows, nwin, block_size, block_overlap, rows, cols, S, npatch,
                             nullptr);
}

int pgsvt_reconstruct_window(const double* u, uint32_t nrows, uint32_t nwin, uint32_t block_size,
                             uint32_t block_overlap, int32_t exp_weighting, const int32_t* rows,
                             const int32_t* cols, double lambda, double* v) {
  return guarded(nullptr, [&](Stats&) {
    if (!u || !rows || !cols || !v) throw Fail(PGSVT_ERR_INVALID_ARG, "null pointer");
    if (!(lambda >= 0)) throw Fail(PGSVT_ERR_INVALID_ARG, "lambda must be >= 0");
    pgsvt_params p;
    pgsvt_default_params(&p);
    p.block_size = block_size;
    p.block_overlap = block_overlap;
    p.exp_weighting = exp_weighting;
    p.optimize_pgure = 0;
    p.lambda = lambda;
    OneWindow ow(u, nrows, nwin, p, (int)nwin / 2, (int)nwin / 2);
    const Geometry& g = ow.pb.g;
    ow.set_positions(rows, cols);
    ow.alloc_factors(1);
    PGSVT_CK(cudaMemsetAsync(ow.d.cnt, 0, sizeof(int32_t) * g.cube(), ow.s));
    PGSVT_CK(launch_fields(ow.pb, ow.d, ow.s));
    PGSVT_CK(launch_search_init(ow.pb, ow.d, ow.s));
    PGSVT_CK(launch_svd(ow.pb, ow.d, ow.s));
    PGSVT_CK(launch_eval_round(ow.pb, ow.d, 2, ow.s));
    double* vd = ow.mem.arr<double>(g.cube());
    PGSVT_CK(launch_cube_out(ow.pb, ow.d, vd, ow.s));
    PGSVT_CK(cudaMemcpyAsync(v, vd, sizeof(double) * g.cube(), cudaMemcpyDeviceToHost, ow.s));
    PGSVT_CK(cudaStreamSynchronize(ow.s));
  });
}

int pgsvt_risk_window(const double* u, uint32_t nrows, uint32_t nwin, uint32_t block_size,
                      uint32_t block_overlap, int32_t exp_weighting, const int32_t* rows,
                      const int32_t* cols, double alpha, double mu, double sigma,
                      int64_t random_seed, uint32_t compat_flags, const double* lambdas,
                      uint32_t nl, double* risk) {
  return guarded(nullptr, [&](Stats&) {
    if (!u || !rows || !cols || !lambdas || !risk) throw Fail(PGSVT_ERR_INVALID_ARG, "null pointer");
    if (alpha < 0 || mu < 0 || sigma < 0) throw Fail(PGSVT_ERR_INVALID_ARG, "noise parameters must be >= 0");
    pgsvt_params p;
    pgsvt_default_params(&p);
    p.block_size = block_size;
    p.block_overlap = block_overlap;
    p.exp_weighting = exp_weighting;
    p.optimize_pgure = 1;
    p.alpha = alpha;
    p.mu = mu;
    p.sigma = sigma;
    p.compat_flags = compat_flags;
    p.random_seed = random_seed;
    p.search_points = kMaxK;
    OneWindow ow(u, nrows, nwin, p, (int)nwin / 2, (int)nwin / 2);
    const Geometry& g = ow.pb.g;
    const size_t C = g.cube();
    ow.set_positions(rows, cols);
    const int ncopies = (compat_flags & PGSVT_COMPAT_INT_DELTA1) ? 3 : 4;
    ow.alloc_factors(ncopies);
    ow.d.fld0 = ow.mem.arr<float>(C);
    ow.d.fld2 = ow.mem.arr<float>(C);
    ow.d.fld1 = ncopies == 4 ? ow.mem.arr<float>(C) : nullptr;
    std::vector<int8_t> h1(C), h2(C);
    make_probes(random_seed, C, h1.data(), h2.data());
    int8_t* d1 = ow.mem.arr<int8_t>(C);
    int8_t* d2 = ow.mem.arr<int8_t>(C);
    PGSVT_CK(cudaMemcpyAsync(d1, h1.data(), C, cudaMemcpyHostToDevice, ow.s));
    PGSVT_CK(cudaMemcpyAsync(d2, h2.data(), C, cudaMemcpyHostToDevice, ow.s));
    ow.d.d1 = d1;
    ow.d.d2code = d2;
    ow.d.probe_stride = 0;
    PGSVT_CK(launch_fields(ow.pb, ow.d, ow.s));
    {  // the largest requested lambda bounds the thresholds the SVD must keep
      double upper = 0.0;
      for (uint32_t j = 0; j < nl; ++j) upper = std::max(upper, lambdas[j]);
      PGSVT_CK(cudaMemcpyAsync(&ow.d.wc->upper, &upper, sizeof(double), cudaMemcpyHostToDevice, ow.s));
      PGSVT_CK(cudaStreamSynchronize(ow.s));
    }
    PGSVT_CK(launch_svd(ow.pb, ow.d, ow.s));
    double* out = ow.mem.arr<double>(kMaxK);
    for (uint32_t j0 = 0; j0 < nl; j0 += kMaxK) {
      const int n = (int)std::min<uint32_t>(kMaxK, nl - j0);
      SearchState hs;
      std::memset(&hs, 0, sizeof(hs));
      for (int j = 0; j < n; ++j) hs.next[j] = lambdas[j0 + j];
      hs.nnext = n;
      hs.done = 0;
      PGSVT_CK(cudaMemcpyAsync(ow.d.st, &hs, sizeof(hs), cudaMemcpyHostToDevice, ow.s));
      PGSVT_CK(launch_risk_round(ow.pb, ow.d, out, ow.s));
      PGSVT_CK(cudaMemcpyAsync(risk + j0, out, sizeof(double) * n, cudaMemcpyDeviceToHost, ow.s));
      PGSVT_CK(cudaStreamSynchronize(ow.s));
    }
  });
}

const char* pgsvt_last_error(void) { return g_err.c_str(); }

const char* pgsvt_version(void) { return "pgsvt-gb300 0.1.0 (sm_103a)"; }

}  // extern "C"
