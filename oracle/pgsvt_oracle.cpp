// pgsvt_oracle.cpp — FP64 CPU restatement of the PGURE-SVT denoising path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the CUDA
// library (tests/, __graft_entry__.smoke()) and the timed CPU baseline of
// bench.py.  Nothing in the product links or calls it.
//
// It restates, function by function, tjof2/pgure-svt 0.6.4:
//   src/pguresvt.hpp:40-169  window slicing, normalisation, orchestration
//   src/arps.hpp:21-375      ARPS block matching (MotionEstimator)
//   src/svt.hpp:24-167       Casorati gather, SVD, threshold, rebuild, average
//   src/pgure.hpp:26-237     probes, perturbed decompositions, PGURE risk
//   src/utils.hpp:96-168     SoftThreshold, thread fan-out over windows
// in double precision.  Third-party pieces that are not in the reference tree
// are restated from their published algorithms:
//   * arma::svd_econ -> LAPACK dgesdd (jobz='S'), Armadillo's default "dc"
//     method; the routine is supplied at run time (scipy's LAPACK).
//   * pcg64 (O'Neill 2014, 128-bit LCG with XSL-RR output) and libstdc++'s
//     std::bernoulli_distribution / generate_canonical for the probes.
//   * NLopt LN_SBPLX (pgure.hpp:206) is NOT restated: the lambda search is the
//     bracketed batch grid search that the CUDA library runs (same schedule),
//     so the lambda trajectory of the reference is not reproduced.
// Summations follow Armadillo's accu() (two interleaved accumulators).
// Compile with -ffp-contract=off so that x86 and Arm give the same bits.

#include "pgsvt_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <exception>
#include <limits>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

// noise_oracle.cpp: NoiseEstimator::Estimate (noise.hpp:36-152)
void orc_noise_estimate_impl(const double* u, uint32_t ny, uint32_t nx, uint32_t T,
                             uint32_t method, double& alpha, double& mu, double& sigma,
                             uint32_t threads = 1);

namespace {

thread_local std::string g_err;
orc_dgesdd_fn g_dgesdd = nullptr;
uint32_t g_stage_threads = 1;  // threads of the per-stage entry points (orc_set_threads)

// fn(begin, end, tid) over [0, n) in `threads` contiguous chunks, one
// std::thread each (on the calling thread when threads <= 1).  Used inside one
// window: every chunk writes its own outputs, so results do not depend on the
// thread count.
template <typename Fn>
void par_chunks(size_t n, uint32_t threads, Fn&& fn) {
  if (threads <= 1 || n < 2) {
    fn((size_t)0, n, 0u);
    return;
  }
  const uint32_t nt = (uint32_t)std::min<size_t>(threads, n);
  std::vector<std::thread> th;
  std::vector<std::exception_ptr> ex(nt);
  th.reserve(nt);
  for (uint32_t k = 0; k < nt; ++k)
    th.emplace_back([&, k] {
      try {
        fn(n * k / nt, n * (k + 1) / nt, k);
      } catch (...) {
        ex[k] = std::current_exception();
      }
    });
  for (auto& t : th) t.join();
  for (auto& e : ex)
    if (e) std::rethrow_exception(e);
}

constexpr uint32_t kCompatSwap = 0x1u;        // pguresvt.hpp:133 vs pgure.hpp:26-30
constexpr uint32_t kCompatZeroMotion = 0x2u;  // arps.hpp:42,60-64
constexpr uint32_t kCompatIntDelta1 = 0x4u;   // pgure.hpp:80 (icube * double)

constexpr double kCostSentinel = 1e9;   // arps.hpp:145 costsScale
constexpr uint32_t kMaxSDSP = 1000000;  // arps.hpp:146

struct Fail : std::runtime_error {
  int code;
  Fail(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// Armadillo accu(): two partial sums over even / odd linear indices.
template <typename F>
inline double accu2(size_t n, F&& f) {
  double v1 = 0.0, v2 = 0.0;
  size_t i = 0, j = 1;
  for (; j < n; i += 2, j += 2) {
    v1 += f(i);
    v2 += f(j);
  }
  if (i < n) v1 += f(i);
  return v1 + v2;
}

// ---------------------------------------------------------------------------
// Probes (pgure.hpp:52-59,167-186)

struct Pcg64 {
  using u128 = unsigned __int128;
  u128 state, inc;
  static u128 mult() {
    return ((u128)2549297995355413924ULL << 64) | 4865540595714422341ULL;
  }
  static u128 default_inc() {
    return ((u128)6364136223846793005ULL << 64) | 1442695040888963407ULL;
  }
  // engine(itype state): state = bump(seed + increment)
  explicit Pcg64(u128 seed) : inc(default_inc()) {
    state = (seed + inc) * mult() + inc;
  }
  // 128-bit engines advance first, then output (output_previous == false).
  uint64_t next() {
    state = state * mult() + inc;
    const uint64_t hi = (uint64_t)(state >> 64), lo = (uint64_t)state;
    const unsigned rot = (unsigned)(hi >> 58);
    const uint64_t x = hi ^ lo;
    return (x >> rot) | (x << ((64u - rot) & 63u));
  }
};

// libstdc++ bernoulli_distribution(p): u = generate_canonical<double,53>,
// which for a 64-bit engine is one draw scaled by 2^-64 (clamped below 1).
inline bool bernoulli_draw(Pcg64& g, double p) {
  double u = (double)g.next() / 18446744073709551616.0;
  if (u >= 1.0) u = std::nextafter(1.0, 0.0);
  return u < p;
}

void make_probes(int64_t seed, size_t n, int8_t* d1, double* d2) {
  Pcg64::u128 s;
  if (seed >= 0) {
    s = (Pcg64::u128)(uint64_t)seed;
  } else {  // std::random_device, as pcg_extras::seed_seq_from<random_device>
    std::random_device rd;
    s = ((Pcg64::u128)(((uint64_t)rd() << 32) | rd()) << 64) |
        (((uint64_t)rd() << 32) | rd());
  }
  Pcg64 g(s);
  const double kappa = 1.0;
  const double vP = 0.5 + 0.5 * kappa / std::sqrt(kappa * kappa + 4);
  const double vQ = 1 - vP;
  const double vQvP = std::sqrt(vQ / vP);
  const double vPvQ = std::sqrt(vP / vQ);
  for (size_t i = 0; i < n; ++i) d1[i] = bernoulli_draw(g, 0.5) ? -1 : 1;
  for (size_t i = 0; i < n; ++i) d2[i] = bernoulli_draw(g, vP) ? -1 * vQvP : vPvQ;
}

// ---------------------------------------------------------------------------
// Geometry

struct Geom {
  uint32_t S;     // frame side (square frames)
  uint32_t bs;    // patch side
  uint32_t nwin;  // window length = 2*fw+1
  uint32_t P;     // ARPS positions (S-bs+1)^2
  uint32_t nMbs;  // S - bs
  Geom(uint32_t s, uint32_t b, uint32_t nw)
      : S(s), bs(b), nwin(nw), P((s - b + 1) * (s - b + 1)), nMbs(s - b) {}
  size_t frame() const { return (size_t)S * S; }
  size_t cube() const { return frame() * nwin; }
};

// Kept patch indices (svt.hpp:61-94).
std::vector<int64_t> patch_list(uint32_t S, uint32_t bs, uint32_t ov) {
  const uint64_t nxMbs = S - bs, nyMbs = S - bs;
  std::vector<int64_t> v;
  for (uint64_t i = 0; i < 1 + nyMbs; i += ov)
    for (uint64_t j = 0; j < 1 + nxMbs; j += ov) v.push_back((int64_t)(i * nyMbs + j));
  for (uint64_t i = 0; i < 1 + nyMbs; i += ov) v.push_back((int64_t)((nyMbs + 1) * i + nxMbs));
  for (uint64_t i = 0; i < 1 + nxMbs; i += ov) v.push_back((int64_t)((nyMbs + 1) * nxMbs + i));
  std::sort(v.begin(), v.end());
  v.erase(std::unique(v.begin(), v.end()), v.end());
  return v;
}

// ---------------------------------------------------------------------------
// ARPS (arps.hpp)

struct Arps {
  const double* A;
  Geom g;
  uint32_t mw;
  double oo;  // 1/(bs*bs), arps.hpp:39
  std::vector<int32_t> mrow, mcol;  // motions(2, P, 2*fw)
  int32_t* prow;
  int32_t* pcol;                    // patches(2, P, nwin)
  uint32_t threads = 1;             // threads over the positions of a frame pair

  Arps(const double* a, Geom gg, uint32_t m, int32_t* r, int32_t* c)
      : A(a), g(gg), mw(m), oo(1.0 / (gg.bs * gg.bs)), prow(r), pcol(c) {
    const size_t slots = (size_t)g.P * (g.nwin - 1);
    mrow.assign(slots, 0);
    mcol.assign(slots, 0);
    std::fill(prow, prow + (size_t)g.P * g.nwin, 0);
    std::fill(pcol, pcol + (size_t)g.P * g.nwin, 0);
  }

  // CostFunction (arps.hpp:148-151): mean squared difference of two blocks.
  double cost(int r0, int c0, int k0, int r1, int c1, int k1) const {
    const size_t S = g.S, F = g.frame();
    const double* a = A + (size_t)k0 * F;
    const double* b = A + (size_t)k1 * F;
    const int bs = (int)g.bs;
    return accu2((size_t)bs * bs, [&](size_t e) {
             const int r = (int)(e % bs), c = (int)(e / bs);
             const double d = a[(r0 + r) + (c0 + c) * S] - b[(r1 + r) + (c1 + c) * S];
             return d * d;
           }) * oo;
  }

  static int first_min(const double* c, int n) {
    double m = c[0];
    for (int k = 1; k < n; ++k) m = std::min(m, c[k]);
    for (int k = 0; k < n; ++k)
      if (c[k] == m) return k;
    return 0;
  }

  // ARPSMotionEstimation (arps.hpp:153-375) for one frame pair.
  void pair(int a1, int a2, int a3) {
    const int W = 2 * (int)mw + 1, M = (int)mw, bs = (int)g.bs, S = (int)g.S;
    const int P = (int)g.P, n1 = 1 + (int)g.nMbs;
    static const int SD[5][2] = {{0, -1}, {-1, 0}, {0, 0}, {1, 0}, {0, 1}};  // (dx, dy)
    par_chunks((size_t)P, threads, [&](size_t b, size_t e, uint32_t) {
    std::vector<uint8_t> seen((size_t)W * W);
    for (int it = (int)b; it < (int)e; ++it) {
      double c[6];
      for (double& x : c) x = kCostSentinel;
      std::fill(seen.begin(), seen.end(), 0);
      int LD[6][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}};
      const int i = it % n1, j = it / n1;
      int x = j, y = i;
      c[2] = cost(i, j, a1, i, j, a2);
      seen[(size_t)M * W + M] = 1;
      int step, nld;
      if (j == 0) {
        step = 2;
        nld = 5;
      } else {
        const int my = mrow[(size_t)a3 * P + it], mx = mcol[(size_t)a3 * P + it];
        const int ay = std::abs(my), ax = std::abs(mx);
        step = (ax <= ay) ? ay : ax;
        if ((ay == 0 && ax == step) || (ax == 0 && ay == step)) {
          nld = 5;
        } else {
          nld = 6;
          LD[5][0] = mx;
          LD[5][1] = my;
        }
      }
      LD[0][0] = 0;     LD[0][1] = -step;
      LD[1][0] = -step; LD[1][1] = 0;
      LD[2][0] = 0;     LD[2][1] = 0;
      LD[3][0] = step;  LD[3][1] = 0;
      LD[4][0] = 0;     LD[4][1] = step;
      for (int k = 0; k < nld; ++k) {  // LDSP
        const int vy = y + LD[k][1], hx = x + LD[k][0];
        const bool skip = k == 2 || step == 0 || hx < 0 || vy < 0 ||
                          hx + bs - 1 >= S || vy + bs - 1 >= S;
        if (!skip) {
          c[k] = cost(i, j, a1, vy, hx, a2);
          seen[(size_t)(LD[k][1] + M) * W + (LD[k][0] + M)] = 1;
        }
      }
      int best = first_min(c, 6);
      x += LD[best][0];
      y += LD[best][1];
      double cur = c[best];
      for (double& v : c) v = kCostSentinel;
      c[2] = cur;
      for (uint32_t n = 0;; ++n) {  // SDSP
        for (int k = 0; k < 5; ++k) {
          const int vy = y + SD[k][1], hx = x + SD[k][0];
          const bool skip = k == 2 || hx < 0 || vy < 0 || hx + bs - 1 >= S ||
                            vy + bs - 1 >= S || hx < j - M || hx > j + M ||
                            vy < i - M || vy > i + M ||
                            seen[(size_t)(vy - i + M) * W + (hx - j + M)] == 1;
          if (!skip) {
            c[k] = cost(i, j, a1, vy, hx, a2);
            seen[(size_t)(vy - i + M) * W + (hx - j + M)] = 1;
          }
        }
        best = first_min(c, 6);
        cur = c[best];
        if (best == 2 || n >= kMaxSDSP) break;
        x += SD[best][0];
        y += SD[best][1];
        for (double& v : c) v = kCostSentinel;
        c[2] = cur;
      }
      mrow[(size_t)a3 * P + it] = y - i;
      mcol[(size_t)a3 * P + it] = x - j;
      prow[(size_t)a2 * P + it] = y;
      pcol[(size_t)a2 * P + it] = x;
    }
    });
  }

  // MotionEstimator::Estimate (arps.hpp:52-134).
  void estimate(uint32_t t, uint32_t tw, uint32_t nimg, bool motion, bool zeroMotion) {
    const int P = (int)g.P, n1 = 1 + (int)g.nMbs, nwin = (int)g.nwin;
    int ref;
    if (t < tw) ref = (int)t;
    else if (t >= nimg - tw) ref = (int)(t - (nimg - g.nwin));
    else ref = (int)tw;
    for (int it = 0; it < P; ++it) {
      prow[(size_t)ref * P + it] = it % n1;
      pcol[(size_t)ref * P + it] = it / n1;
    }
    if (!motion) {
      if (!zeroMotion)  // every frame at the patch's own grid position
        for (int k = 0; k < nwin; ++k)
          if (k != ref)
            for (int it = 0; it < P; ++it) {
              prow[(size_t)k * P + it] = it % n1;
              pcol[(size_t)k * P + it] = it / n1;
            }
      return;
    }
    if (t < tw) {
      const int T = (int)t, loopEnd = nwin - T - 1;
      for (int i = 0; i < loopEnd; ++i) pair(T + i, T + i + 1, T + i);
      for (int i = 0; i < T; ++i) pair(T - i, T - i - 1, T - i);
    } else if (t >= nimg - tw) {
      const int e = (int)(t - (nimg - g.nwin)), loopEnd = 2 * (int)tw - e;
      for (int i = 0; i < loopEnd; ++i) pair(e + i, e + i + 1, e + i);
      for (int i = 0; i < e; ++i) {
        if (2 * (int)tw == e) pair(e - i, e - i - 1, e - i - 1);
        else pair(e - i, e - i - 1, e - i);
      }
    } else {
      const int T = (int)tw;
      for (int i = 0; i < T; ++i) pair(T + i, T + i + 1, T + i);
      for (int i = 0; i < T; ++i) pair(T - i, T - i - 1, T - i);
    }
  }
};

// ---------------------------------------------------------------------------
// SVT (svt.hpp)

struct Svt {
  Geom g;
  std::vector<int64_t> plist;  // kept patches (actualPatches)
  const int32_t* prow;
  const int32_t* pcol;
  uint32_t m, n;
  // per patch: m*n, n, n*n; left uninitialised until dgesdd writes every
  // entry (the threads that compute a patch also first touch its pages)
  std::unique_ptr<double[]> U, S, VT;
  bool expw;
  std::vector<double> weights;   // coverage count per voxel (lambda independent)
  uint32_t threads = 1;          // threads inside this window

  Svt(Geom gg, std::vector<int64_t> pl, const int32_t* r, const int32_t* c, bool e)
      : g(gg), plist(std::move(pl)), prow(r), pcol(c), m(gg.bs * gg.bs), n(gg.nwin), expw(e) {}

  size_t np() const { return plist.size(); }

  void gather(const double* u, size_t it, double* blk) const {
    const size_t P = g.P, S = g.S, F = g.frame();
    const int64_t p = plist[it];
    for (uint32_t k = 0; k < n; ++k) {
      const int y = prow[(size_t)k * P + p], x = pcol[(size_t)k * P + p];
      for (uint32_t c = 0; c < g.bs; ++c)
        for (uint32_t r = 0; r < g.bs; ++r)
          blk[(size_t)k * m + r + c * g.bs] = u[(size_t)k * F + (y + r) + (x + c) * S];
    }
  }

  // Decompose (svt.hpp:58-118); patches split over `threads`, each with its
  // own LAPACK workspace, writing its own factors.
  void decompose(const double* u) {
    if (!g_dgesdd) throw Fail(2, "oracle: no LAPACK dgesdd bound (orc_set_dgesdd)");
    const size_t N = np();
    U.reset(new double[N * m * n]);
    S.reset(new double[N * n]);
    VT.reset(new double[N * n * n]);
    int lwork;
    {
      std::vector<double> blk((size_t)m * n), work(1), s1(n), u1((size_t)m * n), v1((size_t)n * n);
      std::vector<int> iwork(8 * n);
      int M = (int)m, Nn = (int)n, lda = M, ldu = M, ldvt = Nn, lq = -1, info = 0;
      char jobz = 'S';
      g_dgesdd(&jobz, &M, &Nn, blk.data(), &lda, s1.data(), u1.data(), &ldu, v1.data(),
               &ldvt, work.data(), &lq, iwork.data(), &info);
      lwork = std::max(1, (int)work[0]);
    }
    par_chunks(N, threads, [&](size_t b, size_t e, uint32_t) {
      std::vector<double> blk((size_t)m * n), work(lwork);
      std::vector<int> iwork(8 * n);
      int M = (int)m, Nn = (int)n, lda = M, ldu = M, ldvt = Nn, lw = lwork, info = 0;
      char jobz = 'S';
      for (size_t it = b; it < e; ++it) {
        gather(u, it, blk.data());
        g_dgesdd(&jobz, &M, &Nn, blk.data(), &lda, &S[it * n], &U[it * m * n], &ldu,
                 &VT[it * n * n], &ldvt, work.data(), &lw, iwork.data(), &info);
        if (info != 0) throw Fail(3, "oracle: dgesdd failed, info=" + std::to_string(info));
      }
    });
    weights.assign(g.cube(), 0.0);
    par_chunks(n, threads, [&](size_t kb, size_t ke, uint32_t) {  // frames split
      for (size_t it = 0; it < N; ++it) scatter_ones(it, (uint32_t)kb, (uint32_t)ke);
    });
  }

  void scatter_ones(size_t it, uint32_t kb, uint32_t ke) {
    const size_t P = g.P, S = g.S, F = g.frame();
    const int64_t p = plist[it];
    for (uint32_t k = kb; k < ke; ++k) {
      const int y = prow[(size_t)k * P + p], x = pcol[(size_t)k * P + p];
      for (uint32_t c = 0; c < g.bs; ++c)
        for (uint32_t r = 0; r < g.bs; ++r) weights[(size_t)k * F + (y + r) + (x + c) * S] += 1.0;
    }
  }

  // Shrunk singular values (svt.hpp:135-143, utils.hpp:96-106).
  void shrink(size_t it, double lambda, double* sp) const {
    const double* s = &S[it * n];
    if (expw) {
      double smax = s[0];
      for (uint32_t i = 1; i < n; ++i) smax = std::max(smax, s[i]);
      const double a = -0.5 * lambda;
      for (uint32_t i = 0; i < n; ++i) {
        const double w = std::fabs(smax * std::exp(a * (s[i] * s[i])));
        const double sg = (s[i] > 0) - (s[i] < 0);
        sp[i] = sg * std::max(std::fabs(s[i]) - w, 0.0);
      }
    } else {
      for (uint32_t i = 0; i < n; ++i) {
        const double sg = (s[i] > 0) - (s[i] < 0);
        sp[i] = sg * std::max(std::fabs(s[i]) - lambda, 0.0);
      }
    }
  }

  // Reconstruct (svt.hpp:121-167): v = average of U*diag(S')*V^T blocks.
  // With several threads the shrunk values are computed per patch chunk and
  // the frame columns are split in bands, each thread adding, patch by patch
  // in order, the block entries that fall in its band: every voxel sees the
  // same additions in the same order as with one thread.
  void reconstruct(double lambda, double* v) const {
    const size_t P = g.P, S = g.S, F = g.frame(), N = np();
    std::fill(v, v + g.cube(), 0.0);
    std::vector<double> sp(N * n);
    par_chunks(N, threads, [&](size_t b, size_t e, uint32_t) {
      for (size_t it = b; it < e; ++it) shrink(it, lambda, &sp[it * n]);
    });
    par_chunks(S, threads, [&](size_t x0, size_t x1, uint32_t) {
      const int bs = (int)g.bs;
      std::vector<double> us((size_t)m * n), acc(m);
      for (size_t it = 0; it < N; ++it) {
        const double* u = &U[it * m * n];
        const double* vt = &VT[it * n * n];
        const double* s = &sp[it * n];
        const int64_t p = plist[it];
        bool have_us = false;
        for (size_t k = 0; k < n; ++k) {
          const int y = prow[k * P + p], x = pcol[k * P + p];
          if (x + bs <= (int)x0 || x >= (int)x1) continue;
          if (!have_us) {  // u_ei * s'_i, the first product of every term
            for (uint32_t i = 0; i < n; ++i)
              for (uint32_t e = 0; e < m; ++e) us[e + (size_t)i * m] = u[e + (size_t)i * m] * s[i];
            have_us = true;
          }
          const int cb = std::max(0, (int)x0 - x), ce = std::min(bs, (int)x1 - x);
          const size_t e0 = (size_t)cb * bs, e1 = (size_t)ce * bs;
          // block(e, k) = sum_i (u_ei s'_i) vt_ik, i in order: one chain per row
          for (size_t e = e0; e < e1; ++e) acc[e] = 0.0;
          for (uint32_t i = 0; i < n; ++i) {
            const double w = vt[i + k * n];
            const double* ui = &us[(size_t)i * m];
            for (size_t e = e0; e < e1; ++e) acc[e] += ui[e] * w;
          }
          for (int c = cb; c < ce; ++c)
            for (int r = 0; r < bs; ++r) v[k * F + (y + r) + (x + c) * S] += acc[r + (size_t)c * bs];
        }
      }
    });
    const size_t C = g.cube();
    par_chunks(C, threads, [&](size_t b, size_t e, uint32_t) {
      for (size_t i = b; i < e; ++i) {
        const double q = v[i] / weights[i];
        v[i] = std::isfinite(q) ? q : 0.0;
      }
    });
  }
};

// ---------------------------------------------------------------------------
// PGURE (pgure.hpp)

struct Pgure {
  Geom g;
  const double* U;
  double alpha, mu, sigma, sigmasq;  // PGURE members (after the ctor binding)
  double eps1 = 0, eps2 = 0;
  bool optimize, intDelta1;
  std::vector<int8_t> d1;
  std::vector<double> d2;
  std::vector<double> U1, U2p, U2m;
  Svt svt0, svt1, svt2p, svt2m;
  std::vector<double> Uhat, R1, R2p, R2m;
  uint64_t evals = 0;

  Pgure(Geom gg, const double* u, const std::vector<int64_t>& pl, const int32_t* r,
        const int32_t* c, double a_c, double mu_c, double sigma_c, int64_t seed,
        bool expw, bool opt, uint32_t compat, uint32_t threads = 1)
      : g(gg), U(u), optimize(opt), intDelta1(compat & kCompatIntDelta1),
        svt0(gg, pl, r, c, expw), svt1(gg, pl, r, c, expw), svt2p(gg, pl, r, c, expw),
        svt2m(gg, pl, r, c, expw) {
    // PGURE(u, p, alpha, sigma, mu, ...) lands on the ctor's (alpha, mu, sigma).
    alpha = a_c;
    if (compat & kCompatSwap) {
      mu = sigma_c;
      sigma = mu_c;
    } else {
      mu = mu_c;
      sigma = sigma_c;
    }
    sigmasq = sigma * sigma;
    for (Svt* s : {&svt0, &svt1, &svt2p, &svt2m}) s->threads = threads;
    svt0.decompose(U);
    if (!optimize) return;
    const size_t C = g.cube();
    double umax = U[0];
    for (size_t i = 1; i < C; ++i) umax = std::max(umax, U[i]);
    eps1 = umax * 0.0001;
    eps2 = 100 * eps1;
    d1.resize(C);
    d2.resize(C);
    make_probes(seed, C, d1.data(), d2.data());
    U2p.resize(C);
    U2m.resize(C);
    par_chunks(C, threads, [&](size_t b, size_t e, uint32_t) {
      for (size_t i = b; i < e; ++i) {
        U2p[i] = U[i] + (d2[i] * eps2);
        U2m[i] = U[i] - (d2[i] * eps2);
      }
    });
    if (!intDelta1) {
      U1.resize(C);
      for (size_t i = 0; i < C; ++i) U1[i] = U[i] + (d1[i] * eps1);
      svt1.decompose(U1.data());
    }
    svt2p.decompose(U2p.data());
    svt2m.decompose(U2m.data());
    Uhat.resize(C);
    R1.resize(C);
    R2p.resize(C);
    R2m.resize(C);
  }

  // CalculatePGURE (pgure.hpp:120-137)
  double risk(double lambda) {
    ++evals;
    svt0.reconstruct(lambda, Uhat.data());
    if (intDelta1) R1 = Uhat;  // svt1 decomposed U1 == U: identical rebuild
    else svt1.reconstruct(lambda, R1.data());
    svt2p.reconstruct(lambda, R2p.data());
    svt2m.reconstruct(lambda, R2m.data());
    const size_t C = g.cube();
    const double OoN = 1.0 / (g.S * g.S * g.nwin);
    const double* u = U;
    // the five sums, each in accu()'s order; with several threads each sum
    // runs on its own thread (the same additions, so the same bits)
    double t[5];
    auto sum = [&](size_t which) {
      switch (which) {
        case 0: t[0] = accu2(C, [&](size_t i) { const double d = std::fabs(Uhat[i] - u[i]); return d * d; }); break;
        case 1: t[1] = accu2(C, [&](size_t i) { return u[i]; }); break;
        case 2: t[2] = accu2(C, [&](size_t i) {
                  return (double)d1[i] * ((alpha * u[i] - alpha * mu) + sigmasq) * (R1[i] - Uhat[i]);
                }); break;
        case 3: t[3] = accu2(C, [&](size_t i) { return d2[i] * ((R2p[i] - 2 * Uhat[i]) + R2m[i]); }); break;
        default: t[4] = accu2(C, [&](size_t i) { return Uhat[i]; }); break;
      }
    };
    par_chunks(5, svt0.threads, [&](size_t b, size_t e, uint32_t) {
      for (size_t k = b; k < e; ++k) sum(k);
    });
    const double t1 = t[0], t2 = t[1], t3 = t[2], t4 = t[3], t5 = t[4];
    return OoN * (t1 - (alpha + mu) * t2 + (2 / eps1 * t3) -
                  (2 * sigmasq * alpha / (eps2 * eps2) * t4) + (2 * mu * t5) + mu) -
           sigmasq;
  }
};

// ---------------------------------------------------------------------------
// Lambda search: bracketed batch grid search (the schedule the CUDA library
// runs on the device).  Round 0 evaluates K points spaced geometrically over
// [lo, hi]; each later round evaluates K/2 points evenly inside the bracket
// formed by the neighbours of the best point so far (K points in a narrow
// search, or when the bracket reaches down to zero).  Returns the best point
// (ties: smallest lambda).  Stops early when a round improves the best risk by
// no more than tol*|risk| while the bracket is narrower than kNarrowBracket
// times the best point, or when max_eval is reached.
constexpr double kNarrowBracket = 0.25;

struct SearchResult {
  double lambda, risk;
  uint32_t evals;
  bool edge;  // stopped after the round-0 grid: best point on a steep edge
};

// edge_flat >= 0: after the round-0 grid, a best point at either end whose
// neighbour's risk exceeds it by more than edge_flat * |risk| ends the search
// with edge = true (the narrow search's hand-over to the plain one), unless
// that end is a bound of the search: the bottom when include_zero_lo, the
// top when it equals `upper`.
//
// `sentinels` (narrow searches only): points evaluated with the round-0 grid
// but kept out of the point list; one of them below the grid's best ends the
// search with edge = true.
template <typename F>
SearchResult batch_search(F&& risk, double lo, double hi, uint32_t K, uint32_t rounds,
                          double tol, uint32_t max_eval, bool include_zero_lo,
                          double edge_flat = -1.0, double upper = -1.0,
                          const std::vector<double>& sentinels = {}) {
  struct Pt { double l, r; };
  std::vector<Pt> pts;
  if (max_eval < K) K = std::max<uint32_t>(1, max_eval);
  for (uint32_t j = 0; j < K; ++j) {
    const double l = (K == 1) ? hi : lo * std::pow(hi / lo, (double)j / (double)(K - 1));
    pts.push_back({l, risk(l)});
  }
  double sent = std::numeric_limits<double>::infinity();
  for (double l : sentinels) sent = std::min(sent, risk(l));
  uint32_t evals = K + (uint32_t)sentinels.size();
  auto best_of = [&]() {
    size_t b = 0;
    for (size_t i = 1; i < pts.size(); ++i)
      if (pts[i].r < pts[b].r) b = i;
    return b;
  };
  size_t b = best_of();
  SearchResult res{pts[b].l, pts[b].r, evals, false};
  if (sent < pts[b].r) {  // a plain-grid end does better than the narrow grid
    res.edge = true;
    return res;
  }
  const bool bound = (b == 0 && include_zero_lo) || (b + 1 == pts.size() && pts[b].l >= upper &&
                                                     upper > 0.0);
  if (edge_flat >= 0.0 && (b == 0 || b + 1 == pts.size()) && !bound) {
    const size_t nb = (b == 0) ? 1 : pts.size() - 2;
    if (pts.size() < 2 || !(pts[nb].r - pts[b].r <= edge_flat * std::fabs(pts[b].r))) {
      res.edge = true;
      return res;
    }
  }
  for (uint32_t rd = 0; rd < rounds; ++rd) {
    // refinement rounds of the plain search place half the grid's points,
    // unless the bracket reaches down to the zero bound
    const uint32_t Kr = (edge_flat >= 0.0 || (b == 0 && include_zero_lo))
                            ? K : std::max<uint32_t>(2, K / 2);
    if (evals + Kr > max_eval) break;
    const double blo = (b > 0) ? pts[b - 1].l : (include_zero_lo ? 0.0 : pts[b].l);
    const double bhi = (b + 1 < pts.size()) ? pts[b + 1].l : pts[b].l;
    if (!(bhi > blo)) break;
    const double prev = pts[b].r;
    for (uint32_t i = 0; i < Kr; ++i) {
      const double l = blo + (bhi - blo) * (double)(i + 1) / (double)(Kr + 1);
      pts.push_back({l, risk(l)});
    }
    evals += Kr;
    std::stable_sort(pts.begin(), pts.end(), [](const Pt& a, const Pt& c) { return a.l < c.l; });
    b = best_of();
    res.lambda = pts[b].l;
    res.risk = pts[b].r;
    const double nlo = (b > 0) ? pts[b - 1].l : (include_zero_lo ? 0.0 : pts[b].l);
    const double nhi = (b + 1 < pts.size()) ? pts[b + 1].l : pts[b].l;
    if (prev - pts[b].r <= tol * std::fabs(pts[b].r) && nhi - nlo <= kNarrowBracket * pts[b].l)
      break;  // no progress and a narrow bracket
  }
  res.evals = evals;
  return res;
}

// ---- median pre-filter of the ARPS input (pguresvt.hpp:69-84)
//
// X is converted to uint16 slice by slice (arma::conv_to<Mat<uint16_t>>;
// Armadillo 9.880.1 is not in the reference tree: this restatement takes C's
// conversion, truncation toward zero, with values clamped to [0, 65535]) and
// filtered by ConstantTimeMedianFilter (medfilter.hpp:478-541) with radius
// medianSize.  That filter (one stripe here: its stripe count works out to 1
// for every radius, the unsigned arithmetic of medfilter.hpp:512-513) is the
// exact median of the (2r+1)^2 window with coordinates clamped to the frame
// (replicated borders: medfilter.hpp:365-377 for rows, the pad_left /
// pad_right paths for columns).  Restated here as a direct selection.
uint16_t to_u16(double x) {
  if (!(x > 0.0)) return 0;
  if (x >= 65535.0) return 65535;
  return (uint16_t)x;
}

void median_frame(const uint16_t* src, uint16_t* dst, int nx, int ny, int r) {
  std::vector<uint16_t> win((size_t)(2 * r + 1) * (2 * r + 1));
  for (int i = 0; i < ny; ++i)
    for (int j = 0; j < nx; ++j) {
      size_t k = 0;
      for (int di = -r; di <= r; ++di) {
        const int ii = std::min(std::max(i + di, 0), ny - 1);
        for (int dj = -r; dj <= r; ++dj) {
          const int jj = std::min(std::max(j + dj, 0), nx - 1);
          win[k++] = src[(size_t)ii * nx + jj];
        }
      }
      std::nth_element(win.begin(), win.begin() + k / 2, win.begin() + k);
      dst[(size_t)i * nx + j] = win[k / 2];
    }
}

struct Plan {
  uint32_t nrows, nimg, bs, ov, mw, Ntc, fw, nwin;
  Plan(const orc_params& p, uint32_t nr, uint32_t ni) : nrows(nr), nimg(ni) {
    bs = p.block_size;
    ov = p.block_overlap;
    mw = p.motion_window;
    Ntc = (bs * bs < p.traj_length) ? (bs * bs) - 1 : p.traj_length;  // pguresvt.hpp:57
    fw = Ntc / 2;                                                     // pguresvt.hpp:58
    nwin = 2 * fw + 1;
  }
  uint32_t start(uint32_t t) const {  // pguresvt.hpp:100-114
    if (t < fw) return 0;
    if (t >= nimg - fw) return nimg - 2 * fw - 1;
    return t - fw;
  }
  uint32_t out_slice(uint32_t t) const {  // pguresvt.hpp:155-166
    if (t < fw) return t;
    if (t >= nimg - fw) return t - (nimg - Ntc);
    return fw;
  }
};

void validate(const orc_params& p, uint32_t nrows, uint32_t ncols, uint32_t nimg) {
  if (nrows != ncols) throw Fail(1, "frames must be square (arps.hpp:186-187)");
  if (p.block_size < 1 || p.block_size > nrows) throw Fail(1, "block_size out of range");
  if (p.block_overlap < 1 || p.block_overlap > p.block_size) throw Fail(1, "block_overlap out of range");
  if (p.traj_length < 1) throw Fail(1, "traj_length must be >= 1");
  Plan pl(p, nrows, nimg);
  if (pl.Ntc < 1 || nimg < pl.nwin) throw Fail(1, "sequence shorter than the trajectory window");
  if (p.motion_estimation && p.motion_window < 1) throw Fail(1, "motion_window must be >= 1");
  if (p.median_size > 0 && 2 * p.median_size + 1 > nrows)
    throw Fail(1, "median window wider than the frame (medfilter.hpp:347-348)");
  if (!p.optimize_pgure && p.lambda < 0) throw Fail(1, "lambda must be >= 0 without optimisation");
}

// One window: pguresvt.hpp:90-167.  Returns the lambda used.
struct WindowOut {
  double lambda, risk;
  uint32_t evals;
  double alpha, mu, sigma;  // noise parameters of the window (estimates(t, 1..3))
};

WindowOut run_window(const double* X, const double* Z, const orc_params& p, const Plan& pl,
                     uint32_t t, double* Yslice) {
  const Geom g(pl.nrows, pl.bs, pl.nwin);
  const size_t F = g.frame(), C = g.cube();
  std::vector<double> u(X + (size_t)pl.start(t) * F, X + (size_t)pl.start(t) * F + C);
  double umax = u[0];
  for (double x : u) umax = std::max(umax, x);
  for (double& x : u) x /= umax;
  // ARPS input w: the median-filtered window over its own maximum, or u
  // itself without the filter (pguresvt.hpp:85-88,100-120)
  std::vector<double> w;
  if (Z) {
    w.assign(Z + (size_t)pl.start(t) * F, Z + (size_t)pl.start(t) * F + C);
    double wmax = w[0];
    for (double x : w) wmax = std::max(wmax, x);
    for (double& x : w) x /= wmax;
  }
  // noise parameters: user values, the rest estimated on u when optimising
  // (pguresvt.hpp:62-65,122-127)
  double na = p.alpha >= 0 ? p.alpha : -1.0, nm = p.mu >= 0 ? p.mu : -1.0;
  double ns = p.sigma >= 0 ? p.sigma : -1.0;
  if (p.optimize_pgure)
    orc_noise_estimate_impl(u.data(), g.S, g.S, g.nwin, p.noise_method, na, nm, ns,
                            std::max(1u, p.window_threads));
  std::vector<int32_t> rows((size_t)g.P * g.nwin), cols((size_t)g.P * g.nwin);
  {
    Arps a(Z ? w.data() : u.data(), g, pl.mw, rows.data(), cols.data());
    a.threads = std::max(1u, p.window_threads);
    a.estimate(t, pl.fw, pl.nimg, p.motion_estimation != 0, p.compat_flags & kCompatZeroMotion);
  }
  Pgure pg(g, u.data(), patch_list(g.S, g.bs, pl.ov), rows.data(), cols.data(), na, nm, ns,
           p.random_seed, p.exp_weighting != 0, p.optimize_pgure != 0, p.compat_flags,
           std::max(1u, p.window_threads));
  WindowOut out{p.lambda, 0.0, 0, na, nm, ns};
  if (p.optimize_pgure) {
    const double OoN = 1.0 / (pl.nrows * pl.nrows * pl.Ntc);  // pguresvt.hpp:60
    double startp = (p.lambda >= 0.0) ? p.lambda : accu2(C, [&](size_t i) { return u[i]; }) * OoN;
    startp = std::max(0.0, startp);
    const double upper = std::max(100.0, startp);
    const uint32_t K = p.search_points ? p.search_points : 8;
    const uint32_t R = p.search_rounds ? p.search_rounds : 4;
    const uint32_t maxe = p.max_iter ? p.max_iter : 1;
    auto rf = [&](double l) { return pg.risk(l); };
    SearchResult sr;
    const double hint = p.lambda_hints ? p.lambda_hints[t] : p.lambda_hint;
    if (hint > 0) {
      const double span = p.hint_span > 1 ? p.hint_span : 2.0;
      const uint32_t Kh = std::min(K, p.hint_points ? p.hint_points : 4u);
      const uint32_t Rh = p.hint_rounds ? p.hint_rounds : 2u;
      const double flat = p.hint_flat > 0 ? p.hint_flat : 1e-3;
      const double h = std::min(hint, upper);
      const double lo = h / span, hi = std::min(upper, h * span);
      // the plain grid's ends the narrow grid does not reach, as far as the
      // round's size (K) and the evaluation budget leave room
      const uint32_t kh = maxe < Kh ? std::max<uint32_t>(1, maxe) : Kh;
      const int room = std::min((int)K - (int)kh, (int)maxe - (int)kh);
      std::vector<double> sent;
      if (room > 0 && lo > upper * 1e-4) sent.push_back(upper * 1e-4);
      if (room > (int)sent.size() && hi < upper) sent.push_back(upper);
      sr = batch_search(rf, lo, hi, Kh, Rh, p.tol, maxe, lo <= upper * 1e-4, flat, upper, sent);
      if (sr.edge) {  // proposal not bracketed: fall back to the full search
        const SearchResult full = batch_search(rf, upper * 1e-4, upper, K, R, p.tol,
                                               maxe > sr.evals ? maxe - sr.evals : 1, true);
        const uint32_t e = sr.evals + full.evals;
        if (full.risk < sr.risk) sr = full;
        sr.evals = e;
      }
    } else {
      sr = batch_search(rf, upper * 1e-4, upper, K, R, p.tol, maxe, true);
    }
    out = {sr.lambda, sr.risk, sr.evals, na, nm, ns};
  }
  std::vector<double> v(C);
  pg.svt0.reconstruct(out.lambda, v.data());
  const uint32_t os = pl.out_slice(t);
  for (size_t i = 0; i < F; ++i) Yslice[i] = v[(size_t)os * F + i] * umax;
  return out;
}

template <typename Fn>
void fan_out(uint32_t n, int64_t njobs, Fn&& fn) {  // utils.hpp:108-168
  uint32_t cores = (njobs > 0) ? (uint32_t)njobs : std::thread::hardware_concurrency();
  if (njobs == 0 || cores <= 1 || n <= 1) {
    for (uint32_t a = 0; a < n; ++a) fn(a);
    return;
  }
  std::vector<std::thread> th;
  std::vector<std::string> errs(std::min(cores, n));
  std::vector<int> codes(errs.size(), 0);
  const uint32_t nt = (uint32_t)errs.size();
  const uint32_t per = (n + nt - 1) / nt;
  for (uint32_t k = 0; k < nt; ++k) {
    th.emplace_back([&, k]() {
      try {
        for (uint32_t a = k * per; a < std::min(n, (k + 1) * per); ++a) fn(a);
      } catch (const Fail& f) {
        codes[k] = f.code;
        errs[k] = f.what();
      } catch (const std::exception& e) {
        codes[k] = 3;
        errs[k] = e.what();
      }
    });
  }
  for (auto& x : th) x.join();
  for (size_t k = 0; k < errs.size(); ++k)
    if (codes[k]) throw Fail(codes[k], errs[k]);
}

template <typename Fn>
int guarded(Fn&& fn) {
  try {
    g_err.clear();
    fn();
    return 0;
  } catch (const Fail& f) {
    g_err = f.what();
    return f.code;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 3;
  }
}

}  // namespace

extern "C" {

void orc_set_dgesdd(orc_dgesdd_fn fn) { g_dgesdd = fn; }
void orc_set_threads(uint32_t n) { g_stage_threads = n < 1 ? 1 : n; }
const char* orc_last_error(void) { return g_err.c_str(); }

int orc_probes(int64_t seed, uint64_t n, int8_t* d1, double* d2) {
  return guarded([&] { make_probes(seed, n, d1, d2); });
}

int orc_patch_list(uint32_t side, uint32_t bs, uint32_t ov, int64_t* out, uint64_t* count) {
  return guarded([&] {
    if (bs < 1 || bs > side || ov < 1) throw Fail(1, "bad patch geometry");
    const auto v = patch_list(side, bs, ov);
    *count = v.size();
    if (out) std::copy(v.begin(), v.end(), out);
  });
}

int orc_arps_window(const double* w, uint32_t side, uint32_t nwin, uint32_t bs, uint32_t mw,
                    uint32_t time_iter, uint32_t frame_window, uint32_t nimages, int32_t motion,
                    uint32_t compat, int32_t* rows, int32_t* cols) {
  return guarded([&] {
    if (nwin != 2 * frame_window + 1) throw Fail(1, "nwin must be 2*frame_window+1");
    Arps a(w, Geom(side, bs, nwin), mw, rows, cols);
    a.threads = g_stage_threads;
    a.estimate(time_iter, frame_window, nimages, motion != 0, compat & kCompatZeroMotion);
  });
}

int orc_svd_window(const double* u, uint32_t side, uint32_t nwin, uint32_t bs, uint32_t ov,
                   const int32_t* rows, const int32_t* cols, double* S, uint64_t* npatch) {
  return guarded([&] {
    Svt s(Geom(side, bs, nwin), patch_list(side, bs, ov), rows, cols, true);
    s.threads = g_stage_threads;
    s.decompose(u);
    *npatch = s.np();
    if (S) std::copy(s.S.get(), s.S.get() + s.np() * s.n, S);
  });
}

int orc_reconstruct_window(const double* u, uint32_t side, uint32_t nwin, uint32_t bs,
                           uint32_t ov, int32_t expw, const int32_t* rows, const int32_t* cols,
                           double lambda, double* v) {
  return guarded([&] {
    Svt s(Geom(side, bs, nwin), patch_list(side, bs, ov), rows, cols, expw != 0);
    s.threads = g_stage_threads;
    s.decompose(u);
    s.reconstruct(lambda, v);
  });
}

int orc_risk_window(const double* u, uint32_t side, uint32_t nwin, uint32_t bs, uint32_t ov,
                    int32_t expw, const int32_t* rows, const int32_t* cols, double alpha,
                    double mu, double sigma, int64_t seed, uint32_t compat, const double* lambdas,
                    uint32_t nl, double* risk) {
  return guarded([&] {
    const Geom g(side, bs, nwin);
    Pgure pg(g, u, patch_list(side, bs, ov), rows, cols, alpha, mu, sigma, seed, expw != 0,
             true, compat, g_stage_threads);
    for (uint32_t i = 0; i < nl; ++i) risk[i] = pg.risk(lambdas[i]);
  });
}

int orc_noise_estimate(const double* u, uint32_t nrows, uint32_t ncols, uint32_t nslices,
                       uint32_t method, double* alpha, double* mu, double* sigma) {
  return guarded([&] {
    orc_noise_estimate_impl(u, nrows, ncols, nslices, method, *alpha, *mu, *sigma);
  });
}

// HotPixelFilter (hotpixel.hpp:19-64) on uint16 frames, in place, with the
// element-type semantics of Armadillo 9.880.1 (not in the reference tree):
// medians of uint16 data are uint16 (even count: lo + (hi - lo)/2 in integer
// arithmetic); `slice - median` and `... > threshold * mad` convert the double
// operand to uint16 and compute in uint16 (differences wrap modulo 65536).
int orc_hot_pixel(uint16_t* seq, uint32_t nr, uint32_t nc, uint32_t nimg, double thr) {
  return guarded([&] {
    auto med16 = [](std::vector<uint16_t> v) -> uint16_t {
      const size_t n = v.size(), h = n / 2;
      std::nth_element(v.begin(), v.begin() + h, v.end());
      if (n % 2) return v[h];
      const uint16_t lo = *std::max_element(v.begin(), v.begin() + h);
      return (uint16_t)(lo + (uint16_t)((v[h] - lo) / 2));
    };
    auto med_of_cols = [&](const uint16_t* a, uint16_t sub) {
      std::vector<uint16_t> cm(nc), col(nr);
      for (uint32_t c = 0; c < nc; ++c) {
        for (uint32_t r = 0; r < nr; ++r) col[r] = (uint16_t)(a[r + (size_t)c * nr] - sub);
        cm[c] = med16(col);
      }
      return med16(cm);
    };
    for (uint32_t f = 0; f < nimg; ++f) {
      uint16_t* a = seq + (size_t)f * nr * nc;
      const double median = (double)med_of_cols(a, 0);
      const uint16_t mu16 = (uint16_t)median;
      const double mad = (double)med_of_cols(a, mu16) * (1.0 / 0.6745);
      const double t = thr * mad;
      const uint16_t tu = !(t > 0.0) ? 0 : (t >= 65535.0 ? 65535 : (uint16_t)t);
      std::vector<size_t> out;
      for (size_t i = 0; i < (size_t)nr * nc; ++i)
        if ((uint16_t)(a[i] - mu16) > tu) out.push_back(i);
      for (size_t i : out) {
        const uint32_t r = (uint32_t)(i % nr), c = (uint32_t)(i / nr);
        if (r > 0 && r < nr - 1 && c > 0 && c < nc - 1) {
          double w[8] = {(double)a[(r - 1) + (size_t)(c - 1) * nr], (double)a[(r - 1) + (size_t)c * nr],
                         (double)a[(r - 1) + (size_t)(c + 1) * nr], (double)a[r + (size_t)(c - 1) * nr],
                         (double)a[r + (size_t)(c + 1) * nr], (double)a[(r + 1) + (size_t)(c - 1) * nr],
                         (double)a[(r + 1) + (size_t)c * nr], (double)a[(r + 1) + (size_t)(c + 1) * nr]};
          std::sort(w, w + 8);
          a[i] = (uint16_t)(0.5 * (w[3] + w[4]));
        } else {
          a[i] = (uint16_t)median;
        }
      }
    }
  });
}

int orc_median_filter(const uint16_t* src, uint16_t* dst, uint32_t nx, uint32_t ny,
                      uint32_t r) {
  return guarded([&] { median_frame(src, dst, (int)nx, (int)ny, (int)r); });
}

int orc_denoise(const double* X, uint32_t nrows, uint32_t ncols, uint32_t nimages,
                const orc_params* p, double* Y, double* est, orc_report* rep) {
  return guarded([&] {
    const auto t0 = std::chrono::steady_clock::now();
    validate(*p, nrows, ncols, nimages);
    const Plan pl(*p, nrows, nimages);
    const size_t F = (size_t)nrows * ncols;
    std::fill(Y, Y + F * nimages, 0.0);
    std::fill(est, est + (size_t)nimages * 4, 0.0);
    std::vector<uint32_t> evals(nimages, 0);
    uint32_t fb = p->frame_begin, fe = p->frame_end;  // output frames computed
    if (fb == 0 && fe == 0) fe = nimages;
    if (fb >= fe || fe > nimages) throw Fail(1, "bad frame range");
    std::vector<double> Z;
    if (p->median_size > 0) {  // pguresvt.hpp:69-80
      Z.resize(F * nimages);
      fan_out(nimages, p->n_jobs, [&](uint32_t i) {
        std::vector<uint16_t> a(F), b(F);
        for (size_t k = 0; k < F; ++k) a[k] = to_u16(X[(size_t)i * F + k]);
        median_frame(a.data(), b.data(), (int)ncols, (int)nrows, (int)p->median_size);
        for (size_t k = 0; k < F; ++k) Z[(size_t)i * F + k] = b[k];
      });
    }
    fan_out(fe - fb, p->n_jobs, [&](uint32_t k) {
      const uint32_t t = fb + k;
      const WindowOut o = run_window(X, Z.empty() ? nullptr : Z.data(), *p, pl, t,
                                     Y + (size_t)t * F);
      est[t] = o.lambda;  // pguresvt.hpp:150-153 (unswapped alpha, mu, sigma)
      est[t + nimages] = o.alpha;
      est[t + 2 * (size_t)nimages] = o.mu;
      est[t + 3 * (size_t)nimages] = o.sigma;
      evals[t] = o.evals;
      if (p->risk_out) p->risk_out[t] = o.risk;
      if (p->evals_out) p->evals_out[t] = o.evals;
    });
    if (rep) {
      rep->windows = fe - fb;
      rep->risk_evals = 0;
      for (uint32_t e : evals) rep->risk_evals += e;
      rep->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
  });
}

}  // extern "C"
