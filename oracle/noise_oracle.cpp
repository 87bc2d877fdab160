// noise_oracle.cpp — FP64 restatement of the reference's noise estimator
// (test infrastructure only; part of libpgsvt_oracle.so).
//
// Follows src/noise.hpp:35-458 of tjof2/pgure-svt 0.6.4 statement by
// statement, with Armadillo's semantics written out: accu() sums with two
// interleaved accumulators (even / odd elements), median() of an even count
// is lo + (hi - lo) / 2, stable_sort_index() is a stable sort.  Armadillo
// itself is not in the reference tree (9.880.1 pinned by its install script),
// so those three are restatements of its documented behaviour.
//
// Reproduced as written, including:
//  * QuadTree (noise.hpp:411-453) recurses on the node that was last in the
//    tree before the split and on the first three children only, so the
//    root is tested twice, its children are appended twice and every
//    split's fourth child is never tested (it stays a leaf);
//  * the parent shedding loop (noise.hpp:67-72) never sheds the smallest
//    parent index, so a split root stays among the leaves (whole-frame
//    mean and variance are part of the fit);
//  * ConvolveFIR / SplitBlockQ index borders with x+1 == N -> 1 and
//    x == 0 -> N-2 (noise.hpp:184-190, 393-397).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <stdexcept>
#include <thread>
#include <vector>

namespace orc_noise {

// Armadillo accu(): two accumulators over even and odd positions
template <typename F>
double accu(size_t n, F&& f) {
  double v1 = 0.0, v2 = 0.0;
  size_t i = 0, j = 1;
  for (; j < n; i += 2, j += 2) {
    v1 += f(i);
    v2 += f(j);
  }
  if (i < n) v1 += f(i);
  return v1 + v2;
}

double median(std::vector<double> a) {  // Armadillo median() of a vector
  const size_t n = a.size(), half = n / 2;
  std::nth_element(a.begin(), a.begin() + half, a.end());
  if (n % 2 == 0) {
    const double lo = *std::max_element(a.begin(), a.begin() + half);
    return lo + (a[half] - lo) / 2.0;
  }
  return a[half];
}

// 2.5% points of F(N^2 - 1, N^2 - 1) to six digits, as tabulated for
// N = 2, 4, ..., 4096 (noise.hpp:167-178)
const double kF0025[12] = {15.4392, 2.86209, 1.64602, 1.27893, 1.13046, 1.06318,
                           1.03110, 1.01543, 1.00769, 1.00384, 1.00192, 1.00096};

struct Frame {  // one slice: Ny rows x Nx cols, column-major
  const double* a;
  uint32_t ny;
  double at(uint32_t r, uint32_t c) const { return a[r + (size_t)c * ny]; }
};

struct Estimator {
  uint32_t method, size = 8;
  // tree: columns (row offset, col offset, side); del: indices of split nodes
  std::vector<uint32_t> ti, tj, ts, del;

  bool split_block(const Frame& f, uint32_t i0, uint32_t j0, uint32_t N) const {
    if (N <= size) return false;  // noise.hpp:184-188
    const double l = 5.0;
    std::vector<double> A((size_t)N * N), res((size_t)N * N);
    for (uint32_t c = 0; c < N; ++c)
      for (uint32_t r = 0; r < N; ++r) A[r + (size_t)c * N] = f.at(i0 + r, j0 + c);
    auto a = [&](uint32_t r, uint32_t c) { return A[r + (size_t)c * N]; };
    for (uint32_t x = 0; x < N; ++x)
      for (uint32_t y = 0; y < N; ++y) {
        const uint32_t xp = (x + 1 == N) ? 1 : x + 1, yp = (y + 1 == N) ? 1 : y + 1;
        const uint32_t xm = (x == 0) ? N - 2 : x - 1, ym = (y == 0) ? N - 2 : y - 1;
        res[y + (size_t)x * N] = l * a(y, x) - (a(yp, x) + a(ym, x) + a(y, xm) + a(y, xp));
      }
    const double sq = std::sqrt(30.0);
    for (double& v : res) v /= sq;
    const size_t R = (size_t)N * N;
    const double OoR = 1.0 / (double)R, OoRm1 = 1.0 / (double)(R - 1);
    const double mz = accu(R, [&](size_t k) { return A[k]; }) * OoR;
    const double Sz = accu(R, [&](size_t k) { const double d = A[k] - mz; return d * d; }) * OoRm1;
    const double mr = accu(R, [&](size_t k) { return res[k]; }) * OoR;
    const double Se = accu(R, [&](size_t k) { const double d = res[k] - mr; return d * d; }) * OoRm1;
    const double stat = (Sz > Se) ? Sz / Se : Se / Sz;
    int idx = -1;
    for (int k = 0; k < 12; ++k)
      if ((1u << (k + 1)) == N) idx = k;
    if (idx < 0) throw std::runtime_error("noise estimation needs power-of-two frames (noise.hpp:216)");
    return stat > kF0025[idx];
  }

  void quadtree(const Frame& f, uint32_t part) {  // noise.hpp:411-453
    const uint32_t i = ti[part], j = tj[part];
    uint32_t s = ts[part];
    if (!split_block(f, i, j, s)) return;
    s /= 2;
    const uint32_t n = (uint32_t)ti.size() - 1;
    const uint32_t ci[4] = {i, i + s, i, i + s}, cj[4] = {j, j, j + s, j + s};
    for (int k = 0; k < 4; ++k) {
      ti.push_back(ci[k]);
      tj.push_back(cj[k]);
      ts.push_back(s);
    }
    del.push_back(part);
    uint32_t iter = n;
    do {
      quadtree(f, iter);
      iter++;
    } while (iter < n + 4);
  }

  static double iqd(std::vector<double> a) {  // InterquartileDistance
    std::sort(a.begin(), a.end());
    const uint32_t N = (uint32_t)a.size();
    const uint32_t m = (uint32_t)std::floor((std::floor((N + 1) / 2) + 1) / 2);
    return a[N - m - 1] - a[m - 1];
  }

  static void huber(const std::vector<double>& x, std::vector<double>& w) {
    const double p = 0.75;
    for (size_t k = 0; k < x.size(); ++k) w[k] = (std::fabs(x[k]) < p) ? 1.0 : p / std::fabs(x[k]);
  }

  static double robust_mean(const std::vector<double>& A) {  // noise.hpp:239-270
    const uint32_t I = 10000;
    const size_t N = A.size();
    const double tol = 1e-6, eps = 1e-12;
    double m = 0.0, m0 = 1e12;
    std::vector<double> w(N, 1.0), r(N);
    for (uint32_t it = 0; it < I; ++it) {
      m = accu(N, [&](size_t k) { return w[k] * A[k]; });
      const double aux = accu(N, [&](size_t k) { return w[k]; });
      m = (std::fabs(aux) < eps) ? m0 : m / aux;
      for (size_t k = 0; k < N; ++k) r[k] = A[k] - m;
      const double e = accu(N, [&](size_t k) { return std::fabs(r[k]); }) / (double)N;
      if (std::fabs(m0 - m) < tol || e < tol) break;
      m0 = m;
      const double d = iqd(r) + eps;
      for (double& v : r) v *= 1.0 / d;
      huber(r, w);
    }
    return m;
  }

  static double robust_var(const std::vector<double>& A) {  // noise.hpp:232-236
    const double med = median(A);
    std::vector<double> dv(A.size());
    for (size_t k = 0; k < A.size(); ++k) dv[k] = std::fabs(A[k] - med);
    const double sig = 1.4826 * median(dv);
    return sig * sig;
  }

  // ConvolveFIR (noise.hpp:386-409): in(x,y) - (1/8) * (its 8 neighbours),
  // summed in the column-major order of the 3x3 product with Armadillo's
  // two accumulators; returned column-major like the reference's reshape
  static std::vector<double> laplace(const std::vector<double>& in, uint32_t N) {
    std::vector<double> out((size_t)N * N, 0.0);
    auto a = [&](uint32_t r, uint32_t c) { return in[r + (size_t)c * N]; };
    for (uint32_t x = 0; x < N; ++x)
      for (uint32_t y = 0; y < N; ++y) {
        const uint32_t xp = (x + 1 == N) ? 1 : x + 1, yp = (y + 1 == N) ? 1 : y + 1;
        const uint32_t xm = (x == 0) ? N - 2 : x - 1, ym = (y == 0) ? N - 2 : y - 1;
        const double nb[9] = {a(xm, ym), a(xm, y), a(xm, yp), a(x, ym), a(x, y),
                              a(x, yp), a(xp, ym), a(xp, y), a(xp, yp)};
        out[y + (size_t)x * N] = accu(9, [&](size_t k) { return nb[k] * (k == 4 ? 1.0 : -0.125); });
      }
    return out;
  }

  static std::vector<double> wls_fit(const std::vector<double>& x, const std::vector<double>& y) {
    const uint32_t I = 10000;
    const size_t N = x.size();
    const double tol = 1e-6, eps = 1e-12;
    double a0 = 1e12, b0 = 1e12, p0 = 0.0, p1 = 0.0;
    std::vector<double> w(N, 1.0), w2(N), r(N);
    for (uint32_t it = 0; it < I; ++it) {  // noise.hpp:310-357
      for (size_t k = 0; k < N; ++k) w2[k] = w[k] * w[k];
      const double sw2 = accu(N, [&](size_t k) { return w2[k]; });
      const double sw2x = accu(N, [&](size_t k) { return w2[k] * x[k]; });
      const double sw2y = accu(N, [&](size_t k) { return w2[k] * y[k]; });
      p0 = sw2 * accu(N, [&](size_t k) { return w2[k] * (x[k] * y[k]); }) - sw2x * sw2y;
      const double aux = sw2 * accu(N, [&](size_t k) { return w2[k] * (x[k] * x[k]); }) - sw2x * sw2x;
      p0 = (std::fabs(aux) < eps) ? a0 : p0 / aux;
      p1 = sw2y - p0 * sw2x;
      p1 = (std::fabs(aux) < eps) ? b0 : p1 / sw2;
      for (size_t k = 0; k < N; ++k) r[k] = y[k] - (x[k] * p0 + p1);
      const double e = accu(N, [&](size_t k) { return std::fabs(r[k]); }) / (double)N;
      if ((std::fabs(a0 - p0) < tol && std::fabs(b0 - p1) < tol) || e < tol) break;
      a0 = p0;
      b0 = p1;
      const double d = iqd(r) + eps;
      for (double& v : r) v /= d;
      huber(r, w);
    }
    return {p0, p1};
  }

  static double mode(const std::vector<double>& A) {  // ComputeMode, noise.hpp:272-297
    const double M = *std::max_element(A.begin(), A.end());
    const size_t N = A.size();
    const double dyn = 1.0 * N;
    std::vector<double> a(N);
    for (size_t k = 0; k < N; ++k) a[k] = std::round(A[k] * dyn / M);
    uint32_t maxCount = 0;
    double maxValue = 0.0;
    for (size_t i = 0; i < N; ++i) {
      uint32_t count = 0;
      for (size_t j = 0; j < N; ++j)
        if (a[j] == a[i]) count++;
      if (count > maxCount) {
        maxCount = count;
        maxValue = a[i];
      }
    }
    return maxValue * M / dyn;
  }

  // Leaf statistics of one frame (noise.hpp:40-104), appended in the
  // reference's order.
  void frame_stats(const double* uf, uint32_t ny, uint32_t nx, std::vector<double>& means,
                   std::vector<double>& vars) {
    const Frame fr{uf, ny};
    ti.assign(1, 0);
    tj.assign(1, 0);
    ts.assign(1, nx);
    del.clear();
    quadtree(fr, 0);
    std::vector<uint32_t> d = del;
    std::sort(d.begin(), d.end());
    d.erase(std::unique(d.begin(), d.end()), d.end());
    std::vector<char> keep(ti.size(), 1);
    for (size_t k = d.size() > 0 ? d.size() - 1 : 0; k > 0; --k) keep[d[k]] = 0;
    for (size_t n = 0; n < ti.size(); ++n) {
      if (!keep[n]) continue;
      const uint32_t x = ti[n], y = tj[n], s = ts[n];
      std::vector<double> col((size_t)s * s);
      for (uint32_t c = 0; c < s; ++c)
        for (uint32_t r = 0; r < s; ++r) col[r + (size_t)c * s] = fr.at(x + r, y + c);
      const double m = robust_mean(col);
      const double v = robust_var(laplace(col, s));
      if (m >= 0.0 && v >= 0.0) {  // noise.hpp:100-102 (-1 marks unused slots)
        means.push_back(m);
        vars.push_back(v);
      }
    }
  }

  // Estimate (noise.hpp:36-152) on a normalised window: Ny x Nx x T.  The
  // frames' statistics are independent: with threads > 1 they are computed
  // concurrently (one estimator per frame) and concatenated in frame order.
  void estimate(const double* u, uint32_t ny, uint32_t nx, uint32_t T, double& alpha,
                double& mu, double& sigma, uint32_t threads = 1) {
    std::vector<double> means, vars;
    if (threads <= 1) {
      for (uint32_t f = 0; f < T; ++f) frame_stats(u + (size_t)f * nx * ny, ny, nx, means, vars);
    } else {
      std::vector<std::vector<double>> fm(T), fv(T);
      std::vector<std::thread> th;
      const uint32_t nt = std::min(threads, T);
      for (uint32_t k = 0; k < nt; ++k)
        th.emplace_back([&, k] {
          for (uint32_t f = T * k / nt; f < T * (k + 1) / nt; ++f) {
            Estimator e;
            e.method = method;
            e.frame_stats(u + (size_t)f * nx * ny, ny, nx, fm[f], fv[f]);
          }
        });
      for (auto& t : th) t.join();
      for (uint32_t f = 0; f < T; ++f) {
        means.insert(means.end(), fm[f].begin(), fm[f].end());
        vars.insert(vars.end(), fv[f].begin(), fv[f].end());
      }
    }
    std::vector<size_t> idx(means.size());
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return means[a] < means[b]; });
    std::vector<double> rm(means.size()), rv(means.size());
    for (size_t k = 0; k < idx.size(); ++k) {
      rm[k] = means[idx[k]];
      rv[k] = vars[idx[k]];
    }
    const std::vector<double> ab = wls_fit(rm, rv);
    alpha = (alpha >= 0.0) ? alpha : ab[0];
    switch (method) {
      case 1: {
        const int L = (int)std::floor(1.0 * (double)((size_t)nx * ny / means.size()));
        const uint32_t ie = (uint32_t)std::round(0.05 * L);
        // the first ie + 1 leaves; clamped to the leaf count (the reference
        // reads past its arrays when ie + 1 exceeds it)
        const size_t ne = std::min<size_t>((size_t)ie + 1, rm.size());
        std::vector<double> a(rm.begin(), rm.begin() + ne), b(rv.begin(), rv.begin() + ne);
        mu = (mu >= 0.0) ? mu : mode(a);
        const double dSi = mode(b);
        sigma = (sigma >= 0.0) ? sigma : std::sqrt(dSi);
        break;
      }
      case 2: {
        mu = (mu >= 0.0) ? mu : mode(rm);
        const double dSi = mode(rv);
        sigma = (sigma >= 0.0) ? sigma
                               : std::sqrt(std::max(dSi, std::max(ab[1] + ab[0] * dSi, 0.0)));
        break;
      }
      case 3:
        mu = (mu >= 0.0) ? mu : mode(rm);
        sigma = (sigma >= 0.0) ? sigma : std::sqrt(std::fabs(ab[1] + ab[0] * mu));
        break;
      default:  // 4
        mu = (mu >= 0.0) ? mu : rm[0];
        sigma = (sigma >= 0.0) ? sigma : std::sqrt(std::fabs(ab[1] + ab[0] * mu));
        break;
    }
  }
};

}  // namespace orc_noise

// C++ entry used by pgsvt_oracle.cpp and the C API
void orc_noise_estimate_impl(const double* u, uint32_t ny, uint32_t nx, uint32_t T,
                             uint32_t method, double& alpha, double& mu, double& sigma,
                             uint32_t threads) {
  orc_noise::Estimator e;
  e.method = method;
  e.estimate(u, ny, nx, T, alpha, mu, sigma, threads);
}
