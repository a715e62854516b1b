// tlr_fdq.cpp -- FD-q rule generation on the host (tlr_fdq_rule).
//
// Bounded rules follow the reference's equal-error construction
// (src/Python/fdq_nodes.py:65-216, 280-304).  N auxiliary nodes in (-1, 1)
// are parameterised by N log gaps (the last of N + 1 gaps fixed to log 1,
// fdq_nodes.py:72-89).  For a continuation order o, every interval between
// adjacent auxiliary nodes carries the error polynomial E(x) = prod (x - s_j)
// over the o auxiliary nodes nearest to it; the rule's N + 1 nodes are the
// extrema of those polynomials inside their intervals plus the endpoints
// -1 and +1, and the auxiliary nodes are chosen so that log|E| is the same
// at all N + 1 nodes (fdq_nodes.py:118-149).  The reference solves each
// order 2..q by trust-region least squares with a 3-point finite-difference
// Jacobian (fdq_nodes.py:152-181).  The system is square (N parameters,
// N adjacent differences), so here every order is a damped Newton solve
// with the exact Jacobian: at an extremum x* of E the stationarity
// sum_j 1 / (x* - s_j) = 0 makes d log|E(x*)| / d s_k = -1 / (x* - s_k),
// and the Jacobian factors into a banded matrix times the (explicitly
// invertible) derivative of the softmax parameterisation.
// The result is symmetrised and checked as in fdq_nodes.py:184-216.
//
// Weights for derivative orders 0..2 come from Fornberg's recursion
// (B. Fornberg, "Generation of finite difference formulas on arbitrarily
// spaced grids", Math. Comp. 51 (1988) 699-706; the reference's
// fdq_nodes.py:226-277).  Periodic rules are uniform with centred stencils
// (fdq_nodes.py:307-353).  Every rule passes the reference's metadata and
// polynomial-moment checks (fdq_nodes.py:356-455) before it is returned.
//
// Pure host code: the node solve is a sequence of banded Newton steps,
// O(N q^2) each, that no device launch would speed up.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <limits>
#include <string>
#include <vector>

#include "../../include/tailor_gb300.h"

namespace tlr {
void set_global_error(const std::string &msg);
}

namespace {

using Vec = std::vector<double>;

struct RuleError {
  int status;
  std::string msg;
};

[[noreturn]] void fail(int status, const char *fmt, double v = 0.0) {
  char buf[256];
  std::snprintf(buf, sizeof buf, fmt, v);
  throw RuleError{status, buf};
}

// Auxiliary nodes and the softmax gaps behind them: gap_k proportional to
// exp(theta_k), k = 0..N with theta_N = 0; aux_i = -1 + 2 sum_{k<=i} gap_k.
struct Aux {
  Vec x, gap, cum;  // x[N], gap[N+1], cum[N] (cum_i = sum_{k<=i} gap_k)
};

Aux aux_from(const Vec &theta) {
  const int n = (int)theta.size();
  Aux a;
  a.gap.resize(n + 1);
  double mx = 0.0;
  for (double t : theta) mx = std::max(mx, t);
  double sum = 0.0;
  for (int k = 0; k <= n; ++k) {
    a.gap[k] = std::exp((k < n ? theta[k] : 0.0) - mx);
    sum += a.gap[k];
  }
  for (double &g : a.gap) g /= sum;
  a.x.resize(n);
  a.cum.resize(n);
  double c = 0.0;
  for (int i = 0; i < n; ++i) {
    c += a.gap[i];
    a.cum[i] = c;
    a.x[i] = -1.0 + 2.0 * c;
  }
  return a;
}

// The extremum of prod (x - s_j) strictly between adjacent roots a < b: the
// zero of g(x) = sum 1/(x - s_j), which falls monotonically from +inf to
// -inf on (a, b).  Newton steps kept inside a shrinking bracket; ends when
// the bracket or the step reaches the last representable digits.
double extremum(const double *s, int o, double a, double b) {
  double lo = std::nextafter(a, b), hi = std::nextafter(b, a);
  double x = 0.5 * (lo + hi);
  for (int it = 0; it < 200; ++it) {
    double g = 0.0, dg = 0.0;
    for (int j = 0; j < o; ++j) {
      const double r = 1.0 / (x - s[j]);
      g += r;
      dg -= r * r;
    }
    if (g == 0.0) return x;
    if (g > 0.0)
      lo = x;
    else
      hi = x;
    double xn = x - g / dg;
    if (!(xn > lo && xn < hi)) xn = 0.5 * (lo + hi);
    if (std::fabs(xn - x) <= 2.0 * std::numeric_limits<double>::epsilon() * std::fabs(x) ||
        hi <= std::nextafter(lo, hi))
      return xn;
    x = xn;
  }
  return x;
}

// Rule nodes (extrema plus endpoints), their log error amplitudes and the
// first auxiliary index of each node's stencil, for continuation order o.
struct EqualError {
  Vec nodes, logerr;
  std::vector<int> start;
};

EqualError equal_error(const Vec &aux, int o) {
  const int n = (int)aux.size();
  EqualError d;
  d.nodes.resize(n + 1);
  d.logerr.resize(n + 1);
  d.start.resize(n + 1);
  auto first = [&](int interval) { return std::clamp(interval - (o - 1) / 2, 0, n - o); };
  d.nodes[0] = -1.0;
  d.nodes[n] = 1.0;
  d.start[0] = first(0);
  d.start[n] = first(n - 2);
  for (int i = 0; i + 1 < n; ++i) {
    d.start[i + 1] = first(i);
    d.nodes[i + 1] = extremum(aux.data() + d.start[i + 1], o, aux[i], aux[i + 1]);
  }
  for (int i = 0; i <= n; ++i) {
    double e = 0.0;
    for (int j = 0; j < o; ++j) e += std::log(std::fabs(d.nodes[i] - aux[d.start[i] + j]));
    d.logerr[i] = e;
  }
  return d;
}

Vec residual_of(const EqualError &d) {
  Vec r(d.logerr.size() - 1);
  for (size_t i = 0; i < r.size(); ++i) r[i] = d.logerr[i + 1] - d.logerr[i];
  return r;
}

double norm2(const Vec &v) {
  double s = 0.0;
  for (double x : v) s += x * x;
  return std::sqrt(s);
}

double norm_inf(const Vec &v) {
  double s = 0.0;
  for (double x : v) s = std::max(s, std::fabs(x));
  return s;
}

// Newton step of the adjacent log-error differences r in theta, J step = -r,
// with J factored as J = M A:
//   M (N x N, banded): M(i, k) = dE(i+1, k) - dE(i, k), where
//     dE(i, k) = d logerr_i / d aux_k = -1 / (node_i - aux_k) for k in node
//     i's stencil (the other entries are zero);
//   A (N x N): d aux_i / d theta_m = 2 gap_m ([m <= i] - cum_i).
// M u = -r is solved by banded Gaussian elimination with partial pivoting;
// A step = u has the closed form below (y_m = gap_m step_m, S its prefix
// sums, T = S_{N-1}: u_i / 2 = S_i - cum_i T), so a step costs O(N o^2)
// instead of the O(N^3) of a dense Jacobian.
bool newton_step(const Aux &a, const EqualError &d, int o, const Vec &r, Vec &step) {
  const int n = (int)a.x.size();
  // rows of M as [lo, lo + width) windows of a dense n x n store
  Vec M((size_t)n * n, 0.0);
  std::vector<int> lo(n), hi(n);
  for (int i = 0; i < n; ++i) {
    lo[i] = std::min(d.start[i], d.start[i + 1]);
    hi[i] = std::max(d.start[i], d.start[i + 1]) + o;  // exclusive
    double *row = &M[(size_t)i * n];
    for (int j = 0; j < o; ++j) {
      const int k1 = d.start[i + 1] + j, k0 = d.start[i] + j;
      row[k1] += -1.0 / (d.nodes[i + 1] - a.x[k1]);
      row[k0] -= -1.0 / (d.nodes[i] - a.x[k0]);
    }
  }
  int kl = 0, ku = 0;  // band of M
  for (int i = 0; i < n; ++i) {
    kl = std::max(kl, i - lo[i]);
    ku = std::max(ku, hi[i] - 1 - i);
  }
  const int kue = kl + ku;  // upper band after row interchanges
  Vec u(n);
  for (int i = 0; i < n; ++i) u[i] = -r[i];
  for (int c = 0; c < n; ++c) {
    const int rend = std::min(n, c + kl + 1), cend = std::min(n, c + kue + 1);
    int p = c;
    for (int rr = c + 1; rr < rend; ++rr)
      if (std::fabs(M[(size_t)rr * n + c]) > std::fabs(M[(size_t)p * n + c])) p = rr;
    if (!(std::fabs(M[(size_t)p * n + c]) > 0.0)) return false;
    if (p != c) {
      for (int k = c; k < cend; ++k) std::swap(M[(size_t)p * n + k], M[(size_t)c * n + k]);
      std::swap(u[p], u[c]);
    }
    const double inv = 1.0 / M[(size_t)c * n + c];
    const double *mc = &M[(size_t)c * n];
    for (int rr = c + 1; rr < rend; ++rr) {
      double *mr = &M[(size_t)rr * n];
      const double f = mr[c] * inv;
      if (f == 0.0) continue;
      for (int k = c + 1; k < cend; ++k) mr[k] -= f * mc[k];
      u[rr] -= f * u[c];
    }
  }
  for (int rr = n - 1; rr >= 0; --rr) {
    double v = u[rr];
    const int cend = std::min(n, rr + kue + 1);
    for (int k = rr + 1; k < cend; ++k) v -= M[(size_t)rr * n + k] * u[k];
    u[rr] = v / M[(size_t)rr * n + rr];
  }
  // A step = u
  const double T = u[n - 1] / (2.0 * (1.0 - a.cum[n - 1]));
  double prev = 0.0;
  step.assign(n, 0.0);
  for (int i = 0; i < n; ++i) {
    const double S = 0.5 * u[i] + a.cum[i] * T;
    step[i] = (S - prev) / a.gap[i];
    prev = S;
  }
  for (double v : step)
    if (!std::isfinite(v)) return false;
  return true;
}

// Newton solve of one continuation order from theta (updated in place).
// Returns the final max-norm residual.
double newton_order(Vec &theta, int o, int *iterations) {
  const int n = (int)theta.size();
  Aux a = aux_from(theta);
  EqualError d = equal_error(a.x, o);
  Vec r = residual_of(d);
  int it = 0;
  for (; it < 100; ++it) {
    if (norm_inf(r) < 1e-14) break;
    Vec step;
    if (!newton_step(a, d, o, r, step)) break;
    const double r0 = norm2(r);
    double t = 1.0;
    bool better = false;
    Vec trial(n);
    Aux at;
    EqualError dt;
    Vec rt;
    for (int ls = 0; ls < 40; ++ls, t *= 0.5) {
      for (int i = 0; i < n; ++i) trial[i] = theta[i] + t * step[i];
      at = aux_from(trial);
      dt = equal_error(at.x, o);
      rt = residual_of(dt);
      if (norm2(rt) < (1.0 - 1e-4 * t) * r0) {
        better = true;
        break;
      }
    }
    if (!better) break;  // no decrease left: the residual is at rounding level
    theta.swap(trial);
    a = std::move(at);
    d = std::move(dt);
    r.swap(rt);
    if (t * norm_inf(step) < 1e-15) break;
  }
  if (iterations) *iterations += it;
  return norm_inf(r);
}

void bounded_nodes(int n, int q, double *nodes, double *logerr) {
  // uniform auxiliary start: the N interval midpoints of [-1, 1]
  Vec theta(n);
  {
    Vec gaps(n + 1);
    double prev = -1.0;
    for (int i = 0; i <= n; ++i) {
      const double x = i < n ? -1.0 + (2.0 * i + 1.0) / n : 1.0;
      gaps[i] = x - prev;
      prev = x;
    }
    for (int i = 0; i < n; ++i) theta[i] = std::log(gaps[i] / gaps[n]);
  }
  int its = 0;
  for (int o = 2; o <= q; ++o) {
    const double res = newton_order(theta, o, &its);
    if (!std::isfinite(res) || res > 1e-9)
      fail(TLR_ERR_RULE, "FD-q node solve failed at a continuation order: ||residual||_inf=%.3e",
           res);
  }
  const Aux a = aux_from(theta);
  const EqualError d = equal_error(a.x, q);
  for (int i = 0; i <= n; ++i) {
    nodes[i] = 0.5 * (d.nodes[i] - d.nodes[n - i]);
    logerr[i] = 0.5 * (d.logerr[i] + d.logerr[n - i]);
  }
  nodes[0] = -1.0;
  nodes[n] = 1.0;
  // fdq_nodes.py:197-216
  double sym = 0.0, eq = 0.0;
  for (int i = 0; i <= n; ++i) {
    if (!std::isfinite(nodes[i]) || !std::isfinite(logerr[i]))
      fail(TLR_ERR_RULE, "FD-q nodes and diagnostics must be finite");
    if (i < n && !(nodes[i + 1] > nodes[i]))
      fail(TLR_ERR_RULE, "FD-q nodes must be strictly increasing");
    sym = std::max(sym, std::fabs(nodes[i] + nodes[n - i]));
    if (i < n) eq = std::max(eq, std::fabs(logerr[i + 1] - logerr[i]));
  }
  if (sym > 5e-11) fail(TLR_ERR_RULE, "FD-q nodes are not symmetric: error=%.3e", sym);
  if (eq > 1e-9) fail(TLR_ERR_RULE, "FD-q equal-error validation failed: residual=%.3e", eq);
}

// Weights w[k][j], k = 0..2, of the derivative-k formula at x0 over the
// points z[0..m-1] (Fornberg's recursion: the weights for the first i + 1
// points are updated from those for the first i points).
void fornberg(double x0, const double *z, int m, double *w /* [3][m] */) {
  const int kmax = 2;
  for (int i = 0; i < 3 * m; ++i) w[i] = 0.0;
  auto W = [&](int k, int j) -> double & { return w[k * m + j]; };
  W(0, 0) = 1.0;
  double prod_prev = 1.0;  // prod_{j < i-1} (z_{i-1} - z_j)
  double dx_prev = z[0] - x0;
  for (int i = 1; i < m; ++i) {
    const int kl = std::min(i, kmax);
    double prod = 1.0;
    const double dx_last = dx_prev;  // z_{i-1} - x0
    const double dx = z[i] - x0;
    for (int j = 0; j < i; ++j) {
      const double dz = z[i] - z[j];
      prod *= dz;
      if (j == i - 1) {
        // new point i from the old weights of point i - 1
        for (int k = kl; k >= 1; --k)
          W(k, i) = prod_prev * (k * W(k - 1, i - 1) - dx_last * W(k, i - 1)) / prod;
        W(0, i) = -prod_prev * dx_last * W(0, i - 1) / prod;
      }
      for (int k = kl; k >= 1; --k) W(k, j) = (dx * W(k, j) - k * W(k - 1, j)) / dz;
      W(0, j) = dx * W(0, j) / dz;
    }
    prod_prev = prod;
    dx_prev = dx;
  }
}

// Polynomial-moment and stencil checks of fdq_nodes.py:396-455.
void check_rule(int nc, int q, int periodic, double period, const double *nodes,
                const int *idx, const int *off, const double *w) {
  const int s = q + 1;
  const double h = period / nc;
  for (int i = 0; i < nc; ++i) {
    bool self = false;
    for (int j = 0; j < s; ++j) {
      const int c = idx[i * s + j];
      if (c < 0 || c >= nc) fail(TLR_ERR_RULE, "stencil_indices contain an out-of-range column");
      if (periodic) {
        if (((i + off[i * s + j]) % nc + nc) % nc != c || off[i * s + j] != j - q / 2)
          fail(TLR_ERR_RULE, "periodic stencil indices and offsets are inconsistent");
      } else {
        if (c - i != off[i * s + j] || (j > 0 && c != idx[i * s + j - 1] + 1))
          fail(TLR_ERR_RULE, "bounded stencil offsets are inconsistent");
      }
      self |= c == i;
    }
    if (!self) fail(TLR_ERR_RULE, "every FD-q stencil must contain its evaluation node");
  }
  for (int k = 0; k < 3; ++k)
    for (int p = 0; p <= q; ++p) {
      Vec expect(nc), approx(nc);
      double emax = 0.0;
      for (int i = 0; i < nc; ++i) {
        double c = 1.0;
        for (int f = 0; f < k; ++f) c *= (double)(p - f);
        expect[i] = p < k ? 0.0 : c * std::pow(nodes[i], p - k);
        emax = std::max(emax, std::fabs(expect[i]));
        double sum = 0.0;
        for (int j = 0; j < s; ++j) {
          const double x = periodic ? nodes[i] + h * off[i * s + j] : nodes[idx[i * s + j]];
          const double wv = w[((size_t)k * nc + i) * s + j];
          if (!std::isfinite(wv)) fail(TLR_ERR_RULE, "FD-q weights must be finite");
          sum += wv * std::pow(x, p);
        }
        approx[i] = sum;
      }
      const double atol = 2e-8 * std::max(1.0, emax);
      for (int i = 0; i < nc; ++i)
        if (std::fabs(approx[i] - expect[i]) > atol + 2e-8 * std::fabs(expect[i]))
          fail(TLR_ERR_RULE, "FD-q weights fail the polynomial test: error=%.3e",
               std::fabs(approx[i] - expect[i]));
    }
}

}  // namespace

extern "C" int tlr_fdq_rule(int node_count, int q, int periodic, double period, double *nodes,
                            int *stencil_indices, int *stencil_offsets, double *weights,
                            double *log_error) {
  try {
    if (!nodes || !stencil_indices || !stencil_offsets || !weights)
      fail(TLR_ERR_ARG, "null output array");
    const int s = q + 1;
    if (periodic) {
      // fdq_nodes.py:307-330
      if (node_count < 3) fail(TLR_ERR_ARG, "node_count must be at least 3");
      if (q < 2 || q >= node_count) fail(TLR_ERR_ARG, "periodic q must satisfy 2 <= q < node_count");
      if (q % 2) fail(TLR_ERR_ARG, "periodic q must be even for a centered stencil");
      if (!std::isfinite(period) || period <= 0.0)
        fail(TLR_ERR_ARG, "period must be finite and positive");
      const double h = period / node_count, origin = -0.5 * period;
      for (int i = 0; i < node_count; ++i) nodes[i] = origin + h * i;
      Vec z(s), wv(3 * s);
      for (int i = 0; i < node_count; ++i) {
        for (int j = 0; j < s; ++j) {
          const int o = j - q / 2;
          stencil_offsets[i * s + j] = o;
          stencil_indices[i * s + j] = ((i + o) % node_count + node_count) % node_count;
          z[j] = nodes[i] + h * o;
        }
        fornberg(nodes[i], z.data(), s, wv.data());
        for (int k = 0; k < 3; ++k)
          for (int j = 0; j < s; ++j)
            weights[((size_t)k * node_count + i) * s + j] = wv[k * s + j];
      }
      if (log_error)
        for (int i = 0; i < node_count; ++i) log_error[i] = 0.0;
      for (int i = 0; i + 1 < node_count; ++i)
        if (std::fabs(nodes[i + 1] - nodes[i] - h) > 2e-13 * std::max(1.0, h))
          fail(TLR_ERR_RULE, "periodic nodes must be uniformly spaced");
    } else {
      // fdq_nodes.py:49-62: N = node_count - 1 intervals, 2 <= q <= N
      const int n = node_count - 1;
      if (n < 2) fail(TLR_ERR_ARG, "N must be at least 2");
      if (q < 2 || q > n) fail(TLR_ERR_ARG, "q must satisfy 2 <= q <= N");
      period = 2.0;
      Vec le(node_count);
      bounded_nodes(n, q, nodes, le.data());
      if (log_error) std::copy(le.begin(), le.end(), log_error);
      Vec z(s), wv(3 * s);
      for (int i = 0; i < node_count; ++i) {
        const int st = std::clamp(i - q / 2, 0, node_count - q - 1);  // fdq_nodes.py:65-69
        for (int j = 0; j < s; ++j) {
          stencil_indices[i * s + j] = st + j;
          stencil_offsets[i * s + j] = st + j - i;
          z[j] = nodes[st + j];
        }
        fornberg(nodes[i], z.data(), s, wv.data());
        for (int k = 0; k < 3; ++k)
          for (int j = 0; j < s; ++j)
            weights[((size_t)k * node_count + i) * s + j] = wv[k * s + j];
      }
    }
    check_rule(node_count, q, periodic, period, nodes, stencil_indices, stencil_offsets, weights);
  } catch (const RuleError &e) {
    tlr::set_global_error(e.msg);
    return e.status;
  }
  return TLR_OK;
}
