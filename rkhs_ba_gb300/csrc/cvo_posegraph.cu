// cvo_posegraph.cu -- FP64 SE(3) pose-graph solver (host code).
//
// The reference's pose graph (src/graph_optimizer/PoseGraph.cpp) adds a prior on the
// first keyframe (:321-345, sigmas 0.1 rad / 0.1 m), a between factor from the last
// keyframe to every new keyframe (:421-470, sigmas 0.3 rad / 0.1 m) and loop-closure
// between factors among keyframes (:367-419), and hands them to GTSAM (ISAM2 or a
// batch fixed-lag smoother, :471-495).  GTSAM is not available here; this solver
// minimises the same objective with its published factor definitions (GTSAM 4,
// Pose3 with the exponential-map retraction):
//   prior    e = Log(P^-1 X)                 (PriorFactor<Pose3>)
//   between  e = Log(Z^-1 (Xi^-1 Xj))        (BetweenFactor<Pose3>)
//   cost     1/2 sum |e ./ sigma|^2,  e = (omega, rho) rotation first
// by Levenberg-Marquardt over X <- X Exp(delta), with Jacobians by central
// differences of the FP64 error and a dense Cholesky solve of the 6N x 6N normal
// equations.  The result is the batch optimum that ISAM2's estimate converges to;
// the fixed-lag smoother's marginalisation of old keyframes is not reproduced.
#include <cmath>
#include <cstring>
#include <map>
#include <vector>
#include "cvo_internal.h"

namespace cvo_gb {

namespace {

struct Pose {
  double R[9];   // row-major
  double t[3];
};

Pose pose_from12(const double *p) {
  Pose X;
  for (int r = 0; r < 3; r++) {
    for (int c = 0; c < 3; c++) X.R[3 * r + c] = p[4 * r + c];
    X.t[r] = p[4 * r + 3];
  }
  return X;
}

void pose_to12(const Pose &X, double *p) {
  for (int r = 0; r < 3; r++) {
    for (int c = 0; c < 3; c++) p[4 * r + c] = X.R[3 * r + c];
    p[4 * r + 3] = X.t[r];
  }
}

Pose compose(const Pose &A, const Pose &B) {
  Pose C;
  for (int r = 0; r < 3; r++) {
    for (int c = 0; c < 3; c++)
      C.R[3 * r + c] = A.R[3 * r] * B.R[c] + A.R[3 * r + 1] * B.R[3 + c] + A.R[3 * r + 2] * B.R[6 + c];
    C.t[r] = A.R[3 * r] * B.t[0] + A.R[3 * r + 1] * B.t[1] + A.R[3 * r + 2] * B.t[2] + A.t[r];
  }
  return C;
}

Pose inverse(const Pose &A) {
  Pose B;
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) B.R[3 * r + c] = A.R[3 * c + r];
  for (int r = 0; r < 3; r++) B.t[r] = -(B.R[3 * r] * A.t[0] + B.R[3 * r + 1] * A.t[1] + B.R[3 * r + 2] * A.t[2]);
  return B;
}

// hat(w) * v and hat(w)^2 * v
void cross3(const double *a, const double *b, double *o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

// Rotation logarithm (angle-axis vector), robust near 0 and near pi.
void so3_log(const double *R, double *w) {
  const double tr = R[0] + R[4] + R[8];
  const double c = std::max(-1.0, std::min(1.0, 0.5 * (tr - 1.0)));
  const double v[3] = {R[7] - R[5], R[2] - R[6], R[3] - R[1]};   // 2 sin(theta) axis
  if (c > 1.0 - 1e-10) {
    // theta ~ 0: first order plus the cubic term of theta / sin(theta)
    const double s2 = 0.25 * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    const double f = 0.5 * (1.0 + s2 / 6.0);
    for (int k = 0; k < 3; k++) w[k] = f * v[k];
    return;
  }
  const double theta = std::acos(c);
  if (c < -0.999) {
    // theta ~ pi: axis from the largest diagonal of (R + I) / 2 = a a^T (1 - cos) / 2 + cos I ...
    int k = 0;
    if (R[4] > R[0]) k = 1;
    if (R[8] > R[3 * k + k]) k = 2;
    double a[3];
    const double d = std::sqrt(std::max(0.0, (R[3 * k + k] - c) / (1.0 - c)));
    a[k] = d;
    for (int j = 0; j < 3; j++)
      if (j != k) a[j] = (R[3 * k + j] + R[3 * j + k]) / (2.0 * (1.0 - c) * d);
    // sign from the antisymmetric part (sin(theta) > 0 for theta < pi)
    const double dot = a[0] * v[0] + a[1] * v[1] + a[2] * v[2];
    const double sgn = dot < 0.0 ? -1.0 : 1.0;
    const double na = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    for (int j = 0; j < 3; j++) w[j] = sgn * theta * a[j] / na;
    return;
  }
  const double f = theta / (2.0 * std::sin(theta));
  for (int k = 0; k < 3; k++) w[k] = f * v[k];
}

// SE(3) logarithm: xi = (omega, rho), t = V(omega) rho.
void se3_log(const Pose &X, double *xi) {
  double w[3];
  so3_log(X.R, w);
  const double th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  const double th = std::sqrt(th2);
  // V^-1 = I - 1/2 W + k W^2,  k = (1 - th sin(th) / (2 (1 - cos th))) / th^2
  double k;
  if (th < 1e-5) k = 1.0 / 12.0 + th2 / 720.0;
  else k = (1.0 - th * std::sin(th) / (2.0 * (1.0 - std::cos(th)))) / th2;
  double wt[3], wwt[3];
  cross3(w, X.t, wt);
  cross3(w, wt, wwt);
  for (int j = 0; j < 3; j++) {
    xi[j] = w[j];
    xi[3 + j] = X.t[j] - 0.5 * wt[j] + k * wwt[j];
  }
}

Pose se3_exp(const double *xi) {
  const double *w = xi, *rho = xi + 3;
  const double th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  const double th = std::sqrt(th2);
  double A, B, C;   // sin/th, (1-cos)/th^2, (th - sin)/th^3
  if (th < 1e-5) {
    A = 1.0 - th2 / 6.0;
    B = 0.5 - th2 / 24.0;
    C = 1.0 / 6.0 - th2 / 120.0;
  } else {
    A = std::sin(th) / th;
    B = (1.0 - std::cos(th)) / th2;
    C = (th - std::sin(th)) / (th2 * th);
  }
  const double W[9] = {0, -w[2], w[1], w[2], 0, -w[0], -w[1], w[0], 0};
  double W2[9];
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) W2[3 * r + c] = W[3 * r] * W[c] + W[3 * r + 1] * W[3 + c] + W[3 * r + 2] * W[6 + c];
  Pose X;
  for (int i = 0; i < 9; i++) {
    const double I = (i % 4 == 0) ? 1.0 : 0.0;
    X.R[i] = I + A * W[i] + B * W2[i];
  }
  for (int r = 0; r < 3; r++) {
    double s = rho[r];
    for (int c = 0; c < 3; c++) s += B * W[3 * r + c] * rho[c] + C * W2[3 * r + c] * rho[c];
    X.t[r] = s;
  }
  return X;
}

Pose retract(const Pose &X, const double *d) { return compose(X, se3_exp(d)); }

struct Factor {
  int kind;            // 0 prior, 1 between
  long long a, b;      // keys (b unused for a prior)
  Pose Z;              // measurement (prior pose or relative pose)
  double isig[6];      // 1 / sigma
};

void factor_error(const Factor &f, const Pose &Xa, const Pose &Xb, double *e) {
  Pose E = f.kind == 0 ? compose(inverse(f.Z), Xa) : compose(inverse(f.Z), compose(inverse(Xa), Xb));
  se3_log(E, e);
  for (int k = 0; k < 6; k++) e[k] *= f.isig[k];
}

// Dense Cholesky solve of A x = b (A symmetric positive definite, n x n, row-major);
// returns false if A is not positive definite.
bool chol_solve(int n, std::vector<double> &A, std::vector<double> &b) {
  for (int j = 0; j < n; j++) {
    double s = A[(size_t)j * n + j];
    for (int k = 0; k < j; k++) s -= A[(size_t)j * n + k] * A[(size_t)j * n + k];
    if (!(s > 0.0)) return false;
    const double d = std::sqrt(s);
    A[(size_t)j * n + j] = d;
    for (int i = j + 1; i < n; i++) {
      double t = A[(size_t)i * n + j];
      for (int k = 0; k < j; k++) t -= A[(size_t)i * n + k] * A[(size_t)j * n + k];
      A[(size_t)i * n + j] = t / d;
    }
  }
  for (int i = 0; i < n; i++) {
    double s = b[i];
    for (int k = 0; k < i; k++) s -= A[(size_t)i * n + k] * b[k];
    b[i] = s / A[(size_t)i * n + i];
  }
  for (int i = n - 1; i >= 0; i--) {
    double s = b[i];
    for (int k = i + 1; k < n; k++) s -= A[(size_t)k * n + i] * b[k];
    b[i] = s / A[(size_t)i * n + i];
  }
  return true;
}

}  // namespace

struct PoseGraphSolver {
  std::map<long long, int> index;   // key -> variable slot
  std::vector<long long> keys;
  std::vector<Pose> X;
  std::vector<Factor> factors;
  bool has_prior = false;

  double cost(const std::vector<Pose> &V) const {
    double c = 0.0, e[6];
    for (const Factor &f : factors) {
      factor_error(f, V[index.at(f.a)], f.kind == 1 ? V[index.at(f.b)] : V[index.at(f.a)], e);
      for (int k = 0; k < 6; k++) c += 0.5 * e[k] * e[k];
    }
    return c;
  }

  // Levenberg-Marquardt; returns 0, or a status for a graph without a prior.
  int optimize(int max_iters, double *c0_out, double *c1_out, int *iters_out) {
    const int n = (int)X.size(), dim = 6 * n;
    double c = cost(X);
    if (c0_out) *c0_out = c;
    int it = 0;
    if (n == 0 || factors.empty()) {
      if (c1_out) *c1_out = c;
      if (iters_out) *iters_out = 0;
      return CVO_OK;
    }
    if (!has_prior) return CVO_ERR_UNSUPPORTED;   // gauge freedom: the normal equations are singular
    double lambda = 1e-4;
    const double h = 1e-6;
    std::vector<double> H, g, Hd, gd;
    for (; it < max_iters; it++) {
      // normal equations J^T J, J^T e with central-difference Jacobians per variable block
      H.assign((size_t)dim * dim, 0.0);
      g.assign(dim, 0.0);
      for (const Factor &f : factors) {
        const int ia = index.at(f.a), ib = f.kind == 1 ? index.at(f.b) : ia;
        double e[6];
        factor_error(f, X[ia], X[ib], e);
        const int nv = f.kind == 1 ? 2 : 1;
        const int slot[2] = {ia, ib};
        double J[2][6][6];   // J[v][row][col]
        for (int v = 0; v < nv; v++)
          for (int col = 0; col < 6; col++) {
            double d[6] = {0, 0, 0, 0, 0, 0}, ep[6], em[6];
            d[col] = h;
            Pose Pp = retract(X[slot[v]], d);
            d[col] = -h;
            Pose Pm = retract(X[slot[v]], d);
            if (v == 0) {
              factor_error(f, Pp, f.kind == 1 ? X[ib] : Pp, ep);
              factor_error(f, Pm, f.kind == 1 ? X[ib] : Pm, em);
            } else {
              factor_error(f, X[ia], Pp, ep);
              factor_error(f, X[ia], Pm, em);
            }
            for (int row = 0; row < 6; row++) J[v][row][col] = (ep[row] - em[row]) / (2.0 * h);
          }
        for (int v = 0; v < nv; v++) {
          const int ov = 6 * slot[v];
          for (int p = 0; p < 6; p++) {
            double s = 0.0;
            for (int r = 0; r < 6; r++) s += J[v][r][p] * e[r];
            g[ov + p] += s;
          }
          for (int u = 0; u < nv; u++) {
            const int ou = 6 * slot[u];
            for (int p = 0; p < 6; p++)
              for (int q = 0; q < 6; q++) {
                double s = 0.0;
                for (int r = 0; r < 6; r++) s += J[v][r][p] * J[u][r][q];
                H[(size_t)(ov + p) * dim + ou + q] += s;
              }
          }
        }
      }
      bool accepted = false;
      for (int tries = 0; tries < 12 && !accepted; tries++) {
        Hd = H;
        gd.assign(dim, 0.0);
        for (int i = 0; i < dim; i++) {
          Hd[(size_t)i * dim + i] += lambda * std::max(H[(size_t)i * dim + i], 1e-12);
          gd[i] = -g[i];
        }
        if (!chol_solve(dim, Hd, gd)) {
          lambda *= 10.0;
          continue;
        }
        std::vector<Pose> Xn(n);
        for (int i = 0; i < n; i++) Xn[i] = retract(X[i], &gd[6 * i]);
        const double cn = cost(Xn);
        if (cn <= c) {
          double step2 = 0.0;
          for (double v : gd) step2 += v * v;
          const double dc = c - cn;
          X.swap(Xn);
          c = cn;
          lambda = std::max(lambda / 10.0, 1e-12);
          accepted = true;
          if (dc <= 1e-12 * std::max(c, 1e-300) || step2 < 1e-20) {
            it++;
            if (c1_out) *c1_out = c;
            if (iters_out) *iters_out = it;
            return CVO_OK;
          }
        } else {
          lambda *= 10.0;
        }
      }
      if (!accepted) break;   // no step lowers the cost: converged to the solver's precision
    }
    if (c1_out) *c1_out = c;
    if (iters_out) *iters_out = it;
    return CVO_OK;
  }
};

}  // namespace cvo_gb

using namespace cvo_gb;

struct cvo_pose_graph { PoseGraphSolver s; };

static bool valid_sigmas(const double *s) {
  if (!s) return false;
  for (int k = 0; k < 6; k++)
    if (!(s[k] > 0.0) || !std::isfinite(s[k])) return false;
  return true;
}

static bool finite12(const double *p) {
  if (!p) return false;
  for (int k = 0; k < 12; k++)
    if (!std::isfinite(p[k])) return false;
  return true;
}

extern "C" int cvo_pose_graph_create(cvo_pose_graph **out) try {
  if (!out) return CVO_ERR_INVALID_ARG;
  *out = new cvo_pose_graph();
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_pose_graph_destroy(cvo_pose_graph *g) try {
  delete g;
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_pose_graph_insert(cvo_pose_graph *g, int64_t key, const double pose[12]) try {
  if (!g || !finite12(pose)) return CVO_ERR_INVALID_ARG;
  PoseGraphSolver &s = g->s;
  auto it = s.index.find(key);
  if (it != s.index.end()) {
    s.X[it->second] = pose_from12(pose);
  } else {
    s.index[key] = (int)s.X.size();
    s.keys.push_back(key);
    s.X.push_back(pose_from12(pose));
  }
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_pose_graph_add_prior(cvo_pose_graph *g, int64_t key, const double pose[12], const double sigmas[6]) try {
  if (!g || !finite12(pose) || !valid_sigmas(sigmas)) return CVO_ERR_INVALID_ARG;
  if (g->s.index.find(key) == g->s.index.end()) return CVO_ERR_INVALID_ARG;
  Factor f;
  f.kind = 0;
  f.a = f.b = key;
  f.Z = pose_from12(pose);
  for (int k = 0; k < 6; k++) f.isig[k] = 1.0 / sigmas[k];
  g->s.factors.push_back(f);
  g->s.has_prior = true;
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_pose_graph_add_between(cvo_pose_graph *g, int64_t from, int64_t to, const double rel[12],
                                          const double sigmas[6]) try {
  if (!g || !finite12(rel) || !valid_sigmas(sigmas) || from == to) return CVO_ERR_INVALID_ARG;
  if (g->s.index.find(from) == g->s.index.end() || g->s.index.find(to) == g->s.index.end()) return CVO_ERR_INVALID_ARG;
  Factor f;
  f.kind = 1;
  f.a = from;
  f.b = to;
  f.Z = pose_from12(rel);
  for (int k = 0; k < 6; k++) f.isig[k] = 1.0 / sigmas[k];
  g->s.factors.push_back(f);
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_pose_graph_optimize(cvo_pose_graph *g, int max_iters, double *initial_cost, double *final_cost,
                                       int *iters) try {
  if (!g || max_iters < 0) return CVO_ERR_INVALID_ARG;
  return g->s.optimize(max_iters, initial_cost, final_cost, iters);
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_pose_graph_get(const cvo_pose_graph *g, int64_t key, double pose[12]) try {
  if (!g || !pose) return CVO_ERR_INVALID_ARG;
  auto it = g->s.index.find(key);
  if (it == g->s.index.end()) return CVO_ERR_INVALID_ARG;
  pose_to12(g->s.X[it->second], pose);
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_pose_graph_size(const cvo_pose_graph *g, int *n_poses, int *n_factors) try {
  if (!g) return CVO_ERR_INVALID_ARG;
  if (n_poses) *n_poses = (int)g->s.X.size();
  if (n_factors) *n_factors = (int)g->s.factors.size();
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_pose_graph_cost(const cvo_pose_graph *g, double *cost) try {
  if (!g || !cost) return CVO_ERR_INVALID_ARG;
  *cost = g->s.cost(g->s.X);
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}
