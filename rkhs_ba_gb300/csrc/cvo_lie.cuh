// cvo_lie.cuh -- device SE(3) helpers and the step-size root rule.
#pragma once
#include <cfloat>
#include "cvo_device.cuh"

namespace cvo_gb {

// Roots of c3 s^3 + c2 s^2 + c1 s + c0 in closed form (Cardano / trigonometric).
// Returns false for a degenerate cubic (c3 == 0 or non-finite coefficients),
// the case in which the reference's companion-matrix eigen-solve yields NaN
// (poly_solver_order3, src/cvo/LieGroup.cpp:310-326).
__host__ __device__ inline bool cubic_roots(double c3, double c2, double c1, double c0, double re[3], double im[3]) {
  if (c3 == 0.0 || !isfinite(c3) || !isfinite(c2) || !isfinite(c1) || !isfinite(c0)) return false;
  double a = c2 / c3, b = c1 / c3, c = c0 / c3;
  if (!isfinite(a) || !isfinite(b) || !isfinite(c)) return false;
  double a3 = a / 3.0;
  double pp = b - a * a3;
  double qq = 2.0 * a3 * a3 * a3 - a3 * b + c;
  double disc = 0.25 * qq * qq + pp * pp * pp / 27.0;
  if (disc > 0.0) {
    double sd = sqrt(disc);
    double uu = cbrt(-0.5 * qq + sd);
    double vv = cbrt(-0.5 * qq - sd);
    re[0] = uu + vv - a3; im[0] = 0.0;
    re[1] = -0.5 * (uu + vv) - a3; im[1] = 0.5 * sqrt(3.0) * (uu - vv);
    re[2] = re[1]; im[2] = -im[1];
  } else if (pp == 0.0) {
    double r = cbrt(-qq);
    re[0] = re[1] = re[2] = r - a3;
    im[0] = im[1] = im[2] = 0.0;
  } else {
    double mm = 2.0 * sqrt(-pp / 3.0);
    double arg = 3.0 * qq / (pp * mm);
    if (arg > 1.0) arg = 1.0;
    if (arg < -1.0) arg = -1.0;
    double th = acos(arg) / 3.0;
    const double two_pi_3 = 2.0943951023931957;
    for (int k = 0; k < 3; k++) { re[k] = mm * cos(th - two_pi_3 * k) - a3; im[k] = 0.0; }
  }
  return true;
}

// Step rule of compute_step_size (src/cvo/CvoGPU.cu:504-538): smallest positive
// real root of 4E s^3 + 3D s^2 + 2C s + B with |imag| < 1e-5, then clamped to
// [min_step, max_step]; no admissible root gives max_step.
__host__ __device__ inline double step_from_terms(const double bcde[4], double min_step, double max_step) {
  double re[3], im[3];
  double temp = DBL_MAX;
  if (cubic_roots(4.0 * bcde[3], 3.0 * bcde[2], 2.0 * bcde[1], bcde[0], re, im)) {
    for (int t = 0; t < 3; t++)
      if (re[t] > 0 && re[t] < temp && fabs(im[t]) < 1e-5) temp = re[t];
  }
  if (temp > max_step) return max_step;
  if (temp < min_step) return min_step;
  return temp;
}

// Exp_SEK3 for a 6-vector (src/cvo/LieGroup.cpp:245-275) in float; X row-major 3x4.
__device__ inline void exp_sek3(const float v[6], float dt, float X[12]) {
  float w0 = v[0], w1 = v[1], w2 = v[2];
  float theta = __fsqrt_rn(fa(fa(fm(w0, w0), fm(w1, w1)), fm(w2, w2)));
  float R[9], Jl[9];
  if (theta < 1e-6f) {
    for (int t = 0; t < 9; t++) R[t] = Jl[t] = (t % 4 == 0) ? 1.f : 0.f;
  } else {
    float A[9] = {0.f, -w2, w1, w2, 0.f, -w0, -w1, w0, 0.f};
    float A2[9];
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++) {
        float s = fm(A[3 * r], A[c]);
        s = fa(s, fm(A[3 * r + 1], A[3 + c]));
        s = fa(s, fm(A[3 * r + 2], A[6 + c]));
        A2[3 * r + c] = s;
      }
    float theta2 = fm(theta, theta);
    float stheta = sinf(fm(dt, theta));
    float ctheta = cosf(fm(dt, theta));
    float omc = __fdiv_rn(fs(1.f, ctheta), theta2);
    float s1 = __fdiv_rn(stheta, theta);
    float s3 = __fdiv_rn(fs(fm(dt, theta), stheta), fm(theta2, theta));
    for (int t = 0; t < 9; t++) {
      float I = (t % 4 == 0) ? 1.f : 0.f;
      R[t] = fa(fa(I, fm(s1, A[t])), fm(omc, A2[t]));
      Jl[t] = fa(fa(fm(dt, I), fm(omc, A[t])), fm(s3, A2[t]));
    }
  }
  for (int r = 0; r < 3; r++) {
    for (int c = 0; c < 3; c++) X[4 * r + c] = R[3 * r + c];
    X[4 * r + 3] = fa(fa(fm(Jl[3 * r], v[3]), fm(Jl[3 * r + 1], v[4])), fm(Jl[3 * r + 2], v[5]));
  }
}

// ||log(T)|| of an SE(3) element (Sophus::SE3d::log().norm(), used by
// dist_se3_cpu, src/cvo/CvoGPU.cpp:28-33), in double.
__host__ __device__ inline double dist_se3(const double R[9], const double t[3]) {
  double tr = R[0] + R[4] + R[8];
  double cth = 0.5 * (tr - 1.0);
  if (cth > 1.0) cth = 1.0;
  if (cth < -1.0) cth = -1.0;
  double th = acos(cth);
  double vx = 0.5 * (R[7] - R[5]), vy = 0.5 * (R[2] - R[6]), vz = 0.5 * (R[3] - R[1]);
  double w[3];
  const double kPi = 3.141592653589793;
  if (th < 1e-7) {
    w[0] = vx; w[1] = vy; w[2] = vz;
  } else if (kPi - th < 1e-4) {
    double xx = sqrt(fmax(0.0, (R[0] + 1.0) * 0.5)), yy = sqrt(fmax(0.0, (R[4] + 1.0) * 0.5)),
           zz = sqrt(fmax(0.0, (R[8] + 1.0) * 0.5));
    if (xx >= yy && xx >= zz) { yy = (R[1] + R[3]) / (4.0 * xx); zz = (R[2] + R[6]) / (4.0 * xx); }
    else if (yy >= zz) { xx = (R[1] + R[3]) / (4.0 * yy); zz = (R[5] + R[7]) / (4.0 * yy); }
    else { xx = (R[2] + R[6]) / (4.0 * zz); yy = (R[5] + R[7]) / (4.0 * zz); }
    double nn = sqrt(xx * xx + yy * yy + zz * zz);
    double sgn = (vx * xx + vy * yy + vz * zz) < 0 ? -1.0 : 1.0;
    w[0] = sgn * th * xx / nn; w[1] = sgn * th * yy / nn; w[2] = sgn * th * zz / nn;
  } else {
    double f = th / sin(th);
    w[0] = f * vx; w[1] = f * vy; w[2] = f * vz;
  }
  double th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  double thn = sqrt(th2);
  double W[9] = {0, -w[2], w[1], w[2], 0, -w[0], -w[1], w[0], 0};
  double W2[9];
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) W2[3 * r + c] = W[3 * r] * W[c] + W[3 * r + 1] * W[3 + c] + W[3 * r + 2] * W[6 + c];
  double k2;
  if (thn < 1e-7) k2 = 1.0 / 12.0;
  else {
    double half = 0.5 * thn;
    k2 = (1.0 - thn * cos(half) / (2.0 * sin(half))) / th2;
  }
  double u[3];
  for (int r = 0; r < 3; r++) {
    double s = t[r];
    for (int c = 0; c < 3; c++) s += (-0.5 * W[3 * r + c] + k2 * W2[3 * r + c]) * t[c];
    u[r] = s;
  }
  return sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2] + th2);
}

}  // namespace cvo_gb
