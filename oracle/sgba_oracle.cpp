// sgba_oracle.cpp -- CPU FP64 restatement of sophus-rs's Schur-complement
// LM bundle-adjustment inner loop.
//
// TEST INFRASTRUCTURE ONLY: the checker and the timed CPU baseline.  The
// product never links or calls this file.  See sgba_oracle.h.
//
// Reference files restated (paths relative to the sophus-rs workspace):
//   crates/sophus_opt/src/nlls/optimizer_step.rs:366-437      step_nlls_inner
//   crates/sophus_opt/src/nlls/optimizer.rs:345-376,463-520   step/accept/reject/tolerances
//   crates/sophus_opt/src/nlls/optimizer_helpers.rs:159-185,309-321
//   crates/sophus_opt/src/nlls/linear_system/cost_system.rs:74-273
//   crates/sophus_opt/src/nlls/cost/cost_fn.rs:173-433         eval/sort/calc_total_cost
//   crates/sophus_opt/src/nlls/cost/compare_idx.rs:38-125
//   crates/sophus_opt/src/nlls/cost/evaluated_term.rs:52-57,286-327
//   crates/sophus_opt/src/robust_kernel.rs:13-35
//   crates/sophus_opt/src/nlls/functor_library/costs/pinhole_reprojection.rs:42-95
//   crates/sophus_lie/src/groups/rotation3.rs:176-182,363-387,449-492,575-577,761-778
//   crates/sophus_lie/src/groups/affine_group_template.rs:354-410,505-510
//   crates/sophus_lie/src/quaternion.rs:212-225
//   crates/sophus_lie/src/lie_group/lie_group_manifold.rs:33-35,57-64
//   crates/sophus_sensor/src/projections/perspective.rs:30-72
//   crates/sophus_sensor/src/distortions/affine.rs:50-108
//   crates/sophus_sensor/src/distortions/enhanced_unified.rs:55-215  EUCM camera
//   crates/sophus_opt/src/example_problems/ba_problem.rs:69-110     EUCM cost term (free intrinsics)
//   crates/sophus_solver/src/ldlt/schur_ldlt.rs:82-278,450-490,536-812  (range-space KKT)
//   crates/sophus_opt/src/nlls/linear_system/eq_system.rs:149-258  G^T lambda, -c, update_lambdas
//   crates/sophus_opt/src/example_problems/ba_scale_constraint.rs:57-100  TranslationNormConstraint
//   crates/sophus_opt/src/nlls/optimizer.rs:527-535             no gradient test with constraints
//   crates/sophus_opt/src/nlls/functor_library/costs/isometry3_prior.rs  Isometry3PriorCostTerm
//   crates/sophus_opt/src/nlls/functor_library/costs/pose_graph3.rs      PoseGraph3CostTerm
//   crates/sophus_lie/src/groups/rotation3.rs:389-410,778-800, affine_group_template.rs:362-370  SE(3) log
//   crates/sophus_autodiff/src/dual/dual_scalar.rs:400-420      dual atan2
//   crates/sophus_opt/src/nlls/cost/evaluated_term.rs:286-327   precision-weighted terms
//   crates/sophus_solver/src/ldlt/block_sparse_ldlt.rs:99-190,479-747
//   crates/sophus_solver/src/ldlt/dense_ldlt.rs:164-308
//   crates/sophus_solver/src/ldlt/block_diag_ldlt.rs:80-160
//   crates/sophus_solver/src/kernel.rs:84-106
//
// Deviations (documented; they change only rounding, never the algorithm):
//   * S is factored in natural block order; the reference orders blocks with
//     faer's AMD (third-party, not available here).  For the dense reduced
//     camera systems of the BA configurations the fill is identical.
//   * The 3x3 H_mm inverse is the cofactor/adjugate formula with the same
//     "determinant exactly zero => failure" rule as nalgebra's try_inverse.
//   * Bunch-Kaufman fallback for indefinite ill-conditioned pivot blocks is
//     not restated; such a block is reported as a solve failure (a reject).
//   * The small dense inverse of G S^-1 G^T is Gauss-Jordan with partial
//     pivoting where nalgebra's try_inverse uses closed forms up to 3x3.
#include "sgba_oracle.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <thread>
#include <vector>

namespace {

constexpr double kEps = 1e-6;            // sophus_autodiff EPS_F64 (linalg.rs:75)
constexpr double kLdltTolRel = 1e-12;    // BlockSparseLdlt::default tol_rel
constexpr double kMinPositive = DBL_MIN; // f64::MIN_POSITIVE

// ---------------------------------------------------------------------------
// Scalar abstraction: double, float, and a forward-mode dual number.
// ---------------------------------------------------------------------------
template <int N>
struct Dual {
  double v;
  double d[N];
  Dual() : v(0) { for (int i = 0; i < N; ++i) d[i] = 0; }
  Dual(double x) : v(x) { for (int i = 0; i < N; ++i) d[i] = 0; }  // NOLINT
};
template <int N> Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v + b.v); for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i]; return r; }
template <int N> Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v - b.v); for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i]; return r; }
template <int N> Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r(-a.v); for (int i = 0; i < N; ++i) r.d[i] = -a.d[i]; return r; }
template <int N> Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v * b.v); for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i]; return r; }
template <int N> Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v / b.v);
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] * b.v - a.v * b.d[i]) / (b.v * b.v);
  return r; }
template <int N> Dual<N> dsqrt(const Dual<N>& a) {
  double s = std::sqrt(a.v);
  Dual<N> r(s);
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / (2.0 * s);
  return r;
}
template <int N> Dual<N> dsin(const Dual<N>& a) {
  Dual<N> r(std::sin(a.v));
  double c = std::cos(a.v);
  for (int i = 0; i < N; ++i) r.d[i] = c * a.d[i];
  return r;
}
template <int N> Dual<N> dcos(const Dual<N>& a) {
  Dual<N> r(std::cos(a.v));
  double s = -std::sin(a.v);
  for (int i = 0; i < N; ++i) r.d[i] = s * a.d[i];
  return r;
}
// atan2(y, x): d/dy = x / (x^2 + y^2), d/dx = -y / (x^2 + y^2)
// (dual_scalar.rs:400-420).
template <int N> Dual<N> datan2(const Dual<N>& y, const Dual<N>& x) {
  Dual<N> r(std::atan2(y.v, x.v));
  const double inv = 1.0 / (y.v * y.v + x.v * x.v);
  for (int i = 0; i < N; ++i) r.d[i] = (x.v * y.d[i] - y.v * x.d[i]) * inv;
  return r;
}
template <int N> double val(const Dual<N>& a) { return a.v; }

inline double dsqrt(double a) { return std::sqrt(a); }
inline double dsin(double a) { return std::sin(a); }
inline double dcos(double a) { return std::cos(a); }
inline double val(double a) { return a; }
inline double datan2(double y, double x) { return std::atan2(y, x); }
inline float dsqrt(float a) { return std::sqrt(a); }
inline float val(float a) { return a; }

// ---------------------------------------------------------------------------
// SO(3) / SE(3) restated from sophus_lie.
// Params layout: [qw, qx, qy, qz, tx, ty, tz]; tangent layout [omega; nu].
// ---------------------------------------------------------------------------

// QuaternionImpl::mult (quaternion.rs:212-225)
template <class S>
void quat_mult(const S* a, const S* b, S* o) {
  S re = a[0] * b[0] - (a[1] * b[1] + a[2] * b[2] + a[3] * b[3]);
  // ivec = rhs_ivec*lhs_re + lhs_ivec*rhs_re + cross(lhs_ivec, rhs_ivec)
  S c0 = a[2] * b[3] - a[3] * b[2];
  S c1 = a[3] * b[1] - a[1] * b[3];
  S c2 = a[1] * b[2] - a[2] * b[1];
  S i0 = b[1] * a[0] + a[1] * b[0] + c0;
  S i1 = b[2] * a[0] + a[2] * b[0] + c1;
  S i2 = b[3] * a[0] + a[3] * b[0] + c2;
  o[0] = re; o[1] = i0; o[2] = i1; o[3] = i2;
}

// Rotation3Impl::matrix (rotation3.rs:449-492), row-major 3x3.
template <class S>
void rot_matrix(const S* q, S* m) {
  const S r = q[0], x = q[1], y = q[2], z = q[3];
  const S one(1.0), two(2.0);
  S two_x = two * x, two_y = two * y, two_z = two * z, two_r = two * r;
  S two_xx = two_x * x, two_yy = two_y * y, two_zz = two_z * z;
  S two_xy = two_x * y, two_xz = two_x * z, two_yz = two_y * z;
  S two_rx = two_r * x, two_ry = two_r * y, two_rz = two_r * z;
  m[0] = one - (two_yy + two_zz); m[1] = two_xy - two_rz; m[2] = two_xz + two_ry;
  m[3] = two_xy + two_rz; m[4] = one - (two_xx + two_zz); m[5] = two_yz - two_rx;
  m[6] = two_xz - two_ry; m[7] = two_yz + two_rx; m[8] = one - (two_xx + two_yy);
}

// Rotation3Impl::exp (rotation3.rs:363-387)
template <class S>
void so3_exp(const S* w, S* q) {
  S theta_sq = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  S theta_po4 = theta_sq * theta_sq;
  S imag, real;
  if (val(theta_sq) <= kEps * kEps) {
    imag = S(0.5) - S(1.0 / 48.0) * theta_sq + S(1.0 / 3840.0) * theta_po4;
    real = S(1.0) - S(1.0 / 8.0) * theta_sq + S(1.0 / 384.0) * theta_po4;
  } else {
    S theta = dsqrt(theta_sq);
    S half = S(0.5) * theta;
    imag = dsin(half) / theta;
    real = dcos(half);
  }
  q[0] = real; q[1] = imag * w[0]; q[2] = imag * w[1]; q[3] = imag * w[2];
}

// Rotation3Impl::mat_v (rotation3.rs:761-778).  Note the Taylor branch test is
// theta_sq <= EPS (not EPS^2), exactly as in the reference.
template <class S>
void so3_mat_v(const S* w, S* v) {
  S theta_sq = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  // hat(omega)
  S h[9] = {S(0.0), -w[2], w[1], w[2], S(0.0), -w[0], -w[1], w[0], S(0.0)};
  S h2[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      S acc = h[i * 3 + 0] * h[0 * 3 + j];
      acc = acc + h[i * 3 + 1] * h[1 * 3 + j];
      acc = acc + h[i * 3 + 2] * h[2 * 3 + j];
      h2[i * 3 + j] = acc;
    }
  if (val(theta_sq) <= kEps) {
    for (int i = 0; i < 9; ++i) v[i] = S(0.5) * h[i];
  } else {
    S theta = dsqrt(theta_sq);
    S a = (S(1.0) - dcos(theta)) / theta_sq;
    S b = (theta - dsin(theta)) / (theta_sq * theta);
    for (int i = 0; i < 9; ++i) v[i] = a * h[i] + b * h2[i];
  }
  v[0] = v[0] + S(1.0); v[4] = v[4] + S(1.0); v[8] = v[8] + S(1.0);
}

// HasDisambiguate for Rotation3 (rotation3.rs:176-182): keep w >= 0.
template <class S>
void disambiguate(S* q) {
  if (!(0.0 <= val(q[0]))) { for (int i = 0; i < 4; ++i) q[i] = -q[i]; }
}

// Rotation3 are_params_valid (rotation3.rs:314-319): | |q| - 1 | <= EPS.
template <class S>
bool quat_valid(const S* q) {
  double n = std::sqrt(val(q[0]) * val(q[0]) + val(q[1]) * val(q[1]) +
                       val(q[2]) * val(q[2]) + val(q[3]) * val(q[3]));
  return std::fabs(n - 1.0) <= kEps;
}

// AffineGroupTemplateImpl::exp (affine_group_template.rs:354-360)
template <class S>
void se3_exp(const S* xi, S* out) {
  so3_exp(xi, out);
  S v[9];
  so3_mat_v(xi, v);
  for (int i = 0; i < 3; ++i)
    out[4 + i] = v[i * 3 + 0] * xi[3] + v[i * 3 + 1] * xi[4] + v[i * 3 + 2] * xi[5];
  disambiguate(out);
}

// AffineGroupTemplateImpl::group_mul (affine_group_template.rs:387-396)
template <class S>
void se3_mul(const S* a, const S* b, S* out) {
  S q[4];
  quat_mult(a, b, q);
  S r[9];
  rot_matrix(a, r);
  for (int i = 0; i < 3; ++i)
    out[4 + i] = (r[i * 3 + 0] * b[4] + r[i * 3 + 1] * b[5] + r[i * 3 + 2] * b[6]) + a[4 + i];
  for (int i = 0; i < 4; ++i) out[i] = q[i];
  disambiguate(out);
}

// AffineGroupTemplateImpl::inverse (affine_group_template.rs:398-404)
template <class S>
void se3_inverse(const S* a, S* out) {
  S q[4] = {a[0], -a[1], -a[2], -a[3]};
  S r[9];
  rot_matrix(q, r);
  for (int i = 0; i < 3; ++i)
    out[4 + i] = -(r[i * 3 + 0] * a[4] + r[i * 3 + 1] * a[5] + r[i * 3 + 2] * a[6]);
  for (int i = 0; i < 4; ++i) out[i] = q[i];
  disambiguate(out);
}

// Rotation3Impl::log (rotation3.rs:389-410): 2 atan(|v| / w) v / |v| with
// the sign of w folded in, and its series 2 / w - (2/3) |v|^2 / w^3 when
// |v|^2 <= EPS^2.
template <class S>
void so3_log(const S* q, S* w) {
  const S* iv = q + 1;
  S sq = iv[0] * iv[0] + iv[1] * iv[1] + iv[2] * iv[2];
  S qw = q[0];
  S f;
  if (val(sq) <= kEps * kEps) {
    S wsq = qw * qw;
    f = S(2.0) / qw - S(2.0 / 3.0) * sq / (wsq * qw);
  } else {
    S n = dsqrt(sq);
    S sign = val(qw) <= 0.0 ? S(-1.0) : S(1.0);
    S at = sign * datan2(n, sign * qw);
    f = S(2.0) * at / n;
  }
  for (int i = 0; i < 3; ++i) w[i] = iv[i] * f;
}

// Rotation3Impl::mat_v_inverse (rotation3.rs:778-800): I - W/2 + c W^2 with
// c = (1 - (theta/2) cos(theta/2) / sin(theta/2)) / theta^2, and c = 1/12 when
// theta^2 <= EPS.  m row-major.
template <class S>
void so3_mat_v_inverse(const S* w, S* m) {
  S th_sq = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  const S zero(0.0);
  const S hat[9] = {zero, -w[2], w[1], w[2], zero, -w[0], -w[1], w[0], zero};
  S hat_sq[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      hat_sq[i * 3 + j] = hat[i * 3 + 0] * hat[0 * 3 + j] + hat[i * 3 + 1] * hat[1 * 3 + j] +
                          hat[i * 3 + 2] * hat[2 * 3 + j];
  S c;
  if (val(th_sq) <= kEps) {
    c = S(1.0 / 12.0);
  } else {
    S theta = dsqrt(th_sq);
    S half = S(0.5) * theta;
    c = (S(1.0) - (S(0.5) * theta * dcos(half)) / dsin(half)) / (theta * theta);
  }
  for (int i = 0; i < 9; ++i) m[i] = ((i % 4 == 0) ? S(1.0) : zero) - hat[i] * S(0.5) + hat_sq[i] * c;
}

// AffineGroupTemplateImpl::log (affine_group_template.rs:362-370): the
// rotation's log, then V^-1 t; tangent (w, v).
template <class S>
void se3_log(const S* a, S* xi) {
  so3_log<S>(a, xi);
  S m[9];
  so3_mat_v_inverse<S>(xi, m);
  for (int i = 0; i < 3; ++i) xi[3 + i] = m[i * 3 + 0] * a[4] + m[i * 3 + 1] * a[5] + m[i * 3 + 2] * a[6];
}

// Residual g = z - pi(T_wc^-1 * p_w)
// (pinhole_reprojection.rs:42-50; camera.rs:94-99; perspective.rs:30-39;
//  affine.rs:50-62)
template <class S>
void residual_generic(const S* pose, const S* p, const double* intr,
                      const double* uv, S* r, S* x_cam_out = nullptr, int model = ORA_CAMERA_PINHOLE) {
  S cw[7];
  se3_inverse(pose, cw);
  S rm[9];
  rot_matrix(cw, rm);
  S xc[3];
  for (int i = 0; i < 3; ++i)
    xc[i] = (rm[i * 3 + 0] * p[0] + rm[i * 3 + 1] * p[1] + rm[i * 3 + 2] * p[2]) + cw[4 + i];
  S u = xc[0] / xc[2];
  S v = xc[1] / xc[2];
  if (model == ORA_CAMERA_EUCM) {  // enhanced_unified.rs:59-88
    S rho = dsqrt(S(intr[5]) * (u * u + v * v) + S(1.0));
    S norm = S(intr[4]) * rho + S(1.0 - intr[4]);
    u = u / norm;
    v = v / norm;
  }
  S pu = u * S(intr[0]) + S(intr[2]);
  S pv = v * S(intr[1]) + S(intr[3]);
  r[0] = S(uv[0]) - pu;
  r[1] = S(uv[1]) - pv;
  if (x_cam_out) for (int i = 0; i < 3; ++i) x_cam_out[i] = xc[i];
}

// HuberKernel::apply / IsRobustKernel::weight (robust_kernel.rs:13-18,29-35)
inline double huber_apply(double delta, double x) {
  if (std::fabs(x) <= delta) return x * x;
  return 2.0 * delta * std::fabs(x) - delta * delta;
}
inline double huber_weight(double delta, double nrm) {
  if (nrm == 0.0) return 0.0;
  return std::sqrt(huber_apply(delta, nrm)) / nrm;
}

// One evaluated term (evaluated_term.rs:286-327 for (C, F, M) kinds):
// residual weighted by w; H blocks unweighted; cost = r~ . r~.
template <class R>
struct Term {
  R hpp[36];   // J_pose^T J_pose (6x6)
  R hmm[9];    // J_pt^T J_pt (3x3)
  R hmp[18];   // J_pt^T J_pose (3x6)  -- the stored lower block (point row, pose col)
  R gp[6];     // J_pose^T r~
  R gm[3];     // J_pt^T r~
  double cost;
};

// PinholeCameraReprojectionCostTerm::eval (pinhole_reprojection.rs:60-95)
// in f64: residual, d_pi*R_cw, J_pose = d_pi_r_cw * [hat(-p), I], J_pt = -d_pi_r_cw.
void eval_term_f64(const double* pose, const double* p, const double* intr,
                   const double* uv, double huber, double* r, double* jp,
                   double* jm, double* w_out, double* cost_out, double* jc = nullptr,
                   int model = ORA_CAMERA_PINHOLE) {
  double cw[7];
  se3_inverse(pose, cw);
  double rm[9];
  rot_matrix(cw, rm);
  double xc[3];
  for (int i = 0; i < 3; ++i)
    xc[i] = (rm[i * 3 + 0] * p[0] + rm[i * 3 + 1] * p[1] + rm[i * 3 + 2] * p[2]) + cw[4 + i];
  double dpi[6];  // dx_distort_x * dx_proj_x (2x3)
  if (model == ORA_CAMERA_EUCM) {
    // EnhancedUnifiedDistortionImpl::distort / dx_distort_x /
    // dx_distort_params (enhanced_unified.rs:59-88,117-156,158-215), on the
    // z = 1 projection (perspective.rs:30-39); J_cam is 2x6
    const double z = xc[2];
    const double x = xc[0] / z, y = xc[1] / z;
    const double fx = intr[0], fy = intr[1], alpha = intr[4], beta = intr[5];
    const double r2 = x * x + y * y;
    const double rho2 = beta * r2 + 1.0;
    const double rho = std::sqrt(rho2);
    const double norm = alpha * rho + (1.0 - alpha);
    const double mx = x / norm, my = y / norm;
    r[0] = uv[0] - (fx * mx + intr[2]);
    r[1] = uv[1] - (fy * my + intr[3]);
    const double drho_dx = (2.0 * beta * x) / (2.0 * rho);
    const double drho_dy = (2.0 * beta * y) / (2.0 * rho);
    const double dnorm_dx = alpha * drho_dx, dnorm_dy = alpha * drho_dy;
    const double n2 = norm * norm;
    const double dd[4] = {fx * ((norm - x * dnorm_dx) / n2), fx * (-x * dnorm_dy / n2),
                          fy * (-y * dnorm_dx / n2), fy * ((norm - y * dnorm_dy) / n2)};
    // dx_proj_x = [[1/z, 0, -x_c/z^2], [0, 1/z, -y_c/z^2]]
    const double pz[6] = {1.0 / z, 0.0, -xc[0] / (z * z), 0.0, 1.0 / z, -xc[1] / (z * z)};
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 3; ++j) dpi[i * 3 + j] = dd[i * 2 + 0] * pz[0 * 3 + j] + dd[i * 2 + 1] * pz[1 * 3 + j];
    if (jc) {
      const double drho_dbeta = r2 / (2.0 * rho);
      const double dnorm_dalpha = rho - 1.0, dnorm_dbeta = alpha * drho_dbeta;
      const double j[12] = {-mx, 0.0, -1.0, 0.0, -fx * (-x * dnorm_dalpha / n2), -fx * (-x * dnorm_dbeta / n2),
                            0.0, -my, 0.0, -1.0, -fy * (-y * dnorm_dalpha / n2), -fy * (-y * dnorm_dbeta / n2)};
      for (int i = 0; i < 12; ++i) jc[i] = j[i];
    }
  } else {
    double u = xc[0] / xc[2], v = xc[1] / xc[2];
    r[0] = uv[0] - (u * intr[0] + intr[2]);
    r[1] = uv[1] - (v * intr[1] + intr[3]);
    if (jc) {
      // J_cam = -dx_distort_params(proj) (pinhole_reprojection.rs:85;
      // affine.rs:77-108): params (fx, fy, cx, cy), 2x4 row-major
      const double j[8] = {-u, 0.0, -1.0, 0.0, 0.0, -v, 0.0, -1.0};
      for (int i = 0; i < 8; ++i) jc[i] = j[i];
    }
    double z = xc[2];
    const double dp[6] = {intr[0] * (1.0 / z), 0.0, intr[0] * (-xc[0] / (z * z)),
                          0.0, intr[1] * (1.0 / z), intr[1] * (-xc[1] / (z * z))};
    for (int i = 0; i < 6; ++i) dpi[i] = dp[i];
  }
  double d[6];  // d_pi * R_cw (2x3)
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 3; ++j)
      d[i * 3 + j] = dpi[i * 3 + 0] * rm[0 * 3 + j] + dpi[i * 3 + 1] * rm[1 * 3 + j] +
                     dpi[i * 3 + 2] * rm[2 * 3 + j];
  // hat(-p) = [[0, p2, -p1], [-p2, 0, p0], [p1, -p0, 0]]
  const double hm[9] = {0.0, p[2], -p[1], -p[2], 0.0, p[0], p[1], -p[0], 0.0};
  for (int i = 0; i < 2; ++i) {
    for (int j = 0; j < 3; ++j)
      jp[i * 6 + j] = d[i * 3 + 0] * hm[0 * 3 + j] + d[i * 3 + 1] * hm[1 * 3 + j] +
                      d[i * 3 + 2] * hm[2 * 3 + j];
    for (int j = 0; j < 3; ++j) jp[i * 6 + 3 + j] = d[i * 3 + j];
    for (int j = 0; j < 3; ++j) jm[i * 3 + j] = -d[i * 3 + j];
  }
  double w = 1.0;
  double cost;
  if (huber > 0.0) {
    double nrm = std::sqrt(r[0] * r[0] + r[1] * r[1]);
    w = huber_weight(huber, nrm);
    double rw0 = w * r[0], rw1 = w * r[1];
    cost = rw0 * rw0 + rw1 * rw1;
  } else {
    cost = r[0] * r[0] + r[1] * r[1];
  }
  if (w_out) *w_out = w;
  if (cost_out) *cost_out = cost;
}

// Cost only (calc_total_cost treats every variable as Conditioned).
double eval_cost_f64(const double* pose, const double* p, const double* intr,
                     const double* uv, double huber, int model = ORA_CAMERA_PINHOLE) {
  double r[2];
  residual_generic<double>(pose, p, intr, uv, r, nullptr, model);
  if (huber > 0.0) {
    double nrm = std::sqrt(r[0] * r[0] + r[1] * r[1]);
    double w = huber_weight(huber, nrm);
    double rw0 = w * r[0], rw1 = w * r[1];
    return rw0 * rw0 + rw1 * rw1;
  }
  return r[0] * r[0] + r[1] * r[1];
}

template <class R>
void make_term(const double* pose, const double* p, const double* intr,
               const double* uv, double huber, Term<R>* t, int model = ORA_CAMERA_PINHOLE) {
  double r[2], jp[12], jm[6], w, cost;
  eval_term_f64(pose, p, intr, uv, huber, r, jp, jm, &w, &cost, nullptr, model);
  R Jp[12], Jm[6], rw[2];
  for (int i = 0; i < 12; ++i) Jp[i] = static_cast<R>(jp[i]);
  for (int i = 0; i < 6; ++i) Jm[i] = static_cast<R>(jm[i]);
  rw[0] = static_cast<R>(w * r[0]);
  rw[1] = static_cast<R>(w * r[1]);
  for (int a = 0; a < 6; ++a) {
    for (int b = 0; b < 6; ++b) t->hpp[a * 6 + b] = Jp[a] * Jp[b] + Jp[6 + a] * Jp[6 + b];
    t->gp[a] = Jp[a] * rw[0] + Jp[6 + a] * rw[1];
  }
  for (int a = 0; a < 3; ++a) {
    for (int b = 0; b < 3; ++b) t->hmm[a * 3 + b] = Jm[a] * Jm[b] + Jm[3 + a] * Jm[3 + b];
    for (int b = 0; b < 6; ++b) t->hmp[a * 6 + b] = Jm[a] * Jp[b] + Jm[3 + a] * Jp[6 + b];
    t->gm[a] = Jm[a] * rw[0] + Jm[3 + a] * rw[1];
  }
  t->cost = cost;
}

// The blocks of a term that involve Free intrinsics (kinds (F, F, M)), for
// nc = 4 (pinhole) or 6 (EUCM) params: J_cam^T J_cam (nc x nc), J_pose^T J_cam
// (pose row, intrinsics column, 6 x nc), J_pt^T J_cam (point row, 3 x nc)
// and J_cam^T r~, each row-major with row stride nc.
template <class R>
struct CamTerm {
  R hcc[36];
  R hpc[36];
  R hmc[18];
  R gc[6];
};

// make_term plus the intrinsics blocks (same arithmetic for the Term part).
template <class R>
void make_term_cam(const double* pose, const double* p, const double* intr,
                   const double* uv, double huber, Term<R>* t, CamTerm<R>* ct, int model, int nc) {
  double r[2], jp[12], jm[6], jc[12], w, cost;
  eval_term_f64(pose, p, intr, uv, huber, r, jp, jm, &w, &cost, jc, model);
  R Jp[12], Jm[6], Jc[12], rw[2];
  for (int i = 0; i < 12; ++i) Jp[i] = static_cast<R>(jp[i]);
  for (int i = 0; i < 6; ++i) Jm[i] = static_cast<R>(jm[i]);
  for (int i = 0; i < 2 * nc; ++i) Jc[i] = static_cast<R>(jc[i]);
  rw[0] = static_cast<R>(w * r[0]);
  rw[1] = static_cast<R>(w * r[1]);
  for (int a = 0; a < 6; ++a) {
    for (int b = 0; b < 6; ++b) t->hpp[a * 6 + b] = Jp[a] * Jp[b] + Jp[6 + a] * Jp[6 + b];
    t->gp[a] = Jp[a] * rw[0] + Jp[6 + a] * rw[1];
  }
  for (int a = 0; a < 3; ++a) {
    for (int b = 0; b < 3; ++b) t->hmm[a * 3 + b] = Jm[a] * Jm[b] + Jm[3 + a] * Jm[3 + b];
    for (int b = 0; b < 6; ++b) t->hmp[a * 6 + b] = Jm[a] * Jp[b] + Jm[3 + a] * Jp[6 + b];
    t->gm[a] = Jm[a] * rw[0] + Jm[3 + a] * rw[1];
  }
  t->cost = cost;
  *ct = CamTerm<R>{};
  for (int a = 0; a < nc; ++a) {
    for (int b = 0; b < nc; ++b) ct->hcc[a * nc + b] = Jc[a] * Jc[b] + Jc[nc + a] * Jc[nc + b];
    ct->gc[a] = Jc[a] * rw[0] + Jc[nc + a] * rw[1];
  }
  for (int a = 0; a < 6; ++a)
    for (int b = 0; b < nc; ++b) ct->hpc[a * nc + b] = Jp[a] * Jc[b] + Jp[6 + a] * Jc[nc + b];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < nc; ++b) ct->hmc[a * nc + b] = Jm[a] * Jc[b] + Jm[3 + a] * Jc[nc + b];
}

template <class R>
void cam_term_reduce(CamTerm<R>* a, const CamTerm<R>& b) {
  for (int i = 0; i < 36; ++i) a->hcc[i] += b.hcc[i];
  for (int i = 0; i < 36; ++i) a->hpc[i] += b.hpc[i];
  for (int i = 0; i < 18; ++i) a->hmc[i] += b.hmc[i];
  for (int i = 0; i < 6; ++i) a->gc[i] += b.gc[i];
}

template <class R>
void term_reduce(Term<R>* a, const Term<R>& b) {  // EvaluatedCostTerm::reduce
  for (int i = 0; i < 36; ++i) a->hpp[i] += b.hpp[i];
  for (int i = 0; i < 9; ++i) a->hmm[i] += b.hmm[i];
  for (int i = 0; i < 18; ++i) a->hmp[i] += b.hmp[i];
  for (int i = 0; i < 6; ++i) a->gp[i] += b.gp[i];
  for (int i = 0; i < 3; ++i) a->gm[i] += b.gm[i];
  a->cost += b.cost;
}

// nalgebra-style 3x3 try_inverse: cofactor/adjugate, fails iff det == 0.
template <class R>
bool inverse3(const R* m, R* o) {
  R m11 = m[0], m12 = m[1], m13 = m[2];
  R m21 = m[3], m22 = m[4], m23 = m[5];
  R m31 = m[6], m32 = m[7], m33 = m[8];
  R minor_m12_m23 = m22 * m33 - m32 * m23;
  R minor_m11_m23 = m21 * m33 - m31 * m23;
  R minor_m11_m22 = m21 * m32 - m31 * m22;
  R det = m11 * minor_m12_m23 - m12 * minor_m11_m23 + m13 * minor_m11_m22;
  if (det == R(0)) return false;
  o[0] = minor_m12_m23 / det;
  o[1] = (m13 * m32 - m33 * m12) / det;
  o[2] = (m12 * m23 - m22 * m13) / det;
  o[3] = -minor_m11_m23 / det;
  o[4] = (m11 * m33 - m31 * m13) / det;
  o[5] = (m13 * m21 - m23 * m11) / det;
  o[6] = minor_m11_m22 / det;
  o[7] = (m12 * m31 - m32 * m11) / det;
  o[8] = (m11 * m22 - m21 * m12) / det;
  return true;
}

// ---------------------------------------------------------------------------
// Dense LDLT of one diagonal block, PSD-aware (dense_ldlt.rs:164-270).
// a: n x n row-major (lower used); on return unit-lower L in a, d in d.
// Returns 0, -1 on a non-finite pivot, -2 if the block is indefinite with a
// pivot condition below the Bunch-Kaufman threshold (not restated).
// ---------------------------------------------------------------------------
int ldlt_decompose_inplace(int n, double* a, double* d, double rel_tol) {
  double max_abs_pivot = 1.0;
  double min_abs_pivot = DBL_MAX;
  int rank = 0;
  bool has_negative = false;
  for (int j = 0; j < n; ++j) {
    for (int k = 0; k < j; ++k) {
      double s = a[j * n + k];
      for (int p = 0; p < k; ++p) s -= a[j * n + p] * d[p] * a[k * n + p];
      double zero_tol = std::max(max_abs_pivot, 1.0) * rel_tol;
      a[j * n + k] = (std::fabs(d[k]) <= zero_tol) ? 0.0 : s / d[k];
    }
    double djj = a[j * n + j];
    for (int p = 0; p < j; ++p) {
      double ljp = a[j * n + p];
      djj -= d[p] * ljp * ljp;
    }
    if (!std::isfinite(djj)) return -1;
    double zero_tol = std::max(max_abs_pivot, 1.0) * rel_tol;
    if (std::fabs(djj) <= zero_tol) {
      d[j] = 0.0;
    } else {
      if (djj < 0.0) has_negative = true;
      d[j] = djj;
      double ad = std::fabs(djj);
      max_abs_pivot = std::max(max_abs_pivot, ad);
      min_abs_pivot = std::min(min_abs_pivot, ad);
      rank += 1;
    }
    a[j * n + j] = 1.0;
  }
  for (int r = 0; r < n; ++r)
    for (int c = r + 1; c < n; ++c) a[r * n + c] = 0.0;
  double pivot_condition = rank == 0 ? 0.0 : min_abs_pivot / max_abs_pivot;
  if (has_negative && pivot_condition < 1e-10) return -2;  // BK fallback (ldlt.rs:44)
  return 0;
}

// X <- X * (L D L^T)^-1 for an m x n block X (ldlt_right_matsolve_inplace,
// dense_ldlt.rs:300-308): X L^-T, then X D^-1 (PSD-aware), then X L^-1.
void ldlt_right_matsolve(int n, const double* l, const double* d, int m, double* x) {
  // X <- X L^{-T}: solve Y L^T = X row by row: y_j = x_j - sum_{k<j} y_k L[j,k]
  for (int r = 0; r < m; ++r) {
    double* row = x + r * n;
    for (int j = 0; j < n; ++j) {
      double s = row[j];
      for (int k = 0; k < j; ++k) s -= row[k] * l[j * n + k];
      row[j] = s;
    }
    for (int j = 0; j < n; ++j) row[j] = (d[j] == 0.0) ? 0.0 : row[j] / d[j];
    // X <- X L^{-1}: solve Y L = X: y_j = x_j - sum_{k>j} y_k L[k,j]
    for (int j = n - 1; j >= 0; --j) {
      double s = row[j];
      for (int k = j + 1; k < n; ++k) s -= row[k] * l[k * n + j];
      row[j] = s;
    }
  }
}

// y <- (L D L^T)^-1 y for one diagonal block (block_diag_ldlt.rs:118-133).
void ldlt_block_solve_vec(int n, const double* l, const double* d, double* y) {
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < i; ++k) y[i] -= l[i * n + k] * y[k];
  for (int i = 0; i < n; ++i) y[i] = (d[i] == 0.0) ? 0.0 : y[i] / d[i];
  for (int i = n - 1; i >= 0; --i)
    for (int k = i + 1; k < n; ++k) y[i] -= l[k * n + i] * y[k];
}

// Left-looking dense block LDLT in natural order (block_sparse_ldlt.rs:479-747
// without AMD): A (N x N row-major, lower used) with nb blocks of size bs.
struct BlockLdlt {
  int n = 0, bs = 0, nb = 0;
  std::vector<double> lblk;   // off-diagonal L blocks, dense nb x nb of bs x bs
  std::vector<double> ldiag;  // per diag block: unit lower L_jj (bs x bs)
  std::vector<double> d;      // n pivots

  int factorize(int n_, int bs_, const double* a) {
    n = n_; bs = bs_; nb = n / bs;
    lblk.assign(static_cast<size_t>(nb) * nb * bs * bs, 0.0);
    ldiag.assign(static_cast<size_t>(nb) * bs * bs, 0.0);
    d.assign(n, 0.0);
    std::vector<double> ccol(static_cast<size_t>(nb) * bs * bs);
    std::vector<double> qjk(bs * bs), qik(bs * bs);
    for (int j = 0; j < nb; ++j) {
      // load column j (blocks i >= j)
      for (int i = j; i < nb; ++i)
        for (int r = 0; r < bs; ++r)
          for (int c = 0; c < bs; ++c)
            ccol[(static_cast<size_t>(i) * bs + r) * bs + c] = a[(static_cast<size_t>(i) * bs + r) * n + j * bs + c];
      for (int k = 0; k < j; ++k) {
        const double* ljk = &lblk[((static_cast<size_t>(j) * nb + k) * bs) * bs];
        bool nz = false;
        for (int t = 0; t < bs * bs; ++t) if (ljk[t] != 0.0) { nz = true; break; }
        if (!nz) continue;  // L[j,k] absent: k not in the etree reach of j
        const double* lkk = &ldiag[static_cast<size_t>(k) * bs * bs];
        const double* dk = &d[static_cast<size_t>(k) * bs];
        // Q[j,k] = L[j,k] * L[k,k]
        for (int r = 0; r < bs; ++r)
          for (int c = 0; c < bs; ++c) {
            double s = 0.0;
            for (int t = 0; t < bs; ++t) s += ljk[r * bs + t] * lkk[t * bs + c];
            qjk[r * bs + c] = s;
          }
        for (int i = j; i < nb; ++i) {
          const double* qi;
          if (i == j) {
            qi = qjk.data();
          } else {
            const double* lik = &lblk[((static_cast<size_t>(i) * nb + k) * bs) * bs];
            bool nzi = false;
            for (int t = 0; t < bs * bs; ++t) if (lik[t] != 0.0) { nzi = true; break; }
            if (!nzi) continue;
            for (int r = 0; r < bs; ++r)
              for (int c = 0; c < bs; ++c) {
                double s = 0.0;
                for (int t = 0; t < bs; ++t) s += lik[r * bs + t] * lkk[t * bs + c];
                qik[r * bs + c] = s;
              }
            qi = qik.data();
          }
          // C(i,j) -= Q[i,k] diag(d_k) Q[j,k]^T
          double* cij = &ccol[static_cast<size_t>(i) * bs * bs];
          for (int r = 0; r < bs; ++r)
            for (int c = 0; c < bs; ++c) {
              double s = 0.0;
              for (int t = 0; t < bs; ++t) s += qi[r * bs + t] * dk[t] * qjk[c * bs + t];
              cij[r * bs + c] -= s;
            }
        }
      }
      // factor the diagonal block
      double* ljj = &ldiag[static_cast<size_t>(j) * bs * bs];
      std::memcpy(ljj, &ccol[static_cast<size_t>(j) * bs * bs], sizeof(double) * bs * bs);
      int st = ldlt_decompose_inplace(bs, ljj, &d[static_cast<size_t>(j) * bs], kLdltTolRel);
      if (st != 0) return st;
      for (int i = j + 1; i < nb; ++i) {
        double* cij = &ccol[static_cast<size_t>(i) * bs * bs];
        bool nz = false;
        for (int t = 0; t < bs * bs; ++t) if (cij[t] != 0.0) { nz = true; break; }
        if (!nz) continue;
        ldlt_right_matsolve(bs, ljj, &d[static_cast<size_t>(j) * bs], bs, cij);
        std::memcpy(&lblk[((static_cast<size_t>(i) * nb + j) * bs) * bs], cij, sizeof(double) * bs * bs);
      }
    }
    return 0;
  }

  // BlockSparseLdltFactor::solve_inplace (block_sparse_ldlt.rs:99-190)
  void solve(double* x) const {
    for (int j = 0; j < nb; ++j)
      for (int i = j + 1; i < nb; ++i) {
        const double* lij = &lblk[((static_cast<size_t>(i) * nb + j) * bs) * bs];
        for (int r = 0; r < bs; ++r) {
          double s = 0.0;
          for (int c = 0; c < bs; ++c) s += lij[r * bs + c] * x[j * bs + c];
          x[i * bs + r] -= s;
        }
      }
    for (int j = 0; j < nb; ++j)
      ldlt_block_solve_vec(bs, &ldiag[static_cast<size_t>(j) * bs * bs], &d[static_cast<size_t>(j) * bs], x + j * bs);
    for (int j = nb - 1; j >= 0; --j)
      for (int i = j + 1; i < nb; ++i) {
        const double* lij = &lblk[((static_cast<size_t>(i) * nb + j) * bs) * bs];
        for (int c = 0; c < bs; ++c) {
          double s = 0.0;
          for (int r = 0; r < bs; ++r) s += lij[r * bs + c] * x[i * bs + r];
          x[j * bs + c] -= s;
        }
      }
  }
};

// ---------------------------------------------------------------------------
// Problem structure: sorted terms, reduction ranges, active index maps.
// ---------------------------------------------------------------------------
struct Structure {
  int nc = 0, np = 0;
  int64_t no = 0;
  std::vector<int64_t> order;        // sorted term -> original obs index
  std::vector<int64_t> range_begin;  // reduction ranges over sorted terms
  std::vector<int> pose_block;       // pose -> free block idx or -1
  std::vector<int> point_block;      // point -> marg block idx or -1
  int nf = 0, nm = 0;
  // per reduction range: pose, point
  std::vector<int> rng_pose, rng_pt;
  // marg block -> list of reduction ranges (in order) -> used by Schur
  std::vector<int64_t> pt_rng_begin;  // ranges are sorted by point, so contiguous
};

// Params of the camera model: fx fy cx cy, then alpha beta for EUCM.
inline int cam_params(const ora_problem* p) { return p->camera_model == ORA_CAMERA_EUCM ? 6 : 4; }
inline void problem_intrinsics(const ora_problem* p, double* intr6) {
  for (int i = 0; i < 4; ++i) intr6[i] = p->intrinsics[i];
  intr6[4] = p->camera_model == ORA_CAMERA_EUCM ? p->eucm_alpha_beta[0] : 0.0;
  intr6[5] = p->camera_model == ORA_CAMERA_EUCM ? p->eucm_alpha_beta[1] : 0.0;
}

void build_structure(const ora_problem* p, Structure* s) {
  s->nc = p->n_cam; s->np = p->n_pt; s->no = p->n_obs;
  s->order.resize(p->n_obs);
  std::iota(s->order.begin(), s->order.end(), 0);
  // CostFn::sort (cost_fn.rs:354-393) with CompareIdx for kinds (c, f, m):
  // permuted key = (point, pose, intrinsics); stable sort.
  std::stable_sort(s->order.begin(), s->order.end(), [&](int64_t a, int64_t b) {
    if (p->obs_pt[a] != p->obs_pt[b]) return p->obs_pt[a] < p->obs_pt[b];
    return p->obs_cam[a] < p->obs_cam[b];
  });
  s->range_begin.clear(); s->rng_pose.clear(); s->rng_pt.clear();
  int64_t i = 0;
  while (i < p->n_obs) {
    int64_t o = s->order[i];
    int pt = p->obs_pt[o], ps = p->obs_cam[o];
    s->range_begin.push_back(i);
    s->rng_pose.push_back(ps); s->rng_pt.push_back(pt);
    while (i < p->n_obs && p->obs_pt[s->order[i]] == pt && p->obs_cam[s->order[i]] == ps) ++i;
  }
  s->range_begin.push_back(p->n_obs);
  s->pose_block.assign(p->n_cam, -1);
  s->nf = 0;
  for (int c = 0; c < p->n_cam; ++c)
    if (!(p->pose_const && p->pose_const[c])) s->pose_block[c] = s->nf++;
  s->point_block.assign(p->n_pt, -1);
  s->nm = 0;
  for (int q = 0; q < p->n_pt; ++q)
    if (!(p->point_const && p->point_const[q])) s->point_block[q] = s->nm++;
  // ranges grouped by point (sorted), index of first range per point
  s->pt_rng_begin.assign(p->n_pt + 1, 0);
  int64_t nr = static_cast<int64_t>(s->rng_pt.size());
  int64_t r = 0;
  for (int q = 0; q < p->n_pt; ++q) {
    s->pt_rng_begin[q] = r;
    while (r < nr && s->rng_pt[r] == q) ++r;
  }
  s->pt_rng_begin[p->n_pt] = nr;
}

template <class F>
void parallel_for(int64_t n, int n_threads, F&& f) {  // f(begin, end, thread_id)
  if (n_threads <= 1 || n < 1024) { f(int64_t(0), n, 0); return; }
  std::vector<std::thread> th;
  int64_t chunk = (n + n_threads - 1) / n_threads;
  for (int t = 0; t < n_threads; ++t) {
    int64_t b = t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    th.emplace_back([&f, b, e, t]() { f(b, e, t); });
  }
  for (auto& x : th) x.join();
}

// Isometry3PriorCostTerm::eval (isometry3_prior.rs): g = log(T E^-1), J the
// dual-number derivative of log(exp(x) T E^-1) at x = 0, then
// EvaluatedCostTerm::make with the precision W (evaluated_term.rs:286-327):
// lambda_res = W g, gradient J^T W g, Hessian J^T (W J), cost g^T W g.
void prior_term(const double* pose, const double* mean, const double* W, double* g, double* J,
                double* hpp, double* gp, double* cost) {
  double einv[7], te[7];
  se3_inverse<double>(mean, einv);
  se3_mul<double>(pose, einv, te);
  se3_log<double>(te, g);
  using D = Dual<6>;
  D x[6], e[7], td[7], ed[7], a[7], b[7], gd[6];
  for (int i = 0; i < 6; ++i) x[i].d[i] = 1.0;
  se3_exp<D>(x, e);
  for (int i = 0; i < 7; ++i) { td[i] = D(pose[i]); ed[i] = D(einv[i]); }
  se3_mul<D>(e, td, a);
  se3_mul<D>(a, ed, b);
  se3_log<D>(b, gd);
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < 6; ++c) J[r * 6 + c] = gd[r].d[c];
  double lr[6], wj[36];
  for (int r = 0; r < 6; ++r) {
    double acc = 0.0;
    for (int c = 0; c < 6; ++c) acc += W[r * 6 + c] * g[c];
    lr[r] = acc;
    for (int c = 0; c < 6; ++c) {
      double s = 0.0;
      for (int k = 0; k < 6; ++k) s += W[r * 6 + k] * J[k * 6 + c];
      wj[r * 6 + c] = s;
    }
  }
  for (int r = 0; r < 6; ++r) {
    double acc = 0.0;
    for (int k = 0; k < 6; ++k) acc += J[k * 6 + r] * lr[k];
    gp[r] = acc;
    for (int c = 0; c < 6; ++c) {
      double s = 0.0;
      for (int k = 0; k < 6; ++k) s += J[k * 6 + r] * wj[k * 6 + c];
      hpp[r * 6 + c] = s;
    }
  }
  double cst = 0.0;
  for (int r = 0; r < 6; ++r) cst += g[r] * lr[r];
  *cost = cst;
}

// The prior terms sorted by pose (stable), as CostFn::sort orders them; a term
// whose pose index is out of range is left out (ora_optimize rejects it).
std::vector<int> prior_order(const ora_problem* p) {
  std::vector<int> ord;
  for (int k = 0; k < p->n_prior; ++k)
    if (p->prior_pose[k] >= 0 && p->prior_pose[k] < p->n_cam) ord.push_back(k);
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return p->prior_pose[a] < p->prior_pose[b]; });
  return ord;
}

bool priors_valid(const ora_problem* p) {
  for (int k = 0; k < p->n_prior; ++k)
    if (p->prior_pose[k] < 0 || p->prior_pose[k] >= p->n_cam) return false;
  return true;
}

double prior_total_cost(const ora_problem* p, const double* poses) {
  double c = 0.0;
  for (int k : prior_order(p)) {
    double g[6], J[36], h[36], gp[6], cost;
    prior_term(poses + 7 * p->prior_pose[k], p->prior_mean + 7 * k, p->prior_precision + 36 * k, g, J, h, gp,
               &cost);
    c += cost;
  }
  return c;
}

// PoseGraph3CostTerm::eval (pose_graph3.rs): g = log(T_m^-1 T_n M^-1) and
// the Jacobians -/+ Isometry3::dx_log_a_exp_x_b_at_0(T_m^-1, T_n M^-1), taken
// here by dual numbers through log(a exp(x) b) at x = 0; no precision, no
// robust kernel: cost g^T g, gradients J^T g, blocks J_m^T J_m, J_n^T J_n, J_m^T J_n.
void edge_term(const double* tm, const double* tn, const double* mn, double* g, double* Jm, double* Jn,
               double* cost) {
  double a[7], mninv[7], b[7], ab[7];
  se3_inverse<double>(tm, a);
  se3_inverse<double>(mn, mninv);
  se3_mul<double>(tn, mninv, b);
  se3_mul<double>(a, b, ab);
  se3_log<double>(ab, g);
  using D = Dual<6>;
  D x[6], e[7], ad[7], bd[7], t1[7], t2[7], gd[6];
  for (int i = 0; i < 6; ++i) x[i].d[i] = 1.0;
  se3_exp<D>(x, e);
  for (int i = 0; i < 7; ++i) { ad[i] = D(a[i]); bd[i] = D(b[i]); }
  se3_mul<D>(ad, e, t1);
  se3_mul<D>(t1, bd, t2);
  se3_log<D>(t2, gd);
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < 6; ++c) { Jn[r * 6 + c] = gd[r].d[c]; Jm[r * 6 + c] = -gd[r].d[c]; }
  double cst = 0.0;
  for (int r = 0; r < 6; ++r) cst += g[r] * g[r];
  *cost = cst;
}

// The edge terms sorted by (m, n) (stable), as CostFn::sort orders them;
// terms with an out-of-range or repeated pose are left out (ora_optimize
// rejects them).
std::vector<int> edge_order(const ora_problem* p) {
  std::vector<int> ord;
  for (int k = 0; k < p->n_edge; ++k) {
    const int m = p->edge_pose[2 * k], n = p->edge_pose[2 * k + 1];
    if (m >= 0 && m < p->n_cam && n >= 0 && n < p->n_cam && m != n) ord.push_back(k);
  }
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) {
    if (p->edge_pose[2 * a] != p->edge_pose[2 * b]) return p->edge_pose[2 * a] < p->edge_pose[2 * b];
    return p->edge_pose[2 * a + 1] < p->edge_pose[2 * b + 1];
  });
  return ord;
}

bool edges_valid(const ora_problem* p) { return static_cast<int>(edge_order(p).size()) == std::max(0, p->n_edge); }

double edge_total_cost(const ora_problem* p, const double* poses) {
  double c = 0.0;
  for (int k : edge_order(p)) {
    double g[6], Jm[36], Jn[36], cost;
    edge_term(poses + 7 * p->edge_pose[2 * k], poses + 7 * p->edge_pose[2 * k + 1], p->edge_mn + 7 * k, g, Jm, Jn,
              &cost);
    c += cost;
  }
  return c;
}

double total_cost(const ora_problem* p, const double* intr, const double* poses, const double* points,
                  int n_threads) {
  // calc_total_cost (cost_fn.rs:403-433): sequential sum in sorted-term order
  // when not parallel; per-thread partial sums otherwise.
  int nt = std::max(1, n_threads);
  std::vector<double> part(nt, 0.0);
  parallel_for(p->n_obs, nt, [&](int64_t b, int64_t e, int t) {
    double acc = 0.0;
    for (int64_t i = b; i < e; ++i)
      acc += eval_cost_f64(poses + 7 * p->obs_cam[i], points + 3 * p->obs_pt[i],
                           intr, p->obs_uv + 2 * i, p->huber_delta, p->camera_model);
    part[t] = acc;
  });
  // the cost functions in list order: priors, pose-graph edges, reprojection
  double c = p->n_prior > 0 ? prior_total_cost(p, poses) : 0.0;
  if (p->n_edge > 0) c += edge_total_cost(p, poses);
  for (double v : part) c += v;
  return c;
}

// Linear system in Schur-ready form: per free pose U (6x6) + neg_grad,
// per marg point V (3x3) + neg_grad, per reduction range W^T (3x6).
template <class R>
struct System {
  std::vector<R> U, bp;    // nf*36, nf*6
  std::vector<R> V, bm;    // nm*9,  nm*3
  std::vector<R> Wr;       // per reduction range: 3x6 (point row, pose col) -- valid when both active
  // Free intrinsics only (empty otherwise), nc = 4 or 6 params: their nc x nc
  // block and neg_grad, and the blocks coupling them to each free pose
  // (6 x nc) and marg point (3 x nc)
  std::vector<R> Ucc, bc, Hpc, Hmc;
  // pose-pose blocks from the edge terms, lower triangle: block (row fi, col fj), fi > fj
  std::vector<int> off_row, off_col;
  std::vector<R> off_blk;  // 36 per block, row-major
  double max_grad = 0.0;
};

// evaluate + populate_upper_triangular_normal_equation (cost_system.rs:74-273)
template <class R>
void build_system(const ora_problem* p, const Structure& s, const double* intr, const double* poses,
                  const double* points, double nu, int n_threads, System<R>* sys) {
  const bool fc = p->intrinsics_free != 0;
  const int nc = cam_params(p);
  const int model = p->camera_model;
  sys->U.assign(static_cast<size_t>(s.nf) * 36, R(0));
  sys->bp.assign(static_cast<size_t>(s.nf) * 6, R(0));
  sys->V.assign(static_cast<size_t>(s.nm) * 9, R(0));
  sys->bm.assign(static_cast<size_t>(s.nm) * 3, R(0));
  int64_t nr = static_cast<int64_t>(s.rng_pt.size());
  sys->Wr.assign(static_cast<size_t>(nr) * 18, R(0));
  if (fc) sys->Hmc.assign(static_cast<size_t>(s.nm) * 3 * nc, R(0));
  int nt = std::max(1, n_threads);
  // Parallel over points (disjoint V/bm and W); pose (and intrinsics) sums per thread.
  std::vector<std::vector<R>> Ut(nt), bpt(nt), Uct(nt), bct(nt), Hpct(nt);
  parallel_for(p->n_pt, nt, [&](int64_t pb, int64_t pe, int t) {
    Ut[t].assign(static_cast<size_t>(s.nf) * 36, R(0));
    bpt[t].assign(static_cast<size_t>(s.nf) * 6, R(0));
    if (fc) {
      Uct[t].assign(static_cast<size_t>(nc) * nc, R(0));
      bct[t].assign(nc, R(0));
      Hpct[t].assign(static_cast<size_t>(s.nf) * 6 * nc, R(0));
    }
    for (int64_t q = pb; q < pe; ++q) {
      for (int64_t r = s.pt_rng_begin[q]; r < s.pt_rng_begin[q + 1]; ++r) {
        Term<R> term;
        CamTerm<R> cterm;
        bool first = true;
        for (int64_t k = s.range_begin[r]; k < s.range_begin[r + 1]; ++k) {
          int64_t o = s.order[k];
          Term<R> tk;
          if (fc) {
            CamTerm<R> ck;
            make_term_cam<R>(poses + 7 * p->obs_cam[o], points + 3 * p->obs_pt[o], intr,
                             p->obs_uv + 2 * o, p->huber_delta, &tk, &ck, model, nc);
            if (first) cterm = ck; else cam_term_reduce(&cterm, ck);
          } else {
            make_term<R>(poses + 7 * p->obs_cam[o], points + 3 * p->obs_pt[o],
                         intr, p->obs_uv + 2 * o, p->huber_delta, &tk, model);
          }
          if (first) { term = tk; first = false; } else { term_reduce(&term, tk); }
        }
        int pb_ = s.pose_block[s.rng_pose[r]];
        int mb = s.point_block[s.rng_pt[r]];
        if (fc) {
          // the intrinsics are touched by every term: nu I per evaluated term
          R* uc = Uct[t].data();
          for (int i = 0; i < nc * nc; ++i) uc[i] += cterm.hcc[i];
          if (nu != 0.0) for (int i = 0; i < nc; ++i) uc[i * (nc + 1)] += static_cast<R>(nu);
          for (int i = 0; i < nc; ++i) bct[t][i] -= cterm.gc[i];
          if (pb_ >= 0)
            for (int i = 0; i < 6 * nc; ++i) Hpct[t][static_cast<size_t>(pb_) * 6 * nc + i] += cterm.hpc[i];
          if (mb >= 0)
            for (int i = 0; i < 3 * nc; ++i) sys->Hmc[static_cast<size_t>(mb) * 3 * nc + i] += cterm.hmc[i];
        }
        if (pb_ >= 0) {
          R* u = &Ut[t][static_cast<size_t>(pb_) * 36];
          for (int i = 0; i < 36; ++i) u[i] += term.hpp[i];
          if (nu != 0.0) for (int i = 0; i < 6; ++i) u[i * 7] += static_cast<R>(nu);
          for (int i = 0; i < 6; ++i) bpt[t][pb_ * 6 + i] -= term.gp[i];
        }
        if (mb >= 0) {
          R* v = &sys->V[static_cast<size_t>(mb) * 9];
          for (int i = 0; i < 9; ++i) v[i] += term.hmm[i];
          if (nu != 0.0) for (int i = 0; i < 3; ++i) v[i * 4] += static_cast<R>(nu);
          for (int i = 0; i < 3; ++i) sys->bm[static_cast<size_t>(mb) * 3 + i] -= term.gm[i];
          if (pb_ >= 0)
            for (int i = 0; i < 18; ++i) sys->Wr[static_cast<size_t>(r) * 18 + i] = term.hmp[i];
        }
      }
    }
  });
  if (p->n_prior > 0) {
    // the prior cost function comes first: its terms reduced per pose
    // (EvaluatedCostTerm::reduce), nu I once per reduced term (cost_system.rs:229-236)
    std::vector<int> ord = prior_order(p);
    for (size_t k = 0; k < ord.size();) {
      const int pose = p->prior_pose[ord[k]];
      double h[36] = {0.0}, gsum[6] = {0.0};
      size_t k2 = k;
      for (; k2 < ord.size() && p->prior_pose[ord[k2]] == pose; ++k2) {
        double g[6], J[36], hp[36], gp[6], cost;
        prior_term(poses + 7 * pose, p->prior_mean + 7 * ord[k2], p->prior_precision + 36 * ord[k2], g, J, hp,
                   gp, &cost);
        for (int i = 0; i < 36; ++i) h[i] += hp[i];
        for (int i = 0; i < 6; ++i) gsum[i] += gp[i];
      }
      const int fb = s.pose_block[pose];
      if (fb >= 0) {
        R* u = &sys->U[static_cast<size_t>(fb) * 36];
        for (int i = 0; i < 36; ++i) u[i] += static_cast<R>(h[i]);
        if (nu != 0.0) for (int i = 0; i < 6; ++i) u[i * 7] += static_cast<R>(nu);
        for (int i = 0; i < 6; ++i) sys->bp[static_cast<size_t>(fb) * 6 + i] -= static_cast<R>(gsum[i]);
      }
      k = k2;
    }
  }
  if (p->n_edge > 0) {
    // the pose-graph cost function: terms reduced per (m, n); nu I once per
    // reduced term on each free argument (cost_system.rs:190-273)
    std::vector<int> ord = edge_order(p);
    for (size_t k = 0; k < ord.size();) {
      const int m = p->edge_pose[2 * ord[k]], n = p->edge_pose[2 * ord[k] + 1];
      double hmm[36] = {0.0}, hnn[36] = {0.0}, hmn[36] = {0.0}, gm[6] = {0.0}, gn[6] = {0.0};
      size_t k2 = k;
      for (; k2 < ord.size() && p->edge_pose[2 * ord[k2]] == m && p->edge_pose[2 * ord[k2] + 1] == n; ++k2) {
        double g[6], Jm[36], Jn[36], cost;
        edge_term(poses + 7 * m, poses + 7 * n, p->edge_mn + 7 * ord[k2], g, Jm, Jn, &cost);
        for (int r = 0; r < 6; ++r) {
          for (int c = 0; c < 6; ++c) {
            double sm = 0.0, sn = 0.0, so = 0.0;
            for (int q = 0; q < 6; ++q) {
              sm += Jm[q * 6 + r] * Jm[q * 6 + c];
              sn += Jn[q * 6 + r] * Jn[q * 6 + c];
              so += Jm[q * 6 + r] * Jn[q * 6 + c];
            }
            hmm[r * 6 + c] += sm;
            hnn[r * 6 + c] += sn;
            hmn[r * 6 + c] += so;
          }
          double am = 0.0, an = 0.0;
          for (int q = 0; q < 6; ++q) { am += Jm[q * 6 + r] * g[q]; an += Jn[q * 6 + r] * g[q]; }
          gm[r] += am;
          gn[r] += an;
        }
      }
      const int fm = s.pose_block[m], fn = s.pose_block[n];
      const int fbs[2] = {fm, fn};
      const double* hs[2] = {hmm, hnn};
      const double* gs[2] = {gm, gn};
      for (int a = 0; a < 2; ++a) {
        if (fbs[a] < 0) continue;
        R* u = &sys->U[static_cast<size_t>(fbs[a]) * 36];
        for (int i = 0; i < 36; ++i) u[i] += static_cast<R>(hs[a][i]);
        if (nu != 0.0) for (int i = 0; i < 6; ++i) u[i * 7] += static_cast<R>(nu);
        for (int i = 0; i < 6; ++i) sys->bp[static_cast<size_t>(fbs[a]) * 6 + i] -= static_cast<R>(gs[a][i]);
      }
      if (fm >= 0 && fn >= 0) {
        // lower-triangle block: rows of the later free block
        const bool m_lower = fm > fn;
        sys->off_row.push_back(m_lower ? fm : fn);
        sys->off_col.push_back(m_lower ? fn : fm);
        for (int r = 0; r < 6; ++r)
          for (int c = 0; c < 6; ++c)
            sys->off_blk.push_back(static_cast<R>(m_lower ? hmn[r * 6 + c] : hmn[c * 6 + r]));
      }
      k = k2;
    }
  }
  for (int t = 0; t < nt; ++t) {
    if (Ut[t].empty()) continue;
    for (size_t i = 0; i < sys->U.size(); ++i) sys->U[i] += Ut[t][i];
    for (size_t i = 0; i < sys->bp.size(); ++i) sys->bp[i] += bpt[t][i];
  }
  if (fc) {
    sys->Ucc.assign(static_cast<size_t>(nc) * nc, R(0));
    sys->bc.assign(nc, R(0));
    sys->Hpc.assign(static_cast<size_t>(s.nf) * 6 * nc, R(0));
    for (int t = 0; t < nt; ++t) {
      if (Uct[t].empty()) continue;
      for (int i = 0; i < nc * nc; ++i) sys->Ucc[i] += Uct[t][i];
      for (int i = 0; i < nc; ++i) sys->bc[i] += bct[t][i];
      for (size_t i = 0; i < sys->Hpc.size(); ++i) sys->Hpc[i] += Hpct[t][i];
    }
  }
  double mg = 0.0;
  for (auto v : sys->bc) mg = std::max(mg, std::fabs(static_cast<double>(v)));
  for (auto v : sys->bp) mg = std::max(mg, std::fabs(static_cast<double>(v)));
  for (auto v : sys->bm) mg = std::max(mg, std::fabs(static_cast<double>(v)));
  sys->max_grad = mg;
}

// Equality constraints TranslationNormConstraint (ba_scale_constraint.rs:44-100):
// c(T) = |t(T)| - r.  Its Jacobian is taken, as the reference's dual numbers
// take it, under the left perturbation exp(x) * T at x = 0.  The tangent is
// (w, v), rotation first (affine_group_template.rs:162-169); the translation
// moves by w x t + v, so dc/dv = t^T / |t| and dc/dw = t^T [e_k]x t / |t| = 0,
// exactly zero in floating point as well.
struct EqTerms {
  int n = 0;
  std::vector<double> c;    // n residuals
  std::vector<double> jac;  // n x 6, row-major
  std::vector<int> fb;      // free block of each term's pose, -1 when the pose is constant
};

void eq_eval(const ora_problem* p, const Structure* s, const double* poses, EqTerms* e) {
  e->n = p->n_eq;
  e->c.assign(e->n, 0.0);
  e->jac.assign(static_cast<size_t>(e->n) * 6, 0.0);
  e->fb.assign(e->n, -1);
  for (int k = 0; k < e->n; ++k) {
    if (p->eq_pose[k] < 0 || p->eq_pose[k] >= p->n_cam) { e->c[k] = NAN; continue; }
    const double* t = poses + 7 * p->eq_pose[k] + 4;
    double nrm = std::sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    e->c[k] = nrm - p->eq_radius[k];
    for (int i = 0; i < 3; ++i) e->jac[k * 6 + 3 + i] = t[i] / nrm;
    if (s) e->fb[k] = s->pose_block[p->eq_pose[k]];
  }
}

// Inverse of the small dense m x m matrix G S^-1 G^T (nalgebra try_inverse in
// schur_ldlt.rs:723-728): Gauss-Jordan with partial pivoting.  False when a
// pivot is zero or not finite.
bool small_inverse(int m, std::vector<double> a, std::vector<double>* inv) {
  inv->assign(static_cast<size_t>(m) * m, 0.0);
  for (int i = 0; i < m; ++i) (*inv)[i * m + i] = 1.0;
  for (int col = 0; col < m; ++col) {
    int piv = col;
    for (int r = col + 1; r < m; ++r)
      if (std::fabs(a[r * m + col]) > std::fabs(a[piv * m + col])) piv = r;
    double d = a[piv * m + col];
    if (!(std::fabs(d) > 0.0) || !std::isfinite(d)) return false;
    if (piv != col)
      for (int c = 0; c < m; ++c) {
        std::swap(a[piv * m + c], a[col * m + c]);
        std::swap((*inv)[piv * m + c], (*inv)[col * m + c]);
      }
    for (int c = 0; c < m; ++c) { a[col * m + c] /= d; (*inv)[col * m + c] /= d; }
    for (int r = 0; r < m; ++r) {
      if (r == col) continue;
      double f = a[r * m + col];
      if (f == 0.0) continue;
      for (int c = 0; c < m; ++c) { a[r * m + c] -= f * a[col * m + c]; (*inv)[r * m + c] -= f * (*inv)[col * m + c]; }
    }
  }
  return true;
}

// SchurFactor::factorize + solve (schur_ldlt.rs:536-812) with the sequential
// forward pass (schur_ldlt.rs:241-278).  delta = [dx_c; dx_f; dx_m], dx_c the
// nc = 4 (pinhole) or 6 (EUCM) intrinsics when they are free (empty
// otherwise).  In S the intrinsics come first (their family's partition
// precedes the poses'), padded to one 6-row block with an identity so the
// factor keeps 6x6 blocks; the pivot rule restarts at that block as at every
// partition block.
template <class R>
int schur_solve(const ora_problem* p, const Structure& s, const System<R>& sys,
                int n_threads, std::vector<double>* delta, std::vector<double>* s_out,
                std::vector<double>* rhs_out, const EqTerms* eq = nullptr,
                const double* lambda = nullptr) {
  const bool fc = p->intrinsics_free != 0;
  const int nc = cam_params(p);
  const int nf = s.nf;
  const int n6 = nf * 6;
  const int nci = fc ? 6 : 0;   // rows of the (padded) intrinsics block in S
  const int nc4 = fc ? nc : 0;  // intrinsics scalars in delta
  const int n = nci + n6;
  const int nt = std::max(1, n_threads);
  // S_ff = H_ff (diagonal blocks only for BA)
  std::vector<std::vector<R>> St(nt);
  std::vector<std::vector<R>> rt(nt);
  std::vector<R> hinv(static_cast<size_t>(s.nm) * 9);
  std::vector<int> fail(nt, 0);
  parallel_for(p->n_pt, nt, [&](int64_t qb, int64_t qe, int t) {
    St[t].assign(static_cast<size_t>(n) * n, R(0));
    rt[t].assign(n, R(0));
    std::vector<int> fidx;
    std::vector<const R*> hmf;
    std::vector<R> inv_hmf;
    for (int64_t q = qb; q < qe; ++q) {
      int mb = s.point_block[q];
      if (mb < 0) continue;
      R inv[9];
      if (!inverse3<R>(&sys.V[static_cast<size_t>(mb) * 9], inv)) { fail[t] = 1; return; }
      for (int i = 0; i < 9; ++i) hinv[static_cast<size_t>(mb) * 9 + i] = inv[i];
      const R* g = &sys.bm[static_cast<size_t>(mb) * 3];
      R ig[3];
      for (int i = 0; i < 3; ++i) ig[i] = inv[i * 3 + 0] * g[0] + inv[i * 3 + 1] * g[1] + inv[i * 3 + 2] * g[2];
      // non-zero free blocks for this marg block, in free-block order
      fidx.clear(); hmf.clear();
      for (int64_t r = s.pt_rng_begin[q]; r < s.pt_rng_begin[q + 1]; ++r) {
        int fb = s.pose_block[s.rng_pose[r]];
        if (fb < 0) continue;
        fidx.push_back(fb);
        hmf.push_back(&sys.Wr[static_cast<size_t>(r) * 18]);
      }
      size_t L = fidx.size();
      inv_hmf.assign(L * 18, R(0));
      for (size_t a = 0; a < L; ++a)
        for (int i = 0; i < 3; ++i)
          for (int c = 0; c < 6; ++c)
            inv_hmf[a * 18 + i * 6 + c] = inv[i * 3 + 0] * hmf[a][0 * 6 + c] +
                                          inv[i * 3 + 1] * hmf[a][1 * 6 + c] +
                                          inv[i * 3 + 2] * hmf[a][2 * 6 + c];
      for (size_t i = 0; i < L; ++i) {
        int fi = fidx[i];
        // rhs_bar[f_i] -= H_mf_i^T * (H_mm^-1 g_m)
        for (int c = 0; c < 6; ++c)
          rt[t][nci + fi * 6 + c] -= hmf[i][0 * 6 + c] * ig[0] + hmf[i][1 * 6 + c] * ig[1] + hmf[i][2 * 6 + c] * ig[2];
        for (size_t j = 0; j <= i; ++j) {
          int fj = fidx[j];
          size_t ii = i, jj = j;
          int row = fi, col = fj;
          if (fi < fj) { row = fj; col = fi; ii = j; jj = i; }
          // S[row, col] -= H_mf[ii]^T * (H_mm^-1 H_mf[jj])
          R* sb = &St[t][0];
          for (int r2 = 0; r2 < 6; ++r2)
            for (int c2 = 0; c2 < 6; ++c2) {
              R acc = hmf[ii][0 * 6 + r2] * inv_hmf[jj * 18 + 0 * 6 + c2] +
                      hmf[ii][1 * 6 + r2] * inv_hmf[jj * 18 + 1 * 6 + c2] +
                      hmf[ii][2 * 6 + r2] * inv_hmf[jj * 18 + 2 * 6 + c2];
              sb[static_cast<size_t>(nci + row * 6 + r2) * n + nci + col * 6 + c2] -= acc;
            }
        }
      }
      if (fc) {
        // the intrinsics column: Y = H_mc (3 x nc), H_mm^-1 Y
        const R* y = &sys.Hmc[static_cast<size_t>(mb) * 3 * nc];
        R iy[18];
        for (int i = 0; i < 3; ++i)
          for (int c = 0; c < nc; ++c)
            iy[i * nc + c] = inv[i * 3 + 0] * y[0 * nc + c] + inv[i * 3 + 1] * y[1 * nc + c] + inv[i * 3 + 2] * y[2 * nc + c];
        R* sb = &St[t][0];
        for (int c = 0; c < nc; ++c)
          rt[t][c] -= y[0 * nc + c] * ig[0] + y[1 * nc + c] * ig[1] + y[2 * nc + c] * ig[2];
        for (int r2 = 0; r2 < nc; ++r2)
          for (int c2 = 0; c2 < nc; ++c2)
            sb[static_cast<size_t>(r2) * n + c2] -=
                y[0 * nc + r2] * iy[0 * nc + c2] + y[1 * nc + r2] * iy[1 * nc + c2] + y[2 * nc + r2] * iy[2 * nc + c2];
        for (size_t i = 0; i < L; ++i) {
          // S[pose f_i, intrinsics] -= H_mf_i^T (H_mm^-1 Y)
          for (int r2 = 0; r2 < 6; ++r2)
            for (int c2 = 0; c2 < nc; ++c2)
              sb[static_cast<size_t>(nci + fidx[i] * 6 + r2) * n + c2] -=
                  hmf[i][0 * 6 + r2] * iy[0 * nc + c2] + hmf[i][1 * 6 + r2] * iy[1 * nc + c2] +
                  hmf[i][2 * 6 + r2] * iy[2 * nc + c2];
        }
      }
    }
  });
  for (int t = 0; t < nt; ++t) if (fail[t]) return -1;
  std::vector<double> S(static_cast<size_t>(n) * n, 0.0);
  std::vector<double> rhs(n, 0.0);
  {
    // merge fold accumulators in thread order (the reduce step)
    std::vector<R> Sacc(static_cast<size_t>(n) * n, R(0)), racc(n, R(0));
    for (int i = 0; i < nf; ++i)
      for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 6; ++c)
          Sacc[static_cast<size_t>(nci + i * 6 + r) * n + nci + i * 6 + c] = sys.U[static_cast<size_t>(i) * 36 + r * 6 + c];
    for (int i = 0; i < n6; ++i) racc[nci + i] = sys.bp[i];
    for (size_t e = 0; e < sys.off_row.size(); ++e)
      for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 6; ++c)
          Sacc[static_cast<size_t>(nci + sys.off_row[e] * 6 + r) * n + nci + sys.off_col[e] * 6 + c] +=
              sys.off_blk[e * 36 + r * 6 + c];
    if (eq && lambda) {
      // the constraint rows add G^T lambda to the free gradient when the KKT
      // system is populated (eq_system.rs, populate_lower_triangular_kkt_mat)
      for (int k = 0; k < eq->n; ++k) {
        if (eq->fb[k] < 0) continue;
        for (int c = 0; c < 6; ++c) racc[nci + eq->fb[k] * 6 + c] += static_cast<R>(eq->jac[k * 6 + c] * lambda[k]);
      }
    }
    if (fc) {
      for (int r = 0; r < nc; ++r)
        for (int c = 0; c < nc; ++c) Sacc[static_cast<size_t>(r) * n + c] = sys.Ucc[r * nc + c];
      for (int k = nc; k < 6; ++k) Sacc[static_cast<size_t>(k) * n + k] = R(1);  // padding: identity, zero rhs
      for (int i = 0; i < nf; ++i)
        for (int r = 0; r < 6; ++r)
          for (int c = 0; c < nc; ++c)
            Sacc[static_cast<size_t>(nci + i * 6 + r) * n + c] = sys.Hpc[static_cast<size_t>(i) * 6 * nc + r * nc + c];
      for (int c = 0; c < nc; ++c) racc[c] = sys.bc[c];
    }
    for (int t = 0; t < nt; ++t) {
      if (St[t].empty()) continue;
      for (size_t i = 0; i < Sacc.size(); ++i) Sacc[i] += St[t][i];
      for (int i = 0; i < n; ++i) racc[i] += rt[t][i];
    }
    for (size_t i = 0; i < Sacc.size(); ++i) S[i] = static_cast<double>(Sacc[i]);
    for (int i = 0; i < n; ++i) rhs[i] = static_cast<double>(racc[i]);
  }
  // symmetrize from the lower triangle for the dense factor
  for (int r = 0; r < n; ++r)
    for (int c = r + 1; c < n; ++c) S[static_cast<size_t>(r) * n + c] = S[static_cast<size_t>(c) * n + r];
  if (s_out) *s_out = S;
  if (rhs_out) *rhs_out = rhs;
  BlockLdlt f;
  if (f.factorize(n, 6, S.data()) != 0) return -1;
  std::vector<double> dxf(rhs);
  f.solve(dxf.data());
  const int m = eq ? eq->n : 0;
  std::vector<double> dlam(m, 0.0);
  if (m > 0) {
    // Range-space KKT solve (SchurFactor::factorize / solve, schur_ldlt.rs:674-772):
    // Y = S^-1 G^T, M = G Y, dlam = M^-1 (G u - rhs_c) with rhs_c = -c,
    // dx_f = S^-1 (rhs_bar - G^T dlam).
    std::vector<double> G(static_cast<size_t>(m) * n, 0.0);
    for (int k = 0; k < m; ++k)
      if (eq->fb[k] >= 0)
        for (int c = 0; c < 6; ++c) G[static_cast<size_t>(k) * n + nci + eq->fb[k] * 6 + c] = eq->jac[k * 6 + c];
    std::vector<double> Y(static_cast<size_t>(m) * n);  // column k of Y stored as row k
    for (int k = 0; k < m; ++k) {
      std::copy(&G[static_cast<size_t>(k) * n], &G[static_cast<size_t>(k + 1) * n], &Y[static_cast<size_t>(k) * n]);
      f.solve(&Y[static_cast<size_t>(k) * n]);
    }
    std::vector<double> M(static_cast<size_t>(m) * m), Minv;
    for (int a = 0; a < m; ++a)
      for (int b = 0; b < m; ++b) {
        double acc = 0.0;
        for (int i = 0; i < n; ++i) acc += G[static_cast<size_t>(a) * n + i] * Y[static_cast<size_t>(b) * n + i];
        M[a * m + b] = acc;
      }
    if (!small_inverse(m, M, &Minv)) return -2;
    std::vector<double> w(m);
    for (int k = 0; k < m; ++k) {
      double acc = 0.0;
      for (int i = 0; i < n; ++i) acc += G[static_cast<size_t>(k) * n + i] * dxf[i];
      w[k] = acc + eq->c[k];
    }
    for (int a = 0; a < m; ++a) {
      double acc = 0.0;
      for (int b = 0; b < m; ++b) acc += Minv[a * m + b] * w[b];
      dlam[a] = acc;
    }
    dxf = rhs;
    for (int k = 0; k < m; ++k)
      for (int i = 0; i < n; ++i) dxf[i] -= G[static_cast<size_t>(k) * n + i] * dlam[k];
    f.solve(dxf.data());
  }
  delta->assign(static_cast<size_t>(nc4) + static_cast<size_t>(n6) + static_cast<size_t>(s.nm) * 3 + m, 0.0);
  for (int k = 0; k < m; ++k) (*delta)[nc4 + n6 + static_cast<size_t>(s.nm) * 3 + k] = dlam[k];
  for (int i = 0; i < nc4; ++i) (*delta)[i] = dxf[i];
  for (int i = 0; i < n6; ++i) (*delta)[nc4 + i] = dxf[nci + i];
  // back-substitution: dx_m[b] = H_mm^-1 (g_m[b] - sum H_mf[b,f] dx_f[f] - H_mc[b] dx_c)
  for (int q = 0; q < p->n_pt; ++q) {
    int mb = s.point_block[q];
    if (mb < 0) continue;
    double m[3];
    for (int i = 0; i < 3; ++i) m[i] = static_cast<double>(sys.bm[static_cast<size_t>(mb) * 3 + i]);
    for (int64_t r = s.pt_rng_begin[q]; r < s.pt_rng_begin[q + 1]; ++r) {
      int fb = s.pose_block[s.rng_pose[r]];
      if (fb < 0) continue;
      const R* w = &sys.Wr[static_cast<size_t>(r) * 18];
      for (int i = 0; i < 3; ++i) {
        double acc = 0.0;
        for (int c = 0; c < 6; ++c) acc += static_cast<double>(w[i * 6 + c]) * dxf[nci + fb * 6 + c];
        m[i] -= acc;
      }
    }
    if (fc) {
      const R* y = &sys.Hmc[static_cast<size_t>(mb) * 3 * nc];
      for (int i = 0; i < 3; ++i) {
        double acc = 0.0;
        for (int c = 0; c < nc; ++c) acc += static_cast<double>(y[i * nc + c]) * dxf[c];
        m[i] -= acc;
      }
    }
    const R* inv = &hinv[static_cast<size_t>(mb) * 9];
    for (int i = 0; i < 3; ++i)
      (*delta)[nc4 + n6 + mb * 3 + i] = static_cast<double>(inv[i * 3 + 0]) * m[0] +
                                        static_cast<double>(inv[i * 3 + 1]) * m[1] +
                                        static_cast<double>(inv[i * 3 + 2]) * m[2];
  }
  return 0;
}

// VarFamilies::update (var_families.rs:203-209; var_family.rs:101-114;
// lie_group_manifold.rs:57-64): T <- exp(delta) * T, p <- p + delta, and
// free pinhole intrinsics (a vector space) params <- params + delta.
// Returns false if a pose fails the params-validity assertion of from_params.
bool apply_update(const ora_problem* p, const Structure& s, const std::vector<double>& delta,
                  const double* intr, const double* poses, const double* points, double* nintr,
                  double* npose, double* npts) {
  bool ok = true;
  const int nc4 = p->intrinsics_free ? cam_params(p) : 0;
  for (int i = 0; i < 6; ++i) nintr[i] = intr[i] + (i < nc4 ? delta[i] : 0.0);
  std::memcpy(npose, poses, sizeof(double) * 7 * p->n_cam);
  std::memcpy(npts, points, sizeof(double) * 3 * p->n_pt);
  for (int c = 0; c < p->n_cam; ++c) {
    int fb = s.pose_block[c];
    if (fb < 0) continue;
    double e[7];
    se3_exp<double>(&delta[nc4 + fb * 6], e);
    if (!quat_valid(e)) ok = false;
    double out[7];
    se3_mul<double>(e, poses + 7 * c, out);
    if (!quat_valid(out)) ok = false;
    std::memcpy(npose + 7 * c, out, sizeof(out));
  }
  const int64_t off = nc4 + static_cast<int64_t>(s.nf) * 6;
  for (int q = 0; q < p->n_pt; ++q) {
    int mb = s.point_block[q];
    if (mb < 0) continue;
    for (int i = 0; i < 3; ++i) npts[3 * q + i] = points[3 * q + i] + delta[off + mb * 3 + i];
  }
  return ok;
}

// EqSystem::update_lambdas (eq_system.rs): lambda <- lambda - dlam, dlam the
// last n_eq entries of the step.
void update_lambdas(int n_eq, const std::vector<double>& delta, std::vector<double>* lambda) {
  const size_t off = delta.size() - static_cast<size_t>(n_eq);
  for (int k = 0; k < n_eq; ++k) (*lambda)[k] -= delta[off + k];
}

template <class R>
int schur_step_impl(const ora_problem* p, const Structure& s, const double* intr, const double* poses,
                    const double* points, double nu, int n_threads, std::vector<double>* delta,
                    double* max_grad, std::vector<double>* neg_grad, std::vector<double>* S,
                    std::vector<double>* rhs, double gradient_tolerance = -1.0,
                    const EqTerms* eq = nullptr, const double* lambda = nullptr) {
  System<R> sys;
  build_system<R>(p, s, intr, poses, points, nu, n_threads, &sys);
  if (max_grad) *max_grad = sys.max_grad;
  if (neg_grad) {
    neg_grad->clear();
    for (auto v : sys.bc) neg_grad->push_back(static_cast<double>(v));
    for (auto v : sys.bp) neg_grad->push_back(static_cast<double>(v));
    for (auto v : sys.bm) neg_grad->push_back(static_cast<double>(v));
    if (eq) {
      // the KKT right-hand side: + G^T lambda on the free rows, -c on the
      // constraint rows (eq_system.rs, populate_lower_triangular_kkt_mat)
      const size_t nc4 = sys.bc.size();
      for (int k = 0; k < eq->n; ++k) {
        if (eq->fb[k] < 0) continue;
        for (int c = 0; c < 6; ++c)
          (*neg_grad)[nc4 + static_cast<size_t>(eq->fb[k]) * 6 + c] += eq->jac[k * 6 + c] * lambda[k];
      }
      for (int k = 0; k < eq->n; ++k) neg_grad->push_back(-eq->c[k]);
    }
  }
  // check_gradient_tolerance happens before the solve (optimizer_step.rs:382-384);
  // it is skipped when there are equality constraints (optimizer.rs:527-535)
  if (!(eq && eq->n > 0) && sys.max_grad < gradient_tolerance) return 1;
  return schur_solve<R>(p, s, sys, n_threads, delta, S, rhs, eq, lambda);
}

// Covariance queries (SchurFactor::inverse_block, schur_ldlt.rs:815-957) at
// the given variables with zero damping: S^-1 densely (the block LDLT of S
// applied to unit vectors), H_mm^-1 and the rows H_mf per marg block.
struct CovCtx {
  Structure s;
  System<double> sys;
  int n = 0, nci = 0, nc = 0, rank = 0;
  std::vector<double> Sinv;  // n x n: S^-1, or the min-norm pseudo-inverse S+ when S is rank-deficient
};

// MinNormLdlt::pseudo_inverse (min_norm_ldlt.rs:55-140) with the block-sparse
// backend's columns (block_sparse_min_norm_ldlt.rs:98-160): with A = L D L^T,
// L the block factor times the unit-lower factors of the diagonal blocks, E the
// columns of L at the positive pivots J and G = E^T E,
//   A+ = E G^-1 diag(d_J)^-1 G^-1 E^T.
// out: n x n row-major.  Returns 0, or -2 when G cannot be factored.
int pseudo_inverse(const BlockLdlt& f, std::vector<double>* out) {
  const int n = f.n, bs = f.bs, nb = f.nb;
  std::vector<int> J;
  for (int j = 0; j < n; ++j)
    if (f.d[j] > 0.0) J.push_back(j);
  const int r = static_cast<int>(J.size());
  out->assign(static_cast<size_t>(n) * n, 0.0);
  if (r == 0) return 0;
  std::vector<double> E(static_cast<size_t>(n) * r, 0.0);  // n x r row-major
  for (int c = 0; c < r; ++c) {
    const int bj = J[c] / bs, co = J[c] % bs;
    const double* ljj = &f.ldiag[static_cast<size_t>(bj) * bs * bs];
    for (int q = 0; q < bs; ++q) E[static_cast<size_t>(bj * bs + q) * r + c] = ljj[q * bs + co];
    for (int bi = bj + 1; bi < nb; ++bi) {
      const double* lij = &f.lblk[((static_cast<size_t>(bi) * nb + bj) * bs) * bs];
      for (int q = 0; q < bs; ++q) {
        double acc = 0.0;
        for (int t = 0; t < bs; ++t) acc += lij[q * bs + t] * ljj[t * bs + co];
        E[static_cast<size_t>(bi * bs + q) * r + c] = acc;
      }
    }
  }
  std::vector<double> G(static_cast<size_t>(r) * r), gd(r);
  for (int a = 0; a < r; ++a)
    for (int b = 0; b < r; ++b) {
      double acc = 0.0;
      for (int i = 0; i < n; ++i) acc += E[static_cast<size_t>(i) * r + a] * E[static_cast<size_t>(i) * r + b];
      G[static_cast<size_t>(a) * r + b] = acc;
    }
  if (ldlt_decompose_inplace(r, G.data(), gd.data(), kLdltTolRel) != 0) return -2;
  for (int a = 0; a < r; ++a)
    if (!(gd[a] > 0.0)) return -2;  // G is positive definite on the positive-pivot subspace
  std::vector<double> W(E);  // W = E G^-1 diag(d_J)^-1 G^-1
  ldlt_right_matsolve(r, G.data(), gd.data(), n, W.data());
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < r; ++c) W[static_cast<size_t>(i) * r + c] /= f.d[J[c]];
  ldlt_right_matsolve(r, G.data(), gd.data(), n, W.data());
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double acc = 0.0;
      for (int c = 0; c < r; ++c) acc += W[static_cast<size_t>(i) * r + c] * E[static_cast<size_t>(j) * r + c];
      (*out)[static_cast<size_t>(i) * n + j] = acc;
    }
  return 0;
}

int cov_build(const ora_problem* p, CovCtx* c) {
  build_structure(p, &c->s);
  double intr[6];
  problem_intrinsics(p, intr);
  build_system<double>(p, c->s, intr, p->poses, p->points, 0.0, 1, &c->sys);
  std::vector<double> delta, S, rhs;
  if (schur_solve<double>(p, c->s, c->sys, 1, &delta, &S, &rhs) != 0) return -2;
  c->nc = cam_params(p);
  c->nci = p->intrinsics_free ? 6 : 0;
  c->n = c->nci + 6 * c->s.nf;
  const int n = c->n;
  BlockLdlt f;
  if (f.factorize(n, 6, S.data()) != 0) return -2;
  int rank = 0;
  for (int j = 0; j < n; ++j) rank += f.d[j] > 0.0 ? 1 : 0;
  c->rank = rank;
  // a gauge-deficient S: the min-norm pseudo-inverse (SchurFactor::ensure_s_inv,
  // schur_ldlt.rs:847-866); full rank: S^-1 by solves (try_inverse)
  if (rank < n) return pseudo_inverse(f, &c->Sinv);
  c->Sinv.assign(static_cast<size_t>(n) * n, 0.0);
  std::vector<double> e(n);
  for (int j = 0; j < n; ++j) {
    std::fill(e.begin(), e.end(), 0.0);
    e[j] = 1.0;
    f.solve(e.data());
    for (int i = 0; i < n; ++i) c->Sinv[static_cast<size_t>(i) * n + j] = e[i];
  }
  return 0;
}

// Offset and size in S of a free variable, or -1.
int cov_free_offset(const ora_problem* p, const CovCtx& c, int kind, int index, int* dim) {
  if (kind == ORA_VAR_INTRINSICS) {
    *dim = c.nc;
    return p->intrinsics_free ? 0 : -1;
  }
  if (kind == ORA_VAR_POSE) {
    *dim = 6;
    if (index < 0 || index >= p->n_cam || c.s.pose_block[index] < 0) return -1;
    return c.nci + 6 * c.s.pose_block[index];
  }
  return -1;
}

// H_mf of point q as a dense 3 x n row block (S's column layout).
std::vector<double> cov_hmf(const ora_problem* p, const CovCtx& c, int q) {
  const int n = c.n, mb = c.s.point_block[q];
  std::vector<double> h(static_cast<size_t>(3) * n, 0.0);
  for (int64_t r = c.s.pt_rng_begin[q]; r < c.s.pt_rng_begin[q + 1]; ++r) {
    int fb = c.s.pose_block[c.s.rng_pose[r]];
    if (fb < 0) continue;
    for (int i = 0; i < 3; ++i)
      for (int k = 0; k < 6; ++k) h[static_cast<size_t>(i) * n + c.nci + fb * 6 + k] = c.sys.Wr[r * 18 + i * 6 + k];
  }
  if (p->intrinsics_free)
    for (int i = 0; i < 3; ++i)
      for (int k = 0; k < c.nc; ++k) h[static_cast<size_t>(i) * n + k] = c.sys.Hmc[static_cast<size_t>(mb) * 3 * c.nc + i * c.nc + k];
  return h;
}

bool cov_hmm_inv(const CovCtx& c, int q, double* inv) {
  return inverse3<double>(&c.sys.V[static_cast<size_t>(c.s.point_block[q]) * 9], inv);
}

// -(S^-1[free rows, :] H_mf_q^T) H_mm[q]^-1  (dim x 3)
void cov_free_marg(const CovCtx& c, int off, int dim, const std::vector<double>& hmf, const double* hinv,
                   double* out) {
  const int n = c.n;
  for (int a = 0; a < dim; ++a) {
    double t[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < 3; ++i)
      for (int k = 0; k < n; ++k) t[i] += c.Sinv[static_cast<size_t>(off + a) * n + k] * hmf[static_cast<size_t>(i) * n + k];
    for (int j = 0; j < 3; ++j) out[a * 3 + j] = -(t[0] * hinv[0 * 3 + j] + t[1] * hinv[1 * 3 + j] + t[2] * hinv[2 * 3 + j]);
  }
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

void ora_se3_exp(const double tangent[6], double out[7]) { se3_exp<double>(tangent, out); }
void ora_se3_mul(const double a[7], const double b[7], double out[7]) { se3_mul<double>(a, b, out); }
void ora_se3_inverse(const double a[7], double out[7]) { se3_inverse<double>(a, out); }

void ora_eval_term(const double pose[7], const double point[3], const double intr[4],
                   const double uv[2], double huber, double r[2], double j_pose[12],
                   double j_point[6], double* weight, double* cost) {
  eval_term_f64(pose, point, intr, uv, huber, r, j_pose, j_point, weight, cost);
}

void ora_eval_term_dual(const double pose[7], const double point[3], const double intr[4],
                        const double uv[2], double j_pose[12], double j_point[6]) {
  // r(delta, dp) = uv - pi((exp(delta) * T_wc)^-1 (p + dp)), derivatives at 0
  // (the reference's DualScalar check, real_lie_group.rs:340-390).
  using D = Dual<9>;
  D xi[6], tw[7], T[7], pt[3], r[2];
  for (int i = 0; i < 6; ++i) { xi[i] = D(0.0); xi[i].d[i] = 1.0; }
  for (int i = 0; i < 7; ++i) T[i] = D(pose[i]);
  for (int i = 0; i < 3; ++i) { pt[i] = D(point[i]); pt[i].d[6 + i] = 1.0; }
  D e[7];
  se3_exp<D>(xi, e);
  se3_mul<D>(e, T, tw);
  residual_generic<D>(tw, pt, intr, uv, r);
  for (int i = 0; i < 2; ++i) {
    for (int j = 0; j < 6; ++j) j_pose[i * 6 + j] = r[i].d[j];
    for (int j = 0; j < 3; ++j) j_point[i * 3 + j] = r[i].d[6 + j];
  }
}

int ora_block_ldlt_solve(int n, int bs, const double* a, const double* b, double* x) {
  BlockLdlt f;
  int st = f.factorize(n, bs, a);
  if (st != 0) return st;
  std::memcpy(x, b, sizeof(double) * n);
  f.solve(x);
  return 0;
}

double ora_total_cost(const ora_problem* p, int n_threads) {
  double intr[6];
  problem_intrinsics(p, intr);
  return total_cost(p, intr, p->poses, p->points, n_threads);
}

void ora_eval_term_ex(const double pose[7], const double point[3], const double intr[6],
                      int32_t camera_model, const double uv[2], double r[2], double j_pose[12],
                      double j_point[6], double j_cam[12]) {
  double w, cost;
  eval_term_f64(pose, point, intr, uv, 0.0, r, j_pose, j_point, &w, &cost, j_cam, camera_model);
}

void ora_eval_term_intrinsics(const double pose[7], const double point[3], const double intr[4],
                              double j_cam[8]) {
  const double uv[2] = {0.0, 0.0};
  double r[2], jp[12], jm[6], w, cost;
  eval_term_f64(pose, point, intr, uv, 0.0, r, jp, jm, &w, &cost, j_cam);
}

int64_t ora_dense_system(const ora_problem* p, double nu, double* h, double* neg_grad) {
  Structure s;
  build_structure(p, &s);
  const int nc = cam_params(p);
  const int64_t c0 = p->intrinsics_free ? nc : 0;  // scalars of the free intrinsics, first
  int64_t n = c0 + static_cast<int64_t>(s.nf) * 6 + static_cast<int64_t>(s.nm) * 3;
  if (!h || !neg_grad) return n;
  double intr[6];
  problem_intrinsics(p, intr);
  System<double> sys;
  build_system<double>(p, s, intr, p->poses, p->points, nu, 1, &sys);
  std::fill(h, h + n * n, 0.0);
  const int64_t off = c0 + static_cast<int64_t>(s.nf) * 6;
  for (int f = 0; f < s.nf; ++f)
    for (int r = 0; r < 6; ++r) {
      for (int c = 0; c < 6; ++c) h[(c0 + f * 6 + r) * n + c0 + f * 6 + c] = sys.U[f * 36 + r * 6 + c];
      neg_grad[c0 + f * 6 + r] = sys.bp[f * 6 + r];
    }
  for (int m = 0; m < s.nm; ++m)
    for (int r = 0; r < 3; ++r) {
      for (int c = 0; c < 3; ++c) h[(off + m * 3 + r) * n + off + m * 3 + c] = sys.V[m * 9 + r * 3 + c];
      neg_grad[off + m * 3 + r] = sys.bm[m * 3 + r];
    }
  for (size_t e = 0; e < sys.off_row.size(); ++e)
    for (int r = 0; r < 6; ++r)
      for (int c = 0; c < 6; ++c) {
        const double v = sys.off_blk[e * 36 + r * 6 + c];
        h[(c0 + sys.off_row[e] * 6 + r) * n + c0 + sys.off_col[e] * 6 + c] += v;
        h[(c0 + sys.off_col[e] * 6 + c) * n + c0 + sys.off_row[e] * 6 + r] += v;
      }
  for (size_t r = 0; r + 1 < s.range_begin.size(); ++r) {
    int fb = s.pose_block[s.rng_pose[r]], mb = s.point_block[s.rng_pt[r]];
    if (fb < 0 || mb < 0) continue;
    for (int i = 0; i < 3; ++i)
      for (int c = 0; c < 6; ++c) {
        double w = sys.Wr[r * 18 + i * 6 + c];
        h[(off + mb * 3 + i) * n + c0 + fb * 6 + c] += w;
        h[(c0 + fb * 6 + c) * n + off + mb * 3 + i] += w;
      }
  }
  if (c0) {
    for (int r = 0; r < nc; ++r) {
      for (int c = 0; c < nc; ++c) h[r * n + c] = sys.Ucc[r * nc + c];
      neg_grad[r] = sys.bc[r];
    }
    for (int f = 0; f < s.nf; ++f)
      for (int r = 0; r < 6; ++r)
        for (int c = 0; c < nc; ++c) {
          const double v = sys.Hpc[f * 6 * nc + r * nc + c];
          h[(c0 + f * 6 + r) * n + c] = v;
          h[c * n + c0 + f * 6 + r] = v;
        }
    for (int m = 0; m < s.nm; ++m)
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < nc; ++c) {
          const double v = sys.Hmc[m * 3 * nc + r * nc + c];
          h[(off + m * 3 + r) * n + c] = v;
          h[c * n + off + m * 3 + r] = v;
        }
  }
  return n;
}

int ora_schur_step(const ora_problem* p, double nu, int n_threads, int emulate_fp32,
                   double* delta, double* s_out, double* rhs_bar_out) {
  Structure s;
  build_structure(p, &s);
  double intr[6];
  problem_intrinsics(p, intr);
  std::vector<double> d, S, rhs;
  int st = emulate_fp32
               ? schur_step_impl<float>(p, s, intr, p->poses, p->points, nu, n_threads, &d, nullptr,
                                        nullptr, s_out ? &S : nullptr, rhs_bar_out ? &rhs : nullptr)
               : schur_step_impl<double>(p, s, intr, p->poses, p->points, nu, n_threads, &d, nullptr,
                                         nullptr, s_out ? &S : nullptr, rhs_bar_out ? &rhs : nullptr);
  if (st != 0) return st;
  std::memcpy(delta, d.data(), sizeof(double) * d.size());
  if (s_out) std::memcpy(s_out, S.data(), sizeof(double) * S.size());
  if (rhs_bar_out) std::memcpy(rhs_bar_out, rhs.data(), sizeof(double) * rhs.size());
  return 0;
}

int ora_optimize(const ora_problem* p, const ora_params* prm, int n_threads,
                 ora_record* records, int cap, int* n_records, double* poses_out,
                 double* points_out) {
  return ora_optimize_ex(p, prm, n_threads, records, cap, n_records, poses_out, points_out, nullptr);
}

int ora_optimize_ex(const ora_problem* p, const ora_params* prm, int n_threads,
                    ora_record* records, int cap, int* n_records, double* poses_out,
                    double* points_out, double* intrinsics_out) {
  Structure s;
  build_structure(p, &s);
  // SchurMissingFreeOrMarg: no free or no marginalized scalars
  if ((s.nf == 0 && !p->intrinsics_free) || s.nm == 0) return -10;
  std::vector<double> intr(6), nintr(6);
  problem_intrinsics(p, intr.data());
  std::vector<double> poses(p->poses, p->poses + 7 * p->n_cam);
  std::vector<double> points(p->points, p->points + 3 * p->n_pt);
  std::vector<double> npose(poses.size()), npts(points.size());
  for (int k = 0; k < p->n_eq; ++k)
    if (p->eq_pose[k] < 0 || p->eq_pose[k] >= p->n_cam) return -11;
  if (!priors_valid(p)) return -12;
  if (!edges_valid(p)) return -13;
  EqTerms eq;
  std::vector<double> lambda(p->n_eq, 0.0);  // EqSystem::new: zero multipliers
  double merit = total_cost(p, intr.data(), poses.data(), points.data(), n_threads);
  double nu = prm->initial_lm_damping;
  int64_t rejects = 0;
  int64_t steps = 0;
  int nrec = 0;
  int rc = 0;
  for (;;) {
    ora_record rec;
    rec.new_merit = NAN;
    rec.gain_ratio = NAN;
    rec.max_step = NAN;
    rec.accepted = 0;
    int reason = ORA_TERM_NONE;
    std::vector<double> delta, neg_grad;
    double max_grad = 0.0;
    const EqTerms* eqp = nullptr;
    if (p->n_eq > 0) {  // eq_system.eval before the cost system (optimizer_helpers.rs:277-283)
      eq_eval(p, &s, poses.data(), &eq);
      eqp = &eq;
    }
    int st = prm->emulate_fp32
                 ? schur_step_impl<float>(p, s, intr.data(), poses.data(), points.data(), nu, n_threads, &delta,
                                          &max_grad, &neg_grad, nullptr, nullptr,
                                          prm->gradient_tolerance, eqp, lambda.data())
                 : schur_step_impl<double>(p, s, intr.data(), poses.data(), points.data(), nu, n_threads, &delta,
                                           &max_grad, &neg_grad, nullptr, nullptr,
                                           prm->gradient_tolerance, eqp, lambda.data());
    rec.max_grad = max_grad;
    if (st == 1) {
      reason = ORA_TERM_GRADIENT_TOL;
    } else if (st != 0) {
      // handle_solve_failure -> reject_step (optimizer.rs:470-485)
      nu *= 2.0;
      rejects += 1;
      if (rejects >= prm->max_consecutive_rejects) reason = ORA_TERM_MAX_REJECTS;
    } else {
      bool valid = apply_update(p, s, delta, intr.data(), poses.data(), points.data(), nintr.data(),
                                npose.data(), npts.data());
      if (!valid) { rc = -3; }  // the reference panics in from_params
      double new_merit = total_cost(p, nintr.data(), npose.data(), npts.data(), n_threads);
      rec.new_merit = new_merit;
      double max_step = 0.0;
      for (double v : delta) max_step = std::max(max_step, std::fabs(v));
      rec.max_step = max_step;
      if (max_step < prm->parameter_tolerance) {
        if (new_merit < merit) {
          intr.swap(nintr); poses.swap(npose); points.swap(npts); merit = new_merit; rec.accepted = 1;
          update_lambdas(p->n_eq, delta, &lambda);
        }
        reason = ORA_TERM_PARAMETER_TOL;
      } else {
        // compute_gain_ratio (optimizer_helpers.rs:159-173)
        double dd = 0.0, dg = 0.0;
        for (size_t i = 0; i < delta.size(); ++i) { dd += delta[i] * delta[i]; dg += delta[i] * neg_grad[i]; }
        double predicted = nu * dd + dg;
        double actual = merit - new_merit;
        double rho = (std::fabs(predicted) > kMinPositive) ? actual / predicted
                                                            : (actual > 0.0 ? 1.0 : 0.0);
        rec.gain_ratio = rho;
        if (rho > 0.0 && new_merit < merit) {
          double x = 2.0 * rho - 1.0;
          double f = 1.0 - x * x * x;
          nu *= std::max(f, 1.0 / 3.0);
          rejects = 0;
          double rel = (merit - new_merit) / (std::fabs(merit) + kMinPositive);
          if (rel < prm->function_tolerance) reason = ORA_TERM_FUNCTION_TOL;
          intr.swap(nintr); poses.swap(npose); points.swap(npts); merit = new_merit; rec.accepted = 1;
          update_lambdas(p->n_eq, delta, &lambda);
        } else {
          nu *= 2.0;
          rejects += 1;
          if (rejects >= prm->max_consecutive_rejects) reason = ORA_TERM_MAX_REJECTS;
        }
      }
    }
    steps += 1;
    if (steps >= prm->num_iterations && reason == ORA_TERM_NONE) reason = ORA_TERM_MAX_ITERATIONS;
    rec.merit = merit;
    rec.lm_damping = nu;
    rec.termination = reason;
    if (nrec < cap && records) records[nrec] = rec;
    ++nrec;
    if (reason != ORA_TERM_NONE) break;
  }
  if (n_records) *n_records = nrec;
  if (poses_out) std::memcpy(poses_out, poses.data(), sizeof(double) * poses.size());
  if (points_out) std::memcpy(points_out, points.data(), sizeof(double) * points.size());
  if (intrinsics_out) std::memcpy(intrinsics_out, intr.data(), sizeof(double) * 6);
  return rc;
}

int ora_covariance_block(const ora_problem* p, int32_t row_kind, int32_t row_index, int32_t col_kind,
                         int32_t col_index, double* out, int32_t* rows, int32_t* cols) {
  CovCtx c;
  const int st = cov_build(p, &c);
  if (st != 0) return st;
  auto point_ok = [&](int q) { return q >= 0 && q < p->n_pt && c.s.point_block[q] >= 0; };
  const bool rf = row_kind != ORA_VAR_POINT, cf = col_kind != ORA_VAR_POINT;
  int rd = 3, cd = 3;
  const int ro = rf ? cov_free_offset(p, c, row_kind, row_index, &rd) : (point_ok(row_index) ? 0 : -1);
  const int co = cf ? cov_free_offset(p, c, col_kind, col_index, &cd) : (point_ok(col_index) ? 0 : -1);
  if (ro < 0 || co < 0) return -1;
  if (rows) *rows = rd;
  if (cols) *cols = cd;
  const int n = c.n;
  if (rf && cf) {
    for (int a = 0; a < rd; ++a)
      for (int b = 0; b < cd; ++b) out[a * cd + b] = c.Sinv[static_cast<size_t>(ro + a) * n + co + b];
    return 0;
  }
  if (rf || cf) {  // free x marg, or its transpose
    const int q = rf ? col_index : row_index;
    const int off = rf ? ro : co, dim = rf ? rd : cd;
    double hinv[9];
    if (!cov_hmm_inv(c, q, hinv)) return -2;
    std::vector<double> fm(static_cast<size_t>(dim) * 3);
    cov_free_marg(c, off, dim, cov_hmf(p, c, q), hinv, fm.data());
    for (int a = 0; a < dim; ++a)
      for (int j = 0; j < 3; ++j) {
        if (rf) out[a * 3 + j] = fm[a * 3 + j];
        else out[j * dim + a] = fm[a * 3 + j];
      }
    return 0;
  }
  // marg x marg: H_mm[i]^-1 H_mf_i S^-1 H_mf_j^T H_mm[j]^-1 (+ H_mm[i]^-1 on the diagonal)
  double hi[9], hj[9];
  if (!cov_hmm_inv(c, row_index, hi) || !cov_hmm_inv(c, col_index, hj)) return -2;
  const std::vector<double> fi = cov_hmf(p, c, row_index), fj = cov_hmf(p, c, col_index);
  double core[9];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      double acc = 0.0;
      for (int k = 0; k < n; ++k) {
        double sk = 0.0;
        for (int l = 0; l < n; ++l) sk += c.Sinv[static_cast<size_t>(k) * n + l] * fj[static_cast<size_t>(b) * n + l];
        acc += fi[static_cast<size_t>(a) * n + k] * sk;
      }
      core[a * 3 + b] = acc;
    }
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      double v = 0.0;
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) v += hi[a * 3 + k] * core[k * 3 + l] * hj[l * 3 + b];
      if (row_index == col_index) v += hi[a * 3 + b];
      out[a * 3 + b] = v;
    }
  return 0;
}

void ora_eval_prior(const double pose[7], const double mean[7], const double precision[36], double r[6],
                    double j_pose[36], double* cost) {
  double h[36], gp[6];
  prior_term(pose, mean, precision, r, j_pose, h, gp, cost);
}

void ora_se3_log(const double params[7], double out[6]) { se3_log<double>(params, out); }

void ora_eval_edge(const double pose_m[7], const double pose_n[7], const double m_from_n[7], double r[6],
                   double j_m[36], double j_n[36], double* cost) {
  edge_term(pose_m, pose_n, m_from_n, r, j_m, j_n, cost);
}

int ora_min_norm_pinv(int n, int bs, const double* a, double* out) {
  if (n <= 0 || bs <= 0 || n % bs != 0) return -1;
  BlockLdlt f;
  if (f.factorize(n, bs, a) != 0) return -2;
  std::vector<double> pinv;
  int rank = 0;
  for (int j = 0; j < n; ++j) rank += f.d[j] > 0.0 ? 1 : 0;
  if (pseudo_inverse(f, &pinv) != 0) return -2;
  std::memcpy(out, pinv.data(), sizeof(double) * pinv.size());
  return rank;
}

void ora_eq_eval(const ora_problem* p, const double* poses, double* c, double* jac) {
  EqTerms e;
  eq_eval(p, nullptr, poses, &e);
  if (c) std::memcpy(c, e.c.data(), sizeof(double) * e.c.size());
  if (jac) std::memcpy(jac, e.jac.data(), sizeof(double) * e.jac.size());
}

int ora_schur_kkt_step(const ora_problem* p, double nu, const double* lambda, int n_threads, double* delta) {
  for (int k = 0; k < p->n_eq; ++k)
    if (p->eq_pose[k] < 0 || p->eq_pose[k] >= p->n_cam) return -11;
  Structure s;
  build_structure(p, &s);
  double intr[6];
  problem_intrinsics(p, intr);
  EqTerms eq;
  eq_eval(p, &s, p->poses, &eq);
  std::vector<double> d;
  int st = schur_step_impl<double>(p, s, intr, p->poses, p->points, nu, n_threads, &d, nullptr, nullptr,
                                   nullptr, nullptr, -1.0, &eq, lambda);
  if (st != 0) return st;
  std::memcpy(delta, d.data(), sizeof(double) * d.size());
  return 0;
}

}  // extern "C"
