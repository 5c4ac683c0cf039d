// sgba_lie.cuh -- SE(3) in f64 on the device, with forward-mode derivatives
// in six directions, for cost terms on the poses themselves (the pose prior).
// Restates sophus_lie's unit-quaternion rotation and its affine group:
//   Rotation3 multiplication, matrix, log, mat_v_inverse and the w >= 0
//   disambiguation (crates/sophus_lie/src/groups/rotation3.rs:176-182,
//   389-410, 449-492, 778-800; crates/sophus_lie/src/lie_group/quaternion.rs);
//   the affine group's multiplication, inverse and log
//   (crates/sophus_lie/src/groups/affine_group_template.rs:362-404).
// Parameters (qw qx qy qz tx ty tz); tangent (w, v), rotation first.
#pragma once

#include <cuda_runtime.h>

namespace sgba {
namespace lie {

constexpr double kLieEps = 1e-6;  // EPS_F64 (crates/sophus_autodiff/src/linalg.rs:75)

// A value and its derivatives in six directions.
struct D6 {
  double v;
  double d[6];
};

__device__ __forceinline__ D6 dc(double v) {
  D6 r;
  r.v = v;
#pragma unroll
  for (int i = 0; i < 6; ++i) r.d[i] = 0.0;
  return r;
}
__device__ __forceinline__ D6 operator+(const D6& a, const D6& b) {
  D6 r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < 6; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
__device__ __forceinline__ D6 operator-(const D6& a, const D6& b) {
  D6 r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < 6; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
__device__ __forceinline__ D6 operator-(const D6& a) {
  D6 r;
  r.v = -a.v;
#pragma unroll
  for (int i = 0; i < 6; ++i) r.d[i] = -a.d[i];
  return r;
}
__device__ __forceinline__ D6 operator*(const D6& a, const D6& b) {
  D6 r;
  r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < 6; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
__device__ __forceinline__ D6 operator/(const D6& a, const D6& b) {
  D6 r;
  r.v = a.v / b.v;
  const double inv = 1.0 / b.v;
#pragma unroll
  for (int i = 0; i < 6; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * inv;
  return r;
}
__device__ __forceinline__ D6 dsqrt(const D6& a) {
  D6 r;
  r.v = sqrt(a.v);
  const double h = 0.5 / r.v;
#pragma unroll
  for (int i = 0; i < 6; ++i) r.d[i] = a.d[i] * h;
  return r;
}
__device__ __forceinline__ D6 dsin(const D6& a) {
  D6 r;
  r.v = sin(a.v);
  const double c = cos(a.v);
#pragma unroll
  for (int i = 0; i < 6; ++i) r.d[i] = a.d[i] * c;
  return r;
}
__device__ __forceinline__ D6 dcos(const D6& a) {
  D6 r;
  r.v = cos(a.v);
  const double s = -sin(a.v);
#pragma unroll
  for (int i = 0; i < 6; ++i) r.d[i] = a.d[i] * s;
  return r;
}
// atan2(y, x): derivative (x dy - y dx) / (x^2 + y^2)
__device__ __forceinline__ D6 datan2(const D6& y, const D6& x) {
  D6 r;
  r.v = atan2(y.v, x.v);
  const double inv = 1.0 / (y.v * y.v + x.v * x.v);
#pragma unroll
  for (int i = 0; i < 6; ++i) r.d[i] = (x.v * y.d[i] - y.v * x.d[i]) * inv;
  return r;
}

__device__ __forceinline__ double val(double a) { return a; }
__device__ __forceinline__ double val(const D6& a) { return a.v; }
__device__ __forceinline__ double dsqrt(double a) { return sqrt(a); }
__device__ __forceinline__ double dsin(double a) { return sin(a); }
__device__ __forceinline__ double dcos(double a) { return cos(a); }
__device__ __forceinline__ double datan2(double y, double x) { return atan2(y, x); }
template <class S>
__device__ __forceinline__ S cst(double v);
template <>
__device__ __forceinline__ double cst<double>(double v) {
  return v;
}
template <>
__device__ __forceinline__ D6 cst<D6>(double v) {
  return dc(v);
}

// Hamilton product: real a0 b0 - a_v . b_v, imaginary b_v a0 + a_v b0 + a_v x b_v
template <class S>
__device__ void quat_mul(const S* a, const S* b, S* o) {
  const S re = a[0] * b[0] - (a[1] * b[1] + a[2] * b[2] + a[3] * b[3]);
  const S c0 = a[2] * b[3] - a[3] * b[2];
  const S c1 = a[3] * b[1] - a[1] * b[3];
  const S c2 = a[1] * b[2] - a[2] * b[1];
  const S i0 = b[1] * a[0] + a[1] * b[0] + c0;
  const S i1 = b[2] * a[0] + a[2] * b[0] + c1;
  const S i2 = b[3] * a[0] + a[3] * b[0] + c2;
  o[0] = re;
  o[1] = i0;
  o[2] = i1;
  o[3] = i2;
}

// rotation matrix of a unit quaternion, row-major
template <class S>
__device__ void quat_matrix(const S* q, S* m) {
  const S one = cst<S>(1.0), two = cst<S>(2.0);
  const S x2 = two * q[1], y2 = two * q[2], z2 = two * q[3], r2 = two * q[0];
  const S xx = x2 * q[1], yy = y2 * q[2], zz = z2 * q[3];
  const S xy = x2 * q[2], xz = x2 * q[3], yz = y2 * q[3];
  const S rx = r2 * q[1], ry = r2 * q[2], rz = r2 * q[3];
  m[0] = one - (yy + zz);
  m[1] = xy - rz;
  m[2] = xz + ry;
  m[3] = xy + rz;
  m[4] = one - (xx + zz);
  m[5] = yz - rx;
  m[6] = xz - ry;
  m[7] = yz + rx;
  m[8] = one - (xx + yy);
}

// keep the real part non-negative
template <class S>
__device__ void quat_disambiguate(S* q) {
  if (!(0.0 <= val(q[0]))) {
#pragma unroll
    for (int i = 0; i < 4; ++i) q[i] = -q[i];
  }
}

// a * b
template <class S>
__device__ void se3_mul(const S* a, const S* b, S* o) {
  S q[4], m[9];
  quat_mul(a, b, q);
  quat_matrix(a, m);
#pragma unroll
  for (int i = 0; i < 3; ++i) o[4 + i] = (m[3 * i] * b[4] + m[3 * i + 1] * b[5] + m[3 * i + 2] * b[6]) + a[4 + i];
#pragma unroll
  for (int i = 0; i < 4; ++i) o[i] = q[i];
  quat_disambiguate(o);
}

// a^-1: conjugate rotation, -R^T t
__device__ inline void se3_inverse(const double* a, double* o) {
  double q[4] = {a[0], -a[1], -a[2], -a[3]};
  double m[9];
  quat_matrix(q, m);
  for (int i = 0; i < 3; ++i) o[4 + i] = -(m[3 * i] * a[4] + m[3 * i + 1] * a[5] + m[3 * i + 2] * a[6]);
  for (int i = 0; i < 4; ++i) o[i] = q[i];
  quat_disambiguate(o);
}

// rotation log: 2 atan(|v| / w) v / |v| (sign of w folded in), or the series
// 2 / w - (2/3) |v|^2 / w^3 for |v|^2 <= eps^2
template <class S>
__device__ void so3_log(const S* q, S* w) {
  const S sq = q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  const S qw = q[0];
  S f;
  if (val(sq) <= kLieEps * kLieEps) {
    const S wsq = qw * qw;
    f = cst<S>(2.0) / qw - cst<S>(2.0 / 3.0) * sq / (wsq * qw);
  } else {
    const S n = dsqrt(sq);
    const S sign = val(qw) <= 0.0 ? cst<S>(-1.0) : cst<S>(1.0);
    const S at = sign * datan2(n, sign * qw);
    f = cst<S>(2.0) * at / n;
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) w[i] = q[1 + i] * f;
}

// V(w)^-1 = I - W/2 + c W^2, c = (1 - (theta/2) cos(theta/2) / sin(theta/2)) / theta^2
// (1/12 for theta^2 <= eps); row-major
template <class S>
__device__ void so3_mat_v_inverse(const S* w, S* m) {
  const S th_sq = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  const S z = cst<S>(0.0);
  const S hat[9] = {z, -w[2], w[1], w[2], z, -w[0], -w[1], w[0], z};
  S c;
  if (val(th_sq) <= kLieEps) {
    c = cst<S>(1.0 / 12.0);
  } else {
    const S th = dsqrt(th_sq);
    const S half = cst<S>(0.5) * th;
    c = (cst<S>(1.0) - (cst<S>(0.5) * th * dcos(half)) / dsin(half)) / (th * th);
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const S h2 = hat[3 * i] * hat[j] + hat[3 * i + 1] * hat[3 + j] + hat[3 * i + 2] * hat[6 + j];
      m[3 * i + j] = (i == j ? cst<S>(1.0) : z) - hat[3 * i + j] * cst<S>(0.5) + h2 * c;
    }
}

// log of (q, t): (w, V(w)^-1 t)
template <class S>
__device__ void se3_log(const S* a, S* xi) {
  so3_log(a, xi);
  S m[9];
  so3_mat_v_inverse(xi, m);
#pragma unroll
  for (int i = 0; i < 3; ++i) xi[3 + i] = m[3 * i] * a[4] + m[3 * i + 1] * a[5] + m[3 * i + 2] * a[6];
}

// exp(x) at x = 0 carried as derivatives: rotation (1, x_w / 2), translation x_v
// (the first-order terms of both branches of the group exponential at zero)
__device__ inline void se3_exp_at_zero(D6* e) {
  for (int i = 0; i < 7; ++i) e[i] = dc(i == 0 ? 1.0 : 0.0);
  for (int i = 0; i < 3; ++i) e[1 + i].d[i] = 0.5;
  for (int i = 0; i < 3; ++i) e[4 + i].d[3 + i] = 1.0;
}

}  // namespace lie
}  // namespace sgba
