// sgba_kernels.cu -- per-iteration kernels of the GB300 Schur-LM bundle
// adjustment (everything except the reduced-camera-system factorization,
// which lives in sgba_solver.cu).
//
// Precision plan (GB300 runs FP32 at ~64x its FP64 rate):
//   * Jacobians and all block products in FP32 on the CUDA cores;
//   * every sum that the reference forms in f64 (Hessian blocks, gradients,
//     Schur complement, cost, step statistics) is carried in float-float
//     (sgba_dd.cuh) and stored as f64;
//   * f64 proper only for the SE(3) update of the poses and tiny scalars.
// Reductions use fixed partitions and fixed trees: results are
// bit-reproducible from run to run.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <vector>
#include <mutex>

#include "sgba_dd.cuh"
#include "sgba_internal.h"

namespace sgba {

namespace {

constexpr int kCostThreads = 256;
constexpr int kCostMaxBlocks = 1216;  // 8 x 152 SMs
constexpr double kEps = 1e-6;         // EPS_F64 (crates/sophus_autodiff/src/linalg.rs:75)

__device__ __forceinline__ bool halted(const Ctrl* c) { return c->done != 0; }
__device__ __forceinline__ bool skipping(const Ctrl* c) { return c->done != 0 || c->skip != 0; }

__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* addr, double v) {
  // Non-negative doubles order like their bit patterns.
  if (!(v >= 0.0)) v = (v != v) ? __longlong_as_double(0x7ff8000000000000ll) : 0.0;
  atomicMax(addr, static_cast<unsigned long long>(__double_as_longlong(v)));
}

// --- SE(3) in f64 (restated from sophus_lie, see the oracle for citations) --
// Rotation3Impl::matrix (crates/sophus_lie/src/groups/rotation3.rs:449-492)
__device__ void rot_matrix(const double* q, double* m) {
  double r = q[0], x = q[1], y = q[2], z = q[3];
  double tx = 2.0 * x, ty = 2.0 * y, tz = 2.0 * z, tr = 2.0 * r;
  double txx = tx * x, tyy = ty * y, tzz = tz * z;
  double txy = tx * y, txz = tx * z, tyz = ty * z;
  double trx = tr * x, try_ = tr * y, trz = tr * z;
  m[0] = 1.0 - (tyy + tzz); m[1] = txy - trz; m[2] = txz + try_;
  m[3] = txy + trz; m[4] = 1.0 - (txx + tzz); m[5] = tyz - trx;
  m[6] = txz - try_; m[7] = tyz + trx; m[8] = 1.0 - (txx + tyy);
}

// Left-perturbation update T <- exp(xi) * T
// (crates/sophus_lie/src/lie_group/lie_group_manifold.rs:33-35,57-64;
//  exp: crates/sophus_lie/src/groups/affine_group_template.rs:354-360,
//       crates/sophus_lie/src/groups/rotation3.rs:363-387 and mat_v :761-778;
//  group_mul: affine_group_template.rs:387-396, quaternion.rs:212-225;
//  disambiguate: rotation3.rs:176-182).
__device__ void se3_left_update(const double* xi, const double* T, double* out) {
  const double w0 = xi[0], w1 = xi[1], w2 = xi[2];
  double th2 = w0 * w0 + w1 * w1 + w2 * w2;
  double eq[4];
  if (th2 <= kEps * kEps) {
    double th4 = th2 * th2;
    double im = 0.5 - (1.0 / 48.0) * th2 + (1.0 / 3840.0) * th4;
    eq[0] = 1.0 - (1.0 / 8.0) * th2 + (1.0 / 384.0) * th4;
    eq[1] = im * w0; eq[2] = im * w1; eq[3] = im * w2;
  } else {
    double th = sqrt(th2);
    double s, c;
    sincos(0.5 * th, &s, &c);
    double im = s / th;
    eq[0] = c; eq[1] = im * w0; eq[2] = im * w1; eq[3] = im * w2;
  }
  // mat_v * nu
  double h[9] = {0.0, -w2, w1, w2, 0.0, -w0, -w1, w0, 0.0};
  double v[9];
  if (th2 <= kEps) {
    for (int i = 0; i < 9; ++i) v[i] = 0.5 * h[i];
  } else {
    double h2[9];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        h2[i * 3 + j] = h[i * 3 + 0] * h[0 * 3 + j] + h[i * 3 + 1] * h[1 * 3 + j] + h[i * 3 + 2] * h[2 * 3 + j];
    double th = sqrt(th2);
    double a = (1.0 - cos(th)) / th2;
    double b = (th - sin(th)) / (th2 * th);
    for (int i = 0; i < 9; ++i) v[i] = a * h[i] + b * h2[i];
  }
  v[0] += 1.0; v[4] += 1.0; v[8] += 1.0;
  double et[3];
  for (int i = 0; i < 3; ++i) et[i] = v[i * 3 + 0] * xi[3] + v[i * 3 + 1] * xi[4] + v[i * 3 + 2] * xi[5];
  if (!(0.0 <= eq[0])) { for (int i = 0; i < 4; ++i) eq[i] = -eq[i]; }
  // exp(xi) * T
  const double* b = T;
  double q[4];
  q[0] = eq[0] * b[0] - (eq[1] * b[1] + eq[2] * b[2] + eq[3] * b[3]);
  q[1] = b[1] * eq[0] + eq[1] * b[0] + (eq[2] * b[3] - eq[3] * b[2]);
  q[2] = b[2] * eq[0] + eq[2] * b[0] + (eq[3] * b[1] - eq[1] * b[3]);
  q[3] = b[3] * eq[0] + eq[3] * b[0] + (eq[1] * b[2] - eq[2] * b[1]);
  double r[9];
  rot_matrix(eq, r);
  for (int i = 0; i < 3; ++i)
    out[4 + i] = (r[i * 3 + 0] * b[4] + r[i * 3 + 1] * b[5] + r[i * 3 + 2] * b[6]) + et[i];
  if (!(0.0 <= q[0])) { for (int i = 0; i < 4; ++i) q[i] = -q[i]; }
  for (int i = 0; i < 4; ++i) out[i] = q[i];
}

// HuberKernel (crates/sophus_opt/src/robust_kernel.rs:13-35): weight applied to
// the residual; H stays J^T J.
__device__ __forceinline__ float huber_weight_f(float huber, float r0, float r1) {
  if (!(huber > 0.0f)) return 1.0f;
  float nrm = sqrtf(r0 * r0 + r1 * r1);
  if (nrm == 0.0f) return 0.0f;
  if (nrm <= huber) return 1.0f;
  return sqrtf(2.0f * huber * nrm - huber * huber) / nrm;
}

// Accumulator of a float-float dot product: hi carries the running sum through
// an exact TwoSum, the rounding errors of the products and of the sums go into
// the float lo.
struct Acc {
  float hi, lo;
};
__device__ __forceinline__ Acc acc_zero() { return Acc{0.0f, 0.0f}; }
__device__ __forceinline__ void acc_madd(Acc& a, dd x, dd y) {
  const float p = __fmul_rn(x.hi, y.hi);
  float e = __fmaf_rn(x.hi, y.hi, -p);
  e = __fmaf_rn(x.hi, y.lo, e);
  e = __fmaf_rn(x.lo, y.hi, e);
  const float s = __fadd_rn(a.hi, p);
  const float bb = __fsub_rn(s, a.hi);
  const float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  a.hi = s;
  a.lo = __fadd_rn(a.lo, __fadd_rn(err, e));
}
__device__ __forceinline__ void acc_addf(Acc& a, float y) {
  const float s = __fadd_rn(a.hi, y);
  const float bb = __fsub_rn(s, a.hi);
  const float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(y, bb));
  a.hi = s;
  a.lo = __fadd_rn(a.lo, err);
}
__device__ __forceinline__ dd acc_get(const Acc& a) { return dd_fast_two_sum(a.hi, a.lo); }

// The same weighting in float-float: r~ = w r with w = sqrt(rho(|r|)) / |r|.
__device__ __forceinline__ void huber_weighted_dd(float huber, dd huber_dd, dd r0, dd r1, dd* o0, dd* o1) {
  if (!(huber > 0.0f)) {
    *o0 = r0;
    *o1 = r1;
    return;
  }
  const dd n2 = dd_add(dd_mul(r0, r0), dd_mul(r1, r1));
  const dd nrm = dd_sqrt(n2);
  if (nrm.hi == 0.0f) {
    *o0 = dd_make(0.0f, 0.0f);
    *o1 = dd_make(0.0f, 0.0f);
    return;
  }
  if (nrm.hi < huber || (nrm.hi == huber_dd.hi && nrm.lo <= huber_dd.lo)) {
    *o0 = r0;
    *o1 = r1;
    return;
  }
  const dd rho = dd_sub(dd_mul(dd_add(huber_dd, huber_dd), nrm), dd_mul(huber_dd, huber_dd));
  const dd w = dd_div(dd_sqrt(rho), nrm);
  *o0 = dd_mul(w, r0);
  *o1 = dd_mul(w, r1);
}

// The camera of the projection: fx fy (cx cy enter only the residual) and,
// for the enhanced unified camera model, alpha beta
// (crates/sophus_sensor/src/distortions/enhanced_unified.rs:59-88).  The
// device intrinsics hold fx fy cx cy alpha beta (alpha = beta = 0 for the
// pinhole).  The kernels that evaluate Jacobians are instantiated per camera
// model (template flag E), so the pinhole path carries no EUCM code.
struct CamF {
  float fx, fy, alpha, beta;
};
struct CamD {
  dd fx, fy, alpha, beta, one_m_alpha;
};
__device__ __forceinline__ CamF cam_f(const double* intr) {
  return CamF{__double2float_rn(intr[0]), __double2float_rn(intr[1]), __double2float_rn(intr[4]),
              __double2float_rn(intr[5])};
}
__device__ __forceinline__ CamD cam_dd(const double* intr) {
  return CamD{dd_from_double(intr[0]), dd_from_double(intr[1]), dd_from_double(intr[4]), dd_from_double(intr[5]),
              dd_from_double(1.0 - intr[4])};
}

// EUCM distortion of the z = 1 projection (x, y): the distorted point
// (x / norm, y / norm) with rho = sqrt(beta (x^2 + y^2) + 1),
// norm = alpha rho + (1 - alpha)  (enhanced_unified.rs:59-88), in float-float.
__device__ __forceinline__ dd eucm_norm_dd(const CamD& c, dd x, dd y, dd* rho_out, dd* r2_out) {
  const dd r2 = dd_add(dd_mul(x, x), dd_mul(y, y));
  const dd rho = dd_sqrt(dd_add(dd_mul(c.beta, r2), dd_make(1.0f, 0.0f)));
  if (rho_out) *rho_out = rho;
  if (r2_out) *r2_out = r2;
  return dd_add(dd_mul(c.alpha, rho), c.one_m_alpha);
}

// Jacobians of r = z - pi(T_cw p) w.r.t. the left pose perturbation (2x6,
// tangent [omega; nu]) and the point (2x3), in FP32
// (crates/sophus_opt/src/nlls/functor_library/costs/pinhole_reprojection.rs:60-95).
// For the EUCM camera d pi = M d proj with M the 2x2 derivative of the
// distortion, dx_distort_x (enhanced_unified.rs:117-156):
//   M = [fx (norm - x n_x), -fx x n_y; -fy y n_x, fy (norm - y n_y)] / norm^2,
//   n_x = alpha beta x / rho, n_y = alpha beta y / rho,
// and d proj = [1, 0, -x; 0, 1, -y] / z (perspective.rs:30-39).
struct JacF {
  float jp[12];  // row-major 2x6
  float jm[6];   // row-major 2x3
};
template <bool E>  // E: the EUCM camera, else the pinhole
__device__ __forceinline__ void jacobians_f(const float* pt /*R_cw 9 + t_cw 3*/, float px, float py,
                                            float pz, const CamF& c, JacF* J) {
  float xc = pt[0] * px + pt[1] * py + pt[2] * pz + pt[9];
  float yc = pt[3] * px + pt[4] * py + pt[5] * pz + pt[10];
  float zc = pt[6] * px + pt[7] * py + pt[8] * pz + pt[11];
  float iz = 1.0f / zc;
  // D = dpi * R_cw (2x3)
  float D[6];
  if constexpr (!E) {
    float a0 = c.fx * iz, a2 = -c.fx * xc * iz * iz;
    float b1 = c.fy * iz, b2 = -c.fy * yc * iz * iz;
    for (int k = 0; k < 3; ++k) {
      D[k] = a0 * pt[0 * 3 + k] + a2 * pt[2 * 3 + k];
      D[3 + k] = b1 * pt[1 * 3 + k] + b2 * pt[2 * 3 + k];
    }
  } else {
    const float x = xc * iz, y = yc * iz;
    const float rho = sqrtf(c.beta * (x * x + y * y) + 1.0f);
    const float nrm = c.alpha * rho + (1.0f - c.alpha);
    const float in2 = 1.0f / (nrm * nrm);
    const float ab = c.alpha * c.beta / rho;
    const float nx = ab * x, ny = ab * y;
    const float m00 = c.fx * (nrm - x * nx) * in2, m01 = -c.fx * x * ny * in2;
    const float m10 = -c.fy * y * nx * in2, m11 = c.fy * (nrm - y * ny) * in2;
    const float a0 = m00 * iz, a1 = m01 * iz, a2 = -(m00 * x + m01 * y) * iz;
    const float b0 = m10 * iz, b1 = m11 * iz, b2 = -(m10 * x + m11 * y) * iz;
    for (int k = 0; k < 3; ++k) {
      D[k] = a0 * pt[0 * 3 + k] + a1 * pt[1 * 3 + k] + a2 * pt[2 * 3 + k];
      D[3 + k] = b0 * pt[0 * 3 + k] + b1 * pt[1 * 3 + k] + b2 * pt[2 * 3 + k];
    }
  }
  for (int r = 0; r < 2; ++r) {
    const float* d = D + 3 * r;
    // D * hat(-p)
    J->jp[r * 6 + 0] = -d[1] * pz + d[2] * py;
    J->jp[r * 6 + 1] = d[0] * pz - d[2] * px;
    J->jp[r * 6 + 2] = -d[0] * py + d[1] * px;
    J->jp[r * 6 + 3] = d[0];
    J->jp[r * 6 + 4] = d[1];
    J->jp[r * 6 + 5] = d[2];
    J->jm[r * 3 + 0] = -d[0];
    J->jm[r * 3 + 1] = -d[1];
    J->jm[r * 3 + 2] = -d[2];
  }
}


constexpr int kZS = 20;  // floats per Z row block (18 used; padded for float4 loads)
constexpr int kZD = kZddFloats;  // floats per float-float Z (36 used; padded for float4 loads)

// Sum over the 32 lanes of a warp of `nv` float values per lane, in
// float-float: values are transposed through shared memory (red[nv][33]) and
// lane v < nv adds the 32 entries of value v.  Returns the total of value
// `lane` (valid for lane < nv).  Deterministic (fixed order).
template <int NV>
__device__ __forceinline__ dd warp_transpose_sum(const float* vals, float (*red)[33]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int v = 0; v < NV; ++v) red[v][lane] = vals[v];
  __syncwarp();
  dd acc = dd_make(0.f, 0.f);
  if (lane < NV) {
#pragma unroll 8
    for (int l = 0; l < 32; ++l) acc = dd_add_f(acc, red[lane][l]);
  }
  __syncwarp();
  return acc;
}

// The same Jacobians in float-float, for ill-conditioned point blocks.
struct JacD {
  dd jp[12];
  dd jm[6];
};
template <bool E>
__device__ void jacobians_dd(const float* Pd /*R_cw 9 + t_cw 3, (hi, lo) pairs*/, dd px, dd py, dd pz, const CamD& c,
                             JacD* J) {
  dd R[9], t[3];
  for (int i = 0; i < 9; ++i) R[i] = dd_make(Pd[2 * i], Pd[2 * i + 1]);
  for (int i = 0; i < 3; ++i) t[i] = dd_make(Pd[18 + 2 * i], Pd[18 + 2 * i + 1]);
  dd xc = dd_add(dd_add(dd_add(dd_mul(R[0], px), dd_mul(R[1], py)), dd_mul(R[2], pz)), t[0]);
  dd yc = dd_add(dd_add(dd_add(dd_mul(R[3], px), dd_mul(R[4], py)), dd_mul(R[5], pz)), t[1]);
  dd zc = dd_add(dd_add(dd_add(dd_mul(R[6], px), dd_mul(R[7], py)), dd_mul(R[8], pz)), t[2]);
  dd iz = dd_div(dd_make(1.0f, 0.0f), zc);
  dd D[6];
  if constexpr (!E) {
    dd iz2 = dd_mul(iz, iz);
    dd a0 = dd_mul(c.fx, iz), a2 = dd_neg(dd_mul(dd_mul(c.fx, xc), iz2));
    dd b1 = dd_mul(c.fy, iz), b2 = dd_neg(dd_mul(dd_mul(c.fy, yc), iz2));
    for (int k = 0; k < 3; ++k) {
      D[k] = dd_add(dd_mul(a0, R[0 * 3 + k]), dd_mul(a2, R[2 * 3 + k]));
      D[3 + k] = dd_add(dd_mul(b1, R[1 * 3 + k]), dd_mul(b2, R[2 * 3 + k]));
    }
  } else {
    const dd x = dd_mul(xc, iz), y = dd_mul(yc, iz);
    dd rho;
    const dd nrm = eucm_norm_dd(c, x, y, &rho, nullptr);
    const dd in2 = dd_div(dd_make(1.0f, 0.0f), dd_mul(nrm, nrm));
    const dd ab = dd_div(dd_mul(c.alpha, c.beta), rho);
    const dd nx = dd_mul(ab, x), ny = dd_mul(ab, y);
    const dd m00 = dd_mul(dd_mul(c.fx, dd_sub(nrm, dd_mul(x, nx))), in2);
    const dd m01 = dd_neg(dd_mul(dd_mul(c.fx, dd_mul(x, ny)), in2));
    const dd m10 = dd_neg(dd_mul(dd_mul(c.fy, dd_mul(y, nx)), in2));
    const dd m11 = dd_mul(dd_mul(c.fy, dd_sub(nrm, dd_mul(y, ny))), in2);
    const dd a0 = dd_mul(m00, iz), a1 = dd_mul(m01, iz);
    const dd a2 = dd_neg(dd_mul(dd_add(dd_mul(m00, x), dd_mul(m01, y)), iz));
    const dd b0 = dd_mul(m10, iz), b1 = dd_mul(m11, iz);
    const dd b2 = dd_neg(dd_mul(dd_add(dd_mul(m10, x), dd_mul(m11, y)), iz));
    for (int k = 0; k < 3; ++k) {
      D[k] = dd_add(dd_add(dd_mul(a0, R[0 * 3 + k]), dd_mul(a1, R[1 * 3 + k])), dd_mul(a2, R[2 * 3 + k]));
      D[3 + k] = dd_add(dd_add(dd_mul(b0, R[0 * 3 + k]), dd_mul(b1, R[1 * 3 + k])), dd_mul(b2, R[2 * 3 + k]));
    }
  }
  for (int r = 0; r < 2; ++r) {
    const dd* d = D + 3 * r;
    J->jp[r * 6 + 0] = dd_add(dd_neg(dd_mul(d[1], pz)), dd_mul(d[2], py));
    J->jp[r * 6 + 1] = dd_sub(dd_mul(d[0], pz), dd_mul(d[2], px));
    J->jp[r * 6 + 2] = dd_add(dd_neg(dd_mul(d[0], py)), dd_mul(d[1], px));
    J->jp[r * 6 + 3] = d[0];
    J->jp[r * 6 + 4] = d[1];
    J->jp[r * 6 + 5] = d[2];
    J->jm[r * 3 + 0] = dd_neg(d[0]);
    J->jm[r * 3 + 1] = dd_neg(d[1]);
    J->jm[r * 3 + 2] = dd_neg(d[2]);
  }
}

// ---------------------------------------------------------------------------
// Pose tables: T_cw = T_wc^-1 in f64, published as float and float-float.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void pose_table(const double* T, float* pf, float* pd) {
  double qc[4] = {T[0], -T[1], -T[2], -T[3]};
  double R[9];
  rot_matrix(qc, R);
  double t[3];
  for (int i = 0; i < 3; ++i) t[i] = -(R[i * 3 + 0] * T[4] + R[i * 3 + 1] * T[5] + R[i * 3 + 2] * T[6]);
  for (int i = 0; i < 9; ++i) {
    pf[i] = __double2float_rn(R[i]);
    dd v = dd_from_double(R[i]);
    pd[2 * i] = v.hi;
    pd[2 * i + 1] = v.lo;
  }
  for (int i = 0; i < 3; ++i) {
    pf[9 + i] = __double2float_rn(t[i]);
    dd v = dd_from_double(t[i]);
    pd[18 + 2 * i] = v.hi;
    pd[18 + 2 * i + 1] = v.lo;
  }
}

// Pose tables of every camera.  With `begin` set (the first kernel of an LM
// iteration) thread 0 also opens the iteration: clears the step flags and
// maxima and the count of points queued for the float-float redo.
__device__ __forceinline__ void pose_tables_body(int nc, const double* __restrict__ poses, float* __restrict__ pose_f,
                              float* __restrict__ pose_dd, const Ctrl* ctrl, int respect_skip, Ctrl* begin,
                              int32_t* zero_count, int bid_, int nblk_) {
  if (respect_skip ? skipping(ctrl) : halted(ctrl)) return;
  if (begin && bid_ == 0 && threadIdx.x == 0) {
    begin->skip = 0;
    begin->accept = 0;
    begin->max_grad_bits = 0ull;
    begin->max_step_bits = 0ull;
    begin->alpha = 0.0;
    begin->pcg_done = 0;
    if (zero_count) *zero_count = 0;
  }
  int j = bid_ * blockDim.x + threadIdx.x;
  if (j >= nc) return;
  pose_table(poses + 7 * j, pose_f + 12 * j, pose_dd + 24 * j);
}
__global__ void k_pose_tables(int nc, const double* __restrict__ poses, float* __restrict__ pose_f,
                              float* __restrict__ pose_dd, const Ctrl* ctrl, int respect_skip, Ctrl* begin,
                              int32_t* zero_count) {
  pose_tables_body(nc, poses, pose_f, pose_dd, ctrl, respect_skip, begin, zero_count, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------------------
// Cost: calc_total_cost (crates/sophus_opt/src/nlls/cost/cost_fn.rs:403-433)
// in float-float; also publishes the FP32 residual for the next linearisation.
// ---------------------------------------------------------------------------
struct CostArgs {
  int64_t no;
  const double2* uv;
  const int32_t* opose;
  const int32_t* opt;
  const float* pose_dd;
  const double* points;
  float2* res_out;
  float2* res_lo_out;  // low parts of the residuals (float-float linearization), or null
  double* partials;
  dd fx, fy, cx, cy;    // intrinsics when intr is null (the allocation-free entry point)
  const double* intr;   // device intrinsics fx fy cx cy (current or trial), or null
  float huber;
  dd huber_dd;
  int respect_skip;
  // trial cost of an LM iteration: the last block to finish runs the decision
  Ctrl* decide;  // null: no decision
  const double* upd_part;
  int n_upd;
  Record* recs;
  Record* last;
  int n_extra;  // partials after the blocks' own (the pose priors' cost) that the decision adds
};

__device__ void decide_body(const double* cost_part, int n_cost, const double* upd_part, int n_upd, Ctrl* ctrl,
                            Record* recs, Record* last);

template <bool E>
__device__ __forceinline__ void cost_body(CostArgs a, const Ctrl* ctrl, int bid_, int nblk_) {
  const dd fx_ = a.intr ? dd_from_double(a.intr[0]) : a.fx, fy_ = a.intr ? dd_from_double(a.intr[1]) : a.fy;
  const dd cx_ = a.intr ? dd_from_double(a.intr[2]) : a.cx, cy_ = a.intr ? dd_from_double(a.intr[3]) : a.cy;
  // EUCM camera: the z = 1 projection is divided by norm
  const CamD camd = E ? cam_dd(a.intr) : CamD{};
  if (a.decide && !halted(ctrl) && skipping(ctrl)) {
    // no trial (gradient tolerance or a failed solve): decide at once
    if (bid_ == 0) decide_body(a.partials, 0, a.upd_part, a.n_upd, a.decide, a.recs, a.last);
    return;
  }
  if (a.respect_skip ? skipping(ctrl) : halted(ctrl)) return;
  dd acc = dd_make(0.0f, 0.0f);
  for (int64_t o = bid_ * static_cast<int64_t>(blockDim.x) + threadIdx.x; o < a.no;
       o += static_cast<int64_t>(nblk_) * blockDim.x) {
    const float* P = a.pose_dd + 24 * a.opose[o];
    const double* pw = a.points + 3 * a.opt[o];
    dd p0 = dd_from_double(pw[0]), p1 = dd_from_double(pw[1]), p2 = dd_from_double(pw[2]);
    dd xc[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      dd r0 = dd_make(P[2 * (i * 3 + 0)], P[2 * (i * 3 + 0) + 1]);
      dd r1 = dd_make(P[2 * (i * 3 + 1)], P[2 * (i * 3 + 1) + 1]);
      dd r2 = dd_make(P[2 * (i * 3 + 2)], P[2 * (i * 3 + 2) + 1]);
      dd tt = dd_make(P[18 + 2 * i], P[18 + 2 * i + 1]);
      xc[i] = dd_add(dd_add(dd_add(dd_mul(r0, p0), dd_mul(r1, p1)), dd_mul(r2, p2)), tt);
    }
    dd u = dd_div(xc[0], xc[2]);
    dd v = dd_div(xc[1], xc[2]);
    if (E) {
      const dd nrm = eucm_norm_dd(camd, u, v, nullptr, nullptr);
      u = dd_div(u, nrm);
      v = dd_div(v, nrm);
    }
    double2 z = a.uv[o];
    dd ru = dd_sub(dd_from_double(z.x), dd_add(dd_mul(u, fx_), cx_));
    dd rv = dd_sub(dd_from_double(z.y), dd_add(dd_mul(v, fy_), cy_));
    dd n2 = dd_add(dd_mul(ru, ru), dd_mul(rv, rv));
    dd c = n2;
    if (a.huber > 0.0f) {
      dd nrm = dd_sqrt(n2);
      if (!(nrm.hi <= a.huber || (nrm.hi == a.huber_dd.hi && nrm.lo <= a.huber_dd.lo))) {
        // 2 delta |r| - delta^2
        c = dd_sub(dd_mul(dd_add(a.huber_dd, a.huber_dd), nrm), dd_mul(a.huber_dd, a.huber_dd));
      }
    }
    acc = dd_add(acc, c);
    const float rh = ru.hi + ru.lo, vh = rv.hi + rv.lo;
    a.res_out[o] = make_float2(rh, vh);
    if (a.res_lo_out) a.res_lo_out[o] = make_float2((ru.hi - rh) + ru.lo, (rv.hi - vh) + rv.lo);
  }
  // block reduction (fixed tree)
  __shared__ float sh_hi[kCostThreads / 32], sh_lo[kCostThreads / 32];
  acc = dd_warp_sum(acc);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) { sh_hi[w] = acc.hi; sh_lo[w] = acc.lo; }
  __syncthreads();
  if (w == 0) {
    dd v = (lane < (int)(blockDim.x >> 5)) ? dd_make(sh_hi[lane], sh_lo[lane]) : dd_make(0.0f, 0.0f);
    v = dd_warp_sum(v);
    if (lane == 0) a.partials[bid_] = dd_to_double(v);
  }
  if (a.decide) {
    __shared__ bool s_last;
    __threadfence();
    if (threadIdx.x == 0) s_last = (atomicAdd(&a.decide->cost_ticket, 1) == static_cast<int>(nblk_) - 1);
    __syncthreads();
    if (s_last) {
      __threadfence();
      if (threadIdx.x == 0) a.decide->cost_ticket = 0;
      decide_body(a.partials, static_cast<int>(nblk_) + a.n_extra, a.upd_part, a.n_upd, a.decide, a.recs, a.last);
    }
  }
}
template <bool E>
__global__ void __launch_bounds__(kCostThreads) k_cost(CostArgs a, const Ctrl* ctrl) {
  cost_body<E>(a, ctrl, blockIdx.x, gridDim.x);
}

// Sum n double partials with one CTA (fixed tree, float-float).
__device__ double block_sum_partials(const double* part, int n) {
  __shared__ float sh_hi[32], sh_lo[32];
  dd acc = dd_make(0.0f, 0.0f);
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc = dd_add(acc, dd_from_double(part[i]));
  acc = dd_warp_sum(acc);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) { sh_hi[w] = acc.hi; sh_lo[w] = acc.lo; }
  __syncthreads();
  double out = 0.0;
  if (w == 0) {
    dd v = (lane < (int)(blockDim.x >> 5)) ? dd_make(sh_hi[lane], sh_lo[lane]) : dd_make(0.0f, 0.0f);
    v = dd_warp_sum(v);
    out = dd_to_double(v);
  }
  __syncthreads();
  return out;  // valid in warp 0
}

__global__ void k_init_merit(const double* part, int n, Ctrl* ctrl) {
  double s = block_sum_partials(part, n);
  if (threadIdx.x == 0) {
    ctrl->merit = s;
    ctrl->new_merit = s;
  }
}


// ---------------------------------------------------------------------------
// Landmark pass: one warp per marginalized point.  Builds the point block
// V_i = sum J_pt^T J_pt (+ nu * n_terms I), its gradient, the 3x3 Cholesky
// factor C and Z_g = W_g C^-T for every term g of the point, where
// W_g = J_pose^T J_pt.  Then the Schur complement contribution of the point
// is sum_{a,b} Z_a Z_b^T and its rhs contribution Z_a (C^-1 b_m)
// (compute_marg_block_contrib, crates/sophus_solver/src/ldlt/schur_ldlt.rs:82-135).
// FP32 per-lane sums, float-float across lanes, FP32 3x3 factor.
// ---------------------------------------------------------------------------
struct LinArgs {
  int32_t np;
  const int64_t* pt_g_begin;
  const int64_t* g_begin;
  const int32_t* g_pose;
  const int32_t* pose_fb;
  const int32_t* pt_mb;
  const double* cnt_m;
  const float* pose_f;
  const float* pose_dd;
  const double* points;
  const float2* res;
  const double* intr;  // device intrinsics fx fy cx cy
  float huber;
  float* zmat;
  float* cinv;   // 6 float-float per point: C^-1 (00 10 11 20 21 22)
  float* cvec;   // 3 float-float per point: C^-1 b_m
  double* bm;
  double nu_override;
  int use_override;
  int nu_ctrl;  // with use_override: take the damping from the control block (batched final pass)
  int* fail;
  // chunked pass (k_landmark_chunks)
  const int32_t* g_pt;
  const int32_t* chunk_pt;   // point chunks: nchunk + 1
  int32_t nchunk;
  int32_t* slow_list;        // ill-conditioned points found by the chunked pass
  int32_t* slow_count;
  // FP32 Cholesky of a point block is kept while each pivot keeps more than
  // this fraction of its diagonal entry; otherwise the block is rebuilt in
  // float-float
  float well_tol;
  // list mode of k_landmark: only the listed points, float-float path forced
  const int32_t* list;
  const int32_t* list_count;
  // float-float linearization: every point on the float-float path, residual
  // low parts and the Huber weight in float-float, Z kept as float-float pairs
  int force_dd;
  const float2* res_lo;
  float* zdd;  // kZD floats per term: Z (6x3) as (hi, lo) pairs
  dd huber_dd;
};

template <bool E>
__device__ __forceinline__ void landmark_body(LinArgs a, Ctrl* ctrl, int bid_, int nblk_) {
  const CamF cam_ = cam_f(a.intr);
  const CamD camd_ = cam_dd(a.intr);
  (void)cam_; (void)camd_;
  if (halted(ctrl)) return;
  __shared__ float red[8][9][33];
  // float-float path: the Jacobians of each lane's first term (a term with
  // one observation), kept from the sums for the Z pass; [value][lane]
  __shared__ float jcache[8][36][32];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int warps_per_block = blockDim.x >> 5;
  const double nu = (a.use_override && !a.nu_ctrl) ? a.nu_override : ctrl->nu;
  double warp_max = 0.0;  // max |neg_grad| of this warp's points
  const int64_t nitems = a.list ? static_cast<int64_t>(*a.list_count) : static_cast<int64_t>(a.np);
  for (int64_t item = static_cast<int64_t>(bid_) * warps_per_block + wib; item < nitems;
       item += static_cast<int64_t>(nblk_) * warps_per_block) {
    const int64_t i = a.list ? static_cast<int64_t>(a.list[item]) : item;
    const int mb = a.pt_mb[i];
    if (mb < 0) continue;  // constant point: no H_mm block
    const float px = __double2float_rn(a.points[3 * i + 0]);
    const float py = __double2float_rn(a.points[3 * i + 1]);
    const float pz = __double2float_rn(a.points[3 * i + 2]);
    const int64_t g0 = a.pt_g_begin[i], g1 = a.pt_g_begin[i + 1];
    dd Vd[6], b[3];
    bool well = false;
    float c00 = 0.f, c10 = 0.f, c20 = 0.f, c11 = 0.f, c21 = 0.f, t11 = 0.f, t22 = 0.f;  // FP32 Cholesky
    if (!a.force_dd) {  // the float-float linearization skips the FP32 pass
    float v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // V00 V01 V02 V11 V12 V22, g0 g1 g2
    for (int64_t g = g0 + lane; g < g1; g += 32) {
      const float* P = a.pose_f + 12 * a.g_pose[g];
      for (int64_t o = a.g_begin[g]; o < a.g_begin[g + 1]; ++o) {
        JacF J;
        jacobians_f<E>(P, px, py, pz, cam_, &J);
        float2 r = a.res[o];
        float w = huber_weight_f(a.huber, r.x, r.y);
        float r0 = w * r.x, r1 = w * r.y;
        const float* m = J.jm;
        v[0] += m[0] * m[0] + m[3] * m[3];
        v[1] += m[0] * m[1] + m[3] * m[4];
        v[2] += m[0] * m[2] + m[3] * m[5];
        v[3] += m[1] * m[1] + m[4] * m[4];
        v[4] += m[1] * m[2] + m[4] * m[5];
        v[5] += m[2] * m[2] + m[5] * m[5];
        v[6] += m[0] * r0 + m[3] * r1;
        v[7] += m[1] * r0 + m[4] * r1;
        v[8] += m[2] * r0 + m[5] * r1;
      }
    }
    dd tot = warp_transpose_sum<9>(v, red[wib]);
    // damping nu * (number of reduced terms) on the diagonal (entries 0, 3, 5)
    if (lane == 0 || lane == 3 || lane == 5) tot = dd_add(tot, dd_from_double(nu * a.cnt_m[mb]));
    if (lane >= 6) tot = dd_neg(tot);  // neg_grad b_m = -sum J^T r~
    // broadcast the 9 sums through shared memory (cheaper than shuffles here)
    if (lane < 9) {
      red[wib][0][lane] = tot.hi;
      red[wib][1][lane] = tot.lo;
    }
    __syncwarp();
#pragma unroll
    for (int k = 0; k < 6; ++k) Vd[k] = dd_make(red[wib][0][k], red[wib][1][k]);
#pragma unroll
    for (int k = 0; k < 3; ++k) b[k] = dd_make(red[wib][0][6 + k], red[wib][1][6 + k]);
    __syncwarp();
    if (lane == 0) {
      double* bp = a.bm + 3 * mb;
      bp[0] = dd_to_double(b[0]);
      bp[1] = dd_to_double(b[1]);
      bp[2] = dd_to_double(b[2]);
      warp_max = fmax(warp_max, fmax(fabs(bp[0]), fmax(fabs(bp[1]), fabs(bp[2]))));
    }
    // Cholesky V' = C C^T (V layout: 00 01 02 11 12 22).  FP32 when the point
    // block is well conditioned; float-float when a pivot lost more than three
    // digits to cancellation (e.g. a point seen once: its depth is held only by
    // the damping).  The branch is uniform across the warp.
    float V[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) V[k] = Vd[k].hi + Vd[k].lo;
    c00 = sqrtf(V[0]);
    c10 = V[1] / c00;
    c20 = V[2] / c00;
    t11 = V[3] - c10 * c10;
    c11 = sqrtf(t11);
    c21 = (V[4] - c20 * c10) / c11;
    t22 = V[5] - c20 * c20 - c21 * c21;
    well = !a.list && V[0] > 0.f && t11 > a.well_tol * V[3] && t22 > a.well_tol * V[5];
    }
    const dd pxd = dd_from_double(a.points[3 * i + 0]);
    const dd pyd = dd_from_double(a.points[3 * i + 1]);
    const dd pzd = dd_from_double(a.points[3 * i + 2]);
    if (!well) {
      // The FP32 Jacobians leave a rounding-level component of the gradient and
      // of W along the weakly constrained direction, which 1/(nu n) would
      // amplify: rebuild the whole point block in float-float.
      dd acc[9];
      for (int k = 0; k < 9; ++k) acc[k] = dd_make(0.f, 0.f);
      for (int64_t g = g0 + lane; g < g1; g += 32) {
        const float* Pd = a.pose_dd + 24 * a.g_pose[g];
        const bool keep = (g == g0 + lane) && (a.g_begin[g + 1] - a.g_begin[g] == 1);
        for (int64_t o = a.g_begin[g]; o < a.g_begin[g + 1]; ++o) {
          JacD J;
          jacobians_dd<E>(Pd, pxd, pyd, pzd, camd_, &J);
          if (keep) {
#pragma unroll
            for (int k = 0; k < 12; ++k) { jcache[wib][2 * k][lane] = J.jp[k].hi; jcache[wib][2 * k + 1][lane] = J.jp[k].lo; }
#pragma unroll
            for (int k = 0; k < 6; ++k) { jcache[wib][24 + 2 * k][lane] = J.jm[k].hi; jcache[wib][25 + 2 * k][lane] = J.jm[k].lo; }
          }
          float2 r = a.res[o];
          dd r0, r1;
          if (a.res_lo) {
            const float2 rl = a.res_lo[o];
            huber_weighted_dd(a.huber, a.huber_dd, dd_make(r.x, rl.x), dd_make(r.y, rl.y), &r0, &r1);
          } else {
            const float w = huber_weight_f(a.huber, r.x, r.y);
            r0 = dd_from_float(w * r.x);
            r1 = dd_from_float(w * r.y);
          }
          const dd* m = J.jm;
          acc[0] = dd_add(acc[0], dd_add(dd_mul(m[0], m[0]), dd_mul(m[3], m[3])));
          acc[1] = dd_add(acc[1], dd_add(dd_mul(m[0], m[1]), dd_mul(m[3], m[4])));
          acc[2] = dd_add(acc[2], dd_add(dd_mul(m[0], m[2]), dd_mul(m[3], m[5])));
          acc[3] = dd_add(acc[3], dd_add(dd_mul(m[1], m[1]), dd_mul(m[4], m[4])));
          acc[4] = dd_add(acc[4], dd_add(dd_mul(m[1], m[2]), dd_mul(m[4], m[5])));
          acc[5] = dd_add(acc[5], dd_add(dd_mul(m[2], m[2]), dd_mul(m[5], m[5])));
          acc[6] = dd_add(acc[6], dd_add(dd_mul(m[0], r0), dd_mul(m[3], r1)));
          acc[7] = dd_add(acc[7], dd_add(dd_mul(m[1], r0), dd_mul(m[4], r1)));
          acc[8] = dd_add(acc[8], dd_add(dd_mul(m[2], r0), dd_mul(m[5], r1)));
        }
      }
      for (int k = 0; k < 9; ++k) acc[k] = dd_warp_sum(acc[k]);
      const dd damp = dd_from_double(nu * a.cnt_m[mb]);
      for (int k = 0; k < 6; ++k) Vd[k] = acc[k];
      Vd[0] = dd_add(Vd[0], damp);
      Vd[3] = dd_add(Vd[3], damp);
      Vd[5] = dd_add(Vd[5], damp);
      for (int k = 0; k < 3; ++k) b[k] = dd_neg(acc[6 + k]);
      if (lane == 0) {
        double* bp = a.bm + 3 * mb;
        bp[0] = dd_to_double(b[0]);
        bp[1] = dd_to_double(b[1]);
        bp[2] = dd_to_double(b[2]);
        if (a.force_dd) warp_max = fmax(warp_max, fmax(fabs(bp[0]), fmax(fabs(bp[1]), fabs(bp[2]))));
      }
    }
    dd I[6];  // C^-1 (00 10 11 20 21 22)
    bool ok;
    if (well) {
      const float c22 = sqrtf(t22);
      const float i00 = 1.f / c00, i11 = 1.f / c11, i22 = 1.f / c22;
      const float i10 = -c10 * i00 * i11;
      const float i21 = -c21 * i11 * i22;
      const float i20 = -(c20 * i00 + c21 * i10) * i22;
      ok = isfinite(i00) && isfinite(i11) && isfinite(i22) && isfinite(i10) && isfinite(i20) && isfinite(i21);
      I[0] = dd_from_float(i00); I[1] = dd_from_float(i10); I[2] = dd_from_float(i11);
      I[3] = dd_from_float(i20); I[4] = dd_from_float(i21); I[5] = dd_from_float(i22);
    } else {
      ok = Vd[0].hi > 0.0f;
      dd e00 = dd_sqrt(Vd[0]);
      dd e10 = dd_div(Vd[1], e00), e20 = dd_div(Vd[2], e00);
      dd u11 = dd_sub(Vd[3], dd_mul(e10, e10));
      ok = ok && u11.hi > 0.0f;
      dd e11 = dd_sqrt(u11);
      dd e21 = dd_div(dd_sub(Vd[4], dd_mul(e20, e10)), e11);
      dd u22 = dd_sub(dd_sub(Vd[5], dd_mul(e20, e20)), dd_mul(e21, e21));
      ok = ok && u22.hi > 0.0f;
      dd e22 = dd_sqrt(u22);
      const dd one = dd_make(1.0f, 0.0f);
      I[0] = dd_div(one, e00);
      I[2] = dd_div(one, e11);
      I[5] = dd_div(one, e22);
      I[1] = dd_neg(dd_div(dd_mul(e10, I[0]), e11));
      I[4] = dd_neg(dd_div(dd_mul(e21, I[2]), e22));
      I[3] = dd_neg(dd_div(dd_add(dd_mul(e20, I[0]), dd_mul(e21, I[1])), e22));
      for (int k = 0; k < 6; ++k) ok = ok && isfinite(I[k].hi);
    }
    if (!ok) {
      if (lane == 0 && !a.use_override) atomicExch(a.fail, 1);
      continue;
    }
    if (lane == 0) {
      float* ci = a.cinv + 12 * mb;
#pragma unroll
      for (int k = 0; k < 6; ++k) { ci[2 * k] = I[k].hi; ci[2 * k + 1] = I[k].lo; }
      // c = C^-1 b in float-float
      dd cv0 = dd_mul(b[0], I[0]);
      dd cv1 = dd_add(dd_mul(b[0], I[1]), dd_mul(b[1], I[2]));
      dd cv2 = dd_add(dd_add(dd_mul(b[0], I[3]), dd_mul(b[1], I[4])), dd_mul(b[2], I[5]));
      float* cvp = a.cvec + 6 * mb;
      cvp[0] = cv0.hi; cvp[1] = cv0.lo; cvp[2] = cv1.hi; cvp[3] = cv1.lo; cvp[4] = cv2.hi; cvp[5] = cv2.lo;
    }
    const float i00 = I[0].hi, i10 = I[1].hi, i11 = I[2].hi, i20 = I[3].hi, i21 = I[4].hi, i22 = I[5].hi;
    if (a.use_override) continue;  // final Hessian pass: no Schur data
    // pass 2: Z_g = W_g C^-T for terms with a free pose
    for (int64_t g = g0 + lane; g < g1; g += 32) {
      const int pj = a.g_pose[g];
      if (a.pose_fb[pj] < 0) continue;
      const float* P = a.pose_f + 12 * pj;
      float W[18];
      float Z[20];
      if (well) {
#pragma unroll
        for (int k = 0; k < 18; ++k) W[k] = 0.f;
        for (int64_t o = a.g_begin[g]; o < a.g_begin[g + 1]; ++o) {
          JacF J;
          jacobians_f<E>(P, px, py, pz, cam_, &J);
#pragma unroll
          for (int r = 0; r < 6; ++r)
#pragma unroll
            for (int q = 0; q < 3; ++q) W[r * 3 + q] += J.jp[r] * J.jm[q] + J.jp[6 + r] * J.jm[3 + q];
        }
        // Z[r][t] = sum_{s<=t} W[r][s] * Cinv[t][s]
#pragma unroll
        for (int r = 0; r < 6; ++r) {
          Z[r * 3 + 0] = W[r * 3 + 0] * i00;
          Z[r * 3 + 1] = W[r * 3 + 0] * i10 + W[r * 3 + 1] * i11;
          Z[r * 3 + 2] = W[r * 3 + 0] * i20 + W[r * 3 + 1] * i21 + W[r * 3 + 2] * i22;
        }
      } else {
        // W and Z in float-float: the large entries of C^-1 cancel against W
        dd Wd[18];
        for (int k = 0; k < 18; ++k) Wd[k] = dd_make(0.f, 0.f);
        const float* Pd = a.pose_dd + 24 * pj;
        const bool kept = (g == g0 + lane) && (a.g_begin[g + 1] - a.g_begin[g] == 1);
        for (int64_t o = a.g_begin[g]; o < a.g_begin[g + 1]; ++o) {
          JacD J;
          if (kept) {  // the same Jacobians as in the sums above
#pragma unroll
            for (int k = 0; k < 12; ++k) J.jp[k] = dd_make(jcache[wib][2 * k][lane], jcache[wib][2 * k + 1][lane]);
#pragma unroll
            for (int k = 0; k < 6; ++k) J.jm[k] = dd_make(jcache[wib][24 + 2 * k][lane], jcache[wib][25 + 2 * k][lane]);
          } else {
            jacobians_dd<E>(Pd, pxd, pyd, pzd, camd_, &J);
          }
          for (int r = 0; r < 6; ++r)
            for (int q = 0; q < 3; ++q)
              Wd[r * 3 + q] = dd_add(Wd[r * 3 + q], dd_add(dd_mul(J.jp[r], J.jm[q]), dd_mul(J.jp[6 + r], J.jm[3 + q])));
        }
        float* zd = a.zdd ? a.zdd + kZD * g : nullptr;
        for (int r = 0; r < 6; ++r) {
          dd z0 = dd_mul(I[0], Wd[r * 3 + 0]);
          dd z1 = dd_add(dd_mul(I[1], Wd[r * 3 + 0]), dd_mul(I[2], Wd[r * 3 + 1]));
          dd z2 = dd_add(dd_add(dd_mul(I[3], Wd[r * 3 + 0]), dd_mul(I[4], Wd[r * 3 + 1])), dd_mul(I[5], Wd[r * 3 + 2]));
          Z[r * 3 + 0] = z0.hi + z0.lo;
          Z[r * 3 + 1] = z1.hi + z1.lo;
          Z[r * 3 + 2] = z2.hi + z2.lo;
          if (zd) {
            zd[6 * r + 0] = z0.hi; zd[6 * r + 1] = z0.lo;
            zd[6 * r + 2] = z1.hi; zd[6 * r + 3] = z1.lo;
            zd[6 * r + 4] = z2.hi; zd[6 * r + 5] = z2.lo;
          }
        }
      }
      // padding entry 18 flags a term whose float-float Z is in zdd (the
      // back-substitution and the reduced rhs of such a point read it there)
      Z[18] = (!well && a.zdd) ? 1.f : 0.f;
      Z[19] = 0.f;
      float4* dst = reinterpret_cast<float4*>(a.zmat + kZS * g);
#pragma unroll
      for (int q = 0; q < 5; ++q) dst[q] = make_float4(Z[4 * q], Z[4 * q + 1], Z[4 * q + 2], Z[4 * q + 3]);
    }
  }
  __shared__ double s_max[8];
  if (lane == 0) s_max[wib] = warp_max;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int q = 0; q < warps_per_block; ++q) m = fmax(m, s_max[q]);
    atomic_max_nonneg(&ctrl->max_grad_bits, m);
  }
}
template <bool E>
__global__ void __launch_bounds__(256, 2) k_landmark(LinArgs a, Ctrl* ctrl) {
  landmark_body<E>(a, ctrl, blockIdx.x, gridDim.x);
}

// Landmark pass by chunks of consecutive points (<= kLmkTerms terms): one
// thread per term for the Jacobian products, one thread per point for the
// float-float sums, the damping and the 3x3 Cholesky, then one thread per
// term for Z = W C^-T.  Same arithmetic as k_landmark's well-conditioned
// path except that each term's FP32 contribution is summed in float-float
// directly.  A point whose Cholesky loses more than three digits goes to
// slow_list and is redone by k_landmark (list mode, float-float path).
constexpr int kLmkTerms = 256;

template <bool E>
__device__ __forceinline__ void landmark_chunks_body(LinArgs a, Ctrl* ctrl, int bid_, int nblk_) {
  const CamF cam_ = cam_f(a.intr);
  const CamD camd_ = cam_dd(a.intr);
  (void)cam_; (void)camd_;
  if (halted(ctrl)) return;
  extern __shared__ float lsm[];        // [cap][9] term contributions
  __shared__ float sci[kLmkTerms][6];   // C^-1 per point of the chunk (FP32)
  __shared__ float2 ssum[kLmkTerms][9]; // per point: the 9 sums over its terms (float-float)
  __shared__ unsigned char sok[kLmkTerms];
  __shared__ double smax[8];
  const int tid = threadIdx.x;
  const double nu = ctrl->nu;
  double tmax = 0.0;
  for (int c = bid_; c < a.nchunk; c += nblk_) {
    const int p0 = a.chunk_pt[c], p1 = a.chunk_pt[c + 1];
    const int64_t t0 = a.pt_g_begin[p0];
    const int nt = static_cast<int>(a.pt_g_begin[p1] - t0);
    // pass A: per-term V and J_m^T r~ contributions
    for (int t = tid; t < nt; t += blockDim.x) {
      const int64_t g = t0 + t;
      const int i = a.g_pt[g];
      const float px = __double2float_rn(a.points[3 * i + 0]);
      const float py = __double2float_rn(a.points[3 * i + 1]);
      const float pz = __double2float_rn(a.points[3 * i + 2]);
      const float* P = a.pose_f + 12 * a.g_pose[g];
      float v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      for (int64_t o = a.g_begin[g]; o < a.g_begin[g + 1]; ++o) {
        JacF J;
        jacobians_f<E>(P, px, py, pz, cam_, &J);
        const float2 r = a.res[o];
        const float w = huber_weight_f(a.huber, r.x, r.y);
        const float r0 = w * r.x, r1 = w * r.y;
        const float* m = J.jm;
        v[0] += m[0] * m[0] + m[3] * m[3];
        v[1] += m[0] * m[1] + m[3] * m[4];
        v[2] += m[0] * m[2] + m[3] * m[5];
        v[3] += m[1] * m[1] + m[4] * m[4];
        v[4] += m[1] * m[2] + m[4] * m[5];
        v[5] += m[2] * m[2] + m[5] * m[5];
        v[6] += m[0] * r0 + m[3] * r1;
        v[7] += m[1] * r0 + m[4] * r1;
        v[8] += m[2] * r0 + m[5] * r1;
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) lsm[9 * t + k] = v[k];
    }
    __syncthreads();
    // pass B1: every sum of every point, a thread per (point, value), over the
    // point's terms in order (points of long tracks no longer serialise a
    // single thread over all nine sums)
    for (int e = tid; e < 9 * (p1 - p0); e += blockDim.x) {
      const int q = e / 9, k = e - 9 * q;
      const int tb = static_cast<int>(a.pt_g_begin[p0 + q] - t0), te = static_cast<int>(a.pt_g_begin[p0 + q + 1] - t0);
      dd sacc = dd_make(0.f, 0.f);
      for (int t = tb; t < te; ++t) sacc = dd_add_f(sacc, lsm[9 * t + k]);
      ssum[q][k] = make_float2(sacc.hi, sacc.lo);
    }
    __syncthreads();
    // pass B2: per point
    for (int q = tid; q < p1 - p0; q += blockDim.x) {
      const int i = p0 + q;
      const int mb = a.pt_mb[i];
      sok[q] = 0;
      if (mb < 0) continue;
      dd acc[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) acc[k] = dd_make(ssum[q][k].x, ssum[q][k].y);
      const dd damp = dd_from_double(nu * a.cnt_m[mb]);
      acc[0] = dd_add(acc[0], damp);
      acc[3] = dd_add(acc[3], damp);
      acc[5] = dd_add(acc[5], damp);
      dd b[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) b[k] = dd_neg(acc[6 + k]);
      double* bp = a.bm + 3 * mb;
      bp[0] = dd_to_double(b[0]);
      bp[1] = dd_to_double(b[1]);
      bp[2] = dd_to_double(b[2]);
      tmax = fmax(tmax, fmax(fabs(bp[0]), fmax(fabs(bp[1]), fabs(bp[2]))));
      float V[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) V[k] = acc[k].hi + acc[k].lo;
      const float c00 = sqrtf(V[0]);
      const float c10 = V[1] / c00, c20 = V[2] / c00;
      const float t11 = V[3] - c10 * c10;
      const float c11 = sqrtf(t11);
      const float c21 = (V[4] - c20 * c10) / c11;
      const float t22 = V[5] - c20 * c20 - c21 * c21;
      const bool well = V[0] > 0.f && t11 > a.well_tol * V[3] && t22 > a.well_tol * V[5];
      if (!well) {
        a.slow_list[atomicAdd(a.slow_count, 1)] = i;
        continue;
      }
      const float c22 = sqrtf(t22);
      const float i00 = 1.f / c00, i11 = 1.f / c11, i22 = 1.f / c22;
      const float i10 = -c10 * i00 * i11;
      const float i21 = -c21 * i11 * i22;
      const float i20 = -(c20 * i00 + c21 * i10) * i22;
      const bool ok = isfinite(i00) && isfinite(i11) && isfinite(i22) && isfinite(i10) && isfinite(i20) && isfinite(i21);
      if (!ok) {
        atomicExch(a.fail, 1);
        continue;
      }
      const dd I[6] = {dd_from_float(i00), dd_from_float(i10), dd_from_float(i11),
                       dd_from_float(i20), dd_from_float(i21), dd_from_float(i22)};
      float* ci = a.cinv + 12 * mb;
#pragma unroll
      for (int k = 0; k < 6; ++k) { ci[2 * k] = I[k].hi; ci[2 * k + 1] = I[k].lo; }
      const dd cv0 = dd_mul(b[0], I[0]);
      const dd cv1 = dd_add(dd_mul(b[0], I[1]), dd_mul(b[1], I[2]));
      const dd cv2 = dd_add(dd_add(dd_mul(b[0], I[3]), dd_mul(b[1], I[4])), dd_mul(b[2], I[5]));
      float* cvp = a.cvec + 6 * mb;
      cvp[0] = cv0.hi; cvp[1] = cv0.lo; cvp[2] = cv1.hi; cvp[3] = cv1.lo; cvp[4] = cv2.hi; cvp[5] = cv2.lo;
      sci[q][0] = i00; sci[q][1] = i10; sci[q][2] = i11; sci[q][3] = i20; sci[q][4] = i21; sci[q][5] = i22;
      sok[q] = 1;
    }
    __syncthreads();
    // pass C: Z_g = W_g C^-T for terms with a free pose
    for (int t = tid; t < nt; t += blockDim.x) {
      const int64_t g = t0 + t;
      const int i = a.g_pt[g];
      const int q = i - p0;
      if (!sok[q]) continue;
      const int pj = a.g_pose[g];
      if (a.pose_fb[pj] < 0) continue;
      const float px = __double2float_rn(a.points[3 * i + 0]);
      const float py = __double2float_rn(a.points[3 * i + 1]);
      const float pz = __double2float_rn(a.points[3 * i + 2]);
      const float* P = a.pose_f + 12 * pj;
      float W[18];
#pragma unroll
      for (int k = 0; k < 18; ++k) W[k] = 0.f;
      for (int64_t o = a.g_begin[g]; o < a.g_begin[g + 1]; ++o) {
        JacF J;
        jacobians_f<E>(P, px, py, pz, cam_, &J);
#pragma unroll
        for (int r = 0; r < 6; ++r)
#pragma unroll
          for (int u = 0; u < 3; ++u) W[r * 3 + u] += J.jp[r] * J.jm[u] + J.jp[6 + r] * J.jm[3 + u];
      }
      const float i00 = sci[q][0], i10 = sci[q][1], i11 = sci[q][2], i20 = sci[q][3], i21 = sci[q][4], i22 = sci[q][5];
      float Z[20];
#pragma unroll
      for (int r = 0; r < 6; ++r) {
        Z[r * 3 + 0] = W[r * 3 + 0] * i00;
        Z[r * 3 + 1] = W[r * 3 + 0] * i10 + W[r * 3 + 1] * i11;
        Z[r * 3 + 2] = W[r * 3 + 0] * i20 + W[r * 3 + 1] * i21 + W[r * 3 + 2] * i22;
      }
      Z[18] = 0.f;
      Z[19] = 0.f;
      float4* dst = reinterpret_cast<float4*>(a.zmat + kZS * g);
#pragma unroll
      for (int u = 0; u < 5; ++u) dst[u] = make_float4(Z[4 * u], Z[4 * u + 1], Z[4 * u + 2], Z[4 * u + 3]);
    }
    __syncthreads();
  }
  // max |neg_grad| over the block
  for (int off = 16; off > 0; off >>= 1) tmax = fmax(tmax, __shfl_xor_sync(0xffffffffu, tmax, off));
  if ((tid & 31) == 0) smax[tid >> 5] = tmax;
  __syncthreads();
  if (tid == 0) {
    double m = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) m = fmax(m, smax[q]);
    atomic_max_nonneg(&ctrl->max_grad_bits, m);
  }
}
template <bool E>
__global__ void __launch_bounds__(256) k_landmark_chunks(LinArgs a, Ctrl* ctrl) {
  landmark_chunks_body<E>(a, ctrl, blockIdx.x, gridDim.x);
}

// The float-float landmark pass of loop-shaped problems by chunks of
// consecutive points (<= kLmkTerms terms): every lane busy on a term (a
// point's track is ~8 terms there, so a warp per point left 3/4 of its lanes
// idle).  Pass A, a thread per term: float-float Jacobians (kept in shared
// memory), Huber-weighted residual, the term's V and J_m^T r~ contributions.
// Pass B, a thread per point: the sums in term order, damping, float-float
// Cholesky and C^-1, C^-1 b.  Pass C, a thread per term: W = sum J_p^T J_m
// over the term's observations and Z = W C^-T in float-float.  The same
// arithmetic as k_landmark's float-float path; only the order of the sums
// over a point's terms differs (sequential here, a lane tree there).
constexpr int kLmkDDTermFloats = 18 + 36;  // 9 float-float sums + the Jacobians (18 float-float)

template <bool E>
__global__ void __launch_bounds__(256) k_landmark_chunks_dd(LinArgs a, Ctrl* ctrl) {
  const CamF cam_ = cam_f(a.intr);
  const CamD camd_ = cam_dd(a.intr);
  (void)cam_; (void)camd_;
  if (halted(ctrl)) return;
  extern __shared__ float lsd[];               // [cap][kLmkDDTermFloats]
  __shared__ float sci[kLmkTerms][12];         // C^-1 of each point of the chunk (float-float)
  __shared__ float2 ssum[kLmkTerms][9];        // per point: the 9 sums over its terms
  __shared__ unsigned char sok[kLmkTerms];
  __shared__ double smax[8];
  const int tid = threadIdx.x;
  const double nu = ctrl->nu;
  double tmax = 0.0;
  for (int c = blockIdx.x; c < a.nchunk; c += gridDim.x) {
    const int p0 = a.chunk_pt[c], p1 = a.chunk_pt[c + 1];
    const int64_t t0 = a.pt_g_begin[p0];
    const int nt = static_cast<int>(a.pt_g_begin[p1] - t0);
    // pass A
    for (int t = tid; t < nt; t += blockDim.x) {
      const int64_t g = t0 + t;
      const int i = a.g_pt[g];
      const dd px = dd_from_double(a.points[3 * i + 0]);
      const dd py = dd_from_double(a.points[3 * i + 1]);
      const dd pz = dd_from_double(a.points[3 * i + 2]);
      JacD J;
      jacobians_dd<E>(a.pose_dd + 24 * a.g_pose[g], px, py, pz, camd_, &J);
      float* ts = lsd + static_cast<int64_t>(t) * kLmkDDTermFloats;
#pragma unroll
      for (int k = 0; k < 12; ++k) { ts[18 + 2 * k] = J.jp[k].hi; ts[19 + 2 * k] = J.jp[k].lo; }
#pragma unroll
      for (int k = 0; k < 6; ++k) { ts[42 + 2 * k] = J.jm[k].hi; ts[43 + 2 * k] = J.jm[k].lo; }
      dd acc[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) acc[k] = dd_make(0.f, 0.f);
      const dd* m = J.jm;
      for (int64_t o = a.g_begin[g]; o < a.g_begin[g + 1]; ++o) {
        const float2 r = a.res[o], rl = a.res_lo[o];
        dd r0, r1;
        huber_weighted_dd(a.huber, a.huber_dd, dd_make(r.x, rl.x), dd_make(r.y, rl.y), &r0, &r1);
        acc[0] = dd_add(acc[0], dd_add(dd_mul(m[0], m[0]), dd_mul(m[3], m[3])));
        acc[1] = dd_add(acc[1], dd_add(dd_mul(m[0], m[1]), dd_mul(m[3], m[4])));
        acc[2] = dd_add(acc[2], dd_add(dd_mul(m[0], m[2]), dd_mul(m[3], m[5])));
        acc[3] = dd_add(acc[3], dd_add(dd_mul(m[1], m[1]), dd_mul(m[4], m[4])));
        acc[4] = dd_add(acc[4], dd_add(dd_mul(m[1], m[2]), dd_mul(m[4], m[5])));
        acc[5] = dd_add(acc[5], dd_add(dd_mul(m[2], m[2]), dd_mul(m[5], m[5])));
        acc[6] = dd_add(acc[6], dd_add(dd_mul(m[0], r0), dd_mul(m[3], r1)));
        acc[7] = dd_add(acc[7], dd_add(dd_mul(m[1], r0), dd_mul(m[4], r1)));
        acc[8] = dd_add(acc[8], dd_add(dd_mul(m[2], r0), dd_mul(m[5], r1)));
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) { ts[2 * k] = acc[k].hi; ts[2 * k + 1] = acc[k].lo; }
    }
    __syncthreads();
    // pass B1: a thread per (point, sum), over the point's terms in order
    for (int e = tid; e < 9 * (p1 - p0); e += blockDim.x) {
      const int q = e / 9, k = e - 9 * q;
      const int tb = static_cast<int>(a.pt_g_begin[p0 + q] - t0), te = static_cast<int>(a.pt_g_begin[p0 + q + 1] - t0);
      dd sacc = dd_make(0.f, 0.f);
      for (int t = tb; t < te; ++t) {
        const float* ts = lsd + static_cast<int64_t>(t) * kLmkDDTermFloats;
        sacc = dd_add(sacc, dd_make(ts[2 * k], ts[2 * k + 1]));
      }
      ssum[q][k] = make_float2(sacc.hi, sacc.lo);
    }
    __syncthreads();
    // pass B2: per point
    for (int q = tid; q < p1 - p0; q += blockDim.x) {
      const int i = p0 + q;
      const int mb = a.pt_mb[i];
      sok[q] = 0;
      if (mb < 0) continue;
      dd acc[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) acc[k] = dd_make(ssum[q][k].x, ssum[q][k].y);
      const dd damp = dd_from_double(nu * a.cnt_m[mb]);
      dd Vd[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) Vd[k] = acc[k];
      Vd[0] = dd_add(Vd[0], damp);
      Vd[3] = dd_add(Vd[3], damp);
      Vd[5] = dd_add(Vd[5], damp);
      dd b[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) b[k] = dd_neg(acc[6 + k]);
      double* bp = a.bm + 3 * mb;
      bp[0] = dd_to_double(b[0]);
      bp[1] = dd_to_double(b[1]);
      bp[2] = dd_to_double(b[2]);
      tmax = fmax(tmax, fmax(fabs(bp[0]), fmax(fabs(bp[1]), fabs(bp[2]))));
      bool ok = Vd[0].hi > 0.0f;
      const dd e00 = dd_sqrt(Vd[0]);
      const dd e10 = dd_div(Vd[1], e00), e20 = dd_div(Vd[2], e00);
      const dd u11 = dd_sub(Vd[3], dd_mul(e10, e10));
      ok = ok && u11.hi > 0.0f;
      const dd e11 = dd_sqrt(u11);
      const dd e21 = dd_div(dd_sub(Vd[4], dd_mul(e20, e10)), e11);
      const dd u22 = dd_sub(dd_sub(Vd[5], dd_mul(e20, e20)), dd_mul(e21, e21));
      ok = ok && u22.hi > 0.0f;
      const dd e22 = dd_sqrt(u22);
      const dd one = dd_make(1.0f, 0.0f);
      dd I[6];
      I[0] = dd_div(one, e00);
      I[2] = dd_div(one, e11);
      I[5] = dd_div(one, e22);
      I[1] = dd_neg(dd_div(dd_mul(e10, I[0]), e11));
      I[4] = dd_neg(dd_div(dd_mul(e21, I[2]), e22));
      I[3] = dd_neg(dd_div(dd_add(dd_mul(e20, I[0]), dd_mul(e21, I[1])), e22));
#pragma unroll
      for (int k = 0; k < 6; ++k) ok = ok && isfinite(I[k].hi);
      if (!ok) {
        atomicExch(a.fail, 1);
        continue;
      }
      float* ci = a.cinv + 12 * mb;
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        ci[2 * k] = I[k].hi;
        ci[2 * k + 1] = I[k].lo;
        sci[q][2 * k] = I[k].hi;
        sci[q][2 * k + 1] = I[k].lo;
      }
      const dd cv0 = dd_mul(b[0], I[0]);
      const dd cv1 = dd_add(dd_mul(b[0], I[1]), dd_mul(b[1], I[2]));
      const dd cv2 = dd_add(dd_add(dd_mul(b[0], I[3]), dd_mul(b[1], I[4])), dd_mul(b[2], I[5]));
      float* cvp = a.cvec + 6 * mb;
      cvp[0] = cv0.hi; cvp[1] = cv0.lo; cvp[2] = cv1.hi; cvp[3] = cv1.lo; cvp[4] = cv2.hi; cvp[5] = cv2.lo;
      sok[q] = 1;
    }
    __syncthreads();
    // pass C
    for (int t = tid; t < nt; t += blockDim.x) {
      const int64_t g = t0 + t;
      const int i = a.g_pt[g];
      const int q = i - p0;
      if (!sok[q]) continue;
      const int pj = a.g_pose[g];
      if (a.pose_fb[pj] < 0) continue;
      const float* ts = lsd + static_cast<int64_t>(t) * kLmkDDTermFloats;
      dd jp[12], jm[6];
#pragma unroll
      for (int k = 0; k < 12; ++k) jp[k] = dd_make(ts[18 + 2 * k], ts[19 + 2 * k]);
#pragma unroll
      for (int k = 0; k < 6; ++k) jm[k] = dd_make(ts[42 + 2 * k], ts[43 + 2 * k]);
      dd Wd[18];
#pragma unroll
      for (int k = 0; k < 18; ++k) Wd[k] = dd_make(0.f, 0.f);
      for (int64_t o = a.g_begin[g]; o < a.g_begin[g + 1]; ++o) {
#pragma unroll
        for (int r = 0; r < 6; ++r)
#pragma unroll
          for (int u = 0; u < 3; ++u)
            Wd[r * 3 + u] = dd_add(Wd[r * 3 + u], dd_add(dd_mul(jp[r], jm[u]), dd_mul(jp[6 + r], jm[3 + u])));
      }
      dd I[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) I[k] = dd_make(sci[q][2 * k], sci[q][2 * k + 1]);
      float Z[20];
      float* zd = a.zdd + kZD * g;
#pragma unroll
      for (int r = 0; r < 6; ++r) {
        const dd z0 = dd_mul(I[0], Wd[r * 3 + 0]);
        const dd z1 = dd_add(dd_mul(I[1], Wd[r * 3 + 0]), dd_mul(I[2], Wd[r * 3 + 1]));
        const dd z2 = dd_add(dd_add(dd_mul(I[3], Wd[r * 3 + 0]), dd_mul(I[4], Wd[r * 3 + 1])), dd_mul(I[5], Wd[r * 3 + 2]));
        Z[r * 3 + 0] = z0.hi + z0.lo;
        Z[r * 3 + 1] = z1.hi + z1.lo;
        Z[r * 3 + 2] = z2.hi + z2.lo;
        zd[6 * r + 0] = z0.hi; zd[6 * r + 1] = z0.lo;
        zd[6 * r + 2] = z1.hi; zd[6 * r + 3] = z1.lo;
        zd[6 * r + 4] = z2.hi; zd[6 * r + 5] = z2.lo;
      }
      Z[18] = 1.f;  // float-float Z in zdd
      Z[19] = 0.f;
      float4* dst = reinterpret_cast<float4*>(a.zmat + kZS * g);
#pragma unroll
      for (int u = 0; u < 5; ++u) dst[u] = make_float4(Z[4 * u], Z[4 * u + 1], Z[4 * u + 2], Z[4 * u + 3]);
    }
    __syncthreads();
  }
  for (int off = 16; off > 0; off >>= 1) tmax = fmax(tmax, __shfl_xor_sync(0xffffffffu, tmax, off));
  if ((tid & 31) == 0) smax[tid >> 5] = tmax;
  __syncthreads();
  if (tid == 0) {
    double m = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) m = fmax(m, smax[q]);
    atomic_max_nonneg(&ctrl->max_grad_bits, m);
  }
}

// ---------------------------------------------------------------------------
// Camera pass: one CTA per tile of terms of one free pose.  Accumulates
// U_j = sum J_pose^T J_pose (21 upper entries), g_j = sum J_pose^T r~ and the
// reduced-rhs term sum Z_g (C^-1 b_m).  FP32 warp sums, float-float across
// warps; the Z c products in float-float.
// ---------------------------------------------------------------------------
constexpr int kTileThreads = 256;
constexpr int kTileVals = 33;

struct CamArgs {
  const int32_t* tile_fb;
  const int64_t* tile_begin;
  const int64_t* tile_end;
  const int64_t* cam_g;
  const int64_t* g_begin;
  const int32_t* g_pt;
  const int32_t* fb_pose;
  const int32_t* pt_mb;
  const float* pose_f;
  const double* points;
  const float2* res;
  const float* zmat;
  const float* cvec;
  const double* intr;  // device intrinsics fx fy cx cy
  float huber;
  double* tile_part;
  int with_schur;
  // float-float linearization
  const float* pose_dd;
  const float2* res_lo;
  const float* zdd;
  dd huber_dd;
};

template <bool E>
__device__ __forceinline__ void camera_tiles_body(CamArgs a, const Ctrl* ctrl, int bid_, int nblk_) {
  const CamF cam_ = cam_f(a.intr);
  const CamD camd_ = cam_dd(a.intr);
  (void)cam_; (void)camd_;
  if (halted(ctrl)) return;
  const int tile = bid_;
  const int fb = a.tile_fb[tile];
  const float* P = a.pose_f + 12 * a.fb_pose[fb];
  float u[27];
#pragma unroll
  for (int k = 0; k < 27; ++k) u[k] = 0.f;
  float zc[12];  // 6 float-float values as (hi, lo)
#pragma unroll
  for (int k = 0; k < 12; ++k) zc[k] = 0.f;
  const int64_t e = a.tile_begin[tile] + threadIdx.x;
  if (e < a.tile_end[tile]) {
    const int64_t g = a.cam_g[e];
    const int pi = a.g_pt[g];
    const float px = __double2float_rn(a.points[3 * pi + 0]);
    const float py = __double2float_rn(a.points[3 * pi + 1]);
    const float pz = __double2float_rn(a.points[3 * pi + 2]);
    for (int64_t o = a.g_begin[g]; o < a.g_begin[g + 1]; ++o) {
      JacF J;
      jacobians_f<E>(P, px, py, pz, cam_, &J);
      float2 r = a.res[o];
      float w = huber_weight_f(a.huber, r.x, r.y);
      float r0 = w * r.x, r1 = w * r.y;
      int k = 0;
#pragma unroll
      for (int p = 0; p < 6; ++p) {
#pragma unroll
        for (int q = p; q < 6; ++q) u[k++] += J.jp[p] * J.jp[q] + J.jp[6 + p] * J.jp[6 + q];
        u[21 + p] += J.jp[p] * r0 + J.jp[6 + p] * r1;
      }
    }
    const int mb = a.pt_mb[pi];
    if (a.with_schur && mb >= 0) {
      const float4* Z4 = reinterpret_cast<const float4*>(a.zmat + kZS * g);
      float Z[20];
#pragma unroll
      for (int q = 0; q < 5; ++q) {
        float4 z = Z4[q];
        Z[4 * q] = z.x; Z[4 * q + 1] = z.y; Z[4 * q + 2] = z.z; Z[4 * q + 3] = z.w;
      }
      const float* cv = a.cvec + 6 * mb;
      dd c0 = dd_make(cv[0], cv[1]), c1 = dd_make(cv[2], cv[3]), c2 = dd_make(cv[4], cv[5]);
      if (Z[18] != 0.f && a.zdd) {
        // a point rebuilt in float-float: its float-float Z
        const float* zd = a.zdd + kZD * g;
#pragma unroll
        for (int r = 0; r < 6; ++r) {
          dd t = dd_add(dd_add(dd_mul(c0, dd_make(zd[6 * r + 0], zd[6 * r + 1])),
                               dd_mul(c1, dd_make(zd[6 * r + 2], zd[6 * r + 3]))),
                        dd_mul(c2, dd_make(zd[6 * r + 4], zd[6 * r + 5])));
          zc[2 * r] = t.hi;
          zc[2 * r + 1] = t.lo;
        }
      } else {
#pragma unroll
        for (int r = 0; r < 6; ++r) {
          dd t = dd_add(dd_add(dd_mul_f(c0, Z[r * 3 + 0]), dd_mul_f(c1, Z[r * 3 + 1])), dd_mul_f(c2, Z[r * 3 + 2]));
          zc[2 * r] = t.hi;
          zc[2 * r + 1] = t.lo;
        }
      }
    }
  }
  __shared__ float sh_hi[kTileVals][kTileThreads / 32];
  __shared__ float sh_lo[kTileVals][kTileThreads / 32];
  __shared__ float zred[kTileThreads / 32][27][33];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  // U and g: FP32 sums inside the warp, transposed through shared memory
#pragma unroll
  for (int k = 0; k < 27; ++k) zred[w][k][lane] = u[k];
  __syncwarp();
  if (lane < 27) {
    float v = 0.f;
#pragma unroll 8
    for (int l = 0; l < 32; ++l) v += zred[w][lane][l];
    sh_hi[lane][w] = v;
    sh_lo[lane][w] = 0.f;
  }
  __syncwarp();
  // Z c: float-float across the warp (values 2r = hi, 2r+1 = lo)
#pragma unroll
  for (int k = 0; k < 12; ++k) zred[w][k][lane] = zc[k];
  __syncwarp();
  if (lane < 6) {
    dd acc = dd_make(0.f, 0.f);
    for (int l = 0; l < 32; ++l) acc = dd_add(acc, dd_make(zred[w][2 * lane][l], zred[w][2 * lane + 1][l]));
    sh_hi[27 + lane][w] = acc.hi;
    sh_lo[27 + lane][w] = acc.lo;
  }
  __syncthreads();
  if (threadIdx.x < kTileVals) {
    const int k = threadIdx.x;
    dd v = dd_make(0.f, 0.f);
    for (int q = 0; q < kTileThreads / 32; ++q) v = dd_add(v, dd_make(sh_hi[k][q], sh_lo[k][q]));
    a.tile_part[static_cast<int64_t>(tile) * kTileVals + k] = dd_to_double(v);
  }
}
template <bool E>
__global__ void __launch_bounds__(kTileThreads) k_camera_tiles(CamArgs a, const Ctrl* ctrl) {
  camera_tiles_body<E>(a, ctrl, blockIdx.x, gridDim.x);
}

// Float-float linearization of a camera tile: Jacobians, residual weights,
// products and sums all in float-float (the loop problems' reduced systems
// cancel ~25x, beyond what FP32 products leave).  Same outputs as
// k_camera_tiles.
template <bool E>
__global__ void __launch_bounds__(kTileThreads, 2) k_camera_tiles_dd(CamArgs a, const Ctrl* ctrl) {
  const CamF cam_ = cam_f(a.intr);
  const CamD camd_ = cam_dd(a.intr);
  (void)cam_; (void)camd_;
  if (halted(ctrl)) return;
  const int tile = blockIdx.x;
  const int fb = a.tile_fb[tile];
  const float* Pd = a.pose_dd + 24 * a.fb_pose[fb];
  Acc u[33];
#pragma unroll
  for (int k = 0; k < 33; ++k) u[k] = acc_zero();
  const int64_t e = a.tile_begin[tile] + threadIdx.x;
  if (e < a.tile_end[tile]) {
    const int64_t g = a.cam_g[e];
    const int pi = a.g_pt[g];
    const dd px = dd_from_double(a.points[3 * pi + 0]);
    const dd py = dd_from_double(a.points[3 * pi + 1]);
    const dd pz = dd_from_double(a.points[3 * pi + 2]);
    for (int64_t o = a.g_begin[g]; o < a.g_begin[g + 1]; ++o) {
      JacD J;
      jacobians_dd<E>(Pd, px, py, pz, camd_, &J);
      const float2 r = a.res[o], rl = a.res_lo[o];
      dd r0, r1;
      huber_weighted_dd(a.huber, a.huber_dd, dd_make(r.x, rl.x), dd_make(r.y, rl.y), &r0, &r1);
      int k = 0;
#pragma unroll
      for (int p = 0; p < 6; ++p) {
#pragma unroll
        for (int q = p; q < 6; ++q) {
          acc_madd(u[k], J.jp[p], J.jp[q]);
          acc_madd(u[k], J.jp[6 + p], J.jp[6 + q]);
          ++k;
        }
        acc_madd(u[21 + p], J.jp[p], r0);
        acc_madd(u[21 + p], J.jp[6 + p], r1);
      }
    }
    const int mb = a.pt_mb[pi];
    if (a.with_schur && mb >= 0) {
      const float* zd = a.zdd + kZD * g;
      const float* cv = a.cvec + 6 * mb;
      const dd c0 = dd_make(cv[0], cv[1]), c1 = dd_make(cv[2], cv[3]), c2 = dd_make(cv[4], cv[5]);
#pragma unroll
      for (int r = 0; r < 6; ++r) {
        acc_madd(u[27 + r], dd_make(zd[6 * r + 0], zd[6 * r + 1]), c0);
        acc_madd(u[27 + r], dd_make(zd[6 * r + 2], zd[6 * r + 3]), c1);
        acc_madd(u[27 + r], dd_make(zd[6 * r + 4], zd[6 * r + 5]), c2);
      }
    }
  }
  // float-float sums over the warp (transposed through shared memory, the hi
  // parts then the lo parts), then over the warps in fixed order
  __shared__ float zred[kTileThreads / 32][33][33];
  __shared__ float sh_hi[33][kTileThreads / 32];
  __shared__ float sh_lo[33][kTileThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  Acc t0 = acc_zero(), t1 = acc_zero();  // values lane and lane + 32
#pragma unroll
  for (int k = 0; k < 33; ++k) zred[w][k][lane] = u[k].hi;
  __syncwarp();
  for (int l = 0; l < 32; ++l) acc_addf(t0, zred[w][lane][l]);
  if (lane == 0)
    for (int l = 0; l < 32; ++l) acc_addf(t1, zred[w][32][l]);
  __syncwarp();
#pragma unroll
  for (int k = 0; k < 33; ++k) zred[w][k][lane] = u[k].lo;
  __syncwarp();
  for (int l = 0; l < 32; ++l) acc_addf(t0, zred[w][lane][l]);
  if (lane == 0)
    for (int l = 0; l < 32; ++l) acc_addf(t1, zred[w][32][l]);
  {
    const dd v0 = acc_get(t0);
    sh_hi[lane][w] = v0.hi;
    sh_lo[lane][w] = v0.lo;
    if (lane == 0) {
      const dd v1 = acc_get(t1);
      sh_hi[32][w] = v1.hi;
      sh_lo[32][w] = v1.lo;
    }
  }
  __syncthreads();
  if (threadIdx.x < kTileVals) {
    const int k = threadIdx.x;
    dd v = dd_make(0.f, 0.f);
    for (int q = 0; q < kTileThreads / 32; ++q) v = dd_add(v, dd_make(sh_hi[k][q], sh_lo[k][q]));
    a.tile_part[static_cast<int64_t>(tile) * kTileVals + k] = dd_to_double(v);
  }
}

__device__ __forceinline__ void camera_finalize_body(int nf, const int64_t* fb_tile_begin,
                                                        const double* tile_part, double* ufull, double* bf,
                                                        double* rb, Ctrl* ctrl, int with_schur,
                                                        const int32_t* prior_beg, const double* prior_out,
                                                        const int32_t* e_beg, const int32_t* e_slot,
                                                        const double* e_out, int bid_, int nblk_) {
  if (halted(ctrl)) return;
  const int fb = bid_;
  const int k = threadIdx.x;
  __shared__ double vals[kTileVals];
  if (k < kTileVals) {
    dd acc = dd_make(0.f, 0.f);
    for (int64_t t = fb_tile_begin[fb]; t < fb_tile_begin[fb + 1]; ++t)
      acc = dd_add(acc, dd_from_double(tile_part[t * kTileVals + k]));
    // cost functions on the poses alone (sgba_prior.cu): the priors on this
    // pose in prior order, then its pose-graph records in term order; J^T W J
    // into the 21 upper entries, J^T W g with the gradient sums
    dd pr = dd_make(0.f, 0.f);
    if (prior_beg || e_beg) {
      int idx;
      if (k < 21) {
        int a = 0, rem = k;
        while (rem >= 6 - a) { rem -= 6 - a; ++a; }
        idx = 6 * a + (a + rem);
      } else {
        idx = 36 + (k < 27 ? k - 21 : k - 27);
      }
      if (prior_beg)
        for (int q = prior_beg[fb]; q < prior_beg[fb + 1]; ++q)
          pr = dd_add(pr, dd_from_double(prior_out[static_cast<int64_t>(kPriorOut) * q + idx]));
      if (e_beg)
        for (int q = e_beg[fb]; q < e_beg[fb + 1]; ++q)
          pr = dd_add(pr, dd_from_double(e_out[static_cast<int64_t>(kPriorOut) * e_slot[q] + idx]));
    }
    if (k < 21) {
      acc = dd_add(acc, pr);
    } else if (k < 27) {
      acc = dd_neg(dd_add(acc, pr));  // neg_grad = -sum J^T r~ - sum J^T W g
    } else {
      // reduced rhs: b_f - sum Z c  (b_f = -g)
      dd g = dd_make(0.f, 0.f);
      for (int64_t t = fb_tile_begin[fb]; t < fb_tile_begin[fb + 1]; ++t)
        g = dd_add(g, dd_from_double(tile_part[t * kTileVals + k - 6]));
      g = dd_add(g, pr);
      acc = dd_sub(dd_neg(g), acc);
    }
    vals[k] = dd_to_double(acc);
  }
  __syncthreads();
  if (k < 36) {
    // full 6x6 U from the 21 upper entries
    const int p = k / 6, q = k % 6;
    const int a = p < q ? p : q, b = p < q ? q : p;
    const int idx = a * 6 - a * (a - 1) / 2 + (b - a);
    ufull[36 * fb + k] = vals[idx];
  }
  if (k < 6) {
    bf[6 * fb + k] = vals[21 + k];
    if (with_schur) rb[6 * fb + k] = vals[27 + k];
  }
  if (k == 0) {
    double mg = 0.0;
    for (int p = 0; p < 6; ++p) mg = fmax(mg, fabs(vals[21 + p]));
    atomic_max_nonneg(&ctrl->max_grad_bits, mg);
  }
  if (with_schur) {
    // the last block to finish: gradient-tolerance check before the solve
    // (optimizer_step.rs:382-384) and singular point blocks (SingularMargBlock
    // -> reject); every block's maximum is in by then
    __shared__ bool s_last;
    __threadfence();
    if (k == 0) s_last = (atomicAdd(&ctrl->fin_ticket, 1) == static_cast<int>(nblk_) - 1);
    __syncthreads();
    if (s_last && k == 0) {
      __threadfence();
      const double mg = __longlong_as_double(static_cast<long long>(atomicAdd(&ctrl->max_grad_bits, 0ull)));
      ctrl->max_grad = mg;
      // the gradient check is skipped with equality constraints (optimizer.rs:527-535)
      if (mg < ctrl->gtol && ctrl->n_eq == 0) {
        ctrl->skip = 1;
      } else if (ctrl->fail) {
        ctrl->skip = 2;
      }
      ctrl->fail = 0;
      ctrl->fin_ticket = 0;
    }
  }
}
__global__ void __launch_bounds__(64) k_camera_finalize(int nf, const int64_t* fb_tile_begin,
                                                        const double* tile_part, double* ufull, double* bf,
                                                        double* rb, Ctrl* ctrl, int with_schur,
                                                        const int32_t* prior_beg, const double* prior_out,
                                                        const int32_t* e_beg, const int32_t* e_slot,
                                                        const double* e_out) {
  camera_finalize_body(nf, fb_tile_begin, tile_part, ufull, bf, rb, ctrl, with_schur, prior_beg, prior_out, e_beg,
                       e_slot, e_out, blockIdx.x, gridDim.x);
}


// ---------------------------------------------------------------------------
// Reduced camera system: one warp per lower 6x6 block (row j >= col k).
//   S_jk = [j == k] (U_j + nu n_j I) - sum_{pairs} Z_a Z_b^T
// FP32 products and per-lane FP32 partial sums; float-float across lanes;
// f64 store (both triangles).
// ---------------------------------------------------------------------------
struct SchurArgs {
  int64_t nsb;
  const int32_t* sb_row;
  const int32_t* sb_col;
  const int64_t* sb_pair_begin;
  const int2* pairs;
  int64_t nchunk;                 // pair chunks (each within one block)
  const int64_t* chunk_begin;     // nchunk + 1, into pairs
  const int32_t* block_chunk_begin;  // nsb + 1, into chunks
  float2* part;                   // 36 float-float partials per chunk
  const float* zmat;
  const float* zdd;   // float-float Z (float-float linearization)
  const double* ufull;
  const double* cnt_f;
  double* S;
  float2* S2;  // float-float copy (may be null)
  int n6;
  // pose-graph edges: per lower block the terms whose J_m^T J_n lands there
  // (bit 31: transposed), or null
  const int32_t* eblk_begin;
  const int32_t* eblk_term;
  const double* e_hmn;
};

__device__ __forceinline__ void load_z(const float* zmat, int g, float* z) {
  const float4* p = reinterpret_cast<const float4*>(zmat + kZS * static_cast<int64_t>(g));
#pragma unroll
  for (int q = 0; q < 5; ++q) {
    float4 v = __ldg(p + q);
    z[4 * q] = v.x; z[4 * q + 1] = v.y; z[4 * q + 2] = v.z; z[4 * q + 3] = v.w;
  }
}

// Pass 1, one warp per chunk of at most kSchurChunk observation pairs of one
// block (heavy blocks are split so no warp walks thousands of pairs): FP32
// products and per-lane FP32 sums, float-float across lanes, one partial
// (36 float-float entries) per chunk.
__device__ __forceinline__ void schur_body(SchurArgs a, const Ctrl* ctrl, int bid_, int nblk_) {
  if (skipping(ctrl)) return;
  __shared__ float red[8][36][33];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  for (int64_t ch = static_cast<int64_t>(bid_) * wpb + wib; ch < a.nchunk;
       ch += static_cast<int64_t>(nblk_) * wpb) {
    float acc[36];
#pragma unroll
    for (int e = 0; e < 36; ++e) acc[e] = 0.f;
    const int64_t q1 = a.chunk_begin[ch + 1];
    int64_t q = a.chunk_begin[ch] + lane;
    int2 pr = (q < q1) ? a.pairs[q] : make_int2(0, 0);
    while (q < q1) {
      const int2 nx = (q + 32 < q1) ? a.pairs[q + 32] : make_int2(0, 0);  // next pair, prefetched
      float za[20], zb[20];
      load_z(a.zmat, pr.x, za);
      load_z(a.zmat, pr.y, zb);
#pragma unroll
      for (int r = 0; r < 6; ++r)
#pragma unroll
        for (int c = 0; c < 6; ++c) {
          float v = acc[r * 6 + c];
          v = fmaf(za[r * 3 + 0], zb[c * 3 + 0], v);
          v = fmaf(za[r * 3 + 1], zb[c * 3 + 1], v);
          v = fmaf(za[r * 3 + 2], zb[c * 3 + 2], v);
          acc[r * 6 + c] = v;
        }
      pr = nx;
      q += 32;
    }
    // transpose through shared memory; lane e (< 36) sums entry e in float-float
#pragma unroll
    for (int e = 0; e < 36; ++e) red[wib][e][lane] = acc[e];
    __syncwarp();
    for (int e = lane; e < 36; e += 32) {
      dd t = dd_make(0.f, 0.f);
#pragma unroll 8
      for (int l = 0; l < 32; ++l) t = dd_add_f(t, red[wib][e][l]);
      a.part[36 * ch + e] = make_float2(t.hi, t.lo);
    }
    __syncwarp();
  }
}
__global__ void __launch_bounds__(256, 2) k_schur(SchurArgs a, const Ctrl* ctrl) {
  schur_body(a, ctrl, blockIdx.x, gridDim.x);
}

// Pass 1 of the float-float linearization: the same chunks, float-float Z and
// float-float products and sums (36 accumulators per lane).  The products of
// a pair go by the inner index t (column t of both Z, 24 floats live instead
// of 72), which keeps two CTAs per SM; every accumulator still receives its
// t = 0, 1, 2 terms in that order.
__global__ void __launch_bounds__(256, 2) k_schur_dd(SchurArgs a, const Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  __shared__ float red[8][36][33];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  for (int64_t ch = static_cast<int64_t>(blockIdx.x) * wpb + wib; ch < a.nchunk;
       ch += static_cast<int64_t>(gridDim.x) * wpb) {
    Acc acc[36];
#pragma unroll
    for (int e = 0; e < 36; ++e) acc[e] = acc_zero();
    const int64_t q1 = a.chunk_begin[ch + 1];
    for (int64_t q = a.chunk_begin[ch] + lane; q < q1; q += 32) {
      const int2 pr = a.pairs[q];
      const float2* pa = reinterpret_cast<const float2*>(a.zdd + kZD * static_cast<int64_t>(pr.x));
      const float2* pb = reinterpret_cast<const float2*>(a.zdd + kZD * static_cast<int64_t>(pr.y));
#pragma unroll
      for (int t = 0; t < 3; ++t) {
        float2 za[6], zb[6];  // column t of each Z: (hi, lo) of rows 0..5
#pragma unroll
        for (int r = 0; r < 6; ++r) {
          za[r] = __ldg(pa + 3 * r + t);
          zb[r] = __ldg(pb + 3 * r + t);
        }
#pragma unroll
        for (int r = 0; r < 6; ++r)
#pragma unroll
          for (int c = 0; c < 6; ++c)
            acc_madd(acc[r * 6 + c], dd_make(za[r].x, za[r].y), dd_make(zb[c].x, zb[c].y));
      }
    }
    // lanes' accumulators summed in float-float: hi parts, then lo parts
    Acc t0 = acc_zero(), t1 = acc_zero();  // entries lane and lane + 32
#pragma unroll
    for (int e = 0; e < 36; ++e) red[wib][e][lane] = acc[e].hi;
    __syncwarp();
    for (int l = 0; l < 32; ++l) acc_addf(t0, red[wib][lane][l]);
    if (lane < 4)
      for (int l = 0; l < 32; ++l) acc_addf(t1, red[wib][lane + 32][l]);
    __syncwarp();
#pragma unroll
    for (int e = 0; e < 36; ++e) red[wib][e][lane] = acc[e].lo;
    __syncwarp();
    for (int l = 0; l < 32; ++l) acc_addf(t0, red[wib][lane][l]);
    if (lane < 4)
      for (int l = 0; l < 32; ++l) acc_addf(t1, red[wib][lane + 32][l]);
    const dd v0 = acc_get(t0);
    a.part[36 * ch + lane] = make_float2(v0.hi, v0.lo);
    if (lane < 4) {
      const dd v1 = acc_get(t1);
      a.part[36 * ch + lane + 32] = make_float2(v1.hi, v1.lo);
    }
    __syncwarp();
  }
}

// Pass 2, one warp per lower block of S: the block's chunk partials summed in
// chunk order (float-float), the diagonal U + nu n I added on diagonal
// blocks; f64 store of both triangles (and the float-float copy).
__device__ __forceinline__ void schur_reduce_body(SchurArgs a, const Ctrl* ctrl, int bid_, int nblk_) {
  if (skipping(ctrl)) return;
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const double nu = ctrl->nu;
  for (int64_t blk = static_cast<int64_t>(bid_) * wpb + wib; blk < a.nsb;
       blk += static_cast<int64_t>(nblk_) * wpb) {
    const int j = a.sb_row[blk], k = a.sb_col[blk];
    const int c0 = a.block_chunk_begin[blk], c1 = a.block_chunk_begin[blk + 1];
    for (int e = lane; e < 36; e += 32) {
      dd t = dd_make(0.f, 0.f);
      for (int c = c0; c < c1; ++c) {
        const float2 v = a.part[36 * static_cast<int64_t>(c) + e];
        t = dd_add(t, dd_make(v.x, v.y));
      }
      const int r = e / 6, cc = e % 6;
      dd vd;
      if (j == k) {
        dd base = dd_from_double(a.ufull[36 * j + r * 6 + cc]);
        if (r == cc) base = dd_add(base, dd_from_double(nu * a.cnt_f[j]));
        vd = dd_sub(base, t);
      } else {
        vd = dd_neg(t);
      }
      if (a.eblk_begin)
        for (int q = a.eblk_begin[blk]; q < a.eblk_begin[blk + 1]; ++q) {
          const int32_t tt = a.eblk_term[q];
          const int64_t term = tt & 0x7fffffff;
          const double h = (tt < 0) ? a.e_hmn[36 * term + cc * 6 + r] : a.e_hmn[36 * term + r * 6 + cc];
          vd = dd_add(vd, dd_from_double(h));
        }
      const double v = dd_to_double(vd);
      const int64_t row = 6 * j + r, col = 6 * k + cc;
      a.S[row * a.n6 + col] = v;
      a.S[col * a.n6 + row] = v;
      if (a.S2) {
        a.S2[row * a.n6 + col] = make_float2(vd.hi, vd.lo);
        a.S2[col * a.n6 + row] = make_float2(vd.hi, vd.lo);
      }
    }
  }
}
__global__ void __launch_bounds__(256) k_schur_reduce(SchurArgs a, const Ctrl* ctrl) {
  schur_reduce_body(a, ctrl, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------------------
// Dense reduced systems (local windows: every camera sees most points): S
// formed by tiles of kSdB x kSdB pose blocks instead of observation pairs.
// A CTA (kSdThreads threads) owns one tile of the lower triangle and streams
// every point once, in rounds of kSdPts points: thread (point, slot) fetches
// the Z records of the point's terms with the slot's row pose and column pose
// (the term table T; zeros where there is none) into registers one round
// ahead and stores them into shared memory; every thread then accumulates a
// 3 x 6 piece of the tile, rows (tid / 8) + 16 i and columns (tid % 8) + 8 j,
// so that the rows a warp reads are consecutive (no bank conflicts) and each
// shared-memory load feeds 18 or 9 FMAs (FP32 within a round, float-float
// across rounds, every entry in point order).  The entries are written as
// S = U + nu n I - sum Z Z^T (the formula of k_schur_reduce), in f64 and
// float-float.  Loads per point and tile: 2 kSdB Z records, against two per
// observation pair.
// ---------------------------------------------------------------------------
constexpr int kSdB = 8;          // pose blocks per tile side
constexpr int kSdT = 6 * kSdB;   // 48 rows / columns
constexpr int kSdPts = 16;       // points per round: 16 points x 8 slots, one per thread
constexpr int kSdThreads = 128;

struct SchurDenseArgs {
  int np, nf, n6;
  const int32_t* zterm;  // np x nf: term of (point, free block) or -1
  const float* zmat;
  const double* ufull;
  const double* cnt_f;
  double* S;
  float2* S2;
};

// the Z record (6 x 3 row-major, 20 floats) of term g, or zeros
__device__ __forceinline__ void sd_fetch(const float* zmat, int g, float4* v) {
  if (g >= 0) {
    const float4* src = reinterpret_cast<const float4*>(zmat + kZS * static_cast<int64_t>(g));
#pragma unroll
    for (int q = 0; q < 5; ++q) v[q] = __ldg(src + q);
  } else {
#pragma unroll
    for (int q = 0; q < 5; ++q) v[q] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// the six rows of a fetched record, padded to float4, into shared memory
__device__ __forceinline__ void sd_store(float (*dst)[4], const float4* v) {
  reinterpret_cast<float4*>(dst[0])[0] = make_float4(v[0].x, v[0].y, v[0].z, 0.f);
  reinterpret_cast<float4*>(dst[1])[0] = make_float4(v[0].w, v[1].x, v[1].y, 0.f);
  reinterpret_cast<float4*>(dst[2])[0] = make_float4(v[1].z, v[1].w, v[2].x, 0.f);
  reinterpret_cast<float4*>(dst[3])[0] = make_float4(v[2].y, v[2].z, v[2].w, 0.f);
  reinterpret_cast<float4*>(dst[4])[0] = make_float4(v[3].x, v[3].y, v[3].z, 0.f);
  reinterpret_cast<float4*>(dst[5])[0] = make_float4(v[3].w, v[4].x, v[4].y, 0.f);
}

__device__ __forceinline__ void schur_dense_body(SchurDenseArgs a, const Ctrl* ctrl, int bid_, int nblk_) {
  (void)nblk_;
  if (skipping(ctrl)) return;
  __shared__ __align__(16) float zr[kSdPts][kSdT][4];  // Z rows of the tile's row poses (k = 0..2, padded)
  __shared__ __align__(16) float zc[kSdPts][kSdT][4];  // the same for its column poses
  // tile (ti, tj), tj <= ti, of the lower triangle
  int ti = static_cast<int>((sqrtf(8.0f * static_cast<float>(bid_) + 1.0f) - 1.0f) * 0.5f);
  while (ti * (ti + 1) / 2 > bid_) --ti;
  while ((ti + 1) * (ti + 2) / 2 <= bid_) ++ti;
  const int tj = bid_ - ti * (ti + 1) / 2;
  const int I0 = ti * kSdB, J0 = tj * kSdB;
  const int tid = threadIdx.x;
  const int rq = tid >> 3, cq = tid & 7;  // rows rq + 16 i, columns cq + 8 j
  // this thread's staging slot: point pp of each round, row pose I0 + slot and column pose J0 + slot
  const int pp = tid >> 3, slot = tid & 7;
  const int fr = I0 + slot, fc = J0 + slot;
  auto term_of = [&](int p0, int f) {
    const int i = p0 + pp;
    return (i < a.np && f < a.nf) ? __ldg(a.zterm + static_cast<int64_t>(i) * a.nf + f) : -1;
  };
  float acc[3][6];
  Acc accd[3][6];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      acc[i][j] = 0.0f;
      accd[i][j] = acc_zero();
    }
  // the term indices run two rounds ahead, the Z records one round ahead
  float4 vr[5], vc[5];
  sd_fetch(a.zmat, term_of(0, fr), vr);
  sd_fetch(a.zmat, term_of(0, fc), vc);
  int gr_next = term_of(kSdPts, fr), gc_next = term_of(kSdPts, fc);
  for (int p0 = 0; p0 < a.np; p0 += kSdPts) {
    __syncthreads();  // the previous round's reads are done
    sd_store(&zr[pp][6 * slot], vr);
    sd_store(&zc[pp][6 * slot], vc);
    __syncthreads();
    if (p0 + kSdPts < a.np) {  // next round, in flight during the products
      sd_fetch(a.zmat, gr_next, vr);
      sd_fetch(a.zmat, gc_next, vc);
      gr_next = term_of(p0 + 2 * kSdPts, fr);
      gc_next = term_of(p0 + 2 * kSdPts, fc);
    }
    const int npt = a.np - p0 < kSdPts ? a.np - p0 : kSdPts;
    for (int q = 0; q < npt; ++q) {
      float4 ra[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) ra[i] = reinterpret_cast<const float4*>(&zr[q][rq + 16 * i][0])[0];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        float4 cb[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) cb[j] = reinterpret_cast<const float4*>(&zc[q][cq + 8 * (3 * h + j)][0])[0];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            float w = acc[i][3 * h + j];
            w = fmaf(ra[i].x, cb[j].x, w);
            w = fmaf(ra[i].y, cb[j].y, w);
            w = fmaf(ra[i].z, cb[j].z, w);
            acc[i][3 * h + j] = w;
          }
      }
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        acc_addf(accd[i][j], acc[i][j]);
        acc[i][j] = 0.0f;
      }
  }
  const double nu = ctrl->nu;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      const int row = 6 * I0 + rq + 16 * i, col = 6 * J0 + cq + 8 * j;
      if (row >= a.n6 || col >= a.n6 || col > row) continue;
      const dd t = acc_get(accd[i][j]);
      const int bj = row / 6, bk = col / 6, r = row % 6, cc = col % 6;
      dd vd;
      if (bj == bk) {
        dd base = dd_from_double(a.ufull[36 * bj + r * 6 + cc]);
        if (r == cc) base = dd_add(base, dd_from_double(nu * a.cnt_f[bj]));
        vd = dd_sub(base, t);
      } else {
        vd = dd_neg(t);
      }
      const double w = dd_to_double(vd);
      a.S[static_cast<int64_t>(row) * a.n6 + col] = w;
      a.S[static_cast<int64_t>(col) * a.n6 + row] = w;
      if (a.S2) {
        a.S2[static_cast<int64_t>(row) * a.n6 + col] = make_float2(vd.hi, vd.lo);
        a.S2[static_cast<int64_t>(col) * a.n6 + row] = make_float2(vd.hi, vd.lo);
      }
    }
}
__global__ void __launch_bounds__(kSdThreads, 3) k_schur_dense(SchurDenseArgs a, const Ctrl* ctrl) {
  schur_dense_body(a, ctrl, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------------------
// Back-substitution (SchurFactor::solve, schur_ldlt.rs:782-803):
//   dx_m = V'^-1 (b_m - sum W_g^T dx_f) = C^-T (c - sum Z_g^T dx_f)
// ---------------------------------------------------------------------------
struct BackArgs {
  int32_t np;
  const int64_t* pt_g_begin;
  const int32_t* g_pose;
  const int32_t* pose_fb;
  const int32_t* pt_mb;
  const float* zmat;
  const float* zdd;  // float-float Z (float-float linearization) or null
  const float* zdd_flagged;  // float-float Z of the terms flagged in zmat (other problems)
  const float* cinv;
  const float* cvec;
  const float* xdd;  // dx_f as float-float pairs
  double* dm;
  // scale gauge: the free poses' gauge direction v_f = [0; t_j - c] carried
  // through the same back-substitution, u_m = -C^-T sum Z_g^T v_f (the
  // projection's direction for the points)
  int gauge_kind;
  const double* poses;
  double cx, cy, cz;
  double* um;
  // free intrinsics: dx_m also loses C^-T Zk^T dx_k (dx_k at rows 6 nf .. 6 nf + 5)
  const float* zk;  // nm x kIntrZk or null
  int k0;           // 6 nf
};

// s[q] += (Zk^T dx_k)_q for a point with terms (free intrinsics).
__device__ __forceinline__ void intr_backsub_term(const BackArgs& a, int mb, dd* s) {
  const float* zk = a.zk + kIntrZk * static_cast<int64_t>(mb);
  const float2* xk = reinterpret_cast<const float2*>(a.xdd) + a.k0;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    dd t = s[q];
#pragma unroll
    for (int r = 0; r < kIntrMax; ++r) {
      const float2 xv = xk[r];
      t = dd_add(t, dd_mul(dd_make(xv.x, xv.y), dd_make(zk[2 * (r * 3 + q)], zk[2 * (r * 3 + q) + 1])));
    }
    s[q] = t;
  }
}

__device__ __forceinline__ void backsub_body(BackArgs a, const Ctrl* ctrl, int bid_, int nblk_) {
  if (skipping(ctrl)) return;
  __shared__ float red[8][12][33];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const bool gauge = a.gauge_kind == 1;
  for (int64_t i = static_cast<int64_t>(bid_) * wpb + wib; i < a.np;
       i += static_cast<int64_t>(nblk_) * wpb) {
    const int mb = a.pt_mb[i];
    if (mb < 0) continue;
    dd t[3] = {dd_make(0.f, 0.f), dd_make(0.f, 0.f), dd_make(0.f, 0.f)};
    dd tg[3] = {dd_make(0.f, 0.f), dd_make(0.f, 0.f), dd_make(0.f, 0.f)};  // sum Z^T v_f
    for (int64_t g = a.pt_g_begin[i] + lane; g < a.pt_g_begin[i + 1]; g += 32) {
      const int pj = a.g_pose[g];
      const int fb = a.pose_fb[pj];
      if (fb < 0) continue;
      // Z of the term, read once: float-float under the float-float
      // linearization and for the points rebuilt in float-float (C^-T
      // amplifies the rounding of Z along their weakly held direction), FP32
      // otherwise
      float zr[36];
      bool use_dd = a.zdd != nullptr;
      if (!use_dd) {
        float Z[20];
        load_z(a.zmat, static_cast<int>(g), Z);
        use_dd = Z[18] != 0.f && a.zdd_flagged;
        if (!use_dd) {
#pragma unroll
          for (int k = 0; k < 18; ++k) {
            zr[2 * k] = Z[k];
            zr[2 * k + 1] = 0.f;
          }
        }
      }
      if (use_dd) {
        const float4* zp = reinterpret_cast<const float4*>((a.zdd ? a.zdd : a.zdd_flagged) + kZD * g);
#pragma unroll
        for (int k = 0; k < 9; ++k) {
          const float4 v = __ldg(zp + k);
          zr[4 * k] = v.x; zr[4 * k + 1] = v.y; zr[4 * k + 2] = v.z; zr[4 * k + 3] = v.w;
        }
      }
      // entry (r, q) of Z: (zr[6 r + 2 q], zr[6 r + 2 q + 1]) as (hi, lo)
      const float2* xp = reinterpret_cast<const float2*>(a.xdd) + 6 * fb;
#pragma unroll
      for (int r = 0; r < 6; ++r) {
        const float2 xv = xp[r];
        const dd x = dd_make(xv.x, xv.y);
#pragma unroll
        for (int q = 0; q < 3; ++q) t[q] = dd_add(t[q], dd_mul(x, dd_make(zr[6 * r + 2 * q], zr[6 * r + 2 * q + 1])));
      }
      if (gauge) {
        const double* T = a.poses + 7 * static_cast<int64_t>(pj);
        const dd v[3] = {dd_from_double(T[4] - a.cx), dd_from_double(T[5] - a.cy), dd_from_double(T[6] - a.cz)};
#pragma unroll
        for (int r = 3; r < 6; ++r)
#pragma unroll
          for (int q = 0; q < 3; ++q)
            tg[q] = dd_add(tg[q], dd_mul(v[r - 3], dd_make(zr[6 * r + 2 * q], zr[6 * r + 2 * q + 1])));
      }
    }
    // float-float sum over the lanes: fixed tree through shared memory
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      red[wib][2 * q][lane] = t[q].hi;
      red[wib][2 * q + 1][lane] = t[q].lo;
      red[wib][6 + 2 * q][lane] = tg[q].hi;
      red[wib][6 + 2 * q + 1][lane] = tg[q].lo;
    }
    __syncwarp();
    const int nq = gauge ? 6 : 3;
#pragma unroll
    for (int h = 16; h > 0; h >>= 1) {
      if (lane < h) {
        for (int q = 0; q < nq; ++q) {
          const dd u = dd_add(dd_make(red[wib][2 * q][lane], red[wib][2 * q + 1][lane]),
                              dd_make(red[wib][2 * q][lane + h], red[wib][2 * q + 1][lane + h]));
          red[wib][2 * q][lane] = u.hi;
          red[wib][2 * q + 1][lane] = u.lo;
        }
      }
      __syncwarp();
    }
    if (lane == 0 && gauge) {
      // u_m = -C^-T sum Z^T v_f
      const float* cp = a.cinv + 12 * mb;
      dd ci[6];
      for (int k = 0; k < 6; ++k) ci[k] = dd_make(cp[2 * k], cp[2 * k + 1]);
      const dd g0 = dd_make(red[wib][6][0], red[wib][7][0]);
      const dd g1 = dd_make(red[wib][8][0], red[wib][9][0]);
      const dd g2 = dd_make(red[wib][10][0], red[wib][11][0]);
      const dd u0 = dd_add(dd_add(dd_mul(g0, ci[0]), dd_mul(g1, ci[1])), dd_mul(g2, ci[3]));
      const dd u1 = dd_add(dd_mul(g1, ci[2]), dd_mul(g2, ci[4]));
      const dd u2 = dd_mul(g2, ci[5]);
      a.um[3 * mb + 0] = -dd_to_double(u0);
      a.um[3 * mb + 1] = -dd_to_double(u1);
      a.um[3 * mb + 2] = -dd_to_double(u2);
    }
    if (lane == 0) {
      dd s[3];
      for (int q = 0; q < 3; ++q) s[q] = dd_make(red[wib][2 * q][0], red[wib][2 * q + 1][0]);
      if (a.zk && a.pt_g_begin[i + 1] > a.pt_g_begin[i]) intr_backsub_term(a, mb, s);
      const float* cv = a.cvec + 6 * mb;
      dd c0 = dd_sub(dd_make(cv[0], cv[1]), s[0]);
      dd c1 = dd_sub(dd_make(cv[2], cv[3]), s[1]);
      dd c2 = dd_sub(dd_make(cv[4], cv[5]), s[2]);
      const float* cp = a.cinv + 12 * mb;  // 00 10 11 20 21 22 as (hi, lo)
      dd ci[6];
      for (int k = 0; k < 6; ++k) ci[k] = dd_make(cp[2 * k], cp[2 * k + 1]);
      // C^-T * c : (C^-T)[a][b] = Cinv[b][a]
      dd d0 = dd_add(dd_add(dd_mul(c0, ci[0]), dd_mul(c1, ci[1])), dd_mul(c2, ci[3]));
      dd d1 = dd_add(dd_mul(c1, ci[2]), dd_mul(c2, ci[4]));
      dd d2 = dd_mul(c2, ci[5]);
      a.dm[3 * mb + 0] = dd_to_double(d0);
      a.dm[3 * mb + 1] = dd_to_double(d1);
      a.dm[3 * mb + 2] = dd_to_double(d2);
    }
    __syncwarp();
  }
}
__global__ void __launch_bounds__(256) k_backsub(BackArgs a, const Ctrl* ctrl) {
  backsub_body(a, ctrl, blockIdx.x, gridDim.x);
}

// Back-substitution by chunks of consecutive points (the landmark pass's
// chunks): a thread per term forms Z_g^T dx_f and Z_g^T v_f (float-float),
// then a thread per point sums its terms in order and applies C^-T.  Same
// arithmetic per term as k_backsub; every lane busy (the loops' tracks of
// ~8 terms left 3/4 of a warp-per-point kernel idle).
__device__ __forceinline__ void backsub_chunks_body(BackArgs a, const int32_t* chunk_pt, int nchunk,
                                                        const int32_t* g_pt, const Ctrl* ctrl, int bid_, int nblk_) {
  if (skipping(ctrl)) return;
  extern __shared__ float bsm[];  // [cap][12]: Z^T dx_f, Z^T v_f as (hi, lo)
  __shared__ float2 ssum[kLmkTerms][6];  // per point: the 6 sums over its terms
  const bool gauge = a.gauge_kind == 1;
  const int tid = threadIdx.x;
  for (int c = bid_; c < nchunk; c += nblk_) {
    const int p0 = chunk_pt[c], p1 = chunk_pt[c + 1];
    const int64_t t0 = a.pt_g_begin[p0];
    const int nt = static_cast<int>(a.pt_g_begin[p1] - t0);
    for (int t = tid; t < nt; t += blockDim.x) {
      const int64_t g = t0 + t;
      const int pj = a.g_pose[g];
      const int fb = a.pose_fb[pj];
      dd tt[3] = {dd_make(0.f, 0.f), dd_make(0.f, 0.f), dd_make(0.f, 0.f)};
      dd tg[3] = {dd_make(0.f, 0.f), dd_make(0.f, 0.f), dd_make(0.f, 0.f)};
      if (fb >= 0 && a.pt_mb[g_pt[g]] >= 0) {
        const float2* xp = reinterpret_cast<const float2*>(a.xdd) + 6 * fb;
        dd v[3] = {dd_make(0.f, 0.f), dd_make(0.f, 0.f), dd_make(0.f, 0.f)};
        if (gauge) {
          const double* T = a.poses + 7 * static_cast<int64_t>(pj);
          v[0] = dd_from_double(T[4] - a.cx);
          v[1] = dd_from_double(T[5] - a.cy);
          v[2] = dd_from_double(T[6] - a.cz);
        }
        bool use_dd = a.zdd != nullptr;
        float Z[20];
        if (!use_dd) {
          load_z(a.zmat, static_cast<int>(g), Z);
          use_dd = Z[18] != 0.f && a.zdd_flagged;
        }
        if (use_dd) {
          const float4* zp = reinterpret_cast<const float4*>((a.zdd ? a.zdd : a.zdd_flagged) + kZD * g);
          float zr[36];
#pragma unroll
          for (int k = 0; k < 9; ++k) {
            const float4 w4 = __ldg(zp + k);
            zr[4 * k] = w4.x; zr[4 * k + 1] = w4.y; zr[4 * k + 2] = w4.z; zr[4 * k + 3] = w4.w;
          }
#pragma unroll
          for (int r = 0; r < 6; ++r) {
            const float2 xv = xp[r];
            const dd x = dd_make(xv.x, xv.y);
#pragma unroll
            for (int q = 0; q < 3; ++q) {
              const dd z = dd_make(zr[6 * r + 2 * q], zr[6 * r + 2 * q + 1]);
              tt[q] = dd_add(tt[q], dd_mul(x, z));
              if (gauge && r >= 3) tg[q] = dd_add(tg[q], dd_mul(v[r - 3], z));
            }
          }
        } else {
#pragma unroll
          for (int r = 0; r < 6; ++r) {
            const float2 xv = xp[r];
            const dd x = dd_make(xv.x, xv.y);
#pragma unroll
            for (int q = 0; q < 3; ++q) {
              tt[q] = dd_add(tt[q], dd_mul_f(x, Z[r * 3 + q]));
              if (gauge && r >= 3) tg[q] = dd_add(tg[q], dd_mul_f(v[r - 3], Z[r * 3 + q]));
            }
          }
        }
      }
      float* ts = bsm + static_cast<int64_t>(t) * 12;
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        ts[2 * q] = tt[q].hi;
        ts[2 * q + 1] = tt[q].lo;
        ts[6 + 2 * q] = tg[q].hi;
        ts[7 + 2 * q] = tg[q].lo;
      }
    }
    __syncthreads();
    // the sums of every point, a thread per (point, value), in term order
    for (int e = tid; e < 6 * (p1 - p0); e += blockDim.x) {
      const int q = e / 6, k = e - 6 * q;
      const int tb = static_cast<int>(a.pt_g_begin[p0 + q] - t0), te = static_cast<int>(a.pt_g_begin[p0 + q + 1] - t0);
      dd sacc = dd_make(0.f, 0.f);
      for (int t = tb; t < te; ++t) {
        const float* ts = bsm + static_cast<int64_t>(t) * 12;
        sacc = dd_add(sacc, dd_make(ts[2 * k], ts[2 * k + 1]));
      }
      ssum[q][k] = make_float2(sacc.hi, sacc.lo);
    }
    __syncthreads();
    for (int q = tid; q < p1 - p0; q += blockDim.x) {
      const int i = p0 + q;
      const int mb = a.pt_mb[i];
      if (mb < 0) continue;
      const int tb = static_cast<int>(a.pt_g_begin[i] - t0), te = static_cast<int>(a.pt_g_begin[i + 1] - t0);
      dd sm[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) sm[k] = dd_make(ssum[q][k].x, ssum[q][k].y);
      if (a.zk && te > tb) intr_backsub_term(a, mb, sm);
      const float* cp = a.cinv + 12 * mb;  // 00 10 11 20 21 22 as (hi, lo)
      dd ci[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) ci[k] = dd_make(cp[2 * k], cp[2 * k + 1]);
      const float* cv = a.cvec + 6 * mb;
      const dd c0 = dd_sub(dd_make(cv[0], cv[1]), sm[0]);
      const dd c1 = dd_sub(dd_make(cv[2], cv[3]), sm[1]);
      const dd c2 = dd_sub(dd_make(cv[4], cv[5]), sm[2]);
      // C^-T * c : (C^-T)[a][b] = Cinv[b][a]
      const dd d0 = dd_add(dd_add(dd_mul(c0, ci[0]), dd_mul(c1, ci[1])), dd_mul(c2, ci[3]));
      const dd d1 = dd_add(dd_mul(c1, ci[2]), dd_mul(c2, ci[4]));
      const dd d2 = dd_mul(c2, ci[5]);
      a.dm[3 * mb + 0] = dd_to_double(d0);
      a.dm[3 * mb + 1] = dd_to_double(d1);
      a.dm[3 * mb + 2] = dd_to_double(d2);
      if (gauge) {
        const dd u0 = dd_add(dd_add(dd_mul(sm[3], ci[0]), dd_mul(sm[4], ci[1])), dd_mul(sm[5], ci[3]));
        const dd u1 = dd_add(dd_mul(sm[4], ci[2]), dd_mul(sm[5], ci[4]));
        const dd u2 = dd_mul(sm[5], ci[5]);
        a.um[3 * mb + 0] = -dd_to_double(u0);
        a.um[3 * mb + 1] = -dd_to_double(u1);
        a.um[3 * mb + 2] = -dd_to_double(u2);
      }
    }
    __syncthreads();
  }
}
__global__ void __launch_bounds__(256) k_backsub_chunks(BackArgs a, const int32_t* chunk_pt, int nchunk,
                                                        const int32_t* g_pt, const Ctrl* ctrl) {
  backsub_chunks_body(a, chunk_pt, nchunk, g_pt, ctrl, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------------------
// Free intrinsics (kinds F, F, M: the intrinsics family Free).  The camera's
// params k are one more free variable that every term touches: J_k = d r / d k
// per observation, the camera's -dx_params (pinhole_reprojection.rs:85):
//   pinhole, k = (fx, fy, cx, cy):  J_k = -[[x, 0, 1, 0], [0, y, 0, 1]]
//   EUCM, k = (fx, fy, cx, cy, alpha, beta) (enhanced_unified.rs:158-215):
//     J_k = -[[mx, 0, 1, 0, -fx x (rho - 1) / norm^2, -fx x alpha r2 / (2 rho norm^2)],
//             [0, my, 0, 1, -fy y (rho - 1) / norm^2, -fy y alpha r2 / (2 rho norm^2)]]
//   with (x, y) the z = 1 projection, r2 = x^2 + y^2, (mx, my) = (x, y) / norm;
// with the reference's nu I per reduced term on its diagonal.  Internally the
// intrinsics are the last block of S (rows 6 nf .. 6 nf + 5; the pinhole's 4
// params padded to 6 rows with an identity, as the oracle pads them); the step
// is the same in any order.  The kernels work on 6 params throughout, the
// pinhole's J_k having zero columns 4 and 5.
//   per point i:  Y_i = sum J_k^T J_m,  Zk_i = Y_i C_i^-T,
//   S_kk = sum J_k^T J_k - sum_i Zk_i Zk_i^T + nu n_terms I,
//   S_kj = sum_{terms of pose j} (J_k^T J_p - Zk_i Z_g^T),
//   rhs_k = -sum J_k^T r~ - sum_i Zk_i c_i,
//   dx_m -= C^-T Zk_i^T dx_k in the back-substitution, k <- k + dx_k.
// Everything in float-float (these problems are small: the dense solvers).
// ---------------------------------------------------------------------------
constexpr int kK = kIntrMax;           // 6 params per J_k row
constexpr int kKT = kK * (kK + 1) / 2;  // 21 entries of the S_kk triangle
constexpr int kIntrG = kKT;             // offset of J_k^T r~ in a point's part
constexpr int kIntrZc = kKT + kK;       // offset of Zk c
static_assert(kIntrZc + kK == kIntrPart, "per-point intrinsics part layout");

struct IntrArgs {
  int np, nf, n6;
  int nk;  // free params: 4 (pinhole) or 6 (EUCM)
  int64_t ng;
  const int64_t* pt_g_begin;
  const int64_t* g_begin;
  const int32_t* g_pose;
  const int32_t* g_pt;
  const int32_t* pose_fb;
  const int32_t* pt_mb;
  const float* pose_dd;
  const double* points;
  const float2* res;
  float huber;
  dd huber_dd;
  const double* intr;
  const float* cinv;
  const float* cvec;
  const float* zmat;
  const float* zdd;          // float-float Z of every term (float-float linearization) or null
  const float* zdd_flagged;  // float-float Z of flagged terms
  const int64_t* cam_g;
  const int64_t* tile_begin;
  const int64_t* tile_end;
  const int64_t* fb_tile_begin;
  double* ipart;  // np x kIntrPart
  float* zk;      // nm x kIntrZk: Zk (6x3) as (hi, lo)
  double* scj;    // nf x kIntrScj: S_kj (6x6)
  double* isum;   // kIntrPart sums, then -sum J_k^T r~ (6)
  double* S;
  float2* S2;
  double* rb;
  int fail_check;
};

// The observation's projection Jacobians: J_p, J_m as jacobians_dd and J_k
// (2x6 row-major, columns nk..5 zero).
__device__ void intr_term_jacobians(const float* Pd, dd px, dd py, dd pz, const CamD& c, int nk, JacD* J, dd* jk) {
  dd R[9], t[3];
  for (int i = 0; i < 9; ++i) R[i] = dd_make(Pd[2 * i], Pd[2 * i + 1]);
  for (int i = 0; i < 3; ++i) t[i] = dd_make(Pd[18 + 2 * i], Pd[18 + 2 * i + 1]);
  const dd xc = dd_add(dd_add(dd_add(dd_mul(R[0], px), dd_mul(R[1], py)), dd_mul(R[2], pz)), t[0]);
  const dd yc = dd_add(dd_add(dd_add(dd_mul(R[3], px), dd_mul(R[4], py)), dd_mul(R[5], pz)), t[1]);
  const dd zc = dd_add(dd_add(dd_add(dd_mul(R[6], px), dd_mul(R[7], py)), dd_mul(R[8], pz)), t[2]);
  const dd x = dd_div(xc, zc), y = dd_div(yc, zc);
  const dd zero = dd_make(0.f, 0.f), mone = dd_make(-1.0f, 0.0f);
  for (int k = 0; k < 2 * kK; ++k) jk[k] = zero;
  jk[2] = mone;
  jk[kK + 3] = mone;
  if (nk == 6) {
    dd rho, r2;
    const dd nrm = eucm_norm_dd(c, x, y, &rho, &r2);
    const dd in2 = dd_div(dd_make(1.0f, 0.0f), dd_mul(nrm, nrm));
    const dd da = dd_mul(dd_sub(rho, dd_make(1.0f, 0.0f)), in2);                        // (rho - 1) / norm^2
    const dd db = dd_div(dd_mul(dd_mul(c.alpha, r2), in2), dd_add(rho, rho));        // alpha r2 / (2 rho norm^2)
    jk[0] = dd_neg(dd_div(x, nrm));
    jk[kK + 1] = dd_neg(dd_div(y, nrm));
    const dd fxx = dd_mul(c.fx, x), fyy = dd_mul(c.fy, y);
    jk[4] = dd_mul(fxx, da);
    jk[5] = dd_mul(fxx, db);
    jk[kK + 4] = dd_mul(fyy, da);
    jk[kK + 5] = dd_mul(fyy, db);
  } else {
    jk[0] = dd_neg(x);
    jk[kK + 1] = dd_neg(y);
  }
  if (nk == 6) jacobians_dd<true>(Pd, px, py, pz, c, J);
  else jacobians_dd<false>(Pd, px, py, pz, c, J);
}

// One thread per point: its terms' J_k^T J_k, J_k^T r~, Y = J_k^T J_m, then
// with the point's C^-1 (landmark pass) Zk = Y C^-T and its parts of S_kk and
// rhs_k.
__global__ void __launch_bounds__(128) k_intr_points(IntrArgs a, const Ctrl* ctrl) {
  if (halted(ctrl)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.np) return;
  const CamD cam = cam_dd(a.intr);
  const dd px = dd_from_double(a.points[3 * i]), py = dd_from_double(a.points[3 * i + 1]),
           pz = dd_from_double(a.points[3 * i + 2]);
  dd hkk[kKT], gk[kK], Y[3 * kK];
  for (int k = 0; k < kKT; ++k) hkk[k] = dd_make(0.f, 0.f);
  for (int k = 0; k < kK; ++k) gk[k] = dd_make(0.f, 0.f);
  for (int k = 0; k < 3 * kK; ++k) Y[k] = dd_make(0.f, 0.f);
  for (int64_t g = a.pt_g_begin[i]; g < a.pt_g_begin[i + 1]; ++g) {
    JacD J;
    dd jk[2 * kK];
    intr_term_jacobians(a.pose_dd + 24 * a.g_pose[g], px, py, pz, cam, a.nk, &J, jk);
    for (int64_t o = a.g_begin[g]; o < a.g_begin[g + 1]; ++o) {
      const float2 r = a.res[o];
      dd r0, r1;
      huber_weighted_dd(a.huber, a.huber_dd, dd_from_float(r.x), dd_from_float(r.y), &r0, &r1);
      int k = 0;
      for (int p = 0; p < kK; ++p) {
        for (int q = p; q < kK; ++q) {
          hkk[k] = dd_add(hkk[k], dd_add(dd_mul(jk[p], jk[q]), dd_mul(jk[kK + p], jk[kK + q])));
          ++k;
        }
        gk[p] = dd_add(gk[p], dd_add(dd_mul(jk[p], r0), dd_mul(jk[kK + p], r1)));
        for (int s2 = 0; s2 < 3; ++s2)
          Y[p * 3 + s2] = dd_add(Y[p * 3 + s2], dd_add(dd_mul(jk[p], J.jm[s2]), dd_mul(jk[kK + p], J.jm[3 + s2])));
      }
    }
  }
  double* out = a.ipart + static_cast<int64_t>(i) * kIntrPart;
  const int mb = a.pt_mb[i];
  dd zz[kKT], zc[kK];
  for (int k = 0; k < kKT; ++k) zz[k] = dd_make(0.f, 0.f);
  for (int k = 0; k < kK; ++k) zc[k] = dd_make(0.f, 0.f);
  if (mb >= 0 && a.pt_g_begin[i + 1] > a.pt_g_begin[i]) {
    const float* cp = a.cinv + 12 * mb;
    dd I[6];
    for (int k = 0; k < 6; ++k) I[k] = dd_make(cp[2 * k], cp[2 * k + 1]);
    const float* cv = a.cvec + 6 * mb;
    const dd c[3] = {dd_make(cv[0], cv[1]), dd_make(cv[2], cv[3]), dd_make(cv[4], cv[5])};
    dd Zk[3 * kK];
    for (int r = 0; r < kK; ++r) {
      Zk[r * 3 + 0] = dd_mul(I[0], Y[r * 3 + 0]);
      Zk[r * 3 + 1] = dd_add(dd_mul(I[1], Y[r * 3 + 0]), dd_mul(I[2], Y[r * 3 + 1]));
      Zk[r * 3 + 2] = dd_add(dd_add(dd_mul(I[3], Y[r * 3 + 0]), dd_mul(I[4], Y[r * 3 + 1])), dd_mul(I[5], Y[r * 3 + 2]));
    }
    int k = 0;
    for (int p = 0; p < kK; ++p) {
      for (int q = p; q < kK; ++q) {
        dd t = dd_make(0.f, 0.f);
        for (int s2 = 0; s2 < 3; ++s2) t = dd_add(t, dd_mul(Zk[p * 3 + s2], Zk[q * 3 + s2]));
        zz[k++] = t;
      }
      dd t = dd_make(0.f, 0.f);
      for (int s2 = 0; s2 < 3; ++s2) t = dd_add(t, dd_mul(Zk[p * 3 + s2], c[s2]));
      zc[p] = t;
    }
    float* zo = a.zk + kIntrZk * static_cast<int64_t>(mb);
    for (int k2 = 0; k2 < 3 * kK; ++k2) {
      zo[2 * k2] = Zk[k2].hi;
      zo[2 * k2 + 1] = Zk[k2].lo;
    }
  }
  for (int k = 0; k < kKT; ++k) out[k] = dd_to_double(dd_sub(hkk[k], zz[k]));
  for (int k = 0; k < kK; ++k) out[kIntrG + k] = dd_to_double(gk[k]);
  for (int k = 0; k < kK; ++k) out[kIntrZc + k] = dd_to_double(zc[k]);
}

// One CTA: the per-point parts summed in a fixed order; the intrinsics'
// neg_grad -sum J_k^T r~ joins the gradient-tolerance maximum.
__global__ void __launch_bounds__(256) k_intr_reduce(IntrArgs a, Ctrl* ctrl) {
  if (halted(ctrl)) return;
  __shared__ float sh_hi[256], sh_lo[256];
  for (int k = 0; k < kIntrPart; ++k) {
    dd acc = dd_make(0.f, 0.f);
    for (int i = threadIdx.x; i < a.np; i += blockDim.x)
      acc = dd_add(acc, dd_from_double(a.ipart[static_cast<int64_t>(i) * kIntrPart + k]));
    sh_hi[threadIdx.x] = acc.hi;
    sh_lo[threadIdx.x] = acc.lo;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
      if (threadIdx.x < h) {
        const dd t = dd_add(dd_make(sh_hi[threadIdx.x], sh_lo[threadIdx.x]),
                            dd_make(sh_hi[threadIdx.x + h], sh_lo[threadIdx.x + h]));
        sh_hi[threadIdx.x] = t.hi;
        sh_lo[threadIdx.x] = t.lo;
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) a.isum[k] = dd_to_double(dd_make(sh_hi[0], sh_lo[0]));
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double mg = 0.0;
    for (int k = 0; k < kK; ++k) {
      const double bk = -a.isum[kIntrG + k];
      a.isum[kIntrPart + k] = bk;
      mg = fmax(mg, fabs(bk));
    }
    atomic_max_nonneg(&ctrl->max_grad_bits, mg);
  }
}

// One CTA per free pose: S_kj = sum over its terms of J_k^T J_p - Zk_i Z_g^T.
// Thread t < nk * 6 of the final sum owns entry t (row t / 6 of S_kj).
__global__ void __launch_bounds__(128) k_intr_cams(IntrArgs a, const Ctrl* ctrl) {
  if (halted(ctrl)) return;
  const int fb = blockIdx.x;
  constexpr int kE = kK * 6;
  __shared__ float sh_hi[kE][129], sh_lo[kE][129];
  dd acc[kE];
  for (int k = 0; k < kE; ++k) acc[k] = dd_make(0.f, 0.f);
  const CamD cam = cam_dd(a.intr);
  const int64_t t0 = a.fb_tile_begin[fb], t1 = a.fb_tile_begin[fb + 1];
  const int64_t e0 = (t1 > t0) ? a.tile_begin[t0] : 0, e1 = (t1 > t0) ? a.tile_end[t1 - 1] : 0;
  for (int64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const int64_t g = a.cam_g[e];
    const int i = a.g_pt[g];
    const dd px = dd_from_double(a.points[3 * i]), py = dd_from_double(a.points[3 * i + 1]),
             pz = dd_from_double(a.points[3 * i + 2]);
    JacD J;
    dd jk[2 * kK];
    intr_term_jacobians(a.pose_dd + 24 * a.g_pose[g], px, py, pz, cam, a.nk, &J, jk);
    for (int64_t o = a.g_begin[g]; o < a.g_begin[g + 1]; ++o)
      for (int p = 0; p < kK; ++p)
        for (int q = 0; q < 6; ++q)
          acc[p * 6 + q] = dd_add(acc[p * 6 + q], dd_add(dd_mul(jk[p], J.jp[q]), dd_mul(jk[kK + p], J.jp[6 + q])));
    const int mb = a.pt_mb[i];
    if (mb >= 0) {
      // Z_g (6x3): float-float where the landmark pass kept it so, else FP32
      dd Z[18];
      const float4* z4 = reinterpret_cast<const float4*>(a.zmat + 20 * g);
      float zf[20];
      for (int k = 0; k < 5; ++k) {
        const float4 w4 = z4[k];
        zf[4 * k] = w4.x; zf[4 * k + 1] = w4.y; zf[4 * k + 2] = w4.z; zf[4 * k + 3] = w4.w;
      }
      const float* zd = a.zdd ? a.zdd + kZddFloats * g : ((zf[18] != 0.f && a.zdd_flagged) ? a.zdd_flagged + kZddFloats * g : nullptr);
      for (int k = 0; k < 18; ++k) Z[k] = zd ? dd_make(zd[2 * k], zd[2 * k + 1]) : dd_from_float(zf[k]);
      const float* zk = a.zk + kIntrZk * static_cast<int64_t>(mb);
      for (int p = 0; p < kK; ++p)
        for (int q = 0; q < 6; ++q) {
          dd t = dd_make(0.f, 0.f);
          for (int s2 = 0; s2 < 3; ++s2)
            t = dd_add(t, dd_mul(dd_make(zk[2 * (p * 3 + s2)], zk[2 * (p * 3 + s2) + 1]), Z[q * 3 + s2]));
          acc[p * 6 + q] = dd_sub(acc[p * 6 + q], t);
        }
    }
  }
  for (int k = 0; k < kE; ++k) {
    sh_hi[k][threadIdx.x] = acc[k].hi;
    sh_lo[k][threadIdx.x] = acc[k].lo;
  }
  __syncthreads();
  if (threadIdx.x < kE) {
    const int k = threadIdx.x;
    dd t = dd_make(0.f, 0.f);
    for (int q = 0; q < static_cast<int>(blockDim.x); ++q) t = dd_add(t, dd_make(sh_hi[k][q], sh_lo[k][q]));
    a.scj[kIntrScj * static_cast<int64_t>(fb) + k] = dd_to_double(t);
  }
}

// The intrinsics rows of S (block nf, both triangles) and of the reduced rhs:
// blocks 0..nf-1 write S_kj, block nf the damped S_kk (rows nk..5 an identity).
__global__ void __launch_bounds__(64) k_intr_fill(IntrArgs a, const Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  const int b = blockIdx.x;
  const int k0 = 6 * a.nf;
  const int e = threadIdx.x;
  if (e >= 36) return;
  const int r = e / 6, c = e % 6;
  if (b < a.nf) {
    const double v = (r < a.nk) ? a.scj[kIntrScj * static_cast<int64_t>(b) + r * 6 + c] : 0.0;
    const int64_t row = k0 + r, col = 6 * b + c;
    a.S[row * a.n6 + col] = v;
    a.S[col * a.n6 + row] = v;
    if (a.S2) {
      const dd vd = dd_from_double(v);
      a.S2[row * a.n6 + col] = make_float2(vd.hi, vd.lo);
      a.S2[col * a.n6 + row] = make_float2(vd.hi, vd.lo);
    }
  } else {
    double v;
    if (r < a.nk && c < a.nk) {
      const int p = r < c ? r : c, q = r < c ? c : r;
      const int idx = p * kK - p * (p - 1) / 2 + (q - p);
      v = a.isum[idx];
      if (r == c) v += ctrl->nu * static_cast<double>(a.ng);
    } else {
      v = (r == c) ? 1.0 : 0.0;
    }
    const int64_t row = k0 + r, col = k0 + c;
    a.S[row * a.n6 + col] = v;
    if (a.S2) {
      const dd vd = dd_from_double(v);
      a.S2[row * a.n6 + col] = make_float2(vd.hi, vd.lo);
    }
    if (c == 0) a.rb[k0 + r] = (r < a.nk) ? a.isum[kIntrPart + r] - a.isum[kIntrZc + r] : 0.0;
  }
}

IntrArgs intr_args(const Sizes& s, const Dev& d) {
  IntrArgs a;
  a.np = s.np;
  a.nf = s.nf;
  a.n6 = s.n6;
  a.nk = s.intr_nk;
  a.ng = s.ng;
  a.pt_g_begin = d.pt_g_begin;
  a.g_begin = d.g_begin;
  a.g_pose = d.g_pose;
  a.g_pt = d.g_pt;
  a.pose_fb = d.pose_fb;
  a.pt_mb = d.pt_mb;
  a.pose_dd = d.pose_dd;
  a.points = d.points;
  a.res = d.res;
  a.huber = static_cast<float>(s.huber > 0 ? s.huber : 0.0);
  a.huber_dd = dd_make(static_cast<float>(s.huber), static_cast<float>(s.huber - static_cast<float>(s.huber)));
  a.intr = d.intr;
  a.cinv = d.cinv;
  a.cvec = d.cvec;
  a.zmat = d.zmat;
  a.zdd = s.lin_dd ? d.zdd : nullptr;
  a.zdd_flagged = d.zdd;
  a.cam_g = d.cam_g;
  a.tile_begin = d.tile_begin;
  a.tile_end = d.tile_end;
  a.fb_tile_begin = d.fb_tile_begin;
  a.ipart = d.intr_part;
  a.zk = d.intr_zk;
  a.scj = d.intr_scj;
  a.isum = d.intr_sum;
  a.S = d.S;
  a.S2 = d.S2;
  a.rb = d.rb;
  a.fail_check = 0;
  return a;
}

int launch_intr_linearize(const Sizes& s, const Dev& d, cudaStream_t st) {
  if (!s.intr_free) return 0;
  const IntrArgs a = intr_args(s, d);
  k_intr_points<<<(s.np + 127) / 128 > 0 ? (s.np + 127) / 128 : 1, 128, 0, st>>>(a, d.ctrl);
  k_intr_reduce<<<1, 256, 0, st>>>(a, d.ctrl);
  if (s.nf > 0) k_intr_cams<<<s.nf, 128, 0, st>>>(a, d.ctrl);
  return s.nf > 0 ? 3 : 2;
}

int launch_intr_fill(const Sizes& s, const Dev& d, cudaStream_t st) {
  if (!s.intr_free) return 0;
  const IntrArgs a = intr_args(s, d);
  k_intr_fill<<<s.nf + 1, 64, 0, st>>>(a, d.ctrl);
  return 1;
}

// ---------------------------------------------------------------------------
// Gauge projection.  With a single constant camera (center c) and no constant
// points, s -> scale about c is an exact symmetry of the cost, so H v = 0 for
// v = ([0; t_j - c] per free pose, p_i - c per point) and b . v = 0.  The exact
// damped step therefore satisfies v^T D delta = 0, D = diag(n_terms).  The
// FP32 assembly leaves a spurious component in the pose step along the weak
// direction v_f of S, amplified by 1/(nu n); the back-substitution carries it
// into the points as u_m = -V^-1 W^T v_f.  For a point determined by its views
// u_m = v_m to O(nu); for a point seen only by the constant camera u_m = 0, and
// for a point seen once u_m lacks its depth component (its damped block
// forgets the gauge direction there).  So the spurious part is alpha u with
// u = (v_f, u_m), and alpha = v^T D delta / v^T D u removes it while keeping
// the exact identity v^T D delta = 0.
// ---------------------------------------------------------------------------
struct GaugeArgs {
  int nf, nm;
  const int32_t* fb_pose;
  const int32_t* mb_pt;
  const double* poses;
  const double* points;
  const double* cnt_f;
  const double* cnt_m;
  const double* xf;
  const double* dm;
  const double* um;  // back-substituted gauge direction of the points
  double cx, cy, cz;
  double* part;  // 2 * gridDim
};

__device__ __forceinline__ void gauge_partials_body(GaugeArgs a, const Ctrl* ctrl, int bid_, int nblk_) {
  if (skipping(ctrl)) return;
  dd num = dd_make(0.f, 0.f), den = dd_make(0.f, 0.f);
  const int64_t n = static_cast<int64_t>(a.nf) + a.nm;
  for (int64_t t = bid_ * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < n;
       t += static_cast<int64_t>(nblk_) * blockDim.x) {
    double v[3], u[3], d[3], w;
    if (t < a.nf) {
      const double* T = a.poses + 7 * a.fb_pose[t];
      v[0] = T[4] - a.cx; v[1] = T[5] - a.cy; v[2] = T[6] - a.cz;
      u[0] = v[0]; u[1] = v[1]; u[2] = v[2];
      d[0] = a.xf[6 * t + 3]; d[1] = a.xf[6 * t + 4]; d[2] = a.xf[6 * t + 5];
      w = a.cnt_f[t];
    } else {
      const int mb = static_cast<int>(t - a.nf);
      const double* p = a.points + 3 * a.mb_pt[mb];
      v[0] = p[0] - a.cx; v[1] = p[1] - a.cy; v[2] = p[2] - a.cz;
      u[0] = a.um[3 * mb]; u[1] = a.um[3 * mb + 1]; u[2] = a.um[3 * mb + 2];
      d[0] = a.dm[3 * mb]; d[1] = a.dm[3 * mb + 1]; d[2] = a.dm[3 * mb + 2];
      w = a.cnt_m[mb];
    }
    dd wd = dd_from_double(w);
    for (int k = 0; k < 3; ++k) {
      dd vk = dd_from_double(v[k]);
      num = dd_add(num, dd_mul(dd_mul(wd, vk), dd_from_double(d[k])));
      den = dd_add(den, dd_mul(dd_mul(wd, vk), dd_from_double(u[k])));
    }
  }
  __shared__ float sh[4][8];
  num = dd_warp_sum(num);
  den = dd_warp_sum(den);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) { sh[0][w] = num.hi; sh[1][w] = num.lo; sh[2][w] = den.hi; sh[3][w] = den.lo; }
  __syncthreads();
  if (threadIdx.x == 0) {
    dd s0 = dd_make(0.f, 0.f), s1 = dd_make(0.f, 0.f);
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
      s0 = dd_add(s0, dd_make(sh[0][q], sh[1][q]));
      s1 = dd_add(s1, dd_make(sh[2][q], sh[3][q]));
    }
    a.part[2 * bid_] = dd_to_double(s0);
    a.part[2 * bid_ + 1] = dd_to_double(s1);
  }
}
__global__ void __launch_bounds__(256) k_gauge_partials(GaugeArgs a, const Ctrl* ctrl) {
  gauge_partials_body(a, ctrl, blockIdx.x, gridDim.x);
}


// ---------------------------------------------------------------------------
// Apply the (projected) step: trial poses exp(delta) * T, trial points p + d
// (VarFamilies::update, crates/sophus_opt/src/variables/var_families.rs:203-209);
// partial sums of delta.delta and delta.neg_grad for the gain ratio and max |delta|.
// ---------------------------------------------------------------------------
struct UpdArgs {
  int nc, np, nf, nm;
  const int32_t* pose_fb;
  const int32_t* pt_mb;
  const double* poses;
  const double* points;
  double* poses_t;
  double* points_t;
  double* xf;   // projected in place
  double* dm;   // projected in place
  const double* bf;
  const double* bm;
  int gauge_kind;
  double cx, cy, cz;
  double* part;  // 2 * gridDim
  const double* gauge_part;  // 2 * gauge_blocks partial sums of the gauge projection
  int gauge_blocks;
  const double* um;          // the points' part of the projection direction
  float* pose_f;   // trial pose tables, written here for the trial cost
  float* pose_dd;
  // free intrinsics: k_t = k + dx_k (dx_k at xf[6 nf .. 6 nf + nk - 1]), neg_grad bk
  int intr_free;
  int intr_nk;
  const double* intr;
  double* intr_t;
  const double* bk;
};

__device__ __forceinline__ void apply_update_body(UpdArgs a, Ctrl* ctrl, int bid_, int nblk_) {
  if (skipping(ctrl)) return;
  // gauge coefficient alpha = sum num / sum den over the k_gauge_partials
  // blocks, formed identically in every CTA (fixed order, warp 0)
  __shared__ double s_alpha;
  double alpha = 0.0;
  if (a.gauge_kind == 1) {
    if (threadIdx.x < 32) {
      dd n = dd_make(0.f, 0.f), d = dd_make(0.f, 0.f);
      for (int q = threadIdx.x; q < a.gauge_blocks; q += 32) {
        n = dd_add(n, dd_from_double(a.gauge_part[2 * q]));
        d = dd_add(d, dd_from_double(a.gauge_part[2 * q + 1]));
      }
      n = dd_warp_sum(n);
      d = dd_warp_sum(d);
      if (threadIdx.x == 0) {
        const double sn = dd_to_double(n), sd = dd_to_double(d);
        s_alpha = (sd > 0.0) ? sn / sd : 0.0;
      }
    }
    __syncthreads();
    alpha = s_alpha;
    if (bid_ == 0 && threadIdx.x == 0) ctrl->alpha = alpha;
  }
  dd sdd = dd_make(0.f, 0.f), sdg = dd_make(0.f, 0.f);
  double mx = 0.0;
  if (a.intr_free && bid_ == 0 && threadIdx.x == 0) {
    // the intrinsics are a vector space: k + dx_k (no gauge component)
    for (int k = 0; k < a.intr_nk; ++k) {
      const double xk = a.xf[6 * a.nf + k];
      a.intr_t[k] = a.intr[k] + xk;
      const dd x = dd_from_double(xk);
      sdd = dd_add(sdd, dd_mul(x, x));
      sdg = dd_add(sdg, dd_mul(x, dd_from_double(a.bk[k])));
      mx = fmax(mx, fabs(xk));
    }
  }
  const int64_t n = static_cast<int64_t>(a.nc) + a.np;
  for (int64_t t = bid_ * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < n;
       t += static_cast<int64_t>(nblk_) * blockDim.x) {
    if (t < a.nc) {
      const int j = static_cast<int>(t);
      const double* T = a.poses + 7 * j;
      double* O = a.poses_t + 7 * j;
      const int fb = a.pose_fb[j];
      if (fb < 0) {
        for (int k = 0; k < 7; ++k) O[k] = T[k];
        pose_table(O, a.pose_f + 12 * j, a.pose_dd + 24 * j);
        continue;
      }
      double xi[6];
      for (int k = 0; k < 6; ++k) xi[k] = a.xf[6 * fb + k];
      xi[3] -= alpha * (T[4] - a.cx);
      xi[4] -= alpha * (T[5] - a.cy);
      xi[5] -= alpha * (T[6] - a.cz);
      for (int k = 0; k < 6; ++k) {
        a.xf[6 * fb + k] = xi[k];
        dd x = dd_from_double(xi[k]);
        sdd = dd_add(sdd, dd_mul(x, x));
        sdg = dd_add(sdg, dd_mul(x, dd_from_double(a.bf[6 * fb + k])));
        mx = fmax(mx, fabs(xi[k]));
      }
      se3_left_update(xi, T, O);
      pose_table(O, a.pose_f + 12 * j, a.pose_dd + 24 * j);
    } else {
      const int i = static_cast<int>(t - a.nc);
      const double* p = a.points + 3 * i;
      double* O = a.points_t + 3 * i;
      const int mb = a.pt_mb[i];
      if (mb < 0) {
        O[0] = p[0]; O[1] = p[1]; O[2] = p[2];
        continue;
      }
      double d[3] = {a.dm[3 * mb], a.dm[3 * mb + 1], a.dm[3 * mb + 2]};
      if (a.gauge_kind == 1) {
        d[0] -= alpha * a.um[3 * mb];
        d[1] -= alpha * a.um[3 * mb + 1];
        d[2] -= alpha * a.um[3 * mb + 2];
      }
      for (int k = 0; k < 3; ++k) {
        a.dm[3 * mb + k] = d[k];
        dd x = dd_from_double(d[k]);
        sdd = dd_add(sdd, dd_mul(x, x));
        sdg = dd_add(sdg, dd_mul(x, dd_from_double(a.bm[3 * mb + k])));
        mx = fmax(mx, fabs(d[k]));
        O[k] = p[k] + d[k];
      }
    }
  }
  __shared__ float sh[4][8];
  __shared__ double shm[8];
  sdd = dd_warp_sum(sdd);
  sdg = dd_warp_sum(sdg);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
    sh[0][w] = sdd.hi; sh[1][w] = sdd.lo; sh[2][w] = sdg.hi; sh[3][w] = sdg.lo;
    shm[w] = mx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    dd s0 = dd_make(0.f, 0.f), s1 = dd_make(0.f, 0.f);
    double m = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
      s0 = dd_add(s0, dd_make(sh[0][q], sh[1][q]));
      s1 = dd_add(s1, dd_make(sh[2][q], sh[3][q]));
      m = fmax(m, shm[q]);
    }
    a.part[2 * bid_] = dd_to_double(s0);
    a.part[2 * bid_ + 1] = dd_to_double(s1);
    atomic_max_nonneg(&ctrl->max_step_bits, m);
  }
}
__global__ void __launch_bounds__(256) k_apply_update(UpdArgs a, Ctrl* ctrl) {
  apply_update_body(a, ctrl, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------------------
// LM decision (step_nlls_inner, crates/sophus_opt/src/nlls/optimizer_step.rs:366-437;
// accept/reject optimizer.rs:463-480; gain ratio optimizer_helpers.rs:159-173).
// ---------------------------------------------------------------------------
__device__ void decide_body(const double* cost_part, int n_cost, const double* upd_part, int n_upd, Ctrl* ctrl,
                            Record* recs, Record* last) {
  const int skip = ctrl->skip;
  double new_merit = 0.0;
  if (skip == 0) new_merit = block_sum_partials(cost_part, n_cost);
  __shared__ double s_dd, s_dg;
  if (skip == 0 && threadIdx.x < 32) {
    dd a = dd_make(0.f, 0.f), b = dd_make(0.f, 0.f);
    for (int q = threadIdx.x; q < n_upd; q += 32) {
      a = dd_add(a, dd_from_double(upd_part[2 * q]));
      b = dd_add(b, dd_from_double(upd_part[2 * q + 1]));
    }
    a = dd_warp_sum(a);
    b = dd_warp_sum(b);
    if (threadIdx.x == 0) {
      s_dd = dd_to_double(a);
      s_dg = dd_to_double(b);
    }
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  Record rec;
  rec.new_merit = nan;
  rec.gain_ratio = nan;
  rec.max_step = nan;
  rec.accepted = 0;
  rec.max_grad = ctrl->max_grad;
  int reason = 0;
  ctrl->accept = 0;
  if (skip == 1) {
    reason = 1 + 1;  // GradientTolerance
  } else if (skip == 2) {
    ctrl->nu *= 2.0;  // handle_solve_failure -> reject_step
    ctrl->rejects += 1;
    if (ctrl->rejects >= ctrl->max_rejects) reason = 5;
  } else {
    const double merit = ctrl->merit;
    const double max_step = __longlong_as_double(static_cast<long long>(ctrl->max_step_bits));
    rec.new_merit = new_merit;
    rec.max_step = max_step;
    ctrl->new_merit = new_merit;
    ctrl->max_step = max_step;
    ctrl->dd_sum = s_dd;
    ctrl->dg_sum = s_dg;
    if (max_step < ctrl->ptol) {
      if (new_merit < merit) {
        ctrl->accept = 1;
        ctrl->merit = new_merit;
        rec.accepted = 1;
        for (int k = 0; k < ctrl->n_eq; ++k) ctrl->eq_lambda[k] -= ctrl->eq_dlam[k];  // update_lambdas
      }
      reason = 3;  // ParameterTolerance
    } else {
      const double predicted = ctrl->nu * s_dd + s_dg;
      const double actual = merit - new_merit;
      const double min_pos = 2.2250738585072014e-308;
      double rho = (fabs(predicted) > min_pos) ? actual / predicted : (actual > 0.0 ? 1.0 : 0.0);
      rec.gain_ratio = rho;
      ctrl->gain_ratio = rho;
      if (rho > 0.0 && new_merit < merit) {
        double x = 2.0 * rho - 1.0;
        double f = 1.0 - x * x * x;
        ctrl->nu *= fmax(f, 1.0 / 3.0);
        ctrl->rejects = 0;
        double rel = (merit - new_merit) / (fabs(merit) + min_pos);
        if (rel < ctrl->ftol) reason = 1;  // FunctionTolerance
        ctrl->accept = 1;
        ctrl->merit = new_merit;
        rec.accepted = 1;
        for (int k = 0; k < ctrl->n_eq; ++k) ctrl->eq_lambda[k] -= ctrl->eq_dlam[k];  // update_lambdas
      } else {
        ctrl->nu *= 2.0;
        ctrl->rejects += 1;
        if (ctrl->rejects >= ctrl->max_rejects) reason = 5;
      }
    }
  }
  ctrl->step += 1;
  if (ctrl->step >= ctrl->num_iterations && reason == 0) reason = 4;  // MaxIterations
  rec.merit = ctrl->merit;
  rec.lm_damping = ctrl->nu;
  rec.termination = reason;
  ctrl->termination = reason;
  if (ctrl->step - 1 < ctrl->record_cap) recs[ctrl->step - 1] = rec;
  *last = rec;
  if (reason != 0) ctrl->done = 1;
}

// Accepted step: trial state becomes the current state.
__device__ __forceinline__ void commit_body(int nc, int np, int64_t no, const double* poses_t, double* poses,
                         const double* points_t, double* points, const float2* res_t, float2* res,
                         const float2* res_lo_t, float2* res_lo, const double* intr_t, double* intr,
                         const Ctrl* ctrl, int bid_, int nblk_) {
  if (!ctrl->accept) return;
  const int64_t stride = static_cast<int64_t>(nblk_) * blockDim.x;
  const int64_t t0 = bid_ * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (intr && t0 < kIntrMax) intr[t0] = intr_t[t0];
  for (int64_t t = t0; t < no; t += stride) res[t] = res_t[t];
  if (res_lo)
    for (int64_t t = t0; t < no; t += stride) res_lo[t] = res_lo_t[t];
  for (int64_t t = t0; t < 7 * static_cast<int64_t>(nc); t += stride) poses[t] = poses_t[t];
  for (int64_t t = t0; t < 3 * static_cast<int64_t>(np); t += stride) points[t] = points_t[t];
}
__global__ void k_commit(int nc, int np, int64_t no, const double* poses_t, double* poses,
                         const double* points_t, double* points, const float2* res_t, float2* res,
                         const float2* res_lo_t, float2* res_lo, const double* intr_t, double* intr,
                         const Ctrl* ctrl) {
  commit_body(nc, np, no, poses_t, poses, points_t, points, res_t, res, res_lo_t, res_lo, intr_t, intr, ctrl, blockIdx.x, gridDim.x);
}

int cost_grid(int64_t no) {
  int64_t b = (no + kCostThreads - 1) / kCostThreads;
  if (b < 1) b = 1;
  if (b > kCostMaxBlocks) b = kCostMaxBlocks;
  return static_cast<int>(b);
}

int warp_grid(int64_t items, int warps_per_block, int cap) {
  int64_t b = (items + warps_per_block - 1) / warps_per_block;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return static_cast<int>(b);
}

constexpr int kUpdBlocks = 152;

// CTAs of the update and gauge kernels: kUpdBlocks, or one per 256 poses and
// points for small problems (local windows), whose update is a few thousand
// items spread over 152 nearly idle CTAs otherwise.
int upd_blocks(const Sizes& s) {
  const int64_t items = static_cast<int64_t>(s.nc) + s.np;
  if (items > 16384) return kUpdBlocks;
  const int64_t b = (items + 255) / 256;
  return b < 1 ? 1 : static_cast<int>(b);
}

}  // namespace

// partials: gauge (2 per block), update (2 per block, then the constraints'
// slot), cost (one per block, then the priors' and the edges')
constexpr int kCostPartOff = 4 * kUpdBlocks + 2;
int cost_partials_needed(const Sizes& s) { return kCostPartOff + cost_grid(s.no) + 2; }

int launch_pose_tables(const Sizes& s, const Dev& d, const double* poses, cudaStream_t st) {
  k_pose_tables<<<(s.nc + 127) / 128, 128, 0, st>>>(s.nc, poses, d.pose_f, d.pose_dd, d.ctrl, 0, nullptr, nullptr);
  return 1;
}

static CostArgs make_cost_args(const Sizes& s, const Dev& d, const double* points, float2* res_out,
                               double* partials, int respect_skip) {
  CostArgs a;
  a.res_lo_out = (res_out == d.res) ? d.res_lo : (res_out == d.res_t ? d.res_lo_t : nullptr);
  a.no = s.no;
  a.uv = d.obs_uv;
  a.opose = d.obs_pose;
  a.opt = d.obs_pt;
  a.pose_dd = d.pose_dd;
  a.points = points;
  a.res_out = res_out;
  a.partials = partials;
  a.fx = a.fy = a.cx = a.cy = dd_make(0.f, 0.f);
  a.intr = (points == d.points_t) ? d.intr_t : d.intr;  // the trial point's intrinsics
  a.huber = static_cast<float>(s.huber > 0 ? s.huber : 0.0);
  a.huber_dd = dd_make(static_cast<float>(s.huber), static_cast<float>(s.huber - static_cast<float>(s.huber)));
  a.respect_skip = respect_skip;
  a.decide = nullptr;
  a.upd_part = nullptr;
  a.n_upd = 0;
  a.recs = nullptr;
  a.last = nullptr;
  a.n_extra = 0;
  return a;
}

int launch_cost(const Sizes& s, const Dev& d, const double* poses, const double* points,
                float2* res_out, double* partials, cudaStream_t st) {
  k_pose_tables<<<(s.nc + 127) / 128, 128, 0, st>>>(s.nc, poses, d.pose_f, d.pose_dd, d.ctrl, 1, nullptr, nullptr);
  CostArgs a = make_cost_args(s, d, points, res_out, partials, 1);
  (s.eucm ? k_cost<true> : k_cost<false>)<<<cost_grid(s.no), kCostThreads, 0, st>>>(a, d.ctrl);
  return 2;
}

int launch_init_merit(const Sizes& s, const Dev& d, cudaStream_t st) {
  k_pose_tables<<<(s.nc + 127) / 128, 128, 0, st>>>(s.nc, d.poses, d.pose_f, d.pose_dd, d.ctrl, 0, nullptr, nullptr);
  CostArgs a = make_cost_args(s, d, d.points, d.res, d.part, 0);
  const int nb = cost_grid(s.no);
  (s.eucm ? k_cost<true> : k_cost<false>)<<<nb, kCostThreads, 0, st>>>(a, d.ctrl);
  const int np = launch_prior_eval(s, d, d.poses, 0, 0, d.part + nb, st);
  const int ne = launch_edge_eval(s, d, d.poses, 0, 0, d.part + nb + np, st);
  k_init_merit<<<1, 256, 0, st>>>(d.part, nb + np + ne, d.ctrl);
  return 3 + np + ne;
}

int launch_iteration_begin(const Sizes& s, const Dev& d, cudaStream_t st) {
  // the iteration is opened by the first kernel of launch_linearize
  (void)s;
  (void)d;
  (void)st;
  return 0;
}

static LinArgs make_lin_args(const Sizes& s, const Dev& d, double nu_override, bool use_override) {
  LinArgs la;
  la.well_tol = s.lmk_well_tol;
  la.np = s.np;
  la.pt_g_begin = d.pt_g_begin;
  la.g_begin = d.g_begin;
  la.g_pose = d.g_pose;
  la.pose_fb = d.pose_fb;
  la.pt_mb = d.pt_mb;
  la.cnt_m = d.cnt_m;
  la.pose_f = d.pose_f;
  la.points = d.points;
  la.pose_dd = d.pose_dd;
  la.res = d.res;
  la.intr = d.intr;
  la.huber = static_cast<float>(s.huber > 0 ? s.huber : 0.0);
  la.huber_dd = dd_make(static_cast<float>(s.huber), static_cast<float>(s.huber - static_cast<float>(s.huber)));
  la.zmat = d.zmat;
  la.cinv = d.cinv;
  la.cvec = d.cvec;
  la.bm = d.bm;
  la.nu_override = nu_override;
  la.use_override = use_override ? 1 : 0;
  la.nu_ctrl = 0;
  la.fail = &d.ctrl->fail;
  la.g_pt = d.g_pt;
  la.list = nullptr;
  la.list_count = nullptr;
  la.chunk_pt = d.lmk_chunk_pt;
  la.nchunk = s.nlchunk;
  la.slow_list = d.slow_list;
  la.slow_count = d.slow_count;
  la.force_dd = s.lin_dd;
  la.res_lo = s.lin_dd ? d.res_lo : nullptr;
  la.zdd = d.zdd;
  return la;
}

static CamArgs make_cam_args(const Sizes& s, const Dev& d, int with_schur) {
  CamArgs ca;
  ca.tile_fb = d.tile_fb;
  ca.tile_begin = d.tile_begin;
  ca.tile_end = d.tile_end;
  ca.cam_g = d.cam_g;
  ca.g_begin = d.g_begin;
  ca.g_pt = d.g_pt;
  ca.fb_pose = d.fb_pose;
  ca.pt_mb = d.pt_mb;
  ca.pose_f = d.pose_f;
  ca.points = d.points;
  ca.res = d.res;
  ca.zmat = d.zmat;
  ca.cvec = d.cvec;
  ca.intr = d.intr;
  ca.huber = static_cast<float>(s.huber > 0 ? s.huber : 0.0);
  ca.tile_part = d.tile_part;
  ca.with_schur = with_schur;
  ca.pose_dd = d.pose_dd;
  ca.res_lo = d.res_lo;
  ca.zdd = d.zdd;
  ca.huber_dd = dd_make(static_cast<float>(s.huber), static_cast<float>(s.huber - static_cast<float>(s.huber)));
  return ca;
}

static int launch_camera(const Sizes& s, const Dev& d, int with_schur, cudaStream_t st) {
  if (s.ntiles == 0) return 0;
  const CamArgs ca = make_cam_args(s, d, with_schur);
  const unsigned nt = static_cast<unsigned>(s.ntiles);
  if (s.lin_dd) (s.eucm ? k_camera_tiles_dd<true> : k_camera_tiles_dd<false>)<<<nt, kTileThreads, 0, st>>>(ca, d.ctrl);
  else (s.eucm ? k_camera_tiles<true> : k_camera_tiles<false>)<<<nt, kTileThreads, 0, st>>>(ca, d.ctrl);
  return 1;
}

static BackArgs make_back_args(const Sizes& s, const Dev& d) {
  BackArgs b;
  b.np = s.np;
  b.pt_g_begin = d.pt_g_begin;
  b.g_pose = d.g_pose;
  b.pose_fb = d.pose_fb;
  b.pt_mb = d.pt_mb;
  b.zmat = d.zmat;
  b.zdd = s.lin_dd ? d.zdd : nullptr;
  b.zdd_flagged = d.zdd;
  b.cinv = d.cinv;
  b.cvec = d.cvec;
  b.xdd = d.xdd;
  b.dm = d.dm;
  b.gauge_kind = s.gauge_kind;
  b.poses = d.poses;
  b.cx = s.gauge_center[0];
  b.cy = s.gauge_center[1];
  b.cz = s.gauge_center[2];
  b.um = d.gauge_um;
  b.zk = s.intr_free ? d.intr_zk : nullptr;
  b.k0 = 6 * s.nf;
  return b;
}

static int launch_backsub(const Sizes& s, const Dev& d, cudaStream_t st) {
  const BackArgs b = make_back_args(s, d);
  if (s.nlchunk > 0 && s.bsub_chunks_ok) {
    const int grid = s.nlchunk < 8192 ? s.nlchunk : 8192;
    k_backsub_chunks<<<grid, 256, sizeof(float) * 12 * static_cast<size_t>(s.lmk_cap), st>>>(
        b, d.lmk_chunk_pt, s.nlchunk, d.g_pt, d.ctrl);
    return 1;
  }
  k_backsub<<<warp_grid(s.np, 8, 4096), 256, 0, st>>>(b, d.ctrl);
  return 1;
}

// Landmark pass: the chunked kernel plus the float-float redo of the points it
// queued, or (final Hessian pass, no chunk table, or the float-float
// linearization) the warp-per-point kernel.
static int launch_landmark(const Sizes& s, const Dev& d, LinArgs la, cudaStream_t st, bool zero_slow = true) {
  if (!la.use_override && s.nlchunk > 0 && s.lin_dd && s.lmk_dd_ok) {
    const int grid = s.nlchunk < 8192 ? s.nlchunk : 8192;
    const size_t smem = sizeof(float) * kLmkDDTermFloats * static_cast<size_t>(s.lmk_cap);
    (s.eucm ? k_landmark_chunks_dd<true> : k_landmark_chunks_dd<false>)<<<grid, 256, smem, st>>>(la, d.ctrl);
    return 1;
  }
  if (!la.use_override && s.nlchunk > 0 && !s.lin_dd) {
    if (zero_slow) cudaMemsetAsync(d.slow_count, 0, sizeof(int32_t), st);
    const int grid = s.nlchunk < 8192 ? s.nlchunk : 8192;
    const size_t smem = sizeof(float) * 9 * static_cast<size_t>(s.lmk_cap);
    (s.eucm ? k_landmark_chunks<true> : k_landmark_chunks<false>)<<<grid, 256, smem, st>>>(la, d.ctrl);
    LinArgs lb = la;
    lb.list = d.slow_list;
    lb.list_count = d.slow_count;
    (s.eucm ? k_landmark<true> : k_landmark<false>)<<<s.lmk_list_grid, 256, 0, st>>>(lb, d.ctrl);
    return 2;
  }
  const int wg = warp_grid(s.np, 8, s.lin_dd ? 16384 : 4096);
  (s.eucm ? k_landmark<true> : k_landmark<false>)<<<wg, 256, 0, st>>>(la, d.ctrl);
  return 1;
}

// Raises the dynamic shared memory limit of both camera-model instances.
template <class K>
static int raise_both(K pinhole, K eucm, size_t bytes) {
  return (raise_dynamic_smem(reinterpret_cast<const void*>(pinhole), bytes) == cudaSuccess &&
          raise_dynamic_smem(reinterpret_cast<const void*>(eucm), bytes) == cudaSuccess)
             ? 0
             : -1;
}

int landmark_setup(int cap) {
  const size_t bytes = sizeof(float) * 9 * static_cast<size_t>(cap);
  if (bytes <= 48 * 1024) return 0;
  return raise_both(k_landmark_chunks<false>, k_landmark_chunks<true>, bytes);
}

int backsub_chunks_setup(int cap) {
  const size_t bytes = sizeof(float) * 12 * static_cast<size_t>(cap);
  if (bytes > 200 * 1024) return -1;
  if (bytes <= 48 * 1024) return 0;
  return raise_dynamic_smem(reinterpret_cast<const void*>(k_backsub_chunks), bytes) == cudaSuccess ? 0 : -1;
}

int landmark_dd_setup(int cap) {
  const size_t bytes = sizeof(float) * kLmkDDTermFloats * static_cast<size_t>(cap);
  if (bytes > 200 * 1024) return -1;
  if (bytes <= 48 * 1024) return 0;
  return raise_both(k_landmark_chunks_dd<false>, k_landmark_chunks_dd<true>, bytes);
}

int launch_linearize(const Sizes& s, const Dev& d, double nu_override, bool use_override,
                     cudaStream_t st) {
  int n = 0;
  // an LM iteration (not the final linearisation) is opened here
  k_pose_tables<<<(s.nc + 127) / 128, 128, 0, st>>>(s.nc, d.poses, d.pose_f, d.pose_dd, d.ctrl, 0,
                                                    use_override ? nullptr : d.ctrl,
                                                    use_override ? nullptr : d.slow_count);
  ++n;
  n += launch_landmark(s, d, make_lin_args(s, d, nu_override, use_override), st, use_override);
  n += launch_intr_linearize(s, d, st);
  n += launch_camera(s, d, use_override ? 0 : 1, st);
  n += launch_prior_eval(s, d, d.poses, 1, 1, nullptr, st);
  n += launch_edge_eval(s, d, d.poses, 1, 1, nullptr, st);
  // the last block of the finalisation runs the gradient check of an LM iteration
  k_camera_finalize<<<s.nf, 64, 0, st>>>(s.nf, d.fb_tile_begin, d.tile_part, d.ufull, d.bf, d.rb, d.ctrl,
                                         use_override ? 0 : 1, s.n_prior > 0 ? d.prior_fb_begin : nullptr,
                                         d.prior_out, s.n_edge > 0 ? d.efb_begin : nullptr, d.efb_slot,
                                         d.edge_out);
  ++n;
  if (!use_override) n += launch_eq_eval(s, d, st);
  return n;
}

static SchurArgs make_schur_args(const Sizes& s, const Dev& d) {
  SchurArgs a;
  a.nsb = s.nsb;
  a.sb_row = d.sb_row;
  a.sb_col = d.sb_col;
  a.sb_pair_begin = d.sb_pair_begin;
  a.pairs = d.pairs;
  a.zmat = d.zmat;
  a.zdd = d.zdd;
  a.ufull = d.ufull;
  a.cnt_f = d.cnt_f;
  a.S = d.S;
  a.S2 = d.S2;
  a.n6 = s.n6;
  a.nchunk = s.nchunk;
  a.chunk_begin = d.chunk_begin;
  a.block_chunk_begin = d.block_chunk_begin;
  a.part = d.schur_part;
  a.eblk_begin = s.n_edge > 0 ? d.eblk_begin : nullptr;
  a.eblk_term = d.eblk_term;
  a.e_hmn = d.edge_hmn;
  return a;
}

static SchurDenseArgs make_schur_dense_args(const Sizes& s, const Dev& d) {
  SchurDenseArgs a;
  a.np = s.np;
  a.nf = s.nf;
  a.n6 = s.n6;
  a.zterm = d.zterm;
  a.zmat = d.zmat;
  a.ufull = d.ufull;
  a.cnt_f = d.cnt_f;
  a.S = d.S;
  a.S2 = d.S2;
  return a;
}

static int schur_dense_grid(const Sizes& s) {
  const int nb = (s.nf + kSdB - 1) / kSdB;
  return nb * (nb + 1) / 2;
}

int launch_schur(const Sizes& s, const Dev& d, cudaStream_t st) {
  if (s.schur_dense) {
    k_schur_dense<<<schur_dense_grid(s), kSdThreads, 0, st>>>(make_schur_dense_args(s, d), d.ctrl);
    return 1 + launch_intr_fill(s, d, st);
  }
  const SchurArgs a = make_schur_args(s, d);
  if (s.lin_dd) k_schur_dd<<<warp_grid(s.nchunk, 8, 65536), 256, 0, st>>>(a, d.ctrl);
  else k_schur<<<warp_grid(s.nchunk, 8, 65536), 256, 0, st>>>(a, d.ctrl);
  k_schur_reduce<<<warp_grid(s.nsb, 8, 8192), 256, 0, st>>>(a, d.ctrl);
  return 2 + launch_intr_fill(s, d, st);
}

static GaugeArgs make_gauge_args(const Sizes& s, const Dev& d) {
  GaugeArgs g;
  g.nf = s.nf;
  g.nm = s.nm;
  g.fb_pose = d.fb_pose;
  g.mb_pt = d.mb_pt;
  g.poses = d.poses;
  g.points = d.points;
  g.cnt_f = d.cnt_f;
  g.cnt_m = d.cnt_m;
  g.xf = d.x;
  g.dm = d.dm;
  g.um = d.gauge_um;
  g.cx = s.gauge_center[0];
  g.cy = s.gauge_center[1];
  g.cz = s.gauge_center[2];
  g.part = d.part;
  return g;
}

static UpdArgs make_upd_args(const Sizes& s, const Dev& d) {
  UpdArgs u;
  u.nc = s.nc;
  u.np = s.np;
  u.nf = s.nf;
  u.nm = s.nm;
  u.pose_fb = d.pose_fb;
  u.pt_mb = d.pt_mb;
  u.poses = d.poses;
  u.points = d.points;
  u.poses_t = d.poses_t;
  u.points_t = d.points_t;
  u.xf = d.x;
  u.dm = d.dm;
  u.bf = d.bf;
  u.bm = d.bm;
  u.gauge_kind = s.gauge_kind;
  u.cx = s.gauge_center[0];
  u.cy = s.gauge_center[1];
  u.cz = s.gauge_center[2];
  u.part = d.part + 2 * kUpdBlocks;
  u.gauge_part = d.part;
  u.gauge_blocks = upd_blocks(s);
  u.um = d.gauge_um;
  u.intr_free = s.intr_free;
  u.intr_nk = s.intr_nk;
  u.intr = d.intr;
  u.intr_t = d.intr_t;
  u.bk = d.intr_sum ? d.intr_sum + kIntrPart : nullptr;
  u.pose_f = d.pose_f;
  u.pose_dd = d.pose_dd;
  return u;
}

int launch_update(const Sizes& s, const Dev& d, cudaStream_t st) {
  int n = 0;
  n += launch_backsub(s, d, st);
  if (s.gauge_kind == 1) {
    k_gauge_partials<<<upd_blocks(s), 256, 0, st>>>(make_gauge_args(s, d), d.ctrl);
    n += 1;
  }
  k_apply_update<<<upd_blocks(s), 256, 0, st>>>(make_upd_args(s, d), d.ctrl);
  ++n;
  n += launch_eq_post(s, d, d.part + 2 * kUpdBlocks + 2 * upd_blocks(s), st);
  return n;
}

int launch_single(const Sizes& s, const Dev& d, int kernel_id, cudaStream_t st) {
  switch (kernel_id) {
    case 1:
      return launch_schur(s, d, st);
    case 2:
      return launch_landmark(s, d, make_lin_args(s, d, 0.0, false), st);
    case 3:
      return launch_camera(s, d, 1, st);
    case 4: {
      CostArgs a = make_cost_args(s, d, d.points_t, d.res_t, d.part + kCostPartOff, 1);
      (s.eucm ? k_cost<true> : k_cost<false>)<<<cost_grid(s.no), kCostThreads, 0, st>>>(a, d.ctrl);
      return 1;
    }
    case 5:
      return launch_factor_solve(s, d, st);
    case 6:
      return launch_backsub(s, d, st);
    default:
      return 0;
  }
}

// trial cost (partials after the update partials; the trial pose tables
// were written by k_apply_update); its last block runs the LM decision
static CostArgs make_decide_args(const Sizes& s, const Dev& d) {
  double* cost_part = d.part + kCostPartOff;
  CostArgs a = make_cost_args(s, d, d.points_t, d.res_t, cost_part, 1);
  a.decide = d.ctrl;
  a.upd_part = d.part + 2 * kUpdBlocks;
  a.n_upd = upd_blocks(s) + (s.n_eq > 0 ? 1 : 0);  // the constraints' slot after the blocks'
  a.recs = d.records;
  a.last = d.last_rec;
  return a;
}

static int commit_grid(const Sizes& s) {
  const int64_t big = s.no > 7 * (int64_t)s.nc ? s.no : 7 * (int64_t)s.nc;
  const int64_t items = big > 3 * (int64_t)s.np ? big : 3 * (int64_t)s.np;
  int cb = static_cast<int>((items + 255) / 256);
  if (cb > 1216) cb = 1216;
  if (cb < 1) cb = 1;
  return cb;
}

int launch_decide(const Sizes& s, const Dev& d, cudaStream_t st) {
  const int nb = cost_grid(s.no);
  CostArgs a = make_decide_args(s, d);
  // the priors' trial cost first: one more partial for the decision
  a.n_extra = launch_prior_eval(s, d, d.poses_t, 0, 2, a.partials + nb, st);
  a.n_extra += launch_edge_eval(s, d, d.poses_t, 0, 2, a.partials + nb + a.n_extra, st);
  (s.eucm ? k_cost<true> : k_cost<false>)<<<nb, kCostThreads, 0, st>>>(a, d.ctrl);
  const int cb = commit_grid(s);
  k_commit<<<cb, 256, 0, st>>>(s.nc, s.np, s.no, d.poses_t, d.poses, d.points_t, d.points, d.res_t, d.res,
                               d.res_lo_t, d.res_lo, s.intr_free ? d.intr_t : nullptr,
                               s.intr_free ? d.intr : nullptr, d.ctrl);
  return 2 + a.n_extra;
}

// ---------------------------------------------------------------------------
// Per-term Jacobians as the linearization evaluates them (sgba_debug_jacobians):
// the pose table of the observing camera and jacobians_f (FP32 linearization)
// or jacobians_dd (float-float linearization and rebuilt point blocks), with
// the same rounding of the inputs as k_landmark / k_camera_tiles.
// ---------------------------------------------------------------------------
namespace {
__global__ void k_debug_jacobians(int64_t n, const int32_t* __restrict__ cam, const int32_t* __restrict__ pt,
                                  const double* __restrict__ poses, const double* __restrict__ points,
                                  const double* __restrict__ intr, int eucm, int precision, double* __restrict__ jp,
                                  double* __restrict__ jm) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  float pf[12], pd[24];
  pose_table(poses + 7 * static_cast<int64_t>(cam[i]), pf, pd);
  const double* pw = points + 3 * static_cast<int64_t>(pt[i]);
  if (precision == 0) {
    JacF J;
    const float qx = __double2float_rn(pw[0]), qy = __double2float_rn(pw[1]), qz = __double2float_rn(pw[2]);
    if (eucm) jacobians_f<true>(pf, qx, qy, qz, cam_f(intr), &J);
    else jacobians_f<false>(pf, qx, qy, qz, cam_f(intr), &J);
    for (int k = 0; k < 12; ++k) jp[12 * i + k] = J.jp[k];
    for (int k = 0; k < 6; ++k) jm[6 * i + k] = J.jm[k];
  } else {
    JacD J;
    const dd qx = dd_from_double(pw[0]), qy = dd_from_double(pw[1]), qz = dd_from_double(pw[2]);
    if (eucm) jacobians_dd<true>(pd, qx, qy, qz, cam_dd(intr), &J);
    else jacobians_dd<false>(pd, qx, qy, qz, cam_dd(intr), &J);
    for (int k = 0; k < 12; ++k) jp[12 * i + k] = dd_to_double(J.jp[k]);
    for (int k = 0; k < 6; ++k) jm[6 * i + k] = dd_to_double(J.jm[k]);
  }
}
}  // namespace

cudaError_t launch_debug_jacobians(const Sizes& s, const Dev& d, int64_t n, const int32_t* cam, const int32_t* pt,
                                   int precision, double* jp, double* jm, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int64_t blocks = (n + 127) / 128;
  k_debug_jacobians<<<static_cast<unsigned>(blocks), 128, 0, st>>>(n, cam, pt, d.poses, d.points, d.intr,
                                                                   s.eucm, precision, jp, jm);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Allocation-free total cost (sgba_total_cost_noalloc).
//
// The same float-float calc_total_cost as k_cost, for callers that hold the
// observations in their own device memory and may not allocate: the scratch
// (pose tables, per-CTA partial sums and a zero Ctrl) is one file-scope
// __device__ array, sized for kNoAllocMaxCams cameras.
// ---------------------------------------------------------------------------
namespace {

constexpr int kNoAllocMaxCams = 4096;
constexpr size_t kNoAllocCtrlBytes = (sizeof(Ctrl) + 255) / 256 * 256;
constexpr size_t kNoAllocPoseFOff = kNoAllocCtrlBytes;
constexpr size_t kNoAllocPoseDDOff = kNoAllocPoseFOff + sizeof(float) * 12 * kNoAllocMaxCams;
constexpr size_t kNoAllocPartOff = kNoAllocPoseDDOff + sizeof(float) * 24 * kNoAllocMaxCams;
constexpr size_t kNoAllocBytes = kNoAllocPartOff + sizeof(double) * kCostMaxBlocks;
static_assert(kNoAllocBytes == 599808, "the scratch size is stated in sgba.h");

// [0, kNoAllocCtrlBytes): a Ctrl whose done and skip fields must read 0 (the
// zero fill of module load; nothing writes it); then the float and
// float-float pose tables; then the partial sums.  The tables and partials
// are fully rewritten by every call before they are read.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned char* g_noalloc_base[kNoAllocMaxDevices] = {};

// k_cost without the residual output and with index checks: an observation
// whose pose or point index is out of range contributes NaN (and is never
// dereferenced), so the returned cost is NaN.
__global__ void __launch_bounds__(kCostThreads) k_cost_noalloc(CostArgs a, int32_t nc, int32_t np) {
  dd acc = dd_make(0.0f, 0.0f);
  bool bad = false;
  for (int64_t o = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; o < a.no;
       o += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int32_t jc = a.opose[o], ip = a.opt[o];
    if (jc < 0 || jc >= nc || ip < 0 || ip >= np) {
      bad = true;
      continue;
    }
    const float* P = a.pose_dd + 24 * jc;
    const double* pw = a.points + 3 * ip;
    dd p0 = dd_from_double(pw[0]), p1 = dd_from_double(pw[1]), p2 = dd_from_double(pw[2]);
    dd xc[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      dd r0 = dd_make(P[2 * (i * 3 + 0)], P[2 * (i * 3 + 0) + 1]);
      dd r1 = dd_make(P[2 * (i * 3 + 1)], P[2 * (i * 3 + 1) + 1]);
      dd r2 = dd_make(P[2 * (i * 3 + 2)], P[2 * (i * 3 + 2) + 1]);
      dd tt = dd_make(P[18 + 2 * i], P[18 + 2 * i + 1]);
      xc[i] = dd_add(dd_add(dd_add(dd_mul(r0, p0), dd_mul(r1, p1)), dd_mul(r2, p2)), tt);
    }
    dd u = dd_div(xc[0], xc[2]);
    dd v = dd_div(xc[1], xc[2]);
    double2 z = a.uv[o];
    dd ru = dd_sub(dd_from_double(z.x), dd_add(dd_mul(u, a.fx), a.cx));
    dd rv = dd_sub(dd_from_double(z.y), dd_add(dd_mul(v, a.fy), a.cy));
    dd n2 = dd_add(dd_mul(ru, ru), dd_mul(rv, rv));
    dd c = n2;
    if (a.huber > 0.0f) {
      dd nrm = dd_sqrt(n2);
      if (!(nrm.hi <= a.huber || (nrm.hi == a.huber_dd.hi && nrm.lo <= a.huber_dd.lo))) {
        c = dd_sub(dd_mul(dd_add(a.huber_dd, a.huber_dd), nrm), dd_mul(a.huber_dd, a.huber_dd));
      }
    }
    acc = dd_add(acc, c);
  }
  if (bad) acc = dd_make(__int_as_float(0x7fc00000), 0.0f);
  __shared__ float sh_hi[kCostThreads / 32], sh_lo[kCostThreads / 32];
  acc = dd_warp_sum(acc);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) { sh_hi[w] = acc.hi; sh_lo[w] = acc.lo; }
  __syncthreads();
  if (w == 0) {
    dd v = (lane < (int)(blockDim.x >> 5)) ? dd_make(sh_hi[lane], sh_lo[lane]) : dd_make(0.0f, 0.0f);
    v = dd_warp_sum(v);
    if (lane == 0) a.partials[blockIdx.x] = dd_to_double(v);
  }
}

__global__ void k_noalloc_finish(const double* part, int n, double* out) {
  double s = block_sum_partials(part, n);
  if (threadIdx.x == 0) out[0] = s;
}

// Per-device set-up, with the device current: the address of the scratch
// array and the loading of the three kernels (CUDA's lazy module loading
// would otherwise do that at the first launch).
cudaError_t noalloc_base(unsigned char** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_base[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    cudaFuncAttributes fa;
    if ((e = cudaFuncGetAttributes(&fa, k_pose_tables)) != cudaSuccess) return e;
    if ((e = cudaFuncGetAttributes(&fa, k_cost_noalloc)) != cudaSuccess) return e;
    if ((e = cudaFuncGetAttributes(&fa, k_noalloc_finish)) != cudaSuccess) return e;
    g_noalloc_base[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_noalloc_base[dev];
  return cudaSuccess;
}

}  // namespace

int noalloc_max_cams() { return kNoAllocMaxCams; }

cudaError_t launch_total_cost_noalloc(int32_t nc, const double* poses, int32_t np, const double* points,
                                      int64_t no, const int32_t* obs_cam, const int32_t* obs_pt,
                                      const double* obs_uv, const double* intr, double huber,
                                      double* cost, cudaStream_t st) {
  unsigned char* base = nullptr;
  cudaError_t e = noalloc_base(&base);
  if (e != cudaSuccess) return e;
  const Ctrl* zero_ctrl = reinterpret_cast<const Ctrl*>(base);
  float* pose_f = reinterpret_cast<float*>(base + kNoAllocPoseFOff);
  float* pose_dd = reinterpret_cast<float*>(base + kNoAllocPoseDDOff);
  double* part = reinterpret_cast<double*>(base + kNoAllocPartOff);
  k_pose_tables<<<(nc + 127) / 128, 128, 0, st>>>(nc, poses, pose_f, pose_dd, zero_ctrl, 0, nullptr, nullptr);
  auto split = [](double x) { return dd_make(static_cast<float>(x), static_cast<float>(x - static_cast<float>(x))); };
  CostArgs a;
  a.no = no;
  a.uv = reinterpret_cast<const double2*>(obs_uv);
  a.opose = obs_cam;
  a.opt = obs_pt;
  a.pose_dd = pose_dd;
  a.points = points;
  a.res_out = nullptr;
  a.res_lo_out = nullptr;
  a.decide = nullptr;
  a.partials = part;
  a.fx = split(intr[0]);
  a.fy = split(intr[1]);
  a.cx = split(intr[2]);
  a.cy = split(intr[3]);
  a.intr = nullptr;
  a.huber = static_cast<float>(huber > 0 ? huber : 0.0);
  a.huber_dd = split(huber);
  a.respect_skip = 0;
  a.n_extra = 0;
  const int nb = cost_grid(no);
  k_cost_noalloc<<<nb, kCostThreads, 0, st>>>(a, nc, np);
  k_noalloc_finish<<<1, 256, 0, st>>>(part, nb, cost);
  return cudaGetLastError();
}


// ---------------------------------------------------------------------------
// Batched local windows: each kernel of an LM iteration launched once for all
// windows of a batch.  Block b of a batched launch is block b - off[w] of
// window w's own grid (off: prefix sums of the per-window grid sizes), run
// with window w's arguments and control block by the same kernel body, so
// each window computes bit for bit what its own launches compute.
// ---------------------------------------------------------------------------
namespace {

template <class A>
struct WinTab {
  const A* args;       // per window
  Ctrl* const* ctrl;   // per window
  const int32_t* off;  // n + 1 prefix sums of the per-window grid sizes
  int n;
};

// the window of batched block b: the largest w with off[w] <= b (windows
// without blocks in this launch have off[w] == off[w + 1] and are skipped)
__device__ __forceinline__ int win_of(const int32_t* off, int n, int b) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(off + mid) <= b) lo = mid;
    else hi = mid;
  }
  return lo;
}

struct WinPos {
  int w, b, nb;
};
template <class A>
__device__ __forceinline__ WinPos win_pos(const WinTab<A>& t) {
  const int w = win_of(t.off, t.n, static_cast<int>(blockIdx.x));
  const int o = __ldg(t.off + w);
  return WinPos{w, static_cast<int>(blockIdx.x) - o, __ldg(t.off + w + 1) - o};
}

struct PoseTabArgs {
  int nc;
  const double* poses;
  float* pose_f;
  float* pose_dd;
  int respect_skip;
  int begin;  // open the iteration (the window's control block)
  int32_t* zero_count;
};
struct FinArgs {
  int nf;
  const int64_t* fb_tile_begin;
  const double* tile_part;
  double* ufull;
  double* bf;
  double* rb;
  int with_schur;
};
struct BsubArgs {
  BackArgs b;
  const int32_t* chunk_pt;
  int nchunk;
  const int32_t* g_pt;
};
struct MeritArgs {
  const double* part;
  int n;
};
struct CommitArgs {
  int nc, np;
  int64_t no;
  const double* poses_t;
  double* poses;
  const double* points_t;
  double* points;
  const float2* res_t;
  float2* res;
  const float2* res_lo_t;
  float2* res_lo;
  const double* intr_t;
  double* intr;
};

__global__ void __launch_bounds__(128) k_pose_tables_w(WinTab<PoseTabArgs> t) {
  const WinPos q = win_pos(t);
  const PoseTabArgs a = t.args[q.w];
  Ctrl* c = t.ctrl[q.w];
  pose_tables_body(a.nc, a.poses, a.pose_f, a.pose_dd, c, a.respect_skip, a.begin ? c : nullptr, a.zero_count, q.b,
                   q.nb);
}
template <bool E>
__global__ void __launch_bounds__(kCostThreads) k_cost_w(WinTab<CostArgs> t) {
  const WinPos q = win_pos(t);
  cost_body<E>(t.args[q.w], t.ctrl[q.w], q.b, q.nb);
}
__global__ void k_init_merit_w(WinTab<MeritArgs> t) {
  const WinPos q = win_pos(t);
  const MeritArgs a = t.args[q.w];
  const double v = block_sum_partials(a.part, a.n);
  if (threadIdx.x == 0) {
    Ctrl* c = t.ctrl[q.w];
    c->merit = v;
    c->new_merit = v;
  }
}
template <bool E>
__global__ void __launch_bounds__(256, 2) k_landmark_w(WinTab<LinArgs> t) {
  const WinPos q = win_pos(t);
  landmark_body<E>(t.args[q.w], t.ctrl[q.w], q.b, q.nb);
}
template <bool E>
__global__ void __launch_bounds__(256) k_landmark_chunks_w(WinTab<LinArgs> t) {
  const WinPos q = win_pos(t);
  landmark_chunks_body<E>(t.args[q.w], t.ctrl[q.w], q.b, q.nb);
}
template <bool E>
__global__ void __launch_bounds__(kTileThreads) k_camera_tiles_w(WinTab<CamArgs> t) {
  const WinPos q = win_pos(t);
  camera_tiles_body<E>(t.args[q.w], t.ctrl[q.w], q.b, q.nb);
}
__global__ void __launch_bounds__(64) k_camera_finalize_w(WinTab<FinArgs> t) {
  const WinPos q = win_pos(t);
  const FinArgs a = t.args[q.w];
  camera_finalize_body(a.nf, a.fb_tile_begin, a.tile_part, a.ufull, a.bf, a.rb, t.ctrl[q.w], a.with_schur, nullptr,
                       nullptr, nullptr, nullptr, nullptr, q.b, q.nb);
}
__global__ void __launch_bounds__(kSdThreads, 3) k_schur_dense_w(WinTab<SchurDenseArgs> t) {
  const WinPos q = win_pos(t);
  schur_dense_body(t.args[q.w], t.ctrl[q.w], q.b, q.nb);
}
__global__ void __launch_bounds__(256, 2) k_schur_w(WinTab<SchurArgs> t) {
  const WinPos q = win_pos(t);
  schur_body(t.args[q.w], t.ctrl[q.w], q.b, q.nb);
}
__global__ void __launch_bounds__(256) k_schur_reduce_w(WinTab<SchurArgs> t) {
  const WinPos q = win_pos(t);
  schur_reduce_body(t.args[q.w], t.ctrl[q.w], q.b, q.nb);
}
__global__ void __launch_bounds__(256) k_backsub_chunks_w(WinTab<BsubArgs> t) {
  const WinPos q = win_pos(t);
  const BsubArgs& a = t.args[q.w];
  backsub_chunks_body(a.b, a.chunk_pt, a.nchunk, a.g_pt, t.ctrl[q.w], q.b, q.nb);
}
__global__ void __launch_bounds__(256) k_gauge_partials_w(WinTab<GaugeArgs> t) {
  const WinPos q = win_pos(t);
  gauge_partials_body(t.args[q.w], t.ctrl[q.w], q.b, q.nb);
}
__global__ void __launch_bounds__(256) k_apply_update_w(WinTab<UpdArgs> t) {
  const WinPos q = win_pos(t);
  apply_update_body(t.args[q.w], t.ctrl[q.w], q.b, q.nb);
}
__global__ void k_commit_w(WinTab<CommitArgs> t) {
  const WinPos q = win_pos(t);
  const CommitArgs a = t.args[q.w];
  commit_body(a.nc, a.np, a.no, a.poses_t, a.poses, a.points_t, a.points, a.res_t, a.res, a.res_lo_t, a.res_lo,
              a.intr_t, a.intr, t.ctrl[q.w], q.b, q.nb);
}
// control blocks of every window from one template (the batch shares its params)
__global__ void k_ctrl_init_w(Ctrl init, Ctrl* const* ctrl, int n) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w < n) *ctrl[w] = init;
}
// control blocks and the first cap records of every window into packed arrays
__global__ void k_collect_w(Ctrl* const* ctrl, Record* const* recs, const int* rec_cap, int n, Ctrl* out,
                            Record* rout, int cap) {
  const int w = blockIdx.x;
  if (w >= n) return;
  const Ctrl* c = ctrl[w];
  if (threadIdx.x == 0) out[w] = *c;
  int nr = c->step < rec_cap[w] ? c->step : rec_cap[w];
  if (nr > cap) nr = cap;
  for (int r = threadIdx.x; r < nr; r += blockDim.x) rout[static_cast<int64_t>(w) * cap + r] = recs[w][r];
}

// One batched kernel's device table and launch shape.
struct KTab {
  const void* args = nullptr;
  const int32_t* off = nullptr;
  int blocks = 0;
  size_t smem = 0;
};

}  // namespace

struct BatchTables {
  int n = 0;
  void* dbuf = nullptr;
  Ctrl** ctrl = nullptr;     // device: n control blocks
  Record** recs = nullptr;   // device: n record buffers
  int* rec_cap = nullptr;    // device: n record capacities
  KTab pose_it, lmk_chunks, lmk_slow, cam, fin, schur, schur_red, schur_dense, bsub, gauge, upd, cost, commit;
  KTab pose_init, cost_init, merit;
  KTab pose_fin, lmk_fin, cam_fin, fin_fin;
  DenseBatch* dense = nullptr;
};

int batch_eligible(const Sizes& s) {
  return (!s.lin_dd && !s.eucm && !s.intr_free && !s.pcg_mode && s.n_prior == 0 && s.n_edge == 0 && s.n_eq == 0 &&
          s.band_c == 0 &&
          (s.small_dense || s.dense_c > 0) &&
          s.nlchunk > 0 && s.bsub_chunks_ok && s.ntiles > 0 && s.nf > 0)
             ? 1
             : 0;
}

int batch_window_count(const BatchTables* t) { return t ? t->n : 0; }

namespace {

// Host staging of the tables: one byte image, uploaded at once.
struct TabImage {
  std::vector<unsigned char> bytes;
  size_t put(const void* p, size_t n) {
    const size_t at = (bytes.size() + 15) / 16 * 16;
    bytes.resize(at + n);
    if (n) std::memcpy(bytes.data() + at, p, n);
    return at;
  }
};

// Collects one kernel's per-window arguments and grid sizes.
template <class A>
struct TabBuild {
  std::vector<A> args;
  std::vector<int32_t> off{0};
  size_t smem = 0;
  void add(const A& a, int blocks, size_t sm = 0) {
    args.push_back(a);
    off.push_back(off.back() + (blocks > 0 ? blocks : 0));
    if (blocks > 0 && sm > smem) smem = sm;
  }
  void stage(TabImage& im, size_t* a_at, size_t* o_at) const {
    *a_at = im.put(args.data(), sizeof(A) * args.size());
    *o_at = im.put(off.data(), sizeof(int32_t) * off.size());
  }
};

}  // namespace

BatchTables* batch_tables_create(const std::vector<BatchWin>& wins, int skip_final_hessian, cudaStream_t st,
                                 cudaError_t* err) {
  *err = cudaSuccess;
  const int n = static_cast<int>(wins.size());
  TabBuild<PoseTabArgs> t_pose_it, t_pose_init, t_pose_fin;
  TabBuild<LinArgs> t_lmk_chunks, t_lmk_slow, t_lmk_fin;
  TabBuild<CamArgs> t_cam, t_cam_fin;
  TabBuild<FinArgs> t_fin, t_fin_fin;
  TabBuild<SchurArgs> t_schur, t_schur_red;
  TabBuild<SchurDenseArgs> t_schur_dense;
  TabBuild<BsubArgs> t_bsub;
  TabBuild<GaugeArgs> t_gauge;
  TabBuild<UpdArgs> t_upd;
  TabBuild<CostArgs> t_cost, t_cost_init;
  TabBuild<CommitArgs> t_commit;
  TabBuild<MeritArgs> t_merit;
  std::vector<Ctrl*> ctrl(n);
  std::vector<Record*> recs(n);
  std::vector<int> rec_cap(n);
  for (int w = 0; w < n; ++w) {
    const Sizes& s = *wins[w].s;
    const Dev& d = *wins[w].d;
    ctrl[w] = d.ctrl;
    recs[w] = d.records;
    rec_cap[w] = d.record_cap;
    const int pose_grid = (s.nc + 127) / 128;
    const int lmk_grid = s.nlchunk < 8192 ? s.nlchunk : 8192;
    // iteration (enqueue_iteration: launch_linearize, launch_schur,
    // launch_factor_solve, launch_update, launch_decide)
    t_pose_it.add(PoseTabArgs{s.nc, d.poses, d.pose_f, d.pose_dd, 0, 1, d.slow_count}, pose_grid);
    const LinArgs la = make_lin_args(s, d, 0.0, false);
    t_lmk_chunks.add(la, lmk_grid, sizeof(float) * 9 * static_cast<size_t>(s.lmk_cap));
    LinArgs lb = la;
    lb.list = d.slow_list;
    lb.list_count = d.slow_count;
    t_lmk_slow.add(lb, s.lmk_list_grid);
    t_cam.add(make_cam_args(s, d, 1), static_cast<int>(s.ntiles));
    t_fin.add(FinArgs{s.nf, d.fb_tile_begin, d.tile_part, d.ufull, d.bf, d.rb, 1}, s.nf);
    const SchurArgs sa = make_schur_args(s, d);
    t_schur.add(sa, s.schur_dense ? 0 : warp_grid(s.nchunk, 8, 65536));
    t_schur_red.add(sa, s.schur_dense ? 0 : warp_grid(s.nsb, 8, 8192));
    t_schur_dense.add(make_schur_dense_args(s, d), s.schur_dense ? schur_dense_grid(s) : 0);
    t_bsub.add(BsubArgs{make_back_args(s, d), d.lmk_chunk_pt, s.nlchunk, d.g_pt}, lmk_grid,
               sizeof(float) * 12 * static_cast<size_t>(s.lmk_cap));
    t_gauge.add(make_gauge_args(s, d), s.gauge_kind == 1 ? upd_blocks(s) : 0);
    t_upd.add(make_upd_args(s, d), upd_blocks(s));
    t_cost.add(make_decide_args(s, d), cost_grid(s.no));
    t_commit.add(CommitArgs{s.nc, s.np, s.no, d.poses_t, d.poses, d.points_t, d.points, d.res_t, d.res, d.res_lo_t,
                            d.res_lo, nullptr, nullptr},
                 commit_grid(s));
    // init (launch_init_merit)
    t_pose_init.add(PoseTabArgs{s.nc, d.poses, d.pose_f, d.pose_dd, 0, 0, nullptr}, pose_grid);
    t_cost_init.add(make_cost_args(s, d, d.points, d.res, d.part, 0), cost_grid(s.no));
    t_merit.add(MeritArgs{d.part, cost_grid(s.no)}, 1);
    // final linearisation (launch_linearize with the damping override)
    t_pose_fin.add(PoseTabArgs{s.nc, d.poses, d.pose_f, d.pose_dd, 0, 0, nullptr}, pose_grid);
    LinArgs lf = make_lin_args(s, d, 0.0, true);
    lf.nu_ctrl = skip_final_hessian ? 1 : 0;
    t_lmk_fin.add(lf, warp_grid(s.np, 8, 4096));
    t_cam_fin.add(make_cam_args(s, d, 0), static_cast<int>(s.ntiles));
    t_fin_fin.add(FinArgs{s.nf, d.fb_tile_begin, d.tile_part, d.ufull, d.bf, d.rb, 0}, s.nf);
  }
  TabImage im;
  const size_t ctrl_at = im.put(ctrl.data(), sizeof(Ctrl*) * n);
  const size_t recs_at = im.put(recs.data(), sizeof(Record*) * n);
  const size_t cap_at = im.put(rec_cap.data(), sizeof(int) * n);
  struct Pending {
    KTab* k;
    size_t a_at, o_at;
  };
  BatchTables* T = new BatchTables();
  std::vector<Pending> pend;
  auto stage = [&](auto& tb, KTab* k) {
    Pending p{k, 0, 0};
    tb.stage(im, &p.a_at, &p.o_at);
    k->blocks = tb.off.back();
    k->smem = tb.smem;
    pend.push_back(p);
  };
  stage(t_pose_it, &T->pose_it);
  stage(t_lmk_chunks, &T->lmk_chunks);
  stage(t_lmk_slow, &T->lmk_slow);
  stage(t_cam, &T->cam);
  stage(t_fin, &T->fin);
  stage(t_schur, &T->schur);
  stage(t_schur_red, &T->schur_red);
  stage(t_schur_dense, &T->schur_dense);
  stage(t_bsub, &T->bsub);
  stage(t_gauge, &T->gauge);
  stage(t_upd, &T->upd);
  stage(t_cost, &T->cost);
  stage(t_commit, &T->commit);
  stage(t_pose_init, &T->pose_init);
  stage(t_cost_init, &T->cost_init);
  stage(t_merit, &T->merit);
  stage(t_pose_fin, &T->pose_fin);
  stage(t_lmk_fin, &T->lmk_fin);
  stage(t_cam_fin, &T->cam_fin);
  stage(t_fin_fin, &T->fin_fin);
  T->n = n;
  cudaError_t e = cudaMallocAsync(&T->dbuf, im.bytes.size() > 0 ? im.bytes.size() : 16, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(T->dbuf, im.bytes.data(), im.bytes.size(), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) {
    *err = e;
    if (T->dbuf) cudaFreeAsync(T->dbuf, st);
    delete T;
    return nullptr;
  }
  unsigned char* base = static_cast<unsigned char*>(T->dbuf);
  T->ctrl = reinterpret_cast<Ctrl**>(base + ctrl_at);
  T->recs = reinterpret_cast<Record**>(base + recs_at);
  T->rec_cap = reinterpret_cast<int*>(base + cap_at);
  for (const Pending& p : pend) {
    p.k->args = base + p.a_at;
    p.k->off = reinterpret_cast<const int32_t*>(base + p.o_at);
  }
  // dynamic shared memory limits of the batched kernels (per function and
  // device, only ever raised)
  if ((T->lmk_chunks.smem > 48 * 1024 &&
       raise_dynamic_smem(reinterpret_cast<const void*>(k_landmark_chunks_w<false>), T->lmk_chunks.smem) !=
           cudaSuccess) ||
      (T->bsub.smem > 48 * 1024 &&
       raise_dynamic_smem(reinterpret_cast<const void*>(k_backsub_chunks_w), T->bsub.smem) != cudaSuccess)) {
    *err = cudaErrorInvalidValue;
    batch_tables_destroy(T, st);
    return nullptr;
  }
  T->dense = dense_batch_create(wins, T->ctrl, st, &e);
  if (!T->dense) {
    *err = e != cudaSuccess ? e : cudaErrorInvalidValue;
    batch_tables_destroy(T, st);
    return nullptr;
  }
  return T;
}

void batch_tables_destroy(BatchTables* t, cudaStream_t st) {
  if (!t) return;
  if (t->dense) dense_batch_destroy(t->dense, st);
  if (t->dbuf) cudaFreeAsync(t->dbuf, st);
  delete t;
}

namespace {

template <class A>
WinTab<A> wtab(const BatchTables* t, const KTab& k) {
  return WinTab<A>{static_cast<const A*>(k.args), t->ctrl, k.off, t->n};
}

}  // namespace

int batch_launch_init(const BatchTables* t, const Ctrl& init, cudaStream_t st) {
  int n = 0;
  k_ctrl_init_w<<<(t->n + 127) / 128, 128, 0, st>>>(init, t->ctrl, t->n);
  ++n;
  if (t->pose_init.blocks) {
    k_pose_tables_w<<<t->pose_init.blocks, 128, 0, st>>>(wtab<PoseTabArgs>(t, t->pose_init));
    ++n;
  }
  if (t->cost_init.blocks) {
    k_cost_w<false><<<t->cost_init.blocks, kCostThreads, 0, st>>>(wtab<CostArgs>(t, t->cost_init));
    ++n;
  }
  if (t->merit.blocks) {
    k_init_merit_w<<<t->merit.blocks, 256, 0, st>>>(wtab<MeritArgs>(t, t->merit));
    ++n;
  }
  return n;
}

int batch_launch_iteration(const BatchTables* t, cudaStream_t st) {
  int n = 0;
  auto go = [&](const KTab& k) { return k.blocks > 0 ? (++n, true) : false; };
  if (go(t->pose_it)) k_pose_tables_w<<<t->pose_it.blocks, 128, 0, st>>>(wtab<PoseTabArgs>(t, t->pose_it));
  if (go(t->lmk_chunks))
    k_landmark_chunks_w<false>
        <<<t->lmk_chunks.blocks, 256, t->lmk_chunks.smem, st>>>(wtab<LinArgs>(t, t->lmk_chunks));
  if (go(t->lmk_slow)) k_landmark_w<false><<<t->lmk_slow.blocks, 256, 0, st>>>(wtab<LinArgs>(t, t->lmk_slow));
  if (go(t->cam)) k_camera_tiles_w<false><<<t->cam.blocks, kTileThreads, 0, st>>>(wtab<CamArgs>(t, t->cam));
  if (go(t->fin)) k_camera_finalize_w<<<t->fin.blocks, 64, 0, st>>>(wtab<FinArgs>(t, t->fin));
  if (go(t->schur)) k_schur_w<<<t->schur.blocks, 256, 0, st>>>(wtab<SchurArgs>(t, t->schur));
  if (go(t->schur_red)) k_schur_reduce_w<<<t->schur_red.blocks, 256, 0, st>>>(wtab<SchurArgs>(t, t->schur_red));
  if (go(t->schur_dense))
    k_schur_dense_w<<<t->schur_dense.blocks, kSdThreads, 0, st>>>(wtab<SchurDenseArgs>(t, t->schur_dense));
  n += launch_dense_batch(t->dense, st);
  if (go(t->bsub)) k_backsub_chunks_w<<<t->bsub.blocks, 256, t->bsub.smem, st>>>(wtab<BsubArgs>(t, t->bsub));
  if (go(t->gauge)) k_gauge_partials_w<<<t->gauge.blocks, 256, 0, st>>>(wtab<GaugeArgs>(t, t->gauge));
  if (go(t->upd)) k_apply_update_w<<<t->upd.blocks, 256, 0, st>>>(wtab<UpdArgs>(t, t->upd));
  if (go(t->cost)) k_cost_w<false><<<t->cost.blocks, kCostThreads, 0, st>>>(wtab<CostArgs>(t, t->cost));
  if (go(t->commit)) k_commit_w<<<t->commit.blocks, 256, 0, st>>>(wtab<CommitArgs>(t, t->commit));
  return n;
}

int batch_launch_final(const BatchTables* t, cudaStream_t st) {
  int n = 0;
  auto go = [&](const KTab& k) { return k.blocks > 0 ? (++n, true) : false; };
  if (go(t->pose_fin)) k_pose_tables_w<<<t->pose_fin.blocks, 128, 0, st>>>(wtab<PoseTabArgs>(t, t->pose_fin));
  if (go(t->lmk_fin)) k_landmark_w<false><<<t->lmk_fin.blocks, 256, 0, st>>>(wtab<LinArgs>(t, t->lmk_fin));
  if (go(t->cam_fin))
    k_camera_tiles_w<false><<<t->cam_fin.blocks, kTileThreads, 0, st>>>(wtab<CamArgs>(t, t->cam_fin));
  if (go(t->fin_fin)) k_camera_finalize_w<<<t->fin_fin.blocks, 64, 0, st>>>(wtab<FinArgs>(t, t->fin_fin));
  return n;
}

int batch_launch_collect(const BatchTables* t, Ctrl* ctrl_out, Record* rec_out, int cap, cudaStream_t st) {
  if (t->n == 0) return 0;
  k_collect_w<<<t->n, 128, 0, st>>>(t->ctrl, t->recs, t->rec_cap, t->n, ctrl_out, rec_out, cap);
  return 1;
}

}  // namespace sgba
