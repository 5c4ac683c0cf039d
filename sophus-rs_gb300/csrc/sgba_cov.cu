// sgba_cov.cu -- covariance and precision queries of the final Hessian on the
// GPU.
//
// Reference: Optimizer::build_solution (crates/sophus_opt/src/nlls/optimizer.rs:609-646)
// evaluates the linear system at the solution with zero damping;
// OptimizationSolution::precision_block / covariance_block
// (crates/sophus_opt/src/nlls/optimizer_types.rs:277-370) answer block queries
// from it.  The Schur factor answers covariance blocks as
// SchurFactor::inverse_block does (crates/sophus_solver/src/ldlt/schur_ldlt.rs:815-957):
//   free x free  S^-1[row, col]
//   free x marg  -(S^-1 H_fm H_mm^-1)[row, col]
//   marg x marg  H_mm^-1 delta_ij + H_mm[i]^-1 H_mf_i S^-1 H_mf_j^T H_mm[j]^-1
// and S^-1 is the min-norm pseudo-inverse E G^-1 diag(d_J)^-1 G^-1 E^T when
// the LDL^T of S has zero pivots (crates/sophus_solver/src/ldlt/min_norm_ldlt.rs:55-140),
// E the columns of L at the positive pivots J and G = E^T E.
//
// Arithmetic: f64 throughout (FP64 pipe).  The covariance inverts S, so its
// error is the error of S times the condition number of S; the LM path's
// FP32 / float-float linearization is accurate enough for a step that the
// next iteration corrects, not for an inverse.  The Hessian of a
// reprojection term is J^T J whatever the robust kernel (the weight acts on
// the residual), so only the Jacobians enter: they are evaluated here in f64
// from the same closed forms as the linearization kernels.
//
// Kernels, in order:
//   k_cov_groups     thread per reduced term (point, pose): J_pose^T J_pose,
//                    W = J_pose^T J_point, J_point^T J_point (times the
//                    term's observation count: its observations share J)
//   k_cov_points     thread per marginalized point: H_mm = sum over its terms
//                    (term order), its inverse (cofactors, singular iff the
//                    determinant is 0, as nalgebra's try_inverse), and
//                    Y = W H_mm^-1 for its terms with a free pose
//   k_cov_s          warp per lower block (a, b) of S: the diagonal block
//                    U_a + priors + edges - sum Y W^T over pose a's terms;
//                    off-diagonal blocks - sum Y_a W_b^T over the points both
//                    poses see (the lanes merge slices of the two poses' term
//                    lists, which are in point order) + J_m^T J_n of edges;
//                    both triangles written.  No atomics: lane sums by a
//                    fixed shuffle tree, one writer per entry.
//   k_cov_panel /    right-looking scalar LDL^T in natural order, one 6-row
//   k_cov_update     pose block per step: every CTA factors the 6x6 diagonal
//                    block redundantly with the reference's pivot rule
//                    (dense_ldlt.rs:164-230: a pivot at most
//                    1e-12 max(1, largest pivot so far in its block) is
//                    zeroed and zeroes its column of L), solves its rows of
//                    the column below, then the trailing lower triangle is
//                    updated in 32 x 32 tiles
//   k_cov_inv_part / Z = S^-1 by the Takahashi recurrence on the factor,
//   k_cov_inv_fin /  block rows last to first:
//   k_cov_inv_diag     Z_rc = delta_rc / d_r - sum_{m > r} L_mr Z_mc  (c >= r);
//                    the sums over m of the block row's columns beyond the
//                    block (thread per column, rows m split over CTAs, reading
//                    rows of Z written by the launches before), their finish
//                    (the 6-row recurrence, the row and its mirror, the
//                    diagonal block's sums), then the 6x6 diagonal block
//   k_cov_gemm       tiled f64 products of the pseudo-inverse (rank-deficient S)
//   k_cov_query      CTA per query: covariance or H blocks from Z, Y, H_mm^-1
#include <cuda_runtime.h>

#include <cfloat>
#include <algorithm>
#include <cstdint>
#include <vector>

#include "sgba_internal.h"
#include "sgba_lie.cuh"

namespace sgba {

namespace {

constexpr int kCovThreads = 256;
constexpr double kCovTolRel = 1e-12;  // BlockSparseLdlt's tol_rel
constexpr int kUT = 32;               // trailing-update tile
constexpr int kInvRows = 256;         // rows of L staged per round of k_cov_inv_part
constexpr int kInvSplitMax = 32;      // ranges of rows m of one block row at most
constexpr int kInvMinRows = 32;       // rows m per range at least
constexpr int kGT = 64, kGK = 16;     // GEMM tile and depth

// ---------------------------------------------------------------------------
// Jacobians of r = uv - pi(T_cw p) in f64 (the closed forms of the
// linearization kernels, pinhole_reprojection.rs:60-95, ba_problem.rs:69-110):
// T_cw = T_wc^-1, D = d pi R_cw (2x3), J_pose = [D hat(-p), D], J_point = -D.
// ---------------------------------------------------------------------------
template <bool E>
__device__ void cov_jacobians(const double* T, const double* p, const double* intr, double* jp, double* jm) {
  double Rwc[9];
  lie::quat_matrix<double>(T, Rwc);
  double R[9], t[3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[3 * i + j] = Rwc[3 * j + i];
  for (int i = 0; i < 3; ++i) t[i] = -(R[3 * i] * T[4] + R[3 * i + 1] * T[5] + R[3 * i + 2] * T[6]);
  const double xc = R[0] * p[0] + R[1] * p[1] + R[2] * p[2] + t[0];
  const double yc = R[3] * p[0] + R[4] * p[1] + R[5] * p[2] + t[1];
  const double zc = R[6] * p[0] + R[7] * p[1] + R[8] * p[2] + t[2];
  const double iz = 1.0 / zc;
  const double fx = intr[0], fy = intr[1];
  double D[6];
  if constexpr (!E) {
    const double a0 = fx * iz, a2 = -fx * xc * iz * iz;
    const double b1 = fy * iz, b2 = -fy * yc * iz * iz;
    for (int k = 0; k < 3; ++k) {
      D[k] = a0 * R[k] + a2 * R[6 + k];
      D[3 + k] = b1 * R[3 + k] + b2 * R[6 + k];
    }
  } else {
    // d pi = M d proj, M the derivative of the EUCM distortion (enhanced_unified.rs:117-156)
    const double al = intr[4], be = intr[5];
    const double x = xc * iz, y = yc * iz;
    const double rho = sqrt(be * (x * x + y * y) + 1.0);
    const double nrm = al * rho + (1.0 - al);
    const double in2 = 1.0 / (nrm * nrm);
    const double ab = al * be / rho;
    const double nx = ab * x, ny = ab * y;
    const double m00 = fx * (nrm - x * nx) * in2, m01 = -fx * x * ny * in2;
    const double m10 = -fy * y * nx * in2, m11 = fy * (nrm - y * ny) * in2;
    const double a0 = m00 * iz, a1 = m01 * iz, a2 = -(m00 * x + m01 * y) * iz;
    const double b0 = m10 * iz, b1 = m11 * iz, b2 = -(m10 * x + m11 * y) * iz;
    for (int k = 0; k < 3; ++k) {
      D[k] = a0 * R[k] + a1 * R[3 + k] + a2 * R[6 + k];
      D[3 + k] = b0 * R[k] + b1 * R[3 + k] + b2 * R[6 + k];
    }
  }
  const double px = p[0], py = p[1], pz = p[2];
  for (int r = 0; r < 2; ++r) {
    const double* d = D + 3 * r;
    jp[r * 6 + 0] = -d[1] * pz + d[2] * py;
    jp[r * 6 + 1] = d[0] * pz - d[2] * px;
    jp[r * 6 + 2] = -d[0] * py + d[1] * px;
    jp[r * 6 + 3] = d[0];
    jp[r * 6 + 4] = d[1];
    jp[r * 6 + 5] = d[2];
    jm[r * 3 + 0] = -d[0];
    jm[r * 3 + 1] = -d[1];
    jm[r * 3 + 2] = -d[2];
  }
}

// index of (a, b), a <= b, in the row-major upper triangle of a k x k matrix
__device__ __forceinline__ int up_idx(int k, int a, int b) { return a * k - a * (a - 1) / 2 + (b - a); }

// Jacobian of r with respect to the camera params (2 x 6 row-major, columns
// beyond the model's 4 or 6 zero): J_cam = -d pi / d params
// (pinhole_reprojection.rs:85, dx_distort_params of perspective.rs and
// enhanced_unified.rs:158-215): fx fy cx cy, then for the EUCM camera
// alpha beta with d(1/norm) / d alpha = -(rho - 1) / norm^2 and
// d(1/norm) / d beta = -alpha r2 / (2 rho norm^2).
template <bool E>
__device__ void cov_cam_jacobian(const double* T, const double* p, const double* intr, double* jc) {
  double Rwc[9];
  lie::quat_matrix<double>(T, Rwc);
  double R[9], t[3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[3 * i + j] = Rwc[3 * j + i];
  for (int i = 0; i < 3; ++i) t[i] = -(R[3 * i] * T[4] + R[3 * i + 1] * T[5] + R[3 * i + 2] * T[6]);
  const double xc = R[0] * p[0] + R[1] * p[1] + R[2] * p[2] + t[0];
  const double yc = R[3] * p[0] + R[4] * p[1] + R[5] * p[2] + t[1];
  const double zc = R[6] * p[0] + R[7] * p[1] + R[8] * p[2] + t[2];
  const double x = xc / zc, y = yc / zc;
  for (int k = 0; k < 12; ++k) jc[k] = 0.0;
  jc[2] = -1.0;
  jc[6 + 3] = -1.0;
  if constexpr (E) {
    const double al = intr[4], be = intr[5];
    const double r2 = x * x + y * y;
    const double rho = sqrt(be * r2 + 1.0);
    const double nrm = al * rho + (1.0 - al);
    const double in2 = 1.0 / (nrm * nrm);
    const double da = (rho - 1.0) * in2;
    const double db = al * r2 * in2 / (2.0 * rho);
    jc[0] = -x / nrm;
    jc[6 + 1] = -y / nrm;
    jc[4] = intr[0] * x * da;
    jc[5] = intr[0] * x * db;
    jc[6 + 4] = intr[1] * y * da;
    jc[6 + 5] = intr[1] * y * db;
  } else {
    jc[0] = -x;
    jc[6 + 1] = -y;
  }
}

template <bool E>
__global__ void __launch_bounds__(kCovThreads) k_cov_groups(int64_t ng, const int64_t* __restrict__ g_begin,
                                                           const int32_t* __restrict__ g_pose,
                                                           const int32_t* __restrict__ g_pt,
                                                           const double* __restrict__ poses,
                                                           const double* __restrict__ points,
                                                           const double* __restrict__ intr, double* __restrict__ rec,
                                                           double* __restrict__ crec) {
  const int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (g >= ng) return;
  double jp[12], jm[6];
  const double* T = poses + 7 * static_cast<int64_t>(g_pose[g]);
  const double* P = points + 3 * static_cast<int64_t>(g_pt[g]);
  cov_jacobians<E>(T, P, intr, jp, jm);
  const double cnt = static_cast<double>(g_begin[g + 1] - g_begin[g]);
  double* o = rec + kCovRec * g;
  int k = 0;
  for (int a = 0; a < 6; ++a)
    for (int b = a; b < 6; ++b) o[k++] = cnt * (jp[a] * jp[b] + jp[6 + a] * jp[6 + b]);
  for (int a = 0; a < 6; ++a)
    for (int j = 0; j < 3; ++j) o[21 + 3 * a + j] = cnt * (jp[a] * jm[j] + jp[6 + a] * jm[3 + j]);
  k = 39;
  for (int i = 0; i < 3; ++i)
    for (int j = i; j < 3; ++j) o[k++] = cnt * (jm[i] * jm[j] + jm[3 + i] * jm[3 + j]);
  if (!crec) return;
  // free camera params: J_cam^T J_cam (21 upper), J_cam^T J_pose (6 x 6), J_cam^T J_point (6 x 3)
  double jc[12];
  cov_cam_jacobian<E>(T, P, intr, jc);
  double* oc = crec + kCovCamRec * g;
  k = 0;
  for (int a = 0; a < 6; ++a)
    for (int b = a; b < 6; ++b) oc[k++] = cnt * (jc[a] * jc[b] + jc[6 + a] * jc[6 + b]);
  for (int a = 0; a < 6; ++a)
    for (int b = 0; b < 6; ++b) oc[21 + 6 * a + b] = cnt * (jc[a] * jp[b] + jc[6 + a] * jp[6 + b]);
  for (int a = 0; a < 6; ++a)
    for (int j = 0; j < 3; ++j) oc[57 + 3 * a + j] = cnt * (jc[a] * jm[j] + jc[6 + a] * jm[3 + j]);
}

// nalgebra's 3x3 try_inverse: adjugate / determinant, singular iff det == 0
__device__ bool inverse3(const double* m, double* o) {
  const double m11 = m[0], m12 = m[1], m13 = m[2];
  const double m21 = m[3], m22 = m[4], m23 = m[5];
  const double m31 = m[6], m32 = m[7], m33 = m[8];
  const double c11 = m22 * m33 - m32 * m23;
  const double c21 = m21 * m33 - m31 * m23;
  const double c31 = m21 * m32 - m31 * m22;
  const double det = m11 * c11 - m12 * c21 + m13 * c31;
  if (det == 0.0) return false;
  o[0] = c11 / det;
  o[1] = (m13 * m32 - m33 * m12) / det;
  o[2] = (m12 * m23 - m22 * m13) / det;
  o[3] = -c21 / det;
  o[4] = (m11 * m33 - m31 * m13) / det;
  o[5] = (m13 * m21 - m23 * m11) / det;
  o[6] = c31 / det;
  o[7] = (m12 * m31 - m32 * m11) / det;
  o[8] = (m11 * m22 - m21 * m12) / det;
  return true;
}

__global__ void __launch_bounds__(kCovThreads) k_cov_points(int np, const int64_t* __restrict__ pt_g_begin,
                                                           const int32_t* __restrict__ g_pose,
                                                           const int32_t* __restrict__ pose_fb,
                                                           const int32_t* __restrict__ pt_mb,
                                                           const double* __restrict__ rec, double* __restrict__ vinv,
                                                           double* __restrict__ y, int* status,
                                                           const double* __restrict__ crec, double* __restrict__ wc,
                                                           double* __restrict__ yc) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= np) return;
  const int mb = pt_mb[q];
  if (mb < 0) return;
  double v[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t g = pt_g_begin[q]; g < pt_g_begin[q + 1]; ++g)
    for (int k = 0; k < 6; ++k) v[k] += rec[kCovRec * g + 39 + k];
  const double V[9] = {v[0], v[1], v[2], v[1], v[3], v[4], v[2], v[4], v[5]};
  double Vi[9];
  double* vo = vinv + 9 * static_cast<int64_t>(mb);
  if (!inverse3(V, Vi)) {
    for (int k = 0; k < 9; ++k) vo[k] = __longlong_as_double(0x7ff8000000000000ll);
    atomicOr(status + 1, 1);
    return;
  }
  for (int k = 0; k < 9; ++k) vo[k] = Vi[k];
  for (int64_t g = pt_g_begin[q]; g < pt_g_begin[q + 1]; ++g) {
    if (pose_fb[g_pose[g]] < 0) continue;
    const double* W = rec + kCovRec * g + 21;
    double* yo = y + 18 * g;
    for (int a = 0; a < 6; ++a)
      for (int j = 0; j < 3; ++j)
        yo[3 * a + j] = W[3 * a] * Vi[j] + W[3 * a + 1] * Vi[3 + j] + W[3 * a + 2] * Vi[6 + j];
  }
  if (!crec) return;
  // free camera params: W_cq = sum of the point's J_cam^T J_point, Y_cq = W_cq H_mm^-1
  double W[18];
  for (int k = 0; k < 18; ++k) W[k] = 0.0;
  for (int64_t g = pt_g_begin[q]; g < pt_g_begin[q + 1]; ++g)
    for (int k = 0; k < 18; ++k) W[k] += crec[kCovCamRec * g + 57 + k];
  double* wo = wc + 18 * static_cast<int64_t>(mb);
  double* yo = yc + 18 * static_cast<int64_t>(mb);
  for (int a = 0; a < 6; ++a)
    for (int j = 0; j < 3; ++j) {
      wo[3 * a + j] = W[3 * a + j];
      yo[3 * a + j] = W[3 * a] * Vi[j] + W[3 * a + 1] * Vi[3 + j] + W[3 * a + 2] * Vi[6 + j];
    }
}

// The camera block of S (free camera params, rows 0..5 of S; rows nk..5 are
// padding: identity): H_cc = sum over every term of J_cam^T J_cam, minus
// sum over the marginalized points of Y_cq W_cq^T.  One CTA; thread t sums
// terms and points t, t + 256, ...; the threads' sums by a fixed tree.
__global__ void __launch_bounds__(kCovThreads) k_cov_cam(int64_t ng, int nm, int nk, int n,
                                                        const double* __restrict__ crec,
                                                        const double* __restrict__ wc, const double* __restrict__ yc,
                                                        double* __restrict__ S, double* __restrict__ hcc) {
  __shared__ double red[kCovThreads];
  double h[21], sc[21];
  for (int k = 0; k < 21; ++k) h[k] = sc[k] = 0.0;
  for (int64_t g = threadIdx.x; g < ng; g += blockDim.x)
    for (int k = 0; k < 21; ++k) h[k] += crec[kCovCamRec * g + k];
  for (int mb = threadIdx.x; mb < nm; mb += blockDim.x) {
    const double* W = wc + 18 * static_cast<int64_t>(mb);
    const double* Y = yc + 18 * static_cast<int64_t>(mb);
    int k = 0;
    for (int a = 0; a < 6; ++a)
      for (int b = a; b < 6; ++b, ++k) sc[k] += Y[3 * a] * W[3 * b] + Y[3 * a + 1] * W[3 * b + 1] + Y[3 * a + 2] * W[3 * b + 2];
  }
  for (int part = 0; part < 2; ++part)
    for (int k = 0; k < 21; ++k) {
      red[threadIdx.x] = part == 0 ? h[k] : sc[k];
      __syncthreads();
      for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
      }
      if (threadIdx.x == 0) {
        if (part == 0) h[k] = red[0];
        else sc[k] = red[0];
      }
      __syncthreads();
    }
  if (threadIdx.x != 0) return;
  for (int a = 0; a < 6; ++a)
    for (int b = 0; b < 6; ++b) {
      const int k = a <= b ? up_idx(6, a, b) : up_idx(6, b, a);
      const bool real = a < nk && b < nk;
      hcc[6 * a + b] = real ? h[k] : 0.0;
      S[static_cast<int64_t>(a) * n + b] = real ? h[k] - sc[k] : (a == b ? 1.0 : 0.0);
    }
}

struct CovSArgs {
  int64_t nsb;
  int n;
  const int32_t* sb_row;
  const int32_t* sb_col;
  const int64_t* fb_tile_begin;
  const int64_t* tile_begin;
  const int64_t* tile_end;
  const int64_t* cam_g;
  const int32_t* g_pt;
  const int32_t* pt_mb;
  const double* rec;
  const double* y;
  const int32_t* prior_beg;  // per free block: its priors (null: none)
  const double* prior_out;
  const int32_t* e_beg;      // per free block: its edge records (null: none)
  const int32_t* e_slot;
  const double* e_out;
  const int32_t* eblk_begin;  // per lower block: its edge terms (bit 31: transposed)
  const int32_t* eblk_term;
  const double* e_hmn;
  double* S;
  double* hdiag;
  int nci;             // rows of the camera block before the poses (6 with free camera params, else 0)
  const double* crec;  // free camera params: per-term camera records (null: conditioned)
  const double* wc;    // per marginalized point W_cq (6 x 3)
  double* hcp;         // per free pose H_ca (camera rows x pose columns, 6 x 6)
};

// the term-list range of free pose fb (its camera tiles are contiguous in cam_g)
__device__ __forceinline__ void cam_range(const CovSArgs& a, int fb, int64_t* b, int64_t* e) {
  const int64_t t0 = a.fb_tile_begin[fb], t1 = a.fb_tile_begin[fb + 1];
  *b = t0 < t1 ? a.tile_begin[t0] : 0;
  *e = t0 < t1 ? a.tile_end[t1 - 1] : 0;
}

// acc (6x6, row-major) -= Y W^T
__device__ __forceinline__ void sub_ywt(double* acc, const double* Y, const double* W) {
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < 6; ++c)
      acc[6 * r + c] -= Y[3 * r] * W[3 * c] + Y[3 * r + 1] * W[3 * c + 1] + Y[3 * r + 2] * W[3 * c + 2];
}

// the 36 lane sums of a warp by a fixed shuffle tree (lane 0 holds the totals)
__device__ __forceinline__ void warp_sum36(double* acc) {
#pragma unroll
  for (int k = 0; k < 36; ++k)
    for (int off = 16; off > 0; off >>= 1) acc[k] += __shfl_down_sync(0xffffffffu, acc[k], off);
}

// A warp per lower block (fa, fb) of S.  Diagonal blocks: the lanes take
// pose fa's terms in turn.  Off-diagonal blocks: lane l merges its slice of
// pose fa's term list (1/32 of it, in point order) with pose fb's list from
// the first term at or after the slice's first point (one binary search).
__global__ void __launch_bounds__(128) k_cov_s(CovSArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t s = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  if (s >= a.nsb) return;  // the whole warp
  const int fa = a.sb_row[s], fb = a.sb_col[s];
  double acc[36];
#pragma unroll
  for (int k = 0; k < 36; ++k) acc[k] = 0.0;
  int64_t ib, ie;
  cam_range(a, fa, &ib, &ie);
  if (fa == fb) {
    for (int64_t i = ib + lane; i < ie; i += 32) {
      const double* h = a.rec + kCovRec * a.cam_g[i];
      for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 6; ++c) acc[6 * r + c] += h[r <= c ? up_idx(6, r, c) : up_idx(6, c, r)];
    }
    warp_sum36(acc);
    if (lane == 0) {
      if (a.prior_beg)
        for (int q = a.prior_beg[fa]; q < a.prior_beg[fa + 1]; ++q)
          for (int k = 0; k < 36; ++k) acc[k] += a.prior_out[static_cast<int64_t>(kPriorOut) * q + k];
      if (a.e_beg)
        for (int q = a.e_beg[fa]; q < a.e_beg[fa + 1]; ++q)
          for (int k = 0; k < 36; ++k) acc[k] += a.e_out[static_cast<int64_t>(kPriorOut) * a.e_slot[q] + k];
      for (int k = 0; k < 36; ++k) a.hdiag[36 * static_cast<int64_t>(fa) + k] = acc[k];
    }
    // the Schur part, then lane 0 adds back the H block it stored
#pragma unroll
    for (int k = 0; k < 36; ++k) acc[k] = 0.0;
    for (int64_t i = ib + lane; i < ie; i += 32) {
      const int64_t g = a.cam_g[i];
      if (a.pt_mb[a.g_pt[g]] < 0) continue;
      sub_ywt(acc, a.y + 18 * g, a.rec + kCovRec * g + 21);
    }
    warp_sum36(acc);
    if (lane == 0)
      for (int k = 0; k < 36; ++k) acc[k] += a.hdiag[36 * static_cast<int64_t>(fa) + k];
  } else {
    int64_t jb, je;
    cam_range(a, fb, &jb, &je);
    const int64_t len = ie - ib;
    int64_t i = ib + len * lane / 32;
    const int64_t iend = ib + len * (lane + 1) / 32;
    int64_t j = je;
    if (i < iend) {
      // first term of pose fb whose point is >= this slice's first point
      const int p0 = a.g_pt[a.cam_g[i]];
      int64_t lo = jb, hi = je;
      while (lo < hi) {
        const int64_t mid = lo + (hi - lo) / 2;
        if (a.g_pt[a.cam_g[mid]] < p0) lo = mid + 1;
        else hi = mid;
      }
      j = lo;
    }
    while (i < iend && j < je) {
      const int64_t gi = a.cam_g[i], gj = a.cam_g[j];
      const int pi = a.g_pt[gi], pj = a.g_pt[gj];
      if (pi < pj) {
        ++i;
      } else if (pj < pi) {
        ++j;
      } else {
        if (a.pt_mb[pi] >= 0) sub_ywt(acc, a.y + 18 * gi, a.rec + kCovRec * gj + 21);
        ++i;
        ++j;
      }
    }
    warp_sum36(acc);
    if (lane == 0 && a.eblk_begin)
      for (int q = a.eblk_begin[s]; q < a.eblk_begin[s + 1]; ++q) {
        const int32_t tt = a.eblk_term[q];
        const int64_t term = tt & 0x7fffffff;
        for (int r = 0; r < 6; ++r)
          for (int c = 0; c < 6; ++c)
            acc[6 * r + c] += (tt < 0) ? a.e_hmn[36 * term + c * 6 + r] : a.e_hmn[36 * term + r * 6 + c];
      }
  }
  const int64_t n = a.n;
  if (lane == 0)
    for (int r = 0; r < 6; ++r)
      for (int c = 0; c < 6; ++c) {
        // the diagonal block from its lower triangle (exactly symmetric)
        const double v = (fa == fb && c > r) ? acc[6 * c + r] : acc[6 * r + c];
        const int64_t row = a.nci + 6 * fa + r, col = a.nci + 6 * fb + c;
        a.S[row * n + col] = v;
        a.S[col * n + row] = v;
      }
  if (fa != fb || !a.crec) return;
  // free camera params: the pose's camera columns S_ac = H_ac - sum over its
  // terms with a marginalized point of Y_g W_cq^T (acc[6 r + k]: pose row r, camera column k)
#pragma unroll
  for (int k = 0; k < 36; ++k) acc[k] = 0.0;
  for (int64_t i = ib + lane; i < ie; i += 32) {
    const double* hc = a.crec + kCovCamRec * a.cam_g[i] + 21;
    for (int k = 0; k < 6; ++k)
      for (int r = 0; r < 6; ++r) acc[6 * r + k] += hc[6 * k + r];
  }
  warp_sum36(acc);
  if (lane == 0)
    for (int k = 0; k < 6; ++k)
      for (int r = 0; r < 6; ++r) a.hcp[36 * static_cast<int64_t>(fa) + 6 * k + r] = acc[6 * r + k];
#pragma unroll
  for (int k = 0; k < 36; ++k) acc[k] = 0.0;
  for (int64_t i = ib + lane; i < ie; i += 32) {
    const int64_t g = a.cam_g[i];
    const int mb = a.pt_mb[a.g_pt[g]];
    if (mb < 0) continue;
    sub_ywt(acc, a.y + 18 * g, a.wc + 18 * static_cast<int64_t>(mb));
  }
  warp_sum36(acc);
  if (lane != 0) return;
  for (int r = 0; r < 6; ++r)
    for (int k = 0; k < 6; ++k) {
      const double v = a.hcp[36 * static_cast<int64_t>(fa) + 6 * k + r] + acc[6 * r + k];
      const int64_t row = a.nci + 6 * fa + r;
      a.S[row * n + k] = v;
      a.S[static_cast<int64_t>(k) * n + row] = v;
    }
}

// ---------------------------------------------------------------------------
// LDL^T
// ---------------------------------------------------------------------------

// dense_ldlt.rs:164-230 on the 6x6 block a (row-major, lower used): unit-lower
// L in a, pivots in d.  Returns 0, 1 for a non-finite pivot, 2 for an
// indefinite block whose pivot condition is below the Bunch-Kaufman threshold.
__device__ int ldlt6(double* a, double* d) {
  double maxp = 1.0, minp = DBL_MAX;
  int rank = 0;
  bool neg = false;
  for (int j = 0; j < 6; ++j) {
    for (int k = 0; k < j; ++k) {
      double s = a[6 * j + k];
      for (int p = 0; p < k; ++p) s -= a[6 * j + p] * d[p] * a[6 * k + p];
      const double tol = fmax(maxp, 1.0) * kCovTolRel;
      a[6 * j + k] = (fabs(d[k]) <= tol) ? 0.0 : s / d[k];
    }
    double djj = a[6 * j + j];
    for (int p = 0; p < j; ++p) djj -= d[p] * a[6 * j + p] * a[6 * j + p];
    if (!isfinite(djj)) return 1;
    const double tol = fmax(maxp, 1.0) * kCovTolRel;
    if (fabs(djj) <= tol) {
      d[j] = 0.0;
    } else {
      if (djj < 0.0) neg = true;
      d[j] = djj;
      maxp = fmax(maxp, fabs(djj));
      minp = fmin(minp, fabs(djj));
      rank += 1;
    }
    a[6 * j + j] = 1.0;
  }
  for (int r = 0; r < 6; ++r)
    for (int c = r + 1; c < 6; ++c) a[6 * r + c] = 0.0;
  const double cond = rank == 0 ? 0.0 : minp / maxp;
  return (neg && cond < 1e-10) ? 2 : 0;
}

// Step k: the diagonal block's factor (every CTA, in shared memory; CTA 0
// publishes it) and L of the rows below: L_i = c_i L_kk^-T D^+.
__global__ void __launch_bounds__(kCovThreads) k_cov_panel(int n, int k, double* S, double* ldiag, double* dpiv,
                                                          int* status) {
  __shared__ double L6[36], d6[6];
  const int c0 = 6 * k;
  if (threadIdx.x == 0) {
    double a[36], d[6];
    for (int r = 0; r < 6; ++r)
      for (int c = 0; c < 6; ++c) a[6 * r + c] = c <= r ? S[static_cast<int64_t>(c0 + r) * n + c0 + c] : 0.0;
    const int st = ldlt6(a, d);
    for (int e = 0; e < 36; ++e) L6[e] = a[e];
    for (int e = 0; e < 6; ++e) d6[e] = d[e];
    if (blockIdx.x == 0) {
      for (int e = 0; e < 36; ++e) ldiag[36 * static_cast<int64_t>(k) + e] = a[e];
      for (int e = 0; e < 6; ++e) dpiv[c0 + e] = d[e];
      if (st) atomicMax(status, st);
    }
  }
  __syncthreads();
  const int i = c0 + 6 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double* row = S + static_cast<int64_t>(i) * n + c0;
  double yv[6];
  for (int j = 0; j < 6; ++j) {
    double v = row[j];
    for (int t = 0; t < j; ++t) v -= yv[t] * L6[6 * j + t];
    yv[j] = v;
  }
  for (int j = 0; j < 6; ++j) row[j] = d6[j] == 0.0 ? 0.0 : yv[j] / d6[j];
}

// Step k: C_ij -= sum_t L_it d_t L_jt on the lower trailing triangle, 32 x 32
// tiles (tiles above the diagonal return at once).
__global__ void __launch_bounds__(kCovThreads) k_cov_update(int n, int k, double* S, const double* dpiv) {
  const int base = 6 * k + 6;
  const int ti = blockIdx.y, tj = blockIdx.x;
  if (tj > ti) return;
  __shared__ double Li[kUT][7], Lj[kUT][7];
  const int i0 = base + ti * kUT, j0 = base + tj * kUT;
  for (int e = threadIdx.x; e < kUT * 6; e += blockDim.x) {
    const int r = e / 6, t = e % 6;
    Li[r][t] = (i0 + r < n) ? S[static_cast<int64_t>(i0 + r) * n + 6 * k + t] : 0.0;
    Lj[r][t] = (j0 + r < n) ? S[static_cast<int64_t>(j0 + r) * n + 6 * k + t] * dpiv[6 * k + t] : 0.0;
  }
  __syncthreads();
  const int jj = threadIdx.x & 31;
  const int j = j0 + jj;
  if (j >= n) return;
  for (int ii = threadIdx.x >> 5; ii < kUT; ii += blockDim.x >> 5) {
    const int i = i0 + ii;
    if (i >= n || j > i) continue;
    double s = 0.0;
    for (int t = 0; t < 6; ++t) s += Li[ii][t] * Lj[jj][t];
    S[static_cast<int64_t>(i) * n + j] -= s;
  }
}

// ---------------------------------------------------------------------------
// Inverse from the factor (Takahashi), block row i (rows r0 = 6i .. r0 + 5),
// three launches: the sums over the rows m >= 6i + 6 split over ranges of m
// (enough CTAs to fill the GPU when few columns remain), the finish (sums in
// range order, the 6-row recurrence, the row and its mirror, and per CTA the
// diagonal block's sums over the new row), the diagonal block.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kCovThreads) k_cov_inv_part(int n, int i, int kchunk, const double* __restrict__ L,
                                                             const double* __restrict__ Z, double* __restrict__ part) {
  const int r0 = 6 * i, cb = r0 + 6, ncols = n - cb;
  const int c = cb + blockIdx.x * blockDim.x + threadIdx.x;
  const int mbeg = cb + blockIdx.y * kchunk, mend = min(n, mbeg + kchunk);
  __shared__ double Ls[kInvRows][6];
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int m0 = mbeg; m0 < mend; m0 += kInvRows) {
    __syncthreads();
    for (int e = threadIdx.x; e < kInvRows * 6; e += blockDim.x) {
      const int mm = e / 6, t = e % 6;
      Ls[mm][t] = (m0 + mm < mend) ? L[static_cast<int64_t>(m0 + mm) * n + r0 + t] : 0.0;
    }
    __syncthreads();
    if (c < n) {
      const int cnt = min(kInvRows, mend - m0);
      const double* zc = Z + static_cast<int64_t>(m0) * n + c;
      for (int mm = 0; mm < cnt; ++mm) {
        const double z = zc[static_cast<int64_t>(mm) * n];
#pragma unroll
        for (int t = 0; t < 6; ++t) acc[t] += Ls[mm][t] * z;
      }
    }
  }
  if (c < n)
    for (int t = 0; t < 6; ++t) part[(static_cast<int64_t>(blockIdx.y) * 6 + t) * ncols + (c - cb)] = acc[t];
}

__global__ void __launch_bounds__(kCovThreads) k_cov_inv_fin(int n, int i, int nk, const double* __restrict__ L,
                                                            const double* __restrict__ ldiag, double* Z,
                                                            const double* __restrict__ part,
                                                            double* __restrict__ dpart) {
  const int r0 = 6 * i, cb = r0 + 6, ncols = n - cb;
  const int c = cb + blockIdx.x * blockDim.x + threadIdx.x;
  double prod[36];
#pragma unroll
  for (int k = 0; k < 36; ++k) prod[k] = 0.0;
  if (c < n) {
    double acc[6];
    for (int t = 0; t < 6; ++t) {
      double s = 0.0;
      for (int ks = 0; ks < nk; ++ks) s += part[(static_cast<int64_t>(ks) * 6 + t) * ncols + (c - cb)];
      acc[t] = s;
    }
    const double* Lb = ldiag + 36 * static_cast<int64_t>(i);
    double z[6];
    for (int t = 5; t >= 0; --t) {
      double v = -acc[t];
      for (int m = t + 1; m < 6; ++m) v -= Lb[6 * m + t] * z[m];
      z[t] = v;
    }
    for (int t = 0; t < 6; ++t) {
      Z[static_cast<int64_t>(r0 + t) * n + c] = z[t];
      Z[static_cast<int64_t>(c) * n + r0 + t] = z[t];
    }
    // the diagonal block's sums over m >= cb: L_m,r0+t Z_m,r0+u with Z_m,r0+u = z_u of column m = c
    const double* lc = L + static_cast<int64_t>(c) * n + r0;
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      const double l = lc[t];
#pragma unroll
      for (int u = 0; u < 6; ++u) prod[6 * t + u] = l * z[u];
    }
  }
  // CTA sums in a fixed order: a shuffle tree per warp, then the warps in order
  __shared__ double ws[kCovThreads / 32][36];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 36; ++k) {
    double v = prod[k];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) ws[warp][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < 36) {
    double s = 0.0;
    for (int w = 0; w < kCovThreads / 32; ++w) s += ws[w][threadIdx.x];
    dpart[36 * static_cast<int64_t>(blockIdx.x) + threadIdx.x] = s;
  }
}

// The 6x6 diagonal block: the finish CTAs' sums in order, then the recurrence
// (columns last to first within each row, rows last to first) in one thread.
__global__ void __launch_bounds__(64) k_cov_inv_diag(int n, int i, int nfin, const double* __restrict__ ldiag,
                                                    const double* __restrict__ dpiv, const double* __restrict__ dpart,
                                                    double* Z) {
  const int r0 = 6 * i;
  __shared__ double acc[36];
  if (threadIdx.x < 36) {
    double s = 0.0;
    for (int b = 0; b < nfin; ++b) s += dpart[36 * static_cast<int64_t>(b) + threadIdx.x];
    acc[threadIdx.x] = s;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  const double* Lb = ldiag + 36 * static_cast<int64_t>(i);
  double Zd[36];
  for (int t = 5; t >= 0; --t)
    for (int u = 5; u >= t; --u) {
      const double dv = dpiv[r0 + t];
      double v = (u == t && dv != 0.0) ? 1.0 / dv : 0.0;
      v -= acc[6 * t + u];
      for (int m = t + 1; m < 6; ++m) v -= Lb[6 * m + t] * (m <= u ? Zd[6 * m + u] : Zd[6 * u + m]);
      Zd[6 * t + u] = v;
    }
  for (int t = 0; t < 6; ++t)
    for (int u = t; u < 6; ++u) {
      Z[static_cast<int64_t>(r0 + t) * n + r0 + u] = Zd[6 * t + u];
      Z[static_cast<int64_t>(r0 + u) * n + r0 + t] = Zd[6 * t + u];
    }
}

// ---------------------------------------------------------------------------
// Pseudo-inverse pieces
// ---------------------------------------------------------------------------

// C[i][j] = sum_k A(i, k) w_k B(k, j) (w null: 1), A(i, k) = A[i a_i + k a_k],
// B(k, j) = B[k b_k + j b_j]; 64 x 64 tiles, 16 deep, 4 x 4 per thread.
__global__ void __launch_bounds__(256) k_cov_gemm(int M, int N, int K, const double* __restrict__ A, int64_t a_i,
                                                 int64_t a_k, const double* __restrict__ w,
                                                 const double* __restrict__ B, int64_t b_k, int64_t b_j,
                                                 double* __restrict__ C, int64_t ldc) {
  __shared__ double As[kGK][kGT + 1], Bs[kGK][kGT + 1];
  const int i0 = blockIdx.y * kGT, j0 = blockIdx.x * kGT;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[4][4];
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) acc[r][c] = 0.0;
  for (int k0 = 0; k0 < K; k0 += kGK) {
    for (int e = threadIdx.x; e < kGK * kGT; e += blockDim.x) {
      const int kk = e / kGT, ii = e % kGT;
      const int k = k0 + kk;
      const int i = i0 + ii, j = j0 + ii;
      double v = (i < M && k < K) ? A[i * a_i + k * a_k] : 0.0;
      if (w && k < K) v *= w[k];
      As[kk][ii] = v;
      Bs[kk][ii] = (j < N && k < K) ? B[k * b_k + j * b_j] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < kGK; ++kk) {
      double av[4], bv[4];
      for (int r = 0; r < 4; ++r) av[r] = As[kk][ty + 16 * r];
      for (int c = 0; c < 4; ++c) bv[c] = Bs[kk][tx + 16 * c];
      for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) acc[r][c] += av[r] * bv[c];
    }
    __syncthreads();
  }
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      const int i = i0 + ty + 16 * r, j = j0 + tx + 16 * c;
      if (i < M && j < N) C[i * ldc + j] = acc[r][c];
    }
}

// E (n x r): the columns J of the scalar unit-lower L (diagonal blocks from
// ldiag, the rest from the factored S).
__global__ void k_cov_build_e(int n, int r, const double* __restrict__ L, const double* __restrict__ ldiag,
                              const int32_t* __restrict__ J, double* __restrict__ E) {
  const int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (e >= static_cast<int64_t>(n) * r) return;
  const int row = static_cast<int>(e / r), c = static_cast<int>(e % r);
  const int col = J[c];
  double v;
  if (row < col) v = 0.0;
  else if (row / 6 == col / 6) v = ldiag[36 * static_cast<int64_t>(row / 6) + 6 * (row % 6) + col % 6];
  else v = L[static_cast<int64_t>(row) * n + col];
  E[e] = v;
}

// rows / columns r..rp-1 of the padded G: identity
__global__ void k_cov_pad_identity(int r, int rp, double* G) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= rp * rp) return;
  const int i = e / rp, j = e % rp;
  if (i >= r || j >= r) G[e] = (i == j) ? 1.0 : 0.0;
}

__global__ void k_cov_recip(int r, const int32_t* __restrict__ J, const double* __restrict__ dpiv,
                            double* __restrict__ w) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < r) w[c] = 1.0 / dpiv[J[c]];
}

// ---------------------------------------------------------------------------
// Queries
// ---------------------------------------------------------------------------
struct CovQArgs {
  int nq, mode, nc, np, n;
  int nci, nk;  // free camera params: rows of their block in S (6) and their count (4 or 6); else 0, 0
  const int32_t* q;
  const int32_t* pose_fb;
  const int32_t* pt_mb;
  const int64_t* pt_g_begin;
  const int32_t* g_pose;
  const double* rec;
  const double* y;
  const double* vinv;
  const double* Z;
  const double* hdiag;
  const double* wc;   // free camera params: W_cq, Y_cq per marginalized point, H_cc, H_ca per free pose
  const double* yc;
  const double* hcc;
  const double* hcp;
  int n_eterm;
  const int32_t* eterm_fm;
  const int32_t* eterm_fn;
  const double* e_hmn;
  double* out;
  int32_t* dims;
};

// (kind, index) -> block: camera 0 (index 0, free params only) -> 0, pose 1
// -> free block, point 2 -> marg block; -1: none
__device__ __forceinline__ int cov_resolve(const CovQArgs& a, int kind, int idx, int* dim) {
  if (kind == 0 && idx == 0 && a.nci > 0) {
    *dim = a.nk;
    return 0;
  }
  if (kind == 1 && idx >= 0 && idx < a.nc) {
    *dim = 6;
    return a.pose_fb[idx];
  }
  if (kind == 2 && idx >= 0 && idx < a.np) {
    *dim = 3;
    return a.pt_mb[idx];
  }
  *dim = 0;
  return -1;
}

// Z row / column of a free variable's block: the camera at 0, pose fb after it
__device__ __forceinline__ int64_t cov_zoff(const CovQArgs& a, int kind, int blk) {
  return kind == 0 ? 0 : a.nci + 6 * static_cast<int64_t>(blk);
}

// sum over the free blocks f of point pt (its terms with a free pose, then the
// camera when its params are free) of Z[row, f] Y_f[:, col]
__device__ double cov_row_times_y(const CovQArgs& a, int64_t row, int pt, int mb, int col) {
  double v = 0.0;
  const double* zr = a.Z + row * a.n;
  for (int64_t g = a.pt_g_begin[pt]; g < a.pt_g_begin[pt + 1]; ++g) {
    const int gb = a.pose_fb[a.g_pose[g]];
    if (gb < 0) continue;
    const double* Y = a.y + 18 * g;
    const double* z = zr + a.nci + 6 * static_cast<int64_t>(gb);
    for (int k = 0; k < 6; ++k) v += z[k] * Y[3 * k + col];
  }
  if (a.nci > 0) {
    const double* Y = a.yc + 18 * static_cast<int64_t>(mb);
    for (int k = 0; k < a.nk; ++k) v += zr[k] * Y[3 * k + col];
  }
  return v;
}

__global__ void __launch_bounds__(64) k_cov_query(CovQArgs a) {
  const int qi = blockIdx.x;
  const int32_t* q = a.q + 4 * qi;
  int rd = 0, cd = 0;
  const int rb = cov_resolve(a, q[0], q[1], &rd), cb = cov_resolve(a, q[2], q[3], &cd);
  const int e = threadIdx.x;
  double* o = a.out + 36 * static_cast<int64_t>(qi);
  if (e < 36) o[e] = 0.0;
  if (rb < 0 || cb < 0) {
    if (e == 0) a.dims[2 * qi] = a.dims[2 * qi + 1] = 0;  // no block (the reference's None)
    return;
  }
  const int rk = q[0], ck = q[2];
  const bool rf = rk != 2, cf = ck != 2;  // free (camera or pose) or marginalized (point)
  const int64_t n = a.n;
  // a query on a point whose H_mm is singular has no covariance
  const bool bad = a.mode == 0 && ((!rf && isnan(a.vinv[9 * static_cast<int64_t>(rb)])) ||
                                   (!cf && isnan(a.vinv[9 * static_cast<int64_t>(cb)])));
  if (e == 0) {
    a.dims[2 * qi] = bad ? -1 : rd;
    a.dims[2 * qi + 1] = bad ? -1 : cd;
  }
  if (bad || e >= rd * cd) return;
  const int r = e / cd, c = e % cd;
  const int rp = q[1], cp = q[3];  // the variables' own indices
  double v = 0.0;
  if (a.mode == 1) {
    // precision: blocks of the undamped H
    if (rk == 0 && ck == 0) {
      v = a.hcc[6 * r + c];
    } else if (rk == 0 || ck == 0) {
      const int other = rk == 0 ? ck : rk, ob = rk == 0 ? cb : rb;
      const int cr = rk == 0 ? r : c, oc = rk == 0 ? c : r;  // camera row, the other block's column
      v = other == 1 ? a.hcp[36 * static_cast<int64_t>(ob) + 6 * cr + oc] : a.wc[18 * static_cast<int64_t>(ob) + 3 * cr + oc];
    } else if (rf && cf) {
      if (rb == cb) {
        v = a.hdiag[36 * static_cast<int64_t>(rb) + 6 * r + c];
      } else {
        for (int t = 0; t < a.n_eterm; ++t) {
          if (a.eterm_fm[t] == rb && a.eterm_fn[t] == cb) v += a.e_hmn[36 * static_cast<int64_t>(t) + 6 * r + c];
          if (a.eterm_fn[t] == rb && a.eterm_fm[t] == cb) v += a.e_hmn[36 * static_cast<int64_t>(t) + 6 * c + r];
        }
      }
    } else if (rf != cf) {
      const int pose = rf ? rp : cp, pt = rf ? cp : rp;
      const int pr = rf ? r : c, pc = rf ? c : r;  // (pose row, point column) of W
      for (int64_t g = a.pt_g_begin[pt]; g < a.pt_g_begin[pt + 1]; ++g)
        if (a.g_pose[g] == pose) v = a.rec[kCovRec * g + 21 + 3 * pr + pc];
    } else if (rp == cp) {
      for (int64_t g = a.pt_g_begin[rp]; g < a.pt_g_begin[rp + 1]; ++g)
        v += a.rec[kCovRec * g + 39 + (r <= c ? up_idx(3, r, c) : up_idx(3, c, r))];
    }
  } else if (rf && cf) {
    v = a.Z[(cov_zoff(a, rk, rb) + r) * n + cov_zoff(a, ck, cb) + c];
  } else if (rf != cf) {
    // -(S^-1[free rows, :] H_fm) H_mm^-1 = -sum over the point's free blocks of Z[rows, block] Y
    const int fk = rf ? rk : ck, fbk = rf ? rb : cb, pt = rf ? cp : rp, mb = rf ? cb : rb;
    const int pr = rf ? r : c, pc = rf ? c : r;
    v = -cov_row_times_y(a, cov_zoff(a, fk, fbk) + pr, pt, mb, pc);
  } else {
    // H_mm[i]^-1 delta_ij + sum over the free blocks g of point i and h of point j of Y_g^T Z[g, h] Y_h
    for (int64_t g = a.pt_g_begin[rp]; g < a.pt_g_begin[rp + 1]; ++g) {
      const int gb = a.pose_fb[a.g_pose[g]];
      if (gb < 0) continue;
      const double* Yg = a.y + 18 * g;
      for (int k = 0; k < 6; ++k)
        v += Yg[3 * k + r] * cov_row_times_y(a, a.nci + 6 * static_cast<int64_t>(gb) + k, cp, cb, c);
    }
    if (a.nci > 0) {
      const double* Yc = a.yc + 18 * static_cast<int64_t>(rb);
      for (int k = 0; k < a.nk; ++k) v += Yc[3 * k + r] * cov_row_times_y(a, k, cp, cb, c);
    }
    if (rp == cp) v += a.vinv[9 * static_cast<int64_t>(rb) + 3 * r + c];
  }
  o[e] = v;
}

inline unsigned blocks_for(int64_t n, int t) { return static_cast<unsigned>((n + t - 1) / t); }

}  // namespace

int launch_cov_assemble(const Sizes& s, const Dev& d, const CovBufs& c, cudaStream_t st) {
  int nl = 0;
  if (s.ng > 0) {
    if (s.eucm)
      k_cov_groups<true><<<blocks_for(s.ng, kCovThreads), kCovThreads, 0, st>>>(s.ng, d.g_begin, d.g_pose, d.g_pt,
                                                                               d.poses, d.points, d.intr, c.rec,
                                                                               c.crec);
    else
      k_cov_groups<false><<<blocks_for(s.ng, kCovThreads), kCovThreads, 0, st>>>(s.ng, d.g_begin, d.g_pose, d.g_pt,
                                                                                d.poses, d.points, d.intr, c.rec,
                                                                                c.crec);
    ++nl;
  }
  if (s.np > 0) {
    k_cov_points<<<blocks_for(s.np, kCovThreads), kCovThreads, 0, st>>>(s.np, d.pt_g_begin, d.g_pose, d.pose_fb,
                                                                       d.pt_mb, c.rec, c.vinv, c.y, c.status, c.crec,
                                                                       c.wc, c.yc);
    ++nl;
  }
  if (c.crec) {
    k_cov_cam<<<1, kCovThreads, 0, st>>>(s.ng, s.nm, c.nk, c.n, c.crec, c.wc, c.yc, c.S, c.hcc);
    ++nl;
  }
  if (s.nsb > 0) {
    CovSArgs a{};
    a.nsb = s.nsb;
    a.n = c.n;
    a.sb_row = d.sb_row;
    a.sb_col = d.sb_col;
    a.fb_tile_begin = d.fb_tile_begin;
    a.tile_begin = d.tile_begin;
    a.tile_end = d.tile_end;
    a.cam_g = d.cam_g;
    a.g_pt = d.g_pt;
    a.pt_mb = d.pt_mb;
    a.rec = c.rec;
    a.y = c.y;
    a.prior_beg = s.n_prior > 0 ? d.prior_fb_begin : nullptr;
    a.prior_out = d.prior_out;
    a.e_beg = s.n_edge > 0 ? d.efb_begin : nullptr;
    a.e_slot = d.efb_slot;
    a.e_out = d.edge_out;
    a.eblk_begin = s.n_edge > 0 ? d.eblk_begin : nullptr;
    a.eblk_term = d.eblk_term;
    a.e_hmn = d.edge_hmn;
    a.S = c.S;
    a.hdiag = c.hdiag;
    a.nci = c.nci;
    a.crec = c.crec;
    a.wc = c.wc;
    a.hcp = c.hcp;
    k_cov_s<<<blocks_for(32 * s.nsb, 128), 128, 0, st>>>(a);
    ++nl;
  }
  return nl;
}

int launch_cov_factor(int n, double* S, double* ldiag, double* dpiv, int* status, cudaStream_t st) {
  const int nb = n / 6;
  int nl = 0;
  for (int k = 0; k < nb; ++k) {
    const int below = n - 6 * k - 6;
    k_cov_panel<<<below > 0 ? blocks_for(below, kCovThreads) : 1, kCovThreads, 0, st>>>(n, k, S, ldiag, dpiv,
                                                                                        status);
    ++nl;
    if (below > 0) {
      const unsigned t = blocks_for(below, kUT);
      k_cov_update<<<dim3(t, t), kCovThreads, 0, st>>>(n, k, S, dpiv);
      ++nl;
    }
  }
  return nl;
}

size_t cov_inverse_work(int n) {
  return static_cast<size_t>(kInvSplitMax) * 6 * n + static_cast<size_t>((n + kCovThreads - 1) / kCovThreads) * 36 + 64;
}

int launch_cov_inverse(int n, const double* L, const double* ldiag, const double* dpiv, double* Z, double* work,
                       cudaStream_t st) {
  const int nb = n / 6;
  int nl = 0;
  int num_sms = 152;
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
  double* part = work;
  double* dpart = work + static_cast<size_t>(kInvSplitMax) * 6 * n;
  for (int i = nb - 1; i >= 0; --i) {
    const int cols = n - 6 * i - 6;
    int nfin = 0;
    if (cols > 0) {
      nfin = static_cast<int>(blocks_for(cols, kCovThreads));
      // split the rows m so that about two CTAs per SM run, each range at least kInvMinRows rows
      int nk = (2 * num_sms + nfin - 1) / nfin;
      nk = std::max(1, std::min({nk, kInvSplitMax, cols / kInvMinRows}));
      const int kchunk = (cols + nk - 1) / nk;
      k_cov_inv_part<<<dim3(nfin, nk), kCovThreads, 0, st>>>(n, i, kchunk, L, Z, part);
      k_cov_inv_fin<<<nfin, kCovThreads, 0, st>>>(n, i, nk, L, ldiag, Z, part, dpart);
      nl += 2;
    }
    k_cov_inv_diag<<<1, 64, 0, st>>>(n, i, nfin, ldiag, dpiv, dpart, Z);
    ++nl;
  }
  return nl;
}

namespace {
void gemm(int M, int N, int K, const double* A, int64_t a_i, int64_t a_k, const double* w, const double* B,
          int64_t b_k, int64_t b_j, double* C, int64_t ldc, cudaStream_t st) {
  if (M <= 0 || N <= 0) return;
  k_cov_gemm<<<dim3(blocks_for(N, kGT), blocks_for(M, kGT)), 256, 0, st>>>(M, N, K, A, a_i, a_k, w, B, b_k, b_j, C,
                                                                          ldc);
}
}  // namespace

cudaError_t cov_pinv(int n, const double* L, const double* ldiag, const double* dpiv, const std::vector<int32_t>& J,
                     double* Z, cudaMemPool_t pool, cudaStream_t st, int* g_ok) {
  *g_ok = 1;
  const int r = static_cast<int>(J.size());
  if (r == 0) return cudaMemsetAsync(Z, 0, sizeof(double) * n * static_cast<size_t>(n), st);
  const int rp = (r + 5) / 6 * 6;
  const size_t nr = static_cast<size_t>(n) * r;
  auto rnd = [](size_t b) { return (b + 255) / 256 * 256; };
  const size_t rr = static_cast<size_t>(r) * r, rpp = static_cast<size_t>(rp) * rp;
  const size_t bytes = rnd(sizeof(int32_t) * r) + 2 * rnd(sizeof(double) * nr) + 2 * rnd(sizeof(double) * rpp) +
                       rnd(sizeof(double) * rr) + rnd(sizeof(double) * r) + rnd(sizeof(double) * rp) +
                       rnd(sizeof(double) * (rp / 6) * 36) + rnd(sizeof(int) * 4) +
                       rnd(sizeof(double) * cov_inverse_work(rp));
  void* buf = nullptr;
  cudaError_t e = cudaMallocFromPoolAsync(&buf, bytes, pool, st);
  if (e != cudaSuccess) return e;
  char* p = static_cast<char*>(buf);
  auto take = [&p](size_t b) {
    void* v = p;
    p += (b + 255) / 256 * 256;
    return v;
  };
  int32_t* dJ = static_cast<int32_t*>(take(sizeof(int32_t) * r));
  double* E = static_cast<double*>(take(sizeof(double) * nr));
  double* F = static_cast<double*>(take(sizeof(double) * nr));
  double* G = static_cast<double*>(take(sizeof(double) * rp * rp));
  double* Gi = static_cast<double*>(take(sizeof(double) * rp * rp));
  double* M = static_cast<double*>(take(sizeof(double) * r * r));
  double* w = static_cast<double*>(take(sizeof(double) * r));
  double* gpiv = static_cast<double*>(take(sizeof(double) * rp));
  double* gdiag = static_cast<double*>(take(sizeof(double) * (rp / 6) * 36));
  int* gst = static_cast<int*>(take(sizeof(int) * 4));
  double* gwork = static_cast<double*>(take(sizeof(double) * cov_inverse_work(rp)));
  std::vector<double> hpiv(rp);
  e = cudaMemcpyAsync(dJ, J.data(), sizeof(int32_t) * r, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(gst, 0, sizeof(int) * 4, st);
  if (e == cudaSuccess) {
    k_cov_build_e<<<blocks_for(static_cast<int64_t>(nr), 256), 256, 0, st>>>(n, r, L, ldiag, dJ, E);
    // G = E^T E (r x r inside the rp x rp padded matrix, identity padding)
    gemm(r, r, n, E, 1, r, nullptr, E, r, 1, G, rp, st);
    k_cov_pad_identity<<<blocks_for(static_cast<int64_t>(rp) * rp, 256), 256, 0, st>>>(r, rp, G);
    launch_cov_factor(rp, G, gdiag, gpiv, gst, st);
    e = cudaMemcpyAsync(hpiv.data(), gpiv, sizeof(double) * rp, cudaMemcpyDeviceToHost, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) {
    for (int k = 0; k < r; ++k)
      if (!(hpiv[k] > 0.0)) *g_ok = 0;  // G is positive definite on the positive-pivot subspace
  }
  if (e == cudaSuccess && *g_ok) {
    launch_cov_inverse(rp, G, gdiag, gpiv, Gi, gwork, st);
    k_cov_recip<<<blocks_for(r, 256), 256, 0, st>>>(r, dJ, dpiv, w);
    gemm(r, r, r, Gi, rp, 1, w, Gi, rp, 1, M, r, st);   // M = G^-1 diag(d_J)^-1 G^-1
    gemm(n, r, r, E, r, 1, nullptr, M, r, 1, F, r, st);  // F = E M
    gemm(n, n, r, F, r, 1, nullptr, E, 1, r, Z, n, st);  // Z = F E^T
    e = cudaGetLastError();
  }
  const cudaError_t ef = cudaFreeAsync(buf, st);
  return e != cudaSuccess ? e : ef;
}

cudaError_t launch_cov_query(const Sizes& s, const Dev& d, const CovBufs& c, int mode, int nq, const int32_t* q,
                             double* out, int32_t* dims, cudaStream_t st) {
  if (nq <= 0) return cudaSuccess;
  CovQArgs a{};
  a.nq = nq;
  a.mode = mode;
  a.nc = s.nc;
  a.np = s.np;
  a.n = c.n;
  a.q = q;
  a.pose_fb = d.pose_fb;
  a.pt_mb = d.pt_mb;
  a.pt_g_begin = d.pt_g_begin;
  a.g_pose = d.g_pose;
  a.rec = c.rec;
  a.y = c.y;
  a.vinv = c.vinv;
  a.Z = c.Z;
  a.hdiag = c.hdiag;
  a.nci = c.nci;
  a.nk = c.nk;
  a.wc = c.wc;
  a.yc = c.yc;
  a.hcc = c.hcc;
  a.hcp = c.hcp;
  a.n_eterm = s.n_edge > 0 ? s.n_eterm : 0;
  a.eterm_fm = d.eterm_fm;
  a.eterm_fn = d.eterm_fn;
  a.e_hmn = d.edge_hmn;
  a.out = out;
  a.dims = dims;
  k_cov_query<<<nq, 64, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace sgba
