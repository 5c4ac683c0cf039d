// sgba_prior.cu -- cost functions on the poses alone, on the GPU: the pose
// prior (Isometry3PriorCostTerm,
// crates/sophus_opt/src/nlls/functor_library/costs/isometry3_prior.rs) and
// the pose-graph edge (PoseGraph3CostTerm, .../costs/pose_graph3.rs).
//
// Each prior k on pose j has a mean E_k and a 6x6 precision W_k; its residual
// is g = log(T_j E_k^-1) and its Jacobian J the derivative of
// log(exp(x) T_j E_k^-1) at x = 0, taken here by forward-mode derivatives in
// f64 (sgba_lie.cuh).  EvaluatedCostTerm::make
// (crates/sophus_opt/src/nlls/cost/evaluated_term.rs:286-327) then gives the
// Hessian block J^T W J, the gradient J^T W g and the cost g^T W g.  The
// priors are few (at most one group per pose) and run in f64 in one CTA; the
// blocks go to the pose's diagonal block in k_camera_finalize (damping once
// per pose with a prior: one reduced term of the prior cost function,
// cost_system.rs:229-236), the costs into one extra partial of the merit and
// of the trial cost.
//
// Each edge on poses (m, n) with the measured pose_m_from_pose_n M has the
// residual g = log(T_m^-1 T_n M^-1), no precision and no robust kernel: cost
// g^T g.  With D the derivative of log(T_m^-1 exp(x) T_n M^-1) at x = 0
// (Isometry3::dx_log_a_exp_x_b_at_0), J_n = D and J_m = -D.  Edges with the
// same (m, n) form one reduced term: J_m^T J_m and J_n^T J_n (+ nu I once per
// term) go to the diagonal blocks, J_m^T J_n to the lower block of S between
// them (k_schur_reduce), -J^T g to the gradients (cost_system.rs:190-273).
#include <cuda_runtime.h>

#include <cstdint>

#include "sgba_dd.cuh"
#include "sgba_internal.h"
#include "sgba_lie.cuh"

namespace sgba {

namespace {

constexpr int kPriorThreads = 256;

struct EdgeArgs {
  int nt;              // reduced terms
  const int32_t* tbeg; // nt + 1: edge ranges
  const int32_t* m;    // per edge
  const int32_t* n;
  const double* mn;    // per edge: pose_m_from_pose_n
  double* out;         // 2 nt records: J^T J (36), J^T g (6); side 0 pose m, side 1 pose n
  double* hmn;         // nt x 36: J_m^T J_n
};

__device__ __forceinline__ bool prior_halted(const Ctrl* c) { return c->done != 0; }
__device__ __forceinline__ bool prior_skipping(const Ctrl* c) { return c->done != 0 || c->skip != 0; }

// Priors (sorted by pose) at the given poses.  lin: also J^T W J and J^T W g
// for the priors on free poses (out, kPriorOut doubles per prior).  The
// costs g^T W g are summed in prior order in float-float and written to
// *cost_sum.  gate: 0 none, 1 the control block's done flag, 2 done or a
// skipped step.
__global__ void __launch_bounds__(kPriorThreads) k_prior_eval(PriorArgs a, const double* __restrict__ poses, int lin,
                                                             int gate, double* cost_sum, const Ctrl* ctrl) {
  if ((gate == 1 && prior_halted(ctrl)) || (gate == 2 && prior_skipping(ctrl))) return;
  dd acc = dd_make(0.0f, 0.0f);
  for (int k = threadIdx.x; k < a.n; k += kPriorThreads) {
    const double* T = poses + 7 * a.pose[k];
    const double* W = a.W + 36 * k;
    double einv[7], te[7], g[6];
    lie::se3_inverse(a.mean + 7 * k, einv);
    lie::se3_mul(T, einv, te);
    lie::se3_log(te, g);
    double wg[6];
    for (int r = 0; r < 6; ++r) {
      double s = 0.0;
      for (int c = 0; c < 6; ++c) s += W[6 * r + c] * g[c];
      wg[r] = s;
    }
    double cst = 0.0;
    for (int r = 0; r < 6; ++r) cst += g[r] * wg[r];
    acc = dd_add(acc, dd_from_double(cst));
    if (lin && a.fb[k] >= 0) {
      lie::D6 e[7], td[7], ed[7], p1[7], p2[7], gd[6];
      lie::se3_exp_at_zero(e);
      for (int i = 0; i < 7; ++i) {
        td[i] = lie::dc(T[i]);
        ed[i] = lie::dc(einv[i]);
      }
      lie::se3_mul(e, td, p1);
      lie::se3_mul(p1, ed, p2);
      lie::se3_log(p2, gd);
      double J[36], WJ[36];
      for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 6; ++c) J[6 * r + c] = gd[r].d[c];
      for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 6; ++c) {
          double s = 0.0;
          for (int q = 0; q < 6; ++q) s += W[6 * r + q] * J[6 * q + c];
          WJ[6 * r + c] = s;
        }
      double* o = a.out + static_cast<int64_t>(kPriorOut) * k;
      for (int r = 0; r < 6; ++r) {
        double s = 0.0;
        for (int q = 0; q < 6; ++q) s += J[6 * q + r] * wg[q];
        o[36 + r] = s;  // J^T W g
        for (int c = 0; c < 6; ++c) {
          double h = 0.0;
          for (int q = 0; q < 6; ++q) h += J[6 * q + r] * WJ[6 * q + c];
          o[6 * r + c] = h;  // J^T W J
        }
      }
    }
  }
  if (!cost_sum) return;
  // fixed tree over the CTA: thread t holds priors t, t + 256, ...
  __shared__ float sh_hi[kPriorThreads], sh_lo[kPriorThreads];
  sh_hi[threadIdx.x] = acc.hi;
  sh_lo[threadIdx.x] = acc.lo;
  __syncthreads();
  for (int h = kPriorThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      const dd v = dd_add(dd_make(sh_hi[threadIdx.x], sh_lo[threadIdx.x]),
                          dd_make(sh_hi[threadIdx.x + h], sh_lo[threadIdx.x + h]));
      sh_hi[threadIdx.x] = v.hi;
      sh_lo[threadIdx.x] = v.lo;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *cost_sum = dd_to_double(dd_make(sh_hi[0], sh_lo[0]));
}

// Reduced edge terms at the given poses (one CTA; a thread per term, its
// edges in order).  lin: the records of both sides and J_m^T J_n.  Costs
// summed as in k_prior_eval.
__global__ void __launch_bounds__(kPriorThreads) k_edge_eval(EdgeArgs a, const double* __restrict__ poses, int lin,
                                                            int gate, double* cost_sum, const Ctrl* ctrl) {
  if ((gate == 1 && prior_halted(ctrl)) || (gate == 2 && prior_skipping(ctrl))) return;
  dd acc = dd_make(0.0f, 0.0f);
  for (int t = threadIdx.x; t < a.nt; t += kPriorThreads) {
    double hmm[36], hnn[36], hmn[36], gm[6], gn[6];
    for (int i = 0; i < 36; ++i) hmm[i] = hnn[i] = hmn[i] = 0.0;
    for (int i = 0; i < 6; ++i) gm[i] = gn[i] = 0.0;
    for (int e = a.tbeg[t]; e < a.tbeg[t + 1]; ++e) {
      const double* Tm = poses + 7 * a.m[e];
      const double* Tn = poses + 7 * a.n[e];
      double ai[7], mninv[7], b[7], ab[7], g[6];
      lie::se3_inverse(Tm, ai);
      lie::se3_inverse(a.mn + 7 * e, mninv);
      lie::se3_mul(Tn, mninv, b);
      lie::se3_mul(ai, b, ab);
      lie::se3_log(ab, g);
      double cst = 0.0;
      for (int r = 0; r < 6; ++r) cst += g[r] * g[r];
      acc = dd_add(acc, dd_from_double(cst));
      if (!lin) continue;
      lie::D6 ex[7], ad[7], bd[7], t1[7], t2[7], gd[6];
      lie::se3_exp_at_zero(ex);
      for (int i = 0; i < 7; ++i) {
        ad[i] = lie::dc(ai[i]);
        bd[i] = lie::dc(b[i]);
      }
      lie::se3_mul(ad, ex, t1);
      lie::se3_mul(t1, bd, t2);
      lie::se3_log(t2, gd);
      // J_n = D, J_m = -D
      for (int r = 0; r < 6; ++r) {
        double sg = 0.0;
        for (int q = 0; q < 6; ++q) sg += gd[q].d[r] * g[q];
        gn[r] += sg;
        gm[r] -= sg;
        for (int c = 0; c < 6; ++c) {
          double s2 = 0.0;
          for (int q = 0; q < 6; ++q) s2 += gd[q].d[r] * gd[q].d[c];
          hnn[6 * r + c] += s2;
          hmm[6 * r + c] += s2;
          hmn[6 * r + c] -= s2;
        }
      }
    }
    if (lin) {
      double* o0 = a.out + static_cast<int64_t>(kPriorOut) * (2 * t);
      double* o1 = o0 + kPriorOut;
      for (int i = 0; i < 36; ++i) {
        o0[i] = hmm[i];
        o1[i] = hnn[i];
        a.hmn[36 * static_cast<int64_t>(t) + i] = hmn[i];
      }
      for (int i = 0; i < 6; ++i) {
        o0[36 + i] = gm[i];
        o1[36 + i] = gn[i];
      }
    }
  }
  if (!cost_sum) return;
  __shared__ float sh_hi[kPriorThreads], sh_lo[kPriorThreads];
  sh_hi[threadIdx.x] = acc.hi;
  sh_lo[threadIdx.x] = acc.lo;
  __syncthreads();
  for (int h = kPriorThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      const dd v = dd_add(dd_make(sh_hi[threadIdx.x], sh_lo[threadIdx.x]),
                          dd_make(sh_hi[threadIdx.x + h], sh_lo[threadIdx.x + h]));
      sh_hi[threadIdx.x] = v.hi;
      sh_lo[threadIdx.x] = v.lo;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *cost_sum = dd_to_double(dd_make(sh_hi[0], sh_lo[0]));
}

// Equality constraints c_k = |t(T_k)| - r_k (TranslationNormConstraint,
// ba_scale_constraint.rs:57-100) at the current poses; under exp(x) T the
// translation moves by w x t + v, so the Jacobian is (0, t^T / |t|).  The
// KKT right-hand side gains G^T lambda on the free rows
// (eq_system.rs, populate_lower_triangular_kkt_mat): added here to the
// gradient and the reduced rhs in constraint order (one thread).
__global__ void k_eq_eval(int n, const int32_t* __restrict__ pose, const int32_t* __restrict__ fb,
                          const double* __restrict__ radius, const double* __restrict__ poses, double* c,
                          double* jac, const double* lambda, double* bf, double* rb, const Ctrl* ctrl) {
  if (prior_skipping(ctrl) || threadIdx.x != 0) return;
  for (int k = 0; k < n; ++k) {
    const double* t = poses + 7 * pose[k] + 4;
    const double nrm = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    c[k] = nrm - radius[k];
    for (int i = 0; i < 3; ++i) jac[3 * k + i] = t[i] / nrm;
    if (fb[k] >= 0)
      for (int i = 0; i < 3; ++i) {
        bf[6 * fb[k] + 3 + i] += jac[3 * k + i] * lambda[k];
        rb[6 * fb[k] + 3 + i] += jac[3 * k + i] * lambda[k];
      }
  }
}

// The multiplier step's share of compute_gain_ratio's sums (its entries of
// the step against -c) and of the largest step entry.
__global__ void k_eq_post(int n, const double* __restrict__ dlam, const double* __restrict__ c, double* slot,
                          Ctrl* ctrl) {
  if (prior_skipping(ctrl) || threadIdx.x != 0) return;
  dd sdd = dd_make(0.f, 0.f), sdg = dd_make(0.f, 0.f);
  double mx = 0.0;
  for (int k = 0; k < n; ++k) {
    const dd x = dd_from_double(dlam[k]);
    sdd = dd_add(sdd, dd_mul(x, x));
    sdg = dd_add(sdg, dd_mul(x, dd_from_double(-c[k])));
    mx = fmax(mx, fabs(dlam[k]));
  }
  slot[0] = dd_to_double(sdd);
  slot[1] = dd_to_double(sdg);
  unsigned long long* addr = &ctrl->max_step_bits;
  const unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(mx));
  atomicMax(addr, bits);  // non-negative doubles order as their bit patterns
}

}  // namespace

int launch_eq_eval(const Sizes& s, const Dev& d, cudaStream_t st) {
  if (s.n_eq <= 0) return 0;
  k_eq_eval<<<1, 32, 0, st>>>(s.n_eq, d.eq_pose, d.eq_fb, d.eq_radius, d.poses, d.eq_c, d.eq_jac, d.eq_lambda, d.bf,
                              d.rb, d.ctrl);
  return 1;
}

int launch_eq_post(const Sizes& s, const Dev& d, double* upd_slot, cudaStream_t st) {
  if (s.n_eq <= 0) return 0;
  k_eq_post<<<1, 32, 0, st>>>(s.n_eq, d.eq_dlam, d.eq_c, upd_slot, d.ctrl);
  return 1;
}

int launch_edge_eval(const Sizes& s, const Dev& d, const double* poses, int lin, int gate, double* cost_sum,
                     cudaStream_t st) {
  if (s.n_edge <= 0) return 0;
  EdgeArgs a{s.n_eterm, d.eterm_begin, d.edge_m, d.edge_n, d.edge_mn, d.edge_out, d.edge_hmn};
  k_edge_eval<<<1, kPriorThreads, 0, st>>>(a, poses, lin, gate, cost_sum, d.ctrl);
  return 1;
}

int launch_prior_eval(const Sizes& s, const Dev& d, const double* poses, int lin, int gate, double* cost_sum,
                      cudaStream_t st) {
  if (s.n_prior <= 0) return 0;
  PriorArgs a{s.n_prior, d.prior_pose, d.prior_fb, d.prior_mean, d.prior_W, d.prior_out};
  k_prior_eval<<<1, kPriorThreads, 0, st>>>(a, poses, lin, gate, cost_sum, d.ctrl);
  return 1;
}

}  // namespace sgba
