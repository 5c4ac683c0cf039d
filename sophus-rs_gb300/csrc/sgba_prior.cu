// sgba_prior.cu -- the pose prior cost function on the GPU
// (Isometry3PriorCostTerm, crates/sophus_opt/src/nlls/functor_library/costs/isometry3_prior.rs).
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
#include <cuda_runtime.h>

#include <cstdint>

#include "sgba_dd.cuh"
#include "sgba_internal.h"
#include "sgba_lie.cuh"

namespace sgba {

namespace {

constexpr int kPriorThreads = 256;

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

}  // namespace

int launch_prior_eval(const Sizes& s, const Dev& d, const double* poses, int lin, int gate, double* cost_sum,
                      cudaStream_t st) {
  if (s.n_prior <= 0) return 0;
  PriorArgs a{s.n_prior, d.prior_pose, d.prior_fb, d.prior_mean, d.prior_W, d.prior_out};
  k_prior_eval<<<1, kPriorThreads, 0, st>>>(a, poses, lin, gate, cost_sum, d.ctrl);
  return 1;
}

}  // namespace sgba
