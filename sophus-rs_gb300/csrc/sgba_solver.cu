// sgba_solver.cu -- factorization and solve of the dense reduced camera
// system S (6 n_f x 6 n_f) on the GPU.
//
// Reference: BlockSparseLdlt::factorize_impl / solve_inplace
// (crates/sophus_solver/src/ldlt/block_sparse_ldlt.rs:99-190, 479-747) with
// per-block PSD-aware pivots (crates/sophus_solver/src/ldlt/dense_ldlt.rs:164-270,
// tol_rel = 1e-12, the relative threshold restarting at every 6x6 pose block).
// In exact arithmetic the block algorithm equals a scalar LDL^T in the same
// (natural) order with that pivot rule, which is what is computed here.
//
// GB300 plan: the factorization runs in FP32 (64x the FP64 rate), blocked
// right-looking with 48-wide panels (diagonal panel, panel TRSM, trailing
// update); the solution is then refined against the f64 S with f64
// residuals, which recovers f64-level accuracy of the step.
#include <cuda_runtime.h>

#include <cstdint>

#include "sgba_internal.h"

namespace sgba {

namespace {

constexpr int kPW = 48;  // panel width (multiple of the 6-dof pose block)
constexpr float kTolRel = 1e-12f;
constexpr int kRefineSteps = 2;

__device__ __forceinline__ bool skipping(const Ctrl* c) { return c->done != 0 || c->skip != 0; }

__global__ void k_s_to_f32(int n, const double* __restrict__ S, float* __restrict__ A, const Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  const int64_t total = static_cast<int64_t>(n) * n;
  for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<int64_t>(gridDim.x) * blockDim.x)
    A[t] = __double2float_rn(S[t]);
}

// Factor the w x w diagonal panel block at (c0, c0) in shared memory.
__global__ void __launch_bounds__(256) k_ldlt_diag(int n, int c0, int w, float* __restrict__ A,
                                                   float* __restrict__ dpiv, Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  __shared__ float a[kPW][kPW + 1];
  __shared__ float col[kPW];
  __shared__ float s_d;
  __shared__ float s_maxp;
  __shared__ int s_bad;
  const int tid = threadIdx.x;
  for (int e = tid; e < w * w; e += blockDim.x) {
    const int i = e / w, k = e % w;
    a[i][k] = (k <= i) ? A[static_cast<int64_t>(c0 + i) * n + c0 + k] : 0.0f;
  }
  if (tid == 0) { s_maxp = 1.0f; s_bad = 0; }
  __syncthreads();
  for (int t = 0; t < w; ++t) {
    if (tid == 0) {
      if ((c0 + t) % 6 == 0) s_maxp = 1.0f;  // new pose block: restart the relative threshold
      float d = a[t][t];
      if (!isfinite(d)) s_bad = 1;
      const float tol = fmaxf(s_maxp, 1.0f) * kTolRel;
      if (fabsf(d) <= tol) {
        d = 0.0f;
      } else {
        s_maxp = fmaxf(s_maxp, fabsf(d));
      }
      s_d = d;
      dpiv[c0 + t] = d;
    }
    __syncthreads();
    const float d = s_d;
    for (int i = t + 1 + tid; i < w; i += blockDim.x) {
      const float v = a[i][t];
      col[i] = v;
      a[i][t] = (d == 0.0f) ? 0.0f : v / d;
    }
    __syncthreads();
    // trailing update inside the panel: a[i][k] -= col[i] * l[k], t < k <= i < w
    const int m = w - t - 1;
    const int pairs = m * (m + 1) / 2;
    for (int e = tid; e < pairs; e += blockDim.x) {
      // decode e -> (ii, kk) with kk <= ii over an m x m lower triangle
      int ii = static_cast<int>((sqrtf(8.0f * e + 1.0f) - 1.0f) * 0.5f);
      while ((ii + 1) * (ii + 2) / 2 <= e) ++ii;
      while (ii * (ii + 1) / 2 > e) --ii;
      const int kk = e - ii * (ii + 1) / 2;
      const int i = t + 1 + ii, k = t + 1 + kk;
      a[i][k] -= col[i] * a[k][t];
    }
    __syncthreads();
  }
  for (int e = tid; e < w * w; e += blockDim.x) {
    const int i = e / w, k = e % w;
    if (k < i) A[static_cast<int64_t>(c0 + i) * n + c0 + k] = a[i][k];
    else if (k == i) A[static_cast<int64_t>(c0 + i) * n + c0 + k] = 1.0f;
  }
  if (tid == 0 && s_bad) ctrl->skip = 2;  // NonFinitePivot -> solve failure -> reject
}

// Rows below the panel: y = a_i L_pp^-T (= L_i * d), L_i = y / d.
__global__ void __launch_bounds__(128) k_ldlt_trsm(int n, int c0, int w, float* __restrict__ A,
                                                   const float* __restrict__ dpiv, float* __restrict__ wpanel,
                                                   const Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  __shared__ float L[kPW][kPW + 1];
  __shared__ float dv[kPW];
  for (int e = threadIdx.x; e < w * w; e += blockDim.x) {
    const int i = e / w, k = e % w;
    L[i][k] = (k < i) ? A[static_cast<int64_t>(c0 + i) * n + c0 + k] : 0.0f;
  }
  for (int t = threadIdx.x; t < w; t += blockDim.x) dv[t] = dpiv[c0 + t];
  __syncthreads();
  const int i = c0 + w + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float* row = A + static_cast<int64_t>(i) * n + c0;
  float y[kPW];
#pragma unroll
  for (int t = 0; t < kPW; ++t) {
    if (t < w) {
      float s = row[t];
#pragma unroll
      for (int k = 0; k < kPW; ++k)
        if (k < t) s = fmaf(-y[k], L[t][k], s);
      y[t] = s;
    }
  }
  float* wp = wpanel + static_cast<int64_t>(i) * kPW;
#pragma unroll
  for (int t = 0; t < kPW; ++t) {
    if (t < w) {
      wp[t] = y[t];
      row[t] = (dv[t] == 0.0f) ? 0.0f : y[t] / dv[t];
    }
  }
}

// Trailing update A[i][k] -= sum_t W[i][t] L[k][t] for c1 <= k <= i < n,
// 32x32 lower tiles.
__global__ void __launch_bounds__(256) k_ldlt_update(int n, int c0, int w, float* __restrict__ A,
                                                     const float* __restrict__ wpanel, const Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  const int c1 = c0 + w;
  // decode the lower tile (I, K), I >= K
  const int e = blockIdx.x;
  int I = static_cast<int>((sqrtf(8.0f * e + 1.0f) - 1.0f) * 0.5f);
  while ((I + 1) * (I + 2) / 2 <= e) ++I;
  while (I * (I + 1) / 2 > e) --I;
  const int K = e - I * (I + 1) / 2;
  const int r0 = c1 + 32 * I, k0 = c1 + 32 * K;
  __shared__ float Ws[32][kPW + 1];
  __shared__ float Ls[32][kPW + 1];
  for (int q = threadIdx.x; q < 32 * kPW; q += blockDim.x) {
    const int rr = q / kPW, t = q % kPW;
    const int i = r0 + rr, k = k0 + rr;
    Ws[rr][t] = (i < n && t < w) ? wpanel[static_cast<int64_t>(i) * kPW + t] : 0.0f;
    Ls[rr][t] = (k < n && t < w) ? A[static_cast<int64_t>(k) * n + c0 + t] : 0.0f;
  }
  __syncthreads();
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int k = k0 + tx;
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  for (int t = 0; t < w; ++t) {
    const float lk = Ls[tx][t];
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[q] = fmaf(Ws[ty + 8 * q][t], lk, acc[q]);
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int i = r0 + ty + 8 * q;
    if (i < n && k < n && k <= i) A[static_cast<int64_t>(i) * n + k] -= acc[q];
  }
}

// x (mode 0) or x += (mode 1) the solution of (L D L^T) x = b, FP32 factor,
// f64 in/out.  One CTA of 1024 threads, 32-row blocks.
__global__ void __launch_bounds__(1024) k_ldlt_solve(int n, const float* __restrict__ A,
                                                     const float* __restrict__ dpiv,
                                                     const double* __restrict__ b, double* __restrict__ x,
                                                     int mode, const Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  extern __shared__ float y[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < n; i += blockDim.x) y[i] = __double2float_rn(b[i]);
  __syncthreads();
  // forward: L y = b
  for (int b0 = 0; b0 < n; b0 += 32) {
    const int r = b0 + warp;
    if (r < n && b0 > 0) {
      const float* row = A + static_cast<int64_t>(r) * n;
      float s = 0.f;
      for (int k = lane; k < b0; k += 32) s = fmaf(row[k], y[k], s);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
      if (lane == 0) y[r] -= s;
    }
    __syncthreads();
    if (warp == 0) {
      const int rr = b0 + lane;
      float v = (rr < n) ? y[rr] : 0.f;
      const int bw = min(32, n - b0);
      for (int t = 0; t < bw; ++t) {
        const float yt = __shfl_sync(0xffffffffu, v, t);
        if (lane > t && rr < n) v = fmaf(-A[static_cast<int64_t>(rr) * n + b0 + t], yt, v);
      }
      if (rr < n) y[rr] = v;
    }
    __syncthreads();
  }
  for (int i = tid; i < n; i += blockDim.x) y[i] = (dpiv[i] == 0.f) ? 0.f : y[i] / dpiv[i];
  __syncthreads();
  // backward: L^T x = z
  const int nblk = (n + 31) / 32;
  for (int bb = nblk - 1; bb >= 0; --bb) {
    const int b0 = 32 * bb, b1 = min(n, b0 + 32);
    if (warp == 0) {
      const int rr = b0 + lane;
      float v = (rr < b1) ? y[rr] : 0.f;
      for (int t = b1 - 1; t >= b0; --t) {
        const float xt = __shfl_sync(0xffffffffu, v, t - b0);
        if (rr < t) v = fmaf(-A[static_cast<int64_t>(t) * n + rr], xt, v);
      }
      if (rr < b1) y[rr] = v;
    }
    __syncthreads();
    for (int r = tid; r < b0; r += blockDim.x) {
      float s = 0.f;
      for (int t = b0; t < b1; ++t) s = fmaf(A[static_cast<int64_t>(t) * n + r], y[t], s);
      y[r] -= s;
    }
    __syncthreads();
  }
  for (int i = tid; i < n; i += blockDim.x) {
    if (mode == 0) x[i] = static_cast<double>(y[i]);
    else x[i] += static_cast<double>(y[i]);
  }
}

// r = b - S x in f64 (S full symmetric), one warp per row.
__global__ void __launch_bounds__(256) k_residual(int n, const double* __restrict__ S,
                                                  const double* __restrict__ b, const double* __restrict__ x,
                                                  double* __restrict__ r, const Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  const int lane = threadIdx.x & 31;
  const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (row >= n) return;
  const double* s = S + static_cast<int64_t>(row) * n;
  double acc = 0.0;
  for (int k = lane; k < n; k += 32) acc = fma(s[k], x[k], acc);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if (lane == 0) r[row] = b[row] - acc;
}

}  // namespace

int solver_launch_count(const Sizes& s) {
  const int panels = (s.n6 + kPW - 1) / kPW;
  return 1 + 3 * panels + 1 + 2 * kRefineSteps;
}

int launch_factor_solve(const Sizes& s, const Dev& d, cudaStream_t st) {
  const int n = s.n6;
  int launches = 0;
  {
    int64_t total = static_cast<int64_t>(n) * n;
    int blocks = static_cast<int>((total + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    if (blocks < 1) blocks = 1;
    k_s_to_f32<<<blocks, 256, 0, st>>>(n, d.S, d.A, d.ctrl);
    ++launches;
  }
  for (int c0 = 0; c0 < n; c0 += kPW) {
    const int w = (n - c0 < kPW) ? (n - c0) : kPW;
    k_ldlt_diag<<<1, 256, 0, st>>>(n, c0, w, d.A, d.dpiv, d.ctrl);
    const int rows = n - c0 - w;
    if (rows > 0) {
      k_ldlt_trsm<<<(rows + 127) / 128, 128, 0, st>>>(n, c0, w, d.A, d.dpiv, d.wpanel, d.ctrl);
      const int nt = (rows + 31) / 32;
      k_ldlt_update<<<nt * (nt + 1) / 2, 256, 0, st>>>(n, c0, w, d.A, d.wpanel, d.ctrl);
    } else {
      // keep the launch count fixed per panel (graph shape independent of n)
      k_ldlt_trsm<<<1, 128, 0, st>>>(n, c0, w, d.A, d.dpiv, d.wpanel, d.ctrl);
      k_ldlt_update<<<1, 256, 0, st>>>(n, n, 0, d.A, d.wpanel, d.ctrl);
    }
    launches += 3;
  }
  const size_t smem = sizeof(float) * static_cast<size_t>(n);
  k_ldlt_solve<<<1, 1024, smem, st>>>(n, d.A, d.dpiv, d.rb, d.x, 0, d.ctrl);
  ++launches;
  for (int it = 0; it < kRefineSteps; ++it) {
    k_residual<<<(n + 7) / 8, 256, 0, st>>>(n, d.S, d.rb, d.x, d.r, d.ctrl);
    k_ldlt_solve<<<1, 1024, smem, st>>>(n, d.A, d.dpiv, d.r, d.x, 1, d.ctrl);
    launches += 2;
  }
  return launches;
}

}  // namespace sgba
