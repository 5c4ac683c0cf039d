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

#include "sgba_dd.cuh"
#include "sgba_internal.h"

namespace sgba {

namespace {

constexpr int kPW = 48;  // panel width (multiple of the 6-dof pose block)
constexpr float kTolRel = 1e-12f;
constexpr int kRefineSteps = 1;

// the factorization is skipped on termination, on a skipped step and when PCG converged
__device__ __forceinline__ bool skipping(const Ctrl* c) { return c->done != 0 || c->skip != 0 || c->pcg_done != 0; }

__global__ void k_s_to_f32(int n, const double* __restrict__ S, float* __restrict__ A, const Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  const int64_t total = static_cast<int64_t>(n) * n;
  for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<int64_t>(gridDim.x) * blockDim.x)
    A[t] = __double2float_rn(S[t]);
}

// Panel step: factor the w x w diagonal block at (c0, c0) and solve the rows
// below it.  Every CTA factors the diagonal block redundantly in shared memory
// (no grid-wide dependency); CTA 0 writes it back.  Then each thread owns one
// row i >= c0 + w:  y = a_i L_pp^-T (= L_i d), L_i = y / d.
constexpr int kPanelThreads = 256;
constexpr int kLowerPairs = kPW * (kPW - 1) / 2;

__global__ void __launch_bounds__(kPanelThreads) k_ldlt_panel(int n, int c0, int w, float* __restrict__ A,
                                                             float* __restrict__ dpiv, float* __restrict__ wpanel,
                                                             Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  __shared__ float a[kPW][kPW + 1];
  __shared__ float col[kPW];
  __shared__ float dsh[kPW];
  __shared__ unsigned short pair_i[kLowerPairs], pair_k[kLowerPairs];
  __shared__ int s_bad;
  const int tid = threadIdx.x;
  for (int e = tid; e < w * w; e += blockDim.x) {
    const int i = e / w, k = e % w;
    a[i][k] = (k <= i) ? A[static_cast<int64_t>(c0 + i) * n + c0 + k] : 0.0f;
  }
  // strictly-lower pairs (i, k), k < i, ordered by column k: the pairs with
  // k > t form a suffix starting at (t + 1) * (2 kPW - 2 - t) / 2
  for (int e = tid; e < kLowerPairs; e += blockDim.x) {
    int k = 0, rem = e;
    while (k < kPW - 1 && rem >= kPW - 1 - k) { rem -= kPW - 1 - k; ++k; }
    pair_k[e] = static_cast<unsigned short>(k);
    pair_i[e] = static_cast<unsigned short>(k + 1 + rem);
  }
  if (tid == 0) s_bad = 0;
  __syncthreads();
  float maxp = 1.0f;  // used by thread 0 only
  for (int t = 0; t < w; ++t) {
    if (tid == 0) {
      if ((c0 + t) % 6 == 0) maxp = 1.0f;  // new pose block: restart the relative threshold
      float d = a[t][t];
      if (!isfinite(d)) s_bad = 1;
      const float tol = fmaxf(maxp, 1.0f) * kTolRel;
      if (fabsf(d) <= tol) d = 0.0f;
      else maxp = fmaxf(maxp, fabsf(d));
      dsh[t] = d;
    }
    __syncthreads();
    const float d = dsh[t];
    for (int i = t + 1 + tid; i < w; i += blockDim.x) {
      const float v = a[i][t];
      col[i] = v;
      a[i][t] = (d == 0.0f) ? 0.0f : v / d;
    }
    __syncthreads();
    // a[i][k] -= col[i] * l[k] for t < k <= i < w: diagonal entries, then the
    // strictly-lower pairs with k > t
    for (int k = t + 1 + tid; k < w; k += blockDim.x) a[k][k] -= col[k] * a[k][t];
    const int first = (t + 1) * (2 * kPW - 2 - t) / 2;
    for (int e = first + tid; e < kLowerPairs; e += blockDim.x) {
      const int i = pair_i[e], k = pair_k[e];
      if (i < w) a[i][k] -= col[i] * a[k][t];
    }
    __syncthreads();
  }
  if (blockIdx.x == 0) {
    for (int e = tid; e < w * w; e += blockDim.x) {
      const int i = e / w, k = e % w;
      if (k < i) A[static_cast<int64_t>(c0 + i) * n + c0 + k] = a[i][k];
      else if (k == i) A[static_cast<int64_t>(c0 + i) * n + c0 + k] = 1.0f;
    }
    for (int t = tid; t < w; t += blockDim.x) dpiv[c0 + t] = dsh[t];
    if (tid == 0 && s_bad) ctrl->skip = 2;  // NonFinitePivot -> solve failure -> reject
  }
  // TRSM for this CTA's rows
  const int i = c0 + w + blockIdx.x * blockDim.x + tid;
  if (i >= n) return;
  float* row = A + static_cast<int64_t>(i) * n + c0;
  float y[kPW];
#pragma unroll
  for (int t = 0; t < kPW; ++t) y[t] = (t < w) ? row[t] : 0.0f;
  // right-looking within the row: once y[k] is final, update every later y[t]
  // (independent FMAs instead of one long dependent dot product)
#pragma unroll
  for (int k = 0; k < kPW - 1; ++k) {
    const float yk = y[k];
#pragma unroll
    for (int t = k + 1; t < kPW; ++t) y[t] = fmaf(-yk, a[t][k], y[t]);
  }
  float* wp = wpanel + static_cast<int64_t>(i) * kPW;
#pragma unroll
  for (int t = 0; t < kPW; ++t) {
    if (t < w) {
      wp[t] = y[t];
      row[t] = (dsh[t] == 0.0f) ? 0.0f : y[t] / dsh[t];
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
// f64 in/out.  One CTA of 1024 threads, 32-row blocks; the 32x32 triangles are
// loaded into registers before their sequential sweep.
__global__ void __launch_bounds__(1024) k_ldlt_solve(int n, const float* __restrict__ A,
                                                     const float* __restrict__ dpiv,
                                                     const double* __restrict__ b, double* __restrict__ x,
                                                     int mode, float* __restrict__ xdd, const Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  extern __shared__ float y[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < n; i += blockDim.x) y[i] = __double2float_rn(b[i]);
  __syncthreads();
  // forward: L y = b (right-looking over 32-row blocks)
  for (int b0 = 0; b0 < n; b0 += 32) {
    const int bw = min(32, n - b0);
    if (warp == 0) {
      const int rr = b0 + lane;
      float tri[32];
#pragma unroll
      for (int t = 0; t < 32; ++t)
        tri[t] = (rr < n && t < lane && t < bw) ? A[static_cast<int64_t>(rr) * n + b0 + t] : 0.f;
      float v = (rr < n) ? y[rr] : 0.f;
#pragma unroll
      for (int t = 0; t < 32; ++t) {
        const float yt = __shfl_sync(0xffffffffu, v, t);
        v = fmaf(-tri[t], yt, v);  // tri[t] == 0 for t >= lane
      }
      if (rr < n) y[rr] = v;
    }
    __syncthreads();
    // rows below the block: y[r] -= L[r][b0:b0+bw] . y[b0:b0+bw]
    for (int r = b0 + bw + tid; r < n; r += blockDim.x) {
      const float* row = A + static_cast<int64_t>(r) * n + b0;
      float s = 0.f;
#pragma unroll 8
      for (int t = 0; t < bw; ++t) s = fmaf(row[t], y[b0 + t], s);
      y[r] -= s;
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
      float tri[32];  // tri[t] = L[b0 + t][rr] for t > lane
#pragma unroll
      for (int t = 0; t < 32; ++t)
        tri[t] = (b0 + t < b1 && t > lane) ? A[static_cast<int64_t>(b0 + t) * n + rr] : 0.f;
      float v = (rr < b1) ? y[rr] : 0.f;
#pragma unroll
      for (int t = 31; t >= 0; --t) {
        const float xt = __shfl_sync(0xffffffffu, v, t);
        v = fmaf(-tri[t], xt, v);
      }
      if (rr < b1) y[rr] = v;
    }
    __syncthreads();
    for (int r = tid; r < b0; r += blockDim.x) {
      float s = 0.f;
#pragma unroll 8
      for (int t = b0; t < b1; ++t) s = fmaf(A[static_cast<int64_t>(t) * n + r], y[t], s);
      y[r] -= s;
    }
    __syncthreads();
  }
  for (int i = tid; i < n; i += blockDim.x) {
    const double xi = (mode == 0) ? static_cast<double>(y[i]) : x[i] + static_cast<double>(y[i]);
    x[i] = xi;
    if (xdd) {
      const dd v = dd_from_double(xi);
      xdd[2 * i] = v.hi;
      xdd[2 * i + 1] = v.lo;
    }
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
  const int pcg = s.pcg_mode ? pcg_launch_count(s) : 0;
  if (s.small_dense) return pcg + 1;
  if (s.dense_c > 0) return pcg + 1;
  if (s.band_c > 0) return pcg + band_launch_count(s);
  const int panels = (s.n6 + kPW - 1) / kPW;
  return pcg + 1 + 2 * panels + 1 + 2 * kRefineSteps;
}

int launch_factor_solve(const Sizes& s, const Dev& d, cudaStream_t st) {
  // PCG first when selected; the exact factorization below skips itself when
  // PCG converged (Ctrl::pcg_done) and is the fallback otherwise
  const int pcg = s.pcg_mode ? launch_pcg(s, d, st) : 0;
  return pcg + launch_exact_solve(s, d, st);
}

int launch_exact_solve(const Sizes& s, const Dev& d, cudaStream_t st) {
  if (s.small_dense) return launch_small_dense(s, d, st);
  if (s.dense_c > 0) return launch_dense_cluster(s, d, st);
  if (s.band_c > 0) return launch_band(s, d, st);
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
    const int rows = n - c0 - w;
    const int pb = rows > 0 ? (rows + kPanelThreads - 1) / kPanelThreads : 1;
    k_ldlt_panel<<<pb, kPanelThreads, 0, st>>>(n, c0, w, d.A, d.dpiv, d.wpanel, d.ctrl);
    if (rows > 0) {
      const int nt = (rows + 31) / 32;
      k_ldlt_update<<<nt * (nt + 1) / 2, 256, 0, st>>>(n, c0, w, d.A, d.wpanel, d.ctrl);
    } else {
      k_ldlt_update<<<1, 256, 0, st>>>(n, n, 0, d.A, d.wpanel, d.ctrl);  // fixed graph shape
    }
    launches += 2;
  }
  const size_t smem = sizeof(float) * static_cast<size_t>(n);
  k_ldlt_solve<<<1, 1024, smem, st>>>(n, d.A, d.dpiv, d.rb, d.x, 0, kRefineSteps == 0 ? d.xdd : nullptr,
                                      d.ctrl);
  ++launches;
  for (int it = 0; it < kRefineSteps; ++it) {
    k_residual<<<(n + 7) / 8, 256, 0, st>>>(n, d.S, d.rb, d.x, d.r, d.ctrl);
    k_ldlt_solve<<<1, 1024, smem, st>>>(n, d.A, d.dpiv, d.r, d.x, 1, it == kRefineSteps - 1 ? d.xdd : nullptr,
                                        d.ctrl);
    launches += 2;
  }
  return launches;
}

}  // namespace sgba
