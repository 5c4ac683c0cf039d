// sgba_pcg.cu -- preconditioned conjugate gradients (PCG) on the reduced
// camera system S dx_f = b, with the exact LDL^T as the fallback.
//
// The reference solves the reduced system only exactly (block LDL^T,
// crates/sophus_solver/src/ldlt/schur_ldlt.rs:536-812, selected through the
// closed LinearSolverEnum, crates/sophus_solver/src/lib.rs:295-318).  This file
// adds an iterative alternative for the same step:
//   * Jacobi scaling S~ = D^-1/2 S D^-1/2 (D = diag S), b~ = D^-1/2 b;
//   * a block preconditioner per free pose: P_j = C_j^-T (I + L_j L_j^T) C_j^-1
//     with C_j the Cholesky factor of the 6x6 diagonal block of S~ (L_j = 0 is
//     block-Jacobi; L_j comes from the learned network, sgba_pcg_net.cu);
//   * CG in FP64 in one cooperative launch (grid barriers with bounded waits);
//     converged when |b~ - S~ x~| <= tol |b~|.  If it is not converged after
//     max_iters iterations (or breaks down, or a barrier wait gives up), the
//     exact factorization that follows in the same iteration runs as usual;
//     otherwise it is skipped (Ctrl::pcg_done).
// Every reduction uses a fixed partition and a fixed order: results are
// bit-reproducible.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "sgba_dd.cuh"
#include "sgba_internal.h"

namespace sgba {

namespace {

constexpr int kPT = 256;                  // threads per CTA
constexpr int kPW = kPT / 32;             // warps per CTA
constexpr long long kBarSpins = 1ll << 22;  // x ~256 ns sleeps: a barrier wait gives up after ~1 s

__device__ __forceinline__ bool skipping(const Ctrl* c) { return c->done != 0 || c->skip != 0; }

struct PcgArgs {
  int nf, n6;
  int64_t nsb;
  const int32_t* sb_row;
  const int32_t* sb_col;
  const int32_t* rowptr;
  const int32_t* cols;
  const int32_t* blks;
  const int32_t* diag;
  const double* S;     // dense n6 x n6 (both triangles of the pattern blocks)
  const double* rb;    // reduced right-hand side (unscaled)
  double* scl;
  double* Sb;
  double* P;
  double* Cinv;
  const float* L;      // learned correction (nf * 21) or null
  double* vec;         // x r p q z
  double* part;
  unsigned* bar;       // [0] arrivals, [1] generation, [2] abort flag
  double* xout;
  float* xdd;
  int max_iters;
  double tol;
};

// ---------------------------------------------------------------- set-up ---

// Jacobi-scaled lower blocks of S (and the scaling itself).
__global__ void __launch_bounds__(kPT) k_pcg_blocks(PcgArgs a, const Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  const int64_t total = a.nsb * 36;
  for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t b = t / 36;
    const int e = static_cast<int>(t % 36);
    const int r = 6 * a.sb_row[b] + e / 6, c = 6 * a.sb_col[b] + e % 6;
    const double dr = a.S[static_cast<int64_t>(r) * a.n6 + r], dc = a.S[static_cast<int64_t>(c) * a.n6 + c];
    const double sr = (dr > 0.0 && isfinite(dr)) ? 1.0 / sqrt(dr) : 1.0;
    const double sc = (dc > 0.0 && isfinite(dc)) ? 1.0 / sqrt(dc) : 1.0;
    a.Sb[t] = a.S[static_cast<int64_t>(r) * a.n6 + c] * sr * sc;
    if (r == c) a.scl[r] = sr;
  }
}

// 6x6 Cholesky B = C C^T (lower, f64); false if a pivot is not positive.
__device__ bool chol6(const double* B, double* C) {
  for (int k = 0; k < 36; ++k) C[k] = 0.0;
  for (int j = 0; j < 6; ++j) {
    double d = B[j * 6 + j];
    for (int k = 0; k < j; ++k) d -= C[j * 6 + k] * C[j * 6 + k];
    if (!(d > 0.0) || !isfinite(d)) return false;
    const double cjj = sqrt(d);
    C[j * 6 + j] = cjj;
    for (int i = j + 1; i < 6; ++i) {
      double v = B[i * 6 + j];
      for (int k = 0; k < j; ++k) v -= C[i * 6 + k] * C[j * 6 + k];
      C[i * 6 + j] = v / cjj;
    }
  }
  return true;
}

// Inverse of a lower-triangular 6x6 (lower).
__device__ void trinv6(const double* C, double* X) {
  for (int k = 0; k < 36; ++k) X[k] = 0.0;
  for (int j = 0; j < 6; ++j) {
    X[j * 6 + j] = 1.0 / C[j * 6 + j];
    for (int i = j + 1; i < 6; ++i) {
      double v = 0.0;
      for (int k = j; k < i; ++k) v -= C[i * 6 + k] * X[k * 6 + j];
      X[i * 6 + j] = v / C[i * 6 + i];
    }
  }
}

}  // namespace

// P_j = Ci^T (I + L L^T) Ci with Ci = C^-1 (C C^T = diagonal block of S~).
// Shared with the training code: the same arithmetic builds the training
// preconditioner.
__device__ void pcg_precond_block(const double* B, const float* Lrow, double* P, double* Ci) {
  double C[36];
  if (!chol6(B, C)) {
    for (int k = 0; k < 36; ++k) {
      P[k] = (k % 7 == 0) ? 1.0 : 0.0;
      Ci[k] = P[k];
    }
    return;
  }
  trinv6(C, Ci);
  double M[36];
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) M[i * 6 + j] = (i == j) ? 1.0 : 0.0;
  if (Lrow) {
    // L lower 6x6 packed row-wise: (0,0) (1,0) (1,1) (2,0) ...
    double Lf[36];
    for (int k = 0; k < 36; ++k) Lf[k] = 0.0;
    int t = 0;
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j <= i; ++j) Lf[i * 6 + j] = static_cast<double>(Lrow[t++]);
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) {
        double v = 0.0;
        for (int k = 0; k < 6; ++k) v += Lf[i * 6 + k] * Lf[j * 6 + k];
        M[i * 6 + j] += v;
      }
  }
  // P = Ci^T M Ci
  double T[36];
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) {
      double v = 0.0;
      for (int k = 0; k < 6; ++k) v += M[i * 6 + k] * Ci[k * 6 + j];
      T[i * 6 + j] = v;
    }
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) {
      double v = 0.0;
      for (int k = 0; k < 6; ++k) v += Ci[k * 6 + i] * T[k * 6 + j];
      P[i * 6 + j] = v;
    }
}

namespace {

__global__ void __launch_bounds__(128) k_pcg_precond(PcgArgs a, const Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.nf) return;
  pcg_precond_block(a.Sb + 36 * static_cast<int64_t>(a.diag[j]), a.L ? a.L + kPcgOut * static_cast<int64_t>(j) : nullptr,
                    a.P + 36 * static_cast<int64_t>(j), a.Cinv + 36 * static_cast<int64_t>(j));
}

// ------------------------------------------------------------------ solve ---

// Grid barrier for a cooperative launch.  Every wait is bounded: after
// kBarSpins sleeps the CTA sets the abort flag and returns false; every CTA
// also returns false once it sees the flag, so no CTA waits twice for a CTA
// that has left.
__device__ bool grid_barrier(unsigned* bar, unsigned nblocks) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* vb = bar;
    const unsigned gen = vb[1];
    __threadfence();
    int ok = 1;
    if (atomicAdd(bar, 1u) == nblocks - 1) {
      bar[0] = 0u;
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      long long spins = 0;
      while (vb[1] == gen) {
        if (vb[2] != 0u) { ok = 0; break; }
        if (++spins > kBarSpins) {
          atomicExch(bar + 2, 1u);
          ok = 0;
          break;
        }
        __nanosleep(256);
      }
    }
    __threadfence();
    if (vb[2] != 0u) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Sum of one partial per CTA (slot k of 4), the same fixed order in every CTA.
__device__ double sum_parts(const double* part, int k) {
  __shared__ double s_sum;
  if (threadIdx.x < 32) {
    double v = 0.0;
    for (int g = threadIdx.x; g < static_cast<int>(gridDim.x); g += 32) v += __ldcg(part + 4 * g + k);
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (threadIdx.x == 0) s_sum = v;
  }
  __syncthreads();
  const double r = s_sum;
  __syncthreads();
  return r;
}

// Per-CTA partials: warp sums (lane 0 of each warp holds them) combined in
// warp order and written to part[4 * blockIdx + k].
__device__ void write_parts(double* part, double v0, double v1, int k0, int k1) {
  __shared__ double s0[kPW], s1[kPW];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int off = 16; off > 0; off >>= 1) {
    v0 += __shfl_down_sync(0xffffffffu, v0, off);
    v1 += __shfl_down_sync(0xffffffffu, v1, off);
  }
  if (lane == 0) {
    s0[w] = v0;
    s1[w] = v1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t0 = 0.0, t1 = 0.0;
    for (int q = 0; q < kPW; ++q) {
      t0 += s0[q];
      t1 += s1[q];
    }
    part[4 * blockIdx.x + k0] = t0;
    if (k1 >= 0) part[4 * blockIdx.x + k1] = t1;
  }
}

// q_j = sum over the full block row j of S~_jk p_k: lanes take entries, each
// lane forms all six rows of its block product, then a fixed shuffle tree.
__device__ __forceinline__ void block_row_matvec(const PcgArgs& a, int j, const double* p, double* q6) {
  const int lane = threadIdx.x & 31;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int e = a.rowptr[j] + lane; e < a.rowptr[j + 1]; e += 32) {
    const int k = a.cols[e];
    const int bi = a.blks[e];
    const bool tr = bi < 0;
    const double* B = a.Sb + 36 * static_cast<int64_t>(bi & 0x7fffffff);
    double pk[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) pk[c] = __ldcg(p + 6 * k + c);
    if (!tr) {
#pragma unroll
      for (int r = 0; r < 6; ++r)
#pragma unroll
        for (int c = 0; c < 6; ++c) acc[r] = fma(B[r * 6 + c], pk[c], acc[r]);
    } else {
#pragma unroll
      for (int r = 0; r < 6; ++r)
#pragma unroll
        for (int c = 0; c < 6; ++c) acc[r] = fma(B[c * 6 + r], pk[c], acc[r]);
    }
  }
#pragma unroll
  for (int r = 0; r < 6; ++r)
    for (int off = 16; off > 0; off >>= 1) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], off);
#pragma unroll
  for (int r = 0; r < 6; ++r) q6[r] = acc[r];
}

__global__ void __launch_bounds__(kPT) k_pcg_solve(PcgArgs a, Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  const int lane = threadIdx.x & 31;
  const int gw = blockIdx.x * kPW + (threadIdx.x >> 5);
  const int nw = gridDim.x * kPW;
  const unsigned nb = gridDim.x;
  double* x = a.vec;
  double* r = a.vec + a.n6;
  double* p = a.vec + 2 * a.n6;
  double* q = a.vec + 3 * a.n6;
  double* z = a.vec + 4 * a.n6;
  // x = 0, r = b~, z = P r, p = z
  double rz = 0.0, bb = 0.0;
  for (int j = gw; j < a.nf; j += nw) {
    double rv = 0.0;
    if (lane < 6) {
      const int i = 6 * j + lane;
      rv = a.scl[i] * a.rb[i];
      x[i] = 0.0;
      r[i] = rv;
    }
    double zv = 0.0;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      const double rc = __shfl_sync(0xffffffffu, rv, c);
      if (lane < 6) zv = fma(a.P[36 * static_cast<int64_t>(j) + lane * 6 + c], rc, zv);
    }
    if (lane < 6) {
      const int i = 6 * j + lane;
      z[i] = zv;
      p[i] = zv;
      rz += rv * zv;
      bb += rv * rv;
    }
  }
  write_parts(a.part, rz, bb, 0, 1);
  bool ok = grid_barrier(a.bar, nb);
  double rho = ok ? sum_parts(a.part, 0) : 0.0;
  const double bnorm2 = ok ? sum_parts(a.part, 1) : 0.0;
  int it = 0;
  int status = ok ? 1 : 3;
  double rr = bnorm2;
  if (ok && !(bnorm2 > 0.0)) status = 0;  // b = 0: x = 0 is exact
  const double tol2 = a.tol * a.tol * bnorm2;
  while (ok && status == 1 && it < a.max_iters) {
    // q = S~ p, p.q
    double pq = 0.0;
    for (int j = gw; j < a.nf; j += nw) {
      double q6[6];
      block_row_matvec(a, j, p, q6);
      if (lane < 6) {
        const int i = 6 * j + lane;
        const double qv = q6[lane];
        q[i] = qv;
        pq += __ldcg(p + i) * qv;
      }
    }
    write_parts(a.part, pq, 0.0, 2, -1);
    if (!(ok = grid_barrier(a.bar, nb))) { status = 3; break; }
    const double pqs = sum_parts(a.part, 2);
    if (!(pqs > 0.0) || !isfinite(pqs)) { status = 2; break; }
    const double alpha = rho / pqs;
    // x += alpha p, r -= alpha q, z = P r
    double rzn = 0.0, rrn = 0.0;
    for (int j = gw; j < a.nf; j += nw) {
      double rv = 0.0;
      if (lane < 6) {
        const int i = 6 * j + lane;
        x[i] = fma(alpha, p[i], x[i]);
        rv = fma(-alpha, q[i], r[i]);
        r[i] = rv;
      }
      double zv = 0.0;
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const double rc = __shfl_sync(0xffffffffu, rv, c);
        if (lane < 6) zv = fma(a.P[36 * static_cast<int64_t>(j) + lane * 6 + c], rc, zv);
      }
      if (lane < 6) {
        z[6 * j + lane] = zv;
        rzn += rv * zv;
        rrn += rv * rv;
      }
    }
    write_parts(a.part, rzn, rrn, 0, 1);
    if (!(ok = grid_barrier(a.bar, nb))) { status = 3; break; }
    const double rho_n = sum_parts(a.part, 0);
    rr = sum_parts(a.part, 1);
    ++it;
    if (rr <= tol2) { status = 0; break; }
    if (!(rho_n > 0.0) || !isfinite(rho_n)) { status = 2; break; }
    const double beta = rho_n / rho;
    rho = rho_n;
    for (int j = gw; j < a.nf; j += nw) {
      if (lane < 6) {
        const int i = 6 * j + lane;
        p[i] = fma(beta, p[i], z[i]);
      }
    }
    if (!(ok = grid_barrier(a.bar, nb))) { status = 3; break; }
  }
  const bool conv = ok && status == 0;
  if (conv) {
    for (int j = gw; j < a.nf; j += nw) {
      if (lane < 6) {
        const int i = 6 * j + lane;
        const double v = a.scl[i] * x[i];
        a.xout[i] = v;
        const dd vd = dd_from_double(v);
        a.xdd[2 * i] = vd.hi;
        a.xdd[2 * i + 1] = vd.lo;
      }
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctrl->pcg_done = conv ? 1 : 0;
    ctrl->pcg_iters = it;
    ctrl->pcg_status = status;
    ctrl->pcg_relres = (bnorm2 > 0.0 && ok) ? sqrt(rr / bnorm2) : 0.0;
    ctrl->pcg_solves += 1;
    ctrl->pcg_fallbacks += conv ? 0 : 1;
    ctrl->pcg_total_iters += it;
  }
}

PcgArgs pcg_args(const Sizes& s, const Dev& d) {
  PcgArgs a;
  a.nf = s.nf;
  a.n6 = s.n6;
  a.nsb = s.nsb;
  a.sb_row = d.sb_row;
  a.sb_col = d.sb_col;
  a.rowptr = d.pcg_rowptr;
  a.cols = d.pcg_cols;
  a.blks = d.pcg_blks;
  a.diag = d.pcg_diag;
  a.S = d.S;
  a.rb = d.rb;
  a.scl = d.pcg_scl;
  a.Sb = d.pcg_S;
  a.P = d.pcg_P;
  a.Cinv = d.pcg_Cinv;
  a.L = (s.pcg_mode == 2) ? d.pcg_L : nullptr;
  a.vec = d.pcg_vec;
  a.part = d.pcg_part;
  a.bar = d.pcg_bar;
  a.xout = d.x;
  a.xdd = d.xdd;
  a.max_iters = s.pcg_max_iters;
  a.tol = s.pcg_tol;
  return a;
}

}  // namespace

int pcg_setup(int nf, int* grid) {
  int dev = 0, sms = 0, per_sm = 0, coop = 0;
  *grid = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) return -1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg_solve, kPT, 0) != cudaSuccess || per_sm < 1)
    return -1;
  const int want = (nf + kPW - 1) / kPW;
  int cap = sms * (per_sm < 2 ? per_sm : 2);
  if (cap > kPcgMaxGrid) cap = kPcgMaxGrid;
  *grid = want < cap ? (want > 0 ? want : 1) : cap;
  return 0;
}

int pcg_launch_count(const Sizes& s) { return 3 + (s.pcg_mode == 2 ? pcg_net_launch_count() : 0); }

int launch_pcg(const Sizes& s, const Dev& d, cudaStream_t st) {
  const PcgArgs a = pcg_args(s, d);
  int n = 0;
  {
    const int64_t total = s.nsb * 36;
    const int blocks = static_cast<int>(std::min<int64_t>((total + kPT - 1) / kPT, 8192));
    k_pcg_blocks<<<blocks > 0 ? blocks : 1, kPT, 0, st>>>(a, d.ctrl);
    ++n;
  }
  if (s.pcg_mode == 2) n += launch_pcg_net(s, d, st);
  k_pcg_precond<<<(s.nf + 127) / 128, 128, 0, st>>>(a, d.ctrl);
  ++n;
  cudaMemsetAsync(d.pcg_bar, 0, 4 * sizeof(unsigned), st);
  {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(s.pcg_grid);
    cfg.blockDim = dim3(kPT);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k_pcg_solve, a, d.ctrl);
    ++n;
  }
  return n;
}

}  // namespace sgba
