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
//   * CG with FP64 vectors and a float-float matrix-vector product, in one
//     cooperative launch (grid barriers with bounded waits);
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
#include "sgba_pcg_dev.cuh"

namespace sgba {

namespace {

constexpr int kPT = 512;                  // threads per CTA
constexpr int kPW = kPT / 32;             // warps per CTA
constexpr long long kBarSpins = 1ll << 22;  // x ~256 ns sleeps: a barrier wait gives up after ~1 s

__device__ __forceinline__ bool skipping(const Ctrl* c) { return c->done != 0 || c->skip != 0; }

// Float-float dot-product accumulator: the running sum through an exact
// TwoSum, the rounding errors of products and sums gathered in the lo part.
struct Acc {
  float hi, lo;
};
__device__ __forceinline__ void acc_madd(Acc& a, dd x, dd y) {
  const float pr = __fmul_rn(x.hi, y.hi);
  float e = __fmaf_rn(x.hi, y.hi, -pr);
  e = __fmaf_rn(x.hi, y.lo, e);
  e = __fmaf_rn(x.lo, y.hi, e);
  const float s = __fadd_rn(a.hi, pr);
  const float bb = __fsub_rn(s, a.hi);
  const float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(pr, bb));
  a.hi = s;
  a.lo = __fadd_rn(a.lo, __fadd_rn(err, e));
}
__device__ __forceinline__ dd acc_get(const Acc& a) { return dd_fast_two_sum(a.hi, a.lo); }

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
  float2* Sb2;         // the same blocks as float-float (hi, lo) pairs
  double* P;
  double* Cinv;
  const float* L;      // learned correction (nf * 21) or null
  double* vec;         // x r u p s w
  double* part;
  unsigned* bar;       // [0] arrivals (monotonic within a launch), [2] abort flag
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
    const double v = a.S[static_cast<int64_t>(r) * a.n6 + c] * sr * sc;
    a.Sb[t] = v;
    const dd vd = dd_from_double(v);
    a.Sb2[t] = make_float2(vd.hi, vd.lo);
    if (r == c) a.scl[r] = sr;
  }
}

}  // namespace

namespace {

__global__ void __launch_bounds__(128) k_pcg_precond(PcgArgs a, const Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.nf) return;
  pcg_precond_block(a.Sb + 36 * static_cast<int64_t>(a.diag[j]), a.L ? a.L + kPcgOut * static_cast<int64_t>(j) : nullptr,
                    a.P + 36 * static_cast<int64_t>(j), a.Cinv + 36 * static_cast<int64_t>(j));
}

// ------------------------------------------------------------------ solve ---

// Grid barrier for a cooperative launch: a monotonic arrival counter; the
// k-th barrier of a launch waits until k * gridDim CTAs have arrived (the
// counter is zeroed before the launch).  Every wait is bounded: after
// kBarSpins polls the CTA sets the abort flag and returns false; every CTA
// also returns false once it sees the flag.
__device__ bool grid_barrier(unsigned* bar, unsigned target) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(bar, 1u);
    int ok = 1;
    long long spins = 0;
    unsigned v;
    for (;;) {
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(bar) : "memory");
      if (v >= target) break;
      unsigned ab;
      asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(ab) : "l"(bar + 2) : "memory");
      if (ab != 0u) { ok = 0; break; }
      if (++spins > kBarSpins) {
        atomicExch(bar + 2, 1u);
        ok = 0;
        break;
      }
      if (spins > 64) __nanosleep(64);
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Sum of one partial per CTA (slot k of kSlots), the same fixed order in
// every CTA.
constexpr int kSlots = 4;
__device__ void sum_parts3(const double* part, double* out) {
  __shared__ double s_sum[3];
  if (threadIdx.x < 32) {
    double v0 = 0.0, v1 = 0.0, v2 = 0.0;
    for (int g = threadIdx.x; g < static_cast<int>(gridDim.x); g += 32) {
      v0 += __ldcg(part + kSlots * g + 0);
      v1 += __ldcg(part + kSlots * g + 1);
      v2 += __ldcg(part + kSlots * g + 2);
    }
    for (int off = 16; off > 0; off >>= 1) {
      v0 += __shfl_down_sync(0xffffffffu, v0, off);
      v1 += __shfl_down_sync(0xffffffffu, v1, off);
      v2 += __shfl_down_sync(0xffffffffu, v2, off);
    }
    if (threadIdx.x == 0) {
      s_sum[0] = v0;
      s_sum[1] = v1;
      s_sum[2] = v2;
    }
  }
  __syncthreads();
  out[0] = s_sum[0];
  out[1] = s_sum[1];
  out[2] = s_sum[2];
  __syncthreads();
}

// Per-CTA partials of three dot products: warp sums combined in warp order.
__device__ void write_parts3(double* part, double v0, double v1, double v2) {
  __shared__ double s[3][kPW];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int off = 16; off > 0; off >>= 1) {
    v0 += __shfl_down_sync(0xffffffffu, v0, off);
    v1 += __shfl_down_sync(0xffffffffu, v1, off);
    v2 += __shfl_down_sync(0xffffffffu, v2, off);
  }
  if (lane == 0) {
    s[0][w] = v0;
    s[1][w] = v1;
    s[2][w] = v2;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double t = 0.0;
    for (int q = 0; q < kPW; ++q) t += s[threadIdx.x][q];
    part[kSlots * blockIdx.x + threadIdx.x] = t;
  }
}

// w_j = sum over the full block row j of S~_jk u_k in float-float (the blocks
// as (hi, lo) FP32 pairs: FP64 runs at 1/64 of the FP32 rate here): lanes
// take entries, each lane forms the six rows of its block product, then a
// fixed shuffle tree.  Returns the six sums in every lane.
__device__ __forceinline__ void block_row_matvec(const PcgArgs& a, int j, const double* u, double* w6) {
  const int lane = threadIdx.x & 31;
  Acc acc[6];
#pragma unroll
  for (int r = 0; r < 6; ++r) acc[r] = Acc{0.0f, 0.0f};
  for (int e = a.rowptr[j] + lane; e < a.rowptr[j + 1]; e += 32) {
    const int k = a.cols[e];
    const int bi = a.blks[e];
    const bool tr = bi < 0;
    const float4* B4 = reinterpret_cast<const float4*>(a.Sb2 + 36 * static_cast<int64_t>(bi & 0x7fffffff));
    dd uk[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) uk[c] = dd_from_double(__ldcg(u + 6 * k + c));
#pragma unroll
    for (int h = 0; h < 18; ++h) {
      const float4 v = B4[h];  // entries 2h, 2h + 1 as (hi, lo)
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int t = 2 * h + q;
        const int rr = tr ? t % 6 : t / 6, cc = tr ? t / 6 : t % 6;
        acc_madd(acc[rr], q ? dd_make(v.z, v.w) : dd_make(v.x, v.y), uk[cc]);
      }
    }
  }
#pragma unroll
  for (int r = 0; r < 6; ++r) {
    dd t = acc_get(acc[r]);
    for (int off = 16; off > 0; off >>= 1)
      t = dd_add(t, dd_make(__shfl_xor_sync(0xffffffffu, t.hi, off), __shfl_xor_sync(0xffffffffu, t.lo, off)));
    w6[r] = dd_to_double(t);
  }
}

// z = P_j r_j for the row's six entries (lane < 6 holds r_{6j+lane}).
__device__ __forceinline__ double precond_row(const PcgArgs& a, int j, double rv) {
  const int lane = threadIdx.x & 31;
  double zv = 0.0;
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    const double rc = __shfl_sync(0xffffffffu, rv, c);
    if (lane < 6) zv = fma(a.P[36 * static_cast<int64_t>(j) + lane * 6 + c], rc, zv);
  }
  return zv;
}

// PCG in the single-reduction form of Chronopoulos and Gear ("s-step
// iterative methods for symmetric linear systems", 1989): one matrix-vector
// product and one fused reduction of (r, u), (w, u), (r, r) per iteration,
// two grid barriers.  x~ solves S~ x~ = b~ (Jacobi-scaled).
__global__ void __launch_bounds__(kPT) k_pcg_solve(PcgArgs a, Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  const int lane = threadIdx.x & 31;
  const int gw = blockIdx.x * kPW + (threadIdx.x >> 5);
  const int nw = gridDim.x * kPW;
  const unsigned nb = gridDim.x;
  unsigned nbar = 0;
  double* x = a.vec;
  double* r = a.vec + a.n6;
  double* u = a.vec + 2 * a.n6;
  double* p = a.vec + 3 * a.n6;
  double* sv = a.vec + 4 * a.n6;  // s = S~ p
  double* w = a.vec + 5 * a.n6;   // w = S~ u
  // x = 0, r = b~, u = P r
  for (int j = gw; j < a.nf; j += nw) {
    double rv = 0.0;
    if (lane < 6) {
      const int i = 6 * j + lane;
      rv = (a.scl ? a.scl[i] : 1.0) * a.rb[i];
      x[i] = 0.0;
      r[i] = rv;
      p[i] = 0.0;
      sv[i] = 0.0;
    }
    const double zv = precond_row(a, j, rv);
    if (lane < 6) u[6 * j + lane] = zv;
  }
  bool ok = grid_barrier(a.bar, (++nbar) * nb);
  double gamma = 0.0, alpha = 0.0, bnorm2 = 0.0, rr = 0.0;
  int it = 0;
  int status = ok ? 1 : 3;
  for (;;) {
    if (!ok) { status = 3; break; }
    // w = S~ u; dots (r, u), (w, u), (r, r)
    double ru = 0.0, wu = 0.0, r2 = 0.0;
    for (int j = gw; j < a.nf; j += nw) {
      double w6[6];
      block_row_matvec(a, j, u, w6);
      if (lane < 6) {
        const int i = 6 * j + lane;
        const double wv = w6[lane], uv = u[i], rv = r[i];
        w[i] = wv;
        ru += rv * uv;
        wu += wv * uv;
        r2 += rv * rv;
      }
    }
    write_parts3(a.part, ru, wu, r2);
    if (!(ok = grid_barrier(a.bar, (++nbar) * nb))) { status = 3; break; }
    double sums[3];
    sum_parts3(a.part, sums);
    const double gamma_n = sums[0], delta = sums[1];
    rr = sums[2];
    if (it == 0) bnorm2 = rr;
    if (!(bnorm2 > 0.0)) { status = 0; break; }  // b = 0: x = 0 is exact
    if (rr <= a.tol * a.tol * bnorm2) { status = 0; break; }
    if (it >= a.max_iters) { status = 1; break; }
    double beta;
    if (it == 0) {
      beta = 0.0;
      alpha = gamma_n / delta;
    } else {
      beta = gamma_n / gamma;
      alpha = gamma_n / (delta - beta * gamma_n / alpha);
    }
    gamma = gamma_n;
    if (!(alpha > 0.0) || !isfinite(alpha) || !(gamma_n > 0.0)) { status = 2; break; }
    // p = u + beta p, s = w + beta s, x += alpha p, r -= alpha s, u = P r
    for (int j = gw; j < a.nf; j += nw) {
      double rv = 0.0;
      if (lane < 6) {
        const int i = 6 * j + lane;
        const double pv = fma(beta, p[i], u[i]);
        const double sn = fma(beta, sv[i], w[i]);
        p[i] = pv;
        sv[i] = sn;
        x[i] = fma(alpha, pv, x[i]);
        rv = fma(-alpha, sn, r[i]);
        r[i] = rv;
      }
      const double zv = precond_row(a, j, rv);
      if (lane < 6) u[6 * j + lane] = zv;
    }
    ++it;
    if (!(ok = grid_barrier(a.bar, (++nbar) * nb))) { status = 3; break; }
  }
  const bool conv = ok && status == 0;
  if (conv) {
    for (int j = gw; j < a.nf; j += nw) {
      if (lane < 6) {
        const int i = 6 * j + lane;
        const double v = (a.scl ? a.scl[i] : 1.0) * x[i];
        if (a.xout) a.xout[i] = v;
        if (a.xdd) {
          const dd vd = dd_from_double(v);
          a.xdd[2 * i] = vd.hi;
          a.xdd[2 * i + 1] = vd.lo;
        }
      }
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && ctrl) {
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
  a.Sb2 = d.pcg_S2;
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

int launch_pcg_blocks_only(const Sizes& s, const Dev& d, cudaStream_t st) {
  const PcgArgs a = pcg_args(s, d);
  const int64_t total = s.nsb * 36;
  const int blocks = static_cast<int>(std::min<int64_t>((total + kPT - 1) / kPT, 8192));
  k_pcg_blocks<<<blocks > 0 ? blocks : 1, kPT, 0, st>>>(a, d.ctrl);
  return 1;
}

int launch_pcg(const Sizes& s, const Dev& d, cudaStream_t st) {
  return launch_pcg_blocks_only(s, d, st) + launch_pcg_scaled(s, d, st);
}

int launch_pcg_scaled(const Sizes& s, const Dev& d, cudaStream_t st) {
  const PcgArgs a = pcg_args(s, d);
  int n = 0;
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
