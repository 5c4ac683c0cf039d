// sgba_dense.cu -- factorization and solve of a dense reduced camera system
// in ONE launch of one thread-block cluster, the matrix resident in the
// cluster's distributed shared memory.
//
// Same arithmetic contract as sgba_solver.cu (the multi-launch path it
// replaces for systems that fit): scalar LDL^T in natural order with the
// PSD-aware pivot rule of the reference (crates/sophus_solver/src/ldlt/dense_ldlt.rs:164-270,
// tol_rel = 1e-12, the relative threshold restarting at every 6x6 pose block;
// a zero pivot zeroes its column of L and its solution entry), FP32 factor,
// of the diagonally scaled matrix, then refinement steps whose residual
// b - S x is formed in float-float from the float-float copy of S written by
// k_schur.
//
// Layout: n is padded to P blocks of kNB = 24 rows (4 pose blocks; padding
// rows are identity).  Row block r (rows 24r..24r+23, columns 0..24r+23) lives
// in the shared memory of cluster rank r % C.  Per panel step p:
//   owner(p), warp 0: LDL^T of the diagonal block, 1/d and the inverse of
//      its unit lower factor; then all its threads store that inverse and
//      1/d into every CTA (DSMEM stores);
//   -- cluster barrier --
//   every CTA, its row blocks r > p: W_rp = A_rp L_pp^-T, L_rp = W_rp D^-1;
//   -- cluster barrier --
//   every CTA, row blocks r > p: A_rs -= W_rp L_sp^T for p < s <= r, L_sp
//      read in place from its owner's shared memory.  The owner of p+1
//      updates block p+1 first; its warp 0 then runs the diagonal step of
//      p+1 while the other warps finish the update.
// Triangular solves: one split cluster barrier per 24-row block; the owner
// of the block does only the critical 24x24 work before arriving (in the
// forward sweep it also stores its piece of y into the next block's owner),
// every CTA folds the older solution pieces into its accumulators while the
// barrier completes.
//
// GB300 notes that shaped the code (measured): a cluster barrier costs ~400
// cycles and a DSMEM load ~200, while warp shuffles in long chains and DSMEM
// stores issued one after another by a single warp are far slower; so
// reductions and broadcasts go through shared memory and data moves between
// CTAs as loads by the consumer.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "sgba_dd.cuh"
#include "sgba_internal.h"

namespace cg = cooperative_groups;

namespace sgba {

namespace {

constexpr int kNB = 24;
constexpr int kLd = 28;              // row stride of the 24x24 inverses (float4 rows)
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxOwn = 24;          // row blocks per CTA
constexpr int kMaxCluster = 16;
constexpr float kTolRel = 1e-12f;
constexpr int kRefine = 2;           // refinement steps against the float-float S (at most)
// Systems of at most kRefineSmallN rows (local windows) refine up to
// kRefineSmall times: their sweeps are a few panel steps, and two steps left
// 7.5e-6 of the step in a 34-camera window (relative, outside the gauge).
constexpr int kRefineSmallN = 240;
constexpr int kRefineSmall = 4;
constexpr float kRefineSkip = 1e-9f;  // predicted relative error below which the second one is skipped
constexpr size_t kSmemLimit = 232448;  // 227 KiB opt-in dynamic shared memory per CTA

__host__ __device__ inline int row_ld(int r) { return kNB * (r + 1) + 4; }

// Shared-memory carve-up of one CTA (floats), identical on host and device.
struct Carve {
  int nown;
  int rowoff[kMaxOwn];
  int wt, linv, dloc, rdloc, lpp, rdp, y, x, xs, xlo, bl, facc, accb, vdef, udef, red, tmp, tmp2, colbuf, ynext, flags, total;
};

__host__ __device__ inline void carve(int P, int C, int rank, Carve* c) {
  int off = 0;
  c->nown = 0;
  for (int r = rank; r < P; r += C) {
    if (c->nown < kMaxOwn) c->rowoff[c->nown] = off;
    ++c->nown;
    off += kNB * row_ld(r);
  }
  const int npad = kNB * P;
  auto take = [&](int n) { int o = off; off += (n + 3) & ~3; return o; };
  c->wt = take(c->nown * kNB * kNB);
  c->linv = take(c->nown * kNB * kLd);
  c->dloc = take(c->nown * kNB);
  c->rdloc = take(c->nown * kNB);
  c->lpp = take(kNB * kLd);
  c->rdp = take(kNB);
  c->y = take(npad);
  c->x = take(npad);
  c->xs = take(npad);
  c->xlo = take(npad);
  c->bl = take(npad);
  c->facc = take(c->nown * kNB);
  c->accb = take(npad);
  c->vdef = take(npad);
  c->udef = take(npad);
  c->red = take(2 * kThreads);
  c->tmp = take(32);
  c->tmp2 = take(32);
  c->colbuf = take(64);
  c->ynext = take(32);
  c->flags = take(4);
  c->total = off;
}

struct DenseArgs {
  int n;             // unpadded order (6 n_f)
  int P;             // 24-row blocks
  const float2* S2;  // n x n float-float (hi, lo), full symmetric
  const double* b;   // n reduced rhs
  double* x;         // n solution (f64)
  float* xdd;        // n solution as float-float pairs
  // scale gauge (one constant camera, no constant point): direction v of the
  // free poses' translations about the constant camera's center
  int gauge;
  const double* poses;
  const int32_t* fb_pose;
  double center[3];
  int npose;         // rows of the free poses (6 n_f; free intrinsics follow them)
  int refine;        // refinement steps at most (cluster solver)
  // equality constraints (one-CTA solver): G row k is jac + 3k at rows
  // 6 fb_k + 3 .. 5; c; the multiplier step out
  int n_eq;
  const int32_t* eq_fb;
  const double* eq_jac;
  const double* eq_c;
  double* eq_dlam;
};

// the factorization is skipped on termination, on a skipped step and when PCG converged
__device__ __forceinline__ bool skipping(const Ctrl* c) { return c->done != 0 || c->skip != 0 || c->pcg_done != 0; }

__device__ __forceinline__ void cl_arrive() { asm volatile("barrier.cluster.arrive.release;\n" ::: "memory"); }
__device__ __forceinline__ void cl_wait() { asm volatile("barrier.cluster.wait.acquire;\n" ::: "memory"); }
__device__ __forceinline__ void cl_sync() {
  cl_arrive();
  cl_wait();
}

// Offsets of every rank's regions (remote addressing), filled at kernel start.
struct RankTab {
  int rowoff[kMaxCluster][kMaxOwn];
  int linv[kMaxCluster], rdloc[kMaxCluster], y[kMaxCluster], x[kMaxCluster], accb[kMaxCluster], flags[kMaxCluster];
  int lpp[kMaxCluster], rdp[kMaxCluster], ynext[kMaxCluster];
};

struct Ctx {
  float* sm;
  const Carve* cv;  // this CTA's carve-up, in shared memory
  const RankTab* T;
  int C, rank, P, n;
  __device__ float* rowblk(int r) const { return sm + cv->rowoff[r / C]; }  // r owned by this CTA
  __device__ int ld(int r) const { return row_ld(r); }
  __device__ bool owns(int r) const { return r % C == rank; }
};

__device__ __forceinline__ float* remote(cg::cluster_group& cl, float* sm, int rank, int off) {
  return cl.map_shared_rank(sm + off, rank);
}

// Diagonal step of block p (owner, warp 0): LDL^T of the 24x24 diagonal block
// in place (lane i keeps row i in registers; each column is broadcast through
// shared memory, read back as float4s; two buffers, one warp barrier per
// pivot), 1/d, and the inverse of its unit lower factor.
__device__ void diag_step(const Ctx& X, int p, int* bad_flag) {
  const int lane = threadIdx.x & 31;
  const int jp = p / X.C;
  float* Ab = X.rowblk(p) + kNB * p;
  const int ld = X.ld(p);
  float* colbuf = X.sm + X.cv->colbuf;  // two 32-float column buffers
  float a[kNB];
#pragma unroll
  for (int k = 0; k < kNB; ++k) a[k] = (lane < kNB && k <= lane) ? Ab[lane * ld + k] : 0.0f;
  float maxp = 1.0f;
  float* dl = X.sm + X.cv->dloc + kNB * jp;
  float* rdl = X.sm + X.cv->rdloc + kNB * jp;
#pragma unroll
  for (int t = 0; t < kNB; ++t) {
    if (t % 6 == 0) maxp = 1.0f;  // 24p is a multiple of 6: a new pose block starts here
    float* cb = colbuf + 32 * (t & 1);  // two buffers: one warp barrier per pivot
    cb[lane] = a[t];
    __syncwarp();
    float col[kNB];
#pragma unroll
    for (int q = 0; q < kNB / 4; ++q) {
      const float4 v = reinterpret_cast<const float4*>(cb)[q];
      col[4 * q] = v.x; col[4 * q + 1] = v.y; col[4 * q + 2] = v.z; col[4 * q + 3] = v.w;
    }
    float dt = col[t];
    const float tol = fmaxf(maxp, 1.0f) * kTolRel;
    if (fabsf(dt) <= tol) dt = 0.0f;
    else maxp = fmaxf(maxp, fabsf(dt));
    const float rd = (dt == 0.0f) ? 0.0f : __frcp_rn(dt);
    const float li = (lane > t) ? a[t] * rd : 0.0f;
    // entries above this lane's diagonal take junk here; they are never read or stored
#pragma unroll
    for (int k = t + 1; k < kNB; ++k) a[k] = fmaf(-li, col[k], a[k]);
    if (lane > t) a[t] = li;
    if (lane == 0) {
      dl[t] = dt;
      rdl[t] = rd;
    }
  }
  __syncwarp();
  if (lane < kNB) {
#pragma unroll
    for (int k = 0; k < kNB; ++k)
      if (k < lane) Ab[lane * ld + k] = a[k];
    Ab[lane * ld + lane] = 1.0f;
  }
  __syncwarp();
  if (lane < kNB && !isfinite(dl[lane])) *bad_flag = 1;  // NonFinitePivot
  // inverse of the unit lower factor: lane j computes column j
  float xc[kNB];
#pragma unroll
  for (int i = 0; i < kNB; ++i) xc[i] = (i == lane) ? 1.0f : 0.0f;
#pragma unroll
  for (int i = 1; i < kNB; ++i) {
    float row[kNB];
#pragma unroll
    for (int q = 0; q < (i + 3) / 4; ++q) {
      const float4 v = reinterpret_cast<const float4*>(Ab + i * ld)[q];
      row[4 * q] = v.x; row[4 * q + 1] = v.y; row[4 * q + 2] = v.z; row[4 * q + 3] = v.w;
    }
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll
    for (int k = 0; k < i; ++k) {
      if (k % 4 == 0) s0 = fmaf(row[k], xc[k], s0);
      else if (k % 4 == 1) s1 = fmaf(row[k], xc[k], s1);
      else if (k % 4 == 2) s2 = fmaf(row[k], xc[k], s2);
      else s3 = fmaf(row[k], xc[k], s3);
    }
    if (i > lane) xc[i] = -((s0 + s1) + (s2 + s3));
  }
  float* Li = X.sm + X.cv->linv + kNB * kLd * jp;
  if (lane < kNB) {
#pragma unroll
    for (int i = 0; i < kNB; ++i) Li[i * kLd + lane] = xc[i];
  }
}

// The owner of block b, all threads, after its diagonal step: Linv_bb and
// 1/d_b into every CTA's lpp / rdp (DSMEM stores; the next cluster barrier
// publishes them). Their previous contents were last read by panel_rows of
// the step before, which every CTA finished before that step's second barrier.
__device__ void push_diag(const Ctx& X, cg::cluster_group& cl, int b) {
  constexpr int kRowsF4 = kNB * (kLd / 4), kAllF4 = kRowsF4 + kNB / 4;
  const int jb = b / X.C;
  const float4* lsrc = reinterpret_cast<const float4*>(X.sm + X.cv->linv + kNB * kLd * jb);
  const float4* rsrc = reinterpret_cast<const float4*>(X.sm + X.cv->rdloc + kNB * jb);
  for (int e = threadIdx.x; e < kAllF4 * X.C; e += kThreads) {
    const int c = e / kAllF4, q = e - c * kAllF4;
    if (q < kRowsF4) {
      reinterpret_cast<float4*>(remote(cl, X.sm, c, X.T->lpp[c]))[q] = lsrc[q];
    } else {
      reinterpret_cast<float4*>(remote(cl, X.sm, c, X.T->rdp[c]))[q - kRowsF4] = rsrc[q - kRowsF4];
    }
  }
}

// Panel step p, every CTA: for the owned row blocks r > p,
// W_rp = A_rp Linv_pp^T (kept transposed for the update) and L_rp = W_rp D^-1
// in place.  Linv_pp and 1/d were pushed by the owner of p.  4x4 register
// tiles from float4 shared-memory reads; every entry is summed over k in order.
__device__ void panel_rows(const Ctx& X, int p) {
  int j0 = 0;
  while (j0 < X.cv->nown && X.rank + j0 * X.C <= p) ++j0;
  const int ntile = (X.cv->nown - j0) * 36;  // 4x4 tiles of each 24x24 block
  const float* lpp = X.sm + X.cv->lpp;
  const float* rdp = X.sm + X.cv->rdp;
  // W = A_rp Linv_pp^T, 4x4 tiles; each entry summed over k in order; stored transposed (wt)
  for (int e = threadIdx.x; e < ntile; e += kThreads) {
    const int jr = j0 + e / 36, rem = e % 36, i0 = 4 * (rem / 6), t0 = 4 * (rem % 6);
    const int r = X.rank + jr * X.C, ld = X.ld(r);
    const float* A0 = X.sm + X.cv->rowoff[jr] + kNB * p;
    float w[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) w[u][v] = 0.f;
#pragma unroll
    for (int q = 0; q < kNB / 4; ++q) {
      float4 av[4], lv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) av[u] = reinterpret_cast<const float4*>(A0 + (i0 + u) * ld)[q];
#pragma unroll
      for (int v = 0; v < 4; ++v) lv[v] = reinterpret_cast<const float4*>(lpp + (t0 + v) * kLd)[q];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          float acc = w[u][v];
          acc = fmaf(av[u].x, lv[v].x, acc);
          acc = fmaf(av[u].y, lv[v].y, acc);
          acc = fmaf(av[u].z, lv[v].z, acc);
          acc = fmaf(av[u].w, lv[v].w, acc);
          w[u][v] = acc;
        }
    }
    float* wt = X.sm + X.cv->wt + kNB * kNB * jr;
#pragma unroll
    for (int v = 0; v < 4; ++v)
      reinterpret_cast<float4*>(wt + (t0 + v) * kNB + i0)[0] = make_float4(w[0][v], w[1][v], w[2][v], w[3][v]);
  }
  __syncthreads();
  // L_rp = W D^-1 in place
  for (int e = threadIdx.x; e < ntile; e += kThreads) {
    const int jr = j0 + e / 36, rem = e % 36, i0 = 4 * (rem / 6), t0 = 4 * (rem % 6);
    const int r = X.rank + jr * X.C, ld = X.ld(r);
    float* A0 = X.sm + X.cv->rowoff[jr] + kNB * p;
    const float* wt = X.sm + X.cv->wt + kNB * kNB * jr;
    float4 wv[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) wv[v] = reinterpret_cast<const float4*>(wt + (t0 + v) * kNB + i0)[0];
    const float4 rv = reinterpret_cast<const float4*>(rdp)[t0 / 4];
    reinterpret_cast<float4*>(A0 + (i0 + 0) * ld + t0)[0] = make_float4(wv[0].x * rv.x, wv[1].x * rv.y, wv[2].x * rv.z, wv[3].x * rv.w);
    reinterpret_cast<float4*>(A0 + (i0 + 1) * ld + t0)[0] = make_float4(wv[0].y * rv.x, wv[1].y * rv.y, wv[2].y * rv.z, wv[3].y * rv.w);
    reinterpret_cast<float4*>(A0 + (i0 + 2) * ld + t0)[0] = make_float4(wv[0].z * rv.x, wv[1].z * rv.y, wv[2].z * rv.z, wv[3].z * rv.w);
    reinterpret_cast<float4*>(A0 + (i0 + 3) * ld + t0)[0] = make_float4(wv[0].w * rv.x, wv[1].w * rv.y, wv[2].w * rv.z, wv[3].w * rv.w);
  }
}

// Owner of p+1: the update of its diagonal block by panel p,
// A_{p+1,p+1} -= W_{p+1,p} L_{p+1,p}^T (lower triangle; both factors local),
// in 4x4 register tiles (21 of them), each entry summed over t in order.
__device__ void diag_update(const Ctx& X, int p) {
  const int r = p + 1, jr = r / X.C, ld = X.ld(r);
  float* Ar = X.rowblk(r);
  const float* wt = X.sm + X.cv->wt + kNB * kNB * jr;
  // 4x4 tiles (i0, k0) of the lower triangle, k0 <= i0: 21 tiles
  for (int e = threadIdx.x; e < 21; e += kThreads) {
    int ib = 0, rem = e;
    while (rem > ib) { rem -= ib + 1; ++ib; }
    const int i0 = 4 * ib, k0 = 4 * rem;
    float acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
#pragma unroll
    for (int q = 0; q < kNB / 4; ++q) {
      float4 lk[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) lk[v] = reinterpret_cast<const float4*>(Ar + (k0 + v) * ld + kNB * p)[q];
      float4 wv[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) wv[c] = reinterpret_cast<const float4*>(wt + (4 * q + c) * kNB + i0)[0];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const float lt[4] = {lk[v].x, lk[v].y, lk[v].z, lk[v].w};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          acc[0][v] = fmaf(wv[c].x, lt[c], acc[0][v]);
          acc[1][v] = fmaf(wv[c].y, lt[c], acc[1][v]);
          acc[2][v] = fmaf(wv[c].z, lt[c], acc[2][v]);
          acc[3][v] = fmaf(wv[c].w, lt[c], acc[3][v]);
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v)
        if (k0 + v <= i0 + u) Ar[(i0 + u) * ld + kNB * r + k0 + v] -= acc[u][v];
  }
}

// Row jj of L_sp (24 floats at column 24p of row block s), local or remote.
__device__ __forceinline__ const float4* lrow(const Ctx& X, cg::cluster_group& cl, int s, int jj, int p) {
  const int os = s % X.C;
  const float* base = (os == X.rank) ? X.sm + X.cv->rowoff[s / X.C]
                                     : remote(cl, X.sm, os, X.T->rowoff[os][s / X.C]);
  return reinterpret_cast<const float4*>(base + jj * row_ld(s) + kNB * p);
}

// Update of panel p for the owned row blocks r in [r_lo, r_hi] by warps
// [w0, w0 + nw): A_r[:, 24(p+1) + col] -= W_rp L_sp[jj]^T with
// col = 24(s - p - 1) + jj.  A lane owns two output columns.
__device__ void update_blocks(const Ctx& X, cg::cluster_group& cl, int p, int r_lo, int r_hi, int w0, int nw) {
  const int warp = (threadIdx.x >> 5) - w0;
  if (warp < 0 || warp >= nw) return;
  const int lane = threadIdx.x & 31;
  int task = 0;
  for (int r = X.rank; r < X.P; r += X.C) {
    if (r < r_lo || r > r_hi) continue;
    const int ncol = kNB * (r - p);
    const int nchunk = (ncol + 63) / 64;
    const float4* wt = reinterpret_cast<const float4*>(X.sm + X.cv->wt + kNB * kNB * (r / X.C));
    float* Ar = X.rowblk(r) + kNB * (p + 1);
    const int ld = X.ld(r);
    for (int ch = 0; ch < nchunk; ++ch, ++task) {
      if (task % nw != warp) continue;
      const int ca = ch * 64 + lane, cb = ca + 32;
      const bool va = ca < ncol, vb = cb < ncol;
      float la[kNB], lb[kNB];
      {
        const int c0 = va ? ca : 0, c1 = vb ? cb : 0;
        const float4* pa = lrow(X, cl, p + 1 + c0 / kNB, c0 % kNB, p);
        const float4* pb = lrow(X, cl, p + 1 + c1 / kNB, c1 % kNB, p);
#pragma unroll
        for (int q = 0; q < kNB / 4; ++q) {
          const float4 u = pa[q], v = pb[q];
          la[4 * q] = u.x; la[4 * q + 1] = u.y; la[4 * q + 2] = u.z; la[4 * q + 3] = u.w;
          lb[4 * q] = v.x; lb[4 * q + 1] = v.y; lb[4 * q + 2] = v.z; lb[4 * q + 3] = v.w;
        }
      }
      float acc0[kNB], acc1[kNB];
#pragma unroll
      for (int i = 0; i < kNB; ++i) { acc0[i] = 0.f; acc1[i] = 0.f; }
#pragma unroll
      for (int k = 0; k < kNB; ++k) {
#pragma unroll
        for (int q = 0; q < kNB / 4; ++q) {
          const float4 w = wt[k * (kNB / 4) + q];
          acc0[4 * q + 0] = fmaf(w.x, la[k], acc0[4 * q + 0]);
          acc0[4 * q + 1] = fmaf(w.y, la[k], acc0[4 * q + 1]);
          acc0[4 * q + 2] = fmaf(w.z, la[k], acc0[4 * q + 2]);
          acc0[4 * q + 3] = fmaf(w.w, la[k], acc0[4 * q + 3]);
          acc1[4 * q + 0] = fmaf(w.x, lb[k], acc1[4 * q + 0]);
          acc1[4 * q + 1] = fmaf(w.y, lb[k], acc1[4 * q + 1]);
          acc1[4 * q + 2] = fmaf(w.z, lb[k], acc1[4 * q + 2]);
          acc1[4 * q + 3] = fmaf(w.w, lb[k], acc1[4 * q + 3]);
        }
      }
      if (va) {
#pragma unroll
        for (int i = 0; i < kNB; ++i) Ar[i * ld + ca] -= acc0[i];
      }
      if (vb) {
#pragma unroll
        for (int i = 0; i < kNB; ++i) Ar[i * ld + cb] -= acc1[i];
      }
    }
  }
}

// L y = bl over the 24-row blocks.  The owner of block p finds y_{p-1} in its
// own ynext (stored there by the owner of p-1 before the previous barrier),
// adds L_{p,p-1} y_{p-1} to its accumulator, forms y_p in its own shared
// memory, stores a copy into the ynext of the owner of p+1 and arrives;
// meanwhile every CTA pulls y_{p-1} and folds it into the accumulators of its
// other blocks.  Pieces of y stay with their owners (the backward pass reads
// only its own).  The next store into a CTA's ynext follows its read: at
// least one cluster barrier later when C > 1, after the warp barrier of the
// same step when C = 1.
__device__ void solve_forward(const Ctx& X, cg::cluster_group& cl) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  float* y = X.sm + X.cv->y;
  float* facc = X.sm + X.cv->facc;
  float* tmp = X.sm + X.cv->tmp;
  const float* bl = X.sm + X.cv->bl;
  for (int e = tid; e < X.cv->nown * kNB; e += kThreads) facc[e] = 0.f;
  __syncthreads();
  cl_sync();
  for (int p = 0; p < X.P; ++p) {
    if (X.owns(p) && warp == 0) {
      const int jp = p / X.C;
      const float* yprev = X.sm + X.cv->ynext;  // y_{p-1}, stored here by its owner
      if (lane < kNB) {
        float s0 = facc[kNB * jp + lane], s1 = 0.f, s2 = 0.f, s3 = 0.f;
        if (p > 0) {
          const float4* lr = reinterpret_cast<const float4*>(X.rowblk(p) + lane * X.ld(p) + kNB * (p - 1));
          const float4* yq = reinterpret_cast<const float4*>(yprev);
#pragma unroll
          for (int q = 0; q < kNB / 4; ++q) {
            const float4 a4 = lr[q], b4 = yq[q];
            s0 = fmaf(a4.x, b4.x, s0); s1 = fmaf(a4.y, b4.y, s1); s2 = fmaf(a4.z, b4.z, s2); s3 = fmaf(a4.w, b4.w, s3);
          }
        }
        tmp[lane] = bl[kNB * p + lane] - ((s0 + s1) + (s2 + s3));
      }
      __syncwarp();
      if (lane < kNB) {
        const float4* li = reinterpret_cast<const float4*>(X.sm + X.cv->linv + kNB * kLd * jp + lane * kLd);
        const float4* t4 = reinterpret_cast<const float4*>(tmp);
        float v0 = 0.f, v1 = 0.f, v2 = 0.f, v3 = 0.f;
#pragma unroll
        for (int q = 0; q < kNB / 4; ++q) {
          const float4 a4 = li[q], b4 = t4[q];
          v0 = fmaf(a4.x, b4.x, v0); v1 = fmaf(a4.y, b4.y, v1); v2 = fmaf(a4.z, b4.z, v2); v3 = fmaf(a4.w, b4.w, v3);
        }
        const float v = (v0 + v1) + (v2 + v3);
        y[kNB * p + lane] = v;
        if (p + 1 < X.P) {  // to the owner of the next block, before this block's barrier
          const int on = (p + 1) % X.C;
          remote(cl, X.sm, on, X.T->ynext[on])[lane] = v;
        }
      }
    }
    __syncthreads();
    cl_arrive();
    if (p > 0) {
      int j0 = 0;
      while (j0 < X.cv->nown && X.rank + j0 * X.C <= p) ++j0;
      if (j0 < X.cv->nown) {
        const int oq = (p - 1) % X.C;
        if (tid < kNB && oq != X.rank) y[kNB * (p - 1) + tid] = remote(cl, X.sm, oq, X.T->y[oq])[kNB * (p - 1) + tid];
        __syncthreads();
        const int rows = (X.cv->nown - j0) * kNB;
        const float* yq = y + kNB * (p - 1);
        for (int e = tid; e < rows; e += kThreads) {
          const int jr = j0 + e / kNB, i = e % kNB;
          const int r = X.rank + jr * X.C;
          const float* lr = X.sm + X.cv->rowoff[jr] + i * X.ld(r) + kNB * (p - 1);
          float s = 0.f;
#pragma unroll
          for (int k = 0; k < kNB; ++k) s = fmaf(lr[k], yq[k], s);
          facc[kNB * jr + i] += s;
        }
      }
    }
    __syncthreads();
    cl_wait();
  }
}

// L^T x = D^-1 y over the blocks in reverse.  Each CTA accumulates the
// contributions L_pq^T x_p of its own blocks p into accb; the owner of block
// p sums the accumulators of all ranks in rank order.  It adds its own
// contribution to block p-1 before arriving, the rest after.  Pieces of x
// stay with their owners; gather_x collects the whole vector.
__device__ void solve_backward(const Ctx& X, cg::cluster_group& cl) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int npad = kNB * X.P;
  const float* y = X.sm + X.cv->y;
  float* x = X.sm + X.cv->x;
  float* accb = X.sm + X.cv->accb;
  float* tmp = X.sm + X.cv->tmp;
  float* tmp2 = X.sm + X.cv->tmp2;
  for (int k = tid; k < npad; k += kThreads) accb[k] = 0.f;
  __syncthreads();
  cl_sync();
  for (int p = X.P - 1; p >= 0; --p) {
    const bool own = X.owns(p);
    if (own && warp == 0) {
      const int jp = p / X.C;
      if (lane < kNB) {
        float part[kMaxCluster];
#pragma unroll
        for (int c = 0; c < kMaxCluster; ++c)
          part[c] = (c < X.C) ? remote(cl, X.sm, c, X.T->accb[c])[kNB * p + lane] : 0.f;
        float s = 0.f;
#pragma unroll
        for (int c = 0; c < kMaxCluster; ++c) s += part[c];
        const float z = y[kNB * p + lane] * X.sm[X.cv->rdloc + kNB * jp + lane];
        tmp[lane] = z - s;
      }
      __syncwarp();
      if (lane < kNB) {
        const float* li = X.sm + X.cv->linv + kNB * kLd * jp;
        float v = 0.f;
#pragma unroll
        for (int i = 0; i < kNB; ++i) v = fmaf(li[i * kLd + lane], tmp[i], v);
        tmp2[lane] = v;
        x[kNB * p + lane] = v;
      }
      __syncwarp();
      if (p > 0 && lane < kNB) {
        const float* ap = X.rowblk(p) + kNB * (p - 1) + lane;
        const int ld = X.ld(p);
        float s = 0.f;
#pragma unroll
        for (int i = 0; i < kNB; ++i) s = fmaf(ap[i * ld], tmp2[i], s);
        accb[kNB * (p - 1) + lane] += s;
      }
    }
    __syncthreads();
    cl_arrive();
    if (own && p > 1) {
      const float* ap = X.rowblk(p);
      const int ld = X.ld(p);
      for (int k = tid; k < kNB * (p - 1); k += kThreads) {
        float s = 0.f;
#pragma unroll
        for (int i = 0; i < kNB; ++i) s = fmaf(ap[i * ld + k], tmp2[i], s);
        accb[k] += s;
      }
    }
    __syncthreads();
    cl_wait();
  }
}

// Every CTA: copy the pieces of x owned by the other ranks (after a barrier).
__device__ void gather_x(const Ctx& X, cg::cluster_group& cl) {
  float* x = X.sm + X.cv->x;
  for (int q = threadIdx.x; q < X.P * (kNB / 4); q += kThreads) {
    const int blk = q / (kNB / 4), ob = blk % X.C;
    if (ob == X.rank) continue;
    reinterpret_cast<float4*>(x)[q] = reinterpret_cast<const float4*>(remote(cl, X.sm, ob, X.T->x[ob]))[q];
  }
  __syncthreads();
}

// Sum over one warp through shared memory (fixed tree, no shuffles).
__device__ dd warp_sum_dd(dd v, float* wred, int lane) {
  wred[2 * lane] = v.hi;
  wred[2 * lane + 1] = v.lo;
  __syncwarp();
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) {
    if (lane < s) {
      const dd u = dd_add(dd_make(wred[2 * lane], wred[2 * lane + 1]),
                          dd_make(wred[2 * (lane + s)], wred[2 * (lane + s) + 1]));
      wred[2 * lane] = u.hi;
      wred[2 * lane + 1] = u.lo;
    }
    __syncwarp();
  }
  const dd r = dd_make(wred[0], wred[1]);
  __syncwarp();
  return r;
}

// Sum over the CTA through shared memory (fixed tree); every thread gets it.
__device__ dd block_sum_dd(dd v, float* red) {
  const int tid = threadIdx.x;
  red[2 * tid] = v.hi;
  red[2 * tid + 1] = v.lo;
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if (tid < s) {
      const dd u = dd_add(dd_make(red[2 * tid], red[2 * tid + 1]), dd_make(red[2 * (tid + s)], red[2 * (tid + s) + 1]));
      red[2 * tid] = u.hi;
      red[2 * tid + 1] = u.lo;
    }
    __syncthreads();
  }
  const dd r = dd_make(red[0], red[1]);
  __syncthreads();
  return r;
}

// bl = D^-1/2 (b - S x) on the owned rows (FP32 of the float-float
// residual), b and S in float-float, x = (xs, xlo) the float-float solution.
__device__ void residual(const Ctx& X, const DenseArgs& a, float alpha) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const float* xh = X.sm + X.cv->xs;
  const float* xl = X.sm + X.cv->xlo;
  const float* vd = X.sm + X.cv->vdef;
  const float* ud = X.sm + X.cv->udef;
  float* bl = X.sm + X.cv->bl;
  float* wred = X.sm + X.cv->red + 64 * warp;
  // deflated operator (retry after a breakdown): subtract alpha u (u . x~), x~ = D^1/2 x
  dd g = dd_make(0.f, 0.f);
  if (alpha != 0.0f) {
    for (int k = tid; k < a.n; k += kThreads) g = dd_add(g, dd_mul_f(dd_make(xh[k], xl[k]), ud[k] / vd[k]));
    g = block_sum_dd(g, X.sm + X.cv->red);
  }
  const dd ag = dd_mul_f(g, alpha);
  for (int jr = 0; jr < X.cv->nown; ++jr) {
    const int r = X.rank + jr * X.C;
    for (int i = warp; i < kNB; i += kWarps) {
      const int row = kNB * r + i;
      if (row >= a.n) {
        if (lane == 0) bl[row] = 0.f;
        continue;
      }
      const float2* srow = a.S2 + static_cast<int64_t>(row) * a.n;
      dd acc = dd_make(0.f, 0.f);
      for (int k0 = lane; k0 < a.n; k0 += 32 * 8) {
        float2 sv[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int k = k0 + 32 * u;
          sv[u] = (k < a.n) ? srow[k] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int k = k0 + 32 * u;
          if (k < a.n) acc = dd_add(acc, dd_mul(dd_make(sv[u].x, sv[u].y), dd_make(xh[k], xl[k])));
        }
      }
      acc = warp_sum_dd(acc, wred, lane);
      if (lane == 0) {
        const dd rr = dd_sub(dd_from_double(a.b[row]), acc);
        bl[row] = (rr.hi + rr.lo) * vd[row] - (ag.hi + ag.lo) * ud[row];
      }
    }
  }
}

__device__ __forceinline__ float* dsm_ptr(const Ctx& X) { return X.sm; }

__device__ void load_rows(const Ctx& X, const DenseArgs& a, float alpha) {
  const int tid = threadIdx.x;
  const float* vd = dsm_ptr(X) + X.cv->vdef;
  const float* ud = dsm_ptr(X) + X.cv->udef;
  float* dsm = dsm_ptr(X);
  // load the owned row blocks (FP32 high part of the scaled S; padding rows are identity)
  for (int jr = 0; jr < X.cv->nown; ++jr) {
    const int r = X.rank + jr * X.C;
    const int w = kNB * (r + 1), ld = X.ld(r);
    float* Ar = dsm + X.cv->rowoff[jr];
    for (int e0 = tid; e0 < kNB * w; e0 += kThreads * 8) {
      float hv[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = e0 + kThreads * u;
        const int i = e / w, col = e - i * w, row = kNB * r + i;
        hv[u] = (e < kNB * w && row < a.n && col < a.n) ? a.S2[static_cast<int64_t>(row) * a.n + col].x : 0.0f;
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = e0 + kThreads * u;
        if (e >= kNB * w) break;
        const int i = e / w, col = e - i * w, row = kNB * r + i;
        Ar[i * ld + col] = (row < a.n && col < a.n) ? fmaf(alpha * ud[row], ud[col], hv[u] * vd[row] * vd[col])
                                                    : (row == col ? 1.0f : 0.0f);
      }
    }
    for (int i = tid; i < kNB; i += kThreads) {
      const int row = kNB * r + i;
      dsm[X.cv->bl + row] = (row < a.n) ? static_cast<float>(a.b[row]) * vd[row] : 0.0f;
    }
  }
  __syncthreads();
}

__device__ void factor(const Ctx& X, cg::cluster_group& cl, int* flags) {
  const int warp = threadIdx.x >> 5;
  if (X.rank == 0 && warp == 0) diag_step(X, 0, flags);
  if (X.rank == 0) {
    __syncthreads();
    push_diag(X, cl, 0);
  }
  for (int p = 0; p < X.P; ++p) {
    cl_sync();  // Linv_pp and 1/d_p pushed into every CTA
    panel_rows(X, p);
    cl_sync();  // L_rp final for every r > p
    if (p + 1 < X.P) {
      if (X.owns(p + 1)) {
        diag_update(X, p);
        __syncthreads();
        if (warp == 0) diag_step(X, p + 1, flags);
        else update_blocks(X, cl, p, p + 2, X.P - 1, 1, kWarps - 1);
      } else {
        update_blocks(X, cl, p, p + 1, X.P - 1, 0, kWarps);
      }
    }
    if (p + 1 < X.P && X.owns(p + 1)) {
      __syncthreads();  // the diagonal step of p + 1 is done
      push_diag(X, cl, p + 1);
    }
  }
  __syncthreads();
}

__device__ __forceinline__ void dense_cluster_body(DenseArgs a, Ctrl* ctrl, int bid_, int nblk_) {
  // Every CTA reads the control block before the first cluster barrier and
  // this kernel writes it only after the last one: the early return is
  // uniform across the cluster.
  if (skipping(ctrl)) return;
  extern __shared__ __align__(16) float dsm[];
  __shared__ RankTab T;
  __shared__ Carve s_cv;
  cg::cluster_group cl = cg::this_cluster();
  Ctx X;
  X.sm = dsm;
  X.C = static_cast<int>(cl.num_blocks());
  X.rank = static_cast<int>(cl.block_rank());
  X.P = a.P;
  X.n = a.n;
  X.cv = &s_cv;
  X.T = &T;
  const int tid = threadIdx.x;
  if (tid == 0) carve(X.P, X.C, X.rank, &s_cv);
  if (tid < X.C) {
    Carve rc;
    carve(X.P, X.C, tid, &rc);
    for (int j = 0; j < kMaxOwn; ++j) T.rowoff[tid][j] = (j < rc.nown) ? rc.rowoff[j] : 0;
    T.linv[tid] = rc.linv;
    T.rdloc[tid] = rc.rdloc;
    T.y[tid] = rc.y;
    T.x[tid] = rc.x;
    T.accb[tid] = rc.accb;
    T.flags[tid] = rc.flags;
    T.lpp[tid] = rc.lpp;
    T.rdp[tid] = rc.rdp;
    T.ynext[tid] = rc.ynext;
  }
  __syncthreads();
  int* flags = reinterpret_cast<int*>(dsm + s_cv.flags);
  if (tid == 0) flags[0] = 0;
  // Symmetric diagonal (Jacobi) scaling: the factor is of D^-1/2 S D^-1/2,
  // D = diag S, an exact change of variables that removes the conditioning
  // due to the mixed units of rotation and translation rows (measured: the
  // reduced system of a 100-camera loop goes from 4e10 to 1.5e7).
  const int npad = kNB * X.P;
  float* vd = dsm + s_cv.vdef;  // D^-1/2 (1 on padding and non-positive diagonals)
  for (int k = tid; k < npad; k += kThreads) {
    float v = 1.0f;
    if (k < a.n) {
      const float dk = a.S2[static_cast<int64_t>(k) * a.n + k].x;
      if (dk > 0.0f && isfinite(dk)) v = 1.0f / sqrtf(dk);
    }
    vd[k] = v;
    dsm[s_cv.udef + k] = 0.0f;  // no deflation unless the factor breaks down
  }
  __syncthreads();
  load_rows(X, a, 0.0f);
  cl_sync();  // every CTA is running before the first DSMEM access
  factor(X, cl, flags);
  // A negative (or non-finite) pivot of the scaled FP32 factor means the
  // scale-gauge eigenvalue was lost to rounding (tiny problems): refactor the
  // scaled system deflated along u = D^1/2 v, the gauge direction in scaled
  // variables (its solution differs from the exact one essentially only along
  // the gauge, which the gauge projection of the full step sets).
  float alpha = 0.0f;
  {
    int bad = 0;
    for (int jr = 0; jr < s_cv.nown; ++jr)
      for (int t = 0; t < kNB; ++t) {
        const float dv = dsm[s_cv.dloc + kNB * jr + t];
        if (!(dv >= 0.0f)) bad = 1;
      }
    if (tid == 0) flags[1] = bad;
    cl_sync();
    int any = 0;
    for (int c = 0; c < X.C; ++c) any |= reinterpret_cast<const int*>(remote(cl, dsm, c, T.flags[c]))[1];
    cl_sync();  // every CTA has read the flags
    if (any && a.gauge) {
      float* ud = dsm + s_cv.udef;
      float* red = dsm + s_cv.red;
      for (int k = tid; k < npad; k += kThreads) {
        float v = 0.0f;
        if (k < a.npose && k % 6 >= 3) {
          const double* tp = a.poses + 7 * a.fb_pose[k / 6];
          v = static_cast<float>(tp[4 + k % 6 - 3] - a.center[k % 6 - 3]) / vd[k];
        }
        ud[k] = v;
      }
      __syncthreads();
      float s2 = 0.0f;
      for (int k = tid; k < npad; k += kThreads) s2 = fmaf(ud[k], ud[k], s2);
      red[tid] = s2;
      __syncthreads();
      for (int h = kThreads / 2; h > 0; h >>= 1) {
        if (tid < h) red[tid] += red[tid + h];
        __syncthreads();
      }
      const float inv = red[0] > 0.0f ? 1.0f / sqrtf(red[0]) : 0.0f;
      __syncthreads();
      for (int k = tid; k < npad; k += kThreads) ud[k] *= inv;
      alpha = 1.0f;  // the scaled diagonal is 1
      if (tid == 0) flags[0] = 0;
      __syncthreads();
      load_rows(X, a, alpha);
      __syncthreads();
      factor(X, cl, flags);
    }
  }
  // x0 = D^-1/2 (LDL^T)^-1 D^-1/2 b in FP32, then up to a.refine corrections against
  // the float-float S; the solution is kept as float-float (xs, xlo) in every CTA.
  solve_forward(X, cl);
  solve_backward(X, cl);
  cl_sync();
  gather_x(X, cl);
  // max |.| over the whole vector (every CTA holds it after gather_x, so every
  // CTA reaches the same value and the same decision below)
  __shared__ float s_red[kThreads];
  auto block_max = [&](float v) {
    s_red[tid] = v;
    __syncthreads();
    for (int h = kThreads / 2; h > 0; h >>= 1) {
      if (tid < h) s_red[tid] = fmaxf(s_red[tid], s_red[tid + h]);
      __syncthreads();
    }
    const float r = s_red[0];
    __syncthreads();
    return r;
  };
  float dprev;  // max |correction| of the previous solve, scaled variables
  {
    float m = 0.0f;
    for (int k = tid; k < npad; k += kThreads) {
      dsm[s_cv.xs + k] = dsm[s_cv.x + k] * vd[k];
      dsm[s_cv.xlo + k] = 0.0f;
      m = fmaxf(m, fabsf(dsm[s_cv.x + k]));
    }
    dprev = block_max(m);
  }
  for (int it = 0; it < a.refine; ++it) {
    residual(X, a, alpha);
    __syncthreads();
    solve_forward(X, cl);
    solve_backward(X, cl);
    cl_sync();
    gather_x(X, cl);
    float dm = 0.0f, xm = 0.0f;
    for (int k = tid; k < npad; k += kThreads) {
      const dd v = dd_add_f(dd_make(dsm[s_cv.xs + k], dsm[s_cv.xlo + k]), dsm[s_cv.x + k] * vd[k]);
      dsm[s_cv.xs + k] = v.hi;
      dsm[s_cv.xlo + k] = v.lo;
      dm = fmaxf(dm, fabsf(dsm[s_cv.x + k]));
      xm = fmaxf(xm, fabsf(v.hi / vd[k]));
    }
    __syncthreads();
    if (it + 1 < a.refine) {
      // the refinement contracts the error by about dm / dprev per step: when
      // the error it predicts after this step, dm^2 / dprev, is below
      // kRefineSkip of the solution (scaled variables), the next step is skipped
      dm = block_max(dm);
      xm = block_max(xm);
      const bool done = dm * dm <= kRefineSkip * dprev * xm;  // NaN keeps refining
      dprev = dm;
      if (done) break;
    }
  }
  for (int jr = 0; jr < s_cv.nown; ++jr) {
    const int r = X.rank + jr * X.C;
    for (int i = tid; i < kNB; i += kThreads) {
      const int row = kNB * r + i;
      if (row >= a.n) continue;
      const float hi = dsm[s_cv.xs + row], lo = dsm[s_cv.xlo + row];
      a.x[row] = static_cast<double>(hi) + static_cast<double>(lo);
      a.xdd[2 * row] = hi;
      a.xdd[2 * row + 1] = lo;
    }
  }
  if (tid == 0 && flags[0]) ctrl->skip = 2;  // NonFinitePivot -> solve failure -> reject
  cl_sync();  // no CTA leaves while another may still read its shared memory
}
__global__ void __launch_bounds__(kThreads, 1) k_dense_cluster(DenseArgs a, Ctrl* ctrl) {
  dense_cluster_body(a, ctrl, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------------------
// Small reduced systems (n <= kSmallMax: local windows of up to 40 cameras):
// one CTA, the lower triangle of S in float-float in shared memory (packed
// by rows), LDL^T with the PSD-aware pivot rule and the forward substitution
// of b fused into it (one barrier per pivot: every thread evaluates the pivot
// itself; the trailing rows are dealt to the warps, a row's entries to the
// lanes), then the diagonal and the backward sweep.  Float-float resolves
// these systems without refinement (their scale gauge is held only by the
// damping, which an FP32 factor with refinement does not resolve for windows
// of 26-40 cameras); the cluster kernel's fixed costs (cluster barriers, a
// large code footprint that starts cold on each SM) dominate at this size.
// ---------------------------------------------------------------------------
constexpr int kSmallMax = 234;

__device__ __forceinline__ dd sd_f2dd(float2 v) { return dd_make(v.x, v.y); }
__device__ __forceinline__ float2 sd_dd2f(dd v) { return make_float2(v.hi, v.lo); }
// packed lower triangle: entry (i, q), q <= i
__device__ __forceinline__ int sd_at(int i, int q) { return i * (i + 1) / 2 + q; }

// 1/d by Newton's iteration from the hardware approximate reciprocal (one
// FP32 step, one float-float step with an exactly formed residual).
__device__ __forceinline__ dd sd_rcp(dd d) {
  float r0;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(d.hi));
  r0 = __fmaf_rn(r0, __fmaf_rn(-d.hi, r0, 1.0f), r0);
  const dd p = dd_mul_f(d, r0);
  const float e = __fsub_rn(__fsub_rn(1.0f, p.hi), p.lo);
  return dd_fast_two_sum(r0, __fmul_rn(r0, e));
}

__device__ __forceinline__ void small_dense_body(DenseArgs a, Ctrl* ctrl, int bid_, int nblk_) {
  (void)bid_;
  (void)nblk_;
  if (skipping(ctrl)) return;
  extern __shared__ __align__(16) float2 sm[];
  const int m = a.n;
  float2* A = sm;                      // lower triangle, packed by rows
  float2* y = sm + m * (m + 1) / 2;    // rhs -> z -> x
  float2* rdv = y + m;                 // reciprocal pivots
  // equality constraints: columns Y_k = S^-1 G_k^T solved beside the rhs
  // (range-space KKT, schur_ldlt.rs:674-772)
  const int ne = a.n_eq;
  float2* yg = rdv + m;                // ne x m
  __shared__ int s_bad;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_bad = 0;
  for (int i = warp; i < m; i += 8)
    for (int j = lane; j <= i; j += 32) A[sd_at(i, j)] = a.S2[static_cast<int64_t>(i) * m + j];
  for (int i = tid; i < m; i += 256) y[i] = sd_dd2f(dd_from_double(a.b[i]));
  for (int e = tid; e < ne * m; e += 256) yg[e] = make_float2(0.0f, 0.0f);
  __syncthreads();
  if (tid < ne && a.eq_fb[tid] >= 0)
    for (int i = 0; i < 3; ++i) yg[tid * m + 6 * a.eq_fb[tid] + 3 + i] = sd_dd2f(dd_from_double(a.eq_jac[3 * tid + i]));
  __syncthreads();
  float maxp = 1.0f;
  for (int t = 0; t < m; ++t) {
    dd dt = sd_f2dd(A[sd_at(t, t)]);
    if (t % 6 == 0) maxp = 1.0f;  // a new pose block
    const float tol = fmaxf(maxp, 1.0f) * 1e-12f;
    bool bad = false;
    if (!isfinite(dt.hi)) {
      bad = true;
      dt = dd_make(0.0f, 0.0f);
    } else if (fabsf(dt.hi) <= tol) {
      dt = dd_make(0.0f, 0.0f);
    } else {
      maxp = fmaxf(maxp, fabsf(dt.hi));
    }
    const dd rd = (dt.hi == 0.0f) ? dd_make(0.0f, 0.0f) : sd_rcp(dt);
    if (tid == 0) {
      rdv[t] = sd_dd2f(rd);
      if (bad) s_bad = 1;
    }
    const dd yt = sd_f2dd(y[t]);
    // trailing rows i > t: a_iq -= (a_it rd) a_qt for t < q <= i; y_i -= (a_it rd) y_t
    for (int i = t + 1 + warp; i < m; i += 8) {
      const dd li = dd_mul(sd_f2dd(A[sd_at(i, t)]), rd);
      const int ri = sd_at(i, 0);
      for (int q = t + 1 + lane; q <= i; q += 32) {
        const dd v = dd_sub(sd_f2dd(A[ri + q]), dd_mul(li, sd_f2dd(A[sd_at(q, t)])));
        A[ri + q] = sd_dd2f(v);
      }
      if (lane == 0) y[i] = sd_dd2f(dd_sub(sd_f2dd(y[i]), dd_mul(li, yt)));
      if (lane >= 1 && lane <= ne) {
        float2* yk = yg + (lane - 1) * m;
        yk[i] = sd_dd2f(dd_sub(sd_f2dd(yk[i]), dd_mul(li, sd_f2dd(yk[t]))));
      }
    }
    __syncthreads();
  }
  // L columns (a_it rd_t), the diagonal solve
  for (int i = warp; i < m; i += 8)
    for (int t = lane; t < i; t += 32) {
      const int e = sd_at(i, t);
      A[e] = sd_dd2f(dd_mul(sd_f2dd(A[e]), sd_f2dd(rdv[t])));
    }
  for (int i = tid; i < m; i += 256) y[i] = sd_dd2f(dd_mul(sd_f2dd(y[i]), sd_f2dd(rdv[i])));
  for (int e = tid; e < ne * m; e += 256) yg[e] = sd_dd2f(dd_mul(sd_f2dd(yg[e]), sd_f2dd(rdv[e % m])));
  __syncthreads();
  // backward: x_t final, then x_i -= L_ti x_t for i < t (the rhs and every Y column)
  for (int t = m - 1; t > 0; --t) {
    const dd xt = sd_f2dd(y[t]);
    const int rt = sd_at(t, 0);
    for (int e = tid; e < (1 + ne) * t; e += 256) {
      const int col = e / t, i = e - col * t;
      float2* v = col == 0 ? y : yg + (col - 1) * m;
      const dd vt = col == 0 ? xt : sd_f2dd(v[t]);
      v[i] = sd_dd2f(dd_sub(sd_f2dd(v[i]), dd_mul(sd_f2dd(A[rt + i]), vt)));
    }
    __syncthreads();
  }
  if (ne > 0) {
    // M = G Y, w = G x + c, dlam = M^-1 w (Gauss-Jordan with partial pivoting,
    // as the small inverse of schur_ldlt.rs:723-728), x -= Y dlam
    __shared__ double s_dlam[kMaxEq];
    if (tid == 0) {
      double M[kMaxEq * kMaxEq], Mi[kMaxEq * kMaxEq], w[kMaxEq];
      for (int p = 0; p < ne; ++p) {
        const int fp = a.eq_fb[p];
        double acc = a.eq_c[p];
        for (int q = 0; q < ne; ++q) M[p * ne + q] = 0.0;
        if (fp >= 0)
          for (int i = 0; i < 3; ++i) {
            const int row = 6 * fp + 3 + i;
            const double gi = a.eq_jac[3 * p + i];
            acc += gi * dd_to_double(sd_f2dd(y[row]));
            for (int q = 0; q < ne; ++q) M[p * ne + q] += gi * dd_to_double(sd_f2dd(yg[q * m + row]));
          }
        w[p] = acc;
      }
      for (int p = 0; p < ne * ne; ++p) Mi[p] = (p / ne == p % ne) ? 1.0 : 0.0;
      bool ok = true;
      for (int col = 0; col < ne && ok; ++col) {
        int piv = col;
        for (int r = col + 1; r < ne; ++r)
          if (fabs(M[r * ne + col]) > fabs(M[piv * ne + col])) piv = r;
        const double dv = M[piv * ne + col];
        if (!(fabs(dv) > 0.0) || !isfinite(dv)) { ok = false; break; }
        if (piv != col)
          for (int c = 0; c < ne; ++c) {
            double t1 = M[piv * ne + c]; M[piv * ne + c] = M[col * ne + c]; M[col * ne + c] = t1;
            double t2 = Mi[piv * ne + c]; Mi[piv * ne + c] = Mi[col * ne + c]; Mi[col * ne + c] = t2;
          }
        for (int c = 0; c < ne; ++c) { M[col * ne + c] /= dv; Mi[col * ne + c] /= dv; }
        for (int r = 0; r < ne; ++r) {
          if (r == col) continue;
          const double f = M[r * ne + col];
          if (f == 0.0) continue;
          for (int c = 0; c < ne; ++c) { M[r * ne + c] -= f * M[col * ne + c]; Mi[r * ne + c] -= f * Mi[col * ne + c]; }
        }
      }
      if (!ok) s_bad = 1;  // a singular M: a failed solve (reject)
      for (int p = 0; p < ne; ++p) {
        double acc = 0.0;
        for (int q = 0; q < ne; ++q) acc += Mi[p * ne + q] * w[q];
        s_dlam[p] = ok ? acc : 0.0;
        a.eq_dlam[p] = s_dlam[p];
      }
    }
    __syncthreads();
    for (int i = tid; i < m; i += 256) {
      dd v = sd_f2dd(y[i]);
      for (int p = 0; p < ne; ++p) v = dd_sub(v, dd_mul(sd_f2dd(yg[p * m + i]), dd_from_double(s_dlam[p])));
      y[i] = sd_dd2f(v);
    }
    __syncthreads();
  }
  for (int i = tid; i < m; i += 256) {
    const dd v = sd_f2dd(y[i]);
    a.x[i] = dd_to_double(v);
    a.xdd[2 * i] = v.hi;
    a.xdd[2 * i + 1] = v.lo;
  }
  if (tid == 0 && s_bad) ctrl->skip = 2;  // NonFinitePivot -> solve failure -> reject
}
__global__ void __launch_bounds__(256, 1) k_small_dense(DenseArgs a, Ctrl* ctrl) {
  small_dense_body(a, ctrl, blockIdx.x, gridDim.x);
}

size_t small_dense_smem(int n, int n_eq = 0) {
  return sizeof(float2) * (static_cast<size_t>(n) * (n + 1) / 2 + (2 + static_cast<size_t>(n_eq)) * n);
}

size_t dense_smem_bytes(int P, int C) {
  size_t m = 0;
  for (int r = 0; r < C; ++r) {
    Carve c;
    carve(P, C, r, &c);
    if (c.nown > kMaxOwn) return SIZE_MAX;
    const size_t b = sizeof(float) * static_cast<size_t>(c.total);
    if (b > m) m = b;
  }
  return m;
}

}  // namespace

namespace {
int dense_cluster_choose(int P, int* cluster, size_t* smem);
}  // namespace

// The choice depends on the padded order alone; it is made once per
// (device, block count) and remembered (the occupancy query is a driver call
// that every problem created on many host threads would otherwise repeat).
int dense_cluster_setup(int n, int* cluster, size_t* smem) {
  *cluster = 0;
  *smem = 0;
  if (n <= 0) return 0;
  const int P = (n + kNB - 1) / kNB;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  static std::mutex mu;
  static std::map<std::pair<int, int>, std::pair<int, size_t>> chosen;
  {
    std::lock_guard<std::mutex> lk(mu);
    const auto it = chosen.find(std::make_pair(dev, P));
    if (it != chosen.end()) {
      *cluster = it->second.first;
      *smem = it->second.second;
      return *cluster;
    }
  }
  const int C = dense_cluster_choose(P, cluster, smem);
  std::lock_guard<std::mutex> lk(mu);
  chosen[std::make_pair(dev, P)] = std::make_pair(*cluster, *smem);
  return C;
}

namespace {
int dense_cluster_choose(int P, int* cluster, size_t* smem) {
  // one CTA per 24-row block up to 8; beyond, 16 (non-portable) or 8
  int sizes[2] = {16, 8};
  int ncand = 2;
  if (P <= 8) {
    sizes[0] = P;
    ncand = 1;
  }
  for (int ci = 0; ci < ncand; ++ci) {
    const int C = sizes[ci];
    const size_t bytes = dense_smem_bytes(P, C);
    if (bytes > kSmemLimit - sizeof(RankTab) - sizeof(Carve) - 1024) continue;
    if (raise_dynamic_smem(reinterpret_cast<const void*>(k_dense_cluster), bytes) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    if (C > 8 && cudaFuncSetAttribute(k_dense_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                     cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(C);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = bytes;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, k_dense_cluster, &cfg) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    if (nclusters < 1) continue;
    *cluster = C;
    *smem = bytes;
    return C;
  }
  return 0;
}
}  // namespace

int small_dense_setup_eq(int n, int n_eq) {
  if (n <= 0 || n > kSmallMax || n_eq < 0 || n_eq > kMaxEq) return 0;
  if (raise_dynamic_smem(reinterpret_cast<const void*>(k_small_dense), small_dense_smem(n, n_eq)) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return 1;
}

int small_dense_setup(int n) {
  if (n <= 0 || n > kSmallMax) return 0;
  if (raise_dynamic_smem(reinterpret_cast<const void*>(k_small_dense), small_dense_smem(n)) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return 1;
}

namespace {

DenseArgs small_dense_args(const Sizes& s, const Dev& d) {
  DenseArgs a{};
  a.n = s.n6;
  a.P = (s.n6 + kNB - 1) / kNB;
  a.S2 = d.S2;
  a.b = d.rb;
  a.x = d.x;
  a.xdd = d.xdd;
  a.n_eq = s.n_eq;
  a.eq_fb = d.eq_fb;
  a.eq_jac = d.eq_jac;
  a.eq_c = d.eq_c;
  a.eq_dlam = d.eq_dlam;
  return a;
}

DenseArgs dense_cluster_args(const Sizes& s, const Dev& d) {
  DenseArgs a{};
  a.n = s.n6;
  a.P = (s.n6 + kNB - 1) / kNB;
  a.S2 = d.S2;
  a.b = d.rb;
  a.x = d.x;
  a.xdd = d.xdd;
  a.gauge = (s.gauge_kind == 1) ? 1 : 0;
  a.poses = d.poses;
  a.fb_pose = d.fb_pose;
  for (int k = 0; k < 3; ++k) a.center[k] = s.gauge_center[k];
  a.npose = 6 * s.nf;
  // weakly held directions (pose-graph edges against pixel terms) need the
  // refinement to run longer; it stops once converged
  a.refine = (s.n6 <= kRefineSmallN || s.n_edge > 0) ? kRefineSmall : kRefine;
  return a;
}

}  // namespace

int launch_small_dense(const Sizes& s, const Dev& d, cudaStream_t st) {
  k_small_dense<<<1, 256, small_dense_smem(s.n6, s.n_eq), st>>>(small_dense_args(s, d), d.ctrl);
  return 1;
}

int launch_dense_cluster(const Sizes& s, const Dev& d, cudaStream_t st) {
  const DenseArgs a = dense_cluster_args(s, d);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(s.dense_c);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = s.dense_smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = s.dense_c;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k_dense_cluster, a, d.ctrl);
  return 1;
}


// ---------------------------------------------------------------------------
// The dense solver of a batch of windows: the windows on the one-CTA solver
// in one launch (one CTA each), the others in one cluster launch per cluster
// size (one cluster each).  Every window runs the kernel body its own launch
// runs, with its own arguments and control block.
// ---------------------------------------------------------------------------
namespace {

__global__ void __launch_bounds__(256, 1) k_small_dense_w(const DenseArgs* args, Ctrl* const* ctrl,
                                                          const int32_t* win) {
  small_dense_body(args[blockIdx.x], ctrl[win[blockIdx.x]], 0, 1);
}

__global__ void __launch_bounds__(kThreads, 1) k_dense_cluster_w(const DenseArgs* args, Ctrl* const* ctrl,
                                                                 const int32_t* win) {
  const int i = static_cast<int>(blockIdx.x / cg::this_cluster().num_blocks());
  dense_cluster_body(args[i], ctrl[win[i]], 0, 1);
}

struct DenseGroup {
  int cluster = 0;  // 0: one-CTA solver
  int count = 0;
  size_t smem = 0;
  const DenseArgs* args = nullptr;
  const int32_t* win = nullptr;
};

}  // namespace

struct DenseBatch {
  void* dbuf = nullptr;
  Ctrl* const* ctrl = nullptr;
  std::vector<DenseGroup> groups;
};

DenseBatch* dense_batch_create(const std::vector<BatchWin>& wins, Ctrl* const* ctrl_dev, cudaStream_t st,
                               cudaError_t* err) {
  *err = cudaSuccess;
  // groups keyed by cluster size (> 0), or by a shared-memory class of the
  // one-CTA solver (<= 0)
  std::vector<int> sizes;
  std::vector<std::vector<DenseArgs>> args;
  std::vector<std::vector<int32_t>> win;
  std::vector<size_t> smem;
  auto group_of = [&](int c) {
    for (size_t g = 0; g < sizes.size(); ++g)
      if (sizes[g] == c) return static_cast<int>(g);
    sizes.push_back(c);
    args.emplace_back();
    win.emplace_back();
    smem.push_back(0);
    return static_cast<int>(sizes.size()) - 1;
  };
  for (size_t w = 0; w < wins.size(); ++w) {
    const Sizes& s = *wins[w].s;
    const Dev& d = *wins[w].d;
    if (s.small_dense) {
      // by shared memory, so that small windows share an SM: <= 56 KiB,
      // <= 112 KiB, larger (keys 0, -1, -2)
      const size_t b = small_dense_smem(s.n6);
      const int g = group_of(b <= 56 * 1024 ? 0 : (b <= 112 * 1024 ? -1 : -2));
      args[g].push_back(small_dense_args(s, d));
      win[g].push_back(static_cast<int32_t>(w));
      smem[g] = std::max(smem[g], small_dense_smem(s.n6));
    } else if (s.dense_c > 0) {
      const int g = group_of(s.dense_c);
      args[g].push_back(dense_cluster_args(s, d));
      win[g].push_back(static_cast<int32_t>(w));
      smem[g] = std::max(smem[g], s.dense_smem);
    } else {
      *err = cudaErrorInvalidValue;
      return nullptr;
    }
  }
  std::vector<unsigned char> img;
  auto put = [&](const void* p, size_t n) {
    const size_t at = (img.size() + 15) / 16 * 16;
    img.resize(at + n);
    if (n) std::memcpy(img.data() + at, p, n);
    return at;
  };
  std::vector<size_t> a_at(sizes.size()), w_at(sizes.size());
  for (size_t g = 0; g < sizes.size(); ++g) {
    a_at[g] = put(args[g].data(), sizeof(DenseArgs) * args[g].size());
    w_at[g] = put(win[g].data(), sizeof(int32_t) * win[g].size());
  }
  DenseBatch* b = new DenseBatch();
  b->ctrl = ctrl_dev;
  cudaError_t e = cudaMallocAsync(&b->dbuf, img.empty() ? 16 : img.size(), st);
  if (e == cudaSuccess && !img.empty()) e = cudaMemcpyAsync(b->dbuf, img.data(), img.size(), cudaMemcpyHostToDevice, st);
  for (size_t g = 0; e == cudaSuccess && g < sizes.size(); ++g) {
    DenseGroup G;
    G.cluster = sizes[g] > 0 ? sizes[g] : 0;
    G.count = static_cast<int>(args[g].size());
    G.smem = smem[g];
    G.args = reinterpret_cast<const DenseArgs*>(static_cast<unsigned char*>(b->dbuf) + a_at[g]);
    G.win = reinterpret_cast<const int32_t*>(static_cast<unsigned char*>(b->dbuf) + w_at[g]);
    const void* fn = G.cluster ? reinterpret_cast<const void*>(k_dense_cluster_w)
                               : reinterpret_cast<const void*>(k_small_dense_w);
    e = raise_dynamic_smem(fn, G.smem);
    if (e == cudaSuccess && G.cluster > 8)
      e = cudaFuncSetAttribute(k_dense_cluster_w, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    b->groups.push_back(G);
  }
  if (e != cudaSuccess) {
    *err = e;
    dense_batch_destroy(b, st);
    return nullptr;
  }
  return b;
}

void dense_batch_destroy(DenseBatch* b, cudaStream_t st) {
  if (!b) return;
  if (b->dbuf) cudaFreeAsync(b->dbuf, st);
  delete b;
}

int launch_dense_batch(const DenseBatch* b, cudaStream_t st) {
  int n = 0;
  for (const DenseGroup& G : b->groups) {
    if (G.count == 0) continue;
    if (G.cluster == 0) {
      k_small_dense_w<<<G.count, 256, G.smem, st>>>(G.args, b->ctrl, G.win);
    } else {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(static_cast<unsigned>(G.cluster * G.count));
      cfg.blockDim = dim3(kThreads);
      cfg.dynamicSmemBytes = G.smem;
      cfg.stream = st;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = G.cluster;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      cudaLaunchKernelEx(&cfg, k_dense_cluster_w, G.args, b->ctrl, G.win);
    }
    ++n;
  }
  return n;
}

}  // namespace sgba
