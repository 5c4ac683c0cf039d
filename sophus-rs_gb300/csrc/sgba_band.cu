// sgba_band.cu -- factorization and solve of a banded reduced camera system
// with a dense border: the reduced system of sequential and loop-shaped bundle
// adjustment (cameras along a path, each point seen by a run of consecutive
// cameras, loop closures between the last and the first cameras).
//
// Reference: BlockSparseLdlt::factorize_impl / solve_inplace
// (crates/sophus_solver/src/ldlt/block_sparse_ldlt.rs:99-190, 479-747) with
// the PSD-aware pivot rule of dense_ldlt.rs:164-270 (tol_rel = 1e-12, the
// running maximum restarting at every 6x6 pose block).  The reference orders
// the blocks by AMD; here the natural order is kept, which for these systems
// has the fill of a band plus dense border rows.  In exact arithmetic every
// order gives the same solution; only rounding differs.
//
// Structure (n = 6 n_f scalars, split after nband rows):
//     S = [ A  C^T ]   A (nband x nband): row r has columns [r - W + 1, r] only;
//         [ C  E   ]   C, E: the last nbd rows, dense (loop closures).
// The natural-order LDL^T factor keeps A's band (fill stays inside each row's
// envelope) and fills the border rows:
//     A = L_A D_A L_A^T,   L_C = C L_A^-T D_A^-1,   E - L_C D_A L_C^T = L_E D_E L_E^T.
// All arithmetic is float-float (48-bit significand) on the Jacobi-scaled
// system D^-1/2 S D^-1/2: the reduced system of a 1500-camera loop has
// kappa 6e10, 7.5e7 after scaling, beyond FP32 (and far beyond TF32/BF16
// factors with refinement) but well inside float-float.
//
// Kernels (one LM iteration):
//   k_band_scale      D^-1/2 from diag S
//   k_band_load       band of A, border rows C | E and the right-hand side, scaled, float-float
//   k_band_factor     one thread-block cluster: right-looking LDL^T of the band, 24-column panels;
//                     rows dealt round-robin over the CTAs; per panel every CTA factors the 24x24
//                     diagonal block (and the inverse of its unit lower factor) redundantly, solves
//                     its own rows of the panel, then updates its own rows of the trailing band
//   k_band_sweepmat   per panel, the sweep matrices X_p L_p and X_p^T L_b^T (one CTA per panel)
//   k_band_fwd        one CTA per border row and one for the right-hand side: z = L_A^-1 c
//   k_band_corner     E - Z D_A^-1 Z^T (one warp per entry; the right-hand side row gives y_C)
//   k_band_corner_solve  LDL^T of the corner and its solve
//   k_band_tvec       t = D_A^-1 y_A - L_C^T x_C
//   k_band_bwd        x_A = L_A^-T t, unscale, write the step
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "sgba_dd.cuh"
#include "sgba_internal.h"

namespace cg = cooperative_groups;

namespace sgba {

namespace {

constexpr int kBP = 24;          // panel width (4 pose blocks)
constexpr int kBT = 256;         // threads per CTA (sweeps, corner)
constexpr int kCT = 1024;        // threads of the corner solve (one CTA; more warps hide its per-pivot chains)
constexpr int kFT = 320;         // threads per CTA of the factor: one per position of the 24x24 lower triangle (300)
static_assert(kFT - 32 >= 6 * 48, "the factor kernel's threads 32.. cover the rows below a panel of the widest band");
constexpr int kMaxWBlocks = 32;  // widest band of the band part, in pose blocks
constexpr int kMaxBorderBlocks = 24;
constexpr int kMaxBorder = 6 * kMaxBorderBlocks;
// A dissected loop's corner (separator + closure) is factored as a dense band
// (W = its rows).  The factor kernel maps the W - 1 rows below a panel to
// threads 32 .. W + 30 of a CTA, so W <= kFT - 32 (288 rows, 48 pose blocks).
constexpr int kMaxCornerBlocks = 48;
constexpr int kMaxW = 6 * kMaxCornerBlocks;  // widest band the factor kernel takes (the corner's)
constexpr int kMaxOwnRows = (kMaxW - 1 + 7) / 8;  // rows of one CTA in a window (cluster >= 8)
constexpr float kTolRel = 1e-12f;
constexpr size_t kSmemLimit = 227 * 1024;

// the factorization is skipped on termination, on a skipped step and when PCG converged
__device__ __forceinline__ bool skipping(const Ctrl* c) { return c->done != 0 || c->skip != 0 || c->pcg_done != 0; }

__device__ __forceinline__ dd f2dd(float2 v) { return dd_make(v.x, v.y); }
__device__ __forceinline__ float2 dd2f(dd v) { return make_float2(v.hi, v.lo); }

// Accumulator of a float-float dot product: hi carries the running sum through
// an exact TwoSum, every rounding error (of the products and of the sums)
// goes into the float lo.  ~11 FP32 operations per term.
struct Acc {
  float hi, lo;
};
__device__ __forceinline__ Acc acc_init(dd v) { return Acc{v.hi, v.lo}; }
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
__device__ __forceinline__ void acc_add(Acc& a, dd y) {
  const float s = __fadd_rn(a.hi, y.hi);
  const float bb = __fsub_rn(s, a.hi);
  const float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(y.hi, bb));
  a.hi = s;
  a.lo = __fadd_rn(a.lo, __fadd_rn(err, y.lo));
}
__device__ __forceinline__ dd acc_get(const Acc& a) { return dd_fast_two_sum(a.hi, a.lo); }

__device__ __forceinline__ dd dd_from_prod(double v) { return dd_from_double(v); }

// 1/d in float-float by Newton's iteration x <- x + x (1 - d x): the
// hardware approximate reciprocal, one FP32 step (~2^-44 squared error terms
// aside, 24 bits), then one float-float step whose residual 1 - d x is formed
// from an exact product (1 - p.hi is exact: p.hi is within a few ulps of 1).
__device__ __forceinline__ dd dd_rcp(dd d) {
  float r0;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(d.hi));
  r0 = __fmaf_rn(r0, __fmaf_rn(-d.hi, r0, 1.0f), r0);
  const dd p = dd_mul_f(d, r0);
  const float e = __fsub_rn(__fsub_rn(1.0f, p.hi), p.lo);
  return dd_fast_two_sum(r0, __fmul_rn(r0, e));
}

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_but_one() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

struct BandArgs {
  int n;      // order of S
  int nband;  // rows of the band part A (multiple of 6)
  int W;      // band width: row r of A holds columns [r - W + 1, r]
  int npan;   // 24-column panels of A
  int nbd;    // border rows (n - nband)
  int ring;   // row slots per CTA in the factor kernel
  int nbuf;   // panel buffers of the backward sweep (2 or 3)
  int nbuf_f; // panel buffers of the forward sweep (2 where two CTAs per SM keep its many rows in one wave)
  const double* S;  // n x n, both triangles
  const double* b;  // reduced right-hand side
  float* scl;       // n: D^-1/2
  float2* Lb;       // nband x W: scaled A, then L_A below the diagonal
  float2* Xinv;     // npan x 24 x 24: inverse of the unit lower diagonal block of each panel
  float2* Mf;       // npan x 24 x W: X_p L_p (the panel's rows, columns c0 - W + 1 .. c0 - 1), forward sweep
  float2* Mb;       // npan x 24 x W: X_p^T L^T (rows c1 .. c1 + W - 2 below the panel), backward sweep
  float2* dpiv;     // n: pivots
  float2* rdpiv;    // n: 1 / pivot (0 for a zero pivot)
  float2* Pbuf;     // (W - 1) x 24: L D of the current panel, rows below it
  float2* Zc;       // (nbd + 1) x nband: border rows of C and the scaled right-hand side, then L_A^-1 of them
  float2* Zd;       // (nbd + 1) x nband: D_A^-1 Zc
  float2* Cn;       // (nbd + 1) x (nbd + 1): E and the border part of the right-hand side, then the corner
  float2* xw;       // n: t (band part) and x_C (border part)
  double* x;        // n: the step (unscaled)
  float* xdd;       // 2n: the step as float-float pairs
  // Nested dissection of a loop: the rows are permuted (perm[r] is the row
  // of S behind row r of the solved system; null: the identity) so that the
  // band part is two independent segments (the loop's two arcs, the second
  // in reverse order), factored and swept concurrently, and the border holds
  // the separator between them and the loop closure.
  const int32_t* perm;
  int nseg;         // 1 or 2
  int seg_row0[2];  // first row of each segment
  int seg_rows[2];  // rows of each segment (multiples of 6)
  int seg_pan0[2];  // first panel of each segment
  int32_t* zlo;     // (nbd + 1) x nseg: first nonzero column of each Zc row in each segment (segment-relative)
  float2* out_scaled;  // backward sweep: the scaled solution goes here (the corner's solve) instead of x / xdd
};

__device__ __forceinline__ int seg_of_row(const BandArgs& a, int r) { return (a.nseg > 1 && r >= a.seg_row0[1]) ? 1 : 0; }
__device__ __forceinline__ int seg_of_panel(const BandArgs& a, int P) {
  return (a.nseg > 1 && P >= a.seg_pan0[1]) ? 1 : 0;
}
__device__ __forceinline__ int prow(const BandArgs& a, int r) { return a.perm ? a.perm[r] : r; }
// One segment as a band of its own: rows, panels and their tables offset.
__device__ __forceinline__ BandArgs seg_view(const BandArgs& a, int sg) {
  BandArgs b = a;
  b.nband = a.seg_rows[sg];
  b.npan = (b.nband + kBP - 1) / kBP;
  b.Lb = a.Lb + static_cast<int64_t>(a.seg_row0[sg]) * a.W;
  b.Xinv = a.Xinv + static_cast<int64_t>(a.seg_pan0[sg]) * kBP * kBP;
  b.Mf = a.Mf + static_cast<int64_t>(a.seg_pan0[sg]) * kBP * a.W;
  b.Mb = a.Mb + static_cast<int64_t>(a.seg_pan0[sg]) * kBP * a.W;
  b.dpiv = a.dpiv + a.seg_row0[sg];
  b.rdpiv = a.rdpiv + a.seg_row0[sg];
  return b;
}


// ---------------------------------------------------------------- set-up ---

__global__ void __launch_bounds__(256) k_band_scale(BandArgs a, const Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < a.n; r += gridDim.x * blockDim.x) {
    const int pr = prow(a, r);
    const double v = a.S[static_cast<int64_t>(pr) * a.n + pr];
    a.scl[r] = (v > 0.0 && isfinite(v)) ? static_cast<float>(1.0 / sqrt(v)) : 1.0f;
  }
}

__global__ void __launch_bounds__(256) k_band_load(BandArgs a, const Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  const int64_t nb_entries = static_cast<int64_t>(a.nband) * a.W;
  const int64_t nz_entries = static_cast<int64_t>(a.nbd + 1) * a.nband;
  const int64_t nc_entries = static_cast<int64_t>(a.nbd + 1) * (a.nbd + 1);
  const int64_t total = nb_entries + nz_entries + nc_entries;
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (e < nb_entries) {
      const int r = static_cast<int>(e / a.W);
      const int c = r - a.W + 1 + static_cast<int>(e % a.W);
      float2 v = make_float2(0.0f, 0.0f);
      if (c >= a.seg_row0[seg_of_row(a, r)]) {  // inside the row's segment
        const double s = a.S[static_cast<int64_t>(prow(a, r)) * a.n + prow(a, c)];
        v = dd2f(dd_from_prod(s * static_cast<double>(a.scl[r]) * static_cast<double>(a.scl[c])));
      }
      a.Lb[e] = v;
    } else if (e < nb_entries + nz_entries) {
      const int64_t q = e - nb_entries;
      const int i = static_cast<int>(q / a.nband), c = static_cast<int>(q % a.nband);
      double v;
      if (i < a.nbd) {
        const int r = a.nband + i;
        v = a.S[static_cast<int64_t>(prow(a, r)) * a.n + prow(a, c)] * static_cast<double>(a.scl[r]) *
            static_cast<double>(a.scl[c]);
      } else {
        v = a.b[prow(a, c)] * static_cast<double>(a.scl[c]);
      }
      a.Zc[q] = dd2f(dd_from_prod(v));
    } else {
      const int64_t q = e - nb_entries - nz_entries;
      const int i = static_cast<int>(q / (a.nbd + 1)), j = static_cast<int>(q % (a.nbd + 1));
      double v = 0.0;
      if (j < a.nbd) {
        const int cj = a.nband + j;
        if (i < a.nbd) {
          const int r = a.nband + i;
          v = a.S[static_cast<int64_t>(prow(a, r)) * a.n + prow(a, cj)] * static_cast<double>(a.scl[r]) *
              static_cast<double>(a.scl[cj]);
        } else {
          v = a.b[prow(a, cj)] * static_cast<double>(a.scl[cj]);
        }
      }
      a.Cn[q] = dd2f(dd_from_prod(v));
    }
  }
}

// ------------------------------------------------------- band factor -------

struct FactorShared {
  float2 dg[kBP][kBP + 1];   // diagonal block; L below the diagonal after the factor
  float2 xi[kBP][kBP + 1];   // inverse of the unit lower factor
  float2 sd[kBP], srd[kBP];  // pivots and their reciprocals
  float2 cols[kBP][kBP];     // cols[t][i]: column t of the diagonal block once final (before pivot t)
  float2 xs[kBP][kBP];       // xs[t][q]: row t of X once final (q < t)
  float2 arow[kMaxOwnRows][kBP];
  const float2* dsrc[kBP];   // diagonal-block rows: their slots in the owners' shared memory
  const float4* psrc[kMaxW]; // L D rows of the panel in their owners' shared memory
  int rofs[kMaxOwnRows];     // own window rows: offset of column 0 in `rows`
  int pre[kMaxOwnRows + 1];  // update work prefix over the own rows
  int bad;
};

// Rows of the band are dealt round-robin: row r belongs to CTA r mod C and
// lives, while it is within reach of the current panel, in slot
// (r / C) mod ring of that CTA's shared memory (ring a power of two).  Rows
// are prefetched with cp.async two panels ahead (the group issued after panel
// p is waited for at panel p + 2), so the live rows span at most W + 72 and
// ring * C >= W + 72 + C keeps two of them out of one slot.  A row is written
// back to global memory once its own panel is factored.
// Per panel: every CTA gathers the 24x24 diagonal block from the owners
// (DSMEM) and factors it redundantly; each CTA solves its own rows of the
// panel and publishes L D of them; after a cluster barrier every CTA gathers
// the panel's L D (DSMEM) and updates its own rows in place.
template <int C>
__global__ void __launch_bounds__(kFT, 1) k_band_factor(BandArgs a0, Ctrl* ctrl) {
  // Every CTA reads the control block before the first cluster barrier and
  // only CTA 0 writes it, after the last one: the early return is uniform.
  if (skipping(ctrl)) return;
  // cluster k factors segment k (the two arcs of a dissected loop run
  // concurrently, each as a band of its own)
  const BandArgs a = seg_view(a0, static_cast<int>(blockIdx.x) / C);
  __shared__ FactorShared sh;
  extern __shared__ __align__(16) float2 dyn[];
  cg::cluster_group cl = cg::this_cluster();
  const int rank = static_cast<int>(cl.block_rank());
  const int tid = threadIdx.x;
  const int W = a.W, rmask = a.ring - 1;
  float2* rows = dyn;                  // ring x W
  float2* pld = rows + a.ring * W;     // ring x kBP: L D of the own rows of the current panel
  float2* pb = pld + a.ring * kBP;     // (W - 1) x (kBP + 1): L D of the panel, all rows below it
  auto slot = [&](int r) { return (r / C) & rmask; };
  // element (r, c) of an own row r: rows[rbase(r) + c]
  auto rbase = [&](int r) { return slot(r) * W + (W - 1 - r); };
  int loaded = 0;  // own rows below this index are resident (or in flight)
  auto prefetch = [&](int hi) {
    hi = min(hi, a.nband);
    if (hi > loaded) {
      const int r0 = loaded + ((rank - loaded % C) + C) % C;
      const int nr = (r0 < hi) ? (hi - r0 + C - 1) / C : 0;
      for (int e = tid; e < nr * W; e += kFT) {
        const int r = r0 + (e / W) * C, k = e % W;
        cp_async8(rows + slot(r) * W + k, a.Lb + static_cast<int64_t>(r) * W + k);
      }
      loaded = hi;
    }
    cp_async_commit();
  };
  if (tid == 0) sh.bad = 0;
  // the position (i, q), q <= i, of the 24x24 diagonal block this thread
  // owns through the factor: thread e < 300 takes entry e of the lower
  // triangle (row-major); fi = kBP: no position
  int fi = kBP, fq = 0;
  if (tid < kBP * (kBP + 1) / 2) {
    int i = 0;
    while ((i + 1) * (i + 2) / 2 <= tid) ++i;
    fi = i;
    fq = tid - i * (i + 1) / 2;
  }
  prefetch(W + 3 * kBP);
  for (int p = 0; p < a.npan; ++p) {
    const int c0 = kBP * p;
    const int w = min(kBP, a.nband - c0);
    const int c1 = c0 + w;
    const int rend = min(c1 + W - 1, a.nband);
    const int rfirst = c1 + ((rank - c1 % C) + C) % C;
    const int nown = (rfirst < rend) ? (rend - rfirst + C - 1) / C : 0;
    // rows < c0 + W + 46 are needed now; the group issued two panels ago
    // covered rows < c0 + W + 48, the newest one may stay in flight
    if (p == 0) cp_async_wait_all();
    else cp_async_wait_but_one();
    __syncthreads();  // the previous panel's readers of the tables below are done
    if (tid < w) {
      const int r = c0 + tid;
      sh.dsrc[tid] = cl.map_shared_rank(rows + slot(r) * W, r % C);  // slot base; column c at c - r + W - 1
    }
    if (tid >= 32 && tid - 32 < rend - c1) {
      const int r = c1 + tid - 32;
      sh.psrc[tid - 32] = reinterpret_cast<const float4*>(cl.map_shared_rank(pld + slot(r) * kBP, r % C));
    }
    if (tid == 64) {
      int acc = 0;
      for (int ri = 0; ri < nown; ++ri) {
        const int r = rfirst + ri * C;
        sh.pre[ri] = acc;
        sh.rofs[ri] = rbase(r);
        acc += r - max(c1, r - W + 1) + 1;
      }
      sh.pre[nown] = acc;
    }
    __syncthreads();
    cl.sync();  // the previous panel's update of rows >= c0 is complete in every CTA
    // (1) diagonal block from its owners, identity for its inverse
    for (int e = tid; e < kBP * kBP; e += kFT) {
      const int i = e / kBP, k = e % kBP;
      float2 v = make_float2(0.0f, 0.0f);
      if (i < w && k <= i && (k - i + W - 1) >= 0) v = sh.dsrc[i][k - i + W - 1];
      sh.dg[i][k] = v;
      sh.xi[i][k] = make_float2(i == k ? 1.0f : 0.0f, 0.0f);
    }
    __syncthreads();
    // (2) LDL^T of the diagonal block, X <- L^-1 alongside (the elementary
    // column eliminations applied to the identity).  Each thread keeps the
    // entry of its position in registers: a_iq while q > t (the trailing
    // update a_iq -= l_it a_qt, l_it = a_it / d_t), then X_iq (X_iq -= l_it
    // X_tq, q <= t), so every pivot is one update per thread.  An entry goes to
    // shared memory once, when it becomes final: column t + 1 of A into
    // cols[t + 1], row t + 1 of X into xs[t + 1]; pivot t reads only those.
    // Every thread evaluates the pivot itself (same inputs, same operations:
    // the same value in every thread), so each pivot costs one barrier; the
    // update is branch-free (both operands loaded, one selected).
    {
      dd areg = dd_make(0.0f, 0.0f), xreg = dd_make(0.0f, 0.0f);
      const int ic = fi < kBP ? fi : 0;
      if (fi < w) {
        areg = f2dd(sh.dg[fi][fq]);
        if (fq == 0) sh.cols[0][fi] = sh.dg[fi][0];
      }
      __syncthreads();
      float maxp = 1.0f;  // running maximum pivot of the 6x6 pose block (>= 1)
      for (int t = 0; t < w; ++t) {
        dd dt = f2dd(sh.cols[t][t]);
        if ((c0 + t) % 6 == 0) maxp = 1.0f;
        // the pivot rule: a pivot that is not finite, or not above 1e-12 of
        // the running maximum (at least 1), is zero; branch-free
        const float ad = fabsf(dt.hi);
        const bool fin = ad <= 3.402823466e38f;
        const bool zero = !fin || !(ad > maxp * kTolRel);
        if (!fin && tid == 0) sh.bad = 1;
        maxp = zero ? maxp : fmaxf(maxp, ad);
        const dd r = dd_rcp(dt);
        dt = zero ? dd_make(0.0f, 0.0f) : dt;
        const dd rd = zero ? dd_make(0.0f, 0.0f) : r;
        if (tid == 0) {
          sh.sd[t] = dd2f(dt);
          sh.srd[t] = dd2f(rd);
        }
        const bool act = (fi > t) && (fi < w);
        const bool isA = fq > t;
        const float2 va = sh.cols[t][ic];
        const float2 ca = sh.cols[t][fq];
        const float2 cx = (fq == t) ? make_float2(1.0f, 0.0f) : sh.xs[t][fq];
        const dd li = dd_mul(f2dd(va), rd);
        Acc acc = acc_init(isA ? areg : xreg);
        acc_madd(acc, dd_neg(li), f2dd(isA ? ca : cx));
        const dd nv = acc_get(acc);
        if (act && isA) areg = nv;
        if (act && !isA) xreg = nv;
        if (act && isA && fq == t + 1) sh.cols[t + 1][fi] = dd2f(nv);
        if (act && !isA && fi == t + 1) sh.xs[t + 1][fq] = dd2f(nv);
        __syncthreads();
      }
      // the block's outputs: below the diagonal u = a_iq as of pivot q - 1
      // (L = u / d on output) and X; the diagonal of xi keeps the identity
      if (fi < w && fq < fi) {
        sh.dg[fi][fq] = dd2f(areg);
        sh.xi[fi][fq] = dd2f(xreg);
      }
      __syncthreads();
    }
    // (3) outputs: X and pivots (spread over the CTAs); the own rows of this
    // panel are final: write them back
    for (int e = rank * kFT + tid; e < kBP * kBP; e += C * kFT)
      a.Xinv[static_cast<int64_t>(p) * kBP * kBP + e] = sh.xi[e / kBP][e % kBP];
    if (rank == C - 1 && tid < w) {
      a.dpiv[c0 + tid] = sh.sd[tid];
      a.rdpiv[c0 + tid] = sh.srd[tid];
    }
    {
      const int d0 = c0 + ((rank - c0 % C) + C) % C;
      const int nd = (d0 < c1) ? (c1 - d0 + C - 1) / C : 0;
      for (int e = tid; e < nd * W; e += kFT) {
        const int r = d0 + (e / W) * C, k = e % W;
        const int c = r - W + 1 + k;
        float2 v = make_float2(0.0f, 0.0f);
        if (c >= 0 && c < c0) {
          v = rows[slot(r) * W + k];
        } else if (c >= c0 && c < r) {
          v = dd2f(dd_mul(f2dd(sh.dg[r - c0][c - c0]), f2dd(sh.srd[c - c0])));
        } else if (c == r) {
          v = make_float2(1.0f, 0.0f);
        }
        a.Lb[static_cast<int64_t>(r) * W + k] = v;
      }
    }
    // (4) own rows of the panel: L_rk = (sum_{j<=k} a_rj X_kj) / d_k
    for (int e = tid; e < nown * kBP; e += kFT) {
      const int ri = e / kBP, j = e % kBP;
      const int r = rfirst + ri * C;
      float2 v = make_float2(0.0f, 0.0f);
      if (j < w && c0 + j >= r - W + 1) v = rows[sh.rofs[ri] + c0 + j];
      sh.arow[ri][j] = v;
    }
    __syncthreads();
    for (int e = tid; e < nown * kBP; e += kFT) {
      const int ri = e / kBP, k = e % kBP;
      const int r = rfirst + ri * C;
      dd l = dd_make(0.0f, 0.0f);
      if (k < w) {
        Acc acc = acc_init(dd_make(0.0f, 0.0f));
        for (int j = 0; j <= k; ++j) acc_madd(acc, f2dd(sh.arow[ri][j]), f2dd(sh.xi[k][j]));
        l = dd_mul(acc_get(acc), f2dd(sh.srd[k]));
        if (c0 + k >= r - W + 1) rows[sh.rofs[ri] + c0 + k] = dd2f(l);
      }
      pld[slot(r) * kBP + k] = dd2f(k < w ? dd_mul(l, f2dd(sh.sd[k])) : l);
    }
    cl.sync();  // L D of every row of the panel is published
    // (5) the panel's L D, all rows below it, from their owners: 16-byte
    // loads (a row is 12 float4), eight in flight per thread
    const int nrows = rend - c1;
    {
      constexpr int kQ = kBP / 2;
      const int nq = nrows * kQ;
      for (int e0 = tid; e0 < nq; e0 += 8 * kFT) {
        float4 v4[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int e = e0 + u * kFT;
          if (e < nq) v4[u] = sh.psrc[e / kQ][e % kQ];
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int e = e0 + u * kFT;
          if (e < nq) {
            const int q = e / kQ, k2 = e % kQ;
            pb[q * (kBP + 1) + 2 * k2] = make_float2(v4[u].x, v4[u].y);
            pb[q * (kBP + 1) + 2 * k2 + 1] = make_float2(v4[u].z, v4[u].w);
          }
        }
      }
    }
    __syncthreads();
    // (6) trailing update of the own rows: a_rc -= sum_k L_rk d_k L_ck, c in [max(c1, r-W+1), r]
    const int total = sh.pre[nown];
    int ri = 0;  // e only grows: the row search carries over
    for (int e = tid; e < total; e += kFT) {
      while (ri + 1 < nown && sh.pre[ri + 1] <= e) ++ri;
      const int r = rfirst + ri * C;
      const int c = max(c1, r - W + 1) + (e - sh.pre[ri]);
      float2* rowr = rows + sh.rofs[ri];
      Acc acc0 = acc_init(f2dd(rowr[c]));
      Acc acc1 = acc_init(dd_make(0.0f, 0.0f));
      const float2* pr = pb + (c - c1) * (kBP + 1);
      const int k0 = max(0, r - W + 1 - c0);  // L_rk is zero left of the band
      int k = k0;
      for (; k + 1 < w; k += 2) {
        acc_madd(acc0, dd_neg(f2dd(rowr[c0 + k])), f2dd(pr[k]));
        acc_madd(acc1, dd_neg(f2dd(rowr[c0 + k + 1])), f2dd(pr[k + 1]));
      }
      if (k < w) acc_madd(acc0, dd_neg(f2dd(rowr[c0 + k])), f2dd(pr[k]));
      acc_add(acc0, acc_get(acc1));
      rowr[c] = dd2f(acc_get(acc0));
    }
    // (7) rows that the panel after next reaches
    prefetch(c0 + W + 4 * kBP);
  }
  cp_async_wait_all();
  cl.sync();  // no CTA leaves while another may still read its shared memory
  if (rank == 0 && tid == 0 && sh.bad) ctrl->skip = 2;  // NonFinitePivot -> solve failure -> reject
}

// ------------------------------------------------ forward substitution ----

// Shared memory of the sweeps: the vector (nband), then nbuf buffers of the
// panel's M (kBP x W), nbuf of its X (kBP x kBP) and nbuf of its 24 input
// values.  The entries of the next nbuf - 1 panels are copied with cp.async
// while a panel is computed (three buffers where they fit, else two).
__host__ __device__ inline size_t sweep_smem_floats2(int nband, int W, int nbuf) {
  return static_cast<size_t>(nband) + 1 + static_cast<size_t>(nbuf) * (static_cast<size_t>(kBP) * W + kBP * kBP + kBP);
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}

// Sum of a float-float value over the kSweepG consecutive lanes of a group
// (butterfly over the group; every lane of the warp takes part).  Lane g = 0
// of the group holds the total; the order is fixed.
constexpr int kSweepG = 8;  // threads per row of a panel in the sweeps (24 rows: 192 threads)
__device__ __forceinline__ dd group_sum(dd s) {
#pragma unroll
  for (int o = kSweepG / 2; o >= 1; o >>= 1) {
    const float h = __shfl_xor_sync(0xffffffffu, s.hi, o);
    const float l = __shfl_xor_sync(0xffffffffu, s.lo, o);
    Acc acc = acc_init(s);
    acc_add(acc, dd_make(h, l));
    s = acc_get(acc);
  }
  return s;
}

// The sweep matrices of every panel (one CTA per panel, after the factor):
//   forward:  z_p = X_p (c_p - L_p z_prev) = X_p c_p - Mf_p z_prev,  Mf_p = X_p L_p
//             (L_p the panel's rows over the W - 1 columns before it);
//   backward: x_p = X_p^T (t_p - L_b^T x_below) = X_p^T t_p - Mb_p x_below,
//             Mb_p = X_p^T L_b^T (L_b the W - 1 rows below the panel over its columns).
// Each sweep step is then one dot product per row of the panel.
__global__ void __launch_bounds__(kBT) k_band_sweepmat(BandArgs a0, const Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  extern __shared__ __align__(16) float2 smx[];
  const int sg = seg_of_panel(a0, static_cast<int>(blockIdx.x));
  const BandArgs a = seg_view(a0, sg);
  const int W = a.W, span = W - 1;
  const int p = static_cast<int>(blockIdx.x) - a0.seg_pan0[sg];
  const int c0 = kBP * p, w = min(kBP, a.nband - c0), c1 = c0 + w;
  const int tid = threadIdx.x;
  float2* Lp = smx;             // kBP x W: the panel's rows, slots as in Lb
  float2* Lq = Lp + kBP * W;    // span x kBP: the rows below, the panel's columns
  float2* X = Lq + span * kBP;  // kBP x kBP
  for (int e = tid; e < kBP * W; e += kBT) {
    const int i = e / W, sl = e % W;
    Lp[e] = (i < w) ? a.Lb[static_cast<int64_t>(c0 + i) * W + sl] : make_float2(0.0f, 0.0f);
  }
  for (int e = tid; e < span * kBP; e += kBT) {
    const int q = e / kBP, k = e % kBP;
    const int r = c1 + q, sl = c0 + k - r + W - 1;
    Lq[e] = (r < a.nband && k < w && sl >= 0) ? a.Lb[static_cast<int64_t>(r) * W + sl] : make_float2(0.0f, 0.0f);
  }
  for (int e = tid; e < kBP * kBP; e += kBT) X[e] = a.Xinv[static_cast<int64_t>(p) * kBP * kBP + e];
  __syncthreads();
  float2* mf = a.Mf + static_cast<int64_t>(p) * kBP * W;
  float2* mb = a.Mb + static_cast<int64_t>(p) * kBP * W;
  for (int e = tid; e < 2 * kBP * W; e += kBT) {
    const int half = e / (kBP * W), e1 = e % (kBP * W);
    const int k = e1 / W, s2 = e1 % W;
    Acc acc = acc_init(dd_make(0.0f, 0.0f));
    if (half == 0) {
      // Mf[k][s] = sum_{k' <= min(k, s)} X[k][k'] L[c0 + k'][col], col = c0 - W + 1 + s (slot s - k')
      if (k < w && s2 < span)
        for (int kk = 0; kk <= k && kk <= s2; ++kk) acc_madd(acc, f2dd(X[k * kBP + kk]), f2dd(Lp[kk * W + s2 - kk]));
      mf[e1] = dd2f(acc_get(acc));
    } else {
      // Mb[k][q] = sum_{i = k}^{w - 1} X[i][k] L[c1 + q][c0 + i]
      if (k < w && s2 < span)
        for (int i = k; i < w; ++i) acc_madd(acc, f2dd(X[i * kBP + k]), f2dd(Lq[s2 * kBP + i]));
      mb[e1] = dd2f(acc_get(acc));
    }
  }
}

// One CTA per row of Zc (border rows of C and the right-hand side):
// z = L_A^-1 c, then Zd = D_A^-1 z.  Per panel, one dot per row: for row k of
// the panel z_k = sum_{k' <= k} X_kk' c_k' - sum_s Mf_ks z_(c0 - W + 1 + s),
// a group of kSweepG threads per row (warps 0..5).  The panel's inputs c come
// from the unchanged Zc row (staged with the panel), so the outputs can go
// straight into the vector; one barrier per panel.
__global__ void __launch_bounds__(kBT) k_band_fwd(BandArgs a0, const Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  extern __shared__ __align__(16) float2 sw[];
  // CTA (row, segment): the row's part in one segment of the band
  const int sg = static_cast<int>(blockIdx.x) % a0.nseg;
  const int row = static_cast<int>(blockIdx.x) / a0.nseg;
  const BandArgs a = seg_view(a0, sg);
  const int W = a.W;
  const int nb = a.nbuf_f;
  float2* v = sw;
  float2* mbuf = v + ((a.nband + 1) & ~1);  // nb x kBP x W (16-byte aligned: W is even)
  float2* xb = mbuf + nb * kBP * W;         // nb x kBP x kBP
  float2* cb = xb + nb * kBP * kBP;         // nb x kBP
  const int tid = threadIdx.x;
  float2* zrow = a0.Zc + static_cast<int64_t>(row) * a0.nband + a0.seg_row0[sg];
  const int h = W / 2;
  const int i0 = tid / h, q0 = tid % h, di = kBT / h, dq = kBT % h;
  auto stage = [&](int p) {
    const int c0 = kBP * p, w = min(kBP, a.nband - c0), buf = p % nb;
    const float2* src = a.Mf + static_cast<int64_t>(p) * kBP * W;
    int i = i0, q = q0;
    while (i < w) {  // the thread's 16-byte pieces, advancing by kBT without a division
      cp_async16(mbuf + (buf * kBP + i) * W + 2 * q, src + i * W + 2 * q);
      q += dq;
      i += di;
      if (q >= h) {
        q -= h;
        ++i;
      }
    }
    for (int e = tid; e < kBP * kBP / 2; e += kBT)
      cp_async16(xb + buf * kBP * kBP + 2 * e, a.Xinv + static_cast<int64_t>(p) * kBP * kBP + 2 * e);
    if (tid < w / 2) cp_async16(cb + buf * kBP + 2 * tid, zrow + c0 + 2 * tid);
    cp_async_commit();
  };
  // the row's first nonzero in the segment: the panels before it stay zero
  __shared__ int s_first;
  if (tid == 0) s_first = a.nband;
  __syncthreads();
  int myfirst = a.nband;
  for (int c = tid; c < a.nband; c += kBT) {
    const float2 z = zrow[c];
    v[c] = z;
    if ((z.x != 0.0f || z.y != 0.0f) && c < myfirst) myfirst = c;
  }
  atomicMin(&s_first, myfirst);
  __syncthreads();
  const int pstart = s_first / kBP;
  if (tid == 0 && a0.zlo) a0.zlo[row * a0.nseg + sg] = s_first;
  for (int s0 = 0; s0 < nb - 1; ++s0) {
    if (pstart + s0 < a.npan) stage(pstart + s0);
    else cp_async_commit();
  }
  const int k = tid / kSweepG, g = tid % kSweepG;
  for (int p = pstart; p < a.npan; ++p) {
    const int c0 = kBP * p;
    const int w = min(kBP, a.nband - c0);
    const int buf = p % nb;
    if (nb == 3) cp_async_wait_but_one();
    else cp_async_wait_all();
    __syncthreads();  // panel p landed; every thread is done with panel p - 1
    if (p + nb - 1 < a.npan) stage(p + nb - 1);
    else cp_async_commit();
    if (tid < kBP * kSweepG) {
      Acc a0 = acc_init(dd_make(0.0f, 0.0f)), a1 = a0, a2 = a0, a3 = a0;
      if (k < w) {
        const float2* xr = xb + buf * kBP * kBP + k * kBP;
        const float2* cp = cb + buf * kBP;
        for (int kk = g; kk <= k; kk += kSweepG) acc_madd(a0, f2dd(xr[kk]), f2dd(cp[kk]));
        const float2* mrow = mbuf + (buf * kBP + k) * W;
        const int vb = c0 - W + 1;  // column of slot 0
        int s2 = max(0, -vb) + g;
        for (; s2 + 3 * kSweepG < W - 1; s2 += 4 * kSweepG) {
          const float2 m0 = mrow[s2], m1 = mrow[s2 + kSweepG], m2 = mrow[s2 + 2 * kSweepG], m3 = mrow[s2 + 3 * kSweepG];
          const float2 v0 = v[vb + s2], v1 = v[vb + s2 + kSweepG], v2 = v[vb + s2 + 2 * kSweepG],
                       v3 = v[vb + s2 + 3 * kSweepG];
          acc_madd(a1, dd_neg(f2dd(m0)), f2dd(v0));
          acc_madd(a2, dd_neg(f2dd(m1)), f2dd(v1));
          acc_madd(a3, dd_neg(f2dd(m2)), f2dd(v2));
          acc_madd(a0, dd_neg(f2dd(m3)), f2dd(v3));
        }
        for (; s2 < W - 1; s2 += kSweepG) acc_madd(a1, dd_neg(f2dd(mrow[s2])), f2dd(v[vb + s2]));
      }
      acc_add(a0, acc_get(a1));
      acc_add(a2, acc_get(a3));
      acc_add(a0, acc_get(a2));
      const dd sm = group_sum(acc_get(a0));
      if (g == 0 && k < w) v[c0 + k] = dd2f(sm);
    }
  }
  cp_async_wait_all();
  __syncthreads();
  float2* drow = a0.Zd + static_cast<int64_t>(row) * a0.nband + a0.seg_row0[sg];
  for (int c = tid; c < a.nband; c += kBT) {
    zrow[c] = v[c];
    drow[c] = dd2f(dd_mul(f2dd(v[c]), f2dd(a.rdpiv[c])));
  }
}

// ----------------------------------------------------------- corner -------

// Lower entries (i, j), j <= i <= nbd, of the corner:
// Cn_ij -= sum_c Zd_ic Zc_jc.  Row nbd (the right-hand side) becomes y_C.
// One 128-thread CTA per 4x4 tile of entries; warp w takes row i = 4 ti + w
// against the tile's four j (the Zc rows are shared through L1).
constexpr int kCornerTile = 4;
__global__ void __launch_bounds__(128) k_band_corner(BandArgs a, const Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int64_t m = a.nbd + 1;
  const int64_t nt = (m + kCornerTile - 1) / kCornerTile;
  const int64_t ntiles = nt * (nt + 1) / 2;
  __shared__ float2 red[kCornerTile][kCornerTile][32];
  for (int64_t q = blockIdx.x; q < ntiles; q += gridDim.x) {
    int ti = static_cast<int>((sqrt(8.0 * static_cast<double>(q) + 1.0) - 1.0) * 0.5);
    while (static_cast<int64_t>(ti) * (ti + 1) / 2 > q) --ti;
    while (static_cast<int64_t>(ti + 1) * (ti + 2) / 2 <= q) ++ti;
    const int tj = static_cast<int>(q - static_cast<int64_t>(ti) * (ti + 1) / 2);
    const int i = kCornerTile * ti + wib;
    Acc acc[kCornerTile];
#pragma unroll
    for (int jj = 0; jj < kCornerTile; ++jj) acc[jj] = acc_init(dd_make(0.0f, 0.0f));
    if (i < m) {
      const float2* zi = a.Zd + static_cast<int64_t>(i) * a.nband;
      const float2* zj = a.Zc + static_cast<int64_t>(kCornerTile * tj) * a.nband;
      for (int sg = 0; sg < a.nseg; ++sg) {
        // the rows are zero before their first nonzero in the segment: the
        // tile's products start at the later of its rows' and columns' first
        int lo = 0;
        if (a.zlo) {
          int li = a.seg_rows[sg], lj = a.seg_rows[sg];
          for (int t = 0; t < kCornerTile; ++t) {
            const int ri = kCornerTile * ti + t, rj = kCornerTile * tj + t;
            if (ri < m) li = min(li, a.zlo[ri * a.nseg + sg]);
            if (rj < m) lj = min(lj, a.zlo[rj * a.nseg + sg]);
          }
          lo = max(li, lj);
        }
        const int cend = a.seg_row0[sg] + a.seg_rows[sg];
        for (int c = a.seg_row0[sg] + lo + lane; c < cend; c += 32) {
          const dd x = f2dd(zi[c]);
#pragma unroll
          for (int jj = 0; jj < kCornerTile; ++jj)
            if (kCornerTile * tj + jj < m) acc_madd(acc[jj], x, f2dd(zj[static_cast<int64_t>(jj) * a.nband + c]));
        }
      }
    }
#pragma unroll
    for (int jj = 0; jj < kCornerTile; ++jj) red[wib][jj][lane] = dd2f(acc_get(acc[jj]));
    __syncwarp();
    if (lane < kCornerTile) {
      const int j = kCornerTile * tj + lane;
      if (i < m && j <= i) {
        Acc t = acc_init(f2dd(a.Cn[static_cast<int64_t>(i) * m + j]));
        for (int l = 0; l < 32; ++l) acc_add(t, dd_neg(f2dd(red[wib][lane][l])));
        a.Cn[static_cast<int64_t>(i) * m + j] = dd2f(acc_get(t));
      }
    }
    __syncwarp();
  }
}

// One CTA: LDL^T of the corner (PSD-aware pivots) with the forward
// substitution of y_C fused into it, then the diagonal and the backward sweep.
// Every thread evaluates each pivot itself (same inputs, same operations), so
// a pivot costs one barrier; column t is scaled to L after the factorization
// (later pivots do not touch it).
__global__ void __launch_bounds__(kCT) k_band_corner_solve(BandArgs a, Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  extern __shared__ __align__(16) float2 cm[];  // nbd x nbd (lower), then y (nbd), then 1/d (nbd)
  __shared__ int sbad;
  const int m = a.nbd;
  const int tid = threadIdx.x;
  if (m == 0) return;
  float2* y = cm + m * m;
  float2* rdv = y + m;
  const int64_t ld = m + 1;
  for (int e = tid; e < m * m; e += kCT) {
    const int i = e / m, j = e % m;
    cm[e] = (j <= i) ? a.Cn[i * ld + j] : make_float2(0.0f, 0.0f);
  }
  for (int j = tid; j < m; j += kCT) y[j] = a.Cn[static_cast<int64_t>(m) * ld + j];
  if (tid == 0) sbad = 0;
  __syncthreads();
  float maxp = 1.0f;
  for (int t = 0; t < m; ++t) {
    dd dt = f2dd(cm[t * m + t]);
    if ((a.nband + t) % 6 == 0) maxp = 1.0f;
    const float tol = fmaxf(maxp, 1.0f) * kTolRel;
    bool bad = false;
    if (!isfinite(dt.hi)) {
      bad = true;
      dt = dd_make(0.0f, 0.0f);
    } else if (fabsf(dt.hi) <= tol) {
      dt = dd_make(0.0f, 0.0f);
    } else {
      maxp = fmaxf(maxp, fabsf(dt.hi));
    }
    const dd rd = (dt.hi == 0.0f) ? dd_make(0.0f, 0.0f) : dd_rcp(dt);
    if (tid == 0) {
      a.dpiv[a.nband + t] = dd2f(dt);
      a.rdpiv[a.nband + t] = dd2f(rd);
      rdv[t] = dd2f(rd);
      if (bad) sbad = 1;
    }
    const int rem = m - t - 1;
    const int ntri = rem * (rem + 1) / 2;
    const dd yt = f2dd(y[t]);
    for (int e = tid; e < ntri + rem; e += kCT) {
      if (e < ntri) {  // trailing (i, k), t < k <= i: a_ik -= a_it rd a_kt
        int ii = static_cast<int>((__fsqrt_rn(8.0f * static_cast<float>(e) + 1.0f) - 1.0f) * 0.5f);
        while (ii * (ii + 1) / 2 > e) --ii;
        while ((ii + 1) * (ii + 2) / 2 <= e) ++ii;
        const int i = t + 1 + ii, k = t + 1 + (e - ii * (ii + 1) / 2);
        const dd li = dd_mul(f2dd(cm[i * m + t]), rd);
        Acc acc = acc_init(f2dd(cm[i * m + k]));
        acc_madd(acc, dd_neg(li), f2dd(cm[k * m + t]));
        cm[i * m + k] = dd2f(acc_get(acc));
      } else {         // forward substitution: y_i -= l_it y_t
        const int i = t + 1 + (e - ntri);
        const dd li = dd_mul(f2dd(cm[i * m + t]), rd);
        Acc acc = acc_init(f2dd(y[i]));
        acc_madd(acc, dd_neg(li), yt);
        y[i] = dd2f(acc_get(acc));
      }
    }
    __syncthreads();
  }
  for (int e = tid; e < m * m; e += kCT) {
    const int i = e / m, t = e % m;
    if (t < i) cm[e] = dd2f(dd_mul(f2dd(cm[e]), f2dd(rdv[t])));
  }
  for (int i = tid; i < m; i += kCT) y[i] = dd2f(dd_mul(f2dd(y[i]), f2dd(rdv[i])));
  __syncthreads();
  for (int t = m - 1; t > 0; --t) {  // x_t final: x_i -= L_ti x_t for i < t
    const dd xt = f2dd(y[t]);
    for (int i = tid; i < t; i += kCT) {
      Acc acc = acc_init(f2dd(y[i]));
      acc_madd(acc, dd_neg(f2dd(cm[t * m + i])), xt);
      y[i] = dd2f(acc_get(acc));
    }
    __syncthreads();
  }
  for (int i = tid; i < m; i += kCT) a.xw[a.nband + i] = y[i];
  if (tid == 0 && sbad) ctrl->skip = 2;
}

// The corner of a dissected loop as a dense band of its own (W = m): its
// lower rows from Cn, and its right-hand side row (y_C) for the sweeps.
__global__ void __launch_bounds__(256) k_band_corner_load(BandArgs ac, const float2* __restrict__ cn,
                                                          const Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  const int m = ac.nband, ld = m + 1;
  const int64_t total = static_cast<int64_t>(m) * m + m;
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (e < static_cast<int64_t>(m) * m) {
      const int r = static_cast<int>(e / m), c = r - m + 1 + static_cast<int>(e % m);
      ac.Lb[e] = (c >= 0) ? cn[static_cast<int64_t>(r) * ld + c] : make_float2(0.0f, 0.0f);
    } else {
      const int j = static_cast<int>(e - static_cast<int64_t>(m) * m);
      ac.Zc[j] = cn[static_cast<int64_t>(m) * ld + j];
    }
  }
}

// t_c = Zd_{rhs,c} - sum_i Zd_ic x_Ci for the band columns.  A CTA takes 32
// columns (a lane each); its 8 warps split the border rows (warp w the rows
// i = w mod 8, two accumulators), and warp 0 adds the 8 partial sums in order.
__global__ void __launch_bounds__(256) k_band_tvec(BandArgs a, const Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  __shared__ float2 part[8][32];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int c = blockIdx.x * 32 + lane;
  Acc a0 = acc_init(dd_make(0.0f, 0.0f)), a1 = a0;
  if (c < a.nband) {
    int i = wib;
    for (; i + 8 < a.nbd; i += 16) {
      const float2 z0 = a.Zd[static_cast<int64_t>(i) * a.nband + c], z1 = a.Zd[static_cast<int64_t>(i + 8) * a.nband + c];
      acc_madd(a0, dd_neg(f2dd(z0)), f2dd(a.xw[a.nband + i]));
      acc_madd(a1, dd_neg(f2dd(z1)), f2dd(a.xw[a.nband + i + 8]));
    }
    if (i < a.nbd) acc_madd(a0, dd_neg(f2dd(a.Zd[static_cast<int64_t>(i) * a.nband + c])), f2dd(a.xw[a.nband + i]));
  }
  acc_add(a0, acc_get(a1));
  part[wib][lane] = dd2f(acc_get(a0));
  __syncthreads();
  if (wib == 0 && c < a.nband) {
    Acc acc = acc_init(f2dd(a.Zd[static_cast<int64_t>(a.nbd) * a.nband + c]));
    for (int w = 0; w < 8; ++w) acc_add(acc, f2dd(part[w][lane]));
    a.xw[c] = dd2f(acc_get(acc));
  }
}

// One CTA: x_A = L_A^-T t (panels from the last), unscale, write the step.
// Per panel, one dot per row: x_k = sum_{i >= k} X_ik t_i - sum_q Mb_kq x_(c1 + q),
// a group of kSweepG threads per row (warps 0..5); t comes from the unchanged
// xw (staged with the panel); one barrier per panel.
__global__ void __launch_bounds__(kBT) k_band_bwd(BandArgs a0, const Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  extern __shared__ __align__(16) float2 sw[];
  // CTA k sweeps segment k
  const int sg = static_cast<int>(blockIdx.x);
  const BandArgs a = seg_view(a0, sg);
  const float2* xw = a0.xw + a0.seg_row0[sg];
  const int W = a.W, span = W - 1;
  const int nb = a.nbuf;
  float2* xv = sw;
  float2* mbuf = xv + ((a.nband + 1) & ~1);  // nb x kBP x W
  float2* xb = mbuf + nb * kBP * W;          // nb x kBP x kBP
  float2* tb = xb + nb * kBP * kBP;          // nb x kBP
  const int tid = threadIdx.x;
  const int h = W / 2;
  const int i0 = tid / h, q0 = tid % h, di = kBT / h, dq = kBT % h;
  auto stage = [&](int p) {
    const int c0 = kBP * p, w = min(kBP, a.nband - c0), buf = p % nb;
    const float2* src = a.Mb + static_cast<int64_t>(p) * kBP * W;
    int i = i0, q = q0;
    while (i < w) {
      cp_async16(mbuf + (buf * kBP + i) * W + 2 * q, src + i * W + 2 * q);
      q += dq;
      i += di;
      if (q >= h) {
        q -= h;
        ++i;
      }
    }
    for (int e = tid; e < kBP * kBP / 2; e += kBT)
      cp_async16(xb + buf * kBP * kBP + 2 * e, a.Xinv + static_cast<int64_t>(p) * kBP * kBP + 2 * e);
    if (tid < w / 2) cp_async16(tb + buf * kBP + 2 * tid, xw + c0 + 2 * tid);
    cp_async_commit();
  };
  for (int c = tid; c < a.nband; c += kBT) xv[c] = xw[c];
  for (int s0 = 0; s0 < nb - 1; ++s0) {
    if (a.npan - 1 - s0 >= 0) stage(a.npan - 1 - s0);
    else cp_async_commit();
  }
  const int k = tid / kSweepG, g = tid % kSweepG;
  for (int p = a.npan - 1; p >= 0; --p) {
    const int c0 = kBP * p;
    const int w = min(kBP, a.nband - c0);
    const int c1 = c0 + w;
    const int buf = p % nb;
    if (nb == 3) cp_async_wait_but_one();
    else cp_async_wait_all();
    __syncthreads();  // panel p landed; every thread is done with panel p + 1
    if (p - (nb - 1) >= 0) stage(p - (nb - 1));
    else cp_async_commit();
    if (tid < kBP * kSweepG) {
      Acc a0 = acc_init(dd_make(0.0f, 0.0f)), a1 = a0, a2 = a0, a3 = a0;
      if (k < w) {
        const float2* x2 = xb + buf * kBP * kBP;
        const float2* tp = tb + buf * kBP;
        for (int i = k + g; i < w; i += kSweepG) acc_madd(a0, f2dd(x2[i * kBP + k]), f2dd(tp[i]));
        const float2* mrow = mbuf + (buf * kBP + k) * W;
        const int nq = min(span, a.nband - c1);
        int q = g;
        for (; q + 3 * kSweepG < nq; q += 4 * kSweepG) {
          const float2 m0 = mrow[q], m1 = mrow[q + kSweepG], m2 = mrow[q + 2 * kSweepG], m3 = mrow[q + 3 * kSweepG];
          const float2 x0 = xv[c1 + q], x1 = xv[c1 + q + kSweepG], x2v = xv[c1 + q + 2 * kSweepG],
                       x3 = xv[c1 + q + 3 * kSweepG];
          acc_madd(a1, dd_neg(f2dd(m0)), f2dd(x0));
          acc_madd(a2, dd_neg(f2dd(m1)), f2dd(x1));
          acc_madd(a3, dd_neg(f2dd(m2)), f2dd(x2v));
          acc_madd(a0, dd_neg(f2dd(m3)), f2dd(x3));
        }
        for (; q < nq; q += kSweepG) acc_madd(a1, dd_neg(f2dd(mrow[q])), f2dd(xv[c1 + q]));
      }
      acc_add(a0, acc_get(a1));
      acc_add(a2, acc_get(a3));
      acc_add(a0, acc_get(a2));
      const dd sm = group_sum(acc_get(a0));
      if (g == 0 && k < w) xv[c0 + k] = dd2f(sm);
    }
  }
  __syncthreads();
  cp_async_wait_all();
  if (a0.out_scaled) {  // the corner's solve: the scaled solution
    for (int r = tid; r < a.nband; r += kBT) a0.out_scaled[a0.seg_row0[sg] + r] = xv[r];
    return;
  }
  // unscale and write the step at the rows of S (the segment's rows; CTA 0
  // also the border rows, solved with the corner)
  auto put = [&](int r, dd v) {
    const dd xs = dd_mul(v, dd_make(a0.scl[r], 0.0f));
    const int pr = prow(a0, r);
    a0.x[pr] = dd_to_double(xs);
    a0.xdd[2 * pr] = xs.hi;
    a0.xdd[2 * pr + 1] = xs.lo;
  };
  for (int r = tid; r < a.nband; r += kBT) put(a0.seg_row0[sg] + r, f2dd(xv[r]));
  if (sg == 0)
    for (int r = a0.nband + tid; r < a0.n; r += kBT) put(r, f2dd(a0.xw[r]));
}

int sweep_nbuf(int nband, int W);
int fwd_nbuf(int nband, int W, int nctas);

BandArgs band_args(const Sizes& s, const Dev& d) {
  BandArgs a{};
  a.n = s.n6;
  a.nband = s.band_rows;
  a.W = s.band_w;
  a.npan = (s.band_rows + kBP - 1) / kBP;
  a.nbd = s.n6 - s.band_rows;
  a.ring = s.band_ring;
  a.S = d.S;
  a.b = d.rb;
  a.scl = d.band_scl;
  a.Lb = d.band_L;
  a.Xinv = d.band_Xinv;
  a.dpiv = d.band_d;
  a.rdpiv = d.band_rd;
  a.Pbuf = d.band_P;
  a.Zc = d.band_Z;
  a.Zd = d.band_Zd;
  a.Mf = d.band_Mf;
  a.Mb = d.band_Mb;
  a.Cn = d.band_E;
  a.xw = d.band_xw;
  a.x = d.x;
  a.xdd = d.xdd;
  a.perm = d.band_perm;
  a.nseg = s.band_nseg > 1 ? 2 : 1;
  a.seg_row0[0] = 0;
  a.seg_rows[0] = a.nseg > 1 ? s.band_seg_rows : a.nband;
  a.seg_row0[1] = a.seg_rows[0];
  a.seg_rows[1] = a.nband - a.seg_rows[0];
  a.seg_pan0[0] = 0;
  a.seg_pan0[1] = (a.seg_rows[0] + kBP - 1) / kBP;
  a.npan = a.seg_pan0[1] + (a.nseg > 1 ? (a.seg_rows[1] + kBP - 1) / kBP : 0);
  const int segmax = a.seg_rows[0] > a.seg_rows[1] ? a.seg_rows[0] : a.seg_rows[1];
  a.nbuf = sweep_nbuf(segmax, a.W);
  a.nbuf_f = fwd_nbuf(segmax, a.W, (a.nbd + 1) * a.nseg);
  a.zlo = d.band_zlo;
  a.out_scaled = nullptr;
  return a;
}

// The corner of a dissected loop as a band solve of its own.
BandArgs corner_args(const Sizes& s, const Dev& d, const BandArgs& a) {
  BandArgs c = a;
  const int m = a.nbd;
  c.n = m;
  c.nband = m;
  c.W = m;
  c.npan = (m + kBP - 1) / kBP;
  c.nbd = 0;
  c.ring = s.band_ring_c;
  c.nbuf = sweep_nbuf(m, m);
  c.nbuf_f = c.nbuf;
  c.Lb = d.band_Lc;
  c.Xinv = d.band_Xc;
  c.Mf = d.band_Mfc;
  c.Mb = d.band_Mbc;
  c.dpiv = a.dpiv + a.nband;
  c.rdpiv = a.rdpiv + a.nband;
  c.Zc = d.band_Zcc;
  c.Zd = d.band_Zdc;
  c.xw = d.band_Zdc;
  c.perm = nullptr;
  c.nseg = 1;
  c.seg_row0[0] = c.seg_row0[1] = 0;
  c.seg_rows[0] = m;
  c.seg_rows[1] = 0;
  c.seg_pan0[0] = c.seg_pan0[1] = 0;
  c.zlo = d.band_zloc;
  c.out_scaled = a.xw + a.nband;
  return c;
}

int band_ring(int W, int C) {
  const int need = (W + 3 * kBP + C - 1) / C + 1;
  int ring = 1;
  while (ring < need) ring <<= 1;
  return ring;
}

size_t factor_dyn_smem(int W, int C) {
  const int ring = band_ring(W, C);
  return sizeof(float2) * (static_cast<size_t>(ring) * W + static_cast<size_t>(ring) * kBP +
                           static_cast<size_t>(W - 1) * (kBP + 1));
}

// Three panel buffers in the sweeps where they fit in shared memory, else two.
int sweep_nbuf(int nband, int W) {
  return sizeof(float2) * sweep_smem_floats2(nband, W, 3) <= kSmemLimit - 4096 ? 3 : 2;
}

size_t sweepmat_smem(int W) {
  return sizeof(float2) * (static_cast<size_t>(kBP) * W + static_cast<size_t>(W - 1) * kBP + kBP * kBP);
}

size_t band_sweep_smem(int nband, int W) {
  return sizeof(float2) * sweep_smem_floats2(nband, W, sweep_nbuf(nband, W));
}

// The forward sweep runs one CTA per border row and segment: with more CTAs
// than SMs, two buffers (two CTAs per SM where they fit) keep the rows in one
// wave; otherwise the deeper prefetch of sweep_nbuf.
int fwd_nbuf(int nband, int W, int nctas) {
  if (nctas > 132 && 2 * (sizeof(float2) * sweep_smem_floats2(nband, W, 2) + 1024) <= kSmemLimit) return 2;
  return sweep_nbuf(nband, W);
}

size_t fwd_sweep_smem(int nband, int W, int nctas) {
  return sizeof(float2) * sweep_smem_floats2(nband, W, fwd_nbuf(nband, W, nctas));
}

}  // namespace

int band_shape(int nf, const std::vector<int32_t>& sb_row, const std::vector<int32_t>& sb_col, int* band_rows,
               int* band_w) {
  *band_rows = 0;
  *band_w = 0;
  if (nf < 8) return 0;
  std::vector<int32_t> first(nf);
  for (int i = 0; i < nf; ++i) first[i] = i;
  for (size_t q = 0; q < sb_row.size(); ++q) {
    const int r = sb_row[q], c = sb_col[q];
    if (r >= 0 && r < nf && c >= 0 && c <= r) first[r] = std::min(first[r], c);
  }
  std::vector<int32_t> prefw(nf);
  int run = 0;
  for (int i = 0; i < nf; ++i) {
    run = std::max(run, i - first[i] + 1);
    prefw[i] = run;
  }
  double best = -1.0;
  int best_rb = 0, best_wb = 0;
  for (int nbdb = 0; nbdb <= kMaxBorderBlocks && nbdb <= nf - 8; ++nbdb) {
    const int rb = nf - nbdb;
    const int wb = prefw[rb - 1];
    if (wb > kMaxWBlocks) continue;
    const double cost = static_cast<double>(rb) * wb * wb + 2.0 * nbdb * rb * wb + static_cast<double>(nbdb) * nbdb * rb;
    if (best < 0.0 || cost < best) {
      best = cost;
      best_rb = rb;
      best_wb = wb;
    }
  }
  if (best < 0.0) return 0;
  *band_rows = 6 * best_rb;
  *band_w = 6 * best_wb;
  return 1;
}

int band_setup(int n, int nband, int W, int nseg, int seg_rows_max, int* cluster, int* ring, int* ring_c) {
  *cluster = 0;
  *ring = 0;
  *ring_c = 0;
  const int m = n - nband;  // border rows
  if (nband <= 0 || W < 6 || W > 6 * kMaxWBlocks) return 0;
  if (nseg > 1 ? (m > kMaxW || m % 6 != 0 || m < kBP) : m > kMaxBorder) return 0;
  const int segmax = nseg > 1 ? seg_rows_max : nband;
  size_t sweep = band_sweep_smem(segmax, W);
  if (sweep > kSmemLimit - 4096) return 0;
  size_t smat = sweepmat_smem(W);
  size_t corner = 16;
  if (nseg > 1) {  // the corner is factored and swept as a dense band (W = m)
    sweep = std::max(sweep, band_sweep_smem(m, m));
    smat = std::max(smat, sweepmat_smem(m));
    if (sweep > kSmemLimit - 4096 || smat > kSmemLimit - 4096) return 0;
  } else {
    corner = sizeof(float2) * static_cast<size_t>(m) * (m + 2);
    if (corner > kSmemLimit - 4096) return 0;
  }
  if (raise_dynamic_smem(reinterpret_cast<const void*>(k_band_fwd), sweep) != cudaSuccess ||
      raise_dynamic_smem(reinterpret_cast<const void*>(k_band_sweepmat), smat) != cudaSuccess ||
      raise_dynamic_smem(reinterpret_cast<const void*>(k_band_bwd), sweep) != cudaSuccess ||
      raise_dynamic_smem(reinterpret_cast<const void*>(k_band_corner_solve), std::max<size_t>(corner, 16)) !=
          cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  const int sizes[2] = {16, 8};
  for (int ci = 0; ci < 2; ++ci) {
    const int C = sizes[ci];
    if (C > 8 && cudaFuncSetAttribute(k_band_factor<16>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                     cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    // the factor's shared memory at this cluster size (the widest band it takes)
    const size_t fs = factor_dyn_smem(nseg > 1 ? std::max(W, m) : W, C);
    if (fs > kSmemLimit - 32 * 1024) continue;
    const void* fk = (C == 16) ? reinterpret_cast<const void*>(k_band_factor<16>)
                               : reinterpret_cast<const void*>(k_band_factor<8>);
    if (raise_dynamic_smem(fk, fs) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(C);
    cfg.blockDim = dim3(kFT);
    cfg.dynamicSmemBytes = fs;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int nclusters = 0;
    const cudaError_t oe = (C == 16) ? cudaOccupancyMaxActiveClusters(&nclusters, k_band_factor<16>, &cfg)
                                     : cudaOccupancyMaxActiveClusters(&nclusters, k_band_factor<8>, &cfg);
    if (oe != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    if (nclusters < nseg) continue;  // the segments' clusters must run at the same time
    *cluster = C;
    *ring = band_ring(W, C);
    *ring_c = nseg > 1 ? band_ring(m, C) : 0;
    return C;
  }
  return 0;
}

namespace {
cudaError_t launch_factor(const BandArgs& a, int C, int nclusters, cudaStream_t st, const Ctrl* ctrl) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(C * nclusters);
  cfg.blockDim = dim3(kFT);
  cfg.dynamicSmemBytes = factor_dyn_smem(a.W, C);
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = C;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  Ctrl* c = const_cast<Ctrl*>(ctrl);
  return (C == 16) ? cudaLaunchKernelEx(&cfg, k_band_factor<16>, a, c) : cudaLaunchKernelEx(&cfg, k_band_factor<8>, a, c);
}
}  // namespace

int launch_band(const Sizes& s, const Dev& d, cudaStream_t st) {
  const BandArgs a = band_args(s, d);
  int launches = 0;
  k_band_scale<<<(a.n + 255) / 256, 256, 0, st>>>(a, d.ctrl);
  ++launches;
  {
    const int64_t total = static_cast<int64_t>(a.nband) * a.W + static_cast<int64_t>(a.nbd + 1) * a.nband +
                          static_cast<int64_t>(a.nbd + 1) * (a.nbd + 1);
    int blocks = static_cast<int>(std::min<int64_t>((total + 255) / 256, 4096));
    k_band_load<<<std::max(blocks, 1), 256, 0, st>>>(a, d.ctrl);
    ++launches;
  }
  launch_factor(a, s.band_c, a.nseg, st, d.ctrl);  // one cluster per segment
  ++launches;
  k_band_sweepmat<<<a.npan, kBT, sweepmat_smem(a.W), st>>>(a, d.ctrl);
  ++launches;
  const int segmax = std::max(a.seg_rows[0], a.seg_rows[1]);
  k_band_fwd<<<(a.nbd + 1) * a.nseg, kBT, fwd_sweep_smem(segmax, a.W, (a.nbd + 1) * a.nseg), st>>>(a, d.ctrl);
  ++launches;
  {
    const int64_t nt = (a.nbd + 1 + kCornerTile - 1) / kCornerTile;
    const int blocks = static_cast<int>(std::min<int64_t>(nt * (nt + 1) / 2, 8192));
    k_band_corner<<<std::max(blocks, 1), 128, 0, st>>>(a, d.ctrl);
    ++launches;
  }
  if (a.nseg > 1) {
    // the corner (separator and loop closure) as a dense band: factor, sweep
    // matrices, forward and backward sweeps of its right-hand side -> x_C
    const BandArgs c = corner_args(s, d, a);
    const int64_t total = static_cast<int64_t>(c.nband) * c.nband + c.nband;
    k_band_corner_load<<<static_cast<int>(std::min<int64_t>((total + 255) / 256, 4096)), 256, 0, st>>>(c, a.Cn,
                                                                                                   d.ctrl);
    launch_factor(c, s.band_c, 1, st, d.ctrl);
    k_band_sweepmat<<<c.npan, kBT, sweepmat_smem(c.W), st>>>(c, d.ctrl);
    k_band_fwd<<<1, kBT, band_sweep_smem(c.nband, c.W), st>>>(c, d.ctrl);
    k_band_bwd<<<1, kBT, band_sweep_smem(c.nband, c.W), st>>>(c, d.ctrl);
    launches += 5;
  } else {
    const size_t corner = sizeof(float2) * static_cast<size_t>(a.nbd) * (a.nbd + 2);
    k_band_corner_solve<<<1, kCT, std::max<size_t>(corner, 16), st>>>(a, d.ctrl);
    ++launches;
  }
  k_band_tvec<<<std::max((a.nband + 31) / 32, 1), 256, 0, st>>>(a, d.ctrl);
  ++launches;
  k_band_bwd<<<a.nseg, kBT, band_sweep_smem(segmax, a.W), st>>>(a, d.ctrl);
  ++launches;
  return launches;
}

int band_launch_count(const Sizes& s) { return s.band_nseg > 1 ? 13 : 9; }


}  // namespace sgba
