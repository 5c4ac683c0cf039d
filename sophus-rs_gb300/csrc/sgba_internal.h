// sgba_internal.h -- structures shared by the host driver (sgba_capi.cpp) and
// the CUDA translation units.  Plain C++ (no CUDA types beyond cudaStream_t).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <memory>
#include <utility>
#include <vector>

namespace sgba {

// floats per term of the float-float Z (6x3 as (hi, lo) pairs, padded to float4)
constexpr int kZddFloats = 40;
// Camera params on the device: fx fy cx cy alpha beta (the enhanced unified
// camera model; alpha = beta = 0 is the pinhole).  Free intrinsics: per point
// the S_kk triangle (21), J_k^T r~ (6) and Zk c (6); per marg point Zk (6x3,
// float-float); per free pose S_kj (6x6).
constexpr int kIntrMax = 6;
constexpr int kIntrPart = 33;
constexpr int kIntrZk = 36;
constexpr int kIntrScj = 36;
constexpr int kIntrSum = kIntrPart + kIntrMax;

// Device-resident LM control block (one per problem).  Written only by the
// single-CTA control kernels, read by every kernel of an iteration.
struct Ctrl {
  // LM state (crates/sophus_opt/src/nlls/optimizer.rs:40-58)
  double nu;            // lm_damping
  double merit;         // current merit
  double new_merit;     // trial merit of the current step
  double gain_ratio;
  double max_step;
  double max_grad;
  double alpha;         // gauge projection coefficient of the current step
  double dd_sum;        // delta . delta
  double dg_sum;        // delta . neg_grad
  double ftol, gtol, ptol;
  long long rejects;
  long long max_rejects;
  int step;             // total_step_count
  int num_iterations;
  int done;             // termination reached: every kernel returns at once
  int skip;             // 0 normal, 1 gradient tolerance, 2 solve failure
  int accept;
  int termination;
  int record_cap;
  int fail;             // a point block failed its Cholesky this iteration
  unsigned long long max_grad_bits;  // atomicMax over non-negative doubles
  unsigned long long max_step_bits;
  int fin_ticket;   // k_camera_finalize: blocks done (the last one runs the gradient check)
  int cost_ticket;  // trial k_cost: blocks done (the last one runs the LM decision)
  // preconditioned conjugate gradients on the reduced system (sgba_pcg.cu)
  int pcg_done;     // 1: PCG reached its tolerance this iteration, the exact factorization is skipped
  int pcg_iters;    // PCG iterations of the latest solve
  int pcg_status;   // 0 ok, 1 iteration cap reached, 2 breakdown, 3 a grid barrier timed out
  int pcg_pad;
  double pcg_relres;            // relative residual reached by the latest solve
  long long pcg_solves;         // PCG solves so far
  long long pcg_fallbacks;      // of which went to the exact factorization
  long long pcg_total_iters;    // PCG iterations so far
  // equality constraints (range-space KKT on the one-CTA solver): their
  // count, the multipliers and the latest step's multiplier change
  int n_eq;
  int eq_pad;
  double* eq_lambda;
  const double* eq_dlam;
};

// Per-step record, layout-identical to sgba_iter_record.
struct Record {
  double merit, new_merit, lm_damping, gain_ratio, max_step, max_grad;
  int32_t accepted, termination;
};

// std::vector allocator that leaves new elements default-initialised (no
// zero fill): the set-up overwrites its large arrays completely, in parallel,
// so the pages are first touched by the threads that fill them.
template <class T>
struct NoInitAlloc : std::allocator<T> {
  template <class U>
  struct rebind {
    using other = NoInitAlloc<U>;
  };
  NoInitAlloc() = default;
  template <class U>
  NoInitAlloc(const NoInitAlloc<U>&) {}
  template <class U>
  void construct(U* ptr) {
    ::new (static_cast<void*>(ptr)) U;
  }
  template <class U, class... Args>
  void construct(U* ptr, Args&&... args) {
    ::new (static_cast<void*>(ptr)) U(std::forward<Args>(args)...);
  }
};
template <class T>
using RawVec = std::vector<T, NoInitAlloc<T>>;

// Host-side plan: everything derived from the problem structure once.
struct Plan {
  int32_t nc = 0, np = 0, nf = 0, nm = 0;
  int64_t no = 0, ng = 0;
  // sorted observations (by point, then pose; stable)
  RawVec<int64_t> ord;               // sorted -> original index
  RawVec<int32_t> obs_pose, obs_pt;
  // groups = reduced cost terms = distinct (point, pose) pairs, sorted
  RawVec<int64_t> g_begin;           // ng+1, into sorted obs
  RawVec<int32_t> g_pose, g_pt;
  std::vector<int64_t> pt_g_begin;   // np+1
  std::vector<int32_t> pose_fb;      // nc: free block or -1
  std::vector<int32_t> pt_mb;        // np: marg block or -1
  std::vector<int32_t> fb_pose;      // nf: pose index of a free block
  std::vector<int32_t> mb_pt;        // nm: point index of a marg block
  std::vector<double> cnt_f, cnt_m;  // reduced terms per free pose / marg point
  // camera lists (all groups of each free pose), split into tiles
  std::vector<int64_t> cam_g_begin;  // nf+1
  RawVec<int64_t> cam_g;             // group ids
  std::vector<int32_t> tile_fb;      // tile -> free block
  std::vector<int64_t> tile_begin;   // tile -> first entry in cam_g
  std::vector<int64_t> tile_end;
  std::vector<int64_t> fb_tile_begin;  // nf+1
  // reduced camera system blocks (lower, row >= col) and Schur pairs
  std::vector<int32_t> sb_row, sb_col;
  std::vector<int64_t> sb_pair_begin;  // nsb+1
  std::vector<int64_t> chunk_begin;   // pair chunks of at most kSchurChunk pairs, within one block
  std::vector<int32_t> block_chunk_begin;
  int64_t n_h_blocks = 0;
  // gauge: 0 none, 1 scale about gauge_center
  int gauge_kind = 0;
  double gauge_center[3] = {0, 0, 0};
  // pose-graph edges (PoseGraph3CostTerm), sorted by (m, n); reduced terms =
  // distinct (m, n): their edge ranges and free blocks (-1: constant pose);
  // per lower block of S the terms whose off-diagonal block lands there
  // (term id, bit 31: transposed), per free block its (term, side) records
  std::vector<int32_t> edge_m, edge_n;
  std::vector<double> edge_mn;
  std::vector<int32_t> eterm_begin, eterm_fm, eterm_fn;
  std::vector<int32_t> eblk_begin, eblk_term;
  std::vector<int32_t> efb_begin, efb_slot;
};

// Device buffers of one problem.
struct Dev {
  // static structure
  double2* obs_uv = nullptr;       // sorted
  int32_t* obs_pose = nullptr;     // sorted
  int32_t* obs_pt = nullptr;       // sorted
  int64_t* g_begin = nullptr;
  int32_t* g_pose = nullptr;
  int32_t* g_pt = nullptr;
  int64_t* pt_g_begin = nullptr;
  int32_t* pose_fb = nullptr;
  int32_t* pt_mb = nullptr;
  int32_t* fb_pose = nullptr;
  int32_t* mb_pt = nullptr;
  double* cnt_f = nullptr;
  double* cnt_m = nullptr;
  int64_t* cam_g = nullptr;
  int32_t* tile_fb = nullptr;
  int64_t* tile_begin = nullptr;
  int64_t* tile_end = nullptr;
  int64_t* fb_tile_begin = nullptr;
  int32_t* sb_row = nullptr;
  int32_t* sb_col = nullptr;
  int64_t* sb_pair_begin = nullptr;
  int2* pairs = nullptr;           // (group a, group b); int32 group ids
  int64_t* chunk_begin = nullptr;  // Schur pair chunks: nchunk + 1, into pairs
  int32_t* block_chunk_begin = nullptr;  // nsb + 1, into chunks
  float2* schur_part = nullptr;    // 36 float-float partials per chunk
  int32_t* lmk_chunk_pt = nullptr; // landmark pass: point chunks (<= 256 terms), nlchunk + 1
  int32_t* zterm = nullptr;        // np x nf: term of each (point, free block) or -1 (tiled Schur pass)
  // pose priors (sgba_prior.cu), sorted by pose: pose, its free block (-1:
  // constant pose), mean (7), precision (36), and per prior J^T W J (36) and
  // J^T W g (6); per free block the range of its priors (nf + 1)
  int32_t* prior_pose = nullptr;
  int32_t* prior_fb = nullptr;
  double* prior_mean = nullptr;
  double* prior_W = nullptr;
  double* prior_out = nullptr;
  int32_t* prior_fb_begin = nullptr;
  int prior_cap = 0;
  // pose-graph edges (sgba_prior.cu): sorted edges, reduced terms, their
  // records (side 0: m, side 1: n; J^T J (36) and J^T g (6) each) and the
  // off-diagonal J_m^T J_n (36) per term; the CSR lists of Plan
  int32_t* edge_m = nullptr;
  int32_t* edge_n = nullptr;
  double* edge_mn = nullptr;
  int32_t* eterm_begin = nullptr;
  int32_t* eterm_fm = nullptr;
  int32_t* eterm_fn = nullptr;
  double* edge_out = nullptr;
  double* edge_hmn = nullptr;
  int32_t* eblk_begin = nullptr;
  int32_t* eblk_term = nullptr;
  int32_t* efb_begin = nullptr;
  int32_t* efb_slot = nullptr;
  // equality constraints |t(pose)| = r (sgba_prior.cu, sgba_dense.cu): pose,
  // free block, radius; per iteration c, the translation part of each G row
  // (3), the multipliers and the step's change of them
  int32_t* eq_pose = nullptr;
  int32_t* eq_fb = nullptr;
  double* eq_radius = nullptr;
  double* eq_c = nullptr;
  double* eq_jac = nullptr;
  double* eq_lambda = nullptr;
  double* eq_dlam = nullptr;
  int eq_cap = 0;
  int32_t* slow_list = nullptr;    // points redone in float-float this iteration
  int32_t* slow_count = nullptr;
  // state
  double* poses = nullptr;         // nc*7
  double* points = nullptr;        // np*3
  double* poses_t = nullptr;       // trial
  double* intr = nullptr;          // kIntrMax: camera params fx fy cx cy alpha beta (device copy; the kernels
                                   // read them here; alpha = beta = 0 for the pinhole)
  double* intr_t = nullptr;        // kIntrMax: trial params (free intrinsics)
  double* points_t = nullptr;
  float2* res = nullptr;           // residual at current state (sorted obs)
  float2* res_t = nullptr;         // residual at trial state
  float2* res_lo = nullptr;        // low parts of res (float-float linearization)
  float2* res_lo_t = nullptr;      // low parts of res_t
  float* zdd = nullptr;            // ng*kZddFloats: Z as float-float pairs (float-float linearization)
  // per iteration
  float* pose_f = nullptr;         // nc*12: R_cw (row-major) + t_cw, float
  float* pose_dd = nullptr;        // nc*24: R_cw + t_cw as (hi,lo) pairs
  float* zmat = nullptr;           // ng*20: Z = W C^-T (6x3 row-major, padded to 20 floats)
  float* cinv = nullptr;           // nm*12: C^-1 lower (00,10,11,20,21,22) as float-float pairs
  float* cvec = nullptr;           // nm*6: C^-1 b_m as float-float pairs
  double* bm = nullptr;            // nm*3: neg_grad of points
  double* bf = nullptr;            // nf*6: neg_grad of poses
  double* ufull = nullptr;         // nf*36: U_j (undamped J^T J) full 6x6
  double* rb = nullptr;            // nf*6: reduced rhs
  double* tile_part = nullptr;     // ntiles*33 partial sums
  double* S = nullptr;             // n6*n6 FP64 (lower valid)
  float2* S2 = nullptr;            // n6*n6 float-float copy of S (cluster solver only)
  // banded solver (sgba_band.cu): band of the scaled S and its factor, border rows, corner
  float* band_scl = nullptr;       // n6: D^-1/2
  float2* band_L = nullptr;        // band_rows x band_w
  float2* band_Xinv = nullptr;     // panels x 24 x 24
  float2* band_Mf = nullptr;       // panels x 24 x band_w: X_p L of the panel's rows (forward sweep)
  float2* band_Mb = nullptr;       // panels x 24 x band_w: X_p^T L^T of the rows below (backward sweep)
  float2* band_d = nullptr;        // n6 pivots
  float2* band_rd = nullptr;       // n6 reciprocal pivots
  float2* band_P = nullptr;        // band_w x 24 panel exchange
  float2* band_Z = nullptr;        // (border + 1) x band_rows
  float2* band_Zd = nullptr;       // (border + 1) x band_rows
  float2* band_E = nullptr;        // (border + 1)^2
  float2* band_xw = nullptr;       // n6
  // nested dissection of a loop (band_nseg = 2)
  int32_t* band_perm = nullptr;    // n6: row of the solved system -> row of S (null: identity)
  int32_t* band_zlo = nullptr;     // (border + 1) x 2: first nonzero column of each border row per segment
  float2* band_Lc = nullptr;       // corner x corner: the corner as a dense band, then its factor
  float2* band_Xc = nullptr;       // its panels x 24 x 24
  float2* band_Mfc = nullptr;      // its sweep matrices
  float2* band_Mbc = nullptr;
  float2* band_Zcc = nullptr;      // its right-hand side row (corner)
  float2* band_Zdc = nullptr;      // its D^-1 z (corner)
  int32_t* band_zloc = nullptr;    // 1
  float* A = nullptr;              // n6*n6 FP32 factor (lower: unit L)
  float* dpiv = nullptr;           // n6 pivots
  float* wpanel = nullptr;         // n6*64 panel scratch (A_ip L^-T)
  double* x = nullptr;             // n6 solution / refinement
  float* xdd = nullptr;            // n6*2: solution as float-float pairs
  double* r = nullptr;             // n6 residual
  double* dm = nullptr;            // nm*3 point steps
  double* gauge_um = nullptr;      // nm*3 the free poses' gauge direction back-substituted into the points
  // free intrinsics (Sizes::intr_free)
  double* intr_part = nullptr;     // np*kIntrPart per-point parts of S_kk, J_k^T r~, Zk c
  float* intr_zk = nullptr;        // nm*kIntrZk Zk = Y C^-T (6x3) as (hi, lo) pairs
  double* intr_scj = nullptr;      // nf*kIntrScj S_kj (6x6)
  double* intr_sum = nullptr;      // kIntrSum: kIntrPart sums + 6 neg_grad of the intrinsics
  double* part = nullptr;          // reduction partials
  int part_cap = 0;
  Ctrl* ctrl = nullptr;
  Record* records = nullptr;
  int record_cap = 0;
  Record* last_rec = nullptr;      // record of the latest step
  // PCG on the reduced system (sgba_pcg.cu); allocated when a PCG solver is selected
  int32_t* pcg_rowptr = nullptr;   // nf + 1: full block rows of S (both triangles)
  int32_t* pcg_cols = nullptr;     // column block of each entry
  int32_t* pcg_blks = nullptr;     // lower block id of each entry; bit 31 set: use its transpose
  int32_t* pcg_diag = nullptr;     // nf: lower block id of each diagonal block
  double* pcg_S = nullptr;         // nsb * 36: Jacobi-scaled lower blocks
  float2* pcg_S2 = nullptr;        // nsb * 36: the same as float-float pairs (the PCG products)
  double* pcg_scl = nullptr;       // n6: D^-1/2
  double* pcg_P = nullptr;         // nf * 36: preconditioner blocks
  double* pcg_Cinv = nullptr;      // nf * 36: inverse Cholesky factor of each scaled diagonal block
  double* pcg_vec = nullptr;       // 6 * n6: x r u p s w (scaled)
  double* pcg_part = nullptr;      // pcg_grid * 4 partial dot products
  unsigned* pcg_bar = nullptr;     // grid barrier: arrival count, generation
  float* pcg_feat = nullptr;       // nf * kPcgFeat node features (learned correction)
  float* pcg_ew = nullptr;         // edge weight (block Frobenius norm) of every full-row entry
  float* pcg_h = nullptr;          // 2 * nf * kPcgHidden hidden states
  float* pcg_msg = nullptr;        // nf * kPcgHidden aggregated messages
  float* pcg_L = nullptr;          // nf * 21: learned correction factor (lower 6x6)
  const uint16_t* pcg_w = nullptr; // BF16 weights of the learned correction (owned by a model), or null
};

// Parameters of the learned block preconditioner on one device: the FP32
// master copy, the BF16 copy the kernels read, Adam moments and a gradient
// buffer (training).
struct PcgModel {
  int device = 0;
  float* w32 = nullptr;
  uint16_t* wbf = nullptr;
  float* m1 = nullptr;
  float* m2 = nullptr;
  float* grad = nullptr;
  long long step = 0;
};

// One reduced system of a training set (device arrays): the full block rows
// of S~ (Jacobi-scaled), b~ and the exact solution x*; den = x*^T b~.
struct PcgSystem {
  int nf = 0;
  int64_t nsb = 0, nnzb = 0;
  int32_t* rowptr = nullptr;
  int32_t* cols = nullptr;
  int32_t* blks = nullptr;
  int32_t* diag = nullptr;
  double* Sb = nullptr;
  float2* Sb2 = nullptr;
  double* b = nullptr;
  double* xs = nullptr;
  double den = 0.0;
};

// Training set and the training / evaluation workspace (sized for the
// largest system).
struct PcgTrainSet {
  int device = 0;
  std::vector<PcgSystem> sys;
  std::vector<void*> ws;
  int cap_nf = 0;
  int64_t cap_nnzb = 0;
  float *feat = nullptr, *ew = nullptr, *wsum = nullptr, *Hs = nullptr, *Ms = nullptr, *Us = nullptr, *L = nullptr;
  double *P = nullptr, *Ci = nullptr, *evec = nullptr, *Se = nullptr, *loss_part = nullptr, *loss = nullptr;
  float *dL = nullptr, *dHa = nullptr, *dHb = nullptr, *dU = nullptr, *dM = nullptr, *dHp = nullptr;
  float* hbuf = nullptr;
  double* vec = nullptr;
  double* part = nullptr;
  unsigned* bar = nullptr;
  Ctrl* ctrl = nullptr;
  double* xout = nullptr;
  float* xdd = nullptr;
  PcgTrainSet() = default;
  PcgTrainSet(const PcgTrainSet&) = delete;
  PcgTrainSet& operator=(const PcgTrainSet&) = delete;
  ~PcgTrainSet();
  cudaError_t reserve(int nf, int64_t nnzb);
  void free_workspace();
};

// Learned block preconditioner: node features, hidden width, message-passing layers.
constexpr int kPcgFeat = 32;
constexpr int kPcgHidden = 64;
constexpr int kPcgLayers = 3;
constexpr int kPcgOut = 21;
// Parameter layout (FP32 master copy; the forward reads a BF16 copy):
//   W_in [kPcgHidden x kPcgFeat], b_in [kPcgHidden],
//   per layer: W_self [H x H], W_msg [H x H], b [H],
//   W_out [kPcgOut x H], b_out [kPcgOut]
constexpr int kPcgParams = kPcgHidden * kPcgFeat + kPcgHidden +
                           kPcgLayers * (2 * kPcgHidden * kPcgHidden + kPcgHidden) + kPcgOut * kPcgHidden + kPcgOut;

struct Sizes {
  int32_t nc, np, nf, nm;
  int64_t no, ng, nsb, ntiles, nchunk;
  int32_t nlchunk, lmk_cap;  // landmark point chunks and the most terms of one chunk
  int n6;
  double intr[kIntrMax];  // fx fy cx cy alpha beta
  double huber;
  int gauge_kind;
  double gauge_center[3];
  int small_dense;    // 1: one-CTA float-float solver (small systems)
  int dense_c;        // cluster size of the single-launch dense solver, 0 = multi-launch path
  size_t dense_smem;  // its dynamic shared memory per CTA
  int band_rows;      // banded solver: rows of the band part (0 = not used)
  int band_w;         // its band width
  int band_c;         // its cluster size
  int band_ring;      // its row slots per CTA
  int band_nseg;      // 2: nested dissection (two band segments, the corner = separator + closure)
  int band_seg_rows;  // rows of the first segment
  int band_ring_c;    // row slots per CTA of the corner's factor
  int lin_dd;          // float-float linearization (Jacobians, products and Z in float-float)
  int schur_dense;     // S by tiles of pose blocks (nearly dense S and Z: local windows), not by pairs
  int n_prior;         // pose priors (a second cost function; 0: none)
  int n_edge;          // pose-graph edges (0: none)
  int n_eq;            // equality constraints |t(pose)| = r (0: none; the one-CTA solver only)
  int n_eterm;         // their reduced terms (distinct (m, n))
  int intr_free;       // the camera params are Free: one more 6-row block, last in S
  int intr_nk;         // free params: 4 (pinhole, padded to 6 rows) or 6 (EUCM)
  int eucm;            // the camera is the enhanced unified camera model (else the pinhole)
  int lmk_dd_ok;       // the chunked float-float landmark pass fits (else the warp-per-point kernel)
  int bsub_chunks_ok;  // the chunked back-substitution fits (else the warp-per-point kernel)
  int pcg_mode;        // 0 exact factorization; 1 PCG, block-Jacobi; 2 PCG, learned correction (fallback: exact)
  int pcg_max_iters;
  double pcg_tol;      // relative residual of the Jacobi-scaled system
  int pcg_grid;        // CTAs of the cooperative PCG kernel
  int64_t pcg_nnzb;    // entries of the full block rows
  float lmk_well_tol;  // point blocks: FP32 Cholesky kept while every pivot keeps this fraction
  int lmk_list_grid;   // CTAs of the float-float redo of the other points
};

// ---- launchers (sgba_kernels.cu / sgba_solver.cu) -------------------------
// Each returns the number of kernel launches it enqueued.
int launch_pose_tables(const Sizes& s, const Dev& d, const double* poses, cudaStream_t st);
int launch_cost(const Sizes& s, const Dev& d, const double* poses, const double* points,
                float2* res_out, double* partials, cudaStream_t st);
int launch_init_merit(const Sizes& s, const Dev& d, cudaStream_t st);
int launch_iteration_begin(const Sizes& s, const Dev& d, cudaStream_t st);
int launch_linearize(const Sizes& s, const Dev& d, double nu_override, bool use_override,
                     cudaStream_t st);
int launch_schur(const Sizes& s, const Dev& d, cudaStream_t st);
int launch_factor_solve(const Sizes& s, const Dev& d, cudaStream_t st);
int launch_exact_solve(const Sizes& s, const Dev& d, cudaStream_t st);  // the factorization alone
int launch_update(const Sizes& s, const Dev& d, cudaStream_t st);
int launch_decide(const Sizes& s, const Dev& d, cudaStream_t st);

int launch_single(const Sizes& s, const Dev& d, int kernel_id, cudaStream_t st);
int cost_partials_needed(const Sizes& s);  // reduction partial slots
int landmark_setup(int cap);  // dynamic shared memory of the chunked landmark pass (0 = ok)
int landmark_dd_setup(int cap);  // the same for its float-float variant (0 = ok)
int backsub_chunks_setup(int cap);  // the chunked back-substitution (0 = ok)
int solver_launch_count(const Sizes& s);

// Single-launch cluster solver (sgba_dense.cu): chooses the cluster size for
// order n (0 = does not fit) and enqueues the factorization + refined solve.
int dense_cluster_setup(int n, int* cluster, size_t* smem);
int launch_dense_cluster(const Sizes& s, const Dev& d, cudaStream_t st);
// Small systems (local windows): one CTA, float-float LDL^T (1 = usable).
int small_dense_setup(int n);
// The same with n_eq equality constraints (their columns beside the rhs).
int small_dense_setup_eq(int n, int n_eq);
int launch_small_dense(const Sizes& s, const Dev& d, cudaStream_t st);

// Raise a kernel's dynamic shared memory limit to at least `bytes` on the
// current device.  The limit is a per-function, per-device setting shared by
// every problem (and every captured graph) in the process, so it only ever
// grows: a later, smaller problem must not lower it under an earlier one's
// launches.  Thread-safe.
cudaError_t raise_dynamic_smem(const void* func, size_t bytes);

// Banded solver (sgba_band.cu) for reduced systems that are a band plus a few
// dense border rows (sequential and loop-shaped problems).  band_shape picks
// the split from the lower block pattern of S (0 = no split within the band
// and border limits); band_setup checks the launch limits and returns the
// cluster size (0 = no).
int band_shape(int nf, const std::vector<int32_t>& sb_row, const std::vector<int32_t>& sb_col, int* band_rows,
               int* band_w);
int band_setup(int n, int nband, int w, int nseg, int seg_rows_max, int* cluster, int* ring, int* ring_c);
int launch_band(const Sizes& s, const Dev& d, cudaStream_t st);
int band_launch_count(const Sizes& s);
// Schur observation-pair lists on the device (sgba_plan.cu): pairs per lower
// block (atomic counts into totals[nf(nf+1)/2]); then the pair list d.pairs in
// (block, point) order from the block map, block offsets and a zeroed
// (chunk x block) table.
cudaError_t pair_totals(const Sizes& s, const Dev& d, int32_t* totals, cudaStream_t st);
cudaError_t pair_fill(const Sizes& s, const Dev& d, const int32_t* bidmap, int64_t nb, const int64_t* block_begin,
                      int32_t nchunk, int32_t* table, cudaStream_t st);
// The term of every (marginalized point, free pose block), -1 where the point
// has none: T[i * nf + fb] (the tiled Schur pass of nearly dense systems).
cudaError_t zterm_fill(const Sizes& s, const Dev& d, int32_t* T, cudaStream_t st);

// PCG on the reduced system (sgba_pcg.cu): grid size for the cooperative
// kernel (0 = cannot launch), and the launch chain (structure arrays uploaded
// by the host).  The exact factorization that follows is skipped when PCG
// converged (Ctrl::pcg_done).
constexpr int kPcgMaxGrid = 2048;  // CTAs of the cooperative PCG kernel at most (partial-sum slots)
int pcg_setup(int nf, int* grid);
int launch_pcg(const Sizes& s, const Dev& d, cudaStream_t st);
// The same after the scaled blocks exist (pcg_S, pcg_S2; d.rb already scaled
// when d.pcg_scl is null): network, preconditioner, solve.
int launch_pcg_scaled(const Sizes& s, const Dev& d, cudaStream_t st);
// Only the Jacobi-scaled blocks (pcg_S, pcg_S2, pcg_scl) from the dense S.
int launch_pcg_blocks_only(const Sizes& s, const Dev& d, cudaStream_t st);
int pcg_launch_count(const Sizes& s);
// The learned correction's forward pass (sgba_pcg_net.cu): node features,
// embedding, message-passing layers and the output head into Dev::pcg_L.
int pcg_net_setup();
int launch_pcg_net(const Sizes& s, const Dev& d, cudaStream_t st);
int pcg_net_launch_count();
// Training (sgba_pcg_net.cu): forward (and backward, accumulating into
// m.grad) on system idx, *loss synchronously when non-null; one Adam step
// (gradients scaled by `scale`, then zeroed); PCG on a stored system
// (mode 1 block-Jacobi, 2 learned).
cudaError_t pcg_loss_grad(PcgModel& m, PcgTrainSet& t, int idx, bool backward, double* loss, cudaStream_t st);
cudaError_t pcg_adam(PcgModel& m, float scale, float lr, float b1, float b2, float eps, cudaStream_t st);
cudaError_t pcg_evaluate(const PcgModel* m, PcgTrainSet& t, int idx, int mode, int max_iters, double tol,
                         int* iters, double* relres, int* status, cudaStream_t st);

// ---- pose priors (sgba_prior.cu) -----------------------------------------
constexpr int kPriorOut = 42;  // per prior: J^T W J (36, row-major), J^T W g (6)
struct PriorArgs {
  int n;
  const int32_t* pose;
  const int32_t* fb;
  const double* mean;
  const double* W;
  double* out;
};
// The priors at `poses`: with lin, their blocks into Dev::prior_out (priors
// on free poses); their total cost into *cost_sum (float-float sum in prior
// order).  gate: 0 always, 1 unless the LM loop is done, 2 unless done or the
// step is skipped.  Returns the launches (0 without priors).
int launch_prior_eval(const Sizes& s, const Dev& d, const double* poses, int lin, int gate, double* cost_sum,
                      cudaStream_t st);
// The pose-graph edges at `poses` (PoseGraph3CostTerm): with lin, per reduced
// term the records of both sides into Dev::edge_out and J_m^T J_n into
// Dev::edge_hmn; their total cost into *cost_sum.  The same gates.
int launch_edge_eval(const Sizes& s, const Dev& d, const double* poses, int lin, int gate, double* cost_sum,
                     cudaStream_t st);
// Equality constraints (TranslationNormConstraint) at the current poses: c and
// G, and G^T lambda added to the free gradient and the reduced rhs (after the
// camera finalisation, before the solve).  Returns the launches.
constexpr int kMaxEq = 8;
int launch_eq_eval(const Sizes& s, const Dev& d, cudaStream_t st);
// After the update: the multiplier step's share of the gain-ratio sums (one
// more update partial at upd_slot) and of the largest step entry.
int launch_eq_post(const Sizes& s, const Dev& d, double* upd_slot, cudaStream_t st);

// ---- batched local windows ----------------------------------------------
// A batch launches every kernel of an LM iteration once for many independent
// problems (local windows).  Block b of a batched launch runs block
// b - off[w] of window w's own grid with window w's arguments and control
// block (off: prefix sums of the per-window grid sizes), so every window
// computes exactly what its own launches compute (sgba_kernels.cu,
// sgba_dense.cu).
struct BatchWin {
  const Sizes* s;
  const Dev* d;
};
// 1: the window's iteration runs in batched launches (FP32 linearization with
// the chunked landmark pass and back-substitution, pinhole camera, fixed
// intrinsics, the one-CTA or one-cluster dense solver, no PCG).
int batch_eligible(const Sizes& s);
// Per-window arguments and block offsets of every batched kernel, uploaded
// to the device once per call (stream-ordered allocation on st).
struct BatchTables;
BatchTables* batch_tables_create(const std::vector<BatchWin>& wins, int skip_final_hessian, cudaStream_t st,
                                 cudaError_t* err);
void batch_tables_destroy(BatchTables* t, cudaStream_t st);
// Initial control blocks (the same for every window), pose tables, cost and
// merit (sgba_optimizer_init).
int batch_launch_init(const BatchTables* t, const Ctrl& init, cudaStream_t st);
// One LM iteration of every window.
int batch_launch_iteration(const BatchTables* t, cudaStream_t st);
// build_solution's final linearisation of every window.
int batch_launch_final(const BatchTables* t, cudaStream_t st);
// Control blocks and the first cap records of every window into packed
// device arrays (n Ctrl, n x cap Record).
int batch_launch_collect(const BatchTables* t, Ctrl* ctrl_out, Record* rec_out, int cap, cudaStream_t st);
int batch_window_count(const BatchTables* t);
// The dense solver of a batch (sgba_dense.cu): one launch for the windows on
// the one-CTA solver, one cluster launch per cluster size.
struct DenseBatch;
DenseBatch* dense_batch_create(const std::vector<BatchWin>& wins, Ctrl* const* ctrl_dev, cudaStream_t st,
                               cudaError_t* err);
void dense_batch_destroy(DenseBatch* b, cudaStream_t st);
int launch_dense_batch(const DenseBatch* b, cudaStream_t st);

// Per-term Jacobians (2x6 pose, 2x3 point) of the given (camera, point) pairs
// at the current variables, as the linearization kernels evaluate them:
// precision 0 FP32, 1 float-float (sgba_debug_jacobians).
cudaError_t launch_debug_jacobians(const Sizes& s, const Dev& d, int64_t n, const int32_t* cam, const int32_t* pt,
                                   int precision, double* jp, double* jm, cudaStream_t st);

// ---- covariance queries of the final Hessian (sgba_cov.cu) ---------------
// Device buffers of one prepared covariance (all f64; the camera block first
// when the camera params are free, as in the reference's family order): per reduced term
// J_pose^T J_pose (21 upper), W = J_pose^T J_point (18) and
// J_point^T J_point (6 upper); per term with a free pose Y = W H_mm^-1 (18);
// per marginalized point H_mm^-1 (9, NaN where H_mm is singular); per free
// pose its undamped diagonal block of H (36); S (n x n, then its LDL^T factor
// in the lower triangle), the diagonal blocks' unit-lower factors and the
// pivots; Z = S^-1 or the min-norm pseudo-inverse S+ (n x n, both triangles).
constexpr int kCovRec = 48;
// per term with free camera params: J_cam^T J_cam (21 upper), J_cam^T J_pose (6 x 6), J_cam^T J_point (6 x 3)
constexpr int kCovCamRec = 80;
struct CovBufs {
  int ready = 0;
  int n = 0;      // rows of S: the camera block (nci rows) and 6 per free pose
  int nci = 0;    // free camera params: 6 rows (their nk params, then identity padding), else 0
  int nk = 0;     // free camera params: 4 (pinhole) or 6 (EUCM)
  int rank = 0;   // pivots > 0
  // free camera params: per term J_cam^T J_cam, J_cam^T J_pose, J_cam^T J_point
  // (80 doubles); per marginalized point W_cq and Y_cq = W_cq H_mm^-1 (6 x 3
  // each); H_cc (6 x 6) and per free pose H_ca (camera rows x pose columns)
  double* crec = nullptr;
  double* wc = nullptr;
  double* yc = nullptr;
  double* hcc = nullptr;
  double* hcp = nullptr;
  double* rec = nullptr;
  double* y = nullptr;
  double* vinv = nullptr;
  double* hdiag = nullptr;
  double* S = nullptr;
  double* Z = nullptr;
  double* ldiag = nullptr;
  double* dpiv = nullptr;
  double* work = nullptr;  // the inverse's partial sums
  int* status = nullptr;  // [0] factor: 1 non-finite pivot, 2 indefinite (Bunch-Kaufman case); [1] singular H_mm
  std::vector<void*> allocs;
};
// H blocks of every reduced term and point, S assembled at the current
// variables with zero damping (the priors' and edges' records must be current).
int launch_cov_assemble(const Sizes& s, const Dev& d, const CovBufs& c, cudaStream_t st);
// LDL^T of the n x n S in place (the reference's per-block pivot rule).
int launch_cov_factor(int n, double* S, double* ldiag, double* dpiv, int* status, cudaStream_t st);
// Z = S^-1 from the factor (full rank); work: cov_inverse_work(n) doubles.
size_t cov_inverse_work(int n);
int launch_cov_inverse(int n, const double* L, const double* ldiag, const double* dpiv, double* Z, double* work,
                       cudaStream_t st);
// Z = S+ = E G^-1 diag(d_J)^-1 G^-1 E^T (rank-deficient S; J the positive
// pivots, host list); temporaries from `pool` on st.  *g_ok = 0 when G has a
// pivot <= 0 (synchronises st).
cudaError_t cov_pinv(int n, const double* L, const double* ldiag, const double* dpiv, const std::vector<int32_t>& J,
                     double* Z, cudaMemPool_t pool, cudaStream_t st, int* g_ok);
// Block queries: per query (row kind, row index, col kind, col index),
// mode 0 covariance, 1 precision (H); out 36 doubles and dims 2 per query.
cudaError_t launch_cov_query(const Sizes& s, const Dev& d, const CovBufs& c, int mode, int nq, const int32_t* q,
                             double* out, int32_t* dims, cudaStream_t st);

// Allocation-free total cost over caller-owned device arrays; the scratch is a
// static __device__ array (sgba_kernels.cu).  Arguments are validated by the
// caller except the observation indices, which the kernel checks.
int noalloc_max_cams();
cudaError_t launch_total_cost_noalloc(int32_t nc, const double* poses, int32_t np, const double* points,
                                      int64_t no, const int32_t* obs_cam, const int32_t* obs_pt,
                                      const double* obs_uv, const double* intr, double huber,
                                      double* cost, cudaStream_t st);

}  // namespace sgba
