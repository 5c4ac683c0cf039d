// sgba_plan.cu -- device-side construction of the Schur observation-pair
// lists (part of sgba_problem_create).
//
// For every marginalized point i and every pair of its terms (a, b) whose
// poses are both free, the reduced camera system block (r, c) = (free block of
// pose(b), free block of pose(a)), r >= c, receives Z_b Z_a^T
// (crates/sophus_solver/src/ldlt/schur_ldlt.rs:82-135).  The pairs of each
// block are stored contiguously, ordered by point, so that the Schur pass is
// deterministic.  Building that list on the host costs more than the whole
// optimization of the 100-camera sphere workload; here it takes three short
// kernels:
//   k_pair_totals   pairs per lower block (atomic counts; order-free);
//   (host)          the block pattern, block offsets;
//   k_pair_count    pairs per (point chunk, block);
//   k_pair_scan     exclusive scan over the chunks of each block (one thread per block);
//   k_pair_fill     one CTA per point chunk walks its points in order, each
//                   point's pairs in parallel (they fall into distinct blocks).
// The order is (block, point), exactly the order of a sequential build.
#include <cuda_runtime.h>

#include <cstdint>

#include "sgba_internal.h"

namespace sgba {

namespace {

__device__ __forceinline__ int64_t lower_id(int64_t r, int64_t c) { return r * (r + 1) / 2 + c; }

// Pair index t of an L-term point -> (b, a), a <= b: row b is the one with
// b(b+1)/2 <= t < (b+1)(b+2)/2. A float estimate of the row (FP64 runs at a
// small fraction of the FP32 rate), then exact integer corrections.
__device__ __forceinline__ void decode_pair(int64_t t, int* b, int* a) {
  int bb = static_cast<int>((sqrtf(8.0f * static_cast<float>(t) + 1.0f) - 1.0f) * 0.5f);
  if (bb < 0) bb = 0;
  while (bb > 0 && static_cast<int64_t>(bb) * (bb + 1) / 2 > t) --bb;
  while (static_cast<int64_t>(bb + 1) * (bb + 2) / 2 <= t) ++bb;
  *b = bb;
  *a = static_cast<int>(t - static_cast<int64_t>(bb) * (bb + 1) / 2);
}

struct PairArgs {
  int32_t np;
  const int64_t* pt_g_begin;
  const int32_t* g_pose;
  const int32_t* pose_fb;
  const int32_t* pt_mb;
  int32_t nchunk;         // point chunks (contiguous, in order)
  const int32_t* bidmap;  // lower id -> block id (or -1)
  int64_t nb;
  int32_t* totals;        // per lower id
  int32_t* table;         // nchunk x nb
  int2* pairs;
};

__device__ __forceinline__ int chunk_first(const PairArgs& a, int c) {
  return static_cast<int>((static_cast<int64_t>(a.np) * c) / a.nchunk);
}

// One warp per point: pairs per lower block.
__global__ void __launch_bounds__(256) k_pair_totals(PairArgs a) {
  const int lane = threadIdx.x & 31;
  for (int64_t i = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; i < a.np;
       i += (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5) {
    if (a.pt_mb[i] < 0) continue;
    const int64_t g0 = a.pt_g_begin[i];
    const int64_t L = a.pt_g_begin[i + 1] - g0;
    for (int64_t t = lane; t < L * (L + 1) / 2; t += 32) {
      int b, c;
      decode_pair(t, &b, &c);
      const int r = a.pose_fb[a.g_pose[g0 + b]], cc = a.pose_fb[a.g_pose[g0 + c]];
      if (r < 0 || cc < 0) continue;
      atomicAdd(a.totals + lower_id(r, cc), 1);
    }
  }
}

// One warp per point: pairs per (point chunk, block).
__global__ void __launch_bounds__(256) k_pair_count(PairArgs a) {
  const int lane = threadIdx.x & 31;
  for (int64_t i = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; i < a.np;
       i += (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5) {
    if (a.pt_mb[i] < 0) continue;
    const int ch = static_cast<int>(((i + 1) * static_cast<int64_t>(a.nchunk) - 1) / a.np);
    const int64_t g0 = a.pt_g_begin[i];
    const int64_t L = a.pt_g_begin[i + 1] - g0;
    for (int64_t t = lane; t < L * (L + 1) / 2; t += 32) {
      int b, c;
      decode_pair(t, &b, &c);
      const int r = a.pose_fb[a.g_pose[g0 + b]], cc = a.pose_fb[a.g_pose[g0 + c]];
      if (r < 0 || cc < 0) continue;
      atomicAdd(a.table + static_cast<int64_t>(ch) * a.nb + a.bidmap[lower_id(r, cc)], 1);
    }
  }
}

// One thread per block b: table[c][b] <- first pair slot of chunk c in block b
// (an exclusive scan over the chunks; neighbouring threads take neighbouring
// blocks, so every step reads and writes one contiguous row of the table).
__global__ void __launch_bounds__(128) k_pair_scan(PairArgs a, const int64_t* block_begin) {
  for (int64_t b = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; b < a.nb;
       b += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    int64_t run = block_begin[b];
    int32_t* e = a.table + b;
    int c = 0;
    for (; c + 16 <= a.nchunk; c += 16) {
      int32_t v[16];
#pragma unroll
      for (int k = 0; k < 16; ++k) v[k] = e[static_cast<int64_t>(c + k) * a.nb];
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        e[static_cast<int64_t>(c + k) * a.nb] = static_cast<int32_t>(run);
        run += v[k];
      }
    }
    for (; c < a.nchunk; ++c) {
      const int32_t v = e[static_cast<int64_t>(c) * a.nb];
      e[static_cast<int64_t>(c) * a.nb] = static_cast<int32_t>(run);
      run += v;
    }
  }
}

// One CTA per point chunk; its points in order, each point's pairs in
// parallel (one pair per block per point, so the slots never collide).
__global__ void __launch_bounds__(256) k_pair_fill(PairArgs a) {
  const int c = blockIdx.x;
  if (c >= a.nchunk) return;
  int32_t* slot = a.table + static_cast<int64_t>(c) * a.nb;
  const int i1 = chunk_first(a, c + 1);
  for (int i = chunk_first(a, c); i < i1; ++i) {
    if (a.pt_mb[i] >= 0) {
      const int64_t g0 = a.pt_g_begin[i];
      const int64_t L = a.pt_g_begin[i + 1] - g0;
      for (int64_t t = threadIdx.x; t < L * (L + 1) / 2; t += blockDim.x) {
        int b, cc;
        decode_pair(t, &b, &cc);
        const int r = a.pose_fb[a.g_pose[g0 + b]], col = a.pose_fb[a.g_pose[g0 + cc]];
        if (r < 0 || col < 0) continue;
        const int32_t bid = a.bidmap[lower_id(r, col)];
        const int32_t pos = slot[bid];
        slot[bid] = pos + 1;
        a.pairs[pos] = make_int2(static_cast<int>(g0 + b), static_cast<int>(g0 + cc));
      }
    }
    __syncthreads();
  }
}

}  // namespace

cudaError_t pair_totals(const Sizes& s, const Dev& d, int32_t* totals, cudaStream_t st) {
  PairArgs a{};
  a.np = s.np;
  a.pt_g_begin = d.pt_g_begin;
  a.g_pose = d.g_pose;
  a.pose_fb = d.pose_fb;
  a.pt_mb = d.pt_mb;
  a.totals = totals;
  int blocks = static_cast<int>((static_cast<int64_t>(s.np) * 32 + 255) / 256);
  if (blocks > 8192) blocks = 8192;
  if (blocks < 1) blocks = 1;
  k_pair_totals<<<blocks, 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t pair_fill(const Sizes& s, const Dev& d, const int32_t* bidmap, int64_t nb, const int64_t* block_begin,
                      int32_t nchunk, int32_t* table, cudaStream_t st) {
  PairArgs a{};
  a.np = s.np;
  a.pt_g_begin = d.pt_g_begin;
  a.g_pose = d.g_pose;
  a.pose_fb = d.pose_fb;
  a.pt_mb = d.pt_mb;
  a.nchunk = nchunk;
  a.bidmap = bidmap;
  a.nb = nb;
  a.table = table;
  a.pairs = d.pairs;
  int blocks = static_cast<int>((static_cast<int64_t>(s.np) * 32 + 255) / 256);
  if (blocks > 8192) blocks = 8192;
  if (blocks < 1) blocks = 1;
  k_pair_count<<<blocks, 256, 0, st>>>(a);
  int sb = static_cast<int>((nb + 127) / 128);
  if (sb > 8192) sb = 8192;
  if (sb < 1) sb = 1;
  k_pair_scan<<<sb, 128, 0, st>>>(a, block_begin);
  k_pair_fill<<<nchunk, 256, 0, st>>>(a);
  return cudaGetLastError();
}

namespace {

// term of each (marginalized point, free pose block): T[i * nf + fb] = g
__global__ void k_zterm(int64_t ng, const int32_t* __restrict__ g_pt, const int32_t* __restrict__ g_pose,
                        const int32_t* __restrict__ pose_fb, const int32_t* __restrict__ pt_mb, int nf,
                        int32_t* __restrict__ T) {
  const int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (g >= ng) return;
  const int fb = pose_fb[g_pose[g]];
  const int i = g_pt[g];
  if (fb < 0 || pt_mb[i] < 0) return;
  T[static_cast<int64_t>(i) * nf + fb] = static_cast<int32_t>(g);
}

}  // namespace

cudaError_t zterm_fill(const Sizes& s, const Dev& d, int32_t* T, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(T, 0xff, sizeof(int32_t) * static_cast<size_t>(s.np) * s.nf, st);
  if (e != cudaSuccess || s.ng == 0) return e;
  const int64_t blocks = (s.ng + 255) / 256;
  k_zterm<<<static_cast<unsigned>(blocks), 256, 0, st>>>(s.ng, d.g_pt, d.g_pose, d.pose_fb, d.pt_mb, s.nf, T);
  return cudaGetLastError();
}

}  // namespace sgba
