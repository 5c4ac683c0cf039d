// sgba_pcg_net.cu -- the learned block preconditioner: a message-passing
// network over the camera covisibility graph (the block pattern of the reduced
// camera system) that predicts, per free pose, the factor L_j of the
// correction in P_j = C_j^-T (I + L_j L_j^T) C_j^-1 (sgba_pcg.cu).
//
// Network (weights BF16, arithmetic and accumulation FP32):
//   node features f_j (kPcgFeat): the 15 off-diagonal entries of the
//     Jacobi-scaled diagonal block B_j, log of the diagonal of B_j^-1, and
//     statistics of the neighbouring blocks' Frobenius norms w_jk;
//   h0_j   = relu(W_in f_j + b_in)
//   m_j    = sum_k w_jk h_k / sum_k w_jk           (k != j, neighbours in S)
//   h'_j   = h_j + relu(W_self h_j + W_msg m_j + b)  (kPcgLayers layers)
//   L_j    = W_out h_j + b_out                      (21 lower-triangular entries)
// With W_out = 0 and b_out = 0 the preconditioner is block-Jacobi.
#include <cuda_runtime.h>

#include <cstdint>

#include "sgba_internal.h"

namespace sgba {

namespace {

constexpr int kNT = 256;  // threads per CTA: one warp per node
constexpr int kNW = kNT / 32;
constexpr int H = kPcgHidden;
constexpr int F = kPcgFeat;

__device__ __forceinline__ bool skipping(const Ctrl* c) { return c->done != 0 || c->skip != 0; }
__device__ __forceinline__ float bf16f(uint16_t u) { return __uint_as_float(static_cast<unsigned>(u) << 16); }

}  // namespace

// Offsets of the parameter blocks (in elements).
__host__ __device__ constexpr int pcg_off_win() { return 0; }
__host__ __device__ constexpr int pcg_off_bin() { return H * F; }
__host__ __device__ constexpr int pcg_off_ws(int l) { return H * F + H + l * (2 * H * H + H); }
__host__ __device__ constexpr int pcg_off_wm(int l) { return pcg_off_ws(l) + H * H; }
__host__ __device__ constexpr int pcg_off_b(int l) { return pcg_off_ws(l) + 2 * H * H; }
__host__ __device__ constexpr int pcg_off_wout() { return pcg_off_ws(kPcgLayers); }
__host__ __device__ constexpr int pcg_off_bout() { return pcg_off_wout() + kPcgOut * H; }
static_assert(pcg_off_bout() + kPcgOut == kPcgParams, "parameter layout");

// Node features of free pose j from the Jacobi-scaled blocks.  Also writes
// the edge weight w_jk of every entry of block row j (0 on the diagonal).
__device__ void pcg_node_features(int j, const int32_t* rowptr, const int32_t* cols, const int32_t* blks,
                                  const int32_t* diag, const double* Sb, float* f, float* ew) {
  // one warp: lanes over the row's entries
  const int lane = threadIdx.x & 31;
  double sw = 0.0, sw2 = 0.0, mw = 0.0;
  int deg = 0;
  for (int e = rowptr[j] + lane; e < rowptr[j + 1]; e += 32) {
    const double* B = Sb + 36 * static_cast<int64_t>(blks[e] & 0x7fffffff);
    double n2 = 0.0;
    for (int t = 0; t < 36; ++t) n2 += B[t] * B[t];
    const double w = sqrt(n2);
    const bool off = cols[e] != j;
    ew[e] = off ? static_cast<float>(w) : 0.0f;
    if (off) {
      sw += w;
      sw2 += n2;
      mw = fmax(mw, w);
      ++deg;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    sw += __shfl_xor_sync(0xffffffffu, sw, o);
    sw2 += __shfl_xor_sync(0xffffffffu, sw2, o);
    mw = fmax(mw, __shfl_xor_sync(0xffffffffu, mw, o));
    deg += __shfl_xor_sync(0xffffffffu, deg, o);
  }
  if (lane == 0) {
    const double* B = Sb + 36 * static_cast<int64_t>(diag[j]);
    int t = 0;
    for (int r = 0; r < 6; ++r)
      for (int c = r + 1; c < 6; ++c) f[t++] = static_cast<float>(B[r * 6 + c]);
    // diagonal of B^-1 by the Cholesky factor (B^-1 = C^-T C^-1)
    double C[36];
    bool ok = true;
    for (int a = 0; a < 36; ++a) C[a] = 0.0;
    for (int c = 0; c < 6 && ok; ++c) {
      double d = B[c * 6 + c];
      for (int k = 0; k < c; ++k) d -= C[c * 6 + k] * C[c * 6 + k];
      if (!(d > 0.0) || !isfinite(d)) { ok = false; break; }
      C[c * 6 + c] = sqrt(d);
      for (int i = c + 1; i < 6; ++i) {
        double v = B[i * 6 + c];
        for (int k = 0; k < c; ++k) v -= C[i * 6 + k] * C[c * 6 + k];
        C[i * 6 + c] = v / C[c * 6 + c];
      }
    }
    double X[36];  // C^-1
    for (int a = 0; a < 36; ++a) X[a] = 0.0;
    if (ok) {
      for (int c = 0; c < 6; ++c) {
        X[c * 6 + c] = 1.0 / C[c * 6 + c];
        for (int i = c + 1; i < 6; ++i) {
          double v = 0.0;
          for (int k = c; k < i; ++k) v -= C[i * 6 + k] * X[k * 6 + c];
          X[i * 6 + c] = v / C[i * 6 + i];
        }
      }
    }
    for (int r = 0; r < 6; ++r) {
      double v = 0.0;
      for (int k = r; k < 6; ++k) v += X[k * 6 + r] * X[k * 6 + r];
      f[15 + r] = ok ? static_cast<float>(log(fmax(v, 1e-30))) : 0.0f;
    }
    f[21] = static_cast<float>(log1p(static_cast<double>(deg)));
    f[22] = static_cast<float>(sw);
    f[23] = static_cast<float>(mw);
    f[24] = static_cast<float>(sqrt(sw2));
    f[25] = static_cast<float>(deg > 0 ? sw / deg : 0.0);
    for (int k = 26; k < F; ++k) f[k] = 0.0f;
  }
  __syncwarp();
}

namespace {

struct NetArgs {
  int nf;
  const int32_t* rowptr;
  const int32_t* cols;
  const int32_t* blks;
  const int32_t* diag;
  const double* Sb;
  const uint16_t* w;  // BF16 parameters
  float* feat;        // nf x F
  float* ew;          // edge weight of every entry
  float* h0;          // nf x H (ping)
  float* h1;          // nf x H (pong)
  float* L;           // nf x 21
};

// Features and the input embedding, one warp per node.
__global__ void __launch_bounds__(kNT) k_net_embed(NetArgs a, const Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  __shared__ float sW[H * F];
  __shared__ float sb[H];
  __shared__ float sf[kNW][F];
  for (int t = threadIdx.x; t < H * F; t += kNT) sW[t] = bf16f(a.w[pcg_off_win() + t]);
  for (int t = threadIdx.x; t < H; t += kNT) sb[t] = bf16f(a.w[pcg_off_bin() + t]);
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j = blockIdx.x * kNW + w; j < a.nf; j += gridDim.x * kNW) {
    pcg_node_features(j, a.rowptr, a.cols, a.blks, a.diag, a.Sb, sf[w], a.ew);
    if (lane == 0)
      for (int k = 0; k < F; ++k) a.feat[static_cast<int64_t>(j) * F + k] = sf[w][k];
    __syncwarp();
    for (int o = lane; o < H; o += 32) {
      float v = sb[o];
      for (int k = 0; k < F; ++k) v = fmaf(sW[o * F + k], sf[w][k], v);
      a.h0[static_cast<int64_t>(j) * H + o] = fmaxf(v, 0.0f);
    }
    __syncwarp();
  }
}

// One message-passing layer (and, for the last, the output head).
__global__ void __launch_bounds__(kNT) k_net_layer(NetArgs a, int layer, const float* hin, float* hout,
                                                   const Ctrl* ctrl) {
  if (skipping(ctrl)) return;
  extern __shared__ float smem[];
  float* sWs = smem;               // H x H
  float* sWm = sWs + H * H;        // H x H
  float* sb = sWm + H * H;         // H
  float* sWo = sb + H;             // 21 x H
  float* sbo = sWo + kPcgOut * H;  // 21
  float* sh = sbo + 32;            // kNW x 2H: own state, message
  const bool last = layer == kPcgLayers - 1;
  for (int t = threadIdx.x; t < H * H; t += kNT) {
    sWs[t] = bf16f(a.w[pcg_off_ws(layer) + t]);
    sWm[t] = bf16f(a.w[pcg_off_wm(layer) + t]);
  }
  for (int t = threadIdx.x; t < H; t += kNT) sb[t] = bf16f(a.w[pcg_off_b(layer) + t]);
  if (last) {
    for (int t = threadIdx.x; t < kPcgOut * H; t += kNT) sWo[t] = bf16f(a.w[pcg_off_wout() + t]);
    for (int t = threadIdx.x; t < kPcgOut; t += kNT) sbo[t] = bf16f(a.w[pcg_off_bout() + t]);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float* hs = sh + w * 2 * H;
  float* ms = hs + H;
  for (int j = blockIdx.x * kNW + w; j < a.nf; j += gridDim.x * kNW) {
    // message: weighted mean of the neighbours' states (fixed entry order)
    float m0 = 0.f, m1 = 0.f, ws = 0.f;
    for (int e = a.rowptr[j]; e < a.rowptr[j + 1]; ++e) {
      const float we = a.ew[e];
      if (we == 0.0f) continue;
      const float* hk = hin + static_cast<int64_t>(a.cols[e]) * H;
      m0 = fmaf(we, hk[lane], m0);
      m1 = fmaf(we, hk[lane + 32], m1);
      ws += we;
    }
    const float inv = ws > 0.f ? 1.0f / ws : 0.0f;
    hs[lane] = hin[static_cast<int64_t>(j) * H + lane];
    hs[lane + 32] = hin[static_cast<int64_t>(j) * H + lane + 32];
    ms[lane] = m0 * inv;
    ms[lane + 32] = m1 * inv;
    __syncwarp();
    float o[2];
    for (int q = 0; q < 2; ++q) {
      const int r = lane + 32 * q;
      float v = sb[r];
      for (int k = 0; k < H; ++k) v = fmaf(sWs[r * H + k], hs[k], v);
      for (int k = 0; k < H; ++k) v = fmaf(sWm[r * H + k], ms[k], v);
      o[q] = hs[r] + fmaxf(v, 0.0f);
    }
    __syncwarp();
    hs[lane] = o[0];
    hs[lane + 32] = o[1];
    __syncwarp();
    if (last) {
      if (lane < kPcgOut) {
        float v = sbo[lane];
        for (int k = 0; k < H; ++k) v = fmaf(sWo[lane * H + k], hs[k], v);
        a.L[static_cast<int64_t>(j) * kPcgOut + lane] = v;
      }
    } else {
      hout[static_cast<int64_t>(j) * H + lane] = o[0];
      hout[static_cast<int64_t>(j) * H + lane + 32] = o[1];
    }
    __syncwarp();
  }
}

constexpr size_t kLayerSmem = sizeof(float) * (2 * H * H + H + kPcgOut * H + 32 + kNW * 2 * H);

NetArgs net_args(const Sizes& s, const Dev& d) {
  NetArgs a;
  a.nf = s.nf;
  a.rowptr = d.pcg_rowptr;
  a.cols = d.pcg_cols;
  a.blks = d.pcg_blks;
  a.diag = d.pcg_diag;
  a.Sb = d.pcg_S;
  a.w = d.pcg_w;
  a.feat = d.pcg_feat;
  a.ew = d.pcg_ew;
  a.h0 = d.pcg_h;
  a.h1 = d.pcg_h + static_cast<int64_t>(s.nf) * H;
  a.L = d.pcg_L;
  return a;
}

}  // namespace

size_t pcg_net_layer_smem() { return kLayerSmem; }

int pcg_net_setup() {
  return raise_dynamic_smem(reinterpret_cast<const void*>(k_net_layer), kLayerSmem) == cudaSuccess ? 0 : -1;
}

int pcg_net_launch_count() { return 1 + kPcgLayers; }

int launch_pcg_net(const Sizes& s, const Dev& d, cudaStream_t st) {
  const NetArgs a = net_args(s, d);
  const int blocks = (s.nf + kNW - 1) / kNW;
  k_net_embed<<<blocks, kNT, 0, st>>>(a, d.ctrl);
  const float* hin = a.h0;
  float* hout = a.h1;
  for (int l = 0; l < kPcgLayers; ++l) {
    k_net_layer<<<blocks, kNT, kLayerSmem, st>>>(a, l, hin, hout, d.ctrl);
    const float* t = hin;
    hin = hout;
    hout = const_cast<float*>(t);
  }
  return 1 + kPcgLayers;
}

}  // namespace sgba
