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

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "sgba_internal.h"
#include "sgba_pcg_dev.cuh"

namespace sgba {

namespace {

constexpr int kNT = 256;  // threads per CTA: one warp per node
constexpr int kNW = kNT / 32;
constexpr int H = kPcgHidden;
constexpr int F = kPcgFeat;

__device__ __forceinline__ bool skipping(const Ctrl* c) { return c->done != 0 || c->skip != 0; }

}  // namespace

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


// ===========================================================================
// Training: reduced systems S~ x* = b~ (Jacobi-scaled) with their exact
// solutions, loss, gradients by hand-written backward kernels, Adam.
//
// Loss of one system: the energy-norm error left by one preconditioned step
// of optimal length from x = 0 (the first step of PCG; invariant to scaling P,
// as PCG is):
//   y = P b~,  N = y^T b~,  Q = y^T S~ y,  den = x*^T b~,
//   loss = min_a |x* - a y|_S~^2 / den = 1 - N^2 / (den Q)
// P = blockdiag(P_j), P_j = Ci_j^T (I + L_j L_j^T) Ci_j.  Backward:
//   g = dloss/dy = (2 N / (den Q)) (a* S~ y - b~),  a* = N / Q,
//   dloss/dP_j = g_j b_j^T,  dloss/dM_j = Ci_j G_j Ci_j^T,
//   dloss/dL_j = (Gm_j + Gm_j^T) L_j,
// then through the head, the message-passing layers (relu, the weighted
// mean of the neighbours) and the embedding.  The forward arithmetic is the
// inference kernels' (same BF16 weights, same FP32 operation order); the
// gradients are FP32 and update the FP32 master weights (Adam).  Every
// reduction runs in a fixed order: training is bit-reproducible.
// ===========================================================================

namespace {

constexpr int kTT = 256;

struct TrainArgs {
  int nf;
  const int32_t* rowptr;
  const int32_t* cols;
  const int32_t* blks;
  const int32_t* diag;
  const double* Sb;
  const double* b;
  const double* xs;
  const uint16_t* w;  // BF16 weights (forward and data gradients)
  float* feat;        // nf x F
  float* ew;          // nnzb
  float* wsum;        // nf
  float* Hs;          // (kPcgLayers + 1) x nf x H
  float* Ms;          // kPcgLayers x nf x H
  float* Us;          // kPcgLayers x nf x H (pre-activations)
  float* L;           // nf x 21
  double* P;          // nf x 36
  double* Ci;         // nf x 36
  double* e;          // n6: y = P b~
  double* Se;         // n6
  double* loss_part;  // per CTA
  float* dL;          // nf x 21
  float* dHa;         // nf x H
  float* dHb;         // nf x H
  float* dU;          // nf x H
  float* dM;          // nf x H
  float* grad;        // kPcgParams (accumulated)
};

__global__ void __launch_bounds__(kTT) k_tr_features(TrainArgs a) {
  __shared__ float sf[kTT / 32][F];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j = blockIdx.x * (kTT / 32) + w; j < a.nf; j += gridDim.x * (kTT / 32)) {
    pcg_node_features(j, a.rowptr, a.cols, a.blks, a.diag, a.Sb, sf[w], a.ew);
    if (lane == 0) {
      for (int k = 0; k < F; ++k) a.feat[static_cast<int64_t>(j) * F + k] = sf[w][k];
      float ws = 0.f;  // the inference kernel's order
      for (int e = a.rowptr[j]; e < a.rowptr[j + 1]; ++e)
        if (a.ew[e] != 0.0f) ws += a.ew[e];
      a.wsum[j] = ws;
    }
    __syncwarp();
  }
}

__global__ void k_tr_embed(TrainArgs a) {
  const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (t >= static_cast<int64_t>(a.nf) * H) return;
  const int64_t j = t / H;
  const int o = static_cast<int>(t % H);
  float v = bf16f(a.w[pcg_off_bin() + o]);
  for (int k = 0; k < F; ++k) v = fmaf(bf16f(a.w[pcg_off_win() + o * F + k]), a.feat[j * F + k], v);
  a.Hs[t] = fmaxf(v, 0.0f);
}

__global__ void k_tr_message(TrainArgs a, int l) {
  const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (t >= static_cast<int64_t>(a.nf) * H) return;
  const int j = static_cast<int>(t / H);
  const int o = static_cast<int>(t % H);
  const float* Hl = a.Hs + static_cast<int64_t>(l) * a.nf * H;
  float m = 0.f, ws = 0.f;
  for (int e = a.rowptr[j]; e < a.rowptr[j + 1]; ++e) {
    const float we = a.ew[e];
    if (we == 0.0f) continue;
    m = fmaf(we, Hl[static_cast<int64_t>(a.cols[e]) * H + o], m);
    ws += we;
  }
  const float inv = ws > 0.f ? 1.0f / ws : 0.0f;
  a.Ms[static_cast<int64_t>(l) * a.nf * H + t] = m * inv;
}

__global__ void k_tr_layer(TrainArgs a, int l) {
  const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (t >= static_cast<int64_t>(a.nf) * H) return;
  const int64_t j = t / H;
  const int o = static_cast<int>(t % H);
  const float* Hl = a.Hs + static_cast<int64_t>(l) * a.nf * H;
  const float* Ml = a.Ms + static_cast<int64_t>(l) * a.nf * H;
  float v = bf16f(a.w[pcg_off_b(l) + o]);
  for (int k = 0; k < H; ++k) v = fmaf(bf16f(a.w[pcg_off_ws(l) + o * H + k]), Hl[j * H + k], v);
  for (int k = 0; k < H; ++k) v = fmaf(bf16f(a.w[pcg_off_wm(l) + o * H + k]), Ml[j * H + k], v);
  a.Us[static_cast<int64_t>(l) * a.nf * H + t] = v;
  a.Hs[static_cast<int64_t>(l + 1) * a.nf * H + t] = Hl[t] + fmaxf(v, 0.0f);
}

__global__ void k_tr_head(TrainArgs a) {
  const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (t >= static_cast<int64_t>(a.nf) * kPcgOut) return;
  const int64_t j = t / kPcgOut;
  const int o = static_cast<int>(t % kPcgOut);
  const float* Hl = a.Hs + static_cast<int64_t>(kPcgLayers) * a.nf * H;
  float v = bf16f(a.w[pcg_off_bout() + o]);
  for (int k = 0; k < H; ++k) v = fmaf(bf16f(a.w[pcg_off_wout() + o * H + k]), Hl[j * H + k], v);
  a.L[t] = v;
}

// P_j, Ci_j and y_j = P_j b_j.
__global__ void k_tr_precond(TrainArgs a) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.nf) return;
  double* P = a.P + 36 * static_cast<int64_t>(j);
  pcg_precond_block(a.Sb + 36 * static_cast<int64_t>(a.diag[j]), a.L + kPcgOut * static_cast<int64_t>(j), P,
                    a.Ci + 36 * static_cast<int64_t>(j));
  for (int r = 0; r < 6; ++r) {
    double y = 0.0;
    for (int c = 0; c < 6; ++c) y += P[r * 6 + c] * a.b[6 * j + c];
    a.e[6 * j + r] = y;
  }
}

// Se = S~ y (FP64, warp per block row) and per-CTA partials of y . S~ y and
// y . b~ (slots 2 * block, 2 * block + 1).
__global__ void __launch_bounds__(kTT) k_tr_matvec(TrainArgs a) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double part = 0.0, partn = 0.0;
  for (int j = blockIdx.x * (kTT / 32) + w; j < a.nf; j += gridDim.x * (kTT / 32)) {
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int e = a.rowptr[j] + lane; e < a.rowptr[j + 1]; e += 32) {
      const int k = a.cols[e];
      const int bi = a.blks[e];
      const double* B = a.Sb + 36 * static_cast<int64_t>(bi & 0x7fffffff);
      for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 6; ++c) acc[r] += (bi < 0 ? B[c * 6 + r] : B[r * 6 + c]) * a.e[6 * k + c];
    }
    for (int r = 0; r < 6; ++r)
      for (int off = 16; off > 0; off >>= 1) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], off);
    if (lane == 0)
      for (int r = 0; r < 6; ++r) {
        a.Se[6 * j + r] = acc[r];
        part += a.e[6 * j + r] * acc[r];
        partn += a.e[6 * j + r] * a.b[6 * j + r];
      }
  }
  __shared__ double sp[2][kTT / 32];
  if (lane == 0) {
    sp[0][w] = part;
    sp[1][w] = partn;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0, tn = 0.0;
    for (int q = 0; q < kTT / 32; ++q) {
      t += sp[0][q];
      tn += sp[1][q];
    }
    a.loss_part[2 * blockIdx.x] = t;
    a.loss_part[2 * blockIdx.x + 1] = tn;
  }
}

// loss[0] = 1 - N^2 / (den Q); loss[1] = Q, loss[2] = N for the backward pass.
__global__ void k_tr_loss(const double* part, int n, double den, double* loss) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double q = 0.0, nn = 0.0;
    for (int i = 0; i < n; ++i) {
      q += part[2 * i];
      nn += part[2 * i + 1];
    }
    loss[0] = (q > 0.0) ? 1.0 - nn * nn / (den * q) : 1.0;
    loss[1] = q;
    loss[2] = nn;
  }
}

// dloss/dL_j (lower-triangular entries).
__global__ void k_tr_dL(TrainArgs a, double den, const double* qn) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.nf) return;
  const double* Ci = a.Ci + 36 * static_cast<int64_t>(j);
  const double q = qn[1], nn = qn[2];
  const double c = (q > 0.0) ? 2.0 * nn / (den * q) : 0.0, astar = (q > 0.0) ? nn / q : 0.0;
  double g[6], bj[6];
  for (int r = 0; r < 6; ++r) {
    bj[r] = a.b[6 * j + r];
    g[r] = c * (astar * a.Se[6 * j + r] - bj[r]);
  }
  // Gm = Ci G Ci^T with G = g b^T: Gm = (Ci g)(Ci b)^T
  double cg[6], cb[6];
  for (int r = 0; r < 6; ++r) {
    double u = 0.0, v = 0.0;
    for (int k = 0; k < 6; ++k) {
      u += Ci[r * 6 + k] * g[k];
      v += Ci[r * 6 + k] * bj[k];
    }
    cg[r] = u;
    cb[r] = v;
  }
  double Lf[36];
  for (int k = 0; k < 36; ++k) Lf[k] = 0.0;
  const float* Lr = a.L + kPcgOut * static_cast<int64_t>(j);
  for (int r = 0, t = 0; r < 6; ++r)
    for (int c = 0; c <= r; ++c, ++t) Lf[r * 6 + c] = Lr[t];
  for (int r = 0, t = 0; r < 6; ++r)
    for (int c = 0; c <= r; ++c, ++t) {
      double v = 0.0;
      for (int k = 0; k < 6; ++k) v += (cg[r] * cb[k] + cb[r] * cg[k]) * Lf[k * 6 + c];
      a.dL[kPcgOut * static_cast<int64_t>(j) + t] = static_cast<float>(v);
    }
}

// out[i, k] += sum_j A[j, i] B[j, k]; with bias: outb[i] += sum_j A[j, i].
__global__ void k_tr_wgrad(int nf, const float* A, int m, const float* B, int n, float* out, float* outb) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m * n) return;
  const int i = t / n, k = t % n;
  float s = 0.f, sb = 0.f;
  for (int j = 0; j < nf; ++j) {
    const float av = A[static_cast<int64_t>(j) * m + i];
    s = fmaf(av, B[static_cast<int64_t>(j) * n + k], s);
    sb += av;
  }
  out[t] += s;
  if (outb && k == 0) outb[i] += sb;
}

// dH (nf x H) = dL W_out
__global__ void k_tr_head_back(TrainArgs a) {
  const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (t >= static_cast<int64_t>(a.nf) * H) return;
  const int64_t j = t / H;
  const int k = static_cast<int>(t % H);
  float v = 0.f;
  for (int o = 0; o < kPcgOut; ++o) v = fmaf(a.dL[j * kPcgOut + o], bf16f(a.w[pcg_off_wout() + o * H + k]), v);
  a.dHa[t] = v;
}

// dU = dH_next * relu'(U)
__global__ void k_tr_du(TrainArgs a, int l, const float* dHn) {
  const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (t >= static_cast<int64_t>(a.nf) * H) return;
  a.dU[t] = a.Us[static_cast<int64_t>(l) * a.nf * H + t] > 0.0f ? dHn[t] : 0.0f;
}

// dM = dU W_msg;  dHp = dH_next + dU W_self
__global__ void k_tr_dm(TrainArgs a, int l, const float* dHn, float* dHp) {
  const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (t >= static_cast<int64_t>(a.nf) * H) return;
  const int64_t j = t / H;
  const int k = static_cast<int>(t % H);
  float vm = 0.f, vs = 0.f;
  for (int o = 0; o < H; ++o) {
    const float du = a.dU[j * H + o];
    vm = fmaf(du, bf16f(a.w[pcg_off_wm(l) + o * H + k]), vm);
    vs = fmaf(du, bf16f(a.w[pcg_off_ws(l) + o * H + k]), vs);
  }
  a.dM[t] = vm;
  dHp[t] = dHn[t] + vs;
}

// dH_l[j] = dHp[j] + sum over neighbours i of (w_ij / wsum_i) dM[i]
__global__ void k_tr_scatter(TrainArgs a, const float* dHp, float* dHl) {
  const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (t >= static_cast<int64_t>(a.nf) * H) return;
  const int j = static_cast<int>(t / H);
  const int k = static_cast<int>(t % H);
  float v = dHp[t];
  for (int e = a.rowptr[j]; e < a.rowptr[j + 1]; ++e) {
    const float we = a.ew[e];
    if (we == 0.0f) continue;
    const int i = a.cols[e];
    const float ws = a.wsum[i];
    if (ws > 0.f) v = fmaf(we * (1.0f / ws), a.dM[static_cast<int64_t>(i) * H + k], v);
  }
  dHl[t] = v;
}

// dpre = dH0 * relu'(H0) (H0 = relu(pre): H0 > 0 <=> pre > 0), in place
__global__ void k_tr_embed_back(TrainArgs a, float* dH0) {
  const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (t >= static_cast<int64_t>(a.nf) * H) return;
  if (!(a.Hs[t] > 0.0f)) dH0[t] = 0.0f;
}

__device__ __forceinline__ uint16_t bf16_rn(float f) {
  unsigned u = __float_as_uint(f);
  u += 0x7fffu + ((u >> 16) & 1u);
  return static_cast<uint16_t>(u >> 16);
}

__global__ void k_tr_adam(int n, float* w, uint16_t* wbf, float* m1, float* m2, float* grad, float scale, float lr,
                          float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g = grad[i] * scale;
  const float m = b1 * m1[i] + (1.0f - b1) * g;
  const float v = b2 * m2[i] + (1.0f - b2) * g * g;
  m1[i] = m;
  m2[i] = v;
  const float wn = w[i] - lr * (m / c1) / (sqrtf(v / c2) + eps);
  w[i] = wn;
  wbf[i] = bf16_rn(wn);
  grad[i] = 0.0f;
}

inline unsigned nblk(int64_t n, int t) { return static_cast<unsigned>((n + t - 1) / t); }

}  // namespace

// ---------------------------------------------------------------- host ----

PcgTrainSet::~PcgTrainSet() {
  cudaSetDevice(device);
  for (auto& s : sys) {
    cudaFree(s.rowptr);
    cudaFree(s.cols);
    cudaFree(s.blks);
    cudaFree(s.diag);
    cudaFree(s.Sb);
    cudaFree(s.Sb2);
    cudaFree(s.b);
    cudaFree(s.xs);
  }
  free_workspace();
}

void PcgTrainSet::free_workspace() {
  for (void* p : ws) cudaFree(p);
  ws.clear();
  cap_nf = 0;
  cap_nnzb = 0;
}

template <class T>
static cudaError_t ws_alloc(PcgTrainSet* t, T** p, size_t n) {
  void* v = nullptr;
  cudaError_t e = cudaMalloc(&v, sizeof(T) * std::max<size_t>(n, 1));
  if (e == cudaSuccess) {
    t->ws.push_back(v);
    *p = static_cast<T*>(v);
  }
  return e;
}

cudaError_t PcgTrainSet::reserve(int nf, int64_t nnzb) {
  if (nf <= cap_nf && nnzb <= cap_nnzb && !ws.empty()) return cudaSuccess;
  free_workspace();
  const size_t n = static_cast<size_t>(nf), nh = n * H;
  cudaError_t e;
  if ((e = ws_alloc(this, &feat, n * F)) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &ew, static_cast<size_t>(nnzb))) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &wsum, n)) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &Hs, (kPcgLayers + 1) * nh)) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &Ms, kPcgLayers * nh)) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &Us, kPcgLayers * nh)) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &L, n * kPcgOut)) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &P, n * 36)) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &Ci, n * 36)) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &evec, 6 * n)) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &Se, 6 * n)) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &loss_part, 2 * 4096)) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &loss, 4)) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &dL, n * kPcgOut)) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &dHa, nh)) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &dHb, nh)) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &dU, nh)) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &dM, nh)) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &dHp, nh)) != cudaSuccess) return e;
  // PCG evaluation of a stored system
  if ((e = ws_alloc(this, &hbuf, 2 * nh)) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &vec, 6 * 6 * n)) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &part, 4 * static_cast<size_t>(kPcgMaxGrid))) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &bar, 4)) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &ctrl, 1)) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &xout, 6 * n)) != cudaSuccess) return e;
  if ((e = ws_alloc(this, &xdd, 12 * n)) != cudaSuccess) return e;
  cap_nf = nf;
  cap_nnzb = nnzb;
  return cudaSuccess;
}

static TrainArgs train_args(PcgTrainSet& t, const PcgSystem& s, const PcgModel& m) {
  TrainArgs a;
  a.nf = s.nf;
  a.rowptr = s.rowptr;
  a.cols = s.cols;
  a.blks = s.blks;
  a.diag = s.diag;
  a.Sb = s.Sb;
  a.b = s.b;
  a.xs = s.xs;
  a.w = m.wbf;
  a.feat = t.feat;
  a.ew = t.ew;
  a.wsum = t.wsum;
  a.Hs = t.Hs;
  a.Ms = t.Ms;
  a.Us = t.Us;
  a.L = t.L;
  a.P = t.P;
  a.Ci = t.Ci;
  a.e = t.evec;
  a.Se = t.Se;
  a.loss_part = t.loss_part;
  a.dL = t.dL;
  a.dHa = t.dHa;
  a.dHb = t.dHb;
  a.dU = t.dU;
  a.dM = t.dM;
  a.grad = m.grad;
  return a;
}

cudaError_t pcg_loss_grad(PcgModel& m, PcgTrainSet& t, int idx, bool backward, double* loss, cudaStream_t st) {
  const PcgSystem& s = t.sys[idx];
  cudaError_t e = t.reserve(s.nf, s.nnzb);
  if (e != cudaSuccess) return e;
  const TrainArgs a = train_args(t, s, m);
  const int64_t nh = static_cast<int64_t>(s.nf) * H;
  const unsigned gw = nblk(s.nf, kTT / 32);
  k_tr_features<<<gw, kTT, 0, st>>>(a);
  k_tr_embed<<<nblk(nh, kTT), kTT, 0, st>>>(a);
  for (int l = 0; l < kPcgLayers; ++l) {
    k_tr_message<<<nblk(nh, kTT), kTT, 0, st>>>(a, l);
    k_tr_layer<<<nblk(nh, kTT), kTT, 0, st>>>(a, l);
  }
  k_tr_head<<<nblk(static_cast<int64_t>(s.nf) * kPcgOut, kTT), kTT, 0, st>>>(a);
  k_tr_precond<<<nblk(s.nf, 128), 128, 0, st>>>(a);
  const unsigned mvb = std::min<unsigned>(gw, 4096);
  k_tr_matvec<<<mvb, kTT, 0, st>>>(a);
  k_tr_loss<<<1, 32, 0, st>>>(t.loss_part, static_cast<int>(mvb), s.den, t.loss);
  if (backward) {
    float* g = m.grad;
    k_tr_dL<<<nblk(s.nf, 128), 128, 0, st>>>(a, s.den, t.loss);
    k_tr_wgrad<<<nblk(kPcgOut * H, 128), 128, 0, st>>>(s.nf, t.dL, kPcgOut, t.Hs + kPcgLayers * nh, H,
                                                       g + pcg_off_wout(), g + pcg_off_bout());
    k_tr_head_back<<<nblk(nh, kTT), kTT, 0, st>>>(a);
    float* dHn = t.dHa;  // gradient w.r.t. H_{l+1}
    float* dHl = t.dHb;
    for (int l = kPcgLayers - 1; l >= 0; --l) {
      k_tr_du<<<nblk(nh, kTT), kTT, 0, st>>>(a, l, dHn);
      k_tr_wgrad<<<nblk(H * H, 128), 128, 0, st>>>(s.nf, t.dU, H, t.Hs + l * nh, H, g + pcg_off_ws(l),
                                                   g + pcg_off_b(l));
      k_tr_wgrad<<<nblk(H * H, 128), 128, 0, st>>>(s.nf, t.dU, H, t.Ms + l * nh, H, g + pcg_off_wm(l), nullptr);
      k_tr_dm<<<nblk(nh, kTT), kTT, 0, st>>>(a, l, dHn, t.dHp);
      k_tr_scatter<<<nblk(nh, kTT), kTT, 0, st>>>(a, t.dHp, dHl);
      std::swap(dHn, dHl);
    }
    k_tr_embed_back<<<nblk(nh, kTT), kTT, 0, st>>>(a, dHn);
    k_tr_wgrad<<<nblk(H * F, 128), 128, 0, st>>>(s.nf, dHn, H, t.feat, F, g + pcg_off_win(), g + pcg_off_bin());
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (loss) {
    if ((e = cudaMemcpyAsync(loss, t.loss, sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t pcg_adam(PcgModel& m, float scale, float lr, float b1, float b2, float eps, cudaStream_t st) {
  m.step += 1;
  const float c1 = 1.0f - std::pow(b1, static_cast<float>(m.step));
  const float c2 = 1.0f - std::pow(b2, static_cast<float>(m.step));
  k_tr_adam<<<nblk(kPcgParams, 256), 256, 0, st>>>(kPcgParams, m.w32, m.wbf, m.m1, m.m2, m.grad, scale, lr, b1, b2,
                                                   eps, c1, c2);
  return cudaGetLastError();
}

cudaError_t pcg_evaluate(const PcgModel* m, PcgTrainSet& t, int idx, int mode, int max_iters, double tol,
                         int* iters, double* relres, int* status, cudaStream_t st) {
  const PcgSystem& s = t.sys[idx];
  cudaError_t e = t.reserve(s.nf, s.nnzb);
  if (e != cudaSuccess) return e;
  int grid = 0;
  if (pcg_setup(s.nf, &grid) != 0 || grid < 1) return cudaErrorNotSupported;
  if (mode == 2 && pcg_net_setup() != 0) return cudaErrorInvalidValue;
  Sizes z;
  std::memset(&z, 0, sizeof(z));
  z.nf = s.nf;
  z.n6 = 6 * s.nf;
  z.nsb = s.nsb;
  z.pcg_mode = mode;
  z.pcg_max_iters = max_iters;
  z.pcg_tol = tol;
  z.pcg_grid = grid;
  z.pcg_nnzb = s.nnzb;
  Dev d;
  d.pcg_rowptr = s.rowptr;
  d.pcg_cols = s.cols;
  d.pcg_blks = s.blks;
  d.pcg_diag = s.diag;
  d.pcg_S = s.Sb;
  d.pcg_S2 = s.Sb2;
  d.pcg_scl = nullptr;  // the stored system is scaled already
  d.rb = const_cast<double*>(s.b);
  d.pcg_P = t.P;
  d.pcg_Cinv = t.Ci;
  d.pcg_vec = t.vec;
  d.pcg_part = t.part;
  d.pcg_bar = t.bar;
  d.pcg_feat = t.feat;
  d.pcg_ew = t.ew;
  d.pcg_h = t.hbuf;
  d.pcg_L = t.L;
  d.pcg_w = m ? m->wbf : nullptr;
  d.x = t.xout;
  d.xdd = t.xdd;
  d.ctrl = t.ctrl;
  if ((e = cudaMemsetAsync(t.ctrl, 0, sizeof(Ctrl), st)) != cudaSuccess) return e;
  launch_pcg_scaled(z, d, st);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  Ctrl c;
  if ((e = cudaMemcpyAsync(&c, t.ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  *iters = c.pcg_iters;
  *relres = c.pcg_relres;
  *status = c.pcg_status;
  return cudaSuccess;
}

}  // namespace sgba
