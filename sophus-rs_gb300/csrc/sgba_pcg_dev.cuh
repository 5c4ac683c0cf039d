// sgba_pcg_dev.cuh -- device code shared by the PCG solver (sgba_pcg.cu) and
// the learned preconditioner's network and training (sgba_pcg_net.cu): the
// 6x6 block preconditioner, the network's parameter layout and node features.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "sgba_internal.h"

namespace sgba {

__device__ __forceinline__ float bf16f(uint16_t u) { return __uint_as_float(static_cast<unsigned>(u) << 16); }

// 6x6 Cholesky B = C C^T (lower, f64); false if a pivot is not positive.
__device__ __forceinline__ bool chol6(const double* B, double* C) {
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
__device__ __forceinline__ void trinv6(const double* C, double* X) {
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

// P_j = Ci^T (I + L L^T) Ci with Ci = C^-1 (C C^T = diagonal block of S~).
// Shared with the training code: the same arithmetic builds the training
// preconditioner.
__device__ __forceinline__ void pcg_precond_block(const double* B, const float* Lrow, double* P, double* Ci) {
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


constexpr int kPcgH = kPcgHidden;
constexpr int kPcgF = kPcgFeat;
// Offsets of the parameter blocks (in elements).
__host__ __device__ constexpr int pcg_off_win() { return 0; }
__host__ __device__ constexpr int pcg_off_bin() { return kPcgH * kPcgF; }
__host__ __device__ constexpr int pcg_off_ws(int l) { return kPcgH * kPcgF + kPcgH + l * (2 * kPcgH * kPcgH + kPcgH); }
__host__ __device__ constexpr int pcg_off_wm(int l) { return pcg_off_ws(l) + kPcgH * kPcgH; }
__host__ __device__ constexpr int pcg_off_b(int l) { return pcg_off_ws(l) + 2 * kPcgH * kPcgH; }
__host__ __device__ constexpr int pcg_off_wout() { return pcg_off_ws(kPcgLayers); }
__host__ __device__ constexpr int pcg_off_bout() { return pcg_off_wout() + kPcgOut * kPcgH; }
static_assert(pcg_off_bout() + kPcgOut == kPcgParams, "parameter layout");

// Node features of free pose j from the Jacobi-scaled blocks.  Also writes
// the edge weight w_jk of every entry of block row j (0 on the diagonal).
__device__ __forceinline__ void pcg_node_features(int j, const int32_t* rowptr, const int32_t* cols, const int32_t* blks,
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
    for (int k = 26; k < kPcgF; ++k) f[k] = 0.0f;
  }
  __syncwarp();
}


}  // namespace sgba
