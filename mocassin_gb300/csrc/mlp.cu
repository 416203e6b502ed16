// mlp.cu -- the learned warm start of the cell update: a small MLP from the
// Jste sums of a cell (log10 of the 33 photoionisation and 33 heating sums,
// of sum Jste and of Hden) to log10 Te and log10 of the 40 ionic fractions,
// trained on the GPU on cell states that the cell update produced.
//
// Network 80 -> 128 (ReLU) -> 128 (ReLU) -> 48 (padded sizes; 68 features,
// 41 targets).  Arithmetic: each layer rounds its inputs and its weights to
// BF16 and accumulates in FP32 (the operand precision of a BF16 tensor-core
// product), weights kept in FP32 for Adam.  The layers run on CUDA cores:
// the whole network is ~66 kFLOP per cell (15 GFLOP for a 61^3 grid, well
// under a millisecond), nothing next to the cell update it warm-starts.
//
// Kernels
//   mlp_dense_kernel   out[m][o] = act(b[o] + sum_i bf16(in[m][i]) bf16(S[i][o]))
//                      for 128 rows per block; S is the layer's weight matrix
//                      staged in shared memory in (input, output) order, so
//                      the same kernel gives the forward pass (S = W^T) and
//                      the data gradient (S = W, inputs dZ, ReLU' fused)
//   mlp_wgrad_kernel   dW[o][i] += sum_m dZ[m][o] bf16(in[m][i]), db[o] += sum dZ
//   mlp_loss_kernel    dY = 2 (Y - T) / (B 41) on the 41 targets, sum of squares
//   mlp_adam_kernel    Adam (beta 0.9 / 0.999, eps 1e-8) on the FP32 weights
//   features / apply   the per-cell features from the moments, and the
//                      prediction written into the cell state
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "mc_device.cuh"
#include "mc_launch.h"

namespace mcg {

namespace {

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

constexpr int kRows = 128;

// act: 0 linear, 1 ReLU.  mask (data gradient): inputs are multiplied by
// (mask[m][i] > 0), the ReLU derivative of the layer output they belong to.
// Block (x, y): rows 128 x .. 128 x + 127, outputs 16 y .. 16 y + 15.
constexpr int kOC = 16;
__global__ void __launch_bounds__(kRows) mlp_dense_kernel(int M, int nin, int nout, const float *in, int ldin,
                                                          const float *mask, const float *W, bool transposed,
                                                          const float *bias, int act, bool round_in, float *out,
                                                          int ldout) {
  extern __shared__ float sh[];
  float *S = sh;                        // [nin][kOC]
  float *X = sh + (size_t)nin * kOC;    // [nin][kRows]
  const int t = threadIdx.x, m = blockIdx.x * kRows + t, o0 = blockIdx.y * kOC;
  // weights: forward S[i][o] = W[o][i] (W is [nout][nin]); data gradient
  // S[i][o] = W[i][o] (W is [nin][nout] = the forward layer's [out][in])
  for (int q = t; q < nin * kOC; q += kRows) {
    const int i = q / kOC, o = o0 + q % kOC;
    S[q] = bf16r(transposed ? W[(size_t)i * nout + o] : W[(size_t)o * nin + i]);
  }
  for (int i = 0; i < nin; ++i) {
    float v = 0.f;
    if (m < M) {
      v = in[(size_t)m * ldin + i];
      if (mask && !(mask[(size_t)m * ldin + i] > 0.f)) v = 0.f;
      if (round_in) v = bf16r(v);
    }
    X[i * kRows + t] = v;
  }
  __syncthreads();
  if (m >= M) return;
  float acc[kOC];
#pragma unroll
  for (int j = 0; j < kOC; ++j) acc[j] = bias ? bias[o0 + j] : 0.f;
  for (int i = 0; i < nin; ++i) {
    const float x = X[i * kRows + t];
    const float *sr = S + (size_t)i * kOC;
#pragma unroll
    for (int j = 0; j < kOC; ++j) acc[j] += x * sr[j];
  }
#pragma unroll
  for (int j = 0; j < kOC; ++j) {
    float v = acc[j];
    if (act == 1) v = v > 0.f ? v : 0.f;
    out[(size_t)m * ldout + o0 + j] = v;
  }
}

// dW[o][i] += sum_m dZ[m][o] * bf16(in[m][i]); db[o] += sum_m dZ[m][o]
__global__ void __launch_bounds__(256) mlp_wgrad_kernel(int M, int nin, int nout, const float *dz, const float *mask,
                                                        const float *in, float *dW, float *db) {
  constexpr int R = 32;
  extern __shared__ float sh[];
  float *Z = sh;                    // [R][nout]
  float *X = sh + R * nout;         // [R][nin]
  const int t = threadIdx.x;
  const int npair = nin * nout;
  const int per = (npair + 255) / 256;  // <= 64
  float acc[64];
  for (int p = 0; p < 64; ++p) acc[p] = 0.f;
  float bacc = 0.f;
  for (int r0 = blockIdx.x * R; r0 < M; r0 += gridDim.x * R) {
    __syncthreads();
    for (int q = t; q < R * nout; q += 256) {
      const int r = q / nout, o = q % nout;
      float v = r0 + r < M ? dz[(size_t)(r0 + r) * nout + o] : 0.f;
      if (mask && r0 + r < M && !(mask[(size_t)(r0 + r) * nout + o] > 0.f)) v = 0.f;
      Z[q] = v;
    }
    for (int q = t; q < R * nin; q += 256) {
      const int r = q / nin, i = q % nin;
      X[q] = r0 + r < M ? bf16r(in[(size_t)(r0 + r) * nin + i]) : 0.f;
    }
    __syncthreads();
    for (int p = 0; p < per; ++p) {
      const int q = p * 256 + t;
      if (q >= npair) break;
      const int o = q / nin, i = q % nin;
      float a = acc[p];
      for (int r = 0; r < R; ++r) a += Z[r * nout + o] * X[r * nin + i];
      acc[p] = a;
    }
    if (t < nout)
      for (int r = 0; r < R; ++r) bacc += Z[r * nout + t];
  }
  for (int p = 0; p < per; ++p) {
    const int q = p * 256 + t;
    if (q < npair) atomicAdd(&dW[q], acc[p]);
  }
  if (t < nout) atomicAdd(&db[t], bacc);
}

// dY[m][o] = 2 (Y - Tn) / (M * nt) for o < nt; loss += sum (Y - Tn)^2
__global__ void mlp_loss_kernel(int M, int nt, int ld, const float *y, const float *tn, float *dy, double *loss) {
  double s = 0.;
  const float k = 2.f / ((float)M * (float)nt);
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < (long long)M * ld;
       q += (long long)gridDim.x * blockDim.x) {
    const int o = (int)(q % ld);
    float g = 0.f;
    if (o < nt) {
      const float d = y[q] - tn[q];
      g = k * d;
      s += (double)d * d;
    }
    dy[q] = g;
  }
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0 && s != 0.) atomicAdd(loss, s);
}

// the step count t lives on the device so that a captured training step can
// be replayed: bias corrections 0.9^t, 0.999^t and the cosine decay of the
// learning rate over the call (to 5 %) are formed here
__global__ void mlp_adam_kernel(int n, float *w, const float *g, float *m1, float *m2, const int *dstep, int step0,
                                int steps, float lr0) {
  const int t = *dstep + 1;
  const float b1t = powf(0.9f, (float)t), b2t = powf(0.999f, (float)t);
  const float lr = lr0 * (0.05f + 0.95f * 0.5f * (1.f + cosf(3.14159265f * (float)(t - 1 - step0) / (float)steps)));
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float a = 0.9f * m1[i] + 0.1f * gi, b = 0.999f * m2[i] + 0.001f * gi * gi;
    m1[i] = a;
    m2[i] = b;
    const float mh = a / (1.f - b1t), vh = b / (1.f - b2t);
    w[i] -= lr * mh / (sqrtf(vh) + 1e-8f);
  }
}

// a minibatch of training rows: row r = the Philox draw of (step, r) modulo n
__global__ void mlp_step_kernel(int *dstep) { *dstep += 1; }

__global__ void mlp_gather_kernel(int B, long long n, uint32_t seed, const int *dstep, const float *xs, const float *ts,
                                  const float *fmean, const float *fstd, const float *tmean, const float *tstd,
                                  float *xb, float *tb) {
  const int step = *dstep;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < B; r += gridDim.x * blockDim.x) {
    const uint4 v = philox4x32_10(make_uint4((uint32_t)r, (uint32_t)step, 0x4d4c50u, 0u), seed, 0x9e3779b9u);
    const long long src = (long long)(((unsigned long long)v.x << 32 | v.y) % (unsigned long long)n);
    for (int i = 0; i < kMlpIn; ++i)
      xb[(size_t)r * kMlpIn + i] = (xs[(size_t)src * kMlpIn + i] - fmean[i]) / fstd[i];
    for (int o = 0; o < kMlpOut; ++o)
      tb[(size_t)r * kMlpOut + o] = (ts[(size_t)src * kMlpOut + o] - tmean[o]) / tstd[o];
  }
}

// per-column sums of the training buffer (FP64) for the normalisation
__global__ void mlp_stats_kernel(long long n, int cols, const float *a, double *sum, double *sq) {
  for (int col = blockIdx.y; col < cols; col += gridDim.y) {
    double s = 0., s2 = 0.;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x) {
      const double v = a[(size_t)r * cols + col];
      s += v;
      s2 += v * v;
    }
    for (int o = 16; o; o >>= 1) {
      s += __shfl_xor_sync(0xffffffffu, s, o);
      s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if ((threadIdx.x & 31) == 0) {
      atomicAdd(&sum[col], s);
      atomicAdd(&sq[col], s2);
    }
  }
}

// features of cell c: log10 of sum Jste, of the 33 photoionisation and 33
// heating sums, of Hden; targets: log10 Te and log10 of the 40 fractions
__device__ __forceinline__ void cell_features(const float *mom, long long ms, int c, const double *hden, float *f) {
  f[0] = log10f(fmaxf(mom[c], 1e-30f));
  for (int b = 0; b < 33; ++b) f[1 + b] = log10f(mom[(size_t)(1 + b) * ms + c] + 1e-20f);
  for (int b = 0; b < 33; ++b) f[34 + b] = log10f(fmaxf(mom[(size_t)(34 + b) * ms + c], 1e-30f));
  f[67] = log10f((float)hden[c]);
  for (int i = 68; i < kMlpIn; ++i) f[i] = 0.f;
}

__device__ __forceinline__ int stage_count(int e) { return e == 0 ? 2 : (e == 1 ? 3 : 7); }

// appends (features, targets) of every hit cell to the training buffer
__global__ void mlp_collect_kernel(int nc, const float *mom, long long ms, const double *hden, const double *te,
                                   const double *X, const int *flags, long long cap, unsigned long long *count,
                                   float *xs, float *ts) {
  for (int c = 1 + blockIdx.x * blockDim.x + threadIdx.x; c <= nc; c += gridDim.x * blockDim.x) {
    // only states the update balanced (no noTeBal, no noIonBal) teach the model
    if (!(mom[c] > 0.f) || (flags[c] & 3)) continue;
    const unsigned long long k = atomicAdd(count, 1ull);
    if ((long long)k >= cap) continue;
    float f[kMlpIn];
    cell_features(mom, ms, c, hden, f);
    for (int i = 0; i < kMlpIn; ++i) xs[k * kMlpIn + i] = f[i];
    float *t = ts + k * kMlpOut;
    t[0] = log10f((float)te[c]);
    int o = 1;
    for (int e = 0; e < 7; ++e)
      for (int s = 1; s <= stage_count(e); ++s) t[o++] = log10f(fmaxf((float)X[((size_t)c * 7 + e) * 8 + s], 1e-20f));
    for (; o < kMlpOut; ++o) t[o] = 0.f;
  }
}

// normalised features of every cell (row c; rows of cells without packets are zero)
__global__ void mlp_infer_features_kernel(int nc, const float *mom, long long ms, const double *hden, const float *fmean,
                                          const float *fstd, float *x) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c <= nc; c += gridDim.x * blockDim.x) {
    float f[kMlpIn];
    const bool hit = c >= 1 && mom[c] > 0.f;
    if (hit) cell_features(mom, ms, c, hden, f);
    for (int i = 0; i < kMlpIn; ++i) x[(size_t)c * kMlpIn + i] = hit ? (f[i] - fmean[i]) / fstd[i] : 0.f;
  }
}

// writes the prediction into the cell state of every hit cell, keeping the
// previous Te, Ne and X for the convergence test of the update and for the
// fallback to the plain solve
__global__ void mlp_apply_kernel(int nc, const float *mom, const float *y, const float *tmean, const float *tstd,
                                 double *te, double *ne, double *X, double *te_prev, double *ne_prev, double *x_prev) {
  for (int c = 1 + blockIdx.x * blockDim.x + threadIdx.x; c <= nc; c += gridDim.x * blockDim.x) {
    double *Xc = X + (size_t)c * 56;
    te_prev[c] = te[c];
    ne_prev[c] = ne[c];
    for (int i = 0; i < 56; ++i) x_prev[(size_t)c * 56 + i] = Xc[i];
    if (!(mom[c] > 0.f)) continue;
    const float *yc = y + (size_t)c * kMlpOut;
    double t = pow(10., (double)(yc[0] * tstd[0] + tmean[0]));
    if (!(t > 100.)) t = 100.;
    if (t > 1.e6) t = 1.e6;
    te[c] = t;
    int o = 1;
    for (int e = 0; e < 7; ++e) {
      const int ns = stage_count(e);
      double v[8], sum = 0.;
      for (int s = 1; s <= ns; ++s, ++o) {
        v[s] = pow(10., (double)(yc[o] * tstd[o] + tmean[o]));
        sum += v[s];
      }
      for (int s = 1; s <= ns; ++s) {
        double x = v[s] / sum;
        if (x > 0.99999) x = 0.99999;
        if (x < 1.e-20) x = 1.e-20;
        Xc[e * 8 + s] = x;
      }
    }
  }
}

}  // namespace

size_t mlp_dense_smem(int nin, int nout) {
  (void)nout;
  return ((size_t)nin * kOC + (size_t)nin * kRows) * sizeof(float);
}

cudaError_t launch_mlp_dense(int M, int nin, int nout, const float *in, int ldin, const float *mask, const float *W,
                             bool transposed, const float *bias, int act, bool round_in, float *out, int ldout,
                             cudaStream_t s) {
  if (nout % 16 != 0 || nin > kMlpHid) return cudaErrorInvalidValue;
  const size_t sh = mlp_dense_smem(nin, nout);  // within the limit mlp_prepare set
  mlp_dense_kernel<<<dim3((M + kRows - 1) / kRows, nout / kOC), kRows, sh, s>>>(M, nin, nout, in, ldin, mask, W,
                                                                                transposed, bias, act, round_in, out,
                                                                                ldout);
  return cudaGetLastError();
}

cudaError_t launch_mlp_wgrad(int M, int nin, int nout, const float *dz, const float *mask, const float *in, float *dW,
                             float *db, int num_sms, cudaStream_t s) {
  if (nin * nout > 64 * 256 || nout > 256) return cudaErrorInvalidValue;
  const size_t sh = (size_t)32 * (nin + nout) * sizeof(float);
  int blocks = (M + 31) / 32;
  if (blocks > num_sms * 2) blocks = num_sms * 2;
  mlp_wgrad_kernel<<<blocks, 256, sh, s>>>(M, nin, nout, dz, mask, in, dW, db);
  return cudaGetLastError();
}

cudaError_t launch_mlp_loss(int M, int nt, int ld, const float *y, const float *tn, float *dy, double *loss,
                            cudaStream_t s) {
  mlp_loss_kernel<<<256, 256, 0, s>>>(M, nt, ld, y, tn, dy, loss);
  return cudaGetLastError();
}

cudaError_t launch_mlp_adam(int n, float *w, const float *g, float *m1, float *m2, const int *dstep, int step0,
                            int steps, float lr, cudaStream_t s) {
  mlp_adam_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, w, g, m1, m2, dstep, step0, steps, lr);
  return cudaGetLastError();
}

cudaError_t launch_mlp_step(int *dstep, cudaStream_t s) {
  mlp_step_kernel<<<1, 1, 0, s>>>(dstep);
  return cudaGetLastError();
}

cudaError_t launch_mlp_gather(int B, long long n, uint32_t seed, const int *dstep, const float *xs, const float *ts,
                              const float *fmean, const float *fstd, const float *tmean, const float *tstd, float *xb,
                              float *tb, cudaStream_t s) {
  mlp_gather_kernel<<<(B + 255) / 256, 256, 0, s>>>(B, n, seed, dstep, xs, ts, fmean, fstd, tmean, tstd, xb, tb);
  return cudaGetLastError();
}

cudaError_t mlp_prepare() {
  return cudaFuncSetAttribute(mlp_dense_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)mlp_dense_smem(kMlpHid, kMlpHid));
}

cudaError_t launch_mlp_stats(long long n, int cols, const float *a, double *sum, double *sq, cudaStream_t s) {
  mlp_stats_kernel<<<dim3(64, cols), 256, 0, s>>>(n, cols, a, sum, sq);
  return cudaGetLastError();
}

cudaError_t launch_mlp_collect(int nc, const float *mom, long long ms, const double *hden, const double *te,
                               const double *X, const int *flags, long long cap, unsigned long long *count, float *xs,
                               float *ts, int num_sms, cudaStream_t s) {
  mlp_collect_kernel<<<num_sms * 4, 256, 0, s>>>(nc, mom, ms, hden, te, X, flags, cap, count, xs, ts);
  return cudaGetLastError();
}

cudaError_t launch_mlp_infer_features(int nc, const float *mom, long long ms, const double *hden, const float *fmean,
                                      const float *fstd, float *x, int num_sms, cudaStream_t s) {
  mlp_infer_features_kernel<<<num_sms * 4, 256, 0, s>>>(nc, mom, ms, hden, fmean, fstd, x);
  return cudaGetLastError();
}

cudaError_t launch_mlp_apply(int nc, const float *mom, const float *y, const float *tmean, const float *tstd, double *te,
                             double *ne, double *X, double *te_prev, double *ne_prev, double *x_prev, int num_sms,
                             cudaStream_t s) {
  mlp_apply_kernel<<<num_sms * 4, 256, 0, s>>>(nc, mom, y, tmean, tstd, te, ne, X, te_prev, ne_prev, x_prev);
  return cudaGetLastError();
}

}  // namespace mcg
