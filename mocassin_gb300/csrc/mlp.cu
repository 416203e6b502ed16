// mlp.cu -- the learned warm start of the cell update: an MLP from the Jste
// sums of a cell (log10 of the 33 photoionisation and 33 heating sums, of
// sum Jste and of Hden) to log10 Te and log10 of the 40 ionic fractions,
// trained on the GPU on cell states that the cell update produced.
//
// Network: four layers, 80 -> 256 (ReLU) -> 256 (ReLU) -> 256 (ReLU) -> 48
// (padded sizes; 68 features, 41 targets).  Arithmetic: each layer rounds its
// operands to BF16 and accumulates in FP32 (the operand precision of a BF16
// tensor-core product), weights kept in FP32 for Adam.  The prediction over
// a grid runs the four layers on the tensor cores (mlp_fwd_tc_kernel: 0.57
// ms for the 227k cells of a 61^3 grid); training (steps of a few thousand
// rows) runs them on CUDA cores as tiled GEMMs, ~330 kFLOP per row forward.
//
// Kernels
//   mlp_fwd_tc_kernel  the forward layers on tcgen05 (below)
//   mlp_gemm_kernel    C[m][n] = act(b[n] + sum_k A(m,k) B(k,n)) in 64 x 64
//                      tiles, 16-deep K steps through shared memory, 4 x 4
//                      outputs per thread; B is a layer's weights read as
//                      W^T (forward) or W (data gradient, the ReLU mask of
//                      the layer output fused on A)
//   mlp_wgrad_kernel   dW[n][k] += sum_m dZ(m,n) bf16(X(m,k)) in 64 x 64 tiles,
//                      the rows split over blocks (FP32 atomics); the bias
//                      gradient in mlp_bgrad_kernel
//   mlp_loss_kernel    dY = 2 (Y - T) / (B 41) on the 41 targets, sum of squares
//   mlp_adam_kernel    Adam (beta 0.9 / 0.999, eps 1e-8) on the FP32 weights
//   features / apply   the per-cell features from the moments, and the
//                      prediction written into the cell state
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>

#include "mc_device.cuh"
#include "mc_launch.h"
#include "tc_util.cuh"

namespace mcg {

namespace {

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

constexpr int kTM = 64, kTN = 64, kTK = 16;  // GEMM tile: rows, columns, depth

// C[m][n] = act(bias[n] + sum_k A(m,k) B(k,n)), A(m,k) = a[m*lda + k] (zero
// where mask[m*lda + k] <= 0, BF16-rounded if round_a), B(k,n) = bf16 of
// w[n*K + k] (wt: a layer's [N][K] weights, the forward pass) or w[k*N + n]
// (the data gradient through a layer of [K][N] weights).  256 threads.
__global__ void __launch_bounds__(256) mlp_gemm_kernel(int M, int N, int K, const float *a, int lda,
                                                       const float *mask, bool round_a, const float *w, bool wt,
                                                       const float *bias, int act, float *c, int ldc) {
  __shared__ float As[kTK][kTM + 4], Bs[kTK][kTN + 4];
  const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
  const int m0 = blockIdx.x * kTM, n0 = blockIdx.y * kTN;
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
  for (int k0 = 0; k0 < K; k0 += kTK) {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int q = t + 256 * e;
      {  // A: 64 rows x 16 k, k fastest
        const int r = q / kTK, k = q % kTK, m = m0 + r, kk = k0 + k;
        float v = 0.f;
        if (m < M && kk < K) {
          v = a[(size_t)m * lda + kk];
          if (mask && !(mask[(size_t)m * lda + kk] > 0.f)) v = 0.f;
          if (round_a) v = bf16r(v);
        }
        As[k][r] = v;
      }
      if (wt) {  // B(k,n) = w[n][k]: k fastest
        const int n = q / kTK, k = q % kTK, nn = n0 + n, kk = k0 + k;
        Bs[k][n] = nn < N && kk < K ? bf16r(w[(size_t)nn * K + kk]) : 0.f;
      } else {   // B(k,n) = w[k][n]: n fastest
        const int k = q / kTN, n = q % kTN, nn = n0 + n, kk = k0 + k;
        Bs[k][n] = nn < N && kk < K ? bf16r(w[(size_t)kk * N + nn]) : 0.f;
      }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kTK; ++k) {
      float av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = As[k][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bv[j] = Bs[k][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] += av[i] * bv[j];
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + ty * 4 + i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tx * 4 + j;
      if (n >= N) continue;
      float v = acc[i][j] + (bias ? bias[n] : 0.f);
      if (act == 1) v = v > 0.f ? v : 0.f;
      c[(size_t)m * ldc + n] = v;
    }
  }
}

// sum_m dZ(m,n) bf16(X(m,k)), dZ(m,n) = dz[m*N + n] (zero where
// mask[m*N + n] <= 0), over the rows of split blockIdx.z, into P[z][n][k];
// tiles of 64 n x 64 k.  The splits are added in order by
// mlp_grad_reduce_kernel (no atomics), so a training run is reproducible.
__global__ void __launch_bounds__(256) mlp_wgrad_kernel(int M, int N, int K, const float *dz, const float *mask,
                                                        const float *x, float *P, int rows_per_split) {
  __shared__ float Zs[kTK][kTN + 4], Xs[kTK][kTN + 4];
  const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
  const int n0 = blockIdx.x * kTN, k0 = blockIdx.y * kTN;
  const int mb = blockIdx.z * rows_per_split, me = min(M, mb + rows_per_split);
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
  for (int r0 = mb; r0 < me; r0 += kTK) {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int q = t + 256 * e;
      const int r = q / kTN, col = q % kTN, m = r0 + r;
      float zv = 0.f, xv = 0.f;
      if (m < me) {
        const int n = n0 + col, k = k0 + col;
        if (n < N) {
          zv = dz[(size_t)m * N + n];
          if (mask && !(mask[(size_t)m * N + n] > 0.f)) zv = 0.f;
        }
        if (k < K) xv = bf16r(x[(size_t)m * K + k]);
      }
      Zs[r][col] = zv;
      Xs[r][col] = xv;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kTK; ++r) {
      float zv[4], xv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) zv[i] = Zs[r][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) xv[j] = Xs[r][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] += zv[i] * xv[j];
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int n = n0 + ty * 4 + i;
    if (n >= N) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int k = k0 + tx * 4 + j;
      if (k < K) P[((size_t)blockIdx.z * N + n) * K + k] = acc[i][j];
    }
  }
}

// sum_m dZ(m,n) over the rows of block row blockIdx.y into Pb[y][n] (the
// eight warps' sums added in order)
__global__ void mlp_bgrad_kernel(int M, int N, const float *dz, const float *mask, float *Pb) {
  __shared__ float part[8][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int n = blockIdx.x * 32 + lane;
  float acc = 0.f;
  if (n < N)
    for (int m = blockIdx.y * 8 + warp; m < M; m += gridDim.y * 8) {
      float v = dz[(size_t)m * N + n];
      if (mask && !(mask[(size_t)m * N + n] > 0.f)) v = 0.f;
      acc += v;
    }
  part[warp][lane] = acc;
  __syncthreads();
  if (warp == 0 && n < N) {
    float t = 0.f;
    for (int w = 0; w < 8; ++w) t += part[w][lane];
    Pb[(size_t)blockIdx.y * N + n] = t;
  }
}

// dW[i] += sum_z P[z][i] (i < NK) and db[n] += sum_y Pb[y][n], in order
__global__ void mlp_grad_reduce_kernel(int NK, int splits, const float *P, float *dW, int N, int ysplits,
                                       const float *Pb, float *db) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NK + N; i += gridDim.x * blockDim.x) {
    float t = 0.f;
    if (i < NK) {
      for (int z = 0; z < splits; ++z) t += P[(size_t)z * NK + i];
      dW[i] += t;
    } else if (db) {
      const int n = i - NK;
      for (int y = 0; y < ysplits; ++y) t += Pb[(size_t)y * N + n];
      db[n] += t;
    }
  }
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

// per-column sums of the training buffer (FP64) for the normalisation: the
// partial sums of block x go to sum[x * cols + col] and sq[...], added in
// order by the host
__global__ void mlp_stats_kernel(long long n, int cols, const float *a, double *sum, double *sq) {
  __shared__ double ps[8], pq[8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
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
    if (lane == 0) { ps[warp] = s; pq[warp] = s2; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0., t2 = 0.;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { t += ps[w]; t2 += pq[w]; }
      sum[(size_t)blockIdx.x * cols + col] = t;
      sq[(size_t)blockIdx.x * cols + col] = t2;
    }
    __syncthreads();
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

// a cell whose state teaches the model: it has packets and the update
// balanced it (no noTeBal, no noIonBal)
__device__ __forceinline__ bool collect_hit(const float *mom, const int *flags, int c) {
  return mom[c] > 0.f && !(flags[c] & 3);
}

// The training rows are appended in cell order (reproducible): block b owns
// cells [1 + b chunk, 1 + (b+1) chunk), counts its rows first, then writes
// them after the rows of the blocks before it.
__global__ void mlp_collect_count_kernel(int nc, int chunk, const float *mom, const int *flags, unsigned int *cnt) {
  const int c0 = 1 + blockIdx.x * chunk, c1 = min(nc + 1, c0 + chunk);
  unsigned int n = 0;
  for (int t0 = c0; t0 < c1; t0 += blockDim.x) {
    const int c = t0 + threadIdx.x;
    n += __syncthreads_count(c < c1 && collect_hit(mom, flags, c));
  }
  if (threadIdx.x == 0) cnt[blockIdx.x] = n;
}

// writes (features, targets) of the block's hit cells at count + (rows of
// the blocks before) + (rank within the block); rows past cap are dropped
__global__ void mlp_collect_kernel(int nc, int chunk, const float *mom, long long ms, const double *hden,
                                   const double *te, const double *X, const int *flags, long long cap,
                                   const unsigned long long *count, const unsigned int *cnt, float *xs, float *ts) {
  __shared__ unsigned int wsum[32];
  __shared__ unsigned long long sbase;
  if (threadIdx.x == 0) {
    unsigned long long b = *count;
    for (int j = 0; j < (int)blockIdx.x; ++j) b += cnt[j];
    sbase = b;
  }
  __syncthreads();
  unsigned long long base = sbase;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int c0 = 1 + blockIdx.x * chunk, c1 = min(nc + 1, c0 + chunk);
  for (int t0 = c0; t0 < c1; t0 += blockDim.x) {
    const int c = t0 + threadIdx.x;
    const bool hit = c < c1 && collect_hit(mom, flags, c);
    const unsigned int bal = __ballot_sync(0xffffffffu, hit);
    if (lane == 0) wsum[warp] = __popc(bal);
    __syncthreads();
    unsigned int off = __popc(bal & ((1u << lane) - 1u)), tot = 0;
    for (int w = 0; w < nw; ++w) {
      const unsigned int v = wsum[w];
      off += w < warp ? v : 0u;
      tot += v;
    }
    const unsigned long long k = base + off;
    if (hit && (long long)k < cap) {
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
    base += tot;
    __syncthreads();  // wsum is reused by the next tile
  }
}

// count += the rows of every block
__global__ void mlp_collect_total_kernel(int nblocks, const unsigned int *cnt, unsigned long long *count) {
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int j = 0; j < nblocks; ++j) t += cnt[j];
    *count += t;
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

// ---- the forward layers on tcgen05 ------------------------------------
// out[m][n] = act(bias[n] + sum_k bf16(a[m*lda + k]) bf16(w[n*K + k])), the
// same products as mlp_gemm_kernel's forward pass, with the sums in the
// tensor cores' FP32 accumulators.  A persistent CTA of 256 threads per SM
// keeps the layer's BF16 weights (N x K, K-major core matrices) in shared
// memory and takes 128-row tiles of A in turn: the threads convert the
// tile's FP32 rows (float4 loads, a warp covering 8 rows x 32 k so both the
// loads and the 16-byte shared stores are conflict-free) into the K-major
// BF16 layout, one thread issues the K / 16 MMAs (128 x N x 16) into one of
// two TMEM accumulators, and while they run the threads drain the other
// accumulator (the previous tile) through tcgen05.ld, bias, ReLU and the
// stores.  Every mbarrier wait is bounded; a wait that gives up sets
// g_mlp_tc_error and ends the CTA's loop.
constexpr int kFwdM = 128, kFwdThreads = 256;

__device__ int g_mlp_tc_error;

__device__ __forceinline__ uint32_t mlp_pack_bf16x2(float a, float b) {
  return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(a)) |
         ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(b)) << 16);
}

// rows [r0, r0 + nrows) x K of src (row stride ld, rows >= rmax read as 0)
// into BF16 K-major core matrices at dst
__device__ __forceinline__ void mlp_stage_rows(unsigned char *dst, const float *src, long long ld, int r0, int nrows,
                                               int rmax, int K, int warp, int lane) {
  const int kgroups = (K + 31) / 32, total = (nrows / 8) * kgroups;
  const int rr = lane >> 2, kc = lane & 3;
  constexpr int kU = 8;  // warp steps whose loads are in flight together
  for (int it0 = warp; it0 < total; it0 += kU * (kFwdThreads / 32)) {
    float4 v[kU][2];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int it = it0 + u * (kFwdThreads / 32);
      const int r = (it / kgroups) * 8 + rr, k = (it % kgroups) * 32 + kc * 8;
      v[u][0] = v[u][1] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (it < total && r0 + r < rmax && k < K) {
        const float4 *p = (const float4 *)(src + (long long)(r0 + r) * ld + k);
        v[u][0] = __ldg(p);
        v[u][1] = __ldg(p + 1);
      }
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int it = it0 + u * (kFwdThreads / 32);
      const int r = (it / kgroups) * 8 + rr, k = (it % kgroups) * 32 + kc * 8;
      if (it < total && k < K)
        *(uint4 *)(dst + kmajor_off(r, k, K)) =
            make_uint4(mlp_pack_bf16x2(v[u][0].x, v[u][0].y), mlp_pack_bf16x2(v[u][0].z, v[u][0].w),
                       mlp_pack_bf16x2(v[u][1].x, v[u][1].y), mlp_pack_bf16x2(v[u][1].z, v[u][1].w));
    }
  }
}

__global__ void __launch_bounds__(kFwdThreads, 1) mlp_fwd_tc_kernel(int M, int N, int K, const float *a, int lda,
                                                                      const float *w, const float *bias, int act,
                                                                      float *out, int ldo, int ncols) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char *sW = sm, *sA = sm + (size_t)N * K * 2;
  uint64_t *bar = (uint64_t *)(sA + (size_t)kFwdM * K * 2);  // [2]: the accumulators' MMAs done
  uint32_t *tslot = (uint32_t *)(bar + 2);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(1));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar + 1)), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  // the layer's weights, once
  mlp_stage_rows(sW, w, K, 0, (N + 7) / 8 * 8, N, K, warp, lane);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  const uint32_t idesc = mma_idesc(kFwdM, N);
  const uint32_t lbo = 128, sbo = (uint32_t)(K / 8) * 128;
  const int ntiles = (M + kFwdM - 1) / kFwdM;
  uint32_t phase[2] = {0u, 0u};
  bool failed = false;
  int prev = -1;  // the tile whose accumulator is still to be drained
  int i = 0;
  auto drain = [&](int tile, int buf) {
    // warp w: TMEM lanes 32 (w % 4) .., columns of half w / 4
    const int q = warp & 3, half = warp >> 2;
    const int r = tile * kFwdM + 32 * q + lane;
    const int c_lo = half * ((N + 63) / 64) * 32, c_hi = min(N, c_lo + ((N + 63) / 64) * 32);
    for (int c0 = c_lo; c0 < c_hi; c0 += 32) {
      uint32_t v[32];
      tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(buf * (ncols / 2) + c0), v);
      if (r < M) {
        float *o = out + (long long)r * ldo;
#pragma unroll
        for (int u = 0; u < 32; u += 4) {
          if (c0 + u >= N) break;
          float x[4];
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            float t = __uint_as_float(v[u + e]) + (bias ? __ldg(bias + c0 + u + e) : 0.f);
            x[e] = act == 1 ? (t > 0.f ? t : 0.f) : t;
          }
          *(float4 *)(o + c0 + u) = make_float4(x[0], x[1], x[2], x[3]);
        }
      }
    }
  };
  for (int tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x, ++i) {
    const int buf = i & 1;
    if (i > 0) {
      // the A buffer is free once the previous tile's MMAs are done
      const bool ok = mbar_wait(smem_addr(bar + (buf ^ 1)), phase[buf ^ 1]);
      phase[buf ^ 1] ^= 1u;
      if (__syncthreads_or(!ok)) { failed = true; break; }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    }
    mlp_stage_rows(sA, a, lda, tile * kFwdM, kFwdM, M, K, warp, lane);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t aa = smem_addr(sA), ww = smem_addr(sW), d = tmem + (uint32_t)(buf * (ncols / 2));
      for (int st = 0; st < K / 16; ++st) {
        const uint32_t ko = (uint32_t)st * 256;
        umma_bf16(d, smem_desc(aa + ko, lbo, sbo), smem_desc(ww + ko, lbo, sbo), idesc, st > 0 ? 1u : 0u);
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_addr(bar + buf))
                   : "memory");
    }
    // the previous tile's accumulator (its MMAs were waited for above)
    if (prev >= 0) drain(prev, buf ^ 1);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    prev = tile;
  }
  if (!failed && prev >= 0) {
    const int buf = (i - 1) & 1;
    const bool ok = mbar_wait(smem_addr(bar + buf), phase[buf]);
    if (__syncthreads_or(!ok)) failed = true;
    else {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      drain(prev, buf);
    }
  }
  if (failed && tid == 0) atomicExch(&g_mlp_tc_error, 1);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

size_t mlp_fwd_smem(int N, int K) { return (size_t)N * K * 2 + (size_t)kFwdM * K * 2 + 64; }

}  // namespace

// the forward layers on tcgen05 (N, K multiples of 16, N <= 256, K <= 256,
// lda and ldo multiples of 4); the kernel's shared memory is set by
// mlp_prepare(), before any capture
cudaError_t launch_mlp_forward_tc(int M, int N, int K, const float *a, int lda, const float *w, const float *bias,
                                  int act, float *c, int ldc, int num_sms, cudaStream_t s) {
  if (M < 1 || N < 16 || N > 256 || N % 16 || K < 16 || K > 256 || K % 16 || lda % 4 || ldc % 4)
    return cudaErrorInvalidValue;
  int ncols = 32;
  while (ncols < 2 * N) ncols <<= 1;
  const int ntiles = (M + kFwdM - 1) / kFwdM;
  const int blocks = ntiles < num_sms ? ntiles : num_sms;
  // at least 116 KB of shared memory: one CTA per SM, so the TMEM columns of
  // co-resident CTAs never have to wait for each other
  size_t sh = mlp_fwd_smem(N, K);
  if (sh < 116 * 1024) sh = 116 * 1024;
  mlp_fwd_tc_kernel<<<blocks, kFwdThreads, sh, s>>>(M, N, K, a, lda, w, bias, act, c, ldc, ncols);
  return cudaGetLastError();
}

int mlp_tc_take_error() {
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_mlp_tc_error, sizeof v) != cudaSuccess) return -1;
  if (v) {
    const int z = 0;
    cudaMemcpyToSymbol(g_mlp_tc_error, &z, sizeof z);
  }
  return v;
}

cudaError_t launch_mlp_gemm(int M, int N, int K, const float *a, int lda, const float *mask, bool round_a,
                            const float *w, bool wt, const float *bias, int act, float *c, int ldc, cudaStream_t s) {
  if (M < 1 || N < 1 || K < 1) return cudaErrorInvalidValue;
  mlp_gemm_kernel<<<dim3((M + kTM - 1) / kTM, (N + kTN - 1) / kTN), 256, 0, s>>>(M, N, K, a, lda, mask, round_a, w,
                                                                                wt, bias, act, c, ldc);
  return cudaGetLastError();
}

// row splits of the weight gradient: enough to fill the SMs twice, at least
// 64 rows each; the rows per split (a multiple of kTK) in *per
static int wgrad_splits(int M, int N, int K, int num_sms, int *per) {
  const int tiles = ((N + kTN - 1) / kTN) * ((K + kTN - 1) / kTN);
  int splits = std::max(1, std::min((M + 63) / 64, (2 * num_sms + tiles - 1) / tiles));
  *per = ((M + splits - 1) / splits + kTK - 1) / kTK * kTK;
  return (M + *per - 1) / *per;
}
static int bgrad_splits(int M) { return std::max(1, std::min(64, (M + 255) / 256)); }

size_t mlp_wgrad_scratch_floats(int M, int N, int K, int num_sms) {
  int per = 0;
  return (size_t)wgrad_splits(M, N, K, num_sms, &per) * N * K + (size_t)bgrad_splits(M) * N;
}

cudaError_t launch_mlp_wgrad(int M, int N, int K, const float *dz, const float *mask, const float *x, float *dW,
                             float *db, float *scratch, size_t scratch_floats, int num_sms, cudaStream_t s) {
  if (M < 1 || N < 1 || K < 1) return cudaErrorInvalidValue;
  if (!scratch || scratch_floats < mlp_wgrad_scratch_floats(M, N, K, num_sms)) return cudaErrorInvalidValue;
  int per = 0;
  const int splits = wgrad_splits(M, N, K, num_sms, &per), ys = bgrad_splits(M);
  float *P = scratch, *Pb = scratch + (size_t)splits * N * K;
  mlp_wgrad_kernel<<<dim3((N + kTN - 1) / kTN, (K + kTN - 1) / kTN, splits), 256, 0, s>>>(M, N, K, dz, mask, x, P,
                                                                                          per);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (db) {
    mlp_bgrad_kernel<<<dim3((N + 31) / 32, ys), 256, 0, s>>>(M, N, dz, mask, Pb);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  const int n = N * K + N;
  mlp_grad_reduce_kernel<<<std::min((n + 255) / 256, num_sms * 4), 256, 0, s>>>(N * K, splits, P, dW, N, ys, Pb, db);
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
  return raise_smem_limit((const void *)mlp_fwd_tc_kernel, (int)mlp_fwd_smem(256, 256));
}

cudaError_t launch_mlp_stats(long long n, int cols, const float *a, double *sum, double *sq, cudaStream_t s) {
  mlp_stats_kernel<<<dim3(kMlpStatBlocks, cols), 256, 0, s>>>(n, cols, a, sum, sq);
  return cudaGetLastError();
}

int mlp_collect_blocks(int num_sms) { return num_sms * 4; }

cudaError_t launch_mlp_collect(int nc, const float *mom, long long ms, const double *hden, const double *te,
                               const double *X, const int *flags, long long cap, unsigned long long *count, float *xs,
                               float *ts, unsigned int *blk_counts, int num_sms, cudaStream_t s) {
  const int nb = mlp_collect_blocks(num_sms);
  const int chunk = (nc + nb - 1) / nb;
  if (nc < 1) return cudaSuccess;
  mlp_collect_count_kernel<<<nb, 256, 0, s>>>(nc, chunk, mom, flags, blk_counts);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  mlp_collect_kernel<<<nb, 256, 0, s>>>(nc, chunk, mom, ms, hden, te, X, flags, cap, count, blk_counts, xs, ts);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  mlp_collect_total_kernel<<<1, 32, 0, s>>>(nb, blk_counts, count);
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
