// cellupdate.cu -- launchers of the per-cell gas update (cellupdate.cuh),
// the FP64 instantiation (compiled with -fmad=false, host code with
// -ffp-contract=off, so the spline tables and the kernel round like the FP64
// oracle), the update statistics and the opacity-species kernel.
#include "cellupdate.cuh"

namespace mcg {

namespace {

__global__ void update_stats_kernel(int nc, const int *conv, const int *niter, const int *flags, const double *dte,
                                    UpdStatsDev *s) {
  unsigned long long hit = 0, cv = 0, nte = 0, nio = 0, it = 0, small = 0, fb = 0;
  double dmax = 0.;
  for (int c = 1 + blockIdx.x * blockDim.x + threadIdx.x; c <= nc; c += gridDim.x * blockDim.x) {
    if (dte[c] < 0.) continue;
    ++hit;
    cv += conv[c];
    nte += flags[c] & 1;
    nio += (flags[c] >> 1) & 1;
    fb += (flags[c] >> 2) & 1;
    it += niter[c];
    small += dte[c] < 0.01;
    dmax = fmax(dmax, dte[c]);
  }
  for (int o = 16; o; o >>= 1) {
    hit += __shfl_xor_sync(0xffffffffu, hit, o);
    cv += __shfl_xor_sync(0xffffffffu, cv, o);
    nte += __shfl_xor_sync(0xffffffffu, nte, o);
    nio += __shfl_xor_sync(0xffffffffu, nio, o);
    it += __shfl_xor_sync(0xffffffffu, it, o);
    small += __shfl_xor_sync(0xffffffffu, small, o);
    fb += __shfl_xor_sync(0xffffffffu, fb, o);
    dmax = fmax(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&s->hit, hit);
    atomicAdd(&s->converged, cv);
    atomicAdd(&s->no_te, nte);
    atomicAdd(&s->no_ion, nio);
    atomicAdd(&s->iters, it);
    atomicAdd(&s->small, small);
    atomicAdd(&s->fallback, fb);
    atomicMax(&s->dmax_bits, (unsigned long long)__double_as_longlong(dmax));
  }
}

// den[k][cell] = X(e_k, s_k) abund(e_k) Hden(cell) for the opacity rows
__global__ void species_kernel(int nc, int nsp, const int *sp_e, const int *sp_s, const double *X, const double *ab,
                               const double *hden, float *den) {
  const int nc1 = nc + 1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (long long)nsp * nc1;
       i += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(i / nc1), c = (int)(i % nc1);
    const int e = sp_e[k];
    den[i] = c == 0 ? 0.f : (float)(X[((size_t)c * kNE + e) * kNX + sp_s[k]] * ab[e] * hden[c]);
  }
}

// the grains' rows of the opacity rebuild (iteration_mod.f90:193-210):
// sublimated sizes drop out
__global__ void grain_density_kernel(int nc1, int nsizes, const float *weight, const float *ndust, const float *tdust,
                                     float t_sub, float *den) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (long long)nsizes * nc1;
       i += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(i / nc1), c = (int)(i % nc1);
    const bool keep = !tdust || tdust[(size_t)(1 + k) * nc1 + c] < t_sub;
    den[i] = c == 0 || !keep ? 0.f : weight[k] * ndust[c];
  }
}

}  // namespace

cudaError_t launch_grain_density(int nc1, int nsizes, const float *weight, const float *ndust, const float *tdust,
                                 float t_sub, float *den, int num_sms, cudaStream_t stream) {
  grain_density_kernel<<<num_sms * 4, 256, 0, stream>>>(nc1, nsizes, weight, ndust, tdust, t_sub, den);
  return cudaGetLastError();
}

cudaError_t launch_cell_update(const UpdArgs &a, int fp32, void *scratch, int num_sms, cudaStream_t stream) {
  if (fp32) return launch_cell_update_fp32(a, scratch, num_sms, stream);
  const int cells = a.nc;
  int blocks = (cells + kW - 1) / kW;
  if (blocks > num_sms * 16) blocks = num_sms * 16;
  if (blocks < 1) blocks = 1;
  // grains: each warp stages its cell's photon flux per bin in shared memory
  const size_t sh = a.g.nsizes > 0 ? (size_t)kW * a.g.nb * sizeof(double) : 0;
  if (sh > 48 * 1024) {
    cudaError_t e = raise_smem_limit((const void *)cell_update_kernel<double, false>, sh);
    if (e != cudaSuccess) return e;
  }
  cell_update_kernel<double, false><<<blocks, kW * 32, sh, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_update_stats(int nc, const int *conv, const int *niter, const int *flags, const double *dte,
                                UpdStatsDev *s, int num_sms, cudaStream_t stream) {
  update_stats_kernel<<<num_sms, 256, 0, stream>>>(nc, conv, niter, flags, dte, s);
  return cudaGetLastError();
}

cudaError_t launch_species(int nc, int nsp, const int *sp_e, const int *sp_s, const double *X, const double *ab,
                           const double *hden, float *den, int num_sms, cudaStream_t stream) {
  species_kernel<<<num_sms * 4, 256, 0, stream>>>(nc, nsp, sp_e, sp_s, X, ab, hden, den);
  return cudaGetLastError();
}

// natural cubic-spline second derivatives (spline with yp1 = ypn = 1e30,
// interpolation_mod.f90:182-253), the same operations as the oracle's
void spline_natural(const double *x, const double *y, int n, double *y2) {
  double u[kNT];
  y2[0] = 0.;
  u[0] = 0.;
  for (int m = 1; m < n - 1; ++m) {
    const double sig = (x[m] - x[m - 1]) / (x[m + 1] - x[m - 1]);
    const double p = sig * y2[m - 1] + 2.;
    y2[m] = (sig - 1.) / p;
    double um = y[m + 1];
    um = um - y[m];
    um = um / (x[m + 1] - x[m]);
    um = um - (y[m] - y[m - 1]) / (x[m] - x[m - 1]);
    u[m] = (6. * um / (x[m + 1] - x[m - 1]) - sig * u[m - 1]) / p;
  }
  y2[n - 1] = (0. - 0. * u[n - 2]) / (0. * y2[n - 2] + 1.);
  for (int m = n - 2; m >= 0; --m) y2[m] = y2[m] * y2[m + 1] + u[m];
}

}  // namespace mcg
