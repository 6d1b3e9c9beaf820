// FP64 reductions on the device state: cem_error norms, field energy and the
// blow-up check.  Partial results per CTA are summed on the host in CTA order,
// so every result is deterministic run to run.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "nekgpu_internal.h"

namespace nekgpu {

namespace {

constexpr int kRedBlocks = 512;
constexpr int kRedThreads = 256;

// per CTA: for each of the 6 components, sum err*bm1*err and max|err|
// (cem_error, src/cem_common.F:1335-1355)
__global__ void k_norms(const double* __restrict__ u, const double* __restrict__ exact,
                        const double* __restrict__ bm1, long npts, double* __restrict__ part) {
  __shared__ double ss[6][kRedThreads];
  __shared__ double sm[6][kRedThreads];
  double s[6] = {0, 0, 0, 0, 0, 0}, m[6] = {0, 0, 0, 0, 0, 0};
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < npts;
       i += (long)gridDim.x * blockDim.x) {
    const double b = bm1[i];
    for (int q = 0; q < 6; ++q) {
      const double err = exact[q * npts + i] - u[q * npts + i];
      s[q] += err * b * err;
      m[q] = fmax(m[q], fabs(err));
    }
  }
  for (int q = 0; q < 6; ++q) { ss[q][threadIdx.x] = s[q]; sm[q][threadIdx.x] = m[q]; }
  __syncthreads();
  for (int w = kRedThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int q = 0; q < 6; ++q) {
        ss[q][threadIdx.x] += ss[q][threadIdx.x + w];
        sm[q][threadIdx.x] = fmax(sm[q][threadIdx.x], sm[q][threadIdx.x + w]);
      }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int q = 0; q < 6; ++q) {
      part[blockIdx.x * 12 + q] = ss[q][0];
      part[blockIdx.x * 12 + 6 + q] = sm[q][0];
    }
}

// per CTA: sum |H|^2/hbm1 + |E|^2/ebm1 (= bm1*(mu|H|^2 + eps|E|^2))
__global__ void k_energy(const double* __restrict__ u, const double* __restrict__ hbm1,
                         const double* __restrict__ ebm1, long npts, double* __restrict__ part) {
  __shared__ double ss[kRedThreads];
  double s = 0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < npts;
       i += (long)gridDim.x * blockDim.x) {
    double h = 0, e = 0;
    for (int q = 0; q < 3; ++q) h += u[q * npts + i] * u[q * npts + i];
    for (int q = 3; q < 6; ++q) e += u[q * npts + i] * u[q * npts + i];
    s += h / hbm1[i] + e / ebm1[i];
  }
  ss[threadIdx.x] = s;
  __syncthreads();
  for (int w = kRedThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) ss[threadIdx.x] += ss[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = ss[0];
}

// chk_blowup (src/cem_common.F:1150-1165): flags |u| > 1e20 or non-finite
__global__ void k_blowup(const double* __restrict__ u, long n, int* flag) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    const double v = u[i];
    if (!(fabs(v) <= 1.0e20)) { atomicExch(flag, 1); return; }
  }
}

}  // namespace

static const double* state_ptr(Context* c) { return c->d_u[c->cur]; }

int util_norms(Context* c, const double* d_exact, double l2[6], double linf[6]) {
  k_norms<<<kRedBlocks, kRedThreads, 0, c->stream>>>(state_ptr(c), d_exact, c->d_bm1, c->npts,
                                                      c->d_red);
  if (check_cuda(cudaGetLastError())) return NEKGPU_ERR_CUDA;
  std::vector<double> part(kRedBlocks * 12);
  if (check_cuda(cudaMemcpyAsync(part.data(), c->d_red, part.size() * sizeof(double),
                                 cudaMemcpyDeviceToHost, c->stream)))
    return NEKGPU_ERR_CUDA;
  if (check_cuda(cudaStreamSynchronize(c->stream))) return NEKGPU_ERR_CUDA;
  for (int q = 0; q < 6; ++q) {
    double s = 0, m = 0;
    for (int b = 0; b < kRedBlocks; ++b) {
      s += part[b * 12 + q];
      m = std::fmax(m, part[b * 12 + 6 + q]);
    }
    s = s / c->volume;
    l2[q] = s > 0 ? std::sqrt(s) : s;
    linf[q] = m;
  }
  return NEKGPU_OK;
}

int util_energy(Context* c, double* energy) {
  k_energy<<<kRedBlocks, kRedThreads, 0, c->stream>>>(state_ptr(c), c->d_hbm1, c->d_ebm1,
                                                       c->npts, c->d_red);
  if (check_cuda(cudaGetLastError())) return NEKGPU_ERR_CUDA;
  std::vector<double> part(kRedBlocks);
  if (check_cuda(cudaMemcpyAsync(part.data(), c->d_red, part.size() * sizeof(double),
                                 cudaMemcpyDeviceToHost, c->stream)))
    return NEKGPU_ERR_CUDA;
  if (check_cuda(cudaStreamSynchronize(c->stream))) return NEKGPU_ERR_CUDA;
  double s = 0;
  for (double p : part) s += p;
  *energy = 0.5 * s;
  return NEKGPU_OK;
}

int util_blowup(Context* c, int* bad) {
  if (check_cuda(cudaMemsetAsync(c->d_status + 1, 0, sizeof(int), c->stream)))
    return NEKGPU_ERR_CUDA;
  k_blowup<<<kRedBlocks, kRedThreads, 0, c->stream>>>(state_ptr(c), 6 * c->npts,
                                                       c->d_status + 1);
  if (check_cuda(cudaGetLastError())) return NEKGPU_ERR_CUDA;
  int h = 0;
  if (check_cuda(cudaMemcpyAsync(&h, c->d_status + 1, sizeof(int), cudaMemcpyDeviceToHost,
                                 c->stream)))
    return NEKGPU_ERR_CUDA;
  if (check_cuda(cudaStreamSynchronize(c->stream))) return NEKGPU_ERR_CUDA;
  *bad = h;
  return NEKGPU_OK;
}

}  // namespace nekgpu
