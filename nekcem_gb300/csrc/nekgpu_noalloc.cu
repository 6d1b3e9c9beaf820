// cem_error norms through an entry point that allocates no memory.
//
// Who needs it: a caller that cannot call cudaMalloc / cudaFree once it is
// time stepping -- for example a driver that hands all free device memory to
// its own pool at start-up, or a time loop that must not risk an allocation
// failure, or the synchronisation that cudaFree brings, between two steps.
// nekgpu_norms() allocates a device copy of the exact fields on every call;
// nekgpu_norms_noalloc() takes the exact fields already on the device and
// keeps its only scratch -- the per-block partial sums of the reduction -- in
// the fixed array below, which every GPU that loads this library holds until
// the process exits.
//
// Rules that come with the fixed array:
//  * at most kMaxBlocks * kPointsPerBlock = 8,388,608 nodes per call; a larger
//    mesh gets NEKGPU_ERR_TOO_LARGE;
//  * every call on a device uses the same array, so calls whose GPU work can
//    overlap (two contexts on different streams, or another host thread)
//    race and give wrong results; serialise them;
//  * the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (once per device, with that device current); make
//    that first call before any stream capture;
//  * the call works on the context's own device: when another device is
//    current it makes the context's device current for the call and puts the
//    caller's device back before returning.
// Nothing in the array has to start at zero: each call writes every partial
// it later reads.
#include <cuda_runtime.h>

#include <cmath>

#include "nekgpu_internal.h"

namespace nekgpu {

namespace {

constexpr int kThreads = 256;
constexpr int kPointsPerBlock = 2048;  // 8 nodes per thread
constexpr int kMaxBlocks = 4096;       // => 8,388,608 nodes
constexpr int kMaxDevices = 64;

// per block: 6 sums of err*bm1*err, then 6 maxima of |err|; then 12 finals
static __device__ __align__(256) double g_norm_scratch[(kMaxBlocks + 1) * 12];

// device address of g_norm_scratch, looked up once per device
double* g_scratch_ptr[kMaxDevices] = {nullptr};

__global__ void k_norm_partials(const double* __restrict__ u, const double* __restrict__ exact,
                                const double* __restrict__ bm1, long npts,
                                double* __restrict__ part) {
  __shared__ double ss[12][kThreads];
  double s[6] = {0, 0, 0, 0, 0, 0}, m[6] = {0, 0, 0, 0, 0, 0};
  const long base = (long)blockIdx.x * kPointsPerBlock;
  for (int r = 0; r < kPointsPerBlock / kThreads; ++r) {
    const long i = base + r * kThreads + threadIdx.x;
    if (i >= npts) break;
    const double b = bm1[i];
    for (int q = 0; q < 6; ++q) {
      const double err = exact[q * npts + i] - u[q * npts + i];
      s[q] += err * b * err;
      m[q] = fmax(m[q], fabs(err));
    }
  }
  for (int q = 0; q < 6; ++q) {
    ss[q][threadIdx.x] = s[q];
    ss[6 + q][threadIdx.x] = m[q];
  }
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int q = 0; q < 6; ++q) {
        ss[q][threadIdx.x] += ss[q][threadIdx.x + w];
        ss[6 + q][threadIdx.x] = fmax(ss[6 + q][threadIdx.x], ss[6 + q][threadIdx.x + w]);
      }
    __syncthreads();
  }
  if (threadIdx.x < 12) part[blockIdx.x * 12 + threadIdx.x] = ss[threadIdx.x][0];
}

// one thread per result, partials combined in block order (deterministic)
__global__ void k_norm_final(int nblocks, double* __restrict__ part) {
  const int q = threadIdx.x;
  if (q >= 12) return;
  double acc = 0.0;
  for (int b = 0; b < nblocks; ++b) {
    const double v = part[b * 12 + q];
    acc = q < 6 ? acc + v : fmax(acc, v);
  }
  part[kMaxBlocks * 12 + q] = acc;
}

}  // namespace

namespace {

// Set-up (first call per device) and the reduction on the current device,
// which is the context's; allocates nothing.
int norms_on_device(Context* c, int dev, const double* exact_dev, double l2[6], double linf[6]) {
  if (!g_scratch_ptr[dev]) {
    double* p = nullptr;
    if (check_cuda(cudaGetSymbolAddress((void**)&p, g_norm_scratch))) return NEKGPU_ERR_CUDA;
    g_scratch_ptr[dev] = p;
  }
  double* part = g_scratch_ptr[dev];
  const int nblocks = (int)((c->npts + kPointsPerBlock - 1) / kPointsPerBlock);
  k_norm_partials<<<nblocks, kThreads, 0, c->stream>>>(c->d_u[c->cur], exact_dev, c->d_bm1,
                                                        c->npts, part);
  if (check_cuda(cudaGetLastError())) return NEKGPU_ERR_CUDA;
  k_norm_final<<<1, 32, 0, c->stream>>>(nblocks, part);
  if (check_cuda(cudaGetLastError())) return NEKGPU_ERR_CUDA;
  double fin[12];
  if (check_cuda(cudaMemcpyAsync(fin, part + kMaxBlocks * 12, sizeof(fin), cudaMemcpyDeviceToHost,
                                 c->stream)))
    return NEKGPU_ERR_CUDA;
  if (check_cuda(cudaStreamSynchronize(c->stream))) return NEKGPU_ERR_CUDA;
  for (int q = 0; q < 6; ++q) {
    const double s = fin[q] / c->volume;
    l2[q] = s > 0 ? std::sqrt(s) : s;
    linf[q] = fin[6 + q];
  }
  return NEKGPU_OK;
}

}  // namespace

int norms_noalloc(Context* c, const double* exact_dev, double l2[6], double linf[6]) {
  if (c->npts > (long)kMaxBlocks * kPointsPerBlock) return NEKGPU_ERR_TOO_LARGE;
  const int dev = c->device;
  if (dev < 0 || dev >= kMaxDevices) return NEKGPU_ERR_UNSUPPORTED;
  int prev = 0;
  if (check_cuda(cudaGetDevice(&prev))) return NEKGPU_ERR_CUDA;
  if (prev != dev && check_cuda(cudaSetDevice(dev))) return NEKGPU_ERR_CUDA;
  const int st = norms_on_device(c, dev, exact_dev, l2, linf);
  if (prev != dev && check_cuda(cudaSetDevice(prev)) && st == NEKGPU_OK) return NEKGPU_ERR_CUDA;
  return st;
}

}  // namespace nekgpu
