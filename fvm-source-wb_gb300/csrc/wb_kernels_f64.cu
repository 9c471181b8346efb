// wb_kernels_f64.cu -- FP64 "plain" instantiations and the FP64 diagnostics.
#include "wb_types.h"
namespace wb {
__constant__ Tab1D<double> c_tab[KMAX + 1];
}
#include "wb_launch.cuh"
WB_DEFINE_PRECISION_ENTRY_POINTS(double)

namespace wb {

size_t diag_partial_bytes(int nx, int ny) {
  size_t nblk = (size_t)((nx + 31) / 32) * ((ny + 7) / 8);
  return nblk * NV * 3 * sizeof(double) + 64 * sizeof(double);
}

cudaError_t launch_norms(const AuxArgs &A, const Tab1D<double> *Td, const double *a,
                         const double *b, double *partial, double *out, int K_, int B_,
                         cudaStream_t s) {
  dim3 blk(32, 8), grd = cell_grid(A.nx, A.ny, blk);
  WB_DISPATCH_KB(K_, B_, { k_norms<K, BASIS><<<grd, blk, 0, s>>>(A, Td, a, b, partial); });
  k_norms_final<<<1, 32, 0, s>>>(partial, (int)(grd.x * grd.y), out);
  return cudaGetLastError();
}

// Self-test of the bounded device wait of the TMA staging: an mbarrier whose phase nothing
// completes.  The wait gives up after `polls` polls and reports it in the error word, as a
// stage kernel would; nothing is in flight when the kernel returns.
__global__ void k_wait_selftest(int *err, int polls) {
  __shared__ unsigned long long bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  const bool done = mbar_wait(&bar, 0u, polls);
  if (!done && threadIdx.x == 0) atomicOr(err, 2);
}

cudaError_t launch_wait_selftest(int *err, int polls, cudaStream_t s) {
  k_wait_selftest<<<1, 32, 0, s>>>(err, polls);
  return cudaGetLastError();
}

cudaError_t launch_f32_to_f64(double *out, const float *in, long long n, cudaStream_t s) {
  k_convert<double, float><<<1216, 256, 0, s>>>(out, in, n);
  return cudaGetLastError();
}
cudaError_t launch_f64_to_f32(float *out, const double *in, long long n, cudaStream_t s) {
  k_convert<float, double><<<1216, 256, 0, s>>>(out, in, n);
  return cudaGetLastError();
}

// Device-to-device copy of n 16-byte words on the SMs: inside a pipeline whose host copies
// occupy the copy engines, a cudaMemcpyAsync between device buffers would queue behind them.
__global__ void __launch_bounds__(256) k_copy16(uint4 *__restrict__ out,
                                                const uint4 *__restrict__ in, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    __stcs(out + i, __ldcs(in + i));
}
cudaError_t launch_copy_device(void *out, const void *in, size_t bytes, cudaStream_t s) {
  if (bytes % 16 != 0 || ((uintptr_t)out | (uintptr_t)in) % 16 != 0) return cudaErrorInvalidValue;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  k_copy16<<<nsm * 8, 256, 0, s>>>((uint4 *)out, (const uint4 *)in, (long long)(bytes / 16));
  return cudaGetLastError();
}

}  // namespace wb
