// wb_noalloc.cu -- error norms of two device-resident FP64 modal states without any
// device allocation.
//
// Some callers cannot allocate device memory at the moment they need the norms: a host
// whose device memory is all owned by its own pool or by another runtime, or a time loop
// that must not pay the device-wide synchronisation cudaMalloc/cudaFree imply.  For them
// this entry point keeps its reduction scratch in a fixed array that is part of the
// library image: it exists on every device that loads the library, for the life of the
// process.  The first call on a device (and again after the device's context has been
// re-created, e.g. by cudaDeviceReset) sets the device up; calls sharing the array must
// not overlap on the GPU.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/wb_capi.h"
#include "wb_tables.h"
#include "wb_types.h"
namespace wb {
__constant__ Tab1D<double> c_tab[KMAX + 1];  // required by the shared kernel headers
}
#include "wb_launch.cuh"

namespace wb {
// the FP64 norm reduction of wb_kernels_f64.cu, with caller-provided tables and scratch
static cudaError_t launch_norms_on(const AuxArgs &A, const Tab1D<double> *Td, const double *a,
                                   const double *b, double *partial, double *out, int K_,
                                   int B_, cudaStream_t s) {
  dim3 blk(32, 8), grd = cell_grid(A.nx, A.ny, blk);
  WB_DISPATCH_KB(K_, B_, { k_norms<K, BASIS><<<grd, blk, 0, s>>>(A, Td, a, b, partial); });
  k_norms_final<<<1, 32, 0, s>>>(partial, (int)(grd.x * grd.y), out);
  return cudaGetLastError();
}
}  // namespace wb

namespace {

// 16384 blocks of 32x8 cells (grids of up to 4,194,304 cells); 12 partial sums per block
// plus the 12 final values: 1.5 MB per device.
constexpr int kMaxBlocks = WB_NORMS_NOALLOC_MAX_CELLS / 256;
constexpr int kPartials = kMaxBlocks * wb::NV * 3;
static __device__ __align__(256) double g_norm_scratch[kPartials + 64];
static __device__ __align__(256) wb::Tab1D<double> g_norm_tabs[wb::KMAX + 1];

struct DeviceSetup {
  bool done = false;
  unsigned long long ctx_id = 0;       // the CUDA context the set-up was done in
  double *scratch = nullptr;           // device address of g_norm_scratch
  wb::Tab1D<double> *tabs = nullptr;   // device address of g_norm_tabs
};
constexpr int kMaxDevices = 64;
DeviceSetup g_setup[kMaxDevices];
std::mutex g_setup_mutex;

// Unique id of the current CUDA context (cuCtxGetId through the runtime's driver entry
// point, no link to libcuda), 0 where it is not available.  A context torn down by
// cudaDeviceReset and created again gets a new id, and with it new copies of the arrays.
unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext *);
  using GetId = CUresult (*)(CUcontext, unsigned long long *);
  static std::once_flag once;
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(p);
    cudaGetLastError();
  });
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&c) == CUDA_SUCCESS && c && get_id(c, &id) == CUDA_SUCCESS)
    return id;
  return 0;
}

// Once per device and context, with that device current (the runtime has made its
// primary context current): the symbol addresses (a host-side name of a __device__ array
// is not a device address) and the basis tables.
int setup_device(int dev, DeviceSetup **out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  DeviceSetup &s = g_setup[dev];
  // no context current yet (id 0) or another one than at set-up: set up (again); the
  // runtime calls below make the device's context current
  if (s.done && (s.ctx_id == 0 || s.ctx_id != current_context_id())) s = DeviceSetup();
  if (!s.done) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_norm_scratch) != cudaSuccess) return WB_ERR_CUDA;
    s.scratch = static_cast<double *>(p);
    if (cudaGetSymbolAddress(&p, g_norm_tabs) != cudaSuccess) return WB_ERR_CUDA;
    s.tabs = static_cast<wb::Tab1D<double> *>(p);
    wb::Tab1D<double> t[wb::KMAX + 1];
    wb::make_tab1d(t);
    if (cudaMemcpyToSymbol(g_norm_tabs, t, sizeof(t)) != cudaSuccess) return WB_ERR_CUDA;
    s.ctx_id = current_context_id();
    s.done = true;
  }
  *out = &s;
  return WB_OK;
}

}  // namespace

extern "C" int wb_norms_device_noalloc(int32_t nx, int32_t ny, int32_t order, int32_t basis,
                                       double lx, double ly, const double *a, const double *b,
                                       size_t plane_stride, void *stream, double l1[4],
                                       double linf[4], double l2[4]) {
  if (!a || nx < 1 || ny < 1 || order < 0 || order > wb::KMAX || (basis != 0 && basis != 1) ||
      !(lx > 0.0) || !(ly > 0.0) || plane_stride < (size_t)nx * (size_t)ny)
    return WB_ERR_ARG;
  const long long nbx = (nx + 31) / 32, nby = (ny + 7) / 8;
  if ((long long)nx * ny > WB_NORMS_NOALLOC_MAX_CELLS || nbx * nby > kMaxBlocks)
    return WB_ERR_ARG;  // larger than the fixed scratch: use wb_norms
  // every call copies its results back and waits for the stream, which a stream capture
  // does not allow: refuse before touching the caller's capture
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(static_cast<cudaStream_t>(stream), &cs) != cudaSuccess) {
    cudaGetLastError();
    return WB_ERR_CUDA;
  }
  if (cs != cudaStreamCaptureStatusNone) return WB_ERR_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return WB_ERR_CUDA;
  }
  DeviceSetup *s = nullptr;
  int rc = setup_device(dev, &s);
  if (rc) {
    cudaGetLastError();
    return rc;
  }
  wb::AuxArgs A;
  std::memset(&A, 0, sizeof(A));
  A.nx = nx;
  A.ny = ny;
  A.pitch = nx;
  A.plane = (long long)plane_stride;
  A.dx = lx / nx;
  A.dy = ly / ny;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // every block writes its own partial slot and the final pass reads exactly those
  // slots, so nothing in the shared array has to start at zero
  double *out = s->scratch;             // 12 final values
  double *partial = s->scratch + 64;    // per-block partials
  if (wb::launch_norms_on(A, s->tabs, a, b, partial, out, order, basis, st) != cudaSuccess) {
    cudaGetLastError();
    return WB_ERR_CUDA;
  }
  double h[12];
  if (cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    cudaGetLastError();
    return WB_ERR_CUDA;
  }
  for (int v = 0; v < 4; ++v) {
    if (l1) l1[v] = h[v];
    if (l2) l2[v] = std::sqrt(h[4 + v]);
    if (linf) linf[v] = h[8 + v];
  }
  return WB_OK;
}
