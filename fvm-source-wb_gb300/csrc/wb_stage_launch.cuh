// wb_stage_launch.cuh -- launch of the persistent stage kernel for the compiled tile
// shapes.  Included by the per-(precision, degree) stage translation units.
#pragma once
#include "wb_stage.cuh"

namespace wb {

template <typename R, int K, int BASIS, int TX, int TY>
static cudaError_t launch_stage_tile(const StageArgs<R> &A, cudaStream_t s) {
  const int lim = A.limiter && A.lim_y && K >= 1;
  const size_t smem = stage_smem_bytes<R>(K, BASIS, TX, TY, lim);
  auto kern = k_stage<R, K, BASIS, TX, TY>;
  static int per_sm[2] = {0, 0};  // occupancy per limiter setting, queried once
  if (per_sm[lim] == 0) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return e;
    }
    int n = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, TX * TY, smem);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return e;
    }
    per_sm[lim] = n > 0 ? n : 1;
  }
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const long long ntiles = (long long)((A.nx + TX - 1) / TX) * ((A.ny + TY - 1) / TY);
  long long grid = (long long)nsm * per_sm[lim];
  if (grid > ntiles) grid = ntiles;
  kern<<<(unsigned)grid, TX * TY, smem, s>>>(A);
  return cudaGetLastError();
}

// Compiled tile shapes: FP32 (32x8, 16x16), FP64 (16x8).
template <typename R, int K, int BASIS>
static cudaError_t launch_stage_shape(const StageArgs<R> &A, int TX, int TY, cudaStream_t s) {
  if constexpr (std::is_same<R, float>::value) {
    if (TX == 32 && TY == 8) return launch_stage_tile<R, K, BASIS, 32, 8>(A, s);
    if (TX == 16 && TY == 16) return launch_stage_tile<R, K, BASIS, 16, 16>(A, s);
  } else {
    if (TX == 16 && TY == 8) return launch_stage_tile<R, K, BASIS, 16, 8>(A, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace wb

// One stage translation unit: its constant tables, their upload, and the launcher for
// degree K in one basis.
#define WB_STAGE_TU(R, K, BASIS, TAG)                                                       \
  namespace wb {                                                                            \
  cudaError_t upload_tables_##TAG(const Tab1D<R> *t) {                                      \
    return cudaMemcpyToSymbol(c_tab, t, sizeof(Tab1D<R>) * (KMAX + 1));                    \
  }                                                                                         \
  cudaError_t launch_stage_##TAG(const StageArgs<R> &A, int TX, int TY, cudaStream_t s) {   \
    return launch_stage_shape<R, K, BASIS>(A, TX, TY, s);                                   \
  }                                                                                         \
  }
