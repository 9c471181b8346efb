// wb_stage_launch.cuh -- launch of one persistent stage kernel.  Included by the
// per-instance translation units that build.py generates from wb_stage_instances.h.
#pragma once
#include <cstring>
#include "wb_stage.cuh"
#include "wb_stage_instances.h"

namespace wb {

template <typename R, int K, int BASIS, int TX, int TY, int VAR, int CPT>
static cudaError_t launch_stage_kernel(const StageArgs<R> &A, const CUtensorMap *tm,
                                       cudaStream_t s) {
  constexpr int NT = TX * TY / CPT;  // threads per CTA
  const int lim = A.limiter == 1 && A.lim_y && K >= 1;
  const size_t smem = stage_smem_bytes<R>(K, BASIS, TX, TY, lim);
  auto kern = k_stage<R, K, BASIS, TX, TY, VAR, CPT>;
  CUtensorMap none;
  std::memset(&none, 0, sizeof(none));
  // The kernel's dynamic shared-memory limit is one attribute for both limiter settings:
  // it is set once to the larger size (the minmod limiter stages the second-ring means);
  // the occupancy is queried per setting.
  static int per_sm[2] = {0, 0};
  if (per_sm[0] == 0) {
    const size_t s0 = stage_smem_bytes<R>(K, BASIS, TX, TY, 0);
    const size_t s1 = stage_smem_bytes<R>(K, BASIS, TX, TY, K >= 1 ? 1 : 0);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(s0 > s1 ? s0 : s1));
    if (e != cudaSuccess) {
      cudaGetLastError();
      return e;
    }
    for (int l = 0; l < 2; ++l) {
      int n = 0;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, NT, l ? s1 : s0);
      if (e != cudaSuccess) {
        cudaGetLastError();
        return e;
      }
      per_sm[l] = n > 0 ? n : 1;
    }
  }
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const long long ntiles = (long long)((A.nx + TX - 1) / TX) * ((A.ny + TY - 1) / TY);
  long long grid = (long long)nsm * per_sm[lim];
  if (grid > ntiles) grid = ntiles;
  kern<<<(unsigned)grid, NT, smem, s>>>(A, tm ? *tm : none);
  return cudaGetLastError();
}

}  // namespace wb

// One compiled stage kernel (a line of wb_stage_instances.h) and its launcher.
#define WB_STAGE_INSTANCE(P, R, K, BT, B, TX, TY, VAR, CPT)                                 \
  namespace wb {                                                                            \
  cudaError_t WB_STAGE_INSTANCE_NAME(P, K, BT, TX, TY, VAR, CPT)(                            \
      const StageArgs<R> &A, const CUtensorMap *tm, cudaStream_t s) {                       \
    return launch_stage_kernel<R, K, B, TX, TY, VAR, CPT>(A, tm, s);                        \
  }                                                                                         \
  }
