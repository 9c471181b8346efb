// wb_batch_launch.cuh -- launch of one batched stage kernel (a line of WB_BATCH_INSTANCES in
// wb_stage_instances.h).  Included by the per-instance translation units build.py makes.
#pragma once
#include "wb_types.h"
namespace wb {
__constant__ Tab1D<float> c_tab[KMAX + 1];  // declared for the shared kernel header
}
#include "wb_batch_kernel.cuh"
#include "wb_stage_instances.h"

namespace wb {

template <int K, int TX, int TY, bool POS, int CPT>
static cudaError_t launch_batch_stage_t(const StageArgs<float> &Q, const StageArgs<float> *args,
                                        const CUtensorMap *tmaps, const int4 *items, int nitems,
                                        int bufsz, size_t smem, int *grid_out, cudaStream_t s) {
  constexpr int NT = TX * TY / CPT;  // threads per CTA
  auto kern = k_batch_stage<float, K, TX, TY, POS, CPT>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem);
  if (e != cudaSuccess) return e;
  int grid = nsm * (per_sm > 0 ? per_sm : 1);
  if (grid > nitems) grid = nitems;
  if (grid_out) *grid_out = grid;
  kern<<<grid, NT, smem, s>>>(Q, args, tmaps, items, nitems, bufsz);
  return cudaGetLastError();
}

}  // namespace wb

#define WB_BATCH_INSTANCE(K, TX, TY, POS, CPT)                                               \
  namespace wb {                                                                            \
  cudaError_t WB_BATCH_INSTANCE_NAME(K, TX, TY, POS, CPT)(                                  \
      const StageArgs<float> &Q, const StageArgs<float> *args, const CUtensorMap *tmaps,    \
      const int4 *items, int nitems, int bufsz, size_t smem, int *grid_out, cudaStream_t s) { \
    return launch_batch_stage_t<K, TX, TY, POS != 0, CPT>(Q, args, tmaps, items, nitems,    \
                                                         bufsz, smem, grid_out, s);         \
  }                                                                                         \
  }
