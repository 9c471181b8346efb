// wb_kernels_f32.cu -- FP32-perturbation instantiations (FP64 equilibrium factors are
// rounded once to FP32 tables; see wb_stage.cuh for the exact-difference form).
#include "wb_types.h"
namespace wb {
__constant__ Tab1D<float> c_tab[KMAX + 1];
}
#include "wb_launch.cuh"
WB_DEFINE_PRECISION_ENTRY_POINTS(float)

#include "wb_batch_kernel.cuh"

namespace wb {

template <int K, bool POS>
static cudaError_t launch_batch_stage_t(const StageArgs<float> *args, const int4 *items,
                                        int nitems, int bufsz, size_t smem, int *grid_out,
                                        cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(k_batch_stage<float, K, POS>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_stage<float, K, POS>, 256, smem);
  if (e != cudaSuccess) return e;
  int grid = nsm * (per_sm > 0 ? per_sm : 1);
  if (grid > nitems) grid = nitems;
  if (grid_out) *grid_out = grid;
  k_batch_stage<float, K, POS><<<grid, 256, smem, s>>>(args, items, nitems, bufsz);
  return cudaGetLastError();
}

cudaError_t launch_batch_stage(const StageArgs<float> *args, const int4 *items, int nitems,
                               int bufsz, size_t smem, int pos, int K, int *grid_out,
                               cudaStream_t s) {
  switch (K) {
    case 0: return launch_batch_stage_t<0, false>(args, items, nitems, bufsz, smem, grid_out, s);
    case 1:
      return pos ? launch_batch_stage_t<1, true>(args, items, nitems, bufsz, smem, grid_out, s)
                 : launch_batch_stage_t<1, false>(args, items, nitems, bufsz, smem, grid_out, s);
    case 2:
      return pos ? launch_batch_stage_t<2, true>(args, items, nitems, bufsz, smem, grid_out, s)
                 : launch_batch_stage_t<2, false>(args, items, nitems, bufsz, smem, grid_out, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_batch_max_speed(const StageArgs<float> *args, const float *const *state,
                                   const int4 *items, int nitems, cudaStream_t s) {
  int grid = nitems < 4096 ? nitems : 4096;
  k_batch_max_speed<float><<<grid, 256, 0, s>>>(args, state, items, nitems);
  return cudaGetLastError();
}

}  // namespace wb
