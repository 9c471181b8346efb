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

template <int K, int TX, int TY, bool POS>
static cudaError_t launch_batch_stage_t(const StageArgs<float> *args, const int4 *items,
                                        int nitems, int bufsz, size_t smem, int *grid_out,
                                        cudaStream_t s) {
  auto kern = k_batch_stage<float, K, TX, TY, POS>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TX * TY, smem);
  if (e != cudaSuccess) return e;
  int grid = nsm * (per_sm > 0 ? per_sm : 1);
  if (grid > nitems) grid = nitems;
  if (grid_out) *grid_out = grid;
  kern<<<grid, TX * TY, smem, s>>>(args, items, nitems, bufsz);
  return cudaGetLastError();
}

template <int TX, int TY>
static cudaError_t launch_batch_tile(const StageArgs<float> *args, const int4 *items, int nitems,
                                     int bufsz, size_t smem, int pos, int K, int *grid_out,
                                     cudaStream_t s) {
  switch (K) {
    case 0: return launch_batch_stage_t<0, TX, TY, false>(args, items, nitems, bufsz, smem, grid_out, s);
    case 1:
      return pos ? launch_batch_stage_t<1, TX, TY, true>(args, items, nitems, bufsz, smem, grid_out, s)
                 : launch_batch_stage_t<1, TX, TY, false>(args, items, nitems, bufsz, smem, grid_out, s);
    case 2:
      return pos ? launch_batch_stage_t<2, TX, TY, true>(args, items, nitems, bufsz, smem, grid_out, s)
                 : launch_batch_stage_t<2, TX, TY, false>(args, items, nitems, bufsz, smem, grid_out, s);
    default: return cudaErrorInvalidValue;
  }
}

bool batch_tile_supported(int TX, int TY) {
  return (TX == 32 && TY == 8) || (TX == 16 && TY == 16);
}

cudaError_t launch_batch_stage(const StageArgs<float> *args, const int4 *items, int nitems,
                               int bufsz, size_t smem, int pos, int K, int TX, int TY,
                               int *grid_out, cudaStream_t s) {
  if (TX == 32 && TY == 8)
    return launch_batch_tile<32, 8>(args, items, nitems, bufsz, smem, pos, K, grid_out, s);
  if (TX == 16 && TY == 16)
    return launch_batch_tile<16, 16>(args, items, nitems, bufsz, smem, pos, K, grid_out, s);
  return cudaErrorInvalidValue;
}

cudaError_t launch_batch_max_speed(const StageArgs<float> *args, const float *const *state,
                                   const int4 *items, int nitems, cudaStream_t s) {
  int grid = nitems < 4096 ? nitems : 4096;
  k_batch_max_speed<float><<<grid, 256, 0, s>>>(args, state, items, nitems);
  return cudaGetLastError();
}

}  // namespace wb
