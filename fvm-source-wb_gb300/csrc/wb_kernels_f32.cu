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

cudaError_t launch_batch_begin_step(const StageArgs<float> *args, int n, cudaStream_t s) {
  k_batch_begin_step<float><<<(n + 127) / 128, 128, 0, s>>>(args, n);
  return cudaGetLastError();
}

cudaError_t launch_batch_errors(const StageArgs<float> *args, int n, int *out, cudaStream_t s) {
  k_batch_errors<float><<<(n + 127) / 128, 128, 0, s>>>(args, n, out);
  return cudaGetLastError();
}

cudaError_t launch_batch_max_speed(const StageArgs<float> *args, const float *const *state,
                                   const int4 *items, int nitems, cudaStream_t s) {
  int grid = nitems < 4096 ? nitems : 4096;
  k_batch_max_speed<float><<<grid, 256, 0, s>>>(args, state, items, nitems);
  return cudaGetLastError();
}

}  // namespace wb
