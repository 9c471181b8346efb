// wb_stage_f32_k0.cu -- persistent stage kernels: float, degree 0, tensor basis.
#include "wb_types.h"
namespace wb {
__constant__ Tab1D<float> c_tab[KMAX + 1];
}
#include "wb_stage_launch.cuh"
WB_STAGE_TU(float, 0, 0, f32_k0)
