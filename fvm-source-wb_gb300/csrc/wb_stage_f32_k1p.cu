// wb_stage_f32_k1p.cu -- persistent stage kernels: float, degree 1, total-degree basis.
#include "wb_types.h"
namespace wb {
__constant__ Tab1D<float> c_tab[KMAX + 1];
}
#include "wb_stage_launch.cuh"
WB_STAGE_TU(float, 1, 1, f32_k1p)
