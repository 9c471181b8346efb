// wb_kernels_f32.cu -- FP32-perturbation instantiations (FP64 equilibrium factors are
// rounded once to FP32 tables; see wb_stage.cuh for the exact-difference form).
#include "wb_types.h"
namespace wb {
__constant__ Tab1D<float> c_tab[KMAX + 1];
}
#include "wb_launch.cuh"
WB_DEFINE_PRECISION_ENTRY_POINTS(float)
