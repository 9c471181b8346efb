// wb_stage_f64_k2p.cu -- persistent stage kernels: double, degree 2, total-degree basis.
#include "wb_types.h"
namespace wb {
__constant__ Tab1D<double> c_tab[KMAX + 1];
}
#include "wb_stage_launch.cuh"
WB_STAGE_TU(double, 2, 1, f64_k2p)
