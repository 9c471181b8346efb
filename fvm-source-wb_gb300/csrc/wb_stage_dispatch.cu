// wb_stage_dispatch.cu -- picks the compiled stage kernel for a launch: precision, degree,
// basis, tile shape, and the variant -- positivity limiter and HLLC flux (wb_stage_instances.h).
#include <cuda.h>

#include <type_traits>

#include "wb_internal.h"
#include "wb_stage_instances.h"

namespace wb {

#define WB_DECL(P, R, K, BT, B, TX, TY, VAR)                                                  \
  cudaError_t WB_STAGE_INSTANCE_NAME(P, K, BT, TX, TY, VAR)(const StageArgs<R> &A,          \
                                                            const CUtensorMap *tm, cudaStream_t s);
WB_STAGE_INSTANCES(WB_DECL)
#undef WB_DECL

namespace {

// The positivity instantiation runs when limiter 2 acts in this launch: on the staged
// input (lim_y) or on a limited RK input.
template <typename R>
bool wants_positivity(const StageArgs<R> &A, int K) {
  if (K < 1 || A.limiter != 2) return false;
  for (int o = 0; o < 2; ++o)
    for (int i = 0; i < 2; ++i)
      if (A.o[o].in[i] && A.o[o].lim[i]) return true;
  return A.lim_y != 0;
}

template <typename R>
int variant(const StageArgs<R> &A, int K) {
  return (wants_positivity(A, K) ? WB_VAR_POSITIVITY : 0) | (A.riemann == 1 ? WB_VAR_HLLC : 0);
}

template <typename R>
void effective_tile(const StageArgs<R> &A, int K, int *TX, int *TY) {
  if (variant(A, K) != 0) {  // the variants are compiled for the default tile of the precision
    *TX = std::is_same<R, float>::value ? 32 : 16;
    *TY = 8;
  }
}

template <typename R>
cudaError_t dispatch(const StageArgs<R> &A, int K, int basis, int TX, int TY,
                     const CUtensorMap *tm, cudaStream_t s) {
  const int b = K == 0 ? 1 : basis;  // one mode: both bases are the same kernel
  const int var = variant(A, K);
  effective_tile(A, K, &TX, &TY);
#define WB_CASE(P, R_, K_, BT, B_, TX_, TY_, VAR_)                                            \
  if constexpr (std::is_same<R, R_>::value) {                                               \
    if (K == K_ && b == B_ && TX == TX_ && TY == TY_ && var == VAR_)                        \
      return WB_STAGE_INSTANCE_NAME(P, K_, BT, TX_, TY_, VAR_)(A, tm, s);                   \
  }
  WB_STAGE_INSTANCES(WB_CASE)
#undef WB_CASE
  return cudaErrorInvalidValue;
}

}  // namespace

cudaError_t launch_stage(const StageArgs<float> &A, int K, int basis, int TX, int TY,
                         const CUtensorMap *tm, cudaStream_t s) {
  return dispatch(A, K, basis, TX, TY, tm, s);
}
cudaError_t launch_stage(const StageArgs<double> &A, int K, int basis, int TX, int TY,
                         const CUtensorMap *tm, cudaStream_t s) {
  return dispatch(A, K, basis, TX, TY, tm, s);
}
void stage_tile(const StageArgs<float> &A, int K, int *TX, int *TY) { effective_tile(A, K, TX, TY); }
void stage_tile(const StageArgs<double> &A, int K, int *TX, int *TY) { effective_tile(A, K, TX, TY); }

bool tile_supported(int precision_fp32, int tx, int ty) {
#define WB_TILE(P, R_, K_, BT, B_, TX_, TY_, VAR_)                                            \
  if (VAR_ == 0 && std::is_same<R_, float>::value == (precision_fp32 != 0) && tx == TX_ &&  \
      ty == TY_)                                                                            \
    return true;
  WB_STAGE_INSTANCES(WB_TILE)
#undef WB_TILE
  return false;
}

}  // namespace wb
