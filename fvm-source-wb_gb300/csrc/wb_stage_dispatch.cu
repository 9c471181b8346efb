// wb_stage_dispatch.cu -- picks the compiled stage kernel for a launch: precision, degree,
// basis, tile shape, cells per thread, and the variant -- positivity limiter and HLLC flux
// (wb_stage_instances.h); and the batched form's kernel by degree, tile, positivity limiter
// and cells per thread.
#include <cuda.h>

#include <type_traits>

#include "wb_internal.h"
#include "wb_stage_instances.h"

namespace wb {

#define WB_DECL(P, R, K, BT, B, TX, TY, VAR, CPT)                                             \
  cudaError_t WB_STAGE_INSTANCE_NAME(P, K, BT, TX, TY, VAR, CPT)(                           \
      const StageArgs<R> &A, const CUtensorMap *tm, cudaStream_t s);
WB_STAGE_INSTANCES(WB_DECL)
#undef WB_DECL
#define WB_BDECL(K, TX, TY, POS, CPT)                                                         \
  cudaError_t WB_BATCH_INSTANCE_NAME(K, TX, TY, POS, CPT)(                                  \
      const StageArgs<float> &Q, const StageArgs<float> *args, const CUtensorMap *tmaps,    \
      const int4 *items, int nitems, int bufsz, size_t smem, int *grid_out, cudaStream_t s);
WB_BATCH_INSTANCES(WB_BDECL)
#undef WB_BDECL

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
void effective_tile(const StageArgs<R> &A, int K, int *TX, int *TY, int *CPT) {
  if (variant(A, K) != 0) {  // the variants are compiled for the default tile of the precision
    *TX = std::is_same<R, float>::value ? 32 : 16;
    *TY = 8;
    *CPT = 1;
  }
}

template <typename R>
cudaError_t dispatch(const StageArgs<R> &A, int K, int basis, int TX, int TY, int CPT,
                     const CUtensorMap *tm, cudaStream_t s) {
  const int b = K == 0 ? 1 : basis;  // one mode: both bases are the same kernel
  const int var = variant(A, K);
  effective_tile(A, K, &TX, &TY, &CPT);
#define WB_CASE(P, R_, K_, BT, B_, TX_, TY_, VAR_, CPT_)                                      \
  if constexpr (std::is_same<R, R_>::value) {                                               \
    if (K == K_ && b == B_ && TX == TX_ && TY == TY_ && var == VAR_ && CPT == CPT_)         \
      return WB_STAGE_INSTANCE_NAME(P, K_, BT, TX_, TY_, VAR_, CPT_)(A, tm, s);             \
  }
  WB_STAGE_INSTANCES(WB_CASE)
#undef WB_CASE
  return cudaErrorInvalidValue;
}

}  // namespace

cudaError_t launch_stage(const StageArgs<float> &A, int K, int basis, int TX, int TY, int CPT,
                         const CUtensorMap *tm, cudaStream_t s) {
  return dispatch(A, K, basis, TX, TY, CPT, tm, s);
}
cudaError_t launch_stage(const StageArgs<double> &A, int K, int basis, int TX, int TY, int CPT,
                         const CUtensorMap *tm, cudaStream_t s) {
  return dispatch(A, K, basis, TX, TY, CPT, tm, s);
}
void stage_tile(const StageArgs<float> &A, int K, int *TX, int *TY, int *CPT) {
  effective_tile(A, K, TX, TY, CPT);
}
void stage_tile(const StageArgs<double> &A, int K, int *TX, int *TY, int *CPT) {
  effective_tile(A, K, TX, TY, CPT);
}

bool tile_supported(int precision_fp32, int order, int basis, int tx, int ty, int cpt) {
  const int b = order == 0 ? 1 : basis;
#define WB_TILE(P, R_, K_, BT, B_, TX_, TY_, VAR_, CPT_)                                      \
  if (VAR_ == 0 && std::is_same<R_, float>::value == (precision_fp32 != 0) && K_ == order && \
      B_ == b && tx == TX_ && ty == TY_ && cpt == CPT_)                                     \
    return true;
  WB_STAGE_INSTANCES(WB_TILE)
#undef WB_TILE
  return false;
}

int tile_candidates(int precision_fp32, int order, int basis, int (*out)[3], int max) {
  const int b = order == 0 ? 1 : basis;
  int n = 0;
#define WB_CAND(P, R_, K_, BT, B_, TX_, TY_, VAR_, CPT_)                                      \
  if (VAR_ == 0 && std::is_same<R_, float>::value == (precision_fp32 != 0) && K_ == order && \
      B_ == b && n < max) {                                                                 \
    out[n][0] = TX_;                                                                        \
    out[n][1] = TY_;                                                                        \
    out[n][2] = CPT_;                                                                       \
    ++n;                                                                                    \
  }
  WB_STAGE_INSTANCES(WB_CAND)
#undef WB_CAND
  return n;
}

cudaError_t launch_batch_stage(const StageArgs<float> &Q, const StageArgs<float> *args,
                               const CUtensorMap *tmaps, const int4 *items, int nitems,
                               int bufsz, size_t smem, int pos, int K, int TX, int TY, int CPT,
                               int *grid_out, cudaStream_t s) {
  const int p = pos && K >= 1 ? 1 : 0;
#define WB_BCASE(K_, TX_, TY_, POS_, CPT_)                                                    \
  if (K == K_ && TX == TX_ && TY == TY_ && p == POS_ && CPT == CPT_)                         \
    return WB_BATCH_INSTANCE_NAME(K_, TX_, TY_, POS_, CPT_)(Q, args, tmaps, items, nitems,   \
                                                           bufsz, smem, grid_out, s);
  WB_BATCH_INSTANCES(WB_BCASE)
#undef WB_BCASE
  return cudaErrorInvalidValue;
}

bool batch_tile_supported(int order, int tx, int ty, int cpt) {
#define WB_BTILE(K_, TX_, TY_, POS_, CPT_)                                                    \
  if (POS_ == 0 && K_ == order && tx == TX_ && ty == TY_ && cpt == CPT_) return true;
  WB_BATCH_INSTANCES(WB_BTILE)
#undef WB_BTILE
  return false;
}

int batch_tile_candidates(int order, int (*out)[3], int max) {
  int n = 0;
#define WB_BCAND(K_, TX_, TY_, POS_, CPT_)                                                    \
  if (POS_ == 0 && K_ == order && n < max) {                                                \
    out[n][0] = TX_;                                                                        \
    out[n][1] = TY_;                                                                        \
    out[n][2] = CPT_;                                                                       \
    ++n;                                                                                    \
  }
  WB_BATCH_INSTANCES(WB_BCAND)
#undef WB_BCAND
  return n;
}

}  // namespace wb
