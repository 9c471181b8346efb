// wb_internal.h -- entry points between the host layer (wb_capi.cu) and the
// per-precision kernel translation units.
#pragma once
#include <cuda.h>
#include "wb_types.h"
#include "../../include/wb_capi.h"

namespace wb {

#define WB_DECLARE_PRECISION_ENTRY_POINTS(R)                                                   \
  cudaError_t upload_tables_aux(const Tab1D<R> *t);                                            \
  cudaError_t launch_limit(const StageArgs<R> &A, R *u, int K, int basis, cudaStream_t s);     \
  cudaError_t launch_max_speed(const StageArgs<R> &A, const R *u, int K, int basis,            \
                               cudaStream_t s);                                                \
  cudaError_t launch_init_ic(const AuxArgs &A, const IcArgs &I, const Tab1D<double> *Td, R *u, \
                             int K, int basis, cudaStream_t s);                                \
  cudaError_t launch_to_fortran(const R *soa, double *f, int nx, int ny, long long P, int K,   \
                                cudaStream_t s);                                               \
  cudaError_t launch_from_fortran(const double *f, R *soa, int nx, int ny, long long P, int K, \
                                  cudaStream_t s);                                             \
  cudaError_t launch_sums(const AuxArgs &A, const Tab1D<double> *Td, const R *u,               \
                          double *partial, double *out, int K, int basis, cudaStream_t s);

WB_DECLARE_PRECISION_ENTRY_POINTS(float)
WB_DECLARE_PRECISION_ENTRY_POINTS(double)

// Stage kernels (wb_stage_dispatch.cu): the compiled kernel for precision, degree K,
// basis, tile TX x TY and CPT cells per thread (and the positivity limiter when the launch
// needs it).  tm: the tensor map of the staged input for the effective tile (stage_tile),
// or null.
cudaError_t launch_stage(const StageArgs<float> &A, int K, int basis, int TX, int TY, int CPT,
                         const CUtensorMap *tm, cudaStream_t s);
cudaError_t launch_stage(const StageArgs<double> &A, int K, int basis, int TX, int TY, int CPT,
                         const CUtensorMap *tm, cudaStream_t s);
// The tile the launch will run (variants run on the default tile of the precision).
void stage_tile(const StageArgs<float> &A, int K, int *TX, int *TY, int *CPT);
void stage_tile(const StageArgs<double> &A, int K, int *TX, int *TY, int *CPT);
// Tile shapes (TX, TY, cells per thread) the stage kernels are compiled for, and the list
// of them for one precision, degree and basis (the autotuner's candidates).
bool tile_supported(int precision_fp32, int order, int basis, int tx, int ty, int cpt);
int tile_candidates(int precision_fp32, int order, int basis, int (*out)[3], int max);

// Constant-memory basis tables of the auxiliary kernels, both precisions.
inline cudaError_t upload_tables(const Tab1D<float> *t32, const Tab1D<double> *t64) {
  cudaError_t e = upload_tables_aux(t32);
  if (e != cudaSuccess) return e;
  return upload_tables_aux(t64);
}

// FP64-only diagnostics and precision conversion (defined in wb_kernels_f64.cu)
cudaError_t launch_norms(const AuxArgs &A, const Tab1D<double> *Td, const double *a,
                         const double *b, double *partial, double *out, int K, int basis,
                         cudaStream_t s);
cudaError_t launch_f32_to_f64(double *out, const float *in, long long n, cudaStream_t s);
cudaError_t launch_wait_selftest(int *err, int polls, cudaStream_t s);
cudaError_t launch_f64_to_f32(float *out, const double *in, long long n, cudaStream_t s);
// device-to-device copy on the SMs (16-byte aligned buffers, a multiple of 16 bytes)
cudaError_t launch_copy_device(void *out, const void *in, size_t bytes, cudaStream_t s);

// batched form (FP32): persistent stage over a work list (Q: the group's shared constants,
// args: every instance's arguments); per-instance max speed
// tmaps: the instances' tensor maps of the staged input on the group's tile (indexed like
// args), used when Q.use_tma
cudaError_t launch_batch_stage(const StageArgs<float> &Q, const StageArgs<float> *args,
                               const CUtensorMap *tmaps, const int4 *items, int nitems,
                               int bufsz, size_t smem, int pos, int K, int TX, int TY, int CPT,
                               int *grid_out, cudaStream_t s);
// the tile shapes (TX, TY, cells per thread) the batch kernels compile for degree K
bool batch_tile_supported(int order, int tx, int ty, int cpt);
int batch_tile_candidates(int order, int (*out)[3], int max);
cudaError_t launch_batch_max_speed(const StageArgs<float> *args, const float *const *state,
                                   const int4 *items, int nitems, cudaStream_t s);
// every instance's device error word into out[0 .. n)
cudaError_t launch_batch_errors(const StageArgs<float> *args, int n, int *out, cudaStream_t s);
// start of a step for the n instances (time step, time, step count, next speed slots)
cudaError_t launch_batch_begin_step(const StageArgs<float> *args, int n, cudaStream_t s);

}  // namespace wb

// Context internals used by the batched form (defined in wb_capi.cu).
struct wb_ctx;
namespace wb {
// wb_create with the rows of every plane padded to a multiple of row_align elements
int ctx_create(const wb_config *cfg, int row_align, wb_ctx **out);
// RK2 stage arguments of a context for step phase p (0..5: buffer rotation mod 3 and
// parity mod 2, counted from the context's current position); FP32 contexts only.
int ctx_rk2_stage_args(wb_ctx *c, int phase, int dt_mode, double dt, StageArgs<float> out[2]);
// the tensor map staging TX x TY tiles (with halo) of the context's state buffer `base`;
// null where TMA cannot address it or is disabled (WB_NO_TMA=1)
const CUtensorMap *ctx_state_tmap(wb_ctx *c, const void *base, int TX, int TY);
// device address of the current state and of the context's run state
const float *ctx_state_f32(wb_ctx *c);
DevState *ctx_dev_state(wb_ctx *c);
// tile shape chosen for the context
void ctx_tile(wb_ctx *c, int *tx, int *ty, int *cpt);
// advance the host-side buffer rotation / parity bookkeeping by n RK2 steps
void ctx_advance(wb_ctx *c, int n);
// mark the fused wave-speed maxima of the current state as valid
void ctx_set_speed_valid(wb_ctx *c, bool v);
bool ctx_speed_valid(wb_ctx *c);
int ctx_parity(wb_ctx *c);
size_t ctx_dofs(wb_ctx *c);

// bytes of the partial-sum buffer the diagnostics need for an nx x ny grid
size_t diag_partial_bytes(int nx, int ny);

}  // namespace wb
