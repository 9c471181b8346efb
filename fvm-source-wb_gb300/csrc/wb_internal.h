// wb_internal.h -- entry points between the host layer (wb_capi.cu) and the
// per-precision kernel translation units.
#pragma once
#include "wb_types.h"

namespace wb {

#define WB_DECLARE_PRECISION_ENTRY_POINTS(R)                                                   \
  cudaError_t upload_tables(const Tab1D<R> *t);                                                \
  cudaError_t launch_stage(const StageArgs<R> &A, int K, int basis, int TX, int TY,            \
                           cudaStream_t s);                                                    \
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

// FP64-only diagnostics and precision conversion (defined in wb_kernels_f64.cu)
cudaError_t launch_norms(const AuxArgs &A, const Tab1D<double> *Td, const double *a,
                         const double *b, double *partial, double *out, int K, int basis,
                         cudaStream_t s);
cudaError_t launch_f32_to_f64(double *out, const float *in, long long n, cudaStream_t s);
cudaError_t launch_f64_to_f32(float *out, const double *in, long long n, cudaStream_t s);

// bytes of the partial-sum buffer the diagnostics need for an nx x ny grid
size_t diag_partial_bytes(int nx, int ny);

}  // namespace wb
