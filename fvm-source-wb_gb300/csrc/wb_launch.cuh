// wb_launch.cuh -- host-side dispatch from runtime (order, basis) to the compiled
// kernel instantiations of one precision.  Included once per precision TU.
#pragma once
#include "wb_aux.cuh"
#include "wb_internal.h"

namespace wb {

// (K, basis) -> instantiation; degree 0 has a single mode in both bases.
#define WB_DISPATCH_KB(K_, B_, ...)                        \
  do {                                                      \
    if ((K_) == 0) { constexpr int K = 0, BASIS = 0; __VA_ARGS__; } \
    else if ((K_) == 1 && (B_) == 0) { constexpr int K = 1, BASIS = 0; __VA_ARGS__; } \
    else if ((K_) == 1) { constexpr int K = 1, BASIS = 1; __VA_ARGS__; } \
    else if ((K_) == 2 && (B_) == 0) { constexpr int K = 2, BASIS = 0; __VA_ARGS__; } \
    else { constexpr int K = 2, BASIS = 1; __VA_ARGS__; }          \
  } while (0)

static inline dim3 cell_grid(int nx, int ny, dim3 blk) {
  return dim3((nx + blk.x - 1) / blk.x, (ny + blk.y - 1) / blk.y);
}

template <typename R>
static cudaError_t launch_limit_t(const StageArgs<R> &A, R *u, int K_, int B_, cudaStream_t s) {
  if (K_ < 1) return cudaSuccess;
  dim3 blk(32, 8), grd = cell_grid(A.nx, A.ny, blk);
  WB_DISPATCH_KB(K_, B_, { k_limit<R, K, BASIS><<<grd, blk, 0, s>>>(A, u); });
  return cudaGetLastError();
}

template <typename R>
static cudaError_t launch_max_speed_t(const StageArgs<R> &A, const R *u, int K_, int B_,
                                      cudaStream_t s) {
  dim3 blk(32, 8), grd = cell_grid(A.nx, A.ny, blk);
  WB_DISPATCH_KB(K_, B_, { k_max_speed<R, K, BASIS><<<grd, blk, 0, s>>>(A, u); });
  return cudaGetLastError();
}

template <typename R>
static cudaError_t launch_init_ic_t(const AuxArgs &A, const IcArgs &I, const Tab1D<double> *Td,
                                    R *u, int K_, int B_, cudaStream_t s) {
  dim3 blk(32, 4), grd = cell_grid(A.nx, A.ny, blk);
  WB_DISPATCH_KB(K_, B_, { k_init_ic<R, K, BASIS><<<grd, blk, 0, s>>>(A, I, Td, u); });
  return cudaGetLastError();
}

template <typename R>
static cudaError_t launch_to_fortran_t(const R *soa, double *f, int nx, int ny, long long P, int K_,
                                       cudaStream_t s) {
  dim3 blk(32, 8), grd = cell_grid(nx, ny, blk);
  if (K_ == 0) k_soa_to_fortran<R, 0><<<grd, blk, 0, s>>>(soa, f, nx, ny, P);
  else if (K_ == 1) k_soa_to_fortran<R, 1><<<grd, blk, 0, s>>>(soa, f, nx, ny, P);
  else k_soa_to_fortran<R, 2><<<grd, blk, 0, s>>>(soa, f, nx, ny, P);
  return cudaGetLastError();
}

template <typename R>
static cudaError_t launch_from_fortran_t(const double *f, R *soa, int nx, int ny, long long P,
                                         int K_, cudaStream_t s) {
  dim3 blk(32, 8), grd = cell_grid(nx, ny, blk);
  if (K_ == 0) k_fortran_to_soa<R, 0><<<grd, blk, 0, s>>>(f, soa, nx, ny, P);
  else if (K_ == 1) k_fortran_to_soa<R, 1><<<grd, blk, 0, s>>>(f, soa, nx, ny, P);
  else k_fortran_to_soa<R, 2><<<grd, blk, 0, s>>>(f, soa, nx, ny, P);
  return cudaGetLastError();
}

template <typename R>
static cudaError_t launch_sums_t(const AuxArgs &A, const Tab1D<double> *Td, const R *u,
                                 double *partial, double *out, int K_, int B_, cudaStream_t s) {
  dim3 blk(32, 8), grd = cell_grid(A.nx, A.ny, blk);
  WB_DISPATCH_KB(K_, B_, { k_sums<R, K, BASIS><<<grd, blk, 0, s>>>(A, Td, u, partial); });
  k_sums_final<<<1, 32, 0, s>>>(partial, (int)(grd.x * grd.y), out);
  return cudaGetLastError();
}

}  // namespace wb

// Defines the exported per-precision entry points declared in wb_internal.h.
#define WB_DEFINE_PRECISION_ENTRY_POINTS(R)                                                    \
  namespace wb {                                                                               \
  cudaError_t upload_tables_aux(const Tab1D<R> *t) {                                           \
    return cudaMemcpyToSymbol(c_tab, t, sizeof(Tab1D<R>) * (KMAX + 1));                       \
  }                                                                                            \
  cudaError_t launch_limit(const StageArgs<R> &A, R *u, int K, int basis, cudaStream_t s) {    \
    return launch_limit_t<R>(A, u, K, basis, s);                                               \
  }                                                                                            \
  cudaError_t launch_max_speed(const StageArgs<R> &A, const R *u, int K, int basis,            \
                               cudaStream_t s) {                                               \
    return launch_max_speed_t<R>(A, u, K, basis, s);                                           \
  }                                                                                            \
  cudaError_t launch_init_ic(const AuxArgs &A, const IcArgs &I, const Tab1D<double> *Td, R *u, \
                             int K, int basis, cudaStream_t s) {                               \
    return launch_init_ic_t<R>(A, I, Td, u, K, basis, s);                                      \
  }                                                                                            \
  cudaError_t launch_to_fortran(const R *soa, double *f, int nx, int ny, long long P, int K,   \
                                cudaStream_t s) {                                              \
    return launch_to_fortran_t<R>(soa, f, nx, ny, P, K, s);                                    \
  }                                                                                            \
  cudaError_t launch_from_fortran(const double *f, R *soa, int nx, int ny, long long P, int K, \
                                  cudaStream_t s) {                                            \
    return launch_from_fortran_t<R>(f, soa, nx, ny, P, K, s);                                  \
  }                                                                                            \
  cudaError_t launch_sums(const AuxArgs &A, const Tab1D<double> *Td, const R *u,               \
                          double *partial, double *out, int K, int basis, cudaStream_t s) {    \
    return launch_sums_t<R>(A, Td, u, partial, out, K, basis, s);                              \
  }                                                                                            \
  }
