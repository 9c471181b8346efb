// wb_batch_kernel.cuh -- persistent kernels of the batched form: every CTA walks a work
// list of (instance, tile) items spanning all instances of the batch (each with its
// own grid, degree and equilibrium), one launch per RK stage.  Included by the FP32
// translation unit (the batch runs the FP32-perturbation form).
#pragma once
#include "wb_stage.cuh"

namespace wb {

// item = {instance, i0, j0, (K << 24) | (TX << 12) | TY}
__device__ __forceinline__ void unpack_item(int4 w, int &K, int &TX, int &TY) {
  K = (w.w >> 24) & 0xff;
  TX = (w.w >> 12) & 0xfff;
  TY = w.w & 0xfff;
}

// Stage the item `w` of degree K (instance arguments copied to sA, tile staged into buf)
// with NT threads.
template <typename R, int K, int TX, int TY, int NT>
__device__ __forceinline__ void item_load(const StageArgs<R> *__restrict__ args, const int4 w,
                                          StageArgs<R> &sA, double &sdt, R *buf, int tid) {
  constexpr int nthr = NT;
  static_assert(sizeof(StageArgs<R>) % 4 == 0, "word copy");
  const int *src = reinterpret_cast<const int *>(args + w.x);
  for (int k = tid; k < (int)(sizeof(StageArgs<R>) / 4); k += nthr)
    reinterpret_cast<int *>(&sA)[k] = src[k];
  const StageArgs<R> &A = args[w.x];
  // the instance's time step (k_batch_begin_step computed it once per step), staged with
  // the tile
  if (tid == 0) cp_async<8>(&sdt, &A.dev->dt[A.parity]);
  const bool lim = A.limiter == 1 && A.lim_y && K >= 1;  // the same for the whole group
  tile_load_async<R, K, 1, TX, TY, NT>(A, lim, w.y, w.z, buf, tid);
}

// Resident CTAs per SM the degree-K batch kernel is compiled for (register budget
// 65536 / (256 x this)); its shared memory (two staged tiles + the face fluxes) allows it.
__host__ __device__ constexpr int batch_min_blocks(int K) { return K == 0 ? 4 : K == 1 ? 3 : 2; }

// Persistent batched stage for the items of one group (degree K, TX x TY tiles, CPT cells
// per thread, one set of physical constants): CTAs stride over the group's work list; the
// next item is staged (cp.async) while the current one is computed.  bufsz = the largest
// tile buffer of the group.  One kernel per degree gives each its own register budget (and
// occupancy) and no runtime dispatch on K.  Q: the stage arguments of one instance of the
// group, whose physical constants, boundary conditions, limiter and stage flags every
// instance of the group shares; as a kernel parameter they are free operands of the
// arithmetic (from shared memory they cost a load each and registers to hold them).  The
// item's own arguments (grid, buffers, spacing, equilibrium kind, run state) come from
// `args`, staged into shared memory with the tile.
template <typename R, int K, int TX, int TY, bool POS, int CPT>
__global__ void __launch_bounds__(TX * TY / CPT, batch_min_blocks(K))
    k_batch_stage(const __grid_constant__ StageArgs<R> Q, const StageArgs<R> *__restrict__ args,
                  const int4 *__restrict__ items, int nitems, int bufsz) {
  constexpr int NT = TX * TY / CPT;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(16) StageArgs<R> sA[2];  // instance arguments of the staged items
  __shared__ double sdt[2];                     // and their time steps
  const int tid = threadIdx.x;
  double *red = reinterpret_cast<double *>(smem_raw);
  R *bufs = reinterpret_cast<R *>(smem_raw + 64 * sizeof(double));
  R *flux = bufs + 2 * bufsz;
  // Item it is staged while item it - G is computed; the barrier after its arrival also
  // frees the previous item's buffer, argument slot and flux area (as in k_stage).
  const int G = gridDim.x;
  int it = blockIdx.x;
  if (it < nitems) item_load<R, K, TX, TY, NT>(args, items[it], sA[0], sdt[0], bufs, tid);
  cp_async_commit();
  for (int k = 0; it < nitems; it += G, ++k) {
    cp_async_wait<0>();
    __syncthreads();
    if (it + G < nitems)
      item_load<R, K, TX, TY, NT>(args, items[it + G], sA[(k + 1) & 1], sdt[(k + 1) & 1],
                                  bufs + ((k + 1) & 1) * bufsz, tid);
    cp_async_commit();
    const int4 w = items[it];
    const StageArgs<R> &I = sA[k & 1];
    R *buf = bufs + (k & 1) * bufsz;
    const double dt = sdt[k & 1];
    const bool lim = Q.limiter == 1 && Q.lim_y && K >= 1;
    tile_compute<R, K, 1, TX, TY, POS ? WB_VAR_POSITIVITY : 0, CPT>(
        Q, I, lim, w.y, w.z, buf, flux, red, tid, dt, nullptr, false, true);
  }
  cp_async_wait<0>();
}

// Start of a step, one thread per instance: the step's time step (stage_dt, whose FP64
// divisions are slow on this part, once per instance instead of once per work item) into
// dev->dt[parity], and what the first stage of k_stage does for a single grid -- the next
// time and step count, and the cleared slots of the next wave-speed maxima.  args: the
// instances' first-stage arguments of the step.
template <typename R>
__global__ void __launch_bounds__(128) k_batch_begin_step(const StageArgs<R> *__restrict__ args,
                                                          int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const StageArgs<R> &A = args[i];
  const double dt = stage_dt(A);
  DevState *S = A.dev;
  S->dt[A.parity] = dt;
  S->t[A.parity ^ 1] = S->t[A.parity] + dt;
  S->nstep[A.parity ^ 1] = S->nstep[A.parity] + (dt > 0.0 ? 1 : 0);
  S->smax[A.parity ^ 1][0] = 0ull;
  S->smax[A.parity ^ 1][1] = 0ull;
}

// Per-instance wave-speed maxima of the cell means into dev->smax[parity] (the batched
// compute_max_speed), over the same work list.
template <typename R>
__global__ void __launch_bounds__(256)
    k_batch_max_speed(const StageArgs<R> *__restrict__ args, const R *const *__restrict__ state,
                      const int4 *__restrict__ items, int nitems) {
  __shared__ double red[64];
  const int tid = threadIdx.x;
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const int4 w = items[it];
    int K, TX, TY;
    unpack_item(w, K, TX, TY);
    const StageArgs<R> &A = args[w.x];
    const R *u = state[w.x];
    const int NQ = K + 1, NB = num_modes(K, 1);
    const Tab1D<R> &T = c_tab[K];
    // every cell of the item (a tile may hold more cells than the block has threads)
    double spx = 0.0, spy = 0.0;
    for (int c = tid; c < TX * TY; c += blockDim.x) {
      const int gi = w.y + c % TX, gj = w.z + c / TX;
      if (gi >= A.nx || gj >= A.ny) continue;
      const long long cell = (long long)gj * A.pitch + gi;
      R rbar = R(0), pbar = R(0);
      for (int qa = 0; qa < NQ; ++qa)
        for (int qb = 0; qb < NQ; ++qb) {
          R re, pe;
          eq_point(A, A.fxv[gi * NQ + qa], A.fyv[gj * NQ + qb], re, pe);
          R ww = R(0.25) * T.wq[qa] * T.wq[qb];
          rbar += re * ww;
          pbar += pe * ww;
        }
      R d0 = u[(long long)(0 * NB) * A.plane + cell], d1 = u[(long long)(1 * NB) * A.plane + cell];
      R d2 = u[(long long)(2 * NB) * A.plane + cell], d3 = u[(long long)(3 * NB) * A.plane + cell];
      R r, p, sx, sy;
      mean_wave_speed(A, rbar, pbar, d0, d1, d2, d3, r, p, sx, sy);
      if (!isfinite(sx) || !isfinite(sy)) {
        atomicOr(&A.dev->err, 1);
        continue;
      }
      spx = fmax(spx, (double)sx);
      spy = fmax(spy, (double)sy);
    }
    double mx = block_max(spx, red, tid, blockDim.x);
    double my = block_max(spy, red, tid, blockDim.x);
    if (tid == 0) {
      atomicMax(&A.dev->smax[A.parity][0], (unsigned long long)__double_as_longlong(mx));
      atomicMax(&A.dev->smax[A.parity][1], (unsigned long long)__double_as_longlong(my));
    }
  }
}

}  // namespace wb
