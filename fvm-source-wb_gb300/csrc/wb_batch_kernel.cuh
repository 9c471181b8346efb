// wb_batch_kernel.cuh -- persistent kernels of the batched form: every CTA walks a work
// list of (instance, tile) items spanning all instances of the batch (each with its
// own grid, degree and equilibrium), one launch per RK stage.  Included by the FP32
// translation unit (the batch runs the FP32-perturbation form).
#pragma once
#include "wb_stage.cuh"

namespace wb {

// item = {instance, i0, j0, (interior << 30) | (K << 24) | (TX << 12) | TY}; interior: the
// tile's staged block lies inside the grid (tma_tile), so a TMA copy can stage its modes
__device__ __forceinline__ bool item_interior(int4 w) { return (w.w >> 30) & 1; }
__device__ __forceinline__ void unpack_item(int4 w, int &K, int &TX, int &TY) {
  K = (w.w >> 24) & 0x3f;
  TX = (w.w >> 12) & 0xfff;
  TY = w.w & 0xfff;
}

// Copy one instance's stage arguments into shared memory: NCH 16-byte cp.async chunks,
// issued by threads first .. first + step - 1 of the caller's (thread t issues chunks
// t, t + step, ...).
template <typename R>
__device__ __forceinline__ void args_copy_async(const StageArgs<R> *src, StageArgs<R> *dst,
                                                const int t, const int step) {
  static_assert(sizeof(StageArgs<R>) % 16 == 0, "16-byte chunks");
  constexpr int NCH = (int)(sizeof(StageArgs<R>) / 16);
  for (int c = t; c < NCH; c += step)
    cp_async<16>(reinterpret_cast<char *>(dst) + 16 * c,
                 reinterpret_cast<const char *>(src) + 16 * c);
}

// A tensor map in global memory, written there by a host copy, made visible to the
// tensor-map proxy of the calling thread before its TMA copies use it, and fetched into
// the descriptor cache ahead of them.
__device__ __forceinline__ void tensormap_acquire(const CUtensorMap *m) {
  asm volatile("fence.proxy.tensormap::generic.acquire.sys [%0], 128;\n" ::"l"(m) : "memory");
  asm volatile("prefetch.tensormap [%0];\n" ::"l"(m) : "memory");
}

// Stage the tile of item w (its instance's arguments A already in shared memory) into buf,
// and the instance's time step (k_batch_begin_step computed it once per step) into sdt.
// An interior tile's modes come by one TMA copy through the instance's tensor map (when
// use_tma; thread NT - 32 acquired that map when the item's descriptor arrived).  `bar`
// (the buffer's mbarrier, one arrival per phase) gets exactly one arrival per item -- with
// the TMA byte count, or a plain one when the tile comes by cp.async -- so its phase parity
// for the j-th item in the buffer is j & 1 and no thread keeps any other record.  The
// bookkeeping is the last warp's: it has the fewest face passes.
template <typename R, int K, int TX, int TY, int NT>
__device__ __forceinline__ void item_stage(const StageArgs<R> &A, const int4 &w, double &sdt,
                                           R *buf, unsigned long long *bar,
                                           const CUtensorMap *__restrict__ tmaps,
                                           const int use_tma, int tid) {
  if (tid == NT - 1) cp_async<8>(&sdt, &A.dev->dt[A.parity]);
  const bool lim = A.limiter == 1 && A.lim_y && K >= 1;  // the same for the whole group
  const bool tma = item_interior(w) && tma_tile<TX, TY>(use_tma, A.nx, A.ny, w.y, w.z);
  if (tid == NT - 32) {
    if (tma) {
      constexpr unsigned bytes = NV * num_modes(K, 1) * (TY + 2) * (TX + 8) * sizeof(R);
      mbar_expect_tx(bar, bytes);
      tma_load_3d(buf, tmaps + w.x, w.y - 4, w.z - 1, 0, bar);  // the modes start the buffer
    } else {
      mbar_arrive(bar);
    }
  }
  tile_load_async<R, K, 1, TX, TY, NT>(A, lim, w.y, w.z, buf, tid, !tma);
}

// Shared-memory bytes of a batch CTA on TX x TY tiles of degree K (with the minmod rows):
// reduction scratch, two staged tiles, the face fluxes and the three item slots.
__host__ __device__ constexpr int batch_smem_bytes(int K, int TX, int TY) {
  return 64 * 8 +
         4 * (2 * ((NV * num_modes(K, 1) * (TX + 8) * (TY + 2) + NV * 2 * (TX + 8) +
                    (K + 1) * (TX + 2) + TX + 1 + (K + 1) * (TY + 2) + TY + 1 + 31) &
                   ~31) +
              NV * (K + 1) * (TY * (TX + 1) + (TY + 1) * TX)) +
         3 * ((int)sizeof(StageArgs<float>) + 16 + 8) + 16;
}
// Resident CTAs per SM the batch kernel is compiled for (its register budget is
// 65536 / (threads x this)): 4, 3 and 2 for degrees 0, 1 and 2, but never more than the
// shared memory admits (228 KB per SM, 1 KB of it reserved per CTA), where a higher count
// would only cap the registers (degree 1 on 32x16 tiles fits two: 122 registers instead
// of 80 and spills).
__host__ __device__ constexpr int batch_min_blocks(int K, int TX, int TY) {
  return (K == 0 ? 4 : K == 1 ? 3 : 2) < 233472 / (batch_smem_bytes(K, TX, TY) + 1024)
             ? (K == 0 ? 4 : K == 1 ? 3 : 2)
             : 233472 / (batch_smem_bytes(K, TX, TY) + 1024);
}

// Whether a batch launch stages interior items by TMA: tensor maps given, and the staging
// buffers 128-byte aligned as TMA destinations must be (checked, never assumed).  Kernel
// constants only, so it is recomputed where used rather than held in a register.
template <typename R>
__device__ __forceinline__ bool batch_tma_ok(const StageArgs<R> &Q, const CUtensorMap *tmaps,
                                             const R *bufs, int bufsz) {
  return Q.use_tma && tmaps != nullptr && (smem_u32(bufs) & 127u) == 0u &&
         ((bufsz * (int)sizeof(R)) & 127) == 0;
}

// Persistent batched stage for the items of one group (degree K, TX x TY tiles, CPT cells
// per thread, one set of physical constants): CTAs stride over the group's work list; the
// next item is staged (one TMA copy through its instance's tensor map for an interior
// tile, cp.async otherwise) while the current one is computed.  bufsz = the largest tile
// buffer of the group; tmaps = the instances' tensor maps for this stage's input (or
// null).  One kernel per degree gives each its own register budget (and
// occupancy) and no runtime dispatch on K.  Q: the stage arguments of one instance of the
// group, whose physical constants, boundary conditions, limiter and stage flags every
// instance of the group shares; as a kernel parameter they are free operands of the
// arithmetic (from shared memory they cost a load each and registers to hold them).  The
// item's own arguments (grid, buffers, spacing, equilibrium kind, run state) come from
// `args`, staged into shared memory with the tile.
template <typename R, int K, int TX, int TY, bool POS, int CPT>
__global__ void __launch_bounds__(TX * TY / CPT, batch_min_blocks(K, TX, TY))
    k_batch_stage(const __grid_constant__ StageArgs<R> Q, const StageArgs<R> *__restrict__ args,
                  const CUtensorMap *__restrict__ tmaps, const int4 *__restrict__ items,
                  int nitems, int bufsz) {
  constexpr int NT = TX * TY / CPT;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  // Three item slots: the item being computed, the item being staged, and the item whose
  // descriptor and instance arguments are on their way.  Every per-item value the threads
  // read comes from shared memory, so no warp waits on a global load at an item's start.
  __shared__ StageArgs<R> sA[3];      // instance arguments
  __shared__ __align__(16) int4 sW[3];  // work-list descriptors
  __shared__ double sdt[3];             // the instances' time steps
  __shared__ unsigned long long bar[2];  // one arrival per item staged into buffer b
  const int tid = threadIdx.x;
  double *red = reinterpret_cast<double *>(smem_raw);
  R *bufs = reinterpret_cast<R *>(smem_raw + 64 * sizeof(double));
  R *flux = bufs + 2 * bufsz;
  const int G = gridDim.x;
  const int it = blockIdx.x;
  // prologue: descriptors and arguments of items it and it + G, then item it's tile
  if (tid < 2 && it + tid * G < nitems) sW[tid] = items[it + tid * G];
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_fence_init();
  }
  __syncthreads();
  for (int j = 0; j < 2; ++j)
    if (it + j * G < nitems) {
      args_copy_async(args + sW[j].x, &sA[j], tid, NT);
      if (tid == NT - 32 && batch_tma_ok(Q, tmaps, bufs, bufsz) && item_interior(sW[j]))
        tensormap_acquire(tmaps + sW[j].x);
    }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  if (it < nitems)
    item_stage<R, K, TX, TY, NT>(sA[0], sW[0], sdt[0], bufs, &bar[0], tmaps,
                                 batch_tma_ok(Q, tmaps, bufs, bufsz), tid);
  cp_async_commit();
  // Item it (slot s, buffer k & 1) is computed while item it + G (slot s1) is staged; the
  // descriptor of item it + 2G (slot s2, which item it - G has left) comes by one cp.async
  // of the last warp's first thread right after the barrier, and the last warp copies that
  // item's arguments once it has computed its cells.  (The face passes fall unevenly on
  // the warps -- the first warps take the extra pass of a tile -- so the last warp has time
  // to spare.)  The barrier after item it's data arrives also frees item it - G's buffer,
  // slot and the flux area (as in k_stage).
  constexpr int LW = NT - 32;  // the last warp's first thread
  // Only k is carried across the compute body (registers are what the body lacks): the
  // item, its slot and its buffer follow from it.
  for (int k = 0; blockIdx.x + k * G < nitems; ++k) {
    const int it = blockIdx.x + k * G, s = k % 3, s1 = (k + 1) % 3;
    cp_async_wait<0>();
    // item it is the (k >> 1)-th of buffer k & 1; a wait that gives up stops the CTA
    const bool bad = !mbar_wait(&bar[k & 1], (k >> 1) & 1);
    if (bad && tid == 0) atomicOr(&sA[s].dev->err, 2);
    if (__syncthreads_or(bad)) {
      (void)mbar_wait(&bar[k & 1], (k >> 1) & 1);  // nothing may still be copying at exit
      break;
    }
    if (tid == LW && it + 2 * G < nitems) cp_async<16>(&sW[(k + 2) % 3], &items[it + 2 * G]);
    cp_async_commit();
    if (it + G < nitems)
      item_stage<R, K, TX, TY, NT>(sA[s1], sW[s1], sdt[s1], bufs + ((k + 1) & 1) * bufsz,
                                   &bar[(k + 1) & 1], tmaps,
                                   batch_tma_ok(Q, tmaps, bufs, bufsz), tid);
    cp_async_commit();
    const bool lim = Q.limiter == 1 && Q.lim_y && K >= 1;
    tile_compute<R, K, 1, TX, TY, POS ? WB_VAR_POSITIVITY : 0, CPT>(
        Q, sA[s], lim, sW[s].y, sW[s].z, bufs + (k & 1) * bufsz, flux, red, tid, sdt[s],
        nullptr, false, true);
    if (tid >= LW && blockIdx.x + (k + 2) * G < nitems) {
      // thread LW's descriptor copy is its second-newest group (the staging is the newest)
      const int s2 = (k + 2) % 3;
      int x = 0;
      if (tid == LW) {
        cp_async_wait<1>();
        x = sW[s2].x;
        if (batch_tma_ok(Q, tmaps, bufs, bufsz) && item_interior(sW[s2]))
          tensormap_acquire(tmaps + x);
      }
      x = __shfl_sync(0xffffffffu, x, 0);
      args_copy_async(args + x, &sA[s2], tid - LW, 32);
      cp_async_commit();
    }
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

// Every instance's device error word into out[i] (one small copy back for the whole batch
// instead of one synchronous copy per instance).
template <typename R>
__global__ void __launch_bounds__(128) k_batch_errors(const StageArgs<R> *__restrict__ args, int n,
                                                      int *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = args[i].dev->err;
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
