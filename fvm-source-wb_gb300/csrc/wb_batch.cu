// wb_batch.cu -- batched form: n independent instances (own grid, degree, equilibrium,
// perturbation) advanced together, per RK stage one persistent launch per group (the
// instances of one degree on one tile shape) over the group's work list of cell tiles,
// with the step sequence replayed from a CUDA graph.  wb_batch_autotune picks each
// (degree, size class) group's tile by timing.
//
// Each instance is a full FP32-perturbation context (its own state buffers, equilibrium
// tables and run state, hence its own CFL time step); the batch owns the work list, the
// per-instance stage arguments for the six step phases (buffer rotation mod 3 x step
// parity mod 2) and one stream.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/wb_capi.h"
#include "wb_internal.h"

using namespace wb;

struct wb_batch {
  std::vector<wb_ctx *> inst;
  std::vector<wb_config> cfgs;
  int device = 0;
  cudaStream_t stream = nullptr;
  // one stream per group and the fork/join events that order them against `stream`: the
  // groups advance disjoint instances, so each runs its two stages on its own branch
  static constexpr int kMaxBranches = 8;
  cudaStream_t branch[kMaxBranches] = {};
  cudaEvent_t fork = nullptr, join[kMaxBranches] = {};
  int4 *items = nullptr;  // all items, one contiguous range per group
  int nitems = 0;
  size_t items_cap = 0;
  // A group = the items of one degree K on one tile shape (and cells per thread) whose
  // instances share their physical constants, launched by its own kernel; rep is one of
  // its instances, whose stage arguments carry the group's constants to the launch.
  struct Group {
    int K, TX, TY, CPT, off, count, buf;
    size_t smem;
    int rep;
  };
  std::vector<Group> groups;
  // physics class of each instance: the first instance with the same physical constants,
  // boundary conditions and limiter (what the stage kernel takes from its launch constants)
  std::vector<int> phys;
  // Tile of each instance: pinned by its config, or the choice for its (degree, size class)
  std::vector<int> pin_tx, pin_ty, pin_cpt, size_class;
  // until wb_batch_autotune: the single grid's measured best per degree
  int choice[3][2][3] = {{{32, 16, 2}, {32, 16, 2}}, {{32, 16, 2}, {32, 16, 2}}, {{32, 8, 1}, {32, 8, 1}}};
  int pos = 0;                        // some instance runs the positivity limiter
  StageArgs<float> *args = nullptr;  // [6 phases][2 stages][n]
  std::vector<StageArgs<float>> hargs;  // host copy of args (the groups' launch constants)
  // Tensor maps of every stage's staged input on its instance's tile, indexed like args
  // ([6 phases][2 stages][n]; interior tiles are staged by one TMA copy), and a table for
  // the autotuner's candidates ([n], stage 1 of the current phase).  tma_ok: built.
  CUtensorMap *tmaps = nullptr, *tm_tune = nullptr;
  bool tma_ok = false;
  std::vector<int> tile_of_tx, tile_of_ty;  // each instance's tile in the work list
  const float **state_ptrs = nullptr;  // [6 phases][n] current state per phase
  int *errs = nullptr;                 // [n] the instances' device error words (wb_batch_sync)
  int phase = 0;
  int dt_mode = -1;
  double dt = 0.0;
  bool speed_valid = false;
  cudaGraphExec_t graph = nullptr;
  std::string err;
};

namespace {

int berr(wb_batch *b, int code, const std::string &m) {
  if (b) b->err = m;
  return code;
}
#define BCK(call)                                                                          \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) return berr(b, WB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Encode (cached per instance buffer and tile by the instance) the tensor maps of the
// instances' staged inputs: for args slots [first, first + count) of the host copy, on tile
// tx[i] x ty[i] of instance i, into the device table `dst`.  ok: every map could be made
// (false: WB_NO_TMA=1, or no encoder; the kernels then stage by cp.async).
int upload_tmaps(wb_batch *b, size_t first, size_t count, const std::vector<int> &tx,
                 const std::vector<int> &ty, CUtensorMap *dst, bool *ok) {
  const size_t n = b->inst.size();
  std::vector<CUtensorMap> h(count);
  std::memset(h.data(), 0, count * sizeof(CUtensorMap));
  *ok = true;
  for (size_t k = 0; k < count && *ok; ++k) {
    const size_t i = (first + k) % n;
    if (tx[i] <= 0) continue;  // not in this work list
    const CUtensorMap *m = ctx_state_tmap(b->inst[i], b->hargs[first + k].x, tx[i], ty[i]);
    if (!m) *ok = false;
    else h[k] = *m;
  }
  if (!*ok) return WB_OK;
  BCK(cudaMemcpyAsync(dst, h.data(), count * sizeof(CUtensorMap), cudaMemcpyHostToDevice, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  return WB_OK;
}

// The tensor maps of the work list (after the arguments or the tiles changed).
int build_tmaps(wb_batch *b) {
  b->tma_ok = false;
  if (b->hargs.empty() || b->tile_of_tx.empty()) return WB_OK;
  const size_t n = b->inst.size();
  if (!b->tmaps) BCK(cudaMalloc(&b->tmaps, (size_t)6 * 2 * n * sizeof(CUtensorMap)));
  return upload_tmaps(b, 0, (size_t)6 * 2 * n, b->tile_of_tx, b->tile_of_ty, b->tmaps, &b->tma_ok);
}

// (Re)build the per-phase stage arguments for the current dt mode.
int build_args(wb_batch *b, int dt_mode, double dt) {
  const int n = (int)b->inst.size();
  std::vector<StageArgs<float>> h((size_t)6 * 2 * n);
  std::vector<const float *> sp((size_t)6 * n);
  for (int p = 0; p < 6; ++p)
    for (int i = 0; i < n; ++i) {
      StageArgs<float> two[2];
      int rc = ctx_rk2_stage_args(b->inst[i], (p - b->phase + 6) % 6, dt_mode, dt, two);
      if (rc) return berr(b, rc, "instance is not an FP32 RK2 context");
      h[((size_t)p * 2 + 0) * n + i] = two[0];
      h[((size_t)p * 2 + 1) * n + i] = two[1];
      sp[(size_t)p * n + i] = two[0].x;
    }
  BCK(cudaMemcpyAsync(b->args, h.data(), h.size() * sizeof(StageArgs<float>), cudaMemcpyHostToDevice, b->stream));
  b->hargs = h;
  int rc = build_tmaps(b);
  if (rc) return rc;
  BCK(cudaMemcpyAsync(b->state_ptrs, sp.data(), sp.size() * sizeof(float *), cudaMemcpyHostToDevice, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  b->dt_mode = dt_mode;
  b->dt = dt;
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  return WB_OK;
}

// One launch for the step's start (every instance's time step), then per group its stage-1
// and stage-2 launches.  Groups advance disjoint instances, so each group's two stages
// run on a branch of their own (its stream, forked from and joined back to the batch
// stream): a group's second stage waits only for its own first stage, and the groups' launch
// tails overlap.  With more groups than branches the extra groups share the last branch.
int launch_phase(wb_batch *b, int p) {
  const int n = (int)b->inst.size();
  int grid = 0;
  BCK(launch_batch_begin_step(b->args + ((size_t)p * 2 + 0) * n, n, b->stream));
  BCK(cudaEventRecord(b->fork, b->stream));
  const int nb = std::min((int)b->groups.size(), wb_batch::kMaxBranches);
  for (int k = 0; k < nb; ++k) BCK(cudaStreamWaitEvent(b->branch[k], b->fork, 0));
  for (size_t gi = 0; gi < b->groups.size(); ++gi) {
    const wb_batch::Group &g = b->groups[gi];
    cudaStream_t s = b->branch[std::min((int)gi, nb - 1)];
    for (int st = 0; st < 2; ++st) {
      const size_t a = ((size_t)p * 2 + st) * n;
      StageArgs<float> Q = b->hargs[a + g.rep];
      Q.use_tma = b->tma_ok;
      BCK(launch_batch_stage(Q, b->args + a, b->tma_ok ? b->tmaps + a : nullptr, b->items + g.off,
                             g.count, g.buf, g.smem, b->pos, g.K, g.TX, g.TY, g.CPT, &grid, s));
    }
  }
  for (int k = 0; k < nb; ++k) {
    BCK(cudaEventRecord(b->join[k], b->branch[k]));
    BCK(cudaStreamWaitEvent(b->stream, b->join[k], 0));
  }
  return WB_OK;
}

// Whether two instances' stage arguments agree in everything the stage kernel takes from
// its launch constants rather than from the instance (tile_compute's A): physical
// constants, boundary conditions, limiter and flux options.
bool same_launch_constants(const StageArgs<float> &a, const StageArgs<float> &c) {
  return a.bc_x == c.bc_x && a.bc_y == c.bc_y && a.llf_speed == c.llf_speed &&
         a.limiter == c.limiter && a.lim_y == c.lim_y && a.riemann == c.riemann &&
         a.gamma == c.gamma && a.gm1 == c.gm1 && a.igm1 == c.igm1 && a.hgam == c.hgam &&
         a.gx == c.gx && a.gy == c.gy && a.rho0 == c.rho0 && a.p0 == c.p0 &&
         a.kpoly == c.kpoly && a.npoly == c.npoly && a.lim_norm == c.lim_norm &&
         a.lim_tol == c.lim_tol && a.pos_eps == c.pos_eps;
}

// Size class of an instance for the tile choice: small grids (side < 128) and the rest.
int size_class_of(const wb_config &c) { return std::max(c.nx, c.ny) < 128 ? 0 : 1; }

void instance_tile(const wb_batch *b, int i, int *tx, int *ty, int *cpt) {
  if (b->pin_tx[i] > 0) {
    *tx = b->pin_tx[i];
    *ty = b->pin_ty[i];
    *cpt = b->pin_cpt[i];
  } else {
    const int *t = b->choice[b->cfgs[i].order][b->size_class[i]];
    *tx = t[0];
    *ty = t[1];
    *cpt = t[2];
  }
}

// Items and groups of the instances `sel` (each on tile instance_tile, or on tx x ty at
// fcpt cells per thread when given), appended to items / groups.
void make_items(const wb_batch *b, const std::vector<int> &sel, int ftx, int fty, int fcpt,
                std::vector<int4> &items, std::vector<wb_batch::Group> &groups,
                std::vector<int> &tile_tx, std::vector<int> &tile_ty) {
  tile_tx.assign(b->inst.size(), 0);
  tile_ty.assign(b->inst.size(), 0);
  struct Key {
    int K, TX, TY, CPT, cls, i;
  };
  std::vector<Key> keys;
  for (int i : sel) {
    int tx = ftx, ty = fty, cpt = fcpt;
    if (tx <= 0) instance_tile(b, i, &tx, &ty, &cpt);
    keys.push_back({b->cfgs[i].order, tx, ty, cpt, b->phys[i], i});
  }
  // degree 2 first (the costliest launches start first), then by tile shape and physics
  std::stable_sort(keys.begin(), keys.end(), [](const Key &x, const Key &y) {
    if (x.K != y.K) return x.K > y.K;
    if (x.TX != y.TX) return x.TX > y.TX;
    if (x.TY != y.TY) return x.TY < y.TY;
    if (x.CPT != y.CPT) return x.CPT < y.CPT;
    return x.cls < y.cls;
  });
  int cls = -1;
  for (size_t k = 0; k < keys.size(); ++k) {
    const Key &q = keys[k];
    const wb_config &c = b->cfgs[q.i];
    tile_tx[q.i] = q.TX;
    tile_ty[q.i] = q.TY;
    if (groups.empty() || groups.back().K != q.K || groups.back().TX != q.TX ||
        groups.back().TY != q.TY || groups.back().CPT != q.CPT || cls != q.cls) {
      groups.push_back({q.K, q.TX, q.TY, q.CPT, (int)items.size(), 0, 0, 0, q.i});
      cls = q.cls;
    }
    wb_batch::Group &g = groups.back();
    // row by row; within a row the columns rotated by the row index, so that a CTA's
    // items it, it + G, ... do not keep to one tile column when G is a multiple of the row's
    // tile count (the boundary columns, staged element by element, would fall to the same
    // CTAs and make them stragglers)
    // Interior tiles (the staged block inside the grid) are flagged for TMA staging.
    // (Flagging them only on instances of at least 512 tiles, whose maps a CTA's successive
    // items mostly share, measured 3.66 ms per cfg4 step against 3.51 for all.)
    const int ntx = (c.nx + q.TX - 1) / q.TX;
    for (int r = 0, j0 = 0; j0 < c.ny; ++r, j0 += q.TY)
      for (int k = 0; k < ntx; ++k) {
        const int i0 = ((k + r) % ntx) * q.TX;
        const bool interior = i0 >= 4 && i0 + q.TX + 4 <= c.nx && j0 >= 1 && j0 + q.TY + 1 <= c.ny;
        items.push_back(make_int4(q.i, i0, j0,
                                  (interior ? 1 << 30 : 0) | (q.K << 24) | (q.TX << 12) | q.TY));
        ++g.count;
      }
    const TileLayout L = tile_layout(q.K, WB_BASIS_P, q.TX, q.TY, c.limiter == 1 && q.K >= 1);
    g.buf = std::max(g.buf, L.buf);
    const size_t flux = (size_t)NV * (q.K + 1) * ((size_t)q.TY * (q.TX + 1) + (size_t)(q.TY + 1) * q.TX);
    g.smem = std::max(g.smem, 64 * sizeof(double) + (2 * (size_t)g.buf + flux) * sizeof(float));
  }
}

// Upload items to b->items (grown as needed).
int upload_items(wb_batch *b, const std::vector<int4> &items) {
  if (items.size() > b->items_cap) {
    cudaFree(b->items);
    b->items = nullptr;
    b->items_cap = 0;
    BCK(cudaMalloc(&b->items, items.size() * sizeof(int4)));
    b->items_cap = items.size();
  }
  BCK(cudaMemcpyAsync(b->items, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice,
                      b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  return WB_OK;
}

// The work list of the current tile choices (the graph, which holds the old list, goes).
int build_worklist(wb_batch *b) {
  std::vector<int> all(b->inst.size());
  for (size_t i = 0; i < all.size(); ++i) all[i] = (int)i;
  std::vector<int4> items;
  std::vector<wb_batch::Group> groups;
  make_items(b, all, 0, 0, 0, items, groups, b->tile_of_tx, b->tile_of_ty);
  int rc = upload_items(b, items);
  if (!rc) rc = build_tmaps(b);
  if (rc) return rc;
  b->nitems = (int)items.size();
  b->groups = groups;
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  return WB_OK;
}

int ensure_batch_speed(wb_batch *b) {
  if (b->speed_valid) return WB_OK;
  const int n = (int)b->inst.size();
  for (int i = 0; i < n; ++i) {
    DevState *d = ctx_dev_state(b->inst[i]);
    BCK(cudaMemsetAsync(&d->smax[ctx_parity(b->inst[i])][0], 0, 2 * sizeof(unsigned long long), b->stream));
  }
  const int p = b->phase;
  BCK(launch_batch_max_speed(b->args + ((size_t)p * 2 + 0) * n, b->state_ptrs + (size_t)p * n,
                             b->items, b->nitems, b->stream));
  b->speed_valid = true;
  return WB_OK;
}

}  // namespace

extern "C" {

const char *wb_batch_last_error(const wb_batch *b) { return b ? b->err.c_str() : "null batch"; }

int wb_batch_destroy(wb_batch *b) {
  if (!b) return WB_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  cudaFree(b->items);
  cudaFree(b->args);
  cudaFree(b->tmaps);
  cudaFree(b->tm_tune);
  cudaFree(b->state_ptrs);
  cudaFree(b->errs);
  for (wb_ctx *c : b->inst) wb_destroy(c);
  for (int k = 0; k < wb_batch::kMaxBranches; ++k) {
    if (b->branch[k]) cudaStreamDestroy(b->branch[k]);
    if (b->join[k]) cudaEventDestroy(b->join[k]);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return WB_OK;
}

int wb_batch_create(const wb_config *cfgs, int32_t n, wb_batch **out) {
  if (!cfgs || !out || n < 1) return WB_ERR_ARG;
  wb_batch *b = new wb_batch();
  *out = b;
  b->device = cfgs[0].device;
  for (int i = 0; i < n; ++i) {
    const wb_config &c = cfgs[i];
    if (c.precision != WB_PREC_FP32 || c.integrator != WB_RK2 || c.device != b->device ||
        c.basis != WB_BASIS_P)
      return berr(b, WB_ERR_CONFIG,
                  "batch instances must be FP32-perturbation, SSP-RK2, total-degree basis, one device");
    if (c.tile_x > 0 &&
        !batch_tile_supported(c.order, c.tile_x, c.tile_y, c.cells_per_thread > 0 ? c.cells_per_thread : 1))
      return berr(b, WB_ERR_CONFIG,
                  "batch tiles are 32x8 or 16x16 at one cell per thread, 32x16 at two, 32x32 at four "
                  "(degree 0), or 0: chosen by the batch");
    if (c.riemann != WB_RIEMANN_LLF)
      return berr(b, WB_ERR_CONFIG, "the batch runs the LLF flux");
  }
  BCK(cudaSetDevice(b->device));
  BCK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  BCK(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
  for (int k = 0; k < wb_batch::kMaxBranches; ++k) {
    BCK(cudaStreamCreateWithFlags(&b->branch[k], cudaStreamNonBlocking));
    BCK(cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming));
  }
  for (int i = 0; i < n; ++i) {
    wb_config c = cfgs[i];
    b->pin_tx.push_back(c.tile_x > 0 ? c.tile_x : 0);
    b->pin_ty.push_back(c.tile_x > 0 ? c.tile_y : 0);
    b->pin_cpt.push_back(c.tile_x > 0 ? (c.cells_per_thread > 0 ? c.cells_per_thread : 1) : 0);
    b->size_class.push_back(size_class_of(c));
    if (c.tile_x <= 0) {  // the instance context's own tile is not used by the batch
      c.tile_x = 32;
      c.tile_y = 8;
      c.cells_per_thread = 1;
    }
    // rows padded to 16 bytes: every instance's tiles are staged in 16-byte chunks
    wb_ctx *ctx = nullptr;
    int rc = ctx_create(&c, 4, &ctx);
    if (rc) {
      std::string m = std::string("instance ") + std::to_string(i) + ": " + wb_last_error(ctx);
      wb_destroy(ctx);
      return berr(b, rc, m);
    }
    b->inst.push_back(ctx);
    b->cfgs.push_back(c);
    if (c.limiter == 2 && c.order >= 1) b->pos = 1;
    // physics class: compared on the stage arguments the kernel takes as launch constants
    StageArgs<float> ai[2], aj[2];
    if ((rc = ctx_rk2_stage_args(ctx, 0, 1, 0.0, ai))) return berr(b, rc, "instance arguments");
    int cls = i;
    for (int j = 0; j < i && cls == i; ++j)
      if (b->phys[j] == j && !ctx_rk2_stage_args(b->inst[j], 0, 1, 0.0, aj) &&
          same_launch_constants(ai[0], aj[0]))
        cls = j;
    b->phys.push_back(cls);
  }
  int rc = build_worklist(b);
  if (rc) return rc;
  BCK(cudaMalloc(&b->args, (size_t)6 * 2 * n * sizeof(StageArgs<float>)));
  BCK(cudaMalloc(&b->state_ptrs, (size_t)6 * n * sizeof(float *)));
  BCK(cudaMalloc(&b->errs, (size_t)n * sizeof(int)));
  return build_args(b, 1, 0.0);
}

int wb_batch_init_perturbation(wb_batch *b, const wb_perturbation *ics) {
  if (!b || !ics) return WB_ERR_ARG;
  BCK(cudaSetDevice(b->device));
  // every instance restarts from phase 0 of its rotation
  for (size_t i = 0; i < b->inst.size(); ++i) {
    int rc = wb_init_perturbation(b->inst[i], &ics[i]);
    if (rc) return berr(b, rc, std::string("instance ") + std::to_string(i) + ": " + wb_last_error(b->inst[i]));
  }
  b->phase = 0;
  b->speed_valid = false;
  return build_args(b, b->dt_mode < 0 ? 1 : b->dt_mode, b->dt);
}

int wb_batch_step(wb_batch *b, int32_t nsteps, double dt) {
  if (!b || nsteps < 0) return WB_ERR_ARG;
  BCK(cudaSetDevice(b->device));
  const int mode = dt > 0.0 ? 0 : 1;
  int rc;
  if (mode != b->dt_mode || (mode == 0 && dt != b->dt))
    if ((rc = build_args(b, mode, dt))) return rc;
  if ((rc = ensure_batch_speed(b))) return rc;
  int left = nsteps;
  while (left > 0) {
    if (b->phase == 0 && left >= 6) {
      if (!b->graph) {
        cudaGraph_t g;
        BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        for (int p = 0; p < 6; ++p) {
          rc = launch_phase(b, p);
          if (rc) {
            cudaStreamEndCapture(b->stream, &g);
            return rc;
          }
        }
        BCK(cudaStreamEndCapture(b->stream, &g));
        BCK(cudaGraphInstantiate(&b->graph, g, 0));
        cudaGraphDestroy(g);
      }
      BCK(cudaGraphLaunch(b->graph, b->stream));
      left -= 6;
      for (wb_ctx *c : b->inst) ctx_advance(c, 6);
      continue;
    }
    if ((rc = launch_phase(b, b->phase))) return rc;
    b->phase = (b->phase + 1) % 6;
    for (wb_ctx *c : b->inst) ctx_advance(c, 1);
    --left;
  }
  for (wb_ctx *c : b->inst) ctx_set_speed_valid(c, true);
  return WB_OK;
}

int wb_batch_autotune(wb_batch *b, int32_t reps, int32_t *tiles) {
  if (!b || reps < 1) return WB_ERR_ARG;
  BCK(cudaSetDevice(b->device));
  int rc = ensure_batch_speed(b);
  if (rc) return rc;
  const int n = (int)b->inst.size();
  // Candidates are timed on stage-1 launches of the current phase.  Stage 1 writes only
  // the buffer its real launch overwrites next; the step start before them writes the
  // phase's time step and the next-parity time and speed slots, which the real step
  // rewrites with the same values, so the instances' states are not changed.
  const StageArgs<float> *a1 = b->args + ((size_t)b->phase * 2 + 0) * n;
  BCK(launch_batch_begin_step(a1, n, b->stream));
  int cand[16][3];
  if (!b->tm_tune) BCK(cudaMalloc(&b->tm_tune, (size_t)n * sizeof(CUtensorMap)));
  // The candidates' items go through the work-list buffer, which a captured graph reads
  // (and which may be reallocated): the graph goes first.
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  BCK(cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return berr(b, WB_ERR_CUDA, "cudaEventCreate failed");
  }
  rc = WB_OK;
  for (int K = 0; K < 3 && !rc; ++K)
    for (int cls = 0; cls < 2 && !rc; ++cls) {
      std::vector<int> sel;
      for (int i = 0; i < n; ++i)
        if (b->pin_tx[i] == 0 && b->cfgs[i].order == K && b->size_class[i] == cls) sel.push_back(i);
      if (sel.empty()) continue;
      const int ncand = batch_tile_candidates(K, cand, 16);
      float best = 0.f;
      for (int c = 0; c < ncand && !rc; ++c) {
        std::vector<int4> items;
        std::vector<wb_batch::Group> groups;
        std::vector<int> ttx, tty;
        make_items(b, sel, cand[c][0], cand[c][1], cand[c][2], items, groups, ttx, tty);
        if ((rc = upload_items(b, items))) break;
        bool tok = false;
        if ((rc = upload_tmaps(b, (size_t)b->phase * 2 * n, n, ttx, tty, b->tm_tune, &tok))) break;
        float ms = 0.f;
        for (int r = 0; r <= reps && !rc; ++r) {  // launch 0 warms up
          if (r == 1 && cudaEventRecord(e0, b->stream) != cudaSuccess) rc = WB_ERR_CUDA;
          for (const wb_batch::Group &g : groups)
            if (!rc) {
              StageArgs<float> Q = b->hargs[(size_t)b->phase * 2 * n + g.rep];
              Q.use_tma = tok;
              if (launch_batch_stage(Q, a1, tok ? b->tm_tune : nullptr, b->items + g.off, g.count,
                                     g.buf, g.smem, b->pos, g.K, g.TX, g.TY, g.CPT, nullptr,
                                     b->stream) != cudaSuccess)
                rc = berr(b, WB_ERR_CUDA, "autotune launch failed");
            }
        }
        if (rc) break;
        if (cudaEventRecord(e1, b->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
            cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
          rc = berr(b, WB_ERR_CUDA, "autotune timing failed");
          break;
        }
        if (c == 0 || ms < best) {
          best = ms;
          b->choice[K][cls][0] = cand[c][0];
          b->choice[K][cls][1] = cand[c][1];
          b->choice[K][cls][2] = cand[c][2];
        }
      }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  // the real work list again, also after a failure (the buffer holds candidate items)
  const int rw = build_worklist(b);
  if (rc) return rc;
  if (rw) return rw;
  if (tiles)
    for (int K = 0; K < 3; ++K)
      for (int cls = 0; cls < 2; ++cls) {
        tiles[(K * 2 + cls) * 3 + 0] = b->choice[K][cls][0];
        tiles[(K * 2 + cls) * 3 + 1] = b->choice[K][cls][1];
        tiles[(K * 2 + cls) * 3 + 2] = b->choice[K][cls][2];
      }
  return WB_OK;
}

int wb_batch_sync(wb_batch *b) {
  if (!b) return WB_ERR_ARG;
  BCK(cudaSetDevice(b->device));
  // every instance's error word in one launch and one copy (a synchronous read per instance
  // costs about 10 us each: milliseconds for a batch of hundreds)
  const int n = (int)b->inst.size();
  std::vector<int> e(n);
  BCK(launch_batch_errors(b->args, n, b->errs, b->stream));
  BCK(cudaMemcpyAsync(e.data(), b->errs, n * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  for (int i = 0; i < n; ++i) {
    if (e[i] & 2)
      return berr(b, WB_ERR_TIMEOUT, "instance " + std::to_string(i) +
                                         ": a bounded device wait (tile copy) gave up");
    if (e[i])
      return berr(b, WB_ERR_NONPHYSICAL,
                  "instance " + std::to_string(i) +
                      ": non-finite or non-positive density/pressure in a cell mean");
  }
  return WB_OK;
}

int wb_batch_download(wb_batch *b, int32_t index, double *delta) {
  if (!b || !delta || index < 0 || index >= (int)b->inst.size()) return WB_ERR_ARG;
  BCK(cudaSetDevice(b->device));
  BCK(cudaStreamSynchronize(b->stream));
  int rc = wb_download_state(b->inst[index], delta, WB_LAYOUT_SOA);
  if (rc) return berr(b, rc, wb_last_error(b->inst[index]));
  return WB_OK;
}

int wb_batch_total_dofs(wb_batch *b, int64_t *dofs) {
  if (!b || !dofs) return WB_ERR_ARG;
  int64_t s = 0;
  for (wb_ctx *c : b->inst) s += (int64_t)ctx_dofs(c);
  *dofs = s;
  return WB_OK;
}

}  // extern "C"
