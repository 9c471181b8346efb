// wb_batch.cu -- batched form: n independent instances (own grid, degree, equilibrium,
// perturbation) advanced together by one persistent launch per RK stage over a work
// list of cell tiles, with the step sequence replayed from a CUDA graph.
//
// Each instance is a full FP32-perturbation context (its own state buffers, equilibrium
// tables and run state, hence its own CFL time step); the batch owns the work list, the
// per-instance stage arguments for the six step phases (buffer rotation mod 3 x step
// parity mod 2) and one stream.
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
  int4 *items = nullptr;  // all items, degree 2 first, then 1, then 0
  int nitems = 0;
  int koff[3] = {0, 0, 0};  // per degree: first item, item count, tile buffer, shared memory
  int kcount[3] = {0, 0, 0};
  int kbuf[3] = {0, 0, 0};
  size_t ksmem[3] = {0, 0, 0};
  int pos = 0;                        // some instance runs the positivity limiter
  StageArgs<float> *args = nullptr;  // [6 phases][2 stages][n]
  const float **state_ptrs = nullptr;  // [6 phases][n] current state per phase
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

// One launch per degree and stage; every stage-1 launch precedes every stage-2 launch
// (stream order), and launches of different degrees touch disjoint instances.
int launch_phase(wb_batch *b, int p) {
  const int n = (int)b->inst.size();
  int grid = 0;
  for (int st = 0; st < 2; ++st)
    for (int K = 2; K >= 0; --K)
      if (b->kcount[K] > 0)
        BCK(launch_batch_stage(b->args + ((size_t)p * 2 + st) * n, b->items + b->koff[K],
                               b->kcount[K], b->kbuf[K], b->ksmem[K], b->pos, K, &grid, b->stream));
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
  cudaFree(b->state_ptrs);
  for (wb_ctx *c : b->inst) wb_destroy(c);
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
    if (c.tile_x > 0 && (c.tile_x != 32 || c.tile_y != 8))
      return berr(b, WB_ERR_CONFIG, "the batch runs 32x8 tiles");
    if (c.riemann != WB_RIEMANN_LLF)
      return berr(b, WB_ERR_CONFIG, "the batch runs the LLF flux");
  }
  BCK(cudaSetDevice(b->device));
  BCK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  std::vector<int4> items;
  int bufmax[3] = {0, 0, 0};
  size_t fluxmax[3] = {0, 0, 0};
  for (int i = 0; i < n; ++i) {
    wb_config c = cfgs[i];
    if (c.tile_x <= 0) {
      c.tile_x = 32;
      c.tile_y = 8;
    }
    wb_ctx *ctx = nullptr;
    int rc = wb_create(&c, &ctx);
    if (rc) {
      std::string m = std::string("instance ") + std::to_string(i) + ": " + wb_last_error(ctx);
      wb_destroy(ctx);
      return berr(b, rc, m);
    }
    b->inst.push_back(ctx);
    b->cfgs.push_back(c);
    int tx, ty;
    ctx_tile(ctx, &tx, &ty);
    for (int j0 = 0; j0 < c.ny; j0 += ty)
      for (int i0 = 0; i0 < c.nx; i0 += tx)
        items.push_back(make_int4(i, i0, j0, (c.order << 24) | (tx << 12) | ty));
    const TileLayout L = tile_layout(c.order, WB_BASIS_P, tx, ty, c.limiter == 1 && c.order >= 1);
    if (c.limiter == 2 && c.order >= 1) b->pos = 1;
    const int K = c.order;
    bufmax[K] = std::max(bufmax[K], L.buf);
    fluxmax[K] = std::max(fluxmax[K], (size_t)NV * (K + 1) * ((size_t)ty * (tx + 1) + (size_t)(ty + 1) * tx));
  }
  // one contiguous range per degree (2, 1, 0), each launched by its own kernel
  std::stable_sort(items.begin(), items.end(), [](const int4 &a, const int4 &c) {
    return (a.w >> 24) > (c.w >> 24);
  });
  b->nitems = (int)items.size();
  for (const int4 &w : items) b->kcount[(w.w >> 24) & 0xff]++;
  b->koff[2] = 0;
  b->koff[1] = b->kcount[2];
  b->koff[0] = b->kcount[2] + b->kcount[1];
  for (int K = 0; K < 3; ++K) {
    b->kbuf[K] = bufmax[K];
    b->ksmem[K] = 64 * sizeof(double) + (2 * (size_t)bufmax[K] + fluxmax[K]) * sizeof(float);
  }
  BCK(cudaMalloc(&b->items, items.size() * sizeof(int4)));
  BCK(cudaMemcpy(b->items, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice));
  BCK(cudaMalloc(&b->args, (size_t)6 * 2 * n * sizeof(StageArgs<float>)));
  BCK(cudaMalloc(&b->state_ptrs, (size_t)6 * n * sizeof(float *)));
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

int wb_batch_sync(wb_batch *b) {
  if (!b) return WB_ERR_ARG;
  BCK(cudaSetDevice(b->device));
  BCK(cudaStreamSynchronize(b->stream));
  for (size_t i = 0; i < b->inst.size(); ++i) {
    int rc = wb_sync(b->inst[i]);
    if (rc) return berr(b, rc, std::string("instance ") + std::to_string(i) + ": " + wb_last_error(b->inst[i]));
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
