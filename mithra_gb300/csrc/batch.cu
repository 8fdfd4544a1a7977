// Batched instances (parameter sweeps) and launch-shape tuning.
//
// A sweep runs many small, independent FEL simulations (own mesh, bunch, undulator).  Each
// instance is an ordinary context; a batch composes the instances' captured step graphs as child
// graphs of one parent graph per step phase, so one cudaGraphLaunch advances every instance by
// one field step and their kernels overlap on the device.  The autotuner picks, per instance,
// the grid cap of the grid-stride kernels and the z extent of the bulk-tensor stencil tiles by
// timing real steps.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "../../include/mithra_gpu.h"
#include "ctx.h"

using namespace mithra;

struct mithra_batch {
  std::vector<mithra_ctx*> ctx;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t exec[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  std::vector<unsigned> generation[6];  // instance graph generations each parent graph was built from
  std::string err;
};

namespace {

int batch_fail(mithra_batch* b, int code, const char* msg) {
  b->err = msg;
  return code;
}

void drop(mithra_batch* b, int key) {
  if (b->exec[key]) cudaGraphExecDestroy(b->exec[key]);
  b->exec[key] = nullptr;
  b->generation[key].clear();
}

bool current(const mithra_batch* b, int key) {
  if (!b->exec[key] || b->generation[key].size() != b->ctx.size()) return false;
  for (size_t i = 0; i < b->ctx.size(); i++)
    if (b->generation[key][i] != b->ctx[i]->graph_generation) return false;
  return true;
}

// Parent graph of one step phase: one child graph per instance, no dependencies between them.
int build(mithra_batch* b, int key) {
  drop(b, key);
  cudaGraph_t parent;
  if (cudaGraphCreate(&parent, 0) != cudaSuccess) return batch_fail(b, MITHRA_ERR_CUDA, "cudaGraphCreate");
  for (mithra_ctx* c : b->ctx) {
    cudaGraph_t g;
    int r = capture_step(c, &g);
    if (r) {
      cudaGraphDestroy(parent);
      return r;
    }
    cudaGraphNode_t node;
    cudaError_t e = cudaGraphAddChildGraphNode(&node, parent, nullptr, 0, g);  // the child is cloned
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      cudaGraphDestroy(parent);
      return batch_fail(b, MITHRA_ERR_CUDA, cudaGetErrorString(e));
    }
  }
  cudaError_t e = cudaGraphInstantiate(&b->exec[key], parent, 0);
  cudaGraphDestroy(parent);
  if (e != cudaSuccess) return batch_fail(b, MITHRA_ERR_CUDA, cudaGetErrorString(e));
  for (mithra_ctx* c : b->ctx) b->generation[key].push_back(c->graph_generation);
  return MITHRA_OK;
}

}  // namespace

extern "C" {

int mithra_batch_create(mithra_ctx* const* ctxs, int n, mithra_batch** out) {
  if (!ctxs || n <= 0 || !out) return MITHRA_ERR_ARG;
  *out = nullptr;
  for (int i = 0; i < n; i++) {
    if (!ctxs[i]) return MITHRA_ERR_ARG;
    if (ctxs[i]->device != ctxs[0]->device) return MITHRA_ERR_ARG;
    if (step_key(ctxs[i]) != step_key(ctxs[0])) return MITHRA_ERR_STATE;
    for (int j = 0; j < i; j++)
      if (ctxs[j] == ctxs[i]) return MITHRA_ERR_ARG;
  }
  mithra_batch* b = new mithra_batch();
  b->ctx.assign(ctxs, ctxs + n);
  b->device = ctxs[0]->device;
  if (cudaSetDevice(b->device) != cudaSuccess || cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete b;
    return MITHRA_ERR_CUDA;
  }
  *out = b;
  return MITHRA_OK;
}

int mithra_batch_run(mithra_batch* b, int64_t nsteps) {
  if (!b || nsteps < 0) return MITHRA_ERR_ARG;
  for (mithra_ctx* c : b->ctx) {
    if (step_key(c) != step_key(b->ctx[0])) return batch_fail(b, MITHRA_ERR_STATE, "instances out of step");
    // the instances' own streams may still hold work (uploads): finish it before the batch stream
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return MITHRA_ERR_CUDA;
    int r = prepare_run(c, nsteps);
    if (r) return r;
  }
  for (int64_t s = 0; s < nsteps; s++) {
    const int key = step_key(b->ctx[0]);
    if (!current(b, key)) {
      int r = build(b, key);
      if (r) return r;
    }
    if (cudaGraphLaunch(b->exec[key], b->stream) != cudaSuccess) return batch_fail(b, MITHRA_ERR_CUDA, "graph launch");
    for (mithra_ctx* c : b->ctx) after_step(c);
  }
  if (cudaStreamSynchronize(b->stream) != cudaSuccess) return batch_fail(b, MITHRA_ERR_CUDA, "batch stream");
  for (mithra_ctx* c : b->ctx) {
    int r = finish_run(c);
    if (r) return r;
  }
  return MITHRA_OK;
}

int mithra_batch_run_timed(mithra_batch* b, int64_t nsteps, double* device_ms) {
  if (!b || !device_ms) return MITHRA_ERR_ARG;
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return MITHRA_ERR_CUDA;
  cudaEventRecord(e0, b->stream);
  int r = mithra_batch_run(b, nsteps);
  cudaEventRecord(e1, b->stream);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *device_ms = ms;
  return r;
}

int mithra_batch_destroy(mithra_batch* b) {
  if (!b) return MITHRA_ERR_ARG;
  for (int k = 0; k < 6; k++) drop(b, k);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return MITHRA_OK;
}

int mithra_gpu_set_tuning(mithra_ctx* ctx, const mithra_tuning* t) {
  if (!ctx || !t) return MITHRA_ERR_ARG;
  if (t->blocks_per_sm < 2 || t->blocks_per_sm > 64 || t->slab_planes < 16 || t->slab_planes > 256)
    return fail(ctx, MITHRA_ERR_ARG, "tuning out of range (blocks_per_sm %d, slab_planes %d)", t->blocks_per_sm,
                t->slab_planes);
  if (t->blocks_per_sm != ctx->tune.blocks_per_sm || t->slab_planes != ctx->tune.slab_planes) {
    ctx->tune = *t;
    invalidate_graphs(ctx);
  }
  return MITHRA_OK;
}

int mithra_gpu_set_wait_limit(mithra_ctx* ctx, int64_t iterations) {
  if (!ctx || iterations > 4000000000LL) return MITHRA_ERR_ARG;
  if (iterations < 0) iterations = -1;
  if (iterations != ctx->wait_limit) {
    ctx->wait_limit = iterations;
    invalidate_graphs(ctx);  // the limit is a launch argument baked into captured steps
  }
  return MITHRA_OK;
}

int mithra_gpu_get_tuning(const mithra_ctx* ctx, mithra_tuning* t) {
  if (!ctx || !t) return MITHRA_ERR_ARG;
  *t = ctx->tune;
  return MITHRA_OK;
}

int mithra_gpu_autotune(mithra_ctx* ctx, int steps_per_trial, mithra_tuning* chosen, double* ms_per_step) {
  if (!ctx || steps_per_trial < 1) return MITHRA_ERR_ARG;
  static const int kBlocks[] = {4, 8, 16, 32};
  static const int kSlabs[] = {32, 64, 128};
  const int n_slab = (ctx->precision == MITHRA_PRECISION_FP32) ? 3 : 1;  // the FP64 form has no slab tiles
  mithra_tuning best = ctx->tune;
  double best_ms = 1e300;
  for (int bi = 0; bi < 4; bi++)
    for (int si = 0; si < n_slab; si++) {
      mithra_tuning t{kBlocks[bi], n_slab == 1 ? ctx->tune.slab_planes : kSlabs[si]};
      int r = mithra_gpu_set_tuning(ctx, &t);
      if (r) return r;
      if ((r = mithra_gpu_run(ctx, 1))) return r;  // captures this shape's graphs
      double ms = 0.0;
      if ((r = mithra_gpu_run_timed(ctx, steps_per_trial, &ms))) return r;
      ms /= steps_per_trial;
      if (ms < best_ms) { best_ms = ms; best = t; }
    }
  int r = mithra_gpu_set_tuning(ctx, &best);
  if (r) return r;
  if (chosen) *chosen = best;
  if (ms_per_step) *ms_per_step = best_ms;
  return MITHRA_OK;
}

}  // extern "C"
