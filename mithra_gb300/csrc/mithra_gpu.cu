// Context, stage orchestration and C ABI of the GB300 FdTd library (see include/mithra_gpu.h).
//
// One context = one domain on one GPU, one CUDA stream.  All device state (three time levels of
// A and phi, E/B, particles, power ring buffers, the time state) stays resident; a field step is
// a fixed sequence of kernels that is captured once per buffer rotation into a CUDA graph and
// replayed, so a march of many steps needs no host round trip.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mithra_gpu.h"
#include "ctx.h"
#include "field_kernels.cuh"
#include "particle_kernels.cuh"
#include "power_kernels.cuh"
#include "diag_kernels.cuh"

using namespace mithra;

namespace mithra {

int fail(mithra_ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

int grid_stride_blocks(const mithra_ctx* ctx, long long work, int block) {
  long long b = (work + block - 1) / block;
  long long cap = (long long)ctx->sm_count * ctx->tune.blocks_per_sm;
  return (int)std::max<long long>(1, std::min(b, cap));
}

int timer_begin(mithra_ctx* ctx, const char* name, int* slot, cudaEvent_t* a, cudaEvent_t* b) {
  *slot = -1;
  for (size_t i = 0; i < ctx->timers.size(); i++)
    if (ctx->timers[i].name == name) *slot = (int)i;
  if (*slot < 0) {
    ctx->timers.push_back({name, 0.0, 0});
    *slot = (int)ctx->timers.size() - 1;
  }
  if (ctx->ev_pool.size() >= 2) {
    *a = ctx->ev_pool.back(); ctx->ev_pool.pop_back();
    *b = ctx->ev_pool.back(); ctx->ev_pool.pop_back();
  } else {
    CK(cudaEventCreate(a));
    CK(cudaEventCreate(b));
  }
  CK(cudaEventRecord(*a, ctx->stream));
  return MITHRA_OK;
}

int timer_end(mithra_ctx* ctx, int slot, cudaEvent_t a, cudaEvent_t b) {
  CK(cudaEventRecord(b, ctx->stream));
  ctx->pending.push_back({slot, {a, b}});
  return MITHRA_OK;
}

int harvest_timers(mithra_ctx* ctx) {
  if (ctx->pending.empty()) return MITHRA_OK;
  CK(cudaStreamSynchronize(ctx->stream));
  for (auto& pe : ctx->pending) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, pe.second.first, pe.second.second));
    ctx->timers[pe.first].ms += ms;
    ctx->timers[pe.first].launches += 1;
    ctx->ev_pool.push_back(pe.second.first);
    ctx->ev_pool.push_back(pe.second.second);
  }
  ctx->pending.clear();
  return MITHRA_OK;
}

int staging(mithra_ctx* ctx, size_t bytes, void** p) {
  if (bytes > ctx->staging_bytes) {
    if (ctx->staging) {
      CK(cudaStreamSynchronize(ctx->stream));
      CK(cudaFree(ctx->staging));
      ctx->staging = nullptr;
    }
    CK(cudaMalloc(&ctx->staging, bytes));
    ctx->staging_bytes = bytes;
  }
  *p = ctx->staging;
  return MITHRA_OK;
}

void invalidate_graphs(mithra_ctx* ctx) {
  for (auto& gr : ctx->graph)
    if (gr) { cudaGraphExecDestroy(gr); gr = nullptr; }
  ctx->graph_generation++;
}

}  // namespace mithra

namespace {

constexpr int kPowerBlock = 128;

// ---- stages (each one reference member function) ---------------------------------------------

int run_potential(mithra_ctx* ctx, PotentialArgs<double> p, bool vector) {
  const GridDev& g = ctx->g;
  dim3 blk(32, 8), grd((g.N1 - 2 + 31) / 32, (g.N0 - 2 + 7) / 8, g.N2 - 2);
  const long long nfaces = 2LL * ((long long)(g.N1 - 2) * (g.N2 - 2) + (long long)(g.N0 - 2) * (g.N2 - 2) +
                                  (long long)(g.N0 - 2) * (g.N1 - 2));
  const long long nedges = 4LL * ((g.N2 - 2) + (g.N0 - 2) + (g.N1 - 2));
  int r;
  if (g.solver == 1)
    r = timed(ctx, vector ? "potential_interior_nsfd" : "scalar_interior_nsfd",
              [&] { k_potential_interior<double, true><<<grd, blk, 0, ctx->stream>>>(g, p); });
  else
    r = timed(ctx, vector ? "potential_interior_fd" : "scalar_interior_fd",
              [&] { k_potential_interior<double, false><<<grd, blk, 0, ctx->stream>>>(g, p); });
  if (r) return r;
  if (vector && ctx->seed_active && (r = stage_seed(ctx, p.np1))) return r;
  r = timed(ctx, vector ? "potential_faces" : "scalar_faces", [&] {
    k_potential_faces<double><<<grid_stride_blocks(ctx, nfaces, 256), 256, 0, ctx->stream>>>(g, p);
  });
  if (r) return r;
  if (g.order == 2) {
    r = timed(ctx, vector ? "potential_edges" : "scalar_edges", [&] {
      k_potential_edges<double><<<grid_stride_blocks(ctx, nedges, 256), 256, 0, ctx->stream>>>(g, p);
    });
    if (r) return r;
    r = timed(ctx, vector ? "potential_corners" : "scalar_corners",
              [&] { k_potential_corners<double><<<1, 32, 0, ctx->stream>>>(g, p); });
    if (r) return r;
  }
  return MITHRA_OK;
}

// full = true evaluates every interior plane; otherwise only the particle slab and the planes
// a power sample reads (the nodes the reference's lazy evaluation can touch).
int stage_eval_eb(mithra_ctx* ctx, bool full = false) {
  const GridDev& g = ctx->g;
  const double* fn = g.space_charge ? ctx->F[ctx->idx[1]] : nullptr;
  EBArgs<double> eb{ctx->A[ctx->idx[0]], ctx->A[ctx->idx[1]], fn, ctx->E64, ctx->B64,
                    full ? nullptr : ctx->st, ctx->plane_needed,
                    -1.0 / g.dt, 1.0 / (2.0 * g.dx), 1.0 / (2.0 * g.dy), 1.0 / (2.0 * g.dz)};
  constexpr int ks = 32;  // planes per block of the z-marching kernel
  dim3 grd((g.N1 - 2 + EBZ_TJ - 1) / EBZ_TJ, (g.N0 - 2 + EBZ_TI - 1) / EBZ_TI, (g.N2 - 2 + ks - 1) / ks);
  return timed(ctx, "eval_eb", [&] { k_eval_eb_z<double><<<grd, EBZ_TJ * EBZ_TI, 0, ctx->stream>>>(g, eb, ks); });
}

int stage_field_update(mithra_ctx* ctx) {
  if (ctx->precision == MITHRA_PRECISION_FP32) return fp32_field_update(ctx);
  const GridDev& g = ctx->g;
  int r;
  const Coeffs<double> k = make_coeffs<double>(g);
  PotentialArgs<double> pa{ctx->A[ctx->idx[0]], ctx->A[ctx->idx[1]], ctx->A[ctx->idx[2]], 3, g.a[4], k, ctx->Jedge, ctx->st};
  if ((r = run_potential(ctx, pa, true))) return r;
  if (g.space_charge) {
    PotentialArgs<double> pf{ctx->F[ctx->idx[0]], ctx->F[ctx->idx[1]], ctx->F[ctx->idx[2]], 1, g.a[5], k};
    if ((r = run_potential(ctx, pf, false))) return r;
  }
  return stage_eval_eb(ctx);
}

int stage_push(mithra_ctx* ctx, int save_rnm) {
  if (ctx->precision == MITHRA_PRECISION_FP32) return fp32_push(ctx, save_rnm);
  int r;
  if (ctx->P.und_planes) {
    const GridDev& g = ctx->g;
    const int n = ctx->P.n_und * (g.N2 + 1) * kUndSub;
    r = timed(ctx, "undulator_table", [&] {
      k_undulator_table64<<<std::max(1, (n + 255) / 256), 256, 0, ctx->stream>>>(
          ctx->und_dev, ctx->P.n_und, g.N2, g.zmin, g.dz, ctx->P.gamma, ctx->P.beta * ctx->P.c0, ctx->P.dt_shift,
          ctx->st, (UndPlane64*)ctx->und_table);
    });
    if (r) return r;
  }
  r = timed(ctx, "push", [&] {
    const int blocks = grid_stride_blocks(ctx, (long long)ctx->capacity, 256);
    if (ctx->P.n_opt + ctx->P.n_ext > 0)
      k_push_fp64<true><<<blocks, 256, 0, ctx->stream>>>(ctx->g, ctx->P, ctx->und_dev, ctx->pt, ctx->E64, ctx->B64,
                                                         ctx->st, save_rnm);
    else
      k_push_fp64<false><<<blocks, 256, 0, ctx->stream>>>(ctx->g, ctx->P, ctx->und_dev, ctx->pt, ctx->E64, ctx->B64,
                                                          ctx->st, save_rnm);
  });
  if (r) return r;
  return timed(ctx, "substep_end", [&] {
    k_substep_end<double><<<1, 1024, 0, ctx->stream>>>(ctx->pt, ctx->st, ctx->P.bunch_time_step);
  });
}

int stage_save_positions(mithra_ctx* ctx) {
  if (ctx->precision == MITHRA_PRECISION_FP32) return fp32_save_positions(ctx);
  return timed(ctx, "save_positions", [&] {
    k_save_positions<double><<<grid_stride_blocks(ctx, (long long)ctx->capacity, 256), 256, 0, ctx->stream>>>(ctx->pt, ctx->st);
  });
}

int stage_erase(mithra_ctx* ctx) {
  if (ctx->precision == MITHRA_PRECISION_FP32) return fp32_erase(ctx);
  return timed(ctx, "erase", [&] {
    k_erase_outside<double><<<grid_stride_blocks(ctx, (long long)ctx->capacity, 256), 256, 0, ctx->stream>>>(ctx->g, ctx->pt, ctx->st);
  });
}

// Solver::powerSample for every output.  `partial` (optional) replaces each output's own buffer
// of per-block partial sums: the sample kernel writes every slot the finish kernel reads within
// the same output, so one scratch array can serve all outputs in turn.
int stage_power(mithra_ctx* ctx, double* partial = nullptr) {
  for (size_t o = 0; o < ctx->power.size(); o++) {
    PowerDev pw = ctx->power[o].dev;
    if (partial) pw.partial = partial;
    const int blocks = pw.N * pw.blocks_per_plane;
    const size_t shm = (size_t)kPowerBlock * pw.Nl * sizeof(double);
    int r = timed(ctx, "power_sample", [&] {
      if (ctx->precision == MITHRA_PRECISION_FP64)
        k_power_sample<kPowerBlock, double><<<blocks, kPowerBlock, shm, ctx->stream>>>(ctx->g, pw, ctx->E64, ctx->B64,
                                                                                        ctx->g.cstride, 1, ctx->st);
      else
        k_power_sample<kPowerBlock, float><<<blocks, kPowerBlock, shm, ctx->stream>>>(ctx->g, pw, ctx->E, ctx->E + 4, 1,
                                                                                       kEBNode, ctx->st);
    });
    if (r) return r;
    const int last = (o + 1 == ctx->power.size());
    r = timed(ctx, "power_finish", [&] { k_power_finish<<<1, 256, 0, ctx->stream>>>(pw, ctx->st, last); });
    if (r) return r;
  }
  return MITHRA_OK;
}

DiagParticles diag_particles(const mithra_ctx* ctx);

// Solver::screenProfile (src/solver.cpp:2205-2257), when screens are set.
int stage_screen(mithra_ctx* ctx) {
  if (ctx->n_screens == 0) return MITHRA_OK;
  ScreenDev S;
  S.gamma = ctx->P.gamma; S.beta = ctx->P.beta; S.c0 = ctx->P.c0; S.dt_shift = ctx->P.dt_shift; S.dt = ctx->g.dt;
  S.n = ctx->n_screens; S.lz = ctx->screen_lz; S.rec = ctx->screen_rec; S.key = ctx->screen_key;
  S.count = ctx->screen_count; S.cap = ctx->screen_cap;
  const DiagParticles P = diag_particles(ctx);
  return timed(ctx, "screen", [&] {
    k_screen<<<grid_stride_blocks(ctx, (long long)ctx->capacity, 256), 256, 0, ctx->stream>>>(ctx->g, P, S, ctx->st);
  });
}

void rotate(mithra_ctx* ctx) {
  const int np1 = ctx->idx[0], n = ctx->idx[1], nm1 = ctx->idx[2];
  ctx->idx[0] = nm1;
  ctx->idx[1] = np1;
  ctx->idx[2] = n;
}

int stage_current(mithra_ctx* ctx) {
  if (ctx->precision == MITHRA_PRECISION_FP32) return fp32_current(ctx);
  const GridDev& g = ctx->g;
  double* J = ctx->Jedge;  // edge form; the field update reads it (PotentialArgs::jedge)
  CK(cudaMemsetAsync(J, 0, (size_t)3 * g.cstride * sizeof(double), ctx->stream));
  double* rho = nullptr;
  if (g.space_charge) {
    rho = ctx->F[ctx->idx[0]];
    CK(cudaMemsetAsync(rho, 0, (size_t)g.cstride * sizeof(double), ctx->stream));
  }
  return timed(ctx, "deposit", [&] {
    k_deposit_fp64<<<grid_stride_blocks(ctx, (long long)ctx->capacity, 256), 256, 0, ctx->stream>>>(g, ctx->pt, ctx->st, J, rho);
  });
}

int stage_advance_time(mithra_ctx* ctx) {
  return timed(ctx, "advance_time", [&] { k_advance_time<<<1, 32, 0, ctx->stream>>>(ctx->st, ctx->g.dt); });
}

// Number of iterations of `for (Double t = 0.0; t < nUpdateBunch_; t += 1.0)` (src/solver.cpp:1316).
int n_substeps(const mithra_ctx* ctx) {
  int n = 0;
  for (double t = 0.0; t < ctx->push_desc.n_update_bunch; t += 1.0) n++;
  return n;
}

// The body of the main loop of Solver::solve (src/solver.cpp:1300-1399), diagnostics other
// than the screens and the power sample omitted.  Ends with the buffer rotation of
// FdTd::fieldShift.
int enqueue_step(mithra_ctx* ctx) {
  int r;
  if ((r = stage_field_update(ctx))) return r;
  const int ns = n_substeps(ctx);
  for (int s = 0; s < ns; s++)
    if ((r = stage_push(ctx, s == 0))) return r;
  if (ns == 0 && (r = stage_save_positions(ctx))) return r;
  // The mixed-form push flags non-finite particles itself, so its erase pass is needed only
  // when no push ran.
  if ((ctx->precision != MITHRA_PRECISION_FP32 || ns == 0) && (r = stage_erase(ctx))) return r;
  if ((r = stage_screen(ctx))) return r;
  if ((r = stage_power(ctx))) return r;
  rotate(ctx);
  if ((r = stage_current(ctx))) return r;
  return stage_advance_time(ctx);
}

// Makes room for `extra` more rows in the device row log; the count of rows already logged is
// tracked on the host, so no device round trip is needed when there is room.
int ensure_rows(mithra_ctx* ctx, long long extra) {
  if (ctx->power.empty()) return MITHRA_OK;
  const long long need = ctx->rows_pending + extra;
  if (need <= ctx->row_cap) return MITHRA_OK;
  CK(cudaStreamSynchronize(ctx->stream));
  long long cap = std::max(need, 2 * ctx->row_cap + 64);
  for (auto& po : ctx->power) {
    const long long rowlen = (long long)po.dev.N * (1 + po.dev.Nl);
    double* nr = nullptr;
    CK(dalloc(&nr, (size_t)(cap * rowlen)));
    if (po.rows) {
      CK(cudaMemcpyAsync(nr, po.rows, (size_t)(ctx->row_cap * rowlen) * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
      CK(cudaStreamSynchronize(ctx->stream));
      CK(cudaFree(po.rows));
    }
    po.rows = nr;
    po.dev.rows = nr;
    po.dev.row_cap = cap;
  }
  ctx->row_cap = cap;
  invalidate_graphs(ctx);
  return MITHRA_OK;
}

BeamDev beam_from_desc(const mithra_beam_desc& d) {
  BeamDev b{};
  b.type = d.type;
  for (int c = 0; c < 3; c++) { b.pos[c] = d.position[c]; b.dir[c] = d.direction[c]; b.pol[c] = d.polarization[c]; }
  // cross(direction, polarization), src/fieldvector.h:197-204
  b.yv[0] = b.dir[1] * b.pol[2] - b.dir[2] * b.pol[1];
  b.yv[1] = b.dir[2] * b.pol[0] - b.dir[0] * b.pol[2];
  b.yv[2] = b.dir[0] * b.pol[1] - b.dir[1] * b.pol[0];
  b.amplitude = d.amplitude; b.r0 = d.radius[0]; b.r1 = d.radius[1]; b.o0 = d.order[0]; b.o1 = d.order[1];
  b.l = d.wavelength; b.zR0 = d.rayleigh[0]; b.zR1 = d.rayleigh[1];
  b.sig.type = d.signal_type; b.sig.t0 = d.signal_t0; b.sig.s = d.signal_s; b.sig.f0 = d.signal_f0;
  b.sig.cep = d.signal_cep; b.sig.nR = d.signal_nr; b.sig.g0 = d.signal_sigma[0]; b.sig.g1 = d.signal_sigma[1];
  return b;
}

// Uploads the module table and the laser beams (optical undulators first, then the external
// fields) and points the push parameters at them.
int upload_beams(mithra_ctx* ctx) {
  std::vector<BeamDev> all(ctx->opt_beams);
  all.insert(all.end(), ctx->ext_beams.begin(), ctx->ext_beams.end());
  PushDev& P = ctx->P;
  P.n_opt = (int)ctx->opt_beams.size();
  P.ext0 = P.n_opt;
  P.n_ext = (int)ctx->ext_beams.size();
  P.beams = all.empty() ? nullptr : ctx->beams_dev;
  if (!all.empty())
    CK(cudaMemcpyAsync(ctx->beams_dev, all.data(), all.size() * sizeof(BeamDev), cudaMemcpyHostToDevice, ctx->stream));
  if (P.n_und)
    CK(cudaMemcpyAsync(ctx->und_dev, ctx->und_host.data(), P.n_und * sizeof(UndDev), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  invalidate_graphs(ctx);
  return MITHRA_OK;
}

int check_state(mithra_ctx* ctx) {
  CK(cudaMemcpyAsync(ctx->st_host, ctx->st, sizeof(StateDev), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (ctx->st_host->overflow)
    return fail(ctx, MITHRA_ERR_CAPACITY, "particle capacity %lld exceeded by z-face copies", ctx->st_host->capacity);
  if (ctx->f32.tma_error) {
    int e = 0;
    CK(cudaMemcpy(&e, ctx->f32.tma_error, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) return fail(ctx, MITHRA_ERR_STATE, "interior stencil: bulk-tensor copy %s (code %d)",
                       e == 2 ? "refused on an unaligned shared-memory slot" : "wait timed out", e);
  }
  return MITHRA_OK;
}

}  // namespace

namespace mithra {

int step_key(const mithra_ctx* ctx) { return ctx->idx[0] + 3 * ctx->f32.parity; }

int capture_step(mithra_ctx* ctx, cudaGraph_t* out) {
  const int saved[3] = {ctx->idx[0], ctx->idx[1], ctx->idx[2]};
  const Fp32State saved_f32 = ctx->f32;
  ctx->f32.sort_pending = false;  // a step graph sorts on its rotation only
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  ctx->launch_counter = 0;
  const int r = enqueue_step(ctx);
  ctx->launches_per_step = ctx->launch_counter;
  cudaError_t ce = cudaStreamEndCapture(ctx->stream, out);
  // enqueue_step rotated the indices (and swapped the particle buffer sets) while recording;
  // restore them so that a launch of the graph followed by after_step applies them once.
  ctx->idx[0] = saved[0]; ctx->idx[1] = saved[1]; ctx->idx[2] = saved[2];
  ctx->f32 = saved_f32;
  if (r) return r;
  if (ce != cudaSuccess) return fail(ctx, MITHRA_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
  return MITHRA_OK;
}

void after_step(mithra_ctx* ctx) {
  rotate(ctx);
  if (ctx->precision == MITHRA_PRECISION_FP32 && fp32_sorts_this_step(ctx)) {
    fp32_after_step(ctx);
    ctx->f32.sort_pending = false;
  }
}

int prepare_run(mithra_ctx* ctx, int64_t nsteps) {
  if (!ctx->particles_loaded) return fail(ctx, MITHRA_ERR_STATE, "no particles uploaded");
  int r = ensure_rows(ctx, nsteps);
  if (r) return r;
  if (!ctx->power.empty()) ctx->rows_pending += nsteps;
  return MITHRA_OK;
}

int finish_run(mithra_ctx* ctx) { return check_state(ctx); }

int stage_seed(mithra_ctx* ctx, void* anp1) {
  const GridDev& g = ctx->g;
  if (g.N0 < 5 || g.N1 < 5 || g.N2 < 5) return MITHRA_OK;  // no TF/SF planes inside the domain
  for (int dir = 0; dir < 3; dir++) {
    const long long items = (long long)((dir == 0) ? g.N1 - 4 : g.N0 - 4) * ((dir == 2) ? g.N1 - 4 : g.N2 - 4);
    const int blocks = grid_stride_blocks(ctx, items, 256);
    int r = timed(ctx, "seed_inject", [&] {
      if (ctx->precision == MITHRA_PRECISION_FP64)
        k_seed_inject<double><<<blocks, 256, 0, ctx->stream>>>(g, ctx->seed, (double*)anp1, ctx->st, dir);
      else
        k_seed_inject<float><<<blocks, 256, 0, ctx->stream>>>(g, ctx->seed, (float*)anp1, ctx->st, dir);
    });
    if (r) return r;
  }
  return MITHRA_OK;
}

}  // namespace mithra


// ---- C ABI ----------------------------------------------------------------------------------

extern "C" {

int mithra_gpu_last_error(const mithra_ctx* ctx, char* buf, size_t len) {
  if (!ctx || !buf || !len) return MITHRA_ERR_ARG;
  snprintf(buf, len, "%s", ctx->err.c_str());
  return MITHRA_OK;
}

int mithra_gpu_create(const mithra_grid_desc* gd, const mithra_push_desc* pd, int precision, int device,
                      size_t particle_capacity, mithra_ctx** out) {
  if (!gd || !pd || !out) return MITHRA_ERR_ARG;
  *out = nullptr;
  if (gd->N0 < 4 || gd->N1 < 4 || gd->N2 < 4) return MITHRA_ERR_ARG;
  if (gd->solver != 0 && gd->solver != 1) return MITHRA_ERR_ARG;
  if (gd->truncation_order != 1 && gd->truncation_order != 2) return MITHRA_ERR_ARG;
  if (precision != MITHRA_PRECISION_FP64 && precision != MITHRA_PRECISION_FP32) return MITHRA_ERR_ARG;
  mithra_ctx* ctx = new mithra_ctx();
  ctx->device = device;
  ctx->precision = precision;
  ctx->grid_desc = *gd;
  ctx->push_desc = *pd;
  int rc = [&]() -> int {
    CK(cudaSetDevice(device));
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    ctx->sm_count = sms;
    CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    GridDev& g = ctx->g;
    g.N0 = gd->N0; g.N1 = gd->N1; g.N2 = gd->N2;
    g.P1 = (int)round_up(gd->N1, 8);
    g.plane = (long long)g.N0 * g.P1;
    g.cstride = round_up((long long)g.N2 * g.plane, 64);
    g.solver = gd->solver; g.order = gd->truncation_order; g.space_charge = gd->space_charge;
    memcpy(g.a, gd->a, sizeof g.a);
    g.nsfd_alpha = gd->nsfd_alpha; g.nsfd_beta = gd->nsfd_beta;
    memcpy(g.bB, gd->bB, sizeof g.bB); memcpy(g.cB, gd->cB, sizeof g.cB); memcpy(g.dB, gd->dB, sizeof g.dB);
    memcpy(g.eE, gd->eE, sizeof g.eE); memcpy(g.fE, gd->fE, sizeof g.fE); memcpy(g.gE, gd->gE, sizeof g.gE);
    memcpy(g.hC, gd->hC, sizeof g.hC);
    g.dt = gd->dt; g.dx = gd->dx; g.dy = gd->dy; g.dz = gd->dz;
    g.rdx = 1.0 / gd->dx; g.rdy = 1.0 / gd->dy; g.rdz = 1.0 / gd->dz;
    g.xmin = gd->xmin; g.xmax = gd->xmax; g.ymin = gd->ymin; g.ymax = gd->ymax;
    g.zmin = gd->zmin; g.zmax = gd->zmax; g.zp0 = gd->zp0; g.zp1 = gd->zp1; g.Lz = gd->Lz;
    PushDev& P = ctx->P;
    P.dtb = pd->dtb; P.r1 = pd->r1; P.r2 = pd->r2; P.gamma = pd->gamma; P.beta = pd->beta; P.c0 = pd->c0;
    P.dt_shift = pd->dt_shift; P.bunch_time_step = pd->bunch_time_step; P.n_und = 0; P.und0_dist = 0.0;
    P.inv_r2 = 1.0 / pd->r2;
    P.und_planes = nullptr;
    P.gdz = pd->gamma * gd->dz;
    P.gdz_sub = P.gdz / kUndSub;
    P.beams = nullptr; P.ext0 = 0; P.n_ext = 0; P.n_opt = 0;
    CK(dalloc(&ctx->und_dev, kMaxUndulators));
    CK(dalloc(&ctx->beams_dev, kMaxUndulators + MITHRA_MAX_EXT_FIELDS));
    const size_t nf = (size_t)3 * g.cstride;
    ctx->capacity = std::max<size_t>(particle_capacity, 1);
    if (precision == MITHRA_PRECISION_FP64) {
      CK(dalloc(&ctx->Jedge, nf));
      CK(cudaMemsetAsync(ctx->Jedge, 0, nf * sizeof(double), ctx->stream));
      for (int b = 0; b < 3; b++) {
        CK(dalloc(&ctx->A[b], nf));
        CK(cudaMemsetAsync(ctx->A[b], 0, nf * sizeof(double), ctx->stream));
        if (g.space_charge) {
          CK(dalloc(&ctx->F[b], (size_t)g.cstride));
          CK(cudaMemsetAsync(ctx->F[b], 0, (size_t)g.cstride * sizeof(double), ctx->stream));
        }
      }
      ParticlesDev<double>& pt = ctx->pt;
      const size_t c = ctx->capacity;
      CK(dalloc(&pt.x, c)); CK(dalloc(&pt.y, c)); CK(dalloc(&pt.z, c));
      CK(dalloc(&pt.gx, c)); CK(dalloc(&pt.gy, c)); CK(dalloc(&pt.gz, c));
      CK(dalloc(&pt.mx, c)); CK(dalloc(&pt.my, c)); CK(dalloc(&pt.mz, c));
      CK(dalloc(&pt.q, c)); CK(dalloc(&pt.e, c));
      CK(dalloc(&pt.status, c)); CK(dalloc(&pt.cross, c));
    } else {
      int r = fp32_alloc(ctx);
      if (r) return r;
    }
    if (precision == MITHRA_PRECISION_FP64) {
      CK(dalloc(&ctx->E64, nf));
      CK(dalloc(&ctx->B64, nf));
      CK(cudaMemsetAsync(ctx->E64, 0, nf * sizeof(double), ctx->stream));
      CK(cudaMemsetAsync(ctx->B64, 0, nf * sizeof(double), ctx->stream));
    } else {
      const size_t ne = (size_t)kEBNode * g.cstride;  // node records {E, 0, B, 0}
      CK(dalloc(&ctx->E, ne));
      CK(cudaMemsetAsync(ctx->E, 0, ne * sizeof(float), ctx->stream));
    }
    CK(dalloc(&ctx->plane_needed, (size_t)g.N2));
    CK(cudaMemsetAsync(ctx->plane_needed, 0, (size_t)g.N2, ctx->stream));
    CK(dalloc(&ctx->st, 1));
    CK(cudaMallocHost((void**)&ctx->st_host, sizeof(StateDev)));
    memset(ctx->st_host, 0, sizeof(StateDev));
    ctx->st_host->capacity = (long long)ctx->capacity;
    ctx->st_host->k_lo = 0;
    ctx->st_host->k_hi = g.N2 - 1;
    ctx->st_host->k_lo_next = 0x7fffffff;
    ctx->st_host->k_hi_next = -0x7fffffff;
    CK(cudaMemcpyAsync(ctx->st, ctx->st_host, sizeof(StateDev), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return MITHRA_OK;
  }();
  if (rc) {
    char msg[512];
    snprintf(msg, sizeof msg, "%s", ctx->err.c_str());
    mithra_gpu_destroy(ctx);
    fprintf(stderr, "mithra_gpu_create: %s\n", msg);
    return rc;
  }
  *out = ctx;
  return MITHRA_OK;
}

int mithra_gpu_destroy(mithra_ctx* ctx) {
  if (!ctx) return MITHRA_ERR_ARG;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  invalidate_graphs(ctx);
  for (int b = 0; b < 3; b++) { cudaFree(ctx->A[b]); cudaFree(ctx->F[b]); }
  ParticlesDev<double>& pt = ctx->pt;
  void* ps[] = {pt.x, pt.y, pt.z, pt.gx, pt.gy, pt.gz, pt.mx, pt.my, pt.mz, pt.q, pt.e, pt.status, pt.cross};
  for (void* p : ps) cudaFree(p);
  fp32_free(ctx);
  cudaFree(ctx->staging);
  cudaFree(ctx->E64); cudaFree(ctx->B64); cudaFree(ctx->plane_needed); cudaFree(ctx->und_table);
  cudaFree(ctx->eb_planes);
  cudaFree(ctx->E); cudaFree(ctx->B); cudaFree(ctx->st); cudaFree(ctx->und_dev); cudaFree(ctx->beams_dev); cudaFree(ctx->Jedge);
  cudaFree(ctx->diag_partial); cudaFree(ctx->diag_out);
  cudaFree(ctx->screen_lz); cudaFree(ctx->screen_rec); cudaFree(ctx->screen_key); cudaFree(ctx->screen_count);
  if (ctx->st_host) cudaFreeHost(ctx->st_host);
  for (auto& po : ctx->power) {
    void* qs[] = {po.z, po.dzr, po.tw_re, po.tw_im, po.fdt, po.partial, po.rows, po.plane_k, po.plane_slot, po.run};
    for (void* q : qs) cudaFree(q);
  }
  for (auto& pe : ctx->pending) { cudaEventDestroy(pe.second.first); cudaEventDestroy(pe.second.second); }
  for (auto e : ctx->ev_pool) cudaEventDestroy(e);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return MITHRA_OK;
}

int mithra_gpu_synchronize(mithra_ctx* ctx) {
  if (!ctx) return MITHRA_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  return check_state(ctx);
}

int mithra_gpu_set_undulators(mithra_ctx* ctx, const mithra_undulator_desc* und, int n) {
  if (!ctx || n < 0 || n > MITHRA_MAX_UNDULATORS || (n && !und)) return MITHRA_ERR_ARG;
  ctx->und_host.assign(n, UndDev{});
  ctx->opt_beams.clear();
  const double c0 = ctx->P.c0;
  for (int u = 0; u < n; u++) {
    UndDev& U = ctx->und_host[u];
    U.type = und[u].type; U.k = und[u].k; U.lu = und[u].lu; U.rb = und[u].rb;
    U.length = und[u].length; U.dist = und[u].dist; U.theta = und[u].theta;
    // Solver::undulatorField, src/solver.cpp:1805-1812 (same expressions, evaluated once here).
    U.b0 = (U.lu != 0.0) ? kEM * c0 * 2 * kPI / U.lu * U.k / kEC : 0.0;
    U.ku = (U.lu != 0.0) ? 2 * kPI / U.lu : 0.0;
    U.ct = cos(U.theta);
    U.st = sin(U.theta);
    U.ul = U.length * U.lu;
    U.has_prev = u > 0;
    U.has_next = u + 1 < n;
    if (u > 0) U.r0_prev = und[u - 1].rb + und[u - 1].length * und[u - 1].lu - U.rb;  // src/beam.cc:35
    if (u + 1 < n) U.r0_next = und[u + 1].rb - U.rb - U.length * U.lu;                  // src/beam.cc:60
    U.ct_f = (float)U.ct; U.st_f = (float)U.st; U.ku_f = (float)U.ku; U.b0_f = (float)U.b0; U.ul_f = (float)U.ul;
    U.r0_prev_f = (float)U.r0_prev; U.r0_next_f = (float)U.r0_next;
    U.kgdz = U.ku * ctx->P.gdz;
    U.kgdz_sub = U.ku * ctx->P.gdz_sub;
    U.beam = -1;
    if (U.type == 1) {
      U.beam = (int)ctx->opt_beams.size();
      ctx->opt_beams.push_back(beam_from_desc(und[u].beam));
    }
  }
  cudaFree(ctx->und_table);
  ctx->und_table = nullptr;
  ctx->P.und_planes = nullptr;
  if (ctx->precision == MITHRA_PRECISION_FP32) {
    if (n) CK(cudaMalloc(&ctx->und_table, (size_t)n * (ctx->g.N2 + 1) * 2 * sizeof(float)));
  } else if (n) {
    // FP64 form: the per-plane phase table, where every static module advances its phase by
    // less than kUndTableMaxKgdz across a cell
    bool small = true;
    for (const UndDev& U : ctx->und_host) small = small && (U.type != 0 || std::fabs(U.kgdz) <= kUndTableMaxKgdz);
    if (small) {
      CK(cudaMalloc(&ctx->und_table, (size_t)n * (ctx->g.N2 + 1) * kUndSub * sizeof(UndPlane64)));
      ctx->P.und_planes = (const UndPlane64*)ctx->und_table;
    }
  }
  invalidate_graphs(ctx);  // the push's launch arguments change
  ctx->P.n_und = n;
  ctx->P.und0_dist = n ? und[0].dist : 0.0;
  return upload_beams(ctx);
}

int mithra_gpu_set_seed(mithra_ctx* ctx, const mithra_seed_desc* sd) {
  if (!ctx) return MITHRA_ERR_ARG;
  ctx->seed_active = sd && fabs(sd->beam.amplitude) > 1.0e-50;  // src/fdtd.cpp:307
  if (!ctx->seed_active) {
    invalidate_graphs(ctx);
    return MITHRA_OK;
  }
  if (sd->beam.type < 0 || sd->beam.type > 7) return fail(ctx, MITHRA_ERR_ARG, "seed beam type %d", sd->beam.type);
  SeedDev& S = ctx->seed;
  S.b = beam_from_desc(sd->beam);
  S.gamma = sd->gamma; S.beta = sd->beta; S.c0 = sd->c0; S.dt = sd->dt;
  // Seed::fields, src/classes.cpp:790-796: wavelength and Rayleigh lengths (same expressions).
  S.l = S.c0 / S.b.sig.f0;
  S.zRp = kPI * S.b.r0 * S.b.r0 / S.l;
  S.zRs = kPI * S.b.r1 * S.b.r1 / S.l;
  S.a1 = ctx->g.a[1]; S.a2 = ctx->g.a[2]; S.a3 = ctx->g.a[3];
  invalidate_graphs(ctx);
  return MITHRA_OK;
}

int mithra_gpu_set_external_fields(mithra_ctx* ctx, const mithra_beam_desc* fields, int n) {
  if (!ctx || n < 0 || n > MITHRA_MAX_EXT_FIELDS || (n && !fields)) return MITHRA_ERR_ARG;
  ctx->ext_beams.clear();
  for (int x = 0; x < n; x++) {
    if (fields[x].type < 0 || fields[x].type > 7) return fail(ctx, MITHRA_ERR_ARG, "external field %d: beam type %d", x, fields[x].type);
    ctx->ext_beams.push_back(beam_from_desc(fields[x]));
  }
  return upload_beams(ctx);
}

int mithra_gpu_set_power(mithra_ctx* ctx, const mithra_power_desc* outs, int n) {
  if (!ctx || n < 0 || n > MITHRA_MAX_POWER_OUTPUTS || (n && !outs)) return MITHRA_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  for (auto& po : ctx->power) {
    void* qs[] = {po.z, po.dzr, po.tw_re, po.tw_im, po.fdt, po.partial, po.rows, po.plane_k, po.plane_slot, po.run};
    for (void* q : qs) cudaFree(q);
  }
  ctx->power.clear();
  ctx->row_cap = 0;
  const GridDev& g = ctx->g;
  for (int o = 0; o < n; o++) {
    const mithra_power_desc& d = outs[o];
    if (d.N <= 0 || d.Nl < 0 || d.Nf <= 0 || !d.z || (d.Nl && (!d.twiddle_re || !d.twiddle_im))) return MITHRA_ERR_ARG;
    // The sample kernel reduces the Nl powers of a block in shared memory (kPowerBlock x Nl doubles).
    const size_t shm = (size_t)kPowerBlock * d.Nl * sizeof(double);
    if (shm > 220 * 1024) return fail(ctx, MITHRA_ERR_ARG, "%d frequencies exceed the power sampler's limit of 220", d.Nl);
    if (shm > 48 * 1024) {
      CK(cudaFuncSetAttribute(k_power_sample<kPowerBlock, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
      CK(cudaFuncSetAttribute(k_power_sample<kPowerBlock, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
    }
    PowerOut po;
    std::vector<int> pk(d.N), ps(d.N);
    std::vector<double> pz(d.N);
    int nz = 0;
    for (int k = 0; k < d.N; k++) {
      // src/radiation.cpp:51-53 and :162-167
      if (d.z[k] < g.zp1 && d.z[k] >= g.zp0) {
        double c;
        pz[k] = modf((d.z[k] - g.zmin) / g.dz, &c);
        pk[k] = (int)c;
        ps[k] = nz++;
      } else {
        pk[k] = -1; ps[k] = 0; pz[k] = 0.0;
      }
    }
    PowerDev& pw = po.dev;
    pw.N = d.N; pw.Nl = d.Nl; pw.Nf = d.Nf; pw.nz = std::max(nz, 1); pw.pc = d.pc;
    pw.gamma = ctx->P.gamma; pw.beta = ctx->P.beta; pw.c0 = ctx->P.c0; pw.dt_shift = ctx->P.dt_shift;
    pw.nodes_i = g.N0 - 4; pw.nodes_j = g.N1 - 4;
    const long long nodes = (long long)pw.nodes_i * pw.nodes_j;
    pw.blocks_per_plane = (int)std::max<long long>(1, (nodes + kPowerBlock - 1) / kPowerBlock);
    CK(dalloc(&po.z, d.N)); CK(dalloc(&po.dzr, d.N)); CK(dalloc(&po.plane_k, d.N)); CK(dalloc(&po.plane_slot, d.N));
    CK(dalloc(&po.tw_re, (size_t)d.Nl * d.Nf)); CK(dalloc(&po.tw_im, (size_t)d.Nl * d.Nf));
    const size_t fdt_n = (size_t)d.Nf * 4 * pw.nz * (size_t)std::max<long long>(nodes, 1);
    CK(dalloc(&po.fdt, fdt_n));
    CK(cudaMemsetAsync(po.fdt, 0, fdt_n * sizeof(double), ctx->stream));
    if (ctx->precision == MITHRA_PRECISION_FP32 && d.Nl) {
      // The mixed form keeps the DFT sums per node and updates them with the slot that changes.
      const size_t run_n = (size_t)d.Nl * 8 * pw.nz * (size_t)std::max<long long>(nodes, 1);
      CK(dalloc(&po.run, run_n));
      CK(cudaMemsetAsync(po.run, 0, run_n * sizeof(double), ctx->stream));
    }
    CK(dalloc(&po.partial, (size_t)d.N * pw.blocks_per_plane * std::max(d.Nl, 1)));
    CK(cudaMemcpyAsync(po.z, d.z, d.N * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(po.dzr, pz.data(), d.N * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(po.plane_k, pk.data(), d.N * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(po.plane_slot, ps.data(), d.N * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    if (d.Nl) {
      CK(cudaMemcpyAsync(po.tw_re, d.twiddle_re, (size_t)d.Nl * d.Nf * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
      CK(cudaMemcpyAsync(po.tw_im, d.twiddle_im, (size_t)d.Nl * d.Nf * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    pw.z = po.z; pw.plane_k = po.plane_k; pw.plane_dzr = po.dzr; pw.plane_slot = po.plane_slot;
    pw.tw_re = po.tw_re; pw.tw_im = po.tw_im; pw.fdt = po.fdt; pw.partial = po.partial; pw.run = po.run;
    pw.rows = nullptr; pw.row_cap = 0;
    ctx->power.push_back(po);
  }
  // Planes whose E/B a power sample reads (cell k and k+1 of each owned plane).
  {
    std::vector<uint8_t> flags((size_t)g.N2, 0);
    for (int o = 0; o < n; o++)
      for (int k = 0; k < outs[o].N; k++)
        if (outs[o].z[k] < g.zp1 && outs[o].z[k] >= g.zp0) {
          double c;
          modf((outs[o].z[k] - g.zmin) / g.dz, &c);
          const int kc = (int)c;
          if (kc >= 0 && kc < g.N2) flags[kc] = 1;
          if (kc + 1 >= 0 && kc + 1 < g.N2) flags[kc + 1] = 1;
        }
    CK(cudaMemcpyAsync(ctx->plane_needed, flags.data(), flags.size(), cudaMemcpyHostToDevice, ctx->stream));
    // the same as a list of interior planes (planes 0 and N2-1 are copies of 1 and N2-2)
    std::vector<int> list;
    for (int k = 0; k < g.N2; k++)
      if (flags[(size_t)k]) {
        const int kk = std::min(std::max(k, 1), g.N2 - 2);
        if (std::find(list.begin(), list.end(), kk) == list.end()) list.push_back(kk);
      }
    cudaFree(ctx->eb_planes);
    ctx->eb_planes = nullptr;
    ctx->n_eb_planes = (int)list.size();
    if (!list.empty()) {
      CK(dalloc(&ctx->eb_planes, list.size()));
      CK(cudaMemcpyAsync(ctx->eb_planes, list.data(), list.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    }
  }
  // Reset the row log.
  CK(cudaMemcpyAsync(ctx->st_host, ctx->st, sizeof(StateDev), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->st_host->n_power_rows = 0;
  CK(cudaMemcpyAsync(ctx->st, ctx->st_host, sizeof(StateDev), cudaMemcpyHostToDevice, ctx->stream));
  ctx->rows_pending = 0;
  invalidate_graphs(ctx);
  return ensure_rows(ctx, 256);
}

int mithra_gpu_upload_fields(mithra_ctx* ctx, const double* anp1, const double* an, const double* anm1) {
  if (!ctx) return MITHRA_ERR_ARG;
  const GridDev& g = ctx->g;
  const size_t n = (size_t)g.N0 * g.N1 * g.N2 * 3;
  double* staging = nullptr;
  { int r = mithra::staging(ctx, n * sizeof(double), (void**)&staging); if (r) return r; }
  const double* src[3] = {anp1, an, anm1};
  for (int l = 0; l < 3; l++) {
    if (!src[l]) continue;
    CK(cudaMemcpyAsync(staging, src[l], n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    if (ctx->precision == MITHRA_PRECISION_FP64)
      k_aos_to_soa<double, double><<<grid_stride_blocks(ctx, n / 3, 256), 256, 0, ctx->stream>>>(g, staging, ctx->A[ctx->idx[l]], 3);
    else
      k_aos_to_soa<float, double><<<grid_stride_blocks(ctx, n / 3, 256), 256, 0, ctx->stream>>>(g, staging, fp32_field(ctx, l), 3);
    CK(cudaGetLastError());
  }
  if (anp1 && ctx->precision == MITHRA_PRECISION_FP64) {  // anp1 now holds the current in node form
    static const int zero = 0;
    CK(cudaMemcpyAsync(&ctx->st->j_edges, &zero, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return MITHRA_OK;
}

int mithra_gpu_download_fields(mithra_ctx* ctx, double* anp1, double* an, double* anm1) {
  if (!ctx) return MITHRA_ERR_ARG;
  const GridDev& g = ctx->g;
  const size_t n = (size_t)g.N0 * g.N1 * g.N2 * 3;
  double* staging = nullptr;
  { int r = mithra::staging(ctx, n * sizeof(double), (void**)&staging); if (r) return r; }
  double* dst[3] = {anp1, an, anm1};
  if (anp1 && ctx->precision == MITHRA_PRECISION_FP64) {
    // A current still in edge form is returned in the reference's node form (J in anp1_).
    int edges = 0;
    CK(cudaMemcpyAsync(&edges, &ctx->st->j_edges, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (edges) {
      k_materialize_j<<<grid_stride_blocks(ctx, (long long)n, 256), 256, 0, ctx->stream>>>(g, ctx->Jedge, ctx->A[ctx->idx[0]]);
      CK(cudaGetLastError());
    }
  }
  for (int l = 0; l < 3; l++) {
    if (!dst[l]) continue;
    if (ctx->precision == MITHRA_PRECISION_FP64)
      k_soa_to_aos<double, double><<<grid_stride_blocks(ctx, n / 3, 256), 256, 0, ctx->stream>>>(g, ctx->A[ctx->idx[l]], staging, 3);
    else
      k_soa_to_aos<float, double><<<grid_stride_blocks(ctx, n / 3, 256), 256, 0, ctx->stream>>>(g, fp32_field(ctx, l), staging, 3);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(dst[l], staging, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  return MITHRA_OK;
}

int mithra_gpu_upload_scalar(mithra_ctx* ctx, const double* fnp1, const double* fn, const double* fnm1) {
  if (!ctx) return MITHRA_ERR_ARG;
  if (!ctx->g.space_charge) return fail(ctx, MITHRA_ERR_STATE, "context has no scalar potential");
  const GridDev& g = ctx->g;
  const size_t n = (size_t)g.N0 * g.N1 * g.N2;
  double* staging = nullptr;
  { int r = mithra::staging(ctx, n * sizeof(double), (void**)&staging); if (r) return r; }
  const double* src[3] = {fnp1, fn, fnm1};
  for (int l = 0; l < 3; l++) {
    if (!src[l]) continue;
    CK(cudaMemcpyAsync(staging, src[l], n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    if (ctx->precision == MITHRA_PRECISION_FP64)
      k_aos_to_soa<double, double><<<grid_stride_blocks(ctx, n, 256), 256, 0, ctx->stream>>>(g, staging, ctx->F[ctx->idx[l]], 1);
    else
      k_aos_to_soa<float, double><<<grid_stride_blocks(ctx, n, 256), 256, 0, ctx->stream>>>(g, staging, fp32_scalar(ctx, l), 1);
    CK(cudaGetLastError());
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return MITHRA_OK;
}

int mithra_gpu_download_scalar(mithra_ctx* ctx, double* fnp1, double* fn, double* fnm1) {
  if (!ctx) return MITHRA_ERR_ARG;
  if (!ctx->g.space_charge) return fail(ctx, MITHRA_ERR_STATE, "context has no scalar potential");
  const GridDev& g = ctx->g;
  const size_t n = (size_t)g.N0 * g.N1 * g.N2;
  double* staging = nullptr;
  { int r = mithra::staging(ctx, n * sizeof(double), (void**)&staging); if (r) return r; }
  double* dst[3] = {fnp1, fn, fnm1};
  for (int l = 0; l < 3; l++) {
    if (!dst[l]) continue;
    if (ctx->precision == MITHRA_PRECISION_FP64)
      k_soa_to_aos<double, double><<<grid_stride_blocks(ctx, n, 256), 256, 0, ctx->stream>>>(g, ctx->F[ctx->idx[l]], staging, 1);
    else
      k_soa_to_aos<float, double><<<grid_stride_blocks(ctx, n, 256), 256, 0, ctx->stream>>>(g, fp32_scalar(ctx, l), staging, 1);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(dst[l], staging, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  return MITHRA_OK;
}

int mithra_gpu_download_eb(mithra_ctx* ctx, float* en, float* bn) {
  if (!ctx) return MITHRA_ERR_ARG;
  const GridDev& g = ctx->g;
  const size_t n = (size_t)g.N0 * g.N1 * g.N2 * 3;
  float* staging = nullptr;
  { int r = mithra::staging(ctx, n * sizeof(float), (void**)&staging); if (r) return r; }
  float* dst[2] = {en, bn};
  const double* srcs64[2] = {ctx->E64, ctx->B64};
  for (int l = 0; l < 2; l++) {
    if (!dst[l]) continue;
    if (ctx->precision == MITHRA_PRECISION_FP64)
      k_soa_to_aos<double, float><<<grid_stride_blocks(ctx, n / 3, 256), 256, 0, ctx->stream>>>(g, srcs64[l], staging, 3);
    else
      k_eb_to_aos<<<grid_stride_blocks(ctx, n / 3, 256), 256, 0, ctx->stream>>>(g, ctx->E, 4 * l, staging);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(dst[l], staging, n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  return MITHRA_OK;
}

namespace {
// Records already in device memory (host upload or device initialisation) -> particle arrays.
int particles_from_device_records(mithra_ctx* ctx, const double* staging, size_t n);
}  // namespace

int mithra_gpu_upload_particles(mithra_ctx* ctx, const double* rec, size_t n) {
  if (!ctx || (n && !rec)) return MITHRA_ERR_ARG;
  if (n > ctx->capacity) return fail(ctx, MITHRA_ERR_CAPACITY, "%zu particles exceed capacity %zu", n, ctx->capacity);
  double* staging = nullptr;
  { int r = mithra::staging(ctx, std::max<size_t>(n, 1) * 11 * sizeof(double), (void**)&staging); if (r) return r; }
  if (n) CK(cudaMemcpyAsync(staging, rec, n * 11 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  return particles_from_device_records(ctx, staging, n);
}

int mithra_gpu_upload_particles_device(mithra_ctx* ctx, const double* dev_rec, size_t n) {
  if (!ctx || (n && !dev_rec)) return MITHRA_ERR_ARG;
  if (n > ctx->capacity) return fail(ctx, MITHRA_ERR_CAPACITY, "%zu particles exceed capacity %zu", n, ctx->capacity);
  return particles_from_device_records(ctx, dev_rec, n);
}

}  // extern "C"

namespace {
int particles_from_device_records(mithra_ctx* ctx, const double* staging, size_t n) {
  if (ctx->precision == MITHRA_PRECISION_FP64) {
    k_records_to_soa<<<grid_stride_blocks(ctx, (long long)n, 256), 256, 0, ctx->stream>>>(staging, (long long)n, ctx->pt);
    CK(cudaGetLastError());
  } else {
    int r = fp32_records_to_soa(ctx, staging, (long long)n);
    if (r) return r;
  }
  CK(cudaMemcpyAsync(ctx->st_host, ctx->st, sizeof(StateDev), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->st_host->n_particles = (long long)n;
  ctx->st_host->n_cross = 0;
  ctx->st_host->overflow = 0;
  ctx->st_host->k_lo = 0;
  ctx->st_host->k_hi = ctx->g.N2 - 1;
  ctx->st_host->k_lo_next = 0x7fffffff;
  ctx->st_host->k_hi_next = -0x7fffffff;
  ctx->st_host->next_id = (long long)n;
  CK(cudaMemcpyAsync(ctx->st, ctx->st_host, sizeof(StateDev), cudaMemcpyHostToDevice, ctx->stream));
  if (ctx->precision == MITHRA_PRECISION_FP32) {
    // Until the first sort, the deposit takes every particle as one outside the tiles (the
    // particles keep their upload order, which z-face copies and downloads follow); the next
    // step sorts.
    const int r = fp32_unsorted(ctx, (long long)n);
    if (r) return r;
    ctx->f32.sort_pending = true;
  }
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->particles_loaded = true;
  return MITHRA_OK;
}
}  // namespace

extern "C" {

int mithra_gpu_particle_count(mithra_ctx* ctx, size_t* n) {
  if (!ctx || !n) return MITHRA_ERR_ARG;
  CK(cudaMemcpyAsync(ctx->st_host, ctx->st, sizeof(StateDev), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  *n = (size_t)ctx->st_host->n_particles;
  return MITHRA_OK;
}

int mithra_gpu_download_particles(mithra_ctx* ctx, double* rec, size_t cap, size_t* n) {
  if (!ctx || !n || (cap && !rec)) return MITHRA_ERR_ARG;
  size_t slots = 0;
  int r = mithra_gpu_particle_count(ctx, &slots);
  if (r) return r;
  double* staging = nullptr;
  long long* dn = nullptr;
  if ((r = mithra::staging(ctx, (std::max<size_t>(slots, 1) * 11 + 1) * sizeof(double), (void**)&staging))) return r;
  dn = (long long*)(staging + std::max<size_t>(slots, 1) * 11);
  if (ctx->precision == MITHRA_PRECISION_FP64) {
    k_soa_to_records<<<1, 1024, 0, ctx->stream>>>(ctx->pt, ctx->st, staging, (long long)slots, dn);
    CK(cudaGetLastError());
  } else {
    r = fp32_soa_to_records(ctx, staging, (long long)slots, dn);
    if (r) return r;
  }
  long long live = 0;
  CK(cudaMemcpyAsync(&live, dn, sizeof live, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  const size_t take = std::min<size_t>((size_t)live, cap);
  if (take) CK(cudaMemcpyAsync(rec, staging, take * 11 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  *n = (size_t)live;
  if ((size_t)live > cap) return fail(ctx, MITHRA_ERR_CAPACITY, "buffer holds %zu of %lld particles", cap, live);
  return MITHRA_OK;
}

int mithra_gpu_set_time(mithra_ctx* ctx, const mithra_time_state* t) {
  if (!ctx || !t) return MITHRA_ERR_ARG;
  CK(cudaMemcpyAsync(ctx->st_host, ctx->st, sizeof(StateDev), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->st_host->time = t->time;
  ctx->st_host->time_bunch = t->time_bunch;
  ctx->st_host->n_time = t->n_time;
  ctx->st_host->n_time_bunch = t->n_time_bunch;
  CK(cudaMemcpyAsync(ctx->st, ctx->st_host, sizeof(StateDev), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return MITHRA_OK;
}

int mithra_gpu_get_time(mithra_ctx* ctx, mithra_time_state* t) {
  if (!ctx || !t) return MITHRA_ERR_ARG;
  CK(cudaMemcpyAsync(ctx->st_host, ctx->st, sizeof(StateDev), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  t->time = ctx->st_host->time;
  t->time_bunch = ctx->st_host->time_bunch;
  t->n_time = ctx->st_host->n_time;
  t->n_time_bunch = ctx->st_host->n_time_bunch;
  return MITHRA_OK;
}

int mithra_gpu_field_update(mithra_ctx* ctx) {
  if (!ctx) return MITHRA_ERR_ARG;
  int r = stage_field_update(ctx);
  if (r) return r;
  return harvest_timers(ctx);
}

int mithra_gpu_field_evaluate(mithra_ctx* ctx) {
  if (!ctx) return MITHRA_ERR_ARG;
  int r = ctx->precision == MITHRA_PRECISION_FP32 ? fp32_eval_eb(ctx, true) : stage_eval_eb(ctx, true);
  if (r) return r;
  return harvest_timers(ctx);
}

int mithra_gpu_save_positions(mithra_ctx* ctx) {
  if (!ctx) return MITHRA_ERR_ARG;
  return stage_save_positions(ctx);
}

int mithra_gpu_bunch_update(mithra_ctx* ctx) {
  if (!ctx) return MITHRA_ERR_ARG;
  if (!ctx->particles_loaded) return fail(ctx, MITHRA_ERR_STATE, "no particles uploaded");
  int r = stage_push(ctx, 0);
  if (r) return r;
  if ((r = harvest_timers(ctx))) return r;
  return check_state(ctx);
}

int mithra_gpu_recycle(mithra_ctx* ctx) {
  if (!ctx) return MITHRA_ERR_ARG;
  return stage_erase(ctx);
}

int mithra_gpu_screen_profile(mithra_ctx* ctx) {
  if (!ctx) return MITHRA_ERR_ARG;
  return stage_screen(ctx);
}

int mithra_gpu_power_sample(mithra_ctx* ctx) {
  if (!ctx) return MITHRA_ERR_ARG;
  int r = ensure_rows(ctx, 1);
  if (r) return r;
  if ((r = stage_power(ctx))) return r;
  if (!ctx->power.empty()) ctx->rows_pending += 1;  // counted once the row's kernels are queued
  return MITHRA_OK;
}

int mithra_gpu_field_shift(mithra_ctx* ctx) {
  if (!ctx) return MITHRA_ERR_ARG;
  rotate(ctx);
  return MITHRA_OK;
}

int mithra_gpu_current_update(mithra_ctx* ctx) {
  if (!ctx) return MITHRA_ERR_ARG;
  int r = stage_current(ctx);
  if (r) return r;
  return stage_erase(ctx);
}

int mithra_gpu_advance_time(mithra_ctx* ctx) {
  if (!ctx) return MITHRA_ERR_ARG;
  return stage_advance_time(ctx);
}

int mithra_gpu_run(mithra_ctx* ctx, int64_t nsteps) {
  if (!ctx || nsteps < 0) return MITHRA_ERR_ARG;
  if (!ctx->particles_loaded) return fail(ctx, MITHRA_ERR_STATE, "no particles uploaded");
  int r = ensure_rows(ctx, nsteps);
  if (r) return r;
  if (!ctx->power.empty()) ctx->rows_pending += nsteps;
  if (ctx->timing) {
    for (int64_t s = 0; s < nsteps; s++)
      if ((r = enqueue_step(ctx))) return r;
    if ((r = harvest_timers(ctx))) return r;
    return check_state(ctx);
  }
  for (int64_t s = 0; s < nsteps; s++) {
    if (ctx->precision == MITHRA_PRECISION_FP32 && ctx->f32.sort_pending) {
      // The step's deposit runs after its rotation, which brings idx[2] to idx[0].
      if (ctx->idx[2] != 0) {  // not a sorting step: the sort an upload asks for, outside the graphs
        if ((r = enqueue_step(ctx))) return r;
        continue;
      }
    }
    const int key = step_key(ctx);
    if (!ctx->graph[key]) {
      cudaGraph_t graph;
      if ((r = capture_step(ctx, &graph))) return r;
      CK(cudaGraphInstantiate(&ctx->graph[key], graph, 0));
      CK(cudaGraphDestroy(graph));
    }
    CK(cudaGraphLaunch(ctx->graph[key], ctx->stream));
    after_step(ctx);
  }
  return check_state(ctx);
}

int mithra_gpu_run_timed(mithra_ctx* ctx, int64_t nsteps, double* device_ms) {
  if (!ctx || !device_ms) return MITHRA_ERR_ARG;
  int r = ensure_rows(ctx, nsteps);
  if (r) return r;
  if (!ctx->particles_loaded) return fail(ctx, MITHRA_ERR_STATE, "no particles uploaded");
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  CK(cudaEventRecord(a, ctx->stream));
  r = mithra_gpu_run(ctx, nsteps);
  if (r) { cudaEventDestroy(a); cudaEventDestroy(b); return r; }
  CK(cudaEventRecord(b, ctx->stream));
  CK(cudaEventSynchronize(b));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *device_ms = ms;
  return MITHRA_OK;
}

int mithra_gpu_launches_per_step(mithra_ctx* ctx, int* n) {
  if (!ctx || !n) return MITHRA_ERR_ARG;
  if (!ctx->launches_per_step) {
    // Count by recording one step into a throw-away capture.
    cudaGraph_t graph;
    const int saved[3] = {ctx->idx[0], ctx->idx[1], ctx->idx[2]};
    const Fp32State saved_f32 = ctx->f32;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    ctx->launch_counter = 0;
    int r = enqueue_step(ctx);
    cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
    ctx->idx[0] = saved[0]; ctx->idx[1] = saved[1]; ctx->idx[2] = saved[2];
    ctx->f32 = saved_f32;
    if (r) return r;
    if (ce != cudaSuccess) return fail(ctx, MITHRA_ERR_CUDA, "capture: %s", cudaGetErrorString(ce));
    cudaGraphDestroy(graph);
    ctx->launches_per_step = ctx->launch_counter;
  }
  *n = ctx->launches_per_step;
  return MITHRA_OK;
}

int mithra_host_alloc(size_t bytes, void** p) {
  if (!p) return MITHRA_ERR_ARG;
  return cudaMallocHost(p, std::max<size_t>(bytes, 1)) == cudaSuccess ? MITHRA_OK : MITHRA_ERR_CUDA;
}

int mithra_host_free(void* p) {
  if (!p) return MITHRA_ERR_ARG;
  return cudaFreeHost(p) == cudaSuccess ? MITHRA_OK : MITHRA_ERR_CUDA;
}

int mithra_gpu_run_prelude(mithra_ctx* ctx) {
  if (!ctx) return MITHRA_ERR_ARG;
  if (!ctx->particles_loaded) return fail(ctx, MITHRA_ERR_STATE, "no particles uploaded");
  mithra_time_state t;
  int r = mithra_gpu_get_time(ctx, &t);
  if (r) return r;
  if (!(t.time < 0.0)) return MITHRA_OK;
  // No field update happens before time zero, so the lazily evaluated E/B of the reference are
  // those of the initial potentials throughout the prelude.
  r = ctx->precision == MITHRA_PRECISION_FP32 ? fp32_eval_eb(ctx, true) : stage_eval_eb(ctx, true);
  if (r) return r;
  const int ns = n_substeps(ctx);
  while (t.time < 0.0) {
    for (int s = 0; s < ns; s++)
      if ((r = stage_push(ctx, s == 0))) return r;
    if (ns == 0 && (r = stage_save_positions(ctx))) return r;
    if ((r = stage_screen(ctx))) return r;  // before the recycling here (src/solver.cpp:1248)
    if ((r = stage_erase(ctx))) return r;
    if ((r = stage_advance_time(ctx))) return r;
    if ((r = harvest_timers(ctx))) return r;
    if ((r = mithra_gpu_get_time(ctx, &t))) return r;
  }
  return check_state(ctx);
}

int mithra_gpu_power_rows(mithra_ctx* ctx, double* out, size_t cap_values, size_t* n_values) {
  if (!ctx || !n_values) return MITHRA_ERR_ARG;
  CK(cudaMemcpyAsync(ctx->st_host, ctx->st, sizeof(StateDev), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  const long long rows = std::min(ctx->st_host->n_power_rows, ctx->row_cap);
  size_t per_row = 0;
  for (auto& po : ctx->power) per_row += (size_t)po.dev.N * (1 + po.dev.Nl);
  const size_t need = per_row * (size_t)rows;
  *n_values = need;
  if (!out) return MITHRA_OK;
  if (cap_values < need) return fail(ctx, MITHRA_ERR_ARG, "power row buffer too small (%zu < %zu)", cap_values, need);
  std::vector<double> tmp;
  size_t w = 0;
  for (long long r = 0; r < rows; r++)
    for (auto& po : ctx->power) {
      const size_t rowlen = (size_t)po.dev.N * (1 + po.dev.Nl);
      CK(cudaMemcpyAsync(out + w, po.rows + r * rowlen, rowlen * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
      w += rowlen;
    }
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->st_host->n_power_rows = 0;
  CK(cudaMemcpyAsync(&ctx->st->n_power_rows, &ctx->st_host->n_power_rows, sizeof(long long), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->rows_pending = 0;
  return MITHRA_OK;
}

}  // extern "C"

namespace {

DiagParticles diag_particles(const mithra_ctx* ctx) {
  DiagParticles P{};
  const GridDev& g = ctx->g;
  P.xmin = g.xmin; P.ymin = g.ymin; P.zmin = g.zmin; P.dx = g.dx; P.dy = g.dy; P.dz = g.dz;
  if (ctx->precision == MITHRA_PRECISION_FP64) {
    const ParticlesDev<double>& t = ctx->pt;
    P.x = t.x; P.y = t.y; P.z = t.z; P.gx = t.gx; P.gy = t.gy; P.gz = t.gz; P.q = t.q; P.status = t.status;
    P.mx = t.mx; P.my = t.my; P.mz = t.mz;
  } else {
    const ParticlesF32& t = ctx->f32.pt;
    P.cell = t.cell; P.fx = t.fx; P.fy = t.fy; P.fz = t.fz; P.gxf = t.gx; P.gyf = t.gy; P.gzf = t.gz; P.qf = t.q;
    P.status = t.status;
    P.mcell = t.mcell; P.mfx = t.mfx; P.mfy = t.mfy; P.mfz = t.mfz; P.id = t.id;
  }
  return P;
}

// Runs one diagnostic reduction (`launch` issues the block kernel) and copies nv totals to out.
template <typename F>
int diag_reduce(mithra_ctx* ctx, int nv, F launch, double* out, int* nblocks_out) {
  if (!ctx->diag_partial) {
    CK(cudaMalloc(&ctx->diag_partial, (size_t)kDiagMaxBlocks * 16 * sizeof(double2)));
    CK(cudaMalloc(&ctx->diag_out, 16 * sizeof(double)));
  }
  const int nb = std::min(kDiagMaxBlocks, grid_stride_blocks(ctx, (long long)ctx->capacity, kDiagBlock));
  launch(nb);
  k_diag_finish<<<1, 32, 0, ctx->stream>>>((const double2*)ctx->diag_partial, nb, nv, ctx->diag_out);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, ctx->diag_out, nv * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (nblocks_out) *nblocks_out = nb;
  return MITHRA_OK;
}

}  // namespace

extern "C" {

int mithra_gpu_bunch_sample(mithra_ctx* ctx, double* row) {
  if (!ctx || !row) return MITHRA_ERR_ARG;
  double s[kDiagValues];
  const DiagParticles P = diag_particles(ctx);
  int r = diag_reduce(ctx, kDiagValues, [&](int nb) {
    k_bunch_moments<<<nb, kDiagBlock, 0, ctx->stream>>>(ctx->g, P, ctx->st, (double2*)ctx->diag_partial);
  }, s, nullptr);
  if (r) return r;
  mithra_time_state t;
  if ((r = mithra_gpu_get_time(ctx, &t))) return r;
  // Solver::bunchSample, src/solver.cpp:1613-1634: means, then sqrt(<v^2> - <v>^2).
  const double qT = s[0];
  row[0] = t.time_bunch;
  for (int c = 0; c < 3; c++) {
    const double rT = s[1 + c] / qT, r2T = s[4 + c] / qT, gbT = s[7 + c] / qT, gb2T = s[10 + c] / qT;
    row[1 + c] = rT;
    row[4 + c] = gbT;
    row[7 + c] = sqrt(r2T - rT * rT);
    row[10 + c] = sqrt(gb2T - gbT * gbT);
  }
  return MITHRA_OK;
}

int mithra_gpu_field_sample(mithra_ctx* ctx, const double* points, size_t n, double* out) {
  if (!ctx || (n && (!points || !out))) return MITHRA_ERR_ARG;
  if (n == 0) return MITHRA_OK;
  if (n > (1u << 24)) return fail(ctx, MITHRA_ERR_ARG, "too many sampling points (%zu)", n);
  // E/B at every interior node from the current A^{n+1}, A^n: the nodes the reference's lazy
  // evaluation reaches from a sampling point (src/fdtd.cpp:878-885).
  int r = ctx->precision == MITHRA_PRECISION_FP32 ? fp32_eval_eb(ctx, true) : stage_eval_eb(ctx, true);
  if (r) return r;
  double* buf = nullptr;  // points, then results
  if ((r = mithra::staging(ctx, n * 12 * sizeof(double), (void**)&buf))) return r;
  CK(cudaMemcpyAsync(buf, points, n * 3 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  const int blocks = (int)((n + 127) / 128);
  if (ctx->precision == MITHRA_PRECISION_FP64)
    k_field_sample<double, double><<<blocks, 128, 0, ctx->stream>>>(ctx->g, ctx->E64, ctx->B64, ctx->g.cstride, 1,
                                                                    ctx->A[ctx->idx[1]], buf, (int)n, buf + 3 * n);
  else
    k_field_sample<float, float><<<blocks, 128, 0, ctx->stream>>>(ctx->g, ctx->E, ctx->E + 4, 1, kEBNode,
                                                                  fp32_field(ctx, 1), buf, (int)n, buf + 3 * n);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, buf + 3 * n, n * 9 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return MITHRA_OK;
}

int mithra_gpu_bunching_factor(mithra_ctx* ctx, double k, double* b) {
  if (!ctx || !b) return MITHRA_ERR_ARG;
  double s[3];
  const DiagParticles P = diag_particles(ctx);
  int r = diag_reduce(ctx, 3, [&](int nb) {
    k_bunching<<<nb, kDiagBlock, 0, ctx->stream>>>(ctx->g, P, ctx->st, k, (double2*)ctx->diag_partial);
  }, s, nullptr);
  if (r) return r;
  *b = (s[0] != 0.0) ? sqrt(s[1] * s[1] + s[2] * s[2]) / s[0] : 0.0;
  return MITHRA_OK;
}

int mithra_gpu_set_screens(mithra_ctx* ctx, const double* lz, int n, long long capacity) {
  if (!ctx || n < 0 || (n > 0 && !lz) || capacity < 0) return MITHRA_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  cudaFree(ctx->screen_lz); cudaFree(ctx->screen_rec); cudaFree(ctx->screen_key); cudaFree(ctx->screen_count);
  ctx->screen_lz = nullptr; ctx->screen_rec = nullptr; ctx->screen_key = nullptr; ctx->screen_count = nullptr;
  ctx->n_screens = 0;
  ctx->screen_cap = 0;
  invalidate_graphs(ctx);  // the step graphs gain or lose the screen kernel
  if (n == 0) return MITHRA_OK;
  const long long cap = capacity > 0 ? capacity : std::max(1024LL, (long long)ctx->capacity);
  CK(cudaMalloc(&ctx->screen_lz, (size_t)n * sizeof(double)));
  CK(cudaMalloc(&ctx->screen_rec, (size_t)n * cap * 6 * sizeof(double)));
  CK(cudaMalloc(&ctx->screen_key, (size_t)n * cap * sizeof(long long)));
  CK(cudaMalloc(&ctx->screen_count, (size_t)n * sizeof(unsigned long long)));
  CK(cudaMemcpyAsync(ctx->screen_lz, lz, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemsetAsync(ctx->screen_count, 0, (size_t)n * sizeof(unsigned long long), ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->n_screens = n;
  ctx->screen_cap = cap;
  return MITHRA_OK;
}

int mithra_gpu_screen_clear(mithra_ctx* ctx) {
  if (!ctx) return MITHRA_ERR_ARG;
  if (ctx->n_screens == 0) return MITHRA_OK;
  CK(cudaMemsetAsync(ctx->screen_count, 0, (size_t)ctx->n_screens * sizeof(unsigned long long), ctx->stream));
  return MITHRA_OK;
}

int mithra_gpu_screen_records(mithra_ctx* ctx, int screen, double* out, long long cap_rows, long long* n_rows) {
  if (!ctx || !n_rows || screen < 0 || screen >= ctx->n_screens || cap_rows < 0) return MITHRA_ERR_ARG;
  unsigned long long count = 0;
  CK(cudaMemcpyAsync(&count, ctx->screen_count + screen, sizeof(count), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if ((long long)count > ctx->screen_cap)
    return fail(ctx, MITHRA_ERR_CAPACITY, "screen %d: %llu records for a capacity of %lld", screen, count,
                ctx->screen_cap);
  *n_rows = (long long)count;
  if (!out || count == 0) return MITHRA_OK;
  if (cap_rows < (long long)count) return fail(ctx, MITHRA_ERR_ARG, "screen rows buffer too small (%lld < %llu)", cap_rows, count);
  std::vector<double> rec((size_t)count * 6);
  std::vector<long long> key((size_t)count);
  const size_t base = (size_t)screen * (size_t)ctx->screen_cap;
  CK(cudaMemcpyAsync(rec.data(), ctx->screen_rec + base * 6, rec.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(key.data(), ctx->screen_key + base, key.size() * sizeof(long long), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  // the reference's file order: steps in order, particles in list order within a step
  std::vector<long long> order((size_t)count);
  for (size_t i = 0; i < order.size(); i++) order[i] = (long long)i;
  std::sort(order.begin(), order.end(), [&](long long a, long long b) { return key[a] < key[b]; });
  for (size_t i = 0; i < order.size(); i++) {
    const double* src = rec.data() + (size_t)order[i] * 6;
    double* dst = out + i * 7;
    for (int c = 0; c < 6; c++) dst[c] = src[c];
    dst[6] = (double)(key[order[i]] >> 40);  // nTime_ of the step
  }
  return MITHRA_OK;
}

int mithra_gpu_enable_timing(mithra_ctx* ctx, int on) {
  if (!ctx) return MITHRA_ERR_ARG;
  int r = harvest_timers(ctx);
  if (r) return r;
  ctx->timing = on != 0;
  for (auto& t : ctx->timers) { t.ms = 0.0; t.launches = 0; }
  return MITHRA_OK;
}

int mithra_gpu_kernel_times(mithra_ctx* ctx, char* names, size_t name_len, double* ms, int cap, int* n) {
  if (!ctx || !n) return MITHRA_ERR_ARG;
  int r = harvest_timers(ctx);
  if (r) return r;
  *n = (int)ctx->timers.size();
  for (int i = 0; i < std::min(cap, *n); i++) {
    if (names) snprintf(names + (size_t)i * name_len, name_len, "%s", ctx->timers[i].name.c_str());
    if (ms) {
      ms[2 * i] = ctx->timers[i].ms;
      ms[2 * i + 1] = (double)ctx->timers[i].launches;
    }
  }
  return MITHRA_OK;
}

}  // extern "C"


// ---- power sample without allocation ----------------------------------------------------
//
// mithra_gpu_power_sample may allocate: it grows the device row log when it is full, and its
// per-block partial sums live in a buffer of the context.  Some callers cannot allow an
// allocation at that point: a host loop that has already given the whole of device memory to
// fields and particles (cudaMalloc would fail), or one that must not stall on the device-wide
// synchronisation that cudaFree implies while other streams are running.  The variant below
// keeps the partial sums in a fixed array in device memory that is part of the loaded module,
// and refuses, with an error, to grow the row log.

namespace {

// Partial sums of one power output: (planes x blocks per plane x frequencies) doubles.  The
// sample kernel writes every slot that the finish kernel then reads, within the same call, so
// nothing in this array needs to start at zero.  There is ONE array per device, shared by all
// contexts on that device: two calls that overlap in time on one device (different contexts,
// streams or host threads) race on it, and the caller must order them.
constexpr long long kStaticPartialMax = 1LL << 17;  // 131072 doubles = 1 MiB
static __device__ __align__(256) double g_static_partial[kStaticPartialMax];

// Device address of g_static_partial on the context's device, looked up with that device current.
// The host-side name g_static_partial is only a stand-in for the symbol, not a device address.
// The address is looked up on every call rather than cached, so it stays right after the device
// is reset or the module reloaded.  The first lookup on a device does set-up work in the runtime
// (it may load the module), so callers should make their first call before any stream capture.
int static_partial_address(mithra_ctx* ctx, double** out) {
  int prev = -1;
  CK(cudaGetDevice(&prev));
  if (prev != ctx->device) CK(cudaSetDevice(ctx->device));
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_static_partial);
  if (prev != ctx->device) CK(cudaSetDevice(prev));
  if (e != cudaSuccess || !p)
    return fail(ctx, MITHRA_ERR_CUDA, "cudaGetSymbolAddress(g_static_partial): %s", cudaGetErrorString(e));
  *out = static_cast<double*>(p);
  return MITHRA_OK;
}

}  // namespace

extern "C" int mithra_gpu_power_sample_noalloc(mithra_ctx* ctx) {
  if (!ctx) return MITHRA_ERR_ARG;
  if (ctx->power.empty()) return MITHRA_OK;
  for (const auto& po : ctx->power) {
    const long long need = (long long)po.dev.N * po.dev.blocks_per_plane * std::max(po.dev.Nl, 1);
    if (need > kStaticPartialMax)
      return fail(ctx, MITHRA_ERR_CAPACITY,
                  "power output needs %lld partial sums (%d planes x %d blocks x %d frequencies); the fixed "
                  "array holds %lld: use mithra_gpu_power_sample",
                  need, po.dev.N, po.dev.blocks_per_plane, po.dev.Nl, kStaticPartialMax);
  }
  if (ctx->rows_pending + 1 > ctx->row_cap)
    return fail(ctx, MITHRA_ERR_CAPACITY,
                "power row log full (%lld rows): drain it with mithra_gpu_power_rows before sampling again",
                ctx->row_cap);
  double* partial = nullptr;
  int r = static_partial_address(ctx, &partial);
  if (r) return r;
  // The same launches as mithra_gpu_power_sample, partial sums redirected to the fixed array.
  if ((r = stage_power(ctx, partial))) return r;
  ctx->rows_pending += 1;  // counted once the row's kernels are queued
  return MITHRA_OK;
}
