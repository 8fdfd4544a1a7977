// Mixed-precision form: buffers and stages (see fp32_kernels.cuh for the arithmetic split).
#include <algorithm>

#include "ctx.h"
#include "field_kernels.cuh"
#include "fp32_kernels.cuh"
#include "sort_kernels.cuh"
#include "eb_tma.cuh"
#include "tma_stencil.cuh"

namespace mithra {

namespace {

PushF32 push_constants(const mithra_ctx* ctx) {
  const GridDev& g = ctx->g;
  const PushDev& P = ctx->P;
  PushF32 C;
  C.rdx = (float)(1.0 / g.dx); C.rdy = (float)(1.0 / g.dy); C.rdz = (float)(1.0 / g.dz);
  C.dx = (float)g.dx; C.dy = (float)g.dy; C.dz = (float)g.dz;
  C.xmin = (float)g.xmin; C.ymin = (float)g.ymin;
  C.r1 = (float)P.r1; C.r2 = (float)P.r2; C.dtb = (float)P.dtb;
  C.N0 = g.N0; C.N1 = g.N1; C.N2 = g.N2;
  C.zmin = g.zmin; C.dzd = g.dz; C.gamma = P.gamma; C.bc = P.beta * P.c0;
  C.dt_shift = P.dt_shift;
  C.n_und = P.n_und;
  C.und0_dist = P.und0_dist;
  C.gamma_f = (float)P.gamma; C.bc_f = (float)(P.beta * P.c0); C.gdz = (float)(P.gamma * g.dz);
  C.zmin_f = (float)g.zmin; C.dz_f = (float)g.dz; C.und0_dist_f = (float)P.und0_dist;
  C.rb0_f = ctx->und_host.empty() ? 0.0f : (float)ctx->und_host[0].rb;
  C.P64 = P;
  C.xmin_d = g.xmin; C.ymin_d = g.ymin; C.dxd = g.dx; C.dyd = g.dy;
  return C;
}

CellMap cell_map(const mithra_ctx* ctx) {
  const GridDev& g = ctx->g;
  return CellMap{g.xmin, g.ymin, g.zmin, g.dx, g.dy, g.dz};
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link-time libcuda).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int make_tma_maps(mithra_ctx* ctx) {
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  CK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
  if (!fn || q != cudaDriverEntryPointSuccess) return fail(ctx, MITHRA_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  EncodeTiledFn encode = (EncodeTiledFn)fn;
  const GridDev& g = ctx->g;
  Fp32State& f = ctx->f32;
  const cuuint64_t dims[4] = {(cuuint64_t)g.P1, (cuuint64_t)g.N0, (cuuint64_t)g.N2, 3};
  const cuuint64_t strides[3] = {(cuuint64_t)g.P1 * 4, (cuuint64_t)g.plane * 4, (cuuint64_t)g.cstride * 4};
  const cuuint32_t box_an[4] = {TMA_BW, TMA_BH, 1, 1}, box_c[4] = {TMA_BW, TMA_TI, 1, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  for (int b = 0; b < 3; b++) {
    CUresult r1 = encode((CUtensorMap*)f.map_an[b], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, f.A[b], dims, strides, box_an,
                         estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    CUresult r2 = encode((CUtensorMap*)f.map_c[b], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, f.A[b], dims, strides, box_c,
                         estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r1 != CUDA_SUCCESS || r2 != CUDA_SUCCESS)
      return fail(ctx, MITHRA_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d, %d)", (int)r1, (int)r2);
  }
  CK(dalloc(&f.tma_error, 1));
  CK(cudaMemsetAsync(f.tma_error, 0, sizeof(int), ctx->stream));
  CK(cudaFuncSetAttribute(k_potential_interior_tma<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTmaStencilSmem));
  CK(cudaFuncSetAttribute(k_potential_interior_tma<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTmaStencilSmem));
  CK(cudaFuncSetAttribute(k_eval_eb_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kEbTmaSmem));
  f.tma_ready = true;
  return MITHRA_OK;
}

int run_interior_tma(mithra_ctx* ctx, const PotentialArgs<float>& p) {
  const GridDev& g = ctx->g;
  Fp32State& f = ctx->f32;
  TmaStencilArgs a;
  a.np1 = p.np1; a.N0 = g.N0; a.N1 = g.N1; a.N2 = g.N2; a.P1 = g.P1; a.plane = g.plane; a.cstride = g.cstride;
  a.a0 = p.k.a0; a.a1 = p.k.a1; a.a2 = p.k.a2; a.a3 = p.k.a3; a.asrc = p.asrc; a.al = p.k.al; a.be = p.k.be;
  a.error = f.tma_error;
  a.ks = ctx->tune.slab_planes;
  a.spin_limit = ctx->wait_limit < 0 ? TMA_SPIN_LIMIT : (unsigned)ctx->wait_limit;
  a.yfaces = p.yfaces_done;
  for (int q = 0; q < 5; q++) a.cB[q] = p.k.cB[q];
  const int nslab = (g.N2 - 2 + a.ks - 1) / a.ks;
  dim3 grd((g.N1 - 2 + TMA_TJ - 1) / TMA_TJ, (g.N0 - 2 + TMA_TI - 1) / TMA_TI, 3 * nslab);
  const CUtensorMap* an = (const CUtensorMap*)f.map_an[ctx->idx[1]];
  const CUtensorMap* am = (const CUtensorMap*)f.map_c[ctx->idx[2]];
  const CUtensorMap* jm = (const CUtensorMap*)f.map_c[ctx->idx[0]];
  if (g.solver == 1)
    return timed(ctx, "potential_interior_nsfd", [&] {
      k_potential_interior_tma<true><<<grd, TMA_TJ * TMA_TI, kTmaStencilSmem, ctx->stream>>>(*an, *am, *jm, a);
    });
  return timed(ctx, "potential_interior_fd", [&] {
    k_potential_interior_tma<false><<<grd, TMA_TJ * TMA_TI, kTmaStencilSmem, ctx->stream>>>(*an, *am, *jm, a);
  });
}

int run_potential_f32(mithra_ctx* ctx, PotentialArgs<float> p, bool vector) {
  const GridDev& g = ctx->g;
  dim3 blk(32, 8), grd((g.N1 - 2 + 31) / 32, (g.N0 - 2 + 7) / 8, g.N2 - 2);
  const long long nfaces = 2LL * ((long long)(g.N1 - 2) * (g.N2 - 2) + (long long)(g.N0 - 2) * (g.N2 - 2) +
                                  (long long)(g.N0 - 2) * (g.N1 - 2));
  const long long nedges = 4LL * ((g.N2 - 2) + (g.N0 - 2) + (g.N1 - 2));
  int r;
  // the bulk-tensor stencil also updates the y faces when no seed injection comes in between
  if (vector && ctx->f32.tma_ready) p.yfaces_done = ctx->seed_active ? 0 : 1;
  if (vector && ctx->f32.tma_ready)
    r = run_interior_tma(ctx, p);
  else if (g.solver == 1)
    r = timed(ctx, vector ? "potential_interior_nsfd" : "scalar_interior_nsfd",
              [&] { k_potential_interior<float, true><<<grd, blk, 0, ctx->stream>>>(g, p); });
  else
    r = timed(ctx, vector ? "potential_interior_fd" : "scalar_interior_fd",
              [&] { k_potential_interior<float, false><<<grd, blk, 0, ctx->stream>>>(g, p); });
  if (r) return r;
  if (vector && ctx->seed_active && (r = stage_seed(ctx, p.np1))) return r;
  r = timed(ctx, vector ? "potential_faces" : "scalar_faces", [&] {
    k_potential_faces<float><<<grid_stride_blocks(ctx, nfaces, 256), 256, 0, ctx->stream>>>(g, p);
  });
  if (r) return r;
  if (g.order == 2) {
    r = timed(ctx, vector ? "potential_edges" : "scalar_edges", [&] {
      k_potential_edges<float><<<grid_stride_blocks(ctx, nedges, 256), 256, 0, ctx->stream>>>(g, p);
    });
    if (r) return r;
    r = timed(ctx, vector ? "potential_corners" : "scalar_corners",
              [&] { k_potential_corners<float><<<1, 32, 0, ctx->stream>>>(g, p); });
    if (r) return r;
  }
  return MITHRA_OK;
}

}  // namespace

namespace {
int alloc_particles(mithra_ctx* ctx, ParticlesF32& pt) {
  const size_t c = ctx->capacity;
  CK(dalloc(&pt.cell, c)); CK(dalloc(&pt.mcell, c));
  CK(dalloc(&pt.fx, c)); CK(dalloc(&pt.fy, c)); CK(dalloc(&pt.fz, c));
  CK(dalloc(&pt.gx, c)); CK(dalloc(&pt.gy, c)); CK(dalloc(&pt.gz, c));
  CK(dalloc(&pt.mfx, c)); CK(dalloc(&pt.mfy, c)); CK(dalloc(&pt.mfz, c));
  CK(dalloc(&pt.q, c)); CK(dalloc(&pt.e, c)); CK(dalloc(&pt.status, c)); CK(dalloc(&pt.cross, c));
  CK(dalloc(&pt.id, c));
  return MITHRA_OK;
}

void free_particles(ParticlesF32& pt) {
  void* ps[] = {pt.cell, pt.mcell, pt.fx, pt.fy, pt.fz, pt.gx, pt.gy, pt.gz, pt.mfx, pt.mfy, pt.mfz,
                pt.q, pt.e, pt.status, pt.cross, pt.id};
  for (void* p : ps) cudaFree(p);
  pt = ParticlesF32{};
}

TileGrid tile_grid(const mithra_ctx* ctx) {
  const TileGridHost& h = ctx->f32.tiles;
  return TileGrid{h.ntx, h.nty, h.ntz, h.n_tiles, h.bin_outside, h.bin_erased, h.n_bins};
}
}  // namespace

int fp32_alloc(mithra_ctx* ctx) {
  const GridDev& g = ctx->g;
  Fp32State& f = ctx->f32;
  const size_t nf = (size_t)3 * g.cstride;
  for (int b = 0; b < 3; b++) {
    CK(dalloc(&f.A[b], nf));
    CK(cudaMemsetAsync(f.A[b], 0, nf * sizeof(float), ctx->stream));
    if (g.space_charge) {
      CK(dalloc(&f.F[b], (size_t)g.cstride));
      CK(cudaMemsetAsync(f.F[b], 0, (size_t)g.cstride * sizeof(float), ctx->stream));
    }
  }
  int r;
  if ((r = alloc_particles(ctx, f.pt))) return r;
  if ((r = alloc_particles(ctx, f.alt))) return r;
  TileGridHost& t = f.tiles;
  t.ntx = (g.N0 + TX - 1) / TX;
  t.nty = (g.N1 + TY - 1) / TY;
  t.ntz = (g.N2 + TZ - 1) / TZ;
  t.n_tiles = t.ntx * t.nty * t.ntz;
  t.bin_outside = t.n_tiles;
  t.bin_erased = t.n_tiles + 1;
  t.n_bins = t.n_tiles + 2;
  CK(dalloc(&f.counts, (size_t)t.n_bins));
  CK(cudaMemsetAsync(f.counts, 0, (size_t)t.n_bins * sizeof(int), ctx->stream));
  CK(dalloc(&f.offsets, (size_t)t.n_bins + 1));
  if ((t.n_bins + 1023) / 1024 > 1024) return fail(ctx, MITHRA_ERR_ARG, "mesh too large for the tile sort (%d tiles)", t.n_tiles);
  CK(dalloc(&f.block_sums, 1025));
  CK(dalloc(&f.work, (size_t)t.n_tiles));
  CK(dalloc(&f.work_count, 3));
  CK(cudaMemsetAsync(f.work_count, 0, 3 * sizeof(int), ctx->stream));
  CK(dalloc(&f.key, ctx->capacity));
  CK(dalloc(&f.rank, ctx->capacity));
  CK(cudaFuncSetAttribute(k_deposit_tiled, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          (int)(3 * TILE_NODES * sizeof(float))));
  return make_tma_maps(ctx);
}

void fp32_after_step(mithra_ctx* ctx) {
  std::swap(ctx->f32.pt, ctx->f32.alt);
  ctx->f32.parity ^= 1;
}

void fp32_free(mithra_ctx* ctx) {
  Fp32State& f = ctx->f32;
  for (int b = 0; b < 3; b++) { cudaFree(f.A[b]); cudaFree(f.F[b]); f.A[b] = f.F[b] = nullptr; }
  free_particles(f.pt);
  free_particles(f.alt);
  cudaFree(f.counts); cudaFree(f.offsets); cudaFree(f.key); cudaFree(f.rank); cudaFree(f.tma_error);
  cudaFree(f.block_sums);
  cudaFree(f.work); cudaFree(f.work_count);
  f.work = f.work_count = nullptr;
  f.counts = f.offsets = f.key = f.rank = f.tma_error = f.block_sums = nullptr;
  f.tma_ready = false;
}

float* fp32_field(mithra_ctx* ctx, int level) { return ctx->f32.A[ctx->idx[level]]; }
float* fp32_scalar(mithra_ctx* ctx, int level) { return ctx->f32.F[ctx->idx[level]]; }

int fp32_records_to_soa(mithra_ctx* ctx, const double* staging, long long n) {
  k_records_to_f32<<<grid_stride_blocks(ctx, n, 256), 256, 0, ctx->stream>>>(staging, n, ctx->f32.pt, cell_map(ctx));
  CK(cudaGetLastError());
  return MITHRA_OK;
}

// Live particles in creation order (the reference's list order; z-face copies after the
// particles present at upload, in the order they were appended).
int fp32_soa_to_records(mithra_ctx* ctx, double* staging, long long slots, long long* n_out) {
  CK(cudaMemcpyAsync(ctx->st_host, ctx->st, sizeof(StateDev), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  const long long id_cap = std::max<long long>(ctx->st_host->next_id, 1);
  double* rows = nullptr;
  uint8_t* valid = nullptr;
  CK(dalloc(&rows, (size_t)id_cap * 11));
  CK(dalloc(&valid, (size_t)id_cap));
  CK(cudaMemsetAsync(valid, 0, (size_t)id_cap, ctx->stream));
  k_f32_to_rows_by_id<<<grid_stride_blocks(ctx, slots, 256), 256, 0, ctx->stream>>>(ctx->f32.pt, ctx->st, rows, valid,
                                                                                    id_cap, cell_map(ctx));
  k_compact_rows<<<1, 1024, 0, ctx->stream>>>(rows, valid, id_cap, staging, slots, n_out);
  cudaError_t e = cudaGetLastError();
  CK(cudaStreamSynchronize(ctx->stream));
  cudaFree(rows);
  cudaFree(valid);
  CK(e);
  return MITHRA_OK;
}

int fp32_eval_eb(mithra_ctx* ctx, bool full) {
  const GridDev& g = ctx->g;
  const EBConstF32 c{(float)(1.0 / g.dt), (float)(0.5 / (2.0 * g.dx)), (float)(0.5 / (2.0 * g.dy)),
                     (float)(0.5 / (2.0 * g.dz))};
  Fp32State& f = ctx->f32;
  if (!g.space_charge && f.tma_ready) {
    // Bulk-tensor z-slabs over the planes the particles occupy (every plane when `full`), then
    // the power-sampling planes outside them.
    EbTmaArgs a;
    a.EB = ctx->E;
    a.N0 = g.N0; a.N1 = g.N1; a.N2 = g.N2; a.P1 = g.P1; a.plane = g.plane;
    a.rdt = c.rdt; a.hx = c.hx; a.hy = c.hy; a.hz = c.hz;
    a.ks = ctx->tune.slab_planes;
    a.st = full ? nullptr : ctx->st;
    a.spin_limit = ctx->wait_limit < 0 ? TMA_SPIN_LIMIT : (unsigned)ctx->wait_limit;
    a.error = f.tma_error;
    const int nslab = (g.N2 - 2 + a.ks - 1) / a.ks;
    dim3 grd((g.N1 - 2 + TMA_TJ - 1) / TMA_TJ, (g.N0 - 2 + TMA_TI - 1) / TMA_TI, nslab);
    const CUtensorMap* a0 = (const CUtensorMap*)f.map_an[ctx->idx[1]];
    const CUtensorMap* a1 = (const CUtensorMap*)f.map_an[ctx->idx[0]];
    int r = timed(ctx, "eval_eb", [&] {
      k_eval_eb_tma<<<grd, TMA_TJ * TMA_TI, kEbTmaSmem, ctx->stream>>>(*a0, *a1, a);
    });
    if (r || full || ctx->n_eb_planes == 0) return r;
    int bx = 32;
    while (bx < 128 && bx < g.N1 - 2) bx *= 2;
    const int by = 256 / bx;
    dim3 pblk(bx, by), pgrd((g.N1 - 2 + bx - 1) / bx, (g.N0 - 2 + by - 1) / by, ctx->n_eb_planes);
    return timed(ctx, "eval_eb_planes", [&] {
      k_eval_eb_planes_f32<<<pgrd, pblk, 0, ctx->stream>>>(g, c, f.A[ctx->idx[0]], f.A[ctx->idx[1]], ctx->E,
                                                          ctx->eb_planes);
    });
  }
  const float* fn = g.space_charge ? ctx->f32.F[ctx->idx[1]] : nullptr;
  // Blocks of 256 threads whose rows span as much of a j row as possible (up to 128 nodes): on a
  // 128-node row, 128 x 2 blocks evaluate in 0.291 ms where 32 x 8 take 0.316 (128x128x2048).
  int bx = 32;
  while (bx < 128 && bx < g.N1 - 2) bx *= 2;
  const int by = 256 / bx;
  dim3 blk(bx, by), grd((g.N1 - 2 + bx - 1) / bx, (g.N0 - 2 + by - 1) / by, g.N2 - 2);
  return timed(ctx, "eval_eb", [&] {
    k_eval_eb_f32<<<grd, blk, 0, ctx->stream>>>(g, c, ctx->f32.A[ctx->idx[0]], ctx->f32.A[ctx->idx[1]], fn, ctx->E,
                                                 1, g.N2 - 2, full ? nullptr : ctx->st, ctx->plane_needed);
  });
}

int fp32_field_update(mithra_ctx* ctx) {
  const GridDev& g = ctx->g;
  Fp32State& f = ctx->f32;
  int r;
  const Coeffs<float> k = make_coeffs<float>(g);
  PotentialArgs<float> pa{f.A[ctx->idx[0]], f.A[ctx->idx[1]], f.A[ctx->idx[2]], 3, (float)g.a[4], k};
  if ((r = run_potential_f32(ctx, pa, true))) return r;
  if (g.space_charge) {
    PotentialArgs<float> pf{f.F[ctx->idx[0]], f.F[ctx->idx[1]], f.F[ctx->idx[2]], 1, (float)g.a[5], k};
    if ((r = run_potential_f32(ctx, pf, false))) return r;
  }
  return fp32_eval_eb(ctx);
}

int fp32_push(mithra_ctx* ctx, int save_rnm) {
  const GridDev& g = ctx->g;
  const PushF32 C = push_constants(ctx);
  UndTableEntry* table = (UndTableEntry*)ctx->und_table;
  int r;
  if (C.n_und > 0) {
    r = timed(ctx, "undulator_table", [&] {
      k_undulator_table<<<std::max(1, (C.n_und * (g.N2 + 1) + 255) / 256), 256, 0, ctx->stream>>>(
          ctx->und_dev, C.n_und, g.N2, g.zmin, g.dz, C.gamma, C.bc, C.dt_shift, ctx->st, table);
    });
    if (r) return r;
  }
  r = timed(ctx, "push", [&] {
    const int blocks = grid_stride_blocks(ctx, (long long)ctx->capacity, 256);
    if (C.P64.n_opt + C.P64.n_ext > 0)
      k_push_f32<true><<<blocks, 256, 0, ctx->stream>>>(C, ctx->und_dev, table, ctx->f32.pt, ctx->E, g.plane, g.P1,
                                                        ctx->st, save_rnm);
    else
      k_push_f32<false><<<blocks, 256, 0, ctx->stream>>>(C, ctx->und_dev, table, ctx->f32.pt, ctx->E, g.plane, g.P1,
                                                         ctx->st, save_rnm);
  });
  if (r) return r;
  return timed(ctx, "substep_end", [&] {
    k_substep_end_f32<<<1, 1024, 0, ctx->stream>>>(ctx->f32.pt, ctx->st, ctx->P.bunch_time_step);
  });
}

int fp32_save_positions(mithra_ctx* ctx) {
  return timed(ctx, "save_positions", [&] {
    k_save_positions_f32<<<grid_stride_blocks(ctx, (long long)ctx->capacity, 256), 256, 0, ctx->stream>>>(ctx->f32.pt, ctx->st);
  });
}

int fp32_erase(mithra_ctx* ctx) {
  return timed(ctx, "erase", [&] {
    k_erase_f32<<<grid_stride_blocks(ctx, (long long)ctx->capacity, 256), 256, 0, ctx->stream>>>(ctx->f32.pt, ctx->st);
  });
}

int fp32_current(mithra_ctx* ctx) {
  const GridDev& g = ctx->g;
  float* J = ctx->f32.A[ctx->idx[0]];
  CK(cudaMemsetAsync(J, 0, (size_t)3 * g.cstride * sizeof(float), ctx->stream));
  float* rho = nullptr;
  if (g.space_charge) {
    rho = ctx->f32.F[ctx->idx[0]];
    CK(cudaMemsetAsync(rho, 0, (size_t)g.cstride * sizeof(float), ctx->stream));
  }
  DepositF32 D{g.N0, g.N1, g.N2, (float)g.dx, (float)g.dy, (float)g.dz};
  Fp32State& f = ctx->f32;
  const TileGrid T = tile_grid(ctx);
  if (fp32_sorts_this_step(ctx) || f.sort_pending) {
    const int r = fp32_sort(ctx);
    if (r) return r;
  }
  CK(cudaMemsetAsync(f.work_count + 2, 0, sizeof(int), ctx->stream));  // the deposit's next list entry
  return timed(ctx, "deposit", [&] {
    k_deposit_tiled<<<ctx->sm_count * kDepositBlocksPerSM, kDepositBlock, 3 * TILE_NODES * sizeof(float), ctx->stream>>>(
        D, T, f.pt, f.offsets, f.work, f.work_count, f.work_count + 2, ctx->st, J, rho, g.cstride, g.plane, g.P1);
  });
}

// The particles are sorted by tile on one step in three (the step whose rotation puts the new
// potential in buffer 0), so a cycle of six steps swaps the buffer sets twice and a step's graph
// stays a function of (rotation, buffer set).  In between, a particle deposits from the tile of
// the last sort: in the boosted frame it moves a fraction of a cell per step, so it stays inside
// that tile's one-cell halo almost always, and the deposit sends it to global atomics when not.
bool fp32_sorts_this_step(const mithra_ctx* ctx) { return ctx->idx[0] == 0; }

int fp32_unsorted(mithra_ctx* ctx, long long n) {
  const TileGrid T = tile_grid(ctx);
  k_offsets_unsorted<<<(T.n_bins + 1 + 255) / 256, 256, 0, ctx->stream>>>(ctx->f32.offsets, T.n_tiles, T.n_bins,
                                                                          (int)n, ctx->f32.work_count);
  CK(cudaGetLastError());
  return MITHRA_OK;
}

int fp32_sort(mithra_ctx* ctx) {
  Fp32State& f = ctx->f32;
  const TileGrid T = tile_grid(ctx);
  const int blocks = grid_stride_blocks(ctx, (long long)ctx->capacity, 256);
  int r = timed(ctx, "tile_hist", [&] {
    k_tile_hist<<<blocks, 256, 0, ctx->stream>>>(T, f.pt, ctx->st, f.counts, f.key, f.rank);
  });
  if (r) return r;
  const int nsb = (T.n_bins + 1023) / 1024;
  r = timed(ctx, "tile_scan", [&] { k_scan_blocks<<<nsb, 1024, 0, ctx->stream>>>(f.counts, f.offsets, f.block_sums, T.n_bins); });
  if (r) return r;
  r = timed(ctx, "tile_scan_totals", [&] { k_scan_totals<<<1, 1024, 0, ctx->stream>>>(f.block_sums, nsb); });
  if (r) return r;
  r = timed(ctx, "tile_scan_add", [&] {
    k_scan_add<<<nsb, 1024, 0, ctx->stream>>>(f.counts, f.offsets, f.block_sums, T.n_bins, nsb, ctx->st);
  });
  if (r) return r;
  CK(cudaMemsetAsync(f.work_count, 0, 2 * sizeof(int), ctx->stream));
  r = timed(ctx, "tile_worklist", [&] {
    k_tile_worklist<<<(T.n_tiles + 255) / 256, 256, 0, ctx->stream>>>(f.offsets, T.n_tiles, f.work, f.work_count);
  });
  if (r) return r;
  r = timed(ctx, "tile_scatter", [&] {
    k_tile_scatter<<<blocks, 256, 0, ctx->stream>>>(f.pt, f.alt, f.key, f.rank, f.offsets, T.n_bins);
  });
  if (r) return r;
  fp32_after_step(ctx);  // the sorted set becomes current
  f.sort_pending = false;
  return MITHRA_OK;
}

}  // namespace mithra
