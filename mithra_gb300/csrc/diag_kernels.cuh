// Bunch diagnostics on the device: the moments of Solver::bunchSample (src/solver.cpp:1582-1635)
// and the bunching factor |sum q exp(i k z)| / sum q (the quantity FEL studies read from the
// bunch dumps of Solver::bunchProfile, src/solver.cpp:1763-1792).
//
// Sums are FP64 and compensated: every thread keeps a Neumaier sum per quantity, warps and blocks
// combine (sum, compensation) pairs with an error-free two-sum, and one block adds the block
// results in block order.  The result does not depend on the particle order beyond the last
// bits, and is reproducible for a fixed launch shape.
#pragma once
#include "device_common.cuh"

namespace mithra {

constexpr int kDiagBlock = 256;
constexpr int kDiagMaxBlocks = 1024;
constexpr int kDiagValues = 13;  // q, q r (3), q r^2 (3), q gb (3), q gb^2 (3)

struct CSum {
  double s, c;
};

__device__ __forceinline__ void csum_add(CSum& a, double v) {  // Neumaier
  const double t = a.s + v;
  a.c += (fabs(a.s) >= fabs(v)) ? (a.s - t) + v : (v - t) + a.s;
  a.s = t;
}

__device__ __forceinline__ CSum csum_merge(CSum a, CSum b) {
  CSum r;
  r.s = a.s + b.s;
  const double bb = r.s - a.s;
  r.c = a.c + b.c + ((a.s - (r.s - bb)) + (b.s - bb));
  return r;
}

// Block-level reduction of NV compensated sums; thread 0 writes them to out[blockIdx.x * NV ...].
template <int NV>
__device__ __forceinline__ void csum_block_store(CSum* v, double2* out) {
  __shared__ double2 sh[kDiagBlock / 32][NV];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NV; q++) {
    for (int o = 16; o > 0; o >>= 1) {
      CSum w{__shfl_down_sync(0xffffffffu, v[q].s, o), __shfl_down_sync(0xffffffffu, v[q].c, o)};
      v[q] = csum_merge(v[q], w);
    }
    if (lane == 0) sh[warp][q] = make_double2(v[q].s, v[q].c);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 0; q < NV; q++) {
      CSum a{sh[0][q].x, sh[0][q].y};
      for (int w = 1; w < kDiagBlock / 32; w++) a = csum_merge(a, CSum{sh[w][q].x, sh[w][q].y});
      out[blockIdx.x * NV + q] = make_double2(a.s, a.c);
    }
  }
}

// Particle position (and gamma*beta) in FP64 for either particle form.
struct DiagParticles {
  // FP64 form
  const double *x, *y, *z, *gx, *gy, *gz, *q;
  // mixed form
  const long long* cell;
  const float *fx, *fy, *fz, *gxf, *gyf, *gzf, *qf;
  const uint8_t* status;
  // previous position (rnm) and list order, for the screen crossing
  const double *mx, *my, *mz;
  const long long* mcell;
  const float *mfx, *mfy, *mfz;
  const int* id;
  double xmin, ymin, zmin, dx, dy, dz;
  __device__ __forceinline__ void get_rnm(long long p, double* r) const {
    if (x) {
      r[0] = mx[p]; r[1] = my[p]; r[2] = mz[p];
    } else {
      int i, j, k;
      unpack_cell(mcell[p], i, j, k);
      r[0] = xmin + ((double)i + (double)mfx[p]) * dx;
      r[1] = ymin + ((double)j + (double)mfy[p]) * dy;
      r[2] = zmin + ((double)k + (double)mfz[p]) * dz;
    }
  }
  // position in the reference's particle list (erased particles never reach here)
  __device__ __forceinline__ long long order(long long p) const { return x ? p : (long long)id[p]; }
  __device__ __forceinline__ void get(long long p, double* r, double* g, double& qq) const {
    if (x) {
      r[0] = x[p]; r[1] = y[p]; r[2] = z[p];
      g[0] = gx[p]; g[1] = gy[p]; g[2] = gz[p];
      qq = q[p];
    } else {
      int i, j, k;
      unpack_cell(cell[p], i, j, k);
      r[0] = xmin + ((double)i + (double)fx[p]) * dx;
      r[1] = ymin + ((double)j + (double)fy[p]) * dy;
      r[2] = zmin + ((double)k + (double)fz[p]) * dz;
      g[0] = gxf[p]; g[1] = gyf[p]; g[2] = gzf[p];
      qq = qf[p];
    }
  }
};

// particleInProcessor, src/solver.cpp:2292-2296.
__device__ __forceinline__ bool in_processor(const GridDev& g, double z) {
  const double zr = pmod_d(z - g.zmin, g.Lz) + g.zmin;
  return zr >= g.zp0 && zr < g.zp1;
}

__global__ void __launch_bounds__(kDiagBlock) k_bunch_moments(GridDev g, DiagParticles P, const StateDev* st,
                                                              double2* partial) {
  CSum v[kDiagValues];
#pragma unroll
  for (int q = 0; q < kDiagValues; q++) v[q] = CSum{0.0, 0.0};
  const long long n = st->n_particles;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    if (P.status[p] & 1) continue;
    double r[3], gb[3], q;
    P.get(p, r, gb, q);
    if (!in_processor(g, r[2])) continue;
    csum_add(v[0], q);
#pragma unroll
    for (int c = 0; c < 3; c++) {
      csum_add(v[1 + c], q * r[c]);
      csum_add(v[4 + c], r[c] * r[c] * q);
      csum_add(v[7 + c], q * gb[c]);
      csum_add(v[10 + c], gb[c] * gb[c] * q);
    }
  }
  csum_block_store<kDiagValues>(v, partial);
}

__global__ void __launch_bounds__(kDiagBlock) k_bunching(GridDev g, DiagParticles P, const StateDev* st, double k,
                                                         double2* partial) {
  CSum v[3] = {{0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}};
  const long long n = st->n_particles;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    if (P.status[p] & 1) continue;
    double r[3], gb[3], q;
    P.get(p, r, gb, q);
    if (!in_processor(g, r[2])) continue;
    double sn, cs;
    sincos(k * r[2], &sn, &cs);
    csum_add(v[0], q);
    csum_add(v[1], q * cs);
    csum_add(v[2], q * sn);
  }
  csum_block_store<3>(v, partial);
}

// Lab-frame screens of Solver::screenProfile (src/solver.cpp:2205-2257).  rec holds 6 doubles
// per record (x, y, t, gbx, gby, gbz_lab), key the sort key (n_time << 40 | list order) that
// restores the reference's file order (steps in order, particles in list order).
struct ScreenDev {
  double gamma, beta, c0, dt_shift, dt;
  int n;
  const double* lz;
  double* rec;
  long long* key;
  unsigned long long* count;
  long long cap;  // records per screen
};

// Solver::interp (src/solver.cpp:2283-2286) without contraction.
__device__ __forceinline__ double screen_interp(double x0, double x1, double y0, double y1, double x) {
  return __dadd_rn(y0, __dmul_rn(__ddiv_rn(__dsub_rn(x, x0), __dsub_rn(x1, x0)), __dsub_rn(y1, y0)));
}

// Every particle in the domain whose lab z (gamma (z + beta c0 t)) passes a screen between the
// start (rnm, timeBunch - dt) and the end (rnp, timeBunch) of the step is recorded: x, y and the
// lab time interpolated linearly in lab z to the screen, the momentum after the step and its lab
// longitudinal component.  The reference's operation order is kept, without contraction, so the
// FP64 form reproduces its values from the same positions.
__global__ void __launch_bounds__(256) k_screen(GridDev g, DiagParticles P, ScreenDev S, const StateDev* st) {
  const long long n = st->n_particles;
  const double tb = st->time_bunch;
  const long long step = st->n_time;
  const double bc = __dmul_rn(S.beta, S.c0), boc = __ddiv_rn(S.beta, S.c0);
  const double tm0 = __dadd_rn(__dsub_rn(tb, S.dt), S.dt_shift);        // timeBunch_ - dt + dt_
  const double tp0 = __dadd_rn(tb, S.dt_shift);                           // timeBunch_ + dt_
  const double tt_m = __dsub_rn(__dadd_rn(tb, S.dt_shift), S.dt);         // timeBunch_ + dt_ - dt
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    if (P.status[p] & 1) continue;
    double r[3], gb[3], q;
    P.get(p, r, gb, q);
    if (!in_processor(g, r[2])) continue;
    double rm[3];
    P.get_rnm(p, rm);
    const double lzm = __dmul_rn(S.gamma, __dadd_rn(rm[2], __dmul_rn(bc, tm0)));
    const double lzp = __dmul_rn(S.gamma, __dadd_rn(r[2], __dmul_rn(bc, tp0)));
    for (int i = 0; i < S.n; i++) {
      const double lzs = S.lz[i];
      if (lzm >= lzs || lzp < lzs) continue;
      const unsigned long long slot = atomicAdd(&S.count[i], 1ull);
      if ((long long)slot >= S.cap) continue;  // counted; the host reports the overflow
      double* o = S.rec + ((long long)i * S.cap + (long long)slot) * 6;
      o[0] = screen_interp(lzm, lzp, rm[0], r[0], lzs);
      o[1] = screen_interp(lzm, lzp, rm[1], r[1], lzs);
      const double tm = __dmul_rn(S.gamma, __dadd_rn(tt_m, __dmul_rn(boc, rm[2])));
      const double tp = __dmul_rn(S.gamma, __dadd_rn(tp0, __dmul_rn(boc, r[2])));
      o[2] = screen_interp(lzm, lzp, tm, tp, lzs);
      o[3] = gb[0];
      o[4] = gb[1];
      const double n2 = __dadd_rn(__dadd_rn(__dmul_rn(gb[0], gb[0]), __dmul_rn(gb[1], gb[1])), __dmul_rn(gb[2], gb[2]));
      o[5] = __dmul_rn(S.gamma, __dadd_rn(gb[2], __dmul_rn(S.beta, __dsqrt_rn(__dadd_rn(1.0, n2)))));
      S.key[(long long)i * S.cap + (long long)slot] = (step << 40) | P.order(p);
    }
  }
}

// Adds the block results in block order; out[q] = compensated total of quantity q.
__global__ void k_diag_finish(const double2* partial, int nblocks, int nv, double* out) {
  const int q = threadIdx.x;
  if (q >= nv) return;
  CSum a{0.0, 0.0};
  for (int b = 0; b < nblocks; b++) a = csum_merge(a, CSum{partial[b * nv + q].x, partial[b * nv + q].y});
  out[q] = a.s + a.c;
}

// FdTd::fieldSample (src/fdtd.cpp:851-950): E, B and A^n at each point, trilinear with the
// reference's weights (modf of the cell coordinate); out[9 p + 0..8] = E, B, A.  Component c of
// node m of E (B) is E[c * ecs + m * ens] (see k_power_sample); A is in component planes.
template <typename TE, typename TA>
__global__ void k_field_sample(GridDev g, const TE* __restrict__ E, const TE* __restrict__ B, long long ecs, int ens,
                               const TA* __restrict__ A, const double* __restrict__ pts, int n,
                               double* __restrict__ out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const double* r = pts + 3 * p;
  double c;
  const double dxr = modf((r[0] - g.xmin) / g.dx, &c); const int i = (int)c;
  const double dyr = modf((r[1] - g.ymin) / g.dy, &c); const int j = (int)c;
  const double dzr = modf((r[2] - g.zmin) / g.dz, &c); const int k = (int)c;
  double* o = out + 9 * (long long)p;
  if (i < 0 || j < 0 || k < 0 || i > g.N0 - 2 || j > g.N1 - 2 || k > g.N2 - 2) {  // outside the mesh
    for (int q = 0; q < 9; q++) o[q] = nan("");
    return;
  }
  const long long m = node_index(g, k, i, j), sI = g.P1, sK = g.plane, cs = g.cstride;
  const long long nd[8] = {m, m + sI, m + 1, m + sI + 1, m + sK, m + sK + sI, m + sK + 1, m + sK + sI + 1};
  const double w[8] = {(1.0 - dxr) * (1.0 - dyr) * (1.0 - dzr), dxr * (1.0 - dyr) * (1.0 - dzr),
                       (1.0 - dxr) * dyr * (1.0 - dzr),         dxr * dyr * (1.0 - dzr),
                       (1.0 - dxr) * (1.0 - dyr) * dzr,         dxr * (1.0 - dyr) * dzr,
                       (1.0 - dxr) * dyr * dzr,                 dxr * dyr * dzr};
  for (int comp = 0; comp < 3; comp++) {
    double e = 0.0, b = 0.0, a = 0.0;
    for (int q = 0; q < 8; q++) {
      e += w[q] * (double)E[comp * ecs + nd[q] * ens];
      b += w[q] * (double)B[comp * ecs + nd[q] * ens];
      a += w[q] * (double)A[comp * cs + nd[q]];
    }
    o[comp] = e; o[3 + comp] = b; o[6 + comp] = a;
  }
}

}  // namespace mithra
