// Kernels of the mixed-precision form.
//
// Storage: potentials, J, rho, E and B in FP32; particles as an integer cell (packed 64-bit) plus
// an FP32 offset inside the cell (in cell units) and FP32 gamma*beta.  FP64 is kept where the
// magnitudes need it: the lab-frame undulator coordinate lz (up to ~1e6 length units, whose
// phase ku*lz must be exact to ~1e-7 rad) is formed and range-reduced in FP64, and the time
// state stays FP64.  Everything else runs on the FP32 pipes.
#pragma once
#include "beam_fields.cuh"
#include "device_common.cuh"

namespace mithra {

// E and B from FP32 potentials (the FdTd::fieldEvaluate formulas, src/fdtd.cpp:818-845, in
// float; with space charge src/fdtdSC.cpp:1116-1118).
struct EBConstF32 {
  float rdt, hx, hy, hz;  // 1/dt and 0.5/(2 d) per axis
};


// E and B of one interior node (FdTd::fieldEvaluate, src/fdtd.cpp:818-845; SC src/fdtdSC.cpp:1110-1140)
// from A^{n+1} (A1), A^n (A0) and phi^n (fn, space charge only), with the copies of planes 1 and
// N2-2 into the boundary planes (src/fdtd.cpp:755-772).
__device__ __forceinline__ void eval_eb_node_f32(const GridDev& g, const EBConstF32& c, const float* __restrict__ A1,
                                                 const float* __restrict__ A0, const float* __restrict__ fn,
                                                 float* __restrict__ EB, int k, int i, int j) {
  const long long m = node_index(g, k, i, j);
  const long long cs = g.cstride, sI = g.P1, sK = g.plane;
  const float rdt = c.rdt, hx = c.hx, hy = c.hy, hz = c.hz;
  float e0 = (A0[m] - A1[m]) * rdt;
  float e1 = (A0[cs + m] - A1[cs + m]) * rdt;
  float e2 = (A0[2 * cs + m] - A1[2 * cs + m]) * rdt;
  if (fn) {
    e0 -= (fn[m + sI] - fn[m - sI]) * (2.0f * hx);
    e1 -= (fn[m + 1] - fn[m - 1]) * (2.0f * hy);
    e2 -= (fn[m + sK] - fn[m - sK]) * (2.0f * hz);
  }
  const float *X0 = A0, *Y0 = A0 + cs, *Z0 = A0 + 2 * cs, *X1 = A1, *Y1 = A1 + cs, *Z1 = A1 + 2 * cs;
  const float b0 = ((Z0[m + 1] + Z1[m + 1]) - (Z0[m - 1] + Z1[m - 1])) * hy -
                   ((Y0[m + sK] + Y1[m + sK]) - (Y0[m - sK] + Y1[m - sK])) * hz;
  const float b1 = ((X0[m + sK] + X1[m + sK]) - (X0[m - sK] + X1[m - sK])) * hz -
                   ((Z0[m + sI] + Z1[m + sI]) - (Z0[m - sI] + Z1[m - sI])) * hx;
  const float b2 = ((Y0[m + sI] + Y1[m + sI]) - (Y0[m - sI] + Y1[m - sI])) * hx -
                   ((X0[m + 1] + X1[m + 1]) - (X0[m - 1] + X1[m - 1])) * hy;
  store_eb(EB, m, e0, e1, e2, b0, b1, b2);
  if (k == 1) store_eb(EB, m - sK, e0, e1, e2, b0, b1, b2);
  if (k == g.N2 - 2) store_eb(EB, m + sK, e0, e1, e2, b0, b1, b2);
}

__global__ void __launch_bounds__(256) k_eval_eb_f32(GridDev g, EBConstF32 c, const float* __restrict__ A1,
                                                     const float* __restrict__ A0,
                                                     const float* __restrict__ fn, float* __restrict__ EB,
                                                     int k_lo, int k_hi, const StateDev* st,
                                                     const uint8_t* plane_needed) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int i = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z + k_lo;
  if (j > g.N1 - 2 || i > g.N0 - 2 || k > k_hi) return;
  if (!eb_plane_wanted(k, st, plane_needed, g.N2)) return;
  eval_eb_node_f32(g, c, A1, A0, fn, EB, k, i, j);
}

// E and B on the planes of a list (the power-sampling planes outside the particle slab).
__global__ void __launch_bounds__(256) k_eval_eb_planes_f32(GridDev g, EBConstF32 c, const float* __restrict__ A1,
                                                            const float* __restrict__ A0, float* __restrict__ EB,
                                                            const int* __restrict__ planes) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int i = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (j > g.N1 - 2 || i > g.N0 - 2) return;
  eval_eb_node_f32(g, c, A1, A0, nullptr, EB, planes[blockIdx.z], i, j);
}

// Per-launch constants of the mixed-precision push, prepared on the host from GridDev/PushDev.
struct PushF32 {
  float rdx, rdy, rdz;           // 1/d in cell units per length unit
  float dx, dy, dz;
  float xmin, ymin;              // for the transverse undulator coordinate
  float r1, r2, dtb;
  int N0, N1, N2;
  double zmin, dzd, gamma, bc;   // FP64: z reconstruction and the lab frame (bc = beta*c0)
  double dt_shift;
  int n_und;
  double und0_dist;
  float gamma_f, bc_f, gdz;      // gamma, beta*c0 and gamma*dz in FP32
  float zmin_f, dz_f, und0_dist_f;
  float rb0_f;                   // rb of the first undulator module
  PushDev P64;                   // FP64 parameters for the laser beams (optical undulators, external fields)
  double xmin_d, ymin_d, dxd, dyd;
};

// Static undulator field (src/solver.cpp:1798-1824, src/beam.cc:14-76).
//
// The lab coordinate lz = gamma (z + beta c0 (timeBunch + dt_)) - rb reaches ~1e6 length units,
// so the phase ku*lz cannot be formed in FP32.  With z = zmin + (k + fz) dz it splits into a
// per-plane part, computed in FP64 and reduced modulo 2 pi once per substep for every plane k
// (k_undulator_table), and an in-cell part (ku gamma dz) fz that is small and formed in FP32.
struct UndTableEntry {
  float lz;     // lab coordinate of plane k (relative to the module start)
  float phase;  // ku * lz reduced to [-pi, pi]
};

__global__ void k_undulator_table(const UndDev* __restrict__ und, int n_und, int N2, double zmin, double dz,
                                  double gamma, double bc, double dt_shift, const StateDev* st,
                                  UndTableEntry* table) {
  const double tshift = bc * (st->time_bunch + dt_shift);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n_und * (N2 + 1); t += gridDim.x * blockDim.x) {
    const int u = t / (N2 + 1), k = t % (N2 + 1);
    const double lz = gamma * (zmin + (double)k * dz + tshift) - und[u].rb;
    const double ph = und[u].ku * lz;
    const double n = rint(ph * (1.0 / (2.0 * kPI)));
    table[t].lz = (float)lz;
    table[t].phase = (float)fma(-n, 2.0 * kPI, ph);
  }
}

// Lab-frame z, gamma (z + beta c0 (timeBunch + dt_)), of a particle outside the mesh's z range,
// in FP64.  Out of line, so that the FP64 instructions run only for the (rare) particles that
// need them instead of being predicated into every thread's path.
__device__ __noinline__ double lab_z_outside(double zmin, double dzd, double gamma, double tshift, int k, float fz) {
  return gamma * (zmin + ((double)k + (double)fz) * dzd + tshift);
}

// The same lab z rounded to float, out of line like lab_z_outside: GB300 converts double to float
// on its FP64 pipe, and only particles outside the mesh's z range need the conversion.
__device__ __noinline__ float to_float_outside(double v) { return (float)v; }

// Undulator lz and phase ku*lz reduced modulo 2 pi, from the FP64 lab z (particles outside the mesh).
__device__ __noinline__ float2 undulator_phase_outside(double labz, double rb, double ku) {
  const double lzd = labz - rb;
  const double ph = ku * lzd;
  return make_float2((float)lzd, (float)fma(-rint(ph * (1.0 / (2.0 * kPI))), 2.0 * kPI, ph));
}

__device__ __forceinline__ void undulator_f32(const UndDev* __restrict__ und, const UndTableEntry* __restrict__ table,
                                              int n_und, int N2, float gdz, int k, float fz, double labz_outside,
                                              float x, float y, float* bt, float* et, float gamma_f, float bc_f) {
  for (int u = 0; u < n_und; u++) {
    const UndDev& U = und[u];
    if (U.type != 0) continue;
    float lz, phase;
    if (k >= 0 && k <= N2) {
      const UndTableEntry te = table[u * (N2 + 1) + k];
      lz = fmaf(gdz, fz, te.lz);
      phase = fmaf(U.ku_f * gdz, fz, te.phase);
    } else {  // outside the mesh along z (rare): form the phase in FP64
      const float2 lp = undulator_phase_outside(labz_outside, U.rb, U.ku);
      lz = lp.x;
      phase = lp.y;
    }
    const float ct = U.ct_f, st = U.st_f, ku = U.ku_f, b0 = U.b0_f;
    const float ly = x * ct + y * st;
    float s_ly, c_ly;
    {
      const float a = ku * ly;
      const float e = __expf(a);
      const float ie = 1.0f / e;
      c_ly = 0.5f * (e + ie);
      if (fabsf(a) < 0.05f) {  // short series where e - 1/e cancels
        const float a2 = a * a;
        s_ly = a * (1.0f + a2 * (1.0f / 6.0f) * (1.0f + a2 * (1.0f / 20.0f)));
      } else {
        s_ly = 0.5f * (e - ie);
      }
    }
    float d1, bz;
    if (lz >= 0.0f && lz <= U.ul_f) {
      float sn, cs;
      __sincosf(phase, &sn, &cs);
      d1 = b0 * c_ly * sn * gamma_f;
      bz = b0 * s_ly * cs;
    } else {
      const float t0 = (lz < 0.0f) ? lz : lz - U.ul_f;
      const float kt = ku * t0;
      float sz = __expf(-0.5f * kt * kt);
      const bool has = (lz < 0.0f) ? U.has_prev : U.has_next;
      if (has) {
        const float r0 = (lz < 0.0f) ? U.r0_prev_f : U.r0_next_f;
        const bool cut = (lz < 0.0f) ? (t0 < r0 || r0 == 0.0f) : (t0 > r0 || r0 == 0.0f);
        if (cut) sz = 0.0f;
        else {
          const float a = 3.1415926535f * t0 / r0;
          sz *= 0.35875f + 0.48829f * __cosf(a) + 0.14128f * __cosf(2.0f * a) + 0.01168f * __cosf(3.0f * a);
        }
      }
      d1 = b0 * c_ly * sz * ku * t0 * gamma_f;
      bz = b0 * s_ly * sz;
    }
    bt[0] += d1 * ct;
    bt[1] += d1 * st;
    bt[2] += bz;
    d1 *= bc_f;
    et[1] += d1 * ct;
    et[0] -= d1 * st;
  }
}

// One bunch substep (src/solver.cpp:1424-1549) in the mixed form.  Positions are (cell, offset)
// in cell units; the owned-domain test of the reference (wrapped z in [zp0, zp1)) is always true
// for one domain and is folded into the crossing test.
// BEAMS: the job defines optical undulators or external fields (a separate instantiation keeps
// the FP64 laser-beam code, and its registers, out of the common kernel).
template <bool BEAMS>
__global__ void __launch_bounds__(256, BEAMS ? 1 : 4) k_push_f32(PushF32 C, const UndDev* __restrict__ und,
                                                  const UndTableEntry* __restrict__ table, ParticlesF32 pt,
                                                  const float* __restrict__ EB, long long plane, int P1,
                                                  StateDev* st, int save_rnm) {
  const long long n = st->n_particles;
  const double tb = st->time_bunch;
  const double tshift = C.bc * (tb + C.dt_shift);  // beta c0 (timeBunch + dt_)
  unsigned long long local_cross = 0, local_nt = 0;
  // The next particle's state is loaded before the current one's gather and Boris step, so each
  // thread keeps two particles' loads in flight.
  struct Loaded {
    long long cell;
    float fx, fy, fz, gx, gy, gz;
    uint8_t status, e;
  };
  auto load = [&](long long q) {
    Loaded L;
    L.status = pt.status[q];
    L.cell = pt.cell[q];
    L.fx = pt.fx[q]; L.fy = pt.fy[q]; L.fz = pt.fz[q];
    L.gx = pt.gx[q]; L.gy = pt.gy[q]; L.gz = pt.gz[q];
    L.e = pt.e[q];
    return L;
  };
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  Loaded cur{};
  if (p < n) cur = load(p);
  for (; p < n; p += stride) {
    Loaded nxt{};
    if (p + stride < n) nxt = load(p + stride);
    int8_t cross = 0;
    if (!(cur.status & 1)) {
      const long long cell = cur.cell;
      int i, j, k;
      unpack_cell(cell, i, j, k);
      const int Lk = C.N2 - 1;
      float fx = cur.fx, fy = cur.fy, fz = cur.fz;
      if (save_rnm) { pt.mcell[p] = cell; pt.mfx[p] = fx; pt.mfy[p] = fy; pt.mfz[p] = fz; }
      const float x = C.xmin + ((float)i + fx) * C.dx, y = C.ymin + ((float)j + fy) * C.dy;
      const bool b1x = (i >= 1 && i <= C.N0 - 3 && (i > 1 || fx > 0.0f));
      const bool b1y = (j >= 1 && j <= C.N1 - 3 && (j > 1 || fy > 0.0f));
      const bool b1z = (k >= 0 && k <= C.N2 - 2);
      float bt[3] = {0.f, 0.f, 0.f}, et[3] = {0.f, 0.f, 0.f};
      const bool k_in = (k >= 0 && k <= C.N2);
      double labz_outside = 0.0;
      if (!k_in) labz_outside = lab_z_outside(C.zmin, C.dzd, C.gamma, tshift, k, fz);
      undulator_f32(und, table, C.n_und, C.N2, C.gdz, k, fz, labz_outside, x, y, bt, et, C.gamma_f, C.bc_f);
      if (BEAMS) {
        // Laser beams in FP64: their phase, like the undulator's, is a large lab-frame coordinate.
        const double xd = C.xmin_d + ((double)i + (double)fx) * C.dxd;
        const double yd = C.ymin_d + ((double)j + (double)fy) * C.dyd;
        const double zd = C.zmin + ((double)k + (double)fz) * C.dzd;
        double b64[3] = {0.0, 0.0, 0.0}, e64[3] = {0.0, 0.0, 0.0};
        laser_beams_add(C.P64, und, C.n_und, tb, xd, yd, zd, b64, e64);
        for (int c = 0; c < 3; c++) { bt[c] += (float)b64[c]; et[c] += (float)e64[c]; }
      }
      uint8_t e = cur.e;
      if (e) {
        if (b1x && b1y && b1z) {
          const long long m = (long long)k * plane + (long long)i * P1 + j;
          const long long sI = P1, sK = plane;
          const float wx0 = 1.0f - fx, wy0 = 1.0f - fy, wz0 = 1.0f - fz;
          const float w[8] = {wx0 * wy0 * wz0, fx * wy0 * wz0, wx0 * fy * wz0, fx * fy * wz0,
                              wx0 * wy0 * fz, fx * wy0 * fz, wx0 * fy * fz, fx * fy * fz};
          const long long nd[8] = {m, m + sI, m + 1, m + sI + 1, m + sK, m + sK + sI, m + sK + 1, m + sK + sI + 1};
          // Node records {E, 0, B, 0}: one 32-byte load per node.  Each component still sums
          // its eight terms in node order onto the undulator field.
#pragma unroll
          for (int q = 0; q < 8; q++) {
            float4 e, b;
            load_eb(EB, nd[q], e, b);
            et[0] = fmaf(w[q], e.x, et[0]); et[1] = fmaf(w[q], e.y, et[1]); et[2] = fmaf(w[q], e.z, et[2]);
            bt[0] = fmaf(w[q], b.x, bt[0]); bt[1] = fmaf(w[q], b.y, bt[1]); bt[2] = fmaf(w[q], b.z, bt[2]);
          }
        } else if (!b1x && !b1y && b1z) {
          local_nt++;
        }
      } else if (C.n_und > 0) {
        // lz without the module offset rb: rb of the first module is zero after the shift of
        // src/solver.cpp:184-185, so it is the first table entry's lz.
        float lz;
        if (k_in) lz = fmaf(C.gdz, fz, table[k].lz + C.rb0_f);
        else lz = to_float_outside(labz_outside);
        e = (lz > -C.und0_dist_f) ? 1 : 0;
        pt.e[p] = e;
      } else {
        pt.e[p] = 1;
      }
      // Boris rotation and drift (src/solver.cpp:1519-1541) in FP32.
      float gx = cur.gx, gy = cur.gy, gz = cur.gz;
      const float mx = fmaf(C.r1, et[0], gx), my = fmaf(C.r1, et[1], gy), mz = fmaf(C.r1, et[2], gz);
      const float d1 = sqrtf(1.0f + (mx * mx + my * my + mz * mz));
      const float f = C.r2 / d1;
      const float px = fmaf(f, my * bt[2] - mz * bt[1], mx);
      const float py = fmaf(f, mz * bt[0] - mx * bt[2], my);
      const float pz = fmaf(f, mx * bt[1] - my * bt[0], mz);
      const float bt2 = bt[0] * bt[0] + bt[1] * bt[1] + bt[2] * bt[2];
      const float s = 2.0f / (d1 / C.r2 + f * bt2);
      gx = fmaf(s, py * bt[2] - pz * bt[1], mx) + C.r1 * et[0];
      gy = fmaf(s, pz * bt[0] - px * bt[2], my) + C.r1 * et[1];
      gz = fmaf(s, px * bt[1] - py * bt[0], mz) + C.r1 * et[2];
      pt.gx[p] = gx; pt.gy[p] = gy; pt.gz[p] = gz;
      const float gg = C.dtb * rsqrtf(1.0f + (gx * gx + gy * gy + gz * gz));
      fx = fmaf(gg * C.rdx, gx, fx);
      fy = fmaf(gg * C.rdy, gy, fy);
      const float dzc = gg * C.rdz * gz;
      fz += dzc;
      const float ix = floorf(fx), iy = floorf(fy), iz = floorf(fz);
      i += (int)ix; j += (int)iy; k += (int)iz;
      fx -= ix; fy -= iy; fz -= iz;
      pt.cell[p] = pack_cell(i, j, k);
      pt.fx[p] = fx; pt.fy[p] = fy; pt.fz[p] = fz;
      // The erase of non-finite particles (k_erase_f32), done here while the values are in registers.
      if (!isfinite(gx + gy + gz + fx + fy + fz)) {
        pt.status[p] = cur.status | 1;
        atomicAdd(&st->nonfinite, 1);
      }
      // z-face crossing of the wrapped position (src/solver.cpp:1544-1548), in cells: kw is the
      // cell of pmod(z - zmin, Lz) before the drift, the particle's own cell inside the mesh (the
      // integer modulo, tens of instructions, only outside it).
      const int ko = k - (int)iz;
      const int kw = (ko >= 0 && ko < Lk) ? ko : ((ko % Lk) + Lk) % Lk;
      const int kwn = kw + (int)iz;
      if (kwn < 0) cross = 1;
      else if (kwn >= Lk) cross = 2;
    }
    pt.cross[p] = cross;
    local_cross += (cross != 0);
    cur = nxt;
  }
  for (int o = 16; o > 0; o >>= 1) {
    local_cross += __shfl_down_sync(0xffffffffu, local_cross, o);
    local_nt += __shfl_down_sync(0xffffffffu, local_nt, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (local_cross) atomicAdd(&st->n_cross, local_cross);
    if (local_nt) atomicAdd(&st->n_transverse, local_nt);
  }
}

// The ordered append of z-face copies (src/solver.cpp:1551-1568) and the bunch time advance,
// for the mixed-form particle arrays (one block).
// Copies of the particles that crossed a z face in one pass, ordered by id when they fit here
// (the reference appends them in its list order, which the ids follow); more than this many in
// one pass are appended in array order.
constexpr int kCrossSorted = 2048;

__device__ __forceinline__ void copy_particle(const ParticlesF32& pt, long long d, long long p, int id) {
  pt.cell[d] = pt.cell[p]; pt.fx[d] = pt.fx[p]; pt.fy[d] = pt.fy[p]; pt.fz[d] = pt.fz[p];
  pt.gx[d] = pt.gx[p]; pt.gy[d] = pt.gy[p]; pt.gz[d] = pt.gz[p];
  pt.mcell[d] = pt.mcell[p]; pt.mfx[d] = pt.mfx[p]; pt.mfy[d] = pt.mfy[p]; pt.mfz[d] = pt.mfz[p];
  pt.q[d] = pt.q[p]; pt.e[d] = pt.e[p]; pt.status[d] = pt.status[p]; pt.cross[d] = 0;
  pt.id[d] = id;
}

__global__ void __launch_bounds__(1024) k_substep_end_f32(ParticlesF32 pt, StateDev* st, double bunch_time_step) {
  __shared__ long long s_base;
  __shared__ int s_warp[32];
  __shared__ int s_count;
  __shared__ int s_idx[kCrossSorted];
  __shared__ int s_key[kCrossSorted];
  const unsigned long long ncross = st->n_cross;
  if (ncross) {
    const long long n = st->n_particles;
    if (threadIdx.x == 0) s_base = n;
    __syncthreads();
    if ((long long)(n + ncross) > st->capacity) {
      if (threadIdx.x == 0) st->overflow = 1;
    } else {
      const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      for (int pass = 1; pass <= 2; pass++) {
        // this pass's crossing particles, in array order, into s_idx
        if (threadIdx.x == 0) s_count = 0;
        __syncthreads();
        for (long long c0 = 0; c0 < n; c0 += blockDim.x) {
          const long long p = c0 + threadIdx.x;
          const int take = (p < n) && (pt.cross[p] == pass);
          const unsigned bal = __ballot_sync(0xffffffffu, take);
          if (lane == 0) s_warp[warp] = __popc(bal);
          __syncthreads();
          int before = 0, total = 0;
          for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            if (w < warp) before += s_warp[w];
            total += s_warp[w];
          }
          before += __popc(bal & ((1u << lane) - 1u));
          const int slot = s_count + before;
          if (take && slot < kCrossSorted) s_idx[slot] = (int)p;
          __syncthreads();
          if (threadIdx.x == 0) s_count += total;
          __syncthreads();
        }
        const int m = s_count;
        if (m <= kCrossSorted) {
          // rank by id (ids are distinct): copy t goes to s_base + #{u : id_u < id_t}
          for (int t = threadIdx.x; t < m; t += blockDim.x) s_key[t] = pt.id[s_idx[t]];
          __syncthreads();
          for (int t = threadIdx.x; t < m; t += blockDim.x) {
            const int key = s_key[t];
            int r = 0;
            for (int u = 0; u < m; u++) r += s_key[u] < key;
            const long long d = s_base + r;
            copy_particle(pt, d, s_idx[t], (int)(st->next_id + (d - n)));
          }
        } else {
          for (long long c0 = 0; c0 < n; c0 += blockDim.x) {
            const long long p = c0 + threadIdx.x;
            const int take = (p < n) && (pt.cross[p] == pass);
            const unsigned bal = __ballot_sync(0xffffffffu, take);
            if (lane == 0) s_warp[warp] = __popc(bal);
            __syncthreads();
            int before = 0, total = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
              if (w < warp) before += s_warp[w];
              total += s_warp[w];
            }
            before += __popc(bal & ((1u << lane) - 1u));
            if (take) {
              const long long d = s_base + before;
              copy_particle(pt, d, p, (int)(st->next_id + (d - n)));
            }
            __syncthreads();
            if (threadIdx.x == 0) s_base += total;
            __syncthreads();
          }
          continue;
        }
        __syncthreads();
        if (threadIdx.x == 0) s_base += m;
        __syncthreads();
      }
      if (threadIdx.x == 0) {
        st->next_id += s_base - n;
        st->n_particles = s_base;
      }
    }
  }
  if (threadIdx.x == 0) {
    st->n_cross = 0;
    st->time_bunch += bunch_time_step;
    st->n_time_bunch += 1;
  }
}

// Erasure of particles whose wrapped z is outside the domain (src/solver.cpp:493-503): with cells,
// the wrapped cell index always lands inside, so only non-finite states are erased.
__global__ void __launch_bounds__(256) k_erase_f32(ParticlesF32 pt, StateDev* st) {
  const long long n = st->n_particles;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    if (pt.status[p] & 1) continue;
    if (!isfinite(pt.gx[p] + pt.gy[p] + pt.gz[p] + pt.fx[p] + pt.fy[p] + pt.fz[p])) {
      pt.status[p] |= 1;
      atomicAdd(&st->nonfinite, 1);
    }
  }
}

__global__ void k_save_positions_f32(ParticlesF32 pt, const StateDev* st) {
  const long long n = st->n_particles;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    pt.mcell[p] = pt.cell[p]; pt.mfx[p] = pt.fx[p]; pt.mfy[p] = pt.fy[p]; pt.mfz[p] = pt.fz[p];
  }
}

// Zigzag deposit (src/fdtd.cpp:38-185) in cell-relative FP32 coordinates: both endpoints are
// expressed relative to the lower of their two cells along each axis, so the relay point and
// the half-segment midpoints keep full FP32 resolution at any mesh size.
struct DepositF32 {
  int N0, N1, N2;
  float dx, dy, dz;
};

__device__ __forceinline__ void deposit_half_f32(float* J, long long cs, long long m, long long sI, long long sK,
                                                 float qh, float ax, float ay, float az, float jx, float jy, float jz) {
  const float x1 = 1.0f - ax, x2 = ax, y1 = 1.0f - ay, y2 = ay, z1 = 1.0f - az, z2 = az;
  const long long nd[8] = {m, m + sI, m + 1, m + sI + 1, m + sK, m + sK + sI, m + sK + 1, m + sK + sI + 1};
  const float wx[8] = {y1 * z1, y1 * z1, y2 * z1, y2 * z1, y1 * z2, y1 * z2, y2 * z2, y2 * z2};
  const float wy[8] = {x1 * z1, x2 * z1, x1 * z1, x2 * z1, x1 * z2, x2 * z2, x1 * z2, x2 * z2};
  const float wz[8] = {x1 * y1, x2 * y1, x1 * y2, x2 * y2, x1 * y1, x2 * y1, x1 * y2, x2 * y2};
  const float qx = qh * jx, qy = qh * jy, qz = qh * jz;
#pragma unroll
  for (int q = 0; q < 8; q++) {
    atomicAdd(J + nd[q], wx[q] * qx);
    atomicAdd(J + cs + nd[q], wy[q] * qy);
    atomicAdd(J + 2 * cs + nd[q], wz[q] * qz);
  }
}

__device__ __forceinline__ bool inside_f32(const DepositF32& D, int i, int j, int k, float fx, float fy) {
  return (i >= 1 && i <= D.N0 - 3 && (i > 1 || fx > 0.0f)) && (j >= 1 && j <= D.N1 - 3 && (j > 1 || fy > 0.0f)) &&
         (k >= 0 && k <= D.N2 - 2);
}

// Relay point along one axis: returns the relay coordinate relative to `base` (the lower cell).
__device__ __forceinline__ float relay_axis(int cm, int cp, float fm, float fp, int* base, float* rm, float* rp) {
  const int b = min(cm, cp);
  *base = b;
  *rm = (float)(cm - b) + fm;
  *rp = (float)(cp - b) + fp;
  const float lo = (float)(max(cm, cp) - b), hi = 1.0f;
  return fminf(hi, fmaxf(lo, 0.5f * (*rm + *rp)));
}

// Records (11 doubles) <-> mixed-form particles.  Cell = floor((x - xmin)/dx) in FP64.
struct CellMap {
  double xmin, ymin, zmin, dx, dy, dz;
};

__global__ void k_records_to_f32(const double* __restrict__ rec, long long n, ParticlesF32 pt, CellMap M) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const double* r = rec + 11 * p;
    auto split = [](double v, int& c, float& f) {
      const double fl = floor(v);
      c = (int)fl;
      f = (float)(v - fl);
      if (f >= 1.0f) { f = 0.0f; c += 1; }
    };
    int i, j, k;
    float fx, fy, fz;
    split((r[1] - M.xmin) / M.dx, i, fx);
    split((r[2] - M.ymin) / M.dy, j, fy);
    split((r[3] - M.zmin) / M.dz, k, fz);
    pt.cell[p] = pack_cell(i, j, k);
    pt.fx[p] = fx; pt.fy[p] = fy; pt.fz[p] = fz;
    split((r[4] - M.xmin) / M.dx, i, fx);
    split((r[5] - M.ymin) / M.dy, j, fy);
    split((r[6] - M.zmin) / M.dz, k, fz);
    pt.mcell[p] = pack_cell(i, j, k);
    pt.mfx[p] = fx; pt.mfy[p] = fy; pt.mfz[p] = fz;
    pt.gx[p] = (float)r[7]; pt.gy[p] = (float)r[8]; pt.gz[p] = (float)r[9];
    pt.q[p] = (float)r[0];
    pt.e[p] = r[10] == 1.0 ? 1 : 0;
    pt.status[p] = 0;
    pt.cross[p] = 0;
    pt.id[p] = (int)p;
  }
}

}  // namespace mithra
