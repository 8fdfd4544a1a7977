// Particle kernels of the FP64 form: the bunch push (gather + Boris + drift with the analytic
// static-undulator field), the single-domain z-face exchange, particle erasure and the
// zigzag current deposit.
#pragma once
#include "beam_fields.cuh"
#include "device_common.cuh"

namespace mithra {

// Undulator lz and phase for the FP64 push on kUndSub sub-planes per cell: lz = gamma (zmin +
// (k + s / kUndSub) dz + beta c0 (timeBunch + dt_)) - rb on sub-plane s of node plane k, with the
// sine and cosine of ku lz.  Entries per static module: (N2 + 1) * kUndSub.
__global__ void k_undulator_table64(const UndDev* __restrict__ und, int n_und, int N2, double zmin, double dz,
                                    double gamma, double bc, double dt_shift, const StateDev* st,
                                    UndPlane64* __restrict__ table) {
  const double tshift = bc * (st->time_bunch + dt_shift);
  const int per = (N2 + 1) * kUndSub;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n_und * per; t += gridDim.x * blockDim.x) {
    const int u = t / per, q = t % per;
    const double lz = gamma * (zmin + ((double)(q / kUndSub) + (double)(q % kUndSub) / kUndSub) * dz + tshift) - und[u].rb;
    double s, c;
    sincos(und[u].ku * lz, &s, &c);
    table[t] = UndPlane64{lz, s, c};
  }
}

// Largest phase advance across one cell (ku gamma dz) for which the push takes the undulator
// phase from the table: the advance within a sub-plane interval then stays below 1/4, where
// sin_cos_series_short holds.  The bench jobs advance 0.78 rad per boosted-frame cell.
constexpr double kUndTableMaxKgdz = 1.0;

// Solver::undulatorField for static modules (src/solver.cpp:1798-1824) and
// Solver::staticUndulator (src/beam.cc:14-76).  Adds the lab-frame undulator field, boosted
// into the bunch frame, to bt/et.  Optical modules are laser beams (laser_beams_add), added
// after the static ones.
// kz, fz: node plane below z and the offset above it in cells ((z - zmin)/dz = kz + fz).  On a
// plane of the table, with fz = (s + r) / kUndSub for sub-plane s, lz = lz_ks + gamma dz r /
// kUndSub and sin, cos of ku lz come from the sub-plane's values and the series of the phase
// advance d = ku gamma dz r / kUndSub (|d| < 1/4) by the angle-sum formulas: about 22 FP64
// operations instead of a sincos with its range reduction.
__device__ __forceinline__ void static_undulator_field(const UndDev* __restrict__ und, int n_und,
                                                       const PushDev& P, double timeBunch,
                                                       double x, double y, double z, int N2, int kz, double fz,
                                                       double* bt, double* et) {
  const bool tab = P.und_planes != nullptr && kz >= 0 && kz <= N2;
  for (int u = 0; u < n_und; u++) {
    const UndDev& U = und[u];
    if (U.type != 0) continue;  // optical modules: laser_beams_add
    double lz, sn = 0.0, cs = 0.0;
    if (tab) {
      const double f4 = fz * kUndSub;        // exact
      const int sub = ifloor_d(f4);           // 0 .. kUndSub - 1
      const double r = f4 - double_of_int(sub);  // exact
      const UndPlane64 te = P.und_planes[(u * (N2 + 1) + kz) * kUndSub + sub];
      lz = fma(P.gdz_sub, r, te.lz);
      double sd, cd;
      sin_cos_series_short(U.kgdz_sub * r, &sd, &cd);
      sn = te.s * cd + te.c * sd;
      cs = te.c * cd - te.s * sd;
    } else {
      lz = P.gamma * (z + P.beta * P.c0 * (timeBunch + P.dt_shift)) - U.rb;
    }
    const double ly = x * U.ct + y * U.st;
    double s_ly, c_ly;
    {
      // cosh and sinh: Taylor series for |ku ly| < 0.1 (truncation below 1e-19 relative; the FP64
      // pipe is the bound of this kernel), else from one exponential.
      const double kl = U.ku * ly;
      if ((long long)(bits_of(kl) & 0x7fffffffffffffffULL) < 0x3fb999999999999aLL) {  // |kl| < 0.1
        const double a2 = kl * kl;
        s_ly = kl * (1.0 + a2 * (1.0 / 6.0) * (1.0 + a2 * (1.0 / 20.0) * (1.0 + a2 * (1.0 / 42.0) * (1.0 + a2 * (1.0 / 72.0)))));
        c_ly = 1.0 + a2 * 0.5 * (1.0 + a2 * (1.0 / 12.0) * (1.0 + a2 * (1.0 / 30.0) * (1.0 + a2 * (1.0 / 56.0) * (1.0 + a2 * (1.0 / 90.0)))));
      } else {
        const double ex = exp(kl), iex = 1.0 / ex;
        c_ly = 0.5 * (ex + iex);
        s_ly = 0.5 * (ex - iex);
      }
    }
    double d1, bz;
    const long long klz = dkey(lz);
    if (klz >= 0 && klz <= dkey(U.ul)) {  // 0 <= lz <= ul
      if (!tab) sincos(U.ku * lz, &sn, &cs);
      d1 = U.b0 * c_ly * sn * P.gamma;
      bz = U.b0 * s_ly * cs;
    } else {
      double t0 = (lz < 0.0) ? lz : lz - U.ul;
      const double kt = U.ku * t0;
      double sz = exp(-(kt * kt) / 2.0);
      const bool has = (lz < 0.0) ? U.has_prev : U.has_next;
      if (has) {
        const double r0 = (lz < 0.0) ? U.r0_prev : U.r0_next;
        const bool cut = (lz < 0.0) ? (lz < r0 || r0 == 0.0) : (t0 > r0 || r0 == 0.0);
        if (cut) sz = 0.0;
        else
          sz *= 0.35875 + 0.48829 * cos(kPI * t0 / r0) + 0.14128 * cos(2.0 * kPI * t0 / r0) +
                0.01168 * cos(3.0 * kPI * t0 / r0);
      }
      d1 = U.b0 * c_ly * sz * U.ku * t0 * P.gamma;
      bz = U.b0 * s_ly * sz;
    }
    bt[0] += d1 * U.ct;
    bt[1] += d1 * U.st;
    bt[2] += bz;
    d1 *= P.c0 * P.beta;
    et[1] += d1 * U.ct;
    et[0] += -d1 * U.st;
  }
}

// One Solver::bunchUpdate for every particle (src/solver.cpp:1424-1549).
// save_rnm: also perform `rnm = rnp` first (src/solver.cpp:1311-1312).
// BEAMS: the job defines optical undulators or external fields (see k_push_f32).
template <bool BEAMS>
__global__ void __launch_bounds__(256) k_push_fp64(GridDev g, PushDev P, const UndDev* __restrict__ und,
                                                   ParticlesDev<double> pt, const double* __restrict__ E,
                                                   const double* __restrict__ B, StateDev* st, int save_rnm) {
  const long long n = st->n_particles;
  const double timeBunch = st->time_bunch;
  const long long cs = g.cstride;
  unsigned long long local_cross = 0, local_nt = 0;
  // Comparisons, modf and the index conversions on the integer pipes (see k_deposit_fp64).
  const long long kxh = dkey(g.xmax - g.dx), kxl = dkey(g.xmin + g.dx), kyh = dkey(g.ymax - g.dy),
                  kyl = dkey(g.ymin + g.dy), kzh = dkey(g.zp1), kzl = dkey(g.zp0), kLz = dkey(g.Lz);
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    int8_t cross = 0;
    if (!(pt.status[p] & 1)) {
      double x = pt.x[p], y = pt.y[p], z = pt.z[p];
      if (save_rnm) { pt.mx[p] = x; pt.my[p] = y; pt.mz[p] = z; }
      const double za = z - g.zmin;
      const long long kza = dkey(za);
      double zr = ((kza >= 0 && kza < kLz) ? za : pmod_d(za, g.Lz)) + g.zmin;  // pmod_d's own fast path
      const long long kzr = dkey(zr);
      if (kzr >= kzl && kzr < kzh) {
        const long long kx = dkey(x), ky = dkey(y), kz = dkey(z);
        const bool b1x = (kx < kxh && kx > kxl);
        const bool b1y = (ky < kyh && ky > kyl);
        const bool b1z = (kz < kzh && kz >= kzl);
        // z in cells, split as the gather's modf does: plane k and offset dzr
        double kd;
        const double dzr = modf_d(za * g.rdz, &kd);
        const int k = itrunc_d(kd);
        double bt[3] = {0.0, 0.0, 0.0}, et[3] = {0.0, 0.0, 0.0};
        static_undulator_field(und, P.n_und, P, timeBunch, x, y, z, g.N2, (kza >= 0) ? k : -1, dzr, bt, et);
        if (BEAMS) laser_beams_add(P, und, P.n_und, timeBunch, x, y, z, bt, et);
        double e = pt.e[p];
        if (__double_as_longlong(e) == 0x3ff0000000000000LL) {  // e == 1.0
          if (b1x && b1y && b1z) {
            double d1;
            const double dxr = modf_d((x - g.xmin) * g.rdx, &d1); const int i = itrunc_d(d1);
            const double dyr = modf_d((y - g.ymin) * g.rdy, &d1); const int j = itrunc_d(d1);
            const long long m = node_index(g, k, i, j);
            const long long sI = g.P1, sK = g.plane;
            const double wx0 = 1.0 - dxr, wy0 = 1.0 - dyr, wz0 = 1.0 - dzr;
            const double w[8] = {wx0 * wy0 * wz0, dxr * wy0 * wz0, wx0 * dyr * wz0, dxr * dyr * wz0,
                                 wx0 * wy0 * dzr, dxr * wy0 * dzr, wx0 * dyr * dzr, dxr * dyr * dzr};
            const long long nd[8] = {m, m + sI, m + 1, m + sI + 1, m + sK, m + sK + sI, m + sK + 1, m + sK + sI + 1};
#pragma unroll
            for (int c = 0; c < 3; c++) {
              double se = et[c], sb = bt[c];
#pragma unroll
              for (int q = 0; q < 8; q++) {
                se += w[q] * __ldg(E + c * cs + nd[q]);
                sb += w[q] * __ldg(B + c * cs + nd[q]);
              }
              et[c] = se; bt[c] = sb;
            }
          } else if (!b1x && !b1y && b1z) {
            local_nt++;
          }
        } else if (P.n_und > 0) {
          const double lz = P.gamma * (z + P.beta * P.c0 * (timeBunch + P.dt_shift));
          e = (lz > -P.und0_dist) ? 1.0 : 0.0;
          pt.e[p] = e;
        } else {
          pt.e[p] = 1.0;
        }
        // Boris rotation, src/solver.cpp:1519-1535.
        double gx = pt.gx[p], gy = pt.gy[p], gz = pt.gz[p];
        const double mx = gx + P.r1 * et[0], my = gy + P.r1 * et[1], mz = gz + P.r1 * et[2];
        // d1 = sqrt(1 + |m|^2) and 1/d1 from one reciprocal square root (the reference divides
        // by the square root; the two differ by rounding)
        const double u1 = 1.0 + (mx * mx + my * my + mz * mz);
        const double rd1 = rsqrt(u1);
        const double d1 = u1 * rd1;
        const double f = P.r2 * rd1;
        const double px = f * (my * bt[2] - mz * bt[1]) + mx;
        const double py = f * (mz * bt[0] - mx * bt[2]) + my;
        const double pz = f * (mx * bt[1] - my * bt[0]) + mz;
        const double bt2 = bt[0] * bt[0] + bt[1] * bt[1] + bt[2] * bt[2];
        const double s = 2.0 * rcp_nr(d1 * P.inv_r2 + f * bt2);
        gx = s * (py * bt[2] - pz * bt[1]) + mx + P.r1 * et[0];
        gy = s * (pz * bt[0] - px * bt[2]) + my + P.r1 * et[1];
        gz = s * (px * bt[1] - py * bt[0]) + mz + P.r1 * et[2];
        pt.gx[p] = gx; pt.gy[p] = gy; pt.gz[p] = gz;
        // Drift, src/solver.cpp:1538-1541.
        const double gg = P.dtb * rsqrt(1.0 + (gx * gx + gy * gy + gz * gz));
        const double drz = gg * gz;
        pt.x[p] = x + gg * gx; pt.y[p] = y + gg * gy; pt.z[p] = z + drz;
        zr += drz;
        const long long kzn = dkey(zr);
        if (!is_nan_bits(zr)) {  // a NaN position crosses no face (its FP64 comparisons are false)
          if (kzn < kzl) cross = 1;
          else if (kzn >= kzh) cross = 2;
        }
      }
    }
    pt.cross[p] = cross;
    local_cross += (cross != 0);
  }
  // Block-aggregated counters.
  for (int o = 16; o > 0; o >>= 1) {
    local_cross += __shfl_down_sync(0xffffffffu, local_cross, o);
    local_nt += __shfl_down_sync(0xffffffffu, local_nt, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (local_cross) atomicAdd(&st->n_cross, local_cross);
    if (local_nt) atomicAdd(&st->n_transverse, local_nt);
  }
}

// After each push: the single-rank self-exchange of src/solver.cpp:1551-1568 appends a copy of
// every particle that crossed below zp0 (first) and then of every one that crossed at or above
// zp1, each group in particle order; then timeBunch_ += dt_b, ++nTimeBunch_ (src/solver.cpp:1319).
// One block; the ordered append runs only when a crossing happened.
template <typename T>
__global__ void __launch_bounds__(1024) k_substep_end(ParticlesDev<T> pt, StateDev* st, double bunch_time_step) {
  __shared__ long long s_base;
  __shared__ int s_warp[32];
  const unsigned long long ncross = st->n_cross;
  if (ncross) {
    const long long n = st->n_particles;
    if (threadIdx.x == 0) s_base = n;
    __syncthreads();
    if ((long long)(n + ncross) > st->capacity) {
      if (threadIdx.x == 0) st->overflow = 1;
    } else {
      for (int pass = 1; pass <= 2; pass++) {
        for (long long c0 = 0; c0 < n; c0 += blockDim.x) {
          const long long p = c0 + threadIdx.x;
          const int take = (p < n) && (pt.cross[p] == pass);
          const unsigned bal = __ballot_sync(0xffffffffu, take);
          const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
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
            pt.x[d] = pt.x[p]; pt.y[d] = pt.y[p]; pt.z[d] = pt.z[p];
            pt.gx[d] = pt.gx[p]; pt.gy[d] = pt.gy[p]; pt.gz[d] = pt.gz[p];
            pt.mx[d] = pt.mx[p]; pt.my[d] = pt.my[p]; pt.mz[d] = pt.mz[p];
            pt.q[d] = pt.q[p]; pt.e[d] = pt.e[p];
            pt.status[d] = pt.status[p]; pt.cross[d] = 0;
          }
          __syncthreads();
          if (threadIdx.x == 0) s_base += total;
          __syncthreads();
        }
      }
      if (threadIdx.x == 0) st->n_particles = s_base;
    }
  }
  if (threadIdx.x == 0) {
    st->n_cross = 0;
    st->time_bunch += bunch_time_step;
    st->n_time_bunch += 1;
  }
}

// time_ += dt; ++nTime_ (src/solver.cpp:1396-1399).
// Also hands the particle slab accumulated by this step's deposit to the next step.
__global__ void k_advance_time(StateDev* st, double dt) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    st->time += dt;
    st->n_time += 1;
    if (st->k_lo_next <= st->k_hi_next) {
      st->k_lo = st->k_lo_next;
      st->k_hi = st->k_hi_next;
    }
    st->k_lo_next = 0x7fffffff;
    st->k_hi_next = -0x7fffffff;
  }
}

// Solver::recycleParticles / the erasure in FdTd::currentCommunicate (src/solver.cpp:493-503,
// src/fdtd.cpp:214-224): erase particles whose wrapped z lies outside [zp0, zp1).
// The comparisons run on the integer pipes (dkey): with the FP64 ones the pass was bound by the
// FP64 pipe, with them it is a read of z and the status byte.
template <typename T>
__global__ void __launch_bounds__(256) k_erase_outside(GridDev g, ParticlesDev<T> pt, StateDev* st) {
  const long long n = st->n_particles;
  const long long kLz = dkey(g.Lz), kz0 = dkey(g.zp0), kz1 = dkey(g.zp1);
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    if (pt.status[p] & 1) continue;
    const double za = (double)pt.z[p] - g.zmin;
    const long long ka = dkey(za);
    const double zr = ((ka >= 0 && ka < kLz) ? za : pmod_d(za, g.Lz)) + g.zmin;  // pmod_d's own fast path
    const long long kr = dkey(zr);
    if ((kr < kz0 || kr >= kz1) && !is_nan_bits(zr)) pt.status[p] |= 1;  // a NaN compares false
  }
}

// FdTd::currentUpdate, zigzag (Umeda) deposit (src/fdtd.cpp:38-185), FP64 atomics into J
// (the anp1 buffer, zeroed before).  With rho != nullptr also the charge deposit of
// src/fdtdSC.cpp:140-161.
// The same half segment in edge form.  The reference adds one value to both ends of a cell edge
// (Jx to nodes i and i+1 with weights of y and z only, src/fdtd.cpp:105-130, and likewise Jy, Jz),
// so each value is added once, to the edge's lower node, into Je; the node current is
// Je(node) + Je(node - unit step), formed where it is read.  12 atomics instead of 24.
__device__ __forceinline__ void deposit_half_edges(double* Je, long long cs, long long m, long long sI, long long sK,
                                                   double qh, double dxh, double dyh, double dzh, double jx,
                                                   double jy, double jz) {
  const double x1 = 1.0 - dxh, x2 = dxh, y1 = 1.0 - dyh, y2 = dyh, z1 = 1.0 - dzh, z2 = dzh;
  const double qx = qh * jx, qy = qh * jy, qz = qh * jz;
  // q j w_u w_v as (q j w_v) w_u: six FP64 multiplies per component instead of eight (the kernel
  // is bound by the FP64 pipe); the values differ from the reference's products by rounding only.
  const double ax = qx * z1, bx = qx * z2, ay = qy * z1, by = qy * z2, az = qz * y1, bz = qz * y2;
  atomicAdd(Je + m, ax * y1);
  atomicAdd(Je + m + 1, ax * y2);
  atomicAdd(Je + m + sK, bx * y1);
  atomicAdd(Je + m + 1 + sK, bx * y2);
  double* Jy = Je + cs;
  atomicAdd(Jy + m, ay * x1);
  atomicAdd(Jy + m + sI, ay * x2);
  atomicAdd(Jy + m + sK, by * x1);
  atomicAdd(Jy + m + sI + sK, by * x2);
  double* Jz = Je + 2 * cs;
  atomicAdd(Jz + m, az * x1);
  atomicAdd(Jz + m + sI, az * x2);
  atomicAdd(Jz + m + 1, bz * x1);
  atomicAdd(Jz + m + sI + 1, bz * x2);
}

// J: the edge-form current buffer (zeroed by the caller); rho: node charge, or null.
__global__ void __launch_bounds__(256) k_deposit_fp64(GridDev g, ParticlesDev<double> pt, StateDev* st,
                                                      double* J, double* rho) {
  const long long n = st->n_particles;
  const long long cs = g.cstride, sI = g.P1, sK = g.plane;
  if (blockIdx.x == 0 && threadIdx.x == 0) st->j_edges = 1;  // J is written in edge form
  int kmin = 0x7fffffff, kmax = -0x7fffffff;
  // The kernel is bound by GB300's FP64 issue rate: comparisons, floors, conversions, min/max and
  // modf's truncation run on the integer pipes (dkey, ifloor_d, double_of_int, dmin_k, modf_d),
  // with the same results as the FP64 instructions.
  const long long kxh = dkey(g.xmax - g.dx), kxl = dkey(g.xmin + g.dx), kyh = dkey(g.ymax - g.dy),
                  kyl = dkey(g.ymin + g.dy), kzh = dkey(g.zp1), kzl = dkey(g.zp0);
  auto inside = [&](double a, double b, double c) {
    const long long ka = dkey(a), kb = dkey(b), kc = dkey(c);
    return ka < kxh && ka > kxl && kb < kyh && kb > kyl && kc < kzh && kc >= kzl;
  };
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    if (pt.status[p] & 1) continue;
    const double rp0 = pt.x[p], rp1 = pt.y[p], rp2 = pt.z[p];
    const double tzp = (rp2 - g.zmin) * g.rdz;  // positions in cells from here on
    const int kp = ifloor_d(tzp);
    kmin = min(kmin, kp);
    kmax = max(kmax, kp);
    const double rm0 = pt.mx[p], rm1 = pt.my[p], rm2 = pt.mz[p];
    const bool bp = inside(rp0, rp1, rp2);
    const bool bm = inside(rm0, rm1, rm2);
    if (!(bp || bm)) continue;
    const double qh = pt.q[p] * 0.5;
    const double txp = (rp0 - g.xmin) * g.rdx, typ = (rp1 - g.ymin) * g.rdy;
    const double txm = (rm0 - g.xmin) * g.rdx, tym = (rm1 - g.ymin) * g.rdy, tzm = (rm2 - g.zmin) * g.rdz;
    const int ip = ifloor_d(txp), jp = ifloor_d(typ);
    const int im = ifloor_d(txm), jm = ifloor_d(tym), km = ifloor_d(tzm);
    // The relay point of the zigzag scheme in cells: the midpoint clamped to [origin of the upper
    // cell, origin of the lower cell + 1] (src/fdtd.cpp:80-85 in length units; the half segments'
    // midpoints and currents follow from it with fewer FP64 operations in cell units).
    const double u0 = dmin_k(double_of_int(min(im, ip)) + 1.0, dmax_k(double_of_int(max(im, ip)), 0.5 * (txm + txp)));
    const double u1 = dmin_k(double_of_int(min(jm, jp)) + 1.0, dmax_k(double_of_int(max(jm, jp)), 0.5 * (tym + typ)));
    const double u2 = dmin_k(double_of_int(min(km, kp)) + 1.0, dmax_k(double_of_int(max(km, kp)), 0.5 * (tzm + tzp)));
    double c;
    if (bp) {
      const long long m = node_index(g, kp, ip, jp);
      const double dxp = modf_d(0.5 * (txp + u0), &c);
      const double dyp = modf_d(0.5 * (typ + u1), &c);
      const double dzp = modf_d(0.5 * (tzp + u2), &c);
      deposit_half_edges(J, cs, m, sI, sK, qh, dxp, dyp, dzp, (txp - u0) * g.dx, (typ - u1) * g.dy, (tzp - u2) * g.dz);
      if (rho) {
        const double fx = modf_d(txp, &c), fy = modf_d(typ, &c), fz = modf_d(tzp, &c);
        const double q = pt.q[p];
        const double x1 = 1.0 - fx, y1 = 1.0 - fy, z1 = 1.0 - fz;
        atomicAdd(rho + m, q * x1 * y1 * z1);
        atomicAdd(rho + m + sI, q * fx * y1 * z1);
        atomicAdd(rho + m + 1, q * x1 * fy * z1);
        atomicAdd(rho + m + sI + 1, q * fx * fy * z1);
        atomicAdd(rho + m + sK, q * x1 * y1 * fz);
        atomicAdd(rho + m + sK + sI, q * fx * y1 * fz);
        atomicAdd(rho + m + sK + 1, q * x1 * fy * fz);
        atomicAdd(rho + m + sK + sI + 1, q * fx * fy * fz);
      }
    }
    if (bm) {
      const long long m = node_index(g, km, im, jm);
      const double dxm = modf_d(0.5 * (txm + u0), &c);
      const double dym = modf_d(0.5 * (tym + u1), &c);
      const double dzm = modf_d(0.5 * (tzm + u2), &c);
      deposit_half_edges(J, cs, m, sI, sK, qh, dxm, dym, dzm, (u0 - txm) * g.dx, (u1 - tym) * g.dy, (u2 - tzm) * g.dz);
    }
  }
  slab_update(st, kmin, kmax);
}

// rnm = rnp (src/solver.cpp:1311-1312) as a stand-alone stage.
template <typename T>
__global__ void k_save_positions(ParticlesDev<T> pt, const StateDev* st) {
  const long long n = st->n_particles;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    pt.mx[p] = pt.x[p]; pt.my[p] = pt.y[p]; pt.mz[p] = pt.z[p];
  }
}

// Particle records (11 doubles) <-> device SoA.
__global__ void k_records_to_soa(const double* __restrict__ rec, long long n, ParticlesDev<double> pt) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const double* r = rec + 11 * p;
    pt.q[p] = r[0];
    pt.x[p] = r[1]; pt.y[p] = r[2]; pt.z[p] = r[3];
    pt.mx[p] = r[4]; pt.my[p] = r[5]; pt.mz[p] = r[6];
    pt.gx[p] = r[7]; pt.gy[p] = r[8]; pt.gz[p] = r[9];
    pt.e[p] = r[10];
    pt.status[p] = 0; pt.cross[p] = 0;
  }
}

// Gathers the live particles in slot order (erased ones removed, as the reference's list
// erasure does) into 11-double records.  One block: slot order is preserved by a block scan.
__global__ void __launch_bounds__(1024) k_soa_to_records(ParticlesDev<double> pt, const StateDev* st,
                                                         double* rec, long long cap, long long* n_out) {
  __shared__ int s_warp[32];
  __shared__ long long s_base;
  const long long n = st->n_particles;
  if (threadIdx.x == 0) s_base = 0;
  __syncthreads();
  for (long long c0 = 0; c0 < n; c0 += blockDim.x) {
    const long long p = c0 + threadIdx.x;
    const int take = (p < n) && !(pt.status[p] & 1);
    const unsigned bal = __ballot_sync(0xffffffffu, take);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) s_warp[warp] = __popc(bal);
    __syncthreads();
    int before = 0, total = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
      if (w < warp) before += s_warp[w];
      total += s_warp[w];
    }
    before += __popc(bal & ((1u << lane) - 1u));
    const long long d = s_base + before;
    if (take && d < cap) {
      double* r = rec + 11 * d;
      r[0] = pt.q[p];
      r[1] = pt.x[p]; r[2] = pt.y[p]; r[3] = pt.z[p];
      r[4] = pt.mx[p]; r[5] = pt.my[p]; r[6] = pt.mz[p];
      r[7] = pt.gx[p]; r[8] = pt.gy[p]; r[9] = pt.gz[p];
      r[10] = pt.e[p];
    }
    __syncthreads();
    if (threadIdx.x == 0) s_base += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) *n_out = s_base;
}

}  // namespace mithra
