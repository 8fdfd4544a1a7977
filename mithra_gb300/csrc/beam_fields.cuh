// Analytic laser fields on the device, in FP64 in both forms: the seed that the total-field /
// scattered-field planes inject into A (Seed::fields, src/classes.cpp:740-855, injected by
// src/fdtd.cpp:307-373), and the laser beams that act directly on the particles, as external
// fields (Solver::externalField, src/solver.cpp:1886-1947) or as optical undulators
// (src/solver.cpp:1825-1878), with the eight beam shapes of src/beam.cc:80-496.
//
// Differences from the reference, where its behaviour is not defined or depends on call order:
//  * A super-Gaussian seed sums its elements into a fresh vector at every node; the reference
//    keeps adding into the vector of the previous call.
//  * Standing beams inside an optical undulator use tlm = t0 + z/c0, as external fields do;
//    the reference leaves tlm unset on that path.
//  * The standing super-Gaussian beam uses the beam's wavelength l_ where the reference reads an
//    unset ubp.l (src/beam.cc:466).
#pragma once
#include "device_common.cuh"

namespace mithra {

// Rounded products and sums that the compiler may not fuse into FMAs.  The carrier phase
// 2 pi f0 (t - t0) of a laser reaches 1e5 rad or more, so the retarded time that feeds it is
// formed with the reference's roundings, operation by operation.
__host__ __device__ inline double mul_rn(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
__host__ __device__ inline double add_rn(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
__host__ __device__ inline double dot3_rn(const double* a, const double* b) {
  return add_rn(add_rn(mul_rn(a[0], b[0]), mul_rn(a[1], b[1])), mul_rn(a[2], b[2]));
}

// Signal::self, src/classes.cpp:533-576.
__host__ __device__ inline double signal_self(const SignalDev& g, double t, double phase) {
  const double u = t - g.t0;
  if (fabs(u) > 10.0 * g.s) return 0.0;
  const double carrier = cos(add_rn(add_rn(mul_rn(mul_rn(2.0 * kPI, g.f0), u), g.cep), phase));
  switch (g.type) {
    case 0: return -carrier * 2.7724 * u / (g.s * g.s) * exp(-1.3863 * u * u / (g.s * g.s));
    case 1: { const double w = u / g.s; return carrier * exp(-1.3863 * (w * w)); }
    case 2: return carrier / cosh(u / g.s);
    case 3:
    case 4: {
      double env = 1.0;
      if (g.type == 4) {
        const double w0 = u / g.g0, w1 = u / g.g1;
        env = sqrt(sqrt((1.0 + w0 * w0) * (1.0 + w1 * w1)));
      }
      if (u <= -g.s / 2.0) { const double w = (u + g.s / 2.0) * g.f0 / g.nR; return carrier * env * exp(-(w * w)); }
      if (u <= g.s / 2.0) return carrier * env;
      const double w = (u - g.s / 2.0) * g.f0 / g.nR;
      return carrier * env * exp(-(w * w));
    }
  }
  return 0.0;
}

__host__ __device__ inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// Seed::fields at the bunch-frame point r and field time `time`, into a (overwritten).
__host__ __device__ inline void seed_fields(const SeedDev& S, const double r[3], double time, double a[3]) {
  const BeamDev& b = S.b;
  const double rl2 = mul_rn(S.gamma, add_rn(r[2], mul_rn(mul_rn(S.beta, S.c0), add_rn(time, S.dt))));
  double tl = mul_rn(S.gamma, add_rn(add_rn(time, S.dt), mul_rn(S.beta / S.c0, r[2])));
  const double rv[3] = {r[0] - b.pos[0], r[1] - b.pos[1], rl2 - b.pos[2]};
  const double z = dot3_rn(rv, b.dir);
  tl -= z / S.c0;
  a[0] = a[1] = a[2] = 0.0;
  if (b.type == 0 || b.type == 1) {
    const double ts = signal_self(b.sig, tl, 0.0);
    if (fabs(ts) < 1.0e-6) return;
    if (b.type == 1) {
      const double x = dot3(rv, b.pol), y = dot3(rv, b.yv);
      if (fabs(x) > b.r0 || fabs(y) > b.r1) return;
    }
    for (int c = 0; c < 3; c++) a[c] = b.amplitude * ts * b.pol[c];
  } else if (b.type == 2 || b.type == 3) {
    if (fabs(signal_self(b.sig, tl, 0.0)) < 1.0e-6) return;
    const double x = dot3(rv, b.pol), y = dot3(rv, b.yv);
    const double wrp = sqrt(1.0 + z * z / (S.zRp * S.zRp));
    const double wrs = sqrt(1.0 + z * z / (S.zRs * S.zRs));
    const double xp = x / (S.zRp * wrp), ys = y / (S.zRs * wrs);
    const double p = 0.5 * (atan(z / S.zRp) + atan(z / S.zRs) - kPI) - kPI * z / S.l * (xp * xp + ys * ys);
    const double ts = signal_self(b.sig, tl, p);
    const double gx = x / (b.r0 * wrp), gy = y / (b.r1 * wrs);
    const double t = exp(-(gx * gx) - (gy * gy)) / sqrt(wrs * wrp) * b.amplitude;
    // The super-Gaussian elements of Seed::fields do not depend on the element index.
    const double n = (b.type == 2) ? 1.0 : (double)((2 * b.o0 + 1) * (2 * b.o1 + 1));
    for (int c = 0; c < 3; c++) a[c] = n * (t * ts * b.pol[c]);
  }
  a[2] *= S.gamma;
}

// TF/SF planes of FdTd::fieldUpdate for a domain that owns both z ends (src/fdtd.cpp:307-373,
// KI = 2, KF = np - 2).  One launch per direction, in the reference's order (x, y, z), so that
// nodes shared by two families of planes receive the additions in the same order.
//   dir 0: items (j, k), j in [2, N1-3], k in [2, N2-3]: nodes i = 1, 2, N0-2, N0-3
//   dir 1: items (i, k), i in [2, N0-3]:                 nodes j = 1, 2, N1-2, N1-3
//   dir 2: items (i, j), i, j in the interior ranges:    nodes k = 1, 2, N2-2, N2-3
template <typename T>
__global__ void __launch_bounds__(256) k_seed_inject(GridDev g, SeedDev S, T* __restrict__ anp1, const StateDev* st,
                                                     int dir) {
  const double time = st->time;
  const int na = (dir == 0) ? g.N1 - 4 : g.N0 - 4;
  const int nb = (dir == 2) ? g.N1 - 4 : g.N2 - 4;
  const long long items = (long long)na * nb;
  const double coef = (dir == 0) ? S.a1 : (dir == 1) ? S.a2 : S.a3;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < items; t += (long long)gridDim.x * blockDim.x) {
    const int ia = 2 + (int)(t % na), ib = 2 + (int)(t / na);
    // (target node index along the normal, neighbour offset to the sampled point, sign)
    const int nn = (dir == 0) ? g.N0 : (dir == 1) ? g.N1 : g.N2;
    const int tgt[4] = {1, 2, nn - 2, nn - 3};
    const int off[4] = {+1, -1, -1, +1};
    const double sgn[4] = {-1.0, 1.0, -1.0, 1.0};
#pragma unroll
    for (int q = 0; q < 4; q++) {
      int i, j, k;
      if (dir == 0) { i = tgt[q]; j = ia; k = ib; }
      else if (dir == 1) { i = ia; j = tgt[q]; k = ib; }
      else { i = ia; j = ib; k = tgt[q]; }
      // Solver::rc, src/solver.cpp:2302-2315, at the neighbour along the normal.
      const int is = (dir == 0) ? i + off[q] : i, js = (dir == 1) ? j + off[q] : j, ks = (dir == 2) ? k + off[q] : k;
      const double r[3] = {add_rn(g.xmin, mul_rn((double)is, g.dx)), add_rn(g.ymin, mul_rn((double)js, g.dy)),
                           add_rn(g.zmin, mul_rn((double)ks, g.dz))};
      double a[3];
      seed_fields(S, r, time, a);
      const long long m = node_index(g, k, i, j);
#pragma unroll
      for (int c = 0; c < 3; c++) {
        T* p = anp1 + c * g.cstride + m;
        *p = (T)((double)*p + sgn[q] * (coef * a[c]));
      }
    }
  }
}

// One beam of src/beam.cc:80-496 at the lab-frame offset rv from the beam's reference point,
// distance z along its direction, and retarded times tl = t0 - z/c0, tlm = t0 + z/c0.
__host__ __device__ inline void beam_fields(const BeamDev& s, double c0, const double rv[3], double z, double tl, double tlm,
                                   double eT[3], double bT[3]) {
  for (int c = 0; c < 3; c++) eT[c] = bT[c] = 0.0;
  const int type = s.type;
  const bool standing = type >= 4;
  if (type == 0 || type == 1 || type == 4 || type == 5) {
    if (type == 1 || type == 5) {
      const double xr = dot3(rv, s.pol) / s.r0, yr = dot3(rv, s.yv) / s.r1;
      if (xr * xr + yr * yr > 1.0) return;
    }
    double fe, fb;
    const double ts = signal_self(s.sig, tl, 0.0);
    if (!standing) {
      if (fabs(ts) < 1.0e-6) return;
      fe = fb = ts;
    } else {
      const double tsm = signal_self(s.sig, tlm, 0.0);
      fe = ts - tsm;
      fb = ts + tsm;
      if (fabs(fe) < 1.0e-6 && fabs(fb) < 1.0e-6) return;
    }
    for (int c = 0; c < 3; c++) {
      eT[c] = s.amplitude * fe * s.pol[c];
      bT[c] = s.amplitude * fb / c0 * s.yv[c];
    }
    return;
  }
  const double x = dot3(rv, s.pol), y = dot3(rv, s.yv);
  const double wrp = sqrt(1.0 + z * z / (s.zR0 * s.zR0));
  const double wrs = sqrt(1.0 + z * z / (s.zR1 * s.zR1));
  const bool super = (type == 3 || type == 7);
  if (!super) {
    if (fabs(x / wrp) > 4.0 * s.r0 || fabs(y / wrs) > 4.0 * s.r1) return;
  } else if ((fabs(x) - s.o0 * s.r0) > 4.0 * s.r0 * wrp || (fabs(y) - s.o1 * s.r1) > 4.0 * s.r1 * wrs) {
    return;
  }
  {
    const double ts = signal_self(s.sig, tl, 0.0);
    if (!standing) {
      if (fabs(ts) < 1.0e-6) return;
    } else {
      const double tsm = signal_self(s.sig, tlm, 0.0);
      if (fabs(ts - tsm) < 1.0e-6 && fabs(ts + tsm) < 1.0e-6) return;
    }
  }
  const double atanP = atan(z / s.zR0), atanS = atan(z / s.zR1);
  const double amp = super ? s.amplitude / sqrt(wrs * wrp) : 0.0;
  const int ni = super ? s.o0 : 0, nj = super ? s.o1 : 0;
  for (int i = -ni; i <= ni; i++)
    for (int j = -nj; j <= nj; j++) {
      const double x0 = (x - i * s.r0) / wrp, y0 = (y - j * s.r1) / wrs;
      if (super && (fabs(x0) > 4.0 * s.r0 || fabs(y0) > 4.0 * s.r1)) continue;
      // the super-Gaussian phase uses the untransformed y (src/beam.cc:266, :466)
      const double yq = super ? y / s.zR1 : y0 / s.zR1, xq = x0 / s.zR0;
      const double p0 = 0.5 * (atanP + atanS) - kPI * z / s.l * (xq * xq + yq * yq);
      const double gx = x0 / s.r0, gy = y0 / s.r1;
      const double t = super ? amp * exp(-(gx * gx) - (gy * gy)) : exp(-(gx * gx) - (gy * gy)) / sqrt(wrs * wrp) * s.amplitude;
      double e1, b1, e2, b2;  // carriers of (ex, by) and of ez, bz
      const double pa = p0 - kPI / 2.0, pb = p0 + atanP, pc = p0 + atanS;
      const double ta = signal_self(s.sig, tl, pa), tb = signal_self(s.sig, tl, pb), tc = signal_self(s.sig, tl, pc);
      if (!standing) {
        e1 = ta; b1 = ta; e2 = tb; b2 = tc;
      } else {
        const double ma = signal_self(s.sig, tlm, pa), mb = signal_self(s.sig, tlm, -pb), mc = signal_self(s.sig, tlm, -pc);
        e1 = ta - ma; b1 = ta + ma; e2 = tb - mb; b2 = tc - mc;
      }
      const double cex = t * e1, cby = t * b1 / c0;
      const double cez = t * (-x0 / s.zR0) * e2, cbz = t * (-y0 / s.zR1) * b2 / c0;
      for (int c = 0; c < 3; c++) {
        eT[c] += cex * s.pol[c] + cez * s.dir[c];
        bT[c] += cby * s.yv[c] + cbz * s.dir[c];
      }
    }
}

// One laser beam seen by a particle at bunch-frame r, boosted into the bunch frame and added to
// bt / et (src/solver.cpp:1825-1877, :1886-1944).
__host__ __device__ inline void beam_add(const BeamDev& s, const PushDev& P, double timeBunch, double x, double y, double z,
                                double* bt, double* et) {
  const double rl2 = mul_rn(P.gamma, add_rn(z, mul_rn(mul_rn(P.beta, P.c0), add_rn(timeBunch, P.dt_shift))));
  const double t0 = mul_rn(P.gamma, add_rn(add_rn(timeBunch, P.dt_shift), mul_rn(P.beta / P.c0, z)));
  const double rv[3] = {x - s.pos[0], y - s.pos[1], rl2 - s.pos[2]};
  const double zz = dot3_rn(rv, s.dir);
  double eT[3], bT[3];
  beam_fields(s, P.c0, rv, zz, t0 - zz / P.c0, t0 + zz / P.c0, eT, bT);
  bt[0] += P.gamma * (bT[0] + P.beta / P.c0 * eT[1]);
  bt[1] += P.gamma * (bT[1] - P.beta / P.c0 * eT[0]);
  bt[2] += bT[2];
  et[0] += P.gamma * (eT[0] - P.beta * P.c0 * bT[1]);
  et[1] += P.gamma * (eT[1] + P.beta * P.c0 * bT[0]);
  et[2] += eT[2];
}

// Every laser beam acting on a particle: the optical undulator modules in module order, then the
// external fields.
__device__ __forceinline__ void laser_beams_add(const PushDev& P, const UndDev* __restrict__ und, int n_und,
                                             double timeBunch, double x, double y, double z, double* bt, double* et) {
  for (int u = 0; u < n_und; u++)
    if (und[u].type == 1 && und[u].beam >= 0) beam_add(P.beams[und[u].beam], P, timeBunch, x, y, z, bt, et);
  for (int xf = 0; xf < P.n_ext; xf++) beam_add(P.beams[P.ext0 + xf], P, timeBunch, x, y, z, bt, et);
}

}  // namespace mithra
