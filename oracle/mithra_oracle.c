/*
 * CPU restatement of the MITHRA FdTd time-marching loop (oracle).  TEST INFRASTRUCTURE ONLY:
 * loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs, never by the
 * product library.  See mithra_oracle.h for the layout and the reference lines restated.
 *
 * Build with -ffp-contract=off: every expression below keeps the reference's operation order,
 * so with one thread the results are bit-identical to the reference built the same way.
 * With more threads (bench CPU baseline) the field, E/B and push loops are split over z-planes
 * or particles, which changes nothing; only the deposit sums then land in a different order.
 */
#include "mithra_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Constants of src/stdinclude.h:43-52 (PI is the reference's truncated value). */
static const double MO_PI = 3.1415926535;

static int g_threads = 1;
void mo_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
int mo_get_threads(void) { return g_threads; }

/* ------------------------------------------------------------------------------------------ */
/* Field stencils.  `nc` is the number of components per node (3 for A, 1 for phi); the        */
/* component loop is the outer one in AdvanceField (src/database.cpp:44-134), but components   */
/* are independent, so each is written out separately.                                       */
/* ------------------------------------------------------------------------------------------ */

/* AdvanceField::advanceMagneticPotentialFD / advanceScalarPotentialFD, src/database.cpp:91-134.
 * src = coefficient a[4] (J) or a[5] (rho). */
static inline double fd_point(const double* a, double asrc, const double* an, const double* anm1,
                              const double* jsrc, long l, long sI, long sJ, long sK) {
  return a[0] * an[l] - anm1[l] +
         a[1] * (an[l + sI] + an[l - sI]) +
         a[2] * (an[l + sJ] + an[l - sJ]) +
         a[3] * (an[l + sK] + an[l - sK]) +
         asrc * jsrc[l];
}

/* AdvanceField::advanceMagneticPotentialNSFD / advanceScalarPotentialNSFD, src/database.cpp:44-88. */
static inline double nsfd_point(const double* a, double alpha, double beta, double asrc,
                                const double* an, const double* anm1, const double* jsrc, long l,
                                long sI, long sJ, long sK) {
  return a[0] * an[l] - anm1[l] + alpha * (
         a[1] * (an[l + sI] + an[l - sI] + beta * (an[l + sI + sK] + an[l + sI - sK] + an[l - sI + sK] + an[l - sI - sK])) +
         a[2] * (an[l + sJ] + an[l - sJ] + beta * (an[l + sJ + sK] + an[l + sJ - sK] + an[l - sJ + sK] + an[l - sJ - sK]))) +
         a[3] * (an[l + sK] + an[l - sK]) +
         asrc * jsrc[l];
}

/* AdvanceField::advanceBoundaryF/S, src/database.cpp:137-176, with the argument pattern of the
 * six face loops of src/fdtd.cpp:377-472: `in` points into the domain, o1/o2 are the tangents. */
static inline double face_point(const double* B, const double* anp1, const double* an,
                                const double* anm1, long m, long in, long o1, long o2) {
  return B[0] * (anm1[m] + anp1[m + in]) +
         B[1] * anm1[m + in] +
         B[2] * (an[m] + an[m + in]) +
         B[3] * (an[m + in + o1] + an[m + in - o1] + an[m + o1] + an[m - o1]) +
         B[4] * (an[m + in + o2] + an[m + in - o2] + an[m + o2] + an[m - o2]);
}

/* AdvanceField::advanceEdgeF/S, src/database.cpp:179-229, with the argument pattern of the edge
 * loops of src/fdtd.cpp:474-645: a, b point into the domain along the two normals, t along the edge. */
static inline double edge_point(const double* E, const double* anp1, const double* an,
                                const double* anm1, long m, long a, long b, long t) {
  return E[0] * (anp1[m + a] + anm1[m + b]) +
         E[1] * (anm1[m + a] + anp1[m + b]) +
         E[2] * (anm1[m] + anp1[m + a + b]) +
         E[3] * (an[m] + an[m + a] + an[m + b] + an[m + a + b]) +
         E[4] * (an[m - t] + an[m + a - t] + an[m + b - t] + an[m + a + b - t] +
                 an[m + t] + an[m + a + t] + an[m + b + t] + an[m + a + b + t]) -
         anm1[m + a + b];
}

/* AdvanceField::advanceCornerF/S, src/database.cpp:232-288, with the argument pattern of the
 * corner calls of src/fdtd.cpp:647-725: a (x), b (y), c (z) point into the domain. */
static inline double corner_point(const double* h, const double* anp1, const double* an,
                                  const double* anm1, long m, long a, long b, long c) {
  const long P1 = m + a, P2 = m + b, P3 = m + c, P4 = m + a + b, P5 = m + c + a, P6 = m + c + b,
             P7 = m + a + b + c;
  return -(an[m] * h[16] + anm1[m] * h[8] +
           anp1[P1] * h[1] + an[P1] * h[16] + anm1[P1] * h[9] +
           anp1[P2] * h[2] + an[P2] * h[16] + anm1[P2] * h[10] +
           anp1[P3] * h[3] + an[P3] * h[16] + anm1[P3] * h[11] +
           anp1[P4] * h[4] + an[P4] * h[16] + anm1[P4] * h[12] +
           anp1[P5] * h[5] + an[P5] * h[16] + anm1[P5] * h[13] +
           anp1[P6] * h[6] + an[P6] * h[16] + anm1[P6] * h[14] +
           anp1[P7] * h[7] + an[P7] * h[16] + anm1[P7] * h[15]) / h[0];
}

/* One potential (vector with nc = 3 or scalar with nc = 1): the whole sequence of
 * FdTd::fieldUpdate for one rank that owns both z ends. */
static void seed_inject(const mo_field* f, const mo_seed* seed, double time, double* anp1);

static void potential_update(const mo_field* f, int nc, double asrc, double* anp1, const double* an,
                             const double* anm1, const mo_seed* seed, double time) {
  const long N0 = f->N0, N1 = f->N1, np = f->np, N1N0 = N1 * N0;
  const long sI = nc * N1, sJ = nc, sK = nc * N1N0;
  const double* jsrc = anp1;  /* the source is read in place: J in anp1_ / rho in fnp1_ */

  /* Interior nodes, src/fdtd.cpp:270-303 (src/fdtdSC.cpp:318-372). */
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (long k = 1; k < np - 1; k++)
    for (long i = 1; i < N0 - 1; i++)
      for (long j = 1; j < N1 - 1; j++) {
        long l = nc * (N1N0 * k + N1 * i + j);
        for (int c = 0; c < nc; c++) {
          double v = (f->solver == 1)
                         ? nsfd_point(f->a, f->nsfd_alpha, f->nsfd_beta, asrc, an + c, anm1 + c, jsrc + c, l, sI, sJ, sK)
                         : fd_point(f->a, asrc, an + c, anm1 + c, jsrc + c, l, sI, sJ, sK);
          anp1[l + c] = v;
        }
      }

  /* TF/SF seed injection, src/fdtd.cpp:307-373 (vector potential only). */
  if (nc == 3 && seed && fabs(seed->beam.amplitude) > 1.0e-50) seed_inject(f, seed, time, anp1);

  /* Faces, src/fdtd.cpp:377-472. */
  for (long j = 1; j < N1 - 1; j++)
    for (long k = 1; k < np - 1; k++)
      for (int c = 0; c < nc; c++) {
        long m0 = nc * (N1N0 * k + j) + c;
        long m1 = nc * (N1N0 * k + N1N0 - N1 + j) + c;
        anp1[m0] = face_point(f->bB, anp1, an, anm1, m0, sI, sJ, sK);
        anp1[m1] = face_point(f->bB, anp1, an, anm1, m1, -sI, sJ, sK);
      }
  for (long i = 1; i < N0 - 1; i++)
    for (long k = 1; k < np - 1; k++)
      for (int c = 0; c < nc; c++) {
        long m0 = nc * (N1N0 * k + N1 * i) + c;
        long m1 = nc * (N1N0 * k + N1 * i + N1 - 1) + c;
        anp1[m0] = face_point(f->cB, anp1, an, anm1, m0, sJ, sI, sK);
        anp1[m1] = face_point(f->cB, anp1, an, anm1, m1, -sJ, sI, sK);
      }
  for (long i = 1; i < N0 - 1; i++)
    for (long j = 1; j < N1 - 1; j++)
      for (int c = 0; c < nc; c++) {
        long m0 = nc * (N1 * i + j) + c;
        long m1 = nc * (N1N0 * (np - 1) + N1 * i + j) + c;
        anp1[m0] = face_point(f->dB, anp1, an, anm1, m0, sK, sI, sJ);
        anp1[m1] = face_point(f->dB, anp1, an, anm1, m1, -sK, sI, sJ);
      }

  if (f->order != 2) return;

  /* Edges along z, src/fdtd.cpp:480-522. */
  for (long k = 1; k < np - 1; k++)
    for (int c = 0; c < nc; c++) {
      long b = nc * N1N0 * k + c;
      anp1[b] = edge_point(f->eE, anp1, an, anm1, b, sI, sJ, sK);
      long m = b + nc * N1 * (N0 - 1);
      anp1[m] = edge_point(f->eE, anp1, an, anm1, m, -sI, sJ, sK);
      m = b + nc * (N1 - 1);
      anp1[m] = edge_point(f->eE, anp1, an, anm1, m, sI, -sJ, sK);
      m = b + nc * (N1 * (N0 - 1) + N1 - 1);
      anp1[m] = edge_point(f->eE, anp1, an, anm1, m, -sI, -sJ, sK);
    }
  /* Edges along x, src/fdtd.cpp:527-579. */
  for (long i = 1; i < N0 - 1; i++)
    for (int c = 0; c < nc; c++) {
      long m = nc * (N1 * i) + c;
      anp1[m] = edge_point(f->fE, anp1, an, anm1, m, sJ, sK, sI);
      m = nc * (N1 * i + N1 - 1) + c;
      anp1[m] = edge_point(f->fE, anp1, an, anm1, m, -sJ, sK, sI);
      m = nc * (N1 * i + N1N0 * (np - 1)) + c;
      anp1[m] = edge_point(f->fE, anp1, an, anm1, m, sJ, -sK, sI);
      m = nc * (N1 * i + N1N0 * (np - 1) + N1 - 1) + c;
      anp1[m] = edge_point(f->fE, anp1, an, anm1, m, -sJ, -sK, sI);
    }
  /* Edges along y, src/fdtd.cpp:584-645. */
  for (long j = 1; j < N1 - 1; j++)
    for (int c = 0; c < nc; c++) {
      long m = nc * j + c;
      anp1[m] = edge_point(f->gE, anp1, an, anm1, m, sK, sI, sJ);
      m = nc * (N1N0 - N1 + j) + c;
      anp1[m] = edge_point(f->gE, anp1, an, anm1, m, sK, -sI, sJ);
      m = nc * (N1N0 * (np - 1) + j) + c;
      anp1[m] = edge_point(f->gE, anp1, an, anm1, m, -sK, sI, sJ);
      m = nc * (N1N0 * (np - 1) + N1 * (N0 - 1) + j) + c;
      anp1[m] = edge_point(f->gE, anp1, an, anm1, m, -sK, -sI, sJ);
    }
  /* Corners, src/fdtd.cpp:647-725. */
  for (int c = 0; c < nc; c++)
    for (int zk = 0; zk < 2; zk++)
      for (int xi = 0; xi < 2; xi++)
        for (int yj = 0; yj < 2; yj++) {
          long i = xi ? N0 - 1 : 0, j = yj ? N1 - 1 : 0, k = zk ? np - 1 : 0;
          long m = nc * (N1N0 * k + N1 * i + j) + c;
          anp1[m] = corner_point(f->hC, anp1, an, anm1, m, xi ? -sI : sI, yj ? -sJ : sJ, zk ? -sK : sK);
        }
}

void mo_field_update(const mo_field* f, double* anp1, const double* an, const double* anm1) {
  potential_update(f, 3, f->a[4], anp1, an, anm1, NULL, 0.0);
}

void mo_field_update_seeded(const mo_field* f, const mo_seed* seed, double time, double* anp1, const double* an,
                            const double* anm1) {
  potential_update(f, 3, f->a[4], anp1, an, anm1, seed, time);
}

void mo_scalar_update(const mo_field* f, double* fnp1, const double* fn, const double* fnm1) {
  potential_update(f, 1, f->a[5], fnp1, fn, fnm1, NULL, 0.0);
}

/* ------------------------------------------------------------------------------------------ */
/* Seed and laser-beam fields.                                                                 */
/* ------------------------------------------------------------------------------------------ */

static inline double dot3(const double* x, const double* y) { return x[0] * y[0] + x[1] * y[1] + x[2] * y[2]; }
static inline void cross3(const double* x, const double* y, double* z) {
  z[0] = x[1] * y[2] - x[2] * y[1];
  z[1] = x[2] * y[0] - x[0] * y[2];
  z[2] = x[0] * y[1] - x[1] * y[0];
}

/* Signal::self, src/classes.cpp:533-576. */
static double signal_self(const mo_signal* g, double t, double phase) {
  const double t0 = g->t0, s = g->s, f0 = g->f0, cep = g->cep, nR = g->nR;
  if (fabs(t - t0) > 10.0 * s) return 0.0;
  if (g->type == 0)
    return -cos(2 * MO_PI * f0 * (t - t0) + cep + phase) * 2.7724 * (t - t0) / (s * s) *
           exp(-1.3863 * (t - t0) * (t - t0) / (s * s));
  if (g->type == 1) return cos(2 * MO_PI * f0 * (t - t0) + cep + phase) * exp(-1.3863 * pow((t - t0) / s, 2));
  if (g->type == 2) return cos(2 * MO_PI * f0 * (t - t0) + cep + phase) / cosh((t - t0) / s);
  if (g->type == 3) {
    if (t - t0 <= -s / 2.0) return cos(2 * MO_PI * f0 * (t - t0) + cep + phase) * exp(-pow((t - t0 + s / 2.0) * f0 / nR, 2));
    if (t - t0 <= s / 2.0) return cos(2 * MO_PI * f0 * (t - t0) + cep + phase);
    return cos(2 * MO_PI * f0 * (t - t0) + cep + phase) * exp(-pow((t - t0 - s / 2.0) * f0 / nR, 2));
  }
  if (g->type == 4) {
    const double env = pow((1.0 + pow((t - t0) / g->sig0, 2)) * (1.0 + pow((t - t0) / g->sig1, 2)), 0.25);
    if (t - t0 <= -s / 2.0)
      return cos(2 * MO_PI * f0 * (t - t0) + cep + phase) * env * exp(-pow((t - t0 + s / 2.0) * f0 / nR, 2));
    if (t - t0 <= s / 2.0) return cos(2 * MO_PI * f0 * (t - t0) + cep + phase) * env;
    return cos(2 * MO_PI * f0 * (t - t0) + cep + phase) * env * exp(-pow((t - t0 - s / 2.0) * f0 / nR, 2));
  }
  return 0.0;
}

void mo_seed_fields(const mo_seed* sd, const double r[3], double time, double a[3]) {
  const mo_beam* s = &sd->beam;
  const double c0 = sd->c0;
  double rl[3] = {r[0], r[1], sd->gamma * (r[2] + sd->beta * c0 * (time + sd->dt))};
  double tl = sd->gamma * (time + sd->dt + sd->beta / c0 * r[2]);
  double rv[3] = {rl[0] - s->position[0], rl[1] - s->position[1], rl[2] - s->position[2]};
  double z = dot3(rv, s->direction);
  tl -= z / c0;
  double p = 0.0, tsignal, x, y, yv[3];
  if (s->type == 0) {
    tsignal = signal_self(&s->signal, tl, p);
    if (fabs(tsignal) < 1.0e-6) a[0] = a[1] = a[2] = 0.0;
    else for (int c = 0; c < 3; c++) a[c] = s->amplitude * tsignal * s->polarization[c];
  } else if (s->type == 1) {
    tsignal = signal_self(&s->signal, tl, p);
    x = dot3(rv, s->polarization);
    cross3(s->direction, s->polarization, yv);
    y = dot3(rv, yv);
    if (fabs(tsignal) < 1.0e-6 || fabs(x) > s->radius[0] || fabs(y) > s->radius[1]) a[0] = a[1] = a[2] = 0.0;
    else for (int c = 0; c < 3; c++) a[c] = s->amplitude * tsignal * s->polarization[c];
  } else if (s->type == 2 || s->type == 3) {
    tsignal = signal_self(&s->signal, tl, p);
    if (fabs(tsignal) < 1.0e-6) {
      a[0] = a[1] = a[2] = 0.0;
    } else {
      x = dot3(rv, s->polarization);
      cross3(s->direction, s->polarization, yv);
      y = dot3(rv, yv);
      double l = c0 / s->signal.f0;
      double zRp = MO_PI * s->radius[0] * s->radius[0] / l;
      double wrp = sqrt(1.0 + z * z / (zRp * zRp));
      double zRs = MO_PI * s->radius[1] * s->radius[1] / l;
      double wrs = sqrt(1.0 + z * z / (zRs * zRs));
      if (s->type == 2) {
        p = 0.5 * (atan(z / zRp) + atan(z / zRs) - MO_PI) - MO_PI * z / l * (pow(x / (zRp * wrp), 2) + pow(y / (zRs * wrs), 2));
        tsignal = signal_self(&s->signal, tl, p);
        double t = exp(-pow(x / (s->radius[0] * wrp), 2) - pow(y / (s->radius[1] * wrs), 2)) / sqrt(wrs * wrp) * s->amplitude;
        for (int c = 0; c < 3; c++) a[c] = t * tsignal * s->polarization[c];
      } else {
        for (int i = -s->order[0]; i <= s->order[0]; i++)
          for (int j = -s->order[1]; j <= s->order[1]; j++) {
            p = 0.5 * (atan(z / zRp) + atan(z / zRs) - MO_PI) - MO_PI * z / l * (pow(x / (zRp * wrp), 2) + pow(y / (zRs * wrs), 2));
            tsignal = signal_self(&s->signal, tl, p);
            double t = exp(-pow(x / (s->radius[0] * wrp), 2) - pow(y / (s->radius[1] * wrs), 2)) / sqrt(wrs * wrp) * s->amplitude;
            for (int c = 0; c < 3; c++) a[c] += t * tsignal * s->polarization[c];
          }
      }
    }
  }
  a[2] *= sd->gamma;
}

/* TF/SF seed injection of FdTd::fieldUpdate for one rank owning both z ends
 * (src/fdtd.cpp:307-373, KI = 2, KF = np - 2).  atemp is carried from call to call as in the
 * reference, which matters only for seeds that accumulate into it. */
static void seed_inject(const mo_field* f, const mo_seed* seed, double time, double* anp1) {
  const long N0 = f->N0, N1 = f->N1, np = f->np, N1N0 = N1 * N0;
  double atemp[3] = {0.0, 0.0, 0.0};
  const long KI = 2, KF = np - 2;
#define MO_RC(mm, out)                                              \
  do {                                                               \
    long k_ = (mm) / N1N0, i_ = ((mm) % N1N0) / N1;                  \
    long j_ = (mm) - (N1N0 * k_ + N1 * i_);                          \
    (out)[0] = f->xmin + i_ * f->dx;                                 \
    (out)[1] = f->ymin + j_ * f->dy;                                 \
    (out)[2] = f->zmin + (k_ + f->k0) * f->dz;                       \
  } while (0)
#define MO_ADD(m, sgn, coef)                                                   \
  do {                                                                         \
    for (int c = 0; c < 3; c++) anp1[3 * (m) + c] sgn## = (coef) * atemp[c];  \
  } while (0)
  double rc[3];
  for (long j = 2; j < N1 - 2; j++)
    for (long k = KI; k < KF; k++) {
      long m = N1N0 * k + N1 * 1 + j;
      MO_RC(m + N1, rc); mo_seed_fields(seed, rc, time, atemp); MO_ADD(m, -, f->a[1]);
      m = N1N0 * k + N1 * 2 + j;
      MO_RC(m - N1, rc); mo_seed_fields(seed, rc, time, atemp); MO_ADD(m, +, f->a[1]);
      m = N1N0 * k + N1 * (N0 - 2) + j;
      MO_RC(m - N1, rc); mo_seed_fields(seed, rc, time, atemp); MO_ADD(m, -, f->a[1]);
      m = N1N0 * k + N1 * (N0 - 3) + j;
      MO_RC(m + N1, rc); mo_seed_fields(seed, rc, time, atemp); MO_ADD(m, +, f->a[1]);
    }
  for (long i = 2; i < N0 - 2; i++)
    for (long k = KI; k < KF; k++) {
      long m = N1N0 * k + N1 * i + 1;
      MO_RC(m + 1, rc); mo_seed_fields(seed, rc, time, atemp); MO_ADD(m, -, f->a[2]);
      m = N1N0 * k + N1 * i + 2;
      MO_RC(m - 1, rc); mo_seed_fields(seed, rc, time, atemp); MO_ADD(m, +, f->a[2]);
      m = N1N0 * k + N1 * i + N1 - 2;
      MO_RC(m - 1, rc); mo_seed_fields(seed, rc, time, atemp); MO_ADD(m, -, f->a[2]);
      m = N1N0 * k + N1 * i + N1 - 3;
      MO_RC(m + 1, rc); mo_seed_fields(seed, rc, time, atemp); MO_ADD(m, +, f->a[2]);
    }
  for (long i = 2; i < N0 - 2; i++)
    for (long j = 2; j < N1 - 2; j++) {
      long m = N1N0 * 1 + N1 * i + j;
      MO_RC(m + N1N0, rc); mo_seed_fields(seed, rc, time, atemp); MO_ADD(m, -, f->a[3]);
      m = N1N0 * 2 + N1 * i + j;
      MO_RC(m - N1N0, rc); mo_seed_fields(seed, rc, time, atemp); MO_ADD(m, +, f->a[3]);
    }
  for (long i = 2; i < N0 - 2; i++)
    for (long j = 2; j < N1 - 2; j++) {
      long m = N1N0 * (np - 2) + N1 * i + j;
      MO_RC(m - N1N0, rc); mo_seed_fields(seed, rc, time, atemp); MO_ADD(m, -, f->a[3]);
      m = N1N0 * (np - 3) + N1 * i + j;
      MO_RC(m + N1N0, rc); mo_seed_fields(seed, rc, time, atemp); MO_ADD(m, +, f->a[3]);
    }
#undef MO_RC
#undef MO_ADD
}

/* FdTd::fieldEvaluate, src/fdtd.cpp:818-845 (SC: src/fdtdSC.cpp:1110-1140).  FieldVector::dv
 * and ::mdv (src/fieldvector.h:87-107) store into float after each step, so E is rounded to float
 * twice; B is computed in double and rounded once. */
static inline void eval_node(const mo_field* f, long m, const double* anp1, const double* an,
                             const double* fn, float* en, float* bn) {
  const long N1 = f->N1, N1N0 = (long)f->N1 * f->N0;
  const double dt = f->dt, dx2 = 2.0 * f->dx, dy2 = 2.0 * f->dy, dz2 = 2.0 * f->dz;
  for (int c = 0; c < 3; c++) {
    float e = (float)(anp1[3 * m + c] / (-dt));
    e = (float)((double)e - an[3 * m + c] / (-dt));
    en[3 * m + c] = e;
  }
  if (fn) {
    en[3 * m + 0] = (float)((double)en[3 * m + 0] - (fn[m + N1] - fn[m - N1]) / dx2);
    en[3 * m + 1] = (float)((double)en[3 * m + 1] - (fn[m + 1] - fn[m - 1]) / dy2);
    en[3 * m + 2] = (float)((double)en[3 * m + 2] - (fn[m + N1N0] - fn[m - N1N0]) / dz2);
  }
  bn[3 * m + 0] = (float)(0.5 * ((an[3 * (m + 1) + 2] - an[3 * (m - 1) + 2]) / dy2 -
                                 (an[3 * (m + N1N0) + 1] - an[3 * (m - N1N0) + 1]) / dz2 +
                                 (anp1[3 * (m + 1) + 2] - anp1[3 * (m - 1) + 2]) / dy2 -
                                 (anp1[3 * (m + N1N0) + 1] - anp1[3 * (m - N1N0) + 1]) / dz2));
  bn[3 * m + 1] = (float)(0.5 * ((an[3 * (m + N1N0)] - an[3 * (m - N1N0)]) / dz2 -
                                 (an[3 * (m + N1) + 2] - an[3 * (m - N1) + 2]) / dx2 +
                                 (anp1[3 * (m + N1N0)] - anp1[3 * (m - N1N0)]) / dz2 -
                                 (anp1[3 * (m + N1) + 2] - anp1[3 * (m - N1) + 2]) / dx2));
  bn[3 * m + 2] = (float)(0.5 * ((an[3 * (m + N1) + 1] - an[3 * (m - N1) + 1]) / dx2 -
                                 (an[3 * (m + 1)] - an[3 * (m - 1)]) / dy2 +
                                 (anp1[3 * (m + N1) + 1] - anp1[3 * (m - N1) + 1]) / dx2 -
                                 (anp1[3 * (m + 1)] - anp1[3 * (m - 1)]) / dy2));
}

void mo_eval_eb(const mo_field* f, const double* anp1, const double* an, const double* fn, float* en,
                float* bn) {
  const long N0 = f->N0, N1 = f->N1, np = f->np, N1N0 = N1 * N0;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (long k = 1; k < np - 1; k++)
    for (long i = 1; i < N0 - 1; i++)
      for (long j = 1; j < N1 - 1; j++) eval_node(f, N1N0 * k + N1 * i + j, anp1, an, fn, en, bn);
  /* Planes k = 0 and k = np-1 are copies of k = 1 and k = np-2, src/fdtd.cpp:755-772. */
  for (long i = 1; i < N0 - 1; i++)
    for (long j = 1; j < N1 - 1; j++) {
      long m = N1 * i + j, mt = N1N0 * (np - 1) + N1 * i + j;
      for (int c = 0; c < 3; c++) {
        en[3 * m + c] = en[3 * (m + N1N0) + c];
        bn[3 * m + c] = bn[3 * (m + N1N0) + c];
        en[3 * mt + c] = en[3 * (mt - N1N0) + c];
        bn[3 * mt + c] = bn[3 * (mt - N1N0) + c];
      }
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Particle push.                                                                              */
/* ------------------------------------------------------------------------------------------ */

/* pmod, src/stdinclude.cpp:88-93. */
static inline double mo_pmod(double a, double b) {
  double x = fmod(a, b);
  x += (x < 0.0) ? b : 0.0;
  return x;
}

/* The per-call state of one laser-beam evaluation (the fields of UpdateBunchParallel that the
 * beam functions of src/beam.cc:80-496 use). */
typedef struct {
  double rv[3], z, tl, tlm, p0;
  double eT[3], bT[3];
} beam_state;

static inline void set3(double* d, double a, const double* v) { for (int c = 0; c < 3; c++) d[c] = a * v[c]; }
static inline void add3(double* d, double a, const double* v) { for (int c = 0; c < 3; c++) d[c] += a * v[c]; }

/* Solver::planeWave .. standingSuperGaussianBeam, src/beam.cc:80-496.  For the super-gaussian
 * standing beam the reference reads an unset ubp.l (src/beam.cc:466); s->l (l_) is used here. */
static void beam_fields(const mo_beam* s, double c0, beam_state* u) {
  const int type = s->type;
  double ts, tsm, tse, tsb, x = 0.0, y = 0.0, yv[3], x0, y0, wrp, wrs, atanP, atanS, t, p1, af;
  double ex[3], ez[3], by[3], bz[3];
  if (type == 0 || type == 1 || type == 4 || type == 5) {
    if (type == 1 || type == 5) {
      x = dot3(u->rv, s->polarization);
      cross3(s->direction, s->polarization, yv);
      y = dot3(u->rv, yv);
    }
    if (type == 5 && pow(x / s->radius[0], 2) + pow(y / s->radius[1], 2) > 1.0) goto zero;
    if (type == 0 || type == 1) {
      ts = signal_self(&s->signal, u->tl, u->p0);
      if (fabs(ts) < 1.0e-6) goto zero;
      if (type == 1 && pow(x / s->radius[0], 2) + pow(y / s->radius[1], 2) > 1.0) goto zero;
      set3(u->eT, s->amplitude * ts, s->polarization);
      cross3(s->direction, s->polarization, u->bT);
      set3(u->bT, s->amplitude * ts / c0, u->bT);
      return;
    }
    ts = signal_self(&s->signal, u->tl, u->p0);
    tsm = signal_self(&s->signal, u->tlm, u->p0);
    tse = ts - tsm;
    tsb = ts + tsm;
    if (fabs(tse) < 1.0e-6 && fabs(tsb) < 1.0e-6) goto zero;
    set3(u->eT, s->amplitude * tse, s->polarization);
    cross3(s->direction, s->polarization, u->bT);
    set3(u->bT, s->amplitude * tsb / c0, u->bT);
    return;
  }
  x = dot3(u->rv, s->polarization);
  cross3(s->direction, s->polarization, yv);
  y = dot3(u->rv, yv);
  wrp = sqrt(1.0 + u->z * u->z / (s->zR[0] * s->zR[0]));
  wrs = sqrt(1.0 + u->z * u->z / (s->zR[1] * s->zR[1]));
  if (type == 2 || type == 6) {
    x0 = x / wrp;
    y0 = y / wrs;
    if (fabs(x0) > 4.0 * s->radius[0] || fabs(y0) > 4.0 * s->radius[1]) goto zero;
    ts = signal_self(&s->signal, u->tl, u->p0);
    if (type == 2) {
      if (fabs(ts) < 1.0e-6) goto zero;
    } else {
      tsm = signal_self(&s->signal, u->tlm, u->p0);
      tse = ts - tsm;
      tsb = ts + tsm;
      if (fabs(tse) < 1.0e-6 && fabs(tsb) < 1.0e-6) goto zero;
    }
    atanP = atan(u->z / s->zR[0]);
    atanS = atan(u->z / s->zR[1]);
    u->p0 = 0.5 * (atanP + atanS) - MO_PI * u->z / s->l * (pow(x0 / s->zR[0], 2) + pow(y0 / s->zR[1], 2));
    t = exp(-pow(x0 / s->radius[0], 2) - pow(y0 / s->radius[1], 2)) / sqrt(wrs * wrp);
    t *= s->amplitude;
    if (type == 2) {
      p1 = u->p0 - MO_PI / 2.0;
      ts = signal_self(&s->signal, u->tl, p1);
      set3(ex, t * ts, s->polarization);
      set3(by, t * ts / c0, yv);
      p1 = u->p0 + atanP;
      ts = signal_self(&s->signal, u->tl, p1);
      set3(ez, t * (-x0 / s->zR[0]) * ts, s->direction);
      p1 = u->p0 + atanS;
      ts = signal_self(&s->signal, u->tl, p1);
      set3(bz, t * (-y0 / s->zR[1]) / c0 * ts, s->direction);
    } else {
      p1 = u->p0 - MO_PI / 2.0;
      ts = signal_self(&s->signal, u->tl, p1);
      p1 = u->p0 - MO_PI / 2.0;
      tsm = signal_self(&s->signal, u->tlm, p1);
      set3(ex, t * (ts - tsm), s->polarization);
      set3(by, t / c0 * (ts + tsm), yv);
      p1 = u->p0 + atanP;
      ts = signal_self(&s->signal, u->tl, p1);
      p1 = -p1;
      tsm = signal_self(&s->signal, u->tlm, p1);
      set3(ez, t * (-x0 / s->zR[0]) * (ts - tsm), s->direction);
      p1 = u->p0 + atanS;
      ts = signal_self(&s->signal, u->tl, p1);
      p1 = -p1;
      tsm = signal_self(&s->signal, u->tlm, p1);
      set3(bz, t * (-y0 / s->zR[1]) / c0 * (ts - tsm), s->direction);
    }
    for (int c = 0; c < 3; c++) { u->eT[c] = ex[c]; u->eT[c] += ez[c]; u->bT[c] = by[c]; u->bT[c] += bz[c]; }
    return;
  }
  /* super-gaussian (3) and its standing variant (7) */
  if ((fabs(x) - s->order[0] * s->radius[0]) > 4.0 * s->radius[0] * wrp ||
      (fabs(y) - s->order[1] * s->radius[1]) > 4.0 * s->radius[1] * wrs)
    goto zero;
  ts = signal_self(&s->signal, u->tl, u->p0);
  if (type == 3) {
    if (fabs(ts) < 1.0e-6) goto zero;
  } else {
    tsm = signal_self(&s->signal, u->tlm, u->p0);
    tse = ts - tsm;
    tsb = ts + tsm;
    if (fabs(tse) < 1.0e-6 && fabs(tsb) < 1.0e-6) goto zero;
  }
  atanP = atan(u->z / s->zR[0]);
  atanS = atan(u->z / s->zR[1]);
  af = s->amplitude / sqrt(wrs * wrp);
  for (int c = 0; c < 3; c++) ex[c] = ez[c] = bz[c] = by[c] = 0.0;
  for (int i = -s->order[0]; i <= s->order[0]; i++)
    for (int j = -s->order[1]; j <= s->order[1]; j++) {
      x0 = (x - i * s->radius[0]) / wrp;
      y0 = (y - j * s->radius[1]) / wrs;
      if (fabs(x0) > 4.0 * s->radius[0] || fabs(y0) > 4.0 * s->radius[1]) continue;
      u->p0 = 0.5 * (atanP + atanS) - MO_PI * u->z / s->l * (pow(x0 / s->zR[0], 2) + pow(y / s->zR[1], 2));
      t = af * exp(-pow(x0 / s->radius[0], 2) - pow(y0 / s->radius[1], 2));
      if (type == 3) {
        p1 = u->p0 - MO_PI / 2.0;
        ts = signal_self(&s->signal, u->tl, p1);
        add3(ex, t * ts, s->polarization);
        add3(by, t * ts / c0, yv);
        p1 = u->p0 + atanP;
        ts = signal_self(&s->signal, u->tl, p1);
        add3(ez, t * (-x0 / s->zR[0]) * ts, s->direction);
        p1 = u->p0 + atanS;
        ts = signal_self(&s->signal, u->tl, p1);
        add3(bz, t * (-y0 / s->zR[1]) * ts / c0, s->direction);
      } else {
        p1 = u->p0 - MO_PI / 2.0;
        ts = signal_self(&s->signal, u->tl, p1);
        p1 = u->p0 - MO_PI / 2.0;
        tsm = signal_self(&s->signal, u->tlm, p1);
        add3(ex, t * (ts - tsm), s->polarization);
        add3(by, t * (ts + tsm) / c0, yv);
        p1 = u->p0 + atanP;
        ts = signal_self(&s->signal, u->tl, p1);
        p1 = -p1;
        tsm = signal_self(&s->signal, u->tlm, p1);
        add3(ez, t * (-x0 / s->zR[0]) * (ts - tsm), s->direction);
        p1 = u->p0 + atanS;
        ts = signal_self(&s->signal, u->tl, p1);
        p1 = -p1;
        tsm = signal_self(&s->signal, u->tlm, p1);
        add3(bz, t * (-y0 / s->zR[1]) * (ts - tsm) / c0, s->direction);
      }
    }
  for (int c = 0; c < 3; c++) { u->eT[c] = ex[c]; u->eT[c] += ez[c]; u->bT[c] = by[c]; u->bT[c] += bz[c]; }
  return;
zero:
  for (int c = 0; c < 3; c++) u->eT[c] = u->bT[c] = 0.0;
}

/* The boost of a lab-frame beam field into the bunch frame, added to bt/et
 * (src/solver.cpp:1870-1877, :1937-1944). */
static inline void boost_add(const mo_push* p, const beam_state* u, double* bt, double* et) {
  bt[0] += p->gamma * (u->bT[0] + p->beta / p->c0 * u->eT[1]);
  bt[1] += p->gamma * (u->bT[1] - p->beta / p->c0 * u->eT[0]);
  bt[2] += u->bT[2];
  et[0] += p->gamma * (u->eT[0] - p->beta * p->c0 * u->bT[1]);
  et[1] += p->gamma * (u->eT[1] + p->beta * p->c0 * u->bT[0]);
  et[2] += u->eT[2];
}

/* One laser beam at the lab point of bunch-frame r and timeBunch: rv, z, tl and tlm of
 * src/solver.cpp:1829-1840 and :1890-1904.  The optical-undulator branch of the reference
 * never sets tlm (standing beams there read a stale value); t0 + z/c0 is used for both. */
static void beam_at(const mo_push* p, const mo_beam* s, double timeBunch, const double* r, beam_state* u) {
  double rl[3] = {r[0], r[1], p->gamma * (r[2] + p->beta * p->c0 * (timeBunch + p->dt_shift))};
  double t0 = p->gamma * (timeBunch + p->dt_shift + p->beta / p->c0 * r[2]);
  for (int c = 0; c < 3; c++) u->rv[c] = rl[c] - s->position[c];
  u->z = dot3(u->rv, s->direction);
  u->tl = t0 - u->z / p->c0;
  u->tlm = t0 + u->z / p->c0;
  u->p0 = 0.0;
  beam_fields(s, p->c0, u);
}

/* Solver::undulatorField (src/solver.cpp:1798-1880): static modules with
 * Solver::staticUndulator (src/beam.cc:14-76).  ub_.b0/ku/ct/st are recomputed per module per
 * particle in the reference; the values are the same every time. */
static void static_undulators(const mo_push* p, double timeBunch, const double* r, double* bt,
                              double* et) {
  for (int u = 0; u < p->n_und; u++) {
    const mo_undulator* U = &p->und[u];
    if (U->type == 1) {
      beam_state st;
      beam_at(p, &U->beam, timeBunch, r, &st);
      boost_add(p, &st, bt, et);
      continue;
    }
    if (U->type != 0) continue;
    double b0 = (U->lu != 0.0) ? 9.109e-31 * p->c0 * 2 * MO_PI / U->lu * U->k / 1.602e-19 : 0.0;
    double ku = (U->lu != 0.0) ? 2 * MO_PI / U->lu : 0.0;
    double ct = cos(U->theta), st = sin(U->theta);
    double lz = p->gamma * (r[2] + p->beta * p->c0 * (timeBunch + p->dt_shift)) - U->rb;
    double ly = r[0] * ct + r[1] * st;
    double d1, sz, t0, r0;
    double ul = U->length * U->lu;
    if (lz >= 0.0 && lz <= ul) {
      d1 = b0 * cosh(ku * ly) * sin(ku * lz) * p->gamma;
      bt[0] += d1 * ct;
      bt[1] += d1 * st;
      bt[2] += b0 * sinh(ku * ly) * cos(ku * lz);
      d1 *= p->c0 * p->beta;
      et[1] += d1 * ct;
      et[0] += -d1 * st;
      et[2] += 0.0;
    } else if (lz < 0.0) {
      sz = exp(-pow(ku * lz, 2) / 2.0);
      if (u != 0) {
        const mo_undulator* P = &p->und[u - 1];
        r0 = P->rb + P->length * P->lu - U->rb;
        if (lz < r0 || r0 == 0.0) sz = 0.0;
        else
          sz *= 0.35875 + 0.48829 * cos(MO_PI * lz / r0) + 0.14128 * cos(2.0 * MO_PI * lz / r0) +
                0.01168 * cos(3.0 * MO_PI * lz / r0);
      }
      d1 = b0 * cosh(ku * ly) * sz * ku * lz * p->gamma;
      bt[0] += d1 * ct;
      bt[1] += d1 * st;
      bt[2] += b0 * sinh(ku * ly) * sz;
      d1 *= p->c0 * p->beta;
      et[1] += d1 * ct;
      et[0] += -d1 * st;
      et[2] += 0.0;
    } else if (lz > ul) {
      t0 = lz - ul;
      sz = exp(-pow(ku * t0, 2) / 2.0);
      if (u + 1 != p->n_und) {
        const mo_undulator* Nx = &p->und[u + 1];
        r0 = Nx->rb - U->rb - U->length * U->lu;
        if (t0 > r0 || r0 == 0.0) sz = 0.0;
        else
          sz *= 0.35875 + 0.48829 * cos(MO_PI * t0 / r0) + 0.14128 * cos(2.0 * MO_PI * t0 / r0) +
                0.01168 * cos(3.0 * MO_PI * t0 / r0);
      }
      d1 = b0 * cosh(ku * ly) * sz * ku * t0 * p->gamma;
      bt[0] += d1 * ct;
      bt[1] += d1 * st;
      bt[2] += b0 * sinh(ku * ly) * sz;
      d1 *= p->c0 * p->beta;
      et[1] += d1 * ct;
      et[0] += -d1 * st;
      et[2] += 0.0;
    }
  }
}

typedef struct { double et[3], bt[3]; int flag; } push_out;

/* The per-particle body of Solver::bunchUpdate, src/solver.cpp:1437-1549.  Returns the crossing
 * flag: 0 none, 1 below zp0, 2 at or above zp1, -1 not owned (skipped), and counts particles outside
 * the transverse domain into *nt. */
static int push_one(const mo_push* p, double timeBunch, double* q, const float* en, const float* bn,
                    long* nt) {
  double* rnp = q + 1;
  double* gb = q + 7;
  double* e = q + 10;
  const long N1 = p->N1, N1N0 = (long)p->N1 * p->N0;

  double zr = mo_pmod(rnp[2] - p->zmin, p->Lz) + p->zmin;
  if (!((zr >= p->zp0) && (zr < p->zp1))) return -1;

  int b1x = (rnp[0] < p->xmax - p->dx && rnp[0] > p->xmin + p->dx);
  int b1y = (rnp[1] < p->ymax - p->dy && rnp[1] > p->ymin + p->dy);
  int b1z = (rnp[2] < p->zp1 && rnp[2] >= p->zp0);

  double bt[3] = {0.0, 0.0, 0.0}, et[3] = {0.0, 0.0, 0.0};
  static_undulators(p, timeBunch, rnp, bt, et);
  /* Solver::externalField, src/solver.cpp:1886-1947. */
  for (int x = 0; x < p->n_ext; x++) {
    beam_state st;
    beam_at(p, &p->ext[x], timeBunch, rnp, &st);
    boost_add(p, &st, bt, et);
  }

  if (*e == 1.0) {
    if (b1x && b1y && b1z) {
      double d1;
      double dxr = modf((rnp[0] - p->xmin) / p->dx, &d1); int i = (int)d1;
      double dyr = modf((rnp[1] - p->ymin) / p->dy, &d1); int j = (int)d1;
      double dzr = modf((rnp[2] - p->zmin) / p->dz, &d1); int k = (int)d1;
      long m = (long)(k - p->k0) * N1N0 + (long)i * N1 + j;
      const long nodes[8] = {m, m + N1, m + 1, m + N1 + 1, m + N1N0, m + N1N0 + N1, m + N1N0 + 1, m + N1N0 + N1 + 1};
      const double w[8] = {(1.0 - dxr) * (1.0 - dyr) * (1.0 - dzr), dxr * (1.0 - dyr) * (1.0 - dzr),
                           (1.0 - dxr) * dyr * (1.0 - dzr),         dxr * dyr * (1.0 - dzr),
                           (1.0 - dxr) * (1.0 - dyr) * dzr,         dxr * (1.0 - dyr) * dzr,
                           (1.0 - dxr) * dyr * dzr,                 dxr * dyr * dzr};
      for (int n = 0; n < 8; n++)
        for (int c = 0; c < 3; c++) et[c] += w[n] * en[3 * nodes[n] + c];
      for (int n = 0; n < 8; n++)
        for (int c = 0; c < 3; c++) bt[c] += w[n] * bn[3 * nodes[n] + c];
    } else if (!b1x && !b1y && b1z) {
      (*nt)++;
    }
  } else if (p->n_und > 0) {
    double lz = p->gamma * (rnp[2] + p->beta * p->c0 * (timeBunch + p->dt_shift));
    *e = (lz > -p->und[0].dist) ? 1.0 : 0.0;
  } else {
    *e = 1.0;
  }

  /* Boris rotation, src/solver.cpp:1519-1535. */
  double gbm[3], gbp[3], gbpl[3], d1;
  for (int c = 0; c < 3; c++) gbm[c] = gb[c] + p->r1 * et[c];
  gbp[0] = gbm[1] * bt[2] - gbm[2] * bt[1];
  gbp[1] = gbm[2] * bt[0] - gbm[0] * bt[2];
  gbp[2] = gbm[0] * bt[1] - gbm[1] * bt[0];
  d1 = sqrt(1.0 + (gbm[0] * gbm[0] + gbm[1] * gbm[1] + gbm[2] * gbm[2]));
  for (int c = 0; c < 3; c++) gbp[c] = p->r2 / d1 * gbp[c];
  for (int c = 0; c < 3; c++) gbp[c] += gbm[c];
  gbpl[0] = gbp[1] * bt[2] - gbp[2] * bt[1];
  gbpl[1] = gbp[2] * bt[0] - gbp[0] * bt[2];
  gbpl[2] = gbp[0] * bt[1] - gbp[1] * bt[0];
  double bt2 = bt[0] * bt[0] + bt[1] * bt[1] + bt[2] * bt[2];
  double s = 2.0 / (d1 / p->r2 + p->r2 / d1 * bt2);
  for (int c = 0; c < 3; c++) gbpl[c] = s * gbpl[c];
  for (int c = 0; c < 3; c++) gbpl[c] += gbm[c];
  for (int c = 0; c < 3; c++) gb[c] = gbpl[c];
  for (int c = 0; c < 3; c++) gb[c] += p->r1 * et[c];

  /* Drift, src/solver.cpp:1538-1541. */
  double g = p->dtb / sqrt(1.0 + (gb[0] * gb[0] + gb[1] * gb[1] + gb[2] * gb[2]));
  double dr[3];
  for (int c = 0; c < 3; c++) dr[c] = g * gb[c];
  for (int c = 0; c < 3; c++) rnp[c] += dr[c];

  zr += dr[2];
  if (zr < p->zp0) return 1;
  if (zr >= p->zp1) return 2;
  return 0;
}

long mo_push_substep(const mo_push* p, double timeBunch, double* rec, long n, long cap,
                     const float* en, const float* bn, long* n_transverse_out) {
  signed char* flag = (signed char*)malloc(n > 0 ? (size_t)n : 1);
  long nt = 0;
#pragma omp parallel for num_threads(g_threads) schedule(static) reduction(+ : nt)
  for (long i = 0; i < n; i++) {
    long nt_i = 0;
    flag[i] = (signed char)push_one(p, timeBunch, rec + MO_REC * i, en, bn, &nt_i);
    nt += nt_i;
  }
  if (n_transverse_out) *n_transverse_out = nt;
  /* Self-exchange with one rank (src/solver.cpp:1551-1568): particles that crossed below zp0
   * come back first (they were sent with tag 1 to rankB = 0 and received from rankF = 0), then
   * those that crossed at or above zp1, each group in list order, appended to the list. */
  long extra = 0;
  for (long i = 0; i < n; i++) extra += (flag[i] == 1 || flag[i] == 2);
  if (n + extra > cap) { free(flag); return -1; }
  long w = n;
  for (int pass = 1; pass <= 2; pass++)
    for (long i = 0; i < n; i++)
      if (flag[i] == pass) { memcpy(rec + MO_REC * w, rec + MO_REC * i, MO_REC * sizeof(double)); w++; }
  free(flag);
  return w;
}

/* ------------------------------------------------------------------------------------------ */
/* Zigzag deposit, src/fdtd.cpp:38-185 (+ rho, src/fdtdSC.cpp:140-161).                        */
/* ------------------------------------------------------------------------------------------ */

/* The reference adds in place; the atomic form is used only by the multi-threaded CPU baseline. */
static inline void addv(double* p, double v, int at) {
  if (at) {
#pragma omp atomic
    p[0] += v;
  } else {
    p[0] += v;
  }
}

static inline void add_half_segment(const mo_deposit* d, double* J, long m, double q, double dxh,
                                    double dyh, double dzh, const double* jc, int at) {
  const long N1 = d->N1, N1N0 = (long)d->N1 * d->N0;
  double x1 = 1.0 - dxh, x2 = dxh, y1 = 1.0 - dyh, y2 = dyh, z1 = 1.0 - dzh, z2 = dzh;
  addv(&J[3 * (m) + 0], q * 0.5 * y1 * z1 * jc[0], at);
  addv(&J[3 * (m + N1) + 0], q * 0.5 * y1 * z1 * jc[0], at);
  addv(&J[3 * (m + 1) + 0], q * 0.5 * y2 * z1 * jc[0], at);
  addv(&J[3 * (m + N1 + 1) + 0], q * 0.5 * y2 * z1 * jc[0], at);
  addv(&J[3 * (m + N1N0) + 0], q * 0.5 * y1 * z2 * jc[0], at);
  addv(&J[3 * (m + N1N0 + N1) + 0], q * 0.5 * y1 * z2 * jc[0], at);
  addv(&J[3 * (m + N1N0 + 1) + 0], q * 0.5 * y2 * z2 * jc[0], at);
  addv(&J[3 * (m + N1N0 + N1 + 1) + 0], q * 0.5 * y2 * z2 * jc[0], at);

  addv(&J[3 * (m) + 1], q * 0.5 * x1 * z1 * jc[1], at);
  addv(&J[3 * (m + N1) + 1], q * 0.5 * x2 * z1 * jc[1], at);
  addv(&J[3 * (m + 1) + 1], q * 0.5 * x1 * z1 * jc[1], at);
  addv(&J[3 * (m + N1 + 1) + 1], q * 0.5 * x2 * z1 * jc[1], at);
  addv(&J[3 * (m + N1N0) + 1], q * 0.5 * x1 * z2 * jc[1], at);
  addv(&J[3 * (m + N1N0 + N1) + 1], q * 0.5 * x2 * z2 * jc[1], at);
  addv(&J[3 * (m + N1N0 + 1) + 1], q * 0.5 * x1 * z2 * jc[1], at);
  addv(&J[3 * (m + N1N0 + N1 + 1) + 1], q * 0.5 * x2 * z2 * jc[1], at);

  addv(&J[3 * (m) + 2], q * 0.5 * x1 * y1 * jc[2], at);
  addv(&J[3 * (m + N1) + 2], q * 0.5 * x2 * y1 * jc[2], at);
  addv(&J[3 * (m + 1) + 2], q * 0.5 * x1 * y2 * jc[2], at);
  addv(&J[3 * (m + N1 + 1) + 2], q * 0.5 * x2 * y2 * jc[2], at);
  addv(&J[3 * (m + N1N0) + 2], q * 0.5 * x1 * y1 * jc[2], at);
  addv(&J[3 * (m + N1N0 + N1) + 2], q * 0.5 * x2 * y1 * jc[2], at);
  addv(&J[3 * (m + N1N0 + 1) + 2], q * 0.5 * x1 * y2 * jc[2], at);
  addv(&J[3 * (m + N1N0 + N1 + 1) + 2], q * 0.5 * x2 * y2 * jc[2], at);
}

static inline void add_rho(const mo_deposit* d, double* rho, long m, double q, const double* rp, int at) {
  const long N1 = d->N1, N1N0 = (long)d->N1 * d->N0;
  double c;
  double dxp = modf((rp[0] - d->xmin) / d->dx, &c);
  double dyp = modf((rp[1] - d->ymin) / d->dy, &c);
  double dzp = modf((rp[2] - d->zmin) / d->dz, &c);
  double x1 = 1.0 - dxp, x2 = dxp, y1 = 1.0 - dyp, y2 = dyp, z1 = 1.0 - dzp, z2 = dzp;
  addv(&rho[m], q * x1 * y1 * z1, at);
  addv(&rho[m + N1], q * x2 * y1 * z1, at);
  addv(&rho[m + 1], q * x1 * y2 * z1, at);
  addv(&rho[m + N1 + 1], q * x2 * y2 * z1, at);
  addv(&rho[m + N1N0], q * x1 * y1 * z2, at);
  addv(&rho[m + N1N0 + N1], q * x2 * y1 * z2, at);
  addv(&rho[m + N1N0 + 1], q * x1 * y2 * z2, at);
  addv(&rho[m + N1N0 + N1 + 1], q * x2 * y2 * z2, at);
}

static inline double dmin(double a, double b) { return a < b ? a : b; }
static inline double dmax(double a, double b) { return a > b ? a : b; }
static inline int imin(int a, int b) { return a < b ? a : b; }
static inline int imax(int a, int b) { return a > b ? a : b; }

static void deposit_one(const mo_deposit* d, const double* q, double* J, double* rho, int at) {
  const double* rp = q + 1;
  const double* rm = q + 4;
  const long N1 = d->N1, N1N0 = (long)d->N1 * d->N0;
  int bp = (rp[0] < d->xmax - d->dx && rp[0] > d->xmin + d->dx && rp[1] < d->ymax - d->dy &&
            rp[1] > d->ymin + d->dy && rp[2] < d->zp1 && rp[2] >= d->zp0);
  int bm = (rm[0] < d->xmax - d->dx && rm[0] > d->xmin + d->dx && rm[1] < d->ymax - d->dy &&
            rm[1] > d->ymin + d->dy && rm[2] < d->zp1 && rm[2] >= d->zp0);
  if (!(bp || bm)) return;
  double qq = q[0];
  int ip = (int)floor((rp[0] - d->xmin) / d->dx);
  int jp = (int)floor((rp[1] - d->ymin) / d->dy);
  int kp = (int)floor((rp[2] - d->zmin) / d->dz);
  int im = (int)floor((rm[0] - d->xmin) / d->dx);
  int jm = (int)floor((rm[1] - d->ymin) / d->dy);
  int km = (int)floor((rm[2] - d->zmin) / d->dz);
  double r[3];
  r[0] = dmin(imin(im, ip) * d->dx + d->dx + d->xmin, dmax(imax(im, ip) * d->dx + d->xmin, 0.5 * (rm[0] + rp[0])));
  r[1] = dmin(imin(jm, jp) * d->dy + d->dy + d->ymin, dmax(imax(jm, jp) * d->dy + d->ymin, 0.5 * (rm[1] + rp[1])));
  r[2] = dmin(imin(km, kp) * d->dz + d->dz + d->zmin, dmax(imax(km, kp) * d->dz + d->zmin, 0.5 * (rm[2] + rp[2])));
  double jcm[3] = {r[0] - rm[0], r[1] - rm[1], r[2] - rm[2]};
  double jcp[3] = {rp[0] - r[0], rp[1] - r[1], rp[2] - r[2]};
  double c;
  if (bp) {
    long m = N1N0 * (kp - d->k0) + N1 * ip + jp;
    double dxp = modf((0.5 * (rp[0] + r[0]) - d->xmin) / d->dx, &c);
    double dyp = modf((0.5 * (rp[1] + r[1]) - d->ymin) / d->dy, &c);
    double dzp = modf((0.5 * (rp[2] + r[2]) - d->zmin) / d->dz, &c);
    add_half_segment(d, J, m, qq, dxp, dyp, dzp, jcp, at);
    if (rho) add_rho(d, rho, m, qq, rp, at);
  }
  if (bm) {
    long m = N1N0 * (km - d->k0) + N1 * im + jm;
    double dxm = modf((0.5 * (rm[0] + r[0]) - d->xmin) / d->dx, &c);
    double dym = modf((0.5 * (rm[1] + r[1]) - d->ymin) / d->dy, &c);
    double dzm = modf((0.5 * (rm[2] + r[2]) - d->zmin) / d->dz, &c);
    add_half_segment(d, J, m, qq, dxm, dym, dzm, jcm, at);
  }
}

void mo_deposit_current(const mo_deposit* d, const double* rec, long n, double* J, double* rho) {
  if (g_threads <= 1) {
    for (long i = 0; i < n; i++) deposit_one(d, rec + MO_REC * i, J, rho, 0);
    return;
  }
  /* Multi-threaded CPU baseline only: threads take disjoint particle ranges and add into the
   * shared arrays atomically, so the sums land in a different order than the reference's. */
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (long i = 0; i < n; i++) deposit_one(d, rec + MO_REC * i, J, rho, 1);
}

long mo_erase_outside(double zmin, double Lz, double zp0, double zp1, double* rec, long n) {
  long w = 0;
  for (long i = 0; i < n; i++) {
    double zr = mo_pmod(rec[MO_REC * i + 3] - zmin, Lz) + zmin;
    if (zr < zp0 || zr >= zp1) continue;
    if (w != i) memcpy(rec + MO_REC * w, rec + MO_REC * i, MO_REC * sizeof(double));
    w++;
  }
  return w;
}

/* ------------------------------------------------------------------------------------------ */
/* Radiated power, src/radiation.cpp:127-232.                                                  */
/* ------------------------------------------------------------------------------------------ */

void mo_power_sample(const mo_power* p, unsigned nTime, const float* en, const float* bn, double* pG) {
  const long N0 = p->N0, N1 = p->N1, N1N0 = N1 * N0;
  const unsigned slot = nTime % (unsigned)p->Nf;
  long nodes_per_plane = N1N0;
  int kz = 0;
  for (int k = 0; k < p->N; k++)
    for (int l = 0; l < p->Nl; l++) pG[k * p->Nl + l] = 0.0;
  for (int k = 0; k < p->N; k++) {
    if (!(p->z[k] < p->zp1 && p->z[k] >= p->zp0)) continue;
    double c;
    double dzr = modf((p->z[k] - p->zmin) / p->dz, &c);
    int kk = (int)c;
    for (long i = 2; i < N0 - 2; i++)
      for (long j = 2; j < N1 - 2; j++) {
        long mi = (long)(kk - p->k0) * N1N0 + i * N1 + j;
        long ni = (long)kz * N1N0 + i * N1 + j;
        double et0 = (1.0 - dzr) * en[3 * mi + 0] + dzr * en[3 * (mi + N1N0) + 0];
        double et1 = (1.0 - dzr) * en[3 * mi + 1] + dzr * en[3 * (mi + N1N0) + 1];
        double bt0 = (1.0 - dzr) * bn[3 * mi + 0] + dzr * bn[3 * (mi + N1N0) + 0];
        double bt1 = (1.0 - dzr) * bn[3 * mi + 1] + dzr * bn[3 * (mi + N1N0) + 1];
        double* f = p->fdt + ((size_t)slot * (size_t)(p->N * nodes_per_plane) + (size_t)ni) * 4;
        f[0] = p->gamma * (et0 + p->c0 * p->beta * bt1);
        f[1] = p->gamma * (et1 - p->c0 * p->beta * bt0);
        f[2] = p->gamma * (bt0 - p->beta / p->c0 * et1);
        f[3] = p->gamma * (bt1 + p->beta / p->c0 * et0);
        for (int l = 0; l < p->Nl; l++) {
          /* ew1 += fdt0*ep, bw1 += fdt3*em, ew2 += fdt1*ep, bw2 += fdt2*em, with
           * ep = (cos, sin) and em = (cos, -sin): the std::complex products of a real and a
           * complex number are two real multiplies. */
          double ew1r = 0.0, ew1i = 0.0, bw1r = 0.0, bw1i = 0.0, ew2r = 0.0, ew2i = 0.0, bw2r = 0.0, bw2i = 0.0;
          for (int m = 0; m < p->Nf; m++) {
            const double* g = p->fdt + ((size_t)m * (size_t)(p->N * nodes_per_plane) + (size_t)ni) * 4;
            double cr = p->ep_re[l * p->Nf + m], ci = p->ep_im[l * p->Nf + m];
            ew1r += g[0] * cr; ew1i += g[0] * ci;
            bw1r += g[3] * cr; bw1i += g[3] * (-ci);
            ew2r += g[1] * cr; ew2i += g[1] * ci;
            bw2r += g[2] * cr; bw2i += g[2] * (-ci);
          }
          pG[k * p->Nl + l] += p->pc * ((ew1r * bw1r - ew1i * bw1i) - (ew2r * bw2r - ew2i * bw2i));
        }
      }
    kz++;
  }
}

/* ------------------------------------------------------------------------------------------ */
/* Bunch diagnostics.                                                                          */
/* ------------------------------------------------------------------------------------------ */

/* particleInProcessor, src/solver.cpp:2292-2296. */
static int in_processor(double zmin, double Lz, double zp0, double zp1, double z) {
  double zr = mo_pmod(z - zmin, Lz) + zmin;
  return (zr >= zp0) && (zr < zp1);
}

void mo_bunch_sample(double zmin, double Lz, double zp0, double zp1, const double* rec, long n, double* out) {
  double q = 0.0, r[3] = {0, 0, 0}, r2[3] = {0, 0, 0}, gb[3] = {0, 0, 0}, gb2[3] = {0, 0, 0};
  for (long i = 0; i < n; i++) {
    const double* c = rec + MO_REC * i;
    if (!in_processor(zmin, Lz, zp0, zp1, c[3])) continue;
    q += c[0];
    for (int l = 0; l < 3; l++) r[l] += c[0] * c[1 + l];
    for (int l = 0; l < 3; l++) gb[l] += c[0] * c[7 + l];
    for (int l = 0; l < 3; l++) {
      r2[l] += c[1 + l] * c[1 + l] * c[0];
      gb2[l] += c[7 + l] * c[7 + l] * c[0];
    }
  }
  for (int l = 0; l < 3; l++) {
    double rT = r[l] / q, r2T = r2[l] / q, gbT = gb[l] / q, gb2T = gb2[l] / q;
    out[l] = rT;
    out[3 + l] = gbT;
    out[6 + l] = sqrt(r2T - rT * rT);
    out[9 + l] = sqrt(gb2T - gbT * gbT);
  }
}

double mo_bunching_factor(double zmin, double Lz, double zp0, double zp1, const double* rec, long n, double k) {
  double q = 0.0, cr = 0.0, ci = 0.0;
  for (long i = 0; i < n; i++) {
    const double* c = rec + MO_REC * i;
    if (!in_processor(zmin, Lz, zp0, zp1, c[3])) continue;
    q += c[0];
    cr += c[0] * cos(k * c[3]);
    ci += c[0] * sin(k * c[3]);
  }
  return q != 0.0 ? sqrt(cr * cr + ci * ci) / q : 0.0;
}

/* Solver::interp, src/solver.cpp:2283-2286. */
static double screen_interp(double x0, double x1, double y0, double y1, double x) {
  return y0 + (x - x0) / (x1 - x0) * (y1 - y0);
}

/* Solver::screenProfile, src/solver.cpp:2205-2257: the step runs from timeBunch - dt to timeBunch
 * with the particle at rnm and rnp; x, y and the lab time are interpolated linearly in the lab z
 * to the screen, the momentum is the one after the step (stair-case). */
long mo_screen_profile(const mo_screen* s, const double* lz_screen, int n_screens, double time_bunch,
                       const double* rec, long n, double* out, long cap) {
  long w = 0;
  for (int i = 0; i < n_screens; i++) {
    const double lzs = lz_screen[i];
    for (long p = 0; p < n; p++) {
      const double* c = rec + MO_REC * p;
      if (!in_processor(s->zmin, s->Lz, s->zp0, s->zp1, c[3])) continue;
      const double lzm = s->gamma * (c[6] + s->beta * s->c0 * (time_bunch - s->dt + s->dt_shift));
      if (lzm >= lzs) continue;
      const double lzp = s->gamma * (c[3] + s->beta * s->c0 * (time_bunch + s->dt_shift));
      if (lzp < lzs) continue;
      if (w < cap) {
        double* o = out + 7 * w;
        o[0] = screen_interp(lzm, lzp, c[4], c[1], lzs);
        o[1] = screen_interp(lzm, lzp, c[5], c[2], lzs);
        const double tm = s->gamma * (time_bunch + s->dt_shift - s->dt + s->beta / s->c0 * c[6]);
        const double tp = s->gamma * (time_bunch + s->dt_shift + s->beta / s->c0 * c[3]);
        o[2] = screen_interp(lzm, lzp, tm, tp, lzs);
        o[3] = c[7];
        o[4] = c[8];
        o[5] = s->gamma * (c[9] + s->beta * sqrt(1.0 + (c[7] * c[7] + c[8] * c[8] + c[9] * c[9])));
        o[6] = (double)p;
      }
      w++;
    }
  }
  return w;
}

void mo_field_sample(const mo_field* f, const double* an, const float* en, const float* bn, const double* pts,
                     long n, double* out) {
  const long N1 = f->N1, N1N0 = (long)f->N1 * f->N0;
  for (long p = 0; p < n; p++) {
    const double* r = pts + 3 * p;
    double c1;
    double dxr = modf((r[0] - f->xmin) / f->dx, &c1); int i = (int)c1;
    double dyr = modf((r[1] - f->ymin) / f->dy, &c1); int j = (int)c1;
    double dzr = modf((r[2] - f->zmin) / f->dz, &c1); int k = (int)c1;
    long m = (long)(k - f->k0) * N1N0 + (long)i * N1 + j;
    const long nd[8] = {m, m + N1, m + 1, m + N1 + 1, m + N1N0, m + N1N0 + N1, m + N1N0 + 1, m + N1N0 + N1 + 1};
    const double w[8] = {(1.0 - dxr) * (1.0 - dyr) * (1.0 - dzr), dxr * (1.0 - dyr) * (1.0 - dzr),
                         (1.0 - dxr) * dyr * (1.0 - dzr),         dxr * dyr * (1.0 - dzr),
                         (1.0 - dxr) * (1.0 - dyr) * dzr,         dxr * (1.0 - dyr) * dzr,
                         (1.0 - dxr) * dyr * dzr,                 dxr * dyr * dzr};
    double* o = out + 9 * p;
    for (int c = 0; c < 3; c++) {
      o[c] = w[0] * en[3 * nd[0] + c];
      o[3 + c] = w[0] * bn[3 * nd[0] + c];
      o[6 + c] = w[0] * an[3 * nd[0] + c];
    }
    for (int q = 1; q < 8; q++)
      for (int c = 0; c < 3; c++) {
        o[c] += w[q] * en[3 * nd[q] + c];
        o[3 + c] += w[q] * bn[3 * nd[q] + c];
        o[6 + c] += w[q] * an[3 * nd[q] + c];
      }
  }
}
