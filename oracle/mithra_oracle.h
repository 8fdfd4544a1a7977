/*
 * CPU restatement of the MITHRA FdTd time-marching loop, in plain C.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle that the CUDA path is checked against.
 * Only tests/, __graft_entry__.smoke() and the CPU-baseline legs of bench.py may load it.
 * The product library never links, loads or calls it.
 *
 * Layout follows the reference exactly so that its state can be compared with dumps of
 * the reference itself: vector fields are arrays of N1N0*np records of 3 doubles, node
 * m = N1N0*k + N1*i + j (src/solver.cpp:674, :2302-2315); particles are records of 11
 * doubles  q, rnp[3], rnm[3], gb[3], e  (src/stdinclude.h:130-144).
 *
 * Every function states the reference lines it restates.  The arithmetic is written in
 * the reference's order so that, compiled with -ffp-contract=off, it reproduces the
 * reference's rounding.
 */
#ifndef MITHRA_ORACLE_H
#define MITHRA_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MO_REC 11          /* doubles per particle record */
#define MO_MAX_UND 64
#define MO_MAX_EXT 16

/* Signal (src/classes.h:159-195): type 0 neumann, 1 gaussian, 2 secant, 3 flat-top,
 * 4 inverse-gaussian; cep in radians, f0 = 1/l as set by Signal::initialize. */
typedef struct {
  int type;
  double t0, s, f0, cep, nR, sig0, sig1;
} mo_signal;

/* The laser-beam part shared by Seed, optical Undulator and ExtField (src/classes.h:201-462).
 * type: SeedType 0 plane-wave, 1 truncated plane-wave, 2 gaussian, 3 super-gaussian,
 * 4..7 their standing variants.  l and zR are the members l_, zR_ set by initialize. */
typedef struct {
  int type;
  double position[3], direction[3], polarization[3];
  double amplitude, radius[2];
  int order[2];
  double l, zR[2];
  mo_signal signal;
} mo_beam;

/* Seed with the frame parameters that Seed::fields uses (src/classes.cpp:740-855). */
typedef struct {
  mo_beam beam;
  double gamma, beta, c0, dt;
} mo_seed;

typedef struct {
  int N0, N1, np, k0;       /* nodes along x, y, and along z in this domain */
  int solver;               /* 0 = FD, 1 = NSFD */
  int order;                /* Mur truncation order, 1 or 2 */
  int space_charge;         /* 1: also advance the scalar potential */
  double a[6];              /* uf_.a */
  double nsfd_alpha, nsfd_beta;  /* uf_.af.alpha_, uf_.af.beta_ (= beta/alpha) */
  double bB[5], cB[5], dB[5];
  double eE[5], fE[5], gE[5];
  double hC[17];
  double dt, dx, dy, dz;
  double xmin, ymin, zmin;  /* node (0,0,0) position, for the TF/SF seed points rc(m) */
} mo_field;

typedef struct {
  int type;                 /* 0 static, 1 optical */
  double k, lu, rb, length, dist, theta;
  mo_beam beam;             /* the optical undulator's laser beam */
} mo_undulator;

typedef struct {
  int N0, N1, np, k0;
  double xmin, xmax, ymin, ymax, zmin, zmax, zp0, zp1, Lz;
  double dx, dy, dz;
  double dtb;               /* ub_.dtb = c0 * bunch time step */
  double r1, r2;            /* ub_.r1, ub_.r2 */
  double gamma, beta, c0, dt_shift;  /* gamma_, beta_, c0_, dt_ */
  int n_und;
  mo_undulator und[MO_MAX_UND];
  int n_ext;                /* EXTERNAL-FIELD entries (src/solver.cpp:1886-1947) */
  mo_beam ext[MO_MAX_EXT];
} mo_push;

typedef struct {
  int N0, N1, np, k0;
  double xmin, ymin, zmin, xmax, ymax;
  double dx, dy, dz;
  double dv, rc;            /* uc_.dv, uc_.rc (unused by the deposit itself) */
  double zp0, zp1, Lz;
} mo_deposit;

typedef struct {
  int N0, N1, np, k0;
  int N;                    /* sampling planes */
  int Nl, Nf;
  double zmin, dz, zp0, zp1, gamma, beta, c0, pc;
  const double* z;          /* N boosted plane positions */
  const double* ep_re;      /* Nl*Nf twiddles cos(w j dt) */
  const double* ep_im;      /* Nl*Nf twiddles sin(w j dt) */
  double* fdt;              /* Nf * Nz * N1N0 * 4 ring buffer (state) */
} mo_power;

/* One FdTd::fieldUpdate without the MPI halo (src/fdtd.cpp:231-725): interior FD/NSFD update
 * of A (J is read from anp1 in place), Mur faces, and for order 2 edges and corners. */
void mo_field_update(const mo_field* f, double* anp1, const double* an, const double* anm1);

/* mo_field_update with the TF/SF injection of the seed (src/fdtd.cpp:307-373) between the
 * interior update and the Mur boundaries; `time` is time_ of the step.  seed == NULL or an
 * amplitude not above 1e-50 injects nothing, as in the reference. */
void mo_field_update_seeded(const mo_field* f, const mo_seed* seed, double time, double* anp1, const double* an,
                            const double* anm1);

/* Seed::fields (src/classes.cpp:740-855) at one bunch-frame point.  `a` is an accumulator as
 * in the reference: plane-wave and gaussian seeds overwrite it, the super-gaussian adds to it. */
void mo_seed_fields(const mo_seed* s, const double r[3], double time, double a[3]);

/* The scalar-potential counterpart used with space charge (src/fdtdSC.cpp:260-1087):
 * interior update with rho read from fnp1 in place, Mur faces, edges, corners. */
void mo_scalar_update(const mo_field* f, double* fnp1, const double* fn, const double* fnm1);

/* FdTd::fieldEvaluate applied to every interior node (src/fdtd.cpp:818-845) and the copies of
 * planes k=1, np-2 into k=0, np-1 (src/fdtd.cpp:742-774).  With fn != NULL the space-charge
 * electric field -grad(phi) is added as in src/fdtdSC.cpp:1110-1140. */
void mo_eval_eb(const mo_field* f, const double* anp1, const double* an, const double* fn,
                float* en, float* bn);

/* One Solver::bunchUpdate over all particles (src/solver.cpp:1424-1576) with the undulator
 * fields (static: src/solver.cpp:1798-1824, src/beam.cc:14-76; optical: src/solver.cpp:1825-1878)
 * and the external fields (src/solver.cpp:1886-1947, src/beam.cc:80-496).  Particles that cross a z
 * face are appended again, as the single-rank self-exchange does (src/solver.cpp:1544-1568).
 * Returns the new particle count (<= cap), or -1 when cap would be exceeded. */
long mo_push_substep(const mo_push* p, double timeBunch, double* rec, long n, long cap,
                     const float* en, const float* bn, long* n_transverse_out);

/* FdTd::currentUpdate (src/fdtd.cpp:38-185): zigzag deposit into J (which must be zeroed
 * first, src/fdtd.cpp:23-32).  With rho != NULL also the charge deposit of
 * src/fdtdSC.cpp:140-161. */
void mo_deposit_current(const mo_deposit* d, const double* rec, long n, double* J, double* rho);

/* The particle erasure of FdTd::currentCommunicate / Solver::recycleParticles
 * (src/fdtd.cpp:214-224, src/solver.cpp:493-503, :2292-2296).  Returns the new count. */
long mo_erase_outside(double zmin, double Lz, double zp0, double zp1, double* rec, long n);

/* Solver::powerSample for one FEL output (src/radiation.cpp:127-232).  nTime selects the ring
 * slot.  Writes N*Nl powers into pG. */
void mo_power_sample(const mo_power* p, unsigned nTime, const float* en, const float* bn, double* pG);

/* FdTd::fieldSample (src/fdtd.cpp:851-950) at n points (x, y, z): out[9 p ..] = E (from en),
 * B (from bn), A^n (from an), trilinear with the weights of the reference. */
void mo_field_sample(const mo_field* f, const double* an, const float* en, const float* bn, const double* pts,
                     long n, double* out);

/* Solver::bunchSample (src/solver.cpp:1582-1635) for one domain: out[0..2] <r>, [3..5] <gb>,
 * [6..8] rms r, [9..11] rms gb, summed in particle order as the reference does. */
void mo_bunch_sample(double zmin, double Lz, double zp0, double zp1, const double* rec, long n, double* out);

/* |sum q exp(i k z)| / sum q over the particles of the domain, in particle order. */
double mo_bunching_factor(double zmin, double Lz, double zp0, double zp1, const double* rec, long n, double k);

/* Lab-frame screen crossing of Solver::screenProfile (src/solver.cpp:2205-2257). */
typedef struct {
  double gamma, beta, c0;   /* moving frame */
  double dt_shift;          /* dt_ */
  double dt;                /* mesh_.timeStep_ */
  double zmin, Lz, zp0, zp1;
} mo_screen;

/* Solver::screenProfile for one domain, after the substeps of a step that ends at time_bunch:
 * for each screen (lab z, in the given order) and each particle of the list (in order) whose lab
 * z passes the screen during the step, one row (x, y, t, gbx, gby, gbz_lab, list index) in out.
 * Returns the number of rows (at most cap are written). */
long mo_screen_profile(const mo_screen* s, const double* lz_screen, int n_screens, double time_bunch,
                       const double* rec, long n, double* out, long cap);

/* Thread count used by the parallel loops (1 = serial, bitwise reproduction of the reference). */
void mo_set_threads(int n);
int mo_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
