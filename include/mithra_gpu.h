/*
 * mithra_gpu.h : C ABI of the GB300 FdTd/FdTdSC time-marching library (libmithra_gb300.so).
 *
 * The reference selects its solver at src/mithra.cpp:86-93 and drives it through the virtual
 * interface of MITHRA::Solver (src/solver.h:139-178) plus the non-virtual Solver::solve and
 * Solver::bunchUpdate (src/solver.h:75-78).  This ABI is what that interface needs from a
 * device: an opaque context that owns all device memory, entry points for each stage of one
 * field step, and a fused multi-step march.  Plain pointers and sizes only; no C++ types cross
 * it and no pointer passed in is retained after a call returns.
 *
 * Host buffers use the reference's own layouts:
 *   vector fields : N1N0*N2 records of 3 doubles, node m = N1N0*k + N1*i + j (src/solver.cpp:674)
 *   E and B       : N1N0*N2 records of 3 floats (src/solver.h:244-245)
 *   particles     : records of 11 doubles  q, rnp[3], rnm[3], gb[3], e  (src/stdinclude.h:130-144,
 *                   the MPI_CHARGE datatype of src/solver.cpp:55)
 *
 * Every call returns MITHRA_OK (0) or a negative status; mithra_gpu_last_error() gives the text.
 * A context is used by one host thread at a time and owns one CUDA stream.
 */
#ifndef MITHRA_GPU_H
#define MITHRA_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MITHRA_OK 0
#define MITHRA_ERR_ARG (-1)        /* invalid argument or size */
#define MITHRA_ERR_CUDA (-2)       /* CUDA runtime failure */
#define MITHRA_ERR_CAPACITY (-3)   /* particle capacity exceeded */
#define MITHRA_ERR_STATE (-4)      /* call out of order (e.g. no particles uploaded) */
#define MITHRA_ERR_NONFINITE (-5)  /* NaN or Inf detected in the state */
#define MITHRA_ERR_PARSE (-6)      /* job file could not be parsed */

#define MITHRA_PRECISION_FP64 0    /* plain form: FP64 throughout, E/B stored as float */
#define MITHRA_PRECISION_FP32 1    /* mixed form: FP32 fields/particles, FP64 phase and frames */

#define MITHRA_MAX_UNDULATORS 64
#define MITHRA_MAX_POWER_OUTPUTS 8
#define MITHRA_MAX_EXT_FIELDS 16

typedef struct mithra_ctx mithra_ctx;

/* Mesh, solver and field-update coefficients: the values Solver::initializeMesh and
 * Solver::initializeField compute (src/solver.cpp:601-842). */
typedef struct {
  int32_t N0, N1, N2;          /* nodes along x, y, z */
  int32_t solver;              /* 0 = FD, 1 = NSFD (src/stdinclude.h:40) */
  int32_t truncation_order;    /* Mur order, 1 or 2 */
  int32_t space_charge;        /* 1 selects the FdTdSC path */
  double a[6];                 /* uf_.a */
  double nsfd_alpha, nsfd_beta;/* uf_.af.alpha_, uf_.af.beta_ */
  double bB[5], cB[5], dB[5];  /* Mur face coefficients */
  double eE[5], fE[5], gE[5];  /* Mur edge coefficients */
  double hC[17];               /* Mur corner coefficients */
  double dt, dx, dy, dz;       /* field time step and boosted mesh resolution */
  double xmin, xmax, ymin, ymax, zmin, zmax;
  double zp0, zp1;             /* z range owned by the (single) domain, src/solver.cpp:676-683 */
  double Lz;                   /* boosted mesh length along z */
} mithra_grid_desc;

/* Particle-update constants: Solver::initializeBunchUpdate and the frame parameters
 * (src/solver.cpp:1050-1059, :191-213, :322). */
typedef struct {
  double dtb;                  /* ub_.dtb = c0 * bunch time step */
  double bunch_time_step;      /* bunch_.timeStep_ (the timeBunch increment) */
  double r1, r2;               /* ub_.r1, ub_.r2 */
  double gamma, beta, c0;      /* moving-frame gamma_, beta_, c0_ */
  double dt_shift;             /* dt_ */
  double n_update_bunch;       /* nUpdateBunch_ (the substep loop runs while t < this) */
} mithra_push_desc;

/* A laser beam after Seed/Undulator/ExtField::initialize (src/classes.cpp:646-735, :1007-1075,
 * :1162-1260): the members of those classes that the field evaluation reads. */
typedef struct {
  int32_t type;                /* SeedType: 0 plane-wave, 1 truncated plane-wave, 2 gaussian,
                                  3 super-gaussian, 4..7 the standing variants of 0..3 */
  double position[3], direction[3], polarization[3];
  double amplitude;            /* amplitude_ */
  double radius[2];            /* radius_ */
  int32_t order[2];            /* order_ */
  double wavelength;           /* l_ */
  double rayleigh[2];          /* zR_ */
  int32_t signal_type;         /* 0 neumann, 1 gaussian, 2 secant-hyperbolic, 3 flat-top,
                                  4 inverse-gaussian */
  double signal_t0, signal_s, signal_f0, signal_cep, signal_nr;  /* Signal t0_, s_, f0_, cep_, nR_ */
  double signal_sigma[2];      /* Signal sigmaInvG_ */
} mithra_beam_desc;

/* The seed of FdTd::fieldUpdate's TF/SF injection (src/fdtd.cpp:307-373, Seed::fields
 * src/classes.cpp:740-855) with the frame members of Seed. */
typedef struct {
  mithra_beam_desc beam;
  double gamma, beta, c0, dt;  /* Seed gamma_, beta_, c0_, dt_ */
} mithra_seed_desc;

/* One undulator module after Solver::setSimulationParameters (sorted, rb shifted).  An optical
 * undulator (type 1) also carries its laser beam. */
typedef struct {
  int32_t type;                /* 0 static, 1 optical */
  double k, lu, rb, length, dist, theta;
  mithra_beam_desc beam;       /* used when type == 1 */
} mithra_undulator_desc;

/* One radiation-power output (src/radiation.cpp:18-121). */
typedef struct {
  int32_t N;                   /* sampling planes */
  int32_t Nl;                  /* frequencies */
  int32_t Nf;                  /* DFT length (ring slots) */
  double pc;                   /* power constant */
  const double* z;             /* N boosted plane positions */
  const double* twiddle_re;    /* Nl*Nf values cos(w_l * j * dt) */
  const double* twiddle_im;    /* Nl*Nf values sin(w_l * j * dt) */
} mithra_power_desc;

/* Time state of Solver (src/solver.h:253-268). */
typedef struct {
  double time, time_bunch;
  int64_t n_time, n_time_bunch;
} mithra_time_state;

/* ---- context ---------------------------------------------------------------------------- */

/* Replaces `new FdTd(...)` / `new FdTdSC(...)` (src/mithra.cpp:86-90) once the host has run the
 * reference's initialisation.  `particle_capacity` bounds the particle count including the
 * copies the single-domain z-face exchange appends (src/solver.cpp:1551-1568). */
int mithra_gpu_create(const mithra_grid_desc* grid, const mithra_push_desc* push, int precision,
                      int device, size_t particle_capacity, mithra_ctx** out);
int mithra_gpu_destroy(mithra_ctx* ctx);
int mithra_gpu_last_error(const mithra_ctx* ctx, char* buf, size_t len);
int mithra_gpu_synchronize(mithra_ctx* ctx);

/* Undulator modules, replacing the parsed std::vector<Undulator> (src/solver.h:224). */
int mithra_gpu_set_undulators(mithra_ctx* ctx, const mithra_undulator_desc* und, int n);
/* The seed injected through the total-field/scattered-field planes every field update
 * (Solver::seed_, src/solver.h:223; src/fdtd.cpp:307-373).  An amplitude not above 1e-50, or
 * seed == NULL, injects nothing, as in the reference. */
int mithra_gpu_set_seed(mithra_ctx* ctx, const mithra_seed_desc* seed);
/* External laser fields acting on the particles (Solver::extField_, src/solver.h:225;
 * Solver::externalField, src/solver.cpp:1886-1947).  At most MITHRA_MAX_EXT_FIELDS. */
int mithra_gpu_set_external_fields(mithra_ctx* ctx, const mithra_beam_desc* fields, int n);
/* Radiation-power outputs, replacing Solver::initializePowerSample's rp_ (src/radiation.cpp:18-121). */
int mithra_gpu_set_power(mithra_ctx* ctx, const mithra_power_desc* outputs, int n);

/* ---- state transfer --------------------------------------------------------------------- */

/* Fields anp1_ (which holds J between steps), an_, anm1_ (src/solver.h:231-233); any may be NULL. */
int mithra_gpu_upload_fields(mithra_ctx* ctx, const double* anp1, const double* an, const double* anm1);
int mithra_gpu_download_fields(mithra_ctx* ctx, double* anp1, double* an, double* anm1);
/* Scalar potential fnp1_ (rho between steps), fn_, fnm1_ (src/solver.h:236-238), FdTdSC only. */
int mithra_gpu_upload_scalar(mithra_ctx* ctx, const double* fnp1, const double* fn, const double* fnm1);
int mithra_gpu_download_scalar(mithra_ctx* ctx, double* fnp1, double* fn, double* fnm1);
/* E and B as evaluated by the last field step (src/solver.h:244-245). */
int mithra_gpu_download_eb(mithra_ctx* ctx, float* en, float* bn);
/* chargeVectorn_ (src/solver.h:271) as 11-double records. */
int mithra_gpu_upload_particles(mithra_ctx* ctx, const double* rec, size_t n);
/* The same from records already in device memory (on the context's device). */
int mithra_gpu_upload_particles_device(mithra_ctx* ctx, const double* dev_rec, size_t n);
int mithra_gpu_download_particles(mithra_ctx* ctx, double* rec, size_t cap, size_t* n);
int mithra_gpu_particle_count(mithra_ctx* ctx, size_t* n);
int mithra_gpu_set_time(mithra_ctx* ctx, const mithra_time_state* t);
int mithra_gpu_get_time(mithra_ctx* ctx, mithra_time_state* t);

/* ---- stages of one field step (each replaces one reference member function) ------------- */

/* FdTd::fieldUpdate / FdTdSC::fieldUpdate without the MPI halo, plus the eager equivalent of
 * the lazy FdTd::fieldEvaluate (src/fdtd.cpp:231-800, :818-845). */
int mithra_gpu_field_update(mithra_ctx* ctx);
/* FdTd::fieldEvaluate (src/fdtd.cpp:818-845) at every interior node from the current anp1/an,
 * plus the plane copies of src/fdtd.cpp:755-772; field_update already includes it. */
int mithra_gpu_field_evaluate(mithra_ctx* ctx);
/* `rnm = rnp` for all particles (src/solver.cpp:1311-1312). */
int mithra_gpu_save_positions(mithra_ctx* ctx);
/* One Solver::bunchUpdate (src/solver.cpp:1424-1576) followed by timeBunch_ += bunch time step
 * and ++nTimeBunch_ (src/solver.cpp:1319-1320). */
int mithra_gpu_bunch_update(mithra_ctx* ctx);
/* Solver::recycleParticles (src/solver.cpp:493-503). */
int mithra_gpu_recycle(mithra_ctx* ctx);
/* Solver::bunchSample (src/solver.cpp:1582-1635) over the particles of this domain: row[0] =
 * timeBunch_, row[1..3] <r>, row[4..6] <gb>, row[7..9] rms r, row[10..12] rms gb (charge-weighted;
 * compensated FP64 sums). */
int mithra_gpu_bunch_sample(mithra_ctx* ctx, double* row);
/* FdTd::fieldSample (src/fdtd.cpp:851-950) at n points (x, y, z in the bunch frame): out[9 p ..]
 * = E, B, A^n interpolated with the reference's trilinear weights (boosted-frame values; the
 * reference's file adds the lab transform and unit factors).  Evaluates E/B on every interior
 * node first; points outside the mesh give NaN. */
int mithra_gpu_field_sample(mithra_ctx* ctx, const double* points, size_t n, double* out);
/* Bunching factor |sum q exp(i k z)| / sum q at wavenumber k (bunch-frame z), the quantity read
 * from the reference's bunch dumps (Solver::bunchProfile, src/solver.cpp:1763-1792). */
int mithra_gpu_bunching_factor(mithra_ctx* ctx, double k, double* b);
/* Lab-frame screens, Solver::screenProfile (src/solver.cpp:2205-2257), screens from
 * initializeScreenProfile (src/solver.cpp:2145-2199): from now on every step (and every step of
 * mithra_gpu_run_prelude) records the particles whose lab z passes one of the n screens lz[]
 * (um from the undulator start, in the order given).  capacity = records kept per screen (0:
 * the particle capacity of the context); further crossings are counted and reported by
 * mithra_gpu_screen_records as MITHRA_ERR_CAPACITY.  n = 0 removes the screens.  Replaces the
 * files the reference opens per screen: their rows come from mithra_gpu_screen_records. */
int mithra_gpu_set_screens(mithra_ctx* ctx, const double* lz, int n, long long capacity);
/* Solver::screenProfile for the current step alone (the stage-wise form of what every step of
 * mithra_gpu_run does when screens are set). */
int mithra_gpu_screen_profile(mithra_ctx* ctx);
/* Drops the records collected so far (the screens stay). */
int mithra_gpu_screen_clear(mithra_ctx* ctx);
/* Records of screen `screen` in the reference's file order (steps in order, particles in list
 * order): out[7 r ..] = x, y, t (lab, interpolated to the screen), gbx, gby, gbz (lab), nTime_
 * of the step.  out = NULL returns the count in *n_rows. */
int mithra_gpu_screen_records(mithra_ctx* ctx, int screen, double* out, long long cap_rows, long long* n_rows);
/* Solver::powerSample (src/radiation.cpp:127-232); the row is appended to the device row log. */
int mithra_gpu_power_sample(mithra_ctx* ctx);
/* mithra_gpu_power_sample without any device allocation.  No counterpart in the reference: it
 * serves callers that cannot allocate device memory at this point (all of it already given to
 * fields and particles, or no device-wide synchronisation allowed while other streams run).
 * The per-block partial sums go to one fixed 1 MiB array per device (131072 doubles, shared by
 * every context on the device and needing no zeroing); an output that needs more
 * (planes x blocks per plane x frequencies) is refused with MITHRA_ERR_CAPACITY, and so is a
 * call when the row log is full (drain it with mithra_gpu_power_rows).  Each call looks up the
 * array's address on the context's device; the first call on a device may load the module, so
 * make one call before any stream capture.  Calls that overlap in time on one device race on
 * the shared array. */
int mithra_gpu_power_sample_noalloc(mithra_ctx* ctx);
/* FdTd::fieldShift (src/fdtd.cpp:806-812). */
int mithra_gpu_field_shift(mithra_ctx* ctx);
/* FdTd::currentReset + currentUpdate + currentCommunicate (src/fdtd.cpp:23-225). */
int mithra_gpu_current_update(mithra_ctx* ctx);
/* time_ += dt, ++nTime_ (src/solver.cpp:1396-1399). */
int mithra_gpu_advance_time(mithra_ctx* ctx);

/* ---- fused march ------------------------------------------------------------------------ */

/* `nsteps` iterations of the body of Solver::solve's main loop (src/solver.cpp:1300-1414),
 * replayed from CUDA graphs with no host synchronisation between steps. */
int mithra_gpu_run(mithra_ctx* ctx, int64_t nsteps);
/* mithra_gpu_run bracketed by CUDA events recorded on the context's stream; returns the device
 * time of the `nsteps` steps in milliseconds (the stream is synchronised). */
int mithra_gpu_run_timed(mithra_ctx* ctx, int64_t nsteps, double* device_ms);
/* Number of kernels the library launches for one field step of this context. */
int mithra_gpu_launches_per_step(mithra_ctx* ctx, int* n);
/* The negative-time particle loop of Solver::solve (src/solver.cpp:1232-1291): field-free
 * substeps while time_ < 0. */
int mithra_gpu_run_prelude(mithra_ctx* ctx);

/* Power rows recorded since the last call (or since creation): for each row and output, per
 * plane the lab-frame z followed by Nl powers, as written to power-sampling files
 * (src/radiation.cpp:222-229).  `*n_values` returns the number of doubles written. */
int mithra_gpu_power_rows(mithra_ctx* ctx, double* out, size_t cap_values, size_t* n_values);

/* Per-kernel device time accumulated since the last reset (CUDA events on the context stream).
 * names/ms are filled for up to `cap` kernels; returns the count through *n. */
int mithra_gpu_kernel_times(mithra_ctx* ctx, char* names, size_t name_len, double* ms, int cap, int* n);
int mithra_gpu_enable_timing(mithra_ctx* ctx, int on);

/* Page-locked host buffers for transfers that overlap with device work (cudaMallocHost). */
int mithra_host_alloc(size_t bytes, void** p);
int mithra_host_free(void* p);

/* Measured FP64 fused multiply-add rate of `device` in TFLOP/s (an FMA counts two), from a short
 * kernel of independent FMA chains on every SM (no counterpart in the reference).  The FP64 form
 * of the loop is bound by this rate on GB300; the bench reports its kernels against it. */
int mithra_probe_fp64_tflops(int device, double* tflops);

/* ---- job-file level entry points (host initialisation of the reference, then a context) --- */

/* Parses a MITHRA job file (src/readdata.cpp:10-53, src/datainput.cpp:18-751) and runs the
 * reference's FP64 initialisation (Solver::initialize, src/solver.cpp:547-595) on the host.
 * The setup object holds the descriptors above, the initial fields and the particles. */
/* ---- launch shapes ------------------------------------------------------------------------ */

/* Launch shapes of a context (no counterpart in the reference).  blocks_per_sm caps the grid of
 * the particle and boundary kernels (grid-stride loops); slab_planes is the z extent of the tiles
 * of the mixed form's bulk-tensor stencil.  Results do not depend on them beyond the order of
 * atomic additions. */
typedef struct {
  int32_t blocks_per_sm;       /* 2 .. 64, default 16 */
  int32_t slab_planes;         /* 16 .. 256, default 64 */
} mithra_tuning;
int mithra_gpu_set_tuning(mithra_ctx* ctx, const mithra_tuning* t);
int mithra_gpu_get_tuning(const mithra_ctx* ctx, mithra_tuning* t);
/* Times every candidate shape on `steps_per_trial` real field steps of the march (the steps are
 * part of the simulation) and keeps the fastest; writes the chosen shape and its ms per step. */
int mithra_gpu_autotune(mithra_ctx* ctx, int steps_per_trial, mithra_tuning* chosen, double* ms_per_step);
/* Attempts of each bounded barrier wait in the mixed form's bulk-tensor stencil before it gives
 * up (no counterpart in the reference; a negative value restores the default of 2e7, 0 makes
 * every wait give up at once).  A CTA whose wait gives up waits, with the default limit, for the
 * copies it issued, leaves its planes unwritten, and the next call that checks the device state
 * returns MITHRA_ERR_STATE; the error stays set for the context.  Small values exist to
 * exercise that path. */
int mithra_gpu_set_wait_limit(mithra_ctx* ctx, int64_t iterations);

/* ---- batched instances ---------------------------------------------------------------------- */

/* Several independent contexts on one device (a parameter sweep: each with its own mesh, bunch
 * and undulator) stepped together: every field step of all instances is one CUDA graph launch,
 * the per-instance step graphs being child graphs of it, so the instances' kernels run
 * concurrently.  No counterpart in the reference (one job per run).  The contexts must be in the
 * same step phase (buffer rotation and sort parity: contexts created and stepped together are). */
typedef struct mithra_batch mithra_batch;
int mithra_batch_create(mithra_ctx* const* ctxs, int n, mithra_batch** out);
int mithra_batch_run(mithra_batch* b, int64_t nsteps);
int mithra_batch_run_timed(mithra_batch* b, int64_t nsteps, double* device_ms);
int mithra_batch_destroy(mithra_batch* b);

typedef struct mithra_setup mithra_setup;
int mithra_setup_from_job(const char* job_path, mithra_setup** out, char* err, size_t err_len);
int mithra_setup_destroy(mithra_setup* s);
int mithra_setup_grid(const mithra_setup* s, mithra_grid_desc* grid);
int mithra_setup_push(const mithra_setup* s, mithra_push_desc* push);
int mithra_setup_undulators(const mithra_setup* s, mithra_undulator_desc* und, int cap, int* n);
int mithra_setup_seed(const mithra_setup* s, mithra_seed_desc* seed);
int mithra_setup_external_fields(const mithra_setup* s, mithra_beam_desc* fields, int cap, int* n);
int mithra_setup_time(const mithra_setup* s, mithra_time_state* t);
/* The o-th radiation-power output as mithra_gpu_set_power takes it (Solver::initializePowerSample,
 * src/radiation.cpp:18-121: planes, frequencies, DFT length, power constant, boosted plane
 * positions, twiddles); the arrays belong to the setup.  *n returns the number of outputs, and
 * out = NULL asks for that number only. */
int mithra_setup_power(const mithra_setup* s, int o, mithra_power_desc* out, int* n);
int mithra_setup_particles(const mithra_setup* s, double* rec, size_t cap, size_t* n);
int mithra_setup_fields(const mithra_setup* s, double* anp1, double* an, double* anm1);
int mithra_setup_total_time(const mithra_setup* s, double* total_time);
/* Writes `key value` lines (the derived scalars of the initialisation) into buf. */
int mithra_setup_meta(const mithra_setup* s, char* buf, size_t len, size_t* needed);
/* mithra_setup_from_job with the particle phase of Solver::initialize on GPU `device`:
 * Bunch::initializeEllipsoid (src/classes.cpp:104-298), Solver::lorentzBoostBunch
 * (src/solver.cpp:263-423), distributeParticles and shiftBackInTime run as kernels and the
 * particles stay in device memory (mithra_gpu_create_from_setup takes them without a host copy;
 * mithra_setup_particles downloads them).  Ellipsoid bunches with the Halton generator only;
 * other bunch types are refused with MITHRA_ERR_ARG.  Records agree with the host
 * initialisation to the last place of the device's log/sin/cos. */
int mithra_setup_from_job_device(const char* job_path, int device, mithra_setup** out, char* err, size_t err_len);
/* Base name (directory prefixed, as Solver::initializeSeedVTK, src/solver.cpp:961-964) of the
 * i-th field-visualization output; the other parameters of the outputs are in the meta text
 * (vtk<i>_type, _plane, _rhythm (bunch frame), _pos0..2 (bunch frame), _nfield, _f<l>). */
int mithra_setup_vtk_basename(const mithra_setup* s, int i, char* buf, size_t len, size_t* needed);
/* Base name (directory prefixed, src/radiation.cpp:74-76) of the o-th radiation-power output (the
 * FEL-OUTPUT entries that sample power, in order); its files are <base>-<l>.txt, one per
 * frequency, written by the caller from mithra_gpu_power_rows. */
int mithra_setup_power_basename(const mithra_setup* s, int o, char* buf, size_t len, size_t* needed);
/* Base name (directory prefixed) of the lab-frame screens of FEL-OUTPUT entry jf; their files are
 * <base>-p0-screen<i>.txt, i counting that entry's screens in position order. */
int mithra_setup_screen_basename(const mithra_setup* s, int jf, char* buf, size_t len, size_t* needed);
/* File of the bunch-sampling group (directory prefixed, ".txt"), src/solver.cpp:1066-1068; its
 * rows are mithra_gpu_bunch_sample at the bunch-frame rhythm (meta bunch_rhythm). */
int mithra_setup_bunch_sample_file(const mithra_setup* s, char* buf, size_t len, size_t* needed);
/* File of the field-sampling group, <dir><base>-0.txt (src/solver.cpp:916-918); its points (bunch
 * frame, inside the mesh), fields, rhythm and unit factors are in the meta text (fs_*); a row is
 * time_ gamma_ and, per point, the position and the lab-frame fields of mithra_gpu_field_sample. */
int mithra_setup_field_sample_file(const mithra_setup* s, char* buf, size_t len, size_t* needed);
/* Base name of the bunch-profile dumps (src/solver.cpp:1109); a dump <base>-p0-<nTime>.txt holds
 * time_ gamma_ and q, rnp, gb of every particle (Solver::bunchProfile, src/solver.cpp:1763-1792),
 * written by the caller from mithra_gpu_download_particles at the times and rhythm in the meta text. */
int mithra_setup_bunch_profile_basename(const mithra_setup* s, char* buf, size_t len, size_t* needed);

/* ---- field visualization files ----------------------------------------------------------- */

#define MITHRA_VTK_MAX_FIELDS 16
typedef struct {
  int N0, N1, N2;   /* nodes of the mesh */
  int np, k0;       /* planes of this domain and its first plane (one domain: N2, 0) */
  double xmin, ymin, zmin, dx, dy, dz;  /* bunch frame */
  int type;         /* 0 all-domain, 1 in-plane */
  int plane;        /* in-plane: 0 yz (x normal), 1 xz (y normal), 2 xy (z normal) */
  double position[3];                   /* plane position, bunch frame */
  int nfield;
  int field[MITHRA_VTK_MAX_FIELDS];     /* 0..9 = Ex Ey Ez Bx By Bz Ax Ay Az F */
} mithra_vtk_desc;

/* FdTd::fieldVisualizeAllDomain / fieldVisualizeInPlane (src/fdtd.cpp:956-1540; FdTdSC with F,
 * src/fdtdSC.cpp:1263-1920): writes <basename>-p0-<n_time>.vts and, except for the z-normal
 * plane, <basename>-<n_time>.pvts in the reference's text layout, from host copies of E and B
 * (float, 3 per node), A^n (double, 3 per node) and phi^n (NULL without space charge).  The
 * caller evaluates E/B on every node first (mithra_gpu_field_evaluate + mithra_gpu_download_eb). */
int mithra_vtk_write_field(const mithra_vtk_desc* d, const char* basename, long long n_time, const float* en,
                           const float* bn, const double* an, const double* fn);
/* Creates a context from a setup and uploads its state; the power outputs are configured. */
int mithra_gpu_create_from_setup(const mithra_setup* s, int precision, int device,
                                 double capacity_factor, mithra_ctx** out);

#ifdef __cplusplus
}
#endif
#endif
