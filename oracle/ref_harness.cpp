/*
 * Test harness around the UNMODIFIED reference MITHRA sources (compiled from the reference
 * tree by oracle/Makefile.ref into oracle/_ref/).  Test infrastructure only: it produces
 * golden vectors that pin the C restatement in oracle/ and the host set-up code.
 *
 * Every member of MITHRA::Solver is public (src/solver.h:20-345), so the harness drives
 * the reference's own member functions in the order of Solver::solve
 * (src/solver.cpp:1212-1418) and dumps internal state as raw little-endian arrays:
 *   vec3 arrays : N1N0*np records of 3 doubles (the reference AoS layout, m = N1N0*k+N1*i+j)
 *   particles   : records of 11 doubles  q, rnp[3], rnm[3], gb[3], e  (src/stdinclude.h:130-144)
 *
 * Modes
 *   init    JOB OUT                 initialise (incl. the negative-time particle loop), dump state
 *   run     JOB NSTEPS OUT EVERY    initialise, march NSTEPS field steps, dump every EVERY steps
 *   field   JOB IN OUT              load an/anm1/anp1(=J), FdTd::fieldUpdate, evaluate E/B eagerly
 *   push    JOB IN OUT              load an/anp1/particles/timeBunch, one Solver::bunchUpdate
 *   vtk     JOB N OUT               prelude and N steps with the field sampling and visualization where solve()
 *                                   calls it (the reference writes its .vts/.pvts files into the
 *                                   job's directory); OUT/steps.bin lists the nTime_ of each step
 *   screen  JOB N OUT               prelude and N steps with Solver::screenProfile (and bunchSample,
 *                                   bunchProfile, when the job asks for them) where solve()
 *                                   calls it; the reference writes its own screen files into the
 *                                   job's directory, OUT/offsets.bin holds each screen file's size
 *                                   after the prelude and after every step
 *   deposit JOB IN OUT              load particles, currentReset + currentUpdate (+ currentCommunicate)
 *   power   JOB IN OUT K            K calls of Solver::powerSample on loaded field pairs
 *   bunch   JOB IN OUT              Solver::bunchSample moments of loaded particles
 *   fieldsample JOB IN OUT          FdTd::fieldSample at loaded points on loaded A^n, A^{n+1}
 */
#include <cmath>
#include <cstdio>
#include <fstream>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <list>
#include <sys/stat.h>
#include <unistd.h>

#include "classes.h"
#include "datainput.h"
#include "fdtd.h"
#include "fdtdSC.h"
#include "readdata.h"
#include "solver.h"

using namespace MITHRA;

static std::string jp(const std::string& a, const std::string& b) { return a + "/" + b; }

static void write_raw(const std::string& path, const void* p, size_t bytes) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) { perror(path.c_str()); exit(2); }
  if (bytes && fwrite(p, 1, bytes, f) != bytes) { perror("fwrite"); exit(2); }
  fclose(f);
}
static std::vector<char> read_raw(const std::string& path) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) { perror(path.c_str()); exit(2); }
  fseek(f, 0, SEEK_END); long n = ftell(f); fseek(f, 0, SEEK_SET);
  std::vector<char> b((size_t)n);
  if (n && fread(b.data(), 1, (size_t)n, f) != (size_t)n) { perror("fread"); exit(2); }
  fclose(f);
  return b;
}
static void dump_vec3(const std::string& path, std::vector<FieldVector<double> >* v) {
  write_raw(path, v->data(), v->size() * sizeof(FieldVector<double>));
}
static void load_vec3(const std::string& path, std::vector<FieldVector<double> >* v) {
  std::vector<char> b = read_raw(path);
  if (b.size() != v->size() * sizeof(FieldVector<double>)) { fprintf(stderr, "size mismatch %s\n", path.c_str()); exit(2); }
  memcpy(v->data(), b.data(), b.size());
}
static void dump_scalar_field(const std::string& path, std::vector<double>* v) { write_raw(path, v->data(), v->size() * 8); }
static void load_scalar_field(const std::string& path, std::vector<double>* v) {
  std::vector<char> b = read_raw(path);
  if (b.size() != v->size() * 8) { fprintf(stderr, "size mismatch %s\n", path.c_str()); exit(2); }
  memcpy(v->data(), b.data(), b.size());
}
static void dump_particles(const std::string& path, std::list<Charge>& q) {
  std::vector<double> b; b.reserve(q.size() * 11);
  for (auto& c : q) {
    b.push_back(c.q);
    for (int d = 0; d < 3; d++) b.push_back(c.rnp[d]);
    for (int d = 0; d < 3; d++) b.push_back(c.rnm[d]);
    for (int d = 0; d < 3; d++) b.push_back(c.gb[d]);
    b.push_back(c.e);
  }
  write_raw(path, b.data(), b.size() * 8);
}
static void load_particles(const std::string& path, std::list<Charge>& q) {
  std::vector<char> raw = read_raw(path);
  size_t n = raw.size() / (11 * 8);
  const double* d = (const double*)raw.data();
  q.clear();
  for (size_t i = 0; i < n; i++) {
    Charge c; const double* r = d + 11 * i;
    c.q = r[0];
    for (int k = 0; k < 3; k++) { c.rnp[k] = r[1 + k]; c.rnm[k] = r[4 + k]; c.gb[k] = r[7 + k]; }
    c.e = r[10];
    q.push_back(c);
  }
}

static void meta_line(FILE* f, const char* k, double v) { fprintf(f, "%s %.17g\n", k, v); }

/* The laser-beam members shared by Seed, Undulator and ExtField (src/classes.h:201-462). */
template <class B>
static void beam_meta(FILE* f, const std::string& p, B& b) {
  auto kv = [&](const std::string& k, double v) { meta_line(f, (p + k).c_str(), v); };
  kv("type", (double)b.seedType_);
  for (int c = 0; c < 3; c++) {
    kv("pos" + std::to_string(c), b.position_[c]);
    kv("dir" + std::to_string(c), b.direction_[c]);
    kv("pol" + std::to_string(c), b.polarization_[c]);
  }
  kv("amp", b.amplitude_);
  kv("r0", b.radius_.size() > 0 ? b.radius_[0] : 0.0);
  kv("r1", b.radius_.size() > 1 ? b.radius_[1] : 0.0);
  kv("o0", b.order_.size() > 0 ? b.order_[0] : 0);
  kv("o1", b.order_.size() > 1 ? b.order_[1] : 0);
  kv("l", b.l_);
  kv("zR0", b.zR_.size() > 0 ? b.zR_[0] : 0.0);
  kv("zR1", b.zR_.size() > 1 ? b.zR_[1] : 0.0);
  kv("sig_type", (double)b.signal_.signalType_);
  kv("sig_t0", b.signal_.t0_); kv("sig_s", b.signal_.s_); kv("sig_f0", b.signal_.f0_);
  kv("sig_cep", b.signal_.cep_); kv("sig_nR", (double)b.signal_.nR_);
  kv("sig_g0", b.signal_.sigmaInvG_.size() > 0 ? b.signal_.sigmaInvG_[0] : 0.0);
  kv("sig_g1", b.signal_.sigmaInvG_.size() > 1 ? b.signal_.sigmaInvG_[1] : 0.0);
}

static void dump_meta(Solver* s, const std::string& path) {
  FILE* f = fopen(path.c_str(), "w");
  meta_line(f, "N0", s->N0_); meta_line(f, "N1", s->N1_); meta_line(f, "N2", s->N2_); meta_line(f, "np", s->np_);
  meta_line(f, "k0", s->k0_);
  meta_line(f, "xmin", s->xmin_); meta_line(f, "xmax", s->xmax_);
  meta_line(f, "ymin", s->ymin_); meta_line(f, "ymax", s->ymax_);
  meta_line(f, "zmin", s->zmin_); meta_line(f, "zmax", s->zmax_);
  meta_line(f, "zp0", s->zp_[0]); meta_line(f, "zp1", s->zp_[1]);
  meta_line(f, "dx", s->mesh_.meshResolution_[0]); meta_line(f, "dy", s->mesh_.meshResolution_[1]);
  meta_line(f, "dz", s->mesh_.meshResolution_[2]);
  meta_line(f, "Lx", s->mesh_.meshLength_[0]); meta_line(f, "Ly", s->mesh_.meshLength_[1]);
  meta_line(f, "Lz", s->mesh_.meshLength_[2]);
  meta_line(f, "dt", s->mesh_.timeStep_); meta_line(f, "dtb", s->bunch_.timeStep_);
  meta_line(f, "nUpdateBunch", s->nUpdateBunch_);
  meta_line(f, "totalTime", s->mesh_.totalTime_);
  meta_line(f, "time", s->time_); meta_line(f, "timeBunch", s->timeBunch_);
  meta_line(f, "nTime", s->nTime_); meta_line(f, "nTimeBunch", s->nTimeBunch_);
  meta_line(f, "gamma", s->gamma_); meta_line(f, "beta", s->beta_); meta_line(f, "dt_shift", s->dt_);
  meta_line(f, "c0", s->c0_); meta_line(f, "m0", s->m0_); meta_line(f, "e0", s->e0_);
  for (int i = 0; i < 6; i++) { char k[32]; snprintf(k, 32, "a%d", i); meta_line(f, k, s->uf_.a[i]); }
  meta_line(f, "nsfd_alpha", s->uf_.af.alpha_); meta_line(f, "nsfd_beta", s->uf_.af.beta_);
  const char* bn[4] = {"bB", "cB", "dB", 0};
  const double* bv[3] = {s->uf_.bB, s->uf_.cB, s->uf_.dB};
  for (int b = 0; b < 3; b++)
    for (int i = 0; i < 5; i++) { char k[32]; snprintf(k, 32, "%s%d", bn[b], i); meta_line(f, k, bv[b][i]); }
  const char* en[3] = {"eE", "fE", "gE"};
  const double* ev[3] = {s->uf_.eE, s->uf_.fE, s->uf_.gE};
  for (int b = 0; b < 3; b++)
    for (int i = 0; i < 5; i++) { char k[32]; snprintf(k, 32, "%s%d", en[b], i); meta_line(f, k, ev[b][i]); }
  for (int i = 0; i < 17; i++) { char k[32]; snprintf(k, 32, "hC%d", i); meta_line(f, k, s->uf_.hC[i]); }
  meta_line(f, "uc_dv", s->uc_.dv); meta_line(f, "uc_rc", s->uc_.rc);
  meta_line(f, "ub_dtb", s->ub_.dtb); meta_line(f, "ub_r1", s->ub_.r1); meta_line(f, "ub_r2", s->ub_.r2);
  meta_line(f, "n_undulator", (double)s->undulator_.size());
  for (size_t u = 0; u < s->undulator_.size(); u++) {
    char k[64];
    snprintf(k, 64, "und%zu_k", u); meta_line(f, k, s->undulator_[u].k_);
    snprintf(k, 64, "und%zu_lu", u); meta_line(f, k, s->undulator_[u].lu_);
    snprintf(k, 64, "und%zu_rb", u); meta_line(f, k, s->undulator_[u].rb_);
    snprintf(k, 64, "und%zu_length", u); meta_line(f, k, s->undulator_[u].length_);
    snprintf(k, 64, "und%zu_dist", u); meta_line(f, k, s->undulator_[u].dist_);
    snprintf(k, 64, "und%zu_theta", u); meta_line(f, k, s->undulator_[u].theta_);
    snprintf(k, 64, "und%zu_type", u); meta_line(f, k, (double)s->undulator_[u].type_);
    if (s->undulator_[u].type_ == OPTICAL) beam_meta(f, "und" + std::to_string(u) + "_beam_", s->undulator_[u]);
  }
  beam_meta(f, "seed_", s->seed_);
  meta_line(f, "seed_gamma", s->seed_.gamma_); meta_line(f, "seed_beta", s->seed_.beta_);
  meta_line(f, "seed_c0", s->seed_.c0_); meta_line(f, "seed_dt", s->seed_.dt_);
  meta_line(f, "n_ext", (double)s->extField_.size());
  for (size_t x = 0; x < s->extField_.size(); x++) beam_meta(f, "ext" + std::to_string(x) + "_", s->extField_[x]);
  meta_line(f, "n_particles", (double)s->chargeVectorn_.size());
  meta_line(f, "n_fel", (double)s->FEL_.size());
  for (size_t j = 0; j < s->FEL_.size(); j++) {
    char k[64];
    if (!s->FEL_[j].radiationPower_.sampling_) continue;
    snprintf(k, 64, "rp%zu_N", j); meta_line(f, k, s->rp_[j].N);
    snprintf(k, 64, "rp%zu_Nl", j); meta_line(f, k, s->rp_[j].Nl);
    snprintf(k, 64, "rp%zu_Nf", j); meta_line(f, k, s->rp_[j].Nf);
    snprintf(k, 64, "rp%zu_pc", j); meta_line(f, k, s->rp_[j].pc);
    for (unsigned i = 0; i < s->rp_[j].Nl; i++) { snprintf(k, 64, "rp%zu_w%u", j, i); meta_line(f, k, s->rp_[j].w[i]); }
    for (unsigned i = 0; i < s->rp_[j].N; i++) { snprintf(k, 64, "rp%zu_z%u", j, i); meta_line(f, k, s->FEL_[j].radiationPower_.z_[i]); }
  }
  fclose(f);
}

/* The per-step body of Solver::solve, src/solver.cpp:1300-1399, without the file writers other
 * than the power sample (whose values are returned through rp_[].pG). */
static void field_step(Solver* s, FILE* power_out) {
  s->fieldUpdate();
  for (auto it = s->chargeVectorn_.begin(); it != s->chargeVectorn_.end(); it++) it->rnm = it->rnp;
  for (double t = 0.0; t < s->nUpdateBunch_; t += 1.0) {
    s->bunchUpdate();
    s->timeBunch_ += s->bunch_.timeStep_;
    ++s->nTimeBunch_;
  }
  s->recycleParticles();
  s->powerSample();
  if (power_out) {
    for (size_t jf = 0; jf < s->FEL_.size(); jf++) {
      if (!s->FEL_[jf].radiationPower_.sampling_) continue;
      for (unsigned k = 0; k < s->rp_[jf].N; k++) {
        double zl = s->gamma_ * (s->FEL_[jf].radiationPower_.z_[k] + s->beta_ * s->c0_ * (s->timeBunch_ + s->dt_));
        fwrite(&zl, 8, 1, power_out);
        for (unsigned l = 0; l < s->rp_[jf].Nl; l++) fwrite(&s->rp_[jf].pG[k * s->rp_[jf].Nl + l], 8, 1, power_out);
      }
    }
  }
  s->fieldShift();
  s->currentReset();
  s->currentUpdate();
  s->currentCommunicate();
  s->timem1_ += s->mesh_.timeStep_;
  s->time_ += s->mesh_.timeStep_;
  s->timep1_ += s->mesh_.timeStep_;
  ++s->nTime_;
}

/* The negative-time particle loop of Solver::solve, src/solver.cpp:1232-1291 (diagnostics off). */
static void pre_loop(Solver* s) {
  while (s->time_ < 0.0) {
    for (auto it = s->chargeVectorn_.begin(); it != s->chargeVectorn_.end(); it++) it->rnm = it->rnp;
    for (double t = 0.0; t < s->nUpdateBunch_; t += 1.0) {
      s->bunchUpdate();
      s->timeBunch_ += s->bunch_.timeStep_;
      ++s->nTimeBunch_;
    }
    s->recycleParticles();
    s->timem1_ += s->mesh_.timeStep_;
    s->time_ += s->mesh_.timeStep_;
    s->timep1_ += s->mesh_.timeStep_;
    ++s->nTime_;
  }
}

/* Byte size of every open screen file (flushed), in FEL and screen order. */
static void screen_offsets(Solver* s, std::vector<double>& out) {
  for (size_t jf = 0; jf < s->FEL_.size(); jf++) {
    if (!s->FEL_[jf].screenProfile_.sampling_) continue;
    for (size_t i = 0; i < s->scrp_[jf].files.size(); i++) {
      s->scrp_[jf].files[i]->flush();
      out.push_back((double)s->scrp_[jf].files[i]->tellp());
    }
  }
}

/* FdTd::fieldEvaluate reads the potentials through the uf_ pointers that fieldUpdate sets
 * (src/fdtd.cpp:240-245); modes that evaluate fields without a field update set them here. */
static void bind_field_pointers(Solver* s) {
  s->uf_.anp1 = &(*s->anp1_)[0][0];
  s->uf_.an = &(*s->an_)[0][0];
  s->uf_.anm1 = &(*s->anm1_)[0][0];
  s->uf_.jn = &(*s->anp1_)[0][0];
  s->uf_.en = &s->en_[0][0];
  s->uf_.bn = &s->bn_[0][0];
  if (s->mesh_.spaceCharge_) {
    s->uf_.fnp1 = &(*s->fnp1_)[0];
    s->uf_.fn = &(*s->fn_)[0];
    s->uf_.fnm1 = &(*s->fnm1_)[0];
    s->uf_.rn = &(*s->fnp1_)[0];
  }
}

/* The E/B state FdTd::fieldUpdate leaves behind (src/fdtd.cpp:742-774): planes k = 1 and
 * np-2 evaluated, copied into k = 0 and np-1, and flagged as evaluated. */
static void eval_boundary_planes(Solver* s) {
  for (int i = 1; i < s->N0_ - 1; i++)
    for (int j = 1; j < s->N1_ - 1; j++) {
      long m = s->N1N0_ + s->N1_ * i + j;
      s->fieldEvaluate(m);
      s->pic_[m - s->N1N0_] = true;
      s->en_[m - s->N1N0_] = s->en_[m];
      s->bn_[m - s->N1N0_] = s->bn_[m];
      m = (long)s->N1N0_ * (s->np_ - 2) + s->N1_ * i + j;
      s->fieldEvaluate(m);
      s->pic_[m + s->N1N0_] = true;
      s->en_[m + s->N1N0_] = s->en_[m];
      s->bn_[m + s->N1N0_] = s->bn_[m];
    }
}

static void dump_state(Solver* s, const std::string& dir) {
  mkdir(dir.c_str(), 0755);
  dump_meta(s, jp(dir, "meta.txt"));
  dump_vec3(jp(dir, "an.bin"), s->an_);
  dump_vec3(jp(dir, "anm1.bin"), s->anm1_);
  dump_vec3(jp(dir, "anp1.bin"), s->anp1_);
  if (s->mesh_.spaceCharge_) {
    dump_scalar_field(jp(dir, "fn.bin"), s->fn_);
    dump_scalar_field(jp(dir, "fnm1.bin"), s->fnm1_);
    dump_scalar_field(jp(dir, "fnp1.bin"), s->fnp1_);
  }
  dump_particles(jp(dir, "particles.bin"), s->chargeVectorn_);
}

int main(int argc, char** argv) {
  if (argc < 4) { fprintf(stderr, "usage: %s MODE JOB OUT ...\n", argv[0]); return 2; }
  std::string mode = argv[1];
  int dummy_argc = 1;
  MPI_Init(&dummy_argc, &argv);

  /* Parse exactly as main does, src/mithra.cpp:48-75. */
  std::list<std::string> jobFile = read_file(argv[2]);
  cleanJobFile(jobFile);
  Mesh mesh; mesh.initialize();
  Bunch bunch; Seed seed;
  std::vector<Undulator> undulator; std::vector<ExtField> extField; std::vector<FreeElectronLaser> FEL;
  ParseDarius parser(jobFile, mesh, bunch, seed, undulator, extField, FEL);
  parser.setJobParameters();

  Solver* s;
  if (mesh.spaceCharge_) s = new FdTdSC(mesh, bunch, seed, undulator, extField, FEL);
  else s = new FdTd(mesh, bunch, seed, undulator, extField, FEL);
  s->initialize();

  if (mode == "init") {
    pre_loop(s);
    dump_state(s, argv[3]);
  } else if (mode == "run") {
    int nsteps = atoi(argv[3]);
    std::string out = argv[4];
    int every = argc > 5 ? atoi(argv[5]) : nsteps;
    mkdir(out.c_str(), 0755);
    pre_loop(s);
    dump_state(s, jp(out, "step0"));
    FILE* pw = fopen(jp(out, "power.bin").c_str(), "wb");
    for (int n = 1; n <= nsteps; n++) {
      field_step(s, pw);
      if (n % every == 0 || n == nsteps) dump_state(s, jp(out, "step" + std::to_string(n)));
    }
    fclose(pw);
  } else if (mode == "vtk") {
    // Solver::solve's field visualization (src/solver.cpp:1328-1340) after recycleParticles.
    int nsteps = atoi(argv[3]);
    std::string out = argv[4];
    mkdir(out.c_str(), 0755);
    pre_loop(s);
    std::vector<double> steps;
    for (int n = 1; n <= nsteps; n++) {
      steps.push_back((double)s->nTime_);
      s->fieldUpdate();
      for (auto it = s->chargeVectorn_.begin(); it != s->chargeVectorn_.end(); it++) it->rnm = it->rnp;
      for (double t = 0.0; t < s->nUpdateBunch_; t += 1.0) {
        s->bunchUpdate();
        s->timeBunch_ += s->bunch_.timeStep_;
        ++s->nTimeBunch_;
      }
      s->recycleParticles();
      if (s->seed_.sampling_ && fmod(s->time_, s->seed_.samplingRhythm_) < s->mesh_.timeStep_ && s->time_ > 0.0)
        s->fieldSample();
      for (unsigned int i = 0; i < s->seed_.vtk_.size(); i++) {
        if (s->seed_.vtk_[i].sample_ && fmod(s->time_, s->seed_.vtk_[i].rhythm_) < s->mesh_.timeStep_ && s->time_ > 0.0) {
          if (s->seed_.vtk_[i].type_ == ALLDOMAIN) s->fieldVisualizeAllDomain(i);
          else if (s->seed_.vtk_[i].type_ == INPLANE) s->fieldVisualizeInPlane(i);
        }
      }
      s->powerSample();
      s->fieldShift();
      s->currentReset();
      s->currentUpdate();
      s->currentCommunicate();
      s->timem1_ += s->mesh_.timeStep_;
      s->time_ += s->mesh_.timeStep_;
      s->timep1_ += s->mesh_.timeStep_;
      ++s->nTime_;
    }
    write_raw(jp(out, "steps.bin"), steps.data(), steps.size() * 8);
  } else if (mode == "screen") {
    // The negative-time loop and the field steps with screenProfile at its places in
    // Solver::solve: after the substeps in the prelude (src/solver.cpp:1248), after
    // recycleParticles in the main loop (src/solver.cpp:1374).
    int nsteps = atoi(argv[3]);
    std::string out = argv[4];
    mkdir(out.c_str(), 0755);
    std::vector<double> offs;
    while (s->time_ < 0.0) {
      for (auto it = s->chargeVectorn_.begin(); it != s->chargeVectorn_.end(); it++) it->rnm = it->rnp;
      for (double t = 0.0; t < s->nUpdateBunch_; t += 1.0) {
        s->bunchUpdate();
        s->timeBunch_ += s->bunch_.timeStep_;
        ++s->nTimeBunch_;
      }
      s->screenProfile();
      if (s->bunch_.sampling_ && fmod(s->time_ + s->mesh_.timeShift_, s->bunch_.rhythm_) < s->mesh_.timeStep_ &&
          (s->time_ + s->mesh_.timeShift_ > 0.0))
        s->bunchSample();
      if (s->bunch_.bunchProfile_) {
        for (unsigned int i = 0; i < s->bunch_.bunchProfileTime_.size(); i++)
          if (s->time_ - s->bunch_.bunchProfileTime_[i] < s->mesh_.timeStep_ && s->time_ > s->bunch_.bunchProfileTime_[i])
            s->bunchProfile();
        if (fmod(s->time_ + s->mesh_.timeShift_, s->bunch_.bunchProfileRhythm_) < s->mesh_.timeStep_ &&
            (s->time_ + s->mesh_.timeShift_ > 0.0) && (s->bunch_.bunchProfileRhythm_ != 0.0))
          s->bunchProfile();
      }
      s->recycleParticles();
      s->timem1_ += s->mesh_.timeStep_;
      s->time_ += s->mesh_.timeStep_;
      s->timep1_ += s->mesh_.timeStep_;
      ++s->nTime_;
    }
    screen_offsets(s, offs);
    for (int n = 1; n <= nsteps; n++) {
      s->fieldUpdate();
      for (auto it = s->chargeVectorn_.begin(); it != s->chargeVectorn_.end(); it++) it->rnm = it->rnp;
      for (double t = 0.0; t < s->nUpdateBunch_; t += 1.0) {
        s->bunchUpdate();
        s->timeBunch_ += s->bunch_.timeStep_;
        ++s->nTimeBunch_;
      }
      s->recycleParticles();
      if (s->bunch_.sampling_ && fmod(s->time_ + s->mesh_.timeShift_, s->bunch_.rhythm_) < s->mesh_.timeStep_ &&
          (s->time_ + s->mesh_.timeShift_ > 0.0))
        s->bunchSample();
      if (s->bunch_.bunchProfile_) {
        for (unsigned int i = 0; i < s->bunch_.bunchProfileTime_.size(); i++)
          if (s->time_ - s->bunch_.bunchProfileTime_[i] < s->mesh_.timeStep_ && s->time_ > s->bunch_.bunchProfileTime_[i])
            s->bunchProfile();
        if (fmod(s->time_ + s->mesh_.timeShift_, s->bunch_.bunchProfileRhythm_) < s->mesh_.timeStep_ &&
            (s->time_ + s->mesh_.timeShift_ > 0.0) && (s->bunch_.bunchProfileRhythm_ != 0.0))
          s->bunchProfile();
      }
      s->screenProfile();
      s->powerSample();
      s->fieldShift();
      s->currentReset();
      s->currentUpdate();
      s->currentCommunicate();
      s->timem1_ += s->mesh_.timeStep_;
      s->time_ += s->mesh_.timeStep_;
      s->timep1_ += s->mesh_.timeStep_;
      ++s->nTime_;
      screen_offsets(s, offs);
    }
    write_raw(jp(out, "offsets.bin"), offs.data(), offs.size() * 8);
  } else if (mode == "field") {
    std::string in = argv[3], out = argv[4];
    mkdir(out.c_str(), 0755);
    load_vec3(jp(in, "an.bin"), s->an_);
    load_vec3(jp(in, "anm1.bin"), s->anm1_);
    load_vec3(jp(in, "anp1.bin"), s->anp1_);
    if (mesh.spaceCharge_) {
      load_scalar_field(jp(in, "fn.bin"), s->fn_);
      load_scalar_field(jp(in, "fnm1.bin"), s->fnm1_);
      load_scalar_field(jp(in, "fnp1.bin"), s->fnp1_);
    }
    s->fieldUpdate();
    for (int k = 2; k < s->np_ - 2; k++)
      for (int i = 1; i < s->N0_ - 1; i++)
        for (int j = 1; j < s->N1_ - 1; j++) s->fieldEvaluate((long)s->N1N0_ * k + s->N1_ * i + j);
    dump_vec3(jp(out, "anp1.bin"), s->anp1_);
    if (mesh.spaceCharge_) dump_scalar_field(jp(out, "fnp1.bin"), s->fnp1_);
    write_raw(jp(out, "en.bin"), s->en_.data(), s->en_.size() * 12);
    write_raw(jp(out, "bn.bin"), s->bn_.data(), s->bn_.size() * 12);
  } else if (mode == "push") {
    std::string in = argv[3], out = argv[4];
    mkdir(out.c_str(), 0755);
    load_vec3(jp(in, "an.bin"), s->an_);
    load_vec3(jp(in, "anp1.bin"), s->anp1_);
    if (mesh.spaceCharge_) load_scalar_field(jp(in, "fn.bin"), s->fn_);
    load_particles(jp(in, "particles.bin"), s->chargeVectorn_);
    std::vector<char> tb = read_raw(jp(in, "timebunch.bin"));
    memcpy(&s->timeBunch_, tb.data(), 8);
    std::fill(s->pic_.begin(), s->pic_.end(), false);
    bind_field_pointers(s);
    eval_boundary_planes(s);
    s->bunchUpdate();
    dump_particles(jp(out, "particles.bin"), s->chargeVectorn_);
  } else if (mode == "deposit") {
    std::string in = argv[3], out = argv[4];
    mkdir(out.c_str(), 0755);
    load_particles(jp(in, "particles.bin"), s->chargeVectorn_);
    s->currentReset();
    s->currentUpdate();
    dump_vec3(jp(out, "anp1.bin"), s->anp1_);
    if (mesh.spaceCharge_) dump_scalar_field(jp(out, "fnp1.bin"), s->fnp1_);
    s->currentCommunicate();
    dump_particles(jp(out, "particles.bin"), s->chargeVectorn_);
  } else if (mode == "fieldsample") {
    // FdTd::fieldSample at each loaded point (one point per call), on loaded A^n / A^{n+1}; the
    // interpolated et, bt, at it leaves in sf_ are dumped at full precision.
    std::string in = argv[3], out = argv[4];
    mkdir(out.c_str(), 0755);
    load_vec3(jp(in, "an.bin"), s->an_);
    load_vec3(jp(in, "anp1.bin"), s->anp1_);
    std::vector<char> raw = read_raw(jp(in, "points.bin"));
    const double* pts = (const double*)raw.data();
    const size_t np = raw.size() / 24;
    std::fill(s->pic_.begin(), s->pic_.end(), false);
    bind_field_pointers(s);
    eval_boundary_planes(s);
    std::ofstream sink("/dev/null");
    s->sf_.file = &sink;
    s->sf_.N = 1;
    s->seed_.samplingPosition_.assign(1, FieldVector<Double>(0.0));
    std::vector<double> v;
    for (size_t n = 0; n < np; n++) {
      for (int c = 0; c < 3; c++) s->seed_.samplingPosition_[0][c] = pts[3 * n + c];
      s->fieldSample();
      for (int c = 0; c < 3; c++) v.push_back(s->sf_.et[c]);
      for (int c = 0; c < 3; c++) v.push_back(s->sf_.bt[c]);
      for (int c = 0; c < 3; c++) v.push_back(s->sf_.at[c]);
    }
    write_raw(jp(out, "sample.bin"), v.data(), v.size() * 8);
  } else if (mode == "bunch") {
    // Solver::bunchSample on loaded particles; the moments it writes (4 digits) are dumped here
    // at full precision from its own sb_ members: <r>, <gb>, rms r, rms gb.
    std::string in = argv[3], out = argv[4];
    mkdir(out.c_str(), 0755);
    load_particles(jp(in, "particles.bin"), s->chargeVectorn_);
    std::ofstream sink("/dev/null");
    s->sb_.file = &sink;
    s->bunchSample();
    std::vector<double> v(12);
    for (int l = 0; l < 3; l++) {
      v[l] = s->sb_.rT[l];
      v[3 + l] = s->sb_.gbT[l];
      v[6 + l] = sqrt(s->sb_.r2T[l] - s->sb_.rT[l] * s->sb_.rT[l]);
      v[9 + l] = sqrt(s->sb_.gb2T[l] - s->sb_.gbT[l] * s->sb_.gbT[l]);
    }
    write_raw(jp(out, "bunch.bin"), v.data(), v.size() * 8);
  } else if (mode == "power") {
    std::string in = argv[3], out = argv[4];
    int K = atoi(argv[5]);
    mkdir(out.c_str(), 0755);
    FILE* pw = fopen(jp(out, "power.bin").c_str(), "wb");
    for (int t = 0; t < K; t++) {
      load_vec3(jp(in, "an_" + std::to_string(t) + ".bin"), s->an_);
      load_vec3(jp(in, "anp1_" + std::to_string(t) + ".bin"), s->anp1_);
      std::fill(s->pic_.begin(), s->pic_.end(), false);
      bind_field_pointers(s);
      eval_boundary_planes(s);
      s->powerSample();
      for (size_t jf = 0; jf < s->FEL_.size(); jf++) {
        if (!s->FEL_[jf].radiationPower_.sampling_) continue;
        fwrite(s->rp_[jf].pG.data(), 8, s->rp_[jf].pG.size(), pw);
      }
      ++s->nTime_;
    }
    fclose(pw);
  } else {
    fprintf(stderr, "unknown mode %s\n", mode.c_str());
    return 2;
  }
  MPI_Finalize();
  return 0;
}
