// C ABI of the host initialisation (mithra_setup_*) and the job-level context constructor.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <exception>

#include "mithra_gpu.h"
#include "setup.h"

struct mithra_setup {
  mithra::host::Setup s;
};

using mithra::host::Setup;

extern "C" {

int mithra_setup_from_job(const char* job_path, mithra_setup** out, char* err, size_t err_len) {
  if (!job_path || !out) return MITHRA_ERR_ARG;
  *out = nullptr;
  mithra_setup* h = new mithra_setup();
  try {
    h->s.job = mithra::host::parse_job_file(job_path);
  } catch (const std::exception& e) {
    if (err && err_len) snprintf(err, err_len, "%s", e.what());
    delete h;
    return MITHRA_ERR_PARSE;
  }
  try {
    h->s.initialize();
  } catch (const std::exception& e) {
    if (err && err_len) snprintf(err, err_len, "%s", e.what());
    delete h;
    return MITHRA_ERR_ARG;
  }
  *out = h;
  return MITHRA_OK;
}

int mithra_setup_from_job_device(const char* job_path, int device, mithra_setup** out, char* err, size_t err_len) {
  if (!job_path || !out) return MITHRA_ERR_ARG;
  *out = nullptr;
  mithra_setup* h = new mithra_setup();
  try {
    h->s.job = mithra::host::parse_job_file(job_path);
  } catch (const std::exception& e) {
    if (err && err_len) snprintf(err, err_len, "%s", e.what());
    delete h;
    return MITHRA_ERR_PARSE;
  }
  h->s.device_init = true;
  h->s.dstore.device = device;
  try {
    h->s.initialize();
  } catch (const std::exception& e) {
    if (err && err_len) snprintf(err, err_len, "%s", e.what());
    mithra::devinit::release(h->s.dstore);
    delete h;
    return MITHRA_ERR_ARG;
  }
  *out = h;
  return MITHRA_OK;
}

int mithra_setup_destroy(mithra_setup* s) {
  if (!s) return MITHRA_ERR_ARG;
  mithra::devinit::release(s->s.dstore);
  delete s;
  return MITHRA_OK;
}

int mithra_setup_grid(const mithra_setup* s, mithra_grid_desc* g) {
  if (!s || !g) return MITHRA_ERR_ARG;
  s->s.fill_grid(g);
  return MITHRA_OK;
}

int mithra_setup_push(const mithra_setup* s, mithra_push_desc* p) {
  if (!s || !p) return MITHRA_ERR_ARG;
  s->s.fill_push(p);
  return MITHRA_OK;
}

}  // extern "C"

namespace {
mithra_beam_desc beam_desc(const mithra::host::Beam& b) {
  mithra_beam_desc d{};
  d.type = (int32_t)b.seedType;
  for (int c = 0; c < 3; c++) {
    d.position[c] = b.position[c];
    d.direction[c] = b.direction[c];
    d.polarization[c] = b.polarization[c];
  }
  d.amplitude = b.amplitude;
  for (int c = 0; c < 2; c++) {
    d.radius[c] = c < (int)b.radius.size() ? b.radius[c] : 0.0;
    d.order[c] = c < (int)b.order.size() ? b.order[c] : 0;
    d.rayleigh[c] = c < (int)b.zR.size() ? b.zR[c] : 0.0;
    d.signal_sigma[c] = c < (int)b.signal.sigmaInvG.size() ? b.signal.sigmaInvG[c] : 0.0;
  }
  d.wavelength = b.l;
  d.signal_type = (int32_t)b.signal.type;
  d.signal_t0 = b.signal.t0; d.signal_s = b.signal.s; d.signal_f0 = b.signal.f0;
  d.signal_cep = b.signal.cep; d.signal_nr = (double)b.signal.nR;
  return d;
}
}  // namespace

extern "C" {

int mithra_setup_seed(const mithra_setup* s, mithra_seed_desc* seed) {
  if (!s || !seed) return MITHRA_ERR_ARG;
  const auto& S = s->s.job.seed;
  seed->beam = beam_desc(S);
  seed->gamma = S.gamma; seed->beta = S.beta; seed->c0 = S.c0; seed->dt = S.dt;
  return MITHRA_OK;
}

int mithra_setup_external_fields(const mithra_setup* s, mithra_beam_desc* fields, int cap, int* n) {
  if (!s || !n) return MITHRA_ERR_ARG;
  const auto& X = s->s.job.extFields;
  *n = (int)X.size();
  for (int x = 0; x < std::min<int>(cap, (int)X.size()); x++) fields[x] = beam_desc(X[x]);
  return MITHRA_OK;
}

int mithra_setup_undulators(const mithra_setup* s, mithra_undulator_desc* und, int cap, int* n) {
  if (!s || !n) return MITHRA_ERR_ARG;
  const auto& U = s->s.job.undulators;
  *n = (int)U.size();
  for (int u = 0; u < std::min<int>(cap, (int)U.size()); u++) {
    und[u].type = U[u].type == mithra::host::STATIC ? 0 : 1;
    und[u].k = U[u].k;
    und[u].lu = U[u].lu;
    und[u].rb = U[u].rb;
    und[u].length = (double)U[u].length;
    und[u].dist = U[u].dist;
    und[u].theta = U[u].theta;
    und[u].beam = beam_desc(U[u]);
  }
  return MITHRA_OK;
}

int mithra_setup_power(const mithra_setup* s, int o, mithra_power_desc* out, int* n) {
  if (!s || !n) return MITHRA_ERR_ARG;
  const auto& P = s->s.power;
  *n = (int)P.size();
  if (!out) return MITHRA_OK;
  if (o < 0 || o >= (int)P.size()) return MITHRA_ERR_ARG;
  const auto& pc = P[(size_t)o];
  out->N = pc.N; out->Nl = pc.Nl; out->Nf = pc.Nf; out->pc = pc.pc;
  out->z = pc.z.data(); out->twiddle_re = pc.tw_re.data(); out->twiddle_im = pc.tw_im.data();
  return MITHRA_OK;
}

int mithra_setup_time(const mithra_setup* s, mithra_time_state* t) {
  if (!s || !t) return MITHRA_ERR_ARG;
  t->time = s->s.time;
  t->time_bunch = s->s.timeBunch;
  t->n_time = s->s.nTime;
  t->n_time_bunch = s->s.nTimeBunch;
  return MITHRA_OK;
}

int mithra_setup_total_time(const mithra_setup* s, double* total_time) {
  if (!s || !total_time) return MITHRA_ERR_ARG;
  *total_time = s->s.job.mesh.totalTime;
  return MITHRA_OK;
}

int mithra_setup_particles(const mithra_setup* s, double* rec, size_t cap, size_t* n) {
  if (!s || !n) return MITHRA_ERR_ARG;
  if (s->s.device_init) {  // copy of the device records
    *n = s->s.dstore.n;
    if (!rec || !*n) return MITHRA_OK;
    char err[256];
    return mithra::devinit::download(s->s.dstore, rec, std::min(cap, *n), err, sizeof err) ? MITHRA_ERR_CUDA : MITHRA_OK;
  }
  const auto& C = s->s.charges;
  *n = C.size();
  if (!rec) return MITHRA_OK;
  for (size_t i = 0; i < std::min(cap, C.size()); i++) {
    double* r = rec + 11 * i;
    r[0] = C[i].q;
    for (int d = 0; d < 3; d++) { r[1 + d] = C[i].rnp[d]; r[4 + d] = C[i].rnm[d]; r[7 + d] = C[i].gb[d]; }
    r[10] = C[i].e;
  }
  return cap < C.size() ? MITHRA_ERR_CAPACITY : MITHRA_OK;
}

int mithra_setup_fields(const mithra_setup* s, double* anp1, double* an, double* anm1) {
  if (!s) return MITHRA_ERR_ARG;
  const size_t n = (size_t)s->s.N1N0 * s->s.np * 3;
  if (anp1) memset(anp1, 0, n * sizeof(double));
  if (an) {
    if (s->s.an.empty()) memset(an, 0, n * sizeof(double));
    else memcpy(an, s->s.an.data(), n * sizeof(double));
  }
  if (anm1) {
    if (s->s.anm1.empty()) memset(anm1, 0, n * sizeof(double));
    else memcpy(anm1, s->s.anm1.data(), n * sizeof(double));
  }
  return MITHRA_OK;
}

int mithra_setup_vtk_basename(const mithra_setup* s, int i, char* buf, size_t len, size_t* needed) {
  if (!s || i < 0 || i >= (int)s->s.job.seed.vtk.size()) return MITHRA_ERR_ARG;
  const std::string& b = s->s.job.seed.vtk[(size_t)i].basename;
  if (needed) *needed = b.size() + 1;
  if (!buf) return MITHRA_OK;
  if (len < b.size() + 1) return MITHRA_ERR_ARG;
  memcpy(buf, b.c_str(), b.size() + 1);
  return MITHRA_OK;
}

int mithra_setup_power_basename(const mithra_setup* s, int o, char* buf, size_t len, size_t* needed) {
  if (!s || o < 0 || o >= (int)s->s.power_fel_index.size()) return MITHRA_ERR_ARG;
  const auto& rp = s->s.job.fel[(size_t)s->s.power_fel_index[(size_t)o]].radiationPower;
  // Solver::initializePowerSample, src/radiation.cpp:74-76
  const std::string b = (!rp.basename.empty() && rp.basename[0] == '/') ? rp.basename : rp.directory + rp.basename;
  if (needed) *needed = b.size() + 1;
  if (!buf) return MITHRA_OK;
  if (len < b.size() + 1) return MITHRA_ERR_ARG;
  memcpy(buf, b.c_str(), b.size() + 1);
  return MITHRA_OK;
}

int mithra_setup_screen_basename(const mithra_setup* s, int jf, char* buf, size_t len, size_t* needed) {
  if (!s || jf < 0 || jf >= (int)s->s.job.fel.size()) return MITHRA_ERR_ARG;
  const auto& sp = s->s.job.fel[(size_t)jf].screenProfile;
  if (!sp.sampling) return MITHRA_ERR_ARG;
  // Solver::initializeScreenProfile, src/solver.cpp:2154
  const std::string b = (!sp.basename.empty() && sp.basename[0] == '/') ? sp.basename : sp.directory + sp.basename;
  if (needed) *needed = b.size() + 1;
  if (!buf) return MITHRA_OK;
  if (len < b.size() + 1) return MITHRA_ERR_ARG;
  memcpy(buf, b.c_str(), b.size() + 1);
  return MITHRA_OK;
}

int mithra_setup_bunch_sample_file(const mithra_setup* s, char* buf, size_t len, size_t* needed) {
  if (!s || !s->s.job.bunch.sampling) return MITHRA_ERR_ARG;
  const auto& b = s->s.job.bunch;
  // Solver::initializeBunchUpdate, src/solver.cpp:1066-1068
  const std::string f = ((!b.basename.empty() && b.basename[0] == '/') ? b.basename : b.directory + b.basename) + ".txt";
  if (needed) *needed = f.size() + 1;
  if (!buf) return MITHRA_OK;
  if (len < f.size() + 1) return MITHRA_ERR_ARG;
  memcpy(buf, f.c_str(), f.size() + 1);
  return MITHRA_OK;
}

int mithra_setup_field_sample_file(const mithra_setup* s, char* buf, size_t len, size_t* needed) {
  if (!s || !s->s.job.seed.sampling) return MITHRA_ERR_ARG;
  const auto& f = s->s.job.seed.samp;
  // Solver::initializeSeedSampling, src/solver.cpp:916-918 (rank 0 of one)
  const std::string name =
      ((!f.basename.empty() && f.basename[0] == '/') ? f.basename : f.directory + f.basename) + "-0.txt";
  if (needed) *needed = name.size() + 1;
  if (!buf) return MITHRA_OK;
  if (len < name.size() + 1) return MITHRA_ERR_ARG;
  memcpy(buf, name.c_str(), name.size() + 1);
  return MITHRA_OK;
}

int mithra_setup_bunch_profile_basename(const mithra_setup* s, char* buf, size_t len, size_t* needed) {
  if (!s || !s->s.job.bunch.profile) return MITHRA_ERR_ARG;
  const auto& b = s->s.job.bunch;
  // Solver::initializeBunchUpdate, src/solver.cpp:1109
  const std::string f = (!b.profileBasename.empty() && b.profileBasename[0] == '/') ? b.profileBasename
                                                                                  : b.profileDirectory + b.profileBasename;
  if (needed) *needed = f.size() + 1;
  if (!buf) return MITHRA_OK;
  if (len < f.size() + 1) return MITHRA_ERR_ARG;
  memcpy(buf, f.c_str(), f.size() + 1);
  return MITHRA_OK;
}

int mithra_setup_meta(const mithra_setup* s, char* buf, size_t len, size_t* needed) {
  if (!s) return MITHRA_ERR_ARG;
  const std::string m = s->s.meta();
  if (needed) *needed = m.size() + 1;
  if (!buf) return MITHRA_OK;
  if (len < m.size() + 1) return MITHRA_ERR_ARG;
  memcpy(buf, m.c_str(), m.size() + 1);
  return MITHRA_OK;
}

int mithra_gpu_create_from_setup(const mithra_setup* s, int precision, int device, double capacity_factor,
                                 mithra_ctx** out) {
  if (!s || !out) return MITHRA_ERR_ARG;
  const Setup& S = s->s;
  mithra_grid_desc g;
  mithra_push_desc p;
  S.fill_grid(&g);
  S.fill_push(&p);
  if (capacity_factor < 1.0) capacity_factor = 1.0;
  const size_t cap = (size_t)std::ceil(S.particle_count() * capacity_factor) + 1024;
  int r = mithra_gpu_create(&g, &p, precision, device, cap, out);
  if (r) return r;
  mithra_ctx* ctx = *out;
  auto bail = [&](int code) { mithra_gpu_destroy(ctx); *out = nullptr; return code; };
  std::vector<mithra_undulator_desc> und(S.job.undulators.size());
  int nu = 0;
  if ((r = mithra_setup_undulators(s, und.data(), (int)und.size(), &nu))) return bail(r);
  if ((r = mithra_gpu_set_undulators(ctx, und.data(), nu))) return bail(r);
  mithra_seed_desc seed;
  if ((r = mithra_setup_seed(s, &seed)) || (r = mithra_gpu_set_seed(ctx, &seed))) return bail(r);
  std::vector<mithra_beam_desc> ext(S.job.extFields.size());
  int nx = 0;
  if ((r = mithra_setup_external_fields(s, ext.data(), (int)ext.size(), &nx))) return bail(r);
  if (nx > MITHRA_MAX_EXT_FIELDS)
    return bail(MITHRA_ERR_ARG);
  if ((r = mithra_gpu_set_external_fields(ctx, ext.data(), nx))) return bail(r);
  std::vector<mithra_power_desc> pw(S.power.size());
  for (size_t o = 0; o < pw.size(); o++) {
    int np = 0;
    if ((r = mithra_setup_power(s, (int)o, &pw[o], &np))) return bail(r);
  }
  if ((r = mithra_gpu_set_power(ctx, pw.data(), (int)pw.size()))) return bail(r);
  const size_t nf = (size_t)S.N1N0 * S.np * 3;
  std::vector<double> a1(nf, 0.0);
  const double* an = S.an.empty() ? a1.data() : S.an.data();
  const double* anm1 = S.anm1.empty() ? a1.data() : S.anm1.data();
  if ((r = mithra_gpu_upload_fields(ctx, a1.data(), an, anm1))) return bail(r);
  if (S.device_init) {
    if (S.dstore.device != device) return bail(MITHRA_ERR_ARG);  // records live on another device
    if ((r = mithra_gpu_upload_particles_device(ctx, S.dstore.rec, S.dstore.n))) return bail(r);
  } else {
    std::vector<double> rec(S.charges.size() * 11);
    size_t n = 0;
    if ((r = mithra_setup_particles(s, rec.data(), S.charges.size(), &n))) return bail(r);
    if ((r = mithra_gpu_upload_particles(ctx, rec.data(), n))) return bail(r);
  }
  mithra_time_state t;
  mithra_setup_time(s, &t);
  if ((r = mithra_gpu_set_time(ctx, &t))) return bail(r);
  return MITHRA_OK;
}

}  // extern "C"
