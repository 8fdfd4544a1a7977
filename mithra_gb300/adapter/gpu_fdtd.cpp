/*
 * gpu_fdtd.cpp : the reference-side adapter (see gpu_fdtd.h).
 *
 * Every descriptor field is read from the member of the initialised Solver that the
 * corresponding reference code reads:
 *   grid   : N0_, N1_, N2_ (np_ = N2_ on one rank), mesh_.solver_, truncationOrder_, spaceCharge_,
 *            uf_.a, uf_.af.alpha_/beta_, the Mur coefficients uf_.bB .. uf_.hC (src/solver.cpp:695-825),
 *            mesh_.timeStep_, meshResolution_, xmin_ .. zmax_, zp_, meshLength_[2]
 *   push   : ub_.dtb, bunch_.timeStep_, ub_.r1, ub_.r2, gamma_, beta_, c0_, dt_, nUpdateBunch_
 *            (src/solver.cpp:1050-1059)
 *   beams  : seed_, undulator_[u] (optical ones) and extField_[x] after initialize:
 *            seedType_, position_, direction_, polarization_, amplitude_, radius_, order_, l_,
 *            zR_, signal_ (src/classes.cpp:646-735, :1007-1075, :1162-1260)
 *   power  : rp_[jf].N, Nl, Nf, pc, FEL_[jf].radiationPower_.z_ (boosted) and the twiddles
 *            rp_[jf].ep (src/radiation.cpp:18-121)
 *   time   : time_, timeBunch_, nTime_, nTimeBunch_
 */
#include "gpu_fdtd.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <iterator>
#include <list>

namespace MITHRA {

namespace {

template <class Beam>
mithra_beam_desc beam_of(const Beam& b) {
  mithra_beam_desc d = mithra_beam_desc();
  d.type = (int32_t)b.seedType_;
  for (int c = 0; c < 3; c++) {
    d.position[c] = b.position_[c];
    d.direction[c] = b.direction_[c];
    d.polarization[c] = b.polarization_[c];
  }
  d.amplitude = b.amplitude_;
  for (int c = 0; c < 2; c++) {
    d.radius[c] = c < (int)b.radius_.size() ? b.radius_[c] : 0.0;
    d.order[c] = c < (int)b.order_.size() ? b.order_[c] : 0;
    d.rayleigh[c] = c < (int)b.zR_.size() ? b.zR_[c] : 0.0;
    d.signal_sigma[c] = c < (int)b.signal_.sigmaInvG_.size() ? b.signal_.sigmaInvG_[c] : 0.0;
  }
  d.wavelength = b.l_;
  d.signal_type = (int32_t)b.signal_.signalType_;
  d.signal_t0 = b.signal_.t0_;
  d.signal_s = b.signal_.s_;
  d.signal_f0 = b.signal_.f0_;
  d.signal_cep = b.signal_.cep_;
  d.signal_nr = (double)b.signal_.nR_;
  return d;
}

// The reference's error convention (printmessage, then exit(1)) for a library status.
[[noreturn]] void fail_like_reference(const std::string& what) {
  printmessage(std::string(__FILE__), __LINE__, std::string(" GPU solver: ") + what);
  exit(1);
}

}  // namespace

void describe_for_gpu(Solver& s, GpuDescriptors& d) {
  mithra_grid_desc& g = d.grid;
  g = mithra_grid_desc();
  g.N0 = s.N0_;
  g.N1 = s.N1_;
  g.N2 = s.np_;
  g.solver = s.mesh_.solver_ == NSFD ? 1 : 0;
  g.truncation_order = (int32_t)s.mesh_.truncationOrder_;
  g.space_charge = s.mesh_.spaceCharge_ ? 1 : 0;
  for (int i = 0; i < 6; i++) g.a[i] = s.uf_.a[i];
  g.nsfd_alpha = s.uf_.af.alpha_;
  g.nsfd_beta = s.uf_.af.beta_;
  for (int i = 0; i < 5; i++) {
    g.bB[i] = s.uf_.bB[i]; g.cB[i] = s.uf_.cB[i]; g.dB[i] = s.uf_.dB[i];
    g.eE[i] = s.uf_.eE[i]; g.fE[i] = s.uf_.fE[i]; g.gE[i] = s.uf_.gE[i];
  }
  for (int i = 0; i < 17; i++) g.hC[i] = s.uf_.hC[i];
  g.dt = s.mesh_.timeStep_;
  g.dx = s.mesh_.meshResolution_[0];
  g.dy = s.mesh_.meshResolution_[1];
  g.dz = s.mesh_.meshResolution_[2];
  g.xmin = s.xmin_; g.xmax = s.xmax_;
  g.ymin = s.ymin_; g.ymax = s.ymax_;
  g.zmin = s.zmin_; g.zmax = s.zmax_;
  g.zp0 = s.zp_[0]; g.zp1 = s.zp_[1];
  g.Lz = s.mesh_.meshLength_[2];

  mithra_push_desc& p = d.push;
  p = mithra_push_desc();
  p.dtb = s.ub_.dtb;
  p.bunch_time_step = s.bunch_.timeStep_;
  p.r1 = s.ub_.r1;
  p.r2 = s.ub_.r2;
  p.gamma = s.gamma_;
  p.beta = s.beta_;
  p.c0 = s.c0_;
  p.dt_shift = s.dt_;
  p.n_update_bunch = s.nUpdateBunch_;

  d.seed = mithra_seed_desc();
  d.seed.beam = beam_of(s.seed_);
  d.seed.gamma = s.seed_.gamma_;
  d.seed.beta = s.seed_.beta_;
  d.seed.c0 = s.seed_.c0_;
  d.seed.dt = s.seed_.dt_;

  d.undulators.clear();
  for (size_t u = 0; u < s.undulator_.size(); u++) {
    const Undulator& U = s.undulator_[u];
    mithra_undulator_desc x = mithra_undulator_desc();
    x.type = U.type_ == STATIC ? 0 : 1;
    x.k = U.k_;
    x.lu = U.lu_;
    x.rb = U.rb_;
    x.length = (double)U.length_;
    x.dist = U.dist_;
    x.theta = U.theta_;
    x.beam = beam_of(U);
    d.undulators.push_back(x);
  }
  d.ext_fields.clear();
  for (size_t e = 0; e < s.extField_.size(); e++) d.ext_fields.push_back(beam_of(s.extField_[e]));

  d.power.clear();
  d.power_fel.clear();
  d.power_z.clear();
  d.power_re.clear();
  d.power_im.clear();
  for (unsigned jf = 0; jf < s.FEL_.size(); jf++) {
    if (!s.FEL_[jf].radiationPower_.sampling_) continue;
    const SampleRadiationPower& rp = s.rp_[jf];
    d.power_fel.push_back(jf);
    d.power_z.push_back(std::vector<double>(s.FEL_[jf].radiationPower_.z_.begin(), s.FEL_[jf].radiationPower_.z_.end()));
    std::vector<double> re, im;
    for (unsigned l = 0; l < rp.Nl; l++)
      for (unsigned j = 0; j < rp.Nf; j++) {
        re.push_back(rp.ep[l][j].real());
        im.push_back(rp.ep[l][j].imag());
      }
    d.power_re.push_back(re);
    d.power_im.push_back(im);
    mithra_power_desc w = mithra_power_desc();
    w.N = (int32_t)rp.N;
    w.Nl = (int32_t)rp.Nl;
    w.Nf = (int32_t)rp.Nf;
    w.pc = rp.pc;
    d.power.push_back(w);
  }
  for (size_t o = 0; o < d.power.size(); o++) {  // the vectors no longer move
    d.power[o].z = d.power_z[o].data();
    d.power[o].twiddle_re = d.power_re[o].data();
    d.power[o].twiddle_im = d.power_im[o].data();
  }

  d.time.time = s.time_;
  d.time.time_bunch = s.timeBunch_;
  d.time.n_time = s.nTime_;
  d.time.n_time_bunch = s.nTimeBunch_;
  d.total_time = s.mesh_.totalTime_;
  d.n_particles = s.chargeVectorn_.size();
}

int solve_on_gpu(Solver& s, int precision, int device, std::string& error) {
  GpuDescriptors d;
  describe_for_gpu(s, d);
  mithra_ctx* ctx = NULL;
  // capacity: the particles plus room for the copies the single-domain z-face exchange appends
  const size_t capacity = 2 * d.n_particles + 1024;
  int r = mithra_gpu_create(&d.grid, &d.push, precision, device, capacity, &ctx);
  if (r) {
    error = "mithra_gpu_create failed";
    return r;
  }
  char buf[512];
  auto check = [&](int status, const char* what) {
    if (status && error.empty()) {
      mithra_gpu_last_error(ctx, buf, sizeof buf);
      error = std::string(what) + ": " + buf;
    }
    return status;
  };
  const size_t nodes = (size_t)s.N1N0_ * s.np_;
  std::vector<double> rec;
  long steps = 0;
  if (check(mithra_gpu_set_undulators(ctx, d.undulators.data(), (int)d.undulators.size()), "undulators") ||
      check(mithra_gpu_set_seed(ctx, &d.seed), "seed") ||
      check(mithra_gpu_set_external_fields(ctx, d.ext_fields.data(), (int)d.ext_fields.size()), "external fields") ||
      check(mithra_gpu_set_power(ctx, d.power.data(), (int)d.power.size()), "power outputs") ||
      check(mithra_gpu_upload_fields(ctx, &(*s.anp1_)[0][0], &(*s.an_)[0][0], &(*s.anm1_)[0][0]), "fields"))
    goto done;
  if (s.mesh_.spaceCharge_ &&
      check(mithra_gpu_upload_scalar(ctx, &(*s.fnp1_)[0], &(*s.fn_)[0], &(*s.fnm1_)[0]), "scalar potential"))
    goto done;
  rec.reserve(11 * d.n_particles);
  for (std::list<Charge>::const_iterator q = s.chargeVectorn_.begin(); q != s.chargeVectorn_.end(); ++q) {
    rec.push_back(q->q);
    for (int c = 0; c < 3; c++) rec.push_back(q->rnp[c]);
    for (int c = 0; c < 3; c++) rec.push_back(q->rnm[c]);
    for (int c = 0; c < 3; c++) rec.push_back(q->gb[c]);
    rec.push_back(q->e);
  }
  if (check(mithra_gpu_upload_particles(ctx, rec.data(), d.n_particles), "particles") ||
      check(mithra_gpu_set_time(ctx, &d.time), "time state") ||
      check(mithra_gpu_run_prelude(ctx), "prelude"))
    goto done;
  {
    // the main loop runs while time_ < totalTime_, time_ advancing by repeated addition
    mithra_time_state t;
    if (check(mithra_gpu_get_time(ctx, &t), "time state")) goto done;
    for (double time = t.time; time < d.total_time; time += s.mesh_.timeStep_) steps++;
  }
  // march in chunks, writing each chunk's power rows into the reference's own streams
  for (long done_steps = 0; done_steps < steps;) {
    const long n = std::min<long>(steps - done_steps, 1024);
    if (check(mithra_gpu_run(ctx, n), "march")) goto done;
    size_t nv = 0;
    if (check(mithra_gpu_power_rows(ctx, NULL, 0, &nv), "power rows")) goto done;
    std::vector<double> rows(nv);
    if (nv && check(mithra_gpu_power_rows(ctx, rows.data(), nv, &nv), "power rows")) goto done;
    size_t per_row = 0;
    for (size_t o = 0; o < d.power.size(); o++) per_row += (size_t)d.power[o].N * (1 + d.power[o].Nl);
    for (size_t row = 0; per_row && row < nv / per_row; row++) {
      const double* v = rows.data() + row * per_row;
      for (size_t o = 0; o < d.power.size(); o++) {
        SampleRadiationPower& rp = s.rp_[d.power_fel[o]];
        for (unsigned l = 0; l < rp.Nl; l++) {
          for (unsigned k = 0; k < rp.N; k++)
            *(rp.file[l]) << v[k * (1 + rp.Nl)] << "\t" << v[k * (1 + rp.Nl) + 1 + l] << "\t";
          *(rp.file[l]) << std::endl;
        }
        v += (size_t)rp.N * (1 + rp.Nl);
      }
    }
    done_steps += n;
  }
  {
    // the final state back into the solver's members
    if (check(mithra_gpu_download_fields(ctx, &(*s.anp1_)[0][0], &(*s.an_)[0][0], &(*s.anm1_)[0][0]), "fields"))
      goto done;
    if (s.mesh_.spaceCharge_ &&
        check(mithra_gpu_download_scalar(ctx, &(*s.fnp1_)[0], &(*s.fn_)[0], &(*s.fnm1_)[0]), "scalar potential"))
      goto done;
    size_t n = 0;
    if (check(mithra_gpu_download_particles(ctx, NULL, 0, &n), "particles")) goto done;
    rec.assign(11 * n, 0.0);
    if (check(mithra_gpu_download_particles(ctx, rec.data(), n, &n), "particles")) goto done;
    s.chargeVectorn_.clear();
    for (size_t i = 0; i < n; i++) {
      const double* v = &rec[11 * i];
      Charge q;
      q.q = v[0];
      for (int c = 0; c < 3; c++) {
        q.rnp[c] = v[1 + c];
        q.rnm[c] = v[4 + c];
        q.gb[c] = v[7 + c];
      }
      q.e = v[10];
      s.chargeVectorn_.push_back(q);
    }
    std::vector<float> en(3 * nodes), bn(3 * nodes);
    if (check(mithra_gpu_download_eb(ctx, en.data(), bn.data()), "E and B")) goto done;
    for (size_t m = 0; m < nodes; m++)
      for (int c = 0; c < 3; c++) {
        s.en_[m][c] = en[3 * m + c];
        s.bn_[m][c] = bn[3 * m + c];
      }
    mithra_time_state t;
    if (check(mithra_gpu_get_time(ctx, &t), "time state")) goto done;
    s.time_ = t.time;
    s.timeBunch_ = t.time_bunch;
    s.nTime_ = (unsigned int)t.n_time;
    s.nTimeBunch_ = (unsigned int)t.n_time_bunch;
  }
done:
  const int status = error.empty() ? 0 : -1;
  mithra_gpu_destroy(ctx);
  return status;
}

template <class Base>
void GpuSolver<Base>::solve() {
  this->initialize();  // the reference's parsing results and FP64 initialisation, unchanged
  std::string error;
  if (solve_on_gpu(*this, precision_, device_, error)) fail_like_reference(error);
}

template class GpuSolver<FdTd>;
template class GpuSolver<FdTdSC>;

}  // namespace MITHRA
