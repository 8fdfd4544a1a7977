// Host-side FP64 initialisation (see setup.h).  Each block cites the reference lines it
// restates; expressions keep the reference's operation order so that, compiled with
// -ffp-contract=off against the same libm, the particle records and coefficients are
// bit-identical to the reference's.
#include "setup.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace mithra {
namespace host {

namespace {
[[noreturn]] void die(const std::string& m) { throw std::runtime_error(m); }
double norm2(const Vec3& v) { return v[0] * v[0] + v[1] * v[1] + v[2] * v[2]; }
double dot(const Vec3& a, const Vec3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
Vec3 cross(const Vec3& x, const Vec3& y) {
  return {x[1] * y[2] - x[2] * y[1], x[2] * y[0] - x[0] * y[2], x[0] * y[1] - x[1] * y[0]};
}
}  // namespace

// The bunch generator's quasi-random sequence (src/stdinclude.cpp:45-73): point `index` of the
// Halton sequence in dimension `dim`, reflected, i.e. 1 minus the radical inverse of index + 1 in
// the dim-th prime base.
double halton(unsigned dim, unsigned index) {
  static const int kPrimes[20] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61, 67, 71};
  if (dim >= 20) die(" dimension can not be larger than 20. ");
  const int base = kPrimes[dim];
  double inverse = 0.0;
  int scale = base;
  for (int digits = (int)(index + 1); digits > 0; digits /= base) {
    inverse += (digits % base) / (double)scale;
    scale *= base;
  }
  return 1.0 - inverse;
}

// a modulo b in [0, b) for b > 0 (src/stdinclude.cpp:88-93); a zero remainder comes out as +0.
double pmod(double a, double b) {
  const double r = std::fmod(a, b);
  return r + (r < 0.0 ? b : 0.0);
}

// Signal::self, src/classes.cpp:557-598.
double Signal::self(double t, double phase) const {
  if (std::fabs(t - t0) > 10.0 * s) return 0.0;
  switch (type) {
    case NEUMANN:
      return -std::cos(2 * PI * f0 * (t - t0) + cep + phase) * 2.7724 * (t - t0) / (s * s) *
             std::exp(-1.3863 * (t - t0) * (t - t0) / (s * s));
    case GAUSSIAN: {
      double u = (t - t0) / s;
      return std::cos(2 * PI * f0 * (t - t0) + cep + phase) * std::exp(-1.3863 * (u * u));
    }
    case SECANT:
      return std::cos(2 * PI * f0 * (t - t0) + cep + phase) / std::cosh((t - t0) / s);
    case FLATTOP:
      if (t - t0 <= -s / 2.0) {
        double u = (t - t0 + s / 2.0) * f0 / nR;
        return std::cos(2 * PI * f0 * (t - t0) + cep + phase) * std::exp(-(u * u));
      } else if (t - t0 <= s / 2.0) {
        return std::cos(2 * PI * f0 * (t - t0) + cep + phase);
      } else {
        double u = (t - t0 - s / 2.0) * f0 / nR;
        return std::cos(2 * PI * f0 * (t - t0) + cep + phase) * std::exp(-(u * u));
      }
    case INVGAUSSIAN: {
      double u0 = (t - t0) / sigmaInvG[0], u1 = (t - t0) / sigmaInvG[1];
      double env = std::pow((1.0 + u0 * u0) * (1.0 + u1 * u1), 0.25);
      if (t - t0 <= -s / 2.0) {
        double u = (t - t0 + s / 2.0) * f0 / nR;
        return std::cos(2 * PI * f0 * (t - t0) + cep + phase) * env * std::exp(-(u * u));
      } else if (t - t0 <= s / 2.0) {
        return std::cos(2 * PI * f0 * (t - t0) + cep + phase) * env;
      } else {
        double u = (t - t0 - s / 2.0) * f0 / nR;
        return std::cos(2 * PI * f0 * (t - t0) + cep + phase) * env * std::exp(-(u * u));
      }
    }
  }
  return 0.0;
}

// Seed::fields, src/classes.cpp:740-855.
void Seed::fields(const Vec3& r, double time, Vec3& a) const {
  Vec3 rl{r[0], r[1], gamma * (r[2] + beta * c0 * (time + dt))};
  double tl = gamma * (time + dt + beta / c0 * r[2]);
  Vec3 rv{rl[0] - position[0], rl[1] - position[1], rl[2] - position[2]};
  double z = dot(rv, direction);
  tl -= z / c0;
  double p = 0.0, tsignal;
  if (seedType == PLANEWAVE) {
    tsignal = signal.self(tl, p);
    if (std::fabs(tsignal) < 1.0e-6) a = {0.0, 0.0, 0.0};
    else for (int c = 0; c < 3; c++) a[c] = amplitude * tsignal * polarization[c];
  } else if (seedType == PLANEWAVETRUNCATED) {
    tsignal = signal.self(tl, p);
    double x = dot(rv, polarization);
    Vec3 yv = cross(direction, polarization);
    double y = dot(rv, yv);
    if (std::fabs(tsignal) < 1.0e-6 || std::fabs(x) > radius[0] || std::fabs(y) > radius[1]) a = {0.0, 0.0, 0.0};
    else for (int c = 0; c < 3; c++) a[c] = amplitude * tsignal * polarization[c];
  } else if (seedType == GAUSSIANBEAM || seedType == SUPERGAUSSIANBEAM) {
    tsignal = signal.self(tl, p);
    if (std::fabs(tsignal) < 1.0e-6) {
      if (seedType == GAUSSIANBEAM) a = {0.0, 0.0, 0.0};
      else a = {0.0, 0.0, 0.0};
    } else {
      double x = dot(rv, polarization);
      Vec3 yv = cross(direction, polarization);
      double y = dot(rv, yv);
      double ll = c0 / signal.f0;
      double zRp = PI * radius[0] * radius[0] / ll;
      double wrp = std::sqrt(1.0 + z * z / (zRp * zRp));
      double zRs = PI * radius[1] * radius[1] / ll;
      double wrs = std::sqrt(1.0 + z * z / (zRs * zRs));
      auto term = [&]() {
        double u = x / (zRp * wrp), v = y / (zRs * wrs);
        double ph = 0.5 * (std::atan(z / zRp) + std::atan(z / zRs) - PI) - PI * z / ll * (u * u + v * v);
        double ts = signal.self(tl, ph);
        double gx = x / (radius[0] * wrp), gy = y / (radius[1] * wrs);
        double t = std::exp(-(gx * gx) - (gy * gy)) / std::sqrt(wrs * wrp) * amplitude;
        return t * ts;
      };
      if (seedType == GAUSSIANBEAM) {
        double v = term();
        for (int c = 0; c < 3; c++) a[c] = v * polarization[c];
      } else {
        for (int i = -order[0]; i <= order[0]; i++)
          for (int j = -order[1]; j <= order[1]; j++) {
            double v = term();
            for (int c = 0; c < 3; c++) a[c] += v * polarization[c];
          }
      }
    }
  }
  a[2] *= gamma;
}

namespace {

// Bunch::initializeManual, src/classes.cpp:87-99.
void init_manual(const BunchInit& b, std::vector<Charge>& qv, int ia) {
  Charge c;
  c.q = b.cloudCharge;
  c.rnp = b.position[ia];
  for (int d = 0; d < 3; d++) c.gb[d] = b.initialGamma * b.betaVector[d];
  qv.push_back(c);
}

namespace {
// Draws of an ellipsoid bunch from the Halton sequence, as Bunch::initializeEllipsoid lays them
// out (src/classes.cpp:104-298): draw i of a bunch uses point base + i (base = particles already
// in the list) of dimensions 0/1 (transverse position, Box-Muller radius and angle), 2/3
// (longitudinal position), 4/5 and 6/7 (momentum spread); a beamlet's shot noise uses dimensions
// 8/9 at the index of its wavelength slot.  Every expression keeps the reference's evaluation
// order, so the records come out bit for bit the same.
struct EllipsoidDraws {
  const BunchInit& b;
  unsigned base;

  // sigma sqrt(-2 ln u) times cos or sin of 2 pi v, (u, v) the points of dimensions (du, dv)
  double normal(double sigma, unsigned du, unsigned dv, unsigned i, bool cosine) const {
    const double radius = sigma * std::sqrt(-2.0 * std::log(halton(du, base + i)));
    const double angle = 2.0 * PI * halton(dv, base + i);
    return radius * (cosine ? std::cos(angle) : std::sin(angle));
  }
  // longitudinal offset of a draw of the main part
  double z_main(unsigned i) const {
    if (b.distribution == "uniform") return (2.0 * halton(2, base + i) - 1.0) * b.sigmaPosition[2];
    return normal(b.sigmaPosition[2], 2, 3, i, false);
  }
  // longitudinal offset of a draw of the uniform profile's edges: a normal of rms 2 lambda moved
  // out past +-sigma_z
  double z_edge(unsigned i) const {
    const double z = normal(2.0 * b.lambda, 2, 3, i, false);
    return z + ((z < 0.0) ? (-b.sigmaPosition[2]) : (b.sigmaPosition[2]));
  }
};
}  // namespace

// An ellipsoid bunch, Bunch::initializeEllipsoid (src/classes.cpp:104-298) on one rank: the main
// part's draws, for a uniform profile followed by the draws of its soft edges, each kept inside the
// truncation and turned into a beamlet of four particles a quarter wavelength apart (one particle
// when no wavelength is set).  The reference's `random` generator draws from an unseeded rand(),
// so no two runs agree; it is refused here.
void init_ellipsoid(BunchInit b, std::vector<Charge>& qv, int ia) {
  if (b.bF > 2.0 || b.bF < 0.0) die("The bunching factor can not be larger than one or a negative value !!!");
  if (b.distribution != "uniform" && b.distribution != "gaussian")
    die("The longitudinal type is not correctly given to the code !!!");
  if (b.generator == "random")
    die("generator = random draws from an unseeded random number generator and cannot reproduce a run; use halton");
  if (b.numberOfParticles % 4 != 0) b.numberOfParticles += 4 - b.numberOfParticles % 4;
  const unsigned per_beamlet = (b.lambda == 0.0) ? 1 : 4;
  const unsigned n_main = b.numberOfParticles / per_beamlet;
  // the uniform profile's edges add 2 lambda sqrt(2 pi) / (2 sigma_z) of the main part's draws
  const unsigned n_draws =
      (b.distribution == "uniform")
          ? unsigned(n_main * (1.0 + 2.0 * b.lambda * std::sqrt(2.0 * PI) / (2.0 * b.sigmaPosition[2])))
          : n_main;
  const EllipsoidDraws draw{b, (unsigned)qv.size()};
  auto z_of = [&](unsigned i) { return i < n_main ? draw.z_main(i) : draw.z_edge(i); };

  // Shot noise: the bunch front (smallest z of all draws) anchors the wavelength slots; each slot
  // has its own bunching amplitude (default 1 / sqrt(electrons per wavelength)) and phase.
  double z_front = 1e100, amplitude = 0.0;
  if (b.shotNoise) {
    for (unsigned i = 0; i < n_draws; i++) z_front = std::min(z_of(i), z_front);
    z_front = z_front + b.position[ia][2];
    const double electrons_per_wavelength = b.cloudCharge * b.lambda / (2.0 * b.sigmaPosition[2]);
    amplitude = (b.bF == 0.0) ? 1.0 / std::sqrt(electrons_per_wavelength) : b.bF;
  }
  auto add_beamlet = [&](const Charge& centre) {
    Charge p = centre;
    for (unsigned m = 0; m < per_beamlet; m++) {
      if (b.shotNoise) {
        const unsigned slot = int((centre.rnp[2] - z_front) / b.lambda);
        const double a = amplitude * std::sqrt(-2.0 * std::log(halton(8, slot)));
        p.rnp[2] = centre.rnp[2] - b.lambda / 4 * m;
        p.rnp[2] -= b.lambda / PI * a * std::sin(2.0 * PI / b.lambda * p.rnp[2] + 2.0 * PI * halton(9, slot));
      } else if (b.lambda != 0.0) {
        p.rnp[2] = centre.rnp[2] - b.lambda / 4 * m;
        p.rnp[2] -= b.lambda / PI * b.bF * std::sin(2.0 * PI / b.lambda * p.rnp[2] + b.bFP * PI / 180.0);
      }
      qv.push_back(p);
    }
  };

  Charge centre;
  centre.q = b.cloudCharge / b.numberOfParticles;
  Vec3 gb_mean;
  for (int d = 0; d < 3; d++) gb_mean[d] = b.initialGamma * b.betaVector[d];
  for (unsigned i = 0; i < n_draws; i++) {
    const Vec3 r{draw.normal(b.sigmaPosition[0], 0, 1, i, true), draw.normal(b.sigmaPosition[1], 0, 1, i, false),
                 z_of(i)};
    const Vec3 t{draw.normal(b.sigmaGammaBeta[0], 4, 5, i, true), draw.normal(b.sigmaGammaBeta[1], 4, 5, i, false),
                 draw.normal(b.sigmaGammaBeta[2], 6, 7, i, true)};
    if (std::fabs(r[0]) < b.tranTrun && std::fabs(r[1]) < b.tranTrun && std::fabs(r[2]) < b.longTrun) {
      for (int d = 0; d < 3; d++) centre.rnp[d] = b.position[ia][d] + r[d];
      for (int d = 0; d < 3; d++) centre.gb[d] = gb_mean[d] + t[d];
      add_beamlet(centre);
    }
  }
}

// Bunch::initialize3DCrystal, src/classes.cpp:307-353 (note: the reference clears the charge
// vector first, so only the last position survives for several positions).
void init_crystal(const BunchInit& b, std::vector<Charge>& qv, int ia) {
  const unsigned nprod = b.numbers[0] * b.numbers[1] * b.numbers[2];
  if (nprod == 0 || b.numberOfParticles % nprod != 0) die("The number of the particles and their lattice numbers do not match !!!");
  Vec3 gb;
  for (int d = 0; d < 3; d++) gb[d] = b.initialGamma * b.betaVector[d];
  const unsigned np = b.numberOfParticles / nprod;
  qv.clear();
  for (unsigned i = 0; i < b.numbers[0]; i++)
    for (unsigned j = 0; j < b.numbers[1]; j++)
      for (unsigned k = 0; k < b.numbers[2]; k++)
        for (unsigned l = 0; l < np; l++) {
          Charge c;
          c.q = b.cloudCharge / b.numberOfParticles;
          c.rnp[0] = b.position[ia][0] + (i + 1.0 - 0.5 * b.numbers[0]) * b.latticeConstants[0];
          c.rnp[1] = b.position[ia][1] + (j + 1.0 - 0.5 * b.numbers[1]) * b.latticeConstants[1];
          c.rnp[2] = b.position[ia][2] + (k + 1.0 - 0.5 * b.numbers[2]) * b.latticeConstants[2];
          c.rnp[0] += 0.5 * b.sigmaPosition[0] * std::sqrt(-2.0 * std::log(halton(0, i))) * std::sin(2.0 * PI * halton(1, i));
          c.rnp[1] += 0.5 * b.sigmaPosition[1] * std::sqrt(-2.0 * std::log(halton(2, i))) * std::sin(2.0 * PI * halton(3, i));
          c.rnp[2] += 0.5 * b.sigmaPosition[2] * std::sqrt(-2.0 * std::log(halton(4, i))) * std::sin(2.0 * PI * halton(5, i));
          c.gb = gb;
          c.gb[0] += b.sigmaGammaBeta[0] * std::sqrt(-2.0 * std::log(halton(6, i))) * std::sin(2.0 * PI * halton(7, i));
          c.gb[1] += b.sigmaGammaBeta[1] * std::sqrt(-2.0 * std::log(halton(8, i))) * std::sin(2.0 * PI * halton(9, i));
          c.gb[2] += b.sigmaGammaBeta[2] * std::sqrt(-2.0 * std::log(halton(10, i))) * std::sin(2.0 * PI * halton(11, i));
          qv.push_back(c);
        }
}

// Bunch::initializeFile, src/classes.cpp:359-413: six columns x y z gbx gby gbz per particle.
void init_file(const BunchInit& b, std::vector<Charge>& qv, int ia) {
  qv.clear();
  std::ifstream f(b.fileName.c_str());
  Charge c;
  c.q = b.cloudCharge / b.numberOfParticles;
  while (f.good()) {
    f >> c.rnp[0] >> c.rnp[1] >> c.rnp[2] >> c.gb[0] >> c.gb[1] >> c.gb[2];
    for (int d = 0; d < 3; d++) c.rnp[d] += b.position[ia][d];
    qv.push_back(c);
  }
  if (b.numberOfParticles != qv.size())
    die("The number of the particles and the file size do not match !!! The file contains " + std::to_string(qv.size()) + " particles.");
}

// Solver::computeFileGamma, src/solver.cpp:509-541.
void compute_file_gamma(BunchInit& b) {
  std::ifstream f(b.fileName.c_str());
  double ignore;
  Vec3 gb{0, 0, 0};
  b.initialGamma = 0.0;
  b.initialDirection = {0, 0, 0};
  while (f.good()) {
    f >> ignore >> ignore >> ignore >> gb[0] >> gb[1] >> gb[2];
    b.initialGamma += std::sqrt(1 + norm2(gb));
    for (int d = 0; d < 3; d++) b.initialDirection[d] += gb[d];
  }
  b.initialGamma /= b.numberOfParticles;
  const double n = std::sqrt(norm2(b.initialDirection));
  for (int d = 0; d < 3; d++) b.initialDirection[d] /= n;
}

void scale_beam(Beam& b, double c0) {  // src/solver.cpp:77-125
  b.c0 = c0;
  b.signal.t0 /= c0;
  b.signal.f0 *= c0;
  b.signal.s /= c0;
  b.l = c0 / b.signal.f0;
  b.zR = {PI * b.radius[0] * b.radius[0] / b.l, PI * b.radius[1] * b.radius[1] / b.l};
}

}  // namespace

void Setup::dev_check(int r) {
  if (r) die(dev_err);
}

// Solver::initializeBunch for device initialisation: every bunch-initialization group must be
// an ellipsoid with the Halton generator; each position of a group is one call of
// Bunch::initializeEllipsoid (src/classes.cpp:104-298) with the scalar prologue computed here
// exactly as init_ellipsoid does and the particle loops on the device.
void Setup::init_bunch_on_device() {
  for (auto& bi : job.bunch.inits) {
    if (bi.type != "ellipsoid")
      die("device initialisation supports ellipsoid bunches only (bunch type " + bi.type + ")");
    if (bi.generator == "random") die("device initialisation supports the Halton generator only");
    if (bi.distribution != "uniform" && bi.distribution != "gaussian")
      die("The longitudinal type is not correctly given to the code !!!");
  }
  for (auto& bi : job.bunch.inits) {
    if (bi.position.empty()) bi.position.push_back({0.0, 0.0, 0.0});
    const size_t group_start = dstore.n;
    for (size_t ia = 0; ia < bi.position.size(); ia++) {
      BunchInit b = bi;
      if (b.numberOfParticles % 4 != 0) b.numberOfParticles += 4 - b.numberOfParticles % 4;
      if (b.bF > 2.0 || b.bF < 0.0) die("The bunching factor can not be larger than one or a negative value !!!");
      devinit::Ellipsoid e;
      e.Np = b.numberOfParticles;
      e.Np0 = (unsigned)(dstore.n - group_start);
      e.ng = (b.lambda == 0.0) ? 1 : 4;
      e.n_main = e.Np / e.ng;
      e.n_taper = unsigned(e.Np / e.ng * (1.0 + 2.0 * b.lambda * std::sqrt(2.0 * PI) / (2.0 * b.sigmaPosition[2])));
      e.gaussian = (b.distribution == "gaussian") ? 1 : 0;
      e.shot_noise = b.shotNoise ? 1 : 0;
      e.q = b.cloudCharge / e.Np;
      for (int d = 0; d < 3; d++) {
        e.gb[d] = b.initialGamma * b.betaVector[d];
        e.sig_r[d] = b.sigmaPosition[d];
        e.sig_gb[d] = b.sigmaGammaBeta[d];
        e.pos[d] = b.position[ia][d];
      }
      e.tran_trun = b.tranTrun;
      e.long_trun = b.longTrun;
      e.lambda = b.lambda;
      e.bF_user = b.bF;
      e.bFP = b.bFP;
      double zmin = 1e100, bF = 0.0;
      if (b.shotNoise) {
        dev_check(devinit::candidate_zmin(dstore.device, e, &zmin, dev_err, sizeof dev_err));
        zmin = zmin + b.position[ia][2];
        const double Ne = b.cloudCharge * b.lambda / (2.0 * b.sigmaPosition[2]);
        bF = (b.bF == 0.0) ? 1.0 / std::sqrt(Ne) : b.bF;
      }
      dev_check(devinit::generate(dstore, e, zmin, bF, dev_err, sizeof dev_err));
    }
  }
}

void Setup::initialize() {
  Mesh& mesh = job.mesh;
  Bunch& bunch = job.bunch;
  Seed& seed = job.seed;
  std::vector<Undulator>& und = job.undulators;
  if (mesh.lengthScale == 0.0 || mesh.timeScale == 0.0) die("length-scale and time-scale must be given in MESH");
  // Solver::Solver, src/solver.cpp:58-61.
  c0 = C0() / mesh.lengthScale * mesh.timeScale;
  m0 = MU_ZERO / mesh.lengthScale;
  e0 = 1.0 / (c0 * c0 * m0);

  // Solver::setSimulationParameters, src/solver.cpp:68-214.
  scale_beam(seed, c0);
  for (auto& u : und) scale_beam(u, c0);
  for (auto& e : job.extFields) scale_beam(e, c0);
  seed.amplitude = seed.a0 * EM * c0 / EC;
  for (auto& u : und) u.amplitude = u.a0 * EM * c0 * 2 * PI * u.signal.f0 / EC;
  for (auto& e : job.extFields) e.amplitude = e.a0 * EM * c0 * 2 * PI * e.signal.f0 / EC;
  double gam = 0.0;
  for (auto& b : bunch.inits) {
    if (b.type == "file") compute_file_gamma(b);
    gam += b.initialGamma / bunch.inits.size();
  }
  double gmin = 1.0e100, gmax = -1.0e100, g = 0.0;
  for (auto& u : und) {
    if (u.type == STATIC) {
      g = gam / std::sqrt(1.0 + u.k * u.k / 2.0);
      gmin = (gmin < g) ? gmin : g;
      gmax = (gmax > g) ? gmax : g;
    } else if (u.signal.type == FLATTOP) {
      g = gam / std::sqrt(1.0 + u.a0 * u.a0 / 2.0);
      gmin = (gmin < g) ? gmin : g;
      gmax = (gmax > g) ? gmax : g;
    } else {
      g = gam / std::sqrt(1.0 + u.a0 * u.a0 / 2.0);
      gmin = (gmin < g) ? gmin : g;
      g = gam;
      gmax = (gmax > g) ? gmax : g;
    }
  }
  if (mesh.gamma == -1.0) gamma = (und.size() == 0) ? gam : (gmin + gmax) / 2.0;
  else gamma = mesh.gamma;
  beta = std::sqrt(1.0 - 1.0 / (gamma * gamma));
  for (auto& u : und)
    if (u.type == OPTICAL) u.lu /= (1 + beta);
  std::sort(und.begin(), und.end(), [](const Undulator& x, const Undulator& y) { return x.rb < y.rb; });
  for (auto it = und.rbegin(); it != und.rend(); ++it) it->rb -= und[0].rb;
  for (auto& b : bunch.inits) {
    b.initialBeta = std::sqrt(1.0 - 1.0 / (b.initialGamma * b.initialGamma));
    for (int d = 0; d < 3; d++) b.betaVector[d] = b.initialBeta * b.initialDirection[d];
    b.lambda = (und.size() > 0) ? und[0].lu / (2.0 * gamma * gamma) * b.betaVector[2] / beta : 0.0;
  }
  seed.beta = beta;
  seed.gamma = gamma;

  // Solver::initializeBunch, src/solver.cpp:1130-1178.
  if (device_init) init_bunch_on_device();
  for (auto& b : bunch.inits) {
    if (device_init) break;
    std::vector<Charge> qv;
    if (b.position.empty()) b.position.push_back({0.0, 0.0, 0.0});
    if (b.type == "manual")
      for (size_t ia = 0; ia < b.position.size(); ia++) init_manual(b, qv, (int)ia);
    else if (b.type == "ellipsoid")
      for (size_t ia = 0; ia < b.position.size(); ia++) init_ellipsoid(b, qv, (int)ia);
    else if (b.type == "3D-crystal")
      for (size_t ia = 0; ia < b.position.size(); ia++) init_crystal(b, qv, (int)ia);
    else if (b.type == "file")
      for (size_t ia = 0; ia < b.position.size(); ia++) init_file(b, qv, (int)ia);
    charges.insert(charges.end(), qv.begin(), qv.end());
  }
  timeBunch = time;

  // Solver::lorentzBoostMesh, src/solver.cpp:220-257.
  mesh.meshLength[2] *= gamma;
  mesh.meshResolution[2] *= gamma;
  mesh.meshCenter[2] *= gamma;
  mesh.totalTime /= gamma;
  mesh.timeShift /= gamma;
  if (mesh.solver == NSFD) {
    double t = 1.0 / std::sqrt((mesh.meshResolution[2] / mesh.meshResolution[0]) * (mesh.meshResolution[2] / mesh.meshResolution[0]) +
                               (mesh.meshResolution[2] / mesh.meshResolution[1]) * (mesh.meshResolution[2] / mesh.meshResolution[1]));
    if (t < 1.02) {
      mesh.meshResolution[0] *= 1.02 / t;
      mesh.meshResolution[1] *= 1.02 / t;
    }
    mesh.timeStep = mesh.meshResolution[2] / c0;
  } else {
    mesh.timeStep = 0.98 / (c0 * std::sqrt(1.0 / (mesh.meshResolution[0] * mesh.meshResolution[0]) +
                                           1.0 / (mesh.meshResolution[1] * mesh.meshResolution[1]) +
                                           1.0 / (mesh.meshResolution[2] * mesh.meshResolution[2])));
  }

  // Solver::initializeMesh, src/solver.cpp:601-689 (one domain).
  N0 = (int)(mesh.meshLength[0] / mesh.meshResolution[0]) + 2;
  N1 = (int)(mesh.meshLength[1] / mesh.meshResolution[1]) + 2;
  N2 = (int)(mesh.meshLength[2] / mesh.meshResolution[2]) + 2;
  N1N0 = N1 * N0;
  mesh.meshLength[0] = (N0 - 1) * mesh.meshResolution[0];
  mesh.meshLength[1] = (N1 - 1) * mesh.meshResolution[1];
  mesh.meshLength[2] = (N2 - 1) * mesh.meshResolution[2];
  np = N2;
  k0 = 0;
  xmin = mesh.meshCenter[0] - mesh.meshLength[0] / 2.0;
  xmax = mesh.meshCenter[0] + mesh.meshLength[0] / 2.0;
  ymin = mesh.meshCenter[1] - mesh.meshLength[1] / 2.0;
  ymax = mesh.meshCenter[1] + mesh.meshLength[1] / 2.0;
  zmin = mesh.meshCenter[2] - mesh.meshLength[2] / 2.0;
  zmax = mesh.meshCenter[2] + mesh.meshLength[2] / 2.0;
  zp[0] = zmin + (unsigned)(0 + k0) * mesh.meshResolution[2];
  zp[1] = zmin + (unsigned)(np - 1 + k0) * mesh.meshResolution[2];
  timep1 = mesh.timeStep;
  time = 0.0;
  timem1 = -mesh.timeStep;

  auto in_domain = [&](double z) {
    double zr = pmod(z - zmin, mesh.meshLength[2]) + zmin;
    return (zr >= zp[0]) && (zr < zp[1]);
  };
  auto distribute = [&]() {  // Solver::distributeParticles with one rank, src/solver.cpp:429-487
    if (device_init) {
      dev_check(devinit::distribute(dstore, zmin, mesh.meshLength[2], zp[0], zp[1], dev_err, sizeof dev_err));
      return;
    }
    std::vector<Charge> kept;
    kept.reserve(charges.size());
    for (auto& c : charges)
      if (in_domain(c.rnp[2])) kept.push_back(c);
    charges.swap(kept);
  };

  // Solver::lorentzBoostBunch, src/solver.cpp:263-423.
  bunch.timeStep /= gamma;
  bunch.rhythm /= gamma;  // src/solver.cpp:281-285
  bunch.vtkRhythm /= gamma;
  for (auto& t : bunch.profileTime) t /= gamma;
  bunch.profileRhythm /= gamma;
  if (bunch.profile && bunch.profileRhythm == 0 && bunch.profileTime.empty())
    die("The profiling rhythm of the bunch is zero and no time is set although profiling of the bunch is activated !!!");
  if (bunch.sampling && bunch.rhythm == 0)
    die("The sampling rhythm of the bunch is zero although sampling is activated !!!");
  if (bunch.timeStep == 0) bunch.timeStep = mesh.timeStep;
  else bunch.timeStep = mesh.timeStep / std::ceil(mesh.timeStep / bunch.timeStep);
  nUpdateBunch = mesh.timeStep / bunch.timeStep;
  double zmaxL = -1.0e100;
  if (device_init) dev_check(devinit::boost(dstore, gamma, beta, &zmaxL, dev_err, sizeof dev_err));
  for (auto& q : charges) {
    double gq = std::sqrt(1.0 + norm2(q.gb));
    double bz = q.gb[2] / gq;
    q.rnp[2] *= gamma;
    q.gb[2] = gamma * gq * (bz - beta);
    zmaxL = std::max(zmaxL, q.rnp[2]);
  }
  double zmaxG = zmaxL;
  if (und.size() > 0) {
    double nl = (und[0].type == STATIC) ? 2.0 : 5.0 * und[0].signal.nR;
    if (und[0].dist == 0.0) und[0].dist = nl * und[0].lu;
    dt_shift = -1.0 / (beta * und[0].c0) * (zmaxG + und[0].dist / gamma);
  }
  seed.dt = dt_shift;
  bunch.zu = zmaxG;
  bunch.beta = beta;
  if (device_init) dev_check(devinit::back_propagate(dstore, bunch.zu, beta, dev_err, sizeof dev_err));
  for (auto& q : charges) {
    double gq = std::sqrt(1.0 + norm2(q.gb));
    q.rnp[0] += q.gb[0] / gq * (q.rnp[2] - bunch.zu) * beta;
    q.rnp[1] += q.gb[1] / gq * (q.rnp[2] - bunch.zu) * beta;
    q.rnp[2] += q.gb[2] / gq * (q.rnp[2] - bunch.zu) * beta;
  }
  if (mesh.optimizePosition && und.size() > 0) {
    double zL = 0.0, bzL = 0.0;
    if (device_init) dev_check(devinit::sums_z_bz(dstore, &zL, &bzL, dev_err, sizeof dev_err));
    for (auto& q : charges) {
      zL += q.rnp[2];
      bzL += q.gb[2] / std::sqrt(1 + norm2(q.gb));
    }
    double zG = zL, bzG = bzL;
    unsigned NqG = (unsigned)particle_count();
    zG /= NqG;
    bzG /= NqG;
    double shift = bzG * (zmaxG + und[0].dist / gamma - zG) / (bzG + beta) + zG;
    zmaxG -= shift;
    bunch.zu = zmaxG;
    dt_shift = -1.0 / (beta * und[0].c0) * (zmaxG + und[0].dist / gamma);
    seed.dt = dt_shift;
    if (device_init) dev_check(devinit::shift_z(dstore, shift, dev_err, sizeof dev_err));
    for (auto& q : charges) q.rnp[2] -= shift;
  }
  distribute();
  if (mesh.totalDist > 0.0) {
    double Lu = 0.0;
    for (auto& u : und) Lu += u.lu * u.length / gamma;
    double zEnd = mesh.totalDist / gamma;
    double zMin = 1e100, bz = 0;
    if (device_init) {
      dev_check(devinit::min_z(dstore, &zMin, dev_err, sizeof dev_err));
      dev_check(devinit::sums_z_bz(dstore, nullptr, &bz, dev_err, sizeof dev_err));
    }
    for (auto& q : charges) {
      zMin = std::min(zMin, q.rnp[2]);
      bz += q.gb[2] / std::sqrt(1 + norm2(q.gb));
    }
    unsigned Nq = (unsigned)particle_count();
    bz /= Nq;
    mesh.totalTime = 1 / (c0 * (bz + beta)) * (zEnd - beta * c0 * dt_shift - zMin + bz / beta * Lu);
  }

  // Solver::initializeField, src/solver.cpp:695-842.
  const double dx = mesh.meshResolution[0], dy = mesh.meshResolution[1], dz = mesh.meshResolution[2];
  const double dt = mesh.timeStep;
  uc_dv = -m0 * EC / mesh.timeStep / (dx * dy * dz);
  uc_rc = -EC / e0 / (dx * dy * dz);
  {
    double bet = (1.0 + 0.02 / ((dz / dx) * (dz / dx) + (dz / dy) * (dz / dy))) / 4.0;
    double alp = 1.0 - 2.0 * bet;
    nsfd_alpha = alp;
    nsfd_beta = bet / alp;
    const double rx = (c0 * dt / dx) * (c0 * dt / dx), ry = (c0 * dt / dy) * (c0 * dt / dy),
                 rz = (c0 * dt / dz) * (c0 * dt / dz);
    a[0] = 2.0 * (1.0 - alp * rx - alp * ry - rz);
    a[1] = rx;
    a[2] = ry;
    a[3] = rz - 2.0 * (bet * rx + bet * ry);
    a[4] = (c0 * dt) * (c0 * dt) * uc_dv;
    a[5] = (c0 * dt) * (c0 * dt) * uc_rc;
  }
  const double to = (double)mesh.truncationOrder;
  {
    double alpha1 = 0.0, alpha2 = 0.0;
    double p = (1.0 + std::cos(alpha1) * std::cos(alpha2)) / (std::cos(alpha1) + std::cos(alpha2));
    double q = -1.0 / (std::cos(alpha1) + std::cos(alpha2));
    double d = 1.0 / (2.0 * dt * dx) + p / (2.0 * c0 * dt * dt);
    bB[0] = (1.0 / (2.0 * dt * dx) - p / (2.0 * c0 * dt * dt)) / d;
    bB[1] = (-1.0 / (2.0 * dt * dx) - p / (2.0 * c0 * dt * dt)) / d;
    bB[2] = (p / (c0 * dt * dt) + q * (to - 1.0) * (c0 / (dy * dy) + c0 / (dz * dz))) / d;
    bB[3] = -q * (to - 1.0) * (c0 / (2.0 * dy * dy)) / d;
    bB[4] = -q * (to - 1.0) * (c0 / (2.0 * dz * dz)) / d;
    d = 1.0 / (2.0 * dt * dy) + p / (2.0 * c0 * dt * dt);
    cB[0] = (1.0 / (2.0 * dt * dy) - p / (2.0 * c0 * dt * dt)) / d;
    cB[1] = (-1.0 / (2.0 * dt * dy) - p / (2.0 * c0 * dt * dt)) / d;
    cB[2] = (p / (c0 * dt * dt) + q * (to - 1.0) * (c0 / (dx * dx) + c0 / (dz * dz))) / d;
    cB[3] = -q * (to - 1.0) * (c0 / (2.0 * dx * dx)) / d;
    cB[4] = -q * (to - 1.0) * (c0 / (2.0 * dz * dz)) / d;
    d = 1.0 / (2.0 * dt * dz) + p / (2.0 * c0 * dt * dt);
    dB[0] = (1.0 / (2.0 * dt * dz) - p / (2.0 * c0 * dt * dt)) / d;
    dB[1] = (-1.0 / (2.0 * dt * dz) - p / (2.0 * c0 * dt * dt)) / d;
    dB[2] = (p / (c0 * dt * dt) + q * (to - 1.0) * (c0 / (dx * dx) + c0 / (dy * dy))) / d;
    dB[3] = -q * (to - 1.0) * (c0 / (2.0 * dx * dx)) / d;
    dB[4] = -q * (to - 1.0) * (c0 / (2.0 * dy * dy)) / d;
    auto edge = [&](double* E, double ha, double hb, double ht) {  // ha, hb normal; ht along the edge
      double de = (1.0 / hb + 1.0 / ha) / (4.0 * dt) + 3.0 / (8.0 * c0 * dt * dt);
      E[0] = (-(1.0 / hb - 1.0 / ha) / (4.0 * dt) - 3.0 / (8.0 * c0 * dt * dt)) / de;
      E[1] = ((1.0 / hb - 1.0 / ha) / (4.0 * dt) - 3.0 / (8.0 * c0 * dt * dt)) / de;
      E[2] = ((1.0 / hb + 1.0 / ha) / (4.0 * dt) - 3.0 / (8.0 * c0 * dt * dt)) / de;
      E[3] = (3.0 / (4.0 * c0 * dt * dt) - c0 / (4.0 * ht * ht)) / de;
      E[4] = c0 / (8.0 * ht * ht) / de;
    };
    edge(eE, dx, dy, dz);  // src/solver.cpp:784-790: 1/dy + 1/dx, along z
    edge(fE, dy, dz, dx);  // :792-798: 1/dz + 1/dy, along x
    edge(gE, dz, dx, dy);  // :800-806: 1/dx + 1/dz, along y
    const double c4 = 1.0 / (4.0 * c0 * dt * dt);
    const double sx[8] = {-1, 1, -1, -1, 1, 1, -1, 1}, sy[8] = {-1, -1, 1, -1, 1, -1, 1, 1},
                 sz[8] = {-1, -1, -1, 1, -1, 1, 1, 1};
    for (int i = 0; i < 8; i++) {  // src/solver.cpp:808-824
      double s = sx[i] > 0 ? 1.0 / dx : -1.0 / dx;
      s = sy[i] > 0 ? s + 1.0 / dy : s - 1.0 / dy;
      s = sz[i] > 0 ? s + 1.0 / dz : s - 1.0 / dz;
      hC[i] = s / (8.0 * dt) - c4;
      hC[8 + i] = -(s) / (8.0 * dt) - c4;
    }
    hC[16] = 1.0 / (2.0 * c0 * dt * dt);
  }
  if (seed.amplitude > 1.0e-50) {  // src/solver.cpp:828-839
    const size_t n = (size_t)N1N0 * np * 3;
    an.assign(n, 0.0);
    anm1.assign(n, 0.0);
    for (int i = 2; i < N0 - 2; i++)
      for (int j = 2; j < N1 - 2; j++)
        for (int k = 2; k < np - 2; k++) {
          long m = (long)N1N0 * k + (long)N1 * i + j;
          Vec3 r{xmin + i * mesh.meshResolution[0], ymin + j * mesh.meshResolution[1],
                 zmin + (unsigned)(k + k0) * mesh.meshResolution[2]};
          Vec3 a1{an[3 * m], an[3 * m + 1], an[3 * m + 2]};
          seed.fields(r, time, a1);
          Vec3 a2{anm1[3 * m], anm1[3 * m + 1], anm1[3 * m + 2]};
          seed.fields(r, timem1, a2);
          for (int c = 0; c < 3; c++) { an[3 * m + c] = a1[c]; anm1[3 * m + c] = a2[c]; }
        }
  }

  // Solver::initializeBunchUpdate, src/solver.cpp:1050-1059.
  ub_dtb = c0 * bunch.timeStep;
  ub_r1 = -EC / (EM * c0) * bunch.timeStep / 2.0;
  ub_r2 = -EC / EM * bunch.timeStep / 2.0;

  // Solver::initializeSeedSampling, src/solver.cpp:848-932: bunch-frame rhythm and positions, the
  // points of a line, and only points inside the mesh kept.  The range check reads ub_.dx ...
  // before initializeBunchUpdate sets them; the mesh resolution is used here.
  if (seed.sampling) {
    FieldSampling& f = seed.samp;
    if (f.rhythm == 0) die("The sampling rhythm of the field is zero although sampling is activated !!!");
    f.rhythm /= gamma;
    for (auto& p : f.position) p[2] *= gamma;
    f.lineBegin[2] *= gamma;
    f.lineEnd[2] *= gamma;
    if (f.type == OVERLINE) {
      Vec3 l = f.lineEnd;
      for (int d = 0; d < 3; d++) l[d] -= f.lineBegin[d];
      const double n = f.res;
      for (int d = 0; d < 3; d++) l[d] /= n;
      for (unsigned i = 0; i < (unsigned)f.res; i++) {
        Vec3 p;
        for (int d = 0; d < 3; d++) p[d] = f.lineBegin[d] + i * l[d];
        f.position.push_back(p);
      }
    }
    std::vector<Vec3> kept;
    const double* res = mesh.meshResolution.data();
    for (const auto& p : f.position)
      if (p[0] < xmax - res[0] && p[0] > xmin + res[0] && p[1] < ymax - res[1] && p[1] > ymin + res[1] &&
          p[2] < zmax - res[2] && p[2] > zmin + res[2] && p[2] < zp[1] && p[2] >= zp[0])
        kept.push_back(p);
    f.position = kept;
  }

  // Solver::initializeSeedVTK, src/solver.cpp:938-1016: the rhythm and the plane position go to
  // the bunch frame, the directory is prefixed to a relative base name, and an in-plane output
  // whose plane lies outside the mesh is dropped.  The reference drops it from the vector it is
  // iterating over and then advances the index, so the output after a dropped one is skipped
  // (left unboosted); that is reproduced.  Its range check reads ub_.dx, ub_.dy, ub_.dz before
  // initializeBunchUpdate sets them; the mesh resolution is used here.
  for (size_t i = 0; i < job.seed.vtk.size(); i++) {
    FieldVtk& v = job.seed.vtk[i];
    if (!v.sample) continue;
    if (v.rhythm == 0) die("The visualization rhythm of the field is zero although visualization is activated !!!");
    v.rhythm /= gamma;
    v.position[2] *= gamma;
    if (v.basename.empty() || v.basename[0] != '/') v.basename = v.directory + v.basename;
    if (v.type != VTK_INPLANE) continue;
    bool outside = false;
    if (v.plane == VTK_XNORMAL)
      outside = v.position[0] > xmax - mesh.meshResolution[0] || v.position[0] < xmin + mesh.meshResolution[0];
    else if (v.plane == VTK_YNORMAL)
      outside = v.position[1] > ymax - mesh.meshResolution[1] || v.position[1] < ymin + mesh.meshResolution[1];
    else
      outside = v.position[2] > zmax - mesh.meshResolution[2] || v.position[2] < zmin + mesh.meshResolution[2];
    if (outside) job.seed.vtk.erase(job.seed.vtk.begin() + (long)i);
  }

  // Solver::initializePowerSample, src/radiation.cpp:18-121.
  for (size_t jf = 0; jf < job.fel.size(); jf++) {
    RadiationPower& rp = job.fel[jf].radiationPower;
    if (!rp.sampling) continue;
    if (und.empty()) die("radiation-power sampling needs an undulator");
    for (auto& z : rp.z) z *= gamma;
    rp.lineBegin *= gamma;
    rp.lineEnd *= gamma;
    double dl = std::fabs(rp.lineEnd - rp.lineBegin) / rp.res;
    if (rp.samplingType == OVERLINE) {
      double l = 0.0;
      while (std::fabs(l) < std::fabs(rp.lineEnd - rp.lineBegin)) {
        rp.z.push_back(rp.lineBegin + l);
        l += dl;
      }
    }
    PowerCfg pc;
    pc.N = (int)rp.z.size();
    pc.z = rp.z;
    dl = (rp.lambdaMax - rp.lambdaMin) / rp.lambdaRes;
    for (double rw = rp.lambdaMin; rw < rp.lambdaMax; rw += dl) rp.lambda.push_back(rw);
    pc.Nl = (int)rp.lambda.size();
    pc.lambda = rp.lambda;
    unsigned Nf = 0;
    pc.w.resize(pc.Nl);
    for (int i = 0; i < pc.Nl; i++) {
      double dtr = und[0].lu / rp.lambda[i] / (gamma * c0);
      Nf = (unsigned(3.0 * dtr / mesh.timeStep) > Nf) ? unsigned(3.0 * dtr / mesh.timeStep) : Nf;
      pc.w[i] = 2 * PI / dtr;
    }
    pc.Nf = (int)Nf;
    pc.pc = 2.0 * dx * dy / (m0 * Nf * Nf) * std::pow(mesh.lengthScale, 2) / std::pow(mesh.timeScale, 3);
    pc.tw_re.resize((size_t)pc.Nl * Nf);
    pc.tw_im.resize((size_t)pc.Nl * Nf);
    for (int i = 0; i < pc.Nl; i++)
      for (unsigned j = 0; j < Nf; j++) {
        pc.tw_re[(size_t)i * Nf + j] = std::cos(pc.w[i] * j * mesh.timeStep);
        pc.tw_im[(size_t)i * Nf + j] = std::sin(pc.w[i] * j * mesh.timeStep);
      }
    if (pc.Nf == 0) die("radiation-power sampling with no frequency");
    power.push_back(pc);
    power_fel_index.push_back((int)jf);
  }

  // Lab-frame screens, Solver::initializeScreenProfile (src/solver.cpp:2145-2199): the given
  // positions plus, with a rhythm, 0, rhythm, 2 rhythm, ... up to the undulator end, sorted.  The
  // reference bounds the rhythm by undulator_.end(), one past the last module (undefined); the
  // last module is used here.
  for (size_t jf = 0; jf < job.fel.size(); jf++) {
    const ScreenProfile& sp = job.fel[jf].screenProfile;
    if (!sp.sampling) continue;
    std::vector<double> pos = sp.pos;
    if (sp.rhythm > 0.0 && !job.undulators.empty()) {
      const Undulator& U = job.undulators.back();
      for (double z = 0.0; z < U.rb + U.length * U.lu; z += sp.rhythm) pos.push_back(z);
    }
    std::sort(pos.begin(), pos.end());
    if (pos.empty()) die("No position is set for the screen although the screen sampling is activated !!!");
    for (double z : pos) {
      screen_z.push_back(z);
      screen_fel.push_back((int)jf);
    }
  }

  // Solver::shiftBackInTime, src/solver.cpp:1184-1206.
  if (mesh.timeShift != 0.0) {
    timem1 -= mesh.timeShift;
    time -= mesh.timeShift;
    timep1 -= mesh.timeShift;
    timeBunch -= mesh.timeShift;
    if (device_init) dev_check(devinit::time_shift(dstore, c0, mesh.timeShift, dev_err, sizeof dev_err));
    for (auto& q : charges) {
      double t = c0 * mesh.timeShift / std::sqrt(1.0 + norm2(q.gb));
      for (int d = 0; d < 3; d++) q.rnp[d] -= t * q.gb[d];
    }
    distribute();
  }
}

void Setup::fill_grid(mithra_grid_desc* g) const {
  const Mesh& mesh = job.mesh;
  *g = mithra_grid_desc{};
  g->N0 = N0; g->N1 = N1; g->N2 = N2;
  g->solver = mesh.solver == NSFD ? 1 : 0;
  g->truncation_order = mesh.truncationOrder;
  g->space_charge = mesh.spaceCharge ? 1 : 0;
  for (int i = 0; i < 6; i++) g->a[i] = a[i];
  g->nsfd_alpha = nsfd_alpha; g->nsfd_beta = nsfd_beta;
  for (int i = 0; i < 5; i++) {
    g->bB[i] = bB[i]; g->cB[i] = cB[i]; g->dB[i] = dB[i];
    g->eE[i] = eE[i]; g->fE[i] = fE[i]; g->gE[i] = gE[i];
  }
  for (int i = 0; i < 17; i++) g->hC[i] = hC[i];
  g->dt = mesh.timeStep;
  g->dx = mesh.meshResolution[0]; g->dy = mesh.meshResolution[1]; g->dz = mesh.meshResolution[2];
  g->xmin = xmin; g->xmax = xmax; g->ymin = ymin; g->ymax = ymax; g->zmin = zmin; g->zmax = zmax;
  g->zp0 = zp[0]; g->zp1 = zp[1];
  g->Lz = mesh.meshLength[2];
}

void Setup::fill_push(mithra_push_desc* p) const {
  *p = mithra_push_desc{};
  p->dtb = ub_dtb;
  p->bunch_time_step = job.bunch.timeStep;
  p->r1 = ub_r1; p->r2 = ub_r2;
  p->gamma = gamma; p->beta = beta; p->c0 = c0;
  p->dt_shift = dt_shift;
  p->n_update_bunch = nUpdateBunch;
}

namespace {
// Laser-beam parameters under the keys the reference harness writes for them.
template <class KV>
void beam_meta(KV& kv, const std::string& p, const Beam& b) {
  kv(p + "type", (double)b.seedType);
  for (int c = 0; c < 3; c++) {
    kv(p + "pos" + std::to_string(c), b.position[c]);
    kv(p + "dir" + std::to_string(c), b.direction[c]);
    kv(p + "pol" + std::to_string(c), b.polarization[c]);
  }
  kv(p + "amp", b.amplitude);
  kv(p + "r0", b.radius.size() > 0 ? b.radius[0] : 0.0);
  kv(p + "r1", b.radius.size() > 1 ? b.radius[1] : 0.0);
  kv(p + "o0", b.order.size() > 0 ? b.order[0] : 0);
  kv(p + "o1", b.order.size() > 1 ? b.order[1] : 0);
  kv(p + "l", b.l);
  kv(p + "zR0", b.zR.size() > 0 ? b.zR[0] : 0.0);
  kv(p + "zR1", b.zR.size() > 1 ? b.zR[1] : 0.0);
  kv(p + "sig_type", (double)b.signal.type);
  kv(p + "sig_t0", b.signal.t0); kv(p + "sig_s", b.signal.s); kv(p + "sig_f0", b.signal.f0);
  kv(p + "sig_cep", b.signal.cep); kv(p + "sig_nR", (double)b.signal.nR);
  kv(p + "sig_g0", b.signal.sigmaInvG.size() > 0 ? b.signal.sigmaInvG[0] : 0.0);
  kv(p + "sig_g1", b.signal.sigmaInvG.size() > 1 ? b.signal.sigmaInvG[1] : 0.0);
}
}  // namespace

std::string Setup::meta() const {
  std::ostringstream o;
  char buf[96];
  auto kv = [&](const std::string& k, double v) {
    snprintf(buf, sizeof buf, "%.17g", v);
    o << k << " " << buf << "\n";
  };
  const Mesh& mesh = job.mesh;
  kv("N0", N0); kv("N1", N1); kv("N2", N2); kv("np", np); kv("k0", k0);
  kv("xmin", xmin); kv("xmax", xmax); kv("ymin", ymin); kv("ymax", ymax); kv("zmin", zmin); kv("zmax", zmax);
  kv("zp0", zp[0]); kv("zp1", zp[1]);
  kv("dx", mesh.meshResolution[0]); kv("dy", mesh.meshResolution[1]); kv("dz", mesh.meshResolution[2]);
  kv("Lx", mesh.meshLength[0]); kv("Ly", mesh.meshLength[1]); kv("Lz", mesh.meshLength[2]);
  kv("dt", mesh.timeStep); kv("dtb", job.bunch.timeStep); kv("nUpdateBunch", nUpdateBunch);
  kv("totalTime", mesh.totalTime); kv("time", time); kv("timeBunch", timeBunch);
  kv("nTime", (double)nTime); kv("nTimeBunch", (double)nTimeBunch);
  kv("gamma", gamma); kv("beta", beta); kv("dt_shift", dt_shift); kv("c0", c0); kv("m0", m0); kv("e0", e0);
  for (int i = 0; i < 6; i++) kv("a" + std::to_string(i), a[i]);
  kv("nsfd_alpha", nsfd_alpha); kv("nsfd_beta", nsfd_beta);
  const double* bs[6] = {bB, cB, dB, eE, fE, gE};
  const char* bn[6] = {"bB", "cB", "dB", "eE", "fE", "gE"};
  for (int b = 0; b < 6; b++)
    for (int i = 0; i < 5; i++) kv(std::string(bn[b]) + std::to_string(i), bs[b][i]);
  for (int i = 0; i < 17; i++) kv("hC" + std::to_string(i), hC[i]);
  kv("uc_dv", uc_dv); kv("uc_rc", uc_rc); kv("ub_dtb", ub_dtb); kv("ub_r1", ub_r1); kv("ub_r2", ub_r2);
  kv("n_undulator", (double)job.undulators.size());
  for (size_t u = 0; u < job.undulators.size(); u++) {
    const Undulator& U = job.undulators[u];
    const std::string p = "und" + std::to_string(u) + "_";
    kv(p + "k", U.k); kv(p + "lu", U.lu); kv(p + "rb", U.rb); kv(p + "length", U.length);
    kv(p + "dist", U.dist); kv(p + "theta", U.theta); kv(p + "type", (double)U.type);
    if (U.type == OPTICAL) beam_meta(kv, p + "beam_", U);
  }
  beam_meta(kv, "seed_", job.seed);
  kv("seed_gamma", job.seed.gamma); kv("seed_beta", job.seed.beta);
  kv("seed_c0", job.seed.c0); kv("seed_dt", job.seed.dt);
  kv("n_ext", (double)job.extFields.size());
  for (size_t x = 0; x < job.extFields.size(); x++) beam_meta(kv, "ext" + std::to_string(x) + "_", job.extFields[x]);
  kv("n_particles", (double)particle_count());
  kv("n_fel", (double)job.fel.size());
  for (size_t o2 = 0; o2 < power.size(); o2++) {
    const PowerCfg& pc = power[o2];
    const std::string p = "rp" + std::to_string(power_fel_index[o2]) + "_";
    kv(p + "N", pc.N); kv(p + "Nl", pc.Nl); kv(p + "Nf", pc.Nf); kv(p + "pc", pc.pc);
    for (int i = 0; i < pc.Nl; i++) kv(p + "w" + std::to_string(i), pc.w[i]);
    for (int i = 0; i < pc.N; i++) kv(p + "z" + std::to_string(i), pc.z[i]);
  }
  kv("time_shift", mesh.timeShift);
  {
    const FieldSampling& f = job.seed.samp;
    kv("fs_sampling", job.seed.sampling ? 1.0 : 0.0);
    kv("fs_rhythm", f.rhythm);
    kv("fs_n", job.seed.sampling ? (double)f.position.size() : 0.0);
    for (size_t i = 0; job.seed.sampling && i < f.position.size(); i++)
      for (int d = 0; d < 3; d++) kv("fs_p" + std::to_string(i) + "_" + std::to_string(d), f.position[i][d]);
    kv("fs_nfield", (double)f.field.size());
    for (size_t l = 0; l < f.field.size(); l++) kv("fs_f" + std::to_string(l), (double)f.field[l]);
    // unit factors of the file (src/solver.cpp:925-927)
    kv("fs_Ce", mesh.lengthScale / std::pow(mesh.timeScale, 2));
    kv("fs_Cb", 1.0 / (mesh.lengthScale * mesh.timeScale));
    kv("fs_Ca", 1.0 / mesh.timeScale);
  }
  kv("bunch_profile", job.bunch.profile ? 1.0 : 0.0);
  kv("bunch_profile_rhythm", job.bunch.profileRhythm);
  kv("bunch_profile_ntime", (double)job.bunch.profileTime.size());
  for (size_t i = 0; i < job.bunch.profileTime.size(); i++) kv("bunch_profile_t" + std::to_string(i), job.bunch.profileTime[i]);
  kv("bunch_sampling", job.bunch.sampling ? 1.0 : 0.0);
  kv("bunch_rhythm", job.bunch.rhythm);
  kv("n_vtk", (double)job.seed.vtk.size());
  for (size_t i = 0; i < job.seed.vtk.size(); i++) {
    const FieldVtk& v = job.seed.vtk[i];
    const std::string p = "vtk" + std::to_string(i) + "_";
    kv(p + "sample", v.sample ? 1.0 : 0.0);
    kv(p + "type", (double)v.type);
    kv(p + "plane", (double)v.plane);
    kv(p + "rhythm", v.rhythm);
    for (int d = 0; d < 3; d++) kv(p + "pos" + std::to_string(d), v.position[d]);
    kv(p + "nfield", (double)v.field.size());
    for (size_t l = 0; l < v.field.size(); l++) kv(p + "f" + std::to_string(l), (double)v.field[l]);
  }
  for (size_t i = 0; i < screen_z.size(); i++) {
    const std::string p = "scr" + std::to_string(i) + "_";
    kv(p + "z", screen_z[i]);
    kv(p + "fel", (double)screen_fel[i]);
  }
  kv("n_screens", (double)screen_z.size());
  return o.str();
}

}  // namespace host
}  // namespace mithra
