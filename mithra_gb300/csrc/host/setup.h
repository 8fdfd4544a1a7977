// Host-side FP64 initialisation of a MITHRA run, restating Solver::initialize
// (src/solver.cpp:547-595) and the bunch generators of src/classes.cpp:84-417.  Produces the
// descriptors of include/mithra_gpu.h, the initial potentials and the particle records.
#pragma once
#include <string>
#include <vector>

#include "mithra_gpu.h"
#include "devinit.h"
#include "params.h"

namespace mithra {
namespace host {

struct Charge {  // src/stdinclude.h:130-144
  double q = 0.0;
  Vec3 rnp{0, 0, 0}, rnm{0, 0, 0}, gb{0, 0, 0};
  double e = 0.0;
};

struct PowerCfg {
  int N = 0, Nl = 0, Nf = 0;
  double pc = 0.0;
  std::vector<double> z, w, tw_re, tw_im;
  std::vector<double> lambda;
};

struct Setup {
  Job job;
  double c0 = 0, m0 = 0, e0 = 0, gamma = 0, beta = 0, dt_shift = 0;
  int N0 = 0, N1 = 0, N2 = 0, np = 0, k0 = 0, N1N0 = 0;
  double xmin = 0, xmax = 0, ymin = 0, ymax = 0, zmin = 0, zmax = 0, zp[2] = {0, 0};
  double time = 0, timep1 = 0, timem1 = 0, timeBunch = 0;
  long long nTime = 0, nTimeBunch = 0;
  double nUpdateBunch = 0;
  std::vector<Charge> charges;
  // Particles generated and transformed on the device (Setup::device_init); `charges` stays empty.
  bool device_init = false;
  devinit::Store dstore;
  size_t particle_count() const { return device_init ? dstore.n : charges.size(); }
  char dev_err[256] = {0};
  void dev_check(int r);
  void init_bunch_on_device();
  // Field-update coefficients (uf_), current and bunch-update constants (uc_, ub_).
  double a[6] = {0}, nsfd_alpha = 0, nsfd_beta = 0;
  double bB[5] = {0}, cB[5] = {0}, dB[5] = {0}, eE[5] = {0}, fE[5] = {0}, gE[5] = {0}, hC[17] = {0};
  double uc_dv = 0, uc_rc = 0, ub_dtb = 0, ub_r1 = 0, ub_r2 = 0;
  std::vector<double> an, anm1;  // initial potentials (seed fill), reference AoS layout; empty = zero
  std::vector<PowerCfg> power;   // one per FEL entry with radiation-power sampling
  std::vector<double> screen_z;  // lab z of the screens (FEL entries in order, positions sorted)
  std::vector<int> screen_fel;   // FEL entry of each screen
  std::vector<int> power_fel_index;

  void initialize();
  std::string meta() const;
  void fill_grid(mithra_grid_desc* g) const;
  void fill_push(mithra_push_desc* p) const;
};

double halton(unsigned dim, unsigned index);
double pmod(double a, double b);

}  // namespace host
}  // namespace mithra
