// Device-side bunch initialisation: the particle phase of Solver::initialize for ellipsoid bunches
// (Bunch::initializeEllipsoid, src/classes.cpp:104-298; Solver::lorentzBoostBunch,
// src/solver.cpp:263-423; distributeParticles, :429-487; shiftBackInTime, :1184-1206) run on the
// GPU instead of the host.  The host keeps every scalar decision (gamma, dt_, the shifts); the
// particles live in a device buffer of 11-double records (the layout of the reference's Charge)
// that the context converts into its own particle arrays without a host round trip.
//
// Implemented in init_kernels.cu, compiled without FMA contraction, so every record agrees with
// the host initialisation except where the device's log/sin/cos round differently from the host
// C library (a unit in the last place).
#pragma once
#include <cstddef>

namespace mithra {
namespace devinit {

struct Store {
  int device = 0;
  double* rec = nullptr;  // 11 doubles per particle: q, rnp[3], rnm[3], gb[3], e
  size_t n = 0, cap = 0;
};

// One call of Bunch::initializeEllipsoid for one position.
struct Ellipsoid {
  unsigned Np;        // numberOfParticles (a multiple of 4)
  unsigned Np0;       // particles the bunch group holds before this position (Halton offset)
  unsigned ng;        // beamlet size: 4, or 1 without an FEL wavelength
  unsigned n_main;    // Np / ng candidates
  unsigned n_taper;   // candidates incl. the Gaussian taper of a uniform bunch
  int gaussian;       // longitudinal distribution: 0 uniform, 1 gaussian
  int shot_noise;
  double q;           // cloudCharge / Np
  double gb[3];       // initialGamma * betaVector
  double sig_r[3], sig_gb[3];
  double tran_trun, long_trun;
  double pos[3];
  double lambda, bF_user, bFP;
};

int reserve(Store& s, size_t cap, char* err, size_t err_len);
void release(Store& s);
// Shot-noise reference position: the minimum candidate z before truncation (relative to pos).
int candidate_zmin(int device, const Ellipsoid& e, double* zmin, char* err, size_t err_len);
// Appends the particles of one position; zmin (absolute) and bF as the reference computes them.
int generate(Store& s, const Ellipsoid& e, double zmin, double bF, char* err, size_t err_len);
// z -> gamma z, gb_z -> gamma (gamma_q) (beta_z - beta); returns the largest boosted z.
int boost(Store& s, double gamma, double beta, double* zmax, char* err, size_t err_len);
int back_propagate(Store& s, double zu, double beta, char* err, size_t err_len);
// sum of z and of beta_z over all particles (compensated)
int sums_z_bz(Store& s, double* z, double* bz, char* err, size_t err_len);
int shift_z(Store& s, double shift, char* err, size_t err_len);
// keeps the particles whose wrapped z is in [zp0, zp1), in order
int distribute(Store& s, double zmin, double Lz, double zp0, double zp1, char* err, size_t err_len);
int min_z(Store& s, double* zmin, char* err, size_t err_len);
int time_shift(Store& s, double c0, double shift, char* err, size_t err_len);
// the first n records to host memory
int download(const Store& s, double* rec, size_t n, char* err, size_t err_len);

}  // namespace devinit
}  // namespace mithra
