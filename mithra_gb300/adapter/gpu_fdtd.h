/*
 * gpu_fdtd.h : the reference-side adapter that runs MITHRA's time-marching loop on the GPU.
 *
 * A maintainer of MITHRA adds this header and gpu_fdtd.cpp to the reference's build (they include
 * the reference's own src/fdtd.h, src/fdtdSC.h and this repository's include/mithra_gpu.h, and
 * link against libmithra_gb300.so).  The solver choice in main (src/mithra.cpp:86-93) becomes
 *
 *     if (mesh.spaceCharge_) { GpuFdTdSC s(mesh, bunch, seed, undulator, extField, FEL); s.solve(); }
 *     else                   { GpuFdTd   s(mesh, bunch, seed, undulator, extField, FEL); s.solve(); }
 *
 * GpuSolver<Base>::solve() keeps the reference's parsing and initialisation (Solver::initialize,
 * src/solver.cpp:547-595), hands the initialised state to the device through the C ABI, marches
 * the prelude and the main loop there (src/solver.cpp:1232-1414), writes the power rows into the
 * reference's own power-sampling streams (the text of src/radiation.cpp:222-229), and writes the
 * final fields, particles and time state back into the solver's members.  Solver::solve is not
 * virtual (src/solver.h:75), so solve() is called on the GpuSolver object itself.
 *
 * describe_for_gpu() is the translation from the reference's members to the library's
 * descriptors; it is usable on its own (the tests compare it with the library's own host set-up).
 */
#ifndef MITHRA_GPU_FDTD_H
#define MITHRA_GPU_FDTD_H

#include <string>
#include <vector>

#include "fdtd.h"
#include "fdtdSC.h"
#include "mithra_gpu.h"

namespace MITHRA {

/* Everything the library needs from an initialised Solver.  The power descriptors point into
 * the vectors of this object. */
struct GpuDescriptors {
  mithra_grid_desc grid;
  mithra_push_desc push;
  mithra_seed_desc seed;
  mithra_time_state time;
  std::vector<mithra_undulator_desc> undulators;
  std::vector<mithra_beam_desc> ext_fields;
  std::vector<mithra_power_desc> power;        /* the FEL outputs that sample power, in order */
  std::vector<unsigned> power_fel;             /* index into FEL_ of each power output */
  std::vector<std::vector<double> > power_z, power_re, power_im;
  double total_time;
  size_t n_particles;
};

/* Fills `d` from a Solver after initialize() (and before any step). */
void describe_for_gpu(Solver& s, GpuDescriptors& d);

/* Runs the whole of Solver::solve on the device; returns the library's status (0 on success) and
 * writes the reference-style message for a failure. */
int solve_on_gpu(Solver& s, int precision, int device, std::string& error);

template <class Base>
class GpuSolver : public Base {
 public:
  GpuSolver(Mesh& mesh, Bunch& bunch, Seed& seed, std::vector<Undulator>& undulator,
            std::vector<ExtField>& extField, std::vector<FreeElectronLaser>& FEL,
            int precision = MITHRA_PRECISION_FP64, int device = 0)
      : Base(mesh, bunch, seed, undulator, extField, FEL), precision_(precision), device_(device) {}

  /* Solver::solve on the GPU: a failure is reported like the reference's own errors
   * (printmessage, then exit(1)). */
  void solve();

 private:
  int precision_, device_;
};

typedef GpuSolver<FdTd> GpuFdTd;
typedef GpuSolver<FdTdSC> GpuFdTdSC;

}  // namespace MITHRA

#endif
