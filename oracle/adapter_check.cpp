/*
 * Test driver of the reference-side adapter (mithra_gb300/adapter/gpu_fdtd.cpp).
 * TEST INFRASTRUCTURE ONLY: linked with the UNMODIFIED reference objects built by
 * oracle/Makefile.ref, it parses a job exactly as the reference's main does
 * (src/mithra.cpp:48-93), runs Solver::initialize through the adapter's solver class, and writes
 * the descriptors describe_for_gpu() builds from the initialised members, so that a test can
 * compare them with the library's own host set-up.  It stops before mithra_gpu_create.
 *
 *   adapter_check JOB OUT     writes OUT/grid.bin, push.bin, seed.bin, time.bin (raw structs),
 *                             undulators.bin, ext.bin (arrays of structs), power<o>.bin
 *                             (N Nl Nf as int32, pc, then z[N], re[Nl*Nf], im[Nl*Nf] as doubles)
 *                             and scalars.txt (total time, particle count)
 */
#include <cstdio>
#include <cstdlib>
#include <list>
#include <string>
#include <vector>

#include "classes.h"
#include "datainput.h"
#include "gpu_fdtd.h"
#include "readdata.h"

using namespace MITHRA;

static void write_raw(const std::string& path, const void* p, size_t bytes) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) { perror(path.c_str()); exit(2); }
  if (bytes && fwrite(p, 1, bytes, f) != bytes) { perror("fwrite"); exit(2); }
  fclose(f);
}

int main(int argc, char** argv) {
  if (argc != 3) { fprintf(stderr, "usage: %s JOB OUT\n", argv[0]); return 2; }
  int dummy_argc = 1;
  MPI_Init(&dummy_argc, &argv);
  std::list<std::string> jobFile = read_file(argv[1]);
  cleanJobFile(jobFile);
  Mesh mesh; mesh.initialize();
  Bunch bunch; Seed seed;
  std::vector<Undulator> undulator; std::vector<ExtField> extField; std::vector<FreeElectronLaser> FEL;
  ParseDarius parser(jobFile, mesh, bunch, seed, undulator, extField, FEL);
  parser.setJobParameters();

  Solver* s;
  if (mesh.spaceCharge_) s = new GpuFdTdSC(mesh, bunch, seed, undulator, extField, FEL);
  else s = new GpuFdTd(mesh, bunch, seed, undulator, extField, FEL);
  s->initialize();
  GpuDescriptors d;
  describe_for_gpu(*s, d);

  const std::string out = argv[2];
  write_raw(out + "/grid.bin", &d.grid, sizeof d.grid);
  write_raw(out + "/push.bin", &d.push, sizeof d.push);
  write_raw(out + "/seed.bin", &d.seed, sizeof d.seed);
  write_raw(out + "/time.bin", &d.time, sizeof d.time);
  write_raw(out + "/undulators.bin", d.undulators.data(), d.undulators.size() * sizeof(mithra_undulator_desc));
  write_raw(out + "/ext.bin", d.ext_fields.data(), d.ext_fields.size() * sizeof(mithra_beam_desc));
  for (size_t o = 0; o < d.power.size(); o++) {
    const mithra_power_desc& p = d.power[o];
    std::vector<char> b;
    const int32_t hdr[3] = {p.N, p.Nl, p.Nf};
    b.insert(b.end(), (const char*)hdr, (const char*)hdr + sizeof hdr);
    b.insert(b.end(), (const char*)&p.pc, (const char*)&p.pc + sizeof p.pc);
    b.insert(b.end(), (const char*)p.z, (const char*)(p.z + p.N));
    b.insert(b.end(), (const char*)p.twiddle_re, (const char*)(p.twiddle_re + (size_t)p.Nl * p.Nf));
    b.insert(b.end(), (const char*)p.twiddle_im, (const char*)(p.twiddle_im + (size_t)p.Nl * p.Nf));
    write_raw(out + "/power" + std::to_string(o) + ".bin", b.data(), b.size());
  }
  FILE* f = fopen((out + "/scalars.txt").c_str(), "w");
  fprintf(f, "%.17g %zu %zu\n", d.total_time, d.n_particles, d.power.size());
  fclose(f);
  MPI_Finalize();
  return 0;
}
