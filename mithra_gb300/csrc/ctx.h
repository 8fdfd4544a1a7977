// Internal definition of the library context shared by the translation units of the CUDA part.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <utility>
#include <vector>

#include "../../include/mithra_gpu.h"
#include "device_common.cuh"

namespace mithra {

struct PowerOut {
  PowerDev dev{};
  double *z = nullptr, *dzr = nullptr, *tw_re = nullptr, *tw_im = nullptr, *fdt = nullptr,
         *partial = nullptr, *rows = nullptr, *run = nullptr;
  int *plane_k = nullptr, *plane_slot = nullptr;
};

struct KernelTimer {
  std::string name;
  double ms = 0.0;
  long long launches = 0;
};

// Device buffers of the mixed-precision form (allocated only when it is selected).
struct TileGridHost {
  int ntx = 0, nty = 0, ntz = 0, n_tiles = 0, bin_outside = 0, bin_erased = 0, n_bins = 0;
};

struct Fp32State {
  float* A[3] = {nullptr, nullptr, nullptr};
  float* F[3] = {nullptr, nullptr, nullptr};
  ParticlesF32 pt{};
  ParticlesF32 alt{};  // second buffer set: the tile sort scatters into it, then the two swap
  int parity = 0;      // which of the two sets is current (flips at every sort)
  // Particles uploaded since the last sort: the next step sorts whatever its rotation (run
  // directly, outside the step graphs), so that a resumed march does not push and deposit
  // unsorted particles until the next step of the sort's rotation.
  bool sort_pending = false;
  int* counts = nullptr;
  int* offsets = nullptr;
  int* key = nullptr;
  int* rank = nullptr;
  int* block_sums = nullptr;  // 1024 block totals of the bin scan + grand total
  int* work = nullptr;        // occupied tiles of the last sort (the deposit's work list)
  int* work_count = nullptr;  // [heavy, light] entries of the list, then the deposit's next entry
  TileGridHost tiles;
  // TMA descriptors of the three A buffers (4D: j, i, k, component): box with halo rows for
  // A^n, box of the tile rows for A^{n-1} and J.
  alignas(64) unsigned char map_an[3][128];
  alignas(64) unsigned char map_c[3][128];
  bool tma_ready = false;
  int* tma_error = nullptr;
};

}  // namespace mithra

struct mithra_ctx {
  int device = 0;
  int precision = MITHRA_PRECISION_FP64;
  cudaStream_t stream = nullptr;
  mithra::GridDev g{};
  mithra::PushDev P{};
  mithra_grid_desc grid_desc{};
  mithra_push_desc push_desc{};
  std::vector<mithra::UndDev> und_host;
  mithra::UndDev* und_dev = nullptr;
  std::vector<mithra::BeamDev> opt_beams;  // laser beams of the optical undulators, in module order
  std::vector<mithra::BeamDev> ext_beams;  // external fields
  mithra::BeamDev* beams_dev = nullptr;    // opt_beams then ext_beams
  mithra::SeedDev seed{};
  bool seed_active = false;
  double* A[3] = {nullptr, nullptr, nullptr};  // FP64 form: three time levels of A (SoA)
  double* F[3] = {nullptr, nullptr, nullptr};  // FP64 form: three time levels of phi
  double* Jedge = nullptr;  // FP64 form: current of the deposit in edge form (k_deposit_fp64)
  mithra::ParticlesDev<double> pt{};
  mithra::Fp32State f32{};
  float* E = nullptr;  // mixed form: E and B as node records {E, 0, B, 0} (kEBNode floats per node)
  float* B = nullptr;  // unused (B of node m is E[kEBNode m + 4 + c])
  double* E64 = nullptr;  // FP64 form: E and B as doubles holding float-rounded values
  double* B64 = nullptr;
  uint8_t* plane_needed = nullptr;  // N2 flags: planes read by a power sample
  int* eb_planes = nullptr;         // the interior planes whose E/B those flags require (mixed form)
  int n_eb_planes = 0;
  void* und_table = nullptr;        // mixed form: per-plane undulator lz and phase
  int idx[3] = {0, 1, 2};  // buffer index of np1, n, nm1
  size_t capacity = 0;
  mithra::StateDev* st = nullptr;
  mithra::StateDev* st_host = nullptr;  // pinned mirror
  std::vector<mithra::PowerOut> power;
  long long row_cap = 0;
  long long rows_pending = 0;  // power rows appended since the last drain (host-side count)
  cudaGraphExec_t graph[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};  // buffer rotation x sort parity
  bool timing = false;
  std::vector<mithra::KernelTimer> timers;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
  bool particles_loaded = false;
  std::string err;
  int sm_count = 152;
  unsigned graph_generation = 0;  // incremented whenever the captured step graphs are dropped
  mithra_tuning tune{16, 64};     // launch shapes (mithra_gpu_set_tuning / mithra_gpu_autotune)
  long long wait_limit = -1;      // attempts of a device barrier wait (negative: the kernels' default)
  int launches_per_step = 0;
  int launch_counter = 0;
  void* diag_partial = nullptr;  // bunch diagnostics: per-block compensated sums (allocated on first use)
  double* diag_out = nullptr;
  void* staging = nullptr;  // device staging buffer for host-layout transfers
  size_t staging_bytes = 0;
  // lab-frame screens (mithra_gpu_set_screens): records appended by k_screen every step
  int n_screens = 0;
  long long screen_cap = 0;              // records per screen
  double* screen_lz = nullptr;           // [n_screens]
  double* screen_rec = nullptr;          // [n_screens][screen_cap][6]
  long long* screen_key = nullptr;       // [n_screens][screen_cap]
  unsigned long long* screen_count = nullptr;  // [n_screens]
};

namespace mithra {

int fail(mithra_ctx* c, int code, const char* fmt, ...);
int grid_stride_blocks(const mithra_ctx* ctx, long long work, int block);
int timer_begin(mithra_ctx* ctx, const char* name, int* slot, cudaEvent_t* a, cudaEvent_t* b);
int timer_end(mithra_ctx* ctx, int slot, cudaEvent_t a, cudaEvent_t b);
int harvest_timers(mithra_ctx* ctx);
void invalidate_graphs(mithra_ctx* ctx);

#define CK(call)                                                                                        \
  do {                                                                                                  \
    cudaError_t e_ = (call);                                                                            \
    if (e_ != cudaSuccess) return ::mithra::fail(ctx, MITHRA_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

template <typename T>
cudaError_t dalloc(T** p, size_t n) {
  return cudaMalloc((void**)p, (n ? n : 1) * sizeof(T));
}

inline long long round_up(long long v, long long m) { return (v + m - 1) / m * m; }

// Returns a device staging buffer of at least `bytes` (kept for later transfers).
int staging(mithra_ctx* ctx, size_t bytes, void** p);

// Launches one kernel through `fn` on ctx->stream; in timing mode it is bracketed by CUDA
// events recorded on the same stream and accumulated under `name`.
template <typename Fn>
int timed(mithra_ctx* ctx, const char* name, Fn fn) {
  int slot = 0;
  cudaEvent_t a = nullptr, b = nullptr;
  if (ctx->timing) {
    int r = timer_begin(ctx, name, &slot, &a, &b);
    if (r) return r;
  }
  fn();
  ctx->launch_counter++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(ctx, MITHRA_ERR_CUDA, "launch %s: %s", name, cudaGetErrorString(e));
  if (ctx->timing) return timer_end(ctx, slot, a, b);
  return MITHRA_OK;
}

// TF/SF injection of the seed into the new vector potential (float or double storage).
int stage_seed(mithra_ctx* ctx, void* anp1);

// One field step as a graph, for composing several contexts into one launch (batch.cu):
// step_key names the rotation / sort-parity state a captured step belongs to, capture_step
// records one step without applying it, after_step applies the host-side state change of a
// launched step, prepare_run / finish_run bracket a run of steps (row log, state checks).
int step_key(const mithra_ctx* ctx);
int capture_step(mithra_ctx* ctx, cudaGraph_t* out);
void after_step(mithra_ctx* ctx);
int prepare_run(mithra_ctx* ctx, int64_t nsteps);
int finish_run(mithra_ctx* ctx);

// Mixed-precision form (fp32_form.cu).
int fp32_alloc(mithra_ctx* ctx);
void fp32_free(mithra_ctx* ctx);
float* fp32_field(mithra_ctx* ctx, int level);   // level 0 = np1, 1 = n, 2 = nm1
float* fp32_scalar(mithra_ctx* ctx, int level);
int fp32_records_to_soa(mithra_ctx* ctx, const double* staging, long long n);
int fp32_soa_to_records(mithra_ctx* ctx, double* staging, long long slots, long long* n_out);
int fp32_field_update(mithra_ctx* ctx);
int fp32_eval_eb(mithra_ctx* ctx, bool full = false);
int fp32_push(mithra_ctx* ctx, int save_rnm);
int fp32_save_positions(mithra_ctx* ctx);
int fp32_erase(mithra_ctx* ctx);
int fp32_current(mithra_ctx* ctx);
int fp32_sort(mithra_ctx* ctx);          // tile sort into the other buffer set, which becomes current
int fp32_unsorted(mithra_ctx* ctx, long long n);  // bins that hold all n particles outside the tiles
bool fp32_sorts_this_step(const mithra_ctx* ctx);
void fp32_after_step(mithra_ctx* ctx);  // swap the particle buffer sets as one step's sort did

}  // namespace mithra
