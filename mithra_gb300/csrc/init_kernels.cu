// Device-side bunch initialisation (see host/devinit.h): ellipsoid bunches generated from the
// Halton sequence, boosted, back-propagated, distributed and shifted on the GPU.
//
// This translation unit is compiled with --fmad=false: every product and sum is rounded on its
// own, as in the host build (-ffp-contract=off), so the arithmetic matches the host
// initialisation operation for operation; only log/sin/cos/sqrt... come from the device math
// library (sqrt and division are correctly rounded on both sides, log/sin/cos may differ in the
// last place).
//
// Order: the reference appends particles candidate by candidate and drops the truncated ones, so
// the output order is the candidate order.  Candidates are split into one contiguous chunk per
// block; a block counts its survivors, one block scans the counts, and each block then walks its
// chunk again and writes its survivors at their place (ballot ranks within a warp, running sum
// across the block's tiles).  The same scheme compacts the particles kept by distribute().
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "host/devinit.h"

namespace mithra {
namespace devinit {
namespace {

constexpr double kPI = 3.1415926535;  // src/stdinclude.h:43 (the reference's truncated value)
constexpr int kBlock = 256;
constexpr int kMaxBlocks = 1024;
constexpr int REC = 11;

// Halton radical inverse, halton(i, j) of src/stdinclude.cpp:45-73 (1 - x of base prime[i]).
__device__ double halton(unsigned i, unsigned j) {
  const unsigned prime[20] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61, 67, 71};
  const int p = (int)prime[i];
  int p0 = p, k = (int)(j + 1);
  double x = 0.0;
  while (k > 0) {
    const int a = k % p;
    x += a / (double)p0;
    k = k / p;
    p0 *= p;
  }
  return 1.0 - x;
}

__device__ __forceinline__ double gauss_r(double s, unsigned d0, unsigned d1, unsigned n, bool use_sin) {
  const double a = sqrt(-2.0 * log(halton(d0, n)));
  const double ph = 2.0 * kPI * halton(d1, n);
  return s * a * (use_sin ? sin(ph) : cos(ph));
}

// Longitudinal offset of candidate i (index n = i + Np0), main or taper part.
__device__ double candidate_z(const Ellipsoid& e, unsigned i) {
  const unsigned n = i + e.Np0;
  if (i < e.n_main) {
    if (!e.gaussian) return (2.0 * halton(2, n) - 1.0) * e.sig_r[2];
    return gauss_r(e.sig_r[2], 2, 3, n, true);
  }
  double t0 = 2.0 * e.lambda * sqrt(-2.0 * log(halton(2, n))) * sin(2.0 * kPI * halton(3, n));
  t0 += (t0 < 0.0) ? (-e.sig_r[2]) : (e.sig_r[2]);
  return t0;
}

// Position and momentum offsets of candidate i; true when it survives the truncation.
__device__ bool candidate(const Ellipsoid& e, unsigned i, double* r, double* t) {
  const unsigned n = i + e.Np0;
  r[0] = gauss_r(e.sig_r[0], 0, 1, n, false);
  r[1] = gauss_r(e.sig_r[1], 0, 1, n, true);
  r[2] = candidate_z(e, i);
  t[0] = gauss_r(e.sig_gb[0], 4, 5, n, false);
  t[1] = gauss_r(e.sig_gb[1], 4, 5, n, true);
  t[2] = gauss_r(e.sig_gb[2], 6, 7, n, false);
  return fabs(r[0]) < e.tran_trun && fabs(r[1]) < e.tran_trun && fabs(r[2]) < e.long_trun;
}

unsigned n_candidates(const Ellipsoid& e) { return e.gaussian ? e.n_main : e.n_taper; }

// Total order of doubles as unsigned 64-bit keys (for atomicMin / atomicMax).
__device__ __forceinline__ unsigned long long dkey(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
double from_key(unsigned long long k) {
  const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  double v;
  memcpy(&v, &b, 8);
  return v;
}

__global__ void k_candidate_zmin(Ellipsoid e, unsigned n, unsigned long long* out) {
  unsigned long long best = ~0ull;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const unsigned long long k = dkey(candidate_z(e, i));
    best = k < best ? k : best;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long y = __shfl_down_sync(0xffffffffu, best, o);
    best = y < best ? y : best;
  }
  if ((threadIdx.x & 31) == 0) atomicMin(out, best);
}

// ---- order-preserving compaction over per-block chunks -----------------------------------

// Exclusive rank of a true flag among the block's threads for one tile, and the tile's total.
__device__ int tile_rank(bool flag, int* s_warp, int* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned bal = __ballot_sync(0xffffffffu, flag);
  if (lane == 0) s_warp[warp] = __popc(bal);
  __syncthreads();
  int before = 0, sum = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
    if (w < warp) before += s_warp[w];
    sum += s_warp[w];
  }
  __syncthreads();
  *total = sum;
  return before + __popc(bal & ((1u << lane) - 1u));
}

struct CandidatePred {
  Ellipsoid e;
  __device__ bool operator()(unsigned i) const {
    double r[3], t[3];
    return candidate(e, i, r, t);
  }
};

struct DomainPred {
  const double* rec;
  double zmin, Lz, zp0, zp1;
  __device__ bool operator()(unsigned i) const {  // Solver::particleInProcessor
    const double z = rec[(size_t)REC * i + 3];
    double x = fmod(z - zmin, Lz);
    x += (x < 0.0) ? Lz : 0.0;
    const double zr = x + zmin;
    return zr >= zp0 && zr < zp1;
  }
};

template <typename Pred>
__global__ void k_count(Pred pred, unsigned n, unsigned chunk, int* counts) {
  __shared__ int s_warp[kBlock / 32];
  const unsigned beg = blockIdx.x * chunk, end = min(n, beg + chunk);
  int count = 0;
  for (unsigned base = beg; base < end; base += blockDim.x) {
    const unsigned i = base + threadIdx.x;
    int total;
    tile_rank(i < end && pred(i), s_warp, &total);
    count += total;
  }
  if (threadIdx.x == 0) counts[blockIdx.x] = count;
}

__global__ void k_scan_counts(int* counts, int nblocks) {  // one block of kMaxBlocks threads
  __shared__ int s[kMaxBlocks];
  s[threadIdx.x] = threadIdx.x < (unsigned)nblocks ? counts[threadIdx.x] : 0;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int b = 0; b < nblocks; b++) {
      const int v = s[b];
      s[b] = run;
      run += v;
    }
    counts[nblocks] = run;
  }
  __syncthreads();
  if (threadIdx.x < (unsigned)nblocks) counts[threadIdx.x] = s[threadIdx.x];
}

// Candidates -> records: ng beamlet particles per survivor (insert of initializeEllipsoid).
__global__ void k_emit(Ellipsoid e, unsigned n, unsigned chunk, const int* offsets, double zmin, double bF,
                       double* out) {
  __shared__ int s_warp[kBlock / 32];
  const unsigned beg = blockIdx.x * chunk, end = min(n, beg + chunk);
  int run = offsets[blockIdx.x];
  for (unsigned base = beg; base < end; base += blockDim.x) {
    const unsigned i = base + threadIdx.x;
    double r[3], t[3];
    const bool keep = i < end && candidate(e, i, r, t);
    int total;
    const int rank = tile_rank(keep, s_warp, &total);
    if (keep) {
      double c[3], gb[3];
      for (int d = 0; d < 3; d++) { c[d] = e.pos[d] + r[d]; gb[d] = e.gb[d] + t[d]; }
      double* o = out + (size_t)REC * ((size_t)(run + rank) * e.ng);
      for (unsigned ii = 0; ii < e.ng; ii++, o += REC) {
        double z = c[2];
        if (e.shot_noise) {
          const int bmi = int((c[2] - zmin) / e.lambda);
          const double bFi = bF * sqrt(-2.0 * log(halton(8, (unsigned)bmi)));
          z = c[2] - e.lambda / 4 * ii;
          z -= e.lambda / kPI * bFi * sin(2.0 * kPI / e.lambda * z + 2.0 * kPI * halton(9, (unsigned)bmi));
        } else if (e.lambda != 0.0) {
          z = c[2] - e.lambda / 4 * ii;
          z -= e.lambda / kPI * e.bF_user * sin(2.0 * kPI / e.lambda * z + e.bFP * kPI / 180.0);
        }
        o[0] = e.q;
        o[1] = c[0]; o[2] = c[1]; o[3] = z;
        o[4] = 0.0; o[5] = 0.0; o[6] = 0.0;
        o[7] = gb[0]; o[8] = gb[1]; o[9] = gb[2];
        o[10] = 0.0;
      }
    }
    run += total;
  }
}

__global__ void k_compact_records(DomainPred pred, unsigned n, unsigned chunk, const int* offsets, double* out) {
  __shared__ int s_warp[kBlock / 32];
  const unsigned beg = blockIdx.x * chunk, end = min(n, beg + chunk);
  int run = offsets[blockIdx.x];
  for (unsigned base = beg; base < end; base += blockDim.x) {
    const unsigned i = base + threadIdx.x;
    const bool keep = i < end && pred(i);
    int total;
    const int rank = tile_rank(keep, s_warp, &total);
    if (keep)
      for (int c = 0; c < REC; c++) out[(size_t)REC * (run + rank) + c] = pred.rec[(size_t)REC * i + c];
    run += total;
  }
}

// ---- per-particle maps and reductions ----------------------------------------------------

__device__ __forceinline__ double gq_of(const double* r) { return sqrt(1.0 + (r[7] * r[7] + r[8] * r[8] + r[9] * r[9])); }

__global__ void k_boost(double* rec, size_t n, double gamma, double beta, unsigned long long* zmax) {
  unsigned long long best = 0ull;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    double* r = rec + REC * p;
    const double gq = gq_of(r);
    const double bz = r[9] / gq;
    r[3] *= gamma;
    r[9] = gamma * gq * (bz - beta);
    const unsigned long long k = dkey(r[3]);
    best = k > best ? k : best;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long y = __shfl_down_sync(0xffffffffu, best, o);
    best = y > best ? y : best;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(zmax, best);
}

__global__ void k_back_propagate(double* rec, size_t n, double zu, double beta) {
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    double* r = rec + REC * p;
    const double gq = gq_of(r);
    const double z = r[3];
    r[1] += r[7] / gq * (z - zu) * beta;
    r[2] += r[8] / gq * (z - zu) * beta;
    r[3] += r[9] / gq * (z - zu) * beta;
  }
}

// Per-block compensated (Neumaier) sums of z and beta_z; min of z as an ordered key.
__global__ void k_sums(const double* rec, size_t n, double* partial, unsigned long long* zmin) {
  double s[2] = {0.0, 0.0}, c[2] = {0.0, 0.0};
  unsigned long long best = ~0ull;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    const double* r = rec + REC * p;
    const double v[2] = {r[3], r[9] / gq_of(r)};
    for (int q = 0; q < 2; q++) {
      const double tt = s[q] + v[q];
      c[q] += (fabs(s[q]) >= fabs(v[q])) ? (s[q] - tt) + v[q] : (v[q] - tt) + s[q];
      s[q] = tt;
    }
    const unsigned long long k = dkey(r[3]);
    best = k < best ? k : best;
  }
  __shared__ double sh[kBlock][2];
  sh[threadIdx.x][0] = s[0] + c[0];
  sh[threadIdx.x][1] = s[1] + c[1];
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long y = __shfl_down_sync(0xffffffffu, best, o);
    best = y < best ? y : best;
  }
  if ((threadIdx.x & 31) == 0) atomicMin(zmin, best);
  __syncthreads();
  if (threadIdx.x == 0) {
    double a[2] = {0.0, 0.0}, ac[2] = {0.0, 0.0};
    for (int t = 0; t < (int)blockDim.x; t++)
      for (int q = 0; q < 2; q++) {
        const double v = sh[t][q], tt = a[q] + v;
        ac[q] += (fabs(a[q]) >= fabs(v)) ? (a[q] - tt) + v : (v - tt) + a[q];
        a[q] = tt;
      }
    partial[2 * blockIdx.x] = a[0] + ac[0];
    partial[2 * blockIdx.x + 1] = a[1] + ac[1];
  }
}

__global__ void k_shift_z(double* rec, size_t n, double shift) {
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x)
    rec[REC * p + 3] -= shift;
}

__global__ void k_time_shift(double* rec, size_t n, double c0, double shift) {
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    double* r = rec + REC * p;
    const double t = c0 * shift / gq_of(r);
    for (int d = 0; d < 3; d++) r[1 + d] -= t * r[7 + d];
  }
}

int fail(char* err, size_t len, const char* what, cudaError_t e) {
  if (err && len) snprintf(err, len, "device initialisation: %s: %s", what, cudaGetErrorString(e));
  return -3;  // MITHRA_ERR_CUDA
}

#define DI_CK(x, what)                                   \
  do {                                                   \
    cudaError_t e_ = (x);                                \
    if (e_ != cudaSuccess) return fail(err, err_len, what, e_); \
  } while (0)

int grid_for(size_t n) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t want = (n + kBlock - 1) / kBlock;
  const size_t cap = (size_t)(sms > 0 ? sms : 1) * 8;
  return (int)std::max<size_t>(1, std::min(want, cap));
}

// Chunking of n items over at most kMaxBlocks blocks, chunk a multiple of the block size.
void chunking(size_t n, unsigned* chunk, int* nblocks) {
  size_t c = (n + kMaxBlocks - 1) / kMaxBlocks;
  c = ((c + kBlock - 1) / kBlock) * kBlock;
  if (c == 0) c = kBlock;
  *chunk = (unsigned)c;
  *nblocks = (int)std::max<size_t>(1, (n + c - 1) / c);
}

}  // namespace

int reserve(Store& s, size_t cap, char* err, size_t err_len) {
  if (cap <= s.cap) return 0;
  DI_CK(cudaSetDevice(s.device), "cudaSetDevice");
  double* p = nullptr;
  DI_CK(cudaMalloc(&p, cap * REC * sizeof(double)), "cudaMalloc");
  if (s.n) DI_CK(cudaMemcpy(p, s.rec, s.n * REC * sizeof(double), cudaMemcpyDeviceToDevice), "cudaMemcpy");
  cudaFree(s.rec);
  s.rec = p;
  s.cap = cap;
  return 0;
}

void release(Store& s) {
  if (s.rec) {
    cudaSetDevice(s.device);
    cudaFree(s.rec);
  }
  s.rec = nullptr;
  s.n = s.cap = 0;
}

int candidate_zmin(int device, const Ellipsoid& e, double* zmin, char* err, size_t err_len) {
  DI_CK(cudaSetDevice(device), "cudaSetDevice");
  unsigned long long* d = nullptr;
  DI_CK(cudaMalloc(&d, sizeof(*d)), "cudaMalloc");
  const unsigned long long init = ~0ull;
  cudaMemcpy(d, &init, sizeof(init), cudaMemcpyHostToDevice);
  const unsigned n = n_candidates(e);
  k_candidate_zmin<<<grid_for(n), kBlock>>>(e, n, d);
  unsigned long long k = 0;
  const cudaError_t r = cudaMemcpy(&k, d, sizeof(k), cudaMemcpyDeviceToHost);
  cudaFree(d);
  DI_CK(r, "candidate zmin");
  *zmin = (n > 0) ? from_key(k) : 1e100;
  return 0;
}

int generate(Store& s, const Ellipsoid& e, double zmin, double bF, char* err, size_t err_len) {
  DI_CK(cudaSetDevice(s.device), "cudaSetDevice");
  const unsigned n = n_candidates(e);
  if (n == 0) return 0;
  unsigned chunk;
  int nb;
  chunking(n, &chunk, &nb);
  int* counts = nullptr;
  DI_CK(cudaMalloc(&counts, (kMaxBlocks + 1) * sizeof(int)), "cudaMalloc");
  CandidatePred pred{e};
  k_count<<<nb, kBlock>>>(pred, n, chunk, counts);
  k_scan_counts<<<1, kMaxBlocks>>>(counts, nb);
  int survivors = 0;
  cudaError_t r = cudaMemcpy(&survivors, counts + nb, sizeof(int), cudaMemcpyDeviceToHost);
  if (r != cudaSuccess) { cudaFree(counts); return fail(err, err_len, "candidate count", r); }
  const size_t add = (size_t)survivors * e.ng;
  int rr = reserve(s, s.n + add, err, err_len);
  if (rr) { cudaFree(counts); return rr; }
  k_emit<<<nb, kBlock>>>(e, n, chunk, counts, zmin, bF, s.rec + REC * s.n);
  r = cudaDeviceSynchronize();
  cudaFree(counts);
  DI_CK(r, "generate");
  s.n += add;
  return 0;
}

int boost(Store& s, double gamma, double beta, double* zmax, char* err, size_t err_len) {
  DI_CK(cudaSetDevice(s.device), "cudaSetDevice");
  unsigned long long* d = nullptr;
  DI_CK(cudaMalloc(&d, sizeof(*d)), "cudaMalloc");
  cudaMemset(d, 0, sizeof(*d));
  if (s.n) k_boost<<<grid_for(s.n), kBlock>>>(s.rec, s.n, gamma, beta, d);
  unsigned long long k = 0;
  const cudaError_t r = cudaMemcpy(&k, d, sizeof(k), cudaMemcpyDeviceToHost);
  cudaFree(d);
  DI_CK(r, "boost");
  *zmax = s.n ? from_key(k) : -1.0e100;
  return 0;
}

int back_propagate(Store& s, double zu, double beta, char* err, size_t err_len) {
  DI_CK(cudaSetDevice(s.device), "cudaSetDevice");
  if (s.n) k_back_propagate<<<grid_for(s.n), kBlock>>>(s.rec, s.n, zu, beta);
  DI_CK(cudaDeviceSynchronize(), "back-propagation");
  return 0;
}

namespace {
int sums_and_min(Store& s, double* z, double* bz, double* zmin, char* err, size_t err_len) {
  DI_CK(cudaSetDevice(s.device), "cudaSetDevice");
  const int nb = grid_for(s.n);
  double* partial = nullptr;
  unsigned long long* dmin = nullptr;
  DI_CK(cudaMalloc(&partial, 2 * (size_t)nb * sizeof(double)), "cudaMalloc");
  DI_CK(cudaMalloc(&dmin, sizeof(*dmin)), "cudaMalloc");
  const unsigned long long init = ~0ull;
  cudaMemcpy(dmin, &init, sizeof(init), cudaMemcpyHostToDevice);
  if (s.n) k_sums<<<nb, kBlock>>>(s.rec, s.n, partial, dmin);
  std::vector<double> h(2 * (size_t)nb, 0.0);
  unsigned long long k = ~0ull;
  cudaError_t r = cudaMemcpy(h.data(), partial, h.size() * sizeof(double), cudaMemcpyDeviceToHost);
  if (r == cudaSuccess) r = cudaMemcpy(&k, dmin, sizeof(k), cudaMemcpyDeviceToHost);
  cudaFree(partial);
  cudaFree(dmin);
  DI_CK(r, "sums");
  double a[2] = {0.0, 0.0}, c[2] = {0.0, 0.0};
  for (int b = 0; b < (s.n ? nb : 0); b++)
    for (int q = 0; q < 2; q++) {
      const double v = h[2 * b + q], t = a[q] + v;
      c[q] += (std::fabs(a[q]) >= std::fabs(v)) ? (a[q] - t) + v : (v - t) + a[q];
      a[q] = t;
    }
  if (z) *z = a[0] + c[0];
  if (bz) *bz = a[1] + c[1];
  if (zmin) *zmin = s.n ? from_key(k) : 1e100;
  return 0;
}
}  // namespace

int sums_z_bz(Store& s, double* z, double* bz, char* err, size_t err_len) { return sums_and_min(s, z, bz, nullptr, err, err_len); }

int min_z(Store& s, double* zmin, char* err, size_t err_len) { return sums_and_min(s, nullptr, nullptr, zmin, err, err_len); }

int shift_z(Store& s, double shift, char* err, size_t err_len) {
  DI_CK(cudaSetDevice(s.device), "cudaSetDevice");
  if (s.n) k_shift_z<<<grid_for(s.n), kBlock>>>(s.rec, s.n, shift);
  DI_CK(cudaDeviceSynchronize(), "shift");
  return 0;
}

int distribute(Store& s, double zmin, double Lz, double zp0, double zp1, char* err, size_t err_len) {
  DI_CK(cudaSetDevice(s.device), "cudaSetDevice");
  if (s.n == 0) return 0;
  unsigned chunk;
  int nb;
  chunking(s.n, &chunk, &nb);
  int* counts = nullptr;
  double* out = nullptr;
  DI_CK(cudaMalloc(&counts, (kMaxBlocks + 1) * sizeof(int)), "cudaMalloc");
  DomainPred pred{s.rec, zmin, Lz, zp0, zp1};
  k_count<<<nb, kBlock>>>(pred, (unsigned)s.n, chunk, counts);
  k_scan_counts<<<1, kMaxBlocks>>>(counts, nb);
  int kept = 0;
  cudaError_t r = cudaMemcpy(&kept, counts + nb, sizeof(int), cudaMemcpyDeviceToHost);
  if (r == cudaSuccess) r = cudaMalloc(&out, std::max<size_t>(1, s.cap) * REC * sizeof(double));
  if (r != cudaSuccess) { cudaFree(counts); return fail(err, err_len, "distribute", r); }
  k_compact_records<<<nb, kBlock>>>(pred, (unsigned)s.n, chunk, counts, out);
  r = cudaDeviceSynchronize();
  cudaFree(counts);
  if (r != cudaSuccess) { cudaFree(out); return fail(err, err_len, "distribute", r); }
  cudaFree(s.rec);
  s.rec = out;
  s.n = (size_t)kept;
  return 0;
}

int time_shift(Store& s, double c0, double shift, char* err, size_t err_len) {
  DI_CK(cudaSetDevice(s.device), "cudaSetDevice");
  if (s.n) k_time_shift<<<grid_for(s.n), kBlock>>>(s.rec, s.n, c0, shift);
  DI_CK(cudaDeviceSynchronize(), "time shift");
  return 0;
}

int download(const Store& s, double* rec, size_t n, char* err, size_t err_len) {
  DI_CK(cudaSetDevice(s.device), "cudaSetDevice");
  if (n) DI_CK(cudaMemcpy(rec, s.rec, n * REC * sizeof(double), cudaMemcpyDeviceToHost), "download");
  return 0;
}

}  // namespace devinit
}  // namespace mithra
