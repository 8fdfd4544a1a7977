// Shared device-side definitions of the GB300 FdTd library.
//
// Device layout (both precision forms):
//   * every scalar field component is its own array of N2 planes of N0 rows of P1 values
//     (P1 = N1 rounded up to a multiple of 8), node (k, i, j) at k*plane + i*P1 + j;
//     the three components of A (and of E, B) are `cstride` apart.  SoA keeps each stencil
//     load a coalesced row segment; the padded pitch keeps rows 16-byte aligned for vector
//     and bulk-tensor copies.
//   * particles are structure-of-arrays (position, momentum, previous position, charge, entry
//     flag), plus a status byte (bit 0: erased) and a crossing byte written by the push.
#pragma once
#include <cstring>
#include <cstdint>
#include <cuda_runtime.h>

namespace mithra {

constexpr int kMaxUndulators = 64;
constexpr double kPI = 3.1415926535;  // src/stdinclude.h:43 (truncated value kept for parity)
constexpr double kEM = 9.109e-31;     // src/stdinclude.h:51
constexpr double kEC = 1.602e-19;     // src/stdinclude.h:50

struct GridDev {
  int N0, N1, N2, P1;
  long long plane;    // N0 * P1
  long long cstride;  // distance between components
  int solver, order, space_charge;
  double a[6];
  double nsfd_alpha, nsfd_beta;
  double bB[5], cB[5], dB[5], eE[5], fE[5], gE[5], hC[17];
  double dt, dx, dy, dz;
  double rdx, rdy, rdz;  // reciprocals of dx, dy, dz
  double xmin, xmax, ymin, ymax, zmin, zmax, zp0, zp1, Lz;
};

__host__ __device__ inline long long node_index(const GridDev& g, int k, int i, int j) {
  return (long long)k * g.plane + (long long)i * g.P1 + j;
}

// Laser beams (evaluated in beam_fields.cuh).
struct SignalDev {  // Signal (src/classes.h:159-195); cep in radians, f0 = 1 / wavelength
  int type;         // 0 neumann, 1 gaussian, 2 secant-hyperbolic, 3 flat-top, 4 inverse-gaussian
  double t0, s, f0, cep, nR, g0, g1;
};

struct BeamDev {  // the laser-beam members shared by Seed, Undulator and ExtField
  int type;       // SeedType: 0 plane, 1 truncated plane, 2 gaussian, 3 super-gaussian, 4..7 standing
  double pos[3], dir[3], pol[3];
  double yv[3];   // cross(direction, polarization)
  double amplitude, r0, r1;
  int o0, o1;
  double l, zR0, zR1;
  SignalDev sig;
};

struct SeedDev {
  BeamDev b;
  double gamma, beta, c0, dt;  // Seed::gamma_, beta_, c0_, dt_
  double l, zRp, zRs;          // c0 / f0 and the two Rayleigh lengths of Seed::fields
  double a1, a2, a3;           // uf_.a[1..3], the TF/SF coefficients
};

struct UndDev {
  int type;
  int beam;  // optical modules: index of the laser beam in PushDev::beams, else -1
  double k, lu, rb, length, dist, theta;
  // Per-module constants of Solver::undulatorField (src/solver.cpp:1805-1812), computed on
  // the host with the reference's expressions so that they are bit-identical.
  double b0, ku, ct, st, ul;  // ul = length * lu
  double r0_prev, r0_next;    // gap to the previous / next module (src/beam.cc:35, :60)
  int has_prev, has_next;
  // FP32 copies for the mixed form.
  float ct_f, st_f, ku_f, b0_f, ul_f, r0_prev_f, r0_next_f;
  double kgdz;      // ku * gamma * dz: the phase advance across one cell along z
  double kgdz_sub;  // the same across one sub-plane interval of the FP64 phase table
};

// Sub-planes per cell of the FP64 form's undulator phase table (k_undulator_table64).
constexpr int kUndSub = 4;

// FP64 form: a static module's lz and the sine and cosine of its phase ku*lz on node plane k,
// for the bunch time of one substep (k_undulator_table64).
struct UndPlane64 {
  double lz, s, c;
};

struct PushDev {
  double dtb, r1, r2, gamma, beta, c0, dt_shift, bunch_time_step;
  double inv_r2;  // 1 / r2
  // FP64 form: per-plane undulator phases (UndPlane64, n_und x (N2 + 1)), or null where the
  // phase advance across a cell is too large for the short series of the push.
  const UndPlane64* und_planes;
  double gdz;     // gamma * dz
  double gdz_sub; // gamma * dz / kUndSub
  int n_und;
  double und0_dist;
  // Laser beams acting on the particles: optical undulators (indexed by UndDev::beam) and,
  // from ext0 on, the n_ext external fields.
  const BeamDev* beams;
  int ext0, n_ext, n_opt;
};

// Device-resident time and bookkeeping state of one context.  The kernels advance it
// themselves so that a captured step graph can be replayed without host involvement.
struct StateDev {
  double time, time_bunch;
  long long n_time, n_time_bunch;
  long long n_particles;     // particle slots in use (erased ones included)
  long long capacity;
  unsigned long long n_cross;       // particles that crossed a z face in the last substep
  unsigned long long n_transverse;  // particles outside the transverse domain (diagnostic)
  int overflow;                     // set when appended copies would exceed the capacity
  int nonfinite;
  int j_edges;  // FP64 form: the current of the last deposit is held in edge form (see k_deposit_fp64)
  long long n_power_rows;
  long long power_row_cap;
  // z-slab (cells) occupied by particles: E/B are evaluated only where a gather can read them.
  int k_lo, k_hi;            // range used by this step's E/B evaluation
  int k_lo_next, k_hi_next;  // accumulated by the deposit for the next step
  long long next_id;         // mixed form: id given to the next z-face copy
};

// Min/max of particle cells along z, reduced per warp and folded into the state with atomics.
// Every warp of a deposit reaches this with a range, and atomics on the two words serialise in
// one L2 slice, so a warp reads the words first and issues an atomic only when its range extends
// them; a stale read costs an extra atomic, never a wrong range.
__device__ __forceinline__ void slab_update(StateDev* st, int kmin, int kmax) {
  for (int o = 16; o > 0; o >>= 1) {
    kmin = min(kmin, __shfl_down_sync(0xffffffffu, kmin, o));
    kmax = max(kmax, __shfl_down_sync(0xffffffffu, kmax, o));
  }
  if ((threadIdx.x & 31) == 0 && kmin <= kmax) {
    if (kmin < *reinterpret_cast<volatile int*>(&st->k_lo_next)) atomicMin(&st->k_lo_next, kmin);
    if (kmax > *reinterpret_cast<volatile int*>(&st->k_hi_next)) atomicMax(&st->k_hi_next, kmax);
  }
}

template <typename T>
struct ParticlesDev {
  T *x, *y, *z;        // rnp
  T *gx, *gy, *gz;     // gb
  T *mx, *my, *mz;     // rnm
  T *q, *e;
  uint8_t* status;     // bit 0: erased
  int8_t* cross;       // 0 none, 1 below zp0, 2 at/above zp1
};

// Particles of the mixed-precision form: integer cell coordinates packed into one 64-bit word
// (21 bits per axis, biased by 2^20, so positions far outside the mesh stay representable), the
// FP32 offset inside the cell in units of the cell size, FP32 gamma*beta.  The previous position
// is kept in the same form for the deposit.
struct ParticlesF32 {
  long long* cell;
  float *fx, *fy, *fz;
  float *gx, *gy, *gz;
  long long* mcell;
  float *mfx, *mfy, *mfz;
  float* q;
  uint8_t* e;
  uint8_t* status;
  int8_t* cross;
  int* id;  // creation index: initial list position, or the slot of a z-face copy
};

constexpr long long kCellBias = 1LL << 20;
__host__ __device__ __forceinline__ long long pack_cell(int i, int j, int k) {
  return ((long long)(i + kCellBias) << 42) | ((long long)(j + kCellBias) << 21) | (long long)(k + kCellBias);
}
__host__ __device__ __forceinline__ void unpack_cell(long long c, int& i, int& j, int& k) {
  i = (int)((c >> 42) & 0x1FFFFF) - (int)kCellBias;
  j = (int)((c >> 21) & 0x1FFFFF) - (int)kCellBias;
  k = (int)(c & 0x1FFFFF) - (int)kCellBias;
}

// One radiation-power output on the device (see power_kernels.cuh).
struct PowerDev {
  int N, Nl, Nf;
  int nz;                   // planes owned by this domain
  double pc;                // power constant (src/radiation.cpp:106)
  double gamma, beta, c0, dt_shift;
  const double* z;          // N boosted plane positions
  const int* plane_k;       // N: cell index of the plane, or -1 when outside [zp0, zp1)
  const double* plane_dzr;  // N: fractional position inside that cell
  const int* plane_slot;    // N: compressed index kz of each owned plane
  const double* tw_re;      // Nl*Nf twiddles cos(w_l j dt)
  const double* tw_im;      // Nl*Nf twiddles sin(w_l j dt)
  double* fdt;              // ring buffer: Nf slots x 4 values x nz planes x nodes
  double* run;              // mixed form: running DFT sums, (Nl x 8) x nz planes x nodes; null: full sums
  double* partial;          // (blocks) x Nl
  double* rows;             // row log: row_cap rows of N*(1+Nl) doubles
  int nodes_i, nodes_j;     // N0-4, N1-4
  int blocks_per_plane;
  long long row_cap;
};

// E and B of the mixed form are stored node by node: node m holds the 32-byte record
// {Ex, Ey, Ez, 0, Bx, By, Bz, 0} at EB + 8 m.  A particle's gather reads each of its 8 nodes with
// one 32-byte load from one sector (component planes would take 6 sectors per node), and the
// evaluation writes a node with one 32-byte store (256-bit vector loads and stores, sm_100 and
// later).  Component c of node m: E at
// EB[8 m + c], B at EB[8 m + 4 + c].
constexpr int kEBNode = 8;

__device__ __forceinline__ void store_eb(float* EB, long long m, float e0, float e1, float e2, float b0, float b1,
                                         float b2) {
  asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(EB + (long long)kEBNode * m), "f"(e0),
               "f"(e1), "f"(e2), "f"(0.0f), "f"(b0), "f"(b1), "f"(b2), "f"(0.0f)
               : "memory");
}

// One node record as a single 32-byte load (a 256-bit vector load, sm_100 and later), through
// the read-only path: the gather reads 8 records per particle, one load instruction each.
__device__ __forceinline__ void load_eb(const float* EB, long long m, float4& e, float4& b) {
  asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=f"(e.x), "=f"(e.y), "=f"(e.z), "=f"(e.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
      : "l"(EB + (long long)kEBNode * m));
}

// True when node plane k has to be evaluated: inside the particle slab (with two cells of margin
// for the motion during the step) or read by a power sample.
__device__ __forceinline__ bool eb_plane_wanted(int k, const StateDev* st, const uint8_t* planes, int N2) {
  if (!st) return true;
  const int lo = st->k_lo - 2, hi = st->k_hi + 3;
  if (k >= lo && k <= hi) return true;
  if (planes && (planes[k] || (k == 1 && planes[0]) || (k == N2 - 2 && planes[N2 - 1]))) return true;
  return false;
}

// Conversions between double and float done on the integer pipes.  GB300 issues FP64 work at a
// small fraction of its FP32 rate and a hardware F2F conversion costs about two FP64 slots, while
// E/B evaluation of the FP64 form converts 18 times per node (the reference stores E, B as
// float).  Both functions are exact: round-to-nearest-even for double -> float, bit widening for
// float -> double; zero is handled here, subnormal/inf/nan go to the hardware conversion.
__host__ __device__ __forceinline__ unsigned long long bits_of(double x) {
#ifdef __CUDA_ARCH__
  return (unsigned long long)__double_as_longlong(x);
#else
  unsigned long long u;
  memcpy(&u, &x, 8);
  return u;
#endif
}
__host__ __device__ __forceinline__ double double_of(unsigned long long u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, 8);
  return x;
#endif
}
__host__ __device__ __forceinline__ unsigned bits_of(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  unsigned u;
  memcpy(&u, &x, 4);
  return u;
#endif
}
__host__ __device__ __forceinline__ float float_of(unsigned u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float x;
  memcpy(&x, &u, 4);
  return x;
#endif
}

__host__ __device__ __forceinline__ float to_float_rn(double x) {
  const unsigned long long u = bits_of(x);
  const unsigned hi = (unsigned)(u >> 32), lo = (unsigned)u;
  const unsigned e = (hi >> 20) & 0x7ffu;
  const unsigned sign = hi & 0x80000000u;
  if (e >= 897u && e <= 1150u) {  // a normal float before rounding (float exponent 1..254)
    unsigned r = ((e - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rem = lo & 0x1fffffffu, half = 0x10000000u;
    r += (rem > half) | ((rem == half) & (r & 1u));  // a carry into the exponent is correct, up to inf
    return float_of(sign | r);
  }
  if (((hi & 0x7fffffffu) | lo) == 0u) return float_of(sign);  // +-0
  return (float)x;
}

__host__ __device__ __forceinline__ double to_double(float f) {
  const unsigned b = bits_of(f);
  const unsigned e = (b >> 23) & 0xffu;
  if (e != 0u && e != 255u) {
    const unsigned hi = (b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7fffffu) >> 3);
    return double_of(((unsigned long long)hi << 32) | ((unsigned long long)(b & 7u) << 29));
  }
  if ((b & 0x7fffffffu) == 0u) return double_of((unsigned long long)(b & 0x80000000u) << 32);  // +-0
  return (double)f;
}

// Comparisons, floors and truncations of doubles on the integer pipes, for the FP64 kernels that
// GB300's FP64 rate bounds: a DSETP, DMNMX, FRND or F2I takes an FP64 issue slot, a few integer
// instructions do not.  All are exact.
//
// dkey: a 64-bit integer that orders as the double does (not NaN; -0 and +0 equal):
// a < b exactly when dkey(a) < dkey(b).
__host__ __device__ __forceinline__ long long dkey(double x) {
  const long long b = (long long)bits_of(x);
  const long long s = b >> 63;  // -1 for negative, else 0
  return (b ^ (s & 0x7fffffffffffffffLL)) - s;
}

// x is a NaN, from its bits: dkey orders NaNs beyond the infinities, where every FP64 comparison
// with them is false, so a caller that relies on those comparisons being false tests for NaN first.
__host__ __device__ __forceinline__ bool is_nan_bits(double x) {
  return (bits_of(x) & 0x7fffffffffffffffULL) > 0x7ff0000000000000ULL;
}

// floor(t) as an int for |t| < 2^31, from the bits of t (negative t, rare in the callers, takes
// the hardware path).
__host__ __device__ __forceinline__ int ifloor_d(double t) {
  const long long b = (long long)bits_of(t);
  if (b < 0) return (int)floor(t);
  const int e = (int)(b >> 52) - 1023;
  if (e < 0) return 0;
  const long long m = (b & 0xfffffffffffffLL) | 0x10000000000000LL;
  return (int)(m >> (52 - e));
}

// modf for |t| < 2^31: returns t - trunc(t) and stores trunc(t), formed by clearing the fraction
// bits of t (one FP64 subtraction, exact; an integral t gives +0 where modf gives a signed zero).
__host__ __device__ __forceinline__ double modf_d(double t, double* ip) {
  const long long b = (long long)bits_of(t);
  const int e = (int)((b >> 52) & 0x7ff) - 1023;
  long long tb;
  if (e < 0) tb = b & (long long)0x8000000000000000ULL;  // |t| < 1: trunc(t) = +-0
  else if (e >= 52) tb = b;                                // already integral
  else tb = b & ~((1LL << (52 - e)) - 1);
  const double tr = double_of((unsigned long long)tb);
  *ip = tr;
  return t - tr;
}

// trunc(t) as an int for |t| < 2^31 and the bits of trunc(t) from modf_d (no FP64 conversion).
__host__ __device__ __forceinline__ int itrunc_d(double tr) {
  const long long b = (long long)bits_of(tr);
  const int e = (int)((b >> 52) & 0x7ff) - 1023;
  if (e < 0) return 0;
  const int mag = (int)(((b & 0xfffffffffffffLL) | 0x10000000000000LL) >> (52 - e));
  return b < 0 ? -mag : mag;
}

// (double)n for an int, exactly, from the bits (no FP64 conversion).
__host__ __device__ __forceinline__ double double_of_int(int n) {
  if (n == 0) return 0.0;
  const unsigned long long sign = n < 0 ? 0x8000000000000000ULL : 0ULL;
  const unsigned mag = n < 0 ? 0u - (unsigned)n : (unsigned)n;
#ifdef __CUDA_ARCH__
  const int top = 31 - __clz(mag);
#else
  const int top = 31 - __builtin_clz(mag);
#endif
  const unsigned long long m = ((unsigned long long)mag << (52 - top)) & 0xfffffffffffffULL;
  return double_of(sign | ((unsigned long long)(1023 + top) << 52) | m);
}

// The smaller / larger of two doubles (not NaN) by their integer keys (fmin / fmax up to the
// sign of a zero result).
__host__ __device__ __forceinline__ double dmin_k(double a, double b) { return dkey(b) < dkey(a) ? b : a; }
__host__ __device__ __forceinline__ double dmax_k(double a, double b) { return dkey(a) < dkey(b) ? b : a; }

// sin d and cos d for |d| <= 1/4 (the push's advance within one sub-plane interval of the phase
// table): Taylor series in d^2 (coefficients (-1)^n/(2n+1)! and (-1)^n/(2n)!) by Horner's rule,
// cut after d^11 and d^12 (the first terms left out, d^13/13! and d^14/14!, stay below 3e-18), 14
// FP64 operations and no range reduction.
__host__ __device__ __forceinline__ void sin_cos_series_short(double d, double* sd, double* cd) {
  const double d2 = d * d;
  double ps = -1.0 / 39916800.0;                           // -1/11!
  ps = fma(ps, d2, 1.0 / 362880.0);                        //  1/9!
  ps = fma(ps, d2, -1.0 / 5040.0);                         // -1/7!
  ps = fma(ps, d2, 1.0 / 120.0);                           //  1/5!
  ps = fma(ps, d2, -1.0 / 6.0);                            // -1/3!
  *sd = fma(d * d2, ps, d);
  double pc = 1.0 / 479001600.0;                           //  1/12!
  pc = fma(pc, d2, -1.0 / 3628800.0);                      // -1/10!
  pc = fma(pc, d2, 1.0 / 40320.0);                         //  1/8!
  pc = fma(pc, d2, -1.0 / 720.0);                          // -1/6!
  pc = fma(pc, d2, 1.0 / 24.0);                            //  1/4!
  pc = fma(pc, d2, -0.5);                                  // -1/2!
  *cd = fma(d2, pc, 1.0);
}

// 1/x for a positive normal x: the hardware's approximate reciprocal and two Newton steps (each
// doubling the correct bits), within about one unit in the last place of the correctly rounded
// quotient; five FP64 operations where a division takes about ten.
__device__ __forceinline__ double rcp_nr(double x) {
  double r;
#ifdef __CUDA_ARCH__
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
#else
  r = 1.0 / x;
#endif
  double e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  e = fma(-x, r, 1.0);
  return fma(r, e, r);
}

// pmod, src/stdinclude.cpp:88-93.
__device__ __forceinline__ double pmod_d(double a, double b) {
  if (a >= 0.0 && a < b) return a;  // fmod is exact and returns a here
  double x = fmod(a, b);
  x += (x < 0.0) ? b : 0.0;
  return x;
}

}  // namespace mithra
