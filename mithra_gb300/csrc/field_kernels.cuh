// Field kernels: the leapfrog potential update with Mur absorbing boundaries and the E/B
// evaluation, for one rank that owns the whole z range.
//
// Dependency order inside one FdTd::fieldUpdate (src/fdtd.cpp:231-725): interior nodes
// (J/rho read in place from anp1/fnp1), then the six faces (which read interior anp1), then
// the twelve edges (which read face anp1), then the eight corners (which read edge anp1).
// Each stage is one launch; within a stage every node is independent.
#pragma once
#include "device_common.cuh"

namespace mithra {

// Coefficients in the arithmetic type of the kernel, converted once on the host.
template <typename T>
struct Coeffs {
  T a0, a1, a2, a3, al, be;
  T bB[5], cB[5], dB[5], eE[5], fE[5], gE[5], hC[17];
};

template <typename T>
Coeffs<T> make_coeffs(const GridDev& g) {
  Coeffs<T> c;
  c.a0 = (T)g.a[0]; c.a1 = (T)g.a[1]; c.a2 = (T)g.a[2]; c.a3 = (T)g.a[3];
  c.al = (T)g.nsfd_alpha; c.be = (T)g.nsfd_beta;
  for (int i = 0; i < 5; i++) {
    c.bB[i] = (T)g.bB[i]; c.cB[i] = (T)g.cB[i]; c.dB[i] = (T)g.dB[i];
    c.eE[i] = (T)g.eE[i]; c.fE[i] = (T)g.fE[i]; c.gE[i] = (T)g.gE[i];
  }
  for (int i = 0; i < 17; i++) c.hC[i] = (T)g.hC[i];
  return c;
}

template <typename T>
struct PotentialArgs {
  T* np1;        // anp1 (holds J on entry) or fnp1 (holds rho)
  const T* n;    // an / fn
  const T* nm1;  // anm1 / fnm1
  int ncomp;     // 3 for A, 1 for phi
  T asrc;        // a[4] for J, a[5] for rho
  Coeffs<T> k;
  // FP64 vector potential: when st->j_edges is set, the source is the edge-form current of the
  // deposit, J_c(node) = Je_c(node) + Je_c(node - unit step along c), instead of np1.
  const T* jedge = nullptr;
  StateDev* st = nullptr;
  // The y faces (j = 0 and N1-1) were updated by the interior kernel already (the mixed form's
  // bulk-tensor stencil, when no seed is injected): the face kernel leaves them out.
  int yfaces_done = 0;
};

// Interior update, AdvanceField::advanceMagneticPotentialFD/NSFD and the scalar variants
// (src/database.cpp:44-134) called from src/fdtd.cpp:270-303.  One thread per node, looping
// over the components; FP64 FMAs are allowed (the result agrees with the reference to a few
// ulp per step).
template <typename T, bool NSFD>
__global__ void __launch_bounds__(256) k_potential_interior(GridDev g, PotentialArgs<T> p) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int i = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  if (j > g.N1 - 2 || i > g.N0 - 2) return;
  const long long m = node_index(g, k, i, j);
  const long long sI = g.P1, sK = g.plane;
  const T a0 = p.k.a0, a1 = p.k.a1, a2 = p.k.a2, a3 = p.k.a3, as = p.asrc;
  const bool edges = p.jedge != nullptr && p.st->j_edges;
  for (int c = 0; c < p.ncomp; c++) {
    const T* an = p.n + c * g.cstride;
    const T* am = p.nm1 + c * g.cstride;
    T* ap = p.np1 + c * g.cstride;
    T src;
    if (edges) {
      const T* je = p.jedge + c * g.cstride;
      src = je[m] + je[m - (c == 0 ? sI : c == 1 ? 1 : sK)];
    } else {
      src = ap[m];
    }
    T v;
    if (NSFD) {
      const T al = p.k.al, be = p.k.be;
      T sx = an[m + sI] + an[m - sI] + be * (an[m + sI + sK] + an[m + sI - sK] + an[m - sI + sK] + an[m - sI - sK]);
      T sy = an[m + 1] + an[m - 1] + be * (an[m + 1 + sK] + an[m + 1 - sK] + an[m - 1 + sK] + an[m - 1 - sK]);
      v = a0 * an[m] - am[m] + al * (a1 * sx + a2 * sy) + a3 * (an[m + sK] + an[m - sK]) + as * src;
    } else {
      v = a0 * an[m] - am[m] + a1 * (an[m + sI] + an[m - sI]) + a2 * (an[m + 1] + an[m - 1]) +
          a3 * (an[m + sK] + an[m - sK]) + as * src;
    }
    ap[m] = v;
  }
}

// Mur faces, AdvanceField::advanceBoundaryF/S (src/database.cpp:137-176) with the argument
// pattern of src/fdtd.cpp:377-472: `in` points into the domain, o1/o2 along the face.
template <typename T>
__device__ __forceinline__ T face_value(const T* B, const T* np1, const T* n, const T* nm1,
                                        long long m, long long in, long long o1, long long o2) {
  return B[0] * (nm1[m] + np1[m + in]) + B[1] * nm1[m + in] + B[2] * (n[m] + n[m + in]) +
         B[3] * (n[m + in + o1] + n[m + in - o1] + n[m + o1] + n[m - o1]) +
         B[4] * (n[m + in + o2] + n[m + in - o2] + n[m + o2] + n[m - o2]);
}

template <typename T>
__global__ void __launch_bounds__(256) k_potential_faces(GridDev g, PotentialArgs<T> p) {
  const long long nx = (long long)(g.N1 - 2) * (g.N2 - 2);
  const long long ny = p.yfaces_done ? 0 : (long long)(g.N0 - 2) * (g.N2 - 2);
  const long long nz = (long long)(g.N0 - 2) * (g.N1 - 2);
  const long long total = 2 * (nx + ny + nz);
  const long long sI = g.P1, sK = g.plane;
  // The interior update has consumed the edge-form current: A^{n+1} now fills np1.
  if (p.st && blockIdx.x == 0 && threadIdx.x == 0) p.st->j_edges = 0;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    long long m, in, o1, o2;
    const T* B;
    long long u = t;
    if (u < 2 * nx) {  // x faces: j in [1,N1-2], k in [1,N2-2]
      int side = u >= nx; u -= side * nx;
      int j = 1 + (int)(u % (g.N1 - 2)), k = 1 + (int)(u / (g.N1 - 2));
      m = node_index(g, k, side ? g.N0 - 1 : 0, j);
      in = side ? -sI : sI; o1 = 1; o2 = sK; B = p.k.bB;
    } else if ((u -= 2 * nx) < 2 * ny) {  // y faces: i in [1,N0-2], k in [1,N2-2]
      int side = u >= ny; u -= side * ny;
      int i = 1 + (int)(u % (g.N0 - 2)), k = 1 + (int)(u / (g.N0 - 2));
      m = node_index(g, k, i, side ? g.N1 - 1 : 0);
      in = side ? -1 : 1; o1 = sI; o2 = sK; B = p.k.cB;
    } else {  // z faces: i in [1,N0-2], j in [1,N1-2]
      u -= 2 * ny;
      int side = u >= nz; u -= side * nz;
      int j = 1 + (int)(u % (g.N1 - 2)), i = 1 + (int)(u / (g.N1 - 2));
      m = node_index(g, side ? g.N2 - 1 : 0, i, j);
      in = side ? -sK : sK; o1 = sI; o2 = 1; B = p.k.dB;
    }
    for (int c = 0; c < p.ncomp; c++) {
      const long long off = c * g.cstride;
      p.np1[off + m] = face_value<T>(B, p.np1 + off, p.n + off, p.nm1 + off, m, in, o1, o2);
    }
  }
}

// Mur edges, AdvanceField::advanceEdgeF/S (src/database.cpp:179-229) with the argument
// pattern of src/fdtd.cpp:480-645: a, b point into the domain, t runs along the edge.
template <typename T>
__device__ __forceinline__ T edge_value(const T* E, const T* np1, const T* n, const T* nm1,
                                        long long m, long long a, long long b, long long t) {
  return E[0] * (np1[m + a] + nm1[m + b]) + E[1] * (nm1[m + a] + np1[m + b]) +
         E[2] * (nm1[m] + np1[m + a + b]) + E[3] * (n[m] + n[m + a] + n[m + b] + n[m + a + b]) +
         E[4] * (n[m - t] + n[m + a - t] + n[m + b - t] + n[m + a + b - t] + n[m + t] + n[m + a + t] +
                 n[m + b + t] + n[m + a + b + t]) -
         nm1[m + a + b];
}

template <typename T>
__global__ void __launch_bounds__(256) k_potential_edges(GridDev g, PotentialArgs<T> p) {
  const long long ez = g.N2 - 2, ex = g.N0 - 2, ey = g.N1 - 2;
  const long long total = 4 * (ez + ex + ey);
  const long long sI = g.P1, sK = g.plane;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    long long u = t, m, a, b, tt;
    const T* E;
    if (u < 4 * ez) {  // edges along z (eE), src/fdtd.cpp:480-522
      int which = (int)(u / ez); int k = 1 + (int)(u % ez);
      int hi_i = which & 1, hi_j = which >> 1;
      m = node_index(g, k, hi_i ? g.N0 - 1 : 0, hi_j ? g.N1 - 1 : 0);
      a = hi_i ? -sI : sI; b = hi_j ? -1 : 1; tt = sK; E = p.k.eE;
    } else if ((u -= 4 * ez) < 4 * ex) {  // edges along x (fE), src/fdtd.cpp:527-579
      int which = (int)(u / ex); int i = 1 + (int)(u % ex);
      int hi_j = which & 1, hi_k = which >> 1;
      m = node_index(g, hi_k ? g.N2 - 1 : 0, i, hi_j ? g.N1 - 1 : 0);
      a = hi_j ? -1 : 1; b = hi_k ? -sK : sK; tt = sI; E = p.k.fE;
    } else {  // edges along y (gE), src/fdtd.cpp:584-645
      u -= 4 * ex;
      int which = (int)(u / ey); int j = 1 + (int)(u % ey);
      int hi_i = which & 1, hi_k = which >> 1;
      m = node_index(g, hi_k ? g.N2 - 1 : 0, hi_i ? g.N0 - 1 : 0, j);
      a = hi_k ? -sK : sK; b = hi_i ? -sI : sI; tt = 1; E = p.k.gE;
    }
    for (int c = 0; c < p.ncomp; c++) {
      const long long off = c * g.cstride;
      p.np1[off + m] = edge_value<T>(E, p.np1 + off, p.n + off, p.nm1 + off, m, a, b, tt);
    }
  }
}

// Mur corners, AdvanceField::advanceCornerF/S (src/database.cpp:232-288), src/fdtd.cpp:647-725.
template <typename T>
__global__ void k_potential_corners(GridDev g, PotentialArgs<T> p) {
  const int t = threadIdx.x;
  if (t >= 8 * p.ncomp) return;
  const int c = t / 8, w = t % 8;
  const int hi_i = w & 1, hi_j = (w >> 1) & 1, hi_k = w >> 2;
  const long long off = c * g.cstride;
  const T* np1 = p.np1 + off;
  const T* n = p.n + off;
  const T* nm1 = p.nm1 + off;
  const long long m = node_index(g, hi_k ? g.N2 - 1 : 0, hi_i ? g.N0 - 1 : 0, hi_j ? g.N1 - 1 : 0);
  const long long a = hi_i ? -(long long)g.P1 : g.P1, b = hi_j ? -1 : 1, cc = hi_k ? -g.plane : g.plane;
  const T* h = p.k.hC;
  const long long P1 = m + a, P2 = m + b, P3 = m + cc, P4 = m + a + b, P5 = m + cc + a, P6 = m + cc + b,
                  P7 = m + a + b + cc;
  T s = n[m] * h[16] + nm1[m] * h[8] + np1[P1] * h[1] + n[P1] * h[16] + nm1[P1] * h[9] +
        np1[P2] * h[2] + n[P2] * h[16] + nm1[P2] * h[10] + np1[P3] * h[3] + n[P3] * h[16] +
        nm1[P3] * h[11] + np1[P4] * h[4] + n[P4] * h[16] + nm1[P4] * h[12] + np1[P5] * h[5] +
        n[P5] * h[16] + nm1[P5] * h[13] + np1[P6] * h[6] + n[P6] * h[16] + nm1[P6] * h[14] +
        np1[P7] * h[7] + n[P7] * h[16] + nm1[P7] * h[15];
  p.np1[off + m] = -s / h[0];
}

// E and B at every interior node, the eager form of FdTd::fieldEvaluate (src/fdtd.cpp:818-845;
// with space charge src/fdtdSC.cpp:1110-1140), plus the copies into planes k = 0 and N2-1
// (src/fdtd.cpp:755-772).  E is rounded to float twice as FieldVector<float>::dv and ::mdv do
// (src/fieldvector.h:87-107); B once.
template <typename T>
struct EBArgs {
  const T* anp1;
  const T* an;
  const T* fn;   // scalar potential phi^n, or nullptr without space charge
  T* E;          // 3 components, cstride apart; values are float-rounded
  T* B;
  const StateDev* st;          // slab of particle cells, or nullptr for every plane
  const uint8_t* plane_needed; // N2 flags: planes a power sample reads, or nullptr
  double rmdt, rdx2, rdy2, rdz2;  // -1/dt and 1/(2 d) per axis
};


// The evaluation marches along z: a block owns a 32 x 8 (j, i) tile and a run of `ks` planes.  The
// curl reads S = A^n + A^{n+1} of each component at the node's neighbours, where every value is read
// by four neighbouring nodes; each S is formed once per plane (with a one-node halo in i and j)
// into a ring of three planes in shared memory, with a third fewer FP64 operations than forming it
// at every use (the FP64 form is bound by the FP64 pipe).  Planes outside the particle slab and the
// power planes are skipped, and a run of wanted planes starts by forming S of its first plane's
// two neighbours.
constexpr int EBZ_TJ = 32, EBZ_TI = 8, EBZ_W = EBZ_TJ + 2, EBZ_H = EBZ_TI + 2;

template <typename T>
__global__ void __launch_bounds__(EBZ_TJ * EBZ_TI) k_eval_eb_z(GridDev g, EBArgs<T> p, int ks) {
  __shared__ double sS[3][3][EBZ_H][EBZ_W];  // ring slot (plane % 3), component, local i, local j
  const int tx = threadIdx.x % EBZ_TJ, ty = threadIdx.x / EBZ_TJ;
  const int i0 = blockIdx.y * EBZ_TI, j0 = blockIdx.x * EBZ_TJ;  // halo origin: node (i0, j0)
  const int i = i0 + 1 + ty, j = j0 + 1 + tx;                    // this thread's node
  const bool in = i <= g.N0 - 2 && j <= g.N1 - 2;
  const int kb = 1 + (int)blockIdx.z * ks, ke = min(g.N2 - 2, kb + ks - 1);
  const long long cs = g.cstride, sI = g.P1, sK = g.plane;
  const T *A1 = p.anp1, *A0 = p.an;
  const double rmdt = p.rmdt, rdx2 = p.rdx2, rdy2 = p.rdy2, rdz2 = p.rdz2;
  const double hx = 0.5 * rdx2, hy = 0.5 * rdy2, hz = 0.5 * rdz2;
  auto fill = [&](int k) {  // S of plane k over the tile and its halo
    const int slot = k % 3;
    for (int t = threadIdx.x; t < EBZ_H * EBZ_W; t += EBZ_TJ * EBZ_TI) {
      const int li = t / EBZ_W, lj = t % EBZ_W;
      const int gi = i0 + li, gj = j0 + lj;
      if (gi < g.N0 && gj < g.N1) {
        const long long m = node_index(g, k, gi, gj);
#pragma unroll
        for (int c = 0; c < 3; c++) sS[slot][c][li][lj] = (double)A0[c * cs + m] + A1[c * cs + m];
      }
    }
  };
  int filled = -2;  // highest plane whose S is in the ring, with the two below it
  for (int k = kb; k <= ke; k++) {
    if (!eb_plane_wanted(k, p.st, p.plane_needed, g.N2)) continue;  // uniform across the block
    if (filled != k) {  // a new run: S of planes k-1 and k
      __syncthreads();
      fill(k - 1);
      fill(k);
    } else {
      __syncthreads();  // every thread is done with plane k-2, whose slot plane k+1 takes
    }
    fill(k + 1);
    filled = k + 1;
    __syncthreads();
    if (!in) continue;
    const long long m = node_index(g, k, i, j);
    float e[3], b[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      float ef = to_float_rn((double)A1[c * cs + m] * rmdt);
      ef = to_float_rn(to_double(ef) - (double)A0[c * cs + m] * rmdt);
      e[c] = ef;
    }
    if (p.fn) {
      e[0] = to_float_rn(to_double(e[0]) - ((double)p.fn[m + sI] - (double)p.fn[m - sI]) * rdx2);
      e[1] = to_float_rn(to_double(e[1]) - ((double)p.fn[m + 1] - (double)p.fn[m - 1]) * rdy2);
      e[2] = to_float_rn(to_double(e[2]) - ((double)p.fn[m + sK] - (double)p.fn[m - sK]) * rdz2);
    }
    const int sc = k % 3, sm = (k + 2) % 3, sp = (k + 1) % 3;
    const int li = ty + 1, lj = tx + 1;
    const double bx = (sS[sc][2][li][lj + 1] - sS[sc][2][li][lj - 1]) * hy - (sS[sp][1][li][lj] - sS[sm][1][li][lj]) * hz;
    const double by = (sS[sp][0][li][lj] - sS[sm][0][li][lj]) * hz - (sS[sc][2][li + 1][lj] - sS[sc][2][li - 1][lj]) * hx;
    const double bz = (sS[sc][1][li + 1][lj] - sS[sc][1][li - 1][lj]) * hx - (sS[sc][0][li][lj + 1] - sS[sc][0][li][lj - 1]) * hy;
    b[0] = to_float_rn(bx); b[1] = to_float_rn(by); b[2] = to_float_rn(bz);
    T eo[3], bo[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      eo[c] = (T)to_double(e[c]);
      bo[c] = (T)to_double(b[c]);
      p.E[c * cs + m] = eo[c];
      p.B[c * cs + m] = bo[c];
    }
    if (k == 1) {
#pragma unroll
      for (int c = 0; c < 3; c++) { p.E[c * cs + m - sK] = eo[c]; p.B[c * cs + m - sK] = bo[c]; }
    }
    if (k == g.N2 - 2) {
#pragma unroll
      for (int c = 0; c < 3; c++) { p.E[c * cs + m + sK] = eo[c]; p.B[c * cs + m + sK] = bo[c]; }
    }
  }
}

// Layout conversion between the reference's AoS records (m = N1N0*k + N1*i + j, `ncomp`
// values per node) and the padded SoA device layout.
template <typename Tdev, typename Thost>
__global__ void k_aos_to_soa(GridDev g, const Thost* __restrict__ src, Tdev* __restrict__ dst, int ncomp) {
  const long long total = (long long)g.N0 * g.N1 * g.N2;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < total;
       r += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(r % g.N1);
    const long long ki = r / g.N1;
    const int i = (int)(ki % g.N0), k = (int)(ki / g.N0);
    const long long m = node_index(g, k, i, j);
    for (int c = 0; c < ncomp; c++) dst[c * g.cstride + m] = (Tdev)src[r * ncomp + c];
  }
}

// E or B (off = 0 or 4) of every node as records of 3 floats in the reference's node order
// (mithra_gpu_download_eb).
static __global__ void k_eb_to_aos(GridDev g, const float* __restrict__ EB, int off, float* __restrict__ dst) {
  const long long total = (long long)g.N0 * g.N1 * g.N2;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < total;
       r += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(r % g.N1);
    const long long ki = r / g.N1;
    const int i = (int)(ki % g.N0), k = (int)(ki / g.N0);
    const float* src = EB + (long long)kEBNode * node_index(g, k, i, j) + off;
    for (int c = 0; c < 3; c++) dst[r * 3 + c] = src[c];
  }
}

template <typename Tdev, typename Thost>
__global__ void k_soa_to_aos(GridDev g, const Tdev* __restrict__ src, Thost* __restrict__ dst, int ncomp) {
  const long long total = (long long)g.N0 * g.N1 * g.N2;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < total;
       r += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(r % g.N1);
    const long long ki = r / g.N1;
    const int i = (int)(ki % g.N0), k = (int)(ki / g.N0);
    const long long m = node_index(g, k, i, j);
    for (int c = 0; c < ncomp; c++) dst[r * ncomp + c] = (Thost)src[c * g.cstride + m];
  }
}

}  // namespace mithra

namespace mithra {

// Node values of an edge-form current (the inverse view of k_deposit_fp64's layout):
// J_c(node) = Je_c(node) + Je_c(node - unit step along c), the second term only where that
// neighbour exists.
static __global__ void __launch_bounds__(256) k_materialize_j(GridDev g, const double* __restrict__ je, double* __restrict__ J) {
  const long long nodes = (long long)g.N0 * g.N1 * g.N2;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < 3 * nodes;
       t += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(t / nodes);
    long long r = t % nodes;
    const int j = (int)(r % g.N1); r /= g.N1;
    const int i = (int)(r % g.N0);
    const int k = (int)(r / g.N0);
    const long long m = node_index(g, k, i, j);
    const double* e = je + c * g.cstride;
    double v = e[m];
    if (c == 0 && i > 0) v += e[m - g.P1];
    if (c == 1 && j > 0) v += e[m - 1];
    if (c == 2 && k > 0) v += e[m - g.plane];
    J[c * g.cstride + m] = v;
  }
}

}  // namespace mithra
