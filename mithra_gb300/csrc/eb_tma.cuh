// E/B evaluation of the mixed form with TMA-staged z-slabs (FdTd::fieldEvaluate,
// src/fdtd.cpp:818-845, evaluated eagerly on the planes the particles occupy).
//
// Each CTA owns a TMA_TJ x TMA_TI (j, i) tile and marches along k over a slab of planes.  E needs
// A^n and A^{n+1} at the node; B = curl(A^n + A^{n+1}) / (2 d) needs all three components with a
// one-node halo in i and j and the neighbouring planes k-1, k+1.  Every plane of the six arrays
// (three components of A^n and of A^{n+1}, boxes of the interior stencil's A^n tensor map: the
// tile plus its halo) is brought into shared memory once by cp.async.bulk.tensor, in a ring of
// EB_R plane slots kept EB_D planes ahead of the plane computed, so A is read from HBM once per
// slab (plus the thin halos) and E, B are written as the node records of the mixed form (two
// 16-byte stores per node, 32 bytes of which 24 carry E and B).
//
// Waits are bounded, as in the interior stencil: a CTA whose barrier does not complete records
// the failure in the error word, waits (with the default limit) for the copy groups it issued
// and has not seen complete, and leaves.
#pragma once
#include "tma_stencil.cuh"

namespace mithra {

constexpr int EB_D = 2;                         // planes in flight ahead of plane k+1
constexpr int EB_R = EB_D + 3;                  // ring: k-1, k, k+1 in use plus EB_D ahead
constexpr int EB_BOX = TMA_BW * TMA_BH * 4;     // bytes of one component box (the A^n box)
constexpr int EB_BOX_SLOT = ((EB_BOX + 127) / 128) * 128;
constexpr int EB_PLANE = 6 * EB_BOX_SLOT;       // X, Y, Z of A^n then of A^{n+1}
constexpr size_t kEbTmaSmem = (size_t)EB_R * EB_PLANE + 128;

struct EbTmaArgs {
  float* EB;  // node records {E, 0, B, 0} (store_eb)
  int N0, N1, N2, P1;
  long long plane;
  float rdt, hx, hy, hz;
  int ks;                 // planes per slab
  const StateDev* st;     // particle slab (k_lo, k_hi); null: every plane
  unsigned spin_limit;
  int* error;
};

__global__ void __launch_bounds__(TMA_TJ * TMA_TI) k_eval_eb_tma(const __grid_constant__ CUtensorMap map_a0,  // A^n
                                                                 const __grid_constant__ CUtensorMap map_a1,  // A^{n+1}
                                                                 EbTmaArgs a) {
  extern __shared__ __align__(128) unsigned char s_raw[];
  unsigned char* s_base = s_raw + ((128u - (smem_addr(s_raw) & 127u)) & 127u);
  // slot r, array q (0..2: A^n x, y, z; 3..5: A^{n+1} x, y, z)
  auto box = [&](int r, int q) {
    return reinterpret_cast<float(*)[TMA_BW]>(s_base + (size_t)r * EB_PLANE + (size_t)q * EB_BOX_SLOT);
  };
  __shared__ __align__(8) unsigned long long bar[EB_R];
  __shared__ int s_abort;

  const int tx = threadIdx.x % TMA_TJ, ty = threadIdx.x / TMA_TJ;
  const int nslab = (a.N2 - 2 + a.ks - 1) / a.ks;
  const int jb = blockIdx.x * TMA_TJ, ib = blockIdx.y * TMA_TI;  // box origin (= first node - 1)
  int k_first = 1 + (int)blockIdx.z * a.ks;
  int k_last = min(a.N2 - 2, k_first + a.ks - 1);
  if (blockIdx.z >= (unsigned)nslab) return;
  if (a.st) {  // the planes the particles occupy (the reference evaluates lazily near particles)
    k_first = max(k_first, a.st->k_lo - 2);
    k_last = min(k_last, a.st->k_hi + 3);
  }
  if (k_first > k_last) return;
  const int j = jb + 1 + tx, i = ib + 1 + ty;
  const int p0 = k_first - 1;  // first plane loaded
  const int p_end = k_last + 1;  // last plane needed
  // plane p lives in slot p % EB_R and completes the ((p - p0) / EB_R)-th phase of bar[p % EB_R]
  auto parity = [&](int p) { return (unsigned)(((p - p0) / EB_R) & 1); };
  auto issue = [&](int p) {
    unsigned long long* b = &bar[p % EB_R];
    mbar_expect_tx(b, 6u * EB_BOX);
    for (int c = 0; c < 3; c++) {
      tma_load_4d(&box(p % EB_R, c)[0][0], &map_a0, jb, ib, p, c, b);
      tma_load_4d(&box(p % EB_R, 3 + c)[0][0], &map_a1, jb, ib, p, c, b);
    }
  };
  int issued = p0 - 1, completed = p0 - 1;  // thread 0's record of the plane groups
  if (threadIdx.x == 0) {
    for (int b = 0; b < EB_R; b++) mbar_init(&bar[b], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_abort = 0;
    bool ok = true;  // every slot a copy may target is checked before any copy is issued
    for (int r = 0; r < EB_R; r++)
      for (int q = 0; q < 6; q++) ok = ok && ((smem_addr(&box(r, q)[0][0]) & 127u) == 0u);
    if (ok) {
      for (int p = p0; p <= min(p_end, p0 + EB_R - 1); p++) {
        issue(p);
        issued = p;
      }
    } else {
      atomicExch(a.error, 2);
      s_abort = 1;
    }
  }
  __syncthreads();
  if (s_abort) return;  // nothing was issued
  // planes p0 and p0 + 1 (= k_first - 1, k_first) before the first plane computed
  bool pro_ok = true;  // this thread saw planes p0 and p0 + 1 land
  for (int p = p0; p <= p0 + 1; p++) {
    if (!mbar_wait(&bar[p % EB_R], parity(p), a.spin_limit)) {
      s_abort = 1;
      pro_ok = false;
    } else if (threadIdx.x == 0 && completed == p - 1) {
      completed = p;  // contiguous only
    }
  }
  const float rdt = a.rdt, hx = a.hx, hy = a.hy, hz = a.hz;
  const bool in = i <= a.N0 - 2 && j <= a.N1 - 2;
  const int y = ty + 1, x = tx + 1;  // the node in the boxes
  for (int k = k_first; k <= k_last; k++) {
    // No barrier after the wait: a thread whose wait gives up skips the plane, and the abort is
    // seen by all after the end-of-plane barrier.
    const bool ok = mbar_wait(&bar[(k + 1) % EB_R], parity(k + 1), a.spin_limit);
    if (!ok)
      s_abort = 1;
    else if (threadIdx.x == 0 && completed == k)
      completed = k + 1;
    if (ok && pro_ok && in) {
      const int rc = k % EB_R, rm = (k - 1) % EB_R, rp = (k + 1) % EB_R;
      const float(*X0)[TMA_BW] = box(rc, 0);
      const float(*Y0)[TMA_BW] = box(rc, 1);
      const float(*Z0)[TMA_BW] = box(rc, 2);
      const float(*X1)[TMA_BW] = box(rc, 3);
      const float(*Y1)[TMA_BW] = box(rc, 4);
      const float(*Z1)[TMA_BW] = box(rc, 5);
      // the arithmetic of k_eval_eb_f32, term for term
      const float e0 = (X0[y][x] - X1[y][x]) * rdt;
      const float e1 = (Y0[y][x] - Y1[y][x]) * rdt;
      const float e2 = (Z0[y][x] - Z1[y][x]) * rdt;
      const float b0 = ((Z0[y][x + 1] + Z1[y][x + 1]) - (Z0[y][x - 1] + Z1[y][x - 1])) * hy -
                       ((box(rp, 1)[y][x] + box(rp, 4)[y][x]) - (box(rm, 1)[y][x] + box(rm, 4)[y][x])) * hz;
      const float b1 = ((box(rp, 0)[y][x] + box(rp, 3)[y][x]) - (box(rm, 0)[y][x] + box(rm, 3)[y][x])) * hz -
                       ((Z0[y + 1][x] + Z1[y + 1][x]) - (Z0[y - 1][x] + Z1[y - 1][x])) * hx;
      const float b2 = ((Y0[y + 1][x] + Y1[y + 1][x]) - (Y0[y - 1][x] + Y1[y - 1][x])) * hx -
                       ((X0[y][x + 1] + X1[y][x + 1]) - (X0[y][x - 1] + X1[y][x - 1])) * hy;
      const long long m = (long long)k * a.plane + (long long)i * a.P1 + j;
      store_eb(a.EB, m, e0, e1, e2, b0, b1, b2);
      if (k == 1) store_eb(a.EB, m - a.plane, e0, e1, e2, b0, b1, b2);  // plane 0 copies plane 1 (src/fdtd.cpp:755-772)
      if (k == a.N2 - 2) store_eb(a.EB, m + a.plane, e0, e1, e2, b0, b1, b2);
    }
    __syncthreads();  // slot of plane k-1 free: the next group may overwrite it
    if (s_abort) break;
    if (threadIdx.x == 0 && k + 1 + EB_D + 1 <= p_end) {
      issue(k + EB_D + 2);  // slot (k + EB_D + 2) % EB_R = (k - 1) % EB_R
      issued = k + EB_D + 2;
    }
  }
  if (s_abort) {
    if (threadIdx.x == 0) {
      atomicExch(a.error, 1);
      for (int p = completed + 1; p <= issued; p++) mbar_wait(&bar[p % EB_R], parity(p), TMA_SPIN_LIMIT);
    }
    __syncthreads();
  }
}

}  // namespace mithra
