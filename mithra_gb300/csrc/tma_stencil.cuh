// Interior potential update of the mixed form with TMA-staged z-slabs.
//
// Each CTA owns a TJ x TI tile of (j, i) for one component and marches along k over a slab of
// KS planes.  Planes of A^n (with a one-node halo), A^{n-1} and J are brought into shared memory
// by cp.async.bulk.tensor under mbarriers: a ring of six A^n planes (k-1, k, k+1 in use, three
// ahead in flight) and four of A^{n-1} and J.  One thread per tile column computes A^{n+1} for the plane
// from shared memory (FD: 7 points; NSFD: the 15-point stencil of src/database.cpp:44-72) and
// stores it with coalesced row writes.  Every byte of A^n, A^{n-1}, J is read from HBM once per
// slab (plus the thin halos), which is what the 48 B/node roofline assumes.
//
// Waits are bounded: a CTA whose barrier does not complete within the iteration limit records
// the failure in an error word and leaves after a bounded drain, instead of spinning forever.
// The drain waits, with the default limit, for every copy group the CTA issued and has not seen
// complete, so no bulk copy is still landing in shared memory when the CTA exits.
#pragma once
#include <cuda.h>

#include "device_common.cuh"

namespace mithra {

constexpr int TMA_TJ = 32;               // tile width along j (threads along x)
constexpr int TMA_TI = 16;               // tile height along i
constexpr int TMA_BW = TMA_TJ + 4;       // box width: j0-1 .. j0+TJ, rounded up to 16 bytes
constexpr int TMA_BH = TMA_TI + 2;       // A^n box height incl. halo rows
constexpr int TMA_KS = 64;               // default planes per slab (TmaStencilArgs::ks)
constexpr unsigned TMA_SPIN_LIMIT = 20000000u;

struct TmaStencilArgs {
  float* np1;        // A^{n+1} (holds J on entry), SoA with cstride between components
  int N0, N1, N2, P1;
  long long plane, cstride;
  float a0, a1, a2, a3, asrc, al, be;
  int ks;            // planes per slab (the z extent of a CTA's tile)
  int yfaces;        // also the Mur faces j = 0 and N1-1 (AdvanceField::advanceBoundaryF with the
                     // face pattern of src/fdtd.cpp:377-472): only when nothing changes A^{n+1} at
                     // j = 1 or N1-2 between the interior update and the faces (no seed injection)
  float cB[5];       // the y-face coefficients
  unsigned spin_limit;  // iterations of one barrier wait before it gives up (TMA_SPIN_LIMIT)
  int* error;        // set to 1 when a barrier wait gives up, 2 for an unaligned slot
};

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

// Bounded wait on phase `parity`; returns false when the limit is reached.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, unsigned limit) {
  for (unsigned it = 0; it < limit; it++) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// 4D tiled load (x = j, y = i, z = k, w = component) into shared memory, completing on `bar`.
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int x, int y, int z, int w,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];"
      ::"r"(smem_addr(dst)), "l"(map), "r"(x), "r"(y), "r"(z), "r"(w), "r"(smem_addr(bar))
      : "memory");
}

constexpr int TMA_D = 3;                    // plane groups in flight ahead of the one computed
constexpr int TMA_RAN = TMA_D + 3;          // A^n ring: k-1, k, k+1 in use plus D ahead
constexpr int TMA_RC = TMA_D + 1;           // A^{n-1} / J ring and barriers
// Shared-memory slots of bulk-tensor copies start on 128-byte boundaries: slot strides are
// rounded up to multiples of 128 bytes and the dynamic base is aligned at run time.
constexpr int TMA_SLOT_AN = ((TMA_BW * TMA_BH * 4 + 127) / 128) * 128;   // bytes per A^n slot
constexpr int TMA_SLOT_C = ((TMA_BW * TMA_TI * 4 + 127) / 128) * 128;    // bytes per A^{n-1}/J slot
constexpr int TMA_OFF_AM = TMA_RAN * TMA_SLOT_AN;
constexpr int TMA_OFF_J = TMA_OFF_AM + TMA_RC * TMA_SLOT_C;
constexpr int TMA_SMEM_USED = TMA_OFF_J + TMA_RC * TMA_SLOT_C;

template <bool NSFD>
__global__ void __launch_bounds__(TMA_TJ * TMA_TI, 4) k_potential_interior_tma(
    const __grid_constant__ CUtensorMap map_an,    // A^n, box TMA_BW x TMA_BH
    const __grid_constant__ CUtensorMap map_anm1,  // A^{n-1}, box TMA_BW x TMA_TI
    const __grid_constant__ CUtensorMap map_j,     // J (the A^{n+1} buffer), box TMA_BW x TMA_TI
    TmaStencilArgs a) {
  extern __shared__ __align__(128) unsigned char s_raw[];
  unsigned char* s_base = s_raw + ((128u - (smem_addr(s_raw) & 127u)) & 127u);
  auto an_slot = [&](int r) { return reinterpret_cast<float(*)[TMA_BW]>(s_base + r * TMA_SLOT_AN); };
  auto am_slot = [&](int r) { return reinterpret_cast<float(*)[TMA_BW]>(s_base + TMA_OFF_AM + r * TMA_SLOT_C); };
  auto j_slot = [&](int r) { return reinterpret_cast<float(*)[TMA_BW]>(s_base + TMA_OFF_J + r * TMA_SLOT_C); };
  __shared__ __align__(8) unsigned long long bar[TMA_RC + 1];  // one per group slot; last: prologue
  __shared__ int s_abort;
  __shared__ float s_face[2][TMA_TI];

  const int tx = threadIdx.x % TMA_TJ, ty = threadIdx.x / TMA_TJ;
  const int nslab = (a.N2 - 2 + a.ks - 1) / a.ks;
  const int comp = blockIdx.z / nslab, slab = blockIdx.z % nslab;
  const int jb = blockIdx.x * TMA_TJ;   // box origin along j (= j0 - 1, 16-byte aligned)
  const int ib = blockIdx.y * TMA_TI;   // A^n box origin along i (= i0 - 1)
  const int k_first = 1 + slab * a.ks;
  const int k_last = min(a.N2 - 2, k_first + a.ks - 1);
  const int j = jb + 1 + tx, i = ib + 1 + ty;
  const bool last_cta = (int)blockIdx.x == (a.N1 - 3) / TMA_TJ;  // holds j = N1 - 2
  const bool face_cta = a.yfaces && (jb == 0 || last_cta);
  const unsigned bytes_an = TMA_BW * TMA_BH * 4, bytes_c = TMA_BW * TMA_TI * 4;

  // The parity of the wait for plane kk's group on its barrier kk % RC: the planes of a slab use
  // the barriers in turn, so barrier g completes its n-th phase for the n-th plane that maps to it.
  auto group_parity = [&](int kk) { return (unsigned)(((kk - k_first) / TMA_RC) & 1); };
  auto aligned = [&](const void* d) { return (smem_addr(d) & 127u) == 0u; };
  auto issue_group = [&](int kk) {  // A^n(kk+1), A^{n-1}(kk), J(kk) on barrier kk % RC
    unsigned long long* b = &bar[kk % TMA_RC];
    mbar_expect_tx(b, bytes_an + 2 * bytes_c);
    tma_load_4d(&an_slot((kk + 1) % TMA_RAN)[0][0], &map_an, jb, ib, kk + 1, comp, b);
    tma_load_4d(&am_slot(kk % TMA_RC)[0][0], &map_anm1, jb, ib + 1, kk, comp, b);
    tma_load_4d(&j_slot(kk % TMA_RC)[0][0], &map_j, jb, ib + 1, kk, comp, b);
  };

  // Thread 0's record of the copy groups: the last plane whose group it issued and the last one
  // whose wait it saw complete (the drain waits for the groups in between).
  int issued = k_first - 1, completed = k_first - 1;
  if (threadIdx.x == 0) {
    for (int b = 0; b <= TMA_RC; b++) mbar_init(&bar[b], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_abort = 0;
    // Every slot a copy may target is checked once, before any copy is issued: a copy only goes
    // to a 128-byte aligned slot, and an unaligned layout is recorded as an error with nothing
    // in flight.
    bool ok = true;
    for (int r = 0; r < TMA_RAN; r++) ok = ok && aligned(&an_slot(r)[0][0]);
    for (int r = 0; r < TMA_RC; r++) ok = ok && aligned(&am_slot(r)[0][0]) && aligned(&j_slot(r)[0][0]);
    if (ok) {
      mbar_expect_tx(&bar[TMA_RC], 2 * bytes_an);
      tma_load_4d(&an_slot((k_first - 1) % TMA_RAN)[0][0], &map_an, jb, ib, k_first - 1, comp, &bar[TMA_RC]);
      tma_load_4d(&an_slot(k_first % TMA_RAN)[0][0], &map_an, jb, ib, k_first, comp, &bar[TMA_RC]);
      for (int kk = k_first; kk < k_first + TMA_D && kk <= k_last; kk++) {
        issue_group(kk);
        issued = kk;
      }
    } else {
      atomicExch(a.error, 2);
      s_abort = 1;
    }
  }
  __syncthreads();
  if (s_abort) return;  // nothing was issued
  const bool prologue_done = mbar_wait(&bar[TMA_RC], 0, a.spin_limit);
  if (!prologue_done) s_abort = 1;

  float* out = a.np1 + (long long)comp * a.cstride;
  unsigned phases = 0u;  // bit b: parity of the next wait on bar[b] (flipped only by a completed wait)
  for (int k = k_first; k <= k_last; k++) {
    const int g = k % TMA_RC;
    if (threadIdx.x == 0 && k + TMA_D <= k_last && !s_abort) {  // reuses the slots of planes k-1, k-2
      issue_group(k + TMA_D);
      issued = k + TMA_D;
    }
    if (!mbar_wait(&bar[g], (phases >> g) & 1u, a.spin_limit)) {
      s_abort = 1;
    } else {
      phases ^= 1u << g;
      if (threadIdx.x == 0) completed = k;
    }
    __syncthreads();
    if (s_abort) break;
    if (i <= a.N0 - 2 && j <= a.N1 - 2) {
      const float(*c)[TMA_BW] = an_slot(k % TMA_RAN);
      const float(*m)[TMA_BW] = an_slot((k - 1) % TMA_RAN);
      const float(*p)[TMA_BW] = an_slot((k + 1) % TMA_RAN);
      const float(*am)[TMA_BW] = am_slot(g);
      const float(*jj)[TMA_BW] = j_slot(g);
      const int y = ty + 1, x = tx + 1;
      const float v = c[y][x];
      float r;
      if (NSFD) {
        const float sx = c[y + 1][x] + c[y - 1][x] + a.be * (p[y + 1][x] + m[y + 1][x] + p[y - 1][x] + m[y - 1][x]);
        const float sy = c[y][x + 1] + c[y][x - 1] + a.be * (p[y][x + 1] + m[y][x + 1] + p[y][x - 1] + m[y][x - 1]);
        r = a.a0 * v - am[ty][x] + a.al * (a.a1 * sx + a.a2 * sy) + a.a3 * (p[y][x] + m[y][x]) +
            a.asrc * jj[ty][x];
      } else {
        r = a.a0 * v - am[ty][x] + a.a1 * (c[y + 1][x] + c[y - 1][x]) + a.a2 * (c[y][x + 1] + c[y][x - 1]) +
            a.a3 * (p[y][x] + m[y][x]) + a.asrc * jj[ty][x];
      }
      const long long row = (long long)k * a.plane + (long long)i * a.P1;
      out[row + j] = r;
      if (j == 1) s_face[0][ty] = r;          // A^{n+1} next to the y faces, for the face update below
      if (j == a.N1 - 2) s_face[1][ty] = r;
    }
    if (face_cta) {
      // The y-face nodes of this tile's rows (j = 0 in the first tile column, j = N1-1 in the last),
      // one per lane of warps 0 and 1, from the planes still in shared memory: the terms of
      // face_value in its order, cB0 (nm1 face + np1 inner) + cB1 nm1 inner + cB2 (n face + n
      // inner) + cB3 (n inner and face at i +- 1) + cB4 (n inner and face at k +- 1).
      __syncthreads();
      const int side = threadIdx.x >> 5, l = threadIdx.x & 31;
      const int fi = ib + 1 + l;
      if (side < 2 && l < TMA_TI && fi <= a.N0 - 2 && ((side == 0 && jb == 0) || (side == 1 && last_cta))) {
        const int xi = side == 0 ? 1 : a.N1 - 2 - jb, f = side == 0 ? 0 : xi + 1, fy = l + 1;
        const float(*c)[TMA_BW] = an_slot(k % TMA_RAN);
        const float(*m)[TMA_BW] = an_slot((k - 1) % TMA_RAN);
        const float(*p)[TMA_BW] = an_slot((k + 1) % TMA_RAN);
        const float(*am)[TMA_BW] = am_slot(g);
        const float rr = s_face[side][l];
        const float v = a.cB[0] * (am[l][f] + rr) + a.cB[1] * am[l][xi] + a.cB[2] * (c[fy][f] + c[fy][xi]) +
                        a.cB[3] * (c[fy + 1][xi] + c[fy - 1][xi] + c[fy + 1][f] + c[fy - 1][f]) +
                        a.cB[4] * (p[fy][xi] + m[fy][xi] + p[fy][f] + m[fy][f]);
        out[(long long)k * a.plane + (long long)fi * a.P1 + (side == 0 ? 0 : a.N1 - 1)] = v;
      }
    }
    __syncthreads();
  }
  if (s_abort) {
    if (threadIdx.x == 0) {
      atomicExch(a.error, 1);
      // Bounded drain of the copies that may still be in flight into this CTA's shared memory:
      // the prologue's, and every group issued after the last completed wait (a phase that has
      // completed already passes at once).
      if (!prologue_done) mbar_wait(&bar[TMA_RC], 0, TMA_SPIN_LIMIT);
      for (int kk = completed + 1; kk <= issued; kk++) mbar_wait(&bar[kk % TMA_RC], group_parity(kk), TMA_SPIN_LIMIT);
    }
    __syncthreads();
  }
}

constexpr size_t kTmaStencilSmem = (size_t)TMA_SMEM_USED + 128;  // + room to align the base

}  // namespace mithra
