// Tile sort and tiled current deposit of the mixed form.
//
// Every third field step the particles are counting-sorted by deposit tile (TX x TY x TZ cells).  The
// deposit then gives one block to each tile: the block accumulates the zigzag currents of its
// particles in a shared-memory copy of the tile's nodes (with a one-cell halo on each side, since
// the previous position may lie in a neighbouring cell) and adds that copy to J once.  Compared
// with one global atomic per particle contribution (48 per particle) this removes most of the
// traffic to the L2 atomic units; the sort also makes the next push read E/B with locality.
#pragma once
#include "device_common.cuh"
#include "fp32_kernels.cuh"

namespace mithra {

constexpr int TX = 8, TY = 8, TZ = 8;                          // cells per tile (i, j, k)
constexpr int HX = TX + 3, HZ = TZ + 3;                        // nodes per tile along i, k incl. halo
// Along j (contiguous in J) a tile row holds 16 nodes starting 4 before the tile's first cell, so
// each row is four aligned float4 chunks of J: the flush adds whole chunks with vector atomics.
// Nodes used: first cell - 1 .. first cell + TY + 1 (local 3 .. 13).
constexpr int HY = 16, JOFF = 4;
constexpr int TILE_NODES = HX * HY * HZ;
static_assert(TY + 2 + JOFF <= HY && JOFF % 4 == 0 && HY % 4 == 0, "tile row layout");

struct TileGrid {
  int ntx, nty, ntz;   // tiles along i, j, k
  int n_tiles;         // ntx * nty * ntz
  int bin_outside;     // particles outside the tiled cell range
  int bin_erased;      // erased particles (dropped by the sort)
  int n_bins;          // n_tiles + 2
};

__device__ __forceinline__ int tile_key(const TileGrid& T, int i, int j, int k) {
  if (i < 0 || j < 0 || k < 0) return T.bin_outside;
  const int ti = i / TX, tj = j / TY, tk = k / TZ;
  if (ti >= T.ntx || tj >= T.nty || tk >= T.ntz) return T.bin_outside;
  return (tk * T.nty + tj) * T.ntx + ti;
}

// Pass 1: bin of every particle and its rank inside the bin.
// Lanes of a warp that share a bin take consecutive ranks from one atomic (__match_any_sync), so
// after the first sort, when neighbouring particles share tiles, the bin counters see about one
// atomic per warp and the scatter below writes runs of consecutive slots.
__global__ void __launch_bounds__(256) k_tile_hist(TileGrid T, ParticlesF32 pt, const StateDev* st, int* counts,
                                                   int* key, int* rank) {
  const long long n = st->n_particles;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long n_iter = (n + stride - 1) / stride;
  const int lane = threadIdx.x & 31;
  for (long long it = 0; it < n_iter; it++) {
    const long long p = it * stride + blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const bool live = p < n;
    int b = -1;
    if (live) {
      if (pt.status[p] & 1) {
        b = T.bin_erased;
      } else {
        int i, j, k;
        unpack_cell(pt.cell[p], i, j, k);
        b = tile_key(T, i, j, k);
      }
    }
    const unsigned peers = __match_any_sync(0xffffffffu, b);
    const int leader = __ffs(peers) - 1;
    int base = 0;
    if (live && lane == leader) base = atomicAdd(counts + b, __popc(peers));
    base = __shfl_sync(peers, base, leader);
    if (live) {
      key[p] = b;
      rank[p] = base + __popc(peers & ((1u << lane) - 1u));
    }
  }
}

// Pass 2: exclusive scan of the bin counts in three short launches: per-1024-bin block scans,
// a scan of the block totals, and the add-back (which also clears the counts for the next sort
// and sets the particle count to exclude erased particles, kept in the last bin).
__device__ __forceinline__ int block_exclusive_scan_1024(int v, int* s_warp, int* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int w = lane < (int)(blockDim.x >> 5) ? s_warp[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    s_warp[lane] = w;  // inclusive prefix of warp sums
  }
  __syncthreads();
  const int before = (warp ? s_warp[warp - 1] : 0) + x - v;
  *total = s_warp[(blockDim.x >> 5) - 1];
  return before;
}

__global__ void __launch_bounds__(1024) k_scan_blocks(const int* counts, int* offsets, int* block_sums, int n) {
  __shared__ int s_warp[32];
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  const int v = b < n ? counts[b] : 0;
  int total;
  const int ex = block_exclusive_scan_1024(v, s_warp, &total);
  if (b < n) offsets[b] = ex;
  if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) k_scan_totals(int* block_sums, int nblocks) {
  __shared__ int s_warp[32];
  const int v = threadIdx.x < nblocks ? block_sums[threadIdx.x] : 0;
  int total;
  const int ex = block_exclusive_scan_1024(v, s_warp, &total);
  if (threadIdx.x < nblocks) block_sums[threadIdx.x] = ex;
  if (threadIdx.x == 0) block_sums[1024] = total;
}

__global__ void __launch_bounds__(1024) k_scan_add(int* counts, int* offsets, const int* block_sums, int n, int nblocks,
                                                   StateDev* st) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < n) {
    offsets[b] += block_sums[blockIdx.x];
    counts[b] = 0;
  }
  if (b == n - 1) {
    offsets[n] = block_sums[1024];
    st->n_particles = offsets[n - 1];  // the last bin holds the erased particles
  }
}

// Bin offsets before the first sort: every tile empty (an empty work list), all n particles in the
// bin outside the tiles, no erased ones.
__global__ void k_offsets_unsorted(int* offsets, int n_tiles, int n_bins, int n, int* work_count) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b <= n_bins) offsets[b] = b <= n_tiles ? 0 : n;
  if (b == 0) work_count[0] = work_count[1] = 0;  // no occupied tile until the first sort
}

// Pass 3: scatter every particle to its sorted slot in the other buffer set.
// Each thread moves two particles per iteration: all their loads are issued before any store,
// so a thread keeps the destination lookups and 2 x 15 loads in flight (the kernel is bound by
// the latency of the offsets[key] lookup, not by bandwidth).
struct Moved {
  long long cell, mcell;
  float fx, fy, fz, gx, gy, gz, mfx, mfy, mfz, q;
  uint8_t e, status;
  int id;
  long long d;
};

__device__ __forceinline__ Moved move_load(const ParticlesF32& src, const int* __restrict__ key,
                                           const int* __restrict__ rank, const int* __restrict__ offsets,
                                           long long p) {
  Moved m;
  m.d = (long long)offsets[key[p]] + rank[p];
  m.cell = src.cell[p];
  m.fx = src.fx[p]; m.fy = src.fy[p]; m.fz = src.fz[p];
  m.gx = src.gx[p]; m.gy = src.gy[p]; m.gz = src.gz[p];
  m.mcell = src.mcell[p];
  m.mfx = src.mfx[p]; m.mfy = src.mfy[p]; m.mfz = src.mfz[p];
  m.q = src.q[p]; m.e = src.e[p]; m.status = src.status[p]; m.id = src.id[p];
  return m;
}

__device__ __forceinline__ void move_store(const ParticlesF32& dst, const Moved& m) {
  const long long d = m.d;
  dst.cell[d] = m.cell;
  dst.fx[d] = m.fx; dst.fy[d] = m.fy; dst.fz[d] = m.fz;
  dst.gx[d] = m.gx; dst.gy[d] = m.gy; dst.gz[d] = m.gz;
  dst.mcell[d] = m.mcell;
  dst.mfx[d] = m.mfx; dst.mfy[d] = m.mfy; dst.mfz[d] = m.mfz;
  dst.q[d] = m.q; dst.e[d] = m.e; dst.status[d] = m.status; dst.cross[d] = 0;
  dst.id[d] = m.id;
}

__global__ void __launch_bounds__(256) k_tile_scatter(ParticlesF32 src, ParticlesF32 dst, const int* key,
                                                      const int* rank, const int* offsets, int n_bins) {
  const long long n_in = offsets[n_bins];  // every particle of the unsorted set, erased ones included
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n_in; p += 2 * stride) {
    const Moved a = move_load(src, key, rank, offsets, p);
    const bool two = p + stride < n_in;
    Moved b;
    if (two) b = move_load(src, key, rank, offsets, p + stride);
    move_store(dst, a);
    if (two) move_store(dst, b);
  }
}

// Zigzag contribution of one half segment into the shared tile, in edge form: the reference adds
// each Jx value to both ends of an x edge (nodes i and i+1, src/fdtd.cpp:105-130; likewise Jy along
// j and Jz along k), so the tile holds one value per edge, at its lower node, and the flush forms
// node(i) = edge(i) + edge(i-1).  12 shared atomics per half segment instead of 24.  Nodes outside
// the tile (particles that left their tile's halo) go straight to J in node form.
__device__ __forceinline__ void tile_half(float* sJ, float* J, long long cs, long long plane, int P1, int i0, int j0,
                                          int k0, int ic, int jc, int kc, float qh, float ax, float ay, float az,
                                          float jx, float jy, float jz) {
  const float x1 = 1.0f - ax, x2 = ax, y1 = 1.0f - ay, y2 = ay, z1 = 1.0f - az, z2 = az;
  const float qx = qh * jx, qy = qh * jy, qz = qh * jz;
  const int li = ic - i0, lj = jc - j0, lk = kc - k0;  // local node coordinates of the cell origin
  const bool in_tile = li >= 0 && lj >= 0 && lk >= 0 && li + 1 < HX && lj + 1 < HY && lk + 1 < HZ;
  if (in_tile) {
    // layout: ((k * HX + i) * HY + j), j fastest as in J
    constexpr int SI = HY, SK = HX * HY;
    const int s = (lk * HX + li) * HY + lj;
    float* ex = sJ;
    float* ey = sJ + TILE_NODES;
    float* ez = sJ + 2 * TILE_NODES;
    atomicAdd(ex + s, qx * (y1 * z1));
    atomicAdd(ex + s + 1, qx * (y2 * z1));
    atomicAdd(ex + s + SK, qx * (y1 * z2));
    atomicAdd(ex + s + SK + 1, qx * (y2 * z2));
    atomicAdd(ey + s, qy * (x1 * z1));
    atomicAdd(ey + s + SI, qy * (x2 * z1));
    atomicAdd(ey + s + SK, qy * (x1 * z2));
    atomicAdd(ey + s + SI + SK, qy * (x2 * z2));
    atomicAdd(ez + s, qz * (x1 * y1));
    atomicAdd(ez + s + SI, qz * (x2 * y1));
    atomicAdd(ez + s + 1, qz * (x1 * y2));
    atomicAdd(ez + s + SI + 1, qz * (x2 * y2));
    return;
  }
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const int di = (q >> 0) & 1, dj = (q >> 1) & 1, dk = (q >> 2) & 1;
    // weights of src/fdtd.cpp:105-130 for node (i+di, j+dj, k+dk)
    const float wx = (dj ? y2 : y1) * (dk ? z2 : z1);
    const float wy = (di ? x2 : x1) * (dk ? z2 : z1);
    const float wz = (di ? x2 : x1) * (dj ? y2 : y1);
    const long long m = (long long)(kc + dk) * plane + (long long)(ic + di) * P1 + (jc + dj);
    atomicAdd(J + m, wx * qx);
    atomicAdd(J + cs + m, wy * qy);
    atomicAdd(J + 2 * cs + m, wz * qz);
  }
}

// The cell's nodes (cell .. cell + 1 along each axis) lie in the tile's shared copy.
__device__ __forceinline__ bool cell_in_tile(int i0, int j0, int k0, int ic, int jc, int kc) {
  const int li = ic - i0, lj = jc - j0, lk = kc - k0;
  return li >= 0 && lj >= 0 && lk >= 0 && li + 1 < HX && lj + 1 < HY && lk + 1 < HZ;
}

// Both half segments of a particle that stayed in one cell (the common case in the boosted frame,
// where a particle moves a small fraction of a cell per step): the two halves weight the same
// twelve edges, so their sums are formed in registers and added with 12 shared atomics, not 24.
__device__ __forceinline__ void tile_both(float* sJ, int i0, int j0, int k0, int ic, int jc, int kc, float qh,
                                          float axp, float ayp, float azp, float jxp, float jyp, float jzp,
                                          float axm, float aym, float azm, float jxm, float jym, float jzm) {
  const int li = ic - i0, lj = jc - j0, lk = kc - k0;
  const float x1p = 1.0f - axp, y1p = 1.0f - ayp, z1p = 1.0f - azp;
  const float x1m = 1.0f - axm, y1m = 1.0f - aym, z1m = 1.0f - azm;
  constexpr int SI = HY, SK = HX * HY;
  const int s = (lk * HX + li) * HY + lj;
  // the four edges of one component: the sum over both halves of q j u v, where u and v are the
  // linear weights along the two other axes (u1 = 1 - a, u2 = a at the half's midpoint a)
  auto four = [&](float* e, int s1, int s2, float qp, float qm, float u1p, float u2p, float u1m, float u2m,
                  float v1p, float v2p, float v1m, float v2m) {
    const float a = qp * v1p, b = qp * v2p, c = qm * v1m, d = qm * v2m;
    atomicAdd(e + s, a * u1p + c * u1m);
    atomicAdd(e + s + s1, a * u2p + c * u2m);
    atomicAdd(e + s + s2, b * u1p + d * u1m);
    atomicAdd(e + s + s1 + s2, b * u2p + d * u2m);
  };
  four(sJ, 1, SK, qh * jxp, qh * jxm, y1p, ayp, y1m, aym, z1p, azp, z1m, azm);
  four(sJ + TILE_NODES, SI, SK, qh * jyp, qh * jym, x1p, axp, x1m, axm, z1p, azp, z1m, azm);
  four(sJ + 2 * TILE_NODES, SI, 1, qh * jzp, qh * jzm, x1p, axp, x1m, axm, y1p, ayp, y1m, aym);
}

// Both halves of a one-cell particle straight to J in node form (24 atomics instead of 48).
__device__ __forceinline__ void global_both(float* J, long long cs, long long m, long long sI, long long sK,
                                            float qh, float axp, float ayp, float azp, float jxp, float jyp,
                                            float jzp, float axm, float aym, float azm, float jxm, float jym,
                                            float jzm) {
  const float x1p = 1.0f - axp, y1p = 1.0f - ayp, z1p = 1.0f - azp;
  const float x1m = 1.0f - axm, y1m = 1.0f - aym, z1m = 1.0f - azm;
  // one component: edge values w(u, v) at the four (u, v) corners, each added at both ends (s0)
  auto four = [&](float* e, long long s0, long long s1, long long s2, float qp, float qm, float u1p, float u2p,
                  float u1m, float u2m, float v1p, float v2p, float v1m, float v2m) {
    const float a = qp * v1p, b = qp * v2p, c = qm * v1m, d = qm * v2m;
    const float w00 = a * u1p + c * u1m, w10 = a * u2p + c * u2m, w01 = b * u1p + d * u1m, w11 = b * u2p + d * u2m;
    atomicAdd(e + m, w00);
    atomicAdd(e + m + s0, w00);
    atomicAdd(e + m + s1, w10);
    atomicAdd(e + m + s1 + s0, w10);
    atomicAdd(e + m + s2, w01);
    atomicAdd(e + m + s2 + s0, w01);
    atomicAdd(e + m + s1 + s2, w11);
    atomicAdd(e + m + s1 + s2 + s0, w11);
  };
  four(J, sI, 1, sK, qh * jxp, qh * jxm, y1p, ayp, y1m, aym, z1p, azp, z1m, azm);
  four(J + cs, 1, sI, sK, qh * jyp, qh * jym, x1p, axp, x1m, axm, z1p, azp, z1m, azm);
  four(J + 2 * cs, sK, sI, 1, qh * jzp, qh * jzm, x1p, axp, x1m, axm, y1p, ayp, y1m, aym);
}

constexpr int kDepositBlock = 128;
constexpr int kDepositBlocksPerSM = 6;  // persistent deposit blocks per SM (shared copy and registers)
constexpr int kHeavyTile = 512;         // tiles with this many particles lead the work list
// Tiles with fewer particles than this skip the shared copy (zeroing and flushing its 1452 chunks
// costs more than the particles' global atomics).
constexpr int kSparseTile = 64;

// The deposit of one run of particles: the chunks of kDepositBlock particles from `beg`, stepping
// by `stride`, below `end`, each thread taking one particle of each chunk.
// `tiled`: the currents go to the shared tile copy whose node (0, 0, 0) is mesh node (i0, j0, k0)
// (the block then flushes it to J); otherwise straight to J with global atomics.
__device__ __forceinline__ void deposit_run(const DepositF32& D, const ParticlesF32& pt, float* sJ, float* J, float* rho,
                                            long long cs, long long plane, int P1, int beg, int end, int stride,
                                            bool tiled, int i0, int j0, int k0, int& kmin, int& kmax) {
  const long long sI = P1, sK = plane;
  // The particle data of the next iteration is loaded before the current particle's atomics, so
  // each thread keeps two particles' loads in flight (the loop is bound by global-load latency).
  struct Loaded {
    long long cell, mcell;
    float fx, fy, fz, mfx, mfy, mfz, q;
    uint8_t status;
  };
  auto load = [&](int p) {
    Loaded L;
    L.status = pt.status[p];  // particles erased since the last sort stay in their bins until the next
    L.cell = pt.cell[p]; L.mcell = pt.mcell[p];
    L.fx = pt.fx[p]; L.fy = pt.fy[p]; L.fz = pt.fz[p];
    L.mfx = pt.mfx[p]; L.mfy = pt.mfy[p]; L.mfz = pt.mfz[p];
    L.q = pt.q[p];
    return L;
  };
  // The lanes of a warp take particles four apart (thread t: offset 4 * lane + warp in each run of
  // kDepositBlock): consecutive particles, often the four members of one shot-noise beamlet in
  // neighbouring cells, go to different warps, so fewer lanes of one shared atomic meet on an edge.
  static_assert(kDepositBlock == 128, "four warps per deposit block");
  int p = beg + (int)((threadIdx.x & 31) * 4 + (threadIdx.x >> 5));
  Loaded cur{};
  if (p < end) cur = load(p);
  for (; p < end; p += stride) {
    Loaded nxt{};
    if (p + stride < end) nxt = load(p + stride);
    int ip, jp, kp, im, jm, km;
    unpack_cell(cur.cell, ip, jp, kp);
    unpack_cell(cur.mcell, im, jm, km);
    const bool live = !(cur.status & 1);
    if (live) {
      kmin = min(kmin, kp);
      kmax = max(kmax, kp);
    }
    const float fxp = cur.fx, fyp = cur.fy, fzp = cur.fz;
    const float fxm = cur.mfx, fym = cur.mfy, fzm = cur.mfz;
    const bool bp = live && inside_f32(D, ip, jp, kp, fxp, fyp);
    const bool bm = live && inside_f32(D, im, jm, km, fxm, fym);
    if (bp || bm) {
      int bx, by, bz;
      float rxm, rxp, rym, ryp, rzm, rzp;
      const float rx = relay_axis(im, ip, fxm, fxp, &bx, &rxm, &rxp);
      const float ry = relay_axis(jm, jp, fym, fyp, &by, &rym, &ryp);
      const float rz = relay_axis(km, kp, fzm, fzp, &bz, &rzm, &rzp);
      const float qh = 0.5f * cur.q;
      const bool one_cell = bp && bm && ip == im && jp == jm && kp == km;
      if (one_cell) {  // base = the cell itself: both halves in one pass
        const float axp = 0.5f * (rxp + rx), ayp = 0.5f * (ryp + ry), azp = 0.5f * (rzp + rz);
        const float axm = 0.5f * (rxm + rx), aym = 0.5f * (rym + ry), azm = 0.5f * (rzm + rz);
        const float jxp = (rxp - rx) * D.dx, jyp = (ryp - ry) * D.dy, jzp = (rzp - rz) * D.dz;
        const float jxm = (rx - rxm) * D.dx, jym = (ry - rym) * D.dy, jzm = (rz - rzm) * D.dz;
        if (tiled && cell_in_tile(i0, j0, k0, ip, jp, kp))
          tile_both(sJ, i0, j0, k0, ip, jp, kp, qh, axp, ayp, azp, jxp, jyp, jzp, axm, aym, azm, jxm, jym, jzm);
        else
          global_both(J, cs, (long long)kp * plane + (long long)ip * P1 + jp, sI, sK, qh, axp, ayp, azp, jxp, jyp,
                      jzp, axm, aym, azm, jxm, jym, jzm);
      } else {
        if (bp) {
          const float ax = 0.5f * (rxp + rx) - (float)(ip - bx), ay = 0.5f * (ryp + ry) - (float)(jp - by),
                      az = 0.5f * (rzp + rz) - (float)(kp - bz);
          if (tiled)
            tile_half(sJ, J, cs, plane, P1, i0, j0, k0, ip, jp, kp, qh, ax, ay, az, (rxp - rx) * D.dx,
                      (ryp - ry) * D.dy, (rzp - rz) * D.dz);
          else
            deposit_half_f32(J, cs, (long long)kp * plane + (long long)ip * P1 + jp, sI, sK, qh, ax, ay, az,
                             (rxp - rx) * D.dx, (ryp - ry) * D.dy, (rzp - rz) * D.dz);
        }
        if (bm) {
          const float ax = 0.5f * (rxm + rx) - (float)(im - bx), ay = 0.5f * (rym + ry) - (float)(jm - by),
                      az = 0.5f * (rzm + rz) - (float)(km - bz);
          if (tiled)
            tile_half(sJ, J, cs, plane, P1, i0, j0, k0, im, jm, km, qh, ax, ay, az, (rx - rxm) * D.dx,
                      (ry - rym) * D.dy, (rz - rzm) * D.dz);
          else
            deposit_half_f32(J, cs, (long long)km * plane + (long long)im * P1 + jm, sI, sK, qh, ax, ay, az,
                             (rx - rxm) * D.dx, (ry - rym) * D.dy, (rz - rzm) * D.dz);
        }
      }
      if (bp && rho) {
        const long long m = (long long)kp * plane + (long long)ip * P1 + jp;
        const float q = cur.q;
        const float x1 = 1.0f - fxp, y1 = 1.0f - fyp, z1 = 1.0f - fzp;
        atomicAdd(rho + m, q * x1 * y1 * z1);
        atomicAdd(rho + m + sI, q * fxp * y1 * z1);
        atomicAdd(rho + m + 1, q * x1 * fyp * z1);
        atomicAdd(rho + m + sI + 1, q * fxp * fyp * z1);
        atomicAdd(rho + m + sK, q * x1 * y1 * fzp);
        atomicAdd(rho + m + sK + sI, q * fxp * y1 * fzp);
        atomicAdd(rho + m + sK + 1, q * x1 * fyp * fzp);
        atomicAdd(rho + m + sK + sI + 1, q * fxp * fyp * fzp);
      }
    }
    cur = nxt;
  }
  if (!tiled) return;
  __syncthreads();
  // Flush: the node values of every chunk of four nodes along j, node(n) = edge(n) + edge(n - unit
  // step along the component), are added to J with one vector atomic.  A component holds
  // HX * HZ rows of CH chunks; thread t takes the chunks t + u * kDepositBlock (u < 4) of every
  // component, so their positions and bounds are worked out once.  A chunk lies wholly inside or
  // wholly outside a padded row of J (both are aligned to four nodes), and only non-zero chunks,
  // which hold nodes of real cells, are added.
  constexpr int CH = HY / 4, ITEMS = HX * HZ * CH, U = 4;
  static_assert(ITEMS <= U * kDepositBlock, "flush items per thread");
  long long goff[U];
  int flags[U];  // bit 0: chunk in the mesh, bit 1: li > 0, bit 2: lk > 0, bit 3: q > 0
#pragma unroll
  for (int u = 0; u < U; u++) {
    const int item = threadIdx.x + u * kDepositBlock;
    const int q = item % CH, row = item / CH, li = row % HX, lk = row / HX;
    const int gi = i0 + li, gj = j0 + 4 * q, gk = k0 + lk;
    const bool ok = item < ITEMS && gi >= 0 && gj >= 0 && gk >= 0 && gi < D.N0 && gj < P1 && gk < D.N2;
    flags[u] = (ok ? 1 : 0) | (li > 0 ? 2 : 0) | (lk > 0 ? 4 : 0) | (q > 0 ? 8 : 0);
    goff[u] = (long long)gk * plane + (long long)gi * P1 + gj;
  }
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const float* e = sJ + c * TILE_NODES;
    const float4* e4 = reinterpret_cast<const float4*>(e);
    float4 v[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int item = threadIdx.x + u * kDepositBlock;
      v[u] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (!(flags[u] & 1)) continue;
      v[u] = e4[item];
      if (c == 0) {
        if (flags[u] & 2) { const float4 w = e4[item - CH]; v[u].x += w.x; v[u].y += w.y; v[u].z += w.z; v[u].w += w.w; }
      } else if (c == 1) {
        const float* n = e + 4 * item;  // the chunk's first node
        v[u].w += n[2]; v[u].z += n[1]; v[u].y += n[0];
        if (flags[u] & 8) v[u].x += n[-1];
      } else {
        if (flags[u] & 4) { const float4 w = e4[item - CH * HX]; v[u].x += w.x; v[u].y += w.y; v[u].z += w.z; v[u].w += w.w; }
      }
    }
    float* Jc = J + c * cs;
#pragma unroll
    for (int u = 0; u < U; u++)
      if (v[u].x != 0.0f || v[u].y != 0.0f || v[u].z != 0.0f || v[u].w != 0.0f)
        atomicAdd(reinterpret_cast<float4*>(Jc + goff[u]), v[u]);
  }
}

// The occupied tiles of the last sort are handed out one at a time to persistent blocks (a few per
// SM), which take the next entry of the work list with one atomic: the heavy tiles (at least
// kHeavyTile particles) come first, so the light ones even out the blocks' ends, and the empty
// tiles of the mesh (most of them) cost nothing.  A tile's particles deposit into the shared
// copy, which is flushed to J; tiles holding fewer than kSparseTile particles deposit with global
// atomics.  Afterwards every block takes its share of the particles that follow the tiles' bins:
// the bin outside the tiled cells and, on a step that did not sort, the particles appended since
// the last sort (they follow the live particles of the sort, where the bin of erased particles
// began).
__global__ void __launch_bounds__(kDepositBlock, 6)
    k_deposit_tiled(DepositF32 D, TileGrid T, ParticlesF32 pt, const int* offsets, const int* work,
                    const int* work_count, int* work_next, StateDev* st, float* J, float* rho, long long cs,
                    long long plane, int P1) {
  extern __shared__ float sJ[];  // 3 * TILE_NODES
  __shared__ int s_w;
  int kmin = 0x7fffffff, kmax = -0x7fffffff;
  const int n_heavy = work_count[0], n_work = work_count[0] + work_count[1];
  for (;;) {
    if (threadIdx.x == 0) s_w = atomicAdd(work_next, 1);
    __syncthreads();
    const int w = s_w;
    if (w >= n_work) break;
    const int b = w < n_heavy ? work[w] : work[T.n_tiles - 1 - (w - n_heavy)];
    const int beg = offsets[b], end = offsets[b + 1];
    const bool tiled = end - beg >= kSparseTile;
    int i0 = 0, j0 = 0, k0 = 0;
    if (tiled) {
      const int ti = b % T.ntx, tj = (b / T.ntx) % T.nty, tk = b / (T.ntx * T.nty);
      i0 = ti * TX - 1; j0 = tj * TY - JOFF; k0 = tk * TZ - 1;  // halo of one cell below
      float4* s4 = reinterpret_cast<float4*>(sJ);
      for (int q = threadIdx.x; q < 3 * TILE_NODES / 4; q += blockDim.x) s4[q] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();  // the copy is zeroed, and every thread has read s_w
    deposit_run(D, pt, sJ, J, rho, cs, plane, P1, beg, end, kDepositBlock, tiled, i0, j0, k0, kmin, kmax);
    __syncthreads();  // the flush has read the copy the next tile zeroes
  }
  deposit_run(D, pt, sJ, J, rho, cs, plane, P1, offsets[T.bin_outside] + (int)blockIdx.x * kDepositBlock,
              (int)st->n_particles, (int)gridDim.x * kDepositBlock, false, 0, 0, 0, kmin, kmax);
  slab_update(st, kmin, kmax);
}

// The work list of the deposit, built after a sort: the occupied tiles, those with at least
// kHeavyTile particles from the front of `work` (count in work_count[0]), the others from its
// back (count in work_count[1]); one warp-aggregated atomic per warp and list, counts zeroed by
// the caller.
__global__ void __launch_bounds__(256) k_tile_worklist(const int* offsets, int n_tiles, int* work, int* work_count) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = b < n_tiles ? offsets[b + 1] - offsets[b] : 0;
  const int lane = threadIdx.x & 31;
  for (int heavy = 0; heavy < 2; heavy++) {
    const bool take = c > 0 && ((c >= kHeavyTile) == (heavy == 0));
    const unsigned bal = __ballot_sync(0xffffffffu, take);
    int base = 0;
    if (lane == 0 && bal) base = atomicAdd(work_count + heavy, __popc(bal));
    base = __shfl_sync(0xffffffffu, base, 0);
    const int r = base + __popc(bal & ((1u << lane) - 1u));
    if (take) work[heavy == 0 ? r : n_tiles - 1 - r] = b;
  }
}

// Download in creation order: every live particle is written to row `id` of a scratch table with
// a valid flag; a one-block pass then compacts the valid rows in id order.
__global__ void __launch_bounds__(256) k_f32_to_rows_by_id(ParticlesF32 pt, const StateDev* st, double* rows,
                                                           uint8_t* valid, long long id_cap, CellMap M) {
  const long long n = st->n_particles;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    if (pt.status[p] & 1) continue;
    const long long id = pt.id[p];
    if (id < 0 || id >= id_cap) continue;
    double* r = rows + 11 * id;
    int i, j, k;
    unpack_cell(pt.cell[p], i, j, k);
    r[0] = pt.q[p];
    r[1] = M.xmin + ((double)i + (double)pt.fx[p]) * M.dx;
    r[2] = M.ymin + ((double)j + (double)pt.fy[p]) * M.dy;
    r[3] = M.zmin + ((double)k + (double)pt.fz[p]) * M.dz;
    unpack_cell(pt.mcell[p], i, j, k);
    r[4] = M.xmin + ((double)i + (double)pt.mfx[p]) * M.dx;
    r[5] = M.ymin + ((double)j + (double)pt.mfy[p]) * M.dy;
    r[6] = M.zmin + ((double)k + (double)pt.mfz[p]) * M.dz;
    r[7] = pt.gx[p]; r[8] = pt.gy[p]; r[9] = pt.gz[p];
    r[10] = pt.e[p] ? 1.0 : 0.0;
    valid[id] = 1;
  }
}

__global__ void __launch_bounds__(1024) k_compact_rows(const double* rows, const uint8_t* valid, long long id_cap,
                                                       double* rec, long long cap, long long* n_out) {
  __shared__ int s_warp[32];
  __shared__ long long s_base;
  if (threadIdx.x == 0) s_base = 0;
  __syncthreads();
  for (long long c0 = 0; c0 < id_cap; c0 += blockDim.x) {
    const long long p = c0 + threadIdx.x;
    const int take = (p < id_cap) && valid[p];
    const unsigned bal = __ballot_sync(0xffffffffu, take);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) s_warp[warp] = __popc(bal);
    __syncthreads();
    int before = 0, total = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
      if (w < warp) before += s_warp[w];
      total += s_warp[w];
    }
    before += __popc(bal & ((1u << lane) - 1u));
    const long long d = s_base + before;
    if (take && d < cap)
      for (int c = 0; c < 11; c++) rec[11 * d + c] = rows[11 * p + c];
    __syncthreads();
    if (threadIdx.x == 0) s_base += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) *n_out = s_base;
}

}  // namespace mithra
