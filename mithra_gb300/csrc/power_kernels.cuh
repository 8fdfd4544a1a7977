// Radiated power through z-planes, Solver::powerSample (src/radiation.cpp:127-232).
//
// Per sampling plane and transverse node (i, j in [2, N-3]): interpolate E and B in z, transform
// them into the lab frame, store the four values in ring slot nTime % Nf, and run the Nf-tap DFT
// at each frequency (the FP64 form sums the whole ring as the reference does; the mixed form keeps
// the sums per node and adds the change of the one slot that was overwritten).  Per-node
// contributions are summed per block into a partial buffer that a second, single-block kernel
// reduces in a fixed order, so a run is reproducible.
#pragma once
#include "device_common.cuh"

namespace mithra {

// Component c of node m of E (B) is E[c * ecs + m * ens]: component planes (ecs = cstride,
// ens = 1) in the FP64 form, the node records of the mixed form (ecs = 1, ens = kEBNode, B = E + 4).
template <int BLOCK, typename TE>
__global__ void __launch_bounds__(BLOCK) k_power_sample(GridDev g, PowerDev pw, const TE* __restrict__ E,
                                                        const TE* __restrict__ B, long long ecs, int ens,
                                                        const StateDev* st) {
  extern __shared__ double s_red[];  // Nl * BLOCK
  const int plane = blockIdx.x / pw.blocks_per_plane;
  const int bip = blockIdx.x % pw.blocks_per_plane;
  const int k_cell = pw.plane_k[plane];
  const long long nodes = (long long)pw.nodes_i * pw.nodes_j;
  const long long t = (long long)bip * BLOCK + threadIdx.x;
  const unsigned slot = (unsigned)(st->n_time % pw.Nf);
  for (int l = 0; l < pw.Nl; l++) s_red[l * BLOCK + threadIdx.x] = 0.0;
  if (k_cell >= 0 && t < nodes) {
    const int i = 2 + (int)(t / pw.nodes_j), j = 2 + (int)(t % pw.nodes_j);
    const long long mi = node_index(g, k_cell, i, j) * ens;
    const long long cs = ecs, sK = g.plane * ens;
    const double dzr = pw.plane_dzr[plane];
    const double et0 = (1.0 - dzr) * (double)E[mi] + dzr * (double)E[mi + sK];
    const double et1 = (1.0 - dzr) * (double)E[cs + mi] + dzr * (double)E[cs + mi + sK];
    const double bt0 = (1.0 - dzr) * (double)B[mi] + dzr * (double)B[mi + sK];
    const double bt1 = (1.0 - dzr) * (double)B[cs + mi] + dzr * (double)B[cs + mi + sK];
    const long long vstride = (long long)pw.nz * nodes;  // between the four values
    const long long sstride = 4 * vstride;               // between ring slots
    const long long ni = (long long)pw.plane_slot[plane] * nodes + t;
    double* f = pw.fdt + (long long)slot * sstride + ni;
    // Lab-frame fields, src/radiation.cpp:187-191.
    const double f0 = pw.gamma * (et0 + pw.c0 * pw.beta * bt1);
    const double f1 = pw.gamma * (et1 - pw.c0 * pw.beta * bt0);
    const double f2 = pw.gamma * (bt0 - pw.beta / pw.c0 * et1);
    const double f3 = pw.gamma * (bt1 + pw.beta / pw.c0 * et0);
    if (pw.run) {
      // Running sums (mixed form): the sum over the ring changes only in this step's slot, by
      // (new - old) times that slot's twiddle.  Same terms as the loop below, O(1) per step.
      const double d0 = f0 - f[0], d1 = f1 - f[vstride], d2 = f2 - f[2 * vstride], d3 = f3 - f[3 * vstride];
      f[0] = f0; f[vstride] = f1; f[2 * vstride] = f2; f[3 * vstride] = f3;
      const long long all = (long long)pw.nz * nodes;
      for (int l = 0; l < pw.Nl; l++) {
        double* r = pw.run + (long long)l * 8 * all + ni;
        const double cr = __ldg(pw.tw_re + l * pw.Nf + slot), ci = __ldg(pw.tw_im + l * pw.Nf + slot);
        const double ew1r = r[0] + d0 * cr, ew1i = r[all] + d0 * ci, bw1r = r[2 * all] + d3 * cr,
                     bw1i = r[3 * all] - d3 * ci, ew2r = r[4 * all] + d1 * cr, ew2i = r[5 * all] + d1 * ci,
                     bw2r = r[6 * all] + d2 * cr, bw2i = r[7 * all] - d2 * ci;
        r[0] = ew1r; r[all] = ew1i; r[2 * all] = bw1r; r[3 * all] = bw1i;
        r[4 * all] = ew2r; r[5 * all] = ew2i; r[6 * all] = bw2r; r[7 * all] = bw2i;
        s_red[l * BLOCK + threadIdx.x] = pw.pc * ((ew1r * bw1r - ew1i * bw1i) - (ew2r * bw2r - ew2i * bw2i));
      }
    } else {
      f[0] = f0; f[vstride] = f1; f[2 * vstride] = f2; f[3 * vstride] = f3;
      for (int l = 0; l < pw.Nl; l++) {
        double ew1r = 0.0, ew1i = 0.0, bw1r = 0.0, bw1i = 0.0, ew2r = 0.0, ew2i = 0.0, bw2r = 0.0, bw2i = 0.0;
        const double* h = pw.fdt + ni;
        for (int m = 0; m < pw.Nf; m++) {
          const double g0 = h[0], g1 = h[vstride], g2 = h[2 * vstride], g3 = h[3 * vstride];
          const double cr = __ldg(pw.tw_re + l * pw.Nf + m), ci = __ldg(pw.tw_im + l * pw.Nf + m);
          ew1r += g0 * cr; ew1i += g0 * ci;
          bw1r += g3 * cr; bw1i -= g3 * ci;
          ew2r += g1 * cr; ew2i += g1 * ci;
          bw2r += g2 * cr; bw2i -= g2 * ci;
          h += sstride;
        }
        s_red[l * BLOCK + threadIdx.x] = pw.pc * ((ew1r * bw1r - ew1i * bw1i) - (ew2r * bw2r - ew2i * bw2i));
      }
    }
  }
  __syncthreads();
  for (int s = BLOCK / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int l = 0; l < pw.Nl; l++) s_red[l * BLOCK + threadIdx.x] += s_red[l * BLOCK + threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int l = 0; l < pw.Nl; l++) pw.partial[(long long)blockIdx.x * pw.Nl + l] = s_red[l * BLOCK];
}

// Sums the per-block partials of every plane in block order and appends one row to the log:
// per plane  z_lab = gamma (z + beta c0 (timeBunch + dt_))  then Nl powers (src/radiation.cpp:222-229).
__global__ void k_power_finish(PowerDev pw, StateDev* st, int last_output) {
  const long long row = st->n_power_rows;
  const int rowlen = pw.N * (1 + pw.Nl);
  for (int k = threadIdx.x; row < pw.row_cap && k < pw.N; k += blockDim.x) {
    double* r = pw.rows + row * rowlen + (long long)k * (1 + pw.Nl);
    r[0] = pw.gamma * (pw.z[k] + pw.beta * pw.c0 * (st->time_bunch + pw.dt_shift));
    for (int l = 0; l < pw.Nl; l++) {
      double s = 0.0;
      if (pw.plane_k[k] >= 0)
        for (int b = 0; b < pw.blocks_per_plane; b++) s += pw.partial[((long long)k * pw.blocks_per_plane + b) * pw.Nl + l];
      r[1 + l] = s;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && last_output) st->n_power_rows = row + 1;
}

}  // namespace mithra
