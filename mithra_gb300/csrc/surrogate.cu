// Learned surrogate of FEL runs: BF16 tensor-core GEMMs (tc_gemm.cuh) and the kernels of a small
// MLP trained on the device.  This file: the GEMM entry point.
#include <cuda_runtime.h>

#include "../../include/mithra_gpu.h"
#include "tc_gemm.cuh"

using namespace mithra;

namespace {

typedef CUresult (*EncodeTiledFnGemm)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                      const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                      CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFnGemm encode_fn() {
  static EncodeTiledFnGemm fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFnGemm)p;
  }
  return fn;
}

// Row-major BF16 [rows x K] operand as a tensor map with 64 x box_rows boxes and 128-byte swizzle.
bool operand_map(CUtensorMap* map, const void* base, int rows, int K, int box_rows) {
  EncodeTiledFnGemm enc = encode_fn();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)K * 2};
  const cuuint32_t box[2] = {(cuuint32_t)tc::BK, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

extern "C" int mithra_tc_gemm(const void* A, const void* B, float* C, void* C_bf16, const float* bias, int M, int N,
                              int K, int act, void* stream, int* err_dev) {
  if (!A || !B || (!C && !C_bf16) || !err_dev || M <= 0 || N <= 0 || K <= 0) return MITHRA_ERR_ARG;
  if (M % tc::BM || N % tc::BN || K % tc::BK) return MITHRA_ERR_ARG;
  if (((uintptr_t)A | (uintptr_t)B) & 15) return MITHRA_ERR_ARG;
  // Long K loops go through the pipelined TMA kernel; one or two K blocks through the simple one
  // (nothing to overlap, and no tensor maps to encode).
  if (K >= 4 * tc::BK) {
    static bool attr_tma = false;
    if (!attr_tma) {
      if (cudaFuncSetAttribute(tc::k_gemm_bf16_tma<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)tc::gemm_tma_smem<128>()) != cudaSuccess ||
          cudaFuncSetAttribute(tc::k_gemm_bf16_tma<256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)tc::gemm_tma_smem<256>()) != cudaSuccess)
        return MITHRA_ERR_CUDA;
      attr_tma = true;
    }
    const bool wide = N % 256 == 0;  // 128 x 256 tiles halve the A traffic per flop
    CUtensorMap ma, mb;
    if (!operand_map(&ma, A, M, K, tc::BM) || !operand_map(&mb, B, N, K, wide ? 256 : 128)) return MITHRA_ERR_CUDA;
    if (wide)
      tc::k_gemm_bf16_tma<256><<<dim3(M / tc::BM, N / 256), 128, tc::gemm_tma_smem<256>(), (cudaStream_t)stream>>>(
          ma, mb, C, (__nv_bfloat16*)C_bf16, bias, M, N, K, act, err_dev);
    else
      tc::k_gemm_bf16_tma<128><<<dim3(M / tc::BM, N / 128), 128, tc::gemm_tma_smem<128>(), (cudaStream_t)stream>>>(
          ma, mb, C, (__nv_bfloat16*)C_bf16, bias, M, N, K, act, err_dev);
    return cudaGetLastError() == cudaSuccess ? MITHRA_OK : MITHRA_ERR_CUDA;
  }
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(tc::k_gemm_bf16, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc::kGemmSmem) !=
        cudaSuccess)
      return MITHRA_ERR_CUDA;
    attr = true;
  }
  dim3 grid(M / tc::BM, N / tc::BN);
  tc::k_gemm_bf16<<<grid, 128, tc::kGemmSmem, (cudaStream_t)stream>>>(
      (const __nv_bfloat16*)A, (const __nv_bfloat16*)B, C, (__nv_bfloat16*)C_bf16, bias, M, N, K, act, err_dev);
  return cudaGetLastError() == cudaSuccess ? MITHRA_OK : MITHRA_ERR_CUDA;
}

// ---- MLP surrogate ----------------------------------------------------------------------------
//
// Ensemble of fully connected ReLU networks, n_in -> n_hidden x n_layers -> n_out, trained with
// Adam on mean-squared error.  All matrix products run on the tensor cores (k_gemm_bf16, BF16
// operands, FP32 accumulate); master weights, biases, moments and the loss stay FP32.  Widths are
// padded on the device to the GEMM's multiples (inputs to 128, outputs to 128, batch to 128) with
// zero weights and zero inputs, so padding never changes a result.
#include <cuda_bf16.h>

#include <cmath>
#include <random>
#include <vector>

namespace {

using bf16 = __nv_bfloat16;

int round_up(int x, int m) { return (x + m - 1) / m * m; }

__global__ void k_to_bf16_padded(const float* __restrict__ x, int rows, int cols, int ld_in, bf16* __restrict__ y,
                                 int rows_pad, int cols_pad) {
  const long long n = (long long)rows_pad * cols_pad;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(t / cols_pad), c = (int)(t % cols_pad);
    y[t] = __float2bfloat16_rn((r < rows && c < cols) ? x[(long long)r * ld_in + c] : 0.0f);
  }
}

// y[c][r] = x[r][c] for an R x C bf16 matrix.
__global__ void k_transpose_bf16(const bf16* __restrict__ x, int R, int C, bf16* __restrict__ y) {
  __shared__ bf16 t[32][33];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int r = r0 + i, c = c0 + threadIdx.x;
    if (r < R && c < C) t[i][threadIdx.x] = x[(long long)r * C + c];
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int c = c0 + i, r = r0 + threadIdx.x;
    if (r < R && c < C) y[(long long)c * R + r] = t[threadIdx.x][i];
  }
}

// d = (out - y) * 2 / (rows * cols) on the real rows/columns, 0 on padding; also bf16 copy.
__global__ void k_mse_grad(const float* __restrict__ out, int ld_out, const float* __restrict__ y, int ld_y, int rows,
                           int cols, int rows_pad, int cols_pad, float scale, float* __restrict__ d, bf16* __restrict__ db,
                           double* __restrict__ loss) {
  const long long n = (long long)rows_pad * cols_pad;
  double acc = 0.0;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(t / cols_pad), c = (int)(t % cols_pad);
    float g = 0.0f;
    if (r < rows && c < cols) {
      const float e = out[(long long)r * ld_out + c] - y[(long long)r * ld_y + c];
      acc += (double)e * e;
      g = 2.0f * e * scale;
    }
    d[t] = g;
    db[t] = __float2bfloat16_rn(g);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc);
}

// dz = dh * (h > 0) (ReLU derivative through the stored activation), FP32 and bf16.
__global__ void k_relu_back(const float* __restrict__ dh, const float* __restrict__ h, long long n, bf16* __restrict__ dzb) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
    dzb[t] = __float2bfloat16_rn(h[t] > 0.0f ? dh[t] : 0.0f);
}

// db[c] = sum_r dz[r][c] (bf16 input) over the first `rows` rows.
__global__ void k_col_sum(const bf16* __restrict__ dz, int rows, int cols, float* __restrict__ db) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.0f;
  for (int r = 0; r < rows; r++) s += __bfloat162float(dz[(long long)r * cols + c]);
  db[c] = s;
}

__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       long long n, float lr, float b1, float b2, float eps, float c1, float c2,
                       const unsigned char* __restrict__ mask) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    if (mask && !mask[t]) continue;  // padding stays zero
    const float gt = g[t];
    m[t] = b1 * m[t] + (1.0f - b1) * gt;
    v[t] = b2 * v[t] + (1.0f - b2) * gt * gt;
    w[t] -= lr * (m[t] / c1) / (sqrtf(v[t] / c2) + eps);
  }
}

__global__ void k_f32_to_bf16(const float* __restrict__ x, long long n, bf16* __restrict__ y) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
    y[t] = __float2bfloat16_rn(x[t]);
}

int blocks_for(long long n) { return (int)std::min<long long>(4096, std::max<long long>(1, (n + 255) / 256)); }

struct Layer {
  int in, out;            // padded sizes (in: K of the forward GEMM, out: N)
  int in_real, out_real;
  float *w = nullptr, *b = nullptr;     // FP32 master [out x in], [out]
  float *mw = nullptr, *vw = nullptr, *mb = nullptr, *vb = nullptr;
  float *gw = nullptr, *gb = nullptr;   // gradients
  bf16 *wb = nullptr, *wtb = nullptr;   // bf16 W [out x in] and W^T [in x out]
  unsigned char *mask_w = nullptr, *mask_b = nullptr;  // 1 on real entries
};

}  // namespace

struct mithra_mlp {
  int n_in, n_hidden, n_layers, n_out, ensemble, device;
  int in_pad, out_pad;
  std::vector<std::vector<Layer>> nets;  // [member][layer]
  int step = 0;
  int max_batch = 0;
  // activations and work buffers for one member at a time (batch padded)
  bf16* xb = nullptr;                  // input bf16 [B x in_pad]
  std::vector<float*> hf;              // FP32 activations per layer output [B x out]
  std::vector<bf16*> hb;               // bf16 activations
  std::vector<bf16*> hbt;              // bf16 transposed activations [out x B]
  bf16* xbt = nullptr;                 // input transposed [in_pad x B]
  float* dh = nullptr;                 // FP32 gradient w.r.t. a layer input [B x max width]
  bf16* dzb = nullptr;                 // bf16 dZ [B x max width]
  bf16* dzbt = nullptr;                // bf16 dZ^T [max width x B]
  float* dout = nullptr;               // FP32 dOut [B x out_pad]
  double* loss = nullptr;
  int* err = nullptr;
  cudaStream_t stream = nullptr;
};

namespace {

int alloc_batch(mithra_mlp* m, int B) {
  if (B <= m->max_batch) return MITHRA_OK;
  for (auto p : m->hf) cudaFree(p);
  for (auto p : m->hb) cudaFree(p);
  for (auto p : m->hbt) cudaFree(p);
  cudaFree(m->xb); cudaFree(m->xbt); cudaFree(m->dh); cudaFree(m->dzb); cudaFree(m->dzbt); cudaFree(m->dout);
  m->hf.assign(m->n_layers + 1, nullptr);
  m->hb.assign(m->n_layers + 1, nullptr);
  m->hbt.assign(m->n_layers + 1, nullptr);
  const int wmax = std::max(std::max(m->n_hidden, m->out_pad), m->in_pad);
  bool ok = cudaMalloc(&m->xb, (size_t)B * m->in_pad * 2) == cudaSuccess &&
            cudaMalloc(&m->xbt, (size_t)B * m->in_pad * 2) == cudaSuccess &&
            cudaMalloc(&m->dh, (size_t)B * wmax * 4) == cudaSuccess &&
            cudaMalloc(&m->dzb, (size_t)B * wmax * 2) == cudaSuccess &&
            cudaMalloc(&m->dzbt, (size_t)B * wmax * 2) == cudaSuccess &&
            cudaMalloc(&m->dout, (size_t)B * m->out_pad * 4) == cudaSuccess;
  for (int l = 0; ok && l <= m->n_layers; l++) {
    const int w = (l == m->n_layers) ? m->out_pad : m->n_hidden;
    ok = cudaMalloc(&m->hf[l], (size_t)B * w * 4) == cudaSuccess && cudaMalloc(&m->hb[l], (size_t)B * w * 2) == cudaSuccess &&
         cudaMalloc(&m->hbt[l], (size_t)B * w * 2) == cudaSuccess;
  }
  if (!ok) return MITHRA_ERR_CUDA;
  m->max_batch = B;
  return MITHRA_OK;
}

int gemm(mithra_mlp* m, const bf16* A, const bf16* B, float* C, bf16* Cb, const float* bias, int M, int N, int K,
         int act) {
  return mithra_tc_gemm(A, B, C, Cb, bias, M, N, K, act, m->stream, m->err);
}

void transpose(mithra_mlp* m, const bf16* x, int R, int C, bf16* y) {
  dim3 blk(32, 8), grd((C + 31) / 32, (R + 31) / 32);
  k_transpose_bf16<<<grd, blk, 0, m->stream>>>(x, R, C, y);
}

void refresh_bf16(mithra_mlp* m, Layer& L) {
  const long long n = (long long)L.out * L.in;
  k_f32_to_bf16<<<blocks_for(n), 256, 0, m->stream>>>(L.w, n, L.wb);
  transpose(m, L.wb, L.out, L.in, L.wtb);
}

// Forward pass of one member for Bp (padded) rows of xb; leaves activations in hf/hb.
int forward(mithra_mlp* m, std::vector<Layer>& net, int Bp) {
  const bf16* in = m->xb;
  for (int l = 0; l <= m->n_layers; l++) {
    Layer& L = net[l];
    const bool last = (l == m->n_layers);
    int r = gemm(m, in, L.wb, m->hf[l], m->hb[l], L.b, Bp, L.out, L.in, last ? tc::kNone : tc::kRelu);
    if (r) return r;
    in = m->hb[l];
  }
  return MITHRA_OK;
}

// Gradients of the mean-squared error for one member (forward must have run); fills gw, gb.
int backward(mithra_mlp* m, std::vector<Layer>& net, int Bp, int B, const float* Y, int ld_y) {
  const int nl = m->n_layers;
  const long long nout = (long long)Bp * m->out_pad;
  k_mse_grad<<<blocks_for(nout), 256, 0, m->stream>>>(m->hf[nl], m->out_pad, Y, ld_y, B, m->n_out, Bp, m->out_pad,
                                                    1.0f / ((float)B * m->n_out), m->dout, m->dzb, m->loss);
  for (int l = nl; l >= 0; l--) {
    Layer& L = net[l];
    // dZ (bf16, in dzb) -> dW = dZ^T H_{l-1}, db = column sums, dH_{l-1} = dZ W
    transpose(m, m->dzb, Bp, L.out, m->dzbt);
    const bf16* hin = (l == 0) ? m->xb : m->hb[l - 1];
    bf16* hint = (l == 0) ? m->xbt : m->hbt[l - 1];
    transpose(m, hin, Bp, L.in, hint);
    int r = gemm(m, m->dzbt, hint, L.gw, nullptr, nullptr, L.out, L.in, Bp, tc::kNone);
    if (r) return r;
    k_col_sum<<<(L.out + 127) / 128, 128, 0, m->stream>>>(m->dzb, B, L.out, L.gb);
    if (l == 0) break;
    if ((r = gemm(m, m->dzb, L.wtb, m->dh, nullptr, nullptr, Bp, L.in, L.out, tc::kNone))) return r;
    const long long n = (long long)Bp * L.in;
    k_relu_back<<<blocks_for(n), 256, 0, m->stream>>>(m->dh, m->hf[l - 1], n, m->dzb);
  }
  return MITHRA_OK;
}

int load_input(mithra_mlp* m, const float* X, int B, int ld_x, int Bp) {
  const long long n = (long long)Bp * m->in_pad;
  k_to_bf16_padded<<<blocks_for(n), 256, 0, m->stream>>>(X, B, m->n_in, ld_x, m->xb, Bp, m->in_pad);
  return cudaGetLastError() == cudaSuccess ? MITHRA_OK : MITHRA_ERR_CUDA;
}

int check(mithra_mlp* m) {
  if (cudaStreamSynchronize(m->stream) != cudaSuccess) return MITHRA_ERR_CUDA;
  int e = 0;
  cudaMemcpy(&e, m->err, 4, cudaMemcpyDeviceToHost);
  return e ? MITHRA_ERR_STATE : MITHRA_OK;
}

}  // namespace

extern "C" {

int mithra_mlp_create(int n_in, int n_hidden, int n_layers, int n_out, int ensemble, unsigned long long seed,
                      int device, mithra_mlp** out) {
  if (!out || n_in <= 0 || n_hidden <= 0 || n_hidden % 128 || n_layers < 1 || n_out <= 0 || ensemble < 1)
    return MITHRA_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return MITHRA_ERR_CUDA;
  mithra_mlp* m = new mithra_mlp();
  m->n_in = n_in; m->n_hidden = n_hidden; m->n_layers = n_layers; m->n_out = n_out; m->ensemble = ensemble;
  m->device = device;
  m->in_pad = round_up(n_in, 128);
  m->out_pad = round_up(n_out, 128);
  cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
  cudaMalloc(&m->loss, sizeof(double));
  cudaMalloc(&m->err, sizeof(int));
  cudaMemset(m->err, 0, sizeof(int));
  std::mt19937_64 rng(seed);
  m->nets.resize(ensemble);
  for (int e = 0; e < ensemble; e++) {
    for (int l = 0; l <= n_layers; l++) {
      Layer L;
      L.in_real = (l == 0) ? n_in : n_hidden;
      L.out_real = (l == n_layers) ? n_out : n_hidden;
      L.in = (l == 0) ? m->in_pad : n_hidden;
      L.out = (l == n_layers) ? m->out_pad : n_hidden;
      const size_t nw = (size_t)L.out * L.in;
      std::vector<float> w(nw, 0.0f), b(L.out, 0.0f);
      std::vector<unsigned char> mw(nw, 0), mb(L.out, 0);
      std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / L.in_real));  // He initialisation
      for (int o = 0; o < L.out_real; o++) {
        mb[o] = 1;
        for (int i = 0; i < L.in_real; i++) {
          w[(size_t)o * L.in + i] = nd(rng);
          mw[(size_t)o * L.in + i] = 1;
        }
      }
      bool ok = true;
      float** f32[] = {&L.w, &L.mw, &L.vw, &L.gw};
      for (float** p : f32) ok = ok && cudaMalloc(p, nw * 4) == cudaSuccess && cudaMemset(*p, 0, nw * 4) == cudaSuccess;
      float** f32b[] = {&L.b, &L.mb, &L.vb, &L.gb};
      for (float** p : f32b) ok = ok && cudaMalloc(p, L.out * 4) == cudaSuccess && cudaMemset(*p, 0, L.out * 4) == cudaSuccess;
      ok = ok && cudaMalloc(&L.wb, nw * 2) == cudaSuccess && cudaMalloc(&L.wtb, nw * 2) == cudaSuccess &&
           cudaMalloc(&L.mask_w, nw) == cudaSuccess && cudaMalloc(&L.mask_b, L.out) == cudaSuccess;
      if (!ok) return MITHRA_ERR_CUDA;
      cudaMemcpy(L.w, w.data(), nw * 4, cudaMemcpyHostToDevice);
      cudaMemcpy(L.b, b.data(), L.out * 4, cudaMemcpyHostToDevice);
      cudaMemcpy(L.mask_w, mw.data(), nw, cudaMemcpyHostToDevice);
      cudaMemcpy(L.mask_b, mb.data(), L.out, cudaMemcpyHostToDevice);
      m->nets[e].push_back(L);
      refresh_bf16(m, m->nets[e].back());
    }
  }
  *out = m;
  return check(m);
}

int mithra_mlp_destroy(mithra_mlp* m) {
  if (!m) return MITHRA_ERR_ARG;
  cudaStreamSynchronize(m->stream);
  for (auto& net : m->nets)
    for (auto& L : net) {
      void* ps[] = {L.w, L.b, L.mw, L.vw, L.mb, L.vb, L.gw, L.gb, L.wb, L.wtb, L.mask_w, L.mask_b};
      for (void* p : ps) cudaFree(p);
    }
  for (auto p : m->hf) cudaFree(p);
  for (auto p : m->hb) cudaFree(p);
  for (auto p : m->hbt) cudaFree(p);
  void* ps[] = {m->xb, m->xbt, m->dh, m->dzb, m->dzbt, m->dout, m->loss, m->err};
  for (void* p : ps) cudaFree(p);
  cudaStreamDestroy(m->stream);
  delete m;
  return MITHRA_OK;
}

// One Adam step of every member on the same batch; loss_out[e] = the member's mean-squared error.
int mithra_mlp_train_step(mithra_mlp* m, const float* X, const float* Y, int batch, float lr, double* loss_out) {
  if (!m || !X || !Y || batch <= 0) return MITHRA_ERR_ARG;
  const int Bp = round_up(batch, 128);
  int r = alloc_batch(m, Bp);
  if (r) return r;
  m->step++;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.0f - std::pow(b1, (float)m->step), c2 = 1.0f - std::pow(b2, (float)m->step);
  for (int e = 0; e < m->ensemble; e++) {
    auto& net = m->nets[e];
    if ((r = load_input(m, X, batch, m->n_in, Bp))) return r;
    if ((r = forward(m, net, Bp))) return r;
    cudaMemsetAsync(m->loss, 0, sizeof(double), m->stream);
    if ((r = backward(m, net, Bp, batch, Y, m->n_out))) return r;
    for (auto& L : net) {
      const long long nw = (long long)L.out * L.in;
      k_adam<<<blocks_for(nw), 256, 0, m->stream>>>(L.w, L.gw, L.mw, L.vw, nw, lr, b1, b2, eps, c1, c2, L.mask_w);
      k_adam<<<blocks_for(L.out), 256, 0, m->stream>>>(L.b, L.gb, L.mb, L.vb, L.out, lr, b1, b2, eps, c1, c2, L.mask_b);
      refresh_bf16(m, L);
    }
    double l = 0.0;
    cudaMemcpyAsync(&l, m->loss, sizeof(double), cudaMemcpyDeviceToHost, m->stream);
    if ((r = check(m))) return r;
    if (loss_out) loss_out[e] = l / ((double)batch * m->n_out);
  }
  return MITHRA_OK;
}

// out[e][b][o] (device, FP32): every member's prediction for `batch` rows of X.
int mithra_mlp_predict(mithra_mlp* m, const float* X, int batch, float* out) {
  if (!m || !X || !out || batch <= 0) return MITHRA_ERR_ARG;
  const int Bp = round_up(batch, 128);
  int r = alloc_batch(m, Bp);
  if (r) return r;
  for (int e = 0; e < m->ensemble; e++) {
    if ((r = load_input(m, X, batch, m->n_in, Bp))) return r;
    if ((r = forward(m, m->nets[e], Bp))) return r;
    if (cudaMemcpy2DAsync(out + (size_t)e * batch * m->n_out, m->n_out * 4, m->hf[m->n_layers], m->out_pad * 4,
                          m->n_out * 4, batch, cudaMemcpyDeviceToDevice, m->stream) != cudaSuccess)
      return MITHRA_ERR_CUDA;
  }
  return check(m);
}

// Gradients of member e on a batch without updating (host buffers, real entries only, layer by
// layer: W [out_real x in_real] then b [out_real]); the loss of that batch in *loss_out.
int mithra_mlp_gradients(mithra_mlp* m, int e, const float* X, const float* Y, int batch, float* grads, double* loss_out) {
  if (!m || e < 0 || e >= m->ensemble || !X || !Y || !grads || batch <= 0) return MITHRA_ERR_ARG;
  const int Bp = round_up(batch, 128);
  int r = alloc_batch(m, Bp);
  if (r) return r;
  auto& net = m->nets[e];
  if ((r = load_input(m, X, batch, m->n_in, Bp))) return r;
  if ((r = forward(m, net, Bp))) return r;
  cudaMemsetAsync(m->loss, 0, sizeof(double), m->stream);
  if ((r = backward(m, net, Bp, batch, Y, m->n_out))) return r;
  if ((r = check(m))) return r;
  size_t w = 0;
  for (auto& L : net) {
    if (cudaMemcpy2D(grads + w, L.in_real * 4, L.gw, L.in * 4, L.in_real * 4, L.out_real, cudaMemcpyDeviceToHost) != cudaSuccess)
      return MITHRA_ERR_CUDA;
    w += (size_t)L.out_real * L.in_real;
    cudaMemcpy(grads + w, L.gb, L.out_real * 4, cudaMemcpyDeviceToHost);
    w += L.out_real;
  }
  double l = 0.0;
  cudaMemcpy(&l, m->loss, sizeof(double), cudaMemcpyDeviceToHost);
  if (loss_out) *loss_out = l / ((double)batch * m->n_out);
  return MITHRA_OK;
}

// Master weights of member e (host, same order as mithra_mlp_gradients); set or get.
int mithra_mlp_weights(mithra_mlp* m, int e, float* params, int set) {
  if (!m || e < 0 || e >= m->ensemble || !params) return MITHRA_ERR_ARG;
  size_t w = 0;
  for (auto& L : m->nets[e]) {
    if (set) {
      if (cudaMemcpy2D(L.w, L.in * 4, params + w, L.in_real * 4, L.in_real * 4, L.out_real, cudaMemcpyHostToDevice) != cudaSuccess)
        return MITHRA_ERR_CUDA;
    } else if (cudaMemcpy2D(params + w, L.in_real * 4, L.w, L.in * 4, L.in_real * 4, L.out_real, cudaMemcpyDeviceToHost) != cudaSuccess) {
      return MITHRA_ERR_CUDA;
    }
    w += (size_t)L.out_real * L.in_real;
    if (set) cudaMemcpy(L.b, params + w, L.out_real * 4, cudaMemcpyHostToDevice);
    else cudaMemcpy(params + w, L.b, L.out_real * 4, cudaMemcpyDeviceToHost);
    w += L.out_real;
    if (set) refresh_bf16(m, L);
  }
  return check(m);
}

long long mithra_mlp_param_count(const mithra_mlp* m) {
  if (!m) return -1;
  long long n = 0;
  for (auto& L : m->nets[0]) n += (long long)L.out_real * L.in_real + L.out_real;
  return n;
}

}  // extern "C"
