// BF16 GEMM on the 5th-generation tensor cores (tcgen05), FP32 accumulation in tensor memory.
//
//   C[M x N] = A[M x K] * B[N x K]^T (+ bias[N]) (then ReLU if requested)
//
// A and B are row-major with K contiguous (K-major operands).  One CTA of 128 threads computes a
// 128 x 128 tile of C: per 64-wide K block the threads copy the A and B tiles into shared memory
// in the tensor core's no-swizzle layout (8-row x 16-byte core matrices), one thread issues four
// tcgen05.mma (K = 16 each) into a 128-column TMEM accumulator and commits them to an mbarrier;
// after the last block each warp reads its 32 accumulator lanes with tcgen05.ld and applies the
// epilogue.  Every wait is bounded; a CTA that gives up records it in `err`, waits (bounded) for
// its MMAs and frees its TMEM before leaving.
//
// Requirements (checked by the host launcher): M % 128 == 0, N % 128 == 0, K % 64 == 0, 16-byte
// aligned rows.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cstdint>

namespace mithra {
namespace tc {

constexpr int BM = 128, BN = 128, BK = 64;
constexpr int kCoreBytes = 128;                   // 8 rows x 16 bytes
constexpr int kLBO = kCoreBytes;                  // next core matrix along K
constexpr int kSBO = (BK / 8) * kCoreBytes;       // next 8-row group
constexpr int kTileBytes = BM * BK * 2;           // 16 KB per operand tile
constexpr unsigned kSpinLimit = 1u << 26;

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Byte offset of element (row r, k) of a BM x BK (or BN x BK) K-major tile.
__device__ __forceinline__ uint32_t tile_offset(int r, int k) {
  return (uint32_t)((r >> 3) * kSBO + (k >> 3) * kLBO + (r & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor, no swizzle: start address, leading (K) and stride (8-row)
// byte offsets, descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((kLBO >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((kSBO >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::f16: BF16 A and B, FP32 D, both K-major, M x N.
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t* b) {
  asm volatile("mbarrier.init.shared.b64 [%0], 1;" ::"r"(saddr(b)));
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity) {
  for (unsigned it = 0; it < kSpinLimit; it++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(saddr(b)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* b) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(b))
               : "memory");
}

// 32 consecutive FP32 columns of this warp's 32 TMEM lanes: lane l of the warp gets row l.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

enum Epilogue { kNone = 0, kRelu = 1 };

__global__ void __launch_bounds__(128) k_gemm_bf16(const __nv_bfloat16* __restrict__ A, const __nv_bfloat16* __restrict__ B,
                                                   float* __restrict__ C, __nv_bfloat16* __restrict__ Cb,
                                                   const float* __restrict__ bias, int M, int N, int K, int act,
                                                   int* err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* sA = smem_raw + ((1024u - (saddr(smem_raw) & 1023u)) & 1023u);
  uint8_t* sB = sA + kTileBytes;
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_base;
  __shared__ int s_abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(saddr(&tmem_base))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(&bar);
    s_abort = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;
  const uint32_t idesc = instr_desc(BM, BN);
  uint32_t phase = 0;
  bool issued = false;

  for (int k0 = 0; k0 < K; k0 += BK) {
    // A and B tiles into the core-matrix layout: 1024 16-byte chunks per tile, 8 per thread.
#pragma unroll
    for (int v = 0; v < 8; v++) {
      const int idx = tid + v * 128, r = idx >> 3, kc = (idx & 7) * 8;
      const uint4 a = *reinterpret_cast<const uint4*>(A + (size_t)(m0 + r) * K + k0 + kc);
      const uint4 b = *reinterpret_cast<const uint4*>(B + (size_t)(n0 + r) * K + k0 + kc);
      *reinterpret_cast<uint4*>(sA + tile_offset(r, kc)) = a;
      *reinterpret_cast<uint4*>(sB + tile_offset(r, kc)) = b;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // visible to the tensor core
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int s = 0; s < BK / 16; s++)
        mma_bf16(tmem, smem_desc(saddr(sA) + s * 2 * kCoreBytes), smem_desc(saddr(sB) + s * 2 * kCoreBytes), idesc,
                 (k0 > 0 || s > 0) ? 1u : 0u);
      mma_commit(&bar);
    }
    issued = true;
    // the shared tiles are reused only after the MMAs have read them
    if (mbar_wait(&bar, phase)) phase ^= 1u;
    else s_abort = 1;  // keeps `phase`: the drain below waits for this commit
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();
    if (s_abort) break;
  }

  if (!s_abort && issued) {
    const int row = m0 + warp * 32 + lane;
    for (int c0 = 0; c0 < BN; c0 += 32) {
      float v[32];
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
      for (int i = 0; i < 32; i++) {
        const int col = n0 + c0 + i;
        float x = v[i] + (bias ? bias[col] : 0.0f);
        if (act == kRelu) x = fmaxf(x, 0.0f);
        if (C) C[(size_t)row * N + col] = x;
        if (Cb) Cb[(size_t)row * N + col] = __float2bfloat16_rn(x);
      }
    }
  } else if (s_abort && tid == 0) {
    atomicExch(err, 1);
    mbar_wait(&bar, phase);  // bounded drain of the MMAs in flight before the TMEM is freed
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tmem) : "memory");
}

// Dynamic shared memory per CTA: the two tiles plus alignment, rounded up so that at most four
// CTAs share an SM and their 4 x 128 TMEM columns fit the SM's 512 (tcgen05.alloc never waits).
constexpr size_t kGemmSmem = 56 * 1024;
static_assert(2 * kTileBytes + 1024 <= kGemmSmem, "tiles fit");

// ---- pipelined form: TMA loads, a ring of stages, one producer and one MMA thread ------------
//
// A 128 x TBN tile per CTA (TBN = 128 or 256) and K blocks of 64; the operand tiles arrive by
// cp.async.bulk.tensor with 128-byte swizzle into a ring of kStages stages: one thread issues
// the loads of a stage once the tensor core has released it (an mbarrier armed by
// tcgen05.commit), another waits for a stage's bytes to land (an mbarrier with the expected
// transaction count) and issues its four MMAs.  Loads of later stages overlap the MMAs of
// earlier ones.  Shared-memory descriptors use the 128-byte-swizzle K-major layout: rows of 128
// bytes (64 BF16), 8-row groups 1024 bytes apart, the K step of 16 advancing the start by 32 bytes.
constexpr int kStages = 4;
// A 128 x 64 tile and a TBN x 64 tile per stage (TBN = 128 or 256 columns of C per CTA).
template <int TBN>
constexpr int stage_bytes() { return kTileBytes + TBN * BK * 2; }
template <int TBN>
constexpr size_t gemm_tma_smem() { return (size_t)kStages * stage_bytes<TBN>() + 1024; }

__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
  uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;                       // leading byte offset (unused within one swizzle atom)
  d |= (uint64_t)((1024u >> 4) & 0x3FFFu) << 32;  // 8-row groups 1024 bytes apart
  d |= (uint64_t)1 << 46;                       // descriptor version
  d |= (uint64_t)2 << 61;                       // 128-byte swizzle
  return d;
}

__device__ __forceinline__ void mbar_init_count(uint64_t* b, unsigned count) {
  asm volatile("mbarrier.init.shared.b64 [%0], %1;" ::"r"(saddr(b)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared.b64 _, [%0], %1;" ::"r"(saddr(b)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(saddr(bar))
      : "memory");
}

template <int TBN>
__global__ void __launch_bounds__(128, 1) k_gemm_bf16_tma(const __grid_constant__ CUtensorMap map_a,
                                                        const __grid_constant__ CUtensorMap map_b,
                                                        float* __restrict__ C, __nv_bfloat16* __restrict__ Cb,
                                                        const float* __restrict__ bias, int M, int N, int K, int act,
                                                        int* err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* tiles = smem_raw + ((1024u - (saddr(smem_raw) & 1023u)) & 1023u);
  __shared__ __align__(8) uint64_t full[kStages], empty[kStages], done;
  __shared__ uint32_t tmem_base;
  __shared__ int s_abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * TBN;
  const int nk = K / BK;
  constexpr int kSB = stage_bytes<TBN>();

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(&tmem_base)), "n"(TBN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < kStages; s++) {
      mbar_init_count(&full[s], 1);
      mbar_init_count(&empty[s], 1);
    }
    mbar_init_count(&done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_abort = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;

  if (warp == 0 && lane == 0) {  // producer
    int issued = 0;
    volatile int* abort_flag = &s_abort;
    for (int kb = 0; kb < nk && !*abort_flag; kb++) {
      const int s = kb % kStages;
      if (kb >= kStages && !mbar_wait(&empty[s], (uint32_t)(((kb / kStages) - 1) & 1))) {
        s_abort = 1;
        break;
      }
      uint8_t* sa = tiles + s * kSB;
      mbar_expect_tx(&full[s], kSB);
      tma_load_2d(saddr(sa), &map_a, kb * BK, m0, &full[s]);
      tma_load_2d(saddr(sa + kTileBytes), &map_b, kb * BK, n0, &full[s]);
      issued = kb + 1;
    }
    // no copy may still be landing when the CTA leaves: wait (bounded) for the last stages
    for (int kb = issued > kStages ? issued - kStages : 0; kb < issued; kb++)
      if (!mbar_wait(&full[kb % kStages], (uint32_t)((kb / kStages) & 1))) s_abort = 1;
  } else if (warp == 1 && lane == 0) {  // MMA issuer
    const uint32_t idesc = instr_desc(BM, TBN);
    volatile int* abort_flag = &s_abort;
    for (int kb = 0; kb < nk && !*abort_flag; kb++) {
      const int s = kb % kStages;
      if (!mbar_wait(&full[s], (uint32_t)((kb / kStages) & 1))) {
        s_abort = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t a = saddr(tiles + s * kSB), b = a + kTileBytes;
#pragma unroll
      for (int ks = 0; ks < BK / 16; ks++)
        mma_bf16(tmem, smem_desc_sw128(a + ks * 32), smem_desc_sw128(b + ks * 32), idesc, (kb > 0 || ks > 0) ? 1u : 0u);
      mma_commit(&empty[s]);  // the stage is free once these MMAs have read it
    }
    mma_commit(&done);
  }
  // every thread: the accumulator is complete when `done` fires
  const bool ok = mbar_wait(&done, 0u);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  __syncthreads();
  if (ok && !s_abort) {
    const int row = m0 + warp * 32 + lane;
    for (int c0 = 0; c0 < TBN; c0 += 32) {
      float v[32];
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
      for (int i = 0; i < 32; i++) {
        const int col = n0 + c0 + i;
        float x = v[i] + (bias ? bias[col] : 0.0f);
        if (act == kRelu) x = fmaxf(x, 0.0f);
        if (C) C[(size_t)row * N + col] = x;
        if (Cb) Cb[(size_t)row * N + col] = __float2bfloat16_rn(x);
      }
    }
  } else if (tid == 0) {
    atomicExch(err, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(TBN) : "memory");
}

}  // namespace tc
}  // namespace mithra
