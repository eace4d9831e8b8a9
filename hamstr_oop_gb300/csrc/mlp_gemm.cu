// ##################################################################
//
// mlp_gemm.cu -- BF16 tensor-core GEMM for the learned warm start
//
// C[M x N] = A[M x K] * B[N x K]^T, A and B BF16 with K contiguous,
// FP32 accumulation in tensor memory, on the 5th-generation tensor cores:
//   * TMA (cp.async.bulk.tensor) brings 128 x 64 tiles of A and BN x 64
//     tiles of B into shared memory with 128-byte swizzling, STAGES deep,
//     each stage completing an mbarrier by transaction count;
//   * one thread issues tcgen05.mma (kind::f16, M = 128, N = BN, K = 16)
//     per 16-wide slice, accumulating in TMEM, and tcgen05.commit frees
//     the stage for the producer;
//   * all four warps read the accumulator with tcgen05.ld (warp w owns
//     TMEM lanes 32w..32w+31, one output row per thread) and apply the
//     layer's epilogue: bias + GELU for hidden layers (storing the
//     pre-activation, the activation and its transpose), bias for the
//     output layer, GELU' for the backward pass, or plain FP32 partial
//     sums for the split-K weight gradients.
// Every wait is bounded (about two seconds); a timeout raises a flag in
// the caller's error word and the CTA still frees its tensor memory.
// ##################################################################
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cmath>
#include <cstdint>
#include <mutex>
#include <string>

#include "mlp.h"

namespace hamstr {
void set_last_error(const std::string& m);

namespace mlp {

namespace {

constexpr int BM = 128, BK = 64, STAGES = 4;
constexpr int kThreads = 128;
constexpr unsigned long long kWaitNs = 2000000000ull;   // bounded waits: 2 s

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long global_ns()
{
   unsigned long long t;
   asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
   return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
   asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
   asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// true when phase `parity` of the barrier has completed; false after the
// time limit
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
   const unsigned long long t0 = global_ns();
   for (;;) {
      uint32_t ok;
      asm volatile(
          "{\n\t.reg .pred p;\n\t"
          "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
          "selp.u32 %0, 1, 0, p;\n\t}"
          : "=r"(ok)
          : "r"(bar), "r"(parity)
          : "memory");
      if (ok) return true;
      if (global_ns() - t0 > kWaitNs) return false;
   }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int c0, int c1, uint32_t bar)
{
   asm volatile(
       "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
           dst),
       "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(bar)
       : "memory");
}

// shared-memory matrix descriptor: K-major tile with 128-byte swizzling,
// 8-row atoms of 1024 bytes (stride byte offset), version 1
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr)
{
   uint64_t d = 0;
   d |= (uint64_t)((addr & 0x3FFFF) >> 4);          // start address
   d |= (uint64_t)1 << 16;                           // leading byte offset (unused for swizzled K-major)
   d |= (uint64_t)(1024 >> 4) << 32;                 // stride byte offset
   d |= (uint64_t)1 << 46;                           // descriptor version
   d |= (uint64_t)2 << 61;                           // 128-byte swizzle
   return d;
}

// instruction descriptor: kind::f16 with BF16 A and B, FP32 D, both
// K-major, M = 128, N = BN
__host__ __device__ constexpr uint32_t instr_desc(int bn)
{
   return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(bn >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accum)
{
   asm volatile(
       "{\n\t.reg .pred p;\n\t"
       "setp.ne.b32 p, %4, 0;\n\t"
       "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
       "l"(a), "l"(b), "r"(idesc), "r"(accum)
       : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
   asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
   uint32_t r[16];
   asm volatile(
       "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
       "[%16];"
       : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
         "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
       : "r"(taddr));
   asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
   for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z)
{
   return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

struct Epi {
   int mode;
   float* C;                 // EPI_F32 (+ split * M * N), EPI_OUT (ldc = n_out)
   int n_out;                // EPI_OUT: columns written
   const float* bias;        // EPI_HIDDEN, EPI_OUT
   float* Z;                 // EPI_HIDDEN: pre-activation [M][N]
   const float* Zin;         // EPI_BWD: pre-activation of this layer [M][N]
   __nv_bfloat16* H;         // EPI_HIDDEN: GELU(Z) / EPI_BWD: dZ, [M][N]
   __nv_bfloat16* Ht;        // transposed copy [N][M]
   int* err;
};

template <int BN>
__global__ void __launch_bounds__(kThreads, 1)
    gemm_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, int M, int N,
                int kb_per_split, int nkb, Epi ep)
{
   extern __shared__ __align__(1024) unsigned char smem_raw[];
   // 1024-byte aligned stage buffers (the 128-byte swizzle atom)
   unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
   constexpr int A_BYTES = BM * BK * 2, B_BYTES = BN * BK * 2, STAGE = A_BYTES + B_BYTES;
   uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE);   // full[S], empty[S], done
   __shared__ uint32_t tmem_base;
   __shared__ int failed;

   const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
   const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
   const int kb0 = blockIdx.z * kb_per_split;
   const int kb1 = min(nkb, kb0 + kb_per_split);
   const int nk = kb1 - kb0;

   const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + STAGES), done = smem_u32(bars + 2 * STAGES);
   if (threadIdx.x == 0) {
      failed = 0;
      for (int s = 0; s < STAGES; s++) {
         mbar_init(full0 + 8 * s, 1);
         mbar_init(empty0 + 8 * s, 1);
      }
      mbar_init(done, 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
   }
   constexpr uint32_t kCols = BN < 32 ? 32 : BN;   // TMEM columns: a power of two >= 32
   if (warp == 2) {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                   "r"(kCols)
                   : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
   }
   asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
   __syncthreads();
   asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
   const uint32_t tmem = tmem_base;

   if (warp == 0 && lane == 0) {
      // producer: TMA loads of A and B tiles into the stages
      for (int i = 0; i < nk; i++) {
         const int s = i % STAGES, round = i / STAGES;
         if (round > 0 && !mbar_wait(empty0 + 8 * s, (round - 1) & 1)) {
            failed = 1;
            break;
         }
         const uint32_t sa = smem_u32(smem + s * STAGE), sb = sa + A_BYTES;
         mbar_expect_tx(full0 + 8 * s, STAGE);
         tma_load_2d(sa, &mapA, (kb0 + i) * BK, m0, full0 + 8 * s);
         tma_load_2d(sb, &mapB, (kb0 + i) * BK, n0, full0 + 8 * s);
      }
   } else if (warp == 1 && lane == 0) {
      // MMA issuer: four K = 16 slices per 64-wide stage
      const uint32_t idesc = instr_desc(BN);
      for (int i = 0; i < nk; i++) {
         const int s = i % STAGES, round = i / STAGES;
         if (!mbar_wait(full0 + 8 * s, round & 1)) {
            failed = 1;
            break;
         }
         asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
         const uint32_t sa = smem_u32(smem + s * STAGE), sb = sa + A_BYTES;
#pragma unroll
         for (int kk = 0; kk < BK / 16; kk++)
            mma_bf16(tmem, smem_desc(sa + 32 * kk), smem_desc(sb + 32 * kk), idesc, (i > 0 || kk > 0) ? 1u : 0u);
         mma_commit(empty0 + 8 * s);   // the stage is free once these MMAs have read it
      }
      mma_commit(done);                // the accumulator is complete
   }
   __syncwarp();

   // epilogue: every warp waits for the accumulator
   const bool ok = mbar_wait(done, 0);
   asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
   if (!ok || failed) {
      if (threadIdx.x == 0) atomicOr(ep.err, 1);
   } else {
      const int row = 32 * warp + lane, grow = m0 + row;
      const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16);
#pragma unroll 1
      for (int c = 0; c < BN; c += 16) {
         float v[16];
         tmem_ld16(taddr + c, v);
         const int gc = n0 + c;
         if (ep.mode == EPI_F32) {
            float* out = ep.C + (size_t)blockIdx.z * M * N + (size_t)grow * N + gc;
#pragma unroll
            for (int j = 0; j < 16; j += 4) *reinterpret_cast<float4*>(out + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
         } else if (ep.mode == EPI_OUT) {
#pragma unroll
            for (int j = 0; j < 16; j++)
               if (gc + j < ep.n_out) ep.C[(size_t)grow * ep.n_out + gc + j] = v[j] + ep.bias[gc + j];
         } else if (ep.mode == EPI_HIDDEN) {
#pragma unroll
            for (int j = 0; j < 16; j++) {
               const float z = v[j] + ep.bias[gc + j];
               const __nv_bfloat16 h = __float2bfloat16_rn(gelu(z));
               ep.Z[(size_t)grow * N + gc + j] = z;
               ep.H[(size_t)grow * N + gc + j] = h;
               ep.Ht[(size_t)(gc + j) * M + grow] = h;
            }
         } else {   // EPI_BWD: dZ = dH * GELU'(Z)
#pragma unroll
            for (int j = 0; j < 16; j++) {
               const float z = ep.Zin[(size_t)grow * N + gc + j];
               const __nv_bfloat16 g = __float2bfloat16_rn(v[j] * gelu_grad(z));
               ep.H[(size_t)grow * N + gc + j] = g;
               ep.Ht[(size_t)(gc + j) * M + grow] = g;
            }
         }
      }
   }
   asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
   __syncthreads();
   if (warp == 2)
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols) : "memory");
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no
// link-time dependency on the driver library)
PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
   static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
   static std::once_flag once;
   std::call_once(once, [] {
      void* p = nullptr;
      cudaDriverEntryPointQueryResult q;
      if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
          q == cudaDriverEntryPointSuccess)
         fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
   });
   return fn;
}

// rows x k BF16 matrix (k contiguous), box of box_rows x 64
bool make_map(CUtensorMap* map, const void* base, int rows, int k, int box_rows)
{
   auto fn = encode_fn();
   if (!fn) return false;
   cuuint64_t dims[2] = {(cuuint64_t)k, (cuuint64_t)rows};
   cuuint64_t strides[1] = {(cuuint64_t)k * 2};
   cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
   cuuint32_t estr[2] = {1, 1};
   return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN>
int launch(const GemmArgs& a, cudaStream_t st)
{
   CUtensorMap ma, mb;
   if (!make_map(&ma, a.A, a.M, a.K, BM) || !make_map(&mb, a.B, a.N, a.K, BN)) {
      set_last_error("mlp gemm: tensor map encoding failed");
      return HAMSTR_GPU_ERR_CUDA;
   }
   constexpr int smem = STAGES * (BM * BK * 2 + BN * BK * 2) + 1024 + 2 * STAGES * 8 + 8 + 64;
   static bool configured = false;
   if (!configured) {
      if (cudaFuncSetAttribute(gemm_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) {
         set_last_error("mlp gemm: shared memory request refused");
         return HAMSTR_GPU_ERR_CUDA;
      }
      configured = true;
   }
   const int nkb = a.K / BK;
   const int splits = a.splits < 1 ? 1 : (a.splits > nkb ? nkb : a.splits);
   const int per = (nkb + splits - 1) / splits;
   const int gz = (nkb + per - 1) / per;   // every split has at least one K block
   Epi ep;
   ep.mode = a.mode;
   ep.C = a.C;
   ep.n_out = a.n_out;
   ep.bias = a.bias;
   ep.Z = a.Z;
   ep.Zin = a.Zin;
   ep.H = a.H;
   ep.Ht = a.Ht;
   ep.err = a.err;
   dim3 grid(a.M / BM, a.N / BN, gz);
   gemm_kernel<BN><<<grid, kThreads, smem, st>>>(ma, mb, a.M, a.N, per, nkb, ep);
   const cudaError_t e = cudaGetLastError();
   if (e != cudaSuccess) {
      set_last_error(std::string("mlp gemm launch: ") + cudaGetErrorString(e));
      return HAMSTR_GPU_ERR_CUDA;
   }
   return HAMSTR_GPU_OK;
}

}  // namespace

int gemm_splits(int K, int splits)
{
   const int nkb = K / BK;
   splits = splits < 1 ? 1 : (splits > nkb ? nkb : splits);
   const int per = (nkb + splits - 1) / splits;
   return (nkb + per - 1) / per;
}

int gemm(const GemmArgs& a, cudaStream_t st)
{
   if (!a.A || !a.B || !a.err || a.M <= 0 || a.N <= 0 || a.K <= 0 || a.M % BM || a.K % BK ||
       ((uintptr_t)a.A & 15) || ((uintptr_t)a.B & 15)) {
      set_last_error("mlp gemm: need M % 128 == 0, K % 64 == 0, 16-byte aligned operands");
      return HAMSTR_GPU_ERR_ARG;
   }
   if (a.mode == EPI_F32 && !a.C) return HAMSTR_GPU_ERR_ARG;
   if (a.mode == EPI_OUT && (!a.C || !a.bias || a.n_out <= 0 || a.n_out > a.N)) return HAMSTR_GPU_ERR_ARG;
   if (a.mode == EPI_HIDDEN && (!a.bias || !a.Z || !a.H || !a.Ht)) return HAMSTR_GPU_ERR_ARG;
   if (a.mode == EPI_BWD && (!a.Zin || !a.H || !a.Ht)) return HAMSTR_GPU_ERR_ARG;
   if (a.mode != EPI_F32 && a.splits > 1) return HAMSTR_GPU_ERR_ARG;
   switch (a.N) {
      case 16: return launch<16>(a, st);
      case 64: return launch<64>(a, st);
      case 128: return launch<128>(a, st);
      case 256: return launch<256>(a, st);
      default:
         if (a.N % 256 == 0) return launch<256>(a, st);
         set_last_error("mlp gemm: N must be 16, 64, 128 or a multiple of 256");
         return HAMSTR_GPU_ERR_ARG;
   }
}

}  // namespace mlp
}  // namespace hamstr
