// ##################################################################
//
// mlp.h -- kernels of the learned warm start (BF16 tensor cores)
// ##################################################################
#ifndef HAMSTR_GPU_MLP_H
#define HAMSTR_GPU_MLP_H

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/hamstr_gpu.h"

namespace hamstr {
namespace mlp {

// epilogues of the tensor-core GEMM
enum {
   EPI_F32 = 0,     // C (+ split * M * N) = A B^T, FP32
   EPI_HIDDEN = 1,  // Z = A B^T + bias; H = bf16(GELU(Z)), Ht = H^T
   EPI_OUT = 2,     // C[:, :n_out] = (A B^T + bias)[:, :n_out], FP32, row stride n_out
   EPI_BWD = 3,     // H = bf16(A B^T * GELU'(Zin)), Ht = H^T
};

struct GemmArgs {
   const __nv_bfloat16* A = nullptr;   // [M][K]
   const __nv_bfloat16* B = nullptr;   // [N][K]
   int M = 0, N = 0, K = 0, splits = 1, mode = EPI_F32, n_out = 0;
   float* C = nullptr;
   const float* bias = nullptr;
   float* Z = nullptr;
   const float* Zin = nullptr;
   __nv_bfloat16* H = nullptr;
   __nv_bfloat16* Ht = nullptr;
   int* err = nullptr;                  // device word: 1 after a timed-out wait
};

// number of K splits actually used for a request (each split >= one 64-wide block)
int gemm_splits(int K, int splits);
int gemm(const GemmArgs& a, cudaStream_t st);

}  // namespace mlp
}  // namespace hamstr
#endif
