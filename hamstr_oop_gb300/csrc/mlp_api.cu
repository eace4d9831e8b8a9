// ##################################################################
//
// mlp_api.cu -- C ABI of the warm-start network's kernels
// ##################################################################
#include "mlp.h"

using namespace hamstr;

extern "C" int hamstr_mlp_gemm(const void* A, const void* B, int M, int N, int K, int splits, float* C, int* err,
                               void* stream)
{
   mlp::GemmArgs a;
   a.A = static_cast<const __nv_bfloat16*>(A);
   a.B = static_cast<const __nv_bfloat16*>(B);
   a.M = M;
   a.N = N;
   a.K = K;
   a.splits = splits;
   a.mode = mlp::EPI_F32;
   a.C = C;
   a.err = err;
   return mlp::gemm(a, static_cast<cudaStream_t>(stream));
}
