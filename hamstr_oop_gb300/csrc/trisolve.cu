// ##################################################################
//
// trisolve.cu -- batched 4x4 block-tridiagonal solves on device arrays
//
// The reference's TRISOLVER::blockTridag4 (triSolvers.cpp:769-847) and
// blockTridagPeriodic4 (triSolvers.cpp:850-1046) as a batched entry point:
// one warp per line, factor_line + solve_line of line_solve.cuh, so each
// line's solution is bit-identical to one reference call.
// ##################################################################
#include <cuda_runtime.h>

#include <string>

#include "../../include/hamstr_gpu.h"
#include "line_solve.cuh"

namespace hamstr {
void set_last_error(const std::string& m);
}

namespace {

using namespace hamstr;

__global__ void __launch_bounds__(32) block_tridag_kernel(int N, int periodic, const double* __restrict__ A,
                                                          const double* __restrict__ B, const double* __restrict__ C,
                                                          double* __restrict__ F, double* __restrict__ scratch)
{
   const size_t line = blockIdx.x;
   const size_t nb = (size_t)N * 16;
   double* fac = scratch + line * ((size_t)kFacRec * N + 16);
   double* facN = fac + (size_t)kFacRec * N;
   const bool per = periodic != 0;
   factor_line(A + line * nb, B + line * nb, C + line * nb, 16, N, per, fac, facN, threadIdx.x);
   __syncwarp();
   solve_line(fac, facN, N, per, F + line * (size_t)N * 4, threadIdx.x);
}

}  // namespace

namespace hamstr {

// validation shared by the block-tridiagonal entry points
int block_tridag_check(int nlines, int N, int periodic, const double* A, const double* B, const double* C,
                       const double* F)
{
   if (nlines < 0 || N < 1 || (periodic && N < 2) || (periodic != 0 && periodic != 1)) {
      set_last_error("block_tridag4: need nlines >= 0, N >= 1 (open) or N >= 2 (periodic)");
      return HAMSTR_GPU_ERR_ARG;
   }
   if (nlines > 0 && (!A || !B || !C || !F)) {
      set_last_error("block_tridag4: null array");
      return HAMSTR_GPU_ERR_ARG;
   }
   return HAMSTR_GPU_OK;
}

int block_tridag_launch(int nlines, int N, int periodic, const double* A, const double* B, const double* C,
                        double* F, double* scratch, cudaStream_t st)
{
   if (nlines == 0) return HAMSTR_GPU_OK;
   block_tridag_kernel<<<nlines, 32, 0, st>>>(N, periodic, A, B, C, F, scratch);
   const cudaError_t e = cudaGetLastError();
   if (e != cudaSuccess) {
      set_last_error(std::string("block_tridag4 launch: ") + cudaGetErrorString(e));
      return HAMSTR_GPU_ERR_CUDA;
   }
   return HAMSTR_GPU_OK;
}

}  // namespace hamstr

extern "C" int hamstr_gpu_block_tridag4(int nlines, int N, int periodic, const double* A, const double* B,
                                        const double* C, double* F, void* stream)
{
   int st = block_tridag_check(nlines, N, periodic, A, B, C, F);
   if (st || nlines == 0) return st;
   const cudaStream_t s = (cudaStream_t)stream;
   double* scratch = nullptr;
   const size_t bytes = (size_t)nlines * ((size_t)kFacRec * N + 16) * sizeof(double);
   cudaError_t e = cudaMalloc((void**)&scratch, bytes);
   if (e != cudaSuccess) {
      set_last_error(std::string("block_tridag4 scratch: ") + cudaGetErrorString(e));
      return e == cudaErrorMemoryAllocation ? HAMSTR_GPU_ERR_NOMEM : HAMSTR_GPU_ERR_CUDA;
   }
   st = block_tridag_launch(nlines, N, periodic, A, B, C, F, scratch, s);
   e = cudaStreamSynchronize(s);
   cudaFree(scratch);
   if (st) return st;
   if (e != cudaSuccess) {
      set_last_error(std::string("block_tridag4: ") + cudaGetErrorString(e));
      return HAMSTR_GPU_ERR_CUDA;
   }
   return HAMSTR_GPU_OK;
}
