// ##################################################################
//
// checks.cu -- device-side entry points for the numerical self-tests
//
// hamstr_check_softdiv runs the integer-pipe division of softdiv.cuh on
// the GPU over arrays of operands, so tests can compare it bit for bit
// with the hardware division on the same device.  hamstr_check_row_wait
// runs the row count a following line solve waits on (line_solve.cuh
// publish_rows / wait_rows) with a count that is never published, so
// tests see the bounded wait give up and the kernel end.
// ##################################################################
#include <cuda_runtime.h>

#include "../../include/hamstr_gpu.h"
#include "softdiv.cuh"
#include "line_solve.cuh"

namespace {

__global__ void softdiv_kernel(const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ soft,
                               double* __restrict__ hard, int n)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) return;
   soft[i] = hamstr::sd::div(a[i], b[i]);
   hard[i] = a[i] / b[i];
}

__global__ void row_wait_kernel(int* out)
{
   __shared__ int prog;
   const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
   if (threadIdx.x == 0) prog = 0;
   __syncthreads();
   if (w == 0) {
      hamstr::publish_rows(&prog, 3, lane);
   } else {
      const bool a = hamstr::wait_rows(&prog, 1);
      const bool b = hamstr::wait_rows(&prog, 3);
      const bool c = hamstr::wait_rows(&prog, 4);   // never published: gives up at the bound
      if (lane == 0) {
         out[0] = a ? 1 : 0;
         out[1] = b ? 1 : 0;
         out[2] = c ? 1 : 0;
      }
   }
}

}  // namespace

extern "C" int hamstr_check_row_wait(int* out, void* stream)
{
   if (!out) return HAMSTR_GPU_ERR_ARG;
   row_wait_kernel<<<1, 64, 0, static_cast<cudaStream_t>(stream)>>>(out);
   return cudaGetLastError() == cudaSuccess ? HAMSTR_GPU_OK : HAMSTR_GPU_ERR_CUDA;
}

extern "C" int hamstr_check_softdiv(const double* a, const double* b, double* soft, double* hard, int n, void* stream)
{
   if (!a || !b || !soft || !hard || n < 0) return HAMSTR_GPU_ERR_ARG;
   if (n == 0) return HAMSTR_GPU_OK;
   softdiv_kernel<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(a, b, soft, hard, n);
   return cudaGetLastError() == cudaSuccess ? HAMSTR_GPU_OK : HAMSTR_GPU_ERR_CUDA;
}
