// ##################################################################
//
// checks.cu -- device-side entry points for the numerical self-tests
//
// hamstr_check_softdiv runs the integer-pipe division of softdiv.cuh on
// the GPU over arrays of operands, so tests can compare it bit for bit
// with the hardware division on the same device.
// ##################################################################
#include <cuda_runtime.h>

#include "../../include/hamstr_gpu.h"
#include "softdiv.cuh"

namespace {

__global__ void softdiv_kernel(const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ soft,
                               double* __restrict__ hard, int n)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) return;
   soft[i] = hamstr::sd::div(a[i], b[i]);
   hard[i] = a[i] / b[i];
}

}  // namespace

extern "C" int hamstr_check_softdiv(const double* a, const double* b, double* soft, double* hard, int n, void* stream)
{
   if (!a || !b || !soft || !hard || n < 0) return HAMSTR_GPU_ERR_ARG;
   if (n == 0) return HAMSTR_GPU_OK;
   softdiv_kernel<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(a, b, soft, hard, n);
   return cudaGetLastError() == cudaSuccess ? HAMSTR_GPU_OK : HAMSTR_GPU_ERR_CUDA;
}
