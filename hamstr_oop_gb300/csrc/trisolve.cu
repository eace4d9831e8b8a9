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

#include <mutex>
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

// ------------------------------------------------------------------
// Allocation-free variant.
//
// Some callers cannot allocate device memory on every call: code that runs
// in a loop beside work on other streams (cudaFree waits for the whole
// device, so the allocating entry point above stalls everything), and
// hosts whose device memory is owned by their own pool allocator with a
// fixed budget.  This variant runs the same kernel with its scratch in a
// fixed array that the library image places in device memory when it is
// loaded: every GPU that loads the library holds these 8 MiB until the
// process exits, and the call itself allocates nothing.
// ------------------------------------------------------------------
namespace {

constexpr size_t kNoAllocScratchDoubles = size_t(1) << 20;   // 8 MiB
static __device__ __align__(256) double g_tridag_scratch[kNoAllocScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
double* g_scratch_addr[kMaxDevices] = {};

// Device address of g_tridag_scratch on the current device, looked up once
// per device (host code only sees a host-side stand-in for the symbol).
int noalloc_scratch(double** out)
{
   int dev = 0;
   cudaError_t e = cudaGetDevice(&dev);
   if (e != cudaSuccess) {
      set_last_error(std::string("block_tridag4_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
      return HAMSTR_GPU_ERR_CUDA;
   }
   if (dev < 0 || dev >= kMaxDevices) {
      set_last_error("block_tridag4_noalloc: device ordinal beyond 63");
      return HAMSTR_GPU_ERR_ARG;
   }
   std::lock_guard<std::mutex> lock(g_scratch_mutex);
   if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_tridag_scratch);
      if (e != cudaSuccess || !p) {
         set_last_error(std::string("block_tridag4_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
         return HAMSTR_GPU_ERR_CUDA;
      }
      g_scratch_addr[dev] = static_cast<double*>(p);
   }
   *out = g_scratch_addr[dev];
   return HAMSTR_GPU_OK;
}

}  // namespace

extern "C" int hamstr_gpu_block_tridag4_noalloc(int nlines, int N, int periodic, const double* A, const double* B,
                                                const double* C, double* F, void* stream)
{
   int st = block_tridag_check(nlines, N, periodic, A, B, C, F);
   if (st || nlines == 0) return st;
   // per-line need compared against the per-line share, so no product of
   // two large ints can wrap past the limit
   const size_t per_line = (size_t)kFacRec * N + 16;
   if (per_line > kNoAllocScratchDoubles / (size_t)nlines) {
      set_last_error("block_tridag4_noalloc: nlines*(80*N+16) with nlines = " + std::to_string(nlines) +
                     ", N = " + std::to_string(N) + " exceeds the fixed scratch of " +
                     std::to_string(kNoAllocScratchDoubles) + " doubles");
      return HAMSTR_GPU_ERR_ARG;
   }
   double* scratch = nullptr;
   st = noalloc_scratch(&scratch);
   if (st) return st;
   // every scratch value the kernel reads it has written earlier in the same
   // launch, so nothing needs clearing between calls
   return block_tridag_launch(nlines, N, periodic, A, B, C, F, scratch, (cudaStream_t)stream);
}
