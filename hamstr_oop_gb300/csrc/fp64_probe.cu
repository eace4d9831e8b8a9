// ##################################################################
//
// fp64_probe.cu -- FP64 issue rate and latency of the current GPU
//
// Prints the figures the line-solve design is built on: FP64 lane-op and
// warp-instruction throughput with 1..32 active lanes, dependent-op
// latency, division and square-root throughput, and the FP32 rate for
// comparison.  Pure register arithmetic with fixed trip counts.
// Usage: hamstr_fp64_probe
// ##################################################################
#include <cuda_runtime.h>

#include <cstdio>

#define CK(x)                                                                                   \
   do {                                                                                         \
      cudaError_t e_ = (x);                                                                     \
      if (e_ != cudaSuccess) {                                                                  \
         std::printf("CUDA error %s at line %d\n", cudaGetErrorString(e_), __LINE__);          \
         return 1;                                                                              \
      }                                                                                         \
   } while (0)

__global__ void add_lanes(double* out, int iters, double s, int lanes)
{
   if ((int)(threadIdx.x & 31) >= lanes) return;
   double a0 = threadIdx.x * 1e-3, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6,
          a7 = a0 + 7;
   for (int i = 0; i < iters; i++) {
      a0 = __dadd_rn(a0, s); a1 = __dadd_rn(a1, s); a2 = __dadd_rn(a2, s); a3 = __dadd_rn(a3, s);
      a4 = __dadd_rn(a4, s); a5 = __dadd_rn(a5, s); a6 = __dadd_rn(a6, s); a7 = __dadd_rn(a7, s);
   }
   if (a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7 == 12345.678) out[0] = a0;
}

__global__ void fma_full(double* out, int iters, double s)
{
   double a0 = threadIdx.x * 1e-3 + 1, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5,
          a6 = a0 + 6, a7 = a0 + 7;
   for (int i = 0; i < iters; i++) {
      a0 = __fma_rn(a0, s, s); a1 = __fma_rn(a1, s, s); a2 = __fma_rn(a2, s, s); a3 = __fma_rn(a3, s, s);
      a4 = __fma_rn(a4, s, s); a5 = __fma_rn(a5, s, s); a6 = __fma_rn(a6, s, s); a7 = __fma_rn(a7, s, s);
   }
   if (a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7 == 12345.678) out[0] = a0;
}

__global__ void div_full(double* out, int iters, double s)
{
   double a0 = threadIdx.x * 1e-3 + 1, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
   for (int i = 0; i < iters; i++) { a0 = s / a0; a1 = s / a1; a2 = s / a2; a3 = s / a3; }
   if (a0 + a1 + a2 + a3 == 12345.678) out[0] = a0;
}

__global__ void sqrt_full(double* out, int iters, double s)
{
   double a0 = threadIdx.x * 1e-3 + 1, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
   for (int i = 0; i < iters; i++) { a0 = sqrt(a0 + s); a1 = sqrt(a1 + s); a2 = sqrt(a2 + s); a3 = sqrt(a3 + s); }
   if (a0 + a1 + a2 + a3 == 12345.678) out[0] = a0;
}

__global__ void fadd_full(double* out, int iters, float s)
{
   float a0 = threadIdx.x * 1e-3f, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6,
         a7 = a0 + 7;
   for (int i = 0; i < iters; i++) {
      a0 = __fadd_rn(a0, s); a1 = __fadd_rn(a1, s); a2 = __fadd_rn(a2, s); a3 = __fadd_rn(a3, s);
      a4 = __fadd_rn(a4, s); a5 = __fadd_rn(a5, s); a6 = __fadd_rn(a6, s); a7 = __fadd_rn(a7, s);
   }
   if (a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7 == 12345.678f) out[0] = a0;
}

__global__ void lat_add(double* out, long long* cyc, int iters, double s)
{
   double a = threadIdx.x;
   const long long t0 = clock64();
   for (int i = 0; i < iters; i++) { a = __dadd_rn(a, s); a = __dadd_rn(a, s); a = __dadd_rn(a, s); a = __dadd_rn(a, s); }
   const long long t1 = clock64();
   if (threadIdx.x == 0) { cyc[0] = t1 - t0; out[1] = a; }
}

int main()
{
   int dev = 0, nsm = 0, clk = 0;
   CK(cudaGetDevice(&dev));
   CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
   CK(cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, dev));
   cudaDeviceProp prop;
   CK(cudaGetDeviceProperties(&prop, dev));
   std::printf("device %s, %d SMs, max SM clock %d MHz\n", prop.name, nsm, clk / 1000);
   double* out;
   long long* cyc;
   CK(cudaMalloc(&out, 64));
   CK(cudaMalloc(&cyc, 64));
   cudaEvent_t e0, e1;
   CK(cudaEventCreate(&e0));
   CK(cudaEventCreate(&e1));
   const int blocks = nsm * 8, thr = 256;
   auto timed = [&](auto launch) -> float {
      float ms = 0.f;
      for (int rep = 0; rep < 2; rep++) {
         cudaEventRecord(e0);
         launch();
         cudaEventRecord(e1);
         cudaEventSynchronize(e1);
         cudaEventElapsedTime(&ms, e0, e1);
      }
      return ms;
   };
   for (int lanes : {1, 4, 16, 32}) {
      const int iters = 4000;
      const float ms = timed([&] { add_lanes<<<blocks, thr>>>(out, iters, 1e-9, lanes); });
      const double warp_instr = (double)blocks * (thr / 32) * iters * 8;
      std::printf("DADD  %2d active lanes: %7.1f G lane-op/s  %6.2f G warp-instr/s\n", lanes,
                  warp_instr * lanes / ms / 1e6, warp_instr / ms / 1e6);
   }
   {
      const int iters = 4000;
      const float ms = timed([&] { fma_full<<<blocks, thr>>>(out, iters, 0.5); });
      std::printf("DFMA  32 lanes: %7.1f G op/s\n", (double)blocks * thr * iters * 8 / ms / 1e6);
   }
   {
      const int iters = 1000;
      const float ms = timed([&] { div_full<<<blocks, thr>>>(out, iters, 1.25); });
      std::printf("DDIV  32 lanes: %7.1f G op/s\n", (double)blocks * thr * iters * 4 / ms / 1e6);
   }
   {
      const int iters = 1000;
      const float ms = timed([&] { sqrt_full<<<blocks, thr>>>(out, iters, 0.25); });
      std::printf("DSQRT 32 lanes: %7.1f G op/s\n", (double)blocks * thr * iters * 4 / ms / 1e6);
   }
   {
      const int iters = 100000;
      const float ms = timed([&] { fadd_full<<<blocks, thr>>>(out, iters, 1e-3f); });
      std::printf("FADD  32 lanes: %7.1f G op/s\n", (double)blocks * thr * iters * 8 / ms / 1e6);
   }
   for (int warps : {1, 2, 4, 8}) {
      const int iters = 10000;
      lat_add<<<1, 32 * warps>>>(out, cyc, iters, 1e-9);
      CK(cudaDeviceSynchronize());
      long long h = 0;
      CK(cudaMemcpy(&h, cyc, sizeof(h), cudaMemcpyDeviceToHost));
      std::printf("dependent DADD, %d warp(s) in one block: %.1f cycles per op (warp 0)\n", warps,
                  (double)h / (4.0 * iters));
   }
   CK(cudaGetLastError());
   return 0;
}
