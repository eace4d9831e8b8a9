// ##################################################################
//
// forces.cu -- pressure force and moment on the wall faces
//
// A project addition (the reference computes no forces; its wall faces
// are the bFaces list, preprocess.cpp:180-184).  Each wall face gets the
// adjacent cell's pressure times its normal (dy, -dx), which points from
// the fluid cell into the body; the moment is taken about (0.25, 0).  The
// per-face terms are formed in parallel and summed by one thread in
// ascending face order, so the sums equal a serial CPU loop bit for bit.
// One block per instance of a batched handle.
// ##################################################################
#include "device_state.h"

namespace hamstr {

namespace {

__global__ void __launch_bounds__(256) forces_kernel(const double* __restrict__ q, const int* __restrict__ wall_cell,
                                                     const double4* __restrict__ geo, const int* __restrict__ wall0,
                                                     double gm1, double* __restrict__ scr, double* __restrict__ out)
{
   const int k0 = wall0[blockIdx.x], k1 = wall0[blockIdx.x + 1];
   for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
      const double* s = q + 4 * (size_t)wall_cell[k];
      const double4 g = geo[k];   // nx, ny, face midpoint x, y
      const double p = gm1 * (s[3] - 0.5 * (s[1] * s[1] + s[2] * s[2]) / s[0]);
      const double fx = p * g.x;
      const double fy = p * g.y;
      scr[3 * k] = fx;
      scr[3 * k + 1] = fy;
      scr[3 * k + 2] = (g.z - 0.25) * fy - g.w * fx;
   }
   __syncthreads();
   if (threadIdx.x == 0) {
      double Fx = 0.0, Fy = 0.0, M = 0.0;
      for (int k = k0; k < k1; k++) {
         Fx = Fx + scr[3 * k];
         Fy = Fy + scr[3 * k + 1];
         M = M + scr[3 * k + 2];
      }
      out[3 * blockIdx.x] = Fx;
      out[3 * blockIdx.x + 1] = Fy;
      out[3 * blockIdx.x + 2] = M;
   }
}

}  // namespace

void launch_forces(const double* q, const int* wall_cell, const double4* geo, const int* wall0, int ninst,
                   double gm1, double* scr, double* out, cudaStream_t st)
{
   forces_kernel<<<ninst, 256, 0, st>>>(q, wall_cell, geo, wall0, gm1, scr, out);
}

}  // namespace hamstr
