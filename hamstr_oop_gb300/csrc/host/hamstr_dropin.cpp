// ##################################################################
//
// hamstr_dropin.cpp -- the reference's per-face and per-line functions
// over host arrays, run on the GPU
//
// SOLVER::fluxRoe2D / jacobianRoe2D (solver.h:46,49), RECONSTRUCTION::*
// (reconstruction.h:19-108) and TRISOLVER::blockTridag4 /
// blockTridagPeriodic4 (triSolvers.h:40,44) with the reference's
// signatures.  Each call packs the caller's pointer arrays into one
// contiguous block, copies it to a device buffer kept per host thread,
// runs the function-level entry point of include/hamstr_gpu.h on the
// default stream and copies the results back into the caller's arrays.
// ##################################################################
#include "hamstr_host.h"

#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

namespace {

using hamstr::Error;

void check(int st)
{
   if (st != HAMSTR_GPU_OK) {
      std::string m = hamstr_gpu_strerror(st);
      const char* d = hamstr_gpu_last_error();
      if (d && *d) m += std::string(": ") + d;
      throw Error(st, m);
   }
}

void cuda_check(cudaError_t e, const char* what)
{
   if (e != cudaSuccess) throw Error(HAMSTR_GPU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// grow-only device buffer of this host thread (released at thread exit)
struct DeviceBuffer {
   double* p = nullptr;
   size_t n = 0;
   ~DeviceBuffer()
   {
      if (p) cudaFree(p);
   }
   double* get(size_t want)
   {
      if (want > n) {
         if (p) cudaFree(p);
         p = nullptr;
         n = 0;
         cuda_check(cudaMalloc((void**)&p, want * sizeof(double)), "device buffer");
         n = want;
      }
      return p;
   }
};

thread_local DeviceBuffer t_buf;

// the host block <-> device, synchronously on the default stream
double* to_device(const std::vector<double>& h)
{
   double* d = t_buf.get(h.size() ? h.size() : 1);
   cuda_check(cudaMemcpy(d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice), "copy in");
   return d;
}

void from_device(std::vector<double>& h, const double* d)
{
   cuda_check(cudaDeviceSynchronize(), "function-level call");
   cuda_check(cudaMemcpy(h.data(), d, h.size() * sizeof(double), cudaMemcpyDeviceToHost), "copy out");
}

// rows [0, imax) of a double** line array into / out of a flat block
void pack(std::vector<double>& h, size_t off, double** rows, int imax, int nq)
{
   for (int i = 0; i < imax; i++) std::memcpy(h.data() + off + (size_t)i * nq, rows[i], nq * sizeof(double));
}

void unpack(const std::vector<double>& h, size_t off, double** rows, int i0, int i1, int nq)
{
   for (int i = i0; i <= i1; i++) std::memcpy(rows[i], h.data() + off + (size_t)i * nq, nq * sizeof(double));
}

// MUSCL and MUSCL_DERIV: the entries computed on the GPU (see the header)
int muscl_last(int ie, int imax, double qt) { return (qt != 0.0 && ie == imax - 1) ? imax - 2 : ie; }

}  // namespace

// ------------------------------------------------------------------
// SOLVER per-face methods
// ------------------------------------------------------------------
void SOLVER::fluxRoe2D(double* nxyz, double* ql, double* qr, double* flux, double* specRadius, double gamma)
{
   std::vector<double> h(2 + 4 + 4 + 4 + 1, 0.0);
   std::memcpy(h.data(), nxyz, 2 * sizeof(double));
   std::memcpy(h.data() + 2, ql, 4 * sizeof(double));
   std::memcpy(h.data() + 6, qr, 4 * sizeof(double));
   double* d = to_device(h);
   check(hamstr_gpu_flux_roe2d(1, d, d + 2, d + 6, d + 10, d + 14, gamma, nullptr));
   from_device(h, d);
   std::memcpy(flux, h.data() + 10, 4 * sizeof(double));
   *specRadius = h[14];
   if (*specRadius != *specRadius) throw Error(HAMSTR_GPU_ERR_NAN, "NaN in spectral radius (fluxRoe2D)");
}

void SOLVER::jacobianRoe2D(double* nxyz, double* ql, double* qr, double** lmat, double** rmat, double gamma)
{
   std::vector<double> h(2 + 4 + 4 + 32, 0.0);
   std::memcpy(h.data(), nxyz, 2 * sizeof(double));
   std::memcpy(h.data() + 2, ql, 4 * sizeof(double));
   std::memcpy(h.data() + 6, qr, 4 * sizeof(double));
   double* d = to_device(h);
   check(hamstr_gpu_jacobian_roe2d(1, d, d + 2, d + 6, d + 10, d + 26, gamma, nullptr));
   from_device(h, d);
   for (int i = 0; i < 4; i++) {
      std::memcpy(lmat[i], h.data() + 10 + 4 * i, 4 * sizeof(double));
      std::memcpy(rmat[i], h.data() + 26 + 4 * i, 4 * sizeof(double));
   }
}

// ------------------------------------------------------------------
// RECONSTRUCTION
// ------------------------------------------------------------------
namespace RECONSTRUCTION {

void MUSCL(double** f, double** ql, double** qr, double** f2, int is, int ie, double th, double qt, double eps,
           int imax, int nq)
{
   const size_t n = (size_t)imax * nq;
   const int last = muscl_last(ie, imax, qt);
   std::vector<double> h(4 * n, 0.0);
   pack(h, 0, f, imax, nq);
   pack(h, n, ql, imax, nq);
   pack(h, 2 * n, qr, imax, nq);
   if (qt != 0.0) pack(h, 3 * n, f2, imax, nq);
   double* d = to_device(h);
   check(hamstr_gpu_muscl(1, imax, nq, d, d + n, d + 2 * n, d + 3 * n, is, last, th, qt, eps, nullptr));
   from_device(h, d);
   unpack(h, n, ql, is, last, nq);
   unpack(h, 2 * n, qr, is, last, nq);
   if (qt != 0.0) unpack(h, 3 * n, f2, 0, imax - 2, nq);
}

void MUSCL_DERIV(double** f, double** ql, double** qr, double** f2, double** dq, int is, int ie, double th, double qt,
                 double eps, int imax, int nq)
{
   const size_t n = (size_t)imax * nq;
   const int last = muscl_last(ie, imax, qt);
   std::vector<double> h(5 * n, 0.0);
   pack(h, 0, f, imax, nq);
   pack(h, n, dq, imax, nq);
   pack(h, 2 * n, ql, imax, nq);
   pack(h, 3 * n, qr, imax, nq);
   if (qt != 0.0) pack(h, 4 * n, f2, imax, nq);
   double* d = to_device(h);
   check(hamstr_gpu_muscl_deriv(1, imax, nq, d, d + n, d + 2 * n, d + 3 * n, d + 4 * n, is, last, th, qt, eps,
                                nullptr));
   from_device(h, d);
   unpack(h, 2 * n, ql, is, last, nq);
   unpack(h, 3 * n, qr, is, last, nq);
   if (qt != 0.0) unpack(h, 4 * n, f2, 0, imax - 2, nq);
}

void WENO(double** f, double** ql, double** qr, int is, int ie, double epsw, int imax, int nq)
{
   const size_t n = (size_t)imax * nq;
   std::vector<double> h(3 * n, 0.0);
   pack(h, 0, f, imax, nq);
   pack(h, n, ql, imax, nq);
   pack(h, 2 * n, qr, imax, nq);
   double* d = to_device(h);
   check(hamstr_gpu_weno(1, imax, nq, d, d + n, d + 2 * n, is, ie, epsw, nullptr));
   from_device(h, d);
   unpack(h, n, ql, is, imax - 3, nq);
   unpack(h, 2 * n, qr, is, imax - 3, nq);
}

void WENO_DERIV(double** f, double** ql, double** qr, double** dq, int is, int ie, double eps, int imax, int nq)
{
   const size_t n = (size_t)imax * nq;
   std::vector<double> h(4 * n, 0.0);
   pack(h, 0, f, imax, nq);
   pack(h, n, dq, imax, nq);
   pack(h, 2 * n, ql, imax, nq);
   pack(h, 3 * n, qr, imax, nq);
   double* d = to_device(h);
   check(hamstr_gpu_weno_deriv(1, imax, nq, d, d + n, d + 2 * n, d + 3 * n, is, ie, eps, nullptr));
   from_device(h, d);
   unpack(h, 2 * n, ql, is, imax - 3, nq);
   unpack(h, 3 * n, qr, is, imax - 3, nq);
}

}  // namespace RECONSTRUCTION

// ------------------------------------------------------------------
// TRISOLVER
// ------------------------------------------------------------------
namespace TRISOLVER {
namespace {
void block_tridag(double*** a, double*** b, double*** c, double** f, int N, int nq, int periodic)
{
   if (nq != 4) throw Error(HAMSTR_GPU_ERR_ARG, "blockTridag4: nq must be 4");
   if (N < 1) throw Error(HAMSTR_GPU_ERR_ARG, "blockTridag4: N must be positive");
   const size_t nb = 16 * (size_t)N;
   std::vector<double> h(3 * nb + 4 * (size_t)N, 0.0);
   for (int i = 0; i < N; i++)
      for (int k = 0; k < 4; k++) {
         std::memcpy(h.data() + 16 * (size_t)i + 4 * k, a[i][k], 4 * sizeof(double));
         std::memcpy(h.data() + nb + 16 * (size_t)i + 4 * k, b[i][k], 4 * sizeof(double));
         std::memcpy(h.data() + 2 * nb + 16 * (size_t)i + 4 * k, c[i][k], 4 * sizeof(double));
      }
   for (int i = 0; i < N; i++) std::memcpy(h.data() + 3 * nb + 4 * (size_t)i, f[i], 4 * sizeof(double));
   double* d = to_device(h);
   check(hamstr_gpu_block_tridag4(1, N, periodic, d, d + nb, d + 2 * nb, d + 3 * nb, nullptr));
   from_device(h, d);
   for (int i = 0; i < N; i++) std::memcpy(f[i], h.data() + 3 * nb + 4 * (size_t)i, 4 * sizeof(double));
}
}  // namespace

void blockTridag4(double*** a, double*** b, double*** c, double** f, int N, int nq)
{
   block_tridag(a, b, c, f, N, nq, 0);
}

void blockTridagPeriodic4(double*** a, double*** b, double*** c, double** f, int N, int nq)
{
   block_tridag(a, b, c, f, N, nq, 1);
}

}  // namespace TRISOLVER
