// ##################################################################
//
// pointwise.cu -- function-level entry points of the reference's numerics
//
// The solver handle fuses the reference's per-face and per-chain functions
// into whole-mesh kernels.  A caller that uses those functions directly --
// SOLVER::fluxRoe2D / jacobianRoe2D (interfaceFlux.cpp:24-169,
// jacobianRoe.cpp:9-70) and RECONSTRUCTION::MUSCL / WENO / MUSCL_DERIV /
// WENO_DERIV (reconstruction.cpp:16-386) -- gets them here, batched over
// faces or over lines, on device arrays, one thread per face or per
// (line, component, entry).  Every expression keeps the reference's
// operands and association (the unit is compiled with -fmad=false), so
// each output equals one reference call's bit for bit.
//
// Line arrays are [nlines][imax][nq] doubles: entry i, component n of
// line l at (l*imax + i)*nq + n, the reference's f[i][n] per chain.
// ##################################################################
#include <cuda_runtime.h>

#include <string>

#include "../../include/hamstr_gpu.h"
#include "roe.cuh"

namespace hamstr {
void set_last_error(const std::string& m);
}

namespace {

using namespace hamstr;

constexpr int kThreads = 128;

int launched(const char* what)
{
   const cudaError_t e = cudaGetLastError();
   if (e == cudaSuccess) return HAMSTR_GPU_OK;
   set_last_error(std::string(what) + " launch: " + cudaGetErrorString(e));
   return HAMSTR_GPU_ERR_CUDA;
}

unsigned blocks(size_t n) { return (unsigned)((n + kThreads - 1) / kThreads); }

// ---------------- Roe flux and Jacobian, one thread per face -------------
template <bool JAC>
__global__ void __launch_bounds__(kThreads) roe_faces_kernel(int n, const double* __restrict__ nxy,
                                                             const double* __restrict__ ql,
                                                             const double* __restrict__ qr, double gamma,
                                                             double* __restrict__ flux, double* __restrict__ spec,
                                                             double* __restrict__ lmat, double* __restrict__ rmat)
{
   const int f = blockIdx.x * blockDim.x + threadIdx.x;
   if (f >= n) return;
   double L[4], R[4];
#pragma unroll
   for (int k = 0; k < 4; k++) {
      L[k] = ql[4 * (size_t)f + k];
      R[k] = qr[4 * (size_t)f + k];
   }
   RoeOut o;
   double lm[16], rm[16];
   roe_face<JAC, false>(nxy[2 * (size_t)f], nxy[2 * (size_t)f + 1], L, R, gamma, o, lm, rm);
   if (JAC) {
#pragma unroll
      for (int e = 0; e < 16; e++) {
         lmat[16 * (size_t)f + e] = lm[e];
         rmat[16 * (size_t)f + e] = rm[e];
      }
   } else {
#pragma unroll
      for (int k = 0; k < 4; k++) flux[4 * (size_t)f + k] = o.flux[k];
      spec[f] = o.spec;
   }
}

// ---------------- reconstructions along lines ----------------------------
struct Lines {
   int nlines, imax, nq;
   __device__ __forceinline__ size_t at(int l, int i, int n) const { return ((size_t)l * imax + i) * nq + n; }
};

// thread t -> (line, component, entry i) with i in [i0, i0 + ni)
__device__ __forceinline__ bool line_index(const Lines& g, int i0, int ni, int& l, int& n, int& i)
{
   const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
   const size_t per_line = (size_t)g.nq * ni;
   if (ni <= 0 || t >= per_line * g.nlines) return false;
   l = (int)(t / per_line);
   const int r = (int)(t - (size_t)l * per_line);
   n = r / ni;
   i = i0 + r - n * ni;
   return true;
}

// f2[i][n] = f[i+1][n] - f[i][n] for i < imax-1 (reconstruction.cpp:54-55,
// 219-220): the reference leaves these differences in the caller's f2
__global__ void __launch_bounds__(kThreads) diff_kernel(Lines g, const double* __restrict__ f, double* __restrict__ f2)
{
   int l, n, i;
   if (!line_index(g, 0, g.imax - 1, l, n, i)) return;
   f2[g.at(l, i, n)] = f[g.at(l, i + 1, n)] - f[g.at(l, i, n)];
}

// MUSCL (reconstruction.cpp:16-70): first order copies f; otherwise the
// kappa scheme with the reference's limiter.  f2i and f2i1 are the same
// differences the reference stores in f2 and reads back.
__global__ void __launch_bounds__(kThreads) muscl_kernel(Lines g, const double* __restrict__ f,
                                                         double* __restrict__ ql, double* __restrict__ qr, int is,
                                                         int ie, double th, double qt, double eps)
{
   int l, n, i;
   if (!line_index(g, is, ie - is + 1, l, n, i)) return;
   const double fi = f[g.at(l, i, n)];
   if (qt == 0.0) {
      ql[g.at(l, i, n)] = fi;
      qr[g.at(l, i, n)] = fi;
      return;
   }
   const double thm = 1.0 - th;
   const double thp = 1.0 + th;
   const double f2i = f[g.at(l, i + 1, n)] - fi;
   const double f2i1 = fi - f[g.at(l, i - 1, n)];
   const double a1 = 3.0 * (f2i * f2i1 + eps);
   const double a2 = 2.0 * (f2i - f2i1) * (f2i - f2i1) + a1;
   const double f3i = a1 / a2;
   const double f3qt = qt * f3i;
   ql[g.at(l, i, n)] = fi + f3qt * (thm * f2i1 + thp * f2i);
   qr[g.at(l, i, n)] = fi - f3qt * (thp * f2i1 + thm * f2i);
}

// MUSCL_DERIV (reconstruction.cpp:168-236): the linearisation of MUSCL
// about f applied to dq
__global__ void __launch_bounds__(kThreads) muscl_deriv_kernel(Lines g, const double* __restrict__ f,
                                                               const double* __restrict__ dq, double* __restrict__ ql,
                                                               double* __restrict__ qr, int is, int ie, double th,
                                                               double qt, double eps)
{
   int l, n, i;
   if (!line_index(g, is, ie - is + 1, l, n, i)) return;
   const double dqi = dq[g.at(l, i, n)];
   if (qt == 0.0) {
      ql[g.at(l, i, n)] = dqi;
      qr[g.at(l, i, n)] = dqi;
      return;
   }
   const double thm = 1.0 - th;
   const double thp = 1.0 + th;
   const double fi = f[g.at(l, i, n)];
   const double f2i = f[g.at(l, i + 1, n)] - fi;
   const double f2i1 = fi - f[g.at(l, i - 1, n)];
   const double df2i = dq[g.at(l, i + 1, n)] - dqi;
   const double df2i1 = dqi - dq[g.at(l, i - 1, n)];
   const double a1 = 3.0 * (f2i * f2i1 + eps);
   const double da1 = 3.0 * (df2i * f2i1 + f2i * df2i1);
   const double a2 = 2.0 * (f2i - f2i1) * (f2i - f2i1) + a1;
   const double da2 = 2.0 * 2.0 * (f2i - f2i1) * (df2i - df2i1) + da1;
   const double f3i = a1 / a2;
   const double df3i = da1 / a2 - a1 * da2 / (a2 * a2);
   const double f3qt = qt * f3i;
   const double df3qt = qt * df3i;
   ql[g.at(l, i, n)] = dqi + df3qt * (thm * f2i1 + thp * f2i) + f3qt * (thm * df2i1 + thp * df2i);
   qr[g.at(l, i, n)] = dqi - df3qt * (thp * f2i1 + thm * f2i) - f3qt * (thp * df2i1 + thm * df2i);
}

// WENO5 (reconstruction.cpp:78-124) with smoothness power 1 (pow(x, 1) is
// x exactly)
__device__ __forceinline__ double weno5_pt(double a, double b, double c, double d, double e, double epsw)
{
   const double b1 = 13. / 12.;
   const double b2 = 1. / 6.;
   const double djm1 = a - 2. * b + c;
   const double ejm1 = a - 4. * b + 3. * c;
   const double dj = b - 2. * c + d;
   const double ej = b - d;
   const double djp1 = c - 2. * d + e;
   const double ejp1 = 3. * c - 4. * d + e;
   const double dis0 = b1 * djm1 * djm1 + 0.25 * ejm1 * ejm1 + epsw;
   const double dis1 = b1 * dj * dj + 0.25 * ej * ej + epsw;
   const double dis2 = b1 * djp1 * djp1 + 0.25 * ejp1 * ejp1 + epsw;
   const double q30 = 2. * a - 7. * b + 11. * c;
   const double q31 = -b + 5. * c + 2. * d;
   const double q32 = 2. * c + 5. * d - e;
   const double d01 = dis0 / dis1;
   const double d02 = dis0 / dis2;
   const double a1ba0 = 6. * d01;
   const double a2ba0 = 3. * d02;
   const double w0 = 1.0 / (1.0 + a1ba0 + a2ba0);
   const double w1 = a1ba0 * w0;
   const double w2 = 1. - w0 - w1;
   return b2 * (w0 * q30 + w1 * q31 + w2 * q32);
}

// WENO_5 (reconstruction.cpp:243-347): the derivative of WENO5 at
// (a..e) in the direction (a_d..e_d), weights differentiated through the
// smoothness indicators
__device__ __forceinline__ double weno5_deriv_pt(double a, double b, double c, double d, double e, double a_d,
                                                 double b_d, double c_d, double d_d, double e_d, double epsw)
{
   const double b1 = 13. / 12.;
   const double b2 = 1. / 6.;
   const double djm1 = a - 2. * b + c;
   const double ejm1 = a - 4. * b + 3. * c;
   const double dj = b - 2. * c + d;
   const double ej = b - d;
   const double djp1 = c - 2. * d + e;
   const double ejp1 = 3. * c - 4. * d + e;
   const double dis0 = b1 * djm1 * djm1 + 0.25 * ejm1 * ejm1 + epsw;
   const double dis1 = b1 * dj * dj + 0.25 * ej * ej + epsw;
   const double dis2 = b1 * djp1 * djp1 + 0.25 * ejp1 * ejp1 + epsw;
   const double q30 = 2. * a - 7. * b + 11. * c;
   const double q31 = -b + 5. * c + 2. * d;
   const double q32 = 2. * c + 5. * d - e;
   const double d01 = dis0 / dis1;
   const double d02 = dis0 / dis2;
   const double a1ba0 = 6. * d01;
   const double a2ba0 = 3. * d02;
   const double w0 = 1.0 / (1.0 + a1ba0 + a2ba0);
   const double w1 = a1ba0 * w0;
   const double w2 = 1. - w0 - w1;
   const double djm1_d = a_d - 2. * b_d + c_d;
   const double ejm1_d = a_d - 4. * b_d + 3. * c_d;
   const double dj_d = b_d - 2. * c_d + d_d;
   const double ej_d = b_d - d_d;
   const double djp1_d = c_d - 2. * d_d + e_d;
   const double ejp1_d = 3. * c_d - 4. * d_d + e_d;
   const double q30_d = 2. * a_d - 7. * b_d + 11. * c_d;
   const double q31_d = -b_d + 5. * c_d + 2. * d_d;
   const double q32_d = 2. * c_d + 5. * d_d - e_d;
   const double term1 = b2 * w0 * q30_d;
   const double term2 = b2 * w1 * q31_d;
   const double term3 = b2 * w2 * q32_d;
   // the reference's integer literals 2, 3, 6 convert to these doubles
   const double dbeta0 = b1 * 2. * djm1 * djm1_d + 0.25 * 2. * ejm1 * ejm1_d;
   const double dbeta1 = b1 * 2. * dj * dj_d + 0.25 * 2. * ej * ej_d;
   const double dbeta2 = b1 * 2. * djp1 * djp1_d + 0.25 * 2. * ejp1 * ejp1_d;
   const double beta0 = dis0, beta1 = dis1, beta2 = dis2;
   const double down = beta1 * beta2 + 6. * beta0 * beta2 + 3. * beta0 * beta1;
   const double dw0_up_1 = (dbeta1 * beta2 + beta1 * dbeta2) * down;
   const double dw0_up_2 = beta1 * beta2 *
                           (dbeta1 * beta2 + beta1 * dbeta2 + 6. * (dbeta0 * beta2 + beta0 * dbeta2) +
                            3. * (dbeta0 * beta1 + beta0 * dbeta1));
   const double dw0 = (dw0_up_1 - dw0_up_2) / (down * down);
   const double dw1_up_1 = 6. * (dbeta0 * beta2 + beta0 * dbeta2) * down;
   const double dw1_up_2 = 6. * dw0_up_2 / beta1 * beta0;
   const double dw1 = (dw1_up_1 - dw1_up_2) / (down * down);
   const double dw2_up_1 = 3. * (dbeta0 * beta1 + beta0 * dbeta1) * down;
   const double dw2_up_2 = 3. * dw0_up_2 / beta2 * beta0;
   const double dw2 = (dw2_up_1 - dw2_up_2) / (down * down);
   return term1 + term2 + term3 + b2 * dw0 * q30 + b2 * dw1 * q31 + b2 * dw2 * q32;
}

// WENO (reconstruction.cpp:133-160) and, with DERIV, WENO_DERIV
// (reconstruction.cpp:353-386): entries is .. imax-3
template <bool DERIV>
__global__ void __launch_bounds__(kThreads) weno_kernel(Lines g, const double* __restrict__ f,
                                                        const double* __restrict__ dq, double* __restrict__ ql,
                                                        double* __restrict__ qr, int is, double eps)
{
   int l, n, i;
   if (!line_index(g, is, g.imax - 2 - is, l, n, i)) return;
   double v[5], dv[5];
#pragma unroll
   for (int k = 0; k < 5; k++) {
      v[k] = f[g.at(l, i - 2 + k, n)];
      if (DERIV) dv[k] = dq[g.at(l, i - 2 + k, n)];
   }
   if (DERIV) {
      ql[g.at(l, i, n)] = weno5_deriv_pt(v[0], v[1], v[2], v[3], v[4], dv[0], dv[1], dv[2], dv[3], dv[4], eps);
      qr[g.at(l, i, n)] = weno5_deriv_pt(v[4], v[3], v[2], v[1], v[0], dv[4], dv[3], dv[2], dv[1], dv[0], eps);
   } else {
      ql[g.at(l, i, n)] = weno5_pt(v[0], v[1], v[2], v[3], v[4], eps);
      qr[g.at(l, i, n)] = weno5_pt(v[4], v[3], v[2], v[1], v[0], eps);
   }
}

// shared argument checks of the line entry points: the reference reads
// f2[i-1], f2[i] (MUSCL: entries i-1 .. i+1) for i in [is, ie] and, WENO,
// f[i-2 .. i+2] for i in [is, imax-3]
int check_lines(const char* what, int nlines, int imax, int nq, int is, int ie, int lo, int hi_off)
{
   if (nlines < 0 || imax < 1 || nq < 1 || is < lo || ie < is - 1 || ie > imax - 1 - hi_off) {
      set_last_error(std::string(what) + ": need nlines >= 0, imax >= 1, nq >= 1 and " + std::to_string(lo) +
                     " <= is <= ie + 1, ie <= imax - " + std::to_string(1 + hi_off) + " (is = " +
                     std::to_string(is) + ", ie = " + std::to_string(ie) + ", imax = " + std::to_string(imax) + ")");
      return HAMSTR_GPU_ERR_ARG;
   }
   return HAMSTR_GPU_OK;
}

}  // namespace

extern "C" {

int hamstr_gpu_flux_roe2d(int n, const double* nxy, const double* ql, const double* qr, double* flux, double* spec,
                          double gamma, void* stream)
{
   if (n < 0 || (n > 0 && (!nxy || !ql || !qr || !flux || !spec))) {
      set_last_error("flux_roe2d: n >= 0 and non-null arrays");
      return HAMSTR_GPU_ERR_ARG;
   }
   if (n == 0) return HAMSTR_GPU_OK;
   roe_faces_kernel<false><<<blocks(n), kThreads, 0, (cudaStream_t)stream>>>(n, nxy, ql, qr, gamma, flux, spec,
                                                                             nullptr, nullptr);
   return launched("flux_roe2d");
}

int hamstr_gpu_jacobian_roe2d(int n, const double* nxy, const double* ql, const double* qr, double* lmat,
                              double* rmat, double gamma, void* stream)
{
   if (n < 0 || (n > 0 && (!nxy || !ql || !qr || !lmat || !rmat))) {
      set_last_error("jacobian_roe2d: n >= 0 and non-null arrays");
      return HAMSTR_GPU_ERR_ARG;
   }
   if (n == 0) return HAMSTR_GPU_OK;
   roe_faces_kernel<true><<<blocks(n), kThreads, 0, (cudaStream_t)stream>>>(n, nxy, ql, qr, gamma, nullptr,
                                                                            nullptr, lmat, rmat);
   return launched("jacobian_roe2d");
}

int hamstr_gpu_muscl(int nlines, int imax, int nq, const double* f, double* ql, double* qr, double* f2, int is,
                     int ie, double th, double qt, double eps, void* stream)
{
   const bool third = qt != 0.0;
   int st = check_lines("muscl", nlines, imax, nq, is, ie, third ? 1 : 0, third ? 1 : 0);
   if (st) return st;
   if (nlines > 0 && (!f || !ql || !qr || (third && !f2))) {
      set_last_error("muscl: null array");
      return HAMSTR_GPU_ERR_ARG;
   }
   if (nlines == 0) return HAMSTR_GPU_OK;
   const Lines g{nlines, imax, nq};
   const cudaStream_t s = (cudaStream_t)stream;
   if (third && imax > 1) diff_kernel<<<blocks((size_t)nlines * nq * (imax - 1)), kThreads, 0, s>>>(g, f, f2);
   if (ie >= is)
      muscl_kernel<<<blocks((size_t)nlines * nq * (ie - is + 1)), kThreads, 0, s>>>(g, f, ql, qr, is, ie, th, qt, eps);
   return launched("muscl");
}

int hamstr_gpu_muscl_deriv(int nlines, int imax, int nq, const double* f, const double* dq, double* ql, double* qr,
                           double* f2, int is, int ie, double th, double qt, double eps, void* stream)
{
   const bool third = qt != 0.0;
   int st = check_lines("muscl_deriv", nlines, imax, nq, is, ie, third ? 1 : 0, third ? 1 : 0);
   if (st) return st;
   if (nlines > 0 && (!dq || !ql || !qr || (third && (!f || !f2)))) {
      set_last_error("muscl_deriv: null array");
      return HAMSTR_GPU_ERR_ARG;
   }
   if (nlines == 0) return HAMSTR_GPU_OK;
   const Lines g{nlines, imax, nq};
   const cudaStream_t s = (cudaStream_t)stream;
   if (third && imax > 1) diff_kernel<<<blocks((size_t)nlines * nq * (imax - 1)), kThreads, 0, s>>>(g, f, f2);
   if (ie >= is)
      muscl_deriv_kernel<<<blocks((size_t)nlines * nq * (ie - is + 1)), kThreads, 0, s>>>(g, f, dq, ql, qr, is, ie,
                                                                                          th, qt, eps);
   return launched("muscl_deriv");
}

int hamstr_gpu_weno(int nlines, int imax, int nq, const double* f, double* ql, double* qr, int is, int ie,
                    double epsw, void* stream)
{
   (void)epsw;   // the reference overwrites its epsw argument with 1e-15 (reconstruction.cpp:145)
   int st = check_lines("weno", nlines, imax, nq, is, ie, 2, 0);
   if (st) return st;
   if (nlines > 0 && (!f || !ql || !qr)) {
      set_last_error("weno: null array");
      return HAMSTR_GPU_ERR_ARG;
   }
   if (nlines == 0 || imax - 2 <= is) return HAMSTR_GPU_OK;
   const Lines g{nlines, imax, nq};
   weno_kernel<false><<<blocks((size_t)nlines * nq * (imax - 2 - is)), kThreads, 0, (cudaStream_t)stream>>>(
      g, f, nullptr, ql, qr, is, 1e-15);
   return launched("weno");
}

int hamstr_gpu_weno_deriv(int nlines, int imax, int nq, const double* f, const double* dq, double* ql, double* qr,
                          int is, int ie, double eps, void* stream)
{
   int st = check_lines("weno_deriv", nlines, imax, nq, is, ie, 2, 0);
   if (st) return st;
   if (nlines > 0 && (!f || !dq || !ql || !qr)) {
      set_last_error("weno_deriv: null array");
      return HAMSTR_GPU_ERR_ARG;
   }
   if (nlines == 0 || imax - 2 <= is) return HAMSTR_GPU_OK;
   const Lines g{nlines, imax, nq};
   weno_kernel<true><<<blocks((size_t)nlines * nq * (imax - 2 - is)), kThreads, 0, (cudaStream_t)stream>>>(
      g, f, dq, ql, qr, is, eps);
   return launched("weno_deriv");
}

}  // extern "C"
