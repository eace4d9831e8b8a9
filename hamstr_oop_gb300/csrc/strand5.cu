// ##################################################################
//
// strand5.cu -- the 5-variable (3D strand) numerics at function level
//
// The reference carries a 3D strand build (-DDim3) whose driver does not
// compile (io.cpp:306), but its 5-variable numerics are compiled in every
// build: SOLVER::fluxRoe3D (interfaceFlux.cpp:176-319), jacobianRoe3D
// (jacobianRoe.cpp:92-620, frozen eigenvalues, IMODE 1) and the 5x5
// block-tridiagonal solvers TRISOLVER::blockTridag / blockTridagPeriodic
// (triSolvers.cpp:443-766).  They are given here batched on device arrays:
// one thread per face or per line, every expression with the reference's
// operands and association (-fmad=false, IEEE division and square root),
// so each output equals one reference call's bit for bit.
// ##################################################################
#include <cuda_runtime.h>

#include <string>

#include "../../include/hamstr_gpu.h"

namespace hamstr {
void set_last_error(const std::string& m);
}

namespace {

using namespace hamstr;

constexpr int kThreads = 128;

unsigned blocks(size_t n) { return (unsigned)((n + kThreads - 1) / kThreads); }

int launched(const char* what)
{
   const cudaError_t e = cudaGetLastError();
   if (e == cudaSuccess) return HAMSTR_GPU_OK;
   set_last_error(std::string(what) + " launch: " + cudaGetErrorString(e));
   return HAMSTR_GPU_ERR_CUDA;
}

// ---------------- Roe flux, 5 variables (interfaceFlux.cpp:176-319) -------
__global__ void __launch_bounds__(kThreads) flux_roe3d_kernel(int n, const double* __restrict__ nxyz,
                                                              const double* __restrict__ qlv,
                                                              const double* __restrict__ qrv, double gamma,
                                                              double* __restrict__ flux, double* __restrict__ spec)
{
   const int f = blockIdx.x * blockDim.x + threadIdx.x;
   if (f >= n) return;
   const double* ql = qlv + 5 * (size_t)f;
   const double* qr = qrv + 5 * (size_t)f;
   const double gm1 = gamma - 1.0;
   const double nxd = nxyz[3 * (size_t)f], nyd = nxyz[3 * (size_t)f + 1], nzd = nxyz[3 * (size_t)f + 2];
   const double area = sqrt(nxd * nxd + nyd * nyd + nzd * nzd);
   const double invArea = 1. / area;
   const double nx = nxd * invArea, ny = nyd * invArea, nz = nzd * invArea;
   const double rol = ql[0], ul = ql[1] / ql[0], vl = ql[2] / ql[0], wl = ql[3] / ql[0];
   const double pl = gm1 * (ql[4] - 0.5 * rol * (ul * ul + vl * vl + wl * wl));
   const double hl = (ql[4] + pl) / rol;
   const double ror = qr[0], ur = qr[1] / qr[0], vr = qr[2] / qr[0], wr = qr[3] / qr[0];
   const double pr = gm1 * (qr[4] - 0.5 * ror * (ur * ur + vr * vr + wr * wr));
   const double hr = (qr[4] + pr) / ror;
   const double dp = pr - pl;
   const double uconr = ur * nx + vr * ny + wr * nz;
   const double uconl = ul * nx + vl * ny + wl * nz;
   const double fact = sqrt(ror / rol);
   const double A = 1.0 / (1.0 + fact), B = fact / (1.0 + fact);
   const double robar = rol * fact;
   const double ubar = ul * A + ur * B, vbar = vl * A + vr * B, wbar = wl * A + wr * B, hbar = hl * A + hr * B;
   const double cbar = sqrt(gm1 * (hbar - 0.5 * (ubar * ubar + vbar * vbar + wbar * wbar)));
   const double uconbar = ubar * nx + vbar * ny + wbar * nz;
   const double eig1 = fabs(uconbar), eig2 = fabs(uconbar + cbar), eig3 = fabs(uconbar - cbar);
   spec[f] = eig1 + cbar;
   const double term1 = -eig1 + 0.5 * (eig2 + eig3);
   const double term2 = 0.5 * (eig2 - eig3);
   const double del1 = term1 * dp / cbar / cbar + term2 * robar * (uconr - uconl) / cbar;
   const double del2 = term1 * (uconr - uconl) * robar + term2 * dp / cbar;
   double fm[5];
#pragma unroll
   for (int i = 0; i < 5; i++) fm[i] = eig1 * (qr[i] - ql[i]);
   fm[0] = fm[0] + del1;
   fm[1] = fm[1] + del1 * ubar + del2 * nx;
   fm[2] = fm[2] + del1 * vbar + del2 * ny;
   fm[3] = fm[3] + del1 * wbar + del2 * nz;
   fm[4] = fm[4] + del1 * hbar + del2 * uconbar;
   const double fl[5] = {rol * uconl, rol * uconl * ul + nx * pl, rol * uconl * vl + ny * pl,
                         rol * uconl * wl + nz * pl, (ql[4] + pl) * uconl};
   const double fr[5] = {ror * uconr, ror * uconr * ur + nx * pr, ror * uconr * vr + ny * pr,
                         ror * uconr * wr + nz * pr, (qr[4] + pr) * uconr};
#pragma unroll
   for (int i = 0; i < 5; i++) flux[5 * (size_t)f + i] = 0.5 * (fl[i] + fr[i] - fm[i]);
}

// ---------------- Roe Jacobian, 5 variables (jacobianRoe.cpp:92-620) -----
// One side's primitive state and the derivatives of its primitives with
// respect to its conserved variables (jacobianRoe.cpp:170-260)
struct Side {
   double ro, u, v, w, p, h, ucon;
   double du[5], dv[5], dw[5], dp[5], ducon[5];
};

__device__ __forceinline__ void side_of(const double* q, double gm1, double nx, double ny, double nz, Side& s)
{
   s.ro = q[0];
   s.u = q[1] / q[0];
   s.v = q[2] / q[0];
   s.w = q[3] / q[0];
   s.p = gm1 * (q[4] - 0.5 * s.ro * (s.u * s.u + s.v * s.v + s.w * s.w));
   s.h = (q[4] + s.p) / s.ro;
   s.ucon = s.u * nx + s.v * ny + s.w * nz;
#pragma unroll
   for (int i = 0; i < 5; i++) {
      s.du[i] = 0.0;
      s.dv[i] = 0.0;
      s.dw[i] = 0.0;
   }
   s.du[0] = -s.u / s.ro;
   s.du[1] = 1.0 / s.ro;
   s.dv[0] = -s.v / s.ro;
   s.dv[2] = 1.0 / s.ro;
   s.dw[0] = -s.w / s.ro;
   s.dw[3] = 1.0 / s.ro;
   s.dp[0] = 0.5 * gm1 * (s.u * s.u + s.v * s.v + s.w * s.w);
   s.dp[1] = -gm1 * s.u;
   s.dp[2] = -gm1 * s.v;
   s.dp[3] = -gm1 * s.w;
   s.dp[4] = gm1;
   s.ducon[0] = -s.ucon / s.ro;
   s.ducon[1] = nx / s.ro;
   s.ducon[2] = ny / s.ro;
   s.ducon[3] = nz / s.ro;
   s.ducon[4] = 0.0;
}

// the native-flux Jacobian of one side (jacobianRoe.cpp:573-605), row k
__device__ __forceinline__ double native_row(const Side& s, double q4, int k, int i, double nx, double ny, double nz)
{
   const double dro = (i == 0) ? 1.0 : 0.0;
   const double dq5 = (i == 4) ? 1.0 : 0.0;
   switch (k) {
      case 0: return dro * s.ucon + s.ro * s.ducon[i];
      case 1: return (dro * s.ucon * s.u + s.ro * s.ducon[i] * s.u + s.ro * s.ucon * s.du[i]) + nx * s.dp[i];
      case 2: return (dro * s.ucon * s.v + s.ro * s.ducon[i] * s.v + s.ro * s.ucon * s.dv[i]) + ny * s.dp[i];
      case 3: return (dro * s.ucon * s.w + s.ro * s.ducon[i] * s.w + s.ro * s.ucon * s.dw[i]) + nz * s.dp[i];
      default: return (dq5 + s.dp[i]) * s.ucon + (q4 + s.p) * s.ducon[i];
   }
}

__global__ void __launch_bounds__(kThreads) jacobian_roe3d_kernel(int n, const double* __restrict__ nxyz,
                                                                  const double* __restrict__ qlv,
                                                                  const double* __restrict__ qrv, double gam,
                                                                  double* __restrict__ lmat,
                                                                  double* __restrict__ rmat)
{
   const int f = blockIdx.x * blockDim.x + threadIdx.x;
   if (f >= n) return;
   const double* ql = qlv + 5 * (size_t)f;
   const double* qr = qrv + 5 * (size_t)f;
   const double gm1 = gam - 1.0;
   const double nxd = nxyz[3 * (size_t)f], nyd = nxyz[3 * (size_t)f + 1], nzd = nxyz[3 * (size_t)f + 2];
   const double area = sqrt(nxd * nxd + nyd * nyd + nzd * nzd);
   const double nx = nxd / area, ny = nyd / area, nz = nzd / area;
   Side L, R;
   side_of(ql, gm1, nx, ny, nz, L);
   side_of(qr, gm1, nx, ny, nz, R);
   // Roe averages and frozen eigenvalues (jacobianRoe.cpp:262-337, IMODE 1)
   const double fact = sqrt(R.ro / L.ro);
   const double A = 1.0 / (1.0 + fact), B = fact / (1.0 + fact);
   const double robar = L.ro * fact;
   const double ubar = L.u * A + R.u * B, vbar = L.v * A + R.v * B, wbar = L.w * A + R.w * B;
   const double hbar = L.h * A + R.h * B;
   const double cbar = sqrt(gm1 * (hbar - 0.5 * (ubar * ubar + vbar * vbar + wbar * wbar)));
   const double uconbar = ubar * nx + vbar * ny + wbar * nz;
   const double eig1 = fabs(uconbar), eig2 = fabs(uconbar + cbar), eig3 = fabs(uconbar - cbar);
   const double term1 = -eig1 + 0.5 * (eig2 + eig3);
   const double term2 = 0.5 * (eig2 - eig3);
   // dissipation Jacobian, column by column, then 0.5 (native - dissipation)
   // (jacobianRoe.cpp:488-562, 611-618)
#pragma unroll
   for (int i = 0; i < 5; i++) {
      const double dd1l = -term1 * L.dp[i] / cbar / cbar - term2 * robar * L.ducon[i] / cbar;
      const double dd1r = +term1 * R.dp[i] / cbar / cbar + term2 * robar * R.ducon[i] / cbar;
      const double dd2l = -term1 * L.ducon[i] * robar - term2 * L.dp[i] / cbar;
      const double dd2r = +term1 * R.ducon[i] * robar + term2 * R.dp[i] / cbar;
      double dl[5], dr[5];
#pragma unroll
      for (int k = 0; k < 5; k++) {
         const double im = (k == i) ? 1.0 : 0.0;
         dl[k] = 0.0 - eig1 * im;
         dr[k] = 0.0 + eig1 * im;
      }
      dl[0] = dl[0] + dd1l;
      dr[0] = dr[0] + dd1r;
      dl[1] = dl[1] + dd1l * ubar + dd2l * nx;
      dr[1] = dr[1] + dd1r * ubar + dd2r * nx;
      dl[2] = dl[2] + dd1l * vbar + dd2l * ny;
      dr[2] = dr[2] + dd1r * vbar + dd2r * ny;
      dl[3] = dl[3] + dd1l * wbar + dd2l * nz;
      dr[3] = dr[3] + dd1r * wbar + dd2r * nz;
      dl[4] = dl[4] + dd1l * hbar + dd2l * uconbar;
      dr[4] = dr[4] + dd1r * hbar + dd2r * uconbar;
#pragma unroll
      for (int k = 0; k < 5; k++) {
         lmat[25 * (size_t)f + 5 * k + i] = 0.5 * (native_row(L, ql[4], k, i, nx, ny, nz) - dl[k]);
         rmat[25 * (size_t)f + 5 * k + i] = 0.5 * (native_row(R, qr[4], k, i, nx, ny, nz) - dr[k]);
      }
   }
}

// ---------------- 5x5 block-tridiagonal solvers (triSolvers.cpp:443-766) -
// unpivoted LU with reciprocal pivots (triSolvers.cpp:481-506)
struct LU5 {
   double b11, b21, b22, b31, b32, b33, b41, b42, b43, b44, b51, b52, b53, b54, b55;
   double u12, u13, u14, u15, u23, u24, u25, u34, u35, u45;
};

__device__ __forceinline__ LU5 lu5_factor(const double* b)
{
   LU5 u;
   u.b11 = 1. / b[0];
   u.u12 = b[1] * u.b11;
   u.u13 = b[2] * u.b11;
   u.u14 = b[3] * u.b11;
   u.u15 = b[4] * u.b11;
   u.b21 = b[5];
   u.b22 = 1. / (b[6] - u.b21 * u.u12);
   u.u23 = (b[7] - u.b21 * u.u13) * u.b22;
   u.u24 = (b[8] - u.b21 * u.u14) * u.b22;
   u.u25 = (b[9] - u.b21 * u.u15) * u.b22;
   u.b31 = b[10];
   u.b32 = b[11] - u.b31 * u.u12;
   u.b33 = 1. / (b[12] - u.b31 * u.u13 - u.b32 * u.u23);
   u.u34 = (b[13] - u.b31 * u.u14 - u.b32 * u.u24) * u.b33;
   u.u35 = (b[14] - u.b31 * u.u15 - u.b32 * u.u25) * u.b33;
   u.b41 = b[15];
   u.b42 = b[16] - u.b41 * u.u12;
   u.b43 = b[17] - u.b41 * u.u13 - u.b42 * u.u23;
   u.b44 = 1. / (b[18] - u.b41 * u.u14 - u.b42 * u.u24 - u.b43 * u.u34);
   u.u45 = (b[19] - u.b41 * u.u15 - u.b42 * u.u25 - u.b43 * u.u35) * u.b44;
   u.b51 = b[20];
   u.b52 = b[21] - u.b51 * u.u12;
   u.b53 = b[22] - u.b51 * u.u13 - u.b52 * u.u23;
   u.b54 = b[23] - u.b51 * u.u14 - u.b52 * u.u24 - u.b53 * u.u34;
   u.b55 = 1. / (b[24] - u.b51 * u.u15 - u.b52 * u.u25 - u.b53 * u.u35 - u.b54 * u.u45);
   return u;
}

// x[0], x[s], ..., x[4s] <- LU^{-1} x (triSolvers.cpp:508-518)
__device__ __forceinline__ void lu5_solve(const LU5& u, double* x, int s)
{
   const double d1 = x[0] * u.b11;
   const double d2 = (x[s] - u.b21 * d1) * u.b22;
   const double d3 = (x[2 * s] - u.b31 * d1 - u.b32 * d2) * u.b33;
   const double d4 = (x[3 * s] - u.b41 * d1 - u.b42 * d2 - u.b43 * d3) * u.b44;
   const double d5 = (x[4 * s] - u.b51 * d1 - u.b52 * d2 - u.b53 * d3 - u.b54 * d4) * u.b55;
   const double x3 = d4 - u.u45 * d5;
   const double x2 = d3 - u.u34 * x3 - u.u35 * d5;
   const double x1 = d2 - u.u23 * x2 - u.u24 * x3 - u.u25 * d5;
   x[4 * s] = d5;
   x[3 * s] = x3;
   x[2 * s] = x2;
   x[s] = x1;
   x[0] = d1 - u.u12 * x1 - u.u13 * x2 - u.u14 * x3 - u.u15 * d5;
}

// one line per thread, in place: a, b, c [N][5][5] are the reference's
// scratch, f [N][5] becomes the solution
__global__ void __launch_bounds__(kThreads) block_tridag5_kernel(int nlines, int N, int periodic,
                                                                 double* __restrict__ av, double* __restrict__ bv,
                                                                 double* __restrict__ cv, double* __restrict__ fv)
{
   const int line = blockIdx.x * blockDim.x + threadIdx.x;
   if (line >= nlines) return;
   const size_t nb = 25 * (size_t)N;
   double* a = av + line * nb;
   double* b = bv + line * nb;
   double* c = cv + line * nb;
   double* f = fv + line * 5 * (size_t)N;
   auto A = [&](int i, int k, int j) -> double& { return a[25 * (size_t)i + 5 * k + j]; };
   auto Bm = [&](int i, int k, int j) -> double& { return b[25 * (size_t)i + 5 * k + j]; };
   auto C = [&](int i, int k, int j) -> double& { return c[25 * (size_t)i + 5 * k + j]; };
   auto F = [&](int i, int k) -> double& { return f[5 * (size_t)i + k]; };
   double t[5][5];
   for (int i = 0; i < N; i++) {
      if (i != 0) {
         for (int k = 0; k < 5; k++)
            for (int j = 0; j < 5; j++)
               for (int l = 0; l < 5; l++) Bm(i, k, j) -= A(i, k, l) * C(i - 1, l, j);
         for (int k = 0; k < 5; k++)
            for (int j = 0; j < 5; j++) F(i, k) -= A(i, k, j) * F(i - 1, j);
         if (periodic) {
            for (int k = 0; k < 5; k++)
               for (int j = 0; j < 5; j++) t[k][j] = 0;
            for (int k = 0; k < 5; k++)
               for (int j = 0; j < 5; j++)
                  for (int l = 0; l < 5; l++) t[k][j] -= A(i, k, l) * A(i - 1, l, j);
            for (int k = 0; k < 5; k++)
               for (int j = 0; j < 5; j++) A(i, k, j) = t[k][j];
         }
      }
      const LU5 u = lu5_factor(&Bm(i, 0, 0));
      lu5_solve(u, &F(i, 0), 1);
      if (!periodic) {
         if (i != N - 1)
            for (int j = 0; j < 5; j++) lu5_solve(u, &C(i, 0, j), 5);
      } else if (i != N - 2) {
         for (int j = 0; j < 5; j++) {
            lu5_solve(u, &C(i, 0, j), 5);
            lu5_solve(u, &A(i, 0, j), 5);
         }
      } else {
         for (int k = 0; k < 5; k++)
            for (int j = 0; j < 5; j++) C(i, j, k) += A(i, j, k);
         for (int j = 0; j < 5; j++) lu5_solve(u, &C(i, 0, j), 5);
         for (int k = 0; k < 5; k++)
            for (int j = 0; j < 5; j++) A(i, k, j) = C(i, k, j);
      }
   }
   if (!periodic) {
      for (int i = N - 2; i >= 0; i--)
         for (int k = 0; k < 5; k++)
            for (int j = 0; j < 5; j++) F(i, k) -= C(i, k, j) * F(i + 1, j);
      return;
   }
   // last-row elimination and solve (triSolvers.cpp:671-749)
   for (int k = 0; k < 5; k++)
      for (int j = 0; j < 5; j++) Bm(N - 1, j, k) = (j == k) ? 1.0 : 0.0;
   for (int i = 0; i < N - 1; i++) {
      for (int k = 0; k < 5; k++)
         for (int j = 0; j < 5; j++) t[k][j] = 0;
      for (int k = 0; k < 5; k++)
         for (int j = 0; j < 5; j++)
            for (int l = 0; l < 5; l++) {
               t[k][j] -= C(N - 1, k, l) * C(i, l, j);
               Bm(N - 1, k, j) -= C(N - 1, k, l) * A(i, l, j);
            }
      for (int k = 0; k < 5; k++)
         for (int j = 0; j < 5; j++) F(N - 1, k) -= C(N - 1, k, j) * F(i, j);
      for (int k = 0; k < 5; k++)
         for (int j = 0; j < 5; j++) C(N - 1, k, j) = t[k][j];
   }
   {
      const LU5 u = lu5_factor(&Bm(N - 1, 0, 0));
      lu5_solve(u, &F(N - 1, 0), 1);
   }
   // back substitution (triSolvers.cpp:751-765)
   for (int k = 0; k < 5; k++)
      for (int j = 0; j < 5; j++) F(N - 2, k) -= (C(N - 2, k, j) * F(N - 1, j));
   for (int i = N - 3; i >= 0; i--)
      for (int k = 0; k < 5; k++)
         for (int j = 0; j < 5; j++) F(i, k) -= (C(i, k, j) * F(i + 1, j) + A(i, k, j) * F(N - 1, j));
}

}  // namespace

extern "C" {

int hamstr_gpu_flux_roe3d(int n, const double* nxyz, const double* ql, const double* qr, double* flux, double* spec,
                          double gamma, void* stream)
{
   if (n < 0 || (n > 0 && (!nxyz || !ql || !qr || !flux || !spec))) {
      set_last_error("flux_roe3d: n >= 0 and non-null arrays");
      return HAMSTR_GPU_ERR_ARG;
   }
   if (n == 0) return HAMSTR_GPU_OK;
   flux_roe3d_kernel<<<blocks(n), kThreads, 0, (cudaStream_t)stream>>>(n, nxyz, ql, qr, gamma, flux, spec);
   return launched("flux_roe3d");
}

int hamstr_gpu_jacobian_roe3d(int n, const double* nxyz, const double* ql, const double* qr, double* lmat,
                              double* rmat, double gamma, void* stream)
{
   if (n < 0 || (n > 0 && (!nxyz || !ql || !qr || !lmat || !rmat))) {
      set_last_error("jacobian_roe3d: n >= 0 and non-null arrays");
      return HAMSTR_GPU_ERR_ARG;
   }
   if (n == 0) return HAMSTR_GPU_OK;
   jacobian_roe3d_kernel<<<blocks(n), kThreads, 0, (cudaStream_t)stream>>>(n, nxyz, ql, qr, gamma, lmat, rmat);
   return launched("jacobian_roe3d");
}

int hamstr_gpu_block_tridag5(int nlines, int N, int periodic, double* A, double* B, double* C, double* F,
                             void* stream)
{
   if (nlines < 0 || N < 1 || (periodic != 0 && periodic != 1) || (periodic && N < 2)) {
      set_last_error("block_tridag5: need nlines >= 0, N >= 1 (open) or N >= 2 (periodic)");
      return HAMSTR_GPU_ERR_ARG;
   }
   if (nlines > 0 && (!A || !B || !C || !F)) {
      set_last_error("block_tridag5: null array");
      return HAMSTR_GPU_ERR_ARG;
   }
   if (nlines == 0) return HAMSTR_GPU_OK;
   block_tridag5_kernel<<<blocks(nlines), kThreads, 0, (cudaStream_t)stream>>>(nlines, N, periodic, A, B, C, F);
   return launched("block_tridag5");
}

}  // extern "C"
