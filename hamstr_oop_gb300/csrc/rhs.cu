// ##################################################################
//
// rhs.cu -- residual, Jacobian and linear-residual kernels
//
//   rhs_face   one thread per face slot: chain stencil gather with ghost
//              states, MUSCL/WENO reconstruction, Roe flux, spectral
//              radius and the two face Jacobians
//              (computeRHS.cpp:154-370, reconstruction.cpp:16-160)
//   rhs_cell   one thread per cell: the residual and spectral-radius sums
//              in the reference's face order, the density norms, and
//              optionally the ADI initialisation (computeRHS.cpp:385-425,
//              ADI.cpp:40-49)
//   lin_face   one thread per face slot: linearised reconstruction of dq
//              and the face matrix-vector products
//              (computeLinearRHS.cpp:148-325, reconstruction.cpp:168-386)
//   lin_cell   one thread per cell: r = r0 - dq - sum(CFL/sigma * flux) in
//              face order, norms, and q += dq after the last sweep
//              (computeLinearRHS.cpp:44-368, ADI.cpp:258-264)
//
// Compiled with -fmad=false (see roe.cuh).  Sums run in the reference's
// order per cell, so every cell value is bit-identical to the reference.
// The L2 norm is reduced as a fixed-shape tree (deterministic, within a
// few ulp of the reference's serial sum); the L-infinity norm is exact.
// ##################################################################
#include "device_state.h"
#include "plan.h"
#include "roe.cuh"

namespace hamstr {

namespace {

constexpr int kThreads = 256;
constexpr double kTh = 0.3333333333333333e+00;   // THIRD (utils.h:52)
constexpr double kThm = 1.0 - kTh;
constexpr double kThp = 1.0 + kTh;
constexpr double kEps = 1e-10;                  // computeRHS.cpp:271

__device__ __forceinline__ void ld4(const double* __restrict__ p, double (&v)[4])
{
   const double2 a = *reinterpret_cast<const double2*>(p);
   const double2 b = *reinterpret_cast<const double2*>(p + 2);
   v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}

__device__ __forceinline__ void st4(double* __restrict__ p, const double (&v)[4])
{
   *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
   *reinterpret_cast<double2*>(p + 2) = make_double2(v[2], v[3]);
}

// stencil entry value (computeRHS.cpp:154-260); with DQ also the dq
// entry (computeLinearRHS.cpp:148-276)
template <bool DQ>
__device__ __forceinline__ void load_sten(const DeviceState& d, int idx, double (&f)[4], double (&df)[4])
{
   const int4 e = d.sten[idx];
   if (e.y == STEN_CELL) {
      ld4(d.q + 4 * e.x, f);
      if (DQ) ld4(d.dq + 4 * e.x, df);
   } else if (e.y == STEN_WALL) {
      const double4 R = d.refl[e.z];
      double s[4];
      ld4(d.q + 4 * e.x, s);
      f[0] = s[0];
      f[1] = (s[1] * R.x + s[2] * R.y);
      f[2] = (s[1] * R.z + s[2] * R.w);
      f[3] = s[3];
      if (DQ) {
         ld4(d.dq + 4 * e.x, s);
         df[0] = s[0];
         df[1] = (s[1] * R.x + s[2] * R.y);
         df[2] = (s[1] * R.z + s[2] * R.w);
         df[3] = s[3];
      }
   } else {
      f[0] = d.fc.rinf;
      f[1] = d.fs1;
      f[2] = d.fs2;
      f[3] = d.fc.einf;
      if (DQ) { df[0] = 0.0; df[1] = 0.0; df[2] = 0.0; df[3] = 0.0; }
   }
}

// MUSCL face states for one component from f[n-1..n+2]
// (reconstruction.cpp:170-183): left of slot n and right of slot n+1.
__device__ __forceinline__ void muscl2(double fm1, double f0, double fp1, double fp2, double& ql_n, double& qr_n1)
{
   const double qt = 0.25;
   const double f2m = f0 - fm1, f20 = fp1 - f0, f2p = fp2 - fp1;
   {
      const double a1 = 3.0 * (f20 * f2m + kEps);
      const double a2 = 2.0 * (f20 - f2m) * (f20 - f2m) + a1;
      const double f3qt = qt * (a1 / a2);
      ql_n = f0 + f3qt * (kThm * f2m + kThp * f20);
   }
   {
      const double a1 = 3.0 * (f2p * f20 + kEps);
      const double a2 = 2.0 * (f2p - f20) * (f2p - f20) + a1;
      const double f3qt = qt * (a1 / a2);
      qr_n1 = fp1 - f3qt * (kThp * f20 + kThm * f2p);
   }
}

// MUSCL_DERIV for one component (reconstruction.cpp:328-349)
__device__ __forceinline__ void muscl_deriv2(double fm1, double f0, double fp1, double fp2,
                                             double dm1, double d0, double dp1, double dp2,
                                             double& ql_n, double& qr_n1)
{
   const double qt = 0.25;
   const double f2m = f0 - fm1, f20 = fp1 - f0, f2p = fp2 - fp1;
   {
      // slot n: f2i = f20, f2i1 = f2m
      const double df2i = dp1 - d0, df2i1 = d0 - dm1;
      const double a1 = 3.0 * (f20 * f2m + kEps);
      const double da1 = 3.0 * (df2i * f2m + f20 * df2i1);
      const double a2 = 2.0 * (f20 - f2m) * (f20 - f2m) + a1;
      const double da2 = 2.0 * 2.0 * (f20 - f2m) * (df2i - df2i1) + da1;
      const double f3i = a1 / a2;
      const double df3i = da1 / a2 - a1 * da2 / (a2 * a2);
      const double f3qt = qt * f3i, df3qt = qt * df3i;
      ql_n = d0 + df3qt * (kThm * f2m + kThp * f20) + f3qt * (kThm * df2i1 + kThp * df2i);
   }
   {
      // slot n+1: f2i = f2p, f2i1 = f20
      const double df2i = dp2 - dp1, df2i1 = dp1 - d0;
      const double a1 = 3.0 * (f2p * f20 + kEps);
      const double da1 = 3.0 * (df2i * f20 + f2p * df2i1);
      const double a2 = 2.0 * (f2p - f20) * (f2p - f20) + a1;
      const double da2 = 2.0 * 2.0 * (f2p - f20) * (df2i - df2i1) + da1;
      const double f3i = a1 / a2;
      const double df3i = da1 / a2 - a1 * da2 / (a2 * a2);
      const double f3qt = qt * f3i, df3qt = qt * df3i;
      qr_n1 = dp1 - df3qt * (kThp * f20 + kThm * f2p) - f3qt * (kThp * df2i1 + kThm * df2i);
   }
}

// WENO5 (reconstruction.cpp:193-239); pow(x, 1) is x
__device__ __forceinline__ double weno5(double a, double b, double c, double d, double e)
{
   const double epsw = 1e-15;
   const double b1 = 13. / 12., b2 = 1. / 6.;
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

// WENO_5 linearisation (reconstruction.cpp:358-462); the linear residual
// passes eps = 1e-10 (computeLinearRHS.cpp:286,292)
__device__ __forceinline__ double weno5_deriv(double a, double b, double c, double d, double e,
                                              double a_d, double b_d, double c_d, double d_d, double e_d)
{
   const double epsw = 1e-10;
   const double b1 = 13. / 12., b2 = 1. / 6.;
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
   const double dbeta0 = b1 * 2 * djm1 * djm1_d + 0.25 * 2 * ejm1 * ejm1_d;
   const double dbeta1 = b1 * 2 * dj * dj_d + 0.25 * 2 * ej * ej_d;
   const double dbeta2 = b1 * 2 * djp1 * djp1_d + 0.25 * 2 * ejp1 * ejp1_d;
   const double beta0 = dis0, beta1 = dis1, beta2 = dis2;
   const double dw0_down = beta1 * beta2 + 6 * beta0 * beta2 + 3 * beta0 * beta1;
   const double dw0_up_1 = (dbeta1 * beta2 + beta1 * dbeta2) * dw0_down;
   const double dw0_up_2 = beta1 * beta2 * (dbeta1 * beta2 + beta1 * dbeta2 + 6 * (dbeta0 * beta2 + beta0 * dbeta2)
                                            + 3 * (dbeta0 * beta1 + beta0 * dbeta1));
   const double dw0 = (dw0_up_1 - dw0_up_2) / (dw0_down * dw0_down);
   const double dw1_up_1 = 6 * (dbeta0 * beta2 + beta0 * dbeta2) * dw0_down;
   const double dw1_up_2 = 6 * dw0_up_2 / beta1 * beta0;
   const double dw1 = (dw1_up_1 - dw1_up_2) / (dw0_down * dw0_down);
   const double dw2_up_1 = 3 * (dbeta0 * beta1 + beta0 * dbeta1) * dw0_down;
   const double dw2_up_2 = 3 * dw0_up_2 / beta2 * beta0;
   const double dw2 = (dw2_up_1 - dw2_up_2) / (dw0_down * dw0_down);
   return term1 + term2 + term3 + b2 * dw0 * q30 + b2 * dw1 * q31 + b2 * dw2 * q32;
}

// reconstructed states at the two sides of a face slot (computeRHS.cpp:266-304)
template <int ORDER>
__device__ __forceinline__ void face_states(const DeviceState& d, int n, bool swap, double (&L)[4], double (&R)[4])
{
   double qln[4], qrn1[4], dummy[4];
   if (ORDER == 1) {
      load_sten<false>(d, n, qln, dummy);
      load_sten<false>(d, n + 1, qrn1, dummy);
   } else if (ORDER == 3) {
      double fm1[4], f0[4], fp1[4], fp2[4];
      load_sten<false>(d, n - 1, fm1, dummy);
      load_sten<false>(d, n, f0, dummy);
      load_sten<false>(d, n + 1, fp1, dummy);
      load_sten<false>(d, n + 2, fp2, dummy);
#pragma unroll
      for (int k = 0; k < 4; k++) muscl2(fm1[k], f0[k], fp1[k], fp2[k], qln[k], qrn1[k]);
   } else {
      double f[6][4];
#pragma unroll
      for (int j = 0; j < 6; j++) load_sten<false>(d, n - 2 + j, f[j], dummy);
#pragma unroll
      for (int k = 0; k < 4; k++) {
         qln[k] = weno5(f[0][k], f[1][k], f[2][k], f[3][k], f[4][k]);
         qrn1[k] = weno5(f[5][k], f[4][k], f[3][k], f[2][k], f[1][k]);
      }
   }
#pragma unroll
   for (int k = 0; k < 4; k++) {
      L[k] = swap ? qln[k] : qrn1[k];
      R[k] = swap ? qrn1[k] : qln[k];
   }
}

// linearised states (computeLinearRHS.cpp:281-315)
template <int ORDER>
__device__ __forceinline__ void face_dstates(const DeviceState& d, int n, bool swap, double (&L)[4], double (&R)[4])
{
   double qln[4], qrn1[4];
   if (ORDER == 1) {
      double f[4];
      load_sten<true>(d, n, f, qln);
      load_sten<true>(d, n + 1, f, qrn1);
   } else if (ORDER == 3) {
      double f[4][4], df[4][4];
#pragma unroll
      for (int j = 0; j < 4; j++) load_sten<true>(d, n - 1 + j, f[j], df[j]);
#pragma unroll
      for (int k = 0; k < 4; k++)
         muscl_deriv2(f[0][k], f[1][k], f[2][k], f[3][k], df[0][k], df[1][k], df[2][k], df[3][k], qln[k], qrn1[k]);
   } else {
      double f[6][4], df[6][4];
#pragma unroll
      for (int j = 0; j < 6; j++) load_sten<true>(d, n - 2 + j, f[j], df[j]);
#pragma unroll
      for (int k = 0; k < 4; k++) {
         qln[k] = weno5_deriv(f[0][k], f[1][k], f[2][k], f[3][k], f[4][k],
                              df[0][k], df[1][k], df[2][k], df[3][k], df[4][k]);
         qrn1[k] = weno5_deriv(f[5][k], f[4][k], f[3][k], f[2][k], f[1][k],
                               df[5][k], df[4][k], df[3][k], df[2][k], df[1][k]);
      }
   }
#pragma unroll
   for (int k = 0; k < 4; k++) {
      L[k] = swap ? qln[k] : qrn1[k];
      R[k] = swap ? qrn1[k] : qln[k];
   }
}

template <int ORDER, bool JAC>
__global__ void __launch_bounds__(kThreads) rhs_face_kernel(DeviceState d)
{
   const int s = blockIdx.x * blockDim.x + threadIdx.x;
   if (s >= d.nSlot || halted(d)) return;
   const int4 sl = d.slot[s];
   const double2 nv = d.normal[s];
   double L[4], R[4];
   face_states<ORDER>(d, sl.x, (sl.w & 1) != 0, L, R);
   RoeOut o;
   double lm[16], rm[16];
   if (!roe_face<JAC>(nv.x, nv.y, L, R, d.fc.gamma, o, lm, rm)) atomicOr(d.status, DEV_ERR_NAN_SPEC);
   st4(d.flux + 4 * (size_t)s, o.flux);
   d.spec[s] = o.spec;
   if (JAC) {
      double* out = d.ff + 32 * (size_t)s;
#pragma unroll
      for (int i = 0; i < 16; i += 2) *reinterpret_cast<double2*>(out + i) = make_double2(lm[i], lm[i + 1]);
#pragma unroll
      for (int i = 0; i < 16; i += 2) *reinterpret_cast<double2*>(out + 16 + i) = make_double2(rm[i], rm[i + 1]);
   }
}

template <int ORDER>
__global__ void __launch_bounds__(kThreads) lin_face_kernel(DeviceState d)
{
   const int s = blockIdx.x * blockDim.x + threadIdx.x;
   if (s >= d.nSlot || halted(d)) return;
   const int4 sl = d.slot[s];
   double dL[4], dR[4];
   face_dstates<ORDER>(d, sl.x, (sl.w & 1) != 0, dL, dR);
   const double* m = d.ff + 32 * (size_t)(sl.w >> 1);
   double g[4];
#pragma unroll
   for (int j = 0; j < 4; j++) {
      double lrow[4], rrow[4];
      ld4(m + 4 * j, lrow);
      ld4(m + 16 + 4 * j, rrow);
      double acc = 0;
#pragma unroll
      for (int k = 0; k < 4; k++) acc += ((lrow[k] * dL[k]) + (rrow[k] * dR[k]));
      g[j] = acc;
   }
   st4(d.flux + 4 * (size_t)s, g);
}

// deterministic block reduction of {sum, max} into norm_part[blockIdx.x]
__device__ __forceinline__ void block_norm(const DeviceState& d, double sq, double am)
{
   __shared__ double s_sq[kThreads / 32], s_am[kThreads / 32];
#pragma unroll
   for (int o = 16; o > 0; o >>= 1) {
      sq += __shfl_xor_sync(0xffffffffu, sq, o);
      am = fmax(am, __shfl_xor_sync(0xffffffffu, am, o));
   }
   const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
   if (l == 0) { s_sq[w] = sq; s_am[w] = am; }
   __syncthreads();
   if (threadIdx.x == 0) {
      double a = 0.0, b = 0.0;
      for (int i = 0; i < kThreads / 32; i++) { a += s_sq[i]; b = fmax(b, s_am[i]); }
      d.norm_part[blockIdx.x] = make_double2(a, b);
   }
}

template <bool ADI_INIT>
__global__ void __launch_bounds__(kThreads) rhs_cell_kernel(DeviceState d)
{
   if (halted(d)) return;
   const int c = blockIdx.x * blockDim.x + threadIdx.x;
   double sq = 0.0, am = 0.0;
   if (c < d.nCell) {
      double r[4] = {0.0, 0.0, 0.0, 0.0};
      double sg = 0.0;
      const int e1 = d.cell_ptr[c + 1];
      for (int e = d.cell_ptr[c]; e < e1; e++) {
         const int ent = d.cell_ent[e];
         const int s = ent >> 1;
         double f[4];
         ld4(d.flux + 4 * (size_t)s, f);
         if (ent & 1) {
#pragma unroll
            for (int k = 0; k < 4; k++) r[k] += f[k];
         } else {
#pragma unroll
            for (int k = 0; k < 4; k++) r[k] -= f[k];
         }
         sg += d.spec[s];
      }
      sq = r[0] * r[0];
      am = fabs(r[0]);
      d.sigma[c] = sg;
      if (ADI_INIT) {
         const double dt = d.fc.cfl / sg;
         d.dtfac[c] = dt;
#pragma unroll
         for (int k = 0; k < 4; k++) r[k] *= dt;
         st4(d.r + 4 * (size_t)c, r);
         st4(d.r0 + 4 * (size_t)c, r);
         const double z[4] = {0.0, 0.0, 0.0, 0.0};
         st4(d.dq + 4 * (size_t)c, z);
      } else {
         st4(d.r + 4 * (size_t)c, r);
      }
   }
   block_norm(d, sq, am);
}

template <bool UPDATE_Q>
__global__ void __launch_bounds__(kThreads) lin_cell_kernel(DeviceState d)
{
   if (halted(d)) return;
   const int c = blockIdx.x * blockDim.x + threadIdx.x;
   double sq = 0.0, am = 0.0;
   if (c < d.nCell) {
      double r[4], r0[4], dq[4];
      ld4(d.r0 + 4 * (size_t)c, r0);
      ld4(d.dq + 4 * (size_t)c, dq);
#pragma unroll
      for (int k = 0; k < 4; k++) r[k] = (r0[k] - dq[k]);
      const double dt = d.dtfac[c];
      const int e1 = d.cell_ptr[c + 1];
      for (int e = d.cell_ptr[c]; e < e1; e++) {
         const int ent = d.cell_ent[e];
         double g[4];
         ld4(d.flux + 4 * (size_t)(ent >> 1), g);
         if (ent & 1) {
#pragma unroll
            for (int k = 0; k < 4; k++) r[k] += (g[k] * dt);
         } else {
#pragma unroll
            for (int k = 0; k < 4; k++) r[k] -= (g[k] * dt);
         }
      }
      st4(d.r + 4 * (size_t)c, r);
      sq = r[0] * r[0];
      am = fabs(r[0]);
      if (UPDATE_Q) {
         double q[4];
         ld4(d.q + 4 * (size_t)c, q);
#pragma unroll
         for (int k = 0; k < 4; k++) q[k] += dq[k];
         st4(d.q + 4 * (size_t)c, q);
      }
   }
   block_norm(d, sq, am);
}

__global__ void norm_final_kernel(DeviceState d, int off, int check_tol)
{
   if (halted(d)) return;
   // one warp: fixed-shape reduction of the block partials
   double a = 0.0, b = 0.0;
   for (int i = threadIdx.x; i < d.norm_blocks; i += 32) {
      const double2 p = d.norm_part[i];
      a += p.x;
      b = fmax(b, p.y);
   }
#pragma unroll
   for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b = fmax(b, __shfl_xor_sync(0xffffffffu, b, o));
   }
   if (threadIdx.x == 0) {
      const double l2 = sqrt(a) / d.nCell;
      d.norms[off] = l2;
      d.norms[off + 1] = b;
      const int it = d.ctl[1];
      if (it < d.hist_cap) {
         d.hist[4 * it + off] = l2;
         d.hist[4 * it + off + 1] = b;
      }
      if (check_tol && *d.tol > 0.0 && l2 <= *d.tol) d.ctl[0] = 1;
   }
}

__global__ void step_end_kernel(DeviceState d)
{
   if (!halted(d)) d.ctl[1] = d.ctl[1] + 1;
}

// explicit update (updateSolution, march.cpp:411-433):
// qnew = qold + (coef*CFL/sigma) * r, per cell and component
__global__ void __launch_bounds__(kThreads) update_kernel(DeviceState d, const double* __restrict__ qold,
                                                          double* __restrict__ qnew, double coef)
{
   const int c = blockIdx.x * blockDim.x + threadIdx.x;
   if (c >= d.nCell || halted(d)) return;
   const double dtfac = coef * d.fc.cfl / d.sigma[c];
   double qo[4], r[4], qn[4];
   ld4(qold + 4 * (size_t)c, qo);
   ld4(d.r + 4 * (size_t)c, r);
#pragma unroll
   for (int k = 0; k < 4; k++) qn[k] = qo[k] + dtfac * r[k];
   st4(qnew + 4 * (size_t)c, qn);
}

__global__ void __launch_bounds__(kThreads) dtfac_kernel(DeviceState d)
{
   const int c = blockIdx.x * blockDim.x + threadIdx.x;
   if (c >= d.nCell) return;
   d.dtfac[c] = d.fc.cfl / d.sigma[c];
}

__global__ void __launch_bounds__(kThreads) adi_init_kernel(DeviceState d)
{
   const int c = blockIdx.x * blockDim.x + threadIdx.x;
   if (c >= d.nCell || halted(d)) return;
   const double dt = d.fc.cfl / d.sigma[c];
   d.dtfac[c] = dt;
   double r[4];
   ld4(d.r + 4 * (size_t)c, r);
#pragma unroll
   for (int k = 0; k < 4; k++) r[k] *= dt;
   st4(d.r + 4 * (size_t)c, r);
   st4(d.r0 + 4 * (size_t)c, r);
   const double z[4] = {0.0, 0.0, 0.0, 0.0};
   st4(d.dq + 4 * (size_t)c, z);
}

__global__ void __launch_bounds__(kThreads) dq_update_kernel(DeviceState d)
{
   const int c = blockIdx.x * blockDim.x + threadIdx.x;
   if (c >= d.nCell || halted(d)) return;
   double r[4], dq[4];
   ld4(d.r + 4 * (size_t)c, r);
   ld4(d.dq + 4 * (size_t)c, dq);
#pragma unroll
   for (int k = 0; k < 4; k++) dq[k] += r[k];
   st4(d.dq + 4 * (size_t)c, dq);
}

inline int blocks_for(int n) { return (n + kThreads - 1) / kThreads; }

}  // namespace

void launch_rhs_face(const DeviceState& d, bool jac, cudaStream_t st)
{
   const int b = blocks_for(d.nSlot);
   switch (d.order * 2 + (jac ? 1 : 0)) {
      case 2: rhs_face_kernel<1, false><<<b, kThreads, 0, st>>>(d); break;
      case 3: rhs_face_kernel<1, true><<<b, kThreads, 0, st>>>(d); break;
      case 6: rhs_face_kernel<3, false><<<b, kThreads, 0, st>>>(d); break;
      case 7: rhs_face_kernel<3, true><<<b, kThreads, 0, st>>>(d); break;
      case 10: rhs_face_kernel<5, false><<<b, kThreads, 0, st>>>(d); break;
      default: rhs_face_kernel<5, true><<<b, kThreads, 0, st>>>(d); break;
   }
}

void launch_rhs_cell(const DeviceState& d, bool adi_init, cudaStream_t st)
{
   if (adi_init) rhs_cell_kernel<true><<<d.norm_blocks, kThreads, 0, st>>>(d);
   else rhs_cell_kernel<false><<<d.norm_blocks, kThreads, 0, st>>>(d);
}

void launch_lin_face(const DeviceState& d, cudaStream_t st)
{
   const int b = blocks_for(d.nSlot);
   if (d.order == 1) lin_face_kernel<1><<<b, kThreads, 0, st>>>(d);
   else if (d.order == 3) lin_face_kernel<3><<<b, kThreads, 0, st>>>(d);
   else lin_face_kernel<5><<<b, kThreads, 0, st>>>(d);
}

void launch_lin_cell(const DeviceState& d, bool update_q, cudaStream_t st)
{
   if (update_q) lin_cell_kernel<true><<<d.norm_blocks, kThreads, 0, st>>>(d);
   else lin_cell_kernel<false><<<d.norm_blocks, kThreads, 0, st>>>(d);
}

void launch_norm_final(const DeviceState& d, int off, bool check_tol, cudaStream_t st)
{
   norm_final_kernel<<<1, 32, 0, st>>>(d, off, check_tol ? 1 : 0);
}

void launch_step_end(const DeviceState& d, cudaStream_t st) { step_end_kernel<<<1, 1, 0, st>>>(d); }

void launch_update(const DeviceState& d, const double* qold, double* qnew, double coef, cudaStream_t st)
{
   update_kernel<<<blocks_for(d.nCell), kThreads, 0, st>>>(d, qold, qnew, coef);
}

void launch_dtfac(const DeviceState& d, cudaStream_t st)
{
   dtfac_kernel<<<blocks_for(d.nCell), kThreads, 0, st>>>(d);
}

void launch_adi_init(const DeviceState& d, cudaStream_t st)
{
   adi_init_kernel<<<blocks_for(d.nCell), kThreads, 0, st>>>(d);
}

void launch_dq_update(const DeviceState& d, cudaStream_t st)
{
   dq_update_kernel<<<blocks_for(d.nCell), kThreads, 0, st>>>(d);
}

}  // namespace hamstr
