// ##################################################################
//
// recon.cuh -- chain stencil gather and reconstructions along a chain
//
// Shared by the FP64 path (rhs.cu, T = double: the reference's arithmetic
// and order, bit-identical) and the mixed-precision path (mixed.cu, the
// linearised reconstruction with T = float).  Every literal goes through
// T(...), so the double instantiation is exactly the reference's
// expression while the float one stays in single precision.
// ##################################################################
#ifndef HAMSTR_GPU_RECON_CUH
#define HAMSTR_GPU_RECON_CUH

#include "device_state.h"
#include "plan.h"
#include "softdiv.cuh"

namespace hamstr {

constexpr double kTh = 0.3333333333333333e+00;   // THIRD (utils.h:52)
constexpr double kEps = 1e-10;                  // computeRHS.cpp:271

// Reconstruction codes (template argument ORDER): 1, 3 (MUSCL with the
// reference's limiter, reconstruction.cpp:16-70), 5 (WENO), and MUSCL with
// one of the project's limiters (no reference counterpart):
//   31  minmod-limited differences of the kappa scheme (Anderson, Thomas and
//       van Leer, AIAA J. 24(9), 1986): a~ = minmod(a, b*beta),
//       b~ = minmod(b, a*beta), beta = (3 - kappa)/(1 - kappa) = 4;
//       ql = f + qt (thm a~ + thp b~), qr = f - qt (thp a~ + thm b~)
//   32  van Albada's differentiable limiter in the same paper's form:
//       s = (2ab + eps)/(a^2 + b^2 + eps), sk = kappa s;
//       ql = f + qt s ((1 - sk) a + (1 + sk) b),
//       qr = f - qt s ((1 + sk) a + (1 - sk) b)
// with a = f_i - f_{i-1}, b = f_{i+1} - f_i, kappa = 1/3, qt = 1/4.  The
// linearised forms (for the sweeps' residual) are the exact derivatives,
// minmod with its selection frozen.
enum { RECON_MUSCL_MINMOD = 31, RECON_MUSCL_VANALBADA = 32 };
__host__ __device__ constexpr bool is_muscl(int r) { return r == 3 || r == RECON_MUSCL_MINMOD || r == RECON_MUSCL_VANALBADA; }

__device__ __forceinline__ void ld4(const double* __restrict__ p, double (&v)[4])
{
   const double2 a = *reinterpret_cast<const double2*>(p);
   const double2 b = *reinterpret_cast<const double2*>(p + 2);
   v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}

__device__ __forceinline__ void ld4(const float* __restrict__ p, float (&v)[4])
{
   const float4 a = *reinterpret_cast<const float4*>(p);
   v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
}

__device__ __forceinline__ void st4(double* __restrict__ p, const double (&v)[4])
{
   *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
   *reinterpret_cast<double2*>(p + 2) = make_double2(v[2], v[3]);
}

__device__ __forceinline__ void st4(float* __restrict__ p, const float (&v)[4])
{
   *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}

// stencil entry value (computeRHS.cpp:154-260), and with dqv also the dq
// entry (computeLinearRHS.cpp:148-276); q is read in FP64 and rounded to T
template <typename T, bool DQ>
__device__ __forceinline__ void load_sten(const DeviceState& d, const T* __restrict__ dqv, int idx, T (&f)[4],
                                          T (&df)[4])
{
   const int4 e = d.sten[idx];
   if (e.y == STEN_CELL) {
      double s[4];
      ld4(d.q + 4 * e.x, s);
#pragma unroll
      for (int k = 0; k < 4; k++) f[k] = T(s[k]);
      if (DQ) ld4(dqv + 4 * e.x, df);
   } else if (e.y == STEN_WALL) {
      const double4 R = d.refl[e.z];
      const T rx = T(R.x), ry = T(R.y), rz = T(R.z), rw = T(R.w);
      double s[4];
      ld4(d.q + 4 * e.x, s);
      const T s0 = T(s[0]), s1 = T(s[1]), s2 = T(s[2]), s3 = T(s[3]);
      f[0] = s0;
      f[1] = (s1 * rx + s2 * ry);
      f[2] = (s1 * rz + s2 * rw);
      f[3] = s3;
      if (DQ) {
         T t[4];
         ld4(dqv + 4 * e.x, t);
         df[0] = t[0];
         df[1] = (t[1] * rx + t[2] * ry);
         df[2] = (t[1] * rz + t[2] * rw);
         df[3] = t[3];
      }
   } else {
      const double4 fsv = d.fstab[e.w];   // the entry's instance
      f[0] = T(fsv.x);
      f[1] = T(fsv.y);
      f[2] = T(fsv.z);
      f[3] = T(fsv.w);
      if (DQ) { df[0] = T(0); df[1] = T(0); df[2] = T(0); df[3] = T(0); }
   }
}

// the increment part of load_sten alone (dq of a cell, its wall mirror, or
// zero at a far-field ghost)
template <typename T>
__device__ __forceinline__ void load_dsten(const DeviceState& d, const T* __restrict__ dqv, int idx, T (&df)[4])
{
   const int4 e = d.sten[idx];
   if (e.y == STEN_CELL) {
      ld4(dqv + 4 * e.x, df);
   } else if (e.y == STEN_WALL) {
      const double4 R = d.refl[e.z];
      const T rx = T(R.x), ry = T(R.y), rz = T(R.z), rw = T(R.w);
      T t[4];
      ld4(dqv + 4 * e.x, t);
      df[0] = t[0];
      df[1] = (t[1] * rx + t[2] * ry);
      df[2] = (t[1] * rz + t[2] * rw);
      df[3] = t[3];
   } else {
      df[0] = T(0);
      df[1] = T(0);
      df[2] = T(0);
      df[3] = T(0);
   }
}

// component k of stencil entry idx, as load_sten<double, false> forms it
__device__ __forceinline__ double sten_comp(const DeviceState& d, int idx, int k)
{
   const int4 e = d.sten[idx];
   if (e.y == STEN_CELL) return d.q[4 * (size_t)e.x + k];
   if (e.y == STEN_WALL) {
      const double* s = d.q + 4 * (size_t)e.x;
      if (k == 0 || k == 3) return s[k];
      const double4 R = d.refl[e.z];
      const double s1 = s[1], s2 = s[2];
      return k == 1 ? (s1 * R.x + s2 * R.y) : (s1 * R.z + s2 * R.w);
   }
   const double4 f = d.fstab[e.w];
   return k == 0 ? f.x : k == 1 ? f.y : k == 2 ? f.z : f.w;
}

// MUSCL face states for one component from f[n-1..n+2]
// (reconstruction.cpp:170-183): left state of slot n, right of slot n+1
__device__ __forceinline__ void muscl2(double fm1, double f0, double fp1, double fp2, double& ql_n, double& qr_n1)
{
   const double qt = 0.25;
   const double thm = 1.0 - kTh, thp = 1.0 + kTh;
   const double f2m = f0 - fm1, f20 = fp1 - f0, f2p = fp2 - fp1;
   {
      const double a1 = 3.0 * (f20 * f2m + kEps);
      const double a2 = 2.0 * (f20 - f2m) * (f20 - f2m) + a1;
      const double f3qt = qt * (a1 / a2);
      ql_n = f0 + f3qt * (thm * f2m + thp * f20);
   }
   {
      const double a1 = 3.0 * (f2p * f20 + kEps);
      const double a2 = 2.0 * (f2p - f20) * (f2p - f20) + a1;
      const double f3qt = qt * (a1 / a2);
      qr_n1 = fp1 - f3qt * (thp * f20 + thm * f2p);
   }
}

// minmod(x, y) as a selection: 0 -> 0, 1 -> x, 2 -> y
__device__ __forceinline__ int minmod_sel(double x, double y)
{
   if (x > 0.0) return (y <= 0.0) ? 0 : ((x <= y) ? 1 : 2);
   if (x < 0.0) return (y >= 0.0) ? 0 : ((x >= y) ? 1 : 2);
   return 0;
}
template <typename T>
__device__ __forceinline__ T pick(int sel, T x, T y) { return sel == 0 ? T(0) : (sel == 1 ? x : y); }

// project limiters (RECON_MUSCL_MINMOD / _VANALBADA), one cell: ql, qr at
// its two faces from a = f - fm, b = fp - f
template <int R>
__device__ __forceinline__ void muscl_lim_cell(double f, double a, double b, double& ql, double& qr)
{
   const double qt = 0.25;
   const double thm = 1.0 - kTh, thp = 1.0 + kTh;
   if (R == RECON_MUSCL_MINMOD) {
      const double at = pick<double>(minmod_sel(a, 4.0 * b), a, 4.0 * b);
      const double bt = pick<double>(minmod_sel(b, 4.0 * a), b, 4.0 * a);
      ql = f + qt * (thm * at + thp * bt);
      qr = f - qt * (thp * at + thm * bt);
   } else {
      const double s = (2.0 * a * b + kEps) / (a * a + b * b + kEps);
      const double sk = kTh * s;
      ql = f + (qt * s) * ((1.0 - sk) * a + (1.0 + sk) * b);
      qr = f - (qt * s) * ((1.0 + sk) * a + (1.0 - sk) * b);
   }
}

template <int R>
__device__ __forceinline__ void muscl2_lim(double fm1, double f0, double fp1, double fp2, double& ql_n, double& qr_n1)
{
   double dummy;
   muscl_lim_cell<R>(f0, f0 - fm1, fp1 - f0, ql_n, dummy);
   muscl_lim_cell<R>(fp1, fp1 - f0, fp2 - fp1, dummy, qr_n1);
}

// linearisation of muscl_lim_cell: dql, dqr from the state differences
// (a, b) and their perturbations (da, db)
template <int R, typename T>
__device__ __forceinline__ void muscl_lim_dcell(T df, T a, T b, T da, T db, T& dql, T& dqr)
{
   const T qt = T(0.25);
   const T thm = T(1.0 - kTh), thp = T(1.0 + kTh);
   if (R == RECON_MUSCL_MINMOD) {
      const int sa = minmod_sel(double(a), 4.0 * double(b));
      const int sb = minmod_sel(double(b), 4.0 * double(a));
      const T dat = pick<T>(sa, da, T(4.0) * db);
      const T dbt = pick<T>(sb, db, T(4.0) * da);
      dql = df + qt * (thm * dat + thp * dbt);
      dqr = df - qt * (thp * dat + thm * dbt);
   } else {
      const T eps = T(kEps), kt = T(kTh);
      const T den = a * a + b * b + eps;
      const T s = (T(2.0) * a * b + eps) / den;
      const T ds = (T(2.0) * (da * b + a * db) - s * (T(2.0) * (a * da + b * db))) / den;
      const T sk = kt * s, dsk = kt * ds;
      const T A = (T(1.0) - sk) * a + (T(1.0) + sk) * b;
      const T dA = (T(1.0) - sk) * da + (T(1.0) + sk) * db + dsk * (b - a);
      const T B = (T(1.0) + sk) * a + (T(1.0) - sk) * b;
      const T dB = (T(1.0) + sk) * da + (T(1.0) - sk) * db + dsk * (a - b);
      dql = df + qt * (ds * A + s * dA);
      dqr = df - qt * (ds * B + s * dB);
   }
}

template <int R, typename T>
__device__ __forceinline__ void muscl_deriv2_lim(T fm1, T f0, T fp1, T fp2, T dm1, T d0, T dp1, T dp2, T& ql_n,
                                                 T& qr_n1)
{
   T dummy;
   muscl_lim_dcell<R, T>(d0, f0 - fm1, fp1 - f0, d0 - dm1, dp1 - d0, ql_n, dummy);
   muscl_lim_dcell<R, T>(dp1, fp1 - f0, fp2 - fp1, dp1 - d0, dp2 - dp1, dummy, qr_n1);
}

// MUSCL_DERIV for one component (reconstruction.cpp:328-349)
template <typename T>
__device__ __forceinline__ void muscl_deriv2(T fm1, T f0, T fp1, T fp2, T dm1, T d0, T dp1, T dp2, T& ql_n, T& qr_n1)
{
   const T qt = T(0.25);
   const T thm = T(1.0 - kTh), thp = T(1.0 + kTh), eps = T(kEps);
   const T f2m = f0 - fm1, f20 = fp1 - f0, f2p = fp2 - fp1;
   {
      // slot n: f2i = f20, f2i1 = f2m
      const T df2i = dp1 - d0, df2i1 = d0 - dm1;
      const T a1 = T(3.0) * (f20 * f2m + eps);
      const T da1 = T(3.0) * (df2i * f2m + f20 * df2i1);
      const T a2 = T(2.0) * (f20 - f2m) * (f20 - f2m) + a1;
      const T da2 = T(2.0 * 2.0) * (f20 - f2m) * (df2i - df2i1) + da1;
      const T f3i = a1 / a2;
      const T df3i = da1 / a2 - a1 * da2 / (a2 * a2);
      const T f3qt = qt * f3i, df3qt = qt * df3i;
      ql_n = d0 + df3qt * (thm * f2m + thp * f20) + f3qt * (thm * df2i1 + thp * df2i);
   }
   {
      // slot n+1: f2i = f2p, f2i1 = f20
      const T df2i = dp2 - dp1, df2i1 = dp1 - d0;
      const T a1 = T(3.0) * (f2p * f20 + eps);
      const T da1 = T(3.0) * (df2i * f20 + f2p * df2i1);
      const T a2 = T(2.0) * (f2p - f20) * (f2p - f20) + a1;
      const T da2 = T(2.0 * 2.0) * (f2p - f20) * (df2i - df2i1) + da1;
      const T f3i = a1 / a2;
      const T df3i = da1 / a2 - a1 * da2 / (a2 * a2);
      const T f3qt = qt * f3i, df3qt = qt * df3i;
      qr_n1 = dp1 - df3qt * (thp * f20 + thm * f2p) - f3qt * (thp * df2i1 + thm * df2i);
   }
}

// WENO5 (reconstruction.cpp:193-239); pow(x, 1) is x.  With SD the
// multiplies run on the integer pipes (p2, pm: identical results)
template <bool SD>
__device__ __forceinline__ double weno5(double a, double b, double c, double d, double e)
{
   const double epsw = 1e-15;
   const double b1 = 13. / 12., b2 = 1. / 6.;
   const double c3 = pm<SD>(3., c);
   const double djm1 = a - p2<1, SD>(b) + c;
   const double ejm1 = a - p2<2, SD>(b) + c3;
   const double dj = b - p2<1, SD>(c) + d;
   const double ej = b - d;
   const double djp1 = c - p2<1, SD>(d) + e;
   const double ejp1 = c3 - p2<2, SD>(d) + e;
   const double dis0 = pm<SD>(pm<SD>(b1, djm1), djm1) + pm<SD>(p2<-2, SD>(ejm1), ejm1) + epsw;
   const double dis1 = pm<SD>(pm<SD>(b1, dj), dj) + pm<SD>(p2<-2, SD>(ej), ej) + epsw;
   const double dis2 = pm<SD>(pm<SD>(b1, djp1), djp1) + pm<SD>(p2<-2, SD>(ejp1), ejp1) + epsw;
   const double q30 = p2<1, SD>(a) - pm<SD>(7., b) + pm<SD>(11., c);
   const double q31 = -b + pm<SD>(5., c) + p2<1, SD>(d);
   const double q32 = p2<1, SD>(c) + pm<SD>(5., d) - e;
   const double d01 = Dv<double, SD>(dis1).div(dis0);
   const double d02 = Dv<double, SD>(dis2).div(dis0);
   const double a1ba0 = pm<SD>(6., d01);
   const double a2ba0 = pm<SD>(3., d02);
   const double w0 = Dv<double, SD>(1.0 + a1ba0 + a2ba0).div(1.0);
   const double w1 = pm<SD>(a1ba0, w0);
   const double w2 = 1. - w0 - w1;
   return pm<SD>(b2, pm<SD>(w0, q30) + pm<SD>(w1, q31) + pm<SD>(w2, q32));
}

// WENO_5 linearisation (reconstruction.cpp:358-462); the linear residual
// passes eps = 1e-10 (computeLinearRHS.cpp:286,292).  Split in two: the
// values formed from the states alone (Weno5Lin, weno5_lin_pre), which stay
// fixed while q does -- through every sweep of a pseudo-time step -- and
// the part that takes the increments (weno5_lin_apply).  weno5_deriv is the
// two in sequence, the same operations in the same order.
template <typename T>
struct Weno5Lin {
   T cdjm1, cejm1, cdj, cej, cdjp1, cejp1;   // (13/12 * 2) d_k and (0.25 * 2) e_k: the dbeta_k coefficients
   T beta0, beta1, beta2, bb12;              // smoothness sums with eps; beta1 * beta2
   T q30, q31, q32;                          // candidate stencils
   T b2w0, b2w1, b2w2;                       // 1/6 * weights
   T dwd, dwd2;                              // the weights' common denominator and its square
};
constexpr int kWeno5LinVals = 18;
static_assert(2 * 4 * kWeno5LinVals == kWlinPerSlot, "kept WENO values per face slot");

template <typename T>
__device__ __forceinline__ void weno5_lin_put(const Weno5Lin<T>& p, T* __restrict__ out, size_t stride)
{
   const T v[kWeno5LinVals] = {p.cdjm1, p.cejm1, p.cdj,  p.cej,  p.cdjp1, p.cejp1, p.beta0, p.beta1, p.beta2,
                               p.bb12,  p.q30,   p.q31,  p.q32,  p.b2w0,  p.b2w1,  p.b2w2,  p.dwd,   p.dwd2};
#pragma unroll
   for (int i = 0; i < kWeno5LinVals; i++) out[stride * i] = v[i];
}

template <typename T>
__device__ __forceinline__ Weno5Lin<T> weno5_lin_get(const T* __restrict__ in, size_t stride)
{
   T v[kWeno5LinVals];
#pragma unroll
   for (int i = 0; i < kWeno5LinVals; i++) v[i] = in[stride * i];
   Weno5Lin<T> p;
   p.cdjm1 = v[0]; p.cejm1 = v[1]; p.cdj = v[2]; p.cej = v[3]; p.cdjp1 = v[4]; p.cejp1 = v[5];
   p.beta0 = v[6]; p.beta1 = v[7]; p.beta2 = v[8]; p.bb12 = v[9];
   p.q30 = v[10]; p.q31 = v[11]; p.q32 = v[12];
   p.b2w0 = v[13]; p.b2w1 = v[14]; p.b2w2 = v[15];
   p.dwd = v[16]; p.dwd2 = v[17];
   return p;
}

// the f-only values from the differences d_k, e_k, the smoothness sums
// (eps added) and the candidate stencils; shared by weno5_lin_pre and
// weno5_with_lin.  Each is an intermediate value of the reference's
// expressions, formed the same way (b1 * 2 is exact).
// The linearisation's multiplies: its divisions already load the integer
// pipes, so only the increment part's first multiplies (candidate
// stencils, the weight and smoothness derivative terms) go there with SD,
// about half of them, and the rest stay on the FP64 pipe (all of them
// there, or none, measured slower)
constexpr bool kLinSoftMul = false;

template <typename T, bool SD>
__device__ __forceinline__ void weno5_lin_fill(Weno5Lin<T>& p, T djm1, T ejm1, T dj, T ej, T djp1, T ejp1)
{
   const T b1 = T(13. / 12.), b2 = T(1. / 6.);
   const T c1 = b1 * T(2);   // exact; the e_k coefficients are 0.25 * 2 = 2^-1
   p.cdjm1 = pm<kLinSoftMul>(c1, djm1);
   p.cejm1 = p2<-1, SD>(ejm1);
   p.cdj = pm<kLinSoftMul>(c1, dj);
   p.cej = p2<-1, SD>(ej);
   p.cdjp1 = pm<kLinSoftMul>(c1, djp1);
   p.cejp1 = p2<-1, SD>(ejp1);
   const Dv<T, SD> r1(p.beta1), r2(p.beta2);
   const T d01 = r1.div(p.beta0);
   const T d02 = r2.div(p.beta0);
   const T a1ba0 = pm<kLinSoftMul>(T(6.), d01);
   const T a2ba0 = pm<kLinSoftMul>(T(3.), d02);
   const T w0 = Dv<T, SD>(T(1.0) + a1ba0 + a2ba0).div(T(1.0));
   const T w1 = pm<kLinSoftMul>(a1ba0, w0);
   const T w2 = T(1.) - w0 - w1;
   p.b2w0 = pm<kLinSoftMul>(b2, w0);
   p.b2w1 = pm<kLinSoftMul>(b2, w1);
   p.b2w2 = pm<kLinSoftMul>(b2, w2);
   p.bb12 = pm<kLinSoftMul>(p.beta1, p.beta2);
   p.dwd = p.bb12 + pm<kLinSoftMul>(pm<kLinSoftMul>(T(6), p.beta0), p.beta2) + pm<kLinSoftMul>(pm<kLinSoftMul>(T(3), p.beta0), p.beta1);
   p.dwd2 = pm<kLinSoftMul>(p.dwd, p.dwd);
}

template <typename T, bool SD>
__device__ __forceinline__ Weno5Lin<T> weno5_lin_pre(T a, T b, T c, T d, T e)
{
   const T epsw = T(1e-10);
   const T b1 = T(13. / 12.);
   Weno5Lin<T> p;
   const T c3 = pm<kLinSoftMul>(T(3.), c);
   const T djm1 = a - p2<1, SD>(b) + c;
   const T ejm1 = a - p2<2, SD>(b) + c3;
   const T dj = b - p2<1, SD>(c) + d;
   const T ej = b - d;
   const T djp1 = c - p2<1, SD>(d) + e;
   const T ejp1 = c3 - p2<2, SD>(d) + e;
   p.beta0 = pm<kLinSoftMul>(pm<kLinSoftMul>(b1, djm1), djm1) + pm<kLinSoftMul>(p2<-2, SD>(ejm1), ejm1) + epsw;
   p.beta1 = pm<kLinSoftMul>(pm<kLinSoftMul>(b1, dj), dj) + pm<kLinSoftMul>(p2<-2, SD>(ej), ej) + epsw;
   p.beta2 = pm<kLinSoftMul>(pm<kLinSoftMul>(b1, djp1), djp1) + pm<kLinSoftMul>(p2<-2, SD>(ejp1), ejp1) + epsw;
   p.q30 = p2<1, SD>(a) - pm<kLinSoftMul>(T(7.), b) + pm<kLinSoftMul>(T(11.), c);
   p.q31 = -b + pm<kLinSoftMul>(T(5.), c) + p2<1, SD>(d);
   p.q32 = p2<1, SD>(c) + pm<kLinSoftMul>(T(5.), d) - e;
   weno5_lin_fill<T, SD>(p, djm1, ejm1, dj, ej, djp1, ejp1);
   return p;
}

template <typename T, bool SD>
__device__ __forceinline__ T weno5_lin_apply(const Weno5Lin<T>& p, T a_d, T b_d, T c_d, T d_d, T e_d)
{
   const T b2 = T(1. / 6.);
   const T c3 = pm<SD>(T(3.), c_d);
   const T djm1_d = a_d - p2<1, SD>(b_d) + c_d;
   const T ejm1_d = a_d - p2<2, SD>(b_d) + c3;
   const T dj_d = b_d - p2<1, SD>(c_d) + d_d;
   const T ej_d = b_d - d_d;
   const T djp1_d = c_d - p2<1, SD>(d_d) + e_d;
   const T ejp1_d = c3 - p2<2, SD>(d_d) + e_d;
   const T q30_d = p2<1, SD>(a_d) - pm<SD>(T(7.), b_d) + pm<SD>(T(11.), c_d);
   const T q31_d = -b_d + pm<SD>(T(5.), c_d) + p2<1, SD>(d_d);
   const T q32_d = p2<1, SD>(c_d) + pm<SD>(T(5.), d_d) - e_d;
   const T term1 = pm<SD>(p.b2w0, q30_d);
   const T term2 = pm<SD>(p.b2w1, q31_d);
   const T term3 = pm<SD>(p.b2w2, q32_d);
   const T dbeta0 = pm<SD>(p.cdjm1, djm1_d) + pm<SD>(p.cejm1, ejm1_d);
   const T dbeta1 = pm<SD>(p.cdj, dj_d) + pm<SD>(p.cej, ej_d);
   const T dbeta2 = pm<SD>(p.cdjp1, djp1_d) + pm<SD>(p.cejp1, ejp1_d);
   const T beta0 = p.beta0, beta1 = p.beta1, beta2 = p.beta2;
   const T dw0_down = p.dwd;
   const T s12 = pm<kLinSoftMul>(dbeta1, beta2) + pm<kLinSoftMul>(beta1, dbeta2);
   const T s6 = pm<kLinSoftMul>(T(6), pm<kLinSoftMul>(dbeta0, beta2) + pm<kLinSoftMul>(beta0, dbeta2));
   const T s3 = pm<kLinSoftMul>(T(3), pm<kLinSoftMul>(dbeta0, beta1) + pm<kLinSoftMul>(beta0, dbeta1));
   const T dw0_up_1 = pm<SD>(s12, dw0_down);
   const T dw0_up_2 = pm<kLinSoftMul>(p.bb12, s12 + s6 + s3);
   const Dv<T, SD> rd(p.dwd2);
   const T dw0 = rd.div(dw0_up_1 - dw0_up_2);
   const T dw1_up_1 = pm<SD>(s6, dw0_down);
   const T dw1_up_2 = pm<kLinSoftMul>(Dv<T, SD>(beta1).div(pm<kLinSoftMul>(T(6), dw0_up_2)), beta0);
   const T dw1 = rd.div(dw1_up_1 - dw1_up_2);
   const T dw2_up_1 = pm<SD>(s3, dw0_down);
   const T dw2_up_2 = pm<kLinSoftMul>(Dv<T, SD>(beta2).div(pm<kLinSoftMul>(T(3), dw0_up_2)), beta0);
   const T dw2 = rd.div(dw2_up_1 - dw2_up_2);
   return term1 + term2 + term3 + pm<kLinSoftMul>(pm<kLinSoftMul>(b2, dw0), p.q30) + pm<kLinSoftMul>(pm<kLinSoftMul>(b2, dw1), p.q31) +
          pm<kLinSoftMul>(pm<kLinSoftMul>(b2, dw2), p.q32);
}

template <typename T, bool SD>
__device__ __forceinline__ T weno5_deriv(T a, T b, T c, T d, T e, T a_d, T b_d, T c_d, T d_d, T e_d)
{
   return weno5_lin_apply<T, SD>(weno5_lin_pre<T, SD>(a, b, c, d, e), a_d, b_d, c_d, d_d, e_d);
}

// weno5 and, from the same differences, the f-only values of its
// linearisation: the smoothness sums differ only in the eps added last
// (1e-15 here, 1e-10 there), so the sum before it is shared
template <bool SD>
__device__ __forceinline__ double weno5_with_lin(double a, double b, double c, double d, double e,
                                                 Weno5Lin<double>& p)
{
   const double b1 = 13. / 12., b2 = 1. / 6.;
   const double c3 = pm<SD>(3., c);
   const double djm1 = a - p2<1, SD>(b) + c;
   const double ejm1 = a - p2<2, SD>(b) + c3;
   const double dj = b - p2<1, SD>(c) + d;
   const double ej = b - d;
   const double djp1 = c - p2<1, SD>(d) + e;
   const double ejp1 = c3 - p2<2, SD>(d) + e;
   const double s0 = pm<SD>(pm<SD>(b1, djm1), djm1) + pm<SD>(p2<-2, SD>(ejm1), ejm1);
   const double s1 = pm<SD>(pm<SD>(b1, dj), dj) + pm<SD>(p2<-2, SD>(ej), ej);
   const double s2 = pm<SD>(pm<SD>(b1, djp1), djp1) + pm<SD>(p2<-2, SD>(ejp1), ejp1);
   const double dis0 = s0 + 1e-15, dis1 = s1 + 1e-15, dis2 = s2 + 1e-15;
   p.q30 = p2<1, SD>(a) - pm<SD>(7., b) + pm<SD>(11., c);
   p.q31 = -b + pm<SD>(5., c) + p2<1, SD>(d);
   p.q32 = p2<1, SD>(c) + pm<SD>(5., d) - e;
   const double d01 = Dv<double, SD>(dis1).div(dis0);
   const double d02 = Dv<double, SD>(dis2).div(dis0);
   const double a1ba0 = pm<kLinSoftMul>(6., d01);
   const double a2ba0 = pm<kLinSoftMul>(3., d02);
   const double w0 = Dv<double, SD>(1.0 + a1ba0 + a2ba0).div(1.0);
   const double w1 = pm<kLinSoftMul>(a1ba0, w0);
   const double w2 = 1. - w0 - w1;
   p.beta0 = s0 + 1e-10;
   p.beta1 = s1 + 1e-10;
   p.beta2 = s2 + 1e-10;
   weno5_lin_fill<double, SD>(p, djm1, ejm1, dj, ej, djp1, ejp1);
   return pm<kLinSoftMul>(b2, pm<kLinSoftMul>(w0, p.q30) + pm<kLinSoftMul>(w1, p.q31) + pm<kLinSoftMul>(w2, p.q32));
}

// reconstructed states at the two sides of a face slot, FP64
// (computeRHS.cpp:266-304)
template <int ORDER, bool SD = true>
__device__ __forceinline__ void face_states(const DeviceState& d, int n, bool swap, double (&L)[4], double (&R)[4])
{
   double qln[4], qrn1[4], dummy[4];
   if (ORDER == 1) {
      load_sten<double, false>(d, nullptr, n, qln, dummy);
      load_sten<double, false>(d, nullptr, n + 1, qrn1, dummy);
   } else if (is_muscl(ORDER)) {
      double fm1[4], f0[4], fp1[4], fp2[4];
      load_sten<double, false>(d, nullptr, n - 1, fm1, dummy);
      load_sten<double, false>(d, nullptr, n, f0, dummy);
      load_sten<double, false>(d, nullptr, n + 1, fp1, dummy);
      load_sten<double, false>(d, nullptr, n + 2, fp2, dummy);
#pragma unroll
      for (int k = 0; k < 4; k++) {
         if (ORDER == 3) muscl2(fm1[k], f0[k], fp1[k], fp2[k], qln[k], qrn1[k]);
         else muscl2_lim<ORDER>(fm1[k], f0[k], fp1[k], fp2[k], qln[k], qrn1[k]);
      }
   } else {
      double f[6][4];
#pragma unroll
      for (int j = 0; j < 6; j++) load_sten<double, false>(d, nullptr, n - 2 + j, f[j], dummy);
#pragma unroll
      for (int k = 0; k < 4; k++) {
         qln[k] = weno5<SD>(f[0][k], f[1][k], f[2][k], f[3][k], f[4][k]);
         qrn1[k] = weno5<SD>(f[5][k], f[4][k], f[3][k], f[2][k], f[1][k]);
      }
   }
#pragma unroll
   for (int k = 0; k < 4; k++) {
      L[k] = swap ? qln[k] : qrn1[k];
      R[k] = swap ? qrn1[k] : qln[k];
   }
}

// linearised states (computeLinearRHS.cpp:281-315) in T, dq from dqv
template <int ORDER, typename T, bool SD = true>
__device__ __forceinline__ void face_dstates(const DeviceState& d, const T* __restrict__ dqv, int n, bool swap,
                                             T (&L)[4], T (&R)[4])
{
   T qln[4], qrn1[4];
   if (ORDER == 1) {
      T f[4];
      load_sten<T, true>(d, dqv, n, f, qln);
      load_sten<T, true>(d, dqv, n + 1, f, qrn1);
   } else if (is_muscl(ORDER)) {
      T f[4][4], df[4][4];
#pragma unroll
      for (int j = 0; j < 4; j++) load_sten<T, true>(d, dqv, n - 1 + j, f[j], df[j]);
#pragma unroll
      for (int k = 0; k < 4; k++) {
         if (ORDER == 3)
            muscl_deriv2<T>(f[0][k], f[1][k], f[2][k], f[3][k], df[0][k], df[1][k], df[2][k], df[3][k], qln[k],
                            qrn1[k]);
         else
            muscl_deriv2_lim<ORDER, T>(f[0][k], f[1][k], f[2][k], f[3][k], df[0][k], df[1][k], df[2][k], df[3][k],
                                       qln[k], qrn1[k]);
      }
   } else {
      T f[6][4], df[6][4];
#pragma unroll
      for (int j = 0; j < 6; j++) load_sten<T, true>(d, dqv, n - 2 + j, f[j], df[j]);
#pragma unroll
      for (int k = 0; k < 4; k++) {
         qln[k] = weno5_deriv<T, SD>(f[0][k], f[1][k], f[2][k], f[3][k], f[4][k], df[0][k], df[1][k], df[2][k],
                                 df[3][k], df[4][k]);
         qrn1[k] = weno5_deriv<T, SD>(f[5][k], f[4][k], f[3][k], f[2][k], f[1][k], df[5][k], df[4][k], df[3][k],
                                  df[2][k], df[1][k]);
      }
   }
#pragma unroll
   for (int k = 0; k < 4; k++) {
      L[k] = swap ? qln[k] : qrn1[k];
      R[k] = swap ? qrn1[k] : qln[k];
   }
}

// One order-5 face state: component k of side `side` (0: left-biased at
// stencil n, 1: right-biased at n+1) of slot s, into d.qface[(4*side + k) *
// nSlot + s]; with WL also the f-only values of its linearisation into
// d.wlin[(18*(4*side + k) + v) * nSlot + s].  The face kernels then read the
// states: computeRHS.cpp:266-304 with its 8 reconstructions per face spread
// over 8 threads.
template <bool SD, bool WL>
__device__ __forceinline__ void recon5_one(const DeviceState& d, int s, int side, int k)
{
   const int n = d.slot[s].x;
   double f[6];
#pragma unroll
   for (int j = 0; j < 6; j++) f[j] = sten_comp(d, n - 2 + j, k);
   const double a = side ? f[5] : f[0], b = side ? f[4] : f[1], c = side ? f[3] : f[2];
   const double e4 = side ? f[2] : f[3], e5 = side ? f[1] : f[4];
   const size_t ns = (size_t)d.nSlot;
   const int sk = 4 * side + k;
   double v;
   if (WL) {
      Weno5Lin<double> p;
      v = weno5_with_lin<SD>(a, b, c, e4, e5, p);
      weno5_lin_put(p, d.wlin + (size_t)(kWeno5LinVals * sk) * ns + s, ns);
   } else {
      v = weno5<SD>(a, b, c, e4, e5);
   }
   d.qface[(size_t)sk * ns + s] = v;
}

// component k of stencil entry idx of the increments dqv, as load_dsten
// forms it
__device__ __forceinline__ double dsten_comp(const DeviceState& d, const double* __restrict__ dqv, int idx, int k)
{
   const int4 e = d.sten[idx];
   if (e.y == STEN_CELL) return dqv[4 * (size_t)e.x + k];
   if (e.y == STEN_WALL) {
      const double* t = dqv + 4 * (size_t)e.x;
      if (k == 0 || k == 3) return t[k];
      const double4 R = d.refl[e.z];
      const double t1 = t[1], t2 = t[2];
      return k == 1 ? (t1 * R.x + t2 * R.y) : (t1 * R.z + t2 * R.w);
   }
   return 0.0;
}

// One linearised order-5 face state (computeLinearRHS.cpp:281-315) of
// slot s into d.qface, like recon5_one: from the f-only values the
// implicit computeRHS kept (WL) or formed here from q, and the increments
template <bool SD, bool WL>
__device__ __forceinline__ void lin_recon5_one(const DeviceState& d, const double* __restrict__ dqv, int s, int side,
                                               int k)
{
   const int n = d.slot[s].x;
   const size_t ns = (size_t)d.nSlot;
   const int sk = 4 * side + k;
   double df[6];
#pragma unroll
   for (int j = 0; j < 6; j++) df[j] = dsten_comp(d, dqv, n - 2 + j, k);
   Weno5Lin<double> p;
   if (WL) {
      p = weno5_lin_get(d.wlin + (size_t)(kWeno5LinVals * sk) * ns + s, ns);
   } else {
      double f[6];
#pragma unroll
      for (int j = 0; j < 6; j++) f[j] = sten_comp(d, n - 2 + j, k);
      p = side ? weno5_lin_pre<double, SD>(f[5], f[4], f[3], f[2], f[1])
               : weno5_lin_pre<double, SD>(f[0], f[1], f[2], f[3], f[4]);
   }
   const double v = side ? weno5_lin_apply<double, SD>(p, df[5], df[4], df[3], df[2], df[1])
                         : weno5_lin_apply<double, SD>(p, df[0], df[1], df[2], df[3], df[4]);
   d.qface[(size_t)sk * ns + s] = v;
}

// the face states recon5_one (or lin_recon5_one) left for slot s, swapped
// as face_states does
__device__ __forceinline__ void face_states_pre(const DeviceState& d, int s, bool swap, double (&L)[4],
                                                double (&R)[4])
{
   const size_t ns = (size_t)d.nSlot;
#pragma unroll
   for (int k = 0; k < 4; k++) {
      const double qln = d.qface[(size_t)k * ns + s], qrn1 = d.qface[(size_t)(4 + k) * ns + s];
      L[k] = swap ? qln : qrn1;
      R[k] = swap ? qrn1 : qln;
   }
}

}  // namespace hamstr
#endif
