// ##################################################################
//
// lu4.cuh -- 4x4 block LU used by the block-tridiagonal line solvers
//
// The unpivoted LU with reciprocal pivots and the matching forward/back
// substitution of triSolvers.cpp:796-821 (blockTridag4) and :900-929
// (blockTridagPeriodic4), in the reference's operation order (callers are
// compiled with -fmad=false).
// ##################################################################
#ifndef HAMSTR_GPU_LU4_CUH
#define HAMSTR_GPU_LU4_CUH

namespace hamstr {

struct LU4 {
   double b11, u12, u13, u14, b21, b22, u23, u24, b31, b32, b33, u34, b41, b42, b43, b44;
};

// unpivoted LU with reciprocal pivots (triSolvers.cpp:796-811)
__device__ __forceinline__ LU4 lu_factor(const double (&b)[16])
{
   LU4 u;
   u.b11 = 1. / b[0];
   u.u12 = b[1] * u.b11;
   u.u13 = b[2] * u.b11;
   u.u14 = b[3] * u.b11;
   u.b21 = b[4];
   u.b22 = 1. / (b[5] - u.b21 * u.u12);
   u.u23 = (b[6] - u.b21 * u.u13) * u.b22;
   u.u24 = (b[7] - u.b21 * u.u14) * u.b22;
   u.b31 = b[8];
   u.b32 = b[9] - u.b31 * u.u12;
   u.b33 = 1. / (b[10] - u.b31 * u.u13 - u.b32 * u.u23);
   u.u34 = (b[11] - u.b31 * u.u14 - u.b32 * u.u24) * u.b33;
   u.b41 = b[12];
   u.b42 = b[13] - u.b41 * u.u12;
   u.b43 = b[14] - u.b41 * u.u13 - u.b42 * u.u23;
   u.b44 = 1. / (b[15] - u.b41 * u.u14 - u.b42 * u.u24 - u.b43 * u.u34);
   return u;
}

// x <- LU^{-1} x (triSolvers.cpp:813-821)
__device__ __forceinline__ void lu_solve(const LU4& u, double& x0, double& x1, double& x2, double& x3)
{
   const double d1 = x0 * u.b11;
   const double d2 = (x1 - u.b21 * d1) * u.b22;
   const double d3 = (x2 - u.b31 * d1 - u.b32 * d2) * u.b33;
   const double d4 = (x3 - u.b41 * d1 - u.b42 * d2 - u.b43 * d3) * u.b44;
   x3 = d4;
   x2 = d3 - u.u34 * x3;
   x1 = d2 - u.u23 * x2 - u.u24 * x3;
   x0 = d1 - u.u12 * x1 - u.u13 * x2 - u.u14 * x3;
}

__device__ __forceinline__ double lu_get(const LU4& u, int e)
{
   double v = u.b11;
   v = (e == 1) ? u.u12 : v;  v = (e == 2) ? u.u13 : v;  v = (e == 3) ? u.u14 : v;
   v = (e == 4) ? u.b21 : v;  v = (e == 5) ? u.b22 : v;  v = (e == 6) ? u.u23 : v;
   v = (e == 7) ? u.u24 : v;  v = (e == 8) ? u.b31 : v;  v = (e == 9) ? u.b32 : v;
   v = (e == 10) ? u.b33 : v; v = (e == 11) ? u.u34 : v; v = (e == 12) ? u.b41 : v;
   v = (e == 13) ? u.b42 : v; v = (e == 14) ? u.b43 : v; v = (e == 15) ? u.b44 : v;
   return v;
}

__device__ __forceinline__ LU4 lu_load(const double* __restrict__ p)
{
   LU4 u;
   u.b11 = p[0];  u.u12 = p[1];  u.u13 = p[2];  u.u14 = p[3];
   u.b21 = p[4];  u.b22 = p[5];  u.u23 = p[6];  u.u24 = p[7];
   u.b31 = p[8];  u.b32 = p[9];  u.b33 = p[10]; u.u34 = p[11];
   u.b41 = p[12]; u.b42 = p[13]; u.b43 = p[14]; u.b44 = p[15];
   return u;
}

// true for an infinite or NaN value: the exponent field all ones, tested on
// the integer pipes (no FP64 instruction)
__device__ __forceinline__ bool nonfinite(double x) { return (__double2hiint(x) & 0x7ff00000) == 0x7ff00000; }
__device__ __forceinline__ bool nonfinite(float x) { return (__float_as_int(x) & 0x7f800000) == 0x7f800000; }

__device__ __forceinline__ double sel4(const double (&x)[4], int k)
{
   double v = x[0];
   v = (k == 1) ? x[1] : v;
   v = (k == 2) ? x[2] : v;
   v = (k == 3) ? x[3] : v;
   return v;
}

}  // namespace hamstr
#endif
