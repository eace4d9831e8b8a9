// ##################################################################
//
// line_solve.cuh -- one 4x4 block-tridiagonal line per warp
//
// blockTridag4 (triSolvers.cpp:769-847) and blockTridagPeriodic4
// (triSolvers.cpp:850-1046) split into the part that depends only on the
// blocks (factor_line) and the right-hand-side replay (solve_line).  The
// replay uses exactly the values the reference computes, in its order, so
// factor_line + solve_line is bit-identical to one reference call.
//
// GB300 runs an FP64 instruction for a whole warp in ~64 cycles whatever
// the number of active lanes, so independent work is packed into lanes:
// lane = 16*h + 4*k + j holds element (k,j) of a 4x4 block; in periodic
// lines half h=0 carries the C' recurrence and half h=1 the fill-in column
// a' (triSolvers.cpp:877-891), which follow the same instruction sequence.
//
// Per-row record (kFacRec = 80 doubles):
//   [ 0..15] A_i             (f update in the forward sweep)
//   [16..31] LU of B'_i      b11 u12 u13 u14 b21 b22 u23 u24 b31 b32 b33 u34 b41 b42 b43 b44
//   [32..47] C'_i            (back substitution)
//   [48..63] a'_i            (periodic fill-in column, back substitution)
//   [64..79] c_{N-1} at elimination step i (periodic, triSolvers.cpp:967-999)
// plus, periodic, facN[16] = LU of the final last-row block.
// ##################################################################
#ifndef HAMSTR_GPU_LINE_SOLVE_CUH
#define HAMSTR_GPU_LINE_SOLVE_CUH

#include "lu4.cuh"

namespace hamstr {

constexpr int kFacRec = 80;
constexpr unsigned kLaneMask = 0xffffffffu;

// Block-Thomas factorisation of one line of N rows by one warp: blocks
// A_i = Ab + i*stride, B_i = Bb + i*stride, C_i = Cb + i*stride (row-major
// 4x4); writes the per-row records `fac` (kFacRec doubles per row) and,
// periodic, the LU of the final last-row block into facN.
__device__ __forceinline__ void factor_line(const double* __restrict__ Ab, const double* __restrict__ Bb,
                                            const double* __restrict__ Cb, size_t stride, int N, bool per,
                                            double* __restrict__ fac, double* __restrict__ facN, int lane)
{
   const int h = lane >> 4, e = lane & 15, k = e >> 2, j = e & 3;
   double A = Ab[e], B = Bb[e], C = Cb[e];
   double P = 0.0;   // previous row's solved C' (h=0) or a' (h=1), element (k,j)
   for (int i = 0; i < N; i++) {
      // next row's blocks are loaded while this row is factored
      double An = 0.0, Bn = 0.0, Cn = 0.0;
      if (i + 1 < N) {
         const size_t o = stride * (size_t)(i + 1);
         An = Ab[o + e];
         Bn = Bb[o + e];
         Cn = Cb[o + e];
      }
      double* rec = fac + (size_t)kFacRec * i;
      if (h == 0) rec[e] = A;
      // b(i) -= a(i) c'(i-1) and, periodic, a(i) = -a(i) a'(i-1)
      double acc = h ? 0.0 : B;
      if (i > 0) {
#pragma unroll
         for (int l = 0; l < 4; l++) {
            const double a = __shfl_sync(kLaneMask, A, 16 * h + 4 * k + l);
            const double x = __shfl_sync(kLaneMask, P, 16 * h + 4 * l + j);
            acc -= a * x;
         }
      } else if (h) {
         acc = A;
      }
      double b[16];
#pragma unroll
      for (int m = 0; m < 16; m++) b[m] = __shfl_sync(kLaneMask, acc, m);
      const LU4 u = lu_factor(b);
      if (h == 0) rec[16 + e] = lu_get(u, e);
      // c'(i) = B'^{-1} c(i), a'(i) = B'^{-1} a(i); at i == N-2 of a
      // periodic chain c(i) += a(i) first and a'(i) = c'(i)
      const bool last2 = per && (i == N - 2);
      double Y = h ? acc : C;
      const double fillv = __shfl_sync(kLaneMask, acc, 16 + e);
      if (last2 && h == 0) Y = C + fillv;
      double y[4];
#pragma unroll
      for (int r = 0; r < 4; r++) y[r] = __shfl_sync(kLaneMask, Y, 16 * h + 4 * r + j);
      lu_solve(u, y[0], y[1], y[2], y[3]);
      double Yp = sel4(y, k);
      const double fromc = __shfl_sync(kLaneMask, Yp, e);
      if (last2 && h == 1) Yp = fromc;
      rec[32 + 16 * h + e] = Yp;
      P = Yp;
      A = An;
      B = Bn;
      C = Cn;
   }
   if (!per) return;
   // last-row elimination (triSolvers.cpp:967-999)
   double cN = __shfl_sync(kLaneMask, P, e);
   double bN = (k == j) ? 1.0 : 0.0;
   double Y = (N > 1) ? fac[32 + 16 * h + e] : 0.0;
   for (int i = 0; i < N - 1; i++) {
      double* rec = fac + (size_t)kFacRec * i;
      const double Yn = (i + 2 < N) ? rec[kFacRec + 32 + 16 * h + e] : 0.0;
      if (h == 0) rec[64 + e] = cN;
      double acc = h ? bN : 0.0;
#pragma unroll
      for (int l = 0; l < 4; l++) {
         const double c = __shfl_sync(kLaneMask, cN, 16 * h + 4 * k + l);
         const double y = __shfl_sync(kLaneMask, Y, 16 * h + 4 * l + j);
         acc -= c * y;
      }
      if (h) bN = acc;
      cN = __shfl_sync(kLaneMask, acc, e);
      Y = Yn;
   }
   double b[16];
#pragma unroll
   for (int m = 0; m < 16; m++) b[m] = __shfl_sync(kLaneMask, bN, 16 + m);
   const LU4 u = lu_factor(b);
   if (h == 0) facN[e] = lu_get(u, e);
}

// x_k -= sum_j M[k][j] * v[j] for the lane's component k = lane & 3, then
// all four components gathered into every lane
__device__ __forceinline__ void matvec_sub(const double (&Mrow)[4], const double (&v)[4], double (&x)[4], int kk)
{
   double t = sel4(x, kk);
#pragma unroll
   for (int jj = 0; jj < 4; jj++) t -= Mrow[jj] * v[jj];
#pragma unroll
   for (int m = 0; m < 4; m++) x[m] = __shfl_sync(kLaneMask, t, m);
}

__device__ __forceinline__ void ld4(const double* __restrict__ p, double (&v)[4])
{
   const double2 a = *reinterpret_cast<const double2*>(p);
   const double2 b = *reinterpret_cast<const double2*>(p + 2);
   v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}

__device__ __forceinline__ void ld16(const double* __restrict__ p, double (&v)[16])
{
#pragma unroll
   for (int m = 0; m < 16; m += 2) {
      const double2 a = *reinterpret_cast<const double2*>(p + m);
      v[m] = a.x;
      v[m + 1] = a.y;
   }
}

__device__ __forceinline__ LU4 lu_from(const double (&v)[16])
{
   LU4 u;
   u.b11 = v[0];  u.u12 = v[1];  u.u13 = v[2];  u.u14 = v[3];
   u.b21 = v[4];  u.b22 = v[5];  u.u23 = v[6];  u.u24 = v[7];
   u.b31 = v[8];  u.b32 = v[9];  u.b33 = v[10]; u.u34 = v[11];
   u.b41 = v[12]; u.b42 = v[13]; u.b43 = v[14]; u.b44 = v[15];
   return u;
}

// Right-hand-side replay of a factored line: fs (N rows of 4, in place)
// <- solution, with the records of factor_line.  All 32 lanes take part.
__device__ __forceinline__ void solve_line(const double* __restrict__ fac, const double* __restrict__ facN, int N,
                                           bool per, double* __restrict__ fs, int lane)
{
   const int kk = lane & 3;
   // forward sweep (triSolvers.cpp:778-822 / 859-933); row i+1 prefetched
   double xp[4] = {0.0, 0.0, 0.0, 0.0};
   double x[4], arow[4] = {0.0, 0.0, 0.0, 0.0}, lu[16];
   ld4(fs, x);
   ld16(fac + 16, lu);
   for (int i = 0; i < N; i++) {
      double xn[4] = {0.0, 0.0, 0.0, 0.0}, an[4] = {0.0, 0.0, 0.0, 0.0}, lun[16];
      if (i + 1 < N) {
         const double* nr = fac + (size_t)kFacRec * (i + 1);
         ld4(fs + 4 * (i + 1), xn);
         ld4(nr + 4 * kk, an);
         ld16(nr + 16, lun);
      } else {
#pragma unroll
         for (int m = 0; m < 16; m++) lun[m] = 0.0;
      }
      if (i > 0) matvec_sub(arow, xp, x, kk);
      const LU4 u = lu_from(lu);
      lu_solve(u, x[0], x[1], x[2], x[3]);
      if (lane < 4) fs[4 * i + lane] = sel4(x, lane);
#pragma unroll
      for (int m = 0; m < 4; m++) { xp[m] = x[m]; x[m] = xn[m]; arow[m] = an[m]; }
#pragma unroll
      for (int m = 0; m < 16; m++) lu[m] = lun[m];
   }
   __syncwarp();
   double xn[4];
   if (per) {
      // f(N-1) -= c_{N-1} f(i), then the last-row solve (triSolvers.cpp:991-1029)
      double fN[4];
#pragma unroll
      for (int m = 0; m < 4; m++) fN[m] = xp[m];
      double fi[4], crow[4];
      ld4(fs, fi);
      ld4(fac + 64 + 4 * kk, crow);
      for (int i = 0; i < N - 1; i++) {
         double fin[4] = {0.0, 0.0, 0.0, 0.0}, cn[4] = {0.0, 0.0, 0.0, 0.0};
         if (i + 2 < N) {
            ld4(fs + 4 * (i + 1), fin);
            ld4(fac + (size_t)kFacRec * (i + 1) + 64 + 4 * kk, cn);
         }
         matvec_sub(crow, fi, fN, kk);
#pragma unroll
         for (int m = 0; m < 4; m++) { fi[m] = fin[m]; crow[m] = cn[m]; }
      }
      const LU4 u = lu_load(facN);
      lu_solve(u, fN[0], fN[1], fN[2], fN[3]);
      __syncwarp();
      if (lane < 4) fs[4 * (N - 1) + lane] = sel4(fN, lane);
      // back substitution (triSolvers.cpp:1032-1045)
#pragma unroll
      for (int m = 0; m < 4; m++) xn[m] = fN[m];
      double xi[4], cr[4], ar[4];
      if (N >= 2) {
         ld4(fs + 4 * (N - 2), xi);
         ld4(fac + (size_t)kFacRec * (N - 2) + 32 + 4 * kk, cr);
         ld4(fac + (size_t)kFacRec * (N - 2) + 48 + 4 * kk, ar);
      }
      for (int i = N - 2; i >= 0; i--) {
         double xin[4] = {0.0, 0.0, 0.0, 0.0}, crn[4] = {0.0, 0.0, 0.0, 0.0}, arn[4] = {0.0, 0.0, 0.0, 0.0};
         if (i > 0) {
            ld4(fs + 4 * (i - 1), xin);
            ld4(fac + (size_t)kFacRec * (i - 1) + 32 + 4 * kk, crn);
            ld4(fac + (size_t)kFacRec * (i - 1) + 48 + 4 * kk, arn);
         }
         double t = sel4(xi, kk);
         if (i == N - 2) {
#pragma unroll
            for (int jj = 0; jj < 4; jj++) t -= (cr[jj] * xn[jj]);
         } else {
#pragma unroll
            for (int jj = 0; jj < 4; jj++) t -= (cr[jj] * xn[jj] + ar[jj] * fN[jj]);
         }
#pragma unroll
         for (int m = 0; m < 4; m++) xn[m] = __shfl_sync(kLaneMask, t, m);
         if (lane < 4) fs[4 * i + lane] = sel4(xn, lane);
#pragma unroll
         for (int m = 0; m < 4; m++) { xi[m] = xin[m]; cr[m] = crn[m]; ar[m] = arn[m]; }
      }
   } else {
      // back substitution (triSolvers.cpp:839-846)
#pragma unroll
      for (int m = 0; m < 4; m++) xn[m] = xp[m];
      double xi[4], cr[4];
      if (N >= 2) {
         ld4(fs + 4 * (N - 2), xi);
         ld4(fac + (size_t)kFacRec * (N - 2) + 32 + 4 * kk, cr);
      }
      for (int i = N - 2; i >= 0; i--) {
         double xin[4] = {0.0, 0.0, 0.0, 0.0}, crn[4] = {0.0, 0.0, 0.0, 0.0};
         if (i > 0) {
            ld4(fs + 4 * (i - 1), xin);
            ld4(fac + (size_t)kFacRec * (i - 1) + 32 + 4 * kk, crn);
         }
         matvec_sub(cr, xn, xi, kk);
         if (lane < 4) fs[4 * i + lane] = sel4(xi, lane);
#pragma unroll
         for (int m = 0; m < 4; m++) { xn[m] = xi[m]; xi[m] = xin[m]; cr[m] = crn[m]; }
      }
   }
}

}  // namespace hamstr
#endif
