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
#include "softdiv.cuh"

namespace hamstr {

constexpr int kFacRec = 80;
constexpr unsigned kLaneMask = 0xffffffffu;

// A factorisation followed by a solving warp of the same block (adi.cu):
// the factoring warp publishes in shared memory how many rows' records it
// has stored (publish_rows: its stores, a block-scope fence, then the
// count); the follower waits until the rows it needs are there
// (wait_rows: the count, then a block-scope fence) before it loads them
// (ldf).
// The factoring warp never waits, so every wait ends; the bound (well
// above the longest legitimate wait, a periodic line's last-row
// elimination) only guards against a broken schedule: a wait that gives up
// returns false, the follower waits no more and the caller raises an error
// word.
constexpr long kFollowSpin = 1L << 24;

__device__ __forceinline__ void publish_rows(int* prog, int n, int lane)
{
   __threadfence_block();
   __syncwarp();
   if (lane == 0) *(volatile int*)prog = n;
}

__device__ __forceinline__ bool wait_rows(const int* prog, int need)
{
   long it = 0;
   while (*(const volatile int*)prog < need)
      if (++it > kFollowSpin) return false;
   __threadfence_block();
   return true;
}

// a record load of a follower: an ordinary coherent load (never the
// read-only path, whose cache need not see stores made during the kernel)
template <bool FOLLOW>
__device__ __forceinline__ double ldf(const double* p)
{
   return FOLLOW ? __ldca(p) : *p;
}

// x <- LU^{-1} x for a 4-vector held one component per lane: component l
// lives in lane base + stride*l, r is this lane's component and lu its LU
// row (L[r][0..r-1], reciprocal pivot, U[r][r+1..3]).  Same operations and
// order as triSolvers.cpp:813-821; lanes whose component is not yet due
// compute values nobody reads.  Returns this lane's solved component and
// leaves the whole solution in xs on every lane.
__device__ __forceinline__ double lu_solve_lanes(const double (&lu)[4], int r, double x, int base, int stride,
                                                 double (&xs)[4])
{
   const double piv = sel4(lu, r);
   double d[4];
#pragma unroll
   for (int l = 0; l < 4; l++) {
      const double t = x * piv;
      d[l] = __shfl_sync(kLaneMask, t, base + stride * l);
      if (l < 3) x = x - lu[l] * d[l];
   }
   xs[3] = d[3];
   const double q3 = lu[3] * xs[3];
   const double x2l = d[2] - q3;
   xs[2] = __shfl_sync(kLaneMask, x2l, base + 2 * stride);
   const double q2 = lu[2] * xs[2];
   const double t1 = d[1] - q2;
   const double x1l = t1 - q3;
   xs[1] = __shfl_sync(kLaneMask, x1l, base + stride);
   const double q1 = lu[1] * xs[1];
   double t0 = d[0] - q1;
   t0 = t0 - q2;
   const double x0l = t0 - q3;
   xs[0] = __shfl_sync(kLaneMask, x0l, base);
   return sel4(xs, r);
}

// LU of a 4x4 block held one element per lane (element e = 4k+j in lane
// base + e), as a wavefront over the lanes: returns in each lane element e
// of the LU record (L below the diagonal, reciprocal pivots on it, U above),
// with the operations and order of triSolvers.cpp:796-811.  With SD the
// pivot reciprocals use the integer-pipe division (softdiv.cuh), equal to
// 1./x: shorter latency, off the FP64 pipe.
template <bool SD>
__device__ __forceinline__ double lu_wavefront(double w, int base, int e)
{
   const int k = e >> 2, j = e & 3;
   const double piv0 = SD ? sd::div(1., __shfl_sync(kLaneMask, w, base)) : 1. / __shfl_sync(kLaneMask, w, base);
   {
      const double m = w * piv0;
      if (k == 0 && j >= 1) w = m;
   }
   {
      const double L = __shfl_sync(kLaneMask, w, base + 4 * k), U = __shfl_sync(kLaneMask, w, base + j);
      const double t = w - L * U;
      if (k >= 1 && j >= 1) w = t;
   }
   const double piv1 = SD ? sd::div(1., __shfl_sync(kLaneMask, w, base + 5)) : 1. / __shfl_sync(kLaneMask, w, base + 5);
   {
      const double m = w * piv1;
      if (k == 1 && j >= 2) w = m;
   }
   {
      const double L = __shfl_sync(kLaneMask, w, base + 4 * k + 1), U = __shfl_sync(kLaneMask, w, base + 4 + j);
      const double t = w - L * U;
      if (k >= 2 && j >= 2) w = t;
   }
   const double piv2 = SD ? sd::div(1., __shfl_sync(kLaneMask, w, base + 10)) : 1. / __shfl_sync(kLaneMask, w, base + 10);
   {
      const double m = w * piv2;
      if (k == 2 && j == 3) w = m;
   }
   {
      const double L = __shfl_sync(kLaneMask, w, base + 14), U = __shfl_sync(kLaneMask, w, base + 11);
      const double t = w - L * U;
      if (k == 3 && j == 3) w = t;
   }
   const double piv3 = SD ? sd::div(1., __shfl_sync(kLaneMask, w, base + 15)) : 1. / __shfl_sync(kLaneMask, w, base + 15);
   if (k == j) w = (k == 0) ? piv0 : (k == 1) ? piv1 : (k == 2) ? piv2 : piv3;
   return w;
}

// lu_wavefront together with the forward substitution of right-hand sides
// through the block being factored (triSolvers.cpp:813-816 for f and
// :825-828 for the columns of c): xc is element (k,j) of c(i) (column j is
// solved by the lanes of column j) and, with F, xf is component k of f(i)
// (the same in the four lanes of row k).  Each substitution step rides on
// the elimination step that produces its pivot and multipliers, so the
// right-hand sides are substituted by the time the last pivot is known
// instead of after the factorisation.  Returns the LU element as
// lu_wavefront does; dc (column j) and df (f) receive the substituted
// values c1..c4 / d1..d4 of the reference in every lane, U the multipliers
// u12 u13 u14 u23 u24 u34 in every lane.
template <bool SD, bool F>
__device__ __forceinline__ double lu_wavefront_rhs(double w, double xc, double xf, int base, int e, double (&dc)[4],
                                                   double (&df)[4], double (&U)[6])
{
   const int k = e >> 2, j = e & 3;
   const double piv0 = SD ? sd::div(1., __shfl_sync(kLaneMask, w, base)) : 1. / __shfl_sync(kLaneMask, w, base);
   {
      const double m = w * piv0;
      if (k == 0 && j >= 1) w = m;
   }
   {
      const double tc = xc * piv0, tf = F ? xf * piv0 : 0.0;
      const double L = __shfl_sync(kLaneMask, w, base + 4 * k), Uj = __shfl_sync(kLaneMask, w, base + j);
      dc[0] = __shfl_sync(kLaneMask, tc, base + j);
      if (F) df[0] = __shfl_sync(kLaneMask, tf, base);
      const double t = w - L * Uj;
      xc = xc - L * dc[0];
      if (F) xf = xf - L * df[0];
      U[0] = __shfl_sync(kLaneMask, w, base + 1);
      U[1] = __shfl_sync(kLaneMask, w, base + 2);
      U[2] = __shfl_sync(kLaneMask, w, base + 3);
      if (k >= 1 && j >= 1) w = t;
   }
   const double piv1 = SD ? sd::div(1., __shfl_sync(kLaneMask, w, base + 5)) : 1. / __shfl_sync(kLaneMask, w, base + 5);
   {
      const double m = w * piv1;
      if (k == 1 && j >= 2) w = m;
   }
   {
      const double tc = xc * piv1, tf = F ? xf * piv1 : 0.0;
      const double L = __shfl_sync(kLaneMask, w, base + 4 * k + 1), Uj = __shfl_sync(kLaneMask, w, base + 4 + j);
      dc[1] = __shfl_sync(kLaneMask, tc, base + 4 + j);
      if (F) df[1] = __shfl_sync(kLaneMask, tf, base + 4);
      const double t = w - L * Uj;
      xc = xc - L * dc[1];
      if (F) xf = xf - L * df[1];
      U[3] = __shfl_sync(kLaneMask, w, base + 6);
      U[4] = __shfl_sync(kLaneMask, w, base + 7);
      if (k >= 2 && j >= 2) w = t;
   }
   const double piv2 = SD ? sd::div(1., __shfl_sync(kLaneMask, w, base + 10)) : 1. / __shfl_sync(kLaneMask, w, base + 10);
   {
      const double m = w * piv2;
      if (k == 2 && j == 3) w = m;
   }
   {
      const double tc = xc * piv2, tf = F ? xf * piv2 : 0.0;
      const double L = __shfl_sync(kLaneMask, w, base + 14), Uj = __shfl_sync(kLaneMask, w, base + 11);
      dc[2] = __shfl_sync(kLaneMask, tc, base + 8 + j);
      if (F) df[2] = __shfl_sync(kLaneMask, tf, base + 8);
      const double t = w - L * Uj;
      xc = xc - L * dc[2];
      if (F) xf = xf - L * df[2];
      U[5] = Uj;
      if (k == 3 && j == 3) w = t;
   }
   const double piv3 = SD ? sd::div(1., __shfl_sync(kLaneMask, w, base + 15)) : 1. / __shfl_sync(kLaneMask, w, base + 15);
   {
      const double tc = xc * piv3, tf = F ? xf * piv3 : 0.0;
      dc[3] = __shfl_sync(kLaneMask, tc, base + 12 + j);
      if (F) df[3] = __shfl_sync(kLaneMask, tf, base + 12);
   }
   if (k == j) w = (k == 0) ? piv0 : (k == 1) ? piv1 : (k == 2) ? piv2 : piv3;
   return w;
}

// back substitution inside one block (triSolvers.cpp:818-821): d holds the
// forward-substituted d1..d4 (or c1..c4), U the multipliers u12 u13 u14 u23
// u24 u34; every component, in the reference's order, in every lane
__device__ __forceinline__ void lu_back4(const double (&d)[4], const double (&U)[6], double (&x)[4])
{
   x[3] = d[3];
   x[2] = d[2] - U[5] * x[3];
   x[1] = (d[1] - U[3] * x[2]) - U[4] * x[3];
   x[0] = ((d[0] - U[0] * x[1]) - U[1] * x[2]) - U[2] * x[3];
}

// Block-Thomas factorisation of one line of N rows by one warp: blocks
// A_i = Ab + i*stride, B_i = Bb + i*stride, C_i = Cb + i*stride (row-major
// 4x4); writes the per-row records `fac` (kFacRec doubles per row) and,
// periodic, the LU of the final last-row block into facN.  Returns, in the
// lanes that hold a pivot, whether a stored reciprocal pivot is infinite or
// NaN (a zero or non-finite pivot; the reference divides by it regardless).
// With prog, the rows are published as they are stored (publish_rows),
// and N + 1 once a periodic line's last-row records are.
template <bool SD = true>
__device__ __forceinline__ bool factor_line(const double* __restrict__ Ab, const double* __restrict__ Bb,
                                            const double* __restrict__ Cb, size_t stride, int N, bool per,
                                            double* __restrict__ fac, double* __restrict__ facN, int lane,
                                            int* prog = nullptr)
{
   const int h = lane >> 4, e = lane & 15, k = e >> 2, j = e & 3;
   double A = Ab[e], B = Bb[e], C = Cb[e];
   // column j of the previous row's solved C' (h=0) or a' (h=1), whole in
   // every lane of the column (the block back substitution runs in each)
   double P[4] = {0.0, 0.0, 0.0, 0.0};
   double Yp = 0.0;   // element (k,j) of it
   bool bad = false;
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
            acc -= a * P[l];
         }
      } else if (h) {
         acc = A;
      }
      // c'(i) = B'^{-1} c(i), a'(i) = B'^{-1} a(i), one column per lane
      // group (component k of column j in lane 16h + 4k + j), substituted
      // along the LU of B'(i), which both halves compute on their own copy;
      // at i == N-2 of a periodic chain c(i) += a(i) first and a'(i) = c'(i)
      const bool last2 = per && (i == N - 2);
      double Y = h ? acc : C;
      const double fillv = __shfl_sync(kLaneMask, acc, 16 + e);
      if (last2 && h == 0) Y = C + fillv;
      double dc[4], df[4], U[6];
      const double w = lu_wavefront_rhs<SD, false>(__shfl_sync(kLaneMask, acc, e), Y, 0.0, 16 * h, e, dc, df, U);
      if (h == 0) rec[16 + e] = w;
      bad |= h == 0 && k == j && nonfinite(w);
      lu_back4(dc, U, P);
      if (last2) {
#pragma unroll
         for (int m = 0; m < 4; m++) {
            const double fromc = __shfl_sync(kLaneMask, P[m], e);
            if (h == 1) P[m] = fromc;
         }
      }
      Yp = sel4(P, k);
      rec[32 + 16 * h + e] = Yp;
      if (prog) publish_rows(prog, i + 1, lane);
      A = An;
      B = Bn;
      C = Cn;
   }
   if (!per) return bad;
   // last-row elimination (triSolvers.cpp:967-999)
   double cN = __shfl_sync(kLaneMask, Yp, e);
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
   const double w = lu_wavefront<SD>(__shfl_sync(kLaneMask, bN, 16 + e), 16 * h, e);
   if (h == 0) facN[e] = w;
   if (prog) publish_rows(prog, N + 1, lane);
   return bad || (h == 0 && k == j && nonfinite(w));
}

// Two open lines per warp, one per half (h = lane >> 4): the same
// operations as factor_line's half 0 on an open line, so each line's
// records are bit-identical to a factor_line call.  Lines of different
// length run to the longer one's count with the shorter half idle (its
// loads and stores skipped).  Short open lines -- the rule on split meshes
// -- leave half of factor_line's warp with nothing to do.
//
// Lane (k,j) keeps column j of the previous row's C' whole (the block back
// substitution runs in every lane of the column), so the next row's
// b(i) -= a(i) c'(i-1) needs no shuffle of it, and the columns of c(i) are
// substituted along the factorisation's wavefront (lu_wavefront_rhs).
// With F the line's first solve runs in the same loop: fs holds f (the
// right-hand sides, rows of 4) and receives the forward sweep's rows
// (triSolvers.cpp:786-822, the reference's own loop), and xlast the last
// row's solution, for the back substitution (back_line_pair).  With prog
// each row is published once its records are stored (publish_rows), for a
// solve that follows in another warp.
template <bool SD, bool F>
__device__ __forceinline__ bool factor_line_pair(const double* __restrict__ Ab, size_t stride, int N,
                                                 double* __restrict__ fac, int lane, double* __restrict__ fs,
                                                 double (&xlast)[4], int* prog = nullptr)
{
   const int h = lane >> 4, e = lane & 15, k = e >> 2, j = e & 3, hb = 16 * h;
   const int Nmax = max(N, __shfl_xor_sync(kLaneMask, N, 16));
   double A = 0.0, B = 0.0, C = 0.0, fv = 0.0;
   if (N > 0) {
      A = Ab[e];
      B = Ab[16 + e];
      C = Ab[32 + e];
      if (F) fv = fs[k];
   }
   double P[4] = {0.0, 0.0, 0.0, 0.0};   // column j of the previous row's C'
   double X[4] = {0.0, 0.0, 0.0, 0.0};   // F: the previous row's solution
   bool bad = false;   // a live row's reciprocal pivot is not finite
   for (int i = 0; i < Nmax; i++) {
      double An = 0.0, Bn = 0.0, Cn = 0.0, fvn = 0.0;
      if (i + 1 < N) {
         const size_t o = stride * (size_t)(i + 1);
         An = Ab[o + e];
         Bn = Ab[o + 16 + e];
         Cn = Ab[o + 32 + e];
         if (F) fvn = fs[4 * (i + 1) + k];
      }
      const bool live = i < N;
      double* rec = fac + (size_t)kFacRec * i;
      if (live) rec[e] = A;
      // b(i) -= a(i) c'(i-1) and f(i) -= a(i) f(i-1), products subtracted in order
      double acc = B, xf = fv;
      if (i > 0) {
#pragma unroll
         for (int l = 0; l < 4; l++) {
            const double a = __shfl_sync(kLaneMask, A, hb + 4 * k + l);
            acc -= a * P[l];
            if (F) xf = xf - a * X[l];
         }
      }
      double dc[4], df[4], U[6];
      const double w = lu_wavefront_rhs<SD, F>(acc, C, xf, hb, e, dc, df, U);
      if (live) rec[16 + e] = w;
      bad |= live && k == j && nonfinite(w);
      lu_back4(dc, U, P);
      if (live) rec[32 + e] = sel4(P, k);
      if (F) {
         double x[4];
         lu_back4(df, U, x);
         if (e < 4 && live) fs[4 * i + e] = sel4(x, e);
#pragma unroll
         for (int m = 0; m < 4; m++)
            if (live) X[m] = x[m];   // the shorter line keeps its last row's solution
      }
      if (prog) publish_rows(prog, i + 1, lane);
      A = An;
      B = Bn;
      C = Cn;
      fv = fvn;
   }
#pragma unroll
   for (int m = 0; m < 4; m++) xlast[m] = X[m];
   return bad;
}

template <bool SD = true>
__device__ __forceinline__ bool factor_line_pair(const double* __restrict__ Ab, size_t stride, int N,
                                                 double* __restrict__ fac, int lane, int* prog = nullptr)
{
   double unused[4];
   return factor_line_pair<SD, false>(Ab, stride, N, fac, lane, nullptr, unused, prog);
}

// back substitution f(i) -= c'(i) f(i+1), i = N-2..0, of two open lines,
// one per half-warp (triSolvers.cpp:839-846): fs holds the forward sweep's
// rows and receives the solution, xlast is row N-1's solution (every lane);
// FOLLOW: the records were stored by another warp of the block (ldf)
template <bool FOLLOW = false>
__device__ __forceinline__ void back_line_pair(const double* __restrict__ fac, int N, double* __restrict__ fs,
                                               int lane, const double (&xlast)[4])
{
   const int e = lane & 15, pj = e & 3, r = lane & 3, hb = lane & 16;
   const int Nmax = max(N, __shfl_xor_sync(kLaneMask, N, 16));
   double xnext[4];
#pragma unroll
   for (int m = 0; m < 4; m++) xnext[m] = xlast[m];
   // a row here is a few dependent operations, shorter than a load: rows
   // ii-1 and ii-2 are in flight while row ii is solved
   double mv = 0.0, xi = 0.0, mv1 = 0.0, xi1 = 0.0;
   if (N >= 2) {
      mv = ldf<FOLLOW>(&fac[(size_t)kFacRec * (N - 2) + 32 + e]);
      xi = fs[4 * (N - 2) + r];
   }
   if (N >= 3) {
      mv1 = ldf<FOLLOW>(&fac[(size_t)kFacRec * (N - 3) + 32 + e]);
      xi1 = fs[4 * (N - 3) + r];
   }
   for (int t = 0; t <= Nmax - 2; t++) {
      const int ii = N - 2 - t;
      double mv2 = 0.0, xi2 = 0.0;
      if (ii > 1) {
         mv2 = ldf<FOLLOW>(&fac[(size_t)kFacRec * (ii - 2) + 32 + e]);
         xi2 = fs[4 * (ii - 2) + r];
      }
      const double prod = mv * sel4(xnext, pj);
      double x = xi;
#pragma unroll
      for (int jj = 0; jj < 4; jj++) x = x - __shfl_sync(kLaneMask, prod, hb + 4 * r + jj);
#pragma unroll
      for (int m = 0; m < 4; m++) xnext[m] = __shfl_sync(kLaneMask, x, hb + m);
      if (e < 4 && ii >= 0) fs[4 * ii + e] = x;
      mv = mv1;
      xi = xi1;
      mv1 = mv2;
      xi1 = xi2;
   }
}

// Right-hand-side replay of two factored open lines, one per half-warp:
// the operations of solve_line's open branch on lanes 0-15, per half.
// FOLLOW: behind the factorisation of the same lines by another warp of
// the block (prog, publish_rows); ok turns false if a wait gave up.
template <bool FOLLOW = false>
__device__ __forceinline__ void solve_line_pair(const double* __restrict__ fac, int N, double* __restrict__ fs, int lane,
                                                const int* prog = nullptr, bool* ok = nullptr)
{
   const int e = lane & 15, pj = e & 3, r = lane & 3, hb = lane & 16;
   const int Nmax = max(N, __shfl_xor_sync(kLaneMask, N, 16));
   double xprev[4] = {0.0, 0.0, 0.0, 0.0};
   double fv = 0.0, av = 0.0, lu[4] = {0.0, 0.0, 0.0, 0.0};
   if (FOLLOW && *ok && Nmax > 0 && !wait_rows(prog, 1)) *ok = false;
   if (N > 0) {
      fv = fs[r];
#pragma unroll
      for (int c = 0; c < 4; c++) lu[c] = ldf<FOLLOW>(&fac[16 + 4 * r + c]);
   }
   for (int i = 0; i < Nmax; i++) {
      double fvn = 0.0, avn = 0.0, lun[4] = {0.0, 0.0, 0.0, 0.0};
      if (FOLLOW && *ok && i + 1 < Nmax && !wait_rows(prog, i + 2)) *ok = false;
      if (i + 1 < N) {
         const double* nr = fac + (size_t)kFacRec * (i + 1);
         fvn = fs[4 * (i + 1) + r];
         avn = ldf<FOLLOW>(&nr[e]);
#pragma unroll
         for (int c = 0; c < 4; c++) lun[c] = ldf<FOLLOW>(&nr[16 + 4 * r + c]);
      }
      double x = fv;
      if (i > 0) {
         const double p = av * sel4(xprev, pj);
#pragma unroll
         for (int jj = 0; jj < 4; jj++) x = x - __shfl_sync(kLaneMask, p, hb + 4 * r + jj);
      }
      double xs[4];
      x = lu_solve_lanes(lu, r, x, hb, 1, xs);
      const bool live = i < N;   // the shorter line keeps its last row's solution
      if (e < 4 && live) fs[4 * i + e] = x;
#pragma unroll
      for (int m = 0; m < 4; m++) {
         if (live) xprev[m] = xs[m];
         lu[m] = lun[m];
      }
      fv = fvn;
      av = avn;
   }
   __syncwarp();
   if (FOLLOW && *ok && !wait_rows(prog, Nmax)) *ok = false;
   back_line_pair<FOLLOW>(fac, N, fs, lane, xprev);
}

// ---- eight open lines per warp, four lanes each --------------------------
// Lane 4g + r works on row r of every block of line g: the row products run
// on all 32 lanes at once, and the block LU and the 4-vector solves run as
// in the warp form (lu_wavefront, lu_solve_lanes) on four lanes.  Same
// operations and order as factor_line / solve_line on an open line, so the
// records are the same.  Lines of a warp run to the longest one's count,
// the shorter ones idle (loads and stores skipped); N = 0 for an unused
// group.

// the LU of B' (lane r holds row r in w[0..3]), lu_wavefront's steps
template <bool SD>
__device__ __forceinline__ void lu_rows_quad(double (&w)[4], int r, int base)
{
   const double piv0 = SD ? sd::div(1., __shfl_sync(kLaneMask, w[0], base)) : 1. / __shfl_sync(kLaneMask, w[0], base);
#pragma unroll
   for (int j = 1; j < 4; j++) {
      const double m = w[j] * piv0;
      if (r == 0) w[j] = m;
   }
#pragma unroll
   for (int j = 1; j < 4; j++) {
      const double U = __shfl_sync(kLaneMask, w[j], base);
      const double t = w[j] - w[0] * U;
      if (r >= 1) w[j] = t;
   }
   const double piv1 = SD ? sd::div(1., __shfl_sync(kLaneMask, w[1], base + 1))
                          : 1. / __shfl_sync(kLaneMask, w[1], base + 1);
#pragma unroll
   for (int j = 2; j < 4; j++) {
      const double m = w[j] * piv1;
      if (r == 1) w[j] = m;
   }
#pragma unroll
   for (int j = 2; j < 4; j++) {
      const double U = __shfl_sync(kLaneMask, w[j], base + 1);
      const double t = w[j] - w[1] * U;
      if (r >= 2) w[j] = t;
   }
   const double piv2 = SD ? sd::div(1., __shfl_sync(kLaneMask, w[2], base + 2))
                          : 1. / __shfl_sync(kLaneMask, w[2], base + 2);
   {
      const double m = w[3] * piv2;
      if (r == 2) w[3] = m;
   }
   {
      const double U = __shfl_sync(kLaneMask, w[3], base + 2);
      const double t = w[3] - w[2] * U;
      if (r == 3) w[3] = t;
   }
   const double piv3 = SD ? sd::div(1., __shfl_sync(kLaneMask, w[3], base + 3))
                          : 1. / __shfl_sync(kLaneMask, w[3], base + 3);
   const double pv = (r == 0) ? piv0 : (r == 1) ? piv1 : (r == 2) ? piv2 : piv3;
#pragma unroll
   for (int j = 0; j < 4; j++)
      if (j == r) w[j] = pv;
}

__device__ __forceinline__ void ld4row(const double* __restrict__ p, double (&v)[4])
{
   const double2 a = *reinterpret_cast<const double2*>(p);
   const double2 b = *reinterpret_cast<const double2*>(p + 2);
   v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}

__device__ __forceinline__ void st4row(double* __restrict__ p, const double (&v)[4])
{
   *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
   *reinterpret_cast<double2*>(p + 2) = make_double2(v[2], v[3]);
}

// factor_line on open line g of the warp: blocks of row i at blk + i*stride
// (A, B, C consecutive, 16 each)
template <bool SD>
__device__ __forceinline__ bool factor_line_quad(const double* __restrict__ blk, size_t stride, int N,
                                                 double* __restrict__ fac, int lane)
{
   const int r = lane & 3, base = lane & ~3;
   const int Nmax = __reduce_max_sync(kLaneMask, N);
   double Pr[4] = {0.0, 0.0, 0.0, 0.0};   // row r of the previous row's C'
   bool bad = false;                      // a live row's reciprocal pivot is not finite
   for (int i = 0; i < Nmax; i++) {
      const bool live = i < N;
      double A[4] = {0.0, 0.0, 0.0, 0.0}, w[4] = {0.0, 0.0, 0.0, 0.0}, C[4] = {0.0, 0.0, 0.0, 0.0};
      double* rec = fac + (size_t)kFacRec * i;
      if (live) {
         const double* b = blk + stride * (size_t)i;
         ld4row(b + 4 * r, A);
         ld4row(b + 16 + 4 * r, w);
         ld4row(b + 32 + 4 * r, C);
         st4row(rec + 4 * r, A);
      }
      if (i > 0) {
         // b(i) -= a(i) c'(i-1): entry (r, j) subtracts a(r,l) c'(l,j), l = 0..3 in order
         double P[4][4];
#pragma unroll
         for (int l = 0; l < 4; l++)
#pragma unroll
            for (int j = 0; j < 4; j++) P[l][j] = __shfl_sync(kLaneMask, Pr[j], base + l);
#pragma unroll
         for (int j = 0; j < 4; j++) {
            double acc = w[j];
#pragma unroll
            for (int l = 0; l < 4; l++) acc -= A[l] * P[l][j];
            w[j] = acc;
         }
      }
      lu_rows_quad<SD>(w, r, base);
      if (live) st4row(rec + 16 + 4 * r, w);
      bad |= live && nonfinite(sel4(w, r));
      // c'(i) = B'^{-1} c(i), column by column (component r of each in this lane)
#pragma unroll
      for (int j = 0; j < 4; j++) {
         double xs[4];
         Pr[j] = lu_solve_lanes(w, r, C[j], base, 1, xs);
      }
      if (live) st4row(rec + 32 + 4 * r, Pr);
   }
   return bad;
}

// solve_line on open line g of the warp: the right-hand side from
// r[fcell[i]] (zero where fcell < 0), the solution into r[scell[i]]; fs
// holds the forward sweep's rows.  Row i+1's record and right-hand side
// are loaded while row i is solved.
__device__ __forceinline__ void solve_line_quad(const double* __restrict__ fac, int N, double* __restrict__ rv,
                                                const int* __restrict__ fcell, const int* __restrict__ scell,
                                                double* __restrict__ fs, int lane)
{
   const int r = lane & 3, base = lane & ~3;
   const int Nmax = __reduce_max_sync(kLaneMask, N);
   double xp[4] = {0.0, 0.0, 0.0, 0.0};
   double a[4] = {0.0, 0.0, 0.0, 0.0}, lu[4] = {0.0, 0.0, 0.0, 0.0}, xr = 0.0;
   if (N > 0) {
      const int fc = fcell[0];
      if (fc >= 0) xr = rv[4 * (size_t)fc + r];
      ld4row(fac + 16 + 4 * r, lu);
   }
   for (int i = 0; i < Nmax; i++) {
      double an[4] = {0.0, 0.0, 0.0, 0.0}, lun[4] = {0.0, 0.0, 0.0, 0.0}, xrn = 0.0;
      if (i + 1 < N) {
         const double* rn = fac + (size_t)kFacRec * (i + 1);
         const int fcn = fcell[i + 1];
         if (fcn >= 0) xrn = rv[4 * (size_t)fcn + r];
         ld4row(rn + 4 * r, an);
         ld4row(rn + 16 + 4 * r, lun);
      }
      double x = xr;
      if (i > 0) {
         // f(i) -= a(i) f(i-1), this component's products in order
#pragma unroll
         for (int j = 0; j < 4; j++) x = x - a[j] * xp[j];
      }
      double xs[4];
      x = lu_solve_lanes(lu, r, x, base, 1, xs);
      const bool live = i < N;
      if (live) fs[4 * i + r] = x;
#pragma unroll
      for (int m = 0; m < 4; m++) {
         if (live) xp[m] = xs[m];
         a[m] = an[m];
         lu[m] = lun[m];
      }
      xr = xrn;
   }
   // back substitution f(i) -= c'(i) f(i+1), i = N-2..0 (t = 0..Nmax-2, i = N-2-t)
   // (row ii-1's C' row and forward value are loaded while row ii is solved)
   if (N > 0) rv[4 * (size_t)scell[N - 1] + r] = sel4(xp, r);
   double xf = 0.0, c[4] = {0.0, 0.0, 0.0, 0.0};
   int sc = 0;
   if (N >= 2) {
      xf = fs[4 * (N - 2) + r];
      ld4row(fac + (size_t)kFacRec * (N - 2) + 32 + 4 * r, c);
      sc = scell[N - 2];
   }
   for (int t = 0; t <= Nmax - 2; t++) {
      const int ii = N - 2 - t;
      double xfn = 0.0, cn[4] = {0.0, 0.0, 0.0, 0.0};
      int scn = 0;
      if (ii > 0) {
         xfn = fs[4 * (ii - 1) + r];
         ld4row(fac + (size_t)kFacRec * (ii - 1) + 32 + 4 * r, cn);
         scn = scell[ii - 1];
      }
      double x = xf;
#pragma unroll
      for (int j = 0; j < 4; j++) x = x - c[j] * xp[j];
#pragma unroll
      for (int m = 0; m < 4; m++) {
         const double v = __shfl_sync(kLaneMask, x, base + m);
         if (ii >= 0) xp[m] = v;
      }
      if (ii >= 0) rv[4 * (size_t)sc + r] = x;
      xf = xfn;
#pragma unroll
      for (int m = 0; m < 4; m++) c[m] = cn[m];
      sc = scn;
   }
}

// ---- one open line per thread -------------------------------------------
// The same operations as factor_line / solve_line on an open line, written
// out for one thread: a warp then carries 32 lines and every FP64
// instruction does 32 lanes of useful work (the warp forms keep 16 or 4).
// Records are those of factor_line, so either form can solve what the
// other factored.  Short open lines -- most of a split mesh -- gain most.

// lu_wavefront on a block held by one thread: element e = 4k + j in w[e]
template <bool SD>
__device__ __forceinline__ void lu4_thread(double (&w)[16])
{
   const double piv0 = SD ? sd::div(1., w[0]) : 1. / w[0];
#pragma unroll
   for (int j = 1; j < 4; j++) w[j] = w[j] * piv0;
#pragma unroll
   for (int k = 1; k < 4; k++)
#pragma unroll
      for (int j = 1; j < 4; j++) w[4 * k + j] = w[4 * k + j] - w[4 * k] * w[j];
   const double piv1 = SD ? sd::div(1., w[5]) : 1. / w[5];
#pragma unroll
   for (int j = 2; j < 4; j++) w[4 + j] = w[4 + j] * piv1;
#pragma unroll
   for (int k = 2; k < 4; k++)
#pragma unroll
      for (int j = 2; j < 4; j++) w[4 * k + j] = w[4 * k + j] - w[4 * k + 1] * w[4 + j];
   const double piv2 = SD ? sd::div(1., w[10]) : 1. / w[10];
   w[11] = w[11] * piv2;
   w[15] = w[15] - w[14] * w[11];
   const double piv3 = SD ? sd::div(1., w[15]) : 1. / w[15];
   w[0] = piv0;
   w[5] = piv1;
   w[10] = piv2;
   w[15] = piv3;
}

// lu_solve_lanes for a vector held by one thread (lu: the 16-entry record)
__device__ __forceinline__ void lu_solve_thread(const double (&lu)[16], double (&x)[4])
{
   const double d0 = x[0] * lu[0];
   double x1 = x[1] - lu[4] * d0;
   double x2 = x[2] - lu[8] * d0;
   double x3 = x[3] - lu[12] * d0;
   const double d1 = x1 * lu[5];
   x2 = x2 - lu[9] * d1;
   x3 = x3 - lu[13] * d1;
   const double d2 = x2 * lu[10];
   x3 = x3 - lu[14] * d2;
   const double s3 = x3 * lu[15];
   const double s2 = d2 - lu[11] * s3;
   const double s1 = (d1 - lu[6] * s2) - lu[7] * s3;
   const double s0 = ((d0 - lu[1] * s1) - lu[2] * s2) - lu[3] * s3;
   x[0] = s0;
   x[1] = s1;
   x[2] = s2;
   x[3] = s3;
}

__device__ __forceinline__ void ld16(const double* __restrict__ p, double (&v)[16])
{
#pragma unroll
   for (int m = 0; m < 16; m += 2) {
      const double2 t = *reinterpret_cast<const double2*>(p + m);
      v[m] = t.x;
      v[m + 1] = t.y;
   }
}

__device__ __forceinline__ void st16(double* __restrict__ p, const double (&v)[16])
{
#pragma unroll
   for (int m = 0; m < 16; m += 2) *reinterpret_cast<double2*>(p + m) = make_double2(v[m], v[m + 1]);
}

// factor_line on an open line by one thread: blocks of row i at
// blk + i*stride (A, B, C consecutive, 16 each), records into fac
template <bool SD>
__device__ __forceinline__ bool factor_line_thread(const double* __restrict__ blk, size_t stride, int N,
                                                   double* __restrict__ fac)
{
   double P[16];   // previous row's C'
   bool bad = false;   // a reciprocal pivot is not finite
   for (int i = 0; i < N; i++) {
      const double* b = blk + stride * (size_t)i;
      double* rec = fac + (size_t)kFacRec * i;
      double A[16], w[16], C[16];
      ld16(b, A);
      ld16(b + 16, w);
      ld16(b + 32, C);
      st16(rec, A);
      if (i > 0) {
         // b(i) -= a(i) c'(i-1), each entry's four products subtracted in order
#pragma unroll
         for (int k = 0; k < 4; k++)
#pragma unroll
            for (int j = 0; j < 4; j++) {
               double acc = w[4 * k + j];
#pragma unroll
               for (int l = 0; l < 4; l++) acc -= A[4 * k + l] * P[4 * l + j];
               w[4 * k + j] = acc;
            }
      }
      lu4_thread<SD>(w);
      st16(rec + 16, w);
      bad |= nonfinite(w[0]) || nonfinite(w[5]) || nonfinite(w[10]) || nonfinite(w[15]);
      // c'(i) = B'^{-1} c(i), column by column
#pragma unroll
      for (int j = 0; j < 4; j++) {
         double x[4] = {C[j], C[4 + j], C[8 + j], C[12 + j]};
         lu_solve_thread(w, x);
#pragma unroll
         for (int k = 0; k < 4; k++) P[4 * k + j] = x[k];
      }
      st16(rec + 32, P);
   }
   return bad;
}

// solve_line on an open line by one thread, the right-hand side read from
// r[fcell[i]] (zero where fcell < 0) and the solution written to
// r[scell[i]]; fs holds the forward sweep's rows.  The next row's record
// and right-hand side are loaded while this row is solved.
__device__ __forceinline__ void solve_line_thread(const double* __restrict__ fac, int N, double* __restrict__ r,
                                                  const int* __restrict__ fcell, const int* __restrict__ scell,
                                                  double* __restrict__ fs)
{
   double xp[4] = {0.0, 0.0, 0.0, 0.0};
   double a[16], lu[16], xr[4] = {0.0, 0.0, 0.0, 0.0};
   {
      const int fc = fcell[0];
      if (fc >= 0) {
         const double2 u = *reinterpret_cast<const double2*>(r + 4 * (size_t)fc);
         const double2 v = *reinterpret_cast<const double2*>(r + 4 * (size_t)fc + 2);
         xr[0] = u.x; xr[1] = u.y; xr[2] = v.x; xr[3] = v.y;
      }
      ld16(fac + 16, lu);
#pragma unroll
      for (int m = 0; m < 16; m++) a[m] = 0.0;
   }
   for (int i = 0; i < N; i++) {
      double an[16], lun[16], xrn[4] = {0.0, 0.0, 0.0, 0.0};
      if (i + 1 < N) {
         const double* rn = fac + (size_t)kFacRec * (i + 1);
         const int fcn = fcell[i + 1];
         if (fcn >= 0) {
            const double2 u = *reinterpret_cast<const double2*>(r + 4 * (size_t)fcn);
            const double2 v = *reinterpret_cast<const double2*>(r + 4 * (size_t)fcn + 2);
            xrn[0] = u.x; xrn[1] = u.y; xrn[2] = v.x; xrn[3] = v.y;
         }
         ld16(rn, an);
         ld16(rn + 16, lun);
      }
      double x[4] = {xr[0], xr[1], xr[2], xr[3]};
      if (i > 0) {
         // f(i) -= a(i) f(i-1), each component's products subtracted in order
#pragma unroll
         for (int k = 0; k < 4; k++)
#pragma unroll
            for (int j = 0; j < 4; j++) x[k] = x[k] - a[4 * k + j] * xp[j];
      }
      lu_solve_thread(lu, x);
      *reinterpret_cast<double2*>(fs + 4 * i) = make_double2(x[0], x[1]);
      *reinterpret_cast<double2*>(fs + 4 * i + 2) = make_double2(x[2], x[3]);
#pragma unroll
      for (int k = 0; k < 4; k++) { xp[k] = x[k]; xr[k] = xrn[k]; }
#pragma unroll
      for (int m = 0; m < 16; m++) { a[m] = an[m]; lu[m] = lun[m]; }
   }
   // back substitution f(i) -= c'(i) f(i+1), i = N-2..0
   {
      double* o = r + 4 * (size_t)scell[N - 1];
      *reinterpret_cast<double2*>(o) = make_double2(xp[0], xp[1]);
      *reinterpret_cast<double2*>(o + 2) = make_double2(xp[2], xp[3]);
   }
   // row i-1's C' and forward value are loaded while row i is solved
   double c[16], xf[4];
   int sc = 0;
   if (N >= 2) {
      ld16(fac + (size_t)kFacRec * (N - 2) + 32, c);
      ld4row(fs + 4 * (N - 2), xf);
      sc = scell[N - 2];
   }
   for (int i = N - 2; i >= 0; i--) {
      double cn[16], xfn[4];
      int scn = 0;
      if (i > 0) {
         ld16(fac + (size_t)kFacRec * (i - 1) + 32, cn);
         ld4row(fs + 4 * (i - 1), xfn);
         scn = scell[i - 1];
      } else {
#pragma unroll
         for (int m = 0; m < 16; m++) cn[m] = 0.0;
#pragma unroll
         for (int m = 0; m < 4; m++) xfn[m] = 0.0;
      }
      double x[4] = {xf[0], xf[1], xf[2], xf[3]};
#pragma unroll
      for (int k = 0; k < 4; k++)
#pragma unroll
         for (int j = 0; j < 4; j++) x[k] = x[k] - c[4 * k + j] * xp[j];
      double* o = r + 4 * (size_t)sc;
      *reinterpret_cast<double2*>(o) = make_double2(x[0], x[1]);
      *reinterpret_cast<double2*>(o + 2) = make_double2(x[2], x[3]);
#pragma unroll
      for (int k = 0; k < 4; k++) { xp[k] = x[k]; xf[k] = xfn[k]; }
#pragma unroll
      for (int m = 0; m < 16; m++) c[m] = cn[m];
      sc = scn;
   }
}

__device__ __forceinline__ void ld4(const double* __restrict__ p, double (&v)[4])
{
   const double2 a = *reinterpret_cast<const double2*>(p);
   const double2 b = *reinterpret_cast<const double2*>(p + 2);
   v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}

// Right-hand-side replay of a factored line: fs (N rows of 4, in place)
// <- solution, with the records of factor_line.  All 32 lanes take part.
//
// Lane r = lane & 3 owns component r of the vector being solved; the 16
// products of a 4x4 matrix-vector step are formed in one instruction by
// lanes e = 4*pr + pj (e = lane & 15) and handed to their owner lanes with
// shuffles, so each row costs about 35 FP64 instructions instead of 60.
// The subtraction order of every component is the reference's.
// FOLLOW: behind the factorisation of the same line by another warp of the
// block (prog, publish_rows); ok turns false if a wait gave up.
template <bool FOLLOW = false>
__device__ __forceinline__ void solve_line(const double* __restrict__ fac, const double* __restrict__ facN, int N,
                                           bool per, double* __restrict__ fs, int lane, const int* prog = nullptr,
                                           bool* ok = nullptr)
{
   const int e = lane & 15, pr = e >> 2, pj = e & 3, hi = lane >> 4;
   const int r = lane & 3;
   // ---- forward sweep (triSolvers.cpp:778-822 / 859-933); row i+1 prefetched
   double xprev[4] = {0.0, 0.0, 0.0, 0.0};
   if (FOLLOW && *ok && !wait_rows(prog, 1)) *ok = false;
   double fv = fs[r], av = 0.0, lu[4];
#pragma unroll
   for (int c = 0; c < 4; c++) lu[c] = ldf<FOLLOW>(&fac[16 + 4 * r + c]);
   for (int i = 0; i < N; i++) {
      double fvn = 0.0, avn = 0.0, lun[4] = {0.0, 0.0, 0.0, 0.0};
      if (i + 1 < N) {
         if (FOLLOW && *ok && !wait_rows(prog, i + 2)) *ok = false;
         const double* nr = fac + (size_t)kFacRec * (i + 1);
         fvn = fs[4 * (i + 1) + r];
         avn = ldf<FOLLOW>(&nr[e]);
#pragma unroll
         for (int c = 0; c < 4; c++) lun[c] = ldf<FOLLOW>(&nr[16 + 4 * r + c]);
      }
      double x = fv;
      if (i > 0) {
         // f(i) -= a(i) f(i-1), the 16 products in one instruction
         const double p = av * sel4(xprev, pj);
#pragma unroll
         for (int jj = 0; jj < 4; jj++) x = x - __shfl_sync(kLaneMask, p, 4 * r + jj);
      }
      double xs[4];
      x = lu_solve_lanes(lu, r, x, 0, 1, xs);
      if (lane < 4) fs[4 * i + lane] = x;
#pragma unroll
      for (int m = 0; m < 4; m++) { xprev[m] = xs[m]; lu[m] = lun[m]; }
      fv = fvn;
      av = avn;
   }
   __syncwarp();
   if (FOLLOW && *ok && !wait_rows(prog, per ? N + 1 : N)) *ok = false;
   if (per) {
      // f(N-1) -= c_{N-1}^{(i)} f(i), i = 0..N-2 (triSolvers.cpp:991-999);
      // the products of rows i and i+1 in one instruction (lanes 0-15, 16-31)
      double fN = sel4(xprev, r);
      int i = 0;
      double c = 0.0, f = 0.0;
      if (hi < N - 1) {
         c = ldf<FOLLOW>(&fac[(size_t)kFacRec * hi + 64 + e]);
         f = fs[4 * hi + pj];
      }
      for (; i < N - 1; i += 2) {
         const int rn = i + 2 + hi;
         double cn = 0.0, fn = 0.0;
         if (rn < N - 1) {
            cn = ldf<FOLLOW>(&fac[(size_t)kFacRec * rn + 64 + e]);
            fn = fs[4 * rn + pj];
         }
         const double p = c * f;
#pragma unroll
         for (int jj = 0; jj < 4; jj++) fN = fN - __shfl_sync(kLaneMask, p, 4 * r + jj);
         if (i + 1 < N - 1) {
#pragma unroll
            for (int jj = 0; jj < 4; jj++) fN = fN - __shfl_sync(kLaneMask, p, 16 + 4 * r + jj);
         }
         c = cn;
         f = fn;
      }
      double luN[4], xn[4];
#pragma unroll
      for (int cc = 0; cc < 4; cc++) luN[cc] = ldf<FOLLOW>(&facN[4 * r + cc]);
      fN = lu_solve_lanes(luN, r, fN, 0, 1, xn);
      __syncwarp();
      if (lane < 4) fs[4 * (N - 1) + lane] = fN;
      // back substitution (triSolvers.cpp:1032-1045):
      // f(i) -= (c'(i) f(i+1) + a'(i) f(N-1)), c' products in lanes 0-15 and
      // a' products in lanes 16-31 of one instruction
      double fNall[4];
#pragma unroll
      for (int m = 0; m < 4; m++) fNall[m] = xn[m];
      double xnext[4];
#pragma unroll
      for (int m = 0; m < 4; m++) xnext[m] = xn[m];
      // rows ii-1 and ii-2 are in flight while row ii is solved
      double mv = 0.0, xi = 0.0, mv1 = 0.0, xi1 = 0.0;
      if (N >= 2) {
         mv = ldf<FOLLOW>(&fac[(size_t)kFacRec * (N - 2) + 32 + 16 * hi + e]);
         xi = fs[4 * (N - 2) + r];
      }
      if (N >= 3) {
         mv1 = ldf<FOLLOW>(&fac[(size_t)kFacRec * (N - 3) + 32 + 16 * hi + e]);
         xi1 = fs[4 * (N - 3) + r];
      }
      for (int ii = N - 2; ii >= 0; ii--) {
         double mv2 = 0.0, xi2 = 0.0;
         if (ii > 1) {
            mv2 = ldf<FOLLOW>(&fac[(size_t)kFacRec * (ii - 2) + 32 + 16 * hi + e]);
            xi2 = fs[4 * (ii - 2) + r];
         }
         const double prod = mv * (hi ? sel4(fNall, pj) : sel4(xnext, pj));
         const double other = __shfl_sync(kLaneMask, prod, e + 16);
         const double sterm = (ii == N - 2) ? prod : prod + other;
         double x = xi;
#pragma unroll
         for (int jj = 0; jj < 4; jj++) x = x - __shfl_sync(kLaneMask, sterm, 4 * r + jj);
#pragma unroll
         for (int m = 0; m < 4; m++) xnext[m] = __shfl_sync(kLaneMask, x, m);
         if (lane < 4) fs[4 * ii + lane] = x;
         mv = mv1;
         xi = xi1;
         mv1 = mv2;
         xi1 = xi2;
      }
   } else {
      // back substitution (triSolvers.cpp:839-846): f(i) -= c'(i) f(i+1)
      double xnext[4];
#pragma unroll
      for (int m = 0; m < 4; m++) xnext[m] = xprev[m];
      // rows ii-1 and ii-2 are in flight while row ii is solved
      double mv = 0.0, xi = 0.0, mv1 = 0.0, xi1 = 0.0;
      if (N >= 2) {
         mv = ldf<FOLLOW>(&fac[(size_t)kFacRec * (N - 2) + 32 + e]);
         xi = fs[4 * (N - 2) + r];
      }
      if (N >= 3) {
         mv1 = ldf<FOLLOW>(&fac[(size_t)kFacRec * (N - 3) + 32 + e]);
         xi1 = fs[4 * (N - 3) + r];
      }
      for (int ii = N - 2; ii >= 0; ii--) {
         double mv2 = 0.0, xi2 = 0.0;
         if (ii > 1) {
            mv2 = ldf<FOLLOW>(&fac[(size_t)kFacRec * (ii - 2) + 32 + e]);
            xi2 = fs[4 * (ii - 2) + r];
         }
         const double prod = mv * sel4(xnext, pj);
         double x = xi;
#pragma unroll
         for (int jj = 0; jj < 4; jj++) x = x - __shfl_sync(kLaneMask, prod, 4 * r + jj);
#pragma unroll
         for (int m = 0; m < 4; m++) xnext[m] = __shfl_sync(kLaneMask, x, m);
         if (lane < 4) fs[4 * ii + lane] = x;
         mv = mv1;
         xi = xi1;
         mv1 = mv2;
         xi1 = xi2;
      }
   }
}

}  // namespace hamstr
#endif
