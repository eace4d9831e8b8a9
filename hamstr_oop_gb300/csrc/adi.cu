// ##################################################################
//
// adi.cu -- ADI line solves (ADI.cpp:55-252, triSolvers.cpp:769-1046)
//
// The block matrices A, B, C of a chain depend only on the face
// Jacobians and sigma, which do not change between the msweep sweeps of
// one pseudo-time step, so the block-Thomas factorisation (everything in
// blockTridag4 / blockTridagPeriodic4 that does not touch f) is done once
// per step for all chains at once (adi_factor), and each sweep replays
// only the right-hand-side part with the stored factors (adi_solve).  The
// stored values are the very values the reference recomputes each sweep,
// so the results are bit-identical.
//
// One warp per chain.  GB300 executes an FP64 instruction for a whole
// warp in ~64 cycles whatever the number of active lanes, so independent
// work is packed into lanes: lane = 16*h + 4*k + j holds element (k,j) of
// a 4x4 block; in periodic chains half h=0 carries the C' recurrence and
// half h=1 the fill-in column a' (triSolvers.cpp:877-891), which follow
// the same instruction sequence.
//
// Per-row factor record (80 doubles):
//   [ 0..15] A_i scaled      (f update in the forward sweep)
//   [16..31] LU of B'_i      b11 u12 u13 u14 b21 b22 u23 u24 b31 b32 b33 u34 b41 b42 b43 b44
//   [32..47] C'_i            (back substitution)
//   [48..63] a'_i            (periodic fill-in column, back substitution)
//   [64..79] c_{N-1} at elimination step i (periodic, triSolvers.cpp:967-999)
// Periodic chains also keep the LU of the final last-row block (facN).
// ##################################################################
#include "device_state.h"
#include "plan.h"

namespace hamstr {

namespace {

constexpr int kFac = 80;
constexpr unsigned kFull = 0xffffffffu;

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

__device__ __forceinline__ double sel4(const double (&x)[4], int k)
{
   double v = x[0];
   v = (k == 1) ? x[1] : v;
   v = (k == 2) ? x[2] : v;
   v = (k == 3) ? x[3] : v;
   return v;
}

// one block entry (row-major element e) in the reference's term order
// (ADI.cpp:103-188): 0.0, then += / -= the listed face-matrix entries
__device__ __forceinline__ double assemble(const DeviceState& d, const int* __restrict__ ops, int e)
{
   double acc = 0.0;
#pragma unroll
   for (int o = 0; o < kOpsPerBlock; o++) {
      const int op = ops[o];
      if (op < 0) break;
      const int slot = op >> 3, sel = (op >> 1) & 3;
      const double* m = d.ff + 32 * (size_t)slot;
      double v;
      const int col = e & 3;
      if (sel == OP_SEL_RREFL && (col == 1 || col == 2)) {
         // rmat with reflected momentum columns (ADI.cpp:151-163)
         const double4 rf = d.refl[d.slot_face[slot]];
         const double r01 = m[16 + (e & ~3) + 1], r02 = m[16 + (e & ~3) + 2];
         v = (col == 1) ? (rf.x * r01 + rf.y * r02) : (rf.z * r01 + rf.w * r02);
      } else {
         v = m[(sel == OP_SEL_L ? 0 : 16) + e];
      }
      if (op & 1) acc -= v;
      else acc += v;
   }
   return acc;
}

__global__ void __launch_bounds__(32) adi_factor_kernel(DeviceState d)
{
   if (halted(d)) return;
   const int ich = blockIdx.x;
   const int lane = threadIdx.x, h = lane >> 4, e = lane & 15, k = e >> 2, j = e & 3;
   const int N = d.chain_nrows[ich], row0 = d.chain_row0[ich];
   const bool per = d.chain_periodic[ich] != 0;
   double P = 0.0;   // previous row's solved C' (h=0) or a' (h=1), element (k,j)
   for (int i = 0; i < N; i++) {
      const int row = row0 + i;
      const int* ops = d.row_ops + 3 * kOpsPerBlock * row;
      const double dt = d.dtfac[d.row_scell[row]];
      double A = assemble(d, ops, e);
      double B = assemble(d, ops + kOpsPerBlock, e);
      double C = assemble(d, ops + 2 * kOpsPerBlock, e);
      A *= dt;
      B *= dt;
      C *= dt;
      if (k == j) B += 1.0;
      double* rec = d.fac + (size_t)kFac * row;
      if (h == 0) rec[e] = A;
      // b(i) -= a(i) c'(i-1) and, periodic, a(i) = -a(i) a'(i-1)
      double acc = h ? 0.0 : B;
      if (i > 0) {
#pragma unroll
         for (int l = 0; l < 4; l++) {
            const double a = __shfl_sync(kFull, A, 16 * h + 4 * k + l);
            const double x = __shfl_sync(kFull, P, 16 * h + 4 * l + j);
            acc -= a * x;
         }
      } else if (h) {
         acc = A;
      }
      double b[16];
#pragma unroll
      for (int m = 0; m < 16; m++) b[m] = __shfl_sync(kFull, acc, m);
      const LU4 u = lu_factor(b);
      if (h == 0) rec[16 + e] = lu_get(u, e);
      // c'(i) = B'^{-1} c(i), a'(i) = B'^{-1} a(i); at i == N-2 of a
      // periodic chain c(i) += a(i) first and a'(i) = c'(i)
      const bool last2 = per && (i == N - 2);
      double Y = h ? acc : C;
      const double fillv = __shfl_sync(kFull, acc, 16 + e);
      if (last2 && h == 0) Y = C + fillv;
      double y[4];
#pragma unroll
      for (int r = 0; r < 4; r++) y[r] = __shfl_sync(kFull, Y, 16 * h + 4 * r + j);
      lu_solve(u, y[0], y[1], y[2], y[3]);
      double Yp = sel4(y, k);
      const double fromc = __shfl_sync(kFull, Yp, e);
      if (last2 && h == 1) Yp = fromc;
      rec[32 + 16 * h + e] = Yp;
      P = Yp;
   }
   if (!per) return;
   // last-row elimination (triSolvers.cpp:967-999)
   double cN = __shfl_sync(kFull, P, e);
   double bN = (k == j) ? 1.0 : 0.0;
   for (int i = 0; i < N - 1; i++) {
      double* rec = d.fac + (size_t)kFac * (row0 + i);
      if (h == 0) rec[64 + e] = cN;
      const double Y = rec[32 + 16 * h + e];
      double acc = h ? bN : 0.0;
#pragma unroll
      for (int l = 0; l < 4; l++) {
         const double c = __shfl_sync(kFull, cN, 16 * h + 4 * k + l);
         const double y = __shfl_sync(kFull, Y, 16 * h + 4 * l + j);
         acc -= c * y;
      }
      if (h) bN = acc;
      cN = __shfl_sync(kFull, acc, e);
   }
   double b[16];
#pragma unroll
   for (int m = 0; m < 16; m++) b[m] = __shfl_sync(kFull, bN, 16 + m);
   const LU4 u = lu_factor(b);
   if (h == 0) d.facN[16 * d.chain_facN[ich] + e] = lu_get(u, e);
}

// x_k -= sum_j M[k][j] * v[j] for the lane's component k = lane & 3, then
// all four components gathered into every lane
__device__ __forceinline__ void matvec_sub(const double* __restrict__ M, const double (&v)[4], double (&x)[4], int kk)
{
   double t = sel4(x, kk);
#pragma unroll
   for (int jj = 0; jj < 4; jj++) t -= M[4 * kk + jj] * v[jj];
#pragma unroll
   for (int m = 0; m < 4; m++) x[m] = __shfl_sync(kFull, t, m);
}

__device__ __forceinline__ void ld4(const double* __restrict__ p, double (&v)[4])
{
   const double2 a = *reinterpret_cast<const double2*>(p);
   const double2 b = *reinterpret_cast<const double2*>(p + 2);
   v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}

__global__ void __launch_bounds__(32) adi_solve_kernel(DeviceState d, int wave_begin)
{
   if (halted(d)) return;
   const int ich = d.wave_chains[wave_begin + blockIdx.x];
   const int lane = threadIdx.x, kk = lane & 3;
   const int N = d.chain_nrows[ich], row0 = d.chain_row0[ich];
   const bool per = d.chain_periodic[ich] != 0;
   double* fs = d.fsc + 4 * (size_t)row0;
   // right-hand side F = r[fcell] (ADI.cpp:116,187)
   for (int r = lane; r < N; r += 32) {
      const int fc = d.row_fcell[row0 + r];
      double v[4] = {0.0, 0.0, 0.0, 0.0};
      if (fc >= 0) ld4(d.r + 4 * (size_t)fc, v);
      *reinterpret_cast<double2*>(fs + 4 * r) = make_double2(v[0], v[1]);
      *reinterpret_cast<double2*>(fs + 4 * r + 2) = make_double2(v[2], v[3]);
   }
   __syncwarp();
   // forward sweep (triSolvers.cpp:778-822 / 859-933)
   double xp[4] = {0.0, 0.0, 0.0, 0.0};
   for (int i = 0; i < N; i++) {
      const double* rec = d.fac + (size_t)kFac * (row0 + i);
      double x[4];
      ld4(fs + 4 * i, x);
      if (i > 0) matvec_sub(rec, xp, x, kk);
      const LU4 u = lu_load(rec + 16);
      lu_solve(u, x[0], x[1], x[2], x[3]);
      if (lane < 4) fs[4 * i + lane] = sel4(x, lane);
#pragma unroll
      for (int m = 0; m < 4; m++) xp[m] = x[m];
   }
   __syncwarp();
   if (per) {
      // f(N-1) -= c_{N-1} f(i), then the last-row solve (triSolvers.cpp:991-1029)
      double fN[4];
#pragma unroll
      for (int m = 0; m < 4; m++) fN[m] = xp[m];
      for (int i = 0; i < N - 1; i++) {
         const double* rec = d.fac + (size_t)kFac * (row0 + i);
         double fi[4];
         ld4(fs + 4 * i, fi);
         matvec_sub(rec + 64, fi, fN, kk);
      }
      const LU4 u = lu_load(d.facN + 16 * d.chain_facN[ich]);
      lu_solve(u, fN[0], fN[1], fN[2], fN[3]);
      __syncwarp();
      if (lane < 4) fs[4 * (N - 1) + lane] = sel4(fN, lane);
      // back substitution (triSolvers.cpp:1032-1045)
      double xn[4];
#pragma unroll
      for (int m = 0; m < 4; m++) xn[m] = fN[m];
      for (int i = N - 2; i >= 0; i--) {
         const double* rec = d.fac + (size_t)kFac * (row0 + i);
         double x[4];
         ld4(fs + 4 * i, x);
         double t = sel4(x, kk);
         if (i == N - 2) {
#pragma unroll
            for (int jj = 0; jj < 4; jj++) t -= (rec[32 + 4 * kk + jj] * xn[jj]);
         } else {
#pragma unroll
            for (int jj = 0; jj < 4; jj++) t -= (rec[32 + 4 * kk + jj] * xn[jj] + rec[48 + 4 * kk + jj] * fN[jj]);
         }
#pragma unroll
         for (int m = 0; m < 4; m++) x[m] = __shfl_sync(kFull, t, m);
         if (lane < 4) fs[4 * i + lane] = sel4(x, lane);
#pragma unroll
         for (int m = 0; m < 4; m++) xn[m] = x[m];
      }
   } else {
      // back substitution (triSolvers.cpp:839-846)
      double xn[4];
#pragma unroll
      for (int m = 0; m < 4; m++) xn[m] = xp[m];
      for (int i = N - 2; i >= 0; i--) {
         const double* rec = d.fac + (size_t)kFac * (row0 + i);
         double x[4];
         ld4(fs + 4 * i, x);
         matvec_sub(rec + 32, xn, x, kk);
         if (lane < 4) fs[4 * i + lane] = sel4(x, lane);
#pragma unroll
         for (int m = 0; m < 4; m++) xn[m] = x[m];
      }
   }
   __syncwarp();
   // scatter back (ADI.cpp:232-244)
   for (int r = lane; r < N; r += 32) {
      const int sc = d.row_scell[row0 + r];
      double v[4];
      ld4(fs + 4 * r, v);
      *reinterpret_cast<double2*>(d.r + 4 * (size_t)sc) = make_double2(v[0], v[1]);
      *reinterpret_cast<double2*>(d.r + 4 * (size_t)sc + 2) = make_double2(v[2], v[3]);
   }
}

}  // namespace

void launch_adi_factor(const DeviceState& d, cudaStream_t st)
{
   adi_factor_kernel<<<d.nChain, 32, 0, st>>>(d);
}

void launch_adi_solve(const DeviceState& d, int wave_begin, int wave_count, cudaStream_t st)
{
   if (wave_count > 0) adi_solve_kernel<<<wave_count, 32, 0, st>>>(d, wave_begin);
}

}  // namespace hamstr
