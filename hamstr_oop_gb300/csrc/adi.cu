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

// blocks A, B, C of every row, scaled by CFL/sigma with B += I
// (ADI.cpp:197-217); one thread per entry, all rows at once
__global__ void __launch_bounds__(256) adi_assemble_kernel(DeviceState d)
{
   const int t = blockIdx.x * blockDim.x + threadIdx.x;
   if (t >= 48 * d.nRow || halted(d)) return;
   const int row = t / 48, e48 = t - 48 * row, b = e48 >> 4, e = e48 & 15;
   double v = assemble(d, d.row_ops + 3 * kOpsPerBlock * row + kOpsPerBlock * b, e);
   v *= d.dtfac[d.row_scell[row]];
   if (b == 1 && (e >> 2) == (e & 3)) v += 1.0;
   d.blk[t] = v;
}

// block-Thomas factorisation of one chain by one warp (see file header)
__device__ __forceinline__ void factor_chain(const DeviceState& d, int ich, int lane)
{
   const int h = lane >> 4, e = lane & 15, k = e >> 2, j = e & 3;
   const int N = d.chain_nrows[ich], row0 = d.chain_row0[ich];
   const bool per = d.chain_periodic[ich] != 0;
   const double* blk = d.blk + 48 * (size_t)row0;
   double A = blk[e], B = blk[16 + e], C = blk[32 + e];
   double P = 0.0;   // previous row's solved C' (h=0) or a' (h=1), element (k,j)
   for (int i = 0; i < N; i++) {
      // next row's blocks are loaded while this row is factored
      double An = 0.0, Bn = 0.0, Cn = 0.0;
      if (i + 1 < N) {
         const double* nb = blk + 48 * (size_t)(i + 1);
         An = nb[e];
         Bn = nb[16 + e];
         Cn = nb[32 + e];
      }
      double* rec = d.fac + (size_t)kFac * (row0 + i);
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
      A = An;
      B = Bn;
      C = Cn;
   }
   if (!per) return;
   // last-row elimination (triSolvers.cpp:967-999)
   double cN = __shfl_sync(kFull, P, e);
   double bN = (k == j) ? 1.0 : 0.0;
   double Y = (N > 1) ? d.fac[(size_t)kFac * row0 + 32 + 16 * h + e] : 0.0;
   for (int i = 0; i < N - 1; i++) {
      double* rec = d.fac + (size_t)kFac * (row0 + i);
      const double Yn = (i + 2 < N) ? rec[kFac + 32 + 16 * h + e] : 0.0;
      if (h == 0) rec[64 + e] = cN;
      double acc = h ? bN : 0.0;
#pragma unroll
      for (int l = 0; l < 4; l++) {
         const double c = __shfl_sync(kFull, cN, 16 * h + 4 * k + l);
         const double y = __shfl_sync(kFull, Y, 16 * h + 4 * l + j);
         acc -= c * y;
      }
      if (h) bN = acc;
      cN = __shfl_sync(kFull, acc, e);
      Y = Yn;
   }
   double b[16];
#pragma unroll
   for (int m = 0; m < 16; m++) b[m] = __shfl_sync(kFull, bN, 16 + m);
   const LU4 u = lu_factor(b);
   if (h == 0) d.facN[16 * d.chain_facN[ich] + e] = lu_get(u, e);
}

// persistent warps, one per SM sub-partition, each with a job list
__global__ void __launch_bounds__(128, 1) adi_factor_kernel(DeviceState d, int nwarps)
{
   if (halted(d)) return;
   const int w = blockIdx.x * 4 + (threadIdx.x >> 5);
   if (w >= nwarps) return;
   const int g = d.sched_warp0[0] + w;
   for (int job = d.sched_warp_ptr[g]; job < d.sched_warp_ptr[g + 1]; job++)
      factor_chain(d, d.sched_jobs[job], threadIdx.x & 31);
}

// x_k -= sum_j M[k][j] * v[j] for the lane's component k = lane & 3, then
// all four components gathered into every lane
__device__ __forceinline__ void matvec_sub(const double (&Mrow)[4], const double (&v)[4], double (&x)[4], int kk)
{
   double t = sel4(x, kk);
#pragma unroll
   for (int jj = 0; jj < 4; jj++) t -= Mrow[jj] * v[jj];
#pragma unroll
   for (int m = 0; m < 4; m++) x[m] = __shfl_sync(kFull, t, m);
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

// right-hand-side replay of one chain's solve with its stored factors
__device__ __forceinline__ void solve_chain(const DeviceState& d, int ich, int lane)
{
   const int kk = lane & 3;
   const int N = d.chain_nrows[ich], row0 = d.chain_row0[ich];
   const bool per = d.chain_periodic[ich] != 0;
   double* fs = d.fsc + 4 * (size_t)row0;
   const double* fac = d.fac + (size_t)kFac * row0;
   // right-hand side F = r[fcell] (ADI.cpp:116,187)
   for (int r = lane; r < N; r += 32) {
      const int fc = d.row_fcell[row0 + r];
      double v[4] = {0.0, 0.0, 0.0, 0.0};
      if (fc >= 0) ld4(d.r + 4 * (size_t)fc, v);
      *reinterpret_cast<double2*>(fs + 4 * r) = make_double2(v[0], v[1]);
      *reinterpret_cast<double2*>(fs + 4 * r + 2) = make_double2(v[2], v[3]);
   }
   __syncwarp();
   // forward sweep (triSolvers.cpp:778-822 / 859-933); row i+1 prefetched
   double xp[4] = {0.0, 0.0, 0.0, 0.0};
   double x[4], arow[4] = {0.0, 0.0, 0.0, 0.0}, lu[16];
   ld4(fs, x);
   ld16(fac + 16, lu);
   for (int i = 0; i < N; i++) {
      double xn[4] = {0.0, 0.0, 0.0, 0.0}, an[4] = {0.0, 0.0, 0.0, 0.0}, lun[16];
      if (i + 1 < N) {
         const double* nr = fac + (size_t)kFac * (i + 1);
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
            ld4(fac + (size_t)kFac * (i + 1) + 64 + 4 * kk, cn);
         }
         matvec_sub(crow, fi, fN, kk);
#pragma unroll
         for (int m = 0; m < 4; m++) { fi[m] = fin[m]; crow[m] = cn[m]; }
      }
      const LU4 u = lu_load(d.facN + 16 * d.chain_facN[ich]);
      lu_solve(u, fN[0], fN[1], fN[2], fN[3]);
      __syncwarp();
      if (lane < 4) fs[4 * (N - 1) + lane] = sel4(fN, lane);
      // back substitution (triSolvers.cpp:1032-1045)
#pragma unroll
      for (int m = 0; m < 4; m++) xn[m] = fN[m];
      double xi[4], cr[4], ar[4];
      if (N >= 2) {
         ld4(fs + 4 * (N - 2), xi);
         ld4(fac + (size_t)kFac * (N - 2) + 32 + 4 * kk, cr);
         ld4(fac + (size_t)kFac * (N - 2) + 48 + 4 * kk, ar);
      }
      for (int i = N - 2; i >= 0; i--) {
         double xin[4] = {0.0, 0.0, 0.0, 0.0}, crn[4] = {0.0, 0.0, 0.0, 0.0}, arn[4] = {0.0, 0.0, 0.0, 0.0};
         if (i > 0) {
            ld4(fs + 4 * (i - 1), xin);
            ld4(fac + (size_t)kFac * (i - 1) + 32 + 4 * kk, crn);
            ld4(fac + (size_t)kFac * (i - 1) + 48 + 4 * kk, arn);
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
         for (int m = 0; m < 4; m++) xn[m] = __shfl_sync(kFull, t, m);
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
         ld4(fac + (size_t)kFac * (N - 2) + 32 + 4 * kk, cr);
      }
      for (int i = N - 2; i >= 0; i--) {
         double xin[4] = {0.0, 0.0, 0.0, 0.0}, crn[4] = {0.0, 0.0, 0.0, 0.0};
         if (i > 0) {
            ld4(fs + 4 * (i - 1), xin);
            ld4(fac + (size_t)kFac * (i - 1) + 32 + 4 * kk, crn);
         }
         matvec_sub(cr, xn, xi, kk);
         if (lane < 4) fs[4 * i + lane] = sel4(xi, lane);
#pragma unroll
         for (int m = 0; m < 4; m++) { xn[m] = xi[m]; xi[m] = xin[m]; cr[m] = crn[m]; }
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

__global__ void __launch_bounds__(128, 1) adi_solve_kernel(DeviceState d, int wave, int nwarps)
{
   if (halted(d)) return;
   const int w = blockIdx.x * 4 + (threadIdx.x >> 5);
   if (w >= nwarps) return;
   const int g = d.sched_warp0[1 + wave] + w;
   for (int job = d.sched_warp_ptr[g]; job < d.sched_warp_ptr[g + 1]; job++)
      solve_chain(d, d.sched_jobs[job], threadIdx.x & 31);
}

}  // namespace

// One block of 4 warps per SM: the dynamic shared-memory request below
// exceeds half an SM's shared memory, so no two blocks share an SM and
// each warp owns an SM sub-partition's FP64 unit.
constexpr int kExclusiveSmem = 120 * 1024;

int adi_configure(int max_dynamic_smem)
{
   const int want = max_dynamic_smem >= kExclusiveSmem ? kExclusiveSmem : 0;
   if (want) {
      if (cudaFuncSetAttribute(adi_factor_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, want) != cudaSuccess)
         return 0;
      if (cudaFuncSetAttribute(adi_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, want) != cudaSuccess)
         return 0;
   }
   return want;
}

void launch_adi_assemble(const DeviceState& d, cudaStream_t st)
{
   const int n = 48 * d.nRow;
   adi_assemble_kernel<<<(n + 255) / 256, 256, 0, st>>>(d);
}

void launch_adi_factor(const DeviceState& d, int nwarps, cudaStream_t st)
{
   adi_factor_kernel<<<(nwarps + 3) / 4, 128, d.exclusive_smem, st>>>(d, nwarps);
}

void launch_adi_solve(const DeviceState& d, int wave, int nwarps, cudaStream_t st)
{
   if (nwarps > 0) adi_solve_kernel<<<(nwarps + 3) / 4, 128, d.exclusive_smem, st>>>(d, wave, nwarps);
}

}  // namespace hamstr
