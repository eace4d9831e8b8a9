// ##################################################################
//
// mixed.cu -- mixed-precision defect correction
//
// The residual that defines the steady state (reconstruction, Roe flux and
// the per-cell sums of computeRHS) stays in FP64 and is bit-identical to the
// reference.  The approximate operator of the implicit step -- the Roe
// Jacobians, the ADI block assembly and block-tridiagonal line solves, and
// the linearised residual of the sweeps (ADI.cpp, computeLinearRHS.cpp) --
// runs in FP32.  Near convergence the FP32 operator only changes how fast
// the FP64 residual falls, not where it goes to zero.
//
// GB300 issues FP32 about 70x faster than FP64 (64-cycle dependent FP64
// latency against 4 for FP32), so the line solves here are one thread per
// chain running the reference's block Thomas elimination in registers,
// with chains of similar length sharing a warp.
// ##################################################################
#include "device_state.h"
#include "plan.h"
#include "recon.cuh"
#include "roe.cuh"

namespace hamstr {

namespace {

constexpr int kThreads = 256;

// ---------------- residual + FP32 Jacobian ----------------
template <int ORDER>
__global__ void __launch_bounds__(kThreads) mx_rhs_face_kernel(DeviceState d)
{
   const int s = blockIdx.x * blockDim.x + threadIdx.x;
   if (s >= d.nSlot || halted(d)) return;
   const int4 sl = d.slot[s];
   const double2 nv = d.normal[s];
   double L[4], R[4];
   face_states<ORDER>(d, sl.x, (sl.w & 1) != 0, L, R);
   RoeOut o;
   if (!roe_face<false>(nv.x, nv.y, L, R, d.fc.gamma, o, nullptr, nullptr)) atomicOr(d.status, DEV_ERR_NAN_SPEC);
   st4(d.flux + 4 * (size_t)s, o.flux);
   d.spec[s] = o.spec;
   const float Lf[4] = {float(L[0]), float(L[1]), float(L[2]), float(L[3])};
   const float Rf[4] = {float(R[0]), float(R[1]), float(R[2]), float(R[3])};
   float lm[16], rm[16];
   roe_jacobian_only<float>(float(nv.x), float(nv.y), Lf, Rf, float(d.fc.gamma), lm, rm);
   float* out = d.ff32 + 32 * (size_t)s;
#pragma unroll
   for (int i = 0; i < 16; i += 4) *reinterpret_cast<float4*>(out + i) = make_float4(lm[i], lm[i + 1], lm[i + 2], lm[i + 3]);
#pragma unroll
   for (int i = 0; i < 16; i += 4)
      *reinterpret_cast<float4*>(out + 16 + i) = make_float4(rm[i], rm[i + 1], rm[i + 2], rm[i + 3]);
}

// r (already scaled by CFL/sigma in FP64) -> FP32 r, r0; dq = 0
__global__ void __launch_bounds__(kThreads) mx_init_kernel(DeviceState d)
{
   const int c = blockIdx.x * blockDim.x + threadIdx.x;
   if (c >= d.nCell || halted(d)) return;
   double r[4];
   ld4(d.r + 4 * (size_t)c, r);
   const float rf[4] = {float(r[0]), float(r[1]), float(r[2]), float(r[3])};
   const float z[4] = {0.f, 0.f, 0.f, 0.f};
   st4(d.r32 + 4 * (size_t)c, rf);
   st4(d.r032 + 4 * (size_t)c, rf);
   st4(d.dq32 + 4 * (size_t)c, z);
}

// FP32 blocks in the reference's term order (ADI.cpp:62-217)
__global__ void __launch_bounds__(kThreads) mx_assemble_kernel(DeviceState d)
{
   const int t = blockIdx.x * blockDim.x + threadIdx.x;
   if (t >= 48 * d.nRow || halted(d)) return;
   const int row = t / 48, e48 = t - 48 * row, b = e48 >> 4, e = e48 & 15;
   const int* ops = d.row_ops + 3 * kOpsPerBlock * row + kOpsPerBlock * b;
   float acc = 0.f;
#pragma unroll
   for (int o = 0; o < kOpsPerBlock; o++) {
      const int op = ops[o];
      if (op < 0) break;
      const int slot = op >> 3, sel = (op >> 1) & 3, col = e & 3;
      const float* m = d.ff32 + 32 * (size_t)slot;
      float v;
      if (sel == OP_SEL_RREFL && (col == 1 || col == 2)) {
         const double4 rf = d.refl[d.slot_face[slot]];
         const float r01 = m[16 + (e & ~3) + 1], r02 = m[16 + (e & ~3) + 2];
         v = (col == 1) ? (float(rf.x) * r01 + float(rf.y) * r02) : (float(rf.z) * r01 + float(rf.w) * r02);
      } else {
         v = m[(sel == OP_SEL_L ? 0 : 16) + e];
      }
      if (op & 1) acc -= v;
      else acc += v;
   }
   acc *= float(d.dtfac[d.row_scell[row]]);
   if (b == 1 && (e >> 2) == (e & 3)) acc += 1.f;
   d.blk32[t] = acc;
}

// ---------------- scalar block-tridiagonal solvers in T ----------------
template <typename T>
struct LUs {
   T b11, u12, u13, u14, b21, b22, u23, u24, b31, b32, b33, u34, b41, b42, b43, b44;
};

template <typename T>
__device__ __forceinline__ LUs<T> lus_factor(const T (&b)[16])
{
   LUs<T> u;
   u.b11 = T(1) / b[0];
   u.u12 = b[1] * u.b11; u.u13 = b[2] * u.b11; u.u14 = b[3] * u.b11;
   u.b21 = b[4];
   u.b22 = T(1) / (b[5] - u.b21 * u.u12);
   u.u23 = (b[6] - u.b21 * u.u13) * u.b22;
   u.u24 = (b[7] - u.b21 * u.u14) * u.b22;
   u.b31 = b[8];
   u.b32 = b[9] - u.b31 * u.u12;
   u.b33 = T(1) / (b[10] - u.b31 * u.u13 - u.b32 * u.u23);
   u.u34 = (b[11] - u.b31 * u.u14 - u.b32 * u.u24) * u.b33;
   u.b41 = b[12];
   u.b42 = b[13] - u.b41 * u.u12;
   u.b43 = b[14] - u.b41 * u.u13 - u.b42 * u.u23;
   u.b44 = T(1) / (b[15] - u.b41 * u.u14 - u.b42 * u.u24 - u.b43 * u.u34);
   return u;
}

template <typename T>
__device__ __forceinline__ void lus_solve(const LUs<T>& u, T& x0, T& x1, T& x2, T& x3)
{
   const T d1 = x0 * u.b11;
   const T d2 = (x1 - u.b21 * d1) * u.b22;
   const T d3 = (x2 - u.b31 * d1 - u.b32 * d2) * u.b33;
   const T d4 = (x3 - u.b41 * d1 - u.b42 * d2 - u.b43 * d3) * u.b44;
   x3 = d4;
   x2 = d3 - u.u34 * x3;
   x1 = d2 - u.u23 * x2 - u.u24 * x3;
   x0 = d1 - u.u12 * x1 - u.u13 * x2 - u.u14 * x3;
}

template <typename T>
__device__ __forceinline__ void lus_cols(const LUs<T>& u, T (&m)[16])
{
#pragma unroll
   for (int j = 0; j < 4; j++) lus_solve(u, m[j], m[4 + j], m[8 + j], m[12 + j]);
}

template <typename T>
__device__ __forceinline__ void ld16(const T* p, T (&v)[16])
{
#pragma unroll
   for (int m = 0; m < 16; m++) v[m] = p[m];
}

template <typename T>
__device__ __forceinline__ void st16(T* p, const T (&v)[16])
{
#pragma unroll
   for (int m = 0; m < 16; m++) p[m] = v[m];
}

// blockTridag4 (triSolvers.cpp:769-847), rows of 48 (A, B, C) in place
template <typename T>
__device__ void tridag_open(T* __restrict__ blk, T* __restrict__ f, int N)
{
   T cp[16], fp[4];
   for (int i = 0; i < N; i++) {
      T* row = blk + 48 * (size_t)i;
      T a[16], b[16], c[16], x[4];
      ld16(row, a);
      ld16(row + 16, b);
      ld16(row + 32, c);
#pragma unroll
      for (int k = 0; k < 4; k++) x[k] = f[4 * i + k];
      if (i != 0) {
#pragma unroll
         for (int k = 0; k < 4; k++)
#pragma unroll
            for (int j = 0; j < 4; j++)
#pragma unroll
               for (int l = 0; l < 4; l++) b[4 * k + j] -= a[4 * k + l] * cp[4 * l + j];
#pragma unroll
         for (int k = 0; k < 4; k++)
#pragma unroll
            for (int j = 0; j < 4; j++) x[k] -= a[4 * k + j] * fp[j];
      }
      const LUs<T> u = lus_factor(b);
      lus_solve(u, x[0], x[1], x[2], x[3]);
      if (i != N - 1) lus_cols(u, c);
      st16(row + 32, c);
#pragma unroll
      for (int k = 0; k < 4; k++) { f[4 * i + k] = x[k]; fp[k] = x[k]; }
#pragma unroll
      for (int m = 0; m < 16; m++) cp[m] = c[m];
   }
   T xn[4];
#pragma unroll
   for (int k = 0; k < 4; k++) xn[k] = f[4 * (N - 1) + k];
   for (int i = N - 2; i >= 0; i--) {
      T c[16], x[4];
      ld16(blk + 48 * (size_t)i + 32, c);
#pragma unroll
      for (int k = 0; k < 4; k++) x[k] = f[4 * i + k];
#pragma unroll
      for (int k = 0; k < 4; k++)
#pragma unroll
         for (int j = 0; j < 4; j++) x[k] -= c[4 * k + j] * xn[j];
#pragma unroll
      for (int k = 0; k < 4; k++) { f[4 * i + k] = x[k]; xn[k] = x[k]; }
   }
}

// blockTridagPeriodic4 (triSolvers.cpp:850-1046), rows of 48 in place;
// a(i) is overwritten by the fill-in column as in the reference
template <typename T>
__device__ void tridag_periodic(T* __restrict__ blk, T* __restrict__ f, int N)
{
   T cp[16], ap[16], fp[4];
   for (int i = 0; i < N; i++) {
      T* row = blk + 48 * (size_t)i;
      T a[16], b[16], c[16], x[4];
      ld16(row, a);
      ld16(row + 16, b);
      ld16(row + 32, c);
#pragma unroll
      for (int k = 0; k < 4; k++) x[k] = f[4 * i + k];
      if (i != 0) {
#pragma unroll
         for (int k = 0; k < 4; k++)
#pragma unroll
            for (int j = 0; j < 4; j++)
#pragma unroll
               for (int l = 0; l < 4; l++) b[4 * k + j] -= a[4 * k + l] * cp[4 * l + j];
#pragma unroll
         for (int k = 0; k < 4; k++)
#pragma unroll
            for (int j = 0; j < 4; j++) x[k] -= a[4 * k + j] * fp[j];
         T t[16];
#pragma unroll
         for (int k = 0; k < 4; k++)
#pragma unroll
            for (int j = 0; j < 4; j++) {
               T acc = T(0);
#pragma unroll
               for (int l = 0; l < 4; l++) acc -= a[4 * k + l] * ap[4 * l + j];
               t[4 * k + j] = acc;
            }
#pragma unroll
         for (int m = 0; m < 16; m++) a[m] = t[m];
      }
      const LUs<T> u = lus_factor(b);
      lus_solve(u, x[0], x[1], x[2], x[3]);
      if (i != N - 2) {
         lus_cols(u, c);
         lus_cols(u, a);
      } else {
#pragma unroll
         for (int m = 0; m < 16; m++) c[m] += a[m];
         lus_cols(u, c);
#pragma unroll
         for (int m = 0; m < 16; m++) a[m] = c[m];
      }
      st16(row, a);
      st16(row + 32, c);
#pragma unroll
      for (int k = 0; k < 4; k++) { f[4 * i + k] = x[k]; fp[k] = x[k]; }
#pragma unroll
      for (int m = 0; m < 16; m++) { cp[m] = c[m]; ap[m] = a[m]; }
   }
   // last-row elimination and solve (triSolvers.cpp:967-1029)
   T bN[16], cN[16], fN[4];
#pragma unroll
   for (int m = 0; m < 16; m++) bN[m] = ((m >> 2) == (m & 3)) ? T(1) : T(0);
   ld16(blk + 48 * (size_t)(N - 1) + 32, cN);
#pragma unroll
   for (int k = 0; k < 4; k++) fN[k] = f[4 * (N - 1) + k];
   for (int i = 0; i < N - 1; i++) {
      T ci[16], ai[16], t[16];
      ld16(blk + 48 * (size_t)i + 32, ci);
      ld16(blk + 48 * (size_t)i, ai);
#pragma unroll
      for (int k = 0; k < 4; k++)
#pragma unroll
         for (int j = 0; j < 4; j++) {
            T acc = T(0);
#pragma unroll
            for (int l = 0; l < 4; l++) {
               acc -= cN[4 * k + l] * ci[4 * l + j];
               bN[4 * k + j] -= cN[4 * k + l] * ai[4 * l + j];
            }
            t[4 * k + j] = acc;
         }
#pragma unroll
      for (int k = 0; k < 4; k++)
#pragma unroll
         for (int j = 0; j < 4; j++) fN[k] -= cN[4 * k + j] * f[4 * i + j];
#pragma unroll
      for (int m = 0; m < 16; m++) cN[m] = t[m];
   }
   const LUs<T> u = lus_factor(bN);
   lus_solve(u, fN[0], fN[1], fN[2], fN[3]);
#pragma unroll
   for (int k = 0; k < 4; k++) f[4 * (N - 1) + k] = fN[k];
   if (N < 2) return;
   {
      T c[16], x[4];
      ld16(blk + 48 * (size_t)(N - 2) + 32, c);
#pragma unroll
      for (int k = 0; k < 4; k++) x[k] = f[4 * (N - 2) + k];
#pragma unroll
      for (int k = 0; k < 4; k++)
#pragma unroll
         for (int j = 0; j < 4; j++) x[k] -= (c[4 * k + j] * fN[j]);
#pragma unroll
      for (int k = 0; k < 4; k++) f[4 * (N - 2) + k] = x[k];
   }
   T xn[4];
#pragma unroll
   for (int k = 0; k < 4; k++) xn[k] = f[4 * (N - 2) + k];
   for (int i = N - 3; i >= 0; i--) {
      T c[16], a[16], x[4];
      ld16(blk + 48 * (size_t)i + 32, c);
      ld16(blk + 48 * (size_t)i, a);
#pragma unroll
      for (int k = 0; k < 4; k++) x[k] = f[4 * i + k];
#pragma unroll
      for (int k = 0; k < 4; k++)
#pragma unroll
         for (int j = 0; j < 4; j++) x[k] -= (c[4 * k + j] * xn[j] + a[4 * k + j] * fN[j]);
#pragma unroll
      for (int k = 0; k < 4; k++) { f[4 * i + k] = x[k]; xn[k] = x[k]; }
   }
}

// one FP32 line solve per thread: F = r[fcell], solve, r[scell] = F
__global__ void __launch_bounds__(64) mx_lines_kernel(DeviceState d, int first, int count)
{
   const int t = blockIdx.x * blockDim.x + threadIdx.x;
   if (t >= count || halted(d)) return;
   const int ich = d.line_chains[first + t];
   const int N = d.chain_nrows[ich], row0 = d.chain_row0[ich];
   float* fs = d.fsc32 + 4 * (size_t)row0;
   for (int r = 0; r < N; r++) {
      const int fc = d.row_fcell[row0 + r];
      float v[4] = {0.f, 0.f, 0.f, 0.f};
      if (fc >= 0) ld4(d.r32 + 4 * (size_t)fc, v);
      st4(fs + 4 * r, v);
   }
   if (d.chain_periodic[ich]) tridag_periodic<float>(d.blk32 + 48 * (size_t)row0, fs, N);
   else tridag_open<float>(d.blk32 + 48 * (size_t)row0, fs, N);
   for (int r = 0; r < N; r++) {
      float v[4];
      ld4(fs + 4 * r, v);
      st4(d.r32 + 4 * (size_t)d.row_scell[row0 + r], v);
   }
}

__global__ void __launch_bounds__(kThreads) mx_dq_update_kernel(DeviceState d)
{
   const int c = blockIdx.x * blockDim.x + threadIdx.x;
   if (c >= d.nCell || halted(d)) return;
   float r[4], dq[4];
   ld4(d.r32 + 4 * (size_t)c, r);
   ld4(d.dq32 + 4 * (size_t)c, dq);
#pragma unroll
   for (int k = 0; k < 4; k++) dq[k] += r[k];
   st4(d.dq32 + 4 * (size_t)c, dq);
}

template <int ORDER>
__global__ void __launch_bounds__(kThreads) mx_lin_face_kernel(DeviceState d)
{
   const int s = blockIdx.x * blockDim.x + threadIdx.x;
   if (s >= d.nSlot || halted(d)) return;
   const int4 sl = d.slot[s];
   float dL[4], dR[4];
   face_dstates<ORDER, float>(d, d.dq32, sl.x, (sl.w & 1) != 0, dL, dR);
   const float* m = d.ff32 + 32 * (size_t)(sl.w >> 1);
   float g[4];
#pragma unroll
   for (int j = 0; j < 4; j++) {
      float acc = 0.f;
#pragma unroll
      for (int k = 0; k < 4; k++) acc += ((m[4 * j + k] * dL[k]) + (m[16 + 4 * j + k] * dR[k]));
      g[j] = acc;
   }
   st4(d.g32 + 4 * (size_t)s, g);
}

template <bool UPDATE_Q>
__global__ void __launch_bounds__(kThreads) mx_lin_cell_kernel(DeviceState d)
{
   if (halted(d)) return;
   const int c = blockIdx.x * blockDim.x + threadIdx.x;
   double sq = 0.0, am = 0.0;
   if (c < d.nCell) {
      float r[4], r0[4], dq[4];
      ld4(d.r032 + 4 * (size_t)c, r0);
      ld4(d.dq32 + 4 * (size_t)c, dq);
#pragma unroll
      for (int k = 0; k < 4; k++) r[k] = r0[k] - dq[k];
      const float dt = float(d.dtfac[c]);
      const int e1 = d.cell_ptr[c + 1];
      for (int e = d.cell_ptr[c]; e < e1; e++) {
         const int ent = d.cell_ent[e];
         float g[4];
         ld4(d.g32 + 4 * (size_t)(ent >> 1), g);
         if (ent & 1) {
#pragma unroll
            for (int k = 0; k < 4; k++) r[k] += g[k] * dt;
         } else {
#pragma unroll
            for (int k = 0; k < 4; k++) r[k] -= g[k] * dt;
         }
      }
      st4(d.r32 + 4 * (size_t)c, r);
      sq = double(r[0]) * double(r[0]);
      am = fabs(double(r[0]));
      if (UPDATE_Q) {
         double q[4];
         ld4(d.q + 4 * (size_t)c, q);
#pragma unroll
         for (int k = 0; k < 4; k++) q[k] += double(dq[k]);
         st4(d.q + 4 * (size_t)c, q);
      }
   }
   // deterministic block reduction into norm_part
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

inline int blocks_for(int n) { return (n + kThreads - 1) / kThreads; }

}  // namespace

void launch_mx_rhs_face(const DeviceState& d, cudaStream_t st)
{
   const int b = blocks_for(d.nSlot);
   if (d.order == 1) mx_rhs_face_kernel<1><<<b, kThreads, 0, st>>>(d);
   else if (d.order == 3) mx_rhs_face_kernel<3><<<b, kThreads, 0, st>>>(d);
   else mx_rhs_face_kernel<5><<<b, kThreads, 0, st>>>(d);
}

void launch_mx_init(const DeviceState& d, cudaStream_t st) { mx_init_kernel<<<blocks_for(d.nCell), kThreads, 0, st>>>(d); }

void launch_mx_assemble(const DeviceState& d, cudaStream_t st)
{
   mx_assemble_kernel<<<blocks_for(48 * d.nRow), kThreads, 0, st>>>(d);
}

void launch_mx_lines(const DeviceState& d, int first, int count, cudaStream_t st)
{
   if (count > 0) mx_lines_kernel<<<(count + 63) / 64, 64, 0, st>>>(d, first, count);
}

void launch_mx_dq_update(const DeviceState& d, cudaStream_t st)
{
   mx_dq_update_kernel<<<blocks_for(d.nCell), kThreads, 0, st>>>(d);
}

void launch_mx_lin_face(const DeviceState& d, cudaStream_t st)
{
   const int b = blocks_for(d.nSlot);
   if (d.order == 1) mx_lin_face_kernel<1><<<b, kThreads, 0, st>>>(d);
   else if (d.order == 3) mx_lin_face_kernel<3><<<b, kThreads, 0, st>>>(d);
   else mx_lin_face_kernel<5><<<b, kThreads, 0, st>>>(d);
}

void launch_mx_lin_cell(const DeviceState& d, bool update_q, cudaStream_t st)
{
   if (update_q) mx_lin_cell_kernel<true><<<d.norm_blocks, kThreads, 0, st>>>(d);
   else mx_lin_cell_kernel<false><<<d.norm_blocks, kThreads, 0, st>>>(d);
}

}  // namespace hamstr
