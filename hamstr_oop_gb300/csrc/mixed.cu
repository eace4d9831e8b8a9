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
// chain running the block Thomas elimination in registers, with chains of
// similar length sharing a warp.
// ##################################################################
#include "device_state.h"
#include "plan.h"
#include "recon.cuh"
#include "roe.cuh"

namespace hamstr {

namespace {

constexpr int kThreads = 256;
static_assert(kThreads == kNormBlock, "cell kernels run one norm block per thread block");

// ---------------- residual + FP32 Jacobian ----------------
// PRE: the order-5 face states come from recon5_kernel
template <int ORDER, bool SD, bool PRE = false>
__global__ void __launch_bounds__(kThreads) mx_rhs_face_kernel(DeviceState d)
{
   // the FP32 Jacobians leave through shared memory, so their stores are
   // whole lines (8 float4 per slot, consecutive slots; row stride 9)
   __shared__ float4 sj[kThreads * 9];
   __shared__ unsigned char live[kThreads];
   if (halted(d)) return;
   const int nb = blockDim.x, s0 = blockIdx.x * nb, s = s0 + threadIdx.x;
   const bool act = s < d.nSlot && !frozen_slot(d, s);
   live[threadIdx.x] = act ? 1 : 0;
   if (act) {
      const int4 sl = d.slot[s];
      const double2 nv = d.normal[s];
      double L[4], R[4];
      if (ORDER == 5 && PRE) face_states_pre(d, s, (sl.w & 1) != 0, L, R);
      else face_states<ORDER, SD>(d, sl.x, (sl.w & 1) != 0, L, R);
      RoeOut o;
      if (!roe_face<false, SD>(nv.x, nv.y, L, R, d.fc.gamma, o, nullptr, nullptr))
         atomicOr(d.status, DEV_ERR_NAN_SPEC);
      st4(d.flux + 4 * (size_t)s, o.flux);
      d.spec[s] = o.spec;
      const float Lf[4] = {float(L[0]), float(L[1]), float(L[2]), float(L[3])};
      const float Rf[4] = {float(R[0]), float(R[1]), float(R[2]), float(R[3])};
      float lm[16], rm[16];
      roe_jacobian_only<float>(float(nv.x), float(nv.y), Lf, Rf, float(d.fc.gamma), lm, rm);
#pragma unroll
      for (int q = 0; q < 4; q++) {
         sj[threadIdx.x * 9 + q] = make_float4(lm[4 * q], lm[4 * q + 1], lm[4 * q + 2], lm[4 * q + 3]);
         sj[threadIdx.x * 9 + 4 + q] = make_float4(rm[4 * q], rm[4 * q + 1], rm[4 * q + 2], rm[4 * q + 3]);
      }
   }
   __syncthreads();
   const int nloc = min(nb, d.nSlot - s0);
   float4* __restrict__ dst = reinterpret_cast<float4*>(d.ff32 + 32 * (size_t)s0);
   for (int c = threadIdx.x; c < 8 * nloc; c += nb)
      if (live[c >> 3]) dst[c] = sj[(c >> 3) * 9 + (c & 7)];
}

// r (already scaled by CFL/sigma in FP64) -> FP32 r, r0; dq = 0
__global__ void __launch_bounds__(kThreads) mx_init_kernel(DeviceState d)
{
   const int c = blockIdx.x * blockDim.x + threadIdx.x;
   if (c >= d.nCell || halted(d) || frozen_cell(d, c)) return;
   double r[4];
   ld4(d.r + 4 * (size_t)c, r);
   const float rf[4] = {float(r[0]), float(r[1]), float(r[2]), float(r[3])};
   const float z[4] = {0.f, 0.f, 0.f, 0.f};
   st4(d.r32 + 4 * (size_t)c, rf);
   st4(d.r032 + 4 * (size_t)c, rf);
   st4(d.dq32 + 4 * (size_t)c, z);
}

// FP32 blocks in the reference's term order (ADI.cpp:62-217), one thread
// per block entry (coalesced); the unfused alternative to mx_row below,
// faster where chains are short (the autotuner picks)
__global__ void __launch_bounds__(kThreads) mx_assemble_kernel(DeviceState d)
{
   // one thread per tiled entry (DeviceState: blk32), so stores are whole lines
   const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
   if (t >= 48 * 32 * (size_t)d.tile_rows || halted(d)) return;
   const int lane = (int)(t & 31);
   const size_t q = t >> 5;
   const int e48 = (int)(q % 48), srow = (int)(q / 48), b = e48 >> 4, e = e48 & 15;
   const int row = d.tile_row[32 * (size_t)srow + lane];
   if (row < 0 || frozen_cell(d, d.row_scell[row])) return;
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

// the tiled index of element e of tile row s in lane `lane` of a W-wide array
__device__ __forceinline__ size_t tix(int s, int W, int e, int lane)
{
   return (((size_t)s * W + e) << 5) + lane;
}

// 16 consecutive elements of a tiled record (stride 32 floats: each load of
// a warp is one 128-byte line)
__device__ __forceinline__ void ld16t(const float* __restrict__ p, float (&v)[16])
{
#pragma unroll
   for (int m = 0; m < 16; m++) v[m] = p[32 * m];
}

__device__ __forceinline__ void st16t(float* __restrict__ p, const float (&v)[16])
{
#pragma unroll
   for (int m = 0; m < 16; m++) p[32 * m] = v[m];
}

// ---------------- FP32 line solves, one thread per chain ----------------
// The same split as the FP64 path: the block factorisation runs once per
// step (mx_factor), each sweep replays the right-hand side (mx_solve).  One
// thread carries a whole chain in registers (FP32 latency is 4 cycles, so
// the recurrence is short), rows are loaded one ahead or several rows at a
// time, and products use FMA since this operator is approximate by design.  Record layout per row
// (80 floats): A, LU of B', C', fill-in a', c_{N-1} at elimination step i.
constexpr int kRec = 80;

struct LUf {
   float p0, u01, u02, u03, l10, p1, u12, u13, l20, l21, p2, u23, l30, l31, l32, p3;
};

__device__ __forceinline__ LUf luf_factor(const float (&b)[16])
{
   LUf u;
   u.p0 = 1.f / b[0];
   u.u01 = b[1] * u.p0; u.u02 = b[2] * u.p0; u.u03 = b[3] * u.p0;
   u.l10 = b[4];
   u.p1 = 1.f / __fmaf_rn(-u.l10, u.u01, b[5]);
   u.u12 = __fmaf_rn(-u.l10, u.u02, b[6]) * u.p1;
   u.u13 = __fmaf_rn(-u.l10, u.u03, b[7]) * u.p1;
   u.l20 = b[8];
   u.l21 = __fmaf_rn(-u.l20, u.u01, b[9]);
   u.p2 = 1.f / __fmaf_rn(-u.l21, u.u12, __fmaf_rn(-u.l20, u.u02, b[10]));
   u.u23 = __fmaf_rn(-u.l21, u.u13, __fmaf_rn(-u.l20, u.u03, b[11])) * u.p2;
   u.l30 = b[12];
   u.l31 = __fmaf_rn(-u.l30, u.u01, b[13]);
   u.l32 = __fmaf_rn(-u.l31, u.u12, __fmaf_rn(-u.l30, u.u02, b[14]));
   u.p3 = 1.f / __fmaf_rn(-u.l32, u.u23, __fmaf_rn(-u.l31, u.u13, __fmaf_rn(-u.l30, u.u03, b[15])));
   return u;
}

__device__ __forceinline__ void luf_solve(const LUf& u, float& x0, float& x1, float& x2, float& x3)
{
   const float d0 = x0 * u.p0;
   const float d1 = __fmaf_rn(-u.l10, d0, x1) * u.p1;
   const float d2 = __fmaf_rn(-u.l21, d1, __fmaf_rn(-u.l20, d0, x2)) * u.p2;
   const float d3 = __fmaf_rn(-u.l32, d2, __fmaf_rn(-u.l31, d1, __fmaf_rn(-u.l30, d0, x3))) * u.p3;
   x3 = d3;
   x2 = __fmaf_rn(-u.u23, x3, d2);
   x1 = __fmaf_rn(-u.u13, x3, __fmaf_rn(-u.u12, x2, d1));
   x0 = __fmaf_rn(-u.u03, x3, __fmaf_rn(-u.u02, x2, __fmaf_rn(-u.u01, x1, d0)));
}

__device__ __forceinline__ void luf_store(float* p, const LUf& u)
{
   const float v[16] = {u.p0, u.u01, u.u02, u.u03, u.l10, u.p1, u.u12, u.u13,
                        u.l20, u.l21, u.p2, u.u23, u.l30, u.l31, u.l32, u.p3};
#pragma unroll
   for (int m = 0; m < 16; m += 4) *reinterpret_cast<float4*>(p + m) = make_float4(v[m], v[m + 1], v[m + 2], v[m + 3]);
}

__device__ __forceinline__ LUf luf_load(const float* p)
{
   float v[16];
#pragma unroll
   for (int m = 0; m < 16; m += 4) {
      const float4 a = *reinterpret_cast<const float4*>(p + m);
      v[m] = a.x; v[m + 1] = a.y; v[m + 2] = a.z; v[m + 3] = a.w;
   }
   LUf u;
   u.p0 = v[0]; u.u01 = v[1]; u.u02 = v[2]; u.u03 = v[3]; u.l10 = v[4]; u.p1 = v[5]; u.u12 = v[6]; u.u13 = v[7];
   u.l20 = v[8]; u.l21 = v[9]; u.p2 = v[10]; u.u23 = v[11]; u.l30 = v[12]; u.l31 = v[13]; u.l32 = v[14]; u.p3 = v[15];
   return u;
}

// the LU record of a tiled row (stride 32 floats)
__device__ __forceinline__ void luf_store_t(float* p, const LUf& u)
{
   const float v[16] = {u.p0, u.u01, u.u02, u.u03, u.l10, u.p1, u.u12, u.u13,
                        u.l20, u.l21, u.p2, u.u23, u.l30, u.l31, u.l32, u.p3};
#pragma unroll
   for (int m = 0; m < 16; m++) p[32 * m] = v[m];
}

__device__ __forceinline__ LUf luf_load_t(const float* p)
{
   LUf u;
   u.p0 = p[0]; u.u01 = p[32]; u.u02 = p[64]; u.u03 = p[96]; u.l10 = p[128]; u.p1 = p[160]; u.u12 = p[192];
   u.u13 = p[224]; u.l20 = p[256]; u.l21 = p[288]; u.p2 = p[320]; u.u23 = p[352]; u.l30 = p[384];
   u.l31 = p[416]; u.l32 = p[448]; u.p3 = p[480];
   return u;
}

__device__ __forceinline__ void ld16f(const float* p, float (&v)[16])
{
#pragma unroll
   for (int m = 0; m < 16; m += 4) {
      const float4 a = *reinterpret_cast<const float4*>(p + m);
      v[m] = a.x; v[m + 1] = a.y; v[m + 2] = a.z; v[m + 3] = a.w;
   }
}

__device__ __forceinline__ void st16f(float* p, const float (&v)[16])
{
#pragma unroll
   for (int m = 0; m < 16; m += 4) *reinterpret_cast<float4*>(p + m) = make_float4(v[m], v[m + 1], v[m + 2], v[m + 3]);
}

// M <- LU^{-1} M, column by column
__device__ __forceinline__ void luf_cols(const LUf& u, float (&m)[16])
{
#pragma unroll
   for (int j = 0; j < 4; j++) luf_solve(u, m[j], m[4 + j], m[8 + j], m[12 + j]);
}

// out = acc - M * X (4x4), acc = nullptr for 0
__device__ __forceinline__ void mm_sub(const float (&M)[16], const float (&X)[16], float (&acc)[16])
{
#pragma unroll
   for (int k = 0; k < 4; k++)
#pragma unroll
      for (int j = 0; j < 4; j++) {
         float a = acc[4 * k + j];
#pragma unroll
         for (int l = 0; l < 4; l++) a = __fmaf_rn(-M[4 * k + l], X[4 * l + j], a);
         acc[4 * k + j] = a;
      }
}

// One FP32 block from its term list, in the reference's term order
// (ADI.cpp:62-217): +/- L or R of a face slot, or R with its velocity
// columns reflected at a wall (ADI.cpp:151-163)
__device__ __forceinline__ void mx_block(const DeviceState& d, const int* __restrict__ ops, float (&M)[16])
{
#pragma unroll
   for (int m = 0; m < 16; m++) M[m] = 0.f;
#pragma unroll
   for (int o = 0; o < kOpsPerBlock; o++) {
      const int op = ops[o];
      if (op < 0) break;
      const int slot = op >> 3, sel = (op >> 1) & 3;
      float v[16];
      ld16f(d.ff32 + 32 * (size_t)slot + (sel == OP_SEL_L ? 0 : 16), v);
      if (sel == OP_SEL_RREFL) {
         const double4 rf = d.refl[d.slot_face[slot]];
#pragma unroll
         for (int k = 0; k < 4; k++) {
            const float r01 = v[4 * k + 1], r02 = v[4 * k + 2];
            v[4 * k + 1] = float(rf.x) * r01 + float(rf.y) * r02;
            v[4 * k + 2] = float(rf.z) * r01 + float(rf.w) * r02;
         }
      }
      if (op & 1) {
#pragma unroll
         for (int m = 0; m < 16; m++) M[m] -= v[m];
      } else {
#pragma unroll
         for (int m = 0; m < 16; m++) M[m] += v[m];
      }
   }
}

// what the fused assembly of one row looks up first: its term lists and
// its scaled cell (the face Jacobians and the CFL/sigma factor follow from
// them), loaded a row earlier than the blocks so that each row waits on
// one memory round trip, not two
struct RowRef {
   int4 ops[3];
   int scell;
};

__device__ __forceinline__ RowRef mx_rowref(const DeviceState& d, int row)
{
   RowRef r;
   const int4* p = reinterpret_cast<const int4*>(d.row_ops + 3 * kOpsPerBlock * (size_t)row);
   r.ops[0] = p[0];
   r.ops[1] = p[1];
   r.ops[2] = p[2];
   r.scell = d.row_scell[row];
   return r;
}

// the three blocks of one ADI row from its looked-up references, scaled by
// CFL/sigma, B + I (ADI.cpp:197-217)
__device__ __forceinline__ void mx_row_ref(const DeviceState& d, const RowRef& r, float (&A)[16], float (&B)[16],
                                           float (&C)[16])
{
   const int oa[4] = {r.ops[0].x, r.ops[0].y, r.ops[0].z, r.ops[0].w};
   const int ob[4] = {r.ops[1].x, r.ops[1].y, r.ops[1].z, r.ops[1].w};
   const int oc[4] = {r.ops[2].x, r.ops[2].y, r.ops[2].z, r.ops[2].w};
   mx_block(d, oa, A);
   mx_block(d, ob, B);
   mx_block(d, oc, C);
   const float s = float(d.dtfac[r.scell]);
#pragma unroll
   for (int m = 0; m < 16; m++) {
      A[m] *= s;
      B[m] *= s;
      C[m] *= s;
   }
#pragma unroll
   for (int k = 0; k < 4; k++) B[5 * k] += 1.f;
}

// FUSED: each thread builds its chain's blocks straight from the FP32 face
// Jacobians (no block array round trip; best for long chains) from the
// references r of the row; otherwise it reads the blocks mx_assemble_kernel
// wrote (tile row s, its lane)
template <bool FUSED>
__device__ __forceinline__ void mx_rows(const DeviceState& d, const RowRef& r, int s, int lane, float (&A)[16],
                                        float (&B)[16], float (&C)[16])
{
   if (FUSED) {
      mx_row_ref(d, r, A, B, C);
   } else {
      ld16t(d.blk32 + tix(s, 48, 0, lane), A);
      ld16t(d.blk32 + tix(s, 48, 16, lane), B);
      ld16t(d.blk32 + tix(s, 48, 32, lane), C);
   }
}

// rows of the periodic last-row elimination whose loads issue together
// where all chains are resident at once (1 otherwise: there the kernel is
// bound by throughput, not by one chain's round trips)
constexpr int kElimChunk = 2;

// all chains, thread p on the chain at position p of line_chains; ED rows of
// the last-row elimination per chunk
template <bool FUSED, int ED>
__global__ void __launch_bounds__(256) mx_factor_kernel(DeviceState d, int count)
{
   const int t = blockIdx.x * blockDim.x + threadIdx.x;
   if (t >= count || halted(d)) return;
   const int ich = d.line_chains[t];
   if (frozen_chain(d, ich) || (d.sp_on && d.chain_spike[ich] >= 0)) return;
   const int N = d.chain_nrows[ich], row0 = d.chain_row0[ich], lane = t & 31, s0 = d.grp_row0[t >> 5];
   const bool per = d.chain_periodic[ich] != 0;
   float A[16], B[16], C[16], cp[16], ap[16];
   bool bad = false;   // a reciprocal pivot is not finite (DEV_ERR_PIVOT)
   RowRef rnext{};   // fused: references of row i + 1, looked up a row ahead
   if (FUSED) {
      const RowRef r0 = mx_rowref(d, row0);
      if (N > 1) rnext = mx_rowref(d, row0 + 1);
      mx_rows<FUSED>(d, r0, s0, lane, A, B, C);
   } else {
      mx_rows<FUSED>(d, rnext, s0, lane, A, B, C);
   }
   for (int i = 0; i < N; i++) {
      float An[16], Bn[16], Cn[16];
      if (i + 1 < N) {
         mx_rows<FUSED>(d, rnext, s0 + i + 1, lane, An, Bn, Cn);
         if (FUSED && i + 2 < N) rnext = mx_rowref(d, row0 + i + 2);
      }
      float* rec = d.fac32 + tix(s0 + i, kRec, 0, lane);
      st16t(rec, A);
      float fill[16];
      if (i > 0) {
         mm_sub(A, cp, B);
#pragma unroll
         for (int m = 0; m < 16; m++) fill[m] = 0.f;
         if (per) mm_sub(A, ap, fill);
      } else {
#pragma unroll
         for (int m = 0; m < 16; m++) fill[m] = A[m];
      }
      const LUf u = luf_factor(B);
      luf_store_t(rec + 32 * 16, u);
      bad |= nonfinite(u.p0) || nonfinite(u.p1) || nonfinite(u.p2) || nonfinite(u.p3);
      if (per && i == N - 2) {
#pragma unroll
         for (int m = 0; m < 16; m++) C[m] += fill[m];
         luf_cols(u, C);
#pragma unroll
         for (int m = 0; m < 16; m++) fill[m] = C[m];
      } else {
         luf_cols(u, C);
         if (per) luf_cols(u, fill);
      }
      st16t(rec + 32 * 32, C);
      if (per) st16t(rec + 32 * 48, fill);
#pragma unroll
      for (int m = 0; m < 16; m++) { cp[m] = C[m]; ap[m] = fill[m]; }
      if (i + 1 < N) {
#pragma unroll
         for (int m = 0; m < 16; m++) { A[m] = An[m]; B[m] = Bn[m]; C[m] = Cn[m]; }
      }
   }
   if (!per) {
      if (bad) atomicOr(d.status, DEV_ERR_PIVOT);
      return;
   }
   // last-row elimination (triSolvers.cpp:967-999).  A row's arithmetic is
   // short, so the loads of ED rows are issued before it; the main loop's
   // arrays are dead here, so a chunk of 2 adds no registers.
   constexpr int D = ED;
   float cN[16], bN[16];
#pragma unroll
   for (int m = 0; m < 16; m++) { cN[m] = cp[m]; bN[m] = ((m >> 2) == (m & 3)) ? 1.f : 0.f; }
   for (int i0 = 0; i0 < N - 1; i0 += D) {
      float ci[D][16], ai[D][16];
#pragma unroll
      for (int u = 0; u < D; u++)
         if (i0 + u < N - 1) {
            const float* rec = d.fac32 + tix(s0 + i0 + u, kRec, 0, lane);
            ld16t(rec + 32 * 32, ci[u]);
            ld16t(rec + 32 * 48, ai[u]);
         }
#pragma unroll
      for (int u = 0; u < D; u++)
         if (i0 + u < N - 1) {
            st16t(d.fac32 + tix(s0 + i0 + u, kRec, 64, lane), cN);
            float tt[16];
#pragma unroll
            for (int m = 0; m < 16; m++) tt[m] = 0.f;
            mm_sub(cN, ci[u], tt);
            mm_sub(cN, ai[u], bN);
#pragma unroll
            for (int m = 0; m < 16; m++) cN[m] = tt[m];
         }
   }
   const LUf uN = luf_factor(bN);
   luf_store(d.facN32 + 16 * d.chain_facN[ich], uN);
   bad |= nonfinite(uN.p0) || nonfinite(uN.p1) || nonfinite(uN.p2) || nonfinite(uN.p3);
   if (bad) atomicOr(d.status, DEV_ERR_PIVOT);
}

// One sweep's solve of one chain per thread (the chain at position first +
// t of line_chains).  The recurrence only carries the 4-vector x in
// registers; everything a row needs (its factor record, its right-hand
// side, the cell it writes) is loaded one row ahead, so the loads overlap
// the previous row's arithmetic.  Solutions go straight to r32 (each cell
// is written once per chain; chains of a wave share no cell).
__global__ void __launch_bounds__(256) mx_solve_kernel(DeviceState d, int first, int count)
{
   const int t = blockIdx.x * blockDim.x + threadIdx.x;
   if (t >= count || halted(d)) return;
   const int p = first + t;
   const int ich = d.line_chains[p];
   if (frozen_chain(d, ich) || (d.sp_on && d.chain_spike[ich] >= 0)) return;
   const int N = d.chain_nrows[ich], row0 = d.chain_row0[ich], lane = p & 31, s0 = d.grp_row0[p >> 5];
   const bool per = d.chain_periodic[ich] != 0;
   const int* fcell = d.row_fcell + row0;
   const int* scell = d.row_scell + row0;
   // forward: f(i) = LU^{-1}(F(i) - A(i) f(i-1)), F(i) = r[fcell]
   float xp[4] = {0.f, 0.f, 0.f, 0.f};
   float a[16], xr[4] = {0.f, 0.f, 0.f, 0.f};
   LUf u;
   int fcn = -1;   // the next row's right-hand-side cell, looked up a row ahead
   {
      const int fc = fcell[0];
      if (fc >= 0) ld4(d.r32 + 4 * (size_t)fc, xr);
      if (N > 1) fcn = fcell[1];
      u = luf_load_t(d.fac32 + tix(s0, kRec, 16, lane));
#pragma unroll
      for (int m = 0; m < 16; m++) a[m] = 0.f;
   }
   for (int i = 0; i < N; i++) {
      // next row's record and right-hand side, in flight during this row
      float an[16], xrn[4] = {0.f, 0.f, 0.f, 0.f};
      LUf un;
      if (i + 1 < N) {
         const float* rn = d.fac32 + tix(s0 + i + 1, kRec, 0, lane);
         if (fcn >= 0) ld4(d.r32 + 4 * (size_t)fcn, xrn);
         fcn = (i + 2 < N) ? fcell[i + 2] : -1;
         ld16t(rn, an);
         un = luf_load_t(rn + 32 * 16);
      }
      float x[4] = {xr[0], xr[1], xr[2], xr[3]};
      if (i > 0) {
#pragma unroll
         for (int k = 0; k < 4; k++)
#pragma unroll
            for (int j = 0; j < 4; j++) x[k] = __fmaf_rn(-a[4 * k + j], xp[j], x[k]);
      }
      luf_solve(u, x[0], x[1], x[2], x[3]);
      float* fs = d.fsc32 + tix(s0 + i, 4, 0, lane);
#pragma unroll
      for (int k = 0; k < 4; k++) fs[32 * k] = x[k];
#pragma unroll
      for (int k = 0; k < 4; k++) xp[k] = x[k];
      if (i + 1 < N) {
#pragma unroll
         for (int m = 0; m < 16; m++) a[m] = an[m];
#pragma unroll
         for (int k = 0; k < 4; k++) xr[k] = xrn[k];
         u = un;
      }
   }
   float xn[4];
   if (per) {
      float fN[4] = {xp[0], xp[1], xp[2], xp[3]};
      for (int i = 0; i < N - 1; i++) {
         float c[16], f[4];
         ld16t(d.fac32 + tix(s0 + i, kRec, 64, lane), c);
         const float* fs = d.fsc32 + tix(s0 + i, 4, 0, lane);
#pragma unroll
         for (int k = 0; k < 4; k++) f[k] = fs[32 * k];
#pragma unroll
         for (int k = 0; k < 4; k++)
#pragma unroll
            for (int j = 0; j < 4; j++) fN[k] = __fmaf_rn(-c[4 * k + j], f[j], fN[k]);
      }
      const LUf uN = luf_load(d.facN32 + 16 * d.chain_facN[ich]);
      luf_solve(uN, fN[0], fN[1], fN[2], fN[3]);
      st4(d.r32 + 4 * (size_t)scell[N - 1], fN);
#pragma unroll
      for (int k = 0; k < 4; k++) xn[k] = fN[k];
      for (int i = N - 2; i >= 0; i--) {
         const float* rec = d.fac32 + tix(s0 + i, kRec, 0, lane);
         float c[16], aa[16], x[4];
         ld16t(rec + 32 * 32, c);
         ld16t(rec + 32 * 48, aa);
         const float* fs = d.fsc32 + tix(s0 + i, 4, 0, lane);
#pragma unroll
         for (int k = 0; k < 4; k++) x[k] = fs[32 * k];
#pragma unroll
         for (int k = 0; k < 4; k++)
#pragma unroll
            for (int j = 0; j < 4; j++) {
               const float sv = (i == N - 2) ? c[4 * k + j] * xn[j] : __fmaf_rn(aa[4 * k + j], fN[j], c[4 * k + j] * xn[j]);
               x[k] -= sv;
            }
         st4(d.r32 + 4 * (size_t)scell[i], x);
#pragma unroll
         for (int k = 0; k < 4; k++) xn[k] = x[k];
      }
   } else {
#pragma unroll
      for (int k = 0; k < 4; k++) xn[k] = xp[k];
      st4(d.r32 + 4 * (size_t)scell[N - 1], xn);
      // back substitution, row i-1's factor and f prefetched
      float c[16], x[4];
      int sc = 0;
      if (N >= 2) {
         ld16t(d.fac32 + tix(s0 + N - 2, kRec, 32, lane), c);
         const float* fs = d.fsc32 + tix(s0 + N - 2, 4, 0, lane);
#pragma unroll
         for (int k = 0; k < 4; k++) x[k] = fs[32 * k];
         sc = scell[N - 2];
      }
      for (int i = N - 2; i >= 0; i--) {
         float cn[16], xnx[4];
         int scn = 0;
         if (i >= 1) {
            ld16t(d.fac32 + tix(s0 + i - 1, kRec, 32, lane), cn);
            const float* fs = d.fsc32 + tix(s0 + i - 1, 4, 0, lane);
#pragma unroll
            for (int k = 0; k < 4; k++) xnx[k] = fs[32 * k];
            scn = scell[i - 1];
         }
#pragma unroll
         for (int k = 0; k < 4; k++)
#pragma unroll
            for (int j = 0; j < 4; j++) x[k] = __fmaf_rn(-c[4 * k + j], xn[j], x[k]);
         st4(d.r32 + 4 * (size_t)sc, x);
#pragma unroll
         for (int k = 0; k < 4; k++) xn[k] = x[k];
         if (i >= 1) {
#pragma unroll
            for (int m = 0; m < 16; m++) c[m] = cn[m];
#pragma unroll
            for (int k = 0; k < 4; k++) x[k] = xnx[k];
            sc = scn;
         }
      }
   }
}

// rows whose loads mx_solve_chunk_kernel issues together
constexpr int kSolveChunk = 4;

// The same solve with the loads of kSolveChunk rows issued together before
// their arithmetic, in each of the row loops.  A row's own arithmetic is a
// few dozen dependent FP32 operations, far shorter than one memory round
// trip, so a chain of N rows waits about N / kSolveChunk round trips instead
// of N.  The operations and their order are those of mx_solve_kernel, so
// the results are identical.  It takes more registers; the host launches it
// for waves whose chains are all resident at once.
__global__ void __launch_bounds__(256) mx_solve_chunk_kernel(DeviceState d, int first, int count)
{
   constexpr int D = kSolveChunk;
   const int t = blockIdx.x * blockDim.x + threadIdx.x;
   if (t >= count || halted(d)) return;
   const int p = first + t;
   const int ich = d.line_chains[p];
   if (frozen_chain(d, ich) || (d.sp_on && d.chain_spike[ich] >= 0)) return;
   const int N = d.chain_nrows[ich], row0 = d.chain_row0[ich], lane = p & 31, s0 = d.grp_row0[p >> 5];
   const bool per = d.chain_periodic[ich] != 0;
   const int* fcell = d.row_fcell + row0;
   const int* scell = d.row_scell + row0;
   // forward: f(i) = LU^{-1}(F(i) - A(i) f(i-1)), F(i) = r[fcell]; the
   // right-hand-side cells of a chunk are looked up during the chunk before
   float xp[4] = {0.f, 0.f, 0.f, 0.f};
   int fcb[D];
#pragma unroll
   for (int u = 0; u < D; u++) fcb[u] = (u < N) ? fcell[u] : -1;
   for (int i0 = 0; i0 < N; i0 += D) {
      float ab[D][16], xb[D][4];
      LUf ub[D];
#pragma unroll
      for (int u = 0; u < D; u++) {
         const int i = i0 + u;
#pragma unroll
         for (int k = 0; k < 4; k++) xb[u][k] = 0.f;
         if (i < N) {
            const float* rec = d.fac32 + tix(s0 + i, kRec, 0, lane);
            if (fcb[u] >= 0) ld4(d.r32 + 4 * (size_t)fcb[u], xb[u]);
            if (i > 0) ld16t(rec, ab[u]);
            ub[u] = luf_load_t(rec + 32 * 16);
         }
      }
#pragma unroll
      for (int u = 0; u < D; u++) fcb[u] = (i0 + D + u < N) ? fcell[i0 + D + u] : -1;
#pragma unroll
      for (int u = 0; u < D; u++) {
         const int i = i0 + u;
         if (i < N) {
            float x[4] = {xb[u][0], xb[u][1], xb[u][2], xb[u][3]};
            if (i > 0) {
#pragma unroll
               for (int k = 0; k < 4; k++)
#pragma unroll
                  for (int j = 0; j < 4; j++) x[k] = __fmaf_rn(-ab[u][4 * k + j], xp[j], x[k]);
            }
            luf_solve(ub[u], x[0], x[1], x[2], x[3]);
            float* fs = d.fsc32 + tix(s0 + i, 4, 0, lane);
#pragma unroll
            for (int k = 0; k < 4; k++) fs[32 * k] = x[k];
#pragma unroll
            for (int k = 0; k < 4; k++) xp[k] = x[k];
         }
      }
   }
   float xn[4];
   if (per) {
      // last row: f(N-1) - sum over i < N-1 of cN(i) f(i), in row order
      float fN[4] = {xp[0], xp[1], xp[2], xp[3]};
      for (int i0 = 0; i0 < N - 1; i0 += D) {
         float cb[D][16], fb[D][4];
#pragma unroll
         for (int u = 0; u < D; u++) {
            const int i = i0 + u;
            if (i < N - 1) {
               ld16t(d.fac32 + tix(s0 + i, kRec, 64, lane), cb[u]);
               const float* fs = d.fsc32 + tix(s0 + i, 4, 0, lane);
#pragma unroll
               for (int k = 0; k < 4; k++) fb[u][k] = fs[32 * k];
            }
         }
#pragma unroll
         for (int u = 0; u < D; u++) {
            if (i0 + u < N - 1) {
#pragma unroll
               for (int k = 0; k < 4; k++)
#pragma unroll
                  for (int j = 0; j < 4; j++) fN[k] = __fmaf_rn(-cb[u][4 * k + j], fb[u][j], fN[k]);
            }
         }
      }
      const LUf uN = luf_load(d.facN32 + 16 * d.chain_facN[ich]);
      luf_solve(uN, fN[0], fN[1], fN[2], fN[3]);
      st4(d.r32 + 4 * (size_t)scell[N - 1], fN);
#pragma unroll
      for (int k = 0; k < 4; k++) xn[k] = fN[k];
      // back substitution with the fill-in column, rows N-2 down to 0
      for (int i0 = N - 2; i0 >= 0; i0 -= D) {
         float cb[D][16], ab[D][16], fb[D][4];
         int sb[D];
#pragma unroll
         for (int u = 0; u < D; u++) {
            const int i = i0 - u;
            if (i >= 0) {
               const float* rec = d.fac32 + tix(s0 + i, kRec, 0, lane);
               ld16t(rec + 32 * 32, cb[u]);
               ld16t(rec + 32 * 48, ab[u]);
               const float* fs = d.fsc32 + tix(s0 + i, 4, 0, lane);
#pragma unroll
               for (int k = 0; k < 4; k++) fb[u][k] = fs[32 * k];
               sb[u] = scell[i];
            }
         }
#pragma unroll
         for (int u = 0; u < D; u++) {
            const int i = i0 - u;
            if (i >= 0) {
               float x[4] = {fb[u][0], fb[u][1], fb[u][2], fb[u][3]};
#pragma unroll
               for (int k = 0; k < 4; k++)
#pragma unroll
                  for (int j = 0; j < 4; j++) {
                     const float sv = (i == N - 2) ? cb[u][4 * k + j] * xn[j]
                                                   : __fmaf_rn(ab[u][4 * k + j], fN[j], cb[u][4 * k + j] * xn[j]);
                     x[k] -= sv;
                  }
               st4(d.r32 + 4 * (size_t)sb[u], x);
#pragma unroll
               for (int k = 0; k < 4; k++) xn[k] = x[k];
            }
         }
      }
   } else {
#pragma unroll
      for (int k = 0; k < 4; k++) xn[k] = xp[k];
      st4(d.r32 + 4 * (size_t)scell[N - 1], xn);
      // back substitution, rows N-2 down to 0
      for (int i0 = N - 2; i0 >= 0; i0 -= D) {
         float cb[D][16], fb[D][4];
         int sb[D];
#pragma unroll
         for (int u = 0; u < D; u++) {
            const int i = i0 - u;
            if (i >= 0) {
               ld16t(d.fac32 + tix(s0 + i, kRec, 32, lane), cb[u]);
               const float* fs = d.fsc32 + tix(s0 + i, 4, 0, lane);
#pragma unroll
               for (int k = 0; k < 4; k++) fb[u][k] = fs[32 * k];
               sb[u] = scell[i];
            }
         }
#pragma unroll
         for (int u = 0; u < D; u++) {
            if (i0 - u >= 0) {
               float x[4] = {fb[u][0], fb[u][1], fb[u][2], fb[u][3]};
#pragma unroll
               for (int k = 0; k < 4; k++)
#pragma unroll
                  for (int j = 0; j < 4; j++) x[k] = __fmaf_rn(-cb[u][4 * k + j], xn[j], x[k]);
               st4(d.r32 + 4 * (size_t)sb[u], x);
#pragma unroll
               for (int k = 0; k < 4; k++) xn[k] = x[k];
            }
         }
      }
   }
}

// ---------------- long periodic chains by segments ----------------------
// A periodic chain of N rows (A_i x_{i-1} + B_i x_i + C_i x_{i+1} = f_i,
// indices mod N) is cut into P segments of about N/P rows, one lane of a
// warp each.  With D_p the block-tridiagonal matrix of segment p alone
// (rows s..e), its solution is
//     x_i = y_i + V_i x_{e+1} + W_i x_{s-1},
// where D_p y = f, D_p V = -C_e (in the last row) and D_p W = -A_s (in the
// first row): V and W are the "spikes", the segment's responses to the
// couplings across its two ends.  With b_p = x_e and t_p = x_s of segment
// p, the rows at the segment ends give a cyclic system in the interface
// pairs Z_p = (b_p, t_{p+1}):
//     b_p     - V_e(p) t_{p+1} - W_e(p) b_{p-1}   = y_e(p)
//     t_{p+1} - V_s(p+1) t_{p+2} - W_s(p+1) b_p   = y_s(p+1)
// i.e. L_p Z_{p-1} + D_p Z_p + U_p Z_{p+1} = R_p with 8x8 blocks, which
// lane 0 solves by a cyclic block elimination onto Z_{P-1}.  This is the
// same linear system the sequential cyclic block Thomas solves (in FP32 it
// differs in rounding only), with N/P + P rows of latency instead of N.
// The segment factors and spikes, and the boundary system's factors, are
// formed once per step; each sweep replays the right-hand side.

// sp_fac record of one row: A, LU of the segment's B', C' (no C' on a
// segment's last row), V, W
constexpr int kSpRec = 80;

// 8x8 row-major matrices of the boundary system (lane 0, local arrays)
// LU with reciprocal pivots: M = L U, U unit upper; L below and on the
// diagonal (the diagonal holding 1/L_kk)
__device__ void m8_lu(float* M)
{
   for (int k = 0; k < 8; k++) {
      const float piv = 1.f / M[9 * k];
      M[9 * k] = piv;
      for (int j = k + 1; j < 8; j++) M[8 * k + j] *= piv;
      for (int i = k + 1; i < 8; i++) {
         const float l = M[8 * i + k];
         for (int j = k + 1; j < 8; j++) M[8 * i + j] = __fmaf_rn(-l, M[8 * k + j], M[8 * i + j]);
      }
   }
}

// x <- M^{-1} x for the 8 values x[0], x[s], .., x[7s]
__device__ void m8_solve(const float* LU, float* x, int s)
{
   for (int i = 0; i < 8; i++) {
      float v = x[s * i];
      for (int k = 0; k < i; k++) v = __fmaf_rn(-LU[8 * i + k], x[s * k], v);
      x[s * i] = v * LU[9 * i];
   }
   for (int i = 6; i >= 0; i--) {
      float v = x[s * i];
      for (int j = i + 1; j < 8; j++) v = __fmaf_rn(-LU[8 * i + j], x[s * j], v);
      x[s * i] = v;
   }
}

// C = alpha C - A B (alpha 0 or 1)
__device__ void m8_msub(float* C, const float* A, const float* B, bool keep)
{
   for (int i = 0; i < 8; i++)
      for (int j = 0; j < 8; j++) {
         float v = keep ? C[8 * i + j] : 0.f;
         for (int k = 0; k < 8; k++) v = __fmaf_rn(-A[8 * i + k], B[8 * k + j], v);
         C[8 * i + j] = v;
      }
}

// y = alpha y - M x on 8-vectors
__device__ __forceinline__ void v8_msub(float* y, const float* M, const float* x)
{
   for (int i = 0; i < 8; i++) {
      float v = y[i];
      for (int k = 0; k < 8; k++) v = __fmaf_rn(-M[8 * i + k], x[k], v);
      y[i] = v;
   }
}

__device__ __forceinline__ void ldm8(const float* __restrict__ p, float* m)
{
   for (int e = 0; e < 64; e += 4) {
      const float4 v = *reinterpret_cast<const float4*>(p + e);
      m[e] = v.x; m[e + 1] = v.y; m[e + 2] = v.z; m[e + 3] = v.w;
   }
}

__device__ __forceinline__ void stm8(float* __restrict__ p, const float* m)
{
   for (int e = 0; e < 64; e += 4) *reinterpret_cast<float4*>(p + e) = make_float4(m[e], m[e + 1], m[e + 2], m[e + 3]);
}

// the blocks of row p of the boundary system from the segments' spike tips
// (sh: [p][4][16] = V_s, W_s, V_e, W_e of segment p)
__device__ void red_blocks(const float* sh, int p, int P, float* L, float* D, float* U)
{
   const int q = (p + 1 == P) ? 0 : p + 1;
   const float* Vs1 = sh + 64 * q;
   const float* Ws1 = sh + 64 * q + 16;
   const float* Ve = sh + 64 * p + 32;
   const float* We = sh + 64 * p + 48;
   for (int e = 0; e < 64; e++) { L[e] = 0.f; D[e] = 0.f; U[e] = 0.f; }
   for (int k = 0; k < 4; k++)
      for (int j = 0; j < 4; j++) {
         L[8 * k + j] = -We[4 * k + j];
         D[8 * k + 4 + j] = -Ve[4 * k + j];
         D[8 * (4 + k) + j] = -Ws1[4 * k + j];
         U[8 * (4 + k) + 4 + j] = -Vs1[4 * k + j];
      }
   for (int k = 0; k < 8; k++) D[9 * k] = 1.f;
}

// sp_red layout of one chain: row p < P-1 at 256 p: LU(M_p), L_p, G_p, B_p;
// then LU(K), L_{P-1}, U_{P-1} at 256 (kSpikeMaxSeg - 1)
__device__ __forceinline__ float* red_row(float* red, int p, int m) { return red + 256 * p + 64 * m; }
__device__ __forceinline__ const float* red_row(const float* red, int p, int m) { return red + 256 * p + 64 * m; }

__global__ void __launch_bounds__(32) mx_spike_factor_kernel(DeviceState d)
{
   __shared__ float tips[kSpikeMaxSeg * 64];
   const int sp = blockIdx.x, lane = threadIdx.x;
   const int ich = d.sp_chain[sp];
   if (halted(d) || frozen_chain(d, ich)) return;
   const int P = d.sp_nseg[sp], row0 = d.chain_row0[ich], rec0 = d.sp_rec0[sp];
   bool bad = false;
   if (lane < P) {
      const int s = d.sp_seg[(kSpikeMaxSeg + 1) * sp + lane], e = d.sp_seg[(kSpikeMaxSeg + 1) * sp + lane + 1] - 1;
      float cp[16], gw[16];
      for (int i = s; i <= e; i++) {
         float A[16], B[16], C[16];
         mx_row_ref(d, mx_rowref(d, row0 + i), A, B, C);
         float* rec = d.sp_fac + (size_t)kSpRec * (rec0 + i);
         st16f(rec, A);
         if (i > s) mm_sub(A, cp, B);
         const LUf u = luf_factor(B);
         luf_store(rec + 16, u);
         bad |= nonfinite(u.p0) || nonfinite(u.p1) || nonfinite(u.p2) || nonfinite(u.p3);
         // left spike, forward: g_s = B'^{-1}(-A_s), g_i = B'^{-1}(-A_i g_{i-1})
         float w[16];
         if (i == s) {
#pragma unroll
            for (int m = 0; m < 16; m++) w[m] = -A[m];
         } else {
#pragma unroll
            for (int m = 0; m < 16; m++) w[m] = 0.f;
            mm_sub(A, gw, w);
         }
         luf_cols(u, w);
         st16f(rec + 64, w);
#pragma unroll
         for (int m = 0; m < 16; m++) gw[m] = w[m];
         if (i < e) {
            luf_cols(u, C);
            st16f(rec + 32, C);
#pragma unroll
            for (int m = 0; m < 16; m++) cp[m] = C[m];
         } else {
            // right spike at the last row: B'^{-1}(-C_e)
#pragma unroll
            for (int m = 0; m < 16; m++) C[m] = -C[m];
            luf_cols(u, C);
            st16f(rec + 48, C);
         }
      }
      // back substitution of both spikes: V_i = -C'_i V_{i+1},
      // W_i = g_i - C'_i W_{i+1}
      float vn[16], wn[16];
      ld16f(d.sp_fac + (size_t)kSpRec * (rec0 + e) + 48, vn);
      ld16f(d.sp_fac + (size_t)kSpRec * (rec0 + e) + 64, wn);
      float* tip = tips + 64 * lane;
      st16f(tip + 32, vn);      // V_e
      st16f(tip + 48, wn);      // W_e
      for (int i = e - 1; i >= s; i--) {
         float* rec = d.sp_fac + (size_t)kSpRec * (rec0 + i);
         float c[16], v[16], w[16];
         ld16f(rec + 32, c);
         ld16f(rec + 64, w);
#pragma unroll
         for (int m = 0; m < 16; m++) v[m] = 0.f;
         mm_sub(c, vn, v);
         mm_sub(c, wn, w);
         st16f(rec + 48, v);
         st16f(rec + 64, w);
#pragma unroll
         for (int m = 0; m < 16; m++) { vn[m] = v[m]; wn[m] = w[m]; }
      }
      st16f(tip, vn);           // V_s
      st16f(tip + 16, wn);      // W_s
   }
   if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(d.status, DEV_ERR_PIVOT);
   __syncwarp();
   if (lane != 0) return;
   // boundary system: M_0 = D_0, M_p = D_p - L_p G_{p-1}; G_p = M_p^{-1} U_p;
   // H_0 = M_0^{-1} L_0, H_p = -M_p^{-1} L_p H_{p-1}; at p = P-2 the
   // coupling U_{P-2} goes to Z_{P-1} itself
   float* red = d.sp_red + (size_t)kSpikeRedStride * sp;
   float L[64], D[64], U[64], G[64], H[64], T[64];
   for (int p = 0; p <= P - 2; p++) {
      red_blocks(tips, p, P, L, D, U);
      if (p > 0) m8_msub(D, L, G, true);                   // M_p = D_p - L_p G_{p-1}
      m8_lu(D);
      stm8(red_row(red, p, 0), D);
      stm8(red_row(red, p, 1), L);
      for (int j = 0; j < 8; j++) m8_solve(D, U + j, 8);   // G_p = M_p^{-1} U_p
      if (p == 0) {
         for (int e = 0; e < 64; e++) H[e] = L[e];
      } else {
         m8_msub(T, L, H, false);                            // T = -L_p H_{p-1}
         for (int e = 0; e < 64; e++) H[e] = T[e];
      }
      for (int j = 0; j < 8; j++) m8_solve(D, H + j, 8);
      for (int e = 0; e < 64; e++) G[e] = U[e];
      stm8(red_row(red, p, 2), G);
      stm8(red_row(red, p, 3), H);                           // H_p, turned into B_p below
   }
   // Z_p = a_p + B_p Z_{P-1}: B_{P-2} = -(G_{P-2} + H_{P-2}),
   // B_p = -G_p B_{p+1} - H_p
   float Bn[64];
   ldm8(red_row(red, P - 2, 3), H);
   for (int e = 0; e < 64; e++) Bn[e] = -(G[e] + H[e]);
   stm8(red_row(red, P - 2, 3), Bn);
   float B0[64];
   for (int e = 0; e < 64; e++) B0[e] = Bn[e];
   for (int p = P - 3; p >= 0; p--) {
      ldm8(red_row(red, p, 2), G);
      ldm8(red_row(red, p, 3), H);
      for (int e = 0; e < 64; e++) T[e] = -H[e];
      m8_msub(T, G, Bn, true);
      stm8(red_row(red, p, 3), T);
      for (int e = 0; e < 64; e++) Bn[e] = T[e];
      if (p == 0)
         for (int e = 0; e < 64; e++) B0[e] = T[e];
   }
   // K = D_{P-1} + L_{P-1} B_{P-2} + U_{P-1} B_0
   red_blocks(tips, P - 1, P, L, D, U);
   ldm8(red_row(red, P - 2, 3), Bn);
   for (int e = 0; e < 64; e++) { L[e] = -L[e]; U[e] = -U[e]; }
   m8_msub(D, L, Bn, true);
   m8_msub(D, U, B0, true);
   for (int e = 0; e < 64; e++) { L[e] = -L[e]; U[e] = -U[e]; }
   m8_lu(D);
   float* last = red + 256 * (kSpikeMaxSeg - 1);
   stm8(last, D);
   stm8(last + 64, L);
   stm8(last + 128, U);
   bool kbad = false;
   for (int k = 0; k < 8; k++) kbad |= nonfinite(D[9 * k]);
   if (kbad) atomicOr(d.status, DEV_ERR_PIVOT);
}

// one sweep's solve of the spike chains sp = first .. first+count-1 of a
// wave: right-hand sides r32[fcell], solutions into r32[scell]
__global__ void __launch_bounds__(32) mx_spike_solve_kernel(DeviceState d, int first)
{
   __shared__ float ry[kSpikeMaxSeg * 8];   // per segment: y_s then y_e
   __shared__ float zs[kSpikeMaxSeg * 8];   // Z_p = (b_p, t_{p+1})
   const int sp = first + blockIdx.x, lane = threadIdx.x;
   const int ich = d.sp_chain[sp];
   if (halted(d) || frozen_chain(d, ich)) return;
   const int P = d.sp_nseg[sp], row0 = d.chain_row0[ich], rec0 = d.sp_rec0[sp];
   int s = 0, e = -1;
   if (lane < P) {
      s = d.sp_seg[(kSpikeMaxSeg + 1) * sp + lane];
      e = d.sp_seg[(kSpikeMaxSeg + 1) * sp + lane + 1] - 1;
      // y' forward: y'_i = B'^{-1}(f_i - A_i y'_{i-1})
      float yp[4] = {0.f, 0.f, 0.f, 0.f};
      for (int i = s; i <= e; i++) {
         const float* rec = d.sp_fac + (size_t)kSpRec * (rec0 + i);
         const int fc = d.row_fcell[row0 + i];
         float x[4] = {0.f, 0.f, 0.f, 0.f};
         if (fc >= 0) ld4(d.r32 + 4 * (size_t)fc, x);
         if (i > s) {
            float a[16];
            ld16f(rec, a);
#pragma unroll
            for (int k = 0; k < 4; k++)
#pragma unroll
               for (int j = 0; j < 4; j++) x[k] = __fmaf_rn(-a[4 * k + j], yp[j], x[k]);
         }
         luf_solve(luf_load(rec + 16), x[0], x[1], x[2], x[3]);
         st4(d.sp_y + 4 * (size_t)(rec0 + i), x);
#pragma unroll
         for (int k = 0; k < 4; k++) yp[k] = x[k];
      }
      // back: y_i = y'_i - C'_i y_{i+1}
#pragma unroll
      for (int k = 0; k < 4; k++) ry[8 * lane + 4 + k] = yp[k];
      for (int i = e - 1; i >= s; i--) {
         const float* rec = d.sp_fac + (size_t)kSpRec * (rec0 + i);
         float c[16], x[4];
         ld16f(rec + 32, c);
         ld4(d.sp_y + 4 * (size_t)(rec0 + i), x);
#pragma unroll
         for (int k = 0; k < 4; k++)
#pragma unroll
            for (int j = 0; j < 4; j++) x[k] = __fmaf_rn(-c[4 * k + j], yp[j], x[k]);
         st4(d.sp_y + 4 * (size_t)(rec0 + i), x);
#pragma unroll
         for (int k = 0; k < 4; k++) yp[k] = x[k];
      }
#pragma unroll
      for (int k = 0; k < 4; k++) ry[8 * lane + k] = yp[k];
   }
   __syncwarp();
   if (lane == 0) {
      // R_p = (y_e(p), y_s(p+1)); g_p = M_p^{-1}(R_p - L_p g_{p-1});
      // a_{P-2} = g_{P-2}, a_p = g_p - G_p a_{p+1};
      // Z_{P-1} = K^{-1}(R_{P-1} - L_{P-1} a_{P-2} - U_{P-1} a_0);
      // Z_p = a_p + B_p Z_{P-1}
      const float* red = d.sp_red + (size_t)kSpikeRedStride * sp;
      float M[64], g[8];
      for (int p = 0; p <= P - 2; p++) {
         for (int k = 0; k < 4; k++) {
            g[k] = ry[8 * p + 4 + k];
            g[4 + k] = ry[8 * (p + 1) + k];
         }
         if (p > 0) {
            float prev[8];
            for (int k = 0; k < 8; k++) prev[k] = zs[8 * (p - 1) + k];
            ldm8(red_row(red, p, 1), M);
            v8_msub(g, M, prev);
         }
         ldm8(red_row(red, p, 0), M);
         m8_solve(M, g, 1);
         for (int k = 0; k < 8; k++) zs[8 * p + k] = g[k];
      }
      for (int p = P - 3; p >= 0; p--) {
         float nx[8];
         for (int k = 0; k < 8; k++) { g[k] = zs[8 * p + k]; nx[k] = zs[8 * (p + 1) + k]; }
         ldm8(red_row(red, p, 2), M);
         v8_msub(g, M, nx);
         for (int k = 0; k < 8; k++) zs[8 * p + k] = g[k];
      }
      const float* last = red + 256 * (kSpikeMaxSeg - 1);
      float z[8], a0[8], ap[8];
      for (int k = 0; k < 4; k++) {
         z[k] = ry[8 * (P - 1) + 4 + k];
         z[4 + k] = ry[k];
      }
      for (int k = 0; k < 8; k++) { ap[k] = zs[8 * (P - 2) + k]; a0[k] = zs[k]; }
      ldm8(last + 64, M);
      v8_msub(z, M, ap);
      ldm8(last + 128, M);
      v8_msub(z, M, a0);
      ldm8(last, M);
      m8_solve(M, z, 1);
      for (int p = 0; p <= P - 2; p++) {
         for (int k = 0; k < 8; k++) g[k] = zs[8 * p + k];
         ldm8(red_row(red, p, 3), M);
         for (int i = 0; i < 8; i++) {
            float v = g[i];
            for (int k = 0; k < 8; k++) v = __fmaf_rn(M[8 * i + k], z[k], v);
            g[i] = v;
         }
         for (int k = 0; k < 8; k++) zs[8 * p + k] = g[k];
      }
      for (int k = 0; k < 8; k++) zs[8 * (P - 1) + k] = z[k];
   }
   __syncwarp();
   if (lane < P) {
      // x_i = y_i + V_i t_{p+1} + W_i b_{p-1}
      float tn[4], bp[4];
      const int pm = (lane == 0) ? P - 1 : lane - 1;
#pragma unroll
      for (int k = 0; k < 4; k++) {
         tn[k] = zs[8 * lane + 4 + k];
         bp[k] = zs[8 * pm + k];
      }
      for (int i = s; i <= e; i++) {
         const float* rec = d.sp_fac + (size_t)kSpRec * (rec0 + i);
         float v[16], w[16], x[4];
         ld16f(rec + 48, v);
         ld16f(rec + 64, w);
         ld4(d.sp_y + 4 * (size_t)(rec0 + i), x);
#pragma unroll
         for (int k = 0; k < 4; k++)
#pragma unroll
            for (int j = 0; j < 4; j++) x[k] = __fmaf_rn(v[4 * k + j], tn[j], __fmaf_rn(w[4 * k + j], bp[j], x[k]));
         st4(d.r32 + 4 * (size_t)d.row_scell[row0 + i], x);
      }
   }
}

__global__ void __launch_bounds__(kThreads) mx_dq_update_kernel(DeviceState d)
{
   const int c = blockIdx.x * blockDim.x + threadIdx.x;
   if (c >= d.nCell || halted(d) || frozen_cell(d, c)) return;
   float r[4], dq[4];
   ld4(d.r32 + 4 * (size_t)c, r);
   ld4(d.dq32 + 4 * (size_t)c, dq);
#pragma unroll
   for (int k = 0; k < 4; k++) dq[k] += r[k];
   st4(d.dq32 + 4 * (size_t)c, dq);
   if (nonfinite(dq[0]) || nonfinite(dq[1]) || nonfinite(dq[2]) || nonfinite(dq[3])) atomicOr(d.status, DEV_ERR_DQ);
}

template <int ORDER>
__global__ void __launch_bounds__(kThreads) mx_lin_face_kernel(DeviceState d)
{
   // the block's face Jacobians staged through shared memory: read with
   // whole-line loads (8 float4 per slot, consecutive slots), then each
   // thread takes its own (row stride 9 float4: no bank conflicts)
   __shared__ float4 sj[kThreads * 9];
   const int nb = blockDim.x, s0 = blockIdx.x * nb, s = s0 + threadIdx.x;
   const int nloc = min(nb, d.nSlot - s0);
   const float4* __restrict__ src = reinterpret_cast<const float4*>(d.ff32 + 32 * (size_t)s0);
   for (int c = threadIdx.x; c < 8 * nloc; c += nb) sj[(c >> 3) * 9 + (c & 7)] = src[c];
   __syncthreads();
   if (s >= d.nSlot || halted(d) || frozen_slot(d, s)) return;
   const int4 sl = d.slot[s];
   float dL[4], dR[4];
   face_dstates<ORDER, float>(d, d.dq32, sl.x, (sl.w & 1) != 0, dL, dR);
   // the Jacobian kept for this face is its owner slot's (a periodic
   // chain's repeated face); almost always the slot itself
   const int own = sl.w >> 1;
   float m[32];
#pragma unroll
   for (int q = 0; q < 8; q++) {
      const float4 v = (own == s) ? sj[threadIdx.x * 9 + q]
                                  : reinterpret_cast<const float4*>(d.ff32 + 32 * (size_t)own)[q];
      m[4 * q] = v.x;
      m[4 * q + 1] = v.y;
      m[4 * q + 2] = v.z;
      m[4 * q + 3] = v.w;
   }
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
   const int c = norm_cell(d);
   double sq = 0.0, am = 0.0;
   if (c >= 0) {
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

namespace {
template <bool SD>
void mx_rhs_face_go(const DeviceState& d, int b, int t, cudaStream_t st)
{
   switch (d.recon) {
      case 1: mx_rhs_face_kernel<1, SD><<<b, t, 0, st>>>(d); break;
      case 3: mx_rhs_face_kernel<3, SD><<<b, t, 0, st>>>(d); break;
      case 5:
         if (d.qface) mx_rhs_face_kernel<5, SD, true><<<b, t, 0, st>>>(d);
         else mx_rhs_face_kernel<5, SD><<<b, t, 0, st>>>(d);
         break;
      case 31: mx_rhs_face_kernel<31, SD><<<b, t, 0, st>>>(d); break;
      default: mx_rhs_face_kernel<32, SD><<<b, t, 0, st>>>(d); break;
   }
}
}  // namespace

void launch_mx_rhs_face(const DeviceState& d, cudaStream_t st)
{
   const int t = d.face_block;
   const int b = (d.nSlot + t - 1) / t;
   if (d.face_soft) mx_rhs_face_go<true>(d, b, t, st);
   else mx_rhs_face_go<false>(d, b, t, st);
}

void launch_mx_assemble(const DeviceState& d, cudaStream_t st)
{
   const size_t n = 48 * 32 * (size_t)d.tile_rows;
   if (!d.mx_fused && n > 0) mx_assemble_kernel<<<(unsigned)((n + kThreads - 1) / kThreads), kThreads, 0, st>>>(d);
}

void launch_mx_init(const DeviceState& d, cudaStream_t st) { mx_init_kernel<<<blocks_for(d.nCell), kThreads, 0, st>>>(d); }

void launch_mx_factor(const DeviceState& d, cudaStream_t st)
{
   const int tb = d.mx_block;
   const unsigned nb = (d.nChain + tb - 1) / tb;
   const bool chunk = d.nChain <= d.mx_chunk_chains;
   if (d.mx_fused) {
      if (chunk) mx_factor_kernel<true, kElimChunk><<<nb, tb, 0, st>>>(d, d.nChain);
      else mx_factor_kernel<true, 1><<<nb, tb, 0, st>>>(d, d.nChain);
   } else {
      if (chunk) mx_factor_kernel<false, kElimChunk><<<nb, tb, 0, st>>>(d, d.nChain);
      else mx_factor_kernel<false, 1><<<nb, tb, 0, st>>>(d, d.nChain);
   }
}

void launch_mx_solve(const DeviceState& d, int first, int count, cudaStream_t st)
{
   const int tb = d.mx_block;
   if (count <= 0) return;
   if (count <= d.mx_chunk_chains) mx_solve_chunk_kernel<<<(count + tb - 1) / tb, tb, 0, st>>>(d, first, count);
   else mx_solve_kernel<<<(count + tb - 1) / tb, tb, 0, st>>>(d, first, count);
}

int mx_solve_chunk_capacity(int block)
{
   int dev = 0, sms = 0, per_sm = 0;
   if (cudaGetDevice(&dev) != cudaSuccess) return 0;
   if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
   if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mx_solve_chunk_kernel, block, 0) != cudaSuccess)
      return 0;
   return sms * per_sm * block;
}

void launch_mx_spike_factor(const DeviceState& d, cudaStream_t st)
{
   if (d.sp_on && d.nSpike > 0) mx_spike_factor_kernel<<<d.nSpike, 32, 0, st>>>(d);
}

void launch_mx_spike_solve(const DeviceState& d, int first, int count, cudaStream_t st)
{
   if (d.sp_on && count > 0) mx_spike_solve_kernel<<<count, 32, 0, st>>>(d, first);
}

void launch_mx_dq_update(const DeviceState& d, cudaStream_t st)
{
   mx_dq_update_kernel<<<blocks_for(d.nCell), kThreads, 0, st>>>(d);
}

void launch_mx_lin_face(const DeviceState& d, cudaStream_t st)
{
   const int kThreads = d.face_block;
   const int b = (d.nSlot + kThreads - 1) / kThreads;
   if (d.lin_order == 1) {
      mx_lin_face_kernel<1><<<b, kThreads, 0, st>>>(d);
      return;
   }
   switch (d.recon) {
      case 1: mx_lin_face_kernel<1><<<b, kThreads, 0, st>>>(d); break;
      case 3: mx_lin_face_kernel<3><<<b, kThreads, 0, st>>>(d); break;
      case 5: mx_lin_face_kernel<5><<<b, kThreads, 0, st>>>(d); break;
      case 31: mx_lin_face_kernel<31><<<b, kThreads, 0, st>>>(d); break;
      default: mx_lin_face_kernel<32><<<b, kThreads, 0, st>>>(d); break;
   }
}

void launch_mx_lin_cell(const DeviceState& d, bool update_q, cudaStream_t st)
{
   if (update_q) mx_lin_cell_kernel<true><<<d.norm_blocks, kThreads, 0, st>>>(d);
   else mx_lin_cell_kernel<false><<<d.norm_blocks, kThreads, 0, st>>>(d);
}

}  // namespace hamstr
