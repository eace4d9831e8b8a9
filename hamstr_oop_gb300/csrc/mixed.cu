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
   // one thread per tiled entry (DeviceState: blk32), in memory order, so
   // stores are whole lines: t = tix(srow, 48, e48, lane)
   const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
   if (t >= 48 * 32 * (size_t)d.tile_rows || halted(d)) return;
   const int lane = (int)((t >> 2) & 31);
   const size_t g = t >> 7;
   const int e48 = (int)(g % 12) * 4 + (int)(t & 3), srow = (int)(g / 12), b = e48 >> 4, e = e48 & 15;
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

// whether chain ich takes the segmented solve: sp_on 1 takes the long
// periodic chains, 2 the long open ones as well
__device__ __forceinline__ bool spike_active(const DeviceState& d, int ich)
{
   return d.sp_on && d.chain_spike[ich] >= 0 && (d.sp_on == 2 || d.chain_periodic[ich]);
}

// the tiled index of element e of tile row s in lane `lane` of a W-wide
// array (W a multiple of 4): each lane's elements 4k .. 4k+3 are one float4,
// and the 32 lanes' float4 of one group lie together, so a warp's access of
// one group is 512 contiguous bytes and takes one instruction per lane
__device__ __forceinline__ size_t tix(int s, int W, int e, int lane)
{
   return (((size_t)s * W + (e & ~3)) << 5) + 4 * lane + (e & 3);
}

// 16 consecutive elements of a tiled record (4 float4, 128 floats apart: each load of
// a warp is one 128-byte line)
__device__ __forceinline__ void ld16t(const float* __restrict__ p, float (&v)[16])
{
#pragma unroll
   for (int q = 0; q < 4; q++) {
      const float4 x = *reinterpret_cast<const float4*>(p + 128 * q);
      v[4 * q] = x.x; v[4 * q + 1] = x.y; v[4 * q + 2] = x.z; v[4 * q + 3] = x.w;
   }
}

__device__ __forceinline__ void st16t(float* __restrict__ p, const float (&v)[16])
{
#pragma unroll
   for (int q = 0; q < 4; q++)
      *reinterpret_cast<float4*>(p + 128 * q) = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
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

// the LU record of a tiled row
__device__ __forceinline__ void luf_store_t(float* p, const LUf& u)
{
   const float v[16] = {u.p0, u.u01, u.u02, u.u03, u.l10, u.p1, u.u12, u.u13,
                        u.l20, u.l21, u.p2, u.u23, u.l30, u.l31, u.l32, u.p3};
   st16t(p, v);
}

__device__ __forceinline__ LUf luf_load_t(const float* p)
{
   float v[16];
   ld16t(p, v);
   LUf u;
   u.p0 = v[0]; u.u01 = v[1]; u.u02 = v[2]; u.u03 = v[3]; u.l10 = v[4]; u.p1 = v[5]; u.u12 = v[6]; u.u13 = v[7];
   u.l20 = v[8]; u.l21 = v[9]; u.p2 = v[10]; u.u23 = v[11]; u.l30 = v[12]; u.l31 = v[13]; u.l32 = v[14]; u.p3 = v[15];
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

// ---- fused assembly with the next row's terms staged in shared memory ----
// Each of a row's up to 3 x kOpsPerBlock face-Jacobian terms is a 64-byte
// block of ff32.  Summing them as they arrive makes the row wait on one
// round trip per term; instead the terms of row i+1 are copied into shared
// memory with asynchronous copies (cp.async, 16 bytes each) while row i is
// factored, and summed, in the same order as mx_block, after it.  Layout:
// float4 q of term t of thread `tid` at ((t * 4 + q) * blockDim + tid), so
// a warp's copies and reads of one float4 are one 512-byte span.
constexpr int kStageTerms = 3 * kOpsPerBlock;

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
   const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
   asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

__device__ __forceinline__ float4* stage_at(float4* stage, int term, int q)
{
   return stage + (size_t)(term * 4 + q) * blockDim.x + threadIdx.x;
}

// issue the copies of row r's terms (terms with op < 0 copy nothing)
__device__ __forceinline__ void mx_stage_row(const DeviceState& d, const RowRef& r, float4* stage)
{
   const int ops[kStageTerms] = {r.ops[0].x, r.ops[0].y, r.ops[0].z, r.ops[0].w, r.ops[1].x, r.ops[1].y,
                                 r.ops[1].z, r.ops[1].w, r.ops[2].x, r.ops[2].y, r.ops[2].z, r.ops[2].w};
#pragma unroll
   for (int t = 0; t < kStageTerms; t++) {
      const int op = ops[t];
      if (op < 0) continue;
      const float* src = d.ff32 + 32 * (size_t)(op >> 3) + (((op >> 1) & 3) == OP_SEL_L ? 0 : 16);
#pragma unroll
      for (int q = 0; q < 4; q++) cp_async16(stage_at(stage, t, q), src + 4 * q);
   }
   cp_async_commit();
}

// mx_block from the staged terms of block b (0, 1, 2 = A, B, C)
__device__ __forceinline__ void mx_block_staged(const DeviceState& d, const int (&ops)[kOpsPerBlock], int b,
                                                const float4* stage, float (&M)[16])
{
#pragma unroll
   for (int m = 0; m < 16; m++) M[m] = 0.f;
#pragma unroll
   for (int o = 0; o < kOpsPerBlock; o++) {
      const int op = ops[o];
      if (op < 0) break;
      float v[16];
#pragma unroll
      for (int q = 0; q < 4; q++) {
         const float4 x = *stage_at(const_cast<float4*>(stage), b * kOpsPerBlock + o, q);
         v[4 * q] = x.x; v[4 * q + 1] = x.y; v[4 * q + 2] = x.z; v[4 * q + 3] = x.w;
      }
      if (((op >> 1) & 3) == OP_SEL_RREFL) {
         const double4 rf = d.refl[d.slot_face[op >> 3]];
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

// mx_row_ref from staged terms and the row's CFL/sigma factor s
__device__ __forceinline__ void mx_row_staged(const DeviceState& d, const RowRef& r, const float4* stage, float s,
                                              float (&A)[16], float (&B)[16], float (&C)[16])
{
   const int oa[4] = {r.ops[0].x, r.ops[0].y, r.ops[0].z, r.ops[0].w};
   const int ob[4] = {r.ops[1].x, r.ops[1].y, r.ops[1].z, r.ops[1].w};
   const int oc[4] = {r.ops[2].x, r.ops[2].y, r.ops[2].z, r.ops[2].w};
   mx_block_staged(d, oa, 0, stage, A);
   mx_block_staged(d, ob, 1, stage, B);
   mx_block_staged(d, oc, 2, stage, C);
#pragma unroll
   for (int m = 0; m < 16; m++) {
      A[m] *= s;
      B[m] *= s;
      C[m] *= s;
   }
#pragma unroll
   for (int k = 0; k < 4; k++) B[5 * k] += 1.f;
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
   if (frozen_chain(d, ich) || spike_active(d, ich)) return;
   const int N = d.chain_nrows[ich], row0 = d.chain_row0[ich], lane = t & 31, s0 = d.grp_row0[t >> 5];
   const bool per = d.chain_periodic[ich] != 0;
   float A[16], B[16], C[16], cp[16], ap[16];
   bool bad = false;   // a reciprocal pivot is not finite (DEV_ERR_PIVOT)
   RowRef rnext{};   // fused: references of row i + 1, looked up a row ahead
   RowRef rstaged{};  // fused: references of the row whose terms are staged
   float snext = 0.f;  // fused: its CFL/sigma factor
   extern __shared__ float4 stage[];   // fused: kStageTerms x 4 float4 per thread
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
         if (FUSED) {
            // row i+1's terms are copied while row i is factored
            mx_stage_row(d, rnext, stage);
            rstaged = rnext;
            snext = float(d.dtfac[rnext.scell]);
            if (i + 2 < N) rnext = mx_rowref(d, row0 + i + 2);
         } else {
            mx_rows<FUSED>(d, rnext, s0 + i + 1, lane, An, Bn, Cn);
         }
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
         if (FUSED) {
            cp_async_wait_all();
            mx_row_staged(d, rstaged, stage, snext, A, B, C);
         } else {
#pragma unroll
            for (int m = 0; m < 16; m++) { A[m] = An[m]; B[m] = Bn[m]; C[m] = Cn[m]; }
         }
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
   if (frozen_chain(d, ich) || spike_active(d, ich)) return;
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
      *reinterpret_cast<float4*>(fs) = make_float4(x[0], x[1], x[2], x[3]);
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
         { const float4 y = *reinterpret_cast<const float4*>(fs); f[0] = y.x; f[1] = y.y; f[2] = y.z; f[3] = y.w; }
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
         { const float4 y = *reinterpret_cast<const float4*>(fs); x[0] = y.x; x[1] = y.y; x[2] = y.z; x[3] = y.w; }
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
         { const float4 y = *reinterpret_cast<const float4*>(fs); x[0] = y.x; x[1] = y.y; x[2] = y.z; x[3] = y.w; }
         sc = scell[N - 2];
      }
      for (int i = N - 2; i >= 0; i--) {
         float cn[16], xnx[4];
         int scn = 0;
         if (i >= 1) {
            ld16t(d.fac32 + tix(s0 + i - 1, kRec, 32, lane), cn);
            const float* fs = d.fsc32 + tix(s0 + i - 1, 4, 0, lane);
            { const float4 y = *reinterpret_cast<const float4*>(fs); xnx[0] = y.x; xnx[1] = y.y; xnx[2] = y.z; xnx[3] = y.w; }
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
   if (frozen_chain(d, ich) || spike_active(d, ich)) return;
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
            *reinterpret_cast<float4*>(fs) = make_float4(x[0], x[1], x[2], x[3]);
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
               { const float4 y = *reinterpret_cast<const float4*>(fs); fb[u][0] = y.x; fb[u][1] = y.y; fb[u][2] = y.z; fb[u][3] = y.w; }
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
               { const float4 y = *reinterpret_cast<const float4*>(fs); fb[u][0] = y.x; fb[u][1] = y.y; fb[u][2] = y.z; fb[u][3] = y.w; }
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
               { const float4 y = *reinterpret_cast<const float4*>(fs); fb[u][0] = y.x; fb[u][1] = y.y; fb[u][2] = y.z; fb[u][3] = y.w; }
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

// ---------------- long chains by segments -------------------------------
// A periodic chain of N rows (A_i x_{i-1} + B_i x_i + C_i x_{i+1} = f_i,
// indices mod N) is cut into P segments of about N/P rows, one lane of a
// warp each.  An open chain is the same system with A_0 and C_{N-1} (which
// its solve never reads) set to zero: its first segment's W and its last
// segment's V spikes vanish, and the cyclic boundary system below has zero
// coupling across the wrap.  With D_p the block-tridiagonal matrix of segment p alone
// (rows s..e), its solution is
//     x_i = y_i + V_i x_{e+1} + W_i x_{s-1},
// where D_p y = f, D_p V = -C_e (in the last row) and D_p W = -A_s (in the
// first row): V and W are the "spikes", the segment's responses to the
// couplings across its two ends.  With b_p = x_e and t_p = x_s of segment
// p, the rows at the segment ends give a cyclic system in the interface
// pairs Z_p = (b_p, t_{p+1}):
//     b_p     - V_e(p) t_{p+1} - W_e(p) b_{p-1}   = y_e(p)
//     t_{p+1} - V_s(p+1) t_{p+2} - W_s(p+1) b_p   = y_s(p+1)
// i.e. L_p Z_{p-1} + D_p Z_p + U_p Z_{p+1} = R_p with 8x8 blocks
//     D_p = [I, -V_e(p); -W_s(p+1), I],  L_p = [-W_e(p), 0; 0, 0],
//     U_p = [0, 0; 0, -V_s(p+1)],
// which lane 0 eliminates onto Z_{P-1} (a cyclic block Thomas of P rows).
// Their sparsity keeps every step in 4x4 blocks: the pivot blocks are
// M_p = [I, X_p; -W_s(p+1), I] and are solved through the 4x4 Schur
// complement S_p = I + W_s(p+1) X_p; the couplings G_p = M_p^{-1} U_p and
// H_p (to Z_{P-1}) have four non-zero columns each.  This is the same
// linear system the sequential cyclic block Thomas solves (in FP32 it
// differs in rounding only), with N/P + P rows of latency instead of N.
// The segment factors and spikes, and the boundary system's factors, are
// formed once per step; each sweep replays the right-hand side.
//
// Layout: the rows of a chain's segments are tiled like the other FP32 line
// data (element e of local row k of segment p at tix(R0 + k, W, e, p), R0
// the chain's first tile row), so every load and store of the warp is one
// 128-byte line.

// sp_fac record of one row: A, LU of the segment's B', C' (no C' on a
// segment's last row), V, W
constexpr int kSpRec = 80;

// sp_red layout of one chain: for p = 0 .. P-2, at kRedRow * p: X_p, LU(S_p),
// G_p (top 4 rows, bottom 4 rows; its non-zero columns 4-7), H_p (top,
// bottom; columns 0-3), W_e(p), W_s(p+1); then at kRedLast: LU(K) (8x8),
// W_e(P-1), V_s(0)
constexpr int kRedRow = 128;
constexpr int kRedLast = kRedRow * (kSpikeMaxSeg - 1);
static_assert(kRedLast + 64 + 32 <= kSpikeRedStride, "boundary-system factors fit their stride");
enum { RX = 0, RS = 16, RGT = 32, RGB = 48, RHT = 64, RHB = 80, RWE = 96, RWS = 112 };

// y -= M x (4x4, 4-vector)
__device__ __forceinline__ void mv_sub(const float (&M)[16], const float (&x)[4], float (&y)[4])
{
#pragma unroll
   for (int k = 0; k < 4; k++)
#pragma unroll
      for (int j = 0; j < 4; j++) y[k] = __fmaf_rn(-M[4 * k + j], x[j], y[k]);
}

__device__ __forceinline__ void mv_add(const float (&M)[16], const float (&x)[4], float (&y)[4])
{
#pragma unroll
   for (int k = 0; k < 4; k++)
#pragma unroll
      for (int j = 0; j < 4; j++) y[k] = __fmaf_rn(M[4 * k + j], x[j], y[k]);
}

// out = M X (4x4)
__device__ __forceinline__ void mm_mul(const float (&M)[16], const float (&X)[16], float (&out)[16])
{
#pragma unroll
   for (int m = 0; m < 16; m++) out[m] = 0.f;
   mm_sub(M, X, out);
#pragma unroll
   for (int m = 0; m < 16; m++) out[m] = -out[m];
}

__device__ __forceinline__ void ld16s(const float* p, float (&v)[16])
{
#pragma unroll
   for (int m = 0; m < 16; m++) v[m] = p[m];
}

__device__ __forceinline__ void st16s(float* p, const float (&v)[16])
{
#pragma unroll
   for (int m = 0; m < 16; m++) p[m] = v[m];
}

// 8x8 row-major LU with reciprocal pivots (K, once per chain and step):
// M = L U, U unit upper; L below and on the diagonal (the diagonal holding
// 1/L_kk)
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

// x <- M^{-1} x with the LU of m8_lu
__device__ void m8_solve(const float* LU, float (&x)[8])
{
   for (int i = 0; i < 8; i++) {
      float v = x[i];
      for (int k = 0; k < i; k++) v = __fmaf_rn(-LU[8 * i + k], x[k], v);
      x[i] = v * LU[9 * i];
   }
   for (int i = 6; i >= 0; i--) {
      float v = x[i];
      for (int j = i + 1; j < 8; j++) v = __fmaf_rn(-LU[8 * i + j], x[j], v);
      x[i] = v;
   }
}

// M [u; v] = [f; h] with M = [I, X; -Ws, I] and the LU of S = I + Ws X:
// v = S^{-1}(h + Ws f), u = f - X v, for the four columns of F and Hh
// (Hh = nullptr for h = 0)
__device__ __forceinline__ void schur_cols(const float (&X)[16], const LUf& s, const float (&Ws)[16],
                                           const float (&F)[16], const float* Hh, float (&U)[16], float (&Vv)[16])
{
#pragma unroll
   for (int m = 0; m < 16; m++) Vv[m] = Hh ? Hh[m] : 0.f;
   float WF[16];
   mm_mul(Ws, F, WF);
#pragma unroll
   for (int m = 0; m < 16; m++) Vv[m] += WF[m];
   luf_cols(s, Vv);
#pragma unroll
   for (int m = 0; m < 16; m++) U[m] = F[m];
   mm_sub(X, Vv, U);
}

__global__ void __launch_bounds__(32) mx_spike_factor_kernel(DeviceState d)
{
   __shared__ __align__(16) float tips[kSpikeMaxSeg * 64];   // per segment: V_s, W_s, V_e, W_e
   const int sp = blockIdx.x, lane = threadIdx.x;
   const int ich = d.sp_chain[sp];
   if (halted(d) || frozen_chain(d, ich) || !spike_active(d, ich)) return;
   const int P = d.sp_nseg[sp], row0 = d.chain_row0[ich], R0 = d.sp_rec0[sp];
   const bool per = d.chain_periodic[ich] != 0;
   const int* seg = d.sp_seg + (kSpikeMaxSeg + 1) * sp;
   bool bad = false;
   if (lane < P) {
      const int s = seg[lane], n = seg[lane + 1] - s;   // n >= 2
      // forward: B'_k = B_k - A_k C'_{k-1}; C'_k = B'^{-1} C_k; the left
      // spike's forward values g_0 = B'^{-1}(-A_0), g_k = B'^{-1}(-A_k g_{k-1});
      // at the last row the right spike B'^{-1}(-C_e).  The next row's blocks
      // are assembled from references looked up a row earlier.
      float A[16], B[16], C[16], cp[16], gw[16];
      RowRef rnext = mx_rowref(d, row0 + s + 1);
      mx_row_ref(d, mx_rowref(d, row0 + s), A, B, C);
      // an open chain: no coupling from its first row back to its last
      if (!per && lane == 0) {
#pragma unroll
         for (int m = 0; m < 16; m++) A[m] = 0.f;
      }
      for (int k = 0; k < n; k++) {
         float An[16], Bn[16], Cn[16];
         if (k + 1 < n) {
            mx_row_ref(d, rnext, An, Bn, Cn);
            if (k + 2 < n) rnext = mx_rowref(d, row0 + s + k + 2);
         }
         float* rec = d.sp_fac + tix(R0 + k, kSpRec, 0, lane);
         st16t(rec, A);
         float w[16];
         if (k == 0) {
#pragma unroll
            for (int m = 0; m < 16; m++) w[m] = -A[m];
         } else {
            mm_sub(A, cp, B);
#pragma unroll
            for (int m = 0; m < 16; m++) w[m] = 0.f;
            mm_sub(A, gw, w);
         }
         const LUf u = luf_factor(B);
         luf_store_t(rec + 32 * 16, u);
         bad |= nonfinite(u.p0) || nonfinite(u.p1) || nonfinite(u.p2) || nonfinite(u.p3);
         luf_cols(u, w);
         st16t(rec + 32 * 64, w);
#pragma unroll
         for (int m = 0; m < 16; m++) gw[m] = w[m];
         if (k + 1 < n) {
            luf_cols(u, C);
            st16t(rec + 32 * 32, C);
#pragma unroll
            for (int m = 0; m < 16; m++) { cp[m] = C[m]; A[m] = An[m]; B[m] = Bn[m]; C[m] = Cn[m]; }
         } else {
            // (an open chain's last row has no coupling forward to its first)
            const bool wrap = per || lane + 1 < P;
#pragma unroll
            for (int m = 0; m < 16; m++) C[m] = wrap ? -C[m] : 0.f;
            luf_cols(u, C);
            st16t(rec + 32 * 48, C);
         }
      }
      // back substitution of both spikes: V_k = -C'_k V_{k+1},
      // W_k = g_k - C'_k W_{k+1}; row k-1's C' and g are loaded while row k
      // is formed
      float vn[16], wn[16], c[16], g[16];
      ld16t(d.sp_fac + tix(R0 + n - 1, kSpRec, 48, lane), vn);
      ld16t(d.sp_fac + tix(R0 + n - 1, kSpRec, 64, lane), wn);
      float* tip = tips + 64 * lane;
      st16s(tip + 32, vn);   // V_e
      st16s(tip + 48, wn);   // W_e
      ld16t(d.sp_fac + tix(R0 + n - 2, kSpRec, 32, lane), c);
      ld16t(d.sp_fac + tix(R0 + n - 2, kSpRec, 64, lane), g);
      for (int k = n - 2; k >= 0; k--) {
         float cn[16], gn[16];
         if (k > 0) {
            ld16t(d.sp_fac + tix(R0 + k - 1, kSpRec, 32, lane), cn);
            ld16t(d.sp_fac + tix(R0 + k - 1, kSpRec, 64, lane), gn);
         }
         float v[16];
#pragma unroll
         for (int m = 0; m < 16; m++) v[m] = 0.f;
         mm_sub(c, vn, v);
         mm_sub(c, wn, g);
         float* rec = d.sp_fac + tix(R0 + k, kSpRec, 0, lane);
         st16t(rec + 32 * 48, v);
         st16t(rec + 32 * 64, g);
#pragma unroll
         for (int m = 0; m < 16; m++) { vn[m] = v[m]; wn[m] = g[m]; }
         if (k > 0) {
#pragma unroll
            for (int m = 0; m < 16; m++) { c[m] = cn[m]; g[m] = gn[m]; }
         }
      }
      st16s(tip, vn);        // V_s
      st16s(tip + 16, wn);   // W_s
   }
   if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(d.status, DEV_ERR_PIVOT);
   __syncwarp();
   if (lane != 0) return;
   // boundary system, p = 0 .. P-2 (q = p + 1):
   //   X_p = -V_e(p) + W_e(p) Gtop_{p-1}  (X_0 = -V_e(0)),  S_p = I + W_s(q) X_p,
   //   G_p = M_p^{-1} [0; -V_s(q)],
   //   H_0 = M_0^{-1} [-W_e(0); 0],  H_p = M_p^{-1} [W_e(p) Htop_{p-1}; 0]
   float* red = d.sp_red + (size_t)kSpikeRedStride * sp;
   float Gt[16], Ht[16], Gb[16], Hb[16];
   bool kbad = false;
   for (int p = 0; p <= P - 2; p++) {
      const int q = p + 1;
      float X[16], We[16], Ws[16], T[16];
      ld16s(tips + 64 * p + 32, X);
      ld16s(tips + 64 * p + 48, We);
      ld16s(tips + 64 * q + 16, Ws);
#pragma unroll
      for (int m = 0; m < 16; m++) X[m] = -X[m];
      if (p > 0) {
         mm_mul(We, Gt, T);
#pragma unroll
         for (int m = 0; m < 16; m++) X[m] += T[m];
      }
      float S[16];
      mm_mul(Ws, X, S);
#pragma unroll
      for (int k = 0; k < 4; k++) S[5 * k] += 1.f;
      const LUf su = luf_factor(S);
      kbad |= nonfinite(su.p0) || nonfinite(su.p1) || nonfinite(su.p2) || nonfinite(su.p3);
      float F[16], Hh[16];
      // G_p: f = 0, h = -V_s(q): v = S^{-1}(-V_s(q)), u = -X v
      ld16s(tips + 64 * q, Hh);
#pragma unroll
      for (int m = 0; m < 16; m++) { Hh[m] = -Hh[m]; F[m] = 0.f; }
      schur_cols(X, su, Ws, F, Hh, Gt, Gb);
      // H_p
      if (p == 0) {
#pragma unroll
         for (int m = 0; m < 16; m++) F[m] = -We[m];
      } else {
         mm_mul(We, Ht, F);
      }
      schur_cols(X, su, Ws, F, nullptr, Ht, Hb);
      float* rr = red + kRedRow * p;
      st16s(rr + RX, X);
      luf_store(rr + RS, su);
      st16s(rr + RGT, Gt);
      st16s(rr + RGB, Gb);
      st16s(rr + RHT, Ht);
      st16s(rr + RHB, Hb);
      st16s(rr + RWE, We);
      st16s(rr + RWS, Ws);
   }
   // Z_p = a_p + B_p Z_{P-1}; only the rows of B_{P-2} (top) and B_0
   // (bottom) enter K: B_{P-2} = -[H_{P-2} | G_{P-2}],
   // B_p = -G_p Bbot_{p+1} - [H_p | 0], carried on its bottom rows
   float Bl[16], Br[16];   // bottom rows of B_p: columns 0-3, 4-7
#pragma unroll
   for (int m = 0; m < 16; m++) { Bl[m] = -Hb[m]; Br[m] = -Gb[m]; }
   float BtopL[16], BtopR[16];   // top rows of B_{P-2}
#pragma unroll
   for (int m = 0; m < 16; m++) { BtopL[m] = -Ht[m]; BtopR[m] = -Gt[m]; }
   for (int p = P - 3; p >= 0; p--) {
      float g[16], h[16], nl[16], nr[16];
      ld16s(red + kRedRow * p + RGB, g);
      ld16s(red + kRedRow * p + RHB, h);
      mm_mul(g, Bl, nl);
      mm_mul(g, Br, nr);
#pragma unroll
      for (int m = 0; m < 16; m++) { Bl[m] = -nl[m] - h[m]; Br[m] = -nr[m]; }
   }
   // K = D_{P-1} + L_{P-1} B_{P-2} + U_{P-1} B_0:
   //   top rows    [I, -V_e(P-1)] - W_e(P-1) Btop_{P-2}
   //   bottom rows [-W_s(0), I]   - V_s(0) Bbot_0
   float K[64], We[16], Vs0[16], M4[16], t[16];
   ld16s(tips + 64 * (P - 1) + 48, We);
   ld16s(tips, Vs0);
   ld16s(tips + 64 * (P - 1) + 32, t);   // V_e(P-1)
   mm_mul(We, BtopL, M4);
#pragma unroll
   for (int k = 0; k < 4; k++)
#pragma unroll
      for (int j = 0; j < 4; j++) {
         K[8 * k + j] = ((k == j) ? 1.f : 0.f) - M4[4 * k + j];
      }
   mm_mul(We, BtopR, M4);
#pragma unroll
   for (int k = 0; k < 4; k++)
#pragma unroll
      for (int j = 0; j < 4; j++) K[8 * k + 4 + j] = -t[4 * k + j] - M4[4 * k + j];
   ld16s(tips + 16, t);   // W_s(0)
   mm_mul(Vs0, Bl, M4);
#pragma unroll
   for (int k = 0; k < 4; k++)
#pragma unroll
      for (int j = 0; j < 4; j++) K[8 * (4 + k) + j] = -t[4 * k + j] - M4[4 * k + j];
   mm_mul(Vs0, Br, M4);
#pragma unroll
   for (int k = 0; k < 4; k++)
#pragma unroll
      for (int j = 0; j < 4; j++) K[8 * (4 + k) + 4 + j] = ((k == j) ? 1.f : 0.f) - M4[4 * k + j];
   m8_lu(K);
   for (int k = 0; k < 8; k++) kbad |= nonfinite(K[9 * k]);
   float* last = red + kRedLast;
   for (int m = 0; m < 64; m++) last[m] = K[m];
   st16s(last + 64, We);
   st16s(last + 80, Vs0);
   if (kbad) atomicOr(d.status, DEV_ERR_PIVOT);
}

// one sweep's solve of the spike chains sp = first .. first+count-1 of a
// wave: right-hand sides r32[fcell], solutions into r32[scell]
__global__ void __launch_bounds__(32) mx_spike_solve_kernel(DeviceState d, int first)
{
   // (red_s is read with float4 loads: 16-byte aligned)
   __shared__ __align__(16) float red_s[kRedLast + 96];   // the chain's boundary-system factors
   __shared__ __align__(16) float ry[kSpikeMaxSeg * 8];   // per segment: y_s then y_e
   __shared__ __align__(16) float zs[kSpikeMaxSeg * 8];   // Z_p = (b_p, t_{p+1})
   const int sp = first + blockIdx.x, lane = threadIdx.x;
   const int ich = d.sp_chain[sp];
   if (halted(d) || frozen_chain(d, ich) || !spike_active(d, ich)) return;
   const int P = d.sp_nseg[sp], row0 = d.chain_row0[ich], R0 = d.sp_rec0[sp];
   const int* seg = d.sp_seg + (kSpikeMaxSeg + 1) * sp;
   {
      // the boundary-system factors into shared memory (lane 0 reads them
      // one step after another below)
      const float* red = d.sp_red + (size_t)kSpikeRedStride * sp;
      const int nrow = kRedRow * (P - 1);
      for (int m = lane; m < nrow; m += 32) red_s[m] = red[m];
      for (int m = lane; m < 96; m += 32) red_s[kRedLast + m] = red[kRedLast + m];
   }
   int s = 0, n = 0;
   if (lane < P) {
      s = seg[lane];
      n = seg[lane + 1] - s;
      const int* fcell = d.row_fcell + row0 + s;
      // forward: y'_k = B'^{-1}(f_k - A_k y'_{k-1}); row k+1's record and
      // right-hand side are loaded while row k is solved
      float a[16], yp[4] = {0.f, 0.f, 0.f, 0.f}, x[4] = {0.f, 0.f, 0.f, 0.f};
      LUf u = luf_load_t(d.sp_fac + tix(R0, kSpRec, 16, lane));
      {
         const int fc = fcell[0];
         if (fc >= 0) ld4(d.r32 + 4 * (size_t)fc, x);
      }
#pragma unroll
      for (int m = 0; m < 16; m++) a[m] = 0.f;
      for (int k = 0; k < n; k++) {
         float an[16], xn[4] = {0.f, 0.f, 0.f, 0.f};
         LUf un;
         if (k + 1 < n) {
            const float* rn = d.sp_fac + tix(R0 + k + 1, kSpRec, 0, lane);
            ld16t(rn, an);
            un = luf_load_t(rn + 32 * 16);
            const int fc = fcell[k + 1];
            if (fc >= 0) ld4(d.r32 + 4 * (size_t)fc, xn);
         }
         if (k > 0) mv_sub(a, yp, x);
         luf_solve(u, x[0], x[1], x[2], x[3]);
#pragma unroll
         for (int c = 0; c < 4; c++) {
            d.sp_y[tix(R0 + k, 4, c, lane)] = x[c];
            yp[c] = x[c];
         }
         if (k + 1 < n) {
#pragma unroll
            for (int m = 0; m < 16; m++) a[m] = an[m];
            u = un;
#pragma unroll
            for (int c = 0; c < 4; c++) x[c] = xn[c];
         }
      }
      // back: y_k = y'_k - C'_k y_{k+1}
#pragma unroll
      for (int c = 0; c < 4; c++) ry[8 * lane + 4 + c] = yp[c];
      float cm[16], yk[4];
      ld16t(d.sp_fac + tix(R0 + n - 2, kSpRec, 32, lane), cm);
#pragma unroll
      for (int c = 0; c < 4; c++) yk[c] = d.sp_y[tix(R0 + n - 2, 4, c, lane)];
      for (int k = n - 2; k >= 0; k--) {
         float cn[16], ykn[4];
         if (k > 0) {
            ld16t(d.sp_fac + tix(R0 + k - 1, kSpRec, 32, lane), cn);
#pragma unroll
            for (int c = 0; c < 4; c++) ykn[c] = d.sp_y[tix(R0 + k - 1, 4, c, lane)];
         }
         mv_sub(cm, yp, yk);
#pragma unroll
         for (int c = 0; c < 4; c++) {
            d.sp_y[tix(R0 + k, 4, c, lane)] = yk[c];
            yp[c] = yk[c];
         }
         if (k > 0) {
#pragma unroll
            for (int m = 0; m < 16; m++) cm[m] = cn[m];
#pragma unroll
            for (int c = 0; c < 4; c++) yk[c] = ykn[c];
         }
      }
#pragma unroll
      for (int c = 0; c < 4; c++) ry[8 * lane + c] = yp[c];
   }
   __syncwarp();
   if (lane == 0) {
      // R_p = (y_e(p), y_s(p+1));
      //   g_p: f = y_e(p) + W_e(p) gtop_{p-1}, h = y_s(p+1):
      //        v = S_p^{-1}(h + W_s(p+1) f), u = f - X_p v;
      //   a_{P-2} = g_{P-2}, a_p = g_p - G_p abot_{p+1};
      //   Z_{P-1} = K^{-1}(R_{P-1} + [W_e(P-1) atop_{P-2}; V_s(0) abot_0]);
      //   Z_{P-2} = g_{P-2} - G_{P-2} zbot - H_{P-2} ztop,
      //   Z_p = g_p - G_p Zbot_{p+1} - H_p ztop
      float gt[4] = {0.f, 0.f, 0.f, 0.f};
      for (int p = 0; p <= P - 2; p++) {
         const float* rr = red_s + kRedRow * p;
         float f[4], v[4], M[16];
#pragma unroll
         for (int c = 0; c < 4; c++) { f[c] = ry[8 * p + 4 + c]; v[c] = ry[8 * (p + 1) + c]; }
         if (p > 0) {
            ld16s(rr + RWE, M);
            mv_add(M, gt, f);
         }
         ld16s(rr + RWS, M);
         mv_add(M, f, v);
         const LUf su = luf_load(rr + RS);
         luf_solve(su, v[0], v[1], v[2], v[3]);
         ld16s(rr + RX, M);
         mv_sub(M, v, f);
#pragma unroll
         for (int c = 0; c < 4; c++) { zs[8 * p + c] = f[c]; zs[8 * p + 4 + c] = v[c]; gt[c] = f[c]; }
      }
      // a_p: only atop_{P-2} and abot_0 enter Z_{P-1}, so the recurrence
      // carries the bottom rows
      float at[4], ab[4], an[4];
#pragma unroll
      for (int c = 0; c < 4; c++) { at[c] = zs[8 * (P - 2) + c]; ab[c] = zs[8 * (P - 2) + 4 + c]; }
      const float yeL[4] = {ry[8 * (P - 1) + 4], ry[8 * (P - 1) + 5], ry[8 * (P - 1) + 6], ry[8 * (P - 1) + 7]};
      const float ys0[4] = {ry[0], ry[1], ry[2], ry[3]};
      const float atL[4] = {at[0], at[1], at[2], at[3]};
      for (int p = P - 3; p >= 0; p--) {
         const float* rr = red_s + kRedRow * p;
         float M[16], ub[4];
#pragma unroll
         for (int c = 0; c < 4; c++) { ub[c] = zs[8 * p + 4 + c]; an[c] = ab[c]; }
         ld16s(rr + RGB, M);
         mv_sub(M, an, ub);
#pragma unroll
         for (int c = 0; c < 4; c++) ab[c] = ub[c];
      }
      // ab = abot_0
      float z[8], M[16];
      const float* last = red_s + kRedLast;
#pragma unroll
      for (int c = 0; c < 4; c++) { z[c] = yeL[c]; z[4 + c] = ys0[c]; }
      {
         float zt[4] = {z[0], z[1], z[2], z[3]}, zb[4] = {z[4], z[5], z[6], z[7]};
         ld16s(last + 64, M);
         mv_add(M, atL, zt);
         ld16s(last + 80, M);
         mv_add(M, ab, zb);
#pragma unroll
         for (int c = 0; c < 4; c++) { z[c] = zt[c]; z[4 + c] = zb[c]; }
      }
      m8_solve(last, z);
      const float ztop[4] = {z[0], z[1], z[2], z[3]};
      float zb[4] = {z[4], z[5], z[6], z[7]};   // bottom of Z_{p+1} (Z_{P-1} = z first)
#pragma unroll
      for (int c = 0; c < 8; c++) zs[8 * (P - 1) + c] = z[c];
      for (int p = P - 2; p >= 0; p--) {
         const float* rr = red_s + kRedRow * p;
         float ut[4], ub[4];
#pragma unroll
         for (int c = 0; c < 4; c++) { ut[c] = zs[8 * p + c]; ub[c] = zs[8 * p + 4 + c]; }
         ld16s(rr + RGT, M);
         mv_sub(M, zb, ut);
         ld16s(rr + RGB, M);
         mv_sub(M, zb, ub);
         ld16s(rr + RHT, M);
         mv_sub(M, ztop, ut);
         ld16s(rr + RHB, M);
         mv_sub(M, ztop, ub);
#pragma unroll
         for (int c = 0; c < 4; c++) { zs[8 * p + c] = ut[c]; zs[8 * p + 4 + c] = ub[c]; zb[c] = ub[c]; }
      }
   }
   __syncwarp();
   if (lane < P) {
      // x_k = y_k + V_k t_{p+1} + W_k b_{p-1}; row k+1's data loaded while
      // row k is formed
      float tn[4], bp[4];
      const int pm = (lane == 0) ? P - 1 : lane - 1;
#pragma unroll
      for (int c = 0; c < 4; c++) {
         tn[c] = zs[8 * lane + 4 + c];
         bp[c] = zs[8 * pm + c];
      }
      const int* scell = d.row_scell + row0 + s;
      float v[16], w[16], x[4];
      ld16t(d.sp_fac + tix(R0, kSpRec, 48, lane), v);
      ld16t(d.sp_fac + tix(R0, kSpRec, 64, lane), w);
#pragma unroll
      for (int c = 0; c < 4; c++) x[c] = d.sp_y[tix(R0, 4, c, lane)];
      int sc = scell[0];
      for (int k = 0; k < n; k++) {
         float vn[16], wn[16], xn[4];
         int scn = 0;
         if (k + 1 < n) {
            ld16t(d.sp_fac + tix(R0 + k + 1, kSpRec, 48, lane), vn);
            ld16t(d.sp_fac + tix(R0 + k + 1, kSpRec, 64, lane), wn);
#pragma unroll
            for (int c = 0; c < 4; c++) xn[c] = d.sp_y[tix(R0 + k + 1, 4, c, lane)];
            scn = scell[k + 1];
         }
         mv_add(w, bp, x);
         mv_add(v, tn, x);
         st4(d.r32 + 4 * (size_t)sc, x);
         if (k + 1 < n) {
#pragma unroll
            for (int m = 0; m < 16; m++) { v[m] = vn[m]; w[m] = wn[m]; }
#pragma unroll
            for (int c = 0; c < 4; c++) x[c] = xn[c];
            sc = scn;
         }
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

// dynamic shared memory of the fused factorisation: the staged terms
size_t mx_factor_stage_bytes(int block) { return (size_t)kStageTerms * 4 * sizeof(float4) * block; }

int mx_configure()
{
   const int want = (int)mx_factor_stage_bytes(128);
   if (cudaFuncSetAttribute(mx_factor_kernel<true, kElimChunk>, cudaFuncAttributeMaxDynamicSharedMemorySize, want) !=
           cudaSuccess ||
       cudaFuncSetAttribute(mx_factor_kernel<true, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, want) !=
           cudaSuccess)
      return 1;
   return 0;
}

void launch_mx_factor(const DeviceState& d, cudaStream_t st)
{
   const int tb = d.mx_block;
   const unsigned nb = (d.nChain + tb - 1) / tb;
   const bool chunk = d.nChain <= d.mx_chunk_chains;
   if (d.mx_fused) {
      const size_t sm = mx_factor_stage_bytes(tb);
      if (chunk) mx_factor_kernel<true, kElimChunk><<<nb, tb, sm, st>>>(d, d.nChain);
      else mx_factor_kernel<true, 1><<<nb, tb, sm, st>>>(d, d.nChain);
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
