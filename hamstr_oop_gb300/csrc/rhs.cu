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
#include "recon.cuh"
#include "roe.cuh"

namespace hamstr {

namespace {

constexpr int kThreads = 256;
static_assert(kThreads == kNormBlock, "cell kernels run one norm block per thread block");
// eight order-5 reconstructions per slot, one thread each (recon5_one):
// the four components of a slot in adjacent lanes (one 32-byte sector of
// q per stencil cell), blockIdx.y the side
template <bool SD, bool WL>
__global__ void __launch_bounds__(kThreads) recon5_kernel(DeviceState d)
{
   const int s = blockIdx.x * (kThreads / 4) + (threadIdx.x >> 2);
   if (s >= d.nSlot || halted(d) || frozen_slot(d, s)) return;
   recon5_one<SD, WL>(d, s, blockIdx.y, threadIdx.x & 3);
}

// PRE: the face states come from recon5_kernel (order 5).  Two blocks per
// SM at least: the Roe Jacobian is a long chain of dependent FP64
// operations, and more warps hide more of it than the few spilled
// registers cost.
template <int ORDER, bool JAC, bool SD, bool PRE = false>
__global__ void __launch_bounds__(kThreads, 2) rhs_face_kernel(DeviceState d)
{
   const int s = blockIdx.x * blockDim.x + threadIdx.x;
   if (s >= d.nSlot || halted(d) || frozen_slot(d, s)) return;
   const int4 sl = d.slot[s];
   const double2 nv = d.normal[s];
   double L[4], R[4];
   if (PRE) face_states_pre(d, s, (sl.w & 1) != 0, L, R);
   else face_states<ORDER, SD>(d, sl.x, (sl.w & 1) != 0, L, R);
   RoeOut o;
   double lm[16], rm[16];
   if (!roe_face<JAC, SD>(nv.x, nv.y, L, R, d.fc.gamma, o, lm, rm)) atomicOr(d.status, DEV_ERR_NAN_SPEC);
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

// eight linearised order-5 reconstructions per slot, one thread each
// (blockIdx.y: the state, as in recon5_kernel)
template <bool SD, bool WL>
__global__ void __launch_bounds__(kThreads) lin_recon5_kernel(DeviceState d)
{
   const int s = blockIdx.x * blockDim.x + threadIdx.x;
   if (s >= d.nSlot || halted(d) || frozen_slot(d, s)) return;
   const int sk = blockIdx.y;
   lin_recon5_one<SD, WL>(d, d.dq, s, sk >> 2, sk & 3);
}

// PRE: the linearised states come from lin_recon5_kernel (order 5)
template <int ORDER, bool SD, bool PRE = false>
__global__ void __launch_bounds__(kThreads) lin_face_kernel(DeviceState d)
{
   const int s = blockIdx.x * blockDim.x + threadIdx.x;
   if (s >= d.nSlot || halted(d) || frozen_slot(d, s)) return;
   const int4 sl = d.slot[s];
   double dL[4], dR[4];
   if (PRE) face_states_pre(d, s, (sl.w & 1) != 0, dL, dR);
   else face_dstates<ORDER, double, SD>(d, d.dq, sl.x, (sl.w & 1) != 0, dL, dR);
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
   const int c = norm_cell(d);
   double sq = 0.0, am = 0.0;
   if (c >= 0) {
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
   const int c = norm_cell(d);
   double sq = 0.0, am = 0.0;
   if (c >= 0) {
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
   // one warp per instance: fixed-shape reduction of its block partials
   __shared__ int s_open;
   if (threadIdx.x == 0) s_open = 0;
   __syncthreads();
   const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
   const int it = d.ctl[1];
   for (int k = w; k < d.nInst; k += nw) {
      if (frozen_inst(d, k)) continue;   // its norms stay those of its last step
      double a = 0.0, b = 0.0;
      for (int i = d.inst_block0[k] + l; i < d.inst_block0[k + 1]; i += 32) {
         const double2 p = d.norm_part[i];
         a += p.x;
         b = fmax(b, p.y);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
         a += __shfl_xor_sync(0xffffffffu, a, o);
         b = fmax(b, __shfl_xor_sync(0xffffffffu, b, o));
      }
      if (l == 0) {
         const double l2 = sqrt(a) / d.inst_ncell[k];
         d.norms[4 * k + off] = l2;
         d.norms[4 * k + off + 1] = b;
         if (it < d.hist_cap) {
            d.hist[4 * ((size_t)it * d.nInst + k) + off] = l2;
            d.hist[4 * ((size_t)it * d.nInst + k) + off + 1] = b;
         }
         if (check_tol && *d.tol > 0.0 && l2 <= *d.tol) {
            if (d.nInst > 1) d.inst_done[k] = 1;   // frozen from this step's ADI on
         } else {
            atomicOr(&s_open, 1);
         }
      }
   }
   __syncthreads();
   // the march stops once every instance's computeRHS L2 has met tol
   if (threadIdx.x == 0 && check_tol && *d.tol > 0.0 && s_open == 0) d.ctl[0] = 1;
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
   if (c >= d.nCell || halted(d) || frozen_cell(d, c)) return;
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
   if (c >= d.nCell || halted(d) || frozen_cell(d, c)) return;
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
   if (c >= d.nCell || halted(d) || frozen_cell(d, c)) return;
   double r[4], dq[4];
   ld4(d.r + 4 * (size_t)c, r);
   ld4(d.dq + 4 * (size_t)c, dq);
#pragma unroll
   for (int k = 0; k < 4; k++) dq[k] += r[k];
   st4(d.dq + 4 * (size_t)c, dq);
   if (nonfinite(dq[0]) || nonfinite(dq[1]) || nonfinite(dq[2]) || nonfinite(dq[3])) atomicOr(d.status, DEV_ERR_DQ);
}

inline int blocks_for(int n) { return (n + kThreads - 1) / kThreads; }

}  // namespace

namespace {
template <bool SD>
void rhs_face_go(const DeviceState& d, bool jac, int b, int t, cudaStream_t st)
{
   switch (d.recon * 2 + (jac ? 1 : 0)) {
      case 2: rhs_face_kernel<1, false, SD><<<b, t, 0, st>>>(d); break;
      case 3: rhs_face_kernel<1, true, SD><<<b, t, 0, st>>>(d); break;
      case 6: rhs_face_kernel<3, false, SD><<<b, t, 0, st>>>(d); break;
      case 7: rhs_face_kernel<3, true, SD><<<b, t, 0, st>>>(d); break;
      case 10:
         if (d.qface) rhs_face_kernel<5, false, SD, true><<<b, t, 0, st>>>(d);
         else rhs_face_kernel<5, false, SD><<<b, t, 0, st>>>(d);
         break;
      case 11:
         if (d.qface) rhs_face_kernel<5, true, SD, true><<<b, t, 0, st>>>(d);
         else rhs_face_kernel<5, true, SD><<<b, t, 0, st>>>(d);
         break;
      case 62: rhs_face_kernel<31, false, SD><<<b, t, 0, st>>>(d); break;
      case 63: rhs_face_kernel<31, true, SD><<<b, t, 0, st>>>(d); break;
      case 64: rhs_face_kernel<32, false, SD><<<b, t, 0, st>>>(d); break;
      default: rhs_face_kernel<32, true, SD><<<b, t, 0, st>>>(d); break;
   }
}
}  // namespace

void launch_recon5(const DeviceState& d, bool keep_lin, cudaStream_t st)
{
   if (d.recon != 5 || !d.qface) return;
   const dim3 b((4 * d.nSlot + kThreads - 1) / kThreads, 2);
   const bool wl = keep_lin && d.wlin;
   if (d.face_soft) {
      if (wl) recon5_kernel<true, true><<<b, kThreads, 0, st>>>(d);
      else recon5_kernel<true, false><<<b, kThreads, 0, st>>>(d);
   } else {
      if (wl) recon5_kernel<false, true><<<b, kThreads, 0, st>>>(d);
      else recon5_kernel<false, false><<<b, kThreads, 0, st>>>(d);
   }
}

void launch_rhs_face(const DeviceState& d, bool jac, cudaStream_t st)
{
   const int t = d.face_block;
   const int b = (d.nSlot + t - 1) / t;
   if (d.face_soft) rhs_face_go<true>(d, jac, b, t, st);
   else rhs_face_go<false>(d, jac, b, t, st);
}

void launch_rhs_cell(const DeviceState& d, bool adi_init, cudaStream_t st)
{
   if (adi_init) rhs_cell_kernel<true><<<d.norm_blocks, kThreads, 0, st>>>(d);
   else rhs_cell_kernel<false><<<d.norm_blocks, kThreads, 0, st>>>(d);
}

void launch_lin_recon5(const DeviceState& d, bool kept, cudaStream_t st)
{
   if (d.recon != 5 || !d.qface || d.lin_order == 1) return;
   const dim3 b((d.nSlot + kThreads - 1) / kThreads, 8);
   const bool wl = kept && d.wlin;
   if (d.face_soft) {
      if (wl) lin_recon5_kernel<true, true><<<b, kThreads, 0, st>>>(d);
      else lin_recon5_kernel<true, false><<<b, kThreads, 0, st>>>(d);
   } else {
      if (wl) lin_recon5_kernel<false, true><<<b, kThreads, 0, st>>>(d);
      else lin_recon5_kernel<false, false><<<b, kThreads, 0, st>>>(d);
   }
}

void launch_lin_face(const DeviceState& d, cudaStream_t st)
{
   const int kThreads = d.face_block;
   const int b = (d.nSlot + kThreads - 1) / kThreads;
   // only the WENO linearisation divides in FP64 here
   if (d.lin_order == 1) {
      lin_face_kernel<1, true><<<b, kThreads, 0, st>>>(d);
      return;
   }
   switch (d.recon) {
      case 1: lin_face_kernel<1, true><<<b, kThreads, 0, st>>>(d); break;
      case 3: lin_face_kernel<3, true><<<b, kThreads, 0, st>>>(d); break;
      case 5:
         if (d.qface) lin_face_kernel<5, true, true><<<b, kThreads, 0, st>>>(d);
         else if (d.face_soft) lin_face_kernel<5, true><<<b, kThreads, 0, st>>>(d);
         else lin_face_kernel<5, false><<<b, kThreads, 0, st>>>(d);
         break;
      case 31: lin_face_kernel<31, true><<<b, kThreads, 0, st>>>(d); break;
      default: lin_face_kernel<32, true><<<b, kThreads, 0, st>>>(d); break;
   }
}

void launch_lin_cell(const DeviceState& d, bool update_q, cudaStream_t st)
{
   if (update_q) lin_cell_kernel<true><<<d.norm_blocks, kThreads, 0, st>>>(d);
   else lin_cell_kernel<false><<<d.norm_blocks, kThreads, 0, st>>>(d);
}

void launch_norm_final(const DeviceState& d, int off, bool check_tol, cudaStream_t st)
{
   norm_final_kernel<<<1, 32 * (d.nInst < 32 ? d.nInst : 32), 0, st>>>(d, off, check_tol ? 1 : 0);
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
