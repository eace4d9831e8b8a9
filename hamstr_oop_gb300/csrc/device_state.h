// ##################################################################
//
// device_state.h -- device buffers of one solver handle and the kernel
// launchers shared between the translation units
//
// Layout in HBM (all FP64 values are the reference's doubles):
//   q, r, r0, dq      [nCell][4]  array-of-structs, 32 B per cell: one
//                                  sector per cell for the stencil gathers
//   sigma, dtfac      [nCell]
//   flux              [nSlot][4]  face flux (computeRHS) or linear flux
//   spec              [nSlot]     spectral radius times area
//   ff                [nSlot][32] lmat[4][4] then rmat[4][4] per face slot
//   stencil           [nSten]     int4 {cell, kind, face, -}
//   slot              [nSlot]     int4 {n, left, right, swap|owner<<1}
//   normal            [nSlot]     double2 face normal (dy, -dx)
//   refl              [nFace]     double4 wall reflection 2x2
//   factor storage    [nRow][80]  per ADI row: A, LU, C', fill', cN
// ##################################################################
#ifndef HAMSTR_GPU_DEVICE_STATE_H
#define HAMSTR_GPU_DEVICE_STATE_H

#include <cuda_runtime.h>

#include "lu4.cuh"

namespace hamstr {

// status bits raised by kernels into DeviceState::status
enum {
   DEV_ERR_NAN_SPEC = 1,     // spectral radius is NaN (interfaceFlux.cpp:117-124)
   DEV_ERR_PIVOT = 2,        // an ADI line's LU pivot is zero or not finite (reciprocal not finite)
   DEV_ERR_DQ = 4,           // an ADI sweep left a non-finite dq
   DEV_ERR_WAIT = 8,         // a line solve gave up waiting for its factorisation (adi.cu; never expected)
};

struct FlowConst {
   double gamma, rinf, uinf, vinf, einf, cfl;
};

constexpr int kWlinPerSlot = 2 * 4 * 18;   // sides x components x values (recon.cuh Weno5Lin)

// FP32 form, segmented solve of long chains: periodic chains of at least
// kSpikeMinRows rows and open chains of at least kSpikeMinOpenRows,
// kSpikeRows rows per segment (at most kSpikeMaxSeg segments, one warp lane
// each), kSpikeRedStride floats of boundary-system factors per chain.  An
// open chain is the cyclic system with its two wrap-around couplings
// (A of its first row, C of its last, which the open solve never reads)
// set to zero.
constexpr int kSpikeMinRows = 64;
constexpr int kSpikeMinOpenRows = 32;
constexpr int kSpikeRows = 16;
constexpr int kSpikeMaxSeg = 32;
constexpr int kSpikeRedStride = 256 * kSpikeMaxSeg;

struct DeviceState {
   int nCell, nFace, nSlot, nSten, nRow, nChain, order, nGhost;
   int recon;              // reconstruction code: order, or 31/32 for MUSCL with a project limiter (recon.cuh)
   int lin_order;          // 0: the sweeps' linearised residual at the scheme's order; 1: at first order
   FlowConst fc;

   // instances: the batched form holds several meshes / flow conditions in
   // one handle (a disjoint union; every launch covers all of them); a
   // plain handle has one.  Norms, histories and forces are per instance.
   int nInst;
   double4* fstab;         // [nInst] freestream ghost state rho, rho u, rho v, E (computeRHS.cpp:239-256)
   int2* cell_blocks;      // [norm_blocks] cells of each norm block; a block never spans two instances
   int* inst_block0;       // [nInst+1] first norm block of each instance
   int* inst_ncell;        // [nInst] cells per instance (the L2 norm's divisor)
   int* inst_done;         // [nInst] 1 once an instance has met the march tolerance (frozen)
   int *slot_inst, *cell_inst, *chain_inst, *block_inst;   // instance of each slot, cell, chain, norm block

   double *q, *r, *r0, *dq, *sigma, *dtfac;
   double* qt;             // second state of the RK3 scheme (solnBlock.h:47)
   double *flux, *spec, *ff;
   // order 5, FP64: f-only values of the WENO linearisation, written by the
   // implicit computeRHS reconstruction and read by the sweeps' linearised
   // reconstructions of the same step ([kWlinPerSlot][nSlot]); null when
   // not kept
   double* wlin;
   // order 5: the two reconstructed states of every slot, [2*4][nSlot]
   // (recon5 kernel, read by the face kernels); null otherwise
   double* qface;
   int4* sten;
   int4* slot;
   int* slot_face;
   double2* normal;
   double4* refl;
   int *cell_ptr, *cell_ent;
   int *chain_periodic, *chain_nrows, *chain_row0;
   int nWave;
   int *wave_chains;
   int *row_scell, *row_fcell, *row_ops;
   int *cell_written;
   double* blk;            // per-row assembled blocks A, B, C (scaled, B + I) [nRow][48]
   int *sched_job0, *sched_njobs, *sched_job_ptr, *sched_jobs;   // persistent-warp job queues (plan.h)
   int* sched_ncrit;       // per schedule: leading jobs that run alone on their SM (plan.h)
   int* sched_ctr;         // [sched_nctr = 1 + msweep*nWave] next-job counters: factorisation, then sweep s
   int sched_nctr;         // wave w at 1 + s*nWave + w; adi_assemble zeroes them
   double* fac;            // per-row factor storage
   double* fsc;            // per-row right-hand side / solution scratch [nRow][4]
   double* facN;           // per periodic chain: final LU of the last row (16)
   int* chain_facN;        // periodic chain -> index into facN (or -1)
   double2* norm_part;     // per-block {sum r_rho^2, max |r_rho|}
   double* norms;          // [nInst][4]: computeRHS L2, Linf, linear L2, Linf of the last reductions
   int* status;            // device error word
   int* ctl;               // [0] stop flag (march converged), [1] step counter
   double* hist;           // [hist_cap][nInst][4] norms per step (march)
   int hist_cap;
   double* tol;            // [0] march stop tolerance on the computeRHS L2 norm (<= 0: off)
   int norm_blocks;
   int exclusive_smem;     // dynamic shared memory that keeps ADI blocks one per SM

   // launch shapes chosen by hamstr_gpu_autotune (host-side only)
   int face_block;         // threads per block of the face kernels (<= 256)
   int adi_wpb;            // warps per block (= per SM) of the persistent FP64 solve kernel (4 or 8)
   int adi_fwpb;           // the same for the FP64 factorisation kernel
   int mx_block;           // threads per block of the FP32 thread-per-chain line kernels
   int mx_fused;           // 1: FP32 blocks assembled inside the factorisation; 0: mx_assemble first
   int mx_chunk_chains;    // FP32 line kernels over at most this many chains load rows in chunks (all resident)
   int face_soft;          // 1: FP64 divisions of the face kernels on the integer pipes (softdiv.cuh)
   int piv_soft;           // 1: the same for the LU pivots of the FP64 line factorisation

   // mixed-precision defect correction (FP64 residual, FP32 operator)
   float* ff32;            // [nSlot][32] FP32 face Jacobians
   // The FP32 line data is tiled by groups of 32 chains in line_chains
   // order, one chain per thread: element e of row i of the chain at
   // position p sits at ((grp_row0[p >> 5] + i) * W + (e & ~3)) * 32 +
   // 4 * (p & 31) + (e & 3) of a W-wide record array (mixed.cu tix): each
   // thread moves four elements as one float4, and a warp's access of one
   // group of four is 512 contiguous bytes.  A group takes as many tile
   // rows as its longest chain.
   float* blk32;           // W = 48: assembled blocks A, B, C (B + I), unfused assembly only
   float* fsc32;           // W = 4: right-hand side / forward sweep
   float* fac32;           // W = 80: factor records
   float* facN32;          // [periodic chains][16]
   int* grp_row0;          // [groups + 1] first tile row of each group of 32 positions
   int* tile_row;          // [tile_rows * 32] ADI row at (tile row, lane), -1 for padding
   int tile_rows;
   float *r32, *r032, *dq32;   // [nCell][4]
   float* g32;             // [nSlot][4] linear face fluxes
   int* line_chains;       // chains of each wave, longest first (thread per chain)

   // FP32 form: long chains solved by segments (mixed.cu).  A chain of N
   // rows (periodic, N >= kSpikeMinRows; open, N >= kSpikeMinOpenRows) is
   // cut into P segments, one warp lane each; each lane factors its segment
   // and the two "spikes" (its local responses to the couplings across its
   // ends), and a small cyclic system on the segment boundaries joins them.
   // Same linear system as the sequential block Thomas, about N/P rows of
   // latency instead of N.
   int sp_on;              // 1: long chains take the segmented solve (shape key)
   int nSpike;             // chains solved by segments
   int* chain_spike;       // [nChain] index into the sp_* arrays, or -1
   int* sp_chain;          // [nSpike] chain id
   int* sp_wave_ptr;       // [nWave+1] spike chains of each wave: sp indices sp_wave_ptr[w] .. [w+1]-1
   int* sp_seg;            // [nSpike][kSpikeMaxSeg+1] first row (in the chain) of each segment, then N
   int* sp_nseg;           // [nSpike] P
   int* sp_rec0;           // [nSpike] first tile row of the chain in sp_fac / sp_y (it takes as many
                           // tile rows as its longest segment has rows)
   float* sp_fac;          // [tile rows][80][32 segments]: A, LU(B'), C' (local), V (right spike),
                           // W (left spike) of local row k of each segment
   float* sp_y;            // [tile rows][4][32 segments]: the sweep's local solutions
   float* sp_red;          // [nSpike][kSpikeRedStride]: factors of the boundary system
};

// true once a march has met its tolerance: every later kernel of the step
// returns at once, so a captured run of steps stops exactly there
__device__ __forceinline__ bool halted(const DeviceState& d) { return *(volatile const int*)d.ctl != 0; }

// A march over a batch freezes each instance at the step whose computeRHS
// L2 norm first meets the tolerance -- the state a plain handle's march
// stops in -- and skips its work from then on.  A plain handle (one
// instance) never reads these arrays.
__device__ __forceinline__ bool frozen_inst(const DeviceState& d, int k) { return d.nInst > 1 && d.inst_done[k] != 0; }
__device__ __forceinline__ bool frozen_slot(const DeviceState& d, int s)
{
   return d.nInst > 1 && d.inst_done[d.slot_inst[s]] != 0;
}
__device__ __forceinline__ bool frozen_cell(const DeviceState& d, int c)
{
   return d.nInst > 1 && d.inst_done[d.cell_inst[c]] != 0;
}
__device__ __forceinline__ bool frozen_chain(const DeviceState& d, int ch)
{
   return d.nInst > 1 && d.inst_done[d.chain_inst[ch]] != 0;
}

// block size of every kernel that reduces norms over cells
constexpr int kNormBlock = 256;

// this thread's cell in a norm-block launch (kNormBlock threads per block,
// one block per d.cell_blocks entry), or -1 past the block's cells
__device__ __forceinline__ int norm_cell(const DeviceState& d)
{
   const int2 cb = d.cell_blocks[blockIdx.x];
   const int c = cb.x + (int)threadIdx.x;
   if (d.nInst > 1 && d.inst_done[d.block_inst[blockIdx.x]] != 0) return -1;
   return c < cb.y ? c : -1;
}

// launchers (rhs.cu)
// order 5: the reconstructed face states (and, keep_lin with d.wlin, the
// WENO linearisation's f-only values) ahead of rhs_face / mx_rhs_face; a
// no-op at other orders
void launch_recon5(const DeviceState& d, bool keep_lin, cudaStream_t st);
void launch_rhs_face(const DeviceState& d, bool jacobian, cudaStream_t st);
void launch_rhs_cell(const DeviceState& d, bool adi_init, cudaStream_t st);
// order 5: the linearised face states into qface ahead of lin_face; kept:
// this step's implicit recon5 wrote d.wlin from the current q (a no-op at
// other orders)
void launch_lin_recon5(const DeviceState& d, bool kept, cudaStream_t st);
void launch_lin_face(const DeviceState& d, cudaStream_t st);
void launch_lin_cell(const DeviceState& d, bool update_q, cudaStream_t st);
// norms -> d.norms[off], d.norms[off+1] and hist row ctl[1] (when logging);
// with check_tol, raises the stop flag when L2 <= tol
void launch_norm_final(const DeviceState& d, int off, bool check_tol, cudaStream_t st);
void launch_step_end(const DeviceState& d, cudaStream_t st);
void launch_dtfac(const DeviceState& d, cudaStream_t st);
// qnew = qold + coef*CFL/sigma * r (march.cpp:411-433)
void launch_update(const DeviceState& d, const double* qold, double* qnew, double coef, cudaStream_t st);
void launch_adi_init(const DeviceState& d, cudaStream_t st);
void launch_dq_update(const DeviceState& d, cudaStream_t st);
// launchers (adi.cu)
// launchers (mixed.cu): FP64 residual + FP32 Jacobian/ADI defect correction
void launch_mx_rhs_face(const DeviceState& d, cudaStream_t st);
void launch_mx_init(const DeviceState& d, cudaStream_t st);
void launch_mx_assemble(const DeviceState& d, cudaStream_t st);   // no-op when d.mx_fused
void launch_mx_factor(const DeviceState& d, cudaStream_t st);
void launch_mx_solve(const DeviceState& d, int first, int count, cudaStream_t st);
// chains the chunked FP32 solve holds resident at once with `block` threads per block (0 on error)
int mx_solve_chunk_capacity(int block);
void launch_mx_dq_update(const DeviceState& d, cudaStream_t st);
// allows the fused FP32 factorisation its staging shared memory (once per
// device, before the first launch); nonzero on failure
int mx_configure();
void launch_mx_lin_face(const DeviceState& d, cudaStream_t st);
void launch_mx_lin_cell(const DeviceState& d, bool update_q, cudaStream_t st);
// segmented solve of the long periodic chains (d.nSpike > 0 and d.sp_on):
// factorisation once per step, the solve of wave w's chains per sweep
void launch_mx_spike_factor(const DeviceState& d, cudaStream_t st);
void launch_mx_spike_solve(const DeviceState& d, int first, int count, cudaStream_t st);
void launch_adi_assemble(const DeviceState& d, cudaStream_t st);
// nwarps persistent warps over the schedule's job queue (nwarps may be 0);
// the solve of wave `wave` in sweep `sweep` takes counter 1 + sweep*nWave + wave
void launch_adi_factor(const DeviceState& d, int nwarps, cudaStream_t st);
void launch_adi_solve(const DeviceState& d, int sweep, int wave, int nwarps, cudaStream_t st);
int adi_configure(int max_dynamic_smem);
// launcher (forces.cu): per instance k, out[3k..3k+2] = {Fx, Fy, M} over
// its wall faces wall0[k]..wall0[k+1]-1; scr = 3 doubles per wall face
void launch_forces(const double* q, const int* wall_cell, const double4* geo, const int* wall0, int ninst,
                   double gm1, double* scr, double* out, cudaStream_t st);

}  // namespace hamstr
#endif
