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
// the same instruction sequence.  Open chains need one half only, so the
// schedule may pair them (two per warp, one per half) or put eight in a
// warp, four lanes each (lane 4g + r on row r of every block).  Short open
// chains may also go 32 to a warp, one per lane (a bundle), which spends
// far fewer warp instructions per row on them.
//
// Per-row factor record (80 doubles):
//   [ 0..15] A_i scaled      (f update in the forward sweep)
//   [16..31] LU of B'_i      b11 u12 u13 u14 b21 b22 u23 u24 b31 b32 b33 u34 b41 b42 b43 b44
//   [32..47] C'_i            (back substitution)
//   [48..63] a'_i            (periodic fill-in column, back substitution)
//   [64..79] c_{N-1} at elimination step i (periodic, triSolvers.cpp:967-999)
// Periodic chains also keep the LU of the final last-row block (facN).
// ##################################################################
#include <algorithm>

#include "device_state.h"
#include "plan.h"
#include "line_solve.cuh"

namespace hamstr {

namespace {


// one block entry (row-major element e) in the reference's term order
// (ADI.cpp:103-188): 0.0, then += / -= the listed face-matrix entries.
// The first term needs no FP64 add: 0.0 + v is v and 0.0 - v is -v, except
// that both are +0.0 when v is a zero, so it is formed on the integer pipes
// with the same result (this kernel is FP64-issue bound).
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
      if (o == 0) {
         acc = sd::zero_plus(v, (op & 1) != 0);
      } else if (op & 1) {
         acc -= v;
      } else {
         acc += v;
      }
   }
   return acc;
}

// blocks A, B, C of every row, scaled by CFL/sigma with B += I
// (ADI.cpp:197-217); one thread per entry, all rows at once
__global__ void __launch_bounds__(256) adi_assemble_kernel(DeviceState d)
{
   const int t = blockIdx.x * blockDim.x + threadIdx.x;
   if (t < d.sched_nctr) d.sched_ctr[t] = 0;   // the line kernels' job counters, for this step
   if (t >= 48 * d.nRow || halted(d)) return;
   const int row = t / 48, e48 = t - 48 * row, b = e48 >> 4, e = e48 & 15;
   if (frozen_cell(d, d.row_scell[row])) return;
   double v = assemble(d, d.row_ops + 3 * kOpsPerBlock * row + kOpsPerBlock * b, e);
   v = sd::mul(v, d.dtfac[d.row_scell[row]]);   // v * CFL/sigma on the integer pipes, identical
   if (b == 1 && (e >> 2) == (e & 3)) v += 1.0;
   d.blk[t] = v;
}

// block-Thomas factorisation of chain ich (its assembled rows in blk)
// (prog: rows published for a following solve, line_solve.cuh publish_rows)
template <bool SD>
__device__ __forceinline__ bool factor_chain(const DeviceState& d, int ich, int lane, int* prog = nullptr)
{
   const int N = d.chain_nrows[ich], row0 = d.chain_row0[ich];
   const bool per = d.chain_periodic[ich] != 0;
   const double* blk = d.blk + 48 * (size_t)row0;
   return factor_line<SD>(blk, blk + 16, blk + 32, 48, N, per, d.fac + (size_t)kFacRec * row0,
               per ? d.facN + 16 * d.chain_facN[ich] : nullptr, lane, prog);
}

// rows of chain ich for this half-warp's work: 0 once its instance is frozen
__device__ __forceinline__ int live_rows(const DeviceState& d, int ich)
{
   return frozen_chain(d, ich) ? 0 : d.chain_nrows[ich];
}

// two open chains, one per half-warp (line_solve.cuh factor_line_pair)
template <bool SD>
__device__ __forceinline__ bool factor_pair(const DeviceState& d, int ia, int ib, int lane, int* prog = nullptr)
{
   const int ich = (lane >> 4) ? ib : ia;
   const int N = live_rows(d, ich), row0 = d.chain_row0[ich];
   return factor_line_pair<SD>(d.blk + 48 * (size_t)row0, 48, N, d.fac + (size_t)kFacRec * row0, lane, prog);
}

// Where a schedule has long jobs to place (ncrit != 0), the first warp of
// block b (one block per SM) starts with job b, so each long job starts on
// an SM of its own; beside a few outliers (ncrit > 0) the other warps of
// the blocks holding them take no job, beside many (ncrit < 0, the loops of
// a quad O-grid) they take jobs as usual.  The counter then numbers the jobs
// after the assigned ones (off = the number of blocks).  Otherwise every
// warp takes every job from the counter (off = 0).

// next job index of a persistent warp: lane 0 takes it from the counter
__device__ __forceinline__ int take_job(int* ctr, int off, int lane)
{
   int k = 0;
   if (lane == 0) k = off + atomicAdd(ctr, 1);
   return __shfl_sync(kLaneMask, k, 0);
}

// Whether a warp takes its next job only after job k: after a long first
// job (warp 0 of block b < nlong, job b).  A job index taken at its start
// would reserve a queued job that then waits behind the long one, and the
// launch would end with it.
__device__ __forceinline__ bool late_next(int k, int k0, int nlong)
{
   return k == k0 && (threadIdx.x >> 5) == 0 && (int)blockIdx.x < nlong;
}

// a warp's first job, or -1 for a warp that stays idle beside an outlier
__device__ __forceinline__ int first_job(int* ctr, int ncrit, int off, int lane)
{
   const int b = blockIdx.x, wib = threadIdx.x >> 5;
   if (ncrit == 0) return take_job(ctr, off, lane);
   if (wib == 0) return b;
   if (b < ncrit) return -1;
   return take_job(ctr, off, lane);
}

// one sweep's solve of chain ich: F = r[fcell] (ADI.cpp:116,187), the
// replay, and the write-back r[scell] = F (ADI.cpp:232-244); FOLLOW: behind
// its factorisation by another warp of the block (line_solve.cuh)
template <bool FOLLOW = false>
__device__ __forceinline__ void solve_chain(const DeviceState& d, int ich, int lane, const int* prog = nullptr,
                                            bool* ok = nullptr)
{
   const int N = d.chain_nrows[ich], row0 = d.chain_row0[ich];
   const bool per = d.chain_periodic[ich] != 0;
   double* fs = d.fsc + 4 * (size_t)row0;
   for (int r = lane; r < N; r += 32) {
      const int fc = d.row_fcell[row0 + r];
      double v[4] = {0.0, 0.0, 0.0, 0.0};
      if (fc >= 0) ld4(d.r + 4 * (size_t)fc, v);
      *reinterpret_cast<double2*>(fs + 4 * r) = make_double2(v[0], v[1]);
      *reinterpret_cast<double2*>(fs + 4 * r + 2) = make_double2(v[2], v[3]);
   }
   __syncwarp();
   solve_line<FOLLOW>(d.fac + (size_t)kFacRec * row0, per ? d.facN + 16 * d.chain_facN[ich] : nullptr, N, per, fs,
                      lane, prog, ok);
   __syncwarp();
   for (int r = lane; r < N; r += 32) {
      const int sc = d.row_scell[row0 + r];
      double v[4];
      ld4(fs + 4 * r, v);
      *reinterpret_cast<double2*>(d.r + 4 * (size_t)sc) = make_double2(v[0], v[1]);
      *reinterpret_cast<double2*>(d.r + 4 * (size_t)sc + 2) = make_double2(v[2], v[3]);
   }
}

// the same for two open chains, one per half-warp
template <bool FOLLOW = false>
__device__ __forceinline__ void solve_pair(const DeviceState& d, int ia, int ib, int lane, const int* prog = nullptr,
                                           bool* ok = nullptr)
{
   const int ich = (lane >> 4) ? ib : ia, l16 = lane & 15;
   const int N = live_rows(d, ich), row0 = d.chain_row0[ich];
   double* fs = d.fsc + 4 * (size_t)row0;
   for (int r = l16; r < N; r += 16) {
      const int fc = d.row_fcell[row0 + r];
      double v[4] = {0.0, 0.0, 0.0, 0.0};
      if (fc >= 0) ld4(d.r + 4 * (size_t)fc, v);
      *reinterpret_cast<double2*>(fs + 4 * r) = make_double2(v[0], v[1]);
      *reinterpret_cast<double2*>(fs + 4 * r + 2) = make_double2(v[2], v[3]);
   }
   __syncwarp();
   solve_line_pair<FOLLOW>(d.fac + (size_t)kFacRec * row0, N, fs, lane, prog, ok);
   __syncwarp();
   for (int r = l16; r < N; r += 16) {
      const int sc = d.row_scell[row0 + r];
      double v[4];
      ld4(fs + 4 * r, v);
      *reinterpret_cast<double2*>(d.r + 4 * (size_t)sc) = make_double2(v[0], v[1]);
      *reinterpret_cast<double2*>(d.r + 4 * (size_t)sc + 2) = make_double2(v[2], v[3]);
   }
}

// a fused first-wave pair job: both chains' right-hand sides gathered,
// then factorisation and the first sweep's forward substitution in one
// pass over the rows (factor_line_pair<SD, true>), the back substitution
// and the write-back; the same values as factor_pair then solve_pair
template <bool SD>
__device__ __forceinline__ bool factor_solve_pair(const DeviceState& d, int ia, int ib, int lane)
{
   const int ich = (lane >> 4) ? ib : ia, l16 = lane & 15;
   const int N = live_rows(d, ich), row0 = d.chain_row0[ich];
   double* fs = d.fsc + 4 * (size_t)row0;
   const double* fac = d.fac + (size_t)kFacRec * row0;
   for (int r = l16; r < N; r += 16) {
      const int fc = d.row_fcell[row0 + r];
      double v[4] = {0.0, 0.0, 0.0, 0.0};
      if (fc >= 0) ld4(d.r + 4 * (size_t)fc, v);
      *reinterpret_cast<double2*>(fs + 4 * r) = make_double2(v[0], v[1]);
      *reinterpret_cast<double2*>(fs + 4 * r + 2) = make_double2(v[2], v[3]);
   }
   __syncwarp();
   double xlast[4];
   const bool bad = factor_line_pair<SD, true>(d.blk + 48 * (size_t)row0, 48, N, d.fac + (size_t)kFacRec * row0,
                                               lane, fs, xlast);
   __syncwarp();
   back_line_pair(fac, N, fs, lane, xlast);
   __syncwarp();
   for (int r = l16; r < N; r += 16) {
      const int sc = d.row_scell[row0 + r];
      double v[4];
      ld4(fs + 4 * r, v);
      *reinterpret_cast<double2*>(d.r + 4 * (size_t)sc) = make_double2(v[0], v[1]);
      *reinterpret_cast<double2*>(d.r + 4 * (size_t)sc + 2) = make_double2(v[2], v[3]);
   }
   return bad;
}

// the factorisation of one job (entries at `job`, first entry `ich`
// without kFusedJob); returns whether a pivot was zero or not finite
template <bool SD>
__device__ __forceinline__ bool factor_job(const DeviceState& d, int job, int ich, int lane)
{
   bool bad = false;
   if (ich & kBundleJob) {
      const int n = ich & 63;
      if (lane < n) {
         const int c = d.sched_jobs[job + 1 + lane];
         if (!frozen_chain(d, c)) {
            const int row0 = d.chain_row0[c];
            bad |= factor_line_thread<SD>(d.blk + 48 * (size_t)row0, 48, d.chain_nrows[c],
                                          d.fac + (size_t)kFacRec * row0);
         }
      }
   } else if (ich & kQuadJob) {
      int c = 0, N = 0;
      if ((lane >> 2) < (ich & 63)) {
         c = d.sched_jobs[job + 1 + (lane >> 2)];
         N = live_rows(d, c);
      }
      const int row0 = d.chain_row0[c];
      bad |= factor_line_quad<SD>(d.blk + 48 * (size_t)row0, 48, N, d.fac + (size_t)kFacRec * row0, lane);
   } else if (ich & kPairJob) {
      bad |= factor_pair<SD>(d, ich & ~kPairJob, d.sched_jobs[job + 1], lane);
   } else if (!frozen_chain(d, ich)) {
      bad |= factor_chain<SD>(d, ich, lane);
   }
   return bad;
}

// one sweep's solve of one job (as factor_job)
__device__ __forceinline__ void solve_job(const DeviceState& d, int job, int ich, int lane)
{
   if (ich & kBundleJob) {
      const int n = ich & 63;
      if (lane < n) {
         const int c = d.sched_jobs[job + 1 + lane];
         if (!frozen_chain(d, c)) {
            const int row0 = d.chain_row0[c];
            solve_line_thread(d.fac + (size_t)kFacRec * row0, d.chain_nrows[c], d.r, d.row_fcell + row0,
                              d.row_scell + row0, d.fsc + 4 * (size_t)row0);
         }
      }
   } else if (ich & kQuadJob) {
      int c = 0, N = 0;
      if ((lane >> 2) < (ich & 63)) {
         c = d.sched_jobs[job + 1 + (lane >> 2)];
         N = live_rows(d, c);
      }
      const int row0 = d.chain_row0[c];
      solve_line_quad(d.fac + (size_t)kFacRec * row0, N, d.r, d.row_fcell + row0, d.row_scell + row0,
                      d.fsc + 4 * (size_t)row0, lane);
   } else if (ich & kPairJob) {
      solve_pair(d, ich & ~kPairJob, d.sched_jobs[job + 1], lane);
   } else if (!frozen_chain(d, ich)) {
      solve_chain(d, ich, lane);
   }
}

// persistent warps, one or two per SM sub-partition, taking jobs from the
// factorisation's queue (longest first) until it is empty; a zero or
// non-finite pivot raises DEV_ERR_PIVOT (the factors are still stored, as
// the reference divides regardless).  A job marked kFusedJob (the first
// wave's chains, when the schedule fuses) is solved for the first sweep by
// the same warp right after its factorisation: its right-hand sides are
// the computeRHS residuals, ready before this kernel, and the chains of
// one wave share no cell, so no other job waits for it.
//
// A long first job of block b (ncrit != 0, b < |ncrit|) that carries its
// first sweep's solve (kFusedJob, one chain or a pair) is solved by the
// block's second warp behind the factorisation of the first (the rows are
// published in shared memory as their records are stored), instead of by
// the factoring warp after it: a row's factorisation takes about three
// times its solve, so the solve adds only its last rows and the back
// substitution to the job's time.  Beside an outlier (ncrit > 0) that
// second warp was idle; beside many long jobs it takes queued jobs after.
template <bool SD>
__global__ void __launch_bounds__(256, 1) adi_factor_kernel(DeviceState d, int nwarps)
{
   __shared__ int prog;   // rows of the block's followed job that are factored
   const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, b = blockIdx.x;
   const int nj = d.sched_njobs[0], j0 = d.sched_job0[0];
   const int ncrit = d.sched_ncrit[0], nlong = ncrit < 0 ? -ncrit : ncrit;
   int fjob = -1, fich = 0;   // the followed job: warp 0's first, solved by warp 1
   if (b < nlong && b < nj && b * (int)(blockDim.x >> 5) + 1 < nwarps) {
      const int job = d.sched_job_ptr[j0 + b], head = d.sched_jobs[job];
      if ((head & kFusedJob) && !(head & (kBundleJob | kQuadJob))) {
         fjob = job;
         fich = head & ~kFusedJob;
      }
   }
   if (threadIdx.x == 0) prog = 0;
   __syncthreads();
   if (halted(d)) return;
   const int w = b * (blockDim.x >> 5) + wib;
   if (w >= nwarps) return;
   int* ctr = d.sched_ctr;
   bool bad = false;
   const int off = ncrit ? (int)gridDim.x : 0;
   int k0;
   if (fjob >= 0 && wib == 1) {
      bool ok = true;
      if (fich & kPairJob) solve_pair<true>(d, fich & ~kPairJob, d.sched_jobs[fjob + 1], lane, &prog, &ok);
      else if (!frozen_chain(d, fich)) solve_chain<true>(d, fich, lane, &prog, &ok);
      if (!ok && lane == 0) atomicOr(d.status, DEV_ERR_WAIT);
      if (ncrit > 0) return;
      k0 = take_job(ctr, off, lane);
   } else {
      k0 = first_job(ctr, ncrit, off, lane);
   }
   if (k0 < 0) return;
   for (int k = k0; k < nj;) {
      // the next job's index is fetched while this one runs, except after
      // a long first job (late_next)
      const bool late = late_next(k, k0, nlong);
      int kn = 0;
      if (!late && lane == 0) kn = off + atomicAdd(ctr, 1);
      const int job = d.sched_job_ptr[j0 + k];
      const int head = d.sched_jobs[job], ich = head & ~kFusedJob;
      if (job == fjob) {
         // factorisation only, its solve follows in warp 1
         if (ich & kPairJob) bad |= factor_pair<SD>(d, ich & ~kPairJob, d.sched_jobs[job + 1], lane, &prog);
         else if (!frozen_chain(d, ich)) bad |= factor_chain<SD>(d, ich, lane, &prog);
      } else if ((head & kFusedJob) && (ich & kPairJob)) {
         bad |= factor_solve_pair<SD>(d, ich & ~kPairJob, d.sched_jobs[job + 1], lane);
      } else {
         bad |= factor_job<SD>(d, job, ich, lane);
         if (head & kFusedJob) {
            __syncwarp();   // the records of every lane are written
            solve_job(d, job, ich, lane);
         }
      }
      if (late && lane == 0) kn = off + atomicAdd(ctr, 1);
      k = __shfl_sync(kLaneMask, kn, 0);
   }
   if (__any_sync(kLaneMask, bad) && lane == 0) atomicOr(d.status, DEV_ERR_PIVOT);
}


__global__ void __launch_bounds__(256, 1) adi_solve_kernel(DeviceState d, int sweep, int wave, int nwarps)
{
   if (halted(d)) return;
   const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
   if (w >= nwarps) return;
   const int lane = threadIdx.x & 31, nj = d.sched_njobs[1 + wave], j0 = d.sched_job0[1 + wave];
   int* ctr = d.sched_ctr + 1 + sweep * d.nWave + wave;
   const int ncrit = d.sched_ncrit[1 + wave], off = ncrit ? (int)gridDim.x : 0;
   const int nlong = ncrit < 0 ? -ncrit : ncrit;
   const int k0 = first_job(ctr, ncrit, off, lane);
   if (k0 < 0) return;
   for (int k = k0; k < nj;) {
      const bool late = late_next(k, k0, nlong);
      int kn = 0;
      if (!late && lane == 0) kn = off + atomicAdd(ctr, 1);
      const int job = d.sched_job_ptr[j0 + k];
      solve_job(d, job, d.sched_jobs[job], lane);
      if (late && lane == 0) kn = off + atomicAdd(ctr, 1);
      k = __shfl_sync(kLaneMask, kn, 0);
   }
}

}  // namespace

// One block per SM: the dynamic shared-memory request below exceeds half
// an SM's shared memory, so no two blocks share an SM.  With 4 warps per
// block each warp owns an SM sub-partition's FP64 unit; the autotuner may
// pick 8 (two per sub-partition) where chains are many and short.
constexpr int kExclusiveSmem = 120 * 1024;

int adi_configure(int max_dynamic_smem)
{
   const int want = max_dynamic_smem >= kExclusiveSmem ? kExclusiveSmem : 0;
   if (want) {
      if (cudaFuncSetAttribute(adi_factor_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, want) !=
              cudaSuccess ||
          cudaFuncSetAttribute(adi_factor_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, want) !=
              cudaSuccess)
         return 0;
      if (cudaFuncSetAttribute(adi_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, want) != cudaSuccess)
         return 0;
   }
   return want;
}

void launch_adi_assemble(const DeviceState& d, cudaStream_t st)
{
   const int n = std::max(48 * d.nRow, d.sched_nctr);
   adi_assemble_kernel<<<(n + 255) / 256, 256, 0, st>>>(d);
}

void launch_adi_factor(const DeviceState& d, int nwarps, cudaStream_t st)
{
   const int wpb = d.adi_fwpb;
   if (nwarps <= 0) return;
   if (d.piv_soft) adi_factor_kernel<true><<<(nwarps + wpb - 1) / wpb, 32 * wpb, d.exclusive_smem, st>>>(d, nwarps);
   else adi_factor_kernel<false><<<(nwarps + wpb - 1) / wpb, 32 * wpb, d.exclusive_smem, st>>>(d, nwarps);
}

void launch_adi_solve(const DeviceState& d, int sweep, int wave, int nwarps, cudaStream_t st)
{
   const int wpb = d.adi_wpb;
   if (nwarps > 0)
      adi_solve_kernel<<<(nwarps + wpb - 1) / wpb, 32 * wpb, d.exclusive_smem, st>>>(d, sweep, wave, nwarps);
}

}  // namespace hamstr
