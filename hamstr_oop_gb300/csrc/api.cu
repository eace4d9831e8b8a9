// ##################################################################
//
// api.cu -- the device solver handle and its C ABI (include/hamstr_gpu.h)
//
// A pseudo-time step (march.cpp:381-386) is the launch sequence
//   rhs_face(J) rhs_cell(+ADI init) norm  adi_factor
//   msweep x { adi_solve per wave, dq += r, lin_face, lin_cell, [norm] }
//   step_end
// captured once into a CUDA graph and replayed; the last lin_cell also
// applies q += dq.  Every kernel returns at once when a march's stop flag
// is up, so a run of captured steps ends exactly at the converged step.
// ##################################################################
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/hamstr_gpu.h"
#include "api_internal.h"
#include "device_state.h"
#include "plan.h"

using namespace hamstr;

namespace {

thread_local std::string g_last_error;

void set_error(const std::string& m) { g_last_error = m; }

}  // namespace

namespace hamstr {
void set_last_error(const std::string& m) { set_error(m); }
}  // namespace hamstr

namespace {

#define CK(call)                                                                        \
   do {                                                                                 \
      cudaError_t e_ = (call);                                                          \
      if (e_ != cudaSuccess) {                                                          \
         set_error(std::string(#call) + ": " + cudaGetErrorString(e_));                 \
         return HAMSTR_GPU_ERR_CUDA;                                                    \
      }                                                                                 \
   } while (0)

template <typename T>
int dalloc(T** p, size_t n, std::vector<void*>& owned)
{
   *p = nullptr;
   if (n == 0) n = 1;
   cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
   if (e != cudaSuccess) {
      set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
      return e == cudaErrorMemoryAllocation ? HAMSTR_GPU_ERR_NOMEM : HAMSTR_GPU_ERR_CUDA;
   }
   owned.push_back((void*)*p);
   return HAMSTR_GPU_OK;
}

template <typename T>
int upload(T** p, const std::vector<T>& v, std::vector<void*>& owned)
{
   int st = dalloc(p, v.size(), owned);
   if (st) return st;
   if (!v.empty()) CK(cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
   return HAMSTR_GPU_OK;
}

// upload in place of an array this handle owns (freed first)
template <typename T>
int reupload(T** p, const std::vector<T>& v, std::vector<void*>& owned)
{
   for (size_t i = 0; i < owned.size(); i++)
      if (owned[i] == (void*)*p) {
         cudaFree(*p);
         owned.erase(owned.begin() + (long)i);
         break;
      }
   return upload(p, v, owned);
}

}  // namespace

struct hamstr_gpu {
   DeviceState d{};
   Plan plan;
   Schedule sched;
   int msweep = 1;
   cudaStream_t stream = nullptr;
   cudaStream_t stream2 = nullptr;      // side stream: parallel branches of the FP32 step
   cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
   std::vector<void*> owned;
   cudaGraphExec_t step_exec = nullptr;
   cudaGraph_t step_graph = nullptr;
   int launches_per_step = 0;
   double tol_host = 0.0;   // staging for the async copy into d.tol
   int mixed = 0;           // 0: FP64 drop-in, 1: FP32 operator defect correction

   // wall faces (right cell tagged -2), ascending face id: the force integral
   std::vector<int> wall_face, wall_n1, wall_n2;
   std::vector<double> wall_normal;     // [nWall][2]
   int* wall_cell = nullptr;            // device: adjacent cell per wall face
   int* wall0 = nullptr;                // device: [nInst+1] first wall face of each instance
   double4* wall_geo = nullptr;         // device: nx, ny, midpoint x, y (after set_geometry)
   double* wall_scr = nullptr;          // device: 3 per wall face + 3 sums per instance

   int nsm = 1;                         // SMs of the device (persistent-warp schedules)
   int adi_lanes = 4;                   // lanes per open chain in the FP64 line kernels: 32, 16 or 4
   int adi_bundle = 0;                  // open chains of up to this many rows one per lane (0: none)
   int adi_fuse = 1;                    // first wave's first-sweep solve inside the factorisation kernel
   // order 5, FP64: the WENO linearisation's f-only values kept from the
   // implicit computeRHS for the sweeps (d.wlin points here when on)
   double* wlin_buf = nullptr;
   int weno_keep = 1;
   int mx_chunk = 1;                    // FP32 solve: rows loaded in chunks where a wave's chains all fit
   std::vector<int> sp_wave_ptr;        // segmented FP32 solve: spike chains of each wave (host copy)
   bool wlin_valid = false;             // kept values match the current q (standalone entry points)

   // instances (a plain handle has one)
   std::vector<int> inst_cell0;         // [nInst+1]
   std::vector<double> inst_free;       // [nInst][4]: rinf uinf vinf einf

   // optional per-launch timing (hamstr_gpu_profile_step)
   std::vector<std::pair<const char*, std::pair<cudaEvent_t, cudaEvent_t>>>* prof = nullptr;
   template <class F>
   void L(const char* name, int& n, F&& launch)
   {
      cudaEvent_t a = nullptr, b = nullptr;
      if (prof) {
         cudaEventCreate(&a);
         cudaEventCreate(&b);
         cudaEventRecord(a, stream);
      }
      launch();
      n++;
      if (prof) {
         cudaEventRecord(b, stream);
         prof->push_back({name, {a, b}});
      }
   }

   // one pseudo-time step of the mixed-precision form
   int enqueue_mixed_step(bool check_tol)
   {
      int n = 0;
      if (d.recon == 5) L("recon5", n, [&] { launch_recon5(d, false, stream); });
      L("mx_rhs_face", n, [&] { launch_mx_rhs_face(d, stream); });
      L("rhs_cell", n, [&] { launch_rhs_cell(d, true, stream); });
      L("norm_final", n, [&] { launch_norm_final(d, 0, check_tol, stream); });
      L("mx_init", n, [&] { launch_mx_init(d, stream); });
      // the segmented chains' kernels touch no chain of the others and no
      // cell of another chain of their wave, so they run beside them on the
      // side stream (a parallel branch of the captured graph); per-kernel
      // timing keeps them in line
      const bool side = d.sp_on && d.nSpike > 0 && !prof;
      cudaStream_t sst = side ? stream2 : stream;
      if (side) {
         CK(cudaEventRecord(ev_fork, stream));
         CK(cudaStreamWaitEvent(stream2, ev_fork, 0));
      }
      if (d.sp_on && d.nSpike > 0) L("mx_spike_factor", n, [&] { launch_mx_spike_factor(d, sst); });
      if (!d.mx_fused) L("mx_assemble", n, [&] { launch_mx_assemble(d, stream); });
      L("mx_factor", n, [&] { launch_mx_factor(d, stream); });
      for (int s = 0; s < msweep; s++) {
         for (int w = 0; w < plan.nWave; w++) {
            const int c0 = sp_wave_ptr[w], cnt = sp_wave_ptr[w + 1] - c0;
            if (side && (s > 0 || w > 0) && cnt > 0) {
               CK(cudaEventRecord(ev_fork, stream));
               CK(cudaStreamWaitEvent(stream2, ev_fork, 0));
            }
            if (d.sp_on && cnt > 0) L("mx_spike_solve", n, [&] { launch_mx_spike_solve(d, c0, cnt, sst); });
            L("mx_solve", n, [&] { launch_mx_solve(d, plan.wave_ptr[w], plan.wave_ptr[w + 1] - plan.wave_ptr[w], stream); });
            if (side && (cnt > 0 || (s == 0 && w == 0))) {
               CK(cudaEventRecord(ev_join, stream2));
               CK(cudaStreamWaitEvent(stream, ev_join, 0));
            }
         }
         L("mx_dq_update", n, [&] { launch_mx_dq_update(d, stream); });
         L("mx_lin_face", n, [&] { launch_mx_lin_face(d, stream); });
         L("mx_lin_cell", n, [&] { launch_mx_lin_cell(d, s == msweep - 1, stream); });
         if (s == msweep - 1) L("norm_final", n, [&] { launch_norm_final(d, 2, false, stream); });
      }
      L("step_end", n, [&] { launch_step_end(d, stream); });
      launches_per_step = n;
      CK(cudaGetLastError());
      return HAMSTR_GPU_OK;
   }

   // allocate the FP32 buffers of the mixed form on first use
   int ensure_mixed_buffers()
   {
      if (d.ff32) return HAMSTR_GPU_OK;
      const size_t nc = (size_t)d.nCell;
      int st;
      if (mx_configure()) {
         set_error("FP32 factorisation: shared-memory attribute refused");
         return HAMSTR_GPU_ERR_CUDA;
      }
      if ((st = dalloc(&d.ff32, 32 * (size_t)d.nSlot, owned))) return st;
      // chains of each wave ordered longest first, so a warp's threads
      // (one chain each) run for similar lengths; the same order tiles the
      // FP32 line data (DeviceState)
      std::vector<int> lc(plan.wave_chains);
      for (int w = 0; w < plan.nWave; w++)
         std::stable_sort(lc.begin() + plan.wave_ptr[w], lc.begin() + plan.wave_ptr[w + 1],
                          [&](int a, int b) { return plan.chain_nrows[a] > plan.chain_nrows[b]; });
      if ((st = upload(&d.line_chains, lc, owned))) return st;
      const int ngrp = (plan.nChain + 31) / 32;
      std::vector<int> grp_row0(ngrp + 1, 0);
      for (int g = 0; g < ngrp; g++) {
         int len = 0;
         for (int p = 32 * g; p < std::min(32 * g + 32, plan.nChain); p++) len = std::max(len, plan.chain_nrows[lc[p]]);
         grp_row0[g + 1] = grp_row0[g] + len;
      }
      d.tile_rows = grp_row0[ngrp];
      std::vector<int> tile_row(32 * (size_t)std::max(d.tile_rows, 1), -1);
      for (int p = 0; p < plan.nChain; p++) {
         const int c = lc[p];
         for (int i = 0; i < plan.chain_nrows[c]; i++)
            tile_row[32 * (size_t)(grp_row0[p >> 5] + i) + (p & 31)] = plan.chain_row0[c] + i;
      }
      if ((st = upload(&d.grp_row0, grp_row0, owned))) return st;
      if ((st = upload(&d.tile_row, tile_row, owned))) return st;
      const size_t tiles = 32 * (size_t)std::max(d.tile_rows, 1);
      if (!d.mx_fused && (st = ensure_blk32())) return st;
      if ((st = dalloc(&d.fsc32, 4 * tiles, owned))) return st;
      if ((st = dalloc(&d.fac32, 80 * tiles, owned))) return st;
      int nper = 0;
      for (int c = 0; c < plan.nChain; c++) nper += plan.chain_periodic[c] ? 1 : 0;
      if ((st = dalloc(&d.facN32, 16 * (size_t)std::max(nper, 1), owned))) return st;
      if ((st = dalloc(&d.r32, 4 * nc, owned))) return st;
      if ((st = dalloc(&d.r032, 4 * nc, owned))) return st;
      if ((st = dalloc(&d.dq32, 4 * nc, owned))) return st;
      if ((st = dalloc(&d.g32, 4 * (size_t)d.nSlot, owned))) return st;
      // long chains take the segmented solve: P segments of about
      // kSpikeRows rows each (at most kSpikeMaxSeg), grouped by wave; their
      // rows are tiled across the segments (sp_rec0 in tile rows)
      {
         std::vector<int> chain_spike(std::max(plan.nChain, 1), -1), sp_chain, sp_seg, sp_nseg, sp_rec0;
         sp_wave_ptr.assign(plan.nWave + 1, 0);
         int rows = 0;
         for (int w = 0; w < plan.nWave; w++) {
            for (int k = plan.wave_ptr[w]; k < plan.wave_ptr[w + 1]; k++) {
               const int c = plan.wave_chains[k];
               const int n = plan.chain_nrows[c];
               if (n < (plan.chain_periodic[c] ? kSpikeMinRows : kSpikeMinOpenRows)) continue;
               const int P = std::min(kSpikeMaxSeg, n / kSpikeRows);
               chain_spike[c] = (int)sp_chain.size();
               sp_chain.push_back(c);
               sp_nseg.push_back(P);
               sp_rec0.push_back(rows);
               int longest = 0;
               for (int p = 0; p <= kSpikeMaxSeg; p++) {
                  sp_seg.push_back(p <= P ? (int)((long long)p * n / P) : n);
                  if (p >= 1 && p <= P) longest = std::max(longest, sp_seg.back() - sp_seg[sp_seg.size() - 2]);
               }
               rows += longest;   // tile rows: local row k of every segment in one
            }
            sp_wave_ptr[w + 1] = (int)sp_chain.size();
         }
         d.nSpike = (int)sp_chain.size();
         if (sp_chain.empty()) {
            sp_chain.push_back(0);
            sp_nseg.push_back(0);
            sp_rec0.push_back(0);
            sp_seg.assign(kSpikeMaxSeg + 1, 0);
         }
         if ((st = upload(&d.chain_spike, chain_spike, owned))) return st;
         if ((st = upload(&d.sp_chain, sp_chain, owned))) return st;
         if ((st = upload(&d.sp_seg, sp_seg, owned))) return st;
         if ((st = upload(&d.sp_nseg, sp_nseg, owned))) return st;
         if ((st = upload(&d.sp_rec0, sp_rec0, owned))) return st;
         if ((st = dalloc(&d.sp_fac, 80 * 32 * (size_t)std::max(rows, 1), owned))) return st;
         if ((st = dalloc(&d.sp_y, 4 * 32 * (size_t)std::max(rows, 1), owned))) return st;
         if ((st = dalloc(&d.sp_red, (size_t)kSpikeRedStride * std::max(d.nSpike, 1), owned))) return st;
      }
      CK(cudaMemsetAsync(d.ff32, 0, 32 * (size_t)d.nSlot * sizeof(float), stream));
      CK(cudaMemsetAsync(d.dq32, 0, 4 * nc * sizeof(float), stream));
      return HAMSTR_GPU_OK;
   }

   // one pseudo-time step on `stream` (graph body)
   int enqueue_step(bool check_tol)
   {
      if (mixed) return enqueue_mixed_step(check_tol);
      int n = 0;
      if (d.recon == 5) L("recon5", n, [&] { launch_recon5(d, d.lin_order != 1, stream); });
      L("rhs_face", n, [&] { launch_rhs_face(d, true, stream); });
      L("rhs_cell", n, [&] { launch_rhs_cell(d, true, stream); });
      L("norm_final", n, [&] { launch_norm_final(d, 0, check_tol, stream); });
      L("adi_assemble", n, [&] { launch_adi_assemble(d, stream); });
      adi_factor_launches(n);
      for (int s = 0; s < msweep; s++) {
         for (int w = 0; w < plan.nWave; w++)
            if (!(adi_fuse && s == 0 && w == 0)) adi_solve_launches(s, w, n);   // fused: done by adi_factor
         L("dq_update", n, [&] { launch_dq_update(d, stream); });
         if (d.recon == 5 && d.lin_order != 1) L("lin_recon5", n, [&] { launch_lin_recon5(d, true, stream); });
         L("lin_face", n, [&] { launch_lin_face(d, stream); });
         L("lin_cell", n, [&] { launch_lin_cell(d, s == msweep - 1, stream); });
         if (s == msweep - 1) L("norm_final", n, [&] { launch_norm_final(d, 2, false, stream); });
      }
      L("step_end", n, [&] { launch_step_end(d, stream); });
      launches_per_step = n;
      CK(cudaGetLastError());
      return HAMSTR_GPU_OK;
   }

   int ensure_blk32()
   {
      if (d.blk32) return HAMSTR_GPU_OK;
      return dalloc(&d.blk32, 48 * 32 * (size_t)std::max(d.tile_rows, 1), owned);
   }

   // drop the captured step (launch shapes or constants changed)
   void invalidate()
   {
      if (step_exec) cudaGraphExecDestroy(step_exec);
      if (step_graph) cudaGraphDestroy(step_graph);
      step_exec = nullptr;
      step_graph = nullptr;
      launches_per_step = 0;
   }

   // launch shapes; a new warps-per-SM count rebuilds the line schedules
   int ensure_wlin()
   {
      if (wlin_buf) return HAMSTR_GPU_OK;
      return dalloc(&wlin_buf, kWlinPerSlot * (size_t)std::max(d.nSlot, 1), owned);
   }

   int upload_schedule()
   {
      int st;
      if ((st = reupload(&d.sched_job0, sched.job0, owned))) return st;
      if ((st = reupload(&d.sched_njobs, sched.njobs, owned))) return st;
      if ((st = reupload(&d.sched_job_ptr, sched.job_ptr, owned))) return st;
      if ((st = reupload(&d.sched_ncrit, sched.ncrit, owned))) return st;
      return reupload(&d.sched_jobs, sched.jobs, owned);
   }

   // the FP64 line kernels of one schedule (0: factorisation, 1 + w: the
   // solve of wave w)
   void adi_factor_launches(int& n)
   {
      if (sched.nwarps[0] > 0) L("adi_factor", n, [&] { launch_adi_factor(d, sched.nwarps[0], stream); });
   }
   void adi_solve_launches(int s, int w, int& n)
   {
      if (sched.nwarps[1 + w] > 0) L("adi_solve", n, [&] { launch_adi_solve(d, s, w, sched.nwarps[1 + w], stream); });
   }

   int apply_shape(int face_block, int adi_wpb, int mx_block, int mx_fused, int face_soft, int piv_soft, int lanes,
                   int wkeep, int bundle, int chunk, int spike, int fuse, int adi_fwpb)
   {
      d.sp_on = spike;
      if (wkeep && d.recon == 5) {
         const int st = ensure_wlin();
         if (st) return st;
         d.wlin = wlin_buf;
      } else {
         d.wlin = nullptr;
      }
      weno_keep = wkeep;
      wlin_valid = false;
      d.face_soft = face_soft;
      d.piv_soft = piv_soft;
      if (!mx_fused && d.ff32) {
         const int st = ensure_blk32();
         if (st) return st;
      }
      d.mx_fused = mx_fused;
      if (adi_wpb != d.adi_wpb || adi_fwpb != d.adi_fwpb || lanes != adi_lanes || bundle != adi_bundle ||
          fuse != adi_fuse) {
         adi_lanes = lanes;
         adi_bundle = bundle;
         adi_fuse = fuse;
         sched = build_schedule(plan, adi_wpb * nsm, lanes, bundle, fuse != 0, adi_fwpb * nsm, nsm);
         const int st = upload_schedule();
         if (st) return st;
      }
      d.face_block = face_block;
      d.adi_wpb = adi_wpb;
      d.adi_fwpb = adi_fwpb;
      d.mx_block = mx_block;
      mx_chunk = chunk;
      d.mx_chunk_chains = chunk ? mx_solve_chunk_capacity(mx_block) : 0;
      invalidate();
      return HAMSTR_GPU_OK;
   }

   int capture()
   {
      if (step_exec) return HAMSTR_GPU_OK;
      CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
      int st = enqueue_step(true);
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamEndCapture(stream, &g);
      if (st) return st;
      if (e != cudaSuccess) {
         set_error(std::string("graph capture: ") + cudaGetErrorString(e));
         return HAMSTR_GPU_ERR_CUDA;
      }
      step_graph = g;
      CK(cudaGraphInstantiate(&step_exec, step_graph, 0));
      return HAMSTR_GPU_OK;
   }

   int reset_ctl(double tol)
   {
      CK(cudaMemsetAsync(d.ctl, 0, 2 * sizeof(int), stream));
      CK(cudaMemsetAsync(d.inst_done, 0, (size_t)d.nInst * sizeof(int), stream));
      if (tol != tol_host) {
         tol_host = tol;
         CK(cudaMemcpyAsync(d.tol, &tol_host, sizeof(double), cudaMemcpyHostToDevice, stream));
      }
      return HAMSTR_GPU_OK;
   }

   int status_check()
   {
      int s = 0;
      CK(cudaMemcpyAsync(&s, d.status, sizeof(int), cudaMemcpyDeviceToHost, stream));
      CK(cudaStreamSynchronize(stream));
      if (!s) return HAMSTR_GPU_OK;
      CK(cudaMemsetAsync(d.status, 0, sizeof(int), stream));
      // the first failure of a step in its order: flux, factorisation, sweep
      if (s & DEV_ERR_NAN_SPEC) {
         set_error("NaN spectral radius (non-physical state)");
         return HAMSTR_GPU_ERR_NAN;
      }
      if (s & DEV_ERR_PIVOT) {
         set_error("zero or non-finite LU pivot in an ADI line factorisation");
         return HAMSTR_GPU_ERR_SINGULAR;
      }
      if (s & DEV_ERR_WAIT) {
         set_error("an ADI line solve gave up waiting for its factorisation");
         return HAMSTR_GPU_ERR_CUDA;
      }
      set_error("non-finite dq after an ADI sweep");
      return HAMSTR_GPU_ERR_NONFINITE;
   }

   int read_norms(double* out, int n)
   {
      CK(cudaMemcpyAsync(out, d.norms, n * sizeof(double), cudaMemcpyDeviceToHost, stream));
      return status_check();
   }
};

extern "C" {

const char* hamstr_gpu_strerror(int st)
{
   switch (st) {
      case HAMSTR_GPU_OK: return "ok";
      case HAMSTR_GPU_ERR_ARG: return "invalid argument";
      case HAMSTR_GPU_ERR_TOPOLOGY: return "mesh/chain topology not supported";
      case HAMSTR_GPU_ERR_CUDA: return "CUDA error";
      case HAMSTR_GPU_ERR_NAN: return "NaN spectral radius";
      case HAMSTR_GPU_ERR_IO: return "missing or malformed input file";
      case HAMSTR_GPU_ERR_NOMEM: return "out of memory";
      case HAMSTR_GPU_ERR_SINGULAR: return "singular ADI block pivot";
      case HAMSTR_GPU_ERR_NONFINITE: return "non-finite ADI update";
      default: return "unknown status";
   }
}

const char* hamstr_gpu_last_error(void) { return g_last_error.c_str(); }

int hamstr_gpu_create(const hamstr_gpu_params* p, int nCell, int nFace, const int* faces, const double* normVec,
                      const double* refMtx, int nChain, const int* faceStartPerChain, const int* chainConn,
                      hamstr_gpu** out)
{
   return hamstr::create_gpu(p, nCell, nFace, faces, normVec, refMtx, nChain, faceStartPerChain, chainConn, nullptr,
                             out);
}

}  // extern "C"

int hamstr::create_gpu(const hamstr_gpu_params* p, int nCell, int nFace, const int* faces, const double* normVec,
                       const double* refMtx, int nChain, const int* faceStartPerChain, const int* chainConn,
                       const InstanceInfo* inst, hamstr_gpu** out)
{
   if (!p || !faces || !normVec || !refMtx || !faceStartPerChain || !chainConn || !out) return HAMSTR_GPU_ERR_ARG;
   *out = nullptr;
   if (p->msweep < 1 || !(p->CFL > 0.0)) {
      set_error("msweep must be >= 1 and CFL > 0");
      return HAMSTR_GPU_ERR_ARG;
   }
   if (p->limiter < HAMSTR_LIMITER_REFERENCE || p->limiter > HAMSTR_LIMITER_VANALBADA) {
      set_error("unknown limiter");
      return HAMSTR_GPU_ERR_ARG;
   }
   MeshInput in;
   in.nCell = nCell;
   in.nFace = nFace;
   in.nChain = nChain;
   in.nChainFace = faceStartPerChain[nChain];
   in.order = p->order;
   in.end_rule = p->chain_end_rule;
   in.faces = faces;
   in.faceStartPerChain = faceStartPerChain;
   in.chainConn = chainConn;
   hamstr_gpu* g = new hamstr_gpu;
   std::string msg;
   try {
      msg = build_plan(in, g->plan);
   } catch (const std::bad_alloc&) {
      delete g;
      return HAMSTR_GPU_ERR_NOMEM;
   }
   if (!msg.empty()) {
      set_error(msg);
      delete g;
      return HAMSTR_GPU_ERR_TOPOLOGY;
   }
   const Plan& P = g->plan;
   DeviceState& d = g->d;
   d.nCell = nCell;
   d.nFace = nFace;
   d.nSlot = P.nSlot;
   d.nSten = P.nSten;
   d.nRow = P.nRow;
   d.nChain = P.nChain;
   d.order = P.order;
   d.recon = (P.order == 3 && p->limiter != HAMSTR_LIMITER_REFERENCE) ? 30 + p->limiter : P.order;
   d.lin_order = 0;
   d.nGhost = P.nGhost;
   d.fc.gamma = p->gamma;
   d.fc.rinf = p->rinf;
   d.fc.uinf = p->uinf;
   d.fc.vinf = p->vinf;
   d.fc.einf = p->einf;
   d.fc.cfl = p->CFL;
   g->msweep = p->msweep;

   // instances: cell and chain ranges, freestream per instance
   InstanceInfo one;
   if (!inst) {
      one.cell0 = {0, nCell};
      one.chain0 = {0, nChain};
      one.freestream = {p->rinf, p->uinf, p->vinf, p->einf};
      inst = &one;
   }
   const int ni = inst->n;
   if (ni < 1 || (int)inst->cell0.size() != ni + 1 || (int)inst->chain0.size() != ni + 1 ||
       (int)inst->freestream.size() != 4 * ni || inst->cell0[0] != 0 || inst->cell0[ni] != nCell ||
       inst->chain0[0] != 0 || inst->chain0[ni] != nChain) {
      set_error("inconsistent instance ranges");
      delete g;
      return HAMSTR_GPU_ERR_ARG;
   }
   d.nInst = ni;
   g->inst_cell0 = inst->cell0;
   g->inst_free = inst->freestream;
   std::vector<double4> fstab(ni);
   for (int k = 0; k < ni; k++) {
      const double* f = &inst->freestream[4 * (size_t)k];
      // computeRHS.cpp:247-250: rinf, rinf*uinf, rinf*vinf, einf
      fstab[k] = make_double4(f[0], f[0] * f[1], f[0] * f[2], f[3]);
   }
   std::vector<int> chain_inst(nChain);
   for (int k = 0; k < ni; k++)
      for (int c = inst->chain0[k]; c < inst->chain0[k + 1]; c++) chain_inst[c] = k;
   std::vector<int2> cell_blocks;
   std::vector<int> inst_block0(1, 0), inst_ncell(ni);
   for (int k = 0; k < ni; k++) {
      for (int c = inst->cell0[k]; c < inst->cell0[k + 1]; c += kNormBlock)
         cell_blocks.push_back(make_int2(c, std::min(c + kNormBlock, inst->cell0[k + 1])));
      inst_block0.push_back((int)cell_blocks.size());
      inst_ncell[k] = inst->cell0[k + 1] - inst->cell0[k];
   }

   // host-side packing
   // stencil entries carry their chain's instance (the freestream to use)
   std::vector<int4> sten(P.nSten);
   for (int c = 0; c < P.nChain; c++) {
      const int e1 = (c + 1 < P.nChain) ? P.chain_sten0[c + 1] : P.nSten;
      for (int i = P.chain_sten0[c]; i < e1; i++)
         sten[i] = make_int4(P.sten_cell[i], P.sten_kind[i], P.sten_face[i], chain_inst[c]);
   }
   std::vector<int4> slot(P.nSlot);
   std::vector<double2> normal(P.nSlot);
   for (int s = 0; s < P.nSlot; s++) {
      slot[s] = make_int4(P.slot_n[s], P.slot_left[s], P.slot_right[s], P.slot_swap[s] | (P.slot_owner[s] << 1));
      normal[s] = make_double2(normVec[2 * (size_t)P.slot_face[s]], normVec[2 * (size_t)P.slot_face[s] + 1]);
   }
   std::vector<double4> refl(nFace);
   for (int f = 0; f < nFace; f++)
      refl[f] = make_double4(refMtx[4 * (size_t)f], refMtx[4 * (size_t)f + 1], refMtx[4 * (size_t)f + 2],
                             refMtx[4 * (size_t)f + 3]);
   std::vector<int> chain_facN(P.nChain, -1);
   int nper = 0;
   for (int c = 0; c < P.nChain; c++)
      if (P.chain_periodic[c]) chain_facN[c] = nper++;
   std::vector<int> cell_written(P.cell_last_wave_writer);
   std::vector<int> wall_cell, wall0(ni + 1, 0);
   for (int f = 0; f < nFace; f++) {
      if (faces[6 * (size_t)f + 4] != -2) continue;
      // instance of the adjacent cell (faces come instance after instance)
      const int lc = faces[6 * (size_t)f + 2];
      int k = (int)(std::upper_bound(inst->cell0.begin(), inst->cell0.end(), lc) - inst->cell0.begin()) - 1;
      wall0[k + 1]++;
      g->wall_face.push_back(f);
      g->wall_n1.push_back(faces[6 * (size_t)f]);
      g->wall_n2.push_back(faces[6 * (size_t)f + 1]);
      g->wall_normal.push_back(normVec[2 * (size_t)f]);
      g->wall_normal.push_back(normVec[2 * (size_t)f + 1]);
      wall_cell.push_back(faces[6 * (size_t)f + 2]);
   }

   int st = HAMSTR_GPU_OK;
   auto& o = g->owned;
   const size_t nc = (size_t)nCell;
#define TRY(x)                          \
   do {                                 \
      st = (x);                         \
      if (st) {                         \
         hamstr_gpu_destroy(g);         \
         return st;                     \
      }                                 \
   } while (0)
   TRY(dalloc(&d.q, 4 * nc, o));
   TRY(dalloc(&d.r, 4 * nc, o));
   TRY(dalloc(&d.qt, 4 * nc, o));
   TRY(dalloc(&d.r0, 4 * nc, o));
   TRY(dalloc(&d.dq, 4 * nc, o));
   TRY(dalloc(&d.sigma, nc, o));
   TRY(dalloc(&d.dtfac, nc, o));
   TRY(dalloc(&d.flux, 4 * (size_t)P.nSlot, o));
   TRY(dalloc(&d.spec, (size_t)P.nSlot, o));
   TRY(dalloc(&d.ff, 32 * (size_t)P.nSlot, o));
   if (d.recon == 5) {
      TRY(dalloc(&d.qface, 8 * (size_t)P.nSlot, o));
      TRY(g->ensure_wlin());
      d.wlin = g->wlin_buf;
   }
   TRY(upload(&d.sten, sten, o));
   TRY(upload(&d.slot, slot, o));
   TRY(upload(&d.slot_face, P.slot_face, o));
   TRY(upload(&d.normal, normal, o));
   TRY(upload(&d.refl, refl, o));
   TRY(upload(&d.cell_ptr, P.cell_ptr, o));
   TRY(upload(&d.cell_ent, P.cell_ent, o));
   TRY(upload(&d.chain_periodic, P.chain_periodic, o));
   TRY(upload(&d.chain_nrows, P.chain_nrows, o));
   TRY(upload(&d.chain_row0, P.chain_row0, o));
   TRY(upload(&d.wave_chains, P.wave_chains, o));
   TRY(upload(&d.row_scell, P.row_scell, o));
   TRY(upload(&d.row_fcell, P.row_fcell, o));
   TRY(upload(&d.row_ops, P.row_ops, o));
   TRY(upload(&d.cell_written, cell_written, o));
   TRY(upload(&d.chain_facN, chain_facN, o));
   {
      int dev = 0, nsm = 0, optin = 0;
      cudaGetDevice(&dev);
      if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0) nsm = 1;
      if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) optin = 0;
      d.exclusive_smem = adi_configure(optin);
      d.face_block = 256;
      d.adi_wpb = 4;
      d.adi_fwpb = 4;
      d.mx_block = 64;
      d.mx_chunk_chains = mx_solve_chunk_capacity(d.mx_block);
      d.sp_on = 1;   // long periodic chains of the FP32 form by segments (2: long open ones too)
      // FP32 assembly inside the factorisation pays off on long chains, as
      // do the hardware pivot divisions (their latency is shorter per row)
      d.mx_fused = (P.nChain > 0 && P.nRow >= 16 * P.nChain) ? 1 : 0;
      d.face_soft = 1;
      d.piv_soft = d.mx_fused ? 0 : 1;
      g->nsm = nsm;
      // the shortest open chains one per lane where chains are short (the
      // autotuner checks the alternatives)
      g->adi_bundle = (P.nChain > 0 && P.nRow < 16 * P.nChain) ? 8 : 0;
      g->sched = build_schedule(P, d.adi_wpb * nsm, g->adi_lanes, g->adi_bundle, g->adi_fuse != 0, d.adi_fwpb * nsm,
                                nsm);
   }
   TRY(g->upload_schedule());
   d.nWave = P.nWave;
   d.sched_nctr = 1 + g->msweep * P.nWave;
   TRY(dalloc(&d.sched_ctr, (size_t)d.sched_nctr, o));
   TRY(dalloc(&d.blk, 48 * (size_t)std::max(P.nRow, 1), o));
   TRY(dalloc(&d.fac, 80 * (size_t)std::max(P.nRow, 1), o));
   TRY(dalloc(&d.fsc, 4 * (size_t)std::max(P.nRow, 1), o));
   TRY(dalloc(&d.facN, 16 * (size_t)std::max(nper, 1), o));
   d.norm_blocks = (int)cell_blocks.size();
   TRY(dalloc(&d.norm_part, (size_t)d.norm_blocks, o));
   TRY(upload(&d.cell_blocks, cell_blocks, o));
   TRY(upload(&d.inst_block0, inst_block0, o));
   TRY(upload(&d.inst_ncell, inst_ncell, o));
   TRY(upload(&d.fstab, fstab, o));
   {
      std::vector<int> slot_inst(P.nSlot), cell_inst(nCell), block_inst(cell_blocks.size());
      for (int k = 0; k < ni; k++)
         for (int c = inst->cell0[k]; c < inst->cell0[k + 1]; c++) cell_inst[c] = k;
      for (int s = 0; s < P.nSlot; s++) slot_inst[s] = cell_inst[P.slot_left[s]];
      for (size_t b = 0; b < cell_blocks.size(); b++) block_inst[b] = cell_inst[cell_blocks[b].x];
      TRY(upload(&d.slot_inst, slot_inst, o));
      TRY(upload(&d.cell_inst, cell_inst, o));
      TRY(upload(&d.chain_inst, chain_inst, o));
      TRY(upload(&d.block_inst, block_inst, o));
      TRY(dalloc(&d.inst_done, (size_t)ni, o));
   }
   TRY(dalloc(&d.norms, 4 * (size_t)ni, o));
   TRY(dalloc(&d.status, 1, o));
   TRY(dalloc(&d.ctl, 2, o));
   TRY(dalloc(&d.tol, 1, o));
   d.hist_cap = std::min(1 << 16, std::max(1024, (1 << 22) / ni));
   TRY(dalloc(&d.hist, 4 * (size_t)d.hist_cap * ni, o));
   for (int k = 0; k < ni; k++) wall0[k + 1] += wall0[k];
   TRY(upload(&g->wall_cell, wall_cell, o));
   TRY(upload(&g->wall0, wall0, o));
   TRY(dalloc(&g->wall_scr, 3 * wall_cell.size() + 3 * (size_t)ni, o));
#undef TRY
   cudaError_t e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
   if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g->stream2, cudaStreamNonBlocking);
   if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->ev_fork, cudaEventDisableTiming);
   if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->ev_join, cudaEventDisableTiming);
   if (e != cudaSuccess) {
      set_error(cudaGetErrorString(e));
      hamstr_gpu_destroy(g);
      return HAMSTR_GPU_ERR_CUDA;
   }
   e = cudaMemsetAsync(d.status, 0, sizeof(int), g->stream);
   if (e == cudaSuccess) e = cudaMemsetAsync(d.ctl, 0, 2 * sizeof(int), g->stream);
   if (e == cudaSuccess) e = cudaMemsetAsync(d.tol, 0, sizeof(double), g->stream);
   if (e == cudaSuccess) e = cudaMemsetAsync(d.ff, 0, 32 * (size_t)P.nSlot * sizeof(double), g->stream);
   if (e == cudaSuccess) e = cudaMemsetAsync(d.dq, 0, 4 * nc * sizeof(double), g->stream);
   if (e == cudaSuccess) e = cudaMemsetAsync(d.r, 0, 4 * nc * sizeof(double), g->stream);
   if (e == cudaSuccess) e = cudaMemsetAsync(d.r0, 0, 4 * nc * sizeof(double), g->stream);
   if (e == cudaSuccess) e = cudaMemsetAsync(d.sigma, 0, nc * sizeof(double), g->stream);
   if (e == cudaSuccess) {
      // freestream initial state (initFlow.cpp:67-91), per instance
      std::vector<double> q(4 * nc);
      for (int k = 0; k < ni; k++) {
         const double* f = &inst->freestream[4 * (size_t)k];
         for (size_t i = (size_t)inst->cell0[k]; i < (size_t)inst->cell0[k + 1]; i++) {
            q[4 * i] = f[0];
            q[4 * i + 1] = f[0] * f[1];
            q[4 * i + 2] = f[0] * f[2];
            q[4 * i + 3] = f[3];
         }
      }
      e = cudaMemcpy(d.q, q.data(), q.size() * sizeof(double), cudaMemcpyHostToDevice);
      if (e == cudaSuccess) e = cudaMemcpy(d.qt, q.data(), q.size() * sizeof(double), cudaMemcpyHostToDevice);
   }
   if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
   if (e != cudaSuccess) {
      set_error(cudaGetErrorString(e));
      hamstr_gpu_destroy(g);
      return HAMSTR_GPU_ERR_CUDA;
   }
   *out = g;
   return HAMSTR_GPU_OK;
}

extern "C" {

int hamstr_gpu_destroy(hamstr_gpu* g)
{
   if (!g) return HAMSTR_GPU_OK;
   if (g->stream) cudaStreamSynchronize(g->stream);
   if (g->step_exec) cudaGraphExecDestroy(g->step_exec);
   if (g->step_graph) cudaGraphDestroy(g->step_graph);
   if (g->stream2) cudaStreamSynchronize(g->stream2);
   for (void* p : g->owned) cudaFree(p);
   if (g->ev_fork) cudaEventDestroy(g->ev_fork);
   if (g->ev_join) cudaEventDestroy(g->ev_join);
   if (g->stream2) cudaStreamDestroy(g->stream2);
   if (g->stream) cudaStreamDestroy(g->stream);
   delete g;
   return HAMSTR_GPU_OK;
}

int hamstr_gpu_get(hamstr_gpu* g, const char* name, double* out)
{
   if (!g || !name || !out) return HAMSTR_GPU_ERR_ARG;
   const DeviceState& d = g->d;
   const size_t nc = (size_t)d.nCell;
   const double* src = nullptr;
   size_t n = 0;
   if (!std::strcmp(name, "q")) { src = d.q; n = 4 * nc; }
   else if (!std::strcmp(name, "qt")) { src = d.qt; n = 4 * nc; }
   else if (!std::strcmp(name, "r")) { src = d.r; n = 4 * nc; }
   else if (!std::strcmp(name, "r0")) { src = d.r0; n = 4 * nc; }
   else if (!std::strcmp(name, "dq")) { src = d.dq; n = 4 * nc; }
   else if (!std::strcmp(name, "sigma")) { src = d.sigma; n = nc; }
   else if (!std::strcmp(name, "ff")) {
      // per-slot Jacobians to face order (sb->ff[iface], computeRHS.cpp:365-370)
      std::vector<double> slots(32 * (size_t)d.nSlot);
      CK(cudaMemcpyAsync(slots.data(), d.ff, slots.size() * sizeof(double), cudaMemcpyDeviceToHost, g->stream));
      CK(cudaStreamSynchronize(g->stream));
      std::memset(out, 0, 32 * (size_t)d.nFace * sizeof(double));
      for (int s = 0; s < d.nSlot; s++)
         if (g->plan.slot_owner[s] == s)
            std::memcpy(out + 32 * (size_t)g->plan.slot_face[s], slots.data() + 32 * (size_t)s, 32 * sizeof(double));
      return HAMSTR_GPU_OK;
   } else {
      set_error(std::string("unknown array ") + name);
      return HAMSTR_GPU_ERR_ARG;
   }
   CK(cudaMemcpyAsync(out, src, n * sizeof(double), cudaMemcpyDeviceToHost, g->stream));
   CK(cudaStreamSynchronize(g->stream));
   return HAMSTR_GPU_OK;
}

int hamstr_gpu_set(hamstr_gpu* g, const char* name, const double* in)
{
   if (!g || !name || !in) return HAMSTR_GPU_ERR_ARG;
   g->wlin_valid = false;   // q may change: the kept WENO values no longer apply
   DeviceState& d = g->d;
   const size_t nc = (size_t)d.nCell;
   double* dst = nullptr;
   size_t n = 0;
   if (!std::strcmp(name, "q")) { dst = d.q; n = 4 * nc; }
   else if (!std::strcmp(name, "qt")) { dst = d.qt; n = 4 * nc; }
   else if (!std::strcmp(name, "r")) { dst = d.r; n = 4 * nc; }
   else if (!std::strcmp(name, "r0")) { dst = d.r0; n = 4 * nc; }
   else if (!std::strcmp(name, "dq")) { dst = d.dq; n = 4 * nc; }
   else if (!std::strcmp(name, "sigma")) { dst = d.sigma; n = nc; }
   else if (!std::strcmp(name, "ff")) {
      std::vector<double> slots(32 * (size_t)d.nSlot);
      for (int s = 0; s < d.nSlot; s++)
         std::memcpy(slots.data() + 32 * (size_t)s, in + 32 * (size_t)g->plan.slot_face[s], 32 * sizeof(double));
      CK(cudaMemcpyAsync(d.ff, slots.data(), slots.size() * sizeof(double), cudaMemcpyHostToDevice, g->stream));
      CK(cudaStreamSynchronize(g->stream));
      return HAMSTR_GPU_OK;
   } else {
      set_error(std::string("unknown array ") + name);
      return HAMSTR_GPU_ERR_ARG;
   }
   CK(cudaMemcpyAsync(dst, in, n * sizeof(double), cudaMemcpyHostToDevice, g->stream));
   CK(cudaStreamSynchronize(g->stream));
   return HAMSTR_GPU_OK;
}

int hamstr_gpu_compute_rhs(hamstr_gpu* g, int implicit, double* l2, double* linf)
{
   if (!g) return HAMSTR_GPU_ERR_ARG;
   int st = g->reset_ctl(0.0);
   if (st) return st;
   launch_recon5(g->d, implicit != 0, g->stream);
   launch_rhs_face(g->d, implicit != 0, g->stream);
   if (implicit) g->wlin_valid = g->d.wlin != nullptr;
   launch_rhs_cell(g->d, false, g->stream);
   launch_norm_final(g->d, 0, false, g->stream);
   CK(cudaGetLastError());
   double n[2];
   st = g->read_norms(n, 2);
   if (st) return st;
   if (l2) *l2 = n[0];
   if (linf) *linf = n[1];
   return HAMSTR_GPU_OK;
}

int hamstr_gpu_linear_rhs(hamstr_gpu* g, double* l2, double* linf)
{
   if (!g) return HAMSTR_GPU_ERR_ARG;
   int st = g->reset_ctl(0.0);
   if (st) return st;
   launch_dtfac(g->d, g->stream);
   launch_lin_recon5(g->d, g->wlin_valid, g->stream);
   launch_lin_face(g->d, g->stream);
   launch_lin_cell(g->d, false, g->stream);
   launch_norm_final(g->d, 2, false, g->stream);
   CK(cudaGetLastError());
   double n[4];
   st = g->read_norms(n, 4);
   if (st) return st;
   if (l2) *l2 = n[2];
   if (linf) *linf = n[3];
   return HAMSTR_GPU_OK;
}

int hamstr_gpu_adi(hamstr_gpu* g, double* l2, double* linf)
{
   if (!g) return HAMSTR_GPU_ERR_ARG;
   int st = g->reset_ctl(0.0);
   if (st) return st;
   const DeviceState& d = g->d;
   launch_adi_init(d, g->stream);
   launch_adi_assemble(d, g->stream);
   const Schedule& S = g->sched;
   launch_adi_factor(d, S.nwarps[0], g->stream);
   for (int s = 0; s < g->msweep; s++) {
      for (int w = 0; w < g->plan.nWave; w++)
         if (!(g->adi_fuse && s == 0 && w == 0)) launch_adi_solve(d, s, w, S.nwarps[1 + w], g->stream);
      launch_dq_update(d, g->stream);
      launch_lin_recon5(d, g->wlin_valid, g->stream);
      launch_lin_face(d, g->stream);
      launch_lin_cell(d, s == g->msweep - 1, g->stream);
   }
   g->wlin_valid = false;   // q += dq
   launch_norm_final(d, 2, false, g->stream);
   CK(cudaGetLastError());
   double n[4];
   st = g->read_norms(n, 4);
   if (st) return st;
   if (l2) *l2 = n[2];
   if (linf) *linf = n[3];
   return HAMSTR_GPU_OK;
}

int hamstr_gpu_step(hamstr_gpu* g, double* norms4)
{
   if (!g) return HAMSTR_GPU_ERR_ARG;
   g->wlin_valid = false;   // q may change: the kept WENO values no longer apply
   int st = g->capture();
   if (st) return st;
   st = g->reset_ctl(0.0);
   if (st) return st;
   CK(cudaGraphLaunch(g->step_exec, g->stream));
   double n[4];
   st = g->read_norms(n, 4);
   if (st) return st;
   if (norms4) std::memcpy(norms4, n, sizeof(n));
   return HAMSTR_GPU_OK;
}

int hamstr_gpu_step_host(hamstr_gpu* g, const double* q_in, double* q_out, double* norms4)
{
   if (!g) return HAMSTR_GPU_ERR_ARG;
   g->wlin_valid = false;   // q changes: the kept WENO values no longer apply
   int st = g->capture();
   if (st) return st;
   const size_t bytes = 4 * (size_t)g->d.nCell * sizeof(double);
   if (q_in) CK(cudaMemcpyAsync(g->d.q, q_in, bytes, cudaMemcpyHostToDevice, g->stream));
   st = g->reset_ctl(0.0);
   if (st) return st;
   CK(cudaGraphLaunch(g->step_exec, g->stream));
   if (q_out) CK(cudaMemcpyAsync(q_out, g->d.q, bytes, cudaMemcpyDeviceToHost, g->stream));
   double n[4];
   st = g->read_norms(n, 4);   // norms and the status word, then the one synchronisation
   if (st) return st;
   if (norms4) std::memcpy(norms4, n, sizeof(n));
   return HAMSTR_GPU_OK;
}

int hamstr_gpu_march(hamstr_gpu* g, int nsteps, double tol, double* hist, int* evals, int* converged)
{
   if (!g || nsteps < 0) return HAMSTR_GPU_ERR_ARG;
   g->wlin_valid = false;   // q may change: the kept WENO values no longer apply
   int st = g->capture();
   if (st) return st;
   DeviceState& d = g->d;
   if (nsteps > d.hist_cap) {
      set_error("nsteps beyond the history capacity of one march call (" + std::to_string(d.hist_cap) + ")");
      return HAMSTR_GPU_ERR_ARG;
   }
   st = g->reset_ctl(tol);
   if (st) return st;
   const size_t row = 4 * (size_t)d.nInst;
   if (hist) {
      std::vector<double> nanfill(row * (size_t)std::max(nsteps, 1), std::nan(""));
      CK(cudaMemcpyAsync(d.hist, nanfill.data(), nanfill.size() * sizeof(double), cudaMemcpyHostToDevice, g->stream));
      CK(cudaStreamSynchronize(g->stream));
   }
   for (int i = 0; i < nsteps; i++) CK(cudaGraphLaunch(g->step_exec, g->stream));
   int ctl[2] = {0, 0};
   CK(cudaMemcpyAsync(ctl, d.ctl, sizeof(ctl), cudaMemcpyDeviceToHost, g->stream));
   st = g->status_check();
   if (st) return st;
   const int rows = ctl[0] ? ctl[1] + 1 : ctl[1];
   if (hist && rows > 0) {
      CK(cudaMemcpyAsync(hist, d.hist, row * (size_t)rows * sizeof(double), cudaMemcpyDeviceToHost, g->stream));
      CK(cudaStreamSynchronize(g->stream));
   }
   if (evals) *evals = rows;
   if (converged) *converged = ctl[0];
   return HAMSTR_GPU_OK;
}

int hamstr_gpu_update_solution(hamstr_gpu* g, const char* qold, const char* qnew, double coef)
{
   if (!g || !qold || !qnew) return HAMSTR_GPU_ERR_ARG;
   g->wlin_valid = false;   // q may change: the kept WENO values no longer apply
   auto pick = [&](const char* n) -> double* {
      if (!std::strcmp(n, "q")) return g->d.q;
      if (!std::strcmp(n, "qt")) return g->d.qt;
      return nullptr;
   };
   double* src = pick(qold);
   double* dst = pick(qnew);
   if (!src || !dst) {
      set_error("updateSolution arrays are \"q\" or \"qt\"");
      return HAMSTR_GPU_ERR_ARG;
   }
   int st = g->reset_ctl(0.0);
   if (st) return st;
   launch_update(g->d, src, dst, coef, g->stream);
   CK(cudaGetLastError());
   return g->status_check();
}

int hamstr_gpu_step_explicit(hamstr_gpu* g, int scheme, double* norms2)
{
   // march.cpp:342-377: "euler" (scheme 0) and the 3-stage "rk3" (scheme 1)
   if (!g || (scheme != 0 && scheme != 1)) return HAMSTR_GPU_ERR_ARG;
   g->wlin_valid = false;   // q may change: the kept WENO values no longer apply
   int st = g->reset_ctl(0.0);
   if (st) return st;
   DeviceState& d = g->d;
   auto rhs = [&]() {
      launch_recon5(d, false, g->stream);
      launch_rhs_face(d, false, g->stream);
      launch_rhs_cell(d, false, g->stream);
      launch_norm_final(d, 0, false, g->stream);
   };
   if (scheme == 0) {
      rhs();
      launch_update(d, d.q, d.q, 1.0, g->stream);
   } else {
      rhs();
      launch_update(d, d.q, d.qt, 0.25, g->stream);
      launch_update(d, d.q, d.q, 8.0 / 15, g->stream);
      rhs();
      launch_update(d, d.qt, d.q, 5.0 / 12, g->stream);
      rhs();
      launch_update(d, d.qt, d.q, 3.0 / 4.0, g->stream);
   }
   CK(cudaGetLastError());
   double n[2];
   st = g->read_norms(n, 2);
   if (st) return st;
   if (norms2) { norms2[0] = n[0]; norms2[1] = n[1]; }
   return HAMSTR_GPU_OK;
}

void* hamstr_gpu_stream(hamstr_gpu* g) { return g ? (void*)g->stream : nullptr; }

int hamstr_gpu_enqueue_steps(hamstr_gpu* g, int n)
{
   if (!g || n < 0) return HAMSTR_GPU_ERR_ARG;
   g->wlin_valid = false;   // q may change: the kept WENO values no longer apply
   int st = g->capture();
   if (st) return st;
   st = g->reset_ctl(0.0);
   if (st) return st;
   for (int i = 0; i < n; i++) CK(cudaGraphLaunch(g->step_exec, g->stream));
   return HAMSTR_GPU_OK;
}

int hamstr_gpu_sync(hamstr_gpu* g)
{
   if (!g) return HAMSTR_GPU_ERR_ARG;
   return g->status_check();
}

int hamstr_gpu_layout(hamstr_gpu* g, int* out)
{
   if (!g || !out) return HAMSTR_GPU_ERR_ARG;
   const Plan& P = g->plan;
   int nper = 0, nperrows = 0;
   for (int c = 0; c < P.nChain; c++)
      if (P.chain_periodic[c]) {
         nper++;
         nperrows += P.chain_nrows[c];
      }
   out[0] = P.nSlot; out[1] = P.nSten; out[2] = P.nRow; out[3] = P.nChain;
   out[4] = P.nWave; out[5] = nper; out[6] = nperrows; out[7] = P.maxRows;
   return HAMSTR_GPU_OK;
}

int hamstr_gpu_launches_per_step(hamstr_gpu* g)
{
   if (!g) return HAMSTR_GPU_ERR_ARG;
   if (!g->launches_per_step) {
      int st = g->capture();
      if (st) return st;
   }
   return g->launches_per_step;
}

int hamstr_gpu_profile_step(hamstr_gpu* g, int reps, const char** names, double* ms, int* launches, int* n)
{
   // eager launches of the current mode's step with events around each kernel
   if (!g || reps < 1 || !names || !ms || !launches || !n) return HAMSTR_GPU_ERR_ARG;
   g->wlin_valid = false;   // q may change: the kept WENO values no longer apply
   int st = g->reset_ctl(0.0);
   if (st) return st;
   std::vector<std::pair<const char*, std::pair<cudaEvent_t, cudaEvent_t>>> rec;
   std::vector<const char*> order;
   std::vector<double> acc;
   std::vector<int> cnt;
   for (int r = 0; r < reps; r++) {
      rec.clear();
      g->prof = &rec;
      st = g->enqueue_step(false);
      g->prof = nullptr;
      if (st) return st;
      CK(cudaStreamSynchronize(g->stream));
      for (auto& e : rec) {
         float t = 0.f;
         cudaEventElapsedTime(&t, e.second.first, e.second.second);
         cudaEventDestroy(e.second.first);
         cudaEventDestroy(e.second.second);
         size_t k = 0;
         while (k < order.size() && std::strcmp(order[k], e.first) != 0) k++;
         if (k == order.size()) {
            order.push_back(e.first);
            acc.push_back(0.0);
            cnt.push_back(0);
         }
         acc[k] += t;
         cnt[k] += 1;
      }
   }
   st = g->status_check();
   if (st) return st;
   const int cap = *n;
   *n = (int)order.size();
   for (int k = 0; k < (int)order.size() && k < cap; k++) {
      names[k] = order[k];
      ms[k] = acc[k] / reps;
      launches[k] = cnt[k] / reps;
   }
   return HAMSTR_GPU_OK;
}

}  // extern "C"

extern "C" int hamstr_gpu_set_geometry(hamstr_gpu* g, int nNode, const double* xy)
{
   if (!g || !xy || nNode <= 0) return HAMSTR_GPU_ERR_ARG;
   const size_t nw = g->wall_face.size();
   std::vector<double4> geo(nw);
   for (size_t k = 0; k < nw; k++) {
      const int a = g->wall_n1[k], b = g->wall_n2[k];
      if (a < 0 || a >= nNode || b < 0 || b >= nNode) {
         set_error("wall face node id outside the node array");
         return HAMSTR_GPU_ERR_ARG;
      }
      geo[k] = make_double4(g->wall_normal[2 * k], g->wall_normal[2 * k + 1], 0.5 * (xy[2 * (size_t)a] + xy[2 * (size_t)b]),
                            0.5 * (xy[2 * (size_t)a + 1] + xy[2 * (size_t)b + 1]));
   }
   if (!g->wall_geo) {
      int st = dalloc(&g->wall_geo, nw, g->owned);
      if (st) return st;
   }
   if (nw) CK(cudaMemcpyAsync(g->wall_geo, geo.data(), nw * sizeof(double4), cudaMemcpyHostToDevice, g->stream));
   CK(cudaStreamSynchronize(g->stream));
   return HAMSTR_GPU_OK;
}

// forces of every instance: out[6k..6k+5] = {Fx, Fy, M, CL, CD, CM}
static int forces_all(hamstr_gpu* g, double* out)
{
   if (!g->wall_geo) {
      set_error("forces need hamstr_gpu_set_geometry first");
      return HAMSTR_GPU_ERR_ARG;
   }
   const DeviceState& d = g->d;
   const int ni = d.nInst;
   const size_t nw = g->wall_face.size();
   double* sums = g->wall_scr + 3 * nw;
   launch_forces(d.q, g->wall_cell, g->wall_geo, g->wall0, ni, d.fc.gamma - 1.0, g->wall_scr, sums, g->stream);
   CK(cudaGetLastError());
   std::vector<double> s(3 * (size_t)ni);
   CK(cudaMemcpyAsync(s.data(), sums, s.size() * sizeof(double), cudaMemcpyDeviceToHost, g->stream));
   CK(cudaStreamSynchronize(g->stream));
   for (int k = 0; k < ni; k++) {
      // coefficients on a unit chord from the instance's freestream (the
      // oracle's ho_forces expressions)
      const double rinf = g->inst_free[4 * k], uinf = g->inst_free[4 * k + 1], vinf = g->inst_free[4 * k + 2];
      const double V2 = uinf * uinf + vinf * vinf;
      const double qinf = 0.5 * rinf * V2;
      const double V = std::sqrt(V2);
      const double ca = uinf / V, sa = vinf / V;
      const double Fx = s[3 * k], Fy = s[3 * k + 1], M = s[3 * k + 2];
      double* o = out + 6 * (size_t)k;
      o[0] = Fx;
      o[1] = Fy;
      o[2] = M;
      o[3] = (Fy * ca - Fx * sa) / qinf;
      o[4] = (Fx * ca + Fy * sa) / qinf;
      o[5] = M / qinf;
   }
   return HAMSTR_GPU_OK;
}

extern "C" int hamstr_gpu_forces(hamstr_gpu* g, double* out)
{
   if (!g || !out) return HAMSTR_GPU_ERR_ARG;
   std::vector<double> all(6 * (size_t)g->d.nInst);
   const int st = forces_all(g, all.data());
   if (st) return st;
   std::memcpy(out, all.data(), 6 * sizeof(double));
   return HAMSTR_GPU_OK;
}

extern "C" int hamstr_gpu_batch_forces(hamstr_gpu* g, double* out)
{
   if (!g || !out) return HAMSTR_GPU_ERR_ARG;
   return forces_all(g, out);
}

extern "C" int hamstr_gpu_instances(hamstr_gpu* g, int* n, int* cell0)
{
   if (!g || !n) return HAMSTR_GPU_ERR_ARG;
   *n = g->d.nInst;
   if (cell0) std::memcpy(cell0, g->inst_cell0.data(), g->inst_cell0.size() * sizeof(int));
   return HAMSTR_GPU_OK;
}

extern "C" int hamstr_gpu_instance_norms(hamstr_gpu* g, double* out)
{
   if (!g || !out) return HAMSTR_GPU_ERR_ARG;
   return g->read_norms(out, 4 * g->d.nInst);
}

extern "C" int hamstr_gpu_autotune(hamstr_gpu* g, int reps, char* report, int report_len)
{
   if (!g || reps < 1) return HAMSTR_GPU_ERR_ARG;
   DeviceState& d = g->d;
   // candidates for the current precision: face-kernel block size, and the
   // line kernels' shape (FP64: warps per SM of the persistent warp-per-chain
   // kernels; FP32: threads per block of the thread-per-chain kernels)
   // (FP32 form with long periodic chains: also their segmented solve or
   // not -- it shortens each chain's latency but does several times the
   // work, which loses where the chains alone fill the GPU)
   struct Cand { int fb, wpb, mb, fused, fsoft, psoft, lanes, bundle, spike, fwpb; float ms; };
   const int wk = g->weno_keep, ck = g->mx_chunk;
   std::vector<int> spikes = {d.sp_on};
   if (g->mixed && d.nSpike > 0) spikes = {0, 1, 2};
   std::vector<Cand> cands;
   for (int fb : {128, 256})
      for (int fsoft : {0, 1}) {
         if (g->mixed) {
            for (int fused : {0, 1})
               for (int mb : {32, 64, 128})
                  for (int sp : spikes)
                     cands.push_back({fb, d.adi_wpb, mb, fused, fsoft, d.piv_soft, g->adi_lanes, g->adi_bundle, sp,
                                      d.adi_fwpb, 0.f});
         } else {
            for (int w : {4, 8})
               for (int fw : {4, 8})
                  for (int psoft : {0, 1})
                     for (int ln : {16, 4})
                        for (int bu : {0, 4, 8, 16})
                           cands.push_back({fb, w, d.mx_block, d.mx_fused, fsoft, psoft, ln, bu, d.sp_on, fw, 0.f});
         }
      }
   // the tuning steps advance the state: keep q and put it back afterwards
   double* qsave = nullptr;
   const size_t qbytes = 4 * (size_t)d.nCell * sizeof(double);
   CK(cudaMallocAsync((void**)&qsave, qbytes, g->stream));
   CK(cudaMemcpyAsync(qsave, d.q, qbytes, cudaMemcpyDeviceToDevice, g->stream));
   cudaEvent_t e0, e1;
   CK(cudaEventCreate(&e0));
   CK(cudaEventCreate(&e1));
   int st = HAMSTR_GPU_OK;
   for (Cand& c : cands) {
      if ((st = g->apply_shape(c.fb, c.wpb, c.mb, c.fused, c.fsoft, c.psoft, c.lanes, wk, c.bundle, ck, c.spike,
                               g->adi_fuse, c.fwpb)))
         break;
      if ((st = g->capture())) break;
      if ((st = g->reset_ctl(0.0))) break;
      CK(cudaGraphLaunch(g->step_exec, g->stream));   // warm-up
      CK(cudaEventRecord(e0, g->stream));
      for (int i = 0; i < reps; i++) CK(cudaGraphLaunch(g->step_exec, g->stream));
      CK(cudaEventRecord(e1, g->stream));
      CK(cudaEventSynchronize(e1));
      CK(cudaEventElapsedTime(&c.ms, e0, e1));
      c.ms /= reps;
      if ((st = g->status_check())) break;
   }
   cudaEventDestroy(e0);
   cudaEventDestroy(e1);
   CK(cudaMemcpyAsync(d.q, qsave, qbytes, cudaMemcpyDeviceToDevice, g->stream));
   CK(cudaFreeAsync(qsave, g->stream));
   CK(cudaStreamSynchronize(g->stream));
   if (st) return st;
   const Cand* best = &cands[0];
   for (const Cand& c : cands)
      if (c.ms < best->ms) best = &c;
   st = g->apply_shape(best->fb, best->wpb, best->mb, best->fused, best->fsoft, best->psoft, best->lanes, wk,
                       best->bundle, ck, best->spike, g->adi_fuse, best->fwpb);
   if (st) return st;
   if (report && report_len > 0) {
      std::string r = "{\"precision\": \"" + std::string(g->mixed ? "mixed" : "fp64") + "\", \"candidates\": [";
      for (size_t i = 0; i < cands.size(); i++) {
         char buf[320];
         std::snprintf(buf, sizeof(buf),
                       "%s{\"face_block\": %d, \"adi_warps_per_sm\": %d, \"mx_block\": %d, \"mx_fused\": %d, "
                       "\"face_softdiv\": %d, \"pivot_softdiv\": %d, \"adi_open_lanes\": %d, \"adi_bundle_rows\": %d, "
                       "\"mx_spike\": %d, \"adi_factor_warps_per_sm\": %d, \"ms\": %.4f}",
                       i ? ", " : "", cands[i].fb, cands[i].wpb, cands[i].mb, cands[i].fused, cands[i].fsoft,
                       cands[i].psoft, cands[i].lanes, cands[i].bundle, cands[i].spike, cands[i].fwpb, cands[i].ms);
         r += buf;
      }
      char buf[320];
      std::snprintf(buf, sizeof(buf),
                    "], \"best\": {\"face_block\": %d, \"adi_warps_per_sm\": %d, \"mx_block\": %d, \"mx_fused\": %d, "
                    "\"face_softdiv\": %d, \"pivot_softdiv\": %d, \"adi_open_lanes\": %d, \"adi_bundle_rows\": %d, "
                    "\"mx_spike\": %d, \"adi_factor_warps_per_sm\": %d}}",
                    best->fb, best->wpb, best->mb, best->fused, best->fsoft, best->psoft, best->lanes, best->bundle,
                    best->spike, best->fwpb);
      r += buf;
      std::snprintf(report, (size_t)report_len, "%s", r.c_str());
   }
   return HAMSTR_GPU_OK;
}

extern "C" int hamstr_gpu_get_shape(hamstr_gpu* g, int* shape)
{
   if (!g || !shape) return HAMSTR_GPU_ERR_ARG;
   const DeviceState& d = g->d;
   const int v[HAMSTR_SHAPE_N] = {d.face_block, d.adi_wpb,    d.mx_block,    d.mx_fused,     d.face_soft,
                                  d.piv_soft,   g->adi_lanes, g->weno_keep, g->adi_bundle, g->mx_chunk,
                                  d.sp_on,      g->adi_fuse, d.adi_fwpb};
   std::memcpy(shape, v, sizeof(v));
   return HAMSTR_GPU_OK;
}

extern "C" int hamstr_gpu_set_shape(hamstr_gpu* g, const int* shape)
{
   if (!g || !shape) return HAMSTR_GPU_ERR_ARG;
   const int* s = shape;
   const bool ok = (s[0] == 128 || s[0] == 256) && (s[1] == 4 || s[1] == 8) &&
                   (s[2] == 32 || s[2] == 64 || s[2] == 128) && (s[3] == 0 || s[3] == 1) &&
                   (s[4] == 0 || s[4] == 1) && (s[5] == 0 || s[5] == 1) && (s[6] == 32 || s[6] == 16 || s[6] == 4) &&
                   (s[7] == 0 || s[7] == 1) && (s[8] >= 0 && s[8] <= 64) && (s[9] == 0 || s[9] == 1) &&
                   (s[10] >= 0 && s[10] <= 2) && (s[11] == 0 || s[11] == 1) && (s[12] == 4 || s[12] == 8);
   if (!ok) {
      set_error("set_shape: a value outside its allowed set");
      return HAMSTR_GPU_ERR_ARG;
   }
   return g->apply_shape(s[0], s[1], s[2], s[3], s[4], s[5], s[6], s[7], s[8], s[9], s[10], s[11], s[12]);
}

extern "C" int hamstr_gpu_set_cfl(hamstr_gpu* g, double cfl)
{
   if (!g || !(cfl > 0.0) || !(cfl < 1e300)) return HAMSTR_GPU_ERR_ARG;
   if (g->d.fc.cfl != cfl) {
      g->d.fc.cfl = cfl;   // kernels take the state by value: recapture the step
      g->invalidate();
   }
   return HAMSTR_GPU_OK;
}

extern "C" int hamstr_gpu_set_sweep_order(hamstr_gpu* g, int order)
{
   if (!g || (order != 0 && order != 1)) return HAMSTR_GPU_ERR_ARG;
   if (g->d.lin_order != order) {
      g->d.lin_order = order;   // kernels take the state by value: recapture the step
      g->wlin_valid = false;
      g->invalidate();
   }
   return HAMSTR_GPU_OK;
}

extern "C" int hamstr_gpu_set_precision(hamstr_gpu* g, int mixed)
{
   if (!g || (mixed != 0 && mixed != 1)) return HAMSTR_GPU_ERR_ARG;
   g->wlin_valid = false;   // q may change: the kept WENO values no longer apply
   if (mixed) {
      int st = g->ensure_mixed_buffers();
      if (st) return st;
   }
   if (g->mixed != mixed) {
      g->mixed = mixed;
      g->invalidate();
   }
   return HAMSTR_GPU_OK;
}
