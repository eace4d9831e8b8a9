// ##################################################################
//
// plan.h -- host-side layout of one mesh for the GPU kernels
//
// The reference rebuilds each chain's stencil, ghost states, block
// assembly pattern and accumulation order on every call
// (computeRHS.cpp:53-149, computeLinearRHS.cpp:52-143, ADI.cpp:62-191).
// All of that depends only on the mesh, so it is derived once here, by the
// reference's own rules, into flat arrays the kernels index directly.
// ##################################################################
#ifndef HAMSTR_GPU_PLAN_H
#define HAMSTR_GPU_PLAN_H

#include <string>
#include <vector>

namespace hamstr {

// stencil entry kinds (sten_kind)
enum { STEN_CELL = 0, STEN_WALL = 1, STEN_FREESTREAM = 2 };

// block assembly operation: (ffslot << 3) | (sel << 1) | neg
enum { OP_SEL_L = 0, OP_SEL_R = 1, OP_SEL_RREFL = 2 };
constexpr int kOpsPerBlock = 4;   // A, B and C each take up to 4 ordered terms

// how open chains take ghost states at their end faces
enum {
   END_RULE_REFERENCE = 0,   // computeRHS.cpp:86-149, 154-260 and ADI.cpp:126-190 exactly
   END_RULE_EXTENDED = 1,    // open chains may end at interior faces (mixed meshes)
};

struct MeshInput {
   int nCell = 0, nFace = 0, nChain = 0, nChainFace = 0;
   int order = 3;
   int end_rule = END_RULE_REFERENCE;
   const int* faces = nullptr;            // 6*nFace: n1 n2 cL eL cR eR (walls tagged -2)
   const int* faceStartPerChain = nullptr;// nChain+1
   const int* chainConn = nullptr;        // nChainFace
};

struct Plan {
   int nCell = 0, nFace = 0, nChain = 0, nSlot = 0, nSten = 0, nRow = 0;
   int order = 3, nGhost = 2, nWave = 0, maxRows = 0;

   // stencil entries, chain after chain (chainSize entries each)
   std::vector<int> sten_cell;   // cell read (mirrored cell for walls, -1 for freestream)
   std::vector<int> sten_kind;   // STEN_*
   std::vector<int> sten_face;   // reflection face for STEN_WALL, else -1
   std::vector<int> chain_sten0; // first stencil entry of each chain

   // processed face slots, in the reference's chain-major face order
   std::vector<int> slot_face, slot_left, slot_right;
   std::vector<int> slot_n;      // global stencil index of slot n (left state qr[n+1], right ql[n])
   std::vector<int> slot_swap;   // 1 for the last face of an open chain (ql[n] | qr[n+1])
   std::vector<int> slot_owner;  // slot whose Jacobian the reference keeps in ff[face] (last writer)

   // per-cell ordered contributions: entry = slot*2 + (cell is the right cell)
   std::vector<int> cell_ptr, cell_ent;

   // chains / ADI rows
   std::vector<int> chain_periodic, chain_nrows, chain_row0, chain_wave;
   std::vector<int> wave_ptr, wave_chains;        // chains grouped by wave
   std::vector<int> row_scell;   // cell scaled by CFL/sigma and written back (ADI.cpp:200-244)
   std::vector<int> row_fcell;   // cell whose residual forms the right-hand side (-1: zero)
   std::vector<int> row_ops;     // 3*kOpsPerBlock per row: A, B, C terms, -1 terminated
   std::vector<int> cell_last_wave_writer;         // 1 if some chain writes this cell
};

// Builds the plan; returns "" on success or a description of the problem.
std::string build_plan(const MeshInput& in, Plan& out);

// Job queues of the persistent FP64 line kernels: schedule 0 is the
// factorisation (all chains), schedule 1+v the solve of wave v.  Schedule
// s holds njobs[s] jobs, longest first; job k of it is the entries
// jobs[job_ptr[job0[s] + k] .. job_ptr[job0[s] + k + 1]).  Each warp takes
// the next job from a counter in device memory, so the longest jobs start
// first and no cost model decides which warp runs what.  A job is
//   - a chain id: the chain on the whole warp (periodic chains; open ones
//     with open_lanes = 32);
//   - (a | kPairJob), b: open chains a and b, one per half-warp
//     (open_lanes = 16);
//   - (kQuadJob | n), c_1 .. c_n: n <= 8 open chains, four lanes each
//     (open_lanes = 4);
//   - (kBundleJob | n), c_1 .. c_n: n <= 32 open chains of at most
//     bundle_rows rows, one per lane.
// nwarps[s] = min(njobs[s], max_warps) warps are launched (max_warps_factor
// for the factorisation), more where long jobs are spread (below).  With
// fuse_first_wave the factorisation's jobs for the first wave's chains are
// packed as that wave's solve packs them and carry kFusedJob on their first
// entry: the warp that factors them runs their first sweep's solve at once.
constexpr int kPairJob = 1 << 30;
constexpr int kBundleJob = 1 << 29;
constexpr int kQuadJob = 1 << 28;
constexpr int kFusedJob = 1 << 27;
// The leading jobs of a schedule whose cost is at least kCritFrac of the
// longest set the launch's length.  ncrit[s] > 0: at most kMaxCrit such
// outliers, each runs alone on its SM (the first warp of block b starts with
// job b and the other warps of those blocks take no job), so no other FP64
// work shares the SM while the chain that sets the launch's length runs.
// ncrit[s] = -n: more of them (the periodic loops of a quad O-grid), the
// first n = min(count, nsm) spread one per SM the same way, with a block on
// each of those SMs, but the other warps keep taking jobs.  0: no spreading
// (nsm = 0 or no long job).
constexpr double kCritFrac = 0.8;
constexpr int kMaxCrit = 8;
struct Schedule {
   std::vector<int> job0, njobs, nwarps;   // per schedule
   std::vector<int> ncrit;                 // per schedule: leading jobs that run alone on their SM
   std::vector<int> job_ptr;               // per job (all schedules), +1
   std::vector<int> jobs;                  // job entries, as above
};
// max_warps_factor (0: max_warps) bounds the factorisation's warps, max_warps the solves';
// both are a multiple of nsm, the number of SMs (one block per SM).
Schedule build_schedule(const Plan& p, int max_warps, int open_lanes, int bundle_rows,
                        bool fuse_first_wave = false, int max_warps_factor = 0, int nsm = 0);

}  // namespace hamstr
#endif
