/*
 * hamstr_gpu.h -- C ABI of the GB300 HAMSTR steady ADI iteration.
 *
 * The reference (HAMSTR_OOP, 2D Euler, line-implicit) is a C++ program with
 * no library boundary: its SOLVER class reaches the mesh and solution
 * through friend access (meshBlock.h:18, solnBlock.h:15) and runs
 * single-threaded on the host.  This header is the boundary its hot path
 * moves behind.  Each entry point names the reference interface it
 * replaces.  The C++ drop-in classes MESHBLOCK / SOLNBLOCK / SOLVER / HAMSTR
 * (hamstr_oop_gb300/csrc/host/) are thin callers of these functions.
 *
 * Conventions
 *   - Plain pointers and sizes; arrays are the reference's layouts:
 *       q, r, r0, dq      [nCell][4] doubles (rho, rho u, rho v, E)
 *       sigma             [nCell]
 *       faces             [nFace][6] ints  n1 n2 cL eL cR eR (io.cpp:349-355),
 *                         after the reader's swap and preprocessing's wall
 *                         tag cR = -2 (io.cpp:360-365, preprocess.cpp:182)
 *       normVec           [nFace][2]  (dy, -dx)  (preprocess.cpp:86-87)
 *       refMtx            [nFace][2][2]          (preprocess.cpp:97-101)
 *       faceStartPerChain [nChain+1], chainConn [nChainFace] (io.cpp:223-264)
 *       ff                [nFace][2][4][4]  FACEMAT lmat, rmat (codetypes.h:64-68)
 *   - Every function returns an int status: 0 on success, a negative
 *     HAMSTR_GPU_ERR_* code otherwise.  Nothing exits the process (the
 *     reference calls exit(1) on a NaN spectral radius,
 *     interfaceFlux.cpp:117-124, and on missing files, io.cpp:19-23).
 *   - A solver handle owns its device memory and one CUDA stream; calls on
 *     one handle are not re-entrant (the reference is single-threaded).
 *     Host arrays belong to the caller; every copy is explicit.
 */
#ifndef HAMSTR_GPU_H
#define HAMSTR_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define HAMSTR_GPU_OK             0
#define HAMSTR_GPU_ERR_ARG       -1   /* bad argument or unknown array name */
#define HAMSTR_GPU_ERR_TOPOLOGY  -2   /* chains/faces the reference cannot process */
#define HAMSTR_GPU_ERR_CUDA      -3   /* CUDA runtime failure; also a line solve that gave up waiting
                                         for its factorisation (never expected) */
#define HAMSTR_GPU_ERR_NAN       -4   /* NaN spectral radius (interfaceFlux.cpp:117-124) */
#define HAMSTR_GPU_ERR_IO        -5   /* missing or malformed case file (io.cpp:19-23,138-141) */
#define HAMSTR_GPU_ERR_NOMEM     -6   /* host or device allocation failed */
/* An ADI line factorisation met a zero or non-finite pivot: the reciprocal
   1/b of triSolvers.cpp:796-811 (and :900-929) is infinite or NaN.  The
   reference divides regardless and carries the inf/NaN on. */
#define HAMSTR_GPU_ERR_SINGULAR  -7
/* An ADI sweep produced a non-finite dq (dq += r, ADI.cpp:247-248); the
   reference prints a NaN residual at most (march.cpp:157-158). */
#define HAMSTR_GPU_ERR_NONFINITE -8

typedef struct hamstr_case hamstr_case; /* host mesh + inputs: MESHBLOCK + SOLNBLOCK */
typedef struct hamstr_gpu hamstr_gpu;   /* device solver: SOLVER */

typedef struct hamstr_gpu_params {
   int    order;      /* 1, 3 (MUSCL) or 5 (WENO)         solnBlock.h:30 */
   int    msweep;     /* ADI sweeps per step              solnBlock.h:34 */
   double CFL;        /*                                  solnBlock.h:41 */
   double gamma;      /* 1.4                              initFlow.cpp:19 */
   double rinf, uinf, vinf, einf;   /* freestream         initFlow.cpp:24-57 */
   /* project option, no reference counterpart: how open chains take ghost
      states at their end faces.  HAMSTR_END_RULE_REFERENCE (0) is
      computeRHS.cpp:86-149, 154-260 and ADI.cpp:126-190 exactly;
      HAMSTR_END_RULE_EXTENDED (1) lets open chains end at interior faces
      (mixed tri/quad meshes): ghosts beyond such a face hold the true
      neighbour's state, its coupling to that neighbour is lagged in ADI
      while both diagonal terms stay implicit, and wall ghosts mirror by
      position.  On meshes whose open chains all end at walls or the far
      field and have at least 3 cells, both rules give the same results. */
   int    chain_end_rule;
   /* project option, no reference counterpart: the MUSCL limiter of order 3.
      HAMSTR_LIMITER_REFERENCE (0) is reconstruction.cpp:16-70; MINMOD (1)
      and VANALBADA (2) are the kappa = 1/3 scheme with minmod-limited
      differences or van Albada's limiter (Anderson, Thomas & van Leer, AIAA
      J. 24(9), 1986).  Orders 1 and 5 ignore it. */
   int    limiter;
} hamstr_gpu_params;

#define HAMSTR_LIMITER_REFERENCE 0
#define HAMSTR_LIMITER_MINMOD    1
#define HAMSTR_LIMITER_VANALBADA 2

#define HAMSTR_END_RULE_REFERENCE 0
#define HAMSTR_END_RULE_EXTENDED  1

/* ---------------- host side (reader, preprocessing, initial state) -------
 * Replaces MESHBLOCK::readMeshData (io.cpp:58-372), SOLNBLOCK::
 * readSolutionInputs (io.cpp:13-51), MESHBLOCK::setViscosity(0) +
 * preprocess (meshBlock.h:52, preprocess.cpp:15-241) and SOLVER::initFlow
 * (initFlow.cpp:12-93): reads <case_dir>/input.hamstr and
 * <case_dir>/input/domain000/*.dat. */
int  hamstr_case_open(const char* case_dir, hamstr_case** out, char* err, int errlen);
void hamstr_case_close(hamstr_case* c);
/* out[10]: nCell nFace nChain nChainFace nMaxChain order msweep nGhost nNode nColor */
int  hamstr_case_sizes(const hamstr_case* c, int* out);
/* out[9]: Mach alpha CFL gamma rinf uinf vinf einf pinf */
int  hamstr_case_params(const hamstr_case* c, double* out);
/* int arrays: faces chainConn faceStartPerChain c2chain bFaces chainsPerColor
 * double arrays: x vol normVec refMtx q  (q is the freestream initial state) */
int  hamstr_case_get_int(const hamstr_case* c, const char* name, int* out, int* count);
int  hamstr_case_get(const hamstr_case* c, const char* name, double* out);
/* overrides of input.hamstr values (order, msweep, CFL) and the freestream */
int  hamstr_case_set_run(hamstr_case* c, int order, int msweep, double cfl);
int  hamstr_case_set_freestream(hamstr_case* c, double uinf, double vinf, double einf);
/* A copy of a case (no reference counterpart), e.g. for the members of a
 * batch that share a mesh; and a new flow condition for a case: Mach and
 * angle of attack in degrees, the freestream and initial state recomputed
 * as initFlow.cpp:24-91 does. */
int  hamstr_case_clone(const hamstr_case* c, hamstr_case** out);
int  hamstr_case_set_flow(hamstr_case* c, double mach, double alpha_deg);
/* Project options (no reference counterpart): "chain_end_rule" =
 * HAMSTR_END_RULE_*, "limiter" = HAMSTR_LIMITER_*.  Used by
 * hamstr_gpu_create_from_case. */
int  hamstr_case_set_option(hamstr_case* c, const char* name, int value);

/* ---------------- device solver ------------------------------------------
 * hamstr_gpu_create replaces SOLVER::SOLVER (solver.cpp:13-81): it copies
 * the mesh and chain arrays to the GPU, derives the per-mesh stencil,
 * accumulation and block-assembly layout once, and sets q to freestream. */
int hamstr_gpu_create(const hamstr_gpu_params* p, int nCell, int nFace,
                      const int* faces, const double* normVec, const double* refMtx,
                      int nChain, const int* faceStartPerChain, const int* chainConn,
                      hamstr_gpu** out);
int hamstr_gpu_create_from_case(const hamstr_case* c, hamstr_gpu** out);
int hamstr_gpu_destroy(hamstr_gpu* g);
const char* hamstr_gpu_strerror(int status);
/* last detailed message (topology problems, CUDA errors) for this thread */
const char* hamstr_gpu_last_error(void);

/* named device arrays to/from host memory: q qt r r0 dq sigma (cell arrays) and
 * ff ([nFace][32], face order as sb->ff; faces outside every chain read 0) */
int hamstr_gpu_get(hamstr_gpu* g, const char* name, double* out);
int hamstr_gpu_set(hamstr_gpu* g, const char* name, const double* in);

/* SOLVER::computeRHS (computeRHS.cpp:17-427): r, sigma and, when implicit,
 * the face Jacobians ff; *l2 = sqrt(sum r_rho^2)/nCell, *linf = max|r_rho|. */
int hamstr_gpu_compute_rhs(hamstr_gpu* g, int implicit, double* l2, double* linf);
/* SOLVER::ADI (ADI.cpp:15-266): msweep line sweeps, dq, q += dq; the norms
 * are those of the final linear residual (computeLinearRHS.cpp:354-368). */
int hamstr_gpu_adi(hamstr_gpu* g, double* l2, double* linf);
/* SOLVER::computeLinearRHS (computeLinearRHS.cpp:13-371) on the current
 * r0, dq, sigma and ff. */
int hamstr_gpu_linear_rhs(hamstr_gpu* g, double* l2, double* linf);
/* SOLVER::stepSolution, ADI branch (march.cpp:381-386):
 * norms4 = {computeRHS L2, Linf, final linear L2, Linf}. */
int hamstr_gpu_step(hamstr_gpu* g, double* norms4);
/* The same step on a host-resident solution, as the reference's
 * stepSolution works on its host q (march.cpp:66): q_in [nCell][4] (NULL:
 * keep the device state) is copied in, the step runs, and q_out (NULL: no
 * copy) and norms4 (may be NULL) come back, with one synchronisation of the
 * handle's stream for all of it.  Host buffers should be page-locked for
 * the copies to overlap nothing else and run at full speed. */
int hamstr_gpu_step_host(hamstr_gpu* g, const double* q_in, double* q_out, double* norms4);
/* SOLVER::marchInTime (march.cpp:15-59) with a convergence stop: runs up
 * to nsteps steps; stops before the ADI of the first step whose computeRHS
 * L2 norm is <= tol (tol <= 0: never) -- on a batched handle, the first
 * step at which every instance's is.  hist (may be NULL) receives 4
 * doubles per computeRHS evaluation and instance ({L2, Linf, linear L2,
 * Linf}, instances in order); *evals = number of rows written,
 * *converged = 1 when the stop fired.  Norms stay on the GPU until the end. */
int hamstr_gpu_march(hamstr_gpu* g, int nsteps, double tol, double* hist, int* evals, int* converged);

/* Arithmetic of the implicit step taken by hamstr_gpu_step / _march /
 * _enqueue_steps (no counterpart in the reference, which is FP64 only):
 *   0 (default)  plain FP64, bit-identical to the reference;
 *   1            defect correction: the residual (reconstruction, Roe flux,
 *                computeRHS sums) stays FP64 and identical to the
 *                reference, while the Roe Jacobians, the ADI line solves and
 *                the linearised residual of the sweeps run in FP32.  The
 *                converged state is the FP64 residual's zero; the iteration
 *                history differs from the reference's. */
int hamstr_gpu_set_precision(hamstr_gpu* g, int mixed);

/* Order of the ADI sweeps' linearised residual (no counterpart in the
 * reference, which always linearises the scheme's reconstruction,
 * computeLinearRHS.cpp:281-292):
 *   0 (default)  the reference's: dq reconstructed at the scheme's order;
 *   1            first order: each face takes dq of its two cells, the
 *                linearisation that matches the line operator (whose blocks
 *                couple neighbouring cells only).
 * The residual, and so the converged state, is unchanged; the iteration's
 * path differs.  The reference's higher-order sweeps can diverge as msweep
 * grows and leave a residual plateau that rises with CFL; the first-order
 * sweeps are a convergent defect-correction iteration. */
int hamstr_gpu_set_sweep_order(hamstr_gpu* g, int order);

/* Batched form (no counterpart in the reference): several cases -- meshes
 * of any sizes and their flow conditions -- in one handle.  They are held
 * as a disjoint union (cells, faces and chains of case k follow those of
 * case k-1), so every kernel launch and every captured step covers all of
 * them.  The cases must share order, msweep, CFL, gamma, limiter and chain
 * end rule; each keeps its own freestream (ghost states and initial
 * state), norms and forces.  Each instance's arithmetic is that of a
 * plain handle on its case, except the reference's cell-id-0 ghost test
 * (computeRHS.cpp:158,170), which the union keeps for the first case only.
 * hamstr_gpu_get/set and the norms of hamstr_gpu_step etc. address the
 * union (instance 0's norms); hamstr_gpu_instances gives the cell offsets
 * (n+1 ints, may be NULL), hamstr_gpu_instance_norms the last norms of each
 * instance ([n][4]), hamstr_gpu_batch_forces the forces of each ([n][6]). */
int hamstr_gpu_create_batch(const hamstr_case* const* cases, int n, hamstr_gpu** out);
int hamstr_gpu_instances(hamstr_gpu* g, int* n, int* cell0);
int hamstr_gpu_instance_norms(hamstr_gpu* g, double* norms);
int hamstr_gpu_batch_forces(hamstr_gpu* g, double* out);

/* Wall forces (no counterpart in the reference, which computes none).
 * hamstr_gpu_set_geometry hands over the node coordinates (x y per node,
 * coord.dat order; io.cpp:144-156) for the faces' midpoints;
 * hamstr_gpu_create_from_case does it itself.  hamstr_gpu_forces then
 * integrates the wall pressure of the current state: for each wall face
 * (right cell -2, ascending face id) p * (dy, -dx) with p from the adjacent
 * cell, summed in face order, and the moment about (0.25, 0).
 * out6 = {Fx, Fy, M, CL, CD, CM} with coefficients on a unit chord and the
 * freestream dynamic pressure and flow direction (instance 0 of a batch). */
int hamstr_gpu_set_geometry(hamstr_gpu* g, int nNode, const double* xy);
int hamstr_gpu_forces(hamstr_gpu* g, double* out6);

/* Autotuner (no reference counterpart): times `reps` steps of the current
 * precision for each candidate launch shape -- face kernels 128 or 256
 * threads per block; FP64 line kernels 4 or 8 persistent warps per SM (one
 * or two per sub-partition; the factorisation and the solves each their
 * own; schedules rebuilt longest-job-first), with open
 * chains two per warp (one per half) or eight per warp (four lanes
 * each), and the shortest (up to 0, 4, 8 or 16 rows) 32 per warp, one per
 * lane; FP32
 * line kernels 32..128 threads per block, with the blocks assembled by a
 * separate coalesced kernel or inside the factorisation, and, where there
 * are long chains, those solved by segments or not (shape key 10); FP64
 * divisions of the face
 * kernels and of the LU pivots on the FP64 pipe or on the integer pipes
 * (bit-identical) -- and keeps the fastest.  The state is restored
 * afterwards; FP64 results do not depend on the shape.  report (may be
 * NULL) receives a JSON summary of the timings (about 240 bytes per
 * candidate, at most 256 candidates). */
int hamstr_gpu_autotune(hamstr_gpu* g, int reps, char* report, int report_len);

/* The launch shape itself (no reference counterpart), HAMSTR_SHAPE_N ints:
 *   [0] face kernels' threads per block: 128 or 256
 *   [1] FP64 line kernels' persistent warps per SM: 4 or 8
 *   [2] FP32 line kernels' threads per block: 32, 64 or 128
 *   [3] FP32 blocks assembled inside the factorisation: 0 or 1
 *   [4] face kernels' divisions on the integer pipes: 0 or 1
 *   [5] FP64 LU pivot reciprocals on the integer pipes: 0 or 1
 *   [6] FP64 line kernels: lanes per open chain -- 32 (a warp), 16 (two
 *       per warp) or 4 (eight per warp): 32, 16 or 4
 *   [7] order 5, FP64: the WENO linearisation's state-only values formed
 *       once per step by the implicit computeRHS and kept for the sweeps
 *       (1 KiB per face slot of device memory): 0 or 1 (default 1; not
 *       tuned by hamstr_gpu_autotune)
 *   [8] FP64 line kernels: open chains of at most this many rows go 32 to
 *       a warp, one per lane (0: none): 0..64
 *   [9] FP32 line kernels: the loads of several rows issued together (4 in
 *       the solve, 2 in the periodic elimination), where the launch's chains
 *       are all resident at once with the larger register count this takes:
 *       0 or 1 (default 1; not tuned)
 *  [10] FP32 line kernels: long chains solved by segments (16 rows each,
 *       up to 32, one warp lane per segment, joined by a small cyclic
 *       system on the segment ends) instead of one thread running the whole
 *       recurrence: 0 none, 1 periodic chains of 64 rows or more, 2 those
 *       and open chains of 32 rows or more (default 1; tuned in the FP32
 *       form where such chains exist).
 *       The same linear system; in FP32 the rounding differs, so the FP32
 *       form's iterates differ in the last bits and its steady state (the
 *       FP64 residual's zero) does not.
 *  [11] FP64 line kernels: the first wave's chains solved for the first
 *       sweep by the warp that has just factored them, inside the
 *       factorisation kernel (the other chains' factorisation goes on
 *       beside them), instead of by a separate launch: 0 or 1 (default 1;
 *       not tuned)
 *  [12] FP64 factorisation kernel: persistent warps per SM, 4 or 8 (as [1]
 *       for the solves; default 4; tuned with it)
 * set_shape checks every value (HAMSTR_GPU_ERR_ARG otherwise); FP64
 * results do not depend on the shape. */
#define HAMSTR_SHAPE_N 13
int hamstr_gpu_get_shape(hamstr_gpu* g, int* shape);
int hamstr_gpu_set_shape(hamstr_gpu* g, const int* shape);

/* ---------------- learned warm start (no reference counterpart) --------
 * C[M][N] (+ split * M * N when splits > 1) = A[M][K] * B[N][K]^T with A, B
 * BF16 (K contiguous, 16-byte aligned device arrays) and FP32 accumulation
 * on the tcgen05 tensor cores; M % 128 == 0, K % 64 == 0, N in {16, 64,
 * 128} or a multiple of 256.  K is cut into `splits` ranges whose partial
 * products go to consecutive M*N slabs.  *err (device int) becomes 1 if a
 * wait timed out.  stream: a cudaStream_t or NULL. */
int hamstr_mlp_gemm(const void* A, const void* B, int M, int N, int K, int splits, float* C, int* err, void* stream);

/* The warm-start network (no reference counterpart): 5 -> 256 -> 256 ->
 * 256 -> 4, GELU, BF16 weights and activations with FP32 accumulation,
 * forward and backward on the tensor cores (hamstr_mlp_gemm), Adam on FP32
 * master weights.  Parameters travel as FP32 in the order W1[256][5] b1
 * W2[256][256] b2 W3[256][256] b3 W4[4][256] b4 (hamstr_mlp_nparams()).
 * Device arrays: features [n][5], targets and outputs [n][4], FP32.
 *   _create: batch capacity (rows per pass), seed of the initial weights;
 *   _forward: outputs for n rows (any n, in chunks of the capacity);
 *   _grad: loss (mean squared error over n <= capacity rows and the 4
 *     outputs) and its gradient, kept for _get_grads;
 *   _train_step: one Adam step (lr; betas 0.9, 0.999) on a minibatch of
 *     `batch` rows (a multiple of 128) drawn from n_all rows by a seeded
 *     hash of (seed, step); step counts from 0. */
typedef struct hamstr_mlp hamstr_mlp;
int hamstr_mlp_nparams(void);
int hamstr_mlp_create(int batch_capacity, unsigned long long seed, hamstr_mlp** out);
int hamstr_mlp_destroy(hamstr_mlp* h);
int hamstr_mlp_set_params(hamstr_mlp* h, const float* params);
int hamstr_mlp_get_params(hamstr_mlp* h, float* params);
int hamstr_mlp_get_grads(hamstr_mlp* h, float* grads);
int hamstr_mlp_forward(hamstr_mlp* h, const float* features, int n, float* outputs);
int hamstr_mlp_grad(hamstr_mlp* h, const float* features, const float* targets, int n, double* loss);
int hamstr_mlp_train_step(hamstr_mlp* h, const float* features, const float* targets, long long n_all, int batch,
                          unsigned long long seed, unsigned long long step, float lr, double* loss);

/* Self-test hook: soft[i] = the integer-pipe division the FP64 kernels use
 * (hamstr_oop_gb300/csrc/softdiv.cuh), hard[i] = the hardware a[i]/b[i],
 * on device arrays of n doubles.  Tests compare them bit for bit. */
int hamstr_check_softdiv(const double* a, const double* b, double* soft, double* hard, int n, void* stream);

/* Self-test hook for the shared-memory row count that a line solve waits on
 * behind its factorisation (hamstr_oop_gb300/csrc/line_solve.cuh): in one
 * block, one warp publishes 3 rows and stops; another waits for 1, 3 and 4
 * rows.  out[0..2] (device ints) receive 1 for a wait that was met and 0 for
 * one that gave up at its bound; expected {1, 1, 0}, and the kernel ends. */
int hamstr_check_row_wait(int* out, void* stream);

/* Changes the pseudo-time CFL number of later steps (no counterpart in the
 * reference, which reads CFL once, io.cpp:37).  Lets a caller ramp CFL up
 * from an impulsive start.  HAMSTR_GPU_ERR_ARG unless cfl > 0. */
int hamstr_gpu_set_cfl(hamstr_gpu* g, double cfl);

/* SOLVER::stepSolution, explicit branches (march.cpp:342-377): scheme 0 is
 * "euler" (computeRHS("explicit") then q += CFL/sigma r), scheme 1 the
 * 3-stage "rk3" through the second state qt.  norms2 = the last
 * computeRHS L2 and Linf. */
int hamstr_gpu_step_explicit(hamstr_gpu* g, int scheme, double* norms2);
/* SOLVER::updateSolution(qold, qnew, coef) (march.cpp:411-433) on the device
 * arrays named "q" or "qt": qnew = qold + coef*CFL/sigma * r. */
int hamstr_gpu_update_solution(hamstr_gpu* g, const char* qold, const char* qnew, double coef);

/* TRISOLVER::blockTridag4 (triSolvers.cpp:769-847) and blockTridagPeriodic4
 * (triSolvers.cpp:850-1046), batched over nlines independent lines of N
 * block rows, on DEVICE arrays:
 *   A, B, C  [nlines][N][4][4] row-major blocks (read only; the reference
 *            overwrites b and c as scratch)
 *   F        [nlines][N][4] right-hand sides, overwritten with the solution
 *            as the reference's f is
 * periodic = 1 selects the cyclic solver (A_0 couples row 0 to row N-1 and
 * C_{N-1} row N-1 to row 0; needs N >= 2); 0 the open one (A_0, C_{N-1}
 * unused).  stream is a cudaStream_t or NULL.  Scratch of (80 N + 16)
 * doubles per line is allocated and freed inside the call, which
 * synchronises the stream. */
int hamstr_gpu_block_tridag4(int nlines, int N, int periodic, const double* A, const double* B,
                             const double* C, double* F, void* stream);

/* The same solve without any device allocation (no counterpart in the
 * reference, which has no GPU).  For callers that cannot allocate device
 * memory on every call: loops that run beside work on other streams (the
 * cudaFree of the entry point above waits for the whole device) and hosts
 * whose device memory belongs to their own pool allocator.  Scratch is a
 * fixed 8 MiB array that every GPU loading the library holds until exit;
 * the call needs nlines*(80*N+16) <= 1048576 doubles and returns
 * HAMSTR_GPU_ERR_ARG beyond that.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress) with that device current;
 * make that first call before any stream capture.  The address is kept
 * for the life of the process, so do not call this entry point after a
 * cudaDeviceReset of that device (the array may then sit elsewhere).
 * The call only enqueues work on `stream` (synchronise it before reading
 * F).  All calls share the one array: calls whose work overlaps on the GPU
 * (different streams, or different host threads) race and must be
 * serialised by the caller. */
int hamstr_gpu_block_tridag4_noalloc(int nlines, int N, int periodic, const double* A, const double* B,
                                     const double* C, double* F, void* stream);

/* ---------------- function-level entry points ---------------------------
 * The reference's per-face and per-chain numerics, batched, on DEVICE
 * arrays; each only enqueues on `stream` (a cudaStream_t or NULL).  Every
 * output equals one reference call's bit for bit.
 *
 * SOLVER::fluxRoe2D (interfaceFlux.cpp:24-169) for n faces: nxy [n][2]
 * (the face normal (dy, -dx), solver.h:46's nxyz), ql, qr [n][4] ->
 * flux [n][4] (times the face area) and spec [n] (spectral radius times the
 * area).  Where the reference exits on a NaN spectral radius
 * (interfaceFlux.cpp:117-124) spec holds the NaN; callers check it. */
int hamstr_gpu_flux_roe2d(int n, const double* nxy, const double* ql, const double* qr, double* flux, double* spec,
                          double gamma, void* stream);
/* SOLVER::jacobianRoe2D (jacobianRoe.cpp:9-70; IMODE 1, frozen Roe
 * eigenvalues) for n faces: lmat, rmat [n][4][4], row-major, times the
 * area -- the reference's lmat2[i][j], rmat2[i][j]. */
int hamstr_gpu_jacobian_roe2d(int n, const double* nxy, const double* ql, const double* qr, double* lmat,
                              double* rmat, double gamma, void* stream);
/* RECONSTRUCTION::MUSCL / MUSCL_DERIV / WENO / WENO_DERIV
 * (reconstruction.h:19-108, reconstruction.cpp:16-386) over nlines
 * independent lines: f, dq, ql, qr, f2 are [nlines][imax][nq] (the
 * reference's f[i][n] per line).  ql, qr are written for the entries the
 * reference writes and left alone elsewhere:
 *   MUSCL, MUSCL_DERIV: i in [is, ie]; qt == 0 copies f (dq), otherwise
 *     the kappa scheme (th, qt, eps as the reference takes them), which
 *     also leaves f2[i] = f[i+1] - f[i] for i < imax-1 as the reference
 *     does.  Needs 1 <= is and ie <= imax-2 when qt != 0: at ie = imax-1
 *     (computeRHS.cpp:267's call) the reference reads f2[imax-1] or
 *     dq[imax], work-array entries left over from an earlier chain, and
 *     its callers never use that last value.
 *   WENO, WENO_DERIV: i in [is, imax-3], is >= 2, from f (dq) at i-2..i+2.
 *     WENO's smoothness epsilon is 1e-15 whatever epsw says (the reference
 *     overwrites the argument, reconstruction.cpp:145); WENO_DERIV uses
 *     eps as given.  The reference reads a copy of f[0..ie]; these read f,
 *     so results agree for ie = imax-1, its callers' value.
 * HAMSTR_GPU_ERR_ARG for indices outside these ranges. */
int hamstr_gpu_muscl(int nlines, int imax, int nq, const double* f, double* ql, double* qr, double* f2, int is,
                     int ie, double th, double qt, double eps, void* stream);
int hamstr_gpu_muscl_deriv(int nlines, int imax, int nq, const double* f, const double* dq, double* ql, double* qr,
                           double* f2, int is, int ie, double th, double qt, double eps, void* stream);
int hamstr_gpu_weno(int nlines, int imax, int nq, const double* f, double* ql, double* qr, int is, int ie,
                    double epsw, void* stream);
int hamstr_gpu_weno_deriv(int nlines, int imax, int nq, const double* f, const double* dq, double* ql, double* qr,
                          int is, int ie, double eps, void* stream);

/* The 5-variable (3D strand) numerics, batched on DEVICE arrays.  The
 * reference's -DDim3 driver does not compile (io.cpp:306), but these
 * functions are compiled in every reference build and are given here at
 * function level, each output equal to one reference call's bit for bit:
 *   SOLVER::fluxRoe3D (interfaceFlux.cpp:176-319): nxyz [n][3], ql, qr
 *     [n][5] (rho, rho u, rho v, rho w, E) -> flux [n][5], spec [n]; unlike
 *     the 2D flux neither is multiplied by the face area;
 *   SOLVER::jacobianRoe3D (jacobianRoe.cpp:92-620, frozen eigenvalues,
 *     IMODE 1) -> lmat, rmat [n][5][5] row-major;
 *   TRISOLVER::blockTridag / blockTridagPeriodic (triSolvers.cpp:443-766,
 *     nq = 5) over nlines lines of N block rows, in place: A, B, C
 *     [nlines][N][5][5] are overwritten as the reference's scratch and F
 *     [nlines][N][5] with the solution; periodic needs N >= 2. */
int hamstr_gpu_flux_roe3d(int n, const double* nxyz, const double* ql, const double* qr, double* flux, double* spec,
                          double gamma, void* stream);
int hamstr_gpu_jacobian_roe3d(int n, const double* nxyz, const double* ql, const double* qr, double* lmat,
                              double* rmat, double gamma, void* stream);
int hamstr_gpu_block_tridag5(int nlines, int N, int periodic, double* A, double* B, double* C, double* F,
                             void* stream);

/* Enqueues n pseudo-time steps on the handle's stream and returns without
 * waiting (no tolerance stop, no host copies): for callers that keep the
 * state on the GPU and synchronise themselves (timing, pipelines). */
int hamstr_gpu_enqueue_steps(hamstr_gpu* g, int n);
/* wait for the handle's stream; returns a pending device error, if any */
int hamstr_gpu_sync(hamstr_gpu* g);
/* layout[8]: nSlot nSten nRow nChain nWave nPeriodicChains nPeriodicRows maxRows */
int hamstr_gpu_layout(hamstr_gpu* g, int* layout);
/* the CUDA stream (cudaStream_t) the handle launches on */
void* hamstr_gpu_stream(hamstr_gpu* g);
/* Per-kernel CUDA-event timing of one step (eager launches on the handle's
 * stream): ms[i] and launches[i] for i < *n kernel names (names[i]). */
int hamstr_gpu_profile_step(hamstr_gpu* g, int reps, const char** names, double* ms, int* launches, int* n);
/* number of kernel launches of one step (for launch accounting) */
int hamstr_gpu_launches_per_step(hamstr_gpu* g);

#ifdef __cplusplus
}
#endif
#endif
