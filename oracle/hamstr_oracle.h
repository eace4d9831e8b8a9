/*
 * hamstr_oracle.h -- CPU restatement of HAMSTR's steady ADI iteration.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the parity tests,
 * the smoke check and the CPU-baseline leg of bench.py call it, the product
 * never does.  It restates, in plain C with the reference's operation order,
 * the reference's case reader (io.cpp:58-372), preprocessing
 * (preprocess.cpp:15-241), flow initialisation (initFlow.cpp:12-93),
 * computeRHS (computeRHS.cpp:17-427), fluxRoe2D (interfaceFlux.cpp:24-169),
 * jacobianRoe2D/3D in the frozen-eigenvalue mode (jacobianRoe.cpp:9-70,
 * 92-620), the reconstructions (reconstruction.cpp), ADI with the 4x4 block
 * tridiagonal solvers (ADI.cpp:15-266, triSolvers.cpp:769-1046) and
 * computeLinearRHS (computeLinearRHS.cpp:13-371).
 *
 * Its results are pinned bit for bit against the reference compiled from its
 * own sources (oracle/Makefile `ref`) and against the committed golden
 * fixtures in tests/golden/.
 *
 * The handle API mirrors oracle/ref_harness.cpp so one Python wrapper drives
 * either implementation.
 */
#ifndef HAMSTR_ORACLE_H
#define HAMSTR_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ho_case ho_case;

/* Reads <case_dir>/input.hamstr and the files under <case_dir>/input/domain000/,
 * preprocesses and initialises to freestream.  NULL on failure, with a
 * message in err. */
ho_case* ho_open(const char* case_dir, char* err, int errlen);
ho_case* ho_clone(const ho_case* c);
void     ho_close(ho_case* c);

/* nCell nFace nChain nChainFace nMaxChain order msweep nGhost nNode nColor */
void ho_sizes(const ho_case* c, int* out);
/* Mach alpha CFL gamma rinf uinf vinf einf pinf */
void ho_params(const ho_case* c, double* out);
void ho_set_freestream(ho_case* c, double uinf, double vinf, double einf);
void ho_set_run(ho_case* c, int order, int msweep, double cfl);

/* Project options (absent from the reference):
 *   "chain_end_rule"  HO_END_RULE_REFERENCE (0, default): ghosts exactly as
 *                     computeRHS.cpp:86-149, 154-260; HO_END_RULE_EXTENDED
 *                     (1): open chains may end at interior faces (mixed
 *                     tri/quad meshes) -- ghosts beyond such a face hold the
 *                     true neighbour's state and the face couples to it
 *                     explicitly in ADI; wall ghosts mirror by position.
 * Returns 0, or -1 for an unknown name or value. */
#define HO_END_RULE_REFERENCE 0
#define HO_END_RULE_EXTENDED 1
/*   "limiter"         MUSCL limiter of order 3: HO_LIMITER_REFERENCE (0,
 *                     default, reconstruction.cpp:16-70), HO_LIMITER_MINMOD
 *                     (1) or HO_LIMITER_VANALBADA (2): the kappa = 1/3 scheme
 *                     with minmod-limited differences or van Albada's
 *                     limiter (Anderson, Thomas & van Leer, AIAA J. 1986). */
#define HO_LIMITER_REFERENCE 0
#define HO_LIMITER_MINMOD 1
#define HO_LIMITER_VANALBADA 2
/*   "sweep_order"     0 (default): the ADI sweeps' linearised residual
 *                     reconstructs dq at the scheme's order
 *                     (computeLinearRHS.cpp:281-292); 1: at first order
 *                     (dq of the two cells of each face), a project option
 *                     that leaves the residual and so the converged state
 *                     unchanged. */
int  ho_set_option(ho_case* c, const char* name, int value);

/* Each returns 0, or -1 when a spectral radius is NaN (the reference exits
 * the process there, interfaceFlux.cpp:117-124). */
int  ho_compute_rhs(ho_case* c, int implicit, double* l2, double* linf);
int  ho_adi(ho_case* c, double* l2, double* linf);
int  ho_linear_rhs(ho_case* c, double* l2, double* linf);
int  ho_step(ho_case* c, double* out4);
int  ho_march(ho_case* c, int n, double* hist);
/* explicit branches of stepSolution (march.cpp:342-377): scheme 0 "euler",
 * 1 "rk3"; out2 = last computeRHS L2, Linf */
int  ho_step_explicit(ho_case* c, int scheme, double* out2);
/* updateSolution (march.cpp:411-433) on "q" / "qt" */
int  ho_update_solution(ho_case* c, const char* qold, const char* qnew, double coef);
/* Runs `iters` steps on each of n independent cases, one host thread per
 * case (OpenMP); the CPU-baseline throughput leg. */
int  ho_march_replicas(ho_case** cases, int n, int iters);

/* Wall pressure force (project addition, no reference counterpart): the
 * wall faces' p * normal, p from the adjacent cell, summed in ascending face
 * order; out = {Fx, Fy, M about (0.25, 0), CL, CD, CM} on a unit chord. */
int ho_forces(const ho_case* c, double* out6);

/* triSolvers.cpp blockTridag4 / blockTridagPeriodic4 on flat [N][4][4]
 * blocks and [N][4] right-hand sides, in place like the reference. */
int ho_block_tridag4(double* a, double* b, double* c, double* f, int N, int periodic);

/* The reference's per-face and per-line functions on flat arrays:
 * SOLVER::fluxRoe2D / jacobianRoe2D (interfaceFlux.cpp:24-169,
 * jacobianRoe.cpp:9-70) for one face, and RECONSTRUCTION::MUSCL /
 * MUSCL_DERIV / WENO / WENO_DERIV (reconstruction.cpp:16-386) for one line
 * of [imax][nq] values, with the reference's loops and index ranges. */
int  ho_flux_roe2d(const double* nxy, const double* ql, const double* qr, double* flux, double* spec, double gamma);
void ho_jacobian_roe2d(const double* nxy, const double* ql, const double* qr, double* lm, double* rm, double gamma);
void ho_muscl_line(const double* f, double* ql, double* qr, double* f2, int is, int ie, double th, double qt,
                   double eps, int imax, int nq);
void ho_muscl_deriv_line(const double* f, double* ql, double* qr, double* f2, const double* dq, int is, int ie,
                         double th, double qt, double eps, int imax, int nq);
void ho_weno_line(const double* f, double* ql, double* qr, int is, int ie, double epsw, int imax, int nq);
void ho_weno_deriv_line(const double* f, double* ql, double* qr, const double* dq, int is, int ie, double eps,
                        int imax, int nq);

/* The 5-variable (3D strand) functions, reachable only from the reference's
 * -DDim3 build (which does not compile, io.cpp:306) but compiled in every
 * build: SOLVER::fluxRoe3D (interfaceFlux.cpp:176-319, flux and spectral
 * radius not scaled by the area), jacobianRoe3D (jacobianRoe.cpp:92-620,
 * IMODE 1; lm, rm [5][5]) and TRISOLVER::blockTridag / blockTridagPeriodic
 * (triSolvers.cpp:443-766; a, b, c [N][5][5] and f [N][5] in place, a, b, c
 * overwritten as the reference's scratch). */
void ho_flux_roe3d(const double* nxyz, const double* ql, const double* qr, double* flux, double* spec, double gamma);
void ho_jacobian_roe3d(const double* nxyz, const double* ql, const double* qr, double* lm, double* rm, double gamma);
int  ho_block_tridag5(double* a, double* b, double* c, double* f, int N, int periodic);

/* Named arrays: q qt r r0 dq sigma ff x vol normVec refMtx (doubles) and
 * faces chainConn faceStartPerChain c2chain bFaces chainsPerColor (ints). */
int ho_get(const ho_case* c, const char* name, double* out);
int ho_set(ho_case* c, const char* name, const double* in);
int ho_get_int(const ho_case* c, const char* name, int* out);

#ifdef __cplusplus
}
#endif
#endif
