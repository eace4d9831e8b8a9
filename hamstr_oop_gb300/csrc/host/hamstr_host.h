// ##################################################################
//
// hamstr_host.h -- drop-in C++ classes of the reference's driver layer
//
// Same class names, public methods and argument meaning as the reference
// (hamstr.h:16-49, meshBlock.h:15-73, solnBlock.h:13-91, solver.h:14-55).
// Differences a caller sees:
//   * errors throw hamstr::Error instead of calling exit(1)
//     (io.cpp:19-23,138-141; interfaceFlux.cpp:117-124);
//   * the solution lives on the GPU; SOLVER::syncHost() refreshes the
//     SOLNBLOCK host arrays (q, r, r0, dq, sigma, ff), and marchInTime()
//     does so at its end;
//   * readMeshData / readSolutionInputs also accept a case root directory
//     (the reference reads ./input... from the working directory).
// ##################################################################
#ifndef HAMSTR_HOST_H
#define HAMSTR_HOST_H

#include <stdexcept>
#include <string>
#include <vector>

#include "../../../include/hamstr_gpu.h"

namespace hamstr {
struct Error : std::runtime_error {
   int status;
   Error(int st, const std::string& m) : std::runtime_error(m), status(st) {}
};
}  // namespace hamstr

struct hamstr_case;

// ------------------------------------------------------------------
class MESHBLOCK
{
   friend class SOLVER;
   friend struct hamstr_case;

  private:
   int myid = 0;
   int nNode = 0, nCell = 0, nFace = 0, nBface = 0, nColor = 0;
   int nChain = 0, nMaxChain = 0, nChainFace = 0, nStrand = 0;
   int sol_visc = 0;
   std::vector<int> conn, faces, chainsPerColor, faceStartPerChain, chainConn;
   std::vector<int> c2chain, bFaces;
   std::vector<double> vol, x, normVec, refMtx;   // normVec [nFace][2], refMtx [nFace][2][2]
   double volmax = 0.0, volmin = 0.0;

  public:
   MESHBLOCK() {}
   ~MESHBLOCK() {}
   // io.cpp:58-372; root "" means the working directory
   void readMeshData(int myid);
   void readMeshData(int myid, const std::string& root);
   // preprocess.cpp:15-241
   void preprocess(void);
   void setViscosity(int visc) { sol_visc = visc; }
};

// ------------------------------------------------------------------
class SOLNBLOCK
{
   friend class SOLVER;
   friend struct hamstr_case;
   friend void hamstr_init_flow(SOLNBLOCK& sb, int nCell);
   friend void hamstr_freestream(SOLNBLOCK& sb, int nCell);

  private:
   int order = 3, timeacc = 0, nsteps = 0, nwrite = 0, msweep = 1, test = 0, outform = 0;
   double Mach = 0, alpha = 0, beta = 0, rey = 0, CFL = 0, dt = 0;
   char timeInteg[64] = {0};
   char scheme[64] = {0};
   int visc = 0;
   int nGhost = 2;
   int chainEndRule = 0;   // project option: HAMSTR_END_RULE_* (not in the reference)
   int limiter = 0;        // project option: HAMSTR_LIMITER_* (not in the reference)
   double uinf = 0, vinf = 0, winf = 0, einf = 0, pinf = 0, rinf = 0;
   double gamma = 0, invGamma = 0, gm1 = 0, c2b = 0, rgas = 0, pr = 0, prtr = 0;
   double LInfNorm = 0, L2Norm = 0;
   // host copies of the solution (refreshed by SOLVER::syncHost)
   std::vector<double> q, qt, r, r0, dq, sigma, ff;

  public:
   SOLNBLOCK() {}
   ~SOLNBLOCK() {}
   // io.cpp:13-51
   void readSolutionInputs(void);
   void readSolutionInputs(const std::string& root);
   // project addition: HAMSTR_END_RULE_* for meshes whose open chains end
   // at interior faces (mixed tri/quad meshes); throws on other values
   void setChainEndRule(int rule);
   // project addition: HAMSTR_LIMITER_* for order 3; throws on other values
   void setLimiter(int lim);
};

// ------------------------------------------------------------------
class SOLVER
{
  private:
   double dt = 0;
   const char* stepType = nullptr;
   MESHBLOCK* mb;
   SOLNBLOCK* sb;
   hamstr_gpu* gpu = nullptr;
   void ensureGpu();

  public:
   SOLVER(MESHBLOCK* mbin, SOLNBLOCK* sbin);
   ~SOLVER();
   void initFlow(void);                  // initFlow.cpp:12-93
   void marchInTime(void);               // march.cpp:15-59
   void stepSolution(void);              // march.cpp:66-134 (ADI, euler, rk3)
   void updateSolution(double* qold, double* qnew, double coef);   // march.cpp:411-433
   void computeRHS(char* option);        // computeRHS.cpp:17-427
   void computeLinearRHS(void);          // computeLinearRHS.cpp:13-371
   void ADI(void);                       // ADI.cpp:15-266
   void basicScreenOutput(void);         // io.cpp:412-446
   // interfaceFlux.cpp:24-169: one face on the GPU (hamstr_gpu_flux_roe2d);
   // a NaN spectral radius throws hamstr::Error (HAMSTR_GPU_ERR_NAN) where
   // the reference exits
   void fluxRoe2D(double* nxyz, double* ql, double* qr, double* flux, double* specRadius, double gamma);
   // jacobianRoe.cpp:9-70: one face on the GPU (hamstr_gpu_jacobian_roe2d)
   void jacobianRoe2D(double* nxyz, double* ql, double* qr, double** lmat, double** rmat, double gamma);
   void syncHost(void);
   hamstr_gpu* device(void) { ensureGpu(); return gpu; }
   double l2Norm() const { return sb->L2Norm; }
   double lInfNorm() const { return sb->LInfNorm; }
};

// ------------------------------------------------------------------
class HAMSTR
{
  private:
   int nGrid, procID;
   MESHBLOCK* mb;
   SOLNBLOCK* sb;
   SOLVER* solv = nullptr;
   std::string root;

  public:
   HAMSTR(const int nprocs, const int myid, const std::string& root = "");
   ~HAMSTR();
   void readInputs(int myid);            // hamstr.cpp:33-48
   void preprocessor(void);              // hamstr.cpp:54-66
   void marchInTime(void);               // hamstr.cpp:72-77
   void welcome(void);
   void thanks(void);
   SOLVER* solver() { return solv; }
};

// ------------------------------------------------------------------
// The reference's numerics namespaces (reconstruction.h:11-110,
// triSolvers.h:18-46) over host arrays, each call run on the GPU through
// the function-level C ABI (hamstr_gpu_muscl etc., hamstr_gpu_block_tridag4)
// with the same arguments and results.  Differences a caller sees: errors
// throw hamstr::Error; MUSCL and MUSCL_DERIV with qt != 0 at ie = imax-1
// (computeRHS.cpp:267's call) leave entry imax-1 of ql and qr as it was
// (the reference fills it from work-array entries left by an earlier
// chain, and its callers never read it); blockTridag4 and
// blockTridagPeriodic4 leave b and c unchanged (the reference uses them as
// scratch) and need nq == 4.
namespace RECONSTRUCTION {
void MUSCL(double** f, double** ql, double** qr, double** f2, int is, int ie, double th, double qt, double eps,
           int imax, int nq);
void WENO(double** f, double** ql, double** qr, int is, int ie, double epsw, int imax, int nq);
void MUSCL_DERIV(double** f, double** ql, double** qr, double** f2, double** dq, int is, int ie, double th, double qt,
                 double eps, int imax, int nq);
void WENO_DERIV(double** f, double** ql, double** qr, double** dq, int is, int ie, double eps, int imax, int nq);
}  // namespace RECONSTRUCTION

namespace TRISOLVER {
void blockTridag4(double*** a, double*** b, double*** c, double** f, int N, int nq);
void blockTridagPeriodic4(double*** a, double*** b, double*** c, double** f, int N, int nq);
}  // namespace TRISOLVER

// freestream + initial state (initFlow.cpp:12-93) on host arrays
void hamstr_init_flow(SOLNBLOCK& sb, int nCell);
// the freestream part of initFlow.cpp:24-91 from sb.Mach and sb.alpha
void hamstr_freestream(SOLNBLOCK& sb, int nCell);

// the C handle behind hamstr_case_* (api.cu)
struct hamstr_case {
   MESHBLOCK mb;
   SOLNBLOCK sb;
   // reference order of the flat accessors
   static void sizes(const hamstr_case& c, int* out);
   static void params(const hamstr_case& c, double* out);
   static int get_int(const hamstr_case& c, const std::string& name, int* out, int* count);
   static int get(const hamstr_case& c, const std::string& name, double* out);
   static void set_run(hamstr_case& c, int order, int msweep, double cfl);
   static void set_freestream(hamstr_case& c, double u, double v, double e);
   static int set_option(hamstr_case& c, const std::string& name, int value);
   static void set_flow(hamstr_case& c, double mach, double alpha);
   static hamstr_gpu_params gpu_params(const hamstr_case& c);
   static void load(hamstr_case& c, const std::string& dir);
   static int create_gpu(const hamstr_case& c, hamstr_gpu** out);
   static int create_batch(const hamstr_case* const* cs, int n, hamstr_gpu** out);
};

#endif
