// ##################################################################
//
// hamstr_host.cpp -- reader, preprocessing and driver classes
//
// Host C++, compiled with -ffp-contract=off so that the normals and
// reflection matrices (the only floating-point work here) round exactly
// as the reference's x86-64 build does, on x86-64 and aarch64 alike.
// ##################################################################
#include "hamstr_host.h"

#include "../api_internal.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <memory>

namespace {

using hamstr::Error;

struct File {
   FILE* fp = nullptr;
   explicit File(const std::string& p) : fp(std::fopen(p.c_str(), "r")) {}
   ~File() { if (fp) std::fclose(fp); }
};

std::string domain_dir(const std::string& root, int myid)
{
   char d[64];
   std::snprintf(d, sizeof(d), "input/domain%03d/", myid);   // io.cpp:72-128
   return (root.empty() ? std::string("./") : root + "/") + d;
}

[[noreturn]] void missing(const std::string& p)
{
   throw Error(HAMSTR_GPU_ERR_IO, "File missing - " + p);
}

[[noreturn]] void malformed(const std::string& p)
{
   throw Error(HAMSTR_GPU_ERR_IO, "malformed file - " + p);
}

}  // namespace

// ==================================================================
// MESHBLOCK::readMeshData (io.cpp:58-372)
// ==================================================================
void MESHBLOCK::readMeshData(int id) { readMeshData(id, ""); }

void MESHBLOCK::readMeshData(int id, const std::string& root)
{
   myid = id;
   if (id >= 1000) throw Error(HAMSTR_GPU_ERR_ARG, "domain id beyond 999");
   const std::string dir = domain_dir(root, id);
   {  // coordinates: nNode, then x y z (z ignored in 2D)
      const std::string p = dir + "coord.dat";
      File f(p);
      if (!f.fp) missing(p);
      if (std::fscanf(f.fp, "%d", &nNode) != 1 || nNode < 0) malformed(p);
      x.assign(2 * (size_t)nNode, 0.0);
      double z;
      for (int i = 0; i < nNode; i++)
         if (std::fscanf(f.fp, "%lf %lf %lf\n", &x[2 * i], &x[2 * i + 1], &z) != 3) malformed(p);
   }
   {  // connectivity (read, unused by the path)
      const std::string p = dir + "conn.dat";
      File f(p);
      if (!f.fp) missing(p);
      if (std::fscanf(f.fp, "%d", &nCell) != 1 || nCell < 0) malformed(p);
      conn.assign(4 * (size_t)nCell, 0);
      for (int i = 0; i < nCell; i++)
         if (std::fscanf(f.fp, "%d %d %d %d\n", &conn[4 * i], &conn[4 * i + 1], &conn[4 * i + 2], &conn[4 * i + 3]) != 4)
            malformed(p);
   }
   {  // colours (read, unused by the reference)
      const std::string p = dir + "ncolors.dat";
      File f(p);
      if (!f.fp) missing(p);
      if (std::fscanf(f.fp, "%d", &nColor) != 1 || nColor < 0) malformed(p);
      chainsPerColor.assign(nColor, 0);
      for (int i = 0; i < nColor; i++)
         if (std::fscanf(f.fp, "%d\n", &chainsPerColor[i]) != 1) malformed(p);
   }
   {  // chain start offsets; a repeated offset (empty chain) is dropped
      const std::string p = dir + "iqloops.dat";
      File f(p);
      if (!f.fp) missing(p);
      int k = 0;
      if (std::fscanf(f.fp, "%d\n", &k) != 1 || k < 1) malformed(p);
      faceStartPerChain.assign(k, 0);
      nMaxChain = 0;
      int j = 0;
      for (int i = 0; i < k; i++) {
         if (std::fscanf(f.fp, "%d\n", &faceStartPerChain[j]) != 1) malformed(p);
         if (i > 0) {
            if (faceStartPerChain[j] == faceStartPerChain[j - 1]) j--;
            // the reference reads index -1 when the first two offsets repeat
            if (j > 0) nMaxChain = std::max(nMaxChain, faceStartPerChain[j] - faceStartPerChain[j - 1]);
         }
         j++;
      }
      nChain = j - 1;
      faceStartPerChain.resize(nChain + 1);
   }
   {  // chain faces
      const std::string p = dir + "qloops.dat";
      File f(p);
      if (!f.fp) missing(p);
      if (std::fscanf(f.fp, "%d", &nChainFace) != 1 || nChainFace < 0) malformed(p);
      chainConn.assign(nChainFace, 0);
      for (int i = 0; i < nChainFace; i++)
         if (std::fscanf(f.fp, "%d", &chainConn[i]) != 1) malformed(p);
   }
   {  // faces: n1 n2 cL cR eL eR stored as n1 n2 cL eL cR eR; left -1 swaps
      const std::string p = dir + "qedges.dat";
      File f(p);
      if (!f.fp) missing(p);
      if (std::fscanf(f.fp, "%d", &nFace) != 1 || nFace < 0) malformed(p);
      faces.assign(6 * (size_t)nFace, 0);
      for (int i = 0; i < nFace; i++) {
         int* r = &faces[6 * (size_t)i];
         if (std::fscanf(f.fp, "%d %d %d %d %d %d\n", &r[0], &r[1], &r[2], &r[4], &r[3], &r[5]) != 6) malformed(p);
         if (r[2] == -1) {
            std::swap(r[0], r[1]);
            std::swap(r[2], r[4]);
            std::swap(r[3], r[5]);
         }
      }
   }
   for (int i = 0; i < nFace; i++)
      for (int k = 0; k < 2; k++) {
         const int n = faces[6 * (size_t)i + k];
         if (n < 0 || n >= nNode) throw Error(HAMSTR_GPU_ERR_TOPOLOGY, "face names a missing node");
      }
   for (int i = 0; i < nFace; i++) {
      const int l = faces[6 * (size_t)i + 2];
      if (l < 0 || l >= nCell) throw Error(HAMSTR_GPU_ERR_TOPOLOGY, "face has no valid left cell");
   }
}

// ==================================================================
// MESHBLOCK::preprocess (preprocess.cpp:15-241)
// ==================================================================
void MESHBLOCK::preprocess(void)
{
   const double boundaryLimit = 3.0;   // preprocess.cpp:9
   vol.assign(nCell, 0.0);
   normVec.assign(2 * (size_t)nFace, 0.0);
   refMtx.assign(4 * (size_t)nFace, 0.0);
   bFaces.assign(nFace, 0);
   c2chain.assign(2 * (size_t)nCell, -1);
   int m = 0;
   for (int i = 0; i < nFace; i++) {
      int* fr = &faces[6 * (size_t)i];
      const int left = fr[2], right = fr[4];
      const double x1 = x[2 * fr[0]], y1 = x[2 * fr[0] + 1];
      const double x2 = x[2 * fr[1]], y2 = x[2 * fr[1] + 1];
      const double nx = (y2 - y1);
      const double ny = -(x2 - x1);
      normVec[2 * i] = nx;
      normVec[2 * i + 1] = ny;
      const double dvedge = 0.5 * (x1 * y2 - x2 * y1);
      double ds = nx * nx + ny * ny;
      ds = 1. / ds;
      double* R = &refMtx[4 * (size_t)i];
      R[0] = 1. - 2. * nx * nx * ds;
      R[1] = -2. * nx * ny * ds;
      R[2] = -2. * ny * nx * ds;
      R[3] = 1. - 2. * ny * ny * ds;
      vol[left] += dvedge;
      if (right > -1) vol[right] -= dvedge;
      if (right == -1) {
         const double r1 = std::sqrt(x1 * x1 + y1 * y1);
         const double r2 = std::sqrt(x2 * x2 + y2 * y2);
         if (0.5 * (r1 + r2) < boundaryLimit) {
            bFaces[m++] = i;
            fr[4] = -(sol_visc + 2);
         }
      }
   }
   nBface = m;
   bFaces.resize(m);
   volmin = 1.0e+15;
   volmax = 0.0;
   for (int i = 0; i < nCell; i++) {
      volmin = (volmin < vol[i]) ? volmin : vol[i];
      volmax = (volmax > vol[i]) ? volmax : vol[i];
   }
   for (int i = 0; i < nChain; i++)
      for (int f = faceStartPerChain[i]; f < faceStartPerChain[i + 1] - 1; f++) {
         const int left = faces[6 * (size_t)chainConn[f] + 2];
         if (c2chain[2 * left] > -1) c2chain[2 * left + 1] = i;
         else c2chain[2 * left] = i;
      }
}

// ==================================================================
// SOLNBLOCK::readSolutionInputs (io.cpp:13-51)
// ==================================================================
void SOLNBLOCK::readSolutionInputs(void) { readSolutionInputs(""); }

void SOLNBLOCK::setChainEndRule(int rule)
{
   if (rule != HAMSTR_END_RULE_REFERENCE && rule != HAMSTR_END_RULE_EXTENDED)
      throw hamstr::Error(HAMSTR_GPU_ERR_ARG, "unknown chain end rule");
   chainEndRule = rule;
}

void SOLNBLOCK::setLimiter(int lim)
{
   if (lim < HAMSTR_LIMITER_REFERENCE || lim > HAMSTR_LIMITER_VANALBADA)
      throw hamstr::Error(HAMSTR_GPU_ERR_ARG, "unknown limiter");
   limiter = lim;
}

void SOLNBLOCK::readSolutionInputs(const std::string& root)
{
   const std::string p = (root.empty() ? std::string("") : root + "/") + "input.hamstr";
   File f(p);
   if (!f.fp) throw Error(HAMSTR_GPU_ERR_IO, "Error: Input file 'input.hamstr' missing (" + p + ")");
   bool ok = true;
   ok &= std::fscanf(f.fp, "Mach=%lf\n", &Mach) == 1;
   ok &= std::fscanf(f.fp, "alpha=%lf\n", &alpha) == 1;
   ok &= std::fscanf(f.fp, "beta=%lf\n", &beta) == 1;
   ok &= std::fscanf(f.fp, "rey=%lf\n", &rey) == 1;
   ok &= std::fscanf(f.fp, "scheme=%63s\n", scheme) == 1;
   ok &= std::fscanf(f.fp, "time integration=%63s\n", timeInteg) == 1;
   ok &= std::fscanf(f.fp, "order=%d\n", &order) == 1;
   ok &= std::fscanf(f.fp, "timeacc=%d\n", &timeacc) == 1;
   ok &= std::fscanf(f.fp, "nsteps=%d\n", &nsteps) == 1;
   ok &= std::fscanf(f.fp, "nwrite=%d\n", &nwrite) == 1;
   ok &= std::fscanf(f.fp, "dt=%lf\n", &dt) == 1;
   ok &= std::fscanf(f.fp, "CFL=%lf\n", &CFL) == 1;
   ok &= std::fscanf(f.fp, "msweep=%d\n", &msweep) == 1;
   ok &= std::fscanf(f.fp, "visc=%d\n", &visc) == 1;
   ok &= std::fscanf(f.fp, "testcase=%d\n", &test) == 1;
   ok &= std::fscanf(f.fp, "output=%d\n", &outform) == 1;
   if (!ok) throw Error(HAMSTR_GPU_ERR_IO, "malformed " + p);
   if (test != 0) throw Error(HAMSTR_GPU_ERR_ARG, "ERROR: Code not implemented for all test cases");
}

// ==================================================================
// initFlow (initFlow.cpp:12-93)
// ==================================================================
void hamstr_init_flow(SOLNBLOCK& sb, int nCell)
{
   sb.gamma = 1.4;
   sb.gm1 = sb.gamma - 1.;
   sb.invGamma = 1. / sb.gamma;
   sb.pr = 0.72;
   sb.prtr = 0.3333333333333333e+00;
   sb.rinf = 1.0;
   sb.pinf = 1.0 / sb.gamma;
   sb.rey = sb.rey / sb.Mach;
   sb.nGhost = (sb.order == 5) ? 3 : 2;
   if (sb.test != 0) throw Error(HAMSTR_GPU_ERR_ARG, "HAMSTR: test condition not implemented");
   hamstr_freestream(sb, nCell);
}

void hamstr_freestream(SOLNBLOCK& sb, int nCell)
{
   const double deg2rad = 3.1415926535897932e+00 / 180.0;   // utils.h:55-57
   sb.uinf = sb.Mach * std::cos(sb.alpha * deg2rad);
   sb.vinf = sb.Mach * std::sin(sb.alpha * deg2rad);
   sb.einf = sb.pinf / (sb.gm1) + 0.5 * sb.rinf * (sb.uinf * sb.uinf + sb.vinf * sb.vinf);
   sb.q.assign(4 * (size_t)nCell, 0.0);
   for (int i = 0; i < nCell; i++) {
      sb.q[4 * (size_t)i + 0] = sb.rinf;
      sb.q[4 * (size_t)i + 1] = sb.rinf * sb.uinf;
      sb.q[4 * (size_t)i + 2] = sb.rinf * sb.vinf;
      sb.q[4 * (size_t)i + 3] = sb.einf;
   }
   sb.qt = sb.q;
}

// ==================================================================
// SOLVER
// ==================================================================
namespace {
void check(int st)
{
   if (st != HAMSTR_GPU_OK) {
      std::string m = hamstr_gpu_strerror(st);
      const char* d = hamstr_gpu_last_error();
      if (d && *d) m += std::string(": ") + d;
      throw Error(st, m);
   }
}
}  // namespace

SOLVER::SOLVER(MESHBLOCK* mbin, SOLNBLOCK* sbin) : mb(mbin), sb(sbin)
{
   stepType = sb->scheme;
   const size_t nc = (size_t)mb->nCell;
   sb->q.assign(4 * nc, 0.0);
   sb->qt.assign(4 * nc, 0.0);
   sb->r.assign(4 * nc, 0.0);
   sb->r0.assign(4 * nc, 0.0);
   sb->dq.assign(4 * nc, 0.0);
   sb->sigma.assign(nc, 0.0);
   sb->ff.assign(32 * (size_t)mb->nFace, 0.0);
}

SOLVER::~SOLVER()
{
   if (gpu) hamstr_gpu_destroy(gpu);
}

void SOLVER::initFlow(void)
{
   hamstr_init_flow(*sb, mb->nCell);
   if (gpu) check(hamstr_gpu_set(gpu, "q", sb->q.data()));
}

void SOLVER::ensureGpu()
{
   if (gpu) return;
   hamstr_gpu_params p;
   p.order = sb->order;
   p.msweep = sb->msweep;
   p.CFL = sb->CFL;
   p.gamma = sb->gamma;
   p.rinf = sb->rinf;
   p.uinf = sb->uinf;
   p.vinf = sb->vinf;
   p.einf = sb->einf;
   p.chain_end_rule = sb->chainEndRule;
   p.limiter = sb->limiter;
   check(hamstr_gpu_create(&p, mb->nCell, mb->nFace, mb->faces.data(), mb->normVec.data(), mb->refMtx.data(),
                           mb->nChain, mb->faceStartPerChain.data(), mb->chainConn.data(), &gpu));
   check(hamstr_gpu_set_geometry(gpu, mb->nNode, mb->x.data()));
   check(hamstr_gpu_set(gpu, "q", sb->q.data()));
}

void SOLVER::computeRHS(char* option)
{
   ensureGpu();
   const int implicit = (std::strcmp(option, "implicit") == 0) ? 1 : 0;
   check(hamstr_gpu_compute_rhs(gpu, implicit, &sb->L2Norm, &sb->LInfNorm));
}

void SOLVER::computeLinearRHS(void)
{
   ensureGpu();
   check(hamstr_gpu_linear_rhs(gpu, &sb->L2Norm, &sb->LInfNorm));
}

void SOLVER::ADI(void)
{
   ensureGpu();
   check(hamstr_gpu_adi(gpu, &sb->L2Norm, &sb->LInfNorm));
}

void SOLVER::stepSolution(void)
{
   ensureGpu();
   if (std::strcmp(stepType, "ADI") == 0) {
      double n4[4];
      check(hamstr_gpu_step(gpu, n4));
      sb->L2Norm = n4[2];
      sb->LInfNorm = n4[3];
      return;
   }
   int scheme = -1;
   if (std::strcmp(stepType, "euler") == 0) scheme = 0;
   if (std::strcmp(stepType, "rk3") == 0) scheme = 1;
   if (scheme < 0)
      throw Error(HAMSTR_GPU_ERR_ARG, std::string("unknown time marching scheme '") + stepType + "'");
   if (scheme == 0 && sb->visc)
      throw Error(HAMSTR_GPU_ERR_ARG, "viscous explicit step not implemented (march.cpp:344-349)");
   double n2[2];
   check(hamstr_gpu_step_explicit(gpu, scheme, n2));
   sb->L2Norm = n2[0];
   sb->LInfNorm = n2[1];
}

void SOLVER::updateSolution(double* qold, double* qnew, double coef)
{
   // the reference passes its q / qt host arrays; the device copies are updated
   ensureGpu();
   auto name = [&](const double* p) -> const char* {
      if (p == sb->q.data()) return "q";
      if (p == sb->qt.data()) return "qt";
      throw Error(HAMSTR_GPU_ERR_ARG, "updateSolution takes the solver's q or qt arrays");
   };
   check(hamstr_gpu_update_solution(gpu, name(qold), name(qnew), coef));
}

void SOLVER::syncHost(void)
{
   ensureGpu();
   check(hamstr_gpu_get(gpu, "q", sb->q.data()));
   check(hamstr_gpu_get(gpu, "qt", sb->qt.data()));
   check(hamstr_gpu_get(gpu, "r", sb->r.data()));
   check(hamstr_gpu_get(gpu, "r0", sb->r0.data()));
   check(hamstr_gpu_get(gpu, "dq", sb->dq.data()));
   check(hamstr_gpu_get(gpu, "sigma", sb->sigma.data()));
   check(hamstr_gpu_get(gpu, "ff", sb->ff.data()));
}

void SOLVER::marchInTime(void)
{
   // march.cpp:15-59: nsteps steps and the per-step table
   ensureGpu();
   double cpuTime = 0.0;
   for (int n = 0; n < sb->nsteps; n++) {
      const std::clock_t start = std::clock();
      stepSolution();
      const std::clock_t stop = std::clock();
      cpuTime += ((double)(stop - start)) / CLOCKS_PER_SEC;
      if (n == 0) {
         std::printf("\n --------------------------------------------------------------\n");
         std::printf(" |   Iter  | L_2 (density) | L_inf (density) | CPU Time (sec) |\n");
         std::printf(" --------------------------------------------------------------\n");
      }
      std::printf(" |  %*d  |  %e |   %e  |  %e  |\n", 5, n, sb->L2Norm, sb->LInfNorm, cpuTime);
      if (n == sb->nsteps - 1) {
         std::printf(" --------------------------------------------------------------\n");
         std::printf(" |   Iter  | L_2 (density) | L_inf (density) | CPU Time (sec) |\n");
         std::printf(" --------------------------------------------------------------\n");
      }
   }
   syncHost();
}

void SOLVER::basicScreenOutput(void)
{
   std::printf("======================================================================\n");
   std::printf("                       GRID RELATED OUTPUTS                           \n");
   std::printf("======================================================================\n\n");
   std::printf(" Number of nodes            %d\n", mb->nNode);
   std::printf(" Number of cells            %d\n", mb->nCell);
   std::printf(" Number of faces            %d\n", mb->nFace);
   std::printf(" Number of colours          %d\n", mb->nColor);
   std::printf(" Number of chains           %d\n", mb->nChain);
   std::printf(" Number of chain faces      %d\n", mb->nChainFace);
   std::printf(" Maximum length of chain    %d\n", mb->nMaxChain);
   std::printf(" Minimum cell volume        %0.8e\n", mb->volmin);
   std::printf(" Maximum cell volume        %0.8e\n\n", mb->volmax);
   std::printf("======================================================================\n");
   std::printf("                  SOLVER AND FLOW RELATED OUTPUTS                     \n");
   std::printf("======================================================================\n\n");
   std::printf(" Mach number                %0.8e\n", sb->Mach);
   std::printf(" Alpha                      %0.8e\n", sb->alpha);
   std::printf(" U infinity                 %0.8e\n", sb->uinf);
   std::printf(" V infinity                 %0.8e\n", sb->vinf);
   std::printf(" CFL number                 %0.8e\n", sb->CFL);
   std::printf(" Number of steps            %d\n", sb->nsteps);
   std::printf(" Time marching scheme       %s\n", sb->scheme);
   std::printf(" Time integration scheme    %s\n", sb->timeInteg);
   std::printf(" Reconstruction accuracy    %d\n\n", sb->order);
   std::printf("======================================================================\n");
}

// ==================================================================
// HAMSTR (hamstr.cpp:14-77)
// ==================================================================
HAMSTR::HAMSTR(const int nprocs, const int myid, const std::string& r)
    : nGrid(nprocs), procID(myid), mb(new MESHBLOCK), sb(new SOLNBLOCK), root(r)
{
}

HAMSTR::~HAMSTR()
{
   delete solv;
   delete mb;
   delete sb;
}

void HAMSTR::readInputs(int myid)
{
   std::printf("\n HAMSTR: Read input files ... ");
   mb->readMeshData(myid, root);
   sb->readSolutionInputs(root);
   solv = new SOLVER(mb, sb);
   std::printf(" [done]\n");
}

void HAMSTR::preprocessor(void)
{
   std::printf(" HAMSTR: Preprocess data  ... ");
   mb->setViscosity(0);   // the inviscid wall tag; the reference never sets it
   mb->preprocess();
   std::printf(" [done]\n");
   std::printf(" HAMSTR: Initialize flow  ... ");
   solv->initFlow();
   std::printf(" [done]\n");
   solv->basicScreenOutput();
}

void HAMSTR::marchInTime(void)
{
   std::printf(" HAMSTR: Marching in time ... \n");
   solv->marchInTime();
}

void HAMSTR::welcome(void)
{
   std::printf("\n######################################################################\n");
   std::printf("#                                                                    #\n");
   std::printf("#                      HAMSTR  (GB300 path)                          #\n");
   std::printf("#                                                                    #\n");
   std::printf("######################################################################\n");
}

void HAMSTR::thanks(void)
{
   std::printf("\n######################################################################\n");
   std::printf("#                       END OF SIMULATION                            #\n");
   std::printf("######################################################################\n");
}

// ==================================================================
// hamstr_case accessors (flat views for the C ABI)
// ==================================================================
void hamstr_case::sizes(const hamstr_case& c, int* o)
{
   o[0] = c.mb.nCell; o[1] = c.mb.nFace; o[2] = c.mb.nChain; o[3] = c.mb.nChainFace;
   o[4] = c.mb.nMaxChain; o[5] = c.sb.order; o[6] = c.sb.msweep; o[7] = c.sb.nGhost;
   o[8] = c.mb.nNode; o[9] = c.mb.nColor;
}

void hamstr_case::params(const hamstr_case& c, double* o)
{
   o[0] = c.sb.Mach; o[1] = c.sb.alpha; o[2] = c.sb.CFL; o[3] = c.sb.gamma; o[4] = c.sb.rinf;
   o[5] = c.sb.uinf; o[6] = c.sb.vinf; o[7] = c.sb.einf; o[8] = c.sb.pinf;
}

int hamstr_case::get_int(const hamstr_case& c, const std::string& n, int* out, int* count)
{
   const std::vector<int>* v = nullptr;
   if (n == "faces") v = &c.mb.faces;
   else if (n == "chainConn") v = &c.mb.chainConn;
   else if (n == "faceStartPerChain") v = &c.mb.faceStartPerChain;
   else if (n == "c2chain") v = &c.mb.c2chain;
   else if (n == "bFaces") v = &c.mb.bFaces;
   else if (n == "chainsPerColor") v = &c.mb.chainsPerColor;
   else return HAMSTR_GPU_ERR_ARG;
   if (count) *count = (int)v->size();
   if (out) std::memcpy(out, v->data(), sizeof(int) * v->size());
   return HAMSTR_GPU_OK;
}

int hamstr_case::get(const hamstr_case& c, const std::string& n, double* out)
{
   const std::vector<double>* v = nullptr;
   if (n == "x") v = &c.mb.x;
   else if (n == "vol") v = &c.mb.vol;
   else if (n == "normVec") v = &c.mb.normVec;
   else if (n == "refMtx") v = &c.mb.refMtx;
   else if (n == "q") v = &c.sb.q;
   else return HAMSTR_GPU_ERR_ARG;
   std::memcpy(out, v->data(), sizeof(double) * v->size());
   return HAMSTR_GPU_OK;
}

void hamstr_case::set_run(hamstr_case& c, int order, int msweep, double cfl)
{
   c.sb.order = order;
   c.sb.msweep = msweep;
   c.sb.CFL = cfl;
   c.sb.nGhost = (order == 5) ? 3 : 2;
}

void hamstr_case::set_freestream(hamstr_case& c, double u, double v, double e)
{
   c.sb.uinf = u;
   c.sb.vinf = v;
   c.sb.einf = e;
   for (int i = 0; i < c.mb.nCell; i++) {
      c.sb.q[4 * (size_t)i + 0] = c.sb.rinf;
      c.sb.q[4 * (size_t)i + 1] = c.sb.rinf * u;
      c.sb.q[4 * (size_t)i + 2] = c.sb.rinf * v;
      c.sb.q[4 * (size_t)i + 3] = e;
   }
}

void hamstr_case::set_flow(hamstr_case& c, double mach, double alpha)
{
   c.sb.Mach = mach;
   c.sb.alpha = alpha;
   hamstr_freestream(c.sb, c.mb.nCell);
}

int hamstr_case::set_option(hamstr_case& c, const std::string& name, int value)
{
   if (name == "chain_end_rule") {
      if (value != HAMSTR_END_RULE_REFERENCE && value != HAMSTR_END_RULE_EXTENDED) return HAMSTR_GPU_ERR_ARG;
      c.sb.chainEndRule = value;
      return HAMSTR_GPU_OK;
   }
   if (name == "limiter") {
      if (value < HAMSTR_LIMITER_REFERENCE || value > HAMSTR_LIMITER_VANALBADA) return HAMSTR_GPU_ERR_ARG;
      c.sb.limiter = value;
      return HAMSTR_GPU_OK;
   }
   return HAMSTR_GPU_ERR_ARG;
}

void hamstr_case::load(hamstr_case& c, const std::string& dir)
{
   c.mb.readMeshData(0, dir);
   c.sb.readSolutionInputs(dir);
   c.mb.setViscosity(0);
   c.mb.preprocess();
   hamstr_init_flow(c.sb, c.mb.nCell);
}

int hamstr_case::create_gpu(const hamstr_case& c, hamstr_gpu** out)
{
   const hamstr_gpu_params p = gpu_params(c);
   int st = hamstr_gpu_create(&p, c.mb.nCell, c.mb.nFace, c.mb.faces.data(), c.mb.normVec.data(),
                              c.mb.refMtx.data(), c.mb.nChain, c.mb.faceStartPerChain.data(),
                              c.mb.chainConn.data(), out);
   if (st != HAMSTR_GPU_OK) return st;
   st = hamstr_gpu_set_geometry(*out, c.mb.nNode, c.mb.x.data());
   if (st == HAMSTR_GPU_OK) st = hamstr_gpu_set(*out, "q", c.sb.q.data());
   if (st != HAMSTR_GPU_OK) {
      hamstr_gpu_destroy(*out);
      *out = nullptr;
   }
   return st;
}

int hamstr_case::create_batch(const hamstr_case* const* cs, int n, hamstr_gpu** out)
{
   const hamstr_gpu_params p0 = gpu_params(*cs[0]);
   for (int k = 1; k < n; k++) {
      const hamstr_gpu_params p = gpu_params(*cs[k]);
      if (p.order != p0.order || p.msweep != p0.msweep || p.CFL != p0.CFL || p.gamma != p0.gamma ||
          p.limiter != p0.limiter || p.chain_end_rule != p0.chain_end_rule) {
         hamstr::set_last_error("batched cases must share order, msweep, CFL, gamma, limiter and chain end rule");
         return HAMSTR_GPU_ERR_ARG;
      }
   }
   // disjoint union: ids of case k shifted past those of cases 0..k-1
   std::vector<int> faces, fsp, cc;
   std::vector<double> normVec, refMtx, x, q;
   hamstr::InstanceInfo info;
   info.n = n;
   info.cell0.push_back(0);
   info.chain0.push_back(0);
   int co = 0, fo = 0, no = 0, cfo = 0, cho = 0;
   for (int k = 0; k < n; k++) {
      const MESHBLOCK& mb = cs[k]->mb;
      const SOLNBLOCK& sb = cs[k]->sb;
      for (int f = 0; f < mb.nFace; f++) {
         const int* r = &mb.faces[6 * (size_t)f];
         faces.insert(faces.end(), {r[0] + no, r[1] + no, r[2] + co, r[3], r[4] >= 0 ? r[4] + co : r[4], r[5]});
      }
      normVec.insert(normVec.end(), mb.normVec.begin(), mb.normVec.end());
      refMtx.insert(refMtx.end(), mb.refMtx.begin(), mb.refMtx.end());
      x.insert(x.end(), mb.x.begin(), mb.x.end());
      for (int c = 0; c < mb.nChain; c++) fsp.push_back(mb.faceStartPerChain[c] + cfo);
      const int ncf = mb.faceStartPerChain[mb.nChain];
      for (int i = 0; i < ncf; i++) cc.push_back(mb.chainConn[i] + fo);
      q.insert(q.end(), sb.q.begin(), sb.q.end());
      info.freestream.insert(info.freestream.end(), {sb.rinf, sb.uinf, sb.vinf, sb.einf});
      co += mb.nCell;
      fo += mb.nFace;
      no += mb.nNode;
      cfo += ncf;
      cho += mb.nChain;
      info.cell0.push_back(co);
      info.chain0.push_back(cho);
   }
   fsp.push_back(cfo);
   int st = hamstr::create_gpu(&p0, co, fo, faces.data(), normVec.data(), refMtx.data(), cho, fsp.data(), cc.data(),
                               &info, out);
   if (st != HAMSTR_GPU_OK) return st;
   st = hamstr_gpu_set_geometry(*out, no, x.data());
   if (st == HAMSTR_GPU_OK) st = hamstr_gpu_set(*out, "q", q.data());
   if (st != HAMSTR_GPU_OK) {
      hamstr_gpu_destroy(*out);
      *out = nullptr;
   }
   return st;
}

hamstr_gpu_params hamstr_case::gpu_params(const hamstr_case& c)
{
   hamstr_gpu_params p;
   p.order = c.sb.order;
   p.msweep = c.sb.msweep;
   p.CFL = c.sb.CFL;
   p.gamma = c.sb.gamma;
   p.rinf = c.sb.rinf;
   p.uinf = c.sb.uinf;
   p.vinf = c.sb.vinf;
   p.einf = c.sb.einf;
   p.chain_end_rule = c.sb.chainEndRule;
   p.limiter = c.sb.limiter;
   return p;
}

// ==================================================================
// C ABI: host side
// ==================================================================
extern "C" {

int hamstr_case_open(const char* case_dir, hamstr_case** out, char* err, int errlen)
{
   if (!case_dir || !out) return HAMSTR_GPU_ERR_ARG;
   *out = nullptr;
   try {
      std::unique_ptr<hamstr_case> c(new hamstr_case);
      hamstr_case::load(*c, case_dir);
      *out = c.release();
      return HAMSTR_GPU_OK;
   } catch (const hamstr::Error& e) {
      if (err && errlen > 0) std::snprintf(err, errlen, "%s", e.what());
      return e.status;
   } catch (const std::bad_alloc&) {
      if (err && errlen > 0) std::snprintf(err, errlen, "out of host memory");
      return HAMSTR_GPU_ERR_NOMEM;
   }
}

void hamstr_case_close(hamstr_case* c) { delete c; }

int hamstr_case_sizes(const hamstr_case* c, int* out)
{
   if (!c || !out) return HAMSTR_GPU_ERR_ARG;
   hamstr_case::sizes(*c, out);
   return HAMSTR_GPU_OK;
}

int hamstr_case_params(const hamstr_case* c, double* out)
{
   if (!c || !out) return HAMSTR_GPU_ERR_ARG;
   hamstr_case::params(*c, out);
   return HAMSTR_GPU_OK;
}

int hamstr_case_get_int(const hamstr_case* c, const char* name, int* out, int* count)
{
   if (!c || !name) return HAMSTR_GPU_ERR_ARG;
   return hamstr_case::get_int(*c, name, out, count);
}

int hamstr_case_get(const hamstr_case* c, const char* name, double* out)
{
   if (!c || !name || !out) return HAMSTR_GPU_ERR_ARG;
   return hamstr_case::get(*c, name, out);
}

int hamstr_case_set_run(hamstr_case* c, int order, int msweep, double cfl)
{
   if (!c || (order != 1 && order != 3 && order != 5) || msweep < 1 || !(cfl > 0)) return HAMSTR_GPU_ERR_ARG;
   hamstr_case::set_run(*c, order, msweep, cfl);
   return HAMSTR_GPU_OK;
}

int hamstr_case_set_freestream(hamstr_case* c, double uinf, double vinf, double einf)
{
   if (!c) return HAMSTR_GPU_ERR_ARG;
   hamstr_case::set_freestream(*c, uinf, vinf, einf);
   return HAMSTR_GPU_OK;
}

int hamstr_case_clone(const hamstr_case* c, hamstr_case** out)
{
   if (!c || !out) return HAMSTR_GPU_ERR_ARG;
   try {
      *out = new hamstr_case(*c);
   } catch (const std::bad_alloc&) {
      *out = nullptr;
      return HAMSTR_GPU_ERR_NOMEM;
   }
   return HAMSTR_GPU_OK;
}

int hamstr_case_set_flow(hamstr_case* c, double mach, double alpha_deg)
{
   if (!c || !(mach > 0.0) || !(alpha_deg == alpha_deg)) return HAMSTR_GPU_ERR_ARG;
   hamstr_case::set_flow(*c, mach, alpha_deg);
   return HAMSTR_GPU_OK;
}

int hamstr_case_set_option(hamstr_case* c, const char* name, int value)
{
   if (!c || !name) return HAMSTR_GPU_ERR_ARG;
   return hamstr_case::set_option(*c, name, value);
}

int hamstr_gpu_create_batch(const hamstr_case* const* cases, int n, hamstr_gpu** out)
{
   if (!cases || n < 1 || !out) return HAMSTR_GPU_ERR_ARG;
   for (int k = 0; k < n; k++)
      if (!cases[k]) return HAMSTR_GPU_ERR_ARG;
   *out = nullptr;
   try {
      return hamstr_case::create_batch(cases, n, out);
   } catch (const std::bad_alloc&) {
      return HAMSTR_GPU_ERR_NOMEM;
   }
}

int hamstr_gpu_create_from_case(const hamstr_case* c, hamstr_gpu** out)
{
   if (!c || !out) return HAMSTR_GPU_ERR_ARG;
   return hamstr_case::create_gpu(*c, out);
}

}  // extern "C"
