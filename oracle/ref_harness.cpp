// ##################################################################
//
// ref_harness.cpp -- test-only driver for the reference solver
//
// This file is test infrastructure.  It is compiled together with the
// unmodified reference sources (everything but main.cpp) into
// oracle/_ref/libhamstr_ref.so by oracle/Makefile, and is used only to pin
// the C restatement in oracle/hamstr_oracle.c and to write golden fixtures.
// Nothing in the product links or loads it.
//
// It drives the same call sequence as the reference's main
// (main.cpp:30-47, hamstr.cpp:33-77): readMeshData, readSolutionInputs,
// SOLVER construction, preprocess, initFlow, then stepSolution /
// computeRHS / ADI as the tests ask.  Three reference defects are
// neutralised here without touching the reference sources:
//   * MESHBLOCK::sol_visc is never initialised (meshBlock.h:36) but is
//     used to tag walls (preprocess.cpp:182): setViscosity(0) is called
//     before preprocess, the inviscid value the reference intends;
//   * jacobianRoe2D/3D and computeRHS leak their per-call `new` arrays
//     (jacobianRoe.cpp:28-34,142-150; computeRHS.cpp:34-40): a bump
//     arena replaces global operator new while a solver call runs and is
//     reset before the next one, so long runs stay bounded;
//   * the reference reads its inputs from the working directory
//     (io.cpp:19,74-87): the harness changes into the case directory for
//     the read and changes back.
// ##################################################################
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <sys/mman.h>
#include <unistd.h>
#include <limits.h>

#include <vector>

#include "hamstr.h"
#include "reconstruction.h"
#include "triSolvers.h"

// ------------------------------------------------------------------
// bump arena for the per-call leaks
// ------------------------------------------------------------------
static char*  g_arena      = nullptr;
static size_t g_arena_cap  = 0;
static size_t g_arena_used = 0;
static int    g_arena_on   = 0;

static void arena_reset(void) { g_arena_used = 0; }

static void* arena_alloc(size_t n)
{
   if (g_arena_on && g_arena) {
      size_t a = (n + 15) & ~(size_t)15;
      if (g_arena_used + a <= g_arena_cap) {
         void* p = g_arena + g_arena_used;
         g_arena_used += a;
         return p;
      }
   }
   void* p = std::malloc(n ? n : 1);
   if (!p) throw std::bad_alloc();
   return p;
}

static void arena_free(void* p)
{
   if (!p) return;
   if (g_arena && (char*)p >= g_arena && (char*)p < g_arena + g_arena_cap) return;
   std::free(p);
}

void* operator new(size_t n) { return arena_alloc(n); }
void* operator new[](size_t n) { return arena_alloc(n); }
void  operator delete(void* p) noexcept { arena_free(p); }
void  operator delete[](void* p) noexcept { arena_free(p); }
void  operator delete(void* p, size_t) noexcept { arena_free(p); }
void  operator delete[](void* p, size_t) noexcept { arena_free(p); }

struct ArenaScope {
   ArenaScope()  { arena_reset(); g_arena_on = 1; }
   ~ArenaScope() { g_arena_on = 0; }
};

// ------------------------------------------------------------------
// case handle
// ------------------------------------------------------------------
struct RefCase {
   MESHBLOCK* mb;
   SOLNBLOCK* sb;
   SOLVER*    solv;
};

extern "C" {

void* ref_open(const char* case_dir)
{
   if (!g_arena) {
      g_arena_cap = (size_t)4 << 30;
      void* p = mmap(nullptr, g_arena_cap, PROT_READ | PROT_WRITE,
                     MAP_PRIVATE | MAP_ANONYMOUS | MAP_NORESERVE, -1, 0);
      if (p == MAP_FAILED) { g_arena_cap = 0; } else { g_arena = (char*)p; }
   }
   char cwd[PATH_MAX];
   if (!getcwd(cwd, sizeof(cwd))) return nullptr;
   if (chdir(case_dir) != 0) return nullptr;
   RefCase* c = new RefCase;
   c->mb = new MESHBLOCK[1];
   c->sb = new SOLNBLOCK[1];
   c->mb->readMeshData(0);
   c->sb->readSolutionInputs();
   c->solv = new SOLVER(c->mb, c->sb);
   if (chdir(cwd) != 0) return nullptr;
   c->mb->setViscosity(0);
   c->mb->preprocess();
   c->solv->initFlow();
   return c;
}

void ref_close(void* h)
{
   // the reference has no destructors that free its arrays; the handle
   // itself is released and the process reclaims the rest
   delete (RefCase*)h;
}

// sizes: nCell nFace nChain nChainFace nMaxChain order msweep nGhost nNode nColor
void ref_sizes(void* h, int* out)
{
   RefCase* c = (RefCase*)h;
   out[0] = c->mb->nCell;
   out[1] = c->mb->nFace;
   out[2] = c->mb->nChain;
   out[3] = c->mb->nChainFace;
   out[4] = c->mb->nMaxChain;
   out[5] = c->sb->order;
   out[6] = c->sb->msweep;
   out[7] = c->sb->nGhost;
   out[8] = c->mb->nNode;
   out[9] = c->mb->nColor;
}

// freestream and run parameters: Mach alpha CFL gamma rinf uinf vinf einf pinf
void ref_params(void* h, double* out)
{
   RefCase* c = (RefCase*)h;
   out[0] = c->sb->Mach;  out[1] = c->sb->alpha; out[2] = c->sb->CFL;
   out[3] = c->sb->gamma; out[4] = c->sb->rinf;  out[5] = c->sb->uinf;
   out[6] = c->sb->vinf;  out[7] = c->sb->einf;  out[8] = c->sb->pinf;
}

void ref_set_freestream(void* h, double uinf, double vinf, double einf)
{
   RefCase* c = (RefCase*)h;
   c->sb->uinf = uinf; c->sb->vinf = vinf; c->sb->einf = einf;
}

void ref_set_run(void* h, int order, int msweep, double cfl)
{
   RefCase* c = (RefCase*)h;
   c->sb->order = order; c->sb->msweep = msweep; c->sb->CFL = cfl;
   c->sb->nGhost = (order == 5) ? 3 : 2;
}

void ref_compute_rhs(void* h, int implicit, double* l2, double* linf)
{
   RefCase* c = (RefCase*)h;
   char opt_imp[] = "implicit";
   char opt_exp[] = "explicit";
   ArenaScope a;
   c->solv->computeRHS(implicit ? opt_imp : opt_exp);
   *l2 = c->sb->L2Norm; *linf = c->sb->LInfNorm;
}

void ref_adi(void* h, double* l2, double* linf)
{
   RefCase* c = (RefCase*)h;
   ArenaScope a;
   c->solv->ADI();
   *l2 = c->sb->L2Norm; *linf = c->sb->LInfNorm;
}

void ref_linear_rhs(void* h, double* l2, double* linf)
{
   RefCase* c = (RefCase*)h;
   ArenaScope a;
   c->solv->computeLinearRHS();
   *l2 = c->sb->L2Norm; *linf = c->sb->LInfNorm;
}

// one ADI pseudo-time step (march.cpp:381-386) with both norms recorded:
// out[0..1] = computeRHS L2/Linf, out[2..3] = final linear-defect L2/Linf
void ref_step(void* h, double* out)
{
   RefCase* c = (RefCase*)h;
   char opt_imp[] = "implicit";
   ArenaScope a;
   c->solv->computeRHS(opt_imp);
   out[0] = c->sb->L2Norm; out[1] = c->sb->LInfNorm;
   c->solv->ADI();
   out[2] = c->sb->L2Norm; out[3] = c->sb->LInfNorm;
}

// one step of the named scheme ("ADI", "euler", "rk3") through the
// reference's own stepSolution (march.cpp:335-403); out2 = L2, Linf
void ref_step_scheme(void* h, const char* scheme, double* out2)
{
   RefCase* c = (RefCase*)h;
   char saved[20];
   memcpy(saved, c->sb->scheme, sizeof(saved));
   snprintf(c->sb->scheme, sizeof(c->sb->scheme), "%s", scheme);
   ArenaScope a;
   c->solv->stepSolution();
   memcpy(c->sb->scheme, saved, sizeof(saved));
   out2[0] = c->sb->L2Norm; out2[1] = c->sb->LInfNorm;
}

// run n steps; hist gets 4 doubles per step as in ref_step
void ref_march(void* h, int n, double* hist)
{
   for (int i = 0; i < n; i++) ref_step(h, hist + 4 * i);
}

static double* dptr(RefCase* c, const char* name, size_t* n)
{
   int nc = c->mb->nCell;
   if (!strcmp(name, "q"))     { *n = (size_t)NQ * nc; return c->sb->q; }
   if (!strcmp(name, "qt"))    { *n = (size_t)NQ * nc; return c->sb->qt; }
   if (!strcmp(name, "r"))     { *n = (size_t)NQ * nc; return c->sb->r; }
   if (!strcmp(name, "r0"))    { *n = (size_t)NQ * nc; return c->sb->r0; }
   if (!strcmp(name, "dq"))    { *n = (size_t)NQ * nc; return c->sb->dq; }
   if (!strcmp(name, "sigma")) { *n = (size_t)nc;      return c->sb->sigma; }
   if (!strcmp(name, "ff"))    { *n = (size_t)2 * NQ * NQ * c->mb->nFace; return (double*)c->sb->ff; }
   if (!strcmp(name, "x"))     { *n = (size_t)NDIM * c->mb->nNode; return c->mb->x; }
   if (!strcmp(name, "vol"))   { *n = (size_t)nc;      return c->mb->vol; }
   return nullptr;
}

int ref_get(void* h, const char* name, double* out)
{
   RefCase* c = (RefCase*)h;
   size_t n = 0;
   if (!strcmp(name, "normVec")) {
      for (int i = 0; i < c->mb->nFace; i++) {
         out[2 * i] = c->mb->normVec[i][0]; out[2 * i + 1] = c->mb->normVec[i][1];
      }
      return 0;
   }
   if (!strcmp(name, "refMtx")) {
      for (int i = 0; i < c->mb->nFace; i++)
         for (int a = 0; a < 2; a++)
            for (int b = 0; b < 2; b++) out[4 * i + 2 * a + b] = c->mb->refMtx[i][a][b];
      return 0;
   }
   double* p = dptr(c, name, &n);
   if (!p) return -1;
   memcpy(out, p, n * sizeof(double));
   return 0;
}

int ref_set(void* h, const char* name, const double* in)
{
   RefCase* c = (RefCase*)h;
   size_t n = 0;
   double* p = dptr(c, name, &n);
   if (!p) return -1;
   memcpy(p, in, n * sizeof(double));
   return 0;
}

int ref_get_int(void* h, const char* name, int* out)
{
   RefCase* c = (RefCase*)h;
   MESHBLOCK* m = c->mb;
   if (!strcmp(name, "faces"))   { memcpy(out, m->faces, sizeof(int) * 6 * m->nFace); return 0; }
   if (!strcmp(name, "chainConn")) { memcpy(out, m->chainConn, sizeof(int) * m->nChainFace); return 0; }
   if (!strcmp(name, "faceStartPerChain")) { memcpy(out, m->faceStartPerChain, sizeof(int) * (m->nChain + 1)); return 0; }
   if (!strcmp(name, "c2chain")) { memcpy(out, m->c2chain, sizeof(int) * NDIM * m->nCell); return 0; }
   if (!strcmp(name, "bFaces"))  {
      int nb = 0;
      for (int i = 0; i < m->nFace; i++) if (m->faces[6 * i + 4] == -2) nb++;
      memcpy(out, m->bFaces, sizeof(int) * nb); return nb;
   }
   if (!strcmp(name, "chainsPerColor")) { memcpy(out, m->chainsPerColor, sizeof(int) * m->nColor); return 0; }
   return -1;
}

// SOLVER::fluxRoe2D / jacobianRoe2D of the handle's solver on one face
void ref_flux_roe2d(void* h, double* nxy, double* ql, double* qr, double* flux, double* spec, double gamma)
{
   ((RefCase*)h)->solv->fluxRoe2D(nxy, ql, qr, flux, spec, gamma);
}

void ref_jacobian_roe2d(void* h, double* nxy, double* ql, double* qr, double* lm, double* rm, double gamma)
{
   ArenaScope arena;   // jacobianRoe2D / 3D leak their per-call arrays
   double* L[4] = {lm, lm + 4, lm + 8, lm + 12};
   double* R[4] = {rm, rm + 4, rm + 8, rm + 12};
   ((RefCase*)h)->solv->jacobianRoe2D(nxy, ql, qr, L, R, gamma);
}

// SOLVER::fluxRoe3D / jacobianRoe3D of the handle's solver on one face
void ref_flux_roe3d(void* h, double* nxyz, double* ql, double* qr, double* flux, double* spec, double gamma)
{
   ((RefCase*)h)->solv->fluxRoe3D(nxyz, ql, qr, flux, spec, gamma);
}

void ref_jacobian_roe3d(void* h, double* nxyz, double* ql, double* qr, double* lm, double* rm, double gamma)
{
   ArenaScope arena;
   double* L[5] = {lm, lm + 5, lm + 10, lm + 15, lm + 20};
   double* R[5] = {rm, rm + 5, rm + 10, rm + 15, rm + 20};
   ((RefCase*)h)->solv->jacobianRoe3D(nxyz, ql, qr, L, R, gamma);
}

// TRISOLVER::blockTridag / blockTridagPeriodic (nq = 5) on flat [N][5][5] blocks
int ref_block_tridag5(double* a, double* b, double* c, double* f, int N, int periodic)
{
   if (N < 1 || (periodic && N < 2)) return -1;
   std::vector<double**> A(N), B(N), C(N);
   std::vector<double*> F(N), rowsA(5 * (size_t)N), rowsB(5 * (size_t)N), rowsC(5 * (size_t)N);
   for (int i = 0; i < N; i++) {
      for (int k = 0; k < 5; k++) {
         rowsA[5 * i + k] = a + 25 * (size_t)i + 5 * k;
         rowsB[5 * i + k] = b + 25 * (size_t)i + 5 * k;
         rowsC[5 * i + k] = c + 25 * (size_t)i + 5 * k;
      }
      A[i] = &rowsA[5 * i];
      B[i] = &rowsB[5 * i];
      C[i] = &rowsC[5 * i];
      F[i] = f + 5 * (size_t)i;
   }
   if (periodic) TRISOLVER::blockTridagPeriodic(A.data(), B.data(), C.data(), F.data(), N, 5);
   else TRISOLVER::blockTridag(A.data(), B.data(), C.data(), F.data(), N, 5);
   return 0;
}

// RECONSTRUCTION::* on one line of flat [imax][nq] arrays (rows views)
static std::vector<double*> rows(double* p, int imax, int nq)
{
   std::vector<double*> v((size_t)imax + 1);
   for (int i = 0; i < imax; i++) v[i] = p + (size_t)i * nq;
   v[imax] = nullptr;
   return v;
}

void ref_muscl_line(double* f, double* ql, double* qr, double* f2, int is, int ie, double th, double qt, double eps,
                    int imax, int nq)
{
   auto F = rows(f, imax, nq), QL = rows(ql, imax, nq), QR = rows(qr, imax, nq), F2 = rows(f2, imax, nq);
   RECONSTRUCTION::MUSCL(F.data(), QL.data(), QR.data(), F2.data(), is, ie, th, qt, eps, imax, nq);
}

void ref_muscl_deriv_line(double* f, double* ql, double* qr, double* f2, double* dq, int is, int ie, double th,
                          double qt, double eps, int imax, int nq)
{
   auto F = rows(f, imax, nq), QL = rows(ql, imax, nq), QR = rows(qr, imax, nq), F2 = rows(f2, imax, nq);
   auto DQ = rows(dq, imax, nq);
   RECONSTRUCTION::MUSCL_DERIV(F.data(), QL.data(), QR.data(), F2.data(), DQ.data(), is, ie, th, qt, eps, imax, nq);
}

void ref_weno_line(double* f, double* ql, double* qr, int is, int ie, double epsw, int imax, int nq)
{
   auto F = rows(f, imax, nq), QL = rows(ql, imax, nq), QR = rows(qr, imax, nq);
   RECONSTRUCTION::WENO(F.data(), QL.data(), QR.data(), is, ie, epsw, imax, nq);
}

void ref_weno_deriv_line(double* f, double* ql, double* qr, double* dq, int is, int ie, double eps, int imax, int nq)
{
   auto F = rows(f, imax, nq), QL = rows(ql, imax, nq), QR = rows(qr, imax, nq), DQ = rows(dq, imax, nq);
   RECONSTRUCTION::WENO_DERIV(F.data(), QL.data(), QR.data(), DQ.data(), is, ie, eps, imax, nq);
}

// TRISOLVER::blockTridag4 / blockTridagPeriodic4 on flat [N][4][4] blocks
int ref_block_tridag4(double* a, double* b, double* c, double* f, int N, int periodic)
{
   if (N < 1 || (periodic && N < 2)) return -1;
   double*** A = new double**[N];
   double*** B = new double**[N];
   double*** C = new double**[N];
   double** F = new double*[N];
   for (int i = 0; i < N; i++) {
      A[i] = new double*[NQ]; B[i] = new double*[NQ]; C[i] = new double*[NQ];
      F[i] = f + NQ * i;
      for (int k = 0; k < NQ; k++) {
         A[i][k] = a + NQ * NQ * i + NQ * k;
         B[i][k] = b + NQ * NQ * i + NQ * k;
         C[i][k] = c + NQ * NQ * i + NQ * k;
      }
   }
   if (periodic) TRISOLVER::blockTridagPeriodic4(A, B, C, F, N, NQ);
   else TRISOLVER::blockTridag4(A, B, C, F, N, NQ);
   for (int i = 0; i < N; i++) { delete[] A[i]; delete[] B[i]; delete[] C[i]; }
   delete[] A; delete[] B; delete[] C; delete[] F;
   return 0;
}

} // extern "C"
