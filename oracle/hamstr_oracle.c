/*
 * hamstr_oracle.c -- CPU restatement of HAMSTR's steady ADI iteration.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product).  Plain C,
 * compiled with -ffp-contract=off so that each multiply and add rounds
 * separately, exactly as the reference does on x86-64.  Every function names
 * the reference lines it restates; expressions keep the reference's
 * evaluation order (C's left-to-right association), because the GPU path is
 * held to bit-identical results.
 *
 * Deliberate deviations, none of which changes a computed value:
 *   - fluxRoe2D's loop over i<5 on 4-element arrays (interfaceFlux.cpp:138)
 *     runs over the 4 real components;
 *   - the unused sound speeds cl/cr of fluxRoe2D (interfaceFlux.cpp:71,78) and
 *     the unused dc/dh derivative vectors of jacobianRoe3D in frozen mode are
 *     not formed;
 *   - the reconstruction value at the last stencil slot, which the reference
 *     forms from a stale difference and never reads, is not formed;
 *   - a NaN spectral radius returns -1 instead of exiting the process.
 */
#include "hamstr_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define NQ 4
#define BC_FREESTREAM (-1)
#define BC_WALL (-2)
#define BC_INTERDOMAIN (-5)

struct ho_case {
   /* mesh (io.cpp / preprocess.cpp) */
   int nNode, nCell, nFace, nColor, nChain, nMaxChain, nChainFace, nBface;
   double* x;            /* 2*nNode */
   int* conn;            /* 4*nCell */
   int* chainsPerColor;  /* nColor */
   int* faceStart;       /* nChain+1 (read array, K entries) */
   int* chainConn;       /* nChainFace */
   int* faces;           /* 6*nFace: n1 n2 cL eL cR eR */
   int* bFaces;          /* nFace */
   int* c2chain;         /* 2*nCell */
   double* vol;          /* nCell */
   double* normVec;      /* 2*nFace */
   double* refMtx;       /* 4*nFace, row-major 2x2 */
   /* inputs (io.cpp:26-41) */
   double Mach, alpha, beta, rey, dt, CFL;
   int order, timeacc, nsteps, nwrite, msweep, visc, test, outform;
   char scheme[64], timeInteg[64];
   /* flow (initFlow.cpp) */
   double gamma, gm1, rinf, pinf, uinf, vinf, einf;
   int nGhost;
   /* project option, not in the reference: how open chains take ghost
      states at their end faces (HO_END_RULE_*) */
   int end_rule;
   /* project option: MUSCL limiter of order 3 (HO_LIMITER_*) */
   int limiter;
   int sweep_order;   /* project option: 1 = first-order linearised residual in the ADI sweeps */
   double L2Norm, LInfNorm;
   /* solution arrays (solver.cpp:26-38) */
   double *q, *qt, *r, *r0, *dq, *sigma;
   double* ff;           /* nFace * 32: lmat[4][4] then rmat[4][4] */
   /* per-chain work arrays of length nMaxChain+5 */
   int work;
   int* cindx;
   double (*f)[NQ], (*df)[NQ], (*ql)[NQ], (*qr)[NQ], (*f2)[NQ];
   double (*A)[NQ][NQ], (*B)[NQ][NQ], (*C)[NQ][NQ], (*F)[NQ];
};

/* ------------------------------------------------------------------ */
/* reading (io.cpp:13-51, 58-372)                                      */
/* ------------------------------------------------------------------ */

static int rd_inputs(ho_case* c, const char* dir, char* err, int errlen)
{
   char path[4096];
   snprintf(path, sizeof(path), "%s/input.hamstr", dir);
   FILE* fp = fopen(path, "r");
   if (!fp) { snprintf(err, errlen, "missing %s", path); return -1; }
   int ok = 1;
   ok &= fscanf(fp, "Mach=%lf\n", &c->Mach) == 1;
   ok &= fscanf(fp, "alpha=%lf\n", &c->alpha) == 1;
   ok &= fscanf(fp, "beta=%lf\n", &c->beta) == 1;
   ok &= fscanf(fp, "rey=%lf\n", &c->rey) == 1;
   ok &= fscanf(fp, "scheme=%63s\n", c->scheme) == 1;
   ok &= fscanf(fp, "time integration=%63s\n", c->timeInteg) == 1;
   ok &= fscanf(fp, "order=%d\n", &c->order) == 1;
   ok &= fscanf(fp, "timeacc=%d\n", &c->timeacc) == 1;
   ok &= fscanf(fp, "nsteps=%d\n", &c->nsteps) == 1;
   ok &= fscanf(fp, "nwrite=%d\n", &c->nwrite) == 1;
   ok &= fscanf(fp, "dt=%lf\n", &c->dt) == 1;
   ok &= fscanf(fp, "CFL=%lf\n", &c->CFL) == 1;
   ok &= fscanf(fp, "msweep=%d\n", &c->msweep) == 1;
   ok &= fscanf(fp, "visc=%d\n", &c->visc) == 1;
   ok &= fscanf(fp, "testcase=%d\n", &c->test) == 1;
   ok &= fscanf(fp, "output=%d\n", &c->outform) == 1;
   fclose(fp);
   if (!ok) { snprintf(err, errlen, "malformed %s", path); return -1; }
   if (c->test != 0) { snprintf(err, errlen, "testcase %d not implemented", c->test); return -1; }
   return 0;
}

static FILE* open_mesh(const char* dir, const char* name, char* err, int errlen)
{
   char path[4096];
   snprintf(path, sizeof(path), "%s/input/domain000/%s", dir, name);
   FILE* fp = fopen(path, "r");
   if (!fp) snprintf(err, errlen, "missing %s", path);
   return fp;
}

static int rd_mesh(ho_case* c, const char* dir, char* err, int errlen)
{
   FILE* fp;
   int i, j;
   double z;
   if (!(fp = open_mesh(dir, "coord.dat", err, errlen))) return -1;
   if (fscanf(fp, "%d", &c->nNode) != 1) goto bad;
   c->x = (double*)malloc(sizeof(double) * 2 * (c->nNode > 0 ? c->nNode : 1));
   for (i = 0; i < c->nNode; i++)
      if (fscanf(fp, "%lf %lf %lf\n", &c->x[2 * i], &c->x[2 * i + 1], &z) != 3) goto bad;
   fclose(fp);

   if (!(fp = open_mesh(dir, "conn.dat", err, errlen))) return -1;
   if (fscanf(fp, "%d", &c->nCell) != 1) goto bad;
   c->conn = (int*)malloc(sizeof(int) * 4 * (c->nCell > 0 ? c->nCell : 1));
   for (i = 0; i < c->nCell; i++)
      if (fscanf(fp, "%d %d %d %d\n", &c->conn[4 * i], &c->conn[4 * i + 1],
                 &c->conn[4 * i + 2], &c->conn[4 * i + 3]) != 4) goto bad;
   fclose(fp);

   if (!(fp = open_mesh(dir, "ncolors.dat", err, errlen))) return -1;
   if (fscanf(fp, "%d", &c->nColor) != 1) goto bad;
   c->chainsPerColor = (int*)malloc(sizeof(int) * (c->nColor > 0 ? c->nColor : 1));
   for (i = 0; i < c->nColor; i++)
      if (fscanf(fp, "%d\n", &c->chainsPerColor[i]) != 1) goto bad;
   fclose(fp);

   /* chain offsets; consecutive duplicates are dropped (io.cpp:223-245) */
   if (!(fp = open_mesh(dir, "iqloops.dat", err, errlen))) return -1;
   {
      int k;
      if (fscanf(fp, "%d\n", &k) != 1 || k < 1) goto bad;
      c->faceStart = (int*)malloc(sizeof(int) * k);
      c->nMaxChain = 0;
      j = 0;
      for (i = 0; i < k; i++) {
         if (fscanf(fp, "%d\n", &c->faceStart[j]) != 1) goto bad;
         if (i > 0) {
            if (c->faceStart[j] == c->faceStart[j - 1]) j--;
            if (j > 0) {
               int d = c->faceStart[j] - c->faceStart[j - 1];
               if (d > c->nMaxChain) c->nMaxChain = d;
            }
         }
         j++;
      }
      c->nChain = j - 1;
   }
   fclose(fp);

   if (!(fp = open_mesh(dir, "qloops.dat", err, errlen))) return -1;
   if (fscanf(fp, "%d", &c->nChainFace) != 1) goto bad;
   c->chainConn = (int*)malloc(sizeof(int) * (c->nChainFace > 0 ? c->nChainFace : 1));
   for (i = 0; i < c->nChainFace; i++)
      if (fscanf(fp, "%d", &c->chainConn[i]) != 1) goto bad;
   fclose(fp);

   /* faces: row n1 n2 cL cR eL eR stored as n1 n2 cL eL cR eR, swapped
      when the left cell is -1 (io.cpp:344-365) */
   if (!(fp = open_mesh(dir, "qedges.dat", err, errlen))) return -1;
   if (fscanf(fp, "%d", &c->nFace) != 1) goto bad;
   c->faces = (int*)malloc(sizeof(int) * 6 * (c->nFace > 0 ? c->nFace : 1));
   for (i = 0; i < c->nFace; i++) {
      int* fr = c->faces + 6 * i;
      if (fscanf(fp, "%d %d %d %d %d %d\n", &fr[0], &fr[1], &fr[2], &fr[4], &fr[3], &fr[5]) != 6) goto bad;
      if (fr[2] == BC_FREESTREAM) {
         int t;
         t = fr[0]; fr[0] = fr[1]; fr[1] = t;
         t = fr[2]; fr[2] = fr[4]; fr[4] = t;
         t = fr[3]; fr[3] = fr[5]; fr[5] = t;
      }
   }
   fclose(fp);
   return 0;
bad:
   fclose(fp);
   snprintf(err, errlen, "malformed mesh file");
   return -1;
}

/* ------------------------------------------------------------------ */
/* preprocessing (preprocess.cpp:15-241)                               */
/* ------------------------------------------------------------------ */

static void preprocess(ho_case* c)
{
   int i, m = 0;
   c->vol = (double*)calloc(c->nCell > 0 ? c->nCell : 1, sizeof(double));
   c->normVec = (double*)malloc(sizeof(double) * 2 * (c->nFace > 0 ? c->nFace : 1));
   c->refMtx = (double*)malloc(sizeof(double) * 4 * (c->nFace > 0 ? c->nFace : 1));
   c->bFaces = (int*)malloc(sizeof(int) * (c->nFace > 0 ? c->nFace : 1));
   c->c2chain = (int*)malloc(sizeof(int) * 2 * (c->nCell > 0 ? c->nCell : 1));
   for (i = 0; i < c->nFace; i++) {
      int* fr = c->faces + 6 * i;
      int left = fr[2], right = fr[4];
      int i1 = fr[0], i2 = fr[1];
      double x1 = c->x[2 * i1], y1 = c->x[2 * i1 + 1];
      double x2 = c->x[2 * i2], y2 = c->x[2 * i2 + 1];
      double nx = (y2 - y1);
      double ny = -(x2 - x1);
      double dvedge = 0.5 * (x1 * y2 - x2 * y1);
      double ds;
      c->normVec[2 * i] = nx;
      c->normVec[2 * i + 1] = ny;
      ds = nx * nx + ny * ny;
      ds = 1. / ds;
      c->refMtx[4 * i + 0] = 1. - 2. * nx * nx * ds;
      c->refMtx[4 * i + 1] = -2. * nx * ny * ds;
      c->refMtx[4 * i + 2] = -2. * ny * nx * ds;
      c->refMtx[4 * i + 3] = 1. - 2. * ny * ny * ds;
      c->vol[left] += dvedge;
      if (right > -1) c->vol[right] -= dvedge;
      if (right == -1) {
         double r1 = sqrt(x1 * x1 + y1 * y1);
         double r2 = sqrt(x2 * x2 + y2 * y2);
         if (0.5 * (r1 + r2) < 3.0) {
            c->bFaces[m++] = i;
            fr[4] = -(0 + 2); /* sol_visc = 0, the inviscid wall tag */
         }
      }
   }
   c->nBface = m;
   for (i = 0; i < 2 * c->nCell; i++) c->c2chain[i] = -1;
   for (i = 0; i < c->nChain; i++) {
      int f;
      for (f = c->faceStart[i]; f < c->faceStart[i + 1] - 1; f++) {
         int left = c->faces[6 * c->chainConn[f] + 2];
         if (c->c2chain[2 * left] > -1) c->c2chain[2 * left + 1] = i;
         else c->c2chain[2 * left] = i;
      }
   }
}

/* ------------------------------------------------------------------ */
/* flow initialisation (initFlow.cpp:12-93)                            */
/* ------------------------------------------------------------------ */

static void init_flow(ho_case* c)
{
   int i;
   c->gamma = 1.4;
   c->gm1 = c->gamma - 1.;
   c->rinf = 1.0;
   c->pinf = 1.0 / c->gamma;
   c->nGhost = (c->order == 5) ? 3 : 2;
   c->uinf = c->Mach * cos(c->alpha * (3.1415926535897932e+00 / 180.0));
   c->vinf = c->Mach * sin(c->alpha * (3.1415926535897932e+00 / 180.0));
   c->einf = c->pinf / (c->gm1) + 0.5 * c->rinf * (c->uinf * c->uinf + c->vinf * c->vinf);
   for (i = 0; i < c->nCell; i++) {
      c->q[4 * i + 0] = c->rinf;
      c->q[4 * i + 1] = c->rinf * c->uinf;
      c->q[4 * i + 2] = c->rinf * c->vinf;
      c->q[4 * i + 3] = c->einf;
   }
   memcpy(c->qt, c->q, sizeof(double) * NQ * c->nCell);
}

static void alloc_solution(ho_case* c)
{
   int n = c->nCell > 0 ? c->nCell : 1;
   c->q = (double*)calloc((size_t)NQ * n, sizeof(double));
   c->qt = (double*)calloc((size_t)NQ * n, sizeof(double));
   c->r = (double*)calloc((size_t)NQ * n, sizeof(double));
   c->r0 = (double*)calloc((size_t)NQ * n, sizeof(double));
   c->dq = (double*)calloc((size_t)NQ * n, sizeof(double));
   c->sigma = (double*)calloc(n, sizeof(double));
   c->ff = (double*)calloc((size_t)32 * (c->nFace > 0 ? c->nFace : 1), sizeof(double));
   c->work = c->nMaxChain + 6;
   c->cindx = (int*)calloc(c->work, sizeof(int));
   c->f = calloc(c->work, sizeof(*c->f));
   c->df = calloc(c->work, sizeof(*c->df));
   c->ql = calloc(c->work, sizeof(*c->ql));
   c->qr = calloc(c->work, sizeof(*c->qr));
   c->f2 = calloc(c->work, sizeof(*c->f2));
   c->A = calloc(c->work, sizeof(*c->A));
   c->B = calloc(c->work, sizeof(*c->B));
   c->C = calloc(c->work, sizeof(*c->C));
   c->F = calloc(c->work, sizeof(*c->F));
}

/* ------------------------------------------------------------------ */
/* chain stencil (computeRHS.cpp:57-149; computeLinearRHS.cpp:55-143)  */
/* ------------------------------------------------------------------ */

/* Builds cindx for chain ich and returns chainSize.  Closed chains wrap
   around; open chains get negated ghost ids. */
static int chain_stencil(ho_case* c, int ich)
{
   int f1 = c->faceStart[ich], f2 = c->faceStart[ich + 1];
   int g = c->nGhost, m = g, f;
   int* ci = c->cindx;
   int size;
   for (f = f1; f < f2; f++) ci[m++] = c->faces[6 * c->chainConn[f] + 2];
   if (c->chainConn[f1] == c->chainConn[f2 - 1]) {
      ci[m++] = c->faces[6 * c->chainConn[f1 + 1] + 2];
      size = m;
      m = 0;
      for (f = f2 - g - 1; f < f2 - 1; f++) ci[m++] = c->faces[6 * c->chainConn[f] + 2];
   } else if (c->order == 5) {
      m--; ci[m] = -ci[m];
      m++; ci[m] = -ci[m - 3];
      m++; ci[m] = -ci[m - 5];
      size = m + 1;
      ci[0] = -ci[5];
      ci[1] = -ci[4];
      ci[2] = -ci[3];
   } else {
      m--; ci[m] = -ci[m];
      m++; ci[m] = -ci[m - 3];
      size = m + 1;
      ci[0] = -ci[3];
      ci[1] = -ci[2];
   }
   return size;
}

/* One ghost state of the extended end rule: the true neighbour across an
   interior end face, the wall mirror of end cell `mc`, or the freestream. */
static void ghost_ext(ho_case* c, int j, int iface, int mc, const double* dqv)
{
   int right = c->faces[6 * iface + 4], k;
   if (right >= 0) {
      for (k = 0; k < NQ; k++) {
         c->f[j][k] = c->q[NQ * right + k];
         if (dqv) c->df[j][k] = dqv[NQ * right + k];
      }
   } else if (right == BC_WALL) {
      const double* R = c->refMtx + 4 * iface;
      const double* s = c->q + NQ * mc;
      c->f[j][0] = s[0];
      c->f[j][1] = (s[1] * R[0] + s[2] * R[1]);
      c->f[j][2] = (s[1] * R[2] + s[2] * R[3]);
      c->f[j][3] = s[3];
      if (dqv) {
         const double* d = dqv + NQ * mc;
         c->df[j][0] = d[0];
         c->df[j][1] = (d[1] * R[0] + d[2] * R[1]);
         c->df[j][2] = (d[1] * R[2] + d[2] * R[3]);
         c->df[j][3] = d[3];
      }
   } else {
      c->f[j][0] = c->rinf;
      c->f[j][1] = c->rinf * c->uinf;
      c->f[j][2] = c->rinf * c->vinf;
      c->f[j][3] = c->einf;
      if (dqv) c->df[j][0] = c->df[j][1] = c->df[j][2] = c->df[j][3] = 0.0;
   }
}

/* Fills the work arrays f (and df when dqv != NULL) from q (and dq) with
   wall-mirror and freestream ghosts (computeRHS.cpp:154-260,
   computeLinearRHS.cpp:148-276).  Cell id 0 is a ghost only at stencil
   positions nGhost-1 and size-nGhost, as in the reference.

   Under HO_END_RULE_EXTENDED (a project rule for meshes whose open chains
   may end at interior faces) the ghosts of an open chain are set by
   position instead: the k-th ghost beyond an end face (k = 1..nGhost)
   holds the true neighbour's state when the face is interior, the wall
   mirror of the chain's k-th cell from that end (the last one for chains
   shorter than k) at a wall, and the freestream at the far field. */
static int chain_gather(ho_case* c, int ich, int size, const double* dqv)
{
   int f1 = c->faceStart[ich], f2 = c->faceStart[ich + 1];
   int g = c->nGhost, j, k;
   if (c->end_rule == HO_END_RULE_EXTENDED && c->chainConn[f1] != c->chainConn[f2 - 1]) {
      int n = size - 2 * g;     /* cells on the chain */
      for (j = g; j < g + n; j++) {
         int icell = c->cindx[j];
         for (k = 0; k < NQ; k++) {
            c->f[j][k] = c->q[NQ * icell + k];
            if (dqv) c->df[j][k] = dqv[NQ * icell + k];
         }
      }
      for (k = 1; k <= g; k++) {
         int mk = (k - 1 < n - 1) ? k - 1 : n - 1;
         ghost_ext(c, g - k, c->chainConn[f1], c->cindx[g + mk], dqv);
         ghost_ext(c, g + n - 1 + k, c->chainConn[f2 - 1], c->cindx[g + n - 1 - mk], dqv);
      }
      return 0;
   }
   for (j = 0; j < size; j++) {
      int icell = c->cindx[j];
      if (icell >= 0) {
         for (k = 0; k < NQ; k++) {
            c->f[j][k] = c->q[NQ * icell + k];
            if (dqv) c->df[j][k] = dqv[NQ * icell + k];
         }
      }
      if (icell < 0 || (icell == 0 && j == g - 1) || (icell == 0 && j == size - g)) {
         int iface = (j < g) ? c->chainConn[f1] : c->chainConn[f2 - 1];
         int right = c->faces[6 * iface + 4];
         if (right == BC_WALL) {
            const double* R = c->refMtx + 4 * iface;
            const double* s = c->q + NQ * (-icell);
            c->f[j][0] = s[0];
            c->f[j][1] = (s[1] * R[0] + s[2] * R[1]);
            c->f[j][2] = (s[1] * R[2] + s[2] * R[3]);
            c->f[j][3] = s[3];
            if (dqv) {
               const double* d = dqv + NQ * (-icell);
               c->df[j][0] = d[0];
               c->df[j][1] = (d[1] * R[0] + d[2] * R[1]);
               c->df[j][2] = (d[1] * R[2] + d[2] * R[3]);
               c->df[j][3] = d[3];
            }
         } else if (right == BC_INTERDOMAIN) {
            /* empty branch in the reference (no MPI build) */
            if (icell < 0) return -2;
         } else {
            c->f[j][0] = c->rinf;
            c->f[j][1] = c->rinf * c->uinf;
            c->f[j][2] = c->rinf * c->vinf;
            c->f[j][3] = c->einf;
            if (dqv) c->df[j][0] = c->df[j][1] = c->df[j][2] = c->df[j][3] = 0.0;
         }
      }
   }
   return 0;
}

/* ------------------------------------------------------------------ */
/* reconstruction (reconstruction.cpp)                                 */
/* ------------------------------------------------------------------ */

/* MUSCL, reconstruction.cpp:16-70, over slots is..ie-1 */
/* minmod(x, y) as a selection: 0 -> 0, 1 -> x, 2 -> y */
static int minmod_sel(double x, double y)
{
   if (x > 0.0) return (y <= 0.0) ? 0 : ((x <= y) ? 1 : 2);
   if (x < 0.0) return (y >= 0.0) ? 0 : ((x >= y) ? 1 : 2);
   return 0;
}

static double pick(int sel, double x, double y) { return sel == 0 ? 0.0 : (sel == 1 ? x : y); }

/* Project limiters for the kappa = 1/3 MUSCL scheme (no reference
   counterpart), after Anderson, Thomas and van Leer, AIAA J. 24(9), 1986:
   minmod-limited differences a~ = minmod(a, 4b), b~ = minmod(b, 4a), or
   van Albada's s = (2ab + eps)/(a^2 + b^2 + eps) with sk = kappa s.
   a = f_i - f_{i-1}, b = f_{i+1} - f_i. */
static void muscl_lim(ho_case* c, int is, int ie, double qt)
{
   const double th = 0.3333333333333333e+00, eps = 1e-10;
   double thm = 1.0 - th, thp = 1.0 + th;
   int i, n;
   for (n = 0; n < NQ; n++) {
      for (i = 0; i < ie; i++) c->f2[i][n] = c->f[i + 1][n] - c->f[i][n];
      for (i = is; i < ie; i++) {
         double a = c->f2[i - 1][n], b = c->f2[i][n], f = c->f[i][n];
         if (c->limiter == HO_LIMITER_MINMOD) {
            double at = pick(minmod_sel(a, 4.0 * b), a, 4.0 * b);
            double bt = pick(minmod_sel(b, 4.0 * a), b, 4.0 * a);
            c->ql[i][n] = f + qt * (thm * at + thp * bt);
            c->qr[i][n] = f - qt * (thp * at + thm * bt);
         } else {
            double s = (2.0 * a * b + eps) / (a * a + b * b + eps);
            double sk = th * s;
            c->ql[i][n] = f + (qt * s) * ((1.0 - sk) * a + (1.0 + sk) * b);
            c->qr[i][n] = f - (qt * s) * ((1.0 + sk) * a + (1.0 - sk) * b);
         }
      }
   }
}

/* linearisation of muscl_lim (minmod with its selection frozen) */
static void muscl_lim_deriv(ho_case* c, int is, int ie, double qt)
{
   const double th = 0.3333333333333333e+00, eps = 1e-10;
   double thm = 1.0 - th, thp = 1.0 + th;
   int i, n;
   for (n = 0; n < NQ; n++) {
      for (i = 0; i < ie; i++) c->f2[i][n] = c->f[i + 1][n] - c->f[i][n];
      for (i = is; i < ie; i++) {
         double a = c->f2[i - 1][n], b = c->f2[i][n];
         double df = c->df[i][n];
         double da = c->df[i][n] - c->df[i - 1][n], db = c->df[i + 1][n] - c->df[i][n];
         if (c->limiter == HO_LIMITER_MINMOD) {
            double dat = pick(minmod_sel(a, 4.0 * b), da, 4.0 * db);
            double dbt = pick(minmod_sel(b, 4.0 * a), db, 4.0 * da);
            c->ql[i][n] = df + qt * (thm * dat + thp * dbt);
            c->qr[i][n] = df - qt * (thp * dat + thm * dbt);
         } else {
            double den = a * a + b * b + eps;
            double s = (2.0 * a * b + eps) / den;
            double ds = (2.0 * (da * b + a * db) - s * (2.0 * (a * da + b * db))) / den;
            double sk = th * s, dsk = th * ds;
            double A = (1.0 - sk) * a + (1.0 + sk) * b;
            double dA = (1.0 - sk) * da + (1.0 + sk) * db + dsk * (b - a);
            double B = (1.0 + sk) * a + (1.0 - sk) * b;
            double dB = (1.0 + sk) * da + (1.0 - sk) * db + dsk * (a - b);
            c->ql[i][n] = df + qt * (ds * A + s * dA);
            c->qr[i][n] = df - qt * (ds * B + s * dB);
         }
      }
   }
}

static void muscl(ho_case* c, int is, int ie, double qt)
{
   const double th = 0.3333333333333333e+00, eps = 1e-10;
   double thm = 1.0 - th, thp = 1.0 + th;
   int i, n;
   if (qt == 0.0) {
      for (n = 0; n < NQ; n++)
         for (i = is; i <= ie; i++) c->ql[i][n] = c->qr[i][n] = c->f[i][n];
      return;
   }
   if (c->limiter != HO_LIMITER_REFERENCE) {
      muscl_lim(c, is, ie, qt);
      return;
   }
   for (n = 0; n < NQ; n++) {
      for (i = 0; i < ie; i++) c->f2[i][n] = c->f[i + 1][n] - c->f[i][n];
      for (i = is; i < ie; i++) {
         double f2i = c->f2[i][n], f2i1 = c->f2[i - 1][n];
         double a1 = 3.0 * (f2i * f2i1 + eps);
         double a2 = 2.0 * (f2i - f2i1) * (f2i - f2i1) + a1;
         double f3qt = qt * (a1 / a2);
         c->ql[i][n] = c->f[i][n] + f3qt * (thm * f2i1 + thp * f2i);
         c->qr[i][n] = c->f[i][n] - f3qt * (thp * f2i1 + thm * f2i);
      }
   }
}

/* MUSCL_DERIV, reconstruction.cpp:168-236: linearisation of muscl about f
   applied to df, written into ql/qr */
static void muscl_deriv(ho_case* c, int is, int ie, double qt)
{
   const double th = 0.3333333333333333e+00, eps = 1e-10;
   double thm = 1.0 - th, thp = 1.0 + th;
   int i, n;
   if (qt == 0.0) {
      for (n = 0; n < NQ; n++)
         for (i = is; i <= ie; i++) c->ql[i][n] = c->qr[i][n] = c->df[i][n];
      return;
   }
   if (c->limiter != HO_LIMITER_REFERENCE) {
      muscl_lim_deriv(c, is, ie, qt);
      return;
   }
   for (n = 0; n < NQ; n++) {
      for (i = 0; i < ie; i++) c->f2[i][n] = c->f[i + 1][n] - c->f[i][n];
      for (i = is; i < ie; i++) {
         double f2i = c->f2[i][n], f2i1 = c->f2[i - 1][n];
         double df2i = c->df[i + 1][n] - c->df[i][n];
         double df2i1 = c->df[i][n] - c->df[i - 1][n];
         double a1 = 3.0 * (f2i * f2i1 + eps);
         double da1 = 3.0 * (df2i * f2i1 + f2i * df2i1);
         double a2 = 2.0 * (f2i - f2i1) * (f2i - f2i1) + a1;
         double da2 = 2.0 * 2.0 * (f2i - f2i1) * (df2i - df2i1) + da1;
         double f3i = a1 / a2;
         double df3i = da1 / a2 - a1 * da2 / (a2 * a2);
         double f3qt = qt * f3i, df3qt = qt * df3i;
         c->ql[i][n] = c->df[i][n] + df3qt * (thm * f2i1 + thp * f2i) + f3qt * (thm * df2i1 + thp * df2i);
         c->qr[i][n] = c->df[i][n] - df3qt * (thp * f2i1 + thm * f2i) - f3qt * (thp * df2i1 + thm * df2i);
      }
   }
}

/* WENO5 kernel, reconstruction.cpp:78-124 (pow(x,1) == x) */
static double weno5(double a, double b, double cc, double d, double e)
{
   const double epsw = 1e-15;
   double b1 = 13. / 12., b2 = 1. / 6.;
   double djm1 = a - 2. * b + cc;
   double ejm1 = a - 4. * b + 3. * cc;
   double dj = b - 2. * cc + d;
   double ej = b - d;
   double djp1 = cc - 2. * d + e;
   double ejp1 = 3. * cc - 4. * d + e;
   double dis0 = b1 * djm1 * djm1 + 0.25 * ejm1 * ejm1 + epsw;
   double dis1 = b1 * dj * dj + 0.25 * ej * ej + epsw;
   double dis2 = b1 * djp1 * djp1 + 0.25 * ejp1 * ejp1 + epsw;
   double q30 = 2. * a - 7. * b + 11. * cc;
   double q31 = -b + 5. * cc + 2. * d;
   double q32 = 2. * cc + 5. * d - e;
   double d01 = dis0 / dis1, d02 = dis0 / dis2;
   double a1ba0 = 6. * d01, a2ba0 = 3. * d02;
   double w0 = 1.0 / (1.0 + a1ba0 + a2ba0);
   double w1 = a1ba0 * w0;
   double w2 = 1. - w0 - w1;
   return b2 * (w0 * q30 + w1 * q31 + w2 * q32);
}

/* WENO wrapper, reconstruction.cpp:133-160, slots is..size-3 */
static void weno(ho_case* c, int is, int size)
{
   int i, n;
   for (n = 0; n < NQ; n++)
      for (i = is; i < size - 2; i++) {
         c->ql[i][n] = weno5(c->f[i - 2][n], c->f[i - 1][n], c->f[i][n], c->f[i + 1][n], c->f[i + 2][n]);
         c->qr[i][n] = weno5(c->f[i + 2][n], c->f[i + 1][n], c->f[i][n], c->f[i - 1][n], c->f[i - 2][n]);
      }
}

/* WENO_5 linearisation, reconstruction.cpp:243-347 */
static double weno5_deriv_eps(double a, double b, double cc, double d, double e,
                              double a_d, double b_d, double c_d, double d_d, double e_d, double epsw)
{
   double b1 = 13. / 12., b2 = 1. / 6.;
   double djm1 = a - 2. * b + cc;
   double ejm1 = a - 4. * b + 3. * cc;
   double dj = b - 2. * cc + d;
   double ej = b - d;
   double djp1 = cc - 2. * d + e;
   double ejp1 = 3. * cc - 4. * d + e;
   double dis0 = b1 * djm1 * djm1 + 0.25 * ejm1 * ejm1 + epsw;
   double dis1 = b1 * dj * dj + 0.25 * ej * ej + epsw;
   double dis2 = b1 * djp1 * djp1 + 0.25 * ejp1 * ejp1 + epsw;
   double q30 = 2. * a - 7. * b + 11. * cc;
   double q31 = -b + 5. * cc + 2. * d;
   double q32 = 2. * cc + 5. * d - e;
   double d01 = dis0 / dis1, d02 = dis0 / dis2;
   double a1ba0 = 6. * d01, a2ba0 = 3. * d02;
   double w0 = 1.0 / (1.0 + a1ba0 + a2ba0);
   double w1 = a1ba0 * w0;
   double w2 = 1. - w0 - w1;
   double djm1_d = a_d - 2. * b_d + c_d;
   double ejm1_d = a_d - 4. * b_d + 3. * c_d;
   double dj_d = b_d - 2. * c_d + d_d;
   double ej_d = b_d - d_d;
   double djp1_d = c_d - 2. * d_d + e_d;
   double ejp1_d = 3. * c_d - 4. * d_d + e_d;
   double q30_d = 2. * a_d - 7. * b_d + 11. * c_d;
   double q31_d = -b_d + 5. * c_d + 2. * d_d;
   double q32_d = 2. * c_d + 5. * d_d - e_d;
   double term1 = b2 * w0 * q30_d;
   double term2 = b2 * w1 * q31_d;
   double term3 = b2 * w2 * q32_d;
   double dbeta0 = b1 * 2 * djm1 * djm1_d + 0.25 * 2 * ejm1 * ejm1_d;
   double dbeta1 = b1 * 2 * dj * dj_d + 0.25 * 2 * ej * ej_d;
   double dbeta2 = b1 * 2 * djp1 * djp1_d + 0.25 * 2 * ejp1 * ejp1_d;
   double beta0 = dis0, beta1 = dis1, beta2 = dis2;
   double dw0_down = beta1 * beta2 + 6 * beta0 * beta2 + 3 * beta0 * beta1;
   double dw0_up_1 = (dbeta1 * beta2 + beta1 * dbeta2) * dw0_down;
   double dw0_up_2 = beta1 * beta2 * (dbeta1 * beta2 + beta1 * dbeta2 + 6 * (dbeta0 * beta2 + beta0 * dbeta2)
                                      + 3 * (dbeta0 * beta1 + beta0 * dbeta1));
   double dw0 = (dw0_up_1 - dw0_up_2) / (dw0_down * dw0_down);
   double dw1_up_1 = 6 * (dbeta0 * beta2 + beta0 * dbeta2) * dw0_down;
   double dw1_up_2 = 6 * dw0_up_2 / beta1 * beta0;
   double dw1 = (dw1_up_1 - dw1_up_2) / (dw0_down * dw0_down);
   double dw2_up_1 = 3 * (dbeta0 * beta1 + beta0 * dbeta1) * dw0_down;
   double dw2_up_2 = 3 * dw0_up_2 / beta2 * beta0;
   double dw2 = (dw2_up_1 - dw2_up_2) / (dw0_down * dw0_down);
   return term1 + term2 + term3 + b2 * dw0 * q30 + b2 * dw1 * q31 + b2 * dw2 * q32;
}

static double weno5_deriv(double a, double b, double cc, double d, double e,
                          double a_d, double b_d, double c_d, double d_d, double e_d)
{
   /* the caller passes eps=1e-10 (computeLinearRHS.cpp:286) */
   return weno5_deriv_eps(a, b, cc, d, e, a_d, b_d, c_d, d_d, e_d, 1e-10);
}

/* WENO_DERIV wrapper, reconstruction.cpp:353-386 */
static void weno_deriv(ho_case* c, int is, int size)
{
   int i, n;
   for (n = 0; n < NQ; n++)
      for (i = is; i < size - 2; i++) {
         c->ql[i][n] = weno5_deriv(c->f[i - 2][n], c->f[i - 1][n], c->f[i][n], c->f[i + 1][n], c->f[i + 2][n],
                                   c->df[i - 2][n], c->df[i - 1][n], c->df[i][n], c->df[i + 1][n], c->df[i + 2][n]);
         c->qr[i][n] = weno5_deriv(c->f[i + 2][n], c->f[i + 1][n], c->f[i][n], c->f[i - 1][n], c->f[i - 2][n],
                                   c->df[i + 2][n], c->df[i + 1][n], c->df[i][n], c->df[i - 1][n], c->df[i - 2][n]);
      }
}

/* ------------------------------------------------------------------ */
/* Roe flux (interfaceFlux.cpp:24-169)                                 */
/* ------------------------------------------------------------------ */

static int roe_flux(const double* s, const double* ql, const double* qr,
                    double* flux, double* spec, double gamma)
{
   double gm1 = gamma - 1.0;
   double nxd = s[0], nyd = s[1];
   double area = sqrt(nxd * nxd + nyd * nyd);
   double invArea = 1. / area;
   double nx = nxd * invArea, ny = nyd * invArea;
   double rol = ql[0], ul = ql[1] / ql[0], vl = ql[2] / ql[0];
   double pl = gm1 * (ql[3] - 0.5 * rol * (ul * ul + vl * vl));
   double hl = (ql[3] + pl) / rol;
   double ror = qr[0], ur = qr[1] / qr[0], vr = qr[2] / qr[0];
   double pr = gm1 * (qr[3] - 0.5 * ror * (ur * ur + vr * vr));
   double hr = (qr[3] + pr) / ror;
   double dp = pr - pl;
   double uconr = ur * nx + vr * ny, uconl = ul * nx + vl * ny;
   double fact = sqrt(ror / rol);
   double A = 1.0 / (1.0 + fact), B = fact / (1.0 + fact);
   double robar = rol * fact;
   double ubar = ul * A + ur * B, vbar = vl * A + vr * B, hbar = hl * A + hr * B;
   double cbar = gm1 * (hbar - 0.5 * (ubar * ubar + vbar * vbar));
   double uconbar, eig1, eig2, eig3, term1, term2, del1, del2, fm[4], fl[4], fr[4];
   int i;
   cbar = sqrt(cbar);
   uconbar = ubar * nx + vbar * ny;
   eig1 = fabs(uconbar);
   eig2 = fabs(uconbar + cbar);
   eig3 = fabs(uconbar - cbar);
   *spec = eig1 + cbar;
   if (*spec != *spec) return -1;
   term1 = -eig1 + 0.5 * (eig2 + eig3);
   term2 = 0.5 * (eig2 - eig3);
   del1 = term1 * dp / cbar / cbar + term2 * robar * (uconr - uconl) / cbar;
   del2 = term1 * (uconr - uconl) * robar + term2 * dp / cbar;
   for (i = 0; i < 4; i++) fm[i] = eig1 * (qr[i] - ql[i]);
   fm[0] = fm[0] + del1;
   fm[1] = fm[1] + del1 * ubar + del2 * nx;
   fm[2] = fm[2] + del1 * vbar + del2 * ny;
   fm[3] = fm[3] + del1 * hbar + del2 * uconbar;
   fl[0] = rol * uconl;               fr[0] = ror * uconr;
   fl[1] = rol * uconl * ul + nx * pl; fr[1] = ror * uconr * ur + nx * pr;
   fl[2] = rol * uconl * vl + ny * pl; fr[2] = ror * uconr * vr + ny * pr;
   fl[3] = (ql[3] + pl) * uconl;       fr[3] = (qr[3] + pr) * uconr;
   for (i = 0; i < 4; i++) {
      flux[i] = 0.5 * (fl[i] + fr[i] - fm[i]);
      flux[i] *= area;
   }
   *spec *= area;
   return 0;
}

/* ------------------------------------------------------------------ */
/* Roe flux Jacobian, frozen eigenvalues (jacobianRoe.cpp:9-70,92-620) */
/* jacobianRoe3D (IMODE 1) on 5 variables; the 2D form embeds its      */
/* state (w = 0) and reduces with the index map {0,1,2,4} x area.      */
/* ------------------------------------------------------------------ */

static void roe_jacobian3d(const double* nxyz, const double* ql, const double* qr, double lmat[5][5],
                           double rmat[5][5], double gam)
{
   double nxd, nyd, nzd, area, nx, ny, nz;
   double gm1 = gam - 1.0;
   double rol, ul, vl, wl, pl, hl, ror, ur, vr, wr, pr, hr, dp, uconl, uconr;
   double dro_dql[5], dro_dqr[5], du_dql[5], du_dqr[5], dv_dql[5], dv_dqr[5];
   double dw_dql[5], dw_dqr[5], dp_dql[5], dp_dqr[5], ducon_dql[5], ducon_dqr[5];
   double dq5_dql[5], dq5_dqr[5];
   double ddel1_dql[5], ddel1_dqr[5], ddel2_dql[5], ddel2_dqr[5];
   double fact, A, B, robar, ubar, vbar, wbar, hbar, cbar, uconbar, eig1, eig2, eig3, term1, term2;
   double lmat1[5][5], rmat1[5][5];
   int i, j;

   nxd = nxyz[0]; nyd = nxyz[1]; nzd = nxyz[2];
   area = sqrt(nxd * nxd + nyd * nyd + nzd * nzd);
   nx = nxd / area; ny = nyd / area; nz = nzd / area;

   rol = ql[0];
   ul = ql[1] / ql[0]; vl = ql[2] / ql[0]; wl = ql[3] / ql[0];
   pl = gm1 * (ql[4] - 0.5 * rol * (ul * ul + vl * vl + wl * wl));
   hl = (ql[4] + pl) / rol;
   ror = qr[0];
   ur = qr[1] / qr[0]; vr = qr[2] / qr[0]; wr = qr[3] / qr[0];
   pr = gm1 * (qr[4] - 0.5 * ror * (ur * ur + vr * vr + wr * wr));
   hr = (qr[4] + pr) / ror;
   dp = pr - pl;   /* formed as the reference forms it; the Jacobian does not use it */
   (void)dp;
   uconr = ur * nx + vr * ny + wr * nz;
   uconl = ul * nx + vl * ny + wl * nz;

   for (i = 0; i < 5; i++) dro_dql[i] = 0.0;
   dro_dql[0] = 1.0;
   for (i = 0; i < 5; i++) du_dql[i] = 0.0;
   du_dql[0] = -ul / rol; du_dql[1] = 1.0 / rol;
   for (i = 0; i < 5; i++) dv_dql[i] = 0.0;
   dv_dql[0] = -vl / rol; dv_dql[2] = 1.0 / rol;
   for (i = 0; i < 5; i++) dw_dql[i] = 0.0;
   dw_dql[0] = -wl / rol; dw_dql[3] = 1.0 / rol;
   dp_dql[0] = 0.5 * gm1 * (ul * ul + vl * vl + wl * wl);
   dp_dql[1] = -gm1 * ul; dp_dql[2] = -gm1 * vl; dp_dql[3] = -gm1 * wl; dp_dql[4] = gm1;
   for (i = 0; i < 5; i++) dq5_dql[i] = 0.0;
   dq5_dql[4] = 1.0;
   ducon_dql[0] = -uconl / rol; ducon_dql[1] = nx / rol; ducon_dql[2] = ny / rol;
   ducon_dql[3] = nz / rol; ducon_dql[4] = 0.0;

   for (i = 0; i < 5; i++) dro_dqr[i] = 0.0;
   dro_dqr[0] = 1.0;
   for (i = 0; i < 5; i++) du_dqr[i] = 0.0;
   du_dqr[0] = -ur / ror; du_dqr[1] = 1.0 / ror;
   for (i = 0; i < 5; i++) dv_dqr[i] = 0.0;
   dv_dqr[0] = -vr / ror; dv_dqr[2] = 1.0 / ror;
   for (i = 0; i < 5; i++) dw_dqr[i] = 0.0;
   dw_dqr[0] = -wr / ror; dw_dqr[3] = 1.0 / ror;
   dp_dqr[0] = 0.5 * gm1 * (ur * ur + vr * vr + wr * wr);
   dp_dqr[1] = -gm1 * ur; dp_dqr[2] = -gm1 * vr; dp_dqr[3] = -gm1 * wr; dp_dqr[4] = gm1;
   for (i = 0; i < 5; i++) dq5_dqr[i] = 0.0;
   dq5_dqr[4] = 1.0;
   ducon_dqr[0] = -uconr / ror; ducon_dqr[1] = nx / ror; ducon_dqr[2] = ny / ror;
   ducon_dqr[3] = nz / ror; ducon_dqr[4] = 0.0;

   fact = sqrt(ror / rol);
   A = 1.0 / (1.0 + fact);
   B = fact / (1.0 + fact);
   robar = rol * fact;
   ubar = ul * A + ur * B;
   vbar = vl * A + vr * B;
   wbar = wl * A + wr * B;
   hbar = hl * A + hr * B;
   cbar = gm1 * (hbar - 0.5 * (ubar * ubar + vbar * vbar + wbar * wbar));
   cbar = sqrt(cbar);
   uconbar = ubar * nx + vbar * ny + wbar * nz;
   eig1 = fabs(uconbar);
   eig2 = fabs(uconbar + cbar);
   eig3 = fabs(uconbar - cbar);

   term1 = -eig1 + 0.5 * (eig2 + eig3);
   term2 = 0.5 * (eig2 - eig3);
   for (i = 0; i < 5; i++) {
      ddel1_dql[i] = -term1 * dp_dql[i] / cbar / cbar - term2 * robar * ducon_dql[i] / cbar;
      ddel1_dqr[i] = +term1 * dp_dqr[i] / cbar / cbar + term2 * robar * ducon_dqr[i] / cbar;
      ddel2_dql[i] = -term1 * ducon_dql[i] * robar - term2 * dp_dql[i] / cbar;
      ddel2_dqr[i] = +term1 * ducon_dqr[i] * robar + term2 * dp_dqr[i] / cbar;
   }

   for (i = 0; i < 5; i++)
      for (j = 0; j < 5; j++) {
         double im = (i == j) ? 1.0 : 0.0;
         lmat[i][j] = 0.0 - eig1 * im;
         rmat[i][j] = 0.0 + eig1 * im;
      }
   for (i = 0; i < 5; i++) {
      lmat[0][i] = lmat[0][i] + ddel1_dql[i];
      rmat[0][i] = rmat[0][i] + ddel1_dqr[i];
      lmat[1][i] = lmat[1][i] + ddel1_dql[i] * ubar + ddel2_dql[i] * nx;
      rmat[1][i] = rmat[1][i] + ddel1_dqr[i] * ubar + ddel2_dqr[i] * nx;
      lmat[2][i] = lmat[2][i] + ddel1_dql[i] * vbar + ddel2_dql[i] * ny;
      rmat[2][i] = rmat[2][i] + ddel1_dqr[i] * vbar + ddel2_dqr[i] * ny;
      lmat[3][i] = lmat[3][i] + ddel1_dql[i] * wbar + ddel2_dql[i] * nz;
      rmat[3][i] = rmat[3][i] + ddel1_dqr[i] * wbar + ddel2_dqr[i] * nz;
      lmat[4][i] = lmat[4][i] + ddel1_dql[i] * hbar + ddel2_dql[i] * uconbar;
      rmat[4][i] = rmat[4][i] + ddel1_dqr[i] * hbar + ddel2_dqr[i] * uconbar;
   }
   for (i = 0; i < 5; i++) {
      lmat1[0][i] = dro_dql[i] * uconl + rol * ducon_dql[i];
      lmat1[1][i] = dro_dql[i] * uconl * ul + rol * ducon_dql[i] * ul + rol * uconl * du_dql[i];
      lmat1[2][i] = dro_dql[i] * uconl * vl + rol * ducon_dql[i] * vl + rol * uconl * dv_dql[i];
      lmat1[3][i] = dro_dql[i] * uconl * wl + rol * ducon_dql[i] * wl + rol * uconl * dw_dql[i];
      lmat1[2][i] = lmat1[2][i] + ny * dp_dql[i];
      lmat1[1][i] = lmat1[1][i] + nx * dp_dql[i];
      lmat1[3][i] = lmat1[3][i] + nz * dp_dql[i];
      lmat1[4][i] = (dq5_dql[i] + dp_dql[i]) * uconl + (ql[4] + pl) * ducon_dql[i];

      rmat1[0][i] = dro_dqr[i] * uconr + ror * ducon_dqr[i];
      rmat1[1][i] = dro_dqr[i] * uconr * ur + ror * ducon_dqr[i] * ur + ror * uconr * du_dqr[i];
      rmat1[2][i] = dro_dqr[i] * uconr * vr + ror * ducon_dqr[i] * vr + ror * uconr * dv_dqr[i];
      rmat1[3][i] = dro_dqr[i] * uconr * wr + ror * ducon_dqr[i] * wr + ror * uconr * dw_dqr[i];
      rmat1[2][i] = rmat1[2][i] + ny * dp_dqr[i];
      rmat1[1][i] = rmat1[1][i] + nx * dp_dqr[i];
      rmat1[3][i] = rmat1[3][i] + nz * dp_dqr[i];
      rmat1[4][i] = (dq5_dqr[i] + dp_dqr[i]) * uconr + (qr[4] + pr) * ducon_dqr[i];
   }
   for (i = 0; i < 5; i++)
      for (j = 0; j < 5; j++) {
         lmat[i][j] = 0.5 * (lmat1[i][j] - lmat[i][j]);
         rmat[i][j] = 0.5 * (rmat1[i][j] - rmat[i][j]);
      }
}

/* jacobianRoe2D (jacobianRoe.cpp:9-70): the state embedded in 5 variables
   with w = 0 and nz = 0, the 3D Jacobian, rows and columns {0,1,2,4} kept,
   times the face area */
static void roe_jacobian(const double* s, const double* ql2, const double* qr2,
                         double* lm2, double* rm2, double gam)
{
   double ql[5], qr[5], nxyz[3], lmat[5][5], rmat[5][5], area2;
   static const int idiv[4] = {0, 1, 2, 4};
   int i, j;
   ql[0] = ql2[0]; ql[1] = ql2[1]; ql[2] = ql2[2]; ql[3] = 0; ql[4] = ql2[3];
   qr[0] = qr2[0]; qr[1] = qr2[1]; qr[2] = qr2[2]; qr[3] = 0; qr[4] = qr2[3];
   nxyz[0] = s[0]; nxyz[1] = s[1]; nxyz[2] = 0;
   area2 = sqrt(s[0] * s[0] + s[1] * s[1]);
   roe_jacobian3d(nxyz, ql, qr, lmat, rmat, gam);
   for (i = 0; i < 4; i++)
      for (j = 0; j < 4; j++) {
         lm2[4 * i + j] = lmat[idiv[i]][idiv[j]] * area2;
         rm2[4 * i + j] = rmat[idiv[i]][idiv[j]] * area2;
      }
}

/* ------------------------------------------------------------------ */
/* The reference's per-face and per-line functions on flat arrays      */
/* (the checker of the library's function-level entry points)          */
/* ------------------------------------------------------------------ */

/* SOLVER::fluxRoe2D (interfaceFlux.cpp:24-169): -1 where the reference
   exits on a NaN spectral radius */
int ho_flux_roe2d(const double* nxy, const double* ql, const double* qr, double* flux, double* spec, double gamma)
{
   return roe_flux(nxy, ql, qr, flux, spec, gamma);
}

/* SOLVER::jacobianRoe2D (jacobianRoe.cpp:9-70): lm, rm [4][4] row-major */
void ho_jacobian_roe2d(const double* nxy, const double* ql, const double* qr, double* lm, double* rm, double gamma)
{
   roe_jacobian(nxy, ql, qr, lm, rm, gamma);
}

/* SOLVER::fluxRoe3D (interfaceFlux.cpp:176-319) for one face of the 5-variable
   (3D strand) build: unlike the 2D flux, neither the flux nor the spectral
   radius is multiplied by the face area */
void ho_flux_roe3d(const double* nxyz, const double* ql, const double* qr, double* flux, double* spec, double gamma)
{
   double gm1 = gamma - 1.0;
   double nxd = nxyz[0], nyd = nxyz[1], nzd = nxyz[2];
   double area = sqrt(nxd * nxd + nyd * nyd + nzd * nzd);
   double invArea = 1. / area;
   double nx = nxd * invArea, ny = nyd * invArea, nz = nzd * invArea;
   double rol = ql[0], ul = ql[1] / ql[0], vl = ql[2] / ql[0], wl = ql[3] / ql[0];
   double pl = gm1 * (ql[4] - 0.5 * rol * (ul * ul + vl * vl + wl * wl));
   double hl = (ql[4] + pl) / rol;
   double ror = qr[0], ur = qr[1] / qr[0], vr = qr[2] / qr[0], wr = qr[3] / qr[0];
   double pr = gm1 * (qr[4] - 0.5 * ror * (ur * ur + vr * vr + wr * wr));
   double hr = (qr[4] + pr) / ror;
   double dp = pr - pl;
   double uconr = ur * nx + vr * ny + wr * nz, uconl = ul * nx + vl * ny + wl * nz;
   double fact = sqrt(ror / rol);
   double A = 1.0 / (1.0 + fact), B = fact / (1.0 + fact);
   double robar = rol * fact;
   double ubar = ul * A + ur * B, vbar = vl * A + vr * B, wbar = wl * A + wr * B, hbar = hl * A + hr * B;
   double cbar = gm1 * (hbar - 0.5 * (ubar * ubar + vbar * vbar + wbar * wbar));
   double uconbar, eig1, eig2, eig3, term1, term2, del1, del2, fm[5], fl[5], fr[5];
   int i;
   cbar = sqrt(cbar);
   uconbar = ubar * nx + vbar * ny + wbar * nz;
   eig1 = fabs(uconbar);
   eig2 = fabs(uconbar + cbar);
   eig3 = fabs(uconbar - cbar);
   *spec = eig1 + cbar;
   term1 = -eig1 + 0.5 * (eig2 + eig3);
   term2 = 0.5 * (eig2 - eig3);
   del1 = term1 * dp / cbar / cbar + term2 * robar * (uconr - uconl) / cbar;
   del2 = term1 * (uconr - uconl) * robar + term2 * dp / cbar;
   for (i = 0; i < 5; i++) fm[i] = eig1 * (qr[i] - ql[i]);
   fm[0] = fm[0] + del1;
   fm[1] = fm[1] + del1 * ubar + del2 * nx;
   fm[2] = fm[2] + del1 * vbar + del2 * ny;
   fm[3] = fm[3] + del1 * wbar + del2 * nz;
   fm[4] = fm[4] + del1 * hbar + del2 * uconbar;
   fl[0] = rol * uconl;                fr[0] = ror * uconr;
   fl[1] = rol * uconl * ul + nx * pl; fr[1] = ror * uconr * ur + nx * pr;
   fl[2] = rol * uconl * vl + ny * pl; fr[2] = ror * uconr * vr + ny * pr;
   fl[3] = rol * uconl * wl + nz * pl; fr[3] = ror * uconr * wr + nz * pr;
   fl[4] = (ql[4] + pl) * uconl;       fr[4] = (qr[4] + pr) * uconr;
   for (i = 0; i < 5; i++) flux[i] = 0.5 * (fl[i] + fr[i] - fm[i]);
}

/* SOLVER::jacobianRoe3D (jacobianRoe.cpp:92-620, IMODE 1): lm, rm [5][5] */
void ho_jacobian_roe3d(const double* nxyz, const double* ql, const double* qr, double* lm, double* rm, double gamma)
{
   double lmat[5][5], rmat[5][5];
   int i, j;
   roe_jacobian3d(nxyz, ql, qr, lmat, rmat, gamma);
   for (i = 0; i < 5; i++)
      for (j = 0; j < 5; j++) {
         lm[5 * i + j] = lmat[i][j];
         rm[5 * i + j] = rmat[i][j];
      }
}

/* The 5x5 unpivoted LU with reciprocal pivots of triSolvers.cpp:481-506
   (blockTridag and blockTridagPeriodic use the same steps) and its solve
   (:508-518, :523-534) */
typedef struct { double b11, b21, b22, b31, b32, b33, b41, b42, b43, b44, b51, b52, b53, b54, b55,
                 u12, u13, u14, u15, u23, u24, u25, u34, u35, u45; } lu5;

static lu5 lu5_factor(double b[5][5])
{
   lu5 u;
   u.b11 = 1. / b[0][0];
   u.u12 = b[0][1] * u.b11; u.u13 = b[0][2] * u.b11; u.u14 = b[0][3] * u.b11; u.u15 = b[0][4] * u.b11;
   u.b21 = b[1][0];
   u.b22 = 1. / (b[1][1] - u.b21 * u.u12);
   u.u23 = (b[1][2] - u.b21 * u.u13) * u.b22;
   u.u24 = (b[1][3] - u.b21 * u.u14) * u.b22;
   u.u25 = (b[1][4] - u.b21 * u.u15) * u.b22;
   u.b31 = b[2][0];
   u.b32 = b[2][1] - u.b31 * u.u12;
   u.b33 = 1. / (b[2][2] - u.b31 * u.u13 - u.b32 * u.u23);
   u.u34 = (b[2][3] - u.b31 * u.u14 - u.b32 * u.u24) * u.b33;
   u.u35 = (b[2][4] - u.b31 * u.u15 - u.b32 * u.u25) * u.b33;
   u.b41 = b[3][0];
   u.b42 = b[3][1] - u.b41 * u.u12;
   u.b43 = b[3][2] - u.b41 * u.u13 - u.b42 * u.u23;
   u.b44 = 1. / (b[3][3] - u.b41 * u.u14 - u.b42 * u.u24 - u.b43 * u.u34);
   u.u45 = (b[3][4] - u.b41 * u.u15 - u.b42 * u.u25 - u.b43 * u.u35) * u.b44;
   u.b51 = b[4][0];
   u.b52 = b[4][1] - u.b51 * u.u12;
   u.b53 = b[4][2] - u.b51 * u.u13 - u.b52 * u.u23;
   u.b54 = b[4][3] - u.b51 * u.u14 - u.b52 * u.u24 - u.b53 * u.u34;
   u.b55 = 1. / (b[4][4] - u.b51 * u.u15 - u.b52 * u.u25 - u.b53 * u.u35 - u.b54 * u.u45);
   return u;
}

/* x <- LU^{-1} x for the 5 values x[0], x[s], ..., x[4s] */
static void lu5_solve(const lu5* u, double* x, int s)
{
   double d1 = x[0] * u->b11;
   double d2 = (x[s] - u->b21 * d1) * u->b22;
   double d3 = (x[2 * s] - u->b31 * d1 - u->b32 * d2) * u->b33;
   double d4 = (x[3 * s] - u->b41 * d1 - u->b42 * d2 - u->b43 * d3) * u->b44;
   double d5 = (x[4 * s] - u->b51 * d1 - u->b52 * d2 - u->b53 * d3 - u->b54 * d4) * u->b55;
   x[4 * s] = d5;
   x[3 * s] = d4 - u->u45 * d5;
   x[2 * s] = d3 - u->u34 * x[3 * s] - u->u35 * d5;
   x[s] = d2 - u->u23 * x[2 * s] - u->u24 * x[3 * s] - u->u25 * d5;
   x[0] = d1 - u->u12 * x[s] - u->u13 * x[2 * s] - u->u14 * x[3 * s] - u->u15 * d5;
}

/* TRISOLVER::blockTridag (triSolvers.cpp:443-536) and blockTridagPeriodic
   (:540-766), nq = 5, on flat [N][5][5] blocks and [N][5] right-hand sides,
   in place: a, b, c are overwritten as the reference's scratch */
int ho_block_tridag5(double* ap, double* bp, double* cp, double* fp, int N, int periodic)
{
   double (*a)[5][5] = (double (*)[5][5])ap, (*b)[5][5] = (double (*)[5][5])bp, (*c)[5][5] = (double (*)[5][5])cp;
   double (*f)[5] = (double (*)[5])fp;
   double t[5][5];
   int i, j, k, l;
   if (N < 1 || (periodic && N < 2)) return -1;
   for (i = 0; i < N; i++) {
      lu5 u;
      if (i != 0) {
         for (k = 0; k < 5; k++)
            for (j = 0; j < 5; j++)
               for (l = 0; l < 5; l++) b[i][k][j] -= a[i][k][l] * c[i - 1][l][j];
         for (k = 0; k < 5; k++)
            for (j = 0; j < 5; j++) f[i][k] -= a[i][k][j] * f[i - 1][j];
         if (periodic) {
            for (k = 0; k < 5; k++)
               for (j = 0; j < 5; j++) t[k][j] = 0;
            for (k = 0; k < 5; k++)
               for (j = 0; j < 5; j++)
                  for (l = 0; l < 5; l++) t[k][j] -= a[i][k][l] * a[i - 1][l][j];
            for (k = 0; k < 5; k++)
               for (j = 0; j < 5; j++) a[i][k][j] = t[k][j];
         }
      }
      u = lu5_factor(b[i]);
      lu5_solve(&u, f[i], 1);
      if (!periodic) {
         if (i != N - 1)
            for (j = 0; j < 5; j++) lu5_solve(&u, &c[i][0][j], 5);
      } else if (i != N - 2) {
         for (j = 0; j < 5; j++) {
            lu5_solve(&u, &c[i][0][j], 5);
            lu5_solve(&u, &a[i][0][j], 5);
         }
      } else {
         for (k = 0; k < 5; k++)
            for (j = 0; j < 5; j++) c[i][j][k] += a[i][j][k];
         for (j = 0; j < 5; j++) lu5_solve(&u, &c[i][0][j], 5);
         for (k = 0; k < 5; k++)
            for (j = 0; j < 5; j++) a[i][k][j] = c[i][k][j];
      }
   }
   if (!periodic) {
      for (i = N - 2; i >= 0; i--)
         for (k = 0; k < 5; k++)
            for (j = 0; j < 5; j++) f[i][k] -= c[i][k][j] * f[i + 1][j];
      return 0;
   }
   i = N - 1;
   for (k = 0; k < 5; k++)
      for (j = 0; j < 5; j++) b[i][j][k] = (j == k) ? 1.0 : 0.0;
   for (i = 0; i < N - 1; i++) {
      for (k = 0; k < 5; k++)
         for (j = 0; j < 5; j++) t[k][j] = 0;
      for (k = 0; k < 5; k++)
         for (j = 0; j < 5; j++)
            for (l = 0; l < 5; l++) {
               t[k][j] -= c[N - 1][k][l] * c[i][l][j];
               b[N - 1][k][j] -= c[N - 1][k][l] * a[i][l][j];
            }
      for (k = 0; k < 5; k++)
         for (j = 0; j < 5; j++) f[N - 1][k] -= c[N - 1][k][j] * f[i][j];
      for (k = 0; k < 5; k++)
         for (j = 0; j < 5; j++) c[N - 1][k][j] = t[k][j];
   }
   {
      lu5 u = lu5_factor(b[N - 1]);
      lu5_solve(&u, f[N - 1], 1);
   }
   i = N - 2;
   for (k = 0; k < 5; k++)
      for (j = 0; j < 5; j++) f[i][k] -= (c[i][k][j] * f[i + 1][j]);
   for (i = N - 3; i >= 0; i--)
      for (k = 0; k < 5; k++)
         for (j = 0; j < 5; j++) f[i][k] -= (c[i][k][j] * f[i + 1][j] + a[i][k][j] * f[N - 1][j]);
   return 0;
}

/* RECONSTRUCTION::MUSCL (reconstruction.cpp:16-70) on one line: f, ql, qr,
   f2 are [imax][nq]; loops and reads as the reference's, including f2[ie]
   at ie = imax-1, which it does not write */
void ho_muscl_line(const double* f, double* ql, double* qr, double* f2, int is, int ie, double th, double qt,
                   double eps, int imax, int nq)
{
   int i, n, im = imax - 1;
   double thm, thp;
   if (qt == 0.0) {
      for (n = 0; n < nq; n++)
         for (i = is; i <= ie; i++) {
            ql[i * nq + n] = f[i * nq + n];
            qr[i * nq + n] = f[i * nq + n];
         }
      return;
   }
   thm = 1.0 - th;
   thp = 1.0 + th;
   for (n = 0; n < nq; n++) {
      for (i = 0; i < im; i++) f2[i * nq + n] = f[(i + 1) * nq + n] - f[i * nq + n];
      for (i = is; i <= ie; i++) {
         double f2i = f2[i * nq + n], f2i1 = f2[(i - 1) * nq + n];
         double a1 = 3.0 * (f2i * f2i1 + eps);
         double a2 = 2.0 * (f2i - f2i1) * (f2i - f2i1) + a1;
         double f3i = a1 / a2;
         double f3qt = qt * f3i;
         ql[i * nq + n] = f[i * nq + n] + f3qt * (thm * f2i1 + thp * f2i);
         qr[i * nq + n] = f[i * nq + n] - f3qt * (thp * f2i1 + thm * f2i);
      }
   }
}

/* RECONSTRUCTION::MUSCL_DERIV (reconstruction.cpp:168-236) on one line */
void ho_muscl_deriv_line(const double* f, double* ql, double* qr, double* f2, const double* dq, int is, int ie,
                         double th, double qt, double eps, int imax, int nq)
{
   int i, n, im = imax - 1;
   double thm, thp;
   if (qt == 0.0) {
      for (n = 0; n < nq; n++)
         for (i = is; i <= ie; i++) {
            ql[i * nq + n] = dq[i * nq + n];
            qr[i * nq + n] = dq[i * nq + n];
         }
      return;
   }
   thm = 1.0 - th;
   thp = 1.0 + th;
   for (n = 0; n < nq; n++) {
      for (i = 0; i < im; i++) f2[i * nq + n] = f[(i + 1) * nq + n] - f[i * nq + n];
      for (i = is; i <= ie; i++) {
         double f2i = f2[i * nq + n], f2i1 = f2[(i - 1) * nq + n];
         double df2i = dq[(i + 1) * nq + n] - dq[i * nq + n];
         double df2i1 = dq[i * nq + n] - dq[(i - 1) * nq + n];
         double a1 = 3.0 * (f2i * f2i1 + eps);
         double da1 = 3.0 * (df2i * f2i1 + f2i * df2i1);
         double a2 = 2.0 * (f2i - f2i1) * (f2i - f2i1) + a1;
         double da2 = 2.0 * 2.0 * (f2i - f2i1) * (df2i - df2i1) + da1;
         double f3i = a1 / a2;
         double df3i = da1 / a2 - a1 * da2 / (a2 * a2);
         double f3qt = qt * f3i, df3qt = qt * df3i;
         ql[i * nq + n] = dq[i * nq + n] + df3qt * (thm * f2i1 + thp * f2i) + f3qt * (thm * df2i1 + thp * df2i);
         qr[i * nq + n] = dq[i * nq + n] - df3qt * (thp * f2i1 + thm * f2i) - f3qt * (thp * df2i1 + thm * df2i);
      }
   }
}

/* RECONSTRUCTION::WENO (reconstruction.cpp:133-160) on one line: entries
   is .. imax-3 from f[i-2 .. i+2]; the smoothness epsilon is 1e-15 (the
   reference overwrites epsw) */
void ho_weno_line(const double* f, double* ql, double* qr, int is, int ie, double epsw, int imax, int nq)
{
   int i, n;
   (void)ie;
   (void)epsw;
   for (n = 0; n < nq; n++)
      for (i = is; i < imax - 2; i++) {
         ql[i * nq + n] = weno5(f[(i - 2) * nq + n], f[(i - 1) * nq + n], f[i * nq + n], f[(i + 1) * nq + n],
                                f[(i + 2) * nq + n]);
         qr[i * nq + n] = weno5(f[(i + 2) * nq + n], f[(i + 1) * nq + n], f[i * nq + n], f[(i - 1) * nq + n],
                                f[(i - 2) * nq + n]);
      }
}

/* RECONSTRUCTION::WENO_DERIV (reconstruction.cpp:353-386) on one line */
void ho_weno_deriv_line(const double* f, double* ql, double* qr, const double* dq, int is, int ie, double eps,
                        int imax, int nq)
{
   int i, n;
   (void)ie;
   for (n = 0; n < nq; n++)
      for (i = is; i < imax - 2; i++) {
         const double* a = f + n;
         const double* d = dq + n;
         ql[i * nq + n] = weno5_deriv_eps(a[(i - 2) * nq], a[(i - 1) * nq], a[i * nq], a[(i + 1) * nq],
                                          a[(i + 2) * nq], d[(i - 2) * nq], d[(i - 1) * nq], d[i * nq],
                                          d[(i + 1) * nq], d[(i + 2) * nq], eps);
         qr[i * nq + n] = weno5_deriv_eps(a[(i + 2) * nq], a[(i + 1) * nq], a[i * nq], a[(i - 1) * nq],
                                          a[(i - 2) * nq], d[(i + 2) * nq], d[(i + 1) * nq], d[i * nq],
                                          d[(i - 1) * nq], d[(i - 2) * nq], eps);
      }
}

/* ------------------------------------------------------------------ */
/* residual (computeRHS.cpp:17-427)                                    */
/* ------------------------------------------------------------------ */

static void norms(ho_case* c)
{
   int i;
   c->LInfNorm = c->L2Norm = 0.0;
   for (i = 0; i < c->nCell; i++) {
      double t = fabs(c->r[NQ * i]);
      if (c->LInfNorm < t) c->LInfNorm = t;
      c->L2Norm += c->r[NQ * i] * c->r[NQ * i];
   }
   c->L2Norm = sqrt(c->L2Norm) / c->nCell;
}

int ho_compute_rhs(ho_case* c, int implicit, double* l2, double* linf)
{
   int i, j, f, k;
   for (i = 0; i < NQ * c->nCell; i++) c->r[i] = 0.0;
   for (i = 0; i < c->nCell; i++) c->sigma[i] = 0.0;
   for (i = 0; i < c->nChain; i++) {
      int f1 = c->faceStart[i], f2 = c->faceStart[i + 1];
      int size = chain_stencil(c, i);
      int is = c->nGhost - 1, ie = size - 1, n, per;
      if (chain_gather(c, i, size, NULL) != 0) return -2;
      if (c->order == 1 || c->order == 3) muscl(c, is, ie, c->order == 1 ? 0.0 : 0.25);
      if (c->order == 5) weno(c, is, size);
      n = is;
      per = (c->chainConn[f1] == c->chainConn[f2 - 1]);
      for (f = f1; f < f2 - per; f++) {
         int iface = c->chainConn[f];
         int left = c->faces[6 * iface + 2], right = c->faces[6 * iface + 4];
         double L[NQ], R[NQ], flux[NQ], spec;
         for (k = 0; k < NQ; k++) {
            if (f == f2 - per - 1 && per == 0) { L[k] = c->ql[n][k]; R[k] = c->qr[n + 1][k]; }
            else { L[k] = c->qr[n + 1][k]; R[k] = c->ql[n][k]; }
         }
         if (roe_flux(c->normVec + 2 * iface, L, R, flux, &spec, c->gamma) != 0) return -1;
         if (implicit) roe_jacobian(c->normVec + 2 * iface, L, R, c->ff + 32 * iface, c->ff + 32 * iface + 16, c->gamma);
         for (j = 0; j < NQ; j++) c->r[NQ * left + j] -= flux[j];
         c->sigma[left] += spec;
         if (right > -1) {
            for (j = 0; j < NQ; j++) c->r[NQ * right + j] += flux[j];
            c->sigma[right] += spec;
         }
         n++;
      }
   }
   norms(c);
   *l2 = c->L2Norm; *linf = c->LInfNorm;
   return 0;
}

/* ------------------------------------------------------------------ */
/* linear residual (computeLinearRHS.cpp:13-371)                       */
/* ------------------------------------------------------------------ */

int ho_linear_rhs(ho_case* c, double* l2, double* linf)
{
   int i, j, f, k;
   for (i = 0; i < NQ * c->nCell; i++) c->r[i] = (c->r0[i] - c->dq[i]);
   for (i = 0; i < c->nChain; i++) {
      int f1 = c->faceStart[i], f2 = c->faceStart[i + 1];
      int size = chain_stencil(c, i);
      int is = c->nGhost - 1, ie = size - 1, n, per;
      if (chain_gather(c, i, size, c->dq) != 0) return -2;
      if (c->sweep_order == 1 || c->order == 1) muscl_deriv(c, is, ie, 0.0);
      else if (c->order == 3) muscl_deriv(c, is, ie, 0.25);
      else if (c->order == 5) weno_deriv(c, is, size);
      n = is;
      per = (c->chainConn[f1] == c->chainConn[f2 - 1]);
      for (f = f1; f < f2 - per; f++) {
         int iface = c->chainConn[f];
         int left = c->faces[6 * iface + 2], right = c->faces[6 * iface + 4];
         const double* lm = c->ff + 32 * iface;
         const double* rm = lm + 16;
         double dL[NQ], dR[NQ], g[NQ], dtfac;
         for (k = 0; k < NQ; k++) {
            if (f == f2 - per - 1 && per == 0) { dL[k] = c->ql[n][k]; dR[k] = c->qr[n + 1][k]; }
            else { dL[k] = c->qr[n + 1][k]; dR[k] = c->ql[n][k]; }
         }
         for (j = 0; j < NQ; j++) {
            g[j] = 0;
            for (k = 0; k < NQ; k++) g[j] += ((lm[4 * j + k] * dL[k]) + (rm[4 * j + k] * dR[k]));
         }
         dtfac = c->CFL / c->sigma[left];
         for (j = 0; j < NQ; j++) c->r[NQ * left + j] -= (g[j] * dtfac);
         if (right > -1) {
            dtfac = c->CFL / c->sigma[right];
            for (j = 0; j < NQ; j++) c->r[NQ * right + j] += (g[j] * dtfac);
         }
         n++;
      }
   }
   norms(c);
   *l2 = c->L2Norm; *linf = c->LInfNorm;
   return 0;
}

/* ------------------------------------------------------------------ */
/* 4x4 block tridiagonal solvers (triSolvers.cpp:769-1046)             */
/* ------------------------------------------------------------------ */

/* unpivoted LU of a 4x4 block, reciprocal pivots (triSolvers.cpp:796-811) */
typedef struct { double b11, u12, u13, u14, b21, b22, u23, u24, b31, b32, b33, u34, b41, b42, b43, b44; } lu4;

static lu4 lu_factor(double b[NQ][NQ])
{
   lu4 u;
   u.b11 = 1. / b[0][0];
   u.u12 = b[0][1] * u.b11;
   u.u13 = b[0][2] * u.b11;
   u.u14 = b[0][3] * u.b11;
   u.b21 = b[1][0];
   u.b22 = 1. / (b[1][1] - u.b21 * u.u12);
   u.u23 = (b[1][2] - u.b21 * u.u13) * u.b22;
   u.u24 = (b[1][3] - u.b21 * u.u14) * u.b22;
   u.b31 = b[2][0];
   u.b32 = b[2][1] - u.b31 * u.u12;
   u.b33 = 1. / (b[2][2] - u.b31 * u.u13 - u.b32 * u.u23);
   u.u34 = (b[2][3] - u.b31 * u.u14 - u.b32 * u.u24) * u.b33;
   u.b41 = b[3][0];
   u.b42 = b[3][1] - u.b41 * u.u12;
   u.b43 = b[3][2] - u.b41 * u.u13 - u.b42 * u.u23;
   u.b44 = 1. / (b[3][3] - u.b41 * u.u14 - u.b42 * u.u24 - u.b43 * u.u34);
   return u;
}

/* x <- LU^{-1} x for a 4-vector with stride s (triSolvers.cpp:813-821) */
static void lu_solve(const lu4* u, double* x0, double* x1, double* x2, double* x3)
{
   double d1 = *x0 * u->b11;
   double d2 = (*x1 - u->b21 * d1) * u->b22;
   double d3 = (*x2 - u->b31 * d1 - u->b32 * d2) * u->b33;
   double d4 = (*x3 - u->b41 * d1 - u->b42 * d2 - u->b43 * d3) * u->b44;
   *x3 = d4;
   *x2 = d3 - u->u34 * *x3;
   *x1 = d2 - u->u23 * *x2 - u->u24 * *x3;
   *x0 = d1 - u->u12 * *x1 - u->u13 * *x2 - u->u14 * *x3;
}

static void lu_solve_cols(const lu4* u, double m[NQ][NQ])
{
   int j;
   for (j = 0; j < NQ; j++) lu_solve(u, &m[0][j], &m[1][j], &m[2][j], &m[3][j]);
}

/* blockTridag4, triSolvers.cpp:769-847 */
static void block_tridag4(double (*a)[NQ][NQ], double (*b)[NQ][NQ], double (*c)[NQ][NQ], double (*f)[NQ], int N)
{
   int i, j, k, l;
   for (i = 0; i < N; i++) {
      lu4 u;
      if (i != 0) {
         for (k = 0; k < NQ; k++)
            for (j = 0; j < NQ; j++)
               for (l = 0; l < NQ; l++) b[i][k][j] -= a[i][k][l] * c[i - 1][l][j];
         for (k = 0; k < NQ; k++)
            for (j = 0; j < NQ; j++) f[i][k] -= a[i][k][j] * f[i - 1][j];
      }
      u = lu_factor(b[i]);
      lu_solve(&u, &f[i][0], &f[i][1], &f[i][2], &f[i][3]);
      if (i != N - 1) lu_solve_cols(&u, c[i]);
   }
   for (i = N - 2; i >= 0; i--)
      for (k = 0; k < NQ; k++)
         for (j = 0; j < NQ; j++) f[i][k] -= c[i][k][j] * f[i + 1][j];
}

/* blockTridagPeriodic4, triSolvers.cpp:850-1046 */
static void block_tridag_periodic4(double (*a)[NQ][NQ], double (*b)[NQ][NQ], double (*c)[NQ][NQ], double (*f)[NQ], int N)
{
   int i, j, k, l;
   double t[NQ][NQ];
   lu4 u;
   for (i = 0; i < N; i++) {
      if (i != 0) {
         for (k = 0; k < NQ; k++)
            for (j = 0; j < NQ; j++)
               for (l = 0; l < NQ; l++) b[i][k][j] -= a[i][k][l] * c[i - 1][l][j];
         for (k = 0; k < NQ; k++)
            for (j = 0; j < NQ; j++) f[i][k] -= a[i][k][j] * f[i - 1][j];
         for (k = 0; k < NQ; k++)
            for (j = 0; j < NQ; j++) t[k][j] = 0;
         for (k = 0; k < NQ; k++)
            for (j = 0; j < NQ; j++)
               for (l = 0; l < NQ; l++) t[k][j] -= a[i][k][l] * a[i - 1][l][j];
         memcpy(a[i], t, sizeof(t));
      }
      u = lu_factor(b[i]);
      lu_solve(&u, &f[i][0], &f[i][1], &f[i][2], &f[i][3]);
      if (i != N - 2) {
         lu_solve_cols(&u, c[i]);
         lu_solve_cols(&u, a[i]);
      }
      if (i == N - 2) {
         for (k = 0; k < NQ; k++)
            for (j = 0; j < NQ; j++) c[i][j][k] += a[i][j][k];
         lu_solve_cols(&u, c[i]);
         memcpy(a[i], c[i], sizeof(t));
      }
   }
   i = N - 1;
   for (k = 0; k < NQ; k++)
      for (j = 0; j < NQ; j++) b[i][j][k] = (j == k) ? 1.0 : 0.0;
   for (i = 0; i < N - 1; i++) {
      for (k = 0; k < NQ; k++)
         for (j = 0; j < NQ; j++) t[k][j] = 0;
      for (k = 0; k < NQ; k++)
         for (j = 0; j < NQ; j++)
            for (l = 0; l < NQ; l++) {
               t[k][j] -= c[N - 1][k][l] * c[i][l][j];
               b[N - 1][k][j] -= c[N - 1][k][l] * a[i][l][j];
            }
      for (k = 0; k < NQ; k++)
         for (j = 0; j < NQ; j++) f[N - 1][k] -= c[N - 1][k][j] * f[i][j];
      memcpy(c[N - 1], t, sizeof(t));
   }
   u = lu_factor(b[N - 1]);
   lu_solve(&u, &f[N - 1][0], &f[N - 1][1], &f[N - 1][2], &f[N - 1][3]);
   if (N < 2) return; /* the reference indexes row -1 here for N == 1 */
   i = N - 2;
   for (k = 0; k < NQ; k++)
      for (j = 0; j < NQ; j++) f[i][k] -= (c[i][k][j] * f[i + 1][j]);
   for (i = N - 3; i >= 0; i--)
      for (k = 0; k < NQ; k++)
         for (j = 0; j < NQ; j++) f[i][k] -= (c[i][k][j] * f[i + 1][j] + a[i][k][j] * f[N - 1][j]);
}

int ho_block_tridag4(double* a, double* b, double* c, double* f, int N, int periodic)
{
   if (N < 1 || (periodic && N < 2)) return -1;
   if (periodic) block_tridag_periodic4((double(*)[NQ][NQ])a, (double(*)[NQ][NQ])b, (double(*)[NQ][NQ])c, (double(*)[NQ])f, N);
   else block_tridag4((double(*)[NQ][NQ])a, (double(*)[NQ][NQ])b, (double(*)[NQ][NQ])c, (double(*)[NQ])f, N);
   return 0;
}

/* ------------------------------------------------------------------ */
/* ADI (ADI.cpp:15-266)                                                */
/* ------------------------------------------------------------------ */

/* Extended rule: the end faces of open chains that lead into a cell of
   another chain.  Returned as a CSR over cells (the face's right cell),
   ascending face ids; NULL pointers when there are none. */
static void foreign_faces(const ho_case* c, int** ptr, int** ent)
{
   int i, n = 0;
   int* cnt = (int*)calloc((size_t)c->nCell + 1, sizeof(int));
   for (i = 0; i < c->nChain; i++) {
      int f1 = c->faceStart[i], f2 = c->faceStart[i + 1];
      int a = c->chainConn[f1], b = c->chainConn[f2 - 1];
      if (a == b) continue;
      if (c->faces[6 * a + 4] >= 0) { cnt[c->faces[6 * a + 4] + 1]++; n++; }
      if (c->faces[6 * b + 4] >= 0) { cnt[c->faces[6 * b + 4] + 1]++; n++; }
   }
   for (i = 0; i < c->nCell; i++) cnt[i + 1] += cnt[i];
   *ptr = cnt;
   *ent = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
   {
      int* fill = (int*)malloc(sizeof(int) * (size_t)(c->nCell + 1));
      int f;
      memcpy(fill, cnt, sizeof(int) * (size_t)(c->nCell + 1));
      /* ascending face ids: scan faces, keep chain-end faces */
      char* isend = (char*)calloc((size_t)c->nFace + 1, 1);
      for (i = 0; i < c->nChain; i++) {
         int f1 = c->faceStart[i], f2 = c->faceStart[i + 1];
         int a = c->chainConn[f1], b = c->chainConn[f2 - 1];
         if (a == b) continue;
         isend[a] = 1;
         isend[b] = 1;
      }
      for (f = 0; f < c->nFace; f++) {
         int r = c->faces[6 * f + 4];
         if (isend[f] && r >= 0) (*ent)[fill[r]++] = f;
      }
      free(isend);
      free(fill);
   }
}

int ho_adi(ho_case* c, double* l2, double* linf)
{
   int i, j, k, m, f, isweep, rc;
   int *xptr = NULL, *xent = NULL;
   if (c->end_rule == HO_END_RULE_EXTENDED) foreign_faces(c, &xptr, &xent);
   for (i = 0; i < c->nCell; i++) {
      double dtfac = c->CFL / c->sigma[i];
      for (m = 0; m < NQ; m++) {
         c->r[NQ * i + m] *= dtfac;
         c->r0[NQ * i + m] = c->r[NQ * i + m];
         c->dq[NQ * i + m] = 0.0;
      }
   }
   for (isweep = 0; isweep < c->msweep; isweep++) {
      for (i = 0; i < c->nChain; i++) {
         int f1 = c->faceStart[i], f2 = c->faceStart[i + 1];
         int per = (c->chainConn[f1] == c->chainConn[f2 - 1]);
         int size = f2 - per - f1;
         memset(c->A, 0, sizeof(*c->A) * c->work);
         memset(c->B, 0, sizeof(*c->B) * c->work);
         memset(c->C, 0, sizeof(*c->C) * c->work);
         memset(c->F, 0, sizeof(*c->F) * c->work);
         m = 0;
         for (f = f1; f < f2 - per; f++) {
            int iface = c->chainConn[f];
            int left = c->faces[6 * iface + 2], right = c->faces[6 * iface + 4];
            double L[NQ][NQ], R[NQ][NQ];
            int mm1;
            memcpy(L, c->ff + 32 * iface, sizeof(L));
            memcpy(R, c->ff + 32 * iface + 16, sizeof(R));
            if (per) {
               mm1 = (m == 0) ? size - 1 : m - 1;
               for (j = 0; j < NQ; j++) {
                  for (k = 0; k < NQ; k++) {
                     c->B[m][j][k] += L[j][k];
                     c->B[mm1][j][k] -= R[j][k];
                     c->A[m][j][k] += R[j][k];
                     c->C[mm1][j][k] -= L[j][k];
                  }
                  c->F[m][j] = c->r[NQ * left + j];
               }
            } else {
               mm1 = m - 1;
               if (right == BC_WALL) {
                  const double* rf = c->refMtx + 4 * iface;
                  for (j = 0; j < NQ; j++) {
                     double r01 = R[j][1], r02 = R[j][2];
                     R[j][1] = rf[0] * r01 + rf[1] * r02;
                     R[j][2] = rf[2] * r01 + rf[3] * r02;
                  }
               }
               /* extended rule: an interior last face couples explicitly,
                  like the far field (the reference indexes a row past the
                  chain there, ADI.cpp:166-181) */
               int ext_last = (c->end_rule == HO_END_RULE_EXTENDED && f == f2 - 1);
               if ((right < 0 || ext_last) && f == f2 - 1) m--;
               for (j = 0; j < NQ; j++) {
                  for (k = 0; k < NQ; k++) {
                     c->B[m][j][k] += L[j][k];
                     if (mm1 > -1 && right > -1 && !ext_last) {
                        c->A[m][j][k] += R[j][k];
                        c->B[mm1][j][k] -= R[j][k];
                        c->C[mm1][j][k] -= L[j][k];
                     } else if (right == BC_WALL) {
                        c->B[m][j][k] += R[j][k];
                     }
                  }
                  c->F[m][j] = c->r[NQ * left + j];
               }
            }
            m++;
         }
         size = size - (per == 0);
         /* extended rule: a cell's first chain also carries the diagonal
            term of every chain-end face that leads into it from another
            chain (its right-cell Jacobian), so each face's diagonal terms
            stay implicit; only the coupling across the end is lagged */
         if (xptr) {
            m = 0;
            for (f = f1; f < f2 - 1; f++) {
               int left = c->faces[6 * c->chainConn[f] + 2], e;
               if (c->c2chain[2 * left] == i) {
                  for (e = xptr[left]; e < xptr[left + 1]; e++) {
                     const double* R = c->ff + 32 * xent[e] + 16;
                     for (j = 0; j < NQ; j++)
                        for (k = 0; k < NQ; k++) c->B[m][j][k] -= R[4 * j + k];
                  }
               }
               m++;
            }
         }
         m = 0;
         for (f = f1; f < f2 - 1; f++) {
            int left = c->faces[6 * c->chainConn[f] + 2];
            double dtfac = c->CFL / c->sigma[left];
            for (j = 0; j < NQ; j++)
               for (k = 0; k < NQ; k++) {
                  c->A[m][j][k] *= dtfac;
                  c->B[m][j][k] *= dtfac;
                  c->C[m][j][k] *= dtfac;
               }
            for (j = 0; j < NQ; j++) c->B[m][j][j] += 1.0;
            m++;
         }
         if (per) block_tridag_periodic4(c->A, c->B, c->C, c->F, size);
         else block_tridag4(c->A, c->B, c->C, c->F, size);
         m = 0;
         for (f = f1; f < f2 - 1; f++) {
            int left = c->faces[6 * c->chainConn[f] + 2];
            for (j = 0; j < NQ; j++) c->r[NQ * left + j] = c->F[m][j];
            m++;
         }
      }
      for (i = 0; i < NQ * c->nCell; i++) c->dq[i] += c->r[i];
      rc = ho_linear_rhs(c, l2, linf);
      if (rc) { free(xptr); free(xent); return rc; }
   }
   free(xptr);
   free(xent);
   for (i = 0; i < NQ * c->nCell; i++) c->q[i] += c->dq[i];
   *l2 = c->L2Norm; *linf = c->LInfNorm;
   return 0;
}

/* ------------------------------------------------------------------ */
/* march (march.cpp:66-134, ADI branch :381-386)                       */
/* ------------------------------------------------------------------ */

int ho_step(ho_case* c, double* out4)
{
   int rc = ho_compute_rhs(c, 1, &out4[0], &out4[1]);
   if (rc) return rc;
   return ho_adi(c, &out4[2], &out4[3]);
}

/* updateSolution (march.cpp:411-433) */
static void update_solution(ho_case* c, const double* qold, double* qnew, double coef)
{
   int i, j, m = 0;
   for (i = 0; i < c->nCell; i++)
      for (j = 0; j < NQ; j++) {
         double dtfac = coef * c->CFL / c->sigma[i];
         qnew[m] = qold[m] + dtfac * c->r[m];
         m++;
      }
}

int ho_update_solution(ho_case* c, const char* qold, const char* qnew, double coef)
{
   double* s = !strcmp(qold, "q") ? c->q : !strcmp(qold, "qt") ? c->qt : NULL;
   double* d = !strcmp(qnew, "q") ? c->q : !strcmp(qnew, "qt") ? c->qt : NULL;
   if (!s || !d) return -1;
   update_solution(c, s, d, coef);
   return 0;
}

/* explicit branches of stepSolution (march.cpp:342-377) */
int ho_step_explicit(ho_case* c, int scheme, double* out2)
{
   int rc;
   if (scheme == 0) {
      if ((rc = ho_compute_rhs(c, 0, &out2[0], &out2[1]))) return rc;
      update_solution(c, c->q, c->q, 1.);
      return 0;
   }
   if ((rc = ho_compute_rhs(c, 0, &out2[0], &out2[1]))) return rc;
   update_solution(c, c->q, c->qt, 0.25);
   update_solution(c, c->q, c->q, 8.0 / 15);
   if ((rc = ho_compute_rhs(c, 0, &out2[0], &out2[1]))) return rc;
   update_solution(c, c->qt, c->q, 5.0 / 12);
   if ((rc = ho_compute_rhs(c, 0, &out2[0], &out2[1]))) return rc;
   update_solution(c, c->qt, c->q, 3.0 / 4.0);
   return 0;
}

int ho_march(ho_case* c, int n, double* hist)
{
   int i, rc;
   for (i = 0; i < n; i++)
      if ((rc = ho_step(c, hist + 4 * i)) != 0) return rc;
   return 0;
}

int ho_march_replicas(ho_case** cases, int n, int iters)
{
   int i, bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad)
   for (i = 0; i < n; i++) {
      int it;
      double out[4];
      for (it = 0; it < iters; it++)
         if (ho_step(cases[i], out) != 0) { bad++; break; }
   }
   return bad ? -1 : 0;
}

/* ------------------------------------------------------------------ */
/* handle                                                              */
/* ------------------------------------------------------------------ */

/* ------------------------------------------------------------------ */
/* wall forces (project addition; the reference has none)              */
/* ------------------------------------------------------------------ */

/* Pressure force on the wall faces (bFaces, preprocess.cpp:180-184, in
   ascending face order) from the adjacent cell's pressure, its moment
   about (0.25, 0), and the coefficients on a unit chord:
   out = {Fx, Fy, M, CL, CD, CM}. */
int ho_forces(const ho_case* c, double* out)
{
   double Fx = 0.0, Fy = 0.0, M = 0.0;
   double V2, qinf, V, ca, sa;
   int k;
   for (k = 0; k < c->nBface; k++) {
      int f = c->bFaces[k];
      const int* fr = c->faces + 6 * f;
      const double* s = c->q + NQ * fr[2];
      double p = c->gm1 * (s[3] - 0.5 * (s[1] * s[1] + s[2] * s[2]) / s[0]);
      double fx = p * c->normVec[2 * f];
      double fy = p * c->normVec[2 * f + 1];
      double xm = 0.5 * (c->x[2 * fr[0]] + c->x[2 * fr[1]]);
      double ym = 0.5 * (c->x[2 * fr[0] + 1] + c->x[2 * fr[1] + 1]);
      Fx = Fx + fx;
      Fy = Fy + fy;
      M = M + ((xm - 0.25) * fy - ym * fx);
   }
   V2 = c->uinf * c->uinf + c->vinf * c->vinf;
   qinf = 0.5 * c->rinf * V2;
   V = sqrt(V2);
   ca = c->uinf / V;
   sa = c->vinf / V;
   out[0] = Fx;
   out[1] = Fy;
   out[2] = M;
   out[3] = (Fy * ca - Fx * sa) / qinf;
   out[4] = (Fx * ca + Fy * sa) / qinf;
   out[5] = M / qinf;
   return 0;
}

ho_case* ho_open(const char* dir, char* err, int errlen)
{
   ho_case* c = (ho_case*)calloc(1, sizeof(ho_case));
   char dummy[8];
   if (!err) { err = dummy; errlen = sizeof(dummy); }
   if (rd_mesh(c, dir, err, errlen) || rd_inputs(c, dir, err, errlen)) { ho_close(c); return NULL; }
   alloc_solution(c);
   preprocess(c);
   init_flow(c);
   return c;
}

#define DUP(dst, src, n) do { (dst) = malloc(sizeof(*(src)) * (size_t)(n)); memcpy((dst), (src), sizeof(*(src)) * (size_t)(n)); } while (0)

ho_case* ho_clone(const ho_case* s)
{
   ho_case* c = (ho_case*)calloc(1, sizeof(ho_case));
   int nc = s->nCell > 0 ? s->nCell : 1, nf = s->nFace > 0 ? s->nFace : 1;
   *c = *s;
   DUP(c->x, s->x, 2 * (s->nNode > 0 ? s->nNode : 1));
   DUP(c->conn, s->conn, 4 * nc);
   DUP(c->chainsPerColor, s->chainsPerColor, s->nColor > 0 ? s->nColor : 1);
   DUP(c->faceStart, s->faceStart, s->nChain + 1);
   DUP(c->chainConn, s->chainConn, s->nChainFace > 0 ? s->nChainFace : 1);
   DUP(c->faces, s->faces, 6 * nf);
   DUP(c->bFaces, s->bFaces, nf);
   DUP(c->c2chain, s->c2chain, 2 * nc);
   DUP(c->vol, s->vol, nc);
   DUP(c->normVec, s->normVec, 2 * nf);
   DUP(c->refMtx, s->refMtx, 4 * nf);
   alloc_solution(c);
   memcpy(c->q, s->q, sizeof(double) * NQ * nc);
   memcpy(c->qt, s->qt, sizeof(double) * NQ * nc);
   memcpy(c->r, s->r, sizeof(double) * NQ * nc);
   memcpy(c->r0, s->r0, sizeof(double) * NQ * nc);
   memcpy(c->dq, s->dq, sizeof(double) * NQ * nc);
   memcpy(c->sigma, s->sigma, sizeof(double) * nc);
   memcpy(c->ff, s->ff, sizeof(double) * 32 * nf);
   return c;
}

void ho_close(ho_case* c)
{
   if (!c) return;
   free(c->x); free(c->conn); free(c->chainsPerColor); free(c->faceStart);
   free(c->chainConn); free(c->faces); free(c->bFaces); free(c->c2chain);
   free(c->vol); free(c->normVec); free(c->refMtx);
   free(c->q); free(c->qt); free(c->r); free(c->r0); free(c->dq); free(c->sigma); free(c->ff);
   free(c->cindx); free(c->f); free(c->df); free(c->ql); free(c->qr); free(c->f2);
   free(c->A); free(c->B); free(c->C); free(c->F);
   free(c);
}

void ho_sizes(const ho_case* c, int* out)
{
   out[0] = c->nCell; out[1] = c->nFace; out[2] = c->nChain; out[3] = c->nChainFace;
   out[4] = c->nMaxChain; out[5] = c->order; out[6] = c->msweep; out[7] = c->nGhost;
   out[8] = c->nNode; out[9] = c->nColor;
}

void ho_params(const ho_case* c, double* out)
{
   out[0] = c->Mach; out[1] = c->alpha; out[2] = c->CFL; out[3] = c->gamma; out[4] = c->rinf;
   out[5] = c->uinf; out[6] = c->vinf; out[7] = c->einf; out[8] = c->pinf;
}

void ho_set_freestream(ho_case* c, double uinf, double vinf, double einf)
{
   c->uinf = uinf; c->vinf = vinf; c->einf = einf;
}

int ho_set_option(ho_case* c, const char* name, int value)
{
   if (strcmp(name, "limiter") == 0) {
      if (value < HO_LIMITER_REFERENCE || value > HO_LIMITER_VANALBADA) return -1;
      c->limiter = value;
      return 0;
   }
   if (strcmp(name, "chain_end_rule") == 0) {
      if (value != HO_END_RULE_REFERENCE && value != HO_END_RULE_EXTENDED) return -1;
      c->end_rule = value;
      return 0;
   }
   if (strcmp(name, "sweep_order") == 0) {
      if (value != 0 && value != 1) return -1;
      c->sweep_order = value;
      return 0;
   }
   return -1;
}

void ho_set_run(ho_case* c, int order, int msweep, double cfl)
{
   c->order = order; c->msweep = msweep; c->CFL = cfl; c->nGhost = (order == 5) ? 3 : 2;
}

static double* darr(const ho_case* c, const char* name, size_t* n)
{
   if (!strcmp(name, "q"))     { *n = (size_t)NQ * c->nCell; return c->q; }
   if (!strcmp(name, "qt"))    { *n = (size_t)NQ * c->nCell; return c->qt; }
   if (!strcmp(name, "r"))     { *n = (size_t)NQ * c->nCell; return c->r; }
   if (!strcmp(name, "r0"))    { *n = (size_t)NQ * c->nCell; return c->r0; }
   if (!strcmp(name, "dq"))    { *n = (size_t)NQ * c->nCell; return c->dq; }
   if (!strcmp(name, "sigma")) { *n = (size_t)c->nCell; return c->sigma; }
   if (!strcmp(name, "ff"))    { *n = (size_t)32 * c->nFace; return c->ff; }
   if (!strcmp(name, "x"))     { *n = (size_t)2 * c->nNode; return c->x; }
   if (!strcmp(name, "vol"))   { *n = (size_t)c->nCell; return c->vol; }
   if (!strcmp(name, "normVec")) { *n = (size_t)2 * c->nFace; return c->normVec; }
   if (!strcmp(name, "refMtx"))  { *n = (size_t)4 * c->nFace; return c->refMtx; }
   return NULL;
}

int ho_get(const ho_case* c, const char* name, double* out)
{
   size_t n = 0;
   double* p = darr(c, name, &n);
   if (!p) return -1;
   memcpy(out, p, n * sizeof(double));
   return 0;
}

int ho_set(ho_case* c, const char* name, const double* in)
{
   size_t n = 0;
   double* p = darr(c, name, &n);
   if (!p) return -1;
   memcpy(p, in, n * sizeof(double));
   return 0;
}

int ho_get_int(const ho_case* c, const char* name, int* out)
{
   if (!strcmp(name, "faces")) { memcpy(out, c->faces, sizeof(int) * 6 * c->nFace); return 0; }
   if (!strcmp(name, "chainConn")) { memcpy(out, c->chainConn, sizeof(int) * c->nChainFace); return 0; }
   if (!strcmp(name, "faceStartPerChain")) { memcpy(out, c->faceStart, sizeof(int) * (c->nChain + 1)); return 0; }
   if (!strcmp(name, "c2chain")) { memcpy(out, c->c2chain, sizeof(int) * 2 * c->nCell); return 0; }
   if (!strcmp(name, "bFaces")) { memcpy(out, c->bFaces, sizeof(int) * c->nBface); return c->nBface; }
   if (!strcmp(name, "chainsPerColor")) { memcpy(out, c->chainsPerColor, sizeof(int) * c->nColor); return 0; }
   return -1;
}
