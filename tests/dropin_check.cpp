// Test driver of the drop-in C++ functions (test infrastructure): calls
// SOLVER::fluxRoe2D / jacobianRoe2D, RECONSTRUCTION::* and
// TRISOLVER::blockTridag4 / blockTridagPeriodic4 of the library with the
// reference's pointer-array signatures on inputs read from a file, and
// writes their results for tests/test_gpu_host_dropin.py to compare with
// the oracle.
//
//   dropin_check <in> <out>
//
// in:  doubles nf, nl, imax, nq, N; then nxy[nf][2], ql[nf][4], qr[nf][4];
//      f, dq, ql0, qr0, f20 [nl][imax][nq]; a, b, c [N][4][4], rhs [N][4]
// out: flux[nf][4], spec[nf], lmat[nf][16], rmat[nf][16]; for each of the
//      five reconstruction calls below and each line, ql, qr, f2
//      [imax][nq]; the open and the periodic solution [N][4]; then 1.0 if
//      a NaN spectral radius threw hamstr::Error with HAMSTR_GPU_ERR_NAN.
#include <cstdio>
#include <cstring>
#include <vector>

#include "hamstr_host.h"

namespace {
std::vector<double> rd;
size_t pos = 0;
double take() { return rd.at(pos++); }
void takev(double* p, size_t n)
{
   for (size_t i = 0; i < n; i++) p[i] = take();
}
std::vector<double*> rows(double* p, int n, int w)
{
   std::vector<double*> v(n);
   for (int i = 0; i < n; i++) v[i] = p + (size_t)i * w;
   return v;
}
}  // namespace

int main(int argc, char** argv)
{
   if (argc != 3) return 2;
   FILE* fi = std::fopen(argv[1], "rb");
   if (!fi) return 2;
   double x;
   while (std::fread(&x, sizeof(double), 1, fi) == 1) rd.push_back(x);
   std::fclose(fi);
   const int nf = (int)take(), nl = (int)take(), imax = (int)take(), nq = (int)take(), N = (int)take();
   std::vector<double> nxy(2 * nf), ql(4 * nf), qr(4 * nf);
   takev(nxy.data(), nxy.size());
   takev(ql.data(), ql.size());
   takev(qr.data(), qr.size());
   const size_t ln = (size_t)imax * nq;
   std::vector<double> f(nl * ln), dq(nl * ln), ql0(nl * ln), qr0(nl * ln), f20(nl * ln);
   for (auto* v : {&f, &dq, &ql0, &qr0, &f20}) takev(v->data(), v->size());
   std::vector<double> a(16 * N), b(16 * N), c(16 * N), rhs(4 * N);
   for (auto* v : {&a, &b, &c, &rhs}) takev(v->data(), v->size());

   std::vector<double> out;
   auto put = [&](const double* p, size_t n) { out.insert(out.end(), p, p + n); };

   // a solver object for the per-face methods (they use no mesh data)
   MESHBLOCK mb;
   SOLNBLOCK sb;
   SOLVER solver(&mb, &sb);
   std::vector<double> flux(4 * nf), spec(nf), lm(16 * nf), rm(16 * nf);
   for (int k = 0; k < nf; k++) {
      solver.fluxRoe2D(&nxy[2 * k], &ql[4 * k], &qr[4 * k], &flux[4 * k], &spec[k], 1.4);
      double* L[4] = {&lm[16 * k], &lm[16 * k + 4], &lm[16 * k + 8], &lm[16 * k + 12]};
      double* R[4] = {&rm[16 * k], &rm[16 * k + 4], &rm[16 * k + 8], &rm[16 * k + 12]};
      solver.jacobianRoe2D(&nxy[2 * k], &ql[4 * k], &qr[4 * k], L, R, 1.4);
   }
   put(flux.data(), flux.size());
   put(spec.data(), spec.size());
   put(lm.data(), lm.size());
   put(rm.data(), rm.size());

   for (int call = 0; call < 5; call++) {
      for (int l = 0; l < nl; l++) {
         std::vector<double> fl(f.begin() + l * ln, f.begin() + (l + 1) * ln);
         std::vector<double> dl(dq.begin() + l * ln, dq.begin() + (l + 1) * ln);
         std::vector<double> qlv(ql0.begin() + l * ln, ql0.begin() + (l + 1) * ln);
         std::vector<double> qrv(qr0.begin() + l * ln, qr0.begin() + (l + 1) * ln);
         std::vector<double> f2v(f20.begin() + l * ln, f20.begin() + (l + 1) * ln);
         auto F = rows(fl.data(), imax, nq), D = rows(dl.data(), imax, nq), QL = rows(qlv.data(), imax, nq);
         auto QR = rows(qrv.data(), imax, nq), F2 = rows(f2v.data(), imax, nq);
         switch (call) {
            case 0: RECONSTRUCTION::MUSCL(F.data(), QL.data(), QR.data(), F2.data(), 1, imax - 2, 1. / 3., 0.25, 1e-10,
                                          imax, nq); break;
            case 1: RECONSTRUCTION::MUSCL(F.data(), QL.data(), QR.data(), F2.data(), 2, imax - 1, 1. / 3., 0.25, 1e-10,
                                          imax, nq); break;
            case 2: RECONSTRUCTION::MUSCL_DERIV(F.data(), QL.data(), QR.data(), F2.data(), D.data(), 1, imax - 2,
                                                1. / 3., 0.25, 1e-10, imax, nq); break;
            case 3: RECONSTRUCTION::WENO(F.data(), QL.data(), QR.data(), 2, imax - 1, 1e-10, imax, nq); break;
            default: RECONSTRUCTION::WENO_DERIV(F.data(), QL.data(), QR.data(), D.data(), 2, imax - 1, 1e-10, imax, nq);
         }
         put(qlv.data(), ln);
         put(qrv.data(), ln);
         put(f2v.data(), ln);
      }
   }

   for (int per = 0; per < 2; per++) {
      std::vector<double> fa(a), fb(b), fc(c), fr(rhs);
      std::vector<double**> A(N), B(N), C(N);
      std::vector<std::vector<double*>> keep;
      for (int i = 0; i < N; i++) {
         keep.push_back(rows(&fa[16 * i], 4, 4));
         A[i] = keep.back().data();
         keep.push_back(rows(&fb[16 * i], 4, 4));
         B[i] = keep.back().data();
         keep.push_back(rows(&fc[16 * i], 4, 4));
         C[i] = keep.back().data();
      }
      auto Fr = rows(fr.data(), N, 4);
      if (per) TRISOLVER::blockTridagPeriodic4(A.data(), B.data(), C.data(), Fr.data(), N, 4);
      else TRISOLVER::blockTridag4(A.data(), B.data(), C.data(), Fr.data(), N, 4);
      put(fr.data(), fr.size());
   }

   double threw = 0.0;
   {
      double s[2] = {0.3, -0.1}, L[4] = {1.0, 0.1, 0.0, -5.0}, R[4] = {1.0, 0.1, 0.0, 2.5}, fl[4], sp = 0;
      try {
         solver.fluxRoe2D(s, L, R, fl, &sp, 1.4);
      } catch (const hamstr::Error& e) {
         threw = (e.status == HAMSTR_GPU_ERR_NAN) ? 1.0 : 0.0;
      }
   }
   put(&threw, 1);

   FILE* fo = std::fopen(argv[2], "wb");
   if (!fo) return 2;
   std::fwrite(out.data(), sizeof(double), out.size(), fo);
   std::fclose(fo);
   return 0;
}
