// ##################################################################
//
// roe.cuh -- Roe flux and its frozen-eigenvalue Jacobian, per face
//
// Compiled with -fmad=false: every a*b+c below rounds the product and the
// sum separately, the arithmetic of the reference on x86-64, and divisions
// and sqrt are the IEEE correctly rounded operations (the FP64 divisions
// of roe_face run on the integer pipes, softdiv.cuh, with the same
// results).  Expressions keep the reference's association order so the
// results are bit-identical.
//
// Flux: fluxRoe2D, interfaceFlux.cpp:24-169.
// Jacobian: jacobianRoe2D -> jacobianRoe3D with IMODE=1
// (jacobianRoe.cpp:9-70, 92-337, 488-620).  The reference embeds the 2D
// state in 5 variables with w=0 and nz=0 and keeps rows/columns {0,1,2,4}.
// Every term it forms from w, nz or a structurally zero derivative is an
// exact zero (x*0 or 0*x with finite x) added to a non-zero partial sum,
// which leaves the sum unchanged, so those terms are dropped here and only
// the 32 kept entries are formed.  The flux and the Jacobian share the
// primitive states and Roe averages, which the reference computes twice
// with identical expressions.  The Jacobian's unit normal is nxd/area
// (jacobianRoe.cpp:164) while the flux's is nxd*(1/area)
// (interfaceFlux.cpp:62-65); both are formed.
// ##################################################################
#ifndef HAMSTR_GPU_ROE_CUH
#define HAMSTR_GPU_ROE_CUH

#include "softdiv.cuh"

namespace hamstr {

struct RoeOut {
   double flux[4];
   double spec;
};

// lm/rm receive the 4x4 left/right Jacobians (row-major) times the area.
// Returns false when the spectral radius is NaN.
template <bool JAC, bool SD = true>
__device__ __forceinline__ bool roe_face(double nxd, double nyd, const double (&ql)[4],
                                         const double (&qr)[4], double gam, RoeOut& o,
                                         double* __restrict__ lm, double* __restrict__ rm)
{
   const double gm1 = gam - 1.0;
   const double area = sqrt(nxd * nxd + nyd * nyd);
   const Dv<double, SD> by_area(area);
   const double invArea = by_area.div(1.);
   const double nx = nxd * invArea;
   const double ny = nyd * invArea;

   const double rol = ql[0];
   const Dv<double, SD> by_rol(rol);
   const double ul = by_rol.div(ql[1]);
   const double vl = by_rol.div(ql[2]);
   const double pl = gm1 * (ql[3] - p2<-1, SD>(rol) * (ul * ul + vl * vl));
   const double hl = by_rol.div(ql[3] + pl);
   const double ror = qr[0];
   const Dv<double, SD> by_ror(ror);
   const double ur = by_ror.div(qr[1]);
   const double vr = by_ror.div(qr[2]);
   const double pr = gm1 * (qr[3] - p2<-1, SD>(ror) * (ur * ur + vr * vr));
   const double hr = by_ror.div(qr[3] + pr);
   const double dp = pr - pl;
   const double uconr = ur * nx + vr * ny;
   const double uconl = ul * nx + vl * ny;

   const double fact = sqrt(by_rol.div(ror));
   const Dv<double, SD> by_1f(1.0 + fact);
   const double A = by_1f.div(1.0);
   const double B = by_1f.div(fact);
   const double robar = rol * fact;
   const double ubar = ul * A + ur * B;
   const double vbar = vl * A + vr * B;
   const double hbar = hl * A + hr * B;
   double cbar = gm1 * (hbar - p2<-1, SD>(ubar * ubar + vbar * vbar));
   cbar = sqrt(cbar);
   const Dv<double, SD> by_c(cbar);
   const double uconbar = ubar * nx + vbar * ny;

   {
      const double eig1 = fabs(uconbar);
      const double eig2 = fabs(uconbar + cbar);
      const double eig3 = fabs(uconbar - cbar);
      double spec = eig1 + cbar;
      if (spec != spec) return false;
      const double term1 = -eig1 + p2<-1, SD>(eig2 + eig3);
      const double term2 = p2<-1, SD>(eig2 - eig3);
      const double del1 = by_c.div(by_c.div(term1 * dp)) + by_c.div(term2 * robar * (uconr - uconl));
      const double del2 = term1 * (uconr - uconl) * robar + by_c.div(term2 * dp);
      double fm0 = eig1 * (qr[0] - ql[0]);
      double fm1 = eig1 * (qr[1] - ql[1]);
      double fm2 = eig1 * (qr[2] - ql[2]);
      double fm3 = eig1 * (qr[3] - ql[3]);
      fm0 = fm0 + del1;
      fm1 = fm1 + del1 * ubar + del2 * nx;
      fm2 = fm2 + del1 * vbar + del2 * ny;
      fm3 = fm3 + del1 * hbar + del2 * uconbar;
      const double fl0 = rol * uconl, fr0 = ror * uconr;
      const double fl1 = rol * uconl * ul + nx * pl, fr1 = ror * uconr * ur + nx * pr;
      const double fl2 = rol * uconl * vl + ny * pl, fr2 = ror * uconr * vr + ny * pr;
      const double fl3 = (ql[3] + pl) * uconl, fr3 = (qr[3] + pr) * uconr;
      o.flux[0] = p2<-1, SD>(fl0 + fr0 - fm0);
      o.flux[1] = p2<-1, SD>(fl1 + fr1 - fm1);
      o.flux[2] = p2<-1, SD>(fl2 + fr2 - fm2);
      o.flux[3] = p2<-1, SD>(fl3 + fr3 - fm3);
      o.flux[0] *= area;
      o.flux[1] *= area;
      o.flux[2] *= area;
      o.flux[3] *= area;
      spec *= area;
      o.spec = spec;
   }
   if (!JAC) return true;

   // ---------------- Jacobian (jacobianRoe3D, IMODE=1) ----------------
   const double nxj = by_area.div(nxd);
   const double nyj = by_area.div(nyd);
   const double uconlj = ul * nxj + vl * nyj;
   const double uconrj = ur * nxj + vr * nyj;
   const double uconbarj = ubar * nxj + vbar * nyj;
   const double e1 = fabs(uconbarj);
   const double e2 = fabs(uconbarj + cbar);
   const double e3 = fabs(uconbarj - cbar);
   const double t1 = -e1 + p2<-1, SD>(e2 + e3);
   const double t2 = p2<-1, SD>(e2 - e3);
   const double t2rb = t2 * robar;

   // derivative vectors, kept components {rho, rho u, rho v, E}
   // left (jacobianRoe.cpp:209-250)
   const double du0l = by_rol.div(-ul);
   const double irl = by_rol.div(1.0);
   const double dv0l = by_rol.div(-vl);
   const double dp0l = p2<-1, SD>(gm1) * (ul * ul + vl * vl);
   const double dp1l = -gm1 * ul;
   const double dp2l = -gm1 * vl;
   const double dc0l = by_rol.div(-uconlj);
   const double dc1l = by_rol.div(nxj);
   const double dc2l = by_rol.div(nyj);
   // right (jacobianRoe.cpp:257-296)
   const double du0r = by_ror.div(-ur);
   const double irr = by_ror.div(1.0);
   const double dv0r = by_ror.div(-vr);
   const double dp0r = p2<-1, SD>(gm1) * (ur * ur + vr * vr);
   const double dp1r = -gm1 * ur;
   const double dp2r = -gm1 * vr;
   const double dc0r = by_ror.div(-uconrj);
   const double dc1r = by_ror.div(nxj);
   const double dc2r = by_ror.div(nyj);

   // frozen-eigenvalue linearisation of del1/del2 (jacobianRoe.cpp:323-334)
   const double mt1 = -t1;
   double D1l[4], D2l[4], D1r[4], D2r[4];
   D1l[0] = by_c.div(by_c.div(mt1 * dp0l)) - by_c.div(t2rb * dc0l);
   D1l[1] = by_c.div(by_c.div(mt1 * dp1l)) - by_c.div(t2rb * dc1l);
   D1l[2] = by_c.div(by_c.div(mt1 * dp2l)) - by_c.div(t2rb * dc2l);
   D1l[3] = by_c.div(by_c.div(mt1 * gm1));
   D2l[0] = mt1 * dc0l * robar - by_c.div(t2 * dp0l);
   D2l[1] = mt1 * dc1l * robar - by_c.div(t2 * dp1l);
   D2l[2] = mt1 * dc2l * robar - by_c.div(t2 * dp2l);
   D2l[3] = -by_c.div(t2 * gm1);
   D1r[0] = by_c.div(by_c.div(t1 * dp0r)) + by_c.div(t2rb * dc0r);
   D1r[1] = by_c.div(by_c.div(t1 * dp1r)) + by_c.div(t2rb * dc1r);
   D1r[2] = by_c.div(by_c.div(t1 * dp2r)) + by_c.div(t2rb * dc2r);
   D1r[3] = by_c.div(by_c.div(t1 * gm1));
   D2r[0] = t1 * dc0r * robar + by_c.div(t2 * dp0r);
   D2r[1] = t1 * dc1r * robar + by_c.div(t2 * dp1r);
   D2r[2] = t1 * dc2r * robar + by_c.div(t2 * dp2r);
   D2r[3] = by_c.div(t2 * gm1);

   // native flux Jacobians (jacobianRoe.cpp:573-605), kept rows/columns
   const double el = ql[3] + pl, er = qr[3] + pr;
   const double rcl = rol * uconlj, rcr = ror * uconrj;
   double L1[16], R1[16];
   L1[0] = uconlj + rol * dc0l;
   L1[1] = rol * dc1l;
   L1[2] = rol * dc2l;
   L1[3] = 0.0;
   L1[4] = uconlj * ul + rol * dc0l * ul + rcl * du0l + nxj * dp0l;
   L1[5] = rol * dc1l * ul + rcl * irl + nxj * dp1l;
   L1[6] = rol * dc2l * ul + nxj * dp2l;
   L1[7] = nxj * gm1;
   L1[8] = uconlj * vl + rol * dc0l * vl + rcl * dv0l + nyj * dp0l;
   L1[9] = rol * dc1l * vl + nyj * dp1l;
   L1[10] = rol * dc2l * vl + rcl * irl + nyj * dp2l;
   L1[11] = nyj * gm1;
   L1[12] = dp0l * uconlj + el * dc0l;
   L1[13] = dp1l * uconlj + el * dc1l;
   L1[14] = dp2l * uconlj + el * dc2l;
   L1[15] = (1.0 + gm1) * uconlj;
   R1[0] = uconrj + ror * dc0r;
   R1[1] = ror * dc1r;
   R1[2] = ror * dc2r;
   R1[3] = 0.0;
   R1[4] = uconrj * ur + ror * dc0r * ur + rcr * du0r + nxj * dp0r;
   R1[5] = ror * dc1r * ur + rcr * irr + nxj * dp1r;
   R1[6] = ror * dc2r * ur + nxj * dp2r;
   R1[7] = nxj * gm1;
   R1[8] = uconrj * vr + ror * dc0r * vr + rcr * dv0r + nyj * dp0r;
   R1[9] = ror * dc1r * vr + nyj * dp1r;
   R1[10] = ror * dc2r * vr + rcr * irr + nyj * dp2r;
   R1[11] = nyj * gm1;
   R1[12] = dp0r * uconrj + er * dc0r;
   R1[13] = dp1r * uconrj + er * dc1r;
   R1[14] = dp2r * uconrj + er * dc2r;
   R1[15] = (1.0 + gm1) * uconrj;

   // dissipation part (jacobianRoe.cpp:500-521) and the final
   // 0.5*(native - dissipation) times area (jacobianRoe.cpp:611-618, :63-68)
   const double rowc[4] = {0.0, ubar, vbar, hbar};
   const double rown[4] = {0.0, nxj, nyj, uconbarj};
#pragma unroll
   for (int rI = 0; rI < 4; rI++) {
#pragma unroll
      for (int c = 0; c < 4; c++) {
         double ml, mr;
         if (rI == 0) {
            ml = (c == 0) ? (-e1 + D1l[0]) : D1l[c];
            mr = (c == 0) ? (e1 + D1r[0]) : D1r[c];
         } else {
            if (c == rI) {
               ml = -e1 + D1l[c] * rowc[rI] + D2l[c] * rown[rI];
               mr = e1 + D1r[c] * rowc[rI] + D2r[c] * rown[rI];
            } else {
               ml = D1l[c] * rowc[rI] + D2l[c] * rown[rI];
               mr = D1r[c] * rowc[rI] + D2r[c] * rown[rI];
            }
         }
         lm[4 * rI + c] = p2<-1, SD>(L1[4 * rI + c] - ml) * area;
         rm[4 * rI + c] = p2<-1, SD>(R1[4 * rI + c] - mr) * area;
      }
   }
   return true;
}

// The same frozen-eigenvalue Jacobian evaluated entirely in T (used with
// T = float by the mixed-precision defect correction, where the Jacobian is
// only the approximate operator; the FP64 path uses roe_face<true>).
template <typename T>
__device__ __forceinline__ void roe_jacobian_only(T nxd, T nyd, const T (&ql)[4], const T (&qr)[4], T gam,
                                                  T* __restrict__ lm, T* __restrict__ rm)
{
   const T gm1 = gam - T(1);
   const T area = sqrt(nxd * nxd + nyd * nyd);
   const T rol = ql[0], ul = ql[1] / ql[0], vl = ql[2] / ql[0];
   const T pl = gm1 * (ql[3] - T(0.5) * rol * (ul * ul + vl * vl));
   const T hl = (ql[3] + pl) / rol;
   const T ror = qr[0], ur = qr[1] / qr[0], vr = qr[2] / qr[0];
   const T pr = gm1 * (qr[3] - T(0.5) * ror * (ur * ur + vr * vr));
   const T hr = (qr[3] + pr) / ror;
   const T fact = sqrt(ror / rol);
   const T A = T(1) / (T(1) + fact), B = fact / (T(1) + fact);
   const T robar = rol * fact;
   const T ubar = ul * A + ur * B, vbar = vl * A + vr * B, hbar = hl * A + hr * B;
   const T cbar = sqrt(gm1 * (hbar - T(0.5) * (ubar * ubar + vbar * vbar)));
   const T nxj = nxd / area, nyj = nyd / area;
   const T uconlj = ul * nxj + vl * nyj, uconrj = ur * nxj + vr * nyj;
   const T uconbarj = ubar * nxj + vbar * nyj;
   const T e1 = fabs(uconbarj), e2 = fabs(uconbarj + cbar), e3 = fabs(uconbarj - cbar);
   const T t1 = -e1 + T(0.5) * (e2 + e3), t2 = T(0.5) * (e2 - e3), t2rb = t2 * robar;
   const T irl = T(1) / rol, irr = T(1) / ror;
   const T du0l = -ul / rol, dv0l = -vl / rol, du0r = -ur / ror, dv0r = -vr / ror;
   const T dp0l = T(0.5) * gm1 * (ul * ul + vl * vl), dp1l = -gm1 * ul, dp2l = -gm1 * vl;
   const T dp0r = T(0.5) * gm1 * (ur * ur + vr * vr), dp1r = -gm1 * ur, dp2r = -gm1 * vr;
   const T dc0l = -uconlj / rol, dc1l = nxj / rol, dc2l = nyj / rol;
   const T dc0r = -uconrj / ror, dc1r = nxj / ror, dc2r = nyj / ror;
   const T mt1 = -t1;
   T D1l[4], D2l[4], D1r[4], D2r[4];
   D1l[0] = mt1 * dp0l / cbar / cbar - t2rb * dc0l / cbar;
   D1l[1] = mt1 * dp1l / cbar / cbar - t2rb * dc1l / cbar;
   D1l[2] = mt1 * dp2l / cbar / cbar - t2rb * dc2l / cbar;
   D1l[3] = mt1 * gm1 / cbar / cbar;
   D2l[0] = mt1 * dc0l * robar - t2 * dp0l / cbar;
   D2l[1] = mt1 * dc1l * robar - t2 * dp1l / cbar;
   D2l[2] = mt1 * dc2l * robar - t2 * dp2l / cbar;
   D2l[3] = -(t2 * gm1 / cbar);
   D1r[0] = t1 * dp0r / cbar / cbar + t2rb * dc0r / cbar;
   D1r[1] = t1 * dp1r / cbar / cbar + t2rb * dc1r / cbar;
   D1r[2] = t1 * dp2r / cbar / cbar + t2rb * dc2r / cbar;
   D1r[3] = t1 * gm1 / cbar / cbar;
   D2r[0] = t1 * dc0r * robar + t2 * dp0r / cbar;
   D2r[1] = t1 * dc1r * robar + t2 * dp1r / cbar;
   D2r[2] = t1 * dc2r * robar + t2 * dp2r / cbar;
   D2r[3] = t2 * gm1 / cbar;
   const T el = ql[3] + pl, er = qr[3] + pr;
   const T rcl = rol * uconlj, rcr = ror * uconrj;
   T L1[16], R1[16];
   L1[0] = uconlj + rol * dc0l;  L1[1] = rol * dc1l;  L1[2] = rol * dc2l;  L1[3] = T(0);
   L1[4] = uconlj * ul + rol * dc0l * ul + rcl * du0l + nxj * dp0l;
   L1[5] = rol * dc1l * ul + rcl * irl + nxj * dp1l;
   L1[6] = rol * dc2l * ul + nxj * dp2l;
   L1[7] = nxj * gm1;
   L1[8] = uconlj * vl + rol * dc0l * vl + rcl * dv0l + nyj * dp0l;
   L1[9] = rol * dc1l * vl + nyj * dp1l;
   L1[10] = rol * dc2l * vl + rcl * irl + nyj * dp2l;
   L1[11] = nyj * gm1;
   L1[12] = dp0l * uconlj + el * dc0l;  L1[13] = dp1l * uconlj + el * dc1l;
   L1[14] = dp2l * uconlj + el * dc2l;  L1[15] = (T(1) + gm1) * uconlj;
   R1[0] = uconrj + ror * dc0r;  R1[1] = ror * dc1r;  R1[2] = ror * dc2r;  R1[3] = T(0);
   R1[4] = uconrj * ur + ror * dc0r * ur + rcr * du0r + nxj * dp0r;
   R1[5] = ror * dc1r * ur + rcr * irr + nxj * dp1r;
   R1[6] = ror * dc2r * ur + nxj * dp2r;
   R1[7] = nxj * gm1;
   R1[8] = uconrj * vr + ror * dc0r * vr + rcr * dv0r + nyj * dp0r;
   R1[9] = ror * dc1r * vr + nyj * dp1r;
   R1[10] = ror * dc2r * vr + rcr * irr + nyj * dp2r;
   R1[11] = nyj * gm1;
   R1[12] = dp0r * uconrj + er * dc0r;  R1[13] = dp1r * uconrj + er * dc1r;
   R1[14] = dp2r * uconrj + er * dc2r;  R1[15] = (T(1) + gm1) * uconrj;
   const T rowc[4] = {T(0), ubar, vbar, hbar};
   const T rown[4] = {T(0), nxj, nyj, uconbarj};
#pragma unroll
   for (int rI = 0; rI < 4; rI++) {
#pragma unroll
      for (int c = 0; c < 4; c++) {
         T ml, mr;
         if (rI == 0) {
            ml = (c == 0) ? (-e1 + D1l[0]) : D1l[c];
            mr = (c == 0) ? (e1 + D1r[0]) : D1r[c];
         } else if (c == rI) {
            ml = -e1 + D1l[c] * rowc[rI] + D2l[c] * rown[rI];
            mr = e1 + D1r[c] * rowc[rI] + D2r[c] * rown[rI];
         } else {
            ml = D1l[c] * rowc[rI] + D2l[c] * rown[rI];
            mr = D1r[c] * rowc[rI] + D2r[c] * rown[rI];
         }
         lm[4 * rI + c] = T(0.5) * (L1[4 * rI + c] - ml) * area;
         rm[4 * rI + c] = T(0.5) * (R1[4 * rI + c] - mr) * area;
      }
   }
}

}  // namespace hamstr
#endif
