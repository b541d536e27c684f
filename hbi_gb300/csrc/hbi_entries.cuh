// hbi_entries.cuh -- FP64 device Green's functions: traction rate at receiver
// i from unit slip rate on source element j.  These are compiled into the
// assembly kernels (no callback), replacing HACApK_entry_ij
// (m_HACApK_calc_entry_ij.f90:24-90) for the problems on the hot path:
//   '2dvs'  antiplane half space, matels2dpa_ij            (:685-695)
//   '3dph'  Okada (1992) half space, okada_ij              (:1065-1145, okada.f90)
//   '3dnr'  Okada (1992) full space
//   '3dnt'  Nikkhoo & Walter triangular dislocation, FS    (:802-851, TDstressFS.f90)
//   '2dph'  2D edge dislocations in a half space (also '2dnh'), matel2dph2_ij (:92-166)
//   '2dn'   2D plane strain, full space, tensor2d_ij       (:300-339, :697-722)
//   '3dht'  Nikkhoo & Walter triangular dislocation, HS    (:852-898, TDstressFS.f90:7-44, 236-293, 405-1011)
//
// Differences from a literal transcription, all exact:
//  * only displacement *gradients* are formed; the displacement-only terms of
//    Okada's ua/ub/uc (theta, log(R+xi), log(R+eta), I1..I4) never reach the
//    stress and are skipped, so the Okada strain needs no atan/log at all;
//  * the geometric constants shared by ua/ub/uc at one corner are computed once;
//  * per-source trigonometry (strike, dip, rake) comes from tables filled once
//    per geometry (hbi_bemv_dev::cang etc.).
#pragma once
#include <cuda_runtime.h>

namespace hbi {

enum { P_2DVS = 1, P_3DPH = 2, P_3DNR = 3, P_3DNT = 4, P_2DPH = 5, P_2DN = 6, P_3DHT = 7 };

struct DevBemv {
  int problem, n;
  int normal;  // v == 'n'
  double w;
  const double *xcol, *ycol, *zcol, *xel, *xer;
  const double *ang, *angd, *dsl, *dsd, *rake;
  const double *xs1, *xs2, *xs3, *ys1, *ys2, *ys3, *zs1, *zs2, *zs3;
  const double *ev11, *ev12, *ev13, *ev21, *ev22, *ev23, *ev31, *ev32, *ev33;
  const double *yel, *yer;
  // per-element tables (length n)
  const double *cang, *sang, *crake, *srake, *cangd, *sangd, *dipdeg;
  const double *cang2, *sang2;  // cos, sin of 2 ang (2D problems)
};

#define HBI_PI 3.141592653589793238462643383279502884

// T2 = A^T T1 A for a symmetric tensor (Txx,Tyy,Tzz,Txy,Txz,Tyz); A[r][c]
__device__ __forceinline__ void tens_trans_d(const double* T, const double A[3][3], double* o) {
  const double Txx = T[0], Tyy = T[1], Tzz = T[2], Txy = T[3], Txz = T[4], Tyz = T[5];
#define a(r, c) A[(r)-1][(c)-1]
  o[0] = a(1,1)*a(1,1)*Txx + 2*a(1,1)*a(2,1)*Txy + 2*a(1,1)*a(3,1)*Txz + 2*a(2,1)*a(3,1)*Tyz + a(2,1)*a(2,1)*Tyy + a(3,1)*a(3,1)*Tzz;
  o[1] = a(1,2)*a(1,2)*Txx + 2*a(1,2)*a(2,2)*Txy + 2*a(1,2)*a(3,2)*Txz + 2*a(2,2)*a(3,2)*Tyz + a(2,2)*a(2,2)*Tyy + a(3,2)*a(3,2)*Tzz;
  o[2] = a(1,3)*a(1,3)*Txx + 2*a(1,3)*a(2,3)*Txy + 2*a(1,3)*a(3,3)*Txz + 2*a(2,3)*a(3,3)*Tyz + a(2,3)*a(2,3)*Tyy + a(3,3)*a(3,3)*Tzz;
  o[3] = a(1,1)*a(1,2)*Txx + (a(1,1)*a(2,2) + a(2,1)*a(1,2))*Txy + (a(1,1)*a(3,2) + a(1,2)*a(3,1))*Txz + (a(3,2)*a(2,1) + a(3,1)*a(2,2))*Tyz + a(2,2)*a(2,1)*Tyy + a(3,1)*a(3,2)*Tzz;
  o[4] = a(1,1)*a(1,3)*Txx + (a(1,1)*a(2,3) + a(1,3)*a(2,1))*Txy + (a(1,1)*a(3,3) + a(3,1)*a(1,3))*Txz + (a(3,3)*a(2,1) + a(3,1)*a(2,3))*Tyz + a(2,3)*a(2,1)*Tyy + a(3,1)*a(3,3)*Tzz;
  o[5] = a(1,2)*a(1,3)*Txx + (a(1,3)*a(2,2) + a(1,2)*a(2,3))*Txy + (a(1,3)*a(3,2) + a(1,2)*a(3,3))*Txz + (a(2,3)*a(3,2) + a(3,3)*a(2,2))*Tyz + a(2,2)*a(2,3)*Tyy + a(3,2)*a(3,3)*Tzz;
#undef a
}

// ------------------------------------------------------------------------
// 2D antiplane strike slip on a vertical fault in a half space
__device__ __forceinline__ double entry_2dvs(const DevBemv& b, int i, int j) {
  // mu/(2 pi) * [1/(x_i - xr_j) - 1/(x_i - xl_j)] minus the image term; the
  // products are rounded separately (no fused multiply-add) so the value is
  // the same double a strict IEEE evaluation gives.
  const double factor = 32.04 / (2.0 * HBI_PI);
  const double xi = b.xcol[i], xl = b.xel[j], xr = b.xer[j];
  double t1 = __dmul_rn(factor, __dsub_rn(__ddiv_rn(1.0, __dsub_rn(xi, xr)), __ddiv_rn(1.0, __dsub_rn(xi, xl))));
  double t2 = __dmul_rn(factor, __dsub_rn(__ddiv_rn(1.0, __dadd_rn(xi, xr)), __ddiv_rn(1.0, __dadd_rn(xi, xl))));
  return __dsub_rn(t1, t2);
}

// ------------------------------------------------------------------------
// Okada (1992) displacement gradients for a finite rectangle (strike-slip
// disl1, dip-slip disl2; tensile unused on the hot path).  u[0..8] =
// uxx,uyx,uzx,uxy,uyy,uzy,uxz,uyz,uzz.
struct OkCorner {
  double xi2, et2, q2, r, r2, r3, r5, yp, d, x11, y11, x32, y32, ey, ez, fy, fz, gy, gz;
};

__device__ __forceinline__ void ok_corner(double xi, double et, double q, double sd, double cd, OkCorner& c) {
  c.xi2 = xi * xi; c.et2 = et * et; c.q2 = q * q;
  c.r2 = c.xi2 + c.et2 + c.q2;
  c.r = sqrt(c.r2);
  c.r3 = c.r * c.r2;
  c.r5 = c.r3 * c.r2;
  c.yp = et * cd + q * sd;
  c.d = et * sd - q * cd;
  const double rxi = c.r + xi;
  c.x11 = 1.0 / (c.r * rxi);
  c.x32 = (c.r + rxi) * c.x11 * c.x11 / c.r;
  const double ret = c.r + et;
  c.y11 = 1.0 / (c.r * ret);
  c.y32 = (c.r + ret) * c.y11 * c.y11 / c.r;
  c.ey = sd / c.r - c.yp * q / c.r3;
  c.ez = cd / c.r + c.d * q / c.r3;
  c.fy = c.d / c.r3 + c.xi2 * c.y32 * sd;
  c.fz = c.yp / c.r3 + c.xi2 * c.y32 * cd;
  c.gy = 2.0 * c.x11 * sd - c.yp * q * c.x32;
  c.gz = 2.0 * c.x11 * cd + c.d * q * c.x32;
}

// part A (infinite-medium terms), gradient rows 4..12 of Okada's ua
__device__ __forceinline__ void ok_ua(const OkCorner& c, double xi, double et, double q, double sd, double cd,
                                      double s1, double s2, double alpha, double* g) {
  const double alp1 = (1.0 - alpha) / 2.0, alp2 = alpha / 2.0;
  const double xy = xi * c.y11, qy = q * c.y11;
  double a[9], bb[9];
  a[0] = -alp1 * qy - alp2 * c.xi2 * q * c.y32;
  a[1] = -alp2 * xi * q / c.r3;
  a[2] = alp1 * xy + alp2 * xi * c.q2 * c.y32;
  a[3] = alp1 * xy * sd + alp2 * xi * c.fy + c.d / 2.0 * c.x11;
  a[4] = alp2 * c.ey;
  a[5] = alp1 * (cd / c.r + qy * sd) - alp2 * q * c.fy;
  a[6] = alp1 * xy * cd + alp2 * xi * c.fz + c.yp / 2.0 * c.x11;
  a[7] = alp2 * c.ez;
  a[8] = -alp1 * (sd / c.r - qy * cd) - alp2 * q * c.fz;
  bb[0] = -alp2 * xi * q / c.r3;
  bb[1] = -qy / 2.0 - alp2 * et * q / c.r3;
  bb[2] = alp1 / c.r + alp2 * c.q2 / c.r3;
  bb[3] = alp2 * c.ey;
  bb[4] = alp1 * c.d * c.x11 + xy / 2.0 * sd + alp2 * et * c.gy;
  bb[5] = alp1 * c.yp * c.x11 - alp2 * q * c.gy;
  bb[6] = alp2 * c.ez;
  bb[7] = alp1 * c.yp * c.x11 + xy / 2.0 * cd + alp2 * et * c.gz;
  bb[8] = -alp1 * c.d * c.x11 - alp2 * q * c.gz;
#pragma unroll
  for (int k = 0; k < 9; k++) g[k] = (0.0 + s1 * a[k]) + s2 * bb[k];
}

// part B (surface terms), gradient rows of Okada's ub
__device__ __forceinline__ void ok_ub(const OkCorner& c, double xi, double et, double q, double sd, double cd,
                                      double s1, double s2, double alpha, double* g) {
  const double alp3 = (1.0 - alpha) / alpha;
  const double rd = c.r + c.d;
  const double d11 = 1.0 / (c.r * rd);
  const double aj2 = xi * c.yp / rd * d11;
  const double aj5 = -(c.d + c.yp * c.yp / rd) * d11;
  double ak1, ak3, aj3, aj6;
  if (cd != 0.0) {
    ak1 = xi * (d11 - c.y11 * sd) / cd;
    ak3 = (q * c.y11 - c.yp * d11) / cd;
    aj3 = (ak1 - aj2 * sd) / cd;
    aj6 = (ak3 - aj5 * sd) / cd;
  } else {
    const double rd2 = rd * rd;
    ak1 = xi * q / rd * d11;
    ak3 = sd / rd * (c.xi2 * d11 - 1.0);
    aj3 = -xi / rd2 * (c.q2 * d11 - 1.0 / 2.0);
    aj6 = -c.yp / rd2 * (c.xi2 * d11 - 1.0 / 2.0);
  }
  const double xy = xi * c.y11;
  const double ak2 = 1.0 / c.r + ak3 * sd;
  const double ak4 = xy * cd - ak1 * sd;
  const double aj1 = aj5 * cd - aj6 * sd;
  const double aj4 = -xy - aj2 * cd + aj3 * sd;
  const double qx = q * c.x11, qy = q * c.y11;
  double a[9], bb[9];
  a[0] = c.xi2 * q * c.y32 - alp3 * aj1 * sd;
  a[1] = xi * q / c.r3 - alp3 * aj2 * sd;
  a[2] = -xi * c.q2 * c.y32 - alp3 * aj3 * sd;
  a[3] = -xi * c.fy - c.d * c.x11 + alp3 * (xy + aj4) * sd;
  a[4] = -c.ey + alp3 * (1.0 / c.r + aj5) * sd;
  a[5] = q * c.fy - alp3 * (qy - aj6) * sd;
  a[6] = -xi * c.fz - c.yp * c.x11 + alp3 * ak1 * sd;
  a[7] = -c.ez + alp3 * c.yp * d11 * sd;
  a[8] = q * c.fz + alp3 * ak2 * sd;
  bb[0] = xi * q / c.r3 + alp3 * aj4 * sd * cd;
  bb[1] = et * q / c.r3 + qy + alp3 * aj5 * sd * cd;
  bb[2] = -c.q2 / c.r3 + alp3 * aj6 * sd * cd;
  bb[3] = -c.ey + alp3 * aj1 * sd * cd;
  bb[4] = -et * c.gy - xy * sd + alp3 * aj2 * sd * cd;
  bb[5] = q * c.gy + alp3 * aj3 * sd * cd;
  bb[6] = -c.ez - alp3 * ak3 * sd * cd;
  bb[7] = -et * c.gz - xy * cd - alp3 * xi * d11 * sd * cd;
  bb[8] = q * c.gz - alp3 * ak4 * sd * cd;
  (void)qx;
#pragma unroll
  for (int k = 0; k < 9; k++) g[k] = (0.0 + s1 * a[k]) + s2 * bb[k];
}

// part C (depth terms): all 12 rows are needed (rows 1..3 enter the gradient)
__device__ __forceinline__ void ok_uc(const OkCorner& cc, double xi, double et, double q, double z, double sd,
                                      double cd, double s1, double s2, double alpha, double* g12) {
  const double alp4 = 1.0 - alpha, alp5 = alpha;
  const double r = cc.r, r2 = cc.r2, r3 = cc.r3, r5 = cc.r5, d = cc.d, yp = cc.yp;
  const double x11 = cc.x11, y11 = cc.y11, x32 = cc.x32, y32 = cc.y32, xi2 = cc.xi2, et2 = cc.et2, q2 = cc.q2;
  const double c = d + z;
  const double x53 = (8.0 * r2 + 9.0 * r * xi + 3.0 * xi2) * x11 * x11 * x11 / r2;
  const double y53 = (8.0 * r2 + 9.0 * r * et + 3.0 * et2) * y11 * y11 * y11 / r2;
  const double h = q * cd - z;
  const double z32 = sd / r3 - h * y32;
  const double z53 = 3.0 * sd / r5 - h * y53;
  const double y0 = y11 - xi2 * y32;
  const double z0 = z32 - xi2 * z53;
  const double ppy = cd / r3 + q * y32 * sd;
  const double ppz = sd / r3 - q * y32 * cd;
  const double qq = z * y32 + z32 + z0;
  const double qqy = 3.0 * c * d / r5 - qq * sd;
  const double qqz = 3.0 * c * yp / r5 - qq * cd + q * y32;
  const double xy = xi * y11, qy = q * y11;
  const double qr = 3.0 * q / r5;
  const double cdr = (c + d) / r3;
  const double yy0 = yp / r3 - y0 * cd;
  double a[12], bb[12];
  a[0] = alp4 * xy * cd - alp5 * xi * q * z32;
  a[1] = alp4 * (cd / r + 2.0 * qy * sd) - alp5 * c * q / r3;
  a[2] = alp4 * qy * cd - alp5 * (c * et / r3 - z * y11 + xi2 * z32);
  a[3] = alp4 * y0 * cd - alp5 * q * z0;
  a[4] = -alp4 * xi * (cd / r3 + 2.0 * q * y32 * sd) + alp5 * c * xi * qr;
  a[5] = -alp4 * xi * q * y32 * cd + alp5 * xi * (3.0 * c * et / r5 - qq);
  a[6] = -alp4 * xi * ppy * cd - alp5 * xi * qqy;
  a[7] = alp4 * 2.0 * (d / r3 - y0 * sd) * sd - yp / r3 * cd - alp5 * (cdr * sd - et / r3 - c * yp * qr);
  a[8] = -alp4 * q / r3 + yy0 * sd + alp5 * (cdr * cd + c * d * qr - (y0 * cd + q * z0) * sd);
  a[9] = alp4 * xi * ppz * cd - alp5 * xi * qqz;
  a[10] = alp4 * 2.0 * (yp / r3 - y0 * cd) * sd + d / r3 * cd - alp5 * (cdr * cd + c * d * qr);
  a[11] = yy0 * cd - alp5 * (cdr * sd - c * yp * qr - y0 * sd * sd + q * z0 * cd);
  bb[0] = alp4 * cd / r - qy * sd - alp5 * c * q / r3;
  bb[1] = alp4 * yp * x11 - alp5 * c * et * q * x32;
  bb[2] = -d * x11 - xy * sd - alp5 * c * (x11 - q2 * x32);
  bb[3] = -alp4 * xi / r3 * cd + alp5 * c * xi * qr + xi * q * y32 * sd;
  bb[4] = -alp4 * yp / r3 + alp5 * c * et * qr;
  bb[5] = d / r3 - y0 * sd + alp5 * c / r3 * (1.0 - 3.0 * q2 / r2);
  bb[6] = -alp4 * et / r3 + y0 * sd * sd - alp5 * (cdr * sd - c * yp * qr);
  bb[7] = alp4 * (x11 - yp * yp * x32) - alp5 * c * ((d + 2.0 * q * cd) * x32 - yp * et * q * x53);
  bb[8] = xi * ppy * sd + yp * d * x32 + alp5 * c * ((yp + 2.0 * q * sd) * x32 - yp * q2 * x53);
  bb[9] = -q / r3 + y0 * sd * cd - alp5 * (cdr * cd + c * d * qr);
  bb[10] = alp4 * yp * d * x32 - alp5 * c * ((yp - 2.0 * q * sd) * x32 + d * et * q * x53);
  bb[11] = -xi * ppz * sd + x11 - d * d * x32 - alp5 * c * ((d - 2.0 * q * cd) * x32 - d * q2 * x53);
#pragma unroll
  for (int k = 0; k < 12; k++) g12[k] = (0.0 + s1 * a[k]) + s2 * bb[k];
}

// Displacement gradients of Okada's DC3D for strike/dip slip (disl1,disl2).
// grad[0..8] = uxx,uyx,uzx,uxy,uyy,uzy,uxz,uyz,uzz
__device__ __forceinline__ void okada_grad(double alpha, double x, double y, double z, double depth, double sd,
                                           double cd, double al1, double al2, double aw1, double aw2,
                                           double disl1, double disl2, bool fullspace, double* grad) {
  const double pi2 = 2.0 * HBI_PI;
  const double s1 = disl1 / pi2, s2 = disl2 / pi2;
  const double xi[2] = {x - al1, x - al2};
  double u[9];
#pragma unroll
  for (int k = 0; k < 9; k++) u[k] = 0.0;
  double d = depth + z;
  double p = y * cd + d * sd;
  double q = y * sd - d * cd;
  double et[2] = {p - aw1, p - aw2};
#pragma unroll
  for (int k = 0; k < 2; k++)
#pragma unroll
    for (int j = 0; j < 2; j++) {
      OkCorner c;
      ok_corner(xi[j], et[k], q, sd, cd, c);
      double ga[9];
      ok_ua(c, xi[j], et[k], q, sd, cd, s1, s2, alpha, ga);
      double du[9];
      du[0] = -ga[0];
      du[1] = -ga[1] * cd + ga[2] * sd;
      du[2] = -ga[1] * sd - ga[2] * cd;
      du[3] = -ga[3];
      du[4] = -ga[4] * cd + ga[5] * sd;
      du[5] = -ga[4] * sd - ga[5] * cd;
      du[6] = ga[6];
      du[7] = ga[7] * cd - ga[8] * sd;
      du[8] = ga[7] * sd + ga[8] * cd;
      const bool plus = (j + k) != 1;
#pragma unroll
      for (int m = 0; m < 9; m++) u[m] = plus ? u[m] + du[m] : u[m] - du[m];
    }
  if (!fullspace) {
    d = depth - z;
    p = y * cd + d * sd;
    q = y * sd - d * cd;
    et[0] = p - aw1; et[1] = p - aw2;
#pragma unroll 1
    for (int k = 0; k < 2; k++)
#pragma unroll 1
      for (int j = 0; j < 2; j++) {
        OkCorner c;
        ok_corner(xi[j], et[k], q, sd, cd, c);
        double ga[9], gb[9], gc[12];
        ok_ua(c, xi[j], et[k], q, sd, cd, s1, s2, alpha, ga);
        ok_ub(c, xi[j], et[k], q, sd, cd, s1, s2, alpha, gb);
        ok_uc(c, xi[j], et[k], q, z, sd, cd, s1, s2, alpha, gc);
        double du[9];
        // rows 4..12 of Okada's image-source combination (gc offset by 3)
        du[0] = ga[0] + gb[0] + z * gc[3];
        du[1] = (ga[1] + gb[1] + z * gc[4]) * cd - (ga[2] + gb[2] + z * gc[5]) * sd;
        du[2] = (ga[1] + gb[1] - z * gc[4]) * sd + (ga[2] + gb[2] - z * gc[5]) * cd;
        du[3] = ga[3] + gb[3] + z * gc[6];
        du[4] = (ga[4] + gb[4] + z * gc[7]) * cd - (ga[5] + gb[5] + z * gc[8]) * sd;
        du[5] = (ga[4] + gb[4] - z * gc[7]) * sd + (ga[5] + gb[5] - z * gc[8]) * cd;
        du[6] = ga[6] + gb[6] + z * gc[9];
        du[7] = (ga[7] + gb[7] + z * gc[10]) * cd - (ga[8] + gb[8] + z * gc[11]) * sd;
        du[8] = (ga[7] + gb[7] - z * gc[10]) * sd + (ga[8] + gb[8] - z * gc[11]) * cd;
        du[6] = du[6] + gc[0];
        du[7] = du[7] + gc[1] * cd - gc[2] * sd;
        du[8] = du[8] - gc[1] * sd - gc[2] * cd;
        const bool plus = (j + k) != 1;
#pragma unroll
        for (int m = 0; m < 9; m++) u[m] = plus ? u[m] + du[m] : u[m] - du[m];
      }
  }
#pragma unroll
  for (int k = 0; k < 9; k++) grad[k] = u[k];
}

__device__ __forceinline__ double entry_okada(const DevBemv& b, int i, int j, bool fullspace) {
  const double pois = 0.25, rigid = 32.04;
  const double alpha = (1.0 + (0.5 / pois - 1.0)) / (1.0 + 2.0 * (0.5 / pois - 1.0));
  const double ca = b.cang[j], sa = b.sang[j];
  const double ddx = b.xcol[i] - b.xcol[j], ddy = b.ycol[i] - b.ycol[j];
  const double dx = ca * ddx + sa * ddy;
  const double dy = -sa * ddx + ca * ddy;
  const double w = b.w;
  const double z = b.zcol[i];
  const double depth = -b.zcol[j];
  // Okada's sin/cos of the dip in degrees, with its |cos|<1e-6 snap
  double sd = b.sangd[j], cd = b.cangd[j];
  const double rs = b.dsl[j] / w, rd = b.dsd[j] / w;
  double g[9];
  okada_grad(alpha, dx / w, dy / w, z / w, depth / w, sd, cd, -0.5 * rs, 0.5 * rs, -0.5 * rd, 0.5 * rd,
             -b.crake[j], -b.srake[j], fullspace, g);
  const double uxx = g[0], uyx = g[1], uzx = g[2], uxy = g[3], uyy = g[4], uzy = g[5], uxz = g[6], uyz = g[7], uzz = g[8];
  const double exx = uxx, eyy = uyy, ezz = uzz;
  const double exy = 0.5 * (uxy + uyx), eyz = 0.5 * (uyz + uzy), ezx = 0.5 * (uzx + uxz);
  double S[6];
  S[0] = rigid * (exx + eyy + ezz) + 2 * rigid * exx;
  S[1] = rigid * (exx + eyy + ezz) + 2 * rigid * eyy;
  S[2] = rigid * (exx + eyy + ezz) + 2 * rigid * ezz;
  S[3] = 2 * rigid * exy;
  S[4] = 2 * rigid * ezx;
  S[5] = 2 * rigid * eyz;
  // receiver frame: rotation by (strike_j - strike_i) and the receiver dip
  const double rot = b.ang[j] - b.ang[i];
  const double cr = cos(rot), sr = sin(rot);
  const double cdp = cos(b.angd[i]), sdp = sin(b.angd[i]);
  double A[3][3];
  A[0][0] = cr; A[1][0] = -sr; A[2][0] = 0.0;
  A[0][1] = sr * cdp; A[1][1] = cr * cdp; A[2][1] = sdp;
  A[0][2] = sr * sdp; A[1][2] = cr * sdp; A[2][2] = -cdp;
  double p[6];
  tens_trans_d(S, A, p);
  if (b.normal) return p[2];
  return p[4] * b.crake[i] + p[5] * b.srake[i];
}

// ------------------------------------------------------------------------
// Nikkhoo & Walter (2015) angular-dislocation strain and triangular
// dislocation stress in a full space.
__device__ __forceinline__ void ang_dis_strain_d(double x, double y, double z, double sinA, double cosA, double bx,
                                                 double by, double bz, double nu, double* E) {
  const double pi = HBI_PI;
  const double eta = y * cosA - z * sinA;
  const double zeta = y * sinA + z * cosA;
  const double x2 = x * x, y2 = y * y, z2 = z * z;
  const double r2 = x2 + y2 + z2;
  const double r = sqrt(r2);
  const double r3 = r * r2;
  const double rz = r * (r - z);
  const double r2z2 = r2 * ((r - z) * (r - z));
  const double r3z = r3 * (r - z);
  const double W = zeta - r;
  const double W2 = W * W;
  const double Wr = W * r;
  const double W2r = W2 * r;
  const double Wr3 = W * r3;
  const double W2r2 = W2 * r2;
  const double C = (r * cosA - z) / Wr;
  const double S = (r * sinA - y) / Wr;
  const double rFi_rx = (eta / r / (r - zeta) - y / r / (r - z)) / 4 / pi;
  const double rFi_ry = (x / r / (r - z) - cosA * x / r / (r - zeta)) / 4 / pi;
  const double rFi_rz = (sinA * x / r / (r - zeta)) / 4 / pi;
  const double y3 = y * y * y;
  const double k1 = 1.0 / 8 / pi / (1 - nu);
  const double bxk = bx / 8 / pi / (1 - nu);
  const double byk = by / 8 / pi / (1 - nu);
  const double bxx = by * x / 8 / pi / (1 - nu);
  const double bzx = bz * x * sinA / 8 / pi / (1 - nu);
  const double bzs = bz * sinA / 8 / pi / (1 - nu);
  (void)k1;
  E[0] = bx * (rFi_rx) + bxk * (eta / Wr + eta * x2 / W2r2 - eta * x2 / Wr3 + y / rz - x2 * y / r2z2 - x2 * y / r3z) -
         bxx * (((2 * nu + 1) / Wr + x2 / W2r2 - x2 / Wr3) * cosA + (2 * nu + 1) / rz - x2 / r2z2 - x2 / r3z) +
         bzx * ((2 * nu + 1) / Wr + x2 / W2r2 - x2 / Wr3);
  E[1] = by * (rFi_ry) + bxk * ((1 / Wr + S * S - y2 / Wr3) * eta + (2 * nu + 1) * y / rz - y3 / r2z2 - y3 / r3z - 2 * nu * cosA * S) -
         bxx * (1 / rz - y2 / r2z2 - y2 / r3z + (1 / Wr + S * S - y2 / Wr3) * cosA) + bzx * (1 / Wr + S * S - y2 / Wr3);
  E[2] = bz * (rFi_rz) + bxk * (eta / W / r + eta * C * C - eta * z2 / Wr3 + y * z / r3 + 2 * nu * sinA * C) -
         bxx * ((1 / Wr + C * C - z2 / Wr3) * cosA + z / r3) + bzx * (1 / Wr + C * C - z2 / Wr3);
  E[3] = bx * (rFi_ry) / 2 + by * (rFi_rx) / 2 -
         bxk * (x * y2 / r2z2 - nu * x / rz + x * y2 / r3z - nu * x * cosA / Wr + eta * x * S / Wr + eta * x * y / Wr3) +
         byk * (x2 * y / r2z2 - nu * y / rz + x2 * y / r3z + nu * cosA * S + x2 * y * cosA / Wr3 + x2 * cosA * S / Wr) -
         bzs * (nu * S + x2 * S / Wr + x2 * y / Wr3);
  E[4] = bx * (rFi_rz) / 2 + bz * (rFi_rx) / 2 -
         bxk * (-x * y / r3 + nu * x * sinA / Wr + eta * x * C / Wr + eta * x * z / Wr3) +
         byk * (-x2 / r3 + nu / r + nu * cosA * C + x2 * z * cosA / Wr3 + x2 * cosA * C / Wr) -
         bzs * (nu * C + x2 * C / Wr + x2 * z / Wr3);
  E[5] = by * (rFi_rz) / 2 + bz * (rFi_ry) / 2 +
         bxk * (y2 / r3 - nu / r - nu * cosA * C + nu * sinA * S + eta * sinA * cosA / W2 - eta * (y * cosA + z * sinA) / W2r +
                eta * y * z / W2r2 - eta * y * z / Wr3) -
         bxx * (y / r3 + sinA * (cosA * cosA) / W2 - cosA * (y * cosA + z * sinA) / W2r + y * z * cosA / W2r2 - y * z * cosA / Wr3) -
         bzx * (y * z / Wr3 - sinA * cosA / W2 + (y * cosA + z * sinA) / W2r - y * z / W2r2);
}

__device__ __forceinline__ double dot3d(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

__device__ __forceinline__ void td_setup_d(double x, double y, double z, double alpha, double bx, double by, double bz,
                                           double nu, const double* V, const double* side, double* E) {
  const double A11 = side[2], A12 = -side[1], A21 = side[1], A22 = side[2];
  const double y1 = A11 * (y - V[1]) + A12 * (z - V[2]);
  const double z1 = A21 * (y - V[1]) + A22 * (z - V[2]);
  const double by1 = A11 * by + A12 * bz;
  const double bz1 = A21 * by + A22 * bz;
  double e[6], s, c;
  sincos(-HBI_PI + alpha, &s, &c);
  ang_dis_strain_d(x, y1, z1, s, c, bx, by1, bz1, nu, e);
  const double B[3][3] = {{1, 0, 0}, {0, A11, A12}, {0, A21, A22}};
  tens_trans_d(e, B, E);
}

// stress S6 = Sxx,Syy,Szz,Sxy,Sxz,Syz at (X,Y,Z) from triangle P1P2P3 with
// slip (Ss strike, Ds dip, Ts tensile)
__device__ __forceinline__ void td_stress_fs(double X, double Y, double Z, const double* P1, const double* P2,
                                             const double* P3, double Ss, double Ds, double Ts, double mu,
                                             double lambda, double* S6) {
  const double nu = 1 / (1 + lambda / mu) / 2;
  const double bx = Ts, by = Ss, bz = Ds;
  double a[3], c[3], Vn[3], Vs[3], Vd[3];
  for (int k = 0; k < 3; k++) { a[k] = P2[k] - P1[k]; c[k] = P3[k] - P1[k]; }
  Vn[0] = a[1] * c[2] - c[1] * a[2];
  Vn[1] = a[2] * c[0] - c[2] * a[0];
  Vn[2] = a[0] * c[1] - c[0] * a[1];
  double s = sqrt(dot3d(Vn, Vn));
  for (int k = 0; k < 3; k++) Vn[k] = Vn[k] / s;
  // Vstrike = eZ x Vn
  Vs[0] = 0.0 * Vn[2] - Vn[1] * 1.0;
  Vs[1] = 1.0 * Vn[0] - Vn[2] * 0.0;
  Vs[2] = 0.0 * Vn[1] - Vn[0] * 0.0;
  s = sqrt(dot3d(Vs, Vs));
  for (int k = 0; k < 3; k++) Vs[k] = Vs[k] / s;
  if (dot3d(Vs, Vs) == 0.0) { Vs[0] = 0.0 * Vn[2]; Vs[1] = 1.0 * Vn[2]; Vs[2] = 0.0 * Vn[2]; }
  s = sqrt(dot3d(Vs, Vs));
  for (int k = 0; k < 3; k++) Vs[k] = Vs[k] / s;
  Vd[0] = Vn[1] * Vs[2] - Vs[1] * Vn[2];
  Vd[1] = Vn[2] * Vs[0] - Vs[2] * Vn[0];
  Vd[2] = Vn[0] * Vs[1] - Vs[0] * Vn[1];
  double At[3][3];
  for (int k = 0; k < 3; k++) { At[0][k] = Vn[k]; At[1][k] = Vs[k]; At[2][k] = Vd[k]; }
  auto ct = [&](double x1, double x2, double x3, double* o) {
    o[0] = At[0][0] * x1 + At[0][1] * x2 + At[0][2] * x3;
    o[1] = At[1][0] * x1 + At[1][1] * x2 + At[1][2] * x3;
    o[2] = At[2][0] * x1 + At[2][1] * x2 + At[2][2] * x3;
  };
  double xyz[3], p1[3], p2[3] = {0, 0, 0}, p3[3];
  ct(X - P2[0], Y - P2[1], Z - P2[2], xyz);
  ct(P1[0] - P2[0], P1[1] - P2[1], P1[2] - P2[2], p1);
  ct(P3[0] - P2[0], P3[1] - P2[1], P3[2] - P2[2], p3);
  double e12[3], e13[3], e23[3];
  for (int k = 0; k < 3; k++) { e12[k] = p2[k] - p1[k]; e13[k] = p3[k] - p1[k]; e23[k] = p3[k] - p2[k]; }
  s = sqrt(dot3d(e12, e12)); for (int k = 0; k < 3; k++) e12[k] = e12[k] / s;
  s = sqrt(dot3d(e13, e13)); for (int k = 0; k < 3; k++) e13[k] = e13[k] / s;
  s = sqrt(dot3d(e23, e23)); for (int k = 0; k < 3; k++) e23[k] = e23[k] / s;
  double me12[3] = {-e12[0], -e12[1], -e12[2]}, me13[3] = {-e13[0], -e13[1], -e13[2]}, me23[3] = {-e23[0], -e23[1], -e23[2]};
  const double A = acos(dot3d(e12, e13));
  const double B = acos(dot3d(me12, e23));
  const double C = acos(dot3d(e23, e13));
  // configuration of the point relative to the triangle (trimodefinder)
  const double x = xyz[1], y = xyz[2], zz = xyz[0];
  const double den = (p2[2] - p3[2]) * (p1[1] - p3[1]) + (p3[1] - p2[1]) * (p1[2] - p3[2]);
  const double ta = ((p2[2] - p3[2]) * (x - p3[1]) + (p3[1] - p2[1]) * (y - p3[2])) / den;
  const double tb = ((p3[2] - p1[2]) * (x - p3[1]) + (p1[1] - p3[1]) * (y - p3[2])) / den;
  const double tc = 1.0 - ta - tb;
  int mode = 1;
  if ((ta <= 0.0) && (tb > tc) && (tc > ta)) mode = -1;
  if ((tb <= 0.0) && (tc > ta) && (ta > tb)) mode = -1;
  if ((tc <= 0.0) && (ta > tb) && (tb > tc)) mode = -1;
  if ((ta == 0.0) && (tb >= 0.0) && (tc >= 0.0)) mode = 0;
  if ((ta >= 0.0) && (tb == 0.0) && (tc >= 0.0)) mode = 0;
  if ((ta >= 0.0) && (tb >= 0.0) && (tc == 0.0)) mode = 0;
  if ((mode == 0) && (zz != 0.0)) mode = 1;
  double E1[6], E2[6], E3[6], e[6];
  if (mode == 1) {
    td_setup_d(xyz[0], xyz[1], xyz[2], A, bx, by, bz, nu, p1, me13, E1);
    td_setup_d(xyz[0], xyz[1], xyz[2], B, bx, by, bz, nu, p2, e12, E2);
    td_setup_d(xyz[0], xyz[1], xyz[2], C, bx, by, bz, nu, p3, e23, E3);
  } else {
    td_setup_d(xyz[0], xyz[1], xyz[2], A, bx, by, bz, nu, p1, e13, E1);
    td_setup_d(xyz[0], xyz[1], xyz[2], B, bx, by, bz, nu, p2, me12, E2);
    td_setup_d(xyz[0], xyz[1], xyz[2], C, bx, by, bz, nu, p3, me23, E3);
  }
  for (int k = 0; k < 6; k++) e[k] = E1[k] + E2[k] + E3[k];
  if (mode == 0)
    for (int k = 0; k < 6; k++) e[k] = __longlong_as_double(0x7ff8000000000000ULL);
  double Ev[6];
  tens_trans_d(e, At, Ev);
  S6[0] = 2 * mu * Ev[0] + lambda * (Ev[0] + Ev[1] + Ev[2]);
  S6[1] = 2 * mu * Ev[1] + lambda * (Ev[0] + Ev[1] + Ev[2]);
  S6[2] = 2 * mu * Ev[2] + lambda * (Ev[0] + Ev[1] + Ev[2]);
  S6[3] = 2 * mu * Ev[3];
  S6[4] = 2 * mu * Ev[4];
  S6[5] = 2 * mu * Ev[5];
}

__device__ __forceinline__ double entry_td(const DevBemv& b, int i, int j) {
  const double pois = 0.25, rigid = 32.04;
  const double lambda = 2 * pois / (1 - 2 * pois) * rigid;
  const double P1[3] = {b.xs1[j], b.ys1[j], b.zs1[j]};
  const double P2[3] = {b.xs2[j], b.ys2[j], b.zs2[j]};
  const double P3[3] = {b.xs3[j], b.ys3[j], b.zs3[j]};
  double S[6];
  // the reference drives the source with the *receiver's* rake (matel3dn_ij :823-824)
  td_stress_fs(b.xcol[i], b.ycol[i], b.zcol[i], P1, P2, P3, b.crake[i], b.srake[i], 0.0, rigid, lambda, S);
  double A[3][3];
  A[0][0] = b.ev11[i]; A[0][1] = b.ev21[i]; A[0][2] = b.ev31[i];
  A[1][0] = b.ev12[i]; A[1][1] = b.ev22[i]; A[1][2] = b.ev32[i];
  A[2][0] = b.ev13[i]; A[2][1] = b.ev23[i]; A[2][2] = b.ev33[i];
  double p[6];
  tens_trans_d(S, A, p);
  if (b.normal) return -p[2];
  return p[4] * b.crake[i] + p[5] * b.srake[i];
}

// ------------------------------------------------------------------------
// Half space: free-surface correction of the triangular dislocation.
// Strain (v11, v22, v33, v12, v13, v23) of the harmonic (free-surface
// correction) part of an angular dislocation of angle beta whose vertex is at
// depth a, at (y1, y2, y3) in its own frame, for Burgers vector (b1, b2, b3)
// (AngDisStrainFSC, TDstressFS.f90:629-1011; Nikkhoo & Walter 2015, after
// Comninou & Dundurs 1975).  The published expressions are kept term by term;
// the factors that recur across components are named once (R*, Q*).
static __device__ __noinline__ void ang_dis_strain_fsc_d(double y1, double y2, double y3, double beta, double b1,
                                                  double b2, double b3, double nu, double a, double* v) {
  const double sB = sin(beta), cB = cos(beta), ctB = cB / sB;
  const double y3b = y3 + 2 * a;
  const double z1b = y1 * cB + y3b * sB;
  const double z3b = -y1 * sB + y3b * cB;
  const double rb2 = y1 * y1 + y2 * y2 + y3b * y3b;
  const double rb = sqrt(rb2);
  const double W1 = rb * cB + y3b, W2 = cB + a / rb, W3 = cB + y3b / rb, W4 = nu + a / rb;
  const double W5 = 2 * nu + a / rb, W6 = rb + y3b, W7 = rb + z3b, W8 = y3 + a, W9 = 1 + a / rb / cB;
  const double N1 = 1 - 2 * nu, nu2 = 2 - 2 * nu;
  // derivatives of the Burgers function
  const double F2 = z1b / rb / (rb + z3b) - y1 / rb / (rb + y3b);
  const double F1 = y2 / rb / (rb + y3b) - cB * y2 / rb / (rb + z3b);
  const double F3 = -sB * y2 / rb / (rb + z3b);
  const double rb3 = rb * rb * rb, rb4 = rb2 * rb2, rb5 = rb * rb * rb * rb * rb;
  const double W6s = W6 * W6, W7s = W7 * W7, ct2 = ctB * ctB, cB2 = cB * cB;
  const double y1s = y1 * y1, y2s = y2 * y2, y1c = y1 * y1 * y1, y2c = y2 * y2 * y2;
  const double Ys = y1 / rb - sB, Y3 = y3b / rb + 1, C3 = cB * y3b / rb + 1;
  const double Q1 = W1 * (N1 * cB - a / rb) * ctB + nu2 * (rb * sB - y1) * cB;
  const double Q2 = cB / W7 * Q1 - a * y3b * cB * ctB / rb2;
  const double R1 = -N1 * ctB + y1 / W6 * W5 + a * y1 / rb2;
  const double R2 = N1 * ctB - 2 * nu * y1 / W6 - a * y1 / rb * (1 / rb + 1 / W6);
  const double R3 = (-2 + 2 * nu) * cB + W1 / W7 * W9 + a * y3b / rb2 / cB;
  const double R5 = nu2 * cB - W1 / W7 * W9;
  const double R4 = -cB * sB + a * y1 * y3b / rb3 / cB + (rb * sB - y1) / rb * R5;
  const double R7 = y2s * cB2 - a * z1b * ctB / rb * W1;
  const double R6 = cB2 - 1 / rb * (N1 * z1b * ctB + a * cB) + a * y3b * z1b * ctB / rb3 - 1 / rb / W7 * R7;
  const double R9 = y2s * cB * sB - a * z1b / rb * W1;
  const double R8 = sB * (cB - a / rb) + z1b / rb * (1 + a * y3b / rb2) - 1 / rb / W7 * R9;
  const double R10 = W1 / W7 * W2 + a * y3b / rb2;
  const double R11 = a / rb2 + 1 / W6;
  const double R12 = 2 * nu + 1 / rb * (N1 * y1 * ctB + a) - y1s / rb / W6 * W5 - a * y1s / rb3;
  const double R13 = -2 * nu + 1 / rb * (N1 * y1 * ctB - a) + y2s / rb / W6 * W5 + a * y2s / rb3;
  const double R14 = 1 - 2 * nu - W1 / W7 * W2 - a * y3b / rb2;
  const double R15a = nu2 * cB - W1 / W7;
  const double R15b = sB - y3b * z1b / rb2 - z1b * W1 / rb / W7;
  const double R15 = cB * sB + W1 * ctB / rb * R15a + a / rb * R15b;
  const double R16 = 1 + W1 / W7 * W2 + a * y3b / rb2;
  const double R17 = 2 * nu / W6 + a / rb2;
  const double R18 = z1b * cB - a * (rb * sB - y1) / rb / cB;
  const double R19 = -N1 * y1 * ctB + nu * y3b - a + a * y1 * ctB / rb + y1s / W6 * W4;
  const double R20 = y1 * ctB * (1 - W5) + nu * y3b - a + y2s / W6 * W4;
  const double R21 = (1 - W5) * ctB - y1 / W6 * W4;
  const double R22 = (W5 - 1) * ctB + y1 / W6 * W4;
  const double R23 = N1 * ctB - 2 * nu * y1 / W6 - a * y1 / rb2;

  // ---- v11 ----
  const double T11_1 = (-2 + 2 * nu) * N1 * F1 * ct2 - N1 * y2 / W6s * R21 / rb * y1 +
      N1 * y2 / W6 * (a / rb3 * y1 * ctB - 1 / W6 * W4 + y1s / W6s * W4 / rb + y1s / W6 * a / rb3) -
      N1 * y2 * cB * ctB / W7s * W2 * Ys - N1 * y2 * cB * ctB / W7 * a / rb3 * y1 -
      3 * a * y2 * W8 * ctB / rb5 * y1 - y2 * W8 / rb3 / W6 * R1 * y1 - y2 * W8 / rb2 / W6s * R1 * y1 +
      y2 * W8 / rb / W6 * (1 / W6 * W5 - y1s / W6s * W5 / rb - y1s / W6 * a / rb3 + a / rb2 - 2 * a * y1s / rb4) -
      y2 * W8 / rb3 / W7 * Q2 * y1 - y2 * W8 / rb / W7s * Q2 * Ys +
      y2 * W8 / rb / W7 *
          (-cB / W7s * Q1 * Ys +
           cB / W7 * (1 / rb * cB * y1 * (N1 * cB - a / rb) * ctB + W1 * a / rb3 * y1 * ctB + nu2 * (1 / rb * sB * y1 - 1) * cB) +
           2 * a * y3b * cB * ctB / rb4 * y1);
  const double T11_2 = N1 * ((nu2 * ct2 + nu) / rb * y1 / W6 - (nu2 * ct2 + 1) * cB * Ys / W7) -
      N1 / W6s * R19 / rb * y1 +
      N1 / W6 * (-N1 * ctB + a * ctB / rb - a * y1s * ctB / rb3 + 2 * y1 / W6 * W4 - y1c / W6s * W4 / rb - y1c / W6 * a / rb3) +
      N1 * ctB / W7s * R18 * Ys -
      N1 * ctB / W7 * (cB2 - a * (1 / rb * sB * y1 - 1) / rb / cB + a * (rb * sB - y1) / rb3 / cB * y1) -
      a * W8 * ctB / rb3 + 3 * a * y1s * W8 * ctB / rb5 - W8 / W6s * R12 / rb * y1 +
      W8 / W6 * (-1 / rb3 * (N1 * y1 * ctB + a) * y1 + 1 / rb * N1 * ctB - 2 * y1 / rb / W6 * W5 + y1c / rb3 / W6 * W5 +
                 y1c / rb2 / W6s * W5 + y1c / rb4 / W6 * a - 2 * a / rb3 * y1 + 3 * a * y1c / rb5) -
      W8 * ctB / W7s * R4 * Ys +
      W8 * ctB / W7 *
          (a * y3b / rb3 / cB - 3 * a * y1s * y3b / rb5 / cB + (1 / rb * sB * y1 - 1) / rb * R5 - (rb * sB - y1) / rb3 * R5 * y1 +
           (rb * sB - y1) / rb * (-1 / rb * cB * y1 / W7 * W9 + W1 / W7s * W9 * Ys + W1 / W7 * a / rb3 / cB * y1));
  const double T11_3 =
      N1 * (-y2 / W6s * (1 + a / rb) / rb * y1 - y2 / W6 * a / rb3 * y1 + y2 * cB / W7s * W2 * Ys + y2 * cB / W7 * a / rb3 * y1) +
      y2 * W8 / rb3 * R11 * y1 - y2 * W8 / rb * (-2 * a / rb4 * y1 - 1 / W6s / rb * y1) -
      y2 * W8 * cB / rb3 / W7 * R10 * y1 - y2 * W8 * cB / rb / W7s * R10 * Ys +
      y2 * W8 * cB / rb / W7 * (1 / rb * cB * y1 / W7 * W2 - W1 / W7s * W2 * Ys - W1 / W7 * a / rb3 * y1 - 2 * a * y3b / rb4 * y1);

  // ---- v22 ----
  const double T22_1 = N1 * ((nu2 * ct2 - nu) / rb * y2 / W6 - (nu2 * ct2 + 1 - 2 * nu) * cB / rb * y2 / W7) +
      N1 / W6s * R20 / rb * y2 -
      N1 / W6 * (a * y1 * ctB / rb3 * y2 + 2 * y2 / W6 * W4 - y2c / W6s * W4 / rb - y2c / W6 * a / rb3) +
      N1 * z1b * ctB / W7s * W2 / rb * y2 + N1 * z1b * ctB / W7 * a / rb3 * y2 + 3 * a * y2 * W8 * ctB / rb5 * y1 -
      W8 / W6s * R13 / rb * y2 +
      W8 / W6 * (-1 / rb3 * (N1 * y1 * ctB - a) * y2 + 2 * y2 / rb / W6 * W5 - y2c / rb3 / W6 * W5 - y2c / rb2 / W6s * W5 -
                 y2c / rb4 / W6 * a + 2 * a / rb3 * y2 - 3 * a * y2c / rb5) -
      W8 / W7s * R6 / rb * y2 +
      W8 / W7 *
          (1 / rb3 * (N1 * z1b * ctB + a * cB) * y2 - 3 * a * y3b * z1b * ctB / rb5 * y2 + 1 / rb3 / W7 * R7 * y2 +
           1 / rb2 / W7s * R7 * y2 - 1 / rb / W7 * (2 * y2 * cB2 + a * z1b * ctB / rb3 * W1 * y2 - a * z1b * ctB / rb2 * cB * y2));
  const double T22_2 = nu2 * N1 * F2 * ct2 + N1 / W6 * R22 - N1 * y2s / W6s * R22 / rb +
      N1 * y2 / W6 * (-a / rb3 * y2 * ctB - y1 / W6s * W4 / rb * y2 - y2 / W6 * a / rb3 * y1) - N1 * ctB / W7 * W9 +
      N1 * y2s * ctB / W7s * W9 / rb + N1 * y2s * ctB / W7 * a / rb3 / cB - a * W8 * ctB / rb3 +
      3 * a * y2s * W8 * ctB / rb5 + W8 / rb / W6 * R2 - y2s * W8 / rb3 / W6 * R2 - y2s * W8 / rb2 / W6s * R2 +
      y2 * W8 / rb / W6 *
          (2 * nu * y1 / W6s / rb * y2 + a * y1 / rb3 * (1 / rb + 1 / W6) * y2 - a * y1 / rb * (-1 / rb3 * y2 - 1 / W6s / rb * y2)) +
      W8 * ctB / rb / W7 * R3 - y2s * W8 * ctB / rb3 / W7 * R3 - y2s * W8 * ctB / rb2 / W7s * R3 +
      y2 * W8 * ctB / rb / W7 *
          (1 / rb * cB * y2 / W7 * W9 - W1 / W7s * W9 / rb * y2 - W1 / W7 * a / rb3 / cB * y2 - 2 * a * y3b / rb4 / cB * y2);
  const double T22_3 = N1 * (-sB / rb * y2 / W7 + y2 / W6s * (1 + a / rb) / rb * y1 + y2 / W6 * a / rb3 * y1 -
                             z1b / W7s * W2 / rb * y2 - z1b / W7 * a / rb3 * y2) -
      y2 * W8 / rb3 * R11 * y1 + y1 * W8 / rb * (-2 * a / rb4 * y2 - 1 / W6s / rb * y2) + W8 / W7s * R8 / rb * y2 -
      W8 / W7 *
          (sB * a / rb3 * y2 - z1b / rb3 * (1 + a * y3b / rb2) * y2 - 2 * z1b / rb5 * a * y3b * y2 + 1 / rb3 / W7 * R9 * y2 +
           1 / rb2 / W7s * R9 * y2 - 1 / rb / W7 * (2 * y2 * cB * sB + a * z1b / rb3 * W1 * y2 - a * z1b / rb2 * cB * y2));

  // ---- v33 ----
  const double T33_1 = nu2 * (N1 * F3 * ctB - y2 / W6s * W5 * Y3 - 0.5 * y2 / W6 * a / rb3 * 2 * y3b +
                              y2 * cB / W7s * W2 * W3 + 0.5 * y2 * cB / W7 * a / rb3 * 2 * y3b) +
      y2 / rb * R17 - 0.5 * y2 * W8 / rb3 * R17 * 2 * y3b + y2 * W8 / rb * (-2 * nu / W6s * Y3 - a / rb4 * 2 * y3b) +
      y2 * cB / rb / W7 * R14 - 0.5 * y2 * W8 * cB / rb3 / W7 * R14 * 2 * y3b - y2 * W8 * cB / rb / W7s * R14 * W3 +
      y2 * W8 * cB / rb / W7 *
          (-C3 / W7 * W2 + W1 / W7s * W2 * W3 + 0.5 * W1 / W7 * a / rb3 * 2 * y3b - a / rb2 + a * y3b / rb4 * 2 * y3b);
  const double T33_2 = (-2 + 2 * nu) * N1 * ctB * (Y3 / W6 - cB * W3 / W7) + nu2 * y1 / W6s * W5 * Y3 +
      0.5 * nu2 * y1 / W6 * a / rb3 * 2 * y3b + nu2 * sB / W7 * W2 - nu2 * z1b / W7s * W2 * W3 -
      0.5 * nu2 * z1b / W7 * a / rb3 * 2 * y3b + 1 / rb * R23 - 0.5 * W8 / rb3 * R23 * 2 * y3b +
      W8 / rb * (2 * nu * y1 / W6s * Y3 + a * y1 / rb4 * 2 * y3b) - 1 / W7 * R15 + W8 / W7s * R15 * W3 -
      W8 / W7 *
          (C3 * ctB / rb * R15a - 0.5 * W1 * ctB / rb3 * R15a * 2 * y3b + W1 * ctB / rb * (-C3 / W7 + W1 / W7s * W3) -
           0.5 * a / rb3 * R15b * 2 * y3b +
           a / rb * (-z1b / rb2 - y3b * sB / rb2 + y3b * z1b / rb4 * 2 * y3b - sB * W1 / rb / W7 - z1b * C3 / rb / W7 +
                     0.5 * z1b * W1 / rb3 / W7 * 2 * y3b + z1b * W1 / rb / W7s * W3));
  const double T33_3 = nu2 * F3 - nu2 * y2 * sB / W7s * W2 * W3 - 0.5 * nu2 * y2 * sB / W7 * a / rb3 * 2 * y3b +
      y2 * sB / rb / W7 * R16 - 0.5 * y2 * W8 * sB / rb3 / W7 * R16 * 2 * y3b - y2 * W8 * sB / rb / W7s * R16 * W3 +
      y2 * W8 * sB / rb / W7 *
          (C3 / W7 * W2 - W1 / W7s * W2 * W3 - 0.5 * W1 / W7 * a / rb3 * 2 * y3b + a / rb2 - a * y3b / rb4 * 2 * y3b);

  // ---- v12 ----
  const double T12_A = (-2 + 2 * nu) * N1 * F2 * ct2 + N1 / W6 * R21 - N1 * y2s / W6s * R21 / rb +
      N1 * y2 / W6 * (a / rb3 * y2 * ctB + y1 / W6s * W4 / rb * y2 + y2 / W6 * a / rb3 * y1) + N1 * cB * ctB / W7 * W2 -
      N1 * y2s * cB * ctB / W7s * W2 / rb - N1 * y2s * cB * ctB / W7 * a / rb3 + a * W8 * ctB / rb3 -
      3 * a * y2s * W8 * ctB / rb5 + W8 / rb / W6 * R1 - y2s * W8 / rb3 / W6 * R1 - y2s * W8 / rb2 / W6s * R1 +
      y2 * W8 / rb / W6 * (-y1 / W6s * W5 / rb * y2 - y2 / W6 * a / rb3 * y1 - 2 * a * y1 / rb4 * y2) +
      W8 / rb / W7 * Q2 - y2s * W8 / rb3 / W7 * Q2 - y2s * W8 / rb2 / W7s * Q2 +
      y2 * W8 / rb / W7 *
          (-cB / W7s * Q1 / rb * y2 +
           cB / W7 * (1 / rb * cB * y2 * (N1 * cB - a / rb) * ctB + W1 * a / rb3 * y2 * ctB + nu2 / rb * sB * y2 * cB) +
           2 * a * y3b * cB * ctB / rb4 * y2);
  const double T12_B = N1 * ((nu2 * ct2 + nu) / rb * y2 / W6 - (nu2 * ct2 + 1) * cB / rb * y2 / W7) -
      N1 / W6s * R19 / rb * y2 +
      N1 / W6 * (-a * y1 * ctB / rb3 * y2 - y1s / W6s * W4 / rb * y2 - y1s / W6 * a / rb3 * y2) +
      N1 * ctB / W7s * R18 / rb * y2 - N1 * ctB / W7 * (-a / rb2 * sB * y2 / cB + a * (rb * sB - y1) / rb3 / cB * y2) +
      3 * a * y2 * W8 * ctB / rb5 * y1 - W8 / W6s * R12 / rb * y2 +
      W8 / W6 * (-1 / rb3 * (N1 * y1 * ctB + a) * y2 + y1s / rb3 / W6 * W5 * y2 + y1s / rb2 / W6s * W5 * y2 +
                 y1s / rb4 / W6 * a * y2 + 3 * a * y1s / rb5 * y2) -
      W8 * ctB / W7s * R4 / rb * y2 +
      W8 * ctB / W7 *
          (-3 * a * y1 * y3b / rb5 / cB * y2 + 1 / rb2 * sB * y2 * R5 - (rb * sB - y1) / rb3 * R5 * y2 +
           (rb * sB - y1) / rb * (-1 / rb * cB * y2 / W7 * W9 + W1 / W7s * W9 / rb * y2 + W1 / W7 * a / rb3 / cB * y2));
  const double T12_C = N1 * (1 / W6 * (1 + a / rb) - y2s / W6s * (1 + a / rb) / rb - y2s / W6 * a / rb3 - cB / W7 * W2 +
                             y2s * cB / W7s * W2 / rb + y2s * cB / W7 * a / rb3) -
      W8 / rb * R11 + y2s * W8 / rb3 * R11 - y2 * W8 / rb * (-2 * a / rb4 * y2 - 1 / W6s / rb * y2) +
      W8 * cB / rb / W7 * R10 - y2s * W8 * cB / rb3 / W7 * R10 - y2s * W8 * cB / rb2 / W7s * R10 +
      y2 * W8 * cB / rb / W7 * (1 / rb * cB * y2 / W7 * W2 - W1 / W7s * W2 / rb * y2 - W1 / W7 * a / rb3 * y2 - 2 * a * y3b / rb4 * y2);
  const double T12_D = N1 * ((nu2 * ct2 - nu) / rb * y1 / W6 - (nu2 * ct2 + 1 - 2 * nu) * cB * Ys / W7) +
      N1 / W6s * R20 / rb * y1 -
      N1 / W6 * ((1 - W5) * ctB + a * y1s * ctB / rb3 - y2s / W6s * W4 / rb * y1 - y2s / W6 * a / rb3 * y1) -
      N1 * cB * ctB / W7 * W2 + N1 * z1b * ctB / W7s * W2 * Ys + N1 * z1b * ctB / W7 * a / rb3 * y1 - a * W8 * ctB / rb3 +
      3 * a * y1s * W8 * ctB / rb5 - W8 / W6s * R13 / rb * y1 +
      W8 / W6 * (-1 / rb3 * (N1 * y1 * ctB - a) * y1 + 1 / rb * N1 * ctB - y2s / rb3 / W6 * W5 * y1 -
                 y2s / rb2 / W6s * W5 * y1 - y2s / rb4 / W6 * a * y1 - 3 * a * y2s / rb5 * y1) -
      W8 / W7s * R6 * Ys +
      W8 / W7 *
          (1 / rb3 * (N1 * z1b * ctB + a * cB) * y1 - 1 / rb * N1 * cB * ctB + a * y3b * cB * ctB / rb3 -
           3 * a * y3b * z1b * ctB / rb5 * y1 + 1 / rb3 / W7 * R7 * y1 + 1 / rb / W7s * R7 * Ys -
           1 / rb / W7 * (-a * cB * ctB / rb * W1 + a * z1b * ctB / rb3 * W1 * y1 - a * z1b * ctB / rb2 * cB * y1));
  const double T12_E = nu2 * N1 * F1 * ct2 - N1 * y2 / W6s * R22 / rb * y1 +
      N1 * y2 / W6 * (-a / rb3 * y1 * ctB + 1 / W6 * W4 - y1s / W6s * W4 / rb - y1s / W6 * a / rb3) +
      N1 * y2 * ctB / W7s * W9 * Ys + N1 * y2 * ctB / W7 * a / rb3 / cB * y1 + 3 * a * y2 * W8 * ctB / rb5 * y1 -
      y2 * W8 / rb3 / W6 * R2 * y1 - y2 * W8 / rb2 / W6s * R2 * y1 +
      y2 * W8 / rb / W6 *
          (-2 * nu / W6 + 2 * nu * y1s / W6s / rb - a / rb * (1 / rb + 1 / W6) + a * y1s / rb3 * (1 / rb + 1 / W6) -
           a * y1 / rb * (-1 / rb3 * y1 - 1 / W6s / rb * y1)) -
      y2 * W8 * ctB / rb3 / W7 * R3 * y1 - y2 * W8 * ctB / rb / W7s * R3 * Ys +
      y2 * W8 * ctB / rb / W7 *
          (1 / rb * cB * y1 / W7 * W9 - W1 / W7s * W9 * Ys - W1 / W7 * a / rb3 / cB * y1 - 2 * a * y3b / rb4 / cB * y1);
  const double T12_F = N1 * (-sB * Ys / W7 - 1 / W6 * (1 + a / rb) + y1s / W6s * (1 + a / rb) / rb + y1s / W6 * a / rb3 +
                             cB / W7 * W2 - z1b / W7s * W2 * Ys - z1b / W7 * a / rb3 * y1) +
      W8 / rb * R11 - y1s * W8 / rb3 * R11 + y1 * W8 / rb * (-2 * a / rb4 * y1 - 1 / W6s / rb * y1) + W8 / W7s * R8 * Ys -
      W8 / W7 *
          (sB * a / rb3 * y1 + cB / rb * (1 + a * y3b / rb2) - z1b / rb3 * (1 + a * y3b / rb2) * y1 -
           2 * z1b / rb5 * a * y3b * y1 + 1 / rb3 / W7 * R9 * y1 + 1 / rb / W7s * R9 * Ys -
           1 / rb / W7 * (-a * cB / rb * W1 + a * z1b / rb3 * W1 * y1 - a * z1b / rb2 * cB * y1));

  // ---- v13 ----
  const double T13_A = (-2 + 2 * nu) * N1 * F3 * ct2 - N1 * y2 / W6s * R21 * Y3 +
      N1 * y2 / W6 * (0.5 * a / rb3 * 2 * y3b * ctB + y1 / W6s * W4 * Y3 + 0.5 * y1 / W6 * a / rb3 * 2 * y3b) -
      N1 * y2 * cB * ctB / W7s * W2 * W3 - 0.5 * N1 * y2 * cB * ctB / W7 * a / rb3 * 2 * y3b + a / rb3 * y2 * ctB -
      1.5 * a * y2 * W8 * ctB / rb5 * 2 * y3b + y2 / rb / W6 * R1 - 0.5 * y2 * W8 / rb3 / W6 * R1 * 2 * y3b -
      y2 * W8 / rb / W6s * R1 * Y3 +
      y2 * W8 / rb / W6 * (-y1 / W6s * W5 * Y3 - 0.5 * y1 / W6 * a / rb3 * 2 * y3b - a * y1 / rb4 * 2 * y3b) +
      y2 / rb / W7 * Q2 - 0.5 * y2 * W8 / rb3 / W7 * Q2 * 2 * y3b - y2 * W8 / rb / W7s * Q2 * W3 +
      y2 * W8 / rb / W7 *
          (-cB / W7s * Q1 * W3 +
           cB / W7 * (C3 * (N1 * cB - a / rb) * ctB + 0.5 * W1 * a / rb3 * 2 * y3b * ctB + 0.5 * nu2 / rb * sB * 2 * y3b * cB) -
           a * cB * ctB / rb2 + a * y3b * cB * ctB / rb4 * 2 * y3b);
  const double T13_B = N1 * ((nu2 * ct2 + nu) * Y3 / W6 - (nu2 * ct2 + 1) * cB * W3 / W7) - N1 / W6s * R19 * Y3 +
      N1 / W6 * (nu - 0.5 * a * y1 * ctB / rb3 * 2 * y3b - y1s / W6s * W4 * Y3 - 0.5 * y1s / W6 * a / rb3 * 2 * y3b) +
      N1 * ctB / W7s * R18 * W3 -
      N1 * ctB / W7 * (cB * sB - 0.5 * a / rb2 * sB * 2 * y3b / cB + 0.5 * a * (rb * sB - y1) / rb3 / cB * 2 * y3b) -
      a / rb3 * y1 * ctB + 1.5 * a * y1 * W8 * ctB / rb5 * 2 * y3b + 1 / W6 * R12 - W8 / W6s * R12 * Y3 +
      W8 / W6 * (-0.5 / rb3 * (N1 * y1 * ctB + a) * 2 * y3b + 0.5 * y1s / rb3 / W6 * W5 * 2 * y3b + y1s / rb / W6s * W5 * Y3 +
                 0.5 * y1s / rb4 / W6 * a * 2 * y3b + 1.5 * a * y1s / rb5 * 2 * y3b) +
      ctB / W7 * R4 - W8 * ctB / W7s * R4 * W3 +
      W8 * ctB / W7 *
          (a / rb3 / cB * y1 - 1.5 * a * y1 * y3b / rb5 / cB * 2 * y3b + 0.5 / rb2 * sB * 2 * y3b * R5 -
           0.5 * (rb * sB - y1) / rb3 * R5 * 2 * y3b +
           (rb * sB - y1) / rb * (-C3 / W7 * W9 + W1 / W7s * W9 * W3 + 0.5 * W1 / W7 * a / rb3 / cB * 2 * y3b));
  const double T13_C = N1 * (-y2 / W6s * (1 + a / rb) * Y3 - 0.5 * y2 / W6 * a / rb3 * 2 * y3b + y2 * cB / W7s * W2 * W3 +
                             0.5 * y2 * cB / W7 * a / rb3 * 2 * y3b) -
      y2 / rb * R11 + 0.5 * y2 * W8 / rb3 * R11 * 2 * y3b - y2 * W8 / rb * (-a / rb4 * 2 * y3b - 1 / W6s * Y3) +
      y2 * cB / rb / W7 * R10 - 0.5 * y2 * W8 * cB / rb3 / W7 * R10 * 2 * y3b - y2 * W8 * cB / rb / W7s * R10 * W3 +
      y2 * W8 * cB / rb / W7 *
          (C3 / W7 * W2 - W1 / W7s * W2 * W3 - 0.5 * W1 / W7 * a / rb3 * 2 * y3b + a / rb2 - a * y3b / rb4 * 2 * y3b);
  const double T13_D = nu2 * (N1 * F1 * ctB - y1 / W6s * W5 / rb * y2 - y2 / W6 * a / rb3 * y1 + y2 * cB / W7s * W2 * Ys +
                              y2 * cB / W7 * a / rb3 * y1) -
      y2 * W8 / rb3 * R17 * y1 + y2 * W8 / rb * (-2 * nu / W6s / rb * y1 - 2 * a / rb4 * y1) -
      y2 * W8 * cB / rb3 / W7 * R14 * y1 - y2 * W8 * cB / rb / W7s * R14 * Ys +
      y2 * W8 * cB / rb / W7 * (-1 / rb * cB * y1 / W7 * W2 + W1 / W7s * W2 * Ys + W1 / W7 * a / rb3 * y1 + 2 * a * y3b / rb4 * y1);
  const double T13_E = (-2 + 2 * nu) * N1 * ctB * (1 / rb * y1 / W6 - cB * Ys / W7) - nu2 / W6 * W5 +
      nu2 * y1s / W6s * W5 / rb + nu2 * y1s / W6 * a / rb3 + nu2 * cB / W7 * W2 - nu2 * z1b / W7s * W2 * Ys -
      nu2 * z1b / W7 * a / rb3 * y1 - W8 / rb3 * R23 * y1 +
      W8 / rb * (-2 * nu / W6 + 2 * nu * y1s / W6s / rb - a / rb2 + 2 * a * y1s / rb4) + W8 / W7s * R15 * Ys -
      W8 / W7 *
          (1 / rb2 * cB * y1 * ctB * R15a - W1 * ctB / rb3 * R15a * y1 + W1 * ctB / rb * (-1 / rb * cB * y1 / W7 + W1 / W7s * Ys) -
           a / rb3 * R15b * y1 +
           a / rb * (-y3b * cB / rb2 + 2 * y3b * z1b / rb4 * y1 - cB * W1 / rb / W7 - z1b / rb2 * cB * y1 / W7 +
                     z1b * W1 / rb3 / W7 * y1 + z1b * W1 / rb / W7s * Ys));
  const double T13_F = nu2 * F1 - nu2 * y2 * sB / W7s * W2 * Ys - nu2 * y2 * sB / W7 * a / rb3 * y1 -
      y2 * W8 * sB / rb3 / W7 * R16 * y1 - y2 * W8 * sB / rb / W7s * R16 * Ys +
      y2 * W8 * sB / rb / W7 * (1 / rb * cB * y1 / W7 * W2 - W1 / W7s * W2 * Ys - W1 / W7 * a / rb3 * y1 - 2 * a * y3b / rb4 * y1);

  // ---- v23 ----
  const double T23_A = N1 * ((nu2 * ct2 - nu) * Y3 / W6 - (nu2 * ct2 + 1 - 2 * nu) * cB * W3 / W7) + N1 / W6s * R20 * Y3 -
      N1 / W6 * (0.5 * a * y1 * ctB / rb3 * 2 * y3b + nu - y2s / W6s * W4 * Y3 - 0.5 * y2s / W6 * a / rb3 * 2 * y3b) -
      N1 * sB * ctB / W7 * W2 + N1 * z1b * ctB / W7s * W2 * W3 + 0.5 * N1 * z1b * ctB / W7 * a / rb3 * 2 * y3b -
      a / rb3 * y1 * ctB + 1.5 * a * y1 * W8 * ctB / rb5 * 2 * y3b + 1 / W6 * R13 - W8 / W6s * R13 * Y3 +
      W8 / W6 * (-0.5 / rb3 * (N1 * y1 * ctB - a) * 2 * y3b - 0.5 * y2s / rb3 / W6 * W5 * 2 * y3b - y2s / rb / W6s * W5 * Y3 -
                 0.5 * y2s / rb4 / W6 * a * 2 * y3b - 1.5 * a * y2s / rb5 * 2 * y3b) +
      1 / W7 * R6 - W8 / W7s * R6 * W3 +
      W8 / W7 *
          (0.5 / rb3 * (N1 * z1b * ctB + a * cB) * 2 * y3b - 1 / rb * N1 * sB * ctB + a * z1b * ctB / rb3 +
           a * y3b * sB * ctB / rb3 - 1.5 * a * y3b * z1b * ctB / rb5 * 2 * y3b + 0.5 / rb3 / W7 * R7 * 2 * y3b +
           1 / rb / W7s * R7 * W3 -
           1 / rb / W7 * (-a * sB * ctB / rb * W1 + 0.5 * a * z1b * ctB / rb3 * W1 * 2 * y3b - a * z1b * ctB / rb * C3));
  const double T23_B = nu2 * N1 * F3 * ct2 - N1 * y2 / W6s * R22 * Y3 +
      N1 * y2 / W6 * (-0.5 * a / rb3 * 2 * y3b * ctB - y1 / W6s * W4 * Y3 - 0.5 * y1 / W6 * a / rb3 * 2 * y3b) +
      N1 * y2 * ctB / W7s * W9 * W3 + 0.5 * N1 * y2 * ctB / W7 * a / rb3 / cB * 2 * y3b - a / rb3 * y2 * ctB +
      1.5 * a * y2 * W8 * ctB / rb5 * 2 * y3b + y2 / rb / W6 * R2 - 0.5 * y2 * W8 / rb3 / W6 * R2 * 2 * y3b -
      y2 * W8 / rb / W6s * R2 * Y3 +
      y2 * W8 / rb / W6 *
          (2 * nu * y1 / W6s * Y3 + 0.5 * a * y1 / rb3 * (1 / rb + 1 / W6) * 2 * y3b -
           a * y1 / rb * (-0.5 / rb3 * 2 * y3b - 1 / W6s * Y3)) +
      y2 * ctB / rb / W7 * R3 - 0.5 * y2 * W8 * ctB / rb3 / W7 * R3 * 2 * y3b - y2 * W8 * ctB / rb / W7s * R3 * W3 +
      y2 * W8 * ctB / rb / W7 *
          (C3 / W7 * W9 - W1 / W7s * W9 * W3 - 0.5 * W1 / W7 * a / rb3 / cB * 2 * y3b + a / rb2 / cB -
           a * y3b / rb4 / cB * 2 * y3b);
  const double T23_C = N1 * (-sB * W3 / W7 + y1 / W6s * (1 + a / rb) * Y3 + 0.5 * y1 / W6 * a / rb3 * 2 * y3b +
                             sB / W7 * W2 - z1b / W7s * W2 * W3 - 0.5 * z1b / W7 * a / rb3 * 2 * y3b) +
      y1 / rb * R11 - 0.5 * y1 * W8 / rb3 * R11 * 2 * y3b + y1 * W8 / rb * (-a / rb4 * 2 * y3b - 1 / W6s * Y3) -
      1 / W7 * R8 + W8 / W7s * R8 * W3 -
      W8 / W7 *
          (0.5 * sB * a / rb3 * 2 * y3b + sB / rb * (1 + a * y3b / rb2) - 0.5 * z1b / rb3 * (1 + a * y3b / rb2) * 2 * y3b +
           z1b / rb * (a / rb2 - a * y3b / rb4 * 2 * y3b) + 0.5 / rb3 / W7 * R9 * 2 * y3b + 1 / rb / W7s * R9 * W3 -
           1 / rb / W7 * (-a * sB / rb * W1 + 0.5 * a * z1b / rb3 * W1 * 2 * y3b - a * z1b / rb * C3));
  const double T23_D = nu2 * (N1 * F2 * ctB + 1 / W6 * W5 - y2s / W6s * W5 / rb - y2s / W6 * a / rb3 - cB / W7 * W2 +
                              y2s * cB / W7s * W2 / rb + y2s * cB / W7 * a / rb3) +
      W8 / rb * R17 - y2s * W8 / rb3 * R17 + y2 * W8 / rb * (-2 * nu / W6s / rb * y2 - 2 * a / rb4 * y2) +
      W8 * cB / rb / W7 * R14 - y2s * W8 * cB / rb3 / W7 * R14 - y2s * W8 * cB / rb2 / W7s * R14 +
      y2 * W8 * cB / rb / W7 * (-1 / rb * cB * y2 / W7 * W2 + W1 / W7s * W2 / rb * y2 + W1 / W7 * a / rb3 * y2 + 2 * a * y3b / rb4 * y2);
  const double T23_E = (-2 + 2 * nu) * N1 * ctB * (1 / rb * y2 / W6 - cB / rb * y2 / W7) + nu2 * y1 / W6s * W5 / rb * y2 +
      nu2 * y1 / W6 * a / rb3 * y2 - nu2 * z1b / W7s * W2 / rb * y2 - nu2 * z1b / W7 * a / rb3 * y2 -
      W8 / rb3 * R23 * y2 + W8 / rb * (2 * nu * y1 / W6s / rb * y2 + 2 * a * y1 / rb4 * y2) + W8 / W7s * R15 / rb * y2 -
      W8 / W7 *
          (1 / rb2 * cB * y2 * ctB * R15a - W1 * ctB / rb3 * R15a * y2 + W1 * ctB / rb * (-cB / rb * y2 / W7 + W1 / W7s / rb * y2) -
           a / rb3 * R15b * y2 +
           a / rb * (2 * y3b * z1b / rb4 * y2 - z1b / rb2 * cB * y2 / W7 + z1b * W1 / rb3 / W7 * y2 + z1b * W1 / rb2 / W7s * y2));
  const double T23_F = nu2 * F2 + nu2 * sB / W7 * W2 - nu2 * y2s * sB / W7s * W2 / rb - nu2 * y2s * sB / W7 * a / rb3 +
      W8 * sB / rb / W7 * R16 - y2s * W8 * sB / rb3 / W7 * R16 - y2s * W8 * sB / rb2 / W7s * R16 +
      y2 * W8 * sB / rb / W7 * (1 / rb * cB * y2 / W7 * W2 - W1 / W7s * W2 / rb * y2 - W1 / W7 * a / rb3 * y2 - 2 * a * y3b / rb4 * y2);

  // each block enters as b * (1/4 T / pi / (1 - nu)); shear blocks with b/2
#define FSC_K(T) (0.25 * (T) / HBI_PI / (1 - nu))
  v[0] = b1 * FSC_K(T11_1) + b2 * FSC_K(T11_2) + b3 * FSC_K(T11_3);
  v[1] = b1 * FSC_K(T22_1) + b2 * FSC_K(T22_2) + b3 * FSC_K(T22_3);
  v[2] = b1 * FSC_K(T33_1) + b2 * FSC_K(T33_2) + b3 * FSC_K(T33_3);
  v[3] = b1 / 2 * FSC_K(T12_A) + b2 / 2 * FSC_K(T12_B) + b3 / 2 * FSC_K(T12_C) + b1 / 2 * FSC_K(T12_D) +
         b2 / 2 * FSC_K(T12_E) + b3 / 2 * FSC_K(T12_F);
  v[4] = b1 / 2 * FSC_K(T13_A) + b2 / 2 * FSC_K(T13_B) + b3 / 2 * FSC_K(T13_C) + b1 / 2 * FSC_K(T13_D) +
         b2 / 2 * FSC_K(T13_E) + b3 / 2 * FSC_K(T13_F);
  v[5] = b1 / 2 * FSC_K(T23_A) + b2 / 2 * FSC_K(T23_B) + b3 / 2 * FSC_K(T23_C) + b1 / 2 * FSC_K(T23_D) +
         b2 / 2 * FSC_K(T23_E) + b3 / 2 * FSC_K(T23_F);
#undef FSC_K
}

// free-surface correction of the edge PA -> PB (AngSetupFSC_S,
// TDstressFS.f90:405-558); edges within 1e-3 rad of vertical add nothing
static __device__ __noinline__ void ang_setup_fsc_d(double X, double Y, double Z, double bX, double bY, double bZ,
                                             const double* PA, const double* PB, double mu, double lambda,
                                             double* S) {
  const double nu = lambda / (lambda + mu) / 2;
  const double side[3] = {PB[0] - PA[0], PB[1] - PA[1], PB[2] - PA[2]};
  const double beta = acos(-side[2] / sqrt(dot3d(side, side)));
  for (int k = 0; k < 6; k++) S[k] = 0.0;
  if (fabs(beta) < 1e-3 || fabs(HBI_PI - beta) < 1e-3) return;
  double ey1[3] = {side[0], side[1], 0.0};
  const double n1 = sqrt(dot3d(ey1, ey1));
  for (int k = 0; k < 3; k++) ey1[k] = ey1[k] / n1;
  const double ey3[3] = {-0.0, -0.0, -1.0};
  const double ey2[3] = {ey3[1] * ey1[2] - ey1[1] * ey3[2], ey3[2] * ey1[0] - ey1[2] * ey3[0],
                         ey3[0] * ey1[1] - ey1[0] * ey3[1]};
  double A[3][3];
  for (int k = 0; k < 3; k++) { A[0][k] = ey1[k]; A[1][k] = ey2[k]; A[2][k] = ey3[k]; }
  auto ct = [&](double x1, double x2, double x3, double* o) {
    o[0] = A[0][0] * x1 + A[0][1] * x2 + A[0][2] * x3;
    o[1] = A[1][0] * x1 + A[1][1] * x2 + A[1][2] * x3;
    o[2] = A[2][0] * x1 + A[2][1] * x2 + A[2][2] * x3;
  };
  double yA[3], yAB[3], b[3];
  ct(X - PA[0], Y - PA[1], Z - PA[2], yA);
  ct(side[0], side[1], side[2], yAB);
  const double yB[3] = {yA[0] - yAB[0], yA[1] - yAB[1], yA[2] - yAB[2]};
  ct(bX, bY, bZ, b);
  // configuration I (beta * y1A >= 0) takes the angle -pi + beta
  const double ang = (beta * yA[0] >= 0.0) ? -HBI_PI + beta : beta;
  double vA[6], vB[6], v[6], E[6];
  ang_dis_strain_fsc_d(yA[0], yA[1], yA[2], ang, b[0], b[1], b[2], nu, -PA[2], vA);
  ang_dis_strain_fsc_d(yB[0], yB[1], yB[2], ang, b[0], b[1], b[2], nu, -PB[2], vB);
  for (int k = 0; k < 6; k++) v[k] = vB[k] - vA[k];
  tens_trans_d(v, A, E);
  const double tr = E[0] + E[1] + E[2];
  S[0] = 2 * mu * E[0] + lambda * tr;
  S[1] = 2 * mu * E[1] + lambda * tr;
  S[2] = 2 * mu * E[2] + lambda * tr;
  S[3] = 2 * mu * E[3];
  S[4] = 2 * mu * E[4];
  S[5] = 2 * mu * E[5];
}

// TDstressHS (TDstressFS.f90:7-44, 236-293): main dislocation + its image
// through z = 0 + the harmonic correction of the three edges, half space z <= 0
__device__ __forceinline__ void td_stress_hs(double X, double Y, double Z, const double* P1, const double* P2,
                                             const double* P3, double Ss, double Ds, double Ts, double mu,
                                             double lambda, double* S6) {
  double Sm[6], Si[6], Sh[6], Se[6];
  td_stress_fs(X, Y, Z, P1, P2, P3, Ss, Ds, Ts, mu, lambda, Sm);
  const double Q1[3] = {P1[0], P1[1], -P1[2]}, Q2[3] = {P2[0], P2[1], -P2[2]}, Q3[3] = {P3[0], P3[1], -P3[2]};
  td_stress_fs(X, Y, Z, Q1, Q2, Q3, Ss, Ds, Ts, mu, lambda, Si);
  // slip vector (tensile, strike, dip) from the triangle's frame to x, y, z
  const double a[3] = {P2[0] - P1[0], P2[1] - P1[1], P2[2] - P1[2]}, c[3] = {P3[0] - P1[0], P3[1] - P1[1], P3[2] - P1[2]};
  double Vn[3] = {a[1] * c[2] - c[1] * a[2], a[2] * c[0] - c[2] * a[0], a[0] * c[1] - c[0] * a[1]};
  double s = sqrt(dot3d(Vn, Vn));
  for (int k = 0; k < 3; k++) Vn[k] = Vn[k] / s;
  double Vs[3] = {0.0 * Vn[2] - Vn[1] * 1.0, 1.0 * Vn[0] - Vn[2] * 0.0, 0.0 * Vn[1] - Vn[0] * 0.0};
  s = sqrt(dot3d(Vs, Vs));
  for (int k = 0; k < 3; k++) Vs[k] = Vs[k] / s;
  if (dot3d(Vs, Vs) == 0.0) { Vs[0] = 0.0 * Vn[2]; Vs[1] = 1.0 * Vn[2]; Vs[2] = 0.0 * Vn[2]; }
  s = sqrt(dot3d(Vs, Vs));
  for (int k = 0; k < 3; k++) Vs[k] = Vs[k] / s;
  const double Vd[3] = {Vn[1] * Vs[2] - Vs[1] * Vn[2], Vn[2] * Vs[0] - Vs[2] * Vn[0], Vn[0] * Vs[1] - Vs[0] * Vn[1]};
  const double bx = Ts, by = Ss, bz = Ds;
  const double bX = Vn[0] * bx + Vs[0] * by + Vd[0] * bz;
  const double bY = Vn[1] * bx + Vs[1] * by + Vd[1] * bz;
  const double bZ = Vn[2] * bx + Vs[2] * by + Vd[2] * bz;
  for (int k = 0; k < 6; k++) Sh[k] = 0.0;
  const double* P[4] = {P1, P2, P3, P1};
  for (int e = 0; e < 3; e++) {
    ang_setup_fsc_d(X, Y, Z, bX, bY, bZ, P[e], P[e + 1], mu, lambda, Se);
    for (int k = 0; k < 6; k++) Sh[k] += Se[k];
  }
  for (int k = 0; k < 6; k++) S6[k] = Sm[k] + Si[k] + Sh[k];
}

// matel3dh_ij (m_HACApK_calc_entry_ij.f90:852-898): the source slips along
// its own rake (matel3dn_ij uses the receiver's)
__device__ __forceinline__ double entry_td_hs(const DevBemv& b, int i, int j) {
  const double pois = 0.25, rigid = 32.04;
  const double lambda = 2 * pois / (1 - 2 * pois) * rigid;
  const double P1[3] = {b.xs1[j], b.ys1[j], b.zs1[j]};
  const double P2[3] = {b.xs2[j], b.ys2[j], b.zs2[j]};
  const double P3[3] = {b.xs3[j], b.ys3[j], b.zs3[j]};
  double S[6];
  td_stress_hs(b.xcol[i], b.ycol[i], b.zcol[i], P1, P2, P3, b.crake[j], b.srake[j], 0.0, rigid, lambda, S);
  double A[3][3];
  A[0][0] = b.ev11[i]; A[0][1] = b.ev21[i]; A[0][2] = b.ev31[i];
  A[1][0] = b.ev12[i]; A[1][1] = b.ev22[i]; A[1][2] = b.ev32[i];
  A[2][0] = b.ev13[i]; A[2][1] = b.ev23[i]; A[2][2] = b.ev33[i];
  double p[6];
  tens_trans_d(S, A, p);
  if (b.normal) return -p[2];
  return p[4] * b.crake[i] + p[5] * b.srake[i];
}

// ------------------------------------------------------------------------
// 2D plane strain.  mu = 32.04, nu = 0.25, vs = 3.464, vp = 6 (m_const.f90).

// stress (sxx, syy, sxy) at (X, Y) of an edge dislocation at (xs, ys) with
// unit Burgers vector (s1 glide, s2 climb) in the half space Y >= 0 with a
// free surface at Y = 0 (D2dip2, m_HACApK_calc_entry_ij.f90:145-166)
__device__ __forceinline__ void edge_disl_hs_d(double X, double Y, double xs, double ys, double s1, double s2,
                                               double* o) {
  const double dx = X - xs, ym = Y - ys, yp = Y + ys;
  const double r1 = sqrt(dx * dx + ym * ym), r2 = sqrt(dx * dx + yp * yp);
  const double q1 = r1 * r1 * r1 * r1, q2 = r2 * r2 * r2 * r2, q3 = r2 * r2 * r2 * r2 * r2 * r2;
  const double dx2 = dx * dx, dx4 = dx2 * dx2, ym2 = ym * ym, yp2 = yp * yp, yp3 = yp2 * yp;
  const double c = 32.04 / 2.0 / HBI_PI / (1.0 - 0.25);
  const double gxx = ym * (ym2 + 3 * dx2) / q1 - yp * (yp2 + 3 * dx2) / q2 +
                     2 * ys / q3 * (6 * Y * yp * dx2 - ym * yp3 - dx4);
  const double cxx = dx * (ym2 - dx2) / q1 - dx * (yp2 - dx2) / q2 +
                     4 * ys * dx / q3 * ((2 * ys - Y) * yp2 + (3 * Y + 2 * ys) * dx2);
  const double gyy = ym * (ym2 - dx2) / q1 - yp * (yp2 - dx2) / q2 -
                     2 * ys / q3 * (6 * Y * yp * dx2 - (3 * Y + ys) * yp3 + dx4);
  const double cyy = dx * (3 * ym2 + dx2) / q1 - dx * (3 * yp2 + dx2) / q2 - 4 * ys * dx * Y / q3 * (3 * yp2 - dx2);
  const double gxy = dx * (ym2 - dx2) / q1 - dx * (yp2 - dx2) / q2 + 4 * ys * dx * Y / q3 * (3 * yp2 - dx2);
  const double cxy = ym * (ym2 - dx2) / q1 - yp * (yp2 - dx2) / q2 +
                     2 * ys / q3 * (6 * Y * yp * dx2 - dx4 + (ys - Y) * yp3);
  o[0] = s1 * c * gxx + s2 * c * cxx;
  o[1] = s1 * c * gyy - s2 * c * cyy;
  o[2] = s1 * c * gxy + s2 * c * cxy;
}

// matel2dph2_ij (:92-116): unit slip along element j (dip ang(j)), traction
// on receiver i's plane; the per-element cos/sin come from the tables
__device__ __forceinline__ double entry_2dph(const DevBemv& b, int i, int j) {
  const double s1 = b.cang[j], s2 = b.sang[j];
  double p[3], q[3];
  edge_disl_hs_d(b.xcol[i], b.ycol[i], b.xel[j], b.yel[j], s1, s2, p);
  edge_disl_hs_d(b.xcol[i], b.ycol[i], b.xer[j], b.yer[j], s1, s2, q);
  const double sxx = p[0] - q[0], syy = p[1] - q[1], sxy = p[2] - q[2];
  const double c2 = b.cang2[i], s2i = b.sang2[i];  // cos, sin of 2 ang(i)
  if (b.normal) return -0.5 * (sxx + syy) + 0.5 * (sxx - syy) * c2 + sxy * s2i;
  return -0.5 * (sxx - syy) * s2i + sxy * c2;
}

// inte11s / inte12s / inte22s (:697-722) at one dislocation end
__device__ __forceinline__ void plane_kernel_d(double x1, double x2, double* k) {
  const double r = sqrt(x1 * x1 + x2 * x2);
  const double r4 = r * r * r * r;
  const double pa = 3.464 / 6.0;
  k[0] = -2 * 3.464 / HBI_PI * (1 - pa * pa) * x2 * (3 * x1 * x1 + x2 * x2) / r4;
  k[1] = 2 * 3.464 / HBI_PI * (1 - pa * pa) * x1 * (x1 * x1 - x2 * x2) / r4;
  k[2] = 2 * 3.464 / HBI_PI * (1 - pa * pa) * x2 * (x1 * x1 - x2 * x2) / r4;
}

// tensor2d_ij (:300-339), md = 's': full space
__device__ __forceinline__ double entry_2dn(const DevBemv& b, int i, int j) {
  const double cj = b.cang[j], sj = b.sang[j];
  const double dxl = b.xcol[i] - b.xel[j], dyl = b.ycol[i] - b.yel[j];
  const double dxr = b.xcol[i] - b.xer[j], dyr = b.ycol[i] - b.yer[j];
  double kl[3], kr[3];
  plane_kernel_d(cj * dxl + sj * dyl, -sj * dxl + cj * dyl, kl);
  plane_kernel_d(cj * dxr + sj * dyr, -sj * dxr + cj * dyr, kr);
  const double g = -0.5 * 32.04 / 3.464;
  const double k11 = g * (kl[0] - kr[0]), k12 = g * (kl[1] - kr[1]), k22 = g * (kl[2] - kr[2]);
  // rotation by -2 ang(j) to x, y: cos(-2a) = cos 2a, sin(-2a) = -sin 2a
  const double c2 = b.cang2[j], s2 = -b.sang2[j];
  const double sxx = 0.5 * (k11 + k22) + 0.5 * (k11 - k22) * c2 + k12 * s2;
  const double sxy = -0.5 * (k11 - k22) * s2 + k12 * c2;
  const double syy = 0.5 * (k11 + k22) - 0.5 * (k11 - k22) * c2 - k12 * s2;
  const double ci = b.cang2[i], si = b.sang2[i];
  if (b.normal) return -(0.5 * (sxx + syy) - 0.5 * (sxx - syy) * ci - sxy * si);
  return -0.5 * (sxx - syy) * si + sxy * ci;
}

// 0-based element ids
template <int PROB>
__device__ __forceinline__ double entry(const DevBemv& b, int i, int j) {
  if (PROB == P_2DVS) return entry_2dvs(b, i, j);
  if (PROB == P_3DPH) return entry_okada(b, i, j, false);
  if (PROB == P_3DNR) return entry_okada(b, i, j, true);
  if (PROB == P_2DPH) return entry_2dph(b, i, j);
  if (PROB == P_2DN) return entry_2dn(b, i, j);
  if (PROB == P_3DHT) return entry_td_hs(b, i, j);
  return entry_td(b, i, j);
}

}  // namespace hbi
