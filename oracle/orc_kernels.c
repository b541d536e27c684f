/*
 * orc_kernels.c -- oracle restatement of the Green's-function entries on the
 * hot path.  TEST INFRASTRUCTURE ONLY (see hbi_oracle.h).
 *
 *   HACApK_entry_ij dispatch          m_HACApK_calc_entry_ij.f90:24-90
 *   matels2dpa_ij ('2dvs')            m_HACApK_calc_entry_ij.f90:685-695, :55-57
 *   okada_ij ('3dph','3dnr')          m_HACApK_calc_entry_ij.f90:1065-1145
 *   okada / ua / ub / uc              okada.f90:10-597
 *   matel3dn_ij ('3dnt')              m_HACApK_calc_entry_ij.f90:802-851
 *   TDstressFS, TDSetupD, AngDisStrain, TensTrans, CoordTrans,
 *   trimodefinder, DCross             TDstressFS.f90:45-235, 295-403, 560-627, 1012-1019
 *   constants                         m_const.f90:1-11
 *
 * Expressions keep the reference's left-to-right evaluation order; x**2 is
 * x*x and y**3 is (y*y)*y, as a Fortran compiler expands integer powers.
 */
#include "hbi_oracle.h"
#include <math.h>

#define PI (4 * atan(1.0))
static const double POIS = 0.25, RIGID = 32.04;

/* ---------------- 2D antiplane, half space ---------------- */
static double matels2dpa(int i, int j, const double* xcol, double xel_j, double xer_j) {
  double factor = RIGID / (2.0 * PI);
  return factor * (1.0 / (xcol[i] - xer_j) - 1.0 / (xcol[i] - xel_j));
}

/* ---------------- tensor helpers ---------------- */
/* TensTrans (TDstressFS.f90:295-314); A is A(row,col) -> A[row-1][col-1] */
static void tens_trans(double Txx1, double Tyy1, double Tzz1, double Txy1, double Txz1,
                       double Tyz1, const double A[3][3], double* o) {
#define a(r, c) A[(r)-1][(c)-1]
  o[0] = a(1,1)*a(1,1)*Txx1 + 2*a(1,1)*a(2,1)*Txy1 + 2*a(1,1)*a(3,1)*Txz1 + 2*a(2,1)*a(3,1)*Tyz1 +
         a(2,1)*a(2,1)*Tyy1 + a(3,1)*a(3,1)*Tzz1;
  o[1] = a(1,2)*a(1,2)*Txx1 + 2*a(1,2)*a(2,2)*Txy1 + 2*a(1,2)*a(3,2)*Txz1 + 2*a(2,2)*a(3,2)*Tyz1 +
         a(2,2)*a(2,2)*Tyy1 + a(3,2)*a(3,2)*Tzz1;
  o[2] = a(1,3)*a(1,3)*Txx1 + 2*a(1,3)*a(2,3)*Txy1 + 2*a(1,3)*a(3,3)*Txz1 + 2*a(2,3)*a(3,3)*Tyz1 +
         a(2,3)*a(2,3)*Tyy1 + a(3,3)*a(3,3)*Tzz1;
  o[3] = a(1,1)*a(1,2)*Txx1 + (a(1,1)*a(2,2) + a(2,1)*a(1,2))*Txy1 + (a(1,1)*a(3,2) + a(1,2)*a(3,1))*Txz1 +
         (a(3,2)*a(2,1) + a(3,1)*a(2,2))*Tyz1 + a(2,2)*a(2,1)*Tyy1 + a(3,1)*a(3,2)*Tzz1;
  o[4] = a(1,1)*a(1,3)*Txx1 + (a(1,1)*a(2,3) + a(1,3)*a(2,1))*Txy1 + (a(1,1)*a(3,3) + a(3,1)*a(1,3))*Txz1 +
         (a(3,3)*a(2,1) + a(3,1)*a(2,3))*Tyz1 + a(2,3)*a(2,1)*Tyy1 + a(3,1)*a(3,3)*Tzz1;
  o[5] = a(1,2)*a(1,3)*Txx1 + (a(1,3)*a(2,2) + a(1,2)*a(2,3))*Txy1 + (a(1,3)*a(3,2) + a(1,2)*a(3,3))*Txz1 +
         (a(2,3)*a(3,2) + a(3,3)*a(2,2))*Tyz1 + a(2,2)*a(2,3)*Tyy1 + a(3,2)*a(3,3)*Tzz1;
#undef a
}

/* ---------------- Okada (1992) ---------------- */
typedef struct {
  double xi2, et2, q2, r, r2, r3, r5, yp, d, tt, alx, ale, x11, y11, x32, y32, ey, ez, fy, fz, gy,
      gz, hy, hz, rxi, ret;
} dccon_t;

static void dccon(double xi, double et, double q, double sd, double cd, dccon_t* c) {
  c->xi2 = xi * xi; c->et2 = et * et; c->q2 = q * q;
  c->r2 = c->xi2 + c->et2 + c->q2;
  c->r = sqrt(c->r2);
  c->r3 = c->r * c->r2;
  c->r5 = c->r3 * c->r2;
  c->yp = et * cd + q * sd;
  c->d = et * sd - q * cd;
  c->tt = atan(xi * et / (q * c->r));
  c->rxi = c->r + xi;
  c->alx = log(c->rxi);
  c->x11 = 1.0 / (c->r * c->rxi);
  c->x32 = (c->r + c->rxi) * c->x11 * c->x11 / c->r;
  c->ret = c->r + et;
  c->ale = log(c->ret);
  c->y11 = 1.0 / (c->r * c->ret);
  c->y32 = (c->r + c->ret) * c->y11 * c->y11 / c->r;
  c->ey = sd / c->r - c->yp * q / c->r3;
  c->ez = cd / c->r + c->d * q / c->r3;
  c->fy = c->d / c->r3 + c->xi2 * c->y32 * sd;
  c->fz = c->yp / c->r3 + c->xi2 * c->y32 * cd;
  c->gy = 2.0 * c->x11 * sd - c->yp * q * c->x32;
  c->gz = 2.0 * c->x11 * cd + c->d * q * c->x32;
  c->hy = c->d * q * c->x32 + xi * q * c->y32 * sd;
  c->hz = c->yp * q * c->x32 + xi * q * c->y32 * cd;
}

/* ua (okada.f90:227-332) */
static void okada_ua(double xi, double et, double q, double sd, double cd, double disl1,
                     double disl2, double alpha, double* dua) {
  const double pi2 = 8.0 * atan(1.0);
  double alp1 = (1.0 - alpha) / 2.0, alp2 = alpha / 2.0;
  dccon_t c; dccon(xi, et, q, sd, cd, &c);
  double du[12];
  for (int i = 0; i < 12; i++) dua[i] = 0.0;
  double xy = xi * c.y11, qx = q * c.x11, qy = q * c.y11;
  du[0] = c.tt / 2.0 + alp2 * xi * qy;
  du[1] = alp2 * q / c.r;
  du[2] = alp1 * c.ale - alp2 * q * qy;
  du[3] = -alp1 * qy - alp2 * c.xi2 * q * c.y32;
  du[4] = -alp2 * xi * q / c.r3;
  du[5] = alp1 * xy + alp2 * xi * c.q2 * c.y32;
  du[6] = alp1 * xy * sd + alp2 * xi * c.fy + c.d / 2.0 * c.x11;
  du[7] = alp2 * c.ey;
  du[8] = alp1 * (cd / c.r + qy * sd) - alp2 * q * c.fy;
  du[9] = alp1 * xy * cd + alp2 * xi * c.fz + c.yp / 2.0 * c.x11;
  du[10] = alp2 * c.ez;
  du[11] = -alp1 * (sd / c.r - qy * cd) - alp2 * q * c.fz;
  for (int i = 0; i < 12; i++) dua[i] = dua[i] + disl1 / pi2 * du[i];
  du[0] = alp2 * q / c.r;
  du[1] = c.tt / 2.0 + alp2 * et * qx;
  du[2] = alp1 * c.alx - alp2 * q * qx;
  du[3] = -alp2 * xi * q / c.r3;
  du[4] = -qy / 2.0 - alp2 * et * q / c.r3;
  du[5] = alp1 / c.r + alp2 * c.q2 / c.r3;
  du[6] = alp2 * c.ey;
  du[7] = alp1 * c.d * c.x11 + xy / 2.0 * sd + alp2 * et * c.gy;
  du[8] = alp1 * c.yp * c.x11 - alp2 * q * c.gy;
  du[9] = alp2 * c.ez;
  du[10] = alp1 * c.yp * c.x11 + xy / 2.0 * cd + alp2 * et * c.gz;
  du[11] = -alp1 * c.d * c.x11 - alp2 * q * c.gz;
  for (int i = 0; i < 12; i++) dua[i] = dua[i] + disl2 / pi2 * du[i];
}

/* ub (okada.f90:333-475) */
static void okada_ub(double xi, double et, double q, double sd, double cd, double disl1,
                     double disl2, double alpha, double* dub) {
  const double pi2 = 8.0 * atan(1.0);
  double alp3 = (1.0 - alpha) / alpha;
  dccon_t c; dccon(xi, et, q, sd, cd, &c);
  double rd = c.r + c.d;
  double d11 = 1.0 / (c.r * rd);
  double aj2 = xi * c.yp / rd * d11;
  double aj5 = -(c.d + c.yp * c.yp / rd) * d11;
  double ai3, ai4, ak1, ak3, aj3, aj6;
  if (cd != 0.0) {
    if (xi == 0.0) ai4 = 0.0;
    else {
      double xs = sqrt(c.xi2 + c.q2);
      ai4 = 1.0 / cd / cd * (xi / rd * sd * cd +
                             2.0 * atan((et * (xs + q * cd) + xs * (c.r + xs) * sd) / (xi * (c.r + xs) * cd)));
    }
    ai3 = (c.yp * cd / rd - c.ale + sd * log(rd)) / cd / cd;
    ak1 = xi * (d11 - c.y11 * sd) / cd;
    ak3 = (q * c.y11 - c.yp * d11) / cd;
    aj3 = (ak1 - aj2 * sd) / cd;
    aj6 = (ak3 - aj5 * sd) / cd;
  } else {
    double rd2 = rd * rd;
    ai3 = (et / rd + c.yp * q / rd2 - c.ale) / 2.0;
    ai4 = xi * c.yp / rd2 / 2.0;
    ak1 = xi * q / rd * d11;
    ak3 = sd / rd * (c.xi2 * d11 - 1.0);
    aj3 = -xi / rd2 * (c.q2 * d11 - 1.0 / 2.0);
    aj6 = -c.yp / rd2 * (c.xi2 * d11 - 1.0 / 2.0);
  }
  double xy = xi * c.y11;
  double ai1 = -xi / rd * cd - ai4 * sd;
  double ai2 = log(rd) + ai3 * sd;
  double ak2 = 1.0 / c.r + ak3 * sd;
  double ak4 = xy * cd - ak1 * sd;
  double aj1 = aj5 * cd - aj6 * sd;
  double aj4 = -xy - aj2 * cd + aj3 * sd;
  double du[12];
  for (int i = 0; i < 12; i++) dub[i] = 0.0;
  double qx = q * c.x11, qy = q * c.y11;
  du[0] = -xi * qy - c.tt - alp3 * ai1 * sd;
  du[1] = -q / c.r + alp3 * c.yp / rd * sd;
  du[2] = q * qy - alp3 * ai2 * sd;
  du[3] = c.xi2 * q * c.y32 - alp3 * aj1 * sd;
  du[4] = xi * q / c.r3 - alp3 * aj2 * sd;
  du[5] = -xi * c.q2 * c.y32 - alp3 * aj3 * sd;
  du[6] = -xi * c.fy - c.d * c.x11 + alp3 * (xy + aj4) * sd;
  du[7] = -c.ey + alp3 * (1.0 / c.r + aj5) * sd;
  du[8] = q * c.fy - alp3 * (qy - aj6) * sd;
  du[9] = -xi * c.fz - c.yp * c.x11 + alp3 * ak1 * sd;
  du[10] = -c.ez + alp3 * c.yp * d11 * sd;
  du[11] = q * c.fz + alp3 * ak2 * sd;
  for (int i = 0; i < 12; i++) dub[i] = dub[i] + disl1 / pi2 * du[i];
  du[0] = -q / c.r + alp3 * ai3 * sd * cd;
  du[1] = -et * qx - c.tt - alp3 * xi / rd * sd * cd;
  du[2] = q * qx + alp3 * ai4 * sd * cd;
  du[3] = xi * q / c.r3 + alp3 * aj4 * sd * cd;
  du[4] = et * q / c.r3 + qy + alp3 * aj5 * sd * cd;
  du[5] = -c.q2 / c.r3 + alp3 * aj6 * sd * cd;
  du[6] = -c.ey + alp3 * aj1 * sd * cd;
  du[7] = -et * c.gy - xy * sd + alp3 * aj2 * sd * cd;
  du[8] = q * c.gy + alp3 * aj3 * sd * cd;
  du[9] = -c.ez - alp3 * ak3 * sd * cd;
  du[10] = -et * c.gz - xy * cd - alp3 * xi * d11 * sd * cd;
  du[11] = q * c.gz - alp3 * ak4 * sd * cd;
  for (int i = 0; i < 12; i++) dub[i] = dub[i] + disl2 / pi2 * du[i];
}

/* uc (okada.f90:476-597) */
static void okada_uc(double xi, double et, double q, double z, double sd, double cd, double disl1,
                     double disl2, double alpha, double* duc) {
  const double pi2 = 8.0 * atan(1.0);
  double alp4 = 1.0 - alpha, alp5 = alpha;
  dccon_t cc; dccon(xi, et, q, sd, cd, &cc);
  double r = cc.r, r2 = cc.r2, r3 = cc.r3, r5 = cc.r5, d = cc.d, yp = cc.yp;
  double x11 = cc.x11, y11 = cc.y11, x32 = cc.x32, y32 = cc.y32, xi2 = cc.xi2, et2 = cc.et2, q2 = cc.q2;
  double c = d + z;
  double x53 = (8.0 * r2 + 9.0 * r * xi + 3.0 * xi2) * x11 * x11 * x11 / r2;
  double y53 = (8.0 * r2 + 9.0 * r * et + 3.0 * et2) * y11 * y11 * y11 / r2;
  double h = q * cd - z;
  double z32 = sd / r3 - h * y32;
  double z53 = 3.0 * sd / r5 - h * y53;
  double y0 = y11 - xi2 * y32;
  double z0 = z32 - xi2 * z53;
  double ppy = cd / r3 + q * y32 * sd;
  double ppz = sd / r3 - q * y32 * cd;
  double qq = z * y32 + z32 + z0;
  double qqy = 3.0 * c * d / r5 - qq * sd;
  double qqz = 3.0 * c * yp / r5 - qq * cd + q * y32;
  double xy = xi * y11, qy = q * y11;
  double qr = 3.0 * q / r5;
  double cdr = (c + d) / r3;
  double yy0 = yp / r3 - y0 * cd;
  double du[12];
  for (int i = 0; i < 12; i++) duc[i] = 0.0;
  du[0] = alp4 * xy * cd - alp5 * xi * q * z32;
  du[1] = alp4 * (cd / r + 2.0 * qy * sd) - alp5 * c * q / r3;
  du[2] = alp4 * qy * cd - alp5 * (c * et / r3 - z * y11 + xi2 * z32);
  du[3] = alp4 * y0 * cd - alp5 * q * z0;
  du[4] = -alp4 * xi * (cd / r3 + 2.0 * q * y32 * sd) + alp5 * c * xi * qr;
  du[5] = -alp4 * xi * q * y32 * cd + alp5 * xi * (3.0 * c * et / r5 - qq);
  du[6] = -alp4 * xi * ppy * cd - alp5 * xi * qqy;
  du[7] = alp4 * 2.0 * (d / r3 - y0 * sd) * sd - yp / r3 * cd - alp5 * (cdr * sd - et / r3 - c * yp * qr);
  du[8] = -alp4 * q / r3 + yy0 * sd + alp5 * (cdr * cd + c * d * qr - (y0 * cd + q * z0) * sd);
  du[9] = alp4 * xi * ppz * cd - alp5 * xi * qqz;
  du[10] = alp4 * 2.0 * (yp / r3 - y0 * cd) * sd + d / r3 * cd - alp5 * (cdr * cd + c * d * qr);
  du[11] = yy0 * cd - alp5 * (cdr * sd - c * yp * qr - y0 * sd * sd + q * z0 * cd);
  for (int i = 0; i < 12; i++) duc[i] = duc[i] + disl1 / pi2 * du[i];
  du[0] = alp4 * cd / r - qy * sd - alp5 * c * q / r3;
  du[1] = alp4 * yp * x11 - alp5 * c * et * q * x32;
  du[2] = -d * x11 - xy * sd - alp5 * c * (x11 - q2 * x32);
  du[3] = -alp4 * xi / r3 * cd + alp5 * c * xi * qr + xi * q * y32 * sd;
  du[4] = -alp4 * yp / r3 + alp5 * c * et * qr;
  du[5] = d / r3 - y0 * sd + alp5 * c / r3 * (1.0 - 3.0 * q2 / r2);
  du[6] = -alp4 * et / r3 + y0 * sd * sd - alp5 * (cdr * sd - c * yp * qr);
  du[7] = alp4 * (x11 - yp * yp * x32) - alp5 * c * ((d + 2.0 * q * cd) * x32 - yp * et * q * x53);
  du[8] = xi * ppy * sd + yp * d * x32 + alp5 * c * ((yp + 2.0 * q * sd) * x32 - yp * q2 * x53);
  du[9] = -q / r3 + y0 * sd * cd - alp5 * (cdr * cd + c * d * qr);
  du[10] = alp4 * yp * d * x32 - alp5 * c * ((yp - 2.0 * q * sd) * x32 + d * et * q * x53);
  du[11] = -xi * ppz * sd + x11 - d * d * x32 - alp5 * c * ((d - 2.0 * q * cd) * x32 - d * q2 * x53);
  for (int i = 0; i < 12; i++) duc[i] = duc[i] + disl2 / pi2 * du[i];
}

/* okada (okada.f90:10-226) -> u(1:12) = ux,uy,uz,uxx,uyx,uzx,uxy,uyy,uzy,uxz,uyz,uzz */
void orc_okada(double alpha, double x, double y, double z, double depth, double dip, double al1,
               double al2, double aw1, double aw2, double disl1, double disl2, double disl3,
               double* u, int fullspace) {
  (void)disl3;
  const double pi2 = 8.0 * atan(1.0), epso = 1e-6;
  double p18 = pi2 / 360.0;
  double sd = sin(dip * p18), cd = cos(dip * p18);
  if (fabs(cd) < epso) {
    cd = 0.0;
    if (sd > 0.0) sd = 1.0;
    if (sd < 0.0) sd = -1.0;
  }
  double xi[2] = {x - al1, x - al2};
  double d = depth + z;
  double p = y * cd + d * sd;
  double q = y * sd - d * cd;
  double et[2] = {p - aw1, p - aw2};
  double du[12], dua[12], dub[12], duc[12];
  for (int i = 0; i < 12; i++) u[i] = 0.0;
  for (int k = 1; k <= 2; k++)
    for (int j = 1; j <= 2; j++) {
      okada_ua(xi[j - 1], et[k - 1], q, sd, cd, disl1, disl2, alpha, dua);
      du[0] = -dua[0];
      du[1] = -dua[1] * cd + dua[2] * sd;
      du[2] = -dua[1] * sd - dua[2] * cd;
      du[3] = -dua[3];
      du[4] = -dua[4] * cd + dua[5] * sd;
      du[5] = -dua[4] * sd - dua[5] * cd;
      du[6] = -dua[6];
      du[7] = -dua[7] * cd + dua[8] * sd;
      du[8] = -dua[7] * sd - dua[8] * cd;
      du[9] = dua[9];
      du[10] = dua[10] * cd - dua[11] * sd;
      du[11] = dua[10] * sd + dua[11] * cd;
      for (int i = 0; i < 12; i++) {
        if (j + k != 3) u[i] = u[i] + du[i];
        if (j + k == 3) u[i] = u[i] - du[i];
      }
    }
  if (fullspace) return;
  d = depth - z;
  p = y * cd + d * sd;
  q = y * sd - d * cd;
  et[0] = p - aw1; et[1] = p - aw2;
  for (int k = 1; k <= 2; k++)
    for (int j = 1; j <= 2; j++) {
      okada_ua(xi[j - 1], et[k - 1], q, sd, cd, disl1, disl2, alpha, dua);
      okada_ub(xi[j - 1], et[k - 1], q, sd, cd, disl1, disl2, alpha, dub);
      okada_uc(xi[j - 1], et[k - 1], q, z, sd, cd, disl1, disl2, alpha, duc);
      du[0] = dua[0] + dub[0] + z * duc[0];
      du[1] = (dua[1] + dub[1] + z * duc[1]) * cd - (dua[2] + dub[2] + z * duc[2]) * sd;
      du[2] = (dua[1] + dub[1] - z * duc[1]) * sd + (dua[2] + dub[2] - z * duc[2]) * cd;
      du[3] = dua[3] + dub[3] + z * duc[3];
      du[4] = (dua[4] + dub[4] + z * duc[4]) * cd - (dua[5] + dub[5] + z * duc[5]) * sd;
      du[5] = (dua[4] + dub[4] - z * duc[4]) * sd + (dua[5] + dub[5] - z * duc[5]) * cd;
      du[6] = dua[6] + dub[6] + z * duc[6];
      du[7] = (dua[7] + dub[7] + z * duc[7]) * cd - (dua[8] + dub[8] + z * duc[8]) * sd;
      du[8] = (dua[7] + dub[7] - z * duc[7]) * sd + (dua[8] + dub[8] - z * duc[8]) * cd;
      du[9] = dua[9] + dub[9] + z * duc[9];
      du[10] = (dua[10] + dub[10] + z * duc[10]) * cd - (dua[11] + dub[11] + z * duc[11]) * sd;
      du[11] = (dua[10] + dub[10] - z * duc[10]) * sd + (dua[11] + dub[11] - z * duc[11]) * cd;
      du[9] = du[9] + duc[0];
      du[10] = du[10] + duc[1] * cd - duc[2] * sd;
      du[11] = du[11] - duc[1] * sd - duc[2] * cd;
      for (int i = 0; i < 12; i++) {
        if (j + k != 3) u[i] = u[i] + du[i];
        if (j + k == 3) u[i] = u[i] - du[i];
      }
    }
}

/* okada_ij (m_HACApK_calc_entry_ij.f90:1065-1145); i,j 0-based here */
static double okada_ij(int i, int j, const orc_bemv* b, int fullspace) {
  double alpha = (1.0 + (0.5 / POIS - 1.0)) / (1.0 + 2.0 * (0.5 / POIS - 1.0));
  double dx = cos(b->ang[j]) * (b->xcol[i] - b->xcol[j]) + sin(b->ang[j]) * (b->ycol[i] - b->ycol[j]);
  double dy = -sin(b->ang[j]) * (b->xcol[i] - b->xcol[j]) + cos(b->ang[j]) * (b->ycol[i] - b->ycol[j]);
  double w = b->w;
  double z = b->zcol[i];
  double depth = -b->zcol[j];
  double dip = b->angd[j] * 180 / PI;
  double rs = b->dsl[j] / w;
  double rd = b->dsd[j] / w;
  double u[12];
  orc_okada(alpha, dx / w, dy / w, z / w, depth / w, dip, -0.5 * rs, 0.5 * rs, -0.5 * rd, 0.5 * rd,
            -cos(b->rake[j]), -sin(b->rake[j]), 0.0, u, fullspace);
  double uxx = u[3], uyx = u[4], uzx = u[5], uxy = u[6], uyy = u[7], uzy = u[8], uxz = u[9],
         uyz = u[10], uzz = u[11];
  double exx = uxx, eyy = uyy, ezz = uzz;
  double exy = 0.5 * (uxy + uyx), eyz = 0.5 * (uyz + uzy), ezx = 0.5 * (uzx + uxz);
  double sxx = RIGID * (exx + eyy + ezz) + 2 * RIGID * exx;
  double syy = RIGID * (exx + eyy + ezz) + 2 * RIGID * eyy;
  double szz = RIGID * (exx + eyy + ezz) + 2 * RIGID * ezz;
  double sxy = 2 * RIGID * exy, sxz = 2 * RIGID * ezx, syz = 2 * RIGID * eyz;
  double rotang = b->ang[j] - b->ang[i];
  double dpang = b->angd[i];
  double A[3][3];
  A[0][0] = cos(rotang); A[1][0] = -sin(rotang); A[2][0] = 0.0;
  A[0][1] = sin(rotang) * cos(dpang); A[1][1] = cos(rotang) * cos(dpang); A[2][1] = sin(dpang);
  A[0][2] = sin(rotang) * sin(dpang); A[1][2] = cos(rotang) * sin(dpang); A[2][2] = -cos(dpang);
  double p[6];
  tens_trans(sxx, syy, szz, sxy, sxz, syz, (const double(*)[3])A, p);
  if (b->v == 'n') return p[2];
  return p[4] * cos(b->rake[i]) + p[5] * sin(b->rake[i]);
}

/* ---------------- Nikkhoo & Walter triangular dislocation ---------------- */
static void dcross(const double* v1, const double* v2, double* v3) {
  v3[0] = v1[1] * v2[2] - v2[1] * v1[2];
  v3[1] = v1[2] * v2[0] - v2[2] * v1[0];
  v3[2] = v1[0] * v2[1] - v2[0] * v1[1];
}
static double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

static void coord_trans(double x1, double x2, double x3, const double A[3][3], double* o) {
  o[0] = A[0][0] * x1 + A[0][1] * x2 + A[0][2] * x3;
  o[1] = A[1][0] * x1 + A[1][1] * x2 + A[1][2] * x3;
  o[2] = A[2][0] * x1 + A[2][1] * x2 + A[2][2] * x3;
}

/* trimodefinder (TDstressFS.f90:329-350); p* are 2-vectors */
static int trimodefinder(double x, double y, double z, const double* p1, const double* p2,
                         const double* p3) {
  double den = (p2[1] - p3[1]) * (p1[0] - p3[0]) + (p3[0] - p2[0]) * (p1[1] - p3[1]);
  double a = ((p2[1] - p3[1]) * (x - p3[0]) + (p3[0] - p2[0]) * (y - p3[1])) / den;
  double b = ((p3[1] - p1[1]) * (x - p3[0]) + (p1[0] - p3[0]) * (y - p3[1])) / den;
  double c = 1.0 - a - b;
  int t = 1;
  if ((a <= 0.0) && (b > c) && (c > a)) t = -1;
  if ((b <= 0.0) && (c > a) && (a > b)) t = -1;
  if ((c <= 0.0) && (a > b) && (b > c)) t = -1;
  if ((a == 0.0) && (b >= 0.0) && (c >= 0.0)) t = 0;
  if ((a >= 0.0) && (b == 0.0) && (c >= 0.0)) t = 0;
  if ((a >= 0.0) && (b >= 0.0) && (c == 0.0)) t = 0;
  if ((t == 0) && (z != 0.0)) t = 1;
  return t;
}

/* AngDisStrain (TDstressFS.f90:560-627) */
static void ang_dis_strain(double x, double y, double z, double alpha, double bx, double by,
                           double bz, double nu, double* E) {
  const double pi = 4 * atan(1.0);
  double sinA = sin(alpha), cosA = cos(alpha);
  double eta = y * cosA - z * sinA;
  double zeta = y * sinA + z * cosA;
  double x2 = x * x, y2 = y * y, z2 = z * z;
  double r2 = x2 + y2 + z2;
  double r = sqrt(r2);
  double r3 = r * r2;
  double rz = r * (r - z);
  double r2z2 = r2 * ((r - z) * (r - z));
  double r3z = r3 * (r - z);
  double W = zeta - r;
  double W2 = W * W;
  double Wr = W * r;
  double W2r = W2 * r;
  double Wr3 = W * r3;
  double W2r2 = W2 * r2;
  double C = (r * cosA - z) / Wr;
  double S = (r * sinA - y) / Wr;
  double rFi_rx = (eta / r / (r - zeta) - y / r / (r - z)) / 4 / pi;
  double rFi_ry = (x / r / (r - z) - cosA * x / r / (r - zeta)) / 4 / pi;
  double rFi_rz = (sinA * x / r / (r - zeta)) / 4 / pi;
  double y3 = y * y * y;

  E[0] = bx * (rFi_rx) + bx / 8 / pi / (1 - nu) * (eta / Wr + eta * x2 / W2r2 - eta * x2 / Wr3 + y / rz -
          x2 * y / r2z2 - x2 * y / r3z) - by * x / 8 / pi / (1 - nu) * (((2 * nu + 1) / Wr + x2 / W2r2 - x2 / Wr3) * cosA +
          (2 * nu + 1) / rz - x2 / r2z2 - x2 / r3z) + bz * x * sinA / 8 / pi / (1 - nu) * ((2 * nu + 1) / Wr + x2 / W2r2 - x2 / Wr3);

  E[1] = by * (rFi_ry) + bx / 8 / pi / (1 - nu) * ((1 / Wr + S * S - y2 / Wr3) * eta + (2 * nu + 1) * y / rz - y3 / r2z2 -
          y3 / r3z - 2 * nu * cosA * S) - by * x / 8 / pi / (1 - nu) * (1 / rz - y2 / r2z2 - y2 / r3z +
          (1 / Wr + S * S - y2 / Wr3) * cosA) + bz * x * sinA / 8 / pi / (1 - nu) * (1 / Wr + S * S - y2 / Wr3);

  E[2] = bz * (rFi_rz) + bx / 8 / pi / (1 - nu) * (eta / W / r + eta * C * C - eta * z2 / Wr3 + y * z / r3 +
          2 * nu * sinA * C) - by * x / 8 / pi / (1 - nu) * ((1 / Wr + C * C - z2 / Wr3) * cosA + z / r3) +
          bz * x * sinA / 8 / pi / (1 - nu) * (1 / Wr + C * C - z2 / Wr3);

  E[3] = bx * (rFi_ry) / 2 + by * (rFi_rx) / 2 - bx / 8 / pi / (1 - nu) * (x * y2 / r2z2 - nu * x / rz +
          x * y2 / r3z - nu * x * cosA / Wr + eta * x * S / Wr + eta * x * y / Wr3) +
          by / 8 / pi / (1 - nu) * (x2 * y / r2z2 - nu * y / rz + x2 * y / r3z + nu * cosA * S +
          x2 * y * cosA / Wr3 + x2 * cosA * S / Wr) - bz * sinA / 8 / pi / (1 - nu) * (nu * S + x2 * S / Wr + x2 * y / Wr3);

  E[4] = bx * (rFi_rz) / 2 + bz * (rFi_rx) / 2 - bx / 8 / pi / (1 - nu) * (-x * y / r3 + nu * x * sinA / Wr + eta * x * C / Wr +
          eta * x * z / Wr3) + by / 8 / pi / (1 - nu) * (-x2 / r3 + nu / r + nu * cosA * C + x2 * z * cosA / Wr3 +
          x2 * cosA * C / Wr) - bz * sinA / 8 / pi / (1 - nu) * (nu * C + x2 * C / Wr + x2 * z / Wr3);

  E[5] = by * (rFi_rz) / 2 + bz * (rFi_ry) / 2 + bx / 8 / pi / (1 - nu) * (y2 / r3 - nu / r - nu * cosA * C +
          nu * sinA * S + eta * sinA * cosA / W2 - eta * (y * cosA + z * sinA) / W2r + eta * y * z / W2r2 - eta * y * z / Wr3) -
          by * x / 8 / pi / (1 - nu) * (y / r3 + sinA * (cosA * cosA) / W2 - cosA * (y * cosA + z * sinA) /
          W2r + y * z * cosA / W2r2 - y * z * cosA / Wr3) - bz * x * sinA / 8 / pi / (1 - nu) *
          (y * z / Wr3 - sinA * cosA / W2 + (y * cosA + z * sinA) / W2r - y * z / W2r2);
}

/* TDSetupD (TDstressFS.f90:352-403) */
static void td_setup_d(double x, double y, double z, double alpha, double bx, double by, double bz,
                       double nu, const double* TriVertex, const double* SideVec, double* E) {
  const double pi = 4 * atan(1.0);
  double A11 = SideVec[2], A12 = -SideVec[1], A21 = SideVec[1], A22 = SideVec[2];
  double y1 = A11 * (y - TriVertex[1]) + A12 * (z - TriVertex[2]);
  double z1 = A21 * (y - TriVertex[1]) + A22 * (z - TriVertex[2]);
  double by1 = A11 * by + A12 * bz;
  double bz1 = A21 * by + A22 * bz;
  double e[6];
  ang_dis_strain(x, y1, z1, -pi + alpha, bx, by1, bz1, nu, e);
  double B[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  B[0][0] = 1; B[1][1] = A11; B[1][2] = A12; B[2][1] = A21; B[2][2] = A22;
  tens_trans(e[0], e[1], e[2], e[3], e[4], e[5], (const double(*)[3])B, E);
}

/* TDstressFS (TDstressFS.f90:45-235) -> S6 = Sxx,Syy,Szz,Sxy,Sxz,Syz */
void orc_tdstressfs(double X, double Y, double Z, const double* P1, const double* P2,
                    const double* P3, double Ss, double Ds, double Ts, double mu, double lambda,
                    double* S6) {
  double nu = 1 / (1 + lambda / mu) / 2;
  double bx = Ts, by = Ss, bz = Ds;
  double P2mP1[3], P3mP1[3], Vnorm[3], Vstrike[3], Vdip[3];
  for (int k = 0; k < 3; k++) { P2mP1[k] = P2[k] - P1[k]; P3mP1[k] = P3[k] - P1[k]; }
  dcross(P2mP1, P3mP1, Vnorm);
  double s = sqrt(dot3(Vnorm, Vnorm));
  for (int k = 0; k < 3; k++) Vnorm[k] = Vnorm[k] / s;
  const double eY[3] = {0.0, 1.0, 0.0}, eZ[3] = {0.0, 0.0, 1.0};
  dcross(eZ, Vnorm, Vstrike);
  s = sqrt(dot3(Vstrike, Vstrike));
  for (int k = 0; k < 3; k++) Vstrike[k] = Vstrike[k] / s;
  if (dot3(Vstrike, Vstrike) == 0.0)
    for (int k = 0; k < 3; k++) Vstrike[k] = eY[k] * Vnorm[2];
  s = sqrt(dot3(Vstrike, Vstrike));
  for (int k = 0; k < 3; k++) Vstrike[k] = Vstrike[k] / s;
  dcross(Vnorm, Vstrike, Vdip);
  double At[3][3];
  for (int k = 0; k < 3; k++) { At[0][k] = Vnorm[k]; At[1][k] = Vstrike[k]; At[2][k] = Vdip[k]; }
  double xyz[3], p_1[3], p_2[3] = {0.0, 0.0, 0.0}, p_3[3];
  coord_trans(X - P2[0], Y - P2[1], Z - P2[2], (const double(*)[3])At, xyz);
  coord_trans(P1[0] - P2[0], P1[1] - P2[1], P1[2] - P2[2], (const double(*)[3])At, p_1);
  coord_trans(P3[0] - P2[0], P3[1] - P2[1], P3[2] - P2[2], (const double(*)[3])At, p_3);
  double x_ = xyz[0], y_ = xyz[1], z_ = xyz[2];
  double e12[3], e13[3], e23[3];
  for (int k = 0; k < 3; k++) { e12[k] = p_2[k] - p_1[k]; e13[k] = p_3[k] - p_1[k]; e23[k] = p_3[k] - p_2[k]; }
  s = sqrt(dot3(e12, e12)); for (int k = 0; k < 3; k++) e12[k] = e12[k] / s;
  s = sqrt(dot3(e13, e13)); for (int k = 0; k < 3; k++) e13[k] = e13[k] / s;
  s = sqrt(dot3(e23, e23)); for (int k = 0; k < 3; k++) e23[k] = e23[k] / s;
  double me12[3] = {-e12[0], -e12[1], -e12[2]};
  double me13[3] = {-e13[0], -e13[1], -e13[2]};
  double me23[3] = {-e23[0], -e23[1], -e23[2]};
  double A = acos(dot3(e12, e13));
  double B = acos(dot3(me12, e23));
  double C = acos(dot3(e23, e13));
  int mode = trimodefinder(y_, z_, x_, p_1 + 1, p_2 + 1, p_3 + 1);
  double E1[6], E2[6], E3[6], e[6];
  if (mode == 1) {
    td_setup_d(x_, y_, z_, A, bx, by, bz, nu, p_1, me13, E1);
    td_setup_d(x_, y_, z_, B, bx, by, bz, nu, p_2, e12, E2);
    td_setup_d(x_, y_, z_, C, bx, by, bz, nu, p_3, e23, E3);
  } else {
    td_setup_d(x_, y_, z_, A, bx, by, bz, nu, p_1, e13, E1);
    td_setup_d(x_, y_, z_, B, bx, by, bz, nu, p_2, me12, E2);
    td_setup_d(x_, y_, z_, C, bx, by, bz, nu, p_3, me23, E3);
  }
  for (int k = 0; k < 6; k++) e[k] = E1[k] + E2[k] + E3[k];
  if (mode == 0)
    for (int k = 0; k < 6; k++) e[k] = NAN;
  double Ev[6];
  tens_trans(e[0], e[1], e[2], e[3], e[4], e[5], (const double(*)[3])At, Ev);
  S6[0] = 2 * mu * Ev[0] + lambda * (Ev[0] + Ev[1] + Ev[2]);
  S6[1] = 2 * mu * Ev[1] + lambda * (Ev[0] + Ev[1] + Ev[2]);
  S6[2] = 2 * mu * Ev[2] + lambda * (Ev[0] + Ev[1] + Ev[2]);
  S6[3] = 2 * mu * Ev[3];
  S6[4] = 2 * mu * Ev[4];
  S6[5] = 2 * mu * Ev[5];
}

/* matel3dn_ij (m_HACApK_calc_entry_ij.f90:802-851), md='s'; i,j 0-based */
static double matel3dn_ij(int i, int j, const orc_bemv* b) {
  double lambda = 2 * POIS / (1 - 2 * POIS) * RIGID;
  double P1[3] = {b->xs1[j], b->ys1[j], b->zs1[j]};
  double P2[3] = {b->xs2[j], b->ys2[j], b->zs2[j]};
  double P3[3] = {b->xs3[j], b->ys3[j], b->zs3[j]};
  double S[6];
  orc_tdstressfs(b->xcol[i], b->ycol[i], b->zcol[i], P1, P2, P3, cos(b->rake[i]), sin(b->rake[i]),
                 0.0, RIGID, lambda, S);
  double A[3][3];
  A[0][0] = b->ev11[i]; A[0][1] = b->ev21[i]; A[0][2] = b->ev31[i];
  A[1][0] = b->ev12[i]; A[1][1] = b->ev22[i]; A[1][2] = b->ev32[i];
  A[2][0] = b->ev13[i]; A[2][1] = b->ev23[i]; A[2][2] = b->ev33[i];
  double p[6];
  tens_trans(S[0], S[1], S[2], S[3], S[4], S[5], (const double(*)[3])A, p);
  if (b->v == 'n') return -p[2];
  return p[4] * cos(b->rake[i]) + p[5] * sin(b->rake[i]);
}

/* ---------------- half space: free-surface correction -------------------- */
/* Strain (v11, v22, v33, v12, v13, v23) of the harmonic (free-surface
 * correction) part of an angular dislocation of angle beta whose vertex is at
 * depth a, at (y1, y2, y3) in its own frame, for Burgers vector (b1, b2, b3)
 * (AngDisStrainFSC, TDstressFS.f90:629-1011; Nikkhoo & Walter 2015, after
 * Comninou & Dundurs 1975).  The published expressions are kept term by term;
 * the factors that recur across components are named once (R*, Q*). */
static void ang_dis_strain_fsc(double y1, double y2, double y3, double beta, double b1, double b2,
                               double b3, double nu, double a, double v[6]) {
  const double sB = sin(beta), cB = cos(beta), ctB = cB / sB;
  const double y3b = y3 + 2 * a;
  const double z1b = y1 * cB + y3b * sB;
  const double z3b = -y1 * sB + y3b * cB;
  const double rb2 = y1 * y1 + y2 * y2 + y3b * y3b;
  const double rb = sqrt(rb2);
  const double W1 = rb * cB + y3b, W2 = cB + a / rb, W3 = cB + y3b / rb, W4 = nu + a / rb;
  const double W5 = 2 * nu + a / rb, W6 = rb + y3b, W7 = rb + z3b, W8 = y3 + a, W9 = 1 + a / rb / cB;
  const double N1 = 1 - 2 * nu, nu2 = 2 - 2 * nu;
  /* derivatives of the Burgers function */
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

  /* ---- v11 ---- */
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

  /* ---- v22 ---- */
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

  /* ---- v33 ---- */
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

  /* ---- v12 ---- */
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

  /* ---- v13 ---- */
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

  /* ---- v23 ---- */
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

  /* each block enters as b * (1/4 T / pi / (1 - nu)); shear blocks with b/2 */
#define FSC_K(T) (0.25 * (T) / PI / (1 - nu))
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

/* Free-surface correction of one edge PA -> PB of a triangle: the pair of
 * angular dislocations at PA and PB (AngSetupFSC_S, TDstressFS.f90:405-558).
 * Edges within 1e-3 rad of vertical contribute nothing (the reference's
 * threshold).  Output: stress (Sxx, Syy, Szz, Sxy, Sxz, Syz). */
static void ang_setup_fsc_s(double X, double Y, double Z, double bX, double bY, double bZ, const double* PA,
                            const double* PB, double mu, double lambda, double S[6]) {
  const double nu = lambda / (lambda + mu) / 2;
  double side[3] = {PB[0] - PA[0], PB[1] - PA[1], PB[2] - PA[2]};
  const double beta = acos(-side[2] / sqrt(dot3(side, side)));
  for (int k = 0; k < 6; k++) S[k] = 0.0;
  if (fabs(beta) < 1e-3 || fabs(PI - beta) < 1e-3) return;
  /* the edge's frame: ey1 horizontal along the edge, ey3 up (-eZ), ey2 = ey3 x ey1 */
  double ey1[3] = {side[0], side[1], 0.0};
  const double n1 = sqrt(dot3(ey1, ey1));
  for (int k = 0; k < 3; k++) ey1[k] = ey1[k] / n1;
  const double ey3[3] = {-0.0, -0.0, -1.0};
  double ey2[3];
  dcross(ey3, ey1, ey2);
  double A[3][3];
  for (int k = 0; k < 3; k++) { A[0][k] = ey1[k]; A[1][k] = ey2[k]; A[2][k] = ey3[k]; }
  double yA[3], yAB[3], b[3];
  coord_trans(X - PA[0], Y - PA[1], Z - PA[2], (const double(*)[3])A, yA);
  coord_trans(side[0], side[1], side[2], (const double(*)[3])A, yAB);
  const double yB[3] = {yA[0] - yAB[0], yA[1] - yAB[1], yA[2] - yAB[2]};
  coord_trans(bX, bY, bZ, (const double(*)[3])A, b);
  /* configuration I (beta * y1A >= 0) takes the angle -pi + beta */
  const double ang = (beta * yA[0] >= 0.0) ? -PI + beta : beta;
  double vA[6], vB[6], v[6];
  ang_dis_strain_fsc(yA[0], yA[1], yA[2], ang, b[0], b[1], b[2], nu, -PA[2], vA);
  ang_dis_strain_fsc(yB[0], yB[1], yB[2], ang, b[0], b[1], b[2], nu, -PB[2], vB);
  for (int k = 0; k < 6; k++) v[k] = vB[k] - vA[k];
  /* back to the fault-independent frame: E = A^T v A */
  double E[6];
  tens_trans(v[0], v[1], v[2], v[3], v[4], v[5], (const double(*)[3])A, E);
  const double tr = E[0] + E[1] + E[2];
  S[0] = 2 * mu * E[0] + lambda * tr;
  S[1] = 2 * mu * E[1] + lambda * tr;
  S[2] = 2 * mu * E[2] + lambda * tr;
  S[3] = 2 * mu * E[3];
  S[4] = 2 * mu * E[4];
  S[5] = 2 * mu * E[5];
}

/* Harmonic (free-surface) part of a triangular dislocation in the half space
 * z <= 0 (TDstress_HarFunc, TDstressFS.f90:236-293): the slip vector in the
 * fault-independent frame, then the three edges' angular-dislocation pairs. */
static void td_stress_harfunc(double X, double Y, double Z, const double* P1, const double* P2, const double* P3,
                              double Ss, double Ds, double Ts, double mu, double lambda, double S[6]) {
  const double bx = Ts, by = Ss, bz = Ds;
  double a[3] = {P2[0] - P1[0], P2[1] - P1[1], P2[2] - P1[2]}, c[3] = {P3[0] - P1[0], P3[1] - P1[1], P3[2] - P1[2]};
  double Vn[3], Vs[3], Vd[3];
  dcross(a, c, Vn);
  double s = sqrt(dot3(Vn, Vn));
  for (int k = 0; k < 3; k++) Vn[k] = Vn[k] / s;
  const double eY[3] = {0.0, 1.0, 0.0}, eZ[3] = {0.0, 0.0, 1.0};
  dcross(eZ, Vn, Vs);
  s = sqrt(dot3(Vs, Vs));
  for (int k = 0; k < 3; k++) Vs[k] = Vs[k] / s;
  if (dot3(Vs, Vs) == 0.0)
    for (int k = 0; k < 3; k++) Vs[k] = eY[k] * Vn[2];
  s = sqrt(dot3(Vs, Vs));
  for (int k = 0; k < 3; k++) Vs[k] = Vs[k] / s;
  dcross(Vn, Vs, Vd);
  /* columns Vn, Vs, Vd: slip from the triangle's frame to x, y, z */
  double At[3][3];
  for (int k = 0; k < 3; k++) { At[k][0] = Vn[k]; At[k][1] = Vs[k]; At[k][2] = Vd[k]; }
  double bg[3];
  coord_trans(bx, by, bz, (const double(*)[3])At, bg);
  double S1[6], S2[6], S3[6];
  ang_setup_fsc_s(X, Y, Z, bg[0], bg[1], bg[2], P1, P2, mu, lambda, S1);
  ang_setup_fsc_s(X, Y, Z, bg[0], bg[1], bg[2], P2, P3, mu, lambda, S2);
  ang_setup_fsc_s(X, Y, Z, bg[0], bg[1], bg[2], P3, P1, mu, lambda, S3);
  for (int k = 0; k < 6; k++) S[k] = S1[k] + S2[k] + S3[k];
}

/* TDstressHS (TDstressFS.f90:7-44): main dislocation + its image through
 * z = 0 + the harmonic correction, half space z <= 0 */
void orc_tdstresshs(double X, double Y, double Z, const double* P1, const double* P2, const double* P3, double Ss,
                    double Ds, double Ts, double mu, double lambda, double* S6) {
  double Sm[6], Sh[6], Si[6];
  orc_tdstressfs(X, Y, Z, P1, P2, P3, Ss, Ds, Ts, mu, lambda, Sm);
  td_stress_harfunc(X, Y, Z, P1, P2, P3, Ss, Ds, Ts, mu, lambda, Sh);
  const double Q1[3] = {P1[0], P1[1], -P1[2]}, Q2[3] = {P2[0], P2[1], -P2[2]}, Q3[3] = {P3[0], P3[1], -P3[2]};
  orc_tdstressfs(X, Y, Z, Q1, Q2, Q3, Ss, Ds, Ts, mu, lambda, Si);
  for (int k = 0; k < 6; k++) S6[k] = Sm[k] + Si[k] + Sh[k];
}

/* matel3dh_ij (m_HACApK_calc_entry_ij.f90:852-898), md='s': the source slips
 * along its own rake (unlike matel3dn_ij, which uses the receiver's) */
static double matel3dh_ij(int i, int j, const orc_bemv* b) {
  double lambda = 2 * POIS / (1 - 2 * POIS) * RIGID;
  double P1[3] = {b->xs1[j], b->ys1[j], b->zs1[j]};
  double P2[3] = {b->xs2[j], b->ys2[j], b->zs2[j]};
  double P3[3] = {b->xs3[j], b->ys3[j], b->zs3[j]};
  double S[6];
  orc_tdstresshs(b->xcol[i], b->ycol[i], b->zcol[i], P1, P2, P3, cos(b->rake[j]), sin(b->rake[j]), 0.0, RIGID,
                 lambda, S);
  double A[3][3];
  A[0][0] = b->ev11[i]; A[0][1] = b->ev21[i]; A[0][2] = b->ev31[i];
  A[1][0] = b->ev12[i]; A[1][1] = b->ev22[i]; A[1][2] = b->ev32[i];
  A[2][0] = b->ev13[i]; A[2][1] = b->ev23[i]; A[2][2] = b->ev33[i];
  double p[6];
  tens_trans(S[0], S[1], S[2], S[3], S[4], S[5], (const double(*)[3])A, p);
  if (b->v == 'n') return -p[2];
  return p[4] * cos(b->rake[i]) + p[5] * sin(b->rake[i]);
}

/* ---- 2D plane strain (problems 2dph / 2dnh and 2dn) ---------------------- */
static const double VS = 3.464, VP = 6.0; /* m_const.f90 */

/* Stress (sxx, syy, sxy) at (X, Y) of an edge dislocation at (xs, ys) with unit
 * Burgers vector (s1, s2) = (glide, climb) in the half space Y >= 0 whose free
 * surface is Y = 0: the full-space pair at (xs, +-ys) plus the surface
 * correction (D2dip2, m_HACApK_calc_entry_ij.f90:145-166). */
static void edge_disl_hs(double X, double Y, double xs, double ys, double s1, double s2, double out[3]) {
  const double dx = X - xs, ym = Y - ys, yp = Y + ys;
  const double r1 = sqrt(dx * dx + ym * ym), r2 = sqrt(dx * dx + yp * yp);
  const double q1 = r1 * r1 * r1 * r1, q2 = r2 * r2 * r2 * r2, q3 = r2 * r2 * r2 * r2 * r2 * r2;
  const double dx2 = dx * dx, dx4 = dx2 * dx2, ym2 = ym * ym, yp2 = yp * yp, yp3 = yp2 * yp;
  const double c = RIGID / 2.0 / PI / (1.0 - POIS);
  /* glide (s1) and climb (s2) parts of each component */
  const double gxx = ym * (ym2 + 3 * dx2) / q1 - yp * (yp2 + 3 * dx2) / q2 +
                     2 * ys / q3 * (6 * Y * yp * dx2 - ym * yp3 - dx4);
  const double cxx = dx * (ym2 - dx2) / q1 - dx * (yp2 - dx2) / q2 +
                     4 * ys * dx / q3 * ((2 * ys - Y) * yp2 + (3 * Y + 2 * ys) * dx2);
  const double gyy = ym * (ym2 - dx2) / q1 - yp * (yp2 - dx2) / q2 -
                     2 * ys / q3 * (6 * Y * yp * dx2 - (3 * Y + ys) * yp3 + dx4);
  const double cyy = dx * (3 * ym2 + dx2) / q1 - dx * (3 * yp2 + dx2) / q2 -
                     4 * ys * dx * Y / q3 * (3 * yp2 - dx2);
  const double gxy = dx * (ym2 - dx2) / q1 - dx * (yp2 - dx2) / q2 + 4 * ys * dx * Y / q3 * (3 * yp2 - dx2);
  const double cxy = ym * (ym2 - dx2) / q1 - yp * (yp2 - dx2) / q2 +
                     2 * ys / q3 * (6 * Y * yp * dx2 - dx4 + (ys - Y) * yp3);
  out[0] = s1 * c * gxx + s2 * c * cxx;
  out[1] = s1 * c * gyy - s2 * c * cyy;
  out[2] = s1 * c * gxy + s2 * c * cxy;
}

/* traction on a plane at angle a of the x axis from (sxx, syy, sxy): shear
 * (v='s') or normal, compression positive (v='n') */
static double traction_2d_hs(double sxx, double syy, double sxy, double a, char v) {
  if (v == 'n') return -0.5 * (sxx + syy) + 0.5 * (sxx - syy) * cos(2 * a) + sxy * sin(2 * a);
  return -0.5 * (sxx - syy) * sin(2 * a) + sxy * cos(2 * a);
}

/* matel2dph2_ij (m_HACApK_calc_entry_ij.f90:92-116): unit slip on element j
 * (between its ends, along its dip ang(j)) in the half space */
static double matel2dph(int i, int j, const orc_bemv* b) {
  const double s1 = cos(b->ang[j]), s2 = sin(b->ang[j]);
  double p[3], q[3];
  edge_disl_hs(b->xcol[i], b->ycol[i], b->xel[j], b->yel[j], s1, s2, p);
  edge_disl_hs(b->xcol[i], b->ycol[i], b->xer[j], b->yer[j], s1, s2, q);
  return traction_2d_hs(p[0] - q[0], p[1] - q[1], p[2] - q[2], b->ang[i], b->v);
}

/* the full-space integrals inte11s / inte12s / inte22s (:697-722): stress
 * kernel components of a dislocation end at (x1, x2) in its own frame */
static void plane_kernel(double x1, double x2, double k[3]) {
  const double r = sqrt(x1 * x1 + x2 * x2);
  const double r4 = r * r * r * r;
  const double pa = VS / VP;
  k[0] = -2 * VS / PI * (1 - pa * pa) * x2 * (3 * x1 * x1 + x2 * x2) / r4;
  k[1] = 2 * VS / PI * (1 - pa * pa) * x1 * (x1 * x1 - x2 * x2) / r4;
  k[2] = 2 * VS / PI * (1 - pa * pa) * x2 * (x1 * x1 - x2 * x2) / r4;
}

/* tensor2d_ij (m_HACApK_calc_entry_ij.f90:300-339), md='s': full space */
static double tensor2d(int i, int j, const orc_bemv* b) {
  const double cj = cos(b->ang[j]), sj = sin(b->ang[j]);
  const double dxl = b->xcol[i] - b->xel[j], dyl = b->ycol[i] - b->yel[j];
  const double dxr = b->xcol[i] - b->xer[j], dyr = b->ycol[i] - b->yer[j];
  double kl[3], kr[3];
  plane_kernel(cj * dxl + sj * dyl, -sj * dxl + cj * dyl, kl);
  plane_kernel(cj * dxr + sj * dyr, -sj * dxr + cj * dyr, kr);
  const double g = -0.5 * RIGID / VS;
  const double k11 = g * (kl[0] - kr[0]), k12 = g * (kl[1] - kr[1]), k22 = g * (kl[2] - kr[2]);
  /* rotate from the source frame to x, y */
  const double s2 = sin(-2 * b->ang[j]), c2 = cos(-2 * b->ang[j]);
  const double sxx = 0.5 * (k11 + k22) + 0.5 * (k11 - k22) * c2 + k12 * s2;
  const double sxy = -0.5 * (k11 - k22) * s2 + k12 * c2;
  const double syy = 0.5 * (k11 + k22) - 0.5 * (k11 - k22) * c2 - k12 * s2;
  const double a = b->ang[i];
  if (b->v == 'n') return -(0.5 * (sxx + syy) - 0.5 * (sxx - syy) * cos(2 * a) - sxy * sin(2 * a));
  return 0.5 * (sxx - syy) * sin(-2 * a) + sxy * cos(-2 * a);
}

double orc_entry_ij(int i, int j, const orc_bemv* b) {
  int i0 = i - 1, j0 = j - 1;
  switch (b->problem) {
    case ORC_2DVS: {
      /* matels2dpa_ij(xel,xer) - matels2dpa_ij(-xel,-xer) (:55-57) */
      return matels2dpa(i0, j0, b->xcol, b->xel[j0], b->xer[j0]) -
             matels2dpa(i0, j0, b->xcol, -b->xel[j0], -b->xer[j0]);
    }
    case ORC_3DPH: return okada_ij(i0, j0, b, 0);
    case ORC_3DNR: return okada_ij(i0, j0, b, 1);
    case ORC_3DNT: return matel3dn_ij(i0, j0, b);
    case ORC_2DPH: return matel2dph(i0, j0, b);
    case ORC_2DN: return tensor2d(i0, j0, b);
    case ORC_3DHT: return matel3dh_ij(i0, j0, b);
  }
  return NAN;
}
