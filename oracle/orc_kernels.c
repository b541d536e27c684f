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
  }
  return NAN;
}
