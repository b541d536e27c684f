/*
 * orc_rk.c -- oracle restatement of the rate-and-state right-hand side, the
 * Cash-Karp Runge-Kutta step and its error controller, the accepted-step
 * update and the mesh builders of the driver.  TEST INFRASTRUCTURE ONLY.
 *
 *   derivs                 main_LH.f90:2053-2163
 *   deriv (aging, slip)    main_LH.f90:2165-2244
 *   rkqs                   main_LH.f90:2270-2370
 *   rkck                   main_LH.f90:2472-2554
 *   step update            main_LH.f90:1266-1287
 *   coordinate2dp          main_LH.f90:1701-1718
 *   coordinate3ddip        main_LH.f90:1781-1835
 *   evcalc                 main_LH.f90:1940-1990
 *
 * The Cash-Karp coefficients are written in the reference as default-real
 * expressions (3./40., .3, 37./378., ...) assigned to real(8) parameters, so
 * they carry single-precision values widened to double; the rkqs constants
 * SAFETY=0.9, PGROW=-0.2 and tiny=1e-20 likewise.  Restated as such.
 */
#include "hbi_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

static const double RIGID = 32.04, VS = 3.464;
#define PI (4 * atan(1.0))

void orc_cashkarp(double* a, double* b, double* c, double* dc) {
  /* a[0..5] = A2..A6 (a[0] unused=0); b[0..14] = B21,B31,B32,B41..B43,B51..B54,B61..B65;
   * c[0..5] = C1,0,C3,C4,0,C6; dc[0..5] = DC1,0,DC3,DC4,DC5,DC6 */
  a[0] = 0.0; a[1] = .2; a[2] = .3; a[3] = .6; a[4] = 1.0; a[5] = .875;
  b[0] = .2;
  b[1] = (double)(3.f / 40.f); b[2] = (double)(9.f / 40.f);
  b[3] = (double).3f; b[4] = (double)-.9f; b[5] = (double)1.2f;
  b[6] = (double)(-(11.f / 54.f)); b[7] = 2.5; b[8] = (double)(-(70.f / 27.f)); b[9] = (double)(35.f / 27.f);
  b[10] = (double)(1631.f / 55296.f); b[11] = (double)(175.f / 512.f); b[12] = (double)(575.f / 13824.f);
  b[13] = (double)(44275.f / 110592.f); b[14] = (double)(253.f / 4096.f);
  double C1 = (double)(37.f / 378.f), C3 = (double)(250.f / 621.f), C4 = (double)(125.f / 594.f),
         C6 = (double)(512.f / 1771.f);
  c[0] = C1; c[1] = 0; c[2] = C3; c[3] = C4; c[4] = 0; c[5] = C6;
  dc[0] = C1 - (double)(2825.f / 27648.f);
  dc[1] = 0;
  dc[2] = C3 - (double)(18575.f / 48384.f);
  dc[3] = C4 - (double)(13525.f / 55296.f);
  dc[4] = (double)(-(277.f / 14336.f));
  dc[5] = C6 - (double).25f;
}

void orc_rkqs_consts(double* c) {
  c[0] = (double)0.9f;    /* SAFETY */
  c[1] = (double)-0.2f;   /* PGROW */
  c[2] = -0.25;           /* PSHRNK */
  c[3] = (double)1e-20f;  /* tiny */
}

/* deriv (main_LH.f90:2165-2244), aging (evlaw 0) and slip (evlaw 1) laws */
static void deriv(const orc_rsf* p, double sum_gs, double sum_gn, double psitmp, double tautmp,
                  double sigmatmp, double veltmp, double a, double b, double dc, double f0,
                  double* dpsidt, double* dtaudt, double* dsigdt) {
  *dsigdt = sum_gn;
  if (p->limitsigma) {
    if (sigmatmp < p->minsig) *dsigdt = 0;
    if (sigmatmp > p->maxsig) *dsigdt = 0;
  }
  double vref = p->vref;
  if (p->evlaw == 0) {
    if (b == 0) *dpsidt = 0.0;
    else *dpsidt = b / dc * vref * exp((f0 - psitmp) / b) - b * fabs(veltmp) / dc;
  } else {
    double fss = f0 + (a - b) * log(fabs(veltmp) / vref);
    *dpsidt = -(fabs(veltmp) / dc * (fabs(tautmp) / sigmatmp - fss));
  }
  double dvdtau = 2 * vref * exp(-psitmp / a) * cosh(tautmp / sigmatmp / a) / (a * sigmatmp);
  double dvdsig = -(2 * vref * exp(-psitmp / a) * cosh(tautmp / sigmatmp / a) * tautmp / (a * (sigmatmp * sigmatmp)));
  double dvdpsi = -veltmp / a;
  double t = sum_gs - 0.5 * RIGID / VS * (dvdpsi * *dpsidt + dvdsig * *dsigdt);
  *dtaudt = t / (1.0 + 0.5 * RIGID / VS * dvdtau);
}

void orc_derivs(const orc_rsf* p, double x, const double* y, double* dydx) {
  (void)x;
  int n = p->n;
  double* vel = (double*)malloc(sizeof(double) * n);
  double* u = (double*)malloc(sizeof(double) * n);
  double* gs = (double*)malloc(sizeof(double) * n);
  double* gn = (double*)malloc(sizeof(double) * n);
  for (int i = 0; i < n; i++) {
    double psi = y[3 * i], tau = y[3 * i + 1], sig = y[3 * i + 2];
    vel[i] = 2 * p->vref * exp(-psi / p->a[i]) * sinh(tau / sig / p->a[i]);
  }
  for (int i = 0; i < n; i++) u[i] = p->backslip ? (vel[i] + 0.0) - p->vplv[i] : vel[i] + 0.0;
  if (p->nthreads > 1) orc_matvec_omp(n, p->nleaf_s, p->leaves_s, p->off_s, p->body_s, u, gs, p->nthreads);
  else orc_matvec(n, p->nleaf_s, p->leaves_s, p->off_s, p->body_s, u, gs);
  if (p->divide_ds0) for (int i = 0; i < n; i++) gs[i] = gs[i] / p->ds0;
  if (p->nmat < 2) {
    for (int i = 0; i < n; i++) gn[i] = 0.0;
  } else {
    if (p->nthreads > 1) orc_matvec_omp(n, p->nleaf_n, p->leaves_n, p->off_n, p->body_n, u, gn, p->nthreads);
    else orc_matvec(n, p->nleaf_n, p->leaves_n, p->off_n, p->body_n, u, gn);
    if (p->divide_ds0) for (int i = 0; i < n; i++) gn[i] = gn[i] / p->ds0;
  }
  for (int i = 0; i < n; i++) {
    gn[i] = gn[i] + p->sigdot[i];
    gs[i] = gs[i] + p->taudot[i];
    deriv(p, gs[i], gn[i], y[3 * i], y[3 * i + 1], y[3 * i + 2], vel[i], p->a[i], p->b[i], p->dc[i],
          p->f0[i], &dydx[3 * i], &dydx[3 * i + 1], &dydx[3 * i + 2]);
  }
  free(vel); free(u); free(gs); free(gn);
}

void orc_rkck(const orc_rsf* p, const double* y, double x, double h, double* yout, double* yerr) {
  double A[6], B[15], C[6], DC[6];
  orc_cashkarp(A, B, C, DC);
  int len = 3 * p->n;
  double* ak[6];
  for (int s = 0; s < 6; s++) ak[s] = (double*)malloc(sizeof(double) * len);
  double* yt = (double*)malloc(sizeof(double) * len);
  orc_derivs(p, x, y, ak[0]);
  for (int i = 0; i < len; i++) yt[i] = y[i] + B[0] * h * ak[0][i];
  orc_derivs(p, x + A[1] * h, yt, ak[1]);
  for (int i = 0; i < len; i++) yt[i] = y[i] + h * (B[1] * ak[0][i] + B[2] * ak[1][i]);
  orc_derivs(p, x + A[2] * h, yt, ak[2]);
  for (int i = 0; i < len; i++) yt[i] = y[i] + h * (B[3] * ak[0][i] + B[4] * ak[1][i] + B[5] * ak[2][i]);
  orc_derivs(p, x + A[3] * h, yt, ak[3]);
  for (int i = 0; i < len; i++)
    yt[i] = y[i] + h * (B[6] * ak[0][i] + B[7] * ak[1][i] + B[8] * ak[2][i] + B[9] * ak[3][i]);
  orc_derivs(p, x + A[4] * h, yt, ak[4]);
  for (int i = 0; i < len; i++)
    yt[i] = y[i] + h * (B[10] * ak[0][i] + B[11] * ak[1][i] + B[12] * ak[2][i] + B[13] * ak[3][i] + B[14] * ak[4][i]);
  orc_derivs(p, x + A[5] * h, yt, ak[5]);
  for (int i = 0; i < len; i++) yout[i] = y[i] + h * (C[0] * ak[0][i] + C[2] * ak[2][i] + C[3] * ak[3][i] + C[5] * ak[5][i]);
  for (int i = 0; i < len; i++)
    yerr[i] = h * (DC[0] * ak[0][i] + DC[2] * ak[2][i] + DC[3] * ak[3][i] + DC[4] * ak[4][i] + DC[5] * ak[5][i]);
  for (int s = 0; s < 6; s++) free(ak[s]);
  free(yt);
}

double orc_errmax(int len, const double* yerr, const double* ytemp, double eps) {
  double errmax = 0.0;
  for (int i = 0; i < len; i++) {
    if (fabs(yerr[i] / ytemp[i]) / eps > errmax) errmax = fabs(yerr[i] / ytemp[i]) / eps;
    if (ytemp[i] - 1 == ytemp[i]) errmax = 10.0;
  }
  return errmax;
}

int orc_rkqs(const orc_rsf* p, double* y, double* x, double htry, double eps, double dtmax,
             double* hdid, double* hnext, double* errmax_gb, int* nrjct) {
  double K[4];
  orc_rkqs_consts(K);
  const double SAFETY = K[0], PGROW = K[1], PSHRNK = K[2], tiny = K[3];
  int len = 3 * p->n;
  double* ytemp = (double*)malloc(sizeof(double) * len);
  double* yerr = (double*)malloc(sizeof(double) * len);
  double h = htry, e;
  *nrjct = 0;
  for (;;) {
    orc_rkck(p, y, *x, h, ytemp, yerr);
    e = orc_errmax(len, yerr, ytemp, eps);
    if ((e < 1.0) && (e > tiny)) break;
    (*nrjct)++;
    if (e > tiny) {
      double h2 = SAFETY * h * pow(e, PSHRNK);
      h = (0.5 * h > h2) ? 0.5 * h : h2;
    } else {
      h = 0.5 * h;
    }
    double xnew = *x + h;
    if (xnew - *x < 1.e-15) { free(ytemp); free(yerr); *errmax_gb = e; return -1; }
  }
  double hn = 2 * h, g = SAFETY * h * pow(e, PGROW);
  if (g < hn) hn = g;
  if (dtmax < hn) hn = dtmax;
  *hnext = hn;
  *hdid = h;
  *x = *x + h;
  memcpy(y, ytemp, sizeof(double) * len);
  *errmax_gb = e;
  free(ytemp); free(yerr);
  return 0;
}

void orc_step_update(const orc_rsf* p, const double* y, double dtdid, double* psi, double* tau,
                     double* sigma, double* slip, double* vel, double* mu) {
  for (int i = 0; i < p->n; i++) {
    psi[i] = y[3 * i]; tau[i] = y[3 * i + 1]; sigma[i] = y[3 * i + 2];
    slip[i] = slip[i] + (vel[i] + 0.0) * dtdid * 0.5;
    vel[i] = 2 * p->vref * exp(-psi[i] / p->a[i]) * sinh(tau[i] / sigma[i] / p->a[i]);
    slip[i] = slip[i] + (vel[i] + 0.0) * dtdid * 0.5;
    mu[i] = tau[i] / sigma[i];
  }
}

void orc_mesh_2dp(int n, double ds0, double* xel, double* xer, double* xcol, double* ds) {
  for (int i = 1; i <= n; i++) {
    ds[i - 1] = ds0;
    xel[i - 1] = (i - 1) * ds0;
    xer[i - 1] = i * ds0;
    xcol[i - 1] = 0.5 * (xel[i - 1] + xer[i - 1]);
  }
}

void orc_mesh_3ddip(int imax, int jmax, double ds0, double dipangle, double* xcol, double* ycol,
                    double* zcol, double* angd, double* ang) {
  double* yr = (double*)malloc(sizeof(double) * (jmax + 1));
  double* zr = (double*)malloc(sizeof(double) * (jmax + 1));
  yr[0] = 0.0; zr[0] = 0.0;
  for (int j = 1; j <= jmax; j++) {
    yr[j] = yr[j - 1] - ds0 * cos(dipangle * PI / 180.0);
    zr[j] = zr[j - 1] - ds0 * sin(dipangle * PI / 180.0);
  }
  int k = 0;
  for (int i = 1; i <= imax; i++)
    for (int j = 1; j <= jmax; j++) {
      k++;
      xcol[k - 1] = (i - imax / 2 - 0.5) * ds0;
      ycol[k - 1] = 0.5 * (yr[j - 1] + yr[j]);
      zcol[k - 1] = 0.5 * (zr[j - 1] + zr[j]);
      angd[k - 1] = atan2(zr[j - 1] - zr[j], yr[j - 1] - yr[j]);
      ang[k - 1] = 0.0;
    }
  free(yr); free(zr);
}

void orc_evcalc(int n, const double* xs1, const double* xs2, const double* xs3, const double* ys1,
                const double* ys2, const double* ys3, const double* zs1, const double* zs2,
                const double* zs3, double* ev11, double* ev12, double* ev13, double* ev21,
                double* ev22, double* ev23, double* ev31, double* ev32, double* ev33, double* ds) {
  for (int k = 0; k < n; k++) {
    double vba[3] = {xs2[k] - xs1[k], ys2[k] - ys1[k], zs2[k] - zs1[k]};
    double vca[3] = {xs3[k] - xs1[k], ys3[k] - ys1[k], zs3[k] - zs1[k]};
    ev31[k] = vba[1] * vca[2] - vba[2] * vca[1];
    ev32[k] = vba[2] * vca[0] - vba[0] * vca[2];
    ev33[k] = vba[0] * vca[1] - vba[1] * vca[0];
    double rr = sqrt(ev31[k] * ev31[k] + ev32[k] * ev32[k] + ev33[k] * ev33[k]);
    ev31[k] = ev31[k] / rr; ev32[k] = ev32[k] / rr; ev33[k] = ev33[k] / rr;
    if (fabs(ev33[k]) < 1.0) {
      ev11[k] = -ev32[k]; ev12[k] = ev31[k]; ev13[k] = 0.0;
      rr = sqrt(ev11[k] * ev11[k] + ev12[k] * ev12[k]);
      ev11[k] = ev11[k] / rr; ev12[k] = ev12[k] / rr;
    } else {
      ev11[k] = 1.0; ev12[k] = 0.0; ev13[k] = 0.0;
    }
    ev21[k] = ev32[k] * ev13[k] - ev33[k] * ev12[k];
    ev22[k] = ev33[k] * ev11[k] - ev31[k] * ev13[k];
    ev23[k] = ev31[k] * ev12[k] - ev32[k] * ev11[k];
    double t1 = vba[0] * vba[0] + vba[1] * vba[1] + vba[2] * vba[2];
    double t2 = vca[0] * vca[0] + vca[1] * vca[1] + vca[2] * vca[2];
    double t3 = vba[0] * vca[0] + vba[1] * vca[1] + vba[2] * vca[2];
    ds[k] = 0.5 * sqrt(t1 * t2 - t3 * t3);
  }
}

/* ---- step-size proposer MLP (no reference counterpart; checker for the
 *      GPU training kernels).  Double accumulation, float in/out. ---- */
double orc_mlp_loss_grad(int nin, int h, int batch, const float* P, const float* X,
                         const float* T, float* G, float* out) {
  return orc_mlp_loss_grad_tau(nin, h, batch, P, X, T, G, out, -1.0);
}

/* as orc_mlp_loss_grad with the pinball loss of quantile tau when 0 < tau < 1:
 * (1 - tau) r for r = y - t > 0, -tau r otherwise (derivative 0 at r = 0) */
double orc_mlp_loss_grad_tau(int nin, int h, int batch, const float* P, const float* X,
                             const float* T, float* G, float* out, double tau) {
  const float* W1 = P;
  const float* b1 = W1 + h * nin;
  const float* W2 = b1 + h;
  const float* b2 = W2 + h * h;
  const float* W3 = b2 + h;
  const float* b3 = W3 + h;
  size_t np = (size_t)h * nin + h + (size_t)h * h + h + h + 1;
  double* g = (double*)calloc(np, sizeof(double));
  double* a1 = (double*)malloc(sizeof(double) * h);
  double* a2 = (double*)malloc(sizeof(double) * h);
  double* d2 = (double*)malloc(sizeof(double) * h);
  double* d1 = (double*)malloc(sizeof(double) * h);
  double loss = 0.0;
  for (int s = 0; s < batch; s++) {
    const float* x = X + (size_t)s * nin;
    for (int o = 0; o < h; o++) {
      double z = b1[o];
      for (int i = 0; i < nin; i++) z += (double)W1[o * nin + i] * x[i];
      a1[o] = tanh(z);
    }
    for (int o = 0; o < h; o++) {
      double z = b2[o];
      for (int i = 0; i < h; i++) z += (double)W2[o * h + i] * a1[i];
      a2[o] = tanh(z);
    }
    double y = b3[0];
    for (int i = 0; i < h; i++) y += (double)W3[i] * a2[i];
    if (out) out[s] = (float)y;
    double r = y - T[s];
    double dy;
    if (tau > 0.0) {
      loss += r > 0.0 ? (1.0 - tau) * r : -tau * r;
      dy = (r > 0.0 ? 1.0 - tau : (r < 0.0 ? -tau : 0.0)) / batch;
    } else {
      loss += r * r;
      dy = 2.0 * r / batch;
    }
    double* gW1 = g;
    double* gb1 = gW1 + h * nin;
    double* gW2 = gb1 + h;
    double* gb2 = gW2 + h * h;
    double* gW3 = gb2 + h;
    double* gb3 = gW3 + h;
    gb3[0] += dy;
    for (int i = 0; i < h; i++) {
      gW3[i] += dy * a2[i];
      d2[i] = dy * W3[i] * (1.0 - a2[i] * a2[i]);
    }
    for (int o = 0; o < h; o++) {
      gb2[o] += d2[o];
      for (int i = 0; i < h; i++) gW2[o * h + i] += d2[o] * a1[i];
    }
    for (int i = 0; i < h; i++) {
      double acc = 0.0;
      for (int o = 0; o < h; o++) acc += d2[o] * W2[o * h + i];
      d1[i] = acc * (1.0 - a1[i] * a1[i]);
    }
    for (int o = 0; o < h; o++) {
      gb1[o] += d1[o];
      for (int i = 0; i < nin; i++) gW1[o * nin + i] += d1[o] * x[i];
    }
  }
  for (size_t k = 0; k < np; k++) G[k] = (float)g[k];
  free(g); free(a1); free(a2); free(d1); free(d2);
  return loss / batch;
}

/* The time loop of main_LH.f90:1217-1438 without its output files: rkqs, the
 * step update (:1266-1287), the monitors (:1291-1336), the event list
 * (:1338-1388) and the stop controls (:1425-1438), for at most nsteps steps.
 * Per accepted step one record of ORC_CYCLE_REC doubles
 *   k, x, hdid, errmax, nrjct, mvel, loc (0-based maxloc of |vel|), meanslip,
 *   meanmu, maxnorm, minnorm, outfield
 * and per finished event ORC_CYCLE_EV doubles
 *   eventcount, k, onset_time, moment, hypoloc, x.
 * Returns the stop code (0 none, 1 tmax, 2 velmax, 3 velmin, 4 step limit,
 * 5 step size underflow).  y, slip and vel carry the loop state in and out. */
int orc_cycle(const orc_rsf* p, const orc_cycle_params* cp, double* y, double* vel, double* slip,
              const double* ds, long long nsteps, double* rec, long long* nrec, double* ev, int max_ev,
              int* nev) {
  const int n = p->n;
  double* psi = (double*)malloc(sizeof(double) * n);
  double* tau = (double*)malloc(sizeof(double) * n);
  double* sig = (double*)malloc(sizeof(double) * n);
  double* mu = (double*)malloc(sizeof(double) * n);
  double* islip = (double*)calloc(n, sizeof(double));
  double sg = 0.0;
  for (int i = 0; i < n; i++) sg += ds[i];
  double x = 0.0, dtnxt = cp->dtinit, dtout = cp->dtout_inter, tout = dtout, moment0 = 0.0, onset = 0.0;
  int slipping = 0, eventcount = 0, hypoloc = 0, stop = 0;
  long long interval = cp->interval > 0 ? cp->interval : cp->nstep;
  *nrec = 0;
  *nev = 0;
  for (long long k = 1; k <= nsteps; k++) {
    double dtdid, errmax;
    int nrjct;
    if (orc_rkqs(p, y, &x, dtnxt, cp->eps_r, cp->dtmax, &dtdid, &dtnxt, &errmax, &nrjct)) {
      stop = 5;
      break;
    }
    orc_step_update(p, y, dtdid, psi, tau, sig, slip, vel, mu);
    double mvel = -1.0, maxnorm = -INFINITY, minnorm = INFINITY, meanslip = 0.0, meanmu = 0.0;
    int loc = 0;
    for (int i = 0; i < n; i++) {
      if (fabs(vel[i]) > mvel) { mvel = fabs(vel[i]); loc = i; }
      if (sig[i] > maxnorm) maxnorm = sig[i];
      if (sig[i] < minnorm) minnorm = sig[i];
      meanslip += fabs(slip[i]) * ds[i];
      meanmu += mu[i] * ds[i];
    }
    meanslip /= sg;
    meanmu /= sg;
    int outfield = 0;
    if (!slipping && mvel > cp->velth) {
      outfield = 1; slipping = 1; dtout = cp->dtout_co; tout = x + dtout; eventcount++;
      moment0 = meanslip;
      memcpy(islip, slip, sizeof(double) * n);
      hypoloc = loc + 1;
      onset = x;
    }
    if (slipping && mvel < 0.5 * cp->velth) {
      outfield = 1; slipping = 0; dtout = cp->dtout_inter; tout = x + dtout;
      if (*nev < max_ev) {
        double* e = ev + (size_t)(*nev) * ORC_CYCLE_EV;
        e[0] = eventcount; e[1] = (double)k; e[2] = onset; e[3] = meanslip - moment0; e[4] = hypoloc; e[5] = x;
      }
      (*nev)++;
    }
    if (k % interval == 0) outfield = 1;
    if (x > tout) { outfield = 1; tout = x + dtout; }
    double* r = rec + (size_t)(*nrec) * ORC_CYCLE_REC;
    r[0] = (double)k; r[1] = x; r[2] = dtdid; r[3] = errmax; r[4] = nrjct; r[5] = mvel; r[6] = loc;
    r[7] = meanslip; r[8] = meanmu; r[9] = maxnorm; r[10] = minnorm; r[11] = outfield;
    (*nrec)++;
    if (mvel > cp->velmax) { stop = 2; break; }
    if (mvel < cp->velmin) { stop = 3; break; }
    if (x > cp->tmax) { stop = 1; break; }
    if (k == nsteps) stop = 4;
  }
  free(psi); free(tau); free(sig); free(mu); free(islip);
  return stop;
}
