/*
 * hbi_oracle.h -- CPU restatement of HBI's per-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library (hbi_gb300/) links,
 * loads or calls this code; only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py do, and there only as the
 * checker or the timed CPU baseline.
 *
 * Parity status: the reference is Fortran 90 + MPI and no Fortran compiler is
 * available where this is built, so the oracle cannot be checked against the
 * reference binary ("parity unpinned" against reference outputs).  It is pinned
 * instead against known answers that follow from the physics and the
 * algorithms (closed forms, Okada-vs-two-triangles identity, reciprocity, exact
 * low-rank recovery, dense H*1 products); see tests/test_oracle_pins.py.
 *
 * Arithmetic: every routine follows the reference statement by statement, with
 * the reference's evaluation order, its single-precision literals (e.g. the
 * Cash-Karp tableau written as 3./40.) widened exactly as a Fortran compiler
 * widens them, and no FMA contraction (built with -ffp-contract=off).
 *
 * Index conventions: arrays passed in are 0-based C arrays; values that the
 * reference stores as 1-based indices (lod, nstrtl, nstrtt) stay 1-based.
 */
#ifndef HBI_ORACLE_H
#define HBI_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* problem kinds (reference st_bemv%problem) */
#define ORC_2DVS 1
#define ORC_3DPH 2
#define ORC_3DNR 3
#define ORC_3DNT 4
#define ORC_2DPH 5 /* also 2dnh: matel2dph2_ij */
#define ORC_2DN 6  /* tensor2d_ij */
#define ORC_3DHT 7 /* matel3dh_ij */

/* Geometry / kernel selector, the restatement of st_HACApK_calc_entry
 * (m_HACApK_calc_entry_ij.f90:7-19).  All arrays have length n (global order). */
typedef struct {
  int problem;          /* ORC_* */
  int n;
  char v;               /* 's' shear or 'n' normal (st_bemv%v) */
  char md;              /* 's' (st_bemv%md) -- only 's' is on the hot path */
  const double *xcol, *ycol, *zcol;
  const double *xel, *xer;                     /* 2dvs */
  const double *ang, *angd, *dsl, *dsd, *rake; /* okada (rake also for TD) */
  double w;                                    /* okada normalisation ds0 */
  const double *xs1, *xs2, *xs3, *ys1, *ys2, *ys3, *zs1, *zs2, *zs3; /* TD */
  const double *ev11, *ev12, *ev13, *ev21, *ev22, *ev23, *ev31, *ev32, *ev33;
  const double *yel, *yer;                     /* 2dph / 2dn element ends (with xel, xer) */
} orc_bemv;

/* Leaf record (st_HACApK_leafmtx, m_HACApK_base.f90:57-72). 1-based starts. */
typedef struct {
  int ltmtx, kt, nstrtl, ndl, nstrtt, ndt;
} orc_leaf;

/* ---- structure: cluster tree + admissibility + sort (bit-exact) ---- */
/* Builds lod (1-based values, length n) and the sorted leaf list for the
 * one-rank lattice (the whole matrix is one lattice block).  coord is the
 * reference's coord(n,3) column-major.  Returns number of leaves, or <0.
 * leaves_out is malloc'd; free with orc_free. */
int orc_build_structure(int n, const double* coord, const double* param,
                        int* lod, orc_leaf** leaves_out, int* count_check);
void orc_free(void* p);
/* default HACApK param(1:100) as set by HACApK_init on one rank */
void orc_default_params(double* param100);

/* ---- kernel entries (FP64) ---- */
double orc_entry_ij(int i, int j, const orc_bemv* b); /* 1-based i,j */
void orc_okada(double alpha, double x, double y, double z, double depth, double dip,
               double al1, double al2, double aw1, double aw2, double disl1,
               double disl2, double disl3, double* u12, int fullspace);
void orc_tdstressfs(double X, double Y, double Z, const double* P1, const double* P2,
                    const double* P3, double Ss, double Ds, double Ts, double mu,
                    double lambda, double* S6);
/* TDstressHS (TDstressFS.f90:7-44), half space z <= 0 */
void orc_tdstresshs(double X, double Y, double Z, const double* P1, const double* P2,
                    const double* P3, double Ss, double Ds, double Ts, double mu,
                    double lambda, double* S6);

/* ---- ACA+ and fill ---- */
/* One admissible leaf by ACA+ (m_HACApK_base.f90:1748-1946).  U (ndl x kt) and
 * V (ndt x kt), column-major, malloc'd into *U,*V.  Returns kt. */
int orc_acaplus(const orc_leaf* lf, const int* lod, const orc_bemv* b, const double* param,
                double znrmmat, double** U, double** V);
/* Fill every leaf: packs factors in the reference "contiguous" body layout
 * (HACApK_contiguous, m_HACApK_base.f90:3652-3740) with one thread range:
 * low-rank: a1 (ndt x kt) then a2 (ndl x kt); dense: a1(ndt,ndl).
 * kt[] receives ranks; offsets[] (nleaf+1) body offsets; returns body (malloc). */
double* orc_fill(int nleaf, orc_leaf* leaves, const int* lod, const orc_bemv* b,
                 const double* param, int64_t* offsets, int nthreads);
double orc_znrm(int n);                           /* znrm = 1.0/nd in default real */

/* ---- matvec: HACApK_adot_body_lfmtx_hyp_contiguous, one thread range ---- */
void orc_matvec(int n, int nleaf, const orc_leaf* leaves, const int64_t* offsets,
                const double* body, const double* u, double* au);
/* OpenMP version mirroring the reference: byte-balanced thread ranges
 * (setcutthread_lattice), per-thread zaut, atomic accumulation. */
void orc_matvec_omp(int n, int nleaf, const orc_leaf* leaves, const int64_t* offsets,
                    const double* body, const double* u, double* au, int nthreads);
/* rows[] (0-based cluster positions) of the exact operator times u: out[r] =
 * sum_j entry(lod[rows[r]], lod[j]) u[j]; OpenMP over rows */
void orc_rows_matvec(const orc_bemv* b, int n, const int* lod, int nr, const int* rows, const double* u,
                     double* out, int nthreads);

/* ---- meshes (main_LH.f90) ---- */
void orc_mesh_2dp(int n, double ds0, double* xel, double* xer, double* xcol, double* ds);
void orc_mesh_3ddip(int imax, int jmax, double ds0, double dipangle, double* xcol,
                    double* ycol, double* zcol, double* angd, double* ang);
void orc_evcalc(int n, const double* xs1, const double* xs2, const double* xs3,
                const double* ys1, const double* ys2, const double* ys3,
                const double* zs1, const double* zs2, const double* zs3, double* ev11,
                double* ev12, double* ev13, double* ev21, double* ev22, double* ev23,
                double* ev31, double* ev32, double* ev33, double* ds);

/* ---- rate-and-state RHS and Cash-Karp RK (main_LH.f90:2053-2554) ---- */
typedef struct {
  int n;              /* NCELL */
  int nmat;           /* 1 (sigma const) or 2 */
  int evlaw;          /* 0 aging, 1 slip */
  int backslip, limitsigma;
  int divide_ds0;     /* 3dph/3dnr: sum_g /= ds0 */
  double ds0, vref, minsig, maxsig;
  const double *a, *b, *dc, *f0, *vc, *taudot, *sigdot, *vplv; /* length n */
  /* H-matrices (cluster order): leaves + body for 's' and optionally 'n' */
  int nleaf_s; const orc_leaf* leaves_s; const int64_t* off_s; const double* body_s;
  int nleaf_n; const orc_leaf* leaves_n; const int64_t* off_n; const double* body_n;
  int nthreads;       /* matvec threads (1 = deterministic) */
} orc_rsf;

void orc_derivs(const orc_rsf* p, double x, const double* y, double* dydx);
void orc_rkck(const orc_rsf* p, const double* y, double x, double h, double* yout,
              double* yerr);
/* rkqs: returns 0 ok, -1 if step size underflow (reference stops) */
int orc_rkqs(const orc_rsf* p, double* y, double* x, double htry, double eps,
             double dtmax, double* hdid, double* hnext, double* errmax_gb, int* nrjct);
double orc_errmax(int len, const double* yerr, const double* ytemp, double eps);
/* the accepted-step update of main_LH.f90:1266-1287 (no viscous/opening) */
void orc_step_update(const orc_rsf* p, const double* y, double dtdid, double* psi,
                     double* tau, double* sigma, double* slip, double* vel, double* mu);

/* the time loop of main_LH.f90:1217-1438 (no output files) */
typedef struct {
  double eps_r, dtinit, dtmax, tmax, velth, velmax, velmin, dtout_inter, dtout_co;
  long long interval, nstep;
} orc_cycle_params;
#define ORC_CYCLE_REC 12
#define ORC_CYCLE_EV 6
int orc_cycle(const orc_rsf* p, const orc_cycle_params* cp, double* y, double* vel, double* slip,
              const double* ds, long long nsteps, double* rec, long long* nrec, double* ev, int max_ev,
              int* nev);

/* Cash-Karp tableau as the reference's parameter statements produce it */
void orc_cashkarp(double* a6, double* b15, double* c6, double* dc6);
/* rkqs constants: SAFETY, PGROW, PSHRNK, tiny */
void orc_rkqs_consts(double* c4);

/* ---- learned step-size proposer: 3-layer MLP, forward/backward ---- */
/* layer sizes nin -> h -> h -> 1, tanh activations; params packed
 * [W1(h x nin) b1(h) W2(h x h) b2(h) W3(1 x h) b3(1)], row-major.
 * loss = mean((out - target)^2); grad same packing. */
double orc_mlp_loss_grad(int nin, int h, int batch, const float* params, const float* x,
                         const float* target, float* grad, float* out);
double orc_mlp_loss_grad_tau(int nin, int h, int batch, const float* params, const float* x,
                             const float* target, float* grad, float* out, double tau);

#ifdef __cplusplus
}
#endif
#endif
