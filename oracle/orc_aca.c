/*
 * orc_aca.c -- oracle restatement of ACA+ assembly, leaf fill, contiguous
 * packing and the lattice H-matrix-vector product.  TEST INFRASTRUCTURE ONLY.
 *
 *   HACApK_unrm_d, maxabsvalloc_d, minabsvalloc_d, adot_dsm, adotsub_dsm
 *                                     HACApK_lib.f90:31-116
 *   HACApK_calc_vec                   m_HACApK_base.f90:1638-1659
 *   HACApK_acaplus                    m_HACApK_base.f90:1748-1946
 *   HACApK_fill_leafmtx_hyp           m_HACApK_base.f90:1949-2043
 *   znrm (param(61)=3)                m_HACApK_use.f90:191-202
 *   HACApK_setcutthread_lattice       m_HACApK_use.f90:387-431
 *   HACApK_contiguous                 m_HACApK_base.f90:3652-3740
 *   HACApK_adot_body_lfmtx_hyp_contiguous  m_HACApK_solve.f90:2108-2164
 *
 * The reference allocates the ACA scratch zaa/zab without initialising it and
 * one stop branch of ACA+ can fold an unwritten column into the update; this
 * restatement zero-fills the scratch, which is what a fresh large allocation
 * holds.
 */
#include "hbi_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

double orc_znrm(int n) { return (double)(1.0f / (float)n); }

/* HACApK_unrm_d */
static double unrm_d(int nd, const double* za) {
  double zscl = 0.0, zzz = 1.0;
  for (int il = 0; il < nd; il++) {
    double zza = fabs(za[il]);
    if (zza < 1.0e-30) continue;
    if (zscl < zza) {
      zzz = 1.0 + zzz * (zscl / zza) * (zscl / zza);
      zscl = zza;
    } else {
      zzz = zzz + (zza / zscl) * (zza / zscl);
    }
  }
  return zscl * sqrt(zzz);
}

/* HACApK_maxabsvalloc_d: il 1-based */
static void maxabsvalloc(const double* za, double* zz, int* il, int nd) {
  *il = 1; *zz = fabs(za[0]);
  for (int it = 2; it <= nd; it++)
    if (fabs(za[it - 1]) > *zz) { *il = it; *zz = fabs(za[it - 1]); }
}
static void minabsvalloc(const double* za, double* zz, int* il, int nd) {
  *il = 1; *zz = fabs(za[0]);
  for (int it = 2; it <= nd; it++)
    if (fabs(za[it - 1]) < *zz) { *il = it; *zz = fabs(za[it - 1]); }
}

typedef struct {
  double *zaa, *zab; /* zaa(ndl, kcap), zab(ndt, kcap), column-major */
  int ndl, ndt, kcap;
} acabuf_t;

static void ensure_cols(acabuf_t* b, int need) {
  if (need <= b->kcap) return;
  int nc = b->kcap * 2;
  if (nc < need) nc = need;
  double* a = (double*)calloc((size_t)b->ndl * nc, sizeof(double));
  double* c = (double*)calloc((size_t)b->ndt * nc, sizeof(double));
  memcpy(a, b->zaa, sizeof(double) * (size_t)b->ndl * b->kcap);
  memcpy(c, b->zab, sizeof(double) * (size_t)b->ndt * b->kcap);
  free(b->zaa); free(b->zab);
  b->zaa = a; b->zab = c; b->kcap = nc;
}

/* HACApK_calc_vec.  fac: ndp x k factor (column-major, leading dim ldf);
 * coef: other-side factor, row ip taken as zz(1:k) (leading dim ldc).
 * ld==0: row direction (vec over columns), ld==1: column direction. */
static void calc_vec(const double* fac, int ldf, const double* coef, int ldc, int ndp, int k, int ip,
                     double* vec, int nstrtl, int nstrtt, const int* lod, const orc_bemv* bv,
                     const int* lmsk, int ld) {
  for (int ii = 1; ii <= ndp; ii++) {
    if (lmsk[ii - 1] == 0) {
      int ill, itt;
      if (ld == 0) { ill = ip + nstrtl - 1; itt = ii + nstrtt - 1; }
      else { ill = ii + nstrtl - 1; itt = ip + nstrtt - 1; }
      vec[ii - 1] = orc_entry_ij(lod[ill - 1], lod[itt - 1], bv);
    }
  }
  if (k == 0) return;
  /* adotsub_dsm: zau = sum_it fac(:,it)*zz(it); vec = vec - zau */
  for (int ii = 0; ii < ndp; ii++) {
    double zau = 0.0;
    for (int it = 0; it < k; it++) zau = zau + fac[(size_t)it * ldf + ii] * coef[(size_t)it * ldc + (ip - 1)];
    vec[ii] = vec[ii] - zau;
  }
  for (int ii = 0; ii < ndp; ii++)
    if (lmsk[ii] == 1) vec[ii] = 0.0;
}

int orc_acaplus(const orc_leaf* lf, const int* lod, const orc_bemv* bv, const double* param,
                double znrmmat, double** Uout, double** Vout) {
  const int ndl = lf->ndl, ndt = lf->ndt, nstrtl = lf->nstrtl, nstrtt = lf->nstrtt;
  const double eps = param[70];
  const double pACA_EPS = param[71] * eps;
  const int kmax = (int)param[62];
  const double p64 = param[63];
  const double za_ACA_EPS = (double)1.0e-30f;
  double znrm = znrmmat * (double)sqrtf((float)ndl * (float)ndt);
  double ACA_EPS = 0.0;
  if (param[60] == 2 || param[60] == 1) ACA_EPS = pACA_EPS;
  if (param[60] == 3) ACA_EPS = pACA_EPS * znrm;

  acabuf_t B;
  B.ndl = ndl; B.ndt = ndt;
  B.kcap = (ndl < ndt ? ndl : ndt) + 2;
  if (B.kcap > kmax) B.kcap = kmax;
  if (B.kcap < 2) B.kcap = 2;
  B.zaa = (double*)calloc((size_t)ndl * B.kcap, sizeof(double));
  B.zab = (double*)calloc((size_t)ndt * B.kcap, sizeof(double));
  int ntries = (ndl > ndt ? ndl : ndt) + 1, ntries_row = 6, ntries_col = 6;
  int* lrow_msk = (int*)calloc(ndl, sizeof(int));
  int* lcol_msk = (int*)calloc(ndt, sizeof(int));
  double* pa_ref = (double*)calloc(ndl, sizeof(double));
  double* pb_ref = (double*)calloc(ndt, sizeof(double));
  int k = 0;

  int j_ref = 1, i_ref;
  calc_vec(B.zaa, ndl, B.zab, ndt, ndl, k, j_ref, pa_ref, nstrtl, nstrtt, lod, bv, lrow_msk, 1);
  double colnorm = unrm_d(ndl, pa_ref);
  double rownorm;
  minabsvalloc(pa_ref, &rownorm, &i_ref, ndl);
  calc_vec(B.zab, ndt, B.zaa, ndl, ndt, k, i_ref, pb_ref, nstrtl, nstrtt, lod, bv, lcol_msk, 0);
  rownorm = unrm_d(ndt, pb_ref);
  double apxnorm = 0.0;
  int lstop = 0;
  double col_maxval, row_maxval, zinvmax, blknorm;
  int i, j;

  while ((k < kmax) && (ntries_row > 0 || ntries_col > 0) && (ntries > 0)) {
    ntries--;
    ensure_cols(&B, k + 1);
    double* pcol = B.zaa + (size_t)k * ndl;
    double* prow = B.zab + (size_t)k * ndt;
    col_maxval = 0.0; maxabsvalloc(pa_ref, &col_maxval, &i, ndl);
    row_maxval = 0.0; maxabsvalloc(pb_ref, &row_maxval, &j, ndt);
    if (row_maxval > col_maxval) {
      if (j != j_ref) calc_vec(B.zaa, ndl, B.zab, ndt, ndl, k, j, pcol, nstrtl, nstrtt, lod, bv, lrow_msk, 1);
      else memcpy(pcol, pa_ref, sizeof(double) * ndl);
      maxabsvalloc(pcol, &col_maxval, &i, ndl);
      if (col_maxval < ACA_EPS && k >= p64) {
        lstop = 1;
      } else {
        calc_vec(B.zab, ndt, B.zaa, ndl, ndt, k, i, prow, nstrtl, nstrtt, lod, bv, lcol_msk, 0);
        if (fabs(pcol[i - 1]) > (double)1.0e-20f) zinvmax = 1.0 / pcol[i - 1];
        else { k = k - 1 > 0 ? k - 1 : 0; break; }
        for (int ii = 0; ii < ndl; ii++) pcol[ii] = pcol[ii] * zinvmax;
      }
    } else {
      if (i != i_ref) calc_vec(B.zab, ndt, B.zaa, ndl, ndt, k, i, prow, nstrtl, nstrtt, lod, bv, lcol_msk, 0);
      else memcpy(prow, pb_ref, sizeof(double) * ndt);
      maxabsvalloc(prow, &row_maxval, &j, ndt);
      if (row_maxval < ACA_EPS && k >= p64) {
        lstop = 1;
      } else {
        calc_vec(B.zaa, ndl, B.zab, ndt, ndl, k, j, pcol, nstrtl, nstrtt, lod, bv, lrow_msk, 1);
        if (fabs(prow[j - 1]) > (double)1.0e-20f) zinvmax = 1.0 / prow[j - 1];
        else { k = k - 1 > 0 ? k - 1 : 0; break; }
        for (int ii = 0; ii < ndt; ii++) prow[ii] = prow[ii] * zinvmax;
      }
    }
    lrow_msk[i - 1] = 1; lcol_msk[j - 1] = 1;

    if (i != i_ref) {
      zinvmax = -pcol[i_ref - 1];
      for (int ii = 0; ii < ndt; ii++) pb_ref[ii] = pb_ref[ii] + prow[ii] * zinvmax;
      rownorm = unrm_d(ndt, pb_ref);
    }
    if (i == i_ref || rownorm < ACA_EPS) {
      if (i == i_ref) ntries_row++;
      if (ntries_row > 0) {
        rownorm = 0.0; i = i_ref;
        while (i != ((i_ref + ndl - 2) % ndl) + 1 && rownorm < za_ACA_EPS && ntries_row > 0) {
          if (lrow_msk[i - 1] == 0) {
            ensure_cols(&B, k + 1);
            calc_vec(B.zab, ndt, B.zaa, ndl, ndt, k + 1, i, pb_ref, nstrtl, nstrtt, lod, bv, lcol_msk, 0);
            rownorm = unrm_d(ndt, pb_ref);
            if (rownorm < ACA_EPS) lrow_msk[i - 1] = 1;
            ntries_row--;
          } else {
            rownorm = 0.0;
          }
          i = (i % ndl) + 1;
        }
        i_ref = ((i + ndl - 2) % ndl) + 1;
      }
    }
    /* pointers may have moved if ensure_cols grew the buffers */
    pcol = B.zaa + (size_t)k * ndl;
    prow = B.zab + (size_t)k * ndt;

    if (j != j_ref) {
      zinvmax = -prow[j_ref - 1];
      for (int ii = 0; ii < ndl; ii++) pa_ref[ii] = pa_ref[ii] + pcol[ii] * zinvmax;
      colnorm = unrm_d(ndl, pa_ref);
    }
    if (j == j_ref || colnorm < ACA_EPS) {
      if (j == j_ref) ntries_col++;
      if (ntries_col > 0) {
        colnorm = 0.0; j = j_ref;
        while (j != ((j_ref + ndt - 2) % ndt) + 1 && colnorm < za_ACA_EPS && ntries_col > 0) {
          if (lcol_msk[j - 1] == 0) {
            calc_vec(B.zaa, ndl, B.zab, ndt, ndl, k + 1, j, pa_ref, nstrtl, nstrtt, lod, bv, lrow_msk, 1);
            colnorm = unrm_d(ndl, pa_ref);
            if (colnorm < ACA_EPS) lcol_msk[j - 1] = 1;
            ntries_col--;
          } else {
            colnorm = 0.0;
          }
          j = (j % ndt) + 1;
        }
        j_ref = ((j + ndt - 2) % ndt) + 1;
      }
    }

    if (colnorm < ACA_EPS && rownorm < ACA_EPS && k >= p64) { lstop = 1; k = k + 1; }

    if (lstop == 0) {
      blknorm = (unrm_d(ndl, pcol) * unrm_d(ndt, prow));
      if (k == 0) {
        if (param[60] == 1) apxnorm = blknorm;
        else apxnorm = znrm;
      } else {
        if (blknorm < apxnorm * eps && rownorm < apxnorm * eps && colnorm < apxnorm * eps && k >= p64)
          lstop = 1;
      }
    }
    if (lstop == 1 && k >= p64) break;
    k = k + 1;
  }
  free(lrow_msk); free(lcol_msk); free(pa_ref); free(pb_ref);
  int kt = k;
  ensure_cols(&B, kt > 0 ? kt : 1);
  double* U = (double*)malloc(sizeof(double) * (size_t)ndl * (kt > 0 ? kt : 1));
  double* V = (double*)malloc(sizeof(double) * (size_t)ndt * (kt > 0 ? kt : 1));
  memcpy(U, B.zaa, sizeof(double) * (size_t)ndl * kt);
  memcpy(V, B.zab, sizeof(double) * (size_t)ndt * kt);
  free(B.zaa); free(B.zab);
  *Uout = U; *Vout = V;
  return kt;
}

double* orc_fill(int nleaf, orc_leaf* leaves, const int* lod, const orc_bemv* bv,
                 const double* param, int64_t* offsets, int nthreads) {
  double znrm = orc_znrm(bv->n);
  double** U = (double**)calloc(nleaf, sizeof(double*));
  double** V = (double**)calloc(nleaf, sizeof(double*));
#ifdef _OPENMP
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
  for (int ip = 0; ip < nleaf; ip++) {
    orc_leaf* lf = &leaves[ip];
    if (lf->ltmtx == 1) {
      lf->kt = orc_acaplus(lf, lod, bv, param, znrm, &U[ip], &V[ip]);
    } else {
      /* dense: a1(it,il) = entry(lod(ill), lod(itt)), stored a1(ndt,ndl) */
      double* a1 = (double*)malloc(sizeof(double) * (size_t)lf->ndt * lf->ndl);
      for (int il = 1; il <= lf->ndl; il++) {
        int ill = il + lf->nstrtl - 1;
        for (int it = 1; it <= lf->ndt; it++) {
          int itt = it + lf->nstrtt - 1;
          a1[(size_t)(il - 1) * lf->ndt + (it - 1)] = orc_entry_ij(lod[ill - 1], lod[itt - 1], bv);
        }
      }
      V[ip] = a1;
      lf->kt = 0;
    }
  }
  int64_t tot = 0;
  for (int ip = 0; ip < nleaf; ip++) {
    offsets[ip] = tot;
    if (leaves[ip].ltmtx == 1) tot += (int64_t)leaves[ip].kt * (leaves[ip].ndl + leaves[ip].ndt);
    else tot += (int64_t)leaves[ip].ndl * leaves[ip].ndt;
  }
  offsets[nleaf] = tot;
  double* body = (double*)malloc(sizeof(double) * (size_t)(tot > 0 ? tot : 1));
  for (int ip = 0; ip < nleaf; ip++) {
    const orc_leaf* lf = &leaves[ip];
    double* o = body + offsets[ip];
    if (lf->ltmtx == 1) {
      memcpy(o, V[ip], sizeof(double) * (size_t)lf->ndt * lf->kt);
      memcpy(o + (size_t)lf->ndt * lf->kt, U[ip], sizeof(double) * (size_t)lf->ndl * lf->kt);
      free(U[ip]);
    } else {
      memcpy(o, V[ip], sizeof(double) * (size_t)lf->ndt * lf->ndl);
    }
    free(V[ip]);
  }
  free(U); free(V);
  return body;
}

/* body of one thread range [s,e) of HACApK_adot_body_lfmtx_hyp_contiguous */
static void matvec_range(int s, int e, const orc_leaf* leaves, const int64_t* offsets,
                         const double* body, const double* zu, double* zaut, double* zbut, int* ls,
                         int* le) {
  for (int ip = s; ip < e; ip++) {
    const orc_leaf* lf = &leaves[ip];
    int ndl = lf->ndl, ndt = lf->ndt, nstrtl = lf->nstrtl, nstrtt = lf->nstrtt;
    if (nstrtl < *ls) *ls = nstrtl;
    if (nstrtl + ndl - 1 > *le) *le = nstrtl + ndl - 1;
    int64_t idx = offsets[ip];
    if (lf->ltmtx == 1) {
      int kt = lf->kt;
      for (int il = 0; il < kt; il++) zbut[il] = 0.0;
      for (int il = 0; il < kt; il++) {
        for (int it = 1; it <= ndt; it++) {
          int itt = it + nstrtt - 1;
          zbut[il] = zbut[il] + body[idx + it - 1] * zu[itt - 1];
        }
        idx += ndt;
      }
      for (int il = 0; il < kt; il++) {
        for (int it = 1; it <= ndl; it++) {
          int ill = it + nstrtl - 1;
          zaut[ill - 1] = zaut[ill - 1] + body[idx + it - 1] * zbut[il];
        }
        idx += ndl;
      }
    } else {
      for (int il = 1; il <= ndl; il++) {
        int ill = il + nstrtl - 1;
        for (int it = 1; it <= ndt; it++) {
          int itt = it + nstrtt - 1;
          zaut[ill - 1] = zaut[ill - 1] + body[idx + it - 1] * zu[itt - 1];
        }
        idx += ndt;
      }
    }
  }
}

static int ktmax_of(int nleaf, const orc_leaf* leaves) {
  int m = 1;
  for (int i = 0; i < nleaf; i++)
    if (leaves[i].ltmtx == 1 && leaves[i].kt > m) m = leaves[i].kt;
  return m;
}

void orc_matvec(int n, int nleaf, const orc_leaf* leaves, const int64_t* offsets,
                const double* body, const double* u, double* au) {
  double* zaut = (double*)calloc(n, sizeof(double));
  double* zbut = (double*)malloc(sizeof(double) * ktmax_of(nleaf, leaves));
  int ls = n, le = 1;
  matvec_range(0, nleaf, leaves, offsets, body, u, zaut, zbut, &ls, &le);
  for (int i = 0; i < n; i++) au[i] = 0.0;
  for (int il = ls; il <= le; il++) au[il - 1] = au[il - 1] + zaut[il - 1];
  free(zaut); free(zbut);
}

/* thread ranges of HACApK_setcutthread_lattice (m_HACApK_use.f90:387-431) */
static void cut_threads(int nleaf, const orc_leaf* leaves, int nthr, int* lthr) {
  int64_t mem8 = 0;
  for (int ip = 0; ip < nleaf; ip++) {
    const orc_leaf* f = &leaves[ip];
    if (f->ltmtx == 1) mem8 += (int64_t)(f->ndt + f->ndl) * f->kt;
    else mem8 += (int64_t)f->ndl * f->ndt;
  }
  int64_t nth1_mem = mem8 / nthr;
  lthr[0] = 1;
  for (int t = 1; t <= nthr; t++) lthr[t] = nleaf + 1;
  int64_t imem = 0;
  int ith = 1;
  for (int il = 1; il <= nleaf; il++) {
    const orc_leaf* f = &leaves[il - 1];
    if (f->ltmtx == 1) imem += (int64_t)(f->ndl + f->ndt) * f->kt;
    else imem += (int64_t)f->ndl * f->ndt;
    if (imem > nth1_mem * ith) {
      lthr[ith] = il;
      ith++;
      if (ith == nthr) break;
    }
  }
}

void orc_matvec_omp(int n, int nleaf, const orc_leaf* leaves, const int64_t* offsets,
                    const double* body, const double* u, double* au, int nthreads) {
#ifdef _OPENMP
  if (nthreads < 1) nthreads = omp_get_max_threads();
  int* lthr = (int*)malloc(sizeof(int) * (nthreads + 1));
  cut_threads(nleaf, leaves, nthreads, lthr);
  int ktm = ktmax_of(nleaf, leaves);
  for (int i = 0; i < n; i++) au[i] = 0.0;
#pragma omp parallel num_threads(nthreads)
  {
    int ith = omp_get_thread_num();
    double* zaut = (double*)calloc(n, sizeof(double));
    double* zbut = (double*)malloc(sizeof(double) * ktm);
    int ls = n, le = 1;
    matvec_range(lthr[ith] - 1, lthr[ith + 1] - 1, leaves, offsets, body, u, zaut, zbut, &ls, &le);
    for (int il = ls; il <= le; il++) {
#pragma omp atomic
      au[il - 1] += zaut[il - 1];
    }
    free(zaut); free(zbut);
  }
  free(lthr);
#else
  (void)nthreads;
  orc_matvec(n, nleaf, leaves, offsets, body, u, au);
#endif
}

/* Rows of the exact operator times u, for parity checks at sizes where the
 * dense matrix does not fit: out[r] = sum_j entry(lod[rows[r]], lod[j]) u[j]
 * with rows[] 0-based cluster-order positions and u in cluster order (the
 * lattice vector of the reference).  Each row is summed serially in j order;
 * rows are spread over the threads. */
void orc_rows_matvec(const orc_bemv* b, int n, const int* lod, int nr, const int* rows, const double* u,
                     double* out, int nthreads) {
#ifdef _OPENMP
  if (nthreads < 1) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
  for (int r = 0; r < nr; r++) {
    const int gi = lod[rows[r]];
    double t = 0.0;
    for (int j = 0; j < n; j++) t += orc_entry_ij(gi, lod[j], b) * u[j];
    out[r] = t;
  }
#ifndef _OPENMP
  (void)nthreads;
#endif
}
