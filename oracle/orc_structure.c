/*
 * orc_structure.c -- oracle restatement of HACApK's cluster tree, bounding
 * boxes, admissibility recursion and leaf sort for the one-rank lattice
 * H-matrix.  TEST INFRASTRUCTURE ONLY (see hbi_oracle.h).
 *
 * Follows m_HACApK_base.f90:
 *   HACApK_init defaults          :271-302 (param(43)=1 on one rank, :286)
 *   HACApK_generate_cbitree       :3272-3333
 *   HACApK_bndbox                 :3191-3229
 *   HACApK_generate_blrleaf       :2372-2460 (root lattice block, param(42)=nd)
 *   HACApK_count_lntmx            :2878-2934 (count only, cross-check)
 *   HACApK_generate_leafmtx       :2937-2995
 *   HACApK_sort_leafmtx + qsorts  :3114-3166, HACApK_med3 HACApK_lib.f90:155-162
 */
#include "hbi_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

void orc_free(void* p) { free(p); }

void orc_default_params(double* p) {
  /* HACApK_init, m_HACApK_base.f90:271-302.  Literals such as 1.0e-6 are
   * default-real (single precision) constants in the reference and are
   * widened to real*8 on assignment. */
  for (int i = 0; i < 100; i++) p[i] = 0.0;
  p[0] = 1; p[6] = 0; p[7] = 20; p[8] = 1; p[9] = 1; p[10] = 0; p[11] = 0;
  p[20] = 15; p[21] = 1.0f; p[22] = 0; p[40] = 0; p[41] = 0;
  p[42] = 1;                 /* nrank==1 -> param(43)=1 (:286) */
  p[50] = 2.0f; p[51] = 1; p[52] = 100; p[53] = 0;
  p[59] = 2; p[60] = 3; p[61] = 7; p[62] = 1000; p[63] = 1;
  p[71] = (double)1.0e-6f;   /* ACA_EPS factor */
  p[82] = 10; p[84] = 1; p[86] = 8; p[90] = (double)1.0e-6f; p[97] = 50; p[98] = 10;
}

typedef struct {
  int nstrt, nsize, nnson;
  int son[2];
  double bmin[3], bmax[3], zwdth;
} clt_t;

typedef struct {
  clt_t* c;
  int n, cap;
  const double* g; /* coord(n,3) column-major */
  int nd;          /* md, leading dimension of g */
  int minsz;
} tree_t;

static int new_node(tree_t* t) {
  if (t->n == t->cap) {
    t->cap = t->cap ? 2 * t->cap : 256;
    t->c = (clt_t*)realloc(t->c, sizeof(clt_t) * t->cap);
  }
  memset(&t->c[t->n], 0, sizeof(clt_t));
  return t->n++;
}

#define G(t, idx1, dim) ((t)->g[(size_t)(dim) * (t)->nd + (size_t)((idx1)-1)])

/* HACApK_generate_cbitree (:3272-3333).  lod points at lod(1) of this
 * cluster's sub-range; values are 1-based element ids. */
static int cbitree(tree_t* t, int* lod, int nsrt, int nd) {
  int me = new_node(t);
  if (nd <= t->minsz) {
    t->c[me].nstrt = nsrt; t->c[me].nsize = nd; t->c[me].nnson = 0;
    return me;
  }
  double zlmin[3], zlmax[3];
  for (int id = 0; id < 3; id++) {
    zlmin[id] = G(t, lod[0], id); zlmax[id] = zlmin[id];
    for (int il = 2; il <= nd; il++) {
      double zg = G(t, lod[il - 1], id);
      if (zg < zlmin[id]) zlmin[id] = zg;
      else if (zlmax[id] < zg) zlmax[id] = zg;
    }
  }
  double zdiff = zlmax[0] - zlmin[0];
  int ncut = 0;
  for (int id = 0; id < 3; id++) {
    double zidiff = zlmax[id] - zlmin[id];
    if (zidiff > zdiff) { zdiff = zidiff; ncut = id; }
  }
  double zlmid = (zlmax[ncut] + zlmin[ncut]) / 2;
  int nl = 1, nr = nd;
  while (nl < nr) {
    while (nl < nd && G(t, lod[nl - 1], ncut) <= zlmid) nl++;
    /* reference guard is nr>=0; nr never drops below 1 because the cluster
     * minimum along ncut is <= zlmid */
    while (nr >= 1 && G(t, lod[nr - 1], ncut) > zlmid) nr--;
    if (nl < nr) { int nh = lod[nl - 1]; lod[nl - 1] = lod[nr - 1]; lod[nr - 1] = nh; }
  }
  t->c[me].nstrt = nsrt; t->c[me].nsize = nd; t->c[me].nnson = 2;
  int s1 = cbitree(t, lod, nsrt, nl - 1);
  int s2 = cbitree(t, lod + (nl - 1), nsrt + nl - 1, nd - nl + 1);
  t->c[me].son[0] = s1; t->c[me].son[1] = s2;
  return me;
}

/* HACApK_bndbox (:3191-3229) */
static void bndbox(tree_t* t, int me, const int* lod) {
  clt_t* c = &t->c[me];
  int l = 1;
  for (int ic = 0; ic < c->nnson; ic++) {
    if (ic == 0) l = 1;
    else l = l + t->c[c->son[ic - 1]].nsize;
    bndbox(t, c->son[ic], lod + (l - 1));
    c = &t->c[me];
  }
  if (c->nnson == 0) {
    for (int id = 0; id < 3; id++) { c->bmin[id] = G(t, lod[0], id); c->bmax[id] = G(t, lod[0], id); }
    for (int id = 0; id < 3; id++)
      for (int il = 2; il <= c->nsize; il++) {
        double v = G(t, lod[il - 1], id);
        if (v < c->bmin[id]) c->bmin[id] = v;
        if (c->bmax[id] < v) c->bmax[id] = v;
      }
  } else {
    clt_t* s0 = &t->c[c->son[0]];
    for (int id = 0; id < 3; id++) { c->bmin[id] = s0->bmin[id]; c->bmax[id] = s0->bmax[id]; }
    for (int il = 1; il < c->nnson; il++) {
      clt_t* s = &t->c[c->son[il]];
      for (int id = 0; id < 3; id++) {
        if (s->bmin[id] < c->bmin[id]) c->bmin[id] = s->bmin[id];
        if (c->bmax[id] < s->bmax[id]) c->bmax[id] = s->bmax[id];
      }
    }
  }
  double zwdth = (c->bmax[0] - c->bmin[0]) * (c->bmax[0] - c->bmin[0]);
  for (int id = 1; id < 3; id++) zwdth = zwdth + (c->bmax[id] - c->bmin[id]) * (c->bmax[id] - c->bmin[id]);
  c->zwdth = sqrt(zwdth);
}

typedef struct {
  orc_leaf* lf;
  int n, cap;
  int nleaf, nlmax, mdpth, p52;
  double zeta;
} leafgen_t;

static double box_dist2(const clt_t* a, const clt_t* b, int tweak) {
  double zs = 0.0;
  if (tweak)
    for (int id = 0; id < 3; id++) {
      if (a->bmax[id] != b->bmax[id]) zs = 1.0e-16;
      if (a->bmin[id] != b->bmin[id]) zs = 1.0e-16;
    }
  for (int id = 0; id < 3; id++) {
    if (a->bmax[id] < b->bmin[id]) zs = zs + (b->bmin[id] - a->bmax[id]) * (b->bmin[id] - a->bmax[id]);
    else if (b->bmax[id] < a->bmin[id]) zs = zs + (a->bmin[id] - b->bmax[id]) * (a->bmin[id] - b->bmax[id]);
  }
  return zs;
}

static void push_leaf(leafgen_t* L, int ltmtx, const clt_t* cl, const clt_t* ct) {
  if (L->n == L->cap) {
    L->cap = L->cap ? 2 * L->cap : 1024;
    L->lf = (orc_leaf*)realloc(L->lf, sizeof(orc_leaf) * L->cap);
  }
  orc_leaf* f = &L->lf[L->n++];
  f->ltmtx = ltmtx; f->kt = 0;
  f->nstrtl = cl->nstrt; f->ndl = cl->nsize;
  f->nstrtt = ct->nstrt; f->ndt = ct->nsize;
}

/* HACApK_generate_leafmtx (:2937-2995) */
static void gen_leafmtx(leafgen_t* L, const tree_t* t, int il_, int it_, int* ndpth) {
  const clt_t* cl = &t->c[il_];
  const clt_t* ct = &t->c[it_];
  int ndl = cl->nsize, ndt = ct->nsize, nstrtl = cl->nstrt, nstrtt = ct->nstrt;
  *ndpth = *ndpth + 1;
  double zs = box_dist2(cl, ct, 0);
  double zdistlt = sqrt(zs);
  if ((cl->zwdth <= L->zeta * zdistlt || ct->zwdth <= L->zeta * zdistlt) &&
      (ndl >= L->nleaf && ndt >= L->nleaf && ndl <= L->nlmax && ndt <= L->nlmax)) {
    if (L->p52 == 0 || (L->p52 == 1 && ((nstrtl + ndl) != nstrtt && (nstrtt + ndt) != nstrtl))) {
      push_leaf(L, 1, cl, ct);
      return;
    }
  }
  if (*ndpth == L->mdpth || (cl->nnson == 0 || ct->nnson == 0 || ndl <= L->nleaf || ndt <= L->nleaf)) {
    push_leaf(L, 2, cl, ct);
    return;
  }
  for (int a = 0; a < cl->nnson; a++)
    for (int b = 0; b < ct->nnson; b++) {
      gen_leafmtx(L, t, cl->son[a], ct->son[b], ndpth);
      *ndpth = *ndpth - 1;
    }
}

/* HACApK_count_lntmx (:2878-2934) -- the count the reference allocates by */
static void count_lntmx(const leafgen_t* L, const tree_t* t, int il_, int it_, int* ndpth, int* cnt) {
  const clt_t* cl = &t->c[il_];
  const clt_t* ct = &t->c[it_];
  int ndl = cl->nsize, ndt = ct->nsize, nstrtl = cl->nstrt, nstrtt = ct->nstrt;
  *ndpth = *ndpth + 1;
  double zdistlt = sqrt(box_dist2(cl, ct, 1));
  if ((cl->zwdth <= L->zeta * zdistlt || ct->zwdth <= L->zeta * zdistlt) &&
      (ndl >= L->nleaf && ndt >= L->nleaf && ndl <= L->nlmax && ndt <= L->nlmax)) {
    if (L->p52 == 0 || (L->p52 == 1 && ((nstrtl + ndl) != nstrtt && (nstrtt + ndt) != nstrtl))) {
      (*cnt)++;
      return;
    }
  }
  if (*ndpth == L->mdpth || (cl->nnson == 0 || ct->nnson == 0 || ndl <= L->nleaf || ndt <= L->nleaf)) {
    (*cnt)++;
    return;
  }
  for (int a = 0; a < cl->nnson; a++)
    for (int b = 0; b < ct->nnson; b++) {
      count_lntmx(L, t, cl->son[a], ct->son[b], ndpth, cnt);
      *ndpth = *ndpth - 1;
    }
}

/* HACApK_med3 (HACApK_lib.f90:155-162) */
static int med3(int nl, int nr, int nlr2) {
  if (nl < nr) {
    if (nr < nlr2) return nr;
    else if (nlr2 < nl) return nl;
    else return nlr2;
  } else {
    if (nlr2 < nr) return nr;
    else if (nl < nlr2) return nl;
    else return nlr2;
  }
}

/* HACApK_qsort_row_leafmtx / _col_ (:3132-3166), 1-based bounds */
static void qsort_key(orc_leaf* a, int s, int e, int bycol) {
  if (s >= e) return;
  int nl = s, nr = e, nlr2 = nl + (nr - nl) / 2;
#define KEY(x) (bycol ? a[(x)-1].nstrtt : a[(x)-1].nstrtl)
  int nmid = med3(KEY(nl), KEY(nr), KEY(nlr2));
  for (;;) {
    while (KEY(nl) < nmid) nl++;
    while (KEY(nr) > nmid) nr--;
    if (nl >= nr) break;
    orc_leaf w = a[nl - 1]; a[nl - 1] = a[nr - 1]; a[nr - 1] = w;
    nl++; nr--;
  }
#undef KEY
  qsort_key(a, s, nl - 1, bycol);
  qsort_key(a, nr + 1, e, bycol);
}

/* HACApK_sort_leafmtx (:3114-3129) */
static void sort_leafmtx(orc_leaf* a, int nlf) {
  qsort_key(a, 1, nlf, 0);
  int ilp = 1, ips = 1;
  for (int ip = 1; ip <= nlf; ip++) {
    int il = a[ip - 1].nstrtl;
    if (il > ilp) {
      qsort_key(a, ips, ip - 1, 1);
      ilp = il; ips = ip;
    }
  }
  qsort_key(a, ips, nlf, 1);
}

int orc_build_structure(int n, const double* coord, const double* param, int* lod,
                        orc_leaf** leaves_out, int* count_check) {
  double pdef[100];
  if (!param) { orc_default_params(pdef); param = pdef; }
  tree_t t = {0};
  t.g = coord; t.nd = n;
  t.minsz = (int)param[20];
  for (int i = 0; i < n; i++) lod[i] = i + 1;
  int root = cbitree(&t, lod, 1, n);
  bndbox(&t, root, lod);

  /* one rank: npgl=1, param(42)=nd/param(43)/npgl (generate_frame_blrleaf
   * :690), so the root pair is the single lattice block. */
  double p42 = (double)n / param[42] / 1.0;
  int nlttcblk = (int)(p42 + 1);
  leafgen_t L = {0};
  L.nleaf = (int)(param[20] + 1);
  L.nlmax = (int)(param[21] * n);
  L.mdpth = (int)param[52];
  L.p52 = (int)param[51];
  L.zeta = param[50];
  const clt_t* r = &t.c[root];
  int ndpth = 1;
  int cnt = 0;
  if (r->nsize < nlttcblk) {
    /* lattice-block level decision (:2396-2450) with the touching tweak */
    double zdistlt = sqrt(box_dist2(r, r, 1));
    if (r->zwdth <= L.zeta * zdistlt) {
      push_leaf(&L, 1, r, r); cnt = 1;
    } else if (ndpth == L.mdpth || r->nnson == 0 || (r->nsize <= L.nleaf && r->nsize <= L.nleaf)) {
      push_leaf(&L, 2, r, r); cnt = 1;
    } else {
      for (int a = 0; a < r->nnson; a++)
        for (int b = 0; b < r->nnson; b++) {
          int d = ndpth, dc = ndpth;
          gen_leafmtx(&L, &t, r->son[a], r->son[b], &d);
          count_lntmx(&L, &t, r->son[a], r->son[b], &dc, &cnt);
        }
    }
  }
  free(t.c);
  sort_leafmtx(L.lf, L.n);
  if (count_check) *count_check = cnt;
  *leaves_out = L.lf;
  return L.n;
}
