// hbi_aca_impl.cuh -- the ACA+ / dense-fill / entry kernels as templates on
// the problem kind, included by one translation unit per problem family
// (hbi_aca.cu, hbi_aca_okada.cu, hbi_aca_td.cu, hbi_aca_tdhs.cu) so that the
// large Green's functions compile in parallel.
//
// One CTA runs ACA+ (HACApK_acaplus, m_HACApK_base.f90:1748-1946) for one
// admissible leaf.  Pivot search, residual updates and stopping tests are
// FP64; the Green's-function entries are evaluated in the CTA (no callback).
// The control flow (reference row/column, retries, the three stopping tests)
// is the reference's; every thread executes it uniformly on block-reduced
// scalars.  Norms are HACApK's scaled 2-norm combined in a fixed tree, so
// they are deterministic but may differ from the serial loop in the last bit.
#pragma once
#include <cstdint>

#include "hbi_entries.cuh"
#include "hbi_kernels.cuh"

namespace hbi {

struct AcaShared {
  double rv[HBI_ACA_NT];
  double rq[HBI_ACA_NT];
  int ri[HBI_ACA_NT];
};

// ---- block reductions ----------------------------------------------------
// first index of max |v| (HACApK_maxabsvalloc_d); returns 1-based index
template <int NT>
__device__ int blk_argmax_abs(const double* v, int n, double* outv, AcaShared& sh) {
  double best = -1.0;
  int bi = 0x7fffffff;
  for (int i = threadIdx.x; i < n; i += NT) {
    double a = fabs(v[i]);
    if (a > best) { best = a; bi = i; }
  }
  sh.rv[threadIdx.x] = best; sh.ri[threadIdx.x] = bi;
  __syncthreads();
  for (int s = NT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      double b2 = sh.rv[threadIdx.x + s]; int i2 = sh.ri[threadIdx.x + s];
      double b1 = sh.rv[threadIdx.x]; int i1 = sh.ri[threadIdx.x];
      if (b2 > b1 || (b2 == b1 && i2 < i1)) { sh.rv[threadIdx.x] = b2; sh.ri[threadIdx.x] = i2; }
    }
    __syncthreads();
  }
  double rv = sh.rv[0]; int ri = sh.ri[0];
  __syncthreads();
  *outv = rv;
  return ri + 1;
}

// first index of min |v| (HACApK_minabsvalloc_d); returns 1-based index
template <int NT>
__device__ int blk_argmin_abs(const double* v, int n, double* outv, AcaShared& sh) {
  double best = __longlong_as_double(0x7ff0000000000000ULL);
  int bi = 0x7fffffff;
  for (int i = threadIdx.x; i < n; i += NT) {
    double a = fabs(v[i]);
    if (a < best) { best = a; bi = i; }
  }
  sh.rv[threadIdx.x] = best; sh.ri[threadIdx.x] = bi;
  __syncthreads();
  for (int s = NT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      double b2 = sh.rv[threadIdx.x + s]; int i2 = sh.ri[threadIdx.x + s];
      double b1 = sh.rv[threadIdx.x]; int i1 = sh.ri[threadIdx.x];
      if (b2 < b1 || (b2 == b1 && i2 < i1)) { sh.rv[threadIdx.x] = b2; sh.ri[threadIdx.x] = i2; }
    }
    __syncthreads();
  }
  double rv = sh.rv[0]; int ri = sh.ri[0];
  __syncthreads();
  *outv = rv;
  return (ri == 0x7fffffff ? 0 : ri) + 1;
}

// HACApK_unrm_d: scaled 2-norm; per-thread scaled sums, pairwise combined
template <int NT>
__device__ double blk_unrm(const double* v, int n, AcaShared& sh) {
  double scl = 0.0, ssq = 1.0;
  for (int i = threadIdx.x; i < n; i += NT) {
    double a = fabs(v[i]);
    if (a < 1.0e-30) continue;
    if (scl < a) { double t = scl / a; ssq = 1.0 + ssq * t * t; scl = a; }
    else { double t = a / scl; ssq = ssq + t * t; }
  }
  sh.rv[threadIdx.x] = scl; sh.rq[threadIdx.x] = ssq;
  __syncthreads();
  for (int s = NT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      double s1 = sh.rv[threadIdx.x], q1 = sh.rq[threadIdx.x];
      double s2 = sh.rv[threadIdx.x + s], q2 = sh.rq[threadIdx.x + s];
      if (s2 > 0.0) {
        if (s1 < s2) { double t = s1 / s2; q1 = q2 + (s1 > 0.0 ? q1 * t * t : 0.0); s1 = s2; }
        else { double t = s2 / s1; q1 = q1 + q2 * t * t; }
      }
      sh.rv[threadIdx.x] = s1; sh.rq[threadIdx.x] = q1;
    }
    __syncthreads();
  }
  double r = sh.rv[0] * sqrt(sh.rq[0]);
  __syncthreads();
  return r;
}

// HACApK_calc_vec: vec(ii) = A(.,.) - sum_{it<k} fac(ii,it)*coef(ip,it); masked -> 0
template <int PROB, int NT>
__device__ void calc_vec(const DevBemv& b, const int* lod, const double* fac, int ldf, const double* coef, int ldc,
                         int ndp, int k, int ip, double* vec, int row0, int col0, const int* msk, int ld) {
  for (int ii = threadIdx.x; ii < ndp; ii += NT) {
    double v = vec[ii];
    if (msk[ii] == 0) {
      int gi, gj;
      if (ld == 0) { gi = lod[row0 + ip - 1] - 1; gj = lod[col0 + ii] - 1; }
      else { gi = lod[row0 + ii] - 1; gj = lod[col0 + ip - 1] - 1; }
      v = entry<PROB>(b, gi, gj);
    }
    if (k > 0) {
      double zau = 0.0;
      for (int it = 0; it < k; it++)
        zau = __dadd_rn(zau, __dmul_rn(fac[(size_t)it * ldf + ii], __ldg(&coef[(size_t)it * ldc + ip - 1])));
      v = __dsub_rn(v, zau);
      if (msk[ii] == 1) v = 0.0;
    }
    vec[ii] = v;
  }
  __syncthreads();
}

template <int NT>
__device__ void vcopy(double* dst, const double* src, int n) {
  for (int i = threadIdx.x; i < n; i += NT) dst[i] = src[i];
  __syncthreads();
}
template <int NT>
__device__ void vscale(double* v, int n, double s) {
  for (int i = threadIdx.x; i < n; i += NT) v[i] = __dmul_rn(v[i], s);
  __syncthreads();
}
template <int NT>
__device__ void vaxpy(double* y, const double* x, int n, double s) {
  for (int i = threadIdx.x; i < n; i += NT) y[i] = __dadd_rn(y[i], __dmul_rn(x[i], s));
  __syncthreads();
}
__device__ __forceinline__ double rd_shared(const double* p, double* sh) {
  if (threadIdx.x == 0) *sh = *p;
  __syncthreads();
  double v = *sh;
  __syncthreads();
  return v;
}

template <int PROB, int NT>
__global__ void __launch_bounds__(NT) aca_plus_kernel(DevBemv b, const int* __restrict__ lod, const AcaTask* tasks,
                                                      double* arena, int* result, AcaParams P) {
  __shared__ AcaShared sh;
  __shared__ double bcast;
  const AcaTask T = tasks[blockIdx.x];
  const int ndl = T.ndl, ndt = T.ndt, row0 = T.nstrtl - 1, col0 = T.nstrtt - 1;
  const int kcap = T.kcap, kmax = P.kmax;
  double* zaa = arena + T.scratch;            // ndl x kcap
  double* zab = zaa + (size_t)ndl * kcap;     // ndt x kcap
  double* pa_ref = zab + (size_t)ndt * kcap;  // ndl
  double* pb_ref = pa_ref + ndl;              // ndt
  int* lrow = (int*)(pb_ref + ndt);           // ndl
  int* lcol = lrow + ndl;                     // ndt

  const double eps = P.eps;
  const double p64 = P.kmin;
  const double za_ACA_EPS = (double)1.0e-30f;
  const double znrm = P.znrmmat * (double)sqrtf((float)ndl * (float)ndt);
  const double ACA_EPS = P.pACA_EPS * znrm;
  int ntries = max(ndl, ndt) + 1, ntries_row = 6, ntries_col = 6;
  int k = 0, status = 0;

  int j_ref = 1, i_ref;
  calc_vec<PROB, NT>(b, lod, zaa, ndl, zab, ndt, ndl, 0, j_ref, pa_ref, row0, col0, lrow, 1);
  double colnorm = blk_unrm<NT>(pa_ref, ndl, sh);
  double rownorm;
  i_ref = blk_argmin_abs<NT>(pa_ref, ndl, &rownorm, sh);
  calc_vec<PROB, NT>(b, lod, zab, ndt, zaa, ndl, ndt, 0, i_ref, pb_ref, row0, col0, lcol, 0);
  rownorm = blk_unrm<NT>(pb_ref, ndt, sh);
  double apxnorm = 0.0;
  int lstop = 0;
  double col_maxval, row_maxval, zinvmax, blknorm;
  int i, j;

  while ((k < kmax) && (ntries_row > 0 || ntries_col > 0) && (ntries > 0)) {
    ntries--;
    if (k + 1 > kcap) { status = -2; break; }
    double* pcol = zaa + (size_t)k * ndl;
    double* prow = zab + (size_t)k * ndt;
    i = blk_argmax_abs<NT>(pa_ref, ndl, &col_maxval, sh);
    j = blk_argmax_abs<NT>(pb_ref, ndt, &row_maxval, sh);
    bool brk = false;
    if (row_maxval > col_maxval) {
      if (j != j_ref) calc_vec<PROB, NT>(b, lod, zaa, ndl, zab, ndt, ndl, k, j, pcol, row0, col0, lrow, 1);
      else vcopy<NT>(pcol, pa_ref, ndl);
      i = blk_argmax_abs<NT>(pcol, ndl, &col_maxval, sh);
      if (col_maxval < ACA_EPS && k >= p64) {
        lstop = 1;
      } else {
        calc_vec<PROB, NT>(b, lod, zab, ndt, zaa, ndl, ndt, k, i, prow, row0, col0, lcol, 0);
        double piv = rd_shared(&pcol[i - 1], &bcast);
        if (fabs(piv) > (double)1.0e-20f) zinvmax = 1.0 / piv;
        else { k = max(k - 1, 0); brk = true; }
        if (!brk) vscale<NT>(pcol, ndl, zinvmax);
      }
    } else {
      if (i != i_ref) calc_vec<PROB, NT>(b, lod, zab, ndt, zaa, ndl, ndt, k, i, prow, row0, col0, lcol, 0);
      else vcopy<NT>(prow, pb_ref, ndt);
      j = blk_argmax_abs<NT>(prow, ndt, &row_maxval, sh);
      if (row_maxval < ACA_EPS && k >= p64) {
        lstop = 1;
      } else {
        calc_vec<PROB, NT>(b, lod, zaa, ndl, zab, ndt, ndl, k, j, pcol, row0, col0, lrow, 1);
        double piv = rd_shared(&prow[j - 1], &bcast);
        if (fabs(piv) > (double)1.0e-20f) zinvmax = 1.0 / piv;
        else { k = max(k - 1, 0); brk = true; }
        if (!brk) vscale<NT>(prow, ndt, zinvmax);
      }
    }
    if (brk) break;
    if (threadIdx.x == 0) { lrow[i - 1] = 1; lcol[j - 1] = 1; }
    __syncthreads();

    if (i != i_ref) {
      zinvmax = -rd_shared(&pcol[i_ref - 1], &bcast);
      vaxpy<NT>(pb_ref, prow, ndt, zinvmax);
      rownorm = blk_unrm<NT>(pb_ref, ndt, sh);
    }
    if (i == i_ref || rownorm < ACA_EPS) {
      if (i == i_ref) ntries_row++;
      if (ntries_row > 0) {
        rownorm = 0.0; i = i_ref;
        while (i != ((i_ref + ndl - 2) % ndl) + 1 && rownorm < za_ACA_EPS && ntries_row > 0) {
          int m = lrow[i - 1];
          __syncthreads();
          if (m == 0) {
            calc_vec<PROB, NT>(b, lod, zab, ndt, zaa, ndl, ndt, k + 1, i, pb_ref, row0, col0, lcol, 0);
            rownorm = blk_unrm<NT>(pb_ref, ndt, sh);
            if (rownorm < ACA_EPS) { if (threadIdx.x == 0) lrow[i - 1] = 1; __syncthreads(); }
            ntries_row--;
          } else {
            rownorm = 0.0;
          }
          i = (i % ndl) + 1;
        }
        i_ref = ((i + ndl - 2) % ndl) + 1;
      }
    }
    if (j != j_ref) {
      zinvmax = -rd_shared(&prow[j_ref - 1], &bcast);
      vaxpy<NT>(pa_ref, pcol, ndl, zinvmax);
      colnorm = blk_unrm<NT>(pa_ref, ndl, sh);
    }
    if (j == j_ref || colnorm < ACA_EPS) {
      if (j == j_ref) ntries_col++;
      if (ntries_col > 0) {
        colnorm = 0.0; j = j_ref;
        while (j != ((j_ref + ndt - 2) % ndt) + 1 && colnorm < za_ACA_EPS && ntries_col > 0) {
          int m = lcol[j - 1];
          __syncthreads();
          if (m == 0) {
            calc_vec<PROB, NT>(b, lod, zaa, ndl, zab, ndt, ndl, k + 1, j, pa_ref, row0, col0, lrow, 1);
            colnorm = blk_unrm<NT>(pa_ref, ndl, sh);
            if (colnorm < ACA_EPS) { if (threadIdx.x == 0) lcol[j - 1] = 1; __syncthreads(); }
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
      blknorm = blk_unrm<NT>(pcol, ndl, sh) * blk_unrm<NT>(prow, ndt, sh);
      if (k == 0) {
        apxnorm = znrm;
      } else {
        if (blknorm < apxnorm * eps && rownorm < apxnorm * eps && colnorm < apxnorm * eps && k >= p64) lstop = 1;
      }
    }
    if (lstop == 1 && k >= p64) break;
    k = k + 1;
  }
  if (threadIdx.x == 0) result[blockIdx.x] = status < 0 ? status : k;
}

// dense near-field leaves: a1(it, il) = entry(lod(row il), lod(col it)),
// stored per leaf as a1(ndt, ndl) (HACApK_fill_leafmtx_hyp :2025-2030)
template <int PROB>
__global__ void dense_fill_kernel(DevBemv b, const int* __restrict__ lod, const DenseTask* tasks, int ntasks,
                                  const int64_t* __restrict__ task_start, int64_t total, double* store) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    // binary search of the task holding element e
    int lo = 0, hi = ntasks - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (task_start[mid] <= e) lo = mid; else hi = mid - 1;
    }
    const DenseTask T = tasks[lo];
    int64_t loc = e - task_start[lo];
    int il = (int)(loc / T.ndt), it = (int)(loc % T.ndt);
    int gi = lod[T.nstrtl - 1 + il] - 1, gj = lod[T.nstrtt - 1 + it] - 1;
    store[T.off + loc] = entry<PROB>(b, gi, gj);
  }
}

// batched entries for tests / HACApK_entry_ij
template <int PROB>
__global__ void entries_kernel(DevBemv b, const int* ii, const int* jj, int n, double* out) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) out[e] = entry<PROB>(b, ii[e], jj[e]);
}

// the three launchers of one problem kind
#define HBI_PROBLEM_LAUNCHERS(PROB, NAME)                                                                         \
  void launch_aca_##NAME(const DevBemv& b, const int* lod, const AcaTask* tasks, int ntask, double* arena,        \
                         int* result, const AcaParams& P, cudaStream_t st) {                                      \
    aca_plus_kernel<PROB, HBI_ACA_NT><<<ntask, HBI_ACA_NT, 0, st>>>(b, lod, tasks, arena, result, P);            \
  }                                                                                                               \
  void launch_dense_fill_##NAME(const DevBemv& b, const int* lod, const DenseTask* tasks, int ntask,              \
                                const int64_t* task_start, int64_t total, double* store, int blocks,              \
                                cudaStream_t st) {                                                                \
    dense_fill_kernel<PROB><<<blocks, 256, 0, st>>>(b, lod, tasks, ntask, task_start, total, store);              \
  }                                                                                                               \
  void launch_entries_##NAME(const DevBemv& b, const int* ii, const int* jj, int n, double* out, int blocks,      \
                             cudaStream_t st) {                                                                   \
    entries_kernel<PROB><<<blocks, 128, 0, st>>>(b, ii, jj, n, out);                                              \
  }

#define HBI_DECLARE_PROBLEM_LAUNCHERS(NAME)                                                                      \
  void launch_aca_##NAME(const DevBemv& b, const int* lod, const AcaTask* tasks, int ntask, double* arena,        \
                         int* result, const AcaParams& P, cudaStream_t st);                                       \
  void launch_dense_fill_##NAME(const DevBemv& b, const int* lod, const DenseTask* tasks, int ntask,              \
                                const int64_t* task_start, int64_t total, double* store, int blocks,              \
                                cudaStream_t st);                                                                 \
  void launch_entries_##NAME(const DevBemv& b, const int* ii, const int* jj, int n, double* out, int blocks,      \
                             cudaStream_t st);

}  // namespace hbi
