// hbi_capi.cu -- the extern "C" boundary (include/hbi_gpu.h): HACApK-shaped
// entry points over the GB300 kernels, plus the RK45 driver of the
// rate-and-state system.  Host orchestration only; every product runs in the
// kernels of hbi_aca.cu / hbi_matvec.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/hbi_gpu.h"
#include "hbi_kernels.cuh"
#include "hbi_structure.hpp"

using namespace hbi;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CK(x)                                                                                         \
  do {                                                                                                \
    cudaError_t e_ = (x);                                                                             \
    if (e_ != cudaSuccess) return fail(HBI_ERR_CUDA, "%s: %s (%s:%d)", #x, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

template <class T>
cudaError_t dalloc(T** p, size_t n) {
  return cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T));
}
template <class T>
void dfree(T*& p) {
  if (p) cudaFree((void*)p);
  p = nullptr;
}
template <class T>
cudaError_t upload(T** p, const std::vector<T>& v, cudaStream_t st) {
  cudaError_t e = dalloc(p, v.size());
  if (e != cudaSuccess) return e;
  if (v.empty()) return cudaSuccess;
  e = cudaMemcpyAsync(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(st);
}

// geometry of one st_bemv on the device, with per-element trig tables
struct DevGeom {
  DevBemv b{};
  std::vector<void*> allocs;
  ~DevGeom() {
    for (void* p : allocs) cudaFree(p);
  }
  int put(const double** dst, const double* src, int n, cudaStream_t st) {
    *dst = nullptr;
    if (!src) return 0;
    double* d = nullptr;
    CK(dalloc(&d, n));
    allocs.push_back(d);
    CK(cudaMemcpyAsync(d, src, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    *dst = d;
    return 0;
  }
  int put_vec(const double** dst, const std::vector<double>& v, cudaStream_t st) {
    return put(dst, v.data(), (int)v.size(), st);
  }
  int upload(const hbi_bemv* h, cudaStream_t st) {
    const int n = h->nd;
    b.problem = h->problem;
    b.n = n;
    b.normal = (h->v == 'n');
    b.w = h->w;
    int rc = 0;
    rc |= put(&b.xcol, h->xcol, n, st); rc |= put(&b.ycol, h->ycol, n, st); rc |= put(&b.zcol, h->zcol, n, st);
    rc |= put(&b.xel, h->xel, n, st); rc |= put(&b.xer, h->xer, n, st);
    rc |= put(&b.ang, h->ang, n, st); rc |= put(&b.angd, h->angd, n, st);
    rc |= put(&b.dsl, h->dsl, n, st); rc |= put(&b.dsd, h->dsd, n, st); rc |= put(&b.rake, h->rake, n, st);
    rc |= put(&b.xs1, h->xs1, n, st); rc |= put(&b.xs2, h->xs2, n, st); rc |= put(&b.xs3, h->xs3, n, st);
    rc |= put(&b.ys1, h->ys1, n, st); rc |= put(&b.ys2, h->ys2, n, st); rc |= put(&b.ys3, h->ys3, n, st);
    rc |= put(&b.zs1, h->zs1, n, st); rc |= put(&b.zs2, h->zs2, n, st); rc |= put(&b.zs3, h->zs3, n, st);
    rc |= put(&b.ev11, h->ev11, n, st); rc |= put(&b.ev12, h->ev12, n, st); rc |= put(&b.ev13, h->ev13, n, st);
    rc |= put(&b.ev21, h->ev21, n, st); rc |= put(&b.ev22, h->ev22, n, st); rc |= put(&b.ev23, h->ev23, n, st);
    rc |= put(&b.ev31, h->ev31, n, st); rc |= put(&b.ev32, h->ev32, n, st); rc |= put(&b.ev33, h->ev33, n, st);
    rc |= put(&b.yel, h->yel, n, st); rc |= put(&b.yer, h->yer, n, st);
    // host-evaluated trig of the per-source angles, as okada_ij / okada form them
    if (h->ang) {
      std::vector<double> c(n), s(n), c2(n), s2(n);
      for (int i = 0; i < n; i++) {
        c[i] = std::cos(h->ang[i]); s[i] = std::sin(h->ang[i]);
        c2[i] = std::cos(2 * h->ang[i]); s2[i] = std::sin(2 * h->ang[i]);
      }
      rc |= put_vec(&b.cang, c, st); rc |= put_vec(&b.sang, s, st);
      rc |= put_vec(&b.cang2, c2, st); rc |= put_vec(&b.sang2, s2, st);
    }
    if (h->rake) {
      std::vector<double> c(n), s(n);
      for (int i = 0; i < n; i++) { c[i] = std::cos(h->rake[i]); s[i] = std::sin(h->rake[i]); }
      rc |= put_vec(&b.crake, c, st); rc |= put_vec(&b.srake, s, st);
    }
    if (h->angd) {
      const double pi = 4 * std::atan(1.0), pi2 = 8.0 * std::atan(1.0);
      std::vector<double> cd(n), sd(n), dd(n);
      for (int i = 0; i < n; i++) {
        double dip = h->angd[i] * 180 / pi;
        double p18 = pi2 / 360.0;
        double s_ = std::sin(dip * p18), c_ = std::cos(dip * p18);
        if (std::fabs(c_) < 1e-6) {
          c_ = 0.0;
          if (s_ > 0.0) s_ = 1.0;
          if (s_ < 0.0) s_ = -1.0;
        }
        cd[i] = c_; sd[i] = s_; dd[i] = dip;
      }
      rc |= put_vec(&b.cangd, cd, st); rc |= put_vec(&b.sangd, sd, st); rc |= put_vec(&b.dipdeg, dd, st);
    }
    if (rc) return HBI_ERR_CUDA;
    CK(cudaStreamSynchronize(st));
    return 0;
  }
};

int check_bemv(const hbi_bemv* b) {
  if (!b || b->nd < 1) return fail(HBI_ERR_ARG, "st_bemv: null or nd<1");
  if (b->md != 's' && b->md != 0) return fail(HBI_ERR_ARG, "st_bemv%%md='%c' is not on the hot path (only 's')", b->md);
  if (b->v != 's' && b->v != 'n') return fail(HBI_ERR_ARG, "st_bemv%%v must be 's' or 'n'");
  switch (b->problem) {
    case HBI_2DVS:
      if (!b->xcol || !b->xel || !b->xer) return fail(HBI_ERR_ARG, "2dvs needs xcol, xel, xer");
      break;
    case HBI_3DPH:
    case HBI_3DNR:
      if (!b->xcol || !b->ycol || !b->zcol || !b->ang || !b->angd || !b->dsl || !b->dsd || !b->rake || !(b->w > 0))
        return fail(HBI_ERR_ARG, "okada problems need xcol,ycol,zcol,ang,angd,dsl,dsd,rake and w>0");
      break;
    case HBI_2DPH:
    case HBI_2DN:
      if (!b->xcol || !b->ycol || !b->xel || !b->xer || !b->yel || !b->yer || !b->ang)
        return fail(HBI_ERR_ARG, "2dph / 2dn need xcol, ycol, xel, xer, yel, yer, ang");
      break;
    case HBI_3DNT:
    case HBI_3DHT:
      if (!b->xcol || !b->ycol || !b->zcol || !b->xs1 || !b->xs2 || !b->xs3 || !b->ys1 || !b->ys2 || !b->ys3 ||
          !b->zs1 || !b->zs2 || !b->zs3 || !b->ev11 || !b->ev12 || !b->ev13 || !b->ev21 || !b->ev22 || !b->ev23 ||
          !b->ev31 || !b->ev32 || !b->ev33 || !b->rake)
        return fail(HBI_ERR_ARG, "3dnt / 3dht need collocation points, vertices, ev frames and rake");
      break;
    default:
      return fail(HBI_ERR_ARG, "problem %d is not on the hot path", b->problem);
  }
  return 0;
}

}  // namespace

// ---------------------------------------------------------------- handles
struct hbi_ctl_s {
  int nd = 0;
  double param[100];
  int device = 0, sm_count = 152;
  cudaStream_t stream = nullptr;
  bool have_tree = false;
  Structure S;
  int* d_lod = nullptr;
};

struct hbi_leafmtxp_s {
  hbi_ctl* ctl = nullptr;
  std::vector<Leaf> leaves;     // with kt
  std::vector<int64_t> off;     // reference body offsets (nleaf+1)
  double* d_body = nullptr;     // FP64 body in HACApK's contiguous packing
  int ktmax = 0;
  double t_aca = 0, t_dense = 0;
};

struct hbi_lhp_s {
  hbi_ctl* ctl = nullptr;
  int n = 0, storage = 0;
  StreamPlan plan;                 // host copy (conversion maps released after upload)
  void *d_vstore = nullptr, *d_ustore = nullptr;
  S1ItemDev* d_s1 = nullptr;
  S2ItemDev* d_s2 = nullptr;
  int* d_cnt = nullptr;
  void *d_part = nullptr, *d_z = nullptr, *d_gpart = nullptr;
  int32_t* d_midx = nullptr;
  int32_t *d_grow0 = nullptr, *d_gndl = nullptr, *d_gnch = nullptr, *d_gpoff = nullptr;
  int32_t *d_row_fc = nullptr, *d_fc_ptr = nullptr, *d_fc_group = nullptr;
  int32_t *d_fcb_ptr = nullptr, *d_fcb_base = nullptr;
  int32_t *d_w1off[kNumShapes1] = {}, *d_w1item[kNumShapes1] = {}, *d_w2off[kNumShapes2] = {},
          *d_w2item[kNumShapes2] = {};
  // launch shapes chosen for phases 1 and 2, the median time (us) of every
  // shape per phase as timed at construction, and how the choice was made
  int tune_source = 0;  // 0 timed, 1 cached from an operator of the same plan, 2 forced or pinned
  float tune_us[2][kMaxShapes] = {};
  int* d_err = nullptr;
  int* d_dyn = nullptr;  // dynamic schedules: grab and exit counters of phases 1 and 2
  double *d_x = nullptr, *d_y = nullptr;
  MatDev md{};
  std::vector<Leaf> leaves;
  size_t store_bytes = 0;
  double alg_bytes = 0;
};

extern "C" const char* hbi_last_error(void) { return g_err.c_str(); }
extern "C" int hbi_version(void) { return 10000; }

extern "C" int hbi_set_device(int device) {
  CK(cudaSetDevice(device));
  return HBI_OK;
}

extern "C" int hbi_init(int nd, hbi_ctl** out) {
  if (!out || nd < 1) return fail(HBI_ERR_ARG, "hbi_init: nd<1 or null handle");
  hbi_ctl* c = new hbi_ctl_s();
  c->nd = nd;
  default_params(c->param);
  cudaError_t e = cudaGetDevice(&c->device);
  if (e != cudaSuccess) { delete c; return fail(HBI_ERR_CUDA, "no CUDA device: %s", cudaGetErrorString(e)); }
  cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device);
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete c; return fail(HBI_ERR_CUDA, "stream: %s", cudaGetErrorString(e)); }
  *out = c;
  return HBI_OK;
}

extern "C" int hbi_param_set(hbi_ctl* c, const double* p) {
  if (!c || !p) return fail(HBI_ERR_ARG, "hbi_param_set: null");
  memcpy(c->param, p, sizeof(c->param));
  return HBI_OK;
}
extern "C" int hbi_param_get(const hbi_ctl* c, double* p) {
  if (!c || !p) return fail(HBI_ERR_ARG, "hbi_param_get: null");
  memcpy(p, c->param, sizeof(c->param));
  return HBI_OK;
}

extern "C" int hbi_finalize(hbi_ctl* c) {
  if (!c) return HBI_OK;
  dfree(c->d_lod);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return HBI_OK;
}

extern "C" int hbi_get_lod(const hbi_ctl* c, int* lod) {
  if (!c || !lod) return fail(HBI_ERR_ARG, "hbi_get_lod: null");
  if (!c->have_tree) return fail(HBI_ERR_STATE, "hbi_get_lod before hbi_generate");
  memcpy(lod, c->S.lod.data(), sizeof(int) * c->nd);
  return HBI_OK;
}

extern "C" int hbi_cluster_structure(int nd, const double* coord, const double* param, int* lod, int* nleaf,
                                     int* leaves6) {
  if (nd < 1 || !coord || !nleaf) return fail(HBI_ERR_ARG, "hbi_cluster_structure: bad arguments");
  Structure S;
  if (build_structure(nd, coord, param, S) != 0) return fail(HBI_ERR_ARG, "structure");
  if (lod) memcpy(lod, S.lod.data(), sizeof(int) * nd);
  if (leaves6) {
    if (*nleaf < (int)S.leaves.size()) return fail(HBI_ERR_ARG, "leaves6 too small (%d < %d)", *nleaf, (int)S.leaves.size());
    for (size_t i = 0; i < S.leaves.size(); i++) {
      const Leaf& L = S.leaves[i];
      int* o = leaves6 + 6 * i;
      o[0] = L.ltmtx; o[1] = 0; o[2] = L.nstrtl; o[3] = L.ndl; o[4] = L.nstrtt; o[5] = L.ndt;
    }
  }
  *nleaf = (int)S.leaves.size();
  return HBI_OK;
}

extern "C" int hbi_gen_lattice_vector(const hbi_ctl* c, int* ndc, int* lodc) {
  if (!c || !ndc) return fail(HBI_ERR_ARG, "hbi_gen_lattice_vector: null");
  if (!c->have_tree) return fail(HBI_ERR_STATE, "hbi_gen_lattice_vector before hbi_generate");
  // one lattice block: ndc = nd and lodc = lod (m_HACApK_base.f90:3481-3488)
  *ndc = c->nd;
  if (lodc) memcpy(lodc, c->S.lod.data(), sizeof(int) * c->nd);
  return HBI_OK;
}

// ------------------------------------------------------------ generate
static int run_aca(hbi_ctl* c, const DevGeom& G, std::vector<Leaf>& leaves, std::vector<double*>& chunk_of,
                   std::vector<int64_t>& choff, std::vector<double*>& chunks) {
  cudaStream_t st = c->stream;
  const int kmax = (int)c->param[62];
  AcaParams P;
  P.eps = c->param[70];
  P.pACA_EPS = c->param[71] * P.eps;
  P.znrmmat = (double)(1.0f / (float)c->nd);  // znrm=1.0/nd in default real (m_HACApK_use.f90:200)
  P.kmin = c->param[63];
  P.kmax = kmax;
  struct Pend { int leaf, kcap; };
  std::vector<Pend> todo;
  for (int i = 0; i < (int)leaves.size(); i++)
    if (leaves[i].ltmtx == 1) {
      int kc = std::min(leaves[i].ndl, leaves[i].ndt) + 2;
      kc = std::min(kc, std::min(kmax, 48));
      todo.push_back({i, std::max(kc, 2)});
    }
  const char* env = getenv("HBI_ACA_ARENA_MB");
  int64_t arena_elems = (int64_t)(env ? atoll(env) : 2048) * 1024 * 1024 / 8;
  double* arena = nullptr;
  int64_t arena_cap = 0;
  AcaTask* d_tasks = nullptr;
  int* d_res = nullptr;
  int64_t* d_off = nullptr;
  int rc = HBI_OK;
  while (!todo.empty() && rc == HBI_OK) {
    std::sort(todo.begin(), todo.end(), [&](const Pend& a, const Pend& b) {
      int64_t sa = aca_scratch_elems(leaves[a.leaf].ndl, leaves[a.leaf].ndt, a.kcap);
      int64_t sb = aca_scratch_elems(leaves[b.leaf].ndl, leaves[b.leaf].ndt, b.kcap);
      return sa != sb ? sa > sb : a.leaf < b.leaf;
    });
    std::vector<Pend> retry;
    size_t pos = 0;
    while (pos < todo.size()) {
      std::vector<AcaTask> tasks;
      int64_t used = 0;
      while (pos < todo.size()) {
        const Leaf& L = leaves[todo[pos].leaf];
        int64_t need = aca_scratch_elems(L.ndl, L.ndt, todo[pos].kcap);
        need = (need + 31) / 32 * 32;
        if (!tasks.empty() && used + need > arena_elems) break;
        AcaTask t{L.ndl, L.ndt, L.nstrtl, L.nstrtt, todo[pos].kcap, todo[pos].leaf, used};
        tasks.push_back(t);
        used += need;
        pos++;
        if (tasks.size() >= 65535) break;
      }
      if (used > arena_cap) {
        dfree(arena);
        if (dalloc(&arena, used) != cudaSuccess) { rc = fail(HBI_ERR_NOMEM, "ACA arena of %lld doubles", (long long)used); break; }
        arena_cap = used;
      }
      const int nt = (int)tasks.size();
      dfree(d_tasks); dfree(d_res); dfree(d_off);
      if (upload(&d_tasks, tasks, st) != cudaSuccess || dalloc(&d_res, nt) != cudaSuccess ||
          dalloc(&d_off, nt) != cudaSuccess) { rc = fail(HBI_ERR_CUDA, "ACA task upload"); break; }
      if (cudaMemsetAsync(arena, 0, sizeof(double) * used, st) != cudaSuccess) { rc = fail(HBI_ERR_CUDA, "memset"); break; }
      launch_aca(G.b, c->d_lod, d_tasks, nt, arena, d_res, P, st);
      std::vector<int> res(nt);
      cudaError_t e = cudaMemcpyAsync(res.data(), d_res, sizeof(int) * nt, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) { rc = fail(HBI_ERR_CUDA, "ACA kernel: %s", cudaGetErrorString(e)); break; }
      std::vector<int64_t> off(nt, 0);
      int64_t tot = 0;
      for (int t = 0; t < nt; t++) {
        const AcaTask& T = tasks[t];
        if (res[t] == -2) {
          int kc = std::min(std::min(T.ndl, T.ndt) + 2, std::min(kmax, T.kcap * 4));
          if (kc <= T.kcap) { rc = fail(HBI_ERR_LIMIT, "ACA rank cap reached for leaf %d", T.leaf); break; }
          retry.push_back({T.leaf, kc});
          continue;
        }
        leaves[T.leaf].kt = res[t];
        off[t] = tot;
        tot += (int64_t)res[t] * (T.ndl + T.ndt);
      }
      if (rc != HBI_OK) break;
      double* chunk = nullptr;
      if (dalloc(&chunk, tot) != cudaSuccess) { rc = fail(HBI_ERR_NOMEM, "ACA chunk"); break; }
      chunks.push_back(chunk);
      if (cudaMemcpyAsync(d_off, off.data(), sizeof(int64_t) * nt, cudaMemcpyHostToDevice, st) != cudaSuccess) {
        rc = fail(HBI_ERR_CUDA, "offsets"); break;
      }
      launch_aca_compact(d_tasks, nt, d_res, d_off, arena, chunk, st);
      e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) { rc = fail(HBI_ERR_CUDA, "ACA compact: %s", cudaGetErrorString(e)); break; }
      for (int t = 0; t < nt; t++)
        if (res[t] >= 0) { chunk_of[tasks[t].leaf] = chunk; choff[tasks[t].leaf] = off[t]; }
    }
    todo.swap(retry);
  }
  dfree(arena); dfree(d_tasks); dfree(d_res); dfree(d_off);
  return rc;
}

extern "C" int hbi_generate(hbi_leafmtxp** out, const hbi_bemv* bv, hbi_ctl* c, const double* coord, double ztol) {
  if (!out || !c || !coord) return fail(HBI_ERR_ARG, "hbi_generate: null argument");
  int rc = check_bemv(bv);
  if (rc) return rc;
  if (bv->nd != c->nd) return fail(HBI_ERR_ARG, "st_bemv%%nd=%d differs from hbi_init nd=%d", bv->nd, c->nd);
  c->param[70] = ztol;
  if (c->param[20] < 2) c->param[20] = 3;  // HACApK_chk_st_ctl
  if (build_structure(c->nd, coord, c->param, c->S) != 0) return fail(HBI_ERR_ARG, "structure");
  c->have_tree = true;
  dfree(c->d_lod);
  CK(upload(&c->d_lod, c->S.lod, c->stream));
  DevGeom G;
  rc = G.upload(bv, c->stream);
  if (rc) return rc;

  hbi_leafmtxp* lf = new hbi_leafmtxp_s();
  lf->ctl = c;
  lf->leaves = c->S.leaves;
  const int nl = (int)lf->leaves.size();
  std::vector<double*> chunk_of(nl, nullptr), chunks;
  std::vector<int64_t> choff(nl, 0);
  cudaEvent_t e0, e1, e2;
  cudaEventCreate(&e0); cudaEventCreate(&e1); cudaEventCreate(&e2);
  cudaEventRecord(e0, c->stream);
  rc = run_aca(c, G, lf->leaves, chunk_of, choff, chunks);
  if (rc) {
    for (double* p : chunks) cudaFree(p);
    delete lf;
    return rc;
  }
  cudaEventRecord(e1, c->stream);
  // body offsets in HACApK's contiguous packing
  lf->off.assign(nl + 1, 0);
  int64_t tot = 0;
  for (int i = 0; i < nl; i++) {
    lf->off[i] = tot;
    const Leaf& L = lf->leaves[i];
    tot += L.ltmtx == 1 ? (int64_t)L.kt * (L.ndl + L.ndt) : (int64_t)L.ndl * L.ndt;
    if (L.ltmtx == 1) lf->ktmax = std::max(lf->ktmax, L.kt);
  }
  lf->off[nl] = tot;
  cudaError_t ce = dalloc(&lf->d_body, tot);
  if (ce != cudaSuccess) {
    for (double* p : chunks) cudaFree(p);
    delete lf;
    return fail(HBI_ERR_NOMEM, "H-matrix body of %lld doubles", (long long)tot);
  }
  // gather low-rank factors into place
  {
    std::vector<const double*> src;
    std::vector<int64_t> dof, len;
    for (int i = 0; i < nl; i++) {
      const Leaf& L = lf->leaves[i];
      if (L.ltmtx == 1 && L.kt > 0) {
        src.push_back(chunk_of[i] + choff[i]);
        dof.push_back(lf->off[i]);
        len.push_back((int64_t)L.kt * (L.ndl + L.ndt));
      }
    }
    const double** d_src = nullptr;
    int64_t *d_dof = nullptr, *d_len = nullptr;
    std::vector<const double*> srcv(src.begin(), src.end());
    if (upload(&d_src, srcv, c->stream) != cudaSuccess || upload(&d_dof, dof, c->stream) != cudaSuccess ||
        upload(&d_len, len, c->stream) != cudaSuccess)
      return fail(HBI_ERR_CUDA, "segment upload");
    launch_copy_segments(d_src, d_dof, d_len, (int)src.size(), lf->d_body, c->stream);
    CK(cudaStreamSynchronize(c->stream));
    dfree(d_src); dfree(d_dof); dfree(d_len);
    for (double* p : chunks) cudaFree(p);
  }
  // dense near field
  {
    std::vector<DenseTask> dt;
    std::vector<int64_t> start;
    int64_t acc = 0;
    for (int i = 0; i < nl; i++) {
      const Leaf& L = lf->leaves[i];
      if (L.ltmtx != 2) continue;
      dt.push_back(DenseTask{L.ndl, L.ndt, L.nstrtl, L.nstrtt, lf->off[i]});
      start.push_back(acc);
      acc += (int64_t)L.ndl * L.ndt;
    }
    DenseTask* d_dt = nullptr;
    int64_t* d_start = nullptr;
    CK(upload(&d_dt, dt, c->stream));
    CK(upload(&d_start, start, c->stream));
    launch_dense_fill(G.b, c->d_lod, d_dt, (int)dt.size(), d_start, acc, lf->d_body, c->stream);
    cudaEventRecord(e2, c->stream);
    CK(cudaStreamSynchronize(c->stream));
    dfree(d_dt); dfree(d_start);
  }
  float ms1 = 0, ms2 = 0;
  cudaEventElapsedTime(&ms1, e0, e1);
  cudaEventElapsedTime(&ms2, e1, e2);
  lf->t_aca = ms1 * 1e-3;
  lf->t_dense = ms2 * 1e-3;
  cudaEventDestroy(e0); cudaEventDestroy(e1); cudaEventDestroy(e2);
  *out = lf;
  return HBI_OK;
}

extern "C" int hbi_free_leafmtxp(hbi_leafmtxp* lf) {
  if (!lf) return HBI_OK;
  dfree(lf->d_body);
  delete lf;
  return HBI_OK;
}

extern "C" int hbi_leaf_count(const hbi_leafmtxp* lf, int* nleaf, int* ktmax) {
  if (!lf) return fail(HBI_ERR_ARG, "null");
  if (nleaf) *nleaf = (int)lf->leaves.size();
  if (ktmax) *ktmax = lf->ktmax;
  return HBI_OK;
}

extern "C" int hbi_get_leaves(const hbi_leafmtxp* lf, int* o) {
  if (!lf || !o) return fail(HBI_ERR_ARG, "null");
  for (size_t i = 0; i < lf->leaves.size(); i++) {
    const Leaf& L = lf->leaves[i];
    o[6 * i + 0] = L.ltmtx; o[6 * i + 1] = L.kt; o[6 * i + 2] = L.nstrtl;
    o[6 * i + 3] = L.ndl; o[6 * i + 4] = L.nstrtt; o[6 * i + 5] = L.ndt;
  }
  return HBI_OK;
}

extern "C" int hbi_get_body(const hbi_leafmtxp* lf, int64_t* offsets, double* body) {
  if (!lf || !offsets) return fail(HBI_ERR_ARG, "null");
  memcpy(offsets, lf->off.data(), sizeof(int64_t) * lf->off.size());
  if (body) CK(cudaMemcpy(body, lf->d_body, sizeof(double) * lf->off.back(), cudaMemcpyDeviceToHost));
  return HBI_OK;
}

extern "C" int hbi_entry_ij(const hbi_bemv* bv, int n, const int* i, const int* j, double* out) {
  int rc = check_bemv(bv);
  if (rc) return rc;
  if (n < 0 || (n > 0 && (!i || !j || !out))) return fail(HBI_ERR_ARG, "hbi_entry_ij: null arrays");
  if (n == 0) return HBI_OK;
  cudaStream_t st;
  CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  DevGeom G;
  rc = G.upload(bv, st);
  if (rc) { cudaStreamDestroy(st); return rc; }
  std::vector<int> ii(n), jj(n);
  for (int k = 0; k < n; k++) {
    if (i[k] < 1 || i[k] > bv->nd || j[k] < 1 || j[k] > bv->nd) { cudaStreamDestroy(st); return fail(HBI_ERR_ARG, "index out of range"); }
    ii[k] = i[k] - 1; jj[k] = j[k] - 1;
  }
  int *di = nullptr, *dj = nullptr;
  double* dout = nullptr;
  CK(upload(&di, ii, st));
  CK(upload(&dj, jj, st));
  CK(dalloc(&dout, n));
  launch_entries(G.b, di, dj, n, dout, st);
  CK(cudaMemcpyAsync(out, dout, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  dfree(di); dfree(dj); dfree(dout);
  cudaStreamDestroy(st);
  return HBI_OK;
}

static int device_error_status(const MatDev& m, const char* where);

// ----------------------------------------------------- shape autotuner
// Replaces the reference's byte-balanced cut of the leaf list over OpenMP
// threads (m_HACApK_use.f90:387-431, m_HACApK_base.f90:1537-1564): the work
// of a phase is dealt to warps by plan_warp_schedule, and the launch shape
// (warps per block, stages, stage bytes -- which sets the chunk width) is
// chosen per operator and phase by timing every compiled shape on the
// operator itself.  The choice is cached for operators whose plans have the
// same size statistics.

// median of the positive, finite entries of t[0..n); -1 if there is none
static float median_valid(const float* t, int n) {
  std::vector<float> v;
  for (int i = 0; i < n; i++)
    if (t[i] > 0 && std::isfinite(t[i])) v.push_back(t[i]);
  if (v.empty()) return -1.0f;
  std::sort(v.begin(), v.end());
  const size_t m = v.size();
  return m % 2 ? v[m / 2] : 0.5f * (v[m / 2 - 1] + v[m / 2]);
}

extern "C" int hbi_autotune_select(int ncand, int reps, const float* times, float* medians, int* best) {
  if (ncand < 1 || reps < 1 || !times || !best) return fail(HBI_ERR_ARG, "hbi_autotune_select: bad arguments");
  int b = -1;
  float bt = 0.0f;
  for (int c = 0; c < ncand; c++) {
    const float m = median_valid(times + (size_t)c * reps, reps);
    if (medians) medians[c] = m;
    if (m < 0) continue;
    // a later candidate must beat the current best by more than 1%: ties and
    // near-ties keep the earlier (default-first) shape
    if (b < 0 || m < 0.99f * bt) {
      b = c;
      bt = m;
    }
  }
  if (b < 0) return fail(HBI_ERR_ARG, "hbi_autotune_select: no candidate has a valid time");
  *best = b;
  return HBI_OK;
}

namespace {
struct TuneKey {
  int storage, sm;
  int64_t ns1, ns2, vstore, ustore;
  bool operator<(const TuneKey& o) const {
    return std::tie(storage, sm, ns1, ns2, vstore, ustore) < std::tie(o.storage, o.sm, o.ns1, o.ns2, o.vstore, o.ustore);
  }
};
std::mutex g_tune_mu;
std::map<TuneKey, std::pair<int, int>> g_tune_cache;
}  // namespace

static int autotune_stream_shapes(hbi_lhp* h) {
  MatDev& m = h->md;
  for (int ph = 0; ph < 2; ph++)
    for (int sh = 0; sh < kMaxShapes; sh++) h->tune_us[ph][sh] = -1.0f;
  const int f1 = forced_stream_shape(1), f2 = forced_stream_shape(2);
  if (f1 >= 0 && f2 >= 0) {
    m.shape1 = f1;
    m.shape2 = f2;
    h->tune_source = 2;
    return HBI_OK;
  }
  const TuneKey key{h->storage, h->ctl->sm_count, (int64_t)h->plan.p1.size(), (int64_t)h->plan.p2.size(),
                    h->plan.vstore, h->plan.ustore};
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      m.shape1 = f1 >= 0 ? f1 : it->second.first;
      m.shape2 = f2 >= 0 ? f2 : it->second.second;
      h->tune_source = 1;
      return HBI_OK;
    }
  }
  cudaStream_t st = h->ctl->stream;
  constexpr int R = 5;
  float t[2][kMaxShapes * R];
  cudaEvent_t ev[2 * R];
  for (auto& e : ev)
    if (cudaEventCreate(&e) != cudaSuccess) return fail(HBI_ERR_CUDA, "autotune: events");
  CK(cudaMemsetAsync(h->d_x, 0, sizeof(double) * h->n, st));
  int rc = HBI_OK;
  for (int ph = 1; ph <= 2 && rc == HBI_OK; ph++)
    for (int sh = 0; sh < num_shapes(ph); sh++) {
      launch_phase_shape(ph, sh, &m, 1, h->d_x, h->ctl->sm_count, st);  // warm-up
      for (int r = 0; r < R; r++) {
        cudaEventRecord(ev[2 * r], st);
        launch_phase_shape(ph, sh, &m, 1, h->d_x, h->ctl->sm_count, st);
        cudaEventRecord(ev[2 * r + 1], st);
      }
      const cudaError_t e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) {
        rc = fail(HBI_ERR_CUDA, "autotune: %s", cudaGetErrorString(e));
        break;
      }
      for (int r = 0; r < R; r++) {
        float ms = -1.0f;
        if (cudaEventElapsedTime(&ms, ev[2 * r], ev[2 * r + 1]) != cudaSuccess) ms = -1.0f;
        t[ph - 1][sh * R + r] = ms * 1e3f;
      }
    }
  for (auto& e : ev) cudaEventDestroy(e);
  if (rc) return rc;
  rc = device_error_status(m, "hbi_construct_lh (shape autotuner)");
  if (rc) return rc;
  int best[2] = {0, 0};
  for (int ph = 0; ph < 2; ph++) {
    rc = hbi_autotune_select(num_shapes(ph + 1), R, t[ph], h->tune_us[ph], &best[ph]);
    if (rc) return rc;
  }
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune_cache[key] = {best[0], best[1]};
  }
  m.shape1 = f1 >= 0 ? f1 : best[0];
  m.shape2 = f2 >= 0 ? f2 : best[1];
  h->tune_source = (f1 >= 0 || f2 >= 0) ? 2 : 0;
  return HBI_OK;
}

extern "C" int hbi_lh_tuning(const hbi_lhp* h, int* shape1, int* shape2, float* median_us, int* source) {
  if (!h) return fail(HBI_ERR_ARG, "hbi_lh_tuning: null");
  if (shape1) *shape1 = h->md.shape1;
  if (shape2) *shape2 = h->md.shape2;
  if (median_us) {
    int o = 0;
    for (int ph = 0; ph < 2; ph++)
      for (int sh = 0; sh < num_shapes(ph + 1); sh++) median_us[o++] = h->tune_us[ph][sh];
  }
  if (source) *source = h->tune_source;
  return HBI_OK;
}

extern "C" int hbi_lh_set_shapes(hbi_lhp* h, int shape1, int shape2) {
  if (!h || shape1 < 0 || shape1 >= kNumShapes1 || shape2 < 0 || shape2 >= kNumShapes2)
    return fail(HBI_ERR_ARG, "hbi_lh_set_shapes: shapes must be in 0..%d (phase 1) and 0..%d (phase 2)",
                kNumShapes1 - 1, kNumShapes2 - 1);
  h->md.shape1 = shape1;
  h->md.shape2 = shape2;
  h->tune_source = 2;
  return HBI_OK;
}

extern "C" int hbi_stream_shapes(int phase, int* count, int* shapes5) {
  if (!count || (phase != 1 && phase != 2)) return fail(HBI_ERR_ARG, "hbi_stream_shapes: bad arguments");
  *count = num_shapes(phase);
  if (shapes5)
    for (int sh = 0; sh < num_shapes(phase); sh++) {
      const StreamShape& S = stream_shape(phase, sh);
      shapes5[5 * sh] = S.nw;
      shapes5[5 * sh + 1] = S.ns;
      shapes5[5 * sh + 2] = S.sb;
      shapes5[5 * sh + 3] = S.map;
      shapes5[5 * sh + 4] = S.sched;
    }
  return HBI_OK;
}

extern "C" int hbi_plan_block_schedule(int n, const int64_t* cost, const int64_t* key, int nblocks, int nw,
                                       int32_t* woff, int32_t* witem) {
  if (n < 0 || nblocks < 1 || nw < 1 || (n > 0 && (!cost || !key || !witem)) || !woff)
    return fail(HBI_ERR_ARG, "hbi_plan_block_schedule: bad arguments");
  std::vector<int64_t> c(cost, cost + n), k(key, key + n);
  std::vector<int32_t> o, it;
  plan_block_schedule(c, k, nblocks, nw, o, it);
  std::copy(o.begin(), o.end(), woff);
  std::copy(it.begin(), it.end(), witem);
  return HBI_OK;
}

// ---------------------------------------------------------- construct
// ------------------------------------------------- leaf partition (host)
// factor elements of a leaf: kt (ndl + ndt) low rank, ndl ndt dense
static int64_t leaf_elems(const int* q) {
  return q[0] == 1 ? (int64_t)q[1] * (q[3] + q[5]) : (int64_t)q[3] * q[5];
}

extern "C" int hbi_partition_leaves(int nleaf, const int* leaves6, int nranks, int32_t* owner,
                                    int64_t* elems_per_rank) {
  if (nleaf < 0 || (nleaf > 0 && (!leaves6 || !owner)) || nranks < 1)
    return fail(HBI_ERR_ARG, "hbi_partition_leaves: bad arguments");
  // longest first to the least-loaded rank (ties to the lower rank), as the
  // warp schedules deal items; leaves of equal size keep their order
  std::vector<int> order(nleaf);
  for (int i = 0; i < nleaf; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return leaf_elems(leaves6 + 6 * a) > leaf_elems(leaves6 + 6 * b); });
  std::vector<int64_t> load(nranks, 0);
  for (int i : order) {
    int r = 0;
    for (int q = 1; q < nranks; q++)
      if (load[q] < load[r]) r = q;
    owner[i] = r;
    load[r] += leaf_elems(leaves6 + 6 * i);
  }
  if (elems_per_rank)
    for (int q = 0; q < nranks; q++) elems_per_rank[q] = load[q];
  return HBI_OK;
}

static int construct_impl(hbi_lhp** out, const hbi_leafmtxp* lf, hbi_ctl* c, int storage, const int32_t* owner,
                          int rank);

extern "C" int hbi_construct_lh(hbi_lhp** out, const hbi_leafmtxp* lf, hbi_ctl* c, int storage) {
  return construct_impl(out, lf, c, storage, nullptr, 0);
}

extern "C" int hbi_construct_lh_part(hbi_lhp** out, const hbi_leafmtxp* lf, hbi_ctl* c, int storage,
                                     const int32_t* owner, int rank) {
  if (!owner || rank < 0) return fail(HBI_ERR_ARG, "hbi_construct_lh_part: owner table and rank needed");
  return construct_impl(out, lf, c, storage, owner, rank);
}

static int construct_impl(hbi_lhp** out, const hbi_leafmtxp* lf, hbi_ctl* c, int storage, const int32_t* owner,
                          int rank) {
  if (!out || !lf || !c) return fail(HBI_ERR_ARG, "hbi_construct_lh: null");
  if (storage < 0 || storage > 2) return fail(HBI_ERR_ARG, "storage must be HBI_STORE_F64/F32/BF16");
  if (lf->ctl != c || !c->have_tree) return fail(HBI_ERR_STATE, "construct_LH needs the ctl used by generate");
  hbi_lhp* h = new hbi_lhp_s();
  h->ctl = c;
  h->n = c->nd;
  h->storage = storage;
  // the operator's leaves (all, or those of one rank) and their body offsets
  std::vector<int64_t> boff;
  for (size_t i = 0; i < lf->leaves.size(); i++)
    if (!owner || owner[i] == rank) {
      h->leaves.push_back(lf->leaves[i]);
      boff.push_back(lf->off[i]);
    }
  const int esz = storage == ST_F64 ? 8 : storage == ST_F32 ? 4 : 2;
  const size_t acc = storage == ST_F64 ? 8 : 4;
  cudaStream_t st = c->stream;
  // row-tiled stores read by bulk copies (plan_stream)
  StreamPlan& P = h->plan;
  plan_stream(c->nd, h->leaves, boff, 16 / esz, P, 8192);
  const size_t vbytes = (size_t)P.vstore * esz, ubytes = (size_t)P.ustore * esz;
  h->store_bytes = vbytes + ubytes;
  CK(cudaMalloc(&h->d_vstore, std::max<size_t>(vbytes, 16)));
  CK(cudaMalloc(&h->d_ustore, std::max<size_t>(ubytes, 16)));
  CK(cudaMemsetAsync(h->d_vstore, 0, std::max<size_t>(vbytes, 16), st));
  CK(cudaMemsetAsync(h->d_ustore, 0, std::max<size_t>(ubytes, 16), st));
  for (int which = 0; which < 2; which++) {
    std::vector<SegCopy>& map = which == 0 ? P.vcopy : P.ucopy;
    SegCopyDev* d_map = nullptr;
    CK(upload(&d_map, map, st));
    launch_segcopy(lf->d_body, d_map, (int64_t)map.size(), which == 0 ? h->d_vstore : h->d_ustore, storage, st);
    CK(cudaStreamSynchronize(st));
    dfree(d_map);
    std::vector<SegCopy>().swap(map);
  }
  CK(cudaGetLastError());
  const GroupPlan& G = P.gp;
  CK(upload(&h->d_s1, P.p1, st));
  CK(upload(&h->d_s2, P.p2, st));
  CK(upload(&h->d_midx, P.midx, st));
  CK(upload(&h->d_grow0, G.grow0, st));
  CK(upload(&h->d_gndl, G.gndl, st));
  CK(upload(&h->d_gnch, P.gnch, st));
  CK(upload(&h->d_gpoff, P.gpoff2, st));
  CK(upload(&h->d_row_fc, G.row_fc, st));
  CK(upload(&h->d_fc_ptr, G.fc_ptr, st));
  CK(upload(&h->d_fc_group, G.fc_group, st));
  CK(upload(&h->d_fcb_ptr, P.fcb_ptr, st));
  CK(upload(&h->d_fcb_base, P.fcb_base, st));
  CK(dalloc(&h->d_cnt, (size_t)P.ncg));
  CK(cudaMemset(h->d_cnt, 0, sizeof(int) * std::max<int64_t>(P.ncg, 1)));
  CK(dalloc(&h->d_err, 1));
  CK(cudaMemset(h->d_err, 0, sizeof(int)));
  CK(dalloc(&h->d_dyn, 4));
  CK(cudaMemset(h->d_dyn, 0, sizeof(int) * 4));
  CK(cudaMalloc(&h->d_part, std::max<size_t>(P.plen1, 1) * acc));
  CK(cudaMalloc(&h->d_z, std::max<size_t>(P.zlen, 1) * acc));
  CK(cudaMemset(h->d_z, 0, std::max<size_t>(P.zlen, 1) * acc));
  CK(cudaMalloc(&h->d_gpart, std::max<size_t>(P.plen2, 1) * acc));
  CK(dalloc(&h->d_x, h->n));
  CK(dalloc(&h->d_y, h->n));
  MatDev& m = h->md;
  m.n = c->nd;
  m.storage = storage;
  m.vstore = h->d_vstore;
  m.ustore = h->d_ustore;
  m.s1 = h->d_s1;
  m.ns1 = (int)P.p1.size();
  m.s2 = h->d_s2;
  m.ns2 = (int)P.p2.size();
  m.cnt = h->d_cnt;
  m.part = h->d_part;
  m.z = h->d_z;
  m.midx = h->d_midx;
  m.gpart = h->d_gpart;
  m.grow0 = h->d_grow0; m.gndl = h->d_gndl; m.gnch = h->d_gnch; m.gpoff = h->d_gpoff;
  m.row_fc = h->d_row_fc; m.fc_ptr = h->d_fc_ptr; m.fc_group = h->d_fc_group;
  m.fcb_ptr = h->d_fcb_ptr; m.fcb_base = h->d_fcb_base;
  m.scale = 1.0;
  m.skip = nullptr;
  m.err = h->d_err;
  m.dyn = h->d_dyn;
  m.wait = kWaitCyclesDefault;
  m.ncnt = (int)P.ncg;
  // static warp schedules, one per launch shape, for the grid the phase
  // kernels get on this device in that shape: one block of nw warps per SM,
  // fewer for small operators
  for (int ph = 1; ph <= 2; ph++)
    for (int sh = 0; sh < num_shapes(ph); sh++) {
      const StreamShape& S = stream_shape(ph, sh);
      const int nw = S.nw, sb = S.sb;
      const int ni = ph == 1 ? (int)P.p1.size() : (int)P.p2.size();
      if (ni == 0) continue;
      const int need = (ni + nw - 1) / nw;
      const int nblk = need < c->sm_count ? need : c->sm_count;
      // schedule units: warps, or blocks for the block-shared schedule
      const int gw = S.sched == 3 ? nblk : nblk * nw;
      std::vector<int64_t> cost(ni), key(ni);
      for (int i = 0; i < ni; i++) {
        const int ncols = ph == 1 ? P.p1[i].ncols : P.p2[i].ncols, ntp = ph == 1 ? P.p1[i].ntp : P.p2[i].ntp;
        const int cc = chunk_cols(ntp, esz, sb);
        // bytes streamed plus ~1 KB worth of fixed cost per chunk
        cost[i] = (int64_t)ncols * ntp * esz + 1024 * (int64_t)((ncols + cc - 1) / cc);
        key[i] = ph == 1 ? P.p1[i].soff : P.p2[i].soff;
      }
      if (S.sched == 2) continue;  // dynamic: the warps take the items in order from a counter
      std::vector<int32_t> woff, witem;
      if (S.sched == 1) plan_block_schedule(cost, key, nblk, nw, woff, witem);
      else plan_warp_schedule(cost, gw, woff, witem);
      if (ph == 1) {
        CK(upload(&h->d_w1off[sh], woff, st));
        CK(upload(&h->d_w1item[sh], witem, st));
        m.gw1[sh] = gw;
        m.w1off[sh] = h->d_w1off[sh];
        m.w1item[sh] = h->d_w1item[sh];
      } else {
        CK(upload(&h->d_w2off[sh], woff, st));
        CK(upload(&h->d_w2item[sh], witem, st));
        m.gw2[sh] = gw;
        m.w2off[sh] = h->d_w2off[sh];
        m.w2item[sh] = h->d_w2item[sh];
      }
    }
  m.shape1 = m.shape2 = 0;
  h->alg_bytes = (double)P.factor_elems * esz + (double)h->n * 8 * 2;
  prepare_stream_kernels();
  CK(cudaGetLastError());
  int rc = autotune_stream_shapes(h);
  if (rc) {
    hbi_free_lh(h);
    return rc;
  }
  *out = h;
  return HBI_OK;
}

extern "C" int hbi_free_lh(hbi_lhp* h) {
  if (!h) return HBI_OK;
  // RK handles, time loops and ensembles read the stores on streams of their
  // own: let all device work end before the memory goes
  cudaDeviceSynchronize();
  for (void* p : {h->d_vstore, h->d_ustore, (void*)h->d_s1, (void*)h->d_s2, (void*)h->d_cnt, h->d_part, h->d_z,
                  h->d_gpart, (void*)h->d_midx, (void*)h->d_grow0, (void*)h->d_gndl, (void*)h->d_gnch,
                  (void*)h->d_gpoff, (void*)h->d_row_fc, (void*)h->d_fc_ptr, (void*)h->d_fc_group, (void*)h->d_err,
                  (void*)h->d_dyn,
                  (void*)h->d_fcb_ptr, (void*)h->d_fcb_base,
                  (void*)h->d_x, (void*)h->d_y})
    if (p) cudaFree(p);
  for (int sh = 0; sh < kNumShapes1; sh++)
    for (void* p : {(void*)h->d_w1off[sh], (void*)h->d_w1item[sh]})
      if (p) cudaFree(p);
  for (int sh = 0; sh < kNumShapes2; sh++)
    for (void* p : {(void*)h->d_w2off[sh], (void*)h->d_w2item[sh]})
      if (p) cudaFree(p);
  delete h;
  return HBI_OK;
}

namespace hbi {
int take_device_error(const MatDev& m) {
  if (!m.err) return 0;
  int flag = 0;
  if (cudaMemcpy(&flag, m.err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return HBI_ERR_CUDA;
  if (!flag) return 0;
  // a warp that gave up left before its arrivals: the counters start over
  if (cudaMemset(m.err, 0, sizeof(int)) != cudaSuccess ||
      (m.cnt && m.ncnt > 0 && cudaMemset(m.cnt, 0, sizeof(int) * (size_t)m.ncnt) != cudaSuccess) ||
      (m.dyn && cudaMemset(m.dyn, 0, sizeof(int) * 4) != cudaSuccess))
    return HBI_ERR_CUDA;
  return 1;
}
}  // namespace hbi

static int device_error_status(const MatDev& m, const char* where) {
  const int t = take_device_error(m);
  if (t < 0) return fail(HBI_ERR_CUDA, "%s: reading the device error word failed", where);
  if (t > 0)
    return fail(HBI_ERR_DEVICE, "%s: a product kernel gave up waiting for a bulk copy; the result is invalid "
                "(the operator's device state has been reset)", where);
  return HBI_OK;
}

extern "C" int hbi_lh_check_error(hbi_lhp* h) {
  if (!h) return fail(HBI_ERR_ARG, "hbi_lh_check_error: null");
  return device_error_status(h->md, "hbi_lh_check_error");
}

extern "C" int hbi_lh_set_wait_limit(hbi_lhp* h, long long cycles) {
  if (!h) return fail(HBI_ERR_ARG, "hbi_lh_set_wait_limit: null");
  h->md.wait = cycles < 0 ? kWaitCyclesDefault : cycles;
  return HBI_OK;
}

extern "C" int hbi_lh_info(const hbi_lhp* h, int64_t* fe, int64_t* sb, double* ab) {
  if (!h) return fail(HBI_ERR_ARG, "null");
  if (fe) *fe = h->plan.factor_elems;
  if (sb) *sb = (int64_t)h->store_bytes;
  if (ab) *ab = h->alg_bytes;
  return HBI_OK;
}

extern "C" int hbi_adot_lattice_hyp_phase_dev(double* d_au, hbi_lhp* h, const double* d_u, void* stream, int phase) {
  if (!h || !d_u || ((phase == 0 || phase == 3) && !d_au) || phase < 0 || phase > 3)
    return fail(HBI_ERR_ARG, "hbi_adot_lattice_hyp_phase_dev: bad arguments");
  cudaStream_t st = stream ? (cudaStream_t)stream : h->ctl->stream;
  if (phase == 0 || phase == 1) launch_phase1(&h->md, 1, d_u, h->ctl->sm_count, st);
  if (phase == 0 || phase == 2) launch_phase2(&h->md, 1, d_u, h->ctl->sm_count, st);
  if (phase == 0 || phase == 3) {
    double* ys[2] = {d_au, nullptr};
    launch_phase3_plain(&h->md, 1, ys, st);
  }
  CK(cudaGetLastError());
  return HBI_OK;
}

extern "C" int hbi_adot_lattice_hyp_dev(double* d_au, hbi_lhp* h, const double* d_u, void* stream) {
  return hbi_adot_lattice_hyp_phase_dev(d_au, h, d_u, stream, 0);
}

// ----------------------------------------------------- allocation-free product
// The scratch of hbi_adot_lattice_hyp_noalloc: one array in the library's
// device image.  Host code may not use g_noalloc_scratch as an address (on the
// host it names a shadow variable); its device address comes from
// cudaGetSymbolAddress, once per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[HBI_NOALLOC_SCRATCH_BYTES];
static std::mutex g_noalloc_mu;
static void* g_noalloc_addr[128];

static size_t align256(size_t b) { return (b + 255) / 256 * 256; }

extern "C" int hbi_adot_lattice_hyp_noalloc(double* d_au, hbi_lhp* h, const double* d_u, void* stream) {
  if (!h || !d_au || !d_u) return fail(HBI_ERR_ARG, "hbi_adot_lattice_hyp_noalloc: null argument");
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 128) return fail(HBI_ERR_LIMIT, "hbi_adot_lattice_hyp_noalloc: device %d out of range", dev);
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) CK(cudaGetSymbolAddress(&g_noalloc_addr[dev], g_noalloc_scratch));
    base = g_noalloc_addr[dev];
  }
  // layout: [arrival counters][z][phase-1 partials][row-group partials]
  const size_t acc = h->storage == ST_F64 ? 8 : 4;
  const size_t nlr = (size_t)h->plan.ncg;
  const size_t b_cnt = align256(std::max<size_t>(nlr, 1) * sizeof(int));
  const size_t b_z = align256(std::max<int64_t>(h->plan.zlen, 1) * acc);
  const size_t b_part = align256(std::max<int64_t>(h->plan.plen1, 1) * acc);
  const size_t b_gp = align256(std::max<int64_t>(h->plan.plen2, 1) * acc);
  const size_t need = b_cnt + b_z + b_part + b_gp;
  if (need > HBI_NOALLOC_SCRATCH_BYTES)
    return fail(HBI_ERR_LIMIT, "hbi_adot_lattice_hyp_noalloc: operator needs %zu bytes of scratch, the limit is %u",
                need, (unsigned)HBI_NOALLOC_SCRATCH_BYTES);
  unsigned char* p = (unsigned char*)base;
  MatDev md = h->md;
  md.cnt = (int*)p;
  md.z = p + b_cnt;
  md.part = p + b_cnt + b_z;
  md.gpart = p + b_cnt + b_z + b_part;
  md.ncnt = (int)nlr;
  cudaStream_t st = stream ? (cudaStream_t)stream : h->ctl->stream;
  // the counters must start at zero; everything else is written before it is read
  CK(cudaMemsetAsync(md.cnt, 0, nlr * sizeof(int), st));
  double* ys[2] = {d_au, nullptr};
  launch_phase1(&md, 1, d_u, h->ctl->sm_count, st);
  launch_phase2(&md, 1, d_u, h->ctl->sm_count, st);
  launch_phase3_plain(&md, 1, ys, st);
  CK(cudaGetLastError());
  return HBI_OK;
}

extern "C" int hbi_lh_phase_bytes(const hbi_lhp* h, double* p1, double* p2) {
  if (!h) return fail(HBI_ERR_ARG, "null");
  const int esz = h->storage == ST_F64 ? 8 : h->storage == ST_F32 ? 4 : 2;
  double v = 0, rest = 0;
  for (const Leaf& L : h->leaves) {
    if (L.ltmtx == 1) { v += (double)L.kt * L.ndt; rest += (double)L.kt * L.ndl; }
    else rest += (double)L.ndl * L.ndt;
  }
  // phase 1 reads V and x; phase 2 reads U, the dense blocks and (gathered)
  // x; phase 3 writes y (n x 8 bytes, in neither figure)
  if (p1) *p1 = v * esz + (double)h->n * 8;
  if (p2) *p2 = rest * esz + (double)h->n * 8;
  return HBI_OK;
}

extern "C" int hbi_adot_lattice_hyp(double* au, hbi_lhp* h, hbi_ctl* c, double* wws, const double* u) {
  (void)wws;
  if (!h || !au || !u) return fail(HBI_ERR_ARG, "hbi_adot_lattice_hyp: null");
  if (c && c != h->ctl) return fail(HBI_ERR_ARG, "st_ctl does not own st_LHp");
  cudaStream_t st = h->ctl->stream;
  CK(cudaMemcpyAsync(h->d_x, u, sizeof(double) * h->n, cudaMemcpyHostToDevice, st));
  int rc = hbi_adot_lattice_hyp_dev(h->d_y, h, h->d_x, st);
  if (rc) return rc;
  CK(cudaMemcpyAsync(au, h->d_y, sizeof(double) * h->n, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return device_error_status(h->md, "hbi_adot_lattice_hyp");
}

// ---------------------------------------------------------------- RK45
struct hbi_rk_s {
  hbi_lhp* ls = nullptr;
  hbi_lhp* ln = nullptr;
  int n = 0, nmat = 1;
  RkDev R{};
  MatDev mats[2];
  std::vector<double*> allocs;
  double* h_ctl = nullptr;  // pinned: h, eps, emax, huge index
  static constexpr int kSlots = 64;
  double* h_ring = nullptr;  // pinned (h, eps) slots
  cudaEvent_t slot_ev[kSlots] = {};
  int slot_used[kSlots] = {};
  int slot = 0;
  cudaStream_t st = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int launches = 0;
};

static void cash_karp(double* B, double* C, double* DC) {
  // the reference's PARAMETER statements (main_LH.f90:2490-2496) evaluate
  // 3./40., .3, 37./378. ... in default real, then widen to real(8)
  B[0] = .2;
  B[1] = (double)(3.f / 40.f); B[2] = (double)(9.f / 40.f);
  B[3] = (double).3f; B[4] = (double)-.9f; B[5] = (double)1.2f;
  B[6] = (double)(-(11.f / 54.f)); B[7] = 2.5; B[8] = (double)(-(70.f / 27.f)); B[9] = (double)(35.f / 27.f);
  B[10] = (double)(1631.f / 55296.f); B[11] = (double)(175.f / 512.f); B[12] = (double)(575.f / 13824.f);
  B[13] = (double)(44275.f / 110592.f); B[14] = (double)(253.f / 4096.f);
  const double C1 = (double)(37.f / 378.f), C3 = (double)(250.f / 621.f), C4 = (double)(125.f / 594.f),
               C6 = (double)(512.f / 1771.f);
  C[0] = C1; C[1] = 0; C[2] = C3; C[3] = C4; C[4] = 0; C[5] = C6;
  DC[0] = C1 - (double)(2825.f / 27648.f); DC[1] = 0;
  DC[2] = C3 - (double)(18575.f / 48384.f);
  DC[3] = C4 - (double)(13525.f / 55296.f);
  DC[4] = (double)(-(277.f / 14336.f));
  DC[5] = C6 - (double).25f;
}

extern "C" int hbi_rk_create(hbi_rk** out, const hbi_rsf_params* p, hbi_lhp* ls, hbi_lhp* ln) {
  if (!out || !p || !ls) return fail(HBI_ERR_ARG, "hbi_rk_create: null");
  if (p->ncell != ls->n) return fail(HBI_ERR_ARG, "ncell %d != operator size %d", p->ncell, ls->n);
  if (!p->a || !p->b || !p->dc || !p->f0 || !p->taudot || !p->sigdot || !p->vpl)
    return fail(HBI_ERR_ARG, "rsf parameter arrays must be non-null");
  if (ln) {
    if (ln->n != ls->n || ln->storage != ls->storage) return fail(HBI_ERR_ARG, "H_s and H_n differ in size or storage");
    if (ln->leaves.size() != ls->leaves.size()) return fail(HBI_ERR_ARG, "H_s and H_n have different leaf lists");
    for (size_t i = 0; i < ls->leaves.size(); i++) {
      const Leaf &a = ls->leaves[i], &b = ln->leaves[i];
      if (a.ltmtx != b.ltmtx || a.nstrtl != b.nstrtl || a.ndl != b.ndl || a.nstrtt != b.nstrtt || a.ndt != b.ndt)
        return fail(HBI_ERR_ARG, "H_s and H_n have different leaf lists");
    }
  }
  hbi_rk* r = new hbi_rk_s();
  r->ls = ls; r->ln = ln; r->n = p->ncell; r->nmat = ln ? 2 : 1;
  // the RK handle issues all its work on a stream of its own, so its
  // lifetime does not depend on the control blocks of the operators
  if (cudaStreamCreateWithFlags(&r->st, cudaStreamNonBlocking) != cudaSuccess) {
    delete r;
    return fail(HBI_ERR_CUDA, "RK stream");
  }
  const int n = r->n;
  auto mk = [&](double** d, size_t cnt) -> int {
    if (dalloc(d, cnt) != cudaSuccess) return 1;
    r->allocs.push_back(*d);
    return 0;
  };
  auto cp = [&](const double** d, const double* h) -> int {
    double* t;
    if (mk(&t, n)) return 1;
    if (cudaMemcpy(t, h, sizeof(double) * n, cudaMemcpyHostToDevice) != cudaSuccess) return 1;
    *d = t;
    return 0;
  };
  RkDev& R = r->R;
  R.n = n; R.nmat = r->nmat; R.evlaw = p->evlaw; R.backslip = p->backslip; R.limitsigma = p->limitsigma;
  R.vref = p->vref; R.minsig = p->minsig; R.maxsig = p->maxsig;
  R.rigid_over_2vs = 0.5 * 32.04 / 3.464;
  int bad = 0;
  bad |= cp(&R.a, p->a); bad |= cp(&R.b, p->b); bad |= cp(&R.dc, p->dc); bad |= cp(&R.f0, p->f0);
  bad |= cp(&R.taudot, p->taudot); bad |= cp(&R.sigdot, p->sigdot); bad |= cp(&R.vpl, p->vpl);
  bad |= mk(&R.y, 3 * n); bad |= mk(&R.ys, 3 * n); bad |= mk(&R.vs, n); bad |= mk(&R.ws, n); bad |= mk(&R.x0, n);
  bad |= mk(&R.xb[0], n); bad |= mk(&R.xb[1], n); bad |= mk(&R.K, 18 * (size_t)n);
  bad |= mk(&R.yout, 3 * n); bad |= mk(&R.yerr, 3 * n); bad |= mk(&R.ebuf, 3 * n); bad |= mk(&R.ctl, 4);
  if (bad || cudaMallocHost(&r->h_ctl, 4 * sizeof(double)) != cudaSuccess ||
      cudaMallocHost(&r->h_ring, 2 * hbi_rk_s::kSlots * sizeof(double)) != cudaSuccess) {
    hbi_rk_free(r);
    return fail(HBI_ERR_NOMEM, "RK state allocation");
  }
  for (int s = 0; s < hbi_rk_s::kSlots; s++) cudaEventCreateWithFlags(&r->slot_ev[s], cudaEventDisableTiming);
  r->mats[0] = ls->md; r->mats[0].scale = p->scale_s;
  if (ln) { r->mats[1] = ln->md; r->mats[1].scale = p->scale_n; }
  double B[15], C[6], DC[6];
  cash_karp(B, C, DC);
  set_tableau(B, C, DC);
  r->launches = 1 + 6 * 3;  // prepare + per stage: phase 1, phase 2 (both matrices), phase 3
  *out = r;
  return HBI_OK;
}

extern "C" int hbi_rk_free(hbi_rk* r) {
  if (!r) return HBI_OK;
  // a time loop may still run on its own stream with this handle's state
  cudaDeviceSynchronize();
  if (r->gexec) cudaGraphExecDestroy(r->gexec);
  for (double* p : r->allocs) cudaFree(p);
  if (r->h_ctl) cudaFreeHost(r->h_ctl);
  if (r->h_ring) cudaFreeHost(r->h_ring);
  for (int s = 0; s < hbi_rk_s::kSlots; s++)
    if (r->slot_ev[s]) cudaEventDestroy(r->slot_ev[s]);
  if (r->st) cudaStreamDestroy(r->st);
  delete r;
  return HBI_OK;
}

extern "C" int hbi_rk_launches_per_attempt(const hbi_rk* r) { return r ? r->launches : 0; }

namespace hbi {
// for the device-resident time loop (hbi_cycle.cu)
int rk_view(hbi_rk* r, RkView* v) {
  if (!r || !v) return fail(HBI_ERR_ARG, "null");
  v->R = r->R;
  v->mats[0] = r->mats[0];
  v->mats[1] = r->mats[r->nmat == 2 ? 1 : 0];
  v->nmat = r->nmat;
  v->n = r->n;
  v->sm = r->ls->ctl->sm_count;
  return HBI_OK;
}
int set_error(int code, const char* msg) { return fail(code, "%s", msg); }
// the filled leaves of a generate call, for the ensemble's tensor-core stores
int leaf_view(const hbi_leafmtxp* lf, const double** d_body, std::vector<int64_t>* off,
              std::vector<Leaf>* leaves) {
  if (!lf || !d_body || !off || !leaves) return fail(HBI_ERR_ARG, "null");
  *d_body = lf->d_body;
  off->assign(lf->off.begin(), lf->off.begin() + lf->leaves.size());
  *leaves = lf->leaves;
  return HBI_OK;
}
// for the ensemble (hbi_ens.cu)
int lhp_view(hbi_lhp* h, LhpView* v) {
  if (!h || !v) return fail(HBI_ERR_ARG, "null");
  v->md = h->md;
  v->n = h->n;
  v->storage = h->storage;
  v->zlen = h->plan.zlen;
  v->plen1 = h->plan.plen1;
  v->plen2 = h->plan.plen2;
  v->ncg = h->plan.ncg;
  v->sm = h->ctl->sm_count;
  v->leaves = &h->leaves;
  return HBI_OK;
}
}  // namespace hbi

extern "C" int hbi_rk_set_state(hbi_rk* r, const double* y) {
  if (!r || !y) return fail(HBI_ERR_ARG, "null");
  CK(cudaMemcpy(r->R.y, y, sizeof(double) * 3 * r->n, cudaMemcpyHostToDevice));
  return HBI_OK;
}

// the error words of the RK handle's operators (after its stream has drained)
static int rk_device_error(hbi_rk* r, const char* where) {
  for (int k = 0; k < r->nmat; k++) {
    const int rc = device_error_status(r->mats[k], where);
    if (rc) return rc;
  }
  return HBI_OK;
}

extern "C" int hbi_rk_check_error(hbi_rk* r) {
  if (!r) return fail(HBI_ERR_ARG, "hbi_rk_check_error: null");
  CK(cudaStreamSynchronize(r->st));
  return rk_device_error(r, "hbi_rk_check_error");
}

extern "C" int hbi_rk_get_state(hbi_rk* r, double* y) {
  if (!r || !y) return fail(HBI_ERR_ARG, "null");
  CK(cudaStreamSynchronize(r->st));
  int rc = rk_device_error(r, "hbi_rk_get_state");
  if (rc) return rc;
  CK(cudaMemcpy(y, r->R.y, sizeof(double) * 3 * r->n, cudaMemcpyDeviceToHost));
  return HBI_OK;
}

// the six stages of one Cash-Karp attempt (rkck) as a fixed launch sequence
static void enqueue_attempt(hbi_rk* r, cudaStream_t st) {
  RkDev& R = r->R;
  const int sm = r->ls->ctl->sm_count;
  launch_rk_prepare(R, st);
  for (int s = 0; s < 6; s++) {
    const double* xin = s == 0 ? R.x0 : R.xb[s & 1];
    double* xout = R.xb[(s + 1) & 1];
    launch_phase1(r->mats, r->nmat, xin, sm, st);
    launch_phase2(r->mats, r->nmat, xin, sm, st);
    launch_phase3_rk(r->mats, r->nmat, R, s, xout, st);
  }
}

static int launch_attempt(hbi_rk* r, double h, double eps) {
  cudaStream_t st = r->st;
  // (h, eps) travel through a ring of pinned slots; a slot is rewritten only
  // after the copy that last read it has completed
  const int s = r->slot;
  r->slot = (r->slot + 1) % hbi_rk_s::kSlots;
  if (r->slot_used[s]) CK(cudaEventSynchronize(r->slot_ev[s]));
  double* hc = r->h_ring + 2 * s;
  hc[0] = h;
  hc[1] = eps;
  CK(cudaMemcpyAsync(r->R.ctl, hc, 2 * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaEventRecord(r->slot_ev[s], st));
  r->slot_used[s] = 1;
  if (!r->gexec) {
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    enqueue_attempt(r, st);
    CK(cudaStreamEndCapture(st, &g));
    CK(cudaGraphInstantiate(&r->gexec, g, 0));
    cudaGraphDestroy(g);
  }
  CK(cudaGraphLaunch(r->gexec, st));
  return HBI_OK;
}

extern "C" void* hbi_rk_stream(const hbi_rk* r) { return r ? (void*)r->st : nullptr; }

extern "C" int hbi_rk_attempt_async(hbi_rk* r, double h, double eps) {
  if (!r) return fail(HBI_ERR_ARG, "null");
  return launch_attempt(r, h, eps);
}

static int run_attempt(hbi_rk* r, double h, double eps, double* errmax) {
  cudaStream_t st = r->st;
  int rc0 = launch_attempt(r, h, eps);
  if (rc0) return rc0;
  CK(cudaMemcpyAsync(r->h_ctl + 2, r->R.ctl + 2, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  int rc1 = rk_device_error(r, "Runge-Kutta attempt");
  if (rc1) return rc1;
  double e = r->h_ctl[2];
  long long hidx;
  memcpy(&hidx, &r->h_ctl[3], sizeof(hidx));
  if (hidx >= 0) {
    // a component with ytemp-1 == ytemp: the reference resets errmax to 10 at
    // that index, so only later components can raise it (main_LH.f90:2309-2313)
    std::vector<double> eb(3 * (size_t)r->n);
    CK(cudaMemcpy(eb.data(), r->R.ebuf, sizeof(double) * eb.size(), cudaMemcpyDeviceToHost));
    e = 10.0;
    for (size_t c = (size_t)hidx + 1; c < eb.size(); c++)
      if (eb[c] > e) e = eb[c];
  }
  *errmax = e;
  return HBI_OK;
}

extern "C" int hbi_rkck(hbi_rk* r, double h, double eps, double* yout, double* yerr, double* errmax) {
  if (!r) return fail(HBI_ERR_ARG, "null");
  double e;
  int rc = run_attempt(r, h, eps, &e);
  if (rc) return rc;
  if (errmax) *errmax = e;
  if (yout) CK(cudaMemcpy(yout, r->R.yout, sizeof(double) * 3 * r->n, cudaMemcpyDeviceToHost));
  if (yerr) CK(cudaMemcpy(yerr, r->R.yerr, sizeof(double) * 3 * r->n, cudaMemcpyDeviceToHost));
  return HBI_OK;
}

extern "C" int hbi_derivs(hbi_rk* r, const double* y, double* dydx) {
  if (!r || !y || !dydx) return fail(HBI_ERR_ARG, "null");
  // stage 0 of an attempt from y gives k1 = f(y)
  std::vector<double> keep(3 * (size_t)r->n);
  CK(cudaMemcpy(keep.data(), r->R.y, sizeof(double) * keep.size(), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(r->R.y, y, sizeof(double) * keep.size(), cudaMemcpyHostToDevice));
  double e;
  int rc = run_attempt(r, 0.0, 1.0, &e);
  if (rc) return rc;
  CK(cudaMemcpy(dydx, r->R.K, sizeof(double) * keep.size(), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(r->R.y, keep.data(), sizeof(double) * keep.size(), cudaMemcpyHostToDevice));
  return HBI_OK;
}

extern "C" int hbi_rkqs(hbi_rk* r, double* x, double htry, double eps, double dtmax, double* hdid, double* hnext,
                        double* errmax, int* nrjct) {
  if (!r || !x) return fail(HBI_ERR_ARG, "null");
  // rkqs constants: SAFETY=0.9, PGROW=-0.2, PSHRNK=-0.25, tiny=1e-20 written as
  // default-real literals (main_LH.f90:2290)
  const double SAFETY = (double)0.9f, PGROW = (double)-0.2f, PSHRNK = -0.25, tiny = (double)1e-20f;
  double h = htry, e = 0.0;
  int nr = 0;
  for (;;) {
    int rc = run_attempt(r, h, eps, &e);
    if (rc) return rc;
    if ((e < 1.0) && (e > tiny)) break;
    nr++;
    if (e > tiny) h = std::max(0.5 * h, SAFETY * h * std::pow(e, PSHRNK));
    else h = 0.5 * h;
    const double xnew = *x + h;
    if (xnew - *x < 1.e-15) {
      if (errmax) *errmax = e;
      if (nrjct) *nrjct = nr;
      return fail(HBI_ERR_CONVERGE, "Runge-Kutta step size underflow at x=%.17g", *x);
    }
  }
  double hn = std::min(2 * h, SAFETY * h * std::pow(e, PGROW));
  hn = std::min(hn, dtmax);
  CK(cudaMemcpyAsync(r->R.y, r->R.yout, sizeof(double) * 3 * r->n, cudaMemcpyDeviceToDevice, r->st));
  CK(cudaStreamSynchronize(r->st));
  if (hdid) *hdid = h;
  if (hnext) *hnext = hn;
  if (errmax) *errmax = e;
  if (nrjct) *nrjct = nr;
  *x = *x + h;
  return HBI_OK;
}

// ------------------------------------------------- work-plan self check (host)
// Runs plan_stream on a leaf list and walks its items exactly as the phase
// kernels do, in FP64 on the host: y = H x from a HACApK-packed body.  Checks
// every bound the kernels rely on (regions inside the stores and at most one
// stage, 16-byte alignment, indices inside z / x / partials).  stats (8):
// phase-1 items, phase-2 items, V store, U store (elements), z length,
// phase-1 partials, phase-2 partials, conversion segments.
//
// chunks_fit: a column segment of ntp rows gives whole chunks of 16 to 128
// columns inside both stage sizes of the phase kernels (8 KB and 16 KB).
static bool chunks_fit(int ntp, int esz) {
  for (int sb : {8192, 16384}) {
    const int cc = chunk_cols(ntp, esz, sb);
    if (cc < 16 || cc > 128 || (int64_t)cc * ntp * esz > sb) return false;
  }
  return true;
}

extern "C" int hbi_plan_emulate(int n, int nleaf, const int* lv6, const double* body, int vec, const double* x,
                                double* y, int64_t* stats) {
  if (n < 1 || nleaf < 1 || !lv6 || !body || !x || !y || (vec != 2 && vec != 4 && vec != 8))
    return fail(HBI_ERR_ARG, "hbi_plan_emulate: bad arguments");
  std::vector<Leaf> L(nleaf);
  std::vector<int64_t> boff(nleaf);
  int64_t off = 0;
  for (int i = 0; i < nleaf; i++) {
    const int* q = lv6 + 6 * i;
    L[i] = Leaf{q[0], q[1], q[2], q[3], q[4], q[5]};
    boff[i] = off;
    off += L[i].ltmtx == 1 ? (int64_t)L[i].kt * (L[i].ndl + L[i].ndt) : (int64_t)L[i].ndl * L[i].ndt;
  }
  StreamPlan P;
  plan_stream(n, L, boff, vec, P);
  const int esz = 16 / vec;
  std::vector<double> V(P.vstore, 0.0), U(P.ustore, 0.0);
  int64_t nseg_conv = 0;
  for (int w = 0; w < 2; w++) {
    const std::vector<SegCopy>& map = w ? P.ucopy : P.vcopy;
    std::vector<double>& dst = w ? U : V;
    for (const SegCopy& c : map) {
      if (c.dst < 0 || c.dst + c.len > (int64_t)dst.size() || c.dst % vec) return fail(HBI_ERR_STATE, "copy dst");
      if (c.src < 0 || c.src + (int64_t)(c.len - 1) * c.stride >= off) return fail(HBI_ERR_STATE, "copy src");
      if (c.swz < 0 || c.swz >= 8 || (w == 1 && c.swz != 0)) return fail(HBI_ERR_STATE, "copy swizzle");
      for (int r = 0; r < c.len; r++) {
        const int64_t d = c.dst + (int64_t)(((r / vec) ^ c.swz) * vec + r % vec);
        if (d >= (int64_t)dst.size()) return fail(HBI_ERR_STATE, "swizzled copy dst");
        dst[d] = body[c.src + (int64_t)r * c.stride];
      }
    }
    nseg_conv += (int64_t)map.size();
  }
  std::vector<double> z(std::max<int64_t>(P.zlen, 1), 0.0), part(std::max<int64_t>(P.plen1, 1), 0.0);
  for (const S1Item& it : P.p1) {
    if (it.ncols < 1 || it.ntp % vec || it.ntp > 32 * vec || !chunks_fit(it.ntp, esz) || it.cc != chunk_cols(it.ntp, esz, 8192) || it.soff % vec ||
        it.soff + (int64_t)it.ncols * it.ntp > P.vstore || it.x0 < 0 || it.x0 + it.nt > n || it.nt > it.ntp ||
        it.z0 < 0 || it.z0 + it.ncols > P.zlen ||
        (it.ntile > 1 && (it.cg < 0 || it.cg >= P.ncg || it.poff < 0 ||
                          it.poff + (int64_t)it.ntile * it.ncols > P.plen1)))
      return fail(HBI_ERR_STATE, "phase-1 item out of bounds");
    const int nq = it.ntp / vec;
    for (int c = 0; c < it.ncols; c++) {
      // the kernels find logical row r of column c at its swizzled place
      const int sw = vswz(c, nq);
      // every swizzled vector index stays inside the column's segment
      for (int k = 0; k < nq; k++)
        if ((k ^ sw) >= nq) return fail(HBI_ERR_STATE, "phase-1 swizzle leaves the segment");
      double t = 0.0;
      for (int r = 0; r < it.nt; r++)
        t += V[it.soff + (int64_t)c * it.ntp + ((r / vec) ^ sw) * vec + r % vec] * x[it.x0 + r];
      if (it.ntile == 1) z[it.z0 + c] = t;
      else part[it.poff + (int64_t)it.tile * it.ncols + c] = t;
    }
  }
  for (const S1Item& it : P.p1)
    if (it.ntile > 1 && it.tile == 0)
      for (int c = 0; c < it.ncols; c++) {
        double t = 0.0;
        for (int q = 0; q < it.ntile; q++) t += part[it.poff + (int64_t)q * it.ncols + c];
        z[it.z0 + c] = t;
      }
  std::vector<double> gp(std::max<int64_t>(P.plen2, 1), 0.0);
  for (const S2Item& it : P.p2) {
    if (it.ncols < 1 || it.ntp % vec || it.ntp > 32 * vec || !chunks_fit(it.ntp, esz) || it.cc != chunk_cols(it.ntp, esz, 8192) || it.soff % vec ||
        it.soff + (int64_t)it.ncols * it.ntp > P.ustore || it.nr > it.ntp || it.m0 < 0 ||
        it.m0 + (int64_t)it.ncols > (int64_t)P.midx.size() || it.pout < 0 || it.pout + it.nr > P.plen2)
      return fail(HBI_ERR_STATE, "phase-2 item out of bounds");
    for (int r = 0; r < it.nr; r++) {
      double t = 0.0;
      for (int c = 0; c < it.ncols; c++) {
        const int mi = P.midx[it.m0 + c];
        if (mi >= P.zlen || -mi - 1 >= n) return fail(HBI_ERR_STATE, "multiplier index");
        const double mu = mi >= 0 ? z[mi] : x[-mi - 1];
        t += U[it.soff + (int64_t)c * it.ntp + r] * mu;
      }
      gp[it.pout + r] = t;
    }
  }
  const GroupPlan& G = P.gp;
  for (int r = 0; r < n; r++) {
    double t = 0.0, t2 = 0.0;
    const int f = G.row_fc[r];
    for (int e = G.fc_ptr[f]; e < G.fc_ptr[f + 1]; e++) {
      const int g = G.fc_group[e];
      if (P.gnch[g] > 1) return fail(HBI_ERR_STATE, "more than one partial per group");
      for (int c = 0; c < P.gnch[g]; c++) t += gp[P.gpoff2[g] + (int64_t)c * G.gndl[g] + r - G.grow0[g]];
    }
    // the kernels' flat lists give the same terms in the same order
    for (int e = P.fcb_ptr[f]; e < P.fcb_ptr[f + 1]; e++) {
      const int64_t q = (int64_t)P.fcb_base[e] + r;
      if (q < 0 || q >= P.plen2) return fail(HBI_ERR_STATE, "phase-3 partial out of bounds");
      t2 += gp[q];
    }
    if (t2 != t) return fail(HBI_ERR_STATE, "phase-3 lists disagree");
    y[r] = t;
  }
  if (stats) {
    stats[0] = (int64_t)P.p1.size(); stats[1] = (int64_t)P.p2.size(); stats[2] = P.vstore; stats[3] = P.ustore;
    stats[4] = P.zlen; stats[5] = P.plen1; stats[6] = P.plen2; stats[7] = nseg_conv;
  }
  return HBI_OK;
}

// ------------------------------------------- tensor-core plan self check (host)
namespace {
// round to bfloat16 (nearest even) through float, as __float2bfloat16_rn does
float bf16_round(double x) {
  float f = (float)x;
  uint32_t u;
  memcpy(&u, &f, 4);
  if ((u & 0x7f800000u) != 0x7f800000u) u = (u + 0x7fffu + ((u >> 16) & 1u)) & 0xffff0000u;
  else u &= 0xffff0000u;
  memcpy(&f, &u, 4);
  return f;
}
int64_t tc_offset(int np, int n, int k) {
  const int c = k / 16, kk = k % 16;
  return (int64_t)c * np * 32 + (int64_t)(kk / 8) * np * 8 + (int64_t)(n / 8) * 64 + (n % 8) * 8 + (kk % 8);
}
}  // namespace

// y = H x through the tensor-core plan of the ensemble product (one member),
// with the factors rounded to BF16 hi + lo as the device stores them; checks
// every bound the kernels rely on.  stats (4): items of phase 1 and 2, store
// elements of phase 1 and 2.
extern "C" int hbi_plan_warp_schedule(int n, const int64_t* cost, int nwarps, int32_t* woff, int32_t* witem) {
  if (n < 0 || nwarps < 1 || (n > 0 && (!cost || !witem)) || !woff)
    return fail(HBI_ERR_ARG, "hbi_plan_warp_schedule: bad arguments");
  std::vector<int64_t> c(cost, cost + n);
  std::vector<int32_t> o, it;
  plan_warp_schedule(c, nwarps, o, it);
  std::copy(o.begin(), o.end(), woff);
  std::copy(it.begin(), it.end(), witem);
  return HBI_OK;
}

extern "C" int hbi_tc_plan_emulate(int n, int nleaf, const int* lv6, const double* body, const double* x, double* y,
                                   int64_t* stats) {
  if (n < 1 || nleaf < 1 || !lv6 || !body || !x || !y) return fail(HBI_ERR_ARG, "hbi_tc_plan_emulate: arguments");
  std::vector<Leaf> L(nleaf);
  std::vector<int64_t> boff(nleaf);
  int64_t off = 0;
  for (int i = 0; i < nleaf; i++) {
    const int* q = lv6 + 6 * i;
    L[i] = Leaf{q[0], q[1], q[2], q[3], q[4], q[5]};
    boff[i] = off;
    off += L[i].ltmtx == 1 ? (int64_t)L[i].kt * (L[i].ndl + L[i].ndt) : (int64_t)L[i].ndl * L[i].ndt;
  }
  TcPlan T;
  plan_tc(n, L, boff, T);
  std::vector<double> S1(T.store1, 0.0), S2(T.store2, 0.0);
  for (int ph = 1; ph <= 2; ph++) {
    const std::vector<TcCopy>& cp = ph == 1 ? T.copy1 : T.copy2;
    std::vector<double>& S = ph == 1 ? S1 : S2;
    for (const TcCopy& c : cp)
      for (int i = 0; i < c.len; i++) {
        const int nn = c.n0 + i * c.dn, kk = c.k0 + i * c.dk;
        if (nn >= c.np) return fail(HBI_ERR_STATE, "tc copy: n beyond the item");
        const int64_t o = c.item + tc_offset(c.np, nn, kk);
        const int64_t src = c.src + (int64_t)i * c.stride;
        if (src < 0 || src >= off || o < 0 || o + (int64_t)c.np * 16 >= (int64_t)S.size() + 1)
          return fail(HBI_ERR_STATE, "tc copy out of bounds");
        const double v = body[src];
        const double hi = bf16_round(v);
        S[o] = hi;
        S[o + (int64_t)c.np * 16] = bf16_round(v - hi);
      }
  }
  std::vector<double> z(std::max<int64_t>(T.zlen, 1), 0.0), part(std::max<int64_t>(T.plen1, 1), 0.0);
  for (const TcItem& it : T.p1) {
    if (it.np % 8 || it.np > 256 || it.kp % 16 || it.kp > kTcK1 || it.nv > it.np || it.kv > it.kp || it.m0 < 0 ||
        it.m0 + it.kv > n || it.out0 + it.nv > T.zlen || it.soff + (int64_t)it.kp * it.np * 2 > T.store1 ||
        (it.ntile > 1 && it.poff + (int64_t)it.ntile * it.nv > T.plen1))
      return fail(HBI_ERR_STATE, "tc phase-1 item out of bounds");
    for (int c = 0; c < it.nv; c++) {
      double t = 0.0;
      for (int k = 0; k < it.kv; k++) {
        const int64_t o = it.soff + tc_offset(it.np, c, k);
        t += (S1[o] + S1[o + (int64_t)it.np * 16]) * x[it.m0 + k];
      }
      if (it.ntile == 1) z[it.out0 + c] = t;
      else part[it.poff + (int64_t)it.tile * it.nv + c] = t;
    }
  }
  for (const TcItem& it : T.p1)
    if (it.ntile > 1 && it.tile == 0)
      for (int c = 0; c < it.nv; c++) {
        double t = 0.0;
        for (int q = 0; q < it.ntile; q++) t += part[it.poff + (int64_t)q * it.nv + c];
        z[it.out0 + c] = t;
      }
  GroupPlan G;
  plan_groups(n, L, G);
  int64_t plen2 = 0;
  for (size_t g = 0; g < G.grow0.size(); g++) plen2 += G.gndl[g];
  std::vector<double> gp(std::max<int64_t>(plen2, 1), 0.0);
  for (const TcItem& it : T.p2) {
    if (it.np % 8 || it.np > 256 || it.kp % 16 || it.nv > it.np || it.kv > it.kp || it.m0 % 4 ||
        it.m0 + it.kp > (int64_t)T.midx.size() || it.out0 + it.nv > plen2 ||
        it.soff + (int64_t)it.kp * it.np * 2 > T.store2)
      return fail(HBI_ERR_STATE, "tc phase-2 item out of bounds");
    for (int r = 0; r < it.nv; r++) {
      double t = 0.0;
      for (int k = 0; k < it.kv; k++) {
        const int mi = T.midx[it.m0 + k];
        const double mu = mi >= 0 ? z[mi] : x[-mi - 1];
        const int64_t o = it.soff + tc_offset(it.np, r, k);
        t += (S2[o] + S2[o + (int64_t)it.np * 16]) * mu;
      }
      gp[it.out0 + r] = t;
    }
  }
  for (int r = 0; r < n; r++) {
    double t = 0.0;
    const int f = G.row_fc[r];
    int64_t base = 0;
    (void)base;
    for (int e = G.fc_ptr[f]; e < G.fc_ptr[f + 1]; e++) {
      const int g = G.fc_group[e];
      int64_t go = 0;
      for (int q = 0; q < g; q++) go += G.gndl[q];
      t += gp[go + r - G.grow0[g]];
    }
    y[r] = t;
  }
  if (stats) {
    stats[0] = (int64_t)T.p1.size(); stats[1] = (int64_t)T.p2.size(); stats[2] = T.store1; stats[3] = T.store2;
  }
  return HBI_OK;
}
