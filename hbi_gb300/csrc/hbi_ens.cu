// hbi_ens.cu -- an ensemble of rate-and-state systems sharing one pair of
// H-matrices (configuration c4: 64 simulations with their own b and dc on the
// c2 fault).
//
// Every RK stage applies each H-matrix to the 64 members' slip-rate vectors
// at once.  The multi-vector product streams the same row-tiled FP32 stores
// as the single-system product (plan_stream): a block takes one (group, row
// tile) item at a time, its factor chunks arrive by cp.async.bulk (TMA) into
// two shared-memory stages, and the members sit across the lanes:
//   phase 1  Z[col][m] = sum_rows V[row][col] X[row][m]; the item's X rows
//            (rows x 64 members, FP32) are bulk-copied once per item, the next
//            item's while the current one is consumed;
//   phase 2  Y[row][m] = sum_cols U[row][col] B[col][m], B the rows of Z (low
//            rank) or X (dense) of the chunk's columns, gathered by one bulk
//            copy per column; 16 rows x 2 members per thread in registers;
//   phase 3  per (row, member): the covering groups' partial rows, then the
//            FP64 rate-and-state derivative and Cash-Karp stage combination.
// Each member keeps its own FP64 state, step size and rkqs controller
// (main_LH.f90:2270-2370); every member is tried at every ensemble attempt
// with its own h, and accepts or rejects on its own error.  Members that
// reached the time limit keep computing (h = 0) but no longer change.
//
// Simplification against the single-system loop: when a component of a
// member's 5th-order solution is so large that y - 1 == y, the member's
// errmax is raised to at least 10 (a rejection) instead of replaying the
// reference's order-dependent rule.  No events, monitors or files.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/hbi_gpu.h"
#include "hbi_enstc.cuh"
#include "hbi_kernels.cuh"
#include "hbi_rsf.cuh"

namespace hbi {
int set_error(int code, const char* msg);
int lhp_view(hbi_lhp* h, LhpView* v);
int leaf_view(const hbi_leafmtxp* lf, const double** d_body, std::vector<int64_t>* off, std::vector<Leaf>* leaves);


namespace {

constexpr int EM = 64;                   // members (lanes x 2)
constexpr int kChunk = 16384;            // factor bytes per stage
constexpr int kXT = 128 * EM * 4;        // one X tile: 128 rows x 64 members, FP32
constexpr int kBrows = 32 * EM * 4;      // phase-2 multipliers of one chunk: 32 columns x 64 members
constexpr long long kWait = 2LL << 30;   // bounded waits, SM clock cycles

__constant__ double eB[15];
__constant__ double eC[6];
__constant__ double eDC[6];

struct EnsMat {                          // one H-matrix and its ensemble scratch
  MatDev m;
  float* z;                              // zlen x EM
  float* part;                           // plen1 x EM
  int* cnt;                              // per column group
  float* gpart;                          // plen2 x EM
};

struct EnsDev {
  int n, nmat, evlaw, backslip, limitsigma;
  double vref, minsig, maxsig, rigid_over_2vs;
  const double *a, *f0, *taudot, *sigdot, *vpl;  // per element
  const double *b, *dc;                          // per (element, member)
  double *y, *ys, *vs, *ws, *K, *yout, *vel, *slip;  // (element[,component], member)
  float *x0, *xb[2];                             // product inputs (element, member)
  double *h, *x, *hdid, *tlim;                   // per member
  int *accepted, *done, *failed, *nr;            // per member
  unsigned long long* emax;                      // per member, bits of a non-negative double
  int* huge;                                     // per member
  long long* counters;                           // [0] steps [1] rejected
  int* ndone;                                    // host-mapped: members done or failed
  double eps, dtmax;
};

__device__ __forceinline__ uint32_t sa(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void bar_init(uint64_t* b) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sa(b)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void bar_expect(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sa(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool bar_try(uint64_t* b, uint32_t par) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(sa(b)), "r"(par)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void bulk(void* dst, const void* src, uint32_t bytes, uint64_t* b) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   sa(dst)),
               "l"(src), "r"(bytes), "r"(sa(b))
               : "memory");
}
// factor chunks are read once per product: evicted first from L2
__device__ __forceinline__ void bulk_stream(void* dst, const void* src, uint32_t bytes, uint64_t* b) {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
          sa(dst)),
      "l"(src), "r"(bytes), "r"(sa(b)), "l"(pol)
      : "memory");
}
__device__ __forceinline__ void fence_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// block-wide bounded wait; false (and the error word set) on time-out.
// limit: the operator's bound in SM clock cycles; 0 is spent before the
// first probe, so every wait gives up (the error path on demand)
__device__ bool block_wait(uint64_t* b, uint32_t par, int* err, long long limit, int* sh_ok) {
  if (threadIdx.x == 0) {
    int ok = limit > 0 && bar_try(b, par);
    if (!ok && limit > 0) {
      const long long t0 = clock64();
      while (!(ok = bar_try(b, par)))
        if (clock64() - t0 > limit) break;
    }
    *sh_ok = ok;
    if (!ok && err) atomicExch(err, 1);
  }
  __syncthreads();
  const int ok = *sh_ok;
  // every thread observes the completed phase itself (acquire); the phase
  // stays completed until this block refills the stage, so the probe passes
  // at once -- bounded all the same
  if (ok) {
    const long long t1 = clock64();
    while (!bar_try(b, par))
      if (clock64() - t1 > kWait) break;
  }
  return ok != 0;
}

// after a failed wait: let the block's copies still in flight land (bounded)
__device__ void drain_e(uint64_t* bar, int c_seq, int p_seq, int xj) {
  if (threadIdx.x == 0) {
    for (int q = c_seq; q < p_seq; q++) {
      const long long t0 = clock64();
      while (!bar_try(&bar[q & 1], (uint32_t)((q >> 1) & 1)))
        if (clock64() - t0 > kWait) break;
    }
    if (xj >= 0) {
      const long long t0 = clock64();
      while (!bar_try(&bar[2 + (xj & 1)], (uint32_t)((xj >> 1) & 1)))
        if (clock64() - t0 > kWait) break;
    }
  }
  __syncthreads();
}

__device__ __forceinline__ int ccols(int ntp) { return min((kChunk / (ntp * 4)) / 32 * 32, 256); }
__device__ __forceinline__ int arrive_acq_rel(int* p) {
  int old;
  asm volatile("atom.add.acq_rel.gpu.s32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
  return old;
}

// ---------------------------------------------------------------- phase 1
__global__ void __launch_bounds__(256, 2) p1e_kernel(EnsMat A, EnsMat B, int nmat, const float* __restrict__ X) {
  extern __shared__ __align__(128) unsigned char sm[];
  float* xs[2] = {(float*)sm, (float*)(sm + kXT)};
  unsigned char* cs[2] = {sm + 2 * kXT, sm + 2 * kXT + kChunk};
  uint64_t* bar = (uint64_t*)(sm + 2 * kXT + 2 * kChunk);  // [0,1] chunks, [2,3] X tiles
  __shared__ int sh_ok, sh_last;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int i = tid; i < 2 * kXT / 16; i += blockDim.x) ((uint4*)sm)[i] = make_uint4(0, 0, 0, 0);
  if (tid == 0)
    for (int i = 0; i < 4; i++) bar_init(&bar[i]);
  __syncthreads();
  const int n0 = A.m.ns1, ntot = nmat == 2 ? n0 + B.m.ns1 : n0;
  const int G = gridDim.x;
  auto desc = [&](int it) -> S1Item {
    S1Item d{};
    if (it < ntot) d = it < n0 ? A.m.s1[it] : B.m.s1[it - n0];
    return d;
  };
  int p_it = blockIdx.x, p_c0 = 0, p_seq = 0;
  S1Item Dp = desc(p_it);
  auto produce = [&]() {
    if (p_it >= ntot) return;
    const int nc = min(ccols(Dp.ntp), Dp.ncols - p_c0);
    const int s = p_seq & 1;
    if (tid == 0) {
      const uint32_t bytes = (uint32_t)(nc * Dp.ntp * 4);
      const float* src = (const float*)(p_it < n0 ? A.m.vstore : B.m.vstore) + Dp.soff + (int64_t)p_c0 * Dp.ntp;
      fence_async();
      bar_expect(&bar[s], bytes);
      bulk_stream(cs[s], src, bytes, &bar[s]);
    }
    p_seq++;
    p_c0 += nc;
    if (p_c0 >= Dp.ncols) {
      p_it += G;
      p_c0 = 0;
      Dp = desc(p_it);
    }
  };
  auto issue_x = [&](int it, int j) {
    if (it >= ntot || tid != 0) return;
    const S1Item D = desc(it);
    const uint32_t bytes = (uint32_t)(D.nt * EM * 4);
    fence_async();
    bar_expect(&bar[2 + (j & 1)], bytes);
    bulk(xs[j & 1], X + (int64_t)D.x0 * EM, bytes, &bar[2 + (j & 1)]);
  };
  produce();
  produce();
  issue_x(blockIdx.x, 0);
  int c_it = blockIdx.x, c_c0 = 0, c_seq = 0, j = 0;
  S1Item Dc = desc(c_it);
  while (c_it < ntot) {
    const EnsMat& M = c_it < n0 ? A : B;
    if (c_c0 == 0) {
      if (!block_wait(&bar[2 + (j & 1)], (uint32_t)((j >> 1) & 1), M.m.err, M.m.wait, &sh_ok)) {
        drain_e(bar, c_seq, p_seq, -1);
        return;
      }
      issue_x(c_it + G, j + 1);
    }
    const int s = c_seq & 1;
    if (!block_wait(&bar[s], (uint32_t)((c_seq >> 1) & 1), M.m.err, M.m.wait, &sh_ok)) {
      drain_e(bar, c_seq, p_seq, c_it + G < ntot ? j + 1 : -1);
      return;
    }
    const int nc = min(ccols(Dc.ntp), Dc.ncols - c_c0);
    const float* V = (const float*)cs[s];
    const float* xt = xs[j & 1];
    const int nt4 = (Dc.nt + 3) & ~3;
    for (int base = 0; base < nc; base += 32) {
      float acc[4][2];
      bool ok[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        acc[q][0] = acc[q][1] = 0.f;
        ok[q] = base + warp + 8 * q < nc;
      }
      for (int r = 0; r < nt4; r += 4) {
        float x0[4], x1[4];
#pragma unroll
        for (int rr = 0; rr < 4; rr++) {
          x0[rr] = xt[(r + rr) * EM + lane];
          x1[rr] = xt[(r + rr) * EM + lane + 32];
        }
#pragma unroll
        for (int q = 0; q < 4; q++) {
          if (!ok[q]) continue;
          // the V store's swizzle (vswz) of column base + warp + 8q; chunks
          // start at multiples of 32 columns, so chunk and item columns agree mod 8
          const int cl = base + warp + 8 * q;
          const float4 v = *(const float4*)(V + cl * Dc.ntp + (((r >> 2) ^ vswz(cl, Dc.ntp >> 2)) << 2));
          acc[q][0] += v.x * x0[0] + v.y * x0[1] + v.z * x0[2] + v.w * x0[3];
          acc[q][1] += v.x * x1[0] + v.y * x1[1] + v.z * x1[2] + v.w * x1[3];
        }
      }
#pragma unroll
      for (int q = 0; q < 4; q++) {
        if (!ok[q]) continue;
        const int col = c_c0 + base + warp + 8 * q;
        float* dst = Dc.ntile == 1 ? M.z + (int64_t)(Dc.z0 + col) * EM
                                   : M.part + ((int64_t)Dc.poff + (int64_t)Dc.tile * Dc.ncols + col) * EM;
        dst[lane] = acc[q][0];
        dst[lane + 32] = acc[q][1];
      }
    }
    __syncthreads();
    c_seq++;
    produce();
    c_c0 += nc;
    if (c_c0 < Dc.ncols) continue;
    if (Dc.ntile > 1) {
      __threadfence();
      __syncthreads();
      if (tid == 0) sh_last = arrive_acq_rel(&M.cnt[Dc.cg]) == Dc.ntile - 1;
      __syncthreads();
      if (sh_last) {
        for (int idx = tid; idx < Dc.ncols * EM; idx += blockDim.x) {
          const int col = idx / EM, m = idx % EM;
          float t = 0.f;
          for (int q = 0; q < Dc.ntile; q++)
            t += __ldcg(&M.part[((int64_t)Dc.poff + (int64_t)q * Dc.ncols + col) * EM + m]);
          M.z[(int64_t)(Dc.z0 + col) * EM + m] = t;
        }
        if (tid == 0) M.cnt[Dc.cg] = 0;
      }
      __syncthreads();
    }
    c_it += G;
    c_c0 = 0;
    j++;
    Dc = desc(c_it);
  }
}

// ---------------------------------------------------------------- phase 2
__global__ void __launch_bounds__(256, 2) p2e_kernel(EnsMat A, EnsMat B, int nmat, const float* __restrict__ X) {
  extern __shared__ __align__(128) unsigned char sm[];
  constexpr int kStageE = kChunk + kBrows;
  unsigned char* st[2] = {sm, sm + kStageE};
  float* red = (float*)(sm + 2 * kStageE);  // 8 x 16 rows x EM
  uint64_t* bar = (uint64_t*)(sm + 2 * kStageE + 8 * 16 * EM * 4);
  __shared__ int sh_ok;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0)
    for (int i = 0; i < 2; i++) bar_init(&bar[i]);
  __syncthreads();
  const int n0 = A.m.ns2, ntot = nmat == 2 ? n0 + B.m.ns2 : n0;
  const int G = gridDim.x;
  auto desc = [&](int it) -> S2Item {
    S2Item d{};
    if (it < ntot) d = it < n0 ? A.m.s2[it] : B.m.s2[it - n0];
    return d;
  };
  // columns of a phase-2 chunk: at most 32 (one multiplier row per lane)
  auto cc2 = [](int ntp) { return min(ccols(ntp), 32); };
  int p_it = blockIdx.x, p_c0 = 0, p_seq = 0;
  S2Item Dp = desc(p_it);
  auto produce = [&]() {
    if (p_it >= ntot) return;
    const int nc = min(cc2(Dp.ntp), Dp.ncols - p_c0);
    const int s = p_seq & 1;
    if (warp == 0) {
      const EnsMat& PM = p_it < n0 ? A : B;
      int mi = 0;
      if (lane < nc) mi = __ldg(&PM.m.midx[Dp.m0 + p_c0 + lane]);
      if (lane == 0) {
        fence_async();
        bar_expect(&bar[s], (uint32_t)(nc * Dp.ntp * 4 + nc * EM * 4));
        bulk_stream(st[s], (const float*)PM.m.ustore + Dp.soff + (int64_t)p_c0 * Dp.ntp, (uint32_t)(nc * Dp.ntp * 4),
             &bar[s]);
      }
      __syncwarp();
      if (lane < nc) {
        const float* src = mi >= 0 ? PM.z + (int64_t)mi * EM : X + (int64_t)(-mi - 1) * EM;
        fence_async();
        bulk(st[s] + kChunk + lane * EM * 4, src, EM * 4, &bar[s]);
      }
    }
    p_seq++;
    p_c0 += nc;
    if (p_c0 >= Dp.ncols) {
      p_it += G;
      p_c0 = 0;
      Dp = desc(p_it);
    }
  };
  produce();
  produce();
  int c_it = blockIdx.x, c_c0 = 0, c_seq = 0;
  S2Item Dc = desc(c_it);
  float acc[16][2];
#pragma unroll
  for (int i = 0; i < 16; i++) acc[i][0] = acc[i][1] = 0.f;
  while (c_it < ntot) {
    const EnsMat& M = c_it < n0 ? A : B;
    const int s = c_seq & 1;
    if (!block_wait(&bar[s], (uint32_t)((c_seq >> 1) & 1), M.m.err, M.m.wait, &sh_ok)) {
      drain_e(bar, c_seq, p_seq, -1);
      return;
    }
    const int nc = min(cc2(Dc.ntp), Dc.ncols - c_c0);
    // warps: RB row blocks of 16 rows x CSUB column subsets
    const int nrb = (Dc.ntp + 15) / 16;
    const int RB = nrb <= 1 ? 1 : nrb <= 2 ? 2 : nrb <= 4 ? 4 : 8;
    const int CSUB = 8 / RB;
    const int rb = warp % RB, csub = warp / RB;
    const float* U = (const float*)st[s];
    const float* Bm = (const float*)(st[s] + kChunk);
    const int r0 = rb * 16;
    if (r0 < Dc.ntp) {
      const int nq = min(4, (Dc.ntp - r0) / 4);  // float4 row quads of this block
      for (int c = csub; c < nc; c += CSUB) {
        const float b0 = Bm[c * EM + lane], b1 = Bm[c * EM + lane + 32];
#pragma unroll
        for (int q = 0; q < 4; q++) {
          if (q < nq) {
            const float4 u = *(const float4*)(U + c * Dc.ntp + r0 + 4 * q);
            acc[4 * q][0] += u.x * b0; acc[4 * q][1] += u.x * b1;
            acc[4 * q + 1][0] += u.y * b0; acc[4 * q + 1][1] += u.y * b1;
            acc[4 * q + 2][0] += u.z * b0; acc[4 * q + 2][1] += u.z * b1;
            acc[4 * q + 3][0] += u.w * b0; acc[4 * q + 3][1] += u.w * b1;
          }
        }
      }
    }
    __syncthreads();
    c_seq++;
    produce();
    c_c0 += nc;
    if (c_c0 < Dc.ncols) continue;
    // item done: combine the column subsets, write the tile's rows
    if (CSUB > 1) {
#pragma unroll
      for (int i = 0; i < 16; i++) {
        red[((csub * RB + rb) * 16 + i) * EM + lane] = acc[i][0];
        red[((csub * RB + rb) * 16 + i) * EM + lane + 32] = acc[i][1];
      }
      __syncthreads();
      for (int idx = tid; idx < Dc.nr * EM; idx += blockDim.x) {
        const int row = idx / EM, m = idx % EM;
        const int rbb = row / 16, i = row % 16;
        float t = 0.f;
        for (int k = 0; k < CSUB; k++) t += red[((k * RB + rbb) * 16 + i) * EM + m];
        M.gpart[((int64_t)Dc.pout + row) * EM + m] = t;
      }
      __syncthreads();
    } else {
#pragma unroll
      for (int i = 0; i < 16; i++) {
        const int row = r0 + i;
        if (row < Dc.nr) {
          M.gpart[((int64_t)Dc.pout + row) * EM + lane] = acc[i][0];
          M.gpart[((int64_t)Dc.pout + row) * EM + lane + 32] = acc[i][1];
        }
      }
    }
#pragma unroll
    for (int i = 0; i < 16; i++) acc[i][0] = acc[i][1] = 0.f;
    c_it += G;
    c_c0 = 0;
    Dc = desc(c_it);
  }
}

// per (row, member): the covering groups' partial rows, coarse to fine, from
// the flat per-fine-range offset list (independent loads, eight in flight)
__device__ __forceinline__ float group_sum_raw(const EnsMat& M, int r, int m) {
  const MatDev& d = M.m;
  const int f = __ldg(&d.row_fc[r]);
  const int e0 = __ldg(&d.fcb_ptr[f]), e1 = __ldg(&d.fcb_ptr[f + 1]);
  float s = 0.f;
  int e = e0;
  for (; e + 8 <= e1; e += 8) {
    float v[8];
#pragma unroll
    for (int u = 0; u < 8; u++) v[u] = __ldcg(&M.gpart[((int64_t)__ldg(&d.fcb_base[e + u]) + r) * EM + m]);
#pragma unroll
    for (int u = 0; u < 8; u++) s += v[u];
  }
  for (; e < e1; e++) s += __ldcg(&M.gpart[((int64_t)__ldg(&d.fcb_base[e]) + r) * EM + m]);
  return s;
}
// ... times the operator's scale (the traction of the stage)
__device__ __forceinline__ double group_sum_e(const EnsMat& M, int r, int m) {
  return (double)group_sum_raw(M, r, m) * M.m.scale;
}

// ---------------------------------------------------------------- phase 3
__global__ void __launch_bounds__(256) p3e_kernel(EnsMat A, EnsMat B, EnsDev E, int s, float* __restrict__ xnext) {
  __shared__ double se[256];
  __shared__ int sh[256];
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int m = (int)(idx % EM);
  const int r = (int)(idx / EM);
  double emax = -1.0;
  int huge = 0;
  if (r < E.n) {
    const int64_t n3 = 3LL * E.n;
    const double gs = group_sum_e(A, r, m) + E.taudot[r];
    const double gn = (E.nmat == 2 ? group_sum_e(B, r, m) : 0.0) + E.sigdot[r];
    const int64_t i0 = (3LL * r) * EM + m;
    const double psi = E.ys[i0], tau = E.ys[i0 + EM], sig = E.ys[i0 + 2 * EM];
    const double a = E.a[r], f0 = E.f0[r];
    const double bb = E.b[(int64_t)r * EM + m], dc = E.dc[(int64_t)r * EM + m];
    double k[3];
    deriv_dev(E, gs, gn, psi, tau, sig, E.vs[(int64_t)r * EM + m], E.ws[(int64_t)r * EM + m], a, bb, dc, f0, k);
    double* Ks = E.K + (int64_t)s * n3 * EM + i0;
    Ks[0] = k[0]; Ks[EM] = k[1]; Ks[2 * EM] = k[2];
    const double h = E.h[m];
    const double* K0 = E.K + i0;
    const int64_t st = n3 * EM;
    if (s < 5) {
      double yn[3];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const double y = E.y[i0 + c * EM];
        const double k1 = K0[c * EM];
        double v;
        if (s == 0) v = y + eB[0] * h * k[c];
        else if (s == 1) v = y + h * (eB[1] * k1 + eB[2] * k[c]);
        else if (s == 2) v = y + h * (eB[3] * k1 + eB[4] * K0[st + c * EM] + eB[5] * k[c]);
        else if (s == 3)
          v = y + h * (eB[6] * k1 + eB[7] * K0[st + c * EM] + eB[8] * K0[2 * st + c * EM] + eB[9] * k[c]);
        else
          v = y + h * (eB[10] * k1 + eB[11] * K0[st + c * EM] + eB[12] * K0[2 * st + c * EM] +
                       eB[13] * K0[3 * st + c * EM] + eB[14] * k[c]);
        yn[c] = v;
        E.ys[i0 + c * EM] = v;
      }
      double vn, wn;
      slip_rate_w(E.vref, yn[0], yn[1], yn[2], a, &vn, &wn);
      E.vs[(int64_t)r * EM + m] = vn;
      E.ws[(int64_t)r * EM + m] = wn;
      xnext[(int64_t)r * EM + m] = (float)(E.backslip ? (vn + 0.0) - E.vpl[r] : vn + 0.0);
    } else {
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const double y = E.y[i0 + c * EM];
        const double k1 = K0[c * EM], k3 = K0[2 * st + c * EM], k4 = K0[3 * st + c * EM],
                     k5 = K0[4 * st + c * EM], k6 = k[c];
        const double yo = y + h * (eC[0] * k1 + eC[2] * k3 + eC[3] * k4 + eC[5] * k6);
        const double ye = h * (eDC[0] * k1 + eDC[2] * k3 + eDC[3] * k4 + eDC[4] * k5 + eDC[5] * k6);
        E.yout[i0 + c * EM] = yo;
        const double e = fabs(ye / yo) / E.eps;
        if (e > emax) emax = e;
        if (yo - 1 == yo) huge = 1;
      }
    }
  }
  if (s == 5) {
    // per member over the block's rows (threads tid, tid+64, ...), then one atomic
    se[threadIdx.x] = emax;
    sh[threadIdx.x] = huge;
    __syncthreads();
    if (threadIdx.x < EM) {
      double e = -1.0;
      int hg = 0;
      for (int t = threadIdx.x; t < (int)blockDim.x; t += EM) {
        if (se[t] > e) e = se[t];
        hg |= sh[t];
      }
      if (e >= 0.0) atomicMax(&E.emax[threadIdx.x], (unsigned long long)__double_as_longlong(e));
      if (hg) atomicOr(&E.huge[threadIdx.x], 1);
    }
  }
}

// start of an ensemble attempt: stage state = accepted state, its slip rate,
// the stage-1 product input; clear the error maxima
__global__ void prepare_e_kernel(EnsDev E) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx < EM) {
    E.emax[idx] = 0ull;
    E.huge[idx] = 0;
  }
  const int m = (int)(idx % EM);
  const int r = (int)(idx / EM);
  if (r >= E.n) return;
  const int64_t i0 = (3LL * r) * EM + m;
  const double psi = E.y[i0], tau = E.y[i0 + EM], sig = E.y[i0 + 2 * EM];
  E.ys[i0] = psi; E.ys[i0 + EM] = tau; E.ys[i0 + 2 * EM] = sig;
  double v, wv;
  slip_rate_w(E.vref, psi, tau, sig, E.a[r], &v, &wv);
  E.vs[(int64_t)r * EM + m] = v;
  E.ws[(int64_t)r * EM + m] = wv;
  E.x0[(int64_t)r * EM + m] = (float)(E.backslip ? (v + 0.0) - E.vpl[r] : v + 0.0);
}

#define E_SAFETY ((double)0.9f)
#define E_PGROW ((double)-0.2f)
#define E_PSHRNK (-0.25)
#define E_TINY ((double)1e-20f)

// per member: rkqs (main_LH.f90:2296-2360) on the member's own errmax
__global__ void control_e_kernel(EnsDev E) {
  const int m = threadIdx.x;
  __shared__ int nd;
  if (m == 0) nd = 0;
  __syncthreads();
  if (m < EM) {
    int acc = 0;
    if (!E.done[m] && !E.failed[m]) {
      double e = __longlong_as_double((long long)E.emax[m]);
      if (E.huge[m] && e < 10.0) e = 10.0;
      const double h = E.h[m];
      if (e < 1.0 && e > E_TINY) {
        double hn = fmin(2 * h, E_SAFETY * h * pow(e, E_PGROW));
        hn = fmin(hn, E.dtmax);
        const double xn = E.x[m] + h;
        E.hdid[m] = h;
        acc = 1;
        if (xn >= E.tlim[m] || E.tlim[m] - xn <= 0.0) {
          E.x[m] = E.tlim[m];
          E.done[m] = 1;
          E.h[m] = 0.0;
        } else {
          E.x[m] = xn;
          E.h[m] = fmin(hn, E.tlim[m] - xn);
        }
      } else {
        double hs = (e > E_TINY) ? fmax(0.5 * h, E_SAFETY * h * pow(e, E_PSHRNK)) : 0.5 * h;
        if (E.x[m] + hs - E.x[m] < 1.e-15) {
          E.failed[m] = 1;
          E.h[m] = 0.0;
        } else {
          E.h[m] = hs;
        }
        atomicAdd((unsigned long long*)&E.counters[1], 1ull);
      }
    }
    E.accepted[m] = acc;
    if (acc) atomicAdd((unsigned long long*)&E.counters[0], 1ull);
    if (E.done[m] || E.failed[m]) atomicAdd(&nd, 1);
  }
  __syncthreads();
  if (m == 0) {
    *(volatile int*)E.ndone = nd;
    __threadfence_system();
  }
}

// accepted members: y <- yout, slip and slip rate (main_LH.f90:1266-1287)
__global__ void update_e_kernel(EnsDev E) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int m = (int)(idx % EM);
  const int r = (int)(idx / EM);
  if (r >= E.n || !E.accepted[m]) return;
  const int64_t i0 = (3LL * r) * EM + m;
  const double psi = E.yout[i0], tau = E.yout[i0 + EM], sig = E.yout[i0 + 2 * EM];
  E.y[i0] = psi; E.y[i0 + EM] = tau; E.y[i0 + 2 * EM] = sig;
  const double dt = E.hdid[m];
  const int64_t j = (int64_t)r * EM + m;
  double s = E.slip[j] + (E.vel[j] + 0.0) * dt * 0.5;
  const double v = slip_rate(E.vref, psi, tau, sig, E.a[r]);
  s = s + (v + 0.0) * dt * 0.5;
  E.slip[j] = s;
  E.vel[j] = v;
}

size_t smem1() { return 2 * (size_t)kXT + 2 * (size_t)kChunk + 64; }
size_t smem2() { return 2 * (size_t)(kChunk + kBrows) + 8 * 16 * EM * 4 + 64; }

// y (element, member) = the group sums of one product, both matrices
__global__ void __launch_bounds__(256) ens_sum_kernel(EnsMat A, EnsMat B, int nmat, int n, float* __restrict__ ys,
                                                      float* __restrict__ yn) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= (int64_t)n * EM) return;
  const int m = (int)(idx % EM), r = (int)(idx / EM);
  ys[idx] = group_sum_raw(A, r, m);
  if (nmat == 2) yn[idx] = group_sum_raw(B, r, m);
}

}  // namespace
}  // namespace hbi

using namespace hbi;

struct hbi_ens_s {
  EnsDev E{};
  EnsMat M[2]{};
  TcMat T[2]{};
  bool tc = false;
  int nmat = 1, n = 0, sm = 152;
  int64_t ncnt_m[2] = {0, 0}, ncnt_t[2] = {0, 0};  // arrival counters of M[k] and T[k]
  std::vector<void*> allocs;
  int* hnd = nullptr;  // host-mapped done count
  cudaStream_t st = nullptr;
  cudaGraphExec_t g = nullptr;
};

namespace {

int efail(int code, const char* msg) { return set_error(code, msg); }

template <class T>
T* ealloc(hbi_ens* e, size_t n, bool zero = true) {
  void* p = nullptr;
  if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return nullptr;
  if (zero) cudaMemset(p, 0, std::max<size_t>(n, 1) * sizeof(T));
  e->allocs.push_back(p);
  return (T*)p;
}

void enqueue_e(hbi_ens* e) {
  const EnsDev& E = e->E;
  const int64_t tot = (int64_t)E.n * EM;
  const int blocks = (int)((tot + 255) / 256);
  cudaStream_t st = e->st;
  const int g1 = e->sm * 2;
  prepare_e_kernel<<<blocks, 256, 0, st>>>(E);
  for (int s = 0; s < 6; s++) {
    const float* xin = s == 0 ? E.x0 : E.xb[s & 1];
    float* xout = E.xb[(s + 1) & 1];
    if (e->tc) {
      launch_tc(1, e->T[0], e->T[e->nmat - 1], e->nmat, xin, st);
      launch_tc(2, e->T[0], e->T[e->nmat - 1], e->nmat, xin, st);
    } else {
      p1e_kernel<<<g1, 256, smem1(), st>>>(e->M[0], e->M[e->nmat - 1], e->nmat, xin);
      p2e_kernel<<<g1, 256, smem2(), st>>>(e->M[0], e->M[e->nmat - 1], e->nmat, xin);
    }
    p3e_kernel<<<blocks, 256, 0, st>>>(e->M[0], e->M[e->nmat - 1], E, s, xout);
  }
  control_e_kernel<<<1, EM, 0, st>>>(E);
  update_e_kernel<<<blocks, 256, 0, st>>>(E);
}

}  // namespace

namespace {
int recapture(hbi_ens* e);
}

extern "C" int hbi_ens_free(hbi_ens* e) {
  if (!e) return HBI_OK;
  if (e->st) cudaStreamSynchronize(e->st);
  if (e->g) cudaGraphExecDestroy(e->g);
  for (void* p : e->allocs) cudaFree(p);
  if (e->hnd) cudaFreeHost(e->hnd);
  if (e->st) cudaStreamDestroy(e->st);
  delete e;
  return HBI_OK;
}

extern "C" int hbi_ens_create(hbi_ens** out, const hbi_rsf_params* p, hbi_lhp* ls, hbi_lhp* ln, int members,
                              const double* b, const double* dc) {
  if (!out || !p || !ls || !b || !dc) return efail(HBI_ERR_ARG, "hbi_ens_create: null argument");
  if (members != EM) return efail(HBI_ERR_ARG, "hbi_ens_create: the ensemble kernels take exactly 64 members");
  LhpView vs{}, vn{};
  int rc = lhp_view(ls, &vs);
  if (rc) return rc;
  if (ln && (rc = lhp_view(ln, &vn))) return rc;
  if (vs.storage != ST_F32 || (ln && vn.storage != ST_F32))
    return efail(HBI_ERR_ARG, "hbi_ens_create: the ensemble product needs HBI_STORE_F32 operators");
  if (p->ncell != vs.n || (ln && vn.n != vs.n)) return efail(HBI_ERR_ARG, "hbi_ens_create: size mismatch");
  hbi_ens* e = new hbi_ens_s();
  e->n = vs.n;
  e->nmat = ln ? 2 : 1;
  e->sm = vs.sm;
  if (cudaStreamCreateWithFlags(&e->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaHostAlloc(&e->hnd, sizeof(int), cudaHostAllocMapped) != cudaSuccess) {
    hbi_ens_free(e);
    return efail(HBI_ERR_CUDA, "hbi_ens_create: stream");
  }
  *e->hnd = 0;
  const int n = e->n;
  const size_t nm = (size_t)n * EM;
  EnsDev& E = e->E;
  E.n = n;
  E.nmat = e->nmat;
  E.evlaw = p->evlaw;
  E.backslip = p->backslip;
  E.limitsigma = p->limitsigma;
  E.vref = p->vref;
  E.minsig = p->minsig;
  E.maxsig = p->maxsig;
  E.rigid_over_2vs = 0.5 * 32.04 / 3.464;
  bool ok = true;
  auto up = [&](const double* h, size_t cnt) -> const double* {
    double* d = ealloc<double>(e, cnt, false);
    if (!d || cudaMemcpy(d, h, sizeof(double) * cnt, cudaMemcpyHostToDevice) != cudaSuccess) ok = false;
    return d;
  };
  E.a = up(p->a, n);
  E.f0 = up(p->f0, n);
  E.taudot = up(p->taudot, n);
  E.sigdot = up(p->sigdot, n);
  E.vpl = up(p->vpl, n);
  E.b = up(b, nm);
  E.dc = up(dc, nm);
  E.y = ealloc<double>(e, 3 * nm);
  E.ys = ealloc<double>(e, 3 * nm);
  E.vs = ealloc<double>(e, nm);
  E.ws = ealloc<double>(e, nm);
  E.K = ealloc<double>(e, 18 * nm);
  E.yout = ealloc<double>(e, 3 * nm);
  E.vel = ealloc<double>(e, nm);
  E.slip = ealloc<double>(e, nm);
  E.x0 = ealloc<float>(e, nm);
  E.xb[0] = ealloc<float>(e, nm);
  E.xb[1] = ealloc<float>(e, nm);
  E.h = ealloc<double>(e, EM);
  E.x = ealloc<double>(e, EM);
  E.hdid = ealloc<double>(e, EM);
  E.tlim = ealloc<double>(e, EM);
  E.accepted = ealloc<int>(e, EM);
  E.done = ealloc<int>(e, EM);
  E.failed = ealloc<int>(e, EM);
  E.nr = ealloc<int>(e, EM);
  E.emax = ealloc<unsigned long long>(e, EM);
  E.huge = ealloc<int>(e, EM);
  E.counters = ealloc<long long>(e, 4);
  if (cudaHostGetDevicePointer((void**)&E.ndone, e->hnd, 0) != cudaSuccess) ok = false;
  for (int k = 0; k < e->nmat; k++) {
    const LhpView& v = k ? vn : vs;
    EnsMat& M = e->M[k];
    M.m = v.md;
    M.m.scale = k ? p->scale_n : p->scale_s;
    M.z = ealloc<float>(e, (size_t)v.zlen * EM);
    M.part = ealloc<float>(e, (size_t)v.plen1 * EM);
    M.cnt = ealloc<int>(e, (size_t)v.ncg);
    e->ncnt_m[k] = v.ncg;
    M.gpart = ealloc<float>(e, (size_t)v.plen2 * EM);
    if (!M.z || !M.part || !M.cnt || !M.gpart) ok = false;
  }
  for (void* q : {(void*)E.y, (void*)E.K, (void*)E.yout, (void*)E.xb[1], (void*)E.counters})
    if (!q) ok = false;
  if (!ok) {
    hbi_ens_free(e);
    return efail(HBI_ERR_NOMEM, "hbi_ens_create: allocation");
  }
  // the Cash-Karp tableau (main_LH.f90:2490-2496, default-real literals)
  double Bt[15] = {.2, (double)(3.f / 40.f), (double)(9.f / 40.f), (double).3f, (double)-.9f, (double)1.2f,
                   (double)(-(11.f / 54.f)), 2.5, (double)(-(70.f / 27.f)), (double)(35.f / 27.f),
                   (double)(1631.f / 55296.f), (double)(175.f / 512.f), (double)(575.f / 13824.f),
                   (double)(44275.f / 110592.f), (double)(253.f / 4096.f)};
  const double C1 = (double)(37.f / 378.f), C3 = (double)(250.f / 621.f), C4 = (double)(125.f / 594.f),
               C6 = (double)(512.f / 1771.f);
  double Ct[6] = {C1, 0, C3, C4, 0, C6};
  double Dt[6] = {C1 - (double)(2825.f / 27648.f), 0, C3 - (double)(18575.f / 48384.f),
                  C4 - (double)(13525.f / 55296.f), (double)(-(277.f / 14336.f)), C6 - (double).25f};
  if (cudaMemcpyToSymbol(eB, Bt, sizeof Bt) != cudaSuccess || cudaMemcpyToSymbol(eC, Ct, sizeof Ct) != cudaSuccess ||
      cudaMemcpyToSymbol(eDC, Dt, sizeof Dt) != cudaSuccess ||
      cudaFuncSetAttribute(p1e_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1()) != cudaSuccess ||
      cudaFuncSetAttribute(p2e_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2()) != cudaSuccess) {
    hbi_ens_free(e);
    return efail(HBI_ERR_CUDA, "hbi_ens_create: kernel setup");
  }
  cudaGraph_t g;
  if (cudaStreamBeginCapture(e->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    hbi_ens_free(e);
    return efail(HBI_ERR_CUDA, "hbi_ens_create: capture");
  }
  enqueue_e(e);
  if (cudaStreamEndCapture(e->st, &g) != cudaSuccess || cudaGraphInstantiate(&e->g, g, 0) != cudaSuccess) {
    hbi_ens_free(e);
    return efail(HBI_ERR_CUDA, "hbi_ens_create: graph");
  }
  cudaGraphDestroy(g);
  *out = e;
  return HBI_OK;
}

extern "C" int hbi_ens_set_state(hbi_ens* e, const double* y, const double* vel) {
  if (!e || !y || !vel) return efail(HBI_ERR_ARG, "null");
  const size_t nm = (size_t)e->n * EM;
  if (cudaMemcpy(e->E.y, y, sizeof(double) * 3 * nm, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(e->E.vel, vel, sizeof(double) * nm, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(e->E.slip, 0, sizeof(double) * nm) != cudaSuccess)
    return efail(HBI_ERR_CUDA, "hbi_ens_set_state");
  return HBI_OK;
}

extern "C" int hbi_ens_get_state(hbi_ens* e, double* y, double* slip, double* x) {
  if (!e) return efail(HBI_ERR_ARG, "null");
  const size_t nm = (size_t)e->n * EM;
  cudaStreamSynchronize(e->st);
  if ((y && cudaMemcpy(y, e->E.y, sizeof(double) * 3 * nm, cudaMemcpyDeviceToHost) != cudaSuccess) ||
      (slip && cudaMemcpy(slip, e->E.slip, sizeof(double) * nm, cudaMemcpyDeviceToHost) != cudaSuccess) ||
      (x && cudaMemcpy(x, e->E.x, sizeof(double) * EM, cudaMemcpyDeviceToHost) != cudaSuccess))
    return efail(HBI_ERR_CUDA, "hbi_ens_get_state");
  return HBI_OK;
}

namespace {
// a product kernel that gave up a bulk-copy wait invalidates the results;
// the operators' and the ensemble's arrival counters start over
int ens_check_device(hbi_ens* e, const char* who) {
  bool bad = false;
  for (int k = 0; k < e->nmat; k++) {
    const int t = take_device_error(e->M[k].m);
    if (t < 0) return efail(HBI_ERR_CUDA, who);
    if (t > 0) {
      bad = true;
      if (cudaMemset(e->M[k].cnt, 0, sizeof(int) * (size_t)std::max<int64_t>(e->ncnt_m[k], 1)) != cudaSuccess ||
          (e->T[k].cnt &&
           cudaMemset(e->T[k].cnt, 0, sizeof(int) * (size_t)std::max<int64_t>(e->ncnt_t[k], 1)) != cudaSuccess))
        return efail(HBI_ERR_CUDA, who);
    }
  }
  if (bad) return efail(HBI_ERR_DEVICE, "a product kernel gave up waiting for a bulk copy; the results are invalid");
  return HBI_OK;
}
}  // namespace

extern "C" int hbi_ens_run(hbi_ens* e, double eps_r, double dtinit, double dtmax, double t_limit,
                           hbi_ens_status* out) {
  if (!e || !(eps_r > 0) || !(dtinit > 0) || !(t_limit > 0)) return efail(HBI_ERR_ARG, "hbi_ens_run: arguments");
  // the run's constants live in the captured kernels' EnsDev: eps and dtmax
  // are read from device memory through these per-member arrays instead
  std::vector<double> h(EM, std::min(dtinit, t_limit)), x(EM, 0.0), tl(EM, t_limit);
  std::vector<int> z(EM, 0);
  std::vector<long long> c(4, 0);
  if (e->E.eps != eps_r || e->E.dtmax != dtmax) {
    // re-capture with the new constants
    e->E.eps = eps_r;
    e->E.dtmax = dtmax;
    int rc = recapture(e);
    if (rc) return rc;
  }
  if (cudaMemcpy(e->E.h, h.data(), sizeof(double) * EM, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(e->E.x, x.data(), sizeof(double) * EM, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(e->E.tlim, tl.data(), sizeof(double) * EM, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(e->E.done, z.data(), sizeof(int) * EM, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(e->E.failed, z.data(), sizeof(int) * EM, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(e->E.counters, c.data(), sizeof(long long) * 4, cudaMemcpyHostToDevice) != cudaSuccess)
    return efail(HBI_ERR_CUDA, "hbi_ens_run: upload");
  *e->hnd = 0;
  const auto t0 = std::chrono::steady_clock::now();
  long long attempts = 0;
  const int batch = 8;
  for (;;) {
    for (int i = 0; i < batch; i++)
      if (cudaGraphLaunch(e->g, e->st) != cudaSuccess) return efail(HBI_ERR_CUDA, "hbi_ens_run: launch");
    attempts += batch;
    if (cudaStreamSynchronize(e->st) != cudaSuccess) return efail(HBI_ERR_CUDA, "hbi_ens_run: execution");
    if (*(volatile int*)e->hnd >= EM) break;
    if (attempts >= (1LL << 17)) break;  // members still running are reported as not done
  }
  const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::vector<int> fl(EM), dn(EM);
  cudaMemcpy(c.data(), e->E.counters, sizeof(long long) * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(fl.data(), e->E.failed, sizeof(int) * EM, cudaMemcpyDeviceToHost);
  cudaMemcpy(dn.data(), e->E.done, sizeof(int) * EM, cudaMemcpyDeviceToHost);
  if (out) {
    out->attempts = attempts;
    out->steps = c[0];
    out->rejected = c[1];
    out->done = 0;
    out->failed = 0;
    for (int m = 0; m < EM; m++) {
      out->done += dn[m];
      out->failed += fl[m];
    }
    out->wall_s = wall;
  }
  return ens_check_device(e, "hbi_ens_run");
}

extern "C" int hbi_ens_product(hbi_ens* e, const float* x, float* ys, float* yn, int reps, double* ms) {
  if (!e || !x || !ys || (e->nmat == 2 && !yn) || reps < 0)
    return efail(HBI_ERR_ARG, "hbi_ens_product: bad arguments");
  const int64_t tot = (int64_t)e->n * EM;
  const size_t bytes = (size_t)tot * sizeof(float);
  float *dys = nullptr, *dyn = nullptr;
  if (cudaMalloc(&dys, bytes) != cudaSuccess || cudaMalloc(&dyn, bytes) != cudaSuccess) {
    cudaFree(dys);
    return efail(HBI_ERR_NOMEM, "hbi_ens_product: output buffers");
  }
  cudaStream_t st = e->st;
  const int blocks = (int)((tot + 255) / 256);
  auto once = [&]() {
    if (e->tc) {
      launch_tc(1, e->T[0], e->T[e->nmat - 1], e->nmat, e->E.x0, st);
      launch_tc(2, e->T[0], e->T[e->nmat - 1], e->nmat, e->E.x0, st);
    } else {
      p1e_kernel<<<e->sm * 2, 256, smem1(), st>>>(e->M[0], e->M[e->nmat - 1], e->nmat, e->E.x0);
      p2e_kernel<<<e->sm * 2, 256, smem2(), st>>>(e->M[0], e->M[e->nmat - 1], e->nmat, e->E.x0);
    }
    ens_sum_kernel<<<blocks, 256, 0, st>>>(e->M[0], e->M[e->nmat - 1], e->nmat, e->n, dys, dyn);
  };
  int rc = HBI_OK;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaMemcpyAsync(e->E.x0, x, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess) rc = HBI_ERR_CUDA;
  if (rc == HBI_OK) {
    once();
    if (reps > 0) {
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      cudaEventRecord(e0, st);
      for (int r = 0; r < reps; r++) once();
      cudaEventRecord(e1, st);
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) rc = HBI_ERR_CUDA;
  }
  if (rc == HBI_OK && reps > 0 && ms) {
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    *ms = (double)t / reps;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (rc == HBI_OK && (cudaMemcpy(ys, dys, bytes, cudaMemcpyDeviceToHost) != cudaSuccess ||
                       (e->nmat == 2 && cudaMemcpy(yn, dyn, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)))
    rc = HBI_ERR_CUDA;
  cudaFree(dys);
  cudaFree(dyn);
  if (rc != HBI_OK) return efail(rc, "hbi_ens_product: CUDA");
  return ens_check_device(e, "hbi_ens_product");
}

namespace {
int recapture(hbi_ens* e) {
  if (e->g) cudaGraphExecDestroy(e->g);
  e->g = nullptr;
  cudaGraph_t g;
  if (cudaStreamBeginCapture(e->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return efail(HBI_ERR_CUDA, "capture");
  enqueue_e(e);
  if (cudaStreamEndCapture(e->st, &g) != cudaSuccess || cudaGraphInstantiate(&e->g, g, 0) != cudaSuccess)
    return efail(HBI_ERR_CUDA, "graph");
  cudaGraphDestroy(g);
  return HBI_OK;
}
}  // namespace

extern "C" int hbi_ens_use_tensor_cores(hbi_ens* e, const hbi_leafmtxp* lf_s, const hbi_leafmtxp* lf_n) {
  if (!e || !lf_s || (e->nmat == 2 && !lf_n)) return efail(HBI_ERR_ARG, "hbi_ens_use_tensor_cores: null");
  TcPlan tcp[2];
  for (int k = 0; k < e->nmat; k++) {
    const double* body = nullptr;
    std::vector<int64_t> off;
    std::vector<Leaf> leaves;
    int rc = leaf_view(k ? lf_n : lf_s, &body, &off, &leaves);
    if (rc) return rc;
    TcPlan& P = tcp[k];
    plan_tc(e->n, leaves, off, P);
    TcMat& T = e->T[k];
    auto upload = [&](const void* h, size_t bytes) -> void* {
      void* d = nullptr;
      if (cudaMalloc(&d, std::max<size_t>(bytes, 16)) != cudaSuccess) return nullptr;
      e->allocs.push_back(d);
      if (bytes && cudaMemcpy(d, h, bytes, cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
      return d;
    };
    T.p1 = (const TcItem*)upload(P.p1.data(), P.p1.size() * sizeof(TcItem));
    T.n1 = (int)P.p1.size();
    T.p2 = (const TcItem*)upload(P.p2.data(), P.p2.size() * sizeof(TcItem));
    T.n2 = (int)P.p2.size();
    T.midx = (const int32_t*)upload(P.midx.data(), P.midx.size() * sizeof(int32_t));
    __nv_bfloat16* s1 = ealloc<__nv_bfloat16>(e, (size_t)P.store1);
    __nv_bfloat16* s2 = ealloc<__nv_bfloat16>(e, (size_t)P.store2);
    T.s1 = s1;
    T.s2 = s2;
    T.z = ealloc<float>(e, (size_t)P.zlen * EM);
    T.part = ealloc<float>(e, (size_t)P.plen1 * EM);
    T.cnt = ealloc<int>(e, (size_t)P.ncg);
    e->ncnt_t[k] = P.ncg;
    T.gpart = e->M[k].gpart;
    T.err = e->M[k].m.err;
    T.wait = e->M[k].m.wait;
    if (!T.p1 || !T.p2 || !T.midx || !s1 || !s2 || !T.z || !T.part || !T.cnt)
      return efail(HBI_ERR_NOMEM, "hbi_ens_use_tensor_cores: allocation");
    for (int ph = 1; ph <= 2; ph++) {
      const std::vector<TcCopy>& map = ph == 1 ? P.copy1 : P.copy2;
      TcCopy* dm = (TcCopy*)upload(map.data(), map.size() * sizeof(TcCopy));
      if (!dm) return efail(HBI_ERR_NOMEM, "hbi_ens_use_tensor_cores: conversion map");
      launch_tcconv(body, dm, (int64_t)map.size(), ph == 1 ? s1 : s2, e->st);
      if (cudaStreamSynchronize(e->st) != cudaSuccess) return efail(HBI_ERR_CUDA, "hbi_ens_use_tensor_cores: convert");
      cudaFree(dm);
      e->allocs.pop_back();
    }
  }
  // both matrices' items dealt over the SMs, longest first (cost = factor
  // bytes + a fixed cost per item for its epilogue)
  for (int ph = 1; ph <= 2; ph++) {
    std::vector<int64_t> cost;
    for (int k = 0; k < e->nmat; k++) {
      const int cnt = ph == 1 ? e->T[k].n1 : e->T[k].n2;
      const std::vector<TcItem>& items = ph == 1 ? tcp[k].p1 : tcp[k].p2;
      for (int i = 0; i < cnt; i++) cost.push_back((int64_t)items[i].np * items[i].kp * 4 + 64 * 1024);
    }
    std::vector<int32_t> woff, witem;
    plan_warp_schedule(cost, e->sm, woff, witem);
    int32_t* doff = ealloc<int32_t>(e, woff.size(), false);
    int32_t* ditem = ealloc<int32_t>(e, std::max<size_t>(witem.size(), 1), false);
    if (!doff || !ditem) return efail(HBI_ERR_NOMEM, "hbi_ens_use_tensor_cores: schedule");
    cudaMemcpy(doff, woff.data(), woff.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
    if (!witem.empty()) cudaMemcpy(ditem, witem.data(), witem.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
    e->T[0].boff[ph - 1] = doff;
    e->T[0].bitem[ph - 1] = ditem;
  }
  e->T[0].G = e->sm;
  tc_prepare();
  e->tc = true;
  return recapture(e);
}
