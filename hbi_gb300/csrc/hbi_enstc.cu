// hbi_enstc.cu -- the ensemble's multi-vector product on the 5th-generation
// tensor cores (tcgen05).
//
// Each contraction is D^T (N x 64 members) = F (N x K) * A (K x 64), F the
// factor tile (plan_tc, hbi_structure.cpp) on the MMA's M side (128 rows per
// MMA) and the members on its N side (N = 64):
//   phase 1: N = the columns of a column group (z = V^T x), K = a tile's rows
//            (up to 1,024), A = the tile's rows of X (64 members);
//   phase 2: N = the rows of a row-group tile, K = the group's columns,
//            A = the columns' multipliers (rows of z or X).
// F is stored as BF16 hi + lo halves in the canonical no-swizzle K-major
// layout and arrives by cp.async.bulk (TMA) in stages of 32 K; the FP32 rows
// of A arrive with it and are split into BF16 hi + lo in the canonical layout
// by a converter warpgroup.  Accumulation is FP32 in tensor memory; the
// kernel's roles and their hand-offs are described at tc_kernel.
//
// Every wait is bounded (about a second of SM clock); on a time-out the
// operator's error word is set, every role leaves its loop, the block waits
// (bounded) for its copies and MMAs and releases its tensor memory.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "hbi_enstc.cuh"
#include "hbi_kernels.cuh"
#include "hbi_umma.cuh"

namespace hbi {

namespace {

constexpr int EMT = 64;
constexpr int KC = 32;                       // K per stage: two 16-K MMA chunks
constexpr int NST = 4;                       // stages
constexpr int kFac = (KC / 16) * 256 * 64;   // factor hi + lo of a stage, N <= 256: 32 KB
constexpr int kRows = KC * EMT * 4;          // the members' FP32 rows: 8 KB
constexpr int kMem = (KC / 16) * 4096;       // the members' operand, hi + lo: 8 KB
constexpr int kStage = kFac + kRows + kMem;  // 48 KB
constexpr int kThreads = 352;                // producer, MMA, 4 converter, 4 epilogue warps, producer
constexpr uint32_t kTmemCols = 256;          // two accumulators x two 128-row blocks x 64 members
constexpr long long kWaitT = 2LL << 30;

struct Bars {
  uint64_t full[NST];   // a stage's copies landed (producer's expect_tx)
  uint64_t conv[NST];   // the stage's member operand is written (128 converter threads)
  uint64_t empty[NST];  // the stage's MMAs are done (tcgen05.commit)
  uint64_t accf[2];     // an accumulator holds a finished item (tcgen05.commit)
  uint64_t acce[2];     // an accumulator was read back (128 epilogue threads)
  uint64_t done;        // every MMA of the block is done (exit)
  int abort;            // a role gave up waiting: every role leaves its loop
  int flag;             // epilogue broadcast
  uint32_t tslot;       // tensor-memory address
};

__device__ __forceinline__ uint32_t sa(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void binit(uint64_t* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sa(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void bexpect(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sa(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void barrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(sa(b)) : "memory");
}
__device__ __forceinline__ bool btry(uint64_t* b, uint32_t par) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(sa(b)), "r"(par)
      : "memory");
  return ok != 0;
}
// bounded wait, regardless of the abort flag (a block's own copies and MMAs
// before it leaves)
__device__ __forceinline__ bool bwait(uint64_t* b, uint32_t par) {
  const long long t0 = clock64();
  while (!btry(b, par))
    if (clock64() - t0 > kWaitT) return false;
  return true;
}
// bounded wait of a role: gives up when another role did, or after `limit`
// cycles (then records the error and tells the other roles); a limit of 0 is
// spent before the first probe (the error path on demand)
__device__ __forceinline__ bool rwait(uint64_t* b, uint32_t par, Bars* br, int* err, long long limit) {
  const long long t0 = clock64();
  while (limit <= 0 || !btry(b, par)) {
    if (*(volatile int*)&br->abort) return false;
    if (limit <= 0 || clock64() - t0 > limit) {
      *(volatile int*)&br->abort = 1;
      if (err) atomicExch(err, 1);
      return false;
    }
  }
  return true;
}
__device__ __forceinline__ void bcopy(void* dst, const void* src, uint32_t bytes, uint64_t* b) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   sa(dst)),
               "l"(src), "r"(bytes), "r"(sa(b))
               : "memory");
}
// factor chunks are read once per product: evicted first from L2, so that
// z, X and the schedules stay resident
__device__ __forceinline__ void bcopy_stream(void* dst, const void* src, uint32_t bytes, uint64_t* b) {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
          sa(dst)),
      "l"(src), "r"(bytes), "r"(sa(b)), "l"(pol)
      : "memory");
}
__device__ __forceinline__ void fasync() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void group_sync() { asm volatile("bar.sync 1, 128;" ::: "memory"); }
__device__ __forceinline__ int arrive_ar(int* p) {
  int old;
  asm volatile("atom.add.acq_rel.gpu.s32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
  return old;
}

// One block per SM, four roles working on a ring of NST stages:
//   warps 0, 10   producers, taking the stages in turn: bulk copies of the
//                 factor tile's chunks (BF16 hi and lo halves, canonical
//                 K-major) and of the members' FP32 rows (phase 1: rows
//                 m0 + k of X; phase 2: the multiplier rows of z or X, one
//                 copy per run of consecutive rows);
//   warps 2-5     converters: the FP32 rows to BF16 hi / lo in the canonical
//                 K-major layout of the MMA's B operand (member, k);
//   warp 1        MMA: one thread issues, per 16-K chunk and 128-row block of
//                 the item, D += F_hi M_hi + F_hi M_lo + F_lo M_hi (M = 128
//                 factor rows, N = 64 members, K = 16; the lo x lo term is
//                 below FP32 resolution) into one of two tensor-memory
//                 accumulators, and commits each stage back to its producer;
//   warps 6-9     epilogue: read a finished accumulator (tcgen05.ld, one
//                 thread per factor row, 64 members) and write the item's
//                 rows, while the MMAs of the next item run in the other
//                 accumulator.
// PH = 1: z = V^T x (factor rows = the columns of a column group, K = the
// rows of a tile); PH = 2: partial row sums U z + A x (factor rows = the rows
// of a row-group tile, K = the group's columns).
template <int PH>
__global__ void __launch_bounds__(kThreads, 1) tc_kernel(TcMat A, TcMat B, int nmat, const float* __restrict__ X) {
  extern __shared__ __align__(1024) unsigned char sm[];
  Bars* br = reinterpret_cast<Bars*>(sm + NST * kStage);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int s = 0; s < NST; s++) {
      binit(&br->full[s], 1);
      binit(&br->conv[s], 128);
      binit(&br->empty[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      binit(&br->accf[b], 1);
      binit(&br->acce[b], 128);
    }
    binit(&br->done, 1);
    br->abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) umma::tmem_alloc(&br->tslot, kTmemCols);
  umma::fence_before();
  __syncthreads();
  umma::fence_after();
  const uint32_t tbase = br->tslot;
  const int n0 = PH == 1 ? A.n1 : A.n2;
  const int ntot = nmat == 2 ? n0 + (PH == 1 ? B.n1 : B.n2) : n0;
  // this block's items
  const int32_t* lst = nullptr;
  int nit;
  if (A.boff[PH - 1] && A.G == (int)gridDim.x) {
    const int o0 = __ldg(&A.boff[PH - 1][blockIdx.x]);
    nit = __ldg(&A.boff[PH - 1][blockIdx.x + 1]) - o0;
    lst = A.bitem[PH - 1] + o0;
  } else {
    nit = (int)blockIdx.x < ntot ? (ntot - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  }
  auto item_at = [&](int j) -> int { return lst ? __ldg(&lst[j]) : (int)blockIdx.x + j * (int)gridDim.x; };
  auto desc = [&](int it) -> TcItem {
    return PH == 1 ? (it < n0 ? A.p1[it] : B.p1[it - n0]) : (it < n0 ? A.p2[it] : B.p2[it - n0]);
  };
  auto stage = [&](int s) -> unsigned char* { return sm + s * kStage; };
  // every role walks the block's items in order; item ids are loaded two
  // items ahead and descriptors one, so that no role waits on a descriptor
  // load at an item boundary
  struct Walk {
    int j, it, itn, itnn;
    TcItem D, Dn;
  };
  auto walk_init = [&](Walk& w) {
    w.j = 0;
    w.it = nit > 0 ? item_at(0) : 0;
    w.itn = nit > 1 ? item_at(1) : 0;
    w.itnn = nit > 2 ? item_at(2) : 0;
    w.D = nit > 0 ? desc(w.it) : TcItem{};
    w.Dn = nit > 1 ? desc(w.itn) : TcItem{};
  };
  auto walk_next = [&](Walk& w) {
    w.j++;
    w.it = w.itn;
    w.D = w.Dn;
    w.itn = w.itnn;
    w.Dn = w.j + 1 < nit ? desc(w.itn) : TcItem{};
    w.itnn = w.j + 2 < nit ? item_at(w.j + 2) : 0;
  };

  if (warp == 0 || warp == 10) {
    // --------------------------------------------------------- producers
    // two producer warps take the stages in turn (stage q: producer q mod
    // 2); issuing a stage's copies costs a warp about a thousand cycles
    const int pi = warp == 0 ? 0 : 1;
    Walk W;
    walk_init(W);
    int q = 0, k0 = 0;
    // phase 2: this stage's column indices
    auto load_midx = [&]() -> int {
      const int nrow = max(0, min(KC, W.D.kv - k0));
      const TcMat& M = W.it < n0 ? A : B;
      return (PH == 2 && W.j < nit && lane < nrow) ? __ldg(&M.midx[W.D.m0 + k0 + lane]) : 0;
    };
    int mi = pi == 0 ? load_midx() : 0;
    while (W.j < nit) {
      const TcItem& D = W.D;
      const TcMat& M = W.it < n0 ? A : B;
      const int s = q % NST;
      if ((q & 1) != pi) {
        // the other producer's stage: only the walk advances
        q++;
        k0 += KC;
        if (k0 >= D.kp) {
          k0 = 0;
          walk_next(W);
        }
        if ((q & 1) == pi) mi = load_midx();
        continue;
      }
      int w = 1;
      if (q >= NST && lane == 0) w = rwait(&br->empty[s], (uint32_t)((q / NST - 1) & 1), br, A.err, A.wait);
      if (!__shfl_sync(0xffffffffu, w, 0)) break;
      const int kc = min(KC, D.kp - k0);
      const int nrow = max(0, min(kc, D.kv - k0));  // member rows that carry data
      unsigned char* stg = stage(s);
      const uint32_t fbytes = (uint32_t)((kc / 16) * D.np * 64);
      const __nv_bfloat16* fsrc = (PH == 1 ? M.s1 : M.s2) + D.soff + (int64_t)(k0 / 16) * D.np * 32;
      // no proxy fence before the copies: the factor region was last read by
      // the MMAs (the same async proxy, ordered by the empty barrier) and the
      // rows region by the converters, whose loads were consumed before they
      // arrived
      if (lane == 0) {
        bexpect(&br->full[s], fbytes + (uint32_t)(nrow * EMT * 4));
        bcopy_stream(stg, fsrc, fbytes, &br->full[s]);
        if (PH == 1 && nrow > 0)
          bcopy(stg + kFac, X + (int64_t)(D.m0 + k0) * EMT, (uint32_t)(nrow * EMT * 4), &br->full[s]);
      }
      __syncwarp();
      if (PH == 2) {
        // runs of consecutive multiplier rows (a low-rank leaf's z columns,
        // a dense leaf's x rows) go in one copy, issued by the run's first lane
        const int prev = __shfl_up_sync(0xffffffffu, mi, 1);
        const bool cont = lane > 0 && lane < nrow &&
                          ((mi >= 0 && prev >= 0 && mi == prev + 1) || (mi < 0 && prev < 0 && mi == prev - 1));
        const bool head = lane < nrow && !cont;
        const unsigned heads = __ballot_sync(0xffffffffu, head);
        if (head) {
          const unsigned above = heads & ~((2u << lane) - 1u);
          const int len = (above ? __ffs(above) - 1 : nrow) - lane;
          const float* src = mi >= 0 ? M.z + (int64_t)mi * EMT : X + (int64_t)(-mi - 1) * EMT;
          bcopy(stg + kFac + lane * EMT * 4, src, (uint32_t)(len * EMT * 4), &br->full[s]);
        }
      }
      q++;
      k0 += KC;
      if (k0 >= D.kp) {
        k0 = 0;
        walk_next(W);
      }
      if ((q & 1) == pi) mi = load_midx();
    }
    // this producer's copies still in flight land before the block leaves
    // (the last NST stages are the only ones whose phase can still be open)
    if (lane == 0)
      for (int r = max(0, q - NST); r < q; r++)
        if ((r & 1) == pi) bwait(&br->full[r % NST], (uint32_t)((r / NST) & 1));
    __syncwarp();
  } else if (warp == 1) {
    // --------------------------------------------------------------- MMA
    const uint32_t idesc = umma::idesc_bf16_f32(128, EMT);
    int q = 0;
    Walk W;
    walk_init(W);
    for (; W.j < nit; walk_next(W)) {
      const int j = W.j;
      const int b = j & 1;
      const TcItem& D = W.D;
      int w = 1;
      if (j >= 2 && lane == 0) w = rwait(&br->acce[b], (uint32_t)((j / 2 - 1) & 1), br, A.err, A.wait);
      if (!__shfl_sync(0xffffffffu, w, 0)) break;
      const int nmb = (D.np + 127) / 128;
      bool ok = true;
      for (int k0 = 0; k0 < D.kp; k0 += KC, q++) {
        const int s = q % NST;
        if (lane == 0) w = rwait(&br->conv[s], (uint32_t)((q / NST) & 1), br, A.err, A.wait);
        if (!__shfl_sync(0xffffffffu, w, 0)) {
          ok = false;
          break;
        }
        if (lane == 0) {
          umma::fence_after();
          const int kc = min(KC, D.kp - k0);
          const unsigned char* stg = stage(s);
          for (int c = 0; c < kc / 16; c++) {
            const unsigned char* mem = stg + kFac + kRows + c * 4096;
            const uint64_t dmh = umma::smem_desc(mem, 1024, 128);
            const uint64_t dml = umma::smem_desc(mem + 2048, 1024, 128);
            for (int mb = 0; mb < nmb; mb++) {
              const unsigned char* fac = stg + c * D.np * 64 + mb * 2048;
              const uint64_t dfh = umma::smem_desc(fac, (uint32_t)D.np * 16, 128);
              const uint64_t dfl = umma::smem_desc(fac + D.np * 32, (uint32_t)D.np * 16, 128);
              const uint32_t d = tbase + (uint32_t)(b * 128 + mb * EMT);
              umma::mma_bf16(d, dfh, dmh, idesc, (k0 > 0 || c > 0) ? 1 : 0);
              umma::mma_bf16(d, dfh, dml, idesc, 1);
              umma::mma_bf16(d, dfl, dmh, idesc, 1);
            }
          }
          umma::commit(&br->empty[s]);
        }
        __syncwarp();
      }
      if (!ok) break;
      if (lane == 0) umma::commit(&br->accf[b]);
      __syncwarp();
    }
    // every MMA issued by this thread is done before the block leaves
    if (lane == 0) {
      umma::commit(&br->done);
      bwait(&br->done, 0);
    }
    __syncwarp();
  } else if (warp < 6) {
    // -------------------------------------------------------- converters
    const int ct = tid - 64;
    int q = 0;
    bool ok = true;
    Walk W;
    walk_init(W);
    for (; W.j < nit && ok; walk_next(W)) {
      const TcItem& D = W.D;
      for (int k0 = 0; k0 < D.kp; k0 += KC, q++) {
        const int s = q % NST;
        if (!rwait(&br->full[s], (uint32_t)((q / NST) & 1), br, A.err, A.wait)) {
          ok = false;
          break;
        }
        const int kc = min(KC, D.kp - k0);
        const int nrow = max(0, min(kc, D.kv - k0));
        const float* rows = (const float*)(stage(s) + kFac);
        unsigned char* mop = stage(s) + kFac + kRows;
        // one task = one core-matrix row: member m, 8 consecutive k -> 16
        // bytes of hi and 16 bytes of lo
        for (int e = ct; e < (kc / 8) * EMT; e += 128) {
          const int kb = e / EMT, m = e % EMT;
          uint32_t hw[4], lw[4];
#pragma unroll
          for (int i = 0; i < 4; i++) {
            const int k = kb * 8 + 2 * i;
            const float v0 = k < nrow ? rows[k * EMT + m] : 0.f;
            const float v1 = k + 1 < nrow ? rows[(k + 1) * EMT + m] : 0.f;
            const __nv_bfloat162 h2 = __floats2bfloat162_rn(v0, v1);
            const float2 hf = __bfloat1622float2(h2);
            const __nv_bfloat162 l2 = __floats2bfloat162_rn(v0 - hf.x, v1 - hf.y);
            hw[i] = *reinterpret_cast<const uint32_t*>(&h2);
            lw[i] = *reinterpret_cast<const uint32_t*>(&l2);
          }
          const uint32_t o = (uint32_t)(kb / 2) * 4096 + umma::kmajor_offset(m, (kb % 2) * 8, 1024, 128);
          *reinterpret_cast<uint4*>(mop + o) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
          *reinterpret_cast<uint4*>(mop + o + 2048) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
        }
        fasync();
        barrive(&br->conv[s]);
      }
    }
    __syncwarp();
  } else if (warp < 10) {
    // ---------------------------------------------------------- epilogue
    const int et = tid - 192, quad = warp & 3;
    Walk W;
    walk_init(W);
    for (; W.j < nit; walk_next(W)) {
      const int j = W.j;
      const int b = j & 1;
      const TcItem& D = W.D;
      const TcMat& M = W.it < n0 ? A : B;
      if (et == 0) br->flag = rwait(&br->accf[b], (uint32_t)((j / 2) & 1), br, A.err, A.wait) ? 1 : 0;
      group_sync();
      const int ok = br->flag;
      group_sync();
      if (!ok) break;
      umma::fence_after();
      const int nmb = (D.np + 127) / 128;
      for (int mb = 0; mb < nmb; mb++) {
        const int n = mb * 128 + 32 * quad + lane;  // factor row of this thread
        const uint32_t taddr = tbase + ((uint32_t)(32 * quad) << 16) + (uint32_t)(b * 128 + mb * EMT);
        uint32_t v[4][16];
#pragma unroll
        for (int c = 0; c < 4; c++) umma::ld_32x32b_x16_nowait(taddr + 16 * c, v[c]);
        umma::wait_ld();
        if (n < D.nv) {
          float* dst;
          if (PH == 2) dst = M.gpart + ((int64_t)D.out0 + n) * EMT;
          else if (D.ntile == 1) dst = M.z + ((int64_t)D.out0 + n) * EMT;
          else dst = M.part + ((int64_t)D.poff + (int64_t)D.tile * D.nv + n) * EMT;
#pragma unroll
          for (int c = 0; c < 4; c++)
#pragma unroll
            for (int i = 0; i < 16; i += 4)
              *reinterpret_cast<float4*>(dst + 16 * c + i) =
                  make_float4(__uint_as_float(v[c][i]), __uint_as_float(v[c][i + 1]), __uint_as_float(v[c][i + 2]),
                              __uint_as_float(v[c][i + 3]));
        }
        __syncwarp();
      }
      umma::fence_before();
      barrive(&br->acce[b]);
      if (PH == 1 && D.ntile > 1) {
        // the last tile of a column group to arrive sums the tiles in order
        __threadfence();
        group_sync();
        if (et == 0) br->flag = arrive_ar(&M.cnt[D.cg]) == D.ntile - 1;
        group_sync();
        if (br->flag) {
          for (int idx = et; idx < D.nv * EMT; idx += 128) {
            const int col = idx / EMT, mm = idx % EMT;
            float t = 0.f;
            for (int q = 0; q < D.ntile; q++)
              t += __ldcg(&M.part[((int64_t)D.poff + (int64_t)q * D.nv + col) * EMT + mm]);
            M.z[((int64_t)D.out0 + col) * EMT + mm] = t;
          }
          if (et == 0) M.cnt[D.cg] = 0;
        }
        group_sync();
      }
    }
    __syncwarp();
  }
  umma::fence_before();
  __syncthreads();
  umma::fence_after();
  if (warp == 0) {
    umma::tmem_dealloc(tbase, kTmemCols);
    umma::tmem_relinquish();
  }
}

// FP64 body -> BF16 hi / lo canonical stores; one warp per run
__global__ void tcconv_kernel(const double* __restrict__ body, const TcCopy* __restrict__ map, int64_t nmap,
                              __nv_bfloat16* __restrict__ dst) {
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t nw = (gridDim.x * (int64_t)blockDim.x) >> 5;
  for (int64_t q = w; q < nmap; q += nw) {
    const TcCopy c = map[q];
    for (int i = lane; i < c.len; i += 32) {
      const int n = c.n0 + i * c.dn, k = c.k0 + i * c.dk;
      const int ch = k / 16, kk = k % 16;
      const int64_t o = c.item + (int64_t)ch * c.np * 32 + (int64_t)(kk / 8) * c.np * 8 + (int64_t)(n / 8) * 64 +
                        (n % 8) * 8 + (kk % 8);
      const double v = body[c.src + (int64_t)i * c.stride];
      const __nv_bfloat16 hi = __float2bfloat16_rn((float)v);
      const __nv_bfloat16 lo = __float2bfloat16_rn((float)(v - (double)__bfloat162float(hi)));
      dst[o] = hi;
      dst[o + (int64_t)c.np * 16] = lo;
    }
  }
}

}  // namespace

size_t tc_smem_bytes() { return (size_t)NST * kStage + sizeof(Bars); }

void tc_prepare() {
  cudaFuncSetAttribute(tc_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_smem_bytes());
  cudaFuncSetAttribute(tc_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_smem_bytes());
}

// one block per SM of the schedule's grid (a.G)
void launch_tc(int phase, const TcMat& a, const TcMat& b, int nmat, const float* x, cudaStream_t st) {
  const int n = phase == 1 ? a.n1 + (nmat == 2 ? b.n1 : 0) : a.n2 + (nmat == 2 ? b.n2 : 0);
  if (n == 0 || a.G <= 0) return;
  if (phase == 1) tc_kernel<1><<<a.G, kThreads, tc_smem_bytes(), st>>>(a, b, nmat, x);
  else tc_kernel<2><<<a.G, kThreads, tc_smem_bytes(), st>>>(a, b, nmat, x);
}

void launch_tcconv(const double* body, const TcCopy* map, int64_t nmap, __nv_bfloat16* dst, cudaStream_t st) {
  if (nmap == 0) return;
  const int blocks = (int)((nmap + 7) / 8 < 152 * 16 ? (nmap + 7) / 8 : 152 * 16);
  tcconv_kernel<<<blocks, 256, 0, st>>>(body, map, nmap, dst);
}

}  // namespace hbi
