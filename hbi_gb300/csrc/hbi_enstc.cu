// hbi_enstc.cu -- the ensemble's multi-vector product on the 5th-generation
// tensor cores (tcgen05).
//
// Each contraction is D (64 members x N) = A (64 x K) * B^T, B (N x K) the
// factor tile (plan_tc, hbi_structure.cpp):
//   phase 1: N = the columns of a column group (z = V^T x), K = a tile's rows,
//            A = the tile's rows of X (64 members);
//   phase 2: N = the rows of a row-group tile, K = the group's columns,
//            A = the columns' multipliers (rows of z or X).
// B is stored as BF16 hi + lo halves in the canonical no-swizzle K-major
// layout and arrives by cp.async.bulk (TMA) in stages of 32 K; the FP32 rows
// of A arrive with it and are split into BF16 hi + lo by the block's threads
// straight into the canonical layout.  One thread issues, per 16-K chunk,
// D += A_hi B_hi + A_hi B_lo + A_lo B_hi (the lo x lo term is below FP32's
// resolution), accumulating in tensor memory (FP32, 64 lanes x N columns);
// tcgen05.commit on a stage's mbarrier releases the stage.  At the end of an
// item the warpgroup reads D back with tcgen05.ld (M = 64: member i in lane
// (i/16)*32 + i%16) and writes the 64 members' results.
//
// Every wait is bounded (about a second of SM clock); on a time-out the
// operator's error word is set, the block waits (bounded) for its copies and
// MMAs and releases its tensor memory before it leaves.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "hbi_kernels.cuh"
#include "hbi_umma.cuh"

namespace hbi {

struct TcMat {            // one H-matrix's tensor-core stores and ensemble scratch
  const TcItem* p1;
  int n1;
  const TcItem* p2;
  int n2;
  const __nv_bfloat16* s1;  // phase-1 store
  const __nv_bfloat16* s2;  // phase-2 store
  const int32_t* midx;
  float* z;                 // zlen x 64
  float* part;              // plen1 x 64
  int* cnt;                 // per column group piece
  float* gpart;             // rows of the row groups x 64 (the operator's phase-3 layout)
  int* err;
};

namespace {

constexpr int EMT = 64;
constexpr int KC = 32;                    // K per stage
constexpr int kB = 2 * 256 * 64;          // B hi+lo of 2 chunks at N = 256: 32 KB
constexpr int kS = KC * EMT * 4;          // FP32 A rows: 8 KB
constexpr int kA = 2 * 4096;              // A hi+lo of 2 chunks: 8 KB
constexpr int kStageT = kB + kS + kA;
constexpr long long kWaitT = 2LL << 30;

__device__ __forceinline__ uint32_t sa(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void binit(uint64_t* b) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sa(b)) : "memory");
}
__device__ __forceinline__ void bexpect(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sa(b)), "r"(bytes) : "memory");
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
__device__ __forceinline__ bool bwait(uint64_t* b, uint32_t par) {
  const long long t0 = clock64();
  while (!btry(b, par))
    if (clock64() - t0 > kWaitT) return false;
  return true;
}
__device__ __forceinline__ void bcopy(void* dst, const void* src, uint32_t bytes, uint64_t* b) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   sa(dst)),
               "l"(src), "r"(bytes), "r"(sa(b))
               : "memory");
}
__device__ __forceinline__ void fasync() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ int arrive_ar(int* p) {
  int old;
  asm volatile("atom.add.acq_rel.gpu.s32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
  return old;
}

// PH = 1: z = V^T x; PH = 2: partial row sums of U z + A x
template <int PH>
__global__ void __launch_bounds__(128, 2) tc_kernel(TcMat A, TcMat B, int nmat, const float* __restrict__ X) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* stg[2] = {sm, sm + kStageT};
  uint64_t* full = (uint64_t*)(sm + 2 * kStageT);
  uint64_t* mmab = full + 2;
  uint64_t* itemb = full + 4;
  __shared__ uint32_t tslot;
  __shared__ int sh_ok, sh_last;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int i = 0; i < 5; i++) binit(&full[i]);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) umma::tmem_alloc(&tslot, 256);
  umma::fence_before();
  __syncthreads();
  umma::fence_after();
  const uint32_t tbase = tslot;
  const int n0 = PH == 1 ? A.n1 : A.n2;
  const int ntot = nmat == 2 ? n0 + (PH == 1 ? B.n1 : B.n2) : n0;
  const int G = gridDim.x;
  auto desc = [&](int it) -> TcItem {
    TcItem d{};
    if (it < ntot) d = PH == 1 ? (it < n0 ? A.p1[it] : B.p1[it - n0]) : (it < n0 ? A.p2[it] : B.p2[it - n0]);
    return d;
  };
  int failed = 0;
  // producer: stage q of the block's chunk sequence into stg[q & 1]
  int p_it = blockIdx.x, p_k0 = 0, p_seq = 0;
  TcItem Dp = desc(p_it);
  auto produce = [&]() {
    if (p_it >= ntot || failed) return;
    const int s = p_seq & 1;
    const TcMat& M = p_it < n0 ? A : B;
    if (tid == 0 && p_seq >= 2) {
      // the MMAs that read this stage before must be done
      if (!bwait(&mmab[s], (uint32_t)(((p_seq - 2) >> 1) & 1))) failed = 1;
    }
    const int kc = min(KC, Dp.kp - p_k0);
    const int nrow = max(0, min(kc, Dp.kv - p_k0));  // A rows that carry data
    if (warp == 0 && !__shfl_sync(0xffffffffu, failed, 0)) {
      const uint32_t bbytes = (uint32_t)((kc / 16) * Dp.np * 64);
      const __nv_bfloat16* bsrc = (PH == 1 ? M.s1 : M.s2) + Dp.soff + (int64_t)(p_k0 / 16) * Dp.np * 32;
      int mi = 0;
      if (PH == 2 && lane < nrow) mi = __ldg(&M.midx[Dp.m0 + p_k0 + lane]);
      if (lane == 0) {
        fasync();
        bexpect(&full[s], bbytes + (uint32_t)(nrow * EMT * 4));
        bcopy(stg[s], bsrc, bbytes, &full[s]);
        if (PH == 1 && nrow > 0)
          bcopy(stg[s] + kB, X + (int64_t)(Dp.m0 + p_k0) * EMT, (uint32_t)(nrow * EMT * 4), &full[s]);
      }
      __syncwarp();
      if (PH == 2 && lane < nrow) {
        const float* src = mi >= 0 ? M.z + (int64_t)mi * EMT : X + (int64_t)(-mi - 1) * EMT;
        fasync();
        bcopy(stg[s] + kB + lane * EMT * 4, src, EMT * 4, &full[s]);
      }
    }
    p_seq++;
    p_k0 += kc;
    if (p_k0 >= Dp.kp) {
      p_it += G;
      p_k0 = 0;
      Dp = desc(p_it);
    }
  };
  produce();
  produce();
  int c_it = blockIdx.x, c_k0 = 0, c_seq = 0, nitem = 0;
  TcItem Dc = desc(c_it);
  while (c_it < ntot) {
    const TcMat& M = c_it < n0 ? A : B;
    const int s = c_seq & 1;
    if (tid == 0) sh_ok = !failed && bwait(&full[s], (uint32_t)((c_seq >> 1) & 1));
    __syncthreads();
    if (!sh_ok) {
      failed = 1;
      break;
    }
    while (!btry(&full[s], (uint32_t)((c_seq >> 1) & 1))) {
    }
    const int kc = min(KC, Dc.kp - c_k0);
    const int nrow = max(0, min(kc, Dc.kv - c_k0));
    // A: FP32 rows (k, member) -> BF16 hi / lo, canonical K-major (member, k)
    const float* rows = (const float*)(stg[s] + kB);
    unsigned char* aop = stg[s] + kB + kS;
    // one task = one core-matrix row: member m, 8 consecutive k -> 16 bytes
    // of hi and 16 bytes of lo
    for (int e = tid; e < (kc / 8) * EMT; e += blockDim.x) {
      const int kb = e / EMT, m = e % EMT;
      uint32_t hw[4], lw[4];
#pragma unroll
      for (int i = 0; i < 4; i++) {
        const int k0 = kb * 8 + 2 * i;
        const float v0 = k0 < nrow ? rows[k0 * EMT + m] : 0.f;
        const float v1 = k0 + 1 < nrow ? rows[(k0 + 1) * EMT + m] : 0.f;
        const __nv_bfloat162 h2 = __floats2bfloat162_rn(v0, v1);
        const float2 hf = __bfloat1622float2(h2);
        const __nv_bfloat162 l2 = __floats2bfloat162_rn(v0 - hf.x, v1 - hf.y);
        hw[i] = *reinterpret_cast<const uint32_t*>(&h2);
        lw[i] = *reinterpret_cast<const uint32_t*>(&l2);
      }
      const uint32_t o = (uint32_t)(kb / 2) * 4096 + umma::kmajor_offset(m, (kb % 2) * 8, 1024, 128);
      *reinterpret_cast<uint4*>(aop + o) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
      *reinterpret_cast<uint4*>(aop + o + 2048) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
    }
    fasync();
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    const bool last = c_k0 + kc >= Dc.kp;
    if (tid == 0) {
      const uint32_t idesc = umma::idesc_bf16_f32(64, Dc.np);
      for (int c = 0; c < kc / 16; c++) {
        const unsigned char* bh = stg[s] + c * Dc.np * 64;
        const uint64_t dbh = umma::smem_desc(bh, (uint32_t)Dc.np * 16, 128);
        const uint64_t dbl = umma::smem_desc(bh + Dc.np * 32, (uint32_t)Dc.np * 16, 128);
        const uint64_t dah = umma::smem_desc(aop + c * 4096, 1024, 128);
        const uint64_t dal = umma::smem_desc(aop + c * 4096 + 2048, 1024, 128);
        umma::mma_bf16(tbase, dah, dbh, idesc, (c_k0 > 0 || c > 0) ? 1 : 0);
        umma::mma_bf16(tbase, dah, dbl, idesc, 1);
        umma::mma_bf16(tbase, dal, dbh, idesc, 1);
      }
      umma::commit(&mmab[s]);
      if (last) umma::commit(&itemb[0]);
    }
    c_seq++;
    produce();
    c_k0 += kc;
    if (!last) continue;
    // item done: D (64 x np) from tensor memory
    if (tid == 0) sh_ok = !failed && bwait(&itemb[0], (uint32_t)(nitem & 1));
    __syncthreads();
    if (!sh_ok) {
      failed = 1;
      break;
    }
    while (!btry(&itemb[0], (uint32_t)(nitem & 1))) {
    }
    umma::fence_after();
    {
      const int m = 16 * warp + lane;  // valid for lane < 16
      const uint32_t taddr = tbase + ((uint32_t)(32 * warp) << 16);
      // 64 columns per round: four loads in flight, one wait
      for (int n0c = 0; n0c < Dc.np; n0c += 64) {
        uint32_t v[4][16];
#pragma unroll
        for (int q = 0; q < 4; q++) umma::ld_32x32b_x16_nowait(taddr + n0c + 16 * q, v[q]);
        umma::wait_ld();
        if (lane < 16) {
#pragma unroll
          for (int q = 0; q < 4; q++)
#pragma unroll
            for (int i = 0; i < 16; i++) {
              const int nn = n0c + 16 * q + i;
              if (nn < Dc.nv) {
                float* dst;
                if (PH == 2) dst = M.gpart + ((int64_t)Dc.out0 + nn) * EMT;
                else if (Dc.ntile == 1) dst = M.z + ((int64_t)Dc.out0 + nn) * EMT;
                else dst = M.part + ((int64_t)Dc.poff + (int64_t)Dc.tile * Dc.nv + nn) * EMT;
                dst[m] = __uint_as_float(v[q][i]);
              }
            }
        }
      }
    }
    umma::fence_before();
    if (PH == 1 && Dc.ntile > 1) {
      __threadfence();
      __syncthreads();
      if (tid == 0) sh_last = arrive_ar(&M.cnt[Dc.cg]) == Dc.ntile - 1;
      __syncthreads();
      if (sh_last) {
        for (int idx = tid; idx < Dc.nv * EMT; idx += blockDim.x) {
          const int col = idx / EMT, mm = idx % EMT;
          float t = 0.f;
          for (int q = 0; q < Dc.ntile; q++)
            t += __ldcg(&M.part[((int64_t)Dc.poff + (int64_t)q * Dc.nv + col) * EMT + mm]);
          M.z[((int64_t)Dc.out0 + col) * EMT + mm] = t;
        }
        if (tid == 0) M.cnt[Dc.cg] = 0;
      }
    }
    __syncthreads();
    nitem++;
    c_it += G;
    c_k0 = 0;
    Dc = desc(c_it);
  }
  if (failed) {
    // record, then let outstanding copies and MMAs finish (bounded) before
    // the tensor memory is released
    if (tid == 0) {
      if (A.err) atomicExch(A.err, 1);
      for (int q = c_seq; q < p_seq; q++) bwait(&full[q & 1], (uint32_t)((q >> 1) & 1));
      for (int q = max(0, c_seq - 2); q < c_seq; q++) bwait(&mmab[q & 1], (uint32_t)((q >> 1) & 1));
    }
  }
  umma::fence_before();
  __syncthreads();
  if (warp == 0) {
    umma::tmem_dealloc(tbase, 256);
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

size_t tc_smem_bytes() { return 2 * (size_t)kStageT + 64; }

void tc_prepare() {
  cudaFuncSetAttribute(tc_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_smem_bytes());
  cudaFuncSetAttribute(tc_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_smem_bytes());
}

void launch_tc(int phase, const TcMat& a, const TcMat& b, int nmat, const float* x, int sm, cudaStream_t st) {
  const int n = phase == 1 ? a.n1 + (nmat == 2 ? b.n1 : 0) : a.n2 + (nmat == 2 ? b.n2 : 0);
  if (n == 0) return;
  const int grid = n < 2 * sm ? n : 2 * sm;
  if (phase == 1) tc_kernel<1><<<grid, 128, tc_smem_bytes(), st>>>(a, b, nmat, x);
  else tc_kernel<2><<<grid, 128, tc_smem_bytes(), st>>>(a, b, nmat, x);
}

void launch_tcconv(const double* body, const TcCopy* map, int64_t nmap, __nv_bfloat16* dst, cudaStream_t st) {
  if (nmap == 0) return;
  const int blocks = (int)((nmap + 7) / 8 < 152 * 16 ? (nmap + 7) / 8 : 152 * 16);
  tcconv_kernel<<<blocks, 256, 0, st>>>(body, map, nmap, dst);
}

}  // namespace hbi
