// hbi_umma_probe.cu -- tensor-core (tcgen05) building blocks of the ensemble
// product: one H-matrix applied to the slip-rate vectors of 64 simulations at
// once, which turns each product into a dense multi-vector contraction.
//
// This file holds the self-test of the tensor-core path: one
// M=128 x N=64 x K=16 BF16 MMA with FP32 accumulation in tensor memory, from
// operands laid out in shared memory in the canonical no-swizzle K-major
// layout (hbi_umma.cuh), read back by tcgen05.ld.  The host compares it with
// the product computed on the CPU.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/hbi_gpu.h"
#include "hbi_umma.cuh"

namespace hbi {
int set_error(int code, const char* msg);

namespace {

__device__ __forceinline__ void mbar_init_u(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(umma::saddr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait_u(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(umma::saddr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

constexpr int kProbeOperandBytes = 65536;  // each operand region, zeroed

// variant 0: LBO = K-direction core-matrix stride, SBO = M/N-direction stride;
// variant 1: the two swapped (same data layout); variant 2: as 0 with M = 64
// (A's first 64 rows), D read back from all 128 lanes
__global__ void __launch_bounds__(128) umma_probe_kernel(const uint16_t* __restrict__ A,
                                                         const uint16_t* __restrict__ B, float* __restrict__ D,
                                                         int variant, int* status) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* sA = sm;
  unsigned char* sB = sm + kProbeOperandBytes;
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + 2 * kProbeOperandBytes);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + 2 * kProbeOperandBytes + 64);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int i = tid; i < 2 * kProbeOperandBytes / 16; i += blockDim.x) reinterpret_cast<uint4*>(sm)[i] = make_uint4(0, 0, 0, 0);
  __syncthreads();
  // A: 128 x 16 (row, k), B: 64 x 16 (n, k), canonical K-major layouts
  const uint32_t lboA = 2048, sboA = 128, lboB = 1024, sboB = 128;
  for (int e = tid; e < 128 * 16; e += blockDim.x)
    *reinterpret_cast<uint16_t*>(sA + umma::kmajor_offset(e / 16, e % 16, lboA, sboA)) = A[e];
  for (int e = tid; e < 64 * 16; e += blockDim.x)
    *reinterpret_cast<uint16_t*>(sB + umma::kmajor_offset(e / 16, e % 16, lboB, sboB)) = B[e];
  // the tensor core reads shared memory through the async proxy
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (tid == 0) mbar_init_u(bar, 1);
  if (warp == 0) umma::tmem_alloc(tslot, 64);
  umma::fence_before();
  __syncthreads();
  umma::fence_after();
  const uint32_t tbase = *tslot;
  if (tid == 0) {
    uint64_t da, db;
    if (variant != 1) {
      da = umma::smem_desc(sA, lboA, sboA);
      db = umma::smem_desc(sB, lboB, sboB);
    } else {
      da = umma::smem_desc(sA, sboA, lboA);
      db = umma::smem_desc(sB, sboB, lboB);
    }
    umma::mma_bf16(tbase, da, db, umma::idesc_bf16_f32(variant == 2 ? 64 : 128, 64), 0);
    umma::commit(bar);
  }
  // bounded wait for the MMA (about a second of SM clock)
  int ok = 0;
  const long long t0 = clock64();
  while (!(ok = mbar_try_wait_u(bar, 0)))
    if (clock64() - t0 > (2LL << 30)) break;
  ok = __syncthreads_and(ok);
  umma::fence_after();
  if (ok) {
    const int row = 32 * warp + lane;
    const uint32_t taddr = tbase + ((uint32_t)(32 * warp) << 16);
    for (int c = 0; c < 4; c++) {
      float v[16];
      umma::ld_32x32b_x16(taddr + c * 16, v);
      for (int i = 0; i < 16; i++) D[row * 64 + c * 16 + i] = v[i];
    }
  } else if (tid == 0) {
    atomicExch(status, 1);
  }
  umma::fence_before();
  __syncthreads();
  if (warp == 0) {
    umma::tmem_dealloc(tbase, 64);
    umma::tmem_relinquish();
  }
}

}  // namespace
}  // namespace hbi

extern "C" int hbi_umma_probe(const uint16_t* a, const uint16_t* b, float* d, int variant) {
  using namespace hbi;
  if (!a || !b || !d || variant < 0 || variant > 2) return set_error(HBI_ERR_ARG, "hbi_umma_probe: bad arguments");
  uint16_t *da = nullptr, *db = nullptr;
  float* dd = nullptr;
  int* ds = nullptr;
  const size_t smem = 2 * kProbeOperandBytes + 1024;
  int rc = HBI_OK;
  if (cudaMalloc(&da, 128 * 16 * 2) != cudaSuccess || cudaMalloc(&db, 64 * 16 * 2) != cudaSuccess ||
      cudaMalloc(&dd, 128 * 64 * 4) != cudaSuccess || cudaMalloc(&ds, 4) != cudaSuccess) {
    rc = set_error(HBI_ERR_NOMEM, "hbi_umma_probe: allocation");
  } else {
    cudaMemcpy(da, a, 128 * 16 * 2, cudaMemcpyHostToDevice);
    cudaMemcpy(db, b, 64 * 16 * 2, cudaMemcpyHostToDevice);
    cudaMemset(dd, 0, 128 * 64 * 4);
    cudaMemset(ds, 0, 4);
    cudaFuncSetAttribute(umma_probe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    umma_probe_kernel<<<1, 128, smem>>>(da, db, dd, variant, ds);
    cudaError_t e = cudaDeviceSynchronize();
    int st = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&st, ds, 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(d, dd, 128 * 64 * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = set_error(HBI_ERR_CUDA, cudaGetErrorString(e));
    else if (st) rc = set_error(HBI_ERR_CUDA, "hbi_umma_probe: the MMA did not complete in time");
  }
  cudaFree(da);
  cudaFree(db);
  cudaFree(dd);
  cudaFree(ds);
  return rc;
}
