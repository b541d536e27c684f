// hbi_stream.cu -- phases 1 and 2 of the lattice H-matrix-vector product
// (HACApK_adot_body_lfmtx_hyp_contiguous, m_HACApK_solve.f90:2108-2164) as
// streams of bulk asynchronous copies.
//
// The factor store is laid out in row tiles (hbi_structure.cpp, plan_stream):
// every work item reads one contiguous region -- the column segments of one
// tile of a column group (phase 1) or of a row group (phase 2) -- in chunks of
// whole columns that fill one shared-memory stage (8 KB or 16 KB).  Each warp
// of a block owns NS stages with one mbarrier each; one lane starts a
// cp.async.bulk (TMA) copy of a chunk into a free stage while the warp
// consumes an earlier stage; the copies carry an L2 evict-first policy, so
// that the factor stream does not evict the small data every launch reads.
// The small per-item operands (x rows) are loaded one item ahead of their
// use, phase 2's multipliers one chunk ahead.  Which items a warp walks is
// set by the launch shape's schedule (WarpSeq).
//
// Phase 1 maps lanes to a stage in one of two ways: column slots (a segment
// of ntp rows covered by LW = pow2ceil(ntp / VEC) lanes with one 16-byte
// vector each, CS = 32/LW slots side by side, reduced by shuffles) or one
// lane per column over the swizzled V store (p1_columns).  A column's sum
// is final per row tile (z), or a partial combined by the last tile of a
// column group to arrive.  Phase 2 accumulates y rows per lane over the
// column slots and reduces over the slots once per item.  Every sum has a
// fixed order: results are deterministic run to run.
//
// Waits are bounded: a stage that does not complete within the operator's
// wait bound (~1 s of SM clock) sets the operator's error word, the warp waits
// (bounded by ~1 s again) for its other copies and leaves; the host reads and
// clears the word at its next synchronisation (take_device_error).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>
#include <mutex>

#include "hbi_kernels.cuh"

namespace hbi {

namespace {

constexpr long long kWaitCycles = kWaitCyclesDefault;

template <typename T>
struct AccT {
  typedef float type;
};
template <>
struct AccT<double> {
  typedef double type;
};

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(saddr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// lane 0: wait for the phase `parity` of `bar` for at most kWaitCycles
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > kWaitCycles) return false;
  return true;
}

// L2 policy for data read once per product: evicted first, so that the
// factor stream (~1 GB per stage of an RK attempt, against a 126 MB L2) does
// not push out the small data every launch reads -- schedules, item
// descriptors, x, z, partial sums
__device__ __forceinline__ uint64_t l2_evict_first() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}

// bulk copy of streamed factor data, with that policy
__device__ __forceinline__ void bulk_g2s_stream(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
                                                uint64_t pol) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
          saddr(dst)),
      "l"(src), "r"(bytes), "r"(saddr(bar)), "l"(pol)
      : "memory");
}

__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// one 16-byte vector of shared memory as VEC accumulator values
__device__ __forceinline__ void lds16(const double* p, double* o) {
  const double2 v = *reinterpret_cast<const double2*>(p);
  o[0] = v.x;
  o[1] = v.y;
}
__device__ __forceinline__ void lds16(const float* p, float* o) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  o[0] = v.x;
  o[1] = v.y;
  o[2] = v.z;
  o[3] = v.w;
}
__device__ __forceinline__ void lds16(const __nv_bfloat16* p, float* o) {
  const uint4 v = *reinterpret_cast<const uint4*>(p);
  const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
  for (int i = 0; i < 4; i++) {
    o[2 * i] = __uint_as_float(w[i] << 16);
    o[2 * i + 1] = __uint_as_float(w[i] & 0xffff0000u);
  }
}

__device__ __forceinline__ int log2ceil(int n) { return n <= 1 ? 0 : 32 - __clz(n - 1); }

// shared memory of a block: per warp NS stages of SB bytes, then per warp the
// 128 multipliers of its current phase-2 chunk, then the stage barriers, then
// per warp the item ids a dynamic schedule took (kHist)
constexpr int kMaxCols = 128;  // columns of a chunk at most (chunk_cols)
constexpr int kMu = kMaxCols * 8;
constexpr int kHist = 16;
template <int NW, int NS, int SB>
struct Ring {
  unsigned char* buf;  // stage s at buf + s * SB
  void* mu;            // kMaxCols multipliers (Acc) of the warp
  uint64_t* bar;
  int* hist;           // kHist item ids
  int* bctr;           // the block's item counter (block-shared schedule)
  __device__ Ring(unsigned char* smem, int warp) {
    buf = smem + (size_t)warp * NS * SB;
    mu = smem + (size_t)NW * NS * SB + (size_t)warp * kMu;
    bar = reinterpret_cast<uint64_t*>(smem + (size_t)NW * NS * SB + (size_t)NW * kMu) + warp * NS;
    int* tail = reinterpret_cast<int*>(smem + (size_t)NW * NS * SB + (size_t)NW * kMu + (size_t)NW * NS * 8);
    hist = tail + warp * kHist;
    bctr = tail + NW * kHist;
  }
};

// wait for a stage's phase `parity`; all lanes poll together (the loop stays
// converged) and acquire.  Returns false (and records the error) when the
// copy did not arrive within `limit` SM clock cycles; a limit of 0 is spent
// before the first probe, so every wait gives up (the error path on demand).
__device__ __forceinline__ bool stage_ready(uint64_t* bar, uint32_t parity, int* err, long long limit) {
  bool ok = limit > 0 && mbar_try_wait(bar, parity);
  if (!ok && limit > 0) {
    const long long t0 = clock64();
    while (!(ok = mbar_try_wait(bar, parity)))
      if (clock64() - t0 > limit) break;
  }
  // a completed phase stays completed until this warp refills the stage; a
  // warp whose lanes disagree counts as failed
  if (!__all_sync(0xffffffffu, ok)) {
    if ((threadIdx.x & 31) == 0 && err) atomicExch(err, 1);
    return false;
  }
  return true;
}

// after a failed wait: let the warp's copies still in flight land (bounded)
template <int NS>
__device__ void drain(uint64_t* bar, int c_seq, int p_seq) {
  if ((threadIdx.x & 31) == 0)
    for (int q = c_seq; q < p_seq; q++) mbar_wait_bounded(&bar[q % NS], (uint32_t)((q / NS) & 1));
  __syncwarp();
}

// arrival count with release (prior writes of the warp, ordered by the
// __syncwarp before it) and acquire (the partials of the other tiles)
__device__ __forceinline__ int arrive_acq_rel(int* p) {
  int old;
  asm volatile("atom.add.acq_rel.gpu.s32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
  return old;
}

// The items one warp walks, in order: the host's schedule when it was made
// for this grid (m0's list, then m1's), else every GW-th item; or, with a
// dynamic schedule, the items the warp takes from the phase's counter (both
// lists in order, longest first within each), one grab issued ahead so that
// its round trip overlaps the work, the ids kept in the warp's kHist slots
// (a warp looks at most NS + 3 items ahead of the item it consumes).  at(k)
// is the k-th item, ntot past the end.
struct WarpSeq {
  const int32_t *a0 = nullptr, *a1 = nullptr;
  int len0 = 0, len1 = 0, n0 = 0, gw = 0, GW = 1, ntot = 0;
  int* ctr = nullptr;  // dynamic: the phase's item counter
  int* hist = nullptr;
  int ngrab = 0, pend = 0, lane = 0;  // pend: lane 0's grab in flight
  // dynamic: a warp's first two items are fixed (the largest 2 GW items,
  // dealt in snake order), so that the grid does not start with one burst of
  // atomics on the counter; the counter numbers the items after them
  __device__ void make_dynamic(int* counter, int* slots) {
    ctr = counter;
    hist = slots;
    lane = threadIdx.x & 31;
    if (lane == 0) {
      hist[0] = gw < ntot ? gw : ntot;
      hist[1] = 2 * GW - 1 - gw < ntot ? 2 * GW - 1 - gw : ntot;
      pend = atomicAdd(ctr, 1);
    }
    __syncwarp();
    ngrab = 2;
  }
  // block-shared: the warps of a block take the block's items (the host's
  // per-block list, longest first) from a shared-memory counter; hist keeps
  // list positions
  int* sctr = nullptr;
  __device__ void make_block_shared(int* counter, int* slots) {
    sctr = counter;
    hist = slots;
    lane = threadIdx.x & 31;
    if (lane == 0) pend = atomicAdd(sctr, 1);
  }
  __device__ int at(int k) {
    if (sctr) {
      while (ngrab <= k) {
        const int v = __shfl_sync(0xffffffffu, pend, 0);
        if (lane == 0) hist[ngrab % kHist] = v;
        __syncwarp();
        ngrab++;
        if (lane == 0) pend = atomicAdd(sctr, 1);
      }
      const int v = hist[k % kHist];
      if (v < len0) return __ldg(&a0[v]);
      return v - len0 < len1 ? n0 + __ldg(&a1[v - len0]) : ntot;
    }
    if (ctr) {
      while (ngrab <= k) {
        const int v = __shfl_sync(0xffffffffu, pend, 0) + 2 * GW;
        if (lane == 0) hist[ngrab % kHist] = v < ntot ? v : ntot;
        __syncwarp();
        ngrab++;
        if (lane == 0) pend = atomicAdd(ctr, 1);
      }
      return hist[k % kHist];
    }
    if (a0) {
      if (k < len0) return __ldg(&a0[k]);
      k -= len0;
      return k < len1 ? n0 + __ldg(&a1[k]) : ntot;
    }
    const int64_t it = gw + (int64_t)k * GW;
    return it < ntot ? (int)it : ntot;
  }
};

// a warp of a dynamically scheduled phase leaves: its last grab is ordered
// before it counts itself out, and the last warp of the grid out resets the
// phase's counters for the next launch
__device__ __forceinline__ void dyn_leave(const WarpSeq& q, int* exits, int nwarps) {
  if (!q.ctr) return;
  __syncwarp();
  if (q.lane == 0) {
    // release: the warp's grabs, the one still in flight included, come
    // before its count; acquire: the last warp's reset comes after them all
    if (arrive_acq_rel(exits) == nwarps - 1) {
      atomicExch(q.ctr, 0);
      atomicExch(exits, 0);
    }
  }
  __syncwarp();
}

__device__ __forceinline__ WarpSeq warp_seq(const MatDev& m0, const MatDev& m1, int nmat, int phase, int shape,
                                            int gw, int GW, int n0, int ntot) {
  WarpSeq q;
  q.n0 = n0;
  q.gw = gw;
  q.GW = GW;
  q.ntot = ntot;
  const int32_t* off0 = phase == 1 ? m0.w1off[shape] : m0.w2off[shape];
  const int32_t* off1 = phase == 1 ? m1.w1off[shape] : m1.w2off[shape];
  const int g0 = phase == 1 ? m0.gw1[shape] : m0.gw2[shape], g1 = phase == 1 ? m1.gw1[shape] : m1.gw2[shape];
  if (off0 && g0 == GW && (nmat == 1 || (off1 && g1 == GW))) {
    q.a0 = (phase == 1 ? m0.w1item[shape] : m0.w2item[shape]) + __ldg(&off0[gw]);
    q.len0 = __ldg(&off0[gw + 1]) - __ldg(&off0[gw]);
    if (nmat == 2) {
      q.a1 = (phase == 1 ? m1.w1item[shape] : m1.w2item[shape]) + __ldg(&off1[gw]);
      q.len1 = __ldg(&off1[gw + 1]) - __ldg(&off1[gw]);
    }
  }
  return q;
}

}  // namespace

// Column sums of one stage under the lane-per-column mapping: st holds nc
// column segments of ntp rows (the item's chunk width is cc), xs the item's
// x tile (32 x VEC values); put(cl, sum) receives chunk column cl.  With 16
// columns per chunk, lanes L and L + 16 take halves of column L's vectors
// (their logical indices; the swizzle permutes within the column).
// the VEC x values of logical vector k of the x tile, as 16-byte loads
__device__ __forceinline__ void ldx(const float* xs, int k, float (&o)[4]) {
  const float4 v = reinterpret_cast<const float4*>(xs)[k];
  o[0] = v.x;
  o[1] = v.y;
  o[2] = v.z;
  o[3] = v.w;
}
__device__ __forceinline__ void ldx(const double* xs, int k, double (&o)[2]) {
  const double2 v = reinterpret_cast<const double2*>(xs)[k];
  o[0] = v.x;
  o[1] = v.y;
}
__device__ __forceinline__ void ldx(const float* xs, int k, float (&o)[8]) {
  const float4 a = reinterpret_cast<const float4*>(xs)[2 * k], b = reinterpret_cast<const float4*>(xs)[2 * k + 1];
  o[0] = a.x;
  o[1] = a.y;
  o[2] = a.z;
  o[3] = a.w;
  o[4] = b.x;
  o[5] = b.y;
  o[6] = b.z;
  o[7] = b.w;
}

template <typename T, typename Acc, typename Put>
__device__ __forceinline__ void p1_columns(const T* st, int ntp, int nc, int cc, const Acc* xs, int lane, Put put) {
  constexpr int VEC = 16 / sizeof(T);
  const int nq = ntp / VEC;  // 16-byte vectors per column segment
  if (cc <= 16 && nq == 32) {
    // full-height segments (512 bytes), 16 per chunk: lane L + 16h sums
    // logical vectors 16h .. 16h + 15 of column L.  The swizzle of column L
    // is L & 7 and permutes within aligned groups of eight, so the eight
    // physical offsets are computed once and the loop is fully unrolled.
    const int h = lane >> 4, cl = lane & 15;
    Acc acc[VEC];
#pragma unroll
    for (int v = 0; v < VEC; v++) acc[v] = 0;
    if (cl < nc) {
      const T* cp = st + cl * ntp + 16 * h * VEC;
      const int sw = cl & 7;
      const Acc* xh = xs + 16 * h * VEC;
#pragma unroll
      for (int i = 0; i < 16; i++) {
        Acc a[VEC], xv[VEC];
        lds16(cp + ((i & 8) + ((i & 7) ^ sw)) * VEC, a);
        ldx(xh, i, xv);
#pragma unroll
        for (int v = 0; v < VEC; v++) acc[v] += a[v] * xv[v];
      }
    }
    Acc t = acc[0];
#pragma unroll
    for (int v = 1; v < VEC; v++) t += acc[v];
    t += __shfl_xor_sync(0xffffffffu, t, 16);
    if (h == 0 && cl < nc) put(cl, t);
  } else if (cc <= 16) {
    const int h = lane >> 4, cl = lane & 15;
    const int half = (nq + 1) >> 1;
    const int k0 = h ? half : 0, k1 = h ? nq : half;
    Acc acc[VEC];
#pragma unroll
    for (int v = 0; v < VEC; v++) acc[v] = 0;
    if (cl < nc) {
      const T* cp = st + cl * ntp;
      const int sw = vswz(cl, nq);
#pragma unroll 4
      for (int k = k0; k < k1; k++) {
        const int ph = k ^ sw;
        Acc a[VEC];
        lds16(cp + ph * VEC, a);
#pragma unroll
        for (int v = 0; v < VEC; v++) acc[v] += a[v] * xs[k * VEC + v];
      }
    }
    Acc t = acc[0];
#pragma unroll
    for (int v = 1; v < VEC; v++) t += acc[v];
    t += __shfl_xor_sync(0xffffffffu, t, 16);
    if (h == 0 && cl < nc) put(cl, t);
  } else {
    // one lane per column, columns lane, lane + 32, ...
    for (int cl = lane; cl < nc; cl += 32) {
      const T* cp = st + cl * ntp;
      const int sw = vswz(cl, nq);
      Acc acc[VEC];
#pragma unroll
      for (int v = 0; v < VEC; v++) acc[v] = 0;
#pragma unroll 4
      for (int k = 0; k < nq; k++) {
        const int ph = k ^ sw;
        Acc a[VEC];
        lds16(cp + ph * VEC, a);
#pragma unroll
        for (int v = 0; v < VEC; v++) acc[v] += a[v] * xs[k * VEC + v];
      }
      Acc t = acc[0];
#pragma unroll
      for (int v = 1; v < VEC; v++) t += acc[v];
      put(cl, t);
    }
  }
}

// ---------------------------------------------------------------- phase 1
// Item = one row tile of a column group over all its columns; streamed in
// chunks of up to SB bytes.  Column sums of a chunk go to z (one tile) or to
// the tile's partials; the last tile of the group to finish sums the
// partials.  The V store is swizzled per column segment (vswz): logical
// 16-byte vector k of column c sits at k ^ vswz(c, ntp / VEC).
//
// MAP 0: the LW lanes of a column segment split its rows (one vector each)
// and reduce by shuffles; CS = 32 / LW columns side by side.
// MAP 1: one lane per column (two lanes, each half the rows, when a chunk has
// only 16 columns), the item's x tile in the warp's shared-memory buffer:
// no cross-lane reduction, VEC independent accumulator chains per lane.
template <typename T, int NW, int NS, int SB, int MAP, int SCHED>
__global__ void __launch_bounds__(NW * 32, 1) p1_stream_kernel(MatDev m0, MatDev m1, int nmat,
                                                               const double* __restrict__ x, int shape) {
  typedef typename AccT<T>::type Acc;
  constexpr int VEC = 16 / sizeof(T);
  constexpr int ESZ = sizeof(T);
  constexpr int BF = SB / 512;  // columns of a chunk of full-height (512-byte) segments
  extern __shared__ __align__(128) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  Ring<NW, NS, SB> R(smem, warp);
  Acc* xs = (Acc*)R.mu;  // MAP 1: the current item's x tile (32 x VEC values)
  if (lane == 0) {
    for (int s = 0; s < NS; s++) mbar_init(&R.bar[s], 1);
    fence_mbar_init();
  }
  __syncwarp();
  const int gw = blockIdx.x * NW + warp, GW = gridDim.x * NW;
  const int n0 = m0.ns1, ntot = nmat == 2 ? n0 + m1.ns1 : n0;
  // descriptors are loaded ahead of their use; the chunk width, which
  // follows from this shape's stage size, is derived only when an item
  // becomes current, so that no warp waits for a descriptor load it issued
  // just before
  auto desc = [&](int it) -> S1ItemDev {
    S1ItemDev d{};
    if (it < ntot) d = it < n0 ? m0.s1[it] : m1.s1[it - n0];
    return d;
  };
  auto current = [&](S1ItemDev d) {
    d.cc = d.ntp > 0 ? chunk_cols(d.ntp, ESZ, SB) : 16;
    return d;
  };
  WarpSeq seq;
  if constexpr (SCHED == 3) {
    // the block's list, shared by its warps through a counter
    if (threadIdx.x == 0) *R.bctr = 0;
    __syncthreads();
    seq = warp_seq(m0, m1, nmat, 1, shape, blockIdx.x, gridDim.x, n0, ntot);
    if (seq.a0) seq.make_block_shared(R.bctr, R.hist);
    else seq = warp_seq(m0, m1, nmat, 1, shape, gw, GW, n0, ntot);
  } else {
    seq = warp_seq(m0, m1, nmat, 1, shape, gw, GW, n0, ntot);
  }
  if constexpr (SCHED == 2) seq.make_dynamic(m0.dyn + 0, R.hist);
  int* const exits = m0.dyn + 1;
  // producer: walks this warp's items chunk by chunk, NS chunks ahead; the
  // item ids are fetched two items ahead, the descriptors one
  int p_k = 0, p_it = seq.at(0), p_itn = seq.at(1), p_itnn = seq.at(2), p_c0 = 0, p_seq = 0;
  S1ItemDev Dp = current(desc(p_it)), Dpn = desc(p_itn);
  auto produce = [&]() {
    if (p_it >= ntot) return;
    const int nc = min(Dp.cc, Dp.ncols - p_c0);
    const int s = p_seq % NS;
    if (lane == 0) {
      const uint32_t bytes = (uint32_t)(nc * Dp.ntp * ESZ);
      const T* src = (const T*)(p_it < n0 ? m0.vstore : m1.vstore) + Dp.soff + (int64_t)p_c0 * Dp.ntp;
      // no proxy fence: the stage's only generic accesses are this warp's
      // loads of its previous chunk, whose values were consumed (sums and
      // stores issued, __syncwarp) before the copy that overwrites it
      mbar_expect_tx(&R.bar[s], bytes);
      bulk_g2s_stream(R.buf + s * SB, src, bytes, &R.bar[s], l2_evict_first());
    }
    p_seq++;
    p_c0 += nc;
    if (p_c0 >= Dp.ncols) {
      p_k++;
      p_it = p_itn;
      p_itn = p_itnn;
      p_itnn = seq.at(p_k + 2);
      p_c0 = 0;
      Dp = current(Dpn);
      Dpn = desc(p_itn);
    }
  };
  for (int q = 0; q < NS; q++) produce();
  // the factor copies above read only static data; x, z, the partials and
  // the loop flags belong to earlier kernels of the stream
  pdl_launch_dependents();
  pdl_wait_prior();
  if (m0.skip && __ldcg(m0.skip)) {
    // a halted loop skips the product: let the copies already started land
    drain<NS>(R.bar, 0, p_seq);
    dyn_leave(seq, exits, GW);
    return;
  }
  // consumer: item ids three ahead, descriptors two
  int c_k = 0, c_it = seq.at(0), c_i1 = seq.at(1), c_i2 = seq.at(2), c_i3 = seq.at(3), c_c0 = 0, c_seq = 0;
  S1ItemDev Dc = current(desc(c_it)), Dn = desc(c_i1), Dnn = desc(c_i2);
  // x rows of an item: MAP 0, lane j of each column slot holds rows
  // j*VEC .. j*VEC+VEC-1; MAP 1, lane L holds rows L*VEC .. (for the tile)
  auto load_x = [&](const S1ItemDev& D, Acc* xv) {
    const int lw = MAP == 1 ? 5 : log2ceil(max(1, D.ntp / VEC));
    const int j = lane & ((1 << lw) - 1);
#pragma unroll
    for (int v = 0; v < VEC; v++) {
      const int r = j * VEC + v;
      xv[v] = (D.ncols > 0 && r < D.nt) ? (Acc)__ldg(&x[D.x0 + r]) : Acc(0);
    }
  };
  auto put_x = [&](const Acc* xv) {
    if constexpr (MAP == 1) {
      __syncwarp();
#pragma unroll
      for (int v = 0; v < VEC; v++) xs[lane * VEC + v] = xv[v];
      __syncwarp();
    }
  };
  Acc xc[VEC], xn[VEC];
  load_x(Dc, xc);
  load_x(Dn, xn);
  put_x(xc);
  // the arrival of a finished multi-tile item is resolved one chunk later, so
  // that the atomic's round trip overlaps the next chunk
  int pend_old = 0, pend_cg = -1, pend_ntile = 0, pend_ncols = 0, pend_poff = 0, pend_z0 = 0, pend_sec = 0;
  auto resolve = [&]() {
    if (pend_cg < 0) return;
    const int last = __shfl_sync(0xffffffffu, pend_old == pend_ntile - 1 ? 1 : 0, 0);
    if (last) {
      __syncwarp();  // lane 0's acquire orders the reads of every lane
      const MatDev& PM = pend_sec ? m1 : m0;
      Acc* z = (Acc*)PM.z;
      const Acc* part = (const Acc*)PM.part;
      for (int col = lane; col < pend_ncols; col += 32) {
        Acc t = 0;
        for (int q = 0; q < pend_ntile; q++) t += __ldcg(&part[pend_poff + (int64_t)q * pend_ncols + col]);
        z[pend_z0 + col] = t;
      }
      if (lane == 0) PM.cnt[pend_cg] = 0;
    }
    pend_cg = -1;
  };
  while (c_it < ntot) {
    const bool sec = c_it >= n0;
    const MatDev& M = sec ? m1 : m0;
    const int s = c_seq % NS;
    if (!stage_ready(&R.bar[s], (uint32_t)((c_seq / NS) & 1), M.err, M.wait)) {
      drain<NS>(R.bar, c_seq, p_seq);
      dyn_leave(seq, exits, GW);
      return;
    }
    const int nc = min(Dc.cc, Dc.ncols - c_c0);
    const T* st = (const T*)(R.buf + s * SB);
    const int nq = Dc.ntp / VEC;  // 16-byte vectors per column segment
    Acc* z = (Acc*)M.z;
    Acc* part = (Acc*)M.part;
    auto put = [&](int col, Acc v) {
      if (Dc.ntile == 1) z[Dc.z0 + col] = v;
      else part[Dc.poff + (int64_t)Dc.tile * Dc.ncols + col] = v;
    };
    if constexpr (MAP == 1) {
      p1_columns<T>(st, Dc.ntp, nc, Dc.cc, xs, lane, [&](int cl, Acc v) { put(c_c0 + cl, v); });
    } else {
      const int lw = log2ceil(nq), LW = 1 << lw, CS = 32 >> lw;
      const int slot = lane >> lw, j = lane & (LW - 1);
      if (LW == 32) {
        // tall tiles: BF columns at a time, reduced by a butterfly
        // reduce-scatter inside groups of BF lanes (BF-1 shuffle-adds per lane
        // for BF columns), then across the groups; lane L ends with the sum of
        // column r0 + L % BF
        for (int r0 = 0; r0 < nc; r0 += BF) {
          Acc p[BF];
          if (nq == 32 && r0 + BF <= nc) {
            // a full block of BF full-height columns: no predicates; the
            // swizzle of column r0 + u is u & 7 (r0 is a multiple of 16)
#pragma unroll
            for (int u = 0; u < BF; u++) {
              Acc a[VEC];
              lds16(st + (r0 + u) * (32 * VEC) + (lane ^ (u & 7)) * VEC, a);
              p[u] = a[0] * xc[0];
#pragma unroll
              for (int v = 1; v < VEC; v++) p[u] += a[v] * xc[v];
            }
          } else {
#pragma unroll
            for (int u = 0; u < BF; u++) {
              p[u] = 0;
              if (r0 + u < nc && j < nq) {
                Acc a[VEC];
                lds16(st + (r0 + u) * Dc.ntp + (j ^ vswz(r0 + u, nq)) * VEC, a);
#pragma unroll
                for (int v = 0; v < VEC; v++) p[u] += a[v] * xc[v];
              }
            }
          }
#pragma unroll
          for (int lev = BF / 2; lev >= 1; lev >>= 1) {
            const bool upper = (lane & lev) != 0;
#pragma unroll
            for (int i = 0; i < lev; i++) {
              const Acc send = upper ? p[i] : p[i + lev];
              const Acc keep = upper ? p[i + lev] : p[i];
              p[i] = keep + __shfl_xor_sync(0xffffffffu, send, lev);
            }
          }
#pragma unroll
          for (int o = BF; o < 32; o <<= 1) p[0] += __shfl_xor_sync(0xffffffffu, p[0], o);
          if (lane < BF && r0 + lane < nc) put(c_c0 + r0 + lane, p[0]);
        }
      } else
      // eight columns per slot at a time, so that their lane reductions
      // (shuffle chains) proceed side by side
      for (int r0 = 0; r0 < nc; r0 += 8 * CS) {
        constexpr int UC_ = 8;
        Acc p[UC_];
#pragma unroll
        for (int u = 0; u < UC_; u++) {
          const int sg = r0 + u * CS + slot;
          p[u] = 0;
          if (sg < nc && j < nq) {
            Acc a[VEC];
            lds16(st + sg * Dc.ntp + (j ^ vswz(sg, nq)) * VEC, a);
#pragma unroll
            for (int v = 0; v < VEC; v++) p[u] += a[v] * xc[v];
          }
        }
        for (int o = 1; o < LW; o <<= 1)
#pragma unroll
          for (int u = 0; u < UC_; u++) p[u] += __shfl_xor_sync(0xffffffffu, p[u], o);
        if (j == 0) {
#pragma unroll
          for (int u = 0; u < UC_; u++) {
            const int sg = r0 + u * CS + slot;
            if (sg < nc) put(c_c0 + sg, p[u]);
          }
        }
      }
    }
    __syncwarp();
    c_seq++;
    produce();
    resolve();
    c_c0 += nc;
    if (c_c0 < Dc.ncols) continue;
    // item done: the last row tile of a column group to arrive sums the
    // tiles in order (resolved after the next chunk)
    if (Dc.ntile > 1) {
      __syncwarp();
      if (lane == 0) pend_old = arrive_acq_rel(&M.cnt[Dc.cg]);
      pend_cg = Dc.cg;
      pend_ntile = Dc.ntile;
      pend_ncols = Dc.ncols;
      pend_poff = Dc.poff;
      pend_z0 = Dc.z0;
      pend_sec = sec;
    }
    c_k++;
    c_it = c_i1;
    c_i1 = c_i2;
    c_i2 = c_i3;
    c_i3 = seq.at(c_k + 3);
    c_c0 = 0;
    Dc = current(Dn);
    Dn = Dnn;
#pragma unroll
    for (int v = 0; v < VEC; v++) xc[v] = xn[v];
    put_x(xc);
    load_x(Dn, xn);
    Dnn = desc(c_i2);
  }
  resolve();
  dyn_leave(seq, exits, GW);
}

// ---------------------------------------------------------------- phase 2
// Item = one row tile of a row group over all its columns, streamed in chunks
// of up to SB bytes.  A chunk's multipliers (z for low-rank columns, x for
// dense ones) are fetched ahead of it: the column indices when the chunk's
// copy starts (NS chunks ahead), the gather of z / x one chunk ahead, so that
// neither latency falls between a stage's arrival and its use.  Lanes
// accumulate their rows over the item's chunks; one reduction over the
// column slots per item.
//
// GA: how many chunks ahead the multipliers are gathered (1, or 2 with three
// or more stages: the indices of chunk c + 2 are in the FIFO when chunk c
// starts); two register sets of multipliers then cover two chunk times of
// load latency.
template <typename T, int NW, int NS, int SB, int GA, int SCHED>
__global__ void __launch_bounds__(NW * 32, 1) p2_stream_kernel(MatDev m0, MatDev m1, int nmat,
                                                               const double* __restrict__ x, int shape) {
  typedef typename AccT<T>::type Acc;
  constexpr int VEC = 16 / sizeof(T);
  constexpr int ESZ = sizeof(T);
  constexpr int KP = kMaxCols / 32;  // multipliers per lane of one chunk
  static_assert(NS >= 2, "the multiplier gather runs one chunk ahead");
  static_assert(GA == 1 || (GA == 2 && NS >= 3), "a gather two chunks ahead needs three stages");
  extern __shared__ __align__(128) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  Ring<NW, NS, SB> R(smem, warp);
  Acc* musm = (Acc*)R.mu;
  if (lane == 0) {
    for (int s = 0; s < NS; s++) mbar_init(&R.bar[s], 1);
    fence_mbar_init();
  }
  __syncwarp();
  const int gw = blockIdx.x * NW + warp, GW = gridDim.x * NW;
  const int n0 = m0.ns2, ntot = nmat == 2 ? n0 + m1.ns2 : n0;
  // descriptors are loaded an item ahead; the chunk width is derived when
  // the item becomes current (no wait on a load issued just before)
  auto desc = [&](int it) -> S2ItemDev {
    S2ItemDev d{};
    if (it < ntot) d = it < n0 ? m0.s2[it] : m1.s2[it - n0];
    return d;
  };
  auto current = [&](S2ItemDev d) {
    d.cc = d.ntp > 0 ? chunk_cols(d.ntp, ESZ, SB) : 16;
    return d;
  };
  // column indices of a chunk in flight: lane L holds columns L + 32 i
  struct Pend {
    int32_t idx[KP];
    int nc, sec;
  };
  WarpSeq seq;
  if constexpr (SCHED == 3) {
    // the block's list, shared by its warps through a counter
    if (threadIdx.x == 0) *R.bctr = 0;
    __syncthreads();
    seq = warp_seq(m0, m1, nmat, 2, shape, blockIdx.x, gridDim.x, n0, ntot);
    if (seq.a0) seq.make_block_shared(R.bctr, R.hist);
    else seq = warp_seq(m0, m1, nmat, 2, shape, gw, GW, n0, ntot);
  } else {
    seq = warp_seq(m0, m1, nmat, 2, shape, gw, GW, n0, ntot);
  }
  if constexpr (SCHED == 2) seq.make_dynamic(m0.dyn + 2, R.hist);
  int* const exits = m0.dyn + 3;
  int p_k = 0, p_it = seq.at(0), p_itn = seq.at(1), p_itnn = seq.at(2), p_c0 = 0, p_seq = 0;
  S2ItemDev Dp = current(desc(p_it)), Dpn = desc(p_itn);
  auto produce = [&](Pend& pd) {
    pd.nc = 0;
    pd.sec = 0;
#pragma unroll
    for (int i = 0; i < KP; i++) pd.idx[i] = 0;
    if (p_it >= ntot) return;
    const int nc = min(Dp.cc, Dp.ncols - p_c0);
    const int s = p_seq % NS;
    const MatDev& PM = p_it < n0 ? m0 : m1;
    if (lane == 0) {
      const uint32_t bytes = (uint32_t)(nc * Dp.ntp * ESZ);
      const T* src = (const T*)PM.ustore + Dp.soff + (int64_t)p_c0 * Dp.ntp;
      // no proxy fence: as in phase 1, the stage's previous contents were
      // loaded and consumed before the copy that overwrites them
      mbar_expect_tx(&R.bar[s], bytes);
      bulk_g2s_stream(R.buf + s * SB, src, bytes, &R.bar[s], l2_evict_first());
    }
#pragma unroll
    for (int i = 0; i < KP; i++) {
      const int k = lane + 32 * i;
      if (k < nc) pd.idx[i] = __ldg(&PM.midx[Dp.m0 + p_c0 + k]);
    }
    pd.nc = nc;
    pd.sec = p_it >= n0;
    p_seq++;
    p_c0 += nc;
    if (p_c0 >= Dp.ncols) {
      p_k++;
      p_it = p_itn;
      p_itn = p_itnn;
      p_itnn = seq.at(p_k + 2);
      p_c0 = 0;
      Dp = current(Dpn);
      Dpn = desc(p_itn);
    }
  };
  auto gather = [&](const Pend& pd, Acc* mu) {
    const Acc* zv = (const Acc*)(pd.sec ? m1.z : m0.z);
#pragma unroll
    for (int i = 0; i < KP; i++) {
      const int k = lane + 32 * i;
      const int mi = pd.idx[i];
      mu[i] = k < pd.nc ? (mi >= 0 ? __ldcg(&zv[mi]) : (Acc)__ldg(&x[-mi - 1])) : Acc(0);
    }
  };
  // FIFO of the chunks in flight, oldest first
  Pend fifo[NS];
#pragma unroll
  for (int q = 0; q < NS; q++) produce(fifo[q]);
  // factor copies and column indices are static data; z, x, the partials and
  // the loop flags belong to earlier kernels of the stream
  pdl_launch_dependents();
  pdl_wait_prior();
  if (m0.skip && __ldcg(m0.skip)) {
    drain<NS>(R.bar, 0, p_seq);
    dyn_leave(seq, exits, GW);
    return;
  }
  Acc mu[KP], mu2[KP];
  gather(fifo[0], mu);
  if constexpr (GA == 2) gather(fifo[1], mu2);
  int c_k = 0, c_it = seq.at(0), c_i1 = seq.at(1), c_i2 = seq.at(2), c_c0 = 0, c_seq = 0;
  S2ItemDev Dc = current(desc(c_it)), Dn = desc(c_i1);
  Acc acc[VEC];
#pragma unroll
  for (int v = 0; v < VEC; v++) acc[v] = 0;
  while (c_it < ntot) {
    const bool sec = c_it >= n0;
    const MatDev& M = sec ? m1 : m0;
    const int s = c_seq % NS;
    if (!stage_ready(&R.bar[s], (uint32_t)((c_seq / NS) & 1), M.err, M.wait)) {
      drain<NS>(R.bar, c_seq, p_seq);
      dyn_leave(seq, exits, GW);
      return;
    }
    const int nc = min(Dc.cc, Dc.ncols - c_c0);
    const T* st = (const T*)(R.buf + s * SB);
    // this chunk's multipliers to shared memory; start the next chunk's gather
#pragma unroll
    for (int i = 0; i < KP; i++) musm[lane + 32 * i] = mu[i];
    __syncwarp();
    if constexpr (GA == 2) {
#pragma unroll
      for (int i = 0; i < KP; i++) mu[i] = mu2[i];
      gather(fifo[2], mu2);
    } else {
      gather(fifo[1], mu);
    }
    const int nq = Dc.ntp / VEC;
    const int lw = log2ceil(nq), LW = 1 << lw, CS = 32 >> lw;
    const int slot = lane >> lw, j = lane & (LW - 1);
    if (nq == 32 && nc == 16) {
      // a full chunk of full-height segments (16 columns of 512 bytes): the
      // same sums as below, unrolled, the multipliers read as 16-byte vectors
      Acc acc2[VEC], m16[16];
#pragma unroll
      for (int v = 0; v < VEC; v++) acc2[v] = 0;
#pragma unroll
      for (int c = 0; c < 16; c += 16 / sizeof(Acc)) {
        if constexpr (sizeof(Acc) == 4) {
          const float4 q = reinterpret_cast<const float4*>(musm)[c / 4];
          m16[c] = q.x;
          m16[c + 1] = q.y;
          m16[c + 2] = q.z;
          m16[c + 3] = q.w;
        } else {
          const double2 q = reinterpret_cast<const double2*>(musm)[c / 2];
          m16[c] = q.x;
          m16[c + 1] = q.y;
        }
      }
      const T* sj = st + j * VEC;
#pragma unroll
      for (int c = 0; c < 16; c += 2) {
        Acc a[VEC], b[VEC];
        lds16(sj + c * (32 * VEC), a);
        lds16(sj + (c + 1) * (32 * VEC), b);
#pragma unroll
        for (int v = 0; v < VEC; v++) {
          acc[v] += a[v] * m16[c];
          acc2[v] += b[v] * m16[c + 1];
        }
      }
#pragma unroll
      for (int v = 0; v < VEC; v++) acc[v] += acc2[v];
    } else if (j < nq) {
      // two accumulator sets over alternating columns: independent FMA chains
      Acc acc2[VEC];
#pragma unroll
      for (int v = 0; v < VEC; v++) acc2[v] = 0;
      int r0 = 0;
      for (; r0 + 2 * CS <= nc; r0 += 2 * CS) {
        const int sg = r0 + slot;
        const Acc mu0 = musm[sg], mu1 = musm[sg + CS];
        Acc a[VEC], b[VEC];
        lds16(st + sg * Dc.ntp + j * VEC, a);
        lds16(st + (sg + CS) * Dc.ntp + j * VEC, b);
#pragma unroll
        for (int v = 0; v < VEC; v++) {
          acc[v] += a[v] * mu0;
          acc2[v] += b[v] * mu1;
        }
      }
      for (; r0 < nc; r0 += CS) {
        const int sg = r0 + slot;
        if (sg < nc) {
          const Acc m = musm[sg];
          Acc a[VEC];
          lds16(st + sg * Dc.ntp + j * VEC, a);
#pragma unroll
          for (int v = 0; v < VEC; v++) acc[v] += a[v] * m;
        }
      }
#pragma unroll
      for (int v = 0; v < VEC; v++) acc[v] += acc2[v];
    }
    __syncwarp();
    c_seq++;
#pragma unroll
    for (int q = 0; q + 1 < NS; q++) fifo[q] = fifo[q + 1];
    produce(fifo[NS - 1]);
    c_c0 += nc;
    if (c_c0 < Dc.ncols) continue;
    // item done: combine the column slots, write the tile's rows
#pragma unroll
    for (int v = 0; v < VEC; v++)
      for (int o = LW; o < 32; o <<= 1) acc[v] += __shfl_xor_sync(0xffffffffu, acc[v], o);
    if (slot == 0 && j < nq) {
      Acc* gp = (Acc*)M.gpart + Dc.pout;
#pragma unroll
      for (int v = 0; v < VEC; v++)
        if (j * VEC + v < Dc.nr) gp[j * VEC + v] = acc[v];
    }
#pragma unroll
    for (int v = 0; v < VEC; v++) acc[v] = 0;
    c_k++;
    c_it = c_i1;
    c_i1 = c_i2;
    c_i2 = seq.at(c_k + 2);
    c_c0 = 0;
    Dc = current(Dn);
    Dn = desc(c_i1);
  }
  dyn_leave(seq, exits, GW);
}

// ------------------------------------------------------ store conversion
// one warp per column segment: dst[r'] = (T) body[src + r * stride], r < len,
// with r' the row's place under the segment's vector swizzle
template <typename T>
__global__ void segcopy_kernel(const double* __restrict__ body, const SegCopyDev* __restrict__ map, int64_t nmap,
                               T* __restrict__ dst) {
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t nw = (gridDim.x * (int64_t)blockDim.x) >> 5;
  for (int64_t q = w; q < nmap; q += nw) {
    const SegCopyDev c = map[q];
    constexpr int VEC = 16 / sizeof(T);
    for (int r = lane; r < c.len; r += 32) {
      const double v = body[c.src + (int64_t)r * c.stride];
      const int64_t d = c.dst + ((r / VEC) ^ c.swz) * VEC + r % VEC;
      if constexpr (sizeof(T) == 8) dst[d] = v;
      else if constexpr (sizeof(T) == 4) dst[d] = (float)v;
      else dst[d] = __double2bfloat16(v);
    }
  }
}

// ------------------------------------------------------------- launchers
namespace {

// warps per block, stages per warp and stage bytes (one block per SM); the
// block's shared memory: NW x NS x SB + multipliers + barriers
template <int NW, int NS, int SB>
constexpr size_t smem_bytes() {
  return (size_t)NW * NS * SB + (size_t)NW * kMu + (size_t)NW * NS * 8 + (size_t)NW * kHist * 4 + 16;
}

template <typename K>
void set_smem_once(K kernel, size_t bytes) {
  static std::mutex mu;
  static const void* done[64];
  static int ndone = 0;
  std::lock_guard<std::mutex> lock(mu);
  for (int i = 0; i < ndone; i++)
    if (done[i] == (const void*)kernel) return;
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (ndone < 64) done[ndone++] = (const void*)kernel;
}

// HBI_STREAM_SHAPE1=s / HBI_STREAM_SHAPE2=s force launch shape s of phase 1 /
// phase 2 for every operator
int env_shape(int phase) {
  static int shape[2] = {-2, -2};
  int& v = shape[phase - 1];
  if (v == -2) {
    const char* e = getenv(phase == 1 ? "HBI_STREAM_SHAPE1" : "HBI_STREAM_SHAPE2");
    v = e ? atoi(e) : -1;
    if (v < -1 || v >= num_shapes(phase)) v = -1;
  }
  return v;
}

template <typename T, int S>
void launch_p1s(const MatDev& m0, const MatDev& m1, int nmat, const double* x, int sm, int n, cudaStream_t st) {
  constexpr int NW = kShapes1[S].nw, NS = kShapes1[S].ns, SB = kShapes1[S].sb, MAP = kShapes1[S].map;
  const int need = (n + NW - 1) / NW;
  const int grid = need < sm ? (need > 0 ? need : 1) : sm;
  // phase 1 starts after its predecessor has completed (no programmatic
  // launch): a phase-1 block needs nearly all of an SM's registers, and one
  // started early would keep the rest of the previous stage's phase-3 blocks
  // off its SM
  launch_kernel(p1_stream_kernel<T, NW, NS, SB, MAP, kShapes1[S].sched>, dim3(grid), dim3(NW * 32),
                smem_bytes<NW, NS, SB>(), st, false, m0, m1, nmat, x, S);
}

template <typename T, int S>
void launch_p2s(const MatDev& m0, const MatDev& m1, int nmat, const double* x, int sm, int n, cudaStream_t st) {
  constexpr int NW = kShapes2[S].nw, NS = kShapes2[S].ns, SB = kShapes2[S].sb, GA = kShapes2[S].map + 1;
  const int need = (n + NW - 1) / NW;
  const int grid = need < sm ? (need > 0 ? need : 1) : sm;
  launch_kernel(p2_stream_kernel<T, NW, NS, SB, GA, kShapes2[S].sched>, dim3(grid), dim3(NW * 32),
                smem_bytes<NW, NS, SB>(), st, pdl_enabled(), m0, m1, nmat, x, S);
}

template <typename T>
void launch_typed(int phase, int shape, const MatDev& m0, const MatDev& m1, int nmat, const double* x, int sm,
                  cudaStream_t st) {
  const int n = phase == 1 ? m0.ns1 + (nmat == 2 ? m1.ns1 : 0) : m0.ns2 + (nmat == 2 ? m1.ns2 : 0);
  if (n == 0) return;
  static_assert(kNumShapes1 == 10 && kNumShapes2 == 8, "one case per shape");
  if (phase == 1) {
    switch (shape) {
      case 1: launch_p1s<T, 1>(m0, m1, nmat, x, sm, n, st); break;
      case 2: launch_p1s<T, 2>(m0, m1, nmat, x, sm, n, st); break;
      case 3: launch_p1s<T, 3>(m0, m1, nmat, x, sm, n, st); break;
      case 4: launch_p1s<T, 4>(m0, m1, nmat, x, sm, n, st); break;
      case 5: launch_p1s<T, 5>(m0, m1, nmat, x, sm, n, st); break;
      case 6: launch_p1s<T, 6>(m0, m1, nmat, x, sm, n, st); break;
      case 7: launch_p1s<T, 7>(m0, m1, nmat, x, sm, n, st); break;
      case 8: launch_p1s<T, 8>(m0, m1, nmat, x, sm, n, st); break;
      case 9: launch_p1s<T, 9>(m0, m1, nmat, x, sm, n, st); break;
      default: launch_p1s<T, 0>(m0, m1, nmat, x, sm, n, st);
    }
  } else {
    switch (shape) {
      case 1: launch_p2s<T, 1>(m0, m1, nmat, x, sm, n, st); break;
      case 2: launch_p2s<T, 2>(m0, m1, nmat, x, sm, n, st); break;
      case 3: launch_p2s<T, 3>(m0, m1, nmat, x, sm, n, st); break;
      case 4: launch_p2s<T, 4>(m0, m1, nmat, x, sm, n, st); break;
      case 5: launch_p2s<T, 5>(m0, m1, nmat, x, sm, n, st); break;
      case 6: launch_p2s<T, 6>(m0, m1, nmat, x, sm, n, st); break;
      case 7: launch_p2s<T, 7>(m0, m1, nmat, x, sm, n, st); break;
      default: launch_p2s<T, 0>(m0, m1, nmat, x, sm, n, st);
    }
  }
}

template <typename T, int S>
void prepare_p1() {
  constexpr int NW = kShapes1[S].nw, NS = kShapes1[S].ns, SB = kShapes1[S].sb, MAP = kShapes1[S].map;
  static_assert(smem_bytes<NW, NS, SB>() <= 227 * 1024, "shape exceeds the shared memory of a block");
  set_smem_once(p1_stream_kernel<T, NW, NS, SB, MAP, kShapes1[S].sched>, smem_bytes<NW, NS, SB>());
}

template <typename T, int S>
void prepare_p2() {
  constexpr int NW = kShapes2[S].nw, NS = kShapes2[S].ns, SB = kShapes2[S].sb, GA = kShapes2[S].map + 1;
  static_assert(smem_bytes<NW, NS, SB>() <= 227 * 1024, "shape exceeds the shared memory of a block");
  set_smem_once(p2_stream_kernel<T, NW, NS, SB, GA, kShapes2[S].sched>, smem_bytes<NW, NS, SB>());
}

template <typename T>
void prepare_type() {
  prepare_p1<T, 0>();
  prepare_p1<T, 1>();
  prepare_p1<T, 2>();
  prepare_p1<T, 3>();
  prepare_p1<T, 4>();
  prepare_p1<T, 5>();
  prepare_p1<T, 6>();
  prepare_p1<T, 7>();
  prepare_p1<T, 8>();
  prepare_p1<T, 9>();
  prepare_p2<T, 0>();
  prepare_p2<T, 1>();
  prepare_p2<T, 2>();
  prepare_p2<T, 3>();
  prepare_p2<T, 4>();
  prepare_p2<T, 5>();
  prepare_p2<T, 6>();
  prepare_p2<T, 7>();
}

}  // namespace

int forced_stream_shape(int phase) { return env_shape(phase); }

bool pdl_enabled() {
  static int on = -1;
  if (on < 0) {
    const char* e = getenv("HBI_PDL");
    on = (e && e[0] == '1') ? 1 : 0;
  }
  return on == 1;
}

// the large shared-memory opt-in of the phase kernels, once per process and
// before any stream capture
void prepare_stream_kernels() {
  prepare_type<double>();
  prepare_type<float>();
  prepare_type<__nv_bfloat16>();
}

void launch_phase_shape(int phase, int shape, const MatDev* mats, int nmat, const double* x, int sm, cudaStream_t st) {
  const MatDev& m0 = mats[0];
  const MatDev& m1 = nmat == 2 ? mats[1] : mats[0];
  if (m0.storage == ST_F64) launch_typed<double>(phase, shape, m0, m1, nmat, x, sm, st);
  else if (m0.storage == ST_F32) launch_typed<float>(phase, shape, m0, m1, nmat, x, sm, st);
  else launch_typed<__nv_bfloat16>(phase, shape, m0, m1, nmat, x, sm, st);
}

// both H-matrices of a stage in one grid per phase (same storage type), in
// the launch shape chosen for the first
void launch_phase1(const MatDev* mats, int nmat, const double* x, int sm, cudaStream_t st) {
  launch_phase_shape(1, mats[0].shape1, mats, nmat, x, sm, st);
}

void launch_phase2(const MatDev* mats, int nmat, const double* x, int sm, cudaStream_t st) {
  launch_phase_shape(2, mats[0].shape2, mats, nmat, x, sm, st);
}

void launch_segcopy(const double* body, const SegCopyDev* map, int64_t nmap, void* dst, int storage,
                    cudaStream_t st) {
  if (nmap == 0) return;
  const int blocks = (int)std::min<int64_t>((nmap + 7) / 8, 152 * 16);
  if (storage == ST_F64) segcopy_kernel<double><<<blocks, 256, 0, st>>>(body, map, nmap, (double*)dst);
  else if (storage == ST_F32) segcopy_kernel<float><<<blocks, 256, 0, st>>>(body, map, nmap, (float*)dst);
  else segcopy_kernel<__nv_bfloat16><<<blocks, 256, 0, st>>>(body, map, nmap, (__nv_bfloat16*)dst);
}

}  // namespace hbi
