// hbi_kernels.cuh -- device-side task records and kernel launchers shared by
// the C ABI (hbi_capi.cu) and the kernel translation units.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "hbi_entries.cuh"
#include "hbi_structure.hpp"

#ifndef HBI_ACA_NT
#define HBI_ACA_NT 128
#endif

namespace hbi {

// ---- assembly ------------------------------------------------------------
struct AcaTask {
  int ndl, ndt, nstrtl, nstrtt, kcap, leaf;
  int64_t scratch;  // element offset of this task's scratch in the arena
};
struct DenseTask {
  int ndl, ndt, nstrtl, nstrtt;
  int64_t off;  // element offset in the FP64 store (a1(ndt,ndl))
};
struct AcaParams {
  double eps, pACA_EPS, znrmmat, kmin;
  int kmax;
};
inline int64_t aca_scratch_elems(int ndl, int ndt, int kcap) {
  // zaa, zab, pa_ref, pb_ref (doubles) + two int masks (rounded to doubles)
  return (int64_t)(ndl + ndt) * kcap + (ndl + ndt) + ((int64_t)(ndl + ndt) + 1) / 2 + 2;
}

void launch_aca(const DevBemv& b, const int* lod, const AcaTask* tasks, int ntask, double* arena, int* result,
                const AcaParams& P, cudaStream_t st);
void launch_aca_compact(const AcaTask* tasks, int ntask, const int* kt, const int64_t* dst_off, const double* arena,
                        double* dst, cudaStream_t st);
void launch_dense_fill(const DevBemv& b, const int* lod, const DenseTask* tasks, int ntask, const int64_t* task_start,
                       int64_t total, double* store, cudaStream_t st);
void launch_entries(const DevBemv& b, const int* ii, const int* jj, int n, double* out, cudaStream_t st);

// ---- matvec ----------------------------------------------------------------
enum { ST_F64 = 0, ST_F32 = 1, ST_BF16 = 2 };

// bound of the product kernels' bulk-copy waits: about one second of SM clock
constexpr long long kWaitCyclesDefault = 2LL << 30;

// Launch shapes of the phase kernels: warps per block (one block per SM),
// shared-memory stages per warp and bytes per stage, a variant -- for phase
// 1 the lane mapping (0: the lanes of a column segment split its rows and
// reduce by shuffles; 1: one lane per column, no cross-lane reduction), for
// phase 2 how far ahead the multipliers are gathered (0: one chunk, 1: two)
// -- and the schedule (0: the phase's items dealt over all warps longest
// first, statically; 1: each block a run of items consecutive in the store,
// plan_block_schedule; 2: dynamic, every warp takes the next item, longest
// first, from a global counter when it needs one; 3: the items dealt over
// the blocks longest first, and each block's warps take its items from a
// shared-memory counter).  Every shape is compiled for every storage type;
// hbi_construct_lh times them on the operator and keeps the fastest per
// phase (autotune_stream_shapes).  Shape 0 of each phase is the default.
struct StreamShape {
  int nw, ns, sb, map, sched;
};
constexpr int kNumShapes1 = 10, kNumShapes2 = 8, kMaxShapes = 10;
constexpr StreamShape kShapes1[kNumShapes1] = {{12, 2, 8192, 0, 0}, {8, 3, 8192, 0, 0}, {6, 2, 16384, 0, 0},
                                               {12, 2, 8192, 1, 0}, {8, 3, 8192, 1, 0}, {6, 2, 16384, 1, 0},
                                               {12, 2, 8192, 1, 1}, {12, 2, 8192, 0, 1}, {12, 2, 8192, 1, 2},
                                               {12, 2, 8192, 1, 3}};
constexpr StreamShape kShapes2[kNumShapes2] = {{12, 2, 8192, 0, 0}, {8, 3, 8192, 0, 0}, {6, 2, 16384, 0, 0},
                                               {10, 2, 8192, 0, 0}, {8, 3, 8192, 1, 0}, {12, 2, 8192, 0, 1},
                                               {12, 2, 8192, 0, 2}, {12, 2, 8192, 0, 3}};
inline const StreamShape& stream_shape(int phase, int s) { return phase == 1 ? kShapes1[s] : kShapes2[s]; }
inline int num_shapes(int phase) { return phase == 1 ? kNumShapes1 : kNumShapes2; }

// Programmatic dependent launch of the product chain (phase 1 -> phase 2 ->
// phase 3; phase 1 itself starts after its predecessor has completed): a
// kernel launched with the programmatic stream-serialization attribute may
// start while its predecessor drains; it first does what depends on nothing
// the predecessors write (barrier set-up, the schedule, the first bulk copies
// of factor data), then waits for the predecessor grid to complete
// (pdl_wait_prior; transitively all earlier kernels of the stream).
// pdl_launch_dependents lets the next grid start as soon as this grid's SMs
// free up.  Both are no-ops in a grid launched without the attribute.
// Off by default (a Cash-Karp attempt on the 65,536-element Okada plane took
// 1.559 ms with it, 1.423 ms without); HBI_PDL=1 turns it on.
__device__ __forceinline__ void pdl_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait_prior() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
bool pdl_enabled();

// kernel launch, with the programmatic stream-serialization attribute when pdl
template <typename... KArgs, typename... Args>
cudaError_t launch_kernel(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, bool pdl,
                          Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k, args...);
}

// work items of the streamed product (plan_stream in hbi_structure.cpp)
typedef S1Item S1ItemDev;
typedef S2Item S2ItemDev;
typedef SegCopy SegCopyDev;

struct MatDev {            // one H-matrix on the device
  int n;
  int storage;             // element type of the stores (ST_*)
  const void* vstore;      // phase-1 store: V tiles of the column groups
  const void* ustore;      // phase-2 store: U / A tiles of the row groups
  const S1ItemDev* s1;
  int ns1;
  const S2ItemDev* s2;
  int ns2;
  int* cnt;                // phase-1 column-chunk arrival counters (self-resetting)
  void* part;              // phase-1 per-tile partial column sums (Acc type)
  void* z;                 // z = V^T x per low-rank column (Acc type)
  const int32_t* midx;     // phase-2 column multipliers: z index, or -(x index)-1
  void* gpart;             // phase-2 partial row sums (Acc type)
  // phase 3: rows -> covering row groups -> their column chunks
  const int32_t *grow0, *gndl, *gnch, *gpoff;
  const int32_t *row_fc, *fc_ptr, *fc_group;
  const int32_t *fcb_ptr, *fcb_base;  // per fine range: gpart offsets (+ row) of its non-empty groups
  double scale;            // result multiplier (1/ds0 for 3dph, else 1)
  const int* skip;         // when non-null and nonzero, phases 1-2 do nothing
  int* err;                // set to nonzero when a bulk copy did not arrive in time
  long long wait;          // bound of a stage wait in SM clock cycles (0: every wait gives up at once)
  int ncnt;                // number of arrival counters in cnt
  int* dyn;                // dynamic schedules: [2 (phase - 1)] items taken, [2 (phase - 1) + 1] warps done
  // static warp schedules (hbi_structure.hpp, plan_warp_schedule), one per
  // launch shape s, for a grid of gw1[s] / gw2[s] warps: warp w walks
  // item[off[w] .. off[w+1]) of its phase
  const int32_t *w1off[kNumShapes1], *w1item[kNumShapes1], *w2off[kNumShapes2], *w2item[kNumShapes2];
  int gw1[kNumShapes1], gw2[kNumShapes2];
  int shape1, shape2;      // launch shapes of phases 1 and 2 (indices into kShapes1 / kShapes2)
};

// RK (Cash-Karp) stage state on the device; all arrays in cluster order
struct RkDev {
  int n, nmat, evlaw, backslip, limitsigma;
  double vref, minsig, maxsig, rigid_over_2vs;
  const double *a, *b, *dc, *f0, *taudot, *sigdot, *vpl;
  double* y;       // accepted state (3n): psi,tau,sigma interleaved
  double* ys;      // stage state (3n)
  double* vs;      // slip rate of the stage state (n)
  double* ws;      // 2 vref e^(-psi/a) cosh(tau/(sigma a)) of the stage state (n)
  double* x0;      // matvec input of stage 0 (n)
  double* xb[2];   // ping-pong matvec inputs of stages 1..5 (n)
  double* K;       // stage derivatives, 6 x 3n
  double* yout;    // 5th-order solution (3n)
  double* yerr;    // embedded error (3n)
  double* ebuf;    // |yerr/yout|/eps per component (3n)
  double* ctl;     // [0]=h [1]=eps  [2]=emax (as bits) [3]=huge index (as int64)
  // time-loop flags (null outside the device-resident loop): [0] halted,
  // [1] halted or retrying, [2] retrying the same state (stage 1 is reused)
  const int* flags;
};

// host view of an operator, for the ensemble (hbi_ens.cu)
struct LhpView {
  MatDev md;
  int n, storage, sm;
  int64_t zlen, plen1, plen2, ncg;
  const std::vector<Leaf>* leaves;
};

// host view of an RK handle, for the device-resident time loop (hbi_cycle.cu)
struct RkView {
  RkDev R;
  MatDev mats[2];
  int nmat, n, sm;
};

// phase 1: z = V^T x; phase 2: per-group row partials of U z + A x;
// phase 3: per-row sum of the group partials (plain, or with the RK epilogue)
void launch_segcopy(const double* body, const SegCopyDev* map, int64_t nmap, void* dst, int storage,
                    cudaStream_t st);
void prepare_stream_kernels();
// the shape index of `phase` forced by HBI_STREAM_SHAPE1 / HBI_STREAM_SHAPE2, or -1
int forced_stream_shape(int phase);
// one phase (1 or 2) of the product with launch shape `shape` (the grid of
// m0's schedule for it; m1, when nmat == 2, has one for the same shape)
void launch_phase_shape(int phase, int shape, const MatDev* mats, int nmat, const double* x, int sm_count,
                        cudaStream_t st);
void launch_phase1(const MatDev* mats, int nmat, const double* x, int sm_count, cudaStream_t st);
void launch_phase2(const MatDev* mats, int nmat, const double* x, int sm_count, cudaStream_t st);
void launch_phase3_plain(const MatDev* mats, int nmat, double* const* y, cudaStream_t st);
void launch_phase3_rk(const MatDev* mats, int nmat, const RkDev& rk, int stage, double* xnext, cudaStream_t st);
// host: 1 when a product kernel of the operator gave up a wait since the last
// call (the operator's error word and arrival counters are then cleared, on
// the legacy stream: the caller has synchronised the products), 0 if not, a
// negative HBI_ERR_CUDA on a failed copy
int take_device_error(const MatDev& m);
void launch_rk_prepare(const RkDev& rk, cudaStream_t st);
void set_tableau(const double* B15, const double* C6, const double* DC6);
// dst[dst_off[i] : +len[i]] = src[i][0 : len[i]]
void launch_copy_segments(const double* const* src, const int64_t* dst_off, const int64_t* len, int nseg,
                          double* dst, cudaStream_t st);


}  // namespace hbi
