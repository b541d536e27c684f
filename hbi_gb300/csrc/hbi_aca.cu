// hbi_aca.cu -- batched ACA+ low-rank assembly and dense near-field fill:
// the launchers per problem kind and the problem-independent kernels.  The
// kernels themselves are in hbi_aca_impl.cuh; the Okada and triangular
// problems are instantiated in their own translation units.
#include <cstdint>

#include "hbi_aca_impl.cuh"

namespace hbi {

HBI_PROBLEM_LAUNCHERS(P_2DVS, 2dvs)
HBI_PROBLEM_LAUNCHERS(P_2DPH, 2dph)
HBI_PROBLEM_LAUNCHERS(P_2DN, 2dn)
HBI_DECLARE_PROBLEM_LAUNCHERS(3dph)
HBI_DECLARE_PROBLEM_LAUNCHERS(3dnr)
HBI_DECLARE_PROBLEM_LAUNCHERS(3dnt)
HBI_DECLARE_PROBLEM_LAUNCHERS(3dht)

// copy kt columns of V (zab) then U (zaa) of each task into a compact block
// in HACApK's packing: [a1 = V (ndt x kt)][a2 = U (ndl x kt)]
__global__ void aca_compact_kernel(const AcaTask* tasks, const int* kt, const int64_t* dst_off, const double* arena,
                                   double* dst) {
  const AcaTask T = tasks[blockIdx.x];
  const int k = kt[blockIdx.x];
  if (k <= 0) return;
  const double* zaa = arena + T.scratch;
  const double* zab = zaa + (size_t)T.ndl * T.kcap;
  double* o = dst + dst_off[blockIdx.x];
  const int64_t nv = (int64_t)T.ndt * k, nu = (int64_t)T.ndl * k;
  for (int64_t e = threadIdx.x; e < nv; e += blockDim.x) o[e] = zab[e];
  for (int64_t e = threadIdx.x; e < nu; e += blockDim.x) o[nv + e] = zaa[e];
}

__global__ void copy_segments_kernel(const double* const* src, const int64_t* dst_off, const int64_t* len, int nseg,
                                     double* dst) {
  for (int sg = blockIdx.x; sg < nseg; sg += gridDim.x) {
    const double* s = src[sg];
    double* d = dst + dst_off[sg];
    const int64_t n = len[sg];
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) d[e] = s[e];
  }
}

void launch_copy_segments(const double* const* src, const int64_t* dst_off, const int64_t* len, int nseg,
                          double* dst, cudaStream_t st) {
  if (nseg <= 0) return;
  copy_segments_kernel<<<nseg < 152 * 16 ? nseg : 152 * 16, 256, 0, st>>>(src, dst_off, len, nseg, dst);
}

#define HBI_DISPATCH(CALL, ...)                 \
  switch (b.problem) {                          \
    case P_2DVS: CALL##_2dvs(__VA_ARGS__); break; \
    case P_3DPH: CALL##_3dph(__VA_ARGS__); break; \
    case P_3DNR: CALL##_3dnr(__VA_ARGS__); break; \
    case P_3DNT: CALL##_3dnt(__VA_ARGS__); break; \
    case P_2DPH: CALL##_2dph(__VA_ARGS__); break; \
    case P_2DN: CALL##_2dn(__VA_ARGS__); break;   \
    case P_3DHT: CALL##_3dht(__VA_ARGS__); break; \
  }

void launch_aca(const DevBemv& b, const int* lod, const AcaTask* tasks, int ntask, double* arena, int* result,
                const AcaParams& P, cudaStream_t st) {
  HBI_DISPATCH(launch_aca, b, lod, tasks, ntask, arena, result, P, st)
}

void launch_aca_compact(const AcaTask* tasks, int ntask, const int* kt, const int64_t* dst_off, const double* arena,
                        double* dst, cudaStream_t st) {
  aca_compact_kernel<<<ntask, 256, 0, st>>>(tasks, kt, dst_off, arena, dst);
}

void launch_dense_fill(const DevBemv& b, const int* lod, const DenseTask* tasks, int ntask, const int64_t* task_start,
                       int64_t total, double* store, cudaStream_t st) {
  if (total <= 0) return;
  int64_t blocks = (total + 255) / 256;
  if (blocks > 152 * 64) blocks = 152 * 64;
  HBI_DISPATCH(launch_dense_fill, b, lod, tasks, ntask, task_start, total, store, (int)blocks, st)
}

void launch_entries(const DevBemv& b, const int* ii, const int* jj, int n, double* out, cudaStream_t st) {
  if (n <= 0) return;
  const int blocks = (n + 127) / 128;
  HBI_DISPATCH(launch_entries, b, ii, jj, n, out, blocks, st)
}

}  // namespace hbi
