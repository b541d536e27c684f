// hbi_aca_okada.cu -- ACA+, dense fill and entry kernels for Okada rectangles (half and full space)
// (kernels in hbi_aca_impl.cuh).
#include "hbi_aca_impl.cuh"

namespace hbi {

HBI_PROBLEM_LAUNCHERS(P_3DPH, 3dph)
HBI_PROBLEM_LAUNCHERS(P_3DNR, 3dnr)

}  // namespace hbi
