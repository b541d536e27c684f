// hbi_aca_td.cu -- ACA+, dense fill and entry kernels for triangular dislocations in a full space
// (kernels in hbi_aca_impl.cuh).
#include "hbi_aca_impl.cuh"

namespace hbi {

HBI_PROBLEM_LAUNCHERS(P_3DNT, 3dnt)

}  // namespace hbi
