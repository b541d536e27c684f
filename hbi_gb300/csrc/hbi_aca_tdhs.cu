// hbi_aca_tdhs.cu -- ACA+, dense fill and entry kernels for triangular dislocations in a half space
// (kernels in hbi_aca_impl.cuh).
#include "hbi_aca_impl.cuh"

namespace hbi {

HBI_PROBLEM_LAUNCHERS(P_3DHT, 3dht)

}  // namespace hbi
