// FP64 instantiations of the register-resident pass kernels (lengths 16..2048
// and the mixed-radix lists of at most 12 values per thread).
#include "static_inst.cuh"

namespace ffcz {

#define TT double
DEFINE_LOOKUPS(double, CASES_F64)
#undef TT

}  // namespace ffcz
