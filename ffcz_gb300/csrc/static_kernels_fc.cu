// Instantiations of the plain form's forward-with-clamp strided pass
// (MODE_FC) for every compile-time length, FP32 and FP64, in a translation
// unit of their own so the build stays parallel.
#include "static_inst.cuh"

namespace ffcz {

#define TT float
DEFINE_FC_LOOKUP(float, CASES_F32)
#undef TT
#define TT double
DEFINE_FC_LOOKUP(double, CASES_F64)
#undef TT

}  // namespace ffcz
