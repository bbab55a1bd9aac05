// lookup_unionized.cu -- lookup kernels instantiated for the unionized grid type.
#include "lookup_kernels.cuh"

namespace xsgb {
XSGB_DEFINE_GRID(unionized, XS_UNIONIZED)
}  // namespace xsgb
