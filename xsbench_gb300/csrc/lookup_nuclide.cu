// lookup_nuclide.cu -- lookup kernels instantiated for the nuclide grid type.
#include "lookup_kernels.cuh"

namespace xsgb {
XSGB_DEFINE_GRID(nuclide, XS_NUCLIDE)
}  // namespace xsgb
