// lookup_hash.cu -- lookup kernels instantiated for the hash grid type.
#include "lookup_kernels.cuh"

namespace xsgb {
XSGB_DEFINE_GRID(hash, XS_HASH)
}  // namespace xsgb
