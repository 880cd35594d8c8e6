// Generic kernel instantiations for geometry 3 (quad), orders 1 and 2; order 3
// is in rkdg_gen_quad3.cu so the two compile in parallel.
#include "rkdg_inst.cuh"

namespace rkdg {
RKDG_INSTANTIATE(3, 1)
RKDG_INSTANTIATE(3, 2)
}  // namespace rkdg
