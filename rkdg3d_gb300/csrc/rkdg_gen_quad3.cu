// Generic kernel instantiations for geometry 3 (quad), order 3.
#include "rkdg_inst.cuh"

namespace rkdg {
RKDG_INSTANTIATE(3, 3)
}  // namespace rkdg
