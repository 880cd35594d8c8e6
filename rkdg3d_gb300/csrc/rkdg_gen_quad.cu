// Generic kernel instantiations for geometry 3 (quad).
#include "rkdg_inst.cuh"

namespace rkdg {
RKDG_INSTANTIATE(3, 1)
RKDG_INSTANTIATE(3, 2)
RKDG_INSTANTIATE(3, 3)
}  // namespace rkdg
