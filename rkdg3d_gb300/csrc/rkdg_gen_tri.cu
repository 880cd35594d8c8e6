// Generic kernel instantiations for geometry 2 (tri).
#include "rkdg_inst.cuh"

namespace rkdg {
RKDG_INSTANTIATE(2, 1)
RKDG_INSTANTIATE(2, 2)
}  // namespace rkdg
