// Generic kernel instantiations for geometry 5 (hex).
#include "rkdg_inst.cuh"

namespace rkdg {
RKDG_INSTANTIATE(5, 1)
RKDG_INSTANTIATE(5, 2)
}  // namespace rkdg
