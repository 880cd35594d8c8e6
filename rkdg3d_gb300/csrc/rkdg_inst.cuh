// Explicit instantiation helpers for the generic kernels (one translation
// unit per geometry keeps the build parallel).
#pragma once

#include <algorithm>

#include "rkdg_generic.cuh"
#include "rkdg_launch.h"

namespace rkdg {

constexpr int kGenericBlock = 128;

// Threads per CTA: the tuned value (a multiple of 32 up to kGenericMaxBlock)
// or the default.
inline int generic_block(int b) {
  return (b >= 32 && b <= kGenericMaxBlock && b % 32 == 0) ? b : kGenericBlock;
}

template <int G, int P>
cudaError_t launch_rhs_t(int prec, const RhsParams& prm, const void* u, const void* ep,
                         cudaStream_t st) {
  constexpr int NVAL = El<G, P>::NEQ * El<G, P>::ND;
  const int blk = prec == 0 ? generic_block(prm.block)
                            : std::min(generic_block(prm.block), generic_max_block<float, NVAL>());
  const int grid = (prm.ne + blk - 1) / blk;
  if (prec == 0)
    k_rhs_generic<G, P, double><<<grid, blk, 0, st>>>(prm, (const double*)u,
                                                      *(const EpiParams<double>*)ep);
  else
    k_rhs_generic<G, P, float><<<grid, blk, 0, st>>>(prm, (const float*)u,
                                                     *(const EpiParams<float>*)ep);
  return cudaGetLastError();
}

template <int G, int P>
cudaError_t launch_limit_t(int mode, const LimParams& prm, void* u, float* ulo, cudaStream_t st) {
  constexpr int NVAL = El<G, P>::NEQ * El<G, P>::ND;
  const int blk = mode == 0 ? generic_block(prm.block)
                            : std::min(generic_block(prm.block), generic_max_block<float, NVAL>());
  const int grid = (prm.ne + blk - 1) / blk;
  if (mode == 0)
    k_limit_generic<G, P, double, false><<<grid, blk, 0, st>>>(prm, (double*)u, nullptr);
  else if (mode == 1)
    k_limit_generic<G, P, float, false><<<grid, blk, 0, st>>>(prm, (float*)u, nullptr);
  else
    k_limit_generic<G, P, float, true><<<grid, blk, 0, st>>>(prm, (float*)u, ulo);
  return cudaGetLastError();
}

template <int G, int P>
cudaError_t launch_means_t(int mode, int ne, long long ndofs, const RefTables* tab, const void* u,
                           const float* ulo, double* means, cudaStream_t st) {
  const int grid = (ne + kGenericBlock - 1) / kGenericBlock;
  if (mode == 0)
    k_means_generic<G, P, double><<<grid, kGenericBlock, 0, st>>>(ne, ndofs, tab, (const double*)u,
                                                                  nullptr, means);
  else
    k_means_generic<G, P, float><<<grid, kGenericBlock, 0, st>>>(
        ne, ndofs, tab, (const float*)u, mode == 2 ? ulo : nullptr, means);
  return cudaGetLastError();
}

#define RKDG_INSTANTIATE(G, P)                                                                 \
  template cudaError_t launch_rhs_t<G, P>(int, const RhsParams&, const void*, const void*,     \
                                          cudaStream_t);                                       \
  template cudaError_t launch_limit_t<G, P>(int, const LimParams&, void*, float*, cudaStream_t); \
  template cudaError_t launch_means_t<G, P>(int, int, long long, const RefTables*, const void*, \
                                            const float*, double*, cudaStream_t);

}  // namespace rkdg
