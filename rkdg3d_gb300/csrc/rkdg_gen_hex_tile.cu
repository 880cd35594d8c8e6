// Hexahedra: the face-once tiled right-hand-side kernel (rkdg_hex_tile.cuh),
// in its own translation unit so that it compiles next to the team kernels.
#include "rkdg_hex_tile.cuh"
#include "rkdg_launch.h"

namespace rkdg {

template <int P, typename R>
static cudaError_t launch_tile(const RhsParams& prm, const R* u, const EpiParams<R>& ep,
                               cudaStream_t st) {
  using S = TileSize<P>;
  if (prm.tile_hs < 1 || prm.tile_hs > RKDG_TILE_HMAX + 1) return cudaErrorInvalidValue;
  const size_t smem = S::template smem_bytes<R>(prm.tile_hs);
  static bool configured = false;
  if (!configured) {  // room for the largest halo stride
    cudaError_t e = cudaFuncSetAttribute(k_rhs_hex_tile<P, R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)S::template smem_bytes<R>(RKDG_TILE_HMAX + 1));
    if (e != cudaSuccess) return e;
    configured = true;
  }
  k_rhs_hex_tile<P, R><<<prm.ntile, S::NT, smem, st>>>(prm, u, ep);
  return cudaGetLastError();
}

// Tensor-core variant (FP32, P = 2): three CTAs per SM (66 KB of shared
// memory each) and 64 tensor-memory columns per CTA.
static cudaError_t launch_tile_tc(const RhsParams& prm, const float* u, const EpiParams<float>& ep,
                                  cudaStream_t st) {
  using S = TileSize<2>;
  if (prm.tile_hs < 1 || prm.tile_hs > RKDG_TILE_HMAX + 1 || !prm.tcb) return cudaErrorInvalidValue;
  const size_t smem = S::smem_bytes_tc(prm.tile_hs);
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_rhs_hex_tile<2, float, true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)S::smem_bytes_tc(RKDG_TILE_HMAX + 1));
    if (e != cudaSuccess) return e;
    configured = true;
  }
  k_rhs_hex_tile<2, float, true><<<prm.ntile, S::NT, smem, st>>>(prm, u, ep);
  return cudaGetLastError();
}

cudaError_t launch_hex_tile_tc(const RhsParams& prm, const void* u, const void* ep, cudaStream_t st) {
  if (!prm.htile || prm.ntile <= 0) return cudaErrorInvalidValue;
  return launch_tile_tc(prm, (const float*)u, *(const EpiParams<float>*)ep, st);
}

cudaError_t launch_hex_tile(int p, int prec, const RhsParams& prm, const void* u, const void* ep,
                            cudaStream_t st) {
  if (!prm.htile || prm.ntile <= 0) return cudaErrorInvalidValue;
  if (p == 1)
    return prec == 0 ? launch_tile<1, double>(prm, (const double*)u, *(const EpiParams<double>*)ep, st)
                     : launch_tile<1, float>(prm, (const float*)u, *(const EpiParams<float>*)ep, st);
  if (p == 2)
    return prec == 0 ? launch_tile<2, double>(prm, (const double*)u, *(const EpiParams<double>*)ep, st)
                     : launch_tile<2, float>(prm, (const float*)u, *(const EpiParams<float>*)ep, st);
  return cudaErrorInvalidValue;
}

}  // namespace rkdg
