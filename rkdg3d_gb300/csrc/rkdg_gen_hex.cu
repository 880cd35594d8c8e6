// Hexahedra: sum-factorised right-hand side kernels (rkdg_hex.cuh) plus the
// generic limiter and cell-mean kernels.
#include "rkdg_hex.cuh"
#include "rkdg_inst.cuh"

namespace rkdg {

template <int P, typename R>
static cudaError_t launch_hex_sf(const RhsParams& prm, const R* u, const EpiParams<R>& ep,
                                 cudaStream_t st) {
  using S = HexSize<P>;
  const size_t smem = S::template smem_bytes<R>();
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_rhs_hex_sf<P, R>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  const int grid = (prm.ne + S::EPB - 1) / S::EPB;
  k_rhs_hex_sf<P, R><<<grid, 32 * S::EPB, smem, st>>>(prm, u, ep);
  return cudaGetLastError();
}

template <>
cudaError_t launch_rhs_t<5, 1>(int prec, const RhsParams& prm, const void* u, const void* ep,
                               cudaStream_t st) {
  if (prec == 0)
    return launch_hex_sf<1, double>(prm, (const double*)u, *(const EpiParams<double>*)ep, st);
  return launch_hex_sf<1, float>(prm, (const float*)u, *(const EpiParams<float>*)ep, st);
}
template <>
cudaError_t launch_rhs_t<5, 2>(int prec, const RhsParams& prm, const void* u, const void* ep,
                               cudaStream_t st) {
  if (prec == 0)
    return launch_hex_sf<2, double>(prm, (const double*)u, *(const EpiParams<double>*)ep, st);
  return launch_hex_sf<2, float>(prm, (const float*)u, *(const EpiParams<float>*)ep, st);
}

template cudaError_t launch_limit_t<5, 1>(int, const LimParams&, void*, float*, cudaStream_t);
template cudaError_t launch_limit_t<5, 2>(int, const LimParams&, void*, float*, cudaStream_t);
template cudaError_t launch_means_t<5, 1>(int, int, long long, const RefTables*, const void*,
                                          const float*, double*, cudaStream_t);
template cudaError_t launch_means_t<5, 2>(int, int, long long, const RefTables*, const void*,
                                          const float*, double*, cudaStream_t);

}  // namespace rkdg
