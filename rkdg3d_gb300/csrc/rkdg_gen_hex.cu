// Hexahedra: register-resident team kernels (rkdg_hex_team.cuh) for the
// right-hand side, the warp-per-element sum-factorised kernel
// (rkdg_hex.cuh) for the FP64 path, plus the generic limiter and cell-mean
// kernels.
#include "rkdg_hex.cuh"
#include "rkdg_hex_team.cuh"
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

template <int P, typename R, int MODE>
static cudaError_t launch_hex_team_mode(const RhsParams& prm, const R* u, const EpiParams<R>& ep,
                                        cudaStream_t st) {
  using S = TeamSize<P>;
  const size_t smem = S::template smem_bytes<R, MODE>();
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_rhs_hex_team<P, R, MODE>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  const int grid = (prm.ne + S::EPB - 1) / S::EPB;
  k_rhs_hex_team<P, R, MODE><<<grid, S::THREADS, smem, st>>>(prm, u, ep);
  return cudaGetLastError();
}

template <int P, typename R>
static cudaError_t launch_hex_team(const RhsParams& prm, const R* u, const EpiParams<R>& ep,
                                   cudaStream_t st) {
  return launch_hex_team_mode<P, R, 0>(prm, u, ep, st);
}

// Face pass then element pass (each face evaluated once); falls back to the
// fused kernel without a slot buffer and for the face-only evaluation.
template <int P, typename R>
static cudaError_t launch_hex_split(const RhsParams& prm, const R* u, const EpiParams<R>& ep,
                                    cudaStream_t st) {
  if (!prm.fslot || prm.faces_only) return launch_hex_team_mode<P, R, 0>(prm, u, ep, st);
  cudaError_t e = launch_hex_team_mode<P, R, 1>(prm, u, ep, st);
  if (e != cudaSuccess) return e;
  return launch_hex_team_mode<P, R, 2>(prm, u, ep, st);
}

// Shared-face rounds (each face inside a CTA evaluated once); the fused
// kernel where the context holds no schedule.
template <int P, typename R>
static cudaError_t launch_hex_shared(const RhsParams& prm, const R* u, const EpiParams<R>& ep,
                                     cudaStream_t st) {
  if (!prm.hsched) return launch_hex_team_mode<P, R, 0>(prm, u, ep, st);
  return launch_hex_team_mode<P, R, 3>(prm, u, ep, st);
}

// Defaults (64^3 periodic pulse on a GB300, per RK step): FP32 Q2 -- the
// face-once tiled kernel (2.39 ms against 3.15 for the fused team kernel);
// FP32 Q1 -- the fused team kernel (1.39 ms against 1.57 split and 1.42
// shared-face); FP64 Q1 -- face pass + element pass, whose
// FP64 fluxes are evaluated once per face (21.6 ms against 27.4 shared-face
// and 36.3 fused; the fused kernel where the context holds no flux slots);
// FP64 Q2 -- shared-face rounds (55.7 ms against 68.3 fused and 125.5 warp
// per element).
template <>
cudaError_t launch_rhs_t<5, 1>(int prec, const RhsParams& prm, const void* u, const void* ep,
                               cudaStream_t st) {
  if (prec == 0)
    return launch_hex_split<1, double>(prm, (const double*)u, *(const EpiParams<double>*)ep, st);
  return launch_hex_team<1, float>(prm, (const float*)u, *(const EpiParams<float>*)ep, st);
}
template <>
cudaError_t launch_rhs_t<5, 2>(int prec, const RhsParams& prm, const void* u, const void* ep,
                               cudaStream_t st) {
  if (prec == 0)
    return launch_hex_shared<2, double>(prm, (const double*)u, *(const EpiParams<double>*)ep, st);
  if (prm.htile) return launch_hex_tile(2, 1, prm, u, ep, st);
  return launch_hex_team<2, float>(prm, (const float*)u, *(const EpiParams<float>*)ep, st);
}

template cudaError_t launch_limit_t<5, 1>(int, const LimParams&, void*, float*, cudaStream_t);
template cudaError_t launch_limit_t<5, 2>(int, const LimParams&, void*, float*, cudaStream_t);
template cudaError_t launch_means_t<5, 1>(int, int, long long, const RefTables*, const void*,
                                          const float*, double*, cudaStream_t);
template cudaError_t launch_means_t<5, 2>(int, int, long long, const RefTables*, const void*,
                                          const float*, double*, cudaStream_t);

// The hexahedral right-hand-side kernels, selectable for tests and the
// autotuner (0 = default choice above, 1 = warp-per-element sum
// factorisation, 2 = team kernel, 3 = face pass + element pass, 4 = team
// kernel with shared-face rounds, 5 = face-once tiled kernel where the
// context holds tiles, 6 = the tiled kernel with the volume contraction on
// the tensor cores for FP32 Q2, else the default).
cudaError_t launch_hex_variant(int variant, int p, int prec, const RhsParams& prm, const void* u,
                               const void* ep, cudaStream_t st) {
  if (variant == 5 && prm.htile) return launch_hex_tile(p, prec, prm, u, ep, st);
  if (variant == 6 && prm.htile && prm.tcb && p == 2 && prec == 1) return launch_hex_tile_tc(prm, u, ep, st);
  if (variant == 4) {
    if (p == 1)
      return prec == 0 ? launch_hex_shared<1, double>(prm, (const double*)u, *(const EpiParams<double>*)ep, st)
                       : launch_hex_shared<1, float>(prm, (const float*)u, *(const EpiParams<float>*)ep, st);
    return prec == 0 ? launch_hex_shared<2, double>(prm, (const double*)u, *(const EpiParams<double>*)ep, st)
                     : launch_hex_shared<2, float>(prm, (const float*)u, *(const EpiParams<float>*)ep, st);
  }
  if (variant == 3) {
    if (p == 1)
      return prec == 0 ? launch_hex_split<1, double>(prm, (const double*)u, *(const EpiParams<double>*)ep, st)
                       : launch_hex_split<1, float>(prm, (const float*)u, *(const EpiParams<float>*)ep, st);
    return prec == 0 ? launch_hex_split<2, double>(prm, (const double*)u, *(const EpiParams<double>*)ep, st)
                     : launch_hex_split<2, float>(prm, (const float*)u, *(const EpiParams<float>*)ep, st);
  }
  if (variant == 1) {
    if (p == 1)
      return prec == 0 ? launch_hex_sf<1, double>(prm, (const double*)u, *(const EpiParams<double>*)ep, st)
                       : launch_hex_sf<1, float>(prm, (const float*)u, *(const EpiParams<float>*)ep, st);
    return prec == 0 ? launch_hex_sf<2, double>(prm, (const double*)u, *(const EpiParams<double>*)ep, st)
                     : launch_hex_sf<2, float>(prm, (const float*)u, *(const EpiParams<float>*)ep, st);
  }
  if (variant == 2) {
    if (p == 1)
      return prec == 0 ? launch_hex_team<1, double>(prm, (const double*)u, *(const EpiParams<double>*)ep, st)
                       : launch_hex_team<1, float>(prm, (const float*)u, *(const EpiParams<float>*)ep, st);
    return prec == 0 ? launch_hex_team<2, double>(prm, (const double*)u, *(const EpiParams<double>*)ep, st)
                     : launch_hex_team<2, float>(prm, (const float*)u, *(const EpiParams<float>*)ep, st);
  }
  return p == 1 ? launch_rhs_t<5, 1>(prec, prm, u, ep, st) : launch_rhs_t<5, 2>(prec, prm, u, ep, st);
}

}  // namespace rkdg
