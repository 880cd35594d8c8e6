// Kernel launchers (host-callable), implemented in the .cu files.
#pragma once

#include <cuda_runtime.h>

#include "rkdg_common.h"

namespace rkdg {

bool generic_supported(int geom, int p);
// prec: 0 = FP64, 1 = FP32.  ep points to EpiParams<double> or EpiParams<float>.
cudaError_t launch_rhs(int geom, int p, int prec, const RhsParams& prm, const void* u,
                       const void* ep, cudaStream_t st);
// Same with a hexahedral kernel variant (0 default, 1 warp per element, 2 team).
cudaError_t launch_rhs_v(int variant, int geom, int p, int prec, const RhsParams& prm,
                         const void* u, const void* ep, cudaStream_t st);
cudaError_t launch_hex_variant(int variant, int p, int prec, const RhsParams& prm, const void* u,
                               const void* ep, cudaStream_t st);
// Face-once tiled hexahedral kernel (orders 1 and 2; needs prm.htile).
cudaError_t launch_hex_tile(int p, int prec, const RhsParams& prm, const void* u, const void* ep,
                            cudaStream_t st);
// the tile kernel with the volume contraction on the tensor cores (FP32, Q2)
cudaError_t launch_hex_tile_tc(const RhsParams& prm, const void* u, const void* ep, cudaStream_t st);
// mode: 0 = double in place, 1 = float in place, 2 = float pair (u = hi, ulo = lo)
cudaError_t launch_limit(int geom, int p, int mode, const LimParams& prm, void* u, float* ulo,
                         cudaStream_t st);
// mode: 0 = double, 1 = float, 2 = float pair
cudaError_t launch_means(int geom, int p, int mode, int ne, long long ndofs,
                         const RefTables* tab, const void* u, const float* ulo, double* means,
                         cudaStream_t st);

// Hanging faces of a nonconforming mesh (rkdg_nc.cu): fluxes at the slave
// points (and the wave speed), then, with gather, the per-element face terms
// prm.xface that the element kernels add.  u: FP64 (prec 0) or FP32 state.
cudaError_t launch_nc(int geom, int p, int prec, const RhsParams& prm, const NcParams& nc,
                      const void* u, bool gather, cudaStream_t st);

cudaError_t launch_riemann_batch(int dim, int prec, int n, const double* u1, const double* u2,
                                 const double* nor, double* flux, double* speed, double gamma,
                                 double covolume, int rs, int avg, cudaStream_t st);
cudaError_t launch_split(long long n, const double* x, float* hi, float* lo, cudaStream_t st);
cudaError_t launch_join(long long n, const float* hi, const float* lo, double* x,
                        cudaStream_t st);
cudaError_t launch_to_float(long long n, const double* x, float* y, cudaStream_t st);
cudaError_t launch_copy_f(long long n, const float* x, float* y, cudaStream_t st);
// per-block partial sums of sum_e w_e * sum_j wmean_j u[k][e][j]  -> partial[k][block]
cudaError_t launch_totals(int nd, int neq, int ne, long long ndofs, const RefTables* tab,
                          const double* wdet, const double* u, double* partial, int nblocks,
                          cudaStream_t st);

cudaError_t launch_batch_init(const BatchState& bs, double dt0, cudaStream_t st);
// Rebuild the map of the active work from the problems' active flags.
cudaError_t launch_batch_map(const BatchState& bs, cudaStream_t st);
cudaError_t launch_batch_control(const BatchState& bs, cudaGraphConditionalHandle h,
                                 int use_handle, cudaStream_t st);

// discrete adjoint (FP64)
bool adjoint_supported(int geom, int p);
cudaError_t launch_minv_apply(int geom, int p, int ne, long long ndofs, const RefTables* tab,
                              const double* egeo, const double* kb, double* r, cudaStream_t st);
cudaError_t launch_rhs_vjp(int geom, int p, const RhsParams& prm, const double* u, const double* r,
                           double* ub, cudaStream_t st);
// u_bar += the hanging faces' part of (dz/du)^T r (nonconforming meshes).
cudaError_t launch_nc_vjp(int geom, int p, const RhsParams& prm, const NcParams& nc, const double* u,
                          const double* r, double* ub, cudaStream_t st);
cudaError_t launch_limit_vjp(int geom, int p, const LimParams& prm, const double* z,
                             const double* yb, double* zb, double* cross, cudaStream_t st);
cudaError_t launch_limit_vjp_gather(int geom, int p, const LimParams& prm, const double* cross,
                                    double* zb, cudaStream_t st);
cudaError_t launch_axpy(long long n, double a, const double* x, double* y, cudaStream_t st);
cudaError_t launch_scale_copy(long long n, double a, const double* x, double* y, cudaStream_t st);
// Fixed means scratch of rkdg_limit_static on `device` (must be current).
cudaError_t static_means_scratch(int device, double** out);

// Template launch helpers shared by the per-geometry translation units.
template <int G, int P>
cudaError_t launch_rhs_t(int prec, const RhsParams& prm, const void* u, const void* ep,
                         cudaStream_t st);
template <int G, int P>
cudaError_t launch_limit_t(int mode, const LimParams& prm, void* u, float* ulo, cudaStream_t st);
template <int G, int P>
cudaError_t launch_means_t(int mode, int ne, long long ndofs, const RefTables* tab, const void* u,
                           const float* ulo, double* means, cudaStream_t st);

}  // namespace rkdg
