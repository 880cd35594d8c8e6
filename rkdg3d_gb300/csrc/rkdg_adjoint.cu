// Launchers of the discrete-adjoint kernels (rkdg_adjoint.cuh).
#include "rkdg_adjoint.cuh"
#include "rkdg_launch.h"

namespace rkdg {

bool adjoint_supported(int geom, int p) {
  return (geom == 2 && (p == 1 || p == 2)) || (geom == 3 && p >= 1 && p <= 3) ||
         (geom == 5 && (p == 1 || p == 2));
}

#define RKDG_ADJ_DISPATCH(CALL)       \
  switch (geom * 10 + p) {            \
    case 21: return CALL(2, 1);       \
    case 22: return CALL(2, 2);       \
    case 31: return CALL(3, 1);       \
    case 32: return CALL(3, 2);       \
    case 33: return CALL(3, 3);       \
    case 51: return CALL(5, 1);       \
    case 52: return CALL(5, 2);       \
    default: return cudaErrorInvalidValue; \
  }

template <int G, int P>
static cudaError_t minv_t(int ne, long long ndofs, const RefTables* tab, const double* egeo,
                          const double* kb, double* r, cudaStream_t st) {
  k_minv_apply<G, P><<<(ne + 127) / 128, 128, 0, st>>>(ne, ndofs, tab, egeo, kb, r);
  return cudaGetLastError();
}
cudaError_t launch_minv_apply(int geom, int p, int ne, long long ndofs, const RefTables* tab,
                              const double* egeo, const double* kb, double* r, cudaStream_t st) {
#define CALL_MINV(G, P) minv_t<G, P>(ne, ndofs, tab, egeo, kb, r, st)
  RKDG_ADJ_DISPATCH(CALL_MINV)
#undef CALL_MINV
}

template <int G, int P>
static cudaError_t rhs_vjp_t(const RhsParams& prm, const double* u, const double* r, double* ub,
                             cudaStream_t st) {
  k_rhs_vjp<G, P><<<(prm.ne + 63) / 64, 64, 0, st>>>(prm, u, r, ub);
  return cudaGetLastError();
}
cudaError_t launch_rhs_vjp(int geom, int p, const RhsParams& prm, const double* u, const double* r,
                           double* ub, cudaStream_t st) {
#define CALL_RV(G, P) rhs_vjp_t<G, P>(prm, u, r, ub, st)
  RKDG_ADJ_DISPATCH(CALL_RV)
#undef CALL_RV
}

template <int G, int P>
static cudaError_t nc_vjp_t(const RhsParams& prm, const NcParams& nc, const double* u,
                            const double* r, double* ub, cudaStream_t st) {
  using E = El<G, P>;
  k_nc_vjp_point<G, P><<<(nc.nnc * E::NQF + 63) / 64, 64, 0, st>>>(prm, nc, u, r);
  if (nc.nel > 0)
    k_nc_vjp_gather<G, P><<<(nc.nel * E::ND + 127) / 128, 128, 0, st>>>(nc, prm.tab, prm.ndofs, ub);
  return cudaGetLastError();
}
cudaError_t launch_nc_vjp(int geom, int p, const RhsParams& prm, const NcParams& nc, const double* u,
                          const double* r, double* ub, cudaStream_t st) {
  if (nc.nnc <= 0) return cudaSuccess;
#define CALL_NV(G, P) nc_vjp_t<G, P>(prm, nc, u, r, ub, st)
  RKDG_ADJ_DISPATCH(CALL_NV)
#undef CALL_NV
}

template <int G, int P>
static cudaError_t lim_vjp_t(const LimParams& prm, const double* z, const double* yb, double* zb,
                             double* cross, cudaStream_t st) {
  k_limit_vjp<G, P><<<(prm.ne + 63) / 64, 64, 0, st>>>(prm, z, yb, zb, cross);
  return cudaGetLastError();
}
cudaError_t launch_limit_vjp(int geom, int p, const LimParams& prm, const double* z,
                             const double* yb, double* zb, double* cross, cudaStream_t st) {
#define CALL_LV(G, P) lim_vjp_t<G, P>(prm, z, yb, zb, cross, st)
  RKDG_ADJ_DISPATCH(CALL_LV)
#undef CALL_LV
}

template <int G, int P>
static cudaError_t gather_t(const LimParams& prm, const double* cross, double* zb, cudaStream_t st) {
  k_limit_vjp_gather<G, P><<<(prm.ne + 127) / 128, 128, 0, st>>>(prm, cross, zb);
  return cudaGetLastError();
}
cudaError_t launch_limit_vjp_gather(int geom, int p, const LimParams& prm, const double* cross,
                                    double* zb, cudaStream_t st) {
#define CALL_G(G, P) gather_t<G, P>(prm, cross, zb, st)
  RKDG_ADJ_DISPATCH(CALL_G)
#undef CALL_G
}

__global__ void k_axpy(long long n, double a, const double* __restrict__ x, double* __restrict__ y) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] += a * x[i];
}
__global__ void k_scale_copy(long long n, double a, const double* __restrict__ x,
                             double* __restrict__ y) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = a * x[i];
}

static int grid_n(long long n) {
  long long g = (n + 255) / 256;
  return (int)(g > 152 * 32 ? 152 * 32 : (g < 1 ? 1 : g));
}
cudaError_t launch_axpy(long long n, double a, const double* x, double* y, cudaStream_t st) {
  k_axpy<<<grid_n(n), 256, 0, st>>>(n, a, x, y);
  return cudaGetLastError();
}
cudaError_t launch_scale_copy(long long n, double a, const double* x, double* y, cudaStream_t st) {
  k_scale_copy<<<grid_n(n), 256, 0, st>>>(n, a, x, y);
  return cudaGetLastError();
}

}  // namespace rkdg
