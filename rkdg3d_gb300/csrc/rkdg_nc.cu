// Hanging faces of nonconforming (adapted) meshes.
//
// The reference runs on MFEM meshes made nonconforming by EnsureNCMesh
// (case_manager.cpp:269) and adapted by its refiner / derefiner
// (main.cpp:564-696).  MFEM's NonlinearForm::Mult integrates every slave
// face of a nonconforming face as an interior face -- Elem1 = the slave's
// fine element with the slave face's own points, normal and |J_f|, Elem2 =
// the coarse element that owns the master face, evaluated at the slave
// points mapped into it -- and skips the master face.  The element kernels
// treat both kinds of face as faces without an integrator; these two
// kernels supply their terms:
//   k_nc_flux    one thread per slave-face point: both traces, the numerical
//                flux (Elem1, Elem2 order), the wave speed, w_q |J_f| Fhat;
//   k_nc_gather  one thread per (element, variable, node) of an element
//                touched by hanging faces: its face term, summed over its
//                slave faces and points in a fixed order (no atomics), added
//                by the element kernels before the inverse mass.
#include "rkdg_generic.cuh"
#include "rkdg_launch.h"

namespace rkdg {

template <int DIM, typename R>
__global__ void __launch_bounds__(128) k_nc_flux(const __grid_constant__ RhsParams prm,
                                                 const __grid_constant__ NcParams nc,
                                                 const R* __restrict__ u) {
  constexpr int NEQ = DIM + 2;
  const RefTables* T = prm.tab;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  R lmax = R(0);
  if (t < nc.nnc * nc.nqf) {
    const int f = t / nc.nqf, q = t - f * nc.nqf;
    const int e1 = nc.face[f * 4], lf1 = nc.face[f * 4 + 1], e2 = nc.face[f * 4 + 2];
    const int ne = prm.ne, nd = nc.nd;
    const long long NDa = prm.ndofs;
    const R* fg = (const R*)prm.fgeo;
    R n[DIM];
#pragma unroll
    for (int c = 0; c < DIM; ++c) n[c] = fg[(long long)(lf1 * (DIM + 1) + c) * ne + e1];
    const R jac = fg[(long long)(lf1 * (DIM + 1) + DIM) * ne + e1];
    const double* B1 = T->B[lf1][q];
    const double* B2 = nc.bnc + ((long long)f * nc.nqf + q) * nd;
    R s1[NEQ], s2[NEQ];
#pragma unroll
    for (int k = 0; k < NEQ; ++k) {
      const R* u1 = u + k * NDa + (long long)e1 * nd;
      const R* u2 = u + k * NDa + (long long)e2 * nd;
      R a = R(0), b = R(0);
      for (int s = 0; s < nd; ++s) {
        a += u1[s] * (R)B1[s];
        b += u2[s] * (R)B2[s];
      }
      s1[k] = a;
      s2[k] = b;
    }
    const R gamma = (R)prm.gamma, cov = (R)prm.covolume;
    R F[NEQ];
    lmax = checked_speed(prm, riemann<DIM>(s1, s2, n, F, gamma, cov, prm.rs, prm.avg), e1);
    const R wq = (R)T->wf[q];
    R* out = (R*)nc.flux + ((long long)f * nc.nqf + q) * NEQ;
#pragma unroll
    for (int k = 0; k < NEQ; ++k) out[k] = (F[k] * wq) * jac;
  }
  block_max_commit<R>(lmax, prm.mcs);
}

template <int DIM, typename R>
__global__ void __launch_bounds__(128) k_nc_gather(const __grid_constant__ RhsParams prm,
                                                   const __grid_constant__ NcParams nc) {
  constexpr int NEQ = DIM + 2;
  const RefTables* T = prm.tab;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nd = nc.nd, nqf = nc.nqf;
  if (t >= nc.nel * NEQ * nd) return;
  const int i = t / (NEQ * nd), rem = t - i * NEQ * nd;
  const int k = rem / nd, j = rem - k * nd;
  const R* fl = (const R*)nc.flux;
  R s = R(0);
  for (int c = nc.ptr[i]; c < nc.ptr[i + 1]; ++c) {
    const int f = nc.ent[c] >> 1, side = nc.ent[c] & 1;
    const int lf1 = nc.face[f * 4 + 1];
    const R sg = side ? R(1) : R(-1);
    for (int q = 0; q < nqf; ++q) {
      const R phi = side ? (R)nc.bnc[((long long)f * nqf + q) * nd + j] : (R)T->B[lf1][q][j];
      s += sg * fl[((long long)f * nqf + q) * NEQ + k] * phi;
    }
  }
  ((R*)nc.xface)[((long long)i * NEQ + k) * nd + j] = s;
}

// Both kernels for one right-hand-side evaluation (prec 0: FP64 state,
// 1: FP32 stage input); the gather is skipped for the face-only speed.
cudaError_t launch_nc(int dim, int prec, const RhsParams& prm, const NcParams& nc, const void* u,
                      bool gather, cudaStream_t st) {
  if (nc.nnc <= 0) return cudaSuccess;
  const int bs = 128;
  const int g1 = (nc.nnc * nc.nqf + bs - 1) / bs;
  const int g2 = (nc.nel * (dim + 2) * nc.nd + bs - 1) / bs;
#define RKDG_NC_LAUNCH(D, R)                                                        \
  do {                                                                              \
    k_nc_flux<D, R><<<g1, bs, 0, st>>>(prm, nc, (const R*)u);                       \
    if (gather && g2 > 0) k_nc_gather<D, R><<<g2, bs, 0, st>>>(prm, nc);            \
  } while (0)
  if (dim == 2) {
    if (prec == 0) RKDG_NC_LAUNCH(2, double); else RKDG_NC_LAUNCH(2, float);
  } else {
    if (prec == 0) RKDG_NC_LAUNCH(3, double); else RKDG_NC_LAUNCH(3, float);
  }
#undef RKDG_NC_LAUNCH
  return cudaGetLastError();
}

}  // namespace rkdg
