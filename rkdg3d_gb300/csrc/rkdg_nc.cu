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
//   k_nc_face    64 / NQF slave faces per CTA: both traces at each point, the
//                numerical flux (Elem1, Elem2 order), the wave speed, then the
//                face's term for each of its two elements;
//   k_nc_gather  one thread per (element, node) of an element touched by
//                hanging faces: the sum of its faces' terms in a fixed order
//                (no atomics), which the element kernels add before the
//                inverse mass.
#include "rkdg_generic.cuh"
#include "rkdg_launch.h"

namespace rkdg {

// Compile-time node and face-point counts (ND, NQF) unroll the loops.
// k_nc_face: FPC = 64 / NQF slave faces per CTA.  Each thread evaluates one
// point flux into shared memory; then the CTA forms each face's term for
// both its elements, term[side][k][j] = sign * sum_q w_q |J_f| Fhat_k(q)
// phi_j(q) (phi of the fine element's own face points, or of the coarse
// element at the mapped points), sign -1 on the fine (Elem1) side.
constexpr int kNcFaceThreads = 64;

template <int DIM, int ND, int NQF, typename R>
__global__ void __launch_bounds__(kNcFaceThreads) k_nc_face(const __grid_constant__ RhsParams prm,
                                                            const __grid_constant__ NcParams nc,
                                                            const R* __restrict__ u,
                                                            int with_terms) {
  constexpr int NEQ = DIM + 2, FPC = kNcFaceThreads / NQF;
  static_assert(FPC >= 1, "one thread per face point");
  __shared__ R sF[FPC][NQF][NEQ];
  const RefTables* T = prm.tab;
  const int lf = threadIdx.x / NQF, q = threadIdx.x - lf * NQF;
  const int f = blockIdx.x * FPC + lf;
  R lmax = R(0);
  int pb = -1;  // batched problems: the face's problem (both elements share it)
  bool live = lf < FPC && f < nc.nnc;
  if (live && prm.prob) {
    pb = prm.prob[nc.face[f * 4]];
    live = prm.pactive[pb] != 0;
  }
  if (live) {
    const int e1 = nc.face[f * 4], lf1 = nc.face[f * 4 + 1], e2 = nc.face[f * 4 + 2];
    const int ne = prm.ne;
    const long long NDa = prm.ndofs;
    const R* fg = (const R*)prm.fgeo;
    R n[DIM];
#pragma unroll
    for (int c = 0; c < DIM; ++c) n[c] = fg[(long long)(lf1 * (DIM + 1) + c) * ne + e1];
    const R jac = fg[(long long)(lf1 * (DIM + 1) + DIM) * ne + e1];
    const double* B1 = T->B[lf1][q];
    const double* B2 = nc.bnc + ((long long)f * NQF + q) * ND;
    R b1[ND], b2[ND];
#pragma unroll
    for (int s = 0; s < ND; ++s) {
      b1[s] = (R)B1[s];
      b2[s] = (R)B2[s];
    }
    R s1[NEQ], s2[NEQ];
#pragma unroll
    for (int k = 0; k < NEQ; ++k) {
      const R* u1 = u + k * NDa + (long long)e1 * ND;
      const R* u2 = u + k * NDa + (long long)e2 * ND;
      R a = R(0), b = R(0);
#pragma unroll
      for (int s = 0; s < ND; ++s) {
        a += u1[s] * b1[s];
        b += u2[s] * b2[s];
      }
      s1[k] = a;
      s2[k] = b;
    }
    const R gamma = (R)(pb >= 0 ? prm.pgamma[pb] : prm.gamma);
    const R cov = (R)(pb >= 0 ? prm.pcov[pb] : prm.covolume);
    R F[NEQ];
    lmax = checked_speed(prm, riemann<DIM>(s1, s2, n, F, gamma, cov, prm.rs, prm.avg), e1, pb);
    const R wq = (R)T->wf[q];
#pragma unroll
    for (int k = 0; k < NEQ; ++k) sF[lf][q][k] = (F[k] * wq) * jac;
  }
  if (prm.prob) {
    // per-problem maximum; a face point of an idle problem keeps lmax = 0,
    // and atomic_max_nonneg issues no atomic for a speed that is not positive
    if (pb >= 0) atomic_max_nonneg(prm.pmcs + pb, (double)lmax);
    __syncthreads();  // sF is complete after it
  } else {
    block_max_commit<R>(lmax, prm.mcs);  // contains a CTA barrier: sF is complete after it
  }
  if (!with_terms) return;
  for (int o = threadIdx.x; o < FPC * 2 * ND; o += blockDim.x) {
    const int c = o / (2 * ND), r = o - c * 2 * ND;
    const int side = r / ND, j = r - side * ND;
    const int fc = blockIdx.x * FPC + c;
    if (fc >= nc.nnc) break;
    if (prm.prob && !prm.pactive[prm.prob[nc.face[fc * 4]]]) continue;  // idle problem
    const int lf1 = nc.face[fc * 4 + 1];
    const R sg = side ? R(1) : R(-1);
    R acc[NEQ];
#pragma unroll
    for (int k = 0; k < NEQ; ++k) acc[k] = R(0);
#pragma unroll
    for (int qq = 0; qq < NQF; ++qq) {
      const R w = sg * (R)(side ? nc.bnc[((long long)fc * NQF + qq) * ND + j] : T->B[lf1][qq][j]);
#pragma unroll
      for (int k = 0; k < NEQ; ++k) acc[k] += sF[c][qq][k] * w;
    }
    R* term = (R*)nc.flux + (long long)fc * 2 * NEQ * ND;
#pragma unroll
    for (int k = 0; k < NEQ; ++k) term[(side * NEQ + k) * ND + j] = acc[k];
  }
}

// k_nc_gather: one thread per (element, node) of an element touched by
// hanging faces, adding its faces' terms in list order.
template <int DIM, int ND, typename R>
__global__ void __launch_bounds__(128) k_nc_gather(const __grid_constant__ NcParams nc) {
  constexpr int NEQ = DIM + 2;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nc.nel * ND) return;
  const int i = t / ND, j = t - i * ND;
  const R* terms = (const R*)nc.flux;
  R s[NEQ];
#pragma unroll
  for (int k = 0; k < NEQ; ++k) s[k] = R(0);
  for (int c = nc.ptr[i]; c < nc.ptr[i + 1]; ++c) {
    const int f = nc.ent[c] >> 1, side = nc.ent[c] & 1;
    const R* tv = terms + ((long long)f * 2 + side) * NEQ * ND + j;
#pragma unroll
    for (int k = 0; k < NEQ; ++k) s[k] += tv[k * ND];
  }
#pragma unroll
  for (int k = 0; k < NEQ; ++k) ((R*)nc.xface)[((long long)i * NEQ + k) * ND + j] = s[k];
}

template <int G, int P>
static void nc_launch_gp(int prec, const RhsParams& prm, const NcParams& nc, const void* u,
                         bool gather, cudaStream_t st) {
  using E = El<G, P>;
  const int fpc = kNcFaceThreads / E::NQF;
  const int g1 = (nc.nnc + fpc - 1) / fpc;
  const int g2 = (nc.nel * E::ND + 127) / 128;
  if (prec == 0) {
    k_nc_face<E::DIM, E::ND, E::NQF, double><<<g1, kNcFaceThreads, 0, st>>>(prm, nc, (const double*)u, gather);
    if (gather && g2 > 0) k_nc_gather<E::DIM, E::ND, double><<<g2, 128, 0, st>>>(nc);
  } else {
    k_nc_face<E::DIM, E::ND, E::NQF, float><<<g1, kNcFaceThreads, 0, st>>>(prm, nc, (const float*)u, gather);
    if (gather && g2 > 0) k_nc_gather<E::DIM, E::ND, float><<<g2, 128, 0, st>>>(nc);
  }
}

// Both kernels for one right-hand-side evaluation (prec 0: FP64 state,
// 1: FP32 stage input); the gather is skipped for the face-only speed.
cudaError_t launch_nc(int geom, int p, int prec, const RhsParams& prm, const NcParams& nc,
                      const void* u, bool gather, cudaStream_t st) {
  if (nc.nnc <= 0) return cudaSuccess;
  switch (geom * 10 + p) {
    case 21: nc_launch_gp<2, 1>(prec, prm, nc, u, gather, st); break;
    case 22: nc_launch_gp<2, 2>(prec, prm, nc, u, gather, st); break;
    case 31: nc_launch_gp<3, 1>(prec, prm, nc, u, gather, st); break;
    case 32: nc_launch_gp<3, 2>(prec, prm, nc, u, gather, st); break;
    case 33: nc_launch_gp<3, 3>(prec, prm, nc, u, gather, st); break;
    case 51: nc_launch_gp<5, 1>(prec, prm, nc, u, gather, st); break;
    case 52: nc_launch_gp<5, 2>(prec, prm, nc, u, gather, st); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace rkdg
