// Discrete adjoint (vector-Jacobian products) of the FP64 right-hand side and
// limiter, one thread per element, dense reference operators.
//
// Right-hand side y = M^-1 z(u): given k_bar, r = M^-1 k_bar (M symmetric),
// then u_bar = (dz/du)^T r with
//   volume  z_j += sum_m sum_r D[r][j][m] G_r(u_m),  G_r = sum_d adj(J)[r][d] F_d
//           -> u_bar_m += (dF_d/du)^T (sum_r adj[r][d] sum_j D[r][j][m] r_j)
//   faces   z_e1 -= w|J| Fhat B1,  z_e2 += w|J| Fhat B2
//           -> Fhat_bar = w|J| (-B1 r_e1 + B2 r_e2),
//              u_bar_own += B_own (dFhat/du_own)^T Fhat_bar
// Jacobians of the Euler flux and of the numerical flux (with the ghost state
// of boundary faces) come from the same templates instantiated with Dual<5>,
// so every branch is differentiated on its active side.  Each element
// differentiates only with respect to its own trace, so no atomics are needed.
//
// Limiter (Multi, BJ-family indicator): the limited values are
// v_i = mean + m^nd (u_i - mean) (the nd-fold application of
// limiter_multiplier.cpp:24-38), m = density indicator.  The indicator is
// recomputed with Dual numbers over the element's density DOFs and the
// density means of its stencil; the derivative with respect to a
// neighbour's mean is stored per face and gathered by the neighbour.
#pragma once

#include "rkdg_common.h"
#include "rkdg_dual.cuh"
#include "rkdg_generic.cuh"
#include "rkdg_physics.cuh"

namespace rkdg {

// r = M^-1 k_bar per element (reference inverse mass / det J).
template <int G, int P>
__global__ void k_minv_apply(int ne, long long ndofs, const RefTables* tab, const double* egeo,
                             const double* __restrict__ kb, double* __restrict__ r) {
  using E = El<G, P>;
  constexpr int ND = E::ND, NEQ = E::NEQ, DIM = E::DIM;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const double idet = egeo[(long long)(DIM * DIM) * ne + e];
  const double* ng = tab->ngeo_e;  // per-node geometry (bilinear quads): diagonal mass, per-node 1/det J
  for (int k = 0; k < NEQ; ++k) {
    double in[ND];
#pragma unroll
    for (int j = 0; j < ND; ++j) in[j] = kb[k * ndofs + (long long)e * ND + j];
#pragma unroll
    for (int i = 0; i < ND; ++i) {
      double v = 0.0;
#pragma unroll
      for (int j = 0; j < ND; ++j) v += tab->Minv[j][i] * in[j];
      r[k * ndofs + (long long)e * ND + i] = v * (ng ? ng[((long long)(DIM * DIM) * ND + i) * ne + e] : idet);
    }
  }
}

template <int G, int P>
__global__ void __launch_bounds__(64)
    k_rhs_vjp(const RhsParams prm, const double* __restrict__ u, const double* __restrict__ r,
              double* __restrict__ ubar) {
  using E = El<G, P>;
  constexpr int DIM = E::DIM, ND = E::ND, NEQ = E::NEQ, NFPE = E::NFPE, NQF = E::NQF;
  using D = Dual<NEQ>;
  const RefTables* T = prm.tab;
  const int ne = prm.ne;
  const long long NDa = prm.ndofs;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const D gamma = D(prm.gamma), cov = D(prm.covolume);
  double acc[NEQ][ND];
  for (int k = 0; k < NEQ; ++k)
    for (int s = 0; s < ND; ++s) acc[k][s] = 0.0;
  // faces
  const double* fg = (const double*)prm.fgeo;
  for (int lf = 0; lf < NFPE; ++lf) {
    const int nb = prm.fnbr[lf * ne + e];
    if (nb == -1) continue;
    const int code = prm.fcode[lf * ne + e];
    D n[DIM];
    for (int c = 0; c < DIM; ++c) n[c] = D(fg[(long long)(lf * (DIM + 1) + c) * ne + e]);
    const double jac = fg[(long long)(lf * (DIM + 1) + DIM) * ne + e];
    const int side = (code >> 3) & 1, lfo = code & 7, pid = code >> 4;
    int e1 = e, lf1 = lf, e2 = nb, lf2 = lfo;
    if (nb >= 0 && side) {
      e1 = nb;
      lf1 = lfo;
      e2 = e;
      lf2 = lf;
    }
    for (int q = 0; q < NQF; ++q) {
      const int q2 = T->perm[pid][q];
      const double* B1 = T->B[lf1][q];
      const double* B2 = nb >= 0 ? T->B[lf2][q2] : nullptr;
      D s1[NEQ], s2[NEQ];
      double fbar[NEQ];
      for (int k = 0; k < NEQ; ++k) {
        double v1 = 0.0, r1 = 0.0;
        for (int s = 0; s < ND; ++s) {
          v1 += u[k * NDa + (long long)e1 * ND + s] * B1[s];
          r1 += r[k * NDa + (long long)e1 * ND + s] * B1[s];
        }
        double v2 = 0.0, r2 = 0.0;
        if (nb >= 0)
          for (int s = 0; s < ND; ++s) {
            v2 += u[k * NDa + (long long)e2 * ND + s] * B2[s];
            r2 += r[k * NDa + (long long)e2 * ND + s] * B2[s];
          }
        const bool own1 = (nb < 0) || side == 0;
        s1[k] = own1 ? D::var(v1, k) : D(v1);
        s2[k] = own1 ? D(v2) : D::var(v2, k);
        fbar[k] = T->wf[q] * jac * (-r1 + (nb >= 0 ? r2 : 0.0));
      }
      if (nb < 0) {
        const BCSlot& bc = prm.bc[-2 - nb];
        right_state<DIM>(bc.type, bc.state, s1, s2, n, gamma, cov, (decltype(gamma))prm.rgas);
      }
      D F[NEQ];
      riemann<DIM>(s1, s2, n, F, gamma, cov, prm.rs, prm.avg);
      const double* Bo = T->B[lf][side ? q2 : q];
      for (int kk = 0; kk < NEQ; ++kk) {
        double g = 0.0;
        for (int k = 0; k < NEQ; ++k) g += fbar[k] * F[k].d[kk];
        for (int s = 0; s < ND; ++s) acc[kk][s] += Bo[s] * g;
      }
    }
  }
  // volume
  double adj[DIM][DIM];
  for (int rr = 0; rr < DIM; ++rr)
    for (int d = 0; d < DIM; ++d) adj[rr][d] = ((const double*)prm.egeo)[(long long)(rr * DIM + d) * ne + e];
  for (int m = 0; m < ND; ++m) {
    if (T->ngeo_e)  // bilinear quads: adj(J) at the node
      for (int rr = 0; rr < DIM; ++rr)
        for (int d = 0; d < DIM; ++d) adj[rr][d] = T->ngeo_e[((long long)(rr * DIM + d) * ND + m) * ne + e];
    D st[NEQ];
    for (int k = 0; k < NEQ; ++k) st[k] = D::var(u[k * NDa + (long long)e * ND + m], k);
    D F[NEQ][DIM];
    flux_and_speed<DIM>(st, F, gamma, cov);
    for (int k = 0; k < NEQ; ++k) {
      double gbar[DIM];
      for (int rr = 0; rr < DIM; ++rr) {
        double s = 0.0;
        for (int j = 0; j < ND; ++j) s += T->D[rr][j][m] * r[k * NDa + (long long)e * ND + j];
        gbar[rr] = s;
      }
      for (int d = 0; d < DIM; ++d) {
        double fb = 0.0;
        for (int rr = 0; rr < DIM; ++rr) fb += adj[rr][d] * gbar[rr];
        for (int kk = 0; kk < NEQ; ++kk) acc[kk][m] += fb * F[k][d].d[kk];
      }
    }
  }
  for (int k = 0; k < NEQ; ++k)
    for (int s = 0; s < ND; ++s) ubar[k * NDa + (long long)e * ND + s] = acc[k][s];
}

// Hanging faces of a nonconforming mesh (see rkdg_nc.cu).  The element VJP
// above skips them (they carry no integrator of their own); here, per slave
// point q, Fhat_bar = w_q |J_f| (-B1 r_fine + Bc r_coarse) and, with the
// flux differentiated once per side, g_side = (dFhat/du_side)^T Fhat_bar
// (k_nc_vjp_point, stored [face][q][side][k]); k_nc_vjp_gather then adds
// phi_j(q) g_side over each touched element's slave faces to u_bar.
template <int G, int P>
__global__ void __launch_bounds__(64)
    k_nc_vjp_point(const RhsParams prm, const NcParams nc, const double* __restrict__ u,
                   const double* __restrict__ r) {
  using E = El<G, P>;
  constexpr int DIM = E::DIM, ND = E::ND, NEQ = E::NEQ, NQF = E::NQF;
  using D = Dual<NEQ>;
  const RefTables* T = prm.tab;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nc.nnc * NQF) return;
  const int f = t / NQF, q = t - f * NQF;
  const int e1 = nc.face[f * 4], lf1 = nc.face[f * 4 + 1], e2 = nc.face[f * 4 + 2];
  const int ne = prm.ne;
  const long long NDa = prm.ndofs;
  const double* fg = (const double*)prm.fgeo;
  D n[DIM];
  for (int c = 0; c < DIM; ++c) n[c] = D(fg[(long long)(lf1 * (DIM + 1) + c) * ne + e1]);
  const double jac = fg[(long long)(lf1 * (DIM + 1) + DIM) * ne + e1];
  const double* B1 = T->B[lf1][q];
  const double* B2 = nc.bnc + ((long long)f * NQF + q) * ND;
  double v1[NEQ], v2[NEQ], fbar[NEQ];
  for (int k = 0; k < NEQ; ++k) {
    double a = 0.0, b = 0.0, ra = 0.0, rb = 0.0;
    for (int s = 0; s < ND; ++s) {
      a += u[k * NDa + (long long)e1 * ND + s] * B1[s];
      ra += r[k * NDa + (long long)e1 * ND + s] * B1[s];
      b += u[k * NDa + (long long)e2 * ND + s] * B2[s];
      rb += r[k * NDa + (long long)e2 * ND + s] * B2[s];
    }
    v1[k] = a;
    v2[k] = b;
    fbar[k] = T->wf[q] * jac * (-ra + rb);
  }
  const D gamma = D(prm.gamma), cov = D(prm.covolume);
  double* g = (double*)nc.flux + ((long long)f * NQF + q) * 2 * NEQ;
  for (int side = 0; side < 2; ++side) {
    D s1[NEQ], s2[NEQ];
    for (int k = 0; k < NEQ; ++k) {
      s1[k] = side == 0 ? D::var(v1[k], k) : D(v1[k]);
      s2[k] = side == 1 ? D::var(v2[k], k) : D(v2[k]);
    }
    D F[NEQ];
    riemann<DIM>(s1, s2, n, F, gamma, cov, prm.rs, prm.avg);
    for (int kk = 0; kk < NEQ; ++kk) {
      double s = 0.0;
      for (int k = 0; k < NEQ; ++k) s += fbar[k] * F[k].d[kk];
      g[side * NEQ + kk] = s;
    }
  }
}

template <int G, int P>
__global__ void __launch_bounds__(128)
    k_nc_vjp_gather(const NcParams nc, const RefTables* __restrict__ T, long long NDa,
                    double* __restrict__ ubar) {
  using E = El<G, P>;
  constexpr int ND = E::ND, NEQ = E::NEQ, NQF = E::NQF;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nc.nel * ND) return;
  const int i = t / ND, j = t - i * ND;
  double s[NEQ];
  for (int k = 0; k < NEQ; ++k) s[k] = 0.0;
  const double* gb = (const double*)nc.flux;
  for (int c = nc.ptr[i]; c < nc.ptr[i + 1]; ++c) {
    const int f = nc.ent[c] >> 1, side = nc.ent[c] & 1;
    const int lf1 = nc.face[f * 4 + 1];
    for (int q = 0; q < NQF; ++q) {
      const double phi = side ? nc.bnc[((long long)f * NQF + q) * ND + j] : T->B[lf1][q][j];
      const double* g = gb + (((long long)f * NQF + q) * 2 + side) * NEQ;
      for (int k = 0; k < NEQ; ++k) s[k] += phi * g[k];
    }
  }
  const int e = nc.elem[i];
  for (int k = 0; k < NEQ; ++k) ubar[k * NDa + (long long)e * ND + j] += s[k];
}

// The limiter's stencil of element e (limiter.cpp:95-123): its face
// neighbours, then the elements across its hanging faces (nonconforming
// meshes).  stencil_size / stencil_at enumerate it; an entry is -1 where a
// face has no neighbour.
__device__ __forceinline__ int lim_ncrow(const LimParams& prm, int e) {
  return prm.ncidx ? prm.ncidx[e] : -1;
}
__device__ __forceinline__ int stencil_size(const LimParams& prm, int row, int nfpe) {
  return nfpe + (row >= 0 ? prm.nc_ptr[row + 1] - prm.nc_ptr[row] : 0);
}
__device__ __forceinline__ int stencil_at(const LimParams& prm, int e, int row, int nfpe, int i) {
  if (i < nfpe) return prm.fnbr[i * prm.ne + e];
  const int ent = prm.nc_ent[prm.nc_ptr[row] + i - nfpe];
  return prm.nc_face[(ent >> 1) * 4 + ((ent & 1) ? 0 : 2)];
}
// Local faces of e that are slave or master faces: they carry indicator
// points although no conforming neighbour lies across them.
__device__ __forceinline__ unsigned hanging_faces(const LimParams& prm, int row) {
  unsigned m = 0;
  if (row >= 0)
    for (int c = prm.nc_ptr[row]; c < prm.nc_ptr[row + 1]; ++c) {
      const int f = prm.nc_ent[c] >> 1, side = prm.nc_ent[c] & 1;
      m |= 1u << prm.nc_face[f * 4 + (side ? 3 : 1)];
    }
  return m;
}

// Limiter VJP, own part.  The stencil's density minimum and maximum are
// each one element's mean (the first one in stencil order on ties, as the
// forward min/max keeps it); the derivative with respect to them goes to
// cross[0..3][e] = (argmin element or -1 for e itself, d/dmin, argmax
// element or -1, d/dmax), which k_limit_vjp_gather hands to those elements.
template <int G, int P>
__global__ void __launch_bounds__(64)
    k_limit_vjp(const LimParams prm, const double* __restrict__ z, const double* __restrict__ ybar,
                double* __restrict__ zbar, double* __restrict__ cross) {
  using E = El<G, P>;
  constexpr int DIM = E::DIM, ND = E::ND, NEQ = E::NEQ, NFPE = E::NFPE, NQL = E::NQL, NV = E::NV;
  constexpr int NVAR = ND + 3;  // nodal densities, own mean, stencil min, stencil max
  using D = Dual<NVAR>;
  const RefTables* T = prm.tab;
  const int ne = prm.ne;
  const long long NDa = prm.ndofs;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  double el[NEQ][ND], yb[NEQ][ND], um[NEQ];
  for (int k = 0; k < NEQ; ++k) {
    um[k] = prm.means[(long long)k * ne + e];
    for (int j = 0; j < ND; ++j) {
      el[k][j] = z[k * NDa + (long long)e * ND + j];
      yb[k][j] = ybar[k * NDa + (long long)e * ND + j];
    }
  }
  for (int i = 0; i < 4; ++i) cross[(long long)i * ne + e] = i == 0 || i == 2 ? -1.0 : 0.0;
  const int row = lim_ncrow(prm, e);
  const int nst = stencil_size(prm, row, NFPE);
  const unsigned ncfaces = hanging_faces(prm, row);
  double zb[NEQ][ND];
  for (int k = 0; k < NEQ; ++k)
    for (int j = 0; j < ND; ++j) zb[k][j] = 0.0;
  // density indicator with derivatives
  D m;
  int amin = -1, amax = -1;
  double elind_last = 1.0;
  if (prm.indicator == 0) {
    m = D(1.0);
  } else if (prm.indicator == 1) {
    m = D(0.0);
    elind_last = 0.0;
  } else {
    D rho[ND];
    for (int j = 0; j < ND; ++j) rho[j] = D::var(el[0][j], j);
    const D mself = D::var(um[0], ND);
    double mIv = um[0] < 1e9 ? um[0] : 1e9, MIv = um[0] > -1e9 ? um[0] : -1e9;
    for (int i = 0; i < nst; ++i) {
      const int nb = stencil_at(prm, e, row, NFPE, i);
      if (nb < 0) continue;
      const double v = prm.means[nb];
      if (v < mIv) {
        mIv = v;
        amin = nb;
      }
      if (v > MIv) {
        MIv = v;
        amax = nb;
      }
    }
    const D mI = amin >= 0 ? D::var(mIv, ND + 1) : (mself < D(1e9) ? mself : D(1e9));
    const D MI = amax >= 0 ? D::var(MIv, ND + 2) : (mself > D(-1e9) ? mself : D(-1e9));
    D yMin = D(1e9);
    for (int lf = 0; lf < NFPE; ++lf) {
      if (prm.fnbr[lf * ne + e] < 0 && !((ncfaces >> lf) & 1u)) continue;
      for (int q = 0; q < NQL; ++q) {
        D v = D(0.0);
        for (int j = 0; j < ND; ++j) v += rho[j] * T->Bl[lf][q][j];
        const D diff = v - mself;
        D y;
        if (diff > D(1e-3))
          y = (MI - mself) / diff;
        else if (diff < D(-1e-3))
          y = (mI - mself) / diff;
        else
          y = D(1.0);
        if (prm.function == 0) {
          yMin = y < yMin ? y : yMin;
          yMin = yMin > D(1.0) ? D(1.0) : yMin;
        } else if (prm.function == 1) {
          const D yc = (y * y + 2.0 * y) / (y * y + y + 2.0);
          yMin = yc < yMin ? yc : yMin;
        } else {
          const double ys = 1.5;
          const D yr = y / ys;
          const D yc = y < D(1.0) ? y + (3.0 - 2.0 * ys) * yr * yr + (ys - 2.0) * yr * yr * yr : D(1.0);
          yMin = yc < yMin ? yc : yMin;
        }
      }
    }
    m = yMin;
    // FinDiff looks at the last equation's indicator; recompute it plainly
    if (prm.limiter == 0) {
      const int kl = NEQ - 1;
      double mIl = um[kl], MIl = um[kl], yl = 1e9;
      for (int i = 0; i < nst; ++i) {
        const int nb = stencil_at(prm, e, row, NFPE, i);
        if (nb < 0) continue;
        const double v = prm.means[(long long)kl * ne + nb];
        mIl = v < mIl ? v : mIl;
        MIl = v > MIl ? v : MIl;
      }
      for (int lf = 0; lf < NFPE; ++lf) {
        if (prm.fnbr[lf * ne + e] < 0 && !((ncfaces >> lf) & 1u)) continue;
        for (int q = 0; q < NQL; ++q) {
          double v = 0.0;
          for (int j = 0; j < ND; ++j) v += el[kl][j] * T->Bl[lf][q][j];
          const double diff = v - um[kl];
          double y = diff > 1e-3 ? (MIl - um[kl]) / diff : (diff < -1e-3 ? (mIl - um[kl]) / diff : 1.0);
          double yc;
          if (prm.function == 0) {
            yc = y < 1.0 ? y : 1.0;
          } else if (prm.function == 1) {
            yc = (y * y + 2.0 * y) / (y * y + y + 2.0);
          } else {
            const double yr = y / 1.5;
            yc = y < 1.0 ? y + 0.0 * yr * yr - 0.5 * yr * yr * yr : 1.0;
          }
          yl = yc < yl ? yc : yl;
        }
      }
      elind_last = yl;
    }
  }
  const double* w = T->wmn_e ? T->wmn_e + (long long)e * ND : T->wmean;
  if (prm.limiter == 1) {
    const int reps = (prm.quirks & 1) ? 1 : ND;
    const double mv = m.v;
    double pm1 = 1.0;  // m^(reps-1)
    for (int i = 1; i < reps; ++i) pm1 *= mv;
    const double mnd = pm1 * mv;
    const double dmnd = reps * pm1;
    // forward values to test the last-hope reset
    bool reset = false;
    if (prm.last_hope) {
      for (int v = 0; v < NV && !reset; ++v) {
        double fv[NEQ];
        for (int k = 0; k < NEQ; ++k) {
          double s = 0.0;
          for (int j = 0; j < ND; ++j) s += (um[k] + mnd * (el[k][j] - um[k])) * T->Bv[v][j];
          fv[k] = s;
        }
        if (!state_is_physical<DIM>(fv, prm.gamma, prm.covolume)) reset = true;
      }
    }
    if (reset) {
      for (int k = 0; k < NEQ; ++k) {
        double sy = 0.0;
        for (int i = 0; i < ND; ++i) sy += yb[k][i];
        for (int j = 0; j < ND; ++j) zb[k][j] += w[j] * sy;
      }
    } else {
      double mbar = 0.0;
      for (int k = 0; k < NEQ; ++k) {
        double sy = 0.0;
        for (int i = 0; i < ND; ++i) {
          sy += yb[k][i];
          mbar += yb[k][i] * dmnd * (el[k][i] - um[k]);
        }
        for (int j = 0; j < ND; ++j) zb[k][j] += w[j] * (1.0 - mnd) * sy + mnd * yb[k][j];
      }
      if (prm.indicator == 2) {
        for (int j = 0; j < ND; ++j) zb[0][j] += mbar * (m.d[j] + m.d[ND] * w[j]);
        cross[(long long)0 * ne + e] = amin;
        cross[(long long)1 * ne + e] = mbar * m.d[ND + 1];
        cross[(long long)2 * ne + e] = amax;
        cross[(long long)3 * ne + e] = mbar * m.d[ND + 2];
      }
    }
  } else {
    if (elind_last < 0.999) {
      for (int k = 0; k < NEQ; ++k) {
        double sy = 0.0;
        for (int i = 0; i < ND; ++i) sy += yb[k][i];
        for (int j = 0; j < ND; ++j) zb[k][j] += w[j] * sy;
      }
    } else {
      for (int k = 0; k < NEQ; ++k)
        for (int j = 0; j < ND; ++j) zb[k][j] += yb[k][j];
    }
  }
  for (int k = 0; k < NEQ; ++k)
    for (int j = 0; j < ND; ++j) zbar[k * NDa + (long long)e * ND + j] = zb[k][j];
}

// Gather, for element c, the derivatives that the elements of its stencil
// (which hold c in theirs) took with respect to c's density mean (mean =
// sum_j w_j rho_j), each stencil element once.
template <int G, int P>
__global__ void k_limit_vjp_gather(const LimParams prm, const double* __restrict__ cross,
                                   double* __restrict__ zbar) {
  using E = El<G, P>;
  constexpr int ND = E::ND, NFPE = E::NFPE;
  const int ne = prm.ne;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ne) return;
  const int row = lim_ncrow(prm, c);
  const int nst = stencil_size(prm, row, NFPE);
  double s = 0.0;
  for (int i = 0; i < nst; ++i) {
    const int e = stencil_at(prm, c, row, NFPE, i);
    if (e < 0 || e == c) continue;
    bool seen = false;
    for (int i2 = 0; i2 < i && !seen; ++i2) seen = stencil_at(prm, c, row, NFPE, i2) == e;
    if (seen) continue;
    if (cross[e] == (double)c) s += cross[(long long)ne + e];
    if (cross[(long long)2 * ne + e] == (double)c) s += cross[(long long)3 * ne + e];
  }
  if (s != 0.0)
    for (int j = 0; j < ND; ++j)
      zbar[(long long)c * ND + j] +=
          (prm.tab->wmn_e ? prm.tab->wmn_e[(long long)c * ND + j] : prm.tab->wmean[j]) * s;
}

}  // namespace rkdg
