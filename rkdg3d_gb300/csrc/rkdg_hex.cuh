// Sum-factorised hexahedral right-hand side (DG Q_p on affine hexahedra).
//
// One warp per element, eight consecutive elements per CTA (256 threads).
// The CTA stages its elements' DOFs in shared memory with coalesced loads
// (each variable of the tile is one contiguous run of 8*(p+1)^3 values).
// Per element:
//   faces   for each local face: contract the element (and the neighbour
//           element) along the face normal with the 1D basis at the face
//           (sum factorisation, (p+1)^2 values per variable), interpolate to
//           the (p+2)^2 face points, numerical flux per point with the
//           arguments ordered (Elem1, Elem2, Elem1-outward normal) as
//           FaceIntegrator::AssembleFaceVector (face_integrator.cpp:11-276),
//           then lift back with the transposed tensor trace.
//   volume  nodal Euler flux (FE_Evolution::GetFlux, fe_evolution.cpp:219-
//           245), contravariant components with adj(J), and the collocated
//           (phi, grad phi) operator applied one direction at a time:
//           3 x (p+1) terms per node and variable instead of (p+1)^3 x 3.
//   mass    the exact hexahedral mass matrix (rule order 2p+2) is
//           det J * (M1 x M1 x M1); its inverse is applied as three 1D
//           sweeps (fe_evolution.cpp:178-208).
#pragma once

#include "rkdg_common.h"
#include "rkdg_generic.cuh"
#include "rkdg_physics.cuh"

namespace rkdg {

template <int P>
struct HexSize {
  static constexpr int N1 = P + 1, NQ1 = P + 2, ND = N1 * N1 * N1, NQF = NQ1 * NQ1, NEQ = 5,
                       NF2 = N1 * N1, EPB = 8;
  static constexpr int TAB = 6 * NQF * NF2 + 2 * N1 + 2 * N1 * N1 + N1 + NQF;
  static constexpr int WARP = 2 * NEQ * ND + 3 * NEQ * ND + 3 * NEQ * NQF + 2 * NEQ * NF2 + NEQ * ND;
  static constexpr int TAB_AL = (TAB + 3) & ~3;
  template <typename R>
  static constexpr size_t smem_bytes() {
    return sizeof(R) * (size_t)(TAB_AL + EPB * WARP);
  }
};

// node index of (jn along axis nax, i0 along the lower tangential axis, i1
// along the upper tangential axis)
template <int N1>
__device__ __forceinline__ int hex_node(int nax, int jn, int i0, int i1) {
  if (nax == 0) return jn + N1 * (i0 + N1 * i1);
  if (nax == 1) return i0 + N1 * (jn + N1 * i1);
  return i0 + N1 * (i1 + N1 * jn);
}

// Per-value Runge-Kutta epilogue; returns the combined value (for means).
template <typename R>
__device__ __forceinline__ double epi_value(const EpiParams<R>& ep, long long idx, R y) {
  if (ep.mode == 0) {
    ep.out64[idx] = (double)y;
    return 0.0;
  }
  if constexpr (std::is_same<R, double>::value) {
    double v = ep.base ? ep.base[idx] : 0.0;
    for (int j = 0; j < ep.nprev; ++j) v += ep.cprev[j] * ep.kprev[j][idx];
    v += ep.ccur * y;
    if (ep.kout) ep.kout[idx] = y;
    if (ep.out64) ep.out64[idx] = v;
    if (ep.out32) ep.out32[idx] = (float)v;
    return v;
  } else {
    if (!ep.final_stage) {
      float inc = ep.baselo[idx];
      for (int j = 0; j < ep.nprev; ++j) inc = fmaf(ep.cprev_hi[j], ep.kprev[j][idx], inc);
      inc = fmaf(ep.ccur_hi, y, inc);
      const float v = ep.basehi[idx] + inc;
      if (ep.kout) ep.kout[idx] = y;
      ep.out32[idx] = v;
      return (double)v;
    }
    float sh = 0.0f, sl = 0.0f, ph, pl;
    for (int j = 0; j < ep.nprev; ++j) {
      ds_mul_f(ep.cprev_hi[j], ep.cprev_lo[j], ep.kprev[j][idx], ph, pl);
      ds_add(sh, sl, ph, pl);
    }
    ds_mul_f(ep.ccur_hi, ep.ccur_lo, y, ph, pl);
    ds_add(sh, sl, ph, pl);
    float h = ep.basehi[idx], l = ep.baselo[idx];
    ds_add(h, l, sh, sl);
    ep.out32[idx] = h;
    ep.outlo[idx] = l;
    return (double)h + (double)l;
  }
}

// Same epilogue, returning the combined value as a pair (hi, lo); lo is zero
// except for the float-pair conserved state of the final stage.
template <typename R>
__device__ __forceinline__ void epi_value2(const EpiParams<R>& ep, long long idx, R y, R& hi,
                                           R& lo) {
  lo = R(0);
  if (ep.mode == 0) {
    ep.out64[idx] = (double)y;
    hi = y;
    return;
  }
  if constexpr (std::is_same<R, double>::value) {
    double v = ep.base ? ep.base[idx] : 0.0;
    for (int j = 0; j < ep.nprev; ++j) v += ep.cprev[j] * ep.kprev[j][idx];
    v += ep.ccur * y;
    if (ep.kout) ep.kout[idx] = y;
    if (ep.out64) ep.out64[idx] = v;
    if (ep.out32) ep.out32[idx] = (float)v;
    hi = v;
  } else {
    if (!ep.final_stage) {
      float inc = ep.baselo[idx];
      for (int j = 0; j < ep.nprev; ++j) inc = fmaf(ep.cprev_hi[j], ep.kprev[j][idx], inc);
      inc = fmaf(ep.ccur_hi, y, inc);
      const float v = ep.basehi[idx] + inc;
      if (ep.kout) ep.kout[idx] = y;
      ep.out32[idx] = v;
      hi = v;
      return;
    }
    float sh = 0.0f, sl = 0.0f, ph, pl;
    for (int j = 0; j < ep.nprev; ++j) {
      ds_mul_f(ep.cprev_hi[j], ep.cprev_lo[j], ep.kprev[j][idx], ph, pl);
      ds_add(sh, sl, ph, pl);
    }
    ds_mul_f(ep.ccur_hi, ep.ccur_lo, y, ph, pl);
    ds_add(sh, sl, ph, pl);
    float h = ep.basehi[idx], l = ep.baselo[idx];
    ds_add(h, l, sh, sl);
    ep.out32[idx] = h;
    ep.outlo[idx] = l;
    hi = h;
    lo = l;
  }
}

template <int P, typename R>
__global__ void __launch_bounds__(256)
    k_rhs_hex_sf(const RhsParams prm, const R* __restrict__ u, const EpiParams<R> ep) {
  using S = HexSize<P>;
  constexpr int N1 = S::N1, ND = S::ND, NQF = S::NQF, NEQ = S::NEQ, NF2 = S::NF2, EPB = S::EPB;
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ unsigned char sPerm[RKDG_MAX_PERM][NQF];
  R* sm = reinterpret_cast<R*>(smraw);
  R* tB2 = sm;                        // [6][NQF][NF2]
  R* tLend = tB2 + 6 * NQF * NF2;     // [2][N1]
  R* tD1 = tLend + 2 * N1;            // [N1][N1]
  R* tMinv = tD1 + N1 * N1;           // [N1][N1]
  R* tW1 = tMinv + N1 * N1;           // [N1]
  R* tWf = tW1 + N1;                  // [NQF]
  const RefTables* T = prm.tab;
  const int tid = threadIdx.x;
  for (int t = tid; t < 6 * NQF * NF2; t += blockDim.x) {
    const int r = t % NF2, q = (t / NF2) % NQF, lf = t / (NF2 * NQF);
    tB2[t] = (R)T->B2[lf][q][r];
  }
  for (int t = tid; t < 2 * N1; t += blockDim.x) tLend[t] = (R)T->lend[t / N1][t % N1];
  for (int t = tid; t < N1 * N1; t += blockDim.x) {
    tD1[t] = (R)T->d1[t / N1][t % N1];
    tMinv[t] = (R)T->minv1[t / N1][t % N1];
  }
  for (int t = tid; t < N1; t += blockDim.x) tW1[t] = (R)T->w1[t];
  for (int t = tid; t < NQF; t += blockDim.x) tWf[t] = (R)T->wf[t];
  for (int t = tid; t < RKDG_MAX_PERM * NQF; t += blockDim.x)
    sPerm[t / NQF][t % NQF] = (unsigned char)T->perm[t / NQF][t % NQF];

  const int warp = tid >> 5, lane = tid & 31;
  R* wb = sm + S::TAB_AL + warp * S::WARP;
  R* sU = wb;                         // [NEQ][ND] own DOFs
  R* sAcc = sU + NEQ * ND;            // [NEQ][ND]
  R* sG = sAcc + NEQ * ND;            // [3][NEQ][ND] contravariant fluxes / sweeps
  R* sTO = sG + 3 * NEQ * ND;         // [NEQ][NQF] own trace
  R* sTN = sTO + NEQ * NQF;           // [NEQ][NQF] neighbour trace
  R* sF = sTN + NEQ * NQF;            // [NEQ][NQF] lifted flux values
  R* sVO = sF + NEQ * NQF;            // [NEQ][NF2]
  R* sVN = sVO + NEQ * NF2;           // [NEQ][NF2]
  R* sNb = sVN + NEQ * NF2;           // [NEQ][ND] neighbour DOFs

  const int ne = prm.ne;
  const long long NDa = prm.ndofs;
  const int e0 = blockIdx.x * EPB;
  const int nel = min(EPB, ne - e0);
  // cooperative, coalesced load of the tile's DOFs
  for (int k = 0; k < NEQ; ++k)
    for (int t = tid; t < nel * ND; t += blockDim.x)
      sm[S::TAB_AL + (t / ND) * S::WARP + k * ND + (t % ND)] =
          u[k * NDa + (long long)e0 * ND + t];
  __syncthreads();

  const R gamma = (R)prm.gamma, cov = (R)prm.covolume;
  R lmax = R(0);
  const int e = e0 + warp;
  if (warp < nel) {
    for (int t = lane; t < NEQ * ND; t += 32) sAcc[t] = R(0);
    const R* fg = (const R*)prm.fgeo;
    for (int lf = 0; lf < 6; ++lf) {
      const int nb = prm.fnbr[lf * ne + e];
      if (nb == -1) continue;
      const int code = prm.fcode[lf * ne + e];
      R n[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) n[c] = fg[(long long)(lf * 4 + c) * ne + e];
      const R jac = fg[(long long)(lf * 4 + 3) * ne + e];
      const int side = (code >> 3) & 1, lfo = code & 7, pid = code >> 4;
      const int naxO = T->fax[lf], sdO = T->fside[lf];
      if (nb >= 0)
        for (int t = lane; t < NEQ * ND; t += 32)
          sNb[t] = u[(t / ND) * NDa + (long long)nb * ND + (t % ND)];
      // contraction along the face normal
      for (int o = lane; o < NEQ * NF2; o += 32) {
        const int k = o / NF2, r = o % NF2, i0 = r / N1, i1 = r % N1;
        R v = R(0);
#pragma unroll
        for (int jn = 0; jn < N1; ++jn) v += tLend[sdO * N1 + jn] * sU[k * ND + hex_node<N1>(naxO, jn, i0, i1)];
        sVO[o] = v;
      }
      int naxN = 0, sdN = 0;
      if (nb >= 0) {
        naxN = T->fax[lfo];
        sdN = T->fside[lfo];
        __syncwarp();
        for (int o = lane; o < NEQ * NF2; o += 32) {
          const int k = o / NF2, r = o % NF2, i0 = r / N1, i1 = r % N1;
          R v = R(0);
#pragma unroll
          for (int jn = 0; jn < N1; ++jn) v += tLend[sdN * N1 + jn] * sNb[k * ND + hex_node<N1>(naxN, jn, i0, i1)];
          sVN[o] = v;
        }
      }
      __syncwarp();
      // traces at the canonical face points
      for (int o = lane; o < NEQ * NQF; o += 32) {
        const int k = o / NQF, q = o % NQF;
        const R* b2 = tB2 + (lf * NQF + q) * NF2;
        R v = R(0);
#pragma unroll
        for (int r = 0; r < NF2; ++r) v += b2[r] * sVO[k * NF2 + r];
        sTO[o] = v;
        if (nb >= 0) {
          const R* b2n = tB2 + (lfo * NQF + q) * NF2;
          R w = R(0);
#pragma unroll
          for (int r = 0; r < NF2; ++r) w += b2n[r] * sVN[k * NF2 + r];
          sTN[o] = w;
        }
      }
      __syncwarp();
      // numerical flux at the Elem1 points
      if (lane < NQF) {
        const int q = lane, q2 = sPerm[pid][q];
        R s1[NEQ], s2[NEQ];
        int own = q;
        if (nb >= 0) {
          if (side == 0) {
#pragma unroll
            for (int k = 0; k < NEQ; ++k) {
              s1[k] = sTO[k * NQF + q];
              s2[k] = sTN[k * NQF + q2];
            }
          } else {
#pragma unroll
            for (int k = 0; k < NEQ; ++k) {
              s1[k] = sTN[k * NQF + q];
              s2[k] = sTO[k * NQF + q2];
            }
            own = q2;
          }
        } else {
#pragma unroll
          for (int k = 0; k < NEQ; ++k) s1[k] = sTO[k * NQF + q];
          const BCSlot& bc = prm.bc[-2 - nb];
          right_state<3>(bc.type, bc.state, s1, s2, n, gamma, cov, (R)prm.rgas);
        }
        R F[NEQ];
        const R sp = checked_speed(prm, riemann<3>(s1, s2, n, F, gamma, cov, prm.rs, prm.avg), e);
        lmax = fmax(lmax, sp);
        const R sg = side ? R(1) : R(-1);
        const R wq = tWf[q];
#pragma unroll
        for (int k = 0; k < NEQ; ++k) sF[k * NQF + own] = sg * (F[k] * wq) * jac;
      }
      __syncwarp();
      if (!prm.faces_only) {
        // lift: transposed tensor trace
        for (int o = lane; o < NEQ * NF2; o += 32) {
          const int k = o / NF2, r = o % NF2;
          R v = R(0);
#pragma unroll
          for (int q = 0; q < NQF; ++q) v += tB2[(lf * NQF + q) * NF2 + r] * sF[k * NQF + q];
          sVO[o] = v;
        }
        __syncwarp();
        for (int o = lane; o < NEQ * ND; o += 32) {
          const int k = o / ND, j = o % ND;
          const int jx = j % N1, jy = (j / N1) % N1, jz = j / (N1 * N1);
          const int jn = naxO == 0 ? jx : (naxO == 1 ? jy : jz);
          const int i0 = naxO == 0 ? jy : jx, i1 = naxO == 2 ? jy : jz;
          sAcc[o] += tLend[sdO * N1 + jn] * sVO[k * NF2 + i0 * N1 + i1];
        }
      }
      __syncwarp();
    }
    if (!prm.faces_only) {
      const R* eg = (const R*)prm.egeo;
      R adj[3][3];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int d = 0; d < 3; ++d) adj[r][d] = eg[(long long)(r * 3 + d) * ne + e];
      const R idet = eg[(long long)9 * ne + e];
      // nodal fluxes -> contravariant components
      for (int j = lane; j < ND; j += 32) {
        R st[NEQ];
#pragma unroll
        for (int k = 0; k < NEQ; ++k) st[k] = sU[k * ND + j];
        R F[NEQ][3];
        lmax = fmax(lmax, flux_and_speed<3>(st, F, gamma, cov));
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int k = 0; k < NEQ; ++k)
            sG[(r * NEQ + k) * ND + j] = adj[r][0] * F[k][0] + adj[r][1] * F[k][1] + adj[r][2] * F[k][2];
      }
      __syncwarp();
      // collocated (phi, grad phi), one direction at a time; plus the face
      // terms of hanging faces (nonconforming meshes)
      const R* xf = nullptr;
      if (prm.ncidx && prm.ncidx[e] >= 0) xf = (const R*)prm.xface + (long long)prm.ncidx[e] * NEQ * ND;
      for (int o = lane; o < NEQ * ND; o += 32) {
        const int k = o / ND, j = o % ND;
        const int jx = j % N1, jy = (j / N1) % N1, jz = j / (N1 * N1);
        R zx = R(0), zy = R(0), zz = R(0);
#pragma unroll
        for (int m = 0; m < N1; ++m) {
          zx += tD1[jx * N1 + m] * sG[(0 * NEQ + k) * ND + m + N1 * (jy + N1 * jz)];
          zy += tD1[jy * N1 + m] * sG[(1 * NEQ + k) * ND + jx + N1 * (m + N1 * jz)];
          zz += tD1[jz * N1 + m] * sG[(2 * NEQ + k) * ND + jx + N1 * (jy + N1 * m)];
        }
        sAcc[o] += tW1[jy] * tW1[jz] * zx + tW1[jx] * tW1[jz] * zy + tW1[jx] * tW1[jy] * zz;
        if (xf) sAcc[o] += xf[o];
      }
      __syncwarp();
      // inverse mass: three 1D sweeps (x into sG, y back into sAcc, z in registers)
      for (int o = lane; o < NEQ * ND; o += 32) {
        const int k = o / ND, j = o % ND;
        const int jx = j % N1, jy = (j / N1) % N1, jz = j / (N1 * N1);
        R v = R(0);
#pragma unroll
        for (int m = 0; m < N1; ++m) v += tMinv[jx * N1 + m] * sAcc[k * ND + m + N1 * (jy + N1 * jz)];
        sG[o] = v;
      }
      __syncwarp();
      for (int o = lane; o < NEQ * ND; o += 32) {
        const int k = o / ND, j = o % ND;
        const int jx = j % N1, jy = (j / N1) % N1, jz = j / (N1 * N1);
        R v = R(0);
#pragma unroll
        for (int m = 0; m < N1; ++m) v += tMinv[jy * N1 + m] * sG[k * ND + jx + N1 * (m + N1 * jz)];
        sAcc[o] = v;
      }
      __syncwarp();
      double msum[NEQ];
#pragma unroll
      for (int k = 0; k < NEQ; ++k) msum[k] = 0.0;
      for (int o = lane; o < NEQ * ND; o += 32) {
        const int k = o / ND, j = o % ND;
        const int jx = j % N1, jy = (j / N1) % N1, jz = j / (N1 * N1);
        R v = R(0);
#pragma unroll
        for (int m = 0; m < N1; ++m) v += tMinv[jz * N1 + m] * sAcc[k * ND + jx + N1 * (jy + N1 * m)];
        const double c = epi_value<R>(ep, k * NDa + (long long)e * ND + j, v * idet);
#pragma unroll
        for (int kk = 0; kk < NEQ; ++kk)
          if (kk == k) msum[kk] += T->wmean[j] * c;
      }
      if (ep.mode == 1 && (ep.means || ep.means32)) {
#pragma unroll
        for (int k = 0; k < NEQ; ++k) {
          double s = msum[k];
#pragma unroll
          for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
          if (lane == 0) store_mean(ep, (long long)k * ne + e, s);
        }
      }
    }
  }
  block_max_commit<R>(lmax, prm.mcs);
}

}  // namespace rkdg
