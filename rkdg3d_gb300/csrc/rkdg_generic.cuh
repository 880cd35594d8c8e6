// Generic (dense reference-operator) element kernels: one thread per element.
//
// Used for every supported (geometry, order) pair; hexahedra additionally
// have sum-factorised kernels (rkdg_hex.cuh).  Reference operators live in
// shared memory, converted to the arithmetic type R.  The right-hand side of
// one element is the reference's FE_Evolution::Mult restricted to that
// element (fe_evolution.cpp:102-216): every face of the element computes the
// numerical flux at the face points with the arguments ordered (Elem1,
// Elem2, Elem1-outward normal) exactly as FaceIntegrator::AssembleFaceVector
// (face_integrator.cpp:11-276), so the two elements of a face obtain
// bit-identical fluxes and the scheme stays conservative to round-off
// without atomics.
#pragma once

#include "rkdg_common.h"
#include "rkdg_physics.cuh"

namespace rkdg {

// Largest CTA the generic (thread-per-element) kernels are launched with.
constexpr int kGenericMaxBlock = 256;

// ---- double-single (float pair) helpers for the FP32-bulk path --------------
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ void ds_add(float& hi, float& lo, float bh, float bl) {
  float s, e;
  two_sum(hi, bh, s, e);
  e += lo + bl;
  hi = s + e;
  lo = e - (hi - s);
}
// (ch, cl) * k as a float pair
__device__ __forceinline__ void ds_mul_f(float ch, float cl, float k, float& ph, float& pl) {
  ph = ch * k;
  pl = fmaf(ch, k, -ph) + cl * k;
}

__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* addr, double v) {
  if (!(v > 0.0)) return;
  atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

// Block-wide max of a per-thread wave speed, committed with one atomicMax per
// block (the MPI_Allreduce(MAX) of main.cpp:543 on one device).
template <typename R>
__device__ __forceinline__ void block_max_commit(R v, unsigned long long* dst) {
  double vd = (double)v;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) vd = fmax(vd, __shfl_xor_sync(0xffffffffu, vd, o));
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __shared__ double redd[32];
  if (lane == 0) redd[w] = vd;
  __syncthreads();
  if (w == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    double x = lane < nw ? redd[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
    if (lane == 0) atomic_max_nonneg(dst, x);
  }
}

__device__ __forceinline__ void flag_error(int* err, int code, int where) {
  if (atomicCAS(&err[0], 0, code) == 0) err[1] = where;
}

// The reference aborts when a face wave speed is negative
// (face_integrator.cpp:214-218).  That is how its solvers report a
// non-physical state (-1), but HLLC's signed max(SL, SR) (rs_hllc.cpp:98) is
// also negative in supersonic flow against the normal.  With quirk bit 0 only
// the -1 of a non-physical state is an error; the speed enters the max as 0.
// In a batch of independent problems (pb >= 0) a non-physical state stops
// only its own problem: the problem is marked failed and the others go on.
template <typename R>
__device__ __forceinline__ R checked_speed(const RhsParams& prm, R sp, int e, int pb = -1) {
  if (sp < R(0)) {
    if (!(prm.quirks & 1) || sp == R(-1)) {
      if (pb >= 0 && prm.pfail)
        prm.pfail[pb] = 1;
      else
        flag_error(prm.err, 2, e);
    }
    return R(0);
  }
  return sp;
}

// Per-problem max wave speed for batched problems: elements of one problem
// are contiguous, so a warp holds a few contiguous runs; a segmented shuffle
// reduction leaves each run's max in its first lane, which commits it.
__device__ __forceinline__ void segmented_max_commit(double v, int pb,
                                                     unsigned long long* pmcs) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const double o = __shfl_down_sync(0xffffffffu, v, off);
    const int opb = __shfl_down_sync(0xffffffffu, pb, off);
    if (lane + off < 32 && opb == pb) v = fmax(v, o);
  }
  const int prev = __shfl_up_sync(0xffffffffu, pb, 1);
  if (pb >= 0 && (lane == 0 || prev != pb)) atomic_max_nonneg(&pmcs[pb], v);
}

// Batched problems with a map of the active work: the i-th element of the
// active problems (in problem order), and its problem pb.
__device__ __forceinline__ int active_element(const int* cum, const int* pid, const int* poff, int na,
                                              int i, int& pb) {
  int lo = 0, hi = na;  // cum[lo] <= i < cum[lo + 1]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (cum[mid] <= i)
      lo = mid;
    else
      hi = mid;
  }
  pb = pid[lo];
  return poff[pb] + (i - cum[lo]);
}

// Split c*s (c a tableau coefficient, s a problem's dt) into a float pair.
__device__ __forceinline__ void split_scaled(double c, double s, float& hi, float& lo) {
  const double v = c * s;
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

// Epilogue for one element and one equation: y[i], i < ND.  dts scales the
// coefficients of batched problems (1 otherwise).
template <int ND, typename R>
__device__ __forceinline__ void epilogue(const EpiParams<R>& ep, long long base_idx,
                                         const R* y, const R* wmean, int ne, int e, int k,
                                         double dts) {
  if (ep.mode == 0) {
#pragma unroll
    for (int i = 0; i < ND; ++i) ep.out64[base_idx + i] = (double)y[i];
    return;
  }
  if constexpr (std::is_same<R, double>::value) {
    double m = 0.0;
#pragma unroll
    for (int i = 0; i < ND; ++i) {
      const long long idx = base_idx + i;
      double v = ep.base ? ep.base[idx] : 0.0;
      for (int j = 0; j < ep.nprev; ++j) v += (ep.cprev[j] * dts) * ep.kprev[j][idx];
      v += (ep.ccur * dts) * y[i];
      if (ep.kout) ep.kout[idx] = y[i];
      if (ep.out64) ep.out64[idx] = v;
      if (ep.out32) ep.out32[idx] = (float)v;
      m += wmean[i] * v;
    }
    if (ep.means) ep.means[(long long)k * ne + e] = m;
  } else {
    float mh = 0.0f, ml = 0.0f;
    float ch[3], cl[3], cch, ccl;
    if (ep.pdt) {
      for (int j = 0; j < ep.nprev; ++j) split_scaled(ep.cprev[j], dts, ch[j], cl[j]);
      split_scaled(ep.ccur, dts, cch, ccl);
    } else {
      for (int j = 0; j < ep.nprev; ++j) {
        ch[j] = ep.cprev_hi[j];
        cl[j] = ep.cprev_lo[j];
      }
      cch = ep.ccur_hi;
      ccl = ep.ccur_lo;
    }
    if (!ep.final_stage) {
#pragma unroll
      for (int i = 0; i < ND; ++i) {
        const long long idx = base_idx + i;
        float inc = ep.baselo[idx];
        for (int j = 0; j < ep.nprev; ++j) inc = fmaf(ch[j], ep.kprev[j][idx], inc);
        inc = fmaf(cch, y[i], inc);
        const float v = ep.basehi[idx] + inc;
        if (ep.kout) ep.kout[idx] = y[i];
        ep.out32[idx] = v;
        float ph, pl;
        ds_mul_f(wmean[i], 0.0f, v, ph, pl);
        ds_add(mh, ml, ph, pl);
      }
    } else {
#pragma unroll
      for (int i = 0; i < ND; ++i) {
        const long long idx = base_idx + i;
        float sh = 0.0f, sl = 0.0f, ph, pl;
        for (int j = 0; j < ep.nprev; ++j) {
          ds_mul_f(ch[j], cl[j], ep.kprev[j][idx], ph, pl);
          ds_add(sh, sl, ph, pl);
        }
        ds_mul_f(cch, ccl, y[i], ph, pl);
        ds_add(sh, sl, ph, pl);
        float h = ep.basehi[idx], l = ep.baselo[idx];
        ds_add(h, l, sh, sl);
        ep.out32[idx] = h;
        ep.outlo[idx] = l;
        ds_mul_f(wmean[i], 0.0f, h, ph, pl);
        ds_add(mh, ml, ph, pl);
        ds_add(mh, ml, wmean[i] * l, 0.0f);
      }
    }
    if (ep.means) ep.means[(long long)k * ne + e] = (double)mh + (double)ml;
  }
}

// ---- right-hand side --------------------------------------------------------
template <int G, int P, typename R>
__global__ void __launch_bounds__(kGenericMaxBlock)
    k_rhs_generic(const RhsParams prm, const R* __restrict__ u, const EpiParams<R> ep) {
  using E = El<G, P>;
  constexpr int DIM = E::DIM, ND = E::ND, NEQ = E::NEQ, NFPE = E::NFPE, NQF = E::NQF;
  __shared__ R sB[NFPE][NQF][ND];
  __shared__ R sD[DIM][ND][ND];
  __shared__ R sMinv[ND][ND];
  __shared__ R sW[NQF];
  __shared__ R sWm[ND];
  __shared__ unsigned char sPerm[RKDG_MAX_PERM][NQF];
  const RefTables* T = prm.tab;
  // batched problems with a map of the active work: CTAs past it are idle
  if (prm.act_cum && (int)(blockIdx.x * blockDim.x) >= prm.act_cum[*prm.act_n]) return;
  for (int t = threadIdx.x; t < NFPE * NQF * ND; t += blockDim.x) {
    const int s = t % ND, q = (t / ND) % NQF, lf = t / (ND * NQF);
    sB[lf][q][s] = (R)T->B[lf][q][s];
  }
  for (int t = threadIdx.x; t < DIM * ND * ND; t += blockDim.x) {
    const int m = t % ND, j = (t / ND) % ND, r = t / (ND * ND);
    sD[r][j][m] = (R)T->D[r][j][m];
  }
  for (int t = threadIdx.x; t < ND * ND; t += blockDim.x) sMinv[t / ND][t % ND] = (R)T->Minv[t / ND][t % ND];
  for (int t = threadIdx.x; t < NQF; t += blockDim.x) sW[t] = (R)T->wf[t];
  for (int t = threadIdx.x; t < ND; t += blockDim.x) sWm[t] = (R)T->wmean[t];
  for (int t = threadIdx.x; t < RKDG_MAX_PERM * NQF; t += blockDim.x)
    sPerm[t / NQF][t % NQF] = (unsigned char)T->perm[t / NQF][t % NQF];
  __syncthreads();

  const int ne = prm.ne;
  const long long NDa = prm.ndofs;
  R gamma = (R)prm.gamma, cov = (R)prm.covolume;
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  R lmax = R(0);
  bool live = e < ne;
  int pb = -1;
  double dts = 1.0;
  if (prm.act_cum) {
    const int na = *prm.act_n;
    live = e < prm.act_cum[na];
    if (live) e = active_element(prm.act_cum, prm.act_pid, prm.poff, na, e, pb);
  }
  if (live && prm.prob) {
    if (!prm.act_cum) pb = prm.prob[e];
    live = prm.pactive[pb] != 0;
    gamma = (R)prm.pgamma[pb];
    cov = (R)prm.pcov[pb];
    if (ep.pdt) dts = ep.pdt[pb];
  }
  if (live) {
    R acc[NEQ][ND];
#pragma unroll
    for (int k = 0; k < NEQ; ++k)
#pragma unroll
      for (int s = 0; s < ND; ++s) acc[k][s] = R(0);
    const R* fg = (const R*)prm.fgeo;
    for (int lf = 0; lf < NFPE; ++lf) {
      const int nb = prm.fnbr[lf * ne + e];
      if (nb == -1) continue;
      const int code = prm.fcode[lf * ne + e];
      R n[DIM];
#pragma unroll
      for (int c = 0; c < DIM; ++c) n[c] = fg[(long long)(lf * (DIM + 1) + c) * ne + e];
      const R jac = fg[(long long)(lf * (DIM + 1) + DIM) * ne + e];
      const int side = (code >> 3) & 1, lfo = code & 7, pid = code >> 4;
      int e1 = e, lf1 = lf, e2 = nb, lf2 = lfo;
      if (nb >= 0 && side) {
        e1 = nb;
        lf1 = lfo;
        e2 = e;
        lf2 = lf;
      }
      const R sg = side ? R(1) : R(-1);
      for (int q = 0; q < NQF; ++q) {
        const int q2 = sPerm[pid][q];
        R s1[NEQ], s2[NEQ];
        const R* B1 = sB[lf1][q];
#pragma unroll
        for (int k = 0; k < NEQ; ++k) {
          const R* uk = u + k * NDa + (long long)e1 * ND;
          R v = R(0);
#pragma unroll
          for (int s = 0; s < ND; ++s) v += uk[s] * B1[s];
          s1[k] = v;
        }
        if (nb >= 0) {
          const R* B2 = sB[lf2][q2];
#pragma unroll
          for (int k = 0; k < NEQ; ++k) {
            const R* uk = u + k * NDa + (long long)e2 * ND;
            R v = R(0);
#pragma unroll
            for (int s = 0; s < ND; ++s) v += uk[s] * B2[s];
            s2[k] = v;
          }
        } else {
          const BCSlot& bc = prm.bc[-2 - nb];
          right_state<DIM>(bc.type, bc.state, s1, s2, n, gamma, cov, (decltype(gamma))prm.rgas);
        }
        R F[NEQ];
        const R sp = checked_speed(prm, riemann<DIM>(s1, s2, n, F, gamma, cov, prm.rs, prm.avg), e, pb);
        lmax = fmax(lmax, sp);
        const R* Bo = sB[lf][side ? q2 : q];
        const R wq = sW[q];
#pragma unroll
        for (int k = 0; k < NEQ; ++k) {
          const R t = sg * (F[k] * wq) * jac;
#pragma unroll
          for (int s = 0; s < ND; ++s) acc[k][s] += t * Bo[s];
        }
      }
    }
    if (!prm.faces_only) {
      const R* eg = (const R*)prm.egeo;
      const R* ng = (const R*)prm.ngeo;  // per-node geometry (bilinear quads) or null
      R adj[DIM][DIM];
#pragma unroll
      for (int r = 0; r < DIM; ++r)
#pragma unroll
        for (int d = 0; d < DIM; ++d) adj[r][d] = eg[(long long)(r * DIM + d) * ne + e];
      const R idet = eg[(long long)(DIM * DIM) * ne + e];
#pragma unroll
      for (int m = 0; m < ND; ++m) {
        if (ng) {
#pragma unroll
          for (int r = 0; r < DIM; ++r)
#pragma unroll
            for (int d = 0; d < DIM; ++d) adj[r][d] = ng[((long long)(r * DIM + d) * ND + m) * ne + e];
        }
        R st[NEQ];
#pragma unroll
        for (int k = 0; k < NEQ; ++k) st[k] = u[k * NDa + (long long)e * ND + m];
        R F[NEQ][DIM];
        const R sp = flux_and_speed<DIM>(st, F, gamma, cov);
        lmax = fmax(lmax, sp);
#pragma unroll
        for (int k = 0; k < NEQ; ++k)
#pragma unroll
          for (int r = 0; r < DIM; ++r) {
            R gc = R(0);
#pragma unroll
            for (int d = 0; d < DIM; ++d) gc += adj[r][d] * F[k][d];
#pragma unroll
            for (int j = 0; j < ND; ++j) acc[k][j] += sD[r][j][m] * gc;
          }
      }
      if (prm.ncidx) {  // hanging faces of a nonconforming mesh
        const int ix = prm.ncidx[e];
        if (ix >= 0) {
          const R* xf = (const R*)prm.xface + (long long)ix * NEQ * ND;
#pragma unroll
          for (int k = 0; k < NEQ; ++k)
#pragma unroll
            for (int j = 0; j < ND; ++j) acc[k][j] += xf[k * ND + j];
        }
      }
#pragma unroll
      for (int k = 0; k < NEQ; ++k) {
        R y[ND];
#pragma unroll
        for (int i = 0; i < ND; ++i) {
          R v = R(0);
#pragma unroll
          for (int j = 0; j < ND; ++j) v += sMinv[i][j] * acc[k][j];
          // the collocated mass of a quad is diagonal, so a per-node 1/det J
          // (bilinear quads) applies row by row
          y[i] = v * (ng ? ng[((long long)(DIM * DIM) * ND + i) * ne + e] : idet);
        }
        if (T->wmn_e) {  // this element's own cell-mean weights
          R wl[ND];
#pragma unroll
          for (int i = 0; i < ND; ++i) wl[i] = (R)T->wmn_e[(long long)e * ND + i];
          epilogue<ND, R>(ep, k * NDa + (long long)e * ND, y, wl, ne, e, k, dts);
        } else {
          epilogue<ND, R>(ep, k * NDa + (long long)e * ND, y, sWm, ne, e, k, dts);
        }
      }
    }
  }
  if (prm.prob)
    segmented_max_commit((double)lmax, live ? pb : -1, prm.pmcs);
  else
    block_max_commit<R>(lmax, prm.mcs);
}

// ---- limiter ------------------------------------------------------------------
// Nodal basis of the reference element at an arbitrary reference point (the
// tensor GL Lagrange basis, or the triangle basis from its monomial expansion).
template <int G, int P>
__device__ __forceinline__ void basis_at(const RefTables* T, const double* xi,
                                         double (&phi)[El<G, P>::ND]) {
  using E = El<G, P>;
  constexpr int DIM = E::DIM, ND = E::ND;
  if constexpr (G == 2) {
    double px[P + 1], py[P + 1];
    px[0] = py[0] = 1.0;
#pragma unroll
    for (int a = 1; a <= P; ++a) {
      px[a] = px[a - 1] * xi[0];
      py[a] = py[a - 1] * xi[1];
    }
#pragma unroll
    for (int j = 0; j < ND; ++j) phi[j] = 0.0;
#pragma unroll
    for (int m = 0; m < ND; ++m) {
      const double mv = px[T->tmono[m][0]] * py[T->tmono[m][1]];
#pragma unroll
      for (int j = 0; j < ND; ++j) phi[j] += T->tcoef[m][j] * mv;
    }
  } else {
    constexpr int N1 = P + 1;
    double l[DIM][N1];
#pragma unroll
    for (int d = 0; d < DIM; ++d)
#pragma unroll
      for (int i = 0; i < N1; ++i) {
        double v = 1.0;
#pragma unroll
        for (int m = 0; m < N1; ++m)
          if (m != i) v *= (xi[d] - T->x1n[m]) / (T->x1n[i] - T->x1n[m]);
        l[d][i] = v;
      }
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      double v = l[0][j % N1] * l[1][(j / N1) % N1];
      if constexpr (DIM == 3) v *= l[2][j / (N1 * N1)];
      phi[j] = v;
    }
  }
}

// IndicatorShu::checkDiscontinuity (indicator_shu.cpp:13-74) for element e:
// for every cell k of the stencil (e, then its face neighbours) the average
// over e of k's polynomial extrapolated there (Averager::
// computeStencilExtrapAverages, averager.cpp:154-273: the element rule of
// order p + OrderW on e mapped into k's reference frame), and
//   value = min(1, Ck max|mean_e| / (sum_k |mean_e - extrap_k| + eps)),
// Ck = 0.03, eps = 1e-6, or 1 where both are below eps.  The maximum runs over
// the stencil but reads e's own mean every time, as the reference does.
template <int G, int P, bool DS, typename R>
__device__ __forceinline__ void shu_indicator(const LimParams& prm, const R* __restrict__ u,
                                              const float* __restrict__ ulo, int e,
                                              R (&val)[El<G, P>::NEQ]) {
  using E = El<G, P>;
  constexpr int DIM = E::DIM, ND = E::ND, NEQ = E::NEQ, NFPE = E::NFPE;
  const RefTables* T = prm.tab;
  const int ne = prm.ne;
  const long long NDa = prm.ndofs;
  const double* ea = prm.eaff;
  double Je[DIM][DIM], xe[DIM], ume[NEQ], sum[NEQ];
#pragma unroll
  for (int i = 0; i < DIM; ++i) {
#pragma unroll
    for (int r = 0; r < DIM; ++r) Je[i][r] = ea[(long long)(i * DIM + r) * ne + e];
    xe[i] = ea[(long long)(DIM * DIM + i) * ne + e];
  }
#pragma unroll
  for (int k = 0; k < NEQ; ++k) {
    ume[k] = prm.means[(long long)k * ne + e];
    sum[k] = 0.0;
  }
  double wsum = 0.0;
  for (int q = 0; q < T->nqs; ++q) wsum += T->ws[q];
  // stencil: the cell, its face neighbours, then the elements across its
  // hanging faces (ElementToElementTable, limiter.cpp:118-123)
  const int ncrow = prm.ncidx ? prm.ncidx[e] : -1;
  const int nnc = ncrow >= 0 ? prm.nc_ptr[ncrow + 1] - prm.nc_ptr[ncrow] : 0;
  for (int s = -1; s < NFPE + nnc; ++s) {
    int kc;
    if (s < 0) {
      kc = e;
    } else if (s < NFPE) {
      kc = prm.fnbr[s * ne + e];
    } else {
      const int ent = prm.nc_ent[prm.nc_ptr[ncrow] + s - NFPE];
      kc = prm.nc_face[(ent >> 1) * 4 + ((ent & 1) ? 0 : 2)];
    }
    if (kc < 0) continue;  // boundary faces are not in the stencil
    // e's reference point xi -> k's reference point A xi + b
    double A[DIM][DIM], b[DIM];
    if (kc == e) {
#pragma unroll
      for (int i = 0; i < DIM; ++i) {
#pragma unroll
        for (int r = 0; r < DIM; ++r) A[i][r] = i == r ? 1.0 : 0.0;
        b[i] = 0.0;
      }
    } else {
      double Jk[DIM][DIM], Ki[DIM][DIM], dx[DIM];
#pragma unroll
      for (int i = 0; i < DIM; ++i) {
#pragma unroll
        for (int r = 0; r < DIM; ++r) Jk[i][r] = ea[(long long)(i * DIM + r) * ne + kc];
        dx[i] = xe[i] - ea[(long long)(DIM * DIM + i) * ne + kc];
      }
      if constexpr (DIM == 2) {
        const double id = 1.0 / (Jk[0][0] * Jk[1][1] - Jk[0][1] * Jk[1][0]);
        Ki[0][0] = Jk[1][1] * id;
        Ki[0][1] = -Jk[0][1] * id;
        Ki[1][0] = -Jk[1][0] * id;
        Ki[1][1] = Jk[0][0] * id;
      } else {
        const double c00 = Jk[1][1] * Jk[2][2] - Jk[1][2] * Jk[2][1];
        const double c01 = Jk[0][2] * Jk[2][1] - Jk[0][1] * Jk[2][2];
        const double c02 = Jk[0][1] * Jk[1][2] - Jk[0][2] * Jk[1][1];
        const double id = 1.0 / (Jk[0][0] * c00 + Jk[1][0] * c01 + Jk[2][0] * c02);
        Ki[0][0] = c00 * id;
        Ki[0][1] = c01 * id;
        Ki[0][2] = c02 * id;
        Ki[1][0] = (Jk[1][2] * Jk[2][0] - Jk[1][0] * Jk[2][2]) * id;
        Ki[1][1] = (Jk[0][0] * Jk[2][2] - Jk[0][2] * Jk[2][0]) * id;
        Ki[1][2] = (Jk[0][2] * Jk[1][0] - Jk[0][0] * Jk[1][2]) * id;
        Ki[2][0] = (Jk[1][0] * Jk[2][1] - Jk[1][1] * Jk[2][0]) * id;
        Ki[2][1] = (Jk[0][1] * Jk[2][0] - Jk[0][0] * Jk[2][1]) * id;
        Ki[2][2] = (Jk[0][0] * Jk[1][1] - Jk[0][1] * Jk[1][0]) * id;
      }
#pragma unroll
      for (int i = 0; i < DIM; ++i) {
        b[i] = 0.0;
#pragma unroll
        for (int r = 0; r < DIM; ++r) {
          double a = 0.0;
#pragma unroll
          for (int m = 0; m < DIM; ++m) a += Ki[i][m] * Je[m][r];
          A[i][r] = a;
          b[i] += Ki[i][r] * dx[r];
        }
      }
    }
    // W_j = mean over e of k's basis function j
    double W[ND];
#pragma unroll
    for (int j = 0; j < ND; ++j) W[j] = 0.0;
    for (int q = 0; q < T->nqs; ++q) {
      double xk[DIM];
#pragma unroll
      for (int i = 0; i < DIM; ++i) {
        double v = b[i];
#pragma unroll
        for (int r = 0; r < DIM; ++r) v += A[i][r] * T->xs[q][r];
        xk[i] = v;
      }
      double phi[ND];
      basis_at<G, P>(T, xk, phi);
      const double wq = T->ws[q] / wsum;
#pragma unroll
      for (int j = 0; j < ND; ++j) W[j] += wq * phi[j];
    }
#pragma unroll
    for (int k = 0; k < NEQ; ++k) {
      double ex = 0.0;
#pragma unroll
      for (int j = 0; j < ND; ++j) {
        const long long idx = k * NDa + (long long)kc * ND + j;
        double v = (double)u[idx];
        if constexpr (DS) v += (double)ulo[idx];
        ex += v * W[j];
      }
      sum[k] += fabs(ume[k] - ex);
    }
  }
#pragma unroll
  for (int k = 0; k < NEQ; ++k) {
    const double mx = fabs(ume[k]);
    const double v = (mx < 1e-6 && sum[k] < 1e-6) ? 1.0 : fmin(1.0, 0.03 * mx / (sum[k] + 1e-6));
    val[k] = (R)v;
  }
}

// Limiter::update for one element (limiter.cpp:22-94): stencil = the element
// and its face neighbours (ElementToElementTable, limiter.cpp:115-123), the
// BJ-family indicator at the order-2 points of its interior faces
// (indicator_bj.cpp:88-200, updateYMin 15-86), then LimiterMultiplier::limit
// (limiter_multiplier.cpp:12-99, including the nd-fold application of the
// density factor, quirks Q4/Q5, and the last-hope vertex check) or
// LimiterFinDiff::limit (limiter_findiff.cpp:3-33, last equation only, Q6).
// The update reads only this element's values and the cell means, so it is
// done in place.  DS = true: the values are a float pair (u = hi, ulo = lo)
// and the multiplier update runs in double-single arithmetic.  The indicator
// (face-point values, stencil min/max, the +-1e-3 switches and the limiter
// function) is evaluated in FP64 for every state type, from the float state
// (and its low word) where the state is FP32, so that the FP32-bulk path takes
// the reference's FP64 branch decisions on the values it holds.
template <int G, int P, typename R, bool DS>
__global__ void __launch_bounds__(kGenericMaxBlock)
    k_limit_generic(const LimParams prm, R* __restrict__ u, float* __restrict__ ulo) {
  using E = El<G, P>;
  constexpr int DIM = E::DIM, ND = E::ND, NEQ = E::NEQ, NFPE = E::NFPE, NQL = E::NQL, NV = E::NV;
  __shared__ double sBl[NFPE][NQL][ND];
  __shared__ R sBv[NV][ND];
  const RefTables* T = prm.tab;
  // batched problems with a map of the active work: CTAs past it are idle
  if (prm.act_cum && (int)(blockIdx.x * blockDim.x) >= prm.act_cum[*prm.act_n]) return;
  for (int t = threadIdx.x; t < NFPE * NQL * ND; t += blockDim.x) {
    const int s = t % ND, q = (t / ND) % NQL, lf = t / (ND * NQL);
    sBl[lf][q][s] = T->Bl[lf][q][s];
  }
  for (int t = threadIdx.x; t < NV * ND; t += blockDim.x) sBv[t / ND][t % ND] = (R)T->Bv[t / ND][t % ND];
  __syncthreads();
  const int ne = prm.ne;
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  int pmap = -1;
  if (prm.act_cum) {  // batched problems: the i-th element of the active ones
    const int na = *prm.act_n;
    if (e >= prm.act_cum[na]) return;
    e = active_element(prm.act_cum, prm.act_pid, prm.poff, na, e, pmap);
  }
  if (e >= ne) return;
  const long long NDa = prm.ndofs;
  R gamma = (R)prm.gamma, cov = (R)prm.covolume;
  if (prm.prob) {
    const int pb = prm.act_cum ? pmap : prm.prob[e];
    if (!prm.pactive[pb]) return;
    gamma = (R)prm.pgamma[pb];
    cov = (R)prm.pcov[pb];
  }
  R el[NEQ][ND];
  float lo[DS ? NEQ : 1][DS ? ND : 1];
#pragma unroll
  for (int k = 0; k < NEQ; ++k)
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      el[k][j] = u[k * NDa + (long long)e * ND + j];
      if constexpr (DS) lo[k][j] = ulo[k * NDa + (long long)e * ND + j];
    }
  R um[NEQ];
  float umh[NEQ], uml[NEQ];
#pragma unroll
  for (int k = 0; k < NEQ; ++k) {
    const double m = prm.means[(long long)k * ne + e];
    um[k] = (R)m;
    umh[k] = (float)m;
    uml[k] = (float)(m - (double)umh[k]);
  }
  double minValue;
  double elind[NEQ];
  if (prm.indicator == 0) {
    minValue = 1.0;
#pragma unroll
    for (int k = 0; k < NEQ; ++k) elind[k] = 1.0;
  } else if (prm.indicator == 1) {
    minValue = 0.0;
#pragma unroll
    for (int k = 0; k < NEQ; ++k) elind[k] = 0.0;
  } else if (prm.indicator == 3) {
    R sv[NEQ];
    shu_indicator<G, P, DS>(prm, u, ulo, e, sv);
#pragma unroll
    for (int k = 0; k < NEQ; ++k) elind[k] = (double)sv[k];
    minValue = 1.0;  // FinDiff only: the Multi limiter is rejected with Shu
  } else {
    double mI[NEQ], MI[NEQ], yMin[NEQ], umd[NEQ];
#pragma unroll
    for (int k = 0; k < NEQ; ++k) {
      umd[k] = prm.means[(long long)k * ne + e];
      mI[k] = umd[k] < 1e9 ? umd[k] : 1e9;
      MI[k] = umd[k] > -1e9 ? umd[k] : -1e9;
      yMin[k] = 1e9;
    }
    for (int lf = 0; lf < NFPE; ++lf) {
      const int nb = prm.fnbr[lf * ne + e];
      if (nb < 0) continue;
#pragma unroll
      for (int k = 0; k < NEQ; ++k) {
        const double v = prm.means[(long long)k * ne + nb];
        mI[k] = v < mI[k] ? v : mI[k];
        MI[k] = v > MI[k] ? v : MI[k];
      }
    }
    // hanging faces: the elements across them are stencil cells
    // (ElementToElementTable, limiter.cpp:118-123) and the element's own
    // slave or master faces carry indicator points (limiter.cpp:125-161)
    unsigned ncfaces = 0;
    if (prm.ncidx && prm.ncidx[e] >= 0) {
      const int row = prm.ncidx[e];
      for (int c = prm.nc_ptr[row]; c < prm.nc_ptr[row + 1]; ++c) {
        const int f = prm.nc_ent[c] >> 1, side = prm.nc_ent[c] & 1;
        const int nb = prm.nc_face[f * 4 + (side ? 0 : 2)];
        ncfaces |= 1u << prm.nc_face[f * 4 + (side ? 3 : 1)];
#pragma unroll
        for (int k = 0; k < NEQ; ++k) {
          const double v = prm.means[(long long)k * ne + nb];
          mI[k] = v < mI[k] ? v : mI[k];
          MI[k] = v > MI[k] ? v : MI[k];
        }
      }
    }
    for (int lf = 0; lf < NFPE; ++lf) {
      const int nb = prm.fnbr[lf * ne + e];
      if (nb < 0 && !((ncfaces >> lf) & 1u)) continue;  // only interior faces carry indicator points
#pragma unroll
      for (int q = 0; q < NQL; ++q) {
#pragma unroll
        for (int k = 0; k < NEQ; ++k) {
          double v = 0.0;
#pragma unroll
          for (int j = 0; j < ND; ++j) {
            v += (double)el[k][j] * sBl[lf][q][j];
            if constexpr (DS) v += (double)lo[k][j] * sBl[lf][q][j];
          }
          const double diff = v - umd[k];
          double y;
          if (diff > 1e-3)
            y = (MI[k] - umd[k]) / diff;
          else if (diff < -1e-3)
            y = (mI[k] - umd[k]) / diff;
          else
            y = 1.0;
          if (prm.function == 0) {
            yMin[k] = y < yMin[k] ? y : yMin[k];
            yMin[k] = yMin[k] > 1.0 ? 1.0 : yMin[k];
          } else if (prm.function == 1) {
            const double yc = (y * y + 2.0 * y) / (y * y + y + 2.0);
            yMin[k] = yc < yMin[k] ? yc : yMin[k];
          } else {
            const double ys = 1.5;
            const double yr = y / ys;
            const double yc = y < 1.0 ? y + (3.0 - 2.0 * ys) * yr * yr + (ys - 2.0) * yr * yr * yr : 1.0;
            yMin[k] = yc < yMin[k] ? yc : yMin[k];
          }
        }
      }
    }
#pragma unroll
    for (int k = 0; k < NEQ; ++k) elind[k] = yMin[k];
    minValue = yMin[0];
  }
  if (prm.limiter == 1) {
    if constexpr (G != 2) {
      if (prm.quirks & 2) {
        // linearize (limiter_multiplier.cpp:101-178): mean + centre gradient
        // . (x_j - c); a linear state is its own linearisation, so once here
        // equals the reference's application before every multiplier pass
#pragma unroll
        for (int k = 0; k < NEQ; ++k) {
          double g[3] = {0.0, 0.0, 0.0};
#pragma unroll
          for (int d = 0; d < DIM; ++d)
#pragma unroll
            for (int j = 0; j < ND; ++j) {
              double v = (double)el[k][j];
              if constexpr (DS) v += (double)lo[k][j];
              g[d] += v * T->dcen[j][d];
            }
          const double m = prm.means[(long long)k * ne + e];
#pragma unroll
          for (int j = 0; j < ND; ++j) {
            double v = m;
#pragma unroll
            for (int d = 0; d < DIM; ++d) v -= g[d] * (0.5 - T->xlin[j][d]);
            el[k][j] = (R)v;
            if constexpr (DS) lo[k][j] = (float)(v - (double)(float)v);
          }
        }
      }
    }
    const int reps = (prm.quirks & 1) ? 1 : ND;
#pragma unroll
    for (int k = 0; k < NEQ; ++k)
      for (int r = 0; r < reps; ++r)
#pragma unroll
        for (int j = 0; j < ND; ++j) {
          if constexpr (DS) {
            float h = (float)el[k][j], l = lo[k][j];
            ds_add(h, l, -umh[k], -uml[k]);
            float ph, pl;
            ds_mul_f(h, l, (float)minValue, ph, pl);
            ds_add(ph, pl, umh[k], uml[k]);
            el[k][j] = (R)ph;
            lo[k][j] = pl;
          } else {
            el[k][j] = um[k] + (R)minValue * (el[k][j] - um[k]);
          }
        }
    if (prm.last_hope) {
      for (int v = 0; v < NV; ++v) {
        R fv[NEQ];
#pragma unroll
        for (int k = 0; k < NEQ; ++k) {
          R s = R(0);
#pragma unroll
          for (int j = 0; j < ND; ++j) {
            s += el[k][j] * sBv[v][j];
            if constexpr (DS) s += lo[k][j] * sBv[v][j];
          }
          fv[k] = s;
        }
        if (!state_is_physical<DIM>(fv, gamma, cov)) {
#pragma unroll
          for (int k = 0; k < NEQ; ++k)
#pragma unroll
            for (int j = 0; j < ND; ++j) {
              if constexpr (DS) {
                el[k][j] = (R)umh[k];
                lo[k][j] = uml[k];
              } else {
                el[k][j] = um[k];
              }
            }
        }
      }
    }
  } else {
    const bool totalInd = elind[NEQ - 1] < 0.999;
    if (totalInd) {
#pragma unroll
      for (int k = 0; k < NEQ; ++k)
#pragma unroll
        for (int j = 0; j < ND; ++j) {
          if constexpr (DS) {
            el[k][j] = (R)umh[k];
            lo[k][j] = uml[k];
          } else {
            el[k][j] = um[k];
          }
        }
    }
  }
#pragma unroll
  for (int k = 0; k < NEQ; ++k)
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      u[k * NDa + (long long)e * ND + j] = el[k][j];
      if constexpr (DS) ulo[k * NDa + (long long)e * ND + j] = lo[k][j];
    }
}

// ---- cell means (Averager::computeMeanValues, averager.cpp:84-109) -----------
// GridFunction::GetElementAverages = (int u) / (int 1); for affine elements the
// Jacobian cancels and the weights are the reference integrals of the basis
// functions normalised to sum 1.  lo (optional) is the low word of a float pair.
template <int G, int P, typename T>
__global__ void k_means_generic(int ne, long long ndofs, const RefTables* tab,
                                const T* __restrict__ u, const float* __restrict__ ulo,
                                double* __restrict__ means) {
  using E = El<G, P>;
  constexpr int ND = E::ND, NEQ = E::NEQ;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
#pragma unroll
  for (int k = 0; k < NEQ; ++k) {
    double m = 0.0;
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      double v = (double)u[k * ndofs + (long long)e * ND + j];
      if (ulo) v += (double)ulo[k * ndofs + (long long)e * ND + j];
      m += (tab->wmn_e ? tab->wmn_e[(long long)e * ND + j] : tab->wmean[j]) * v;
    }
    means[(long long)k * ne + e] = m;
  }
}

}  // namespace rkdg
