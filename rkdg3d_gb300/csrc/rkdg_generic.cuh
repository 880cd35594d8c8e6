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
// The FP32 right-hand-side and limiter kernels of small elements (Q1 quads,
// P1 triangles: NEQ * ND <= 16 values) are latency bound at the occupancy
// their registers allow: they run at most 128 threads per CTA and are compiled
// for six (right-hand side, 80 registers) or five (limiter, 96 registers) CTAs
// per SM with a few spilled values, which measured 7-8% faster on the batched
// and triangle workloads than the 12-16 warps of their uncapped registers.
// Larger elements would spill kilobytes at that cap and keep the default.
template <typename R, int NVAL>
__host__ __device__ constexpr bool generic_small() {
  return std::is_same<R, float>::value && NVAL <= 16;
}
template <typename R, int NVAL>
__host__ __device__ constexpr int generic_max_block() {
  return generic_small<R, NVAL>() ? 128 : kGenericMaxBlock;
}
template <typename R, int NVAL, bool LIMITER>
__host__ __device__ constexpr int generic_min_blocks() {
  return generic_small<R, NVAL>() ? (LIMITER ? 5 : 6) : 1;
}

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

// ---- vector access to the element rows of float arrays ------------------------
// An element's ND values of one variable are contiguous (byNODES layout, offset
// (k * ne + e) * ND).  The float arrays the FP32-bulk path reads and writes are
// the library's own allocations (256-byte aligned), so a row is 16-byte
// aligned when ND % 4 == 0 and 8-byte aligned when ND % 2 == 0.  Double
// arrays may be the caller's and are accessed element by element.
template <typename T, int ND>
struct RowVec {
  static constexpr int W = std::is_same<T, float>::value ? (ND % 4 == 0 ? 4 : (ND % 2 == 0 ? 2 : 1)) : 1;
};
template <int W, typename T>
__device__ __forceinline__ void ld_vec(const T* __restrict__ p, T* v) {
  if constexpr (W == 4) {
    const float4 t = *reinterpret_cast<const float4*>(p);
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
  } else if constexpr (W == 2) {
    const float2 t = *reinterpret_cast<const float2*>(p);
    v[0] = t.x; v[1] = t.y;
  } else {
    v[0] = p[0];
  }
}
template <int W, typename T>
__device__ __forceinline__ void st_vec(T* __restrict__ p, const T* v) {
  if constexpr (W == 4) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  } else if constexpr (W == 2) {
    *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
  } else {
    p[0] = v[0];
  }
}
// a whole row of N values
template <int N, typename T>
__device__ __forceinline__ void ld_row(const T* __restrict__ p, T* v) {
  constexpr int W = RowVec<T, N>::W;
#pragma unroll
  for (int i = 0; i < N; i += W) ld_vec<W>(p + i, v + i);
}
template <int N, typename T>
__device__ __forceinline__ void st_row(T* __restrict__ p, const T* v) {
  constexpr int W = RowVec<T, N>::W;
#pragma unroll
  for (int i = 0; i < N; i += W) st_vec<W>(p + i, v + i);
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
template <typename R>
__device__ __forceinline__ void segmented_max_commit(R v, int pb, unsigned long long* pmcs) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const R o = __shfl_down_sync(0xffffffffu, v, off);
    const int opb = __shfl_down_sync(0xffffffffu, pb, off);
    if (lane + off < 32 && opb == pb) v = fmax(v, o);
  }
  const int prev = __shfl_up_sync(0xffffffffu, pb, 1);
  if (pb >= 0 && (lane == 0 || prev != pb)) atomic_max_nonneg(&pmcs[pb], (double)v);
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

// (ch, cl) * (sh, sl) as a float pair: a tableau coefficient times a
// problem's dt, both float pairs.
__device__ __forceinline__ void ds_mul(float ch, float cl, float sh, float sl, float& ph, float& pl) {
  const float p = ch * sh;
  float e = fmaf(ch, sh, -p);
  e = fmaf(ch, sl, e);
  e = fmaf(cl, sh, e);
  ph = p + e;
  pl = e - (ph - p);
}

// Epilogue for one element and one equation: y[i], i < ND.  dts scales the
// coefficients of batched problems (1 otherwise): a double for a double
// state, a float pair (dts2) for the float path.
template <int ND, typename R>
__device__ __forceinline__ void epilogue(const EpiParams<R>& ep, long long base_idx,
                                         const R* y, const R* wmean, int ne, int e, int k,
                                         double dts, float2 dts2) {
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
    if (ep.means || ep.means32) store_mean(ep, (long long)k * ne + e, m);
  } else {
    // rows in vectors of W values; at most three previous stages (the
    // tableaux have up to four stages), unrolled so the coefficients stay in
    // registers
    constexpr int W = RowVec<float, ND>::W;
    float mh = 0.0f, ml = 0.0f;
    float ch[3], cl[3], cch = ep.ccur_hi, ccl = ep.ccur_lo;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      ch[j] = ep.cprev_hi[j];
      cl[j] = ep.cprev_lo[j];
    }
    if (ep.pdt || ep.pdt2) {  // unscaled tableau coefficients times the problem's dt
#pragma unroll
      for (int j = 0; j < 3; ++j)
        if (j < ep.nprev) ds_mul(ch[j], cl[j], dts2.x, dts2.y, ch[j], cl[j]);
      ds_mul(cch, ccl, dts2.x, dts2.y, cch, ccl);
    }
    if (!ep.final_stage) {
#pragma unroll
      for (int i0 = 0; i0 < ND; i0 += W) {
        const long long idx = base_idx + i0;
        float inc[W], bh[W], kp[W], v[W];
        ld_vec<W>(ep.baselo + idx, inc);
        ld_vec<W>(ep.basehi + idx, bh);
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          if (j < ep.nprev) {
            ld_vec<W>(ep.kprev[j] + idx, kp);
#pragma unroll
            for (int w = 0; w < W; ++w) inc[w] = fmaf(ch[j], kp[w], inc[w]);
          }
        }
#pragma unroll
        for (int w = 0; w < W; ++w) {
          inc[w] = fmaf(cch, y[i0 + w], inc[w]);
          v[w] = bh[w] + inc[w];
        }
        if (ep.kout) st_vec<W>(ep.kout + idx, y + i0);
        st_vec<W>(ep.out32 + idx, v);
#pragma unroll
        for (int w = 0; w < W; ++w) {
          float ph, pl;
          ds_mul_f(wmean[i0 + w], 0.0f, v[w], ph, pl);
          ds_add(mh, ml, ph, pl);
        }
      }
    } else {
#pragma unroll
      for (int i0 = 0; i0 < ND; i0 += W) {
        const long long idx = base_idx + i0;
        float sh[W], sl[W], kp[W], h[W], l[W];
#pragma unroll
        for (int w = 0; w < W; ++w) sh[w] = sl[w] = 0.0f;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          if (j < ep.nprev) {
            ld_vec<W>(ep.kprev[j] + idx, kp);
#pragma unroll
            for (int w = 0; w < W; ++w) {
              float ph, pl;
              ds_mul_f(ch[j], cl[j], kp[w], ph, pl);
              ds_add(sh[w], sl[w], ph, pl);
            }
          }
        }
        ld_vec<W>(ep.basehi + idx, h);
        ld_vec<W>(ep.baselo + idx, l);
#pragma unroll
        for (int w = 0; w < W; ++w) {
          float ph, pl;
          ds_mul_f(cch, ccl, y[i0 + w], ph, pl);
          ds_add(sh[w], sl[w], ph, pl);
          ds_add(h[w], l[w], sh[w], sl[w]);
        }
        st_vec<W>(ep.out32 + idx, h);
        st_vec<W>(ep.outlo + idx, l);
#pragma unroll
        for (int w = 0; w < W; ++w) {
          float ph, pl;
          ds_mul_f(wmean[i0 + w], 0.0f, h[w], ph, pl);
          ds_add(mh, ml, ph, pl);
          ds_add(mh, ml, wmean[i0 + w] * l[w], 0.0f);
        }
      }
    }
    // (mh, ml) stays normalised through ds_add: it is the float pair of the
    // mean as it stands
    if (ep.means32)
      ep.means32[(long long)k * ne + e] = make_float2(mh, ml);
    else if (ep.means)
      ep.means[(long long)k * ne + e] = (double)mh + (double)ml;
  }
}

// ---- right-hand side --------------------------------------------------------
template <int G, int P, typename R>
__global__ void __launch_bounds__(generic_max_block<R, El<G, P>::NEQ * El<G, P>::ND>(),
                                  generic_min_blocks<R, El<G, P>::NEQ * El<G, P>::ND, false>())
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
  float2 dts2 = make_float2(1.0f, 0.0f);
  if (prm.act_cum) {
    const int na = *prm.act_n;
    live = e < prm.act_cum[na];
    if (live) e = active_element(prm.act_cum, prm.act_pid, prm.poff, na, e, pb);
  }
  if (live && prm.prob) {
    if (!prm.act_cum) pb = prm.prob[e];
    live = prm.pactive[pb] != 0;
    if constexpr (std::is_same<R, float>::value) {
      // FP32 copies: no FP64 conversions per element
      gamma = prm.pgamma32 ? prm.pgamma32[pb] : (R)prm.pgamma[pb];
      cov = prm.pcov32 ? prm.pcov32[pb] : (R)prm.pcov[pb];
      if (ep.pdt2) {
        dts2 = ep.pdt2[pb];
      } else if (ep.pdt) {
        dts = ep.pdt[pb];
        const float h = (float)dts;
        dts2 = make_float2(h, (float)(dts - (double)h));
      }
    } else {
      gamma = (R)prm.pgamma[pb];
      cov = (R)prm.pcov[pb];
      if (ep.pdt) dts = ep.pdt[pb];
    }
  }
  if (live) {
    R acc[NEQ][ND];
#pragma unroll
    for (int k = 0; k < NEQ; ++k)
#pragma unroll
      for (int s = 0; s < ND; ++s) acc[k][s] = R(0);
    // small float elements (Q1 quads, P1 triangles): the element's own rows
    // are loaded once, with vector loads, for its faces and volume term, and
    // each neighbour's rows once per face
    constexpr bool HOIST = std::is_same<R, float>::value && NEQ * ND <= 16;
    R own[HOIST ? NEQ : 1][HOIST ? ND : 1];
    if constexpr (HOIST) {
#pragma unroll
      for (int k = 0; k < NEQ; ++k) ld_row<ND>(u + k * NDa + (long long)e * ND, own[k]);
    }
    const R* fg = (const R*)prm.fgeo;
    for (int lf = 0; lf < NFPE; ++lf) {
      const int nb = prm.fnbr[lf * ne + e];
      if (nb == -1) continue;
      const int code = prm.fcode[lf * ne + e];
      if constexpr (HOIST) {
        R n[DIM];
#pragma unroll
        for (int c = 0; c < DIM; ++c) n[c] = fg[(long long)(lf * (DIM + 1) + c) * ne + e];
        const R jac = fg[(long long)(lf * (DIM + 1) + DIM) * ne + e];
        const int side = (code >> 3) & 1, lfo = code & 7, pid = code >> 4;
        // sw: this element is side 2 of the face (the trace order of the
        // Riemann solver), as in the general path below
        const bool sw = nb >= 0 && side;
        R nbr[NEQ][ND];
        if (nb >= 0) {
#pragma unroll
          for (int k = 0; k < NEQ; ++k) ld_row<ND>(u + k * NDa + (long long)nb * ND, nbr[k]);
        }
        const R sg = side ? R(1) : R(-1);
        for (int q = 0; q < NQF; ++q) {
          const int q2 = sPerm[pid][q];
          R to[NEQ], tn[NEQ], s1[NEQ], s2[NEQ];
          const R* Bw = sB[lf][sw ? q2 : q];
#pragma unroll
          for (int k = 0; k < NEQ; ++k) {
            R v = R(0);
#pragma unroll
            for (int j = 0; j < ND; ++j) v += own[k][j] * Bw[j];
            to[k] = v;
          }
          if (nb >= 0) {
            const R* Bn = sB[lfo][sw ? q : q2];
#pragma unroll
            for (int k = 0; k < NEQ; ++k) {
              R v = R(0);
#pragma unroll
              for (int j = 0; j < ND; ++j) v += nbr[k][j] * Bn[j];
              tn[k] = v;
            }
#pragma unroll
            for (int k = 0; k < NEQ; ++k) {
              s1[k] = sw ? tn[k] : to[k];
              s2[k] = sw ? to[k] : tn[k];
            }
          } else {
#pragma unroll
            for (int k = 0; k < NEQ; ++k) s1[k] = to[k];
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
            for (int j = 0; j < ND; ++j) acc[k][j] += t * Bo[j];
          }
        }
      } else {
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
        for (int k = 0; k < NEQ; ++k) {
          if constexpr (HOIST)
            st[k] = own[k][m];
          else
            st[k] = u[k * NDa + (long long)e * ND + m];
        }
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
          epilogue<ND, R>(ep, k * NDa + (long long)e * ND, y, wl, ne, e, k, dts, dts2);
        } else {
          epilogue<ND, R>(ep, k * NDa + (long long)e * ND, y, sWm, ne, e, k, dts, dts2);
        }
      }
    }
  }
  if (prm.prob)
    segmented_max_commit<R>(lmax, live ? pb : -1, prm.pmcs);
  else
    block_max_commit<R>(lmax, prm.mcs);
}

// ---- limiter ------------------------------------------------------------------
// Cell means for the limiter: FP64, or the FP32 path's float pairs.
__device__ __forceinline__ bool mean_lt(double a, double b) { return a < b; }
__device__ __forceinline__ bool mean_lt(float2 a, float2 b) {
  return a.x < b.x || (a.x == b.x && a.y < b.y);
}
template <bool F32>
__device__ __forceinline__ typename std::conditional<F32, float2, double>::type load_mean(
    const LimParams& prm, long long i) {
  if constexpr (F32)
    return prm.means32[i];
  else
    return prm.means[i];
}
// a mean as a double (either representation)
__device__ __forceinline__ double mean_value(const LimParams& prm, long long i) {
  if (prm.means32) {
    const float2 m = prm.means32[i];
    return (double)m.x + (double)m.y;
  }
  return prm.means[i];
}

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
    ume[k] = mean_value(prm, (long long)k * ne + e);
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
// takes its branch decisions (face-point value minus mean against the +-1e-3
// switches, stencil min/max) on the values the state holds: in FP64 for a
// double state; for a float state in double-single arithmetic (face-point
// values from the float state and its low word with the float-pair basis
// table, about 44 significant bits, so a switch differs from FP64 only within
// ~1e-13 relative of its threshold), and the ratio and limiter function,
// which only scale the float multiplier, in FP32.  GB300's FP64 rate is a
// small fraction of its FP32 rate, and an FP64 indicator made the limiter
// the FP32 path's largest kernel.
template <int G, int P, typename R, bool DS>
__global__ void __launch_bounds__(generic_max_block<R, El<G, P>::NEQ * El<G, P>::ND>(),
                                  generic_min_blocks<R, El<G, P>::NEQ * El<G, P>::ND, true>())
    k_limit_generic(const LimParams prm, R* __restrict__ u, float* __restrict__ ulo) {
  using E = El<G, P>;
  constexpr int DIM = E::DIM, ND = E::ND, NEQ = E::NEQ, NFPE = E::NFPE, NQL = E::NQL, NV = E::NV;
  constexpr bool F32 = std::is_same<R, float>::value;
  // face-point basis: FP64, or a float pair (hi, lo) for a float state
  __shared__ typename std::conditional<F32, float2, double>::type sBl[NFPE][NQL][ND];
  __shared__ R sBv[NV][ND];
  const RefTables* T = prm.tab;
  // batched problems with a map of the active work: CTAs past it are idle
  if (prm.act_cum && (int)(blockIdx.x * blockDim.x) >= prm.act_cum[*prm.act_n]) return;
  for (int t = threadIdx.x; t < NFPE * NQL * ND; t += blockDim.x) {
    const int s = t % ND, q = (t / ND) % NQL, lf = t / (ND * NQL);
    const double b = T->Bl[lf][q][s];
    if constexpr (F32) {
      const float h = (float)b;
      sBl[lf][q][s] = make_float2(h, (float)(b - (double)h));
    } else {
      sBl[lf][q][s] = b;
    }
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
    if constexpr (F32) {
      gamma = prm.pgamma32 ? prm.pgamma32[pb] : (R)prm.pgamma[pb];
      cov = prm.pcov32 ? prm.pcov32[pb] : (R)prm.pcov[pb];
    } else {
      gamma = (R)prm.pgamma[pb];
      cov = (R)prm.pcov[pb];
    }
  }
  R el[NEQ][ND];
  float lo[DS ? NEQ : 1][DS ? ND : 1];
#pragma unroll
  for (int k = 0; k < NEQ; ++k) {
    ld_row<ND>(u + k * NDa + (long long)e * ND, el[k]);
    if constexpr (DS) ld_row<ND>(ulo + k * NDa + (long long)e * ND, lo[k]);
  }
  R um[NEQ];
  float umh[NEQ], uml[NEQ];
#pragma unroll
  for (int k = 0; k < NEQ; ++k) {
    if constexpr (F32) {
      const float2 m = prm.means32[(long long)k * ne + e];
      um[k] = m.x;
      umh[k] = m.x;
      uml[k] = m.y;
    } else {
      const double m = prm.means[(long long)k * ne + e];
      um[k] = (R)m;
      umh[k] = (float)m;
      uml[k] = (float)(m - (double)umh[k]);
    }
  }
  // the indicator's results: FP64, or FP32 for a float state (they only
  // scale the FP32 multiplier and feed FinDiff's 0.999 test, where no float
  // lies between 0.999 and its FP32 rounding)
  using IndT = typename std::conditional<F32, float, double>::type;
  IndT minValue;
  IndT elind[NEQ];
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
    for (int k = 0; k < NEQ; ++k) elind[k] = (IndT)sv[k];
    minValue = 1.0;  // FinDiff only: the Multi limiter is rejected with Shu
  } else {
    // stencil min / max of the means, started from the element's own mean
    // clamped to +-1e9: FP64, or for the float path float pairs compared
    // lexicographically (a normalised pair orders as its value)
    using MeanT = typename std::conditional<F32, float2, double>::type;
    MeanT mI[NEQ], MI[NEQ];
    IndT yMin[NEQ];
    double umd[NEQ];
#pragma unroll
    for (int k = 0; k < NEQ; ++k) {
      if constexpr (F32) {
        const float2 own = make_float2(umh[k], uml[k]);
        const float2 big = make_float2(1e9f, 0.0f), small = make_float2(-1e9f, 0.0f);
        mI[k] = mean_lt(own, big) ? own : big;
        MI[k] = mean_lt(small, own) ? own : small;
      } else {
        umd[k] = prm.means[(long long)k * ne + e];
        mI[k] = umd[k] < 1e9 ? umd[k] : 1e9;
        MI[k] = umd[k] > -1e9 ? umd[k] : -1e9;
      }
      yMin[k] = 1e9;
    }
    for (int lf = 0; lf < NFPE; ++lf) {
      const int nb = prm.fnbr[lf * ne + e];
      if (nb < 0) continue;
#pragma unroll
      for (int k = 0; k < NEQ; ++k) {
        const MeanT v = load_mean<F32>(prm, (long long)k * ne + nb);
        if (mean_lt(v, mI[k])) mI[k] = v;
        if (mean_lt(MI[k], v)) MI[k] = v;
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
          const MeanT v = load_mean<F32>(prm, (long long)k * ne + nb);
          if (mean_lt(v, mI[k])) mI[k] = v;
          if (mean_lt(MI[k], v)) MI[k] = v;
        }
      }
    }
    if constexpr (F32) {
      // double-single: the +-1e-3 switches as float pairs, the numerators of
      // the ratio (stencil max / min minus the mean) rounded to FP32
      const float th = 1e-3f, tl = (float)(1e-3 - (double)1e-3f);
      float nMax[NEQ], nMin[NEQ], yMf[NEQ];
#pragma unroll
      for (int k = 0; k < NEQ; ++k) {
        nMax[k] = (MI[k].x - umh[k]) + (MI[k].y - uml[k]);
        nMin[k] = (mI[k].x - umh[k]) + (mI[k].y - uml[k]);
        yMf[k] = 1e9f;
      }
      for (int lf = 0; lf < NFPE; ++lf) {
        const int nb = prm.fnbr[lf * ne + e];
        if (nb < 0 && !((ncfaces >> lf) & 1u)) continue;  // only interior faces carry indicator points
#pragma unroll
        for (int q = 0; q < NQL; ++q) {
#pragma unroll
          for (int k = 0; k < NEQ; ++k) {
            // value at the point minus the mean, as a float pair
            float sh = -umh[k], sl = -uml[k];
#pragma unroll
            for (int j = 0; j < ND; ++j) {
              const float2 bq = sBl[lf][q][j];
              const float x = (float)el[k][j];
              const float ph = x * bq.x;
              float pl = fmaf(x, bq.x, -ph);
              pl = fmaf(x, bq.y, pl);
              if constexpr (DS) pl = fmaf(lo[k][j], bq.x, pl);
              float t, er;
              two_sum(sh, ph, t, er);
              er += sl + pl;
              sh = t + er;
              sl = er - (sh - t);
            }
            const bool above = sh > th || (sh == th && sl > tl);
            const bool below = sh < -th || (sh == -th && sl < -tl);
            const float y = above ? nMax[k] / sh : (below ? nMin[k] / sh : 1.0f);
            if (prm.function == 0) {
              yMf[k] = fminf(fminf(y, yMf[k]), 1.0f);
            } else if (prm.function == 1) {
              const float yc = (y * y + 2.0f * y) / (y * y + y + 2.0f);
              yMf[k] = fminf(yc, yMf[k]);
            } else {
              const float ys = 1.5f;
              const float yr = y / ys;
              const float yc = y < 1.0f ? y + (3.0f - 2.0f * ys) * yr * yr + (ys - 2.0f) * yr * yr * yr : 1.0f;
              yMf[k] = fminf(yc, yMf[k]);
            }
          }
        }
      }
#pragma unroll
      for (int k = 0; k < NEQ; ++k) yMin[k] = yMf[k];
    } else {
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
          const double m = mean_value(prm, (long long)k * ne + e);
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
    const bool totalInd = elind[NEQ - 1] < IndT(0.999);
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
  for (int k = 0; k < NEQ; ++k) {
    st_row<ND>(u + k * NDa + (long long)e * ND, el[k]);
    if constexpr (DS) st_row<ND>(ulo + k * NDa + (long long)e * ND, lo[k]);
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
