// Register-resident hexahedral right-hand side: a team of 5 lanes per element,
// one lane per conserved variable.
//
// Every linear tensor operation of the DG right-hand side acts on one variable
// at a time, so a lane keeps its variable's (p+1)^3 nodal values and
// accumulators in registers and applies, with compile-time indices,
//   * the contraction along each face normal and the interpolation to the
//     (p+2)^2 face points (sum factorisation),
//   * the lifting of the face fluxes (transposed tensor trace),
//   * the collocated (phi, grad phi) operator one direction at a time,
//   * the inverse of the exact mass matrix det J (M1 x M1 x M1) as three
//     1D sweeps (fe_evolution.cpp:178-208).
// Only the pointwise nonlinear work needs all five variables: the nodal Euler
// flux (FE_Evolution::GetFlux, fe_evolution.cpp:219-245) and the numerical
// flux at the face points (FaceIntegrator::AssembleFaceVector,
// face_integrator.cpp:11-276, arguments ordered Elem1, Elem2, Elem1-outward
// normal); the team spreads those points over its lanes and exchanges the
// states through a small shared-memory buffer.  Six teams per warp, four warps
// per CTA (24 elements); the CTA loads its elements' DOFs and applies the
// Runge-Kutta epilogue with coalesced accesses.
#pragma once

#include "rkdg_common.h"
#include "rkdg_generic.cuh"
#include "rkdg_hex.cuh"
#include "rkdg_physics.cuh"

namespace rkdg {

template <typename R>
__device__ __forceinline__ const HexOps<R>& hex_ops(const HexOpsPair& h);
template <>
__device__ __forceinline__ const HexOps<float>& hex_ops<float>(const HexOpsPair& h) {
  return h.f;
}
template <>
__device__ __forceinline__ const HexOps<double>& hex_ops<double>(const HexOpsPair& h) {
  return h.d;
}

template <int P>
struct TeamSize {
  static constexpr int N1 = P + 1, NQ1 = P + 2, ND = N1 * N1 * N1, NQF = NQ1 * NQ1, NEQ = 5,
                       NF2 = N1 * N1;
  static constexpr int TPW = 6, WARPS = 4, EPB = TPW * WARPS, THREADS = 32 * WARPS;
  // per team exchange: max(traces + fluxes, volume fluxes), padded to whole
  // 32-word rows; team t of a warp starts xoff(t) words into its row so that
  // the team-parallel stores (30 lanes) and the warp-parallel flux reads (two
  // teams of 16 points) fall in distinct banks
  // MODE 0 (fused right-hand side) needs both; MODE 3 (shared-face rounds)
  // both plus the slot's 24 face-geometry values; MODE 1 (face pass) the two
  // traces only; MODE 2 (element pass) the volume fluxes only.
  static constexpr int XF = 3 * NEQ * NQF, XV = 3 * NEQ * ND;
  template <int MODE>
  __host__ __device__ static constexpr int xch() {
    return MODE == 1 ? 2 * NEQ * NQF
                     : (MODE == 2 ? XV : (MODE == 3 ? (XF + 24 > XV ? XF + 24 : XV) : (XF > XV ? XF : XV)));
  }
  // row stride: a multiple of 32 words with room for the offsets (team t + 1
  // may start up to 11 words earlier within its row than team t)
  template <int MODE>
  __host__ __device__ static constexpr int xstr() { return (xch<MODE>() + 11 + 31) & ~31; }
  template <int MODE>
  __host__ __device__ static constexpr int wstr() { return TPW * xstr<MODE>() + 32; }
  __host__ __device__ static constexpr int xoff(int t) { return 16 * (t & 1) + 5 * (t >> 1); }
  // MODE 3 keeps the CTA's schedule and the slots' exchange-row offsets
  // behind the exchange rows
  static constexpr size_t SCHED_BYTES = (sizeof(HexTeamSched) + 15) / 16 * 16;
  template <typename R, int MODE>
  static constexpr size_t smem_bytes() {
    return sizeof(R) * (size_t)(EPB * NEQ * ND + WARPS * wstr<MODE>()) +
           (MODE == 3 ? SCHED_BYTES + sizeof(int) * EPB : 0);
  }
  // MODE 3: a slot's face normals and |J_f| (6 x 4 values) sit in its
  // exchange row behind the two traces and the fluxes until the volume phase
  static constexpr int XG = 3 * NEQ * NQF;
  // resident CTAs per SM the register allocation is bounded for
  template <typename R, int MODE>
  __host__ __device__ static constexpr int min_ctas() {
    return sizeof(R) == 4 ? (MODE == 1 ? 5 : 4) : 2;
  }
};

// MFEM hexahedron local faces: normal axis and side.
__host__ __device__ constexpr int hex_face_axis(int lf) {
  return lf == 0 || lf == 5 ? 2 : (lf == 1 || lf == 3 ? 1 : 0);
}
__host__ __device__ constexpr int hex_face_side(int lf) {
  return lf == 2 || lf == 3 || lf == 5 ? 1 : 0;
}
template <int N1>
__host__ __device__ constexpr int hnode(int nax, int jn, int i0, int i1) {
  return nax == 0 ? jn + N1 * (i0 + N1 * i1) : (nax == 1 ? i0 + N1 * (jn + N1 * i1) : i0 + N1 * (i1 + N1 * jn));
}

// Contraction of a register array along face LF's normal: v[i0*N1+i1].
template <int P, int LF, typename R>
__device__ __forceinline__ void team_contract(const R (&u)[(P + 1) * (P + 1) * (P + 1)],
                                              const R* lend, R (&v)[(P + 1) * (P + 1)]) {
  constexpr int N1 = P + 1, NAX = hex_face_axis(LF), SD = hex_face_side(LF);
#pragma unroll
  for (int i0 = 0; i0 < N1; ++i0)
#pragma unroll
    for (int i1 = 0; i1 < N1; ++i1) {
      R s = R(0);
#pragma unroll
      for (int jn = 0; jn < N1; ++jn) s += lend[SD * N1 + jn] * u[hnode<N1>(NAX, jn, i0, i1)];
      v[i0 * N1 + i1] = s;
    }
}

// Same contraction reading the element's values from global memory.
template <int P, int LF, typename R>
__device__ __forceinline__ void team_contract_g(const R* __restrict__ ug, const R* lend,
                                                R (&v)[(P + 1) * (P + 1)]) {
  constexpr int N1 = P + 1, NAX = hex_face_axis(LF), SD = hex_face_side(LF);
#pragma unroll
  for (int i0 = 0; i0 < N1; ++i0)
#pragma unroll
    for (int i1 = 0; i1 < N1; ++i1) {
      R s = R(0);
#pragma unroll
      for (int jn = 0; jn < N1; ++jn) s += lend[SD * N1 + jn] * __ldg(ug + hnode<N1>(NAX, jn, i0, i1));
      v[i0 * N1 + i1] = s;
    }
}

template <int P, typename R>
__device__ __forceinline__ void team_contract_g_any(int lf, const R* __restrict__ ug, const R* lend,
                                                    R (&v)[(P + 1) * (P + 1)]) {
  switch (lf) {
    case 0: team_contract_g<P, 0>(ug, lend, v); break;
    case 1: team_contract_g<P, 1>(ug, lend, v); break;
    case 2: team_contract_g<P, 2>(ug, lend, v); break;
    case 3: team_contract_g<P, 3>(ug, lend, v); break;
    case 4: team_contract_g<P, 4>(ug, lend, v); break;
    default: team_contract_g<P, 5>(ug, lend, v); break;
  }
}

// v (N1 x N1 on the face's tangential axes) -> values at the NQ1 x NQ1 face
// points in tensor order a + NQ1*b, written to dst[(a + NQ1*b) * ST].
template <int P, int ST, typename R>
__device__ __forceinline__ void team_interp(const R (&v)[(P + 1) * (P + 1)], const R* l1d, R* dst) {
  constexpr int N1 = P + 1, NQ1 = P + 2;
  if constexpr (std::is_same<R, float>::value && NQ1 % 2 == 0) {
    // packed FP32 (two face-point rows per instruction); each component is
    // the same fused chain as the scalar form below, so results are identical
    float2 w[NQ1 / 2][N1];
#pragma unroll
    for (int pa = 0; pa < NQ1 / 2; ++pa)
#pragma unroll
      for (int i1 = 0; i1 < N1; ++i1) {
        float2 s = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int i0 = 0; i0 < N1; ++i0)
          s = __ffma2_rn(make_float2(l1d[(2 * pa) * N1 + i0], l1d[(2 * pa + 1) * N1 + i0]),
                         make_float2(v[i0 * N1 + i1], v[i0 * N1 + i1]), s);
        w[pa][i1] = s;
      }
#pragma unroll
    for (int b = 0; b < NQ1; ++b)
#pragma unroll
      for (int pa = 0; pa < NQ1 / 2; ++pa) {
        float2 s = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int i1 = 0; i1 < N1; ++i1)
          s = __ffma2_rn(make_float2(l1d[b * N1 + i1], l1d[b * N1 + i1]), w[pa][i1], s);
        dst[(2 * pa + NQ1 * b) * ST] = s.x;
        dst[(2 * pa + 1 + NQ1 * b) * ST] = s.y;
      }
  } else {
    R w[NQ1][N1];
#pragma unroll
    for (int a = 0; a < NQ1; ++a)
#pragma unroll
      for (int i1 = 0; i1 < N1; ++i1) {
        R s = R(0);
#pragma unroll
        for (int i0 = 0; i0 < N1; ++i0) s += l1d[a * N1 + i0] * v[i0 * N1 + i1];
        w[a][i1] = s;
      }
#pragma unroll
    for (int b = 0; b < NQ1; ++b)
#pragma unroll
      for (int a = 0; a < NQ1; ++a) {
        R s = R(0);
#pragma unroll
        for (int i1 = 0; i1 < N1; ++i1) s += l1d[b * N1 + i1] * w[a][i1];
        dst[(a + NQ1 * b) * ST] = s;
      }
  }
}

// Lift face values f[(a + NQ1*b) * ST] of face LF into the accumulators.
template <int P, int LF, int ST, typename R>
__device__ __forceinline__ void team_lift(const R* f, const R* l1d, const R* lend,
                                          R (&acc)[(P + 1) * (P + 1) * (P + 1)]) {
  constexpr int N1 = P + 1, NQ1 = P + 2, NAX = hex_face_axis(LF), SD = hex_face_side(LF);
  R w[N1][NQ1];
#pragma unroll
  for (int i0 = 0; i0 < N1; ++i0)
#pragma unroll
    for (int b = 0; b < NQ1; ++b) {
      R s = R(0);
#pragma unroll
      for (int a = 0; a < NQ1; ++a) s += l1d[a * N1 + i0] * f[(a + NQ1 * b) * ST];
      w[i0][b] = s;
    }
#pragma unroll
  for (int i0 = 0; i0 < N1; ++i0)
#pragma unroll
    for (int i1 = 0; i1 < N1; ++i1) {
      R s = R(0);
#pragma unroll
      for (int b = 0; b < NQ1; ++b) s += l1d[b * N1 + i1] * w[i0][b];
#pragma unroll
      for (int jn = 0; jn < N1; ++jn) acc[hnode<N1>(NAX, jn, i0, i1)] += lend[SD * N1 + jn] * s;
    }
}

// Same contraction reading the element's staged values from shared memory.
template <int P, int LF, typename R>
__device__ __forceinline__ void team_contract_s(const R* su, const R* lend, R (&v)[(P + 1) * (P + 1)]) {
  constexpr int N1 = P + 1, NAX = hex_face_axis(LF), SD = hex_face_side(LF);
#pragma unroll
  for (int i0 = 0; i0 < N1; ++i0)
#pragma unroll
    for (int i1 = 0; i1 < N1; ++i1) {
      R s = R(0);
#pragma unroll
      for (int jn = 0; jn < N1; ++jn) s += lend[SD * N1 + jn] * su[hnode<N1>(NAX, jn, i0, i1)];
      v[i0 * N1 + i1] = s;
    }
}

template <int P, typename R>
__device__ __forceinline__ void team_contract_s_any(int lf, const R* su, const R* lend,
                                                    R (&v)[(P + 1) * (P + 1)]) {
  switch (lf) {
    case 0: team_contract_s<P, 0>(su, lend, v); break;
    case 1: team_contract_s<P, 1>(su, lend, v); break;
    case 2: team_contract_s<P, 2>(su, lend, v); break;
    case 3: team_contract_s<P, 3>(su, lend, v); break;
    case 4: team_contract_s<P, 4>(su, lend, v); break;
    default: team_contract_s<P, 5>(su, lend, v); break;
  }
}

template <int P, typename R>
__device__ __forceinline__ void team_contract_any(int lf, const R (&u)[(P + 1) * (P + 1) * (P + 1)],
                                                  const R* lend, R (&v)[(P + 1) * (P + 1)]) {
  switch (lf) {
    case 0: team_contract<P, 0>(u, lend, v); break;
    case 1: team_contract<P, 1>(u, lend, v); break;
    case 2: team_contract<P, 2>(u, lend, v); break;
    case 3: team_contract<P, 3>(u, lend, v); break;
    case 4: team_contract<P, 4>(u, lend, v); break;
    default: team_contract<P, 5>(u, lend, v); break;
  }
}

template <int P, int ST, typename R>
__device__ __forceinline__ void team_lift_any(int lf, const R* f, const R* l1d, const R* lend,
                                              R (&acc)[(P + 1) * (P + 1) * (P + 1)]) {
  switch (lf) {
    case 0: team_lift<P, 0, ST>(f, l1d, lend, acc); break;
    case 1: team_lift<P, 1, ST>(f, l1d, lend, acc); break;
    case 2: team_lift<P, 2, ST>(f, l1d, lend, acc); break;
    case 3: team_lift<P, 3, ST>(f, l1d, lend, acc); break;
    case 4: team_lift<P, 4, ST>(f, l1d, lend, acc); break;
    default: team_lift<P, 5, ST>(f, l1d, lend, acc); break;
  }
}

// Axis-templated forms with the face's side (0: at 0, 1: at 1 along the
// normal axis NAX) at run time: the same instructions for both faces of an
// axis, so that teams of a warp visiting opposite faces of one axis do not
// diverge.  Same arithmetic, in the same order, as the LF-templated forms.
template <int P, int NAX, typename R>
__device__ __forceinline__ void team_contract_s_ax(int sd, const R* su, const R* lend,
                                                   R (&v)[(P + 1) * (P + 1)]) {
  constexpr int N1 = P + 1;
  R le[N1];
#pragma unroll
  for (int jn = 0; jn < N1; ++jn) le[jn] = sd ? lend[N1 + jn] : lend[jn];
#pragma unroll
  for (int i0 = 0; i0 < N1; ++i0)
#pragma unroll
    for (int i1 = 0; i1 < N1; ++i1) {
      R s = R(0);
#pragma unroll
      for (int jn = 0; jn < N1; ++jn) s += le[jn] * su[hnode<N1>(NAX, jn, i0, i1)];
      v[i0 * N1 + i1] = s;
    }
}

template <int P, int NAX, int ST, typename R>
__device__ __forceinline__ void team_lift_ax(int sd, const R* f, const R* l1d, const R* lend,
                                             R (&acc)[(P + 1) * (P + 1) * (P + 1)]) {
  constexpr int N1 = P + 1, NQ1 = P + 2;
  R le[N1];
#pragma unroll
  for (int jn = 0; jn < N1; ++jn) le[jn] = sd ? lend[N1 + jn] : lend[jn];
  R w[N1][NQ1];
#pragma unroll
  for (int i0 = 0; i0 < N1; ++i0)
#pragma unroll
    for (int b = 0; b < NQ1; ++b) {
      R s = R(0);
#pragma unroll
      for (int a = 0; a < NQ1; ++a) s += l1d[a * N1 + i0] * f[(a + NQ1 * b) * ST];
      w[i0][b] = s;
    }
#pragma unroll
  for (int i0 = 0; i0 < N1; ++i0)
#pragma unroll
    for (int i1 = 0; i1 < N1; ++i1) {
      R s = R(0);
#pragma unroll
      for (int b = 0; b < NQ1; ++b) s += l1d[b * N1 + i1] * w[i0][b];
#pragma unroll
      for (int jn = 0; jn < N1; ++jn) acc[hnode<N1>(NAX, jn, i0, i1)] += le[jn] * s;
    }
}

// The values of one variable of an element ordered along its local face LFO,
// nbv[(i0*N1 + i1)*N1 + jn] = u[node(jn along the normal, i0, i1)], with
// compile-time offsets (GLOBAL: read-only global loads, else shared memory).
template <int P, int LFO, bool GLOBAL, typename R>
__device__ __forceinline__ void team_gather(const R* src, R (&nbv)[(P + 1) * (P + 1) * (P + 1)]) {
  constexpr int N1 = P + 1, NAX = hex_face_axis(LFO);
#pragma unroll
  for (int i0 = 0; i0 < N1; ++i0)
#pragma unroll
    for (int i1 = 0; i1 < N1; ++i1)
#pragma unroll
      for (int jn = 0; jn < N1; ++jn) {
        const R* a = src + hnode<N1>(NAX, jn, i0, i1);
        nbv[(i0 * N1 + i1) * N1 + jn] = GLOBAL ? __ldg(a) : *a;
      }
}

template <int P, bool GLOBAL, typename R>
__device__ __forceinline__ void team_gather_any(int lfo, const R* src,
                                                R (&nbv)[(P + 1) * (P + 1) * (P + 1)]) {
  switch (lfo) {
    case 0: team_gather<P, 0, GLOBAL>(src, nbv); break;
    case 1: team_gather<P, 1, GLOBAL>(src, nbv); break;
    case 2: team_gather<P, 2, GLOBAL>(src, nbv); break;
    case 3: team_gather<P, 3, GLOBAL>(src, nbv); break;
    case 4: team_gather<P, 4, GLOBAL>(src, nbv); break;
    default: team_gather<P, 5, GLOBAL>(src, nbv); break;
  }
}

// Dispatch on a face's normal axis only (three code copies instead of six;
// the side enters at run time).
template <int P, bool GLOBAL, typename R>
__device__ __forceinline__ void team_gather_axis(int lfo, const R* src,
                                                 R (&nbv)[(P + 1) * (P + 1) * (P + 1)]) {
  switch (hex_face_axis(lfo)) {  // the gather order depends on the axis only
    case 0: team_gather<P, 2, GLOBAL>(src, nbv); break;
    case 1: team_gather<P, 1, GLOBAL>(src, nbv); break;
    default: team_gather<P, 0, GLOBAL>(src, nbv); break;
  }
}
template <int P, typename R>
__device__ __forceinline__ void team_contract_s_axis(int lf, const R* su, const R* lend,
                                                     R (&v)[(P + 1) * (P + 1)]) {
  switch (hex_face_axis(lf)) {
    case 0: team_contract_s_ax<P, 0>(hex_face_side(lf), su, lend, v); break;
    case 1: team_contract_s_ax<P, 1>(hex_face_side(lf), su, lend, v); break;
    default: team_contract_s_ax<P, 2>(hex_face_side(lf), su, lend, v); break;
  }
}
template <int P, int ST, typename R>
__device__ __forceinline__ void team_lift_axis(int lf, const R* f, const R* l1d, const R* lend,
                                               R (&acc)[(P + 1) * (P + 1) * (P + 1)]) {
  switch (hex_face_axis(lf)) {
    case 0: team_lift_ax<P, 0, ST>(hex_face_side(lf), f, l1d, lend, acc); break;
    case 1: team_lift_ax<P, 1, ST>(hex_face_side(lf), f, l1d, lend, acc); break;
    default: team_lift_ax<P, 2, ST>(hex_face_side(lf), f, l1d, lend, acc); break;
  }
}

// Phase 1 of one face (runtime index LF) for the team's variable k: the own
// trace and, across an interior face, the neighbour's trace at the face
// points, stored point-major (To[q*NEQ + k], Tn[q*NEQ + k]).  The own values
// are read from the staged tile su (compile-time offsets, a small switch over
// the face); the neighbour's values come from the staged tile when it is
// there, else from global memory, with compile-time offsets per face.
template <int P, typename R>
__device__ __forceinline__ void team_traces(const int LF, const R* __restrict__ ug, long long NDa,
                                            int k, const R* su, R* xch,
                                            const R* l1d, const R* lend, int nb, int code,
                                            const R* sU, int e0, int nel) {
  using S = TeamSize<P>;
  constexpr int N1 = S::N1, ND = S::ND, NQF = S::NQF, NEQ = S::NEQ, NF2 = S::NF2;
  R* To = xch;
  R* Tn = To + NEQ * NQF;
  const int lfo = code & 7;
  // issue the neighbour's loads first; the own-side work hides their latency
  R nbv[ND];
  if (nb >= 0) {
    if (nb >= e0 && nb < e0 + nel)  // neighbour staged in this tile
      team_gather_axis<P, false>(lfo, sU + ((nb - e0) * NEQ + k) * ND, nbv);
    else
      team_gather_axis<P, true>(lfo, ug + k * NDa + (long long)nb * ND, nbv);
  }
  {
    R v[N1 * N1];
    team_contract_s_axis<P>(LF, su, lend, v);
    team_interp<P, NEQ>(v, l1d, To + k);
  }
  if (nb >= 0) {
    const int sdn = hex_face_side(lfo);
    R v[N1 * N1];
#pragma unroll
    for (int r = 0; r < NF2; ++r) {
      R s = R(0);
#pragma unroll
      for (int jn = 0; jn < N1; ++jn) s += lend[sdn * N1 + jn] * nbv[r * N1 + jn];
      v[r] = s;
    }
    team_interp<P, NEQ>(v, l1d, Tn + k);
  }
}

// Phase 2 of face LF: the numerical flux at the face points of all the warp's
// elements, spread over the 32 lanes (point pt of the warp = team pt / NQF,
// point pt % NQF); arguments in Elem1, Elem2 order with the Elem1-outward
// normal (face_integrator.cpp:11-276), boundary faces through the boundary
// condition's right state.  MODE 0 writes sign * w_q * |J_f| * Fhat to the
// team's Fh[q*NEQ + k] in its own tensor order.  MODE 1 (face pass) handles
// only the faces the element owns (Elem1 of an interior face, or a boundary
// face) and writes the value into the flux slots of both elements
// (prm.fslot[element][local face][k][tensor point]) with each side's sign.
template <int P, typename R, int MODE>
__device__ __forceinline__ void warp_fluxes(const int LF, const RhsParams& prm, int lane, int wel0,
                                            int nel, R* wx, const R* wf,
                                            const unsigned char (*perm)[(P + 2) * (P + 2)],
                                            const unsigned char (*fab)[(P + 2) * (P + 2)],
                                            const int (*sfnb)[6], const unsigned char (*sfcd)[6],
                                            int e0, R gamma, R cov, R& lmax) {
  using S = TeamSize<P>;
  constexpr int NQF = S::NQF, NEQ = S::NEQ, TPW = S::TPW, XSTR = S::template xstr<MODE>();
#pragma unroll 1
  for (int pt = lane; pt < TPW * NQF; pt += 32) {
    const int t = pt / NQF, q = pt - t * NQF;
    const int el = wel0 + t;
    if (el >= nel) continue;
    const int nb = sfnb[el][LF];
    if (nb == -1) continue;
    const int code = sfcd[el][LF];
    const int side = (code >> 3) & 1, lfo = code & 7, pid = code >> 4;
    if (MODE == 1 && side) continue;  // the face's Elem1 evaluates it
    R* To = wx + t * XSTR + S::xoff(t);
    const R* Tn = To + NEQ * NQF;
    R* Fh = To + 2 * NEQ * NQF;
    const R* fg = (const R*)prm.fgeo + (long long)(LF * 4) * prm.ne + e0 + el;
    R n[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) n[c] = __ldg(fg + (long long)c * prm.ne);
    const R jac = __ldg(fg + 3LL * prm.ne);
    R s1[NEQ], s2[NEQ];
    int own = fab[LF][q], other = 0;
    if (nb >= 0) {
      const int q2 = perm[pid][q];
      const int a1 = side ? fab[lfo][q] : fab[LF][q];
      const int a2 = side ? fab[LF][q2] : fab[lfo][q2];
      const R* T1 = side ? Tn : To;
      const R* T2 = side ? To : Tn;
#pragma unroll
      for (int kk = 0; kk < NEQ; ++kk) {
        s1[kk] = T1[a1 * NEQ + kk];
        s2[kk] = T2[a2 * NEQ + kk];
      }
      if (side) own = a2;
      other = a2;
    } else {
#pragma unroll
      for (int kk = 0; kk < NEQ; ++kk) s1[kk] = To[own * NEQ + kk];
      const BCSlot& bc = prm.bc[-2 - nb];
      right_state<3>(bc.type, bc.state, s1, s2, n, gamma, cov, (R)prm.rgas);
    }
    R F[NEQ];
    const R sp = checked_speed(prm, riemann<3>(s1, s2, n, F, gamma, cov, prm.rs, prm.avg), e0 + el);
    lmax = fmax(lmax, sp);
    if constexpr (MODE == 1) {
      R* fs = (R*)prm.fslot;
      const R w = wf[q] * jac;
      R* so = fs + ((long long)(e0 + el) * 6 + LF) * (NEQ * NQF) + own;
#pragma unroll
      for (int kk = 0; kk < NEQ; ++kk) so[kk * NQF] = -w * F[kk];
      if (nb >= 0) {
        R* sn = fs + ((long long)nb * 6 + lfo) * (NEQ * NQF) + other;
#pragma unroll
        for (int kk = 0; kk < NEQ; ++kk) sn[kk * NQF] = w * F[kk];
      }
    } else {
      const R w = (side ? R(1) : R(-1)) * wf[q] * jac;
#pragma unroll
      for (int kk = 0; kk < NEQ; ++kk) Fh[own * NEQ + kk] = w * F[kk];
    }
  }
}

// MODE 3: the rounds of the CTA's schedule (HexTeamSched).  In round r each
// slot's team forms its own trace at its round-r face (To of its exchange
// row); the CTA's threads, five per job, form the traces of the out-of-CTA
// neighbours listed for the round (Tn of the listed slot's row); after a
// barrier the CTA evaluates each listed face once, all threads over all
// points, in Elem1, Elem2 order (face_integrator.cpp:11-276), writing
// sign * w_q * |J_f| * Fhat to the evaluating slot's Fh and, across an
// in-CTA face, the opposite-signed value to the partner's Fh; after a second
// barrier each team lifts its face.  A face inside the CTA thus costs one
// trace per side and one numerical flux, where the fused kernel (MODE 0)
// forms both traces and the flux once per side.
template <int P, typename R>
__device__ __forceinline__ void shared_rounds(const RhsParams& prm, const R* __restrict__ u,
                                              long long NDa, const HexTeamSched& S, R* sX,
                                              const int* rowoff, R* xch,
                                              const R* su, int el, bool act, int k, const R* l1d,
                                              const R* lend, const R* wf,
                                              const unsigned char (*perm)[(P + 2) * (P + 2)],
                                              const unsigned char (*fab)[(P + 2) * (P + 2)],
                                              const int (*sfnb)[6], const unsigned char (*sfcd)[6],
                                              R gamma, R cov, R& lmax,
                                              R (&acc)[(P + 1) * (P + 1) * (P + 1)]) {
  using T = TeamSize<P>;
  constexpr int N1 = T::N1, ND = T::ND, NQF = T::NQF, NEQ = T::NEQ, NF2 = T::NF2;
  constexpr int XG = T::XG;
  auto row = [&](int sl) { return sX + rowoff[sl]; };
  const int tid = threadIdx.x;
  const int jb = tid / NEQ, jk = tid - NEQ * jb;  // this thread's job: (listed slot, variable)
#pragma unroll 1
  for (int r = 0; r < S.nr; ++r) {
    const int lf = act ? S.rlf[el][r] : 0xFF;
    const bool mine = lf != 0xFF && sfnb[el][lf] != -1;
    const bool job = jb < S.njb[r];
    const int ax = S.rax[r];  // uniform over the CTA: axis-templated code, side at run time
    int jsl = 0, jlfo = 0;
    R nbv[ND];
    if (job) {  // issue the neighbour's loads first; the own trace hides their latency
      jsl = S.jb[r][jb];
      const int jlf = S.rlf[jsl][r];
      jlfo = sfcd[jsl][jlf] & 7;
      const R* src = u + jk * NDa + (long long)sfnb[jsl][jlf] * ND;
      switch (ax) {  // the gather order depends on the face's axis only
        case 0: team_gather<P, 2, true>(src, nbv); break;
        case 1: team_gather<P, 1, true>(src, nbv); break;
        case 2: team_gather<P, 0, true>(src, nbv); break;
        default: team_gather_any<P, true>(jlfo, src, nbv); break;
      }
    }
    if (mine) {
      R v[NF2];
      switch (ax) {
        case 0: team_contract_s_ax<P, 0>(hex_face_side(lf), su, lend, v); break;
        case 1: team_contract_s_ax<P, 1>(hex_face_side(lf), su, lend, v); break;
        case 2: team_contract_s_ax<P, 2>(hex_face_side(lf), su, lend, v); break;
        default: team_contract_s_any<P>(lf, su, lend, v); break;
      }
      team_interp<P, NEQ>(v, l1d, xch + k);
    }
    if (job) {
      const int sdn = hex_face_side(jlfo);
      R v[NF2];
#pragma unroll
      for (int i = 0; i < NF2; ++i) {
        R s = R(0);
#pragma unroll
        for (int jn = 0; jn < N1; ++jn) s += lend[sdn * N1 + jn] * nbv[i * N1 + jn];
        v[i] = s;
      }
      team_interp<P, NEQ>(v, l1d, row(jsl) + NEQ * NQF + jk);
    }
    __syncthreads();
#pragma unroll 1
    for (int pt = tid; pt < S.nfl[r] * NQF; pt += blockDim.x) {
      const int f = pt / NQF, q = pt - f * NQF;
      const unsigned d = S.fd[r][f];
      const int fs = d & 31, flf = (d >> 5) & 7, prt = (d >> 8) & 31, side = (d >> 13) & 1;
      const int lfo = (d >> 14) & 7, pid = (d >> 17) & 7;
      const bool interior = (d >> 20) & 1;
      int nb = 0;
      if (!interior) {
        nb = sfnb[fs][flf];  // boundary condition slot of the context's current set
        if (nb == -1) continue;
      }
      R* To = row(fs);
      const R* Tn = prt != 31 ? row(prt) : To + NEQ * NQF;
      const R* g = To + XG + flf * 4;
      R n[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) n[c] = g[c];
      const R jac = g[3];
      R s1[NEQ], s2[NEQ];
      int own = fab[flf][q], other = 0;
      if (interior) {
        const int q2 = perm[pid][q];
        const int a1 = side ? fab[lfo][q] : fab[flf][q];
        const int a2 = side ? fab[flf][q2] : fab[lfo][q2];
        const R* T1 = side ? Tn : To;
        const R* T2 = side ? To : Tn;
#pragma unroll
        for (int kk = 0; kk < NEQ; ++kk) {
          s1[kk] = T1[a1 * NEQ + kk];
          s2[kk] = T2[a2 * NEQ + kk];
        }
        if (side) own = a2;
        other = a2;
      } else {
#pragma unroll
        for (int kk = 0; kk < NEQ; ++kk) s1[kk] = To[own * NEQ + kk];
        const BCSlot& bc = prm.bc[-2 - nb];
        right_state<3>(bc.type, bc.state, s1, s2, n, gamma, cov, (R)prm.rgas);
      }
      R F[NEQ];
      const R sp = checked_speed(prm, riemann<3>(s1, s2, n, F, gamma, cov, prm.rs, prm.avg), S.el[fs]);
      lmax = fmax(lmax, sp);
      const R w = wf[q] * jac;
      const R wo = side ? w : -w;
      R* Fh = To + 2 * NEQ * NQF;
#pragma unroll
      for (int kk = 0; kk < NEQ; ++kk) Fh[own * NEQ + kk] = wo * F[kk];
      if (prt != 31) {  // the partner is the face's Elem2
        R* Fp = row(prt) + 2 * NEQ * NQF;
#pragma unroll
        for (int kk = 0; kk < NEQ; ++kk) Fp[other * NEQ + kk] = w * F[kk];
      }
    }
    __syncthreads();
    if (mine && !prm.faces_only) {
      const R* fh = xch + 2 * NEQ * NQF + k;
      switch (ax) {
        case 0: team_lift_ax<P, 0, NEQ>(hex_face_side(lf), fh, l1d, lend, acc); break;
        case 1: team_lift_ax<P, 1, NEQ>(hex_face_side(lf), fh, l1d, lend, acc); break;
        case 2: team_lift_ax<P, 2, NEQ>(hex_face_side(lf), fh, l1d, lend, acc); break;
        default: team_lift_any<P, NEQ>(lf, fh, l1d, lend, acc); break;
      }
    }
  }
}

// MODE 0: the whole right-hand side of the CTA's elements (every face
// evaluated by both its elements).  MODE 1 + MODE 2 (two launches): a face pass
// that evaluates each face once into per-element flux slots, then an element
// pass that lifts the six slots and adds the volume term, inverse mass and
// Runge-Kutta epilogue.  MODE 3: the CTA's slots hold the elements its
// schedule names, and faces inside the CTA are evaluated once
// (shared_rounds); volume term and epilogue as MODE 0.
template <int P, typename R, int MODE>
__global__ void __launch_bounds__(128, TeamSize<P>::template min_ctas<R, MODE>())
    k_rhs_hex_team(const __grid_constant__ RhsParams prm, const R* __restrict__ u,
                   const EpiParams<R> ep) {
  using S = TeamSize<P>;
  constexpr int N1 = S::N1, ND = S::ND, NQF = S::NQF, NEQ = S::NEQ, EPB = S::EPB;
  constexpr int XSTR = S::template xstr<MODE>(), WSTR = S::template wstr<MODE>();
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ unsigned char sPerm[RKDG_HEX_MAX_PERM][NQF];
  __shared__ unsigned char sFab[6][NQF];
  R* sm = reinterpret_cast<R*>(smraw);
  const HexOps<R>& H = hex_ops<R>(prm.hops);  // 1D operators (kernel parameters)
  const R* tL1 = H.l1d;         // [NQ1][N1]
  const R* tLend = H.lend;      // [2][N1]
  const R* tD1 = H.d1;          // [N1][N1]
  const R* tMinv = H.minv1;     // [N1][N1]
  const R* tW1 = H.w1;          // [N1]
  const R* tWf = H.wf;          // [NQF]
  R* sU = sm;                   // [EPB][NEQ][ND]
  R* sX = sU + EPB * NEQ * ND;  // [WARPS][WSTR] team exchange rows
  const RefTables* T = prm.tab;
  const int tid = threadIdx.x;
  const int ne = prm.ne;
  const int e0 = blockIdx.x * EPB;
  HexTeamSched* sS = nullptr;    // MODE 3: this CTA's schedule
  int* sRowOff = nullptr;        // MODE 3: exchange-row offset of each slot
  if constexpr (MODE == 3) {
    sS = reinterpret_cast<HexTeamSched*>(sX + S::WARPS * WSTR);
    sRowOff = reinterpret_cast<int*>(reinterpret_cast<unsigned char*>(sS) + S::SCHED_BYTES);
    const int* src = reinterpret_cast<const int*>(prm.hsched + blockIdx.x);
    for (int t = tid; t < (int)(sizeof(HexTeamSched) / 4); t += blockDim.x)
      reinterpret_cast<int*>(sS)[t] = src[t];
    if (tid < EPB) sRowOff[tid] = (tid / S::TPW) * WSTR + (tid % S::TPW) * XSTR + S::xoff(tid % S::TPW);
    __syncthreads();
  }
  // element of slot el: consecutive elements, or the schedule's (MODE 3)
  auto eid = [&](int el) { return MODE == 3 ? sS->el[el] : e0 + el; };
  for (int t = tid; t < min(T->nperm, RKDG_HEX_MAX_PERM) * NQF; t += blockDim.x)
    sPerm[t / NQF][t % NQF] = (unsigned char)T->perm[t / NQF][t % NQF];
  for (int t = tid; t < 6 * NQF; t += blockDim.x) sFab[t / NQF][t % NQF] = (unsigned char)T->fab[t / NQF][t % NQF];

  const long long NDa = prm.ndofs;
  const int nel = min(EPB, ne - e0);
  __shared__ int sFnb[EPB][6];
  __shared__ unsigned char sFcd[EPB][6];  // pid << 4 | side << 3 | other local face
  for (int t = tid; t < nel * 6; t += blockDim.x) {
    const int lf = t / nel, el = t % nel;
    sFnb[el][lf] = prm.fnbr[lf * ne + eid(el)];
    sFcd[el][lf] = (unsigned char)prm.fcode[lf * ne + eid(el)];
  }
  for (int k = 0; k < NEQ; ++k)
    for (int t = tid; t < nel * ND; t += blockDim.x)
      sU[((t / ND) * NEQ + k) * ND + (t % ND)] =
          u[k * NDa + (MODE == 3 ? (long long)sS->el[t / ND] * ND + t % ND : (long long)e0 * ND + t)];
  __syncthreads();

  const int warp = tid >> 5, lane = tid & 31;
  const int team = lane / NEQ, tl = lane - NEQ * team;
  const int el = warp * S::TPW + team;  // element slot in the CTA
  const bool act = team < S::TPW && el < nel;
  // the five lanes of a team synchronise among themselves only (teams may
  // skip different faces)
  const unsigned mask = act ? (0x1Fu << (team * NEQ)) : 0u;
  const R gamma = (R)prm.gamma, cov = (R)prm.covolume;
  R lmax = R(0);
  const int e = act ? eid(el) : 0;
  const int k = tl;
  const int wel0 = warp * S::TPW;
  R* wx = sX + warp * WSTR;
  R* xch = wx + (team < S::TPW ? team * XSTR + S::xoff(team) : 0);
  const R* su = sU + (el * NEQ + k) * ND;  // this lane's staged values
  R acc[ND];
#pragma unroll
  for (int i = 0; i < ND; ++i) acc[i] = R(0);
  if constexpr (MODE == 3) {
    if (act) {  // the slot's face geometry into its exchange row
      const R* fg = (const R*)prm.fgeo;
      for (int i = k; i < 24; i += NEQ) xch[S::XG + i] = __ldg(fg + (long long)i * ne + e);
    }
    shared_rounds<P, R>(prm, u, NDa, *sS, sX, sRowOff, xch, su, el, act, k, tL1, tLend, tWf, sPerm,
                        sFab, sFnb, sFcd, gamma, cov, lmax, acc);
  } else if constexpr (MODE != 2) {
    // the warp steps through the six faces together: traces per team, the
    // numerical fluxes over all 32 lanes, the lifting per team again (MODE 0)
#pragma unroll 1
    for (int lf = 0; lf < 6; ++lf) {
      const int nb = act ? sFnb[el][lf] : -1;
      const bool mine = nb != -1 && (MODE == 0 || ((sFcd[el][lf] >> 3) & 1) == 0);
      if (MODE == 1 && !__any_sync(0xffffffffu, mine)) continue;
      if (mine)
        team_traces<P, R>(lf, u, NDa, k, su, xch, tL1, tLend, nb, sFcd[el][lf], sU, e0, nel);
      __syncwarp();
      warp_fluxes<P, R, MODE>(lf, prm, lane, wel0, nel, wx, tWf, sPerm, sFab, sFnb, sFcd, e0, gamma,
                              cov, lmax);
      __syncwarp();
      if (MODE == 0 && nb != -1 && !prm.faces_only)
        team_lift_axis<P, NEQ>(lf, xch + 2 * NEQ * NQF + k, tL1, tLend, acc);
    }
    if constexpr (MODE == 1) {
      block_max_commit<R>(lmax, prm.mcs);
      return;
    }
  } else if (act) {
    // lift the six flux slots the face pass wrote for this element
    const R* fs = (const R*)prm.fslot + (long long)e * 6 * (NEQ * NQF) + k * NQF;
#pragma unroll 1
    for (int lf = 0; lf < 6; ++lf) {
      if (sFnb[el][lf] == -1) continue;
      R fv[NQF];
#pragma unroll
      for (int q = 0; q < NQF; ++q) fv[q] = __ldg(fs + lf * (NEQ * NQF) + q);
      team_lift_axis<P, 1>(lf, fv, tL1, tLend, acc);
    }
  }
  // neighbours inside the tile were read from the staged DOFs, which the
  // volume phase below overwrites with the result
  __syncthreads();
  if (act) {
    if (!prm.faces_only) {
      // nodal fluxes: lane tl handles nodes tl, tl+5, ...; contravariant
      // components of all variables go to the exchange buffer [3][NEQ][ND]
      const R* eg = (const R*)prm.egeo;
      R adj[3][3];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int d = 0; d < 3; ++d) adj[r][d] = eg[(long long)(r * 3 + d) * ne + e];
      const R idet = eg[(long long)9 * ne + e];
#pragma unroll
      for (int rr = 0; rr < (ND + NEQ - 1) / NEQ; ++rr) {
        const int m = tl + NEQ * rr;
        if (m < ND) {
          R st[NEQ];
#pragma unroll
          for (int kk = 0; kk < NEQ; ++kk) st[kk] = sU[(el * NEQ + kk) * ND + m];
          R F[NEQ][3];
          lmax = fmax(lmax, flux_and_speed<3>(st, F, gamma, cov));
#pragma unroll
          for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int kk = 0; kk < NEQ; ++kk)
              xch[(r * NEQ + kk) * ND + m] = adj[r][0] * F[kk][0] + adj[r][1] * F[kk][1] + adj[r][2] * F[kk][2];
        }
      }
      __syncwarp(mask);
      R g[ND];
      // x direction
#pragma unroll
      for (int i = 0; i < ND; ++i) g[i] = xch[(0 * NEQ + k) * ND + i];
#pragma unroll
      for (int jz = 0; jz < N1; ++jz)
#pragma unroll
        for (int jy = 0; jy < N1; ++jy)
#pragma unroll
          for (int jx = 0; jx < N1; ++jx) {
            R s = R(0);
#pragma unroll
            for (int m = 0; m < N1; ++m) s += tD1[jx * N1 + m] * g[m + N1 * (jy + N1 * jz)];
            acc[jx + N1 * (jy + N1 * jz)] += tW1[jy] * tW1[jz] * s;
          }
#pragma unroll
      for (int i = 0; i < ND; ++i) g[i] = xch[(1 * NEQ + k) * ND + i];
#pragma unroll
      for (int jz = 0; jz < N1; ++jz)
#pragma unroll
        for (int jy = 0; jy < N1; ++jy)
#pragma unroll
          for (int jx = 0; jx < N1; ++jx) {
            R s = R(0);
#pragma unroll
            for (int m = 0; m < N1; ++m) s += tD1[jy * N1 + m] * g[jx + N1 * (m + N1 * jz)];
            acc[jx + N1 * (jy + N1 * jz)] += tW1[jx] * tW1[jz] * s;
          }
#pragma unroll
      for (int i = 0; i < ND; ++i) g[i] = xch[(2 * NEQ + k) * ND + i];
#pragma unroll
      for (int jz = 0; jz < N1; ++jz)
#pragma unroll
        for (int jy = 0; jy < N1; ++jy)
#pragma unroll
          for (int jx = 0; jx < N1; ++jx) {
            R s = R(0);
#pragma unroll
            for (int m = 0; m < N1; ++m) s += tD1[jz * N1 + m] * g[jx + N1 * (jy + N1 * m)];
            acc[jx + N1 * (jy + N1 * jz)] += tW1[jx] * tW1[jy] * s;
          }
      if (prm.ncidx) {  // hanging faces of a nonconforming mesh
        const int ix = prm.ncidx[e];
        if (ix >= 0) {
          const R* xf = (const R*)prm.xface + ((long long)ix * NEQ + k) * ND;
#pragma unroll
          for (int i = 0; i < ND; ++i) acc[i] += xf[i];
        }
      }
      // inverse mass: x, y, z sweeps
#pragma unroll
      for (int jz = 0; jz < N1; ++jz)
#pragma unroll
        for (int jy = 0; jy < N1; ++jy)
#pragma unroll
          for (int jx = 0; jx < N1; ++jx) {
            R s = R(0);
#pragma unroll
            for (int m = 0; m < N1; ++m) s += tMinv[jx * N1 + m] * acc[m + N1 * (jy + N1 * jz)];
            g[jx + N1 * (jy + N1 * jz)] = s;
          }
#pragma unroll
      for (int jz = 0; jz < N1; ++jz)
#pragma unroll
        for (int jy = 0; jy < N1; ++jy)
#pragma unroll
          for (int jx = 0; jx < N1; ++jx) {
            R s = R(0);
#pragma unroll
            for (int m = 0; m < N1; ++m) s += tMinv[jy * N1 + m] * g[jx + N1 * (m + N1 * jz)];
            acc[jx + N1 * (jy + N1 * jz)] = s;
          }
      __syncwarp(mask);
#pragma unroll
      for (int jz = 0; jz < N1; ++jz)
#pragma unroll
        for (int jy = 0; jy < N1; ++jy)
#pragma unroll
          for (int jx = 0; jx < N1; ++jx) {
            R s = R(0);
#pragma unroll
            for (int m = 0; m < N1; ++m) s += tMinv[jz * N1 + m] * acc[jx + N1 * (jy + N1 * m)];
            // the right-hand side replaces this variable's staged DOFs (the
            // team's nodal fluxes have been formed already)
            sU[(el * NEQ + k) * ND + jx + N1 * (jy + N1 * jz)] = s * idet;
          }
    }
  }
  __syncthreads();
  if (!prm.faces_only) {
    // coalesced Runge-Kutta epilogue over the CTA's elements; the combined
    // state (hi, lo) is kept in shared memory when the limiter needs means
    const bool need_means = ep.mode == 1 && (ep.means || ep.means32);
    if (ep.mode == 1 && !need_means) {
      // chunked: all loads of a chunk are issued before its stores (the final
      // stage updates the state in place, which would otherwise serialise
      // the memory latency value by value)
      constexpr int CH = 8;
      const int total = NEQ * nel * ND;
      for (int c0 = tid; c0 < total; c0 += CH * blockDim.x) {
        long long idx[CH];
        R y[CH], bh[CH], bl[CH], kp[3][CH];
#pragma unroll
        for (int c = 0; c < CH; ++c) {
          const int g = c0 + c * blockDim.x;
          const int gg = g < total ? g : c0;
          const int k = gg / (nel * ND), t = gg % (nel * ND);
          idx[c] = k * NDa + (MODE == 3 ? (long long)sS->el[t / ND] * ND + t % ND : (long long)e0 * ND + t);
          y[c] = sU[((t / ND) * NEQ + k) * ND + (t % ND)];
          if constexpr (std::is_same<R, double>::value) {
            bh[c] = ep.base ? ep.base[idx[c]] : R(0);
            bl[c] = R(0);
          } else {
            bh[c] = ep.basehi[idx[c]];
            bl[c] = ep.baselo[idx[c]];
          }
#pragma unroll
          for (int j = 0; j < 3; ++j)
            if (j < ep.nprev) kp[j][c] = ep.kprev[j][idx[c]];
        }
#pragma unroll
        for (int c = 0; c < CH; ++c) {
          if (c0 + c * blockDim.x >= total) break;
          if constexpr (std::is_same<R, double>::value) {
            double v = bh[c];
#pragma unroll
            for (int j = 0; j < 3; ++j)
              if (j < ep.nprev) v += ep.cprev[j] * kp[j][c];
            v += ep.ccur * y[c];
            if (ep.kout) ep.kout[idx[c]] = y[c];
            if (ep.out64) ep.out64[idx[c]] = v;
            if (ep.out32) ep.out32[idx[c]] = (float)v;
          } else if (!ep.final_stage) {
            float inc = bl[c];
#pragma unroll
            for (int j = 0; j < 3; ++j)
              if (j < ep.nprev) inc = fmaf(ep.cprev_hi[j], kp[j][c], inc);
            inc = fmaf(ep.ccur_hi, y[c], inc);
            if (ep.kout) ep.kout[idx[c]] = y[c];
            ep.out32[idx[c]] = bh[c] + inc;
          } else {
            float sh = 0.0f, sl = 0.0f, ph, pl;
#pragma unroll
            for (int j = 0; j < 3; ++j)
              if (j < ep.nprev) {
                ds_mul_f(ep.cprev_hi[j], ep.cprev_lo[j], kp[j][c], ph, pl);
                ds_add(sh, sl, ph, pl);
              }
            ds_mul_f(ep.ccur_hi, ep.ccur_lo, y[c], ph, pl);
            ds_add(sh, sl, ph, pl);
            float h = bh[c], l = bl[c];
            ds_add(h, l, sh, sl);
            ep.out32[idx[c]] = h;
            ep.outlo[idx[c]] = l;
          }
        }
      }
    } else {
      for (int k = 0; k < NEQ; ++k)
        for (int t = tid; t < nel * ND; t += blockDim.x) {
          const int s = ((t / ND) * NEQ + k) * ND + (t % ND);
          R hi, lo;
          epi_value2<R>(ep, k * NDa + (MODE == 3 ? (long long)sS->el[t / ND] * ND + t % ND : (long long)e0 * ND + t),
                        sU[s], hi, lo);
          if (need_means) {
            sU[s] = hi;
            sX[s] = lo;
          }
        }
    }
    if (need_means) {
      __syncthreads();
      // cell means of the combined state, one (element, variable) per thread
      for (int t = tid; t < nel * NEQ; t += blockDim.x) {
        double m = 0.0;
        for (int i = 0; i < ND; ++i) m += T->wmean[i] * ((double)sU[t * ND + i] + (double)sX[t * ND + i]);
        store_mean(ep, (long long)(t % NEQ) * ne + eid(t / NEQ), m);
      }
    }
  }
  block_max_commit<R>(lmax, prm.mcs);
}

}  // namespace rkdg
