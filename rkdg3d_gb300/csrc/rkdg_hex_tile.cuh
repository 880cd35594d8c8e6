// Face-once tiled hexahedral right-hand side (k_rhs_hex_tile).
//
// One CTA per tile of RKDG_TILE_E hexahedra that are consecutive in the Morton
// order of their centres (HexTile, built on the host).  NEQ * E threads; thread
// (variable k, slot el) keeps its element's right-hand-side accumulators of
// variable k in registers for the whole stage, and reads the element's staged
// values from shared memory (a warp holds one variable of 32 elements, so
// variable-dependent code never diverges).  The faces are processed one normal
// axis at a time:
//   1. each thread forms its element's traces on the axis's two faces at the
//      (p+2)^2 face points (contraction along the normal, then the 2D
//      interpolation, sum-factorised) into shared memory; threads without a
//      face job form the traces of the out-of-tile elements across the
//      tile's faces ("halo", from global memory);
//   2. the CTA evaluates every face of the axis ONCE, spread over all threads
//      point by point: a face between two tile elements is evaluated with both
//      stored traces and its result is written to both sides (the two halves of
//      the face term of FaceIntegrator::AssembleFaceVector,
//      face_integrator.cpp:11-276: Elem1, Elem2 argument order, the
//      Elem1-outward normal, -w|J_f| F on Elem1's side and +w|J_f| F on
//      Elem2's); a boundary face through its boundary condition's right state
//      (boundary_integrator.cpp:12-194);
//   3. each thread lifts its two faces' weighted fluxes into its accumulators.
// Then the collocated volume term (FE_Evolution::GetFlux and the Aflux product,
// fe_evolution.cpp:157-171, 219-245), the inverse of the exact mass matrix
// det J (M1 x M1 x M1) as three 1D sweeps (fe_evolution.cpp:178-208), and the
// Runge-Kutta stage epilogue with coalesced accesses.
//
// Against the five-lane team kernel this evaluates a face inside the tile
// once instead of twice, forms each trace once, and spreads the pointwise
// numerical fluxes over every thread of the CTA.
#pragma once

#include "rkdg_common.h"
#include "rkdg_generic.cuh"
#include "rkdg_hex_team.cuh"
#include "rkdg_physics.cuh"
#include "rkdg_tc.cuh"

namespace rkdg {

template <int P>
struct TileSize {
  static constexpr int N1 = P + 1, NQ1 = P + 2, ND = N1 * N1 * N1, NQF = NQ1 * NQ1, NEQ = 5,
                       NF2 = N1 * N1;
  static constexpr int E = RKDG_TILE_E, NT = NEQ * E, HM = RKDG_TILE_HMAX;
  // staged DOFs [NEQ][E][ND]; own traces / weighted fluxes of one axis
  // [2][NEQ][NQF][TS] (slot fastest, padded: the threads of a warp -- 32
  // slots -- store a trace point into distinct banks, and the 16 points of
  // one face, read by 16 threads, fall into distinct banks too); halo traces
  // [NEQ][NQF][hs] likewise, hs (odd) = the mesh's largest halo list, so
  // that a structured mesh (32 halos on an axis of a 4 x 4 x 2 tile) keeps
  // four CTAs of the FP32 kernel on an SM
  static constexpr int TS = E + 1;
  static constexpr int OFF_T = NEQ * E * ND, OFF_H = OFF_T + 2 * NEQ * NQF * TS;
  template <typename R>
  static constexpr size_t smem_bytes(int hs) { return sizeof(R) * (size_t)(OFF_H + NEQ * NQF * hs); }
  template <typename R>
  __host__ __device__ static constexpr int min_ctas() { return sizeof(R) == 4 ? 4 : 2; }
  // tensor-core variant (FP32, P = 2): after the staged DOFs, the volume
  // operands A_hi, A_lo ([160 rows (variable, slot)][32 nodes], core-matrix
  // layout) and one direction's B_hi, B_lo ([32][32]) alias the trace and
  // halo regions
  static constexpr int TC_ROWS = NEQ * E, TC_A = TC_ROWS * 32, TC_B = 32 * 32;
  static constexpr int TC_FLOATS = 2 * TC_A + 2 * TC_B;
  static constexpr size_t smem_bytes_tc(int hs) {
    return sizeof(float) * (size_t)(OFF_T + (2 * NEQ * NQF * TS + NEQ * NQF * hs > TC_FLOATS
                                                 ? 2 * NEQ * NQF * TS + NEQ * NQF * hs
                                                 : TC_FLOATS));
  }
};

// Local face of axis AX on side SD (MFEM hexahedron numbering).
__host__ __device__ constexpr int hex_axis_face(int ax, int sd) {
  return ax == 0 ? (sd ? 2 : 4) : (ax == 1 ? (sd ? 3 : 1) : (sd ? 5 : 0));
}

// Trace of an out-of-tile element's variable at the points of its local face
// lfo (tensor order), read from global memory.
template <int P, typename R>
__device__ __forceinline__ void tile_halo_trace(const R* __restrict__ src, int lfo, const R* l1d,
                                                const R* lend, R* dst, int st) {
  constexpr int N1 = P + 1, ND = N1 * N1 * N1, NF2 = N1 * N1;
  R nbv[ND];
  team_gather_any<P, true>(lfo, src, nbv);
  const int sd = hex_face_side(lfo);
  R v[NF2];
#pragma unroll
  for (int r = 0; r < NF2; ++r) {
    R s = R(0);
#pragma unroll
    for (int jn = 0; jn < N1; ++jn) s += lend[sd * N1 + jn] * nbv[r * N1 + jn];
    v[r] = s;
  }
  // 2D interpolation to the face points, tensor order a + NQ1*b at stride st
  constexpr int NQ1 = P + 2;
  R w[NQ1][N1];
#pragma unroll
  for (int a = 0; a < NQ1; ++a)
#pragma unroll
    for (int i1 = 0; i1 < N1; ++i1) {
      R acc = R(0);
#pragma unroll
      for (int i0 = 0; i0 < N1; ++i0) acc += l1d[a * N1 + i0] * v[i0 * N1 + i1];
      w[a][i1] = acc;
    }
#pragma unroll
  for (int b = 0; b < NQ1; ++b)
#pragma unroll
    for (int a = 0; a < NQ1; ++a) {
      R acc = R(0);
#pragma unroll
      for (int i1 = 0; i1 < N1; ++i1) acc += l1d[b * N1 + i1] * w[a][i1];
      dst[(a + NQ1 * b) * st] = acc;
    }
}

// Own traces (AX compile-time: the face pair and its tensor offsets) of the
// thread's variable on the two faces of axis AX, slot-fastest rows.
template <int P, int TS, int AX, typename R>
__device__ __forceinline__ void tile_own_traces(const R* su, const HexOps<R>& H, R* row0, R* row1) {
  constexpr int NF2 = (P + 1) * (P + 1);
  R v[NF2];
  team_contract_s<P, hex_axis_face(AX, 0)>(su, H.lend, v);
  team_interp<P, TS>(v, H.l1d, row0);
  team_contract_s<P, hex_axis_face(AX, 1)>(su, H.lend, v);
  team_interp<P, TS>(v, H.l1d, row1);
}

template <int P, int TS, int AX, typename R>
__device__ __forceinline__ void tile_own_lift(const R* row0, const R* row1, const HexOps<R>& H,
                                              R (&acc)[(P + 1) * (P + 1) * (P + 1)]) {
  team_lift<P, hex_axis_face(AX, 0), TS>(row0, H.l1d, H.lend, acc);
  team_lift<P, hex_axis_face(AX, 1), TS>(row1, H.l1d, H.lend, acc);
}

// One face point of an evaluation: both states (the Elem2 side through the
// boundary condition on a boundary face), the Elem1-outward normal, the
// weight w_q |J_f|, and where each side's weighted flux goes.
template <typename R>
struct TilePoint {
  R s1[5], s2[5], n[3], w;
  R* pa;   // Elem1 side's flux (variable kk at pa[kk * ka]); null: a halo side
  R* pb;   // Elem2 side's; null: a halo side or a boundary face
  int ka, kb, ge;
  bool zero;  // boundary face without an integrator: no face term
};

template <int P, typename R>
__device__ __forceinline__ void tile_point(const RhsParams& prm, const HexTile& T, int ax, int pt,
                                           R* sT, R* sH, const R (*eg)[4],
                                           const unsigned char (*perm)[(P + 2) * (P + 2)],
                                           const unsigned char (*fab)[(P + 2) * (P + 2)],
                                           const R* wf, R gamma, R cov, TilePoint<R>& X) {
  using S = TileSize<P>;
  constexpr int NQF = S::NQF, NEQ = S::NEQ, TS = S::TS;
  const int HS = prm.tile_hs;
  const int j = pt / NQF, q = pt - j * NQF;
  const unsigned d = T.ev[ax][j];
  const int ia = d & 63, ib = (d >> 7) & 63;
  const bool ha = (d >> 6) & 1, hb = (d >> 13) & 1, bnd = (d >> 14) & 1;
  const int lfa = (d >> 15) & 7, lfb = (d >> 18) & 7, pid = (d >> 21) & 7;
  const bool gb = (d >> 24) & 1;
  // a side's value of variable kk at tensor point t: base[kk * k_ + t * q_]
  const int ak = ha ? NQF * HS : NQF * TS, aq = ha ? HS : TS;
  const int bk = hb ? NQF * HS : NQF * TS, bq = hb ? HS : TS;
  R* TA = (ha ? sH + ia : sT + (ia & 1) * (NEQ * NQF * TS) + (ia >> 1)) + fab[lfa][q] * aq;
  X.ge = T.el[(gb ? ib : ia) >> 1];
#pragma unroll
  for (int c = 0; c < 3; ++c) X.n[c] = eg[j][c];
  X.w = wf[q] * eg[j][3];
#pragma unroll
  for (int kk = 0; kk < NEQ; ++kk) X.s1[kk] = TA[kk * ak];
  X.pa = ha ? nullptr : TA;
  X.ka = ak;
  X.zero = false;
  if (bnd) {
    const int nb = prm.fnbr[lfa * prm.ne + X.ge];
    X.pb = nullptr;
    X.kb = 0;
    if (nb == -1) {
      X.zero = true;
#pragma unroll
      for (int kk = 0; kk < NEQ; ++kk) X.s2[kk] = X.s1[kk];
    } else {
      const BCSlot& bc = prm.bc[-2 - nb];
      right_state<3>(bc.type, bc.state, X.s1, X.s2, X.n, gamma, cov, (R)prm.rgas);
    }
  } else {
    R* TB = (hb ? sH + ib : sT + (ib & 1) * (NEQ * NQF * TS) + (ib >> 1)) + fab[lfb][perm[pid][q]] * bq;
#pragma unroll
    for (int kk = 0; kk < NEQ; ++kk) X.s2[kk] = TB[kk * bk];
    X.pb = hb ? nullptr : TB;
    X.kb = bk;
  }
}

template <typename R>
__device__ __forceinline__ void tile_point_store(const TilePoint<R>& X, const R (&F)[5]) {
  if (X.pa) {
#pragma unroll
    for (int kk = 0; kk < 5; ++kk) X.pa[kk * X.ka] = X.zero ? R(0) : -X.w * F[kk];
  }
  if (X.pb) {
#pragma unroll
    for (int kk = 0; kk < 5; ++kk) X.pb[kk * X.kb] = X.w * F[kk];
  }
}

// Face evaluations of axis ax, point by point over the CTA (one copy of the
// pointwise code for all three axes).
template <int P, typename R>
__device__ __forceinline__ void tile_fluxes(const RhsParams& prm, const HexTile& T, int ax, R* sT,
                                            R* sH, const R (*eg)[4],
                                            const unsigned char (*perm)[(P + 2) * (P + 2)],
                                            const unsigned char (*fab)[(P + 2) * (P + 2)],
                                            const R* wf, R& lmax) {
  using S = TileSize<P>;
  constexpr int NQF = S::NQF, NT = S::NT;
  const R gamma = (R)prm.gamma, cov = (R)prm.covolume;
  const int npt = T.nev[ax] * NQF;
#pragma unroll 1
  for (int pt = threadIdx.x; pt < npt; pt += NT) {
    TilePoint<R> A;
    tile_point<P, R>(prm, T, ax, pt, sT, sH, eg, perm, fab, wf, gamma, cov, A);
    R F[5];
    const R sp = riemann<3>(A.s1, A.s2, A.n, F, gamma, cov, prm.rs, prm.avg);
    if (!A.zero) lmax = fmax(lmax, checked_speed(prm, sp, A.ge));
    tile_point_store(A, F);
  }
}

// Collocated derivative sweep along direction R of variable values g (the
// contravariant flux component along R at the nodes), added to acc with the
// other two directions' node weights.
template <int P, int DIR, typename R>
__device__ __forceinline__ void tile_sweep(const R (&g)[(P + 1) * (P + 1) * (P + 1)],
                                           const HexOps<R>& H, R (&acc)[(P + 1) * (P + 1) * (P + 1)]) {
  constexpr int N1 = P + 1;
  const R* tD1 = H.d1;
  const R* tW1 = H.w1;
#pragma unroll
  for (int jz = 0; jz < N1; ++jz)
#pragma unroll
    for (int jy = 0; jy < N1; ++jy)
#pragma unroll
      for (int jx = 0; jx < N1; ++jx) {
        R s = R(0);
#pragma unroll
        for (int m = 0; m < N1; ++m) {
          const int src = DIR == 0 ? m + N1 * (jy + N1 * jz)
                                   : (DIR == 1 ? jx + N1 * (m + N1 * jz) : jx + N1 * (jy + N1 * m));
          const int jd = DIR == 0 ? jx : (DIR == 1 ? jy : jz);
          s += tD1[jd * N1 + m] * g[src];
        }
        const R w = DIR == 0 ? tW1[jy] * tW1[jz] : (DIR == 1 ? tW1[jx] * tW1[jz] : tW1[jx] * tW1[jy]);
        acc[jx + N1 * (jy + N1 * jz)] += w * s;
      }
}

// Float offset of element (row, col) of a K-major TF32 operand with 32
// columns: core matrices of 8 rows x 4 columns (128 bytes), 8 per row group
// along K (LBO 128 bytes), row groups 1024 bytes apart (SBO).
__device__ __forceinline__ int tc_off(int row, int col) {
  return (row >> 3) * 256 + (col >> 2) * 32 + (row & 7) * 4 + (col & 3);
}

// TC = true (FP32, P = 2): the collocated volume contraction on the tensor
// cores (tcgen05, kind::tf32) instead of the three sweeps: per direction r
// the contravariant flux of every (variable, slot) row over the 27 nodes is
// A (160 x 32, split into TF32 hi + lo), the direction's sweep with the other
// two node weights is a dense 27 x 27 operator B_r (hi + lo), and
// A_hi B_hi + A_hi B_lo + A_lo B_hi accumulates over the three directions in
// FP32 in tensor memory: rows 0-127 in columns 0-31, rows 32-159 in columns
// 32-63 (lanes 96-127 hold rows 128-159, read by warp 3 for warp 4).
template <int P, typename R, bool TC = false>
__global__ void __launch_bounds__(TileSize<P>::NT, TC ? 3 : TileSize<P>::template min_ctas<R>())
    k_rhs_hex_tile(const __grid_constant__ RhsParams prm, const R* __restrict__ u,
                   const EpiParams<R> ep) {
  using S = TileSize<P>;
  constexpr int N1 = S::N1, ND = S::ND, NQF = S::NQF, NEQ = S::NEQ, E = S::E, NT = S::NT;
  constexpr int TS = S::TS;
  const int HS = prm.tile_hs;
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ HexTile sTile;
  __shared__ R sGeo[E][10];  // per slot: adj(J) (row r, col d) and 1/det J
  __shared__ R sEG[2 * E][4];  // per evaluation of the current axis: normal, |J_f|
  __shared__ unsigned char sPerm[RKDG_HEX_MAX_PERM][NQF];
  __shared__ unsigned char sFab[6][NQF];
  __shared__ uint64_t sMbar;     // tensor-core completion (TC)
  __shared__ uint32_t sTmem;     // tensor-memory base address (TC)
  __shared__ int sTcFail;        // a completion wait gave up (TC)
  static_assert(!TC || (std::is_same<R, float>::value && P == 2), "tensor-core variant: FP32, P = 2");
  R* sm = reinterpret_cast<R*>(smraw);
  R* sU = sm;              // [NEQ][E][ND]; the right-hand side after the volume phase
  R* sT = sm + S::OFF_T;   // [2][NEQ][NQF][TS]
  R* sH = sm + S::OFF_H;   // [NEQ][NQF][hs]
  const HexOps<R>& H = hex_ops<R>(prm.hops);
  const RefTables* RT = prm.tab;
  const int tid = threadIdx.x;
  const int ne = prm.ne;
  {
    const int* src = reinterpret_cast<const int*>(prm.htile + blockIdx.x);
    for (int t = tid; t < (int)(sizeof(HexTile) / 4); t += NT) reinterpret_cast<int*>(&sTile)[t] = src[t];
  }
  for (int t = tid; t < min(RT->nperm, RKDG_HEX_MAX_PERM) * NQF; t += NT)
    sPerm[t / NQF][t % NQF] = (unsigned char)RT->perm[t / NQF][t % NQF];
  for (int t = tid; t < 6 * NQF; t += NT) sFab[t / NQF][t % NQF] = (unsigned char)RT->fab[t / NQF][t % NQF];
  if constexpr (TC) {
    if (tid == 0) {
      tc::mbar_init(&sMbar, 1);
      sTcFail = 0;
    }
  }
  __syncthreads();
  const int nel = sTile.nel;
  const long long NDa = prm.ndofs;
  // stage the tile's DOFs (runs of ND contiguous values per variable and
  // element): every thread issues all its loads before it stores any
  {
    constexpr int IT = NEQ * E * ND / NT;
    static_assert(IT * NT == NEQ * E * ND, "whole rounds of the CTA");
    R tmp[IT];
#pragma unroll
    for (int it = 0; it < IT; ++it) {
      const int f = tid + it * NT;
      const int k = f / (E * ND), r = f - k * (E * ND), el = r / ND, i = r - el * ND;
      tmp[it] = el < nel ? __ldg(u + k * NDa + (long long)sTile.el[el] * ND + i) : R(0);
    }
#pragma unroll
    for (int it = 0; it < IT; ++it) sU[tid + it * NT] = tmp[it];
  }
  for (int t = tid; t < nel * 10; t += NT) {
    const int sl = t / 10, c = t - sl * 10;
    sGeo[sl][c] = ((const R*)prm.egeo)[(long long)c * ne + sTile.el[sl]];
  }
  __syncthreads();
  const int k = tid / E, el = tid - k * E;  // one variable per warp (E = 32)
  const bool act = el < nel;
  const int e = act ? sTile.el[el] : 0;
  const R* su = sU + (k * E + el) * ND;  // this thread's staged values
  R acc[ND];
#pragma unroll
  for (int i = 0; i < ND; ++i) acc[i] = R(0);
  R lmax = R(0);
  R* row0 = sT + (0 * NEQ + k) * NQF * TS + el;
  R* row1 = sT + (1 * NEQ + k) * NQF * TS + el;
#pragma unroll 1
  for (int ax = 0; ax < 3; ++ax) {
    // 1. traces: own (every face side of the tile has exactly one evaluation,
    // so every stored trace is read once and overwritten by its flux), then
    // the halo, one (variable, halo) per thread
    if (act) {
      switch (ax) {
        case 0: tile_own_traces<P, TS, 0>(su, H, row0, row1); break;
        case 1: tile_own_traces<P, TS, 1>(su, H, row0, row1); break;
        default: tile_own_traces<P, TS, 2>(su, H, row0, row1); break;
      }
    }
    // face geometry of the axis's evaluations (Elem1-outward normal, |J_f|)
    for (int j = tid; j < sTile.nev[ax]; j += NT) {
      const unsigned d = sTile.ev[ax][j];
      const bool gb = (d >> 24) & 1;
      const int ge = sTile.el[(gb ? (d >> 7) & 63 : d & 63) >> 1];
      const int glf = gb ? (d >> 18) & 7 : (d >> 15) & 7;
      const R* fg = (const R*)prm.fgeo + (long long)(glf * 4) * ne + ge;
#pragma unroll
      for (int c = 0; c < 4; ++c) sEG[j][c] = __ldg(fg + (long long)c * ne);
    }
    const int nh = sTile.nh[ax];
    for (int j = tid; j < nh * NEQ; j += NT) {
      const int kk = j / nh, h = j - kk * nh;
      tile_halo_trace<P, R>(u + kk * NDa + (long long)sTile.hel[ax][h] * ND, sTile.hlf[ax][h],
                            H.l1d, H.lend, sH + kk * NQF * HS + h, HS);
    }
    __syncthreads();
    // 2. every face of the axis once
    tile_fluxes<P, R>(prm, sTile, ax, sT, sH, sEG, sPerm, sFab, H.wf, lmax);
    __syncthreads();
    // 3. lifting of the thread's two faces
    if (act && !prm.faces_only) {
      switch (ax) {
        case 0: tile_own_lift<P, TS, 0>(row0, row1, H, acc); break;
        case 1: tile_own_lift<P, TS, 1>(row0, row1, H, acc); break;
        default: tile_own_lift<P, TS, 2>(row0, row1, H, acc); break;
      }
    }
  }
  if (prm.faces_only) {
    block_max_commit<R>(lmax, prm.mcs);
    return;
  }
  // volume term, one direction at a time: the contravariant component along
  // direction r of every variable's nodal flux (FE_Evolution::GetFlux), one
  // (element, node) per thread, into the trace region; then each thread's
  // collocated sweep along r
  R* sG = sT;  // [NEQ][E][ND]
  const R gamma = (R)prm.gamma, cov = (R)prm.covolume;
  if constexpr (TC) {
    float* A0 = sT;                // A_hi; A_lo follows
    float* A1 = sT + S::TC_A;
    float* B0 = sT + 2 * S::TC_A;  // B_hi; B_lo follows
    float* B1 = B0 + S::TC_B;
    constexpr uint32_t IDESC = tc::idesc_tf32(128, 32);
    constexpr int kWaitPolls = 1 << 20;
    const int warp = tid >> 5, lane = tid & 31;
    if (warp == 0) {
      tc::tmem_alloc(&sTmem, 64);
      tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();  // also: the lifts are done with the trace region
    tc::fence_after_sync();
    const uint32_t tbase = sTmem;
    // the K padding (nodes 27-31) of every row stays zero
    for (int t = tid; t < S::TC_ROWS * 5; t += NT) {
      const int row = t / 5, col = 27 + t % 5;
      A0[tc_off(row, col)] = 0.0f;
      A1[tc_off(row, col)] = 0.0f;
    }
    bool failed = false;
#pragma unroll 1
    for (int r = 0; r < 3; ++r) {
      // this direction's operator (hi, lo) from the table
      {
        const float4* src = reinterpret_cast<const float4*>(prm.tcb + (size_t)r * 2 * S::TC_B);
        float4* dst = reinterpret_cast<float4*>(B0);
        for (int t = tid; t < 2 * S::TC_B / 4; t += NT) dst[t] = __ldg(src + t);
      }
      // contravariant fluxes, one (slot, node) per thread (slot fastest: the
      // staged reads stride 27 words), split into the two A operands
      for (int t = tid; t < E * ND; t += NT) {
        const int m = t / E, sl = t - m * E;
        if (sl >= nel) continue;
        R st[NEQ];
#pragma unroll
        for (int kk = 0; kk < NEQ; ++kk) st[kk] = sU[(kk * E + sl) * ND + m];
        R F[NEQ][3];
        const R sp = flux_and_speed<3>(st, F, gamma, cov);
        if (r == 0) lmax = fmax(lmax, sp);
        const R a0 = sGeo[sl][3 * r], a1 = sGeo[sl][3 * r + 1], a2 = sGeo[sl][3 * r + 2];
#pragma unroll
        for (int kk = 0; kk < NEQ; ++kk) {
          const float g = a0 * F[kk][0] + a1 * F[kk][1] + a2 * F[kk][2];
          const float h = tc::tf32_hi(g);
          const int o = tc_off(kk * E + sl, m);
          A0[o] = h;
          A1[o] = g - h;
        }
      }
      tc::fence_async_smem();
      __syncthreads();
      if (tid == 0) {
        tc::fence_after_sync();
        const uint32_t a_base[2] = {tc::smem_u32(A0), tc::smem_u32(A1)};
        const uint32_t b_base[2] = {tc::smem_u32(B0), tc::smem_u32(B1)};
        const int terms[3][2] = {{0, 0}, {0, 1}, {1, 0}};  // (A part, B part)
#pragma unroll
        for (int blk = 0; blk < 2; ++blk)
#pragma unroll
          for (int tm = 0; tm < 3; ++tm)
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
              // block 1 starts at row 32 (row group 4, 4096 bytes); K step ks
              // at column 8 ks (two core matrices, 256 bytes)
              const uint64_t ad = tc::desc_kmajor(a_base[terms[tm][0]] + blk * 4096 + ks * 256, 128, 1024);
              const uint64_t bd = tc::desc_kmajor(b_base[terms[tm][1]] + ks * 256, 128, 1024);
              const uint32_t acc_in = (r > 0 || tm > 0 || ks > 0) ? 1u : 0u;
              tc::mma_tf32(tbase + blk * 32, ad, bd, IDESC, acc_in);
            }
        tc::commit(&sMbar);
      }
      // the MMAs read A and B before either is rewritten
      if (!tc::mbar_wait(&sMbar, r & 1, kWaitPolls)) failed = true;
      if (failed) sTcFail = 1;
      __syncthreads();
      if (sTcFail) break;
    }
    if (sTcFail) {
      // give the tensor core one more bounded wait, free the tensor memory
      // and leave the tile unwritten with the error flagged
      if (tid == 0) flag_error(prm.err, 8, blockIdx.x);
      tc::mbar_wait(&sMbar, 0, kWaitPolls);
      tc::mbar_wait(&sMbar, 1, kWaitPolls);
      tc::fence_before_sync();
      __syncthreads();
      if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tbase, 64);
      }
      return;
    }
    tc::fence_after_sync();
    float v[32];
    if (warp < 4) {
      tc::ld32(tbase + ((uint32_t)(32 * warp) << 16), v);
      if (act) {
#pragma unroll
        for (int i = 0; i < ND; ++i) acc[i] += v[i];
      }
    }
    float* sX = A0;  // rows 128-159 handed from warp 3 to warp 4
    if (warp == 3) {
      tc::ld32(tbase + (96u << 16) + 32u, v);
#pragma unroll
      for (int i = 0; i < ND; ++i) sX[lane * ND + i] = v[i];
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 4 && act) {
#pragma unroll
      for (int i = 0; i < ND; ++i) acc[i] += sX[lane * ND + i];
    }
    if (warp == 0) {
      tc::fence_after_sync();
      tc::tmem_dealloc(tbase, 64);
    }
  } else {
#pragma unroll 1
  for (int r = 0; r < 3; ++r) {
    __syncthreads();  // the lifts (r = 0) or the previous sweeps are done with sT
    for (int t = tid; t < nel * ND; t += NT) {
      const int sl = t / ND, m = t - sl * ND;
      R st[NEQ];
#pragma unroll
      for (int kk = 0; kk < NEQ; ++kk) st[kk] = sU[(kk * E + sl) * ND + m];
      R F[NEQ][3];
      const R sp = flux_and_speed<3>(st, F, gamma, cov);
      if (r == 0) lmax = fmax(lmax, sp);
      const R a0 = sGeo[sl][3 * r], a1 = sGeo[sl][3 * r + 1], a2 = sGeo[sl][3 * r + 2];
#pragma unroll
      for (int kk = 0; kk < NEQ; ++kk) sG[(kk * E + sl) * ND + m] = a0 * F[kk][0] + a1 * F[kk][1] + a2 * F[kk][2];
    }
    __syncthreads();
    if (act) {
      R gv[ND];
#pragma unroll
      for (int i = 0; i < ND; ++i) gv[i] = sG[(k * E + el) * ND + i];
      switch (r) {
        case 0: tile_sweep<P, 0>(gv, H, acc); break;
        case 1: tile_sweep<P, 1>(gv, H, acc); break;
        default: tile_sweep<P, 2>(gv, H, acc); break;
      }
    }
  }
  }
  R g[ND];
  if (act) {
    if (prm.ncidx) {  // hanging faces of a nonconforming mesh
      const int ix = prm.ncidx[e];
      if (ix >= 0) {
        const R* xf = (const R*)prm.xface + ((long long)ix * NEQ + k) * ND;
#pragma unroll
        for (int i = 0; i < ND; ++i) acc[i] += xf[i];
      }
    }
    // inverse mass: x, y, z sweeps, then 1 / det J
    const R* tMinv = H.minv1;
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
    const R idet = sGeo[el][9];
#pragma unroll
    for (int jz = 0; jz < N1; ++jz)
#pragma unroll
      for (int jy = 0; jy < N1; ++jy)
#pragma unroll
        for (int jx = 0; jx < N1; ++jx) {
          R s = R(0);
#pragma unroll
          for (int m = 0; m < N1; ++m) s += tMinv[jz * N1 + m] * acc[jx + N1 * (jy + N1 * m)];
          g[jx + N1 * (jy + N1 * jz)] = s * idet;
        }
  }
  __syncthreads();  // every thread has read the staged DOFs
  if (act) {
#pragma unroll
    for (int i = 0; i < ND; ++i) sU[(k * E + el) * ND + i] = g[i];
  }
  __syncthreads();
  // Runge-Kutta epilogue over the tile, coalesced within each element's run
  const bool need_means = ep.mode == 1 && (ep.means || ep.means32);
  R* sLo = sT;  // low parts of the combined state when the limiter needs means
  const int total = NEQ * nel * ND;
  if (ep.mode == 1 && !need_means) {
    // three values per thread and round (nine rounds cover a tile's 27 values
    // per thread): the loads of a round in flight together, and few enough
    // registers that nothing spills (measured: 2.25 ms per C2 step against
    // 2.36 with eight and 2.70 with twelve)
    constexpr int CH = 3;
    for (int c0 = tid; c0 < total; c0 += CH * NT) {
      long long idx[CH];
      R y[CH], bh[CH], bl[CH], kp[3][CH];
#pragma unroll
      for (int c = 0; c < CH; ++c) {
        const int g = c0 + c * NT;
        const int gg = g < total ? g : c0;
        const int kk = gg / (nel * ND), t = gg - kk * (nel * ND);
        idx[c] = kk * NDa + (long long)sTile.el[t / ND] * ND + t % ND;
        y[c] = sU[(kk * E + t / ND) * ND + t % ND];
        if constexpr (std::is_same<R, double>::value) {
          bh[c] = ep.base ? ep.base[idx[c]] : R(0);
          bl[c] = R(0);
        } else {
          bh[c] = ep.basehi[idx[c]];
          bl[c] = ep.baselo[idx[c]];
        }
#pragma unroll
        for (int jj = 0; jj < 3; ++jj)
          if (jj < ep.nprev) kp[jj][c] = ep.kprev[jj][idx[c]];
      }
#pragma unroll
      for (int c = 0; c < CH; ++c) {
        if (c0 + c * NT >= total) break;
        if constexpr (std::is_same<R, double>::value) {
          double v = bh[c];
#pragma unroll
          for (int jj = 0; jj < 3; ++jj)
            if (jj < ep.nprev) v += ep.cprev[jj] * kp[jj][c];
          v += ep.ccur * y[c];
          if (ep.kout) ep.kout[idx[c]] = y[c];
          if (ep.out64) ep.out64[idx[c]] = v;
          if (ep.out32) ep.out32[idx[c]] = (float)v;
        } else if (!ep.final_stage) {
          float inc = bl[c];
#pragma unroll
          for (int jj = 0; jj < 3; ++jj)
            if (jj < ep.nprev) inc = fmaf(ep.cprev_hi[jj], kp[jj][c], inc);
          inc = fmaf(ep.ccur_hi, y[c], inc);
          if (ep.kout) ep.kout[idx[c]] = y[c];
          ep.out32[idx[c]] = bh[c] + inc;
        } else {
          float sh = 0.0f, sl = 0.0f, ph, pl;
#pragma unroll
          for (int jj = 0; jj < 3; ++jj)
            if (jj < ep.nprev) {
              ds_mul_f(ep.cprev_hi[jj], ep.cprev_lo[jj], kp[jj][c], ph, pl);
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
    for (int f = tid; f < total; f += NT) {
      const int kk = f / (nel * ND), t = f - kk * (nel * ND);
      const int s = (kk * E + t / ND) * ND + t % ND;
      R hi, lo;
      epi_value2<R>(ep, kk * NDa + (long long)sTile.el[t / ND] * ND + t % ND, sU[s], hi, lo);
      if (need_means) {
        sU[s] = hi;
        sLo[s] = lo;
      }
    }
    if (need_means) {
      __syncthreads();
      // cell means of the combined state, one (element, variable) per thread
      for (int t = tid; t < nel * NEQ; t += NT) {
        const int kk = t / nel, s = t - kk * nel;
        double m = 0.0;
        for (int i = 0; i < ND; ++i)
          m += RT->wmean[i] * ((double)sU[(kk * E + s) * ND + i] + (double)sLo[(kk * E + s) * ND + i]);
        store_mean(ep, (long long)kk * ne + sTile.el[s], m);
      }
    }
  }
  block_max_commit<R>(lmax, prm.mcs);
}

}  // namespace rkdg
