// Host side of the GB300 RKDG C ABI (include/rkdg_gpu.h).
//
// Owns the device tables that replace MFEM's face/element transformations,
// the Runge-Kutta stage orchestration of ExplicitRKLimitedSolver::Step
// (rk_explicit_limited.cpp:30-82) and the time loop of main.cpp:467-553,
// 701-733.  All arithmetic on the hot path runs in the CUDA kernels; this file
// only builds tables, sizes buffers and enqueues launches.
#include "rkdg_gpu.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "rkdg_common.h"
#include "rkdg_hexsched.h"
#include "rkdg_ncmesh.h"
#include "rkdg_launch.h"
#include "rkdg_refelem.h"

using rkdg::BCSlot;
using rkdg::EpiParams;
using rkdg::HexTeamSched;
using rkdg::HexTile;
using rkdg::LimParams;
using rkdg::RefTables;
using rkdg::RhsParams;

struct rkdg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  long long err_where = -1;
  long long launches = 0;
  // physics and scheme
  int rs = RKDG_RS_RUSANOV, avg = RKDG_AVG_TRRS;
  double gamma = 1.4, cov = 0.0, gasR = 1.0;
  std::map<int, BCSlot> bcs;
  int lim = RKDG_LIM_FINDIFF, ind = RKDG_IND_NOWHERE, fun = RKDG_FUN_MICHALAK, last_hope = 1,
      quirks = 0;
  int s = 3;
  std::vector<double> a{1.0, 0.25, 0.25}, b{1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0}, c{1.0, 0.5};
  int precision = RKDG_FP64;
  int hex_variant = 0;  // RKDG_TUNE_HEX_KERNEL
  int gen_block = 0;    // RKDG_TUNE_GENERIC_BLOCK
  double* d_fslot = nullptr;  // face-pass flux slots (split hexahedral variant)
  size_t fslot_n = 0;
  HexTeamSched* d_hsched = nullptr;  // per-CTA schedules of the shared-face hexahedral kernel
  int hsched_rounds = 0;
  HexTile* d_htile = nullptr;  // tiles of the face-once hexahedral kernel
  float* d_tcb = nullptr;      // volume operators of its tensor-core variant (Q2)
  int ntile = 0;
  int tile_hs = 1;             // halo-buffer stride of its CTAs (odd)
  // hanging faces of a nonconforming mesh (see rkdg_nc.cu)
  int nnc = 0, nc_nel = 0;
  // non-parallelogram quadrilaterals: per-node adj(J) and 1/det J
  // [dim*dim + 1][nd][ne] and per-element cell-mean weights [ne][nd]
  int nonaffine = 0;
  double* d_ngeo64 = nullptr;
  float* d_ngeo32 = nullptr;
  double* d_wmn64 = nullptr;
  float* d_wmn32 = nullptr;
  int* d_nc_face = nullptr;
  double* d_nc_bnc = nullptr;
  double* d_nc_flux = nullptr;
  int* d_nc_elem = nullptr;
  int* d_nc_ptr = nullptr;
  int* d_nc_ent = nullptr;
  int* d_ncidx = nullptr;
  double* d_xface = nullptr;
  int lim_block = 0;    // RKDG_TUNE_LIMITER_BLOCK
  int solver_quirks = 0;
  // mesh (host copies)
  bool has_mesh = false;
  int dim = 0, geom = 0, p = 0, ne = 0, nd = 0, neq = 0, nfpe = 0, nvpe = 0;
  long long ndofs = 0;
  RefTables tab;
  std::vector<int> h_fnbr, h_fattr, h_fcode;
  std::vector<int> h_nc_face;  // hanging faces [nnc][4] (fine element, its face, coarse element, its face)
  std::vector<double> h_fgeo, h_egeo, h_wdet, h_nodes;
  double hmin = 0.0;
  // device tables
  RefTables* d_tab = nullptr;
  int* d_fnbr = nullptr;
  int* d_fcode = nullptr;
  double* d_fgeo64 = nullptr;
  float* d_fgeo32 = nullptr;
  double* d_egeo64 = nullptr;
  double* d_eaff = nullptr;  // [dim*dim + dim][ne] J and vertex 0 (Shu indicator)
  std::vector<double> h_eaff;
  float* d_egeo32 = nullptr;
  double* d_wdet = nullptr;
  unsigned long long* d_mcs = nullptr;  // 8 slots
  int* d_err = nullptr;                 // 2 ints
  double* d_means = nullptr;
  double* d_partial = nullptr;
  // scratch state buffers
  double* d_k64[4] = {nullptr, nullptr, nullptr, nullptr};
  float* d_k32[4] = {nullptr, nullptr, nullptr, nullptr};
  double* d_y64[2] = {nullptr, nullptr};
  float* d_y32[2] = {nullptr, nullptr};
  float* d_xh = nullptr;
  float* d_xl = nullptr;
  unsigned long long* h_mcs = nullptr;  // pinned
  int* h_err = nullptr;                 // pinned
  std::vector<double> h_ehmin;          // per-element GetElementSize(i, 1)
  // batched independent problems
  int nprob = 0;
  std::vector<int> h_poff;
  int* d_prob = nullptr;
  double* d_pgamma = nullptr;
  double* d_pcov = nullptr;
  float* d_pgamma32 = nullptr;  // FP32 copies for the FP32 kernels
  float* d_pcov32 = nullptr;
  float2* d_pdt2 = nullptr;     // dt_real as float pairs
  double* d_phmin = nullptr;
  double* d_pdt = nullptr;
  double* d_pdtr = nullptr;
  double* d_pt = nullptr;
  double* d_psum = nullptr;
  int* d_pactive = nullptr;
  int* d_psteps = nullptr;
  int* d_nactive = nullptr;
  // map of the active work of a batched run (see RhsParams)
  int* d_act_cum = nullptr;
  int* d_act_pid = nullptr;
  int* d_act_n = nullptr;
  int* d_poff = nullptr;
  int* d_pfail = nullptr;
  unsigned long long* d_pmcs = nullptr;  // [4][nprob]
  // discrete adjoint scratch (FP64)
  double* d_adj = nullptr;
  size_t adj_n = 0;

  bool limiter_active() const { return !(lim == RKDG_LIM_FINDIFF && ind == RKDG_IND_NOWHERE); }
};

namespace {

int fail(rkdg_ctx* c, int code, const std::string& msg, long long where = -1) {
  if (c) {
    c->err = msg;
    c->err_where = where;
  }
  return code;
}

#define CUDA_TRY(ctx, call)                                                              \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? RKDG_ERR_ALLOC : RKDG_ERR_CUDA, \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                   \
  } while (0)

template <typename T>
void dfree(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

template <typename T>
cudaError_t dalloc(T*& p, size_t n) {
  dfree(p);
  if (n == 0) return cudaSuccess;
  return cudaMalloc((void**)&p, n * sizeof(T));
}

void free_mesh(rkdg_ctx* c) {
  dfree(c->d_tab);
  dfree(c->d_fnbr);
  dfree(c->d_fcode);
  dfree(c->d_fgeo64);
  dfree(c->d_fgeo32);
  dfree(c->d_egeo64);
  dfree(c->d_egeo32);
  dfree(c->d_wdet);
  dfree(c->d_eaff);
  dfree(c->d_means);
  dfree(c->d_partial);
  for (auto& p : c->d_k64) dfree(p);
  for (auto& p : c->d_k32) dfree(p);
  for (auto& p : c->d_y64) dfree(p);
  for (auto& p : c->d_y32) dfree(p);
  dfree(c->d_xh);
  dfree(c->d_xl);
  dfree(c->d_prob);
  dfree(c->d_pgamma);
  dfree(c->d_pcov);
  dfree(c->d_pgamma32);
  dfree(c->d_pcov32);
  dfree(c->d_pdt2);
  dfree(c->d_phmin);
  dfree(c->d_pdt);
  dfree(c->d_pdtr);
  dfree(c->d_pt);
  dfree(c->d_psum);
  dfree(c->d_pactive);
  dfree(c->d_psteps);
  dfree(c->d_nactive);
  dfree(c->d_act_cum);
  dfree(c->d_act_pid);
  dfree(c->d_act_n);
  dfree(c->d_poff);
  dfree(c->d_pfail);
  dfree(c->d_pmcs);
  dfree(c->d_adj);
  c->adj_n = 0;
  dfree(c->d_fslot);
  c->fslot_n = 0;
  dfree(c->d_hsched);
  c->hsched_rounds = 0;
  dfree(c->d_htile);
  dfree(c->d_tcb);
  c->ntile = 0;
  dfree(c->d_nc_face);
  dfree(c->d_nc_bnc);
  dfree(c->d_nc_flux);
  dfree(c->d_nc_elem);
  dfree(c->d_nc_ptr);
  dfree(c->d_nc_ent);
  dfree(c->d_ncidx);
  dfree(c->d_xface);
  c->nnc = c->nc_nel = 0;
  c->h_nc_face.clear();
  dfree(c->d_ngeo64);
  dfree(c->d_ngeo32);
  dfree(c->d_wmn64);
  dfree(c->d_wmn32);
  c->nonaffine = 0;
  c->nprob = 0;
  c->has_mesh = false;
}

int nvpe_of(int geom) { return geom == 2 ? 3 : (geom == 3 ? 4 : 8); }
int nfpe_of(int geom) { return geom == 2 ? 3 : (geom == 3 ? 4 : 6); }

// Minimum singular value of a dim x dim matrix (row-major).
double min_singular(int dim, const double* J) {
  if (dim == 2) {
    const double s1 = J[0] * J[0] + J[1] * J[1] + J[2] * J[2] + J[3] * J[3];
    const double d = J[0] * J[3] - J[1] * J[2];
    const double disc = std::sqrt(std::max(0.0, s1 * s1 - 4.0 * d * d));
    return std::sqrt(std::max(0.0, 0.5 * (s1 - disc)));
  }
  double M[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double v = 0;
      for (int k = 0; k < 3; ++k) v += J[k * 3 + i] * J[k * 3 + j];
      M[i * 3 + j] = v;
    }
  // smallest eigenvalue of the symmetric matrix M by Jacobi rotations
  double A[9];
  std::memcpy(A, M, sizeof A);
  for (int sweep = 0; sweep < 50; ++sweep) {
    double off = A[1] * A[1] + A[2] * A[2] + A[5] * A[5];
    if (off < 1e-300) break;
    for (int pq = 0; pq < 3; ++pq) {
      const int pi = pq == 2 ? 1 : 0, qi = pq == 0 ? 1 : 2;
      const double apq = A[pi * 3 + qi];
      if (std::fabs(apq) < 1e-300) continue;
      const double th = 0.5 * (A[qi * 3 + qi] - A[pi * 3 + pi]) / apq;
      const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
      const double cs = 1.0 / std::sqrt(t * t + 1.0), sn = t * cs;
      for (int k = 0; k < 3; ++k) {  // columns
        const double akp = A[k * 3 + pi], akq = A[k * 3 + qi];
        A[k * 3 + pi] = cs * akp - sn * akq;
        A[k * 3 + qi] = sn * akp + cs * akq;
      }
      for (int k = 0; k < 3; ++k) {  // rows
        const double apk = A[pi * 3 + k], aqk = A[qi * 3 + k];
        A[pi * 3 + k] = cs * apk - sn * aqk;
        A[qi * 3 + k] = sn * apk + cs * aqk;
      }
    }
  }
  const double lmin = std::min(A[0], std::min(A[4], A[8]));
  return std::sqrt(std::max(0.0, lmin));
}

int refresh_fnbr(rkdg_ctx* c) {
  if (!c->has_mesh) return RKDG_OK;
  std::map<int, int> slot;
  int k = 0;
  for (auto& kv : c->bcs) slot[kv.first] = k++;
  std::vector<int> f(c->h_fnbr);
  for (size_t i = 0; i < f.size(); ++i)
    if (f[i] < 0) {
      auto it = slot.find(c->h_fattr[i]);
      f[i] = it == slot.end() ? -1 : -2 - it->second;
    }
  CUDA_TRY(c, cudaMemcpy(c->d_fnbr, f.data(), f.size() * sizeof(int), cudaMemcpyHostToDevice));
  return RKDG_OK;
}

RhsParams rhs_params(rkdg_ctx* c, int prec, int faces_only, int slot) {
  RhsParams P;
  std::memset(&P, 0, sizeof P);
  P.ne = c->ne;
  P.ndofs = c->ndofs;
  P.fnbr = c->d_fnbr;
  P.fcode = c->d_fcode;
  P.fgeo = prec == 0 ? (const void*)c->d_fgeo64 : (const void*)c->d_fgeo32;
  P.egeo = prec == 0 ? (const void*)c->d_egeo64 : (const void*)c->d_egeo32;
  P.tab = c->d_tab;
  P.gamma = c->gamma;
  P.covolume = c->cov;
  P.rgas = c->gasR;
  P.rs = c->rs;
  P.avg = c->avg;
  P.faces_only = faces_only;
  P.quirks = c->solver_quirks & RKDG_QUIRK_HLLC_NEGATIVE_SPEED_OK;
  int k = 0;
  for (auto& kv : c->bcs) P.bc[k++] = kv.second;
  P.mcs = c->d_mcs + slot;
  P.err = c->d_err;
  P.block = c->gen_block;
  P.fslot = c->d_fslot;
  P.hsched = c->d_hsched;
  P.htile = c->d_htile;
  P.tcb = c->d_tcb;
  P.ntile = c->ntile;
  P.tile_hs = c->tile_hs;
  P.ncidx = c->nnc ? c->d_ncidx : nullptr;
  P.xface = c->d_xface;
  P.ngeo = c->nonaffine ? (prec == 0 ? (const void*)c->d_ngeo64 : (const void*)c->d_ngeo32) : nullptr;
  if (c->geom == RKDG_GEOM_CUBE && c->p <= 2) {
    const int n1 = c->p + 1, nq1 = c->p + 2;
    const RefTables& T = c->tab;
    auto fill = [&](auto& H) {
      for (int a = 0; a < nq1; ++a)
        for (int j = 0; j < n1; ++j) H.l1d[a * n1 + j] = T.l1d[a][j];
      for (int sd = 0; sd < 2; ++sd)
        for (int j = 0; j < n1; ++j) H.lend[sd * n1 + j] = T.lend[sd][j];
      for (int j = 0; j < n1; ++j) {
        for (int m = 0; m < n1; ++m) {
          H.d1[j * n1 + m] = T.d1[j][m];
          H.minv1[j * n1 + m] = T.minv1[j][m];
        }
        H.w1[j] = T.w1[j];
      }
      for (int q = 0; q < nq1 * nq1; ++q) H.wf[q] = T.wf[q];
    };
    fill(P.hops.f);
    fill(P.hops.d);
  }
  return P;
}

rkdg::NcParams nc_params(const rkdg_ctx* c) {
  rkdg::NcParams N;
  std::memset(&N, 0, sizeof N);
  N.nnc = c->nnc;
  N.nqf = c->tab.nqf;
  N.nd = c->nd;
  N.neq = c->neq;
  N.nel = c->nc_nel;
  N.face = c->d_nc_face;
  N.bnc = c->d_nc_bnc;
  N.flux = c->d_nc_flux;
  N.elem = c->d_nc_elem;
  N.ptr = c->d_nc_ptr;
  N.ent = c->d_nc_ent;
  N.xface = c->d_xface;
  return N;
}

// One right-hand-side evaluation: on a nonconforming mesh first the hanging
// faces (their wave speeds, and their face terms unless only the speed is
// wanted), then the element kernel.
cudaError_t launch_rhs_nc(rkdg_ctx* c, int prec, const RhsParams& P, const void* in, const void* ep) {
  if (c->nnc) {
    const cudaError_t e = rkdg::launch_nc(c->geom, c->p, prec, P, nc_params(c), in, !P.faces_only, c->stream);
    if (e != cudaSuccess) return e;
    c->launches += P.faces_only ? 1 : 2;
  }
  return rkdg::launch_rhs_v(c->hex_variant, c->geom, c->p, prec, P, in, ep, c->stream);
}

// Kernels one right-hand-side launch issues (the split hexahedral variant
// runs a face pass and an element pass; it is the FP64 Q1 default).
int rhs_kernels(const rkdg_ctx* c, const RhsParams& P) {
  const bool fp64 = P.fgeo == (const void*)c->d_fgeo64;
  const bool split = c->hex_variant == 3 || (c->hex_variant == 0 && c->p == 1 && fp64);
  return (c->geom == RKDG_GEOM_CUBE && split && P.fslot && !P.faces_only) ? 2 : 1;
}

// Flux slots of the split hexahedral variant: [ne][6][neq][nqf] values of
// the widest precision.
int ensure_fslot(rkdg_ctx* c) {
  if (c->geom != RKDG_GEOM_CUBE) return RKDG_OK;
  const size_t n = (size_t)c->ne * 6 * c->neq * c->tab.nqf;
  if (c->d_fslot && c->fslot_n == n) return RKDG_OK;
  dfree(c->d_fslot);
  c->fslot_n = 0;
  CUDA_TRY(c, dalloc(c->d_fslot, n));
  c->fslot_n = n;
  return RKDG_OK;
}

void set_batch(rkdg_ctx* c, RhsParams& P, int slot) {
  P.prob = c->d_prob;
  P.pgamma = c->d_pgamma;
  P.pcov = c->d_pcov;
  P.pgamma32 = c->d_pgamma32;
  P.pcov32 = c->d_pcov32;
  P.pactive = c->d_pactive;
  P.act_cum = c->d_act_cum;
  P.act_pid = c->d_act_pid;
  P.act_n = c->d_act_n;
  P.poff = c->d_poff;
  P.pmcs = c->d_pmcs + (size_t)slot * c->nprob;
  P.pfail = c->d_pfail;
}

LimParams lim_params(rkdg_ctx* c) {
  LimParams L;
  std::memset(&L, 0, sizeof L);
  L.ne = c->ne;
  L.ndofs = c->ndofs;
  L.fnbr = c->d_fnbr;
  L.tab = c->d_tab;
  L.eaff = c->d_eaff;
  L.means = c->d_means;
  L.gamma = c->gamma;
  L.covolume = c->cov;
  L.limiter = c->lim;
  L.indicator = c->ind;
  L.function = c->fun;
  L.last_hope = c->last_hope;
  L.quirks = c->quirks;
  L.block = c->lim_block;
  if (c->nnc) {
    L.ncidx = c->d_ncidx;
    L.nc_ptr = c->d_nc_ptr;
    L.nc_ent = c->d_nc_ent;
    L.nc_face = c->d_nc_face;
  }
  return L;
}

int ensure_scratch(rkdg_ctx* c) {
  const size_t n = (size_t)c->ndofs * c->neq;
  const int nk = std::max(c->s - 1, 0);
  if (c->precision == RKDG_FP64) {
    for (int i = 0; i < 4; ++i) {
      if (i < nk && !c->d_k64[i]) CUDA_TRY(c, dalloc(c->d_k64[i], n));
      if (i >= nk) dfree(c->d_k64[i]);
    }
    for (auto& p : c->d_k32) dfree(p);
    for (int i = 0; i < 2; ++i)
      if (!c->d_y64[i]) CUDA_TRY(c, dalloc(c->d_y64[i], n));
    for (auto& p : c->d_y32) dfree(p);
    dfree(c->d_xh);
    dfree(c->d_xl);
  } else {
    for (int i = 0; i < 4; ++i) {
      if (i < nk && !c->d_k32[i]) CUDA_TRY(c, dalloc(c->d_k32[i], n));
      if (i >= nk) dfree(c->d_k32[i]);
    }
    for (auto& p : c->d_k64) dfree(p);
    for (int i = 0; i < 2; ++i)
      if (!c->d_y32[i]) CUDA_TRY(c, dalloc(c->d_y32[i], n));
    dfree(c->d_y64[1]);
    if (!c->d_y64[0]) CUDA_TRY(c, dalloc(c->d_y64[0], n));  // FP64 scratch for API calls
    if (!c->d_xh) CUDA_TRY(c, dalloc(c->d_xh, n));
    if (!c->d_xl) CUDA_TRY(c, dalloc(c->d_xl, n));
  }
  return RKDG_OK;
}

// TF32 part of an FP32 value (10 explicit mantissa bits, rounded to nearest).
float tf32_hi_host(float x) {
  uint32_t b;
  std::memcpy(&b, &x, 4);
  b = (b + 0x1000u) & 0xFFFFE000u;
  float y;
  std::memcpy(&y, &b, 4);
  return y;
}

// Volume operators of the tensor-core tile kernel (Q2 hexahedra): for
// direction r the collocated sweep along r with the other two node weights,
// acc[j] += w1[j_a] w1[j_b] d1[j_r][m_r] g_r[m] over the nodes m that share
// j's other two indices, as a dense 32 x 32 matrix B_r[j][m] (zero beyond 27),
// split into TF32 hi and the FP32 remainder lo, stored K-major (m along K) in
// 8 x 4 core matrices: float offset (j / 8) * 256 + (m / 4) * 32 +
// (j % 8) * 4 + m % 4.  Layout [r][hi, lo][1024].
std::vector<float> tc_volume_operators(const RefTables& T) {
  std::vector<float> out(3 * 2 * 1024, 0.0f);
  for (int r = 0; r < 3; ++r)
    for (int j = 0; j < 27; ++j)
      for (int m = 0; m < 27; ++m) {
        const int jx = j % 3, jy = (j / 3) % 3, jz = j / 9;
        const int mx = m % 3, my = (m / 3) % 3, mz = m / 9;
        double v = 0.0;
        if (r == 0 && my == jy && mz == jz) v = T.w1[jy] * T.w1[jz] * T.d1[jx][mx];
        if (r == 1 && mx == jx && mz == jz) v = T.w1[jx] * T.w1[jz] * T.d1[jy][my];
        if (r == 2 && mx == jx && my == jy) v = T.w1[jx] * T.w1[jy] * T.d1[jz][mz];
        const float hi = tf32_hi_host((float)v);
        const float lo = (float)(v - (double)hi);
        const int o = (j / 8) * 256 + (m / 4) * 32 + (j % 8) * 4 + m % 4;
        out[(size_t)(r * 2 + 0) * 1024 + o] = hi;
        out[(size_t)(r * 2 + 1) * 1024 + o] = lo;
      }
  return out;
}

int check_device_error(rkdg_ctx* c) {
  if (c->h_err[0] != 0) {
    const int code = c->h_err[0];
    char msg[128];
    if (code == 8)  // a bounded wait on the tensor core gave up (tile kernel)
      snprintf(msg, sizeof msg, "tensor-core completion wait timed out in tile %d", c->h_err[1]);
    else
      snprintf(msg, sizeof msg, "non-physical state in the Riemann solver at element %d",
               c->h_err[1]);
    CUDA_TRY(c, cudaMemsetAsync(c->d_err, 0, 2 * sizeof(int), c->stream));
    return fail(c, code == 2 ? RKDG_ERR_UNPHYSICAL : RKDG_ERR_CUDA, msg, c->h_err[1]);
  }
  return RKDG_OK;
}

LimParams lim_params_for(rkdg_ctx* c, bool batch) {
  LimParams L = lim_params(c);
  if (batch) {
    L.prob = c->d_prob;
    L.pgamma = c->d_pgamma;
    L.pcov = c->d_pcov;
    L.pgamma32 = c->d_pgamma32;
    L.pcov32 = c->d_pcov32;
    L.pactive = c->d_pactive;
    L.act_cum = c->d_act_cum;
    L.act_pid = c->d_act_pid;
    L.act_n = c->d_act_n;
    L.poff = c->d_poff;
  }
  return L;
}

cudaError_t zero_slot(rkdg_ctx* c, int i, bool batch) {
  if (batch)
    return cudaMemsetAsync(c->d_pmcs + (size_t)i * c->nprob, 0,
                           (size_t)c->nprob * sizeof(unsigned long long), c->stream);
  return cudaMemsetAsync(c->d_mcs + i, 0, sizeof(unsigned long long), c->stream);
}

// Enqueue one Runge-Kutta step on the FP64 state x (no host synchronisation).
// batch: every problem uses its own dt_real (d_pdtr) and EoS constants.
int enqueue_step64(rkdg_ctx* c, double* x, double dt, bool batch = false) {
  const int s = c->s;
  const bool lim = c->limiter_active();
  const long long n = c->ndofs * c->neq;
  if (batch) dt = 1.0;
  for (int i = 0; i < s; ++i) {
    const double* in;
    if (i == 0) {
      if (s == 1) {
        CUDA_TRY(c, cudaMemcpyAsync(c->d_y64[0], x, n * sizeof(double), cudaMemcpyDeviceToDevice,
                                    c->stream));
        in = c->d_y64[0];
      } else {
        in = x;
      }
    } else {
      in = c->d_y64[i % 2];
    }
    CUDA_TRY(c, zero_slot(c, i, batch));
    EpiParams<double> ep;
    std::memset(&ep, 0, sizeof ep);
    ep.mode = 1;
    ep.base = x;
    if (batch) {
      ep.prob = c->d_prob;
      ep.pdt = c->d_pdtr;
    }
    double* out;
    if (i < s - 1) {
      const int row = (i + 1) * i / 2;  // MFEM packing: coefficients of y_{i+1}
      for (int j = 0; j < i; ++j) {
        ep.kprev[j] = c->d_k64[j];
        ep.cprev[j] = c->a[row + j] * dt;
      }
      ep.nprev = i;
      ep.ccur = c->a[row + i] * dt;
      ep.kout = c->d_k64[i];
      out = c->d_y64[(i + 1) % 2];
    } else {
      for (int j = 0; j < s - 1; ++j) {
        ep.kprev[j] = c->d_k64[j];
        ep.cprev[j] = c->b[j] * dt;
      }
      ep.nprev = s - 1;
      ep.ccur = c->b[s - 1] * dt;
      out = x;
    }
    ep.out64 = out;
    ep.means = lim ? c->d_means : nullptr;
    RhsParams P = rhs_params(c, 0, 0, i);
    if (batch) set_batch(c, P, i);
    CUDA_TRY(c, launch_rhs_nc(c, 0, P, in, &ep));
    c->launches += rhs_kernels(c, P);
    if (lim) {
      LimParams L = lim_params_for(c, batch);
      CUDA_TRY(c, rkdg::launch_limit(c->geom, c->p, 0, L, out, nullptr, c->stream));
      c->launches++;
    }
  }
  return RKDG_OK;
}

void split_coef(double v, float& hi, float& lo) {
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

// Enqueue one step on the float-pair state (d_xh, d_xl).
int enqueue_step32(rkdg_ctx* c, double dt, bool batch = false) {
  const int s = c->s;
  const bool lim = c->limiter_active();
  const long long n = c->ndofs * c->neq;
  if (batch) dt = 1.0;
  for (int i = 0; i < s; ++i) {
    const float* in;
    if (i == 0) {
      if (s == 1) {
        CUDA_TRY(c, rkdg::launch_copy_f(n, c->d_xh, c->d_y32[0], c->stream));
        c->launches++;
        in = c->d_y32[0];
      } else {
        in = c->d_xh;
      }
    } else {
      in = c->d_y32[i % 2];
    }
    CUDA_TRY(c, zero_slot(c, i, batch));
    EpiParams<float> ep;
    std::memset(&ep, 0, sizeof ep);
    ep.mode = 1;
    ep.basehi = c->d_xh;
    ep.baselo = c->d_xl;
    if (batch) {
      ep.prob = c->d_prob;
      ep.pdt = c->d_pdtr;
      ep.pdt2 = c->d_pdt2;
    }
    if (i < s - 1) {
      const int row = (i + 1) * i / 2;
      for (int j = 0; j < i; ++j) {
        ep.kprev[j] = c->d_k32[j];
        ep.cprev[j] = c->a[row + j] * dt;
        split_coef(c->a[row + j] * dt, ep.cprev_hi[j], ep.cprev_lo[j]);
      }
      ep.nprev = i;
      ep.ccur = c->a[row + i] * dt;
      split_coef(c->a[row + i] * dt, ep.ccur_hi, ep.ccur_lo);
      ep.kout = c->d_k32[i];
      ep.out32 = c->d_y32[(i + 1) % 2];
      ep.final_stage = 0;
    } else {
      for (int j = 0; j < s - 1; ++j) {
        ep.kprev[j] = c->d_k32[j];
        ep.cprev[j] = c->b[j] * dt;
        split_coef(c->b[j] * dt, ep.cprev_hi[j], ep.cprev_lo[j]);
      }
      ep.nprev = s - 1;
      ep.ccur = c->b[s - 1] * dt;
      split_coef(c->b[s - 1] * dt, ep.ccur_hi, ep.ccur_lo);
      ep.out32 = c->d_xh;
      ep.outlo = c->d_xl;
      ep.final_stage = 1;
    }
    // the FP32 path's means are float pairs in the same buffer (8 bytes each)
    ep.means32 = lim ? reinterpret_cast<float2*>(c->d_means) : nullptr;
    RhsParams P = rhs_params(c, 1, 0, i);
    if (batch) set_batch(c, P, i);
    CUDA_TRY(c, launch_rhs_nc(c, 1, P, in, &ep));
    c->launches += rhs_kernels(c, P);
    if (lim) {
      LimParams L = lim_params_for(c, batch);
      L.means = nullptr;
      L.means32 = reinterpret_cast<const float2*>(c->d_means);
      if (i < s - 1)
        CUDA_TRY(c, rkdg::launch_limit(c->geom, c->p, 1, L, c->d_y32[(i + 1) % 2], nullptr, c->stream));
      else
        CUDA_TRY(c, rkdg::launch_limit(c->geom, c->p, 2, L, c->d_xh, c->d_xl, c->stream));
      c->launches++;
    }
  }
  return RKDG_OK;
}

int read_mcs(rkdg_ctx* c, int slot, double* out) {
  CUDA_TRY(c, cudaMemcpyAsync(c->h_mcs, c->d_mcs + slot, sizeof(unsigned long long),
                              cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(c->h_err, c->d_err, 2 * sizeof(int), cudaMemcpyDeviceToHost,
                              c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  int st = check_device_error(c);
  if (st) return st;
  if (out) {
    double v;
    unsigned long long bits = c->h_mcs[0];
    std::memcpy(&v, &bits, sizeof v);
    *out = v;
  }
  return RKDG_OK;
}

// The time loop of main.cpp:509-553,701-733 from time t with the step's
// dt known: dt_real = min(dt, t_end - t), one step, the next dt from the
// last stage's speed (dt_mode 0), t += that dt (the reference books t with
// the new dt), done when t >= t_end - 1e-8 dt.
int run_loop(rkdg_ctx* c, double* x, double t, double dt, double t_end, double cfl, int dt_mode,
             int max_steps, int* steps_out, double* t_out, double* dt_out, double* sum_dt_out) {
  if (!(dt > 0)) return fail(c, RKDG_ERR_INVALID, "non-positive dt");
  const long long n = c->ndofs * c->neq;
  const double denom = 2.0 * c->p + 1.0;
  const bool fp32 = c->precision != RKDG_FP64;
  int st;
  if (fp32) {
    CUDA_TRY(c, rkdg::launch_split(n, x, c->d_xh, c->d_xl, c->stream));
    c->launches++;
  }
  double sum_dt = 0.0;
  int ti = 0;
  bool done = false;
  while (!done) {
    const double dt_real = std::min(dt, t_end - t);
    st = fp32 ? enqueue_step32(c, dt_real) : enqueue_step64(c, x, dt_real);
    if (st) return st;
    sum_dt += dt_real;
    if (dt_mode == 0) {
      double mcs = 0;
      st = read_mcs(c, c->s - 1, &mcs);
      if (st) return st;
      dt = cfl * c->hmin / mcs / denom;
      // The reference loops forever on a non-finite or vanishing dt; stop instead.
      if (!std::isfinite(dt) || !(dt > 0.0) || (t_end < 1e20 && dt < 1e-14 * t_end))
        return fail(c, RKDG_ERR_UNPHYSICAL, "non-finite or vanishing CFL time step", ti);
    }
    t += dt;
    ti++;
    done = (t >= t_end - 1e-8 * dt);
    if (max_steps > 0 && ti >= max_steps) break;
  }
  if (fp32) {
    CUDA_TRY(c, rkdg::launch_join(n, c->d_xh, c->d_xl, x, c->stream));
    c->launches++;
  }
  st = read_mcs(c, c->s - 1, nullptr);
  if (st) return st;
  if (steps_out) *steps_out = ti;
  if (t_out) *t_out = t;
  if (dt_out) *dt_out = dt;
  if (sum_dt_out) *sum_dt_out = sum_dt;
  return RKDG_OK;
}

#define NEED_MESH(c)                                              \
  do {                                                            \
    if (!(c)) return RKDG_ERR_INVALID;                            \
    if (!(c)->has_mesh) return fail(c, RKDG_ERR_NOMESH, "no mesh"); \
    cudaSetDevice((c)->device);                                   \
  } while (0)

}  // namespace

extern "C" {

int rkdg_create(rkdg_ctx** out, int device) {
  if (!out) return RKDG_ERR_INVALID;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return RKDG_ERR_NOT_FOUND;
  if (device < 0 || device >= n) return RKDG_ERR_INVALID;
  rkdg_ctx* c = new rkdg_ctx();
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc((void**)&c->d_mcs, 8 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc((void**)&c->d_err, 2 * sizeof(int)) != cudaSuccess ||
      cudaMallocHost((void**)&c->h_mcs, 8 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMallocHost((void**)&c->h_err, 2 * sizeof(int)) != cudaSuccess ||
      cudaMemset(c->d_err, 0, 2 * sizeof(int)) != cudaSuccess) {
    delete c;
    return RKDG_ERR_CUDA;
  }
  c->own_stream = true;
  *out = c;
  return RKDG_OK;
}

int rkdg_destroy(rkdg_ctx* c) {
  if (!c) return RKDG_ERR_INVALID;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  free_mesh(c);
  dfree(c->d_mcs);
  dfree(c->d_err);
  if (c->h_mcs) cudaFreeHost(c->h_mcs);
  if (c->h_err) cudaFreeHost(c->h_err);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return RKDG_OK;
}

const char* rkdg_last_error(rkdg_ctx* c, long long* where) {
  if (!c) return "null context";
  if (where) *where = c->err_where;
  return c->err.c_str();
}

int rkdg_set_stream(rkdg_ctx* c, void* st) {
  if (!c) return RKDG_ERR_INVALID;
  cudaSetDevice(c->device);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  if (st) {
    c->stream = (cudaStream_t)st;
    c->own_stream = false;
  } else {
    CUDA_TRY(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    c->own_stream = true;
  }
  return RKDG_OK;
}

int rkdg_synchronize(rkdg_ctx* c) {
  if (!c) return RKDG_ERR_INVALID;
  cudaSetDevice(c->device);
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return RKDG_OK;
}

int rkdg_set_physics(rkdg_ctx* c, int rsolver, int averaging, double gamma, double covolume,
                     double gas_constant) {
  if (!c) return RKDG_ERR_INVALID;
  if (rsolver < 0 || rsolver > 3 || averaging < 0 || averaging > 1 || !(gamma > 1.0) ||
      covolume < 0.0)
    return fail(c, RKDG_ERR_INVALID, "invalid physics parameters");
  c->rs = rsolver;
  c->avg = averaging;
  c->gamma = gamma;
  c->cov = covolume;
  c->gasR = gas_constant;
  return RKDG_OK;
}

int rkdg_set_bc(rkdg_ctx* c, int attr, int type, const double* state) {
  if (!c) return RKDG_ERR_INVALID;
  if (type < 0 || type > 10 || attr < 1) return fail(c, RKDG_ERR_INVALID, "invalid boundary condition");
  if ((type == RKDG_BC_FIXED_ROTATED || type == RKDG_BC_SUPERSONIC_INLET || type >= 5) && !state)
    return fail(c, RKDG_ERR_INVALID, "this boundary condition needs a state or its parameters");
  if (!c->bcs.count(attr) && (int)c->bcs.size() >= RKDG_MAX_BC)
    return fail(c, RKDG_ERR_INVALID, "too many boundary attributes");
  BCSlot bc;
  std::memset(&bc, 0, sizeof bc);
  bc.type = type;
  if (state)
    for (int i = 0; i < 5; ++i) bc.state[i] = (i < (c->has_mesh ? c->neq : 5)) ? state[i] : 0.0;
  c->bcs[attr] = bc;
  if (c->has_mesh) {
    cudaSetDevice(c->device);
    return refresh_fnbr(c);
  }
  return RKDG_OK;
}

int rkdg_set_limiter(rkdg_ctx* c, int limiter, int indicator, int function, int last_hope,
                     int quirk_flags) {
  if (!c) return RKDG_ERR_INVALID;
  if (limiter < 0 || limiter > 1 || indicator < 0 || indicator > 3 || function < 0 || function > 2)
    return fail(c, RKDG_ERR_INVALID, "invalid limiter configuration");
  if (indicator == RKDG_IND_SHU && c->has_mesh && c->nonaffine)
    return fail(c, RKDG_ERR_UNSUPPORTED,
                "the Shu indicator maps between elements affinely: not on non-parallelogram quads");
  if (indicator == RKDG_IND_SHU && limiter == RKDG_LIM_MULTI)
    return fail(c, RKDG_ERR_UNSUPPORTED,
                "Shu indicator with the Multi limiter: the reference multiplies by a cell "
                "factor the Shu indicator never sets");
  if ((quirk_flags & RKDG_LIMITER_LINEARIZE) && limiter == RKDG_LIM_MULTI && c->has_mesh &&
      c->geom != RKDG_GEOM_TRIANGLE && !c->tab.lin_ok)
    return fail(c, RKDG_ERR_UNSUPPORTED,
                "linearize needs order 1 (its rule of order p+1 has fewer points than nodes)");
  c->lim = limiter;
  c->ind = indicator;
  c->fun = function;
  c->last_hope = last_hope ? 1 : 0;
  c->quirks = quirk_flags;
  return RKDG_OK;
}

int rkdg_set_tableau(rkdg_ctx* c, int s, const double* a, const double* b, const double* cc) {
  if (!c) return RKDG_ERR_INVALID;
  if (s < 1 || s > 4 || !b || (s > 1 && !a)) return fail(c, RKDG_ERR_INVALID, "invalid tableau");
  c->s = s;
  c->a.assign(a ? a : b, (a ? a : b) + s * (s - 1) / 2);
  c->b.assign(b, b + s);
  if (cc)
    c->c.assign(cc, cc + std::max(s - 1, 0));
  else
    c->c.assign(std::max(s - 1, 0), 0.0);
  if (c->has_mesh) {
    cudaSetDevice(c->device);
    return ensure_scratch(c);
  }
  return RKDG_OK;
}

int rkdg_set_precision(rkdg_ctx* c, int precision) {
  if (!c) return RKDG_ERR_INVALID;
  if (precision != RKDG_FP64 && precision != RKDG_FP32_BULK)
    return fail(c, RKDG_ERR_INVALID, "invalid precision");
  c->precision = precision;
  if (c->has_mesh) {
    cudaSetDevice(c->device);
    return ensure_scratch(c);
  }
  return RKDG_OK;
}

int rkdg_set_solver_quirks(rkdg_ctx* c, int flags) {
  if (!c) return RKDG_ERR_INVALID;
  if (flags & ~(RKDG_QUIRK_HLLC_NEGATIVE_SPEED_OK | RKDG_QUIRK_NO_INITIAL_LIMIT))
    return fail(c, RKDG_ERR_INVALID, "unknown solver quirk flag");
  c->solver_quirks = flags;
  return RKDG_OK;
}

int rkdg_set_tuning(rkdg_ctx* c, int key, int value) {
  if (!c) return RKDG_ERR_INVALID;
  if (key == RKDG_TUNE_HEX_KERNEL && value >= 0 && value <= 6) {
    if (value == 3 && c->has_mesh) {
      const int st = ensure_fslot(c);
      if (st) return st;
    }
    c->hex_variant = value;
    return RKDG_OK;
  }
  const bool block_ok = value == 0 || (value >= 32 && value <= 256 && value % 32 == 0);
  if (key == RKDG_TUNE_GENERIC_BLOCK && block_ok) {
    c->gen_block = value;
    return RKDG_OK;
  }
  if (key == RKDG_TUNE_LIMITER_BLOCK && block_ok) {
    c->lim_block = value;
    return RKDG_OK;
  }
  return fail(c, RKDG_ERR_INVALID, "unknown tuning key or value");
}

int rkdg_upload_mesh(rkdg_ctx* c, const rkdg_mesh_desc* m) {
  if (!c || !m) return RKDG_ERR_INVALID;
  cudaSetDevice(c->device);
  const int dim = m->dim, geom = m->geom, p = m->order, ne = m->num_elements;
  if (!((dim == 2 && (geom == RKDG_GEOM_TRIANGLE || geom == RKDG_GEOM_SQUARE)) ||
        (dim == 3 && geom == RKDG_GEOM_CUBE)))
    return fail(c, RKDG_ERR_UNSUPPORTED, "unsupported geometry / dimension");
  if (!rkdg::generic_supported(geom, p))
    return fail(c, RKDG_ERR_UNSUPPORTED, "unsupported polynomial order for this geometry");
  if (ne <= 0 || !m->elem_vertices || !m->elem_coords || m->num_bdr < 0 ||
      (m->num_bdr > 0 && (!m->bdr_vertices || !m->bdr_attr)))
    return fail(c, RKDG_ERR_INVALID, "invalid mesh description");
  free_mesh(c);
  RefTables T;
  std::vector<rkdg::FacePoint> fpts;
  if (!rkdg::build_ref_tables(geom, p, T, &fpts))
    return fail(c, RKDG_ERR_UNSUPPORTED, "reference tables exceed the supported sizes");
  const int nvpe = nvpe_of(geom), nfpe = nfpe_of(geom), nvpf = dim == 2 ? 2 : 4;
  const int gs = rkdg::geom_slot(geom);
  const int nd = T.nd, neq = dim + 2;
  c->dim = dim;
  c->geom = geom;
  c->p = p;
  c->ne = ne;
  c->nd = nd;
  c->neq = neq;
  c->nfpe = nfpe;
  c->nvpe = nvpe;
  c->ndofs = (long long)ne * nd;
  // ---- element geometry (affine elements) ----
  c->h_egeo.assign((size_t)(dim * dim + 1) * ne, 0.0);
  c->h_eaff.assign((size_t)(dim * dim + dim) * ne, 0.0);
  c->h_wdet.assign(ne, 0.0);
  c->h_ehmin.assign(ne, 0.0);
  c->h_nodes.assign((size_t)dim * c->ndofs, 0.0);
  const double refvol = geom == 2 ? 0.5 : 1.0;
  double hmin = 1e300;
  std::vector<double> Jall((size_t)ne * 9);
  for (int e = 0; e < ne; ++e) {
    const double* X = m->elem_coords + (size_t)e * nvpe * dim;
    double col[3][3] = {{0}};
    const int vi[3] = {1, geom == 2 ? 2 : 3, 4};
    for (int r = 0; r < dim; ++r)
      for (int i = 0; i < dim; ++i) col[r][i] = X[vi[r] * dim + i] - X[i];
    double scale = 0;
    for (int r = 0; r < dim; ++r)
      for (int i = 0; i < dim; ++i) scale = std::max(scale, std::fabs(col[r][i]));
    bool affine = true;
    for (int v = 0; v < nvpe; ++v) {
      const double* rv = rkdg::kRefVert[gs][v];
      for (int i = 0; i < dim; ++i) {
        double pred = X[i];
        for (int r = 0; r < dim; ++r) pred += rv[r] * col[r][i];
        if (std::fabs(pred - X[v * dim + i]) > 1e-9 * scale) affine = false;
      }
    }
    if (!affine) {
      if (geom != RKDG_GEOM_SQUARE)
        return fail(c, RKDG_ERR_UNSUPPORTED,
                    "non-affine hexahedron (bilinear quadrilaterals and affine elements are supported)", e);
      // bilinear quadrilateral: J at the element centre (Mesh::GetElementSize)
      for (int i = 0; i < 2; ++i) {
        col[0][i] = 0.5 * ((X[2 + i] - X[i]) + (X[4 + i] - X[6 + i]));
        col[1][i] = 0.5 * ((X[6 + i] - X[i]) + (X[4 + i] - X[2 + i]));
      }
      c->nonaffine++;
    }
    double J[9] = {0};
    for (int i = 0; i < dim; ++i)
      for (int r = 0; r < dim; ++r) J[i * dim + r] = col[r][i];
    double det, adj[9];
    if (dim == 2) {
      det = J[0] * J[3] - J[1] * J[2];
      adj[0] = J[3];
      adj[1] = -J[1];
      adj[2] = -J[2];
      adj[3] = J[0];
    } else {
      adj[0] = J[4] * J[8] - J[5] * J[7];
      adj[1] = J[2] * J[7] - J[1] * J[8];
      adj[2] = J[1] * J[5] - J[2] * J[4];
      adj[3] = J[5] * J[6] - J[3] * J[8];
      adj[4] = J[0] * J[8] - J[2] * J[6];
      adj[5] = J[2] * J[3] - J[0] * J[5];
      adj[6] = J[3] * J[7] - J[4] * J[6];
      adj[7] = J[1] * J[6] - J[0] * J[7];
      adj[8] = J[0] * J[4] - J[1] * J[3];
      det = J[0] * adj[0] + J[1] * adj[3] + J[2] * adj[6];
    }
    if (!(det > 0.0)) return fail(c, RKDG_ERR_INVALID, "inverted or degenerate element", e);
    for (int rd = 0; rd < dim * dim; ++rd) c->h_egeo[(size_t)rd * ne + e] = adj[rd];
    c->h_egeo[(size_t)(dim * dim) * ne + e] = 1.0 / det;
    c->h_wdet[e] = det * refvol;
    for (int rd = 0; rd < dim * dim; ++rd) c->h_eaff[(size_t)rd * ne + e] = J[rd];
    for (int i = 0; i < dim; ++i) c->h_eaff[(size_t)(dim * dim + i) * ne + e] = X[i];
    double Jp[9];
    std::memcpy(Jp, J, sizeof Jp);
    if (geom == 2) {  // relative to the equilateral reference triangle
      const double A[4] = {1.0, -1.0 / std::sqrt(3.0), 0.0, 2.0 / std::sqrt(3.0)};
      for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) Jp[i * 2 + j] = J[i * 2] * A[j] + J[i * 2 + 1] * A[2 + j];
    }
    c->h_ehmin[e] = min_singular(dim, Jp);
    hmin = std::min(hmin, c->h_ehmin[e]);
    std::memcpy(&Jall[(size_t)e * 9], J, sizeof J);
  }
  c->hmin = hmin;
  // ---- non-parallelogram (bilinear) quadrilaterals ----
  // The volume and mass rules of quads are the Gauss-Legendre nodes (orders
  // 2p and 2p + 1), so the element operator only needs adj(J) and det J at
  // the nodes; cell means use the averages rule (order p + 1) with det J.
  std::vector<double> h_ngeo, h_wmn;
  if (c->nonaffine) {
    rkdg::Basis B(geom, p);
    std::vector<double> rx, rw, phi(nd);
    rkdg::mean_rule(geom, p, rx, rw);
    h_ngeo.assign((size_t)5 * nd * ne, 0.0);
    h_wmn.assign((size_t)ne * nd, 0.0);
    for (int e = 0; e < ne; ++e) {
      const double* X = m->elem_coords + (size_t)e * 8;
      auto jac = [&](const double* xi, double* J) {  // J[i*2 + r] = dx_i / dxi_r
        const double s = xi[0], t = xi[1];
        for (int i = 0; i < 2; ++i) {
          J[i * 2] = (1 - t) * (X[2 + i] - X[i]) + t * (X[4 + i] - X[6 + i]);
          J[i * 2 + 1] = (1 - s) * (X[6 + i] - X[i]) + s * (X[4 + i] - X[2 + i]);
        }
        return J[0] * J[3] - J[1] * J[2];
      };
      for (int j = 0; j < nd; ++j) {
        double J[4];
        const double det = jac(&B.nodes[j * 2], J);
        if (!(det > 0.0)) return fail(c, RKDG_ERR_INVALID, "inverted or degenerate element", e);
        const double adj[4] = {J[3], -J[1], -J[2], J[0]};
        for (int rd = 0; rd < 4; ++rd) h_ngeo[((size_t)rd * nd + j) * ne + e] = adj[rd];
        h_ngeo[((size_t)4 * nd + j) * ne + e] = 1.0 / det;
      }
      double area = 0.0;
      for (size_t q = 0; q < rw.size(); ++q) {
        double J[4];
        const double w = rw[q] * jac(&rx[q * 2], J);
        B.eval(&rx[q * 2], phi.data(), nullptr);
        for (int j = 0; j < nd; ++j) h_wmn[(size_t)e * nd + j] += w * phi[j];
        area += w;
      }
      for (int j = 0; j < nd; ++j) h_wmn[(size_t)e * nd + j] /= area;
      c->h_wdet[e] = area;
    }
  }
  {
    rkdg::Basis B(geom, p);
    for (int e = 0; e < ne; ++e) {
      const double* X = m->elem_coords + (size_t)e * nvpe * dim;
      const double* J = &Jall[(size_t)e * 9];
      for (int j = 0; j < nd; ++j)
        for (int i = 0; i < dim; ++i) {
          double v = X[i];
          if (c->nonaffine && geom == RKDG_GEOM_SQUARE) {  // bilinear map
            const double s = B.nodes[j * 2], t = B.nodes[j * 2 + 1];
            v = (1 - s) * (1 - t) * X[i] + s * (1 - t) * X[2 + i] + s * t * X[4 + i] + (1 - s) * t * X[6 + i];
          } else {
            for (int r = 0; r < dim; ++r) v += J[i * dim + r] * B.nodes[j * dim + r];
          }
          c->h_nodes[(size_t)i * c->ndofs + (long long)e * nd + j] = v;
        }
    }
  }
  // ---- faces ----
  struct Side {
    int e = -1, lf = -1;
  };
  struct FaceRec {
    Side s1, s2;
  };
  std::map<std::array<int, 4>, int> key2f;
  std::vector<FaceRec> faces;
  auto face_key = [&](const int* ids) {
    std::array<int, 4> k = {-1, -1, -1, -1};
    for (int i = 0; i < nvpf; ++i) k[i] = ids[i];
    for (int i = 1; i < nvpf; ++i)
      for (int j = i; j > 0 && k[j - 1] > k[j]; --j) std::swap(k[j - 1], k[j]);
    return k;
  };
  for (int e = 0; e < ne; ++e)
    for (int lf = 0; lf < nfpe; ++lf) {
      int ids[4];
      for (int k = 0; k < nvpf; ++k)
        ids[k] = m->elem_vertices[(size_t)e * nvpe + rkdg::kFaceVert[gs][lf][k]];
      auto key = face_key(ids);
      auto it = key2f.find(key);
      if (it == key2f.end()) {
        key2f[key] = (int)faces.size();
        FaceRec f;
        f.s1 = {e, lf};
        faces.push_back(f);
      } else {
        FaceRec& f = faces[it->second];
        if (f.s2.e >= 0) return fail(c, RKDG_ERR_INVALID, "non-manifold face", e);
        f.s2 = {e, lf};
      }
    }
  std::map<std::array<int, 4>, int> bkey;
  std::vector<rkdg::NcFace> lone;
  for (int i = 0; i < m->num_bdr; ++i) bkey[face_key(m->bdr_vertices + (size_t)i * nvpf)] = m->bdr_attr[i];
  c->h_fnbr.assign((size_t)nfpe * ne, -1);
  c->h_fattr.assign((size_t)nfpe * ne, 0);
  c->h_fcode.assign((size_t)nfpe * ne, 0);
  c->h_fgeo.assign((size_t)nfpe * (dim + 1) * ne, 0.0);
  std::map<std::vector<int>, int> perm_ids;
  {
    std::vector<int> id(T.nqf);
    for (int q = 0; q < T.nqf; ++q) id[q] = q;
    perm_ids[id] = 0;
    for (int q = 0; q < T.nqf; ++q) T.perm[0][q] = q;
  }
  auto fp_of = [&](int lf, int q) -> const rkdg::FacePoint& { return fpts[(size_t)lf * T.nqf + q]; };
  for (auto& kv : key2f) {
    const FaceRec& f = faces[kv.second];
    const int e1 = f.s1.e, lf1 = f.s1.lf;
    const double* X = m->elem_coords + (size_t)e1 * nvpe * dim;
    const int* fv = rkdg::kFaceVert[gs][lf1];
    double nor[3];
    if (dim == 2) {
      const double jx = X[fv[1] * 2] - X[fv[0] * 2], jy = X[fv[1] * 2 + 1] - X[fv[0] * 2 + 1];
      nor[0] = jy;
      nor[1] = -jx;
    } else {
      double ds[3], dt[3];
      for (int i = 0; i < 3; ++i) {
        ds[i] = X[fv[1] * 3 + i] - X[fv[0] * 3 + i];
        dt[i] = X[fv[3] * 3 + i] - X[fv[0] * 3 + i];
      }
      nor[0] = ds[1] * dt[2] - ds[2] * dt[1];
      nor[1] = ds[2] * dt[0] - ds[0] * dt[2];
      nor[2] = ds[0] * dt[1] - ds[1] * dt[0];
    }
    double nm = 0;
    for (int i = 0; i < dim; ++i) nm += nor[i] * nor[i];
    nm = std::sqrt(nm);
    const double inv = 1.0 / nm;
    double nh[3];
    for (int i = 0; i < dim; ++i) nh[i] = nor[i] * inv;
    auto put_geo = [&](int e, int lf) {
      for (int i = 0; i < dim; ++i) c->h_fgeo[(size_t)(lf * (dim + 1) + i) * ne + e] = nh[i];
      c->h_fgeo[(size_t)(lf * (dim + 1) + dim) * ne + e] = nm;
    };
    put_geo(e1, lf1);
    if (f.s2.e < 0) {
      auto bit = bkey.find(kv.first);
      c->h_fattr[(size_t)lf1 * ne + e1] = bit == bkey.end() ? 0 : bit->second;
      if (bit == bkey.end()) lone.push_back({e1, lf1});  // a hanging face (or a hole)
      c->h_fnbr[(size_t)lf1 * ne + e1] = -1;
      continue;
    }
    const int e2 = f.s2.e, lf2 = f.s2.lf;
    put_geo(e2, lf2);
    // point permutation: e1 canonical point q -> e2 canonical point on lf2
    std::vector<int> pm(T.nqf, -1);
    int ids1[4];
    for (int k = 0; k < nvpf; ++k) ids1[k] = m->elem_vertices[(size_t)e1 * nvpe + fv[k]];
    for (int q = 0; q < T.nqf; ++q) {
      const rkdg::FacePoint& P1 = fp_of(lf1, q);
      double N[4];
      if (dim == 2) {
        N[0] = 1 - P1.s[0];
        N[1] = P1.s[0];
      } else {
        N[0] = (1 - P1.s[0]) * (1 - P1.s[1]);
        N[1] = P1.s[0] * (1 - P1.s[1]);
        N[2] = P1.s[0] * P1.s[1];
        N[3] = (1 - P1.s[0]) * P1.s[1];
      }
      double xi2[3] = {0, 0, 0};
      for (int k = 0; k < nvpf; ++k) {
        int lv = -1;
        for (int mm = 0; mm < nvpf; ++mm) {
          const int v2 = rkdg::kFaceVert[gs][lf2][mm];
          if (m->elem_vertices[(size_t)e2 * nvpe + v2] == ids1[k]) lv = v2;
        }
        if (lv < 0) return fail(c, RKDG_ERR_INVALID, "inconsistent face vertices", e2);
        for (int i = 0; i < dim; ++i) xi2[i] += N[k] * rkdg::kRefVert[gs][lv][i];
      }
      for (int q2 = 0; q2 < T.nqf; ++q2) {
        const rkdg::FacePoint& P2 = fp_of(lf2, q2);
        double d = 0;
        for (int i = 0; i < dim; ++i) d = std::max(d, std::fabs(P2.xi[i] - xi2[i]));
        if (d < 1e-10) pm[q] = q2;
      }
      if (pm[q] < 0) return fail(c, RKDG_ERR_INVALID, "face points do not match", e2);
    }
    int pid;
    auto pit = perm_ids.find(pm);
    if (pit == perm_ids.end()) {
      pid = (int)perm_ids.size();
      if (pid >= RKDG_MAX_PERM) return fail(c, RKDG_ERR_UNSUPPORTED, "too many face orientations");
      perm_ids[pm] = pid;
      for (int q = 0; q < T.nqf; ++q) T.perm[pid][q] = pm[q];
    } else {
      pid = pit->second;
    }
    c->h_fnbr[(size_t)lf1 * ne + e1] = e2;
    c->h_fnbr[(size_t)lf2 * ne + e2] = e1;
    c->h_fcode[(size_t)lf1 * ne + e1] = lf2 | (0 << 3) | (pid << 4);
    c->h_fcode[(size_t)lf2 * ne + e2] = lf1 | (1 << 3) | (pid << 4);
  }
  T.nperm = (int)perm_ids.size();
  // ---- hanging faces (nonconforming meshes) ----
  std::vector<rkdg::NcSlave> slaves;
  std::vector<int> nc_face, nc_elem, nc_ptr, nc_ent, ncidx;
  std::vector<double> nc_bnc;
  {
    std::vector<double> fmeas((size_t)nfpe * ne);
    for (int lf = 0; lf < nfpe; ++lf)
      for (int e = 0; e < ne; ++e) fmeas[(size_t)lf * ne + e] = c->h_fgeo[(size_t)(lf * (dim + 1) + dim) * ne + e];
    std::string why;
    if (c->nonaffine && !lone.empty())
      return fail(c, RKDG_ERR_UNSUPPORTED, "hanging faces on non-parallelogram quadrilaterals");
    if (!rkdg::classify_nc_faces(geom, dim, nvpe, m->elem_coords, Jall, fmeas, ne, lone, slaves, why))
      return fail(c, RKDG_ERR_INVALID, why.c_str());
    const int nns = (int)slaves.size();
    if (nns) {
      rkdg::Basis B(geom, p);
      std::vector<std::vector<int>> ents(ne);
      nc_bnc.resize((size_t)nns * T.nqf * nd);
      std::vector<double> phi(nd);
      for (int f = 0; f < nns; ++f) {
        const rkdg::NcSlave& s = slaves[f];
        nc_face.insert(nc_face.end(), {s.e1, s.lf1, s.e2, s.lf2});
        ents[s.e1].push_back(2 * f);
        ents[s.e2].push_back(2 * f + 1);
        const double* X1 = m->elem_coords + (size_t)s.e1 * nvpe * dim;
        const double* X2 = m->elem_coords + (size_t)s.e2 * nvpe * dim;
        for (int q = 0; q < T.nqf; ++q) {
          const rkdg::FacePoint& fp = fp_of(s.lf1, q);
          double x[3] = {0, 0, 0}, xi2[3];
          for (int i = 0; i < dim; ++i) {
            x[i] = X1[i];
            for (int r = 0; r < dim; ++r) x[i] += Jall[(size_t)s.e1 * 9 + i * dim + r] * fp.xi[r];
          }
          rkdg::affine_inverse(dim, X2, &Jall[(size_t)s.e2 * 9], x, xi2);
          B.eval(xi2, phi.data(), nullptr);
          for (int j = 0; j < nd; ++j) nc_bnc[((size_t)f * T.nqf + q) * nd + j] = phi[j];
        }
      }
      ncidx.assign(ne, -1);
      nc_ptr.push_back(0);
      for (int e = 0; e < ne; ++e) {
        if (ents[e].empty()) continue;
        ncidx[e] = (int)nc_elem.size();
        nc_elem.push_back(e);
        nc_ent.insert(nc_ent.end(), ents[e].begin(), ents[e].end());
        nc_ptr.push_back((int)nc_ent.size());
      }
    }
  }
  // the hexahedral kernels keep one byte per point permutation of a square
  // face (at most its 8 orientations)
  if (c->geom == RKDG_GEOM_CUBE && T.nperm > RKDG_HEX_MAX_PERM)
    return fail(c, RKDG_ERR_UNSUPPORTED, "more hexahedral face orientations than a square face has");
  c->tab = T;
  // ---- upload ----
  const size_t nf = (size_t)nfpe * ne;
  if (c->nonaffine) {
    CUDA_TRY(c, dalloc(c->d_wmn64, h_wmn.size()));
    CUDA_TRY(c, cudaMemcpy(c->d_wmn64, h_wmn.data(), h_wmn.size() * sizeof(double), cudaMemcpyHostToDevice));
    std::vector<float> n32(h_ngeo.begin(), h_ngeo.end());
    CUDA_TRY(c, dalloc(c->d_ngeo64, h_ngeo.size()));
    CUDA_TRY(c, dalloc(c->d_ngeo32, n32.size()));
    CUDA_TRY(c, cudaMemcpy(c->d_ngeo64, h_ngeo.data(), h_ngeo.size() * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c->d_ngeo32, n32.data(), n32.size() * sizeof(float), cudaMemcpyHostToDevice));
  }
  c->tab.wmn_e = c->d_wmn64;
  c->tab.ngeo_e = c->d_ngeo64;
  CUDA_TRY(c, dalloc(c->d_tab, 1));
  CUDA_TRY(c, cudaMemcpy(c->d_tab, &c->tab, sizeof(RefTables), cudaMemcpyHostToDevice));
  CUDA_TRY(c, dalloc(c->d_fnbr, nf));
  CUDA_TRY(c, dalloc(c->d_fcode, nf));
  CUDA_TRY(c, cudaMemcpy(c->d_fcode, c->h_fcode.data(), nf * sizeof(int), cudaMemcpyHostToDevice));
  std::vector<float> f32(c->h_fgeo.begin(), c->h_fgeo.end());
  CUDA_TRY(c, dalloc(c->d_fgeo64, c->h_fgeo.size()));
  CUDA_TRY(c, dalloc(c->d_fgeo32, c->h_fgeo.size()));
  CUDA_TRY(c, cudaMemcpy(c->d_fgeo64, c->h_fgeo.data(), c->h_fgeo.size() * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy(c->d_fgeo32, f32.data(), f32.size() * sizeof(float), cudaMemcpyHostToDevice));
  std::vector<float> e32(c->h_egeo.begin(), c->h_egeo.end());
  CUDA_TRY(c, dalloc(c->d_egeo64, c->h_egeo.size()));
  CUDA_TRY(c, dalloc(c->d_egeo32, c->h_egeo.size()));
  CUDA_TRY(c, cudaMemcpy(c->d_egeo64, c->h_egeo.data(), c->h_egeo.size() * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy(c->d_egeo32, e32.data(), e32.size() * sizeof(float), cudaMemcpyHostToDevice));
  CUDA_TRY(c, dalloc(c->d_wdet, (size_t)ne));
  CUDA_TRY(c, cudaMemcpy(c->d_wdet, c->h_wdet.data(), ne * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_TRY(c, dalloc(c->d_eaff, c->h_eaff.size()));
  CUDA_TRY(c, cudaMemcpy(c->d_eaff, c->h_eaff.data(), c->h_eaff.size() * sizeof(double),
                         cudaMemcpyHostToDevice));
  CUDA_TRY(c, dalloc(c->d_means, (size_t)neq * ne));
  CUDA_TRY(c, dalloc(c->d_partial, (size_t)neq * 1024));
  if (!slaves.empty()) {
    const int nns = (int)slaves.size();
    c->nnc = nns;
    c->h_nc_face = nc_face;
    c->nc_nel = (int)nc_elem.size();
    CUDA_TRY(c, dalloc(c->d_nc_face, nc_face.size()));
    CUDA_TRY(c, dalloc(c->d_nc_bnc, nc_bnc.size()));
    // per face: both elements' terms (forward), or per point both sides'
    // flux derivatives (adjoint)
    CUDA_TRY(c, dalloc(c->d_nc_flux, (size_t)nns * 2 * neq * std::max(nd, T.nqf)));
    CUDA_TRY(c, dalloc(c->d_nc_elem, nc_elem.size()));
    CUDA_TRY(c, dalloc(c->d_nc_ptr, nc_ptr.size()));
    CUDA_TRY(c, dalloc(c->d_nc_ent, nc_ent.size()));
    CUDA_TRY(c, dalloc(c->d_ncidx, ncidx.size()));
    CUDA_TRY(c, dalloc(c->d_xface, (size_t)c->nc_nel * neq * nd));
    CUDA_TRY(c, cudaMemcpy(c->d_nc_face, nc_face.data(), nc_face.size() * sizeof(int), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c->d_nc_bnc, nc_bnc.data(), nc_bnc.size() * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c->d_nc_elem, nc_elem.data(), nc_elem.size() * sizeof(int), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c->d_nc_ptr, nc_ptr.data(), nc_ptr.size() * sizeof(int), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c->d_nc_ent, nc_ent.data(), nc_ent.size() * sizeof(int), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c->d_ncidx, ncidx.data(), ncidx.size() * sizeof(int), cudaMemcpyHostToDevice));
  }
  if (c->geom == RKDG_GEOM_CUBE && c->p <= 2) {
    std::vector<HexTeamSched> hs;
    if (rkdg::build_hex_sched(ne, nvpe, m->elem_coords, c->h_fnbr, c->h_fcode, hs, &c->hsched_rounds)) {
      CUDA_TRY(c, dalloc(c->d_hsched, hs.size()));
      CUDA_TRY(c, cudaMemcpy(c->d_hsched, hs.data(), hs.size() * sizeof(HexTeamSched),
                             cudaMemcpyHostToDevice));
    }
    std::vector<HexTile> ht;
    if (rkdg::build_hex_tiles(ne, nvpe, m->elem_coords, c->h_fnbr, c->h_fcode, ht)) {
      CUDA_TRY(c, dalloc(c->d_htile, ht.size()));
      CUDA_TRY(c, cudaMemcpy(c->d_htile, ht.data(), ht.size() * sizeof(HexTile), cudaMemcpyHostToDevice));
      c->ntile = (int)ht.size();
      int mh = 1;
      for (const HexTile& t : ht)
        for (int a = 0; a < 3; ++a) mh = std::max(mh, t.nh[a]);
      c->tile_hs = mh | 1;
    }
    if (c->p == 2) {
      const std::vector<float> tcb = tc_volume_operators(c->tab);
      CUDA_TRY(c, dalloc(c->d_tcb, tcb.size()));
      CUDA_TRY(c, cudaMemcpy(c->d_tcb, tcb.data(), tcb.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
  }
  c->has_mesh = true;
  int st = refresh_fnbr(c);
  if (st) return st;
  if (c->hex_variant == 3 || c->p == 1) {  // the split hexahedral kernels
    const int st = ensure_fslot(c);
    if (st) return st;
  }
  if ((c->quirks & RKDG_LIMITER_LINEARIZE) && c->lim == RKDG_LIM_MULTI &&
      c->geom != RKDG_GEOM_TRIANGLE && !c->tab.lin_ok)
    return fail(c, RKDG_ERR_UNSUPPORTED,
                "linearize needs order 1 (its rule of order p+1 has fewer points than nodes)");
  if (c->nonaffine && c->ind == RKDG_IND_SHU && c->limiter_active())
    return fail(c, RKDG_ERR_UNSUPPORTED,
                "the Shu indicator maps between elements affinely: not on non-parallelogram quads");
  return ensure_scratch(c);
}

int rkdg_sizes(rkdg_ctx* c, long long* ndofs, int* nd, int* neq) {
  if (!c) return RKDG_ERR_INVALID;
  if (!c->has_mesh) return fail(c, RKDG_ERR_NOMESH, "no mesh");
  if (ndofs) *ndofs = c->ndofs;
  if (nd) *nd = c->nd;
  if (neq) *neq = c->neq;
  return RKDG_OK;
}

int rkdg_node_coords_host(rkdg_ctx* c, double* out) {
  if (!c || !out) return RKDG_ERR_INVALID;
  if (!c->has_mesh) return fail(c, RKDG_ERR_NOMESH, "no mesh");
  std::memcpy(out, c->h_nodes.data(), c->h_nodes.size() * sizeof(double));
  return RKDG_OK;
}

int rkdg_hmin(rkdg_ctx* c, double* hmin) {
  if (!c || !hmin) return RKDG_ERR_INVALID;
  if (!c->has_mesh) return fail(c, RKDG_ERR_NOMESH, "no mesh");
  *hmin = c->hmin;
  return RKDG_OK;
}

int rkdg_rhs(rkdg_ctx* c, const double* x, double* y, double* mcs_out) {
  NEED_MESH(c);
  if (!x || !y) return fail(c, RKDG_ERR_INVALID, "null state pointer");
  CUDA_TRY(c, cudaMemsetAsync(c->d_mcs, 0, sizeof(unsigned long long), c->stream));
  const long long n = c->ndofs * c->neq;
  if (c->precision == RKDG_FP64) {
    EpiParams<double> ep;
    std::memset(&ep, 0, sizeof ep);
    ep.mode = 0;
    ep.out64 = y;
    RhsParams P = rhs_params(c, 0, 0, 0);
    CUDA_TRY(c, launch_rhs_nc(c, 0, P, x, &ep));
    c->launches += rhs_kernels(c, P);
  } else {
    CUDA_TRY(c, rkdg::launch_to_float(n, x, c->d_y32[0], c->stream));
    EpiParams<float> ep;
    std::memset(&ep, 0, sizeof ep);
    ep.mode = 0;
    ep.out64 = y;
    RhsParams P = rhs_params(c, 1, 0, 0);
    CUDA_TRY(c, launch_rhs_nc(c, 1, P, c->d_y32[0], &ep));
    c->launches += 1 + rhs_kernels(c, P);
  }
  return read_mcs(c, 0, mcs_out);
}

int rkdg_face_speed(rkdg_ctx* c, const double* x, double* mcs_out) {
  NEED_MESH(c);
  if (!x) return fail(c, RKDG_ERR_INVALID, "null state pointer");
  CUDA_TRY(c, cudaMemsetAsync(c->d_mcs, 0, sizeof(unsigned long long), c->stream));
  EpiParams<double> ep;
  std::memset(&ep, 0, sizeof ep);
  RhsParams P = rhs_params(c, 0, 1, 0);
  CUDA_TRY(c, launch_rhs_nc(c, 0, P, x, &ep));
  c->launches++;
  return read_mcs(c, 0, mcs_out);
}

int rkdg_cell_means(rkdg_ctx* c, const double* x, double* means) {
  NEED_MESH(c);
  if (!x || !means) return fail(c, RKDG_ERR_INVALID, "null pointer");
  CUDA_TRY(c, rkdg::launch_means(c->geom, c->p, 0, c->ne, c->ndofs, c->d_tab, x, nullptr, means, c->stream));
  c->launches++;
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return RKDG_OK;
}

int rkdg_limit(rkdg_ctx* c, double* x) {
  NEED_MESH(c);
  if (!x) return fail(c, RKDG_ERR_INVALID, "null state pointer");
  if (!c->limiter_active()) return RKDG_OK;
  CUDA_TRY(c, rkdg::launch_means(c->geom, c->p, 0, c->ne, c->ndofs, c->d_tab, x, nullptr, c->d_means, c->stream));
  LimParams L = lim_params(c);
  CUDA_TRY(c, rkdg::launch_limit(c->geom, c->p, 0, L, x, nullptr, c->stream));
  c->launches += 2;
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return RKDG_OK;
}

int rkdg_step(rkdg_ctx* c, double* x, double dt, double* next_mcs) {
  NEED_MESH(c);
  if (!x) return fail(c, RKDG_ERR_INVALID, "null state pointer");
  int st = ensure_scratch(c);
  if (st) return st;
  const long long n = c->ndofs * c->neq;
  if (c->precision == RKDG_FP64) {
    st = enqueue_step64(c, x, dt);
  } else {
    CUDA_TRY(c, rkdg::launch_split(n, x, c->d_xh, c->d_xl, c->stream));
    st = enqueue_step32(c, dt);
    if (!st) CUDA_TRY(c, rkdg::launch_join(n, c->d_xh, c->d_xl, x, c->stream));
    c->launches += 2;
  }
  if (st) return st;
  return read_mcs(c, c->s - 1, next_mcs);
}

int rkdg_run(rkdg_ctx* c, double* x, double t_end, double cfl, double dt0, int dt_mode,
             int max_steps, int* steps_out, double* t_out, double* dt_out, double* sum_dt_out) {
  NEED_MESH(c);
  if (!x || dt_mode < 0 || dt_mode > 2) return fail(c, RKDG_ERR_INVALID, "invalid run arguments");
  int st = ensure_scratch(c);
  if (st) return st;
  // The reference limits the projected initial state once before it forms the
  // initial dt and enters the loop (main.cpp:264-265).
  if (!(c->solver_quirks & RKDG_QUIRK_NO_INITIAL_LIMIT)) {
    st = rkdg_limit(c, x);
    if (st) return st;
  }
  double dt = dt0;
  if (dt_mode != 2) {
    double mcs = 0;
    st = rkdg_face_speed(c, x, &mcs);
    if (st) return st;
    if (!(mcs > 0)) return fail(c, RKDG_ERR_INVALID, "zero wave speed: cannot form a CFL dt");
    dt = cfl * c->hmin / mcs / (2.0 * c->p + 1.0);
  }
  return run_loop(c, x, 0.0, dt, t_end, cfl, dt_mode, max_steps, steps_out, t_out, dt_out,
                  sum_dt_out);
}

int rkdg_run_continue(rkdg_ctx* c, double* x, double t0, double dt, double t_end, double cfl,
                      int dt_mode, int max_steps, int* steps_out, double* t_out, double* dt_out,
                      double* sum_dt_out) {
  NEED_MESH(c);
  if (!x || dt_mode < 0 || dt_mode > 2 || !std::isfinite(t0))
    return fail(c, RKDG_ERR_INVALID, "invalid run arguments");
  int st = ensure_scratch(c);
  if (st) return st;
  return run_loop(c, x, t0, dt, t_end, cfl, dt_mode, max_steps, steps_out, t_out, dt_out,
                  sum_dt_out);
}

int rkdg_totals(rkdg_ctx* c, const double* x, double* totals) {
  NEED_MESH(c);
  if (!x || !totals) return fail(c, RKDG_ERR_INVALID, "null pointer");
  const int nb = 256;
  CUDA_TRY(c, rkdg::launch_totals(c->nd, c->neq, c->ne, c->ndofs, c->d_tab, c->d_wdet, x, c->d_partial, nb, c->stream));
  c->launches++;
  std::vector<double> part((size_t)c->neq * nb);
  CUDA_TRY(c, cudaMemcpyAsync(part.data(), c->d_partial, part.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  for (int k = 0; k < c->neq; ++k) {
    long double s = 0;
    for (int b = 0; b < nb; ++b) s += part[(size_t)k * nb + b];
    totals[k] = (double)s;
  }
  return RKDG_OK;
}

int rkdg_riemann_batch(rkdg_ctx* c, int n, const double* u1, const double* u2, const double* nor,
                       double* flux, double* speed) {
  if (!c) return RKDG_ERR_INVALID;
  if (!c->has_mesh) return fail(c, RKDG_ERR_NOMESH, "no mesh (the dimension comes from the mesh)");
  cudaSetDevice(c->device);
  if (n < 0 || (n > 0 && (!u1 || !u2 || !nor || !flux || !speed)))
    return fail(c, RKDG_ERR_INVALID, "invalid Riemann batch arguments");
  CUDA_TRY(c, rkdg::launch_riemann_batch(c->dim, c->precision == RKDG_FP64 ? 0 : 1, n, u1, u2, nor, flux,
                                         speed, c->gamma, c->cov, c->rs, c->avg, c->stream));
  c->launches++;
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return RKDG_OK;
}

int rkdg_batch_setup(rkdg_ctx* c, int nprob, const int* elem_offsets, const double* gamma,
                     const double* covolume) {
  NEED_MESH(c);
  if (nprob <= 0 || !elem_offsets || !gamma || !covolume)
    return fail(c, RKDG_ERR_INVALID, "invalid batch description");
  if (c->geom == RKDG_GEOM_CUBE)
    return fail(c, RKDG_ERR_UNSUPPORTED, "batched problems are supported on triangles and quads");
  if (elem_offsets[0] != 0 || elem_offsets[nprob] != c->ne)
    return fail(c, RKDG_ERR_INVALID, "element offsets must cover the mesh");
  std::vector<int> prob(c->ne);
  std::vector<double> phmin(nprob, 1e300);
  for (int p = 0; p < nprob; ++p) {
    if (elem_offsets[p + 1] <= elem_offsets[p] || !(gamma[p] > 1.0) || covolume[p] < 0.0)
      return fail(c, RKDG_ERR_INVALID, "invalid problem", p);
    for (int e = elem_offsets[p]; e < elem_offsets[p + 1]; ++e) {
      prob[e] = p;
      phmin[p] = std::min(phmin[p], c->h_ehmin[e]);
    }
  }
  // a problem must not share a face with another one
  for (int lf = 0; lf < c->nfpe; ++lf)
    for (int e = 0; e < c->ne; ++e) {
      const int nb = c->h_fnbr[(size_t)lf * c->ne + e];
      if (nb >= 0 && prob[nb] != prob[e])
        return fail(c, RKDG_ERR_INVALID, "problems are connected through a face", e);
    }
  for (int f = 0; f < c->nnc; ++f) {
    const int e1 = c->h_nc_face[(size_t)f * 4], e2 = c->h_nc_face[(size_t)f * 4 + 2];
    if (prob[e1] != prob[e2])
      return fail(c, RKDG_ERR_INVALID, "problems are connected through a hanging face", e1);
  }
  c->nprob = nprob;
  c->h_poff.assign(elem_offsets, elem_offsets + nprob + 1);
  CUDA_TRY(c, dalloc(c->d_prob, (size_t)c->ne));
  CUDA_TRY(c, dalloc(c->d_pgamma, (size_t)nprob));
  CUDA_TRY(c, dalloc(c->d_pcov, (size_t)nprob));
  CUDA_TRY(c, dalloc(c->d_pgamma32, (size_t)nprob));
  CUDA_TRY(c, dalloc(c->d_pcov32, (size_t)nprob));
  CUDA_TRY(c, dalloc(c->d_pdt2, (size_t)nprob));
  CUDA_TRY(c, dalloc(c->d_phmin, (size_t)nprob));
  CUDA_TRY(c, dalloc(c->d_pdt, (size_t)nprob));
  CUDA_TRY(c, dalloc(c->d_pdtr, (size_t)nprob));
  CUDA_TRY(c, dalloc(c->d_pt, (size_t)nprob));
  CUDA_TRY(c, dalloc(c->d_psum, (size_t)nprob));
  CUDA_TRY(c, dalloc(c->d_pactive, (size_t)nprob));
  CUDA_TRY(c, dalloc(c->d_psteps, (size_t)nprob));
  CUDA_TRY(c, dalloc(c->d_nactive, (size_t)1));
  CUDA_TRY(c, dalloc(c->d_act_cum, (size_t)nprob + 1));
  CUDA_TRY(c, dalloc(c->d_act_pid, (size_t)nprob));
  CUDA_TRY(c, dalloc(c->d_act_n, (size_t)1));
  CUDA_TRY(c, dalloc(c->d_poff, (size_t)nprob + 1));
  CUDA_TRY(c, cudaMemcpy(c->d_poff, elem_offsets, (nprob + 1) * sizeof(int), cudaMemcpyHostToDevice));
  CUDA_TRY(c, dalloc(c->d_pfail, (size_t)nprob));
  CUDA_TRY(c, dalloc(c->d_pmcs, (size_t)4 * nprob));
  CUDA_TRY(c, cudaMemcpy(c->d_prob, prob.data(), prob.size() * sizeof(int), cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy(c->d_pgamma, gamma, nprob * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy(c->d_pcov, covolume, nprob * sizeof(double), cudaMemcpyHostToDevice));
  {
    std::vector<float> g32(gamma, gamma + nprob), c32(covolume, covolume + nprob);
    CUDA_TRY(c, cudaMemcpy(c->d_pgamma32, g32.data(), nprob * sizeof(float), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c->d_pcov32, c32.data(), nprob * sizeof(float), cudaMemcpyHostToDevice));
  }
  CUDA_TRY(c, cudaMemcpy(c->d_phmin, phmin.data(), nprob * sizeof(double), cudaMemcpyHostToDevice));
  return RKDG_OK;
}

int rkdg_batch_run(rkdg_ctx* c, double* x, double t_end, double cfl, double dt0, int dt_mode,
                   int max_steps, int use_graph, int* steps_out, double* t_out, double* sum_dt_out) {
  NEED_MESH(c);
  if (c->nprob <= 0) return fail(c, RKDG_ERR_INVALID, "rkdg_batch_setup was not called");
  if (!x || dt_mode < 0 || dt_mode > 2 || !(t_end > 0.0) || (dt_mode == 2 && !(dt0 > 0.0)))
    return fail(c, RKDG_ERR_INVALID, "invalid batch run arguments");
  if (max_steps <= 0 && !(t_end < 1e20)) return fail(c, RKDG_ERR_INVALID, "unbounded batch run");
  int st = ensure_scratch(c);
  if (st) return st;
  const int np = c->nprob;
  const bool fp32 = c->precision != RKDG_FP64;
  const long long n = c->ndofs * c->neq;
  rkdg::BatchState bs;
  std::memset(&bs, 0, sizeof bs);
  bs.t_end = t_end;
  bs.cfl = cfl;
  bs.denom = 2.0 * c->p + 1.0;
  bs.nprob = np;
  bs.dt_mode = dt_mode;
  bs.max_steps = max_steps;
  bs.hmin = c->d_phmin;
  bs.dt = c->d_pdt;
  bs.dtr = c->d_pdtr;
  bs.dtr2 = c->d_pdt2;
  bs.t = c->d_pt;
  bs.sum_dt = c->d_psum;
  bs.active = c->d_pactive;
  bs.steps = c->d_psteps;
  bs.nactive = c->d_nactive;
  bs.act_cum = c->d_act_cum;
  bs.act_pid = c->d_act_pid;
  bs.act_n = c->d_act_n;
  bs.poff = c->d_poff;
  bs.mcs_last = c->d_pmcs + (size_t)(c->s - 1) * np;
  bs.fail = c->d_pfail;
  CUDA_TRY(c, cudaMemsetAsync(c->d_pfail, 0, np * sizeof(int), c->stream));
  // initial dt: face-only max speed per problem (main.cpp:467-484)
  {
    std::vector<int> ones(np, 1);
    CUDA_TRY(c, cudaMemcpyAsync(c->d_pactive, ones.data(), np * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    // the map of the active work (every problem) before any batched launch
    CUDA_TRY(c, rkdg::launch_batch_map(bs, c->stream));
    c->launches++;
    // each problem's projected state is limited once first (main.cpp:264-265)
    if (c->limiter_active() && !(c->solver_quirks & RKDG_QUIRK_NO_INITIAL_LIMIT)) {
      CUDA_TRY(c, rkdg::launch_means(c->geom, c->p, 0, c->ne, c->ndofs, c->d_tab, x, nullptr, c->d_means, c->stream));
      LimParams L = lim_params_for(c, true);
      CUDA_TRY(c, rkdg::launch_limit(c->geom, c->p, 0, L, x, nullptr, c->stream));
      c->launches += 2;
    }
    CUDA_TRY(c, zero_slot(c, c->s - 1, true));
    EpiParams<double> ep;
    std::memset(&ep, 0, sizeof ep);
    RhsParams P = rhs_params(c, 0, 1, 0);
    set_batch(c, P, c->s - 1);
    CUDA_TRY(c, launch_rhs_nc(c, 0, P, x, &ep));
    CUDA_TRY(c, rkdg::launch_batch_init(bs, dt0, c->stream));
    c->launches += 3;  // face speeds, per-problem dt, map of the active work
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  }
  if (fp32) {
    CUDA_TRY(c, rkdg::launch_split(n, x, c->d_xh, c->d_xl, c->stream));
    c->launches++;
  }
  const long long l0 = c->launches;
  long long per_step = 0;
  if (use_graph) {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    CUDA_TRY(c, cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h;
    CUDA_TRY(c, cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    CUDA_TRY(c, cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    CUDA_TRY(c, cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0,
                                              cudaStreamCaptureModeThreadLocal));
    st = fp32 ? enqueue_step32(c, 0.0, true) : enqueue_step64(c, x, 0.0, true);
    cudaError_t ce = st ? cudaSuccess : rkdg::launch_batch_control(bs, h, 1, c->stream);
    cudaGraph_t captured = nullptr;
    cudaError_t ce2 = cudaStreamEndCapture(c->stream, &captured);
    per_step = c->launches - l0 + 1;
    if (st || ce != cudaSuccess || ce2 != cudaSuccess) {
      cudaGraphDestroy(g);
      if (st) return st;
      return fail(c, RKDG_ERR_CUDA, std::string("graph capture failed: ") +
                                        cudaGetErrorString(ce != cudaSuccess ? ce : ce2));
    }
    cudaError_t ie = cudaGraphInstantiate(&ge, g, 0);
    if (ie != cudaSuccess) {
      cudaGraphDestroy(g);
      return fail(c, RKDG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
    }
    cudaError_t le = cudaGraphLaunch(ge, c->stream);
    cudaError_t se = cudaStreamSynchronize(c->stream);
    cudaGraphExecDestroy(ge);
    cudaGraphDestroy(g);
    if (le != cudaSuccess || se != cudaSuccess)
      return fail(c, RKDG_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(le != cudaSuccess ? le : se));
  } else {
    int nact = np;
    long long steps = 0;
    while (nact > 0) {
      st = fp32 ? enqueue_step32(c, 0.0, true) : enqueue_step64(c, x, 0.0, true);
      if (st) return st;
      CUDA_TRY(c, rkdg::launch_batch_control(bs, cudaGraphConditionalHandle(), 0, c->stream));
      c->launches++;
      if (per_step == 0) per_step = c->launches - l0;
      CUDA_TRY(c, cudaMemcpyAsync(c->h_err, c->d_nactive, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
      CUDA_TRY(c, cudaStreamSynchronize(c->stream));
      nact = c->h_err[0];
      if (++steps > 100000000LL) return fail(c, RKDG_ERR_INVALID, "batch run did not terminate");
    }
  }
  if (fp32) {
    CUDA_TRY(c, rkdg::launch_join(n, c->d_xh, c->d_xl, x, c->stream));
    c->launches++;
  }
  std::vector<int> steps(np), failed(np);
  std::vector<double> tt(np), sd(np);
  CUDA_TRY(c, cudaMemcpyAsync(steps.data(), c->d_psteps, np * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(failed.data(), c->d_pfail, np * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(tt.data(), c->d_pt, np * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(sd.data(), c->d_psum, np * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  st = read_mcs(c, 0, nullptr);
  if (st) return st;
  if (use_graph) {
    int mx = 0;
    for (int v : steps) mx = std::max(mx, v);
    c->launches = l0 + per_step * mx;
  }
  for (int p = 0; p < np; ++p) {
    if (steps_out) steps_out[p] = failed[p] ? -steps[p] : steps[p];
    if (t_out) t_out[p] = tt[p];
    if (sum_dt_out) sum_dt_out[p] = sd[p];
  }
  return RKDG_OK;
}

}  // extern "C"

// ---- discrete adjoint --------------------------------------------------------
namespace {

struct Adj {
  double *r, *ub, *zb, *acc, *w, *cross;
  double *kb[4], *z[4], *y[4], *k[4];
};

int adj_bufs(rkdg_ctx* c, Adj& A) {
  const size_t n = (size_t)c->ndofs * c->neq;
  const size_t nvec = 5 + 16;
  const size_t need = nvec * n + (size_t)4 * c->ne;  // + the limiter's min/max derivatives
  if (c->adj_n < need) {
    CUDA_TRY(c, dalloc(c->d_adj, need));
    c->adj_n = need;
  }
  double* p = c->d_adj;
  A.r = p; p += n;
  A.ub = p; p += n;
  A.zb = p; p += n;
  A.acc = p; p += n;
  A.w = p; p += n;
  for (int i = 0; i < 4; ++i) { A.kb[i] = p; p += n; }
  for (int i = 0; i < 4; ++i) { A.z[i] = p; p += n; }
  for (int i = 0; i < 4; ++i) { A.y[i] = p; p += n; }
  for (int i = 0; i < 4; ++i) { A.k[i] = p; p += n; }
  A.cross = p;
  return RKDG_OK;
}

int plain_rhs(rkdg_ctx* c, const double* in, double* out) {
  EpiParams<double> ep;
  std::memset(&ep, 0, sizeof ep);
  ep.mode = 0;
  ep.out64 = out;
  RhsParams P = rhs_params(c, 0, 0, 7);
  CUDA_TRY(c, launch_rhs_nc(c, 0, P, in, &ep));
  c->launches += rhs_kernels(c, P);
  return RKDG_OK;
}

int limit_in_place(rkdg_ctx* c, double* x) {
  if (!c->limiter_active()) return RKDG_OK;
  CUDA_TRY(c, rkdg::launch_means(c->geom, c->p, 0, c->ne, c->ndofs, c->d_tab, x, nullptr, c->d_means, c->stream));
  LimParams L = lim_params(c);
  CUDA_TRY(c, rkdg::launch_limit(c->geom, c->p, 0, L, x, nullptr, c->stream));
  c->launches += 2;
  return RKDG_OK;
}

// out = (df/dy)^T kbar
int rhs_t(rkdg_ctx* c, Adj& A, const double* y, const double* kbar, double* out) {
  CUDA_TRY(c, rkdg::launch_minv_apply(c->geom, c->p, c->ne, c->ndofs, c->d_tab, c->d_egeo64, kbar, A.r, c->stream));
  RhsParams P = rhs_params(c, 0, 0, 7);
  CUDA_TRY(c, rkdg::launch_rhs_vjp(c->geom, c->p, P, y, A.r, out, c->stream));
  if (c->nnc) {  // the hanging faces' share, added to u_bar
    CUDA_TRY(c, rkdg::launch_nc_vjp(c->geom, c->p, P, nc_params(c), y, A.r, out, c->stream));
    c->launches += 2;
  }
  c->launches += 2;
  return RKDG_OK;
}

// out = (dL/dz)^T ybar
int lim_t(rkdg_ctx* c, Adj& A, const double* z, const double* ybar, double* out) {
  const long long n = c->ndofs * c->neq;
  if (!c->limiter_active()) {
    CUDA_TRY(c, cudaMemcpyAsync(out, ybar, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    return RKDG_OK;
  }
  CUDA_TRY(c, rkdg::launch_means(c->geom, c->p, 0, c->ne, c->ndofs, c->d_tab, z, nullptr, c->d_means, c->stream));
  LimParams L = lim_params(c);
  CUDA_TRY(c, rkdg::launch_limit_vjp(c->geom, c->p, L, z, ybar, out, A.cross, c->stream));
  CUDA_TRY(c, rkdg::launch_limit_vjp_gather(c->geom, c->p, L, A.cross, out, c->stream));
  c->launches += 3;
  return RKDG_OK;
}

// Reverse of ExplicitRKLimitedSolver::Step at state x with step dt: xbar holds
// the adjoint of x_{n+1} on entry and of x_n on return.
int step_t(rkdg_ctx* c, Adj& A, const double* x, double dt, double* xbar) {
  const int s = c->s;
  const long long n = c->ndofs * c->neq;
  const size_t bytes = n * sizeof(double);
  int st;
  // forward recompute of the stage values
  if ((st = plain_rhs(c, x, A.k[0]))) return st;
  for (int i = 1; i < s; ++i) {
    const int row = i * (i - 1) / 2;
    CUDA_TRY(c, cudaMemcpyAsync(A.z[i], x, bytes, cudaMemcpyDeviceToDevice, c->stream));
    for (int j = 0; j < i; ++j) CUDA_TRY(c, rkdg::launch_axpy(n, c->a[row + j] * dt, A.k[j], A.z[i], c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(A.y[i], A.z[i], bytes, cudaMemcpyDeviceToDevice, c->stream));
    if ((st = limit_in_place(c, A.y[i]))) return st;
    if ((st = plain_rhs(c, A.y[i], A.k[i]))) return st;
  }
  CUDA_TRY(c, cudaMemcpyAsync(A.w, x, bytes, cudaMemcpyDeviceToDevice, c->stream));
  for (int j = 0; j < s; ++j) CUDA_TRY(c, rkdg::launch_axpy(n, c->b[j] * dt, A.k[j], A.w, c->stream));
  // reverse sweep
  if ((st = lim_t(c, A, A.w, xbar, A.acc))) return st;
  for (int j = 0; j < s; ++j) CUDA_TRY(c, rkdg::launch_scale_copy(n, c->b[j] * dt, A.acc, A.kb[j], c->stream));
  for (int i = s - 1; i >= 1; --i) {
    const int row = i * (i - 1) / 2;
    if ((st = rhs_t(c, A, A.y[i], A.kb[i], A.ub))) return st;
    if ((st = lim_t(c, A, A.z[i], A.ub, A.zb))) return st;
    CUDA_TRY(c, rkdg::launch_axpy(n, 1.0, A.zb, A.acc, c->stream));
    for (int j = 0; j < i; ++j) CUDA_TRY(c, rkdg::launch_axpy(n, c->a[row + j] * dt, A.zb, A.kb[j], c->stream));
  }
  if ((st = rhs_t(c, A, x, A.kb[0], A.ub))) return st;
  CUDA_TRY(c, rkdg::launch_axpy(n, 1.0, A.ub, A.acc, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(xbar, A.acc, bytes, cudaMemcpyDeviceToDevice, c->stream));
  return RKDG_OK;
}

int adjoint_ready(rkdg_ctx* c) {
  if (c->precision != RKDG_FP64)
    return fail(c, RKDG_ERR_UNSUPPORTED, "the discrete adjoint runs on the FP64 path");
  if (!rkdg::adjoint_supported(c->geom, c->p))
    return fail(c, RKDG_ERR_UNSUPPORTED, "no adjoint kernels for this element type / order");
  if (c->nprob > 0) return fail(c, RKDG_ERR_UNSUPPORTED, "no adjoint for batched problems");
  if ((c->quirks & RKDG_LIMITER_LINEARIZE) && c->limiter_active() && c->lim == RKDG_LIM_MULTI &&
      c->geom != RKDG_GEOM_TRIANGLE)
    return fail(c, RKDG_ERR_UNSUPPORTED, "no adjoint for the linearize limiter option");
  if (c->ind == RKDG_IND_SHU && c->limiter_active())
    return fail(c, RKDG_ERR_UNSUPPORTED, "no adjoint for the Shu indicator");
  return RKDG_OK;
}

}  // namespace

extern "C" {

int rkdg_rhs_vjp(rkdg_ctx* c, const double* x, const double* kbar, double* xbar) {
  NEED_MESH(c);
  int st = adjoint_ready(c);
  if (st) return st;
  if (!x || !kbar || !xbar) return fail(c, RKDG_ERR_INVALID, "null pointer");
  Adj A;
  if ((st = adj_bufs(c, A))) return st;
  if ((st = rhs_t(c, A, x, kbar, xbar))) return st;
  return read_mcs(c, 7, nullptr);
}

int rkdg_limit_vjp(rkdg_ctx* c, const double* z, const double* ybar, double* zbar) {
  NEED_MESH(c);
  int st = adjoint_ready(c);
  if (st) return st;
  if (!z || !ybar || !zbar) return fail(c, RKDG_ERR_INVALID, "null pointer");
  Adj A;
  if ((st = adj_bufs(c, A))) return st;
  if ((st = lim_t(c, A, z, ybar, zbar))) return st;
  return read_mcs(c, 7, nullptr);
}

int rkdg_step_vjp(rkdg_ctx* c, const double* x, double dt, double* xbar) {
  NEED_MESH(c);
  int st = adjoint_ready(c);
  if (st) return st;
  if (!x || !xbar) return fail(c, RKDG_ERR_INVALID, "null pointer");
  Adj A;
  if ((st = adj_bufs(c, A))) return st;
  if ((st = step_t(c, A, x, dt, xbar))) return st;
  return read_mcs(c, 7, nullptr);
}

int rkdg_adjoint_run(rkdg_ctx* c, const double* x0, int nsteps, double dt, int every,
                     double* xbar, double* xT) {
  NEED_MESH(c);
  int st = adjoint_ready(c);
  if (st) return st;
  if (!x0 || !xbar || nsteps <= 0 || !(dt > 0.0) || every <= 0)
    return fail(c, RKDG_ERR_INVALID, "invalid adjoint run arguments");
  if ((st = ensure_scratch(c))) return st;
  Adj A;
  if ((st = adj_bufs(c, A))) return st;
  const long long n = c->ndofs * c->neq;
  const size_t bytes = n * sizeof(double);
  const int ncp = (nsteps + every - 1) / every;
  double* store = nullptr;  // ncp checkpoints + `every` segment states
  if (cudaMalloc((void**)&store, (size_t)(ncp + every) * bytes) != cudaSuccess)
    return fail(c, RKDG_ERR_ALLOC, "adjoint checkpoint storage");
  auto cp = [&](int i) { return store + (size_t)i * n; };
  auto seg = [&](int i) { return store + (size_t)(ncp + i) * n; };
  int rc = RKDG_OK;
  do {
    // forward sweep storing a checkpoint every `every` steps
    double* x = seg(0);
    if (cudaMemcpyAsync(x, x0, bytes, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess) {
      rc = fail(c, RKDG_ERR_CUDA, "copy");
      break;
    }
    for (int s = 0; s < nsteps && !rc; ++s) {
      if (s % every == 0 &&
          cudaMemcpyAsync(cp(s / every), x, bytes, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess)
        rc = fail(c, RKDG_ERR_CUDA, "copy");
      if (!rc) rc = enqueue_step64(c, x, dt);
    }
    if (rc) break;
    if (xT && cudaMemcpyAsync(xT, x, bytes, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess) {
      rc = fail(c, RKDG_ERR_CUDA, "copy");
      break;
    }
    if ((rc = read_mcs(c, c->s - 1, nullptr))) break;
    // reverse sweep, segment by segment, recomputing the segment's states
    for (int g = ncp - 1; g >= 0 && !rc; --g) {
      const int s0 = g * every, len = std::min(every, nsteps - s0);
      if (cudaMemcpyAsync(seg(0), cp(g), bytes, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess) {
        rc = fail(c, RKDG_ERR_CUDA, "copy");
        break;
      }
      for (int j = 1; j < len && !rc; ++j) {
        if (cudaMemcpyAsync(seg(j), seg(j - 1), bytes, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess)
          rc = fail(c, RKDG_ERR_CUDA, "copy");
        if (!rc) rc = enqueue_step64(c, seg(j), dt);
      }
      for (int j = len - 1; j >= 0 && !rc; --j) rc = step_t(c, A, seg(j), dt, xbar);
      if (!rc) rc = read_mcs(c, 7, nullptr);
    }
  } while (false);
  cudaStreamSynchronize(c->stream);
  cudaFree(store);
  return rc;
}

long long rkdg_kernel_launches(rkdg_ctx* c) { return c ? c->launches : -1; }

// Autotuner: launches every candidate shape of the stage kernel (and of the
// limiter when one is active) on the caller's state, times them with CUDA
// events on the context's stream and keeps the fastest.  Candidates: the
// hexahedral kernel (warp per element with 8 elements per CTA, five-lane team
// with 24, or the team face pass + element pass) or, on triangles and quads,
// 64 / 128 / 256 elements per CTA.
int rkdg_autotune(rkdg_ctx* c, const double* x, int* hex_kernel, int* generic_block,
                  int* limiter_block) {
  NEED_MESH(c);
  if (!x) return fail(c, RKDG_ERR_INVALID, "null state pointer");
  int st = ensure_scratch(c);
  if (st) return st;
  const long long n = c->ndofs * c->neq;
  const int prec = c->precision == RKDG_FP64 ? 0 : 1;
  const void* in = x;
  if (prec) {
    CUDA_TRY(c, rkdg::launch_to_float(n, x, c->d_y32[0], c->stream));
    in = c->d_y32[0];
    c->launches++;
  }
  cudaEvent_t ev[2];
  CUDA_TRY(c, cudaEventCreate(&ev[0]));
  if (cudaEventCreate(&ev[1]) != cudaSuccess) {
    cudaEventDestroy(ev[0]);
    return fail(c, RKDG_ERR_CUDA, "cudaEventCreate failed");
  }
  struct Events {
    cudaEvent_t* e;
    ~Events() {
      cudaEventDestroy(e[0]);
      cudaEventDestroy(e[1]);
    }
  } guard{ev};
  constexpr int kWarm = 2, kReps = 5;
  // mean time of one right-hand-side launch (plain epilogue into scratch)
  auto time_rhs = [&](float* ms) -> int {
    EpiParams<double> ep64;
    EpiParams<float> ep32;
    std::memset(&ep64, 0, sizeof ep64);
    std::memset(&ep32, 0, sizeof ep32);
    ep64.out64 = ep32.out64 = c->d_y64[0];
    const void* ep = prec ? (const void*)&ep32 : (const void*)&ep64;
    const RhsParams P = rhs_params(c, prec, 0, 0);
    for (int r = 0; r < kWarm + kReps; ++r) {
      if (r == kWarm) CUDA_TRY(c, cudaEventRecord(ev[0], c->stream));
      CUDA_TRY(c, cudaMemsetAsync(c->d_mcs, 0, sizeof(unsigned long long), c->stream));
      CUDA_TRY(c, launch_rhs_nc(c, prec, P, in, ep));
      c->launches += rhs_kernels(c, P);
    }
    CUDA_TRY(c, cudaEventRecord(ev[1], c->stream));
    CUDA_TRY(c, cudaEventSynchronize(ev[1]));
    CUDA_TRY(c, cudaEventElapsedTime(ms, ev[0], ev[1]));
    *ms /= kReps;
    return read_mcs(c, 0, nullptr);  // reports a non-physical input state
  };
  if (c->geom == RKDG_GEOM_CUBE) {
    if ((st = ensure_fslot(c))) return st;
    int best = 0;
    float tbest = 0.0f;
    for (int v = 1; v <= 6; ++v) {
      if ((v == 4 && !c->d_hsched) || (v == 5 && !c->d_htile)) continue;
      if (v == 6 && !(c->d_htile && c->d_tcb && c->precision != RKDG_FP64)) continue;
      c->hex_variant = v;
      float ms = 0.0f;
      if ((st = time_rhs(&ms))) return st;
      if (best == 0 || ms < tbest) best = v, tbest = ms;
    }
    c->hex_variant = best;
    if (best != 3) {
      dfree(c->d_fslot);
      c->fslot_n = 0;
    }
  } else {
    int best = 0;
    float tbest = 0.0f;
    // the FP32 kernels of small elements (Q1 quads, P1 triangles) run at most
    // 128 threads per CTA (their launch bounds)
    const int bmax = (c->precision != RKDG_FP64 && c->neq * c->nd <= 16) ? 128 : 256;
    for (int b = 64; b <= bmax; b *= 2) {
      c->gen_block = b;
      float ms = 0.0f;
      if ((st = time_rhs(&ms))) return st;
      if (best == 0 || ms < tbest) best = b, tbest = ms;
    }
    c->gen_block = best;
  }
  if (c->limiter_active()) {
    // the limiter rewrites its input: time it on a scratch copy
    CUDA_TRY(c, rkdg::launch_means(c->geom, c->p, 0, c->ne, c->ndofs, c->d_tab, x, nullptr, c->d_means, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(c->d_y64[0], x, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    c->launches++;
    int best = 0;
    float tbest = 0.0f;
    const int bmax = (c->precision != RKDG_FP64 && c->neq * c->nd <= 16) ? 128 : 256;
    for (int b = 64; b <= bmax; b *= 2) {
      c->lim_block = b;
      const LimParams L = lim_params(c);
      for (int r = 0; r < kWarm + kReps; ++r) {
        if (r == kWarm) CUDA_TRY(c, cudaEventRecord(ev[0], c->stream));
        CUDA_TRY(c, rkdg::launch_limit(c->geom, c->p, 0, L, c->d_y64[0], nullptr, c->stream));
        c->launches++;
      }
      CUDA_TRY(c, cudaEventRecord(ev[1], c->stream));
      CUDA_TRY(c, cudaEventSynchronize(ev[1]));
      float ms = 0.0f;
      CUDA_TRY(c, cudaEventElapsedTime(&ms, ev[0], ev[1]));
      if (best == 0 || ms < tbest) best = b, tbest = ms;
    }
    c->lim_block = best;
  }
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (hex_kernel) *hex_kernel = c->hex_variant;
  if (generic_block) *generic_block = c->gen_block;
  if (limiter_block) *limiter_block = c->lim_block;
  return RKDG_OK;
}

// rkdg_limit with the cell means in the library's fixed device array: the
// means kernel writes all neq * NE entries before the limiter kernel reads
// them on the same stream, so nothing needs clearing first.
int rkdg_limit_static(rkdg_ctx* c, double* x) {
  NEED_MESH(c);
  if (!x) return fail(c, RKDG_ERR_INVALID, "null state pointer");
  const unsigned long long need = (unsigned long long)c->neq * (unsigned long long)c->ne;
  if (need > RKDG_LIMIT_STATIC_MAX_VALUES)
    return fail(c, RKDG_ERR_INVALID,
                "mesh too large for the fixed limiter scratch: neq * NE = " + std::to_string(need) +
                    " > " + std::to_string(RKDG_LIMIT_STATIC_MAX_VALUES));
  if (!c->limiter_active()) return RKDG_OK;
  double* means = nullptr;
  CUDA_TRY(c, rkdg::static_means_scratch(c->device, &means));
  CUDA_TRY(c, rkdg::launch_means(c->geom, c->p, 0, c->ne, c->ndofs, c->d_tab, x, nullptr, means, c->stream));
  LimParams L = lim_params(c);
  L.means = means;
  CUDA_TRY(c, rkdg::launch_limit(c->geom, c->p, 0, L, x, nullptr, c->stream));
  c->launches += 2;
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return RKDG_OK;
}

}  // extern "C"
