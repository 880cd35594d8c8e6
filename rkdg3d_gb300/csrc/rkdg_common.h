// Shared host/device declarations of the GB300 RKDG library: reference-element
// tables, device mesh tables and kernel parameter blocks.
#pragma once

#include <cstdint>

#if __has_include(<vector_types.h>)
#include <vector_types.h>
#else
// host-only tools built without the CUDA headers (same layout as CUDA's)
struct alignas(8) float2 {
  float x, y;
};
#endif

#define RKDG_MAX_ND 27    // hex Q2 = 27 nodes
#define RKDG_MAX_NFPE 6
#define RKDG_MAX_NQF 16   // hex Q2 face rule: 4x4
#define RKDG_MAX_NQL 4    // limiter face rule (order 2): 2 (segment) or 2x2
#define RKDG_MAX_NV 8
#define RKDG_MAX_PERM 64
#define RKDG_MAX_NQS 27   // Shu indicator rule (hex Q2: 3x3x3)
#define RKDG_HEX_MAX_PERM 8  // orientations of a square face
#define RKDG_MAX_BC 32

namespace rkdg {

// Element traits: compile-time sizes of the supported (geometry, order) pairs.
// Face rules follow the reference's DGTraceIntegrator order (face_integrator.cpp
// :45-58): OrderW + 2p, +1 on simplices; OrderW = 0 (triangle), 1 (bilinear
// quad), 2 (trilinear hex); a segment rule of order q has q/2+1 GL points.
template <int G, int P>
struct El;
template <int P>
struct El<2, P> {  // triangle
  static constexpr int DIM = 2, ND = (P + 1) * (P + 2) / 2, NFPE = 3, NQF = P + 1, NQL = 2,
                       NV = 3, NEQ = 4;
};
template <int P>
struct El<3, P> {  // quadrilateral
  static constexpr int DIM = 2, ND = (P + 1) * (P + 1), NFPE = 4, NQF = P + 1, NQL = 2, NV = 4,
                       NEQ = 4;
};
template <int P>
struct El<5, P> {  // hexahedron
  static constexpr int DIM = 3, ND = (P + 1) * (P + 1) * (P + 1), NFPE = 6,
                       NQF = (P + 2) * (P + 2), NQL = 4, NV = 8, NEQ = 5;
};

// Reference-element tables (built on the host in FP64, copied to the device).
struct RefTables {
  int dim, geom, p, nd, nfpe, nqf, nql, nv, nperm, n1, nq1;
  double D[3][RKDG_MAX_ND][RKDG_MAX_ND];     // D[r][j][m] = sum_q w phi_m d_r phi_j
  double Minv[RKDG_MAX_ND][RKDG_MAX_ND];     // reference inverse mass
  double B[RKDG_MAX_NFPE][RKDG_MAX_NQF][RKDG_MAX_ND];   // traces at face points
  double wf[RKDG_MAX_NQF];                   // face rule weights
  int perm[RKDG_MAX_PERM][RKDG_MAX_NQF];     // elem1 point -> elem2 point
  double Bl[RKDG_MAX_NFPE][RKDG_MAX_NQL][RKDG_MAX_ND];  // limiter face points
  double Bv[RKDG_MAX_NV][RKDG_MAX_ND];       // element vertices
  double wmean[RKDG_MAX_ND];                 // cell-mean weights (sum = 1)
  // 1D tables for the sum-factorised tensor kernels
  double l1d[RKDG_MAX_NQF][8];   // 1D basis at 1D face-rule points  [a][j]
  double w1d[8];                 // 1D face-rule weights
  double lend[2][8];             // 1D basis at 0 and 1
  double d1[8][8];               // d1[j][m] = w_m l_j'(x_m) (collocated volume)
  double minv1[8][8];            // 1D reference inverse mass (exact)
  double lquad[2][8];            // 1D basis at the 2 limiter GL points
  double w1[8];                  // 1D GL node weights
  // hexahedra: per local face, normal axis and side, and the tensor trace
  // weights B2[lf][q][i0*n1+i1] = l(a_q, i0) l(b_q, i1) on the face's two
  // tangential axes (ascending axis order)
  int fax[RKDG_MAX_NFPE], fside[RKDG_MAX_NFPE];
  double B2[RKDG_MAX_NFPE][RKDG_MAX_NQF][9];
  // canonical face point q -> tensor index a + nq1*b (a along the lower
  // tangential axis, b along the upper one)
  int fab[RKDG_MAX_NFPE][RKDG_MAX_NQF];
  // limiter "linearize" option (tensor elements, order 1): reference-space
  // gradients of the basis at the element centre and the points of the
  // element rule of order p+1
  double dcen[RKDG_MAX_ND][3];
  double xlin[RKDG_MAX_ND][3];
  int lin_ok;
  // Shu indicator: the element rule of order p + OrderW (the extrapolated
  // averages of averager.cpp:154-273) and what evaluating the nodal basis at
  // arbitrary reference points needs: the 1D GL nodes (tensor elements) or
  // the monomial expansion phi_j = sum_m tcoef[m][j] x^tmono[m][0] y^tmono[m][1]
  // (triangles)
  // non-parallelogram quadrilateral meshes: cell-mean weights of each
  // element [ne][nd] on the device (null when every element is affine and
  // wmean serves all)
  const double* wmn_e;
  // and their FP64 adj(J), 1/det J at every node, [dim*dim + 1][nd][ne]
  const double* ngeo_e;
  int nqs;
  double xs[RKDG_MAX_NQS][3];
  double ws[RKDG_MAX_NQS];
  double x1n[8];
  int tmono[RKDG_MAX_ND][2];
  double tcoef[RKDG_MAX_ND][RKDG_MAX_ND];
};

// Boundary condition slot.
struct BCSlot {
  int type;
  double state[5];
};

// 1D operators of the tensor-product hexahedral team kernels (order <= 2),
// passed by value inside the kernel parameters so that their entries are
// constant-bank operands of the arithmetic instead of shared-memory loads.
template <typename R>
struct HexOps {
  R l1d[12];   // [NQ1][N1] 1D basis at the face-rule points
  R lend[6];   // [2][N1]   1D basis at 0 and 1
  R d1[9];     // [N1][N1]  collocated derivative w_m l_j'(x_m)
  R minv1[9];  // [N1][N1]  1D inverse mass
  R w1[3];     // 1D node weights
  R wf[16];    // face-rule weights
};
struct HexOpsPair {
  HexOps<float> f;
  HexOps<double> d;
};

// Schedule of one CTA of the shared-face hexahedral team kernel: the CTA's
// 24 element slots (a compact group of elements in Morton order of their
// centres) and the rounds in which the slots visit their six faces.  A face
// whose two elements sit in the same CTA is visited by both in the same
// round and evaluated once; a face to an element outside the CTA needs that
// element's trace from global memory (a "job").
#define RKDG_TEAM_SLOTS 24
#define RKDG_TEAM_MAX_ROUNDS 8
struct HexTeamSched {
  int el[RKDG_TEAM_SLOTS];                                // element of each slot (-1: none)
  unsigned char rlf[RKDG_TEAM_SLOTS][RKDG_TEAM_MAX_ROUNDS];  // local face of round r (0xFF: none)
  unsigned char part[RKDG_TEAM_SLOTS][6];                 // slot across an in-CTA face (0xFF: none)
  // faces the CTA evaluates in round r, one word each: bits 0-4 slot, 5-7
  // its local face, 8-12 slot across an in-CTA face (31: none), 13 Elem2
  // side, 14-16 local face across, 17-19 point permutation id, 20 the face
  // has a neighbour element (0: boundary)
  unsigned int fd[RKDG_TEAM_MAX_ROUNDS][RKDG_TEAM_SLOTS];
  unsigned char jb[RKDG_TEAM_MAX_ROUNDS][RKDG_TEAM_SLOTS];   // slots with an out-of-CTA neighbour in round r
  unsigned char nfl[RKDG_TEAM_MAX_ROUNDS], njb[RKDG_TEAM_MAX_ROUNDS];
  // normal axis shared by every face visited in round r and by the faces
  // across them (-1: mixed; the kernel then branches per face)
  signed char rax[RKDG_TEAM_MAX_ROUNDS];
  int nr;                                                 // rounds used by this CTA
};

// Tile of the face-once hexahedral kernel (k_rhs_hex_tile): RKDG_TILE_E
// elements that are consecutive in the Morton order of their centres (on a
// structured 2^k mesh a 4 x 4 x 2 block).  Per normal axis a of the elements'
// local faces (0: faces 4/2, 1: faces 1/3, 2: faces 0/5) the tile lists the
// face evaluations of its face sides on that axis, each face once: a face
// between two tile elements whose local faces share the axis is evaluated by
// its Elem1 side; a face to an element outside the tile (or across axes) by
// the tile side, with the outside element's trace formed from global memory
// (a "halo"); a boundary face by its element with the boundary condition the
// context holds at launch time.  One word per evaluation:
//   bits 0-5 Elem1 side (face side 2*slot + s, or halo index), 6 Elem1 is a
//   halo, 7-12 Elem2 side (likewise), 13 Elem2 is a halo, 14 boundary face
//   (no Elem2), 15-17 Elem1's local face, 18-20 Elem2's local face, 21-23
//   point permutation id, 24 the face geometry is read at the Elem2 side.
#define RKDG_TILE_E 32
#define RKDG_TILE_HMAX 64  // = 2 * RKDG_TILE_E: every face side of a tile axis can be a halo
struct HexTile {
  int el[RKDG_TILE_E];                      // element of each slot (-1: none)
  int nel;                                  // slots in use
  int nev[3];                               // evaluations per axis
  int nh[3];                                // halo traces per axis
  unsigned int ev[3][2 * RKDG_TILE_E];      // evaluations (packed, see above)
  int hel[3][RKDG_TILE_HMAX];               // halo: element outside the tile
  unsigned char hlf[3][RKDG_TILE_HMAX];     // halo: its local face
};

// Per-element face table entry codes (fcode): bits 0-2 local face of the
// other element, bit 3 = 1 if this element is the face's Elem2, bits 4..
// permutation id.  fnbr: neighbour element id, -1 = boundary face with no
// boundary integrator, <= -2 : boundary condition slot (-2 - fnbr).
struct RhsParams {
  int ne;
  long long ndofs;
  const int* fnbr;      // [nfpe][ne]
  const int* fcode;     // [nfpe][ne]
  const void* fgeo;     // [nfpe][dim+1][ne] elem1-outward unit normal, |J_f|
  const void* egeo;     // [dim*dim+1][ne]   adj(J) (row r, col d), 1/det J
  const RefTables* tab;
  double gamma, covolume;
  double rgas;          // specific gas constant (subsonic inlet / outlet BCs)
  int rs, avg;
  int faces_only;       // 1: face terms only (A.Mult for the initial dt)
  int quirks;           // bit 0: negative HLLC speed is not an error
  BCSlot bc[RKDG_MAX_BC];
  unsigned long long* mcs;  // atomicMax target, bits of a non-negative double
  int* err;                 // [0] status (first writer wins), [1] element
  // batched independent problems (null when the context holds one problem):
  // element -> problem, per-problem EoS constants, active flags and one
  // max-speed slot per problem
  const int* prob;
  const double* pgamma;
  const double* pcov;
  const float* pgamma32;  // the same constants rounded to FP32 (the FP32 kernels)
  const float* pcov32;
  const int* pactive;
  unsigned long long* pmcs;
  int* pfail;           // per-problem failure flag (non-physical state)
  // batched problems, map of the active work (null: every element is
  // launched and idle problems' elements exit): the active problems in
  // order (act_pid[0 .. *act_n)), the exclusive prefix sums of their element
  // counts (act_cum[0 .. *act_n]) and the problems' element offsets
  const int* act_cum;
  const int* act_pid;
  const int* act_n;
  const int* poff;
  int block;            // threads per CTA of the generic kernels (0: default)
  void* fslot;          // hexahedral face-pass flux slots [ne][6][neq][nqf] (or null)
  const HexTeamSched* hsched;  // shared-face hexahedral kernel: one entry per CTA (or null)
  const HexTile* htile;        // face-once tiled hexahedral kernel: one entry per CTA (or null)
  int ntile;
  int tile_hs;                 // its halo-buffer stride: the largest halo list, odd
  // tensor-core variant of the tile kernel (Q2): the volume operator of each
  // direction as a dense 32 x 32 TF32 pair (hi, lo) in the K-major core-matrix
  // layout, [3][2][1024] floats (or null)
  const float* tcb;
  // nonconforming meshes: element -> row of xface (-1: none) and the face
  // terms of the hanging faces, [row][neq][nd] in the kernel's precision,
  // added to the element's face + volume terms before the inverse mass
  const int* ncidx;
  const void* xface;
  // non-parallelogram quadrilaterals: adj(J) and 1/det J at every node,
  // [dim*dim + 1][nd][ne] in the kernel's precision (null: egeo per element)
  const void* ngeo;
  HexOpsPair hops;      // hexahedra (order <= 2): 1D operators
};

// Hanging (nonconforming) faces of an adapted mesh.  Each slave face is
// integrated from its fine element (Elem1, the face's own points and normal)
// against the master face's coarse element (Elem2), evaluated at the slave
// points mapped into it; master faces carry no integrator of their own.
struct NcParams {
  int nnc, nqf, nd, neq, nel;
  const int* face;      // [nnc][4]: fine element, its local face, coarse element, its face
  const double* bnc;    // [nnc][nqf][nd]: coarse element's basis at the mapped points
  void* flux;           // [nnc][2][neq][nd]: each face's term for its fine and coarse element
  const int* elem;      // [nel] elements with hanging-face terms
  const int* ptr;       // [nel + 1] CSR rows of ent
  const int* ent;       // 2 * slave face + side (0: fine, 1: coarse)
  void* xface;          // [nel][neq][nd] (kernel precision)
};

// Stage epilogue.
// mode 0: write the plain right-hand side y = k (FP64) to out64.
// mode 1: Runge-Kutta combination  out = base + sum_j cprev[j] kprev[j] + ccur k.
//   FP64 path: base/out64 are double; out32 optionally receives a float copy.
//   FP32-bulk path: the conserved state is a float pair (hi, lo) (basehi,
//   baselo); an intermediate stage writes its combination as float to out32
//   (the next stage input), the final stage (final_stage = 1) updates (hi, lo)
//   in double-single arithmetic (out32 = hi, outlo = lo).
// kout (optional) stores k itself for later stages; means (optional) receives
// the FP64 cell means of the result [neq][ne].
template <typename R>
struct EpiParams {
  int mode;
  int final_stage;
  int nprev;
  double* out64;
  float* out32;
  float* outlo;
  R* kout;
  const double* base;
  const float* basehi;
  const float* baselo;
  const R* kprev[3];
  double cprev[3];
  float cprev_hi[3], cprev_lo[3];
  double ccur;
  float ccur_hi, ccur_lo;
  double* means;
  // cell means of the FP32-bulk path as float pairs (hi, lo) whose sum is
  // the mean; written instead of `means` when set
  float2* means32;
  // batched problems: when pdt is set, cprev/ccur hold the unscaled tableau
  // coefficients and are multiplied by the problem's dt (pdt[prob[e]])
  const int* prob;
  const double* pdt;
  const float2* pdt2;  // pdt as float pairs (hi, lo), read by the FP32 kernels
};

#ifdef __CUDACC__
// Store one cell mean: as a double, or as a normalised float pair (hi, lo)
// where the FP32-bulk path asked for pairs.
template <typename R>
__device__ __forceinline__ void store_mean(const EpiParams<R>& ep, long long i, double m) {
  if (ep.means32) {
    const float h = (float)m;
    ep.means32[i] = make_float2(h, (float)(m - (double)h));
  } else {
    ep.means[i] = m;
  }
}
#endif

struct LimParams {
  int ne;
  long long ndofs;
  const int* fnbr;
  const RefTables* tab;
  const double* eaff;   // [dim*dim + dim][ne]: J (row i, col r) and vertex 0
  const double* means;  // [neq][ne]
  // the FP32-bulk limiter's means: float pairs (the RHS epilogue's output)
  const float2* means32;  // [neq][ne]
  double gamma, covolume;
  int limiter, indicator, function, last_hope, quirks;
  const int* prob;      // batched problems (or null)
  const double* pgamma;
  const double* pcov;
  const float* pgamma32;  // the same constants rounded to FP32 (the FP32 kernels)
  const float* pcov32;
  const int* pactive;
  const int* act_cum;   // map of the active work (as RhsParams; or null)
  const int* act_pid;
  const int* act_n;
  const int* poff;
  int block;            // threads per CTA (0: default)
  // hanging faces (nonconforming meshes; null otherwise): element -> CSR row
  // of its slave-face entries (2 * face + side) and the faces [nnc][4]
  const int* ncidx;
  const int* nc_ptr;
  const int* nc_ent;
  const int* nc_face;
};

// Device-side time control of batched problems (one entry per problem).
struct BatchState {
  double t_end, cfl, denom;
  int nprob, dt_mode, max_steps;
  const double* hmin;   // [nprob]
  double* dt;           // [nprob] dt of the reference bookkeeping
  double* dtr;          // [nprob] dt_real used by the current step
  float2* dtr2;         // [nprob] the same as float pairs (hi, lo)
  double* t;            // [nprob]
  double* sum_dt;       // [nprob]
  int* active;          // [nprob]
  int* steps;           // [nprob]
  int* nactive;         // [1]
  const unsigned long long* mcs_last;  // [nprob] max speed of the last stage
  int* fail;            // [nprob] set by the kernels on a non-physical state
  // map of the active work, rebuilt after every step (see RhsParams)
  int* act_cum;         // [nprob + 1]
  int* act_pid;         // [nprob]
  int* act_n;           // [1]
  const int* poff;      // [nprob + 1] element offsets
};

}  // namespace rkdg
