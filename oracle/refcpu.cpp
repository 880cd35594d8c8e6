// refcpu — CPU FP64 oracle for the RKDG3D explicit DG hot path.
//
// TEST INFRASTRUCTURE ONLY (the parity checker and the timed CPU baseline).
// The product library never links or loads this file.  PARITY UNPINNED: see
// refcpu.h.  Each function cites the reference file:line it restates.
//
// Build: oracle/Makefile (g++ -O3 -ffp-contract=off -fopenmp, no -march).
#include "refcpu.h"

#include <omp.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// MFEM semantics restated: 1D Gauss-Legendre points on [0,1] (ascending), as
// used by Poly_1D::OpenPoints(p, GaussLegendre) and the segment rules.
// ---------------------------------------------------------------------------
void gauss_legendre01(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  for (int i = 0; i < n; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5));
    double p0 = 1.0, p1 = 0.0, pp = 1.0;
    for (int it = 0; it < 100; ++it) {
      p0 = 1.0;
      p1 = 0.0;
      for (int k = 1; k <= n; ++k) {
        double p2 = p1;
        p1 = p0;
        p0 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p2) / k;
      }
      pp = n * (z * p0 - p1) / (z * z - 1.0);
      double dz = p0 / pp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    p0 = 1.0;
    p1 = 0.0;
    for (int k = 1; k <= n; ++k) {
      double p2 = p1;
      p1 = p0;
      p0 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p2) / k;
    }
    pp = n * (z * p0 - p1) / (z * z - 1.0);
    x[i] = 0.5 * (1.0 - z);
    w[i] = 1.0 / ((1.0 - z * z) * pp * pp);
  }
  if (n == 1) {
    x[0] = 0.5;
    w[0] = 1.0;
  }
}

struct Lagrange1D {
  std::vector<double> x;
  void eval(double y, double* u) const {
    const int n = (int)x.size();
    for (int i = 0; i < n; ++i) {
      double v = 1.0;
      for (int j = 0; j < n; ++j)
        if (j != i) v *= (y - x[j]) / (x[i] - x[j]);
      u[i] = v;
    }
  }
  void deval(double y, double* du) const {
    const int n = (int)x.size();
    for (int i = 0; i < n; ++i) {
      double s = 0.0;
      for (int m = 0; m < n; ++m) {
        if (m == i) continue;
        double v = 1.0 / (x[i] - x[m]);
        for (int j = 0; j < n; ++j)
          if (j != i && j != m) v *= (y - x[j]) / (x[i] - x[j]);
        s += v;
      }
      du[i] = s;
    }
  }
};

// Small dense inverse with partial pivoting (MFEM DenseMatrixInverse: LU).
bool invert(int n, const std::vector<double>& A, std::vector<double>& Ai) {
  std::vector<double> M(A);
  Ai.assign(n * n, 0.0);
  for (int i = 0; i < n; ++i) Ai[i * n + i] = 1.0;
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(M[r * n + c]) > std::fabs(M[piv * n + c])) piv = r;
    if (M[piv * n + c] == 0.0) return false;
    if (piv != c)
      for (int k = 0; k < n; ++k) {
        std::swap(M[piv * n + k], M[c * n + k]);
        std::swap(Ai[piv * n + k], Ai[c * n + k]);
      }
    double d = M[c * n + c];
    for (int k = 0; k < n; ++k) {
      M[c * n + k] /= d;
      Ai[c * n + k] /= d;
    }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      double f = M[r * n + c];
      if (f == 0.0) continue;
      for (int k = 0; k < n; ++k) {
        M[r * n + k] -= f * M[c * n + k];
        Ai[r * n + k] -= f * Ai[c * n + k];
      }
    }
  }
  return true;
}

// ---------------------------------------------------------------------------
// Reference elements: MFEM DG_FECollection(p, dim) with its default
// Gauss-Legendre nodal basis (main.cpp:115).  Quads/hexes: tensor products of
// 1D Lagrange polynomials at GL points, node j = jx + n1*(jy + n1*jz).
// Triangles: L2_TriangleElement nodes (op[i]/w, op[j]/w), w = op[i]+op[j]+
// op[p-i-j], loops j outer, i inner.
// ---------------------------------------------------------------------------
struct FE {
  int geom = 0, dim = 0, p = 0, nd = 0, n1 = 0;
  std::vector<double> nodes;  // nd*dim
  Lagrange1D l1;
  std::vector<int> mono;      // triangle monomial exponents (a,b)
  std::vector<double> coef;   // triangle: coef[m*nd + j]

  void init(int g, int order) {
    geom = g;
    p = order;
    if (g == REF_GEOM_TRIANGLE) {
      dim = 2;
      nd = (p + 1) * (p + 2) / 2;
      std::vector<double> op, ow;
      gauss_legendre01(p + 1, op, ow);
      nodes.clear();
      for (int j = 0; j <= p; ++j)
        for (int i = 0; i + j <= p; ++i) {
          double w = op[i] + op[j] + op[p - i - j];
          nodes.push_back(op[i] / w);
          nodes.push_back(op[j] / w);
        }
      mono.clear();
      for (int b = 0; b <= p; ++b)
        for (int a = 0; a + b <= p; ++a) {
          mono.push_back(a);
          mono.push_back(b);
        }
      std::vector<double> V(nd * nd);
      for (int n = 0; n < nd; ++n)
        for (int m = 0; m < nd; ++m)
          V[n * nd + m] = std::pow(nodes[2 * n], mono[2 * m]) *
                          std::pow(nodes[2 * n + 1], mono[2 * m + 1]);
      invert(nd, V, coef);
    } else {
      dim = (g == REF_GEOM_SQUARE) ? 2 : 3;
      n1 = p + 1;
      std::vector<double> w;
      gauss_legendre01(n1, l1.x, w);
      nd = (dim == 2) ? n1 * n1 : n1 * n1 * n1;
      nodes.assign(nd * dim, 0.0);
      for (int j = 0; j < nd; ++j) {
        int jx = j % n1, jy = (j / n1) % n1, jz = j / (n1 * n1);
        nodes[j * dim + 0] = l1.x[jx];
        nodes[j * dim + 1] = l1.x[jy];
        if (dim == 3) nodes[j * dim + 2] = l1.x[jz];
      }
    }
  }
  void shape(const double* xi, double* phi) const {
    if (geom == REF_GEOM_TRIANGLE) {
      for (int j = 0; j < nd; ++j) phi[j] = 0.0;
      for (int m = 0; m < nd; ++m) {
        double mv = std::pow(xi[0], mono[2 * m]) * std::pow(xi[1], mono[2 * m + 1]);
        for (int j = 0; j < nd; ++j) phi[j] += coef[m * nd + j] * mv;
      }
      return;
    }
    double a[8], b[8], c[8];
    l1.eval(xi[0], a);
    l1.eval(xi[1], b);
    if (dim == 3) l1.eval(xi[2], c);
    for (int j = 0; j < nd; ++j) {
      int jx = j % n1, jy = (j / n1) % n1, jz = j / (n1 * n1);
      phi[j] = a[jx] * b[jy] * (dim == 3 ? c[jz] : 1.0);
    }
  }
  // dphi[j*dim + r] = d phi_j / d xi_r
  void dshape(const double* xi, double* dphi) const {
    if (geom == REF_GEOM_TRIANGLE) {
      for (int j = 0; j < nd * 2; ++j) dphi[j] = 0.0;
      for (int m = 0; m < nd; ++m) {
        int a = mono[2 * m], b = mono[2 * m + 1];
        double dx = a > 0 ? a * std::pow(xi[0], a - 1) * std::pow(xi[1], b) : 0.0;
        double dy = b > 0 ? b * std::pow(xi[0], a) * std::pow(xi[1], b - 1) : 0.0;
        for (int j = 0; j < nd; ++j) {
          dphi[j * 2 + 0] += coef[m * nd + j] * dx;
          dphi[j * 2 + 1] += coef[m * nd + j] * dy;
        }
      }
      return;
    }
    double a[8], b[8], c[8], da[8], db[8], dc[8];
    l1.eval(xi[0], a);
    l1.eval(xi[1], b);
    l1.deval(xi[0], da);
    l1.deval(xi[1], db);
    if (dim == 3) {
      l1.eval(xi[2], c);
      l1.deval(xi[2], dc);
    }
    for (int j = 0; j < nd; ++j) {
      int jx = j % n1, jy = (j / n1) % n1, jz = j / (n1 * n1);
      if (dim == 2) {
        dphi[j * 2 + 0] = da[jx] * b[jy];
        dphi[j * 2 + 1] = a[jx] * db[jy];
      } else {
        dphi[j * 3 + 0] = da[jx] * b[jy] * c[jz];
        dphi[j * 3 + 1] = a[jx] * db[jy] * c[jz];
        dphi[j * 3 + 2] = a[jx] * b[jy] * dc[jz];
      }
    }
  }
};

// ---------------------------------------------------------------------------
// Quadrature (MFEM IntRules.Get semantics): segment order q -> q/2+1 GL
// points; square/cube: tensor products of the segment rule of the same order.
// Triangles: a collapsed-coordinate Gauss product rule exact to degree q.
// Every triangle integrand on this path is a polynomial on an affine element
// integrated by a rule exact for its degree, so the values equal those of
// MFEM's own triangle rules up to rounding.
// ---------------------------------------------------------------------------
struct Rule {
  int n = 0, dim = 0;
  std::vector<double> x, w;
};
Rule rule_segment(int q) {
  Rule r;
  r.dim = 1;
  r.n = q / 2 + 1;
  gauss_legendre01(r.n, r.x, r.w);
  return r;
}
Rule rule_square(int q) {
  Rule s = rule_segment(q), r;
  r.dim = 2;
  r.n = s.n * s.n;
  for (int j = 0; j < s.n; ++j)
    for (int i = 0; i < s.n; ++i) {
      r.x.push_back(s.x[i]);
      r.x.push_back(s.x[j]);
      r.w.push_back(s.w[i] * s.w[j]);
    }
  return r;
}
Rule rule_cube(int q) {
  Rule s = rule_segment(q), r;
  r.dim = 3;
  r.n = s.n * s.n * s.n;
  for (int k = 0; k < s.n; ++k)
    for (int j = 0; j < s.n; ++j)
      for (int i = 0; i < s.n; ++i) {
        r.x.push_back(s.x[i]);
        r.x.push_back(s.x[j]);
        r.x.push_back(s.x[k]);
        r.w.push_back(s.w[i] * s.w[j] * s.w[k]);
      }
  return r;
}
Rule rule_triangle(int q) {
  int n = q / 2 + 2;
  std::vector<double> gx, gw;
  gauss_legendre01(n, gx, gw);
  Rule r;
  r.dim = 2;
  r.n = n * n;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double u = gx[i], v = gx[j];
      r.x.push_back(u);
      r.x.push_back(v * (1.0 - u));
      r.w.push_back(gw[i] * gw[j] * (1.0 - u));
    }
  return r;
}
Rule rule_geom(int geom, int q) {
  if (geom == REF_GEOM_TRIANGLE) return rule_triangle(q);
  if (geom == REF_GEOM_SQUARE) return rule_square(q);
  return rule_cube(q);
}

// MFEM reference vertices and local face (edge) vertex lists.
const double kTriVerts[3][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}};
const double kSqVerts[4][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}};
const double kCubeVerts[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                 {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
const int kTriEdges[3][2] = {{0, 1}, {1, 2}, {2, 0}};
const int kSqEdges[4][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};
const int kCubeFaces[6][4] = {{3, 2, 1, 0}, {0, 1, 5, 4}, {1, 2, 6, 5},
                              {2, 3, 7, 6}, {3, 0, 4, 7}, {4, 5, 6, 7}};

const double* ref_vertex(int geom, int v) {
  if (geom == REF_GEOM_TRIANGLE) return kTriVerts[v];
  if (geom == REF_GEOM_SQUARE) return kSqVerts[v];
  return kCubeVerts[v];
}
int local_face_vertex(int geom, int lf, int k) {
  if (geom == REF_GEOM_TRIANGLE) return kTriEdges[lf][k];
  if (geom == REF_GEOM_SQUARE) return kSqEdges[lf][k];
  return kCubeFaces[lf][k];
}

// Geometric (vertex) shape functions of the element map.
void geom_shape(int geom, const double* xi, double* N, double* dN /*nv*dim*/) {
  double x = xi[0], y = xi[1];
  if (geom == REF_GEOM_TRIANGLE) {
    N[0] = 1 - x - y; N[1] = x; N[2] = y;
    dN[0] = -1; dN[1] = -1; dN[2] = 1; dN[3] = 0; dN[4] = 0; dN[5] = 1;
  } else if (geom == REF_GEOM_SQUARE) {
    N[0] = (1 - x) * (1 - y); N[1] = x * (1 - y); N[2] = x * y; N[3] = (1 - x) * y;
    dN[0] = -(1 - y); dN[1] = -(1 - x);
    dN[2] = (1 - y);  dN[3] = -x;
    dN[4] = y;        dN[5] = x;
    dN[6] = -y;       dN[7] = (1 - x);
  } else {
    double z = xi[2];
    for (int v = 0; v < 8; ++v) {
      const double* r = kCubeVerts[v];
      double fx = r[0] ? x : 1 - x, fy = r[1] ? y : 1 - y, fz = r[2] ? z : 1 - z;
      double gx = r[0] ? 1 : -1, gy = r[1] ? 1 : -1, gz = r[2] ? 1 : -1;
      N[v] = fx * fy * fz;
      dN[v * 3 + 0] = gx * fy * fz;
      dN[v * 3 + 1] = fx * gy * fz;
      dN[v * 3 + 2] = fx * fy * gz;
    }
  }
}
// Face (dim-1) vertex shape functions: segment (a,b) or square (a,b,c,d).
void face_shape(int nvf, const double* s, double* N, double* dN) {
  if (nvf == 2) {
    N[0] = 1 - s[0]; N[1] = s[0];
    dN[0] = -1; dN[1] = 1;
  } else {
    double x = s[0], y = s[1];
    N[0] = (1 - x) * (1 - y); N[1] = x * (1 - y); N[2] = x * y; N[3] = (1 - x) * y;
    dN[0] = -(1 - y); dN[1] = -(1 - x);
    dN[2] = (1 - y);  dN[3] = -x;
    dN[4] = y;        dN[5] = x;
    dN[6] = -y;       dN[7] = (1 - x);
  }
}

// ---------------------------------------------------------------------------
// Physics (src/physics/physics.cpp)
// ---------------------------------------------------------------------------
struct Phys {
  int dim = 2, neq = 4;
  double gamma = 1.4, b = 0.0, R = 1.0;
};

// ComputePressure, physics.cpp:101-112
inline double pressure(const Phys& P, const double* s) {
  const double den = s[0];
  double v2 = 0;
  for (int d = 0; d < P.dim; d++) v2 += s[1 + d] * s[1 + d];
  v2 /= den;
  return (P.gamma - 1.0) * (s[1 + P.dim] - 0.5 * v2) / (1.0 - den * P.b);
}
// ComputeSoundSpeed, physics.cpp:134-140
inline double sound_speed(const Phys& P, const double* s) {
  const double den = s[0];
  const double p = pressure(P, s);
  return std::sqrt(P.gamma * p / den / (1.0 - den * P.b));
}
// StateIsPhysical, physics.cpp:6-50 (covolume-aware pressure)
inline bool state_is_physical(const Phys& P, const double* s) {
  const double den = s[0];
  const double e = s[1 + P.dim];
  if (den < 0 || den != den) return false;
  if (e <= 0 || e != e) return false;
  const double pres = pressure(P, s);
  if (pres <= 0 || pres != pres) return false;
  return true;
}
// StateIsPhysicalSay, physics.cpp:53-97 (perfect-gas pressure, quirk Q10)
inline bool state_is_physical_say(const Phys& P, const double* s) {
  const double den = s[0];
  const double e = s[1 + P.dim];
  if (den < 0 || den != den) return false;
  if (e <= 0 || e != e) return false;
  double v2 = 0;
  for (int i = 0; i < P.dim; i++) v2 += s[1 + i] * s[1 + i];
  v2 /= den;
  const double pres = (P.gamma - 1.0) * (e - 0.5 * v2);
  if (pres <= 0 || pres != pres) return false;
  return true;
}
// ComputeFlux, physics.cpp:143-168; F[k*dim + d] = flux(k, d)
inline void flux_full(const Phys& P, const double* s, double* F) {
  const int dim = P.dim;
  const double den = s[0];
  const double pres = pressure(P, s);
  for (int d = 0; d < dim; d++) {
    F[0 * dim + d] = s[1 + d];
    for (int i = 0; i < dim; i++) F[(1 + i) * dim + d] = s[1 + i] * s[1 + d] / den;
    F[(1 + d) * dim + d] += pres;
  }
  const double H = (s[1 + dim] + pres) / den;
  for (int d = 0; d < dim; d++) F[(1 + dim) * dim + d] = s[1 + d] * H;
}
// ComputeFluxDotN, physics.cpp:171-195
inline void flux_dot_n(const Phys& P, const double* s, const double* nor, double* fn) {
  const int dim = P.dim;
  const double den = s[0];
  const double pres = pressure(P, s);
  double dvn = 0;
  for (int d = 0; d < dim; d++) dvn += s[1 + d] * nor[d];
  fn[0] = dvn;
  for (int d = 0; d < dim; d++) fn[1 + d] = dvn * s[1 + d] / den + pres * nor[d];
  const double H = (s[1 + dim] + pres) / den;
  fn[1 + dim] = dvn * H;
}
// ComputeFluxF, physics.cpp:198-231 (x-flux of a rotated state)
inline void flux_F(const Phys& P, const double* s, double* f) {
  const int dim = P.dim;
  const double pres = pressure(P, s);
  f[0] = s[1];
  f[1] = s[1] * s[1] / s[0] + pres;
  for (int d = 1; d < dim; d++) f[d + 1] = s[1] * s[d + 1] / s[0];
  const double H = (s[1 + dim] + pres) / s[0];
  f[1 + dim] = s[1] * H;
}
// ComputeMaxCharSpeed, physics.cpp:252-266
inline double max_char_speed_of(const Phys& P, const double* s) {
  const double den = s[0];
  double v2 = 0;
  for (int d = 0; d < P.dim; d++) v2 += s[1 + d] * s[1 + d];
  v2 /= den;
  const double sound = sound_speed(P, s);
  const double vel = std::sqrt(v2 / den);
  return vel + sound;
}
inline double sqr(double x) { return x * x; }
// ComputeEinfeldtCharSpeeds, physics.cpp:269-296
inline void einfeldt_speeds(const Phys& P, const double* s1, const double* s2, double* lam) {
  const int dim = P.dim;
  double cL = sound_speed(P, s1), cR = sound_speed(P, s2);
  double ruL = s1[1], ruR = s2[1];
  double uL = ruL / s1[0], uR = ruR / s2[0];
  double sL = std::sqrt(s1[0]), sR = std::sqrt(s2[0]);
  double sum = sL + sR;
  double eta2 = 0.5 * sL * sR / sqr(sL + sR);
  double u_av = (ruL / sL + ruR / sR) / sum;
  double c_av = std::sqrt((sL * sqr(cL) + sR * sqr(cR)) / sum + eta2 * sqr(uR - uL));
  lam[0] = u_av - c_av;
  lam[dim + 1] = u_av + c_av;
  for (int i = 1; i < dim + 1; ++i) lam[i] = u_av;
}
// ComputeToroCharSpeeds (TRRS), physics.cpp:309-350
inline void toro_speeds(const Phys& P, const double* s1, const double* s2, double* lam) {
  const int dim = P.dim;
  const double g = P.gamma;
  double cL = sound_speed(P, s1), cR = sound_speed(P, s2);
  double uL = s1[1] / s1[0], uR = s2[1] / s2[0];
  double pL = pressure(P, s1), pR = pressure(P, s2);
  double z = 0.5 * (g - 1.0) / g;
  double pStar = std::pow((cL + cR - 0.5 * (g - 1.0) * (uR - uL)) /
                              (cL / std::pow(pL, z) + cR / std::pow(pR, z)),
                          1.0 / z);
  double qL = pStar > pL ? std::sqrt(1.0 + 0.5 * (g + 1.0) * (pStar / pL - 1.0) / g) : 1.0;
  double qR = pStar > pR ? std::sqrt(1.0 + 0.5 * (g + 1.0) * (pStar / pR - 1.0) / g) : 1.0;
  lam[0] = uL - qL * cL;
  lam[dim + 1] = uR + qR * cR;
  for (int i = 1; i < dim + 1; ++i) lam[i] = uL;
}

// RiemannSolver::Rotate / InverseRotate, rs_basic.cpp:11-67 (quirk Q14)
inline void rotate(int dim, double* s, const double* nor) {
  double* m = s + 1;
  if (dim == 2) {
    double mx = nor[0] * m[0] + nor[1] * m[1];
    double my = -nor[1] * m[0] + nor[0] * m[1];
    m[0] = mx;
    m[1] = my;
  } else {
    const double sinPsi = nor[2];
    const double cosPsi = std::sqrt(1 - sinPsi * sinPsi);
    const double sinTheta = std::fabs(cosPsi) > 1e-6 ? nor[1] / cosPsi : 1.0;
    const double cosTheta = std::fabs(cosPsi) > 1e-6 ? nor[0] / cosPsi : 0.0;
    double mx = cosPsi * cosTheta * m[0] + cosPsi * sinTheta * m[1] + sinPsi * m[2];
    double my = -sinTheta * m[0] + cosTheta * m[1];
    double mz = -sinPsi * cosTheta * m[0] - sinPsi * sinTheta * m[1] + cosPsi * m[2];
    m[0] = mx;
    m[1] = my;
    m[2] = mz;
  }
}
inline void inverse_rotate(int dim, double* s, const double* nor) {
  double* m = s + 1;
  if (dim == 2) {
    double mx = nor[0] * m[0] - nor[1] * m[1];
    double my = nor[1] * m[0] + nor[0] * m[1];
    m[0] = mx;
    m[1] = my;
  } else {
    const double sinPsi = nor[2];
    const double cosPsi = std::sqrt(1 - sinPsi * sinPsi);
    const double sinTheta = std::fabs(cosPsi) > 1e-6 ? nor[1] / cosPsi : 1.0;
    const double cosTheta = std::fabs(cosPsi) > 1e-6 ? nor[0] / cosPsi : 0.0;
    double mx = cosPsi * cosTheta * m[0] - sinTheta * m[1] - sinPsi * cosTheta * m[2];
    double my = cosPsi * sinTheta * m[0] + cosTheta * m[1] - sinPsi * sinTheta * m[2];
    double mz = sinPsi * m[0] + cosPsi * m[2];
    m[0] = mx;
    m[1] = my;
    m[2] = mz;
  }
}

// RiemannSolver*::Eval.  s1, s2 are working copies (the reference rotates its
// "const" inputs in place through const_cast).  Returns the wave speed or -1.
double rs_eval(const Phys& P, int rs, int avg, double* s1, double* s2, const double* nor,
               double* flux) {
  const int dim = P.dim, neq = P.neq;
  double f1[5], f2[5], lam[5];
  if (rs == 0) {  // Rusanov, rs_rusanov.cpp:6-40
    if (!state_is_physical_say(P, s1)) return -1;
    if (!state_is_physical_say(P, s2)) return -1;
    const double maxE1 = max_char_speed_of(P, s1);
    const double maxE2 = max_char_speed_of(P, s2);
    const double maxE = std::max(maxE1, maxE2);
    flux_dot_n(P, s1, nor, f1);
    flux_dot_n(P, s2, nor, f2);
    double normag = 0;
    for (int i = 0; i < dim; i++) normag += nor[i] * nor[i];
    normag = std::sqrt(normag);
    for (int i = 0; i < neq; i++)
      flux[i] = 0.5 * (f1[i] + f2[i]) / normag - 0.5 * maxE * (s2[i] - s1[i]);
    return maxE;
  }
  if (!state_is_physical_say(P, s1)) return -1;
  if (!state_is_physical_say(P, s2)) return -1;
  rotate(dim, s1, nor);
  rotate(dim, s2, nor);
  flux_F(P, s1, f1);
  flux_F(P, s2, f2);
  if (avg == 1)
    einfeldt_speeds(P, s1, s2, lam);
  else
    toro_speeds(P, s1, s2, lam);
  double ret;
  if (rs == 1) {  // LLF, rs_llf.cpp:6-37
    const double maxE = std::max(std::fabs(lam[0]), std::fabs(lam[dim + 1]));
    for (int i = 0; i < neq; ++i) flux[i] = 0.5 * (f1[i] + f2[i]) - 0.5 * maxE * (s2[i] - s1[i]);
    ret = maxE;
  } else if (rs == 2) {  // HLL, rs_hll.cpp:6-50
    const double maxE = std::max(std::fabs(lam[0]), std::fabs(lam[dim + 1]));
    if (lam[0] >= 0)
      for (int i = 0; i < neq; ++i) flux[i] = f1[i];
    else if (lam[dim + 1] <= 0)
      for (int i = 0; i < neq; ++i) flux[i] = f2[i];
    else
      for (int i = 0; i < neq; ++i)
        flux[i] = (lam[dim + 1] * f1[i] - lam[0] * f2[i] +
                   lam[0] * lam[dim + 1] * (s2[i] - s1[i])) /
                  (lam[dim + 1] - lam[0]);
    ret = maxE;
  } else {  // HLLC, rs_hllc.cpp:71-161, getFStar 39-67
    const double maxE = std::max(lam[0], lam[dim + 1]);
    double SL = lam[0], SR = lam[dim + 1];
    if (SL >= 0)
      for (int i = 0; i < neq; ++i) flux[i] = f1[i];
    else if (SR <= 0)
      for (int i = 0; i < neq; ++i) flux[i] = f2[i];
    else {
      double pL = pressure(P, s1), pR = pressure(P, s2);
      double cL = SL - s1[1] / s1[0];
      double cR = SR - s2[1] / s2[0];
      double sStar = (pR - pL + s1[1] * cL - s2[1] * cR) / (s1[0] * cL - s2[0] * cR);
      const double* st = sStar > 0.0 ? s1 : s2;
      const double* fK = sStar > 0.0 ? f1 : f2;
      double rhoL = st[0];
      double pK = sStar > 0.0 ? pL : pR;
      double SK = sStar > 0.0 ? SL : SR;
      double cK = sStar > 0.0 ? cL : cR;
      double D[5] = {0, 0, 0, 0, 0};
      D[1] = 1.0;
      D[dim + 1] = sStar;
      for (int i = 0; i < neq; ++i)
        flux[i] = (sStar * (st[i] * SK - fK[i]) +
                   D[i] * SK * (pK + rhoL * cK * (sStar - st[1] / st[0]))) *
                  (1.0 / (SK - sStar));
    }
    ret = maxE;
  }
  inverse_rotate(dim, flux, nor);
  return ret;
}

struct BC {
  int type = -1;
  double state[5] = {0, 0, 0, 0, 0};
};

struct Face {
  int e1 = -1, lf1 = -1, e2 = -1, lf2 = -1;
  int fv[4] = {-1, -1, -1, -1};  // face vertex ids in elem1's local order
  double ref2[4][3] = {};        // elem2 reference coords of fv[k]
  bool master = false;           // coarse side of nonconforming faces (not integrated)
};

struct ElemOps {
  std::vector<double> Ae;    // nd x (nd*dim), Ae[j*(nd*dim) + k + d*nd]
  std::vector<double> Minv;  // nd x nd
  std::vector<double> M0;    // nd (averages row)
  double int_psi = 0;
  double detJ_c = 0;         // det J at element centre
};

}  // namespace

struct ref_ctx {
  int dim = 2, geom = REF_GEOM_SQUARE, p = 1, ne = 0, nd = 0, neq = 4;
  int nvpe = 4, nfpe = 4, nvpf = 2, orderW = 1;
  long long ndofs = 0;
  FE fe;
  Phys P;
  int rs = 0, avg = 0;
  std::vector<int> ev;
  std::vector<double> ec;
  std::vector<Face> faces;       // all faces in first-appearance order
  std::vector<int> bdr_face;     // bdr element -> face id
  std::vector<int> bdr_attr;
  std::vector<int> elem_face;    // ne*nfpe
  std::vector<std::vector<int>> el_el;  // ElementToElementTable
  std::map<int, BC> bcs;
  int lim = 0, ind = 0, fun = 2, last_hope = 1, quirks = 0;
  int solver_quirks = 0;  // bit 0: a negative HLLC speed is not an error
  int s = 3;
  std::vector<double> a, b, cc;
  Rule frule, lrule;             // face rule (RHS), order-2 face rule (limiter)
  std::vector<int> op_of;        // element -> ElemOps index
  std::vector<ElemOps> ops;
  // work items of the face pass: interior faces in face order, then boundary
  // elements in boundary order (NonlinearForm::Mult order).
  std::vector<int> item_face, item_bdr;
  std::vector<std::vector<std::pair<int, int>>> elem_items;  // (item, side)
  std::string err;
  // scratch
  std::vector<double> z, flux, means, xnew, y, kbuf;
};

namespace {

int nthreads_cfg = 0;

void elem_map(const ref_ctx* c, int e, const double* xi, double* x, double* J) {
  double N[8], dN[24];
  geom_shape(c->geom, xi, N, dN);
  const int dim = c->dim;
  const double* X = &c->ec[(size_t)e * c->nvpe * dim];
  for (int i = 0; i < dim; ++i) {
    if (x) {
      double v = 0;
      for (int k = 0; k < c->nvpe; ++k) v += N[k] * X[k * dim + i];
      x[i] = v;
    }
    if (J)
      for (int r = 0; r < dim; ++r) {
        double v = 0;
        for (int k = 0; k < c->nvpe; ++k) v += dN[k * dim + r] * X[k * dim + i];
        J[i * dim + r] = v;
      }
  }
}
double det(int dim, const double* J) {
  if (dim == 2) return J[0] * J[3] - J[1] * J[2];
  return J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
         J[2] * (J[3] * J[7] - J[4] * J[6]);
}
// adj(J)[r][d], adj = det * J^{-1}
void adjugate(int dim, const double* J, double* A) {
  if (dim == 2) {
    A[0] = J[3];
    A[1] = -J[1];
    A[2] = -J[2];
    A[3] = J[0];
    return;
  }
  A[0] = J[4] * J[8] - J[5] * J[7];
  A[1] = J[2] * J[7] - J[1] * J[8];
  A[2] = J[1] * J[5] - J[2] * J[4];
  A[3] = J[5] * J[6] - J[3] * J[8];
  A[4] = J[0] * J[8] - J[2] * J[6];
  A[5] = J[2] * J[3] - J[0] * J[5];
  A[6] = J[3] * J[7] - J[4] * J[6];
  A[7] = J[1] * J[6] - J[0] * J[7];
  A[8] = J[0] * J[4] - J[1] * J[3];
}

// Element operators for one geometry: DomainIntegrator::AssembleElementMatrix2
// (domain_integrator.cpp:8-58, rule order 2p), MassIntegrator + inverse
// (fe_evolution.cpp:42-69, rule order 2p + OrderW), GetElementAverages row
// (averager.cpp:104, rule order p + OrderW).
void build_ops(const ref_ctx* c, int e, ElemOps& o) {
  const int nd = c->nd, dim = c->dim;
  std::vector<double> shape(nd), dsh(nd * dim), dshx(nd * dim);
  double J[9], A[9];
  o.Ae.assign((size_t)nd * nd * dim, 0.0);
  Rule r = rule_geom(c->geom, 2 * c->p);
  for (int i = 0; i < r.n; ++i) {
    const double* ip = &r.x[i * r.dim];
    c->fe.shape(ip, shape.data());
    for (int k = 0; k < nd; ++k) shape[k] *= r.w[i];
    c->fe.dshape(ip, dsh.data());
    elem_map(c, e, ip, nullptr, J);
    adjugate(dim, J, A);
    for (int j = 0; j < nd; ++j)
      for (int d = 0; d < dim; ++d) {
        double v = 0;
        for (int rr = 0; rr < dim; ++rr) v += dsh[j * dim + rr] * A[rr * dim + d];
        dshx[j * dim + d] = v;
      }
    for (int d = 0; d < dim; d++)
      for (int j = 0; j < nd; j++)
        for (int k = 0; k < nd; k++)
          o.Ae[(size_t)j * nd * dim + k + d * nd] += shape[k] * dshx[j * dim + d];
  }
  // mass matrix
  std::vector<double> M(nd * nd, 0.0);
  Rule rm = rule_geom(c->geom, 2 * c->p + c->orderW);
  for (int i = 0; i < rm.n; ++i) {
    const double* ip = &rm.x[i * rm.dim];
    c->fe.shape(ip, shape.data());
    elem_map(c, e, ip, nullptr, J);
    double w = det(dim, J) * rm.w[i];
    for (int a = 0; a < nd; ++a) {
      double wa = w * shape[a];
      for (int bb = 0; bb < nd; ++bb) M[a * nd + bb] += wa * shape[bb];
    }
  }
  invert(nd, M, o.Minv);
  // averages row: trial = fe (order p), test = P0
  o.M0.assign(nd, 0.0);
  Rule ra = rule_geom(c->geom, c->p + 0 + c->orderW);
  for (int i = 0; i < ra.n; ++i) {
    const double* ip = &ra.x[i * ra.dim];
    c->fe.shape(ip, shape.data());
    elem_map(c, e, ip, nullptr, J);
    double w = det(dim, J) * ra.w[i];
    for (int j = 0; j < nd; ++j) o.M0[j] += w * shape[j];
  }
  double s = 0;
  for (int j = 0; j < nd; ++j) s += o.M0[j] * 1.0;
  o.int_psi = s;
  double ctr[3] = {1.0 / 3.0, 1.0 / 3.0, 0.5};
  if (c->geom != REF_GEOM_TRIANGLE) ctr[0] = ctr[1] = 0.5;
  elem_map(c, e, ctr, nullptr, J);
  o.detJ_c = det(dim, J);
}

int face_nvert(int geom) { return geom == REF_GEOM_CUBE ? 4 : 2; }

void sort_key(std::array<int, 4>& k, int n) {
  for (int i = 1; i < n; ++i)
    for (int j = i; j > 0 && k[j - 1] > k[j]; --j) std::swap(k[j - 1], k[j]);
}

// Face geometry at face-reference point s from element e1's face vertices:
// ip1 = Loc1(s) (element-1 reference coords), nor = CalcOrtho(face Jacobian).
void face_point(const ref_ctx* c, const Face& f, const double* s, double* ip1, double* ip2,
                double* nor) {
  const int nvf = c->nvpf, dim = c->dim;
  double N[4], dN[8];
  face_shape(nvf, s, N, dN);
  for (int i = 0; i < 3; ++i) {
    ip1[i] = 0;
    if (ip2) ip2[i] = 0;
  }
  double Jf[3][2] = {{0, 0}, {0, 0}, {0, 0}};
  const double* X = &c->ec[(size_t)f.e1 * c->nvpe * dim];
  for (int k = 0; k < nvf; ++k) {
    int lv = local_face_vertex(c->geom, f.lf1, k);
    const double* rv = ref_vertex(c->geom, lv);
    for (int i = 0; i < dim; ++i) {
      ip1[i] += N[k] * rv[i];
      if (ip2) ip2[i] += N[k] * f.ref2[k][i];
      for (int t = 0; t < dim - 1; ++t) Jf[i][t] += dN[k * (dim - 1) + t] * X[lv * dim + i];
    }
  }
  if (dim == 2) {  // CalcOrtho 2x1
    nor[0] = Jf[1][0];
    nor[1] = -Jf[0][0];
  } else {  // CalcOrtho 3x2: col0 x col1
    nor[0] = Jf[1][0] * Jf[2][1] - Jf[2][0] * Jf[1][1];
    nor[1] = Jf[2][0] * Jf[0][1] - Jf[0][0] * Jf[2][1];
    nor[2] = Jf[0][0] * Jf[1][1] - Jf[1][0] * Jf[0][1];
  }
}

Rule face_rule(const ref_ctx* c, int q) {
  return c->dim == 2 ? rule_segment(q) : rule_square(q);
}

// DGTraceIntegrator order used by face_integrator.cpp:45-58 and
// boundary_integrator.cpp:39-52: OrderW + 2p, +1 on simplices.
int face_order(const ref_ctx* c) {
  int q = c->orderW + 2 * c->p;
  if (c->geom == REF_GEOM_TRIANGLE) q++;
  return q;
}

void compute_right_state(const ref_ctx* c, const BC& bc, const double* s1, double* s2,
                         const double* nor) {
  const int neq = c->neq, dim = c->dim;
  for (int i = 0; i < neq; ++i) s2[i] = s1[i];
  switch (bc.type) {
    case 0:  // slip, boundary_integrator_slip.cpp:7-17
    case 4:  // wall, boundary_integrator_wall.cpp:7-17
      rotate(dim, s2, nor);
      s2[1] *= -1;
      inverse_rotate(dim, s2, nor);
      break;
    case 1:  // open, boundary_integrator_open.cpp:9-12
      break;
    case 2:  // fixed state in the rotated frame, boundary_integrator_constant.cpp:8-20
      rotate(dim, s2, nor);
      for (int i = 0; i < dim + 2; ++i) s2[i] = bc.state[i];
      inverse_rotate(dim, s2, nor);
      break;
    case 3:  // supersonic inlet, boundary_integrator_supersonic_inlet.cpp:8-19
      for (int i = 0; i < dim + 2; ++i) s2[i] = bc.state[i];
      break;
    case 5:  // subsonic inlet, boundary_integrator_subsonic_inlet.cpp:10-19:
             // 2 * fixed - own, in the rotated frame
      rotate(dim, s2, nor);
      for (int i = 0; i < dim + 2; ++i) s2[i] = 2.0 * bc.state[i] - s2[i];
      inverse_rotate(dim, s2, nor);
      break;
    case 6:  // subsonicInletTotalPressure, ..._subsonic_inlet_total_pressure.cpp:10-40
    case 7: {  // subsonicInletFixedPressure, ..._subsonic_inlet_fixed_pressure.cpp:10-36
      const double g = c->P.gamma, R = c->P.R, TTot = bc.state[1];
      double rhoU2 = 0;
      for (int d = 0; d < dim; ++d) rhoU2 += s1[1 + d] * s1[1 + d];
      rhoU2 /= s1[0];
      const double MTTotSq = rhoU2 / s1[0] / g / R / TTot;
      const double MSq = MTTotSq / (1.0 - 0.5 * (g - 1.0) * MTTotSq);
      const double p = bc.type == 6
                           ? bc.state[0] * std::pow(1.0 + 0.5 * (g - 1.0) * MSq, -g / (g - 1.0))
                           : bc.state[0];
      const double T = TTot / (1.0 + 0.5 * (g - 1.0) * MSq);
      const double rho = p / R / T;
      s2[neq - 1] = p / (g - 1.0) + 0.5 * rhoU2 / s1[0] * rho;
      for (int d = 0; d < dim; ++d) s2[1 + d] = s1[1 + d] / s1[0] * rho;
      s2[0] = rho;
      break;
    }
    case 8: {  // fixedPressureOutlet, boundary_integrator_open_fixed_pressure.cpp:10-30
      // (epsIn subtracts 0.5 |m|^2, not 0.5 |m|^2 / rho, as the reference does)
      const double g = c->P.gamma, pFix = bc.state[0];
      double rhoU2 = 0;
      for (int d = 0; d < dim; ++d) rhoU2 += s1[1 + d] * s1[1 + d];
      const double U2 = rhoU2 / s1[0] / s1[0];
      const double epsIn = (s1[neq - 1] - 0.5 * rhoU2) / s1[0];
      const double rho = pFix / (g - 1.0) / epsIn;
      s2[neq - 1] = pFix / (g - 1.0) + 0.5 * rho * U2;
      for (int d = 0; d < dim; ++d) s2[1 + d] = s1[1 + d] / s1[0] * rho;
      s2[0] = rho;
      break;
    }
    case 9: {  // totalPressureFixedTemperatureOutlet, ..._open_total_pressure.cpp:10-40
      // The reference forms m.n from nor[1..dim] (one past the normal's last
      // component); here m.n uses nor[0..dim-1].
      const double g = c->P.gamma, R = c->P.R, pTot = bc.state[0], TFix = bc.state[1];
      double rho2U2 = 0, rhoN = 0;
      for (int d = 0; d < dim; ++d) {
        rho2U2 += s1[1 + d] * s1[1 + d];
        rhoN += s1[1 + d] * nor[d];
      }
      const double U2 = rho2U2 / s1[0] / s1[0];
      const double epsIn = rhoN > 0 ? (s1[neq - 1] - 0.5 * rho2U2) / s1[0] : R / (g - 1.0) * TFix;
      const double M = std::sqrt(rho2U2 / s1[0] / s1[0]) / sound_speed(c->P, s1);  // ComputeM
      double p = M > 1 ? pTot * std::pow(1.0 + 0.5 * (g - 1.0) * M * M, -g / (g - 1.0)) : pTot;
      const double rho = M > 1 ? p / (g - 1.0) / epsIn : p / (0.5 * U2 + (g - 1.0) * epsIn);
      p = M > 1 ? p : p - 0.5 * U2 * rho;
      s2[neq - 1] = p / (g - 1.0) + 0.5 * rho * U2;
      for (int d = 0; d < dim; ++d) s2[1 + d] = s1[1 + d] * (rho / s1[0]);
      s2[0] = rho;
      break;
    }
    case 10: {  // charOutlet, boundary_integrator_char_outlet.cpp:14-57
      // The reference rotates and reads its ghost vector before it assigns it
      // (the previous boundary point's ghost state, or uninitialised memory at
      // the first point); here it enters as the interior state s1.  bc.state
      // holds the outer state (cOut, UOut from it, as the constructor does).
      const double g = c->P.gamma, b = c->P.b;
      const double cOut = sound_speed(c->P, bc.state);
      const double UOut = bc.state[1] / bc.state[0];
      const double cIn = sound_speed(c->P, s1);
      rotate(dim, s2, nor);
      const double UIn = s2[1] / s2[0];
      const double UB = 0.5 * (UIn + UOut) - (cOut - cIn) / (g - 1.0);
      const double cB = -0.25 * (g - 1.0) * (UOut - UIn) + 0.5 * (cOut + cIn);
      const double sB = s2[1] < 0 ? cOut * cOut / std::pow(bc.state[0], g - 1.0) / g
                                  : cIn * cIn / std::pow(s2[0], g - 1.0) / g;
      const double rhoB = std::pow(cB * cB / sB / g, 1.0 / (g - 1.0));
      const double pB = rhoB * cB * cB / g;
      s2[0] = rhoB;
      s2[1] = UB;  // a velocity in the momentum slot, as the reference stores it
      const double v = s2[2] / s2[0], w = dim == 3 ? s2[3] / s2[0] : 0.0;
      // ComputeEnergy, physics.cpp:128-131
      s2[neq - 1] = pB / (g - 1.0) * (1.0 - rhoB * b) + 0.5 * rhoB * (UB * UB + v * v + w * w);
      inverse_rotate(dim, s2, nor);
      break;
    }
  }
}

// One face work item (FaceIntegrator::AssembleFaceVector,
// face_integrator.cpp:11-276, or BoundaryIntegrator::AssembleFaceVector,
// boundary_integrator.cpp:12-194).  out1/out2: nd*neq (DenseMatrix dof x eq,
// column-major: out[k*nd + s]).  Returns false on an unphysical state.
bool face_item(const ref_ctx* c, const double* x, int face, const BC* bc, double* out1,
               double* out2, double& mcs_max, int& bad) {
  const Face& f = c->faces[face];
  const int nd = c->nd, neq = c->neq, dim = c->dim;
  const long long ND = c->ndofs;
  double shape1[125], shape2[125];
  double ip1[3], ip2[3], nor[3];
  double u1[5], u2[5], fluxN[5];
  for (int i = 0; i < nd * neq; ++i) {
    out1[i] = 0;
    if (out2) out2[i] = 0;
  }
  const Rule& r = c->frule;
  for (int q = 0; q < r.n; ++q) {
    const double* s = &r.x[q * r.dim];
    face_point(c, f, s, ip1, bc ? nullptr : ip2, nor);
    c->fe.shape(ip1, shape1);
    for (int k = 0; k < neq; ++k) {
      double v = 0;
      for (int sidx = 0; sidx < nd; ++sidx)
        v += x[k * ND + (long long)f.e1 * nd + sidx] * shape1[sidx];
      u1[k] = v;
    }
    if (!bc) {
      c->fe.shape(ip2, shape2);
      for (int k = 0; k < neq; ++k) {
        double v = 0;
        for (int sidx = 0; sidx < nd; ++sidx)
          v += x[k * ND + (long long)f.e2 * nd + sidx] * shape2[sidx];
        u2[k] = v;
      }
    }
    double normag = 0;
    for (int i = 0; i < dim; i++) normag += nor[i] * nor[i];
    normag = std::sqrt(normag);
    const double inv = 1.0 / normag;  // nor *= 1.0/nor.Norml2()
    for (int i = 0; i < dim; ++i) nor[i] *= inv;
    if (bc) compute_right_state(c, *bc, u1, u2, nor);
    const double mcs = rs_eval(c->P, c->rs, c->avg, u1, u2, nor, fluxN);
    if (mcs < 0 && (!(c->solver_quirks & 1) || mcs == -1.0)) {
      bad = face;
      return false;
    }
    if (mcs > mcs_max) mcs_max = mcs;
    for (int k = 0; k < neq; ++k) fluxN[k] *= r.w[q];
    for (int k = 0; k < neq; k++) {
      for (int sidx = 0; sidx < nd; sidx++) out1[k * nd + sidx] -= fluxN[k] * shape1[sidx] * normag;
      if (!bc)
        for (int sidx = 0; sidx < nd; sidx++) out2[k * nd + sidx] += fluxN[k] * shape2[sidx] * normag;
    }
  }
  return true;
}

int nthreads() { return nthreads_cfg > 0 ? nthreads_cfg : omp_get_max_threads(); }

// A.Mult(x, z): face and boundary integrators, accumulated per element in
// NonlinearForm::Mult order.  Chunked so that the per-item buffers stay
// bounded; per element the additions happen in item order, as in the
// sequential reference.
int faces_mult(ref_ctx* c, const double* x, double* z, double& mcs) {
  const int nd = c->nd, neq = c->neq;
  const long long ND = c->ndofs;
  const int nitems = (int)(c->item_face.size() + c->item_bdr.size());
  const int nif = (int)c->item_face.size();
  const int chunk = 65536;
  const int blk = nd * neq;
  std::vector<double> buf((size_t)std::min(chunk, std::max(nitems, 1)) * 2 * blk);
  std::vector<size_t> cursor(c->ne, 0);
  int bad = -1;
  mcs = std::max(mcs, 0.0);
  for (int i0 = 0; i0 < nitems; i0 += chunk) {
    int i1 = std::min(nitems, i0 + chunk);
    double cmax = mcs;
    int cbad = -1;
#pragma omp parallel for schedule(static) num_threads(nthreads()) reduction(max : cmax)
    for (int it = i0; it < i1; ++it) {
      double* o1 = &buf[(size_t)(it - i0) * 2 * blk];
      double* o2 = o1 + blk;
      int lbad = -1;
      bool ok;
      if (it < nif) {
        ok = face_item(c, x, c->item_face[it], nullptr, o1, o2, cmax, lbad);
      } else {
        int bi = c->item_bdr[it - nif];
        auto itb = c->bcs.find(c->bdr_attr[bi]);
        ok = face_item(c, x, c->bdr_face[bi], &itb->second, o1, nullptr, cmax, lbad);
      }
      if (!ok) {
#pragma omp critical
        { if (cbad < 0 || lbad < cbad) cbad = lbad; }
      }
    }
    if (cbad >= 0) {
      bad = cbad;
      break;
    }
    mcs = cmax;
#pragma omp parallel for schedule(static) num_threads(nthreads())
    for (int e = 0; e < c->ne; ++e) {
      auto& lst = c->elem_items[e];
      size_t& cur = cursor[e];
      while (cur < lst.size() && lst[cur].first < i1) {
        int it = lst[cur].first, side = lst[cur].second;
        const double* o = &buf[(size_t)(it - i0) * 2 * blk + side * blk];
        for (int k = 0; k < neq; ++k)
          for (int sidx = 0; sidx < nd; ++sidx)
            z[k * ND + (long long)e * nd + sidx] += o[k * nd + sidx];
        ++cur;
      }
    }
  }
  if (bad >= 0) {
    const Face& f = c->faces[bad];
    char msg[160];
    snprintf(msg, sizeof msg, "unphysical state at face %d (elements %d %d)", bad, f.e1, f.e2);
    c->err = msg;
    return REF_ERR_UNPHYSICAL;
  }
  return REF_OK;
}

// Averager::computeMeanValues -> GridFunction::GetElementAverages
// (averager.cpp:84-109); means[iEq*NE + e].
void means_of(const ref_ctx* c, const double* x, double* means) {
  const int nd = c->nd, neq = c->neq;
  const long long ND = c->ndofs;
#pragma omp parallel for schedule(static) num_threads(nthreads())
  for (int e = 0; e < c->ne; ++e) {
    const ElemOps& o = c->ops[c->op_of[e]];
    for (int k = 0; k < neq; ++k) {
      double v = 0;
      for (int j = 0; j < nd; ++j) v += o.M0[j] * x[k * ND + (long long)e * nd + j];
      means[k * (long long)c->ne + e] = v / o.int_psi;
    }
  }
}

}  // namespace

extern "C" {

// Nonconforming faces (restating MFEM's NCMesh face lists, which the
// reference gets from EnsureNCMesh + refinement, case_manager.cpp:269,
// main.cpp:564-696): a face that no second element shares and no boundary
// element lists is either a slave -- it lies inside a face of an element on
// the other side -- or that master face.  NonlinearForm::Mult integrates
// each slave face as an interior face with Elem1 = the slave's (fine)
// element and Elem2 = the master's element, whose points are the slave
// face's points mapped into it (Mesh::GetFaceElementTransformations with the
// NC point matrix); master faces are skipped (GetInteriorFaceTransformations
// returns NULL for them).  Every element is affine here, so the mapped
// reference coordinates of the slave's corners give all its points.
namespace {
void inverse_map(const ref_ctx* c, int e, const double* x, double* xi) {
  const int dim = c->dim;
  double xc[3], J[9], xi_c[3];
  for (int i = 0; i < 3; ++i) xi_c[i] = c->geom == REF_GEOM_TRIANGLE ? 1.0 / 3.0 : 0.5;
  elem_map(c, e, xi_c, xc, J);
  double d[3] = {0, 0, 0};
  for (int i = 0; i < dim; ++i) d[i] = x[i] - xc[i];
  if (dim == 2) {
    const double det = J[0] * J[3] - J[1] * J[2];
    xi[0] = xi_c[0] + (J[3] * d[0] - J[1] * d[1]) / det;
    xi[1] = xi_c[1] + (-J[2] * d[0] + J[0] * d[1]) / det;
    xi[2] = 0;
  } else {
    double A[9];  // adjugate / det
    A[0] = J[4] * J[8] - J[5] * J[7];
    A[1] = J[2] * J[7] - J[1] * J[8];
    A[2] = J[1] * J[5] - J[2] * J[4];
    A[3] = J[5] * J[6] - J[3] * J[8];
    A[4] = J[0] * J[8] - J[2] * J[6];
    A[5] = J[2] * J[3] - J[0] * J[5];
    A[6] = J[3] * J[7] - J[4] * J[6];
    A[7] = J[1] * J[6] - J[0] * J[7];
    A[8] = J[0] * J[4] - J[1] * J[3];
    const double det = J[0] * A[0] + J[1] * A[3] + J[2] * A[6];
    for (int r = 0; r < 3; ++r) xi[r] = xi_c[r] + (A[r * 3] * d[0] + A[r * 3 + 1] * d[1] + A[r * 3 + 2] * d[2]) / det;
  }
}

// physical corner k (elem1 local face order) of face f
void face_corner(const ref_ctx* c, const Face& f, int k, double* x) {
  const int lv = local_face_vertex(c->geom, f.lf1, k);
  for (int i = 0; i < c->dim; ++i) x[i] = c->ec[((size_t)f.e1 * c->nvpe + lv) * c->dim + i];
}

double face_measure(const ref_ctx* c, const Face& f) {
  double a[3], b[3], d[3];
  face_corner(c, f, 0, a);
  face_corner(c, f, 1, b);
  if (c->dim == 2) return std::hypot(b[0] - a[0], b[1] - a[1]);
  face_corner(c, f, 3, d);
  double u[3], v[3];
  for (int i = 0; i < 3; ++i) u[i] = b[i] - a[i], v[i] = d[i] - a[i];
  return std::sqrt(std::pow(u[1] * v[2] - u[2] * v[1], 2) + std::pow(u[2] * v[0] - u[0] * v[2], 2) +
                   std::pow(u[0] * v[1] - u[1] * v[0], 2));
}
}  // namespace

bool classify_nc_faces(ref_ctx* c) {
  const int nvf = c->nvpf, dim = c->dim;
  std::vector<char> bdr(c->faces.size(), 0);
  for (int f : c->bdr_face) bdr[f] = 1;
  std::vector<int> lone;
  for (int f = 0; f < (int)c->faces.size(); ++f)
    if (c->faces[f].e2 < 0 && !bdr[f]) lone.push_back(f);
  std::vector<double> covered(c->faces.size(), 0.0);
  std::vector<char> is_slave(c->faces.size(), 0);
  for (int sf : lone) {
    Face& S = c->faces[sf];
    for (int mf : lone) {
      const Face& Mf = c->faces[mf];
      if (mf == sf || Mf.e1 == S.e1) continue;
      // the slave's corners in the master element's reference space, on its face
      const double* r0 = ref_vertex(c->geom, local_face_vertex(c->geom, Mf.lf1, 0));
      const double* r1 = ref_vertex(c->geom, local_face_vertex(c->geom, Mf.lf1, 1));
      const double* r3 = ref_vertex(c->geom, local_face_vertex(c->geom, Mf.lf1, nvf - 1));
      double xi[4][3];
      bool inside = true;
      for (int k = 0; k < nvf && inside; ++k) {
        double x[3];
        face_corner(c, S, k, x);
        inverse_map(c, Mf.e1, x, xi[k]);
        double p[3], s0 = 0, s1 = 0, n0 = 0, n1 = 0;
        for (int i = 0; i < dim; ++i) {
          s0 += (xi[k][i] - r0[i]) * (r1[i] - r0[i]);
          n0 += (r1[i] - r0[i]) * (r1[i] - r0[i]);
          s1 += (xi[k][i] - r0[i]) * (r3[i] - r0[i]);
          n1 += (r3[i] - r0[i]) * (r3[i] - r0[i]);
        }
        s0 /= n0;
        s1 = dim == 3 ? s1 / n1 : 0.0;
        double res = 0;
        for (int i = 0; i < dim; ++i) {
          p[i] = r0[i] + s0 * (r1[i] - r0[i]) + (dim == 3 ? s1 * (r3[i] - r0[i]) : 0.0);
          res = std::max(res, std::fabs(p[i] - xi[k][i]));
        }
        const double tol = 1e-9;
        inside = res < tol && s0 > -tol && s0 < 1 + tol && s1 > -tol && s1 < 1 + tol;
      }
      if (!inside) continue;
      S.e2 = Mf.e1;
      S.lf2 = Mf.lf1;
      for (int k = 0; k < nvf; ++k)
        for (int i = 0; i < 3; ++i) S.ref2[k][i] = i < dim ? xi[k][i] : 0.0;
      is_slave[sf] = 1;
      covered[mf] += face_measure(c, S);
      break;
    }
  }
  for (int f : lone) {
    if (is_slave[f]) continue;
    const double m = face_measure(c, c->faces[f]);
    if (!(std::fabs(covered[f] - m) <= 1e-9 * m)) return false;  // neither slave nor covered master
    c->faces[f].master = true;
  }
  return true;
}

ref_ctx* ref_create(int dim, int geom, int order, int num_elements, const int* elem_vertices,
                    const double* elem_coords, int num_bdr, const int* bdr_vertices,
                    const int* bdr_attr) {
  if (!((dim == 2 && (geom == REF_GEOM_SQUARE || geom == REF_GEOM_TRIANGLE)) ||
        (dim == 3 && geom == REF_GEOM_CUBE)))
    return nullptr;
  if (order < 0 || num_elements <= 0) return nullptr;
  if (order > (geom == REF_GEOM_TRIANGLE ? 4 : 3)) return nullptr;
  ref_ctx* c = new ref_ctx();
  c->dim = dim;
  c->geom = geom;
  c->p = order;
  c->ne = num_elements;
  c->neq = dim + 2;
  c->P.dim = dim;
  c->P.neq = dim + 2;
  c->nvpe = geom == REF_GEOM_TRIANGLE ? 3 : (geom == REF_GEOM_SQUARE ? 4 : 8);
  c->nfpe = geom == REF_GEOM_TRIANGLE ? 3 : (geom == REF_GEOM_SQUARE ? 4 : 6);
  c->nvpf = face_nvert(geom);
  c->orderW = geom == REF_GEOM_TRIANGLE ? 0 : (geom == REF_GEOM_SQUARE ? 1 : 2);
  c->fe.init(geom, order);
  c->nd = c->fe.nd;
  c->ndofs = (long long)c->ne * c->nd;
  c->frule = face_rule(c, face_order(c));
  c->lrule = face_rule(c, 2);
  c->ev.assign(elem_vertices, elem_vertices + (size_t)num_elements * c->nvpe);
  c->ec.assign(elem_coords, elem_coords + (size_t)num_elements * c->nvpe * dim);
  // Faces: Mesh::GenerateFaces semantics, Elem1 = first element (in element
  // order) that has the face, face vertex order taken from Elem1's local face.
  std::map<std::array<int, 4>, int> key2face;
  c->elem_face.assign((size_t)c->ne * c->nfpe, -1);
  const int nvf = c->nvpf;
  for (int e = 0; e < c->ne; ++e) {
    for (int lf = 0; lf < c->nfpe; ++lf) {
      std::array<int, 4> key = {-1, -1, -1, -1};
      int fv[4];
      for (int k = 0; k < nvf; ++k) {
        fv[k] = c->ev[(size_t)e * c->nvpe + local_face_vertex(geom, lf, k)];
        key[k] = fv[k];
      }
      sort_key(key, nvf);
      auto it = key2face.find(key);
      if (it == key2face.end()) {
        Face f;
        f.e1 = e;
        f.lf1 = lf;
        for (int k = 0; k < nvf; ++k) f.fv[k] = fv[k];
        key2face[key] = (int)c->faces.size();
        c->elem_face[(size_t)e * c->nfpe + lf] = (int)c->faces.size();
        c->faces.push_back(f);
      } else {
        Face& f = c->faces[it->second];
        if (f.e2 >= 0) {
          delete c;
          return nullptr;  // non-manifold
        }
        f.e2 = e;
        f.lf2 = lf;
        for (int k = 0; k < nvf; ++k) {
          int found = -1;
          for (int m = 0; m < nvf; ++m)
            if (fv[m] == f.fv[k]) found = local_face_vertex(geom, lf, m);
          const double* rv = ref_vertex(geom, found);
          for (int i = 0; i < 3; ++i) f.ref2[k][i] = rv[i];
        }
        c->elem_face[(size_t)e * c->nfpe + lf] = it->second;
      }
    }
  }
  c->bdr_attr.assign(bdr_attr, bdr_attr + num_bdr);
  c->bdr_face.assign(num_bdr, -1);
  for (int bi = 0; bi < num_bdr; ++bi) {
    std::array<int, 4> key = {-1, -1, -1, -1};
    for (int k = 0; k < nvf; ++k) key[k] = bdr_vertices[(size_t)bi * nvf + k];
    sort_key(key, nvf);
    auto it = key2face.find(key);
    if (it == key2face.end() || c->faces[it->second].e2 >= 0) {
      delete c;
      return nullptr;
    }
    c->bdr_face[bi] = it->second;
  }
  if (!classify_nc_faces(c)) {
    delete c;
    return nullptr;
  }
  // ElementToElementTable
  c->el_el.assign(c->ne, {});
  for (const Face& f : c->faces)
    if (f.e2 >= 0 && f.e2 != f.e1) {
      c->el_el[f.e1].push_back(f.e2);
      c->el_el[f.e2].push_back(f.e1);
    }
  for (auto& v : c->el_el) {
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
  }
  // element operators, shared between elements with bitwise-identical geometry
  std::map<std::vector<double>, int> key2op;
  c->op_of.assign(c->ne, 0);
  for (int e = 0; e < c->ne; ++e) {
    std::vector<double> key;
    const double* X = &c->ec[(size_t)e * c->nvpe * dim];
    for (int k = 1; k < c->nvpe; ++k)
      for (int i = 0; i < dim; ++i) key.push_back(X[k * dim + i] - X[i]);
    auto it = key2op.find(key);
    if (it != key2op.end()) {
      c->op_of[e] = it->second;
      continue;
    }
    ElemOps o;
    build_ops(c, e, o);
    c->op_of[e] = (int)c->ops.size();
    key2op[key] = (int)c->ops.size();
    c->ops.push_back(std::move(o));
  }
  c->a = {1.0, 0.25, 0.25};
  c->b = {1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0};
  c->cc = {1.0, 0.5};
  c->s = 3;
  return c;
}

void ref_destroy(ref_ctx* c) { delete c; }
void ref_set_threads(int n) { nthreads_cfg = n; }
long long ref_ndofs(ref_ctx* c) { return c->ndofs; }
int ref_nd(ref_ctx* c) { return c->nd; }
int ref_neq(ref_ctx* c) { return c->neq; }
const char* ref_last_error(ref_ctx* c) { return c->err.c_str(); }

static void rebuild_items(ref_ctx* c) {
  c->item_face.clear();
  c->item_bdr.clear();
  for (int f = 0; f < (int)c->faces.size(); ++f)
    if (c->faces[f].e2 >= 0) c->item_face.push_back(f);
  for (int bi = 0; bi < (int)c->bdr_face.size(); ++bi)
    if (c->bcs.count(c->bdr_attr[bi])) c->item_bdr.push_back(bi);
  c->elem_items.assign(c->ne, {});
  const int nif = (int)c->item_face.size();
  for (int it = 0; it < nif; ++it) {
    const Face& f = c->faces[c->item_face[it]];
    c->elem_items[f.e1].push_back({it, 0});
    c->elem_items[f.e2].push_back({it, 1});
  }
  for (int i = 0; i < (int)c->item_bdr.size(); ++i) {
    const Face& f = c->faces[c->bdr_face[c->item_bdr[i]]];
    c->elem_items[f.e1].push_back({nif + i, 0});
  }
}

int ref_nfaces(ref_ctx* c, int* interior, int* boundary) {
  int ni = 0, nb = 0;
  for (const Face& f : c->faces) (f.e2 >= 0 ? ni : nb)++;
  if (interior) *interior = ni;
  if (boundary) *boundary = nb;
  return (int)c->faces.size();
}

int ref_set_physics(ref_ctx* c, int rsolver, int averaging, double gamma, double covolume,
                    double gas_constant) {
  if (rsolver < 0 || rsolver > 3 || averaging < 0 || averaging > 1) return REF_ERR_INVALID;
  c->rs = rsolver;
  c->avg = averaging;
  c->P.gamma = gamma;
  c->P.b = covolume;
  c->P.R = gas_constant;
  rebuild_items(c);
  return REF_OK;
}

int ref_set_bc(ref_ctx* c, int attr, int type, const double* state) {
  if (type < 0 || type > 10) return REF_ERR_INVALID;
  if (!state && (type == 2 || type == 3 || type >= 5)) return REF_ERR_INVALID;
  BC bc;
  bc.type = type;
  if (state)
    for (int i = 0; i < c->neq; ++i) bc.state[i] = state[i];
  c->bcs[attr] = bc;
  rebuild_items(c);
  return REF_OK;
}

int ref_right_state(ref_ctx* c, int attr, const double* s1, const double* nor, double* s2) {
  auto it = c->bcs.find(attr);
  if (it == c->bcs.end() || !s1 || !nor || !s2) return REF_ERR_INVALID;
  compute_right_state(c, it->second, s1, s2, nor);
  return REF_OK;
}

int ref_set_limiter(ref_ctx* c, int limiter, int indicator, int function, int last_hope,
                    int quirks) {
  if (limiter < 0 || limiter > 1 || indicator < 0 || indicator > 3 || function < 0 ||
      function > 2 || (indicator == 3 && limiter == 1))
    return REF_ERR_INVALID;
  c->lim = limiter;
  c->ind = indicator;
  c->fun = function;
  c->last_hope = last_hope;
  c->quirks = quirks;
  return REF_OK;
}

int ref_set_solver_quirks(ref_ctx* c, int flags) {
  c->solver_quirks = flags;
  return REF_OK;
}

int ref_set_tableau(ref_ctx* c, int s, const double* a, const double* b, const double* cc) {
  if (s < 1 || s > 4) return REF_ERR_INVALID;
  c->s = s;
  c->a.assign(a, a + s * (s - 1) / 2);
  c->b.assign(b, b + s);
  c->cc.assign(cc, cc + std::max(s - 1, 0));
  return REF_OK;
}

int ref_node_coords(ref_ctx* c, double* out) {
  const int nd = c->nd, dim = c->dim;
  for (int e = 0; e < c->ne; ++e)
    for (int j = 0; j < nd; ++j) {
      double xv[3];
      elem_map(c, e, &c->fe.nodes[j * dim], xv, nullptr);
      for (int i = 0; i < dim; ++i) out[i * c->ndofs + (long long)e * nd + j] = xv[i];
    }
  return REF_OK;
}

// Mesh::GetElementSize(i, 1): minimum singular value of the Jacobian at the
// element centre, relative to the equilateral reference triangle for
// triangles (Geometries.JacToPerfJac); main.cpp:191-201.
double ref_hmin(ref_ctx* c) {
  double hmin = 1e300;
  const int dim = c->dim;
  for (int e = 0; e < c->ne; ++e) {
    double ctr[3] = {0.5, 0.5, 0.5};
    if (c->geom == REF_GEOM_TRIANGLE) ctr[0] = ctr[1] = 1.0 / 3.0;
    double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    elem_map(c, e, ctr, nullptr, J);
    if (c->geom == REF_GEOM_TRIANGLE) {
      // J * PerfGeomToGeomJac, equilateral (0,0),(1,0),(1/2,sqrt3/2) -> ref
      const double A[4] = {1.0, -1.0 / std::sqrt(3.0), 0.0, 2.0 / std::sqrt(3.0)};
      double T[4];
      for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) T[i * 2 + j] = J[i * 2 + 0] * A[0 * 2 + j] + J[i * 2 + 1] * A[1 * 2 + j];
      for (int i = 0; i < 4; ++i) J[i] = T[i];
    }
    double smin;
    if (dim == 2) {
      double a = J[0], b = J[1], cc = J[2], d = J[3];
      double s1 = a * a + b * b + cc * cc + d * d;
      double dt = a * d - b * cc;
      double disc = std::sqrt(std::max(0.0, s1 * s1 - 4 * dt * dt));
      smin = std::sqrt(std::max(0.0, 0.5 * (s1 - disc)));
    } else {
      // eigenvalues of J^T J (symmetric 3x3), closed form
      double M[9];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double v = 0;
          for (int k = 0; k < 3; ++k) v += J[k * 3 + i] * J[k * 3 + j];
          M[i * 3 + j] = v;
        }
      double p1 = M[1] * M[1] + M[2] * M[2] + M[5] * M[5];
      double q = (M[0] + M[4] + M[8]) / 3.0;
      double lmin;
      if (p1 == 0) {
        lmin = std::min(M[0], std::min(M[4], M[8]));
      } else {
        double p2 = sqr(M[0] - q) + sqr(M[4] - q) + sqr(M[8] - q) + 2 * p1;
        double pp = std::sqrt(p2 / 6.0);
        double B[9];
        for (int i = 0; i < 9; ++i) B[i] = (M[i] - (i % 4 == 0 ? q : 0.0)) / pp;
        double r = det(3, B) / 2.0;
        double phi = r <= -1 ? M_PI / 3.0 : (r >= 1 ? 0.0 : std::acos(r) / 3.0);
        lmin = q + 2 * pp * std::cos(phi + 2.0 * M_PI / 3.0);
      }
      smin = std::sqrt(std::max(0.0, lmin));
    }
    hmin = std::min(hmin, smin);
  }
  return hmin;
}

int ref_face_speed(ref_ctx* c, const double* x, double* max_char_speed) {
  std::vector<double> z((size_t)c->ndofs * c->neq, 0.0);
  double mcs = 0.0;
  int st = faces_mult(c, x, z.data(), mcs);
  *max_char_speed = mcs;
  return st;
}

// FE_Evolution::Mult, fe_evolution.cpp:102-216 (+ GetFlux 219-245).
int ref_rhs(ref_ctx* c, const double* x, double* y, double* max_char_speed) {
  const int nd = c->nd, neq = c->neq, dim = c->dim;
  const long long ND = c->ndofs;
  c->z.assign((size_t)ND * neq, 0.0);
  double mcs = 0.0;  // max_char_speed = 0 (fe_evolution.cpp:105)
  int st = faces_mult(c, x, c->z.data(), mcs);
  if (st != REF_OK) return st;
  // GetFlux + Aflux->AddMult per equation + inverse mass, element by element
  double nmax = mcs;
#pragma omp parallel for schedule(static) num_threads(nthreads()) reduction(max : nmax)
  for (int e = 0; e < c->ne; ++e) {
    const ElemOps& o = c->ops[c->op_of[e]];
    double F[5 * 3], st5[5];
    std::vector<double> fl((size_t)nd * dim * neq);  // fl[(k*dim + d)*nd + m]
    for (int m = 0; m < nd; ++m) {
      for (int k = 0; k < neq; ++k) st5[k] = x[k * ND + (long long)e * nd + m];
      flux_full(c->P, st5, F);
      for (int d = 0; d < dim; ++d)
        for (int k = 0; k < neq; ++k) fl[(k * dim + d) * nd + m] = F[k * dim + d];
      const double s = max_char_speed_of(c->P, st5);
      if (s > nmax) nmax = s;
    }
    double* zz = c->z.data();
    for (int k = 0; k < neq; ++k)
      for (int j = 0; j < nd; ++j) {
        double dsum = 0.0;
        for (int d = 0; d < dim; ++d)
          for (int m = 0; m < nd; ++m)
            dsum += o.Ae[(size_t)j * nd * dim + m + d * nd] * fl[(k * dim + d) * nd + m];
        zz[k * ND + (long long)e * nd + j] += 1.0 * dsum;
      }
    // y_e = Me_inv[e] * z_e  (fe_evolution.cpp:178-208)
    for (int k = 0; k < neq; ++k)
      for (int i = 0; i < nd; ++i) {
        double v = 0;
        for (int j = 0; j < nd; ++j) v += o.Minv[i * nd + j] * zz[k * ND + (long long)e * nd + j];
        y[k * ND + (long long)e * nd + i] = v;
      }
  }
  *max_char_speed = nmax;
  return REF_OK;
}

int ref_means(ref_ctx* c, const double* x, double* means) {
  means_of(c, x, means);
  return REF_OK;
}

// IndicatorShu::checkDiscontinuity, indicator_shu.cpp:13-74, with the
// extrapolated averages of Averager::computeStencilExtrapAverages and
// assembleShiftedElementMatrix (averager.cpp:154-273): for each stencil cell k
// (the cell, then ElementToElementTable neighbours) the rule of order
// p + OrderW on the troubled cell e, mapped to physical space by e and back to
// k's reference space, weights k's polynomial by |J_k| w_q; divided by
// int_psi(k) = the integral of 1 over k.
void shu_indicator(const ref_ctx* c, const double* x, const double* mean, int e, double* val) {
  const int nd = c->nd, neq = c->neq, dim = c->dim, ne = c->ne;
  const long long ND = c->ndofs;
  const Rule r = rule_geom(c->geom, c->p + 0 + c->orderW);
  double maxF[5], sumD[5], ume[5];
  for (int k = 0; k < neq; ++k) {
    maxF[k] = -1e9;
    sumD[k] = 0.0;
    ume[k] = mean[k * (long long)ne + e];
  }
  std::vector<int> st(1, e);
  for (int nb : c->el_el[e]) st.push_back(nb);
  double shape[125];
  for (int kc : st) {
    double Jk[9], x0[3], zero[3] = {0, 0, 0}, Kinv[9];
    elem_map(c, kc, zero, x0, Jk);
    const double dk = det(dim, Jk);
    adjugate(dim, Jk, Kinv);
    for (int i = 0; i < dim * dim; ++i) Kinv[i] /= dk;
    double loc[5] = {0, 0, 0, 0, 0};
    for (int q = 0; q < r.n; ++q) {
      double xp[3], ipr[3] = {0, 0, 0};
      elem_map(c, e, &r.x[q * dim], xp, nullptr);  // TransTroubled.Transform
      for (int i = 0; i < dim; ++i)                 // Trans.TransformBack
        for (int m = 0; m < dim; ++m) ipr[i] += Kinv[i * dim + m] * (xp[m] - x0[m]);
      c->fe.shape(ipr, shape);
      const double w = dk * r.w[q];
      for (int k = 0; k < neq; ++k) {
        double v = 0;
        for (int j = 0; j < nd; ++j) v += shape[j] * x[k * ND + (long long)kc * nd + j];
        loc[k] += w * v;
      }
    }
    const double psi = c->ops[c->op_of[kc]].int_psi;
    for (int k = 0; k < neq; ++k) {
      const double ex = loc[k] / psi;
      maxF[k] = std::fabs(ume[k]) > maxF[k] ? std::fabs(ume[k]) : maxF[k];
      sumD[k] += std::fabs(ume[k] - ex);
    }
  }
  const double Ck = 0.03, eps = 1e-6;
  for (int k = 0; k < neq; ++k)
    val[k] = (std::fabs(maxF[k]) < eps && std::fabs(sumD[k]) < eps)
                 ? 1.0
                 : std::min(1.0, Ck * maxF[k] / (sumD[k] + eps));
}

// LimiterMultiplier::linearize, limiter_multiplier.cpp:101-178: every
// variable becomes mean + (reference-space gradient at the centre) . (x_j - c)
// at the points of the element rule of order p+1 (the nodes for p = 1, the
// only order where that rule has nd points).
void linearize(const ref_ctx* c, const double* um, double* el) {
  const int nd = c->nd, neq = c->neq, dim = c->dim;
  const double cen[3] = {0.5, 0.5, 0.5};
  double dphi[125 * 3];
  c->fe.dshape(cen, dphi);
  const Rule r = rule_geom(c->geom, c->p + 1);
  for (int k = 0; k < neq; ++k) {
    double g[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d)
      for (int j = 0; j < nd; ++j) g[d] += el[k * nd + j] * dphi[j * dim + d];
    for (int j = 0; j < nd; ++j) {
      const double* ip = &r.x[j * dim];
      double v = um[k] - g[0] * (cen[0] - ip[0]) - g[1] * (cen[1] - ip[1]);
      if (dim == 3) v -= g[2] * (cen[2] - ip[2]);
      el[k * nd + j] = v;
    }
  }
}

// Limiter::update, limiter.cpp:22-94, with IndicatorBJ::checkDiscontinuity
// (indicator_bj.cpp:88-200), updateYMin (15-86), LimiterMultiplier::limit
// (limiter_multiplier.cpp:12-99), LimiterFinDiff::limit (limiter_findiff.cpp:3-33).
int ref_limit(ref_ctx* c, double* x) {
  const int nd = c->nd, neq = c->neq, dim = c->dim, ne = c->ne;
  if ((c->quirks & 2) && c->lim == 1 && c->geom != REF_GEOM_TRIANGLE && c->p != 1) {
    c->err = "linearize needs order 1 (its rule has fewer points than nodes)";
    return REF_ERR_INVALID;
  }
  const long long ND = c->ndofs;
  c->means.assign((size_t)ne * neq, 0.0);
  means_of(c, x, c->means.data());
  c->xnew.assign(x, x + (size_t)ND * neq);  // xNew = x
  const double* mean = c->means.data();
  const Rule& rl = c->lrule;  // indicator_bj.cpp:150, fixed order 2
  int nverts = c->nvpe;
#pragma omp parallel for schedule(static) num_threads(nthreads())
  for (int e = 0; e < ne; ++e) {
    double el[5 * 125];
    for (int k = 0; k < neq; ++k)
      for (int j = 0; j < nd; ++j) el[k * nd + j] = x[k * ND + (long long)e * nd + j];
    double yMin[5], elind[5];
    double minValue;
    if (c->ind == 0) {  // IndicatorNowhere
      for (int k = 0; k < neq; ++k) elind[k] = 1.0;
      minValue = 1.0;
    } else if (c->ind == 1) {  // IndicatorEverywhere
      for (int k = 0; k < neq; ++k) elind[k] = 0.0;
      minValue = 0.0;
    } else if (c->ind == 3) {  // IndicatorShu (FinDiff only)
      shu_indicator(c, x, mean, e, elind);
      minValue = 1.0;
    } else {
      double mI[5], MI[5], um[5];
      for (int k = 0; k < neq; ++k) {
        mI[k] = 1e9;
        MI[k] = -1e9;
        yMin[k] = 1e9;
      }
      // stencil: the cell itself, then ElementToElementTable neighbours
      auto upd = [&](int kc) {
        for (int k = 0; k < neq; ++k) {
          double v = mean[k * (long long)ne + kc];
          mI[k] = v < mI[k] ? v : mI[k];
          MI[k] = v > MI[k] ? v : MI[k];
        }
      };
      upd(e);
      for (int nb : c->el_el[e]) upd(nb);
      for (int k = 0; k < neq; ++k) um[k] = mean[k * (long long)ne + e];
      double shape[125];
      for (int lf = 0; lf < c->nfpe; ++lf) {
        int fid = c->elem_face[(size_t)e * c->nfpe + lf];
        const Face& f = c->faces[fid];
        // boundary faces are not in the stencil; a master face of hanging
        // faces is (limiter.cpp:158-161, infoNC >= 0), at the cell's own points
        if (f.e2 < 0 && !f.master) continue;
        // the cell's own local face: Loc1 if Elem1 == iCell, else Loc2
        for (int q = 0; q < rl.n; ++q) {
          double ip1[3], ip2[3], nor[3];
          face_point(c, f, &rl.x[q * rl.dim], ip1, ip2, nor);
          const double* eip = (f.e1 == e) ? ip1 : ip2;
          c->fe.shape(eip, shape);
          for (int k = 0; k < neq; ++k) {
            double v = 0;
            for (int j = 0; j < nd; ++j) v += el[k * nd + j] * shape[j];
            double diff = v - um[k];
            double yv;
            if (diff > 1e-3)
              yv = (MI[k] - um[k]) / diff;
            else if (diff < -1e-3)
              yv = (mI[k] - um[k]) / diff;
            else
              yv = 1.0;
            if (c->fun == 0) {  // classical BJ, indicator_bj.cpp:66-68
              yMin[k] = yv < yMin[k] ? yv : yMin[k];
              yMin[k] = yMin[k] > 1.0 ? 1.0 : yMin[k];
            } else if (c->fun == 1) {  // Venkatakrishnan, indicator_bj.cpp:70-72
              double yCur = (yv * yv + 2.0 * yv) / (yv * yv + yv + 2.0);
              yMin[k] = yCur < yMin[k] ? yCur : yMin[k];
            } else {  // Michalak (shipped), indicator_bj.cpp:75-79
              double yStar = 1.5;
              double yRel = yv / yStar;
              double yCur = yv < 1.0 ? yv + (3.0 - 2.0 * yStar) * yRel * yRel +
                                           (yStar - 2.0) * yRel * yRel * yRel
                                     : 1.0;
              yMin[k] = yCur < yMin[k] ? yCur : yMin[k];
            }
          }
        }
      }
      for (int k = 0; k < neq; ++k) elind[k] = yMin[k];
      minValue = yMin[0];  // density factor for every variable (Q5)
    }
    double um[5];
    for (int k = 0; k < neq; ++k) um[k] = mean[k * (long long)ne + e];
    if (c->lim == 1) {  // LimiterMultiplier::limit
      int reps = (c->quirks & 1) ? 1 : nd;  // shadowed iDof loop (Q4)
      const bool lin = (c->quirks & 2) && c->geom != REF_GEOM_TRIANGLE;
      for (int k = 0; k < neq; ++k)
        for (int r = 0; r < reps; ++r) {
          if (lin) linearize(c, um, el);  // limiter_multiplier.cpp:29-30
          for (int j = 0; j < nd; ++j) el[k * nd + j] = um[k] + minValue * (el[k * nd + j] - um[k]);
        }
      if (c->last_hope) {
        double shape[125];
        for (int v = 0; v < nverts; ++v) {
          c->fe.shape(ref_vertex(c->geom, v), shape);
          double fv[5];
          for (int k = 0; k < neq; ++k) {
            double s = 0;
            for (int j = 0; j < nd; ++j) s += el[k * nd + j] * shape[j];
            fv[k] = s;
          }
          if (!state_is_physical(c->P, fv))
            for (int k = 0; k < neq; ++k)
              for (int j = 0; j < nd; ++j) el[k * nd + j] = um[k];
        }
      }
    } else {  // LimiterFinDiff::limit: only the last equation's flag counts (Q6)
      bool totalInd = false;
      for (int k = 0; k < neq; ++k) totalInd = elind[k] < 0.999 ? true : false;
      for (int k = 0; k < neq; ++k)
        for (int j = 0; j < nd; ++j) el[k * nd + j] = totalInd ? um[k] : el[k * nd + j];
    }
    for (int k = 0; k < neq; ++k)
      for (int j = 0; j < nd; ++j) c->xnew[k * ND + (long long)e * nd + j] = el[k * nd + j];
  }
  std::memcpy(x, c->xnew.data(), sizeof(double) * (size_t)ND * neq);
  (void)dim;
  return REF_OK;
}

// ExplicitRKLimitedSolver::Step, rk_explicit_limited.cpp:30-82 (MFEM packing
// of the lower-triangular tableau a[]).
int ref_step(ref_ctx* c, double* x, double dt, double* next_mcs) {
  const size_t n = (size_t)c->ndofs * c->neq;
  const int s = c->s;
  c->kbuf.assign(n * s, 0.0);
  c->y.assign(n, 0.0);
  double mcs = 0;
  int st = ref_rhs(c, x, &c->kbuf[0], &mcs);
  if (st) return st;
  for (int l = 0, i = 1; i < s; i++) {
    double* y = c->y.data();
    const double a0 = c->a[l++] * dt;
    for (size_t q = 0; q < n; ++q) y[q] = x[q] + a0 * c->kbuf[q];
    for (int j = 1; j < i; j++) {
      const double aj = c->a[l++] * dt;
      const double* kj = &c->kbuf[n * j];
      for (size_t q = 0; q < n; ++q) y[q] += aj * kj[q];
    }
    ref_limit(c, y);
    st = ref_rhs(c, y, &c->kbuf[n * i], &mcs);
    if (st) return st;
  }
  for (int i = 0; i < s; i++) {
    const double bi = c->b[i] * dt;
    const double* ki = &c->kbuf[n * i];
    for (size_t q = 0; q < n; ++q) x[q] += bi * ki[q];
  }
  ref_limit(c, x);
  if (next_mcs) *next_mcs = mcs;
  return REF_OK;
}

// The time loop of main.cpp:509-553,701-733 from time t with the next dt
// known (ref_run after its initial limit and dt; ref_run_continue).
static int run_loop(ref_ctx* c, double* x, double t, double dt, double t_end, double cfl,
                    int dt_mode, int max_steps, int* steps_out, double* t_out, double* dt_out,
                    double* sum_dt_out) {
  const double hmin = (dt_mode == 0) ? ref_hmin(c) : 0.0;
  double sum_dt = 0.0;
  int ti = 0;
  bool done = false;
  while (!done) {
    double dt_real = std::min(dt, t_end - t);
    double mcs = 0;
    int st = ref_step(c, x, dt_real, &mcs);
    if (st) return st;
    sum_dt += dt_real;
    if (dt_mode == 0) dt = cfl * hmin / mcs / (2 * c->p + 1);
    if (!std::isfinite(dt) || !(dt > 0.0) || (t_end < 1e20 && dt < 1e-14 * t_end)) {
      c->err = "non-finite or vanishing CFL time step";
      return REF_ERR_UNPHYSICAL;
    }
    t += dt;
    ti++;
    done = (t >= t_end - 1e-8 * dt);
    if (max_steps > 0 && ti >= max_steps) break;
  }
  if (steps_out) *steps_out = ti;
  if (t_out) *t_out = t;
  if (dt_out) *dt_out = dt;
  if (sum_dt_out) *sum_dt_out = sum_dt;
  return REF_OK;
}

int ref_run(ref_ctx* c, double* x, double t_end, double cfl, double dt0, int dt_mode,
            int max_steps, int* steps_out, double* t_out, double* dt_out, double* sum_dt_out) {
  // The projected initial state is limited once before the initial dt and the
  // loop (main.cpp:264-265, `l->update(sol)` after loadInitialSolution).
  if (!(c->solver_quirks & 2)) {
    int st = ref_limit(c, x);
    if (st) return st;
  }
  double dt = dt0;
  if (dt_mode != 2) {
    double mcs;
    int st = ref_face_speed(c, x, &mcs);
    if (st) return st;
    dt = cfl * ref_hmin(c) / mcs / (2 * c->p + 1);
  }
  return run_loop(c, x, 0.0, dt, t_end, cfl, dt_mode, max_steps, steps_out, t_out, dt_out,
                  sum_dt_out);
}

// The loop continued at time t0 with the next dt known: the reference's
// restart (main.cpp:461-490, t and dt from the restart frame), without the
// initial limit and the initial dt.
int ref_run_continue(ref_ctx* c, double* x, double t0, double dt, double t_end, double cfl,
                     int dt_mode, int max_steps, int* steps_out, double* t_out, double* dt_out,
                     double* sum_dt_out) {
  if (!(dt > 0.0)) {
    c->err = "non-positive dt";
    return REF_ERR_INVALID;
  }
  return run_loop(c, x, t0, dt, t_end, cfl, dt_mode, max_steps, steps_out, t_out, dt_out,
                  sum_dt_out);
}

// Discretely conserved totals: sum_e sum_j (int phi_j) u_j per equation.
int ref_totals(ref_ctx* c, const double* x, double* totals) {
  const int nd = c->nd, neq = c->neq;
  const long long ND = c->ndofs;
  for (int k = 0; k < neq; ++k) {
    long double s = 0;
    for (int e = 0; e < c->ne; ++e) {
      const ElemOps& o = c->ops[c->op_of[e]];
      for (int j = 0; j < nd; ++j) s += (long double)o.M0[j] * x[k * ND + (long long)e * nd + j];
    }
    totals[k] = (double)s;
  }
  return REF_OK;
}

// ComputeTotalEnergy, check_total_energy.cpp:3-62 (rule order p+1, whose
// points coincide with the nodes for Q1 quads/hexes).
double ref_total_energy(ref_ctx* c, const double* x) {
  const int nd = c->nd, neq = c->neq;
  const long long ND = c->ndofs;
  Rule r = rule_geom(c->geom, c->p + 1);
  if (r.n < nd) return NAN;
  double tot = 0;
  for (int e = 0; e < c->ne; ++e) {
    double te = 0;
    for (int j = 0; j < nd; ++j) te += r.w[j] * x[(neq - 1) * ND + (long long)e * nd + j];
    tot += te * c->ops[c->op_of[e]].detJ_c;
  }
  return tot;
}

int ref_pointwise(ref_ctx* c, int what, int n, const double* u1, const double* u2,
                  const double* nor, double* out) {
  const int neq = c->neq, dim = c->dim;
  const Phys& P = c->P;
  for (int i = 0; i < n; ++i) {
    double s1[5], s2[5];
    for (int k = 0; k < neq; ++k) {
      s1[k] = u1[i * neq + k];
      s2[k] = u2 ? u2[i * neq + k] : 0.0;
    }
    if (what == 0) {
      double* o = out + (size_t)i * 4;
      o[0] = pressure(P, s1);
      o[1] = sound_speed(P, s1);
      o[2] = max_char_speed_of(P, s1);
      o[3] = state_is_physical(P, s1) ? 1.0 : 0.0;
    } else if (what == 1) {
      flux_full(P, s1, out + (size_t)i * neq * dim);
    } else if (what == 2 || what == 3) {
      rotate(dim, s1, &nor[i * dim]);
      rotate(dim, s2, &nor[i * dim]);
      if (what == 2)
        toro_speeds(P, s1, s2, out + (size_t)i * neq);
      else
        einfeldt_speeds(P, s1, s2, out + (size_t)i * neq);
    } else {
      c->err = "unknown pointwise quantity";
      return REF_ERR_INVALID;
    }
  }
  return REF_OK;
}

int ref_riemann(ref_ctx* c, int n, const double* u1, const double* u2, const double* nor,
                double* flux, double* speed) {
  const int neq = c->neq, dim = c->dim;
  int st = REF_OK;
  for (int i = 0; i < n; ++i) {
    double s1[5], s2[5];
    for (int k = 0; k < neq; ++k) {
      s1[k] = u1[i * neq + k];
      s2[k] = u2[i * neq + k];
    }
    speed[i] = rs_eval(c->P, c->rs, c->avg, s1, s2, &nor[i * dim], &flux[i * neq]);
    if (speed[i] < 0) st = REF_ERR_UNPHYSICAL;
  }
  return st;
}

}  // extern "C"
