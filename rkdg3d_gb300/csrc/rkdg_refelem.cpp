// Reference-element tables of the GB300 RKDG library (host, FP64).
//
// Restates the MFEM behaviour the reference relies on: DG_FECollection(p, dim)
// with its default Gauss-Legendre nodal basis (main.cpp:115), the quadrature
// orders of DomainIntegrator (domain_integrator.cpp:30-32: 2p), MassIntegrator
// (fe_evolution.cpp:58: 2p + OrderW), GetElementAverages (averager.cpp:104:
// p + OrderW), the face rule of FaceIntegrator (face_integrator.cpp:45-58:
// OrderW + 2p, +1 on simplices) and the fixed order-2 face rule of the BJ
// indicator (indicator_bj.cpp:150).
#include "rkdg_refelem.h"

#include <cmath>
#include <cstring>
#include <vector>

namespace rkdg {

namespace {

// Gauss-Legendre nodes/weights on [0,1], ascending.
void gl01(int n, double* x, double* w) {
  for (int i = 0; i < n; ++i) {
    // Newton on P_n from the Tricomi initial guess
    double t = std::cos(M_PI * (4.0 * (n - i) - 1.0) / (4.0 * n + 2.0));
    double dp = 1.0;
    for (int it = 0; it < 64; ++it) {
      double pm = 1.0, p = t;
      for (int k = 2; k <= n; ++k) {
        const double pk = ((2.0 * k - 1.0) * t * p - (k - 1.0) * pm) / k;
        pm = p;
        p = pk;
      }
      if (n == 1) {
        p = t;
        pm = 1.0;
      }
      dp = n * (pm - t * p) / (1.0 - t * t);
      const double dt = p / dp;
      t -= dt;
      if (std::fabs(dt) < 1e-17) break;
    }
    {
      double pm = 1.0, p = t;
      for (int k = 2; k <= n; ++k) {
        const double pk = ((2.0 * k - 1.0) * t * p - (k - 1.0) * pm) / k;
        pm = p;
        p = pk;
      }
      if (n == 1) pm = 1.0;
      dp = n * (pm - t * p) / (1.0 - t * t);
    }
    x[i] = 0.5 * (t + 1.0);
    w[i] = 1.0 / ((1.0 - t * t) * dp * dp);
  }
}

double lag(const std::vector<double>& xs, int i, double y) {
  double v = 1.0;
  for (size_t j = 0; j < xs.size(); ++j)
    if ((int)j != i) v *= (y - xs[j]) / (xs[i] - xs[j]);
  return v;
}
double dlag(const std::vector<double>& xs, int i, double y) {
  double s = 0.0;
  for (size_t m = 0; m < xs.size(); ++m) {
    if ((int)m == i) continue;
    double v = 1.0 / (xs[i] - xs[m]);
    for (size_t j = 0; j < xs.size(); ++j)
      if ((int)j != i && j != m) v *= (y - xs[j]) / (xs[i] - xs[j]);
    s += v;
  }
  return s;
}

bool inv_dense(int n, std::vector<double> A, std::vector<double>& X) {
  X.assign(n * n, 0.0);
  for (int i = 0; i < n; ++i) X[i * n + i] = 1.0;
  for (int c = 0; c < n; ++c) {
    int p = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(A[r * n + c]) > std::fabs(A[p * n + c])) p = r;
    if (A[p * n + c] == 0.0) return false;
    for (int k = 0; k < n; ++k) {
      std::swap(A[p * n + k], A[c * n + k]);
      std::swap(X[p * n + k], X[c * n + k]);
    }
    const double d = 1.0 / A[c * n + c];
    for (int k = 0; k < n; ++k) {
      A[c * n + k] *= d;
      X[c * n + k] *= d;
    }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const double f = A[r * n + c];
      if (f == 0.0) continue;
      for (int k = 0; k < n; ++k) {
        A[r * n + k] -= f * A[c * n + k];
        X[r * n + k] -= f * X[c * n + k];
      }
    }
  }
  return true;
}

struct Pts {
  std::vector<double> x;  // n*dim
  std::vector<double> w;
  int n = 0;
};

Pts seg_rule(int order) {
  Pts r;
  r.n = order / 2 + 1;
  r.x.resize(r.n);
  r.w.resize(r.n);
  gl01(r.n, r.x.data(), r.w.data());
  return r;
}

// Element rule of the given order on the reference element.
Pts elem_rule(int geom, int order) {
  Pts r;
  if (geom == 2) {
    // Conical product Gauss rule, exact to degree 'order'.
    const int n = order / 2 + 2;
    std::vector<double> g(n), gw(n);
    gl01(n, g.data(), gw.data());
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        r.x.push_back(g[i]);
        r.x.push_back(g[j] * (1.0 - g[i]));
        r.w.push_back(gw[i] * gw[j] * (1.0 - g[i]));
      }
    r.n = n * n;
    return r;
  }
  Pts s = seg_rule(order);
  if (geom == 3) {
    for (int j = 0; j < s.n; ++j)
      for (int i = 0; i < s.n; ++i) {
        r.x.push_back(s.x[i]);
        r.x.push_back(s.x[j]);
        r.w.push_back(s.w[i] * s.w[j]);
      }
    r.n = s.n * s.n;
  } else {
    for (int k = 0; k < s.n; ++k)
      for (int j = 0; j < s.n; ++j)
        for (int i = 0; i < s.n; ++i) {
          r.x.push_back(s.x[i]);
          r.x.push_back(s.x[j]);
          r.x.push_back(s.x[k]);
          r.w.push_back(s.w[i] * s.w[j] * s.w[k]);
        }
    r.n = s.n * s.n * s.n;
  }
  return r;
}

// Face (dim-1) rule in the face's own parameter space.
Pts face_rule(int dim, int order) {
  Pts s = seg_rule(order);
  if (dim == 2) return s;
  Pts r;
  for (int j = 0; j < s.n; ++j)
    for (int i = 0; i < s.n; ++i) {
      r.x.push_back(s.x[i]);
      r.x.push_back(s.x[j]);
      r.w.push_back(s.w[i] * s.w[j]);
    }
  r.n = s.n * s.n;
  return r;
}

}  // namespace

const double kRefVert[3][8][3] = {
    {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}},                             // triangle
    {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}},                  // square
    {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},                   // cube
     {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}}};
const int kFaceVert[3][6][4] = {
    {{0, 1}, {1, 2}, {2, 0}},
    {{0, 1}, {1, 2}, {2, 3}, {3, 0}},
    {{3, 2, 1, 0}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}, {4, 5, 6, 7}}};

int geom_slot(int geom) { return geom == 2 ? 0 : (geom == 3 ? 1 : 2); }

Basis::Basis(int geom_, int p_) : geom(geom_), p(p_) {
  if (geom == 2) {
    dim = 2;
    nd = (p + 1) * (p + 2) / 2;
    std::vector<double> op(p + 1), ow(p + 1);
    gl01(p + 1, op.data(), ow.data());
    for (int j = 0; j <= p; ++j)
      for (int i = 0; i + j <= p; ++i) {
        const double w = op[i] + op[j] + op[p - i - j];
        nodes.push_back(op[i] / w);
        nodes.push_back(op[j] / w);
      }
    for (int b = 0; b <= p; ++b)
      for (int a = 0; a + b <= p; ++a) {
        ex.push_back(a);
        ey.push_back(b);
      }
    std::vector<double> V(nd * nd);
    for (int r = 0; r < nd; ++r)
      for (int m = 0; m < nd; ++m)
        V[r * nd + m] = std::pow(nodes[2 * r], ex[m]) * std::pow(nodes[2 * r + 1], ey[m]);
    inv_dense(nd, V, cinv);
  } else {
    dim = geom == 3 ? 2 : 3;
    n1 = p + 1;
    x1.resize(n1);
    std::vector<double> w(n1);
    gl01(n1, x1.data(), w.data());
    nd = dim == 2 ? n1 * n1 : n1 * n1 * n1;
    for (int j = 0; j < nd; ++j) {
      nodes.push_back(x1[j % n1]);
      nodes.push_back(x1[(j / n1) % n1]);
      if (dim == 3) nodes.push_back(x1[j / (n1 * n1)]);
    }
  }
}

void Basis::eval(const double* xi, double* phi, double* dphi) const {
  if (geom == 2) {
    for (int j = 0; j < nd; ++j) {
      phi[j] = 0.0;
      if (dphi) dphi[2 * j] = dphi[2 * j + 1] = 0.0;
    }
    for (int m = 0; m < nd; ++m) {
      const double mv = std::pow(xi[0], ex[m]) * std::pow(xi[1], ey[m]);
      const double mx = ex[m] ? ex[m] * std::pow(xi[0], ex[m] - 1) * std::pow(xi[1], ey[m]) : 0.0;
      const double my = ey[m] ? ey[m] * std::pow(xi[0], ex[m]) * std::pow(xi[1], ey[m] - 1) : 0.0;
      for (int j = 0; j < nd; ++j) {
        const double c = cinv[m * nd + j];
        phi[j] += c * mv;
        if (dphi) {
          dphi[2 * j] += c * mx;
          dphi[2 * j + 1] += c * my;
        }
      }
    }
    return;
  }
  for (int j = 0; j < nd; ++j) {
    const int ix = j % n1, iy = (j / n1) % n1, iz = j / (n1 * n1);
    const double a = lag(x1, ix, xi[0]), b = lag(x1, iy, xi[1]);
    const double c = dim == 3 ? lag(x1, iz, xi[2]) : 1.0;
    phi[j] = a * b * c;
    if (dphi) {
      const double da = dlag(x1, ix, xi[0]), db = dlag(x1, iy, xi[1]);
      const double dc = dim == 3 ? dlag(x1, iz, xi[2]) : 0.0;
      dphi[j * dim + 0] = da * b * c;
      dphi[j * dim + 1] = a * db * c;
      if (dim == 3) dphi[j * dim + 2] = a * b * dc;
    }
  }
}

// Element-reference coordinates of face parameter s on local face lf.
void mean_rule(int geom, int p, std::vector<double>& x, std::vector<double>& w) {
  const int orderW = geom == 2 ? 0 : (geom == 3 ? 1 : 2);
  Pts r = elem_rule(geom, p + orderW);
  x = r.x;
  w = r.w;
}

void face_to_elem(int geom, int lf, const double* s, double* xi) {
  const int g = geom_slot(geom);
  const int dim = geom == 5 ? 3 : 2;
  double N[4];
  int nv;
  if (dim == 2) {
    N[0] = 1 - s[0];
    N[1] = s[0];
    nv = 2;
  } else {
    N[0] = (1 - s[0]) * (1 - s[1]);
    N[1] = s[0] * (1 - s[1]);
    N[2] = s[0] * s[1];
    N[3] = (1 - s[0]) * s[1];
    nv = 4;
  }
  for (int i = 0; i < 3; ++i) xi[i] = 0.0;
  for (int k = 0; k < nv; ++k)
    for (int i = 0; i < dim; ++i) xi[i] += N[k] * kRefVert[g][kFaceVert[g][lf][k]][i];
}

bool build_ref_tables(int geom, int p, RefTables& T, std::vector<FacePoint>* fpts) {
  std::memset(&T, 0, sizeof(T));
  Basis B(geom, p);
  const int dim = B.dim, nd = B.nd;
  const int g = geom_slot(geom);
  const int orderW = geom == 2 ? 0 : (geom == 3 ? 1 : 2);
  const int nfpe = geom == 2 ? 3 : (geom == 3 ? 4 : 6);
  const int nv = geom == 2 ? 3 : (geom == 3 ? 4 : 8);
  if (nd > RKDG_MAX_ND) return false;
  T.dim = dim;
  T.geom = geom;
  T.p = p;
  T.nd = nd;
  T.nfpe = nfpe;
  T.nv = nv;
  T.n1 = B.n1;
  std::vector<double> phi(nd), dphi(nd * 3);
  // volume operator
  {
    Pts r = elem_rule(geom, 2 * p);
    for (int q = 0; q < r.n; ++q) {
      B.eval(&r.x[q * dim], phi.data(), dphi.data());
      for (int rr = 0; rr < dim; ++rr)
        for (int j = 0; j < nd; ++j)
          for (int m = 0; m < nd; ++m) T.D[rr][j][m] += r.w[q] * phi[m] * dphi[j * dim + rr];
    }
  }
  // reference mass and its inverse
  {
    Pts r = elem_rule(geom, 2 * p + orderW);
    std::vector<double> M(nd * nd, 0.0), Mi;
    for (int q = 0; q < r.n; ++q) {
      B.eval(&r.x[q * dim], phi.data(), nullptr);
      for (int i = 0; i < nd; ++i)
        for (int j = 0; j < nd; ++j) M[i * nd + j] += r.w[q] * phi[i] * phi[j];
    }
    if (!inv_dense(nd, M, Mi)) return false;
    for (int i = 0; i < nd; ++i)
      for (int j = 0; j < nd; ++j) T.Minv[i][j] = Mi[i * nd + j];
  }
  // linearize option of the Multi limiter (limiter_multiplier.cpp:101-178)
  if (geom != 2) {
    const double cen[3] = {0.5, 0.5, 0.5};
    B.eval(cen, phi.data(), dphi.data());
    for (int j = 0; j < nd; ++j)
      for (int d = 0; d < dim; ++d) T.dcen[j][d] = dphi[j * dim + d];
    Pts r = elem_rule(geom, p + 1);
    T.lin_ok = r.n >= nd ? 1 : 0;
    for (int j = 0; j < nd && j < r.n; ++j)
      for (int d = 0; d < dim; ++d) T.xlin[j][d] = r.x[j * dim + d];
  }
  // Shu indicator: extrapolation rule and basis data
  {
    Pts r = elem_rule(geom, p + orderW);
    if (r.n > RKDG_MAX_NQS) return false;
    T.nqs = r.n;
    for (int q = 0; q < r.n; ++q) {
      for (int d = 0; d < dim; ++d) T.xs[q][d] = r.x[q * dim + d];
      T.ws[q] = r.w[q];
    }
    for (int i = 0; i < (int)B.x1.size() && i < 8; ++i) T.x1n[i] = B.x1[i];
    if (geom == 2)
      for (int m = 0; m < nd; ++m) {
        T.tmono[m][0] = B.ex[m];
        T.tmono[m][1] = B.ey[m];
        for (int j = 0; j < nd; ++j) T.tcoef[m][j] = B.cinv[m * nd + j];
      }
  }
  // cell-mean weights
  {
    Pts r = elem_rule(geom, p + orderW);
    double tot = 0.0;
    std::vector<double> m0(nd, 0.0);
    for (int q = 0; q < r.n; ++q) {
      B.eval(&r.x[q * dim], phi.data(), nullptr);
      for (int j = 0; j < nd; ++j) m0[j] += r.w[q] * phi[j];
    }
    for (int j = 0; j < nd; ++j) tot += m0[j];
    for (int j = 0; j < nd; ++j) T.wmean[j] = m0[j] / tot;
  }
  // face points of the right-hand side
  {
    int order = orderW + 2 * p + (geom == 2 ? 1 : 0);
    Pts f = face_rule(dim, order);
    if (f.n > RKDG_MAX_NQF) return false;
    T.nqf = f.n;
    for (int q = 0; q < f.n; ++q) T.wf[q] = f.w[q];
    if (fpts) fpts->clear();
    for (int lf = 0; lf < nfpe; ++lf)
      for (int q = 0; q < f.n; ++q) {
        double xi[3];
        face_to_elem(geom, lf, &f.x[q * (dim - 1)], xi);
        B.eval(xi, phi.data(), nullptr);
        for (int s = 0; s < nd; ++s) T.B[lf][q][s] = phi[s];
        if (fpts) {
          FacePoint fp;
          fp.lf = lf;
          fp.q = q;
          for (int i = 0; i < 3; ++i) fp.xi[i] = xi[i];
          for (int i = 0; i < dim - 1; ++i) fp.s[i] = f.x[q * (dim - 1) + i];
          fpts->push_back(fp);
        }
      }
    // 1D data for tensor kernels: face rule points / weights, basis at ends
    Pts s1 = seg_rule(order);
    T.nq1 = s1.n;
    if (geom != 2) {
      for (int a = 0; a < s1.n; ++a) {
        T.w1d[a] = s1.w[a];
        for (int j = 0; j < B.n1; ++j) T.l1d[a][j] = lag(B.x1, j, s1.x[a]);
      }
      for (int j = 0; j < B.n1; ++j) {
        T.lend[0][j] = lag(B.x1, j, 0.0);
        T.lend[1][j] = lag(B.x1, j, 1.0);
      }
      std::vector<double> gx(B.n1), gw(B.n1);
      gl01(B.n1, gx.data(), gw.data());
      for (int j = 0; j < B.n1; ++j)
        for (int m = 0; m < B.n1; ++m) T.d1[j][m] = gw[m] * dlag(B.x1, j, gx[m]);
      // exact 1D mass matrix (p+2 points) and its inverse
      std::vector<double> gx2(B.n1 + 1), gw2(B.n1 + 1);
      gl01(B.n1 + 1, gx2.data(), gw2.data());
      std::vector<double> M1(B.n1 * B.n1, 0.0), Mi1;
      for (int q = 0; q <= B.n1; ++q)
        for (int i = 0; i < B.n1; ++i)
          for (int j = 0; j < B.n1; ++j) M1[i * B.n1 + j] += gw2[q] * lag(B.x1, i, gx2[q]) * lag(B.x1, j, gx2[q]);
      inv_dense(B.n1, M1, Mi1);
      for (int i = 0; i < B.n1; ++i)
        for (int j = 0; j < B.n1; ++j) T.minv1[i][j] = Mi1[i * B.n1 + j];
      Pts l2 = seg_rule(2);
      for (int a = 0; a < 2; ++a)
        for (int j = 0; j < B.n1; ++j) T.lquad[a][j] = lag(B.x1, j, l2.x[a]);
      for (int j = 0; j < B.n1; ++j) T.w1[j] = gw[j];
    }
    if (geom == 5) {
      // tensor trace tables of the hexahedron faces
      for (int lf = 0; lf < nfpe; ++lf) {
        double xi0[3], xi1[3];
        face_to_elem(geom, lf, &f.x[0], xi0);
        face_to_elem(geom, lf, &f.x[(f.n - 1) * 2], xi1);
        int nax = 0;
        for (int i = 0; i < 3; ++i)
          if (std::fabs(xi0[i] - xi1[i]) < 1e-14) nax = i;
        T.fax[lf] = nax;
        T.fside[lf] = xi0[nax] > 0.5 ? 1 : 0;
        const int t0 = nax == 0 ? 1 : 0, t1 = nax == 2 ? 1 : 2;
        for (int q = 0; q < f.n; ++q) {
          double xi[3];
          face_to_elem(geom, lf, &f.x[q * 2], xi);
          int ia = -1, ib = -1;
          for (int a = 0; a < s1.n; ++a) {
            if (std::fabs(s1.x[a] - xi[t0]) < 1e-12) ia = a;
            if (std::fabs(s1.x[a] - xi[t1]) < 1e-12) ib = a;
          }
          if (ia < 0 || ib < 0) return false;
          T.fab[lf][q] = ia + s1.n * ib;
          for (int i0 = 0; i0 < B.n1; ++i0)
            for (int i1 = 0; i1 < B.n1; ++i1)
              T.B2[lf][q][i0 * B.n1 + i1] = lag(B.x1, i0, xi[t0]) * lag(B.x1, i1, xi[t1]);
        }
      }
    }
  }
  // limiter face points (order 2) and vertices
  {
    Pts f = face_rule(dim, 2);
    T.nql = f.n;
    for (int lf = 0; lf < nfpe; ++lf)
      for (int q = 0; q < f.n; ++q) {
        double xi[3];
        face_to_elem(geom, lf, &f.x[q * (dim - 1)], xi);
        B.eval(xi, phi.data(), nullptr);
        for (int s = 0; s < nd; ++s) T.Bl[lf][q][s] = phi[s];
      }
    for (int v = 0; v < nv; ++v) {
      B.eval(kRefVert[g][v], phi.data(), nullptr);
      for (int s = 0; s < nd; ++s) T.Bv[v][s] = phi[s];
    }
  }
  return true;
}

}  // namespace rkdg
