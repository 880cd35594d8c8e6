// Hanging faces of nonconforming meshes (host).
//
// The reference's meshes are nonconforming (EnsureNCMesh,
// case_manager.cpp:269) and its AMR (main.cpp:564-696) leaves hanging
// vertices: a coarse element's face (the master) is split on the other side
// into the faces of several finer elements (the slaves).  The element-vertex
// description an adapter uploads shows these as faces that no second element
// shares and that no boundary element lists.  This file pairs each slave
// with its master geometrically: the slave's corners, mapped into the
// reference space of an element across it, lie on one of that element's
// faces.  A uniform grid of cells about one lone-face diameter wide keeps
// the search linear in the number of lone faces.  Masters must be covered
// by their slaves' measures exactly (to rounding), which rejects holes and
// faces across periodic seams of a partly refined mesh.
#include "rkdg_ncmesh.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <unordered_map>

#include "rkdg_refelem.h"

namespace rkdg {

void affine_inverse(int dim, const double* X0, const double* J, const double* x, double* xi) {
  double d[3] = {0, 0, 0};
  for (int i = 0; i < dim; ++i) d[i] = x[i] - X0[i];
  if (dim == 2) {
    const double det = J[0] * J[3] - J[1] * J[2];
    xi[0] = (J[3] * d[0] - J[1] * d[1]) / det;
    xi[1] = (-J[2] * d[0] + J[0] * d[1]) / det;
    xi[2] = 0.0;
    return;
  }
  // Cramer's rule, column by column
  auto det3 = [](const double* a, const double* b, const double* c) {
    return a[0] * (b[1] * c[2] - b[2] * c[1]) - a[1] * (b[0] * c[2] - b[2] * c[0]) +
           a[2] * (b[0] * c[1] - b[1] * c[0]);
  };
  double c0[3], c1[3], c2[3];
  for (int i = 0; i < 3; ++i) c0[i] = J[i * 3], c1[i] = J[i * 3 + 1], c2[i] = J[i * 3 + 2];
  const double det = det3(c0, c1, c2);
  xi[0] = det3(d, c1, c2) / det;
  xi[1] = det3(c0, d, c2) / det;
  xi[2] = det3(c0, c1, d) / det;
}

bool classify_nc_faces(int geom, int dim, int nvpe, const double* elem_coords,
                       const std::vector<double>& Jall, const std::vector<double>& fmeas, int ne,
                       const std::vector<NcFace>& lone, std::vector<NcSlave>& slaves,
                       std::string& err) {
  slaves.clear();
  const int L = (int)lone.size();
  if (L == 0) return true;
  const int gs = geom_slot(geom), nvf = dim == 2 ? 2 : 4;
  auto corner = [&](const NcFace& f, int k, double* x) {
    const int v = kFaceVert[gs][f.lf][k];
    for (int i = 0; i < dim; ++i) x[i] = elem_coords[((size_t)f.e * nvpe + v) * dim + i];
  };
  // bounding boxes and the cell grid
  std::vector<double> lo((size_t)L * 3, 0.0), hi((size_t)L * 3, 0.0), diam(L, 0.0);
  double org[3] = {1e300, 1e300, 1e300};
  for (int a = 0; a < L; ++a) {
    for (int i = 0; i < 3; ++i) lo[a * 3 + i] = 1e300, hi[a * 3 + i] = -1e300;
    for (int k = 0; k < nvf; ++k) {
      double x[3] = {0, 0, 0};
      corner(lone[a], k, x);
      for (int i = 0; i < dim; ++i) {
        lo[a * 3 + i] = std::min(lo[a * 3 + i], x[i]);
        hi[a * 3 + i] = std::max(hi[a * 3 + i], x[i]);
      }
    }
    for (int i = 0; i < dim; ++i) {
      diam[a] = std::max(diam[a], hi[a * 3 + i] - lo[a * 3 + i]);
      org[i] = std::min(org[i], lo[a * 3 + i]);
    }
  }
  std::vector<double> ds(diam);
  std::nth_element(ds.begin(), ds.begin() + L / 2, ds.end());
  const double h = ds[L / 2] > 0 ? ds[L / 2] : 1.0;
  auto cell_of = [&](const double* x, int* c) {
    for (int i = 0; i < 3; ++i) c[i] = i < dim ? (int)std::floor((x[i] - org[i]) / h) : 0;
  };
  auto key_of = [](const int* c) {
    return ((long long)(c[0] & 0xFFFFF) << 40) | ((long long)(c[1] & 0xFFFFF) << 20) | (long long)(c[2] & 0xFFFFF);
  };
  std::unordered_map<long long, std::vector<int>> grid;
  for (int a = 0; a < L; ++a) {
    int c0[3], c1[3];
    double l[3], u[3];
    for (int i = 0; i < 3; ++i) l[i] = lo[a * 3 + i] - 1e-9 * h, u[i] = hi[a * 3 + i] + 1e-9 * h;
    cell_of(l, c0);
    cell_of(u, c1);
    long long span = 1;
    for (int i = 0; i < dim; ++i) span *= (long long)(c1[i] - c0[i] + 1);
    if (span > 4096) {
      err = "nonconforming face much larger than its neighbours (more than 64 levels apart)";
      return false;
    }
    int c[3];
    for (c[2] = c0[2]; c[2] <= c1[2]; ++c[2])
      for (c[1] = c0[1]; c[1] <= c1[1]; ++c[1])
        for (c[0] = c0[0]; c[0] <= c1[0]; ++c[0]) grid[key_of(c)].push_back(a);
  }
  std::vector<double> covered(L, 0.0);
  std::vector<char> is_slave(L, 0);
  const double tol = 1e-9;
  for (int a = 0; a < L; ++a) {
    const NcFace& S = lone[a];
    double cen[3] = {0, 0, 0};
    double xs[4][3];
    for (int k = 0; k < nvf; ++k) {
      corner(S, k, xs[k]);
      for (int i = 0; i < dim; ++i) cen[i] += xs[k][i] / nvf;
    }
    int c[3];
    cell_of(cen, c);
    auto it = grid.find(key_of(c));
    if (it == grid.end()) continue;
    for (int b : it->second) {
      const NcFace& Mf = lone[b];
      if (b == a || Mf.e == S.e ||
          !(fmeas[(size_t)Mf.lf * ne + Mf.e] > fmeas[(size_t)S.lf * ne + S.e] * (1 + 1e-9)))
        continue;
      const double* X0 = elem_coords + (size_t)Mf.e * nvpe * dim;
      const double* J = &Jall[(size_t)Mf.e * 9];
      // the master face in its element's reference space: r0 + s (r1 - r0) + t (r3 - r0)
      const double* r0 = kRefVert[gs][kFaceVert[gs][Mf.lf][0]];
      const double* r1 = kRefVert[gs][kFaceVert[gs][Mf.lf][1]];
      const double* r3 = kRefVert[gs][kFaceVert[gs][Mf.lf][nvf - 1]];
      bool on = true;
      for (int k = 0; k < nvf && on; ++k) {
        double xi[3];
        affine_inverse(dim, X0, J, xs[k], xi);
        double e0[3] = {0, 0, 0}, e1[3] = {0, 0, 0}, w[3] = {0, 0, 0};
        double s = 0, t = 0, n0 = 0, n1 = 0;
        for (int i = 0; i < dim; ++i) {
          e0[i] = r1[i] - r0[i];
          e1[i] = dim == 3 ? r3[i] - r0[i] : 0.0;
          w[i] = xi[i] - r0[i];
          s += w[i] * e0[i];
          n0 += e0[i] * e0[i];
          t += w[i] * e1[i];
          n1 += e1[i] * e1[i];
        }
        s /= n0;
        t = dim == 3 ? t / n1 : 0.0;
        double off = 0;
        for (int i = 0; i < dim; ++i) off = std::max(off, std::fabs(w[i] - s * e0[i] - t * e1[i]));
        on = off < tol && s > -tol && s < 1 + tol && t > -tol && t < 1 + tol;
      }
      if (!on) continue;
      slaves.push_back({S.e, S.lf, Mf.e, Mf.lf});
      is_slave[a] = 1;
      covered[b] += fmeas[(size_t)S.lf * ne + S.e];
      break;
    }
  }
  for (int a = 0; a < L; ++a) {
    if (is_slave[a]) continue;
    const double m = fmeas[(size_t)lone[a].lf * ne + lone[a].e];
    if (!(std::fabs(covered[a] - m) <= 1e-9 * m)) {
      char buf[160];
      std::snprintf(buf, sizeof buf,
                    "face %d of element %d has no neighbour, no boundary element and no "
                    "hanging faces covering it",
                    lone[a].lf, lone[a].e);
      err = buf;
      return false;
    }
  }
  return true;
}

}  // namespace rkdg
