// Reference-element basis and tables (host).
#pragma once

#include <vector>

#include "rkdg_common.h"

namespace rkdg {

extern const double kRefVert[3][8][3];  // [geom slot][vertex][xyz]
extern const int kFaceVert[3][6][4];    // MFEM local face vertex lists
int geom_slot(int geom);                // 2 -> 0 (triangle), 3 -> 1 (square), 5 -> 2 (cube)

// Nodal Gauss-Legendre L2 basis of DG_FECollection(p, dim).
struct Basis {
  int geom, p, dim = 0, nd = 0, n1 = 0;
  std::vector<double> nodes;  // nd*dim
  std::vector<double> x1;     // 1D GL nodes (tensor elements)
  std::vector<int> ex, ey;    // triangle monomials
  std::vector<double> cinv;   // triangle Vandermonde inverse
  Basis(int geom, int p);
  void eval(const double* xi, double* phi, double* dphi) const;
};

struct FacePoint {
  int lf, q;
  double xi[3];  // element reference coordinates
  double s[2];   // face parameter
};

void face_to_elem(int geom, int lf, const double* s, double* xi);
// The cell-mean rule (order p + OrderW, averager.cpp:104): reference points
// x[n*dim] and weights w[n].
void mean_rule(int geom, int p, std::vector<double>& x, std::vector<double>& w);
bool build_ref_tables(int geom, int p, RefTables& T, std::vector<FacePoint>* fpts);

}  // namespace rkdg
