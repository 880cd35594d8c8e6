// Host classification of the hanging faces of a nonconforming mesh.
#pragma once

#include <string>
#include <vector>

namespace rkdg {

struct NcFace {
  int e, lf;  // element and local face
};
struct NcSlave {
  int e1, lf1;  // fine element (Elem1) and its local face
  int e2, lf2;  // coarse element (Elem2) owning the master face, and that face
};

// lone: faces no second element shares and no boundary element lists.  Each
// is either a slave -- its corners lie on a face of an element across it --
// or a master fully covered by its slaves (face measures from fmeas[lf][e]).
// Affine elements: x = X0 + J xi with X0 = corner 0 and J[e*9 + i*dim + r].
// Returns false with a message when a lone face is neither.
bool classify_nc_faces(int geom, int dim, int nvpe, const double* elem_coords,
                       const std::vector<double>& Jall, const std::vector<double>& fmeas, int ne,
                       const std::vector<NcFace>& lone, std::vector<NcSlave>& slaves,
                       std::string& err);

// Reference coordinates in element e of the physical point x.
void affine_inverse(int dim, const double* X0, const double* J, const double* x, double* xi);

}  // namespace rkdg
