// CPU driver for the hanging-face classification of rkdg3d_gb300/csrc/rkdg_ncmesh.cpp,
// used by tests/test_ncmesh.py.  Reads one binary mesh description
//   int32 dim, geom, nvpe, ne, nlone
//   float64 elem_coords[ne][nvpe][dim]
//   float64 J[ne][9]          (J[i * dim + r] = d x_i / d xi_r, corner 0 at xi = 0)
//   float64 fmeas[nfpe][ne]   (face measures)
//   int32 lone[nlone][2]      (element, local face)
// and prints one JSON object: {"ok": true, "slaves": [[e1, lf1, e2, lf2], ...]}
// or {"ok": false, "error": "..."}.
#include <cstdio>
#include <string>
#include <vector>

#include "rkdg_ncmesh.h"

int main(int argc, char** argv) {
  if (argc != 2) {
    std::fprintf(stderr, "usage: %s mesh.bin\n", argv[0]);
    return 2;
  }
  std::FILE* fh = std::fopen(argv[1], "rb");
  if (!fh) return 2;
  int hdr[5];
  if (std::fread(hdr, sizeof(int), 5, fh) != 5) return 2;
  const int dim = hdr[0], geom = hdr[1], nvpe = hdr[2], ne = hdr[3], nlone = hdr[4];
  const int nfpe = geom == 2 ? 3 : (geom == 3 ? 4 : 6);
  std::vector<double> coords((size_t)ne * nvpe * dim), J((size_t)ne * 9), fmeas((size_t)nfpe * ne);
  std::vector<int> lone_raw((size_t)nlone * 2);
  bool ok = std::fread(coords.data(), sizeof(double), coords.size(), fh) == coords.size() &&
            std::fread(J.data(), sizeof(double), J.size(), fh) == J.size() &&
            std::fread(fmeas.data(), sizeof(double), fmeas.size(), fh) == fmeas.size() &&
            std::fread(lone_raw.data(), sizeof(int), lone_raw.size(), fh) == lone_raw.size();
  std::fclose(fh);
  if (!ok) return 2;
  std::vector<rkdg::NcFace> lone(nlone);
  for (int i = 0; i < nlone; ++i) lone[i] = {lone_raw[2 * i], lone_raw[2 * i + 1]};
  std::vector<rkdg::NcSlave> slaves;
  std::string err;
  if (!rkdg::classify_nc_faces(geom, dim, nvpe, coords.data(), J, fmeas, ne, lone, slaves, err)) {
    std::string esc;
    for (char ch : err) esc += (ch == '"' || ch == '\\') ? '\'' : ch;
    std::printf("{\"ok\": false, \"error\": \"%s\"}\n", esc.c_str());
    return 0;
  }
  std::printf("{\"ok\": true, \"slaves\": [");
  for (size_t i = 0; i < slaves.size(); ++i)
    std::printf("%s[%d, %d, %d, %d]", i ? ", " : "", slaves[i].e1, slaves[i].lf1, slaves[i].e2,
                slaves[i].lf2);
  std::printf("]}\n");
  return 0;
}
