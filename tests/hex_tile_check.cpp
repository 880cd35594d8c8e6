// Host check of the face-once hexahedral tiles (build_hex_tiles in
// rkdg_hexsched.cpp): reads a mesh's face tables from a binary file, builds
// the tiles and verifies that every element sits in exactly one slot, that on
// every axis each face side of a tile element is the tile side of exactly one
// evaluation, that an evaluation between two tile elements names the face's
// Elem1 and Elem2 sides, local faces and point permutation as the face tables
// do, that a halo names the element and local face across, that boundary
// evaluations sit on faces without an element across, and that the lists stay
// within their arrays.  Prints one JSON line with the face evaluations per
// element and the largest halo list.
//
// Input: int32 ne, int32 nvpe, float64 coords[ne*nvpe*3], int32 fnbr[6*ne],
// int32 fcode[6*ne].
#include <cstdio>
#include <vector>

#include "rkdg_hexsched.h"

using namespace rkdg;

static int axis_of(int lf) { return lf == 0 || lf == 5 ? 2 : (lf == 1 || lf == 3 ? 1 : 0); }
static int side_of(int lf) { return lf == 2 || lf == 3 || lf == 5 ? 1 : 0; }

static int fail(const char* what, long long a = -1) {
  printf("{\"ok\": false, \"error\": \"%s\", \"at\": %lld}\n", what, a);
  return 1;
}

int main(int argc, char** argv) {
  if (argc < 2) return fail("usage");
  FILE* f = fopen(argv[1], "rb");
  if (!f) return fail("open");
  int ne = 0, nvpe = 0;
  if (fread(&ne, 4, 1, f) != 1 || fread(&nvpe, 4, 1, f) != 1) return fail("header");
  std::vector<double> X((size_t)ne * nvpe * 3);
  std::vector<int> fnbr((size_t)6 * ne), fcode((size_t)6 * ne);
  if (fread(X.data(), 8, X.size(), f) != X.size() || fread(fnbr.data(), 4, fnbr.size(), f) != fnbr.size() ||
      fread(fcode.data(), 4, fcode.size(), f) != fcode.size())
    return fail("body");
  fclose(f);
  std::vector<HexTile> tiles;
  if (!build_hex_tiles(ne, nvpe, X.data(), fnbr, fcode, tiles)) {
    printf("{\"ok\": true, \"built\": false}\n");
    return 0;
  }
  const int TE = RKDG_TILE_E;
  if ((int)tiles.size() != (ne + TE - 1) / TE) return fail("tile count");
  std::vector<int> seen(ne, 0);
  long long evals = 0, halos = 0, inside = 0;
  int max_halo = 0;
  for (size_t b = 0; b < tiles.size(); ++b) {
    const HexTile& T = tiles[b];
    const int nel = ne - (int)b * TE < TE ? ne - (int)b * TE : TE;
    if (T.nel != nel) return fail("slots in use", b);
    for (int s = 0; s < TE; ++s) {
      if (s < nel) {
        if (T.el[s] < 0 || T.el[s] >= ne) return fail("slot element", b);
        seen[T.el[s]]++;
      } else if (T.el[s] != -1) {
        return fail("unused slot", b);
      }
    }
    for (int a = 0; a < 3; ++a) {
      if (T.nev[a] < 0 || T.nev[a] > 2 * TE) return fail("evaluation count", b);
      if (T.nh[a] < 0 || T.nh[a] > RKDG_TILE_HMAX) return fail("halo count", b);
      max_halo = T.nh[a] > max_halo ? T.nh[a] : max_halo;
      std::vector<int> got(2 * TE, 0), hused(RKDG_TILE_HMAX, 0);
      for (int j = 0; j < T.nev[a]; ++j) {
        const unsigned d = T.ev[a][j];
        const int ia = d & 63, ib = (d >> 7) & 63, lfa = (d >> 15) & 7, lfb = (d >> 18) & 7;
        const int pid = (d >> 21) & 7;
        const bool ha = (d >> 6) & 1, hb = (d >> 13) & 1, bnd = (d >> 14) & 1, gb = (d >> 24) & 1;
        if (lfa > 5 || lfb > 5) return fail("local face", b);
        if (ha && hb) return fail("two halo sides", b);
        if (gb != ha) return fail("geometry side", b);
        ++evals;
        auto tile_side = [&](int fs, int lf) -> int {  // element of a tile face side
          if (fs >= 2 * nel) return -1;
          if (lf != (fs & 1 ? (a == 0 ? 2 : a == 1 ? 3 : 5) : (a == 0 ? 4 : a == 1 ? 1 : 0))) return -2;
          return T.el[fs >> 1];
        };
        if (bnd) {
          if (ha || hb) return fail("boundary with a halo", b);
          const int e = tile_side(ia, lfa);
          if (e < 0) return fail("boundary side", b);
          if (fnbr[(size_t)lfa * ne + e] >= 0) return fail("boundary face has a neighbour", b);
          got[ia]++;
          continue;
        }
        // Elem1 side (A) and Elem2 side (B)
        int e1, e2;
        if (ha) {
          if (ia >= T.nh[a]) return fail("halo index", b);
          hused[ia]++;
          e1 = T.hel[a][ia];
          if (T.hlf[a][ia] != lfa) return fail("halo local face", b);
        } else {
          e1 = tile_side(ia, lfa);
          if (e1 < 0) return fail("Elem1 side", b);
          got[ia]++;
        }
        if (hb) {
          if (ib >= T.nh[a]) return fail("halo index", b);
          hused[ib]++;
          e2 = T.hel[a][ib];
          if (T.hlf[a][ib] != lfb) return fail("halo local face", b);
        } else {
          e2 = tile_side(ib, lfb);
          if (e2 < 0) return fail("Elem2 side", b);
          got[ib]++;
        }
        if (!ha && !hb) ++inside;
        else ++halos;
        const int c1 = fcode[(size_t)lfa * ne + e1], c2 = fcode[(size_t)lfb * ne + e2];
        if (fnbr[(size_t)lfa * ne + e1] != e2 || fnbr[(size_t)lfb * ne + e2] != e1)
          return fail("face partners", b);
        if ((c1 & 7) != lfb || (c2 & 7) != lfa) return fail("face local faces", b);
        if (((c1 >> 3) & 1) != 0 || ((c2 >> 3) & 1) != 1) return fail("Elem1 / Elem2 order", b);
        if (((c1 >> 4) & 7) != pid) return fail("permutation", b);
        if (!ha && !hb && axis_of(lfb) != a) return fail("in-tile face across axes", b);
      }
      for (int s = 0; s < 2 * nel; ++s)
        if (got[s] != 1) return fail("face side not evaluated exactly once", (long long)b * 64 + s);
      for (int h = 0; h < T.nh[a]; ++h)
        if (hused[h] != 1) return fail("halo used once", b);
      (void)side_of;
    }
  }
  for (int e = 0; e < ne; ++e)
    if (seen[e] != 1) return fail("element slots", e);
  printf("{\"ok\": true, \"built\": true, \"evals_per_element\": %.4f, \"inside_faces\": %lld, "
         "\"halo_faces\": %lld, \"max_halo\": %d}\n",
         (double)evals / ne, inside, halos, max_halo);
  return 0;
}
