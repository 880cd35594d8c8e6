// Per-CTA schedules of the shared-face hexahedral team kernel (host).
//
// Grouping: elements sorted by the Morton key of their centre (10 bits per
// axis over the mesh's bounding box), cut into runs of RKDG_TEAM_SLOTS.  On a
// structured 2^k mesh a run of 24 is three 2x2x2 octants, so about 40 of its
// 72 face pairs lie inside the CTA.
//
// Rounds: an edge colouring of the CTA's interior-face graph (vertices =
// slots, one edge per face with both elements in the CTA) in which the
// edges at a slot get distinct colours.  A face whose two sides have the
// same normal axis a (in the elements' own frames) is coloured within the
// axis's two rounds 2a, 2a+1; each edge takes a colour free at both ends,
// and when the free colours differ the two-coloured alternating path from
// one end is flipped (Konig's method, exact on bipartite graphs: on a
// consistently oriented structured block every round then visits faces of
// one axis, which the kernel exploits).  Otherwise, or on an odd cycle, the
// same is tried over all colours, then a new colour is opened.  Faces to
// elements outside the CTA and boundary faces then take a free colour of
// their axis where one is left, else any free colour.
#include "rkdg_hexsched.h"

#include <algorithm>
#include <cstdint>
#include <cstring>

namespace rkdg {

namespace {

int face_axis(int lf) { return lf == 0 || lf == 5 ? 2 : (lf == 1 || lf == 3 ? 1 : 0); }

uint32_t spread10(uint32_t v) {  // bits 0..9 -> every third bit
  v &= 0x3FFu;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

// Elements sorted by the Morton key of their centres (10 bits per axis over
// the bounding box of the corners); ties keep element order.
std::vector<std::pair<uint32_t, int>> morton_order(int ne, int nvpe, const double* coords) {
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (long long i = 0; i < (long long)ne * nvpe; ++i)
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], coords[i * 3 + d]);
      hi[d] = std::max(hi[d], coords[i * 3 + d]);
    }
  std::vector<std::pair<uint32_t, int>> key(ne);
  for (int e = 0; e < ne; ++e) {
    uint32_t k = 0;
    for (int d = 0; d < 3; ++d) {
      double c = 0;
      for (int v = 0; v < nvpe; ++v) c += coords[((long long)e * nvpe + v) * 3 + d];
      c /= nvpe;
      const double ext = hi[d] - lo[d];
      const double t = ext > 0 ? (c - lo[d]) / ext : 0.0;
      const int qi = std::min(1023, std::max(0, (int)(t * 1024.0)));
      k |= spread10((uint32_t)qi) << d;
    }
    key[e] = {k, e};
  }
  std::sort(key.begin(), key.end());
  return key;
}

}  // namespace

bool build_hex_sched(int ne, int nvpe, const double* coords, const std::vector<int>& fnbr,
                     const std::vector<int>& fcode, std::vector<HexTeamSched>& out,
                     int* max_rounds) {
  constexpr int NS = RKDG_TEAM_SLOTS, NR = RKDG_TEAM_MAX_ROUNDS, NONE = 0xFF;
  out.clear();
  if (max_rounds) *max_rounds = 0;
  if (ne <= 0) return true;
  const std::vector<std::pair<uint32_t, int>> key = morton_order(ne, nvpe, coords);
  const int ncta = (ne + NS - 1) / NS;
  std::vector<int> grp(ne), slot(ne);
  for (int i = 0; i < ne; ++i) {
    grp[key[i].second] = i / NS;
    slot[key[i].second] = i % NS;
  }
  out.resize(ncta);
  int nr_max = 0;
  for (int b = 0; b < ncta; ++b) {
    HexTeamSched& S = out[b];
    std::memset(&S, 0, sizeof S);
    std::memset(S.rlf, NONE, sizeof S.rlf);
    std::memset(S.part, NONE, sizeof S.part);
    const int nel = std::min(NS, ne - b * NS);
    for (int s = 0; s < NS; ++s) S.el[s] = s < nel ? key[b * NS + s].second : -1;
    int col[NS][6];
    int lfo[NS][6];
    for (int s = 0; s < NS; ++s)
      for (int f = 0; f < 6; ++f) col[s][f] = -1, lfo[s][f] = 0;
    for (int s = 0; s < nel; ++s)
      for (int f = 0; f < 6; ++f) {
        const int e = S.el[s];
        const int nb = fnbr[(size_t)f * ne + e];
        lfo[s][f] = fcode[(size_t)f * ne + e] & 7;
        if (nb >= 0 && grp[nb] == b) S.part[s][f] = (unsigned char)slot[nb];
      }
    auto is_free = [&](int s, int c) {
      for (int f = 0; f < 6; ++f)
        if (col[s][f] == c) return false;
      return true;
    };
    auto set_edge = [&](int s, int f, int c) {
      col[s][f] = c;
      col[S.part[s][f]][lfo[s][f]] = c;
    };
    // Konig step over the colour set [c0, c1): colour edge (u, fu) with a
    // colour free at both ends, flipping one alternating path if needed
    auto konig = [&](int u, int fu, int c0, int c1) -> bool {
      const int v = S.part[u][fu];
      int a = c0, bb = c0;
      while (a < c1 && !is_free(u, a)) ++a;
      while (bb < c1 && !is_free(v, bb)) ++bb;
      if (a >= c1 || bb >= c1) return false;
      if (is_free(v, a)) {
        set_edge(u, fu, a);
        return true;
      }
      if (is_free(u, bb)) {
        set_edge(u, fu, bb);
        return true;
      }
      // flip the a/bb path that starts at v with its a-edge
      std::vector<std::pair<int, int>> path;
      int x = v, cc = a;
      for (;;) {
        int fx = -1;
        for (int f = 0; f < 6; ++f)
          if (col[x][f] == cc && S.part[x][f] != NONE) fx = f;
        if (fx < 0) break;
        const int y = S.part[x][fx];
        path.push_back({x, fx});
        if (y == u) return false;  // odd cycle
        x = y;
        cc = cc == a ? bb : a;
      }
      for (auto& pe : path) set_edge(pe.first, pe.second, col[pe.first][pe.second] == a ? bb : a);
      set_edge(u, fu, a);
      return true;
    };
    // interior faces of the CTA, each once (from its Elem1 side)
    for (int u = 0; u < nel; ++u)
      for (int fu = 0; fu < 6; ++fu) {
        if (S.part[u][fu] == NONE) continue;
        if ((fcode[(size_t)fu * ne + S.el[u]] >> 3) & 1) continue;
        const int v = S.part[u][fu], ax = face_axis(fu);
        if (ax == face_axis(lfo[u][fu]) && konig(u, fu, 2 * ax, 2 * ax + 2)) continue;
        if (konig(u, fu, 0, 6)) continue;
        int c = 6;
        while (!is_free(u, c) || !is_free(v, c)) ++c;
        set_edge(u, fu, c);
      }
    // faces to elements outside the CTA and boundary faces
    for (int s = 0; s < nel; ++s)
      for (int f = 0; f < 6; ++f) {
        if (col[s][f] >= 0) continue;
        const int ax = face_axis(f);
        int c = is_free(s, 2 * ax) ? 2 * ax : (is_free(s, 2 * ax + 1) ? 2 * ax + 1 : 0);
        while (!is_free(s, c)) ++c;
        col[s][f] = c;
      }
    int nr = 0;
    for (int s = 0; s < nel; ++s)
      for (int f = 0; f < 6; ++f) nr = std::max(nr, col[s][f] + 1);
    if (nr > NR) return false;
    S.nr = nr;
    nr_max = std::max(nr_max, nr);
    for (int s = 0; s < nel; ++s)
      for (int f = 0; f < 6; ++f) S.rlf[s][col[s][f]] = (unsigned char)f;
    for (int r = 0; r < nr; ++r) {
      int nf = 0, nj = 0;
      for (int s = 0; s < nel; ++s) {
        const int f = S.rlf[s][r];
        if (f == NONE) continue;
        const int e = S.el[s];
        const bool inside = S.part[s][f] != NONE;
        const bool elem2 = (fcode[(size_t)f * ne + e] >> 3) & 1;
        if (!inside || !elem2) {
          const int code = fcode[(size_t)f * ne + e];
          const unsigned prt = inside ? S.part[s][f] : 31u;
          S.fd[r][nf++] = (unsigned)s | (unsigned)f << 5 | prt << 8 | (unsigned)((code >> 3) & 1) << 13 |
                          (unsigned)(code & 7) << 14 | (unsigned)((code >> 4) & 7) << 17 |
                          (unsigned)(fnbr[(size_t)f * ne + e] >= 0) << 20;
        }
        if (!inside && fnbr[(size_t)f * ne + e] >= 0) S.jb[r][nj++] = (unsigned char)s;
      }
      S.nfl[r] = (unsigned char)nf;
      S.njb[r] = (unsigned char)nj;
      // one normal axis for the round's faces and the faces across them?
      int ax = -2;
      for (int s = 0; s < nel && ax != -1; ++s) {
        const int f = S.rlf[s][r];
        if (f == NONE) continue;
        const int e = S.el[s];
        int a = face_axis(f);
        if (fnbr[(size_t)f * ne + e] >= 0 && face_axis(fcode[(size_t)f * ne + e] & 7) != a) a = -1;
        ax = ax == -2 ? a : (ax == a ? a : -1);
      }
      S.rax[r] = (signed char)(ax < 0 ? -1 : ax);
    }
  }
  if (max_rounds) *max_rounds = nr_max;
  return true;
}

bool build_hex_tiles(int ne, int nvpe, const double* coords, const std::vector<int>& fnbr,
                     const std::vector<int>& fcode, std::vector<HexTile>& out) {
  constexpr int TE = RKDG_TILE_E, HM = RKDG_TILE_HMAX;
  out.clear();
  if (ne <= 0) return true;
  const std::vector<std::pair<uint32_t, int>> key = morton_order(ne, nvpe, coords);
  const int ntile = (ne + TE - 1) / TE;
  std::vector<int> tile(ne), slot(ne);
  for (int i = 0; i < ne; ++i) {
    tile[key[i].second] = i / TE;
    slot[key[i].second] = i % TE;
  }
  // local faces of each normal axis, by side (MFEM hexahedron numbering)
  const int axface[3][2] = {{4, 2}, {1, 3}, {0, 5}};
  out.resize(ntile);
  for (int b = 0; b < ntile; ++b) {
    HexTile& T = out[b];
    std::memset(&T, 0, sizeof T);
    T.nel = std::min(TE, ne - b * TE);
    for (int s = 0; s < TE; ++s) T.el[s] = s < T.nel ? key[(size_t)b * TE + s].second : -1;
    for (int a = 0; a < 3; ++a) {
      int nev = 0, nh = 0;
      for (int s = 0; s < T.nel; ++s)
        for (int sd = 0; sd < 2; ++sd) {
          const int lf = axface[a][sd], e = T.el[s];
          const unsigned fs = 2u * s + sd;
          const int nb = fnbr[(size_t)lf * ne + e];
          const int code = fcode[(size_t)lf * ne + e];
          const unsigned lfo = code & 7, elem2 = (code >> 3) & 1, pid = (code >> 4) & 7;
          if (nb < 0) {  // boundary (condition looked up at launch) or hanging face
            T.ev[a][nev++] = fs | 1u << 14 | (unsigned)lf << 15;
            continue;
          }
          if (tile[nb] == b && face_axis((int)lfo) == a) {
            if (elem2) continue;  // evaluated from the partner's (Elem1) entry
            const unsigned fo = 2u * slot[nb] + (lfo == (unsigned)axface[a][1] ? 1u : 0u);
            T.ev[a][nev++] = fs | fo << 7 | (unsigned)lf << 15 | lfo << 18 | pid << 21;
            continue;
          }
          if (nh >= HM) return false;
          T.hel[a][nh] = nb;
          T.hlf[a][nh] = (unsigned char)lfo;
          const unsigned h = (unsigned)nh++;
          if (!elem2)
            T.ev[a][nev++] = fs | h << 7 | 1u << 13 | (unsigned)lf << 15 | lfo << 18 | pid << 21;
          else
            T.ev[a][nev++] = h | 1u << 6 | fs << 7 | lfo << 15 | (unsigned)lf << 18 | pid << 21 |
                             1u << 24;
        }
      T.nev[a] = nev;
      T.nh[a] = nh;
    }
  }
  return true;
}

}  // namespace rkdg
