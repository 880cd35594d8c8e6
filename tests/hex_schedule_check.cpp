// Host check of the shared-face hexahedral schedules (rkdg_hexsched.cpp):
// reads a mesh's face tables from a binary file, builds the schedules and
// verifies that every slot visits each of its faces in exactly one round,
// that both sides of a face inside a CTA share the round, that every face
// side is evaluated exactly once, that a round marked with one normal axis
// visits only faces of that axis (on both sides) and that the lists stay
// within their arrays.  Prints one JSON line.
//
// Input: int32 ne, int32 nvpe, float64 coords[ne*nvpe*3], int32 fnbr[6*ne],
// int32 fcode[6*ne].
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "rkdg_hexsched.h"

using namespace rkdg;

static int axis_of(int lf) { return lf == 0 || lf == 5 ? 2 : (lf == 1 || lf == 3 ? 1 : 0); }

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
  std::vector<HexTeamSched> hs;
  int mr = 0;
  if (!build_hex_sched(ne, nvpe, X.data(), fnbr, fcode, hs, &mr)) {
    printf("{\"ok\": true, \"built\": false}\n");
    return 0;
  }
  const int NS = RKDG_TEAM_SLOTS, NONE = 0xFF;
  if ((int)hs.size() != (ne + NS - 1) / NS) return fail("cta count");
  std::vector<int> seen(ne, 0), evals((size_t)6 * ne, 0);
  long long inside = 0, jobs = 0, job_warps = 0, flux_iters = 0, rounds = 0, mixed = 0;
  for (size_t b = 0; b < hs.size(); ++b) {
    const HexTeamSched& S = hs[b];
    const int nel = ne - (int)b * NS < NS ? ne - (int)b * NS : NS;
    if (S.nr < 1 || S.nr > RKDG_TEAM_MAX_ROUNDS) return fail("rounds", b);
    for (int s = 0; s < NS; ++s) {
      if (s < nel) {
        if (S.el[s] < 0 || S.el[s] >= ne) return fail("slot element", b);
        seen[S.el[s]]++;
      } else if (S.el[s] != -1) {
        return fail("unused slot", b);
      }
      for (int r = S.nr; r < RKDG_TEAM_MAX_ROUNDS; ++r)
        if (S.rlf[s][r] != NONE) return fail("face past the last round", b);
    }
    for (int s = 0; s < nel; ++s) {
      int cnt[6] = {0, 0, 0, 0, 0, 0};
      const int e = S.el[s];
      for (int r = 0; r < S.nr; ++r) {
        const int lf = S.rlf[s][r];
        if (lf == NONE) continue;
        if (lf > 5) return fail("local face", b);
        cnt[lf]++;
        const int p = S.part[s][lf];
        if (p == NONE) {
          if (fnbr[(size_t)lf * ne + e] >= 0) {
            // the neighbour is outside the CTA
            for (int t = 0; t < nel; ++t)
              if (S.el[t] == fnbr[(size_t)lf * ne + e]) return fail("missed partner", b);
          }
          continue;
        }
        if (p >= nel) return fail("partner slot", b);
        if (S.el[p] != fnbr[(size_t)lf * ne + e]) return fail("partner element", b);
        if (S.rlf[p][r] != (fcode[(size_t)lf * ne + e] & 7)) return fail("partner round", b);
        inside++;
      }
      for (int lf = 0; lf < 6; ++lf)
        if (cnt[lf] != 1) return fail("face visits", e);
    }
    for (int r = 0; r < S.nr; ++r) {
      if (S.nfl[r] > NS || S.njb[r] > NS) return fail("list length", b);
      rounds++;
      if (S.rax[r] < 0) {
        mixed++;
      } else {
        if (S.rax[r] > 2) return fail("round axis", b);
        for (int s = 0; s < nel; ++s) {
          const int lf = S.rlf[s][r];
          if (lf == NONE) continue;
          const int e = S.el[s];
          if (axis_of(lf) != S.rax[r]) return fail("face off the round axis", b);
          if (fnbr[(size_t)lf * ne + e] >= 0 && axis_of(fcode[(size_t)lf * ne + e] & 7) != S.rax[r])
            return fail("face across off the round axis", b);
        }
      }
      for (int i = 0; i < S.nfl[r]; ++i) {
        const unsigned d = S.fd[r][i];
        const int s = d & 31;
        if (s >= nel) return fail("flux slot", b);
        const int lf = S.rlf[s][r];
        if (lf == NONE || (int)((d >> 5) & 7) != lf) return fail("flux face", b);
        const int e = S.el[s];
        const int code = fcode[(size_t)lf * ne + e];
        const unsigned prt = S.part[s][lf] == NONE ? 31u : S.part[s][lf];
        if (((d >> 8) & 31) != prt || ((d >> 13) & 1) != (unsigned)((code >> 3) & 1) ||
            ((d >> 14) & 7) != (unsigned)(code & 7) || ((d >> 17) & 7) != (unsigned)((code >> 4) & 7) ||
            ((d >> 20) & 1) != (unsigned)(fnbr[(size_t)lf * ne + e] >= 0))
          return fail("flux descriptor", b);
        evals[(size_t)lf * ne + e]++;
        const int p = S.part[s][lf];
        if (p != NONE) {
          if ((fcode[(size_t)lf * ne + e] >> 3) & 1) return fail("Elem2 evaluates", b);
          evals[(size_t)(fcode[(size_t)lf * ne + e] & 7) * ne + S.el[p]]++;
        }
      }
      for (int i = 0; i < S.njb[r]; ++i) {
        const int s = S.jb[r][i];
        if (s >= nel) return fail("job slot", b);
        const int lf = S.rlf[s][r];
        if (lf == NONE || S.part[s][lf] != NONE || fnbr[(size_t)lf * ne + S.el[s]] < 0)
          return fail("job", b);
        jobs++;
      }
      job_warps += (S.njb[r] * 5 + 31) / 32;
      flux_iters += (S.nfl[r] * 16 + 31) / 32;
    }
  }
  for (int e = 0; e < ne; ++e)
    if (seen[e] != 1) return fail("element slots", e);
  for (size_t i = 0; i < evals.size(); ++i)
    if (evals[i] != 1) return fail("face side evaluations", (long long)i);
  printf("{\"ok\": true, \"built\": true, \"ctas\": %zu, \"max_rounds\": %d, \"inside_sides\": %lld, "
         "\"jobs\": %lld, \"job_warps_per_cta\": %.3f, \"flux_warp_iters_per_cta\": %.3f, "
         "\"rounds\": %lld, \"mixed_rounds\": %lld}\n",
         hs.size(), mr, inside, jobs, (double)job_warps / hs.size(), (double)flux_iters / hs.size(),
         rounds, mixed);
  return 0;
}
