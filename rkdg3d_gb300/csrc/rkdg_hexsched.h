// Host construction of the shared-face hexahedral kernel's per-CTA schedules.
#pragma once

#include <vector>

#include "rkdg_common.h"

namespace rkdg {

// Groups the ne hexahedra into CTAs of RKDG_TEAM_SLOTS consecutive elements
// of the Morton order of their centres and colours each CTA's faces into
// rounds: the two sides of a face inside the CTA share a round, an element
// visits one face per round.  coords: each element's nvpe corners (dim 3);
// fnbr / fcode: [6][ne] face tables (fnbr >= 0 for an interior face).
// Returns false when some CTA would need more than RKDG_TEAM_MAX_ROUNDS
// rounds (the kernel is then unavailable for the mesh).
bool build_hex_sched(int ne, int nvpe, const double* coords, const std::vector<int>& fnbr,
                     const std::vector<int>& fcode, std::vector<HexTeamSched>& out,
                     int* max_rounds);

// Tiles of the face-once hexahedral kernel (HexTile): runs of RKDG_TILE_E
// elements of the same Morton order, with their per-axis face evaluations and
// halo lists.  fnbr: topological neighbour (>= 0) or < 0 for a face without
// an element across (boundary or hanging); fcode as the device table.
// A tile axis has at most 2 * RKDG_TILE_E face sides, so the halo lists always
// fit (RKDG_TILE_HMAX); returns false only on inconsistent face tables.
bool build_hex_tiles(int ne, int nvpe, const double* coords, const std::vector<int>& fnbr,
                     const std::vector<int>& fcode, std::vector<HexTile>& out);

}  // namespace rkdg
