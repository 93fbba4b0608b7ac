// Multigrid towers: the block list of every MG level and the type of every
// block face inside it (src/SayakaTower.h:15-224, src/SayakaTower.cpp:28-187).
//
// Tower L holds the leaf blocks with level < L plus all blocks at level L,
// grouped by level from L down to 1 (id order inside a level).  A face is
// FINE_FINE (same-level neighbour handled by the stencil), FINE_BC
// (physical boundary), FINE_CRSE (coarser neighbour; the neighbour is the
// parent's neighbour) or CRSE_FINE (same-level neighbour that is refined
// inside the tower; the fine faces behind it are summed).
#pragma once

#include <vector>

#include "tree.h"

namespace sayaka_gb300 {

enum FaceType { kFaceFineFine = 0, kFaceBC = 1, kFaceFineCrse = 2, kFaceCrseFine = 3 };

struct FaceReg {
  int type;
  int neigh;         // neighbour block (FINE_CRSE: the coarse leaf), or BC code
  int fc_off[3];     // FINE_CRSE: ChildIndexOffset of the mirrored child
  int cf_neigh[4];   // CRSE_FINE: fine blocks on the face, ChildIndex order
};

struct Tower {
  int level = 0;
  std::vector<int> blocks;
  std::vector<int> begin, end;  // [sublevel], sublevel = 1..level
  std::vector<FaceReg> regs;    // [tower position * 6 + face]
  bool empty() const { return blocks.empty(); }
};

// towers for MG levels 1..tree.max_level (index 0 unused)
std::vector<Tower> build_towers(const AmrTree &tree);

}  // namespace sayaka_gb300
