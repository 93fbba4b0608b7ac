#include "tower.h"

#include <thread>

namespace sayaka_gb300 {

static Tower build_one(const AmrTree &t, int L) {
  Tower tw;
  tw.level = L;
  tw.begin.assign(L + 1, 0);
  tw.end.assign(L + 1, 0);
  if (L >= (int)t.levels.size() || t.levels[L].empty()) return tw;
  const int nf = t.num_face(), nc = t.num_child(), half = t.nb / 2;
  size_t cap = 0;
  for (int l = L; l >= 1; l--) cap += t.levels[l].size();
  tw.blocks.reserve(cap);
  tw.regs.reserve(cap * kMaxFace);
  for (int l = L; l >= 1; l--) {
    tw.begin[l] = (int)tw.blocks.size();
    for (int b : t.levels[l]) {
      const TreeNode &n = t.nodes[b];
      if (!(n.leaf() || l == L)) continue;
      tw.blocks.push_back(b);
      for (int f = 0; f < kMaxFace; f++) {
        FaceReg r{};
        r.type = kFaceFineFine;
        r.neigh = -1;
        for (int q = 0; q < 4; q++) r.cf_neigh[q] = -1;
        if (f < nf) {
          const int nbr = n.neighbor[f];
          if (nbr <= kPhysBndry) {
            r.type = kFaceBC;
            r.neigh = nbr;
          } else if (nbr < 0) {
            r.type = kFaceFineCrse;
            r.neigh = t.nodes[n.parent].neighbor[f];
            bool sib;
            const int mc = child_neighbor(n.which_child, f, &sib);
            for (int d = 0; d < t.ndim; d++) r.fc_off[d] = child_side(mc, d) * half;
          } else if (l < L && !t.nodes[nbr].leaf()) {
            r.type = kFaceCrseFine;
            r.neigh = nbr;
            const int dir = f >> 1, opp_side = 1 - (f & 1);
            int q = 0;
            for (int c = 0; c < nc; c++)
              if (child_side(c, dir) == opp_side) r.cf_neigh[q++] = t.nodes[nbr].child[c];
          } else {
            r.type = kFaceFineFine;
            r.neigh = nbr;
          }
        }
        tw.regs.push_back(r);
      }
    }
    tw.end[l] = (int)tw.blocks.size();
  }
  return tw;
}

// the towers are independent: one host thread per level
std::vector<Tower> build_towers(const AmrTree &t) {
  std::vector<Tower> v(t.max_level + 1);
  std::vector<std::thread> th;
  for (int L = 1; L <= t.max_level; L++) th.emplace_back([&v, &t, L] { v[L] = build_one(t, L); });
  for (auto &x : th) x.join();
  return v;
}

}  // namespace sayaka_gb300
