// Host block tree and regrid.  Behaviour follows src/SayakaTree.cpp and
// src/SayakaRegrid.cpp of the SayakaAmr library step by step where block ids
// or table contents depend on the order of operations (see tree.h).
#include "tree.h"

#include <algorithm>
#include <cstdlib>

namespace sayaka_gb300 {

void TreeNode::reset() {
  level = -1;
  std::fill(neighbor, neighbor + kMaxFace, -1);
  std::fill(child, child + kMaxChild, -1);
  parent = -1;
  which_child = -1;
  node_type = -1;
  std::fill(node_type2, node_type2 + kMaxFace, -1);
  flags = -1;
  for (int d = 0; d < 3; d++) lo[d] = hi[d] = center[d] = length[d] = 0.0;
}

void TreeNode::set_box(const double blo[3], const double bhi[3]) {
  for (int d = 0; d < 3; d++) {
    lo[d] = blo[d];
    hi[d] = bhi[d];
    center[d] = 0.5 * (blo[d] + bhi[d]);
    length[d] = bhi[d] - blo[d];
  }
}

void SurrBlocks::reset() {
  std::fill(blocks, blocks + kNumSurr, -1);
  std::fill(types, types + kNumSurr, -1);
  std::fill(bcrefs, bcrefs + kNumSurr, -1);
}

int child_neighbor(int ichild, int face, bool *same_parent) {
  const int dir = face >> 1, side = face & 1;
  *same_parent = child_side(ichild, dir) != side;
  return ichild ^ (1 << dir);
}

static inline int spos(int ii, int jj, int kk) { return (ii + 1) + 3 * (jj + 1) + 9 * (kk + 1); }

int AmrTree::surr_index(int ii, int jj, int kk) const {
  int s = ii + 1;
  if (ndim >= 2) s += 3 * (jj + 1);
  if (ndim == 3) s += 9 * (kk + 1);
  return s;
}

void AmrTree::init(int ndim_, int nb_, int min_level_, int max_level_, int capacity_, bool surroundings) {
  ndim = ndim_;
  nb = nb_;
  min_level = min_level_;
  max_level = max_level_;
  capacity = capacity_;
  num_blocks = 0;
  nodes.assign(capacity, TreeNode());
  for (auto &n : nodes) n.reset();
  refine_flag.assign(capacity, 0);
  coarsen_flag.assign(capacity, 0);
  new_child_flag.assign(capacity, 0);
  surr.assign(surroundings ? capacity : 0, SurrBlocks());
  for (auto &s : surr) s.reset();
  levels.assign(max_level + 1, std::vector<int>());
}

void AmrTree::init_uniform_root(const int ndiv[3], const double plo[3], const double phi[3],
                                const int bc_type[6], const bool periodic[6]) {
  const int n0x = ndiv[0], n0y = ndiv[1], n0z = ndiv[2];
  auto ind = [=](int i, int j, int k) { return i + j * n0x + k * n0x * n0y; };
  num_blocks = n0x * n0y * n0z;
  for (int k = 0; k < n0z; k++)
    for (int j = 0; j < n0y; j++)
      for (int i = 0; i < n0x; i++) {
        TreeNode &r = nodes[ind(i, j, k)];
        double blo[3] = {plo[0], plo[1], plo[2]};
        double bhi[3] = {plo[0], plo[1], plo[2]};
        const int ijk[3] = {i, j, k};
        for (int d = 0; d < ndim; d++) {
          const double h = (phi[d] - plo[d]) / ndiv[d];
          blo[d] += h * ijk[d];
          bhi[d] += h * (ijk[d] + 1);
        }
        r.set_box(blo, bhi);
        r.node_type = kNodeLeaf;
        r.level = 1;
        for (int f = 0; f < num_face(); f++) {
          const int d = f >> 1, s = f & 1;
          int c[3] = {i, j, k};
          const int edge = s == 0 ? 0 : ndiv[d] - 1;
          int nbr;
          if (ijk[d] == edge) {
            if (periodic[f]) {
              c[d] = s == 0 ? ndiv[d] - 1 : 0;
              nbr = ind(c[0], c[1], c[2]);
            } else {
              nbr = bc_type[f];
            }
          } else {
            c[d] += s == 0 ? -1 : 1;
            nbr = ind(c[0], c[1], c[2]);
          }
          r.neighbor[f] = nbr;
        }
      }
}

int AmrTree::init_refine_to_min_level() {
  for (int l = 1; l <= min_level; l++) {
    int rc = regrid();
    if (rc) return rc;
  }
  return 0;
}

int AmrTree::finest_level() const {
  int f = 0;
  for (int i = 0; i < num_blocks; i++) f = std::max(f, nodes[i].level);
  return f;
}

void AmrTree::cell_size(int b, double dx[3]) const {
  for (int d = 0; d < 3; d++) dx[d] = nodes[b].length[d];
  for (int d = 0; d < ndim; d++) dx[d] /= nb;
}

double AmrTree::cell_volume(int b) const {
  double dx[3];
  cell_size(b, dx);
  double v = 1.0;
  for (int d = 0; d < ndim; d++) v *= dx[d];
  return v;
}

void AmrTree::cell_area(int b, double ds[3]) const {
  double dx[3];
  cell_size(b, dx);
  const double v = cell_volume(b);
  ds[0] = ds[1] = ds[2] = 1.0;
  for (int d = 0; d < ndim; d++) ds[d] = v / dx[d];
}

// --------------------------------------------------------------------------
// regrid (src/SayakaRegrid.cpp:26-125)
int AmrTree::regrid() {
  if (min_level < 1 || max_level < min_level) return -2;
  std::vector<int> refine_save(capacity, 0);
  for (int i = 0; i < num_blocks; i++) {
    const int l = nodes[i].level;
    if (l >= max_level) refine_flag[i] = 0;
    if (l <= min_level) coarsen_flag[i] = 0;
    if (l < min_level && nodes[i].leaf()) refine_flag[i] = 1;
    refine_save[i] = refine_flag[i];
  }
  std::fill(new_child_flag.begin(), new_child_flag.end(), 0);

  check_coarsen();
  // a leaf marked for coarsening whose parent is marked for refinement stays
  for (int i = 0; i < num_blocks; i++)
    if (nodes[i].leaf() && coarsen_flag[i] && refine_save[nodes[i].parent]) coarsen_flag[i] = 0;

  bool need = false;
  for (int i = 0; i < num_blocks && !need; i++)
    if (nodes[i].leaf() && (refine_flag[i] || coarsen_flag[i])) need = true;

  if (need) {
    int nrefine = 0;
    for (int i = 0; i < num_blocks; i++)
      if (nodes[i].leaf() && refine_flag[i]) nrefine++;
    int nsave = num_blocks;
    if (nrefine > 0) {
      int rc = refine_blocks();
      if (rc) return rc;
    }
    coarsen_blocks(nsave);
  }
  build_surrounding();
  cache_levels();
  return 0;
}

// 2:1 balance guard for coarsening (src/SayakaRegrid.cpp:127-238)
void AmrTree::check_coarsen() {
  std::vector<int> t1(capacity, 0), t2(capacity, 0), t3(capacity, 0);
  const int nf = num_face();
  for (int i = 0; i < num_blocks; i++)
    if (coarsen_flag[i] && !nodes[i].leaf()) coarsen_flag[i] = 0;
  // blocks next to a refined block
  for (int i = 0; i < num_blocks; i++)
    for (int f = 0; f < nf; f++) {
      const int n = nodes[i].neighbor[f];
      if (n >= 0 && nodes[n].has_children()) {
        t1[i] = 1;
        break;
      }
    }
  if (ndim >= 2) {
    for (int i = 0; i < num_blocks; i++)
      for (int f = 0; f < nf; f++) {
        const int n = nodes[i].neighbor[f];
        if (n >= 0 && t1[n]) {
          t2[i] = 1;
          break;
        }
      }
    for (int i = 0; i < num_blocks; i++)
      if (t1[i] || t2[i]) t2[i] = 1;
  }
  if (ndim == 3) {
    for (int i = 0; i < num_blocks; i++)
      for (int f = 0; f < nf; f++) {
        const int n = nodes[i].neighbor[f];
        if (n >= 0 && t2[n]) {
          t3[i] = 1;
          break;
        }
      }
  }
  for (int i = 0; i < num_blocks; i++)
    if (nodes[i].leaf() && (t1[i] || t2[i] || t3[i])) coarsen_flag[i] = 0;
  for (int i = 0; i < num_blocks; i++)
    if (nodes[i].parent < 0 && coarsen_flag[i]) coarsen_flag[i] = 0;
  // every sibling must agree
  for (int i = 0; i < num_blocks; i++) {
    if (!coarsen_flag[i]) continue;
    const TreeNode &p = nodes[nodes[i].parent];
    for (int c = 0; c < num_child(); c++)
      if (!coarsen_flag[p.child[c]]) {
        coarsen_flag[i] = 0;
        break;
      }
  }
}

// refinement with 2:1 propagation across faces, edges and corners
// (src/SayakaRegrid.cpp:240-510)
int AmrTree::refine_blocks() {
  std::vector<int> t1(capacity), t2(capacity), t3(capacity);
  const int nf = num_face(), nc = num_child();
  std::fill(new_child_flag.begin(), new_child_flag.end(), 0);

  for (;;) {
    for (int i = 0; i < num_blocks; i++)
      if (refine_flag[i] && !nodes[i].leaf()) refine_flag[i] = 0;

    // create children, ids appended in ChildIndex order
    int nblock = num_blocks;
    for (int i = 0; i < num_blocks; i++) {
      if (!refine_flag[i]) continue;
      for (int c = 0; c < nc; c++) {
        if (nblock >= capacity) return -1;
        const int j = nblock++;
        TreeNode &p = nodes[i];
        TreeNode &ch = nodes[j];
        p.child[c] = j;
        ch.level = p.level + 1;
        ch.parent = i;
        ch.which_child = c;
        double blo[3], bhi[3];
        for (int d = 0; d < 3; d++) {
          blo[d] = p.lo[d];
          bhi[d] = p.hi[d];
        }
        for (int d = 0; d < ndim; d++) {
          const double mid = 0.5 * (p.lo[d] + p.hi[d]);
          if (child_side(c, d) == 0)
            bhi[d] = mid;
          else
            blo[d] = mid;
        }
        ch.set_box(blo, bhi);
        ch.flags = p.flags;
        new_child_flag[j] = 1;
      }
    }
    // connect the new children to siblings and to the parents' neighbours
    for (int i = 0; i < num_blocks; i++) {
      if (!refine_flag[i]) continue;
      for (int c = 0; c < nc; c++) {
        const int ic = nodes[i].child[c];
        for (int f = 0; f < nf; f++) {
          bool sib;
          const int jc = child_neighbor(c, f, &sib);
          if (sib) {
            nodes[ic].neighbor[f] = nodes[i].child[jc];
          } else {
            const int pn = nodes[i].neighbor[f];
            if (pn >= 0) {
              const int jchild = nodes[pn].child[jc];
              nodes[ic].neighbor[f] = jchild;
              if (jchild >= 0) nodes[jchild].neighbor[f ^ 1] = ic;
            }
          }
        }
      }
    }
    num_blocks = nblock;

    // node_type2: face tags 2 (has children) / 3 (grandchildren on the far side)
    for (int i = 0; i < num_blocks; i++) {
      int *t2f = nodes[i].node_type2;
      for (int f = 0; f < nf; f++) t2f[f] = 1;
      for (int c = 0; c < nc; c++) {
        const int j = nodes[i].child[c];
        if (j < 0) continue;
        for (int f = 0; f < nf; f++)
          if (t2f[f] != 3) t2f[f] = 2;
        for (int cc = 0; cc < nc; cc++) {
          if (nodes[j].child[cc] < 0) continue;
          for (int d = 0; d < ndim; d++) t2f[2 * d + (1 - child_side(c, d))] = 3;
        }
      }
    }
    set_node_type();

    std::fill(t1.begin(), t1.end(), 0);
    std::fill(t2.begin(), t2.end(), 0);
    std::fill(t3.begin(), t3.end(), 0);
    std::fill(refine_flag.begin(), refine_flag.end(), 0);

    for (int i = 0; i < num_blocks; i++)
      for (int f = 0; f < nf; f++) {
        const int n = nodes[i].neighbor[f];
        if (n >= 0 && nodes[n].node_type2[f] == 3) {
          t1[i] = 1;
          break;
        }
      }
    if (ndim >= 2) {
      for (int i = 0; i < num_blocks; i++) {
        int cnt[3] = {0, 0, 0};
        for (int f = 0; f < nf; f++) {
          const int n = nodes[i].neighbor[f];
          if (n >= 0 && t1[n]) cnt[f >> 1]++;
        }
        if ((cnt[0] && cnt[1]) || (cnt[0] && cnt[2]) || (cnt[1] && cnt[2])) t2[i] = 1;
      }
      for (int i = 0; i < num_blocks; i++)
        if (t2[i] || t1[i]) t2[i] = 1;
    }
    if (ndim == 3) {
      for (int i = 0; i < num_blocks; i++) {
        int cnt[3] = {0, 0, 0};
        for (int f = 0; f < nf; f++) {
          const int n = nodes[i].neighbor[f];
          if (n >= 0 && t2[n]) cnt[f >> 1]++;
        }
        if (cnt[0] && cnt[1] && cnt[2]) t3[i] = 1;
      }
    }
    bool repeat = false;
    for (int i = 0; i < num_blocks; i++) {
      refine_flag[i] = 0;
      if (nodes[i].leaf() && (t1[i] || t2[i] || t3[i])) {
        refine_flag[i] = 1;
        repeat = true;
      }
    }
    if (!repeat) break;
  }

  // new children on the domain boundary inherit the parent's boundary code
  for (int i = 0; i < num_blocks; i++) {
    if (!new_child_flag[i]) continue;
    const int p = nodes[i].parent;
    for (int f = 0; f < nf; f++)
      if (nodes[i].neighbor[f] < 0 && nodes[p].neighbor[f] <= kPhysBndry) nodes[i].neighbor[f] = nodes[p].neighbor[f];
  }
  std::fill(refine_flag.begin(), refine_flag.end(), 0);
  return 0;
}

// remove coarsened blocks and pack ids (src/SayakaRegrid.cpp:515-632)
int AmrTree::coarsen_blocks(int old_num) {
  check_coarsen();
  std::vector<int> newloc(capacity, -1);
  for (int i = 0; i < num_blocks; i++)
    if (coarsen_flag[i]) nodes[i].flags = -1;
  int nblock = num_blocks;
  int ipack = 0;
  for (int i = 0; i < num_blocks; i++) {
    if (!coarsen_flag[i]) {
      if (ipack != i) {
        nodes[ipack] = nodes[i];
        new_child_flag[ipack] = new_child_flag[i];
      }
      newloc[i] = ipack++;
    } else {
      nblock--;
      old_num--;
    }
  }
  for (int i = nblock; i < num_blocks; i++) {
    coarsen_flag[i] = 0;
    nodes[i].reset();
  }
  num_blocks = nblock;
  for (int i = 0; i < num_blocks; i++) {
    TreeNode &n = nodes[i];
    if (n.parent >= 0) n.parent = newloc[n.parent];
    for (int c = 0; c < num_child(); c++)
      if (n.child[c] >= 0) n.child[c] = newloc[n.child[c]];
    for (int f = 0; f < num_face(); f++)
      if (n.neighbor[f] >= 0) n.neighbor[f] = newloc[n.neighbor[f]];
  }
  set_node_type();
  std::fill(coarsen_flag.begin(), coarsen_flag.end(), 0);
  return old_num;
}

// (src/SayakaRegrid.cpp:634-653): the last child inspected decides
void AmrTree::set_node_type() {
  for (int i = 0; i < num_blocks; i++) {
    TreeNode &n = nodes[i];
    n.node_type = kNodeNoLeafChild;
    for (int c = 0; c < num_child(); c++) {
      const int j = n.child[c];
      if (j < 0)
        n.node_type = kNodeLeaf;
      else if (!nodes[j].has_children())
        n.node_type = kNodeHasLeafChild;
    }
  }
}

// 3x3x3 neighbourhood incl. edges and (3D) corners
// (src/SayakaRegrid.cpp:655-945, src/SayakaTree.h:450-523)
void AmrTree::build_surrounding() {
  const int XD = 1, YD = ndim >= 2 ? 1 : 0, ZD = ndim == 3 ? 1 : 0;
  const int center = surr_index(0, 0, 0);
  for (int i = 0; i < num_blocks; i++) {
    SurrBlocks &s = surr[i];
    s.reset();
    s.blocks[spos(0, 0, 0)] = i;
    for (int f = 0; f < num_face(); f++) {
      int p[3] = {0, 0, 0};
      p[f >> 1] = (f & 1) ? 1 : -1;
      s.blocks[spos(p[0], p[1], p[2])] = nodes[i].neighbor[f];
      s.bcrefs[spos(p[0], p[1], p[2])] = center;
    }
    // edges: |ii|+|jj|+|kk| == 2, reached through either adjacent face block
    for (int kk = -ZD; kk <= ZD; kk++)
      for (int jj = -YD; jj <= YD; jj++)
        for (int ii = -XD; ii <= XD; ii++) {
          if (std::abs(ii) + std::abs(jj) + std::abs(kk) != 2) continue;
          int f0, f1, a0[3], a1[3];
          if (ii == 0) {
            f0 = jj == -1 ? 2 : 3;
            a0[0] = ii; a0[1] = 0; a0[2] = kk;
            f1 = kk == -1 ? 4 : 5;
            a1[0] = ii; a1[1] = jj; a1[2] = 0;
          } else if (jj == 0) {
            f0 = ii == -1 ? 0 : 1;
            a0[0] = 0; a0[1] = jj; a0[2] = kk;
            f1 = kk == -1 ? 4 : 5;
            a1[0] = ii; a1[1] = jj; a1[2] = 0;
          } else {
            f0 = ii == -1 ? 0 : 1;
            a0[0] = 0; a0[1] = jj; a0[2] = kk;
            f1 = jj == -1 ? 2 : 3;
            a1[0] = ii; a1[1] = 0; a1[2] = kk;
          }
          const int e = spos(ii, jj, kk);
          int ref = 0;  // 0 none / boundary, 1 same level, 2 coarse
          const int v0 = s.blocks[spos(a0[0], a0[1], a0[2])];
          if (v0 >= 0) {
            ref = 1;
            s.blocks[e] = nodes[v0].neighbor[f0];
            s.bcrefs[e] = surr_index(a0[0], a0[1], a0[2]);
          } else if (v0 <= kPhysBndry) {
            s.blocks[e] = v0;
            s.bcrefs[e] = surr_index(a0[0], a0[1], a0[2]);
          } else {
            ref = 2;
            s.bcrefs[e] = surr_index(a0[0], a0[1], a0[2]);
          }
          const int v1 = s.blocks[spos(a1[0], a1[1], a1[2])];
          if (v1 >= 0) {
            s.blocks[e] = nodes[v1].neighbor[f1];
            s.bcrefs[e] = surr_index(a1[0], a1[1], a1[2]);
          } else if (v1 <= kPhysBndry) {
            if (ref == 0) {
              s.blocks[e] = v1;
              s.bcrefs[e] = surr_index(a1[0], a1[1], a1[2]);
            }
          } else if (ref == 0) {
            s.bcrefs[e] = surr_index(a1[0], a1[1], a1[2]);
          }
        }
    // corners (3D): scan the three edge blocks sharing the corner
    if (ndim == 3) {
      for (int kc = -1; kc <= 1; kc += 2)
        for (int jc = -1; jc <= 1; jc += 2)
          for (int ic = -1; ic <= 1; ic += 2) {
            const int ff[3] = {ic == -1 ? 0 : 1, jc == -1 ? 2 : 3, kc == -1 ? 4 : 5};
            int first = -1, second = -1, ref = -1;  // ref: 0 bc, 1 same, 2 coarse
            for (int d = 0; d < 3; d++) {
              const int a[3] = {d == 0 ? 0 : ic, d == 1 ? 0 : jc, d == 2 ? 0 : kc};
              const int lb = s.blocks[spos(a[0], a[1], a[2])];
              const int sidx = surr_index(a[0], a[1], a[2]);
              if (lb >= 0) {
                ref = 1;
                first = nodes[lb].neighbor[ff[d]];
                second = sidx;
              } else if (lb <= kPhysBndry) {
                if (ref == -1) {
                  ref = 0;
                  first = lb;
                  second = sidx;
                }
              } else if (ref != 1) {
                ref = 2;
                first = -1;
                second = sidx;
              }
            }
            s.blocks[spos(ic, jc, kc)] = first;
            s.bcrefs[spos(ic, jc, kc)] = second;
          }
    }
    for (int kk = -ZD; kk <= ZD; kk++)
      for (int jj = -YD; jj <= YD; jj++)
        for (int ii = -XD; ii <= XD; ii++) {
          const int e = spos(ii, jj, kk);
          s.types[e] = s.blocks[e] >= 0 ? nodes[s.blocks[e]].node_type : -1;
        }
  }
}

void AmrTree::cache_levels() {
  for (int l = 1; l <= max_level; l++) levels[l].clear();
  for (int i = 0; i < num_blocks; i++) levels[nodes[i].level].push_back(i);
}

}  // namespace sayaka_gb300
