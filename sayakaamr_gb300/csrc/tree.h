// Host-side block tree: the AmrTree / regrid / surrounding-block API of the
// SayakaAmr library (src/SayakaTree.h:52-333, src/SayakaRegrid.cpp:26-976),
// re-designed as a runtime-dimension (2D/3D) C++ class whose block tables are
// the device solver's input.
//
// Block ids are assigned in exactly the reference's creation/packing order
// (children appended in ChildIndex order during refinement, survivors packed
// in id order during coarsening) because every table the solver uses --
// neighbour, child, parent, level lists, towers -- is keyed by those ids and
// must be bit-identical to the reference's.
#pragma once

#include <cstdint>
#include <vector>

namespace sayaka_gb300 {

// neighbour codes: >= 0 block id at the same level, -1 coarser level,
// <= kPhysBndry physical boundary code (src/SayakaTree.h:38-40)
constexpr int kPhysBndry = -20;
constexpr int kMaxFace = 6;
constexpr int kMaxChild = 8;
constexpr int kNumSurr = 27;

enum NodeType {
  kNodeInvalid = 0,
  kNodeLeaf = 1,
  kNodeHasLeafChild = 2,
  kNodeNoLeafChild = 3,
};

struct TreeNode {
  int level;
  int neighbor[kMaxFace];
  int child[kMaxChild];
  int parent;
  int which_child;
  int node_type;
  int node_type2[kMaxFace];
  int flags;
  double lo[3], hi[3];
  double center[3], length[3];

  bool leaf() const { return node_type == kNodeLeaf; }
  bool has_children() const { return child[0] >= 0; }
  void reset();
  void set_box(const double blo[3], const double bhi[3]);
};

// 3x3x3 neighbourhood of a block, position (ii,jj,kk) in {-1,0,1}^3 stored at
// (ii+1) + 3*(jj+1) + 9*(kk+1).  bcrefs hold the SurroundingIndex of the
// face/edge block the entry was derived from (src/SayakaTree.h:336-526).
struct SurrBlocks {
  int blocks[kNumSurr];
  int types[kNumSurr];
  int bcrefs[kNumSurr];
  void reset();
};

class AmrTree {
 public:
  // dimension and block shape
  int ndim = 2;
  int nb = 8;  // cells per block edge (even)
  int min_level = 1;
  int max_level = 1;
  int capacity = 0;
  int num_blocks = 0;

  std::vector<TreeNode> nodes;
  std::vector<int> refine_flag;
  std::vector<int> coarsen_flag;
  std::vector<int> new_child_flag;
  std::vector<SurrBlocks> surr;
  // levels[l] = ids of blocks at level l in id order, l = 1..max_level
  std::vector<std::vector<int>> levels;

  int num_face() const { return 2 * ndim; }
  int num_child() const { return 1 << ndim; }

  // allocate `capacity` block slots (src/SayakaTree.cpp:34-91)
  // (surroundings = false: without the 3x3x3 tables, for a tree that only
  // serves as the source of towers)
  void init(int ndim, int nb, int min_level, int max_level, int capacity, bool surroundings = true);
  // root blocks on a uniform grid (src/SayakaTree.cpp:93-201)
  void init_uniform_root(const int ndiv[3], const double lo[3], const double hi[3],
                         const int bc_type[6], const bool periodic[6]);
  // regrid until the minimum level is reached (src/SayakaTree.cpp:204-233)
  int init_refine_to_min_level();
  // apply refine/coarsen flags (src/SayakaRegrid.cpp:26-125).
  // Returns 0, or -1 when the block capacity would overflow.
  int regrid();

  int finest_level() const;
  // SurroundingIndex of position (ii,jj,kk) in {-1,0,1}: the reference's
  // encoding skips dimensions above ndim (src/SayakaSurroundingIndex.h:66-79)
  int surr_index(int ii, int jj, int kk) const;

  // cell metrics computed exactly as src/SayakaTree.h:277-301
  void cell_size(int b, double dx[3]) const;
  double cell_volume(int b) const;
  void cell_area(int b, double ds[3]) const;

 private:
  void check_coarsen();
  int refine_blocks();
  int coarsen_blocks(int old_num);
  void set_node_type();
  void build_surrounding();
  void cache_levels();
};

// ChildIndex helpers (src/SayakaChildIndex.cpp:12-104)
inline int child_side(int ichild, int dir) { return (ichild >> dir) & 1; }
// neighbour of child `ichild` across `face`; *same_parent tells whether it is
// a sibling (true) or a child of the parent's neighbour (false)
int child_neighbor(int ichild, int face, bool *same_parent);

}  // namespace sayaka_gb300
