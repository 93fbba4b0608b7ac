"""CPU restatement of the reference's block tree for building workloads
(ORACLE -- test infrastructure: used by tests/ and by bench.py's reference
arm, so that the reference arm's problems are built without the product
library).

The subset the workloads need: AmrTree::initUniformRootLevel
(src/SayakaTree.cpp:93-201), initRefineToMinLevel (src/SayakaTree.cpp:
204-233) and regrid with refinement flags (src/SayakaRegrid.cpp:26-125:
refineBlocks with its 2:1 propagation across faces, edges and corners,
src/SayakaRegrid.cpp:240-510, and the node types of :634-653), with the same
block ids, links and box arithmetic; coarsening is not restated.  The
interface is that of sayakaamr_gb300.AmrTree (init_uniform_root,
init_refine_to_min_level, set_refine_flags, regrid, tables), and the tables
are bit-identical to the reference's (tests/test_tree_oracle.py checks them
against the reference's dumps and the product's tree).
"""
import numpy as np

PHYS_BNDRY = -20
LEAF, HAS_LEAF_CHILD, NO_LEAF_CHILD = 1, 2, 3


class TreeOracle:
    def __init__(self, ndim, nb, min_level, max_level, capacity=40000):
        self.ndim, self.nb = ndim, nb
        self.min_level, self.max_level, self.capacity = min_level, max_level, capacity
        self.nf, self.nc = 2 * ndim, 1 << ndim
        self.n = 0
        self.level, self.parent, self.which_child, self.node_type = [], [], [], []
        self.neighbor, self.child, self.node_type2 = [], [], []
        self.lo, self.hi = [], []
        self.refine_flag = []

    # -- nodes
    def _new(self):
        self.level.append(-1)
        self.parent.append(-1)
        self.which_child.append(-1)
        self.node_type.append(-1)
        self.neighbor.append([-1] * 6)
        self.child.append([-1] * 8)
        self.node_type2.append([-1] * 6)
        self.lo.append([0.0, 0.0, 0.0])
        self.hi.append([0.0, 0.0, 0.0])
        self.refine_flag.append(0)
        return len(self.level) - 1

    def _leaf(self, i):
        return self.node_type[i] == LEAF

    def _has_children(self, i):
        return self.child[i][0] >= 0

    # -- AmrTree::initUniformRootLevel
    def init_uniform_root(self, ndiv, lo, hi, bc_type, periodic=(0,) * 6):
        nx, ny, nz = (int(v) for v in ndiv)
        ndiv = (nx, ny, nz)

        def ind(i, j, k):
            return i + j * nx + k * nx * ny

        for _ in range(nx * ny * nz):
            self._new()
        self.n = nx * ny * nz
        for k in range(nz):
            for j in range(ny):
                for i in range(nx):
                    r = ind(i, j, k)
                    ijk = (i, j, k)
                    blo = [float(lo[0]), float(lo[1]), float(lo[2])]
                    bhi = list(blo)
                    for d in range(self.ndim):
                        h = (float(hi[d]) - float(lo[d])) / ndiv[d]
                        blo[d] += h * ijk[d]
                        bhi[d] += h * (ijk[d] + 1)
                    self.lo[r], self.hi[r] = blo, bhi
                    self.node_type[r] = LEAF
                    self.level[r] = 1
                    for f in range(self.nf):
                        d, s = f >> 1, f & 1
                        c = [i, j, k]
                        edge = 0 if s == 0 else ndiv[d] - 1
                        if ijk[d] == edge:
                            if periodic[f]:
                                c[d] = ndiv[d] - 1 if s == 0 else 0
                                nbr = ind(*c)
                            else:
                                nbr = int(bc_type[f])
                        else:
                            c[d] += -1 if s == 0 else 1
                            nbr = ind(*c)
                        self.neighbor[r][f] = nbr

    def init_refine_to_min_level(self):
        for _ in range(1, self.min_level + 1):
            self.regrid()

    def set_refine_flags(self, flags):
        for i, v in enumerate(flags):
            self.refine_flag[i] = int(v)

    # -- AmrTree::regrid (refinement only)
    def regrid(self):
        for i in range(self.n):
            lv = self.level[i]
            if lv >= self.max_level:
                self.refine_flag[i] = 0
            if lv < self.min_level and self._leaf(i):
                self.refine_flag[i] = 1
        if any(self._leaf(i) and self.refine_flag[i] for i in range(self.n)):
            self._refine_blocks()
            self._set_node_type()

    def _child_side(self, c, d):
        return (c >> d) & 1

    def _refine_blocks(self):
        nf, nc, nd = self.nf, self.nc, self.ndim
        while True:
            for i in range(self.n):
                if self.refine_flag[i] and not self._leaf(i):
                    self.refine_flag[i] = 0
            refined = [i for i in range(self.n) if self.refine_flag[i]]
            # children appended in ChildIndex order, parent by parent
            for i in refined:
                for c in range(nc):
                    if len(self.level) >= self.capacity:
                        raise RuntimeError("tree capacity exceeded")
                    j = self._new()
                    self.child[i][c] = j
                    self.level[j] = self.level[i] + 1
                    self.parent[j] = i
                    self.which_child[j] = c
                    blo, bhi = list(self.lo[i]), list(self.hi[i])
                    for d in range(nd):
                        mid = 0.5 * (self.lo[i][d] + self.hi[i][d])
                        if self._child_side(c, d) == 0:
                            bhi[d] = mid
                        else:
                            blo[d] = mid
                    self.lo[j], self.hi[j] = blo, bhi
            new_children = list(range(self.n, len(self.level)))
            # links to siblings and to the parents' neighbours' children
            for i in refined:
                for c in range(nc):
                    ic = self.child[i][c]
                    for f in range(nf):
                        d, side = f >> 1, f & 1
                        jc = c ^ (1 << d)
                        if self._child_side(c, d) != side:
                            self.neighbor[ic][f] = self.child[i][jc]
                        else:
                            pn = self.neighbor[i][f]
                            if pn >= 0:
                                jchild = self.child[pn][jc]
                                self.neighbor[ic][f] = jchild
                                if jchild >= 0:
                                    self.neighbor[jchild][f ^ 1] = ic
            self.n = len(self.level)
            # face tags: 2 the block has children, 3 a child has children on the far side
            for i in range(self.n):
                t2 = self.node_type2[i]
                for f in range(nf):
                    t2[f] = 1
                for c in range(nc):
                    j = self.child[i][c]
                    if j < 0:
                        continue
                    for f in range(nf):
                        if t2[f] != 3:
                            t2[f] = 2
                    for cc in range(nc):
                        if self.child[j][cc] < 0:
                            continue
                        for d in range(nd):
                            t2[2 * d + (1 - self._child_side(c, d))] = 3
            self._set_node_type()
            # 2:1 propagation: across faces, then edges (2 directions), then corners (3)
            n = self.n
            t1 = [0] * n
            for i in range(n):
                for f in range(nf):
                    nb_ = self.neighbor[i][f]
                    if nb_ >= 0 and self.node_type2[nb_][f] == 3:
                        t1[i] = 1
                        break
            t2 = [0] * n
            if nd >= 2:
                for i in range(n):
                    cnt = [0, 0, 0]
                    for f in range(nf):
                        nb_ = self.neighbor[i][f]
                        if nb_ >= 0 and t1[nb_]:
                            cnt[f >> 1] += 1
                    if (cnt[0] and cnt[1]) or (cnt[0] and cnt[2]) or (cnt[1] and cnt[2]):
                        t2[i] = 1
                for i in range(n):
                    if t2[i] or t1[i]:
                        t2[i] = 1
            t3 = [0] * n
            if nd == 3:
                for i in range(n):
                    cnt = [0, 0, 0]
                    for f in range(nf):
                        nb_ = self.neighbor[i][f]
                        if nb_ >= 0 and t2[nb_]:
                            cnt[f >> 1] += 1
                    if cnt[0] and cnt[1] and cnt[2]:
                        t3[i] = 1
            repeat = False
            for i in range(n):
                self.refine_flag[i] = 0
                if self._leaf(i) and (t1[i] or t2[i] or t3[i]):
                    self.refine_flag[i] = 1
                    repeat = True
            self._new_children = getattr(self, "_new_children", []) + new_children
            if not repeat:
                break
        # new children on the domain boundary take the parent's boundary code
        for i in self._new_children:
            p = self.parent[i]
            for f in range(nf):
                if self.neighbor[i][f] < 0 and self.neighbor[p][f] <= PHYS_BNDRY:
                    self.neighbor[i][f] = self.neighbor[p][f]
        self._new_children = []
        for i in range(len(self.refine_flag)):
            self.refine_flag[i] = 0

    def _set_node_type(self):
        # the last child inspected decides (src/SayakaRegrid.cpp:634-653)
        for i in range(self.n):
            t = NO_LEAF_CHILD
            for c in range(self.nc):
                j = self.child[i][c]
                if j < 0:
                    t = LEAF
                elif not self._has_children(j):
                    t = HAS_LEAF_CHILD
            self.node_type[i] = t

    # -- tables in the layout of sayakaamr_gb300.AmrTree.tables()
    def tables(self):
        n = self.n
        lo = np.array(self.lo[:n], dtype=np.float64).reshape(-1)
        hi = np.array(self.hi[:n], dtype=np.float64).reshape(-1)
        return dict(ndim=self.ndim, nb=self.nb, num_blocks=n, min_level=self.min_level, max_level=self.max_level,
                    level=np.array(self.level[:n], dtype=np.int32),
                    neighbor=np.array(self.neighbor[:n], dtype=np.int32).reshape(-1),
                    child=np.array(self.child[:n], dtype=np.int32).reshape(-1),
                    parent=np.array(self.parent[:n], dtype=np.int32),
                    which_child=np.array(self.which_child[:n], dtype=np.int32),
                    node_type=np.array(self.node_type[:n], dtype=np.int32),
                    block_len=hi - lo, block_lo=lo, block_hi=hi, block_center=0.5 * (lo + hi),
                    node_type2=np.array(self.node_type2[:n], dtype=np.int32).reshape(-1))
