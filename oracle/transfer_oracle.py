"""CPU restatement of the cell-data transfer across a regrid (ORACLE -- test
infrastructure: imported only by tests/ as the checker of
sayaka_mac_init_from).

Two transfers of a block-structured cell field from an old tree to a new
one, with blocks matched by their root and the child path from it:

* `transfer_injection`: every new leaf takes the old leaf it was, the
  injection from its nearest old leaf ancestor, the average of its old
  children, or zero over a deeper old subtree.
* `transfer_reference`: the reference's own sequence for a cell state with
  PROLONG_CENTERED_LINEAR prolongation and RESTRICT_AVERAGE restriction:
  FillPatch::restrictAll on the old tree (src/SayakaFillPatch.cpp:378-437,
  restrictCellBlockData_Average src/SayakaInterpPatch.cpp:398-444), then
  AmrTree::initNewBlockDataAfterRegrid (src/SayakaRegrid.cpp:987-1105): blocks
  present in both trees keep their data, new blocks are filled level by level
  from their parent by centered-linear interpolation
  (src/SayakaInterpPatch.cpp:228-306), the parent's face ghosts filled from
  its same-level neighbours (fillBlockBndryAtSameLevel,
  src/SayakaFillPatch.cpp:92-180) or by its physical BC
  (BCPatch::fillBasicCellBlockBC, src/SayakaBoundaryPatch.cpp:139-234).

Every floating-point operation is the reference's, in its order, on IEEE
doubles (numpy evaluates elementwise without contraction), so the results
are bit-identical to the reference's.
"""
import numpy as np

NEUMANN, DIRICHLET, SIMPLE_FILL = 0, 1, 2
PHYS_BNDRY = -20


def _path_key(tb, b):
    path = []
    while tb["parent"][b] >= 0:
        path.append(int(tb["which_child"][b]))
        b = int(tb["parent"][b])
    return (b, tuple(reversed(path)))


def _shape(nd, nb):
    return (nb,) * nd  # C order: [k][j][i] in 3D, [j][i] in 2D (cell i + nb*j + nb*nb*k)


def _axis(nd, q):
    """numpy axis of direction q (x is the last axis)"""
    return nd - 1 - q


def average_down(tb, x):
    """FillPatch::restrictAll with RESTRICT_AVERAGE: levels finest-1 .. 1,
    every non-leaf block's cells = (sum of its 2^d fine cells in k, j, i
    order, from 0) * (1 / 2^d).  x: [num_blocks][ncell], returned new."""
    nd, nb = int(tb["ndim"]), int(tb["nb"])
    half = nb // 2
    x = np.array(x, dtype=np.float64).reshape(int(tb["num_blocks"]), -1).copy()
    level = np.asarray(tb["level"])
    child = np.asarray(tb["child"]).reshape(-1, 8)
    leaf = np.asarray(tb["node_type"]) == 1
    wgt = 1.0 / (1 << nd)
    finest = int(level[leaf].max()) if leaf.any() else 1
    for lv in range(finest - 1, 0, -1):
        for b in np.nonzero((level == lv) & ~leaf)[0]:
            cb = x[b].reshape(_shape(nd, nb))
            for c in range(1 << nd):
                f = x[child[b, c]].reshape(_shape(nd, nb))
                s = 0.0
                for kk in range(2 if nd == 3 else 1):
                    for jj in range(2):
                        for ii in range(2):
                            if nd == 2:
                                s = s + f[jj::2, ii::2]
                            else:
                                s = s + f[kk::2, jj::2, ii::2]
                sl = tuple(slice(((c >> q) & 1) * half, ((c >> q) & 1) * half + half)
                           for q in reversed(range(nd)))
                cb[sl] = s * wgt
            x[b] = cb.reshape(-1)
    return x


def _plane(a, nd, q, idx):
    sl = [slice(None)] * nd
    sl[_axis(nd, q)] = idx
    return a[tuple(sl)]


def _padded_parent(tb, x, P, bc_type, bc_val):
    """the parent's cells with one ghost layer on its faces (corners unused)"""
    nd, nb = int(tb["ndim"]), int(tb["nb"])
    a = x[P].reshape(_shape(nd, nb))
    g = np.zeros((nb + 2,) * nd)
    g[(slice(1, nb + 1),) * nd] = a
    level = tb["level"]
    for f in range(2 * nd):
        q, s = f >> 1, f & 1
        n = int(tb["neighbor"][P * 6 + f])
        vref = _plane(a, nd, q, nb - 1 if s else 0)
        if n >= 0 and level[n] == level[P]:
            gv = _plane(x[n].reshape(_shape(nd, nb)), nd, q, 0 if s else nb - 1)
        elif n <= PHYS_BNDRY:
            bt = int(bc_type[P * 6 + f])
            if bt == NEUMANN:
                gv = vref
            elif bt == DIRICHLET:
                gv = 2.0 * bc_val[f] - vref
            else:
                gv = np.full_like(vref, bc_val[f])
        else:  # no same-level neighbour inside the domain: cannot occur in a 2:1-balanced tree
            gv = vref
        sl = [slice(1, nb + 1)] * nd
        sl[_axis(nd, q)] = nb + 1 if s else 0
        g[tuple(sl)] = gv
    return g


def _centered_linear(tb, x, b, bc_type, bc_val):
    """prolongCellBlockData_CenteredLinear of block b from its parent"""
    nd, nb = int(tb["ndim"]), int(tb["nb"])
    half = nb // 2
    P = int(tb["parent"][b])
    wc = int(tb["which_child"][b])
    g = _padded_parent(tb, x, P, bc_type, bc_val)
    fine = np.indices(_shape(nd, nb))  # fine[axis] = index along that numpy axis
    ic = []  # padded coarse index per direction
    rel = []
    for q in range(nd):
        i = fine[_axis(nd, q)]
        ic.append(((wc >> q) & 1) * half + (i >> 1) + 1)
        rel.append(np.where(i & 1, 0.25, -0.25))

    def at(off_q=None, delta=0):
        idx = [c.copy() for c in ic]
        if off_q is not None:
            idx[off_q] = idx[off_q] + delta
        return g[tuple(idx[q] for q in reversed(range(nd)))]

    c0 = at()
    grad = [0.5 * (at(q, 1) - at(q, -1)) for q in range(nd)]
    v = c0 + rel[0] * grad[0]
    v = v + rel[1] * grad[1]
    if nd == 3:
        v = v + rel[2] * grad[2]
    else:
        v = v + 0.0 * 0.0  # krel * crsegrad.z of the 2D build: turns -0 into +0
    return v.reshape(-1)


def transfer_reference(tb_old, x_old, tb_new, bc_type, bc_val):
    """x_old: the old tree's field on every block (non-leaf values are
    replaced by the average of their children first); bc_type: the new
    tree's math BC per block face [num_blocks*6]; bc_val: value per face
    position [6].  Returns (x_new [num_blocks*ncell], new-block flags)."""
    nd, nb = int(tb_new["ndim"]), int(tb_new["nb"])
    ncell = nb ** nd
    xo = average_down(tb_old, x_old)
    where = {_path_key(tb_old, b): b for b in range(int(tb_old["num_blocks"]))}
    nbk = int(tb_new["num_blocks"])
    x = np.zeros((nbk, ncell))
    new = np.zeros(nbk, dtype=np.int32)
    for b in range(nbk):
        ob = where.get(_path_key(tb_new, b))
        if ob is None:
            new[b] = 1
        else:
            x[b] = xo[ob]
    level = np.asarray(tb_new["level"])
    for lv in sorted(set(level[new == 1].tolist())):
        for b in np.nonzero((new == 1) & (level == lv))[0]:
            x[b] = _centered_linear(tb_new, x, int(b), bc_type, bc_val)
    return x.reshape(-1), new


def transfer_injection(tb_old, x_old, tb_new):
    """copy / injection from the nearest old leaf ancestor / average of old
    children / zero, on the new tree's leaves.  Returns (x_new, counts of the
    four kinds)."""
    nd, nb = int(tb_new["ndim"]), int(tb_new["nb"])
    ncell, half = nb ** nd, nb // 2
    x_old = np.asarray(x_old, dtype=np.float64).reshape(-1, ncell)
    where = {_path_key(tb_old, b): b for b in range(int(tb_old["num_blocks"]))}
    old_leaf = np.asarray(tb_old["node_type"]) == 1
    out = np.zeros((int(tb_new["num_blocks"]), ncell))
    c = np.arange(ncell)
    ijk = [c % nb, (c // nb) % nb if nd >= 2 else 0 * c, c // (nb * nb) if nd == 3 else 0 * c]

    def encode(v):
        r = v[0] + nb * v[1]
        return r + nb * nb * v[2] if nd == 3 else r

    kinds = [0, 0, 0, 0]
    for b in np.nonzero(np.asarray(tb_new["node_type"]) == 1)[0]:
        root, path = _path_key(tb_new, b)
        ob = where.get((root, path))
        if ob is not None and old_leaf[ob]:
            out[b] = x_old[ob]
            kinds[0] += 1
            continue
        if ob is None:
            oa, up = None, 0
            for up in range(1, len(path) + 1):
                oa = where.get((root, path[:len(path) - up]))
                if oa is not None:
                    break
            if oa is not None and old_leaf[oa]:
                pc = [a.copy() for a in ijk]
                for digit in reversed(path[len(path) - up:]):
                    for q in range(nd):
                        pc[q] = ((digit >> q) & 1) * half + (pc[q] >> 1)
                out[b] = x_old[oa][encode(pc)]
                kinds[1] += 1
                continue
        if ob is not None:
            kids = np.asarray(tb_old["child"]).reshape(-1, 8)[ob][:1 << nd]
            if np.all(kids >= 0) and np.all(old_leaf[kids]):
                sq = [(a >= half).astype(int) for a in ijk]
                cidx = sum(sq[q] << q for q in range(nd))
                fb = [2 * (ijk[q] - sq[q] * half) for q in range(nd)] + [0] * (3 - nd)
                acc = np.zeros(ncell)
                for kk in range(2 if nd == 3 else 1):
                    for jj in range(2):
                        for ii in range(2):
                            acc = acc + x_old[kids[cidx], encode([fb[0] + ii, fb[1] + jj, fb[2] + kk])]
                out[b] = acc / float(1 << nd)
                kinds[2] += 1
                continue
        kinds[3] += 1
    return out.reshape(-1), kinds
