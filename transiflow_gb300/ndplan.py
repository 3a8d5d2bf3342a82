"""Nested-dissection elimination plan for the structured staggered grid.

The Jacobian couples a cell only to cells at Chebyshev distance <= 1, so a
plane of cells one cell thick separates a box of cells into two independent
halves.  Recursive bisection of the cell box gives a multifrontal elimination
tree: each internal node owns one separator plane, each leaf owns a small box
of cells.  A node's frontal matrix holds its own unknowns followed by its
boundary unknowns -- the cells in the one-cell ring around its box, which all
lie in ancestor separators -- so the Schur complement left after eliminating
the own unknowns is an update for ancestors only.

The plan is computed once per grid on the host and uploaded as flat int32
index arrays; the numeric factorisation and the solves run on the GPU.  Nodes
are grouped by height (leaves first); every node of one height is processed by
the same batched kernel launches.

This module has no dependency on the reference; ``numeric_reference`` is a
NumPy model of the device numerics used by the host-side unit tests.
"""

import numpy as np

__all__ = ['Plan', 'build_plan']


class _Node:
    __slots__ = ('lo', 'hi', 'own', 'bnd', 'children', 'parent', 'height', 'id')

    def __init__(self, lo, hi):
        self.lo, self.hi = lo, hi
        self.own = None
        self.bnd = None
        self.children = []
        self.parent = -1
        self.height = 0
        self.id = -1


def _cells_in(lo, hi, shape):
    nx, ny, nz = shape
    i = np.arange(lo[0], hi[0])
    j = np.arange(lo[1], hi[1])
    k = np.arange(lo[2], hi[2])
    K, J, I = np.meshgrid(k, j, i, indexing='ij')
    return (I + nx * (J + ny * K)).ravel()


def _ring(lo, hi, shape):
    """Cells at Chebyshev distance 1 outside the box, inside the grid."""
    nx, ny, nz = shape
    glo = [max(lo[a] - 1, 0) for a in range(3)]
    ghi = [min(hi[a] + 1, shape[a]) for a in range(3)]
    outer = _cells_in(glo, ghi, shape)
    i = outer % nx
    j = (outer // nx) % ny
    k = outer // (nx * ny)
    inside = (i >= lo[0]) & (i < hi[0]) & (j >= lo[1]) & (j < hi[1]) & (k >= lo[2]) & (k < hi[2])
    return np.sort(outer[~inside])


class Plan:
    """Flat arrays describing the elimination tree (see module docstring)."""


def build_plan(nx, ny, nz, dof, rowptr, cols, leaf_cells=48, pressure_var=None, gauge_cell=0):
    """Build the plan for a grid and its (fixed) sparsity pattern.

    ``rowptr``/``cols`` describe the stencil CSR the device assembles into;
    every stored entry (including zero padding) is routed to exactly one
    frontal matrix or dropped when its column lies outside the front.

    Incompressibility makes the pressure of a box bounded by walls and
    not-yet-eliminated faces determined only up to a constant, so the own
    block of such a box is singular.  Every node whose box does not contain
    the gauge cell therefore hands one pressure unknown (``pressure_var``) up
    to its parent, which keeps each eliminated block nonsingular.
    """
    shape = (nx, ny, nz)
    root = _Node((0, 0, 0), shape)
    nodes = []
    stack = [root]
    while stack:
        v = stack.pop()
        ext = [v.hi[a] - v.lo[a] for a in range(3)]
        ncell = ext[0] * ext[1] * ext[2]
        a = int(np.argmax(ext))
        if ncell <= leaf_cells or ext[a] < 3:
            v.own = _cells_in(v.lo, v.hi, shape)
        else:
            m = v.lo[a] + ext[a] // 2
            slo, shi = list(v.lo), list(v.hi)
            slo[a], shi[a] = m, m + 1
            v.own = _cells_in(slo, shi, shape)
            l_hi = list(v.hi)
            l_hi[a] = m
            r_lo = list(v.lo)
            r_lo[a] = m + 1
            for lo, hi in ((v.lo, tuple(l_hi)), (tuple(r_lo), v.hi)):
                if all(hi[b] > lo[b] for b in range(3)):
                    c = _Node(tuple(lo), tuple(hi))
                    v.children.append(c)
                    stack.append(c)
        v.bnd = _ring(v.lo, v.hi, shape)
        nodes.append(v)
    # heights and a children-first order
    def height(v):
        if not v.children:
            v.height = 0
        else:
            v.height = 1 + max(height(c) for c in v.children)
        return v.height
    height(root)
    nodes.sort(key=lambda v: (v.height, v.lo))
    for t, v in enumerate(nodes):
        v.id = t
    for v in nodes:
        for c in v.children:
            c.parent = v.id

    N = nx * ny * nz * dof
    d = np.arange(dof)
    own_u = [(v.own[:, None] * dof + d).ravel() for v in nodes]
    bnd_u = [(v.bnd[:, None] * dof + d).ravel() for v in nodes]
    if pressure_var is not None:
        gi, gj, gk = gauge_cell % nx, (gauge_cell // nx) % ny, gauge_cell // (nx * ny)
        for t, v in enumerate(nodes):          # children before parents
            if v.parent < 0:
                continue
            inside = all(v.lo[a] <= (gi, gj, gk)[a] < v.hi[a] for a in range(3))
            if inside:
                continue
            o = own_u[t]
            cand = np.flatnonzero(o % dof == pressure_var)
            if not len(cand):
                continue
            q = o[cand[0]]
            own_u[t] = np.delete(o, cand[0])
            own_u[v.parent] = np.append(own_u[v.parent], q)
            bnd_u[t] = np.sort(np.append(bnd_u[t], q))
    p = Plan()
    p.nx, p.ny, p.nz, p.dof, p.n = nx, ny, nz, dof, N
    p.nnodes = len(nodes)
    p.height = np.array([v.height for v in nodes], dtype=np.int32)
    p.parent = np.array([v.parent for v in nodes], dtype=np.int32)
    p.n_own = np.array([len(o) for o in own_u], dtype=np.int32)
    p.n_bnd = np.array([len(b) for b in bnd_u], dtype=np.int32)
    p.f = p.n_own + p.n_bnd
    # unknown index lists: own then boundary, per node
    p.idx_off = np.zeros(p.nnodes + 1, dtype=np.int64)
    p.idx_off[1:] = np.cumsum(p.f)
    p.idx = np.concatenate([np.concatenate([o, b]) for o, b in zip(own_u, bnd_u)]).astype(np.int32)
    # dense front storage offsets (f x f row-major)
    p.front_off = np.zeros(p.nnodes + 1, dtype=np.int64)
    p.front_off[1:] = np.cumsum(p.f.astype(np.int64) ** 2)
    # which node owns each unknown, and its local position there
    owner = np.full(N, -1, dtype=np.int64)
    local = np.full(N, -1, dtype=np.int64)
    for t, o in enumerate(own_u):
        owner[o] = t
        local[o] = np.arange(len(o))
    assert (owner >= 0).all(), 'every unknown must be eliminated exactly once'
    # route matrix entries: entry (r, c) goes to the node that eliminates the
    # earlier of r and c (the lower node in the tree)
    rowptr = np.asarray(rowptr, dtype=np.int64)
    cols = np.asarray(cols, dtype=np.int64)
    rows = np.repeat(np.arange(N), np.diff(rowptr))
    orow, ocol = owner[rows], owner[cols]
    tgt = np.where(p.height[orow] < p.height[ocol], orow,
                   np.where(p.height[orow] > p.height[ocol], ocol, np.minimum(orow, ocol)))
    # position of r and c inside the target front: one sorted table of
    # (node, unknown) keys over every front's index list, searched for all
    # entries at once
    node_of = np.repeat(np.arange(p.nnodes, dtype=np.int64), p.f)
    local_of = np.arange(len(p.idx), dtype=np.int64) - p.idx_off[node_of]
    keys = node_of * N + p.idx
    korder = np.argsort(keys, kind='stable')
    skeys = keys[korder]
    slocal = local_of[korder]
    pos_r = np.full(len(rows), -1, dtype=np.int64)
    pos_c = np.full(len(rows), -1, dtype=np.int64)
    for src, dst in ((rows, pos_r), (cols, pos_c)):
        want = tgt * N + src
        q = np.minimum(np.searchsorted(skeys, want), len(skeys) - 1)
        hit = skeys[q] == want
        dst[hit] = slocal[q[hit]]
    keep = (pos_r >= 0) & (pos_c >= 0)
    # an entry whose row and column are both boundary unknowns of its front
    # cannot occur for true couplings; padding entries that land there are
    # zero and are dropped
    n_own_t = p.n_own[tgt]
    keep &= (pos_r < n_own_t) | (pos_c < n_own_t)
    ent = np.flatnonzero(keep)
    order = np.lexsort((ent, tgt[ent]))
    ent = ent[order]
    p.scat_node = tgt[ent].astype(np.int32)
    p.scat_pos = (p.front_off[tgt[ent]] + pos_r[ent] * p.f[tgt[ent]] + pos_c[ent]).astype(np.int64)
    p.scat_src = ent.astype(np.int32)
    # extend-add: child boundary unknown -> parent front position
    p.ea_map_off = np.zeros(p.nnodes + 1, dtype=np.int64)
    maps = []
    for t, v in enumerate(nodes):
        if v.parent < 0:
            maps.append(np.zeros(0, dtype=np.int32))
            continue
        P = v.parent
        fidx = p.idx[p.idx_off[P]:p.idx_off[P + 1]]
        order = np.argsort(fidx)
        q = np.searchsorted(fidx[order], bnd_u[t])
        assert np.array_equal(fidx[order][q], bnd_u[t]), 'child boundary not inside parent front'
        maps.append(order[q].astype(np.int32))
    p.ea_map_off[1:] = np.cumsum([len(m) for m in maps])
    p.ea_map = np.concatenate(maps).astype(np.int32) if maps else np.zeros(0, np.int32)
    p.levels = [np.flatnonzero(p.height == h).astype(np.int32) for h in range(int(p.height.max()) + 1)]
    p.flops = float(np.sum(2.0 / 3.0 * p.n_own.astype(float) ** 3
                           + 2.0 * p.n_own.astype(float) ** 2 * p.n_bnd
                           + 2.0 * p.n_own.astype(float) * p.n_bnd.astype(float) ** 2))
    return p


def numeric_reference(p, vals, rhs):
    """NumPy model of the device factorisation and solve (host unit tests).

    Partial LU of each front with row pivoting restricted to its own rows,
    Schur complements extend-added into the parent, then a forward and a
    backward sweep over the tree.
    """
    F = [np.zeros((p.f[t], p.f[t])) for t in range(p.nnodes)]
    for node, pos, src in zip(p.scat_node, p.scat_pos, p.scat_src):
        loc = pos - p.front_off[node]
        F[node].flat[loc] += vals[src]
    piv = []
    for t in range(p.nnodes):
        A = F[t]
        n = p.n_own[t]
        perm = np.arange(p.f[t])
        for c in range(n):
            r = c + int(np.argmax(np.abs(A[c:n, c])))
            if r != c:
                A[[c, r]] = A[[r, c]]
                perm[[c, r]] = perm[[r, c]]
            A[c + 1:, c] /= A[c, c]
            A[c + 1:, c + 1:] -= np.outer(A[c + 1:, c], A[c, c + 1:])
        piv.append(perm)
        if p.parent[t] >= 0:
            m = p.ea_map[p.ea_map_off[t]:p.ea_map_off[t + 1]]
            F[p.parent[t]][np.ix_(m, m)] += A[n:, n:]
    x = np.array(rhs, dtype=np.float64)
    for t in range(p.nnodes):
        A, n = F[t], p.n_own[t]
        g = p.idx[p.idx_off[t]:p.idx_off[t + 1]]
        own = x[g[:n]][piv[t][:n]]
        for c in range(n):
            own[c + 1:] -= A[c + 1:n, c] * own[c]
        x[g[:n]] = own
        x[g[n:]] -= A[n:, :n] @ own
    for t in reversed(range(p.nnodes)):
        A, n = F[t], p.n_own[t]
        g = p.idx[p.idx_off[t]:p.idx_off[t + 1]]
        y = x[g[:n]] - A[:n, n:] @ x[g[n:]]
        for c in reversed(range(n)):
            y[c] = (y[c] - A[c, c + 1:n] @ y[c + 1:n]) / A[c, c]
        x[g[:n]] = y
    return x
