"""ORACLE — test infrastructure only. Sparse Cholesky factorisation of the
Newton system, standing in for the reference's CHOLMOD call
(``Math/DIRECT_SOLVER.h:13-65``: ``cholmod_analyze`` + ``cholmod_factorize``
+ ``cholmod_solve``; a factorisation that meets a non-positive pivot returns
failure and the Newton loop switches to gradient descent,
``FEM/Shell/IMPLICIT_EULER.h:515-546``).

CHOLMOD itself (SuiteSparse, with MKL) is not available here, so this is a
multifrontal Cholesky of our own:

* ordering: nested dissection of the vertex graph (3x3 blocks) by geometric
  bisection: a node's vertices are split at the median of their longest
  bounding-box axis, and the vertices of one half that touch the other half
  form the separator, eliminated after both halves; parts of at most
  ``leaf`` vertices are eliminated as one front;
* symbolic: the dissection tree is the assembly tree; a front holds its own
  vertices' DOFs and the later DOFs its subtree couples to;
* numeric: per front, LAPACK/BLAS (potrf, trsm, syrk through SciPy) on the
  dense front, update matrices extend-added into the parent front;
* solve: forward and backward substitution over the tree.

Nothing in the product imports this module.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp


class NotPositiveDefinite(Exception):
    pass


def _extend_add(F11, F21, F22, U, li):
    """Adds a child's update matrix U (lower triangle, column-major) into the
    parent front's blocks at the front positions li (ascending), by the
    oracle library's loop."""
    import ctypes as C

    import oracle as O

    vp = lambda a: C.c_void_p(a.ctypes.data)
    O.lib().ora_extend_add(vp(F11), vp(F21), vp(F22), C.c_long(F11.shape[0]), C.c_long(F22.shape[0]), vp(U),
                           C.c_long(U.shape[0]), vp(li))


def _ranges(starts, lens):
    """Concatenation of arange(s, s + l) for every (s, l)."""
    tot = int(lens.sum())
    if tot == 0:
        return np.zeros(0, np.int64)
    off = np.repeat(np.cumsum(lens) - lens, lens)
    return np.repeat(starts, lens) + (np.arange(tot) - off)


class _Node:
    __slots__ = ("own", "children", "bnd", "L11", "L21", "dofs", "bdofs")

    def __init__(self, own, children):
        self.own = own
        self.children = children


class SparseCholesky:
    """Factor an SPD matrix H (3V x 3V, CSR) whose DOFs come in vertex triples;
    ``coords`` (V x 3) steer the dissection."""

    def __init__(self, H, coords, leaf=96):
        H = sp.csr_matrix(H)
        n = H.shape[0]
        assert n % 3 == 0
        V = n // 3
        self.n = n
        # vertex graph
        Hc = H.tocoo()
        g = sp.coo_matrix((np.ones(Hc.nnz, np.int8), (Hc.row // 3, Hc.col // 3)), shape=(V, V)).tocsr()
        g.sum_duplicates()
        self._gptr, self._gind = g.indptr.astype(np.int64), g.indices.astype(np.int64)
        self._coords = np.asarray(coords, np.float64)
        self._leaf = leaf
        self._side = np.full(V, -1, np.int8)
        self.root = self._dissect(np.arange(V, dtype=np.int64))
        # postorder: children first, own vertices consecutive
        self.order = []
        post = []
        stack = [(self.root, False)]
        while stack:
            nd, done = stack.pop()
            if done:
                post.append(nd)
                continue
            stack.append((nd, True))
            for c in reversed(nd.children):
                stack.append((c, False))
        self.post = post
        pos = np.empty(V, np.int64)
        k = 0
        for nd in post:
            pos[nd.own] = np.arange(k, k + nd.own.size)
            k += nd.own.size
        self._pos = pos
        self._symbolic()
        self._factor(H)

    # ---------------------------------------------------------------- ordering
    def _dissect(self, verts):
        if verts.size <= self._leaf:
            return _Node(verts, [])
        P = self._coords[verts]
        ax = int(np.argmax(P.max(0) - P.min(0)))
        o = np.argsort(P[:, ax], kind="stable")
        half = verts.size // 2
        left, right = verts[o[:half]], verts[o[half:]]
        side = self._side
        side[left] = 0
        side[right] = 1
        # the vertices of either half that touch the other half; the smaller
        # of the two sets is the separator
        seps = []
        for a, b in ((left, 1), (right, 0)):
            lens = self._gptr[a + 1] - self._gptr[a]
            nb = self._gind[_ranges(self._gptr[a], lens)]
            seps.append(np.unique(np.repeat(a, lens)[side[nb] == b]))
        side[verts] = -1
        j = 0 if seps[0].size <= seps[1].size else 1
        sep = seps[j]
        if sep.size >= min(left.size, right.size):  # no useful split: one front
            return _Node(verts, [])
        if j == 0:
            left = left[np.isin(left, sep, assume_unique=True, invert=True)]
        else:
            right = right[np.isin(right, sep, assume_unique=True, invert=True)]
        kids = [self._dissect(left), self._dissect(right)]
        return _Node(sep, [k for k in kids if k.own.size or k.children])

    def _symbolic(self):
        pos = self._pos
        for nd in self.post:
            own = nd.own
            last = pos[own].max() if own.size else -1
            lens = self._gptr[own + 1] - self._gptr[own]
            nb = self._gind[_ranges(self._gptr[own], lens)]
            parts = [nb[pos[nb] > last]]
            for c in nd.children:
                parts.append(c.bnd[pos[c.bnd] > last])
            b = np.unique(np.concatenate(parts)) if parts else np.zeros(0, np.int64)
            nd.bnd = b[np.argsort(pos[b], kind="stable")]
            nd.dofs = (3 * own[:, None] + np.arange(3)).reshape(-1)
            nd.bdofs = (3 * nd.bnd[:, None] + np.arange(3)).reshape(-1)

    # ---------------------------------------------------------------- numeric
    def _factor(self, H):
        upd = {}
        idx_of = np.full(self.n, -1, np.int64)
        potrf, trsm, syrk = sla.lapack.dpotrf, sla.blas.dtrsm, sla.blas.dsyrk
        for nd in self.post:
            k = nd.dofs.size
            front = np.concatenate([nd.dofs, nd.bdofs])
            m = front.size
            r = m - k
            # front blocks, column-major, lower triangles only: F11 (k x k),
            # F21 (r x k), F22 (r x r)
            rows = H[nd.dofs][:, front].toarray()
            F11 = np.asfortranarray(rows[:, :k])
            F21 = np.asfortranarray(rows[:, k:].T)
            F22 = np.zeros((r, r), order="F")
            if nd.children:
                idx_of[front] = np.arange(m)
                for c in nd.children:
                    U = upd.pop(id(c))
                    if U is None:
                        continue
                    _extend_add(F11, F21, F22, U, np.ascontiguousarray(idx_of[c.bdofs]))
            L11, info = potrf(F11, lower=1, overwrite_a=1, clean=1)
            if info != 0 or not np.all(np.isfinite(np.diagonal(L11))):
                raise NotPositiveDefinite(f"pivot {info}")
            nd.L11 = L11
            if r:
                L21 = trsm(1.0, L11, F21, side=1, lower=1, trans_a=1, overwrite_b=1)
                nd.L21 = L21
                upd[id(nd)] = syrk(-1.0, L21, beta=1.0, c=F22, lower=1, overwrite_c=1)
            else:
                nd.L21 = np.zeros((0, k))
                upd[id(nd)] = None

    def solve(self, b):
        y = np.array(b, dtype=np.float64, copy=True)
        for nd in self.post:
            yo = sla.solve_triangular(nd.L11, y[nd.dofs], lower=True, check_finite=False)
            y[nd.dofs] = yo
            if nd.bdofs.size:
                y[nd.bdofs] -= nd.L21 @ yo
        for nd in reversed(self.post):
            r = y[nd.dofs]
            if nd.bdofs.size:
                r = r - nd.L21.T @ y[nd.bdofs]
            y[nd.dofs] = sla.solve_triangular(nd.L11, r, lower=True, trans="T", check_finite=False)
        return y


def solve_spd(H, b, coords):
    """x with H x = b, or None when H is not positive definite (the
    reference's Solve_Direct returning false)."""
    try:
        f = SparseCholesky(H, coords)
    except NotPositiveDefinite:
        return None
    x = f.solve(b)
    return x if np.all(np.isfinite(x)) else None
