"""ORACLE — test infrastructure only. ctypes bindings to the CPU restatement
(``oracle/libidp_oracle.so``) and the Newton driver restating
``FEM/Shell/IMPLICIT_EULER.h:9-891`` for tet meshes with offset IPC contact.

Only tests/, ``__graft_entry__.smoke()`` and the cpu_baseline leg of
bench.py import this module; the product never does.

Parity status: UNPINNED (the reference ships no tests or golden vectors and
cannot be built here). The linear solve is a sparse Cholesky of our own
(``oracle/cholesky.py``, multifrontal with nested dissection) in place of
CHOLMOD (``Math/DIRECT_SOLVER.h:13-65``).
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

try:
    from . import cholesky
except ImportError:  # imported as a top-level module (oracle/ on sys.path)
    import cholesky

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "libidp_oracle.so")
_lib = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_up = C.POINTER(C.c_ubyte)


def build(force=False):
    """Compile the oracle with its Makefile (g++ -ffp-contract=off)."""
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < max(
        os.path.getmtime(os.path.join(_HERE, f)) for f in ("idp_oracle.cpp", "geom.hpp", "deriv.hpp", "shell.hpp")
    ):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB)
        L.ora_surface.restype = C.c_int
        L.ora_tet_energy.restype = C.c_int
        L.ora_constraint_set.restype = C.c_int
        L.ora_barrier_energy.restype = C.c_double
        L.ora_min_dist2.restype = C.c_double
        L.ora_ccd_stepsize.restype = C.c_int
        L.ora_kappa_init.restype = C.c_double
        L.ora_type_pt.restype = C.c_int
        L.ora_type_ee.restype = C.c_int
        L.ora_dist_pt_unclassified.restype = C.c_double
        L.ora_dist_ee_unclassified.restype = C.c_double
        L.ora_orient3d.restype = C.c_int
        L.ora_shell_init.restype = C.c_int
        L.ora_shell_surface.restype = C.c_int
        L.ora_flow_energy.restype = C.c_double
        L.ora_edge_tri_intersections.restype = C.c_long
        L.ora_edge_tri_intersections.argtypes = [C.c_int, _ip, C.c_int, _ip, _dp, _up, C.c_long, _ip]
        L.ora_membrane.restype = C.c_double
        L.ora_bending.restype = C.c_double
        L.ora_dihedral.restype = C.c_double
        L.ora_shell_hinges.restype = C.c_int
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def _u(a):
    return a.ctypes.data_as(_up)


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


# ---------------------------------------------------------------- wrappers
def surface(X, tets):
    X, tets = f64(X), i32(tets)
    V, T = X.shape[0], tets.shape[0]
    capT, capE = 4 * T, 6 * T
    tris = np.zeros((capT, 3), np.int32)
    edges = np.zeros((capE, 2), np.int32)
    nodes = np.zeros(V, np.int32)
    A_t, A_e, A_n = np.zeros(capT), np.zeros(capE), np.zeros(V)
    nT, nE, nN = C.c_int(), C.c_int(), C.c_int()
    rc = lib().ora_surface(V, T, _i(tets), _d(X), capT, capE, C.byref(nT), _i(tris), C.byref(nE), _i(edges),
                           C.byref(nN), _i(nodes), _d(A_t), _d(A_e), _d(A_n))
    assert rc == 0
    return dict(tris=tris[: nT.value].copy(), edges=edges[: nE.value].copy(), nodes=nodes[: nN.value].copy(),
                tri_area=A_t[: nT.value].copy(), edge_area=A_e[: nE.value].copy(), node_area=A_n[: nN.value].copy())


def tet_rest(X, tets):
    X, tets = f64(X), i32(tets)
    T = tets.shape[0]
    IB, vol = np.zeros((T, 3, 3)), np.zeros(T)
    lib().ora_tet_rest(T, _i(tets), _d(X), _d(IB), _d(vol))
    return IB, vol


def tet_energy(X, tets, IB, vol, lam, mu, w):
    E = C.c_double()
    ok = lib().ora_tet_energy(tets.shape[0], _i(tets), _d(f64(X)), _d(IB), _d(vol), _d(lam), _d(mu), C.c_double(w), C.byref(E))
    return (E.value if ok else None)


def tet_gradient(X, tets, IB, vol, lam, mu, w):
    g = np.zeros(X.size)
    lib().ora_tet_gradient(X.shape[0], tets.shape[0], _i(tets), _d(f64(X)), _d(IB), _d(vol), _d(lam), _d(mu), C.c_double(w), _d(g))
    return g


def tet_hessian(X, tets, IB, vol, lam, mu, w, project=True):
    H = np.zeros((tets.shape[0], 12, 12))
    lib().ora_tet_hessian(tets.shape[0], _i(tets), _d(f64(X)), _d(IB), _d(vol), _d(lam), _d(mu), C.c_double(w), int(project), _d(H))
    return H


def constraint_set(X, X0, surf, dbc, dHat2, thickness=0.0):
    X, X0 = f64(X), f64(X0)
    cap = max(1024, 8 * (surf["nodes"].size + surf["edges"].shape[0]))
    while True:
        cons = np.zeros((cap, 4), np.int32)
        info = np.zeros((cap, 2))
        n = lib().ora_constraint_set(X.shape[0], _d(X), _d(X0), surf["nodes"].size, _i(surf["nodes"]),
                                     surf["edges"].shape[0], _i(surf["edges"]), surf["tris"].shape[0], _i(surf["tris"]),
                                     _u(dbc), C.c_double(dHat2), C.c_double(thickness), cap, _i(cons), _d(info))
        if n >= 0:
            return cons[:n].copy(), info[:n].copy()
        cap = -n


def barrier_energy(cons, info, X, X0, dHat2, kappa, thickness=0.0):
    if cons.shape[0] == 0:
        return 0.0
    return lib().ora_barrier_energy(cons.shape[0], _i(cons), _d(info), _d(f64(X)), _d(f64(X0)), C.c_double(dHat2),
                                    C.c_double(kappa), C.c_double(thickness))


def barrier_gradient(cons, info, X, X0, dHat2, kappa, thickness=0.0):
    g = np.zeros(X.size)
    if cons.shape[0]:
        lib().ora_barrier_gradient(cons.shape[0], _i(cons), _d(info), _d(f64(X)), _d(f64(X0)), C.c_double(dHat2),
                                   C.c_double(kappa), C.c_double(thickness), _d(g))
    return g


def barrier_hessian(cons, info, X, X0, dHat2, kappa, thickness=0.0, project=True):
    n = cons.shape[0]
    verts = np.zeros((n, 4), np.int32)
    H = np.zeros((n, 144))
    if n:
        lib().ora_barrier_hessian(n, _i(cons), _d(info), _d(f64(X)), _d(f64(X0)), C.c_double(dHat2), C.c_double(kappa),
                                  C.c_double(thickness), int(project), _i(verts), _d(H))
    return verts, H


def min_dist2(cons, X, thickness=0.0):
    d2 = np.zeros(cons.shape[0])
    if cons.shape[0] == 0:
        return math.inf, d2
    m = lib().ora_min_dist2(cons.shape[0], _i(cons), _d(f64(X)), C.c_double(thickness), _d(d2))
    return m, d2


def ccd_stepsize(X, dirn, surf, dbc, alpha=1.0, thickness=0.0):
    a = C.c_double(alpha)
    rc = lib().ora_ccd_stepsize(surf["nodes"].size, _i(surf["nodes"]), surf["edges"].shape[0], _i(surf["edges"]),
                                surf["tris"].shape[0], _i(surf["tris"]), _u(dbc), _d(f64(X)), _d(f64(dirn)),
                                C.c_double(thickness), C.byref(a))
    return a.value, rc


def shell_init(X, faces, rho, thickness):
    """Face filter, lumped mass and element volumes of a triangle shell
    (Initialize_Discrete_Shell, DISCRETE_SHELL.h:238-333): (keep, mass, vol)."""
    X, faces = f64(X), i32(faces)
    V, F = X.shape[0], faces.shape[0]
    keep, mass, vol = np.zeros(F, np.uint8), np.zeros(V), np.zeros(F)
    lib().ora_shell_init(V, F, _i(faces), _d(X), C.c_double(rho), C.c_double(thickness), _u(keep), _d(mass),
                         _d(vol))
    return keep.astype(bool), mass, vol


def shell_surface(V, faces):
    """Find_Surface_Primitives (MESHIO.h:728-766) of a triangle shell."""
    faces = i32(faces)
    F = faces.shape[0]
    edges, nodes = np.zeros((3 * F, 2), np.int32), np.zeros(V, np.int32)
    ne, nn = C.c_int(), C.c_int()
    rc = lib().ora_shell_surface(V, F, _i(faces), 3 * F, _i(edges), C.byref(ne), _i(nodes), C.byref(nn))
    assert rc == 0
    return {"tris": faces.copy(), "edges": edges[: ne.value].copy(), "nodes": nodes[: nn.value].copy()}


def flow_energy(X, faces, vol, h):
    X, faces = f64(X), i32(faces)
    return lib().ora_flow_energy(X.shape[0], faces.shape[0], _i(faces), _d(f64(vol)), _d(X), C.c_double(h))


def flow_gradient(X, faces, vol, h):
    X, faces = f64(X), i32(faces)
    g = np.zeros(X.size)
    lib().ora_flow_gradient(X.shape[0], faces.shape[0], _i(faces), _d(f64(vol)), _d(X), C.c_double(h), _d(g))
    return g


def flow_hessian(n_dof, faces, vol, h):
    """-h L as scipy CSR (INC_POTENTIAL.h:323-339)."""
    import scipy.sparse as sp

    faces = i32(faces)
    F = faces.shape[0]
    r, c, v = np.zeros(27 * F, np.int32), np.zeros(27 * F, np.int32), np.zeros(27 * F)
    lib().ora_flow_hessian(F, _i(faces), _d(f64(vol)), C.c_double(h), _i(r), _i(c), _d(v))
    return sp.coo_matrix((v, (r, c)), shape=(n_dof, n_dof)).tocsr()


def membrane_rest(X0, faces, thickness, E, nu):
    """Per-face rest data of the NH membrane (F, 7): inverse rest first
    fundamental form (00, 01, 11), its determinant, vol, lambda, mu."""
    X0, faces = f64(X0), i32(faces)
    mem = np.zeros((faces.shape[0], 7))
    lib().ora_membrane_rest(faces.shape[0], _i(faces), _d(X0), C.c_double(thickness), C.c_double(E), C.c_double(nu),
                            _d(mem))
    return mem


def membrane(X, faces, mem, w, grad=False, hess=False, project=True, dbc=None):
    """Membrane energy (and gradient 3V, element Hessians F x 9 x 9); faces
    with all three vertices fixed (dbc) are skipped."""
    X, faces = f64(X), i32(faces)
    g = np.zeros(X.size) if grad else None
    H = np.zeros((faces.shape[0], 9, 9)) if hess else None
    d = None if dbc is None else np.ascontiguousarray(dbc, np.uint8)
    E = lib().ora_membrane(faces.shape[0], _i(faces), _d(X), _d(f64(mem)), C.c_double(w),
                           _d(g) if grad else None, _d(H) if hess else None, int(project),
                           None if d is None else _u(d))
    return E, g, H


def shell_hinges(X0, faces, edges):
    """Hinge stencils (Hn, 4) and rest data (thetabar, ebar, hbar) of a shell."""
    X0, faces, edges = f64(X0), i32(faces), i32(edges)
    hin = np.zeros((edges.shape[0], 4), np.int32)
    info = np.zeros((edges.shape[0], 3))
    n = lib().ora_shell_hinges(X0.shape[0], faces.shape[0], _i(faces), _d(X0), edges.shape[0], _i(edges), _i(hin),
                               _d(info))
    return hin[:n].copy(), info[:n].copy()


def bending(X, hinges, info, k, w, grad=False, hess=False, project=True, dbc=None):
    """Hinge bending energy (and gradient 3V, element Hessians Hn x 12 x 12);
    hinges with all four vertices fixed (dbc) are skipped."""
    X, hinges = f64(X), i32(hinges)
    g = np.zeros(X.size) if grad else None
    H = np.zeros((hinges.shape[0], 12, 12)) if hess else None
    d = None if dbc is None else np.ascontiguousarray(dbc, np.uint8)
    E = lib().ora_bending(hinges.shape[0], _i(hinges), _d(f64(info)), C.c_double(k), _d(X), C.c_double(w),
                          _d(g) if grad else None, _d(H) if hess else None, int(project),
                          None if d is None else _u(d))
    return E, g, H


def dihedral(x):
    """Dihedral angle of a hinge (4 x 3) with its gradient (12) and Hessian (12 x 12)."""
    x = f64(x).reshape(-1)
    g, H = np.zeros(12), np.zeros(144)
    t = lib().ora_dihedral(_d(x), _d(g), _d(H))
    return t, g, H.reshape(12, 12)


def hinge_stiffness(E, nu, thickness, mult=1.0):
    """k = E t^3 / (24 (1 - nu^2)) times bendingStiffMult (DISCRETE_SHELL.h:344-349)."""
    return mult * E * thickness ** 3 / (24.0 * (1.0 - nu * nu))


def orient3d(a, b, c, d):
    """Exact sign of det[a-d; b-d; c-d]."""
    return lib().ora_orient3d(_d(f64(a)), _d(f64(b)), _d(f64(c)), _d(f64(d)))


def edge_tri_intersections(X, surf, dbc=None):
    """Intersecting (triangle, edge) pairs of a surface at X, sorted
    (Check_Edge_Tri_Intersect, FEM/IPC.h:2444-2517, exact predicates)."""
    tris, edges = i32(surf["tris"]), i32(surf["edges"])
    X = f64(X)
    dbc = np.zeros(X.shape[0], np.uint8) if dbc is None else np.ascontiguousarray(dbc, np.uint8)
    cap = 1024
    while True:
        out = np.zeros((cap, 2), np.int32)
        n = lib().ora_edge_tri_intersections(tris.shape[0], _i(tris), edges.shape[0], _i(edges), _d(X), _u(dbc), cap,
                                             _i(out))
        if n <= cap:
            return out[:n].copy()
        cap = n


def kappa_init(mean_mass_diag, dHat2, stiff_mult=1.0):
    km = C.c_double()
    k = lib().ora_kappa_init(C.c_double(mean_mass_diag), C.c_double(dHat2), C.c_double(stiff_mult), C.byref(km))
    return k, km.value


def dist_derivs(kind, x):
    x = f64(x).reshape(-1)
    xx = np.zeros(12)
    xx[: x.size] = x
    d = C.c_double()
    g, H = np.zeros(12), np.zeros(144)
    lib().ora_dist_derivs(kind, _d(xx), C.byref(d), _d(g), _d(H))
    n = {0: 6, 1: 9}.get(kind, 12)
    return d.value, g[:n].copy(), H[: n * n].reshape(n, n).copy()


def make_pd(A):
    A = f64(A).copy()
    lib().ora_make_pd(A.shape[0], _d(A))
    return A


def normal_flow_velocity(X, tris, step, h):
    """Velocity whose predictor moves surface vertices by ``step`` along the
    normalised sum of incident triangle normals (DISCRETE_SHELL.h:359-395)."""
    X = f64(X)
    tris = i32(tris)
    vel = np.zeros_like(X)
    lib().ora_normal_flow(X.shape[0], tris.shape[0], _i(tris), _d(X), C.c_double(step), C.c_double(h), _d(vel))
    return vel


# ---------------------------------------------------------------- Newton step
@dataclass
class Problem:
    """One tet mesh with everything Advance_One_Step_IE_Discrete_Shell reads
    for the tet + offset-IPC configuration."""
    X: np.ndarray            # (V,3) current positions (mutated)
    X0: np.ndarray           # (V,3) rest positions (mollifier threshold, IB)
    tets: np.ndarray         # (T,4) int32
    mass: np.ndarray         # (V,) lumped mass
    lam: np.ndarray          # (T,)
    mu: np.ndarray           # (T,)
    h: float
    dHat2: float
    kappa: list              # [kappa, kappa_max, 0]
    v: np.ndarray            # (V,3) velocity (mutated)
    dbc: np.ndarray = None   # (V,) uint8 fixed-DBC mask
    thickness: float = 0.0
    tol: float = 1e-3
    max_iters: int = 1000
    IB: np.ndarray = None
    vol: np.ndarray = None
    surf: dict = None
    log: list = field(default_factory=list)
    b: np.ndarray = None      # (V,3) body force (None: zero)
    faces: np.ndarray = None  # (F,3) shell faces: flow mode (Advance_One_Step_IE_Flow)
    fvol: np.ndarray = None   # (F,) shell element volumes (area * thickness)
    mem: np.ndarray = None    # (F,7) membrane rest data: an elastic shell (Hinge path) instead of flow mode
    hinges: np.ndarray = None  # (Hn,4) hinge stencils of an elastic shell
    hinfo: np.ndarray = None  # (Hn,3) thetabar, ebar, hbar
    kbend: float = 0.0        # hinge stiffness k
    dbc_rows: np.ndarray = None    # (R,) vertex of each DBC row, in the reference's row order
    dbc_target: np.ndarray = None  # (R,3) DBC target positions: moving DBC (augmented Lagrangian)

    @property
    def flow(self):
        return self.faces is not None and self.mem is None

    @property
    def elastic_shell(self):
        return self.faces is not None and self.mem is not None

    def __post_init__(self):
        self.X = f64(self.X).copy()
        self.X0 = f64(self.X0)
        if self.faces is not None:
            self.faces = i32(self.faces)
            self.tets = np.zeros((0, 4), np.int32)
        self.tets = i32(self.tets)
        if self.dbc is None:
            self.dbc = np.zeros(self.X.shape[0], np.uint8)
        if self.IB is None and self.faces is None:
            self.IB, self.vol = tet_rest(self.X0, self.tets)


def _energy(pb, X, Xtilde, with_barrier, cons, info):
    """Compute_IncPotential (INC_POTENTIAL.h:15-152); None when a tet inverts."""
    h2 = pb.h * pb.h
    if pb.flow:  # INC_POTENTIAL.h:53-73
        E = flow_energy(X, pb.faces, pb.fvol, pb.h)
    elif pb.elastic_shell:  # INC_POTENTIAL.h: membrane + hinge bending
        E = (membrane(X, pb.faces, pb.mem, h2, dbc=pb.dbc)[0]
             + bending(X, pb.hinges, pb.hinfo, pb.kbend, h2, dbc=pb.dbc)[0])
        if not np.isfinite(E):
            return None
    else:
        E = tet_energy(X, pb.tets, pb.IB, pb.vol, pb.lam, pb.mu, h2)
    if E is None:
        return None
    dx = (X - Xtilde)
    E += 0.5 * float(np.dot((pb.mass[:, None] * dx).reshape(-1), dx.reshape(-1)))
    if with_barrier:
        E += barrier_energy(cons, info, X, pb.X0, pb.dHat2, pb.kappa[0], pb.thickness)
    return E


def _gradient(pb, X, Xtilde, cons, info):
    """Compute_IncPotential_Gradient (INC_POTENTIAL.h:154-275)."""
    h2 = pb.h * pb.h
    if pb.flow:  # INC_POTENTIAL.h:191-211
        g = flow_gradient(X, pb.faces, pb.fvol, pb.h)
    elif pb.elastic_shell:
        g = (membrane(X, pb.faces, pb.mem, h2, grad=True, dbc=pb.dbc)[1]
             + bending(X, pb.hinges, pb.hinfo, pb.kbend, h2, grad=True, dbc=pb.dbc)[1])
    else:
        g = tet_gradient(X, pb.tets, pb.IB, pb.vol, pb.lam, pb.mu, h2)
    g += (pb.mass[:, None] * (X - Xtilde)).reshape(-1)
    g += barrier_gradient(cons, info, X, pb.X0, pb.dHat2, pb.kappa[0], pb.thickness)
    return g


def _hessian(pb, X, cons, info, proj=None, dpen=None):
    """Compute_IncPotential_Hessian (INC_POTENTIAL.h:277-395) as scipy CSR;
    proj: the rows projected to the identity (default pb.dbc), dpen: a
    per-vertex diagonal added to the Hessian (Compute_DBC_Hessian,
    Shell/DIRICHLET.h:72-90)."""
    import scipy.sparse as sp

    n = X.size
    h2 = pb.h * pb.h
    if pb.flow:  # INC_POTENTIAL.h:323-339
        Hf = flow_hessian(n, pb.faces, pb.fvol, pb.h).tocoo()
        R, Cc, Vv = [Hf.row], [Hf.col], [Hf.data]
    elif pb.elastic_shell:
        R, Cc, Vv = [], [], []
        for st, Hs in ((pb.faces, membrane(X, pb.faces, pb.mem, h2, hess=True, dbc=pb.dbc)[2]),
                       (pb.hinges, bending(X, pb.hinges, pb.hinfo, pb.kbend, h2, hess=True, dbc=pb.dbc)[2])):
            k = 3 * st.shape[1]
            dofs = (3 * st[:, :, None] + np.arange(3)).reshape(-1, k)
            R.append(np.repeat(dofs[:, :, None], k, axis=2).reshape(-1))
            Cc.append(np.repeat(dofs[:, None, :], k, axis=1).reshape(-1))
            Vv.append(Hs.reshape(-1))
    else:
        He = tet_hessian(X, pb.tets, pb.IB, pb.vol, pb.lam, pb.mu, h2, True)
        dofs = (3 * pb.tets[:, :, None] + np.arange(3)).reshape(-1, 12)
        rows = np.repeat(dofs[:, :, None], 12, axis=2).reshape(-1)
        cols = np.repeat(dofs[:, None, :], 12, axis=1).reshape(-1)
        vals = He.reshape(-1)
        R, Cc, Vv = [rows], [cols], [vals]
    if cons.shape[0]:
        verts, Hb = barrier_hessian(cons, info, X, pb.X0, pb.dHat2, pb.kappa[0], pb.thickness, True)
        for nv in (2, 3, 4):
            sel = (verts >= 0).sum(1) == nv
            if not sel.any():
                continue
            vd = (3 * verts[sel, :nv, None] + np.arange(3)).reshape(-1, 3 * nv)
            k = 3 * nv
            R.append(np.repeat(vd[:, :, None], k, axis=2).reshape(-1))
            Cc.append(np.repeat(vd[:, None, :], k, axis=1).reshape(-1))
            Vv.append(Hb[sel, : k * k].reshape(-1))
    R.append(np.arange(n))
    Cc.append(np.arange(n))
    Vv.append(np.repeat(pb.mass, 3))
    if dpen is not None:
        R.append(np.arange(n))
        Cc.append(np.arange(n))
        Vv.append(np.repeat(dpen, 3))
    H = sp.coo_matrix((np.concatenate(Vv), (np.concatenate(R), np.concatenate(Cc))), shape=(n, n)).tocsr()
    # Project_DBC (Math/CSR_MATRIX.h:130-141): DBC rows/cols -> identity
    pm = pb.dbc if proj is None else proj
    if pm.any():
        m = np.repeat(pm.astype(bool), 3)
        keep = sp.diags((~m).astype(float))
        H = keep @ H @ keep + sp.diags(m.astype(float))
    return H.tocsr()


def dbc_energy(pb, X, stiff):
    """Compute_DBC_Energy (Shell/DIRICHLET.h:26-45): stiff/2 sum m |t - x|^2
    over the DBC rows."""
    d = pb.dbc_target - X[pb.dbc_rows]
    return 0.5 * stiff * float(np.sum(pb.mass[pb.dbc_rows] * np.sum(d * d, axis=1)))


def dbc_dist2(pb, X):
    """Compute_DBC_Dist2 (Shell/DIRICHLET.h:6-24): sum |t - x|^2 over the rows."""
    d = pb.dbc_target - X[pb.dbc_rows]
    return float(np.sum(d * d))


def advance_one_step(pb: Problem, Xtilde=None, verbose=False, on_iter=None):
    """Advance_One_Step_IE_Discrete_Shell<double,3,false,false,false>
    (FEM/Shell/IMPLICIT_EULER.h:151-891) for tets or shells with fixed or
    moving DBC (the augmented Lagrangian of :305-401, 701-757), no friction.
    Returns the Newton iteration count; pb.X and pb.v are updated.
    on_iter(it, Xprev, direction, ncons) is called after each accepted
    Newton step with the iterate the direction was computed at and the size
    of the constraint set at that iterate."""
    h = pb.h
    Xn = pb.X.copy()
    if pb.flow:
        pb.v[:] = 0.0                     # IMPLICIT_EULER.h:207-209
    if Xtilde is None:                    # IMPLICIT_EULER.h:195-216
        if pb.b is None:
            Xtilde = Xn + h * pb.v
        else:                             # x + (h v + h^2 M^-1 b), M lumped
            Xtilde = Xn + (h * pb.v + (h * h) * (f64(pb.b).reshape(-1, 3) / pb.mass[:, None]))
    if pb.surf is None:                   # IMPLICIT_EULER.h:235-241
        pb.surf = shell_surface(pb.X.shape[0], pb.faces) if pb.faces is not None else surface(pb.X0, pb.tets)
    surf, dbc = pb.surf, pb.dbc
    nDBC = int(dbc.sum())
    X = pb.X
    # ---- Dirichlet conditions (IMPLICIT_EULER.h:305-401): rows whose target
    # is the current position are fixed; the others move by the CCD-safe
    # fraction of their displacement, all the way (alpha = 1) or, when
    # contact blocks the way, through the penalty stiff/2 sum m |t - x|^2
    stiff, pen0 = 0.0, 0.0
    proj = dbc
    if pb.dbc_target is not None:
        rows = np.asarray(pb.dbc_rows, np.int64)
        nDBC = rows.size
        disp = pb.dbc_target - X[rows]
        fixed = np.zeros_like(dbc)
        fixed[rows[~np.any(disp != 0, axis=1)]] = 1
        dirn = np.zeros_like(X)
        dirn[rows] = disp
        dbc_alpha = 1.0
        if np.any(disp != 0):
            dbc_alpha, rc = ccd_stepsize(X, dirn.reshape(-1), surf, dbc, 1.0, pb.thickness)
            if rc < 0:
                raise RuntimeError("zero CCD step for the DBC")
        pb.dbc_alpha = dbc_alpha
        if dbc_alpha == 1:
            X[rows] = pb.dbc_target
        else:
            stiff = 1e6
            pen0 = dbc_dist2(pb, Xn)
            proj = fixed
    dpen = None
    cons, info = constraint_set(X, pb.X0, surf, dbc, pb.dHat2, pb.thickness)

    def energy(Xe, barrier, c, i):
        E = _energy(pb, Xe, Xtilde, barrier, c, i)
        if E is not None and stiff:
            E += dbc_energy(pb, Xe, stiff)
        return E

    Eprev = energy(X, True, cons, info)
    progress_log = []
    res_record = deque()
    it = 0
    use_gd = False
    cons_prev, dist2_prev = np.zeros((0, 4), np.int32), np.zeros(0)
    stats = dict(ls_trials=0, ccd_calls=0, alphas=[], t_solve=0.0)
    while True:
        g = _gradient(pb, X, Xtilde, cons, info)
        if stiff:  # Compute_DBC_Gradient (Shell/DIRICHLET.h:47-70)
            gr = g.reshape(-1, 3)
            gr[pb.dbc_rows] += stiff * pb.mass[pb.dbc_rows, None] * (X[pb.dbc_rows] - pb.dbc_target)
            dpen = np.zeros(X.shape[0])
            dpen[pb.dbc_rows] = stiff * pb.mass[pb.dbc_rows]
        else:
            dpen = None
        if proj.any():
            g.reshape(-1, 3)[proj.astype(bool)] = 0
        rhs = -g
        if not use_gd:
            Hm = _hessian(pb, X, cons, info, proj=proj, dpen=dpen)
            t0 = time.perf_counter()
            sol = cholesky.solve_spd(Hm, rhs, X)  # Solve_Direct (DIRECT_SOLVER.h:13-65)
            stats["t_solve"] += time.perf_counter() - t0
            if sol is None:  # not positive definite: gradient descent (IMPLICIT_EULER.h:519-546)
                use_gd = True
                sol = rhs.copy()
        else:
            sol = rhs.copy()
        # ---- Line_Search (IMPLICIT_EULER.h:9-149)
        Xprev = X.copy()
        ncons_prev = int(cons.shape[0])
        p = sol.reshape(-1, 3)
        alpha = 1.0
        while True:
            Xt = Xprev + alpha * p
            if energy(Xt, False, cons, info) is not None:
                break
            alpha /= 2.0
        stats["ccd_calls"] += 1
        alpha, rc = ccd_stepsize(Xprev, sol, surf, dbc, alpha, pb.thickness)
        if rc < 0:
            raise RuntimeError("zero CCD step")
        feasible_alpha = alpha
        E = None
        while True:
            stats["ls_trials"] += 1
            Xt = Xprev + alpha * p
            E = energy(Xt, False, cons, info)
            valid = E is not None
            if valid:
                cons, info = constraint_set(Xt, pb.X0, surf, dbc, pb.dHat2, pb.thickness)
                if cons.shape[0]:
                    md, _ = min_dist2(cons, Xt, pb.thickness)
                    if md <= 0:
                        alpha /= 2
                        E = Eprev + 1
                        continue
                E = energy(Xt, True, cons, info)
            alpha /= 2.0
            if valid and not (E > Eprev):
                break
        X[:] = Xt
        Eprev = E
        stats["alphas"].append(alpha * 2)
        # ---- kappa adaptation (IMPLICIT_EULER.h:566-595)
        if cons_prev.shape[0]:
            _, cur = min_dist2(cons_prev, X, pb.thickness)
            upd = bool(np.any((dist2_prev < 1e-18) & (cur < dist2_prev)))
            if upd and pb.kappa[0] < pb.kappa[1]:
                pb.kappa[0] *= 2
                Eprev = energy(X, True, cons, info)
        dist2 = min_dist2(cons, X, pb.thickness)[1] if cons.shape[0] else np.zeros(0)
        cons_prev, dist2_prev = cons.copy(), dist2
        # ---- stopping criterion (IMPLICIT_EULER.h:647-676, 759, 855)
        n = sol.size // 3
        L2 = math.sqrt(float(np.dot(sol, sol)) / (n - nDBC)) / h
        it += 1
        res_record.append(L2)
        if len(res_record) > 3:
            res_record.popleft()
        L2m = max(res_record)
        if use_gd:
            L2m = pb.tol * 10
        if alpha * 2 < 1e-8 and feasible_alpha > 1e-8:
            use_gd = True
        else:
            use_gd = False
        if stiff:  # augmented Lagrangian progress (IMPLICIT_EULER.h:701-757)
            progress = 1 - math.sqrt(dbc_dist2(pb, X) / pen0)
            progress_log.append((it, progress, stiff))
            if progress < 0.99:
                if L2m < pb.tol * 10 and stiff < 1e8:
                    stiff *= 2
                    Eprev = energy(X, True, cons, info)
                L2m = pb.tol * 10
            else:
                stiff = 0.0
                proj = dbc
                Eprev = energy(X, True, cons, info)
        pb.log.append(dict(it=it, E=Eprev, res=L2, alpha=alpha * 2, ncons=int(cons.shape[0]), kappa=pb.kappa[0],
                           dbc_stiff=stiff))
        if on_iter is not None:
            on_iter(it, Xprev, sol, ncons_prev)
        if verbose:
            print(f"it {it} E {Eprev:.12e} res {L2:.3e} alpha {alpha*2:.3e} C {cons.shape[0]} kappa {pb.kappa[0]:.3e}")
        if (len(res_record) == 3 and L2m <= pb.tol) or it >= pb.max_iters:
            break
        if pb.flow and cons.shape[0] == 0:  # IMPLICIT_EULER.h:850-854
            break
    pb.v = (X - Xn) / h                     # IMPLICIT_EULER.h:882-888
    stats["dbc_progress"] = progress_log
    pb.last_stats = stats
    pb.last_energy = Eprev
    return it


def make_bar_problem(nx=6, ny=6, nz=24, size=(1.0, 1.0, 4.0), angle=2.2 * math.pi, seed=0, E=1e4, nu=0.3,
                     density=1000.0, h=0.1, tol=1e-3, dhat_rel=1e-3):
    """Config-0 style problem: jittered bar, bent self-intersecting target,
    x_tilde = target (v = (target - x)/h as MeshIO.Load_Velocity_X0)."""
    import sys
    sys.path.insert(0, os.path.dirname(_HERE))
    from idp_gb300 import meshgen

    X, tets = meshgen.bar(nx, ny, nz, size=size, seed=seed)
    target = meshgen.bend_target(X, angle=angle, size=size)
    mass = meshgen.lumped_mass(X, tets, density)
    lam, mu = meshgen.lame(E, nu)
    T = tets.shape[0]
    diag = float(np.linalg.norm(X.max(0) - X.min(0)))
    dHat2 = (dhat_rel * diag) ** 2
    k, kmax = kappa_init(float(mass.mean()), dHat2)
    pb = Problem(X=X, X0=X.copy(), tets=tets, mass=mass, lam=np.full(T, lam), mu=np.full(T, mu), h=h, dHat2=dHat2,
                 kappa=[k, kmax, 0.0], v=(target - X) / h, tol=tol)
    pb.target = target
    return pb
