"""Reference-shaped entry points over the C ABI.

``FEM.DiscreteShell.Advance_One_Step_IE_Hinge`` keeps the positional argument
list of the reference's pybind export (``Library/FEM/Shell/DISCRETE_SHELL.h:1110``,
called from ``Python/Drivers/FEMDiscreteShellBase.py:353-361``) and the same
meaning for the arguments this path reads; storages are plain numpy arrays /
dicts instead of JGSL storages. It mutates ``X`` and ``nodeAttr['v']`` in
place and returns the Newton iteration count, like the reference.

``TetIPCSim`` mirrors the slice of ``FEMDiscreteShellBase`` that sets up a
tet mesh with offset IPC (``add_object_3D``, ``initialize_added_objects``,
``initialize_OIPC``, ``advance_one_time_step``).
"""
from __future__ import annotations

import math

import numpy as np

from . import Context, IDPError, IDP_WARN_ITER_CAP, MODE_MIXED, meshgen

_UNSUPPORTED = "not part of the GB300 path (tet meshes with offset IPC only)"


def _empty(x):
    if x is None:
        return True
    try:
        return len(x) == 0
    except TypeError:
        return not x


def barrier_hessian_at(d, dHat2, kappa=1.0):
    """b''(d) of the log barrier (Math/BARRIER.h:44-54)."""
    t2 = d - dHat2
    return kappa * ((math.log(d / dHat2) * -2.0 - t2 * 4.0 / d) + 1.0 / (d * d) * (t2 * t2))


def initialize_oipc(mass_diag_mean, dHat2, stiff_mult=1.0):
    """kappa and kappa_max as Initialize_EIPC<T,false> via Initialize_OIPC
    (FEM/Shell/DISCRETE_SHELL.h:555-577)."""
    H_b = barrier_hessian_at(1.0e-16, dHat2, 1.0)
    k = stiff_mult * 1.0e11 * mass_diag_mean * 3 / (4.0e-16 * H_b)
    return k, 100 * k


class _Cache:
    ctx = None
    key = None


def _context_for(tet, X, nodeAttr, tetEl, dHat2, kappaVec, DBC, h, NewtonTol, thickness, mode):
    key = (id(tet), tet.shape, X.shape, float(dHat2), float(h), float(NewtonTol), float(thickness), mode)
    if _Cache.key == key and _Cache.ctx is not None:
        return _Cache.ctx
    ctx = Context(h=h, newton_tol=NewtonTol, thickness=thickness, mode=mode)
    dbc_idx = None if _empty(DBC) else np.asarray(DBC)[:, 0].astype(np.int32)
    ctx.add_instance(X, tet, nodeAttr["m"], tetEl["lambda"], tetEl["mu"], dHat2, kappaVec[0], kappaVec[1],
                     X0=nodeAttr["x0"], dbc_idx=dbc_idx)
    ctx.commit()
    _Cache.ctx, _Cache.key = ctx, key
    return ctx


class DiscreteShell:
    mode = MODE_MIXED

    @staticmethod
    def Advance_One_Step_IE_Hinge(Elem, segs, DBC, edge2tri, edgeStencil, edgeInfo, thickness, bendingStiffMult,
                                  fiberStiffMult, fiberLimit, s, sHat, kappa_s, b, h, NewtonTol, withCollision,
                                  dHat2, kappaVec, mu, epsv2, fricIterAmt, compNodeRange, muComp, staticSolve, X,
                                  nodeAttr, M, elemAttr, elasticityAttr, tet, tetAttr, tetElasticityAttr, rod,
                                  rodInfo, rodHinge, rodHingeInfo, stitchInfo, stitchRatio, k_stitch, particle,
                                  outputFolder):
        """One implicit-Euler step; X (V,3) and nodeAttr['v'] are updated in
        place, kappaVec[0] receives the adapted kappa. Returns Newton iterations."""
        for name, v in (("Elem", Elem), ("segs", segs), ("rod", rod), ("stitchInfo", stitchInfo),
                        ("particle", particle)):
            if not _empty(v):
                raise NotImplementedError(f"{name}: {_UNSUPPORTED}")
        if mu and mu > 0:
            raise NotImplementedError(f"friction: {_UNSUPPORTED}")
        if staticSolve:
            raise NotImplementedError(f"staticSolve: {_UNSUPPORTED}")
        if not withCollision:
            raise NotImplementedError("withCollision=False: the GB300 path always has IPC contact")
        if b is not None and np.any(np.asarray(b) != 0):
            raise NotImplementedError(f"body force: {_UNSUPPORTED}")
        tet = np.asarray(tet)
        ctx = _context_for(tet, X, nodeAttr, tetElasticityAttr, dHat2, kappaVec, DBC, h, NewtonTol, thickness,
                           DiscreteShell.mode)
        ctx.set_positions(0, X)
        ctx.set_velocity(0, nodeAttr["v"])
        rc, res = ctx.advance(check=False)
        if rc not in (0, IDP_WARN_ITER_CAP):
            raise IDPError(rc, "Advance_One_Step_IE_Hinge")
        Xn, v, k = ctx.state(0)
        X[...] = Xn
        nodeAttr["v"][...] = v
        kappaVec[0] = k[0]
        return res[0]["newton_iters"]


class _FlowCache:
    ctx = None
    key = None


def _flow_context_for(Elem, X, nodeAttr, elasticityAttr, dHat2, kappaVec, DBC, h, NewtonTol, thickness, mode):
    Elem = np.asarray(Elem, dtype=np.int32).reshape(-1, 3)
    key = (id(Elem), Elem.shape, X.shape, float(dHat2), float(h), float(NewtonTol), float(thickness), mode)
    if _FlowCache.key == key and _FlowCache.ctx is not None:
        return _FlowCache.ctx
    # shell thickness and density back from the element volumes (area *
    # thickness) and lumped masses of Initialize_Discrete_Shell
    X0 = np.asarray(nodeAttr["x0"], dtype=np.float64).reshape(-1, 3)
    area = np.linalg.norm(np.cross(X0[Elem[:, 1]] - X0[Elem[:, 0]], X0[Elem[:, 2]] - X0[Elem[:, 0]]), axis=1) / 2
    vol = np.asarray(elasticityAttr["vol"], dtype=np.float64)
    shell_t = float(vol[0] / area[0])
    rho = float(np.sum(nodeAttr["m"]) / np.sum(vol))
    ctx = Context(h=h, newton_tol=NewtonTol, thickness=thickness, mode=mode)
    dbc_idx = None if _empty(DBC) else np.asarray(DBC)[:, 0].astype(np.int32)
    ctx.add_shell_instance(X0, Elem, rho, shell_t, dHat2, kappaVec[0], kappaVec[1], dbc_idx=dbc_idx)
    ctx.commit()
    _FlowCache.ctx, _FlowCache.key = ctx, key
    return ctx


def _advance_flow(Elem, segs, DBC, edge2tri, edgeStencil, edgeInfo, thickness, bendingStiffMult, fiberStiffMult,
                  fiberLimit, s, sHat, kappa_s, b, h, NewtonTol, withCollision, dHat2, kappaVec, mu, epsv2,
                  fricIterAmt, compNodeRange, muComp, staticSolve, X, nodeAttr, M, elemAttr, elasticityAttr, tet,
                  tetAttr, tetElasticityAttr, rod, rodInfo, rodHinge, rodHingeInfo, stitchInfo, stitchRatio, k_stitch,
                  particle, outputFolder):
    """Advance_One_Step_IE_Flow (DISCRETE_SHELL.h:1113): one flow-mode step of
    a triangle shell. b is the body force of Update_Normal_Flow_Neumann
    (magnitude * M_ii * normal), so x_tilde = x + h^2 M^-1 b with v = 0."""
    for name, v in (("segs", segs), ("rod", rod), ("stitchInfo", stitchInfo), ("particle", particle), ("tet", tet)):
        if not _empty(v):
            raise NotImplementedError(f"{name}: not part of the flow-mode shell path")
    if staticSolve or (mu and mu > 0):
        raise NotImplementedError("staticSolve / friction: not part of the flow-mode shell path")
    if not withCollision:
        raise NotImplementedError("withCollision=False: the GB300 path always has IPC contact")
    ctx = _flow_context_for(Elem, X, nodeAttr, elasticityAttr, dHat2, kappaVec, DBC, h, NewtonTol, thickness,
                            DiscreteShell.mode)
    ctx.set_positions(0, X)
    m = np.asarray(nodeAttr["m"], dtype=np.float64)
    bb = np.zeros_like(X) if b is None else np.asarray(b, dtype=np.float64).reshape(-1, 3)
    ctx.set_velocity(0, h * bb / m[:, None])
    rc, res = ctx.advance(check=False)
    if rc not in (0, IDP_WARN_ITER_CAP):
        raise IDPError(rc, "Advance_One_Step_IE_Flow")
    Xn, v, k = ctx.state(0)
    X[...] = Xn
    nodeAttr["v"][...] = v
    kappaVec[0] = k[0]
    return res[0]["newton_iters"]


DiscreteShell.Advance_One_Step_IE_Flow = staticmethod(_advance_flow)


class FEM:
    DiscreteShell = DiscreteShell


class TetIPCSim:
    """The tet + offset-IPC slice of FEMDiscreteShellBase
    (Python/Drivers/FEMDiscreteShellBase.py:14-388)."""

    def __init__(self, dt=0.1, PNTol=1e-3, mode=MODE_MIXED):
        self.dt = dt
        self.PNTol = PNTol
        self.X = np.zeros((0, 3))
        self.tet = np.zeros((0, 4), np.int32)
        self.nodeAttr = {}
        self.tetElasticity = {}
        self.dHat2 = 1e-6
        self.kappa = [1e5, 0.0, 0.0]
        self.thickness = 0.0
        self.DBC = None
        self.PNIterCount = 0
        self.mode = mode

    def add_object_3D(self, X, *args):
        """Append a tet mesh and return its mesh counter. Either
        add_object_3D(filePath, translate, rotCenter, rotAxis, rotDeg, scale)
        as the reference's driver (FEMDiscreteShellBase.py:184-188: a legacy
        VTK file whose points are then transformed), or
        add_object_3D(X, tets[, translate, rotCenter, rotAxis, rotDeg, scale])
        with arrays."""
        from . import meshio

        if isinstance(X, (str, bytes)) or hasattr(X, "__fspath__"):
            self.X, self.tet, counter = meshio.read_tet_vtk(X, self.X, self.tet)
            xf = args
        else:
            tets = np.asarray(args[0], np.int32)
            off, toff = self.X.shape[0], self.tet.shape[0]
            self.X = np.concatenate([self.X, np.asarray(X, float)])
            self.tet = np.concatenate([self.tet, tets + off]).astype(np.int32)
            counter = (off, toff, self.X.shape[0], self.tet.shape[0])
            xf = args[1:]
        if xf:
            translate, rotCenter, rotAxis, rotDeg, scale = xf
            meshio.transform_points(self.X, translate, rotCenter, rotAxis, rotDeg, scale, counter)
        return counter

    def initialize_added_objects(self, velocity, p_density, E, nu):
        m = meshgen.lumped_mass(self.X, self.tet, p_density)
        lam, mu = meshgen.lame(E, nu)
        T = self.tet.shape[0]
        self.nodeAttr = dict(x0=self.X.copy(), v=np.tile(np.asarray(velocity, float), (self.X.shape[0], 1)), m=m)
        self.tetElasticity = {"lambda": np.full(T, lam), "mu": np.full(T, mu)}

    def initialize_OIPC(self, dhat, offset, stiffMult=1.0):
        self.dHat2 = dhat * dhat
        k, km = initialize_oipc(float(self.nodeAttr["m"].mean()), self.dHat2, stiffMult)
        self.kappa = [k, km, 0.0]
        self.thickness = offset

    def advance_one_time_step(self, dt=None):
        DiscreteShell.mode = self.mode
        it = FEM.DiscreteShell.Advance_One_Step_IE_Hinge(
            None, None, self.DBC, None, None, None, self.thickness, 0, None, None, None, None, None, None,
            dt or self.dt, self.PNTol, True, self.dHat2, self.kappa, 0, 1e-6, 1, None, None, False, self.X,
            self.nodeAttr, None, None, None, self.tet, None, self.tetElasticity, None, None, None, None, None, None,
            10, None, "")
        self.PNIterCount += it
        return it
