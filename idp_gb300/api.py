"""Reference-shaped entry points over the C ABI.

``FEM.DiscreteShell.Advance_One_Step_IE_Hinge`` keeps the positional argument
list of the reference's pybind export (``Library/FEM/Shell/DISCRETE_SHELL.h:1110``,
called from ``Python/Drivers/FEMDiscreteShellBase.py:353-361``) and the same
meaning for the arguments this path reads; storages are plain numpy arrays /
dicts instead of JGSL storages. It mutates ``X`` and ``nodeAttr['v']`` in
place and returns the Newton iteration count, like the reference.

With shell elements (``Elem``) it advances an elastic triangle shell
(membrane + hinge bending) instead of a tet mesh.

``FEM.DiscreteShell.Advance_One_Step_IE_Flow`` does the same for the flow-mode
export (``DISCRETE_SHELL.h:1113``) over a triangle-shell instance.

``TetIPCSim`` mirrors the slice of ``FEMDiscreteShellBase`` that sets up a
tet mesh with offset IPC (``add_object_3D``, ``initialize_added_objects``,
``initialize_OIPC``, ``advance_one_time_step``); ``ShellFlowSim`` the slice the
normal-flow scripts drive (``add_shell_3D``, ``initialize``,
``initialize_OIPC``, ``run``).
"""
from __future__ import annotations

import math
import os

import numpy as np

from . import Context, IDPError, IDP_WARN_ITER_CAP, MODE_MIXED, dirichlet, meshgen

_UNSUPPORTED = "not part of the GB300 path (tet meshes and triangle shells with offset IPC and DBC)"


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


def _digest(*arrays):
    """Content key of the arrays that define a context (not their ids: a new
    array can reuse a freed one's address)."""
    import hashlib

    hsh = hashlib.blake2b(digest_size=16)
    for a in arrays:
        a = np.ascontiguousarray(a)
        hsh.update(str((a.dtype.str, a.shape)).encode())
        hsh.update(a.tobytes())
    return hsh.hexdigest()


def _dbc_rows(DBC):
    """Vertex indices and targets of the DBC storage (rows (index, x, y, z),
    the reference's VECTOR_STORAGE<T, dim + 1>, IMPLICIT_EULER.h:155): (None,
    None) without DBC, targets None for a bare index list. A row whose target
    is the vertex's position at a step's start is fixed; the others move there
    (the augmented Lagrangian, IMPLICIT_EULER.h:305-401, 701-757)."""
    if _empty(DBC):
        return None, None
    D = np.asarray(DBC, dtype=np.float64)
    if D.ndim == 1:
        return D.astype(np.int32), None
    idx = D[:, 0].astype(np.int32)
    return idx, (np.ascontiguousarray(D[:, 1:4]) if D.shape[1] >= 4 else None)


def _context_for(tet, X, nodeAttr, tetEl, dHat2, kappaVec, DBC, h, NewtonTol, thickness, mode):
    dbc_idx, _ = _dbc_rows(DBC)
    key = (_digest(tet, nodeAttr["x0"], nodeAttr["m"], tetEl["lambda"], tetEl["mu"],
                   np.zeros(0, np.int32) if dbc_idx is None else dbc_idx),
           X.shape, float(dHat2), float(h), float(NewtonTol), float(thickness), mode,
           tuple(sorted(DiscreteShell.params.items())))
    if _Cache.key == key and _Cache.ctx is not None:
        return _Cache.ctx
    if _Cache.ctx is not None:
        _Cache.ctx.close()
    ctx = Context(h=h, newton_tol=NewtonTol, thickness=thickness, mode=mode, **DiscreteShell.params)
    ctx.add_instance(X, tet, nodeAttr["m"], tetEl["lambda"], tetEl["mu"], dHat2, kappaVec[0], kappaVec[1],
                     X0=nodeAttr["x0"], dbc_idx=dbc_idx)
    ctx.commit()
    _Cache.ctx, _Cache.key = ctx, key
    return ctx


def shell_material(Elem, nodeAttr, elemAttr, elasticityAttr, bendingStiffMult):
    """The elastic-shell material behind the storages Initialize_Discrete_Shell
    fills (FEM/Shell/DISCRETE_SHELL.h:218-357): thickness = vol / area of the
    first face, nu = lambda / (lambda + 2 mu) and E = 2 mu (1 + nu) from
    lambda = E nu / (1 - nu^2), mu = E / (2 (1 + nu)), the bending multiplier
    that gives the hinge stiffness k = bendingStiffMult * elemAttr P[0](0, 0)
    (BENDING.h:54) from E thickness^3 / (24 (1 - nu^2)), and the lumped masses
    (nodeAttr m). Raises ValueError where the faces do not share one material."""
    F = np.asarray(Elem, dtype=np.int32).reshape(-1, 3)
    X0 = np.asarray(nodeAttr["x0"], dtype=np.float64).reshape(-1, 3)
    vol = np.asarray(elasticityAttr["vol"], dtype=np.float64).reshape(-1)
    lam = np.asarray(elasticityAttr["lambda"], dtype=np.float64).reshape(-1)
    mu = np.asarray(elasticityAttr["mu"], dtype=np.float64).reshape(-1)
    if not (vol.size == lam.size == mu.size == F.shape[0]) or F.shape[0] == 0:
        raise ValueError("elasticityAttr: one (vol, lambda, mu) per shell element")
    if np.any(lam != lam[0]) or np.any(mu != mu[0]):
        raise NotImplementedError(f"per-element shell materials: {_UNSUPPORTED}")
    area = np.linalg.norm(np.cross(X0[F[:, 1]] - X0[F[:, 0]], X0[F[:, 2]] - X0[F[:, 0]]), axis=1) / 2
    t = float(vol[0] / area[0])
    if not np.allclose(vol, area * t, rtol=1e-12, atol=0):
        raise NotImplementedError(f"per-element shell thickness: {_UNSUPPORTED}")
    nu = float(lam[0] / (lam[0] + 2 * mu[0]))
    E = float(2 * mu[0] * (1 + nu))
    P = np.asarray(elemAttr["P"], dtype=np.float64)
    k = float(P.reshape(-1)[0]) if P.size else 0.0
    kd = E * t ** 3 / (24.0 * (1.0 - nu * nu))
    m = np.asarray(nodeAttr["m"], dtype=np.float64).reshape(-1)
    return dict(E=E, nu=nu, thickness=t, bending_mult=float(bendingStiffMult) * k / kd,
                density=float(np.sum(m) / np.sum(vol)), mass=m)


def _shell_context_for(Elem, X, nodeAttr, elemAttr, elasticityAttr, bendingStiffMult, dHat2, kappaVec, DBC, h,
                       NewtonTol, thickness, mode):
    dbc_idx, _ = _dbc_rows(DBC)
    P = np.asarray(elemAttr["P"], dtype=np.float64)
    key = ("shell", _digest(np.asarray(Elem, dtype=np.int32), nodeAttr["x0"], nodeAttr["m"], elasticityAttr["vol"],
                            elasticityAttr["lambda"], elasticityAttr["mu"], P.reshape(-1)[:1],
                            np.zeros(0, np.int32) if dbc_idx is None else dbc_idx),
           float(bendingStiffMult), X.shape, float(dHat2), float(h), float(NewtonTol), float(thickness), mode,
           tuple(sorted(DiscreteShell.params.items())))
    if _Cache.key == key and _Cache.ctx is not None:
        return _Cache.ctx
    if _Cache.ctx is not None:
        _Cache.ctx.close()
    mat = shell_material(Elem, nodeAttr, elemAttr, elasticityAttr, bendingStiffMult)
    ctx = Context(h=h, newton_tol=NewtonTol, thickness=thickness, mode=mode, **DiscreteShell.params)
    ctx.add_elastic_shell_instance(X, Elem, mat["density"], mat["E"], mat["nu"], mat["thickness"], dHat2,
                                   kappaVec[0], kappaVec[1], bending_mult=mat["bending_mult"], X0=nodeAttr["x0"],
                                   dbc_idx=dbc_idx, mass=mat["mass"])
    ctx.commit()
    _Cache.ctx, _Cache.key = ctx, key
    return ctx


class DiscreteShell:
    mode = MODE_MIXED
    params: dict = {}  # further idp_params fields for the contexts the calls create

    @staticmethod
    def Advance_One_Step_IE_Hinge(Elem, segs, DBC, edge2tri, edgeStencil, edgeInfo, thickness, bendingStiffMult,
                                  fiberStiffMult, fiberLimit, s, sHat, kappa_s, b, h, NewtonTol, withCollision,
                                  dHat2, kappaVec, mu, epsv2, fricIterAmt, compNodeRange, muComp, staticSolve, X,
                                  nodeAttr, M, elemAttr, elasticityAttr, tet, tetAttr, tetElasticityAttr, rod,
                                  rodInfo, rodHinge, rodHingeInfo, stitchInfo, stitchRatio, k_stitch, particle,
                                  outputFolder):
        """One implicit-Euler step of a tet mesh (tet, tetElasticityAttr) or
        of an elastic triangle shell (Elem with elemAttr, elasticityAttr and
        the rest data of nodeAttr['x0'] that Initialize_Discrete_Shell made;
        the hinge stencils are rebuilt from it on the device, so edgeStencil
        and edgeInfo are not read); X (V,3) and nodeAttr['v'] are updated in
        place, kappaVec[0] receives the adapted kappa. Returns Newton iterations."""
        for name, v in (("segs", segs), ("rod", rod), ("stitchInfo", stitchInfo), ("particle", particle)):
            if not _empty(v):
                raise NotImplementedError(f"{name}: {_UNSUPPORTED}")
        if mu and mu > 0:
            raise NotImplementedError(f"friction: {_UNSUPPORTED}")
        if staticSolve:
            raise NotImplementedError(f"staticSolve: {_UNSUPPORTED}")
        if not withCollision:
            raise NotImplementedError("withCollision=False: the GB300 path always has IPC contact")
        if not _empty(Elem) and not _empty(tet):
            raise NotImplementedError(f"shells and tets in one call: {_UNSUPPORTED}")
        if not _empty(Elem):
            if _empty(elemAttr) or _empty(elasticityAttr):
                raise ValueError("shell elements need elemAttr and elasticityAttr (Initialize_Discrete_Shell)")
            ctx = _shell_context_for(Elem, X, nodeAttr, elemAttr, elasticityAttr, bendingStiffMult, dHat2, kappaVec,
                                     DBC, h, NewtonTol, thickness, DiscreteShell.mode)
        else:
            ctx = _context_for(np.asarray(tet), X, nodeAttr, tetElasticityAttr, dHat2, kappaVec, DBC, h, NewtonTol,
                               thickness, DiscreteShell.mode)
        # per call, as the reference reads them: positions, velocity, the
        # kappa pair (a driver may reset it, e.g. initialize_OIPC) and the
        # body force of the predictor (IMPLICIT_EULER.h:195-216)
        ctx.set_positions(0, X)
        ctx.set_velocity(0, nodeAttr["v"])
        ctx.set_kappa(0, [kappaVec[0], kappaVec[1], 0.0])
        idx, targets = _dbc_rows(DBC)
        if idx is not None:
            ctx.set_dbc_targets(0, targets)
        bb = None if b is None else np.asarray(b, dtype=np.float64).reshape(-1, 3)
        ctx.set_body_force(0, bb if bb is not None and np.any(bb != 0) else None)
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
    dbc_idx, _ = _dbc_rows(DBC)
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
    idx, targets = _dbc_rows(DBC)
    if idx is not None:
        ctx.set_dbc_targets(0, targets)
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


class _DirichletDriver:
    """The Dirichlet part of FEMDiscreteShellBase: DBC rows and motions
    (set_DBC, set_DBC_with_range, load_frame's Reset_Dirichlet) and their
    update before each step (FEMDiscreteShellBase.py:273-299): the motion
    runs while MDBC_tmin < t < MDBC_tmax, its velocities reversing every
    MDBC_period; with seqDBC >= 0 the targets are read from the OBJ sequence
    seqDBCPath/shell<frame>.obj instead, translated by (0, -0.75, 0)."""

    def _init_dbc(self):
        self.DBC = dirichlet.DBCStorage()
        self.DBCMotion = dirichlet.DBCMotion()
        self.t = 0.0
        self.MDBC_tmax = 1e10
        self.MDBC_tmin = -1.0
        self.MDBC_period = 1e10
        self.MDBC_periodCounter = 1
        self.seqDBC = -1
        self.seqDBCPath = ""
        self.curFrameNum = 0
        # rows removed from the back of the motion list over time
        self.DBCPopBackCounter = 0
        self.DBCPopBackFrameCounter = 0
        self.DBCPopBackAmt = 0
        self.DBCPopBackTStart = 0.0
        self.DBCPopBackTEnd = -1.0
        self.DBCPopBackStep = 1
        self.DBCPopBackBatch = 1
        # a second motion list over the same rows, with its own time window
        self.DBCMotion2 = dirichlet.DBCMotion()
        self.MDBC_tmax2 = -1.0
        self.MDBC_tmin2 = 0.0
        self.MDBC_period2 = 1e10
        self.MDBC_periodCounter2 = 1

    def set_DBC(self, DBCRangeMin, DBCRangeMax, v, rotCenter, rotAxis, angVelDeg):
        dirichlet.init_dirichlet(self.X, DBCRangeMin, DBCRangeMax, v, rotCenter, rotAxis, angVelDeg, self.DBC,
                                 self.DBCMotion)

    def set_DBC_with_range(self, DBCRangeMin, DBCRangeMax, v, rotCenter, rotAxis, angVelDeg, vIndRange):
        dirichlet.init_dirichlet(self.X, DBCRangeMin, DBCRangeMax, v, rotCenter, rotAxis, angVelDeg, self.DBC,
                                 self.DBCMotion, vIndRange)

    def set_DBC2_with_range(self, DBCRangeMin, DBCRangeMax, v, rotCenter, rotAxis, angVelDeg, vIndRange):
        dirichlet.init_dirichlet(self.X, DBCRangeMin, DBCRangeMax, v, rotCenter, rotAxis, angVelDeg, self.DBC,
                                 self.DBCMotion2, vIndRange)

    def load_frame(self, filePath):
        """Positions from an OBJ file, DBC targets reset to them
        (FEMDiscreteShellBase.py:244-250)."""
        from . import meshio

        X, _, _ = meshio.read_tri_obj(filePath)
        if X.shape != self.X.shape:
            raise ValueError(f"{filePath}: node count does not match")
        self.X = X
        dirichlet.reset_dirichlet(self.X, self.DBC)

    def load_velocity(self, folderPath, lastFrame, h):
        """Velocity (frame lastFrame - frame lastFrame-1) / h of an OBJ
        sequence (Load_Velocity, Library/Utils/MESHIO.h:967-984), applied
        at the next step."""
        from . import meshio

        X0, _, _ = meshio.read_tri_obj(f"{folderPath}/{lastFrame - 1}.obj")
        X1, _, _ = meshio.read_tri_obj(f"{folderPath}/{lastFrame}.obj")
        if X0.shape != self.X.shape or X1.shape != self.X.shape:
            raise ValueError(f"{folderPath}: node count does not match")
        self._set_velocity((X1 - X0) / h)

    def _step_dbc(self, dt):
        """The DBC updates before a step (FEMDiscreteShellBase.py:275-299):
        the first motion list (or the OBJ sequence), pop-backs, the second
        motion list."""
        if self.MDBC_tmin < self.t < self.MDBC_tmax:
            if self.seqDBC < 0:
                if self.t - self.MDBC_tmin >= self.MDBC_period * self.MDBC_periodCounter:
                    self.MDBC_periodCounter += 1
                    dirichlet.turn_dirichlet(self.DBCMotion)
                dirichlet.step_dirichlet(self.DBCMotion, dt, self.DBC)
            else:
                dirichlet.load_dirichlet(f"{self.seqDBCPath}/shell{self.curFrameNum}.obj", self.seqDBC,
                                         (0.0, -0.75, 0.0), self.DBC)
                self.curFrameNum += 1
        if (self.DBCPopBackCounter < self.DBCPopBackAmt and self.DBCPopBackTStart < self.t < self.DBCPopBackTEnd):
            if self.DBCPopBackFrameCounter % self.DBCPopBackBatch == 0:
                for _ in range(self.DBCPopBackStep):
                    dirichlet.pop_back_dirichlet(self.DBCMotion, self.DBC)
                self.DBCPopBackCounter += 1
            self.DBCPopBackFrameCounter += 1
        if self.MDBC_tmin2 < self.t < self.MDBC_tmax2:
            if self.t - self.MDBC_tmin2 >= self.MDBC_period2 * self.MDBC_periodCounter2:
                self.MDBC_periodCounter2 += 1
                dirichlet.turn_dirichlet(self.DBCMotion2)
            dirichlet.step_dirichlet(self.DBCMotion2, dt, self.DBC)

    def _dbc_arg(self):
        return self.DBC if len(self.DBC) else None


class TetIPCSim(_DirichletDriver):
    """The tet + offset-IPC slice of FEMDiscreteShellBase
    (Python/Drivers/FEMDiscreteShellBase.py:14-388), with its Dirichlet
    conditions (fixed, moving by a velocity and an angular velocity)."""

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
        self.PNIterCount = 0
        self.mode = mode
        self.gravity = (0.0, -9.81, 0.0)
        self.bodyForce = None
        self._init_dbc()

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
        """Masses, velocity, Lame parameters and the gravity body force of the
        added tets (FEMDiscreteShellBase.py:214-221)."""
        m = meshgen.lumped_mass(self.X, self.tet, p_density)
        lam, mu = meshgen.lame(E, nu)
        T = self.tet.shape[0]
        self.nodeAttr = dict(x0=self.X.copy(), v=np.tile(np.asarray(velocity, float), (self.X.shape[0], 1)), m=m)
        self.tetElasticity = {"lambda": np.full(T, lam), "mu": np.full(T, mu)}
        self.bodyForce = meshgen.tet_body_force(self.X, self.tet, p_density, self.gravity)

    def adjust_material(self, meshCounter, densityMult, YoungsMult):
        """Adjust_Material (FEM/Shell/DISCRETE_SHELL.h:532-553): masses and
        body force of the mesh's vertices scaled by densityMult, its tets'
        Lame parameters by YoungsMult."""
        v0, t0, v1, t1 = (int(c) for c in meshCounter)
        self.nodeAttr["m"][v0:v1] *= densityMult
        if self.bodyForce is not None:
            self.bodyForce[v0:v1] *= densityMult
        self.tetElasticity["lambda"][t0:t1] *= YoungsMult
        self.tetElasticity["mu"][t0:t1] *= YoungsMult

    def magnify_body_force(self, DBCRangeMin, DBCRangeMax, magnifyFactor):
        dirichlet.magnify_body_force(self.X, DBCRangeMin, DBCRangeMax, magnifyFactor, self.bodyForce)

    def _set_velocity(self, v):
        self.nodeAttr["v"][:] = v

    def initialize_OIPC(self, dhat, offset, stiffMult=1.0):
        self.dHat2 = dhat * dhat
        k, km = initialize_oipc(float(self.nodeAttr["m"].mean()), self.dHat2, stiffMult)
        self.kappa = [k, km, 0.0]
        self.thickness = offset

    def advance_one_time_step(self, dt=None):
        h = dt or self.dt
        self._step_dbc(h)
        mode, DiscreteShell.mode = DiscreteShell.mode, self.mode  # this driver's precision for its own call only
        try:
            it = FEM.DiscreteShell.Advance_One_Step_IE_Hinge(
                None, None, self._dbc_arg(), None, None, None, self.thickness, 0, None, None, None, None, None,
                self.bodyForce, h, self.PNTol, True, self.dHat2, self.kappa, 0, 1e-6, 1, None, None, False, self.X,
                self.nodeAttr, None, None, None, self.tet, None, self.tetElasticity, None, None, None, None, None,
                None, 10, None, "")
        finally:
            DiscreteShell.mode = mode
        self.PNIterCount += it
        self.t += h
        return it


class ShellFlowSim(_DirichletDriver):
    """The triangle-shell slice of FEMDiscreteShellBase: what the normal-flow
    scripts drive (Projects/FEMShell/12-14_normal_flow.py) — add_shell_3D,
    initialize, initialize_OIPC, the frame loop of SimulationBase
    (Python/Drivers/SimulationBase.py:76-103) and advance_one_time_step with
    Update_Normal_Flow_Neumann (FEMDiscreteShellBase.py:266-276, 332-340) —
    and, with flow off, the elastic shell's Hinge step with gravity and
    Dirichlet conditions (FEMDiscreteShellBase.py:255-361), including the
    character sequences of Projects/FEMShell/16_fix_char_seq.py
    (add_shell_with_scale_3D, lv_fn, seqDBCPath, write)."""

    def __init__(self, precision="double", dim=3, mode=MODE_MIXED):
        if dim != 3:
            raise NotImplementedError("2D shells are not part of this path")
        self.X = np.zeros((0, 3))
        self.Elem = np.zeros((0, 3), np.int32)
        self.dt = 0.04
        self.frame_dt = 0.04
        self.frame_num = 1
        self.PNTol = 1e-3
        self.flow = False
        self.normalFlowMag = 0.0
        self.withCollision = True
        self.gravity = (0.0, -9.81, 0.0)
        self.bodyForce = None  # set by initialize: lumped mass x gravity
        self._bf_dirty = False
        self._v_next = None
        self.bendingStiffMult = 1.0
        self.shell_density = 1000.0
        self.shell_E = 1e5
        self.shell_nu = 0.4
        self.shell_thickness = 0.001
        self.dHat2 = 1e-6
        self.kappa = [1e5, 0.0, 0.0]
        self.thickness = 0.0  # IPC offset
        self.PNIterCount = 0
        self.mode = mode
        self._ctx = None
        self._ctx_h = None
        self._X0 = None
        self.lv_fn = -1
        self.output_folder = ""
        self._init_dbc()

    def add_shell_3D(self, filePath, translate, rotCenter, rotAxis, rotDeg):
        from . import meshio

        self.X, self.Elem, counter = meshio.read_tri_obj(filePath, self.X, self.Elem)
        meshio.transform_points(self.X, translate, rotCenter, rotAxis, rotDeg, (1.0, 1.0, 1.0), counter)
        return counter

    def add_shell_with_scale_3D(self, filePath, translate, scale, rotCenter, rotAxis, rotDeg):
        from . import meshio

        self.X, self.Elem, counter = meshio.read_tri_obj(filePath, self.X, self.Elem)
        meshio.transform_points(self.X, translate, rotCenter, rotAxis, rotDeg, scale, counter)
        return counter

    def write(self, frame_idx):
        """The current shell as <output_folder>/shell<frame>.obj."""
        from . import meshio

        if self.output_folder:
            os.makedirs(self.output_folder, exist_ok=True)
            meshio.write_tri_obj(os.path.join(self.output_folder, f"shell{frame_idx}.obj"), self.X, self.Elem)

    def _mass(self, X=None):
        X, F = (self.X if X is None else X), self.Elem
        area = np.linalg.norm(np.cross(X[F[:, 1]] - X[F[:, 0]], X[F[:, 2]] - X[F[:, 0]]), axis=1) / 2
        m = np.zeros(X.shape[0])
        np.add.at(m, F.reshape(-1), np.repeat(area * self.shell_thickness * self.shell_density / 3, 3))
        return m

    def initialize(self, p_density, E, nu, thickness, caseI):
        """Shell material (Initialize_Shell_Hinge_EIPC's density, E, nu and
        thickness; E and nu do not enter the flow energy), gravity off when
        caseI is nonzero, the body force lumped mass x gravity
        (FEMDiscreteShellBase.py:190-203); in flow mode the open boundary's
        vertices are fixed (FEM.Boundary_Dirichlet)."""
        self.shell_density, self.shell_thickness = float(p_density), float(thickness)
        self.shell_E, self.shell_nu = float(E), float(nu)
        self.thickness = float(thickness)
        if caseI != 0:
            self.gravity = (0.0, 0.0, 0.0)
        self.bodyForce = self._gravity_force(self.X)
        if self.flow:
            dirichlet.boundary_dirichlet(self.X, self.Elem, self.DBC)

    def _gravity_force(self, X):
        return self._mass(X)[:, None] * np.asarray(self.gravity, float)[None, :]

    def add_mannequin(self, filePath, translate, scale, rotCenter, rotAxis, rotDeg):
        """A shell whose every vertex is a fixed DBC row
        (FEMDiscreteShellBase.py:152-157: moved 1e6 along x so that the box
        x >= 0.5 of the bounding box holds exactly its vertices, set_DBC,
        moved back, targets reset to the positions)."""
        from . import meshio

        counter = self.add_shell_with_scale_3D(filePath, translate, scale, rotCenter, rotAxis, rotDeg)
        meshio.transform_points(self.X, (1e6, 0, 0), (0, 0, 0), (1, 0, 0), 0, (1, 1, 1), counter)
        self.set_DBC((0.5, -1, -1), (1.1, 1.1, 1.1), (0, 0, 0), (0, 0, 0), (1, 0, 0), 0)
        meshio.transform_points(self.X, (-1e6, 0, 0), (0, 0, 0), (1, 0, 0), 0, (1, 1, 1), counter)
        dirichlet.reset_dirichlet(self.X, self.DBC)
        return counter

    def magnify_body_force(self, DBCRangeMin, DBCRangeMax, magnifyFactor):
        if self.bodyForce is None:
            self.bodyForce = self._gravity_force(self.X if self._X0 is None else self._X0)
        dirichlet.magnify_body_force(self.X, DBCRangeMin, DBCRangeMax, magnifyFactor, self.bodyForce)
        self._bf_dirty = True

    def _set_velocity(self, v):
        self._v_next = np.array(v, dtype=np.float64).reshape(-1, 3)

    def initialize_OIPC(self, thickness, offset, stiffMult=1.0):
        """Initialize_OIPC (DISCRETE_SHELL.h:555-577): d-hat = thickness,
        kappa from the mean lumped mass (of the rest shape in use)."""
        self.dHat2 = float(thickness) ** 2
        k, km = initialize_oipc(float(self._mass(self._X0).mean()), self.dHat2, stiffMult)
        self.kappa = [k, km, 0.0]
        self.thickness = float(offset)

    def _next_frame_rest_shape(self, dt):
        """The lv_fn sequence (FEMDiscreteShellBase.py:297-310): frame lv_fn of
        seqDBCPath becomes the rest shape (masses and kappa follow), the
        velocity points at it (Load_Velocity_X0, Library/Utils/MESHIO.h:987-1004)
        and the DBC rows take their targets from it (Load_Dirichlet)."""
        from . import meshio

        path = f"{self.seqDBCPath}/{self.lv_fn}.obj"
        newX, _, _ = meshio.read_tri_obj(path)
        if newX.shape != self.X.shape:
            raise ValueError(f"{path}: node count does not match")
        self._X0 = newX
        self.bodyForce = self._gravity_force(newX)
        self.initialize_OIPC(math.sqrt(self.dHat2), self.thickness)  # default stiffMult, as the reference does
        dirichlet.targets_from_points(newX, 0, (0.0, 0.0, 0.0), self.DBC)  # Load_Dirichlet of the same file
        self.lv_fn += 1
        if self._ctx is not None:
            self._ctx.close()
            self._ctx = None
        return (newX - self.X) / dt

    @property
    def context(self):
        """The device context of the last step (None before the first): its
        stats(), state() and intersection_counts()."""
        return self._ctx

    def _context(self, h):
        if self._ctx is not None and self._dbc_n != len(self.DBC):  # the DBC rows changed: rebuild
            self._ctx_h = None
        if self._ctx is None or self._ctx_h != h:
            X = self.X.copy()
            v = None
            if self._ctx is not None:  # a new step size keeps the elastic shell's rest shape and velocity
                v = self._ctx.state(0)[1]
                self._ctx.close()
            elif self._X0 is None:
                self._X0 = X.copy()
            self._ctx = Context(h=h, newton_tol=self.PNTol, thickness=self.thickness, mode=self.mode)
            dbc_idx = self.DBC.indices if len(self.DBC) else None
            self._dbc_n = len(self.DBC)
            if self.flow:
                self._ctx.add_shell_instance(X, self.Elem, self.shell_density, self.shell_thickness, self.dHat2,
                                             self.kappa[0], self.kappa[1], dbc_idx=dbc_idx)
            else:
                self._ctx.add_elastic_shell_instance(X, self.Elem, self.shell_density, self.shell_E, self.shell_nu,
                                                     self.shell_thickness, self.dHat2, self.kappa[0], self.kappa[1],
                                                     bending_mult=self.bendingStiffMult, X0=self._X0,
                                                     dbc_idx=dbc_idx)
                if v is not None:
                    self._ctx.set_velocity(0, v)
                b = self._gravity_force(self._X0) if self.bodyForce is None else self.bodyForce
                if np.any(b != 0):  # b = M g (Initialize_Discrete_Shell)
                    self._ctx.set_body_force(0, b)
                self._bf_dirty = False
            self._ctx.commit()
            self._ctx_h = h
        return self._ctx

    def advance_one_time_step(self, dt):
        """Advance_One_Step_IE_Flow with the normal-flow predictor in flow
        mode, Advance_One_Step_IE_Hinge of the elastic shell otherwise; the
        Dirichlet motion is stepped first; with lv_fn >= 0 the next frame of
        the sequence sets the rest shape, the velocity and the DBC targets."""
        self._step_dbc(dt)
        v_seq = None
        if self.lv_fn >= 0:
            if self.flow:
                raise ValueError("lv_fn frame sequences drive the elastic shell; set flow = False")
            v_seq = self._next_frame_rest_shape(dt)
        ctx = self._context(dt)
        if self._v_next is not None:  # load_velocity
            ctx.set_velocity(0, self._v_next)
            self._v_next = None
        if self._bf_dirty and not self.flow:  # magnify_body_force after the context was built
            ctx.set_body_force(0, self.bodyForce)
            self._bf_dirty = False
        if v_seq is not None:
            ctx.set_velocity(0, v_seq)
        ctx.set_positions(0, self.X)
        ctx.set_kappa(0, self.kappa)
        if len(self.DBC):
            ctx.set_dbc_targets(0, self.DBC.targets)
        if self.flow and self.normalFlowMag != 0:
            ctx.set_normal_flow(0, dt * dt * self.normalFlowMag)
        rc, res = ctx.advance(check=False)
        if rc not in (0, IDP_WARN_ITER_CAP):
            raise IDPError(rc, "advance_one_time_step")
        X, _, k = ctx.state(0)
        self.X[...] = X
        self.kappa[0] = k[0]
        self.PNIterCount += res[0]["newton_iters"]
        self.t += dt
        return res[0]["newton_iters"]

    def advance_one_frame(self, f):
        remain = self.frame_dt
        while remain > 0:
            cur = self.dt if remain > 2 * self.dt else (remain / 2 if remain > self.dt else remain)
            self.advance_one_time_step(cur)
            remain -= cur

    def run(self):
        for f in range(self.frame_num):
            self.advance_one_frame(f + 1)
            self.write(f + 1)
