"""GB300 implementation of IDP's injective-deformation Newton step.

The compute path is the C-ABI library ``libidp_gb300.so`` (hand-written
sm_103a CUDA kernels + C++ host driver, declared in ``include/idp_gb300.h``).
This package only binds it (ctypes) and mirrors the reference's Python-facing
interface. There is no CPU fallback: importing the bindings without the
library raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libidp_gb300.so")

IDP_OK = 0
IDP_ERR_INVALID_ARG = 1
IDP_ERR_CUDA = 2
IDP_ERR_CAPACITY = 3
IDP_ERR_INVERTED = 4
IDP_ERR_NOT_CONVERGED = 5
IDP_ERR_ZERO_STEP = 6
IDP_ERR_NONPOSITIVE_DIST = 7
IDP_ERR_STATE = 8
IDP_WARN_ITER_CAP = 9
IDP_ERR_INTERSECTION = 10
MODE_FP64 = 0
MODE_MIXED = 1

# every entry point include/idp_gb300.h declares
EXPORTS = [
    "idp_default_params", "idp_create", "idp_destroy", "idp_status_str", "idp_add_instance", "idp_set_velocity",
    "idp_set_positions", "idp_commit", "idp_advance", "idp_get_state", "idp_instance_info", "idp_get_surface",
    "idp_eval_energy", "idp_eval_gradient", "idp_constraint_set", "idp_ccd_stepsize", "idp_hessian_apply",
    "idp_newton_direction", "idp_get_stats", "idp_save_state", "idp_restore_state",
    "idp_set_normal_flow", "idp_set_kappa", "idp_tet_energy_noalloc", "idp_check_intersection",
    "idp_check_intersection_all", "idp_reset", "idp_device_bytes", "idp_job_footprint", "idp_server_create",
    "idp_server_create_simulated", "idp_server_submit", "idp_server_wait", "idp_server_drain",
    "idp_server_get_stats", "idp_server_destroy", "idp_add_shell_instance", "idp_step_begin", "idp_step_iterate",
    "idp_set_body_force", "idp_add_elastic_shell_instance", "idp_set_dbc_targets",
]


class Params(C.Structure):
    _fields_ = [("h", C.c_double), ("newton_tol", C.c_double), ("max_newton", C.c_int), ("mode", C.c_int),
                ("pcg_rel_tol", C.c_double), ("pcg_max_iters", C.c_int), ("thickness", C.c_double),
                ("device", C.c_int), ("pcg_grid_min_vertices", C.c_int), ("pcg_grid_cta_vertices", C.c_int),
                ("contact_block_vertices", C.c_int), ("verify_iterates", C.c_int),
                ("caller_vertex_order", C.c_int), ("pcg_local_degree", C.c_int),
                ("surface_device_min_tets", C.c_int)]


class Result(C.Structure):
    _fields_ = [("status", C.c_int), ("newton_iters", C.c_int), ("pcg_iters", C.c_int), ("ls_trials", C.c_int),
                ("num_constraints", C.c_int), ("energy", C.c_double), ("kappa", C.c_double),
                ("residual", C.c_double), ("min_alpha", C.c_double), ("latency_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Stats(C.Structure):
    _fields_ = [("pcg_ms", C.c_double), ("pcg_bytes", C.c_double), ("pcg_iters", C.c_longlong),
                ("pcg_launches", C.c_int), ("tet_ms", C.c_double), ("contact_ms", C.c_double), ("ccd_ms", C.c_double),
                ("total_ms", C.c_double), ("kernel_launches", C.c_longlong), ("barrier_ms", C.c_double),
                ("assembly_ms", C.c_double), ("fp64_fallbacks", C.c_int), ("verify_checks", C.c_longlong),
                ("verify_failures", C.c_longlong)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class JobDesc(C.Structure):
    _fields_ = [("V", C.c_int), ("X", C.c_void_p), ("X0", C.c_void_p), ("T", C.c_int), ("tets", C.c_void_p),
                ("mass", C.c_void_p), ("lam", C.c_void_p), ("mu", C.c_void_p), ("nDBC", C.c_int),
                ("dbc_idx", C.c_void_p), ("dHat2", C.c_double), ("kappa", C.c_double), ("kappa_max", C.c_double),
                ("v", C.c_void_p), ("normal_flow", C.c_double), ("X_out", C.c_void_p), ("v_out", C.c_void_p)]


class JobInfo(C.Structure):
    _fields_ = [("status", C.c_int), ("result", Result), ("submit_ms", C.c_double), ("admit_ms", C.c_double),
                ("done_ms", C.c_double), ("cohort", C.c_int), ("cohort_size", C.c_int), ("footprint", C.c_double)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "result"}
        d["result"] = self.result.as_dict()
        return d


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("completed", C.c_longlong), ("cohorts", C.c_longlong),
                ("peak_resident", C.c_double), ("peak_concurrency", C.c_int), ("device_bytes", C.c_double),
                ("peak_device", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class IDPError(RuntimeError):
    def __init__(self, code, where=""):
        self.code = code
        super().__init__(f"{where}: {status_str(code)} ({code})")


_lib = None
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


def load(path: str | None = None):
    """Load the C-ABI library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"{p} not found: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                          "(there is no CPU fallback)")
    L = C.CDLL(p)
    L.idp_create.restype = C.c_void_p
    L.idp_create.argtypes = [C.POINTER(Params), C.POINTER(C.c_int)]
    L.idp_destroy.argtypes = [C.c_void_p]
    L.idp_status_str.restype = C.c_char_p
    L.idp_default_params.argtypes = [C.POINTER(Params)]
    L.idp_add_instance.argtypes = [C.c_void_p, C.c_int, _dp, _dp, C.c_int, _ip, _dp, _dp, _dp, C.c_int, _ip,
                                   C.c_double, C.c_double, C.c_double]
    L.idp_set_velocity.argtypes = [C.c_void_p, C.c_int, _dp]
    L.idp_add_shell_instance.argtypes = [C.c_void_p, C.c_int, _dp, C.c_int, _ip, C.c_double, C.c_double, C.c_int,
                                         _ip, C.c_double, C.c_double, C.c_double]
    L.idp_set_positions.argtypes = [C.c_void_p, C.c_int, _dp]
    L.idp_set_normal_flow.argtypes = [C.c_void_p, C.c_int, C.c_double]
    L.idp_set_kappa.argtypes = [C.c_void_p, C.c_int, _dp]
    L.idp_tet_energy_noalloc.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
    L.idp_commit.argtypes = [C.c_void_p]
    L.idp_advance.argtypes = [C.c_void_p, C.POINTER(Result)]
    L.idp_step_begin.argtypes = [C.c_void_p]
    L.idp_step_iterate.argtypes = [C.c_void_p, C.c_int, C.POINTER(Result), C.POINTER(C.c_int)]
    L.idp_set_body_force.argtypes = [C.c_void_p, C.c_int, _dp]
    L.idp_set_dbc_targets.argtypes = [C.c_void_p, C.c_int, _dp]
    L.idp_add_elastic_shell_instance.argtypes = [C.c_void_p, C.c_int, _dp, _dp, C.c_int, _ip, _dp, C.c_double,
                                                 C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, _ip,
                                                 C.c_double, C.c_double, C.c_double]
    L.idp_get_state.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp]
    L.idp_instance_info.argtypes = [C.c_void_p, C.c_int] + [C.POINTER(C.c_int)] * 5
    L.idp_get_surface.argtypes = [C.c_void_p, C.c_int, _ip, _ip, _ip]
    L.idp_eval_energy.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp]
    L.idp_eval_gradient.argtypes = [C.c_void_p, C.c_int, _dp, _dp]
    L.idp_constraint_set.argtypes = [C.c_void_p, C.c_int, _dp, C.c_int, _ip, C.POINTER(C.c_int)]
    L.idp_ccd_stepsize.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp]
    L.idp_hessian_apply.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp]
    L.idp_newton_direction.argtypes = [C.c_void_p, C.c_int, _dp, _dp, C.POINTER(C.c_int), _dp]
    L.idp_get_stats.argtypes = [C.c_void_p, C.POINTER(Stats)]
    L.idp_check_intersection.argtypes = [C.c_void_p, C.c_int, _dp, C.c_int, _ip, C.POINTER(C.c_int)]
    L.idp_check_intersection_all.argtypes = [C.c_void_p, _ip]
    L.idp_reset.argtypes = [C.c_void_p]
    L.idp_device_bytes.argtypes = [C.c_void_p, C.POINTER(C.c_size_t)]
    L.idp_job_footprint.restype = C.c_double
    L.idp_job_footprint.argtypes = [C.c_int, C.c_int]
    L.idp_server_create.restype = C.c_void_p
    L.idp_server_create.argtypes = [C.POINTER(Params), C.c_double, C.c_int, C.c_int, C.POINTER(C.c_int)]
    L.idp_server_create_simulated.restype = C.c_void_p
    L.idp_server_create_simulated.argtypes = [C.c_double, C.c_int, C.c_int, C.c_double, C.POINTER(C.c_int)]
    L.idp_server_submit.argtypes = [C.c_void_p, C.POINTER(JobDesc)]
    L.idp_server_wait.argtypes = [C.c_void_p, C.c_int, C.POINTER(JobInfo)]
    L.idp_server_drain.argtypes = [C.c_void_p]
    L.idp_server_get_stats.argtypes = [C.c_void_p, C.POINTER(ServerStats)]
    L.idp_server_destroy.argtypes = [C.c_void_p]
    L.idp_save_state.argtypes = [C.c_void_p]
    L.idp_restore_state.argtypes = [C.c_void_p]
    _lib = L
    return L


def status_str(code: int) -> str:
    try:
        return load().idp_status_str(int(code)).decode()
    except ImportError:
        return str(code)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _pd(a):
    return a.ctypes.data_as(_dp)


def _pi(a):
    return a.ctypes.data_as(_ip)


def default_params(**kw) -> Params:
    p = Params()
    load().idp_default_params(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


class Context:
    """One device arena holding any number of mesh instances."""

    def __init__(self, **params):
        L = load()
        self.params = default_params(**params)
        st = C.c_int()
        self._h = L.idp_create(C.byref(self.params), C.byref(st))
        if not self._h:
            raise IDPError(st.value, "idp_create")
        self._V = []
        self._ndbc = []
        self.committed = False

    def close(self):
        if getattr(self, "_h", None):
            load().idp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, where, ok=(IDP_OK,)):
        if rc not in ok:
            raise IDPError(rc, where)
        return rc

    def add_instance(self, X, tets, mass, lam, mu, dHat2, kappa, kappa_max, X0=None, dbc_idx=None):
        X, tets, mass = _f64(X).reshape(-1, 3), _i32(tets).reshape(-1, 4), _f64(mass)
        V, T = X.shape[0], tets.shape[0]
        lam = _f64(np.broadcast_to(lam, (T,)))
        mu = _f64(np.broadcast_to(mu, (T,)))
        X0 = X if X0 is None else _f64(X0).reshape(-1, 3)
        dbc = _i32(np.zeros(0) if dbc_idx is None else dbc_idx)
        r = load().idp_add_instance(self._h, V, _pd(X), _pd(X0), T, _pi(tets), _pd(mass), _pd(lam), _pd(mu),
                                    dbc.size, _pi(dbc), float(dHat2), float(kappa), float(kappa_max))
        if r < 0:
            raise IDPError(-r, "idp_add_instance")
        self._V.append(V)
        self._ndbc.append(dbc.size)
        return r

    def add_shell_instance(self, X, faces, density, thickness, dHat2, kappa, kappa_max, dbc_idx=None):
        """Triangle shell advanced in flow mode (Laplacian flow energy)."""
        X, faces = _f64(X).reshape(-1, 3), _i32(faces).reshape(-1, 3)
        V = X.shape[0]
        dbc = _i32(np.zeros(0) if dbc_idx is None else dbc_idx)
        r = load().idp_add_shell_instance(self._h, V, _pd(X), faces.shape[0], _pi(faces), float(density),
                                          float(thickness), dbc.size, _pi(dbc), float(dHat2), float(kappa),
                                          float(kappa_max))
        if r < 0:
            raise IDPError(-r, "idp_add_shell_instance")
        self._V.append(V)
        self._ndbc.append(dbc.size)
        return r

    def add_elastic_shell_instance(self, X, faces, density, E, nu, thickness, dHat2, kappa, kappa_max,
                                   bending_mult=1.0, X0=None, dbc_idx=None, mass=None):
        """Elastic triangle shell (neo-Hookean membrane + hinge bending);
        mass (V) overrides the lumped masses from density."""
        X, faces = _f64(X).reshape(-1, 3), _i32(faces).reshape(-1, 3)
        V = X.shape[0]
        X0 = X if X0 is None else _f64(X0).reshape(-1, 3)
        dbc = _i32(np.zeros(0) if dbc_idx is None else dbc_idx)
        m = None if mass is None else _f64(mass)
        if m is not None and m.size != V:
            raise ValueError("mass: one value per vertex")
        r = load().idp_add_elastic_shell_instance(self._h, V, _pd(X), _pd(X0), faces.shape[0], _pi(faces),
                                                  None if m is None else _pd(m), float(density), float(E), float(nu),
                                                  float(thickness), float(bending_mult), dbc.size, _pi(dbc),
                                                  float(dHat2), float(kappa), float(kappa_max))
        if r < 0:
            raise IDPError(-r, "idp_add_elastic_shell_instance")
        self._V.append(V)
        self._ndbc.append(dbc.size)
        return r

    def set_velocity(self, i, v):
        v = _f64(v)
        self._check(load().idp_set_velocity(self._h, i, _pd(v)), "idp_set_velocity")

    def set_body_force(self, i, b):
        """Body force b (V,3) in the predictor x + (h v + h^2 M^-1 b); None removes it."""
        bb = None if b is None else _f64(b)
        self._check(load().idp_set_body_force(self._h, int(i), None if bb is None else _pd(bb)),
                    "idp_set_body_force")

    def set_dbc_targets(self, i, targets):
        """Targets (nDBC, 3) of instance i's DBC vertices in their dbc_idx
        order; vertices whose target differs from their position at a
        step's start move there (augmented Lagrangian). None: all fixed."""
        t = None if targets is None else _f64(targets)
        if t is not None and t.size != 3 * self._ndbc[i]:
            raise ValueError("targets: one (x, y, z) per DBC vertex of the instance")
        self._check(load().idp_set_dbc_targets(self._h, int(i), None if t is None else _pd(t)),
                    "idp_set_dbc_targets")

    def set_normal_flow(self, i, step):
        """x_tilde = x + step * n on surface vertices, x_tilde = x inside
        (instance i, or every instance for i = -1)."""
        self._check(load().idp_set_normal_flow(self._h, int(i), C.c_double(step)), "idp_set_normal_flow")

    def set_kappa(self, i, kappa3):
        k = np.ascontiguousarray(np.asarray(kappa3, dtype=np.float64).reshape(-1)[:3])
        if k.size < 3:
            k = np.concatenate([k, np.zeros(3 - k.size)])
        self._check(load().idp_set_kappa(self._h, int(i), _pd(k)), "idp_set_kappa")

    def set_positions(self, i, X):
        X = _f64(X)
        self._check(load().idp_set_positions(self._h, i, _pd(X)), "idp_set_positions")

    def commit(self):
        self._check(load().idp_commit(self._h), "idp_commit")
        self.committed = True

    def reset(self):
        """Drop the instances, keep the device buffers for the next set."""
        self._check(load().idp_reset(self._h), "idp_reset")
        self._V = []
        self._ndbc = []
        self.committed = False

    def device_bytes(self):
        n = C.c_size_t()
        self._check(load().idp_device_bytes(self._h, C.byref(n)), "idp_device_bytes")
        return n.value

    def advance(self, check=True):
        res = (Result * len(self._V))()
        rc = load().idp_advance(self._h, res)
        out = [r.as_dict() for r in res]
        if check:
            self._check(rc, "idp_advance", ok=(IDP_OK, IDP_WARN_ITER_CAP))
        return rc, out

    def step_begin(self):
        """x^n = x, predictor and initial constraint set / energy (the first
        part of advance)."""
        self._check(load().idp_step_begin(self._h), "idp_step_begin")

    def step_iterate(self, max_iters):
        """At most max_iters Newton iterations; returns (rc, n_active, results)."""
        res = (Result * len(self._V))()
        n = C.c_int()
        rc = load().idp_step_iterate(self._h, int(max_iters), res, C.byref(n))
        if rc in (IDP_ERR_CUDA, IDP_ERR_STATE, IDP_ERR_INVALID_ARG, IDP_ERR_CAPACITY):
            raise IDPError(rc, "idp_step_iterate")
        return rc, n.value, [r.as_dict() for r in res]

    def save_state(self):
        self._check(load().idp_save_state(self._h), "idp_save_state")

    def restore_state(self):
        self._check(load().idp_restore_state(self._h), "idp_restore_state")

    def set_positions_ptr(self, i, ptr):
        """Upload positions from a raw host pointer (e.g. pinned memory)."""
        self._check(load().idp_set_positions(self._h, i, C.cast(ptr, _dp)), "idp_set_positions")

    def set_velocity_ptr(self, i, ptr):
        self._check(load().idp_set_velocity(self._h, i, C.cast(ptr, _dp)), "idp_set_velocity")

    def state_ptr(self, i, x_ptr):
        """Read positions of instance i into a raw host pointer."""
        self._check(load().idp_get_state(self._h, i, C.cast(x_ptr, _dp), None, None), "idp_get_state")

    def stats(self):
        st = Stats()
        self._check(load().idp_get_stats(self._h, C.byref(st)), "idp_get_stats")
        return st.as_dict()

    def state(self, i):
        V = self._V[i]
        X, v, k = np.zeros((V, 3)), np.zeros((V, 3)), np.zeros(3)
        self._check(load().idp_get_state(self._h, i, _pd(X), _pd(v), _pd(k)), "idp_get_state")
        return X, v, k

    def surface(self, i):
        a = [C.c_int() for _ in range(5)]
        self._check(load().idp_instance_info(self._h, i, *[C.byref(x) for x in a]), "idp_instance_info")
        nn, ne, nt = a[2].value, a[3].value, a[4].value
        nodes, edges, tris = np.zeros(nn, np.int32), np.zeros((ne, 2), np.int32), np.zeros((nt, 3), np.int32)
        self._check(load().idp_get_surface(self._h, i, _pi(nodes), _pi(edges), _pi(tris)), "idp_get_surface")
        return dict(nodes=nodes, edges=edges, tris=tris)

    # ---- sub-steps (tests and callers that drive their own loop)
    def energy(self, i, X):
        X = _f64(X)
        e = [C.c_double() for _ in range(3)]
        rc = load().idp_eval_energy(self._h, i, _pd(X), *[C.byref(x) for x in e])
        if rc == IDP_ERR_INVERTED:
            return None
        self._check(rc, "idp_eval_energy")
        return tuple(x.value for x in e)

    def gradient(self, i, X):
        X = _f64(X)
        g = np.zeros(X.size)
        self._check(load().idp_eval_gradient(self._h, i, _pd(X), _pd(g)), "idp_eval_gradient")
        return g

    def constraint_set(self, i, X, cap=None):
        X = _f64(X)
        n = C.c_int()
        cap = cap or max(4096, 16 * self._V[i])
        while True:
            buf = np.zeros((cap, 4), np.int32)
            rc = load().idp_constraint_set(self._h, i, _pd(X), cap, _pi(buf), C.byref(n))
            if rc == IDP_ERR_CAPACITY:
                cap = n.value + 16
                continue
            self._check(rc, "idp_constraint_set")
            return buf[: n.value].copy()

    def ccd_stepsize(self, i, X, d, alpha=1.0):
        X, d = _f64(X), _f64(d)
        a = C.c_double(alpha)
        rc = load().idp_ccd_stepsize(self._h, i, _pd(X), _pd(d), C.byref(a))
        self._check(rc, "idp_ccd_stepsize", ok=(IDP_OK, IDP_WARN_ITER_CAP))
        return a.value, rc

    def intersections(self, i, X=None, cap=1024):
        """Intersecting (triangle, edge) pairs of instance i's surface at X
        (None: its current state), as surface-list indices, sorted."""
        Xa = None if X is None else _f64(X)
        n = C.c_int()
        while True:
            buf = np.zeros((max(cap, 1), 2), np.int32)
            rc = load().idp_check_intersection(self._h, i, None if Xa is None else _pd(Xa), cap, _pi(buf),
                                               C.byref(n))
            if rc == IDP_ERR_CAPACITY:
                cap = n.value + 16
                continue
            self._check(rc, "idp_check_intersection")
            return buf[: n.value].copy()

    def intersection_counts(self):
        """Number of intersecting pairs of every instance at its current state."""
        out = np.zeros(len(self._V), np.int32)
        self._check(load().idp_check_intersection_all(self._h, _pi(out)), "idp_check_intersection_all")
        return out

    def hessian_apply(self, i, X, x):
        X, x = _f64(X), _f64(x)
        y = np.zeros(x.size)
        self._check(load().idp_hessian_apply(self._h, i, _pd(X), _pd(x), _pd(y)), "idp_hessian_apply")
        return y

    def newton_direction(self, i, X):
        X = _f64(X)
        p = np.zeros(X.size)
        it, rel = C.c_int(), C.c_double()
        self._check(load().idp_newton_direction(self._h, i, _pd(X), _pd(p), C.byref(it), C.byref(rel)),
                    "idp_newton_direction")
        return p, it.value, rel.value


def job_footprint(V, T):
    """Admission estimate (bytes) of one job's device memory."""
    return load().idp_job_footprint(int(V), int(T))


class Server:
    """Continuous-batching request server (idp_server_*): jobs queue in
    arrival order; worker threads, each with its own context and stream,
    admit cohorts under the memory budget and solve them concurrently."""

    def __init__(self, hbm_budget, workers=2, max_batch=8, simulated_ms_per_kvertex=None, **params):
        L = load()
        st = C.c_int()
        if simulated_ms_per_kvertex is not None:
            self._h = L.idp_server_create_simulated(float(hbm_budget), int(workers), int(max_batch),
                                                    float(simulated_ms_per_kvertex), C.byref(st))
        else:
            p = default_params(**params)
            self._h = L.idp_server_create(C.byref(p), float(hbm_budget), int(workers), int(max_batch), C.byref(st))
        if not self._h:
            raise IDPError(st.value, "idp_server_create")
        self._keep = {}

    def submit(self, X, tets, mass, lam, mu, dHat2, kappa, kappa_max, v=None, normal_flow=0.0, X0=None,
               dbc_idx=None):
        """Queue one job; returns its id. Output buffers are kept until wait()."""
        X, tets, mass = _f64(X).reshape(-1, 3), _i32(tets).reshape(-1, 4), _f64(mass)
        V, T = X.shape[0], tets.shape[0]
        lam = _f64(np.broadcast_to(lam, (T,)))
        mu = _f64(np.broadcast_to(mu, (T,)))
        X0 = None if X0 is None else _f64(X0).reshape(-1, 3)
        v = None if v is None else _f64(v).reshape(-1, 3)
        dbc = None if dbc_idx is None else _i32(dbc_idx)
        Xo, vo = np.zeros((V, 3)), np.zeros((V, 3))
        ptr = lambda a: None if a is None else a.ctypes.data
        d = JobDesc(V, ptr(X), ptr(X0), T, ptr(tets), ptr(mass), ptr(lam), ptr(mu), 0 if dbc is None else dbc.size,
                    ptr(dbc), float(dHat2), float(kappa), float(kappa_max), ptr(v), float(normal_flow), ptr(Xo),
                    ptr(vo))
        jid = load().idp_server_submit(self._h, C.byref(d))
        if jid < 0:
            raise IDPError(-jid, "idp_server_submit")
        self._keep[jid] = (Xo, vo)
        return jid

    def wait(self, jid):
        """Block until job jid completes: (info dict, X, v)."""
        info = JobInfo()
        rc = load().idp_server_wait(self._h, int(jid), C.byref(info))
        if rc:
            raise IDPError(rc, "idp_server_wait")
        Xo, vo = self._keep.pop(jid)
        return info.as_dict(), Xo, vo

    def drain(self):
        rc = load().idp_server_drain(self._h)
        if rc:
            raise IDPError(rc, "idp_server_drain")

    def stats(self):
        st = ServerStats()
        rc = load().idp_server_get_stats(self._h, C.byref(st))
        if rc:
            raise IDPError(rc, "idp_server_get_stats")
        return st.as_dict()

    def close(self):
        if getattr(self, "_h", None):
            load().idp_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
