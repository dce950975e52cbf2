"""Seeded synthetic tet meshes and deformation targets for the Newton-step
workloads (host-side input generation; numpy only).

* ``bar``: a box on an nx x ny x nz cube grid, every cube split into 5 tets
  (alternating split so faces conform), interior vertices jittered.
* ``bend_target``: maps the bar's centreline onto a circle (optionally with a
  twist), keeping cross-sections orthogonal, which makes the target surface
  self-intersect once the arc spans more than 2*pi.
* ``blob``: a star-shaped body r(u) = 1 + a * sum of real spherical harmonics,
  tetrahedralised on a background cube grid (cubes whose centre is inside).
* ``bar_batch``: many bars with log-uniform tet counts, for batched solves.
* ``cylinder`` / ``anim_keyframe``: the animation-fix sequence's tet cylinder
  and its bent and twisted keyframes.
* ``shell_from_tets``: the boundary of a tet mesh as a closed triangle shell
  (flow-mode workloads).

The reference reads these shapes from .vtk/.obj files
(``Python/Drivers/FEMDiscreteShellBase.py:184-188``); here they are generated
so every workload is reproducible from a seed.
"""
from __future__ import annotations

import math
import numpy as np

# corner index (a, b, c) -> local id a + 2b + 4c
_C = {(a, b, c): a + 2 * b + 4 * c for a in (0, 1) for b in (0, 1) for c in (0, 1)}
_SPLIT_EVEN = [
    [_C[0, 0, 0], _C[1, 1, 0], _C[1, 0, 1], _C[0, 1, 1]],
    [_C[1, 0, 0], _C[0, 0, 0], _C[1, 1, 0], _C[1, 0, 1]],
    [_C[0, 1, 0], _C[0, 0, 0], _C[1, 1, 0], _C[0, 1, 1]],
    [_C[0, 0, 1], _C[0, 0, 0], _C[1, 0, 1], _C[0, 1, 1]],
    [_C[1, 1, 1], _C[1, 1, 0], _C[1, 0, 1], _C[0, 1, 1]],
]
_SPLIT_ODD = [
    [_C[1, 0, 0], _C[0, 1, 0], _C[0, 0, 1], _C[1, 1, 1]],
    [_C[0, 0, 0], _C[1, 0, 0], _C[0, 1, 0], _C[0, 0, 1]],
    [_C[1, 1, 0], _C[1, 0, 0], _C[0, 1, 0], _C[1, 1, 1]],
    [_C[1, 0, 1], _C[1, 0, 0], _C[0, 0, 1], _C[1, 1, 1]],
    [_C[0, 1, 1], _C[0, 1, 0], _C[0, 0, 1], _C[1, 1, 1]],
]


def _orient(X: np.ndarray, tets: np.ndarray) -> np.ndarray:
    """Swap two vertices of every negatively oriented tet."""
    d = X[tets[:, 1:]] - X[tets[:, :1]]
    det = np.einsum("ti,ti->t", d[:, 0], np.cross(d[:, 1], d[:, 2]))
    tets = tets.copy()
    neg = det < 0
    tets[neg, 1], tets[neg, 2] = tets[neg, 2].copy(), tets[neg, 1].copy()
    return tets


def cube_grid_tets(mask: np.ndarray):
    """Tets of the cubes where ``mask[i, j, k]`` is True on a vertex lattice
    of shape (nx+1, ny+1, nz+1). Returns (vertex_ids_used, tets over lattice ids)."""
    nx, ny, nz = mask.shape
    vid = lambda i, j, k: (i * (ny + 1) + j) * (nz + 1) + k  # noqa: E731
    cubes = np.argwhere(mask)
    tets = []
    for i, j, k in cubes:
        corners = np.array([vid(i + a, j + b, k + c) for c in (0, 1) for b in (0, 1) for a in (0, 1)])
        split = _SPLIT_EVEN if (i + j + k) % 2 == 0 else _SPLIT_ODD
        for t in split:
            tets.append(corners[t])
    return np.asarray(tets, dtype=np.int64).reshape(-1, 4)


def _compact(Xlat: np.ndarray, tets: np.ndarray):
    used = np.unique(tets)
    remap = -np.ones(Xlat.shape[0], dtype=np.int64)
    remap[used] = np.arange(used.size)
    return Xlat[used].copy(), remap[tets]


def bar(nx=6, ny=6, nz=24, size=(1.0, 1.0, 4.0), jitter=0.05, seed=0):
    """Box [0,sx]x[0,sy]x[0,sz] on an nx x ny x nz cube grid, 5 tets per cube.
    Interior vertices are jittered uniformly by +-jitter*h (h = cube edge)."""
    sx, sy, sz = size
    xs = np.linspace(0, sx, nx + 1)
    ys = np.linspace(0, sy, ny + 1)
    zs = np.linspace(0, sz, nz + 1)
    X = np.stack(np.meshgrid(xs, ys, zs, indexing="ij"), -1).reshape(-1, 3)
    tets = cube_grid_tets(np.ones((nx, ny, nz), dtype=bool))
    h = min(sx / nx, sy / ny, sz / nz)
    rng = np.random.default_rng(seed)
    ii, jj, kk = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    interior = ((ii > 0) & (ii < nx) & (jj > 0) & (jj < ny) & (kk > 0) & (kk < nz)).reshape(-1)
    J = rng.uniform(-jitter * h, jitter * h, size=X.shape)
    X = X + J * interior[:, None]
    tets = _orient(X, tets)
    return X, tets.astype(np.int32)


def bend_target(X, angle=2.2 * math.pi, radius=0.5, size=(1.0, 1.0, 4.0), twist=0.0):
    """Centreline (x=sx/2, y=sy/2, z in [0,sz]) mapped onto a circle of the
    given radius spanning ``angle`` radians; cross-sections stay orthogonal to
    the centreline (x offset -> radial, y offset -> -z, orientation
    preserving). ``twist``
    rotates cross-sections by twist*s about the centreline."""
    sx, sy, sz = size
    s = X[:, 2] / sz
    th = angle * s
    ox, oy = X[:, 0] - sx / 2, X[:, 1] - sy / 2
    if twist:
        ph = twist * s
        ox, oy = ox * np.cos(ph) - oy * np.sin(ph), ox * np.sin(ph) + oy * np.cos(ph)
    n = np.stack([np.cos(th), np.sin(th), np.zeros_like(th)], -1)
    r = (radius + ox)[:, None]
    # (radial, -z, tangent) is right-handed, so the map keeps tet orientation
    return r * n - oy[:, None] * np.array([0.0, 0.0, 1.0])


def _real_sh(lmax, theta, phi):
    """Real spherical harmonics up to degree lmax (unnormalised associated
    Legendre via scipy), columns ordered (l, m)."""
    from scipy.special import sph_harm_y  # scipy >= 1.15

    cols, lm = [], []
    for l in range(1, lmax + 1):
        for m in range(-l, l + 1):
            Y = sph_harm_y(l, abs(m), theta, phi)
            if m < 0:
                cols.append(math.sqrt(2) * (-1) ** m * Y.imag)
            elif m == 0:
                cols.append(Y.real)
            else:
                cols.append(math.sqrt(2) * (-1) ** m * Y.real)
            lm.append(l)
    return np.stack(cols, -1), np.asarray(lm)


def blob(n=64, lmax=8, amp=0.3, seed=0):
    """Closed bumpy blob r(u) = 1 + amp * sum_{l<=lmax} c_lm Y_lm(u),
    c_lm ~ N(0, 1/l^2), tetrahedralised on an n^3 background grid: every cube
    whose centre lies inside is split into 5 tets. The grid spans the blob's
    largest radius (sampled on 20k Fibonacci directions) plus 2%; at n=64 and
    seed 0 this gives 220,515 tets."""
    rng = np.random.default_rng(seed)
    nlm = sum(2 * l + 1 for l in range(1, lmax + 1))
    ls = np.concatenate([[l] * (2 * l + 1) for l in range(1, lmax + 1)])
    coef = rng.normal(0.0, 1.0, nlm) / ls
    m = 20000
    k = np.arange(m) + 0.5
    Yd, _ = _real_sh(lmax, np.arccos(1.0 - 2.0 * k / m), np.pi * (1.0 + 5.0 ** 0.5) * k)
    ext = 1.02 * float((1.0 + amp * (Yd @ coef)).max())
    g = np.linspace(-ext, ext, n + 1)
    h = g[1] - g[0]
    cc = (g[:-1] + g[1:]) / 2
    C = np.stack(np.meshgrid(cc, cc, cc, indexing="ij"), -1).reshape(-1, 3)
    rr = np.linalg.norm(C, axis=1)
    theta = np.arccos(np.clip(C[:, 2] / np.maximum(rr, 1e-30), -1, 1))
    phi = np.arctan2(C[:, 1], C[:, 0])
    Y, _ = _real_sh(lmax, theta, phi)
    R = 1.0 + amp * (Y @ coef)
    inside = (rr < R).reshape(n, n, n)
    Xlat = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    tets = cube_grid_tets(inside)
    X, tets = _compact(Xlat, tets)
    tets = _orient(X, tets)
    return X, tets.astype(np.int32), h


def cylinder(radius=0.2, length=3.0, n_cross=22, n_len=None):
    """Solid cylinder along z (axis x = y = 0, z in [0, length]) on a cube
    grid of n_cross cells across the diameter: every cube whose centre lies
    within the radius is split into 5 tets. n_len defaults to cubes of equal
    edge. At n_cross=22 (n_len=165) this gives 316,800 tets and 71,214 vertices."""
    h = 2 * radius / n_cross
    n_len = n_len or int(round(length / h))
    gx = np.linspace(-radius, radius, n_cross + 1)
    gz = np.linspace(0.0, length, n_len + 1)
    cx = (gx[:-1] + gx[1:]) / 2
    cz = (gz[:-1] + gz[1:]) / 2
    CX, CY, _ = np.meshgrid(cx, cx, cz, indexing="ij")
    inside = CX ** 2 + CY ** 2 < radius ** 2
    Xlat = np.stack(np.meshgrid(gx, gx, gz, indexing="ij"), -1).reshape(-1, 3)
    tets = cube_grid_tets(inside)
    X, tets = _compact(Xlat, tets)
    tets = _orient(X, tets)
    return X, tets.astype(np.int32)


def bend_twist_target(X, angle, twist, length):
    """Centreline (the z axis, arc length s = z) bent in the x-z plane to a
    circular arc of total angle ``angle`` (either sign; arc length kept) and
    cross-sections twisted by twist * s / length. A point at offset (ox, oy)
    from the axis goes to c(s) + ox N(s) + oy y, with tangent T = (sin ks, 0,
    cos ks), normal N = (cos ks, 0, -sin ks), k = angle / length; (N, y, T)
    is right-handed, so tets keep their orientation while |k| * radius < 1."""
    s = X[:, 2]
    ph = twist * s / length
    ox = X[:, 0] * np.cos(ph) - X[:, 1] * np.sin(ph)
    oy = X[:, 0] * np.sin(ph) + X[:, 1] * np.cos(ph)
    k = angle / length
    if abs(k) < 1e-12:
        c = np.stack([np.zeros_like(s), np.zeros_like(s), s], -1)
        N = np.array([1.0, 0.0, 0.0])[None, :]
    else:
        ks = k * s
        c = np.stack([2.0 * np.sin(ks / 2) ** 2 / k, np.zeros_like(s), np.sin(ks) / k], -1)
        N = np.stack([np.cos(ks), np.zeros_like(s), -np.sin(ks)], -1)
    return c + ox[:, None] * N + oy[:, None] * np.array([0.0, 1.0, 0.0])


def anim_keyframe(X, t, length=3.0, frames=120):
    """Keyframe t of the animation-fix sequence: bend 2.4 pi sin(2 pi t /
    frames) and twist pi cos(2 pi t / (frames / 2)); frames whose bend
    exceeds 2 pi in magnitude self-penetrate."""
    ang = 2.4 * math.pi * math.sin(2 * math.pi * t / frames)
    tw = math.pi * math.cos(2 * math.pi * t / (frames / 2))
    return bend_twist_target(X, ang, tw, length)


def shell_from_tets(X, tets):
    """Boundary of a tet mesh as a closed triangle shell: faces that belong to
    one tet only, oriented outward, over the compacted boundary vertices."""
    outward = np.array([[1, 2, 3], [0, 3, 2], [0, 1, 3], [0, 2, 1]])
    F = tets[:, outward].reshape(-1, 3)
    key = np.sort(F, axis=1)
    _, inv, cnt = np.unique(key, axis=0, return_inverse=True, return_counts=True)
    F = F[cnt[inv.reshape(-1)] == 1]
    used = np.unique(F)
    remap = -np.ones(X.shape[0], dtype=np.int64)
    remap[used] = np.arange(used.size)
    return X[used].copy(), remap[F].astype(np.int32)


def bar_dims_for_tets(target_tets: float):
    """Grid (n, n, 4n) whose 5*4n^3 tets is closest to target_tets."""
    n = max(1, int(round((target_tets / 20.0) ** (1.0 / 3.0))))
    return n, n, 4 * n


def bar_batch(count=256, tmin=1_000, tmax=50_000, seed=0):
    """Bars with tet counts log-uniform in [tmin, tmax] and bend angles uniform
    in [1.5pi, 2.5pi]. Returns a list of dicts (X, tets, target, angle)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        t = math.exp(rng.uniform(math.log(tmin), math.log(tmax)))
        nx, ny, nz = bar_dims_for_tets(t)
        ang = rng.uniform(1.5 * math.pi, 2.5 * math.pi)
        X, tets = bar(nx, ny, nz, jitter=0.05, seed=int(rng.integers(1 << 31)))
        out.append(dict(X=X, tets=tets, target=bend_target(X, angle=ang), angle=ang))
    return out


def _tet_volumes(X, tets):
    d = X[tets[:, 1:]] - X[tets[:, :1]]
    return np.einsum("ti,ti->t", d[:, 0], np.cross(d[:, 1], d[:, 2])) / 6.0


def lumped_mass(X, tets, density):
    """Per-vertex lumped mass, vol * density / 4 per tet corner
    (FEM/ELEM_TO_NODE.h:11-46)."""
    m = np.zeros(X.shape[0])
    np.add.at(m, tets.reshape(-1), np.repeat(_tet_volumes(X, tets) * density / 4.0, 4))
    return m


def tet_body_force(X, tets, density, acc):
    """Body force of a body acceleration acc (V x 3): (vol * density / 4) acc
    added per tet corner, tets in order (Augment_Mass_Matrix_And_Body_Force,
    FEM/ELEM_TO_NODE.h:49-87)."""
    each = _tet_volumes(X, tets) * density / 4.0
    b = np.zeros((X.shape[0], 3))
    np.add.at(b, tets.reshape(-1), np.repeat(each, 4)[:, None] * np.asarray(acc, float)[None, :])
    return b


def lame(E, nu):
    """Lame parameters as NEOHOOKEAN_FUNCTOR::Append (Physics/NEOHOOKEAN.h:45-50)."""
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    mu = E / (2 * (1 + nu))
    return lam, mu
