"""Seeded contact configurations shared by the oracle and GPU parity tests."""
import math

import numpy as np

from idp_gb300 import meshgen


def two_bars(gap, seed=0, n=(2, 2, 4), shift=0.3):
    """Two jittered bars side by side with a small gap in x (many PT/EE pairs)."""
    X, tets = meshgen.bar(*n, size=(1.0, 1.0, 2.0), jitter=0.05, seed=seed)
    Y = X.copy()
    Y[:, 0] += 1.0 + gap
    rng = np.random.default_rng(seed + 100)
    Y[:, 1] += rng.uniform(-shift, shift)
    Y[:, 2] += rng.uniform(-shift, shift)
    return np.concatenate([X, Y]), np.concatenate([tets, tets + X.shape[0]]).astype(np.int32)


def folded_bar(seed=0, n=(3, 3, 10), angle=2.05 * math.pi, frac=1.0, radius=0.52):
    """A bar and a configuration part-way to a self-overlapping circle; returns
    (rest X, tets, deformed positions). frac < 1 stops before the overlap."""
    X, tets = meshgen.bar(*n, size=(1.0, 1.0, 3.0), jitter=0.05, seed=seed)
    T = meshgen.bend_target(X, angle=angle * frac, radius=radius, size=(1.0, 1.0, 3.0))
    return X, tets, T


def problem(X, tets, density=1000.0, E=1e4, nu=0.3, dhat_rel=1e-3, dHat=None):
    from oracle import kappa_init

    mass = meshgen.lumped_mass(X, tets, density)
    lam, mu = meshgen.lame(E, nu)
    diag = float(np.linalg.norm(X.max(0) - X.min(0)))
    dHat2 = (dhat_rel * diag) ** 2 if dHat is None else dHat * dHat
    k, km = kappa_init(float(mass.mean()), dHat2)
    return dict(mass=mass, lam=lam, mu=mu, dHat2=dHat2, kappa=k, kappa_max=km)


def sphere_shell(levels=2, r=1.0, seed=0, noise=0.02):
    """A closed triangulated sphere (octahedron subdivided `levels` times,
    outward faces), radii jittered by `noise` (seeded)."""
    verts = [np.array(v, float) for v in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1))]
    faces = [(0, 2, 4), (2, 1, 4), (1, 3, 4), (3, 0, 4), (2, 0, 5), (1, 2, 5), (3, 1, 5), (0, 3, 5)]
    for _ in range(levels):
        cache, nf = {}, []

        def mid(a, b):
            k = (min(a, b), max(a, b))
            if k not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[k] = len(verts) - 1
            return cache[k]

        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (ab, b, bc), (ca, bc, c), (ab, bc, ca)]
        faces = nf
    X = r * np.array(verts)
    rng = np.random.default_rng(seed)
    X *= 1 + noise * rng.standard_normal((X.shape[0], 1))
    return X, np.array(faces, np.int32)


def shell_problem(X, faces, density=1000.0, E=1e5, nu=0.3, thickness=0.01, dhat_rel=1e-3, dHat=None):
    """Elastic-shell parameters as the Hinge path's drivers set them
    (Initialize_Discrete_Shell masses, Initialize_OIPC kappa)."""
    from oracle import kappa_init

    F = faces.shape[0]
    mass = np.zeros(X.shape[0])
    for f in range(F):
        a, b, c = faces[f]
        area = np.linalg.norm(np.cross(X[b] - X[a], X[c] - X[a])) / 2
        mass[[a, b, c]] += area * thickness * density / 3
    diag = float(np.linalg.norm(X.max(0) - X.min(0)))
    dHat2 = (dhat_rel * diag) ** 2 if dHat is None else dHat * dHat
    k, km = kappa_init(float(mass.mean()), dHat2)
    return dict(mass=mass, density=density, E=E, nu=nu, thickness=thickness, dHat2=dHat2, kappa=k, kappa_max=km)
