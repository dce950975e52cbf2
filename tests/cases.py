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
