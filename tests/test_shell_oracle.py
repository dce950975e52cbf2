"""The oracle's discrete-shell elasticity (the Hinge path's membrane and
hinge bending): derivatives against finite differences, rest-state
identities, and the hinge stencils of small meshes."""
import numpy as np
import pytest


def sphere_shell(n=6, r=1.0, seed=0):
    """A closed triangulated sphere (subdivided octahedron), outward faces."""
    verts = [np.array(v, float) for v in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1))]
    faces = [(0, 2, 4), (2, 1, 4), (1, 3, 4), (3, 0, 4), (2, 0, 5), (1, 2, 5), (3, 1, 5), (0, 3, 5)]
    for _ in range(n // 3):
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
    X *= 1 + 0.02 * rng.standard_normal((X.shape[0], 1))
    return X, np.array(faces, np.int32)


def fd_grad(f, x, eps=1e-6):
    g = np.zeros(x.size)
    for i in range(x.size):
        xp, xm = x.copy().reshape(-1), x.copy().reshape(-1)
        xp[i] += eps
        xm[i] -= eps
        g[i] = (f(xp.reshape(x.shape)) - f(xm.reshape(x.shape))) / (2 * eps)
    return g


def test_dihedral_angle_derivatives_fd(oracle):
    rng = np.random.default_rng(1)
    for _ in range(6):
        x = rng.normal(size=(4, 3))
        t, g, H = oracle.dihedral(x)
        assert abs(t) <= np.pi
        gf = fd_grad(lambda y: oracle.dihedral(y)[0], x)
        assert np.linalg.norm(g - gf) <= 1e-7 * np.linalg.norm(gf)
        Hf = np.stack([fd_grad(lambda y, i=i: oracle.dihedral(y)[1][i], x) for i in range(12)])
        assert np.linalg.norm(H - Hf) <= 1e-6 * np.linalg.norm(Hf)
        assert np.allclose(H, H.T, atol=1e-12 * np.abs(H).max())
        # rigid motions: the angle is invariant, its gradient sums to zero
        assert np.linalg.norm(g.reshape(4, 3).sum(0)) <= 1e-12 * np.linalg.norm(g)


def test_membrane_rest_state_and_derivatives_fd(oracle):
    X0, F = sphere_shell(6)
    mem = oracle.membrane_rest(X0, F, 0.01, 1e5, 0.3)
    E0, g0, _ = oracle.membrane(X0, F, mem, 1.0, grad=True)
    assert abs(E0) <= 1e-12 and np.abs(g0).max() <= 1e-9  # rest state: no energy, no force
    rng = np.random.default_rng(2)
    X = X0 + 0.03 * rng.normal(size=X0.shape)
    E, g, H = oracle.membrane(X, F, mem, 0.01, grad=True, hess=True, project=False)
    gf = fd_grad(lambda y: oracle.membrane(y, F, mem, 0.01)[0], X)
    assert np.linalg.norm(g - gf) <= 1e-6 * np.linalg.norm(gf)
    # element Hessians against FD of the element gradients (a few faces)
    for f in range(0, F.shape[0], max(1, F.shape[0] // 5)):
        sub = F[f:f + 1]
        x = X.copy()

        def ge(y, i):
            return oracle.membrane(y, sub, mem[f:f + 1], 0.01, grad=True)[1][3 * sub[0][i // 3] + i % 3]

        Hf = np.stack([fd_grad(lambda y, i=i: ge(y, i), x)[(3 * sub[0][:, None] + np.arange(3)).reshape(-1)]
                       for i in range(9)])
        Hs = oracle.membrane(X, sub, mem[f:f + 1], 0.01, hess=True, project=False)[2][0]
        assert np.linalg.norm(Hs - Hf) <= 1e-5 * np.linalg.norm(Hf)
    # projection leaves PSD matrices with no negative eigenvalue
    _, _, Hp = oracle.membrane(X, F, mem, 0.01, hess=True, project=True)
    assert min(np.linalg.eigvalsh(h).min() for h in Hp) >= -1e-9 * max(np.abs(h).max() for h in Hp)


def test_hinges_and_bending_fd(oracle):
    X0, F = sphere_shell(6)
    surf = oracle.shell_surface(X0.shape[0], F)
    hin, info = oracle.shell_hinges(X0, F, surf["edges"])
    # closed surface: every edge is a hinge; hbar and ebar positive
    assert hin.shape[0] == surf["edges"].shape[0]
    assert np.all(info[:, 1] > 0) and np.all(info[:, 2] > 0)
    # the hinge edge is the surface edge, the opposite vertices are the faces' third vertices
    assert np.array_equal(hin[:, 1:3], surf["edges"])
    fs = {tuple(sorted(f)) for f in F.tolist()}
    for a, b, c, d in hin.tolist():
        assert tuple(sorted((a, b, c))) in fs and tuple(sorted((d, b, c))) in fs
    k = oracle.hinge_stiffness(1e5, 0.3, 0.01)
    E0, g0, _ = oracle.bending(X0, hin, info, k, 1.0, grad=True)
    assert abs(E0) <= 1e-20 and np.abs(g0).max() <= 1e-12
    rng = np.random.default_rng(3)
    X = X0 + 0.05 * rng.normal(size=X0.shape)
    E, g, H = oracle.bending(X, hin, info, k, 0.01, grad=True, hess=True, project=False)
    gf = fd_grad(lambda y: oracle.bending(y, hin, info, k, 0.01)[0], X)
    assert E > 0 and np.linalg.norm(g - gf) <= 1e-6 * np.linalg.norm(gf)
    # a flat sheet: rest angles zero
    Xp = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]], float)
    Fp = np.array([[0, 1, 2], [1, 3, 2]], np.int32)
    sp = oracle.shell_surface(4, Fp)
    hp, ip = oracle.shell_hinges(Xp, Fp, sp["edges"])
    assert hp.shape[0] == 1 and abs(ip[0, 0]) <= 1e-15
    assert ip[0, 1] == pytest.approx(np.sqrt(2.0)) and ip[0, 2] == pytest.approx(2.0 / (6 * np.sqrt(2.0)))
