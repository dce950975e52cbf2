"""Mesh files of the reference's drivers (idp_gb300.meshio, restating
Utils/MESHIO.h readers and writers) on hand-written and round-tripped files."""
import math

import numpy as np
import pytest


def test_obj_reader_faces_quads_and_offsets(tmp_path):
    from idp_gb300 import meshio

    p = tmp_path / "m.obj"
    p.write_text("# comment\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvn 0 0 1\nvt 0 0\n"
                 "f 1 2 3\nf 1/1 3/3 4/4\nf 1//1 2//1 3//1 4//1\n")
    X, F, cnt = meshio.read_tri_obj(p)
    assert X.shape == (4, 3) and cnt == (0, 0, 4, 4)
    # plain triangle, slash tokens, then a quad split into (0,1,2) and (0,2,3)
    assert F.tolist() == [[0, 1, 2], [0, 2, 3], [0, 1, 2], [0, 2, 3]]
    # appending offsets the new faces by the vertices already present
    X2, F2, cnt2 = meshio.read_tri_obj(p, X, F)
    assert cnt2 == (4, 4, 8, 8)
    assert F2[4:].tolist() == (F + 4).tolist()


def scan_obj(path):
    """The reference's OBJ scan line by line: the first three numbers of each
    "v " line, _face_indices on each "f" line (quads split)."""
    from idp_gb300 import meshio

    pts, tris = [], []
    for line in open(path).read().splitlines():
        if line.startswith("v "):
            pts.append([float(x) for x in line[2:].split()[:3]])
        elif line.startswith("f"):
            tri, quad = meshio._face_indices(line)
            tris.append(tri)
            if quad is not None:
                tris.append([tri[0], tri[2], quad])
    return np.array(pts, dtype=np.float64).reshape(-1, 3), np.array(tris, dtype=np.int64).reshape(-1, 3)


@pytest.mark.parametrize("faces", ["f 1 2 3\nf 3 2 4\n", "f 1 2 3\nf  3 2 4\n", "f 1 2 3\nf 3\t2 4\n",
                                   "f 1 2 3\nf 3 2 4 1\n", "f 1/7/1 2/8/2 3/9/3\n", "f 1 2 3\nf -1 -2 -3\n",
                                   "f 1 2 3\nf +3 2 4\n", "f 1 2 3 \n"])
def test_obj_reader_matches_the_line_scan(tmp_path, faces):
    """The vectorised reader gives the line-by-line scan's arrays bit for bit:
    vertex coordinates in shortest-repr, %e and %.17g forms (with and without
    a w coordinate) and face lines that take the plain-triangle path or fall
    back to it (extra spaces, tabs, quads, slashes, signs, trailing space)."""
    from idp_gb300 import meshio

    rng = np.random.default_rng(3)
    vals = rng.standard_normal((4, 3)) * 10.0 ** rng.integers(-20, 20, (4, 3))
    fmt = [lambda v: repr(float(v)), lambda v: "%e" % v, lambda v: "%.17g" % v, lambda v: repr(float(v))]
    body = "".join("v " + " ".join(f(x) for x in row) + (" 1.0" if i == 3 else "") + "\n"
                   for i, (row, f) in enumerate(zip(vals, fmt)))
    p = tmp_path / "m.obj"
    p.write_text(body + faces)
    X, F, _ = meshio.read_tri_obj(p)
    Xs, Fs = scan_obj(p)
    assert np.array_equal(X, Xs) and np.array_equal(F, Fs.astype(np.int32))


def test_vtk_round_trip_and_counters(tmp_path):
    from idp_gb300 import meshgen, meshio

    X, T = meshgen.bar(2, 3, 4, seed=0)
    p = tmp_path / "bar.vtk"
    meshio.write_tet_vtk(p, X, T)
    X1, T1, cnt = meshio.read_tet_vtk(p)
    assert np.array_equal(X1, X) and np.array_equal(T1, T)
    assert cnt == (0, 0, X.shape[0], T.shape[0])
    X2, T2, cnt2 = meshio.read_tet_vtk(p, X1, T1)
    assert cnt2 == (X.shape[0], T.shape[0], 2 * X.shape[0], 2 * T.shape[0])
    assert np.array_equal(T2[T.shape[0]:], T + X.shape[0])
    bad = tmp_path / "bad.vtk"
    bad.write_text(p.read_text().replace(f"POINTS {X.shape[0]}", f"POINTS {X.shape[0] + 1}"))
    with pytest.raises(ValueError):
        meshio.read_tet_vtk(bad)


def test_obj_round_trip(tmp_path):
    from idp_gb300 import meshgen, meshio

    X, T, _ = meshgen.blob(n=10, lmax=3, seed=0)
    Xs, F = meshgen.shell_from_tets(X, T)
    p = tmp_path / "s.obj"
    meshio.write_tri_obj(p, Xs, F)
    X1, F1, _ = meshio.read_tri_obj(p)
    assert np.array_equal(F1, F)
    assert np.allclose(X1, Xs, rtol=1e-6, atol=1e-7)  # %e keeps 7 significant digits


def test_transform_points():
    from idp_gb300 import meshio

    X = np.array([[1.0, 0.0, 0.0], [2.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
    Y = meshio.transform_points(X.copy(), (0, 0, 10), (0, 0, 0), (0, 0, 1), 90.0, (2, 2, 2), (0, 0, 2, 0))
    assert np.allclose(Y[0], [0.0, 2.0, 10.0]) and np.allclose(Y[1], [0.0, 4.0, 10.0])
    assert np.array_equal(Y[2], X[2])  # outside the counter's range
    # rotation about an axis through a centre keeps distances to the axis
    rng = np.random.default_rng(0)
    P = rng.normal(size=(20, 3))
    Q = meshio.transform_points(P.copy(), (0, 0, 0), (1, 1, 1), (1, 2, 3), 37.0, (1, 1, 1))
    a = np.array([1, 2, 3]) / math.sqrt(14)
    d = lambda Z: np.linalg.norm(np.cross(Z - 1.0, a), axis=1)
    assert np.allclose(d(P), d(Q))


def test_tet_sim_reads_vtk(tmp_path):
    from idp_gb300 import meshgen, meshio
    from idp_gb300.api import TetIPCSim

    X, T = meshgen.bar(2, 2, 3, seed=1)
    p = tmp_path / "b.vtk"
    meshio.write_tet_vtk(p, X, T)
    sim = TetIPCSim()
    cnt = sim.add_object_3D(str(p), (1.0, 0.0, 0.0), (0, 0, 0), (1, 0, 0), 0.0, (1, 1, 1))
    cnt2 = sim.add_object_3D(str(p), (0.0, 5.0, 0.0), (0, 0, 0), (1, 0, 0), 0.0, (1, 1, 1))
    assert cnt == (0, 0, X.shape[0], T.shape[0])
    assert cnt2[0] == X.shape[0] and sim.tet.shape[0] == 2 * T.shape[0]
    assert np.allclose(sim.X[: X.shape[0]], X + [1.0, 0.0, 0.0])
    assert np.allclose(sim.X[X.shape[0]:], X + [0.0, 5.0, 0.0])


def test_obj_reader_matches_the_line_scan_on_random_faces(tmp_path):
    """Random face lines (index forms i, i/j, i//k, i/j/k; one or two spaces,
    tabs, trailing blanks, signs, quads) and plain ones: the reader's arrays
    equal the line scan's."""
    hyp = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")
    from idp_gb300 import meshio

    idx = st.integers(1, 9)
    token = st.one_of(idx.map(str), st.tuples(idx, idx).map(lambda t: f"{t[0]}/{t[1]}"),
                      st.tuples(idx, idx).map(lambda t: f"{t[0]}//{t[1]}"), idx.map(lambda i: f"+{i}"),
                      st.tuples(idx, idx, idx).map(lambda t: f"{t[0]}/{t[1]}/{t[2]}"))
    sep = st.sampled_from([" ", " ", " ", "  ", "\t"])
    face = st.tuples(st.lists(st.tuples(sep, token), min_size=3, max_size=4), st.sampled_from(["", " ", "\t"])).map(
        lambda t: "f" + "".join(a + b for a, b in t[0]) + t[1])
    plain = st.lists(idx, min_size=3, max_size=3).map(lambda t: "f " + " ".join(map(str, t)))
    body = "".join(f"v {i} {2 * i} {3 * i}\n" for i in range(9))
    n = [0]

    @hyp.settings(max_examples=150, deadline=None)
    @hyp.given(st.lists(st.one_of(face, plain), min_size=1, max_size=6))
    def check(lines):
        n[0] += 1
        p = tmp_path / f"r{n[0]}.obj"
        p.write_text(body + "\n".join(lines) + "\n")
        X, F, _ = meshio.read_tri_obj(p)
        Xs, Fs = scan_obj(p)
        assert np.array_equal(X, Xs) and np.array_equal(F, Fs.astype(np.int32))

    check()
