"""CPU checks of the C-ABI boundary: the library builds for sm_103a, loads
without a GPU, and exports every entry point include/idp_gb300.h declares;
the Python bindings declare the same set."""
import os
import re
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "idp_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(idp_[a-z_0-9]+)\s*\(", src)))


def test_library_exports_header_symbols(gpu_lib):
    import idp_gb300

    names = header_functions()
    assert names, "no declarations parsed"
    for n in names:
        assert hasattr(gpu_lib, n), n
    assert sorted(idp_gb300.EXPORTS) == names
    out = subprocess.run(["nm", "-D", "--defined-only", idp_gb300.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (idp_[a-z_0-9]+)$", out, flags=re.M))
    assert set(names) <= exported


def test_status_strings(gpu_lib):
    import idp_gb300

    for code in range(11):
        s = idp_gb300.status_str(code)
        assert isinstance(s, str) and s and s != "unknown status"


def test_create_without_gpu_fails_cleanly(gpu_lib):
    import idp_gb300
    import torch

    if torch.cuda.is_available():
        return
    try:
        idp_gb300.Context()
    except idp_gb300.IDPError as e:
        assert e.code == idp_gb300.IDP_ERR_CUDA
    else:
        raise AssertionError("context created without a GPU")


def test_reference_shaped_shim_rejects_unsupported_inputs(gpu_lib):
    import numpy as np
    import pytest
    from idp_gb300.api import FEM

    args = [None] * 42
    args[0] = np.zeros((3, 3))  # shell elements are not part of this path
    with pytest.raises(NotImplementedError):
        FEM.DiscreteShell.Advance_One_Step_IE_Hinge(*args)


def test_reference_shaped_shim_reads_dbc_rows(gpu_lib):
    """DBC rows (index, x, y, z) give the vertex list and the targets (a
    target away from the vertex's position is a moving DBC, solved by the
    augmented Lagrangian); a bare index list has no targets."""
    import numpy as np
    from idp_gb300.api import _dbc_rows

    idx, t = _dbc_rows(np.array([[1, 3.0, 4.0, 5.5], [3, 0.0, 1.0, 2.0]]))
    assert list(idx) == [1, 3] and np.array_equal(t, [[3.0, 4.0, 5.5], [0.0, 1.0, 2.0]])
    idx, t = _dbc_rows(np.array([2, 0]))
    assert list(idx) == [2, 0] and t is None
    assert _dbc_rows(None) == (None, None)
