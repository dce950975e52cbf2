"""The allocation-free elastic-energy entry point, idp_tet_energy_noalloc.

It serves callers that must not allocate device memory while they run (a
host application that reserved the GPU budget up front and lends the library
only its own buffers, or a frame loop that cannot take the device-wide
synchronisation of cudaMalloc/cudaFree). Its scratch is one fixed array in
the library shared by every call, so this file checks two calls in a row
(the second must not see the first one's leftovers, in particular the
inversion flag) against the context entry point idp_eval_energy, whose
elastic term is the same quantity, and against the CPU oracle's elastic
energy; and that a run of calls leaves the device's free memory unchanged.
The file name makes pytest collect it last.
"""
import ctypes as C
import math

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

TOL = 1e-9  # relative, as the other energy parity tests


def _rest(X0, tets):
    """Row-major inverse rest basis (columns x1-x0, x2-x0, x3-x0) and volume."""
    Dm = np.stack([X0[tets[:, k]] - X0[tets[:, 0]] for k in (1, 2, 3)], axis=-1)
    return np.linalg.inv(Dm).reshape(-1, 9), np.linalg.det(Dm) / 6.0


def _dev(torch, a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).cuda()


def test_tet_energy_noalloc_matches_context_entry(gpu_lib, oracle):
    import torch

    import idp_gb300 as idp
    from idp_gb300 import meshgen

    h = 0.1
    X0, tets = meshgen.bar(6, 6, 24, seed=0)  # 4,320 tets: five 1024-tet chunks
    T = tets.shape[0]
    pr = cases.problem(X0, tets)
    ctx = idp.Context(h=h, mode=idp.MODE_FP64)
    ctx.add_instance(X0, tets, pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], pr["kappa"], pr["kappa_max"])
    ctx.commit()

    IB, vol = _rest(X0, tets)
    d_tets = _dev(torch, tets, np.int32)
    d_IB = _dev(torch, IB, np.float64)
    d_vol = _dev(torch, vol, np.float64)
    d_lam = _dev(torch, np.full(T, pr["lam"]), np.float64)
    d_mu = _dev(torch, np.full(T, pr["mu"]), np.float64)
    energy = torch.full((1,), math.nan, dtype=torch.float64, device="cuda")
    inverted = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def call(X):
        d_X = _dev(torch, X, np.float64)
        rc = gpu_lib.idp_tet_energy_noalloc(T, d_tets.data_ptr(), d_X.data_ptr(), d_IB.data_ptr(), d_vol.data_ptr(),
                                            d_lam.data_ptr(), d_mu.data_ptr(), h * h, energy.data_ptr(),
                                            inverted.data_ptr(), stream)
        assert rc == idp.IDP_OK, idp.status_str(rc)
        torch.cuda.synchronize()
        return float(energy.item()), int(inverted.item())

    rng = np.random.default_rng(11)
    bent = meshgen.bend_target(X0, angle=0.8 * math.pi, radius=1.2)
    shaken = X0 + rng.uniform(-0.02, 0.02, X0.shape)
    # two calls in a row, each against the context entry point and the oracle
    lam_t, mu_t = np.full(T, pr["lam"]), np.full(T, pr["mu"])
    for X in (bent, shaken):
        e, bad = call(X)
        ref = ctx.energy(0, X)
        assert ref is not None
        assert bad == 0
        assert abs(e - ref[0]) <= TOL * abs(ref[0]), (e, ref[0])
        e_or = oracle.tet_energy(X, tets, np.ascontiguousarray(IB.reshape(-1, 3, 3)), vol, lam_t, mu_t, h * h)
        assert abs(e - e_or) <= TOL * abs(e_or), (e, e_or)

    # no device allocation: free memory unchanged over a run of calls
    d_X = _dev(torch, shaken, np.float64)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(20):
        rc = gpu_lib.idp_tet_energy_noalloc(T, d_tets.data_ptr(), d_X.data_ptr(), d_IB.data_ptr(), d_vol.data_ptr(),
                                            d_lam.data_ptr(), d_mu.data_ptr(), h * h, energy.data_ptr(),
                                            inverted.data_ptr(), stream)
        assert rc == idp.IDP_OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0

    # an inverted configuration raises the flag; the next call starts clean
    mirrored = X0 * np.array([-1.0, 1.0, 1.0])
    e_bad, bad = call(mirrored)
    assert bad == 1 and ctx.energy(0, mirrored) is None
    e2, bad2 = call(bent)
    assert bad2 == 0
    assert e2 == call(bent)[0]
    assert abs(e2 - ctx.energy(0, bent)[0]) <= TOL * abs(ctx.energy(0, bent)[0])

    # sizes beyond the fixed scratch are rejected before any GPU work
    rc = gpu_lib.idp_tet_energy_noalloc(16_777_217, d_tets.data_ptr(), d_tets.data_ptr(), d_IB.data_ptr(),
                                        d_vol.data_ptr(), d_lam.data_ptr(), d_mu.data_ptr(), 1.0, energy.data_ptr(),
                                        inverted.data_ptr(), stream)
    assert rc == idp.IDP_ERR_CAPACITY
    ctx.close()
