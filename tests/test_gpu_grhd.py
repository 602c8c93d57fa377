"""GRHD conservative <-> primitive conversion on the GPU through the C ABI
against the oracle restatement (same operation order, no FMA contraction:
bit for bit), round trips, atmosphere resets and argument checks."""
import numpy as np
import pytest

import nmesh_gb300 as ng
from oracle import nmo
from test_grhd_oracle import random_prims

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(autouse=True)
def _gpu(cuda_ok):
    yield


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("conformal", [False, True])
def test_gpu_prim2con_con2prim_bitexact_vs_oracle(conformal):
    n = 20000
    prim = random_prims(n, seed=11)
    ps = None
    if conformal:
        ps = 1.0 + np.random.default_rng(12).uniform(0, 0.5, n)
        prim[1:4] /= ps ** 2
    g = ng.GrhdParams()
    dprim = _dev(prim)
    dcons = torch.zeros_like(dprim)
    dps = _dev(ps) if ps is not None else None
    ng.grhd_prim2con_device(g, n, dps.data_ptr() if dps is not None else 0,
                            dprim.data_ptr(), dcons.data_ptr())
    torch.cuda.synchronize()
    cons_o = nmo.grhd_prim2con(prim, ps)
    cons = dcons.cpu().numpy()
    assert np.array_equal(cons, cons_o)
    # spoil some points: atmosphere and failures
    cons[0, :50] = 1e-20
    cons[4, 50:100] = -3.0
    cons[:, 100:110] = np.nan
    guess = prim.copy()
    guess[4] *= 0.7
    dcons = _dev(cons)
    dguess = _dev(guess)
    dst = torch.zeros(n, dtype=torch.int32, device="cuda")
    ng.grhd_con2prim_device(g, n, dps.data_ptr() if dps is not None else 0,
                            dcons.data_ptr(), dguess.data_ptr(), dst.data_ptr())
    torch.cuda.synchronize()
    po, co, so = nmo.grhd_con2prim(cons, guess, ps)
    assert np.array_equal(dst.cpu().numpy(), so)
    assert np.array_equal(dguess.cpu().numpy(), po)
    assert np.array_equal(dcons.cpu().numpy(), co)
    assert (so[:110] < 0).all() and (so[110:] >= 0).all()
    rel = np.abs(po[:, 110:] - prim[:, 110:]) / np.maximum(np.abs(prim[:, 110:]), 1e-300)
    assert rel[[0, 4]].max() <= 1e-9


def test_gpu_grhd_rejects_bad_params():
    d = torch.zeros(10, dtype=torch.float64, device="cuda")
    with pytest.raises(ng.NmgError):
        ng.grhd_prim2con_device(ng.GrhdParams(gamma=1.0), 2, 0, d.data_ptr(), d.data_ptr())
    with pytest.raises(ng.NmgError):
        ng.grhd_con2prim_device(ng.GrhdParams(maxits=0), 2, 0, d.data_ptr(), d.data_ptr(),
                                d.data_ptr())
