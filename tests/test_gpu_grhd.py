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


def test_gpu_grhd_fluxes_sources_bitexact_vs_oracle():
    n = 5000
    rng = np.random.default_rng(21)
    prim = random_prims(n, seed=22)
    psi = rng.uniform(1.0, 1.4, n)
    prim[1:4] /= psi ** 2
    alpha = rng.uniform(0.4, 1.0, n)
    da = rng.normal(size=(3, n))
    dp = rng.normal(size=(3, n))
    g = ng.GrhdParams()
    dprim, dpsi_, dal = _dev(prim), _dev(psi), _dev(alpha)
    dflux = torch.zeros_like(dprim)
    dlam = torch.zeros(2 * n, dtype=torch.float64, device="cuda")
    for d in range(3):
        ng.grhd_fluxes_device(g, n, d, dal.data_ptr(), dpsi_.data_ptr(), dprim.data_ptr(),
                              dflux.data_ptr(), dlam.data_ptr())
        torch.cuda.synchronize()
        fo, lo = nmo.grhd_fluxes(prim, d, alpha, psi)
        assert np.array_equal(dflux.cpu().numpy(), fo)
        assert np.array_equal(dlam.cpu().numpy().reshape(2, n), lo)
    dsrc = torch.zeros_like(dprim)
    dda, ddp = _dev(da), _dev(dp)      # kept alive until the kernel has run
    ng.grhd_sources_device(g, n, dal.data_ptr(), dpsi_.data_ptr(), dda.data_ptr(),
                           ddp.data_ptr(), dprim.data_ptr(), dsrc.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(dsrc.cpu().numpy(), nmo.grhd_sources(prim, alpha, psi, da, dp))
