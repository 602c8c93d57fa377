"""Parity of the CUDA path (through the C ABI) with the reference's own
outputs (golden fixtures) and with the oracle, FP64.  Tolerances: relative
L2 <= 1e-12 for one RHS evaluation and for a few RK4 steps (RTOL_RHS,
RTOL_RK4 in helpers.py); integer/index work (face tables) is exact."""
import numpy as np
import pytest

import nmesh_gb300 as ng
from helpers import (BIG_CASE, CASES, DTAUTO_CASES, PI, RTOL_RHS, RTOL_RK4, big_case_u0,
                     build_mesh, gaussian_pulses, load, oracle_for, perm_to_mesh, rel_l2,
                     to_mesh_order)

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _gpu(cuda_ok):
    yield


VARIANTS = ["eo", "eof", "eofu", "gather"]


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("case", CASES)
def test_rhs_matches_reference(case, variant):
    d, meta = load(case)
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    ev.set_kernel(variant)
    r = ev.rhs(to_mesh_order(d["u0"], perm), 0.0)
    assert rel_l2(r[perm], d["r0"]) <= RTOL_RHS
    # pointwise: no node off by more than 1e-11 of the largest |r|
    assert np.abs(r[perm] - d["r0"]).max() <= 1e-11 * np.abs(d["r0"]).max()


@pytest.mark.parametrize("variant", VARIANTS + ["auto"])
@pytest.mark.parametrize("case", CASES)
def test_rk4_matches_reference(case, variant):
    d, meta = load(case)
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    ev.set_kernel(variant)
    u = ev.rk4_steps_host(to_mesh_order(d["u0"], perm), 0.0, meta["dt"], meta["steps"])
    assert rel_l2(u[perm], d["u_final"]) <= RTOL_RK4
    # the single-step entry point gives the same state
    ev.set_state(to_mesh_order(d["u0"], perm))
    t = 0.0
    for s in range(meta["steps"]):
        ev.rk4_step(t, meta["dt"])
        t += meta["dt"]
    assert rel_l2(ev.get_state()[perm], d["u_final"]) <= RTOL_RK4


@pytest.mark.parametrize("n,luni", [(2, 1), (3, 2), (4, 1), (5, 1), (6, 1), (7, 0), (8, 1), (9, 1),
                                    (10, 0), (11, 0), (12, 0)])
@pytest.mark.parametrize("variant", VARIANTS)
def test_cubed_spheres_outgoing_vs_oracle(n, luni, variant):
    """Every compiled order: Gaussian pulses, outgoing-radiation outer
    boundary (restated, no reference counterpart), against the oracle."""
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=n, luni=luni, cs_dc=1.0, cs_r0fac=20.0)
    u = gaussian_pulses(m.coords(), seed=n * 10 + luni, rmin=1.0, rmax=6.0)
    u += 1e-3 * np.random.default_rng(n).standard_normal(u.shape)
    o = oracle_for(m, bc=1)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_kernel(variant)
    r = ev.rhs(u, 0.0)
    ro = o.rhs(u, 0.0)
    assert rel_l2(r, ro) <= RTOL_RHS
    dt = 0.02 / n ** 2
    uf = ev.rk4_steps_host(u, 0.0, dt, 3)
    uo = o.rk4(u, dt, 3)
    assert rel_l2(uf, uo) <= RTOL_RK4


@pytest.mark.parametrize("n,luni", [(5, 1), (5, 0), (4, 2)])
@pytest.mark.parametrize("variant", VARIANTS)
def test_periodic_box_vs_oracle(n, luni, variant):
    """Periodic cube [0, 2 pi]^3 (the reference has no periodic faces; the
    oracle restates them as plain face connections).  luni=0 makes the only
    element its own neighbour on all six faces."""
    m = ng.Mesh.build(ng.MESH_BOX, n=n, luni=luni, xc=(PI, PI, PI), box_dout=PI,
                      periodic=True)
    nb, _ = m.faces()
    assert (nb >= 0).all()
    rng = np.random.default_rng(luni)
    xyz = m.coords()
    amp = rng.uniform(0.5, 1.5)
    arg = xyz.sum(axis=1)
    u = amp * np.stack([-np.sqrt(3) * np.cos(arg), np.cos(arg), np.cos(arg), np.cos(arg),
                        np.sin(arg)], 1)
    u += 0.01 * rng.standard_normal(u.shape)
    o = oracle_for(m, period=2 * PI)
    ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=(1.0, 1.0, 1.0))
    ev.set_kernel(variant)
    assert rel_l2(ev.rhs(u), o.rhs(u)) <= RTOL_RHS
    dt = 0.25 * (2 * PI / 2 ** luni) / (n - 1) ** 2
    assert rel_l2(ev.rk4_steps_host(u, 0.0, dt, 4), o.rk4(u, dt, 4)) <= RTOL_RK4


def test_rhs_device_pointers_and_determinism():
    import torch
    d, meta = load("cs7_l1_n5")
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    u = to_mesh_order(d["u0"], perm)
    w = torch.from_numpy(u).cuda()
    r = torch.empty_like(w)
    torch.cuda.synchronize()
    ev.rhs_device(w.data_ptr(), r.data_ptr(), 0.0)
    torch.cuda.synchronize()
    r1 = ev.rhs(u)
    ev.rhs_device(w.data_ptr(), r.data_ptr(), 0.0)
    torch.cuda.synchronize()
    # bitwise deterministic across calls and entry points
    assert np.array_equal(r.cpu().numpy(), r1)
    assert rel_l2(r1[perm], d["r0"]) <= RTOL_RHS


def test_zero_steps_and_bad_arguments():
    d, meta = load("box_l1_n5")
    m = build_mesh(meta)
    ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    u = np.ones(ev.shape)
    assert np.array_equal(ev.rk4_steps_host(u, 0.0, 0.01, 0), u)
    with pytest.raises(ng.NmgError):
        ev.rk4_steps(0.0, 0.01, -1)
    with pytest.raises(ng.NmgError):
        ng.Evolution(m, bc=7)


def test_autotuner_and_every_tile_shape():
    """The autotuner times every compiled variant/tile shape; each one of
    them must give the reference's RHS."""
    d, meta = load("cs7_l1_n5")
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    u = to_mesh_order(d["u0"], perm)
    ev.rhs(u)
    info = ev.kernel_info()
    assert "timings" in info
    cands = info.split("candidates:")[1].split("|")[0].split()
    assert any(c.startswith("eo") for c in cands) and any(c.startswith("gather") for c in cands)
    for c in cands:
        ev.set_kernel(c)
        assert rel_l2(ev.rhs(u)[perm], d["r0"]) <= RTOL_RHS, c
    with pytest.raises(ng.NmgError):
        ev.set_kernel("nonsense")


@pytest.mark.parametrize("variant", ["eo:2:128", "eo:4:256", "gather", "eof"])
@pytest.mark.parametrize("nsteps", [1, 3])
def test_host_round_trip_streams_last_stage_bitwise(variant, nsteps):
    """nmg_rk4_steps_host runs its last stage in element chunks and copies
    each chunk back while the next computes; the state equals the resident
    multi-step path bit for bit."""
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=5, luni=2, cs_dc=1.0, cs_r0fac=20.0)
    u = gaussian_pulses(m.coords(), seed=4, rmin=1.0, rmax=6.0)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_kernel(variant)
    got = ev.rk4_steps_host(u, 0.0, 0.01, nsteps)
    ev.set_state(u)
    ev.rk4_steps(0.0, 0.01, nsteps)
    assert np.array_equal(got, ev.get_state())


def test_periodic_cube_plane_wave_workload():
    """The periodic-cube workload: [0, 2 pi]^3, 8^3 elements, n = 5, plane
    wave psi = A sin(x + y + z) with a seeded amplitude, LLF, RK4 with
    dt = 0.25 (2 pi / 8) / 16, 10 steps: the oracle within 1e-12 and the exact
    solution within the scheme's truncation error."""
    m = ng.Mesh.build(ng.MESH_BOX, n=5, luni=3, xc=(PI, PI, PI), box_dout=PI, periodic=True)
    A = np.random.default_rng(2024).uniform(0.5, 1.5)
    xyz = m.coords()
    om = np.sqrt(3.0)

    def exact(t):
        arg = xyz[:, 0] + xyz[:, 1] + xyz[:, 2] - om * t
        c, s = np.cos(arg), np.sin(arg)
        return A * np.stack([-om * c, c, c, c, s], 1)

    dt = 0.25 * (2 * PI / 8) / 16
    u0 = exact(0.0)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    u = ev.rk4_steps_host(u0, 0.0, dt, 10)
    o = oracle_for(m, bc=1, period=2 * PI)
    assert rel_l2(u, o.rk4(u0, dt, 10)) <= RTOL_RK4
    assert rel_l2(u, exact(10 * dt)) <= 1e-3


@pytest.mark.parametrize("case", DTAUTO_CASES)
def test_step_with_auto_dt_matches_reference(case):
    """A step of the reference's run with dt = auto, taken with the mesh's
    own automatic dt."""
    d, meta = load(case)
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    if "fv" in meta:
        ev.set_fv(meta["fv"]["rec"], meta["fv"]["extrap"])
    u = ev.rk4_steps_host(to_mesh_order(d["u0"], perm), 0.0, m.auto_dt(), meta["steps"])
    assert rel_l2(u[perm], d["u_final"]) <= RTOL_RK4


@pytest.mark.parametrize("variant", ["auto", "eo", "gather"])
def test_benchmark_order_level2_matches_reference(variant):
    """The benchmark's mesh family and order (7 CubedSpheres, 9 LGL nodes)
    at level 2, 448 elements, 1.6 M DOF, against the reference's own run:
    the RHS and 10 RK4 steps with the benchmark's dt formula, on the
    elements the fixture keeps and through the full norms."""
    d, meta = load(BIG_CASE)
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    u0 = to_mesh_order(big_case_u0(d, meta), perm)
    ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    ev.set_kernel(variant)
    sel = d["sel"]
    r = ev.rhs(u0, 0.0)[perm]
    assert rel_l2(r[sel], d["r0_sel"]) <= RTOL_RHS
    assert abs(np.linalg.norm(r.ravel()) / float(d["r0_norm"]) - 1) <= RTOL_RHS
    ev.set_state(u0)
    ev.rk4_steps(0.0, meta["dt"], meta["steps"])
    u = ev.get_state()[perm]
    assert rel_l2(u[sel], d["u_final_sel"]) <= RTOL_RK4
    assert abs(np.linalg.norm(u.ravel()) / float(d["u_final_norm"]) - 1) <= RTOL_RK4


def test_benchmark_workload_drift_over_100_steps():
    """The benchmark's workload at level 2 (7 CubedSpheres, n = 9, 448
    elements): 8 seeded Gaussian pulses (the benchmark's seed), outgoing
    boundary, dt = 0.25 (2 / 2^2) / 8^2, graph-captured RK4 steps with the
    autotuned kernel as the benchmark takes them, against the oracle after
    1, 10 and 100 steps: relative L2 <= 1e-12 at every checkpoint (the
    measured drift is printed)."""
    n, L = 9, 2
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=n, luni=L, cs_dc=1.0, cs_r0fac=20.0)
    u0 = gaussian_pulses(m.coords(), seed=1234)
    dt = 0.25 * (2.0 / 2 ** L) / (n - 1) ** 2
    o = oracle_for(m, bc=1)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_state(u0)
    assert rel_l2(ev.rhs(u0, 0.0), o.rhs(u0, 0.0)) <= RTOL_RHS
    uo, done, drift = u0, 0, {}
    for target in (1, 10, 100):
        ev.rk4_steps(done * dt, dt, target - done)
        uo = o.rk4(uo, dt, target - done, t=done * dt)
        done = target
        drift[target] = rel_l2(ev.get_state(), uo)
    print(f"\nbenchmark workload at level 2, relative L2 GPU vs oracle after 1/10/100 steps: "
          f"{drift[1]:.3e} {drift[10]:.3e} {drift[100]:.3e}")
    assert max(drift.values()) <= RTOL_RK4


def test_full_benchmark_workload_against_oracle_and_properties():
    """The benchmark's workload at its full size (7 x 16^3 elements, n = 9,
    104.5 M DOF, 8 seeded pulses, outgoing boundary, its dt): the RHS and
    one RK4 step with the autotuned kernel against the oracle on the
    oracle's own mesh (within 1e-12), two runs of a step bitwise equal, and
    the linearity of the step, step(a u + b v) = a step(u) + b step(v)."""
    n, L = 9, 4
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=n, luni=L, cs_dc=1.0, cs_r0fac=20.0)
    from oracle import nmo
    pat, bbox, curvi, xyz, dXdx = nmo.generate_mesh(nmo.MESH_CUBEDSPHERES7, n, L)
    assert np.array_equal(m.elements()[1], bbox)
    o = nmo.OracleMesh(bbox, curvi, dXdx, xyz, nmo.match_faces_conforming(xyz, n), n, bc=1)
    del dXdx
    u = gaussian_pulses(xyz, seed=1234)
    del xyz
    dt = 0.25 * (2.0 / 2 ** L) / (n - 1) ** 2
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    r = ev.rhs(u, 0.0)
    assert rel_l2(r, o.rhs(u, 0.0)) <= RTOL_RHS
    del r
    ev.set_state(u)
    ev.rk4_steps(0.0, dt, 1)
    s1 = ev.get_state()
    assert rel_l2(s1, o.rk4(u, dt, 1)) <= RTOL_RK4
    ev.set_state(u)
    ev.rk4_steps(0.0, dt, 1)
    assert np.array_equal(ev.get_state(), s1)
    v = np.random.default_rng(5).standard_normal(u.shape) * 1e-3
    ev.set_state(v)
    ev.rk4_steps(0.0, dt, 1)
    sv = ev.get_state()
    ev.set_state(2.0 * u - 3.0 * v)
    ev.rk4_steps(0.0, dt, 1)
    assert rel_l2(ev.get_state(), 2.0 * s1 - 3.0 * sv) <= 1e-13
    ev.close()
