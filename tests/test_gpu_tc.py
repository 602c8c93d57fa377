"""The tensor-core stage kernel ("tc", n = 7, 8, 9; most cases at 9, the benchmark's order).  Its directional derivatives
are exact integer digit products on the FP16 tensor cores: seven signed
8-bit digits per value on a per-element-field fixed-point grid, seven digit
groups summed in FP32 without rounding, recombined in 64-bit integers into
FP64.  Held to the same bar as the FP64 variants: the reference's own runs
at n = 9 and the oracle within relative L2 1e-12 (RTOL_RHS, RTOL_RK4),
bitwise determinism, and the inputs that stress a fixed-point grid: fields
spanning many orders of magnitude across and inside elements, scales near
the ends of the FP64 range, all-zero fields, NaN."""
import numpy as np
import pytest

import nmesh_gb300 as ng
from helpers import (BIG_CASE, PI, RTOL_RHS, RTOL_RK4, big_case_u0, build_mesh,
                     gaussian_pulses, load, oracle_for, perm_to_mesh, rel_l2, to_mesh_order)

pytestmark = pytest.mark.gpu

TC = ["tc:1:192", "tc:1:256"]


@pytest.fixture(autouse=True)
def _gpu(cuda_ok):
    yield


@pytest.mark.parametrize("variant", TC)
def test_tc_matches_reference_run_n9(variant):
    d, meta = load("cs7_l0_n9")
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    ev.set_kernel(variant)
    u0 = to_mesh_order(d["u0"], perm)
    r = ev.rhs(u0, 0.0)
    assert rel_l2(r[perm], d["r0"]) <= RTOL_RHS
    assert np.abs(r[perm] - d["r0"]).max() <= 1e-11 * np.abs(d["r0"]).max()
    u = ev.rk4_steps_host(u0, 0.0, meta["dt"], meta["steps"])
    assert rel_l2(u[perm], d["u_final"]) <= RTOL_RK4


@pytest.mark.parametrize("variant", TC)
def test_tc_benchmark_order_level2_matches_reference(variant):
    d, meta = load(BIG_CASE)
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    u0 = to_mesh_order(big_case_u0(d, meta), perm)
    ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    ev.set_kernel(variant)
    sel = d["sel"]
    r = ev.rhs(u0, 0.0)[perm]
    assert rel_l2(r[sel], d["r0_sel"]) <= RTOL_RHS
    ev.set_state(u0)
    ev.rk4_steps(0.0, meta["dt"], meta["steps"])
    u = ev.get_state()[perm]
    assert rel_l2(u[sel], d["u_final_sel"]) <= RTOL_RK4


@pytest.mark.parametrize("variant", TC)
@pytest.mark.parametrize("numflux", ["LLF", "upwind"])
def test_tc_outgoing_pulses_vs_oracle(variant, numflux):
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=9, luni=1, cs_dc=1.0, cs_r0fac=20.0)
    u = gaussian_pulses(m.coords(), seed=91, rmin=1.0, rmax=6.0)
    u += 1e-3 * np.random.default_rng(9).standard_normal(u.shape)
    o = oracle_for(m, bc=1, numflux=numflux)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_numflux(numflux)
    ev.set_kernel(variant)
    r, ro = ev.rhs(u, 0.0), o.rhs(u, 0.0)
    assert rel_l2(r, ro) <= RTOL_RHS
    dt = 0.02 / 81
    assert rel_l2(ev.rk4_steps_host(u, 0.0, dt, 3), o.rk4(u, dt, 3)) <= RTOL_RK4


def test_tc_periodic_box_cartesian_vs_oracle():
    m = ng.Mesh.build(ng.MESH_BOX, n=9, luni=1, xc=(PI, PI, PI), box_dout=PI, periodic=True)
    u = np.random.default_rng(3).standard_normal((m.nelem, 5, m.np))
    o = oracle_for(m, bc=1, period=2 * PI)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_kernel("tc")
    assert rel_l2(ev.rhs(u, 0.0), o.rhs(u, 0.0)) <= RTOL_RHS
    dt = 0.25 * (2 * PI / 2) / 64
    assert rel_l2(ev.rk4_steps_host(u, 0.0, dt, 2), o.rk4(u, dt, 2)) <= RTOL_RK4


def _per_element_err(r, ro):
    """max over elements of max|r - ro| / max|ro| inside the element"""
    num = np.abs(r - ro).reshape(r.shape[0], -1).max(1)
    den = np.abs(ro).reshape(r.shape[0], -1).max(1)
    return float((num / np.maximum(den, 1e-300)).max())


def test_tc_dynamic_range_across_and_inside_elements():
    """Elements scaled by factors 10^-150 .. 10^150 (the grid follows each
    element's field), inside elements values spread over 30 orders of
    magnitude, and the whole state near either end of the FP64 range: per
    element the error stays within 1e-12 of the element's largest |r| (the
    bound of block fixed point: a few units of 2^-53 of the element's
    largest value times max |D_i.|)."""
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=9, luni=0, cs_dc=1.0, cs_r0fac=20.0)
    rng = np.random.default_rng(17)
    u = rng.standard_normal((m.nelem, 5, m.np))
    u *= 10.0 ** rng.uniform(-15, 15, size=u.shape)  # inside elements
    scale = 10.0 ** rng.uniform(-150, 150, size=(m.nelem, 1, 1))
    o = oracle_for(m, bc=1)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_kernel("tc")
    for s in (1.0, 1e-280, 1e280, scale):
        us = u * s
        r, ro = ev.rhs(us, 0.0), o.rhs(us, 0.0)
        assert np.isfinite(r).all()
        if np.ndim(s) == 0:
            assert _per_element_err(r, ro) <= 1e-12, s
        else:
            # faces couple elements of different scales: compare against the
            # FP64 variant per element relative to the element's own |r|
            ev2 = ng.Evolution(m, ng.BC_OUTGOING)
            ev2.set_kernel("eo")
            assert _per_element_err(r, ev2.rhs(us, 0.0)) <= 1e-12
            ev2.close()


def test_tc_zero_and_nan_fields():
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=9, luni=0, cs_dc=1.0, cs_r0fac=20.0)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_kernel("tc")
    z = np.zeros((m.nelem, 5, m.np))
    assert np.array_equal(ev.rhs(z, 0.0), z)
    # one field of one element zero, the rest random: the zero field adds exact zeros
    u = np.random.default_rng(1).standard_normal(z.shape)
    u[3, 2] = 0.0
    o = oracle_for(m, bc=1)
    assert rel_l2(ev.rhs(u, 0.0), o.rhs(u, 0.0)) <= RTOL_RHS
    # a NaN in an element's field gives NaN in that element's RHS
    u[5, 1, 100] = np.nan
    r = ev.rhs(u, 0.0)
    assert np.isnan(r[5]).any()
    far = [e for e in range(m.nelem) if e != 5 and e not in m.faces()[0][5]]
    assert np.isfinite(r[far]).all()


def test_tc_bitwise_deterministic_and_round_trip():
    """Two evaluations are bitwise equal, and the streamed host round trip
    (element lists, chunked last stage) equals resident stepping bit for bit."""
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=9, luni=1, cs_dc=1.0, cs_r0fac=20.0)
    u = gaussian_pulses(m.coords(), seed=5, rmin=1.0, rmax=6.0)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_kernel("tc")
    assert np.array_equal(ev.rhs(u, 0.0), ev.rhs(u, 0.0))
    got = ev.rk4_steps_host(u, 0.0, 0.001, 3)
    ev.set_state(u)
    ev.rk4_steps(0.0, 0.001, 3)
    assert np.array_equal(got, ev.get_state())


def test_tc_mixed_mesh_vs_oracle():
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=9, luni=0, cs_dc=1.0, cs_r0fac=20.0, fv=[0, 3])
    u = gaussian_pulses(m.coords(), seed=12, rmin=1.0, rmax=6.0)
    u += 1e-2 * np.random.default_rng(12).standard_normal(u.shape)
    rec, ex = "WENOm5_2", "dnfn_extrap1"
    o = oracle_for(m, bc=1, fv_rec=rec, fv_extrap=ex)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_fv(rec, ex)
    ev.set_kernel("tc")
    ev.set_kernel("fvx")
    assert rel_l2(ev.rhs(u, 0.0), o.rhs(u, 0.0)) <= RTOL_RHS
    assert rel_l2(ev.rk4_steps_host(u, 0.0, 0.002, 2), o.rk4(u, 0.002, 2)) <= RTOL_RK4


def test_tc_nonconforming_faces_vs_oracle():
    """Patches 0 and 3 one level finer (amr_hrefine_p): the traces of the
    non-conforming faces reach the tensor-core kernel through the interface
    slots, as they reach the FP64 variants."""
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=9, luni=1, cs_dc=1.0, cs_r0fac=20.0,
                      hrefine=(0, 3))
    u = gaussian_pulses(m.coords(), seed=33, rmin=1.0, rmax=4.0)
    u += 1e-3 * np.random.default_rng(33).standard_normal(u.shape)
    o = oracle_for(m, bc=1)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_kernel("tc")
    assert rel_l2(ev.rhs(u, 0.0), o.rhs(u, 0.0)) <= RTOL_RHS
    dt = 0.001
    assert rel_l2(ev.rk4_steps_host(u, 0.0, dt, 3), o.rk4(u, dt, 3)) <= RTOL_RK4


@pytest.mark.parametrize("method", ["Euler", "sspRK3"])
def test_tc_other_integrators_vs_oracle(method):
    """The Euler and sspRK3 epilogue modes of the tensor-core kernel."""
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=9, luni=0, cs_dc=1.0, cs_r0fac=20.0)
    u = gaussian_pulses(m.coords(), seed=8, rmin=1.0, rmax=4.0)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_kernel("tc")
    ev.set_evolve_method(method)
    dt = 0.001
    got = ev.evolve_steps_host(u, 0.0, dt, 4)
    want = oracle_for(m, bc=1).evolve(u, dt, 4, method=method)
    assert rel_l2(got, want) <= RTOL_RK4


@pytest.mark.parametrize("variant", ["tc:1:128", "tc:1:256"])
@pytest.mark.parametrize("n", [7, 8])
def test_tc_orders_7_8_outgoing_vs_oracle(n, variant):
    """The tensor-core kernel at 7 and 8 points per direction (3 tiles and
    the line left over; 4 tiles)."""
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=n, luni=1, cs_dc=1.0, cs_r0fac=20.0)
    u = gaussian_pulses(m.coords(), seed=70 + n, rmin=1.0, rmax=6.0)
    u += 1e-3 * np.random.default_rng(n).standard_normal(u.shape)
    o = oracle_for(m, bc=1)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_kernel(variant)
    assert rel_l2(ev.rhs(u, 0.0), o.rhs(u, 0.0)) <= RTOL_RHS
    dt = 0.02 / n ** 2
    assert rel_l2(ev.rk4_steps_host(u, 0.0, dt, 3), o.rk4(u, dt, 3)) <= RTOL_RK4
    ev.set_state(u)
    ev.rk4_steps(0.0, dt, 3)
    assert np.array_equal(ev.rk4_steps_host(u, 0.0, dt, 3), ev.get_state())


@pytest.mark.parametrize("n", [7, 8])
def test_tc_orders_7_8_periodic_box_vs_oracle(n):
    m = ng.Mesh.build(ng.MESH_BOX, n=n, luni=1, xc=(PI, PI, PI), box_dout=PI, periodic=True)
    u = np.random.default_rng(n).standard_normal((m.nelem, 5, m.np))
    o = oracle_for(m, bc=1, period=2 * PI)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_kernel("tc")
    assert rel_l2(ev.rhs(u, 0.0), o.rhs(u, 0.0)) <= RTOL_RHS


def test_tc_order7_mixed_mesh_matches_reference():
    """The reference's own run of a mixed mesh at 7 points (inner cube finite
    volume, shells DG), with the tensor-core kernel for the DG elements."""
    d, meta = load("mixcs7_l0_n7_w5dnfn")
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    ev.set_fv(meta["fv"]["rec"], meta["fv"]["extrap"])
    ev.set_kernel("tc")
    ev.set_kernel("fvx")
    r = ev.rhs(to_mesh_order(d["u0"], perm), 0.0)
    assert rel_l2(r[perm], d["r0"]) <= RTOL_RHS
    u = ev.rk4_steps_host(to_mesh_order(d["u0"], perm), 0.0, meta["dt"], meta["steps"])
    assert rel_l2(u[perm], d["u_final"]) <= RTOL_RK4


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()


@pytest.mark.parametrize("n,kind", [(9, "cs7"), (9, "cs7h"), (8, "cs7"), (7, "cs7"), (8, "box")])
def test_tcvjp_matches_the_fp64_transposed_kernel(n, kind):
    """The tensor-core transposed stage ("tcvjp", the default at n = 7..9)
    against the FP64 one ("vjp"): the RHS VJP and an RK4-step VJP within
    1e-12, on curvilinear, non-conforming and Cartesian meshes."""
    import torch
    if kind == "box":
        m = ng.Mesh.build(ng.MESH_BOX, n=n, luni=1, xc=(PI, PI, PI), box_dout=PI, periodic=True)
    else:
        m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=n, luni=0 if kind == "cs7h" else 1, cs_dc=1.0,
                          cs_r0fac=20.0, hrefine=(0,) if kind == "cs7h" else ())
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    rb = np.random.default_rng(n).standard_normal(ev.shape)
    outs = {}
    for k in ("tcvjp", "vjp"):
        ev.set_kernel(k)
        w = torch.zeros(ev.size, dtype=torch.float64, device="cuda")
        ev.rhs_vjp_device(_dev(rb).data_ptr(), w.data_ptr())
        ub = _dev(rb)
        ev.rk4_step_vjp_device(ub.data_ptr(), 0.0, 0.01 / n)
        torch.cuda.synchronize()
        outs[k] = (w.cpu().numpy(), ub.cpu().numpy())
    assert rel_l2(outs["tcvjp"][0], outs["vjp"][0]) <= RTOL_RHS
    assert rel_l2(outs["tcvjp"][1], outs["vjp"][1]) <= RTOL_RK4
