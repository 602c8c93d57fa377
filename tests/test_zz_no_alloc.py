"""The allocation-free RK4 step (nmg_rk4_step_noalloc), for callers that
cannot call cudaMalloc while they step (their device memory comes from their
own pool or a framework allocator, or their footprint must not grow in the
middle of a run): its stage buffers live in a static device array instead of
context-owned allocations.

Each case takes the fixture's steps through the C ABI, one call per step,
every call after the first finding the previous call's stale contents in the
shared scratch array, and compares every step with the regular entry point
(nmg_rk4_step) and the last one with the reference's own run of the same
steps (the fixture's u_final).  The cases cover conforming DG meshes (at
n = 9 with the tensor-core stage kernel, set on both contexts), a mixed
DG / finite-volume mesh and a mesh with non-conforming faces (both with the
untuned default kernels), the MRS and minmodB limiters and the exponential
filter.
This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

import nmesh_gb300 as ng
from helpers import (RTOL_RK4, build_mesh, limiter_kwargs, load, perm_to_mesh, rel_l2,
                     to_mesh_order)

pytestmark = pytest.mark.gpu

CASES = ["cs7_l1_n5", "cs7_l0_n9", "mixcs7_l0_n7_w5dnfn", "nc_cs7_l0_n5_h0",
         "lim_cs7_l1_n4_a0.05", "mmb_cs7_l1_n4_a0.2_b0.8", "filt_cs7_l1_n6"]


def _noalloc(ev, t, dt, u_in, u_out):
    return ng.lib().nmg_rk4_step_noalloc(ev._h, ctypes.c_double(t), ctypes.c_double(dt),
                                         ctypes.c_void_p(u_in.data_ptr()),
                                         ctypes.c_void_p(u_out.data_ptr()))


def _context(m, meta):
    ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    if m.n == 9:
        ev.set_kernel("tc")
    if "fv" in meta:
        ev.set_fv(meta["fv"]["rec"], meta["fv"]["extrap"])
    if "limiter" in meta:
        ev.set_limiter(**limiter_kwargs(meta))
    if meta.get("filter"):
        ev.set_filter(True)
    return ev


@pytest.mark.parametrize("case", CASES)
def test_noalloc_steps_match_regular_steps_and_reference(cuda_ok, case):
    import torch
    d, meta = load(case)
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    u0 = to_mesh_order(d["u0"], perm)
    dt, ns = meta["dt"], meta["steps"]
    assert ns >= 2

    # regular entry point: state resident in the context
    ref = _context(m, meta)
    ref.set_state(u0)
    regular = []
    for s in range(ns):
        ref.rk4_step(s * dt, dt)
        regular.append(ref.get_state())

    # allocation-free entry point: caller-owned input and output buffers,
    # used in turn as input and output
    ev = _context(m, meta)
    a = torch.from_numpy(u0.copy()).cuda()
    b = torch.empty_like(a)
    torch.cuda.synchronize()
    for s in range(ns):
        assert _noalloc(ev, s * dt, dt, a, b) == 0, ng.lib().nmg_last_error(ev._h)
        got = b.cpu().numpy()
        assert rel_l2(got, regular[s]) <= RTOL_RK4, f"step {s + 1}"
        a, b = b, a
    # the reference's own run of the same steps
    assert rel_l2(got[perm], d["u_final"]) <= RTOL_RK4


def test_noalloc_rejects_bad_buffers(cuda_ok):
    import torch
    d, meta = load("box_l1_n5")
    m = build_mesh(meta)
    ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    a = torch.zeros(ev.size, dtype=torch.float64, device="cuda")
    assert _noalloc(ev, 0.0, 0.01, a, a) == 1          # aliasing in/out
    assert b"distinct" in ng.lib().nmg_last_error(ev._h)
    assert ng.lib().nmg_rk4_step_noalloc(ev._h, 0.0, 0.01, None, None) == 1


def test_noalloc_rejects_states_above_the_limit(cuda_ok):
    import torch
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=9, luni=3, cs_dc=1.0, cs_r0fac=20.0)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    assert ev.size > 2097152
    a = torch.zeros(16, dtype=torch.float64, device="cuda")
    b = torch.zeros(16, dtype=torch.float64, device="cuda")
    assert _noalloc(ev, 0.0, 0.001, a, b) == 1
    assert b"NMG_NOALLOC_MAX_STATE" in ng.lib().nmg_last_error(ev._h)
    np.testing.assert_equal(a.cpu().numpy(), 0.0)
