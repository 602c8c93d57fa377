"""The allocation-free RK4 step (nmg_rk4_step_noalloc), for callers that
cannot call cudaMalloc while they step: its stage buffers live in a static
device array instead of context-owned allocations.  Checked through the C
ABI against the regular entry point (nmg_rk4_step) on two calls in a row,
the second one finding the first one's stale contents in the shared
scratch array.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

import nmesh_gb300 as ng
from helpers import RTOL_RK4, build_mesh, load, perm_to_mesh, rel_l2, to_mesh_order

pytestmark = pytest.mark.gpu


def _noalloc(ev, t, dt, u_in, u_out):
    return ng.lib().nmg_rk4_step_noalloc(ev._h, ctypes.c_double(t), ctypes.c_double(dt),
                                         ctypes.c_void_p(u_in.data_ptr()),
                                         ctypes.c_void_p(u_out.data_ptr()))


def test_noalloc_step_matches_regular_step(cuda_ok):
    import torch
    d, meta = load("cs7_l1_n5")
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    u0 = to_mesh_order(d["u0"], perm)
    dt = meta["dt"]

    # regular entry point: state resident in the context
    ref = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    ref.set_kernel("eo")
    ref.set_state(u0)
    ref.rk4_step(0.0, dt)
    r1 = ref.get_state()
    ref.rk4_step(dt, dt)
    r2 = ref.get_state()

    # allocation-free entry point: caller-owned input and output buffers
    ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    ev.set_kernel("eo")
    a = torch.from_numpy(u0.copy()).cuda()
    b = torch.empty_like(a)
    torch.cuda.synchronize()
    assert _noalloc(ev, 0.0, dt, a, b) == 0
    s1 = b.cpu().numpy()
    assert _noalloc(ev, dt, dt, b, a) == 0
    s2 = a.cpu().numpy()
    assert rel_l2(s1, r1) <= RTOL_RK4
    assert rel_l2(s2, r2) <= RTOL_RK4
    # one step of the reference's own run
    assert rel_l2(s1[perm], ev.rk4_steps_host(u0, 0.0, dt, 1)[perm]) <= RTOL_RK4


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
