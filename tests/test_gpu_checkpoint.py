"""A GPU run restarts from the reference's checkpoint and writes its own
(nmg_checkpoint_read / nmg_checkpoint_write on a context)."""
import numpy as np
import pytest

import nmesh_gb300 as ng
from helpers import (GOLDEN, RTOL_RK4, build_mesh, load, oracle_for, perm_to_mesh, rel_l2,
                     to_mesh_order)

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["ckpt_box_l1_n4", "ckpt_cs7_l1_n3"])
def test_restart_from_reference_checkpoint(case, tmp_path):
    d, meta = load(case)
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    ref = f"{GOLDEN}/{case}_variables.bin"
    ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    ev.checkpoint_read(ref)
    u1 = to_mesh_order(d["u_final"], perm)
    assert np.array_equal(ev.get_state(), u1)
    # the resident state written back is the reference's file, byte for byte
    ev.checkpoint_write(tmp_path / "same.bin")
    assert (tmp_path / "same.bin").read_bytes() == open(ref, "rb").read()
    # continue the run on the GPU: step 2 from the restart, against the oracle
    t1, dt = meta["dt"], meta["dt"]
    ev.rk4_step(t1, dt)
    o = oracle_for(m, bc=0, k=meta["k"])
    want = o.rk4(u1, dt, 1, t=t1)
    got = ev.get_state()
    assert rel_l2(got, want) <= RTOL_RK4
    ev.checkpoint_write(tmp_path / "next.bin")
    assert np.array_equal(ng.checkpoint_read_host(m, tmp_path / "next.bin"), got)


def test_restarts_every_step_match_an_uninterrupted_run(tmp_path):
    """The reference's checkpoint test: a run written to a checkpoint every
    iteration and restarted from it each time matches the uninterrupted run
    (here bit for bit: the file holds the doubles exactly)."""
    d, meta = load("ckpt_cs7_l1_n3")
    m = build_mesh(meta)
    u0 = to_mesh_order(d["u0"], perm_to_mesh(m, d))
    dt, nsteps = meta["dt"], 4
    a = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    a.set_kernel("eo")
    a.set_state(u0)
    for s in range(nsteps):
        a.rk4_step(s * dt, dt)
    ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    ev.set_kernel("eo")
    ev.set_state(u0)
    for s in range(nsteps):
        ev.rk4_step(s * dt, dt)
        ev.checkpoint_write(tmp_path / "variables.bin")
        ev.close()
        ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
        ev.set_kernel("eo")
        ev.checkpoint_read(tmp_path / "variables.bin")
    assert np.array_equal(ev.get_state(), a.get_state())
