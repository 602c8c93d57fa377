"""Generate the golden fixtures in tests/golden/ by running the reference
itself (oracle/_ref/nmesh, built from the reference sources by
oracle/ref/Makefile) with the dump add-on module.

Run in a container where the reference sources exist:
    make -C oracle/ref -j8 && python tests/golden/make_golden.py

Each case is one reference run of scalarwave1 with LLF flux and RK4:
the dump module perturbs the plane-wave initial data with seeded noise,
dumps u0 and r0 = RHS(u0, 0) (reference evolve_setrhs_mesh), the run takes
`steps` RK4 steps, and the final u is dumped.  The fixture stores the
element descriptors (patch, n, bbox), the geometry the reference computed
(x, dXdx, sqrtgdiag), u0, r0 and u_final, plus the case parameters.
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle.refdump import read_dump  # noqa: E402

PI = 3.141592653589793

# name -> (mesh parameters, n, luni, k, dt, steps, perturbation, seed)
CASES = {
    # one Cartesian box patch [0, 2 pi]^3 (the periodic-cube workload's
    # geometry; the reference itself has exact plane-wave outer faces)
    "box_l1_n5": dict(mesh="box", n=5, luni=1, k=(1.0, 1.0, 1.0),
                      dt=0.25 * (2 * PI / 2) / 16, steps=3, eps=0.01, seed=7),
    "box_l2_n4": dict(mesh="box", n=4, luni=2, k=(1.0, -0.5, 0.25),
                      dt=0.01, steps=2, eps=0.05, seed=11),
    # inner cube [-1,1]^3 plus 6 cubed-sphere patches out to r = 20
    "cs7_l0_n9": dict(mesh="cs7", n=9, luni=0, k=(0.3, -0.2, 0.1),
                      dt=0.002, steps=2, eps=0.01, seed=3),
    "cs7_l1_n5": dict(mesh="cs7", n=5, luni=1, k=(0.3, -0.2, 0.1),
                      dt=0.004, steps=2, eps=0.02, seed=5),
    "cs7_l1_n4": dict(mesh="cs7", n=4, luni=1, k=(0.25, 0.15, -0.3),
                      dt=0.004, steps=2, eps=0.02, seed=9),
    # finite-volume elements everywhere: uniform points (amr_uniform_p),
    # fin. vol. mode (amr_fv_p), WENO reconstruction at the midpoints
    "fvbox_l1_n7_w5no": dict(mesh="box", n=7, luni=1, k=(1.0, 1.0, 1.0),
                             dt=0.005, steps=2, eps=0.05, seed=21,
                             fv=dict(rec="WENOm5_2", extrap="no")),
    "fvbox_l1_n7_w5dnfn": dict(mesh="box", n=7, luni=1, k=(1.0, -0.5, 0.25),
                               dt=0.005, steps=2, eps=0.05, seed=22,
                               fv=dict(rec="WENOm5_2", extrap="dnfn_extrap1")),
    "fvbox_l2_n5_w3dnfn": dict(mesh="box", n=5, luni=2, k=(0.5, 1.0, -1.0),
                               dt=0.004, steps=2, eps=0.1, seed=23,
                               fv=dict(rec="WENOm3_2", extrap="dnfn_extrap1")),
    "fvbox_l0_n13_w5dnfn": dict(mesh="box", n=13, luni=0, k=(1.0, 0.5, 0.25),
                                dt=0.004, steps=2, eps=0.3, seed=24,
                                fv=dict(rec="WENOm5_2", extrap="dnfn_extrap1")),
    "fvcs7_l0_n7_w5dnfn": dict(mesh="cs7", n=7, luni=0, k=(0.3, -0.2, 0.1),
                               dt=0.002, steps=2, eps=0.02, seed=25,
                               fv=dict(rec="WENOm5_2", extrap="dnfn_extrap1")),
    "fvcs7_l0_n6_w5no": dict(mesh="cs7", n=6, luni=0, k=(0.25, 0.15, -0.3),
                             dt=0.002, steps=2, eps=0.02, seed=26,
                             fv=dict(rec="WENOm5_2", extrap="no")),
    # mixed meshes: the inner cube (patch 0) finite-volume, the six
    # cubed-sphere patches DG; face traces across the DG / FV interface are
    # interpolated (Lagrange from DG, piecewise linear from FV)
    "mixcs7_l0_n7_w5dnfn": dict(mesh="cs7", n=7, luni=0, k=(0.3, -0.2, 0.1),
                                dt=0.002, steps=2, eps=0.02, seed=27,
                                fv=dict(rec="WENOm5_2", extrap="dnfn_extrap1",
                                        patches="0")),
    "mixcs7_l1_n5_w3no": dict(mesh="cs7", n=5, luni=1, k=(0.25, 0.15, -0.3),
                              dt=0.002, steps=2, eps=0.02, seed=28,
                              fv=dict(rec="WENOm3_2", extrap="no", patches="0")),
    # DG data with Persson's modal indicator of u0 (every element, field)
    "trbl_cs7_l1_n6": dict(mesh="cs7", n=6, luni=1, k=(0.9, -0.7, 0.5),
                           dt=0.002, steps=1, eps=0.05, seed=29, persson=True),
    # 0d norms (volume integrals, extrema) of u0 on DG and on mixed meshes
    "norms_cs7_l1_n5": dict(mesh="cs7", n=5, luni=1, k=(0.3, -0.2, 0.1),
                            dt=0.002, steps=1, eps=0.05, seed=30, norms=True),
    "norms_mixcs7_l0_n6": dict(mesh="cs7", n=6, luni=0, k=(0.3, 0.2, -0.1),
                               dt=0.002, steps=1, eps=0.05, seed=31, norms=True,
                               fv=dict(rec="WENOm3_2", extrap="dnfn_extrap1",
                                       patches="0")),
    # the reference's default numerical flux (scalarwave1_numflux = upwind)
    "upw_cs7_l1_n5": dict(mesh="cs7", n=5, luni=1, k=(0.3, -0.2, 0.1),
                          dt=0.004, steps=2, eps=0.02, seed=32, numflux="upwind"),
    "upw_box_l1_n6": dict(mesh="box", n=6, luni=1, k=(1.0, -0.5, 0.25),
                          dt=0.01, steps=2, eps=0.05, seed=33, numflux="upwind"),
    "upw_mixcs7_l0_n7_w5dnfn": dict(mesh="cs7", n=7, luni=0, k=(0.3, -0.2, 0.1),
                                    dt=0.002, steps=2, eps=0.02, seed=34, numflux="upwind",
                                    fv=dict(rec="WENOm5_2", extrap="dnfn_extrap1",
                                            patches="0")),
    "upw_fvbox_l1_n7_w5no": dict(mesh="box", n=7, luni=1, k=(1.0, 1.0, 1.0),
                                 dt=0.005, steps=2, eps=0.05, seed=35, numflux="upwind",
                                 fv=dict(rec="WENOm5_2", extrap="no")),
    # the reference's own checkpoint of the final state (variables.bin)
    "ckpt_box_l1_n4": dict(mesh="box", n=4, luni=1, k=(1.0, -0.5, 0.25),
                           dt=0.01, steps=1, eps=0.01, seed=36, checkpoint=True),
    "ckpt_cs7_l1_n3": dict(mesh="cs7", n=3, luni=1, k=(0.3, -0.2, 0.1),
                           dt=0.002, steps=1, eps=0.01, seed=37, checkpoint=True),
    # WENO-Z reconstruction inside, WENOm3_2 near the ends (fv_rec = WENOmZ_2,
    # the reconstruction of the reference's own mixed DG/FV test parfile)
    "fvcs7_l0_n7_wZdnfn": dict(mesh="cs7", n=7, luni=0, k=(0.3, -0.2, 0.1),
                               dt=0.002, steps=2, eps=0.05, seed=42,
                               fv=dict(rec="WENOmZ_2", extrap="dnfn_extrap1")),
    "fvbox_l1_n8_wZno": dict(mesh="box", n=8, luni=1, k=(1.0, -0.5, 0.25),
                             dt=0.004, steps=2, eps=0.1, seed=43,
                             fv=dict(rec="WENOmZ_2", extrap="no")),
    "mixcs7_l1_n6_wZdnfn": dict(mesh="cs7", n=6, luni=1, k=(0.25, 0.15, -0.3),
                                dt=0.002, steps=2, eps=0.02, seed=44,
                                fv=dict(rec="WENOmZ_2", extrap="dnfn_extrap1",
                                        patches="0 2 4")),
    # the reference's other time integrators (evolve_method = sspRK3 / Euler);
    # the mixed case follows its own FV-DG test parfile (FV patches 0 2 4,
    # WENOmZ_2, sspRK3) with one n for all directions
    "ssp3_cs7_l1_n5": dict(mesh="cs7", n=5, luni=1, k=(0.3, -0.2, 0.1),
                           dt=0.002, steps=3, eps=0.02, seed=45, method="sspRK3"),
    "eul_box_l1_n5": dict(mesh="box", n=5, luni=1, k=(1.0, -0.5, 0.25),
                          dt=0.002, steps=3, eps=0.02, seed=46, method="Euler"),
    "ssp3_mixcs7_l1_n6_wZdnfn": dict(mesh="cs7", n=6, luni=1, k=(0.8, -0.5, 0.33166247903554),
                                     dt=0.002, steps=3, eps=0.02, seed=47, method="sspRK3",
                                     fv=dict(rec="WENOmZ_2", extrap="dnfn_extrap1",
                                             patches="0 2 4")),
    # fv_surface_interp = parabolic (as in the reference's FV-DG test parfile)
    "mixcs7_l0_n7_w5parab": dict(mesh="cs7", n=7, luni=0, k=(0.3, -0.2, 0.1),
                                 dt=0.002, steps=2, eps=0.02, seed=48,
                                 fv=dict(rec="WENOm5_2", extrap="dnfn_extrap1",
                                         patches="0", surf="parabolic")),
    "ssp3_mixcs7_l0_n7_wZparab": dict(mesh="cs7", n=7, luni=0, k=(0.8, -0.5, 0.33166247903554),
                                      dt=0.002, steps=3, eps=0.02, seed=49, method="sspRK3",
                                      fv=dict(rec="WENOmZ_2", extrap="dnfn_extrap1",
                                              patches="0 2 4", surf="parabolic")),
    # coordinates_midpoint_data = yes: FV flux factors and normals at the
    # midpoints (the reference's FV-DG test parfile sets it)
    "fvcs7_l0_n7_w5dnfn_mid": dict(mesh="cs7", n=7, luni=0, k=(0.3, -0.2, 0.1),
                                   dt=0.002, steps=2, eps=0.05, seed=50,
                                   fv=dict(rec="WENOm5_2", extrap="dnfn_extrap1", mid=True)),
    "fvcs7_l1_n6_w3no_mid": dict(mesh="cs7", n=6, luni=1, k=(0.25, 0.15, -0.3),
                                 dt=0.002, steps=2, eps=0.05, seed=51,
                                 fv=dict(rec="WENOm3_2", extrap="no", mid=True)),
    "ssp3_mixcs7_l0_n7_wZparab_mid": dict(mesh="cs7", n=7, luni=0,
                                          k=(0.8, -0.5, 0.33166247903554), dt=0.002, steps=3,
                                          eps=0.02, seed=52, method="sspRK3",
                                          fv=dict(rec="WENOmZ_2", extrap="dnfn_extrap1",
                                                  patches="0 2 4", surf="parabolic",
                                                  mid=True)),
    # dt = auto: the reference's dtfac * hmin (uniform_dtfac on FV elements)
    "dtauto_cs7_l1_n5": dict(mesh="cs7", n=5, luni=1, k=(0.3, -0.2, 0.1),
                             dt="auto", steps=1, eps=0.02, seed=53),
    "dtauto_box_l2_n6": dict(mesh="box", n=6, luni=2, k=(1.0, -0.5, 0.25),
                             dt="auto", steps=1, eps=0.02, seed=54),
    "dtauto_mixcs7_l0_n7": dict(mesh="cs7", n=7, luni=0, k=(0.3, -0.2, 0.1),
                                dt="auto", steps=1, eps=0.02, seed=55,
                                fv=dict(rec="WENOm5_2", extrap="dnfn_extrap1", patches="2")),
    # evolve_filter_all = yes: the exponential modal filter after every step
    "filt_cs7_l1_n6": dict(mesh="cs7", n=6, luni=1, k=(0.3, -0.2, 0.1),
                           dt=0.002, steps=3, eps=0.05, seed=56, filter=True),
    "filt_mixcs7_l0_n7": dict(mesh="cs7", n=7, luni=0, k=(0.3, -0.2, 0.1),
                              dt=0.002, steps=2, eps=0.05, seed=57, filter=True,
                              fv=dict(rec="WENOm5_2", extrap="dnfn_extrap1", patches="0")),
    # non-conforming faces: the listed patches refined one level further
    # (amr_hrefine_p), face traces interpolated across the level jump
    "nc_cs7_l0_n5_h0": dict(mesh="cs7", n=5, luni=0, k=(0.3, -0.2, 0.1),
                            dt=0.002, steps=2, eps=0.02, seed=38, hrefine="0"),
    "nc_cs7_l0_n4_h1": dict(mesh="cs7", n=4, luni=0, k=(0.25, 0.15, -0.3),
                            dt=0.002, steps=2, eps=0.02, seed=39, hrefine="1"),
    "nc_cs7_l1_n5_h02": dict(mesh="cs7", n=5, luni=1, k=(0.3, -0.2, 0.1),
                             dt=0.002, steps=2, eps=0.02, seed=40, hrefine="0 2"),
    "nc_upw_cs7_l0_n6_h35": dict(mesh="cs7", n=6, luni=0, k=(0.3, 0.2, -0.1),
                                 dt=0.002, steps=2, eps=0.02, seed=41, hrefine="3 5",
                                 numflux="upwind"),
    # non-conforming faces inside patches: nested-sphere refinement about
    # x = 0 (amr_hrefine_sphere_levels / _radius)
    "sph_box_l1_n5_s2r2": dict(mesh="box", n=5, luni=1, k=(1.0, -0.5, 0.25),
                               dt=0.002, steps=2, eps=0.02, seed=42, sphere=(2, 2)),
    "sph_box_l2_n4_s1r3": dict(mesh="box", n=4, luni=2, k=(0.5, 1.0, -1.0),
                               dt=0.002, steps=2, eps=0.02, seed=43, sphere=(1, 3)),
    "sph_cs7_l1_n4_s1r6": dict(mesh="cs7", n=4, luni=1, k=(0.3, -0.2, 0.1),
                               dt=0.002, steps=2, eps=0.02, seed=44, sphere=(1, 6)),
    # the MRS limiter (scalarwave1_limiter = MRS) with a small limiter_alpha
    # so that noisy elements are limited
    "lim_box_l1_n5_a0.01": dict(mesh="box", n=5, luni=1, k=(1.0, -0.5, 0.25),
                                dt=0.002, steps=3, eps=0.3, seed=45, limiter=0.01),
    "lim_cs7_l1_n4_a0.05": dict(mesh="cs7", n=4, luni=1, k=(0.3, -0.2, 0.1),
                                dt=0.002, steps=2, eps=0.3, seed=46, limiter=0.05),
    "lim_nc_cs7_l0_n5_h0_a0.02": dict(mesh="cs7", n=5, luni=0, k=(0.3, -0.2, 0.1),
                                      dt=0.002, steps=2, eps=0.3, seed=47, hrefine="0",
                                      limiter=0.02),
    # the minmodB limiter (scalarwave1_limiter = minmodB): bound alpha h,
    # slopes against beta/sqrt3 times the face neighbours' average jumps;
    # scaleBound = yes scales the bound by the neighbours' mean |average|
    "mmb_box_l1_n5_a0.05": dict(mesh="box", n=5, luni=1, k=(1.0, -0.5, 0.25),
                                dt=0.002, steps=3, eps=0.3, seed=48, limiter=0.05,
                                limname="minmodB"),
    "mmb_cs7_l1_n4_a0.2_b0.8": dict(mesh="cs7", n=4, luni=1, k=(0.3, -0.2, 0.1),
                                    dt=0.002, steps=2, eps=0.3, seed=49, limiter=0.2,
                                    limname="minmodB", beta=0.8),
    "mmb_nc_cs7_l0_n5_h0_a0.1_sb": dict(mesh="cs7", n=5, luni=0, k=(0.3, -0.2, 0.1),
                                        dt=0.002, steps=2, eps=0.3, seed=50, hrefine="0",
                                        limiter=0.1, limname="minmodB", scalebound=True),
    "mmb_mixcs7_l0_n7_w5dnfn_a0.1": dict(mesh="cs7", n=7, luni=0, k=(0.3, -0.2, 0.1),
                                         dt=0.002, steps=2, eps=0.3, seed=51, limiter=0.1,
                                         limname="minmodB",
                                         fv=dict(rec="WENOm5_2", extrap="dnfn_extrap1",
                                                 patches="0")),
    # the benchmark's mesh family and order at level 2 (448 elements of 9^3
    # LGL nodes, 1.6 M DOF) with the benchmark's dt formula at that level,
    # 0.25 (2 / 2^2) / 8^2, and 10 steps.  amp = 0: the initial data is the
    # seeded noise alone, which the tests regenerate bit for bit
    # (helpers.dump_noise), so u0 is not stored; r0 and u_final are kept
    # for every `keep`-th element (reference order) plus their full norms
    "cs7_l2_n9_noise": dict(mesh="cs7", n=9, luni=2, k=(0.3, -0.2, 0.1),
                            dt=0.001953125, steps=10, eps=0.01, seed=60, amp=0.0, keep=14),
}


def parfile(case, prefix):
    c = CASES[case]
    lines = [
        "physics = scalarwave1 nmgdump",
        f"evolve_method = {c.get('method', 'RK4')}",
        f"dt = {c['dt'] if c['dt'] == 'auto' else repr(c['dt'])}",
        f"iterations = {c['steps']}",
        f"amr_luni = {c['luni']}",
        f"amr_n0 = {c['n']}", f"amr_n1 = {c['n']}", f"amr_n2 = {c['n']}",
        "scalarwave1_k = %r %r %r" % tuple(c["k"]),
        f"scalarwave1_numflux = {c.get('numflux', 'LLF')}",
        f"nmgdump_prefix = {prefix}",
        f"nmgdump_amp = {c.get('amp', 1.0)!r}",
        f"nmgdump_perturb = {c['eps']!r}",
        f"nmgdump_seed = {c['seed']}",
        f"nmgdump_persson = {'yes' if c.get('persson') else 'no'}",
        f"nmgdump_norms = {'yes' if c.get('norms') else 'no'}",
        "logfile_creation = no",
        "sysmon_hours = -1",
    ]
    if c["mesh"] == "box":
        lines += ["amr_mesh_type = 1 BoxMesh",
                  f"amr_mesh_xc = {PI!r} {PI!r} {PI!r}",
                  f"amr_BoxMesh_dout = {PI!r}"]
        pats = "0"
    else:
        lines += ["amr_mesh_type = 7 CubedSpheres",
                  "amr_CubedSphere_dc = 1", "amr_CubedSphere_r0fac = 20"]
        pats = "0 1 2 3 4 5 6"
    if c.get("checkpoint"):
        lines += ["checkpoint = yes"]
    if c.get("filter"):
        lines += ["evolve_filter_all = yes"]
    if c.get("hrefine"):
        lines += [f"amr_hrefine_p = {c['hrefine']}"]
    if "limiter" in c:
        lines += [f"scalarwave1_limiter = {c.get('limname', 'MRS')}",
                  f"limiter_alpha = {c['limiter']!r}",
                  f"limiter_beta = {c.get('beta', 0.5)!r}",
                  f"limiter_scaleBound = {'yes' if c.get('scalebound') else 'no'}"]
    if c.get("sphere"):
        lines += [f"amr_hrefine_sphere_levels = {c['sphere'][0]}",
                  f"amr_hrefine_sphere_radius = {c['sphere'][1]}"]
    if "fv" in c:
        pats = c["fv"].get("patches", pats)
        lines += [f"amr_uniform_p = {pats}", f"amr_fv_p = {pats}",
                  f"fv_rec = {c['fv']['rec']}",
                  f"fv_divf_extrap = {c['fv']['extrap']}",
                  f"fv_surface_interp = {c['fv'].get('surf', 'linear')}",
                  f"coordinates_midpoint_data = {'yes' if c['fv'].get('mid') else 'no'}"]
    return "\n".join(lines) + "\n"


def run_case(case, exe, outdir):
    with tempfile.TemporaryDirectory() as tmp:
        prefix = os.path.join(tmp, "d")
        par = os.path.join(tmp, case + ".par")
        with open(par, "w") as fp:
            fp.write(parfile(case, prefix))
        env = dict(os.environ, OMP_NUM_THREADS="1")
        res = subprocess.run([exe, par], cwd=tmp, env=env,
                             capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"{case}: reference failed\n{res.stdout[-3000:]}")
        d0 = read_dump(prefix + "_rhs.bin", True)
        d1 = read_dump(prefix + "_final.bin", False)
        pers = None
        if CASES[case].get("persson"):
            raw = np.fromfile(prefix + "_persson.bin", dtype="<i4", count=1)
            pers = np.fromfile(prefix + "_persson.bin", dtype="<f8", offset=4)
            pers = pers.reshape(int(raw[0]), 5)
        dt_ref = np.fromfile(prefix + "_dt.bin", dtype="<f8")
        norms = None
        if CASES[case].get("norms"):
            norms = np.fromfile(prefix + "_norms.bin", dtype="<f8")
        if CASES[case].get("checkpoint"):
            import shutil
            src = os.path.join(tmp, case, "checkpoint", "variables.bin")
            shutil.copyfile(src, os.path.join(outdir, case + "_variables.bin"))
    c = CASES[case]
    meta = dict(case=case, **{k: v for k, v in c.items()})
    extra = {}
    if "fv" in c:   # fin.-vol. cases also keep the flag and det(dXb/dx)
        extra = dict(use_fv=d0["use_fv"], det_dXbdx=d0["det_dXbdx"])
    if pers is not None:
        extra["persson"] = pers
    if norms is not None:      # Vol, then per field VolInt, Int v^2, min, max
        extra["norms"] = norms
    if c["dt"] == "auto":      # the reference's automatic dt of the run
        extra["dt_ref"] = dt_ref
    if "keep" in c:   # slim fixture: u0 is regenerated, r0 / u_final sampled
        sel = np.arange(0, len(d0["pat"]), c["keep"])
        np.savez_compressed(
            os.path.join(outdir, case + ".npz"),
            meta=json.dumps(meta), pat=d0["pat"], n=d0["n"], bbox=d0["bbox"], sel=sel,
            r0_sel=d0["r"][sel], u_final_sel=d1["u"][sel],
            r0_norm=np.linalg.norm(d0["r"].ravel()),
            u_final_norm=np.linalg.norm(d1["u"].ravel()),
            u0_sum=np.sum(d0["u"]))
        print(f"{case}: {len(d0['pat'])} elements, {len(sel)} kept")
        return
    np.savez_compressed(
        os.path.join(outdir, case + ".npz"),
        meta=json.dumps(meta), pat=d0["pat"], n=d0["n"], bbox=d0["bbox"],
        x=d0["x"], dXdx=d0["dXdx"], sqrtgdiag=d0["sqrtgdiag"],
        u0=d0["u"], r0=d0["r"], u_final=d1["u"], **extra)
    print(f"{case}: {len(d0['pat'])} elements written")


def main():
    exe = os.path.join(ROOT, "oracle", "_ref", "nmesh")
    if not os.path.exists(exe):
        raise SystemExit("build the reference first: make -C oracle/ref")
    cases = sys.argv[1:] or list(CASES)
    for case in cases:
        run_case(case, exe, HERE)


if __name__ == "__main__":
    main()
