"""Benchmark of the GB300-native nmesh evolution path.

Workload (the cubed-sphere configuration the headline metric is quoted on):
scalarwave1 (first-order wave, 5 FP64 fields), 7 CubedSpheres mesh (inner
cube [-1,1]^3 + 6 cubed-sphere patches out to r = 20), uniform level 4
(7 x 16^3 = 28672 elements), 9 LGL nodes per direction (N = 8), 104,509,440
DOF, seeded sum of 8 Gaussian pulses, outgoing-radiation outer boundary,
LLF flux, classic RK4.  A bench step is one RK4 step (4 fused RHS+update
stage kernels).  Every state buffer is 836 MB, far larger than the 129 MB
L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line on rank 0.  --impl reference times the CPU
implementation of the same path on the host cores (the oracle's C
restatement of the reference, pinned bit-exact to the reference itself).
Under torchrun every rank runs an independent replica (the path is
replicas-only on this pool); value = all ranks' DOF-stage updates divided by
the max over ranks of the timed region.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "FP64 DOF-updates/s per RK stage"
UNIT = "DOF-stage/s"
NFIELDS = 5


def workload_config(n, luni):
    E = 7 * 8 ** luni
    return {
        "workload": (f"scalarwave1 RK4, 7 CubedSpheres (cube dc=1 + 6 cubed spheres to r=20), "
                     f"7x{2 ** luni}^3 elements, {n} LGL nodes/dir (N={n - 1}), "
                     f"8 seeded Gaussian pulses, outgoing-radiation outer boundary, LLF"),
        "elements": E,
        "nodes_per_dir": n,
        "dof": E * n ** 3 * NFIELDS,
        "rk_stages_per_step": 4,
        "l2": "no flush: every state buffer (%.0f MB) exceeds the 129 MB L2"
              % (E * n ** 3 * NFIELDS * 8 / 1e6),
    }


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init_dist(world, backend):
    if world <= 1:
        return None
    import torch.distributed as dist
    dist.init_process_group(backend=backend)
    return dist


def max_over_ranks(dist, value, device=None):
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clock / throttle-reason sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def fp64_work_per_stage(variant, nelem, ncurvi, n, nnz_curvi=7):
    """(flops, instructions) of FP64 work one stage kernel issues, counted
    from the kernel source (FMA = 2 flops, 1 instruction; add/mul = 1, 1).
    Curvilinear elements of the cubed-sphere map have nnz_curvi = 7 nonzero
    chain-rule factors per node.  Face nodes: 4 subtractions + 10 FMA.
    RK update: stage average 1.75 FMA per DOF."""
    np_, nn = n ** 3, n * n
    ncart = nelem - ncurvi
    if variant.startswith("tc"):
        # derivatives on the tensor cores; FP64: the chain rule (one FMA per
        # nonzero metric entry and derivative), one int64 -> FP64 conversion
        # per derivative output (counted as an instruction, no flop)
        # plus the line left over in each pass at odd n (n^2 = 16 k + 1): an
        # FP64 dot product per output
        left = n * n if (n * n) % 16 == 1 else 0
        fields = ncart * 6 + ncurvi * (3 + nnz_curvi)
        vol_i = ncart * np_ * (6 + 6) + ncurvi * np_ * (2 * nnz_curvi + 3 + nnz_curvi) + \
            fields * left
        vol_f = ncart * np_ * 12 + ncurvi * np_ * 4 * nnz_curvi + fields * left * 2
    elif variant.startswith("eo"):
        M, odd = n // 2, n % 2
        # per line: e/o adds, S and T sums (first term a multiply), outputs
        ins = 2 * M + M * (M + odd) + M * M + 2 * M + odd * M
        fl = 2 * M + M * (1 + 2 * (M + odd - 1)) + M * (1 + 2 * (M - 1)) + 2 * M \
            + odd * (1 + 2 * (M - 1))
        lines_cart, lines_curv = 6 * nn, (3 + nnz_curvi) * nn
        vol_i = ncart * (lines_cart * ins + 6 * np_) + \
            ncurvi * (lines_curv * ins + 2 * nnz_curvi * np_ + 2 * np_)
        vol_f = ncart * (lines_cart * fl + 12 * np_) + \
            ncurvi * (lines_curv * fl + 4 * nnz_curvi * np_ + 2 * np_)
    else:
        vol_i = ncart * np_ * (6 * n + 6) + ncurvi * np_ * (12 * n + 18)
        vol_f = ncart * np_ * (12 * n + 9) + ncurvi * np_ * (24 * n + 36)
    surf_i, surf_f = nelem * 6 * nn * 14, nelem * 6 * nn * 24
    rk_i = nelem * np_ * NFIELDS * 1.75
    return vol_f + surf_f + 2 * rk_i, vol_i + surf_i + rk_i


def tc_mma_per_stage(nelem, ncurvi, nnz_curvi=7):
    """mma.m16n8k16 (FP16 in, FP32 accumulate) of the tensor-core variant per
    stage at n = 9: per element and pass one field per nonzero chain-rule row
    entry plus pi, 5 tiles of 16 lines (the 81st line is FP64), 5 k-steps x
    8 n-tiles."""
    fields = (nelem - ncurvi) * 6 + ncurvi * (3 + nnz_curvi)
    return fields * 5 * 40


def fp64_variant_line(kinfo, nelem, ncurvi, n, fp64_peak):
    """The all-FP64 stage kernel (eo) beside the selected one, from the
    autotuner's timings of the same run: with the tensor-core variant most
    of the FP64 work leaves the FP64 pipe, so the selected kernel's FP64
    fraction is not its bound; this is the FP64 form's own fraction."""
    timings = {}
    for tok in kinfo.split(" | timings: ")[-1].split():
        if "=" in tok and tok.endswith("ms"):
            k, v = tok.split("=")
            timings[k] = float(v[:-2])
    eo = {k: v for k, v in timings.items() if k.startswith("eo:")}
    if not eo:
        return None
    best = min(eo, key=eo.get)
    flops, ins = fp64_work_per_stage(best, nelem, ncurvi, n)
    ms = eo[best]
    return {"kernel": best, "launch_ms_autotune": ms,
            "fp64_gflops": flops / (ms / 1e3) / 1e9,
            "frac": flops / (ms / 1e3) / 1e9 / fp64_peak,
            "issue_frac": ins / (ms / 1e3) / (fp64_peak * 1e9 / 2),
            "note": "the selected tensor-core kernel issues ~40 % fewer FP64 "
                    "instructions and is latency-bound (ncu: FP64 pipe 55 % busy, tensor "
                    "pipe 10 %, profiles/tc_kernel_n9_cubedspheres_l3_stage1.md); its "
                    "roofline_fp64 counts only its own FP64 work"}


def alg_bytes_per_stage(nelem, ncurvi, n):
    """Algorithmic HBM bytes of one stage: state streams (RK4 average of
    16 streams / 4 stages = 4 streams x 8 B per DOF) + the chain-rule metric
    of curvilinear elements (9 doubles per node)."""
    np_ = n ** 3
    return nelem * np_ * NFIELDS * 4 * 8 + ncurvi * np_ * 9 * 8


def run_ours(args, rank, world, local):
    import torch
    import nmesh_gb300 as ng
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import gaussian_pulses

    torch.cuda.set_device(local)
    dist = init_dist(world, "nccl")
    n, luni = args.n, args.luni
    cfg = workload_config(n, luni)
    mesh = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=n, luni=luni, cs_dc=1.0, cs_r0fac=20.0)
    pat, _ = mesh.elements()
    ncurvi = int((pat > 0).sum())
    xyz = mesh.coords()
    u0 = gaussian_pulses(xyz, seed=1234 + rank)
    del xyz
    ev = ng.Evolution(mesh, ng.BC_OUTGOING)
    ev.set_state(u0)
    dx_min = 2.0 / 2 ** luni  # inner cube element edge
    dt = 0.25 * dx_min / (n - 1) ** 2
    dof = cfg["dof"]

    stream = torch.cuda.ExternalStream(ev.stream)
    # warm-up (also captures the step graphs)
    ev.rk4_steps(0.0, dt, args.warmup)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    l0 = ev.launches
    e0.record(stream)
    ev.rk4_steps(args.warmup * dt, dt, args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    launches = ev.launches - l0
    ms = e0.elapsed_time(e1)
    ms_max = max_over_ranks(dist, ms, torch.device("cuda", local))
    stages = 4 * args.steps
    value = world * dof * stages / (ms_max / 1e3)

    # end to end through the public API with host buffers: every step copies
    # u from pinned host memory to HBM, takes the RK4 step and copies u back
    host_u = torch.empty(ev.size, dtype=torch.float64, pin_memory=True).numpy()
    host_u[:] = ev.get_state().ravel()
    ev.rk4_steps_host(host_u, 0.0, dt, 1, inplace=True)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for s in range(args.steps):
        ev.rk4_steps_host(host_u, s * dt, dt, 1, inplace=True)
    t_e2e = time.perf_counter() - t0
    t_e2e = max_over_ranks(dist, t_e2e, torch.device("cuda", local))
    e2e_value = world * dof * stages / t_e2e

    # adjoint cost on the same mesh and data: one transposed RK4 step, and
    # the checkpointed gradient of J = sum_s dt sum W phi^2 over a short
    # horizon (forward sweep + recompute + adjoint sweep)
    adjoint = None
    if not args.no_adjoint:
        ev.set_state(u0)
        lam = torch.from_numpy(u0.ravel().copy()).cuda()
        torch.cuda.synchronize()
        ev.rk4_step_vjp_device(lam.data_ptr(), 0.0, dt)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        nv = 5
        for s in range(nv):
            ev.rk4_step_vjp_device(lam.data_ptr(), 0.0, dt)
        torch.cuda.synchronize()
        vjp_ms = 1e3 * (time.perf_counter() - t0) / nv
        xyz = mesh.coords()
        r = np.linalg.norm(xyz, axis=1)
        del xyz
        Wt = torch.from_numpy(np.where((r >= 17.0) & (r <= 19.0), 1.0, 0.0)).cuda()
        del r
        g = torch.empty_like(lam)
        nsteps_adj, ckpt = args.adj_steps, args.adj_ckpt
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Jv = ev.adjoint_gradient_device(Wt.data_ptr(), g.data_ptr(), 0.0, dt, nsteps_adj, ckpt)
        torch.cuda.synchronize()
        grad_ms = 1e3 * (time.perf_counter() - t0)
        fwd_ms = ms_max / args.steps
        adjoint = {"vjp_step_ms": vjp_ms, "forward_step_ms": fwd_ms,
                   "vjp_step_over_forward_step": vjp_ms / fwd_ms,
                   "gradient": f"J = sum_s dt sum W phi^2 on the shell 17<=r<=19, "
                               f"{nsteps_adj} RK4 steps, checkpoints every {ckpt}",
                   "gradient_ms": grad_ms, "J": Jv,
                   "gradient_cost_per_step_over_forward_step": grad_ms / (nsteps_adj * fwd_ms)}
        del lam, g, Wt

    kinfo = ev.kernel_info()
    state_bytes = int(ev.size * 8)
    batched = None
    fvres = None
    grhd = None
    config1 = None
    if rank == 0 and (not args.no_batched or not args.no_fv or not args.no_grhd or
                      not args.no_config1):
        ev.close()  # free the workload's buffers for the sub-benchmarks
        if not args.no_batched:
            batched = batched_bench(args)
        if not args.no_fv:
            fvres = fv_bench(args)
        if not args.no_grhd:
            grhd = grhd_bench(args)
        if not args.no_config1:
            config1 = config1_bench(args)

    fp64_peak = ng.fp64_peak_gflops()
    dmma_peak = ng.fp64_dmma_peak_gflops()
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fp:
            peaks = json.load(fp)
    except OSError:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    per_launch_ms = ms / stages
    alg_bytes = alg_bytes_per_stage(mesh.nelem, ncurvi, n)
    alg_bytes_stage1 = mesh.nelem * n ** 3 * NFIELDS * 3 * 8 + ncurvi * n ** 3 * 9 * 8
    variant = kinfo.split(" | ")[0]
    flops, fp64_ins = fp64_work_per_stage(variant, mesh.nelem, ncurvi, n)
    achieved_gbs = alg_bytes / (per_launch_ms / 1e3) / 1e9
    achieved_gflops = flops / (per_launch_ms / 1e3) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "dg_stage_kernel_n9_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as fp:
            traffic = json.load(fp).get("bytes_per_launch_full_size")

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args, n, luni)

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Gaussian pulses on the generated mesh)",
            "config": cfg,
            "parallelism": f"replicas x{world}",
            "e2e": {"value": e2e_value, "unit": UNIT,
                    "h2d_bytes_per_step": state_bytes,
                    "d2h_bytes_per_step": state_bytes},
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak,
                         "unit": "GB/s", "frac": achieved_gbs / hbm_peak,
                         "traffic": traffic,
                         "traffic_launch": "stage 1 of the RK4 step (reads u, writes the "
                                           "accumulator and w: 3 state streams + metric), "
                                           "captured at level 3 and scaled x8; "
                                           "alg_bytes_per_launch is the 4-stage average "
                                           "(3, 5, 5, 3 state streams)",
                         "alg_bytes_stage1": alg_bytes_stage1,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)",
                         "alg_bytes_per_launch": alg_bytes,
                         "kernel": kinfo.split(" | ")[0],
                         "autotune": kinfo.split(" | timings: ")[-1],
                         "launch_ms": per_launch_ms},
            "roofline_fp64": {"bound": "fp64", "achieved": achieved_gflops, "peak": fp64_peak,
                              "unit": "GFLOP/s", "frac": achieved_gflops / fp64_peak,
                              "flops_per_launch": flops,
                              "fp64_instructions_per_launch": fp64_ins,
                              "issue_frac": fp64_ins / (per_launch_ms / 1e3) / (fp64_peak * 1e9 / 2),
                              "peak_source": "FP64 FMA probe run live (nmg_fp64_peak)",
                              "dmma_probe_gflops": dmma_peak},
            "fp64_variant": fp64_variant_line(kinfo, mesh.nelem, ncurvi, n, fp64_peak),
            "tensor": ({"mma_m16n8k16_per_launch": tc_mma_per_stage(mesh.nelem, ncurvi),
                        "tflops": tc_mma_per_stage(mesh.nelem, ncurvi) * 4096 /
                        (per_launch_ms / 1e3) / 1e12,
                        "note": "FP16 tensor-core products of 8-bit digits (exact integers); "
                                "the tensor pipe is not the bound (legacy mma.sync rate "
                                "~0.5 per clock per SM, ncu tensor pipe ~10 % active)"}
                       if variant.startswith("tc") else None),
            "clocks": clk,
            "cpu_baseline": cpu,
            "adjoint": adjoint,
            "batched": batched,
            "fv": fvres,
            "grhd": grhd,
            "config1": config1,
        }
        print(json.dumps(out))
    ev.close()
    if dist:
        dist.destroy_process_group()


def batch_problem_specs(count, seed=4242):
    """Seeded set of independent problems: element counts log-uniform in
    [64, 32768] (realised by the nearest box (8^L) mesh or 7-cubed-sphere
    mesh with k of its patches one level finer, (7-k) 8^L + k 8^(L+1)
    elements, k in 0..3: refinement levels 0..5 with non-conforming faces
    between levels), orders N uniform in {3..9} (n = N+1 nodes): per patch
    on the cubed spheres without level jumps (parts of different n joined
    by interpolated traces), per problem otherwise."""
    rng = np.random.default_rng(seed)
    specs = []
    opts = [("box", L, 0, 8 ** L) for L in range(2, 6)] + \
        [("cs7", L, k, (7 - k) * 8 ** L + k * 8 ** (L + 1)) for L in range(0, 5)
         for k in range(4) if (7 - k) * 8 ** L + k * 8 ** (L + 1) <= 40000]
    for _ in range(count):
        target = np.exp(rng.uniform(np.log(64), np.log(32768)))
        kind, L, k, E = min(opts, key=lambda o: abs(np.log(o[3]) - np.log(target)))
        n = int(rng.integers(3, 10)) + 1
        href = tuple(sorted(int(p) for p in rng.choice(7, k, replace=False))) if k else ()
        orders = (n,)
        if kind == "cs7" and not k:
            orders = tuple(int(rng.integers(3, 10)) + 1 for _ in range(7))
        specs.append((kind, L, orders, E, href))
    return specs


def batch_meshes(specs):
    """Meshes of the problems (one per part) and each mesh's problem."""
    import nmesh_gb300 as ng
    meshes, owner = [], []
    for pid, (kind, L, orders, E, href) in enumerate(specs):
        if kind == "box":
            meshes.append(ng.Mesh.build(ng.MESH_BOX, n=orders[0], luni=L, xc=(PI, PI, PI),
                                        box_dout=PI, periodic=True))
            owner.append(pid)
        elif len(orders) == 1:
            meshes.append(ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=orders[0], luni=L, cs_dc=1.0,
                                        cs_r0fac=20.0, hrefine=href))
            owner.append(pid)
        else:
            for n in sorted(set(orders)):
                pats = [p for p in range(7) if orders[p] == n]
                meshes.append(ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=n, luni=L, cs_dc=1.0,
                                            cs_r0fac=20.0, patches=pats))
                owner.append(pid)
    return meshes, owner


def _batch_compare(meshes, owner, states, K):
    """Times of K RK4 steps of the problems: batched (one launch per stage
    for all orders, or one per order, graph-captured; parts of one problem
    joined), plain (each problem on its own: a context, or a batch of its
    parts, 4 stage launches per step) and per-problem graphs (each
    single-part problem's step captured; the multi-part ones as in plain)."""
    import torch
    import nmesh_gb300 as ng
    dt = 1e-4
    b = ng.Batch(meshes, ng.BC_OUTGOING, problems=owner)
    for p, u in enumerate(states):
        b.set_state(p, u)
    b.rk4_steps(0.0, dt, 2)  # autotune + graph capture + warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.rk4_steps(2 * dt, dt, K)
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0
    info = b.info()
    linked = b.linked_faces
    b.close()
    runs = []   # (kind, object)
    for pid in sorted(set(owner)):
        idx = [p for p in range(len(meshes)) if owner[p] == pid]
        if len(idx) == 1:
            ev = ng.Evolution(meshes[idx[0]], ng.BC_OUTGOING)
            ev.set_state(states[idx[0]])
            ev.rk4_step(0.0, dt)  # autotune + warm-up
            runs.append(("ctx", ev))
        else:
            pb = ng.Batch([meshes[p] for p in idx], ng.BC_OUTGOING, problems=[0] * len(idx))
            for q, p in enumerate(idx):
                pb.set_state(q, states[p])
            pb.rk4_steps(0.0, dt, 1)
            runs.append(("batch", pb))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(K):
        for kind, obj in runs:
            if kind == "ctx":
                obj.rk4_step((2 + s) * dt, dt)
            else:
                obj.rk4_steps((2 + s) * dt, dt, 1)
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t0
    for kind, obj in runs:
        if kind == "ctx":
            obj.rk4_steps(0.0, dt, 1)  # per-problem graphs captured
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for kind, obj in runs:
        obj.rk4_steps(0.0, dt, K)
    torch.cuda.synchronize()
    t_graphs = time.perf_counter() - t0
    for _, obj in runs:
        obj.close()
    dof = sum(m.nelem * m.np * NFIELDS for m in meshes)
    return {"problems": len(runs), "parts": len(meshes),
            "elements": int(sum(m.nelem for m in meshes)),
            "dof": int(dof), "steps": K, "linked_faces": int(linked),
            "batched_dof_stage_per_s": dof * 4 * K / t_batch,
            "plain_dof_stage_per_s": dof * 4 * K / t_plain,
            "per_problem_graphs_dof_stage_per_s": dof * 4 * K / t_graphs,
            "speedup_vs_plain_launches": t_plain / t_batch,
            "speedup_vs_per_problem_graphs": t_graphs / t_batch,
            "batch_info": info}


def batch_cpu_baseline(specs, count=8):
    """The oracle (OpenMP over the host cores) on a bounded sample of the
    batched workload: the first `count` problems that are single-order and
    without level jumps (meshes from the oracle's own generator), one RK4
    step each, one after the other, as the reference runs one mesh per
    process."""
    from oracle import nmo
    rng = np.random.default_rng(7)
    dof, t, used = 0, 0.0, 0
    for kind, L, orders, E, href in specs:
        if len(orders) > 1 or href or used >= count:
            continue
        n = orders[0]
        if kind == "box":
            g = nmo.generate_mesh(nmo.MESH_BOX, n, L, xc=(PI, PI, PI), box_dout=PI)
            period = 2 * PI
        else:
            g = nmo.generate_mesh(nmo.MESH_CUBEDSPHERES7, n, L)
            period = None
        pat, bbox, curvi, xyz, dXdx = g
        om = nmo.OracleMesh(bbox, curvi, dXdx, xyz,
                            nmo.match_faces_conforming(xyz, n, period=period), n, bc=1)
        u = 1e-3 * rng.standard_normal((len(pat), NFIELDS, n ** 3))
        om.rk4(u, 1e-4, 1)  # warm-up
        t0 = time.perf_counter()
        om.rk4(u, 1e-4, 1)
        t += time.perf_counter() - t0
        dof += len(pat) * NFIELDS * n ** 3
        used += 1
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count()))
    return {"value": dof * 4 / t, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"one RK4 step of each of {used} single-order problems without level "
                      f"jumps, one after the other ({dof} DOF), {t:.2f} s"}


def batched_bench(args):
    """Batched execution of many independent problems against the same
    problems stepped one after the other; for all 64 problems, for the ones
    of at most 4096 elements and for the ones of at most 512 elements, where
    the per-problem launches rather than the arithmetic set the time."""
    specs = batch_problem_specs(args.batch_problems)
    meshes, owner = batch_meshes(specs)
    rng = np.random.default_rng(7)
    states = [1e-3 * rng.standard_normal((m.nelem, NFIELDS, m.np)) for m in meshes]
    out = _batch_compare(meshes, owner, states, args.batch_steps)
    small_pids = {pid for pid, sp in enumerate(specs) if sp[3] <= 4096}
    sel = [p for p in range(len(meshes)) if owner[p] in small_pids]
    sub = _batch_compare([meshes[p] for p in sel], [owner[p] for p in sel],
                         [states[p] for p in sel], args.batch_small_steps)
    tiny_pids = {pid for pid, sp in enumerate(specs) if sp[3] <= 512}
    sel = [p for p in range(len(meshes)) if owner[p] in tiny_pids]
    tiny = _batch_compare([meshes[p] for p in sel], [owner[p] for p in sel],
                          [states[p] for p in sel], args.batch_small_steps)
    orders = sorted({int(m.n) for m in meshes})
    out.update({
        "orders_n": orders,
        "element_counts_min_max": [int(min(sp[3] for sp in specs)),
                                   int(max(sp[3] for sp in specs))],
        "mixed_order_problems": int(sum(1 for sp in specs if len(sp[2]) > 1)),
        "refinement_levels": sorted(set(int(L) + d for _, L, _, _, h in specs
                                        for d in ((0, 1) if h else (0,)))),
        "problems_with_level_jumps": int(sum(1 for s_ in specs if s_[4])),
        "note": "orders per patch on cubed spheres without level jumps (parts joined by "
                "interpolated traces), per problem otherwise; problems with level jumps have "
                "patches one level finer than their neighbours (non-conforming faces); all "
                "problems share dt",
        "cpu_baseline": None if args.no_cpu_baseline else batch_cpu_baseline(specs),
        "small_problems": dict(sub, selection="the problems of at most 4096 elements"),
        "tiny_problems": dict(tiny, selection="the problems of at most 512 elements")})
    return out


PI = 3.141592653589793


def fv_flops_per_stage(nelem, n):
    """Model of the FP64 work of one finite-volume stage (the fast variant;
    add, mul and division one flop, FMA two): per midpoint and direction 8
    WENO5 reconstructions with one-division weights (60 each) and the LLF
    flux with its normal (20); per point the flux differences, the
    J sqrtgdiag factors and the RK4 update (70)."""
    return nelem * (3 * (n - 1) * n * n * (8 * 60 + 20) + n ** 3 * 70)


def config1_bench(args):
    """The periodic-cube workload: [0, 2 pi]^3, 8^3 elements at n = 5 (N = 4),
    plane wave psi = A sin(x + y + z) with a seeded amplitude, LLF, RK4 with
    dt = 0.25 (2 pi / 8) / 16, 10 steps; the 10-step run repeated to time it
    (2.56 MB per state: launch- and latency-bound), resident and through
    host buffers, with the oracle on the same cores."""
    import torch
    import nmesh_gb300 as ng
    n, L, K, reps = 5, 3, 10, args.c1_reps
    m = ng.Mesh.build(ng.MESH_BOX, n=n, luni=L, xc=(PI, PI, PI), box_dout=PI, periodic=True)
    A = np.random.default_rng(2024).uniform(0.5, 1.5)
    xyz = m.coords()
    arg = xyz.sum(axis=1)
    om = np.sqrt(3.0)
    u0 = A * np.stack([-om * np.cos(arg), np.cos(arg), np.cos(arg), np.cos(arg), np.sin(arg)], 1)
    dt = 0.25 * (2 * PI / 8) / 16
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_state(u0)
    ev.rk4_steps(0.0, dt, K)  # autotune, graphs, warm-up
    stream = torch.cuda.ExternalStream(ev.stream)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    l0 = ev.launches
    e0.record(stream)
    for _ in range(reps):
        ev.rk4_steps(0.0, dt, K)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / (reps * K)
    launches = ev.launches - l0
    dof = m.nelem * m.np * NFIELDS
    host_u = torch.empty(ev.size, dtype=torch.float64, pin_memory=True).numpy()
    host_u[:] = u0.ravel()
    ev.rk4_steps_host(host_u, 0.0, dt, K, inplace=True)
    t0 = time.perf_counter()
    for _ in range(reps):
        host_u[:] = u0.ravel()
        ev.rk4_steps_host(host_u, 0.0, dt, K, inplace=True)
    t_e2e = (time.perf_counter() - t0) / (reps * K)
    kinfo = ev.kernel_info()
    ev.close()
    out = {"workload": "scalarwave1 RK4, periodic box [0,2pi]^3, 8^3 elements, n=5 (N=4), "
                       "plane wave psi = A sin(x+y+z), LLF, dt = 0.25 (2pi/8)/16, 10 steps",
           "elements": int(m.nelem), "dof": int(dof), "steps": K, "repeats": reps,
           "ms_per_step": ms, "value": dof * 4 / (ms / 1e3), "unit": UNIT,
           "e2e": {"value": dof * 4 / t_e2e, "unit": UNIT,
                   "h2d_bytes_per_step": dof * 8 / K, "d2h_bytes_per_step": dof * 8 / K,
                   "note": "one host round trip per 10-step run"},
           "kernel": kinfo.split(" | ")[0], "gpu_launches": int(launches)}
    if not args.no_cpu_baseline:
        from oracle import nmo
        pat, bbox, curvi, oxyz, dXdx = nmo.generate_mesh(nmo.MESH_BOX, n, L, xc=(PI, PI, PI),
                                                         box_dout=PI)
        nb = nmo.match_faces_conforming(oxyz, n, period=2 * PI)
        o = nmo.OracleMesh(bbox, curvi, dXdx, oxyz, nb, n, bc=1)
        a = oxyz.sum(axis=1)
        cu = A * np.stack([-om * np.cos(a), np.cos(a), np.cos(a), np.cos(a), np.sin(a)], 1)
        o.rk4(cu, dt, K)
        creps = 5
        t0 = time.perf_counter()
        for _ in range(creps):
            o.rk4(cu, dt, K)
        t = (time.perf_counter() - t0) / (creps * K)
        threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count()))
        out["cpu_baseline"] = {"value": dof * 4 / t, "unit": UNIT, "cores": threads,
                               "kind": "port",
                               "sample": f"{creps} runs of the 10-step workload, "
                                         f"{1e3 * t:.2f} ms per step"}
    return out


def fv_bench(args):
    """All-finite-volume workload: the 7-patch cubed-sphere mesh with every
    element a finite-volume element on n^3 equally spaced points, WENOm5_2
    midpoint states, dnfn_extrap1, outgoing boundary, graph-captured RK4
    steps; the oracle timed on a bounded sample of the same workload."""
    import torch
    import nmesh_gb300 as ng
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import gaussian_pulses
    n, L = args.fv_n, args.fv_luni
    rec, ex = "WENOm5_2", "dnfn_extrap1"
    mesh = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=n, luni=L, cs_dc=1.0, cs_r0fac=20.0, fv=True)
    u0 = gaussian_pulses(mesh.coords(), seed=99)
    ev = ng.Evolution(mesh, ng.BC_OUTGOING)
    ev.set_fv(rec, ex)
    ev.set_state(u0)
    dt = 0.1 * (2.0 / 2 ** L) / (n - 1)
    dof = mesh.nelem * mesh.np * NFIELDS
    stream = torch.cuda.ExternalStream(ev.stream)
    ev.rk4_steps(0.0, dt, 3)  # autotune, graph capture, warm-up
    torch.cuda.synchronize()
    K = args.fv_steps
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    l0 = ev.launches
    e0.record(stream)
    ev.rk4_steps(3 * dt, dt, K)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    launches = ev.launches - l0
    kinfo = ev.kernel_info()
    state_mb = ev.size * 8 / 1e6
    ev.close()
    out = {"workload": f"cubedspheres7 luni={L}, all {mesh.nelem} elements finite-volume "
                       f"on {n}^3 uniform points, fv_rec={rec}, fv_divf_extrap={ex}, "
                       f"outgoing boundary", "elements": int(mesh.nelem), "dof": int(dof),
           "state_mb": state_mb, "steps": K, "ms_per_step": ms / K,
           "value": dof * 4 * K / (ms / 1e3), "unit": UNIT,
           "kernel": kinfo.split(" | ")[0], "autotune": kinfo.split(" | timings: ")[-1],
           "gpu_launches": int(launches)}
    flops = fv_flops_per_stage(mesh.nelem, n)
    peak = ng.fp64_peak_gflops()
    achieved = flops / (ms / 1e3 / (4 * K)) / 1e9
    out["roofline_fp64"] = {"bound": "fp64", "achieved": achieved, "peak": peak,
                            "unit": "GFLOP/s", "frac": achieved / peak,
                            "flops_per_launch_model": flops,
                            "peak_source": "FP64 FMA probe run live (nmg_fp64_peak)",
                            "note": "divisions count one flop here but issue several FP64 "
                                    "instructions; the FP64 pipe utilization from ncu is in "
                                    "profiles/fv_fast_kernel_n13_cubedspheres_l2_rhs.md"}
    if not args.no_cpu_baseline:
        cl = args.fv_cpu_luni
        cxyz, om = cpu_mesh(n, cl, fv=True, fv_rec=rec, fv_extrap=ex)
        u = gaussian_pulses(cxyz, seed=99)
        cdt = 0.1 * (2.0 / 2 ** cl) / (n - 1)
        om.rk4(u, cdt, 1)
        t0 = time.perf_counter()
        om.rk4(u, cdt, args.fv_cpu_steps)
        t = time.perf_counter() - t0
        cdof = om.nelem * n ** 3 * NFIELDS
        threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count()))
        out["cpu_baseline"] = {
            "value": cdof * 4 * args.fv_cpu_steps / t, "unit": UNIT, "cores": threads,
            "kind": "port",
            "sample": f"{args.fv_cpu_steps} RK4 steps of the same workload at level {cl} "
                      f"({om.nelem} elements, {cdof} DOF), {t:.2f} s"}
    return out


GRHD_K = 100.0       # polytropic constant of the initial data, p = K rho^2
GRHD_RHO_ATM = 1e-10


def grhd_initial_prim(xyz, seed, rho0=1e-3, center=(8.0, 0.0, 0.0), width=2.0):
    """Primitives [E, 5, npts] of the GRHD workload at points xyz [E, 3,
    npts]: a Gaussian density blob rho0 exp(-|x - c|^2 / width^2) with 1 %
    seeded uniform perturbations on the atmosphere density, at rest, p = K
    rho^2."""
    rng = np.random.default_rng(seed)
    c = np.asarray(center)[None, :, None]
    r2 = ((xyz - c) ** 2).sum(1)
    rho = GRHD_RHO_ATM + rho0 * np.exp(-r2 / width ** 2) * \
        (1.0 + 0.01 * rng.uniform(-1.0, 1.0, r2.shape))
    prim = np.zeros((xyz.shape[0], 5, xyz.shape[2]))
    prim[:, 0] = rho
    prim[:, 4] = GRHD_K * rho * rho
    return prim


def grhd_flops_per_stage(ndg, nfv, n, nf, c2p_iterations_per_stage, dg_tensor=False):
    """Model of the FP64 work of one GRHD stage (add, mul, FMA, division and
    square root counted as one flop each, FMA as two), from the kernels'
    source: per DG node 3 directional fluxes (45), Cowling sources (35),
    45 derivatives of n terms plus the chain rule (90 n + 90), the RK4
    update (20), and per face node of the element a two-sided LLF with its
    speeds and the lift (170); per finite-volume point the sources (35),
    per direction and cell both face values of the 5 fields from one set of
    WENO5 smoothness indicators (450), per midpoint two prim2con (50) and
    the LLF (95), the divergence (60 for all three directions) and the
    update (20); con2prim 40 per point plus 30 per root-finder iteration
    (counted on the device).  With dg_tensor (the tensor-core DG kernel at
    n = 7, 8, 9) the line derivatives are integer digit products on the
    tensor cores, and only the line left over per direction at odd n
    (one of n^2) is FP64 work."""
    npd, npf = n ** 3, nf ** 3
    deriv = 90 * n
    if dg_tensor:
        deriv = 90 * n / (n * n) if (n * n) % 16 == 1 else 0
    dg = ndg * (npd * (45 + 35 + deriv + 90 + 20) + 6 * n * n * 170)
    fv = nfv * npf * (35 + 3 * 595 + 60 + 20)
    c2p = (ndg * npd + nfv * npf) * 40 + 30 * c2p_iterations_per_stage
    return dg + fv + c2p


def grhd_bench(args):
    """GRHD in the Cowling approximation (isotropic Schwarzschild, M = 1,
    Gamma = 2, atmosphere 1e-10): cubed shell r in [2, 20] of 6 x ndiv^3
    elements at n = 7 LGL points (N = 6), a seeded ~10 % of the elements
    switched to finite volume on nf = 13 equally spaced points (2N + 1),
    Gaussian blob at r = 8, graph-captured RK4 steps; with the oracle's
    restatement timed on a bounded sample."""
    import torch
    import nmesh_gb300 as ng
    n, nf, nd, K = 7, 13, args.grhd_ndiv, args.grhd_steps
    m = ng.Mesh.build(ng.MESH_CUBEDSHELL6, n=n, ndiv=nd, shell_rin=2.0, shell_rout=20.0)
    E = m.nelem
    prim = grhd_initial_prim(m.coords(), seed=33)
    ev = ng.GrhdEvolution(m, mass=1.0, gamma=2.0, rho_atm=GRHD_RHO_ATM,
                          p_atm=GRHD_K * GRHD_RHO_ATM ** 2, nf=nf)
    ev.set_prim(prim)
    flags = np.zeros(E, np.int32)
    flags[np.random.default_rng(34).choice(E, int(round(0.1 * E)), replace=False)] = 1
    ev.set_fv_elements(flags)
    # dt = 0.25 min dx / N^2, min dx the smallest element edge (the arc of
    # the angular edge on the inner sphere)
    hmin = 2.0 * (PI / 2.0) / nd
    dt = 0.25 * hmin / (n - 1) ** 2
    ev.rk4_steps(dt, 2)  # graphs captured, warm-up
    torch.cuda.synchronize()
    ev.reset_stats()
    stream = torch.cuda.ExternalStream(ev.stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    _, _, l0 = ev.stats()
    e0.record(stream)
    ev.rk4_steps(dt, K)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    iters, natm, l1 = ev.stats()
    shares = ev.profile_step(dt)
    tot = sum(shares.values())
    ndg, nfv = E - ev.nfv, ev.nfv
    dof = 5 * (ndg * n ** 3 + nfv * nf ** 3)
    u_dg, u_fv, p_dg, _ = ev.get_state()
    finite = bool(np.isfinite(u_dg).all() and np.isfinite(u_fv).all())
    ev.close()
    dg_tensor = 7 <= n <= 9 and os.environ.get("NMG_GRHD_DG") != "fp64"
    flops = grhd_flops_per_stage(ndg, nfv, n, nf, iters / (4.0 * K), dg_tensor)
    peak = ng.fp64_peak_gflops()
    achieved = flops / (ms / 1e3 / (4 * K)) / 1e9
    out = {"workload": f"GRHD Cowling, isotropic Schwarzschild M=1, Gamma=2, cubed shell "
                       f"r in [2,20], 6x{nd}^3 elements, n={n} (N={n - 1}), {nfv} elements "
                       f"({100.0 * nfv / E:.1f} %) finite volume on {nf}^3 points, WENOm5_2, "
                       f"Gaussian blob rho0=1e-3 at r=8, atmosphere 1e-10, dt={dt:.4g}",
           "elements": int(E), "fv_elements": int(nfv), "dof": int(dof), "steps": K,
           "ms_per_step": ms / K, "value": dof * 4 * K / (ms / 1e3), "unit": UNIT,
           "gpu_launches": int(l1 - l0), "finite": finite,
           "con2prim_iterations_per_point": iters / (4.0 * K) / (ndg * n ** 3 + nfv * nf ** 3),
           "atmosphere_points_per_stage": natm / (4.0 * K),
           "kernel_ms_per_step": shares,
           "dg_kernel": "tensor-core line derivatives" if dg_tensor else "FP64",
           "con2prim_share": shares["con2prim"] / tot if tot > 0 else None,
           "roofline_fp64": {"bound": "fp64", "achieved": achieved, "peak": peak,
                             "unit": "GFLOP/s", "frac": achieved / peak,
                             "flops_per_stage_model": flops,
                             "peak_source": "FP64 FMA probe run live (nmg_fp64_peak)"}}
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = grhd_cpu_baseline(args, n, nf)
    return out


def grhd_cpu_baseline(args, n, nf):
    """The oracle's GRHD restatement (OpenMP over the host cores) on a
    bounded sample: the same workload at ndiv = --grhd-cpu-ndiv, the same
    10 % switch, two RK4 steps."""
    from oracle import nmo
    nd = args.grhd_cpu_ndiv
    E = 6 * nd ** 3
    flags = np.zeros(E, np.int32)
    flags[np.random.default_rng(34).choice(E, int(round(0.1 * E)), replace=False)] = 1
    o = nmo.GrhdOracle(n=n, nf=nf, ndiv=nd, fv=flags, mass=1.0, gamma=2.0, rho_atm=GRHD_RHO_ATM,
                       p_atm=GRHD_K * GRHD_RHO_ATM ** 2)
    pd = grhd_initial_prim(o.xyz, seed=33)
    (_, _, npd), (_, _, npf) = o.shapes
    ud = np.stack([o.prim2con(pd[e], o.psi(o.xyz[e])) for e in range(E)])
    Pm, _ = o.transfer()
    uf, pf = np.zeros((E, 5, npf)), np.zeros((E, 5, npf))
    for e in np.nonzero(flags)[0]:
        uf[e] = o.apply3(Pm, ud[e])
        pf[e] = o.apply3(Pm, pd[e])
    dt = 0.25 * (2.0 * (PI / 2.0) / nd) / (n - 1) ** 2
    steps = 2
    t0 = time.perf_counter()
    o.rk4(ud, uf, pd, pf, dt, steps)
    t = time.perf_counter() - t0
    nfv = int(flags.sum())
    dof = 5 * ((E - nfv) * npd + nfv * npf)
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count()))
    return {"value": dof * 4 * steps / t, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} RK4 steps of the same workload at 6x{nd}^3 elements ({nfv} "
                      f"finite volume, {dof} DOF), {t:.2f} s"}


def cpu_mesh(n, luni, fv=False, fv_rec="WENOm5_2", fv_extrap="dnfn_extrap1"):
    """The oracle's own mesh of the workload (oracle/nmo_mesh.c: geometry
    restated from the reference, neighbour table by face matching); no
    product code is loaded."""
    from oracle import nmo
    pat, bbox, curvi, xyz, dXdx = nmo.generate_mesh(nmo.MESH_CUBEDSPHERES7, n, luni,
                                                    uniform=fv, cs_dc=1.0, cs_r0fac=20.0)
    nbnode = nmo.match_faces_conforming(xyz, n)
    fvk = dict(fv=np.ones(len(pat), np.int32), fv_rec=fv_rec, fv_extrap=fv_extrap) if fv else {}
    om = nmo.OracleMesh(bbox, curvi, dXdx, xyz, nbnode, n, bc=1, **fvk)
    return xyz, om


def cpu_baseline(args, n, luni, steps=None):
    """Time the oracle (C restatement of the reference path, OpenMP over all
    host cores) on a bounded sample of the workload: the same mesh, order,
    data, boundary and dt for `--cpu-steps` RK4 steps."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import gaussian_pulses
    xyz, om = cpu_mesh(n, luni)
    u = gaussian_pulses(xyz, seed=1234)
    del xyz
    dt = 0.25 * (2.0 / 2 ** luni) / (n - 1) ** 2
    nsteps = steps if steps is not None else args.cpu_steps
    u = om.rk4(u, dt, 1)  # warm-up (page-in, OpenMP threads)
    t0 = time.perf_counter()
    om.rk4(u, dt, nsteps)
    t = time.perf_counter() - t0
    dof = om.nelem * n ** 3 * NFIELDS
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count()))
    return {"value": dof * 4 * nsteps / t, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{nsteps} RK4 steps of the full workload ({om.nelem} elements, "
                      f"{dof} DOF), {t:.2f} s"}


def run_reference(args, rank, world):
    """The reference arm: the oracle's C restatement of the reference's RHS
    and RK4 step (bit-exact against the reference's own runs), OpenMP over
    all host cores, on the full workload (same mesh, order, data, boundary,
    dt and config as the GPU arm); its mesh comes from the oracle's own
    generator, so no product code is loaded."""
    if rank != 0:
        return
    n, luni = args.n, args.luni
    cfg = workload_config(n, luni)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import gaussian_pulses
    xyz, om = cpu_mesh(n, luni)
    u = gaussian_pulses(xyz, seed=1234)
    del xyz
    dt = 0.25 * (2.0 / 2 ** luni) / (n - 1) ** 2
    dof = om.nelem * n ** 3 * NFIELDS
    assert dof == cfg["dof"]
    for s in range(args.warmup):
        u = om.rk4(u, dt, 1, t=s * dt)
    t0 = time.perf_counter()
    for s in range(args.steps):
        u = om.rk4(u, dt, 1, t=(args.warmup + s) * dt)
    t = time.perf_counter() - t0
    value = dof * 4 * args.steps / t
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count()))
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Gaussian pulses on the generated mesh)",
        "config": cfg,
        "parallelism": f"host CPU, OpenMP x{threads}",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"each step: one RK4 step of the full workload "
                                   f"({om.nelem} elements, {dof} DOF)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=9)
    ap.add_argument("--luni", type=int, default=4)
    ap.add_argument("--cpu-steps", type=int, default=4)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batch-problems", type=int, default=64)
    ap.add_argument("--batch-steps", type=int, default=5)
    ap.add_argument("--batch-small-steps", type=int, default=50)
    ap.add_argument("--no-fv", action="store_true")
    ap.add_argument("--fv-n", type=int, default=13)
    ap.add_argument("--fv-luni", type=int, default=3)
    ap.add_argument("--fv-steps", type=int, default=5)
    ap.add_argument("--fv-cpu-luni", type=int, default=2)
    ap.add_argument("--fv-cpu-steps", type=int, default=2)
    ap.add_argument("--adj-steps", type=int, default=200)
    ap.add_argument("--adj-ckpt", type=int, default=20)
    ap.add_argument("--no-grhd", action="store_true")
    ap.add_argument("--no-config1", action="store_true")
    ap.add_argument("--c1-reps", type=int, default=20)
    ap.add_argument("--grhd-ndiv", type=int, default=12)
    ap.add_argument("--grhd-steps", type=int, default=50)
    ap.add_argument("--grhd-cpu-ndiv", type=int, default=6)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
