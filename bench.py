"""Benchmark: batched flat-shell time stepping in DOF-steps/s on GB300.

Default workload (N=1): 512 synthetic CFRP plates of U{40..80}^2 order-5
elements (6.25 mm), damage zones, random actuators, carriers {50,75,100} kHz,
FP32 stepping, advanced together (one fused kernel launch per time step,
CUDA-graph chunks).  A bench "step" is one time step of the whole batch.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) each rank advances its own 512 plates (seeded by rank;
weak scaling, no data-path collective); the timed region is bracketed by a
barrier and device synchronisation and rank 0 prints the max over ranks.
``--impl reference`` times the reference's CPU algorithm (the FP64 oracle
port, all host threads) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

ALG_BYTES = {32: 16.0, 64: 32.0}   # algorithmic bytes per DOF-step (u_n, u_n-1, u_n+1, 1/M)
# DRAM bytes (read + write) per DOF of one k_struct_step_f32 launch (tile 32), from an
# ncu capture of one launch on the 64-plate batch (294.1 + 81.1 MB for 30 001 270 DOF;
# the profile summary of k_struct_step_f32 under profiles/); traffic grows with the DOF count
F32_TRAFFIC_PER_DOF = (292.645632e6 + 80.066048e6) / 30001270
# floating-point operations per DOF-step executed by k_struct_step_f32, counted by ncu on
# the same launch (sass__thread_inst_executed_true_per_opcode: 740.6 M FFMA2 x 4, 280.5 M
# FMUL2 x 2, 82.4 M FFMA x 2, 54.7 M FMUL, 147.9 M FADD) over 30 001 270 DOF; lanes without
# an element execute the same instructions on zeros, so this exceeds the useful count
F32_FLOP_PER_DOF = (740.55168e6 * 4 + 280.512e6 * 2 + 82.4435e6 * 2 + 54.743158e6 + 147.884554e6) / 30001270
METRIC = "DOF-steps/s (batched flat-shell SEM forward, 512 uneven plates)"


def peaks():
    try:
        return json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json"))), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0]))
                mx.append(float(p[1]))
            except ValueError:
                continue
            for nm, v in zip(names, p[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def dist_init(args):
    """Rank, world size and local rank from torchrun's environment.  The GPU arm
    uses NCCL (barrier and max of the timers only: plates are independent, so
    the data path has no collective); the CPU reference arm uses gloo."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        rank = int(os.environ["RANK"])
        local = int(os.environ.get("LOCAL_RANK", rank))
        backend = "nccl" if args.impl == "ours" else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
        return rank, ws, local
    return 0, 1, 0


def _on_gpu():
    import torch.distributed as dist
    return dist.get_backend() == "nccl"


def barrier_sync(ws):
    if ws > 1:
        import torch
        import torch.distributed as dist
        if _on_gpu():
            torch.cuda.synchronize()
        dist.barrier()


def max_over_ranks(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if _on_gpu() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rank_batch(W, plates, rank):
    """This rank's shard: its own `plates` plates, seeded by the rank (weak
    scaling: per-rank work is fixed as the number of ranks grows)."""
    return W.batch(n=plates, seed=1000 * rank)


ARM_PARTS = {0xd0c: "Neoverse N1", 0xd40: "Neoverse V1", 0xd49: "Neoverse N2", 0xd4f: "Neoverse V2"}


def cpu_model() -> str:
    """The host CPU's name as /proc/cpuinfo gives it (x86 model name, or the
    Arm implementer/part), for the CPU baseline's record."""
    try:
        info = open("/proc/cpuinfo").read()
        for line in info.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
        part = [line.split(":", 1)[1].strip() for line in info.splitlines() if line.startswith("CPU part")]
        if part:
            code = int(part[0], 16)
            return f"Arm {ARM_PARTS.get(code, hex(code))}"
    except (OSError, ValueError, IndexError):
        pass
    return os.uname().machine


def cpu_reference(scenarios, run, steps, nthreads=0, budget_s=20.0):
    """Oracle (FP64 port of the reference loop) on a bounded sample: the first
    plates of the batch, `steps` time steps each, all host threads."""
    from oracle.oracle import OracleProblem
    done_dof_steps = 0
    t_total = 0.0
    used = 0
    for sc in scenarios:
        orc = OracleProblem(sc.mesh["nodes"], sc.mesh["coords"], sc.mat_table, sc.elem_mat, sc.elem_keep)
        t0 = time.perf_counter()
        orc.run(run.dt, run.nft, sc.signal, nn_first=run.nn_first, eta_xy=run.eta_xy, eta_z=run.eta_z,
                force_dof=sc.force_dof, force_val=sc.force_val, out_dof=sc.out_dof, h=run.h,
                nn_last=run.nn_first + steps - 1, nthreads=nthreads)
        t_total += time.perf_counter() - t0
        done_dof_steps += 5 * sc.mesh["coords"].shape[0] * steps
        used += 1
        if t_total >= budget_s:
            break
    return done_dof_steps / t_total, used, t_total


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def accuracy_record(pkg, scs, run, r32, nsample=16, seed=0):
    """FP32 sensor-signal error of the benchmark batch against FP64: the
    sampled plates (the largest half of the sample, the rest drawn at random)
    run again through the engine's FP64 path (pinned to the oracle) for the
    whole 0.4 ms; relative L2 over each plate's 8 displacement signals and
    their velocities a1 (u(n+1) - u(n-1)), taken from the FP32 results of the
    full 512-plate run."""
    import torch
    W = pkg.workloads
    dof = np.array([W.dof_count([sc]) for sc in scs])
    order = np.argsort(-dof, kind="stable")
    nbig = nsample // 2
    rest = np.random.default_rng(seed).choice(order[nbig:], nsample - nbig, replace=False)
    idx = [int(i) for i in np.concatenate([order[:nbig], rest])]
    with ClockSampler() as clk:
        t0 = time.perf_counter()
        p64 = pkg.Plan([scs[i] for i in idx], run, precision=64, path=0, steps_per_graph=50)
        r64 = p64.forward()
        torch.cuda.synchronize()
        t64 = time.perf_counter() - t0
        path64 = p64.info["path"]
        p64.close()
    ed, ev = [], []
    for k, i in enumerate(idx):
        a, b = r32[i]["displ"][run.nn_first - 1:], r64[k]["displ"][run.nn_first - 1:]
        ed.append(rel_l2(a, b))
        ev.append(rel_l2(a[2:] - a[:-2], b[2:] - b[:-2]))
    elems = [int(np.asarray(scs[i].mesh["nodes"]).shape[0]) for i in idx]
    return {"what": "FP32 (full 512-plate batch run) vs FP64 engine path, sensor signals over the whole run",
            "plates": idx, "elements": elems, "steps": run.nft - run.nn_first + 1,
            "displ_rel_l2_max": max(ed), "displ_rel_l2_median": float(np.median(ed)),
            "velocity_rel_l2_max": max(ev), "velocity_rel_l2_median": float(np.median(ev)),
            "bound": 1e-3, "within_bound": bool(max(max(ed), max(ev)) <= 1e-3),
            "fp64_path": "structured" if path64 == 2 else "general", "fp64_s": t64, "clocks": clk.summary()}


def plain_fp64_record(pkg, value, e2e_value, steps=40):
    """The 30x denominator: the reference-structured FP64 GPU loop
    (baseline/plain_gpu_fp64.py) on one plate of the batch workload and on
    the 200x200-element plate, CUDA events over `steps` steps, outputs checked
    against the engine's FP64 path over the same steps."""
    from baseline.plain_gpu_fp64 import rate
    W = pkg.workloads
    out = {"what": "plain single-scenario FP64 GPU loop (gpuArray operation sequence of main_flat_shell.m:651-750, "
                   "cuSPARSE SpMV + gathers + index_add)"}
    cases = {"batch_plate_0": W.batch(n=1, seed=0), "plate_200x200_pzt": W.plate_pzt(nft=steps + 20)}
    with ClockSampler() as clk:
        for name, (cs, crun) in cases.items():
            v, displ = rate(pkg, cs[0], crun, steps=steps, warmup=5)
            p = pkg.Plan(cs, crun, precision=64, path=1)
            p.reset()
            p.set_signal()
            p.advance(steps + 5)
            ref = p.read_outputs()[0]["displ"][crun.nn_first - 1: crun.nn_first - 1 + steps + 5]
            p.close()
            out[name] = {"dof": W.dof_count(cs), "dof_steps_per_s": v, "steps": steps,
                         "rel_err_vs_engine_fp64": rel_l2(displ, ref) if np.abs(ref).max() > 0 else 0.0}
    big = out["plate_200x200_pzt"]["dof_steps_per_s"]
    small = out["batch_plate_0"]["dof_steps_per_s"]
    out["ratio_batched_fp32_vs_plain_fp64"] = {"vs_200x200_plate": value / big, "vs_batch_plate": value / small,
                                               "e2e_vs_200x200_plate": (e2e_value / big) if e2e_value else None,
                                               "target": 30.0}
    out["clocks"] = clk.summary()
    return out


def adjoint_record(pkg, maps=64, steps=20000, check_steps=2000, nfd=20):
    """Config 5 reduced to what fits the default run: gradient cost / forward
    cost on the full damage-identification batch (64 maps, 50x50 elements,
    20 000 steps, checkpoints every 200, FP32 structured plan) with the state
    store at its default (half the free memory), off (every segment
    recomputed) and at the opt-in setting (the free memory less 8 GiB);
    gradient accuracy on map 0 over the first `check_steps`
    steps: FP32 and FP64 adjoint gradients against central differences of the
    FP64 forward on `nfd` random parameters (all 2 nfd perturbed plates in
    one batched plan)."""
    import torch
    W = pkg.workloads
    out = {"what": "adjoint gradient cost / forward cost, config 5 (64 maps x 50x50 elements)"}
    scs, run, hidden = W.adjoint_maps(n=maps, nft=steps)
    truth = [pkg.Scenario(**{**sc.__dict__, "elem_keep": h}) for sc, h in zip(scs, hidden)]
    with ClockSampler() as clk:
        p = pkg.Plan(truth, run, precision=32, path=2, steps_per_graph=50)
        targets = [r["displ"] for r in p.forward()]
        p.close()
        p = pkg.Plan(scs, run, precision=32, path=2, steps_per_graph=50)
        out["autotune"] = p.autotune(10)
        p.forward()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        p.forward()
        torch.cuda.synchronize()
        t_fwd = time.perf_counter() - t0
        out["forward_s"] = t_fwd
        for label, cap in (("store_default", None), ("store_off", 0), ("store_spare", "spare")):
            p.set_adjoint_store(cap)
            t0 = time.perf_counter()
            p.forward_backward(targets, ckpt_every=200)
            torch.cuda.synchronize()
            t = time.perf_counter() - t0
            out[label] = {"forward_backward_s": t, "ratio": t / t_fwd, "segments_kept": p.stored_segments(),
                          "phases_ms": p.forward_backward_timing()}
        p.close()
    out["dof"] = W.dof_count(scs)
    out["steps"] = run.nft - run.nn_first + 1
    out["target_ratio"] = 3.0
    out["clocks"] = clk.summary()
    # accuracy on a shorter run of map 0
    scs_s, run_s, hid_s = W.adjoint_maps(n=1, nft=check_steps)
    truth_s = pkg.Scenario(**{**scs_s[0].__dict__, "elem_keep": hid_s[0]})
    p = pkg.Plan([truth_s], run_s, precision=64, path=0)
    target = p.forward()[0]["displ"]
    p.close()
    g = {}
    for prec in (32, 64):
        p = pkg.Plan(scs_s, run_s, precision=prec, path=0, steps_per_graph=50)
        _, gr = p.forward_backward([target], ckpt_every=200)
        p.close()
        g[prec] = gr[0]
    rng = np.random.default_rng(7)
    idx = rng.choice(len(g[64]), nfd, replace=False)
    eps = 1e-4
    sc0 = scs_s[0]
    pert = []
    for e in idx:
        for sgn in (-1.0, 1.0):
            k = sc0.elem_keep.copy()
            k[e] += sgn * eps     # d_e = 1 - keep_e: keep - eps is d + eps
            pert.append(pkg.Scenario(**{**sc0.__dict__, "elem_keep": k}))
    p = pkg.Plan(pert, run_s, precision=64, path=0, steps_per_graph=50)
    res = p.forward()
    p.close()
    J = [0.5 * float(np.sum((r["displ"] - target)[run_s.nn_first - 1:] ** 2)) for r in res]
    fd = np.array([(J[2 * q] - J[2 * q + 1]) / (2 * eps) for q in range(nfd)])
    out["accuracy"] = {"steps": check_steps, "params": nfd, "eps": eps,
                       "grad_fp32_vs_fd_rel": rel_l2(g[32][idx], fd),
                       "grad_fp64_vs_fd_rel": rel_l2(g[64][idx], fd),
                       "grad_fp32_vs_fp64_rel": rel_l2(g[32], g[64]), "bound": 1e-3}
    return out


def adjoint_bench(pkg, args):
    """Gradient cost / forward cost on the damage-identification batch, FP32
    gradient vs FP64 gradient, and central differences on 20 parameters."""
    import torch
    W = pkg.workloads
    scs, run, hidden = W.adjoint_maps(n=args.adj_maps, nft=args.adj_steps)
    # targets from the hidden maps (FP64 forward)
    truth = [pkg.Scenario(**{**sc.__dict__, "elem_keep": h}) for sc, h in zip(scs, hidden)]
    p64 = pkg.Plan(truth, run, precision=64, path=1, steps_per_graph=50)
    targets = [r["displ"] for r in p64.forward()]
    p64.close()
    ndof = W.dof_count(scs)
    out = {"metric": "adjoint gradient cost / forward cost", "maps": len(scs), "dof": ndof, "nft": run.nft,
           "ckpt_every": 200, "dtype": "f32 stepping, f64 misfit and gradient"}
    times, t_adj, grads = {}, {}, {}
    for path in (1, 2):
        p = pkg.Plan(scs, run, precision=32, path=path, steps_per_graph=50)
        if path == 2:
            out["autotune_path2"] = p.autotune(10)
        p.forward()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        p.forward()
        torch.cuda.synchronize()
        times[path] = time.perf_counter() - t0
        t0 = time.perf_counter()
        mis32, grads[path] = p.forward_backward(targets, ckpt_every=200)
        torch.cuda.synchronize()
        t_adj[path] = time.perf_counter() - t0
        out[f"phases_ms_path{path}"] = p.forward_backward_timing()
        out[f"stored_segments_path{path}"] = p.stored_segments()
        p.close()
    g32 = grads[2]
    out["forward_s_general_path"] = times[1]
    out["forward_s_structured_path"] = times[2]
    out["forward_backward_s_general_path"] = t_adj[1]
    out["forward_backward_s_structured_path"] = t_adj[2]
    out["ratio_vs_forward_same_path"] = {str(k): t_adj[k] / times[k] for k in (1, 2)}
    out["ratio_vs_fastest_forward"] = min(t_adj.values()) / min(times.values())
    out["grad_rel_diff_structured_vs_general_fp32"] = max(
        float(np.linalg.norm(grads[2][i] - grads[1][i]) / np.linalg.norm(grads[1][i])) for i in range(len(scs)))
    # FP64 reference gradient on the first maps
    nref = min(4, len(scs))
    p = pkg.Plan(scs[:nref], run, precision=64, path=1)
    mis64, g64 = p.forward_backward(targets[:nref], ckpt_every=200)
    p.close()
    out["grad_rel_err_f32_vs_f64"] = max(float(np.linalg.norm(g32[i] - g64[i]) / np.linalg.norm(g64[i]))
                                         for i in range(nref))
    out["misfit_rel_err_f32_vs_f64"] = max(float(abs(mis32[i] - mis64[i]) / mis64[i]) for i in range(nref))
    # central differences (FP64 forward) on 20 random parameters of map 0
    rng = np.random.default_rng(7)
    idx = rng.choice(len(g64[0]), 20, replace=False)
    eps = 1e-4
    sc0 = scs[0]

    def J(keep):
        q = pkg.Plan([pkg.Scenario(**{**sc0.__dict__, "elem_keep": keep})], run, precision=64, path=1,
                     steps_per_graph=50)
        d = q.forward()[0]["displ"]
        q.close()
        r = (d - targets[0])[run.nn_first - 1:]
        return 0.5 * float(np.sum(r * r))

    fd = []
    for e in idx:
        kp, km = sc0.elem_keep.copy(), sc0.elem_keep.copy()
        kp[e] -= eps
        km[e] += eps
        fd.append((J(kp) - J(km)) / (2 * eps))
    fd = np.array(fd)
    out["fd_rel_err_f64_grad"] = float(np.linalg.norm(g64[0][idx] - fd) / np.linalg.norm(fd))
    out["fd_rel_err_f32_grad"] = float(np.linalg.norm(g32[0][idx] - fd) / np.linalg.norm(fd))
    print(json.dumps(out))


def plain_fp64_bench(pkg, args):
    """Reference-structured FP64 GPU loop on single scenarios: one plate of
    the batch workload and the 200x200-element plate; outputs checked against
    the engine's FP64 path over the same steps."""
    from baseline.plain_gpu_fp64 import rate
    W = pkg.workloads
    out = {"metric": "plain single-scenario FP64 GPU path, DOF-steps/s"}
    cases = {"batch_plate": W.batch(n=1, seed=0), "plate_200x200_pzt": W.plate_pzt()}
    for name, (scs, run) in cases.items():
        steps = 40
        v, displ = rate(pkg, scs[0], run, steps=steps, warmup=5)
        p = pkg.Plan(scs, run, precision=64, path=1)
        p.reset()
        p.set_signal()
        p.advance(steps + 5)
        ref = p.read_outputs()[0]["displ"][run.nn_first - 1: run.nn_first - 1 + steps + 5]
        p.close()
        err = float(np.linalg.norm(displ - ref) / max(np.linalg.norm(ref), 1e-300)) if np.abs(ref).max() > 0 else 0.0
        out[name] = {"dof": W.dof_count(scs), "dof_steps_per_s": v, "rel_err_vs_engine_fp64": err, "steps": steps}
    print(json.dumps(out))


def single_plate_bench(pkg, args):
    """One plate (config 1 or 2): whole forward solve in FP64 and FP32 through
    shm_forward (outputs, PZT voltage, frames), FP32 error vs the FP64 run."""
    import torch
    W = pkg.workloads
    if args.workload == "solid":
        scs, run = W.solid_plate()
        ndof = int(3 * np.asarray(scs[0].mesh["coords"]).shape[0])
    else:
        scs, run = W.plate_force() if args.workload == "force" else W.plate_pzt()
        ndof = W.dof_count(scs)
    if args.nft > 0:  # a shorter run of the same plate (profiling)
        run.nft = min(run.nft, args.nft)
        for sc in scs:
            sc.signal = np.asarray(sc.signal)[:run.nft]
    nsteps = run.nft - run.nn_first + 1
    res, out = {}, {"workload": args.workload, "dof": ndof, "nft": run.nft, "dt_s": run.dt,
                    "frames": run.frm_int > 0}
    precs = (64, 32) if args.prec == 0 else (args.prec,)
    for prec in precs:
        if args.workload == "solid":
            p = pkg.SolidPlan(scs, run, precision=prec, steps_per_graph=50)
        else:
            p = pkg.Plan(scs, run, precision=prec, path=0, steps_per_graph=50)
        if p.info["path"] == 2 and prec == 32:
            out["autotune"] = p.autotune(10)
        p.forward(want_frames=run.frm_int > 0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = p.forward(want_frames=run.frm_int > 0)[0]
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        res[prec] = r
        out[f"fp{prec}_dof_steps_per_s"] = ndof * nsteps / dt
        out[f"fp{prec}_s"] = dt
        out[f"fp{prec}_path"] = p.info["path"]
        if prec == 32 and p.info["path"] == 2 and args.workload != "solid":
            # the launch mode the autotuner did not keep, on the same tasks
            mode = bool(p.info["persistent"])
            p.set_persistent(not mode)
            p.forward(want_frames=run.frm_int > 0)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r2 = p.forward(want_frames=run.frm_int > 0)[0]
            torch.cuda.synchronize()
            dt2 = time.perf_counter() - t0
            out["fp32_other_launch_mode"] = {"persistent": not mode, "dof_steps_per_s": ndof * nsteps / dt2,
                                             "same_bits": bool(np.array_equal(r2["displ"], r["displ"]))}
        p.close()
    def rel(a, b):
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
    if len(precs) == 1:
        print(json.dumps(out))
        return
    out["fp32_vs_fp64_displ_rel_l2"] = rel(res[32]["displ"], res[64]["displ"])
    vel32 = np.diff(res[32]["displ"][1:], axis=0)
    vel64 = np.diff(res[64]["displ"][1:], axis=0)
    out["fp32_vs_fp64_velocity_rel_l2"] = rel(vel32, vel64)
    if res[64]["voltage"].size and np.abs(res[64]["voltage"]).max() > 0:
        out["fp32_vs_fp64_voltage_rel_l2"] = rel(res[32]["voltage"], res[64]["voltage"])
    if "frames" in res[64]:
        out["fp32_vs_fp64_frames_rel_l2"] = rel(res[32]["frames"], res[64]["frames"])
    print(json.dumps(out))


def wavefield_bench(pkg, args):
    """Wavefield frames -> grid (spec2meshgrid_flat_shell.m) on the config-2
    plate (200x200 elements, 1.0 M nodes): FP32 forward solve recording all
    five velocity components every 40 steps, then the 512x512 grid of motion 9
    (total velocity, top surface, all five fields per node) interpolated from
    the device-resident frames.  Reports grid points x frames per second of
    the interpolation kernel (CUDA events) and checks it against the host-frame
    path."""
    import torch
    W = pkg.workloads
    scs, run = W.plate_pzt(nft=2001)
    run.frm_int, run.frame_dof, run.frame_kind = 40, 0, 0
    plan = pkg.Plan(scs, run, precision=32, path=0, steps_per_graph=50)
    plan.forward(want_frames=False)
    torch.cuda.synchronize()
    nfr = plan.info["nframes"]
    n = 512
    t0 = time.perf_counter()
    g = pkg.wavefield.Grid(scs[0].mesh, n, n, "top")
    setup_s = time.perf_counter() - t0
    ms = g.time(plan, 9, run.h, "velocity", reps=max(args.steps, 3))
    img = g.from_plan(plan, 9, run.h, "velocity")
    host = plan.read_outputs(want_frames=True)[0]["frames"]
    img_h = g.interpolate(host, [0, 1, 2, 3, 4], 9, run.h)
    nnode = int(np.asarray(scs[0].mesh["coords"]).shape[0])
    uniq = nfr * (5 * nnode * 4 + n * n * 8)        # each field value read once, each pixel written once
    out = {"workload": "wavefield grid 512x512, motion 9, top, config-2 plate", "nnode": nnode, "frames": nfr,
           "setup_s": setup_s, "max_err_m": g.points()["max_err"], "kernel_ms": ms,
           "points_frames_per_s": n * n * nfr / (ms / 1e3),
           "unique_bytes_gbs": uniq / (ms / 1e3) / 1e9,
           "plan_vs_host_frames_max_abs": float(np.abs(img - img_h).max()),
           "peak_abs": float(np.abs(img).max())}
    g.close()
    plan.close()
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--plates", type=int, default=512)
    ap.add_argument("--precision", type=int, default=32)
    ap.add_argument("--graph", type=int, default=50)
    ap.add_argument("--tile", type=int, default=0)
    ap.add_argument("--rows", type=int, default=0)
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--persistent", type=int, default=-1, choices=(-1, 0, 1),
                    help="structured FP32 plans: -1 as the autotuner chose (off without it), 0 per-step "
                         "launches in CUDA graphs, 1 one persistent launch per advance")
    ap.add_argument("--path", type=int, default=0, help="0 auto, 1 general, 2 structured, 3 structured generic")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the accuracy, plain-FP64 and adjoint records of the default line")
    ap.add_argument("--adjoint", action="store_true", help="damage-gradient workload instead of the forward batch")
    ap.add_argument("--workload", choices=("batch", "force", "pzt", "solid", "wavefield"), default="batch",
                    help="batch: 512 plates (default); force: 20x20-element plate; pzt: 200x200 plate with PZT")
    ap.add_argument("--nft", type=int, default=0,
                    help="force/pzt/solid: stop the plate's run after this many steps (0 = the full run)")
    ap.add_argument("--prec", type=int, default=0, choices=(0, 32, 64),
                    help="force/pzt/solid: run one precision only (0 = FP64 and FP32, compared)")
    ap.add_argument("--adj-maps", type=int, default=64)
    ap.add_argument("--adj-steps", type=int, default=20000)
    ap.add_argument("--plain-fp64", action="store_true",
                    help="time the reference-structured FP64 GPU loop (the 30x denominator)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    rank, ws, local = dist_init(args)
    import __graft_entry__ as g
    pkg = g.package()
    if args.adjoint:
        return adjoint_bench(pkg, args)
    if args.plain_fp64:
        return plain_fp64_bench(pkg, args)
    if args.workload == "wavefield":
        return wavefield_bench(pkg, args)
    if args.workload != "batch":
        return single_plate_bench(pkg, args)
    W = pkg.workloads
    scs, run = rank_batch(W, args.plates, rank)
    ndof = W.dof_count(scs)
    config = {"workload": f"batch of {args.plates} flat-shell plates, U{{40..80}}^2 order-5 elements (6.25 mm), "
                          f"1-3 damage zones, random actuator, 5-cycle Hann {{50,75,100}} kHz, 0.4 ms",
              "plates_per_gpu": args.plates, "dof_per_gpu": ndof, "dt_s": run.dt, "nft": run.nft,
              "l2": "inputs larger than L2 (state %.2f GB per buffer)" % (ndof * args.precision / 8 / 1e9),
              "parallelism": f"scenario shards x{ws}"}

    if args.impl == "reference":
        if rank != 0:
            return
        steps = max(5, min(args.steps, 20))
        vals = []
        for _ in range(max(1, min(args.warmup, 1))):
            cpu_reference(scs[:1], run, 3)
        v, used, tt = cpu_reference(scs, run, steps, budget_s=20.0)
        out = {"metric": METRIC, "value": v, "unit": "DOF-steps/s", "n_gpus": ws, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": 1e3 * ndof / v, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config, "impl": "reference",
               "cpu_baseline": {"value": v, "unit": "DOF-steps/s", "cores": os.cpu_count(), "kind": "port",
                                "cpu_model": cpu_model(),
                                "sample": f"first {used} plates x {steps} time steps, FP64 oracle restating "
                                          "main_flat_shell.m:651-917, OpenMP over all host threads"},
               "e2e": {"value": v, "unit": "DOF-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out))
        return

    import torch
    t0 = time.perf_counter()
    plan = pkg.Plan(scs, run, precision=args.precision, path=args.path, steps_per_graph=args.graph,
                    tile_elems=args.tile, device=local, rows_per_block=args.rows)
    setup = {"plan_create_s": time.perf_counter() - t0,
             "what": "shm_plan_create of the whole batch: geometry, mass, task lists, device upload "
                     "(the set-up part of main_flat_shell.m:35-650)"}
    tuned = None
    if plan.info["path"] == 2 and args.tile == 0 and args.rows == 0 and not args.no_tune:
        t0 = time.perf_counter()
        tuned = plan.autotune(10)
        setup["autotune_s"] = time.perf_counter() - t0
    if args.persistent >= 0 and plan.info["path"] == 2 and args.precision == 32:
        plan.set_persistent(bool(args.persistent))
    config["path"] = "general" if plan.info["path"] == 1 else "structured"
    config["tile_elems"] = plan.info["tile"]
    config["rows_per_block"] = plan.info["rows_per_block"]
    config["persistent"] = bool(plan.info["persistent"])
    config["autotuned"] = tuned is not None
    plan.reset()
    plan.set_signal()
    nmax = run.nft - run.nn_first + 1
    if args.warmup + args.steps > nmax:
        raise SystemExit("warmup + steps exceed the run length")
    plan.advance(args.warmup)
    barrier_sync(ws)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = plan.time_steps(args.steps)   # CUDA events on the plan's stream
    torch.cuda.synchronize()
    barrier_sync(ws)
    ms = max_over_ranks(ms, ws)
    sec = ms / 1e3
    value = ndof * ws * args.steps / sec
    per_launch_s = sec / args.steps
    pk, pk_kind = peaks()
    achieved = ALG_BYTES[args.precision] * ndof / per_launch_s / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": achieved / pk["hbm_gbs"],
            "traffic": (F32_TRAFFIC_PER_DOF * ndof if args.precision == 32 and plan.info["path"] == 2 else None),
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch on the 64-plate "
                              "batch, scaled by DOF (bytes per launch)",
            "fp32_tflops": (F32_FLOP_PER_DOF * value / 1e12 if args.precision == 32 and plan.info["path"] == 2
                            else None),
            "flop_per_dof_step": F32_FLOP_PER_DOF if args.precision == 32 else None,
            "basis": f"{ALG_BYTES[args.precision]:.0f} B/DOF-step x {ndof} DOF per step of "
                     f"the fused structured step, CUDA events over {args.steps} steps; peak {pk_kind}"}
    if plan.info["persistent"]:
        launches = 2   # the persistent step kernel and the step-counter kernel
    else:
        launches = args.steps * plan.info["launches_per_step"] + (args.steps // args.graph if args.graph else 1)

    e2e = None
    r32 = None
    if not args.no_e2e:
        # whole forward solve through the public API: H2D of the excitation,
        # every time step, D2H of all sensor signals
        t0 = time.perf_counter()
        r32 = plan.forward()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        nsteps = run.nft - run.nn_first + 1
        e2e_v = max_over_ranks(t1 - t0, ws)
        nout = sum(len(s.out_dof) for s in scs)
        e2e = {"value": ndof * ws * nsteps / e2e_v, "unit": "DOF-steps/s",
               "h2d_bytes_per_step": 8 * len(scs), "d2h_bytes_per_step": 8 * nout,
               "what": f"shm_forward of {nsteps} steps incl. signal upload and sensor download"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        v, used, tt = cpu_reference(scs, run, 10, budget_s=15.0)
        v1, used1, tt1 = cpu_reference(scs[:2], run, 3, nthreads=1, budget_s=5.0)
        cpu = {"value": v, "unit": "DOF-steps/s", "cores": os.cpu_count(), "kind": "port",
               "cpu_model": cpu_model(),
               "sample": f"first {used} plates x 10 time steps ({tt:.1f} s), FP64 oracle, all host threads",
               "single_core_value": v1,
               "single_core_sample": f"first {used1} plates x 3 time steps ({tt1:.1f} s), one thread"}
    info = dict(plan.info)
    plan.close()
    extras = {}
    if rank == 0 and not args.no_extras:
        # the metric's accuracy condition and the other reported targets, each
        # with its own clock record (not part of the timed region above)
        if r32 is not None and args.precision == 32:
            extras["accuracy"] = accuracy_record(pkg, scs, run, r32)
        extras["plain_fp64"] = plain_fp64_record(pkg, value, e2e["value"] if e2e else None)
        extras["adjoint"] = adjoint_record(pkg)
    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": "DOF-steps/s", "n_gpus": ws, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f32" if args.precision == 32 else "f64", "data": "synthetic",
               "config": config, "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk.summary(),
               "gpu_launches": launches, "path": info["path"], "tile": info["tile"], "setup": setup, **extras}
        print(json.dumps(out))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
