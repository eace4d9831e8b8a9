#!/usr/bin/env python3
"""Benchmark of the GB300 HAMSTR steady ADI iteration.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload c2|c1]

A step is one pseudo-time iteration (computeRHS + ADI with msweep sweeps,
march.cpp:381-386) over one mesh.  The metric is cell-iterations per second
(cells x steps / time), whole job.  Workloads (seeded synthetic meshes; the
reference ships none):

  c2  NACA 0012 O-grid 512 x 128 (65,536 cells), WENO (order 5), CFL 20,
      msweep 2, Mach 0.5, alpha 1.25 deg -- the plain FP64 GPU drop-in
      configuration (quadrilaterals; the mixed tri/quad split is not applied)
  c1  NACA 0012 O-grid 128 x 32 (4,096 cells), MUSCL (order 3), CFL 10

gb300 arm ("value"): state resident in HBM, K captured steps timed with CUDA
events on the solver's stream, an L2 flush (write of 512 MiB) between timed
steps.  "e2e": the same steps through the C ABI with host buffers (pinned q
in, step, q and norms out) timed on the host clock.  Multi-GPU runs are
independent replicas (one mesh per rank, no collective on the data path).

reference arm: the reference algorithm on the host cores (the CPU oracle:
the reference library where it was compiled on this machine, else the C
restatement), one independent copy of the mesh per host thread.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "cell-iters/s"
UNIT = "cell-iter/s"
# Each workload: mesh (split = probability that a quad is split into two
# triangles, seeded), reconstruction order, CFL, sweeps, freestream, the
# chain end rule, and a CFL ramp (steps, CFL) run before the measured steps:
# WENO at CFL 20 on the half-split mesh diverges from an impulsive start.
WORKLOADS = {
    "c2": dict(ni=512, nj=128, split=0.5, seed=0, end_rule=1, order=5, CFL=20.0, msweep=2, Mach=0.5, alpha=1.25,
               ramp=((50, 2.0), (50, 5.0), (100, 10.0)),
               name="naca0012_ogrid_512x128_split50_weno5_cfl20_msweep2"),
    "c2quad": dict(ni=512, nj=128, split=0.0, seed=0, end_rule=0, order=5, CFL=20.0, msweep=2, Mach=0.5,
                   alpha=1.25, ramp=(), name="naca0012_ogrid_512x128_weno5_cfl20_msweep2"),
    "c1": dict(ni=128, nj=32, split=0.0, seed=0, end_rule=0, order=3, limiter=1, CFL=10.0, msweep=2, Mach=0.5,
               alpha=1.25, ramp=(), name="naca0012_ogrid_128x32_muscl_minmod_cfl10_msweep2"),
    "c3": dict(ni=1024, nj=256, split=0.3, seed=0, end_rule=1, order=3, limiter=2, CFL=10.0, msweep=2, Mach=0.8,
               alpha=1.25, ramp=((50, 2.0), (50, 5.0)),
               # the converged leg: both operators to L2 <= tol from the ramped state.
               # The reference's sweeps plateau near 2e-9 on this mesh; first-order
               # sweeps (same residual, so the same steady state) converge
               converge=dict(tol=1e-10, cap=20000, sweep_order=1),
               name="naca0012_ogrid_1024x256_split30_muscl_vanalbada_m08_cfl10_msweep2"),
}
# The batched form: `n` flow conditions (Mach, alpha drawn uniformly from a
# seed) on O-grids of four sizes assigned round-robin, all in one handle.
BATCH = {
    "c4": dict(meshes=((128, 32), (256, 64), (384, 96), (512, 128)), n=256, mach=(0.3, 0.85), alpha=(-2.0, 4.0),
               seed=0, order=1, CFL=10.0, msweep=2, precision="mixed",
               name="naca0012_batch256_meshes128x32-512x128_order1_cfl10_msweep2_fp32adi",
               # converged-solve leg: a subset small enough to finish in seconds
               converge=dict(n=16, meshes=((128, 32),), tol=1e-10, cap=6000)),
}
WORKLOADS.update({k: dict(v, batch=True) for k, v in BATCH.items()})

# The learned warm start: train on solver-generated converged states, then
# solve held-out conditions from the network's guess and from freestream.
WORKLOADS["c5"] = dict(warm=True, ni=256, nj=64, split=0.0, seed=0, end_rule=0, order=1, CFL=10.0, msweep=2,
                       Mach=0.5, alpha=1.25, ramp=(), train=2048, test=256, tol=1e-10, cap=15000, epochs=30,
                       batch=16384, lr=2e-3,
                       name="naca0012_256x64_order1_cfl10_warmstart_mlp5-256x3-4_train2048_test256")

# The target form against the plain FP64 drop-in, to convergence: held-out
# flow conditions (Mach U[0.3, 0.85], alpha U[-2, 4] deg, seeded) on the
# 128 x 32 O-grid, first order, CFL 10.  Three forms solve them through a
# ladder of computeRHS L2 tolerances:
#   plain FP64 drop-in: one handle per condition, freestream start, FP64
#     operator, conditions one after another;
#   batched FP32 operator from freestream: one handle for all conditions;
#   target form: batched, FP32 operator, started from the warm-start network
#     (trained on the GPU within the run on `train` solver-converged
#     conditions), the network's inference timed with the solve.
# At L2 <= 1e-10 a state still lies ~1e-3 from the fixed point, each start
# approaching from its own side, so the ladder runs on until every
# condition's fields agree with the plain FP64 drop-in's to 1e-8.
TARGET = dict(ni=128, nj=32, split=0.0, seed=0, end_rule=0, order=1, CFL=10.0, msweep=2, Mach=0.5, alpha=1.25,
              train=64, test=16, tols=(1e-10, 1e-12, 1e-13, 1e-14, 1e-15, 1e-16), cap=12000, epochs=40, batch=16384,
              lr=2e-3, repeats=3, accuracy=1e-8, name="naca0012_ogrid_128x32_order1_cfl10_msweep2_target_form")
L2_FLUSH_BYTES = 512 << 20


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")),
            int(os.environ.get("WORLD_SIZE", "1")))


def max_over_ranks(x: float, world: int) -> float:
    """The largest x over the ranks: a replicated job takes as long as its
    slowest rank (an all-reduce on the process group, NCCL on GPUs, gloo on
    the host)."""
    if world <= 1:
        return x
    import torch
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def make_case(wl: dict, rank: int) -> str:
    from hamstr_oop_gb300 import meshgen  # noqa: F401
    base = os.environ.get("HAMSTR_BENCH_DIR", "/tmp/hamstr_bench")
    d = os.path.join(base, "%s_r%d" % (wl["name"], rank))
    marker = os.path.join(d, "input.hamstr")
    if not os.path.exists(marker):
        meshgen.make_case(d, wl["ni"], wl["nj"], order=wl["order"], CFL=wl["CFL"], msweep=wl["msweep"],
                          Mach=wl["Mach"], alpha=wl["alpha"], nsteps=1, split=wl["split"], seed=wl["seed"])
    return d


LIMITER_NAMES = {0: "reference kappa-limiter", 1: "minmod", 2: "van Albada"}


def workload_config(wl: dict, sizes: dict, world: int) -> dict:
    """The `config` of a single-mesh workload's line, the same for both arms."""
    return {"workload": wl["name"], "cells": sizes["nCell"], "faces": sizes["nFace"], "chains": sizes["nChain"],
            "order": wl["order"], "msweep": wl["msweep"], "CFL": wl["CFL"], "mach": wl["Mach"],
            "alpha_deg": wl["alpha"], "parallelism": "replicas" if world > 1 else "single",
            "l2": "GPU arm: 512 MiB flush write between timed steps (untimed); host arm: state re-set between "
                  "timed steps (untimed)",
            "mesh": mesh_note(wl), "cfl_ramp_before_timing": [list(r) for r in wl["ramp"]],
            "limiter": LIMITER_NAMES[wl.get("limiter", 0)] if wl["order"] == 3 else None}


def mesh_note(wl: dict) -> str:
    if wl["split"] > 0:
        return ("NACA 0012 O-grid, each quad split into two triangles with probability %g (seed %d); "
                "chains from meshgen.extract_chains; extended chain end rule" % (wl["split"], wl["seed"]))
    return "NACA 0012 quadrilateral O-grid; reference chain end rule"


def open_case(wl: dict, case_dir: str):
    from hamstr_oop_gb300 import native
    case = native.Case(case_dir)
    case.set_option("chain_end_rule", wl["end_rule"])
    case.set_option("limiter", wl.get("limiter", 0))
    return case


def open_oracle(wl: dict, case_dir: str):
    from oracle import oracle
    o = oracle.OracleCase(case_dir, "port")
    o.set_option("chain_end_rule", wl["end_rule"])
    o.set_option("limiter", wl.get("limiter", 0))
    return o


def gemm_peak(size: int = 8192, reps: int = 5) -> dict:
    """The tcgen05 GEMM alone on a large square BF16 problem: the tensor
    roofline of the warm-start kernels."""
    import torch
    from hamstr_oop_gb300 import native
    L = native.load()
    A = torch.randn((size, size), device="cuda").to(torch.bfloat16)
    B = torch.randn((size, size), device="cuda").to(torch.bfloat16)
    C = torch.empty((size, size), dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        native._check(L.hamstr_mlp_gemm(A.data_ptr(), B.data_ptr(), size, size, size, 1, C.data_ptr(),
                                        err.data_ptr(), st))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        native._check(L.hamstr_mlp_gemm(A.data_ptr(), B.data_ptr(), size, size, size, 1, C.data_ptr(),
                                        err.data_ptr(), st))
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    ok = int(err.item()) == 0
    rel = float((C[:256, :256] - (A[:256].float() @ B[:256].float().T)).abs().max() /
                (A[:256].float() @ B[:256].float().T).abs().max())
    peaks = measured_peaks()
    tf = 2.0 * size ** 3 / (ms * 1e-3) / 1e12
    return {"M": size, "N": size, "K": size, "ms": ms, "tflops": tf, "ok": ok, "max_rel_err_vs_fp32": rel,
            "peak_tflops": peaks.get("bf16_tflops"), "frac": tf / peaks["bf16_tflops"] if peaks.get("bf16_tflops") else None}


def run_warmstart(args, wl, rank, local_rank, world):
    """C5: data generation with the batched solver, training on the tensor
    cores, and the held-out comparison (warm vs freestream start)."""
    import numpy as np
    import torch
    from hamstr_oop_gb300 import native, warmstart
    torch.cuda.set_device(local_rank)
    native.load()
    ntrain = args.c5_train or wl["train"]
    ntest = args.c5_test or wl["test"]
    case_dir = make_case(wl, 0)
    case = open_case(wl, case_dir)
    t0 = time.perf_counter()
    train_conds = warmstart.conditions(ntrain, seed=0)
    data = warmstart.solve_batch(case, train_conds, wl["tol"], wl["cap"])
    t_data = time.perf_counter() - t0
    model, trep = warmstart.train(case, data["q"], train_conds, epochs=wl["epochs"], batch=wl["batch"], lr=wl["lr"])
    test_conds = warmstart.conditions(ntest, seed=1)
    ev = warmstart.evaluate(case, model, test_conds, wl["tol"], wl["cap"])
    # the plain FP64 drop-in on the first held-out conditions: the baseline
    # and the reference converged state for the warm-started batched form
    nplain = min(8, ntest)
    plain = warmstart.plain_fp64_solves(case, test_conds[:nplain], wl["tol"], wl["cap"])
    qw = ev.pop("_q_warm")
    sw = ev.pop("_steps_warm")
    rel = [float(np.max(np.abs(a - b)) / np.max(np.abs(b))) for a, b in zip(qw[:nplain], plain["q"])]
    plain_cmp = {"conditions": nplain, "solves_per_s": plain["solves_per_s"], "seconds": plain["seconds"],
                 "steps_mean": float(np.mean(plain["steps"])), "all_converged": plain["all_converged"],
                 "warm_batched_steps_mean": float(np.mean(sw[:nplain])),
                 "warm_batched_vs_plain_fp64_max_rel": max(rel), "warm_batched_vs_plain_fp64_rel": rel,
                 "speedup_warm_batched_vs_plain_fp64": ev["solves_per_s_warm"] / plain["solves_per_s"]}
    # at L2 <= 1e-10 each path stops ~1e-3 (relative, max norm) short of the fixed point, in its own
    # direction; tightening the tolerance shows both forms reach the FP64 steady state
    ntight, tol_t = min(4, ntest), 1e-15
    plain_t = warmstart.plain_fp64_solves(case, test_conds[:ntight], tol_t, 15000)
    warm_t = warmstart.solve_batch(case, test_conds[:ntight], tol_t, 15000, q0=model.predict(test_conds[:ntight]))
    rel_t = [float(np.max(np.abs(a - b)) / np.max(np.abs(b))) for a, b in zip(warm_t["q"], plain_t["q"])]
    plain_cmp["tight_tolerance"] = {"tol": tol_t, "conditions": ntight, "all_converged":
                                    bool(plain_t["all_converged"] and warm_t["all_converged"]),
                                    "steps_plain_fp64": plain_t["steps"], "steps_warm_batched": warm_t["steps"],
                                    "warm_batched_vs_plain_fp64_max_rel": max(rel_t),
                                    "warm_batched_vs_plain_fp64_rel": rel_t}
    peak = gemm_peak()
    peaks = measured_peaks()
    trep.pop("loss_curve", None)
    return {"metric": "converged solves/s (L2 <= 1e-10), held-out conditions, warm start",
            "value": ev["solves_per_s_warm"], "unit": "solves/s", "n_gpus": 1, "steps": None, "warmup": None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64 residual, f32 Jacobian/ADI; network bf16 with f32 accumulation", "data": "synthetic",
            "config": {"workload": wl["name"], "mesh": [wl["ni"], wl["nj"]], "train_conditions": ntrain,
                       "test_conditions": ntest, "order": wl["order"], "CFL": wl["CFL"], "msweep": wl["msweep"],
                       "tol": wl["tol"], "cap": wl["cap"]},
            "freestream_start": {"solves_per_s": ev["solves_per_s_freestream"], "steps_mean": ev["steps_freestream_mean"],
                                 "seconds": ev["seconds_freestream"]},
            "warm_start": ev, "plain_fp64_drop_in": plain_cmp, "training": trep,
            "data_generation": {"conditions": ntrain, "seconds": t_data, "all_converged": data["all_converged"],
                                "steps_mean": float(np.mean(data["steps"]))},
            "roofline": {"kernel": "tcgen05 bf16 GEMM (mlp_gemm.cu)", "bound": "tensor",
                         "achieved": peak["tflops"], "peak": peaks.get("bf16_tflops"), "unit": "TFLOP/s",
                         "frac": peak["frac"], "traffic": None, "gemm": peak,
                         "training_gemm_tflops": trep["gemm_tflops"]}}


def batch_conditions(b: dict, n: int = None, meshes=None):
    """[(mesh index, Mach, alpha)] of the batch, seeded."""
    import numpy as np
    n = n or b["n"]
    meshes = meshes or b["meshes"]
    rng = np.random.default_rng(b["seed"])
    mach = rng.uniform(b["mach"][0], b["mach"][1], n)
    alpha = rng.uniform(b["alpha"][0], b["alpha"][1], n)
    return [(k % len(meshes), float(mach[k]), float(alpha[k])) for k in range(n)]


def batch_mesh_dirs(b: dict, meshes) -> list:
    from hamstr_oop_gb300 import meshgen
    base = os.environ.get("HAMSTR_BENCH_DIR", "/tmp/hamstr_bench")
    out = []
    for ni, nj in meshes:
        d = os.path.join(base, "batch_%dx%d_o%d" % (ni, nj, b["order"]))
        if not os.path.exists(os.path.join(d, "input.hamstr")):
            meshgen.make_case(d, ni, nj, order=b["order"], CFL=b["CFL"], msweep=b["msweep"], nsteps=1)
        out.append(d)
    return out


def batch_cases(b: dict, n: int = None, meshes=None) -> list:
    """Host cases of the batch: one read per mesh, cloned per condition."""
    from hamstr_oop_gb300 import native
    meshes = meshes or b["meshes"]
    base = [native.Case(d) for d in batch_mesh_dirs(b, meshes)]
    out = []
    for m, mach, alpha in batch_conditions(b, n, meshes):
        c = base[m].clone()
        c.set_flow(mach, alpha)
        out.append(c)
    return out


def run_batch(args, wl, rank, local_rank, world):
    """The batched form: every condition in one handle, one graph per step."""
    import numpy as np
    import torch
    from hamstr_oop_gb300 import native
    torch.cuda.set_device(local_rank)
    native.load()
    t_setup = time.perf_counter()
    cases = batch_cases(wl)
    g = native.GpuSolver.batch(cases)
    t_setup = time.perf_counter() - t_setup
    nc = g.sizes["nCell"]
    g.set_precision(wl["precision"] == "mixed")
    if args.profile_steps:
        # a plain run for ncu: N captured steps after two warm-up steps
        if args.shape:
            g.set_shape(**parse_shape(args.shape))
        g.enqueue_steps(2)
        g.sync()
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        g.enqueue_steps(args.profile_steps)
        g.sync()
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        if rank == 0:
            print(json.dumps({"profile_steps": args.profile_steps, "workload": wl["name"], "conditions": len(cases),
                              "cells": nc, "launches_per_step": g.launches_per_step()}), flush=True)
        g.close()
        return None
    tune = g.autotune(reps=2)
    hs = torch.cuda.ExternalStream(g.stream)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    g.enqueue_steps(max(args.warmup, 3))
    g.sync()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local_rank)
    sampler.start()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with torch.cuda.stream(hs):
        for k in range(args.steps):
            flush.fill_(float(k))
            starts[k].record(hs)
            g.enqueue_steps(1)
            ends[k].record(hs)
    g.sync()
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = max_over_ranks(sum(s.elapsed_time(e) for s, e in zip(starts, ends)), world)
    value = world * nc * args.steps / (ms * 1e-3)
    prof = g.profile_step(reps=2) if rank == 0 else {}
    # the same batch with the FP64 operator, for comparison
    g.set_precision(False)
    g.enqueue_steps(2)
    g.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(hs):
        e0.record(hs)
        g.enqueue_steps(max(args.steps // 2, 1))
        e1.record(hs)
    g.sync()
    fp64_ms = e0.elapsed_time(e1) / max(args.steps // 2, 1)
    # end to end: q of all conditions in from pinned host memory, one step,
    # q and the per-condition norms out
    g.set_precision(wl["precision"] == "mixed")
    qhost = torch.empty(4 * nc, dtype=torch.float64, pin_memory=True)
    qnp = qhost.numpy()
    qnp[:] = g.get("q")
    e2e_steps = max(1, min(args.steps, 5))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        g.step_host(qnp, qnp)
        g.instance_norms()
    e2e_s = time.perf_counter() - t0
    out = None
    if rank == 0:
        conv = batch_converged(wl) if not args.no_converge else None
        ninst = g.n_instances
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64 residual, f32 Jacobian/ADI" if wl["precision"] == "mixed" else "f64",
               "data": "synthetic",
               "config": {"workload": wl["name"], "conditions": ninst, "cells": nc, "meshes": [list(m) for m in wl["meshes"]],
                          "mach": list(wl["mach"]), "alpha_deg": list(wl["alpha"]), "order": wl["order"],
                          "CFL": wl["CFL"], "msweep": wl["msweep"], "parallelism": "one batched handle",
                          "l2": "512 MiB flush write between timed steps (untimed)", "setup_s": t_setup},
               "e2e": {"value": world * nc * e2e_steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 32 * nc,
                       "d2h_bytes_per_step": 32 * nc + 32 * ninst, "steps": e2e_steps},
               "fp64_operator_ms_per_step": fp64_ms,
               "kernel_ms_per_step": {k: round(v[0], 4) for k, v in prof.items()},
               "converged": conv, "clocks": clocks, "autotune": tune,
               "gpu_launches": g.launches_per_step() * args.steps}
    g.close()
    return out


def batch_converged(wl: dict) -> dict:
    """Time to L2 <= tol for a subset of the batch's conditions: the batched
    form (one handle, its precision) against the plain FP64 drop-in solving
    the same conditions one after another."""
    import numpy as np
    import torch
    from hamstr_oop_gb300 import native
    cv = wl["converge"]
    cases = batch_cases(wl, cv["n"], cv["meshes"])
    out = {"conditions": cv["n"], "meshes": [list(m) for m in cv["meshes"]], "tol": cv["tol"], "cap": cv["cap"]}
    g = native.GpuSolver.batch(cases)
    g.set_precision(wl["precision"] == "mixed")
    g.autotune(reps=2)
    g.march(2, 0.0)
    g.set("q", np.concatenate([c.get("q") for c in cases]))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist, ok = g.march(cv["cap"], cv["tol"])
    dt = time.perf_counter() - t0
    first = [int(np.argmax(hist[:, k, 0] <= cv["tol"])) if (hist[:, k, 0] <= cv["tol"]).any() else None
             for k in range(cv["n"])]
    qb = g.get("q").reshape(-1, 4)
    cell0 = g.instance_cells()
    fb = g.batch_forces()
    g.close()
    out["batched"] = {"all_converged": ok, "steps": int(hist.shape[0]), "seconds": dt,
                      "solves_per_s": cv["n"] / dt if ok else None,
                      "steps_per_condition": first}
    # plain FP64 drop-in, one condition at a time
    t_plain, steps_plain, worst = 0.0, [], 0.0
    dcl = 0.0
    for k, c in enumerate(cases):
        s = native.GpuSolver(c)
        s.march(2, 0.0)
        s.set("q", c.get("q"))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        h, okk = s.march(cv["cap"], cv["tol"])
        t_plain += time.perf_counter() - t0
        steps_plain.append(int(h.shape[0]) if okk else None)
        q64 = s.get("q").reshape(-1, 4)
        worst = max(worst, float(np.max(np.abs(qb[cell0[k]:cell0[k + 1]] - q64)) / np.max(np.abs(q64))))
        dcl = max(dcl, abs(fb[k, 3] - s.forces()["CL"]))
        s.close()
    out["plain_fp64_sequential"] = {"seconds": t_plain, "solves_per_s": cv["n"] / t_plain,
                                    "steps_per_condition": steps_plain}
    out["speedup_batched_vs_plain"] = t_plain / dt
    out["batched_vs_plain_at_tol"] = {"max_abs_over_max_q": worst, "max_dCL": dcl,
                                      "note": "both stopped at the same L2 tolerance"}
    return out


def time_oracle_steps(cases: list, q0: list, steps: int) -> float:
    """Seconds for `steps` pseudo-time steps on every case (one host thread
    each), each step taken from the state q0; the resets are not timed."""
    from oracle import oracle
    total = 0.0
    for _ in range(steps):
        for c, q in zip(cases, q0):
            c.set("q", q)
        t0 = time.perf_counter()
        oracle.march_replicas(cases, 1)
        total += time.perf_counter() - t0
    return total


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index, self.proc, self.lines = index, None, []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "bf16_tflops": float(d.get("bf16_tflops", 1900.0)),
                "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


# FP64 issue peak of the GPU, warp instructions per second: an independent-
# chain DADD loop over all SMs issues 15.8 G warp instructions/s whatever the
# number of active lanes
FP64_WARP_INSTR_PER_S = 15.8e9

# Per-launch figures of the FP64 kernels on the c2 workload (512 x 128 half
# split, WENO, after the CFL ramp, the autotuner's shape on this mesh) from
# one ncu capture of `bench.py --profile-steps 2 --shape ...` (two steps):
#   dram_bytes     dram__bytes_read.sum + dram__bytes_write.sum
#   fp64_inst      smsp__inst_executed_pipe_fp64.sum (warp instructions)
# Kernels launched more than once a step (adi_solve: two waves, two sweeps;
# the per-sweep kernels) give the mean of their launches.
NCU_PER_LAUNCH = {
    "naca0012_ogrid_512x128_split50_weno5_cfl20_msweep2": {
        "recon5": {"dram_bytes": 155.0e6, "fp64_inst": 2898203},
        "rhs_face": {"dram_bytes": 16.8e6, "fp64_inst": 2620380},
        "adi_assemble": {"dram_bytes": 55.1e6, "fp64_inst": 873663},
        "adi_factor": {"dram_bytes": 62.7e6, "fp64_inst": 2700985},   # with the first wave's first solve
        "adi_solve": {"dram_bytes": 20.1e6, "fp64_inst": 300775},
        "lin_recon5": {"dram_bytes": 209.2e6, "fp64_inst": 2554292},
        "lin_face": {"dram_bytes": 55.2e6, "fp64_inst": 328832},
        "lin_cell": {"dram_bytes": 15.6e6, "fp64_inst": 343608},
    },
}


def dataflow_bytes(sizes: dict, msweep: int, jac_bytes: int = 256) -> dict:
    """Compulsory HBM bytes of one pseudo-time step in the reference's
    dataflow, each array read or written once per pass (FP64 vectors of 32
    B/cell, face Jacobians J B/face, face geometry 28 B/face), by component:
      computeRHS + ADI init: q read, r and sigma written, geometry, J written;
        r scaled and copied to r0, dq zeroed (ADI.cpp:40-49)
      line solves, per sweep: J read by the block assembly; r, sigma read and
        the solution written per colour (ADI.cpp:62-244)
      dq += r, per sweep (ADI.cpp:247-248)
      linear residual, per sweep: q, dq, r0, sigma read, r written; J and
        geometry (computeLinearRHS.cpp:13-371)
      update q += dq (ADI.cpp:258-264)"""
    nc, nf, J, s = sizes["nCell"], sizes["nFace"], jac_bytes, msweep
    comp = {"computeRHS": 72 * nc + (28 + J) * nf + 136 * nc,
            "line_solves_per_sweep": 144 * nc + J * nf,
            "dq_update_per_sweep": 96 * nc,
            "linear_rhs_per_sweep": 136 * nc + (J + 28) * nf,
            "update": 96 * nc}
    comp["step"] = (comp["computeRHS"] + comp["update"] +
                    s * (comp["line_solves_per_sweep"] + comp["dq_update_per_sweep"] + comp["linear_rhs_per_sweep"]))
    return comp


# the dataflow component each FP64 kernel belongs to, and its launches per
# component pass (the component's bytes are credited to the kernel that
# carries most of its time)
KERNEL_COMPONENT = {"recon5": "computeRHS", "rhs_face": "computeRHS", "rhs_cell": "computeRHS",
                    "adi_assemble": "line_solves_per_sweep", "adi_factor": "line_solves_per_sweep",
                    "adi_solve": "line_solves_per_sweep", "dq_update": "dq_update_per_sweep",
                    "lin_recon5": "linear_rhs_per_sweep", "lin_face": "linear_rhs_per_sweep",
                    "lin_cell": "linear_rhs_per_sweep"}


def implementation_bytes(kernel: str, lay: dict, sizes: dict, order: int) -> float:
    """HBM bytes one launch of this implementation moves with each of its
    arrays touched once (its own layout: kept WENO values, factor records),
    beside the reference dataflow's compulsory bytes."""
    nc, ns, nr = sizes["nCell"], lay["nSlot"], lay["nRow"]
    npr = lay["nPeriodicRows"]
    sten = {1: 2, 3: 4, 5: 6}[order]
    if kernel == "recon5":
        # order 5, implicit: slot record 16, stencil entries 16 (shared by neighbours), q once
        # per cell; writes the slot's two states 64 and the kept WENO values 8 * 144
        return ns * (16 + 16 + 64 + 8 * 144) + nc * 32
    if kernel == "lin_recon5":
        # slot record 16, stencil 16, kept WENO values 8 * 144, dq once per cell; writes 64
        return ns * (16 + 16 + 8 * 144 + 64) + nc * 32
    if kernel == "rhs_face" and order == 5:
        # slot record 16, normal 16, the states recon5 left 64; writes flux 32, spec 8, ff 256
        return ns * (16 + 16 + 64 + 32 + 8 + 256)
    if kernel == "lin_face" and order == 5:
        # slot record 16, the linearised states 64, ff 256; writes flux 32
        return ns * (16 + 64 + 256 + 32)
    if kernel == "rhs_face":
        # slot record 32 + normal 16 + stencil entries 16*sten/2 (shared by neighbours)
        # + q once per cell; writes flux 32, spec 8, ff 256
        return ns * (32 + 16 + 8 * sten + 32 + 8 + 256) + nc * 32
    if kernel == "lin_face":
        return ns * (32 + 8 * sten + 256 + 32) + nc * 64
    if kernel == "adi_factor":
        # ff once per slot, dtfac, row ops/cells 56 B; writes A, LU, C' (+ a', c_N for periodic rows)
        return ns * 256 + nc * 8 + nr * 56 + (nr - npr) * 8 * 48 + npr * 8 * 80
    if kernel == "adi_solve":
        # per wave launch: rows of that wave read their factors; averaged over waves
        per_row_open, per_row_per = 8 * 48 + 64 + 64, 8 * 80 + 64 + 64
        return ((nr - npr) * per_row_open + npr * per_row_per) / max(lay["nWave"], 1)
    if kernel == "rhs_cell":
        return ns * 40 + nc * (4 + 16 + 96 + 16)
    if kernel == "lin_cell":
        return ns * 32 + nc * (4 + 16 + 8 + 32 + 32 + 32)
    if kernel == "dq_update":
        return nc * 96
    return 0.0


def roofline_of(dom: str, prof: dict, lay: dict, sizes: dict, wl: dict, step_ms: float) -> dict:
    """The roofline of the dominant kernel and of the whole step against
    HBM, with the reference dataflow's compulsory bytes (dataflow_bytes):
    the dominant kernel is credited with its whole component's bytes per
    launch.  Beside it, the FP64 issue rate the path is bound by, from the
    kernel's FP64 warp instructions (ncu) over its CUDA-event time."""
    peaks = measured_peaks()
    per_step = {k: v[0] for k, v in prof.items()}
    avg_ms = per_step[dom] / max(prof[dom][1], 1)
    flow = dataflow_bytes(sizes, wl["msweep"])
    comp = KERNEL_COMPONENT.get(dom)
    alg = flow[comp] if comp else None
    achieved = alg / (avg_ms * 1e-3) / 1e9 if (alg and avg_ms > 0) else None
    ncu = NCU_PER_LAUNCH.get(wl["name"], {}).get(dom, {})
    step_gbs = flow["step"] / (step_ms * 1e-3) / 1e9
    fp64 = None
    if ncu.get("fp64_inst"):
        rate = ncu["fp64_inst"] / (avg_ms * 1e-3)
        fp64 = {"warp_instructions_per_launch": ncu["fp64_inst"], "achieved_per_s": rate,
                "peak_per_s": FP64_WARP_INSTR_PER_S, "frac": rate / FP64_WARP_INSTR_PER_S,
                "source": "ncu smsp__inst_executed_pipe_fp64.sum per launch; CUDA-event launch time"}
    return {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": (achieved / peaks["hbm_gbs"]) if achieved else None,
            "traffic": ncu.get("dram_bytes"),
            "byte_model": "reference dataflow, compulsory bytes (FP64 vectors 32 B/cell, J = 256 B/face, geometry "
                          "28 B/face); the kernel is credited with its component '%s'" % comp,
            "algorithmic_bytes_per_launch": alg,
            "implementation_bytes_per_launch": implementation_bytes(dom, lay, sizes, wl["order"]),
            "avg_launch_ms": avg_ms, "peak_source": peaks["source"] + " HBM copy bandwidth",
            "step": {"bytes": flow["step"], "ms": step_ms, "achieved": step_gbs,
                     "frac": step_gbs / peaks["hbm_gbs"]},
            "fp64_issue": fp64,
            "kernel_ms_per_step": {k: round(v, 4) for k, v in per_step.items()}}


def tune_summary(rep: dict) -> dict:
    """The autotuner's choice, its step time, and the best time with each
    value of each launch-shape key (what each choice is worth)."""
    cands = rep["candidates"]
    out = {"best": rep["best"], "candidates": len(cands), "ms_best": min(c["ms"] for c in cands), "ms_by_value": {}}
    for k in rep["best"]:
        vals = sorted({c[k] for c in cands})
        if len(vals) > 1:
            out["ms_by_value"][k] = {str(v): round(min(c["ms"] for c in cands if c[k] == v), 4) for v in vals}
    return out


def tune_or_set(gpu, shape: str) -> dict:
    """Autotune, or set the given launch shape (no tuning)."""
    if shape:
        gpu.set_shape(**parse_shape(shape))
        return {"best": gpu.shape(), "set_by": "--shape"}
    return tune_summary(gpu.autotune(reps=2))


def parse_shape(text: str) -> dict:
    """'key=value,...' into hamstr_gpu_set_shape keywords."""
    out = {}
    for item in text.split(","):
        k, v = item.split("=")
        out[k.strip()] = int(v)
    return out


def run_gpu(args, wl, rank, local_rank, world):
    import numpy as np
    import torch
    from hamstr_oop_gb300 import native

    torch.cuda.set_device(local_rank)
    native.load()
    case_dir = make_case(wl, rank)
    case = open_case(wl, case_dir)
    gpu = native.GpuSolver(case)
    sizes = case.sizes
    for n, cfl in wl["ramp"]:
        gpu.set_cfl(cfl)
        gpu.enqueue_steps(n)
    gpu.set_cfl(wl["CFL"])
    gpu.sync()
    if args.profile_steps:
        # a plain run of the workload for ncu: ramp, then N captured steps
        gpu.set_precision(args.profile_precision == "mixed")
        if args.shape:
            gpu.set_shape(**parse_shape(args.shape))
        gpu.enqueue_steps(1)   # the graph is captured and warm before the profiled range
        gpu.sync()
        # only the profiled steps lie between profiler start and stop (for
        # `ncu --profile-from-start off`; without a profiler these do nothing)
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        gpu.enqueue_steps(args.profile_steps)
        gpu.sync()
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        if rank == 0:
            print(json.dumps({"profile_steps": args.profile_steps, "precision": args.profile_precision,
                              "workload": wl["name"], "ramp_steps": sum(n for n, _ in wl["ramp"]),
                              "launches_per_step": gpu.launches_per_step()}), flush=True)
        return None
    lay = gpu.layout()
    nc = sizes["nCell"]
    hs = torch.cuda.ExternalStream(gpu.stream)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    # the state the timed steps start from (after the CFL ramp): the host
    # legs time their steps from it too
    q_timed = gpu.get("q")
    # launch shapes from the autotuner (or --shape), then warm-up (W >= 3 steps)
    tune64 = tune_or_set(gpu, args.shape)
    gpu.enqueue_steps(max(args.warmup, 1))
    gpu.sync()

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local_rank)
    sampler.start()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    t0 = time.perf_counter()
    with torch.cuda.stream(hs):
        for k in range(args.steps):
            flush.fill_(float(k))                 # L2 flush, outside the timed events
            starts[k].record(hs)
            gpu.enqueue_steps(1)
            ends[k].record(hs)
    gpu.sync()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    ms = max_over_ranks(sum(s.elapsed_time(e) for s, e in zip(starts, ends)), world)
    if world > 1:
        torch.distributed.barrier()
    value = world * nc * args.steps / (ms * 1e-3)

    # order 5: the same steps without the kept WENO linearisation values
    # (each sweep recomputes them from q instead of reading 1152 B per face)
    keep_trade = None
    if wl["order"] == 5:
        shape0 = gpu.shape()
        gpu.set_shape(weno_keep=0)
        gpu.enqueue_steps(max(args.warmup, 1))
        gpu.sync()
        ks = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ke = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        with torch.cuda.stream(hs):
            for k in range(args.steps):
                flush.fill_(float(k))
                ks[k].record(hs)
                gpu.enqueue_steps(1)
                ke[k].record(hs)
        gpu.sync()
        nokeep_ms = sum(s.elapsed_time(e) for s, e in zip(ks, ke)) / args.steps
        keep_trade = {"kept_ms_per_step": ms / args.steps, "recomputed_ms_per_step": nokeep_ms,
                      "kept_bytes_per_face": 1152}
        gpu.set_shape(**shape0)

    # the mixed-precision form (FP64 residual, FP32 operator) on the same case
    gpu.set_precision(True)
    tunemx = tune_or_set(gpu, args.shape)
    gpu.enqueue_steps(max(args.warmup, 1))
    gpu.sync()
    mstarts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    mends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with torch.cuda.stream(hs):
        for k in range(args.steps):
            flush.fill_(float(k))
            mstarts[k].record(hs)
            gpu.enqueue_steps(1)
            mends[k].record(hs)
    gpu.sync()
    mixed_ms = sum(s.elapsed_time(e) for s, e in zip(mstarts, mends))
    mixed_prof = gpu.profile_step(reps=3) if rank == 0 else {}
    gpu.set_precision(False)

    # end-to-end through the C ABI with host buffers
    qhost = torch.empty(4 * nc, dtype=torch.float64, pin_memory=True)
    qnp = qhost.numpy()
    qnp[:] = gpu.get("q")
    e2e_steps = max(1, min(args.steps, 20))
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        gpu.step_host(qnp, qnp)   # q in from the host buffer, one step, q back into it
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    e2e = {"value": world * nc * e2e_steps / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": 32 * nc, "d2h_bytes_per_step": 32 * nc + 32, "steps": e2e_steps}

    out = None
    if rank == 0:
        prof = gpu.profile_step(reps=3)
        per_step = {k: v[0] for k, v in prof.items()}
        dom = max(per_step, key=per_step.get)
        launches = prof[dom][1]
        avg_ms = per_step[dom] / max(launches, 1)
        roofline = roofline_of(dom, prof, lay, sizes, wl, ms / args.steps)
        cpu = cpu_baseline(wl, case_dir, nc, q_timed) if (world == 1 and not args.no_cpu) else None
        conv = target_form() if not args.no_converge else None
        conv_wl = (converged_errors(wl, case_dir) if (wl.get("converge") and not args.no_converge) else None)
        mixed = {"value": world * nc * args.steps / (mixed_ms * 1e-3), "unit": UNIT,
                 "ms_per_step": mixed_ms / args.steps,
                 "note": "FP64 residual (bit-identical to the reference), FP32 Jacobians, ADI and linear "
                         "residual; converges to the FP64 steady state (tests/test_gpu_mixed.py)",
                 "kernel_ms_per_step": {k: round(v[0], 4) for k, v in mixed_prof.items()},
                 "autotune": tunemx}
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(wl, sizes, world),
            "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks,
            "mixed_precision": mixed, "target_form": conv, "autotune": tune64, "weno_keep_trade": keep_trade,
            "converged": conv_wl,
            "gpu_launches": gpu.launches_per_step() * args.steps,
            "wall_s_timed_region": wall,
        }
    gpu.close()
    return out


def ladder_march(g, tols, cap: int, n_inst: int) -> list:
    """March handle g through the tolerance ladder (each march stops at the
    first step whose computeRHS L2 meets the tolerance, every instance of a
    batch frozen at its own such step): per tolerance the cumulative seconds,
    the steps of each instance and its state."""
    import numpy as np
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out, done = [], 0
    own = [0] * n_inst        # steps each instance took (a batch freezes an instance at its own stop)
    for tol in tols:
        hist, ok = g.march(cap - done, tol)
        secs = time.perf_counter() - t0
        h = hist if hist.ndim == 3 else hist[:, None, :]
        for k in range(n_inst):
            hit = np.flatnonzero(h[:, k, 0] <= tol)
            own[k] += int(hit[0]) + 1 if hit.size else h.shape[0]
        steps = list(own)
        done += h.shape[0]
        out.append({"tol": tol, "seconds": secs, "converged": bool(ok), "steps": steps, "q": g.get("q")})
        if not ok or done >= cap:
            break
    return out


def target_form() -> dict:
    """The benchmark spec's target form (batched, FP32 operator, warm start) and
    the batched FP32 operator from freestream, against the plain FP64
    drop-in one condition at a time: solves/s at every tolerance of the
    ladder, and each condition's max |q - q_fp64| / max |q_fp64|."""
    import numpy as np
    import torch
    from hamstr_oop_gb300 import native, warmstart
    c = TARGET
    case_dir = make_case(c, 0)
    case = open_case(c, case_dir)
    nc = case.sizes["nCell"]
    tols, cap = list(c["tols"]), c["cap"]
    # the network: trained on the GPU here, on solver-converged conditions
    t0 = time.perf_counter()
    train_conds = warmstart.conditions(c["train"], seed=0)
    data = warmstart.solve_batch(case, train_conds, tols[0], cap)
    t_data = time.perf_counter() - t0
    model, trep = warmstart.train(case, data["q"], train_conds, epochs=c["epochs"], batch=c["batch"], lr=c["lr"])
    trep.pop("loss_curve", None)
    conds = warmstart.conditions(c["test"], seed=1)

    shapes = {}   # the launch shapes the autotuner picked for each form

    def batched(warm: bool):
        cs = []
        for m, a in conds:
            h = case.clone()
            h.set_flow(m, a)
            cs.append(h)
        g = native.GpuSolver.batch(cs)
        g.set_precision(True)
        # the default launch shape: the autotuner's pick, timed over a few
        # steps with every condition live, ran slower over whole marches
        # (4.27 against 4.55 solves/s at 1e-16), so the batched forms keep
        # the default while the plain drop-in gets its tuned shape
        shapes["batched_fp32_op_" + ("warm" if warm else "freestream")] = g.shape()
        g.march(2, 0.0)                                   # graph capture, warm-up (untimed)
        fs = np.concatenate([h.get("q") for h in cs])
        runs = []
        for _ in range(c["repeats"]):
            torch.cuda.synchronize()
            tp = time.perf_counter()
            q0 = np.concatenate([q.ravel() for q in model.predict(conds)]) if warm else fs
            g.set("q", q0)
            t_start = time.perf_counter() - tp            # inference and the copy in, charged to the solve
            lad = ladder_march(g, tols, cap, len(conds))
            for r in lad:
                r["seconds"] += t_start
            runs.append(lad)
        cell0 = g.instance_cells()
        g.close()
        return runs, cell0

    warm_runs, cell0 = batched(True)
    cold_runs, _ = batched(False)
    # the plain FP64 drop-in, one condition after another
    plain = []
    shape64 = None   # the FP64 launch shape, tuned on the first condition (the mesh is the same for all)
    for m, a in conds:
        h = case.clone()
        h.set_flow(m, a)
        g = native.GpuSolver(h)
        if shape64 is None:
            g.autotune(reps=6)
            shape64 = g.shape()
            shapes["plain_fp64"] = shape64
        else:
            g.set_shape(**shape64)
        g.march(2, 0.0)
        g.set("q", h.get("q"))
        plain.append(ladder_march(g, tols, cap, 1))
        g.close()

    def rel(qa, qb):
        qa, qb = qa.reshape(-1, 4), qb.reshape(-1, 4)
        return float(np.max(np.abs(qa - qb)) / np.max(np.abs(qb)))

    ladder = []
    for i, tol in enumerate(tols):
        if any(len(p) <= i for p in plain) or any(len(r) <= i for r in warm_runs + cold_runs):
            break
        p_secs = sum(p[i]["seconds"] for p in plain)
        p_ok = all(p[i]["converged"] for p in plain)
        row = {"tol": tol, "plain_fp64": {"seconds": p_secs, "solves_per_s": len(conds) / p_secs,
                                          "steps_mean": float(np.mean([p[i]["steps"][0] for p in plain])),
                                          "all_converged": p_ok}}
        for label, runs in (("batched_fp32_op_warm", warm_runs), ("batched_fp32_op_freestream", cold_runs)):
            secs = sorted(r[i]["seconds"] for r in runs)
            last = runs[-1][i]
            qb = last["q"].reshape(-1, 4)
            rels = [rel(qb[cell0[k]:cell0[k + 1]], plain[k][i]["q"]) for k in range(len(conds))]
            med = secs[len(secs) // 2]
            row[label] = {"seconds_median": med, "seconds_all": secs, "solves_per_s": len(conds) / med,
                          "steps_mean": float(np.mean(last["steps"])), "all_converged": bool(last["converged"]),
                          "max_rel_vs_plain_fp64": max(rels), "rel_vs_plain_fp64": rels,
                          "speedup_vs_plain_fp64": p_secs / med}
        ladder.append(row)
    acc = c["accuracy"]

    def first_meeting(label):
        for r in ladder:
            if (r[label]["max_rel_vs_plain_fp64"] <= acc and r["plain_fp64"]["all_converged"]
                    and r[label]["all_converged"]):
                return r
        return None
    pick = first_meeting("batched_fp32_op_warm")
    cold = first_meeting("batched_fp32_op_freestream")
    out = {"workload": c["name"], "cells_per_condition": nc, "conditions": len(conds),
           "conditions_distribution": "Mach U[0.3, 0.85], alpha U[-2, 4] deg, seed 1 (held out)",
           "cap": cap, "accuracy": acc, "ladder": ladder, "launch_shapes": shapes,
           "warm_start": {"training_conditions": c["train"], "data_generation_seconds": t_data,
                          "data_all_converged": data["all_converged"], "training": trep},
           "tol": pick["tol"] if pick else None,
           "max_rel_vs_fp64": pick["batched_fp32_op_warm"]["max_rel_vs_plain_fp64"] if pick else None,
           "solves_per_s": pick["batched_fp32_op_warm"]["solves_per_s"] if pick else None,
           "plain_fp64_solves_per_s": pick["plain_fp64"]["solves_per_s"] if pick else None,
           "speedup_vs_plain_fp64": pick["batched_fp32_op_warm"]["speedup_vs_plain_fp64"] if pick else None,
           "without_warm_start": {
               "tol": cold["tol"] if cold else None,
               "max_rel_vs_fp64": cold["batched_fp32_op_freestream"]["max_rel_vs_plain_fp64"] if cold else None,
               "solves_per_s": cold["batched_fp32_op_freestream"]["solves_per_s"] if cold else None,
               "plain_fp64_solves_per_s": cold["plain_fp64"]["solves_per_s"] if cold else None,
               "speedup_vs_plain_fp64": cold["batched_fp32_op_freestream"]["speedup_vs_plain_fp64"] if cold else None},
           "note": "tol: the loosest tolerance of the ladder at which every condition's warm-started batched "
                   "FP32-operator state is within `accuracy` (max |q - q_fp64| / max |q_fp64|) of the plain FP64 "
                   "drop-in's state at the same tolerance; the plain drop-in's steps are the oracle's bit for bit"}
    if ladder:
        first = ladder[0]
        out["at_1e-10"] = {"solves_per_s": first["batched_fp32_op_warm"]["solves_per_s"],
                           "plain_fp64_solves_per_s": first["plain_fp64"]["solves_per_s"],
                           "max_rel_vs_fp64": first["batched_fp32_op_warm"]["max_rel_vs_plain_fp64"]}
    return out


def converged_errors(wl: dict, case_dir: str) -> dict:
    """The workload's own mesh and condition to L2 <= tol with the FP64
    drop-in (the oracle's steps, bit for bit) and with the FP32 operator,
    from the same ramped state (with the workload's sweep order: first-order
    sweeps keep the residual, so the steady state, and converge where the
    reference's plateau): steps, seconds, and the FP32-operator state's
    error against the FP64 one in density, pressure and the wall force
    coefficients."""
    import numpy as np
    import torch
    from hamstr_oop_gb300 import native
    cv = wl["converge"]
    out = {"tol": cv["tol"], "cap": cv["cap"], "start": "after the CFL ramp %r" % (list(wl["ramp"]),),
           "sweep_order": cv.get("sweep_order", 0)}
    res = {}
    for label, mixed in (("fp64", False), ("fp32_operator", True)):
        g = native.GpuSolver(open_case(wl, case_dir))
        for n, cfl in wl["ramp"]:
            g.set_cfl(cfl)
            g.march(n, 0.0)
        g.set_cfl(wl["CFL"])
        g.set_precision(mixed)
        if cv.get("sweep_order"):
            g.set_sweep_order(cv["sweep_order"])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        hist, ok = g.march(cv["cap"], cv["tol"])
        dt = time.perf_counter() - t0
        res[label] = (g.get("q").reshape(-1, 4), g.forces())
        out[label] = {"converged": bool(ok), "steps": int(hist.shape[0]), "seconds": dt,
                      "final_l2": float(hist[-1, 0]), "CL": res[label][1]["CL"], "CD": res[label][1]["CD"]}
        g.close()
    (q64, f64), (q32, f32) = res["fp64"], res["fp32_operator"]
    gm1 = 0.4

    def pres(q):
        return gm1 * (q[:, 3] - 0.5 * (q[:, 1] ** 2 + q[:, 2] ** 2) / q[:, 0])
    out["fp32_operator_vs_fp64"] = {
        "density_max_rel": float(np.max(np.abs(q32[:, 0] - q64[:, 0]) / np.abs(q64[:, 0]))),
        "pressure_max_rel": float(np.max(np.abs(pres(q32) - pres(q64)) / np.abs(pres(q64)))),
        "dCL": abs(f32["CL"] - f64["CL"]), "dCD": abs(f32["CD"] - f64["CD"])}
    return out


def cpu_steps(nc: int) -> int:
    """Host-leg sample size: a few seconds of every host thread's work."""
    return 20 if nc <= 20000 else 10


def cpu_baseline(wl, case_dir, nc, q_start, steps=None) -> dict:
    """The oracle on the host cores: one copy of the mesh per thread, a
    bounded sample, each step from the state the GPU's timed steps start
    from (the post-ramp state)."""
    from oracle import oracle
    oracle.build(reference=False)
    threads = os.cpu_count() or 1
    steps = steps or cpu_steps(nc)
    base = open_oracle(wl, case_dir)
    cases = [base] + [base.clone() for _ in range(threads - 1)]
    q0 = [q_start for _ in cases]
    time_oracle_steps(cases, q0, 1)          # warm-up step
    dt = time_oracle_steps(cases, q0, steps)
    for c in cases:
        c.close()
    return {"value": threads * nc * steps / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d pseudo-time steps (each from the state the GPU's timed steps start from) on each of %d "
                      "independent copies of the %s mesh (one per thread)" % (steps, threads, wl["name"])}


def run_reference_batch(args, wl):
    """The reference algorithm (C restatement) on the host cores for the
    batch's conditions: one condition per thread, a bounded sample."""
    from oracle import oracle
    oracle.build(reference=False)
    threads = os.cpu_count() or 1
    hosts = batch_cases(wl, threads)
    dirs = batch_mesh_dirs(wl, wl["meshes"])
    conds = batch_conditions(wl, threads)
    cases = []
    for (m, _, _), h in zip(conds, hosts):
        o = oracle.OracleCase(dirs[m], "port")
        p = h.params
        o.set_freestream(p["uinf"], p["vinf"], p["einf"])
        o.set("q", h.get("q"))
        cases.append(o)
    nc = sum(o.sizes["nCell"] for o in cases)
    q0 = [c.get("q") for c in cases]
    time_oracle_steps(cases, q0, max(args.warmup, 1))
    dt = time_oracle_steps(cases, q0, args.steps)
    for c in cases:
        c.close()
    value = nc * args.steps / dt
    sample = ("each step: one pseudo-time step (from the freestream state) of %d of the batch's conditions, one per "
              "host thread (meshes round-robin as in the batch), C restatement of the reference algorithm" % threads)
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": wl["name"], "cells_sampled": nc, "order": wl["order"],
                                            "msweep": wl["msweep"], "CFL": wl["CFL"]},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_reference(args, wl, rank):
    if rank != 0:
        return None
    if wl.get("batch"):
        return run_reference_batch(args, wl)
    from oracle import oracle
    oracle.build(reference=False)
    case_dir = make_case(wl, 0)
    threads = os.cpu_count() or 1
    base = open_oracle(wl, case_dir)
    nc = base.sizes["nCell"]
    # the GPU arm's CFL ramp, on one host thread, so the timed steps start
    # from the same kind of state (untimed)
    for n, cfl in wl["ramp"]:
        base.set_run(wl["order"], wl["msweep"], cfl)
        base.march(n)
    base.set_run(wl["order"], wl["msweep"], wl["CFL"])
    q_start = base.get("q")
    cases = [base] + [base.clone() for _ in range(threads - 1)]
    q0 = [q_start for _ in cases]
    time_oracle_steps(cases, q0, max(args.warmup, 1))
    dt = time_oracle_steps(cases, q0, args.steps)
    for c in cases:
        c.close()
    value = threads * nc * args.steps / dt
    sample = ("each step: one pseudo-time step (from the state after the GPU arm's CFL ramp, run here on the host) "
              "on each of %d independent copies of the %s mesh (one per host thread), C restatement of the "
              "reference algorithm (oracle/hamstr_oracle.c, bit-identical to the reference on the pinned "
              "fixtures)" % (threads, wl["name"]))
    world = dist_env()[2]
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": workload_config(wl, base.sizes, world),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--no-converge", action="store_true", help="skip the converged-solve leg")
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="only ramp and run this many steps (a plain run for ncu), no timing")
    ap.add_argument("--profile-precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--gemm-only", type=int, default=0, metavar="SIZE",
                    help="only time the tcgen05 BF16 GEMM on SIZE^3 (a plain run for ncu)")
    ap.add_argument("--c5-train", type=int, default=0, help="c5: training conditions (default: the config's)")
    ap.add_argument("--c5-test", type=int, default=0, help="c5: held-out conditions (default: the config's)")
    ap.add_argument("--msweep", type=int, default=0, help="ADI sweeps per step (default: the workload's, 2)")
    ap.add_argument("--batch-conditions", type=int, default=0,
                    help="batched workloads: number of conditions (default: the workload's)")
    ap.add_argument("--shape", default="", help="launch shape instead of the autotuner's, e.g. "
                    "face_block=128,adi_warps_per_sm=8 (hamstr_gpu_set_shape keys)")
    ap.add_argument("--target-only", action="store_true",
                    help="only the target-form leg (batched + FP32 operator + warm start vs the plain FP64 drop-in)")
    args = ap.parse_args()
    rank, local_rank, world = dist_env()
    if args.target_only:
        import torch
        torch.cuda.set_device(local_rank)
        print(json.dumps(target_form()), flush=True)
        return
    if args.gemm_only:
        import torch
        torch.cuda.set_device(local_rank)
        print(json.dumps(gemm_peak(args.gemm_only)), flush=True)
        return
    wl = dict(WORKLOADS[args.workload])
    if args.msweep:
        wl["name"] = wl["name"].replace("msweep%d" % wl["msweep"], "msweep%d" % args.msweep)
        wl["msweep"] = args.msweep
    if args.batch_conditions and wl.get("batch"):
        wl["name"] = wl["name"].replace("batch%d" % wl["n"], "batch%d" % args.batch_conditions)
        wl["n"] = args.batch_conditions
    if args.impl == "reference":
        out = run_reference(args, wl, rank)
        if out is not None:
            print(json.dumps(out), flush=True)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    if wl.get("warm"):
        out = run_warmstart(args, wl, rank, local_rank, world) if rank == 0 else None
    else:
        out = (run_batch if wl.get("batch") else run_gpu)(args, wl, rank, local_rank, world)
    if out is not None:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
