#!/usr/bin/env python
"""Benchmark of the batched per-cell chemistry step on one GB300.

Workload: the synthetic 12-primary-species network (40 aqueous complexes, 6
kinetic TST minerals, 4 ion-exchange and 2 surface-complexation reactions)
on 2,097,152 cells, FP64, dt = 1 day, converged to a 1e-12 relative
residual.  One "step" is one reaction step over all cells.

  value   CONVERGED cell solves/s with the learned warm start, inputs
          resident in HBM (cells whose status is not CONVERGED are not
          counted; device time of the step graph, CUDA events on the
          library's stream, summed over the timed steps; the cell state is
          restored from a pristine copy between steps, outside the timed
          interval).  warm_start.plain_value is the same for the plain
          previous-step guess.
  e2e     the same metric through pfchem_react_batch with pinned host
          buffers: every step uploads inputs and state and downloads state
          and outputs
  cpu_baseline  the oracle (C++ restatement of RReact) on a seeded random
          sample of the same cells on all host cores; also 1 core and the
          literal RReact accumulation
  parity  GPU against the oracle on that sample, for the plain and the
          warm-started step: max / p99 scaled relative errors of totals,
          mineral rates and volume fractions, and the per-cell bar (within
          1e-10 of the oracle, or no farther than it from the root of the
          equations, a long-double solve to a 1e-12-tighter residual)
  reference_path  the same plain step with exact_jacobian_after = 0
          (RReact's damped iteration, cut at 200 iterations): its converged
          solves/s, and how far its capped cells are from RReact run
          without a cap
  calcite_grid  the calcite network on 100^3 cells, temperature-dependent
          log K, plain Newton, graph-captured
  timestepped   128^3 cells x 50 steps of transport + reaction, one CUDA graph
          per step, drift against the oracle on sampled cells

`--impl reference` times the reference's CPU implementation of the step
(the oracle port: PFLOTRAN's Fortran cannot be built in this image) on the
same workload and prints the same JSON line with "impl": "reference".
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "converged cell chemistry solves/s at 1e-12 rel. residual, warm-start vs plain GPU Newton"
UNIT = "cell solves/s"
NCELLS = 2_097_152
# DRAM bytes per cell of the solve kernel, from an ncu capture of one warm-step
# launch on 524,288 cells of the same workload, default compact launch
# (625.0 MB read + 410.6 MB written)
TRAFFIC_BYTES_PER_CELL = (625028864 + 410648320) / 524288
SAMPLE_SEED = 12345


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="pflotran_gb300")
    p.add_argument("--ncells", type=int, default=NCELLS)
    p.add_argument("--cpu-sample", type=int, default=20000)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--autotune", action=argparse.BooleanOptionalAction, default=True,
                   help="choose the launch with pfchem_autotune on a 262,144-cell draw of the workload")
    p.add_argument("--train-samples", type=int, default=8_388_608)
    p.add_argument("--epochs", type=int, default=12)
    p.add_argument("--plain-only", action="store_true")
    p.add_argument("--launch", default=None, metavar="THREADS,BLOCKS_PER_SM,REFILL,VARIANT",
                   help="a fixed launch for every step (pfchem_set_launch) instead of the tuner's")
    p.add_argument("--mlp-backend", choices=("mma.sync", "tcgen05"), default="tcgen05",
                   help="tensor-core path of the warm-start MLP (training and the step's inference)")
    p.add_argument("--exact-jacobian", action=argparse.BooleanOptionalAction, default=True,
                   help="also time the step with the exact Newton Jacobian")
    p.add_argument("--reference-path", action=argparse.BooleanOptionalAction, default=True,
                   help="also time the plain step with exact_jacobian_after = 0")
    p.add_argument("--calcite-grid", action=argparse.BooleanOptionalAction, default=True)
    p.add_argument("--timestepped", action=argparse.BooleanOptionalAction, default=True)
    p.add_argument("--mapping", action=argparse.BooleanOptionalAction, default=True,
                   help="thread-per-cell vs cooperative kernels on three network sizes")
    p.add_argument("--jacobian", choices=("reference", "exact"), default="reference",
                   help="Newton Jacobian of the headline run")
    return p.parse_args()


def rank_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        self.f.flush()
        rows = []
        try:
            for line in open(self.f.name):
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        except Exception:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def make_workload(ncells, device="cpu", rank=0, seed=2024):
    """The synthetic 12-species workload; rank r of a multi-GPU run takes its
    own seeded shard of cells (weak scaling, no data exchange)."""
    from pflotran_gb300 import workloads
    net = workloads.synthetic_network()
    net, opt, cells, dt = workloads.synthetic_cells(ncells, seed=seed + 7919 * rank, net=net, device=device)
    return net, opt, cells, dt


def sample_indices(n, k, seed=SAMPLE_SEED):
    """A seeded random sample of k of the n cells (sorted)."""
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(n, min(k, n), replace=False))


def _opts(opt, **kw):
    from pflotran_gb300 import abi
    o = abi.Options.from_buffer_copy(opt)
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def cpu_baseline(net, opt, cells, dt, sample):
    """The oracle on a seeded random sample of the workload: all host cores
    (the reported baseline), one core on a tenth of the sample, and the
    literal RReact accumulation (accum_scale = 1, absolute residual and
    relative-change tests).  Returns (baseline dict, sample indices, the
    sample's inputs, the oracle's all-core solution)."""
    from oracle import parity
    idx = sample_indices(cells.ncells, sample)
    sub = cells.subset(idx, net)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    ref = parity.solve(net, opt, dt, sub, 0, threads)
    el = time.perf_counter() - t0
    one = sub.subset(np.arange(max(1, len(idx) // 10)), net)
    t0 = time.perf_counter()
    r1 = parity.solve(net, opt, dt, one, 0, 1)
    el1 = time.perf_counter() - t0
    # RReact's literal residual is not divided by dt while its Jacobian is
    # (reaction.F90:3424-3426 vs :5189-5190): its Newton step is dt times too
    # long, so the literal form is timed at dt = 1 s, where the two agree
    lit_opt = _opts(opt, accum_mode=1, residual_tol_kind=0, max_relative_change_tolerance=1e-6)
    t0 = time.perf_counter()
    lit = parity.solve(net, lit_opt, 1.0, sub, 0, threads)
    el_lit = time.perf_counter() - t0
    conv = int((ref.status == 0).sum())
    cb = {"value": conv / el, "unit": UNIT, "cores": threads, "kind": "port",
          "sample": f"{len(idx)} cells drawn at random (seed {SAMPLE_SEED}) from the {cells.ncells}-cell workload, "
                    f"oracle RReact in double, {threads} std::threads; converged cells counted",
          "converged": conv,
          "one_core": {"value": int((r1.status == 0).sum()) / el1, "unit": UNIT, "cells": one.ncells},
          "literal_rreact": {"value": int((lit.status == 0).sum()) / el_lit, "unit": UNIT, "cores": threads,
                             "converged": int((lit.status == 0).sum()), "cells": len(idx),
                             "options": "accum_scale 1 (RReact's residual without /dt), absolute 1e-12 residual, "
                                        "1e-6 relative-change exit, dt 1 s"}}
    return cb, idx, sub, ref


def parity_block(net, opt, dt, sub, ref, gpu_sub, truth, alt=None):
    """GPU against the oracle on the sample: error statement and the per-cell
    bar against the root (and, given `alt`, the oracle's answer from another
    starting guess)."""
    from oracle import parity
    both = (ref.status == 0) & (gpu_sub.status == 0)
    st = parity.error_statement(net, gpu_sub, ref, both)
    bar = parity.per_cell_bar(net, gpu_sub, ref, truth, 1e-10, both & (truth.status == 0), alt=alt)
    out = {"cells": int(both.sum()), "gpu_nonconverged": int((gpu_sub.status != 0).sum()),
           "oracle_nonconverged": int((ref.status != 0).sum()),
           "same_iterations": float(np.mean(ref.iterations[both] == gpu_sub.iterations[both])) if both.any() else None}
    for q, e in st.items():
        ok, exr, ext, ert = bar[q]
        m = both & (truth.status == 0)
        out[q] = dict(e, beyond_1e10=int((exr[both] > 1e-10).sum()), bar_failures=int((~ok).sum()),
                      gpu_vs_root_max=float(ext[m].max()) if m.any() else None,
                      oracle_vs_root_max=float(ert[m].max()) if m.any() else None)
    return out


def _cuda():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def run_reference(args):
    rank, world, _ = rank_env()
    if rank != 0:
        return
    net, opt, cells, dt = make_workload(args.ncells, device="cuda" if _cuda() else "cpu")
    from oracle import parity
    threads = os.cpu_count() or 1
    idx = sample_indices(cells.ncells, args.cpu_sample)
    sub0 = cells.subset(idx, net)
    n = len(idx)
    times, conv = [], []
    for s in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        r = parity.solve(net, opt, dt, sub0, 0, threads)
        el = time.perf_counter() - t0
        if s >= args.warmup:
            times.append(el)
            conv.append(int((r.status == 0).sum()))
    value = float(np.mean(conv)) / (sum(times) / len(times))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"synthetic 12-species network (40 complexes, 6 minerals, 4 ion-exchange, "
                               f"2 surface-complexation), {args.ncells} cells, dt 1 day, 1e-12 rel. residual, "
                               f"exact_jacobian_after {opt.exact_jacobian_after} (the options of the GPU arm)",
                   "sample_cells_per_step": n},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{n} of {args.ncells} cells per step, drawn at random (seed {SAMPLE_SEED}); "
                                   f"oracle C++ restatement of RReact; PFLOTRAN's Fortran cannot be compiled in "
                                   f"this image; converged cells counted"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def calcite_grid(args, local):
    """Config 2: the calcite network on 100^3 cells with temperature-dependent
    log K, plain Newton from the previous-step guess, graph-captured."""
    import torch
    from oracle import parity
    from pflotran_gb300 import workloads
    from pflotran_gb300.lib import ReactionStep
    net, opt, host, dt = workloads.calcite_cells(1_000_000, seed=2, temperature_dependent=True,
                                                 device=f"cuda:{local}")
    step = ReactionStep(net, opt, device=local)
    pristine = host.to_device()
    dev = pristine.copy()
    ms, conv, its = [], [], []
    for s in range(args.warmup + args.steps):
        for f in ("pri_molal", "ionic_strength", "mnrl_volfrac"):
            getattr(dev, f).copy_(getattr(pristine, f))
        torch.cuda.synchronize()
        step.react(dev, dt)
        st = step.stats()
        if s >= args.warmup:
            ms.append(st.kernel_ms)
            conv.append(st.ncells - st.nonconverged)
            its.append(st.sum_iterations / st.ncells)
    g = dev.to_host()
    idx = sample_indices(host.ncells, 20000, SAMPLE_SEED + 1)
    sub = host.subset(idx, net)
    ref = parity.solve(net, opt, dt, sub, 0)
    gsub = g.subset(idx, net)
    both = (ref.status == 0) & (gsub.status == 0)
    return {"workload": "calcite network (3 primaries, 5 complexes, kinetic calcite), 1,000,000 cells, T in "
                        "[10, 60] C with log K linear in T, dt 1 day, plain Newton, graph-captured",
            "value": float(np.sum(conv)) / (float(np.sum(ms)) * 1e-3), "unit": UNIT,
            "ms_per_step": float(np.mean(ms)), "mean_newton_iterations": float(np.mean(its)),
            "nonconverged": int(host.ncells - conv[-1]),
            "parity": {"cells": int(both.sum()), **parity.error_statement(net, gsub, ref, both)}}


def mapping_by_size(args, local, ncells=262144):
    """Thread-per-cell (network-specialized) against cooperative kernels
    (8/16/32 lanes per cell) by network size: device time of one step
    (best of 2 after a warm-up) on `ncells` cells of three networks, and the
    launch pfchem_autotune keeps for each."""
    from pflotran_gb300 import abi, workloads
    from pflotran_gb300.lib import PfchemError, ReactionStep
    nets = {"calcite (N=3, 5 complexes, 1 mineral)":
            workloads.calcite_cells(ncells, seed=3, temperature_dependent=True, device=f"cuda:{local}"),
            "synthetic (N=12, 40 complexes, 6 minerals, 4 exchange, 2 surface)":
            workloads.synthetic_cells(ncells, seed=5, device=f"cuda:{local}"),
            "synthetic (N=16, 64 complexes, 8 minerals, 4 exchange, 2 surface)":
            workloads.synthetic_cells(ncells, seed=5, net=workloads.synthetic_network(N=16, Nc=64, Nm=8),
                                      device=f"cuda:{local}")}
    names = {abi.KERNEL_SPECIALIZED: "thread-per-cell specialized", abi.KERNEL_SPECIALIZED_COMPACT:
             "thread-per-cell specialized, compact", abi.KERNEL_COOP8: "8 lanes per cell",
             abi.KERNEL_COOP16: "16 lanes per cell", abi.KERNEL_COOP32: "32 lanes per cell (warp)"}
    out = {}
    for label, (net, opt, host, dt) in nets.items():
        step = ReactionStep(net, opt, device=local)
        pristine = host.to_device()
        res = {}
        default = step.launch()
        for variant in names:
            block = 32 if variant in (abi.KERNEL_SPECIALIZED, abi.KERNEL_SPECIALIZED_COMPACT) else 128
            try:
                bps = None
                for b in range(16, 0, -1):  # as many resident blocks per SM as fit
                    try:
                        step.set_launch(block, b, 1, variant)
                        bps = b
                        break
                    except PfchemError:
                        continue
                if bps is None:
                    raise PfchemError("does not fit on an SM")
                times, its, bad = [], 0.0, 0
                for rep in range(3):
                    dev = pristine.copy()
                    step.react(dev, dt)
                    st = step.stats()
                    if rep:
                        times.append(st.kernel_ms)
                    its, bad = st.sum_iterations / st.ncells, int(st.nonconverged)
                res[names[variant]] = {"ms": min(times), "block_threads": block, "blocks_per_sm": bps,
                                       "mean_newton_iterations": its, "nonconverged": bad}
            except Exception as e:  # a mapping that does not apply to this network
                res[names[variant]] = {"error": str(e)[:200]}
        tuned = step.autotune(pristine.copy(), dt)
        res["autotune_choice"] = {"variant": names.get(tuned.variant, tuned.variant),
                                  "block_threads": tuned.block_threads, "blocks_per_sm": tuned.blocks_per_sm,
                                  "refill_min_idle": tuned.refill_min_idle}
        res["library_default"] = names.get(default.variant, default.variant)
        out[label] = res
        del step, pristine
    return {"cells": ncells, "networks": out}


def timestepped(args, local):
    """Config 5: 128^3 cells x 50 steps, upwind transport + reaction step in
    one CUDA graph per step, learned warm start, drift against the oracle on
    512 sampled cells per step."""
    from oracle import oracle
    from pflotran_gb300.os_run import OperatorSplitRun
    from pflotran_gb300 import abi
    run = OperatorSplitRun(shape=(128, 128, 128), warm_start=True, autotune=False, drift_sample=512, log=None,
                           device=f"cuda:{local}",
                           mlp_backend=abi.MLP_TCGEN05 if args.mlp_backend == "tcgen05" else abi.MLP_MMA_SYNC)
    fn = lambda n_, o_, dt_, c_: oracle.react(n_, o_, dt_, c_, 0, os.cpu_count() or 1)
    recs = run.run(steps=50, oracle_fn=fn)
    react = [r["solves_per_s"] for r in recs if "solves_per_s" in r]
    worst = {k: max(r["drift"].get(k, 0.0) for r in recs) for k in ("pri_molal", "total", "mnrl_rate",
                                                                       "mnrl_volfrac")}
    return {"workload": "128^3 cells of the synthetic 12-species network, 50 steps of 1 day, upwind transport "
                        f"({run.nsub} sub-steps) + reaction step with the learned warm start ({args.mlp_backend} "
                        f"MLP), one CUDA graph per step",
            "steps": len(recs),
            "reaction_solves_per_s_mean": float(np.mean(react)) if react else None,
            "reaction_solves_per_s_first_last": [react[0], react[-1]] if react else None,
            "step_solves_per_s_mean": float(np.mean([r["step_solves_per_s"] for r in recs])),
            "transport_ms_mean": float(np.mean([r["transport_ms"] for r in recs if "transport_ms" in r]))
            if react else None,
            "mean_newton_iterations_first_last": [recs[0]["mean_iterations"], recs[-1]["mean_iterations"]],
            "nonconverged_max": int(max(r["nonconverged"] for r in recs)),
            "warm_start_used_frac_first_last": [recs[0]["warm_start_used"] / run.n,
                                                recs[-1]["warm_start_used"] / run.n],
            "drift_max_vs_oracle": worst, "drift_cells_per_step": run.drift_sample,
            "train": run.report.get("train")}


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import torch
    rank, world, local = rank_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from pflotran_gb300 import abi as _abi
    from pflotran_gb300 import work
    from pflotran_gb300.cells import CellBatch
    from pflotran_gb300.lib import ReactionStep

    net, opt, host, dt = make_workload(args.ncells, device=f"cuda:{local}", rank=rank)
    if args.jacobian == "exact":
        opt.jacobian = _abi.JACOBIAN_EXACT
        args.exact_jacobian = False  # the headline already is the exact-Jacobian run
    n = host.ncells
    step = ReactionStep(net, opt, device=local)
    mlp_backend = _abi.MLP_TCGEN05 if args.mlp_backend == "tcgen05" else _abi.MLP_MMA_SYNC
    step.surrogate_backend(mlp_backend)
    pristine = host.to_device()
    dev = pristine.copy()
    def autotune():
        # the launch search runs on its own draw of the workload, on the
        # step as it is configured (plain, or with the warm start enabled)
        _, _, th, _ = make_workload(min(262144, n), device=f"cuda:{local}", rank=rank, seed=4049)
        t0 = time.perf_counter()
        step.autotune(th.to_device(), dt)
        return {"cells": th.ncells, "s": time.perf_counter() - t0}

    def launch_dict(L, tune):
        return {"block_threads": L.block_threads, "blocks_per_sm": L.blocks_per_sm,
                "refill_min_idle": L.refill_min_idle, "variant": L.variant,
                "source": "pfchem_autotune" if tune else "library default", "autotune": tune}

    if args.launch:
        args.autotune = False
        step.set_launch(*[int(x) for x in args.launch.split(",")])
    tune = autotune() if args.autotune else None
    launch = step.launch()
    plain_launch = launch_dict(launch, tune)

    def restore():
        for f in CellBatch.FIELDS:
            a = getattr(pristine, f)
            if a is not None:
                getattr(dev, f).copy_(a)

    def timed(clk_index):
        for _ in range(args.warmup):
            restore()
            step.react(dev, dt)
        torch.cuda.synchronize()
        r = {"ms": [], "iters": [], "alt": [], "slots": [], "drain": [], "conv": []}
        with Clocks(clk_index) as clk:
            for _ in range(args.steps):
                restore()
                torch.cuda.synchronize()
                if world > 1:
                    torch.distributed.barrier()
                step.react(dev, dt)
                st = step.stats()
                r["ms"].append(st.kernel_ms)
                r["iters"].append(st.sum_iterations)
                r["alt"].append(st.alt_guess_used)
                r["slots"].append(st.lane_slots)
                r["drain"].append(st.drain_ms)
                r["conv"].append(st.ncells - st.nonconverged)
                torch.cuda.synchronize()
        r["clocks"] = clk.summary()
        r["total_ms"] = float(np.sum(r["ms"]))
        r["eff"] = float(np.sum(r["iters"])) / float(np.sum(r["slots"])) if np.sum(r["slots"]) else None
        r["drain_ms"] = float(np.mean(r["drain"]))
        r["value"] = world * float(np.sum(r["conv"])) / (r["total_ms"] * 1e-3)
        r["nonconverged"] = int(n - r["conv"][-1])
        return r

    # plain Newton from the previous-step guess
    plain = timed(local)
    g_plain = dev.to_host()
    warm = None
    pred_sample = None
    if not args.plain_only:
        # learned warm start: trained on solves of a fresh seeded draw by the same kernel
        from pflotran_gb300 import surrogate, workloads
        t0 = time.perf_counter()
        X, molal = surrogate.generate(step, lambda m, s: workloads.synthetic_cells(m, seed=s, net=net,
                                                                                    device=f"cuda:{local}")[2],
                                      args.train_samples, 7001, dt)
        t_gen = time.perf_counter() - t0
        rep, t_fit = surrogate.fit(step, X, molal, epochs=args.epochs)
        del X, molal
        # surrogate-only error on the benchmark cells against the converged FP64 solution
        restore()
        pred = step.surrogate_predict(dev).view(net.N, n)
        ok = torch.from_numpy(g_plain.status == 0).to(pred.device)
        sol = torch.from_numpy(g_plain.pri_molal).to(pred.device).view(net.N, n)
        err = (torch.log(pred) - torch.log(sol))[:, ok].abs()
        plain_guess = torch.from_numpy(host.pri_molal).to(pred.device).view(net.N, n)
        err0 = (torch.log(plain_guess) - torch.log(sol))[:, ok].abs()
        if not args.no_cpu and rank == 0:
            pidx = sample_indices(n, args.cpu_sample)
            pred_sample = pred[:, torch.as_tensor(pidx, device=pred.device)].cpu().numpy().copy()
        del pred
        # inference alone: features + the fused four-layer MLP (+ weight
        # packing and the guess copy) over all cells, best of 3 synchronous calls
        step.surrogate_backend(_abi.MLP_MMA_SYNC)
        inf_ms = []
        for _ in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            g_ = step.surrogate_predict(dev)
            inf_ms.append((time.perf_counter() - t0) * 1e3)
            del g_
        inf_flops = 2.0 * (16 * 256 + 2 * 256 * 256 + 256 * 16) * n
        inference = {"ms": min(inf_ms), "tflops": inf_flops / (min(inf_ms) * 1e-3) / 1e12,
                     "flops": inf_flops,
                     "frac_of_bf16_peak": inf_flops / (min(inf_ms) * 1e-3) / 1e12 / _bf16_peak(),
                     "peak_source": "MEASURED_PEAKS.json bf16_tflops (cuBLAS burst)",
                     "backend": "mma.sync fused one-kernel inference"}
        # the same inference on the tcgen05 path (layer by layer, TMEM accumulators)
        try:
            step.surrogate_backend(_abi.MLP_TCGEN05)
            t_ms = []
            for _ in range(3):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                g_ = step.surrogate_predict(dev)
                t_ms.append((time.perf_counter() - t0) * 1e3)
                del g_
            inference["tcgen05"] = {"ms": min(t_ms), "tflops": inf_flops / (min(t_ms) * 1e-3) / 1e12,
                                    "frac_of_bf16_peak": inf_flops / (min(t_ms) * 1e-3) / 1e12 / _bf16_peak()}
        except Exception as e:
            inference["tcgen05"] = {"error": str(e)[:200]}
        finally:
            step.surrogate_backend(mlp_backend)
        inference["backend_in_step"] = args.mlp_backend
        step.surrogate_enable(True)
        if args.autotune:
            # the warm step has its own best launch (fewer iterations per cell)
            tune = autotune()
            launch = step.launch()
        warm = dict(report=rep, t_gen=t_gen, t_fit=t_fit, inference=inference,
                    err_rms=float(err.pow(2).mean().sqrt()), err_p50=float(err.max(0).values.median()),
                    err0_rms=float(err0.pow(2).mean().sqrt()), err0_p50=float(err0.max(0).values.median()))
        del err, err0, sol, plain_guess
    head = timed(local) if warm is not None else plain
    g = dev.to_host()

    # RReact's damped path (exact_jacobian_after = 0), plain
    refpath = None
    g_ref = None
    if args.reference_path and args.jacobian == "reference":
        if warm is not None:
            step.surrogate_enable(False)
        step.set_options(_opts(opt, exact_jacobian_after=0))
        rp = timed(local)
        g_ref = dev.to_host()
        refpath = {"value": rp["value"], "ms_per_step": rp["total_ms"] / args.steps,
                   "mean_newton_iterations": float(np.mean(rp["iters"])) / n,
                   "nonconverged": rp["nonconverged"], "queue_drain_ms": rp["drain_ms"],
                   "lane_efficiency": rp["eff"], "max_iterations": int(g_ref.iterations.max())}
        step.set_options(opt)
        if warm is not None:
            step.surrogate_enable(True)
    exact = None
    exact_out = {}
    if args.exact_jacobian:
        # the same step with the exact Newton Jacobian (same equations and root)
        step.set_options(_opts(opt, jacobian=_abi.JACOBIAN_EXACT))
        exact = {}
        for mode in (("plain", "warm") if warm is not None else ("plain",)):
            if warm is not None:
                step.surrogate_enable(mode == "warm")
            r = timed(local)
            ge = dev.to_host()
            exact_out[mode] = ge
            exact[mode] = {"value": r["value"], "ms_per_step": r["total_ms"] / args.steps,
                           "mean_newton_iterations": float(np.mean(r["iters"])) / n,
                           "max_newton_iterations": int(ge.iterations.max()),
                           "lane_efficiency": r["eff"], "queue_drain_ms": r["drain_ms"],
                           "nonconverged": r["nonconverged"]}
        if warm is not None:
            exact["speedup_warm_vs_plain"] = exact["warm"]["value"] / exact["plain"]["value"]
            # the learned warm start with exact Newton against the plain
            # RReact Newton (reference Jacobian): both within the per-cell bar
            # of the reference (parity.exact_warm_vs_reference_oracle)
            exact["speedup_warm_exact_vs_plain_reference"] = exact["warm"]["value"] / plain["value"]
        step.set_options(opt)
        if warm is not None:
            step.surrogate_enable(True)
    total_ms = head["total_ms"]
    if world > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    conv_per_step = float(np.mean(head["conv"]))
    value = world * conv_per_step / (ms_per_step * 1e-3)

    # end-to-end through the public API with pinned host buffers
    pinned = CellBatch(n)
    for f in CellBatch.FIELDS:
        a = getattr(host, f)
        if a is not None:
            t = torch.empty(a.size, dtype=torch.float64 if a.dtype == np.float64 else torch.int32).pin_memory()
            t.numpy()[:] = a
            setattr(pinned, f, t.numpy())
    h2d = sum(getattr(pinned, f).nbytes for f in ("temperature", "saturation", "den_kg", "porosity", "volume",
                                                   "soil_particle_density", "total", "pri_molal", "ionic_strength",
                                                   "mnrl_volfrac", "mnrl_area", "total_sorb_eq",
                                                   "eqionx_ref_cation_sorbed_conc", "srfcplxrxn_free_site_conc")
              if getattr(pinned, f) is not None)
    d2h = sum(getattr(pinned, f).nbytes for f in ("pri_molal", "ionic_strength", "mnrl_volfrac", "total_sorb_eq",
                                                   "eqionx_ref_cation_sorbed_conc", "srfcplxrxn_free_site_conc",
                                                   "total_out", "mnrl_rate", "iterations", "status")
              if getattr(pinned, f) is not None)
    state_fields = ("pri_molal", "ionic_strength", "mnrl_volfrac", "total_sorb_eq",
                    "eqionx_ref_cation_sorbed_conc", "srfcplxrxn_free_site_conc")
    e2e_s, e2e_conv = [], []
    for s in range(args.warmup + args.steps):
        for f in state_fields:
            a = getattr(pinned, f)
            if a is not None:
                a[:] = getattr(host, f)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        bad = step.react(pinned, dt)
        el = time.perf_counter() - t0
        if s >= args.warmup:
            e2e_s.append(el)
            e2e_conv.append(n - bad)
    e2e_value = world * float(np.mean(e2e_conv)) / (sum(e2e_s) / len(e2e_s))

    # roofline: FP64-issue bound; algorithmic flops per launch / device time
    mean_iters = float(np.mean(head["iters"])) / n
    flops = work.step_flops(net, g.iterations, isothermal=bool(opt.use_isothermal))
    achieved_tflops = flops / (ms_per_step * 1e-3) / 1e12
    probe = fp64_peak(local)
    bytes_step = work.bytes_per_cell(net) * n
    hbm_gbs = bytes_step / (ms_per_step * 1e-3) / 1e9
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    wline = None
    if warm is not None:
        r = warm["report"]
        wline = {"plain_value": plain["value"], "plain_ms_per_step": plain["total_ms"] / args.steps,
                 "plain_launch": plain_launch,
                 "plain_mean_newton_iterations": float(np.mean(plain["iters"])) / n,
                 "plain_nonconverged": plain["nonconverged"],
                 "plain_lane_efficiency": plain["eff"], "plain_queue_drain_ms": plain["drain_ms"],
                 "speedup_vs_plain": value / plain["value"],
                 "alt_guess_used_frac": float(np.mean(head["alt"])) / n,
                 "surrogate": {"arch": "16-256-256-256-12 GELU MLP, BF16 weights/activations, FP32 accumulate "
                                       + ("(tcgen05.mma, TMEM accumulators)" if args.mlp_backend == "tcgen05"
                                          else "(mma.sync m16n8k16)"),
                               "train_samples": int(r.samples), "epochs": args.epochs, "steps": int(r.steps),
                               "first_loss": r.first_loss, "final_loss": r.final_loss,
                               "train_ms_device": r.train_ms, "data_generation_s": warm["t_gen"],
                               "ln_m_error_rms": warm["err_rms"], "ln_m_maxerr_median": warm["err_p50"],
                               "plain_guess_ln_m_error_rms": warm["err0_rms"],
                               "plain_guess_ln_m_maxerr_median": warm["err0_p50"],
                               "inference": warm["inference"]}}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"synthetic 12-species network (40 complexes, 6 minerals, 4 ion-exchange, "
                               f"2 surface-complexation), {n} cells per GPU, dt 1 day, plain Newton from the "
                               f"previous-step guess, 1e-12 rel. residual, exact_jacobian_after "
                               f"{opt.exact_jacobian_after}; converged cells counted",
                   "ncells": n, "l2": "inputs ~1.3 GB >> L2; state restored from a pristine copy between steps",
                   "launch": launch_dict(launch, tune),
                   "parallelism": "replicas" if world > 1 else "single"},
        "mean_newton_iterations": mean_iters, "converged_cells": int((g.status == 0).sum()),
        "nonconverged": head["nonconverged"],
        "lane_efficiency": head["eff"], "queue_drain_ms": head["drain_ms"],
        "iteration_histogram": np.bincount(g.iterations).tolist(),
        # per step: prologue + persistent solve; the warm start adds the weight
        # packing (one launch per layer) and the fused MLP inference
        "gpu_launches": args.steps * (2 if warm is None else 2 + (4 + 1 if args.mlp_backend == "mma.sync" else
                                                                   1 + ((n + 262143) // 262144) * 10)),
        "roofline": {"bound": "fp64", "achieved": achieved_tflops, "peak": probe, "unit": "TFLOP/s",
                     "frac": achieved_tflops / probe if probe else None,
                     "traffic": TRAFFIC_BYTES_PER_CELL * n,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one pfchem_gen_react "
                                       "launch on 524288 cells of this workload (warm step, compact layout), "
                                       "scaled by cells",
                     "peak_source": "measured DFMA throughput on this GPU (pfchem_probe_fp64_peak, FMA = 2 flops)",
                     "flops_per_step": flops,
                     "hbm": {"achieved": hbm_gbs, "peak": hbm_peak, "unit": "GB/s", "frac": hbm_gbs / hbm_peak,
                             "bytes_per_step": bytes_step, "peak_source": "MEASURED_PEAKS.json hbm_gbs"}},
        "clocks": head["clocks"],
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
    }
    if exact is not None:
        line["exact_jacobian"] = exact
    if refpath is not None:
        line["reference_path"] = refpath
    if args.jacobian == "exact":
        line["config"]["workload"] += ", exact Newton Jacobian (PFCHEM_JACOBIAN_EXACT)"
    if wline is not None:
        line["warm_start"] = wline
        line["config"]["workload"] = line["config"]["workload"].replace(
            "plain Newton from the previous-step guess", "learned BF16 warm start with per-cell fallback, "
                                                         "FP64 Newton finishing")
    if rank == 0 and not args.no_cpu:
        from oracle import parity
        cb, idx, sub, ref = cpu_baseline(net, opt, host, dt, args.cpu_sample)
        line["cpu_baseline"] = cb
        truth = parity.truth_solve(net, opt, dt, sub, ref)
        par = {"sample": f"{len(idx)} cells drawn at random (seed {SAMPLE_SEED})",
               "root": f"oracle in long double, exact undamped Newton to a 1e-16 relative residual from the "
                       f"oracle's solution; {int((truth.status == 0).sum())} cells solved",
               "plain": parity_block(net, opt, dt, sub, ref, g_plain.subset(idx, net), truth)}
        if warm is not None and pred_sample is not None:
            ref_w = parity.solve(net, opt, dt, sub, 0, alt_guess=pred_sample.ravel())
            par["warm"] = parity_block(net, opt, dt, sub, ref_w, g.subset(idx, net), truth, alt=ref)
            both = (ref.status == 0) & (g.subset(idx, net).status == 0)
            par["warm_vs_plain_oracle"] = parity.error_statement(net, g.subset(idx, net), ref, both)
        for mode, ge in exact_out.items():
            # the exact-Jacobian solves against the oracle's RReact (reference
            # Jacobian, same options otherwise): the per-cell bar
            par[f"exact_{mode}_vs_reference_oracle"] = parity_block(net, opt, dt, sub, ref, ge.subset(idx, net), truth)
        line["parity"] = par
        if g_ref is not None:
            # RReact's damped path: the cells the 200-iteration cap stops,
            # against RReact without a cap
            capped = np.flatnonzero(g_ref.status != 0)
            if len(capped):
                cs = capped[sample_indices(len(capped), 2000, SAMPLE_SEED + 2)]
                hsub = host.subset(cs, net)
                free = parity.solve(net, _opts(opt, exact_jacobian_after=0, max_iterations=1_000_000), dt, hsub)
                ok = free.status == 0
                e = parity.cell_errors(net, g_ref.subset(cs, net), free)["total"]
                line["reference_path"]["capped_cells"] = {
                    "sampled": len(cs), "converge_without_cap": int(ok.sum()),
                    "uncapped_iterations_p50_p99_max": [float(np.percentile(free.iterations[ok], q))
                                                        for q in (50, 99, 100)] if ok.any() else None,
                    "capped_answer_vs_uncapped_total_median_max": [float(np.median(e[ok])), float(e[ok].max())]
                    if ok.any() else None}
    if rank == 0 and args.calcite_grid:
        line["calcite_grid"] = calcite_grid(args, local)
    if rank == 0 and args.timestepped:
        line["timestepped"] = timestepped(args, local)
    if rank == 0 and args.mapping:
        line["mapping_by_size"] = mapping_by_size(args, local)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def _bf16_peak():
    try:
        return float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["bf16_tflops"])
    except Exception:
        return 1910.0


def fp64_peak(device):
    import ctypes as C
    from pflotran_gb300.build import PROBE, build
    build()
    l = C.CDLL(PROBE)
    l.pfchem_probe_fp64_peak.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    tf = C.c_double()
    ms = C.c_double()
    if l.pfchem_probe_fp64_peak(device, 4096, C.byref(tf), C.byref(ms)) != 0:
        return None
    return tf.value


if __name__ == "__main__":
    main()
