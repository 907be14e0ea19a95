#!/usr/bin/env python
"""Benchmark of the batched per-cell chemistry step on one GB300.

Workload: the synthetic 12-primary-species network (40 aqueous complexes, 6
kinetic TST minerals, 4 ion-exchange and 2 surface-complexation reactions)
on 2,097,152 cells, FP64, dt = 1 day, converged to a 1e-12 relative
residual.  One "step" is one reaction step over all cells.

  value   converged cell solves/s with inputs resident in HBM (device time of
          the solve, CUDA events on the library's stream, summed over the
          timed steps; the cell state is restored from a pristine copy between
          steps, outside the timed interval)
  e2e     the same metric through pfchem_react_batch with pinned host
          buffers: every step uploads inputs and state and downloads state
          and outputs
  cpu_baseline  the oracle (C++ restatement of RReact) on a bounded sample
          of the same cells on all host cores

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
# DRAM bytes per cell of the solve kernel, from an ncu capture of one launch
# on 524,288 cells of the same workload (561.5 MB read + 290.3 MB written)
TRAFFIC_BYTES_PER_CELL = (561539840 + 290312704) / 524288


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="pflotran_gb300")
    p.add_argument("--ncells", type=int, default=NCELLS)
    p.add_argument("--cpu-sample", type=int, default=20000)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--autotune", action="store_true")
    p.add_argument("--train-samples", type=int, default=8_388_608)
    p.add_argument("--epochs", type=int, default=12)
    p.add_argument("--plain-only", action="store_true")
    p.add_argument("--exact-jacobian", action=argparse.BooleanOptionalAction, default=True,
                   help="also time the step with the exact Newton Jacobian")
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


def make_workload(ncells, device="cpu", rank=0):
    """The synthetic 12-species workload; rank r of a multi-GPU run takes its
    own seeded shard of cells (weak scaling, no data exchange)."""
    from pflotran_gb300 import workloads
    net = workloads.synthetic_network()
    net, opt, cells, dt = workloads.synthetic_cells(ncells, seed=2024 + 7919 * rank, net=net, device=device)
    return net, opt, cells, dt


def cpu_baseline(net, opt, cells, dt, sample):
    from oracle import oracle
    idx = np.arange(min(sample, cells.ncells))
    sub = cells.subset(idx, net)
    sub.iterations = np.zeros(len(idx), np.int32)
    sub.status = np.zeros(len(idx), np.int32)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    oracle.react(net.as_struct(), opt, dt, sub, 0, threads)
    el = time.perf_counter() - t0
    return {"value": len(idx) / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"first {len(idx)} cells of the {cells.ncells}-cell workload, oracle RReact in double, "
                      f"{threads} std::threads"}, sub


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
    from oracle import oracle
    threads = os.cpu_count() or 1
    n = min(args.cpu_sample, cells.ncells)
    sub0 = cells.subset(np.arange(n), net)
    times = []
    for s in range(args.warmup + args.steps):
        sub = sub0.copy()
        t0 = time.perf_counter()
        oracle.react(net.as_struct(), opt, dt, sub, 0, threads)
        el = time.perf_counter() - t0
        if s >= args.warmup:
            times.append(el)
    value = n / (sum(times) / len(times))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"synthetic 12-species network (40 complexes, 6 minerals, 4 ion-exchange, "
                               f"2 surface-complexation), {args.ncells} cells, dt 1 day, 1e-12 rel. residual",
                   "sample_cells_per_step": n},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{n} of {args.ncells} cells per step (oracle C++ restatement of RReact; "
                                   f"PFLOTRAN's Fortran cannot be compiled in this image)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


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
    from pflotran_gb300 import work
    from pflotran_gb300.cells import CellBatch
    from pflotran_gb300.lib import ReactionStep

    net, opt, host, dt = make_workload(args.ncells, device=f"cuda:{local}", rank=rank)
    if args.jacobian == "exact":
        from pflotran_gb300 import abi as _abi
        opt.jacobian = _abi.JACOBIAN_EXACT
        args.exact_jacobian = False  # the headline already is the exact-Jacobian run
    n = host.ncells
    step = ReactionStep(net, opt, device=local)
    pristine = host.to_device()
    dev = pristine.copy()
    if args.autotune:
        step.autotune(dev, dt)
    launch = step.launch()

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
        dev_ms, iters, alt, slots, drains = [], [], [], [], []
        with Clocks(clk_index) as clk:
            for _ in range(args.steps):
                restore()
                torch.cuda.synchronize()
                if world > 1:
                    torch.distributed.barrier()
                step.react(dev, dt)
                st = step.stats()
                dev_ms.append(st.kernel_ms)
                iters.append(st.sum_iterations)
                alt.append(st.alt_guess_used)
                slots.append(st.lane_slots)
                drains.append(st.drain_ms)
                torch.cuda.synchronize()
        eff = float(np.sum(iters)) / float(np.sum(slots)) if np.sum(slots) else None
        timed.drain_ms = float(np.mean(drains))
        return float(np.sum(dev_ms)), iters, alt, clk.summary(), eff

    # plain Newton from the previous-step guess
    plain_ms, plain_iters, _, plain_clocks, plain_eff = timed(local)
    plain_drain = timed.drain_ms
    plain_value = world * n / (plain_ms / args.steps * 1e-3)
    g_plain = dev.to_host()
    warm = None
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
        step.surrogate_enable(True)
        if args.autotune:
            restore()
            step.autotune(dev, dt)
        warm = dict(report=rep, t_gen=t_gen, t_fit=t_fit,
                    err_rms=float(err.pow(2).mean().sqrt()), err_p50=float(err.max(0).values.median()),
                    err0_rms=float(err0.pow(2).mean().sqrt()), err0_p50=float(err0.max(0).values.median()))
    total_ms, iters, alt, clocks, eff = (timed(local) if warm is not None
                                         else (plain_ms, plain_iters, [0], plain_clocks, plain_eff))
    drain = timed.drain_ms if warm is not None else plain_drain
    launch = step.launch()
    g = dev.to_host()
    exact = None
    if args.exact_jacobian:
        # the same step with the exact Newton Jacobian (same equations and root)
        from pflotran_gb300 import abi
        from pflotran_gb300.network import default_options
        step.set_options(default_options(use_isothermal=opt.use_isothermal, jacobian=abi.JACOBIAN_EXACT))
        exact = {}
        for mode in (("plain", "warm") if warm is not None else ("plain",)):
            if warm is not None:
                step.surrogate_enable(mode == "warm")
            if args.autotune:
                restore()
                step.autotune(dev, dt)
            ms, its, _, _, e_eff = timed(local)
            ge = dev.to_host()
            both = (ge.status == 0) & (g.status == 0)
            rel = np.abs(ge.total_out - g.total_out).reshape(net.N, n) / np.maximum(
                np.abs(g.total_out).reshape(net.N, n), 1e-300)
            exact[mode] = {"value": world * n / (ms / args.steps * 1e-3), "ms_per_step": ms / args.steps,
                           "mean_newton_iterations": float(np.mean(its)) / n,
                           "max_newton_iterations": int(ge.iterations.max()),
                           "lane_efficiency": e_eff, "queue_drain_ms": timed.drain_ms,
                           "nonconverged": int((ge.status != 0).sum()),
                           "total_rel_diff_vs_reference_jacobian_max": float(rel[:, both].max())}
        if warm is not None:
            exact["speedup_warm_vs_plain"] = exact["warm"]["value"] / exact["plain"]["value"]
            exact["speedup_vs_reference_jacobian_warm"] = exact["warm"]["value"] / (world * n / (total_ms / args.steps * 1e-3))
        step.set_options(opt)
        step.set_launch(launch.block_threads, launch.blocks_per_sm, launch.refill_min_idle, launch.variant)
        if warm is not None:
            step.surrogate_enable(True)
    if world > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    value = world * n / (ms_per_step * 1e-3)
    conv = int((g.status == 0).sum())

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
    e2e_s = []
    for s in range(args.warmup + args.steps):
        for f in state_fields:
            a = getattr(pinned, f)
            if a is not None:
                a[:] = getattr(host, f)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        step.react(pinned, dt)
        el = time.perf_counter() - t0
        if s >= args.warmup:
            e2e_s.append(el)
    e2e_value = world * n / (sum(e2e_s) / len(e2e_s))

    # roofline: FP64-issue bound; algorithmic flops per launch / device time
    mean_iters = float(np.mean(iters)) / n
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
        wline = {"plain_value": plain_value, "plain_ms_per_step": plain_ms / args.steps,
                 "plain_mean_newton_iterations": float(np.mean(plain_iters)) / n,
                 "plain_lane_efficiency": plain_eff, "plain_queue_drain_ms": plain_drain,
                 "speedup_vs_plain": value / plain_value,
                 "alt_guess_used_frac": float(np.mean(alt)) / n,
                 "surrogate": {"arch": "16-256-256-256-12 GELU MLP, BF16 weights/activations, FP32 accumulate "
                                       "(mma.sync m16n8k16)",
                               "train_samples": int(r.samples), "epochs": args.epochs, "steps": int(r.steps),
                               "first_loss": r.first_loss, "final_loss": r.final_loss,
                               "train_ms_device": r.train_ms, "data_generation_s": warm["t_gen"],
                               "ln_m_error_rms": warm["err_rms"], "ln_m_maxerr_median": warm["err_p50"],
                               "plain_guess_ln_m_error_rms": warm["err0_rms"],
                               "plain_guess_ln_m_maxerr_median": warm["err0_p50"]}}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"synthetic 12-species network (40 complexes, 6 minerals, 4 ion-exchange, "
                               f"2 surface-complexation), {n} cells per GPU, dt 1 day, plain Newton from the "
                               f"previous-step guess, 1e-12 rel. residual",
                   "ncells": n, "l2": "inputs ~1.3 GB >> L2; state restored from a pristine copy between steps",
                   "launch": {"block_threads": launch.block_threads, "blocks_per_sm": launch.blocks_per_sm,
                              "refill_min_idle": launch.refill_min_idle},
                   "parallelism": "replicas" if world > 1 else "single"},
        "mean_newton_iterations": mean_iters, "converged_cells": conv,
        "lane_efficiency": eff, "queue_drain_ms": drain,
        "iteration_histogram": np.bincount(g.iterations).tolist(),
        # per step: prologue + persistent solve; the warm start adds the weight
        # packing (one launch per layer) and the fused MLP inference
        "gpu_launches": args.steps * (2 if warm is None else 2 + 4 + 1),
        "roofline": {"bound": "fp64", "achieved": achieved_tflops, "peak": probe, "unit": "TFLOP/s",
                     "frac": achieved_tflops / probe if probe else None,
                     "traffic": TRAFFIC_BYTES_PER_CELL * n,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one pfchem_gen_react "
                                       "launch on 524288 cells, scaled by cells "
                                       "(profiles/pfchem_gen_react_synthetic12_524k.md)",
                     "peak_source": "measured DFMA throughput on this GPU (pfchem_probe_fp64_peak, FMA = 2 flops)",
                     "flops_per_step": flops,
                     "hbm": {"achieved": hbm_gbs, "peak": hbm_peak, "unit": "GB/s", "frac": hbm_gbs / hbm_peak,
                             "bytes_per_step": bytes_step, "peak_source": "MEASURED_PEAKS.json hbm_gbs"}},
        "clocks": clocks,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
    }
    if exact is not None:
        line["exact_jacobian"] = exact
    if args.jacobian == "exact":
        line["config"]["workload"] += ", exact Newton Jacobian (PFCHEM_JACOBIAN_EXACT)"
    if wline is not None:
        line["warm_start"] = wline
        line["config"]["workload"] = line["config"]["workload"].replace(
            "plain Newton from the previous-step guess", "learned BF16 warm start with per-cell fallback, "
                                                         "FP64 Newton finishing")
    if rank == 0 and not args.no_cpu:
        cb, _ = cpu_baseline(net, opt, host, dt, args.cpu_sample)
        line["cpu_baseline"] = cb
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


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
