"""Benchmark: electrostatic global-placement iterations per second.

Workload (default): the LFE5U-85-scale synthetic netlist — 42,000 movable
unit-area LUT cells on a 210x210 site fabric, 365 fixed perimeter IO cells,
50,000 nets in 2 / 3-5 / 6-32-pin bands with Gaussian index-grid locality
(sigma 12 sites), a 256x256 bin grid, target density 0.9, WA gamma base 4
bin widths, iteration cap 1000. Data are seeded synthetic (no public netlist
is available offline).

A step is one GP iteration: one dynamic Nesterov step with its objective
evaluations plus the multiplier update, on a device-resident instance. Each
step is timed with CUDA events on the engine's stream; between steps the L2
is flushed by writing a 512 MiB buffer (outside the timed region). With N
GPUs every rank places its own instance (replicas, seeds differ) and the
value is all iterations over the max rank time.

`--impl reference` times the CPU restatement of the reference path (the
oracle port; the Rust reference cannot be built here) on the host cores.

Besides the headline, the JSON line carries: `e2e` (the placement through
texo_gp_place from host buffers), `roofline` (with per-stage rooflines and
the persistent kernel's phase clocks), `cpu_baseline`, `batched` (64 mixed
instances), `serving` (Poisson request stream), `precision` (1M cells, three
DCT forms against FP64), `quadratic_seed` (the coarse seed's PCG solve) and
`rudy` (the continuous routing-demand map), `auction` (the legalizer's
single-BEL auction on the placement's targets) and `clustering` (the
register-clustering areas). `--stage-report`, `--batch-only`,
`--serve-only`, `--precision-only`, `--seed-only`, `--rudy-only`,
`--auction-only`, `--clustering-only` and `--ecp5-only` (the device-snapshot
adapter, placement and projection on an ECP5-like fabric) print one of these
alone.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (side, cells, io, nets, sigma, bins, target density, gamma base, cap)
    "lfe5u-85-42k": (210, 42000, 365, 50000, 12.0, 256, 0.9, 4.0, 1000),
    "ecp5-2k": (48, 2000, 96, 2400, 6.0, 64, 1.0, 4.0, 300),
    "stress-1m": (1024, 1000000, 4096, 1200000, 24.0, 1024, 0.9, 4.0, 1000),
}
METRIC = "GP iters/s at 42k cells"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def make_problem(name, seed, lib=None):
    """The seeded synthetic netlist of a workload. `lib` is the library whose
    generator runs (the engine's by default; the reference arm passes the
    oracle library, which carries the same generator, so that it never loads
    the engine)."""
    from texo_gb300 import problem as P
    side, cells, io, nets, sigma = WORKLOADS[name][:5]
    return P.synthetic(side, cells, io, nets, sigma, seed, lib=lib)


def make_params(name, engine, dct):
    from texo_gb300.placer import default_params
    _, _, _, _, _, bins, td, gamma, cap = WORKLOADS[name]
    return default_params(bins_x=bins, bins_y=bins, target_density=td, gamma_base=gamma,
                          max_iterations=cap, best_effort=1, engine=engine, dct_mode=dct)


def problem_bytes(p):
    arrs = [p.capacity, p.initial_xy, p.lower_xy, p.upper_xy, p.member_ptr, p.member_field,
            p.member_offset_xy, p.member_charge, p.member_cell, p.cell_unit, p.cell_offset_xy,
            p.cell_fixed, p.cell_fixed_xy, p.net_ptr, p.pin_cell]
    return int(sum(a.nbytes for a in arrs))


# Algorithmic (compulsory) bytes per launch of each stage: every input read
# once and every output written once, at the sizes of the instance and the
# device's data types (float2 positions and gradients, float preconditioner,
# int32 indices, int64 fixed-point grids read-modify-written by the atomics).
# U units, F fillers, M density members, B bins, E nets, P pins, K fields.
# The GEMM forms of the DCT take four passes (rows, columns, columns, rows);
# the FFT form takes three: rows forward, one column pass (forward, scale by
# the inverse eigenvalues, inverse) and rows inverse with the energy.
def stage_bytes(stage, n):
    U, F, M, B, E, P, K = n["U"], n["F"], n["M"], n["B"], n["E"], n["P"], n["K"]
    nobj = U + F
    grids = 2 if F else 1                     # phys, and fill when there are fillers
    if n.get("dct_form") == 3 and stage.startswith("dct_"):
        # the FFT form keeps t1 / t2 as double-float pairs (8 B a bin)
        return {"dct_rows_fwd": K * B * (4 + 8), "dct_cols": K * B * (8 + 8) + B * 4,
                "dct_rows_inv": K * B * (8 + 4 + 4)}.get(stage, 0)
    return {
        "init": K * B * (8 + 8 + 8) + U * 16,                            # phys, fill := -capfix, 0; WA grads := 0
        "scatter": M * 20 + U * 8 + F * 16 + K * B * 16 * grids,         # members, positions, grid RMW
        "wa": P * 12 + E * 8 + U * 8 + U * 32,                           # pins, nets, positions, int64 grad RMW
        "prep": K * B * (8 + 8 + 4),                                     # phys + fill -> rho
        "dct_row_fwd": K * B * 4 * 2,
        "dct_col_fwd": K * B * 4 * 2,
        "dct_col_inv": K * B * 4 * 2 + B * 4,
        "dct_row_inv": K * B * 4 * 3,
        "gather": U * (4 + 8 + 8 * K) + M * 16 + F * (16 + 8) + K * B * 4,
        "combine": U * 16 + nobj * (8 * K + 8) + F * 4,                  # WA grads, field grads -> gradient
        "extrapolate": nobj * (8 * 4 + 8),                               # x, x_prev, lo, hi -> y
        "candidate": nobj * (8 * 4 + 4 + 8),                             # y, g, lo, hi, P -> c
        "kkt": nobj * (8 * 4 + 4),                                       # x, g, lo, hi, P
        "precond": nobj * (4 + 4 * K + 4),                               # static + per-field charge -> P
        "finalize": 0,
    }.get(stage, 0)


def aggregate_ranks(total_ms, steps, dist=None, device="cuda"):
    """Replicas: every rank places its own instance (seeded by its rank); the
    whole-job value is all ranks' steps over the slowest rank's time."""
    import torch
    world = dist.get_world_size() if dist else 1
    t = torch.tensor([total_ms], dtype=torch.float64, device=device)
    if dist:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    max_ms = float(t.item())
    return max_ms, world * steps / (max_ms / 1000.0)


FFT_PASSES = {"dct_row_fwd": "dct_rows_fwd", "dct_col_fwd": "dct_cols", "dct_row_inv": "dct_rows_inv"}


def dct_stages(n):
    return list(FFT_PASSES.values()) if n.get("dct_form") == 3 else [
        "dct_row_fwd", "dct_col_fwd", "dct_col_inv", "dct_row_inv"]


def named_stages(times, n):
    """Stage times under the names of the instance's DCT form (the FFT form's
    third pass slot is empty and dropped)."""
    if n.get("dct_form") != 3:
        return dict(times)
    return {FFT_PASSES.get(k, k): v for k, v in times.items() if k != "dct_col_inv"}


def eval_bytes(n, persistent=False):
    """Algorithmic bytes of one objective evaluation (all its stages). In the
    persistent engine the density preparation is folded into the first
    transform (phys + fill read, rho and the transform written: 24 B a bin
    instead of 20 + 8), and the combine also reads the KKT inputs (position,
    bounds, preconditioner: 28 B an object)."""
    st = ["init", "scatter", "wa", "prep"] + dct_stages(n) + ["gather", "combine"]
    total = sum(stage_bytes(k, n) for k in st)
    if persistent:
        total += (n["U"] + n["F"]) * 28
        total -= n["K"] * n["B"] * 4
    return total


def reused_eval_bytes(n):
    """Algorithmic bytes of an evaluation that reuses the density side of the
    same coordinates: WA gradients zeroed, WA, and the combine with its KKT
    inputs (persistent engine)."""
    return n["U"] * 16 + stage_bytes("wa", n) + stage_bytes("combine", n) + (n["U"] + n["F"]) * 28


def ncu_traffic(workload, engine):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary of this workload (a `traffic_bytes_per_launch: N` line), if any."""
    import re
    path = os.path.join(ROOT, "profiles", "persistent_%s.txt" % workload if engine == "device"
                        else "stages_%s.txt" % workload)
    try:
        with open(path) as f:
            m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", f.read())
        return float(m.group(1)) if m else None
    except OSError:
        return None


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.rows = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            for line in out.strip().splitlines():
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9:
                    self.rows.append(f)

    def summary(self):
        rows = getattr(self, "rows", [])
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_baseline(name, seconds=15.0, threads=None):
    """The oracle (CPU restatement) on a bounded sample of the same workload."""
    from oracle import ffi
    p = make_problem(name, 0, lib=ffi.lib())
    prm = make_params(name, 0, 0)
    threads = threads or max(1, min(os.cpu_count() or 1, 5))
    o = ffi.Oracle(p, prm)
    iters, total = 0, 0.0
    sample = 4
    while total < seconds:
        t = time.perf_counter()
        st, _, _, s = o.place(threads=threads, max_iterations=sample)
        dt = time.perf_counter() - t
        iters += s.iterations
        total += dt
        if s.iterations < sample:
            break
        sample = min(sample * 2, 64)
    return {"value": iters / total, "unit": "iter/s", "cores": threads, "nproc": os.cpu_count(), "kind": "port",
            "sample": "%d oracle iterations from the start of the %s placement (%.1f s)" % (iters, name, total)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    # the reference's own parallel shape (WA beside the density side, WA in
    # four axis tasks) keeps five threads busy; more cores give it nothing
    threads = max(1, min(os.cpu_count() or 1, 5))
    from oracle import ffi
    p = make_problem(args.workload, 0, lib=ffi.lib())
    prm = make_params(args.workload, 0, 0)
    o = ffi.Oracle(p, prm)
    sample = args.reference_sample
    for _ in range(args.warmup):
        o.place(threads=threads, max_iterations=1)
    iters, total = 0, 0.0
    for _ in range(args.steps):
        t = time.perf_counter()
        _, _, _, s = o.place(threads=threads, max_iterations=sample)
        total += time.perf_counter() - t
        iters += s.iterations
    v = iters / total
    line = {"metric": METRIC, "value": v, "unit": "iter/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config_dict(args),
            "cpu_baseline": {"value": v, "unit": "iter/s", "cores": threads, "nproc": os.cpu_count(),
                             "kind": "port",
                             "sample": "%d-iteration prefix of the placement per step" % sample},
            "e2e": {"value": v, "unit": "iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def batch_workload(n=64, seed0=0, lo=1000, hi=40000, sigma=6.0):
    """Mixed-size instances: cells log-uniform in [lo, hi], fabric side
    ceil(sqrt(cells/0.9)), bin grid the next power of two >= side clamped to
    64..256, 1.2 nets per cell, IO on the perimeter, instance i seeded i."""
    import math
    import numpy as np
    from texo_gb300 import problem as P
    from texo_gb300.placer import default_params
    rng = np.random.default_rng(20261203 + seed0)
    jobs = []
    for i in range(n):
        cells = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        side = math.ceil(math.sqrt(cells / 0.9))
        bins = min(256, max(64, 1 << (side - 1).bit_length()))
        io = min(4 * (side - 1), 2 * side)
        prob = P.synthetic(side, cells, io, int(round(1.2 * cells)), sigma, seed0 + i)
        prm = default_params(bins_x=bins, bins_y=bins, target_density=1.0, gamma_base=4.0, max_iterations=1000,
                             best_effort=1)
        jobs.append((prob, prm))
    return jobs


def run_batched(jobs, chunk=20, device=0):
    """All jobs resident in one batch, advanced `chunk` iterations per launch."""
    import torch
    from texo_gb300.placer import Batch
    b = Batch(hbm_budget=200 << 30, max_slots=len(jobs) + 1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i, (p, prm) in enumerate(jobs):
        assert b.admit(p, i, prm)
    t_admit = time.perf_counter() - t0
    results = {}
    launches = 0
    t_adv = 0.0
    while len(results) < len(jobs):
        ta = time.perf_counter()
        b.advance(chunk)
        t_adv += time.perf_counter() - ta
        launches += 1
        while True:
            r = b.retire()
            if r is None:
                break
            results[r[0]] = r[2]
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    b.close()
    return wall, results, launches, {"admit": t_admit, "advance": t_adv, "retire": wall - t_admit - t_adv}


def run_served(jobs, chunk=20, threads=8):
    """All jobs submitted at once to the serving loop (admission overlaps the
    device work of the jobs already resident)."""
    import torch
    from texo_gb300.placer import Server
    torch.cuda.synchronize()
    with Server(chunk_iterations=chunk, admission_threads=threads) as srv:
        t0 = time.perf_counter()
        for i, (p, prm) in enumerate(jobs):
            srv.submit(p, i, prm)
        results = {}
        while len(results) < len(jobs):
            r = srv.poll(wait_ms=-1)
            results[r[0]] = r[2]
        wall = time.perf_counter() - t0
    return wall, results


def run_serial(jobs, engine):
    import torch
    from texo_gb300.placer import Placer
    total_ms, results = 0.0, {}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i, (p, prm) in enumerate(jobs):
        prm.engine = engine
        g = Placer(p, prm)
        try:
            _, _, s = g.run(allow_nonconverged=True)
        except Exception as e:  # a placement error of this job; keep measuring the rest
            s = {"status": getattr(e, "name", str(e)), "hpwl": None, "iterations": 0, "elapsed_ms": 0.0,
                 "converged": False}
        total_ms += s["elapsed_ms"]
        results[i] = s
        g.close()
    torch.cuda.synchronize()
    return time.perf_counter() - t0, results


def batch_report(n=64):
    import numpy as np
    from texo_gb300 import abi
    jobs = batch_workload(n)
    wall_b, res_b, launches, parts = run_batched(jobs)
    wall_s, res_s = run_served(batch_workload(n))
    wall_d, res_d = run_serial(batch_workload(n), abi.ENGINE_DEVICE)
    wall_h, res_h = run_serial(batch_workload(n), abi.ENGINE_HOST)
    same = sum(1 for i in range(n) if res_b[i]["hpwl"] == res_d[i]["hpwl"])
    same_s = sum(1 for i in range(n) if res_s[i]["hpwl"] == res_d[i]["hpwl"])
    iters = sum(s["iterations"] for s in res_b.values())
    # the batched kernels' roofline: every job's algorithmic bytes (its full
    # and density-reusing evaluations, line-search trials and vector updates,
    # as for the single instance) over the time spent advancing the batch
    total_bytes = 0.0
    for i, (p, prm) in enumerate(jobs):
        st = res_b[i]
        if not st.get("iterations"):
            continue
        nj = dict(U=p.num_units, F=int(np.count_nonzero(p.capacity)), M=int(p.member_ptr[-1]),
                  B=prm.bins_x * prm.bins_y, Hb=prm.bins_y, E=p.num_nets, P=p.num_pins, K=len(p.fields))
        ev, dv, tr = st["evaluations"], st["density_evaluations"], st["line_search_trials"]
        total_bytes += (dv * eval_bytes(nj, persistent=True) + (ev - dv) * reused_eval_bytes(nj)
                        + tr * stage_bytes("candidate", nj)
                        + st["iterations"] * (stage_bytes("precond", nj) + stage_bytes("extrapolate", nj)))
    peak, peak_kind = peaks()
    adv = parts["advance"]
    failed = {i: s["status"] for i, s in res_b.items() if s["status"] not in ("OK", "DID_NOT_CONVERGE")}
    return {"instances": n, "cells": "log-uniform 1k..40k", "placements_per_s_served": n / wall_s,
            "speedup_served_vs_serial_host_fp32": wall_h / wall_s,
            "served_identical_to_alone": "%d/%d" % (same_s, n), "placements_per_s_batched": n / wall_b,
            "placements_per_s_serial_device_engine": n / wall_d,
            "placements_per_s_serial_host_engine_fp32": n / wall_h,
            "speedup_vs_serial_host_fp32": wall_h / wall_b, "iterations_per_s_batched": iters / wall_b,
            "batched_launches": launches, "identical_to_alone": "%d/%d" % (same, n), "failed": failed,
            "converged": sum(1 for s in res_b.values() if s["converged"]),
            "wall_s": {"served": wall_s, "batched": wall_b, "serial_device": wall_d, "serial_host": wall_h},
            "batched_wall_split_s": parts,
            "batched_roofline": {"algorithmic_bytes": total_bytes, "advance_s": adv,
                                 "achieved_gbs": total_bytes / adv / 1e9 if adv > 0 else None,
                                 "peak_gbs": peak, "peak_source": peak_kind,
                                 "frac": total_bytes / adv / 1e9 / peak if adv > 0 else None,
                                 "time": "wall time of the advance calls (the launches and their "
                                         "state copies, host staging included)"}}


def serve_request(i, lo=2000, hi=100000, sigma=6.0):
    """Request i of the serving stream: cells log-uniform in [lo, hi] drawn
    from a generator seeded by the request id, the netlist seeded by it too;
    fabric, bins and nets as in the mixed-instance batch."""
    import math
    import numpy as np
    from texo_gb300 import problem as P
    from texo_gb300.placer import default_params
    rng = np.random.default_rng(1000003 + i)
    cells = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
    side = math.ceil(math.sqrt(cells / 0.9))
    bins = min(256, max(64, 1 << (side - 1).bit_length()))
    io = min(4 * (side - 1), 2 * side)
    prob = P.synthetic(side, cells, io, int(round(1.2 * cells)), sigma, i)
    prm = default_params(bins_x=bins, bins_y=bins, target_density=1.0, gamma_base=4.0, max_iterations=1000,
                         best_effort=1)
    return prob, prm


def serve_report(n_requests=200, probe=32, load=0.8, oracle_sample=6, seed=7):
    """Serving stream: Poisson arrivals at `load` x the measured batched
    capacity of the same request distribution; placements/s and p50/p99
    time-to-converge (submit to retire) of `n_requests` requests; final HPWL
    of a size-stratified sample of requests (smallest to largest) against the
    FP64 oracle."""
    import threading
    import numpy as np
    from texo_gb300.placer import Server
    # capacity: `probe` requests of the same distribution submitted at once
    wall, _ = run_served([serve_request(100000 + k) for k in range(probe)])
    capacity = probe / wall
    rate = load * capacity
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_requests))
    sizes = {}
    results = {}
    with Server(chunk_iterations=20, admission_threads=8) as srv:
        def producer():
            t0 = time.perf_counter()
            for i in range(n_requests):
                prob, prm = serve_request(i)
                sizes[i] = prob.num_units
                delay = arrivals[i] - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
                srv.submit(prob, i, prm)
        th = threading.Thread(target=producer)
        th.start()
        while len(results) < n_requests:
            r = srv.poll(wait_ms=1000)
            if r is not None:
                results[r[0]] = r[2]
        th.join()
    lat = np.array([results[i]["finish_ms"] - results[i]["submit_ms"] for i in range(n_requests)])
    first = min(results[i]["submit_ms"] for i in range(n_requests))
    last = max(results[i]["finish_ms"] for i in range(n_requests))
    ok = [i for i in range(n_requests) if results[i]["status"] in ("OK", "DID_NOT_CONVERGE")]
    conv = [i for i in ok if results[i]["converged"]]
    within = [i for i in ok if max(results[i]["overflow"] or [0.0]) <= 0.10]
    report = {"requests": n_requests, "cells": "log-uniform 2k..100k", "arrivals": "Poisson",
              "offered_per_s": rate, "measured_capacity_per_s": capacity, "load": load,
              "placements_per_s": n_requests / ((last - first) / 1000.0),
              "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
              "converged": len(conv), "overflow_le_0.10": len(within), "failed": n_requests - len(ok)}
    # FP64 oracle on a size-stratified sample: the smallest, the largest and
    # evenly spaced size quantiles between; relative final-HPWL difference
    try:
        from oracle import ffi
        by_size = sorted(ok, key=lambda i: sizes[i])
        picks = sorted({by_size[round(q * (len(by_size) - 1))] for q in np.linspace(0.0, 1.0, oracle_sample)}) \
            if by_size else []
        errs, jobs = [], []
        for i in picks:
            prob, prm = serve_request(i)
            st, _, _, s = ffi.Oracle(prob, prm).place(threads=5)
            if s.hpwl > 0:
                e = abs(results[i]["hpwl"] - s.hpwl) / s.hpwl
                errs.append(e)
                jobs.append({"request": int(i), "units": int(sizes[i]), "rel_err": e})
        report["hpwl_rel_err_vs_fp64_oracle"] = {"jobs": len(errs), "max": max(errs) if errs else None,
                                                 "mean": float(np.mean(errs)) if errs else None,
                                                 "sample": "%d requests at evenly spaced size quantiles "
                                                           "(smallest to largest)" % len(errs),
                                                 "per_job": jobs}
    except Exception as e:  # the oracle is optional on the box
        report["hpwl_rel_err_vs_fp64_oracle"] = {"error": str(e)}
    return report


def stage_report(workload, dct_name, reps):
    """Every stage kernel of the host engine on `workload`, timed at the
    positions one placement ends at (cells spread at overflow <= 0.10):
    each kernel launched `reps` times back to back (CUDA events; inputs
    that fit in L2 stay there between launches), with its algorithmic bytes
    and their rate against the measured HBM peak. The launches are inside
    the NVTX range "stages", so an ncu capture can select them with
    --nvtx --nvtx-include stages/."""
    import torch
    from texo_gb300 import abi
    from texo_gb300.placer import Placer
    dct = {"fp32": abi.DCT_FP32, "tensor": abi.DCT_TENSOR, "bf16x3": abi.DCT_TENSOR, "fp32-gemm": abi.DCT_FP32_GEMM}[dct_name]
    prob = make_problem(workload, 0)
    prm = make_params(workload, abi.ENGINE_HOST, dct)
    peak, kind = peaks()
    with Placer(prob, prm) as g:
        _, _, s = g.run(allow_nonconverged=True)
        n = dict(U=g.units, F=g.num_fillers, M=int(prob.member_ptr[-1]), B=g.bins, Hb=g.bins_y,
                 E=prob.num_nets, P=prob.num_pins, K=g.num_fields, dct_form=g.dct_form())
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("stages")
        st = named_stages(g.stage_times(reps=reps), n)
        torch.cuda.nvtx.range_pop()
    out = {}
    for k, ms in st.items():
        b = stage_bytes(k, n)
        out[k] = {"us": round(ms * 1000, 2), "algorithmic_bytes": b,
                  "gbs": round(b / (ms * 1e-3) / 1e9, 1) if ms > 0 and b else None,
                  "frac": round(b / (ms * 1e-3) / 1e9 / peak, 4) if ms > 0 and b else None}
    return {"metric": "stage kernels at placed positions", "workload": workload, "engine": "host",
            "dct_form": Placer.DCT_FORMS[n["dct_form"]], "sizes": n, "placement_iterations": s["iterations"],
            "final_overflow": s["overflow"], "reps": reps, "peak_gbs": peak, "peak_source": kind,
            "stages": out}


def seed_report(workload="lfe5u-85-42k", reps=5):
    """The coarse quadratic seed's solve (`solve_quadratic`, lib.rs:4586-4752)
    on the bound-to-bound system of `workload` at its initial positions (x
    axis, fixed IO anchored, floating components gauged): the GPU solve
    through texo_gp_quadratic_solve (device time with the copies, and wall
    time of the call from host arrays) against the FP64 oracle restatement
    on one host core (the reference's solve is sequential)."""
    import numpy as np
    from oracle import ffi
    from texo_gb300 import seed
    from texo_gb300.placer import quadratic_solve
    prob = make_problem(workload, 0)
    pos = np.asarray(prob.initial_xy).reshape(-1, 2)
    d, ptr, idx, w, rhs, anch = seed.axis_system(prob, pos, 0)
    d, ptr, idx, w, rhs, floating = seed.finalize_gauges(d, ptr, idx, w, rhs, anch)
    x0 = pos[:, 0].copy()
    for comp in floating:
        x0[comp] -= x0[comp[0]]
    ptr32, idx32 = ptr.astype(np.uint32), idx.astype(np.uint32)
    quadratic_solve(d, ptr32, idx32, w, rhs, x0)   # warm-up (module load, pool)
    gpu_ms, wall_ms = [], []
    for _ in range(reps):
        t0 = time.perf_counter()
        xg, sg = quadratic_solve(d, ptr32, idx32, w, rhs, x0)
        wall_ms.append(1000 * (time.perf_counter() - t0))
        gpu_ms.append(sg["elapsed_ms"])
    t0 = time.perf_counter()
    xr, sr, ok = ffi.solve_quadratic(d, ptr32, idx32, w, rhs, x0)
    cpu_ms = 1000 * (time.perf_counter() - t0)
    nnz = int(ptr[-1])
    # algorithmic bytes of one CG step: the product reads D, the row pointers,
    # the adjacency (index + weight) and the direction, writes q; the updates
    # read p, q, x, r, D and write x, r, z; the direction update reads z, p
    # and writes p (FP64 vectors, int32 indices)
    n = len(d)
    step_bytes = (8 * n + 4 * (n + 1) + 12 * nnz + 8 * n + 8 * n) + (8 * 5 * n + 8 * 3 * n) + (8 * 3 * n)
    best = min(gpu_ms)
    return {"workload": workload, "axis": "x", "units": n, "adjacency_entries": nnz,
            "floating_components": len(floating),
            "gpu": {"iterations": sg["iterations"], "restarts": sg["restarts"], "stop": sg["stop"],
                    "device_ms": best, "wall_ms": min(wall_ms),
                    "relative_residual": float(np.sqrt(sg["final_residual_squared"] / sg["initial_residual_squared"])),
                    "step_gbs": step_bytes * sg["iterations"] / (best * 1e-3) / 1e9},
            "cpu_oracle": {"iterations": int(sr.iterations), "ms": cpu_ms, "cores": 1, "converged": bool(ok)},
            "max_rel_diff_vs_oracle": float(np.max(np.abs(xg - xr)) / np.max(np.abs(xr))),
            "speedup_wall_vs_cpu": cpu_ms / min(wall_ms)}


def scatter_report(workloads=("lfe5u-85-42k", "stress-1m"), reps=20):
    """The host engine's two density-scatter forms (direct: nine global int64
    atomics per object; tiled: counting sort by 32 x 32-bin tile, then a
    shared-memory window per run of the sorted order) on each workload, timed
    with CUDA events at the positions one placement ends at (the scatter
    launch group: init excluded; for the tiled form its count, scan, place
    and scatter kernels), with the grids checked equal between the forms."""
    import numpy as np
    from texo_gb300 import abi
    from texo_gb300.placer import Placer
    out = {}
    for wl in workloads:
        prob = make_problem(wl, 0)
        res, grids = {}, []
        for name, mode in (("direct", abi.SCATTER_DIRECT), ("tiled", abi.SCATTER_TILED)):
            prm = make_params(wl, abi.ENGINE_HOST, abi.DCT_FP32)
            prm.scatter_mode = mode
            with Placer(prob, prm) as g:
                _, c, s = g.run(allow_nonconverged=True)
                grids.append(g.scatter(c))
                st = g.stage_times(reps=reps)
                res[name] = {"scatter_us": round(st["scatter"] * 1000, 2), "iterations": s["iterations"]}
        res["grids_identical"] = bool(np.array_equal(grids[0][0], grids[1][0]) and
                                      np.array_equal(grids[0][1], grids[1][1]))
        out[wl] = res
    return out


def probe(spec):
    """Small, targeted workloads for profiler captures (no timing):
    "tc:N" three tensor-core Poisson solves on an N x N bin grid (a 48 x 48
    problem, so little else runs); "scatter:WORKLOAD" two direct and two
    tiled host-engine scatters of WORKLOAD at spread positions."""
    import numpy as np
    from texo_gb300 import abi
    from texo_gb300.placer import Placer, default_params
    kind, arg = spec.split(":")
    if kind == "tc":
        n = int(arg)
        prob = make_problem("ecp5-2k", 0)
        i = np.arange(n * n)
        d = ((i * 31 + 7) % 101) - 50.0 + ((i * 13 + 5) % 17) / 17.0
        with Placer(prob, default_params(dct_mode=abi.DCT_TENSOR, engine=abi.ENGINE_HOST, bins_x=n, bins_y=n)) as g:
            for _ in range(3):
                g.poisson(d)
    elif kind == "scatter":
        prob = make_problem(arg, 0)
        for mode in (abi.SCATTER_DIRECT, abi.SCATTER_TILED):
            prm = make_params(arg, abi.ENGINE_HOST, abi.DCT_FP32)
            prm.scatter_mode = mode
            with Placer(prob, prm) as g:
                c, lo, hi = g.initial()
                c = lo + (hi - lo) * np.random.default_rng(1).random(c.size)
                for _ in range(2):
                    g.scatter(c)
    else:
        raise SystemExit("unknown probe " + spec)
    return {"probe": spec, "ok": True}


def rudy_report(reps=5):
    """Continuous RUDY demand (`continuous_routing_demand`, eplace.rs:856-937)
    of the 42k workload's net boxes at its placed positions (one device-engine
    placement), on the GPU against the FP64 oracle on one host core (the
    reference's loop is sequential); and of the 1M-cell workload's boxes at
    uniform positions on the GPU, checked against the oracle on a 20,000-box
    sample."""
    import numpy as np
    from oracle import ffi
    from texo_gb300 import abi
    from texo_gb300.placer import Placer, net_bounding_boxes, routing_demand
    out = {}
    prob = make_problem("lfe5u-85-42k", 0)
    with Placer(prob, make_params("lfe5u-85-42k", abi.ENGINE_DEVICE, abi.DCT_FP32)) as g:
        _, coords, _ = g.run(allow_nonconverged=True)
    side = WORKLOADS["lfe5u-85-42k"][0]
    boxes = net_bounding_boxes(prob, coords[: 2 * prob.num_units].reshape(-1, 2))
    routing_demand(side, side, boxes)   # warm-up
    ms = []
    for _ in range(reps):
        h, v, m = routing_demand(side, side, boxes)
        ms.append(m)
    t0 = time.perf_counter()
    hr, vr, ok = ffi.routing_demand(side, side, boxes)
    cpu_ms = 1000 * (time.perf_counter() - t0)
    out["lfe5u-85-42k"] = {"grid": "%dx%d" % (side, side), "boxes": int(len(boxes)), "positions": "placed",
                           "gpu_ms": min(ms), "cpu_oracle_ms": cpu_ms, "cores": 1,
                           "speedup": cpu_ms / min(ms),
                           "max_abs_diff": float(max(np.max(np.abs(h - hr)), np.max(np.abs(v - vr)))),
                           "max_demand": float(max(hr.max(), vr.max()))}
    prob = make_problem("stress-1m", 0)
    side = WORKLOADS["stress-1m"][0]
    pos = np.random.default_rng(0).uniform(0, side - 1, size=(prob.num_units, 2))
    boxes = net_bounding_boxes(prob, pos)
    routing_demand(side, side, boxes)
    ms = []
    for _ in range(reps):
        h, v, m = routing_demand(side, side, boxes)
        ms.append(m)
    sample = boxes[:20000]
    hs, vs, _ = routing_demand(side, side, sample)
    t0 = time.perf_counter()
    hr, vr, ok = ffi.routing_demand(side, side, sample)
    cpu_ms = 1000 * (time.perf_counter() - t0)
    out["stress-1m"] = {"grid": "%dx%d" % (side, side), "boxes": int(len(boxes)), "positions": "uniform",
                        "gpu_ms": min(ms), "oracle_sample_boxes": len(sample),
                        "oracle_sample_ms": cpu_ms,
                        "sample_max_abs_diff": float(max(np.max(np.abs(hs - hr)), np.max(np.abs(vs - vr))))}
    return out


def auction_report(reps=5, workloads=("lfe5u-85-42k", "stress-1m")):
    """The single-BEL capacity auction of the legalizer (`assign_implicitly`,
    legalization/auction.rs:131-247, with the ring walk of mod.rs:876-1021)
    on the rounded targets of each workload's placement (the 42k workload on
    the device engine, 1M cells on the host engine): the GPU's parallel
    auction (device time with the copies, best of `reps`) at the default and
    at the reference's cost scale, against the oracle's one-bidder-at-a-time
    auction on one host core, with the epsilon-optimality certificate of each
    GPU result."""
    import numpy as np
    from oracle import ffi
    from texo_gb300 import abi, legalize
    from texo_gb300.placer import Placer, net_bounding_boxes
    out = {}
    for name in workloads:
        prob = make_problem(name, 0)
        engine = abi.ENGINE_DEVICE if name == "lfe5u-85-42k" else abi.ENGINE_HOST
        with Placer(prob, make_params(name, engine, abi.DCT_FP32)) as g:
            targets, _, _ = g.run(allow_nonconverged=True)
        lo = prob.lower_xy.reshape(-1, 2)
        hi = prob.upper_xy.reshape(-1, 2)
        movable = np.nonzero(np.any(lo != hi, axis=1))[0]
        grid = legalize.site_grid(prob.capacity[0].reshape(1, prob.height, prob.width))
        kind = np.zeros(len(movable), np.uint32)
        xy = np.ascontiguousarray(targets[movable])
        n = len(movable)

        def gpu(scale):
            legalize.auction_singletons(grid, kind, xy, cost_scale=scale)   # warm-up
            runs, walls = [], []
            for _ in range(reps):
                t0 = time.perf_counter()
                runs.append(legalize.auction_singletons(grid, kind, xy, cost_scale=scale))
                walls.append(1000 * (time.perf_counter() - t0))
            best = min(runs, key=lambda r: r.stats["elapsed_ms"])
            st = best.stats
            bad, _, _ = ffi.auction_certificate(grid, kind, xy, best.assignment, best.prices,
                                                cost_scale=st["cost_scale"])
            return {"cost_scale": st["cost_scale"], "gpu_ms": st["elapsed_ms"], "gpu_wall_ms": min(walls),
                    "hpwl_legal": hpwl(best.assignment),
                    "rounds": st["rounds"], "tail_rounds": st["tail_rounds"], "bids": st["bids"],
                    "candidates_examined": st["candidates_examined"],
                    "unmatched": st["unmatched"], "total_displacement": st["total_base_cost"],
                    "mean_displacement": st["total_base_cost"] / max(n, 1),
                    "deterministic_over_reps": all(np.array_equal(r.assignment, best.assignment) for r in runs),
                    "certificate_violations": int(bad)}

        def cpu(scale):
            t0 = time.perf_counter()
            code, a, _, ost = ffi.auction_singletons(grid, kind, xy, cost_scale=scale)
            ms = 1000 * (time.perf_counter() - t0)
            return {"cost_scale": scale, "cpu_ms": ms, "status": int(code), "bids": ost["bids"],
                    "hpwl_legal": hpwl(a) if code == 0 else None,
                    "unmatched": ost["unmatched"], "total_displacement": ost["total_base_cost"]}

        def hpwl(assignment):
            # half-perimeter wirelength over the nets between units with every
            # movable unit at the tile of its BEL (net_bounding_boxes' nets)
            pos = np.array(prob.lower_xy, dtype=np.float64).reshape(-1, 2)
            if assignment is None:
                pos[movable] = xy
            else:
                where = grid.bel_tiles()
                pos[movable, 0] = where[assignment, 1]
                pos[movable, 1] = where[assignment, 2]
            b = net_bounding_boxes(prob, pos)
            return float(np.sum(b[:, 1] - b[:, 0]) + np.sum(b[:, 3] - b[:, 2]))

        default, like = gpu(0), gpu(1)
        ref = cpu(1)
        ref_scaled = cpu(default["cost_scale"]) if default["cost_scale"] != 1 else ref
        out[name] = {"bidders": int(n), "bels": int(grid.num_objects),
                     "grid": "%dx%d" % (prob.width, prob.height),
                     "targets": "rounded targets of the %s-engine placement" % (
                         "device" if engine == abi.ENGINE_DEVICE else "host"),
                     "hpwl_targets": hpwl(None),
                     "gpu": default, "gpu_reference_scale": like, "cpu_oracle": ref,
                     "cpu_oracle_same_scale": ref_scaled, "cores": 1,
                     "speedup_vs_reference_setting": ref["cpu_ms"] / default["gpu_ms"],
                     "speedup_same_scale": ref_scaled["cpu_ms"] / default["gpu_ms"],
                     "displacement_vs_reference_setting":
                         default["total_displacement"] / max(ref["total_displacement"], 1)}
    return out


def ecp5_report(side=104, seed=0):
    """The path from a device snapshot to legal BEL choices on an ECP5-like
    fabric of LFE5U-85 size (side x side tiles, 102^2 PLC tiles of 8 LUT4 +
    8 FF: 83,232 LUTs; seeded synthetic snapshot and netlist, the real
    device database being unavailable): the adapter (snapshot read, choice
    generators, placement problem), the placement on the device engine, and
    `project` with the GPU auctions against the same composition with the
    oracle's one-bidder-at-a-time auctions (the reference's) on one host
    core. The product runs the composition in native code
    (`texo_gp_project`); its per-auction detail comes from the same steps
    driven from Python."""
    import numpy as np
    from oracle import ffi
    from texo_gb300 import ecp5, legalize
    from texo_gb300.placer import default_params, place
    t0 = time.perf_counter()
    arch = ecp5.read_architecture(ecp5.synthetic_architecture(side, side))
    t1 = time.perf_counter()
    nc, units, kinds, nets = ecp5.synthetic_design(arch, seed, luts=30000, ffs=12000, lut_ff_pairs=8000,
                                                   carry=((400, 4), (100, 6)), io=300)
    t2 = time.perf_counter()
    prob, _ = ecp5.placement_problem(arch, nc, units, nets, cell_kind=kinds)
    t3 = time.perf_counter()
    targets, _, st = place(prob, default_params(best_effort=1))
    t4 = time.perf_counter()
    bel_xy = np.stack([arch.bel_x, arch.bel_y], 1)
    timed = {"gpu": 0.0, "cpu": 0.0}
    calls = []

    def gpu_auction(grid, k, tg, scale):
        r = legalize.auction_singletons(grid, k, tg, cost_scale=scale)
        timed["gpu"] += r.stats["elapsed_ms"]
        calls.append({"bidders": int(len(k)), "objects": int(grid.num_objects), "kinds": int(grid.num_kinds),
                      **{f: r.stats[f] for f in ("cost_scale", "rounds", "tail_rounds", "bids", "elapsed_ms",
                                                 "total_base_cost", "unmatched")}})
        return r.assignment, r.stats

    def cpu_auction(grid, k, tg, scale):
        c0 = time.perf_counter()
        code, a, _, s = ffi.auction_singletons(grid, k, tg, cost_scale=max(int(scale), 1))
        timed["cpu"] += 1000 * (time.perf_counter() - c0)
        if code != 0:
            raise RuntimeError("oracle auction status %d" % code)
        return a, s
    legalize.project(arch.width, arch.height, bel_xy, units, targets)   # warm-up
    p0 = time.perf_counter()
    g = legalize.project(arch.width, arch.height, bel_xy, units, targets)   # native composition, GPU auctions
    p1 = time.perf_counter()
    gpu_default_ms = g.stats["elapsed_ms"]
    legalize.project(arch.width, arch.height, bel_xy, units, targets, auction=gpu_auction)
    calls_default = list(calls)
    calls.clear()
    timed["gpu"] = 0.0
    g1 = legalize.project(arch.width, arch.height, bel_xy, units, targets, cost_scale=1, auction=gpu_auction)
    calls_s1 = list(calls)
    gpu_s1_ms = timed["gpu"]
    p1b = time.perf_counter()
    r = legalize.project(arch.width, arch.height, bel_xy, units, targets, cost_scale=1, auction=cpu_auction)
    p2 = time.perf_counter()

    def displacement(pj):
        d = 0
        for u, unit in enumerate(units):
            if len(unit.choices) > 1 and pj.preferred[u] >= 0:
                x, y = bel_xy[unit.choices[pj.preferred[u]][0]]
                d += abs(int(x) - int(targets[u][0])) + abs(int(y) - int(targets[u][1]))
        return d
    bels = g.bels(units)
    # the repair (texo_gp_repair, host code) of the GPU projection, and of the
    # same projection with every tenth movable unit unmatched
    fixed = [len(u.choices) == 1 for u in units]
    q0 = time.perf_counter()
    placed, rs = legalize.repair(arch.width, arch.height, bel_xy, units, targets, g.preferred, fixed)
    q1 = time.perf_counter()
    spoiled = np.array(g.preferred)
    spoiled[[u for u in range(len(units)) if not fixed[u] and u % 10 == 0]] = -1
    q2 = time.perf_counter()
    placed2, rs2 = legalize.repair(arch.width, arch.height, bel_xy, units, targets, spoiled, fixed)
    q3 = time.perf_counter()
    # register control sets (clock, LSR, CE) as shared resources
    rules = ecp5.ff_control_set_rules(arch, ecp5.synthetic_control_sets(kinds, seed=1))
    q4 = time.perf_counter()
    placed3, rs3 = legalize.repair(arch.width, arch.height, bel_xy, units, targets, g.preferred, fixed,
                                   legalize.Legality(rules=rules))
    q5 = time.perf_counter()
    ok3 = bool(np.all(placed3 >= 0) and len(np.unique(placed3)) == len(placed3))
    for cell_values, bel_res in rules:
        seen = {}
        for c, v in cell_values.items():
            ok3 = ok3 and seen.setdefault(bel_res[int(placed3[c])], v) == v
    repair = {"wall_ms": 1e3 * (q1 - q0), "initial_pending": rs["initial_pending"],
              "legal": bool(np.all(placed >= 0) and len(np.unique(placed)) == len(placed)),
              "tenth_unmatched": {"wall_ms": 1e3 * (q3 - q2), "initial_pending": rs2["initial_pending"],
                                  "states_visited": rs2["states_visited"], "units_evicted": rs2["units_evicted"],
                                  "legal": bool(np.all(placed2 >= 0) and len(np.unique(placed2)) == len(placed2))},
              "control_sets": {"registers": len(rules[0][0]) if rules else 0, "wall_ms": 1e3 * (q5 - q4),
                               "initial_pending": rs3["initial_pending"], "states_visited": rs3["states_visited"],
                               "units_evicted": rs3["units_evicted"], "legal": ok3}}
    return {"fabric": "%dx%d" % (side, side), "bels": arch.num_bels, "cells": nc, "units": len(units),
            "nets": prob.num_nets, "stats": g.stats,
            "adapter_s": {"read_snapshot": t1 - t0, "design": t2 - t1, "placement_problem": t3 - t2},
            "placement": {"wall_s": t4 - t3, "iterations": st["iterations"], "converged": st["converged"],
                          "hpwl": st["hpwl"], "overflow": st["overflow"]},
            "project_gpu": {"wall_s": p1 - p0, "auction_gpu_ms": gpu_default_ms, "unplaced": int(np.sum(g.preferred < 0)),
                            "legal": bool(len(np.unique(bels[bels >= 0])) == int(np.sum(bels >= 0))),
                            "total_displacement": displacement(g), "auctions": calls_default},
            "repair": repair,
            "project_gpu_reference_scale": {"auction_gpu_ms": gpu_s1_ms, "total_displacement": displacement(g1),
                                            "auctions": calls_s1},
            "project_reference_auctions": {"wall_s": p2 - p1b, "auction_cpu_ms": timed["cpu"], "cores": 1,
                                           "unplaced": int(np.sum(r.preferred < 0)),
                                           "total_displacement": displacement(r)}}


def routable_report(side=48, seed=0, capacity=10):
    """`eplace::place` with a routing-capacity map (texo_gp_place_routable:
    the area rounds, RUDY and register-clustering proposals, their
    installation) on the ECP5 adapter's problem for a side x side fabric
    (seeded synthetic snapshot and netlist; every register with a seeded
    control set; `capacity` routing tracks per tile edge in each direction),
    on the host-driven engine and on the persistent device engine."""
    import numpy as np
    from texo_gb300 import ecp5
    from texo_gb300.placer import default_params, place_with_routing_capacity
    arch = ecp5.read_architecture(ecp5.synthetic_architecture(side, side))
    n_plc = (side - 2) ** 2
    nc, units, kinds, nets = ecp5.synthetic_design(arch, seed, luts=2 * n_plc, ffs=n_plc,
                                                   lut_ff_pairs=n_plc, carry=((n_plc // 40, 4),), io=4 * side)
    prob, _ = ecp5.placement_problem(arch, nc, units, nets, cell_kind=kinds)
    controls = {c: (clk, lsr, ce) for c, ce, clk, lsr in ecp5.synthetic_control_sets(kinds, seed)}
    cap = np.full((arch.height, arch.width), capacity, np.uint32)
    from texo_gb300 import abi
    out = {"fabric": "%dx%d" % (side, side), "cells": nc, "units": len(units), "nets": prob.num_nets,
           "registers": len(controls), "capacity_per_tile": capacity}
    for name, engine in (("host_engine", abi.ENGINE_HOST), ("device_engine", abi.ENGINE_DEVICE)):
        prm = lambda: default_params(best_effort=1, engine=engine)
        try:
            place_with_routing_capacity(prob, prm(), cap, cap, controls)   # warm-up (module loads)
            t0 = time.perf_counter()
            _, _, st, rep = place_with_routing_capacity(prob, prm(), cap, cap, controls)
            t1 = time.perf_counter()
        except abi.TexoGpError as e:
            out[name] = {"error": e.name}
            continue
        out[name] = {"wall_s": t1 - t0, "rounds": rep["rounds"], "area_rounds": rep["area_rounds"],
                     "iterations": rep["iterations"], "hpwl": st["hpwl"], "overflow": st["overflow"],
                     "converged": st["converged"], "last_relative_increase": rep["last_relative_increase"]}
    if "wall_s" in out["host_engine"] and "wall_s" in out["device_engine"]:
        out["device_vs_host_speedup"] = out["host_engine"]["wall_s"] / out["device_engine"]["wall_s"]
    return out


def clustering_report(reps=5):
    """elfPlace's register-clustering areas (`clustering_areas`,
    register_clustering.rs:17-80) for a synthetic register set: one register
    at each movable position of the 42k-cell placement (device engine), 8
    clock / LSR control sets and 16 clock enables drawn with a fixed seed,
    84,000 movable instances (a LUT and a register per site). The GPU runs
    the whole set (device time with the copies, best of `reps`); the oracle
    runs control set 0 alone on one host core, a bounded sample whose areas
    are the same registers' full-set areas (a register's area depends only
    on its control set)."""
    import numpy as np
    from oracle import ffi
    from texo_gb300 import abi
    from texo_gb300 import routability as R
    from texo_gb300.placer import Placer
    prob = make_problem("lfe5u-85-42k", 0)
    with Placer(prob, make_params("lfe5u-85-42k", abi.ENGINE_DEVICE, abi.DCT_FP32)) as g:
        _, coords, _ = g.run(allow_nonconverged=True)
    movable = np.nonzero(np.any(prob.lower_xy != prob.upper_xy, axis=1))[0]
    xy = coords[: 2 * prob.num_units].reshape(-1, 2)[movable]
    rng = np.random.default_rng(7)
    n = len(movable)
    clock_lsr = np.stack([rng.integers(0, 8, n), np.zeros(n, np.int64)], axis=1).astype(np.uint64)
    ce = rng.integers(0, 16, n).astype(np.uint64)
    count = 2 * n
    R.register_clustering_areas(xy, clock_lsr, ce, count)   # warm-up
    runs = [R.register_clustering_areas(xy, clock_lsr, ce, count) for _ in range(reps)]
    areas, _ = runs[0]
    gpu_ms = min(ms for _, ms in runs)
    same = all(np.array_equal(a, areas) for a, _ in runs)
    sample = np.nonzero(clock_lsr[:, 0] == 0)[0]
    t0 = time.perf_counter()
    code, ref = ffi.register_clustering_areas(xy[sample], clock_lsr[sample], ce[sample], count)
    cpu_ms = 1000 * (time.perf_counter() - t0)
    groups = np.bincount(clock_lsr[:, 0].astype(np.int64))
    pairs = int(np.sum(groups.astype(np.int64) ** 2))
    sample_pairs = len(sample) ** 2
    return {"registers": int(n), "control_sets": 8, "clock_enables": 16, "movable_instances": int(count),
            "positions": "movable positions of the 42k device-engine placement", "pairs": pairs,
            "gpu_ms": gpu_ms, "deterministic_over_reps": bool(same),
            "cpu_oracle_sample": {"registers": int(len(sample)), "pairs": int(sample_pairs), "cpu_ms": cpu_ms,
                                  "status": int(code), "cores": 1},
            "cpu_oracle_full_estimate_ms": cpu_ms * pairs / max(sample_pairs, 1),
            "max_rel_diff_vs_oracle": float(np.max(np.abs(areas[sample] - ref) / np.abs(ref))) if code == 0 else None,
            "mean_area": float(np.mean(areas))}


def precision_report(iterations=1000, seed=0, threads=5):
    """Precision stress (1M cells + 4,096 IO on 1024^2 sites, 1.2M nets,
    1024^2 bins, target density 0.9): potential, field gradient and energy of
    the FP32 FFT, FP32 GEMM and tensor-core (integer-slice) DCT forms against the FP64 oracle at
    identical spread positions, gradient cosine similarity, and each form's
    final HPWL / overflow: once run to the stop rule (overflow <= 0.10), and
    once for exactly `iterations` GP iterations (overflow target 0, so the
    stop rule never fires; gamma then follows the target-0 schedule). The
    oracle cannot run 1000 FP64 iterations of this size in a bench, so the
    final HPWL is compared between the GPU forms."""
    import numpy as np
    from oracle import ffi
    from texo_gb300 import abi
    from texo_gb300.placer import Placer
    prob = make_problem("stress-1m", seed)
    prm64 = make_params("stress-1m", abi.ENGINE_HOST, abi.DCT_FP32)
    prm64.max_iterations = iterations
    t0 = time.perf_counter()
    o = ffi.Oracle(prob, prm64)
    c, lo, hi = o.initial()
    c = (lo + (hi - lo) * np.random.default_rng(seed + 1).random(c.size)).astype(np.float32).astype(np.float64)
    gamma = 4.0
    r = o.evaluate(c, gamma, threads=threads)
    t_oracle = time.perf_counter() - t0

    def nw(a, b):
        return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))

    def cos(a, b):
        return float(np.dot(a.ravel(), b.ravel()) / (np.linalg.norm(a) * np.linalg.norm(b)))

    out = {"workload": "stress-1m", "positions": "uniform in the bounds, FP32-representable",
           "oracle_eval_s": t_oracle}
    for name, mode in (("fp32_fft", abi.DCT_FP32), ("fp32_gemm", abi.DCT_FP32_GEMM), ("tensor", abi.DCT_TENSOR)):
        prm = make_params("stress-1m", abi.ENGINE_HOST, mode)
        prm.max_iterations = iterations
        with Placer(prob, prm) as g:
            form = g.dct_form()
            d = g.evaluate(c, gamma)
            st = g.stage_times(reps=5)
            t1 = time.perf_counter()
            _, _, s = g.run(allow_nonconverged=True)
            run_s = time.perf_counter() - t1
        prm_n = make_params("stress-1m", abi.ENGINE_HOST, mode)
        prm_n.max_iterations = iterations
        prm_n.overflow_target_override = 0.0
        with Placer(prob, prm_n) as g:
            t1 = time.perf_counter()
            _, _, sn = g.run(allow_nonconverged=True)
            fixed = {"iterations": sn["iterations"], "final_hpwl": sn["hpwl"], "final_overflow": sn["overflow"],
                     "run_s": time.perf_counter() - t1, "gpu_ms": sn["elapsed_ms"]}
        out[name] = {"after_%d_iterations" % iterations: fixed,"dct_form": form, "potential_max_rel_err": nw(d["potential"], r["potential"]),
                     "field_gradient_max_rel_err": nw(d["field_gradient"], r["field_gradient"]),
                     "field_gradient_cosine": cos(d["field_gradient"], r["field_gradient"]),
                     "wa_gradient_cosine": cos(d["wa_gradient"], r["wa_gradient"]),
                     "energy_rel_err": abs(d["fields"][0].energy - r["fields"][0].energy) / abs(r["fields"][0].energy),
                     "dct_pass_us": {k: round(1000 * v, 2) for k, v in named_stages(st, {"dct_form": form}).items()
                                     if k.startswith("dct_")},
                     "final_hpwl": s["hpwl"], "final_overflow": s["overflow"], "iterations": s["iterations"],
                     "converged": s["converged"], "run_s": run_s, "gpu_ms": s["elapsed_ms"]}
    out["final_hpwl_tensor_vs_fp32_gemm"] = out["tensor"]["final_hpwl"] / out["fp32_gemm"]["final_hpwl"] - 1.0
    out["final_hpwl_fp32_fft_vs_fp32_gemm"] = out["fp32_fft"]["final_hpwl"] / out["fp32_gemm"]["final_hpwl"] - 1.0
    key = "after_%d_iterations" % iterations
    for a, b in (("tensor", "fp32_gemm"), ("fp32_fft", "fp32_gemm")):
        out["%s_hpwl_%s_vs_%s" % (key, a, b)] = out[a][key]["final_hpwl"] / out[b][key]["final_hpwl"] - 1.0
    return out


def config_dict(args):
    side, cells, io, nets, sigma, bins, td, gamma, cap = WORKLOADS[args.workload]
    return {"workload": args.workload, "cells": cells, "io": io, "nets": nets, "fabric": "%dx%d" % (side, side),
            "bins": "%dx%d" % (bins, bins), "target_density": td, "gamma_base_bins": gamma, "cap": cap,
            "engine": args.engine, "dct": args.dct, "l2": "flushed between steps (512 MiB write)",
            "parallelism": "replicas x%d" % args.gpus}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="lfe5u-85-42k", choices=sorted(WORKLOADS))
    ap.add_argument("--engine", default="device", choices=["host", "device"])
    ap.add_argument("--dct", default="fp32", choices=["fp32", "tensor", "bf16x3", "fp32-gemm"],
                    help="DCT form; bf16x3 is the earlier name of tensor")
    ap.add_argument("--reference-sample", type=int, default=30,
                    help="GP iterations per reference step (each step places from the start, so a short "
                         "prefix would mostly time the model build and the two initial evaluations)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-reps", type=int, default=5, help="whole placements timed for e2e")
    ap.add_argument("--profile", action="store_true",
                    help="warmup and timed steps only (for ncu launch lists)")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-instance batched comparison")
    ap.add_argument("--batch-only", action="store_true", help="print only the batched comparison")
    ap.add_argument("--serve-requests", type=int, default=200,
                    help="requests in the serving-stream report (0 skips it; the full stream is 2000)")
    ap.add_argument("--serve-only", action="store_true", help="print only the serving-stream report")
    ap.add_argument("--no-precision", action="store_true", help="skip the 1M-cell precision report")
    ap.add_argument("--precision-only", action="store_true", help="print only the 1M-cell precision report")
    ap.add_argument("--stage-report", action="store_true",
                    help="print only the per-stage kernel report of --workload at placed positions")
    ap.add_argument("--stage-reps", type=int, default=10)
    ap.add_argument("--seed-only", action="store_true", help="print only the quadratic-seed solve report")
    ap.add_argument("--no-seed", action="store_true", help="skip the quadratic-seed solve report")
    ap.add_argument("--rudy-only", action="store_true", help="print only the RUDY demand report")
    ap.add_argument("--scatter-only", action="store_true", help="print only the density-scatter forms report")
    ap.add_argument("--probe", default="", help="a small workload for profiler captures: tc:N or scatter:WORKLOAD")
    ap.add_argument("--auction-only", action="store_true", help="print only the legalizer auction report")
    ap.add_argument("--clustering-only", action="store_true", help="print only the register-clustering report")
    ap.add_argument("--routable-only", action="store_true",
                    help="print only the routing-capacity (area rounds) report, host vs device engine")
    ap.add_argument("--ecp5-only", action="store_true",
                    help="print only the device-snapshot-to-legal-choices report on an ECP5-like fabric")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return

    import numpy as np
    import torch
    from texo_gb300 import build as engine_build
    engine_build.build()
    from texo_gb300 import abi
    from texo_gb300.placer import Placer, place

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    if args.batch_only:
        if rank == 0:
            print(json.dumps({"metric": "placements/s (64 mixed instances)", "batched": batch_report()}), flush=True)
        return
    if args.precision_only:
        if rank == 0:
            print(json.dumps({"metric": "tensor-core / FP32 / FP64 precision at 1M cells",
                              "precision": precision_report()}), flush=True)
        return
    if args.probe:
        print(json.dumps(probe(args.probe)), flush=True)
        return
    if args.scatter_only:
        if rank == 0:
            print(json.dumps({"metric": "density scatter forms", "scatter": scatter_report()}), flush=True)
        return
    if args.rudy_only:
        if rank == 0:
            print(json.dumps({"metric": "continuous RUDY demand", "rudy": rudy_report()}), flush=True)
        return
    if args.clustering_only:
        if rank == 0:
            print(json.dumps({"metric": "register clustering areas", "clustering": clustering_report()}), flush=True)
        return
    if args.routable_only:
        if rank == 0:
            print(json.dumps({"metric": "eplace with a routing-capacity map", "routable": routable_report()}),
                  flush=True)
        return
    if args.ecp5_only:
        if rank == 0:
            print(json.dumps({"metric": "ECP5 device path", "ecp5": ecp5_report()}), flush=True)
        return
    if args.auction_only:
        if rank == 0:
            print(json.dumps({"metric": "singleton BEL auction", "auction": auction_report()}), flush=True)
        return
    if args.seed_only:
        if rank == 0:
            print(json.dumps({"metric": "quadratic seed solve", "seed": seed_report(args.workload)}), flush=True)
        return
    if args.stage_report:
        if rank == 0:
            print(json.dumps(stage_report(args.workload, args.dct, args.stage_reps)), flush=True)
        return
    if args.serve_only:
        if rank == 0:
            print(json.dumps({"metric": "placements/s + p99 latency (serving stream)",
                              "serving": serve_report(args.serve_requests)}), flush=True)
        return
    engine = abi.ENGINE_HOST if args.engine == "host" else abi.ENGINE_DEVICE
    dct = {"fp32": abi.DCT_FP32, "tensor": abi.DCT_TENSOR, "bf16x3": abi.DCT_TENSOR, "fp32-gemm": abi.DCT_FP32_GEMM}[args.dct]
    prob = make_problem(args.workload, rank)
    prm = make_params(args.workload, engine, dct)
    prm.device = local
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    g = Placer(prob, prm)
    n = dict(U=g.units, F=g.num_fillers, M=int(prob.member_ptr[-1]), B=g.bins, Hb=g.bins_y,
             E=prob.num_nets, P=prob.num_pins, K=g.num_fields, dct_form=g.dct_form())

    state = {"prev": 0, "restarts": 0, "evals": 0, "devals": 0, "trials": 0}

    def one_step():
        _, _, s = g.run(1, allow_nonconverged=True)
        if s["iterations"] <= state["prev"]:
            # the placement finished: start it again (outside the timed region)
            g.reset()
            state.update(restarts=state["restarts"] + 1, evals=0, devals=0, trials=0)
            _, _, s = g.run(1, allow_nonconverged=True)
        state["prev"] = s["iterations"]
        # objective evaluations and line-search trials of this step
        s["d_evals"] = s["evaluations"] - state["evals"]
        s["d_devals"] = s["density_evaluations"] - state["devals"]
        s["d_trials"] = s["line_search_trials"] - state["trials"]
        state.update(evals=s["evaluations"], devals=s["density_evaluations"], trials=s["line_search_trials"])
        return s

    for _ in range(args.warmup):
        s = one_step()
    # timed steps
    total_ms, launches, evals, devals, trials = 0.0, 0, 0, 0, 0
    phases0 = g.device_profile() if engine == abi.ENGINE_DEVICE else None
    restarts0 = state["restarts"]
    with Clocks(local) as clk:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            s = one_step()
            total_ms += s["elapsed_ms"]
            launches += s["kernel_launches"]
            evals += s["d_evals"]
            devals += s["d_devals"]
            trials += s["d_trials"]
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
    max_ms, value = aggregate_ranks(total_ms, args.steps, dist, "cuda")
    # the persistent kernel's own phase clocks (block 0, globaltimer) over
    # the timed steps, per step; barrier_wait is the part of them block 0
    # spent waiting in grid barriers (a restart mid-run resets them)
    phases = None
    if phases0 is not None and state["restarts"] == restarts0:
        p1 = g.device_profile()
        phases = {k: round((p1[k] - phases0[k]) / args.steps, 2) for k in p1}
    if args.profile:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "iter/s", "profile": True,
                              "gpu_launches": int(launches)}), flush=True)
        return
    # per-stage device times (standalone stage kernels) and the roofline
    stages = named_stages(g.stage_times(reps=20), n)
    peak, peak_kind = peaks()
    stage_roofline = {k: {"ms": v, "algorithmic_bytes": stage_bytes(k, n),
                          "gbs": stage_bytes(k, n) / (v * 1e-3) / 1e9 if v > 0 else None}
                      for k, v in stages.items()}
    if engine == abi.ENGINE_DEVICE:
        # one persistent launch per step runs the whole iteration: its
        # algorithmic bytes are the evaluations' (full ones, and ones that
        # reuse the density side and run the wirelength side alone) and the
        # vector updates' of the step; its duration is the step's CUDA-event time
        per_step_bytes = (devals * eval_bytes(n, persistent=True)
                          + (evals - devals) * reused_eval_bytes(n)
                          + trials * stage_bytes("candidate", n)
                          + args.steps * (stage_bytes("precond", n) + stage_bytes("extrapolate", n))) / args.steps
        dom = "k_persistent (one GP iteration per launch)"
        dom_ms = max_ms / args.steps
        achieved = per_step_bytes / (dom_ms * 1e-3) / 1e9
    else:
        order = sorted(stages, key=lambda k: -stages[k])
        dom = order[0]
        per_step_bytes = stage_bytes(dom, n)
        dom_ms = stages[dom]
        achieved = per_step_bytes / (dom_ms * 1e-3) / 1e9
    roofline = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": ncu_traffic(args.workload, args.engine),
                "peak_source": peak_kind, "algorithmic_bytes_per_launch": per_step_bytes,
                "launch_ms": dom_ms, "evaluations_per_step": evals / args.steps,
                "density_evaluations_per_step": devals / args.steps,
                "phases_us_per_step": phases,
                "trials_per_step": trials / args.steps, "stages": stage_roofline}
    # end to end through the C ABI from host buffers
    e2e = None
    if not args.no_e2e:
        # whole placements from host buffers, each one texo_gp_place call
        # (problem copied in, rounded targets copied out); the value is all
        # their iterations over all their wall time
        place(prob, prm)   # warm-up: shared tables and the persistent kernel's first load
        torch.cuda.synchronize()
        runs, iters, wall = [], 0, 0.0
        for _ in range(args.e2e_reps):
            t0 = time.perf_counter()
            targets, _, s2 = place(prob, prm)
            dt = time.perf_counter() - t0
            runs.append(dt)
            iters += s2["iterations"]
            wall += dt
        e2e = {"value": iters / wall, "unit": "iter/s", "h2d_bytes_per_step": problem_bytes(prob),
               "d2h_bytes_per_step": int(targets.nbytes), "placements": args.e2e_reps,
               "placement_s_mean": wall / args.e2e_reps, "placement_s_min": min(runs),
               "placement_s_max": max(runs), "iterations": s2["iterations"], "final_overflow": s2["overflow"],
               "final_hpwl": s2["hpwl"], "converged": s2["converged"]}
    line = {"metric": METRIC, "value": value, "unit": "iter/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": max_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": config_dict(args), "clocks": clk.summary(), "gpu_launches": int(launches),
            "roofline": roofline, "e2e": e2e, "restarts": state["restarts"]}
    if rank == 0 and not args.no_batch:
        line["batched"] = batch_report()
    if rank == 0 and args.serve_requests > 0 and not args.no_batch:
        line["serving"] = serve_report(args.serve_requests)
    if rank == 0 and not args.no_precision and not args.no_batch:
        line["precision"] = precision_report()
    if rank == 0 and not args.no_seed and not args.no_batch:
        line["quadratic_seed"] = seed_report(args.workload)
        line["rudy"] = rudy_report()
        line["auction"] = auction_report()
        line["clustering"] = clustering_report()
    if rank == 0 and not args.no_cpu_baseline:
        try:
            line["cpu_baseline"] = cpu_baseline(args.workload)
        except Exception as e:  # the oracle build can fail on an odd host
            line["cpu_baseline"] = {"value": None, "error": str(e)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
