"""Throughput benchmark of the particle-update path on one GB300.

Workload (the configuration the headline metric is quoted on): the vortex
system, N = 65,536 particles in a periodic box L = 8, natural frequencies
omega_i ~ N(0, 0.5^2), alpha = 0, v0 = 0.02, sigma = 2, rho = 0.25,
D = 0.01, strong-order-1.5 stochastic Runge-Kutta, dt = 0.005, seed 1.
Synthetic inputs: x, y ~ U[0, L), phi ~ U[-pi, pi) from numpy PCG64(1).

The configured run is 10^4 SRK steps from the seeded initial state.  Each
precision form (FP32X, FP32C, FP64, each with the autotuner's choice) runs it
whole, split into --steps bench steps of 10^4 / K simulation steps (CUDA-graph
replays of 100).  L2 is flushed (a 512 MB write) before each bench step,
outside the timers.  Per bench step: CUDA events around the replays (device
time, `value`) and wall clock around the C-ABI call cycle with pinned host
buffers (upload, replays, download: `e2e`); between bench steps the global
and local order parameters (the drift series against FP64).  `value` is the
fastest form whose drift from FP64 in this run stays within 1e-4 (`form`
names it); every form's figures are under `forms`.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(name="vortex_srk_n65536_L8", n=65536, L=8.0, v0=0.02, sigma=2.0, rho=0.25,
                alpha=0.0, D_phi=0.01, dt=0.005, seed=1, omega_sd=0.5, skin=0.05, steps=10000)
SIM_STEPS_PER_BENCH_STEP = 100
# Algorithmic (compulsory) HBM bytes per particle for one SRK step, by phase,
# for state resident in HBM: doubles x, y, phi (24 B), omega (8 B), the cell
# key and index (4 + 4 B written, read back by the sort), the phase rate (8 B)
# and n_i (4 B).
ALG_BYTES = {
    "stage": 24 + 8,          # read x, y, phi; write key, index
    "sort": 2 * 8,            # one digit pass (<= 2048 cells): read + write (key, index)
    "gather": 8 + 40,         # read (key, index); write cell-order x, y, phi, float x/y offsets
    "pass1": 32 + 12,         # read cell-order x, y, phi, offsets; write phase rate, n_i
    "pass2": 32 + 12 + 8 + 24 + 24,  # + own rate/n_i, omega, state in, state out
}
ALG_BYTES_STEP = 168 + 8      # survey accounting for the whole SRK step (+ omega)
# The kernels of each phase, by form (the cell-list forms; a phase that runs
# the cell-tile and the warp-per-cell kernels, for dense and sparse cells,
# counts both).
PHASE_KERNELS = {
    "fp32c": {"stage": ["k_stage"], "sort": ["k_scan_digits", "k_radix_scatter"],
              "gather": ["k_gather<1>", "k_list_units (cell units on)"],
              "pass1": ["k_tile_fp32c<0>", "k_units_fp32c<0> (cell units on)", "k_warp_fp32c<0>"],
              "pass2": ["k_tile_fp32c<1>", "k_units_fp32c<1> (cell units on)", "k_warp_fp32c<1>"]},
    "fp32x": {"stage": ["k_stage"], "sort": ["k_scan_digits", "k_radix_scatter"],
              "gather": ["k_gather<2>", "k_list_units (cell units on)"],
              "pass1": ["k_tile_fp32x<0>", "k_units_fp32x<0> (cell units on)", "k_warp_fp32x<0>",
                        "k_epilogue_fp32x<0>"],
              "pass2": ["k_tile_fp32x<1>", "k_units_fp32x<1> (cell units on)", "k_warp_fp32x<1>",
                        "k_epilogue_fp32x<1>"]},
    "fp64": {"stage": ["k_stage"], "sort": ["k_scan_digits", "k_radix_scatter"],
             "gather": ["k_gather<0>", "k_vgather<0>"], "pass1": ["k_vtile<0,0>", "k_tile_fp64<0>"],
             "pass2": ["k_vtile<0,1>", "k_tile_fp64<1>"]},
}
# DRAM bytes (read + write) per launch of a phase's kernels, from one ncu
# capture (`--ncu-case <form> --cell-list --ncu-state <state>`, cold caches),
# summed over the phase's kernels; keyed by (form, phase).  FP32C pass 2 reads
# the pass-1 neighbour masks (~3.5 MB here) on top of its algorithmic bytes.
NCU_TRAFFIC = {
    ("fp32c", "pass1"): {"bytes": 2.53e6, "state": "clustered (step 4,000, tests/golden/states), "
                                                  "cell units: k_units_fp32c<0> + k_tile_fp32c<0,1>"},
    ("fp32c", "pass2"): {"bytes": 1.017e7, "state": "clustered, cell units: k_units_fp32c<1> + "
                                                   "k_tile_fp32c<1,1>"},
    ("fp32x", "pass1"): {"bytes": 5.83e6, "state": "clustered, cell units: k_units_fp32x<0> + "
                                                  "k_tile_fp32x<0,1> + k_epilogue_fp32x<0>"},
    ("fp32x", "pass2"): {"bytes": 1.257e7, "state": "clustered, cell units: k_units_fp32x<1> + "
                                                   "k_tile_fp32x<1,1> + k_epilogue_fp32x<1>"},
}


def init_inputs(w, seed_offset=0):
    rng = np.random.default_rng(w["seed"] + seed_offset)
    n, L = w["n"], w["L"]
    st = np.empty(3 * n)
    st[0::3] = rng.uniform(0.0, L, n)
    st[1::3] = rng.uniform(0.0, L, n)
    st[2::3] = rng.uniform(-np.pi, np.pi, n)
    omega = rng.normal(0.0, w["omega_sd"], n)
    return st, omega


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index=0):
        self.samples, self.proc, self.index = [], None, index

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4)
                          if s[3 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def cpu_baseline(w, nsteps=3):
    """The oracle port (the reference's arithmetic restated in C, one core),
    on a bounded sample: the full N for a few SRK steps."""
    from oracle import pyoracle as po
    st, omega = init_inputs(w)
    n = w["n"]
    o = po.OracleSystem(n, w["L"], w["v0"], w["sigma"], w["rho"], w["alpha"], w["D_phi"])
    noise = np.random.default_rng(99).standard_normal(2 * n * nsteps)
    o.run(po.SRK, st, 0.0, w["dt"], 1, noise[:2 * n], omega)  # warm
    t0 = time.perf_counter()
    o.run(po.SRK, st, 0.0, w["dt"], nsteps, noise, omega)
    dt = time.perf_counter() - t0
    return {"value": n * nsteps / dt, "unit": "particle-steps/s", "cores": 1, "kind": "port",
            "sample": f"N={n}, {nsteps} SRK steps of the same workload, 1 thread "
                      f"(the reference's path is single-threaded per system)"}


def ensemble_systems(count=512, seed=2, n_range=(256, 32768), density=1000.0):
    """The batched-ensemble configuration: count Chimera systems, N log-uniform
    in n_range, L = sqrt(N / density), alpha ~ U[1.2, 1.6], sigma ~ U[0.5, 2],
    D ~ U[0, 0.02], rho ~ U[0.05, 0.15], v0 = 0.01, from numpy PCG64(seed)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n = int(round(np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1])))))
        L = float(np.sqrt(n / density))
        prm = dict(v0=0.01, sigma=float(rng.uniform(0.5, 2.0)), rho=float(rng.uniform(0.05, 0.15)),
                   alpha=float(rng.uniform(1.2, 1.6)), D_phi=float(rng.uniform(0.0, 0.02)))
        st = np.empty(3 * n)
        st[0::3] = rng.uniform(0.0, L, n)
        st[1::3] = rng.uniform(0.0, L, n)
        st[2::3] = rng.uniform(-np.pi, np.pi, n)
        out.append((k, n, L, prm, st))
    return out


def _cpu_replica_worker(job):
    """One replica of the headline workload on one host core (initial state
    seeded by replica): a warm-up step, a barrier shared with the other
    replicas, then `nsteps` timed SRK steps of the oracle port.  Returns the
    particle-steps done and the wall-clock start and end of the timed steps."""
    k, nsteps, barrier = job
    from oracle import pyoracle as po
    w = WORKLOAD
    st, omega = init_inputs(w, seed_offset=k)
    n = w["n"]
    o = po.OracleSystem(n, w["L"], w["v0"], w["sigma"], w["rho"], w["alpha"], w["D_phi"])
    noise = np.random.default_rng(99 + k).standard_normal(2 * n * nsteps)
    o.run(po.SRK, st, 0.0, w["dt"], 1, noise[:2 * n], omega)  # warm
    barrier.wait()
    t0 = time.time()
    o.run(po.SRK, st, 0.0, w["dt"], nsteps, noise, omega)
    return n * nsteps, t0, time.time()


def cpu_replicas_baseline(nsteps=1):
    """The reference path on every host core: one independent replica of the
    headline workload per core (the reference runs one system per process; its
    only multi-core form is independent systems side by side), started
    together.  Aggregate particle-steps/s over the span of the timed steps."""
    import multiprocessing as mpc
    cores = os.cpu_count() or 1
    ctx = mpc.get_context("spawn")
    with ctx.Manager() as mgr:
        barrier = mgr.Barrier(cores)
        with ctx.Pool(cores) as pool:
            out = pool.map(_cpu_replica_worker, [(k, nsteps, barrier) for k in range(cores)])
    work = sum(wk for wk, _, _ in out)
    span = max(t1 for _, _, t1 in out) - min(t0 for _, t0, _ in out)
    return {"value": work / span, "unit": "particle-steps/s", "cores": cores, "kind": "port",
            "sample": f"{cores} replicas of N={WORKLOAD['n']} (one per host core, started "
                      f"together), {nsteps} SRK step(s) each"}


_ENSEMBLE = None


def _cpu_system_worker(job):
    """One ensemble system on one host core: `steps` Euler steps of the oracle
    port with seeded normals.  Returns particle-steps done and seconds."""
    k, steps = job
    from oracle import pyoracle as po
    global _ENSEMBLE
    if _ENSEMBLE is None:  # once per worker process
        _ENSEMBLE = ensemble_systems()
    _, n, L, prm, st = _ENSEMBLE[k]
    o = po.OracleSystem(n, L, **prm)
    noise = np.random.default_rng(1000 + k).standard_normal(n * steps)
    t0 = time.perf_counter()
    o.run(po.EULER, st, 0.0, 0.01, steps, noise)
    return n * steps, time.perf_counter() - t0


def cpu_ensemble_baseline(count=64, steps=100):
    """The reference's parameter-scan form on the host: one process per system
    over every host core (a spawn pool, started before any GPU work), on a
    seeded sample of `count` of the 512 systems for `steps` Euler steps."""
    import multiprocessing as mpc
    cores = os.cpu_count() or 1
    pick = sorted(np.random.default_rng(5).choice(512, size=count, replace=False).tolist())
    ctx = mpc.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        out = pool.map(_cpu_system_worker, [(k, steps) for k in pick])
    wall = time.perf_counter() - t0
    work = sum(w for w, _ in out)
    return {"value": work / wall, "unit": "particle-steps/s", "cores": cores, "kind": "port",
            "sample": f"{count} of the 512 systems (seeded), {steps} Euler steps each, one "
                      f"process per system over {cores} host cores (wall time incl. pool start)"}


def run_ensemble(precision, graphs, rank=0, sparse_below=None, subset=None):
    """One batch of the ensemble's systems (all, or the indices in `subset`),
    `graphs` replays of a 100-step graph; then a per-phase profile of 5 plain
    steps.  sparse_below: the tuning that picks the neighbour kernel per system
    (None: the library's default)."""
    import torch
    from spc2_langevin_integration_gb300 import abi
    systems = ensemble_systems()
    if subset is not None:
        systems = [systems[i] for i in subset]
    ntot = sum(n for _, n, _, _, _ in systems)
    ctot = sum(abi.cells_of(L, prm["rho"]) for _, _, L, prm, _ in systems)
    b = abi.Batch(abi.STEPPER_EULER, precision, len(systems), ntot, ctot)
    if sparse_below is not None:
        b.set_tuning(abi.TUNE_SPARSE_BELOW, sparse_below)
    for k, n, L, prm, st in systems:
        p = abi.make_params(L=L, stepper=abi.STEPPER_EULER, precision=precision, seed=2,
                            system_id=1000 * rank + k, **prm)
        b.admit(n, p, st)
    stream = torch.cuda.ExternalStream(b.stream)
    b.step(0.01, 100, graph=True)  # capture + warm
    b.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(graphs):
        b.step(0.01, 100, graph=True)
    e1.record(stream)
    b.synchronize()
    ms = e0.elapsed_time(e1)
    prof = b.profile_steps(0.01, 5)
    b.close()
    return ntot, ctot, ms, prof


def served_drift(reqs, precision):
    """Order parameters of served results against the same requests run alone
    in FP64 (a batch of one, same Philox counters): |delta R| and
    |delta R_local| of each request's final state."""
    from spc2_langevin_integration_gb300 import abi
    rows = []
    for r in reqs:
        st, om = r.inputs()
        p64 = r.params(abi.STEPPER_EULER, abi.PRECISION_FP64)
        with abi.Batch(abi.STEPPER_EULER, abi.PRECISION_FP64, 1, r.n, r.cells) as b:
            slot = b.admit(r.n, p64, st, om, steps=r.steps)
            for _ in range((r.steps + 99) // 100):  # frozen once its budget is spent
                b.step(0.01, 100, graph=True)
            ref = b.download(slot)
        o = []
        for state in (ref, r.result):
            with abi.System(r.n, p64) as s:
                s.upload_state(state)
                if om is not None:
                    s.upload_omega(om)
                o.append(s.order_params())
        rows.append({"rid": r.rid, "model": "vortex" if r.model == abi.MODEL_VORTEX else "chimera",
                     "N": r.n, "steps": r.steps, "dR": abs(o[1]["R"] - o[0]["R"]),
                     "dR_local": abs(o[1]["R_local"] - o[0]["R_local"])})
    return {"sample": rows, "max_dR": max(x["dR"] for x in rows),
            "max_dR_local": max(x["dR_local"] for x in rows),
            "within_1e-4": sum(x["dR"] <= 1e-4 and x["dR_local"] <= 1e-4 for x in rows)}


def run_serving(precision, duration, rate, seed=3, drift_sample=12):
    """The served request stream (serve.make_trace) through serve.Server on one
    batch; then, for a sample of the completed requests (every k-th by
    request id among those with N <= 16,384, so the FP64 reruns stay short),
    the order parameters of the served results against the same requests run
    alone in FP64 (skipped for the FP64 form itself, whose served results equal
    the alone runs bit for bit)."""
    from spc2_langevin_integration_gb300 import abi, serve
    trace = serve.make_trace(rate=rate, duration=duration, seed=seed)
    small = [r.rid for r in trace if r.n <= 16384]
    keep = set(small[::max(1, len(small) // drift_sample)][:drift_sample]) \
        if precision != abi.PRECISION_FP64 else set()
    max_n, max_c, max_s = 4_200_000, 1_500_000, 1024
    with abi.Batch(abi.STEPPER_EULER, precision, max_s, max_n, max_c) as b:
        srv = serve.Server(b, abi.STEPPER_EULER, precision, dt=0.01, chunk=50,
                           limits=(max_n, max_c), keep_results=keep)
        st = srv.run(trace)
    out = st.as_dict()
    out.update({"requests": len(trace), "refused": len(srv.refused), "rate_per_s": rate,
                "duration_s": duration, "prefetched": srv.prefetched,
                "batch_capacity": {"particles": max_n, "cells": max_c, "systems": max_s}})
    done = [r for r in trace if r.result is not None]
    if done:
        out["drift_vs_fp64_alone"] = served_drift(done, precision)
    return out


def run_drift(steps=10000, every=100, out_path=None, seed=None):
    """Drift of the order parameters of the FP32-compensated form against FP64.

    (1) The vortex SRK workload (N=65,536, L=8): FP32C and the FP64 GPU path from
    the same state with the same Philox counters (FP32C draws the same Philox
    words through float Box-Muller), global R and local R every `every` steps.
    (2) The Chimera Euler workload (N=1,024, L=1, rho=0.1): FP32C and FP64 on the
    GPU and the CPU oracle, all fed the identical normals (exported from the FP64
    run and injected into the others).
    Both also run FP64 from the initial state with every phase moved by one ulp:
    its drift is the dynamics' own sensitivity, the floor for any perturbation.
    Reports max and mean |delta| over the recorded points.  `seed` replaces the
    vortex workload's seed (its initial state, frequencies and Philox key)."""
    from oracle import pyoracle as po
    from spc2_langevin_integration_gb300 import abi

    def stats(ref, got):
        # pointwise |delta| over the recorded points, and the time means of both
        # series over the second half of the run (the statistical comparison)
        ref, got = np.asarray(ref), np.asarray(got)
        d = np.abs(got - ref)
        h = len(ref) // 2
        return {"max_abs": float(d.max()), "mean_abs": float(d.mean()),
                "time_mean_ref": float(ref[h:].mean()), "time_mean": float(got[h:].mean()),
                "time_sd_ref": float(ref[h:].std())}

    res, dump = {}, {}
    # (1) vortex SRK N=65536
    w = WORKLOAD if seed is None else dict(WORKLOAD, seed=seed)
    st, omega = init_inputs(w)
    st_ulp = st.copy()
    st_ulp[2::3] = np.nextafter(st[2::3], np.inf)
    series = {}
    for name, prec, s0 in (("fp64", abi.PRECISION_FP64, st), ("fp32c", abi.PRECISION_FP32C, st),
                           ("fp64_ulp", abi.PRECISION_FP64, st_ulp)):
        p = abi.make_params(L=w["L"], v0=w["v0"], sigma=w["sigma"], rho=w["rho"], alpha=w["alpha"],
                            D_phi=w["D_phi"], model=abi.MODEL_VORTEX, stepper=abi.STEPPER_SRK,
                            precision=prec, seed=w["seed"])
        rows = []
        with abi.System(w["n"], p) as s:
            s.upload_state(s0)
            s.upload_omega(omega)
            for k in range(every, steps + 1, every):
                s.step(w["dt"], every, graph=True)
                o = s.order_params()
                rows.append((k, o["R"], o["R_local"]))
        series[name] = np.array(rows)
    a64 = series["fp64"]
    res["vortex_srk_n65536"] = {
        "steps": steps, "every": every, "seed": w["seed"],
        "reference": "FP64 GPU path (same Philox counters)",
        "fp32c": {"R": stats(a64[:, 1], series["fp32c"][:, 1]),
                  "R_local": stats(a64[:, 2], series["fp32c"][:, 2])},
        "fp64_one_ulp_phases": {"R": stats(a64[:, 1], series["fp64_ulp"][:, 1]),
                                "R_local": stats(a64[:, 2], series["fp64_ulp"][:, 2])},
        "final_R": {k: float(v[-1, 1]) for k, v in series.items()},
        "final_R_local": {k: float(v[-1, 2]) for k, v in series.items()}}
    dump["vortex_srk_n65536"] = {k: v.tolist() for k, v in series.items()}
    # (2) Chimera Euler N=1024 against the CPU oracle with identical noise
    n, L, dt = 1024, 1.0, 0.01
    prm = dict(v0=0.01, sigma=1.0, rho=0.1, alpha=1.45, D_phi=0.005)
    rng = np.random.default_rng(0)
    st0 = np.empty(3 * n)
    st0[0::3] = rng.uniform(0.0, L, n)
    st0[1::3] = rng.uniform(0.0, L, n)
    st0[2::3] = rng.uniform(-np.pi, np.pi, n)
    st0u = st0.copy()
    st0u[2::3] = np.nextafter(st0[2::3], np.inf)
    orc = po.OracleSystem(n, L, **prm)
    ref = st0.copy()
    t_ref = 0.0
    rows = []
    mk = lambda prec: abi.System(n, abi.make_params(L=L, stepper=abi.STEPPER_EULER, seed=0,  # noqa: E731
                                                    precision=prec, **prm))
    with mk(abi.PRECISION_FP64) as s64, mk(abi.PRECISION_FP32C) as s32, mk(abi.PRECISION_FP64) as s64u:
        s64.upload_state(st0)
        s32.upload_state(st0)
        s64u.upload_state(st0u)
        for k in range(every, steps + 1, every):
            noise = s64.export_noise(k - every, every)
            s32.inject_noise(noise)
            s64u.inject_noise(noise)
            for s in (s64, s32, s64u):
                s.step(dt, every)
            t_ref = orc.run(po.EULER, ref, t_ref, dt, every, noise)
            oo = orc.order_params(ref)
            og = [s.order_params() for s in (s64, s32, s64u)]
            rows.append([k, oo["R"], oo["R_local"]] + [v for o in og for v in (o["R"], o["R_local"])])
    r = np.array(rows)
    res["chimera_euler_n1024"] = {
        "steps": steps, "every": every, "reference": "CPU oracle (identical injected normals)",
        "fp64_gpu": {"R": stats(r[:, 1], r[:, 3]), "R_local": stats(r[:, 2], r[:, 4])},
        "fp32c_gpu": {"R": stats(r[:, 1], r[:, 5]), "R_local": stats(r[:, 2], r[:, 6])},
        "fp64_gpu_one_ulp_phases": {"R": stats(r[:, 1], r[:, 7]), "R_local": stats(r[:, 2], r[:, 8])},
        "final_R": {"oracle": r[-1, 1], "fp64_gpu": r[-1, 3], "fp32c_gpu": r[-1, 5],
                    "fp64_gpu_one_ulp_phases": r[-1, 7]}}
    dump["chimera_euler_n1024"] = r.tolist()
    if out_path:
        with open(out_path, "w") as f:
            json.dump(dump, f)
    return res


def run_drift_ensemble(forms, steps=5000, every=100, subset=None, series_path=None):
    """Per-system drift of the order parameters over the batched ensemble (512
    Chimera systems, Euler, dt = 0.01): one batch per precision form and one
    FP64 batch, the same systems, seeds and Philox counters, stepped `every`
    steps at a time as graph replays; R and R_local of every system after each
    chunk.  forms: (name, precision) pairs compared against the FP64 batch.
    A control arm, FP64 from the initial state with every phase moved by one
    ulp, measures the dynamics' own sensitivity: a system that this arm
    leaves beyond 1e-4 cannot be followed pointwise by any arithmetic that is
    not FP64 bit for bit.  Returns, per arm, the maximum |delta| over systems
    and recorded points, its distribution over the systems, how many systems
    stay within 1e-4, and (forms) how many of those beyond 1e-4 the control
    arm also leaves beyond it."""
    from spc2_langevin_integration_gb300 import abi
    systems = ensemble_systems()
    if subset is not None:
        systems = [systems[i] for i in subset]
    ntot = sum(n for _, n, _, _, _ in systems)
    ctot = sum(abi.cells_of(L, prm["rho"]) for _, _, L, prm, _ in systems)
    cap = len(systems)

    def make(prec, ulp=False):
        b = abi.Batch(abi.STEPPER_EULER, prec, cap, ntot, ctot)
        slots = []
        for k, n, L, prm, st in systems:
            p = abi.make_params(L=L, stepper=abi.STEPPER_EULER, precision=prec, seed=2,
                                system_id=k, **prm)
            if ulp:
                st = st.copy()
                st[2::3] = np.nextafter(st[2::3], np.inf)
            slots.append(b.admit(n, p, st))
        return b, np.array(slots)

    arms = [("fp64", abi.PRECISION_FP64)] + list(forms) + [("fp64_one_ulp_phases", abi.PRECISION_FP64)]
    batches = {name: make(prec, ulp=name.endswith("ulp_phases")) for name, prec in arms}
    rec = {name: {"R": [], "R_local": []} for name, _ in arms}
    for k in range(every, steps + 1, every):
        for name, (b, slots) in batches.items():
            b.step(0.01, every, graph=True)
            o = b.order_params_all(cap)
            rec[name]["R"].append(o["R"][slots])
            rec[name]["R_local"].append(o["R_local"][slots])
    for b, _ in batches.values():
        b.close()
    ref = {q: np.array(rec["fp64"][q]) for q in ("R", "R_local")}
    sizes = np.array([n for _, n, _, _, _ in systems])
    out = {"systems": len(systems), "particles": int(ntot), "steps": steps, "every": every,
           "reference": "FP64 batch (same systems, seeds and Philox counters)"}
    ctrl = {q: np.abs(np.array(rec["fp64_one_ulp_phases"][q]) - ref[q]).max(axis=0)
            for q in ("R", "R_local")}
    for name, _ in list(forms) + [("fp64_one_ulp_phases", None)]:
        res = {}
        for q in ("R", "R_local"):
            d = np.abs(np.array(rec[name][q]) - ref[q])   # [points, systems]
            per_sys = d.max(axis=0)
            beyond = per_sys > 1e-4
            worst = int(per_sys.argmax())
            first = [int(np.argmax(d[:, s] > 1e-4)) if (d[:, s] > 1e-4).any() else -1
                     for s in range(d.shape[1])]
            res[q] = {"max_abs": float(per_sys.max()), "mean_abs": float(d.mean()),
                      "per_system_max_quantiles": {str(p): float(np.quantile(per_sys, p))
                                                   for p in (0.5, 0.9, 0.99)},
                      "systems_within_1e-4": int((per_sys <= 1e-4).sum()),
                      "beyond_1e-4_also_beyond_in_control": int((beyond & (ctrl[q] > 1e-4)).sum()),
                      "worst_system": {"index": int(systems[worst][0]), "N": int(sizes[worst]),
                                       "max_abs": float(per_sys[worst])},
                      "median_first_step_over_1e-4": (
                          float(np.median([every * (f + 1) for f in first if f >= 0]))
                          if any(f >= 0 for f in first) else None)}
        out[name] = res
    if series_path:
        with open(series_path, "w") as f:
            json.dump({name: {q: np.array(v).tolist() for q, v in r.items()}
                       for name, r in rec.items()}, f)
    return out


# Ensemble systems for the oracle drift check: twelve small systems on which
# the FP64 kernels, before the float prefilter's band decision was made
# gap-free, left the CPU oracle by more than 1e-4 within 5,000 steps, and four
# on which they did not.
DRIFT_ORACLE_SYSTEMS = [505, 55, 173, 53, 409, 220, 169, 375, 419, 57, 472, 50, 33, 192, 268, 129]


def _oracle_drift_worker(job):
    """The CPU oracle (the reference's arithmetic, FP64) on one ensemble
    system with the normals the GPU drew: R and R_local every `every` steps."""
    n, L, prm, st, noise_path, steps, every = job
    from oracle import pyoracle as po
    noise = np.load(noise_path, mmap_mode="r")
    o = po.OracleSystem(n, L, **prm)
    s, t, rows = st.copy(), 0.0, []
    for k in range(every, steps + 1, every):
        t = o.run(po.EULER, s, t, 0.01, every, np.ascontiguousarray(noise[(k - every) * n:k * n]))
        op = o.order_params(s)
        rows.append((op["R"], op["R_local"]))
    return rows


def run_drift_oracle(indices, steps=5000, every=100):
    """Order-parameter drift of single ensemble systems against the FP64 CPU
    oracle fed the identical normals: the FP64 GPU path, FP32X and FP32C (the
    same Philox counters as in the batch, where each system's trajectory is
    bitwise its single-handle one).  The oracle runs in spawned host processes,
    one per system."""
    import multiprocessing as mp
    import tempfile
    from spc2_langevin_integration_gb300 import abi
    systems = ensemble_systems()
    forms = [("fp64", abi.PRECISION_FP64), ("fp32x", abi.PRECISION_FP32X),
             ("fp32c", abi.PRECISION_FP32C)]
    gpu, jobs = {}, []
    td = tempfile.mkdtemp()
    for k in indices:
        _, n, L, prm, st = systems[k]
        gpu[k] = {}
        for name, prec in forms:
            p = abi.make_params(L=L, stepper=abi.STEPPER_EULER, precision=prec, seed=2,
                                system_id=k, **prm)
            rows = []
            with abi.System(n, p) as s:
                s.upload_state(st)
                for _ in range(every, steps + 1, every):
                    s.step(0.01, every, graph=True)
                    o = s.order_params()
                    rows.append((o["R"], o["R_local"]))
                if name == "fp64":
                    path = os.path.join(td, f"noise_{k}.npy")
                    np.save(path, s.export_noise(0, steps))
            gpu[k][name] = np.array(rows)
        jobs.append((n, L, prm, st, path, steps, every))
    with mp.get_context("spawn").Pool(min(len(jobs), os.cpu_count() or 1)) as pool:
        orc = pool.map(_oracle_drift_worker, jobs)
    for k in indices:
        os.remove(os.path.join(td, f"noise_{k}.npy"))
    os.rmdir(td)
    out = {"steps": steps, "every": every, "systems": []}
    for k, rows in zip(indices, orc):
        ref = np.array(rows)
        rec = {"index": k, "N": systems[k][1],
               **{q: systems[k][3][q] for q in ("alpha", "sigma", "D_phi", "rho")}}
        for name, _ in forms:
            d = np.abs(gpu[k][name] - ref)
            first = np.flatnonzero(d.max(axis=1) > 1e-4)
            rec[name] = {"max_dR": float(d[:, 0].max()), "max_dR_local": float(d[:, 1].max()),
                         "first_step_over_1e-4": int(every * (first[0] + 1)) if first.size else None}
        out["systems"].append(rec)
    for name, _ in forms:
        out[name + "_within_1e-4"] = sum(r[name]["max_dR"] <= 1e-4 and r[name]["max_dR_local"] <= 1e-4
                                        for r in out["systems"])
    return out


LARGE = dict(name="chimera_rk4_n4194304_L64", n=1 << 22, L=64.0, v0=0.01, sigma=1.0, rho=0.25,
             alpha=1.45, D_phi=0.0, dt=0.01, seed=0, skin=0.05)


def run_large(precision, steps):
    """The large single system: Chimera, N = 2^22 in L = 64, RK4, dt = 0.01,
    positions and phases uniform from seed 0.  The autotuner picks the
    neighbour method on the initial state (2 trial steps per candidate); then
    `steps` steps run as one graph replay, timed with CUDA events."""
    import torch
    from spc2_langevin_integration_gb300 import abi
    w = LARGE
    n, L = w["n"], w["L"]
    rng = np.random.default_rng(w["seed"])
    st = np.empty(3 * n)
    st[0::3] = rng.uniform(0.0, L, n)
    st[1::3] = rng.uniform(0.0, L, n)
    st[2::3] = rng.uniform(-np.pi, np.pi, n)
    p = abi.make_params(L=L, v0=w["v0"], sigma=w["sigma"], rho=w["rho"], alpha=w["alpha"],
                        D_phi=w["D_phi"], stepper=abi.STEPPER_RK4, precision=precision,
                        seed=w["seed"], skin=w["skin"])
    t0 = time.perf_counter()
    cands, k = abi.autotune_ex(n, p, st, dt=w["dt"], trial_steps=2)
    tune_s = time.perf_counter() - t0
    best, tun = abi.params_with(p, cands[k]), cands[k]
    with abi.System(n, best) as s:
        if best.neighbour == abi.NEIGHBOUR_CELL:
            apply_tuning(abi, s, tun)
        s.upload_state(st)
        stream = torch.cuda.ExternalStream(s.stream)
        s.step(w["dt"], steps, graph=True)  # capture + warm
        s.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.step(w["dt"], steps, graph=True)
        e1.record(stream)
        s.synchronize()
        t_ms = e0.elapsed_time(e1)
        final = s.download_state()
        o = s.order_params()
        prof = s.profile_steps(w["dt"], 1)
        launches = s.graph_nodes()
    return {"value": n * steps / (t_ms / 1e3), "unit": "particle-steps/s", "steps": steps,
            "ms_per_step": t_ms / steps, "profile_ms_one_step": prof,
            "gpu_launches_per_replay": launches, "order_params": o, "_state": final,
            "autotune": {"choice": tun, "candidates": cands, "tuning_s": tune_s}}


VA = dict(name="vortex_arrays_srk_n51200_L8", n=51200, L=8.0, velocity=0.1, mu_plus=100.0,
          mu_minus=100.0, xi_a=0.04, xi_r=0.02, D_phi=0.01, kappa=20.0, rho=0.2, dt=0.01, seed=3)


def va_inputs(w):
    rng = np.random.default_rng(w["seed"])
    n, L = w["n"], w["L"]
    st = np.empty(3 * n)
    st[0::3] = rng.uniform(0.0, L, n)
    st[1::3] = rng.uniform(0.0, L, n)
    st[2::3] = rng.uniform(-np.pi, np.pi, n)
    return st


def run_choices():
    """The float forms' kernel choices side by side on one GPU: whole cell
    tiles (one CTA per cell), cell units (SPC_TUNE_CELL_UNITS) and sub-cells
    (SPC_TUNE_SUBCELLS, units of half cells over the half stencils), each
    with a per-phase CUDA-event profile of 20 eager steps (stage, sort,
    gather with the unit listing, pass 1, pass 2, whole step) and the
    graph-replayed step (50 steps, CUDA events on the handle's stream).
    States: the headline workload's seeded initial state, its clustered
    state after 4,000 FP64 steps (tests/golden/states) and a uniform system
    four times denser (N = 262,144 in the same box: 256 particles per cell)."""
    import torch
    from spc2_langevin_integration_gb300 import abi
    w = WORKLOAD
    st0, om0 = init_inputs(w)
    z = np.load(os.path.join(ROOT, "tests", "golden", "states", "vortex_clustered_n65536.npz"))
    wd = dict(w, n=4 * w["n"])
    std, omd = init_inputs(wd)
    cases = {"initial": (w, st0, om0), "clustered": (w, z["state"].copy(), z["omega"].copy()),
             "dense_n262144": (wd, std, omd)}
    rows = {}
    for form, prec in (("fp32c", abi.PRECISION_FP32C), ("fp32x", abi.PRECISION_FP32X)):
        for cname, (ww, st, om) in cases.items():
            p = workload_params(abi, ww, prec)
            p.neighbour = abi.NEIGHBOUR_CELL
            res = {}
            for label, units, sub in (("tiles", 0, 0), ("units", 1, 0), ("subcells", 0, 1)):
                with abi.System(ww["n"], p) as s:
                    s.set_tuning(abi.TUNE_SPARSE_BELOW, 0.0)
                    s.set_tuning(abi.TUNE_CELL_UNITS, units)
                    s.set_tuning(abi.TUNE_SUBCELLS, sub)
                    s.upload_state(st)
                    s.upload_omega(om)
                    s.step(ww["dt"], 5)
                    prof = {k: round(v * 1e3, 1) for k, v in s.profile_steps(ww["dt"], 20).items()}
                    s.prepare_graph(ww["dt"], 50)
                    s.step(ww["dt"], 50, graph=True)
                    stream = torch.cuda.ExternalStream(s.stream)
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    s.synchronize()
                    e0.record(stream)
                    s.step(ww["dt"], 50, graph=True)
                    e1.record(stream)
                    e1.synchronize()
                    res[label] = {"phases_us": prof, "graph_step_us": round(e0.elapsed_time(e1) / 50 * 1e3, 1)}
            rows[f"{form}_{cname}"] = res
    return rows


def run_va(steps, cpu=True):
    """The vortex-arrays model (VortexArraysSystemPtr) with the reference's
    vortex-array parameters (SimulationEnginePtr.cpp:131-139, box side 1 ->
    velocity 0.1, mu+- 100, xi_a 0.04, xi_r 0.02, D 0.01, kappa 20, rho 0.2) at
    density 800 (N = 51,200 in L = 8), SRK-Ptr stepper, plain FP64: graph
    replays of `steps` steps timed with CUDA events; the oracle port on one host
    core for 2 steps beside it."""
    import torch
    from spc2_langevin_integration_gb300 import abi
    w = VA
    st = va_inputs(w)
    prm = {k: w[k] for k in ("velocity", "mu_plus", "mu_minus", "xi_a", "xi_r", "D_phi", "kappa",
                             "rho")}
    out = {}
    with abi.System(w["n"], abi.make_va_params(L=w["L"], stepper=abi.STEPPER_SRK, seed=w["seed"],
                                               **prm)) as s:
        s.upload_state(st)
        stream = torch.cuda.ExternalStream(s.stream)
        s.step(w["dt"], steps, graph=True)  # capture + warm
        s.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.step(w["dt"], steps, graph=True)
        e1.record(stream)
        s.synchronize()
        ms = e0.elapsed_time(e1)
        out = {"value": w["n"] * steps / (ms / 1e3), "unit": "particle-steps/s", "steps": steps,
               "ms_per_step": ms / steps, "profile_ms": s.profile_steps(w["dt"], 3),
               "gpu_launches_per_replay": s.graph_nodes()}
    if cpu:
        from oracle import pyoracle as po
        o = po.OracleVortexArrays(w["n"], w["L"], **prm)
        st2 = st.copy()
        noise = np.random.default_rng(7).standard_normal(2 * w["n"] * 2)
        t0 = time.perf_counter()
        o.run(po.SRK, st2, 0.0, w["dt"], 2, noise)
        dt_cpu = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": w["n"] * 2 / dt_cpu, "unit": "particle-steps/s", "cores": 1,
                               "kind": "port", "sample": f"N={w['n']}, 2 SRK steps, 1 thread"}
    return out


def run_observed(precision, nsteps=2000, every=10):
    """The engine loop with an observer (a frame of the state every `every`
    steps) on the headline workload, two ways, each from a resident state:
      * per-step: one spc_step + state download per step, the host round trip
        the unchanged DoStep API imposes on a reference-style loop;
      * device loop: one spc_run call, chunks of steps as graph replays with
        snapshots of the observed steps copied back while later steps run.
    Both deliver the same frames (checked) to a consumer that reduces each to
    its global order parameter on the host (numpy, ~1 ms per frame at this N);
    device_loop_light hands the frames to a consumer that keeps only the step
    index, which shows the loop's own cost.  particle-steps/s from wall time."""
    from spc2_langevin_integration_gb300 import abi
    w = WORKLOAD
    st, omega = init_inputs(w)
    prm = workload_params(abi, w, precision)
    prm.neighbour = abi.NEIGHBOUR_CELL

    def consume(state):
        ph = state[2::3]
        return complex(np.cos(ph).mean(), np.sin(ph).mean())

    out = {}
    frames = {}
    pattern = [1] + [0] * (every - 1)
    warm = 2 * every * max(1, 64 // every)  # two chunks of the device loop
    for mode in ("per_step", "device_loop", "device_loop_light"):
        with abi.System(w["n"], prm) as s:
            s.upload_state(st)
            s.upload_omega(omega)
            if mode != "per_step":  # captures the chunk graphs outside the timed run
                s.run(w["dt"], warm, every, pattern, lambda *a: False)
            else:
                s.step(w["dt"], warm)
            s.synchronize()
            got = []
            t0 = time.perf_counter()
            if mode == "per_step":
                for k in range(1, nsteps + 1):
                    s.step(w["dt"], 1)
                    state = s.download_state()
                    if k % every == 0:
                        got.append(consume(state))
            elif mode == "device_loop":
                s.run(w["dt"], nsteps, every, pattern,
                      lambda k, t, state: got.append(consume(state)) and False)
                s.synchronize()
            else:  # the loop's own cost: the consumer keeps only the step index
                s.run(w["dt"], nsteps, every, pattern, lambda k, t, state: got.append(k) and False)
                s.synchronize()
            wall = time.perf_counter() - t0
            frames[mode] = got
            out[mode] = {"value": w["n"] * nsteps / wall, "unit": "particle-steps/s", "wall_s": wall,
                         "frames": len(got)}
            if mode != "per_step":
                nodes, gsteps = s.run_graph_nodes()
                out[mode]["graph"] = {"kernel_nodes": nodes, "steps": gsteps}
    out["same_frames"] = frames["per_step"] == frames["device_loop"]
    out["device_loop_over_per_step"] = out["device_loop"]["value"] / out["per_step"]["value"]
    out["config"] = {"workload": w["name"], "steps": nsteps, "frame_every": every,
                     "neighbour": "cell", "precision": "fp32c" if precision else "fp64"}
    return out


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811
        import torch
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return world, rank, local, dist


def reduce_max(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], device="cuda", dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload_params(abi, w, precision, rank=0):
    return abi.make_params(L=w["L"], v0=w["v0"], sigma=w["sigma"], rho=w["rho"], alpha=w["alpha"],
                           D_phi=w["D_phi"], model=abi.MODEL_VORTEX, stepper=abi.STEPPER_SRK,
                           precision=precision, seed=w["seed"], system_id=rank,
                           neighbour=(abi.NEIGHBOUR_CELL if precision == abi.PRECISION_FP32X
                                      else abi.NEIGHBOUR_VERLET), skin=w["skin"])


def tune_form(abi, w, precision, rank=0):
    """The autotuner's choice for this workload and precision (spc_autotune_ex:
    neighbour method and skin, kernel choice, CTAs per cell), with every
    candidate's ms per step.  Returns (params, tuning, info)."""
    st, omega = init_inputs(w, seed_offset=rank)
    t0 = time.perf_counter()
    base = workload_params(abi, w, precision, rank)
    cands, best = abi.autotune_ex(w["n"], base, st, omega, dt=w["dt"], trial_steps=20)
    info = {"choice": cands[best], "candidates": cands, "tuning_s": time.perf_counter() - t0}
    return abi.params_with(base, cands[best]), cands[best], info


def run_form(abi, torch, w, precision, steps, warmup, rank, dist, params=None, sparse_below=None,
             e2e=True, tile_split=None, cell_units=None, subcells=None):
    """Device-timed graph replays of the workload; then (e2e) the same through
    the C-ABI with host buffers, and a per-phase profile.

    The cost of a step grows as the vortex system clusters (denser cells, more
    pairs), so every timed replay, device-timed and end-to-end alike, starts
    from the same warm state: the state after the warm-up replays, kept in
    pinned host memory.  Its upload is outside the CUDA events of the
    device-timed replays and inside the end-to-end timing."""
    import ctypes as C
    n = w["n"]
    st, omega = init_inputs(w, seed_offset=rank)
    p = params if params is not None else workload_params(abi, w, precision, rank)
    s = abi.System(n, p)
    if sparse_below is not None and p.neighbour == abi.NEIGHBOUR_CELL:
        s.set_tuning(abi.TUNE_SPARSE_BELOW, sparse_below)
    if tile_split is not None:
        s.set_tuning(abi.TUNE_TILE_SPLIT, tile_split)
    if cell_units is not None:
        s.set_tuning(abi.TUNE_CELL_UNITS, cell_units)
    if subcells is not None:
        s.set_tuning(abi.TUNE_SUBCELLS, subcells)
    s.upload_state(st)
    s.upload_omega(omega)
    stream = torch.cuda.ExternalStream(s.stream)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    dt = w["dt"]
    for _ in range(warmup):
        s.step(dt, SIM_STEPS_PER_BENCH_STEP, graph=True)
    s.synchronize()
    L = abi.lib()
    ptrs = [C.c_void_p(), C.c_void_p()]
    for q in ptrs:
        L.spc_alloc_pinned(3 * n * 8, C.byref(q))
    warm, host = [np.ctypeslib.as_array((C.c_double * (3 * n)).from_address(q.value)) for q in ptrs]
    warm[:] = s.download_state()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    for k in range(steps):
        s.upload_state(warm)
        flush.zero_()
        torch.cuda.synchronize()
        ev[k][0].record(stream)
        s.step(dt, SIM_STEPS_PER_BENCH_STEP, graph=True)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    ms = sum(a.elapsed_time(b) for a, b in ev)
    ms = reduce_max(dist, ms)
    launches = s.graph_nodes() * steps  # one graph replay per bench step
    e2e_ms, R = None, None
    if e2e:
        # e2e through the C-ABI with host buffers: pinned upload, 100 steps, download
        e2e_ms = 0.0
        for k in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.upload_state(warm)
            s.step(dt, SIM_STEPS_PER_BENCH_STEP, graph=True)
            s.download_state(host)
            e2e_ms += (time.perf_counter() - t0) * 1e3
        e2e_ms = reduce_max(dist, e2e_ms)
    s.upload_state(warm)
    prof = s.profile_steps(dt, 20)
    if e2e:
        R = s.order_params()
    del warm, host
    for q in ptrs:
        L.spc_free_pinned(q)
    s.close()
    return ms, e2e_ms, prof, R, launches


def candidates_per_particle(w, state):
    """Mean candidate tests per particle of the cell-list passes on a state:
    the members of each particle's 3x3 stencil of cells of side L / int(L / rho)."""
    L, nc = w["L"], int(w["L"] / w["rho"])
    cx = np.minimum((state[0::3] / L * nc).astype(np.int64), nc - 1)
    cy = np.minimum((state[1::3] / L * nc).astype(np.int64), nc - 1)
    occ = np.bincount(cy * nc + cx, minlength=nc * nc).reshape(nc, nc)
    sten = sum(np.roll(np.roll(occ, dy, 0), dx, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1))
    return float(sten[cy, cx].mean())


def apply_tuning(abi, s, tun):
    """Set a cell-list handle's kernel choice from a tuning candidate."""
    s.set_tuning(abi.TUNE_SPARSE_BELOW, tun["sparse_below"])
    s.set_tuning(abi.TUNE_TILE_SPLIT, tun["tile_split"])
    s.set_tuning(abi.TUNE_CELL_UNITS, tun.get("cell_units", 0))
    s.set_tuning(abi.TUNE_SUBCELLS, tun.get("subcells", 0))


def phase_sample(abi, w, params, s, state, omega, dt):
    """Outside the timers: a per-phase CUDA-event profile of 10 steps and the
    neighbour work (candidate tests, pairs within rho) on a copy of the current
    state, in a second handle with the same parameters and tuning, so the
    measured handle, its graph and its trajectory are left as they are."""
    with abi.System(w["n"], params) as c:
        if params.neighbour == abi.NEIGHBOUR_CELL:
            for key in (abi.TUNE_SPARSE_BELOW, abi.TUNE_TILE_SPLIT, abi.TUNE_CELL_UNITS,
                        abi.TUNE_SUBCELLS):
                c.set_tuning(key, s.get_tuning(key))
        c.upload_omega(omega)
        c.upload_state(state)
        pairs = float(c.neighbour_counts().mean())
        prof = c.profile_steps(dt, 10)
    return {"profile_ms": prof, "candidates": candidates_per_particle(w, state), "pairs": pairs}


def run_configured(abi, torch, w, precision, params, tuning, steps, warmup, rank, dist,
                   total_steps=None, sample_phases=False):
    """The whole configured run of the workload (w["steps"] simulation steps
    from the seeded initial state, Philox counters from 0), split into `steps`
    bench steps of total_steps / steps simulation steps each (graph replays of
    100).  One pass gives both measurements:
      * device time: CUDA events on the library's stream around each bench
        step's replays (inputs resident in HBM);
      * end to end: wall clock around each bench step's call cycle through the
        C-ABI with pinned host buffers: upload of the step's input state, the
        replays, download of its result (the same state values, so the
        trajectory is the one the device-time measurement follows).
    L2 is flushed (a 512 MB write) before each bench step, outside both timers.
    `warmup` bench steps run first (graph capture, caches); then the state and
    the step counter are reset, so the timed steps are the configured run.
    After each bench step, outside the timers, the global and local order
    parameters are recorded (the drift series), and the handle is tuned again
    on the current, clustering state: a cell-list handle after every bench
    step, in place (spc_retune: kernel choice, CTAs per cell, cell units,
    sub-cells;
    state and step counter are left as they were), a Verlet-row handle when
    its cost per step has moved by more than 25% since its last tuning, by
    spc_autotune_ex over every method, moving to a new handle (state,
    frequencies and step counter carried over) when another method wins.  The step graph is captured again before the next
    bench step (spc_prepare_graph), so no capture falls inside the timers.
    sample_phases: after each bench step, also a phase profile and the
    neighbour work on a copy of the state (phase_sample), for the roofline
    averaged over the run."""
    import ctypes as C
    n = w["n"]
    total = total_steps or w["steps"]
    per = total // steps // SIM_STEPS_PER_BENCH_STEP * SIM_STEPS_PER_BENCH_STEP
    if per <= 0:
        raise ValueError(f"--steps {steps} leaves less than 100 steps per bench step")
    reps = per // SIM_STEPS_PER_BENCH_STEP
    st, omega = init_inputs(w, seed_offset=rank)
    s = abi.System(n, params)
    if params.neighbour == abi.NEIGHBOUR_CELL:
        apply_tuning(abi, s, tuning)
    s.upload_omega(omega)
    stream = torch.cuda.ExternalStream(s.stream)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    dt = w["dt"]
    L = abi.lib()
    q = C.c_void_p()
    L.spc_alloc_pinned(3 * n * 8, C.byref(q))
    host = np.ctypeslib.as_array((C.c_double * (3 * n)).from_address(q.value))
    s.upload_state(st)
    for _ in range(warmup):
        for _ in range(reps):
            s.step(dt, SIM_STEPS_PER_BENCH_STEP, graph=True)
    s.synchronize()
    host[:] = st
    s.upload_state(host)
    s.step_counter = 0
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    wall, series, retunes, samples = [], [], [], []
    launches = 0
    tuned_at = None  # ms per simulation step when last tuned
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    for k in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.upload_state(host)
        ev[k][0].record(stream)
        for _ in range(reps):
            s.step(dt, SIM_STEPS_PER_BENCH_STEP, graph=True)
        ev[k][1].record(stream)
        s.download_state(host)
        wall.append((time.perf_counter() - t0) * 1e3)
        launches += s.graph_nodes() * reps  # the kernels of the graph this bench step replayed
        o = s.order_params()
        series.append((per * (k + 1), o["R"], o["R_local"]))
        cost = ev[k][0].elapsed_time(ev[k][1]) / per
        if sample_phases:
            samples.append(phase_sample(abi, w, params, s, host, omega, dt))
        # a cell-list handle retunes in place after every bench step (a few
        # dozen eager steps, outside the timers); a Verlet-row handle, whose
        # retune builds a handle per candidate, when its cost has moved by 25%
        moved = tuned_at is not None and abs(cost - tuned_at) > 0.25 * tuned_at
        if tuned_at is None and params.neighbour != abi.NEIGHBOUR_CELL:
            tuned_at = cost
        elif (params.neighbour == abi.NEIGHBOUR_CELL or moved) and k + 1 < steps:
            if params.neighbour == abi.NEIGHBOUR_CELL:
                cands, best = s.retune(dt, trial_steps=10)
                choice = cands[best]
            else:
                cands, best = abi.autotune_ex(n, params, host, omega, dt=dt, trial_steps=5)
                choice = cands[best]
                if choice["neighbour"] != "verlet" or choice["skin"] != params.skin:
                    ctr = s.step_counter
                    s.close()
                    params = abi.params_with(params, choice)
                    s = abi.System(n, params)
                    if params.neighbour == abi.NEIGHBOUR_CELL:
                        apply_tuning(abi, s, choice)
                    s.upload_omega(omega)
                    s.upload_state(host)
                    s.step_counter = ctr
                    stream = torch.cuda.ExternalStream(s.stream)
            s.prepare_graph(dt, SIM_STEPS_PER_BENCH_STEP)
            retunes.append({"after_step": per * (k + 1), "choice": choice})
            tuned_at = cost
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    ms = reduce_max(dist, sum(a.elapsed_time(b) for a, b in ev))
    e2e_ms = reduce_max(dist, sum(wall))
    prof = s.profile_steps(dt, 20)  # on the final (clustered) state
    final_state = host.copy()
    del host
    L.spc_free_pinned(q)
    s.close()
    return {"ms": ms, "e2e_ms": e2e_ms, "steps_per_bench_step": per, "series": series,
            "profile_ms": prof, "launches": launches, "retunes": retunes, "samples": samples,
            "final_state": final_state,
            "ms_per_bench_step": [a.elapsed_time(b) for a, b in ev]}


def drift_of(ref_series, series):
    """max |delta| of R and R_local over the recorded points."""
    a, b = np.array(ref_series), np.array(series)
    return {"max_dR": float(np.abs(b[:, 1] - a[:, 1]).max()),
            "max_dR_local": float(np.abs(b[:, 2] - a[:, 2]).max()),
            "points": len(a), "every_steps": int(a[0, 0])}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--drift-series", default=None,
                    help="--workload drift: also write the sampled series to this JSON file")
    ap.add_argument("--ncu-case", choices=["fp32c", "fp32x", "fp64", "ensemble_fp32c", "ensemble_fp32x",
                                           "ensemble_fp64", "va", "allpairs"],
                    default=None,
                    help="run a few plain (ungraphed) steps of the workload (or of an ensemble of "
                         "--ensemble-systems systems) for an ncu capture")
    ap.add_argument("--ensemble-systems", type=int, default=512)
    ap.add_argument("--ensemble-shard", action="store_true",
                    help="ensemble on N GPUs: partition the 512 systems over the ranks by "
                         "footprint (strong scaling) instead of one full ensemble per rank")
    ap.add_argument("--form", choices=["fp32c", "fp32x", "fp64"], default=None,
                    help="time only this precision form of the workload with --neighbour / "
                         "--skin (no autotune): the command for a launch list of the timed region")
    ap.add_argument("--neighbour", choices=["cell", "verlet"], default="cell")
    ap.add_argument("--skin", type=float, default=None)
    ap.add_argument("--tile-split", type=int, default=None,
                    help="--form: CTAs per cell of the cell-tile passes (0: the default, 1)")
    ap.add_argument("--cell-units", type=int, choices=[0, 1], default=None,
                    help="--form / --ncu-case (FP32C, FP32X): run the cells as units of 32 particles x "
                         "one staging round in a second launch of each pass (SPC_TUNE_CELL_UNITS)")
    ap.add_argument("--subcells", type=int, choices=[0, 1], default=None,
                    help="--form / --ncu-case (FP32C, FP32X): bin into half-cells and run the cells as "
                         "units of their halves (SPC_TUNE_SUBCELLS)")
    ap.add_argument("--save-final-states", default=None,
                    help="headline run: write each form's state after the whole run to "
                         "<dir>/final_state_<form>.npz")
    ap.add_argument("--ncu-state", default="initial",
                    help="--ncu-case fp32c/fp32x/fp64: start from the seeded initial state "
                         "('initial'), the clustered state of tests/golden/states (4,000 FP64 "
                         "steps, 'clustered') or a state file of --save-final-states; "
                         "--tile-split and --sparse-below set the kernel choice")
    ap.add_argument("--cell-list", action="store_true",
                    help="--ncu-case fp32c/fp64: the cell-list passes instead of the Verlet rows")
    ap.add_argument("--workload",
                    choices=["vortex", "ensemble", "serve", "drift", "drift-ensemble", "drift-oracle",
                             "large", "va", "observed", "choices"],
                    default="vortex",
                    help="vortex: the headline single-system line; ensemble: 512 systems in one "
                         "batch; serve: the Poisson request stream; drift: FP32C vs FP64 order "
                         "parameters over 10^4 steps; drift-ensemble: per-system order-parameter "
                         "drift of the 512-system ensemble against FP64 over 5,000 steps; "
                         "large: Chimera RK4, N=2^22, L=64; va: the "
                         "vortex-arrays model, N=51,200, L=8; observed: the headline workload "
                         "with a frame every 10 steps, per-step loop vs the device loop; choices: "
                         "phase profiles of cell tiles, cell units and sub-cells (float forms)")
    ap.add_argument("--sparse-below", type=float, default=None,
                    help="ensemble: neighbour-kernel tuning (mean particles per cell below "
                         "which a system runs the warp-per-cell passes)")
    ap.add_argument("--compare-kernels", action="store_true",
                    help="ensemble: also time every system on the cell-tile passes")
    ap.add_argument("--drift-steps", type=int, default=10000)
    ap.add_argument("--drift-seed", type=int, default=None,
                    help="drift: seed of the vortex workload (initial state, frequencies, "
                         "Philox key) in place of its own (1)")
    ap.add_argument("--serve-duration", type=float, default=2.0,
                    help="serve: seconds of the Poisson trace served (2 s: 384 requests, a few "
                         "minutes of device time; the FP64 form takes most of it)")
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-form", choices=["all", "fp32x", "fp32c", "fp64"], default="all",
                    help="serve: the precision forms served (one batch each)")
    args = ap.parse_args()
    if args.workload == "ensemble":
        import torch
        from spc2_langevin_integration_gb300 import abi, replicas
        # the host baseline first: its process pool starts before any GPU call
        cpu = None
        if int(os.environ.get("RANK", "0")) == 0 and not args.no_cpu_baseline:
            cpu = cpu_ensemble_baseline()
        world, rank, local, dist = dist_setup(args)
        subset = None
        if world > 1 and args.ensemble_shard:
            # strong scaling: the 512 systems partitioned by footprint
            sizes = [n for _, n, _, _, _ in ensemble_systems()]
            subset = replicas.shard(sizes, world, rank)
        res = {}
        runs = [("fp32c", abi.PRECISION_FP32C, 20, args.sparse_below),
                ("fp32x", abi.PRECISION_FP32X, 20, args.sparse_below),
                ("fp64", abi.PRECISION_FP64, 3, args.sparse_below)]
        if args.compare_kernels:
            runs += [("fp32c_tile_only", abi.PRECISION_FP32C, 5, 0.0),
                     ("fp64_tile_only", abi.PRECISION_FP64, 1, 0.0)]
        dev = "cuda" if world > 1 else None
        for name, prec, graphs, sb in runs:
            ntot, ctot, ms, prof = run_ensemble(prec, graphs, rank=rank, sparse_below=sb,
                                                subset=subset)
            ms = replicas.max_over_ranks(ms, dist, dev)
            work = replicas.sum_over_ranks(ntot * 100 * graphs, dist, dev)
            res[name] = {"value": work / (ms / 1e3), "steps": 100 * graphs,
                         "ms": ms, "profile_ms": prof, "sparse_below": sb}
        ntot = int(replicas.sum_over_ranks(ntot, dist, dev))
        if rank == 0:
            print(json.dumps({"metric": "particle-steps/s", "workload": "ensemble_512_euler",
                              "value": res["fp32c"]["value"], "unit": "particle-steps/s",
                              "n_gpus": world, "scaling": "strong" if subset is not None else "weak",
                              "systems": 512, "particles": ntot, "cells": ctot,
                              **res,
                              "fp32c_over_fp64": res["fp32c"]["value"] / res["fp64"]["value"],
                              "fp32x_over_fp64": res["fp32x"]["value"] / res["fp64"]["value"],
                              "graph_steps": 100, "l2": "working set > L2 (about 1 GB)",
                              "cpu_baseline": cpu}))
        if dist is not None:
            dist.destroy_process_group()
        return
    if args.workload == "choices":
        print(json.dumps({"workload": "choices", "config": WORKLOAD, "unit": "us per SRK step",
                          "rows": run_choices()}))
        return
    if args.workload == "va":
        print(json.dumps({"metric": "particle-steps/s", "workload": VA["name"], "config": VA,
                          "dtype": "f64", "fp64": run_va(100, cpu=not args.no_cpu_baseline)}))
        return
    if args.workload == "large":
        from spc2_langevin_integration_gb300 import abi
        # each form: a warm replay of `steps` steps, then the timed replay of the
        # next `steps` (the same number for every form, so the final states
        # can be compared: RK4 with D = 0 is deterministic)
        out = {"metric": "particle-steps/s", "workload": LARGE["name"], "config": LARGE,
               "fp32x": run_large(abi.PRECISION_FP32X, 4),
               "fp32c": run_large(abi.PRECISION_FP32C, 4),
               "fp64": run_large(abi.PRECISION_FP64, 4),
               "note": "throughput over a timed prefix of the 2,000-step run (one graph replay "
                       "per form after a warm replay); working set >> L2"}
        ref = out["fp64"].pop("_state")
        for f in ("fp32x", "fp32c"):
            d = (out[f].pop("_state") - ref).reshape(-1, 3)
            d[:, :2] -= LARGE["L"] * np.round(d[:, :2] / LARGE["L"])
            out[f]["max_abs_state_diff_vs_fp64_after_8_steps"] = float(np.abs(d).max())
            out[f + "_over_fp64"] = out[f]["value"] / out["fp64"]["value"]
        print(json.dumps(out))
        return
    if args.workload == "drift":
        out = {"metric": "order-parameter drift, FP32C vs FP64", "workload": "drift"}
        out.update(run_drift(steps=args.drift_steps, out_path=args.drift_series, seed=args.drift_seed))
        print(json.dumps(out))
        return
    if args.workload == "drift-ensemble":
        from spc2_langevin_integration_gb300 import abi
        out = {"metric": "order-parameter drift vs FP64, per system", "workload": "ensemble_512_euler"}
        subset = list(range(args.ensemble_systems)) if args.ensemble_systems < 512 else None
        out.update(run_drift_ensemble([("fp32c", abi.PRECISION_FP32C), ("fp32x", abi.PRECISION_FP32X)],
                                      steps=min(args.drift_steps, 5000), subset=subset,
                                      series_path=args.drift_series))
        print(json.dumps(out))
        return
    if args.workload == "drift-oracle":
        out = {"metric": "order-parameter drift vs the FP64 CPU oracle (identical normals)",
               "workload": "ensemble_512_euler systems"}
        out.update(run_drift_oracle(DRIFT_ORACLE_SYSTEMS, steps=min(args.drift_steps, 5000)))
        print(json.dumps(out))
        return
    if args.workload == "observed":
        from spc2_langevin_integration_gb300 import abi
        out = {"metric": "particle-steps/s with an observer", "workload": "observed"}
        out["fp32c"] = run_observed(abi.PRECISION_FP32C)
        out["fp64"] = run_observed(abi.PRECISION_FP64, nsteps=100)
        print(json.dumps(out))
        return
    if args.workload == "serve":
        from spc2_langevin_integration_gb300 import abi
        out = {"metric": "served time-to-result", "workload": "poisson_requests_euler"}
        for name, prec in (("fp32x", abi.PRECISION_FP32X), ("fp32c", abi.PRECISION_FP32C),
                           ("fp64", abi.PRECISION_FP64)):
            if args.serve_form in ("all", name):
                out[name] = run_serving(prec, args.serve_duration, args.serve_rate)
        print(json.dumps(out))
        return
    if args.ncu_case == "allpairs":
        # one all-pairs system (rho > L/4): N = 4,096 in L = 1, rho = 0.3,
        # Chimera SRK in FP64 (ChimeraSystem.cpp:117-255)
        from spc2_langevin_integration_gb300 import abi
        n, L = 4096, 1.0
        rng = np.random.default_rng(17)
        st = np.empty(3 * n)
        st[0::3] = rng.uniform(0.0, L, n)
        st[1::3] = rng.uniform(0.0, L, n)
        st[2::3] = rng.uniform(-np.pi, np.pi, n)
        p = abi.make_params(L=L, v0=0.01, sigma=1.0, rho=0.3, alpha=1.45, D_phi=0.005,
                            stepper=abi.STEPPER_SRK, seed=17)
        with abi.System(n, p) as s:
            s.upload_state(st)
            s.step(0.01, 3)
            s.synchronize()
        return
    if args.ncu_case == "va":
        from spc2_langevin_integration_gb300 import abi
        w = VA
        prm = {k: w[k] for k in ("velocity", "mu_plus", "mu_minus", "xi_a", "xi_r", "D_phi",
                                 "kappa", "rho")}
        with abi.System(w["n"], abi.make_va_params(L=w["L"], stepper=abi.STEPPER_SRK,
                                                   seed=w["seed"], **prm)) as s:
            s.upload_state(va_inputs(w))
            s.step(w["dt"], 3)
            s.synchronize()
        return
    if args.ncu_case and args.ncu_case.startswith("ensemble"):
        from spc2_langevin_integration_gb300 import abi
        prec = {"fp32c": abi.PRECISION_FP32C, "fp32x": abi.PRECISION_FP32X,
                "fp64": abi.PRECISION_FP64}[args.ncu_case.split("_")[1]]
        systems = ensemble_systems(count=args.ensemble_systems)
        ntot = sum(n for _, n, _, _, _ in systems)
        ctot = sum(abi.cells_of(L, prm["rho"]) for _, _, L, prm, _ in systems)
        with abi.Batch(abi.STEPPER_EULER, prec, len(systems), ntot, ctot) as b:
            if args.sparse_below is not None:
                b.set_tuning(abi.TUNE_SPARSE_BELOW, args.sparse_below)
            for k, n, L, prm, st in systems:
                b.admit(n, abi.make_params(L=L, stepper=abi.STEPPER_EULER, precision=prec, seed=2,
                                           system_id=k, **prm), st)
            b.step(0.01, 3)
            b.synchronize()
        print(json.dumps({"ncu_case": args.ncu_case, "systems": len(systems), "particles": ntot,
                          "cells": ctot}))
        return
    if args.ncu_case:
        from spc2_langevin_integration_gb300 import abi
        w = WORKLOAD
        st, omega = init_inputs(w)
        if args.ncu_state != "initial":
            # "clustered": the workload after 4,000 FP64 steps
            # (tests/golden/make_clustered.py); else a state file written by
            # --save-final-states
            path = (os.path.join(ROOT, "tests", "golden", "states", "vortex_clustered_n65536.npz")
                    if args.ncu_state == "clustered" else args.ncu_state)
            st = np.load(path)["state"].copy()
        prec = {"fp32c": abi.PRECISION_FP32C, "fp32x": abi.PRECISION_FP32X,
                "fp64": abi.PRECISION_FP64}[args.ncu_case]
        p = abi.make_params(L=w["L"], v0=w["v0"], sigma=w["sigma"], rho=w["rho"],
                            alpha=w["alpha"], D_phi=w["D_phi"], model=abi.MODEL_VORTEX,
                            stepper=abi.STEPPER_SRK, precision=prec, seed=w["seed"],
                            neighbour=(abi.NEIGHBOUR_CELL if args.cell_list or prec == abi.PRECISION_FP32X
                                       else abi.NEIGHBOUR_VERLET),
                            skin=w["skin"])
        with abi.System(w["n"], p) as s:
            if p.neighbour == abi.NEIGHBOUR_CELL:
                if args.sparse_below is not None:
                    s.set_tuning(abi.TUNE_SPARSE_BELOW, args.sparse_below)
                if args.tile_split is not None:
                    s.set_tuning(abi.TUNE_TILE_SPLIT, args.tile_split)
                if args.cell_units is not None:
                    s.set_tuning(abi.TUNE_CELL_UNITS, args.cell_units)
                if args.subcells is not None:
                    s.set_tuning(abi.TUNE_SUBCELLS, args.subcells)
            s.upload_state(st)
            s.upload_omega(omega)
            s.step(w["dt"], 3)
            s.synchronize()
        return
    w = WORKLOAD
    world, rank, local, dist = dist_setup(args)
    n_total = w["n"] * world
    config = {"workload": w["name"], "N": w["n"], "L": w["L"], "stepper": "srk",
              "model": "vortex (alignment + natural frequencies)",
              "neighbour": "autotuned per precision (cell list or Verlet rows; see autotune)",
              "dt": w["dt"], "sim_steps_per_bench_step": SIM_STEPS_PER_BENCH_STEP,
              "l2": "flushed between bench steps (512 MB write, outside the timed events)",
              "parallelism": f"replicas{world}"}

    if args.impl == "reference":
        if rank != 0:
            return
        # the reference's CPU path (restated, bit-identical) on the host cores
        from oracle import pyoracle as po  # noqa: F401
        vals = []
        for _ in range(args.warmup):
            cpu_baseline(w, nsteps=1)
        for _ in range(args.steps):
            vals.append(cpu_baseline(w, nsteps=1)["value"])
        v = float(np.mean(vals))
        cb = cpu_baseline(w, nsteps=1)
        allc = cpu_replicas_baseline(nsteps=1)
        print(json.dumps({
            "impl": "reference", "metric": "particle-steps/s", "value": v,
            "unit": "particle-steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
            "cpu_baseline": {"kind": cb["kind"], "cores": 1, "sample": cb["sample"], "value": v},
            # one system uses one core; every core, one replica each:
            "all_cores_replicas": allc,
            "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}))
        return

    import torch
    from spc2_langevin_integration_gb300 import abi
    torch.cuda.set_device(local)
    if args.form:
        prec = {"fp32c": abi.PRECISION_FP32C, "fp32x": abi.PRECISION_FP32X,
                "fp64": abi.PRECISION_FP64}[args.form]
        p = workload_params(abi, w, prec, rank)
        p.neighbour = abi.NEIGHBOUR_VERLET if args.neighbour == "verlet" else abi.NEIGHBOUR_CELL
        if args.skin is not None:
            p.skin = args.skin
        ms, e2e_ms, prof, _, launches = run_form(abi, torch, w, prec, args.steps, args.warmup,
                                                 rank, dist, p, tile_split=args.tile_split,
                                                 cell_units=args.cell_units, subcells=args.subcells)
        if rank == 0:
            print(json.dumps({"form": args.form, "neighbour": args.neighbour, "skin": p.skin,
                              "tile_split": args.tile_split,
                              "value": n_total * SIM_STEPS_PER_BENCH_STEP * args.steps / (ms / 1e3),
                              "ms_per_bench_step": ms / args.steps, "profile_ms": prof,
                              "gpu_launches": launches}))
        return
    forms = [("fp32x", abi.PRECISION_FP32X), ("fp32c", abi.PRECISION_FP32C),
             ("fp64", abi.PRECISION_FP64)]
    tuned = {name: tune_form(abi, w, prec, rank) for name, prec in forms}
    runs = {}
    with ClockSampler(local) as clk:
        for name, prec in forms:
            best, tun, _ = tuned[name]
            runs[name] = run_configured(abi, torch, w, prec, best, tun, args.steps, args.warmup,
                                        rank, dist, sample_phases=True)
    total = runs["fp64"]["steps_per_bench_step"] * args.steps  # 10^4 when K divides it
    if args.save_final_states and rank == 0:
        os.makedirs(args.save_final_states, exist_ok=True)
        for name in runs:
            np.savez(os.path.join(args.save_final_states, f"final_state_{name}.npz"),
                     state=runs[name]["final_state"], omega=init_inputs(w)[1])
    per_form = {}
    for name, _ in forms:
        r = runs[name]
        per_form[name] = {
            "value": n_total * total / (r["ms"] / 1e3),
            "e2e": n_total * total / (r["e2e_ms"] / 1e3),
            "ms_per_step": r["ms"] / args.steps,
            "ms_per_bench_step": r["ms_per_bench_step"],
            "profile_ms_final_state": r["profile_ms"],
            "autotune": tuned[name][2],
            "retunes": r["retunes"],
            "order_params_series": [[int(k), R, Rl] for k, R, Rl in r["series"]]}
        if name != "fp64":
            per_form[name]["drift_vs_fp64"] = drift_of(runs["fp64"]["series"], r["series"])
    # the headline form: the fastest whose drift from FP64 in this run stays
    # within the 1e-4 target (FP64 itself when none does)
    ok = [nm for nm, _ in forms if nm != "fp64"
          and per_form[nm]["drift_vs_fp64"]["max_dR"] <= 1e-4
          and per_form[nm]["drift_vs_fp64"]["max_dR_local"] <= 1e-4]
    head = max(ok, key=lambda nm: per_form[nm]["value"]) if ok else "fp64"
    hr = runs[head]
    value = per_form[head]["value"]
    # the earlier measurement window, for comparison: replays from the state
    # after the warm-up, repeated (the cheapest, unclustered part of the run)
    best, tun, _ = tuned[head]
    ms_w, _, _, _, _ = run_form(abi, torch, w, dict(forms)[head], args.steps, args.warmup, rank,
                                dist, best, tun["sparse_below"], e2e=False,
                                tile_split=tun["tile_split"], cell_units=tun["cell_units"],
                                subcells=tun.get("subcells", 0))
    hbm, peak_kind = peaks()
    # per-phase launch durations averaged over the run: a CUDA-event profile
    # after each bench step (on a copy of the state, outside the timers)
    smp = hr["samples"]
    phases = {k: float(np.mean([x["profile_ms"][k] for x in smp]))
              for k in ("stage", "sort", "gather", "pass1", "pass2")}
    dom = max(phases, key=phases.get)
    achieved = ALG_BYTES[dom] * w["n"] / (phases[dom] * 1e-3) / 1e9
    # compute-side work of one neighbour pass over the run: candidate tests
    # (3x3 cells of side L / int(L / rho)) and pairs within rho per particle,
    # from the same sampled states
    cand = float(np.mean([x["candidates"] for x in smp]))
    pairs = float(np.mean([x["pairs"] for x in smp]))
    p1 = sum(x["profile_ms"]["pass1"] for x in smp) * 1e-3
    traffic = NCU_TRAFFIC.get((head, dom))
    dtypes = {"fp32x": "f32x (f32 pair tests; exact i64 fixed-point neighbour sums; f64 "
                       "per-particle rates, noise, positions, phase)",
              "fp32c": "f32c (f32 sums/trig/increments; f64 cutoff, positions, phase)",
              "fp64": "f64"}
    config = dict(config, sim_steps_per_bench_step=hr["steps_per_bench_step"],
                  run="the whole configured run: %d steps from the seeded initial state "
                      "(Philox counters from 0), in %d bench steps" % (total, args.steps),
                  start_state="seeded initial state; warm-up bench steps run first, then the "
                              "state and step counter are reset")
    out = {
        "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": hr["ms"] / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": dtypes[head],
        "data": "synthetic (seeded uniform positions/phases, normal frequencies)",
        "config": config, "form": head,
        "drift": per_form[head].get("drift_vs_fp64"),
        "forms": per_form,
        "fp32x_over_fp64": per_form["fp32x"]["value"] / per_form["fp64"]["value"],
        "fp32c_over_fp64": per_form["fp32c"]["value"] / per_form["fp64"]["value"],
        "value_warm_window": n_total * SIM_STEPS_PER_BENCH_STEP * args.steps / (ms_w / 1e3),
        "gpu_launches": hr["launches"],
        "roofline": {"bound": "hbm", "kernel": dom, "kernels": PHASE_KERNELS[head][dom],
                     "achieved": achieved, "peak": hbm,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic["bytes"] if traffic else None,
                     "traffic_state": traffic["state"] if traffic else None,
                     "alg_bytes_per_particle": ALG_BYTES[dom],
                     "alg_bytes_per_launch": ALG_BYTES[dom] * w["n"],
                     "phase_ms_run_mean": phases,
                     "timing": "live CUDA-event profile of 10 steps after each of the %d bench "
                               "steps (on a copy of the state, outside the timers), averaged "
                               "over the run" % len(smp),
                     "compute": {"candidate_tests_per_s": w["n"] * cand * len(smp) / p1,
                                 "pair_terms_per_s": w["n"] * pairs * len(smp) / p1,
                                 "candidates_per_particle_run_mean": cand,
                                 "pairs_per_particle_run_mean": pairs},
                     "note": "the neighbour passes are bound by instruction issue and latency "
                             "on an L2-resident working set, not by HBM: the HBM fraction is "
                             "low by construction"},
        "e2e": {"value": per_form[head]["e2e"], "unit": "particle-steps/s",
                "h2d_bytes_per_step": 3 * w["n"] * 8, "d2h_bytes_per_step": 3 * w["n"] * 8,
                "per_call": "pinned state upload, the bench step's steps, state download"},
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(w)
    if rank == 0:
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
