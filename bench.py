"""Benchmark of the GB300 simulation step on the batched multicompartment network.

Workload (one GPU): 10,000 cells with seeded random branching trees (segment
count log-uniform in [1, 500], 0.80 M compartments), HH soma + passive
dendrites, 1 M expTwoSynapse connections at fixed in-degree 100 with
0.5-5 ms delays, 1 M 5 Hz poissonFiringSynapse inputs; dt 0.025 ms.  A bench
"step" is one pass of the simulation loop over STEPS_PER_ITER simulation
steps; `value` is compartment-steps/s (compartments x simulation steps /
device time) with the network resident in HBM; `e2e` runs the whole
configured simulation (1 s, 40,001 steps) through the C ABI from host buffers
(model upload and device layout, stepping, record fetches) on the wall clock.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Under torchrun each rank advances an independent replica (its own seed):
the path does not shard, so `scaling` is weak and no collective is used.
`--impl reference` times the CPU restatement of the reference loop (the
reference's own build needs its source tree, absent where this runs) with
all host threads on the same workload and prints the same line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "compartment-steps/s, batched vs plain GPU, at ≤0.1 ms spike-time error"
UNIT = "compartment-steps/s"
STEPS_PER_ITER = 320          # simulation steps per bench step (16 windows of 20)
L2_FLUSH_BYTES = 256 << 20    # written between timed iterations (> 129 MB L2)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cells", type=int, default=10000)
    ap.add_argument("--seed", type=int, default=1234)
    ap.add_argument("--profile", action="store_true",
                    help="only advance the batched path (init + warmup + steps bench steps) for ncu")
    ap.add_argument("--shape", type=str, default="",
                    help="batched launch shape steps_per_launch,segments_per_warp,segments_per_depth "
                         "(0 = built-in) instead of the autotuner's")
    ap.add_argument("--profile-adjoint", type=float, default=0.0, metavar="MS",
                    help="only run one gradient forward and backward of the ball-and-stick "
                         "configuration over MS ms, for ncu")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# algorithmic bytes per simulation step (each SoA array streamed once, FP32):
# passive compartment 24 B, HH compartment 48 B, izhikevich 16 B, expTwo
# synapse 33 B, expOne 25 B, Poisson source 16 B + its synapse, pulse 12 B,
# delivered event 5 B
# ---------------------------------------------------------------------------
def algorithmic_bytes(low, events_per_step: float) -> dict:
    n_comp = low.n_comp
    chan_gated = (low.chan_types["n_gates"][low.chan_type] > 0).astype(np.int64)
    per_comp = np.add.reduceat(np.concatenate([chan_gated, [0]]), low.comp_chan_off[:-1]) if n_comp else np.zeros(0)
    per_comp[low.comp_chan_off[:-1] == low.comp_chan_off[1:]] = 0
    n_hh = int((per_comp > 0).sum())
    kinds = low.syn_types["kind"]
    syn_b = float(np.where(kinds[low.syn_type] == 1, 33, 25).sum()) if len(low.syn_type) else 0.0
    pois_b = float(np.where(kinds[low.pois_type] == 1, 33 + 16, 25 + 16).sum()) if len(low.pois_type) else 0.0
    cells_b = 48.0 * n_hh + 24.0 * (n_comp - n_hh) + 16.0 * low.n_izh
    inputs_b = syn_b + pois_b + 12.0 * len(low.pulse_target)
    return {"cells": cells_b, "inputs": inputs_b, "deliver": 5.0 * events_per_step,
            "total": cells_b + inputs_b + 5.0 * events_per_step}


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int = 0):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() in ("active", "0x1") or flag == "1":
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def flush_l2(buf):
    import torch
    buf.fill_(1.0)
    torch.cuda.synchronize()


# ---------------------------------------------------------------------------
def out_degree(low) -> np.ndarray:
    """Connection synapses on each spike source's fan-out."""
    return np.bincount(np.asarray(low.syn_src, np.int64), minlength=len(low.src_target)).astype(np.int64)


def cpu_sample(low, threads: int, budget_s: float = 15.0, max_steps: int = 2000):
    """Time the CPU restatement on a bounded number of simulation steps of the
    same workload (the wall clock from the first non-initialisation step to
    the end of the run); returns (compartment-steps/s, steps timed,
    synaptic events/s)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle", "port"))
    import eden_port
    probe = eden_port.run(low, n_steps=4, trace_target=np.zeros(0, np.int32), threads=threads, spike_cap=1 << 20,
                          mark_step=1)
    per = probe["timed_s"] / 4.0
    n = int(max(8, min(max_steps, budget_s / max(per, 1e-6))))
    out = eden_port.run(low, n_steps=n, trace_target=np.zeros(0, np.int32), threads=threads, spike_cap=1 << 24,
                        mark_step=1)
    dt = out["timed_s"]
    events = float(out_degree(low)[out["spike_src"]].sum())
    return low.n_target * n / dt, n, events / dt


def precision_sample(low, n_steps: int = 800, dev: int = 0, trace_target=None):
    """Spike-time and voltage error of the batched GPU path against the
    double-precision oracle (the C restatement built for the GPU in double,
    oracle/gpu64) over the first n_steps of the same network."""
    sys.path.insert(0, os.path.join(ROOT, "oracle", "port"))
    import eden_port
    from eden_gb300.engine import MODE_BATCHED, Simulation
    tt = np.ascontiguousarray(low.trace_target if trace_target is None else trace_target, np.int32)
    f64 = eden_port.run_gpu64(low, n_steps=n_steps, trace_target=tt, spike_cap=1 << 24, device=dev)
    sim = Simulation(low, mode=MODE_BATCHED, device=dev, record_capacity_steps=n_steps + 8, trace_target=tt,
                     spike_capacity=1 << 24)
    rec = sim.run(n_steps)
    sim.close()
    keep = f64["spike_step"] <= n_steps
    a = {}
    for s_, k in zip(f64["spike_src"][keep], f64["spike_step"][keep]):
        a.setdefault(int(s_), []).append(int(k))
    b = {}
    for s_, k in zip(rec.spike_src, rec.spike_step):
        b.setdefault(int(s_), []).append(int(k))
    mismatch, worst = 0, 0
    for c in set(a) | set(b):
        x, y = sorted(a.get(c, [])), sorted(b.get(c, []))
        if len(x) != len(y):
            mismatch += 1
        elif x:
            worst = max(worst, max(abs(p - q) for p, q in zip(x, y)))
    dv = float(np.abs(rec.trace.astype(np.float64) - f64["trace"]).max()) if rec.trace.size else 0.0
    dt_ms = float(low.dt) * 1e-3
    return {"reference": "double-precision GPU oracle (oracle/gpu64: the C restatement in FP64)",
            "steps": n_steps, "ms": n_steps * dt_ms, "spikes": int(keep.sum()), "cells_count_mismatch": mismatch,
            "max_spike_shift_ms": worst * dt_ms, "max_abs_dv_mV": dv}


def adjoint_sample():
    """The adjoint parameter-fitting configuration: 256 ball-and-stick cells
    (soma + 50-compartment cable, HH everywhere), 7 parameters per cell
    (soma and dendrite gNa, gK, gL; Ra) drawn lognormal, a 0.5 nA step for
    150 ms, dt 0.025 ms for 200 ms (8001 steps); loss = MSE of the somatic V
    against the trace of a second seeded parameter draw.  Times one forward
    (trace + checkpoints every 100 steps) and one backward (recomputed
    segments + adjoint) through edenGpuGrad*, the batched simulation of the
    same network, and checks the gradient of the first 16 cells against the
    double-precision forward sensitivities (oracle/cable_grad.py) contracted
    with the same trace gradient over the first 100 ms, and against central
    differences of the single-precision forward over the whole 200 ms."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from cable_grad import Cable, loss_and_trace_grad
    from eden_gb300 import lowering, workloads
    from eden_gb300.engine import MODE_BATCHED, Simulation
    from eden_gb300.gradient import CableGradient, per_cell_density_map, with_weights
    dens = [1, 2, 0, 4, 5, 3]
    spec = workloads.ball_and_stick(seed=1234)
    tspec = workloads.ball_and_stick(seed=4321)
    low = lowering.lower(spec)
    rec = np.ascontiguousarray(low.phys_comp_off[:-1], np.int32)
    pm = per_cell_density_map(low, dens)
    tpm = per_cell_density_map(lowering.lower(tspec), dens)
    g = CableGradient(low, pm, rec_comp=rec, checkpoint_every=100)
    target = g.forward(tpm.values).astype(np.float64)
    fwd, bwd = [], []
    for _ in range(3):
        tr = g.forward(pm.values)
        loss, tg = loss_and_trace_grad(tr.astype(np.float64), target)
        grad = g.backward(tg)
        f, b = g.timing()
        fwd.append(f)
        bwd.append(b)
    g.close()
    sim = Simulation(low, mode=MODE_BATCHED, trace_target=rec)
    sim.run()
    sim_ms = sim.device_ms
    sim.close()
    # accuracy on a bounded sample of 16 cells.  (1) Against the FP64 forward
    # sensitivities over the first 100 ms, where the single- and
    # double-precision trajectories still agree within a fraction of a mV;
    # later a spike can land one step apart in the two, and gradients taken
    # along different trajectories no longer compare.  (2) Over the whole
    # 200 ms, against central differences of the same single-precision
    # forward, on the (cell, parameter) pairs where the loss is smooth at
    # that scale: differences with relative steps 1e-3 and 3e-3 agree within
    # 1 %.  A cell near its firing threshold gains or loses a spike under
    # such a step; those pairs are counted, not compared.
    n_sub, sub_ms = 16, 100.0
    sub = workloads.ball_and_stick(n_inst=n_sub, length_ms=sub_ms, params=spec.params[:n_sub])
    slow = lowering.lower(sub)
    spm = per_cell_density_map(slow, dens)
    srec = np.ascontiguousarray(slow.phys_comp_off[:-1], np.int32)
    gs = CableGradient(slow, spm, rec_comp=srec)
    tr_s = gs.forward(spm.values).astype(np.float64)
    _, tg_s = loss_and_trace_grad(tr_s, target[:slow.n_steps, :n_sub])
    grad_s = gs.backward(tg_s).reshape(-1, 7)
    gs.close()
    cab = Cable(slow, spm.chan_param, spm.cell_ra_param, slow.phys_ra)
    dirs = np.zeros((7, spm.n_params))
    for j in range(7):
        dirs[j, j::7] = 1.0
    _, dtr = cab.run(spm.values, slow.n_steps, srec, dirs)
    g64 = np.einsum("nc,jnc->cj", tg_s, dtr)
    rel = float((np.abs(grad_s - g64).max(0) / np.abs(g64).max(0)).max())
    full = workloads.ball_and_stick(n_inst=n_sub, params=spec.params[:n_sub])
    flow = lowering.lower(full)
    fpm = per_cell_density_map(flow, dens)
    gf = CableGradient(flow, fpm, rec_comp=srec)
    tr_f = gf.forward(fpm.values).astype(np.float64)
    tgt_f = target[:flow.n_steps, :n_sub]
    _, tg_f = loss_and_trace_grad(tr_f, tgt_f)
    grad_f = gf.backward(tg_f).reshape(-1, 7)
    vals = np.asarray(fpm.values, np.float64)

    def central(h):
        fd = np.zeros((n_sub, 7))
        for j in range(7):
            lp = []
            for sgn in (1.0, -1.0):
                v = vals.copy()
                v[j::7] *= 1.0 + sgn * h
                t = gf.forward(v.astype(np.float32)).astype(np.float64)
                lp.append(((t - tgt_f) ** 2).sum(0) / tr_f.size)
            fd[:, j] = (lp[0] - lp[1]) / (2.0 * h * vals[j::7])
        return fd
    fd1, fd3 = central(1e-3), central(3e-3)
    gf.close()
    scale_j = np.abs(fd1).max(0)
    smooth = np.abs(fd1 - fd3) <= 1e-2 * scale_j
    rel_fd = np.abs(grad_f - fd1) / scale_j
    f_ms, b_ms = min(fwd), min(bwd)
    # the same cells with synaptic drive fixed in advance: 8 spike-list expTwo
    # connections per cell on the dendrite and 2 timed expOne inputs on the
    # soma, every weight a parameter as well
    dlow = lowering.lower(workloads.ball_and_stick(seed=1234, syn_drive=8))
    dpm = with_weights(dlow, per_cell_density_map(dlow, dens))
    gd = CableGradient(dlow, dpm, rec_comp=rec, checkpoint_every=100)
    dfwd, dbwd = [], []
    for _ in range(3):
        tr = gd.forward(dpm.values)
        _, tg = loss_and_trace_grad(tr.astype(np.float64), target)
        gd.backward(tg)
        f, b = gd.timing()
        dfwd.append(f)
        dbwd.append(b)
    gd.close()
    # (one FP64 direction per weight: 4 cells over 50 ms)
    nd_sub, dsub_ms = 4, 50.0
    dsub = lowering.lower(workloads.ball_and_stick(n_inst=nd_sub, length_ms=dsub_ms, params=spec.params[:nd_sub],
                                                   syn_drive=8))
    dspm = with_weights(dsub, per_cell_density_map(dsub, dens))
    srec = np.ascontiguousarray(dsub.phys_comp_off[:-1], np.int32)
    gs = CableGradient(dsub, dspm, rec_comp=srec)
    tr_s = gs.forward(dspm.values).astype(np.float64)
    _, tg_s = loss_and_trace_grad(tr_s, target[:dsub.n_steps, :nd_sub])
    grad_d = gs.backward(tg_s)
    gs.close()
    wpar = np.concatenate([dspm.syn_param, dspm.timed_param])
    dcab = Cable(dsub, dspm.chan_param, dspm.cell_ra_param, dsub.phys_ra, dspm.syn_param, dspm.timed_param)
    wdirs = np.zeros((len(wpar), dspm.n_params))
    wdirs[np.arange(len(wpar)), wpar] = 1.0
    _, wdtr = dcab.run(dspm.values, dsub.n_steps, srec, wdirs)
    gw64 = np.einsum("nc,jnc->j", tg_s, wdtr)
    wrel = float(np.abs(grad_d[wpar] - gw64).max() / np.abs(gw64).max())
    f_d, b_d = min(dfwd), min(dbwd)
    return {"config": "ball_and_stick: 256 cells x 51 compartments, 7 parameters each (1792), "
                      "dt 0.025 ms, 200 ms (8001 steps), checkpoints every 100 steps",
            "synaptic_drive": {
                "config": f"the same cells with 8 spike-list expTwo connections and 2 timed expOne inputs each, "
                          f"every weight a parameter too ({dpm.n_params} parameters)",
                "forward_ms": f_d, "backward_ms": b_d, "backward_over_forward": b_d / f_d,
                "weight_grad_max_rel_err_vs_fp64": wrel,
                "grad_check": f"first {nd_sub} cells, first {dsub_ms:g} ms: the weights' GPU adjoint against "
                              "double-precision forward sensitivities, relative to the largest"},
            "loss": loss, "grad_norm": float(np.linalg.norm(grad)),
            "forward_ms": f_ms, "backward_ms": b_ms, "backward_over_forward": b_ms / f_ms,
            "batched_simulation_ms": sim_ms, "backward_over_batched_simulation": b_ms / sim_ms,
            "grad_max_rel_err_vs_fp64": rel,
            "grad_check": f"first {n_sub} cells, first {sub_ms:g} ms: GPU adjoint vs double-precision forward "
                          "sensitivities contracted with the same trace gradient, per parameter, relative "
                          "to that parameter's largest gradient",
            "whole_run_vs_central_differences": {
                "cells": n_sub, "ms": 200.0, "pairs": int(smooth.size), "smooth_pairs": int(smooth.sum()),
                "max_rel_err_smooth": float(rel_fd[smooth].max()) if smooth.any() else None,
                "median_rel_err_all": float(np.median(rel_fd)),
                "check": "GPU adjoint vs central differences (relative step 1e-3) of the same FP32 forward, "
                         "relative to each parameter's largest difference; smooth pairs: steps 1e-3 and "
                         "3e-3 agree within 1 %"}}


def scale_sample(dev: int):
    """The scale configuration: 160,000 izhikevich2007 cells + 40,000
    100-compartment HH-dendrite trees (4.16 M compartments), 20 M expTwo
    synapses (in-degree 100, delays 0.5-10 ms), 20 M Poisson inputs at 2 Hz,
    dt 0.025 ms.  Device memory the context holds, and batched and plain
    throughput over 640 simulation steps after 320 warm-up steps (inputs
    resident; the network is 1.2 GB, far above L2)."""
    import torch
    from eden_gb300 import lowering, workloads
    from eden_gb300.engine import MODE_BATCHED, MODE_PLAIN, Simulation
    t0 = time.perf_counter()
    low = lowering.lower(workloads.mixed_scale())
    t_lower = time.perf_counter() - t0
    out = {"workload": f"mixed_scale: {low.n_izh} izhikevich2007 + {low.n_phys} trees, {low.n_comp} compartments, "
                       f"{len(low.syn_target)} expTwo synapses, {len(low.pois_target)} Poisson inputs at 2 Hz",
           "targets": low.n_target, "host_lowering_s": t_lower}
    for mode, key in ((MODE_BATCHED, "batched"), (MODE_PLAIN, "plain")):
        torch.cuda.synchronize(dev)
        free0 = torch.cuda.mem_get_info(dev)[0]
        t0 = time.perf_counter()
        sim = Simulation(low, mode=mode, device=dev, record_capacity_steps=STEPS_PER_ITER * 2,
                         spike_capacity=1 << 24)
        t_create = time.perf_counter() - t0
        free1 = torch.cuda.mem_get_info(dev)[0]
        sim.initialize()
        sim.run_steps(STEPS_PER_ITER)
        sim.fetch()
        ms, spikes = 0.0, 0
        for _ in range(2):
            ms += sim.run_steps(STEPS_PER_ITER)
            spikes += len(sim.fetch().spike_src)
        sim.close()
        steps = 2 * STEPS_PER_ITER
        fan = len(low.syn_target) / max(len(low.src_target), 1)
        ab = algorithmic_bytes(low, spikes * fan / steps)
        out[key] = {"value": low.n_target * steps / (ms * 1e-3), "unit": UNIT, "ms_per_sim_step": ms / steps,
                    "events_per_s": spikes * fan / (ms * 1e-3),
                    "device_bytes": int(free0 - free1), "create_s": t_create,
                    "step_algorithmic_bytes": ab["total"],
                    "step_algorithmic_gbs": ab["total"] / (ms / steps * 1e-3) / 1e9,
                    "spikes_per_sim_step": spikes / steps}
    out["ratio_batched_over_plain"] = out["batched"]["value"] / out["plain"]["value"]
    # V of ten somas and ten izhikevich cells
    tt = np.concatenate([low.phys_comp_off[:10], low.n_comp + np.arange(min(10, low.n_izh))])
    out["spike_time_error"] = precision_sample(low, n_steps=400, dev=dev, trace_target=tt)
    out["fits_180_gb"] = max(out["batched"]["device_bytes"], out["plain"]["device_bytes"]) < 180e9
    return out


def roofline_object(kernel, achieved, peak, peak_kind, bytes_per_launch, avg_ms, ab, sim_steps, total_ms):
    """The dominant kernel against the HBM roofline.  `achieved` is its
    algorithmic bytes (the per-unit figures above, for the K steps one launch
    advances) over its CUDA-event launch time: an effective rate, which can
    exceed what DRAM moves because a window keeps its units' state on chip
    for K steps.  `traffic` is what ncu counted in DRAM for one launch of the
    same workload (profiles/), and dram_frac_ncu that traffic's rate against
    the peak; their gap from `frac` says the kernel is bounded by instruction
    issue and dependent latency rather than by HBM."""
    traffic = load_profile_traffic()
    out = {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peak, "unit": "GB/s",
           "frac": achieved / peak, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
           "achieved_is": "algorithmic bytes per launch (K steps) / CUDA-event launch time",
           "traffic": traffic, "bytes_per_launch": bytes_per_launch, "avg_launch_ms": avg_ms,
           "step_algorithmic_bytes": ab["total"],
           "step_algorithmic_gbs": ab["total"] * sim_steps / (total_ms * 1e-3) / 1e9}
    if traffic:
        out["dram_gbs_ncu"] = traffic / (avg_ms * 1e-3) / 1e9
        out["dram_frac_ncu"] = out["dram_gbs_ncu"] / peak
        out["limiter"] = ("instruction issue and dependent latency: ncu DRAM traffic is "
                          f"{traffic / bytes_per_launch:.3f} of the algorithmic bytes")
    return out


def config_sample(key: str, dev: int, threads: int):
    """Throughput of a further configuration at its stated size: C1 (1,000
    single-compartment HH cells with DC pulses, dt 0.025 ms) over its whole
    second, or C3 (100,000 izhikevich2007 cells, 10 M expOne synapses, dt
    0.1 ms) over 1,000 steps after 200 warm-up steps; batched and plain
    device time, synaptic events/s, and the CPU restatement on a bounded
    sample of the same network with every host thread."""
    from eden_gb300 import lowering, workloads
    from eden_gb300.engine import MODE_BATCHED, MODE_PLAIN, Simulation
    if key == "c1":
        low = lowering.lower(workloads.single_comp_hh())
        warm, steps = 0, int(low.n_steps)
        desc = "single_comp_hh: 1000 HH cells, DC pulses, no synapses, dt 0.025 ms, the whole 1 s (40,001 steps)"
    else:
        low = lowering.lower(workloads.izh_net())
        warm, steps = 200, 1000
        desc = ("izh_net: 100000 izhikevich2007 cells, 10 M expOne synapses (in-degree 100, delays 1-20 ms), "
                "DC pulses, dt 0.1 ms, 1,000 steps after 200")
    outdeg = out_degree(low)
    out = {"workload": desc, "targets": low.n_target, "synapses": int(len(low.syn_target))}
    for mode, name in ((MODE_BATCHED, "batched"), (MODE_PLAIN, "plain")):
        sim = Simulation(low, mode=mode, device=dev, record_capacity_steps=4096, spike_capacity=1 << 24)
        sim.initialize()
        if warm:
            sim.run_steps(warm)
            sim.fetch()
        ms, ev, done = 0.0, 0, 0
        while done < steps:
            k = min(4000, steps - done)
            ms += sim.run_steps(k)
            ev += int(outdeg[sim.fetch().spike_src].sum())
            done += k
        sim.close()
        out[name] = {"value": low.n_target * steps / (ms * 1e-3), "unit": UNIT, "ms_per_sim_step": ms / steps,
                     "events_per_s": ev / (ms * 1e-3)}
    out["ratio_batched_over_plain"] = out["batched"]["value"] / out["plain"]["value"]
    cval, n, cev = cpu_sample(low, threads, budget_s=10.0, max_steps=40000)
    out["cpu_baseline"] = {"value": cval, "unit": UNIT, "cores": threads, "kind": "port", "events_per_s": cev,
                           "sample": f"the first {n} simulation steps (after the 4 initialisation passes), "
                                     f"C restatement of the reference loop, OpenMP {threads} threads"}
    return out


def load_profile_traffic():
    """DRAM bytes per k_cells_t launch from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "k_cells_t_multicomp_net.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return d.get("dram_bytes_per_launch_scaled")
    return None


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def replica_seed(base: int, rank: int) -> int:
    """Each rank simulates its own replica of the network."""
    return base + rank


def max_over_ranks(x: float, dist) -> float:
    """The slowest rank's figure (timings are taken as the max over ranks)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def profile_adjoint(length_ms: float):
    from eden_gb300 import lowering, workloads
    from eden_gb300.gradient import CableGradient, per_cell_density_map
    low = lowering.lower(workloads.ball_and_stick(length_ms=length_ms))
    pm = per_cell_density_map(low, [1, 2, 0, 4, 5, 3])
    g = CableGradient(low, pm, rec_comp=np.ascontiguousarray(low.phys_comp_off[:-1], np.int32))
    tr = g.forward(pm.values)
    g.backward(np.ones_like(tr) / tr.size)
    print(json.dumps({"forward_ms": g.timing()[0], "backward_ms": g.timing()[1], "steps": low.n_steps}))
    g.close()


def main():
    args = parse()
    if args.profile_adjoint > 0:
        profile_adjoint(args.profile_adjoint)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    from eden_gb300 import lowering, workloads

    spec = workloads.multicomp_net(n_cells=args.cells, seed=replica_seed(args.seed, rank))
    low = lowering.lower(spec)
    config = {"workload": f"multicomp_net: {args.cells} cells, {low.n_comp} compartments, "
                          f"{len(low.syn_target)} expTwo synapses (in-degree 100, delay 0.5-5 ms), "
                          f"{len(low.pois_target)} Poisson inputs at 5 Hz, dt 0.025 ms",
              "cells": args.cells, "compartments": low.n_comp, "synapses": int(len(low.syn_target)),
              "poisson_inputs": int(len(low.pois_target)), "sim_steps_per_bench_step": STEPS_PER_ITER,
              "l2": "flushed (256 MB write) between timed bench steps", "replicas": world, "seed": args.seed}

    if args.impl == "reference":
        # the reference's CPU loop (its C restatement; the reference's own
        # build needs its source tree, absent here) with every host thread:
        # `warmup` bench steps of STEPS_PER_ITER simulation steps untimed,
        # then exactly `steps` bench steps timed on the wall clock
        if rank != 0:
            return
        sys.path.insert(0, os.path.join(ROOT, "oracle", "port"))
        import eden_port
        threads = os.cpu_count() or 1
        n_warm, n_timed = args.warmup * STEPS_PER_ITER, args.steps * STEPS_PER_ITER
        out = eden_port.run(low, n_steps=n_warm + n_timed, trace_target=np.zeros(0, np.int32), threads=threads,
                            spike_cap=1 << 24, mark_step=n_warm + 1)
        timed = out["timed_s"]
        val = low.n_target * n_timed / timed
        timed_spikes = out["spike_src"][out["spike_step"] > n_warm]
        events_s = float(out_degree(low)[timed_spikes].sum()) / timed
        line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": timed / args.steps * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded generator)", "config": config,
                "events_per_s": events_s,
                "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                                 "sample": f"{args.steps} bench steps of {STEPS_PER_ITER} simulation steps each "
                                           f"({n_timed} steps) of the full workload, timed after "
                                           f"{args.warmup} untimed bench steps and the 4 initialisation passes; "
                                           f"C restatement of the reference loop, OpenMP {threads} threads"},
                "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    from eden_gb300 import autotune
    from eden_gb300.engine import MODE_BATCHED, MODE_PLAIN, Simulation
    torch.cuda.set_device(dev)
    # ---- launch shape: the autotuner's choice (searched once per network
    # and device, outside every timed region), or the one given
    if args.shape:
        k, spw, spd = (int(x) for x in args.shape.split(","))
        shape = {"steps_per_launch": k, "segments_per_warp": spw, "segments_per_depth": spd}
        config["launch_shape"] = dict(shape, source="--shape")
    else:
        tuned = autotune.tune(low, dev)
        shape = autotune.options(tuned)
        config["launch_shape"] = dict(shape, source="autotuner", search_s=round(tuned["search_s"], 2),
                                      candidates_timed=len(tuned["tried"]), cached=tuned["cached"])
    if args.profile:
        sim = Simulation(low, mode=MODE_BATCHED, device=dev, record_capacity_steps=STEPS_PER_ITER * 2, **shape)
        sim.initialize()
        for _ in range(args.warmup + args.steps):
            sim.run_steps(STEPS_PER_ITER)
            sim.fetch()
        sim.close()
        print("profile run done")
        return
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    # ---- device-timed batched run (kernel timing on: CUDA events around each launch)
    sim = Simulation(low, mode=MODE_BATCHED, device=dev, kernel_timing=True, record_capacity_steps=STEPS_PER_ITER * 2,
                     **shape)
    sim.initialize()
    for _ in range(max(3, args.warmup)):
        sim.run_steps(STEPS_PER_ITER)
        sim.fetch()
    base_stats = sim.kernel_stats()
    launches0 = sum(n for _, n in base_stats.values())
    clocks = ClockSampler()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    total_ms, spikes, events = 0.0, 0, 0
    outdeg = out_degree(low)
    for _ in range(args.steps):
        flush_l2(flush)
        total_ms += sim.run_steps(STEPS_PER_ITER)
        rec = sim.fetch()
        spikes += len(rec.spike_src)
        events += int(outdeg[rec.spike_src].sum())
    torch.cuda.synchronize()
    clk = clocks.stop()
    stats = sim.kernel_stats()
    sim.close()
    gpu_launches = sum(n for _, n in stats.values()) - launches0
    total_ms = max_over_ranks(total_ms, dist)
    sim_steps = STEPS_PER_ITER * args.steps
    value = world * low.n_target * sim_steps / (total_ms * 1e-3)

    events_per_s = world * events / (total_ms * 1e-3)

    # ---- roofline of the dominant kernel (k_cells_t), bytes per launch
    events_per_step = events / sim_steps
    ab = algorithmic_bytes(low, events_per_step)
    k_ms = {k: (stats[k][0] - base_stats[k][0], stats[k][1] - base_stats[k][1]) for k in stats}
    dom = max(k_ms, key=lambda k: k_ms[k][0])
    steps_per_launch = sim_steps / max(1, k_ms[dom][1])
    bytes_per_launch = {"k_cells_t": ab["cells"], "k_inputs_t": ab["inputs"],
                        "k_deliver_t": ab["deliver"]}.get(dom, ab["total"]) * steps_per_launch
    avg_ms = k_ms[dom][0] / max(1, k_ms[dom][1])
    achieved = bytes_per_launch / (avg_ms * 1e-3) / 1e9
    peak, peak_kind = peaks()

    # ---- plain (per-step) GPU path on the same network, for the batched/plain ratio
    psim = Simulation(low, mode=MODE_PLAIN, device=dev, record_capacity_steps=STEPS_PER_ITER * 2)
    psim.initialize()
    psim.run_steps(STEPS_PER_ITER)
    psim.fetch()
    plain_ms = 0.0
    for _ in range(2):
        flush_l2(flush)
        plain_ms += psim.run_steps(STEPS_PER_ITER)
        psim.fetch()
    psim.close()
    plain_ms = max_over_ranks(plain_ms, dist)
    plain_value = low.n_target * 2 * STEPS_PER_ITER / (plain_ms * 1e-3)

    # ---- end to end through the C ABI, the whole configured run (1 s of
    # simulated time): model upload and layout, stepping, record fetches
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e2e_steps = int(low.n_steps)
    t0 = time.perf_counter()
    esim = Simulation(low, mode=MODE_BATCHED, device=dev, record_capacity_steps=4096, **shape)
    rec_bytes = 0
    esim.initialize()
    done = 0
    while done < e2e_steps:
        k = min(4096, e2e_steps - done)
        esim.run_steps(k)
        r = esim.fetch()
        rec_bytes += r.trace.nbytes + r.trace_step.nbytes + r.spike_src.nbytes + r.spike_step.nbytes
        done += k
    esim.close()
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist)
    model_bytes = sum(a.nbytes for a in esim._keep)
    e2e_value = world * low.n_target * e2e_steps / e2e_s

    # ---- CPU baseline (rank 0 only)
    cpu = precision = adjoint = scale = c1 = c3 = None
    if rank == 0 and world == 1:
        threads = os.cpu_count() or 1
        cval, n, cev = cpu_sample(low, threads, budget_s=15.0)
        cpu = {"value": cval, "unit": UNIT, "cores": threads, "kind": "port", "events_per_s": cev,
               "sample": f"{n} simulation steps of the same network (after 4 init passes), C restatement of "
                         f"the reference loop, OpenMP {threads} threads"}
        precision = precision_sample(low, dev=dev)
        c1 = config_sample("c1", dev, threads)
        c3 = config_sample("c3", dev, threads)
        adjoint = adjoint_sample()
        scale = scale_sample(dev)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator)",
                "config": config,
                "plain_gpu": {"value": plain_value, "unit": UNIT, "ratio_batched_over_plain": value / world / plain_value},
                "e2e": {"value": e2e_value, "unit": UNIT,
                        "h2d_bytes_per_step": model_bytes / (e2e_steps + 4),
                        "d2h_bytes_per_step": rec_bytes / e2e_steps, "steps": e2e_steps,
                        "seconds": e2e_s,
                        "covers": "create (upload, device layout, kernels compiled for the model or "
                                  "taken from the process cache), the whole configured run, record fetches"},
                "events_per_s": events_per_s,
                "events_unit": "synaptic events/s (spikes x their connection fan-out, per second of device time)",
                "gpu_launches": int(gpu_launches),
                "roofline": roofline_object(dom, achieved, peak, peak_kind, bytes_per_launch, avg_ms, ab,
                                            sim_steps, total_ms),
                "kernels_ms": {k: round(v[0], 3) for k, v in k_ms.items()},
                "clocks": clk,
                "cpu_baseline": cpu,
                "spike_time_error": precision,
                "c1": c1,
                "c3": c3,
                "adjoint": adjoint,
                "scale": scale}
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
