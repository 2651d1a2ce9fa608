"""`eden nml <LEMS file>` on the GPU, and the runEden() wrapper.

Drop-in for the reference's command line (eden/Eden.cpp:10379-10546) and its
Python wrapper (testing/python_package/eden_simulator/run_sim.py:22-107):
the same LEMS/NeuroML input, the same output files -- OutputFile trajectories
as "%+16.8g" columns (time in seconds, then each quantity in SI units,
eden/Eden.cpp:10856-10871) and EventOutputFile spikes in TIME_ID / ID_TIME
form (10897-10927) -- and the same `Config: .. Setup: .. Run: ..` timing line
(11951).  Command-line tokens the reference accepts are accepted; `gcc`,
`icc` and the CPU-only debugging tokens are ignored.

    python -m eden_gb300 nml LEMS_file.xml [rng_seed N] [verbose] [plain]
"""
from __future__ import annotations

import os
import sys
import time
from collections import OrderedDict

import numpy as np

from . import lowering, neuroml_io


def _fmt(x: float) -> str:
    return "%+16.8g" % x


def _step_times_us(dt_us: float, last_step: int) -> np.ndarray:
    """Simulation time in us of steps 0..last_step: the reference starts at
    0, runs the initialisation steps at t = 0 and then adds the float dt to a
    double accumulator once per step (eden/Eden.cpp:11486, 11931), so step
    k >= 1 runs at the double sum of k - 1 dts."""
    n = max(int(last_step), 1)
    acc = np.concatenate([[0.0], np.add.accumulate(np.full(n - 1, float(np.float32(dt_us))))])
    return np.concatenate([[0.0], acc])


def _step_times(dt_us: float, last_step: int) -> np.ndarray:
    """The same in seconds, as the output files print it."""
    return _step_times_us(dt_us, last_step) * 1e-6


def trajectory_frames(of: dict, times_us: np.ndarray, steps: np.ndarray):
    """(timestamp in us, sample row) of every frame a trajectory logger emits,
    given the step of each recorded sample (eden/Eden.cpp:11565-11599):
    explicit sample points take the first step at or after each point and
    are stamped with the point; otherwise a step inside [start, end) is
    sampled when the sampling interval has passed since the last frame."""
    frames = []
    if of.get("points"):
        pts, nxt = of["points"], 0
        for r, k in enumerate(steps):
            t = times_us[k]
            while nxt < len(pts) and pts[nxt] <= t:
                frames.append((pts[nxt], r))
                nxt += 1
        return frames
    last = -np.inf
    for r, k in enumerate(steps):
        t = times_us[k]
        if of["start"] <= t < of["end"] and last + of["interval"] <= t:
            frames.append((t, r))
            last = t
    return frames


def event_frames(ef: dict, times_us: np.ndarray, first_step: int, last_step: int, cols_at_step: dict):
    """(timestamp in us, [column indices]) of every frame an event logger
    emits (eden/Eden.cpp:11600-11633): a step inside [start, end) with events,
    or any such step once maximum_interval has passed since the last frame."""
    frames = []
    last = -np.inf
    for k in range(first_step, last_step + 1):
        t = times_us[k]
        if not (ef["start"] <= t < ef["end"]):
            continue
        inst = cols_at_step.get(k, [])
        if inst or last + ef["max_interval"] <= t:
            frames.append((t, inst))
            last = t
    return frames


def write_outputs(spec, low, rec, base_dir: str, n_steps: int) -> list:
    """Write every trajectory and event logger of the simulation in the
    reference's formats (eden/Eden.cpp:10843-10940)."""
    written = []
    last = max([int(rec.trace_step.max()) if len(rec.trace_step) else 1,
                int(rec.spike_step.max()) if len(rec.spike_step) else 1, n_steps])
    times_us = _step_times_us(float(low.dt), last)
    col0 = 0
    for of in getattr(spec, "output_files", []):
        path = os.path.join(base_dir, of["path"])
        ncol = len(of["cols"])
        scale = np.array([c[3] for c in of["cols"]], np.float64)  # engine mV -> the column's units
        block = rec.trace[:, col0:col0 + ncol].astype(np.float64) * scale
        with open(path, "w") as f:
            for t, r in trajectory_frames(of, times_us, rec.trace_step):
                f.write(_fmt(t * 1e-6) + "".join(" " + _fmt(v) for v in block[r]) + "\n")
        col0 += ncol
        written.append(path)
    off = spec.pop_offsets()
    for ef in getattr(spec, "event_files", []):
        path = os.path.join(base_dir, ef["path"])
        sels = ef["sels"]
        col_of_src = {}
        for j, (_sid, _sel, (pop, idx)) in enumerate(sels):
            col_of_src.setdefault(off[pop] + idx, []).append(j)
        cols_at_step = {}
        for s, k in zip(rec.spike_src, rec.spike_step):
            for j in col_of_src.get(int(s), []):
                cols_at_step.setdefault(int(k), []).append(j)
        for k in cols_at_step:
            cols_at_step[k].sort()
        with open(path, "w") as f:
            for t, inst in event_frames(ef, times_us, 1, n_steps, cols_at_step):
                ts = _fmt(t * 1e-6)
                if ef["format"] == "ascii_v0":
                    f.write(ts + "".join(f" {sels[j][0]}" for j in inst) + "\n")
                elif ef["format"] == "ID_TIME":
                    for j in inst:
                        f.write(f"{sels[j][0]} {ts.strip()}\n")
                else:
                    for j in inst:
                        f.write(f"{ts} {sels[j][0]}\n")
        written.append(path)
    return written


def run_lems(lems_file: str, seed: int | None = None, mode: str = "batched", verbose: bool = False,
             out_dir: str | None = None, cable_solver: str = "auto") -> dict:
    """Simulate a LEMS file on the GPU and write its output files next to it
    (or in out_dir).  Returns timing in seconds: config, setup, run."""
    from .engine import MODE_BATCHED, MODE_PLAIN, Simulation
    t0 = time.perf_counter()
    spec = neuroml_io.read_lems(lems_file)
    if seed is not None:
        spec.seed = seed
    spec.cable_solver = cable_solver
    t1 = time.perf_counter()
    low = lowering.lower(spec)
    sim = Simulation(low, mode=MODE_PLAIN if mode == "plain" else MODE_BATCHED)
    t2 = time.perf_counter()
    rec = sim.run()
    t3 = time.perf_counter()
    sim.close()
    base = out_dir or os.path.dirname(os.path.abspath(lems_file))
    files = write_outputs(spec, low, rec, base, low.n_steps)
    if verbose:
        print(f"{low.n_target} targets, {len(low.syn_target)} synapses, {low.n_steps} steps; wrote {files}")
    return {"config": t1 - t0, "setup": t2 - t1, "run": t3 - t2, "files": files}


def main(argv=None) -> int:
    argv = list(sys.argv[1:] if argv is None else argv)
    lems, seed, verbose, mode, cable = None, None, False, "batched", "auto"
    i = 0
    while i < len(argv):
        tok = argv[i]
        if tok == "nml":
            lems = argv[i + 1]
            i += 2
            continue
        if tok == "rng_seed":
            seed = int(argv[i + 1])
            i += 2
            continue
        if tok == "cable_solver":
            # eden/Eden.cpp:10485-10500
            if i + 1 >= len(argv):
                print(f"cmdline: {tok} type missing")
                return 2
            cable = argv[i + 1]
            if cable not in ("auto", "bwd_euler", "fwd_euler"):
                print(f"cmdline: unknown cable solver {cable}")
                return 2
            if cable == "fwd_euler":
                print("Cable solver set to Forward Euler: make sure system is stable")
            i += 2
            continue
        if tok == "verbose":
            verbose = True
        elif tok == "plain":
            mode = "plain"
        elif tok in ("gcc", "icc", "-S", "debug", "debug_netcode", "full_dump", "dump_state_scalar",
                     "dump_raw_layout"):
            pass
        else:
            print(f"unknown command line token {tok}")
            return 2
        i += 1
    if lems is None:
        print("usage: eden nml <LEMS file> [rng_seed N] [verbose] [plain]")
        return 2
    print("--- Extensible Dynamics Engine for Networks (GB300 step loop) ---")
    try:
        t = run_lems(lems, seed=seed, mode=mode, verbose=verbose, cable_solver=cable)
    except (ValueError, OSError) as e:
        print(f"cmdline: could not make sense of NeuroML file: {e}")
        return 1
    print("Config: %.3f Setup: %.3f Run: %.3f " % (t["config"], t["setup"], t["run"]))
    return 0


def runEden(example_lems_file, reload_events=False, threads=None, extra_cmdline_args=None, executable_path=None,
            verbose=False, full_cmdline=None):
    """Run a LEMS/NeuroML2 file on the GPU; same signature and return value as
    the reference wrapper: an OrderedDict of trajectories ('t' and one key per
    OutputColumn quantity) and, with reload_events, one of spike times per
    EventSelection select path.  `threads`, `executable_path` and
    `full_cmdline` concern the CPU executable and are accepted and ignored."""
    args = ["nml", example_lems_file] + list(extra_cmdline_args or [])
    rc = main(args)
    if rc != 0:
        raise RuntimeError("Could not run simulation")
    return reload_saved_data(example_lems_file, reload_events=reload_events)


def reload_saved_data(lems_file_name, reload_events=False):
    """Read back the output files a run wrote (run_sim.py:110-252)."""
    spec = neuroml_io.read_lems(lems_file_name)
    base = os.path.dirname(os.path.abspath(lems_file_name))
    traces, events = OrderedDict(), OrderedDict()
    for of in spec.output_files:
        data = np.loadtxt(os.path.join(base, of["path"]), ndmin=2)
        traces["t"] = data[:, 0]
        for j, (_cid, quantity, _t, _scale) in enumerate(of["cols"]):
            traces[quantity] = data[:, j + 1]
    if reload_events:
        for ef in spec.event_files:
            sel_of = {sid: select for sid, select, _ in ef["sels"]}
            for _sid, select, _ in ef["sels"]:
                events[select] = []
            with open(os.path.join(base, ef["path"])) as f:
                for line in f:
                    parts = line.split()
                    if not parts:
                        continue
                    if ef["format"] == "ascii_v0":
                        t = float(parts[0])
                        for sid in parts[1:]:
                            events[sel_of[int(sid)]].append(t)
                    elif ef["format"] == "TIME_ID":
                        events[sel_of[int(parts[1])]].append(float(parts[0]))
                    else:
                        events[sel_of[int(parts[0])]].append(float(parts[1]))
        return OrderedDict(sorted(traces.items())), OrderedDict(sorted(events.items()))
    return OrderedDict(sorted(traces.items()))
