"""The drop-in front end on the GPU: `python -m eden_gb300 nml <LEMS file>`
and `runEden()` (the reference's command line, eden/Eden.cpp:10379-10546,
and its Python wrapper, testing/python_package/eden_simulator/run_sim.py:22-107)
on LEMS files written for the golden cases, their output files compared with
the reference simulator's own files for the same input (tests/golden/*.npz):
the OutputFile's time column character for character and its values within
the case's box(0.1 ms, mV) tolerance; the EventOutputFile's events by
samecount(0.1 ms); and the extended loggers (EdenOutputFile sampling windows
and sample points, EdenEventOutputFile ascii_v0 / ID_TIME) line for line."""
import os
import subprocess
import sys

import numpy as np
import pytest

from criteria import box_violations, samecount
from eden_gb300 import cli, lowering, neuroml_io
from golden.cases import CASES, LOGGER_FILES, add_eden_loggers, spec_of
from golden_io import load
from helpers import spike_trains

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _events(path, spec, low):
    sid = {s[0]: j for j, s in enumerate(spec.event_files[0]["sels"])}
    e = np.loadtxt(path, ndmin=2).reshape(-1, 2)
    src = low.event_src[[sid[int(i)] for i in e[:, 1]]] if len(e) else np.zeros(0, np.int32)
    return src, np.rint(e[:, 0] / (float(low.dt) * 1e-6)).astype(np.int64) + 1


@pytest.mark.parametrize("mode", ["batched", "plain"])
@pytest.mark.parametrize("name", ["single_comp_hh", "izh_net", "multicomp_poisson", "input_kinds", "input_kinds_fwd"])
def test_command_line_matches_reference_files(name, mode, tmp_path):
    spec0 = spec_of(name)
    lems = neuroml_io.write_lems(spec0, str(tmp_path))
    # the cable solver is a command-line setting, as in the reference
    args = [sys.executable, "-m", "eden_gb300", "nml", os.path.basename(lems), "gcc"] + \
        (["plain"] if mode == "plain" else []) + \
        ([] if spec0.cable_solver == "auto" else ["cable_solver", spec0.cable_solver])
    p = subprocess.run(args, cwd=str(tmp_path), capture_output=True, text=True, timeout=600,
                       env=dict(os.environ, PYTHONPATH=ROOT))
    assert p.returncode == 0, p.stdout + p.stderr
    assert "Config:" in p.stdout and "Setup:" in p.stdout and "Run:" in p.stdout
    spec = neuroml_io.read_lems(lems)
    spec.cable_solver = spec0.cable_solver
    low = lowering.lower(spec)
    z = np.load(os.path.join(HERE, "golden", f"{name}.npz"))
    traj = open(os.path.join(str(tmp_path), spec.output_files[0]["path"])).read().splitlines()
    assert len(traj) == len(z["time_s"])
    assert [l[:16] for l in traj[:3]] == [str(h)[:16] for h in z["trajectory_head"]]
    mine = np.array([[float(x) for x in l.split()] for l in traj])
    ref_trace, ref_src, ref_step = load(name, low)
    dt_ms = float(low.dt) * 1e-3
    nbad, worst = box_violations(ref_trace, mine[:, 1:] * 1e3, dt_ms, 0.1, CASES[name][2])
    assert nbad == 0, f"{nbad} samples outside box, worst {worst} mV"
    src, step = _events(os.path.join(str(tmp_path), spec.event_files[0]["path"]), spec, low)
    wrong, far = samecount(spike_trains(ref_src, ref_step), spike_trains(src, step), int(round(0.1 / dt_ms)))
    assert not wrong and not far, f"spike trains differ: counts {wrong[:5]}, timing {far[:5]}"


def _event_times(lines, fmt):
    """id -> sorted event times (s) of an event file's lines."""
    out = {}
    for line in lines:
        parts = line.split()
        if not parts:
            continue
        if fmt == "ascii_v0":
            for sid in parts[1:]:
                out.setdefault(sid, []).append(float(parts[0]))
        else:
            out.setdefault(parts[0], []).append(float(parts[1]))
    return {k: np.sort(v) for k, v in out.items()}


def test_run_eden_with_extended_loggers(tmp_path):
    """runEden() on the izh_net case with EDEN's extended loggers added, its
    files against the reference's for the same LEMS file: the sampled
    trajectories' timestamps character for character and their values
    within 1 mV (0.001 V) except where a spike moved by a step; every event
    id with the reference's number of events, each within 0.1 ms."""
    lems = neuroml_io.write_lems(spec_of("izh_net"), str(tmp_path))
    add_eden_loggers(lems)
    traces, events = cli.runEden(lems, reload_events=True)
    assert len(traces["t"]) > 0 and sum(len(v) for v in events.values()) > 0
    z = np.load(os.path.join(HERE, "golden", "loggers.npz"))
    units = (1e-3, 1.0, 1.0)  # 1 mV in the columns' output units (V, mV, mV)
    for f in LOGGER_FILES:
        mine = open(os.path.join(str(tmp_path), f)).read().splitlines()
        ref = str(z[os.path.splitext(f)[0]]).splitlines()
        if f.startswith("ev"):
            fmt = "ascii_v0" if f == "ev.txt" else "ID_TIME"
            a, b = _event_times(mine, fmt), _event_times(ref, fmt)
            assert set(a) == set(b), f
            for k in b:
                assert len(a[k]) == len(b[k]) and np.abs(a[k] - b[k]).max() <= 1.0001e-4, (f, k)
        else:
            assert len(mine) == len(ref), f
            assert [l[:16] for l in mine] == [l[:16] for l in ref], f
            a = np.array([[float(x) for x in l.split()] for l in mine])[:, 1:]
            b = np.array([[float(x) for x in l.split()] for l in ref])[:, 1:]
            ok = np.abs(a - b) <= np.array(units)[None, :a.shape[1]]
            assert ok.mean() >= 0.98, (f, ok.mean())
