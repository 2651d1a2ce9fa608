"""The C++ host program on the GPU: a lowered network written to a model
file (eden_gb300/model_file.py) is run by eden_gb300/host/eden_gpu_host
through the C ABI alone -- edenGpuCreate, edenGpuRun in chunks,
edenGpuFetchRecords, edenGpuDestroy -- and its output files are checked

* against the reference simulator's own outputs for the same LEMS file
  (tests/golden/*.npz): samecount(0.1 ms) and box(0.1 ms, the case's mV);
* against the Python front end's files for the same run (eden_gb300/cli.py
  writing the records of eden_gb300/engine.py's Simulation): identical text,
  since both drive the same library with the same kernels."""
import os
import subprocess

import numpy as np
import pytest

from criteria import box_violations, samecount
from eden_gb300 import build, cli, lowering, model_file, neuroml_io
from eden_gb300.engine import MODE_BATCHED, MODE_PLAIN, Simulation
from golden.cases import CASES, spec_of
from golden_io import load
from helpers import spike_trains

pytestmark = pytest.mark.gpu


def _run_host(name, mode, tmp_path, chunk=1000):
    lems = neuroml_io.write_lems(spec_of(name), str(tmp_path))
    spec = neuroml_io.read_lems(lems)
    low = lowering.lower(spec)
    path = str(tmp_path / "model.egm")
    model_file.write_for_spec(path, spec, low)
    traj, ev = str(tmp_path / "host_traj.txt"), str(tmp_path / "host_ev.txt")
    p = subprocess.run([build.build_host(), path, traj, ev, mode, str(chunk)], capture_output=True, text=True,
                       timeout=600)
    assert p.returncode == 0, p.stderr
    assert "Run:" in p.stdout
    return spec, low, traj, ev


@pytest.mark.parametrize("mode", ["batched", "plain"])
@pytest.mark.parametrize("name", ["single_comp_hh", "izh_net", "multicomp_poisson", "spike_sources"])
def test_host_program_matches_reference_outputs(name, mode, tmp_path):
    spec, low, traj, ev = _run_host(name, mode, tmp_path)
    ref_trace, ref_src, ref_step = load(name, low)
    t = np.loadtxt(traj, ndmin=2)
    assert t.shape == (low.n_steps, 1 + len(low.trace_target))
    trace = t[:, 1:] * 1e3
    e = np.loadtxt(ev, ndmin=2).reshape(-1, 2)
    sid = {s[0]: j for j, s in enumerate(spec.event_files[0]["sels"])}
    src = low.event_src[[sid[int(i)] for i in e[:, 1]]] if len(e) else np.zeros(0, np.int32)
    step = np.rint(e[:, 0] / (float(low.dt) * 1e-6)).astype(np.int64) + 1
    dt_ms = float(low.dt) * 1e-3
    wrong, far = samecount(spike_trains(ref_src, ref_step), spike_trains(src, step), int(round(0.1 / dt_ms)))
    assert not wrong and not far, f"spike trains differ: counts {wrong[:5]}, timing {far[:5]}"
    nbad, worst = box_violations(ref_trace, trace, dt_ms, 0.1, CASES[name][2])
    assert nbad == 0, f"{nbad} samples outside box, worst {worst} mV"


@pytest.mark.parametrize("mode", ["batched", "plain"])
def test_host_program_writes_what_the_python_front_end_writes(mode, tmp_path):
    spec, low, traj, ev = _run_host("izh_net", mode, tmp_path, chunk=333)
    sim = Simulation(low, mode=MODE_BATCHED if mode == "batched" else MODE_PLAIN)
    rec = sim.run(chunk=333)  # the same calls: each edenGpuRun starts its own windows
    sim.close()
    out = tmp_path / "py"
    out.mkdir()
    files = cli.write_outputs(spec, low, rec, str(out), low.n_steps)
    assert open(files[0]).read() == open(traj).read()
    assert open(files[1]).read() == open(ev).read()
