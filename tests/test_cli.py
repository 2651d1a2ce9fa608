"""The `eden nml` front end: LEMS in, reference-format output files out.

The files are written from the oracle's records (no GPU here) and compared
with the first lines of the reference's own files for the same LEMS input,
kept in the golden fixtures: the time column must match character for
character, values to the golden case's tolerance, and every line must have
the reference's fixed-width layout ("%+16.8g" columns, eden/Eden.cpp:144-181,
10856-10871; TIME_ID events 10914-10923)."""
import os

import numpy as np
import pytest

import eden_port
from eden_gb300 import cli, lowering, neuroml_io
from eden_gb300.engine import Records
from golden.cases import CASES, LOGGER_FILES, add_eden_loggers, spec_of

HERE = os.path.dirname(os.path.abspath(__file__))


def _write_from_oracle(name, tmp_path, extended=False):
    lems = neuroml_io.write_lems(spec_of(name), str(tmp_path))
    if extended:
        add_eden_loggers(lems)
    spec = neuroml_io.read_lems(lems)
    low = lowering.lower(spec)
    out = eden_port.run(low)
    assert out["rc"] == 0
    n = low.n_steps
    keep = out["spike_step"] <= n
    order = np.lexsort((out["spike_src"][keep], out["spike_step"][keep]))
    rec = Records(out["trace"], np.arange(1, n + 1, dtype=np.int64), out["spike_src"][keep][order],
                  out["spike_step"][keep][order])
    files = cli.write_outputs(spec, low, rec, str(tmp_path), n)
    return lems, spec, files


def _columns(line):
    """Fixed-width fields: a 16-wide timestamp, then ' ' + 16-wide value each."""
    return [line[i:i + 16] for i in range(0, len(line), 17)]


@pytest.mark.parametrize("name", ["single_comp_hh", "izh_net"])
def test_output_files_match_reference_layout(name, tmp_path):
    lems, spec, files = _write_from_oracle(name, tmp_path)
    z = np.load(os.path.join(HERE, "golden", f"{name}.npz"))
    traj = open(files[0]).read().splitlines()
    ref_head = [str(s) for s in z["trajectory_head"]]
    assert len(traj) == len(z["time_s"])
    for mine, ref in zip(traj, ref_head):
        assert len(mine) == len(ref) and (len(mine) - 16) % 17 == 0
        fm, fr = _columns(mine), _columns(ref)
        assert fm[0] == fr[0]                     # timestamps identical
        np.testing.assert_allclose(np.array(fm[1:], float), np.array(fr[1:], float),
                                   atol=CASES[name][2] * 1e-3)
    ev = open(files[1]).read().splitlines()
    ev_head = [str(s) for s in z["events_head"]]
    assert len(ev) == len(z["event_id"])
    for mine, ref in zip(ev, ev_head):
        tm, im = mine[:16], mine[17:]
        tr, ir = ref[:16], ref[17:]
        assert mine[16] == " " and im == ir
        assert abs(float(tm) - float(tr)) <= 0.1e-3


def test_reload_saved_data(tmp_path):
    lems, spec, files = _write_from_oracle("izh_net", tmp_path)
    traces, events = cli.reload_saved_data(lems, reload_events=True)
    quantities = [c[1] for of in spec.output_files for c in of["cols"]]
    assert set(traces) == {"t", *quantities}
    assert np.all(np.diff(traces["t"]) > 0)
    sels = [s[1] for ef in spec.event_files for s in ef["sels"]]
    assert set(events) == set(sels)
    assert sum(len(v) for v in events.values()) == len(open(files[1]).read().splitlines())


def test_step_times_accumulate_like_the_reference():
    t = cli._step_times(25.0, 5)
    assert t[0] == 0.0 and t[1] == 0.0
    np.testing.assert_array_equal(t[2:], np.array([25.0, 50.0, 75.0, 100.0]) * 1e-6)
    # a dt that is not exact in binary: repeated double addition, not k * dt
    dt = float(np.float32(10.0 / 3.0))
    acc, ref = 0.0, []
    for _ in range(1000):
        acc += dt
        ref.append(acc * 1e-6)
    assert np.array_equal(cli._step_times(10.0 / 3.0, 1001)[2:], np.array(ref))


def test_command_line_rejects_unknown_tokens(capsys):
    assert cli.main(["nml", "x.xml", "bogus_token"]) == 2
    assert cli.main([]) == 2
    assert cli.main(["nml", "x.xml", "cable_solver", "rk4"]) == 2
    assert cli.main(["nml", "x.xml", "cable_solver"]) == 2


def test_extended_loggers_match_reference(tmp_path):
    """EdenOutputFile (time window and sampling interval; explicit sample
    points; output_units) and EdenEventOutputFile (ascii_v0 with a time window
    and heartbeat frames; ID_TIME) written from the oracle's records against
    the reference's own files for the same LEMS input: events line for line,
    timestamps character for character, values within 1e-3 of their units."""
    lems, spec, files = _write_from_oracle("izh_net", tmp_path, extended=True)
    z = np.load(os.path.join(HERE, "golden", "loggers.npz"))
    for f in LOGGER_FILES:
        mine = open(os.path.join(str(tmp_path), f)).read().splitlines()
        ref = str(z[os.path.splitext(f)[0]]).splitlines()
        assert len(mine) == len(ref), f
        if f.startswith("ev"):
            assert mine == ref, f
        else:
            assert [l[:16] for l in mine] == [l[:16] for l in ref], f
            a = np.array([[float(x) for x in l.split()] for l in mine])
            b = np.array([[float(x) for x in l.split()] for l in ref])
            np.testing.assert_allclose(a, b, rtol=0, atol=1e-3)
    traces, events = cli.reload_saved_data(lems, reload_events=True)
    assert sum(len(v) for v in events.values()) > 0


def test_logger_sampling_rules():
    times = np.arange(0, 101) * 100.0  # us of steps 0..100 (synthetic: step k at 100 k)
    steps = np.arange(1, 101)          # the step of each recorded row
    of = {"points": None, "start": 1000.0, "end": 3000.0, "interval": 500.0}
    assert [t for t, _ in cli.trajectory_frames(of, times, steps)] == [1000.0, 1500.0, 2000.0, 2500.0]
    of = {"points": [0.0, 250.0, 250.0, 9999.0]}
    assert cli.trajectory_frames(of, times, steps) == [(0.0, 0), (250.0, 2), (250.0, 2), (9999.0, 99)]
    ef = {"start": 0.0, "end": 1000.0, "max_interval": 300.0}
    fr = cli.event_frames(ef, times, 1, 100, {4: [2, 5]})
    assert fr == [(100.0, []), (400.0, [2, 5]), (700.0, [])]
