"""Regenerate the golden fixtures from the reference simulator.

Writes each case of cases.py as LEMS/NeuroML, runs the reference EDEN built
from its own sources (oracle/_ref/eden, see oracle/Makefile) in a scratch
directory, and stores its OutputFile trajectory and EventOutputFile spikes in
tests/golden/<case>.npz.  Needs the reference source tree (to build the
oracle binary); the fixtures it writes are what the tests read.

    python tests/golden/make_golden.py [case ...]
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, HERE)

import reference_runner  # noqa: E402
from cases import CASES, FULL_CASES, LOGGER_FILES, add_eden_loggers, spec_of  # noqa: E402
from eden_gb300 import neuroml_io  # noqa: E402


def make(name):
    spec = spec_of(name)
    stride = FULL_CASES[name][2] if name in FULL_CASES else 1
    with tempfile.TemporaryDirectory() as d:
        lems = neuroml_io.write_lems(spec, d)
        extra = () if spec.cable_solver == "auto" else ("cable_solver", spec.cable_solver)
        out = reference_runner.run(lems, threads=8, extra=extra)
    traj = out["trajectory"].astype(np.float64)[::stride]
    ev = np.array(out.get("events", []), dtype=np.float64).reshape(-1, 2)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), time_s=traj[:, 0], values_si=traj[:, 1:].astype(np.float32),
                        event_time_s=ev[:, 0], event_id=ev[:, 1].astype(np.int32), trace_stride=stride,
                        trajectory_head=out["trajectory_text"].splitlines()[:3],
                        events_head=out.get("events_text", "").splitlines()[:3])
    print(f"{name}: {traj.shape[0]} samples x {traj.shape[1] - 1} columns, {len(ev)} spikes")


def make_loggers():
    """The izh_net case with EDEN's extended loggers (cases.add_eden_loggers)."""
    with tempfile.TemporaryDirectory() as d:
        lems = neuroml_io.write_lems(spec_of("izh_net"), d)
        add_eden_loggers(lems)
        keep = os.path.join(d, "run")
        os.makedirs(keep)
        reference_runner.run(lems, threads=4, keep_dir=keep)
        texts = {os.path.splitext(f)[0]: open(os.path.join(keep, f)).read() for f in LOGGER_FILES}
    np.savez_compressed(os.path.join(HERE, "loggers.npz"), **texts)
    print("loggers:", {k: len(v.splitlines()) for k, v in texts.items()})


if __name__ == "__main__":
    if not reference_runner.available():
        sys.exit("oracle/_ref/eden is not built (make -C oracle ref)")
    names = sys.argv[1:] or list(CASES) + list(FULL_CASES) + ["loggers"]
    for name in names:
        make_loggers() if name == "loggers" else make(name)
