"""Run the reference EDEN simulator (oracle/_ref/eden, built from the
reference sources by oracle/Makefile) on a LEMS file and parse its outputs.

Test infrastructure only.  Used to generate golden fixtures in this
container; the reference tree does not exist where the GPU tests run.
"""
import os
import re
import shutil
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
EDEN = os.path.join(HERE, "_ref", "eden")


def available() -> bool:
    return os.path.exists(EDEN)


def reference_tree():
    """The reference source tree: EDEN_REFERENCE_DIR, else the tree
    oracle/_ref was built from (oracle/Makefile records it), else None."""
    env = os.environ.get("EDEN_REFERENCE_DIR")
    if env:
        return env
    src = os.path.join(HERE, "_ref", "SOURCE")
    if os.path.exists(src):
        return open(src).read().strip() or None
    return None


def validation_network(name: str):
    """Path of one of the reference's own validation networks
    (testing/validation_tests/neuroml/<name>), or None without the tree."""
    ref = reference_tree()
    if ref is None:
        return None
    p = os.path.join(ref, "testing", "validation_tests", "neuroml", name)
    return p if os.path.exists(p) else None


def run(lems_path: str, threads: int = 1, extra=(), keep_dir=None):
    """Returns dict(trajectory=[n, 1+cols] float64 (time s, values SI),
    events=list of (time s, id), run_s=float, stdout=str)."""
    src_dir = os.path.dirname(os.path.abspath(lems_path))
    work = keep_dir or tempfile.mkdtemp(prefix="eden_ref_")
    for f in os.listdir(src_dir):
        if f.endswith(".nml") or f.endswith(".xml") or f.endswith(".txt"):
            shutil.copy(os.path.join(src_dir, f), work)
    env = dict(os.environ, OMP_NUM_THREADS=str(threads), OMP_SCHEDULE="static")
    p = subprocess.run([EDEN, "nml", os.path.basename(lems_path), "gcc", *extra], cwd=work,
                       env=env, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"reference failed ({p.returncode}):\n{p.stdout[-3000:]}\n{p.stderr[-2000:]}")
    m = re.search(r"Run:\s*([0-9.eE+-]+)", p.stdout)
    out = dict(run_s=float(m.group(1)) if m else float("nan"), stdout=p.stdout, dir=work)
    traj = os.path.join(work, "trajectory.txt")
    if os.path.exists(traj):
        out["trajectory"] = np.loadtxt(traj, ndmin=2)
        out["trajectory_text"] = open(traj).read()
    spk = os.path.join(work, "spikes.txt")
    if os.path.exists(spk):
        ev = []
        text = open(spk).read()
        for line in text.splitlines():
            parts = line.split()
            if len(parts) == 2:
                ev.append((float(parts[0]), int(parts[1])))
        out["events"] = ev
        out["events_text"] = text
    if keep_dir is None:
        shutil.rmtree(work, ignore_errors=True)
    return out
