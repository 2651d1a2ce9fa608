"""Per-synapse routing fixtures from the reference simulator's own tables.

Runs the reference EDEN built from its sources (oracle/_ref/eden) with its
`verbose full_dump` options (eden/Eden.cpp:10513-10517) on the
`routing_probe` networks -- spike lists driving izhikevich2007 cells through
expOne synapses -- and reads, from the raw state tables it prints after every
step (eden/Eden.cpp:11894-11922), each synapse's pending spike time
("Next Spike", the single pending slot of eden/Eden.cpp:3646-3686) and the
steps in which it fires (its relative conductance jumps instead of
decaying, eden/Eden.cpp:3449-3462).  The cell type's table signature
(printed by `verbose`, eden/Eden.cpp:6972-6982) names each table; each
izhikevich cell's tables follow in work-item order.  The reference's
synapse order on a cell is matched to the lowered model's through the
weight and delay tables it prints at set-up.

Writes tests/golden/routing_<variant>.npz: for each synapse (lowered order)
the pending slot after every step as float32 bits (changes only:
pend_step, pend_syn, pend_bits) and its firing steps (fire_step, fire_syn).

    python tests/golden/make_routing_golden.py
"""
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import reference_runner  # noqa: E402
from eden_gb300 import lowering, neuroml_io, workloads  # noqa: E402

# variant -> routing_probe keyword arguments: delays from one step up (the
# windowed path then runs one-step windows), from half a step up (spikes
# firing in the step that reads their trigger), and from five steps up
# (five-step windows whose triggers are replayed at the next window)
VARIANTS = {
    "k1": dict(min_delay_ms=0.1),
    "sub_step": dict(min_delay_ms=0.05, seed=99),
    "k5": dict(min_delay_ms=0.5, seed=7),
}
LENGTH_MS = 30.0


def _tables(lines, i):
    """Table rows of a raw dump section starting after line i: each row's
    values (strings); ends at the first line that is not a table row."""
    rows = []
    while i < len(lines):
        parts = lines[i].split("\t")
        if len(parts) < 2 or not parts[1].strip().startswith(("0x", "(nil)")):
            break
        rows.append([p.strip() for p in parts[2:] if p.strip()])
        i += 1
    return rows, i


def parse(stdout):
    lines = stdout.splitlines()
    # table signatures, one block per cell type; the synapses' is the one
    # that has a "Next Spike" table
    blocks, sig = [], None
    for ln in lines:
        if ln.strip() == "Tables:":
            sig = {}
            blocks.append(sig)
            continue
        m = re.match(r"\s*(CF32|SF32|SI64|CI64)\s+(\d+):\s+(.*)$", ln)
        if m and sig is not None:
            sig.setdefault(m.group(1), {})[m.group(3).strip()] = int(m.group(2))
    sig = next(b for b in blocks if any(k.endswith("Next Spike") for k in b.get("SF32", {})))
    const, steps, now_g, next_f32 = None, [], [], []
    i = 0
    while i < len(lines):
        ln = lines[i]
        if ln.startswith("TabConstF32:"):
            const, i = _tables(lines, i + 1)
            continue
        m = re.match(r"State: t = (\S+) us(, initialization step (-?\d+))?", ln)
        if m:
            steps.append(int(m.group(3)) if m.group(2) else None)
        if ln.startswith("RawStateF32:"):
            rows, i = _tables(lines, i + 1)
            now_g.append(rows)
            continue
        if ln.startswith("RawStateNextF32:"):
            rows, i = _tables(lines, i + 1)
            next_f32.append(rows)
            continue
        i += 1
    # number the non-initialisation steps 1, 2, ...
    k = 0
    for j, s in enumerate(steps):
        if s is None:
            k += 1
            steps[j] = k
    return sig, const, steps, now_g, next_f32


def make(variant):
    spec = workloads.routing_probe(length_ms=LENGTH_MS, **VARIANTS[variant])
    low = lowering.lower(spec)
    with tempfile.TemporaryDirectory() as d:
        lems = neuroml_io.write_lems(spec, d)
        out = reference_runner.run(lems, threads=1, extra=("verbose", "full_dump"))
    sig, const, steps, now_f32, next_f32 = parse(out["stdout"])
    s_next = next(v for k, v in sig["SF32"].items() if k.endswith("Next Spike"))
    s_g = next(v for k, v in sig["SF32"].items() if k.endswith("Relative Conductance"))
    c_w = next(v for k, v in sig["CF32"].items() if k.endswith("Weight"))
    c_d = next(v for k, v in sig["CF32"].items() if k.endswith("Delay"))
    n_sf32, n_cf32 = len(sig["SF32"]), len(sig["CF32"])
    n_src = sum(1 for c in low.src_target if c < 0)
    n_post = low.n_izh
    # const tables: one spike-time list per source, then n_cf32 per cell;
    # state tables: the null table, then n_sf32 per cell
    order = []
    for k in range(n_post):
        w_ref = np.array(const[n_src + n_cf32 * k + c_w], np.float64)
        d_ref = np.array(const[n_src + n_cf32 * k + c_d], np.float64)
        mine = np.flatnonzero(low.syn_target == low.n_comp + k)
        w_my = np.asarray(low.syn_weight)[mine].astype(np.float64)
        d_my = np.asarray(low.syn_delay)[mine].astype(np.float64)
        if len(mine) != len(w_ref) or not (np.allclose(w_my, w_ref, rtol=1e-4) and np.allclose(d_my, d_ref, rtol=1e-5)):
            raise RuntimeError(f"cell {k}: synapse order of the reference does not match the lowered model")
        order.append(mine)
    n_syn = len(low.syn_target)
    pend_prev = np.full(n_syn, -np.inf, np.float32)
    g_prev = np.zeros(n_syn)
    ps, pn, pb, fs, fn = [], [], [], [], []
    for j, step in enumerate(steps):
        if step <= 0:
            continue
        for k in range(n_post):
            syn = order[k]
            pend = np.array([np.float32(float(x)) for x in next_f32[j][1 + n_sf32 * k + s_next]], np.float32)
            g_now = np.array(now_f32[j][1 + n_sf32 * k + s_g], np.float64)
            g_next = np.array(next_f32[j][1 + n_sf32 * k + s_g], np.float64)
            fired = g_next > g_now
            for q in np.flatnonzero(fired):
                fs.append(step); fn.append(syn[q])
            ch = pend.view(np.uint32) != pend_prev[syn].view(np.uint32)
            for q in np.flatnonzero(ch):
                ps.append(step); pn.append(syn[q]); pb.append(pend.view(np.uint32)[q])
            pend_prev[syn] = pend
    last = max(s for s in steps if s is not None)
    np.savez_compressed(os.path.join(HERE, f"routing_{variant}.npz"), last_step=last,
                        pend_step=np.array(ps, np.int32), pend_syn=np.array(pn, np.int32),
                        pend_bits=np.array(pb, np.uint32), fire_step=np.array(fs, np.int32),
                        fire_syn=np.array(fn, np.int32))
    print(f"routing_{variant}: {n_syn} synapses, {last} steps, {len(ps)} pending changes, {len(fs)} firings")


if __name__ == "__main__":
    if not reference_runner.available():
        sys.exit("oracle/_ref/eden is not built (make -C oracle ref)")
    for v in sys.argv[1:] or list(VARIANTS):
        make(v)
