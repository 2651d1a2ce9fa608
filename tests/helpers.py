"""Shared helpers for the parity tests."""
from collections import defaultdict

import numpy as np


def spike_trains(src, step):
    """dict source -> sorted array of logging steps."""
    d = defaultdict(list)
    for s, k in zip(np.asarray(src), np.asarray(step)):
        d[int(s)].append(int(k))
    return {k: np.sort(np.array(v)) for k, v in d.items()}


def compare_spikes(a_src, a_step, b_src, b_step, max_shift_steps):
    """Returns (n_cells_with_count_mismatch, max |step difference| over cells
    whose counts agree)."""
    a = spike_trains(a_src, a_step)
    b = spike_trains(b_src, b_step)
    bad, worst = 0, 0
    for k in set(a) | set(b):
        x = a.get(k, np.zeros(0, int))
        y = b.get(k, np.zeros(0, int))
        if len(x) != len(y):
            bad += 1
            continue
        if len(x):
            worst = max(worst, int(np.abs(x - y).max()))
    return bad, worst
