"""Comparison criteria of the reference's validation harness, restated
(testing/validation_tests/eden_tools/validation.py:7-87):

box(dt_box, dv_box): the test trace must stay inside the truth's running
maximum/minimum over a window of int(dt_box/dt)+1 samples, widened by dv_box;
samecount(dt_box): same number of spikes, each within dt_box of the truth's.
"""
import numpy as np
from scipy.ndimage import maximum_filter1d, minimum_filter1d


def box_violations(truth, test, dt, dt_box, dv_box):
    """Number of samples of `test` outside the box around `truth` (per column
    along axis 0) and the worst excursion beyond it."""
    truth = np.asarray(truth, np.float64)
    test = np.asarray(test, np.float64)
    width = int(dt_box / dt + 1e-9) + 1
    hi = maximum_filter1d(truth, width, axis=0, mode="nearest") + dv_box
    lo = minimum_filter1d(truth, width, axis=0, mode="nearest") - dv_box
    over = np.maximum(test - hi, 0.0)
    under = np.maximum(lo - test, 0.0)
    bad = (over > 0) | (under > 0) | np.isnan(test) | np.isnan(truth)
    return int(bad.sum()), float(max(over.max(initial=0), under.max(initial=0)))


def box_violations_strided(truth, test_rows, stride, dt, dt_box, dv_box):
    """box() for a test trace kept every `stride`-th sample (rows 0, stride,
    2 stride, ...): the box is built on the full-rate truth and read at those
    rows."""
    truth = np.asarray(truth, np.float64)
    test = np.asarray(test_rows, np.float64)
    width = int(dt_box / dt + 1e-9) + 1
    hi = (maximum_filter1d(truth, width, axis=0, mode="nearest") + dv_box)[::stride][:len(test)]
    lo = (minimum_filter1d(truth, width, axis=0, mode="nearest") - dv_box)[::stride][:len(test)]
    test = test[:len(hi)]
    over = np.maximum(test - hi, 0.0)
    under = np.maximum(lo - test, 0.0)
    bad = (over > 0) | (under > 0) | np.isnan(test) | np.isnan(hi)
    return int(bad.sum()), float(max(over.max(initial=0), under.max(initial=0)))


def samecount(truth_steps_by_src, test_steps_by_src, max_shift_steps):
    """Cells whose spike counts differ, and cells with a spike more than
    max_shift_steps away from the truth's."""
    wrong_count, too_far = [], []
    for k in set(truth_steps_by_src) | set(test_steps_by_src):
        a = np.asarray(truth_steps_by_src.get(k, []))
        b = np.asarray(test_steps_by_src.get(k, []))
        if len(a) != len(b):
            wrong_count.append(k)
        elif len(a) and np.abs(a - b).max() > max_shift_steps:
            too_far.append(k)
    return wrong_count, too_far
