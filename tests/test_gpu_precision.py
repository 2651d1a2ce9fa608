"""The GPU path (single precision) against the double-precision oracle on
the golden networks, in both modes: equal spike counts and every spike
within 0.1 ms -- the spike-time error the batched path is measured at."""
import numpy as np
import pytest

import eden_port
from eden_gb300 import lowering
from eden_gb300.engine import MODE_BATCHED, MODE_PLAIN, Simulation
from golden.cases import CASES, spec_of
from helpers import compare_spikes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_BATCHED], ids=["plain", "batched"])
@pytest.mark.parametrize("name", list(CASES))
def test_gpu_within_stated_error_of_double(name, mode):
    low = lowering.lower(spec_of(name))
    f64 = eden_port.run(low, double=True)
    sim = Simulation(low, mode=mode)
    rec = sim.run()
    sim.close()
    shift = int(round(0.1 / (float(low.dt) * 1e-3)))
    bad, worst = compare_spikes(f64["spike_src"], f64["spike_step"], rec.spike_src, rec.spike_step, shift)
    assert bad == 0, f"{bad} cells with a different spike count"
    assert worst <= shift, f"a spike {worst} steps from the double-precision one"


@pytest.mark.parametrize("name", list(CASES))
def test_gpu_double_oracle_matches_host_double_oracle(name):
    """The FP64 GPU oracle (the C restatement built for the GPU in double
    precision) against the same restatement on the host: the same spikes at
    the same steps, and traces equal to double rounding (the two differ only
    in exp/log and the order of the spike log, which is sorted)."""
    low = lowering.lower(spec_of(name))
    host = eden_port.run(low, double=True)
    gpu = eden_port.run_gpu64(low)
    assert gpu["rc"] == 0
    np.testing.assert_array_equal(gpu["spike_src"], host["spike_src"])
    np.testing.assert_array_equal(gpu["spike_step"], host["spike_step"])
    # the host build returns its double trace rounded to float
    np.testing.assert_allclose(gpu["trace"], host["trace"], rtol=0, atol=1e-4)


def test_full_length_multicomp_against_gpu_double_oracle():
    """The batched path over a whole 200 ms run of a recurrent multicompartment
    network against the FP64 GPU oracle: until the first spike-time
    difference appears, the runs agree spike for spike; afterwards the
    recurrent network decorrelates (a one-step shift changes its inputs), so
    over the whole run only the population statistics are compared: total
    spike count within 2 % and per-cell rates correlated above 0.9."""
    from eden_gb300 import workloads
    low = lowering.lower(workloads.multicomp_net(n_cells=300, in_degree=50, length_ms=200.0))
    f64 = eden_port.run_gpu64(low)
    sim = Simulation(low, mode=MODE_BATCHED)
    rec = sim.run()
    sim.close()
    assert f64["rc"] == 0 and len(f64["spike_src"]) > 100
    n = len(low.src_target)
    ca = np.bincount(f64["spike_src"], minlength=n).astype(float)
    cb = np.bincount(rec.spike_src, minlength=n).astype(float)
    assert abs(cb.sum() - ca.sum()) <= 0.02 * ca.sum()
    assert np.corrcoef(ca, cb)[0, 1] > 0.9
    # the first 10 ms spike for spike
    shift = int(round(0.1 / (float(low.dt) * 1e-3)))
    k = int(round(10.0 / (float(low.dt) * 1e-3)))
    fa, fb = f64["spike_step"] <= k, rec.spike_step <= k
    bad, worst = compare_spikes(f64["spike_src"][fa], f64["spike_step"][fa], rec.spike_src[fb], rec.spike_step[fb],
                                shift)
    assert bad == 0 and worst <= shift


# Interpolated crossing times: the FP32 oracle's differ from the FP64
# oracle's by at most 1.3 us on these cases; the GPU's are held to 5 us.
CROSSING_ATOL_US = 5.0


def _fp64_crossings(low, trace, srcs):
    """(source, logging step) -> crossing time (us) from the FP64 trace of
    each source's compartment, interpolated linearly within the step."""
    dt = float(low.dt)
    out = {}
    for j, s in enumerate(srcs):
        v = trace[:, j].astype(np.float64)
        th = float(low.src_threshold[s])
        n = np.flatnonzero((v[:-1] < th) & (th < v[1:]))  # trace row n is the start of step n + 1
        t = n * dt + dt * (th - v[n]) / (v[n + 1] - v[n])
        for k, tc in zip(n, t):
            out[(int(s), int(k) + 2)] = tc
    return out


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_BATCHED], ids=["plain", "batched"])
@pytest.mark.parametrize("name", ["single_comp_hh", "multicomp_poisson", "ball_and_stick", "gate_kinds",
                                  "spike_sources"])
def test_interpolated_crossing_times_against_double(name, mode):
    """Each spike of a physical cell carries its threshold-crossing time,
    interpolated in double between the step's starting and final potential;
    it lies within CROSSING_ATOL_US of the same interpolation on the FP64
    oracle's trace, inside its logged step.  Point neurons and sources with
    no membrane carry NaN."""
    low = lowering.lower(spec_of(name))
    srcs = np.flatnonzero((low.src_target >= 0) & (low.src_target < low.n_comp))
    f64 = eden_port.run(low, trace_target=low.src_target[srcs].astype(np.int32), double=True)
    ref = _fp64_crossings(low, f64["trace"], srcs)
    sim = Simulation(low, mode=mode)
    rec = sim.run()
    sim.close()
    phys = np.isin(rec.spike_src, srcs)
    assert np.isnan(rec.spike_time[~phys]).all()
    assert np.isfinite(rec.spike_time[phys]).all() and phys.any()
    dt = float(low.dt)
    matched = 0
    for s, k, tc in zip(rec.spike_src[phys], rec.spike_step[phys], rec.spike_time[phys]):
        # inside the step that crossed (logged one step later)
        assert (k - 2) * dt - 1e-6 <= tc <= (k - 1) * dt + 1e-6
        if (int(s), int(k)) in ref:
            assert abs(tc - ref[(int(s), int(k))]) <= CROSSING_ATOL_US
            matched += 1
    assert matched >= 0.9 * phys.sum()


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_BATCHED], ids=["plain", "batched"])
def test_cells_that_can_lose_diagonal_dominance_are_solved_in_double(mode):
    """Negative weights on the synapses onto six cells' somas make their
    membrane conductance able to go negative, and with it a cable-matrix
    row's diagonal dominance: edenGpuCreate flags exactly those six cells,
    eliminates their matrices in double precision, and the network stays
    within the parity tolerances of the FP64 oracle: samecount(0.1 ms) and
    box(0.1 ms, 0.5 mV) on every soma over the recurrent network's first
    15 ms."""
    from criteria import box_violations
    from eden_gb300 import workloads
    low = lowering.lower(workloads.multicomp_net(n_cells=24, in_degree=20, length_ms=15.0, max_seg=80))
    neg = np.isin(low.syn_target, low.phys_comp_off[:6])
    low.syn_weight = np.where(neg, -0.5 * low.syn_weight, low.syn_weight).astype(np.float32)
    somas = np.ascontiguousarray(low.phys_comp_off[:-1], np.int32)
    f64 = eden_port.run(low, trace_target=somas, double=True)
    sim = Simulation(low, mode=mode, trace_target=somas)
    try:
        assert sim.fp64_cells() == 6
        rec = sim.run()
    finally:
        sim.close()
    shift = int(round(0.1 / (float(low.dt) * 1e-3)))
    bad, worst = compare_spikes(f64["spike_src"], f64["spike_step"], rec.spike_src, rec.spike_step, shift)
    assert bad == 0 and worst <= shift
    assert len(rec.spike_src) > 0
    nbad, w = box_violations(f64["trace"], rec.trace, float(low.dt) * 1e-3, 0.1, 0.5)
    assert nbad == 0, f"{nbad} samples outside box(0.1 ms, 0.5 mV), worst {w} mV"


def test_no_cell_is_flagged_without_negative_conductances():
    from eden_gb300 import workloads
    low = lowering.lower(workloads.multicomp_net(n_cells=12, in_degree=10, length_ms=1.0, max_seg=40))
    sim = Simulation(low)
    try:
        assert sim.fp64_cells() == 0
    finally:
        sim.close()
