"""GPU path vs the oracle (the C restatement of the reference loop) on the
same seeded inputs, through the C ABI, in both execution modes.

Tolerances (the reference validation harness's own criteria, restated in
tests/criteria.py): spike trains samecount with every spike within 0.1 ms;
membrane potential inside box(0.1 ms, 0.5 mV) of the oracle's trace.  The
two differ only by single-precision rounding (CUDA's expf/logf against
glibc's, and the order of the synaptic current sums), which can move a spike
by one 25 us step; the recurrent multicompartment case is chaotic, so it is
compared over its first 15 ms only."""
import numpy as np
import pytest

import eden_port
from eden_gb300 import lowering, workloads
from eden_gb300.engine import MODE_BATCHED, MODE_PLAIN, Simulation
from criteria import box_violations, samecount
from golden.cases import CASES, spec_of
from golden_io import load, logged
from helpers import spike_trains

pytestmark = pytest.mark.gpu



# networks checked against the oracle only (no reference fixtures): HH
# channels and synapses on dendrites, so that non-flat compartments sit
# inside the trees with flat ones above and below them; the mixed
# point-neuron / multicompartment network; and large cells whose trees are
# wider than a warp at some depth
EXTRA = {
    "multicomp_active_dendrites": lambda: workloads.multicomp_net(
        n_cells=24, in_degree=20, length_ms=40.0, max_seg=80, n_recorded=6, hh_dend_frac=0.2,
        syn_on_dendrites=True),
    "mixed_small": lambda: workloads.mixed_scale(n_izh=400, n_mc=100, in_degree=20, length_ms=30.0, n_seg=30),
    # cells of up to 500 compartments, one with 83 compartments at one depth
    "multicomp_large_cells": lambda: workloads.multicomp_net(n_cells=12, in_degree=20, length_ms=30.0, max_seg=500,
                                                             n_recorded=6),
}


def _spec(name):
    return EXTRA[name]() if name in EXTRA else spec_of(name)


@pytest.fixture(scope="module")
def oracle_runs():
    cache = {}

    def get(name):
        if name not in cache:
            low = lowering.lower(_spec(name))
            cache[name] = (low, eden_port.run(low))
        return cache[name]
    return get


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_BATCHED], ids=["plain", "batched"])
@pytest.mark.parametrize("name", list(CASES) + list(EXTRA))
def test_gpu_matches_oracle(name, mode, oracle_runs):
    low, ref = oracle_runs(name)
    sim = Simulation(low, mode=mode)
    rec = sim.run()
    sim.close()
    assert rec.trace.shape == ref["trace"].shape
    dt_ms = float(low.dt) * 1e-3
    shift = int(round(0.1 / dt_ms))
    wrong, far = samecount(spike_trains(ref["spike_src"], ref["spike_step"]),
                           spike_trains(rec.spike_src, rec.spike_step), shift)
    assert not wrong, f"spike counts differ for cells {wrong[:10]}"
    assert not far, f"spikes more than 0.1 ms apart for cells {far[:10]}"
    assert np.isfinite(rec.trace).all()
    assert len(ref["spike_src"]) > 0
    if rec.trace.shape[1]:
        nbad, worst = box_violations(ref["trace"], rec.trace, dt_ms, 0.1, 0.5)
        assert nbad == 0, f"{nbad} samples outside box(0.1 ms, 0.5 mV), worst by {worst} mV"


@pytest.mark.parametrize("name", list(CASES))
def test_gpu_matches_reference_outputs(name, oracle_runs):
    """The GPU path against the reference simulator's own fixture outputs."""
    low, _ = oracle_runs(name)
    ref_trace, ref_src, ref_step = load(name, low)
    sim = Simulation(low, mode=MODE_BATCHED)
    rec = sim.run()
    sim.close()
    dt_ms = float(low.dt) * 1e-3
    wrong, far = samecount(spike_trains(ref_src, ref_step), spike_trains(*logged(rec.spike_src, rec.spike_step, low)),
                           int(round(0.1 / dt_ms)))
    assert not wrong and not far, f"spike trains differ: counts {wrong[:5]}, timing {far[:5]}"
    nbad, worst = box_violations(ref_trace, rec.trace, dt_ms, 0.1, CASES[name][2])
    assert nbad == 0, f"{nbad} samples outside box, worst {worst} mV"


@pytest.mark.parametrize("blocks", [1, 3])
def test_blocks_running_several_ctas_in_turn(blocks):
    """With fewer cell-kernel blocks than CTAs (networks of more than 32
    CTAs per SM, forced here on a small one), every block runs several CTAs
    one after another in its shared memory; the records equal those of one
    CTA per block bit for bit."""
    low = lowering.lower(EXTRA["mixed_small"]())
    out = []
    for cap in (0, blocks):
        sim = Simulation(low, mode=MODE_BATCHED, max_cell_blocks=cap)
        try:
            out.append(sim.run())
        finally:
            sim.close()
    a, b = out
    assert len(a.spike_src) > 0
    np.testing.assert_array_equal(a.trace, b.trace)
    np.testing.assert_array_equal(a.spike_src, b.spike_src)
    np.testing.assert_array_equal(a.spike_step, b.spike_step)


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_BATCHED], ids=["plain", "batched"])
def test_gate_state_columns(mode):
    """Trace columns of gate states (the OutputColumn path
    .../membraneProperties/<channelDensity>/<ionChannel>/<gate>/q) beside
    potentials, on HH somata and HH dendrite compartments inside forests:
    the GPU's columns against the oracle's, potentials within box(0.1 ms,
    0.5 mV) and gate states within box(0.1 ms, 0.005)."""
    from eden_gb300.network import OutputColumn
    spec = workloads.multicomp_net(n_cells=8, in_degree=10, length_ms=30.0, max_seg=40, n_recorded=4,
                                   hh_dend_frac=0.3)
    cols = []
    for c in range(4):
        ct = spec.cell_type(spec.populations[c].cell_type)
        segs = [0] + [int(s) for s in np.nonzero(ct.densities[1].seg_mask)[0] if s > 0][:1]
        for seg in segs:
            cols.append(OutputColumn(spec.populations[c].name, 0, seg))
            for k, gname in ((1, "m"), (1, "h"), (2, "n")):
                cols.append(OutputColumn(spec.populations[c].name, 0, seg, f"q:cd{k}/{gname}"))
    spec.trace_columns = cols
    low = lowering.lower(spec)
    assert (low.trace_target <= -2).sum() == 3 * (len(cols) // 4)
    ref = eden_port.run(low)
    sim = Simulation(low, mode=mode)
    rec = sim.run()
    sim.close()
    dt_ms = float(low.dt) * 1e-3
    is_q = np.array([c.quantity != "v" for c in cols])
    assert rec.trace.shape == ref["trace"].shape
    assert np.all((rec.trace[:, is_q] > 0) & (rec.trace[:, is_q] < 1))
    nbad, worst = box_violations(ref["trace"][:, ~is_q], rec.trace[:, ~is_q], dt_ms, 0.1, 0.5)
    assert nbad == 0, f"potentials: {nbad} samples outside the box, worst {worst} mV"
    nbad, worst = box_violations(ref["trace"][:, is_q], rec.trace[:, is_q], dt_ms, 0.1, 0.005)
    assert nbad == 0, f"gate states: {nbad} samples outside the box, worst {worst}"
