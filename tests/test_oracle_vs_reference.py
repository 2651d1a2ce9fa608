"""The oracle (C restatement of the reference loop, oracle/port) against the
reference simulator's own outputs on the same seeded networks (fixtures in
tests/golden/, produced by tests/golden/make_golden.py from the reference
built from its sources).

Criteria: the reference harness's samecount (every spike within 0.1 ms) and
box(0.1 ms, 1 mV) (testing/validation_tests/eden_tools/validation.py:7-87,
restated in tests/criteria.py).  The reference compiles its kernels with
-Ofast, so the two agree to rounding, not bit for bit."""
import numpy as np
import pytest

import eden_port
from criteria import box_violations, box_violations_strided, samecount
from eden_gb300 import lowering
from golden.cases import CASES, FULL_CASES, spec_of
from golden_io import load, logged
from helpers import spike_trains


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_matches_reference(name):
    low = lowering.lower(spec_of(name))
    ref_trace, ref_src, ref_step = load(name, low)
    out = eden_port.run(low)
    assert out["rc"] == 0
    assert out["trace"].shape == ref_trace.shape
    dt_ms = float(low.dt) * 1e-3
    wrong, far = samecount(spike_trains(ref_src, ref_step), spike_trains(*logged(out["spike_src"], out["spike_step"], low)),
                           int(round(0.1 / dt_ms)))
    assert not wrong, f"spike counts differ for cells {wrong[:10]}"
    assert not far, f"spikes more than 0.1 ms apart for cells {far[:10]}"
    nbad, worst = box_violations(ref_trace, out["trace"], dt_ms, 0.1, CASES[name][2])
    assert nbad == 0, f"{nbad} samples outside box(0.1 ms, {CASES[name][2]} mV), worst {worst} mV"


def test_golden_fixtures_are_nontrivial():
    for name in CASES:
        low = lowering.lower(spec_of(name))
        _, src, _ = load(name, low)
        assert len(src) > 0, f"{name}: no spikes in the reference output"


@pytest.mark.parametrize("name", list(FULL_CASES))
def test_oracle_matches_reference_at_configuration_size(name):
    """C1 as stated (1,000 cells, 1 s) and C3 with 10,000 cells and 1 M
    synapses over 100 ms: every spike within 0.1 ms of the reference's, and
    the reference's trajectory (stored every `stride`-th sample) inside
    box(0.1 ms, 0.5 mV) of the oracle's."""
    low = lowering.lower(spec_of(name))
    ref_trace, ref_src, ref_step = load(name, low)
    out = eden_port.run(low, spike_cap=1 << 22)
    assert out["rc"] == 0
    dt_ms = float(low.dt) * 1e-3
    wrong, far = samecount(spike_trains(ref_src, ref_step), spike_trains(out["spike_src"], out["spike_step"]),
                           int(round(0.1 / dt_ms)))
    assert not wrong and not far, f"spike trains differ: counts {wrong[:5]}, timing {far[:5]}"
    assert len(ref_src) > 50000
    nbad, worst = box_violations_strided(out["trace"], ref_trace, FULL_CASES[name][2], dt_ms, 0.1, 0.5)
    assert nbad == 0, f"{nbad} samples outside box(0.1 ms, 0.5 mV), worst {worst} mV"
