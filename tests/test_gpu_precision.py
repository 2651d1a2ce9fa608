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
