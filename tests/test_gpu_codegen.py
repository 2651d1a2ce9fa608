"""Kernels compiled at creation for the model's channel sets (NVRTC) against
the built-in kernels: the generated routines perform the same operations, so
spike trains are identical and trajectories agree to rounding."""
import numpy as np
import pytest

from eden_gb300 import lowering
from eden_gb300.engine import MODE_BATCHED, Simulation
from golden.cases import spec_of

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["multicomp_poisson", "ball_and_stick", "izh_net", "input_kinds", "gate_kinds",
                                  "voltage_clamps"])
def test_generated_kernels_match_builtin(name):
    low = lowering.lower(spec_of(name))
    builtin = Simulation(low, mode=MODE_BATCHED, codegen=-1)
    ra = builtin.run()
    assert builtin.generated_source() == ""
    builtin.close()
    gen = Simulation(low, mode=MODE_BATCHED, codegen=1)
    rb = gen.run()
    src = gen.generated_source()
    gen.close()
    assert "k_cells_t" in src and "rtc_channels" in src
    if low.n_comp:
        assert "case 0:" in src
    np.testing.assert_array_equal(ra.spike_src, rb.spike_src)
    np.testing.assert_array_equal(ra.spike_step, rb.spike_step)
    np.testing.assert_allclose(rb.trace, ra.trace, rtol=0, atol=1e-3)
