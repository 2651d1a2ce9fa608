"""The reference's own validation networks (its testing/validation_tests),
read by this package's NeuroML reader and run by the oracle, against the
reference simulator's output on the same files.  Runs where the reference
tree and its build (oracle/_ref) are present; skipped elsewhere.  The GPU
path is checked against the oracle by the parity tests on the seeded cases
that cover the same input kinds."""
import os
import shutil
import tempfile

import numpy as np
import pytest

import eden_port
import reference_runner
from criteria import box_violations
from eden_gb300 import lowering, neuroml_io


# (network, its trajectory file, tolerance in mV; gate states within 1 %
# of that in absolute terms).  The spiking networks reach 0.014 mV on the
# upstroke of a spike, where V moves 4-5 mV per step: the reference's kernels
# are compiled with -Ofast.
@pytest.mark.parametrize("name,outfile,tol_mv", [
    ("LEMS_EdenTest_CoreInputs.xml", "results.gen.txt", 0.01),
    ("LEMS_EdenTest_PassiveCompartment.xml", None, 0.01),
    ("LEMS_EdenTest1.xml", "results1.txt", 0.05),   # frustum dendrites, gap junction, synapse, a gate's state
    ("LEMS_EdenTest2.xml", "results1.txt", 0.05),   # HH cell with its m, h and n recorded
    # 14 spiking cells joined by gap junctions and expOne connections over
    # 100 ms: spikes move by a step, so the reference's own criterion,
    # box(0.1 ms, 0.5 mV), is the measure (tol_mv None)
    ("LEMS_EdenTest_DomainDecomposition.xml", "results.gen.txt", None),
    # izhikevichCell populations customised per instance by `set cell` and
    # `set input`, and expOne connections by `set synapse`
    ("EdenTest_Extension_CustomSetup.nml", "results.gen.txt", 0.1),
    # every core synapse on passive cells driven by one HH cell: the chemical
    # ones (expOne, expTwo, expThree, alpha, alphaCurrent, blockingPlastic
    # with its voltage block and Tsodyks-Markram plasticity, the PyNN ones)
    # and the continuous ones (linearGraded, graded, silent, a gap junction)
    ("LEMS_EdenTest_CoreSynapses.xml", "results.gen.txt", 0.05),
])
def test_oracle_matches_the_reference_on_its_validation_network(name, outfile, tol_mv):
    path = reference_runner.validation_network(name)
    if path is None or not reference_runner.available():
        pytest.skip("reference tree or its build not present")
    spec = neuroml_io.read_lems(path)
    low = lowering.lower(spec)
    work = tempfile.mkdtemp(prefix="eden_val_")
    try:
        reference_runner.run(path, threads=2, keep_dir=work)
        files = [outfile] if outfile else [f for f in os.listdir(work) if f.endswith(".txt") and "spike" not in f
                                           and f not in os.listdir(os.path.dirname(path))]
        ref = np.loadtxt(os.path.join(work, files[0]), ndmin=2)
    finally:
        shutil.rmtree(work, ignore_errors=True)
    out = eden_port.run(low)
    assert out["rc"] == 0
    mine = out["trace"].astype(np.float64)
    # engine units: mV for potentials, gate states as they are
    scale = np.array([c[3] for of in spec.output_files for c in of["cols"]], np.float64)
    ref_eng = ref[:, 1:] / scale
    assert mine.shape == ref_eng.shape
    if tol_mv is None:
        nbad, worst = box_violations(ref_eng, mine, float(low.dt) * 1e-3, 0.1, 0.5)
        assert nbad == 0, f"{nbad} samples outside box(0.1 ms, 0.5 mV), worst {worst} mV"
        return
    tol = np.where(scale == 1.0, tol_mv * 1e-2, tol_mv)
    assert (np.abs(mine - ref_eng) <= tol).all(), np.abs(mine - ref_eng).max(0)


# The reference's half_vs_half criteria for EdenTest_Extension_CustomSetup.nml
# (testing/validation_tests/validation_tests.py:31-42), as pairs of output
# columns whose traces must be identical: each customised instance of pop0
# against the uncustomised cell it reproduces, and the two connections of
# ToPopp_ExpWild customised into copies of ToPopp_ExpSlow and ToPopp_ExpFast.
CUSTOM_SETUP_PAIRS = [(5, 0), (6, 1), (7, 2), (8, 3), (9, 4), (10, 12), (11, 13)]


def test_custom_setup_network_halves_are_identical_on_the_oracle():
    path = reference_runner.validation_network("EdenTest_Extension_CustomSetup.nml")
    if path is None:
        pytest.skip("reference tree not present")
    spec = neuroml_io.read_lems(path)
    low = lowering.lower(spec)
    assert len(spec.synapses) == 3 and len(low.syn_types) == 5
    tr = eden_port.run(low)["trace"]
    for a, b in CUSTOM_SETUP_PAIRS:
        np.testing.assert_array_equal(tr[:, a], tr[:, b])
    # the customisation is what makes them equal
    import copy
    plain = copy.copy(spec)
    plain.custom_setup = []
    tr0 = eden_port.run(lowering.lower(plain))["trace"]
    assert all(np.abs(tr0[:, a] - tr0[:, b]).max() > 1.0 for a, b in CUSTOM_SETUP_PAIRS)
