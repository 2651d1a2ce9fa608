"""Gate kinds beyond gateHHrates (gateHHtauInf, gateHHratesTau,
gateHHratesInf, gateHHratesTauInf), q10Settings and the network temperature:
host side.  The oracle's gate loop is pinned against the reference by the
gate_kinds golden case (tests/test_oracle_vs_reference.py) and the GPU path
against both by the parity tests."""
import numpy as np
import pytest

from eden_gb300 import lowering, neuroml_io, workloads
from eden_gb300.network import RATE_SIGMOID, Gate, Rate


def test_gate_kinds_and_q10_are_lowered():
    spec = workloads.gate_kinds()
    ct = lowering.lower(spec).chan_types
    names = [c.name for c in spec.channels]
    na, kdr, ka = names.index("naT"), names.index("kdr"), names.index("kA")
    assert list(ct["gate_kind"][na][:2]) == [lowering.GATE_KINDS["ratesInf"], lowering.GATE_KINDS["tauInf"]]
    assert ct["gate_kind"][kdr][0] == lowering.GATE_KINDS["ratesTau"]
    assert list(ct["gate_kind"][ka][:2]) == [lowering.GATE_KINDS["ratesTauInf"], lowering.GATE_KINDS["rates"]]
    # fixedTimeCourse in us, steady state dimensionless
    assert ct["tau_kind"][na][1] == lowering.RATE_FIXED and ct["tau_rate"][na][1] == np.float32(3000.0)
    assert ct["inf_kind"][na][1] == RATE_SIGMOID and ct["inf_mid"][na][1] == np.float32(-62.0)
    # q10ExpTemp 3 from 6.3 degC at 16.3 degC; q10Fixed 1.5
    assert abs(float(ct["q10"][na][0]) - 3.0) < 1e-5
    assert ct["q10"][kdr][0] == np.float32(1.5)


def test_q10_defaults():
    gate = Gate("x", 1, Rate(0, 1.0, 0.0, 1.0), Rate(0, 1.0, 0.0, 1.0))
    assert lowering.gate_q10(gate, 30.0) == np.float32(1.0)
    gate.q10 = ("exp", 2.0, 6.3)
    assert lowering.gate_q10(gate, 6.3) == np.float32(1.0)
    assert abs(float(lowering.gate_q10(gate, 26.3)) - 4.0) < 1e-5


def test_round_trip_keeps_gate_kinds_and_temperature(tmp_path):
    spec = workloads.gate_kinds()
    back = neuroml_io.read_lems(neuroml_io.write_lems(spec, str(tmp_path)))
    assert back.temperature == pytest.approx(16.3)
    a, b = lowering.lower(spec).chan_types, lowering.lower(back).chan_types
    for f in a.dtype.names:
        np.testing.assert_array_equal(a[f], b[f], err_msg=f)


def test_incomplete_gate_is_refused():
    spec = workloads.gate_kinds()
    spec.channels[1].gates[1].tau = None          # a tauInf gate without its timeCourse
    with pytest.raises(ValueError, match="timeCourse"):
        lowering.lower(spec)


@pytest.mark.parametrize("old,new", [
    ('<timeCourse type="fixedTimeCourse" tau="3.0ms"/>', '<timeCourse type="myTau" tau="3.0ms"/>'),
    ('<gateHHtauInf id="h"', '<gateKS id="h"'),
])
def test_unsupported_gate_forms_are_refused(tmp_path, old, new):
    lems = neuroml_io.write_lems(workloads.gate_kinds(), str(tmp_path))
    nml = tmp_path / "gate_kinds.nml"
    text = nml.read_text()
    assert old in text
    text = text.replace(old, new)
    if "gateKS" in new:
        text = text.replace("</gateHHtauInf>", "</gateKS>")
    nml.write_text(text)
    with pytest.raises(ValueError):
        neuroml_io.read_lems(lems)
