"""Loading the reference's golden outputs in the oracle's terms."""
import os

import numpy as np

from eden_gb300.lowering import POINT_FN

HERE = os.path.dirname(os.path.abspath(__file__))


def load(name, lowered):
    """Returns (trace_mV [samples, columns], spike_src, spike_log_step)."""
    z = np.load(os.path.join(HERE, "golden", f"{name}.npz"))
    # volts to mV, except dimensionless columns (a fitzHughNagumoCell's V)
    scale = np.full(len(lowered.trace_target), 1e3)
    for j, t in enumerate(lowered.trace_target):
        k = int(t) - lowered.n_comp
        if k >= 0 and len(lowered.izh_kind) > k and int(lowered.izh_kind[k]) == POINT_FN:
            scale[j] = 1.0
    trace = z["values_si"].astype(np.float64) * scale
    dt_s = float(lowered.dt) * 1e-6
    ids = z["event_id"]
    src = lowered.event_src[ids] if len(ids) else np.zeros(0, np.int32)
    # an event stamped t_n was emitted in step n and is logged at step n + 1
    step = np.rint(z["event_time_s"] / dt_s).astype(np.int64) + 1
    return trace, src, step


def logged(src, step, lowered):
    """The spikes of the sources the reference's event file records (an
    event-set reader's events are delivered as spikes of its sources, which
    the reference does not log)."""
    keep = np.isin(np.asarray(src), lowered.event_src)
    return np.asarray(src)[keep], np.asarray(step)[keep]


class RoutingFixture:
    """A synapse-by-synapse record of the reference's routing
    (tests/golden/routing_<variant>.npz): the pending slot of every synapse
    after each step (stored as its changes) and the steps each fired in."""

    def __init__(self, z, n_syn):
        self.n_syn = n_syn
        self.last_step = int(z["last_step"])
        self.pend_step, self.pend_syn, self.pend_bits = z["pend_step"], z["pend_syn"], z["pend_bits"]
        self.fire_step, self.fire_syn = z["fire_step"], z["fire_syn"]

    def pending_after(self, step):
        """float32 pending slot of every synapse after step `step`."""
        bits = np.full(self.n_syn, np.float32(-np.inf)).view(np.uint32)
        keep = self.pend_step <= step
        bits[self.pend_syn[keep]] = self.pend_bits[keep]  # changes are in step order
        return bits.view(np.float32)

    def fire_count_through(self, step):
        keep = self.fire_step <= step
        return np.bincount(self.fire_syn[keep], minlength=self.n_syn).astype(np.int64)


def routing_fixture(variant, n_syn):
    return RoutingFixture(np.load(os.path.join(HERE, "golden", f"routing_{variant}.npz")), n_syn)
