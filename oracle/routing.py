"""Synaptic event routing restated from the reference -- test infrastructure.

Given the spike log of a run (spike source, logging step) and each connection
synapse's source and delay, this replays the reference's delivery and
single-pending-spike rule independently of any simulator:

* a threshold crossing in step n sets the trigger of every synapse on the
  source's fan-out for the next step (eden/Eden.cpp:3946-3995, the atomic OR
  into the next-step trigger table at 3988); the spike is logged at step
  n + 1, the step that reads the trigger (the logging phase runs on the
  "now" state at the start of a step, 11555-11635);
* the synapse reading a trigger at time t (eden/Eden.cpp:3646-3686): the
  spike fires now if t <= t + delay < t + dt; it becomes the single pending
  spike only if the pending one is already due (pend < t + dt) and earlier
  than it (pend < t + delay); a pending spike fires in the one step whose
  interval [t, t + dt) holds it.  The pending slot starts at -inf
  (eden/Eden.cpp:9081-9094).

Times are the reference's: step k >= 1 runs at the double sum of k - 1 float
dts (11486, 11931), used as a float; t + delay and t + dt are float sums.
"""
from collections import defaultdict

import numpy as np

F32 = np.float32


def step_times(dt_us: float, last_step: int) -> np.ndarray:
    """float32 time (us) of steps 0..last_step (steps <= 0 run at t = 0)."""
    n = max(int(last_step), 1)
    acc = np.concatenate([[0.0], np.add.accumulate(np.full(n - 1, float(F32(dt_us))))])
    return np.concatenate([[0.0], acc]).astype(F32)


def route(syn_src, syn_delay, spike_src, spike_step, dt_us, last_step):
    """Pending slot of every synapse after all triggers read at steps
    <= last_step, and how many steps each synapse fired in (steps 1..last_step).

    Returns (pending float32 [n_syn], fire_count int64 [n_syn])."""
    pend, steps = route_steps(syn_src, syn_delay, spike_src, spike_step, dt_us, last_step)
    return pend, np.array([len(x) for x in steps], np.int64)


def route_steps(syn_src, syn_delay, spike_src, spike_step, dt_us, last_step):
    """route(), with each synapse's firing steps (sorted) in place of the
    count: returns (pending float32 [n_syn], list of int64 arrays)."""
    syn_src = np.asarray(syn_src)
    syn_delay = np.asarray(syn_delay, F32)
    times = step_times(dt_us, last_step + 1)
    dt = F32(dt_us)
    by_src = defaultdict(list)
    order = np.argsort(np.asarray(spike_step), kind="stable")
    for i in order:
        k = int(spike_step[i])
        if 1 <= k <= last_step:
            by_src[int(spike_src[i])].append(k)
    n = len(syn_src)
    pend = np.full(n, -np.inf, F32)
    steps_of = [np.zeros(0, np.int64) for _ in range(n)]
    t_end = times[1:last_step + 1]           # times of steps 1..last_step
    t_end_dt = (t_end + dt).astype(F32)

    def due_step(p):
        # the step k in 1..last_step with t_k <= p < t_k + dt (first such)
        j = int(np.searchsorted(t_end, p, side="right")) - 1
        for jj in (j - 1, j):
            if 0 <= jj < len(t_end) and t_end[jj] <= p < t_end_dt[jj]:
                return jj + 1
        return None

    for s in range(n):
        steps = by_src.get(int(syn_src[s]))
        if not steps:
            continue
        d = syn_delay[s]
        p = F32(-np.inf)
        fired = set()
        for k in steps:
            t = times[k]
            fresh = F32(t + d)
            tdt = F32(t + dt)
            if t <= fresh < tdt:
                fired.add(k)
            if p < tdt and p < fresh:
                p = fresh
                ks = due_step(p)
                if ks is not None:
                    fired.add(ks)
        pend[s] = p
        steps_of[s] = np.array(sorted(k for k in fired if k <= last_step), np.int64)
    return pend, steps_of


def route_pending(syn_src, syn_delay, spike_src, spike_step, dt_us, last_step):
    """The pending slot of every synapse after all triggers read at steps
    <= last_step, as route() computes it, vectorised over each spike's
    fan-out (in step order; spikes of one step reach disjoint synapses) so
    that it runs at full network sizes."""
    syn_src = np.asarray(syn_src)
    syn_delay = np.asarray(syn_delay, F32)
    n_src = int(syn_src.max()) + 1 if len(syn_src) else 0
    order = np.argsort(syn_src, kind="stable")
    fan0 = np.zeros(n_src + 1, np.int64)
    np.add.at(fan0, syn_src + 1, 1)
    fan0 = np.cumsum(fan0)
    times = step_times(dt_us, last_step + 1)
    dt = F32(dt_us)
    pend = np.full(len(syn_src), -np.inf, F32)
    spike_src = np.asarray(spike_src)
    spike_step = np.asarray(spike_step)
    keep = (spike_step >= 1) & (spike_step <= last_step) & (spike_src < n_src)
    for k, s in sorted(zip(spike_step[keep].tolist(), spike_src[keep].tolist())):
        syn = order[fan0[s]:fan0[s + 1]]
        t = times[k]
        fresh = (t + syn_delay[syn]).astype(F32)
        p = pend[syn]
        pend[syn] = np.where((p < F32(t + dt)) & (p < fresh), fresh, p)
    return pend
