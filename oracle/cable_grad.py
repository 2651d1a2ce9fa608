"""Double-precision forward run and forward-mode parameter sensitivities of
multicompartment cells -- test infrastructure for the GPU adjoint
(edenGpuGrad*): imported by tests/ and bench.py's accuracy leg only, never
by the product package.

The step is the reference's, restated in double precision and vectorised
over all compartments:

* gates (eden/Eden.cpp:5126-5259): rates of EXP / EXPLINEAR / SIGMOID form
  (5164-5181) at the old V, exponential Euler towards inf = a/(a+b) with
  factor exp(-dt q10 (a+b)), clamped to [1e-6, 1 - 1e-6]; the four
  initialisation passes (steps <= 0, 3251) set every gate to inf(V0) and
  leave V;
* channel currents with the old gates, i = gbase fopen (E - V) 1e-5 A,
  g = gbase fopen 1e-5 A (5678-5717, 5805-5898); pulse inputs (3798-3826)
  at the double step time (11486, 11931);
* V pre-update d = G/C + sum 1/(RC), x = V + dt (I + V G)/C (6057-6107);
* backward-Euler Hines solve of M V' = x (6114-6225), M = 1 + dt d on the
  diagonal, -dt/(R C_child) in the child's row and -dt/(R C_parent) in the
  parent's row.

* synaptic drive with events fixed in advance (timedSynapticInput inputs
  and connections from spike sources; their firing steps from the listed
  steps and from the reference's single-pending-spike rule,
  oracle/routing.py): each synapse's unit-weight exposure g^(n) -- expTwo
  gbase (B - A), expOne G -- by forward Euler between events and the
  event's jump instead of the decay in its step
  (LEMS_CoreComponents.inc.xml:145-180, eden/Eden.cpp:3424-3466), times its
  weight (3708-3710), adds g (E - V) and g to the compartment's I and G.

A cell's axial resistances scale with its resistivity Ra, so every axial
term is multiplied by s = Ra_lowered / Ra.

Tangents (forward mode) go through the same phases for any set of
directions in parameter space: dq' = dQ/dV dV + dQ/dq dq (0 where the gate
clamped), dg = (dgbase fopen + gbase dfopen) 1e-5 A plus dw g^ for a weight,
dx = dV + dt dGE / C,
dV' = M^-1 (dx - dM V').  The trace is V at the start of steps 1..N of the
recorded compartments; its derivative along a direction is returned per
step, so any loss's directional derivative follows by the chain rule.
"""
from __future__ import annotations

import numpy as np

RATE_EXP, RATE_EXPLINEAR, RATE_SIGMOID = 0, 1, 2


def _rates(kind, r, mid, s, v):
    """Rate value and d(rate)/dV, elementwise (eden/Eden.cpp:5164-5181)."""
    x = (v - mid) / s
    with np.errstate(over="ignore", invalid="ignore", divide="ignore"):
        ex = np.exp(x)
        emx = np.exp(-x)
        em1 = np.expm1(-x)               # e^-x - 1
        # EXPLINEAR r x / (1 - e^-x), r where V == mid; its slope by the
        # Taylor series 1/2 + x/6 - x^3/180 near x = 0
        small = np.abs(x) < 1e-3
        f = np.where(x == 0, 1.0, x / np.where(em1 == 0, 1.0, -em1))
        fp = np.where(small, 0.5 + x / 6.0 - x ** 3 / 180.0,
                      (-em1 - x * (1.0 + em1)) / np.where(em1 == 0, 1.0, em1 * em1))
        fp = np.where(x < -60.0, 0.0, fp)
        val = np.where(kind == RATE_EXP, r * ex,
                       np.where(kind == RATE_SIGMOID, r / (1.0 + emx), r * f))
        dval = np.where(kind == RATE_EXP, val / s,
                        np.where(kind == RATE_SIGMOID, val * (1.0 / (1.0 + 1.0 / emx)) / s, r * fp / s))
    return val, dval


class Cable:
    """The cells of a lowered model (physical cells only), with a parameter
    map: chan_param[ch] / cell_ra_param[c] give the parameter index or -1."""

    def __init__(self, low, chan_param, cell_ra_param=None, cell_ra=None, syn_param=None, timed_param=None):
        if low.n_izh or len(low.pois_target) or len(low.gap_target) or low.cable_solver:
            raise ValueError("physical cells with HH channels, pulse inputs and fixed synaptic drive only, "
                             "backward-Euler cable solve")
        self.low = low
        self.syn_param = np.full(len(low.syn_target), -1) if syn_param is None else np.asarray(syn_param, np.int64)
        self.timed_param = (np.full(len(low.timed_target), -1) if timed_param is None
                            else np.asarray(timed_param, np.int64))
        self.dt = float(low.dt)
        n = low.n_comp
        self.n = n
        off = np.asarray(low.phys_comp_off, np.int64)
        ncell = len(off) - 1
        self.cell_of = np.repeat(np.arange(ncell), np.diff(off))
        lp = np.asarray(low.comp_parent, np.int64)
        parent = np.where(lp >= 0, off[self.cell_of] + lp, -1)
        self.parent = parent
        depth = np.zeros(n, np.int64)
        for i in range(n):                # parents precede children
            if parent[i] >= 0:
                depth[i] = depth[parent[i]] + 1
        order = np.lexsort((np.arange(n), parent, depth))   # by depth, then parent
        self.levels = []                  # per depth >= 1: children (grouped by parent), parents, group starts
        for lvl in range(1, int(depth.max()) + 1 if n else 1):
            nodes = order[depth[order] == lvl]
            par = parent[nodes]
            starts = np.concatenate([[0], np.nonzero(np.diff(par))[0] + 1])
            self.levels.append((nodes, par, par[starts], starts))
        self.roots = np.nonzero(parent < 0)[0]
        f64 = lambda a: np.asarray(a, np.float64)
        self.C, self.A, self.IRC, self.V0 = f64(low.comp_c), f64(low.comp_area), f64(low.comp_inv_rc), f64(low.comp_v0)
        R = f64(low.comp_r_axial)
        dt = self.dt
        pc = np.where(parent >= 0, parent, 0)
        with np.errstate(invalid="ignore", divide="ignore"):
            self.U = np.where(parent >= 0, -dt / (R * self.C), 0.0)
            self.L = np.where(parent >= 0, -dt / (R * self.C[pc]), 0.0)
        # channels and their gates
        self.chan_comp = np.repeat(np.arange(n), np.diff(low.comp_chan_off))
        nch = len(self.chan_comp)
        ct = low.chan_types
        self.chan_param = np.asarray(chan_param if chan_param is not None else np.full(nch, -1), np.int64)
        self.gbase = f64(low.chan_gbase)
        self.erev = f64(low.chan_erev)
        ng_of = ct["n_gates"][low.chan_type]
        self.chan_g0 = np.concatenate([[0], np.cumsum(ng_of)])[:-1]
        self.chan_ng = ng_of
        gate_chan = np.repeat(np.arange(nch), ng_of)
        gate_k = np.arange(len(gate_chan)) - self.chan_g0[gate_chan]
        tt = low.chan_type[gate_chan]
        self.gate_comp = self.chan_comp[gate_chan]
        self.gate_chan = gate_chan
        self.g_inst = ct["gate_instances"][tt, gate_k].astype(np.int64)
        self.fk, self.fr = ct["fwd_kind"][tt, gate_k], f64(ct["fwd_rate"][tt, gate_k])
        self.fm, self.fs = f64(ct["fwd_mid"][tt, gate_k]), f64(ct["fwd_scale"][tt, gate_k])
        self.rk, self.rr = ct["rev_kind"][tt, gate_k], f64(ct["rev_rate"][tt, gate_k])
        self.rm, self.rs = f64(ct["rev_mid"][tt, gate_k]), f64(ct["rev_scale"][tt, gate_k])
        self.q10 = f64(ct["q10"][tt, gate_k])
        self.maxg = int(ng_of.max()) if nch else 0
        # pulses
        self.pt = np.asarray(low.pulse_target, np.int64)
        self.ps, self.pd = f64(low.pulse_start), f64(low.pulse_duration)
        self.paw = f64(low.pulse_amplitude) * f64(low.pulse_weight)
        self.ra_param = np.asarray(cell_ra_param if cell_ra_param is not None else np.full(ncell, -1), np.int64)
        self.cell_ra = f64(cell_ra if cell_ra is not None else np.ones(ncell))

    # -- Hines solve on the depth levels -----------------------------------
    def _factor(self, D, Ue, Le):
        D = D.copy()
        ratios = []
        for nodes, par, upar, starts in reversed(self.levels):
            ratio = Le[nodes] / D[nodes]
            D[upar] -= np.add.reduceat(ratio * Ue[nodes], starts)
            ratios.append(ratio)
        return D, ratios[::-1]

    def _apply(self, D, ratios, Ue, X):
        """Solve with the factored matrix; X is [k, n] and is overwritten."""
        for (nodes, par, upar, starts), ratio in zip(reversed(self.levels), reversed(ratios)):
            X[:, upar] -= np.add.reduceat(ratio * X[:, nodes], starts, axis=1)
        X[:, self.roots] /= D[self.roots]
        for nodes, par, upar, starts in self.levels:
            X[:, nodes] = (X[:, nodes] - Ue[nodes] * X[:, par]) / D[nodes]
        return X

    def _gates(self, v, q):
        al, dal = _rates(self.fk, self.fr, self.fm, self.fs, v)
        be, dbe = _rates(self.rk, self.rr, self.rm, self.rs, v)
        sm = al + be
        inf = al / sm
        b = np.exp(-self.dt * self.q10 * sm)
        qn = b * q + (1.0 - b) * inf
        clamped = ~((qn > 1e-6) & (qn < 1 - 1e-6))
        qn = np.clip(qn, 1e-6, 1 - 1e-6)
        db = -self.dt * self.q10 * (dal + dbe) * b
        dinf = (dal * be - al * dbe) / (sm * sm)
        dqdq = np.where(clamped, 0.0, b)
        dqdv = np.where(clamped, 0.0, db * (q - inf) + (1.0 - b) * dinf)
        return qn, dqdq, dqdv, inf

    def drive(self, n_steps):
        """The synaptic drive over steps 1..n_steps: (compartment, reversal
        potential, weight parameter or -1, fixed weight) per item and its
        unit-weight exposure [n_items, n_steps + 1] (column n = step n)."""
        import routing
        low = self.low
        st = low.syn_types
        items = []
        for k in range(len(low.timed_target)):
            ev = np.asarray(low.timed_step[low.timed_off[k]:low.timed_off[k + 1]], np.int64)
            items.append((int(low.timed_target[k]), int(low.timed_type[k]), int(self.timed_param[k]),
                          float(low.timed_weight[k]), set(ev.tolist())))
        if len(low.syn_target):
            if (np.asarray(low.src_target)[np.asarray(low.syn_src)] >= 0).any():
                raise ValueError("a synapse's presynaptic cell spikes: its events are not fixed")
            _, steps = routing.route_steps(low.syn_src, low.syn_delay, low.ext_src, low.ext_step, float(low.dt),
                                           n_steps)
            for k in range(len(low.syn_target)):
                items.append((int(low.syn_target[k]), int(low.syn_type[k]), int(self.syn_param[k]),
                              float(low.syn_weight[k]), set(steps[k].tolist())))
        ghat = np.zeros((len(items), n_steps + 1))
        meta = []
        dt = self.dt
        for i, (comp, ty, par, w, ev) in enumerate(items):
            two = int(st["kind"][ty]) == 1
            gb, td, tr = float(st["gbase"][ty]), float(st["tau_decay"][ty]), float(st["tau_rise"][ty])
            wf = float(st["weight_prop"][ty]) * float(st["waveform_factor"][ty]) if two else 0.0
            a = b = 0.0
            for n in range(1, n_steps + 1):
                ghat[i, n] = gb * (b - a) if two else a
                if n in ev:
                    a, b = (a + wf, b + wf) if two else (a + gb, b)
                else:
                    a, b = (a - dt * a / tr, b - dt * b / td) if two else (a - dt * a / td, b)
            meta.append((comp, float(st["erev"][ty]), par, w))
        return meta, ghat

    def run(self, params, n_steps, rec_comp, directions=None):
        """trace [N, n_rec] (float64) and, with directions [k, n_params], its
        derivatives [k, N, n_rec] along each direction."""
        params = np.asarray(params, np.float64)
        meta, ghat = self.drive(n_steps)
        d_comp = np.array([x[0] for x in meta], np.int64)
        d_erev = np.array([x[1] for x in meta])
        d_par = np.array([x[2] for x in meta], np.int64)
        d_w = np.where(d_par >= 0, params[np.where(d_par >= 0, d_par, 0)], np.array([x[3] for x in meta]))
        D0 = np.zeros((0, len(params))) if directions is None else np.asarray(directions, np.float64)
        k = D0.shape[0]
        n, dt = self.n, self.dt
        rec = np.asarray(rec_comp, np.int64)
        has_ra = self.ra_param >= 0
        ra = np.where(has_ra, params[np.where(has_ra, self.ra_param, 0)], 1.0)
        s_cell = np.where(has_ra, self.cell_ra / ra, 1.0)
        ds_cell = np.where(has_ra, -s_cell / ra, 0.0)[None, :] * np.where(
            has_ra[None, :], D0[:, np.where(has_ra, self.ra_param, 0)], 0.0)
        s = s_cell[self.cell_of]
        ds = ds_cell[:, self.cell_of]
        has_p = self.chan_param >= 0
        gb = np.where(has_p, params[np.where(has_p, self.chan_param, 0)], self.gbase)
        dgb = np.where(has_p[None, :], D0[:, np.where(has_p, self.chan_param, 0)], 0.0)
        Ue, Le, irc = self.U * s, self.L * s, self.IRC * s
        dUe, dLe, dirc = self.U * ds, self.L * ds, self.IRC * ds
        Achan = self.A[self.chan_comp]
        V = self.V0.copy()
        _, _, _, q = self._gates(V[self.gate_comp], np.zeros(len(self.gate_comp)))
        dV = np.zeros((k, n))
        dq = np.zeros((k, len(q)))
        trace = np.zeros((n_steps, len(rec)))
        dtrace = np.zeros((k, n_steps, len(rec)))
        t = 0.0
        nch = len(self.chan_comp)
        for step in range(1, n_steps + 1):
            trace[step - 1] = V[rec]
            dtrace[:, step - 1] = dV[:, rec]
            if step == n_steps:
                break
            vg = V[self.gate_comp]
            qn, dqdq, dqdv, _ = self._gates(vg, q)
            dqn = dqdq * dq + dqdv * dV[:, self.gate_comp]
            pw = q ** self.g_inst
            dpw = np.where(self.g_inst > 0, self.g_inst * q ** np.maximum(self.g_inst - 1, 0), 0.0) * dq
            fopen = np.ones(nch)
            dfopen = np.zeros((k, nch))
            for g in range(self.maxg):
                m = self.chan_ng > g
                idx = self.chan_g0[m] + g
                dfopen[:, m] = dfopen[:, m] * pw[idx] + fopen[m] * dpw[:, idx]
                fopen[m] = fopen[m] * pw[idx]
            gc = gb * fopen * 1e-5 * Achan
            dgc = (dgb * fopen + gb * dfopen) * 1e-5 * Achan
            G = np.bincount(self.chan_comp, gc, minlength=n)
            GE = np.bincount(self.chan_comp, gc * self.erev, minlength=n)
            dG = np.stack([np.bincount(self.chan_comp, dgc[j], minlength=n) for j in range(k)]) if k else dV
            dGE = np.stack([np.bincount(self.chan_comp, dgc[j] * self.erev, minlength=n) for j in range(k)]) if k else dV
            on = (self.ps <= t) & (t <= self.ps + self.pd)
            Iin = np.bincount(self.pt, np.where(on, self.paw, 0.0), minlength=n)
            if len(meta):
                gs = d_w * ghat[:, step]
                G = G + np.bincount(d_comp, gs, minlength=n)
                GE = GE + np.bincount(d_comp, gs * d_erev, minlength=n)
                if k:
                    dgs = np.where(d_par[None, :] >= 0, D0[:, np.where(d_par >= 0, d_par, 0)], 0.0) * ghat[:, step]
                    dG = dG + np.stack([np.bincount(d_comp, dgs[j], minlength=n) for j in range(k)])
                    dGE = dGE + np.stack([np.bincount(d_comp, dgs[j] * d_erev, minlength=n) for j in range(k)])
            I = GE - G * V + Iin
            d = G / self.C + irc
            x = V + dt * (I + V * G) / self.C
            Dp, ratios = self._factor(1.0 + dt * d, Ue, Le)
            Vn = self._apply(Dp, ratios, Ue, x[None, :].copy())[0]
            if k:
                dd = dG / self.C + dirc
                dx = dV + dt * dGE / self.C
                dMV = dt * dd * Vn[None, :]
                child = self.parent >= 0
                ci = np.nonzero(child)[0]
                pi = self.parent[ci]
                dMV[:, ci] += dUe[:, ci] * Vn[pi]
                np.add.at(dMV.T, pi, (dLe[:, ci] * Vn[ci]).T)
                dV = self._apply(Dp, ratios, Ue, dx - dMV)
            V, q, dq = Vn, qn, dqn
            t += dt
        return trace, dtrace


def loss_and_trace_grad(trace, target):
    """MSE over all samples and its gradient with respect to the trace."""
    diff = trace - target
    return float(np.mean(diff ** 2)), 2.0 * diff / diff.size
