"""Gradients of recorded membrane potentials through libeden_gpu's adjoint
kernels (include/eden_gpu.h, edenGpuGrad*), and their torch.autograd form.

`CableGradient` owns one gradient context for a lowered model of
independent physical cells (HH channels, pulse inputs) and a map from model
quantities to parameters: channel conductivities (mS/cm2) and cell axial
resistivities (ohm cm).  `forward(params)` returns the recorded trace
[n_steps, n_rec] (V at the start of steps 1..n_steps, mV);
`backward(trace_grad)` returns d(loss)/d(params) given d(loss)/d(trace), by
the discrete adjoint of the step with checkpointed recomputation.

`CableGradient.apply(params)` is the same as a differentiable torch
function of the parameter tensor:

    g = CableGradient(low, param_map)
    trace = g.apply(params)              # params: torch tensor, requires_grad
    loss = ((trace - target) ** 2).mean()
    loss.backward()                      # params.grad from the adjoint kernel

The reference has no gradient path; the step it differentiates is the
reference's (eden/Eden.cpp:5126-5259, 5805-5898, 6057-6107, 6114-6225).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from .engine import EdenGpuError, load_library
from .lowering import LoweredModel, to_cmodel


class CGradSpec(ctypes.Structure):
    _fields_ = [("n_params", ctypes.c_int32), ("chan_param", ctypes.c_void_p),
                ("cell_ra_param", ctypes.c_void_p), ("cell_ra", ctypes.c_void_p),
                ("n_rec", ctypes.c_int32), ("rec_comp", ctypes.c_void_p), ("n_steps", ctypes.c_int64),
                ("checkpoint_every", ctypes.c_int32), ("device", ctypes.c_int32),
                ("syn_param", ctypes.c_void_p), ("timed_param", ctypes.c_void_p),
                ("reserved", ctypes.c_int32 * 4)]


def _bind(lib):
    if getattr(lib, "_grad_bound", False):
        return lib
    P = ctypes.c_void_p
    lib.edenGpuGradCreate.argtypes = [P, P, ctypes.POINTER(P)]
    lib.edenGpuGradCreate.restype = ctypes.c_int
    lib.edenGpuGradForward.argtypes = [P, P, P]
    lib.edenGpuGradForward.restype = ctypes.c_int
    lib.edenGpuGradBackward.argtypes = [P, P, P]
    lib.edenGpuGradBackward.restype = ctypes.c_int
    lib.edenGpuGradTiming.argtypes = [P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    lib.edenGpuGradTiming.restype = ctypes.c_int
    lib.edenGpuGradLastError.argtypes = [P]
    lib.edenGpuGradLastError.restype = ctypes.c_char_p
    lib.edenGpuGradDestroy.argtypes = [P]
    lib.edenGpuGradDestroy.restype = None
    lib._grad_bound = True
    return lib


@dataclass
class ParamMap:
    """Which model quantities are parameters: chan_param[ch] (or -1) for each
    channel instance of the lowered model, cell_ra_param[c] (or -1) for each
    physical cell, syn_param[s] / timed_param[i] (or -1) for each connection
    synapse and timed input (its weight), and the parameter values the model
    was lowered with."""
    n_params: int
    chan_param: np.ndarray
    cell_ra_param: np.ndarray
    values: np.ndarray
    syn_param: np.ndarray | None = None
    timed_param: np.ndarray | None = None


def with_weights(low: LoweredModel, pmap: ParamMap, synapses: bool = True, timed: bool = True) -> ParamMap:
    """pmap extended by one parameter per connection synapse and per timed
    input (their weights), numbered after pmap's."""
    n = pmap.n_params
    syn = np.full(len(low.syn_target), -1, np.int32)
    tim = np.full(len(low.timed_target), -1, np.int32)
    vals = [pmap.values]
    if synapses and len(syn):
        syn[:] = n + np.arange(len(syn))
        n += len(syn)
        vals.append(np.asarray(low.syn_weight, np.float32))
    if timed and len(tim):
        tim[:] = n + np.arange(len(tim))
        n += len(tim)
        vals.append(np.asarray(low.timed_weight, np.float32))
    return ParamMap(n, pmap.chan_param, pmap.cell_ra_param, np.concatenate(vals).astype(np.float32), syn, tim)


def per_cell_density_map(low: LoweredModel, densities: list[int], ra: bool = True) -> ParamMap:
    """Parameters per physical cell: the conductivity of each listed
    channelDensity (by its index in the cell type's list) and, with ra, the
    cell's axial resistivity.  Cell c's parameters are c * k .. c * k + k - 1
    (k = len(densities) + ra), in that order."""
    if low.chan_density is None or low.phys_ra is None:
        raise ValueError("lowered model lacks channel density indices")
    k = len(densities) + (1 if ra else 0)
    n_cells = low.n_phys
    chan_param = np.full(len(low.chan_type), -1, np.int32)
    values = np.zeros(n_cells * k, np.float32)
    cell_of_comp = np.repeat(np.arange(n_cells), np.diff(low.phys_comp_off))
    chan_comp = np.repeat(np.arange(low.n_comp), np.diff(low.comp_chan_off))
    slot_of = {d: j for j, d in enumerate(densities)}
    for ch in range(len(chan_param)):
        j = slot_of.get(int(low.chan_density[ch]))
        if j is not None:
            c = int(cell_of_comp[chan_comp[ch]])
            chan_param[ch] = c * k + j
            values[c * k + j] = low.chan_gbase[ch]
    cell_ra_param = np.full(n_cells, -1, np.int32)
    if ra:
        cell_ra_param[:] = np.arange(n_cells) * k + k - 1
        values[cell_ra_param] = low.phys_ra.astype(np.float32)
    return ParamMap(n_cells * k, chan_param, cell_ra_param, values)


class CableGradient:
    """One gradient context (edenGpuGradCreate) on one GPU."""

    def __init__(self, low: LoweredModel, pmap: ParamMap, rec_comp=None, n_steps: int | None = None,
                 checkpoint_every: int = 100, device: int = 0):
        self.lib = _bind(load_library())
        self.low = low
        self.pmap = pmap
        self.rec_comp = np.ascontiguousarray(low.trace_target if rec_comp is None else rec_comp, np.int32)
        self.n_steps = int(low.n_steps if n_steps is None else n_steps)
        self.n_rec = len(self.rec_comp)
        self.device = device
        cm, self._keep = to_cmodel(low)
        self._chan = np.ascontiguousarray(pmap.chan_param, np.int32)
        self._rap = np.ascontiguousarray(pmap.cell_ra_param, np.int32)
        self._ra = np.ascontiguousarray(low.phys_ra, np.float32)
        self._sp = None if pmap.syn_param is None else np.ascontiguousarray(pmap.syn_param, np.int32)
        self._tp = None if pmap.timed_param is None else np.ascontiguousarray(pmap.timed_param, np.int32)
        spec = CGradSpec(n_params=pmap.n_params, chan_param=self._chan.ctypes.data,
                         cell_ra_param=self._rap.ctypes.data, cell_ra=self._ra.ctypes.data,
                         n_rec=self.n_rec, rec_comp=self.rec_comp.ctypes.data, n_steps=self.n_steps,
                         checkpoint_every=checkpoint_every, device=device,
                         syn_param=None if self._sp is None or not len(self._sp) else self._sp.ctypes.data,
                         timed_param=None if self._tp is None or not len(self._tp) else self._tp.ctypes.data)
        h = ctypes.c_void_p()
        rc = self.lib.edenGpuGradCreate(ctypes.byref(cm), ctypes.byref(spec), ctypes.byref(h))
        self.h = h
        if rc != 0:
            msg = self._err()
            self.close()
            raise EdenGpuError(rc, msg)

    def _err(self) -> str:
        m = self.lib.edenGpuGradLastError(self.h)
        return m.decode() if m else ""

    def _check(self, rc: int):
        if rc != 0:
            raise EdenGpuError(rc, self._err())

    def forward_ptr(self, params_ptr: int, trace_ptr: int):
        """edenGpuGradForward on raw pointers (host or device)."""
        self._check(self.lib.edenGpuGradForward(self.h, ctypes.c_void_p(params_ptr), ctypes.c_void_p(trace_ptr)))

    def backward_ptr(self, trace_grad_ptr: int, grad_ptr: int):
        self._check(self.lib.edenGpuGradBackward(self.h, ctypes.c_void_p(trace_grad_ptr), ctypes.c_void_p(grad_ptr)))

    def forward(self, params) -> np.ndarray:
        p = np.ascontiguousarray(params, np.float32)
        trace = np.zeros((self.n_steps, max(self.n_rec, 1)), np.float32)
        self.forward_ptr(p.ctypes.data, trace.ctypes.data)
        return trace[:, :self.n_rec]

    def backward(self, trace_grad) -> np.ndarray:
        tg = np.ascontiguousarray(trace_grad, np.float32).reshape(self.n_steps, self.n_rec)
        grad = np.zeros(max(self.pmap.n_params, 1), np.float32)
        self.backward_ptr(tg.ctypes.data, grad.ctypes.data)
        return grad[:self.pmap.n_params]

    def timing(self) -> tuple[float, float]:
        """Device ms of the last forward and backward."""
        f, b = ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.edenGpuGradTiming(self.h, ctypes.byref(f), ctypes.byref(b)))
        return f.value, b.value

    def apply(self, params):
        """The trace as a differentiable function of a torch parameter tensor."""
        return _trace_function()(params, self)

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.lib.edenGpuGradDestroy(self.h)
        self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_TraceFn = None


def _trace_function():
    """torch.autograd.Function over CableGradient (built on first use so that
    the module imports without torch)."""
    global _TraceFn
    if _TraceFn is not None:
        return _TraceFn
    import torch

    class TraceFn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, params, g: CableGradient):
            p = params.detach().to(torch.float32).contiguous()
            trace = torch.empty((g.n_steps, max(g.n_rec, 1)), dtype=torch.float32, device=p.device)
            if p.is_cuda:
                torch.cuda.current_stream(p.device).synchronize()
            g.forward_ptr(p.data_ptr(), trace.data_ptr())
            ctx.g = g
            ctx.dtype = params.dtype
            return trace[:, :g.n_rec]

        @staticmethod
        def backward(ctx, grad_trace):
            g = ctx.g
            tg = grad_trace.detach().to(torch.float32).contiguous()
            grad = torch.empty(max(g.pmap.n_params, 1), dtype=torch.float32, device=tg.device)
            if tg.is_cuda:
                torch.cuda.current_stream(tg.device).synchronize()
            g.backward_ptr(tg.data_ptr(), grad.data_ptr())
            return grad[:g.pmap.n_params].to(ctx.dtype), None

    _TraceFn = TraceFn.apply
    return _TraceFn
