"""ctypes wrapper of the C restatement (libeden_port.so, and libeden_port64.so:
the same loop in double precision).

Test infrastructure only: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product package.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libeden_port.so")
LIB64 = os.path.join(HERE, "libeden_port64.so")


def build() -> str:
    subprocess.check_call(["make", "-s", "-C", os.path.dirname(HERE), "port"])
    return LIB


_libs = {}


def _load(double=False):
    path = LIB64 if double else LIB
    if path not in _libs:
        if not os.path.exists(path):
            build()
        lib = ctypes.CDLL(path)
        lib.eden_port_run.restype = ctypes.c_int
        _libs[path] = lib
    return _libs[path]


def run(lowered, n_steps=None, trace_target=None, threads=0, spike_cap=None, double=False, mark_step=None):
    """Run the port; returns dict(trace [n_steps, n_trace] f32, spike_src,
    spike_step, syn_fire_count, syn_final_pending, rc).  With `mark_step`,
    also `timed_s`: the wall-clock seconds from the start of that step to
    the end of the run."""
    from eden_gb300.lowering import to_cmodel
    lib = _load(double)
    cm, keep = to_cmodel(lowered)
    if n_steps is None:
        n_steps = lowered.n_steps
    tt = np.ascontiguousarray(lowered.trace_target if trace_target is None else trace_target, np.int32)
    trace = np.zeros((n_steps, max(len(tt), 1)), np.float32)
    if spike_cap is None:
        spike_cap = max(1024, len(lowered.src_target) * max(1, n_steps // 50))
    ssrc = np.zeros(spike_cap, np.int32)
    sstep = np.zeros(spike_cap, np.int64)
    nsp = ctypes.c_int64(0)
    n_syn = len(lowered.syn_target)
    fire = np.zeros(max(n_syn, 1), np.int64)
    pend = np.zeros(max(n_syn, 1), np.float32)
    mark = ctypes.c_int64.in_dll(lib, "eden_port_mark_step")
    mark.value = (1 << 63) - 1 if mark_step is None else int(mark_step)
    rc = lib.eden_port_run(ctypes.byref(cm), ctypes.c_int64(n_steps), ctypes.c_int32(len(tt)),
                           tt.ctypes.data_as(ctypes.c_void_p), trace.ctypes.data_as(ctypes.c_void_p),
                           ctypes.c_int64(spike_cap), ssrc.ctypes.data_as(ctypes.c_void_p),
                           sstep.ctypes.data_as(ctypes.c_void_p), ctypes.byref(nsp),
                           fire.ctypes.data_as(ctypes.c_void_p), pend.ctypes.data_as(ctypes.c_void_p),
                           ctypes.c_int32(threads))
    n = min(nsp.value, spike_cap)
    out = dict(trace=trace[:, :len(tt)], spike_src=ssrc[:n].copy(), spike_step=sstep[:n].copy(),
               syn_fire_count=fire[:n_syn].copy(), syn_final_pending=pend[:n_syn].copy(), rc=rc,
               n_spikes=nsp.value)
    if mark_step is not None:
        out["timed_s"] = ctypes.c_double.in_dll(lib, "eden_port_end_s").value - \
            ctypes.c_double.in_dll(lib, "eden_port_mark_s").value
        mark.value = (1 << 63) - 1
    return out


LIBGPU64 = os.path.join(HERE, "libeden_port_gpu64.so")


def run_gpu64(lowered, n_steps=None, trace_target=None, spike_cap=None, device=0):
    """The same loop in double precision on the GPU (oracle/gpu64): returns
    dict(trace [n_steps, n_trace] float64, spike_src, spike_step, rc)."""
    from eden_gb300.lowering import to_cmodel
    if LIBGPU64 not in _libs:
        if not os.path.exists(LIBGPU64):
            subprocess.check_call(["make", "-s", "-C", os.path.dirname(HERE), "gpu64"])
        lib = ctypes.CDLL(LIBGPU64)
        lib.eden_port_gpu_run.restype = ctypes.c_int
        _libs[LIBGPU64] = lib
    lib = _libs[LIBGPU64]
    cm, keep = to_cmodel(lowered)
    if n_steps is None:
        n_steps = lowered.n_steps
    tt = np.ascontiguousarray(lowered.trace_target if trace_target is None else trace_target, np.int32)
    trace = np.zeros((n_steps, max(len(tt), 1)), np.float64)
    if spike_cap is None:
        spike_cap = max(1024, len(lowered.src_target) * max(1, n_steps // 50))
    ssrc = np.zeros(spike_cap, np.int32)
    sstep = np.zeros(spike_cap, np.int64)
    nsp = ctypes.c_int64(0)
    rc = lib.eden_port_gpu_run(ctypes.byref(cm), ctypes.c_int64(n_steps), ctypes.c_int32(len(tt)),
                               tt.ctypes.data_as(ctypes.c_void_p), trace.ctypes.data_as(ctypes.c_void_p),
                               ctypes.c_int64(spike_cap), ssrc.ctypes.data_as(ctypes.c_void_p),
                               sstep.ctypes.data_as(ctypes.c_void_p), ctypes.byref(nsp), ctypes.c_int32(device))
    n = min(nsp.value, spike_cap)
    return dict(trace=trace[:, :len(tt)], spike_src=ssrc[:n].copy(), spike_step=sstep[:n].copy(), rc=rc,
                n_spikes=nsp.value)
