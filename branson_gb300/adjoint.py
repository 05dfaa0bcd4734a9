"""Adjoint of one transport step: dL/dsigma_a per cell for L = sum_c w_c
E_abs[c], through the C ABI pair bgs_adjoint_forward / bgs_adjoint_backward.

``Tape`` is the saved context of one forward (the step's photon start
states and cell coefficients, on the device); ``AdjointStep`` runs forwards
(optionally with photon counts frozen from an earlier forward, so perturbed
runs share photons and random streams) and backwards.  ``absorbed_energy``
wraps the pair as a ``torch.autograd.Function`` for harness use: its
forward maps a CPU float64 tensor of per-cell sigma_a to the absorbed-energy
tally, its backward maps dL/dE_abs to dL/dsigma_a.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib
from ._lib import BransonError
from .engine import ReplicatedIMC


class Tape:
    """Saved context of one adjoint forward (device memory, freed on close)."""

    def __init__(self, lib, handle: C.c_void_p, n_cells: int):
        self.lib = lib
        self.handle = handle
        self.n_cells = n_cells

    def counts(self) -> np.ndarray:
        out = np.empty(3 * self.n_cells, np.uint32)
        rc = self.lib.bgs_adjoint_counts(self.handle, _lib.ptr(out))
        if rc != 0:
            raise BransonError(rc, "bgs_adjoint_counts")
        return out

    def info(self) -> dict:
        inf = _lib.AdjointInfo()
        rc = self.lib.bgs_adjoint_get_info(self.handle, C.byref(inf))
        if rc != 0:
            raise BransonError(rc, "bgs_adjoint_get_info")
        return {k: getattr(inf, k) for k, _ in _lib.AdjointInfo._fields_ if k != "reserved"}

    def close(self) -> None:
        if self.handle:
            self.lib.bgs_adjoint_release(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def step_forward(imc: ReplicatedIMC, sigma_a: Optional[np.ndarray] = None, counts: Optional[np.ndarray] = None,
                 tape: Optional[Tape] = None, save: bool = True, algorithm: int = _lib.HISTORY):
    """bgs_adjoint_forward on any context: one step's sourcing and transport
    at the context's current step number, the context left at that step;
    returns (abs_E, tape) -- tape is None when save is False."""
    n = imc.n_cells
    sig = None if sigma_a is None else np.ascontiguousarray(sigma_a, dtype=np.float64)
    if sig is not None and sig.shape != (n,):
        raise ValueError("one sigma_a per cell")
    cnt = None if counts is None else np.ascontiguousarray(counts, dtype=np.uint32)
    if cnt is not None and cnt.shape != (3 * n,):
        raise ValueError("3*n_cells photon counts (emission | source | initial census)")
    nd = imc.next_dt()
    if nd <= 0.0:
        nd = imc.dt
    p = _lib.StepParams(imc.step_no, algorithm, imc.dt, nd)
    abs_E = np.empty(n)
    h = C.c_void_p(tape.handle.value if tape is not None and tape.handle else None) if save else None
    rc = imc.lib.bgs_adjoint_forward(imc.ctx, C.byref(p), _lib.ptr(sig), _lib.ptr(cnt), _lib.ptr(abs_E),
                                     C.byref(h) if save else None)
    imc._check(rc, "bgs_adjoint_forward")
    if not save:
        return abs_E, None
    if tape is None:
        tape = Tape(imc.lib, h, n)
    else:
        tape.handle = h
    return abs_E, tape


class AdjointStep(ReplicatedIMC):
    """A replicated IMC context whose current step can be run as a
    differentiable function sigma_a -> E_abs."""

    def forward(self, sigma_a: Optional[np.ndarray] = None, counts: Optional[np.ndarray] = None,
                tape: Optional[Tape] = None, save: bool = True, algorithm: int = _lib.HISTORY):
        """One step's sourcing and transport at the current step number; returns
        (abs_E, tape) -- tape is None when save is False."""
        return step_forward(self, sigma_a, counts, tape, save, algorithm)

    def backward(self, tape: Tape, grad_abs_E: np.ndarray) -> np.ndarray:
        w = np.ascontiguousarray(grad_abs_E, dtype=np.float64)
        if w.shape != (self.n_cells,):
            raise ValueError("one dL/dE_abs per cell")
        out = np.empty(self.n_cells)
        self._check(self.lib.bgs_adjoint_backward(self.ctx, tape.handle, _lib.ptr(w), _lib.ptr(out)),
                    "bgs_adjoint_backward")
        return out


def absorbed_energy(step: AdjointStep, sigma_a, counts: Optional[np.ndarray] = None):
    """E_abs(sigma_a) as a torch autograd node (CPU float64 tensors)."""
    import torch

    class _AbsorbedEnergy(torch.autograd.Function):
        @staticmethod
        def forward(ctx, sig):
            abs_E, tape = step.forward(sig.detach().cpu().numpy(), counts=counts)
            ctx.tape = tape
            return torch.from_numpy(abs_E)

        @staticmethod
        def backward(ctx, grad_out):
            g = step.backward(ctx.tape, grad_out.detach().cpu().numpy())
            return torch.from_numpy(g)

    return _AbsorbedEnergy.apply(sigma_a)


def batch_forward(batch, sigma_a=None, counts=None, tapes=None):
    """bgs_batch_adjoint_forward: the adjoint forward of every problem of a
    BatchIMC at its current step.  sigma_a / counts: None or one entry per
    problem (each None or an array).  Returns (abs_E list, tape list)."""
    probs = batch.problems
    n = len(probs)
    params = (_lib.StepParams * n)()
    for i, p in enumerate(probs):
        nd = p.next_dt()
        params[i] = _lib.StepParams(p.step_no, _lib.HISTORY, p.dt, nd if nd > 0.0 else p.dt)
    keep = []

    def ptr_array(items, dtype):
        if items is None:
            return None
        arr = (C.c_void_p * n)()
        for i, a in enumerate(items):
            if a is not None:
                a = np.ascontiguousarray(a, dtype=dtype)
                keep.append(a)
                arr[i] = a.ctypes.data
        return arr

    sig = ptr_array(sigma_a, np.float64)
    cnt = ptr_array(counts, np.uint32)
    abs_out = [np.empty(p.n_cells) for p in probs]
    abs_ptrs = (C.c_void_p * n)(*[a.ctypes.data for a in abs_out])
    handles = (C.c_void_p * n)()
    if tapes is not None:
        for i, t in enumerate(tapes):
            handles[i] = t.handle.value if t is not None and t.handle else None
    batch._check(batch.lib.bgs_batch_adjoint_forward(batch.handle, params, sig, cnt, abs_ptrs, handles),
                 "bgs_batch_adjoint_forward")
    out_tapes = []
    for i, p in enumerate(probs):
        h = C.c_void_p(handles[i])
        if tapes is not None and tapes[i] is not None:
            tapes[i].handle = h
            out_tapes.append(tapes[i])
        else:
            out_tapes.append(Tape(batch.lib, h, p.n_cells))
    return abs_out, out_tapes


def batch_backward(batch, tapes, grads):
    """bgs_batch_adjoint_backward: every problem's dL/dsigma_a from its tape
    and dL/dE_abs, in one replay launch."""
    probs = batch.problems
    n = len(probs)
    w = [np.ascontiguousarray(g, dtype=np.float64) for g in grads]
    out = [np.empty(p.n_cells) for p in probs]
    handles = (C.c_void_p * n)(*[t.handle.value for t in tapes])
    w_ptrs = (C.c_void_p * n)(*[a.ctypes.data for a in w])
    o_ptrs = (C.c_void_p * n)(*[a.ctypes.data for a in out])
    batch._check(batch.lib.bgs_batch_adjoint_backward(batch.handle, handles, w_ptrs, o_ptrs),
                 "bgs_batch_adjoint_backward")
    return out
