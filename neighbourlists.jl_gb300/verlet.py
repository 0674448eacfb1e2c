"""Verlet-skin reuse of a neighbour list across MD steps (no counterpart in
the reference, which rebuilds every call).

The list is built with cutoff + skin and kept, with the positions it was
built from, on the device.  At every later step the largest displacement
since the build is measured on the device (one 8-byte read back); while it is
at most skin / 2 no pair can have come closer than the cutoff without being
in the list, so the pairs are kept and only R = (X[j] - X[i]) + C'S is
recomputed for the new positions, with the reference's arithmetic.  Beyond
that the list is rebuilt.  Pairs in the list may be up to cutoff + skin apart:
callers that need the exact cutoff compare |R| with it.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from ._lib import check, lib
from .api import _ptr, _stream_handle, pair_vectors
from .engine import NeighbourListEngine

__all__ = ["VerletList"]


class VerletList:
    def __init__(self, nat: int, cell, cutoff: float, skin: float, pbc, int_type=torch.int32, half: bool = False,
                 device="cuda", dtype=torch.float64):
        """dtype=torch.float32: Float32 positions (list, R and the skin test
        in single precision, the reference with T = Float32)."""
        if not skin > 0:
            raise ValueError("skin must be positive")
        self.cutoff, self.skin = float(cutoff), float(skin)
        self.engine = NeighbourListEngine(nat, cell, self.cutoff + self.skin, pbc, int_type=int_type,
                                          device=device, half=half, dtype=dtype)
        self.f32 = dtype == torch.float32
        self.X_ref = None
        self._d2 = torch.zeros(1, dtype=dtype, device=self.engine.device)
        self.rebuilds = 0
        self.reuses = 0

    def max_displacement(self, X: torch.Tensor, stream=None) -> float:
        """Largest displacement since the build, measured on ``stream`` (default:
        the current stream) and read back on that same stream."""
        st = stream if stream is not None else torch.cuda.current_stream(self.engine.device)
        disp = lib().nl_max_displacement_sq_f32 if self.f32 else lib().nl_max_displacement_sq
        check(disp(_ptr(X), _ptr(self.X_ref), int(X.shape[0]), _ptr(self._d2), _stream_handle(st)))
        with torch.cuda.stream(st):
            d2 = float(self._d2.item())
        return d2 ** 0.5

    def update(self, X: torch.Tensor, stream=None) -> bool:
        """Brings the list to positions X; returns True if it was rebuilt."""
        X = X.contiguous()
        d = self.max_displacement(X, stream) if self.X_ref is not None else float("inf")
        if not d <= 0.5 * self.skin:  # also NaN
            self.engine.run(X, stream)
            self.X_ref = X.clone()
            self.rebuilds += 1
            return True
        P = self.engine.total_pairs()
        if P and self.engine.R is not None:
            pair_vectors(X, self.engine.cell, self.engine.i[:P], self.engine.j[:P], self.engine.S[:P],
                         out=self.engine.R[:P], stream=stream)
        self.reuses += 1
        return False

    def pairlist(self, X: torch.Tensor):
        return self.engine.pairlist(X)
