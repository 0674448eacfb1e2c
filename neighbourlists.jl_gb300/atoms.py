"""System-level entry points, mirroring the reference's AtomsBase extension
(ext/NeighbourListsAtomsBaseExt.jl:17-140).

A "system" is anything with positions (N x 3), a cell (3 x 3, rows are the
lattice vectors) or None for an isolated system, and a periodicity (3 bools);
positions and cell are in the unit of ``length_unit`` (a scale factor that
strips units: value_in_length_unit = value * length_unit).

For an isolated system the reference builds the cell from the positions'
bounding box, diag(max - min + 1) per axis (_get_cell_matrix, :17-38), and
leaves the positions where they are; this module does exactly that, so the
outputs are those of the reference's PairList(system, cutoff).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np
import torch

from .api import build_cell_list, materialize_pairlist

__all__ = ["System", "isolated_cell", "cell_matrix", "neighbour_list_system", "build_cell_list_system"]


@dataclass
class System:
    positions: object                 # (N, 3) numpy array or torch tensor
    cell: Optional[np.ndarray]        # 3x3 rows = lattice vectors, or None (isolated)
    periodicity: Sequence[bool]


def isolated_cell(positions) -> np.ndarray:
    """Bounding-box cell of an isolated 3-D system: diag(max - min + 1)."""
    X = positions.detach().cpu().numpy() if isinstance(positions, torch.Tensor) else np.asarray(positions)
    X = X.reshape(-1, 3).astype(np.float64)
    if X.shape[0] == 0:
        raise ValueError("an isolated system needs at least one atom to define its bounding box")
    ext = (X.max(axis=0) - X.min(axis=0)) + 1.0
    return np.diag(ext)


def cell_matrix(system: System, length_unit: float = 1.0) -> np.ndarray:
    if system.cell is None:
        return isolated_cell(_positions(system, length_unit))
    return np.asarray(system.cell, dtype=np.float64).reshape(3, 3) * length_unit


def _positions(system: System, length_unit: float):
    X = system.positions
    if isinstance(X, torch.Tensor):
        X = X.to(torch.float64)
        return X * length_unit if length_unit != 1.0 else X
    X = np.asarray(X, dtype=np.float64).reshape(-1, 3)
    return X * length_unit if length_unit != 1.0 else X


def build_cell_list_system(system: System, cutoff: float, length_unit: float = 1.0, int_type=torch.int32):
    """build_cell_list(system, cutoff) (AtomsBase extension :75-87)."""
    X = _positions(system, length_unit)
    return build_cell_list(X, float(cutoff) * length_unit, cell_matrix(system, length_unit),
                           tuple(bool(b) for b in system.periodicity), int_type=int_type)


def neighbour_list_system(system: System, cutoff: float, length_unit: float = 1.0, lazy: bool = False,
                          int_type=torch.int32):
    """neighbour_list(system, cutoff; lazy) (AtomsBase extension :116-140)."""
    clist = build_cell_list_system(system, cutoff, length_unit, int_type)
    return clist if lazy else materialize_pairlist(clist)
