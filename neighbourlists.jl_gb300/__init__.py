"""GB300 (sm_103a) neighbour-list engine, a drop-in for the sort-based path of
NeighbourLists.jl: neighbour_list -> build_cell_list -> materialize_pairlist /
for_each_neighbour.  All compute runs in hand-written CUDA kernels behind the
C ABI of libnlgpu.so (include/nlgpu.h)."""
from ._lib import NLError, LIB_PATH, lib  # noqa: F401
from .api import (  # noqa: F401
    PairList,
    SortedCellList,
    analyze_cell,
    build_cell_list,
    count_neighbours,
    cutoff,
    for_each_neighbour,
    lazy_reduce,
    legacy_pairlist,
    materialize_pairlist,
    max_neighbours,
    maxneigs,
    neighbour_list,
    neighbours,
    neigs,
    neigss,
    nneigs,
    npairs,
    nsites,
    num_neighbours,
    pair_vectors,
    pairs,
    query_neighbours,
    sites,
)
from .atoms import System, build_cell_list_system, isolated_cell, neighbour_list_system  # noqa: F401
from .batch import BatchNeighbourList  # noqa: F401
from .engine import NeighbourListEngine  # noqa: F401
from .serving import NeighbourListServer, Request, poisson_trace  # noqa: F401
from .tuning import autotune  # noqa: F401
from .verlet import VerletList  # noqa: F401
