"""treeamr: GB300-native ghost filling for block-structured AMR.

A drop-in for the ghost-fill path of TreeAMR.jl: the host builds the
reference's ``GhostSchedule`` (forest, field set, operators) and the CUDA
library ``libtreeamr_cuda.so`` replays it on one GPU.
"""
from .forest import (Forest, MortonKey, OUTER, OUTFLOW, REFLECTING, alldirections, childoffset,
                     curve_key, parentkey, sortedchildkeys)
from .operators import Conservative, Operators, PointValue, check_operators, lagrange_weights
from .storage import (EvenParity, FieldSet, NoParity, OddParity, RotationPair, cellcentered,
                      coordinates, staggers, vertexcentered)
from .schedule import GhostSchedule, TransferGroup, Stencil1D, GroupKey
from .ghosts import boundary_by_coordinates, fill_ghosts
from .state import gather, scatter, scatter_fill, statearray, statelength, statevector

__all__ = [
    "Forest", "MortonKey", "alldirections", "childoffset", "curve_key", "parentkey",
    "sortedchildkeys", "OUTER", "OUTFLOW", "REFLECTING",
    "Operators", "PointValue", "Conservative", "check_operators", "lagrange_weights",
    "FieldSet", "RotationPair", "EvenParity", "OddParity", "NoParity", "cellcentered", "vertexcentered",
    "staggers", "coordinates",
    "GhostSchedule", "TransferGroup", "Stencil1D", "GroupKey",
    "fill_ghosts", "boundary_by_coordinates",
    "statelength", "statevector", "statearray", "scatter", "gather", "scatter_fill",
]
