"""nsl_gb300: GB300-native (sm_103a) implementation of NSL's fermion-matrix hot path.

The compute lives in libnslgpu.so (CUDA kernels behind the C ABI of include/nsl_gb300.h); this package mirrors the
reference C++ API on top of it: lattices (Ring, Honeycomb), HubbardExp, HubbardDiag, CG, the Hubbard actions and the leapfrog
integrators, and Markov-chain files in NSL's HDF5 node layout (without HDF5).
"""
from .context import Context, default_context
from .fermion_matrix import HubbardDiag, HubbardExp, MatrixCombination, Species
from .lattice import Honeycomb, Ring, SpatialLattice
from .markov_io import MarkovChainFile
from .solver import CG, cg_group

__all__ = ["Context", "default_context", "HubbardExp", "HubbardDiag", "MatrixCombination", "Species", "Honeycomb", "Ring",
           "SpatialLattice", "CG", "cg_group", "MarkovChainFile"]
