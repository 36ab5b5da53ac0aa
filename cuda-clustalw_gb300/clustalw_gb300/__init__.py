"""GB300-native full-pairwise distance stage of ClustalW 2.0.11.

The alignment work runs in lib/libcwgpu.so (hand-written sm_103a CUDA behind
the C ABI of include/cwgpu.h); this package is the host-side mirror of the
reference's pairwise plugin interface plus workload generators.
"""
from . import native, pairwise, synth  # noqa: F401
from .matrices import load_matrix  # noqa: F401
from .native import Context, CwgpuError, Params, Plan  # noqa: F401
from .pairwise import Alignment, DistMatrix, FullPairwiseAlign, PairwiseSettings, SymMatrix  # noqa: F401
