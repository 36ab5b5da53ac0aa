"""Pairwise substitution matrices and scale values as the reference produces
them.

data/pairwise_matrices.json holds the int[32][32] matrix, PairScaleValues and
matAvg that SubMatrix::getPairwiseMatrix (substitutionMatrix/SubMatrix.cpp:
256-390) returns for the default protein (Gonnet 250) and DNA (IUB) settings,
plus the default pairwise gap penalties (general/UserParameters.cpp:79-82).
They were written by running the unmodified reference (oracle/_ref/refharness)
from tests/golden/make_golden.py; they are data, not re-derived here.
"""
import json
import os

import numpy as np

DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "pairwise_matrices.json")


def load_matrix(kind):
    """kind: 'protein' (Gonnet, gap open 10.0, extension 0.1) or 'dna' (IUB,
    gap open 15.0, extension 6.66). Returns (matrix[32,32] int32, params dict)."""
    with open(DATA) as f:
        d = json.load(f)[kind]
    return np.array(d["matrix"], dtype=np.int32).reshape(32, 32), dict(d["params"])
