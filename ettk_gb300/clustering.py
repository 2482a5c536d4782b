"""Host-side selection rules of the classification iteration (nbfLoopClustering and the refinement loop of
MPI_Classification), over a distance table as ProjectionRotationMetric3D.getDistances fills it for pairs
ordered volume-major: row v * R + r holds volume v against class r, the distance in column 0 of candidate 0.

These run in the CUDA library's host code (no device work, no context) so that the C-ABI serves callers
outside Python too.
"""
import ctypes

import numpy as np

from . import _lib
from .metric import EttkError

# rules of best_alignment_and_clean
CLEAN = 0     # nbfLoopClustering::asignBestAlignmentAndClean: |distance|, keep distance < cutoff
AVERAGE = 1   # weights of the next global average (MPI_Classification.cpp:922-934): keep distance <= cutoff
SELECT = 2    # the cleaned volume list (MPI_Classification.cpp:1137-1150): keep distance < cutoff


def _table(D, R):
    D = np.ascontiguousarray(D, np.float32)
    if D.ndim == 1:
        D = D.reshape(-1, 1)
    rows = D.shape[0]
    if R < 1 or rows % R:
        raise ValueError("the table must hold V * R rows")
    return D, rows // R, int(np.prod(D.shape[1:]))


def best_alignment_and_clean(D, R, top_fraction, rule=CLEAN):
    """Best class per volume and the top-fraction outlier cutoff (inc/em/nbfLoopClustering.h:2590-2637 for
    rule CLEAN). Returns (best [V] int32, distance [V] float32, keep [V] bool, cutoff float; inf when
    top_fraction >= 1)."""
    D, V, ld = _table(D, R)
    best = np.zeros(V, np.int32)
    dist = np.zeros(V, np.float32)
    keep = np.zeros(V, np.int32)
    cut = ctypes.c_float()
    rc = _lib.load().ettk_gpu_outlier_cutoff(R, V, D.ctypes.data, ld, float(top_fraction), int(rule),
                                             best.ctypes.data, dist.ctypes.data, keep.ctypes.data,
                                             ctypes.byref(cut))
    if rc != _lib.ETTK_OK:
        raise EttkError(rc, "outlier_cutoff: invalid table or arguments")
    return best, dist, keep.astype(bool), cut.value


def soft_weights(D, R):
    """Soft class weights of nbfLoopClustering::computeNewReferences (inc/em/nbfLoopClustering.h:2406-2502).
    Returns (W [R][V] float32, radii [R] float32)."""
    D, V, ld = _table(D, R)
    W = np.zeros((R, V), np.float32)
    radii = np.zeros(R, np.float32)
    rc = _lib.load().ettk_gpu_soft_weights(R, V, D.ctypes.data, ld, W.ctypes.data, radii.ctypes.data)
    if rc != _lib.ETTK_OK:
        raise EttkError(rc, "soft_weights: invalid table")
    return W, radii


def mra_assign(S):
    """Class choice of the MRA loop (nbfLoopClustering::doMra): S[v][r][j] is the distance of volume v, under the
    alignment it received from reference r, against reference j. Returns labels [V] int32."""
    S = np.ascontiguousarray(S, np.float32)
    V, R, R2 = S.shape
    if R != R2:
        raise ValueError("S must be V x R x R")
    labels = np.zeros(V, np.int32)
    rc = _lib.load().ettk_gpu_mra_assign(R, V, S.ctypes.data, labels.ctypes.data)
    if rc != _lib.ETTK_OK:
        raise EttkError(rc, "mra_assign: invalid table")
    return labels
