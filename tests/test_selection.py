"""Selection rules of the classification iteration, run through the C-ABI's host-only entry points (no
device work) against plain numpy restatements of the reference's code:

- nbfLoopClustering::asignBestAlignmentAndClean (inc/em/nbfLoopClustering.h:2590-2637): best class by
  minIndex (first on ties), |distance|, cutoff = sorted[(int)(fraction * (n - 1))] with a float product,
  keep distance < cutoff;
- the refinement loop of src/MPI_Classification.cpp: next-average weights distance <= cutoff (922-934) and
  the cleaned list distance < cutoff (1137-1150);
- nbfLoopClustering::computeNewReferences (2406-2502): radius max + 0.025 ln 0.01 (double, stored float),
  sigmoid (1 + 2e) / (1 + e) - 1 with a float exponent, truncation at 0.01;
- nbfLoopClustering::doMra's class choice (1523-1592): per volume the alignment whose distances against all
  references sum lowest (double sum stored as float, first minimum).

Index and comparison rules are integer work and must agree exactly; soft weights go through expf, so they are
held to 2 float ulps of the numpy restatement. Against the same rules written in the reference's own Blitz / C++
expressions (tests/golden/clustering.npz, and oracle/_ref/libblitz_ref.so itself when built) everything,
soft weights included, is bit-exact."""
import os

import numpy as np
import pytest

import pyoracle
from ettk_gb300 import clustering

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "clustering.npz")
FRACTIONS = (0.0, 0.29, 0.5, 0.9, 1.0)


def as_table(d):
    V, R = d.shape
    D = -np.ones((V * R, 17, 1), np.float32)
    D[:, 0, 0] = d.reshape(-1)
    return D


def test_matches_reference_golden():
    g = np.load(GOLDEN)
    d = g["d"]
    R = d.shape[1]
    W, radii = clustering.soft_weights(as_table(d), R)
    assert np.array_equal(W, g["W"]) and np.array_equal(radii, g["radii"])
    for rule in (0, 1, 2):
        for f in FRACTIONS:
            best, dist, keep, _ = clustering.best_alignment_and_clean(as_table(d), R, f, rule)
            k = "%d_%g" % (rule, f)
            assert np.array_equal(best, g["best_" + k]) and np.array_equal(dist, g["dist_" + k]), k
            assert np.array_equal(keep, g["keep_" + k]), k


def test_mra_assign_matches_reference_golden():
    g = np.load(GOLDEN)
    assert np.array_equal(clustering.mra_assign(g["S"]), g["mra_labels"])


@pytest.mark.parametrize("V,R", [(1, 1), (9, 2), (200, 5)])
def test_mra_assign(V, R):
    rng = np.random.default_rng(V + R)
    S = rng.uniform(0.1, 1.0, (V, R, R)).astype(np.float32)
    S[::4] = np.round(S[::4] * 3) / 3
    labels = clustering.mra_assign(S)
    sums = S.astype(np.float64).sum(axis=2).astype(np.float32)  # sum over the references, stored as float
    assert np.array_equal(labels, np.argmin(sums, axis=1))
    ref = pyoracle.ref_mra_assign(S)
    if ref is not None:
        assert np.array_equal(labels, ref)
    bad = S.copy()
    bad[0, 0, 0] = np.nan
    with pytest.raises(Exception):
        clustering.mra_assign(bad)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_matches_reference_library(seed):
    rng = np.random.default_rng(seed)
    V, R = 37 * seed, seed + 1
    d = rng.uniform(0.1, 1.0, (V, R)).astype(np.float32)
    d[::3] = np.round(d[::3] * 4) / 4
    ref = pyoracle.ref_soft_weights(d)
    if ref is None:
        pytest.skip("reference harness not built here (oracle/build_ref.sh needs the reference tree)")
    W, radii = clustering.soft_weights(as_table(d), R)
    assert np.array_equal(W, ref[0]) and np.array_equal(radii, ref[1])
    for rule in (0, 1, 2):
        for f in (0.0, 0.37, 0.8, 1.0):
            best, dist, keep, _ = clustering.best_alignment_and_clean(as_table(d), R, f, rule)
            rb, rd, rk = pyoracle.ref_cutoff(d, f, rule)
            assert np.array_equal(best, rb) and np.array_equal(dist, rd) and np.array_equal(keep, rk)


def table(V, R, cols=17, seed=0, ties=False):
    rng = np.random.default_rng(seed)
    D = -np.ones((V * R, cols, 1), np.float32)
    d = rng.uniform(0.2, 0.9, (V, R)).astype(np.float32)
    if ties:
        d = np.round(d * 8) / 8  # many equal distances, within and across volumes
    D[:, 0, 0] = d.reshape(-1)
    return D, d


def np_cutoff(d, fraction, rule):
    best = np.argmin(d, axis=1)  # first minimum, as blitz minIndex
    dist = d[np.arange(d.shape[0]), best]
    if rule == clustering.CLEAN:
        dist = np.abs(dist)
    if not fraction < 1:
        return best, dist, np.ones(len(dist), bool), np.inf
    at = int(np.float32(fraction) * np.float32(len(dist) - 1))
    cut = np.sort(dist)[at]
    keep = dist <= cut if rule == clustering.AVERAGE else dist < cut
    return best, dist, keep, cut


@pytest.mark.parametrize("rule", [clustering.CLEAN, clustering.AVERAGE, clustering.SELECT])
@pytest.mark.parametrize("fraction", [0.0, 0.3, 0.7, 0.95, 1.0, 1.5])
@pytest.mark.parametrize("ties", [False, True])
def test_outlier_cutoff(rule, fraction, ties):
    for V, R in [(1, 1), (7, 1), (100, 3), (1001, 4)]:
        D, d = table(V, R, seed=V * 10 + R, ties=ties)
        if rule != clustering.CLEAN and V > 1:
            d[0, :] = -np.abs(d[0, :])  # a negative distance: |.| only for the clean rule
            D[0:R, 0, 0] = d[0, :]
        best, dist, keep, cut = clustering.best_alignment_and_clean(D, R, fraction, rule)
        eb, ed, ek, ec = np_cutoff(d, fraction, rule)
        assert np.array_equal(best, eb) and np.array_equal(dist, ed.astype(np.float32))
        assert np.array_equal(keep, ek), (V, R, fraction)
        assert cut == ec


def test_cutoff_float_index():
    # 0.9 * 10 in float is 9.0000002 -> index 9; in double it would also be 9, but 0.7 * 10 = 7.0000005 in
    # float (7 in double): both truncate to 7. 0.29 * 100 = 29.000000953674316 (float) vs 28.999999999999996
    # (double): the float product selects index 29, the double one 28.
    d = np.arange(101, dtype=np.float32)[:, None] / 100
    D = -np.ones((101, 17, 1), np.float32)
    D[:, 0, 0] = d[:, 0]
    _, _, keep, cut = clustering.best_alignment_and_clean(D, 1, 0.29, clustering.CLEAN)
    assert cut == np.float32(0.29) and keep.sum() == 29


def test_cutoff_rejects_nan():
    D, _ = table(5, 2)
    D[3, 0, 0] = np.nan
    with pytest.raises(Exception):
        clustering.best_alignment_and_clean(D, 2, 0.5)


def np_soft(d):
    R = d.shape[1]
    W = np.zeros((R, d.shape[0]), np.float32)
    radii = np.zeros(R, np.float32)
    decay = np.float32(0.025)
    for r in range(R):
        rad = np.float32(np.float64(d[:, r].max()) + np.float64(decay) * np.log(0.01))
        radii[r] = rad
        e = np.exp((-(d[:, r] - rad)) / decay).astype(np.float64)
        w = ((1 + 2.0 * e) / (1 + 1.0 * e) - 1.0).astype(np.float32)
        W[r] = np.where(w > 0.01, w, 0)
    return W, radii


@pytest.mark.parametrize("V,R", [(1, 1), (50, 1), (300, 5)])
def test_soft_weights(V, R):
    D, d = table(V, R, seed=V + R)
    d[: V // 3] = d[: V // 3] * 0.2 + 0.6  # a band near the largest distances, where the truncation acts
    D[:, 0, 0] = d.reshape(-1)
    W, radii = clustering.soft_weights(D, R)
    eW, er = np_soft(d)
    assert np.array_equal(radii, er)
    # exp may differ by an ulp between libm and numpy; the weights then by a few float ulps
    assert np.allclose(W, eW, rtol=3e-7, atol=1e-7)
    assert np.array_equal(W > 0, eW > 0)
    assert (W[W > 0] > 0.01).all() and (W <= 1).all()


def test_soft_weights_radius_semantics():
    # one volume: radius = d + 0.025 ln 0.01, the weight there is (1 + 2/100)/(1 + 1/100) - 1 < 0.01 -> 0
    D = -np.ones((1, 17, 1), np.float32)
    D[0, 0, 0] = 0.5
    W, radii = clustering.soft_weights(D, 1)
    assert W[0, 0] == 0
    assert abs(radii[0] - (0.5 + 0.025 * np.log(0.01))) < 1e-7


def test_host_entries_reject_bad_arguments():
    import ctypes
    from ettk_gb300 import _lib
    L = _lib.load()
    D, _ = table(4, 2)
    buf_i = np.zeros(8, np.int32)
    buf_f = np.zeros(8, np.float32)
    cut = ctypes.c_float()
    # class count, volume count, row stride and rule out of range; missing outputs
    for R, V, ld, rule in [(0, 4, 17, 0), (2, 0, 17, 0), (2, 4, 0, 0), (2, 4, 17, 3), (2, 4, 17, -1)]:
        assert L.ettk_gpu_outlier_cutoff(R, V, D.ctypes.data, ld, 0.5, rule, buf_i.ctypes.data, buf_f.ctypes.data,
                                         buf_i.ctypes.data, ctypes.byref(cut)) == _lib.ETTK_ERR_ARG
    assert L.ettk_gpu_outlier_cutoff(2, 4, D.ctypes.data, 17, 0.5, 0, None, buf_f.ctypes.data, buf_i.ctypes.data,
                                     None) == _lib.ETTK_ERR_ARG
    assert L.ettk_gpu_outlier_cutoff(2, 4, D.ctypes.data, 17, float("nan"), 0, buf_i.ctypes.data, buf_f.ctypes.data,
                                     buf_i.ctypes.data, None) == _lib.ETTK_ERR_NAN
    W = np.zeros(16, np.float32)
    assert L.ettk_gpu_soft_weights(0, 4, D.ctypes.data, 17, W.ctypes.data, None) == _lib.ETTK_ERR_ARG
    assert L.ettk_gpu_soft_weights(2, 4, D.ctypes.data, 17, None, None) == _lib.ETTK_ERR_ARG
    S = np.ones((4, 2, 2), np.float32)
    assert L.ettk_gpu_mra_assign(2, 4, S.ctypes.data, None) == _lib.ETTK_ERR_ARG
    assert L.ettk_gpu_mra_assign(0, 4, S.ctypes.data, buf_i.ctypes.data) == _lib.ETTK_ERR_ARG
    assert L.ettk_gpu_mra_assign(2, 4, S.ctypes.data, buf_i.ctypes.data) == _lib.ETTK_OK
