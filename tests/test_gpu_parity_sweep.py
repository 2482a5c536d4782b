"""Parity sweep: full alignments on the GPU (through the C ABI) against the oracle, pair by pair.

Covers every pair of the 32^3 B=16 workload (200 particles, fixed +-60 degree wedges), 32 pairs of the
64^3 B=32 workload (per-particle wedges with rotated tilt axes) and, at 32^3, every non-default option
branch of the getDistances path:

- number_of_candidates 3 with D holding 3 candidate slots and 19 columns (inc/em/nbfCorrelationImageMetric.h:
  1984-2001: column 0 of every slot first set to FLT_MAX, scale and overlap 1 per candidate,
  inc/em/nbfProjectionRotationMetric3D.h:874-881);
- 19 columns with one candidate: the wedge overlap of the final transform (getWedgeOverlap,
  inc/em/nbfCorrelationImageMetric.h:532-565, written at 1973-1976);
- a rotation search restricted to 30 degrees (isTransformValid, inc/em/nbfImageMetric.h:415-459, and the beta
  rows cut from the SO(3) peak search, inc/em/nbfProjectionRotationMetric3D.h:602);
- a B-factor (buildBFactorHalf, inc/em/nbfFourierFilter.h:778-797);
- distances not normalised by the overlap, and missing-wedge compensation off (inc/em/nbfImageMetric.h:151-158);
- mutual correlation (|F|^(1/2) spherical projections, inc/em/nbfProjectionRotationMetric3D.h:318-325; F / |F|^(1/2)
  before the CCF filter, inc/em/nbfFourierFilter.h:586-606);
- the resume rule: rows of D whose first entry is not -1 are left as they are (getDistances 1944-1946).

Criterion per pair (the parity bar of this path): the same SO(3) grid cell (rotation entries equal to 1e-5;
both sides build them from the same grid angles), the same half-voxel shift (translations equal to 1e-4) and
the distance within 1e-4 relative. The oracle runs on all host cores (its ctypes calls release the GIL). With
ETTK_PARITY_SUMMARY set, the agreement counts of every case are written there as JSON.
"""
import json
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import pyoracle
from ettk_gb300 import synthetic
from ettk_gb300.metric import ProjectionRotationMetric3D, WedgedSubImage3D

pytestmark = pytest.mark.gpu

KW = ("lwedge", "uwedge", "normal", "matrix", "position", "cut_offset")
SUMMARY = {}


def vol(img, meta):
    return WedgedSubImage3D(img, **{k: meta[k] for k in KW})


def oracle_all(params, ds, idx):
    """pyoracle.align of particles idx against reference 0, on all host cores."""
    def one(i):
        return pyoracle.align(params, ds.references[0], ds.ref_meta[0], ds.particles[i], ds.meta[i])
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        return list(ex.map(one, idx))


def gpu_all(params, ds, idx, cols=17, ncand=1, D=None):
    m = ProjectionRotationMetric3D(params)
    try:
        m.set_references([vol(ds.references[0], ds.ref_meta[0])])
        m.set_particles([vol(ds.particles[i], ds.meta[i]) for i in idx])
        return m.getDistances([(0, k) for k in range(len(idx))], D=D, cols=cols, ncand=ncand)
    finally:
        m.close()


def same_pose(T, M):
    return bool(np.allclose(T[:3, :3], M[:3, :3], atol=1e-5) and np.allclose(T[:3, 3], M[:3, 3], atol=1e-4))


def same_distance(d, o):
    return abs(float(d) - float(o)) <= 1e-4 * abs(float(o))


def record(case, n, cells, shifts, dists, extra=None):
    SUMMARY[case] = dict(pairs=n, same_cell=cells, same_shift=shifts, distance_1e4=dists, **(extra or {}))
    path = os.environ.get("ETTK_PARITY_SUMMARY")
    if path:
        with open(path, "w") as f:
            json.dump(SUMMARY, f, indent=1, sort_keys=True)


def check_rows(case, D, orc, off=1):
    """Slot 0 of every row against the oracle's best alignment; returns the mismatching pairs."""
    bad, cells, shifts, dists = [], 0, 0, 0
    for i, o in enumerate(orc):
        T = D[i, off:off + 16, 0].reshape(4, 4)
        c = bool(np.allclose(T[:3, :3], o["matrix"][:3, :3], atol=1e-5))
        s = c and bool(np.allclose(T[:3, 3], o["matrix"][:3, 3], atol=1e-4))
        d = same_distance(D[i, 0, 0], o["distance"])
        cells += c
        shifts += s
        dists += d
        if not (c and s and d):
            bad.append((i, float(D[i, 0, 0]), o["distance"], T[:3, 3].tolist(), o["matrix"][:3, 3].tolist()))
    record(case, len(orc), cells, shifts, dists)
    return bad


@pytest.fixture(scope="module")
def ds32():
    return synthetic.generate("align32_b16")


def test_sweep_workload32_all_pairs(ds32):
    """All 200 pairs of the 32^3 B=16 workload."""
    idx = list(range(len(ds32.meta)))
    assert len(idx) == 200
    D = gpu_all(ds32.params, ds32, idx)
    orc = oracle_all(ds32.params, ds32, idx)
    bad = check_rows("align32_b16_all", D, orc)
    assert not bad, bad


def test_sweep_workload64_32_pairs():
    """32 pairs of the 64^3 B=32 workload (per-particle wedges with in-plane tilt axes)."""
    ds = synthetic.generate("align64_b32", n_particles=32)
    idx = list(range(32))
    D = gpu_all(ds.params, ds, idx)
    orc = oracle_all(ds.params, ds, idx)
    bad = check_rows("align64_b32_32", D, orc)
    assert not bad, bad


BRANCHES = {
    "rotation_restricted_30": dict(restrict_rotation=30.0),
    "bfactor_2": dict(bfactor=2.0),
    "overlap_normalisation_off": dict(overlap_normalized=False),
    "wedge_compensation_off": dict(wedge_compensation=False),
    "candidate_peaks_3": dict(candidate_peaks=3),
    "mutual_correlation": dict(mutual_correlation=True),
}


@pytest.mark.parametrize("case", sorted(BRANCHES))
def test_sweep_branch(ds32, case):
    params = dict(ds32.params, **BRANCHES[case])
    idx = list(range(24))
    D = gpu_all(params, ds32, idx)
    orc = oracle_all(params, ds32, idx)
    bad = check_rows(case, D, orc)
    assert not bad, bad


def test_sweep_overlap_column(ds32):
    """19 columns, one candidate: distance, scale 1, getWedgeOverlap at the final transform, matrix."""
    params = dict(ds32.params)
    idx = list(range(24))
    D = gpu_all(params, ds32, idx, cols=19)
    orc = oracle_all(params, ds32, idx)
    bad = check_rows("cols19_overlap", D, orc, off=3)
    assert not bad, bad
    assert np.all(D[:, 1, 0] == 1.0)
    ov = np.array([o["wedge_overlap"] for o in orc], np.float64)
    assert np.all((ov > 0) & (ov < 1))  # the particles' wedges are effective
    err = np.abs(D[:, 2, 0] - ov) / ov
    SUMMARY["cols19_overlap"]["overlap_max_rel_err"] = float(err.max())
    assert err.max() <= 1e-4, err.max()
    # 18 columns: the scale only
    D18 = gpu_all(params, ds32, idx[:4], cols=18)
    assert np.all(D18[:, 1, 0] == 1.0)
    assert np.allclose(D18[:, 2:18, 0], D[:4, 3:19, 0])


def test_sweep_three_candidates(ds32):
    """number_of_candidates 3 into 3 slots of 19 columns, each slot against the oracle's candidate."""
    params = dict(ds32.params, number_of_candidates=3)
    idx = list(range(24))
    D = gpu_all(params, ds32, idx, cols=19, ncand=3)
    orc = oracle_all(params, ds32, idx)
    bad, slots = [], 0
    for i, o in enumerate(orc):
        n = len(o["cand_distance"])
        for c in range(3):
            if c < n:
                T = D[i, 3:19, c].reshape(4, 4)
                ok = (same_pose(T, o["cand_matrix"][c]) and same_distance(D[i, 0, c], o["cand_distance"][c])
                      and D[i, 1, c] == 1.0 and D[i, 2, c] == 1.0)
                slots += 1
                if not ok:
                    bad.append((i, c, float(D[i, 0, c]), o["cand_distance"][c]))
            else:
                if D[i, 0, c] != np.finfo(np.float32).max:
                    bad.append((i, c, "unused slot", float(D[i, 0, c])))
    SUMMARY["three_candidates"] = dict(pairs=len(orc), slots_compared=slots, mismatches=len(bad))
    record("three_candidates_rows", len(orc), *(3 * [len(orc) - len(bad)]))
    assert not bad, bad


def test_sweep_resume_rule(ds32):
    """Rows whose D[i][0][0] != -1 on entry are skipped and keep every entry; the others are computed."""
    params = dict(ds32.params)
    idx = list(range(8))
    D = -np.ones((8, 17, 1), np.float32)
    keep = [1, 2, 5]
    for i in keep:
        D[i] = 7.0 + i
    before = D.copy()
    D = gpu_all(params, ds32, idx, D=D)
    for i in keep:
        assert np.array_equal(D[i], before[i])
    todo = [i for i in idx if i not in keep]
    orc = oracle_all(params, ds32, todo)
    bad = check_rows("resume_rule", D[todo], orc)
    assert not bad, bad


def _ellipsoid(M, a, b, c):
    """A binary ellipsoid in a cube of edge M, [z][y][x] (x fastest, as a mask file holds it), values 0 / 1.5."""
    z, y, x = np.mgrid[0:M, 0:M, 0:M] - M / 2.0
    return np.where((x / a) ** 2 + (y / b) ** 2 + (z / c) ** 2 <= 1.0, 1.5, 0.0).astype(np.float32)


@pytest.mark.parametrize("offset", [8, -8])
def test_sweep_external_mask(ds32, offset):
    """An external mask (nbfImageFilter::setMaskFile, used as the CCF's referenceMask by
    nbfFourierImageMetric::reinitializeHalf, inc/em/nbfFourierImageMetric.h:667-676) of edge N + 8 (centre cropped)
    and N - 8 (centred into the box): the library's processed mask equals the oracle's, 24 alignments match the
    oracle's with the same mask, and clearing the mask gives the spherical-mask results again."""
    params = dict(ds32.params)
    N = params["N"]
    mask = _ellipsoid(N + offset, 0.34 * (N + offset), 0.28 * (N + offset), 0.38 * (N + offset))
    m1 = pyoracle.file_mask(params, mask, 0.5)
    idx = list(range(24))
    m = ProjectionRotationMetric3D(params)
    try:
        m.setMaskFile(mask, 0.5)
        got = m.reference_mask().transpose(2, 1, 0)
        err = float(np.abs(got - m1).max())
        assert err <= 1e-6, err
        m.set_references([vol(ds32.references[0], ds32.ref_meta[0])])
        m.set_particles([vol(ds32.particles[i], ds32.meta[i]) for i in idx])
        pairs = [(0, k) for k in range(len(idx))]
        D = m.getDistances(pairs)
        m.setMaskFile(None, 0.0)
        D0 = m.getDistances(pairs)
    finally:
        m.close()
    orc = oracle_all(dict(params, reference_mask=m1), ds32, idx)
    bad = check_rows("external_mask_%d" % (N + offset), D, orc)
    SUMMARY["external_mask_%d" % (N + offset)]["mask_max_abs_err"] = err
    assert not bad, bad
    assert np.array_equal(D0, gpu_all(params, ds32, idx))
    assert not np.allclose(D[:, 0, 0], D0[:, 0, 0])
