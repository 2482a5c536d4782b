"""Average variance (nbfWedgedAverageImage3D::getImageVarianceMPI, inc/em/nbfWedgedAverageImage3D.h:440-493) and
n-fold symmetrisation (nbfImageFilter::symmetrize, inc/em/nbfImageFilter.h:527-554) against the oracle's FP64
restatements; 1e-5 relative RMS, as the class average.

Rotational symmetrisation (src/MPI_Classification.cpp:1005-1024): the oracle's restatement is pinned bit for
bit to the reference's own nbfCylindricalDomain3 / nbfLinearInterpolator (tests/golden/rotsym_n16.npz, and the
harness library itself when it is built); the GPU (FP64, no contraction; only cos / sin / atan2 may differ in
their last bits) is held to 1e-6 of the maximum per voxel, i.e. float output rounding."""
import os

import numpy as np
import pytest

import pyoracle
from ettk_gb300 import synthetic
from ettk_gb300.metric import ProjectionRotationMetric3D, WedgedSubImage3D

KW = ("lwedge", "uwedge", "normal", "matrix", "position", "cut_offset")


def rel_rms(g, o):
    return float(np.sqrt(np.mean((g - o) ** 2)) / np.sqrt(np.mean(o ** 2)))


@pytest.fixture(scope="module")
def ds32():
    return synthetic.generate("align32_b16", n_particles=5)


def test_oracle_symmetrize_fold1_is_identity(ds32):
    v = ds32.references[0]
    assert np.array_equal(pyoracle.symmetrize(ds32.params, v, 1).transpose(2, 1, 0), v.astype(np.float64))


@pytest.mark.gpu
@pytest.mark.parametrize("fold", [1, 2, 3, 6])
def test_symmetrize(ds32, fold):
    m = ProjectionRotationMetric3D(ds32.params)
    try:
        g = m.symmetrize(ds32.references[0], fold)
    finally:
        m.close()
    o = pyoracle.symmetrize(ds32.params, ds32.references[0], fold).transpose(2, 1, 0)
    assert rel_rms(g, o) <= 1e-5, (fold, rel_rms(g, o))


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "rotsym_n16.npz")


def test_oracle_rotational_matches_reference_golden():
    g = np.load(GOLDEN)
    for v, out in zip(g["vol"], g["out"]):
        assert np.array_equal(pyoracle.symmetrize_rotational(v), out)


def test_oracle_rotational_matches_reference_library():
    rng = np.random.default_rng(5)
    v = rng.standard_normal((32, 32, 32)).astype(np.float32)
    r = pyoracle.ref_symmetrize_rotational(v)
    if r is None:
        pytest.skip("reference harness not built here (oracle/build_ref.sh needs the reference tree)")
    assert np.array_equal(pyoracle.symmetrize_rotational(v), r)


def test_oracle_rotational_is_symmetric():
    # voxels at the same distance from the axis in one plane carry the same value up to the angle weight's
    # rounding; (x, y) -> (y, x) and the quarter turns about (N/2, N/2) keep the distance
    g = np.load(GOLDEN)
    o = pyoracle.symmetrize_rotational(g["vol"][1])  # [x][y][z]
    N = o.shape[0]
    inner = o[1:, 1:, :]  # indices 1..N-1: the quarter turns about N/2 map them onto themselves
    for t in (inner.transpose(1, 0, 2), np.rot90(inner, 1, (0, 1)), np.rot90(inner, 2, (0, 1))):
        assert np.abs(t - inner).max() <= 1e-12 * np.abs(inner).max()
    assert N == 16


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["reference", "particle"])
def test_symmetrize_rotational(ds32, which):
    vol = ds32.references[0] if which == "reference" else ds32.particles[1]
    m = ProjectionRotationMetric3D(ds32.params)
    try:
        g = m.symmetrize_rotational(vol)
    finally:
        m.close()
    o = pyoracle.symmetrize_rotational(vol).transpose(2, 1, 0)
    assert np.abs(g - o).max() <= 1e-6 * np.abs(o).max(), np.abs(g - o).max() / np.abs(o).max()


@pytest.mark.gpu
def test_variance(ds32):
    members = [0, 1, 2, 3, 4]
    weights = [1.0, 1.0, 0.5, -0.25, 0.0]
    mats = []
    for i in members:
        T = np.eye(4)
        T[:3, :3] = ds32.truth[i]["rotation"]
        T[:3, 3] = ds32.truth[i]["shift"]
        mats.append(T)
    o_avg = pyoracle.average(ds32.params, [ds32.particles[i] for i in members], [ds32.meta[i] for i in members],
                             weights, mats)  # [x][y][z]
    avg = o_avg.transpose(2, 1, 0).astype(np.float32)  # the same (float) average for both sides
    m = ProjectionRotationMetric3D(ds32.params)
    try:
        m.set_particles([WedgedSubImage3D(ds32.particles[i], **{k: ds32.meta[i][k] for k in KW}) for i in members])
        g = m.variance(members, weights, mats, avg)
    finally:
        m.close()
    o = pyoracle.variance(ds32.params, [ds32.particles[i] for i in members], [ds32.meta[i] for i in members], weights,
                          mats, avg.transpose(2, 1, 0).astype(np.float64)).transpose(2, 1, 0)
    assert rel_rms(g, o) <= 1e-5, rel_rms(g, o)


def _shifted_rot_z(deg, shift):
    from ettk_gb300 import classification
    T = classification._rot_z(deg)
    S = np.eye(4)
    S[:3, 3] = shift
    return T @ S


@pytest.mark.gpu
def test_mean_images(ds32):
    """ettk_gpu_mean_images: the mean of getImage of a fixed image under rotations with translations, against the
    oracle's FP64 getImage (1e-5 relative RMS)."""
    vol = ds32.references[0]
    ts = [np.eye(4), _shifted_rot_z(120.0, (1.5, -0.5, 0.25)), _shifted_rot_z(240.0, (-1.0, 2.0, 0.5))]
    m = ProjectionRotationMetric3D(ds32.params)
    try:
        g = m.mean_images(vol, ts)
    finally:
        m.close()
    full = {"lwedge": -90.0, "uwedge": 90.0}
    o = np.mean([pyoracle.get_image(ds32.params, vol, full, t) for t in ts], axis=0).transpose(2, 1, 0)
    assert rel_rms(g, o) <= 1e-5, rel_rms(g, o)


@pytest.mark.gpu
def test_symmetrize_aligned(ds32):
    """The aligned n-fold step of the global-average loop (nbfLoopClustering::symmetrize with alignment,
    inc/em/nbfLoopClustering.h:5950-6076) on the GPU against the oracle: the same CCF transforms for every fold, and
    the symmetrised image within 1e-5 relative RMS."""
    from ettk_gb300 import classification
    fold = 3
    vol = ds32.references[0]
    m = ProjectionRotationMetric3D(ds32.params)
    try:
        img, ts = classification.symmetrize_aligned(m, vol, fold)
    finally:
        m.close()
    p = ds32.params
    full = {"lwedge": -90.0, "uwedge": 90.0}
    to = [np.eye(4)]
    for f in range(1, fold):
        _, t = pyoracle.ccf(p, vol, full, vol, full, classification._rot_z(f * 360.0 / fold))
        to.append(t)
    for a, b in zip(ts, to):
        assert np.allclose(a, b, atol=1e-6), (a, b)
    shifted = np.mean([pyoracle.get_image(p, vol, full, t) for t in to], axis=0)  # [x][y][z]
    o = pyoracle.symmetrize(p, np.ascontiguousarray(shifted.transpose(2, 1, 0)).astype(np.float32), fold)
    assert rel_rms(img, o.transpose(2, 1, 0)) <= 1e-5, rel_rms(img, o.transpose(2, 1, 0))
