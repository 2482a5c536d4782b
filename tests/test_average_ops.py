"""Average variance (nbfWedgedAverageImage3D::getImageVarianceMPI, inc/em/nbfWedgedAverageImage3D.h:440-493) and
n-fold symmetrisation (nbfImageFilter::symmetrize, inc/em/nbfImageFilter.h:527-554) against the oracle's FP64
restatements; 1e-5 relative RMS, as the class average."""
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
