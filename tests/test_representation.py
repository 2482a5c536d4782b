"""Low-dimensional representations (nbfFourierImageMetric::getLowDimensionRepresentationHalf,
inc/em/nbfFourierImageMetric.h:1967-2034) and the distances between them (nbfCorrelationImageMetric::getDistances
(file, D), inc/em/nbfCorrelationImageMetric.h:1726-1871), the pairwise step of the unsupervised classification.

Representations: three unnormalised FP32 3-D transforms on the GPU against the oracle's FP64 ones, held to 2e-5
of the largest coefficient magnitude (5e-5 with the n-fold symmetrisation's extra reslices); the band (which
coefficients, in which order) and the wedge bits exactly.

The oracle restates the loop with the roundings Blitz gives it (complex<float> element arithmetic, sum() in
double, mean() in float); tests/golden/repr_dist.npz holds the outputs of that loop written in the reference's
own Blitz expressions on its vendored Blitz (oracle/_ref/libblitz_ref.so). The distances are bit-exact: the
GPU kernel accumulates every pair sequentially in k with each operation rounded as on the CPU."""
import os

import numpy as np
import pytest

import pyoracle
from ettk_gb300 import synthetic
from ettk_gb300.metric import ProjectionRotationMetric3D, WedgedSubImage3D

KW = ("lwedge", "uwedge", "normal", "matrix", "position", "cut_offset")

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "repr_dist.npz")


def rand_repr(V, K, depth, seed, binary=True):
    rng = np.random.default_rng(seed)
    R = rng.standard_normal((V, K, depth)).astype(np.float32)
    if depth == 3:
        R[:, :, 2] = (rng.random((V, K)) > 0.25) if binary else rng.uniform(0, 1.5, (V, K))
    return np.ascontiguousarray(R, np.float32)


def test_oracle_matches_reference_golden():
    g = np.load(GOLDEN)
    for norm in (0, 1):
        assert np.array_equal(pyoracle.representation_distances(g["R3"], norm), g["D3_%d" % norm])
        assert np.array_equal(pyoracle.representation_distances(g["R1"], norm), g["D1_%d" % norm])


@pytest.mark.parametrize("binary", [True, False])
def test_oracle_matches_reference_library(binary):
    R = rand_repr(21, 517, 3, 5, binary)
    r = pyoracle.ref_representation_distances(R, True)
    if r is None:
        pytest.skip("reference harness not built here (oracle/build_ref.sh needs the reference tree)")
    assert np.array_equal(pyoracle.representation_distances(R, True), r)
    assert np.array_equal(pyoracle.representation_distances(R, False), pyoracle.ref_representation_distances(R, False))


def test_oracle_properties():
    R = rand_repr(6, 64, 3, 9)
    D = pyoracle.representation_distances(R, True)
    assert np.array_equal(D, D.T) and (np.diag(D) == 0).all() and (D >= 0).all()
    R[3] = R[1]
    D = pyoracle.representation_distances(R, True)
    assert D[1, 3] == 0


@pytest.fixture(scope="module")
def metric():
    m = ProjectionRotationMetric3D(synthetic.default_params(synthetic.WORKLOADS["align32_b16"]))
    yield m
    m.close()


@pytest.mark.gpu
def test_gpu_golden(metric):
    g = np.load(GOLDEN)
    for norm in (0, 1):
        assert np.array_equal(metric.representation_distances(g["R3"], norm), g["D3_%d" % norm])
        assert np.array_equal(metric.representation_distances(g["R1"], norm), g["D1_%d" % norm])


@pytest.mark.gpu
@pytest.mark.parametrize("V,K", [(1, 5), (2, 3), (70, 1007), (97, 64)])
@pytest.mark.parametrize("depth", [3, 1])
@pytest.mark.parametrize("norm", [1, 0])
def test_gpu_matches_oracle(metric, V, K, depth, norm):
    R = rand_repr(V, K, depth, V * K + depth, binary=(V % 2 == 0))
    g = metric.representation_distances(R, norm)
    o = pyoracle.representation_distances(R, norm)
    assert np.array_equal(g, o), np.abs(g - o).max()


@pytest.mark.gpu
def test_gpu_rejects_bad_input(metric):
    R = rand_repr(4, 10, 3, 1)
    R[2, 3, 0] = np.inf
    with pytest.raises(Exception):
        metric.representation_distances(R)
    with pytest.raises(Exception):
        metric.representation_distances(np.zeros((3, 4, 2), np.float32))


@pytest.fixture(scope="module")
def ds32():
    return synthetic.generate("align32_b16", n_particles=4)


def test_oracle_representation_band_and_linearity(ds32):
    R = pyoracle.representation(ds32.params, ds32.particles[0], ds32.meta[0])
    assert R.shape[1] == 3 and set(np.unique(R[:, 2])) <= {0.0, 1.0}
    R3 = pyoracle.representation(ds32.params, ds32.particles[0], ds32.meta[0], fold=3)
    assert R3.shape == R.shape and (R3[:, 2] == 1).all()  # n-fold: wedge image 1 (fold > 1 branch)
    assert np.array_equal(pyoracle.representation(ds32.params, ds32.particles[0], ds32.meta[0], fold=1), R)
    R2 = pyoracle.representation(ds32.params, 2 * ds32.particles[0], ds32.meta[0])
    assert np.allclose(R2[:, :2], 2 * R[:, :2], rtol=1e-6, atol=1e-6 * np.abs(R[:, :2]).max())


@pytest.mark.gpu
@pytest.mark.parametrize("fold", [2, 3])
def test_gpu_representations_nfold(ds32, fold):
    n = len(ds32.meta)
    m = ProjectionRotationMetric3D(ds32.params)
    try:
        m.set_particles([WedgedSubImage3D(ds32.particles[i], **{k: ds32.meta[i][k] for k in KW}) for i in range(n)])
        g = m.representations([1, 2], fold=fold)
    finally:
        m.close()
    o = np.stack([pyoracle.representation(ds32.params, ds32.particles[i], ds32.meta[i], fold=fold) for i in (1, 2)])
    assert g.shape == o.shape and (g[:, :, 2] == 1).all()
    assert np.abs(g[:, :, :2] - o[:, :, :2]).max() <= 5e-5 * np.abs(o[:, :, :2]).max()


@pytest.mark.gpu
def test_gpu_representations(ds32):
    n = len(ds32.meta)
    m = ProjectionRotationMetric3D(ds32.params)
    try:
        m.set_particles([WedgedSubImage3D(ds32.particles[i], **{k: ds32.meta[i][k] for k in KW}) for i in range(n)])
        g = m.representations([3, 0, 1, 2])
        D = m.representation_distances(g)
    finally:
        m.close()
    o = np.stack([pyoracle.representation(ds32.params, ds32.particles[i], ds32.meta[i]) for i in (3, 0, 1, 2)])
    assert g.shape == o.shape
    assert np.array_equal(g[:, :, 2], o[:, :, 2])
    assert np.abs(g[:, :, :2] - o[:, :, :2]).max() <= 2e-5 * np.abs(o[:, :, :2]).max()
    Do = pyoracle.representation_distances(o, True)
    assert np.allclose(D, Do, rtol=1e-4, atol=1e-6 * Do.max())


def test_oracle_real_representation(ds32):
    """getLowDimensionRepresentationReal (bin factor 1, the image filter's mask): the band-pass-filtered image
    (nbfFourierFilter::executeHalf on a real array: C2R(filter R2C(A shift)) shift / N^3) at the voxels where the
    mask exceeds 0.5, against numpy's FFTs; invariant to an affine change of the input values up to the scale."""
    p = ds32.params
    N = p["N"]
    C = pyoracle.representation_real(p, ds32.particles[0], ds32.meta[0])
    img = pyoracle.get_image(p, ds32.particles[0], ds32.meta[0])  # [x][y][z]
    m, _, f = pyoracle.masks(p)
    x, y, z = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    s = np.where((x + y + z) % 2, -1.0, 1.0)
    F = np.fft.rfftn(img * s) * f
    e = np.fft.irfftn(F, s=(N, N, N), axes=(0, 1, 2)) * s
    expect = e[m > 0.5]
    assert C.shape == expect.shape
    assert np.abs(C - expect).max() <= 1e-9 * np.abs(expect).max()
    C2 = pyoracle.representation_real(p, 3 * ds32.particles[0] + 1.5, ds32.meta[0])
    assert np.abs(C2 - 3 * C).max() <= 1e-6 * np.abs(C).max()


def _rot_z(deg):
    """vtkTransform::RotateZ(deg) as a 4x4 matrix."""
    c, s = np.cos(np.radians(deg)), np.sin(np.radians(deg))
    T = np.eye(4)
    T[:2, :2] = [[c, -s], [s, c]]
    return T


def test_oracle_real_representation_bin_and_fold(ds32):
    """getLowDimensionRepresentationReal's other branches in the oracle: binning by 2 keeps the bin-1 image's values at
    the even indices where the mask at those indices exceeds 0.5; the n-fold branch equals the composition of the
    one-member wedged average (weights 1 / fold, matrix * RotateZ(f * 360 / fold)), the band-pass filter and the
    n-fold symmetrisation of the filtered image."""
    p = ds32.params
    N = p["N"]
    vol, meta = ds32.particles[1], ds32.meta[1]
    m, _, f = pyoracle.masks(p)
    x, y, z = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    s = np.where((x + y + z) % 2, -1.0, 1.0)

    def filt(img):
        return np.fft.irfftn(np.fft.rfftn(img * s) * f, s=(N, N, N), axes=(0, 1, 2)) * s

    e = filt(pyoracle.get_image(p, vol, meta))
    C2 = pyoracle.representation_real(p, vol, meta, bin_factor=2)
    keep = m[::2, ::2, ::2] > 0.5
    assert C2.shape == (int(keep.sum()),)
    assert np.abs(C2 - e[::2, ::2, ::2][keep]).max() <= 1e-9 * np.abs(C2).max()
    fold = 3
    M0 = np.asarray(meta["matrix"], np.float64).reshape(4, 4)
    mats = [M0 @ _rot_z(k * 360.0 / fold) for k in range(fold)]
    avg = pyoracle.average(p, [vol] * fold, [meta] * fold, [np.float32(1.0 / fold)] * fold, mats)
    fa = filt(avg)
    sym = pyoracle.symmetrize(p, np.ascontiguousarray(fa.transpose(2, 1, 0)).astype(np.float32), fold)
    C3 = pyoracle.representation_real(p, vol, meta, fold=fold)
    assert np.abs(C3 - sym[m > 0.5]).max() <= 1e-6 * np.abs(C3).max()


@pytest.mark.gpu
@pytest.mark.parametrize("fold,bin_factor", [(1, 1), (1, 2), (3, 1), (2, 2)])
def test_gpu_representations_real(ds32, fold, bin_factor):
    """ettk_gpu_representations_real against the oracle (FP32 transforms and reslices against FP64): within 5e-5 of
    the largest value for the plain image, 2e-4 through the n-fold branch's average and symmetrisation; the kept voxels
    (how many, in which order) exactly; distances of the depth-1 array bit-exact against the oracle's loop."""
    n = len(ds32.meta)
    m = ProjectionRotationMetric3D(ds32.params)
    try:
        m.set_particles([WedgedSubImage3D(ds32.particles[i], **{k: ds32.meta[i][k] for k in KW}) for i in range(n)])
        g = m.representations_real([2, 0, 3], fold=fold, bin_factor=bin_factor)
        D = m.representation_distances(g)
    finally:
        m.close()
    o = np.stack([pyoracle.representation_real(ds32.params, ds32.particles[i], ds32.meta[i], fold=fold,
                                               bin_factor=bin_factor) for i in (2, 0, 3)])
    assert g.shape == o.shape + (1,)
    tol = 5e-5 if fold == 1 else 2e-4
    assert np.abs(g[:, :, 0] - o).max() <= tol * np.abs(o).max()
    assert np.array_equal(D, pyoracle.representation_distances(g, True))
