"""Oracle checks (CPU): the FP64 restatement against the reference's own SOFT 1.0 (compiled from
the reference sources under oracle/_ref when the reference tree is present), against numpy's FFT,
and against the committed golden fixtures (tests/golden, made by tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

import pyoracle

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_fft_matches_numpy():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((8, 16, 32))
    X = pyoracle.rfft3d(x)
    assert np.abs(X - np.fft.rfftn(x)).max() < 1e-10
    y = pyoracle.irfft3d(X, 32)
    assert np.abs(y - x * x.size).max() < 1e-8


def test_c2r_ignores_imaginary_nyquist_terms():
    # FFTW hc2r semantics on the last axis: Im of the k=0 and k=n/2 terms (after the leading-axis
    # inverse transforms) does not reach the output
    rng = np.random.default_rng(1)
    X = rng.standard_normal((4, 4, 5)) + 1j * rng.standard_normal((4, 4, 5))
    y = pyoracle.irfft3d(X, 8)
    Z = np.fft.ifft(np.fft.ifft(X, axis=0), axis=1) * 16
    Z[..., 0] = Z[..., 0].real
    Z[..., 4] = Z[..., 4].real
    ref = np.fft.irfft(Z, 8, axis=2) * 8
    assert np.abs(y - ref).max() < 1e-9


@pytest.mark.parametrize("B", [4, 8, 16])
def test_so3_against_soft_library(B):
    R = pyoracle.ref_lib()
    if R is None:
        pytest.skip("SOFT reference library not built (reference tree absent)")
    n = 2 * B
    rng = np.random.default_rng(B)
    F1 = rng.standard_normal((n, n))
    F2 = rng.standard_normal((n, n))
    C = pyoracle.soft(B, F1, F2)
    Cr = np.zeros((n, n, n))
    R.ref_soft(B, F1, F2, Cr)
    assert np.abs(C - Cr).max() <= 1e-9 * np.abs(Cr).max()
    Rm = pyoracle.rotate(B, F1, 0.4, 1.1, 2.3)
    Rr = np.zeros((n, n))
    R.ref_rotate(B, F1, 0.4, 1.1, 2.3, Rr)
    assert np.abs(Rm - Rr).max() <= 1e-9 * np.abs(Rr).max()
    cR = np.zeros(B * B)
    cI = np.zeros(B * B)
    R.ref_fst(B, F1, cR, cI)
    c = pyoracle.sht(B, F1)
    idx = 0
    for m in range(B):
        for l in range(m, B):
            assert abs(c[l, m + B] - (cR[idx] + 1j * cI[idx])) < 1e-9 * (1 + abs(c[l, m + B]))
            idx += 1


def _golden(name):
    p = os.path.join(GOLD, name)
    if not os.path.exists(p):
        pytest.skip("golden fixture %s missing" % name)
    return np.load(p, allow_pickle=False)


def test_soft_fixture_vectors():
    """SOFT's own S^2 test signal (randomS2sig_bw8.dat) through the reference SOFT build: the oracle
    reproduces the stored correlation and rotation outputs."""
    g = _golden("soft_bw8.npz")
    B = 8
    C = pyoracle.soft(B, g["sig"], g["pat"])
    assert np.abs(C - g["C"]).max() <= 1e-9 * np.abs(g["C"]).max()
    Rm = pyoracle.rotate(B, g["sig"], *g["angles"])
    assert np.abs(Rm - g["R"]).max() <= 1e-9 * np.abs(g["R"]).max()


def test_alignment_golden():
    """Frozen oracle outputs for the 32^3 B=16 workload (first particles); pins the oracle against
    accidental changes."""
    g = _golden("align32_b16.npz")
    from ettk_gb300 import synthetic
    ds = synthetic.generate("align32_b16", n_particles=int(g["n"]))
    import hashlib
    assert hashlib.sha256(ds.particles.tobytes()).hexdigest() == str(g["particles_sha256"])
    for i in range(int(g["n"])):
        o = pyoracle.align(ds.params, ds.references[0], ds.ref_meta[0], ds.particles[i], ds.meta[i])
        assert abs(o["distance"] - g["distance"][i]) <= 1e-6 * abs(g["distance"][i])
        assert np.allclose(o["matrix"], g["matrix"][i], atol=1e-9)


def test_ccf_restriction_zero_scores_the_pose():
    """getDistances type 2 at translation restriction 0 (doMra's scoring): the restriction is max(0 * 2, 1) = 1 on
    the 2x grid (inc/em/nbfFourierImageMetric.h:1224-1225), so the shift moves by at most half a voxel per axis;
    with the search open (restriction 6) the same offset pose is pulled back by about the 2-voxel offset."""
    from ettk_gb300 import synthetic
    ds = synthetic.generate("align32_b16", n_particles=1)
    T = np.eye(4)
    T[:3, :3] = ds.truth[0]["rotation"]
    T[:3, 3] = ds.truth[0]["shift"]
    T[0, 3] += 2.0
    p0 = dict(ds.params, restrict_translation=0.0)
    d0, t0 = pyoracle.ccf(p0, ds.references[0], ds.ref_meta[0], ds.particles[0], ds.meta[0], T)
    d6, t6 = pyoracle.ccf(ds.params, ds.references[0], ds.ref_meta[0], ds.particles[0], ds.meta[0], T)
    assert np.abs(t0[:3, 3] - T[:3, 3]).max() <= 0.5
    assert t6[0, 3] - T[0, 3] < -1.5
    assert d6 < d0


def _ellipsoid(M, a, b, c):
    """A binary ellipsoid in a cube of edge M, [z][y][x] (x fastest, as a mask file holds it), values 0 / 1.5."""
    z, y, x = np.mgrid[0:M, 0:M, 0:M] - M / 2.0
    return np.where((x / a) ** 2 + (y / b) ** 2 + (z / c) ** 2 <= 1.0, 1.5, 0.0).astype(np.float32)


def test_file_mask_centring_binarising_softening():
    """buildMaskFromFile + softenMask (inc/em/nbfImageFilter.h:319-381, 474-494) as the oracle restates them: a
    larger mask gives the same m1 as its centred crop, a smaller one the same as its zero-padded centring, values
    above the threshold only count (binarised), the result is softened with the mask sigma, and M = N - 1 (where the
    reference indexes outside the mask) is refused."""
    params = {"N": 32, "B": 16, "mask_radius": 11.0, "mask_sigma": 2.0, "square_mask_size": 2.0, "bp_low": .01,
              "bp_high": .5, "bp_low_sigma": .01, "bp_high_sigma": .05, "restrict_translation": 6.0,
              "restrict_rotation": 180.0, "candidate_peaks": 5, "number_of_candidates": 1,
              "wedge_compensation": True, "overlap_normalized": True}
    N = params["N"]
    big = _ellipsoid(N + 8, 11.0, 9.0, 12.0)
    m_big = pyoracle.file_mask(params, big, 0.5)
    m_crop = pyoracle.file_mask(params, big[4:4 + N, 4:4 + N, 4:4 + N], 0.5)
    assert np.array_equal(m_big, m_crop)
    small = _ellipsoid(N - 8, 8.0, 7.0, 9.0)
    padded = np.zeros((N, N, N), np.float32)
    padded[4:4 + N - 8, 4:4 + N - 8, 4:4 + N - 8] = small
    assert np.array_equal(pyoracle.file_mask(params, small, 0.5), pyoracle.file_mask(params, padded, 0.5))
    # binarised: scaling the values above the threshold changes nothing; a threshold above them empties the mask
    assert np.array_equal(pyoracle.file_mask(params, 7.0 * big, 0.5), m_big)
    assert not pyoracle.file_mask(params, big, 2.0).any()
    # softened: without the Gaussian the mask is the binary ellipsoid itself ([x][y][z] order)
    hard = pyoracle.file_mask(dict(params, mask_sigma=0.0), big[4:4 + N, 4:4 + N, 4:4 + N], 0.5)
    assert np.array_equal(hard, (big[4:4 + N, 4:4 + N, 4:4 + N] > 0.5).astype(np.float32).transpose(2, 1, 0))
    assert m_big.min() >= 0.0 and m_big.max() <= 1.0 + 1e-6
    assert ((m_big > 0.01) & (m_big < 0.99)).any()  # a soft edge
    assert np.abs(m_big.sum() - hard.sum()) < 1e-3 * hard.sum()  # the smoothing keeps the mass (interior mask)
    with pytest.raises(ValueError):
        pyoracle.file_mask(params, _ellipsoid(N - 1, 8.0, 7.0, 9.0), 0.5)
