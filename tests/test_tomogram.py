"""Particles cut from a tomogram (nbfWedgedSubImage3D::getImage's tomogram branch,
inc/em/nbfWedgedSubImage3D.h:602-828): the GPU reslices every particle straight out of one tomogram at its
position / cut offset; the oracle cuts the same tomogram with the same metadata.

The synthetic tomogram holds four 32^3 particles over seeded noise: one at an integer position, one at a
fractional position, one with a cut offset, and one whose box leaves the tomogram on two sides (voxels
outside take the mean of the inside, as in the reference). Two widths: 112 (rows of 16-byte multiples,
bulk-tensor staging) and 110 (per-tap global loads). Tolerances are those of the fixed-image parity tests:
spherical projections 1e-4 of the maximum, distances 1e-4 relative, rotations 1e-5, shifts 1e-4, class
average 1e-5 relative RMS."""
import numpy as np
import pytest

import pyoracle
from ettk_gb300 import synthetic
from ettk_gb300.metric import ProjectionRotationMetric3D, WedgedSubImage3D

pytestmark = pytest.mark.gpu

N = 32
# (box origin x, y, z pasted into the tomogram, position offset, cut offset)
PLACES = [((2, 20, 8), (0.0, 0.0, 0.0), 0.0),
          ((38, 20, 8), (0.25, -0.5, 0.0), 0.0),
          ((74, 20, 8), (0.0, 0.0, 1.5), 1.5),
          ((-6, -4, 4), (0.0, 0.0, 0.0), 0.0)]


def make_tomogram(ds, nx, ny=72, nz=48, seed=11):
    rng = np.random.default_rng(seed)
    t = 0.3 * rng.standard_normal((nz, ny, nx)).astype(np.float32)
    metas = []
    for i, ((ox, oy, oz), d, cut) in enumerate(PLACES):
        src = ds.particles[i]
        zs, ys, xs = (slice(max(0, -o), min(N, n - o)) for o, n in ((oz, nz), (oy, ny), (ox, nx)))
        zd, yd, xd = (slice(max(0, o), min(n, o + N)) for o, n in ((oz, nz), (oy, ny), (ox, nx)))
        t[zd, yd, xd] += src[zs, ys, xs]
        m = dict(ds.meta[i])
        m["position"] = (ox + N / 2 + d[0], oy + N / 2 + d[1], oz + N / 2 + d[2])
        m["cut_offset"] = cut
        metas.append(m)
    return t, metas


@pytest.fixture(scope="module")
def ds32():
    return synthetic.generate("align32_b16", n_particles=len(PLACES))


@pytest.mark.parametrize("nx", [112, 110])
def test_tomogram_parity(ds32, nx):
    tomo, metas = make_tomogram(ds32, nx)
    n = len(metas)
    m = ProjectionRotationMetric3D(ds32.params)
    try:
        ref = ds32.ref_meta[0]
        m.set_references([WedgedSubImage3D(ds32.references[0], **{k: ref[k] for k in
                                                                   ("lwedge", "uwedge", "normal", "matrix",
                                                                    "position", "cut_offset")})])
        m.set_particles_tomogram(tomo, metas)
        proj = [m.spherical_projection(0, p) for p in range(n)]
        D = m.getDistances([(0, p) for p in range(n)])
        mats = []
        for i in range(n):
            T = np.eye(4)
            T[:3, :3] = ds32.truth[i]["rotation"]
            T[:3, 3] = ds32.truth[i]["shift"]
            mats.append(T)
        weights = [1.0, 0.5, 1.0, 0.75]
        avg = m.average(list(range(n)), weights, mats)
    finally:
        m.close()
    for p in range(n):
        o = pyoracle.spherical_projection(ds32.params, tomo, metas[p])
        assert np.abs(proj[p] - o).max() <= 1e-4 * np.abs(o).max(), p
    for p in range(n):
        o = pyoracle.align(ds32.params, ds32.references[0], ds32.ref_meta[0], tomo, metas[p])
        T = D[p, 1:17, 0].reshape(4, 4)
        assert abs(D[p, 0, 0] - o["distance"]) <= 1e-4 * abs(o["distance"]), p
        assert np.allclose(T[:3, :3], o["matrix"][:3, :3], atol=1e-5), p
        assert np.allclose(T[:3, 3], o["matrix"][:3, 3], atol=1e-4), p
    o = pyoracle.average(ds32.params, [tomo] * n, metas, weights, mats).transpose(2, 1, 0)
    err = np.sqrt(np.mean((avg - o) ** 2)) / np.sqrt(np.mean(o ** 2))
    assert err <= 1e-5, err


def test_tomogram_rejects_bad_input(ds32):
    m = ProjectionRotationMetric3D(ds32.params)
    try:
        tomo, metas = make_tomogram(ds32, 112)
        bad = tomo.copy()
        bad[3, 4, 5] = np.nan
        with pytest.raises(Exception):
            m.set_particles_tomogram(bad, metas)
        with pytest.raises(Exception):
            m.set_particles_tomogram(tomo, [])
    finally:
        m.close()
