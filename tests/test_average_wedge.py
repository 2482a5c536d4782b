"""Spherical missing wedge of a class average (nbfWedgedAverageImage3D::updateAccumulatedSphericalWedgeImageMPI and
updateSphericalWedgeImage, inc/em/nbfWedgedAverageImage3D.h:612-665) and its use as a reference's wedge in the
SO(3) stage (nbfWedge3D::setSphericalImage as the MRA loop transfers it, inc/em/nbfLoopClustering.h:1270-1278).

The member counts are integer work: GPU and oracle must agree exactly (same float cos / sin tables, the plane
products in FP64 in the reference's order). An alignment against a reference carrying such a wedge is held
to the tolerances of the other alignment parity tests (distance 1e-4 relative, rotation 1e-5, shift 1e-4)."""
import numpy as np
import pytest

import pyoracle
from ettk_gb300 import synthetic
from ettk_gb300.metric import ProjectionRotationMetric3D, WedgedSubImage3D

KW = ("lwedge", "uwedge", "normal", "matrix", "position", "cut_offset")


def vol(img, meta):
    return WedgedSubImage3D(img, **{k: meta[k] for k in KW})


def analytic_wedge(lw, uw, B):
    """Binary spherical wedge of an unrotated volume (nbfWedge3D::set normals, getSphericalImage formula)."""
    n = 2 * B
    a1, a2 = np.deg2rad(90.0 - uw), np.deg2rad(90.0 - lw)
    n1 = np.array([np.cos(-a1), 0.0, -np.sin(-a1)])
    n2 = np.array([np.cos(-a2), 0.0, -np.sin(-a2)])
    phiK, thetaK = np.float32(np.pi / (n - 1)), np.float32(2 * np.pi / (n - 1))
    k = np.arange(n, dtype=np.float32)
    cj, sj = np.cos(k * thetaK).astype(np.float64), np.sin(k * thetaK).astype(np.float64)
    si, ci = np.sin(k * phiK).astype(np.float64), np.cos(k * phiK).astype(np.float64)
    a = n1[0] * cj[None, :] * si[:, None] + n1[1] * sj[None, :] * si[:, None] + n1[2] * ci[:, None]
    b = n2[0] * cj[None, :] * si[:, None] + n2[1] * sj[None, :] * si[:, None] + n2[2] * ci[:, None]
    return (a * b <= 0).astype(np.float32)


def members(ds, n):
    mats = []
    for i in range(n):
        T = np.eye(4)
        T[:3, :3] = ds.truth[i]["rotation"]
        T[:3, 3] = ds.truth[i]["shift"]
        mats.append(T)
    return mats


@pytest.fixture(scope="module")
def ds32():
    return synthetic.generate("align32_b16", n_particles=8)


def test_oracle_single_member_is_its_wedge():
    # one unrotated member: count = its binary wedge, max 1, and the average keeps exactly that wedge
    B = 16
    p = synthetic.default_params(synthetic.WORKLOADS["align32_b16"])
    v = np.zeros((32, 32, 32), np.float32)
    meta = {"lwedge": -55.0, "uwedge": 65.0, "position": (16.0, 16.0, 16.0)}
    w, c = pyoracle.average_spherical_wedge(p, [v], [meta], [1.0], [np.eye(4)])
    e = analytic_wedge(-55.0, 65.0, B)
    assert np.array_equal(c, e) and np.array_equal(w, e)


def test_oracle_zero_weights_skipped_and_full_wedges_count():
    p = synthetic.default_params(synthetic.WORKLOADS["align32_b16"])
    v = np.zeros((32, 32, 32), np.float32)
    part = {"lwedge": -60.0, "uwedge": 60.0, "position": (16.0, 16.0, 16.0)}
    full = {"lwedge": -90.0, "uwedge": 90.0, "position": (16.0, 16.0, 16.0)}
    _, c = pyoracle.average_spherical_wedge(p, [v, v, v], [part, full, part], [1.0, 1.0, 0.0], [np.eye(4)] * 3)
    assert np.array_equal(c, analytic_wedge(-60.0, 60.0, 16) + 1)


@pytest.mark.gpu
def test_average_spherical_wedge(ds32):
    n = len(ds32.meta)
    weights = [1.0, 0.5, 1.0, 0.0, -0.25, 1.0, 1.0, 1.0]
    mats = members(ds32, n)
    m = ProjectionRotationMetric3D(ds32.params)
    try:
        m.set_particles([vol(ds32.particles[i], ds32.meta[i]) for i in range(n)])
        g, gc = m.average_spherical_wedge(list(range(n)), weights, mats)
    finally:
        m.close()
    o, oc = pyoracle.average_spherical_wedge(ds32.params, [ds32.particles[i] for i in range(n)],
                                             [ds32.meta[i] for i in range(n)], weights, mats)
    assert np.array_equal(gc, oc)
    assert np.array_equal(g, o)
    assert 0 < g.sum() < g.size  # the members' rotated wedges leave a partial wedge


@pytest.mark.gpu
def test_reference_with_average_wedge(ds32):
    n = len(ds32.meta)
    mats = members(ds32, n)
    w, _ = pyoracle.average_spherical_wedge(ds32.params, [ds32.particles[i] for i in range(n)],
                                            [ds32.meta[i] for i in range(n)], [1.0] * n, mats)
    m = ProjectionRotationMetric3D(ds32.params)
    try:
        m.set_references([vol(ds32.references[0], ds32.ref_meta[0])])
        m.set_reference_spherical_wedge(0, w)
        m.set_particles([vol(ds32.particles[i], ds32.meta[i]) for i in range(3)])
        D = m.getDistances([(0, p) for p in range(3)])
    finally:
        m.close()
    ref_meta = dict(ds32.ref_meta[0])
    ref_meta["spherical_wedge"] = w
    for p in range(3):
        o = pyoracle.align(ds32.params, ds32.references[0], ref_meta, ds32.particles[p], ds32.meta[p])
        assert o["use_window1"] == 1
        T = D[p, 1:17, 0].reshape(4, 4)
        assert abs(D[p, 0, 0] - o["distance"]) <= 1e-4 * abs(o["distance"]), p
        assert np.allclose(T[:3, :3], o["matrix"][:3, :3], atol=1e-5), p
        assert np.allclose(T[:3, 3], o["matrix"][:3, 3], atol=1e-4), p


@pytest.mark.gpu
def test_set_reference_spherical_wedge_rejects_bad_input(ds32):
    m = ProjectionRotationMetric3D(ds32.params)
    try:
        m.set_references([vol(ds32.references[0], ds32.ref_meta[0])])
        bad = np.ones((32, 32), np.float32)
        bad[1, 2] = np.nan
        with pytest.raises(Exception):
            m.set_reference_spherical_wedge(0, bad)
        with pytest.raises(Exception):
            m.set_reference_spherical_wedge(1, np.ones((32, 32), np.float32))
    finally:
        m.close()
