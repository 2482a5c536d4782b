"""Continuous 6-DOF pose refinement (the hand-written adjoint; no counterpart in the reference, whose refine()
is a Powell search over RotateX/Y/Z with one CCF per step).

Gradient checks at poses off the optimum (ground truth perturbed by 3 degrees and 0.3 voxel):
  * against the FP64 host gradient: central differences (h = 1e-4 rad / voxel) of the oracle's FP64
    restatement of the same objective; agreement to 2% of the gradient norm (the GPU path is FP32);
  * against central differences of the GPU objective itself (h = 1e-3), 3% of the gradient norm;
  * the objective value against the oracle's to 1e-4.
Refinement: the line search only accepts improvements, so rho never decreases; on particles whose grid hit
is in the right basin the median rotation error against ground truth drops.
"""
import numpy as np
import pytest

import pyoracle
from ettk_gb300 import synthetic
from ettk_gb300.metric import ProjectionRotationMetric3D, WedgedSubImage3D

pytestmark = pytest.mark.gpu

KW = ("lwedge", "uwedge", "normal", "matrix", "position", "cut_offset")


def vol(img, meta):
    return WedgedSubImage3D(img, **{k: meta[k] for k in KW})


def rot(axis, deg):
    a = np.asarray(axis, float)
    a /= np.linalg.norm(a)
    t = np.radians(deg)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(t) * K + (1 - np.cos(t)) * K @ K


def truth_pose(ds, i):
    T = np.eye(4)
    T[:3, :3] = ds.truth[i]["rotation"]
    T[:3, 3] = ds.truth[i]["shift"]
    return T


def rot_err_deg(T, ds, i):
    c = np.clip((np.trace(T[:3, :3] @ np.asarray(ds.truth[i]["rotation"]).T) - 1) / 2, -1, 1)
    return np.degrees(np.arccos(c))


@pytest.fixture(scope="module")
def ds32():
    return synthetic.generate("align32_b16", n_particles=3)


def test_refine_gradient(ds32):
    n = 3
    m = ProjectionRotationMetric3D(ds32.params)
    try:
        m.set_references([vol(ds32.references[0], ds32.ref_meta[0])])
        m.set_particles([vol(ds32.particles[i], ds32.meta[i]) for i in range(n)])
        idx = [(0, i) for i in range(n)]
        poses = []
        for i in range(n):
            T = truth_pose(ds32, i)
            T[:3, :3] = T[:3, :3] @ rot([1, 2, 3][i:] + [1, 2, 3][:i], 3.0)
            T[:3, 3] += 0.3
            poses.append(T)
        rho, g = m.refine_objective(idx, poses, np.zeros((n, 6)))
        gfd = np.zeros((n, 6))
        h = 1e-3
        for k in range(6):
            th = np.zeros((n, 6))
            th[:, k] = h
            rp = m.refine_objective(idx, poses, th, grad=False)
            th[:, k] = -h
            gfd[:, k] = (rp - m.refine_objective(idx, poses, th, grad=False)) / (2 * h)
    finally:
        m.close()
    args = (ds32.params, ds32.references[0], ds32.ref_meta[0])
    for i in range(n):
        r64 = pyoracle.refine_objective(*args, ds32.particles[i], ds32.meta[i], poses[i], np.zeros(6))
        assert abs(rho[i] - r64) <= 1e-4
        g64 = np.zeros(6)
        h64 = 1e-4
        for k in range(6):
            th = np.zeros(6)
            th[k] = h64
            rp = pyoracle.refine_objective(*args, ds32.particles[i], ds32.meta[i], poses[i], th)
            th[k] = -h64
            g64[k] = (rp - pyoracle.refine_objective(*args, ds32.particles[i], ds32.meta[i], poses[i], th)) / (2 * h64)
        assert np.linalg.norm(g[i] - g64) <= 2e-2 * np.linalg.norm(g64), (i, g[i], g64)
        assert np.linalg.norm(gfd[i] - g[i]) <= 3e-2 * np.linalg.norm(g[i]), (i, gfd[i], g[i])


def test_refine_improves_alignment():
    n = 12
    ds = synthetic.generate("align64_b32", n_particles=n)
    m = ProjectionRotationMetric3D(ds.params)
    try:
        m.set_references([vol(ds.references[0], ds.ref_meta[0])])
        m.set_particles([vol(ds.particles[i], ds.meta[i]) for i in range(n)])
        idx = [(0, i) for i in range(n)]
        D = m.getDistances(idx)
        coarse = [D[i, 1:17, 0].reshape(4, 4).astype(np.float64) for i in range(n)]
        rho0 = m.refine_objective(idx, coarse, np.zeros((n, 6)), grad=False)
        D2 = m.refine(idx, D.copy(), iterations=15)
    finally:
        m.close()
    rho1 = 1.0 - D2[:, 0, 0].astype(np.float64)
    assert np.all(rho1 >= rho0 - 1e-5)
    e0 = np.array([rot_err_deg(coarse[i], ds, i) for i in range(n)])
    e1 = np.array([rot_err_deg(D2[i, 1:17, 0].reshape(4, 4), ds, i) for i in range(n)])
    good = e0 < 20.0  # grid hit in the right basin
    assert good.sum() >= n // 2
    assert np.median(e1[good]) < np.median(e0[good])
