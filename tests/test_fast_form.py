"""The fast alignment form (ettk_gpu_align_pairs_refined): coarse SO(3) hit, one CCF per kept peak, batched local
refinement by the analytic gradient of the masked normalised correlation (no counterpart in the reference).

- Objective and gradient against the oracle's FP64 restatement with its analytic FP64 gradient
  (oracle_refined_objective): rho to 1e-4 relative, gradient to 2% of its largest component.
- Gradient against central finite differences of the GPU objective itself (h = 1e-3 rad / 1e-3 voxel), to 5% of
  the largest component (the trilinear interpolant of the band-limited particle is smooth at that scale).
- Alignments: every refined pose scores at least the coarse pose it started from, and on pairs of the 64^3 B=32
  workload the refined poses are at least as close to the generating poses as the plain form's (median rotation
  and shift error), through the same D layout (19 columns with the wedge overlap, extra candidate slots FLT_MAX,
  the resume rule).
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


def metric(ds, n, **extra):
    m = ProjectionRotationMetric3D(dict(ds.params, **extra))
    m.set_references([vol(ds.references[0], ds.ref_meta[0])])
    m.set_particles([vol(ds.particles[i], ds.meta[i]) for i in range(n)])
    return m


def offset_pose(truth, rng, deg=3.0, vox=0.4):
    """The generating pose perturbed by a rotation of `deg` degrees about a random axis and a shift of `vox`."""
    ax = rng.standard_normal(3)
    ax /= np.linalg.norm(ax)
    a = np.radians(deg)
    K = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
    R = np.eye(3) + np.sin(a) * K + (1 - np.cos(a)) * K @ K
    T = np.eye(4)
    T[:3, :3] = truth["rotation"] @ R
    d = rng.standard_normal(3)
    T[:3, 3] = truth["shift"] + vox * d / np.linalg.norm(d)
    return T


def errors(D, ds, off=1):
    rot, sh = [], []
    for i in range(D.shape[0]):
        T = D[i, off:off + 16, 0].reshape(4, 4).astype(np.float64)
        Rt = np.asarray(ds.truth[i]["rotation"])
        c = np.clip((np.trace(T[:3, :3] @ Rt.T) - 1) / 2, -1, 1)
        rot.append(np.degrees(np.arccos(c)))
        sh.append(np.linalg.norm(T[:3, 3] - np.asarray(ds.truth[i]["shift"])))
    return np.array(rot), np.array(sh)


@pytest.fixture(scope="module")
def ds32():
    return synthetic.generate("align32_b16", n_particles=4)


def test_objective_and_gradient_against_fp64_oracle(ds32):
    rng = np.random.default_rng(3)
    n = 3
    poses = [offset_pose(ds32.truth[i], rng) for i in range(n)]
    theta = np.array([[0.01, -0.02, 0.015, 0.2, -0.1, 0.3], [0, 0, 0, 0, 0, 0], [-0.03, 0.01, 0.0, -0.4, 0.2, 0.0]])
    m = metric(ds32, n)
    try:
        rho, g = m.refined_objective([(0, i) for i in range(n)], poses, theta)
    finally:
        m.close()
    for i in range(n):
        ro, go = pyoracle.refined_objective(ds32.params, ds32.references[0], ds32.ref_meta[0], ds32.particles[i],
                                            ds32.meta[i], poses[i], theta[i])
        assert abs(rho[i] - ro) <= 1e-4 * abs(ro), (rho[i], ro)
        assert np.abs(g[i] - go).max() <= 2e-2 * np.abs(go).max(), (g[i], go)


def test_gradient_against_central_differences(ds32):
    rng = np.random.default_rng(4)
    n = 2
    poses = [offset_pose(ds32.truth[i], rng) for i in range(n)]
    h = 1e-3
    m = metric(ds32, n)
    try:
        pairs = [(0, i) for i in range(n)]
        rho0, g = m.refined_objective(pairs, poses, np.zeros((n, 6)))
        fd = np.zeros((n, 6))
        for k in range(6):
            th = np.zeros((n, 6))
            th[:, k] = h
            rp = m.refined_objective(pairs, poses, th, grad=False)
            rm = m.refined_objective(pairs, poses, -th, grad=False)
            fd[:, k] = (rp - rm) / (2 * h)
    finally:
        m.close()
    for i in range(n):
        assert np.abs(fd[i] - g[i]).max() <= 5e-2 * np.abs(g[i]).max(), (fd[i], g[i])


@pytest.fixture(scope="module")
def ds64():
    return synthetic.generate("align64_b32", n_particles=24)


@pytest.mark.parametrize("coarse", [0, 1, 2])
def test_fast_form_against_plain_form(ds64, coarse):
    """The fast form (coarse = 1: its SO(3) search on the half grid at B/2, split-BF16 Wigner contraction; 2: the
    screened candidates also resampled trilinearly) against
    the plain form on the same pairs: refined rows score at least their coarse start, and the median errors against
    the generating poses are no worse than the plain grid's over the pairs the grid puts in the right basin."""
    n = 24
    pairs = [(0, i) for i in range(n)]
    m = metric(ds64, n)
    mf = metric(ds64, n, fast_coarse_so3=coarse, wigner_precision=2 if coarse else 0)
    try:
        Dp = m.getDistances(pairs)
        D0 = mf.getDistancesRefined(pairs, iterations=0)
        Df = mf.getDistancesRefined(pairs, cols=19, ncand=2, iterations=16)
    finally:
        m.close()
        mf.close()
    assert np.all(Df[:, 0, 1] == np.finfo(np.float32).max)
    assert np.all(Df[:, 1, 0] == 1.0)
    assert np.all((Df[:, 2, 0] > 0) & (Df[:, 2, 0] <= 1.0))
    # refined poses score at least the coarse pose they start from (1 - rho, rho with the same filtered reference)
    assert np.all(Df[:, 0, 0] <= D0[:, 0, 0] + 1e-6)
    rp, sp = errors(Dp, ds64)
    rf, sf = errors(Df, ds64, off=3)
    hit = rp < 20.0
    assert hit.sum() >= n // 2
    assert np.median(rf[hit]) <= np.median(rp[hit]), (np.median(rf[hit]), np.median(rp[hit]))
    assert np.median(sf[hit]) <= np.median(sp[hit]), (np.median(sf[hit]), np.median(sp[hit]))


def test_fast_form_resume_rule(ds64):
    n = 6
    D = -np.ones((n, 17, 1), np.float32)
    D[2] = 5.0
    m = metric(ds64, n)
    try:
        D = m.getDistancesRefined([(0, i) for i in range(n)], D=D, iterations=4)
    finally:
        m.close()
    assert np.all(D[2] == 5.0)
    others = [i for i in range(n) if i != 2]
    assert np.all(D[others, 0, 0] < 1.0)


def _rodrigues(w):
    t = np.linalg.norm(w)
    if t == 0:
        return np.eye(3)
    k = w / t
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + np.sin(t) * K + (1 - np.cos(t)) * K @ K


def _ascend(m, pair, T, radius, iters=30):
    """Gradient ascent of the fast form's objective from pose T (step rule of the library's optimizer), evaluated
    through the C ABI; returns the final pose and rho."""
    rho, g = m.refined_objective([pair], [T], np.zeros((1, 6)))
    rho, g = rho[0], g[0]
    alpha = 0.5
    for _ in range(iters):
        gu = np.concatenate([g[:3] / radius, g[3:]])
        nrm = np.linalg.norm(gu)
        if not nrm > 0 or alpha < 1e-3:
            break
        Q = np.eye(4)
        Q[:3, :3] = _rodrigues(gu[:3] / nrm * alpha / radius)
        Q[:3, 3] = gu[3:] / nrm * alpha
        Tt = T @ Q
        rt, gt = m.refined_objective([pair], [Tt], np.zeros((1, 6)))
        if rt[0] > rho:
            T, rho, g, alpha = Tt, rt[0], gt[0], min(alpha * 1.6, 4.0)
        else:
            alpha *= 0.35
    return T, rho


def test_error_floor_of_the_objective():
    """Where the objective itself puts the pose at this signal-to-noise ratio: ascent started at the generating
    poses of the continuous-pose, sub-voxel-shift workload ends away from them, at a correlation at least that of
    the generating pose; the fast form's poses lie within twice that floor's median error of the generating ones.
    The floor (printed) bounds what any optimiser of this objective can reach on these data."""
    ds = synthetic.generate("refine64_b32", n_particles=16)
    n = 16
    m = metric(ds, n)
    radius = 0.6 * ds.params["mask_radius"]
    try:
        floor_rot, floor_sh = [], []
        for i in range(n):
            T0 = np.eye(4)
            T0[:3, :3] = ds.truth[i]["rotation"]
            T0[:3, 3] = ds.truth[i]["shift"]
            r0 = m.refined_objective([(0, i)], [T0], np.zeros((1, 6)), grad=False)[0]
            T, rho = _ascend(m, (0, i), T0, radius)
            assert rho >= r0
            c = np.clip((np.trace(T[:3, :3] @ T0[:3, :3].T) - 1) / 2, -1, 1)
            floor_rot.append(np.degrees(np.arccos(c)))
            floor_sh.append(np.linalg.norm(T[:3, 3] - T0[:3, 3]))
        Df = m.getDistancesRefined([(0, i) for i in range(n)], iterations=16)
    finally:
        m.close()
    rf, sf = errors(Df, ds)
    hit = rf < 20.0
    fr, fs = float(np.median(floor_rot)), float(np.median(floor_sh))
    print("objective error floor: median %.3f deg, %.3f voxel; fast form: %.3f deg, %.3f voxel"
          % (fr, fs, np.median(rf[hit]), np.median(sf[hit])))
    assert hit.sum() >= n // 2
    assert np.median(rf[hit]) <= 2.0 * fr + 0.5
    assert np.median(sf[hit]) <= 2.0 * fs + 0.1
