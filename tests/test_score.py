"""getDistances with typeOfMetric 2 on the GPU (ettk_gpu_score_pairs): one translational CCF per pair at the
particle's own alignment matrix (nbfFourierImageMetricCore, inc/em/nbfFourierImageMetricCore.h:35-66), as doMra
scores every volume under every reference's alignment with the translation restriction set to 0
(inc/em/nbfLoopClustering.h:1523-1592). Against the oracle's executeFourierNewHalf at the identity transform of
the same volume: distance within 1e-4 relative, the same half-voxel shift, the wedge overlap of 19-column rows
within 1e-4, and doMra's class choice from the scores.
"""
import numpy as np
import pytest

import pyoracle
from ettk_gb300 import synthetic
from ettk_gb300.metric import ProjectionRotationMetric3D, WedgedSubImage3D

pytestmark = pytest.mark.gpu

KW = ("lwedge", "uwedge", "normal", "position", "cut_offset")


def _duplicates(ds, n, rng):
    """Each of the first n particles under its generating pose and under a pose 6 degrees and 1 voxel off it."""
    metas, parts = [], []
    for i in range(n):
        for off in (0.0, 1.0):
            ax = rng.standard_normal(3)
            ax /= np.linalg.norm(ax)
            a = np.radians(6.0) * off
            K = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
            T = np.eye(4)
            T[:3, :3] = ds.truth[i]["rotation"] @ (np.eye(3) + np.sin(a) * K + (1 - np.cos(a)) * K @ K)
            T[:3, 3] = np.asarray(ds.truth[i]["shift"]) + off * np.array([1.0, 0.0, 0.0])
            meta = {k: ds.meta[i][k] for k in KW}
            meta["matrix"] = T
            metas.append(meta)
            parts.append(i)
    return metas, parts


@pytest.mark.parametrize("restrict", [0.0, -1.0])
def test_score_pairs_against_oracle(restrict):
    ds = synthetic.generate("align32_b16", n_particles=4)
    rng = np.random.default_rng(17)
    metas, parts = _duplicates(ds, 4, rng)
    m = ProjectionRotationMetric3D(ds.params)
    try:
        m.set_references([WedgedSubImage3D(ds.references[0], **{k: ds.ref_meta[0][k] for k in KW + ("matrix",)})])
        m.set_particles([WedgedSubImage3D(ds.particles[parts[v]], **metas[v]) for v in range(len(metas))])
        D = m.getDistances([(0, v) for v in range(len(metas))], cols=19, typeOfMetric=2, restrict_translation=restrict)
    finally:
        m.close()
    params = dict(ds.params)
    if restrict >= 0:
        params["restrict_translation"] = restrict
    for v, meta in enumerate(metas):
        d, t = pyoracle.ccf(params, ds.references[0], ds.ref_meta[0], ds.particles[parts[v]], meta, np.eye(4))
        T = D[v, 3:19, 0].reshape(4, 4)
        assert abs(D[v, 0, 0] - d) <= 1e-4 * abs(d), (v, D[v, 0, 0], d)
        assert np.allclose(T[:3, 3], t[:3, 3], atol=1e-6), (v, T[:3, 3], t[:3, 3])
        if restrict == 0.0:
            assert np.allclose(T, np.eye(4))
        assert D[v, 1, 0] == 1.0
        ov = pyoracle.wedge_overlap(params, ds.references[0], ds.ref_meta[0], ds.particles[parts[v]], meta, T)
        assert abs(D[v, 2, 0] - ov) <= 1e-4 * ov


def test_mra_scoring_and_class_choice():
    """doMra's scoring of every duplicate against every reference, then its class choice (ettk_gpu_mra_assign)."""
    from ettk_gb300 import clustering
    ds = synthetic.generate("mra32_b16", n_particles=6)
    R = len(ds.references)
    metas = []
    for i in range(6):  # volume i duplicated under an alignment per reference (its generating pose for every one)
        for r in range(R):
            meta = {k: ds.meta[i][k] for k in KW}
            T = np.eye(4)
            T[:3, :3] = ds.truth[i]["rotation"]
            T[:3, 3] = ds.truth[i]["shift"]
            meta["matrix"] = T
            metas.append(meta)
    m = ProjectionRotationMetric3D(ds.params)
    try:
        m.set_references([WedgedSubImage3D(ref, **{k: rm[k] for k in KW + ("matrix",)})
                          for ref, rm in zip(ds.references, ds.ref_meta)])
        m.set_particles([WedgedSubImage3D(ds.particles[v // R], **metas[v]) for v in range(len(metas))])
        pairs = [(j, v) for v in range(len(metas)) for j in range(R)]
        D = m.getDistances(pairs, typeOfMetric=2, restrict_translation=0.0)
    finally:
        m.close()
    S = D[:, 0, 0].reshape(6, R, R)  # S[v][r][j]: duplicate (v, r) against reference j
    params = dict(ds.params, restrict_translation=0.0)
    So = np.zeros_like(S)
    for v in range(6):
        for r in range(R):
            for j in range(R):
                So[v, r, j], _ = pyoracle.ccf(params, ds.references[j], ds.ref_meta[j], ds.particles[v],
                                              metas[v * R + r], np.eye(4))
    assert np.all(np.abs(S - So) <= 1e-4 * np.abs(So))
    assert np.array_equal(clustering.mra_assign(S), clustering.mra_assign(So))


def test_metric_types_zero_and_one():
    """getDistances' other metric types route to the batched forms: type 0 (refinement on) is getDistancesRefined,
    type 1 (refinement from the own alignment) is the type-2 CCF followed by refine; same rows bit for bit."""
    ds = synthetic.generate("align32_b16", n_particles=3)
    m = ProjectionRotationMetric3D(ds.params)
    try:
        m.set_references([WedgedSubImage3D(ds.references[0], **{k: ds.ref_meta[0][k] for k in KW + ("matrix",)})])
        m.set_particles([WedgedSubImage3D(ds.particles[i], **{k: ds.meta[i][k] for k in KW + ("matrix",)})
                         for i in range(3)])
        pairs = [(0, i) for i in range(3)]
        assert np.array_equal(m.getDistances(pairs, typeOfMetric=0), m.getDistancesRefined(pairs))
        D1 = m.getDistances(pairs, typeOfMetric=1)
        D2 = m.refine(pairs, m.getDistances(pairs, typeOfMetric=2))
        assert np.array_equal(D1, D2)
    finally:
        m.close()
