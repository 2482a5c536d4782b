"""Multireference classification (align -> assign to the closest class -> wedge-weighted re-average, the loop of
src/MPI_Classification.cpp) through ettk_gpu_classify on a small three-class case with shared blobs and uneven
class sizes. The stages it composes (alignment, class average) are pinned against the oracle in
test_gpu_parity.py; here the loop itself is checked: labels against the generating classes, and each class
average closest to its own generating reference."""
import numpy as np
import pytest

from ettk_gb300 import synthetic
from ettk_gb300.metric import ProjectionRotationMetric3D, WedgedSubImage3D

pytestmark = pytest.mark.gpu

KW = ("lwedge", "uwedge", "normal", "matrix", "position", "cut_offset")


def test_classify_three_classes():
    ds = synthetic.generate("mra32_b16", n_particles=30)
    truth = np.array([t["ref"] for t in ds.truth])
    rng = np.random.default_rng(3)
    # starting references: the generating volumes with independent noise of their own variance (SNR 1)
    start = [r + rng.standard_normal(r.shape).astype(np.float32) * r.std() for r in ds.references]
    m = ProjectionRotationMetric3D(ds.params)
    try:
        m.set_references([WedgedSubImage3D(s, **{k: ds.ref_meta[i][k] for k in KW}) for i, s in enumerate(start)])
        m.set_particles([WedgedSubImage3D(ds.particles[i], **{k: ds.meta[i][k] for k in KW})
                         for i in range(len(ds.meta))])
        labels, refs, dist = m.classify(iterations=2)
    finally:
        m.close()
    assert labels.shape == truth.shape and np.all((labels >= 0) & (labels < 3))
    assert np.all(np.isfinite(dist)) and np.all(dist >= 0)
    assert np.mean(labels == truth) >= 0.8
    for r in range(3):
        if not np.any(truth == r):
            continue
        cc = [np.corrcoef(refs[r].ravel(), ds.references[q].ravel())[0, 1] for q in range(3)]
        assert int(np.argmax(cc)) == r, cc
