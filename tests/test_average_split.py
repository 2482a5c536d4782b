"""The class average split across contexts (ettk_gpu_average_partial / ettk_gpu_average_finish): getImageMPI's
accumulators of all members finished give ettk_gpu_average's result bit for bit; accumulators of two member subsets
summed on the host give the same average to 1e-6 relative RMS, and the oracle's average to 1e-5 (the parity bar of
class averages)."""
import numpy as np
import pytest

import pyoracle
from ettk_gb300 import synthetic
from ettk_gb300.metric import ProjectionRotationMetric3D, WedgedSubImage3D

pytestmark = pytest.mark.gpu

KW = ("lwedge", "uwedge", "normal", "matrix", "position", "cut_offset")


def test_partial_accumulators_and_finish():
    ds = synthetic.generate("align32_b16", n_particles=6)
    members = [0, 1, 2, 3, 4]
    weights = [1.0, 1.0, 0.5, -0.25, 1.0]
    mats = []
    for i in members:
        T = np.eye(4)
        T[:3, :3] = ds.truth[i]["rotation"]
        T[:3, 3] = ds.truth[i]["shift"]
        mats.append(T)
    m = ProjectionRotationMetric3D(ds.params)
    try:
        m.set_particles([WedgedSubImage3D(ds.particles[i], **{k: ds.meta[i][k] for k in KW}) for i in range(6)])
        avg = m.average(members, weights, mats)
        whole = m.average_finish(*m.average_partial(members, weights, mats))
        a = m.average_partial(members[:2], weights[:2], mats[:2])
        b = m.average_partial(members[2:], weights[2:], mats[2:])
        split = m.average_finish(*(x + y for x, y in zip(a, b)))
    finally:
        m.close()
    assert np.array_equal(whole, avg)
    rms = np.sqrt(np.mean(avg ** 2))
    assert np.sqrt(np.mean((split - avg) ** 2)) <= 1e-6 * rms
    o = pyoracle.average(ds.params, [ds.particles[i] for i in members], [ds.meta[i] for i in members], weights,
                         mats).transpose(2, 1, 0)
    assert np.sqrt(np.mean((split - o) ** 2)) <= 1e-5 * np.sqrt(np.mean(o ** 2))
