"""Bounded device waits: a wait that runs out reports ETTK_ERR_TIMEOUT and leaves the context usable.

ettk_gpu_wait_probe runs one kernel whose mbarrier nothing arrives at (a flag that nothing sets), polled a small
number of times; the wait gives up, flags the status word, and the call returns ETTK_ERR_TIMEOUT with the status
cleared. The same context then aligns pairs as before (the reference's sentinel conventions are untouched: the rows
carry distances and transforms). No fault, trap or hang is involved.
"""
import ctypes

import numpy as np
import pytest

from ettk_gb300 import _lib, synthetic
from ettk_gb300.metric import ProjectionRotationMetric3D, WedgedSubImage3D

pytestmark = pytest.mark.gpu

KW = ("lwedge", "uwedge", "normal", "matrix", "position", "cut_offset")


def test_wait_that_runs_out_reports_timeout_and_context_stays_usable():
    ds = synthetic.generate("align32_b16", n_particles=2)
    m = ProjectionRotationMetric3D(ds.params)
    try:
        m.set_references([WedgedSubImage3D(ds.references[0], **{k: ds.ref_meta[0][k] for k in KW})])
        m.set_particles([WedgedSubImage3D(ds.particles[i], **{k: ds.meta[i][k] for k in KW}) for i in range(2)])
        D0 = m.getDistances([(0, 0), (0, 1)])
        rc = m.L.ettk_gpu_wait_probe(m._ctx, 1000)
        assert rc == _lib.ETTK_ERR_TIMEOUT
        buf = ctypes.create_string_buffer(256)
        m.L.ettk_gpu_last_error(m._ctx, buf, 256)
        assert b"wait" in buf.value
        D1 = m.getDistances([(0, 0), (0, 1)])  # the status word was cleared: the next call succeeds
        assert np.array_equal(D0, D1)
        assert m.L.ettk_gpu_wait_probe(m._ctx, 0) == _lib.ETTK_ERR_ARG
    finally:
        m.close()
