"""The allocation-free SO(3) correlation entry point (ettk_gpu_soft_noalloc).

It serves callers that cannot call cudaMalloc where they score spherical signals (for example an
application whose memory pool already owns the device memory). This test calls it through the C ABI
on device buffers, twice in a row with different inputs (so stale contents of its shared scratch
array would show), and compares each result with the context-based ettk_gpu_soft entry point to the
tolerance used for the SO(3) stage elsewhere (1e-4 of the correlation's range). It lives in a file
that pytest collects last.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_soft_noalloc_matches_soft():
    import torch
    from ettk_gb300 import _lib, synthetic
    from ettk_gb300.metric import ProjectionRotationMetric3D

    L = _lib.load()
    B, n = 16, 32
    params = synthetic.default_params(synthetic.WORKLOADS["align32_b16"])
    m = ProjectionRotationMetric3D(params)
    try:
        rng = np.random.default_rng(2026)
        for _ in range(2):
            F1 = rng.random((n, n)).astype(np.float32)
            F2 = rng.random((n, n)).astype(np.float32)
            C_ref = m.soft(F1, F2, scaled=False)
            d1 = torch.from_numpy(F1).cuda()
            d2 = torch.from_numpy(F2).cuda()
            dC = torch.full((n, n, n), float("nan"), device="cuda")
            torch.cuda.synchronize()
            stream = torch.cuda.current_stream().cuda_stream
            rc = L.ettk_gpu_soft_noalloc(B, d1.data_ptr(), d2.data_ptr(), dC.data_ptr(), stream)
            assert rc == _lib.ETTK_OK
            torch.cuda.synchronize()
            C = dC.cpu().numpy()
            assert np.isfinite(C).all()
            assert np.abs(C - C_ref).max() <= 1e-4 * (C_ref.max() - C_ref.min())
        big = torch.zeros(128, 128, device="cuda")
        out = torch.zeros(128, 128, 128, device="cuda")
        assert L.ettk_gpu_soft_noalloc(64, big.data_ptr(), big.data_ptr(), out.data_ptr(), None) == _lib.ETTK_ERR_ARG
    finally:
        m.close()
