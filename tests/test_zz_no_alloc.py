"""The allocation-free SO(3) correlation entry point (ettk_gpu_soft_noalloc).

It serves callers that cannot call cudaMalloc where they score spherical signals (for example an
application whose memory pool already owns the device memory, or a process under a fixed memory
budget). These tests call it through the C ABI on device buffers:

- twice in a row with different inputs (so stale contents of its shared scratch array would show) at both
  accepted bandwidths, B = 8 and B = 16, comparing each result with the oracle (FP64) and with the
  context-based ettk_gpu_soft entry point, to the SO(3) stage's tolerance (1e-4 of the correlation's range);
- after a warm-up call, further calls leave the device's free memory unchanged;
- in a fresh process, the first call (the one that sets the device's array up) made on a non-blocking stream
  gives the same result;
- bandwidths beyond the array's limit are refused with ETTK_ERR_ARG.

The file is collected last.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

import pyoracle

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _call(L, B, F1, F2, stream):
    import torch
    n = 2 * B
    d1 = torch.from_numpy(F1).cuda()
    d2 = torch.from_numpy(F2).cuda()
    dC = torch.full((n, n, n), float("nan"), device="cuda")
    torch.cuda.synchronize()
    rc = L.ettk_gpu_soft_noalloc(B, d1.data_ptr(), d2.data_ptr(), dC.data_ptr(), stream)
    torch.cuda.synchronize()
    return rc, dC.cpu().numpy()


@pytest.mark.parametrize("B", [8, 16])
def test_soft_noalloc_matches_oracle_and_soft(B):
    import torch
    from ettk_gb300 import _lib, synthetic
    from ettk_gb300.metric import ProjectionRotationMetric3D

    L = _lib.load()
    n = 2 * B
    params = dict(synthetic.default_params(synthetic.WORKLOADS["align32_b16"]), B=B)
    m = ProjectionRotationMetric3D(params)
    try:
        rng = np.random.default_rng(2026 + B)
        for _ in range(2):
            F1 = rng.random((n, n)).astype(np.float32)
            F2 = rng.random((n, n)).astype(np.float32)
            C_ctx = m.soft(F1, F2, scaled=False)
            C_orc = pyoracle.soft(B, F1.astype(np.float64), F2.astype(np.float64))
            rc, C = _call(L, B, F1, F2, torch.cuda.current_stream().cuda_stream)
            assert rc == _lib.ETTK_OK
            assert np.isfinite(C).all()
            span = C_orc.max() - C_orc.min()
            assert np.abs(C - C_orc).max() <= 1e-4 * span
            assert np.abs(C - C_ctx).max() <= 1e-4 * span
            assert np.unravel_index(C.argmax(), C.shape) == np.unravel_index(C_orc.argmax(), C_orc.shape)
    finally:
        m.close()


def test_soft_noalloc_allocates_nothing():
    import torch
    from ettk_gb300 import _lib

    L = _lib.load()
    B, n = 16, 32
    rng = np.random.default_rng(7)
    d1 = torch.from_numpy(rng.random((n, n)).astype(np.float32)).cuda()
    d2 = torch.from_numpy(rng.random((n, n)).astype(np.float32)).cuda()
    dC = torch.zeros((n, n, n), device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    assert L.ettk_gpu_soft_noalloc(B, d1.data_ptr(), d2.data_ptr(), dC.data_ptr(), stream) == _lib.ETTK_OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert L.ettk_gpu_soft_noalloc(B, d1.data_ptr(), d2.data_ptr(), dC.data_ptr(), stream) == _lib.ETTK_OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    big = torch.zeros(128, 128, device="cuda")
    out = torch.zeros(128, 128, 128, device="cuda")
    assert L.ettk_gpu_soft_noalloc(64, big.data_ptr(), big.data_ptr(), out.data_ptr(), None) == _lib.ETTK_ERR_ARG
    assert L.ettk_gpu_soft_noalloc(32, big.data_ptr(), big.data_ptr(), out.data_ptr(), None) == _lib.ETTK_ERR_ARG


_FRESH = r"""
import sys
sys.path[:0] = [{root!r}, {oracle!r}]
import numpy as np, torch
import pyoracle
from ettk_gb300 import _lib
L = _lib.load()
B, n = 16, 32
rng = np.random.default_rng(99)
F1 = rng.random((n, n)).astype(np.float32)
F2 = rng.random((n, n)).astype(np.float32)
d1 = torch.from_numpy(F1).cuda(); d2 = torch.from_numpy(F2).cuda()
dC = torch.full((n, n, n), float("nan"), device="cuda")
torch.cuda.synchronize()
s = torch.cuda.Stream()   # created non-blocking: not ordered after the legacy default stream
rc = L.ettk_gpu_soft_noalloc(B, d1.data_ptr(), d2.data_ptr(), dC.data_ptr(), s.cuda_stream)
s.synchronize()
assert rc == _lib.ETTK_OK, rc
C = dC.cpu().numpy()
O = pyoracle.soft(B, F1.astype(np.float64), F2.astype(np.float64))
err = np.abs(C - O).max() / (O.max() - O.min())
assert err <= 1e-4, err
print("fresh-process first call ok", err)
"""


def test_soft_noalloc_first_call_on_nonblocking_stream():
    code = _FRESH.format(root=ROOT, oracle=os.path.join(ROOT, "oracle"))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
