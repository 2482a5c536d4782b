"""Volume-list metadata marshalling (ettk_volume_meta of include/ettk_gpu.h) from the volume-list columns:
the numpy column fill must give the same bytes as filling the ctypes structure field by field. CPU only."""
import ctypes

import numpy as np

from ettk_gb300 import _lib


def _field_by_field(metas):
    arr = (_lib.VolumeMeta * len(metas))()
    for i, m in enumerate(metas):
        v = arr[i]
        v.lwedge, v.uwedge = m["lwedge"], m["uwedge"]
        v.normal[:] = [float(x) for x in m.get("normal", (0.0, 0.0, 0.0))]
        v.matrix[:] = [float(x) for x in np.asarray(m.get("matrix", np.eye(4)), np.float64).reshape(16)]
        v.position[:] = [float(x) for x in m["position"]]
        v.cut_offset = float(m.get("cut_offset", 0.0))
    return arr


def test_make_meta_bytes():
    rng = np.random.default_rng(7)
    metas = []
    for i in range(37):
        m = {"lwedge": float(rng.uniform(-70, -40)), "uwedge": float(rng.uniform(40, 70)),
             "position": tuple(rng.uniform(0, 500, 3))}
        if i % 3:
            m["normal"] = tuple(rng.uniform(-180, 180, 3))
        if i % 4:
            m["matrix"] = rng.standard_normal((4, 4))
        if i % 5:
            m["cut_offset"] = float(rng.uniform(-3, 3))
        metas.append(m)
    a = _lib.make_meta(metas)
    b = _field_by_field(metas)
    assert ctypes.sizeof(a) == ctypes.sizeof(b)
    assert bytes(a) == bytes(b)


def test_make_meta_empty():
    assert ctypes.sizeof(_lib.make_meta([])) == 0
