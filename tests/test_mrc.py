"""MRC volume I/O (nbfMrcReader / nbfMrcWriter, inc/io/nbfMrcReader.h:255-350) and the tomogram
normalisation of nbfWedgedSubImage3D::getImage (inc/em/nbfWedgedSubImage3D.h:618-628). CPU only."""
import numpy as np
import pytest

from ettk_gb300 import mrc


def test_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    v = rng.standard_normal((7, 5, 12)).astype(np.float32)  # [z][y][x]
    p = tmp_path / "t.mrc"
    mrc.write(p, v, voxel_size=2.5)
    h = mrc.read_header(p)
    assert (h["nx"], h["ny"], h["nz"], h["mode"], h["byte_order"], h["nsymbt"]) == (12, 5, 7, 2, "<", 0)
    assert np.allclose(h["voxel_size"], 2.5)
    assert p.stat().st_size == 1024 + v.nbytes
    raw = p.read_bytes()
    assert raw[208:212] == b"MAP "
    hv = np.frombuffer(raw, "<f4", 3, 76)  # dmin, dmax, dmean
    assert np.allclose(hv, (v.min(), v.max(), v.mean()), atol=1e-6)
    assert np.array_equal(mrc.read(p), v)


def _raw_file(path, data, mode, bo, nsymbt=0, stamp=True):
    nz, ny, nx = data.shape
    iv = np.zeros(256, bo + "i4")
    iv[0:4] = (nx, ny, nz, mode)
    iv[7:10] = (nx, ny, nz)
    iv[23] = nsymbt
    hdr = bytearray(iv.tobytes())
    if stamp:
        hdr[212:214] = b"\x44\x44" if bo == "<" else b"\x11\x11"
    with open(path, "wb") as f:
        f.write(bytes(hdr))
        f.write(b"\x07" * nsymbt)
        f.write(np.ascontiguousarray(data).astype(data.dtype.newbyteorder(bo)).tobytes())


@pytest.mark.parametrize("mode,dtype", [(0, np.uint8), (1, np.int16), (2, np.float32), (6, np.uint16),
                                        (12, np.float16)])
@pytest.mark.parametrize("bo", ["<", ">"])
def test_modes_and_byte_order(tmp_path, mode, dtype, bo):
    rng = np.random.default_rng(mode)
    d = (rng.integers(0, 200, (4, 3, 6)) - (0 if mode in (0, 6) else 100)).astype(dtype)
    p = tmp_path / "m.mrc"
    _raw_file(p, d, mode, bo)
    assert np.array_equal(mrc.read(p), d.astype(np.float32))


def test_extended_header_and_no_stamp(tmp_path):
    d = np.arange(2 * 3 * 4, dtype=np.float32).reshape(2, 3, 4)
    p = tmp_path / "e.mrc"
    _raw_file(p, d, 2, ">", nsymbt=256, stamp=False)
    h = mrc.read_header(p)
    assert h["byte_order"] == ">" and h["nsymbt"] == 256
    assert np.array_equal(mrc.read(p), d)


def test_bad_files(tmp_path):
    p = tmp_path / "short.mrc"
    p.write_bytes(b"\0" * 100)
    with pytest.raises(ValueError):
        mrc.read(p)
    d = np.zeros((2, 2, 2), np.float32)
    q = tmp_path / "mode.mrc"
    _raw_file(q, d, 4, "<")
    with pytest.raises(ValueError):
        mrc.read(q)
    r = tmp_path / "trunc.mrc"
    _raw_file(r, d, 2, "<")
    r.write_bytes(r.read_bytes()[:-4])
    with pytest.raises(ValueError):
        mrc.read(r)


def test_normalize():
    rng = np.random.default_rng(5)
    t = (3.0 + 2.0 * rng.standard_normal((9, 10, 11))).astype(np.float32)
    n = mrc.normalize(t)
    s = t[::4, ::4, ::4].astype(np.float64)
    ref = (t - s.mean()) / s.std()
    assert np.allclose(n, ref, atol=1e-5)
    assert n.dtype == np.float32
