"""MRC volume I/O for tomograms and particle boxes (the reference's nbfMrcReader / nbfMrcWriter,
inc/io/nbfMrcReader.h:255-350, inc/io/nbfMrcWriter.h:30-135), plus the zero-mean / unit-variance
normalisation that nbfWedgedSubImage3D::getImage applies to a tomogram when asked
(inc/em/nbfWedgedSubImage3D.h:618-628).

Arrays are [z][y][x] (x fastest), the file's own order. Differences from the reference reader, all on
files the reference cannot read or reads wrongly:
  * the data start at 1024 + NSYMBT (the extended-header length at byte 92); the reference always
    starts at 1024, which is the same for files without an extended header;
  * modes 0 (bytes, unsigned as the reference declares them), 1 (int16), 2 (float32), 6 (uint16) and
    12 (float16) are read; the reference's branch structure accepts only mode 2;
  * the byte order comes from the machine stamp (bytes 212-213), or, for files without one, from which
    order gives a known mode.
The writer emits mode 2, little endian, MRC2014 ("MAP " at byte 208), with min / max / mean / rms.
"""
import numpy as np

HEADER = 1024
_MODES = {0: np.uint8, 1: np.int16, 2: np.float32, 6: np.uint16, 12: np.float16}


def _byte_order(hdr):
    stamp = hdr[212:214]
    if stamp[0] == 0x44:
        return "<"
    if stamp[0] == 0x11:
        return ">"
    for bo in ("<", ">"):
        if int(np.frombuffer(hdr, bo + "i4", 1, 12)[0]) in _MODES:
            return bo
    raise ValueError("MRC: unknown byte order / mode")


def read_header(path):
    with open(path, "rb") as f:
        hdr = f.read(HEADER)
    if len(hdr) < HEADER:
        raise ValueError("MRC: %s is shorter than its header" % path)
    bo = _byte_order(hdr)
    iv = np.frombuffer(hdr, bo + "i4", 24, 0)
    fv = np.frombuffer(hdr, bo + "f4", 24, 0)
    nx, ny, nz, mode = (int(v) for v in iv[:4])
    if mode not in _MODES:
        raise ValueError("MRC: unsupported mode %d" % mode)
    if min(nx, ny, nz) < 1:
        raise ValueError("MRC: bad dimensions %r" % ((nx, ny, nz),))
    mx, my, mz = (int(v) for v in iv[7:10])
    cella = fv[10:13]
    voxel = tuple(float(cella[i] / m) if m > 0 else 1.0 for i, m in enumerate((mx, my, mz)))
    return {"nx": nx, "ny": ny, "nz": nz, "mode": mode, "byte_order": bo, "nsymbt": int(iv[23]),
            "voxel_size": voxel}


def read(path, dtype=np.float32):
    """Volume of an MRC file as [z][y][x] `dtype` (float32 by default)."""
    h = read_header(path)
    n = h["nx"] * h["ny"] * h["nz"]
    t = np.dtype(_MODES[h["mode"]]).newbyteorder(h["byte_order"])
    with open(path, "rb") as f:
        f.seek(HEADER + h["nsymbt"])
        data = np.fromfile(f, t, n)
    if data.size != n:
        raise ValueError("MRC: %s holds %d of %d voxels" % (path, data.size, n))
    return data.reshape(h["nz"], h["ny"], h["nx"]).astype(dtype)


def write(path, vol, voxel_size=1.0):
    """Writes a [z][y][x] volume as a mode-2 (float32) little-endian MRC file."""
    v = np.ascontiguousarray(vol, dtype="<f4")
    if v.ndim != 3:
        raise ValueError("MRC: volume must be 3-D")
    nz, ny, nx = v.shape
    vs = (float(voxel_size),) * 3 if np.isscalar(voxel_size) else tuple(float(x) for x in voxel_size)
    hdr = bytearray(HEADER)
    iv = np.zeros(56, "<i4")
    fv = iv.view("<f4")
    iv[0:4] = (nx, ny, nz, 2)
    iv[7:10] = (nx, ny, nz)
    fv[10:13] = (nx * vs[0], ny * vs[1], nz * vs[2])
    fv[13:16] = 90.0
    iv[16:19] = (1, 2, 3)
    d64 = v.astype(np.float64)
    fv[19:22] = (d64.min(), d64.max(), d64.mean())
    hdr[:224] = iv.tobytes()
    hdr[208:212] = b"MAP "
    hdr[212:216] = bytes((0x44, 0x44, 0, 0))
    hdr[216:220] = np.float32(d64.std()).astype("<f4").tobytes()
    with open(path, "wb") as f:
        f.write(bytes(hdr))
        f.write(v.tobytes())


def normalize(tomogram):
    """Zero mean and unit variance from the statistics of every fourth voxel along each axis, as
    nbfWedgedSubImage3D::getImage normalises a tomogram before cutting (population deviation, float32)."""
    t = np.asarray(tomogram, np.float32)
    s = t[::4, ::4, ::4].astype(np.float64)
    mean = np.float32(s.mean())
    std = np.float32(np.sqrt(np.sum((s - mean) ** 2) / s.size))
    return ((t - mean) / std).astype(np.float32)
