"""ctypes binding to the oracle (test infrastructure only).

The oracle is the FP64 CPU restatement of the reference's alignment path in
oracle/*.cpp. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg use this module, as the checker; the product never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libsoft_ref.so")
BLITZ_REF_PATH = os.path.join(HERE, "_ref", "libblitz_ref.so")


class OracleParams(ctypes.Structure):
    _fields_ = [
        ("N", ctypes.c_int), ("B", ctypes.c_int),
        ("mask_x", ctypes.c_float), ("mask_y", ctypes.c_float), ("mask_z", ctypes.c_float),
        ("mask_sigma", ctypes.c_float), ("square_mask_size", ctypes.c_float),
        ("bp_low", ctypes.c_float), ("bp_high", ctypes.c_float),
        ("bp_low_sigma", ctypes.c_float), ("bp_high_sigma", ctypes.c_float),
        ("bfactor", ctypes.c_float),
        ("restrict_translation", ctypes.c_float), ("restrict_rotation", ctypes.c_float),
        ("candidate_peaks", ctypes.c_int), ("number_of_candidates", ctypes.c_int),
        ("wedge_compensation", ctypes.c_int), ("overlap_normalized", ctypes.c_int),
        ("mutual_correlation", ctypes.c_int),
        ("reference_mask", ctypes.POINTER(ctypes.c_float)),
    ]


class OracleVolume(ctypes.Structure):
    _fields_ = [
        ("data", ctypes.POINTER(ctypes.c_float)), ("dims", ctypes.c_int * 3),
        ("lwedge", ctypes.c_float), ("uwedge", ctypes.c_float),
        ("normal", ctypes.c_float * 3), ("matrix", ctypes.c_double * 16),
        ("position", ctypes.c_float * 3), ("cut_offset", ctypes.c_float),
        ("spherical_wedge", ctypes.POINTER(ctypes.c_float)),
    ]


class OracleResult(ctypes.Structure):
    _fields_ = [
        ("distance", ctypes.c_float), ("matrix", ctypes.c_double * 16),
        ("n_candidates", ctypes.c_int), ("cand_distance", ctypes.c_float * 8),
        ("cand_matrix", (ctypes.c_double * 16) * 8), ("n_ccf", ctypes.c_int),
        ("n_peaks_q1", ctypes.c_int), ("n_peaks_q2", ctypes.c_int),
        ("use_window1", ctypes.c_int), ("use_window2", ctypes.c_int),
        ("best_cell", ctypes.c_int * 3), ("wedge_overlap", ctypes.c_float),
    ]


def build():
    """Compile the oracle library, then run oracle/build_ref.sh, the recipe that compiles the reference's own
    SOFT sources and Blitz harnesses under _ref where the reference tree is present (it names the tree's
    location, overridable with ETTK_REFERENCE_ROOT, and skips cleanly where the tree is absent)."""
    subprocess.run(["make", "-s", "-C", HERE, "-j8"], check=True)
    subprocess.run([os.path.join(HERE, "build_ref.sh")], check=True, stdout=subprocess.DEVNULL)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        dp = np.ctypeslib.ndpointer(np.float64, flags="C")
        fp = np.ctypeslib.ndpointer(np.float32, flags="C")
        P = ctypes.POINTER(OracleParams)
        V = ctypes.POINTER(OracleVolume)
        L.oracle_align.argtypes = [P, V, V, ctypes.POINTER(OracleResult)]
        L.oracle_get_image.argtypes = [P, V, ctypes.c_void_p, dp]
        L.oracle_spherical_projection.argtypes = [P, V, fp]
        L.oracle_spherical_wedge.argtypes = [P, V, fp]
        L.oracle_wedge_half.argtypes = [P, V, ctypes.c_void_p, fp]
        L.oracle_masks.argtypes = [P, fp, fp, fp]
        L.oracle_file_mask.argtypes = [P, ctypes.c_int, fp, ctypes.c_float, fp]
        L.oracle_soft.argtypes = [ctypes.c_int, dp, dp, dp]
        L.oracle_soft_scaled.argtypes = [ctypes.c_int, dp, dp, dp]
        L.oracle_rotate.argtypes = [ctypes.c_int, dp, ctypes.c_double, ctypes.c_double, ctypes.c_double, dp]
        L.oracle_sht.argtypes = [ctypes.c_int, dp, dp]
        L.oracle_ccf.argtypes = [P, V, V, dp]
        L.oracle_ccf.restype = ctypes.c_float
        L.oracle_refine_objective.argtypes = [P, V, V, dp, dp]
        L.oracle_refine_objective.restype = ctypes.c_double
        L.oracle_refined_objective.argtypes = [P, V, V, dp, dp, ctypes.c_void_p]
        L.oracle_refined_objective.restype = ctypes.c_double
        L.oracle_average.argtypes = [P, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, dp]
        L.oracle_symmetrize.argtypes = [P, V, ctypes.c_int, ctypes.c_void_p]
        L.oracle_variance.argtypes = [P, ctypes.c_int] + [ctypes.c_void_p] * 5
        L.oracle_symmetrize_rotational.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_average_spherical_wedge.argtypes = [P, ctypes.c_int] + [ctypes.c_void_p] * 5
        L.oracle_representation_distances.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p, ctypes.c_int,
                                                                            ctypes.c_void_p]
        L.oracle_representation.argtypes = [P, V, ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
        L.oracle_representation_real.argtypes = [P, V, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                                 ctypes.POINTER(ctypes.c_int)]
        L.oracle_rfft3d.argtypes = [ctypes.c_int] * 3 + [dp, dp]
        L.oracle_normalize_half.argtypes = [ctypes.c_int, dp, ctypes.POINTER(ctypes.c_float)]
        L.oracle_wedge_overlap.argtypes = [P, V, V, dp]
        L.oracle_wedge_overlap.restype = ctypes.c_float
        L.oracle_ccf_distance.argtypes = [ctypes.c_float, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_int, ctypes.c_int]
        L.oracle_ccf_distance.restype = ctypes.c_float
        L.oracle_irfft3d.argtypes = [ctypes.c_int] * 3 + [dp, dp]
        _lib = L
    return _lib


def make_params(p):
    """OracleParams from the alignment parameter dict used across the repo. p["reference_mask"] (optional): the
    CCF's reference mask m1 as file_mask returns it ([x][y][z], N^3)."""
    P = OracleParams(
        N=p["N"], B=p["B"], mask_x=p["mask_radius"], mask_y=p["mask_radius"], mask_z=p["mask_radius"],
        mask_sigma=p["mask_sigma"], square_mask_size=p["square_mask_size"],
        bp_low=p["bp_low"], bp_high=p["bp_high"], bp_low_sigma=p["bp_low_sigma"],
        bp_high_sigma=p["bp_high_sigma"], bfactor=p.get("bfactor", 0.0),
        restrict_translation=p["restrict_translation"], restrict_rotation=p["restrict_rotation"],
        candidate_peaks=p["candidate_peaks"], number_of_candidates=p["number_of_candidates"],
        wedge_compensation=int(p["wedge_compensation"]), overlap_normalized=int(p["overlap_normalized"]),
        mutual_correlation=int(bool(p.get("mutual_correlation", False))))
    rm = p.get("reference_mask")
    if rm is not None:
        rm = np.ascontiguousarray(rm, dtype=np.float32)
        assert rm.size == p["N"] ** 3
        P.reference_mask = rm.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        P._keep = rm
    return P


def file_mask(params, mask, threshold):
    """nbfImageFilter::buildMaskFromFile + softenMask on a mask volume (M, M, M) in [z][y][x] order (x fastest, as
    read from its MRC file): the N^3 reference mask in [x][y][z] order, for params["reference_mask"]."""
    m = np.ascontiguousarray(mask, dtype=np.float32)
    M = m.shape[0]
    assert m.shape == (M, M, M)
    N = params["N"]
    out = np.zeros((N, N, N), np.float32)
    P = make_params(params)
    if lib().oracle_file_mask(ctypes.byref(P), M, m, float(threshold), out) != 0:
        raise ValueError("mask edge %d cannot be centred into %d" % (M, N))
    return out


def make_volume(data, meta):
    """OracleVolume for a fixed image `data` ([z][y][x] numpy, i.e. x fastest) and its metadata."""
    data = np.ascontiguousarray(data, dtype=np.float32)
    v = OracleVolume()
    v.data = data.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    v._keep = data
    nz, ny, nx = data.shape
    v.dims[:] = [nx, ny, nz]
    v.lwedge, v.uwedge = meta["lwedge"], meta["uwedge"]
    v.normal[:] = list(meta.get("normal", (0.0, 0.0, 0.0)))
    v.matrix[:] = list(np.asarray(meta.get("matrix", np.eye(4)), dtype=np.float64).reshape(16))
    v.position[:] = list(meta.get("position", (nx / 2.0, ny / 2.0, nz / 2.0)))
    v.cut_offset = meta.get("cut_offset", 0.0)
    if meta.get("spherical_wedge") is not None:
        w = np.ascontiguousarray(meta["spherical_wedge"], np.float32)
        v.spherical_wedge = w.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        v._keep_w = w
    return v


def align(params, ref, ref_meta, part, part_meta):
    P = make_params(params)
    r = make_volume(ref, ref_meta)
    q = make_volume(part, part_meta)
    out = OracleResult()
    lib().oracle_align(ctypes.byref(P), ctypes.byref(r), ctypes.byref(q), ctypes.byref(out))
    return {
        "distance": out.distance,
        "matrix": np.array(out.matrix[:]).reshape(4, 4),
        "n_ccf": out.n_ccf, "n_peaks_q1": out.n_peaks_q1, "n_peaks_q2": out.n_peaks_q2,
        "use_window1": out.use_window1, "use_window2": out.use_window2,
        "best_cell": tuple(out.best_cell[:]),
        "cand_distance": list(out.cand_distance[:out.n_candidates]),
        "cand_matrix": [np.array(out.cand_matrix[i][:]).reshape(4, 4) for i in range(out.n_candidates)],
        "wedge_overlap": out.wedge_overlap,
    }


def ccf(params, ref, ref_meta, part, part_meta, T):
    P = make_params(params)
    r = make_volume(ref, ref_meta)
    q = make_volume(part, part_meta)
    t = np.ascontiguousarray(np.asarray(T, dtype=np.float64).reshape(16)).copy()
    d = lib().oracle_ccf(ctypes.byref(P), ctypes.byref(r), ctypes.byref(q), t)
    return float(d), t.reshape(4, 4)


def wedge_overlap(params, ref, ref_meta, part, part_meta, T):
    """getWedgeOverlap(T) of the pair (the D column of 19-column rows)."""
    P = make_params(params)
    r = make_volume(ref, ref_meta)
    q = make_volume(part, part_meta)
    t = np.ascontiguousarray(np.asarray(T, dtype=np.float64).reshape(16))
    return float(lib().oracle_wedge_overlap(ctypes.byref(P), ctypes.byref(r), ctypes.byref(q), t))


def refine_objective(params, ref, ref_meta, part, part_meta, T, theta):
    """FP64 objective of the continuous refinement at pose T perturbed by theta (rotation vector in radians
    about the box centre, then shift in voxels)."""
    P = make_params(params)
    r = make_volume(ref, ref_meta)
    q = make_volume(part, part_meta)
    t = np.ascontiguousarray(np.asarray(T, dtype=np.float64).reshape(16))
    th = np.ascontiguousarray(np.asarray(theta, dtype=np.float64).reshape(6))
    return float(lib().oracle_refine_objective(ctypes.byref(P), ctypes.byref(r), ctypes.byref(q), t, th))


def refined_objective(params, ref, ref_meta, part, part_meta, T, theta):
    """FP64 objective of the fast form's local refinement (the reference filtered with the wedges at pose T, the
    particle at T perturbed by theta) and its analytic gradient: (rho, grad[6])."""
    P = make_params(params)
    r = make_volume(ref, ref_meta)
    q = make_volume(part, part_meta)
    t = np.ascontiguousarray(np.asarray(T, dtype=np.float64).reshape(16))
    th = np.ascontiguousarray(np.asarray(theta, dtype=np.float64).reshape(6))
    g = np.zeros(6)
    rho = lib().oracle_refined_objective(ctypes.byref(P), ctypes.byref(r), ctypes.byref(q), t, th, g.ctypes.data)
    return float(rho), g


def get_image(params, vol, meta, T=None):
    P = make_params(params)
    v = make_volume(vol, meta)
    N = params["N"]
    out = np.zeros(N ** 3, dtype=np.float64)
    t = None if T is None else np.ascontiguousarray(np.asarray(T, np.float64).reshape(16))
    lib().oracle_get_image(ctypes.byref(P), ctypes.byref(v), None if t is None else t.ctypes.data, out)
    return out.reshape(N, N, N)  # [x][y][z]


def spherical_projection(params, vol, meta):
    P = make_params(params)
    v = make_volume(vol, meta)
    n = 2 * params["B"]
    out = np.zeros(n * n, dtype=np.float32)
    lib().oracle_spherical_projection(ctypes.byref(P), ctypes.byref(v), out)
    return out.reshape(n, n)


def spherical_wedge(params, meta, N):
    P = make_params(params)
    v = make_volume(np.zeros((N, N, N), np.float32), meta)
    n = 2 * params["B"]
    out = np.zeros(n * n, dtype=np.float32)
    lib().oracle_spherical_wedge(ctypes.byref(P), ctypes.byref(v), out)
    return out.reshape(n, n)


def wedge_half(params, meta, T=None):
    N = params["N"]
    P = make_params(params)
    v = make_volume(np.zeros((N, N, N), np.float32), meta)
    out = np.zeros(N * N * (N // 2 + 1), dtype=np.float32)
    t = None if T is None else np.ascontiguousarray(np.asarray(T, np.float64).reshape(16))
    lib().oracle_wedge_half(ctypes.byref(P), ctypes.byref(v), None if t is None else t.ctypes.data, out)
    return out.reshape(N, N, N // 2 + 1)


def masks(params):
    N = params["N"]
    P = make_params(params)
    m = np.zeros(N ** 3, np.float32)
    mf = np.zeros(N ** 3, np.float32)
    f = np.zeros(N * N * (N // 2 + 1), np.float32)
    lib().oracle_masks(ctypes.byref(P), m, mf, f)
    return m.reshape(N, N, N), mf.reshape(N, N, N), f.reshape(N, N, N // 2 + 1)


def soft(B, F1, F2, scaled=False):
    n = 2 * B
    C = np.zeros(n ** 3, np.float64)
    fn = lib().oracle_soft_scaled if scaled else lib().oracle_soft
    fn(B, np.ascontiguousarray(F1, np.float64), np.ascontiguousarray(F2, np.float64), C)
    return C.reshape(n, n, n)


def rotate(B, F, a, b, g):
    n = 2 * B
    R = np.zeros(n * n, np.float64)
    lib().oracle_rotate(B, np.ascontiguousarray(F, np.float64), a, b, g, R)
    return R.reshape(n, n)


def sht(B, F):
    out = np.zeros(B * 2 * B * 2, np.float64)
    lib().oracle_sht(B, np.ascontiguousarray(F, np.float64), out)
    c = out.reshape(B, 2 * B, 2)
    return c[..., 0] + 1j * c[..., 1]


def average(params, vols, metas, weights, mats):
    """Class average (getImageMPI + getImage), returned as [x][y][z]."""
    P = make_params(params)
    n = len(vols)
    arr = (OracleVolume * n)()
    keep = []
    for i in range(n):
        v = make_volume(vols[i], metas[i])
        keep.append(v)
        arr[i] = v
    w = np.ascontiguousarray(weights, np.float32)
    m = np.ascontiguousarray(np.asarray(mats, np.float64).reshape(n, 16))
    N = params["N"]
    out = np.zeros(N ** 3, np.float64)
    lib().oracle_average(ctypes.byref(P), n, ctypes.addressof(arr), w.ctypes.data, m.ctypes.data, out)
    return out.reshape(N, N, N)


def symmetrize(params, vol, fold):
    """nbfImageFilter::symmetrize of a fixed-image volume ([z][y][x]); returned as [x][y][z]."""
    P = make_params(params)
    N = params["N"]
    meta = {"lwedge": -90.0, "uwedge": 90.0}
    v = make_volume(vol, meta)
    out = np.zeros(N ** 3, np.float64)
    lib().oracle_symmetrize(ctypes.byref(P), ctypes.byref(v), int(fold), out.ctypes.data)
    return out.reshape(N, N, N)


def representation(params, vol, meta, fold=1):
    """getLowDimensionRepresentationHalf of one volume: (K, 3) float32 (re, im, wedge bit)."""
    P = make_params(params)
    v = make_volume(vol, meta)
    K = ctypes.c_int()
    lib().oracle_representation(ctypes.byref(P), ctypes.byref(v), int(fold), None, ctypes.byref(K))
    R = np.zeros((K.value, 3), np.float32)
    lib().oracle_representation(ctypes.byref(P), ctypes.byref(v), int(fold), R.ctypes.data, ctypes.byref(K))
    return R


def representation_real(params, vol, meta, fold=1, bin_factor=1):
    """getLowDimensionRepresentationReal of one volume (the image filter's mask; n-fold branch through the one-member
    wedged average; integer bin factor): (K,) float64."""
    P = make_params(params)
    v = make_volume(vol, meta)
    K = ctypes.c_int()
    if lib().oracle_representation_real(ctypes.byref(P), ctypes.byref(v), int(fold), int(bin_factor), None,
                                        ctypes.byref(K)) != 0:
        raise ValueError("unsupported")
    C = np.zeros(K.value, np.float64)
    lib().oracle_representation_real(ctypes.byref(P), ctypes.byref(v), int(fold), int(bin_factor), C.ctypes.data,
                                     ctypes.byref(K))
    return C


def representation_distances(R, normalized=True):
    """getDistances over a representation array R (V, K, depth); returns (V, V) float32."""
    R = np.ascontiguousarray(R, np.float32)
    if R.ndim == 2:
        R = R[:, :, None]
    V, K, depth = R.shape
    D = np.zeros((V, V), np.float32)
    lib().oracle_representation_distances(V, K, depth, R.ctypes.data, int(bool(normalized)), D.ctypes.data)
    return D


def average_spherical_wedge(params, vols, metas, weights, mats):
    """Spherical wedge of the class average of the volumes under `mats`: (binary wedge, count), [2B][2B]."""
    P = make_params(params)
    n = len(vols)
    arr = (OracleVolume * n)()
    keep = []
    for i in range(n):
        v = make_volume(vols[i], metas[i])
        keep.append(v)
        arr[i] = v
    w = np.ascontiguousarray(np.asarray(weights, np.float32))
    m = np.ascontiguousarray(np.asarray(mats, np.float64).reshape(n, 16))
    n2 = 2 * params["B"]
    count = np.zeros((n2, n2), np.float32)
    wedge = np.zeros((n2, n2), np.float32)
    lib().oracle_average_spherical_wedge(ctypes.byref(P), n, ctypes.addressof(arr), w.ctypes.data, m.ctypes.data,
                                         count.ctypes.data, wedge.ctypes.data)
    return wedge, count


def symmetrize_rotational(vol):
    """Rotational (cylindrical) symmetrisation of an N^3 volume ([z][y][x]); returned as [x][y][z]."""
    v = np.ascontiguousarray(vol, np.float32)
    N = v.shape[0]
    out = np.zeros(N ** 3, np.float64)
    if lib().oracle_symmetrize_rotational(N, v.ctypes.data, out.ctypes.data) != 0:
        raise ValueError("N must be even and at least 4")
    return out.reshape(N, N, N)


def variance(params, vols, metas, weights, mats, avg_xyz):
    """getImageVarianceMPI of the members against an average given as [x][y][z]; returned as [x][y][z]."""
    P = make_params(params)
    n = len(vols)
    arr = (OracleVolume * n)()
    keep = []
    for i in range(n):
        v = make_volume(vols[i], metas[i])
        keep.append(v)
        arr[i] = v
    w = np.ascontiguousarray(weights, np.float32)
    m = np.ascontiguousarray(np.asarray(mats, np.float64).reshape(n, 16))
    a = np.ascontiguousarray(avg_xyz, np.float64)
    N = params["N"]
    out = np.zeros(N ** 3, np.float64)
    lib().oracle_variance(ctypes.byref(P), n, ctypes.addressof(arr), w.ctypes.data, m.ctypes.data, a.ctypes.data,
                          out.ctypes.data)
    return out.reshape(N, N, N)


def normalize_half(F):
    """normalizeFourierHalf of a complex [N][N][N/2+1] half spectrum (a copy): (normalised spectrum, norm)."""
    N = F.shape[0]
    a = np.ascontiguousarray(np.stack([F.real, F.imag], -1), np.float64)
    norm = ctypes.c_float()
    lib().oracle_normalize_half(N, a, ctypes.byref(norm))
    return a[..., 0] + 1j * a[..., 1], norm.value


def ccf_distance(k1_m, maxT, sum_wf, sum_f, overlap, N):
    return lib().oracle_ccf_distance(k1_m, maxT, sum_wf, sum_f, int(bool(overlap)), N)


def rfft3d(x):
    x = np.ascontiguousarray(x, np.float64)
    n0, n1, n2 = x.shape
    out = np.zeros((n0, n1, n2 // 2 + 1, 2), np.float64)
    lib().oracle_rfft3d(n0, n1, n2, x, out)
    return out[..., 0] + 1j * out[..., 1]


def irfft3d(X, n2):
    n0, n1, h = X.shape
    inp = np.ascontiguousarray(np.stack([X.real, X.imag], -1), np.float64)
    out = np.zeros((n0, n1, n2), np.float64)
    lib().oracle_irfft3d(n0, n1, n2, inp, out)
    return out


# ---------------------------------------------------------------- SOFT reference library (this container only)

_ref = None


def ref_lib():
    """The reference's SOFT 1.0 compiled from its own sources (None when absent)."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_PATH):
            return None
        L = ctypes.CDLL(REF_PATH)
        dp = np.ctypeslib.ndpointer(np.float64, flags="C")
        L.ref_soft.argtypes = [ctypes.c_int, dp, dp, dp]
        L.ref_fst.argtypes = [ctypes.c_int, dp, dp, dp]
        L.ref_rotate.argtypes = [ctypes.c_int, dp, ctypes.c_double, ctypes.c_double, ctypes.c_double, dp]
        _ref = L
    return _ref


_blitz_ref = None


def blitz_ref_lib():
    """Harnesses on the reference's Blitz (oracle/_ref/libblitz_ref.so), or None when absent."""
    global _blitz_ref
    if _blitz_ref is None:
        if not os.path.exists(BLITZ_REF_PATH):
            return None
        L = ctypes.CDLL(BLITZ_REF_PATH)
        L.cyl_ref_rotational.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.repr_ref_distances.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.clustering_ref_soft_weights.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 3
        L.clustering_ref_mra_assign.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.filter_ref_half.argtypes = [ctypes.c_int] + [ctypes.c_float] * 5 + [ctypes.c_void_p]
        L.normalize_ref_half.argtypes = [ctypes.c_int, ctypes.c_void_p]
        L.normalize_ref_half.restype = ctypes.c_float
        L.distance_ref.argtypes = [ctypes.c_float, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                   ctypes.c_int]
        L.distance_ref.restype = ctypes.c_float
        L.clustering_ref_cutoff.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_float, ctypes.c_int,
                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        _blitz_ref = L
    return _blitz_ref


def ref_symmetrize_rotational(vol):
    """The reference's own cylindrical-domain classes run through the rotational-symmetry step;
    [x][y][z], or None when the harness library is absent."""
    L = blitz_ref_lib()
    if L is None:
        return None
    v = np.ascontiguousarray(vol, np.float32)
    N = v.shape[0]
    out = np.zeros(N ** 3, np.float64)
    if L.cyl_ref_rotational(N, v.ctypes.data, out.ctypes.data) != 0:
        raise ValueError("N must be even and at least 4")
    return out.reshape(N, N, N)


def ref_representation_distances(R, normalized=True):
    """The representation-distance loop in the reference's Blitz expressions; None when absent."""
    L = blitz_ref_lib()
    if L is None:
        return None
    R = np.ascontiguousarray(R, np.float32)
    if R.ndim == 2:
        R = R[:, :, None]
    V, K, depth = R.shape
    D = np.zeros((V, V), np.float32)
    L.repr_ref_distances(V, K, depth, R.ctypes.data, int(bool(normalized)), D.ctypes.data)
    return D


def ref_soft_weights(d):
    """computeNewReferences' radii and weights in the reference's Blitz expressions for distances d[V][R];
    (W [R][V], radii [R]) or None when the harness library is absent."""
    L = blitz_ref_lib()
    if L is None:
        return None
    d = np.ascontiguousarray(d, np.float32)
    V, R = d.shape
    W = np.zeros((R, V), np.float32)
    radii = np.zeros(R, np.float32)
    L.clustering_ref_soft_weights(R, V, d.ctypes.data, W.ctypes.data, radii.ctypes.data)
    return W, radii


def ref_cutoff(d, fraction, rule):
    """Best class and outlier cutoff in the reference's expressions for distances d[V][R]; (best, dist, keep) or
    None when the harness library is absent."""
    L = blitz_ref_lib()
    if L is None:
        return None
    d = np.ascontiguousarray(d, np.float32)
    V, R = d.shape
    best = np.zeros(V, np.int32)
    dist = np.zeros(V, np.float32)
    keep = np.zeros(V, np.int32)
    L.clustering_ref_cutoff(R, V, d.ctypes.data, float(fraction), int(rule), best.ctypes.data, dist.ctypes.data,
                            keep.ctypes.data)
    return best, dist, keep.astype(bool)


def ref_filter_half(params):
    """The half-grid Fourier filter in the reference's Blitz expressions ([N][N][N/2+1]); None when absent."""
    L = blitz_ref_lib()
    if L is None:
        return None
    N = params["N"]
    out = np.zeros((N, N, N // 2 + 1), np.float32)
    L.filter_ref_half(N, params["bp_low"], params["bp_high"], params["bp_low_sigma"], params["bp_high_sigma"],
                      params.get("bfactor", 0.0), out.ctypes.data)
    return out


def ref_normalize_half(F):
    """normalizeFourierHalf in the reference's Blitz expressions (a copy): (spectrum, norm); None when absent."""
    L = blitz_ref_lib()
    if L is None:
        return None
    a = np.ascontiguousarray(np.stack([F.real, F.imag], -1), np.float64)
    norm = L.normalize_ref_half(F.shape[0], a.ctypes.data)
    return a[..., 0] + 1j * a[..., 1], norm


def ref_ccf_distance(k1_m, maxT, sum_wf, sum_f, overlap, N):
    L = blitz_ref_lib()
    if L is None:
        return None
    return L.distance_ref(k1_m, maxT, sum_wf, sum_f, int(bool(overlap)), N)


def ref_mra_assign(S):
    """doMra's class choice in the reference's Blitz expressions for S[v][r][j]; labels or None when absent."""
    L = blitz_ref_lib()
    if L is None:
        return None
    S = np.ascontiguousarray(S, np.float32)
    V, R, _ = S.shape
    labels = np.zeros(V, np.int32)
    L.clustering_ref_mra_assign(R, V, S.ctypes.data, labels.ctypes.data)
    return labels
