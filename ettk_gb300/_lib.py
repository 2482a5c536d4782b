"""Build and load libettk_gpu.so (the CUDA implementation behind include/ettk_gpu.h).

The library is built in-tree under ettk_gb300/_build for sm_103a. Loading fails loudly when
it is missing: there is no CPU fallback for the alignment path.
"""
import ctypes
import os
import subprocess

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libettk_gpu.so")
SRC = os.path.join(PKG, "csrc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

ETTK_OK, ETTK_ERR_ARG, ETTK_ERR_OOM, ETTK_ERR_CUDA, ETTK_ERR_TIMEOUT, ETTK_ERR_NAN, ETTK_ERR_STATE = range(7)


def build(verbose=False):
    """Compile the CUDA library (nvcc, sm_103a). Returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(SRC, "ettk_gpu.cu"), os.path.join(SRC, "noalloc.cu")]
    deps = srcs + [os.path.join(SRC, f) for f in os.listdir(SRC)] + [os.path.join(ROOT, "include", "ettk_gpu.h")]
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    cmd = ["nvcc", *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off", "-shared",
           "-o", LIB + ".tmp", *srcs]
    subprocess.run(cmd, check=True, stdout=None if verbose else subprocess.DEVNULL)
    os.replace(LIB + ".tmp", LIB)
    return LIB


class Params(ctypes.Structure):
    _fields_ = [
        ("N", ctypes.c_int), ("B", ctypes.c_int),
        ("mask_radius", ctypes.c_float), ("mask_sigma", ctypes.c_float), ("square_mask_size", ctypes.c_float),
        ("bp_low", ctypes.c_float), ("bp_high", ctypes.c_float),
        ("bp_low_sigma", ctypes.c_float), ("bp_high_sigma", ctypes.c_float), ("bfactor", ctypes.c_float),
        ("restrict_translation", ctypes.c_float), ("restrict_rotation", ctypes.c_float),
        ("candidate_peaks", ctypes.c_int), ("number_of_candidates", ctypes.c_int),
        ("wedge_compensation", ctypes.c_int), ("overlap_normalized", ctypes.c_int),
        ("mutual_correlation", ctypes.c_int), ("max_batch", ctypes.c_int), ("wigner_precision", ctypes.c_int),
        ("fast_coarse_so3", ctypes.c_int),
    ]


class Tuning(ctypes.Structure):
    _fields_ = [("synth_job_blocks", ctypes.c_int), ("eval_chunk", ctypes.c_int), ("zpass_oversub", ctypes.c_int),
                ("sample_block", ctypes.c_int)]


class VolumeMeta(ctypes.Structure):
    _fields_ = [
        ("lwedge", ctypes.c_float), ("uwedge", ctypes.c_float), ("normal", ctypes.c_float * 3),
        ("matrix", ctypes.c_double * 16), ("position", ctypes.c_float * 3), ("cut_offset", ctypes.c_float),
    ]


SYMBOLS = [
    "ettk_gpu_create", "ettk_gpu_destroy", "ettk_gpu_set_references", "ettk_gpu_set_particles",
    "ettk_gpu_set_particles_device", "ettk_gpu_align_pairs", "ettk_gpu_ccf", "ettk_gpu_spherical_projection",
    "ettk_gpu_soft", "ettk_gpu_kernel_launches", "ettk_gpu_last_error", "ettk_gpu_stream", "ettk_gpu_profile",
    "ettk_gpu_profile_read", "ettk_gpu_soft_noalloc", "ettk_gpu_average", "ettk_gpu_refine_pairs",
    "ettk_gpu_refine_objective", "ettk_gpu_classify", "ettk_gpu_set_particles_tomogram", "ettk_gpu_variance",
    "ettk_gpu_symmetrize", "ettk_gpu_symmetrize_rotational", "ettk_gpu_outlier_cutoff", "ettk_gpu_soft_weights",
    "ettk_gpu_average_spherical_wedge", "ettk_gpu_set_reference_spherical_wedge",
    "ettk_gpu_representation_distances", "ettk_gpu_representations", "ettk_gpu_representations_real",
    "ettk_gpu_mean_images", "ettk_gpu_set_reference_mask", "ettk_gpu_get_reference_mask", "ettk_gpu_get_tuning", "ettk_gpu_set_tuning", "ettk_gpu_autotune",
    "ettk_gpu_mra_assign",
    "ettk_gpu_align_pairs_refined", "ettk_gpu_refined_objective", "ettk_gpu_score_pairs",
    "ettk_gpu_average_partial", "ettk_gpu_average_finish", "ettk_gpu_wait_probe",
]

_lib = None


def load(path=None):
    """Load the library (building it first when absent). Raises if it cannot be loaded."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB
    if not os.path.exists(path):
        build()
    L = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    P = ctypes.POINTER
    L.ettk_gpu_create.argtypes = [ctypes.c_int, P(Params), P(vp)]
    L.ettk_gpu_destroy.argtypes = [vp]
    L.ettk_gpu_set_references.argtypes = [vp, ctypes.c_int, vp, P(VolumeMeta)]
    L.ettk_gpu_set_particles.argtypes = [vp, ctypes.c_int, vp, P(VolumeMeta)]
    L.ettk_gpu_set_particles_device.argtypes = [vp, ctypes.c_int, vp, P(VolumeMeta)]
    L.ettk_gpu_align_pairs.argtypes = [vp, ctypes.c_int, vp, vp, ctypes.c_int, ctypes.c_int]
    L.ettk_gpu_ccf.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp, P(ctypes.c_float)]
    L.ettk_gpu_spherical_projection.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp]
    L.ettk_gpu_soft.argtypes = [vp, vp, vp, ctypes.c_int, vp]
    L.ettk_gpu_kernel_launches.argtypes = [vp]
    L.ettk_gpu_kernel_launches.restype = ctypes.c_longlong
    L.ettk_gpu_last_error.argtypes = [vp, ctypes.c_char_p, ctypes.c_int]
    L.ettk_gpu_stream.argtypes = [vp]
    L.ettk_gpu_stream.restype = ctypes.c_void_p
    L.ettk_gpu_profile.argtypes = [vp, ctypes.c_int]
    L.ettk_gpu_soft_noalloc.argtypes = [ctypes.c_int, vp, vp, vp, vp]
    L.ettk_gpu_average.argtypes = [vp, ctypes.c_int, vp, vp, vp, vp]
    L.ettk_gpu_refine_pairs.argtypes = [vp, ctypes.c_int, vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.ettk_gpu_refine_objective.argtypes = [vp, ctypes.c_int, vp, vp, vp, vp, vp]
    L.ettk_gpu_align_pairs_refined.argtypes = [vp, ctypes.c_int, vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_int]
    L.ettk_gpu_refined_objective.argtypes = [vp, ctypes.c_int, vp, vp, vp, vp, vp]
    L.ettk_gpu_score_pairs.argtypes = [vp, ctypes.c_int, vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_float]
    L.ettk_gpu_average_partial.argtypes = [vp, ctypes.c_int, vp, vp, vp, vp, vp, vp]
    L.ettk_gpu_average_finish.argtypes = [vp, vp, vp, vp, vp]
    L.ettk_gpu_wait_probe.argtypes = [vp, ctypes.c_int]
    L.ettk_gpu_classify.argtypes = [vp, ctypes.c_int, vp, vp, vp]
    L.ettk_gpu_variance.argtypes = [vp, ctypes.c_int, vp, vp, vp, vp, vp]
    L.ettk_gpu_symmetrize.argtypes = [vp, vp, ctypes.c_int, vp]
    L.ettk_gpu_symmetrize_rotational.argtypes = [vp, vp, vp]
    L.ettk_gpu_average_spherical_wedge.argtypes = [vp, ctypes.c_int, vp, vp, vp, vp, vp]
    L.ettk_gpu_set_reference_spherical_wedge.argtypes = [vp, ctypes.c_int, vp]
    L.ettk_gpu_representations.argtypes = [vp, ctypes.c_int, vp, ctypes.c_int, P(ctypes.c_int), vp]
    L.ettk_gpu_mean_images.argtypes = [vp, vp, ctypes.c_int, vp, vp]
    L.ettk_gpu_set_reference_mask.argtypes = [vp, ctypes.c_int, vp, ctypes.c_float]
    L.ettk_gpu_get_reference_mask.argtypes = [vp, vp]
    L.ettk_gpu_get_tuning.argtypes = [vp, P(Tuning)]
    L.ettk_gpu_set_tuning.argtypes = [vp, P(Tuning)]
    L.ettk_gpu_autotune.argtypes = [vp, ctypes.c_int, vp, ctypes.c_int, P(Tuning), ctypes.c_char_p, ctypes.c_int]
    L.ettk_gpu_representations_real.argtypes = [vp, ctypes.c_int, vp, ctypes.c_int, ctypes.c_int, P(ctypes.c_int), vp]
    L.ettk_gpu_representation_distances.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int,
                                                    vp]
    L.ettk_gpu_outlier_cutoff.argtypes = [ctypes.c_int, ctypes.c_int, vp, ctypes.c_int, ctypes.c_float,
                                          ctypes.c_int, vp, vp, vp, P(ctypes.c_float)]
    L.ettk_gpu_soft_weights.argtypes = [ctypes.c_int, ctypes.c_int, vp, ctypes.c_int, vp, vp]
    L.ettk_gpu_mra_assign.argtypes = [ctypes.c_int, ctypes.c_int, vp, vp]
    L.ettk_gpu_set_particles_tomogram.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int,
                                                  P(VolumeMeta)]
    L.ettk_gpu_profile_read.argtypes = [vp, ctypes.c_int, ctypes.c_char_p, ctypes.c_int, P(ctypes.c_longlong),
                                        P(ctypes.c_double), P(ctypes.c_double)]
    for name in SYMBOLS:
        getattr(L, name).restype = getattr(L, name).restype or ctypes.c_int
    _lib = L
    return L


def make_params(p):
    return Params(
        N=int(p["N"]), B=int(p["B"]), mask_radius=p["mask_radius"], mask_sigma=p["mask_sigma"],
        square_mask_size=p["square_mask_size"], bp_low=p["bp_low"], bp_high=p["bp_high"],
        bp_low_sigma=p["bp_low_sigma"], bp_high_sigma=p["bp_high_sigma"], bfactor=p.get("bfactor", 0.0),
        restrict_translation=p["restrict_translation"], restrict_rotation=p["restrict_rotation"],
        candidate_peaks=int(p["candidate_peaks"]), number_of_candidates=int(p["number_of_candidates"]),
        wedge_compensation=int(bool(p["wedge_compensation"])), overlap_normalized=int(bool(p["overlap_normalized"])),
        mutual_correlation=int(bool(p.get("mutual_correlation", False))), max_batch=int(p.get("max_batch", 0)),
        wigner_precision=int(p.get("wigner_precision", 0)), fast_coarse_so3=int(p.get("fast_coarse_so3", 0)))


_META_DTYPE = np.dtype({"names": [f[0] for f in VolumeMeta._fields_],
                         "formats": [("<f4", (3,)) if f[0] in ("normal", "position") else
                                     ("<f8", (16,)) if f[0] == "matrix" else "<f4" for f in VolumeMeta._fields_],
                         "offsets": [getattr(VolumeMeta, f[0]).offset for f in VolumeMeta._fields_],
                         "itemsize": ctypes.sizeof(VolumeMeta)})


def make_meta(metas):
    """ctypes array of ettk_volume_meta from volume-list metadata dicts (columns filled with numpy)."""
    n = len(metas)
    a = np.zeros(n, _META_DTYPE)
    if n:
        a["lwedge"] = [m["lwedge"] for m in metas]
        a["uwedge"] = [m["uwedge"] for m in metas]
        a["normal"] = [m.get("normal", (0.0, 0.0, 0.0)) for m in metas]
        eye = np.eye(4)
        a["matrix"] = np.asarray([np.asarray(m.get("matrix", eye), np.float64).reshape(16) for m in metas])
        a["position"] = [m["position"] for m in metas]
        a["cut_offset"] = [m.get("cut_offset", 0.0) for m in metas]
    arr = (VolumeMeta * n).from_buffer_copy(a.tobytes()) if n else (VolumeMeta * 0)()
    return arr
