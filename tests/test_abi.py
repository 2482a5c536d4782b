"""The C ABI library builds, loads and exports every symbol include/ettk_gpu.h declares (CPU)."""
import os
import re

from ettk_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "ettk_gpu.h")).read()
    return sorted(set(re.findall(r"\b(ettk_gpu_[a-z_]+)\s*\(", txt)))


def test_header_symbols_exported():
    L = _lib.load()
    names = declared_symbols()
    assert names, "no declarations found"
    for n in names:
        assert hasattr(L, n), n


def test_create_rejects_bad_params():
    import ctypes
    L = _lib.load()
    p = _lib.make_params({"N": 48, "B": 16, "mask_radius": 19, "mask_sigma": 2, "square_mask_size": 2,
                          "bp_low": .01, "bp_high": .5, "bp_low_sigma": .01, "bp_high_sigma": .05,
                          "restrict_translation": 6, "restrict_rotation": 180, "candidate_peaks": 5,
                          "number_of_candidates": 1, "wedge_compensation": 1, "overlap_normalized": 1})
    ctx = ctypes.c_void_p()
    assert L.ettk_gpu_create(0, ctypes.byref(p), ctypes.byref(ctx)) == _lib.ETTK_ERR_ARG
    assert not ctx.value
