"""The Fourier filter, the spectrum normalisation and the CCF distance of the oracle against the reference's own Blitz
expressions (oracle/shim/filter_blitz_wrap.cpp on the reference's vendored Blitz 0.9, frozen in
tests/golden/filter_pins.npz by tests/golden/make_golden.py, and run live where oracle/_ref is built):

- nbfFourierFilter::updateFilterHalf with buildBandPassHalf / buildBFactorHalf (inc/em/nbfFourierFilter.h:492-546,
  737-797): the half-grid filter, bit for bit;
- nbfCorrelationImageMetric::normalizeFourierHalf (inc/em/nbfCorrelationImageMetric.h:497-530): the norm and the
  normalised spectrum, bit for bit;
- the distance of nbfFourierImageMetric::executeFourierNewHalf (inc/em/nbfFourierImageMetric.h:1249-1258), bit for
  bit (the float correlationPeak divided twice in float by the upsampled grid's size).
The library builds its filter with the oracle's expressions and its distance with the same float steps (k_score).
"""
import os

import numpy as np
import pytest

import pyoracle

GOLDEN = np.load(os.path.join(os.path.dirname(__file__), "golden", "filter_pins.npz"))
FILTER_CASES = [(32, .01, .5, .01, .05, 0.0), (64, .01, .5, .01, .05, 0.0), (64, .01, .5, .01, .05, 2.0),
                (32, .05, .3, .02, .08, .5), (16, 0.0, 1.0, .1, .1, 0.0)]


def _params(N, lo, hi, lv, hv, bf):
    return dict(N=N, B=8, mask_radius=N / 2 - 5, mask_sigma=2.0, square_mask_size=2, bp_low=lo, bp_high=hi,
                bp_low_sigma=lv, bp_high_sigma=hv, bfactor=bf, restrict_translation=6.0, restrict_rotation=180.0,
                candidate_peaks=5, number_of_candidates=1, wedge_compensation=True, overlap_normalized=True)


@pytest.mark.parametrize("case", range(len(FILTER_CASES)))
def test_filter_bit_exact(case):
    p = _params(*FILTER_CASES[case])
    _, _, f = pyoracle.masks(p)
    assert np.array_equal(f, GOLDEN["filter_%d" % case])
    live = pyoracle.ref_filter_half(p)
    if live is not None:
        assert np.array_equal(f, live)


@pytest.mark.parametrize("k", [0, 1])
def test_normalize_bit_exact(k):
    F = GOLDEN["spectrum_%d" % k]
    G, norm = pyoracle.normalize_half(F)
    assert np.float32(norm) == GOLDEN["norm_%d" % k]
    assert np.array_equal(G, GOLDEN["normalized_%d" % k])
    live = pyoracle.ref_normalize_half(F)
    if live is not None:
        assert np.array_equal(G, live[0]) and np.float32(norm) == np.float32(live[1])


def test_distance_bit_exact():
    n = len(GOLDEN["dist_N"])
    d = np.array([pyoracle.ccf_distance(float(GOLDEN["dist_k1_m"][i]), float(GOLDEN["dist_maxT"][i]),
                                        float(GOLDEN["dist_sum_wf"][i]), float(GOLDEN["dist_sum_f"][i]),
                                        int(GOLDEN["dist_overlap"][i]), int(GOLDEN["dist_N"][i])) for i in range(n)],
                 np.float32)
    assert np.array_equal(d, GOLDEN["distance"])
