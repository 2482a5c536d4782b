"""Regenerates the golden fixtures in this directory (run in a tree where the reference is present).

soft_bw8.npz   SOFT 1.0's own bandwidth-8 test signals (external/soft-1.0/randomS2sig_bw8.dat and
               randomS2sigA_bw8.dat, real parts) pushed through the reference's SOFT library built from
               its sources (oracle/_ref): the SO(3) correlation as nbfProjectionRotationMetric3D::soft
               computes it, and an S^2 rotation as ::harmonics does.
align32_b16.npz  oracle alignments of the first particles of the 32^3 B=16 workload (a regression pin
               of the oracle itself), with a checksum of the generated particles.
align128_b64.npz oracle alignments of the first two particles of the 128^3 B=64 workload (the large-size
               path: (2N)^3 = 256^3 spherical projections, B=64 SO(3) correlations), with a checksum.
rotsym_n16.npz the rotational-symmetry step of the classification loop run by the reference's own
               cylindrical-domain classes (oracle/_ref/libblitz_ref.so) on a seeded 16^3 volume and on a
               volume with an off-axis blob.
clustering.npz soft class weights, outlier cutoffs (three rules, several fractions) and the MRA class
               choice of seeded distance tables with ties, from the class-selection rules in the reference's expressions
               (oracle/_ref/libblitz_ref.so).
filter_pins.npz the half-grid Fourier filters (band-pass, B-factor), normalizeFourierHalf of seeded spectra and the
               CCF distance of seeded peak inputs, in the reference's own Blitz expressions (oracle/_ref/libblitz_ref.so).
repr_dist.npz  distance matrices between seeded low-dimensional representations (depth 3 with wedge bits,
               and depth 1) from the representation-distance loop in the reference's Blitz expressions
               (oracle/_ref/libblitz_ref.so), overlap-normalised and averaged.

Usage: python make_golden.py [soft|align32|align128|rotsym|repr|clustering|pins ...]   (no argument: all)
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pyoracle  # noqa: E402
from ettk_gb300 import synthetic  # noqa: E402

# The reference tree (read in place for SOFT's own test signals): ETTK_REFERENCE_ROOT must name it.
REF = os.environ.get("ETTK_REFERENCE_ROOT")


def read_s2(path):
    v = np.loadtxt(path)
    return v[0::2].reshape(16, 16)


def align_golden(name, n, out):
    ds = synthetic.generate(name, n_particles=n)
    dist, mats = [], []
    for i in range(n):
        o = pyoracle.align(ds.params, ds.references[0], ds.ref_meta[0], ds.particles[i], ds.meta[i])
        dist.append(o["distance"])
        mats.append(o["matrix"])
    np.savez_compressed(os.path.join(HERE, out), n=n, distance=np.array(dist), matrix=np.array(mats),
                        particles_sha256=hashlib.sha256(ds.particles.tobytes()).hexdigest())


def rotsym_inputs():
    rng = np.random.default_rng(2024)
    noise = rng.standard_normal((16, 16, 16)).astype(np.float32)
    z, y, x = np.mgrid[0:16, 0:16, 0:16]
    blob = np.exp(-((x - 11.3) ** 2 + (y - 6.0) ** 2 + (z - 8.5) ** 2) / 6.0).astype(np.float32)
    return np.stack([noise, blob])


def repr_inputs():
    rng = np.random.default_rng(77)
    V, K = 13, 240
    R3 = np.zeros((V, K, 3), np.float32)
    R3[:, :, 0] = rng.standard_normal((V, K)) * (1 + np.arange(K) % 5)
    R3[:, :, 1] = rng.standard_normal((V, K))
    R3[:, :, 2] = (rng.random((V, K)) > 0.3).astype(np.float32)
    R3[4, :, 2] = 0  # a volume sharing no coefficient with any other: overlap 0 falls back to the mean
    R1 = rng.standard_normal((V, K, 1)).astype(np.float32)
    return R3, R1


CLUSTER_FRACTIONS = (0.0, 0.29, 0.5, 0.9, 1.0)


def clustering_inputs():
    rng = np.random.default_rng(31)
    d = rng.uniform(0.2, 0.9, (101, 4)).astype(np.float32)
    d[::7] = np.round(d[::7] * 8) / 8  # ties within and across volumes
    d[5, :] = -d[5, :]                  # negative distances: |.| only for rule 0
    return d


def mra_inputs():
    rng = np.random.default_rng(41)
    S = rng.uniform(0.3, 0.8, (60, 3, 3)).astype(np.float32)
    S[::5] = np.round(S[::5] * 4) / 4  # ties between the alignments of a volume
    return S


# Fourier filters (N, low, high, low sigma, high sigma, bfactor) of the filter pin: the workloads' band-passes with and
# without a B-factor, another band, and no band-pass at all
FILTER_CASES = [(32, .01, .5, .01, .05, 0.0), (64, .01, .5, .01, .05, 0.0), (64, .01, .5, .01, .05, 2.0),
                (32, .05, .3, .02, .08, .5), (16, 0.0, 1.0, .1, .1, 0.0)]


def pin_inputs():
    """Seeded half spectra for the normalisation pin and CCF peak inputs for the distance pin."""
    rng = np.random.default_rng(20261204)
    spectra = [rng.standard_normal((N, N, N // 2 + 1)) + 1j * rng.standard_normal((N, N, N // 2 + 1)) for N in (8, 16)]
    n = 64
    dist = {"k1_m": rng.uniform(0.5, 3.0, n).astype(np.float32), "maxT": rng.uniform(-1.0, 3.0, n),
            "sum_wf": rng.uniform(1e3, 1e5, n), "sum_f": rng.uniform(1e5, 2e5, n),
            "overlap": rng.integers(0, 2, n).astype(np.int32), "N": rng.choice([16, 32, 64, 128], n).astype(np.int32)}
    return spectra, dist


def main(which):
    if "pins" in which:
        spectra, dist = pin_inputs()
        out = {}
        for c, (N, lo, hi, lv, hv, bf) in enumerate(FILTER_CASES):
            f = pyoracle.ref_filter_half(dict(N=N, bp_low=lo, bp_high=hi, bp_low_sigma=lv, bp_high_sigma=hv, bfactor=bf))
            if f is None:
                raise SystemExit("build oracle/_ref first (oracle/build_ref.sh)")
            out["filter_%d" % c] = f
        for k, F in enumerate(spectra):
            G, norm = pyoracle.ref_normalize_half(F)
            out["spectrum_%d" % k], out["normalized_%d" % k], out["norm_%d" % k] = F, G, np.float32(norm)
        for key, v in dist.items():
            out["dist_" + key] = v
        out["distance"] = np.array([pyoracle.ref_ccf_distance(float(dist["k1_m"][i]), float(dist["maxT"][i]),
                                                              float(dist["sum_wf"][i]), float(dist["sum_f"][i]),
                                                              int(dist["overlap"][i]), int(dist["N"][i]))
                                    for i in range(len(dist["N"]))], np.float32)
        np.savez_compressed(os.path.join(HERE, "filter_pins.npz"), **out)
    if "clustering" in which:
        d = clustering_inputs()
        sw = pyoracle.ref_soft_weights(d)
        if sw is None:
            raise SystemExit("build oracle/_ref first (oracle/build_ref.sh)")
        out = {"d": d, "W": sw[0], "radii": sw[1]}
        for rule in (0, 1, 2):
            for f in CLUSTER_FRACTIONS:
                b, dist, keep = pyoracle.ref_cutoff(d, f, rule)
                out["best_%d_%g" % (rule, f)], out["dist_%d_%g" % (rule, f)], out["keep_%d_%g" % (rule, f)] = b, dist, keep
        S = mra_inputs()
        out["S"], out["mra_labels"] = S, pyoracle.ref_mra_assign(S)
        np.savez_compressed(os.path.join(HERE, "clustering.npz"), **out)
    if "repr" in which:
        R3, R1 = repr_inputs()
        out = {"R3": R3, "R1": R1}
        for norm in (0, 1):
            d3 = pyoracle.ref_representation_distances(R3, norm)
            if d3 is None:
                raise SystemExit("build oracle/_ref first (oracle/build_ref.sh)")
            out["D3_%d" % norm] = d3
            out["D1_%d" % norm] = pyoracle.ref_representation_distances(R1, norm)
        np.savez_compressed(os.path.join(HERE, "repr_dist.npz"), **out)
    if "rotsym" in which:
        vols = rotsym_inputs()
        outs = [pyoracle.ref_symmetrize_rotational(v) for v in vols]
        if outs[0] is None:
            raise SystemExit("build oracle/_ref first (oracle/build_ref.sh)")
        np.savez_compressed(os.path.join(HERE, "rotsym_n16.npz"), vol=vols, out=np.stack(outs))
    if "align32" in which:
        align_golden("align32_b16", 4, "align32_b16.npz")
    if "align128" in which:
        align_golden("align128_b64", 2, "align128_b64.npz")
    if "soft" not in which:
        return
    R = pyoracle.ref_lib()
    if R is None:
        raise SystemExit("build oracle/_ref first (oracle/build_ref.sh)")
    if not REF:
        raise SystemExit("set ETTK_REFERENCE_ROOT to the reference tree (SOFT's test signals are read from it)")
    soft_dir = os.path.join(REF, "external", "soft-1.0")
    sig = read_s2(os.path.join(soft_dir, "randomS2sig_bw8.dat"))
    pat = read_s2(os.path.join(soft_dir, "randomS2sigA_bw8.dat"))
    B = 8
    C = np.zeros((16, 16, 16))
    R.ref_soft(B, np.ascontiguousarray(sig), np.ascontiguousarray(pat), C)
    angles = np.array([0.3, 1.2, 2.0])
    Rr = np.zeros((16, 16))
    R.ref_rotate(B, np.ascontiguousarray(sig), *angles, Rr)
    np.savez_compressed(os.path.join(HERE, "soft_bw8.npz"), sig=sig, pat=pat, C=C, R=Rr, angles=angles)


if __name__ == "__main__":
    main(sys.argv[1:] or ["soft", "align32", "align128", "rotsym", "repr", "clustering", "pins"])
