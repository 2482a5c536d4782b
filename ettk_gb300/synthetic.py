"""Seeded synthetic sub-volume data for the alignment workloads.

No public dataset exists for this path, so the benchmark and parity workloads use
synthetic particles built with the shapes and value distributions of the
workload definitions:

* a reference = sum of isotropic Gaussian blobs on a centred N^3 grid;
* a particle = the reference rotated by a uniform SO(3) rotation (trilinear
  interpolation), shifted by an integer offset (or, for the local-refinement workload, a continuous one), multiplied
  in Fourier space by a
  single-axis missing wedge about Y (the binary plane test of nbfWedge3D,
  inc/em/nbfWedge3D.h:351-356), plus white Gaussian noise at the requested SNR;
* metadata in the reference's volume-list vocabulary: lwedge/uwedge = -tilt/+tilt,
  normal = (0, 0, in-plane tilt-axis angle), identity matrix, position = N/2.

The particle is stored in the tilt-series frame (wedge about Y there). The
reference metric reads it through Euler(normal) (inc/em/nbfWedgedSubImage3D.h:741-763),
so the aligner sees the tilt axis rotated in-plane by the normal angle. With
E = Euler(normal) and particle rotation G, shift s, the pose the metric should
recover is T = [E^-1 G | E^-1 s] (the reslice maps box coordinates x to
stored coordinates E*T*x + N/2).

Random streams come from SeedSequence(seed).spawn(6) in the order
blobs, poses, shifts, wedges, noise, classes; seed = 20261203 + workload index.
"""
from dataclasses import dataclass, field

import numpy as np
from scipy import ndimage

SEED_BASE = 20261203


@dataclass
class Workload:
    name: str
    index: int
    N: int
    B: int
    n_particles: int
    n_blobs: int
    sigma: tuple
    radius: float
    amp: tuple
    shift: int
    snr: float
    tilt: tuple          # (lo, hi) of the +-tilt range in degrees; lo == hi -> fixed
    inplane: bool        # random in-plane tilt-axis angle
    restrict_translation: float
    n_refs: int = 1
    shared_fraction: float = 0.0
    continuous_shift: bool = False  # shifts uniform in [-shift, shift] (sub-voxel) instead of integers


WORKLOADS = {
    # 32^3 single reference, fixed +-60 wedge, B=16, translation search +-6
    "align32_b16": Workload("align32_b16", 0, 32, 16, 200, 20, (1.5, 3.0), 10.0, (0.5, 1.0), 4, 0.1,
                            (60.0, 60.0), False, 6.0),
    # 64^3 single reference, per-particle wedges, B=32
    "align64_b32": Workload("align64_b32", 1, 64, 32, 2000, 40, (3.0, 6.0), 20.0, (0.5, 1.0), 8, 0.05,
                            (45.0, 70.0), True, 10.0),
    # 64^3, 10 references with 30% shared blobs
    "mra64_b32": Workload("mra64_b32", 2, 64, 32, 8000, 40, (3.0, 6.0), 20.0, (0.5, 1.0), 8, 0.05,
                          (45.0, 70.0), True, 10.0, n_refs=10, shared_fraction=0.3),
    # 64^3 local-refinement workload: continuous poses and sub-voxel shifts uniform in +-8, per-particle wedges
    "refine64_b32": Workload("refine64_b32", 3, 64, 32, 4000, 40, (3.0, 6.0), 20.0, (0.5, 1.0), 8, 0.05,
                             (45.0, 70.0), True, 10.0, continuous_shift=True),
    # 32^3, 3 references with 30% shared blobs (small multireference classification case for tests)
    "mra32_b16": Workload("mra32_b16", 5, 32, 16, 60, 20, (1.5, 3.0), 10.0, (0.5, 1.0), 4, 0.1,
                          (60.0, 60.0), False, 6.0, n_refs=3, shared_fraction=0.3),
    # 128^3 precision stress, B=64
    "align128_b64": Workload("align128_b64", 4, 128, 64, 1000, 80, (3.0, 8.0), 40.0, (0.5, 1.0), 8, 0.05,
                             (45.0, 70.0), True, 10.0),
}


def default_params(w: Workload):
    """Alignment parameters of the reference's AlignRigid3D-style setup
    (src/AlignRigid3D.cpp:69-73,121) with the workload's bandwidth and search range."""
    N = w.N
    return {
        "N": N, "B": w.B,
        "mask_radius": N / 2 - 5, "mask_sigma": 2.0, "square_mask_size": 2,
        "bp_low": 0.01, "bp_high": 0.5, "bp_low_sigma": 0.01, "bp_high_sigma": 0.05,
        "bfactor": 0.0,
        "restrict_translation": w.restrict_translation, "restrict_rotation": 180.0,
        "candidate_peaks": 5, "number_of_candidates": 1,
        "wedge_compensation": True, "overlap_normalized": True,
    }


def blob_volume(rng, N, n_blobs, sigma, radius, amp, centres=None):
    g = np.arange(N) - N / 2.0
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    vol = np.zeros((N, N, N), np.float64)
    if centres is None:
        centres = []
        while len(centres) < n_blobs:
            c = rng.uniform(-radius, radius, 3)
            if np.linalg.norm(c) <= radius:
                centres.append(c)
        sig = rng.uniform(sigma[0], sigma[1], n_blobs)
        amps = rng.uniform(amp[0], amp[1], n_blobs)
        centres = list(zip(centres, sig, amps))
    for (c, s, a) in centres:
        vol += a * np.exp(-((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) / (2 * s * s))
    return vol.astype(np.float32), centres


def random_rotation(rng):
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
        [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
        [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
    ])


def euler_normal(normal):
    """Rotation part of RotateZ(-n2) RotateX(-n0) RotateZ(-n1) (degrees)."""
    def rz(a):
        a = np.deg2rad(a)
        return np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])

    def rx(a):
        a = np.deg2rad(a)
        return np.array([[1, 0, 0], [0, np.cos(a), -np.sin(a)], [0, np.sin(a), np.cos(a)]])
    return rz(-normal[2]) @ rx(-normal[0]) @ rz(-normal[1])


def wedge_mask_full(N, lwedge, uwedge):
    """Binary single-axis wedge about Y on the unshifted FFT grid (numpy order [kz][ky][kx])."""
    u = np.deg2rad(90.0 - uwedge)
    lo = np.deg2rad(90.0 - lwedge)
    n1 = np.array([np.cos(-u), 0.0, -np.sin(-u)])
    n2 = np.array([np.cos(-lo), 0.0, -np.sin(-lo)])
    f = np.fft.fftfreq(N) * N
    kz, ky, kx = np.meshgrid(f, f, f, indexing="ij")
    a = n1[0] * kx + n1[1] * ky + n1[2] * kz
    b = n2[0] * kx + n2[1] * ky + n2[2] * kz
    return (a * b <= 0).astype(np.float64)


def make_particle(ref, G, s, lwedge, uwedge, snr, rng_noise):
    N = ref.shape[0]
    c = N / 2.0
    g = np.arange(N) - c
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    pts = np.stack([x - s[0], y - s[1], z - s[2]], 0).reshape(3, -1)
    src = G.T @ pts  # G^-1 (y - s)
    coords = np.stack([src[2] + c, src[1] + c, src[0] + c], 0)
    clean = ndimage.map_coordinates(ref.astype(np.float64), coords, order=1, mode="constant", cval=0.0).reshape(N, N, N)
    if uwedge - lwedge < 180:
        clean = np.real(np.fft.ifftn(np.fft.fftn(clean) * wedge_mask_full(N, lwedge, uwedge)))
    var = clean.var()
    noise = rng_noise.standard_normal(clean.shape) * np.sqrt(var / snr)
    return (clean + noise).astype(np.float32)


@dataclass
class Dataset:
    workload: Workload
    params: dict
    references: list            # list of float32 [z][y][x]
    ref_meta: list
    particles: np.ndarray       # float32 [P][z][y][x]
    meta: list                  # per-particle dicts
    truth: list = field(default_factory=list)   # per-particle dict(rotation 3x3, shift 3, ref index)


def generate(name, n_particles=None, seed=None):
    w = WORKLOADS[name]
    seed = SEED_BASE + w.index if seed is None else seed
    streams = [np.random.default_rng(s) for s in np.random.SeedSequence(seed).spawn(6)]
    r_blobs, r_poses, r_shifts, r_wedges, r_noise, r_classes = streams
    N = w.N
    P = w.n_particles if n_particles is None else n_particles
    refs = []
    if w.n_refs == 1:
        vol, _ = blob_volume(r_blobs, N, w.n_blobs, w.sigma, w.radius, w.amp)
        refs.append(vol)
    else:
        n_shared = int(round(w.shared_fraction * w.n_blobs))
        _, shared = blob_volume(r_blobs, N, n_shared, w.sigma, w.radius, w.amp) if n_shared else (None, [])
        for _r in range(w.n_refs):
            _, own = blob_volume(r_blobs, N, w.n_blobs - n_shared, w.sigma, w.radius, w.amp)
            vol, _ = blob_volume(r_blobs, N, 0, w.sigma, w.radius, w.amp, centres=shared + own)
            refs.append(vol)
    ref_meta = [{"lwedge": -90.0, "uwedge": 90.0, "normal": (0.0, 0.0, 0.0), "matrix": np.eye(4),
                 "position": (N / 2.0,) * 3, "cut_offset": 0.0, "filename": "reference_%d.mrc" % i}
                for i in range(len(refs))]
    if w.n_refs > 1:
        props = r_classes.dirichlet([0.5] * w.n_refs)
        labels = r_classes.choice(w.n_refs, size=P, p=props)
    else:
        labels = np.zeros(P, dtype=int)
    parts = np.zeros((P, N, N, N), np.float32)
    meta, truth = [], []
    for i in range(P):
        G = random_rotation(r_poses)
        if w.continuous_shift:
            s = r_shifts.uniform(-w.shift, w.shift, 3)
        else:
            s = r_shifts.integers(-w.shift, w.shift + 1, 3).astype(np.float64)
        tilt = w.tilt[0] if w.tilt[0] == w.tilt[1] else r_wedges.uniform(w.tilt[0], w.tilt[1])
        phi = r_wedges.uniform(0.0, 360.0) if w.inplane else 0.0
        lw, uw = -float(np.float32(tilt)), float(np.float32(tilt))
        parts[i] = make_particle(refs[labels[i]], G, s, lw, uw, w.snr, r_noise)
        normal = (0.0, 0.0, float(np.float32(phi)))
        E = euler_normal(normal)
        meta.append({"lwedge": lw, "uwedge": uw, "normal": normal, "matrix": np.eye(4),
                     "position": (N / 2.0,) * 3, "cut_offset": 0.0, "filename": "particle_%05d.mrc" % i})
        truth.append({"rotation": E.T @ G, "shift": E.T @ s, "ref": int(labels[i])})
    return Dataset(w, default_params(w), refs, ref_meta, parts, meta, truth)
