"""The global-average refinement loop of MPI_Classification (running mode 0, src/MPI_Classification.cpp:914-1160)
driven through the library, on a ProjectionRotationMetric3D.

Per iteration, as the reference does:
1. weights of the global average: 1 for the volumes whose last distance is within the top-fraction cutoff
   (distance <= cutoff, 922-934; every volume before the first alignment, whose distances start at 1);
2. the wedge-weighted average of all volumes under their current transforms (metric.getImage, 938-953), its
   variance when asked (getImageVariance, 976-983);
3. with apply_rotational_symmetry, the cylindrical profile of the average (1005-1024);
4. unless this is the last pass: every volume aligned against the average (getDistances, 1071-1075; the
   average carries its members' spherical wedge when wedge compensation is on, as the reference's average
   computes it lazily), and each transform composed as T_i <- T_i * A_i (or replaced by A_i when the
   alignments are reset, 1064-1112); the cleaned list keeps distance < cutoff (1137-1150).

The n-fold branch (cluster.symmetrize with its default alignment of each rotated copy, inc/em/nbfLoopClustering.h
5951-6030) is not reproduced here: it re-centres every rotated copy with a CCF before averaging.
"""
import numpy as np

from . import clustering, volume_list
from .metric import WedgedSubImage3D

_FULL = {"lwedge": -90.0, "uwedge": 90.0, "normal": (0.0, 0.0, 0.0)}


def _distance_table(dist):
    D = -np.ones((len(dist), 17, 1), np.float32)
    D[:, 0, 0] = dist
    return D


def _write_list(path, volumes, mats, cut_offsets, keep=None):
    rows = []
    for i, v in enumerate(volumes):
        if keep is not None and not keep[i]:
            continue
        rows.append({"lwedge": v.lwedge, "uwedge": v.uwedge, "position": v.position, "normal": v.normal,
                     "matrix": mats[i], "cut_offset": float(cut_offsets[i]), "filename": v.filename})
    volume_list.write(path, rows)


def refine_global(metric, volumes, iterations, top_fraction=1.0, rotational=False, fold=1, reset_alignments=False,
                  variance=False, list_prefix=None):
    """Runs `iterations` align passes against the global average (iterations + 1 averages). `volumes`: list of
    WedgedSubImage3D (their matrices are the starting transforms). Returns a dict with the final average
    ([z][y][x]), the transforms [V][4][4], the last distances, the weights of the final average, the cleaned-list
    mask of the last pass and, with variance=True, the variance maps of every average. With `list_prefix`, each
    pass writes the reference's volume lists (1110-1147): `<prefix>_volumes_pre_centered_<n>.txt` with the new
    transforms and each volume's distance in the cut-offset column, and with a top fraction below 1 the cleaned
    `<prefix>_volumes_pre_centered_clean_<n>.txt` (n = pass + 1)."""
    if fold > 1:
        raise NotImplementedError("n-fold symmetrisation of the global average (aligned copies) is not reproduced")
    V = len(volumes)
    if V < 1 or iterations < 0:
        raise ValueError("need volumes and iterations >= 0")
    N = metric.params["N"]
    T = [np.asarray(v.matrix, np.float64).reshape(4, 4).copy() for v in volumes]
    dist = np.ones(V, np.float32)  # alignments = 1 before the first pass
    clean = np.ones(V, bool)
    variances = []

    def with_matrices(mats):
        return [WedgedSubImage3D(v.image, lwedge=v.lwedge, uwedge=v.uwedge, normal=v.normal, matrix=m,
                                 position=v.position, cut_offset=v.cut_offset, filename=v.filename)
                for v, m in zip(volumes, mats)]

    members = list(range(V))
    for it in range(iterations + 1):
        if top_fraction < 1:
            _, _, keep, _ = clustering.best_alignment_and_clean(_distance_table(dist), 1, top_fraction,
                                                                clustering.AVERAGE)
            weights = keep.astype(np.float32)
        else:
            weights = np.ones(V, np.float32)
        # one upload per pass, with the transforms the alignment starts from; the average and its wedge reset
        # every member's own matrix and apply T explicitly, so they do not depend on it
        metric.set_particles(with_matrices([np.eye(4)] * V if reset_alignments else T))
        avg = metric.average(members, weights, T)
        if variance:
            variances.append(metric.variance(members, weights, T, avg))
        if rotational:
            avg = metric.symmetrize_rotational(avg)
        if it == iterations:
            break
        metric.set_references([WedgedSubImage3D(avg, matrix=np.eye(4), position=(N / 2.0,) * 3, cut_offset=0.0,
                                                **_FULL)])
        if metric.params.get("wedge_compensation"):
            wedge, _ = metric.average_spherical_wedge(members, weights, T)
            metric.set_reference_spherical_wedge(0, wedge)
        D = metric.getDistances([(0, i) for i in range(V)])
        A = D[:, 1:17, 0].astype(np.float64).reshape(V, 4, 4)
        dist = D[:, 0, 0].copy()
        T = [A[i].copy() if reset_alignments else T[i] @ A[i] for i in range(V)]
        if top_fraction < 1:
            clean = clustering.best_alignment_and_clean(_distance_table(dist), 1, top_fraction, clustering.SELECT)[2]
        if list_prefix is not None:
            _write_list("%s_volumes_pre_centered_%d.txt" % (list_prefix, it + 1), volumes, T, dist)
            if top_fraction < 1:
                _write_list("%s_volumes_pre_centered_clean_%d.txt" % (list_prefix, it + 1), volumes, T, dist, clean)
    out = {"average": avg, "matrices": np.stack(T), "distances": dist, "weights": weights, "clean": clean}
    if variance:
        out["variances"] = variances
    return out
