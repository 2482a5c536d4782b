"""The global-average refinement loop of MPI_Classification (running mode 0, src/MPI_Classification.cpp:914-1160)
driven through the library, on a ProjectionRotationMetric3D.

Per iteration, as the reference does:
1. weights of the global average: 1 for the volumes whose last distance is within the top-fraction cutoff
   (distance <= cutoff, 922-934; every volume before the first alignment, whose distances start at 1);
2. the wedge-weighted average of all volumes under their current transforms (metric.getImage, 938-953), its
   variance when asked (getImageVariance, 976-983);
3. with apply_rotational_symmetry, the cylindrical profile of the average (1005-1024);
   Otherwise, with fold > 1, the aligned n-fold symmetrisation (cluster.symmetrize(globalAverage, symmetry) with its
   default alignment, inc/em/nbfLoopClustering.h:5950-6076): for f = 1 .. fold - 1 the transform RotateZ(f * 360 /
   fold) is re-centred by one CCF of the average against itself (executeFourierNewHalf, the found translation
   composed on the right), the average becomes the mean of its getImage under those transforms, and then the mean
   of that image's getImage under the plain rotations RotateZ(i * 360 / fold); the members' alignments become
   T_i * t_f (one per fold, weight w_i each), which the average's spherical wedge then counts;
4. unless this is the last pass: every volume aligned against the average (getDistances, 1071-1075; the
   average carries its members' spherical wedge when wedge compensation is on, as the reference's average
   computes it lazily), and each transform composed as T_i <- T_i * A_i (or replaced by A_i when the
   alignments are reset, 1064-1112); the cleaned list keeps distance < cutoff (1137-1150).

The CCFs of the n-fold step treat the average as an image without a missing wedge (its own Fourier weights are
not restated), and run in a second context of the same parameters so that the members stay uploaded.
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
                  variance=False, list_prefix=None, sym=None):
    """Runs `iterations` align passes against the global average (iterations + 1 averages). `volumes`: list of
    WedgedSubImage3D (their matrices are the starting transforms). Returns a dict with the final average
    ([z][y][x]), the transforms [V][4][4], the last distances, the weights of the final average, the cleaned-list
    mask of the last pass and, with variance=True, the variance maps of every average. With `list_prefix`, each
    pass writes the reference's volume lists (1110-1147): `<prefix>_volumes_pre_centered_<n>.txt` with the new
    transforms and each volume's distance in the cut-offset column, and with a top fraction below 1 the cleaned
    `<prefix>_volumes_pre_centered_clean_<n>.txt` (n = pass + 1). `sym`: the context of the n-fold step's CCFs
    (fold > 1 without rotational symmetry); by default a ProjectionRotationMetric3D of the metric's parameters,
    closed at the end."""
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
    own = sym is None and fold > 1 and not rotational
    if own:
        from .metric import ProjectionRotationMetric3D
        sym = ProjectionRotationMetric3D(metric.params, device=getattr(metric, "device", 0))
    try:
        return _passes(metric, sym, volumes, iterations, top_fraction, rotational, fold, reset_alignments, variance,
                       list_prefix, N, T, dist, clean, variances, members, with_matrices)
    finally:
        if own:
            sym.close()


def symmetrize_aligned(sym, avg, fold):
    """cluster.symmetrize(average, fold) with alignment (inc/em/nbfLoopClustering.h:5950-6076) on a [z][y][x] average:
    returns the symmetrised image and the fold transforms t_f (t_0 = identity, t_f = RotateZ(f * 360 / fold) times the
    translation one CCF of the average against its rotated self finds). `sym`: a metric context used for the CCFs."""
    N = avg.shape[0]
    img = WedgedSubImage3D(avg, matrix=np.eye(4), position=(N / 2.0,) * 3, cut_offset=0.0, **_FULL)
    sym.set_references([img])
    sym.set_particles([img])
    ts = []
    for f in range(fold):
        t = _rot_z(f * 360.0 / fold)
        if f > 0:
            _, t = sym.ccf(0, 0, t)
        ts.append(t)
    return sym.symmetrize(sym.mean_images(avg, ts), fold), ts


def _rot_z(deg):
    """vtkTransform::RotateZ(deg): the rotation matrix of the unit quaternion (cos(a/2), 0, 0, sin(a/2))."""
    a = np.radians(deg) / 2.0
    w, z = np.cos(a), np.sin(a)
    T = np.eye(4)
    T[0, 0] = T[1, 1] = w * w - z * z
    T[0, 1] = -2.0 * w * z
    T[1, 0] = 2.0 * w * z
    T[2, 2] = w * w + z * z
    return T


def _passes(metric, sym, volumes, iterations, top_fraction, rotational, fold, reset_alignments, variance, list_prefix,
            N, T, dist, clean, variances, members, with_matrices):
    V = len(volumes)
    folds = None
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
        elif fold > 1:
            avg, folds = symmetrize_aligned(sym, avg, fold)
        if it == iterations:
            break
        metric.set_references([WedgedSubImage3D(avg, matrix=np.eye(4), position=(N / 2.0,) * 3, cut_offset=0.0,
                                                **_FULL)])
        if metric.params.get("wedge_compensation"):
            if folds is None:
                wedge, _ = metric.average_spherical_wedge(members, weights, T)
            else:  # the alignments T_i * t_f of every fold, weight w_i each
                wedge, _ = metric.average_spherical_wedge([i for i in members for _ in folds],
                                                          np.repeat(weights, len(folds)),
                                                          [T[i] @ t for i in members for t in folds])
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
