"""The global-average refinement loop (MPI_Classification running mode 0, src/MPI_Classification.cpp:914-1160)
as ettk_gb300.classification.refine_global drives it: the order of the library calls, the weights of each
average (top-fraction cutoff, distance <= cutoff), the composition of the transforms (T <- T A, or A when
the alignments are reset), the cleaned list (distance < cutoff), the rotational symmetrisation of each
average and the spherical wedge handed to the reference. A recording stand-in for the metric replaces the
GPU; the GPU calls themselves have their own parity tests."""
import numpy as np
import pytest

from ettk_gb300 import classification
from ettk_gb300.metric import WedgedSubImage3D


def rot_z(deg):
    a = np.deg2rad(deg)
    T = np.eye(4)
    T[:2, :2] = [[np.cos(a), -np.sin(a)], [np.sin(a), np.cos(a)]]
    return T


class FakeMetric:
    def __init__(self, V, wedge_compensation=True, N=8):
        self.params = {"N": N, "wedge_compensation": wedge_compensation}
        self.V = V
        self.log = []
        self.passes = 0
        rng = np.random.default_rng(3)
        # per pass: distances and a small rotation per volume
        self.dist = [rng.uniform(0.2, 0.9, V).astype(np.float32) for _ in range(5)]
        self.ang = [rng.uniform(-10, 10, V) for _ in range(5)]

    def set_particles(self, vols):
        self.log.append(("set_particles", [v.matrix.copy() for v in vols]))

    def average(self, members, weights, mats):
        self.log.append(("average", list(members), np.asarray(weights).copy(), [np.asarray(m).copy() for m in mats]))
        return np.full((8, 8, 8), float(len(self.log)), np.float32)

    def variance(self, members, weights, mats, avg):
        self.log.append(("variance", avg[0, 0, 0]))
        return np.zeros_like(avg)

    def symmetrize_rotational(self, vol):
        self.log.append(("symmetrize_rotational", vol[0, 0, 0]))
        return vol * 2

    def set_references(self, refs):
        self.log.append(("set_references", refs[0].image[0, 0, 0], refs[0].lwedge, refs[0].uwedge))

    def average_spherical_wedge(self, members, weights, mats):
        self.log.append(("average_spherical_wedge", np.asarray(weights).copy()))
        return np.ones((4, 4), np.float32), None

    def set_reference_spherical_wedge(self, r, wedge):
        self.log.append(("set_reference_spherical_wedge", r))

    def getDistances(self, pairs):
        k = self.passes
        self.passes += 1
        D = -np.ones((len(pairs), 17, 1), np.float32)
        for i, (_, p) in enumerate(pairs):
            D[i, 0, 0] = self.dist[k][p]
            D[i, 1:17, 0] = rot_z(self.ang[k][p]).reshape(16)
        self.log.append(("getDistances", len(pairs)))
        return D


def volumes(V):
    rng = np.random.default_rng(1)
    return [WedgedSubImage3D(np.zeros((8, 8, 8), np.float32), matrix=rot_z(rng.uniform(0, 90))) for _ in range(V)]


def calls(m, name):
    return [c for c in m.log if c[0] == name]


def test_composition_and_call_order():
    V, it = 6, 3
    vols = volumes(V)
    m = FakeMetric(V)
    out = classification.refine_global(m, vols, it)
    assert len(calls(m, "average")) == it + 1 and len(calls(m, "getDistances")) == it
    # T <- T A after every pass
    T = [v.matrix for v in vols]
    for k in range(it):
        T = [T[i] @ rot_z(m.ang[k][i]) for i in range(V)]
    assert np.allclose(out["matrices"], np.stack(T))
    assert np.array_equal(out["distances"], m.dist[it - 1])
    # every average used all volumes with weight 1 and the transforms of that moment
    for k, c in enumerate(calls(m, "average")):
        assert (c[2] == 1).all()
    # the reference is the average (full wedge) and carries the members' spherical wedge
    assert all(c[2] == -90.0 and c[3] == 90.0 for c in calls(m, "set_references"))
    assert len(calls(m, "set_reference_spherical_wedge")) == it
    names = [c[0] for c in m.log]
    first = names.index("getDistances")
    assert names[:first] == ["set_particles", "average", "set_references", "average_spherical_wedge",
                             "set_reference_spherical_wedge"]
    # one upload per pass, carrying the transforms the alignment starts from
    sets = calls(m, "set_particles")
    assert len(sets) == it + 1 and all(np.allclose(a, b.matrix) for a, b in zip(sets[0][1], vols))


def test_top_fraction_weights_and_clean_list():
    V, it, f = 11, 2, 0.5
    m = FakeMetric(V)
    out = classification.refine_global(m, volumes(V), it, top_fraction=f)
    avgs = calls(m, "average")
    assert (avgs[0][2] == 1).all()  # alignments start at 1: every volume within the cutoff
    for k in range(1, it + 1):
        d = m.dist[k - 1]
        cut = np.sort(d)[int(np.float32(f) * np.float32(V - 1))]
        assert np.array_equal(avgs[k][2], (d <= cut).astype(np.float32))
    d = m.dist[it - 1]
    cut = np.sort(d)[int(np.float32(f) * np.float32(V - 1))]
    assert np.array_equal(out["clean"], d < cut)
    assert np.array_equal(out["weights"], (d <= cut).astype(np.float32))


def test_reset_alignments():
    V, it = 4, 2
    m = FakeMetric(V)
    out = classification.refine_global(m, volumes(V), it, reset_alignments=True)
    assert np.allclose(out["matrices"], np.stack([rot_z(m.ang[it - 1][i]) for i in range(V)]))
    # every pass aligns the particles from no transform; the averages still use the composed transforms
    sets = calls(m, "set_particles")
    assert all(np.allclose(mm, np.eye(4)) for s_ in sets for mm in s_[1])
    avgs = calls(m, "average")
    assert np.allclose(np.stack(avgs[1][3]), np.stack([rot_z(m.ang[0][i]) for i in range(V)]))


def test_rotational_variance_and_no_wedge():
    V, it = 3, 1
    m = FakeMetric(V, wedge_compensation=False)
    out = classification.refine_global(m, volumes(V), it, rotational=True, variance=True)
    assert len(calls(m, "symmetrize_rotational")) == it + 1
    assert len(out["variances"]) == it + 1
    names = [c[0] for c in m.log]
    # variance of the plain average, then the symmetrisation, and the reference is the symmetrised volume
    assert names.index("variance") < names.index("symmetrize_rotational") < names.index("set_references")
    sym = calls(m, "symmetrize_rotational")[0][1]
    assert calls(m, "set_references")[0][1] == 2 * sym
    assert not calls(m, "set_reference_spherical_wedge")
    assert out["average"][0, 0, 0] == 2 * calls(m, "symmetrize_rotational")[-1][1]


class FakeSym:
    """Stand-in for the n-fold step's context: the CCF adds a known translation to the transform it is given."""

    def __init__(self):
        self.log = []

    def set_references(self, refs):
        self.log.append(("set_references", refs[0].image[0, 0, 0], refs[0].lwedge))

    def set_particles(self, vols):
        self.log.append(("set_particles", vols[0].image[0, 0, 0]))

    def ccf(self, r, p, T):
        S = np.eye(4)
        S[:3, 3] = (len(self.log), -1.0, 0.5)
        self.log.append(("ccf", np.asarray(T).copy(), np.asarray(T) @ S))
        return 0.5, np.asarray(T) @ S

    def mean_images(self, vol, ts):
        self.log.append(("mean_images", vol[0, 0, 0], [np.asarray(t).copy() for t in ts]))
        return vol + 1

    def symmetrize(self, vol, fold):
        self.log.append(("symmetrize", vol[0, 0, 0], fold))
        return vol * 3


def test_nfold_branch():
    """cluster.symmetrize with alignment (inc/em/nbfLoopClustering.h:5950-6076): fold - 1 CCFs of the average against
    itself from RotateZ(f * 360 / fold), the mean of its images under the re-centred transforms, then the plain
    n-fold symmetrisation; the reference is that image and its spherical wedge counts every member under T_i t_f."""
    V, it, fold = 4, 2, 3
    m, s = FakeMetric(V), FakeSym()
    out = classification.refine_global(m, volumes(V), it, fold=fold, sym=s)
    ccf = [c for c in s.log if c[0] == "ccf"]
    assert len(ccf) == (fold - 1) * (it + 1)
    for f in range(1, fold):
        assert np.allclose(ccf[f - 1][1], rot_z(f * 360.0 / fold), atol=1e-12)
    means = [c for c in s.log if c[0] == "mean_images"]
    syms = [c for c in s.log if c[0] == "symmetrize"]
    assert len(means) == len(syms) == it + 1 and all(c[2] == fold for c in syms)
    ts = means[0][2]
    assert len(ts) == fold and np.allclose(ts[0], np.eye(4))
    # the transforms the mean uses are the CCF outputs
    for f in range(1, fold):
        assert np.allclose(ts[f], ccf[f - 1][2])
    # the reference of the alignment is the symmetrised image
    refs = calls(m, "set_references")
    assert refs[0][1] == 9.0  # the first average holds 2: mean of images + 1, symmetrisation * 3
    # the spherical wedge: every member once per fold, weight 1 each
    w = calls(m, "average_spherical_wedge")
    assert len(w) == it and len(w[0][1]) == V * fold
    assert out["average"][0, 0, 0] == syms[-1][1] * 3


def test_volume_lists(tmp_path):
    from ettk_gb300 import volume_list
    V, it, f = 9, 2, 0.6
    m = FakeMetric(V)
    vols = volumes(V)
    prefix = str(tmp_path / "run")
    out = classification.refine_global(m, vols, it, top_fraction=f, list_prefix=prefix)
    for n in range(1, it + 1):
        rows = volume_list.read("%s_volumes_pre_centered_%d.txt" % (prefix, n))
        assert len(rows) == V
        # the distance of the pass in the cut-offset column (6 significant digits, as the reference prints)
        assert np.allclose([r["cut_offset"] for r in rows], m.dist[n - 1], rtol=1e-5)
        d = m.dist[n - 1]
        cut = np.sort(d)[int(np.float32(f) * np.float32(V - 1))]
        clean = volume_list.read("%s_volumes_pre_centered_clean_%d.txt" % (prefix, n))
        assert len(clean) == int((d < cut).sum())
    last = volume_list.read("%s_volumes_pre_centered_%d.txt" % (prefix, it))
    assert np.allclose(np.stack([r["matrix"] for r in last]), out["matrices"], atol=1e-5)
