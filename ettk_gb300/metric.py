"""Host-side mirror of the reference's metric classes for the alignment path.

`ProjectionRotationMetric3D` keeps the method names and argument meaning of
nbfProjectionRotationMetric3D<float> / nbfCorrelationImageMetric<float,3> / nbfImageMetric<float,3>
(inc/em/nbfProjectionRotationMetric3D.h:90-196, inc/em/nbfCorrelationImageMetric.h:50-121,
inc/em/nbfImageMetric.h:33-99) and computes on the GPU through the C ABI of include/ettk_gpu.h.
Volumes are `WedgedSubImage3D` objects (fixed images plus volume-list metadata).
"""
import ctypes

import numpy as np

from . import _lib


class EttkError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("ettk_gpu error %d: %s" % (code, msg))
        self.code = code


class WedgedSubImage3D:
    """A fixed-image particle with the metadata of one volume-list row
    (nbfWedgedSubImage3D, inc/em/nbfWedgedSubImage3D.h:17-185)."""

    def __init__(self, image, lwedge=-90.0, uwedge=90.0, normal=(0.0, 0.0, 0.0), matrix=None, position=None,
                 cut_offset=0.0, filename="NA"):
        self.image = np.ascontiguousarray(image, dtype=np.float32)  # [z][y][x]
        n = self.image.shape[0]
        self.lwedge, self.uwedge = float(lwedge), float(uwedge)
        self.normal = tuple(float(x) for x in normal)
        self.matrix = np.eye(4) if matrix is None else np.asarray(matrix, np.float64).reshape(4, 4)
        self.position = tuple(position) if position is not None else (n / 2.0,) * 3
        self.cut_offset = float(cut_offset)
        self.filename = filename

    def meta(self):
        return {"lwedge": self.lwedge, "uwedge": self.uwedge, "normal": self.normal, "matrix": self.matrix,
                "position": self.position, "cut_offset": self.cut_offset}


class ProjectionRotationMetric3D:
    """GPU drop-in for nbfProjectionRotationMetric3D<float> in alignment_mode 3."""

    def __init__(self, params, device=0):
        self.L = _lib.load()
        self.params = dict(params)
        self.device = device
        self._ctx = ctypes.c_void_p()
        P = _lib.make_params(self.params)
        self._check(self.L.ettk_gpu_create(device, ctypes.byref(P), ctypes.byref(self._ctx)), "create")
        self._refs = None
        self._parts = None
        self.input1 = self.input2 = None
        self.transform = np.eye(4)
        self.correlationPeak = None

    def close(self):
        if self._ctx:
            self.L.ettk_gpu_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != _lib.ETTK_OK:
            buf = ctypes.create_string_buffer(512)
            if self._ctx:
                self.L.ettk_gpu_last_error(self._ctx, buf, 512)
            raise EttkError(rc, "%s: %s" % (what, buf.value.decode(errors="replace")))

    # -- volume sets (getDistances' list1 / list2) -------------------------------------------
    def set_references(self, volumes):
        vols = np.ascontiguousarray(np.stack([v.image for v in volumes]), np.float32)
        meta = _lib.make_meta([v.meta() for v in volumes])
        self._check(self.L.ettk_gpu_set_references(self._ctx, len(volumes), vols.ctypes.data, meta), "set_references")
        self._refs = volumes

    def set_particles(self, volumes, stacked=None):
        vols = stacked if stacked is not None else np.stack([v.image for v in volumes])
        vols = np.ascontiguousarray(vols, np.float32)
        meta = _lib.make_meta([v.meta() for v in volumes])
        self._check(self.L.ettk_gpu_set_particles(self._ctx, len(volumes), vols.ctypes.data, meta), "set_particles")
        self._parts = volumes

    def set_particles_tomogram(self, tomogram, metas):
        """Particles cut from one tomogram ([z][y][x] float32) at metas[i]["position"] (voxel coordinates of
        the tomogram), as nbfWedgedSubImage3D's tomogram path; metas are volume-list metadata dicts."""
        t = np.ascontiguousarray(tomogram, np.float32)
        nz, ny, nx = t.shape
        meta = _lib.make_meta(metas)
        self._check(self.L.ettk_gpu_set_particles_tomogram(self._ctx, nx, ny, nz, t.ctypes.data, len(metas), meta),
                    "set_particles_tomogram")
        self._parts = [None] * len(metas)

    def set_particles_device(self, dev_ptr, metas):
        meta = _lib.make_meta(metas)
        self._check(self.L.ettk_gpu_set_particles_device(self._ctx, len(metas), ctypes.c_void_p(dev_ptr), meta),
                    "set_particles_device")

    # -- nbfImageMetric interface (single pair) ------------------------------------------------
    def setInput1(self, v):
        self.set_references([v])
        self.input1 = v

    def setInput2(self, v):
        self.set_particles([v])
        self.input2 = v

    def getDistance(self):
        D = self.getDistances([(0, 0)])
        self.correlationPeak = float(D[0, 0, 0])
        self.transform = D[0, 1:17, 0].astype(np.float64).reshape(4, 4)
        return self.correlationPeak

    def getTransform(self):
        return self.transform

    # -- nbfCorrelationImageMetric::getDistances (core overload) ---------------------------------
    def getDistances(self, indexes, D=None, cols=17, ncand=1, typeOfMetric=3, restrict_translation=-1.0):
        """indexes: sequence of (reference index, particle index). D: float32 (npairs, cols, ncand),
        rows pre-filled with -1 are computed (others skipped). The metric types of nbfCorrelationImageMetric::
        getDistances (inc/em/nbfCorrelationImageMetric.h:1918-1930):
          3: the alignment, refinement off (SO(3) search and CCF candidates);
          2: one CCF per pair at the particle's own alignment matrix (nbfFourierImageMetricCore) with the translation
             restriction restrict_translation (negative: the metric's);
          0: the alignment with refinement on; the Powell refinement of each candidate is replaced by the fast
             form's batched gradient refinement (getDistancesRefined, default iterations);
          1: refinement from the particle's own alignment (nbfFourierImageMetric): the type-2 CCF, then the
             batched gradient refinement of that pose (refine)."""
        idx = np.ascontiguousarray(np.asarray(indexes, np.int32).reshape(-1, 2))
        n = idx.shape[0]
        if D is None:
            D = -np.ones((n, cols, ncand), np.float32)
        assert D.dtype == np.float32 and D.flags.c_contiguous and D.shape[0] == n
        if typeOfMetric == 2:
            self._check(self.L.ettk_gpu_score_pairs(self._ctx, n, idx.ctypes.data, D.ctypes.data, D.shape[1],
                                                    D.shape[2], float(restrict_translation)), "score_pairs")
        elif typeOfMetric == 3:
            self._check(self.L.ettk_gpu_align_pairs(self._ctx, n, idx.ctypes.data, D.ctypes.data, D.shape[1],
                                                    D.shape[2]), "align_pairs")
        elif typeOfMetric == 0:
            return self.getDistancesRefined(indexes, D=D)
        elif typeOfMetric == 1:
            todo = D[:, 0, 0] == -1
            self._check(self.L.ettk_gpu_score_pairs(self._ctx, n, idx.ctypes.data, D.ctypes.data, D.shape[1],
                                                    D.shape[2], float(restrict_translation)), "score_pairs")
            if todo.any():
                sub = np.ascontiguousarray(D[todo])
                self.refine(idx[todo], sub)
                D[todo] = sub
        else:
            raise ValueError("typeOfMetric 0, 1, 2 or 3")
        return D

    # -- nbfWedgedAverageImage3D::setAlignments + getImage ----------------------------------------
    def average(self, particles, weights, matrices):
        """Class average of particles (indices into the particle set) with weights and 4x4 alignment
        matrices; returns [z][y][x] float32 (RMS 1)."""
        n = len(particles)
        N = self.params["N"]
        idx = np.ascontiguousarray(particles, np.int32)
        w = np.ascontiguousarray(weights, np.float32)
        M = np.ascontiguousarray(np.asarray(matrices, np.float64).reshape(n, 16))
        out = np.zeros((N, N, N), np.float32)
        self._check(self.L.ettk_gpu_average(self._ctx, n, idx.ctypes.data, w.ctypes.data, M.ctypes.data,
                                            out.ctypes.data), "average")
        return out

    def average_partial(self, particles, weights, matrices):
        """getImageMPI's accumulators (re, im, acc), each float64 [x][y][kz] (N, N, N/2 + 1), for summing across
        contexts or processes before average_finish."""
        n = len(particles)
        N = self.params["N"]
        idx = np.ascontiguousarray(particles, np.int32)
        w = np.ascontiguousarray(weights, np.float32)
        M = np.ascontiguousarray(np.asarray(matrices, np.float64).reshape(n, 16))
        out = [np.zeros((N, N, N // 2 + 1), np.float64) for _ in range(3)]
        self._check(self.L.ettk_gpu_average_partial(self._ctx, n, idx.ctypes.data, w.ctypes.data, M.ctypes.data,
                                                    out[0].ctypes.data, out[1].ctypes.data, out[2].ctypes.data),
                    "average_partial")
        return tuple(out)

    def average_finish(self, re, im, acc):
        """The class average ([z][y][x] float32, RMS 1) from summed accumulators."""
        N = self.params["N"]
        arrs = [np.ascontiguousarray(a, np.float64) for a in (re, im, acc)]
        out = np.zeros((N, N, N), np.float32)
        self._check(self.L.ettk_gpu_average_finish(self._ctx, arrs[0].ctypes.data, arrs[1].ctypes.data,
                                                   arrs[2].ctypes.data, out.ctypes.data), "average_finish")
        return out

    # -- nbfWedgedAverageImage3D::getImageVarianceMPI / nbfImageFilter::symmetrize -------------------------
    def variance(self, particles, weights, matrices, avg):
        """Variance of the members about `avg` ([z][y][x], as average() returns it); returns [z][y][x]."""
        n = len(particles)
        N = self.params["N"]
        idx = np.ascontiguousarray(particles, np.int32)
        w = np.ascontiguousarray(weights, np.float32)
        M = np.ascontiguousarray(np.asarray(matrices, np.float64).reshape(n, 16))
        a = np.ascontiguousarray(avg, np.float32)
        out = np.zeros((N, N, N), np.float32)
        self._check(self.L.ettk_gpu_variance(self._ctx, n, idx.ctypes.data, w.ctypes.data, M.ctypes.data,
                                             a.ctypes.data, out.ctypes.data), "variance")
        return out

    def symmetrize(self, vol, fold):
        """n-fold symmetrisation about z of a [z][y][x] volume; returns [z][y][x]."""
        N = self.params["N"]
        v = np.ascontiguousarray(vol, np.float32)
        out = np.zeros((N, N, N), np.float32)
        self._check(self.L.ettk_gpu_symmetrize(self._ctx, v.ctypes.data, int(fold), out.ctypes.data), "symmetrize")
        return out

    def mean_images(self, vol, transforms):
        """Mean of getImage of a [z][y][x] fixed-image volume under each 4x4 transform; returns [z][y][x]."""
        N = self.params["N"]
        v = np.ascontiguousarray(vol, np.float32)
        t = np.ascontiguousarray(np.asarray(transforms, np.float64).reshape(-1, 16))
        out = np.zeros((N, N, N), np.float32)
        self._check(self.L.ettk_gpu_mean_images(self._ctx, v.ctypes.data, len(t), t.ctypes.data, out.ctypes.data),
                    "mean_images")
        return out

    def setMaskFile(self, mask, threshold):
        """nbfImageFilter::setMaskFile as the alignment uses it: `mask` is the mask file's volume ((M, M, M) in
        [z][y][x] order, x fastest; None restores the spherical mask), binarised at `threshold` and softened; it
        becomes the CCF's reference mask m1."""
        if mask is None:
            self._check(self.L.ettk_gpu_set_reference_mask(self._ctx, 0, None, 0.0), "set_reference_mask")
            return
        m = np.ascontiguousarray(mask, np.float32)
        M = m.shape[0]
        if m.shape != (M, M, M):
            raise ValueError("the mask must be a cube")
        self._check(self.L.ettk_gpu_set_reference_mask(self._ctx, M, m.ctypes.data, float(threshold)),
                    "set_reference_mask")

    def reference_mask(self):
        """The CCF's reference mask m1 in use, (N, N, N) in [z][y][x] order."""
        N = self.params["N"]
        out = np.zeros((N, N, N), np.float32)
        self._check(self.L.ettk_gpu_get_reference_mask(self._ctx, out.ctypes.data), "get_reference_mask")
        return out

    def representations(self, particles, fold=1):
        """getLowDimensionRepresentationHalf of the given particles (n-fold symmetrised about z when fold > 1):
        (M, K, 3) float32 (re, im, wedge bit)."""
        p = np.ascontiguousarray(np.asarray(particles, np.int32))
        K = ctypes.c_int()
        self._check(self.L.ettk_gpu_representations(self._ctx, 0, None, int(fold), ctypes.byref(K), None),
                    "representations")
        R = np.zeros((len(p), K.value, 3), np.float32)
        self._check(self.L.ettk_gpu_representations(self._ctx, len(p), p.ctypes.data, int(fold), ctypes.byref(K),
                                                    R.ctypes.data), "representations")
        return R

    def representations_real(self, particles, fold=1, bin_factor=1):
        """getLowDimensionRepresentationReal of the given particles (the n-fold branch through the one-member wedged
        average when fold > 1; integer bin factor): (M, K, 1) float32, the depth-1 representation array."""
        p = np.ascontiguousarray(np.asarray(particles, np.int32))
        K = ctypes.c_int()
        self._check(self.L.ettk_gpu_representations_real(self._ctx, 0, None, int(fold), int(bin_factor),
                                                         ctypes.byref(K), None), "representations_real")
        R = np.zeros((len(p), K.value, 1), np.float32)
        self._check(self.L.ettk_gpu_representations_real(self._ctx, len(p), p.ctypes.data, int(fold), int(bin_factor),
                                                         ctypes.byref(K), R.ctypes.data), "representations_real")
        return R

    def representation_distances(self, R, overlap_normalized=None):
        """nbfCorrelationImageMetric::getDistances(representations, D): R is (V, K, 3) (re, im, wedge bit) or
        (V, K, 1) float32; returns the symmetric (V, V) distance matrix."""
        R = np.ascontiguousarray(R, np.float32)
        if R.ndim == 2:
            R = R[:, :, None]
        V, K, depth = R.shape
        if overlap_normalized is None:
            overlap_normalized = self.params["overlap_normalized"]
        D = np.zeros((V, V), np.float32)
        self._check(self.L.ettk_gpu_representation_distances(self._ctx, V, K, depth, R.ctypes.data,
                                                             int(bool(overlap_normalized)), D.ctypes.data),
                    "representation_distances")
        return D

    def average_spherical_wedge(self, particles, weights, matrices):
        """Spherical wedge of the class average of `particles` under `matrices` (updateSphericalWedgeImage).
        Returns (binary wedge [2B][2B], member count per sample [2B][2B])."""
        n = len(particles)
        n2 = 2 * self.params["B"]
        p = np.ascontiguousarray(np.asarray(particles, np.int32))
        w = np.ascontiguousarray(np.asarray(weights, np.float32))
        M = np.ascontiguousarray(np.asarray(matrices, np.float64).reshape(n, 16))
        wedge = np.zeros((n2, n2), np.float32)
        count = np.zeros((n2, n2), np.float32)
        self._check(self.L.ettk_gpu_average_spherical_wedge(self._ctx, n, p.ctypes.data, w.ctypes.data, M.ctypes.data,
                                                            count.ctypes.data, wedge.ctypes.data),
                    "average_spherical_wedge")
        return wedge, count

    def set_reference_spherical_wedge(self, r, wedge):
        """Explicit binary spherical wedge [2B][2B] for reference r (nbfWedge3D::setSphericalImage)."""
        w = np.ascontiguousarray(wedge, np.float32)
        assert w.size == (2 * self.params["B"]) ** 2
        self._check(self.L.ettk_gpu_set_reference_spherical_wedge(self._ctx, int(r), w.ctypes.data),
                    "set_reference_spherical_wedge")

    def symmetrize_rotational(self, vol):
        """Rotational (cylindrical) symmetrisation about z of a [z][y][x] volume, as the classification loop's
        apply_rotational_symmetry; returns [z][y][x] (the angular sum, about 180 times the mean)."""
        N = self.params["N"]
        v = np.ascontiguousarray(vol, np.float32)
        out = np.zeros((N, N, N), np.float32)
        self._check(self.L.ettk_gpu_symmetrize_rotational(self._ctx, v.ctypes.data, out.ctypes.data),
                    "symmetrize_rotational")
        return out

    # -- multireference classification (src/MPI_Classification.cpp align -> assign -> re-average) -----
    def classify(self, iterations):
        """Runs `iterations` passes of align all particles x references -> assign to the closest class ->
        wedge-weighted class averages as the new references. Returns (labels, references [R][z][y][x],
        distances)."""
        V = len(self._parts)
        R = len(self._refs)
        N = self.params["N"]
        labels = np.zeros(V, np.int32)
        refs = np.zeros((R, N, N, N), np.float32)
        dist = np.zeros(V, np.float32)
        self._check(self.L.ettk_gpu_classify(self._ctx, int(iterations), labels.ctypes.data, refs.ctypes.data,
                                             dist.ctypes.data), "classify")
        return labels, refs, dist

    # -- continuous pose refinement (no counterpart in the reference) ---------------------------
    def refine(self, indexes, D, iterations=12):
        """Refines candidate 0 of the rows of D (as getDistances returned them) in place by gradient ascent of
        the wedge-constrained normalised correlation; distance becomes 1 - rho. Returns D."""
        idx = np.ascontiguousarray(np.asarray(indexes, np.int32).reshape(-1, 2))
        assert D.dtype == np.float32 and D.flags.c_contiguous and D.shape[0] == idx.shape[0]
        self._check(self.L.ettk_gpu_refine_pairs(self._ctx, idx.shape[0], idx.ctypes.data, D.ctypes.data, D.shape[1],
                                                 D.shape[2], int(iterations)), "refine_pairs")
        return D

    def refine_objective(self, indexes, poses, theta, grad=True):
        """rho (and d rho / d(w, d)) at poses (n x 4 x 4) perturbed by theta (n x 6: rotation vector in
        radians about the box centre, then shift in voxels)."""
        idx = np.ascontiguousarray(np.asarray(indexes, np.int32).reshape(-1, 2))
        n = idx.shape[0]
        T = np.ascontiguousarray(np.asarray(poses, np.float64).reshape(n, 16))
        th = np.ascontiguousarray(np.asarray(theta, np.float64).reshape(n, 6))
        rho = np.zeros(n)
        g = np.zeros((n, 6)) if grad else None
        self._check(self.L.ettk_gpu_refine_objective(self._ctx, n, idx.ctypes.data, T.ctypes.data, th.ctypes.data,
                                                     rho.ctypes.data, g.ctypes.data if grad else None),
                    "refine_objective")
        return (rho, g) if grad else rho

    # -- fast form: coarse SO(3) hit + local refinement (no counterpart in the reference) -------
    def getDistancesRefined(self, indexes, D=None, cols=17, ncand=1, iterations=12, peaks=0):
        """As getDistances, through the fast form (ettk_gpu_align_pairs_refined): CCF of the `peaks` best
        windowed candidates (0: candidate_peaks) and peaks / 3 unwindowed ones, then `iterations` steps of
        continuous refinement; column 0 is 1 - rho at the refined pose."""
        idx = np.ascontiguousarray(np.asarray(indexes, np.int32).reshape(-1, 2))
        n = idx.shape[0]
        if D is None:
            D = -np.ones((n, cols, ncand), np.float32)
        assert D.dtype == np.float32 and D.flags.c_contiguous and D.shape[0] == n
        self._check(self.L.ettk_gpu_align_pairs_refined(self._ctx, n, idx.ctypes.data, D.ctypes.data, D.shape[1],
                                                        D.shape[2], int(iterations), int(peaks)), "align_pairs_refined")
        return D

    def refined_objective(self, indexes, poses, theta, grad=True):
        """The fast form's rho (and d rho / d(w, d)) with the reference filtered at poses (n x 4 x 4) and the
        particle at those poses perturbed by theta (n x 6: rotation vector in radians, shift in voxels)."""
        idx = np.ascontiguousarray(np.asarray(indexes, np.int32).reshape(-1, 2))
        n = idx.shape[0]
        T = np.ascontiguousarray(np.asarray(poses, np.float64).reshape(n, 16))
        th = np.ascontiguousarray(np.asarray(theta, np.float64).reshape(n, 6))
        rho = np.zeros(n)
        g = np.zeros((n, 6)) if grad else None
        self._check(self.L.ettk_gpu_refined_objective(self._ctx, n, idx.ctypes.data, T.ctypes.data, th.ctypes.data,
                                                      rho.ctypes.data, g.ctypes.data if grad else None),
                    "refined_objective")
        return (rho, g) if grad else rho

    # -- diagnostics ---------------------------------------------------------------------------
    def ccf(self, r, p, T):
        t = np.ascontiguousarray(np.asarray(T, np.float64).reshape(16)).copy()
        d = ctypes.c_float()
        self._check(self.L.ettk_gpu_ccf(self._ctx, r, p, t.ctypes.data, ctypes.byref(d)), "ccf")
        return float(d.value), t.reshape(4, 4)

    def spherical_projection(self, r=0, p=-1):
        n = 2 * self.params["B"]
        out = np.zeros((n, n), np.float32)
        self._check(self.L.ettk_gpu_spherical_projection(self._ctx, r, p, out.ctypes.data), "spherical_projection")
        return out

    def soft(self, F1, F2, scaled=False):
        n = 2 * self.params["B"]
        a = np.ascontiguousarray(F1, np.float32)
        b = np.ascontiguousarray(F2, np.float32)
        C = np.zeros((n, n, n), np.float32)
        self._check(self.L.ettk_gpu_soft(self._ctx, a.ctypes.data, b.ctypes.data, int(scaled), C.ctypes.data), "soft")
        return C

    # -- launch shapes (no counterpart in the reference) ---------------------------------------
    def get_tuning(self):
        t = _lib.Tuning()
        self._check(self.L.ettk_gpu_get_tuning(self._ctx, ctypes.byref(t)), "get_tuning")
        return {f[0]: getattr(t, f[0]) for f in _lib.Tuning._fields_}

    def set_tuning(self, tuning):
        t = _lib.Tuning(**{f[0]: int(tuning[f[0]]) for f in _lib.Tuning._fields_})
        self._check(self.L.ettk_gpu_set_tuning(self._ctx, ctypes.byref(t)), "set_tuning")

    def autotune(self, indexes, repeats=3):
        """Chooses the launch shapes on the sample pairs (ettk_gpu_autotune) and applies them; returns
        (tuning dict, list of trials)."""
        import json
        idx = np.ascontiguousarray(np.asarray(indexes, np.int32).reshape(-1, 2))
        t = _lib.Tuning()
        buf = ctypes.create_string_buffer(1 << 16)
        self._check(self.L.ettk_gpu_autotune(self._ctx, idx.shape[0], idx.ctypes.data, int(repeats), ctypes.byref(t),
                                             buf, len(buf)), "autotune")
        return {f[0]: getattr(t, f[0]) for f in _lib.Tuning._fields_}, json.loads(buf.value.decode())

    def stream(self):
        """cudaStream_t of this context (for CUDA-event timing)."""
        return int(self.L.ettk_gpu_stream(self._ctx) or 0)

    def profile(self, enable=True):
        self._check(self.L.ettk_gpu_profile(self._ctx, int(enable)), "profile")

    def profile_read(self):
        out = {}
        i = 0
        while True:
            name = ctypes.create_string_buffer(64)
            n = ctypes.c_longlong()
            ms = ctypes.c_double()
            b = ctypes.c_double()
            if self.L.ettk_gpu_profile_read(self._ctx, i, name, 64, ctypes.byref(n), ctypes.byref(ms), ctypes.byref(b)):
                break
            out[name.value.decode()] = {"launches": n.value, "ms": ms.value, "bytes": b.value}
            i += 1
        return out

    def kernel_launches(self):
        return int(self.L.ettk_gpu_kernel_launches(self._ctx))
