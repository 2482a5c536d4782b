"""Benchmark: alignments/s of the sub-volume alignment path at 64^3, B=32.

One step = aligning a batch of particle x reference pairs (the plain method: SO(3) grid search plus
translational CCF candidates, alignment_mode 3) through the library's getDistances entry point.

  value : pairs/s with the particle volumes already resident in HBM (set_particles_device + align)
  e2e   : pairs/s through the host-buffer API: pinned host volumes copied in every step
          (ettk_gpu_set_particles) and the result rows read back (ettk_gpu_align_pairs)
  fast_form : the same pairs through the fast form (ettk_gpu_align_pairs_refined: coarse SO(3) search on the half
          grid at B/2 with the split-BF16 Wigner contraction, half-grid candidate screening, local refinement):
          alignments/s, speed-up over the plain form, e2e, and both forms' rotation/shift errors against the
          generating poses

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
Under torchrun each rank aligns its own batch on its own GPU (independent replicas, no collective
on the data path); rank 0 prints one JSON line with the max time over ranks.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "align64_b32"
FAST_PRECISION = 2   # split-BF16 Wigner-d contraction on the tensor cores
FAST_ITERATIONS = 9  # local refinement steps of the fast form
FAST_COARSE = 2  # the fast form's SO(3) search on the half grid at B/2, trilinear screening (1: tricubic; 0: full grid)
METRIC = "alignments/s at 64^3 bw=32: plain GPU vs batched+adjoint form at <=0.5deg/0.1 vox"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--pairs", type=int, default=256, help="pairs aligned per step (per GPU)")
    ap.add_argument("--cpu-sample", type=int, default=0, help="pairs in the CPU baseline sample (0 = auto)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--precision-study", action="store_true",
                    help="Wigner-d contraction precision modes on the 128^3 B=64 workload (one JSON line)")
    ap.add_argument("--study-pairs", type=int, default=32)
    ap.add_argument("--adjoint-study", action="store_true",
                    help="plain grid search vs grid search + adjoint refinement on the 64^3 B=32 workload: "
                         "alignments/s and error against the generating poses (one JSON line)")
    ap.add_argument("--refine-iterations", type=int, default=15)
    ap.add_argument("--fast-study", action="store_true",
                    help="plain form against the fast form (coarse SO(3) hit, one CCF per kept peak, local refinement) "
                         "on the 64^3 B=32 workload: alignments/s, stage times and errors against the generating poses")
    ap.add_argument("--fast-iterations", type=int, default=FAST_ITERATIONS)
    ap.add_argument("--workload", default=WORKLOAD, help="workload of the studies (align64_b32, refine64_b32)")
    ap.add_argument("--fast-peaks", type=int, default=0, help="0: the metric's candidate_peaks")
    ap.add_argument("--fast-precision", type=int, default=2, help="Wigner-d contraction of the fast form")
    ap.add_argument("--fast-coarse", type=int, default=FAST_COARSE,
                    help="the fast form's SO(3) search: 0 full grid, 1 half grid at B/2, 2 also trilinear screening")
    ap.add_argument("--fast-only", action="store_true",
                    help="--fast-study without the plain form (the fast form run twice on all pairs, the second timed)")
    ap.add_argument("--tune-study", action="store_true",
                    help="plain-form rate under the default launch shapes, the autotuner's trials, the tuned rate")
    ap.add_argument("--config-table", action="store_true",
                    help="plain and fast form on every alignment configuration, the oracle beside each, one "
                         "classification pass (--study-pairs particles x 10 references)")
    ap.add_argument("--repr-study", action="store_true",
                    help="unsupervised-classification step on the 64^3 workload: low-dimensional representations "
                         "of --study-pairs particles and the distance matrix between them (one JSON line)")
    return ap.parse_args()


# ------------------------------------------------------------------------------- precision study

PRECISION_MODES = {0: "fp32", 1: "bf16", 2: "split_bf16", 3: "tf32", 4: "fp64"}


def precision_study(a):
    """Each Wigner-d contraction mode (ettk_params.wigner_precision) on the 128^3 B=64 workload, against the
    FP64-contraction mode (every other stage identical): CCF score errors, best-rotation and shift agreement over
    the aligned pairs, SO(3) correlation errors on random signals, and alignments/s per mode."""
    import numpy as np
    import torch
    from ettk_gb300 import synthetic
    from ettk_gb300.metric import ProjectionRotationMetric3D, WedgedSubImage3D

    name = "align128_b64"
    P = a.study_pairs
    ds = synthetic.generate(name, n_particles=P)
    kw = ("lwedge", "uwedge", "normal", "matrix", "position", "cut_offset")
    vols = [WedgedSubImage3D(ds.particles[i], **{k: ds.meta[i][k] for k in kw}) for i in range(P)]
    ref = WedgedSubImage3D(ds.references[0], **{k: ds.ref_meta[0][k] for k in kw})
    pairs = [(0, i) for i in range(P)]
    B = ds.params["B"]
    rng = np.random.default_rng(20261207)
    sigs = [(rng.random((2 * B, 2 * B)).astype(np.float32), rng.random((2 * B, 2 * B)).astype(np.float32))
            for _ in range(4)]
    res = {}
    for mode in (4, 0, 1, 2, 3):
        m = ProjectionRotationMetric3D(dict(ds.params, wigner_precision=mode))
        m.set_references([ref])
        m.set_particles(vols)
        m.getDistances(pairs[:2])  # warm-up (tables, buffers)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        D = m.getDistances(pairs)
        dt = time.perf_counter() - t0
        C = [m.soft(f1, f2) for f1, f2 in sigs]
        m.close()
        res[mode] = (D, C, P / dt)
    D4, C4, _ = res[4]
    out = {}
    for mode, (D, C, rate) in res.items():
        rel = np.abs(D[:, 0, 0] - D4[:, 0, 0]) / np.abs(D4[:, 0, 0])
        rot = [np.allclose(D[i, 1:17, 0].reshape(4, 4)[:3, :3], D4[i, 1:17, 0].reshape(4, 4)[:3, :3], atol=1e-5)
               for i in range(P)]
        sh = [np.allclose(D[i, 1:17, 0].reshape(4, 4)[:3, 3], D4[i, 1:17, 0].reshape(4, 4)[:3, 3], atol=1e-4)
              for i in range(P)]
        cerr = [np.abs(c - c4) / (c4.max() - c4.min()) for c, c4 in zip(C, C4)]
        cam = [np.unravel_index(c.argmax(), c.shape) == np.unravel_index(c4.argmax(), c4.shape) for c, c4 in zip(C, C4)]
        out[PRECISION_MODES[mode]] = {
            "alignments_per_s": rate, "score_rel_err_max": float(rel.max()),
            "score_rel_err_rms": float(np.sqrt((rel ** 2).mean())),
            "best_rotation_agreement": float(np.mean(rot)), "shift_agreement": float(np.mean(sh)),
            "so3_corr_err_max": float(max(e.max() for e in cerr)),
            "so3_corr_err_rms": float(np.sqrt(np.mean([(e ** 2).mean() for e in cerr]))),
            "so3_argmax_agreement": float(np.mean(cam))}
    line = {"precision_study": out, "reference_mode": "fp64 contraction (double Wigner-d table and accumulation)",
            "config": {"workload": name, "N": ds.params["N"], "B": B, "pairs": P, "so3_signals": len(sigs),
                       "errors": "scores relative to the fp64 mode; SO(3) correlations relative to its range"}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------- CPU (oracle) arm

def _cpu_worker(args):
    idx, n, workload = args
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from ettk_gb300 import synthetic
    ds = synthetic.generate(workload, n_particles=n)
    t0 = time.perf_counter()
    for i in idx:
        pyoracle.align(ds.params, ds.references[0], ds.ref_meta[0], ds.particles[i], ds.meta[i])
    return time.perf_counter() - t0, len(idx)


def cpu_baseline(n_pairs, workload=WORKLOAD):
    """The oracle (FP64 port of the reference path) on all host cores: one single-threaded process per
    core on a disjoint shard, as the reference runs one MPI worker per core. Returns pairs/s."""
    import multiprocessing as mp
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    pyoracle.build()
    cores = os.cpu_count() or 1
    n_pairs = max(n_pairs, cores)
    shards = [list(range(k, n_pairs, cores)) for k in range(cores)]
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_worker, [(s, n_pairs, workload) for s in shards if s])
    wall = time.perf_counter() - t0
    busy = max(r[0] for r in res)
    return {"value": n_pairs / busy, "unit": "alignments/s", "cores": cores, "kind": "port",
            "sample": "%d pairs of the %s workload, one oracle process per core, %.1f s wall; "
                      "the oracle is built -O3 and transforms with its own radix-2 FFT (the reference's FFTW3 is not "
                      "in the image)" % (n_pairs, workload, wall)}


# ------------------------------------------------------------------------------- clocks

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------- GPU arm

def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    return 6800.0, 1900.0, "fallback"


def adjoint_study(a):
    """Plain form (SO(3) grid + CCF candidates) against plain + adjoint refinement on the same pairs:
    alignments/s of each (device-resident particles, CUDA-synchronised wall time) and the rotation (degrees,
    geodesic) and shift (voxels) errors against the generating poses."""
    import numpy as np
    import torch
    from ettk_gb300 import synthetic
    from ettk_gb300.metric import ProjectionRotationMetric3D, WedgedSubImage3D

    P = a.pairs
    ds = synthetic.generate(WORKLOAD, n_particles=P)
    kw = ("lwedge", "uwedge", "normal", "matrix", "position", "cut_offset")
    m = ProjectionRotationMetric3D(ds.params)
    m.set_references([WedgedSubImage3D(ds.references[0], **{k: ds.ref_meta[0][k] for k in kw})])
    m.set_particles([WedgedSubImage3D(ds.particles[i], **{k: ds.meta[i][k] for k in kw}) for i in range(P)])
    pairs = [(0, i) for i in range(P)]
    for _ in range(max(1, a.warmup)):
        m.refine(pairs[:4], m.getDistances(pairs[:4]), iterations=2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    D = m.getDistances(pairs)
    t1 = time.perf_counter()
    D2 = m.refine(pairs, D.copy(), iterations=a.refine_iterations)
    t2 = time.perf_counter()
    m.close()

    def errors(Dm):
        rot, sh = [], []
        for i in range(P):
            T = Dm[i, 1:17, 0].reshape(4, 4).astype(np.float64)
            Rt = np.asarray(ds.truth[i]["rotation"])
            c = np.clip((np.trace(T[:3, :3] @ Rt.T) - 1) / 2, -1, 1)
            rot.append(np.degrees(np.arccos(c)))
            sh.append(np.linalg.norm(T[:3, 3] - np.asarray(ds.truth[i]["shift"])))
        rot, sh = np.array(rot), np.array(sh)
        hit = rot < 20.0  # grid hit in the right basin
        return {"rotation_deg_median": float(np.median(rot[hit])), "rotation_deg_mean": float(np.mean(rot[hit])),
                "shift_vox_median": float(np.median(sh[hit])), "shift_vox_mean": float(np.mean(sh[hit])),
                "within_0.5deg_0.1vox": float(np.mean((rot < 0.5) & (sh < 0.1))), "basin_hits": int(hit.sum())}

    line = {"adjoint_study": {
        "plain": dict(alignments_per_s=P / (t1 - t0), **errors(D)),
        "plain_plus_adjoint": dict(alignments_per_s=P / (t2 - t0), **errors(D2)),
        "refine_only_pairs_per_s": P / (t2 - t1)},
        "config": {"workload": WORKLOAD, "pairs": P, "refine_iterations": a.refine_iterations,
                   "errors": "against the generating poses, over pairs whose grid hit is within 20 degrees"}}
    print(json.dumps(line), flush=True)


def pose_errors(D, truth, off=1):
    """Geodesic rotation error (degrees) and shift error (voxels) of slot 0 of every row against the generating
    poses."""
    import numpy as np
    rot, sh = [], []
    for i in range(D.shape[0]):
        T = D[i, off:off + 16, 0].reshape(4, 4).astype(np.float64)
        Rt = np.asarray(truth[i]["rotation"])
        c = np.clip((np.trace(T[:3, :3] @ Rt.T) - 1) / 2, -1, 1)
        rot.append(np.degrees(np.arccos(c)))
        sh.append(np.linalg.norm(T[:3, 3] - np.asarray(truth[i]["shift"])))
    return np.array(rot), np.array(sh)


def error_summary(rot, sh, hit):
    import numpy as np
    return {"rotation_deg_median": float(np.median(rot[hit])), "rotation_deg_mean": float(np.mean(rot[hit])),
            "shift_vox_median": float(np.median(sh[hit])), "shift_vox_mean": float(np.mean(sh[hit])),
            "within_0.5deg_0.1vox": float(np.mean((rot < 0.5) & (sh < 0.1))), "basin_hits": int(hit.sum())}


def fast_study(a):
    """Plain form (SO(3) grid + CCF candidates with mirrors, FP32 Wigner) against the fast form (split-BF16 Wigner,
    one CCF per kept peak, batched local refinement) on the same pairs: alignments/s of each (device-resident
    particles, CUDA-synchronised wall time, after one warm-up call of each), the library's stage times, and the
    rotation/shift errors against the generating poses over the pairs whose plain grid hit is within 20 degrees."""
    from ettk_gb300 import synthetic

    P = a.pairs
    ds = synthetic.generate(a.workload, n_particles=P)
    out = compare_forms(ds, P, a.fast_iterations, a.fast_peaks, a.fast_precision, a.fast_only, a.fast_coarse)
    if a.fast_only:
        rf, sf = pose_errors(out["fast"][0], ds.truth)
        line = {"fast_study": {"fast": dict(alignments_per_s=out["fast"][1], **error_summary(rf, sf, rf < 20.0),
                                            families_ms={k: round(v["ms"], 3) for k, v in out["fast"][2].items()})},
                "config": {"workload": a.workload, "pairs": P, "iterations": a.fast_iterations, "peaks": a.fast_peaks,
                           "fast_wigner_precision": a.fast_precision, "fast_coarse_so3": a.fast_coarse}}
        print(json.dumps(line), flush=True)
        return
    rp, sp = pose_errors(out["plain"][0], ds.truth)
    rf, sf = pose_errors(out["fast"][0], ds.truth)
    hit = rp < 20.0
    stages = ("stage_so3", "stage_ccf", "stage_coarse_ccf", "stage_local_refine", "host_align_wall")
    line = {"fast_study": {
        "plain": dict(alignments_per_s=out["plain"][1], **error_summary(rp, sp, hit),
                      stages_ms={k: round(v["ms"], 3) for k, v in out["plain"][2].items() if k in stages}),
        "fast": dict(alignments_per_s=out["fast"][1], **error_summary(rf, sf, hit),
                     basin_hits_fast=int((rf < 20.0).sum()),
                     stages_ms={k: round(v["ms"], 3) for k, v in out["fast"][2].items() if k in stages},
                     families_ms={k: round(v["ms"], 3) for k, v in out["fast"][2].items()}),
        "speedup": out["fast"][1] / out["plain"][1]},
        "config": {"workload": a.workload, "pairs": P, "iterations": a.fast_iterations, "peaks": a.fast_peaks,
                   "fast_wigner_precision": a.fast_precision, "fast_coarse_so3": a.fast_coarse,
                   "errors": "against the generating poses, over pairs whose plain grid hit is within 20 degrees"}}
    print(json.dumps(line), flush=True)


def compare_forms(ds, P, iterations, peaks, precision, fast_only=False, coarse=FAST_COARSE):
    """Plain and fast form on the first P particles of ds against its reference: per form (result rows,
    alignments/s, the library's profile), timed after one warm-up call at full size."""
    import torch
    from ettk_gb300.metric import ProjectionRotationMetric3D, WedgedSubImage3D
    kw = ("lwedge", "uwedge", "normal", "matrix", "position", "cut_offset")
    vols = [WedgedSubImage3D(ds.particles[i], **{k: ds.meta[i][k] for k in kw}) for i in range(P)]
    ref = WedgedSubImage3D(ds.references[0], **{k: ds.ref_meta[0][k] for k in kw})
    pairs = [(0, i) for i in range(P)]
    out = {}
    forms = (("fast", precision),) if fast_only else (("plain", 0), ("fast", precision))
    for form, prec in forms:
        m = ProjectionRotationMetric3D(dict(ds.params, wigner_precision=prec,
                                            fast_coarse_so3=coarse if form == "fast" else 0))
        m.set_references([ref])
        m.set_particles(vols)

        def run(sub):
            if form == "plain":
                return m.getDistances(sub)
            return m.getDistancesRefined(sub, iterations=iterations, peaks=peaks)
        run(pairs)  # warm-up at full size (buffers, tables, the half-grid references)
        m.set_particles(vols)  # drop the cached spherical projections of the warm-up pairs
        torch.cuda.synchronize()
        m.profile(True)
        t0 = time.perf_counter()
        D = run(pairs)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        prof = m.profile_read()
        m.profile(False)
        m.close()
        out[form] = (D, P / (t1 - t0), prof)
    return out


def tune_study(a):
    """The launch-shape autotuner on the headline workload: plain-form alignments/s of P pairs (particles resident,
    CUDA-synchronised wall time of three steps after one warm-up) under the default shapes, the autotuner's trials on a
    64-pair sample, and the same rate under the chosen shapes (result rows compared bit for bit)."""
    import numpy as np
    import torch
    from ettk_gb300 import synthetic
    from ettk_gb300.metric import ProjectionRotationMetric3D, WedgedSubImage3D
    P = a.pairs
    ds = synthetic.generate(WORKLOAD, n_particles=P)
    kw = ("lwedge", "uwedge", "normal", "matrix", "position", "cut_offset")
    metas = [{k: m[k] for k in kw} for m in ds.meta]
    m = ProjectionRotationMetric3D(ds.params)
    m.set_references([WedgedSubImage3D(ds.references[0], **{k: ds.ref_meta[0][k] for k in kw})])
    parts = torch.from_numpy(ds.particles).to("cuda")
    pairs = [(0, i) for i in range(P)]

    def rate():
        def step():
            m.set_particles_device(parts.data_ptr(), metas)
            return m.getDistances(pairs)
        step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(3):
            D = step()
        torch.cuda.synchronize()
        return 3 * P / (time.perf_counter() - t0), D

    r0, D0 = rate()
    m.set_particles_device(parts.data_ptr(), metas)
    best, trials = m.autotune(pairs[:64], repeats=3)
    r1, D1 = rate()
    m.close()
    print(json.dumps({"tune_study": {"default_alignments_per_s": r0, "tuned_alignments_per_s": r1,
                                     "tuned": best, "identical_rows": bool(np.array_equal(D0, D1)),
                                     "trials": trials},
                      "config": {"workload": WORKLOAD, "pairs": P, "sample_pairs": 64}}), flush=True)


def config_table(a):
    """The results table of the configurations: per alignment configuration the plain and the fast form
    (alignments/s, errors against the generating poses) and the oracle on the host cores on a bounded sample;
    for the classification configuration one classify pass (align all particles against all references, assign,
    re-average) timed as pairs/s."""
    import numpy as np
    import torch
    from ettk_gb300 import synthetic
    from ettk_gb300.metric import ProjectionRotationMetric3D, WedgedSubImage3D
    rows = {}
    for name, P, cpu_n in (("align32_b16", 200, 64), ("align64_b32", 256, 32), ("refine64_b32", 256, 32),
                           ("align128_b64", 32, 16)):
        cpu = cpu_baseline(cpu_n, name)
        ds = synthetic.generate(name, n_particles=P)
        out = compare_forms(ds, P, FAST_ITERATIONS, 0, FAST_PRECISION)
        rp, sp = pose_errors(out["plain"][0], ds.truth)
        rf, sf = pose_errors(out["fast"][0], ds.truth)
        hit = rp < 20.0
        rows[name] = {"pairs": P, "cpu": cpu, "plain": dict(alignments_per_s=out["plain"][1], **error_summary(rp, sp, hit)),
                      "fast": dict(alignments_per_s=out["fast"][1], **error_summary(rf, sf, hit)),
                      "speedup": out["fast"][1] / out["plain"][1]}
        print(json.dumps({"config_row": name, **rows[name]}), flush=True)
    # classification: V particles x R references, one pass
    V = a.study_pairs
    ds = synthetic.generate("mra64_b32", n_particles=V)
    kw = ("lwedge", "uwedge", "normal", "matrix", "position", "cut_offset")
    m = ProjectionRotationMetric3D(ds.params)
    m.set_references([WedgedSubImage3D(r, **{k: rm[k] for k in kw}) for r, rm in zip(ds.references, ds.ref_meta)])
    m.set_particles([WedgedSubImage3D(ds.particles[i], **{k: ds.meta[i][k] for k in kw}) for i in range(V)])
    m.classify(1)  # warm-up
    m.set_references([WedgedSubImage3D(r, **{k: rm[k] for k in kw}) for r, rm in zip(ds.references, ds.ref_meta)])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    labels, _, _ = m.classify(1)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    m.close()
    R = len(ds.references)
    rows["mra64_b32"] = {"particles": V, "references": R, "pairs_per_s": V * R / dt, "pass_s": dt,
                         "classes_used": int(len(np.unique(labels)))}
    print(json.dumps({"config_table": rows}), flush=True)


def repr_study(a):
    """getLowDimensionRepresentationHalf of V 64^3 particles and the V x V distance matrix of
    nbfCorrelationImageMetric::getDistances between them, each timed once after one small warm-up call
    (CUDA-synchronised wall time of the library call; the distance kernel's own time from the library's event
    profile). Rates: representations/s, and pair-coefficients/s of the distance kernel (V (V - 1) / 2 pairs
    times K coefficients, each one FP64 accumulation)."""
    import numpy as np
    from ettk_gb300 import synthetic
    from ettk_gb300.metric import ProjectionRotationMetric3D, WedgedSubImage3D

    V = a.study_pairs
    ds = synthetic.generate(WORKLOAD, n_particles=8)  # parameters and per-particle wedge geometries
    N = ds.params["N"]
    rng = np.random.default_rng(5)  # seeded noise volumes: the timings do not depend on the content
    kw = ("lwedge", "uwedge", "normal", "matrix", "position", "cut_offset")
    m = ProjectionRotationMetric3D(ds.params)
    m.set_particles([WedgedSubImage3D(rng.standard_normal((N, N, N), dtype=np.float32),
                                      **{k: ds.meta[i % 8][k] for k in kw}) for i in range(V)])
    m.representation_distances(m.representations([0, 1]))  # warm-up: one launch of each kernel
    m.profile(True)
    t0 = time.perf_counter()
    R = m.representations(list(range(V)))
    t1 = time.perf_counter()
    D = m.representation_distances(R)
    t2 = time.perf_counter()
    prof = m.profile_read()
    m.profile(False)
    m.close()
    K = R.shape[1]
    kd = prof.get("repr_dist", {}).get("ms", float("nan"))
    pk = V * (V - 1) / 2 * K
    line = {"repr_study": {"V": V, "K": K, "representations_per_s": V / (t1 - t0),
                           "distance_matrix_s": t2 - t1, "distance_kernel_ms": kd,
                           "pair_coefficients_per_s": pk / (kd / 1e3),
                           "binary_weights": bool(np.isin(R[:, :, 2], (0.0, 1.0)).all()),
                           "finite": bool(np.isfinite(D).all())},
            "config": {"workload": WORKLOAD, "fold": 1, "overlap_normalized": bool(ds.params["overlap_normalized"]),
                       "data": "seeded noise volumes with the workload's wedge geometries"}}
    print(json.dumps(line), flush=True)


def main():
    a = parse()
    if a.repr_study:
        repr_study(a)
        return
    if a.fast_study:
        fast_study(a)
        return
    if a.config_table:
        config_table(a)
        return
    if a.tune_study:
        tune_study(a)
        return
    if a.adjoint_study:
        adjoint_study(a)
        return
    if a.precision_study:
        precision_study(a)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if a.impl == "reference":
        if rank != 0:
            return
        # The reference's CPU path (C++ on VTK 5.10 + FFTW3 + MPI) cannot be built here (FFTW3, MPI and a
        # VTK build are absent); its FP64 restatement (the oracle) is timed on all host cores instead.
        n = a.cpu_sample or 2 * (os.cpu_count() or 1)
        vals = [cpu_baseline(n) for _ in range(a.steps)]  # a process pool has no warm state to prime
        v = vals[-1]
        per = [x["value"] for x in vals]
        value = statistics.median(per)
        out = {"metric": METRIC, "value": value, "unit": "alignments/s", "n_gpus": a.gpus, "steps": a.steps,
               "warmup": a.warmup, "ms_per_step": 1000.0 * n / value, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
               "config": {"workload": WORKLOAD, "N": 64, "B": 32, "pairs_per_step": n, "method": "alignment_mode 3"},
               "cpu_baseline": {"value": value, "unit": "alignments/s", "cores": v["cores"], "kind": "port",
                                "sample": v["sample"]},
               "e2e": {"value": value, "unit": "alignments/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out), flush=True)
        return

    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        cpu = cpu_baseline(a.cpu_sample or 2 * (os.cpu_count() or 1))

    import numpy as np
    import torch
    from ettk_gb300 import synthetic
    from ettk_gb300.metric import ProjectionRotationMetric3D, WedgedSubImage3D

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    ds = synthetic.generate(WORKLOAD, n_particles=a.pairs)
    P = a.pairs
    N = ds.params["N"]
    kw = ("lwedge", "uwedge", "normal", "matrix", "position", "cut_offset")
    metas = [{k: m[k] for k in kw} for m in ds.meta]
    m = ProjectionRotationMetric3D(ds.params, device=local)
    m.set_references([WedgedSubImage3D(ds.references[0], **{k: ds.ref_meta[0][k] for k in kw})])
    parts_dev = torch.from_numpy(ds.particles).to("cuda")
    parts_host = torch.from_numpy(ds.particles).pin_memory()
    vols = [WedgedSubImage3D(ds.particles[i], **metas[i]) for i in range(P)]
    pairs = [(0, i) for i in range(P)]
    stream = torch.cuda.ExternalStream(m.stream())

    def step_device():
        m.set_particles_device(parts_dev.data_ptr(), metas)
        return m.getDistances(pairs)

    def step_e2e():
        m.set_particles(vols, stacked=parts_host.numpy())
        return m.getDistances(pairs)

    def timed(fn, steps, strm=None):
        strm = strm or stream
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(strm)
        for _ in range(steps):
            fn()
        e1.record(strm)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        if world > 1:
            t = torch.tensor([ms], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        return ms

    for _ in range(a.warmup):
        step_device()
    clocks = ClockSampler(local)
    clocks.start()
    m.profile(True)
    launches0 = m.kernel_launches()
    ms = timed(step_device, a.steps)
    launches = m.kernel_launches() - launches0
    prof = m.profile_read()
    m.profile(False)
    for _ in range(a.warmup):  # the host-buffer path's own first use (its device buffer) outside the timed steps
        step_e2e()
    ms_e2e = timed(step_e2e, a.steps)
    D_plain = step_device()
    # the fast form on the same pairs: split-BF16 Wigner contraction, half-grid candidate screening, local refinement
    mf = ProjectionRotationMetric3D(dict(ds.params, wigner_precision=FAST_PRECISION, fast_coarse_so3=FAST_COARSE),
                                    device=local)
    mf.set_references([WedgedSubImage3D(ds.references[0], **{k: ds.ref_meta[0][k] for k in kw})])
    fstream = torch.cuda.ExternalStream(mf.stream())

    def step_fast():
        mf.set_particles_device(parts_dev.data_ptr(), metas)
        return mf.getDistancesRefined(pairs, iterations=FAST_ITERATIONS)

    def step_fast_e2e():
        mf.set_particles(vols, stacked=parts_host.numpy())
        return mf.getDistancesRefined(pairs, iterations=FAST_ITERATIONS)

    for _ in range(a.warmup):
        step_fast()
    fl0 = mf.kernel_launches()
    ms_fast = timed(step_fast, a.steps, fstream)
    fast_launches = mf.kernel_launches() - fl0
    for _ in range(a.warmup):
        step_fast_e2e()
    ms_fast_e2e = timed(step_fast_e2e, a.steps, fstream)
    D_fast = step_fast()
    mf.close()
    clk = clocks.stop()
    rp, sp = pose_errors(D_plain, ds.truth)
    rf, sf = pose_errors(D_fast, ds.truth)
    hit = rp < 20.0

    hbm, tflops, peak_kind = peaks()
    # device families only: host_* scopes are wall-clock host time, stage_* scopes bracket several families
    kernels = {k: v for k, v in prof.items() if not k.startswith(("host_", "stage_"))}
    dom_name, dom = max(kernels.items(), key=lambda kv: kv[1]["ms"])
    achieved = dom["bytes"] / (dom["ms"] * 1e-3) / 1e9
    total_prof_ms = sum(v["ms"] for v in kernels.values())
    # DRAM bytes per launch of the dominant kernel: the ncu figure per volume (profiles/roofline_traffic.json,
    # dram__bytes_read.sum + dram__bytes_write.sum of a capture) scaled to this run's volumes per launch
    traffic, alg_per_launch, rec = None, dom["bytes"] / max(1, dom["launches"]), None
    try:
        with open(os.path.join(ROOT, "profiles", "roofline_traffic.json")) as f:
            rec = json.load(f).get(dom_name)
        if rec and dom_name == "reslice":
            traffic = rec["dram_bytes_per_volume"] * alg_per_launch / (8.0 * N ** 3)
    except (OSError, ValueError, KeyError):
        traffic = None
    smem = None
    if dom_name == "reslice":
        # The tricubic gather reads 64 taps per output voxel from the staged footprint: with one shared-memory
        # wavefront per clock per SM, a conflict-free gather takes N^3 * 64 / 32 wavefronts per volume. floor_ms is
        # that count over the SMs at the sampled clock; frac = floor_ms / the family's time. The ncu count of shared
        # load wavefronts per volume (bank conflicts and the staging included) gives the pipe's utilisation.
        vols = dom["bytes"] / (8.0 * N ** 3)
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz") or 2070.0
        ideal = N ** 3 * 64 / 32
        floor_ms = vols * ideal / (sms * mhz * 1e6) * 1e3
        smem = {"basis": "shared-memory wavefronts, 1 per clock per SM", "ideal_wavefronts_per_volume": ideal,
                "volumes": vols, "sms": sms, "sm_mhz": mhz, "floor_ms": floor_ms, "frac": floor_ms / dom["ms"]}
        if rec and rec.get("smem_ld_wavefronts_per_volume"):
            w = rec["smem_ld_wavefronts_per_volume"]
            smem["measured_wavefronts_per_volume"] = w
            smem["pipe_utilisation"] = vols * w / (sms * mhz * 1e6) * 1e3 / dom["ms"]
    value = world * P * a.steps / (ms * 1e-3)
    e2e = world * P * a.steps / (ms_e2e * 1e-3)
    out = {
        "metric": METRIC, "value": value, "unit": "alignments/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "N": N, "B": ds.params["B"], "pairs_per_step_per_gpu": P,
                   "method": "alignment_mode 3 (SO(3) grid + CCF candidates), FP32",
                   "l2": "inputs larger than L2 (%.0f MB of particle volumes per step)" % (P * N ** 3 * 4 / 1e6),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": e2e, "unit": "alignments/s", "h2d_bytes_per_step": P * N ** 3 * 4,
                "d2h_bytes_per_step": P * 17 * 4},
        "gpu_launches": launches,
        "fast_form": {
            "value": world * P * a.steps / (ms_fast * 1e-3), "unit": "alignments/s", "ms_per_step": ms_fast / a.steps,
            "speedup_vs_plain": ms / ms_fast,
            "e2e": {"value": world * P * a.steps / (ms_fast_e2e * 1e-3), "unit": "alignments/s",
                    "h2d_bytes_per_step": P * N ** 3 * 4, "d2h_bytes_per_step": P * 17 * 4},
            "gpu_launches": fast_launches,
            "method": "SO(3) grid on the %s with split-BF16 tcgen05 Wigner contraction, CCF of the candidatePeaks + "
                      "1 best candidates on half-grid Fourier crops (%s resampling), %d steps of local 6-DOF "
                      "refinement by the analytic gradient of the masked normalised correlation"
                      % ("half grid at B/2" if FAST_COARSE else "full grid",
                         "trilinear" if FAST_COARSE >= 2 else "tricubic", FAST_ITERATIONS),
            "errors": {"plain": error_summary(rp, sp, hit), "fast": dict(error_summary(rf, sf, hit),
                                                                         basin_hits_fast=int((rf < 20.0).sum())),
                       "note": "against the generating poses; medians and means over the pairs whose plain grid hit "
                               "is within 20 degrees"}},
        "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "peak_source": peak_kind, "traffic": traffic,
                     "algorithmic_bytes_per_launch": alg_per_launch,
                     "kernel_share": dom["ms"] / total_prof_ms if total_prof_ms else None, "smem": smem,
                     "families": {k: {"ms": round(v["ms"], 3), "launches": v["launches"],
                                      "GBps": round(v["bytes"] / (v["ms"] * 1e-3) / 1e9, 1) if v["ms"] else None}
                                  for k, v in sorted(prof.items(), key=lambda kv: -kv[1]["ms"])}},
        "clocks": clk,
    }
    if cpu:
        out["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(out), flush=True)
    m.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
