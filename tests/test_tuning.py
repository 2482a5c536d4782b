"""Launch-shape autotuner (ettk_gpu_autotune) and its cache (ettk_gb300/tuning.py). The shapes never change a
result: every trial's rows must equal the first trial's bit for bit, and alignments under the chosen shapes equal
those under the defaults."""
import numpy as np
import pytest

from ettk_gb300 import synthetic, tuning
from ettk_gb300.metric import ProjectionRotationMetric3D, WedgedSubImage3D

KW = ("lwedge", "uwedge", "normal", "matrix", "position", "cut_offset")


def test_cache_round_trip(tmp_path):
    path = str(tmp_path / "t.json")
    assert tuning.load("GB300", 64, 32, path) is None
    t = {"synth_job_blocks": 32, "eval_chunk": 2048, "zpass_oversub": 2, "sample_block": 256}
    tuning.store("GB300", 64, 32, t, path)
    tuning.store("GB300", 32, 16, dict(t, eval_chunk=8192), path)
    assert tuning.load("GB300", 64, 32, path) == t
    assert tuning.load("GB300", 32, 16, path)["eval_chunk"] == 8192
    assert tuning.load("B200", 64, 32, path) is None
    with open(path, "w") as f:
        f.write("{not json")
    assert tuning.load("GB300", 64, 32, path) is None


@pytest.mark.gpu
def test_autotune_keeps_results_and_applies_its_choice(tmp_path):
    ds = synthetic.generate("align32_b16", n_particles=12)
    m = ProjectionRotationMetric3D(ds.params)
    try:
        m.set_references([WedgedSubImage3D(ds.references[0], **{k: ds.ref_meta[0][k] for k in KW})])
        m.set_particles([WedgedSubImage3D(ds.particles[i], **{k: ds.meta[i][k] for k in KW}) for i in range(12)])
        pairs = [(0, i) for i in range(12)]
        default = m.get_tuning()
        assert default == {"synth_job_blocks": 64, "eval_chunk": 4096, "zpass_oversub": 1, "sample_block": 128}
        D0 = m.getDistances(pairs)
        best, trials = m.autotune(pairs, repeats=1)
        assert len(trials) == 1 + 3 + 3 + 1 + 2
        assert all(t["identical"] for t in trials)
        assert m.get_tuning() == best
        m.set_particles([WedgedSubImage3D(ds.particles[i], **{k: ds.meta[i][k] for k in KW}) for i in range(12)])
        assert np.array_equal(m.getDistances(pairs), D0)
        with pytest.raises(Exception):
            m.set_tuning(dict(best, sample_block=96))
        path = str(tmp_path / "t.json")
        assert tuning.tuned(m, "test-gpu", pairs, repeats=1, path=path) == tuning.load("test-gpu", 32, 16, path)
    finally:
        m.close()
