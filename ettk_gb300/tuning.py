"""A cache of launch shapes chosen by the autotuner (ettk_gpu_autotune), one entry per GPU model, box edge and
bandwidth, in a JSON file (ETTK_TUNING_CACHE, else ~/.cache/ettk_gb300/tuning.json). The shapes never change a
result, so a stale or foreign entry can only cost speed."""
import json
import os

FIELDS = ("synth_job_blocks", "eval_chunk", "zpass_oversub", "sample_block")


def cache_path():
    return os.environ.get("ETTK_TUNING_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "ettk_gb300",
                                                                 "tuning.json")


def key(device_name, N, B):
    return "%s|N%d|B%d" % (device_name, int(N), int(B))


def load(device_name, N, B, path=None):
    """The cached shapes for (device, N, B), or None."""
    try:
        with open(path or cache_path()) as f:
            entry = json.load(f).get(key(device_name, N, B))
    except (OSError, ValueError):
        return None
    if not isinstance(entry, dict) or any(k not in entry for k in FIELDS):
        return None
    return {k: int(entry[k]) for k in FIELDS}


def store(device_name, N, B, tuning, path=None):
    """Writes the shapes for (device, N, B), keeping the other entries (atomic replace)."""
    path = path or cache_path()
    try:
        with open(path) as f:
            data = json.load(f)
        if not isinstance(data, dict):
            data = {}
    except (OSError, ValueError):
        data = {}
    data[key(device_name, N, B)] = {k: int(tuning[k]) for k in FIELDS}
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def tuned(metric, device_name, sample_pairs, repeats=3, path=None):
    """Applies the cached shapes for the metric's (device, N, B), or runs the autotuner on sample_pairs and caches
    its choice. Returns the shapes in use."""
    N, B = metric.params["N"], metric.params["B"]
    t = load(device_name, N, B, path)
    if t is None:
        t, _ = metric.autotune(sample_pairs, repeats=repeats)
        store(device_name, N, B, t, path)
    else:
        metric.set_tuning(t)
    return t
