"""Launch-shape and kernel-form autotuner with a cache file.

No reference counterpart (the reference has no GPU code).  A candidate is a
set of launch knobs (nfem_knob_set: Darcy row-pass blocks per SM, Darcy
cell-pass block size, elasticity warps per block) plus form attributes (the
Darcy one-pass / two-pass / cell-chunk choice).  `tune` times every
candidate on the caller's own assembly with CUDA events (L2 flushed before
each repetition), keeps the fastest, applies it, and stores it in a JSON
cache keyed by GPU name and workload signature; `apply_cached` restores a
stored choice without timing.

Cache file: $NFEM_TUNING_CACHE, else ~/.cache/nfempy_gb300/tuning.json.
"""
import json
import os

import torch

from . import _lib

KNOBS = {"darcy_rows_blocks_per_sm": 0, "darcy_cells_block": 1, "elas_warps": 2, "elas_rows": 3, "coarse_tc": 4, "darcy_f64_records": 5}


def cache_path():
    return os.environ.get("NFEM_TUNING_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "nfempy_gb300", "tuning.json"))


def _load():
    try:
        with open(cache_path()) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _store(data):
    path = cache_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as fh:
        json.dump(data, fh, indent=1, sort_keys=True)
    os.replace(tmp, path)


def gpu_name():
    return torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"


def set_knobs(knobs):
    for name, value in knobs.items():
        _lib.call("nfem_knob_set", KNOBS[name], int(value))


def reset_knobs():
    set_knobs({k: 0 for k in KNOBS})


def apply(config, form=None):
    """Set a candidate's knobs and its form attributes."""
    reset_knobs()
    set_knobs(config.get("knobs", {}))
    if form is not None:
        for k, v in config.get("form", {}).items():
            setattr(form, k, v)


def apply_cached(key, form=None):
    """Apply the stored choice for `key`; returns it, or None when absent."""
    entry = _load().get(gpu_name(), {}).get(key)
    if entry is not None:
        apply(entry["config"], form)
    return entry


def _time(fn, reps, flush):
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    fn()
    for e0, e1 in ev:
        flush.zero_()
        e0.record()
        fn()
        e1.record()
    torch.cuda.synchronize()
    return min(a.elapsed_time(b) for a, b in ev)


def tune(key, run, candidates, form=None, reps=5, store=True):
    """Time `run()` under every candidate (dicts with "knobs" and "form"),
    apply the fastest and cache it under `key`.  Returns (best config, its
    ms, {candidate index: ms})."""
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    times = {}
    for i, cfg in enumerate(candidates):
        apply(cfg, form)
        times[i] = _time(run, reps, flush)
    best = min(times, key=times.get)
    apply(candidates[best], form)
    if store:
        data = _load()
        data.setdefault(gpu_name(), {})[key] = {"config": candidates[best], "ms": times[best],
                                                "candidates": len(candidates)}
        _store(data)
    return candidates[best], times[best], times


def darcy_candidates(dim):
    """The Darcy assembly's forms and launch shapes."""
    out = []
    for rec in (False, True):
        for bps in (0, 4, 6, 8):
            for cb in ((256,) if not rec else (128, 256, 512)):
                out.append({"form": {"use_records": rec, "use_chunks": False},
                            "knobs": {"darcy_rows_blocks_per_sm": bps, "darcy_cells_block": cb}})
    out.append({"form": {"use_records": False, "use_chunks": True}, "knobs": {}})
    return out


def elasticity_candidates():
    return ([{"form": {}, "knobs": {"elas_rows": 2}}, {"form": {}, "knobs": {"elas_rows": 3}}]
            + [{"form": {}, "knobs": {"elas_rows": 1, "elas_warps": w}} for w in (2, 4, 8)])


def darcy_key(space, dtype):
    return f"darcy{space.dim}d_{str(dtype).split('.')[-1]}_cells{space.n_cells}_rows{space.n_dof}"
