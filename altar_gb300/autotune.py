"""Launch-shape autotuner for the fused forward models.

Each forward model exposes a few launch variants (chains per CTA and the
register budget that sets how many CTAs share an SM, ``ag_forward_variants``).
``tune`` times every variant on a sample of the actual problem with CUDA events
and keeps the fastest; results are cached as JSON keyed by
(model, observations, chains, GPU name) so later runs skip the trials.
The cache path is ``$ALTAR_GB300_TUNE_CACHE`` or ``~/.cache/altar_gb300/autotune.json``.
"""
import json
import os

import torch

from . import _native


def cache_path():
    return os.environ.get("ALTAR_GB300_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "altar_gb300", "autotune.json"))


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save(table):
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(table, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass


def key(kind, m, n, nvar):
    return f"model={kind} m={m} n={n} variants={nvar} gpu={torch.cuda.get_device_name()}"


def tune(strategy, theta, reps=3, sample=8192, use_cache=True):
    """Pick the fastest launch variant of ``strategy`` (a forward-model strategy) for θ's shape."""
    lib = _native.load()
    kind = strategy.kind
    nvar = lib.ag_forward_variants(kind)
    n_full = theta.shape[0]
    k = key(kind, strategy.stations.m, n_full, nvar)
    table = _load() if use_cache else {}
    if k in table:
        strategy.layout.variant = int(table[k]["variant"])
        return table[k]
    th = theta[: min(sample, n_full)].contiguous()
    out = torch.empty(th.shape[0], dtype=torch.float64, device=th.device)
    stream = torch.cuda.current_stream()
    times = []
    for v in range(nvar):
        strategy.layout.variant = v
        strategy.forward(th, out)                     # warm-up (and first-launch costs)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for a, b in ev:
            a.record(stream)
            strategy.forward(th, out)
            b.record(stream)
        torch.cuda.synchronize()
        times.append(min(a.elapsed_time(b) for a, b in ev))
    best = min(range(nvar), key=lambda v: times[v])
    strategy.layout.variant = best
    entry = {"variant": best, "ms": times, "sample_chains": th.shape[0]}
    if use_cache:
        table[k] = entry
        _save(table)
    return entry
