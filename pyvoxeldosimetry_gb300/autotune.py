"""FFT-length autotuner for the convolution plans.

Any FFT length P >= N + K - 1 gives the same linear convolution; the lengths
differ in cost: the padded volume grows with P, but the number of arithmetic
instructions per point depends on P's factorisation (a 288 = 16 x 18 transform
costs markedly less per point than a 280 = 14 x 20 one).  For each axis the
tuner times the candidate lengths that have register four-step kernels
(P <= 1.3 (N + K - 1)), one axis at a time with the other two fixed, on the
real pipeline (per-step CUDA events, L2 flushed between steps), and keeps the
fastest.  Results are cached per device model and problem in a JSON file
(``$PVD_CACHE_DIR`` or ``~/.cache/pyvoxeldosimetry_gb300``), like FFT wisdom.
"""
from __future__ import annotations

import json
import os
import threading
from pathlib import Path
from typing import Sequence, Tuple

import numpy as np
import torch

from . import _native as N

_lock = threading.Lock()
MAX_OVER = 1.3


def cache_path() -> Path:
    base = os.environ.get("PVD_CACHE_DIR")
    d = Path(base) if base else Path.home() / ".cache" / "pyvoxeldosimetry_gb300"
    return d / "fft_tuning.json"


def _load_cache() -> dict:
    p = cache_path()
    try:
        return json.loads(p.read_text())
    except (OSError, ValueError):
        return {}


def _store_cache(c: dict) -> None:
    p = cache_path()
    try:
        p.parent.mkdir(parents=True, exist_ok=True)
        tmp = p.with_suffix(".tmp")
        tmp.write_text(json.dumps(c, indent=1, sort_keys=True))
        tmp.replace(p)
    except OSError:
        pass


def candidates(need: int, max_over: float = MAX_OVER) -> list:
    c = [L for L in N.fast_lengths() if need <= L <= need * max_over]
    return c if c else [0]  # 0: let the plan choose (generic kernels)


def _radial(k: Sequence[int]) -> np.ndarray:
    idx = np.indices(tuple(k), dtype=np.float64)
    r = np.sqrt(sum((idx[i] - k[i] // 2) ** 2 for i in range(3)))
    return np.exp(-r / 2.0) / np.maximum(r, 0.6) ** 2


def _time_plan(shape, kmax, n_kernels, mode, density, pads, device, reps) -> float:
    from .conv import ConvPlan
    with ConvPlan(shape, kmax=kmax, n_kernels=n_kernels, mode=mode, pad=pads, device=device) as p:
        k = _radial(kmax)
        for s in range(n_kernels):
            p.set_kernel(s, k, normalize=True)
        g = torch.Generator(device=device).manual_seed(0)
        a = torch.rand(shape, generator=g, device=device)
        rho = torch.rand(shape, generator=g, device=device) + 0.5 if density else None
        out = torch.empty((n_kernels, *shape), device=device)
        flush = torch.empty(64 * 1024 * 1024, device=device)
        for _ in range(2):
            p.execute(a, density=rho, out=out)
        st = torch.cuda.current_stream(device)
        times = []
        for i in range(reps):
            flush.fill_(float(i))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            p.execute(a, density=rho, out=out)
            e1.record(st)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        del flush
        return float(np.median(times))


def tune(shape: Sequence[int], kmax: Sequence[int], n_kernels: int = 1, mode: str = "linear",
         density: bool = True, device=None, reps: int = 5, use_cache: bool = True) -> Tuple[int, int, int]:
    """FFT lengths (P0, P1, P2) for a LINEAR plan; 0 entries mean 'plan default'."""
    shape = tuple(int(s) for s in shape)
    kmax = tuple(int(k) for k in kmax)
    if mode != "linear":
        return (0, 0, 0)
    device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    name = torch.cuda.get_device_name(device)
    key = f"{name}|{shape}|{kmax}|{n_kernels}|{int(bool(density))}"
    with _lock:
        cache = _load_cache() if use_cache else {}
        if key in cache:
            return tuple(cache[key]["pads"])
        need = [n + k - 1 for n, k in zip(shape, kmax)]
        cand = [candidates(x) for x in need]
        cur = [c[0] for c in cand]
        timings = {}

        def run(pads):
            t = tuple(pads)
            if t not in timings:
                timings[t] = _time_plan(shape, kmax, n_kernels, mode, density,
                                        tuple(x if x else 0 for x in t), device, reps)
            return timings[t]

        for axis in (0, 1, 2):
            best, best_t = cur[axis], None
            for L in cand[axis]:
                trial = list(cur)
                trial[axis] = L
                t = run(trial)
                if best_t is None or t < best_t:
                    best, best_t = L, t
            cur[axis] = best
        result = tuple(cur)
        if use_cache:
            cache = _load_cache()
            cache[key] = {"pads": list(result), "ms": timings[result],
                          "tried": {",".join(map(str, k)): v for k, v in timings.items()}}
            _store_cache(cache)
        return result
