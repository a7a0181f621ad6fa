"""Autotuner of the sigma build: picks, per active-space shape and precision, the fastest of the
kernel variants that give the same sigma (no counterpart in the reference, whose sigma has one
code path).

Variants: the same-spin kernel's columns per thread (default or half), the opposite-spin grid
(one thread block per alpha string, or one per SM looping over them), and in FP32 the
opposite-spin term on the tensor cores or the CUDA cores and the same-spin terms as sparse row
products or dense tensor-core GEMMs. Each candidate builds sigma for one
seeded vector `reps` times after a warm-up; times come from CUDA events on the current stream.
Choices are cached per (norb, na, nb, precision) for the process, so a pool of solvers of one
shape tunes once.
"""

from __future__ import annotations

import itertools

import numpy as np

_CACHE = {}


def _torch():
    import torch

    return torch


def _apply(sb, choice):
    for name, value in choice.items():
        sb.set_variant(name, value)


def candidates(sb, precision, fixed=None):
    """Variant combinations to time; names in `fixed` keep their given value."""
    fixed = fixed or {}
    opts = {"narrow_same_spin": (0, 1), "persistent_opposite": (0, 1)}
    if precision == "fp32" and sb.set_tensor_cores(True):
        opts["tensor_cores"] = (1, 0)
    if precision == "fp32" and "dense_same_spin" not in fixed:
        # same-spin terms as dense tensor-core GEMMs, where the space allows them
        try:
            sb.set_variant("dense_same_spin", 0)
            sb.set_variant("dense_same_spin", 1)
            opts["dense_same_spin"] = (0, 1)
        except ValueError:
            pass
        sb.set_variant("dense_same_spin", 0)
    for name, value in fixed.items():
        opts[name] = (value,)
    names = list(opts)
    return [dict(zip(names, vals)) for vals in itertools.product(*(opts[n] for n in names))]


def autotune_sigma(sb, norb, na, nb, precision="fp64", reps=2, seed=17, fixed=None):
    """Time every variant on this builder and apply the fastest; variants named in `fixed` keep
    their values. Returns {"choice": {...}, "ms": best, "default_ms": first candidate,
    "timings": [(choice, ms), ...]}."""
    key = (norb, na, nb, precision) if not fixed else (norb, na, nb, precision, tuple(sorted(fixed.items())))
    if not hasattr(sb, "_tuned"):
        sb._tuned = {}
    if key in _CACHE:
        sb._tuned[precision] = dict(_CACHE[key]["choice"])
        if sb.get_precision() == precision:
            _apply(sb, _CACHE[key]["choice"])
        return _CACHE[key]
    torch = _torch()
    ndet = sb.lists.ndet
    prev = sb.get_precision()
    sb.set_precision(precision)
    g = torch.Generator(device="cuda").manual_seed(seed)
    c = torch.rand(ndet, generator=g, dtype=torch.float64, device="cuda") - 0.5
    out = torch.empty_like(c)
    timings = []
    for choice in candidates(sb, precision, fixed):
        _apply(sb, choice)
        sb.Hamiltonian(c, out)  # warm-up (kernel attributes, scratch)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            sb.Hamiltonian(c, out)
        b.record()
        b.synchronize()
        timings.append((choice, a.elapsed_time(b) / reps))
    best = min(timings, key=lambda t: t[1])
    sb._tuned[precision] = dict(best[0])
    sb.set_precision(prev)  # applies the tuned variants of the restored precision, if any
    if prev == precision:
        _apply(sb, best[0])
    res = {"choice": best[0], "ms": best[1], "default_ms": timings[0][1],
           "timings": [(dict(ch), float(ms)) for ch, ms in timings]}
    _CACHE[key] = res
    return res


def cached_choice(norb, na, nb, precision):
    r = _CACHE.get((norb, na, nb, precision))
    return None if r is None else dict(r["choice"])


def clear_cache():
    _CACHE.clear()
