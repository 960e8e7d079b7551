"""Block-size autotuning of the native kernels, with an on-disk cache.

Plays the role of lib/gpt/core/auto_tune.py:99-136 (auto_tuned_class: a tag
string names the tuned object, its SHA-256 names a JSON cache file, the
cache holds {"tag", "params", "results"}) for the four kernel classes of an
operator: the hopping kernel with a per-thread epilogue, the hopping kernel
with the Mobius s-matrix epilogue, the site-local kernel and the CG update.
Timing happens in the library (gbf_tune: CUDA events on scratch fields);
this module only keys, stores and re-applies the result.

The cache directory is $GPT_GB300_TUNE_DIR, default ".gpt_gb300_tune" in
the working directory.
"""
import ctypes
import gc
import hashlib
import json
import os

from . import _lib

_runtime_cache = {}


def cache_dir():
    return os.environ.get("GPT_GB300_TUNE_DIR", ".gpt_gb300_tune")


def _device_name():
    import torch

    return torch.cuda.get_device_name(torch.cuda.current_device()) if torch.cuda.is_available() else "none"


def tag_of(op):
    """Everything the best block sizes can depend on."""
    dims = "x".join(str(d) for d in op.U_grid.fdimensions)
    return (f"gbferm/{op.name}/{op.precision.name}/{dims}/Ls{op.Ls}/rhs{op.n_rhs}/"
            f"link{op.link_bytes()}/{_device_name()}")


def cache_file(tag):
    return os.path.join(cache_dir(), hashlib.sha256(tag.encode()).hexdigest() + ".json")


def load(tag):
    fn = cache_file(tag)
    if fn in _runtime_cache:
        return _runtime_cache[fn]
    try:
        with open(fn, "rt") as f:
            data = json.load(f)
        if data.get("tag") != tag or not data.get("params"):
            return None
    except (OSError, ValueError):
        return None
    _runtime_cache[fn] = data
    return data


def save(tag, params, results):
    fn = cache_file(tag)
    data = {"tag": tag, "params": [int(x) for x in params], "results": [float(x) for x in results]}
    os.makedirs(os.path.dirname(fn) or ".", exist_ok=True)
    tmp = fn + f".{os.getpid()}.tmp"
    with open(tmp, "wt") as f:
        json.dump(data, f)
    os.replace(tmp, fn)
    _runtime_cache[fn] = data
    return data


def apply(op, params):
    arr = (ctypes.c_int * 4)(*[int(x) for x in params])
    _lib.check(_lib.load().gbf_set_tuning(op.obj, arr))


def tune(op, force=False, stream=None):
    """Tune `op` (or re-apply its cached result); returns the cache record."""
    from . import core

    tag = tag_of(op)
    if not force:
        data = load(tag)
        if data is not None and len(data["params"]) == 4:
            apply(op, data["params"])
            return data
    bd = (ctypes.c_int * 4)()
    us = (ctypes.c_double * 4)()
    s = core.stream_ptr() if stream is None else stream
    _lib.check(_lib.load().gbf_tune(op.obj, s, bd, us))
    return save(tag, list(bd), list(us))


def rhs_group(make_op, n_sources, candidates=None, budget_bytes=None, iterations=3, tag=None, force=False):
    """Choose how many right-hand sides to pack into one operator (the RHS
    block size) by timing `iterations` eo2_ne CG iterations of the packed
    operator for each candidate size and minimising the time of all groups,
    ceil(n_sources / k) * t_iteration(k).

    make_op(k) builds the operator that the solve spends its time in (the
    inner-precision one) with n_rhs = k.  Candidates whose device footprint,
    extrapolated from the memory the k = 1 trial used, would not fit
    `budget_bytes` (default: 80 % of the free device memory) are skipped.
    Returns {"tag", "params": [k], "results": [[k, ms per iteration], ...]};
    cached like the block sizes when `tag` is given."""
    import math

    import torch

    from . import core

    if tag is not None and not force:
        data = load(tag)
        if data is not None:
            return data
    if candidates is None:
        candidates = [k for k in range(1, min(n_sources, 16) + 1) if n_sources % k == 0]
    free0, _ = torch.cuda.mem_get_info()
    budget = budget_bytes if budget_bytes is not None else int(0.8 * free0)
    L = _lib.load()
    results = []
    per_rhs = None
    for k in sorted(candidates):
        if per_rhs is not None and k * per_rhs > budget:
            continue
        torch.cuda.synchronize()
        before = torch.cuda.mem_get_info()[0]
        op = make_op(k)
        b = op.F_lattice()
        x = op.F_lattice()
        # a seeded Gaussian source for every packed right-hand side
        V = b.layout.grid.gsites * b.layout.Ls
        nat = torch.empty(V * 24, dtype=torch.float64, device="cuda")
        for j in range(k):
            _lib.check(L.gbf_random_spinor(V * 12, 7 + j, nat.data_ptr(), core.stream_ptr()))
            _lib.check(L.gbf_field_import(b.layout.op, nat.data_ptr(), b.ptr, j, int(b.layout.five_d), core.stream_ptr()))
        del nat
        op._solve_eo2ne_cg(x, b, 1e-30, 1, 0, 1)  # warm-up (allocates the workspace)
        torch.cuda.synchronize()
        used = before - torch.cuda.mem_get_info()[0]
        r = op._solve_eo2ne_cg(x, b, 1e-30, iterations, 0, 1)
        ms = sum(r.kernel_ms) / max(1, r.iterations)
        results.append([k, ms])
        if per_rhs is None:
            per_rhs = max(1, used)
        del op, b, x
        # an operator object is part of reference cycles (its matrix
        # operators close over it): collect it now so that its device memory
        # is released before the next, larger candidate
        gc.collect()
        torch.cuda.synchronize()
    best = min(results, key=lambda kr: math.ceil(n_sources / kr[0]) * kr[1])
    data = {"tag": tag, "params": [int(best[0])], "results": [[int(k), float(ms)] for k, ms in results]}
    if tag is not None:
        data = save_rhs(tag, data)
    return data


def save_rhs(tag, data):
    fn = cache_file(tag)
    os.makedirs(os.path.dirname(fn) or ".", exist_ok=True)
    tmp = fn + f".{os.getpid()}.tmp"
    with open(tmp, "wt") as f:
        json.dump(data, f)
    os.replace(tmp, fn)
    _runtime_cache[fn] = data
    return data
