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
        if data.get("tag") != tag or len(data.get("params", [])) != 4:
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
        if data is not None:
            apply(op, data["params"])
            return data
    bd = (ctypes.c_int * 4)()
    us = (ctypes.c_double * 4)()
    s = core.stream_ptr() if stream is None else stream
    _lib.check(_lib.load().gbf_tune(op.obj, s, bd, us))
    return save(tag, list(bd), list(us))
