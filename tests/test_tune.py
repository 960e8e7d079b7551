"""Block-size autotuner: cache handling (CPU) and tuned launches (GPU).

The cache follows lib/gpt/core/auto_tune.py:99-136 (tag -> SHA-256 file
name, {"tag", "params", "results"} record, tag checked on load).
"""
import ctypes
import json
import os

import numpy as np
import pytest

from gpt_gb300 import _lib
from gpt_gb300 import tune as T


def test_cache_roundtrip_and_tag_check(tmp_path, monkeypatch):
    monkeypatch.setenv("GPT_GB300_TUNE_DIR", str(tmp_path))
    T._runtime_cache.clear()
    tag = "gbferm/wilson_clover/single/8x8x8x8/Ls1/rhs1/link48/dev"
    assert T.load(tag) is None
    T.save(tag, [128, 0, 256, 64], [1.0, 0.0, 2.0, 3.0])
    T._runtime_cache.clear()
    d = T.load(tag)
    assert d["params"] == [128, 0, 256, 64] and d["tag"] == tag
    # a file whose tag differs (hash collision or edited file) is ignored
    fn = T.cache_file(tag)
    rec = json.load(open(fn))
    rec["tag"] = "other"
    json.dump(rec, open(fn, "w"))
    T._runtime_cache.clear()
    assert T.load(tag) is None
    # a truncated file is ignored too
    open(fn, "w").write("{")
    assert T.load(tag) is None
    assert os.path.dirname(fn) == str(tmp_path)


def test_tuning_entry_points_reject_null_arguments():
    L = _lib.load()
    bd = (ctypes.c_int * 4)(64, 0, 64, 64)
    assert L.gbf_set_tuning(None, bd) == 1
    assert L.gbf_tune(None, None, bd, None) == 1
    assert b"null" in L.gbf_last_error()


# ---------------------------------------------------------------------------
# GPU: tuned operators give the same results
# ---------------------------------------------------------------------------
torch = pytest.importorskip("torch")
gpu = pytest.mark.gpu


def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")


def _rand(shape, seed):
    r = np.random.default_rng(seed)
    return r.standard_normal(shape) + 1j * r.standard_normal(shape)


@gpu
@pytest.mark.parametrize("kind,params", [
    ("wilson_clover", dict(mass=0.1, csw_r=1.0, csw_t=1.0, boundary_phases=[1, 1, 1, -1])),
    ("mobius", dict(Ls=8, b=1.5, c=0.5, M5=1.8, mass_plus=0.1, mass_minus=0.1, boundary_phases=[1, 1, 1, -1])),
])
def test_tuned_operator_matches_untuned(kind, params, tmp_path, monkeypatch):
    _need_gpu()
    import gpt_gb300 as g
    import oracle as o

    monkeypatch.setenv("GPT_GB300_TUNE_DIR", str(tmp_path))
    T._runtime_cache.clear()
    dims = [8, 8, 8, 8]
    U = g.qcd.gauge.random_su3(g.grid(dims), 0.4, 31).U
    Uf = g.qcd.gauge.gauge_field(g.grid(dims, g.double), U)
    mk = g.qcd.fermion.wilson_clover if kind == "wilson_clover" else g.qcd.fermion.mobius
    op64 = mk(Uf, params)
    op = op64.converted(g.single)
    src_np = _rand(op.F_lattice()[:].shape, 4)
    src = op.F_lattice()
    src[:] = src_np
    before = op.M(src)[:].copy()

    rec = op.tune()
    bd = rec["params"]
    N5 = op.Ls * op.n_rhs
    for cls, b in enumerate(bd):
        if cls == 1 and kind != "mobius":
            assert b == 0
            continue
        assert 0 < b <= 256 and b % N5 == 0 and ((b // N5) & (b // N5 - 1)) == 0
        assert rec["results"][cls] > 0
    # applying an operator does not depend on the block size: bitwise equal
    after = op.M(src)[:]
    assert np.array_equal(before, after)

    # a second operator of the same kind picks the cached choice without timing
    op2 = op64.converted(g.single)
    rec2 = op2.tune()
    assert rec2["params"] == bd and os.path.exists(T.cache_file(rec["tag"]))

    # the tuned CG still solves the system (oracle: FP64 residual of M x = b)
    ref = (o.wilson_clover(U, dims, **params) if kind == "wilson_clover"
           else o.mobius(U, dims, **params))
    b = _rand(ref.shape(), 9)
    inv = g.algorithms.inverter
    pc = g.qcd.fermion.preconditioner
    cg = inv.cg({"eps": 1e-5, "maxiter": 4000})
    x = inv.preconditioned(pc.eo2_ne(), cg)(op)(_to(op, b))[:]
    assert cg.last.converged
    r = b - ref.apply("M", x)
    assert np.sqrt(o.norm2(r) / o.norm2(b)) < 1e-4


def _to(op, arr):
    lat = op.F_lattice()
    lat[:] = arr
    return lat


def test_rhs_group_cache_record(tmp_path, monkeypatch):
    monkeypatch.setenv("GPT_GB300_TUNE_DIR", str(tmp_path))
    T._runtime_cache.clear()
    rec = T.save_rhs("rhs/mobius/test", {"tag": "rhs/mobius/test", "params": [3], "results": [[1, 2.0], [3, 5.0]]})
    T._runtime_cache.clear()
    assert T.load("rhs/mobius/test")["params"] == [3] and rec["results"][1] == [3, 5.0]


@gpu
def test_rhs_group_tuner_picks_a_timed_candidate(tmp_path, monkeypatch):
    _need_gpu()
    import gpt_gb300 as g

    monkeypatch.setenv("GPT_GB300_TUNE_DIR", str(tmp_path))
    T._runtime_cache.clear()
    dims = [4, 4, 4, 8]
    U = g.qcd.gauge.random_su3(g.grid(dims, g.double), 0.4, 3)
    base = dict(Ls=4, b=1.5, c=0.5, M5=1.8, mass_plus=0.1, mass_minus=0.1, boundary_phases=[1, 1, 1, -1])
    rec = T.rhs_group(lambda k: g.qcd.fermion.mobius_operator(U, dict(base, n_rhs=k), precision=g.single), 4,
                      candidates=[1, 2, 4], tag="rhs/test")
    assert [r[0] for r in rec["results"]] == [1, 2, 4]
    assert all(r[1] > 0 for r in rec["results"])
    assert rec["params"][0] in (1, 2, 4)
    assert T.rhs_group(None, 4, tag="rhs/test")["params"] == rec["params"]  # cached
