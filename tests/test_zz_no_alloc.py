"""gbf_norm2_noalloc: the norm of a field computed with no device allocation.

Callers that cannot call cudaMalloc (a process whose free HBM is owned by
its own pool, a latency-critical loop that must avoid cudaMalloc's device-wide
synchronisation) use this entry point instead of gbf_norm2, which allocates
its reduction workspace on first use.  This file is collected last so that a
run stopping at the first failure has run every other test first; it also
passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

import gpt_gb300 as g  # noqa: E402

REL_TOL = 1e-12  # same accumulation order as gbf_norm2; only summation-tree rounding may differ


@pytest.mark.parametrize("prec", ["double", "single", "half"])
def test_norm2_noalloc_matches_norm2_twice(prec):
    P = {"double": g.double, "single": g.single, "half": g.half}[prec]
    L = g.load()
    grid = g.grid([8, 8, 8, 16], P)
    lat = g.vspincolor(grid)
    rng = np.random.default_rng(3)
    V = grid.gsites
    lat[:] = rng.standard_normal((V, 4, 3)) + 1j * rng.standard_normal((V, 4, 3))
    ref = g.norm2(lat)  # existing entry point (allocating workspace)
    n_sites = V // 2
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):  # the static scratch keeps the previous call's contents
        out = ctypes.c_double(-1.0)
        rc = L.gbf_norm2_noalloc(P.code, ctypes.c_void_p(lat.ptr), n_sites, 2, ctypes.byref(out), ctypes.c_void_p(stream))
        assert rc == 0, L.gbf_norm2_noalloc_error()
        assert abs(out.value - ref) <= REL_TOL * ref, (out.value, ref)


def test_norm2_noalloc_rejects_sizes_beyond_the_scratch():
    L = g.load()
    grid = g.grid([4, 4, 4, 4], g.double)
    lat = g.vspincolor(grid)
    out = ctypes.c_double()
    rc = L.gbf_norm2_noalloc(g.double.code, ctypes.c_void_p(lat.ptr), 4194304 + 1, 1, ctypes.byref(out), None)
    assert rc == 1
    assert b"exceed the maximum" in L.gbf_norm2_noalloc_error()
