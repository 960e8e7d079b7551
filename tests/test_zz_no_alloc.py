"""gbf_norm2_noalloc: the norm of a field computed with no device allocation.

Callers that cannot call cudaMalloc (a process whose free HBM is owned by
its own pool, a latency-critical loop that must avoid cudaMalloc's device-wide
synchronisation) use this entry point instead of gbf_norm2, which allocates
its reduction workspace on first use.  This file is collected last so that a
run stopping at the first failure has run every other test first; it also
passes on its own in a fresh process.

Each precision is checked against numpy's sum over the values the field holds
(read back in the natural layout) and against the allocating gbf_norm2, on
two calls in a row (the static scratch keeps the previous call's contents),
and the second call must leave the device's free memory unchanged (the
first launch of a kernel may still load its code under CUDA's lazy loading).
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

import gpt_gb300 as g  # noqa: E402

# per-site sums run in the field's arithmetic precision, the cross-site sums
# in FP64: FP64 and double-float agree with numpy to rounding of the sum, FP32
# and FP16 storage (FP32 arithmetic) to a few FP32 ulps
NUMPY_TOL = {"double": 1e-12, "double_float": 1e-12, "single": 1e-6, "half": 1e-6}
# same kernels' per-site arithmetic as gbf_norm2; only the summation tree differs
NORM2_TOL = 1e-12
PREC = {"double": g.double, "double_float": g.double_float, "single": g.single, "half": g.half}


def _call(L, code, ptr, n_sites, nhalves, stream):
    out = ctypes.c_double(-1.0)
    rc = L.gbf_norm2_noalloc(code, ctypes.c_void_p(ptr), n_sites, nhalves, ctypes.byref(out), ctypes.c_void_p(stream))
    assert rc == 0, L.gbf_norm2_noalloc_error()
    return out.value


@pytest.mark.parametrize("prec", ["double", "double_float", "single", "half"])
def test_norm2_noalloc_matches_numpy_and_norm2_twice(prec):
    P = PREC[prec]
    L = g.load()
    grid = g.grid([8, 8, 8, 16], P)
    lat = g.vspincolor(grid)
    rng = np.random.default_rng(3)
    V = grid.gsites
    lat[:] = rng.standard_normal((V, 4, 3)) + 1j * rng.standard_normal((V, 4, 3))
    held = lat[:]  # the values the field holds after rounding to its storage
    want = float(np.vdot(held.ravel(), held.ravel()).real)
    ref = g.norm2(lat)  # the existing, allocating entry point
    n_sites = V // 2
    stream = torch.cuda.current_stream().cuda_stream
    # set-up call: zero sites loads the module and looks up the scratch address
    assert _call(L, P.code, lat.ptr, 0, 2, stream) == 0.0
    for k in range(2):
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        got = _call(L, P.code, lat.ptr, n_sites, 2, stream)
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert abs(got - want) <= NUMPY_TOL[prec] * want, (k, got, want)
        assert abs(got - ref) <= NORM2_TOL * ref, (k, got, ref)
        if k == 1:  # the first launch may still load the kernel's code
            assert free1 == free0, (free0, free1)


def test_norm2_noalloc_rejects_sizes_beyond_the_scratch():
    L = g.load()
    grid = g.grid([4, 4, 4, 4], g.double)
    lat = g.vspincolor(grid)
    out = ctypes.c_double()
    rc = L.gbf_norm2_noalloc(g.double.code, ctypes.c_void_p(lat.ptr), 4194304 + 1, 1, ctypes.byref(out), None)
    assert rc == 1
    assert b"exceed the maximum" in L.gbf_norm2_noalloc_error()
