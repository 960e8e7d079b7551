"""The bulk-copy staged hop (hop5t_kernel: neighbour spinors moved into
shared memory by cp.async.bulk copies tracked on mbarriers, selected with
GBF_HOP5=2) against the oracle.  The switch is read when the library loads,
so the checks run in a child process: Mobius Ls 8 and Ls 12 x 12 packed rhs
in FP32 (one 4D site per block and 16 sites per block), every opcode of the
hop within the FP32 tolerance, and a packed mixed-precision solve (reducing
launches that loop over tiles) to the FP64 oracle's true residual 1e-10."""
import os
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # collected on CPU hosts, skipped there
    pytest.skip("needs a GPU", allow_module_level=True)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r'''
import numpy as np
import gpt_gb300 as g
import oracle as o

def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)

inv, pc = g.algorithms.inverter, g.qcd.fermion.preconditioner
for dims, Ls, n_rhs in [([4, 2, 6, 4], 8, 1), ([8, 8, 8, 8], 12, 12)]:
    U = g.qcd.gauge.random_su3(g.grid(dims), 0.4, 5).U
    p = dict(Ls=Ls, b=1.5, c=0.5, M5=1.8, mass_plus=0.1, mass_minus=0.1, boundary_phases=[1.0, 1.0, 1.0, -1.0])
    ref = o.mobius(U, dims, **p)
    op = g.qcd.fermion.mobius(g.qcd.gauge.gauge_field(g.grid(dims, g.double), U), dict(p, n_rhs=n_rhs))
    o32 = op.converted(g.single)
    rng = np.random.default_rng(3)
    srcs = [rng.standard_normal(ref.shape()) + 1j * rng.standard_normal(ref.shape()) for _ in range(n_rhs)]
    S = o32.F_lattice()
    for k in range(n_rhs):
        S.set_natural(srcs[k], k)
    par = o.parity_of_sites(dims).reshape(-1, 1, 1, 1)
    for name in ["M", "Mdag", "Dhop", "DhopDag"]:
        d = o32.F_lattice()
        o32._apply(name, d, S)
        for k in range(n_rhs):
            assert rel(d.get_natural(k), ref.apply(name, srcs[k])) < 1e-6, (name, k)
    for name in ["Meooe", "MeooeDag"]:
        for sp in [g.even, g.odd]:
            d = o32.F_lattice()
            o32._apply(name, d.half(sp.inv()), S.half(sp))
            for k in range(n_rhs):
                want = ref.apply(name, srcs[k] * (par == sp.code), sp.inv().code)
                assert rel(d.get_natural(k), want) < 1e-6, (name, sp, k)
    P = op.F_lattice()
    for k in range(n_rhs):
        P.set_natural(srcs[k], k)
    dc = inv.defect_correcting(inv.mixed_precision(inv.preconditioned(pc.eo2_ne(), inv.cg({"eps": 1e-5, "maxiter": 4000})),
                                                   g.single, g.double), eps=1e-10, maxiter=40)
    X = dc(op)(P)
    for k in range(n_rhs):
        r = srcs[k] - ref.apply("M", X.get_natural(k))
        assert np.sqrt(o.norm2(r) / o.norm2(srcs[k])) < 1e-10, k
print("bulk-hop-ok")
'''


def test_bulk_copy_hop_vs_oracle():
    env = dict(os.environ, GBF_HOP5="2")
    r = subprocess.run([sys.executable, "-c", CHILD], cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "bulk-hop-ok" in r.stdout, r.stdout[-2000:] + r.stderr[-4000:]
