"""Solve-level parity of the device path with the reference's own goldens:
the Wilson point-source correlator of tests/qcd/fermion_operators.py:190-218,
computed with the GPU operator in single precision (as the reference does)
from the oracle's restatement of gpt's RNG and gauge recipe."""
import json
import os

import numpy as np
import pytest

import oracle as o

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

import gpt_gb300 as g  # noqa: E402

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))


def test_gpu_wilson_point_correlator_golden():
    G = GOLD["wilson_correlator"]
    dims = G["grid"]
    V = int(np.prod(dims))
    U = o.random(G["seed"]).gauge(o.grid(dims), G["gauge_scale"]).astype(np.complex64).astype(np.complex128)
    ph = [complex(np.cos(k), np.sin(k)) for k in G["boundary_phases_exp_i"]]
    Uf = g.qcd.gauge.gauge_field(g.grid(dims, g.double), U)
    w = g.qcd.fermion.wilson_clover(Uf, dict(kappa=G["kappa"], csw_r=0.0, csw_t=0.0, boundary_phases=ph, n_rhs=12))
    w = w.converted(g.single)
    p = G["point"]
    idx = p[0] + dims[0] * (p[1] + dims[1] * (p[2] + dims[2] * p[3]))
    src_np = np.zeros((12, V, 4, 3), dtype=np.complex128)
    for col in range(12):
        src_np[col, idx, col // 3, col % 3] = 1.0
    src = w.F_lattice()
    src[:] = src_np
    inv = g.algorithms.inverter
    pc = g.qcd.fermion.preconditioner
    cg = inv.cg({"eps": G["cg_eps"], "maxiter": 1000})
    x = inv.preconditioned(pc.eo2_ne(), cg)(w)(src)[:]
    assert cg.last.converged
    corr = (np.abs(x.reshape(12, dims[3], V // dims[3], 12)) ** 2).sum(axis=(0, 2, 3))
    assert np.linalg.norm(corr - np.array(G["correlator"])) < G["tol"]
