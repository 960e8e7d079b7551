"""Gauge fields for the fermion operators (lib/gpt/qcd/gauge/create.py).

A gauge field is held in gpt's natural host layout, complex128 [4, V, 3, 3]
(link U_mu(x), site x = x0 + L0*(x1 + L1*(x2 + L2*x3))); the operators copy
it to the device and pack it there (ImportGauge analogue).
"""
import numpy as np

from .. import core


class gauge_field:
    """Links U_mu(x) in the natural layout: a host numpy array
    complex128 [4, V, 3, 3], or a device tensor (float64 view of the same
    layout) for fields that never leave HBM."""

    def __init__(self, grid, U):
        self.grid = grid
        self.device = None
        if hasattr(U, "is_cuda") and U.is_cuda:
            assert U.dtype.is_floating_point and U.numel() == 4 * grid.gsites * 18
            self.device = U.contiguous()
            self.U = None
        else:
            U = np.ascontiguousarray(U, dtype=np.complex128)
            assert U.shape == (4, grid.gsites, 3, 3), U.shape
            self.U = U

    def ptr(self):
        """(pointer, on_device) for gbf_update_gauge."""
        if self.device is not None:
            return self.device.data_ptr(), 1
        return self.U.ctypes.data, 0

    def host(self):
        if self.U is None:
            self.U = self.device.cpu().numpy().view(np.complex128).reshape(4, self.grid.gsites, 3, 3)
        return self.U

    def __getitem__(self, mu):
        return self.host()[mu]

    def __len__(self):
        return 4


def random_su3_device(grid, eps, seed):
    """Same recipe as random_su3, generated in HBM by gbf_random_gauge
    (counter-based Philox4x32-10 random numbers; a different stream than numpy)."""
    import ctypes

    import torch

    from .. import _lib

    U = torch.empty(4 * grid.gsites * 18, dtype=torch.float64, device="cuda")
    dims = (ctypes.c_int * 4)(*grid.fdimensions)
    _lib.check(_lib.load().gbf_random_gauge(dims, float(eps), int(seed), U.data_ptr(), core.stream_ptr()))
    return gauge_field(grid, U)


def unit(grid):
    U = np.zeros((4, grid.gsites, 3, 3), dtype=np.complex128)
    U[:, :, 0, 0] = U[:, :, 1, 1] = U[:, :, 2, 2] = 1.0
    return gauge_field(grid, U)


def _exp_i_hermitian_traceless(Q):
    """exp(iQ) for a batch of 3x3 Hermitian traceless Q by the Cayley-Hamilton
    form exp(iQ) = f0 + f1 Q + f2 Q^2 of Morningstar and Peardon,
    Phys. Rev. D 69 (2004) 054501, eqs. (23)-(34)."""
    Q2 = Q @ Q
    c0 = np.real(np.trace(Q2 @ Q, axis1=1, axis2=2)) / 3.0
    c1 = np.real(np.trace(Q2, axis1=1, axis2=2)) / 2.0
    neg = c0 < 0
    c0a = np.abs(c0)
    c0max = 2.0 * (c1 / 3.0) ** 1.5
    ratio = np.clip(np.divide(c0a, c0max, out=np.zeros_like(c0a), where=c0max > 0), -1.0, 1.0)
    theta = np.arccos(ratio)
    u = np.sqrt(c1 / 3.0) * np.cos(theta / 3.0)
    w = np.sqrt(c1) * np.sin(theta / 3.0)
    small = np.abs(w) < 0.05
    w2 = w * w
    xi0 = np.where(small, 1.0 - w2 / 6.0 * (1.0 - w2 / 20.0 * (1.0 - w2 / 42.0)), np.sin(w) / np.where(small, 1.0, w))
    e2iu = np.exp(2j * u)
    emiu = np.exp(-1j * u)
    cw = np.cos(w)
    u2 = u * u
    h0 = (u2 - w2) * e2iu + emiu * (8.0 * u2 * cw + 2j * u * (3.0 * u2 + w2) * xi0)
    h1 = 2.0 * u * e2iu - emiu * (2.0 * u * cw - 1j * (3.0 * u2 - w2) * xi0)
    h2 = e2iu - emiu * (cw + 3j * u * xi0)
    den = 9.0 * u2 - w2
    bad = np.abs(den) < 1e-12
    den = np.where(bad, 1.0, den)
    f0, f1, f2 = h0 / den, h1 / den, h2 / den
    f0 = np.where(neg, np.conj(f0), f0)
    f1 = np.where(neg, -np.conj(f1), f1)
    f2 = np.where(neg, np.conj(f2), f2)
    U = f0[:, None, None] * np.eye(3) + f1[:, None, None] * Q + f2[:, None, None] * Q2
    if np.any(bad):  # Q ~ 0: Taylor series
        idx = np.nonzero(bad)[0]
        X = 1j * Q[idx]
        T = np.broadcast_to(np.eye(3), X.shape).astype(np.complex128)
        term = T.copy()
        for k in range(1, 20):
            term = term @ X / k
            T = T + term
        U[idx] = T
    return U


def random_su3(grid, eps, seed):
    """The benchmark gauge recipe: U_mu(x) = exp(i eps H), H Hermitian traceless
    with complex-Gaussian entries, drawn from numpy's PCG64(seed)."""
    V = grid.gsites
    rng = np.random.Generator(np.random.PCG64(seed))
    out = np.empty((4 * V, 3, 3), dtype=np.complex128)
    chunk = 1 << 20
    for s in range(0, 4 * V, chunk):
        n = min(chunk, 4 * V - s)
        A = rng.standard_normal((n, 3, 3)) + 1j * rng.standard_normal((n, 3, 3))
        H = 0.5 * (A + np.conj(np.swapaxes(A, 1, 2)))
        tr = np.real(np.trace(H, axis1=1, axis2=2)) / 3.0
        H = H - tr[:, None, None] * np.eye(3)
        out[s:s + n] = _exp_i_hermitian_traceless(eps * H)
    return gauge_field(grid, out.reshape(4, V, 3, 3))


def plaquette(U):
    """Average plaquette (lib/gpt/qcd/gauge/stencil/plaquette.py:25-47), host numpy."""
    dims = U.grid.fdimensions
    V = U.grid.gsites
    x = np.arange(V)
    coords = []
    r = x.copy()
    for L in dims:
        coords.append(r % L)
        r //= L

    def shift(mu):
        c = [cc.copy() for cc in coords]
        c[mu] = (c[mu] + 1) % dims[mu]
        return c[0] + dims[0] * (c[1] + dims[1] * (c[2] + dims[2] * c[3]))

    fw = [shift(m) for m in range(4)]
    tot = 0.0
    for mu in range(4):
        for nu in range(mu):
            H = U.host()
            P = H[mu] @ H[nu][fw[mu]] @ np.conj(np.swapaxes(H[mu][fw[nu]], 1, 2)) @ np.conj(np.swapaxes(H[nu], 1, 2))
            tot += np.real(np.trace(P, axis1=1, axis2=2)).sum()
    return 2.0 * tot / V / 4 / 3 / 3
