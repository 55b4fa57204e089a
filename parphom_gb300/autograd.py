"""Differentiable phonon frequencies: a torch.autograd.Function over the C ABI.

`PhononSpectrum(cell).frequencies(q, phi)` returns w(q) in cm^-1 (nq, 3N),
differentiable with respect to the reduced q-points (nq, 3) and the force
constants phi (3N, 3N, symmetric, the reference's matrix after
force_read.F90:187-189).

Backward:
* dL/dq from Hellmann-Feynman: dw/dk = c^2 Re(e^H dD/dk e) / (2|w|), the
  quantity the group velocity is built from (write_output.F90:443-446), and
  dw/dq_red = rec_lat . dw/dk (k = rec_lat^T q_red);
* dL/dPhi by `pp_backward_phi`: dL/dlambda_j = dL/dw_j * c^2/(2|w_j|)
  (c = 15.633302*33.35641), averaged over clusters of degenerate
  eigenvalues so that the result depends only on the eigenspaces, then
  G = sum_q Re(M_q^T o P_q), M_q = Z diag(dL/dlambda) Z^H.  Eigenvectors are
  recomputed in batches during the backward pass (nothing of size n^2 per q
  is kept between forward and backward unless keep_vectors=True).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import api, geometry

C1 = float(np.float32(15.633302))
C2 = float(np.float32(33.35641))
C_OMEGA = C1 * C2
VEL_FACTOR = ((((1.0 * C2) * float(np.float32(np.float32(15.633302) * np.float32(15.633302)))) * 100.0) * 2.0) \
    * float(np.float32(3.141592653589793))
DEGEN_REL = 1e-9


class PhononSpectrum:
    """Geometry of one cell; force constants and q-points are arguments."""

    def __init__(self, lat, real_pos, masses, at_types, crys=None, precision=api.PP_PREC_MIXED,
                 batch: int = 8, keep_vectors: bool = False):
        self.lat = np.asarray(lat, np.float64)
        self.real_pos = np.asarray(real_pos, np.float64)
        self.crys = geometry.crys_from_positions(self.lat, self.real_pos) if crys is None else np.asarray(crys)
        self.masses = np.asarray(masses, np.float64)
        self.at_types = np.asarray(at_types, np.int64)
        self.rec_lat = geometry.reciprocal_lattice(self.lat)
        self.n = 3 * self.real_pos.shape[0]
        self.precision = precision
        self.batch = batch
        self.keep_vectors = keep_vectors

    @classmethod
    def from_cell(cls, cell, **kw):
        return cls(cell.lat, cell.real_pos, cell.masses, cell.at_types, **kw)

    def context(self, phi_np: np.ndarray) -> api.PhononContext:
        return api.PhononContext(self.lat, self.crys, self.real_pos, self.masses, self.at_types, phi_np)

    def frequencies(self, q: torch.Tensor, phi: torch.Tensor) -> torch.Tensor:
        return _Spectrum.apply(q, phi, self)


def _cluster_mean(lam: np.ndarray, c: np.ndarray) -> np.ndarray:
    """Replace weights inside clusters of (numerically) equal eigenvalues by
    their mean, so that sum_j c_j e_j e_j^H is basis independent there."""
    out = c.copy()
    scale = max(np.abs(lam).max(), 1e-300)
    j = 0
    m = len(lam)
    while j < m:
        k = j + 1
        while k < m and lam[k] - lam[k - 1] <= DEGEN_REL * scale:
            k += 1
        if k - j > 1:
            out[j:k] = c[j:k].mean()
        j = k
    return out


class _Spectrum(torch.autograd.Function):
    @staticmethod
    def forward(fctx, q, phi, cell: PhononSpectrum):
        q_np = q.detach().cpu().numpy().astype(np.float64)
        phi_np = phi.detach().cpu().numpy().astype(np.float64)
        ctx = cell.context(phi_np)
        opts = api.EigOpts(jobz="V", vel=True, vel_method="A", precision=cell.precision)
        res = ctx.solve(q_np, opts, want_z=cell.keep_vectors)
        w = res.w
        # dw/dk (cm^-1 A) from the velocities: vel = Re(e^H dD e)/max(2|w|,1e-3) * F
        a = np.abs(w)
        dwdk = res.vel * (C_OMEGA ** 2 / VEL_FACTOR) * (np.maximum(2 * a, 1e-3) / np.maximum(2 * a, 1e-300))[..., None]
        dwdq = dwdk @ cell.rec_lat.T          # (nq, n, 3): dw/dq_i = sum_k rec_lat[i,k] dw/dk_k
        fctx.cell = cell
        fctx.ctx = ctx
        fctx.q_np = q_np
        fctx.w = w
        fctx.z = res.z
        fctx.dwdq = dwdq
        fctx.dev = q.device
        fctx.phi_dev = phi.device
        return torch.as_tensor(w, dtype=torch.float64, device=q.device)

    @staticmethod
    def backward(fctx, gw):
        gw_np = gw.detach().cpu().numpy().astype(np.float64)
        grad_q = grad_phi = None
        if fctx.needs_input_grad[0]:
            grad_q = torch.as_tensor(np.einsum("tn,tnk->tk", gw_np, fctx.dwdq), dtype=torch.float64,
                                     device=fctx.dev)
        if fctx.needs_input_grad[1]:
            grad_phi = torch.as_tensor(_grad_phi(fctx, gw_np), dtype=torch.float64, device=fctx.phi_dev)
        return grad_q, grad_phi, None


def _grad_phi(fctx, gw: np.ndarray) -> np.ndarray:
    cell, ctx = fctx.cell, fctx.ctx
    n = cell.n
    w = fctx.w
    lam = np.sign(w) * (w / C_OMEGA) ** 2
    # dL/dlambda = dL/dw * dw/dlambda, dw/dlambda = c^2 / (2|w|)
    wgt = gw * (C_OMEGA ** 2) / np.maximum(2 * np.abs(w), 1e-3)
    for t in range(len(wgt)):
        wgt[t] = _cluster_mean(lam[t], wgt[t])
    dev = torch.device("cuda", torch.cuda.current_device())
    G = torch.zeros((n, n), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    L = api.load()
    nq = len(wgt)
    B = max(1, min(cell.batch, nq))
    opts = api.EigOpts(jobz="V", vel=False, precision=cell.precision)
    for t0 in range(0, nq, B):
        qb = fctx.q_np[t0:t0 + B]
        b = len(qb)
        if fctx.z is not None:
            z = torch.as_tensor(np.ascontiguousarray(fctx.z[t0:t0 + b].transpose(0, 2, 1)), device=dev)
        else:
            qf = torch.as_tensor(np.asfortranarray(qb).ravel(order="F"), device=dev)
            wd = torch.zeros((b, n), dtype=torch.float64, device=dev)
            m = torch.zeros(b, dtype=torch.int64, device=dev)
            nz = torch.zeros_like(m)
            info = torch.zeros_like(m)
            z = torch.zeros((b, n, n), dtype=torch.complex128, device=dev)   # per q: column-major n x n
            ctx.solve_device(qf, opts, wd, m, nz, info, z_dev=z, stream=stream.cuda_stream)
        qd = torch.as_tensor(np.ascontiguousarray(qb), device=dev)
        wg = torch.as_tensor(np.ascontiguousarray(wgt[t0:t0 + b]), device=dev)
        rc = L.pp_backward_phi(ctx._h, ctypes.c_void_p(qd.data_ptr()), b, ctypes.c_void_p(z.data_ptr()), n,
                               2 * n * n, n, ctypes.c_void_p(wg.data_ptr()), n, ctypes.c_void_p(G.data_ptr()),
                               int(cell.precision), ctypes.c_void_p(stream.cuda_stream))
        if rc != 0:
            raise api.PPError(rc, "pp_backward_phi")
    torch.cuda.synchronize(dev)
    # G is column-major (r + n*c); symmetric, so the transpose is the same matrix
    return G.cpu().numpy().T.copy()
