"""Differentiable phonon frequencies: a torch.autograd.Function over the C ABI.

`PhononSpectrum(cell).frequencies(q, phi)` returns w(q) in cm^-1 (nq, 3N),
differentiable with respect to the reduced q-points (nq, 3) and the force
constants phi (3N, 3N, symmetric, the reference's matrix after
force_read.F90:187-189).

Device-resident: the cell's context (geometry tables, workspace, captured
graphs) is created once and kept; later forward passes only replace Phi on
the device (pp_ctx_update_fc, from the tensor's own device memory).  q, phi,
the frequencies, the velocities and the gradients stay on the GPU when the
inputs are there; nothing of size n^2 goes through host memory.

Backward:
* dL/dq from Hellmann-Feynman: dw/dk = c^2 Re(e^H dD/dk e) / (2|w|), the
  quantity the group velocity is built from (write_output.F90:443-446), and
  dw/dq_red = rec_lat . dw/dk (k = rec_lat^T q_red);
* dL/dPhi by `pp_backward_phi`: dL/dlambda_j = dL/dw_j * c^2/(2|w_j|)
  (c = 15.633302*33.35641), averaged over clusters of degenerate
  eigenvalues so that the result depends only on the eigenspaces, then
  G = sum_q Re(M_q^T o P_q), M_q = Z diag(dL/dlambda) Z^H.  Eigenvectors are
  recomputed in chunks of `batch` q-points during the backward pass (nothing
  of size n^2 per q is kept between forward and backward unless
  keep_vectors=True).
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
                 batch: int = 8, keep_vectors: bool = False, device=None):
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
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self._ctx = None
        self._phi = None        # the tensor last uploaded (kept alive: its address cannot be reused)
        self._phi_ver = None    # its (address, version, layout) key

    @classmethod
    def from_cell(cls, cell, **kw):
        return cls(cell.lat, cell.real_pos, cell.masses, cell.at_types, **kw)

    def context_for(self, phi: torch.Tensor) -> api.PhononContext:
        """The cell's context with `phi` as its force constants: created on
        the first call, Phi replaced on the device afterwards (skipped when
        the same tensor, unchanged, was uploaded last)."""
        # same storage, layout and version as the tensor uploaded last (which is
        # kept alive, so no other tensor can have taken its address)
        key = (phi.data_ptr(), phi._version, tuple(phi.shape), tuple(phi.stride()), phi.device, phi.dtype)
        if self._ctx is not None and key == self._phi_ver:
            return self._ctx
        if self._ctx is None:
            fc = phi.detach().to(torch.float64).cpu().numpy()
            self._ctx = api.PhononContext(self.lat, self.crys, self.real_pos, self.masses, self.at_types, fc)
        else:
            # column-major device copy (the transpose of the row-major tensor)
            fcd = phi.detach().to(device=self.device, dtype=torch.float64).T.contiguous()
            torch.cuda.current_stream(self.device).synchronize()
            self._ctx.update_fc_device(fcd.data_ptr(), self.n)
        self._phi, self._phi_ver = phi, key
        return self._ctx

    def close(self):
        if self._ctx is not None:
            self._ctx.close()
            self._ctx = None
        self._phi = None

    def frequencies(self, q: torch.Tensor, phi: torch.Tensor) -> torch.Tensor:
        return _Spectrum.apply(q, phi, self)


def cluster_mean(lam: torch.Tensor, c: torch.Tensor) -> torch.Tensor:
    """Replace weights inside clusters of (numerically) equal eigenvalues by
    their mean, so that sum_j c_j e_j e_j^H is basis independent there.
    lam, c: (nq, m), lam ascending per row; on the device."""
    nq, m = lam.shape
    scale = lam.abs().amax(dim=1, keepdim=True).clamp_min(1e-300)
    new = torch.ones_like(lam, dtype=torch.bool)
    new[:, 1:] = (lam[:, 1:] - lam[:, :-1]) > DEGEN_REL * scale
    cid = torch.cumsum(new.to(torch.int64), dim=1) - 1 + m * torch.arange(nq, device=lam.device)[:, None]
    flat = cid.reshape(-1)
    s = torch.zeros(nq * m, dtype=c.dtype, device=c.device).scatter_add_(0, flat, c.reshape(-1))
    k = torch.zeros(nq * m, dtype=c.dtype, device=c.device).scatter_add_(0, flat, torch.ones_like(c).reshape(-1))
    return (s / k.clamp_min(1))[flat].reshape(nq, m)


class _Spectrum(torch.autograd.Function):
    @staticmethod
    def forward(fctx, q, phi, cell: PhononSpectrum):
        dev = cell.device
        ctx = cell.context_for(phi)
        n = cell.n
        qd = q.detach().to(device=dev, dtype=torch.float64)
        nq = qd.shape[0]
        qf = qd.T.contiguous().reshape(-1)           # q[t + nq*k]
        w = torch.zeros((nq, n), dtype=torch.float64, device=dev)
        vel = torch.zeros((nq, n, 3), dtype=torch.float64, device=dev)
        m = torch.zeros(nq, dtype=torch.int64, device=dev)
        nz, info = torch.zeros_like(m), torch.zeros_like(m)
        z = torch.zeros((nq, n, n), dtype=torch.complex128, device=dev) if cell.keep_vectors else None
        opts = api.EigOpts(jobz="V" if z is not None else "N", vel=True, vel_method="A", precision=cell.precision)
        ctx.solve_device(qf, opts, w, m, nz, info, vel_dev=vel, z_dev=z,
                         stream=torch.cuda.current_stream(dev).cuda_stream)
        if int(info.max()) != 0:
            raise api.PPError(int(info.max()), "eigensolver info")
        # dw/dk (cm^-1 A) from the velocities: vel = Re(e^H dD e)/max(2|w|,1e-3) * F
        a = w.abs()
        dwdk = vel * (C_OMEGA ** 2 / VEL_FACTOR) * (torch.clamp_min(2 * a, 1e-3) / torch.clamp_min(2 * a, 1e-300))[
            ..., None]
        rec = torch.as_tensor(cell.rec_lat, dtype=torch.float64, device=dev)
        dwdq = dwdk @ rec.T                             # dw/dq_i = sum_k rec_lat[i,k] dw/dk_k
        fctx.save_for_backward(phi)   # the backward's eigenvectors need this Phi in the context
        fctx.cell = cell
        fctx.q = qd
        fctx.w = w
        fctx.z = z
        fctx.dwdq = dwdq
        fctx.q_dev, fctx.phi_dev = q.device, phi.device
        return w.to(q.device)

    @staticmethod
    def backward(fctx, gw):
        gw = gw.detach().to(device=fctx.cell.device, dtype=torch.float64)
        grad_q = grad_phi = None
        if fctx.needs_input_grad[0]:
            grad_q = torch.einsum("tn,tnk->tk", gw, fctx.dwdq).to(fctx.q_dev)
        if fctx.needs_input_grad[1]:
            grad_phi = _grad_phi(fctx, gw).to(fctx.phi_dev)
        return grad_q, grad_phi, None


def _grad_phi(fctx, gw: torch.Tensor) -> torch.Tensor:
    cell = fctx.cell
    phi, = fctx.saved_tensors
    ctx = cell.context_for(phi)      # re-uploads Phi if a later forward replaced it
    n = cell.n
    dev = cell.device
    w = fctx.w
    lam = torch.sign(w) * (w / C_OMEGA) ** 2
    # dL/dlambda = dL/dw * dw/dlambda, dw/dlambda = c^2 / (2|w|)
    wgt = cluster_mean(lam, gw * (C_OMEGA ** 2) / torch.clamp_min(2 * w.abs(), 1e-3)).contiguous()
    G = torch.zeros((n, n), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    L = api.load()
    nq = w.shape[0]
    B = max(1, min(cell.batch, nq))
    opts = api.EigOpts(jobz="V", vel=False, precision=cell.precision)
    for t0 in range(0, nq, B):
        qb = fctx.q[t0:t0 + B]
        b = qb.shape[0]
        if fctx.z is not None:
            z = fctx.z[t0:t0 + b]
        else:
            wd = torch.zeros((b, n), dtype=torch.float64, device=dev)
            m = torch.zeros(b, dtype=torch.int64, device=dev)
            nz, info = torch.zeros_like(m), torch.zeros_like(m)
            z = torch.zeros((b, n, n), dtype=torch.complex128, device=dev)   # per q: column-major n x n
            ctx.solve_device(qb.T.contiguous().reshape(-1), opts, wd, m, nz, info, z_dev=z,
                             stream=stream.cuda_stream)
        qd = qb.contiguous()
        wg = wgt[t0:t0 + b].contiguous()
        rc = L.pp_backward_phi(ctx._h, ctypes.c_void_p(qd.data_ptr()), b, ctypes.c_void_p(z.data_ptr()), n,
                               2 * n * n, n, ctypes.c_void_p(wg.data_ptr()), n, ctypes.c_void_p(G.data_ptr()),
                               int(cell.precision), ctypes.c_void_p(stream.cuda_stream))
        if rc != 0:
            raise api.PPError(rc, "pp_backward_phi")
    # G is column-major (r + n*c) and symmetric: its row-major view is the same matrix
    return G
