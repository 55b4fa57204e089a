"""Density of states on the GPU from the frequencies of a q-grid.

Mirrors `moire_phonon_utils.density_of_states` (Utilities/pyphutil/
pyphutil.py:214-359): the q-grid is taken to Cartesian coordinates
(rec_lat^T q), Delaunay-triangulated in the plane, the triangles mapped to
the irreducible points, and the per-triangle sums of bz_integration.f90 are
normalised as DOS *= 1/(3 ntri)/A_moire and ND *= 1/(3 ntri)/A_moire *
3 natom/nbands, A_moire = |det lat[0:2,0:2]| * 0.01 (nm^2).  The smearing
methods weight each q-point's bands by its weight and divide by natom.

The smearing wrapper of the reference passes the whole array of local
weights where the Fortran routine takes one weight per q-point; here each
q-point gets its own weight.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import api

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int64)


def _lib():
    L = api.load()
    if not getattr(L, "_dos_bound", False):
        L.pp_dos_triangulation.argtypes = [_dp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, _dp, _ip,
                                           ctypes.c_int64, _dp, ctypes.c_int64, _dp, _dp]
        L.pp_dos_triangulation.restype = ctypes.c_int
        L.pp_dos_smearing.argtypes = [ctypes.c_int32, _dp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, _dp,
                                      ctypes.c_double, _dp, ctypes.c_int64, ctypes.c_int64, _dp]
        L.pp_dos_smearing.restype = ctypes.c_int
        vp, i64 = ctypes.c_void_p, ctypes.c_int64
        L.pp_dos_triangulation_device.argtypes = [vp, i64, i64, i64, vp, i64, vp, i64, vp, i64, vp, vp, vp]
        L.pp_dos_triangulation_device.restype = ctypes.c_int
        L.pp_dos_smearing_device.argtypes = [ctypes.c_int32, vp, i64, i64, i64, vp, ctypes.c_double, vp, i64, i64,
                                             vp, vp]
        L.pp_dos_smearing_device.restype = ctypes.c_int
        L.pp_velocity_weights_device.argtypes = [vp, i64, i64, i64, ctypes.c_int32, ctypes.c_int32, vp, i64, vp]
        L.pp_velocity_weights_device.restype = ctypes.c_int
        L._dos_bound = True
    return L


def triangulate(grid_red: np.ndarray, rec_lat: np.ndarray, mapping: np.ndarray | None = None) -> np.ndarray:
    """Delaunay triangles of the full grid in Cartesian coordinates, with
    vertices renumbered to the rows of the irreducible-point list (the sorted
    unique values of `mapping`; identity when mapping is None)."""
    from scipy.spatial import Delaunay
    g = np.asarray(grid_red, np.float64) @ np.asarray(rec_lat)
    tri = Delaunay(g[:, :2]).simplices
    if mapping is None:
        return np.ascontiguousarray(tri, np.int64)
    up = np.unique(mapping)
    pos = {v: i for i, v in enumerate(up)}
    return np.array([[pos[mapping[v]] for v in t] for t in tri], np.int64)


def linear_triangulation(freq: np.ndarray, tri: np.ndarray, energy: np.ndarray, func: np.ndarray | None = None):
    """Raw per-triangle sums (dos, nd) of bz_integration.linear_triangulation."""
    freq = np.ascontiguousarray(freq, np.float64)
    nk, nb = freq.shape
    tri = np.ascontiguousarray(tri, np.int64)
    E = np.ascontiguousarray(energy, np.float64)
    f = None if func is None else np.ascontiguousarray(func, np.float64)
    dos = np.zeros(len(E))
    nd = np.zeros(len(E))
    rc = _lib().pp_dos_triangulation(freq.ctypes.data_as(_dp), nb, nk, nb, f.ctypes.data_as(_dp) if f is not None
                                     else None, tri.ctypes.data_as(_ip), len(tri), E.ctypes.data_as(_dp), len(E),
                                     dos.ctypes.data_as(_dp), nd.ctypes.data_as(_dp))
    if rc != 0:
        raise api.PPError(rc, "pp_dos_triangulation")
    return dos, nd


def density_of_states(freq, tri, energy, lat, natom, func=None):
    """(DOS, ND) with the reference's normalisation."""
    nb = np.asarray(freq).shape[1]
    dos, nd = linear_triangulation(freq, tri, energy, func)
    area = abs(np.linalg.det(np.asarray(lat)[0:2, 0:2])) * 0.01
    ntri = len(tri)
    return dos * (1 / ntri / 3) / area, nd * (1 / ntri / 3) / area * 3 * natom / nb


def smearing_dos(freq, weights, energy, width, natom, method="gaussian"):
    freq = np.ascontiguousarray(freq, np.float64)
    nq, nb = freq.shape
    w = np.ascontiguousarray(weights, np.float64)
    E = np.ascontiguousarray(energy, np.float64)
    out = np.zeros(len(E))
    m = {"gaussian": 1, "lorentzian": 2}[method]
    rc = _lib().pp_dos_smearing(m, freq.ctypes.data_as(_dp), nb, nq, nb, w.ctypes.data_as(_dp), float(width),
                                E.ctypes.data_as(_dp), len(E), int(natom), out.ctypes.data_as(_dp))
    if rc != 0:
        raise api.PPError(rc, "pp_dos_smearing")
    return out


# ---- device-resident forms (torch tensors in, torch tensors out) ----------
def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def linear_triangulation_device(freq_dev, tri_dev, energy_dev, nbands=None, func_dev=None, stream=0):
    """Raw per-triangle sums (dos, nd) on the device.  freq_dev (nk, ldf) and
    func_dev (nk, ldfunc) float64 rows per q-point, e.g. the w output of
    PhononContext.solve_device; the first `nbands` columns are used."""
    import torch
    nk, ldf = freq_dev.shape
    nb = ldf if nbands is None else int(nbands)
    ne = int(energy_dev.shape[0])
    dos = torch.empty(ne, dtype=torch.float64, device=freq_dev.device)
    nd = torch.empty_like(dos)
    ldfunc = func_dev.shape[1] if func_dev is not None else nb
    rc = _lib().pp_dos_triangulation_device(_ptr(freq_dev), ldf, nk, nb, _ptr(func_dev), ldfunc, _ptr(tri_dev),
                                            int(tri_dev.shape[0]), _ptr(energy_dev), ne, _ptr(dos), _ptr(nd),
                                            ctypes.c_void_p(int(stream)))
    if rc != 0:
        raise api.PPError(rc, "pp_dos_triangulation_device")
    return dos, nd


def smearing_dos_device(freq_dev, weights_dev, energy_dev, width, natom, method="gaussian", nbands=None, stream=0):
    import torch
    nq, ldf = freq_dev.shape
    nb = ldf if nbands is None else int(nbands)
    ne = int(energy_dev.shape[0])
    out = torch.empty(ne, dtype=torch.float64, device=freq_dev.device)
    m = {"gaussian": 1, "lorentzian": 2}[method]
    rc = _lib().pp_dos_smearing_device(m, _ptr(freq_dev), ldf, nq, nb, _ptr(weights_dev), float(width),
                                       _ptr(energy_dev), ne, int(natom), _ptr(out), ctypes.c_void_p(int(stream)))
    if rc != 0:
        raise api.PPError(rc, "pp_dos_smearing_device")
    return out


def velocity_weights_device(vel_dev, a=-1, b=-1, nbands=None, stream=0):
    """Transport-DOS weights v_a v_b (or |v|^2 with a = b = -1) per (q, mode)
    from a (nq, n, 3) velocity tensor of PhononContext.solve_device."""
    import torch
    nq, n, _ = vel_dev.shape
    nb = n if nbands is None else int(nbands)
    func = torch.empty((nq, nb), dtype=torch.float64, device=vel_dev.device)
    rc = _lib().pp_velocity_weights_device(_ptr(vel_dev), 3 * n, nq, nb, int(a), int(b), _ptr(func), nb,
                                           ctypes.c_void_p(int(stream)))
    if rc != 0:
        raise api.PPError(rc, "pp_velocity_weights_device")
    return func
