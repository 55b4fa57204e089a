"""ORACLE — test infrastructure only.

CPU restatement of the reference's per-q hot path, used by tests/, by
__graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker.
Nothing in the product (parphom_gb300/, the C-ABI library) imports it.

What it restates (qtm-iisc/PARPHOM, Phonon_Calculations/SRC/):
  * D(q) and dD/dq element by element — dynamical_matrix.F90:49-262, in C
    (oracle/dynmat_ref.c, loaded through ctypes);
  * geometry: crys = (lat^T)^-1 x and rec_lat = 2 pi_f (lat^-1)^T —
    lammps_read.F90:198-200, 228, 250-309 (also in C);
  * the eigensolve: pzheevx(jobz, range, 'U', n, ...) at diagonalize.F90:73-97.
    pzheevx is ScaLAPACK (Intel MKL / AOCL; not vendored in the reference).
    Its serial counterpart with the same argument semantics is LAPACK zheevx,
    called here through scipy.linalg.lapack (OpenBLAS 0.3.x LAPACK): upper
    triangle referenced, range A/I/V, half-open value interval (vl, vu], il/iu
    1-based, abstol.  The value bounds are passed as vl/c and vu/c with
    c = float32(15.633302) * float32(33.35641) rounded to float32, exactly as
    diagonalize.F90:75,94 do (the bounds are compared with eigenvalues of D,
    i.e. squared frequencies, not with frequencies);
  * eigenvalue map eval = sqrt|lam| * sign(lam) (diagonalize.F90:119) and the
    cm^-1 conversion eval * 15.633302 * 33.35641 (write_output.F90:135);
  * group velocities (write_output.F90:410-446): V_k = E^H (dD_k E), keep
    Re diag(V_k), divide by max(2|w_cm|, 1e-3) and multiply by
    33.35641 * 15.633302**2 * 10**2 * 2 * pi_f, single-precision literals
    reproduced.  The reference's second pzgemm passes the same array as B and
    C (write_output.F90:419-421); the restatement computes the intended
    product E^H (dD E).

Parity status: the element routine and unit conversions are restated line by
line; the eigen-oracle is LAPACK zheevx.  The reference ships no output that
matches its shipped force constants (the golden band file's Gamma spectrum
differs from the shipped FORCE_CONSTANTS by up to 27%), so numerical parity
with a reference run is unpinned; the oracle is pinned by the reference's own
known-answer invariance check (Examples/tblg_21.8/check_symm.py with
q_pt_symm.dat) on the shipped N=28 force constants, stored in tests/golden/.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")

F32 = np.float32
C1 = float(F32(15.633302))
C2 = float(F32(33.35641))
C_RANGE = float(F32(F32(15.633302) * F32(33.35641)))       # diagonalize.F90:75
VEL_C2SQ = float(F32(F32(15.633302) * F32(15.633302)))     # (15.633302)**2 in REAL*4
PI_F = float(F32(3.141592653589793))


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "dynmat_ref.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-o", LIB, src, "-lm"])
    return LIB


_lib = None


def _load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB)
        dp = ctypes.POINTER(ctypes.c_double)
        lib.oracle_dynamical_matrix.argtypes = [ctypes.c_int64, dp, dp, dp, dp, dp, dp, dp, ctypes.c_int,
                                                ctypes.c_char, dp]
        lib.oracle_dynamical_matrix.restype = None
        lib.oracle_crys.argtypes = [ctypes.c_int64, dp, dp, dp]
        lib.oracle_matinvtransp3.argtypes = [dp, dp]
        lib.oracle_linsolve.argtypes = [dp, dp, dp]
        lib.oracle_image_mask.argtypes = [ctypes.c_int64, dp, dp, dp, ctypes.c_int64, ctypes.c_int64]
        lib.oracle_image_mask.restype = ctypes.c_uint32
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def fortran_lat(lat_rows: np.ndarray) -> np.ndarray:
    """(3,3) rows=a_i -> column-major buffer of Fortran lat(i,j)."""
    return np.asfortranarray(np.asarray(lat_rows, np.float64)).ravel(order="F").copy()


def geometry(lat_rows: np.ndarray, real_pos: np.ndarray):
    """Returns (crys (natom,3), rec_lat rows (3,3)) as the reference computes them."""
    lib = _load()
    natom = real_pos.shape[0]
    lat_f = fortran_lat(lat_rows)
    pos_f = np.asfortranarray(real_pos, np.float64).ravel(order="F").copy()
    crys_f = np.zeros(natom * 3)
    lib.oracle_crys(natom, _p(lat_f), _p(pos_f), _p(crys_f))
    rec_f = np.zeros(9)
    lib.oracle_matinvtransp3(_p(lat_f), _p(rec_f))
    return crys_f.reshape(3, natom).T.copy(), rec_f.reshape(3, 3, order="F").copy()


class System:
    """Reference-side state (moire%*, force_const%mat) for one cell."""

    def __init__(self, lat, real_pos, masses, at_types, fc):
        self.lat = np.asarray(lat, np.float64)
        self.real_pos = np.asarray(real_pos, np.float64)
        self.natom = self.real_pos.shape[0]
        self.n = 3 * self.natom
        self.masses = np.asarray(masses, np.float64)
        self.at_types = np.asarray(at_types, np.int64)
        self.mass_atom = self.masses[self.at_types - 1].copy()
        self.fc = np.asfortranarray(fc, np.float64)
        self.crys, self.rec_lat = geometry(self.lat, self.real_pos)
        self._lat_f = fortran_lat(self.lat)
        self._rec_f = fortran_lat(self.rec_lat)
        self._crys_f = np.asfortranarray(self.crys).ravel(order="F").copy()
        self._pos_f = np.asfortranarray(self.real_pos).ravel(order="F").copy()
        self._fc_f = self.fc.ravel(order="F").copy()

    @classmethod
    def from_cell(cls, cell, fc):
        return cls(cell.lat, cell.real_pos, cell.masses, cell.at_types, fc)

    def dynmat(self, q, derivative: int = 0, vel_method: str = "A") -> np.ndarray:
        lib = _load()
        n = self.n
        out = np.zeros(2 * n * n)
        qq = np.ascontiguousarray(q, np.float64)
        lib.oracle_dynamical_matrix(self.natom, _p(self._lat_f), _p(self._rec_f), _p(self._crys_f), _p(self._pos_f),
                                    _p(self.mass_atom), _p(self._fc_f), _p(qq), int(derivative),
                                    vel_method.encode()[:1], _p(out))
        return out.view(np.complex128).reshape(n, n, order="F")

    def image_mask(self, I: int, J: int) -> int:
        lib = _load()
        return int(lib.oracle_image_mask(self.natom, _p(self._lat_f), _p(self._crys_f), _p(self._pos_f), I, J))


def zheevx_ref(D: np.ndarray, jobz: str = "N", rng: str = "A", vl: float = 0.0, vu: float = 0.0,
               il: int = 1, iu: int = 1, abstol: float = float(F32(1e-15))):
    """pzheevx semantics through serial LAPACK zheevx (uplo='U').
    vl/vu are in cm^-1 and are converted as diagonalize.F90:75 does."""
    from scipy.linalg import lapack
    n = D.shape[0]
    kw = dict(compute_v=1 if jobz == "V" else 0, range=rng.encode(), lower=0, abstol=abstol)
    if rng == "V":
        kw.update(vl=vl / C_RANGE, vu=vu / C_RANGE)
    elif rng == "I":
        kw.update(il=int(il), iu=int(iu))
    w, z, m, ifail, info = lapack.zheevx(D, **kw)
    m = int(m)
    return w[:m].copy(), (z[:, :m].copy() if jobz == "V" else None), int(info)


def lambda_to_cm(lam: np.ndarray) -> np.ndarray:
    """diagonalize.F90:119 then write_output.F90:135."""
    ev = np.sqrt(np.abs(lam)) * np.where(lam >= 0, 1.0, -1.0)
    return (ev * C1) * C2


def velocity_from_diag(vdiag_re: np.ndarray, w_cm: np.ndarray) -> np.ndarray:
    """write_output.F90:443-446 applied to Re diag(E^H dD_k E)."""
    x = vdiag_re / np.maximum(2.0 * np.abs(w_cm), 1e-3)
    return ((((x * C2) * VEL_C2SQ) * 100.0) * 2.0) * PI_F


def solve_q(sysr: System, q, jobz="N", rng="A", vl=0.0, vu=0.0, il=1, iu=1,
            abstol=float(F32(1e-15)), vel=False, vel_method="A"):
    """One q of the reference loop body (calculations.F90:49-53):
    returns dict(w_cm, lam, z, vel (nz,3) or None, info)."""
    D = sysr.dynmat(q, 0)
    if vel:
        jobz = "V"   # read_input.F90:483-485
    lam, z, info = zheevx_ref(D, jobz, rng, vl, vu, il, iu, abstol)
    w_cm = lambda_to_cm(lam)
    out = dict(w_cm=w_cm, lam=lam, z=z, vel=None, info=info)
    if vel:
        v = np.zeros((z.shape[1], 3))
        for k in range(3):
            dD = sysr.dynmat(q, k + 1, vel_method)
            vk = np.einsum("im,im->m", z.conj(), dD @ z).real
            v[:, k] = velocity_from_diag(vk, w_cm)
        out["vel"] = v
    return out
