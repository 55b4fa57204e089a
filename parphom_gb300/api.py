"""Python binding of libparphom_gpu.so (the C ABI in include/parphom_gpu.h).

`PhononContext` mirrors the reference driver's state after
read_lammps_data / read_force_constants (Phonon_Calculations/SRC/main.F90:53-62)
and `PhononContext.solve` the per-q loop body of calculations.F90:49-53:
D(q) assembly, the pzheevx-equivalent eigensolve and the group velocities.
Arguments keep the reference's names and meaning (jobz/range/vl/vu/il/iu/
abstol/orfac as in diagonalize.F90:73-97, `vel_method` 'A'/'C' as in
read_input.F90:178-194).  There is no CPU fallback: without the library or a
GPU every call raises.
"""
from __future__ import annotations

import ctypes
import dataclasses
import os
from typing import Optional

import numpy as np

from . import build as _build

PP_PREC_FP64 = 0
PP_PREC_MIXED = 1
PP_FLAG_ENFORCE_ASR = 1

INFO_NOCONV = 1
INFO_NOORTH = 2
INFO_NOMEM = 4
INFO_NOTCOMP = 8
INFO_TIMEOUT = 16
INFO_NAN = 32

EXPORTED = ("pp_ctx_create", "pp_ctx_destroy", "pp_solve_batch", "pp_solve_batch_device", "pp_dynamical_matrix",
            "pp_strerror", "pp_version", "pp_kernel_launches", "pp_ktimer_enable", "pp_ktimer_report",
            "pp_heevx_values_noalloc", "pp_backward_phi", "pp_solve_multi", "pp_debug_stall_tc_wait",
            "pp_ctx_update_fc", "pp_dos_triangulation_device", "pp_dos_smearing_device",
            "pp_velocity_weights_device", "pp_autotune_report")
PP_ERR_SIZE = 1008
PP_NOALLOC_MAX_N = 1536

_i64 = ctypes.c_int64
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int64)


class PPSystem(ctypes.Structure):
    _fields_ = [("natom", _i64), ("ntypes", _i64), ("lat", _dp), ("crys", _dp), ("real_pos", _dp),
                ("mass", _dp), ("at_types", _ip)]


class PPEigOpts(ctypes.Structure):
    _fields_ = [("jobz", ctypes.c_char), ("range", ctypes.c_char), ("vel_method", ctypes.c_char),
                ("uplo", ctypes.c_char), ("vel", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("vl", ctypes.c_double), ("vu", ctypes.c_double), ("il", _i64), ("iu", _i64),
                ("abstol", ctypes.c_double), ("orfac", ctypes.c_double), ("raw_lambda", ctypes.c_int32),
                ("want_resid", ctypes.c_int32)]


class PPResultView(ctypes.Structure):
    _fields_ = [("m", _ip), ("nz", _ip), ("w", _dp), ("ldw", _i64), ("z", _dp), ("ldz", _i64), ("zstride", _i64),
                ("vel", _dp), ("velstride", _i64), ("resid", _dp), ("werr", _dp), ("zerr", _dp)]


class PPError(RuntimeError):
    def __init__(self, code: int, what: str):
        self.code = code
        super().__init__(f"{what}: {strerror(code)} (code {code})")


_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load the C-ABI library (building it first if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise FileNotFoundError(f"{path} is not built")
        _build.build()
    L = ctypes.CDLL(path)
    L.pp_ctx_create.argtypes = [ctypes.POINTER(PPSystem), _dp, _i64, _i64, ctypes.POINTER(ctypes.c_void_p)]
    L.pp_ctx_create.restype = ctypes.c_int
    L.pp_ctx_update_fc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, _i64, _i64, ctypes.c_int32]
    L.pp_ctx_update_fc.restype = ctypes.c_int
    L.pp_ctx_destroy.argtypes = [ctypes.c_void_p]
    L.pp_ctx_destroy.restype = ctypes.c_int
    L.pp_solve_batch.argtypes = [ctypes.c_void_p, _dp, _i64, _i64, ctypes.POINTER(PPEigOpts),
                                 ctypes.POINTER(PPResultView), _ip]
    L.pp_solve_batch.restype = ctypes.c_int
    L.pp_solve_batch_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, _i64, _i64, ctypes.POINTER(PPEigOpts),
                                        ctypes.POINTER(PPResultView), ctypes.c_void_p, ctypes.c_void_p]
    L.pp_solve_batch_device.restype = ctypes.c_int
    L.pp_dynamical_matrix.argtypes = [ctypes.c_void_p, _dp, _i64, ctypes.c_char, _dp, _i64]
    L.pp_dynamical_matrix.restype = ctypes.c_int
    L.pp_strerror.argtypes = [ctypes.c_int]
    L.pp_strerror.restype = ctypes.c_char_p
    L.pp_version.restype = _i64
    L.pp_kernel_launches.restype = _i64
    L.pp_heevx_values_noalloc.argtypes = [ctypes.c_void_p, _i64, _i64, ctypes.c_char, ctypes.c_double,
                                          ctypes.c_double, _i64, _i64, ctypes.c_double, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.pp_heevx_values_noalloc.restype = ctypes.c_int
    L.pp_solve_multi.argtypes = [ctypes.POINTER(ctypes.c_void_p), _i64, _ip, _dp, _i64, _i64,
                                 ctypes.POINTER(PPEigOpts), ctypes.POINTER(PPResultView), _ip]
    L.pp_solve_multi.restype = ctypes.c_int
    L.pp_backward_phi.argtypes = [ctypes.c_void_p, ctypes.c_void_p, _i64, ctypes.c_void_p, _i64, _i64, _i64,
                                  ctypes.c_void_p, _i64, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]
    L.pp_backward_phi.restype = ctypes.c_int
    L.pp_autotune_report.argtypes = [ctypes.c_char_p, _i64]
    L.pp_autotune_report.restype = ctypes.c_int
    L.pp_debug_stall_tc_wait.argtypes = [_i64, _i64]
    L.pp_debug_stall_tc_wait.restype = ctypes.c_int
    L.pp_ktimer_enable.argtypes = [ctypes.c_char_p]
    L.pp_ktimer_enable.restype = ctypes.c_int
    L.pp_ktimer_report.argtypes = [ctypes.c_char_p, _i64]
    L.pp_ktimer_report.restype = ctypes.c_int
    _lib = L
    return L


def strerror(code: int) -> str:
    try:
        return load().pp_strerror(int(code)).decode()
    except Exception:  # library not loadable: plain text
        return f"error {code}"


def _p(a: np.ndarray):
    return a.ctypes.data_as(_dp)


@dataclasses.dataclass
class EigOpts:
    """pzheevx options (diagonalize.F90:73-97) plus the velocity switches."""
    jobz: str = "N"
    range: str = "A"
    vl: float = 0.0
    vu: float = 0.0
    il: int = 1
    iu: int = 1
    abstol: float = float(np.float32(1e-15))
    orfac: float = float(np.float32(1e-15))
    vel: bool = False
    vel_method: str = "A"
    precision: int = PP_PREC_FP64
    raw_lambda: bool = False
    want_resid: bool = False   # per-eigenpair error estimates (Result.resid/werr/zerr)

    def to_c(self) -> PPEigOpts:
        return PPEigOpts(self.jobz.encode()[:1], self.range.encode()[:1], self.vel_method.encode()[:1], b"U",
                         int(bool(self.vel)), int(self.precision), float(self.vl), float(self.vu), int(self.il),
                         int(self.iu), float(self.abstol), float(self.orfac), int(bool(self.raw_lambda)),
                         int(bool(self.want_resid)))


@dataclasses.dataclass
class Result:
    m: np.ndarray          # (nq,) eigenvalues found
    nz: np.ndarray         # (nq,) eigenvectors computed
    w: np.ndarray          # (nq, n) frequencies (cm^-1) or eigenvalues; entries >= m are unset
    z: Optional[np.ndarray]    # (nq, n, mz) complex, column j = eigenvector j; mz = n, or iu-il+1 for range I
    vel: Optional[np.ndarray]  # (nq, n, 3) m/s
    info: np.ndarray       # (nq,) pzheevx-style bits
    resid: Optional[np.ndarray] = None  # (nq, n) ||D z - lambda z|| (want_resid)
    werr: Optional[np.ndarray] = None   # (nq, n) error bound of w (cm^-1, or lambda units)
    zerr: Optional[np.ndarray] = None   # (nq, n) bound on sin(angle) of each eigenvector


class PhononContext:
    """One cell on the current GPU (pp_ctx)."""

    def __init__(self, lat, crys, real_pos, masses, at_types, fc, enforce_asr: bool = False):
        L = load()
        self._lib = L
        self.natom = int(np.asarray(real_pos).shape[0])
        self.n = 3 * self.natom
        lat_f = np.asfortranarray(np.asarray(lat, np.float64)).ravel(order="F").copy()
        crys_f = np.asfortranarray(np.asarray(crys, np.float64)).ravel(order="F").copy()
        pos_f = np.asfortranarray(np.asarray(real_pos, np.float64)).ravel(order="F").copy()
        mass = np.ascontiguousarray(masses, np.float64)
        types = np.ascontiguousarray(at_types, np.int64)
        fcf = np.asfortranarray(fc, np.float64)
        self._keep = (lat_f, crys_f, pos_f, mass, types)
        sysc = PPSystem(self.natom, len(mass), _p(lat_f), _p(crys_f), _p(pos_f), _p(mass),
                        types.ctypes.data_as(_ip))
        h = ctypes.c_void_p()
        rc = L.pp_ctx_create(ctypes.byref(sysc), fcf.ctypes.data_as(_dp), self.n,
                             PP_FLAG_ENFORCE_ASR if enforce_asr else 0, ctypes.byref(h))
        if rc != 0:
            raise PPError(rc, "pp_ctx_create")
        self._h = h

    @classmethod
    def from_cell(cls, cell, fc, crys=None, **kw):
        from .geometry import crys_from_positions
        if crys is None:
            crys = crys_from_positions(cell.lat, cell.real_pos)
        return cls(cell.lat, crys, cell.real_pos, cell.masses, cell.at_types, fc, **kw)

    def update_fc(self, fc, enforce_asr: bool = False) -> None:
        """Replace Phi (host array, symmetric (3N, 3N)); geometry tables kept."""
        fcf = np.asfortranarray(fc, np.float64)
        rc = self._lib.pp_ctx_update_fc(self._h, ctypes.c_void_p(fcf.ctypes.data), self.n,
                                        PP_FLAG_ENFORCE_ASR if enforce_asr else 0, 0)
        if rc != 0:
            raise PPError(rc, "pp_ctx_update_fc")

    def update_fc_device(self, fc_ptr: int, ldfc: int, enforce_asr: bool = False) -> None:
        """Replace Phi from device memory (column-major float64, ld ldfc)."""
        rc = self._lib.pp_ctx_update_fc(self._h, ctypes.c_void_p(int(fc_ptr)), int(ldfc),
                                        PP_FLAG_ENFORCE_ASR if enforce_asr else 0, 1)
        if rc != 0:
            raise PPError(rc, "pp_ctx_update_fc")

    def close(self):
        if getattr(self, "_h", None):
            self._lib.pp_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def dynamical_matrix(self, q, derivative: int = 0, vel_method: str = "A") -> np.ndarray:
        """create_dynamical_matrix(q, derivative) (dynamical_matrix.F90:49-191)."""
        n = self.n
        out = np.zeros(2 * n * n)
        qq = np.ascontiguousarray(q, np.float64)
        rc = self._lib.pp_dynamical_matrix(self._h, _p(qq), int(derivative), vel_method.encode()[:1], _p(out), n)
        if rc != 0:
            raise PPError(rc, "pp_dynamical_matrix")
        return out.view(np.complex128).reshape(n, n, order="F")

    def solve(self, q, opts: EigOpts | None = None, want_z: bool = True) -> Result:
        """Solve a list of q-points (shape (nq,3), reduced coordinates)."""
        opts = opts or EigOpts()
        q = np.atleast_2d(np.asarray(q, np.float64))
        nq = q.shape[0]
        n = self.n
        qf = np.asfortranarray(q)
        m = np.zeros(nq, np.int64)
        nz = np.zeros(nq, np.int64)
        info = np.zeros(nq, np.int64)
        w = np.zeros((nq, n))
        vecs = opts.jobz == "V" or opts.vel
        # eigenvector columns per q: all of them, or the index range
        mz = int(opts.iu - opts.il + 1) if opts.range == "I" else n
        z = np.zeros((nq, mz, n), np.complex128) if (vecs and want_z) else None
        vel = np.zeros((nq, n, 3)) if opts.vel else None
        zv = z.view(np.float64) if z is not None else None
        errs = [np.zeros((nq, n)) for _ in range(3)] if opts.want_resid else [None] * 3
        rv = PPResultView(m.ctypes.data_as(_ip), nz.ctypes.data_as(_ip), _p(w), n,
                          _p(zv) if zv is not None else None, n, 2 * n * mz,
                          _p(vel) if vel is not None else None, 3 * n,
                          *[_p(e) if e is not None else None for e in errs])
        oc = opts.to_c()
        rc = self._lib.pp_solve_batch(self._h, qf.ctypes.data_as(_dp), nq, nq, ctypes.byref(oc), ctypes.byref(rv),
                                      info.ctypes.data_as(_ip))
        if rc != 0:
            raise PPError(rc, "pp_solve_batch")
        if z is not None:
            # per q the buffer holds z[2*(r + n*j)] (column-major) -> numpy (r, j)
            z = np.ascontiguousarray(z.transpose(0, 2, 1))
        return Result(m=m, nz=nz, w=w, z=z, vel=vel, info=info, resid=errs[0], werr=errs[1], zerr=errs[2])

    def solve_device(self, q_dev, opts: EigOpts, w_dev, m_dev, nz_dev, info_dev, vel_dev=None, z_dev=None,
                     stream: int = 0, resid_dev=None, werr_dev=None, zerr_dev=None) -> None:
        """pp_solve_batch_device: q_dev (nq,3) float64 device tensor in Fortran
        order (q[t + nq*k]); outputs are device tensors sized like
        `Result`'s fields (w_dev (nq,n), vel_dev (nq,n,3), z_dev (nq,n,n)
        complex128, m/nz/info (nq,) int64, the error estimates (nq,n)).
        Enqueued on `stream`."""
        n = self.n
        nq = int(m_dev.shape[0])

        def ptr(t):
            return ctypes.cast(t.data_ptr(), _dp) if t is not None else None
        rv = PPResultView(ctypes.cast(m_dev.data_ptr(), _ip), ctypes.cast(nz_dev.data_ptr(), _ip),
                          ctypes.cast(w_dev.data_ptr(), _dp), n, ptr(z_dev), n, 2 * n * n, ptr(vel_dev), 3 * n,
                          ptr(resid_dev), ptr(werr_dev), ptr(zerr_dev))
        oc = opts.to_c()
        rc = self._lib.pp_solve_batch_device(self._h, ctypes.c_void_p(q_dev.data_ptr()), nq, nq, ctypes.byref(oc),
                                             ctypes.byref(rv), ctypes.c_void_p(info_dev.data_ptr()),
                                             ctypes.c_void_p(int(stream)))
        if rc != 0:
            raise PPError(rc, "pp_solve_batch_device")


def solve_multi(contexts, cell, q, opts: EigOpts | None = None, want_z: bool = True) -> Result:
    """pp_solve_multi: q-points of several cells (`cell[t]` indexes
    `contexts`) solved in shared batches of mixed matrix orders.  Arrays are
    sized for the largest cell (n_max); entries beyond a cell's own 3N are
    unset."""
    opts = opts or EigOpts()
    L = load()
    q = np.atleast_2d(np.asarray(q, np.float64))
    nq = q.shape[0]
    cell = np.ascontiguousarray(cell, np.int64)
    nmax = max(c.n for c in contexts)
    qf = np.asfortranarray(q)
    m = np.zeros(nq, np.int64)
    nz = np.zeros(nq, np.int64)
    info = np.zeros(nq, np.int64)
    w = np.zeros((nq, nmax))
    vecs = opts.jobz == "V" or opts.vel
    z = np.zeros((nq, nmax, nmax), np.complex128) if (vecs and want_z) else None
    vel = np.zeros((nq, nmax, 3)) if opts.vel else None
    zv = z.view(np.float64) if z is not None else None
    errs = [np.zeros((nq, nmax)) for _ in range(3)] if opts.want_resid else [None] * 3
    rv = PPResultView(m.ctypes.data_as(_ip), nz.ctypes.data_as(_ip), _p(w), nmax,
                      _p(zv) if zv is not None else None, nmax, 2 * nmax * nmax,
                      _p(vel) if vel is not None else None, 3 * nmax,
                      *[_p(e) if e is not None else None for e in errs])
    handles = (ctypes.c_void_p * len(contexts))(*[c._h.value for c in contexts])
    oc = opts.to_c()
    rc = L.pp_solve_multi(handles, len(contexts), cell.ctypes.data_as(_ip), qf.ctypes.data_as(_dp), nq, nq,
                          ctypes.byref(oc), ctypes.byref(rv), info.ctypes.data_as(_ip))
    if rc != 0:
        raise PPError(rc, "pp_solve_multi")
    if z is not None:
        z = np.ascontiguousarray(z.transpose(0, 2, 1))
    return Result(m=m, nz=nz, w=w, z=z, vel=vel, info=info, resid=errs[0], werr=errs[1], zerr=errs[2])


def heevx_values_noalloc(a_ptr: int, lda: int, n: int, w_ptr: int, m_ptr: int, info_ptr: int, range: str = "A",
                         vl: float = 0.0, vu: float = 0.0, il: int = 1, iu: int = 1,
                         abstol: float = float(np.float32(1e-15)), stream: int = 0) -> int:
    """pp_heevx_values_noalloc on device pointers; returns the C return code.

    For callers that cannot allocate device memory: the library allocates
    nothing during the call (its scratch is a fixed array compiled into it,
    n <= PP_NOALLOC_MAX_N).  The matrix at a_ptr (complex128, column-major,
    upper triangle read) is overwritten."""
    L = load()
    return int(L.pp_heevx_values_noalloc(ctypes.c_void_p(a_ptr), int(lda), int(n), range.encode()[:1], float(vl),
                                         float(vu), int(il), int(iu), float(abstol), ctypes.c_void_p(w_ptr),
                                         ctypes.c_void_p(m_ptr), ctypes.c_void_p(info_ptr),
                                         ctypes.c_void_p(int(stream))))


def kernel_timer(names: str) -> None:
    """Record CUDA events around every launch of the named kernel classes
    (comma separated: hemv, her2k, vhx, applyV, invit, bisect, assemble, vel);
    empty string disables."""
    load().pp_ktimer_enable(names.encode())


def kernel_timer_report() -> dict:
    """{kernel class: (launches, total milliseconds)} since the last enable."""
    L = load()
    buf = ctypes.create_string_buffer(4096)
    L.pp_ktimer_report(buf, 4096)
    out = {}
    for line in buf.value.decode().splitlines():
        k, n, ms = line.split()
        out[k] = (int(n), float(ms))
    return out


def debug_stall_tc_wait(matrix: int, cycles: int) -> None:
    """Test hook: make the next tensor-core trailing update of batch matrix
    `matrix` give up its first wait after `cycles` SM clocks (-1 disarms)."""
    rc = load().pp_debug_stall_tc_wait(int(matrix), int(cycles))
    if rc != 0:
        raise PPError(rc, "pp_debug_stall_tc_wait")


def autotune_report() -> list:
    """The autotuner's choices so far, one string per tuned combination."""
    L = load()
    buf = ctypes.create_string_buffer(8192)
    L.pp_autotune_report(buf, 8192)
    return [x for x in buf.value.decode().splitlines() if x]


def kernel_launches() -> int:
    return int(load().pp_kernel_launches())
