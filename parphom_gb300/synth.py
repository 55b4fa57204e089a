"""Synthetic commensurate twisted-bilayer-graphene cells, spring-model force
constants and q-point sets.

The reference computes force constants with LAMMPS finite differences
(Force_Constant_Generation/get_force_constant.py:227-295); LAMMPS is not part
of this package, so the benchmark and test cells are built here from a seeded
spring model with the same data contract the reference's driver consumes:

* geometry in the LAMMPS data-file convention read by
  Phonon_Calculations/SRC/lammps_read.F90:66-83 (lattice rows
  a1=(xhi-xlo,0,0), a2=(xy,yhi-ylo,0), a3=(xz,yz,zhi-zlo)), one atom type
  (carbon, 12.011 amu);
* force constants as the real, symmetric 3N x 3N matrix Phi whose element
  (3I+a, 3J+b) (0-based) is the HDF5 dataset entry dset[J, I, b, a]
  (force_read.F90:115-137, 223-252), acoustic sum rule enforced.

Commensurate cells follow the (m, r=1) family: N = 4(3m^2+3m+1) atoms and
cos(theta) = (3m^2+3m+1/2)/(3m^2+3m+1); m = 3, 5, 8, 11, 30 give
N = 148, 364, 868, 1588, 11164 at 9.43, 6.01, 3.89, 2.88, 1.08 degrees.

Spring model (per bond, each periodic image counted): the 3x3 coupling
K = k * (r r^T) + t * k * (1 - r r^T) with r the unit bond vector and a
transverse fraction t = 0.1, so every branch has a restoring force.
Intralayer shells 1/2/3 use k = 25/4/1.5 eV/A^2; interlayer bonds shorter
than 5 A use k = 0.25 * exp(-(d - 3.35)/0.6) eV/A^2.  Each bond constant is
multiplied by (1 + noise * g), g ~ N(0,1) from numpy's default_rng(seed).
Phi_IJ = -sum(K over bonds I-J), Phi_II = -sum_{J != I} Phi_IJ.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

A_CC = 2.46            # graphene lattice constant (A)
D_INTER = 3.35         # interlayer distance (A)
MASS_C = 12.011        # amu
INTRA_K = (25.0, 4.0, 1.5)
INTRA_SHELLS = (A_CC / math.sqrt(3.0), A_CC, 2.0 * A_CC / math.sqrt(3.0))
INTER_K0 = 0.25
INTER_DECAY = 0.6
INTER_CUTOFF = 5.0
TRANSVERSE = 0.1

TWIST_M = {148: 3, 364: 5, 868: 8, 1588: 11, 11164: 30}


@dataclasses.dataclass
class Cell:
    """A periodic cell in the reference driver's conventions (0-based arrays)."""
    natom: int
    lat: np.ndarray        # (3,3), row i = lattice vector a_i (Fortran moire%lat)
    real_pos: np.ndarray   # (natom,3) Cartesian positions (A)
    at_types: np.ndarray   # (natom,) 1-based type index
    masses: np.ndarray     # (ntypes,) amu
    layer: np.ndarray      # (natom,) 0/1
    theta_deg: float = 0.0
    m: int = 0

    @property
    def n(self) -> int:
        return 3 * self.natom


def twist_angle(m: int) -> float:
    c = (3 * m * m + 3 * m + 0.5) / (3 * m * m + 3 * m + 1)
    return math.degrees(math.acos(c))


def _layer_sites(p1, p2, basis, t1, t2, nrange):
    """Lattice sites n1 p1 + n2 p2 + basis inside the parallelogram (t1, t2)."""
    tinv = np.linalg.inv(np.array([t1, t2]).T)
    n1, n2 = np.meshgrid(np.arange(-nrange, nrange + 1), np.arange(-nrange, nrange + 1), indexing="ij")
    pts = []
    for b in basis:
        r = n1[..., None] * p1 + n2[..., None] * p2 + b
        r = r.reshape(-1, 2)
        f = r @ tinv.T
        eps = 1e-9
        keep = np.all((f >= -eps) & (f < 1.0 - eps), axis=1)
        pts.append(r[keep])
    return np.concatenate(pts, axis=0)


def tblg_cell(m: int, vacuum: float = 20.0) -> Cell:
    """Commensurate twisted bilayer graphene with twist index m (r = 1)."""
    a1 = A_CC * np.array([1.0, 0.0])
    a2 = A_CC * np.array([0.5, math.sqrt(3.0) / 2.0])
    t1 = m * a1 + (m + 1) * a2
    t2 = -(m + 1) * a1 + (2 * m + 1) * a2
    # layer 2 is layer 1 rotated by theta about the origin: the same supercell
    # vectors are (m+1) a1' + m a2' and -m a1' + (2m+1) a2' in its own lattice.
    u1 = (m + 1) * a1 + m * a2
    theta = math.atan2(t1[1], t1[0]) - math.atan2(u1[1], u1[0])
    rot = np.array([[math.cos(theta), -math.sin(theta)], [math.sin(theta), math.cos(theta)]])
    b1, b2 = rot @ a1, rot @ a2
    chk = -m * b1 + (2 * m + 1) * b2
    assert np.allclose(chk, t2, atol=1e-9), "commensurate construction failed"
    nr = 3 * m + 4
    l1 = _layer_sites(a1, a2, [np.zeros(2), (a1 + a2) / 3.0], t1, t2, nr)
    # AB registry at theta = 0: layer 2 shifted by one bond inside its own lattice
    shift = (b1 + b2) / 3.0
    l2 = _layer_sites(b1, b2, [shift, shift + (b1 + b2) / 3.0], t1, t2, nr)
    nexp = 2 * (3 * m * m + 3 * m + 1)
    assert len(l1) == nexp and len(l2) == nexp, (len(l1), len(l2), nexp)
    # rotate so that t1 lies along x (LAMMPS restricted triclinic box)
    phi = math.atan2(t1[1], t1[0])
    rz = np.array([[math.cos(-phi), -math.sin(-phi)], [math.sin(-phi), math.cos(-phi)]])
    T1, T2 = rz @ t1, rz @ t2
    L = float(np.linalg.norm(t1))
    z0 = vacuum / 2.0
    pos = np.zeros((2 * nexp, 3))
    pos[:nexp, :2] = l1 @ rz.T
    pos[nexp:, :2] = l2 @ rz.T
    pos[:nexp, 2] = z0
    pos[nexp:, 2] = z0 + D_INTER
    lat = np.array([[T1[0], 0.0, 0.0], [T2[0], T2[1], 0.0], [0.0, 0.0, D_INTER + vacuum]])
    # wrap in-plane fractional coordinates into [0, 1)
    f = pos @ np.linalg.inv(lat)
    f[:, :2] -= np.floor(f[:, :2])
    pos = f @ lat
    assert abs(lat[0, 0] - L) < 1e-9
    natom = 2 * nexp
    layer = np.concatenate([np.zeros(nexp, np.int64), np.ones(nexp, np.int64)])
    return Cell(natom=natom, lat=lat, real_pos=pos, at_types=np.ones(natom, np.int64),
                masses=np.array([MASS_C]), layer=layer, theta_deg=math.degrees(theta), m=m)


def tblg_cell_natom(natom: int) -> Cell:
    return tblg_cell(TWIST_M[natom])


def _bonds(cell: Cell, cutoff: float):
    """All (I, J, image shift (i,j), vector, distance) with 0 < d < cutoff."""
    from scipy.spatial import cKDTree
    lat = cell.lat
    pos = cell.real_pos
    shifts = [(i, j) for i in range(-2, 3) for j in range(-2, 3)]
    imgs = np.concatenate([pos + i * lat[0] + j * lat[1] for (i, j) in shifts], axis=0)
    img_id = np.repeat(np.arange(len(shifts)), cell.natom)
    tree = cKDTree(imgs)
    out_i, out_j, out_s = [], [], []
    for I, lst in enumerate(tree.query_ball_point(pos, cutoff)):
        for k in lst:
            J = k % cell.natom
            s = img_id[k]
            if J == I and shifts[s] == (0, 0):
                continue
            out_i.append(I)
            out_j.append(J)
            out_s.append(s)
    I = np.array(out_i, np.int64)
    J = np.array(out_j, np.int64)
    S = np.array(out_s, np.int64)
    sh = np.array(shifts, np.float64)[S]
    vec = pos[J] + sh[:, :1] * lat[0] + sh[:, 1:2] * lat[1] - pos[I]
    d = np.linalg.norm(vec, axis=1)
    return I, J, S, vec, d


def spring_force_constants(cell: Cell, seed: int = 0, noise: float = 0.01,
                           perturb: float = 0.0, perturb_seed: int = 1) -> np.ndarray:
    """Dense, symmetric, ASR-enforced Phi (3N x 3N, float64, eV/A^2).

    `noise` multiplies every bond constant by (1 + noise * N(0,1)) drawn from
    default_rng(seed); `perturb` additionally multiplies by
    (1 + perturb * U(-1,1)) drawn from default_rng(perturb_seed) (the
    'target' force constants of the fitting workload)."""
    N = cell.natom
    I, J, S, vec, d = _bonds(cell, INTER_CUTOFF)
    # keep each unordered bond once (I < J, or I == J with a canonical image)
    same_layer = cell.layer[I] == cell.layer[J]
    kval = np.zeros(len(d))
    for shell, k in zip(INTRA_SHELLS, INTRA_K):
        sel = same_layer & (np.abs(d - shell) < 0.12)
        kval[sel] = k
    inter = (~same_layer) & (d < INTER_CUTOFF)
    kval[inter] = INTER_K0 * np.exp(-(d[inter] - D_INTER) / INTER_DECAY)
    use = kval > 0
    I, J, S, vec, d, kval = I[use], J[use], S[use], vec[use], d[use], kval[use]
    # canonical orientation: one draw of noise per unordered bond
    key_lo = np.minimum(I, J)
    key_hi = np.maximum(I, J)
    # image index of the reversed bond is the mirrored shift
    nsh = 5
    si, sj = S // nsh - 2, S % nsh - 2
    canon_s = np.where(I <= J, S, (-si + 2) * nsh + (-sj + 2))
    keys = (key_lo * N + key_hi) * 25 + canon_s
    uniq, inv = np.unique(keys, return_inverse=True)
    rng = np.random.default_rng(seed)
    fac = 1.0 + noise * rng.standard_normal(len(uniq))
    if perturb:
        prng = np.random.default_rng(perturb_seed)
        fac = fac * (1.0 + perturb * prng.uniform(-1.0, 1.0, len(uniq)))
    kval = kval * fac[inv]
    rhat = vec / d[:, None]
    K = kval[:, None, None] * ((1.0 - TRANSVERSE) * rhat[:, :, None] * rhat[:, None, :]
                               + TRANSVERSE * np.eye(3)[None])
    # Phi is filled in its (3N x 3N) layout and symmetrised in place tile by
    # tile, so that the N = 11164 cell needs one 9 GB matrix and no copies.
    n = 3 * N
    phi = np.zeros((n, n))
    a = np.arange(3)
    rows = (3 * I)[:, None, None] + a[None, :, None]
    cols = (3 * J)[:, None, None] + a[None, None, :]
    np.add.at(phi.reshape(-1), (rows * n + cols).ravel(), -K.ravel())
    _symmetrize_inplace(phi)
    blocks = phi.reshape(N, 3, N, 3)
    idx = np.arange(N)
    blocks[idx, :, idx, :] = 0.0
    blocks[idx, :, idx, :] = -blocks.sum(axis=2)
    _symmetrize_inplace(phi)
    return phi


def _symmetrize_inplace(a: np.ndarray, tile: int = 2048) -> None:
    """a <- (a + a^T) / 2 without a second n x n array."""
    n = a.shape[0]
    for i0 in range(0, n, tile):
        i1 = min(n, i0 + tile)
        for j0 in range(i0, n, tile):
            j1 = min(n, j0 + tile)
            s = 0.5 * (a[i0:i1, j0:j1] + a[j0:j1, i0:i1].T)
            a[i0:i1, j0:j1] = s
            a[j0:j1, i0:i1] = s.T


def phi_to_dataset(phi: np.ndarray) -> np.ndarray:
    """Phi (3N x 3N) -> HDF5 dataset layout (N,N,3,3) with
    dset[J, I, b, a] = Phi[3I+a, 3J+b] (force_read.F90:223-252)."""
    n = phi.shape[0]
    N = n // 3
    return np.ascontiguousarray(phi.reshape(N, 3, N, 3).transpose(2, 0, 3, 1))


def dataset_to_phi(dset: np.ndarray) -> np.ndarray:
    N = dset.shape[0]
    return np.ascontiguousarray(dset.transpose(1, 3, 0, 2).reshape(3 * N, 3 * N))


# ---- q-point sets (reduced reciprocal coordinates) -------------------------
GAMMA = np.array([0.0, 0.0, 0.0])
K_PT = np.array([2.0 / 3.0, 1.0 / 3.0, 0.0])
M_PT = np.array([0.5, 0.0, 0.0])


def band_path(nq: int) -> np.ndarray:
    """nq points along Gamma-K-M-Gamma, spaced by Cartesian length for a
    hexagonal cell with 60-degree lattice vectors."""
    b = np.array([[1.0, -1.0 / math.sqrt(3.0)], [0.0, 2.0 / math.sqrt(3.0)]])
    nodes = [GAMMA, K_PT, M_PT, GAMMA]
    seg = [np.linalg.norm((nodes[i + 1][:2] - nodes[i][:2]) @ b) for i in range(3)]
    s = np.linspace(0.0, sum(seg), nq)
    out = np.zeros((nq, 3))
    acc = np.cumsum([0.0] + seg)
    for k, x in enumerate(s):
        i = min(int(np.searchsorted(acc, x, side="right") - 1), 2)
        t = (x - acc[i]) / seg[i]
        out[k] = nodes[i] + t * (nodes[i + 1] - nodes[i])
    return out


def uniform_grid(nk: int) -> np.ndarray:
    """Gamma-centred nk x nk grid in the kz = 0 plane."""
    i, j = np.meshgrid(np.arange(nk), np.arange(nk), indexing="ij")
    return np.stack([i.ravel() / nk, j.ravel() / nk, np.zeros(nk * nk)], axis=1)


def around_k(nq: int, radius: float = 0.02, seed: int = 2) -> np.ndarray:
    rng = np.random.default_rng(seed)
    ang = 2 * math.pi * np.arange(nq) / nq
    r = radius * (0.25 + 0.75 * rng.random(nq))
    q = np.repeat(K_PT[None], nq, axis=0)
    q[:, 0] += r * np.cos(ang)
    q[:, 1] += r * np.sin(ang)
    return q


def random_qpoints(nq: int, seed: int = 3) -> np.ndarray:
    rng = np.random.default_rng(seed)
    q = rng.uniform(-0.5, 0.5, (nq, 3))
    q[:, 2] = 0.0
    return q
