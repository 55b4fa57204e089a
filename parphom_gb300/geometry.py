"""Cell geometry as the reference driver derives it from the LAMMPS data.

* crys(I,:) = linsolve(real_pos(I,:), lat): u = (A^-1)^T x with A^-1 from
  cofactors (lammps_read.F90:198-200, 281-309);
* rec_lat = 2 pi_f (lat^-1)^T (lammps_read.F90:228, 250-274), where pi_f is
  the float-rounded value of the source literal 6.283185307179586 / 2.

Evaluation order follows the reference so that crys matches it to the last
bit on IEEE hardware without fused multiply-adds.
"""
from __future__ import annotations

import numpy as np

PI2_F = float(np.float32(6.283185307179586))


def _inv_cofactor(A: np.ndarray):
    a = lambda i, j: float(A[i - 1, j - 1])  # noqa: E731
    det = (a(1, 1) * a(2, 2) * a(3, 3) - a(1, 1) * a(2, 3) * a(3, 2)
           - a(1, 2) * a(2, 1) * a(3, 3) + a(1, 2) * a(2, 3) * a(3, 1)
           + a(1, 3) * a(2, 1) * a(3, 2) - a(1, 3) * a(2, 2) * a(3, 1))
    detinv = 1.0 / det
    B = np.zeros((3, 3))
    B[0, 0] = +detinv * (a(2, 2) * a(3, 3) - a(2, 3) * a(3, 2))
    B[1, 0] = -detinv * (a(2, 1) * a(3, 3) - a(2, 3) * a(3, 1))
    B[2, 0] = +detinv * (a(2, 1) * a(3, 2) - a(2, 2) * a(3, 1))
    B[0, 1] = -detinv * (a(1, 2) * a(3, 3) - a(1, 3) * a(3, 2))
    B[1, 1] = +detinv * (a(1, 1) * a(3, 3) - a(1, 3) * a(3, 1))
    B[2, 1] = -detinv * (a(1, 1) * a(3, 2) - a(1, 2) * a(3, 1))
    B[0, 2] = +detinv * (a(1, 2) * a(2, 3) - a(1, 3) * a(2, 2))
    B[1, 2] = -detinv * (a(1, 1) * a(2, 3) - a(1, 3) * a(2, 1))
    B[2, 2] = +detinv * (a(1, 1) * a(2, 2) - a(1, 2) * a(2, 1))
    return detinv, B


def crys_from_positions(lat: np.ndarray, real_pos: np.ndarray) -> np.ndarray:
    _, B = _inv_cofactor(np.asarray(lat, np.float64))
    x = np.asarray(real_pos, np.float64)
    # u(i) = sum_k B(k,i) x(k), summed k = 1, 2, 3 in order
    return (B[0][None, :] * x[:, 0:1] + B[1][None, :] * x[:, 1:2]) + B[2][None, :] * x[:, 2:3]


def reciprocal_lattice(lat: np.ndarray) -> np.ndarray:
    A = np.asarray(lat, np.float64)
    detinv, _ = _inv_cofactor(A)
    a = lambda i, j: float(A[i - 1, j - 1])  # noqa: E731
    B = np.zeros((3, 3))
    B[0, 0] = +detinv * (a(2, 2) * a(3, 3) - a(2, 3) * a(3, 2)) * PI2_F
    B[0, 1] = -detinv * (a(2, 1) * a(3, 3) - a(2, 3) * a(3, 1)) * PI2_F
    B[0, 2] = +detinv * (a(2, 1) * a(3, 2) - a(2, 2) * a(3, 1)) * PI2_F
    B[1, 0] = -detinv * (a(1, 2) * a(3, 3) - a(1, 3) * a(3, 2)) * PI2_F
    B[1, 1] = +detinv * (a(1, 1) * a(3, 3) - a(1, 3) * a(3, 1)) * PI2_F
    B[1, 2] = -detinv * (a(1, 1) * a(3, 2) - a(1, 2) * a(3, 1)) * PI2_F
    B[2, 0] = +detinv * (a(1, 2) * a(2, 3) - a(1, 3) * a(2, 2)) * PI2_F
    B[2, 1] = -detinv * (a(1, 1) * a(2, 3) - a(1, 3) * a(2, 1)) * PI2_F
    B[2, 2] = +detinv * (a(1, 1) * a(2, 2) - a(1, 2) * a(2, 1)) * PI2_F
    return B
