"""ORACLE — test infrastructure only.

CPU restatement of the reference's BZ-integration routines used for the
density of states (Utilities/pyphutil/fortran_routines/bz_integration.f90):
linear_triangulation :12-48 with sort_freq :50-65 and integrate_triangle
:68-133, and standard_integration :154-179 with gaussian/lorentzian :181-199
(PI there is the single-precision literal, as in the dynamical matrix).
Plain loops over (energy, triangle, band) for the small test cases.
"""
import numpy as np

PI_F = float(np.float32(3.141592653589793))


def _integrate_triangle(a, Ef):
    dos = nd = 0.0
    if a[3][0] == Ef:
        dos, nd = 0.0, a[0][1] + a[1][1] + a[2][1]
    if a[2][0] == Ef:
        e0, f0 = a[0]
        e1, f1 = a[1]
        e2, f2 = a[3]
        del02 = (e2 - Ef) / (e2 - e0)
        del12 = (e2 - Ef) / (e2 - e1)
        ddel02 = 1 / (e0 - e2)
        ddel12 = 1 / (e1 - e2)
        nd = ((1 - del12 * del02 ** 2) * f0 + (1 - del02 * del12 ** 2) * f1
              + (1 - 3 * del12 * del02 + del12 * del02 ** 2 + del02 * del12 ** 2) * f2)
        dos = ((-2 * del02 * ddel02 * del12 - ddel12 * del02 ** 2) * f0
               + (-ddel02 * del12 ** 2 - 2 * del02 * del12 * ddel12) * f1
               + (-3 * del12 * ddel02 - 3 * del02 * ddel12 + 2 * del02 * del12 * ddel02
                  + ddel12 * del02 ** 2 + 2 * del02 * del12 * ddel12 + ddel02 * del12 ** 2) * f2)
    if a[1][0] == Ef:
        e0, f0 = a[0]
        e1, f1 = a[2]
        e2, f2 = a[3]
        del10 = (Ef - e0) / (e1 - e0)
        del20 = (Ef - e0) / (e2 - e0)
        ddel10 = 1 / (e1 - e0)
        ddel20 = 1 / (e2 - e0)
        n = (3 - del10 - del20) * f0 + del10 * f1 + del20 * f2
        dos = ddel10 * del20 * n + del10 * ddel20 * n + del10 * del20 * ((-ddel10 - ddel20) * f0 + ddel10 * f1
                                                                         + ddel20 * f2)
        nd = n * del10 * del20
    if a[0][0] == Ef:
        dos = nd = 0.0
    return dos, nd


def linear_triangulation(freq, func, tri, energy):
    """freq/func (nk, nbands); tri (ntri, 3) 0-based; returns (dos, nd)."""
    ne = len(energy)
    dos = np.zeros(ne)
    nd = np.zeros(ne)
    nb = freq.shape[1]
    for i, Ef in enumerate(energy):
        for t in tri:
            for k in range(nb):
                a = [[Ef, 0.0]] + [[freq[v, k], func[v, k]] for v in t]
                for p in range(4):
                    for r in range(p + 1, 4):
                        if a[p][0] > a[r][0]:
                            a[p], a[r] = a[r], a[p]
                d, n = _integrate_triangle(a, Ef)
                dos[i] += d
                nd[i] += n
    return dos, nd


def smearing(method, freq, weights, width, energy, natom):
    e = np.asarray(energy)[:, None, None]
    e0 = np.asarray(freq)[None]
    if method == 1:
        d = np.exp(-(((e - e0) / width) ** 2) / 2) / (np.sqrt(2 * PI_F) * width)
    else:
        d = ((width / 2) / ((e - e0) ** 2 + (width / 2) ** 2)) * (1 / PI_F)
    return (d * np.asarray(weights)[None, :, None]).sum(axis=(1, 2)) / natom
