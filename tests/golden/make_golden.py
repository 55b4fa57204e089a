"""Generate the committed golden fixtures from the reference's example data.

Run with the root of a qtm-iisc/PARPHOM checkout as the one required argument:

    python tests/golden/make_golden.py REF

Inputs (all from qtm-iisc/PARPHOM):
  Force_Constant_Generation/Examples/tblg_21.8/FORCE_CONSTANTS  (HDF5, (28,28,3,3) f64)
  Phonon_Calculations/Examples/tblg_21.8/lammps.dat              (molecular style)
  Phonon_Calculations/Examples/tblg_21.8/q_pt_symm.dat           (3 K-equivalent q)
  Phonon_Calculations/Examples/tblg_21.8/q_points_band.dat       (300 q)
  Phonon_Calculations/Examples/tblg_21.8/reference_band_eigvals.txt (h5dump of the
                                                                  shipped band file)
Outputs:
  tests/golden/tblg21_8_inputs.npz   geometry, Phi (3N x 3N), q sets
  tests/golden/tblg21_8_bands_h5dump.npz  the shipped band eigenvalues (300 x 84),
                                     a format/structure pin only: they were not
                                     produced from the shipped FORCE_CONSTANTS
  tests/golden/tblg21_8_oracle.npz   oracle outputs (w_cm, velocities) at the
                                     K-equivalent points and Gamma
  tests/golden/inputs/*              the example input files (inp*.dat, inp.dos*)
                                     of Phonon_Calculations/Examples, copied
                                     unchanged, for the input-parser tests
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from parphom_gb300 import inputs, synth  # noqa: E402
from parphom_gb300 import hdf5 as h5  # noqa: E402
from oracle import oracle as O  # noqa: E402


def parse_h5dump_eigs(path):
    txt = open(path).read()
    groups = re.findall(r'GROUP "(\d{12})" \{(.*?)\n      \}\n   \}', txt, re.S)
    out = {}
    for name, body in re.findall(r'GROUP "(\d{12})" \{(.*?)DATASET "q_vec"', txt, re.S):
        m = re.search(r'DATASET "eigenvalues".*?DATA \{(.*?)\}', body, re.S)
        vals = re.sub(r"\(\d+\):", " ", m.group(1)).replace(",", " ").split()
        out[int(name)] = np.array([float(v) for v in vals])
    del groups
    return out


# example input files copied for the parser tests: (example dir, file name)
EXAMPLE_INPUTS = [("tblg_21.8", "inp.dat"), ("tblg_21.8", "inp.dos"), ("tblg_21.8", "inp.dos_tersoff"),
                  ("tblg_21.8", "inp_symm.dat"), ("tbmos2_38.2", "inp.dat"), ("tbmos2_38.2", "inp_dos.dat"),
                  ("tbwse2_21.8", "inp.dat"), ("tbwse2_21.8", "inp.dos")]


def copy_example_inputs(ref):
    out = os.path.join(HERE, "inputs")
    os.makedirs(out, exist_ok=True)
    for d, f in EXAMPLE_INPUTS:
        src = os.path.join(ref, "Phonon_Calculations/Examples", d, f)
        with open(src, "rb") as fi, open(os.path.join(out, f"{d}__{f}"), "wb") as fo:
            fo.write(fi.read())


def main(ref):
    copy_example_inputs(ref)
    ex = os.path.join(ref, "Phonon_Calculations/Examples/tblg_21.8")
    fcf = os.path.join(ref, "Force_Constant_Generation/Examples/tblg_21.8/FORCE_CONSTANTS")
    dset = h5.read_dataset(fcf, "force_constants")
    assert dset.shape == (28, 28, 3, 3)
    phi = synth.dataset_to_phi(dset)
    ld = inputs.read_lammps_data(os.path.join(ex, "lammps.dat"), 28, 1, "molecular")
    q_symm = inputs.read_q_file(os.path.join(ex, "q_pt_symm.dat"), 3)
    q_band = inputs.read_q_file(os.path.join(ex, "q_points_band.dat"), 300)
    np.savez_compressed(os.path.join(HERE, "tblg21_8_inputs.npz"), lat=ld.lat, real_pos=ld.real_pos,
                        masses=ld.masses, at_types=ld.at_types, phi=phi, q_symm=q_symm, q_band=q_band)
    eig = parse_h5dump_eigs(os.path.join(ex, "reference_band_eigvals.txt"))
    keys = sorted(eig)
    arr = np.stack([eig[k] for k in keys])
    bf = h5.File(os.path.join(ex, "phbands_21.8.hdf5"))
    names = bf.keys()
    full = np.stack([bf[g + "/eigenvalues"] for g in names])
    qv = np.stack([bf[g + "/q_vec"] for g in names])
    np.savez_compressed(os.path.join(HERE, "tblg21_8_bands_h5dump.npz"), groups=np.array(keys), eigenvalues=arr,
                        hdf5_groups=np.array(names), hdf5_eigenvalues=full, hdf5_q_vec=qv)
    S = O.System(ld.lat, ld.real_pos, ld.masses, ld.at_types, phi)
    qs = np.vstack([q_symm, np.zeros((1, 3))])
    res = [O.solve_q(S, q, vel=True, vel_method="A") for q in qs]
    np.savez_compressed(os.path.join(HERE, "tblg21_8_oracle.npz"), q=qs,
                        w_cm=np.stack([r["w_cm"] for r in res]), vel=np.stack([r["vel"] for r in res]))
    print("wrote fixtures;", arr.shape, "band groups")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <root of a qtm-iisc/PARPHOM checkout>")
    main(sys.argv[1])
