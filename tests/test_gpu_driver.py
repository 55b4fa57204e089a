"""`python -m parphom_gb300 inp.dat` end to end on the GPU: the reference's
input files in, the reference's HDF5 output layout out, values against the
oracle."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from parphom_gb300 import driver, hdf5, inputs, synth
from tests import parity

pytestmark = pytest.mark.gpu

INP = """# parphom input
lammps file location         : ./
lammps file name             : cell.dat
natom                        : 28
atom types                   : 1
atom style                   : atomic
q file location              : ./
q file name                  : q.dat
nqpt                         : 4
force constant file location : ./
force constant file name     : FORCE_CONSTANTS
force constant dataset       : force_constants
compute eigvecs              : {evec}
range                        : A
group velocity               : yes
velocity method              : a
output file name             : phbands
output_file_location         : ./
print progress               : no
"""


@pytest.mark.parametrize("evec", ["yes", "no"])
def test_driver_end_to_end(tmp_path, golden_dir, evec):
    z = np.load(os.path.join(golden_dir, "tblg21_8_inputs.npz"))
    inputs.write_lammps_data(str(tmp_path / "cell.dat"), z["lat"], z["masses"], z["at_types"], z["real_pos"])
    hdf5.write_file(str(tmp_path / "FORCE_CONSTANTS"), {"force_constants": synth.phi_to_dataset(z["phi"])})
    qs = np.vstack([z["q_symm"], [[0.1, 0.05, 0.0]]])
    np.savetxt(tmp_path / "q.dat", qs, fmt="%+.10f")
    (tmp_path / "inp.dat").write_text(INP.format(evec=evec))
    out = driver.run(str(tmp_path / "inp.dat"), precision="mixed")
    assert out.endswith("phbands.hdf5")
    f = hdf5.File(out)
    assert f.keys() == [f"{t:012d}" for t in range(1, 5)]
    ld = inputs.read_lammps_data(str(tmp_path / "cell.dat"), 28, 1, "atomic")
    S = O.System(ld.lat, ld.real_pos, ld.masses, ld.at_types, z["phi"])
    refs = [O.solve_q(S, q, vel=True) for q in qs]
    vmax = max(np.abs(r["vel"]).max() for r in refs)
    for t, q in enumerate(qs):
        g = f"{t + 1:012d}"
        expect = ["eigenvalues", "q_vec", "vel"] + (["evec"] if evec == "yes" else [])
        assert sorted(f.keys(g)) == sorted(expect)
        ref = refs[t]
        np.testing.assert_array_equal(f[g + "/q_vec"], q)
        w = f[g + "/eigenvalues"]
        D = S.dynmat(q)
        parity.check_frequencies(w, ref["w_cm"], ref["lam"], 84, np.abs(ref["lam"]).max())
        v = f[g + "/vel"]
        assert v.shape == (84, 3)
        parity.check_velocities(v, ref["vel"], ref["lam"], np.abs(ref["lam"]).max(), vmax)
        if evec == "yes":
            e = f[g + "/evec"]
            Z = (e["r"] + 1j * e["i"]).T
            parity.check_vectors(Z, ref["lam"], D, 1e-11, 1e-10)
    # a second run does not overwrite: the output is renamed _v1 (read_input.F90:487-513)
    out2 = driver.run(str(tmp_path / "inp.dat"), precision="fp64", quiet=True)
    assert out2.endswith("phbands_v1.hdf5")
