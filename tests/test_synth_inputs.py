import numpy as np
import pytest

from parphom_gb300 import geometry, inputs, synth


@pytest.mark.parametrize("m,natom,theta", [(3, 148, 9.43), (5, 364, 6.01), (8, 868, 3.89), (11, 1588, 2.88)])
def test_commensurate_cells(m, natom, theta):
    c = synth.tblg_cell(m)
    assert c.natom == natom
    assert abs(c.theta_deg - theta) < 0.01
    f = c.real_pos @ np.linalg.inv(c.lat)
    assert f[:, :2].min() >= 0 and f[:, :2].max() < 1


def test_force_constants_properties():
    c = synth.tblg_cell(3)
    phi = synth.spring_force_constants(c, seed=0)
    assert np.array_equal(phi, phi.T)
    blocks = phi.reshape(c.natom, 3, c.natom, 3)
    assert np.abs(blocks.sum(axis=2)).max() < 1e-12     # acoustic sum rule
    phi2 = synth.spring_force_constants(c, seed=0)
    assert np.array_equal(phi, phi2)                    # seeded
    phi3 = synth.spring_force_constants(c, seed=0, perturb=0.03)
    assert 0 < np.abs(phi3 - phi).max() < 0.05 * np.abs(phi).max()
    d = synth.phi_to_dataset(phi)
    assert np.array_equal(synth.dataset_to_phi(d), phi)
    assert d[1, 0, 2, 1] == phi[3 * 0 + 1, 3 * 1 + 2]  # dset[J,I,b,a] = Phi[3I+a, 3J+b]


def test_q_sets():
    p = synth.band_path(64)
    assert p.shape == (64, 3) and np.allclose(p[0], 0) and np.allclose(p[-1], 0)
    g = synth.uniform_grid(32)
    assert g.shape == (1024, 3)


INPUT = """# test input
lammps file location         : ./data
lammps file name             : cell.dat
natom                        : 28
atom types                   : 1
atom style                   : molecular
q file name                  : q.dat   ! trailing comment
nqpt                         : 3
compute eigvecs              : yes
range                        : I
min index                    : 13
max index                    : 16
group velocity               : yes
velocity method              : cd
abstol                       : 1E-16
unknown key                  : 5
output file name             : out
"""


def test_input_parser(tmp_path):
    cfg = inputs.parse_input(INPUT, check_output_exists=False)
    assert cfg.lammps_location == "./data/"
    assert cfg.natom == 28 and cfg.atom_style == "molecular"
    assert cfg.q_name == "q.dat"
    assert cfg.range_ == "I" and (cfg.il, cfg.iu) == (13, 16) and (cfg.vl, cfg.vu) == (0.0, 0.0)
    assert cfg.comp_evec == "V" and cfg.group_velocity and cfg.velocity_method == "C"
    assert cfg.abstol == 1e-16
    assert any("not recognised" in w for w in cfg.warnings)
    assert cfg.mb == 29 and cfg.nb == 29          # min(32, natom)/nprocs + 1
    assert cfg.output_name == "out.hdf5"
    (tmp_path / "out.hdf5").write_text("x")
    cfg2 = inputs.parse_input(INPUT.replace("./data", str(tmp_path)).replace("output file name             : out",
                                                                              f"output file name : out\noutput file location : {tmp_path}"))
    assert cfg2.output_name == "out_v1.hdf5"
    with pytest.raises(inputs.InputError):
        inputs.parse_input(INPUT.replace("max index                    : 16", "max index : 2"),
                           check_output_exists=False)


def test_range_defaults():
    cfg = inputs.parse_input("natom : 10\nrange : A\nmin index : 3\n", check_output_exists=False)
    assert (cfg.il, cfg.iu) == (1, 10)
    cfg = inputs.parse_input("natom : 10\nrange : X\n", check_output_exists=False)
    assert cfg.range_ == "A"


def test_lammps_roundtrip(tmp_path):
    c = synth.tblg_cell(3)
    p = tmp_path / "cell.dat"
    inputs.write_lammps_data(str(p), c.lat, c.masses, c.at_types, c.real_pos)
    ld = inputs.read_lammps_data(str(p), c.natom, 1, "atomic")
    np.testing.assert_allclose(ld.lat, c.lat, atol=1e-12)
    np.testing.assert_allclose(ld.real_pos, c.real_pos, atol=1e-12)
    cr = geometry.crys_from_positions(ld.lat, ld.real_pos)
    np.testing.assert_allclose(cr @ ld.lat, ld.real_pos, atol=1e-10)
