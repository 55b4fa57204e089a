"""The native host driver parphom_gpu.x (C++): input parser, LAMMPS reader,
geometry and HDF5 reader/writer against the Python mirror of the reference
driver (no GPU needed; the end-to-end run is in test_gpu_host_driver.py)."""
import dataclasses
import json
import os
import subprocess

import numpy as np
import pytest

from parphom_gb300 import build, geometry, hdf5, inputs, synth


@pytest.fixture(scope="module")
def exe():
    return build.build_host()


def run(exe, *args, cwd=None):
    r = subprocess.run([exe, *args], capture_output=True, text=True, cwd=cwd)
    assert r.returncode == 0, r.stderr
    return r.stdout


INPUTS = [
    "natom: 28\nrange: I\nmin index: 3\nmax index : 9\ncompute eigvecs: yes\ngroup velocity: maybe\n"
    "abstol: 1d-12\nfoo: bar\nvelocity method: cd\n",
    "# comment\nLAMMPS FILE NAME : cell.dat ! trailing\nnatom : 1588\natom_types: 2\nrange : V\n"
    "min eigval: 0.5\nmax eigval: 3D2\ngroup velocity: yes\nprint progress: no\noutput file name: out\n",
    "natom: 4\nrange: X\ncompute eigvecs: no\nnum qpools: 2\nmb: 8\n",
]


@pytest.mark.parametrize("text", INPUTS)
def test_parse_input_matches_python(exe, tmp_path, text):
    (tmp_path / "inp.dat").write_text(text)
    c = json.loads(run(exe, "--parse-input", str(tmp_path / "inp.dat"), cwd=tmp_path))
    p = dataclasses.asdict(inputs.read_input(str(tmp_path / "inp.dat")))
    assert c == p


def test_existing_output_is_renamed(exe, tmp_path):
    (tmp_path / "inp.dat").write_text("natom: 2\noutput file name: res\n")
    (tmp_path / "res.hdf5").write_bytes(b"")
    (tmp_path / "res_v1.hdf5").write_bytes(b"")
    c = json.loads(run(exe, "--parse-input", "inp.dat", cwd=tmp_path))
    assert c["output_name"] == "res_v2.hdf5"


@pytest.mark.parametrize("style", ["atomic", "molecular", "full"])
def test_lammps_reader_and_geometry(exe, tmp_path, style):
    cell = synth.tblg_cell(3)
    path = tmp_path / "cell.dat"
    inputs.write_lammps_data(str(path), cell.lat, cell.masses, cell.at_types, cell.real_pos)
    if style != "atomic":  # insert the molecule id (and charge for full)
        lines = path.read_text().splitlines()
        k = lines.index("Atoms # atomic") + 2
        for i in range(k, k + cell.natom):
            p = lines[i].split()
            lines[i] = " ".join([p[0], "1", p[1]] + (["0.0"] if style == "full" else []) + p[2:])
        path.write_text("\n".join(lines) + "\n")
    out = run(exe, "--read-lammps", str(path), str(cell.natom), "1", style).splitlines()
    ld = inputs.read_lammps_data(str(path), cell.natom, 1, style)
    lat = np.array([[float(x) for x in l.split()[1:]] for l in out[:3]])
    np.testing.assert_array_equal(lat, ld.lat)
    assert float(out[3].split()[1]) == ld.masses[0]
    atoms = np.array([[float(x) for x in l.split()[1:]] for l in out[4:]])
    np.testing.assert_array_equal(atoms[:, 0], ld.at_types)
    np.testing.assert_array_equal(atoms[:, 1:4], ld.real_pos)
    # crys in the reference's evaluation order, bit for bit
    np.testing.assert_array_equal(atoms[:, 4:7], geometry.crys_from_positions(ld.lat, ld.real_pos))


def test_hdf5_reader_and_writer_round_trip(exe, tmp_path):
    rng = np.random.default_rng(0)
    fc = rng.standard_normal((5, 5, 3, 3))
    ev = rng.standard_normal((4, 6)) + 1j * rng.standard_normal((4, 6))
    tree = {"force_constants": fc, "ints": np.array([1, -2, 3])}
    for t in range(1, 131):  # more members than one symbol-table node holds
        tree[f"{t:012d}"] = {"q_vec": rng.standard_normal(3), "eigenvalues": rng.standard_normal(6),
                             "evec": ev * t, "vel": rng.standard_normal((4, 3))}
    hdf5.write_file(str(tmp_path / "py.h5"), tree)
    keys = run(exe, "--h5-keys", str(tmp_path / "py.h5"), "/").split()
    assert keys == sorted(tree)
    out = run(exe, "--h5-read", str(tmp_path / "py.h5"), "force_constants").split()
    assert out[:5] == ["shape", "5", "5", "3", "3"]
    np.testing.assert_array_equal(np.array(out[5:], float), fc.ravel())
    out = run(exe, "--h5-read", str(tmp_path / "py.h5"), "000000000007/evec").split()
    np.testing.assert_array_equal(np.array(out[3:], float), np.stack([ev.real, ev.imag], -1).ravel() * 7)
    # the C++ writer's output, read back by the Python reader
    run(exe, "--h5-copy", str(tmp_path / "py.h5"), str(tmp_path / "cc.h5"))
    f, g = hdf5.File(str(tmp_path / "cc.h5")), hdf5.File(str(tmp_path / "py.h5"))
    assert f.keys() == g.keys()
    for k in ["force_constants", "ints", "000000000001/q_vec", "000000000130/vel", "000000000042/eigenvalues"]:
        np.testing.assert_array_equal(f[k], g[k])
    a, b = f["000000000099/evec"], g["000000000099/evec"]
    assert a.dtype.names == ("r", "i")
    np.testing.assert_array_equal(a["r"], b["r"])
    np.testing.assert_array_equal(a["i"], b["i"])


def test_bad_inputs_fail_with_a_message(exe, tmp_path):
    (tmp_path / "inp.dat").write_text("natom: 2\nrange: I\nmin index: 5\nmax index: 2\n")
    r = subprocess.run([exe, "--parse-input", "inp.dat"], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 1 and "Invalid input for eigenvalue indices" in r.stderr
    r = subprocess.run([exe, "--h5-read", str(tmp_path / "inp.dat"), "x"], capture_output=True, text=True)
    assert r.returncode == 1 and "not an HDF5 file" in r.stderr


# The reference's own example input files (copied unchanged by
# tests/golden/make_golden.py).  Expected fields are read off each file by
# the rules of read_input.F90: comments cut at '!' or '#' (:95-103), keys
# upper-cased with spaces or underscores (:110-245), a trailing '/' added to
# locations (:415-440), range 'A' sets il=1, iu=natom, vl=vu=0 (:457-470),
# group velocity forces comp_evec 'V' (:483-485), '.hdf5' appended to the
# output name (:487-513).
_TBLG = "../../../Force_Constant_Generation/Examples/tblg_21.8/"
_EXPECT = {
    "tblg_21.8__inp.dat": dict(natom=28, atom_types=1, atom_style="molecular", q_name="q_points_band.dat",
                               nqpt=300, fc_location=_TBLG, fc_name="FORCE_CONSTANTS", compute_eigvecs=True,
                               comp_evec="V", group_velocity=True, velocity_method="A", range_="A", il=1, iu=28,
                               vl=0.0, vu=0.0, mb=4, nb=4, abstol=1e-14, orfac=1e-14,
                               output_name="phbands_21.8.hdf5", output_location="./", print_progress=True),
    "tblg_21.8__inp.dos": dict(nqpt=27, q_name="dos_21.8_15X15.dat", compute_eigvecs=False, comp_evec="N",
                               group_velocity=False, velocity_method="A", mb=8, nb=8, abstol=1e-16,
                               output_name="phbands_21.8_dos_15X15.hdf5", output_location="./"),
    "tblg_21.8__inp.dos_tersoff": dict(lammps_location=_TBLG, lammps_name="lammps.dat_tersoff",
                                       fc_name="FORCE_CONSTANTS_TERSOFF", output_location="./",
                                       output_name="phbands_21.8_dos_15X15_tersoff.hdf5"),
    "tblg_21.8__inp_symm.dat": dict(q_name="q_pt_symm.dat", nqpt=3, velocity_method="C", group_velocity=True,
                                    comp_evec="V", output_name="phbandsymm.hdf5"),
    "tbmos2_38.2__inp.dat": dict(natom=42, atom_types=6, atom_style="atomic",
                                 lammps_location="/home/mshinjan/Phonons/MoirePhonons/Force_Constant_Generation/"
                                                 "Examples/tbmos2_38.2/",
                                 q_name="qpt_bands_KKp.dat", nqpt=201, mb=16, nb=16, iu=42, velocity_method="A",
                                 group_velocity=True),
    "tbmos2_38.2__inp_dos.dat": dict(nqpt=1802, fc_location="./", fc_name="FC_hdf5", group_velocity=False,
                                     compute_eigvecs=True, comp_evec="V", mb=32, nb=32,
                                     output_name="phdos_9.43_mos2.hdf5"),
    "tbwse2_21.8__inp.dat": dict(q_name="q_points_band.dat", nqpt=300, lammps_name="lammps.dat_final",
                                 fc_location="../../../Force_Constant_Generation/Examples/tbwse2_21.8/",
                                 velocity_method="A", group_velocity=True),
    "tbwse2_21.8__inp.dos": dict(q_name="full_grid_100X100", nqpt=10000, abstol=1e-15, orfac=1e-15,
                                 fc_location="/home/mshinjan/Twister/examples/Homobilayer_hex/WSe2/Angle_21.78/"),
}


@pytest.mark.parametrize("name", sorted(_EXPECT))
def test_reference_example_inputs(exe, golden_dir, tmp_path, name):
    """Both parsers (C++ host driver and its Python mirror) read each shipped
    example input to the values the reference's parser gives."""
    src = os.path.join(golden_dir, "inputs", name)
    dst = tmp_path / "inp.dat"
    dst.write_bytes(open(src, "rb").read())
    c = json.loads(run(exe, "--parse-input", str(dst), cwd=tmp_path))
    p = dataclasses.asdict(inputs.read_input(str(dst)))
    assert c == p
    for k, v in _EXPECT[name].items():
        assert p[k] == v, (name, k, p[k], v)
