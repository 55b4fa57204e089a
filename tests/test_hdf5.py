"""HDF5 reader/writer (written from the public format specification) on the
reference's layouts: the (N,N,3,3) force-constant dataset and the per-q
output groups with q_vec, eigenvalues, compound evec {r, i} and vel."""
import os

import numpy as np

from parphom_gb300 import hdf5 as h5
from parphom_gb300 import synth


def test_output_layout_roundtrip(tmp_path):
    rng = np.random.default_rng(1)
    n, nz = 12, 7
    path = str(tmp_path / "out.hdf5")
    groups = {}
    with h5.Writer(path) as w:
        for g in range(1, 301):   # more members than one symbol-table node holds
            ds = {"q_vec": rng.random(3), "eigenvalues": rng.random(n),
                  "evec": rng.random((nz, n)) + 1j * rng.random((nz, n)), "vel": rng.random((nz, 3))}
            w.add_group(f"{g:012d}", ds)
            groups[f"{g:012d}"] = ds
    f = h5.File(path)
    assert f.keys() == sorted(groups)
    for g, ds in groups.items():
        assert f.keys(g) == ["eigenvalues", "evec", "q_vec", "vel"]
        ev = f[g + "/evec"]
        assert ev.dtype.names == ("r", "i") and ev.shape == (nz, n)
        np.testing.assert_array_equal(ev["r"] + 1j * ev["i"], ds["evec"])
        np.testing.assert_array_equal(f[g + "/vel"], ds["vel"])
        np.testing.assert_array_equal(f[g + "/eigenvalues"], ds["eigenvalues"])


def test_force_constant_file_roundtrip(tmp_path, golden_dir):
    z = np.load(os.path.join(golden_dir, "tblg21_8_inputs.npz"))
    dset = synth.phi_to_dataset(z["phi"])
    p = str(tmp_path / "FC")
    h5.write_file(p, {"force_constants": dset})
    back = h5.read_dataset(p, "force_constants")
    assert back.shape == (28, 28, 3, 3)
    np.testing.assert_array_equal(synth.dataset_to_phi(back), z["phi"])


def test_superblock_and_errors(tmp_path):
    p = tmp_path / "x.hdf5"
    h5.write_file(str(p), {"a": np.arange(5, dtype=np.int64)})
    b = p.read_bytes()
    assert b[:8] == h5.SIG and b[8] == 0
    np.testing.assert_array_equal(h5.read_dataset(str(p), "a"), np.arange(5))
    (tmp_path / "bad").write_bytes(b"not hdf5" * 20)
    import pytest
    with pytest.raises(h5.HDF5Error):
        h5.File(str(tmp_path / "bad"))
