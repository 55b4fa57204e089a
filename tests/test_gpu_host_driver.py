"""parphom_gpu.x end to end on the GPU: the same run as the Python driver
(shipped 28-atom cell), compared dataset by dataset."""
import os
import subprocess

import numpy as np
import pytest

from parphom_gb300 import build, driver, hdf5, inputs, synth
from tests.test_gpu_driver import INP

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("evec", ["yes", "no"])
def test_host_driver_matches_python_driver(tmp_path, golden_dir, evec):
    exe = build.build_host()
    z = np.load(os.path.join(golden_dir, "tblg21_8_inputs.npz"))
    for d in ("py", "cc"):
        p = tmp_path / d
        p.mkdir()
        inputs.write_lammps_data(str(p / "cell.dat"), z["lat"], z["masses"], z["at_types"], z["real_pos"])
        hdf5.write_file(str(p / "FORCE_CONSTANTS"), {"force_constants": synth.phi_to_dataset(z["phi"])})
        qs = np.vstack([z["q_symm"], [[0.1, 0.05, 0.0]]])
        np.savetxt(p / "q.dat", qs, fmt="%+.10f")
        (p / "inp.dat").write_text(INP.format(evec=evec))
    out_py = driver.run(str(tmp_path / "py" / "inp.dat"), precision="mixed")
    r = subprocess.run([exe, str(tmp_path / "cc" / "inp.dat"), "--precision", "mixed"], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    out_cc = r.stdout.strip().splitlines()[-1]
    assert out_cc.endswith("phbands.hdf5")
    f, g = hdf5.File(out_cc), hdf5.File(out_py)
    assert f.keys() == g.keys() == [f"{t:012d}" for t in range(1, 5)]
    for grp in f.keys():
        assert f.keys(grp) == g.keys(grp)
        for k in f.keys(grp):
            a, b = f[f"{grp}/{k}"], g[f"{grp}/{k}"]
            if a.dtype.names:
                np.testing.assert_array_equal(a["r"], b["r"])
                np.testing.assert_array_equal(a["i"], b["i"])
            else:
                np.testing.assert_array_equal(a, b)
