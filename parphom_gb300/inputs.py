"""Readers for the reference's input formats, with the reference's semantics.

* `read_input`  — the `key : value` file of Phonon_Calculations/SRC/read_input.F90
  (parser :90-250, defaults :368-404, sanitising :415-517).
* `read_lammps_data` — LAMMPS data file, atomic/molecular/full styles
  (lammps_read.F90:28-243): five header lines skipped, box bounds, tilt
  factors, masses, atoms.
* `read_q_file` — `nqpt` lines of reduced coordinates, extra columns ignored
  (q_read.F90:41-131).

These only parse; geometry derived from the data (crys, rec_lat) is computed
by `geometry.prepare` exactly as lammps_read.F90 does.
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np

_YES = ("yes", "true", "Yes", "True", "YES", "TRUE")
_NO = ("no", "false", "No", "False", "NO", "FALSE")


@dataclasses.dataclass
class InputConfig:
    lammps_location: str = "./"
    lammps_name: str = "lammps.dat"
    atom_style: str = "A"
    atom_types: int = 1
    natom: int = 1
    q_location: str = "./"
    q_name: str = "q_file.dat"
    nqpt: int = 1
    fc_location: str = "./"
    fc_name: str = "FC_hdf5"
    fc_dataset: str = "force_constants"
    num_qpools: int = 1
    compute_eigvecs: bool = False
    comp_evec: str = "N"
    group_velocity: bool = False
    velocity_method: str = "A"
    range_: str = "A"
    vl: float = 0.0
    vu: float = 0.0
    il: int = 1
    iu: int = 1
    abstol: float = float(np.float32(1e-15))
    orfac: float = float(np.float32(1e-15))
    mb: int = -1
    nb: int = -1
    output_name: str = "results"
    output_location: str = "./"
    print_progress: bool = True
    warnings: list = dataclasses.field(default_factory=list)


class InputError(ValueError):
    """Raised where the reference prints an error and calls `exit`."""


def _fortran_real(s: str) -> float:
    return float(s.strip().split()[0].replace("d", "e").replace("D", "e"))


def _fortran_int(s: str) -> int:
    return int(s.strip().split()[0])


def parse_input(text: str, nprocs: int = 1, check_output_exists: bool = True) -> InputConfig:
    cfg = InputConfig()
    for raw in text.splitlines():
        data = raw.strip()
        if not data or data[0] in "#! ":
            continue
        for c in "!#":
            pos = data.find(c)
            if pos >= 0:
                data = data[:pos]
        pos = data.find(":")
        if pos >= 0:
            key, val = data[:pos].upper().strip(), data[pos + 1:].strip()
        else:   # index() == 0: empty key, the whole line as value
            key, val = "", data.strip()
        if key in ("LAMMPS FILE LOCATION", "LAMMPS_FILE_LOCATION"):
            cfg.lammps_location = val
        elif key in ("LAMMPS_FILE_NAME", "LAMMPS FILE NAME"):
            cfg.lammps_name = val
        elif key == "NATOM":
            cfg.natom = _fortran_int(val)
        elif key in ("ATOM_STYLE", "ATOM STYLE"):
            cfg.atom_style = val
        elif key in ("ATOM_TYPES", "ATOM TYPES"):
            cfg.atom_types = _fortran_int(val)
        elif key in ("FORCE CONSTANT FILE LOCATION", "FORCE_CONSTANT_FILE_LOCATION"):
            cfg.fc_location = val
        elif key in ("FORCE CONSTANT FILE NAME", "FORCE_CONSTANT_FILE_NAME"):
            cfg.fc_name = val
        elif key in ("FORCE CONSTANT DATASET", "FORCE_CONSTANT_DATASET"):
            cfg.fc_dataset = val
        elif key in ("Q_FILE_LOCATION", "Q FILE LOCATION"):
            cfg.q_location = val
        elif key in ("Q_FILE_NAME", "Q FILE NAME"):
            cfg.q_name = val
        elif key == "NQPT":
            cfg.nqpt = _fortran_int(val)
        elif key in ("NUM_QPOOLS", "NUM QPOOLS"):
            # only read by builds with -D__QPOOL; otherwise "not recognised"
            cfg.warnings.append(f"Command {key} not recognised")
        elif key in ("COMPUTE_EIGVECS", "COMPUTE EIGVECS"):
            if val in _YES:
                cfg.comp_evec, cfg.compute_eigvecs = "V", True
            else:
                if val not in _NO:
                    cfg.warnings.append(f"Could not interpret command {val}; eigenvectors will not be computed.")
                cfg.comp_evec, cfg.compute_eigvecs = "N", False
        elif key in ("GROUP VELOCITY", "GROUP_VELOCITY"):
            if val in _YES:
                cfg.group_velocity = True
            else:
                if val not in _NO:
                    cfg.warnings.append(f"Could not interpret command {val}; velocity will not be computed.")
                cfg.group_velocity = False
        elif key in ("VELOCITY METHOD", "VELOCITY_METHOD"):
            if val in ("cd", "CD", "central_difference", "CENTRAL_DIFFERENCE"):
                cfg.velocity_method = "C"
            else:
                if val not in ("A", "a", "Analytic", "analytic"):
                    cfg.warnings.append(f"Could not interpret command {val}; analytic derivative used.")
                cfg.velocity_method = "A"
        elif key == "RANGE":
            if val in ("A", "V", "I"):
                cfg.range_ = val
            else:   # read_input.F90:202-206: message composed, range left unchanged
                cfg.warnings.append(f"Could not interpret command{val}")
        elif key in ("MAX_EIGVAL", "MAX EIGVAL"):
            cfg.vu = _fortran_real(val)
        elif key in ("MIN_EIGVAL", "MIN EIGVAL"):
            cfg.vl = _fortran_real(val)
        elif key in ("MAX_INDEX", "MAX INDEX"):
            cfg.iu = _fortran_int(val)
        elif key in ("MIN_INDEX", "MIN INDEX"):
            cfg.il = _fortran_int(val)
        elif key == "ABSTOL":
            cfg.abstol = _fortran_real(val)
        elif key == "ORFAC":
            cfg.orfac = _fortran_real(val)
        elif key == "MB":
            cfg.mb = _fortran_int(val)
        elif key == "NB":
            cfg.nb = _fortran_int(val)
        elif key in ("OUTPUT FILE NAME", "OUTPUT_FILE_NAME"):
            cfg.output_name = val
        elif key in ("OUTPUT FILE LOCATION", "OUTPUT_FILE_LOCATION"):
            cfg.output_location = val
        elif key in ("PRINT PROGRESS", "PRINT_PROGRESS"):
            if val in _YES:
                cfg.print_progress = True
            elif val in _NO:
                cfg.print_progress = False
            else:
                cfg.warnings.append(f"Could not interpret command {val}; progress will be printed.")
                cfg.print_progress = True
        else:
            cfg.warnings.append(f"Command {key} not recognised")
    sanitize(cfg, nprocs, check_output_exists)
    return cfg


def sanitize(cfg: InputConfig, nprocs: int = 1, check_output_exists: bool = True) -> None:
    """read_input.F90:415-517."""
    for attr in ("lammps_location", "q_location", "output_location", "fc_location"):
        v = getattr(cfg, attr)
        if not v.endswith("/"):
            setattr(cfg, attr, v + "/")
    if cfg.mb == -1:
        cfg.mb = min(32, cfg.natom) // nprocs + 1
    if cfg.nb == -1:
        cfg.nb = min(32, cfg.natom) // nprocs + 1
    if cfg.range_ == "V":
        cfg.il, cfg.iu = 1, cfg.natom
    elif cfg.range_ == "I":
        cfg.vl, cfg.vu = 0.0, 0.0
    elif cfg.range_ == "A":
        cfg.il, cfg.iu, cfg.vl, cfg.vu = 1, cfg.natom, 0.0, 0.0
    if cfg.range_ == "I" and cfg.il > cfg.iu:
        raise InputError("Invalid input for eigenvalue indices to be computed")
    if cfg.range_ == "V" and cfg.vl > cfg.vu:
        raise InputError("Invalid input for the interval in which eigenvalue is to be computed")
    if cfg.group_velocity:
        cfg.comp_evec = "V"
    full = os.path.join(cfg.output_location, cfg.output_name + ".hdf5")
    if check_output_exists and os.path.exists(full):
        k = 0
        while True:
            k += 1
            name = f"{cfg.output_name}_v{k}"
            if not os.path.exists(os.path.join(cfg.output_location, name + ".hdf5")):
                break
        cfg.output_name = name + ".hdf5"
    else:
        cfg.output_name = cfg.output_name + ".hdf5"


def read_input(path: str, nprocs: int = 1) -> InputConfig:
    with open(path) as f:
        return parse_input(f.read(), nprocs)


@dataclasses.dataclass
class LammpsData:
    lat: np.ndarray        # (3,3) rows a_i
    masses: np.ndarray     # (ntypes,)
    at_types: np.ndarray   # (natom,) 1-based
    real_pos: np.ndarray   # (natom,3)
    image: np.ndarray      # (natom,3) image flags (read, unused as in the reference)


def read_lammps_data(path: str, natom: int, ntypes: int, atom_style: str) -> LammpsData:
    with open(path) as f:
        lines = f.read().splitlines()
    it = iter(lines)
    for _ in range(5):
        next(it)

    def nums(line, k):   # list-directed READ of k values
        return [float(x) for x in line.split()[:k]]
    x1, x2 = nums(next(it), 2)
    y1, y2 = nums(next(it), 2)
    z1, z2 = nums(next(it), 2)
    xy, xz, yz = nums(next(it), 3)
    lat = np.array([[x2 - x1, 0, 0], [xy, y2 - y1, 0], [xz, yz, z2 - z1]], np.float64)
    for _ in range(3):
        next(it)
    masses = np.zeros(ntypes)
    for i in range(ntypes):
        p = next(it).split()
        masses[i] = float(p[1])
    for _ in range(3):
        next(it)
    types = np.zeros(natom, np.int64)
    pos = np.zeros((natom, 3))
    img = np.zeros((natom, 3))
    style = atom_style
    for i in range(natom):
        p = next(it).split()
        if style in ("atomic", "Atomic", "ATOMIC"):
            types[i] = int(p[1])
            pos[i] = [float(v) for v in p[2:5]]
            img[i] = [float(v) for v in p[5:8]]
        elif style in ("molecular", "Molecular", "MOLECULAR"):
            types[i] = int(p[2])
            pos[i] = [float(v) for v in p[3:6]]
            img[i] = [float(v) for v in p[6:9]]
        elif style in ("full", "Full", "FULL"):
            types[i] = int(p[2])
            pos[i] = [float(v) for v in p[4:7]]
            img[i] = [float(v) for v in p[7:10]]
        else:
            raise InputError("Atom style not supported. Supported styles are atomic and molecular")
    return LammpsData(lat=lat, masses=masses, at_types=types, real_pos=pos, image=img)


def read_q_file(path: str, nqpt: int) -> np.ndarray:
    q = np.zeros((nqpt, 3))
    with open(path) as f:
        for i in range(nqpt):
            p = f.readline().split()
            q[i] = [float(v) for v in p[:3]]
    return q


def write_lammps_data(path: str, lat: np.ndarray, masses, at_types, real_pos) -> None:
    """Atomic-style data file readable by `read_lammps_data` and by the
    reference's reader (lammps_read.F90:66-133)."""
    natom = len(at_types)
    with open(path, "w") as f:
        f.write("LAMMPS data file (synthetic)\n\n")
        f.write(f"{natom} atoms\n{len(masses)} atom types\n\n")
        f.write(f"0.0 {lat[0, 0]:.16e} xlo xhi\n")
        f.write(f"0.0 {lat[1, 1]:.16e} ylo yhi\n")
        f.write(f"0.0 {lat[2, 2]:.16e} zlo zhi\n")
        f.write(f"{lat[1, 0]:.16e} {lat[2, 0]:.16e} {lat[2, 1]:.16e} xy xz yz\n\nMasses\n\n")
        for i, m in enumerate(masses):
            f.write(f"{i + 1} {m}\n")
        f.write("\nAtoms # atomic\n\n")
        for i in range(natom):
            x = real_pos[i]
            f.write(f"{i + 1} {int(at_types[i])} {x[0]:.16e} {x[1]:.16e} {x[2]:.16e} 0 0 0\n")
