"""`python -m parphom_gb300 <input file>`: the parphom.x run on one GB300.

Same inputs and outputs as the reference program (Phonon_Calculations/SRC/
main.F90:40-70): the `key : value` input file, the LAMMPS data file, the
(N,N,3,3) HDF5 force-constant dataset and the q-point file are read with the
reference's semantics; the per-q loop (calculations.F90:49-53) runs on the
GPU through the C ABI in batches; the output file gets one group per q-point
named '%012d' (global 1-based index) with `q_vec` (3,), `eigenvalues` (m,) in
cm^-1, `evec` (nz, 3N) compound {r, i} when `compute eigvecs: yes`, and `vel`
(nz, 3) in m/s when `group velocity: yes` (write_output.F90:98-143, 178-312,
377-484).  The output is written once all q-points are done.
"""
from __future__ import annotations

import argparse
import contextlib
import datetime
import os
import sys

import numpy as np

from . import api, geometry, hdf5, inputs, replicas, synth


def prepare_force_constants(dset: np.ndarray) -> np.ndarray:
    """force_read.F90:115-189: element (3I+a, 3J+b) = dset[J, I, b, a], then
    Phi <- 1/2 Phi^T + 1/2 Phi.  (The reference's pdgeadd passes the same
    array as A and C; for symmetric input, which the generator and the
    shipped files are, that is Phi itself; here the intended symmetric part
    is formed.)"""
    phi = synth.dataset_to_phi(np.asarray(dset, np.float64))
    return 0.5 * phi.T + 0.5 * phi


def _msg(cfg, text):
    if cfg.print_progress:
        now = datetime.datetime.now().strftime("%d/%m/%Y %H:%M:%S")
        print(f"{text} on {now}", flush=True)


def run(input_path: str, precision: str = "mixed", batch: int | None = None, quiet: bool = False) -> str:
    base = os.path.dirname(os.path.abspath(input_path))
    cwd = os.getcwd()
    os.chdir(base)   # relative locations in the input are relative to the run directory
    try:
        cfg = inputs.read_input(os.path.basename(input_path))
        if quiet:
            cfg.print_progress = False
        for w in cfg.warnings:
            print(w, file=sys.stderr)
        ld = inputs.read_lammps_data(cfg.lammps_location + cfg.lammps_name, cfg.natom, cfg.atom_types,
                                     cfg.atom_style)
        dset = hdf5.read_dataset(cfg.fc_location + cfg.fc_name, cfg.fc_dataset)
        if dset.shape != (cfg.natom, cfg.natom, 3, 3):
            raise inputs.InputError(f"force-constant dataset has shape {dset.shape}, expected "
                                    f"({cfg.natom},{cfg.natom},3,3)")
        phi = prepare_force_constants(dset)
        _msg(cfg, "Force constants read and symmetrized")
        q = inputs.read_q_file(cfg.q_location + cfg.q_name, cfg.nqpt)
        crys = geometry.crys_from_positions(ld.lat, ld.real_pos)
        prec = api.PP_PREC_MIXED if precision == "mixed" else api.PP_PREC_FP64
        opts = api.EigOpts(jobz=cfg.comp_evec, range=cfg.range_, vl=cfg.vl, vu=cfg.vu, il=cfg.il, iu=cfg.iu,
                           abstol=cfg.abstol, orfac=cfg.orfac, vel=cfg.group_velocity,
                           vel_method=cfg.velocity_method, precision=prec)
        out_path = cfg.output_location + cfg.output_name
        n = 3 * cfg.natom
        B = batch or max(1, min(len(q), 64))
        # one process per GPU under torchrun: rank r solves q[r::world], rank 0 writes
        world, rank, local = replicas.world_info()
        group = None
        if world > 1:
            import torch
            torch.cuda.set_device(local)
            group = replicas.init_group(world, rank)
        nmine = len(replicas.shard(len(q), rank, world))
        who = f"rank {rank}: " if world > 1 else ""
        done = [0]
        with api.PhononContext(ld.lat, crys, ld.real_pos, ld.masses, ld.at_types, phi) as ctx, \
                (hdf5.Writer(out_path) if rank == 0 else contextlib.nullcontext()) as wr:

            def solve(qb):
                res = ctx.solve(qb, opts, want_z=cfg.compute_eigvecs)
                _msg(cfg, f"{who}q-points {done[0] + 1}-{done[0] + len(qb)} of {nmine} solved (n = {n})")
                done[0] += len(qb)
                return replicas.split_result(res, len(qb))

            def write(t, r):
                if r["info"]:
                    print(f"q-point {t + 1}: eigensolver info {r['info']}", file=sys.stderr)
                ds = {"q_vec": q[t], "eigenvalues": r["w"]}
                if cfg.compute_eigvecs and "z" in r:
                    ds["evec"] = np.ascontiguousarray(r["z"].T)
                if cfg.group_velocity and "vel" in r:
                    ds["vel"] = r["vel"]
                wr.add_group(f"{t + 1:012d}", ds)

            replicas.run_sharded(q, B, solve, write if rank == 0 else None, world, rank, group)
        _msg(cfg, f"Results written to {out_path}")
        return os.path.join(base, out_path)
    finally:
        os.chdir(cwd)


def main(argv=None):
    p = argparse.ArgumentParser(prog="python -m parphom_gb300", description=__doc__.splitlines()[0])
    p.add_argument("input")
    p.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    p.add_argument("--batch", type=int, default=None)
    a = p.parse_args(argv)
    print(run(a.input, a.precision, a.batch))


if __name__ == "__main__":
    main()
