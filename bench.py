#!/usr/bin/env python
"""Benchmark of the phonon hot path on GB300.

Workload (one "step"): a batch of q-points of the theta = 2.88 deg twisted
bilayer graphene cell (N = 1588 atoms, 3N = 4764), synthetic spring-model
force constants (seed 0), q-points on the Gamma-K-M-Gamma path (128 points,
cycled), frequencies + analytic group velocities (jobz forced to 'V' by the
velocity switch), mixed-precision form.  `value` is q-points/s with inputs
resident in HBM; `e2e` the same through the host C-ABI call (q from pinned
host memory in, frequencies and velocities back to host memory).  Every
matrix (363 MB per q in double-float complex) is larger than L2, so no L2
flush is needed between steps.

Also measured: the plain FP64 form on a batch of the same size (the
ratio the metric names), the largest frequency difference between the two
forms, per-kernel CUDA-event times for the roofline, SM clocks during the
timed region, and the CPU oracle on one q (cpu_baseline).

`--impl reference` times the reference-equivalent CPU path (the oracle:
C restatement of the D(q) assembly + LAPACK zheevx + dense dD/dq velocities)
on the host cores, one q per step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "q-pts/s (w+v_g) at N=1588: mixed/batched vs FP64 GPU at |dw|<1e-4 cm^-1"
UNIT = "q-pts/s"
WORKLOAD = "tBLG theta=2.88deg N=1588 (3N=4764), spring FC seed 0, band-path q, w + analytic v_g"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--batch", type=int, default=32, help="q-points per step and rank")
    p.add_argument("--m", type=int, default=11, help="twist index (11 -> N=1588)")
    p.add_argument("--fp64-batch", type=int, default=0, help="q per FP64-form step (0: same as --batch)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-fp64", action="store_true")
    p.add_argument("--no-clocks", action="store_true", help="do not sample nvidia-smi (profiler runs)")
    p.add_argument("--roofline-kernels", default="assemble,colupd,refl,hemv,dots,wcorr,wfin,her2k,bisect,invit,vhx,btred,applyV,vel,xhz")
    p.add_argument("--no-configs", action="store_true", help="skip the samples of the other configurations")
    p.add_argument("--large-cell", type=int, default=0, metavar="NQ",
                   help="instead of the headline bench: NQ q-points around K of the N=11164 cell, range I 1..256 "
                        "with eigenvectors and velocities, with residual and orthogonality checks")
    return p.parse_args()


def workload(m):
    from parphom_gb300 import geometry, synth
    cell = synth.tblg_cell(m)
    phi = synth.spring_force_constants(cell, seed=0)
    crys = geometry.crys_from_positions(cell.lat, cell.real_pos)
    q_all = synth.band_path(128)
    return cell, phi, crys, q_all


class Clocks:
    """nvidia-smi sampling during the timed region (the child is always
    terminated, also on error exit)."""

    def __init__(self, index, enabled=True):
        self.p = None
        if not enabled:
            return
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
            import atexit
            atexit.register(self._kill)
        except Exception:
            self.p = None

    def _kill(self):
        if self.p is not None and self.p.poll() is None:
            self.p.kill()

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["not sampled"]}
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        rows = []
        for line in open(self.f.name):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args):
    """The reference-equivalent CPU path on the host cores, one q per step."""
    world, rank, _ = dist_setup(args)
    if rank != 0:
        return
    from oracle import oracle as O
    cell, phi, crys, q_all = workload(args.m)
    S = O.System.from_cell(cell, phi)
    cores = os.cpu_count()
    # LAPACK has nothing to warm up: each warm-up step only assembles D(q).
    for i in range(args.warmup):
        S.dynmat(q_all[(7 * i + 3) % len(q_all)])
    # one q-point per timed step; the sample stops early once ~150 s of CPU
    # time have been spent (one q of this cell takes ~50 s on 16 Grace cores)
    times = []
    for i in range(args.steps):
        t0 = time.perf_counter()
        O.solve_q(S, q_all[(7 * i + 3) % len(q_all)], vel=True, vel_method="A")
        times.append(time.perf_counter() - t0)
        if sum(times) > 150.0:
            break
    t = sum(times)
    v = len(times) / t
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": len(times),
            "steps_requested": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / len(times),
            "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "q_per_step": 1, "l2": "inputs larger than L2"},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "1 q-point per step: oracle D(q) (C restatement) + LAPACK zheevx (OpenBLAS, "
                                       "all host threads) + dense dD/dq velocities"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def large_cell(nq):
    """theta = 1.08 deg, N = 11164 (n = 33492): lowest 256 modes with
    eigenvectors and analytic velocities, mixed form; per q the residual
    ||D z - lambda z|| / ||D||_1, the orthogonality of Z and the Rayleigh
    quotients, with D assembled in FP64 by the library's own assembly."""
    import torch
    from parphom_gb300 import api, synth
    t0 = time.perf_counter()
    cell = synth.tblg_cell(30)
    phi = synth.spring_force_constants(cell)
    ctx = api.PhononContext.from_cell(cell, phi.T)  # symmetric: its F-ordered view, no copy
    qs = synth.around_k(16)[:nq]
    opts = api.EigOpts(jobz="V", range="I", il=1, iu=256, vel=True, vel_method="A", precision=api.PP_PREC_MIXED)
    t1 = time.perf_counter()
    res = ctx.solve(qs, opts)
    t2 = time.perf_counter()
    dev = torch.device("cuda")
    cw = float(np.float32(15.633302)) * float(np.float32(33.35641))
    checks = []
    for t in range(nq):
        m = int(res.m[t])
        D = torch.as_tensor(ctx.dynamical_matrix(qs[t]), device=dev)
        Z = torch.as_tensor(res.z[t][:, :m], device=dev)
        lam = torch.as_tensor(np.sign(res.w[t, :m]) * (res.w[t, :m] / cw) ** 2, device=dev)
        DZ = D @ Z
        dn = float(torch.abs(D).sum(dim=0).max().item())
        del D
        checks.append({"q": qs[t].tolist(), "m": m, "info": int(res.info[t]),
                       "nonfinite_columns": int((~torch.isfinite(Z.real) | ~torch.isfinite(Z.imag)).any(dim=0).sum()),
                       "residual": float((torch.linalg.vector_norm(DZ - Z * lam[None, :], dim=0).max() / dn).item()),
                       "orthogonality": float(torch.abs(Z.conj().T @ Z - torch.eye(m, dtype=Z.dtype, device=dev))
                                              .max().item()),
                       "w_lowest_cm1": res.w[t, :3].tolist(), "w_256_cm1": float(res.w[t, m - 1])})
        torch.cuda.empty_cache()
    print(json.dumps({"metric": "s per q-point (lowest 256 modes + eigenvectors + v_g) at N=11164", "value": (t2 - t1) / nq,
                      "unit": "s/q", "higher_is_better": False, "n_q": nq, "precision": "mixed",
                      "setup_s": t1 - t0, "checks": checks}), flush=True)
    ctx.close()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.large_cell:
        large_cell(args.large_cell)
        return
    import torch
    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from parphom_gb300 import api

    cell, phi, crys, q_all = workload(args.m)
    n = cell.n
    ctx = api.PhononContext(cell.lat, crys, cell.real_pos, cell.masses, cell.at_types, phi)
    B = args.batch
    dev = torch.device("cuda", local)
    # this rank's q-points: a disjoint slice of the path per rank, cycled
    from parphom_gb300 import replicas
    q_rank = q_all[replicas.shard(len(q_all), rank, world)]
    nbat = max(1, len(q_rank) // B)
    q_dev = [torch.tensor(np.asfortranarray(np.resize(q_rank[b * B:(b + 1) * B], (B, 3))).ravel(order="F"),
                          dtype=torch.float64, device=dev) for b in range(nbat)]
    w_dev = torch.zeros((B, n), dtype=torch.float64, device=dev)
    v_dev = torch.zeros((B, n, 3), dtype=torch.float64, device=dev)
    m_dev = torch.zeros(B, dtype=torch.int64, device=dev)
    nz_dev = torch.zeros_like(m_dev)
    info_dev = torch.zeros_like(m_dev)
    opts = api.EigOpts(jobz="N", vel=True, vel_method="A", precision=api.PP_PREC_MIXED)
    # a dedicated stream: the library's work and the timing events share it
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)

    def step(i):
        ctx.solve_device(q_dev[i % nbat], opts, w_dev, m_dev, nz_dev, info_dev, vel_dev=v_dev,
                         stream=stream.cuda_stream)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    l0 = api.kernel_launches()
    clk = Clocks(local, enabled=not args.no_clocks)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(args.steps):
        step(args.warmup + i)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    barrier()
    launches = api.kernel_launches() - l0
    t = e0.elapsed_time(e1) / 1e3
    if world > 1:
        tt = torch.tensor([t], device=dev)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t = float(tt.item())
    # per-kernel CUDA events: the same steps again with a start/stop event
    # around every launch of the selected kernel classes (the captured graph
    # is bypassed while the timer is on)
    ktimes = {}
    if args.roofline_kernels:
        api.kernel_timer(args.roofline_kernels)
        for i in range(args.steps):
            step(args.warmup + i)
        torch.cuda.synchronize()
        ktimes = api.kernel_timer_report()
        api.kernel_timer("")
    assert int(info_dev.max().item()) == 0 and int(m_dev.min().item()) == n
    value = world * B * args.steps / t

    extra = {}
    # plain FP64 form on the same q, and the frequency difference of the two forms
    if not args.no_fp64:
        Bf = args.fp64_batch or B
        qf = np.resize(q_rank[3:3 + Bf], (Bf, 3))   # off Gamma
        o64 = api.EigOpts(jobz="N", vel=True, vel_method="A", precision=api.PP_PREC_FP64)
        omx = api.EigOpts(jobz="N", vel=True, vel_method="A", precision=api.PP_PREC_MIXED)
        ctx.solve(qf, o64, want_z=False)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r64 = ctx.solve(qf, o64, want_z=False)
        t64 = time.perf_counter() - t0
        rmx = ctx.solve(qf, omx, want_z=False)
        # |w| >= 1 cm^-1 (acoustic modes near Gamma are judged on lambda in the tests)
        big = np.abs(r64.w) >= 1.0
        dw = float(np.abs(r64.w - rmx.w)[big].max())
        vmax = float(np.abs(r64.vel).max())
        dv = max(per_mode_dv(rmx.vel[t], r64.vel[t], w_to_lambda(r64.w[t]), vmax) for t in range(Bf))
        extra["fp64_form"] = {"value": Bf / t64, "unit": UNIT, "q_per_step": Bf,
                              "note": "same pipeline, IEEE double in every stage; host API, one step"}
        extra["mixed_over_fp64"] = None  # filled below from e2e-comparable numbers
        extra["library_fp64_context"] = cusolver_context(ctx, qf[:2], dev)
        extra["accuracy"] = {"max_abs_dw_cm1_mixed_vs_fp64": dw, "max_dv_rel_per_mode_mixed_vs_fp64": dv,
                             "q_compared": Bf,
                             "rule": "modes with |w| >= 1 cm^-1; velocities per mode relative to "
                                     "max(|v|, 1e-3 max|v|), cluster sums inside clusters closer than "
                                     "1e-6 ||D||"}
    # end to end through the host C ABI
    e2e = None
    if not args.no_e2e:
        qh = np.resize(q_rank[:B], (B, 3))
        ctx.solve(qh, opts, want_z=False)
        t0 = time.perf_counter()
        for i in range(args.steps):
            ctx.solve(np.resize(q_rank[(i * B) % len(q_rank):][:B], (B, 3)), opts, want_z=False)
        te = time.perf_counter() - t0
        e2e = {"value": world * B * args.steps / te if world == 1 else B * args.steps / te * world, "unit": UNIT,
               "h2d_bytes_per_step": 8 * 3 * B, "d2h_bytes_per_step": 8 * B * (n + 3 * n + 3)}
        if "fp64_form" in extra:
            extra["mixed_over_fp64"] = e2e["value"] / extra["fp64_form"]["value"]
    # roofline of the dominant kernel class
    roof = None
    if ktimes:
        dom = max(ktimes, key=lambda k: ktimes[k][1])
        roof = roofline_for(dom, ktimes[dom], n, B * args.steps)
        roof["kernel_ms_share"] = {k: round(v[1] / sum(x[1] for x in ktimes.values()), 4) for k, v in ktimes.items()}
    if rank == 0 and not args.no_configs:
        extra["configs"] = other_configs(dev)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu, ref = cpu_baseline(cell, phi, q_all)
        extra.setdefault("accuracy", {})["vs_oracle"] = oracle_accuracy(ctx, ref, q_all[3], dev)
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "df32x2 (double-float), f64 tridiagonal",
                "data": "synthetic",
                "config": {"workload": WORKLOAD, "q_per_step_per_gpu": B, "precision": "mixed",
                           "l2": "inputs larger than L2 (363 MB matrix per q)", "parallelism": f"replicas x{world}",
                           "autotuned": api.autotune_report()},
                "e2e": e2e, "gpu_launches": int(launches), "clocks": clocks, "roofline": roof,
                "cpu_baseline": cpu}
        line.update(extra)
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


# DRAM bytes (read + write) over algorithmic bytes of one k_hemv_lower launch,
# measured with ncu --set full at N=1588, batch 4, column 300: 695.7 MB for
# 637.5 MB (reads 1.032x; the partial sums written for the w-completion 5.9%).
HEMV_TRAFFIC_RATIO = 1.091


def roofline_for(kclass, rec, n, nq):
    """Algorithmic work of the dominant kernel class over the timed region."""
    launches, ms = rec
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    src = "of measured" if "hbm_gbs" in peaks else "of fallback"
    if kclass == "hemv":
        # each column i reads the lower triangle of the trailing (n-i-1)^2
        # block once: m(m+1)/2 16-byte elements, m = n-i-1
        byts = nq * 16.0 * sum((n - i - 1) * (n - i) / 2 for i in range(n - 1))
        ach = byts / (ms / 1e3) / 1e9
        return {"bound": "hbm", "kernel": "k_hemv_lower (double-float Hermitian mat-vec, lower triangle)",
                "achieved": ach, "peak": hbm,
                "unit": "GB/s", "frac": ach / hbm, "peak_source": src,
                "traffic": HEMV_TRAFFIC_RATIO * byts / launches,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch (column 300, "
                                  "batch 4) = 1.091 x its algorithmic bytes, scaled to this average launch",
                "launches": launches, "avg_launch_ms": ms / launches,
                "algorithmic_bytes_per_launch": byts / launches}
    # FP32-pipe kernels (double-float arithmetic): count complex MACs
    macs = {"her2k": 2.0 * sum((n - k) ** 2 * 32 for k in range(32, n, 32)),
            "vhx": sum(n * (n - k) * 32.0 for k in range(0, n, 32)),
            "applyV": sum(n * (n - k) * 32.0 for k in range(0, n, 32))}.get(kclass)
    if macs is None:
        return {"bound": "hbm", "kernel": kclass, "achieved": None, "peak": hbm, "unit": "GB/s", "frac": None,
                "launches": launches, "avg_launch_ms": ms / launches}
    flops = 8.0 * macs * nq
    ach = flops / (ms / 1e3) / 1e12
    return {"bound": "fp32-simt (double-float)", "kernel": kclass, "achieved": ach, "peak": None, "unit": "TFLOP/s",
            "frac": None, "launches": launches, "avg_launch_ms": ms / launches}


ALL_KERNELS = "assemble,colupd,refl,hemv,dots,wcorr,wfin,her2k,bisect,invit,vhx,btred,applyV,vel,xhz"


def timed(fn, nq, n, kclasses=ALL_KERNELS):
    """q-points/s of one call of fn through the host C ABI (host buffers in and
    out, copies included), after one untimed call of the same batch (which
    tunes and captures its launch configuration), then the same call again
    with per-kernel events for the roofline of its dominant kernel class."""
    import torch
    fn()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    from parphom_gb300 import api
    api.kernel_timer(kclasses)
    fn()
    torch.cuda.synchronize()
    kt = api.kernel_timer_report()
    api.kernel_timer("")
    roof = None
    if kt:
        dom = max(kt, key=lambda k: kt[k][1])
        if isinstance(n, (list, tuple)):   # cells of several orders: (order, q-points) pairs
            parts = [roofline_for(dom, kt[dom], ni, qi) for ni, qi in n]
            roof = dict(parts[0])
            if roof.get("achieved") is not None:
                roof["achieved"] = sum(pp["achieved"] for pp in parts)
                roof["frac"] = roof["achieved"] / roof["peak"] if roof.get("peak") else None
        else:
            roof = roofline_for(dom, kt[dom], n, nq)
        roof = {k: roof.get(k) for k in ("kernel", "bound", "achieved", "unit", "frac", "peak")}
        roof["share_of_kernel_time"] = round(kt[dom][1] / sum(v[1] for v in kt.values()), 3)
    return out, {"value": nq / dt, "unit": UNIT, "s": dt, "n_q": nq, "roofline": roof}


def oracle_check(S, q, w, vel, m=None):
    """Largest frequency difference (|w| >= 1 cm^-1) and per-mode velocity
    difference of one q-point against the oracle."""
    from oracle import oracle as O
    ref = O.solve_q(S, q, vel=vel is not None, vel_method="A")
    k = len(ref["w_cm"]) if m is None else m
    big = np.abs(ref["w_cm"]) >= 1.0
    out = {"q": list(map(float, q)), "max_abs_dw_cm1": float(np.abs(w[:k] - ref["w_cm"])[big].max())}
    if vel is not None:
        out["max_dv_rel_per_mode"] = per_mode_dv(vel[:k], ref["vel"], ref["lam"], float(np.abs(ref["vel"]).max()))
    return out


def other_configs(dev):
    """Short samples of the other configurations of the workload list (each
    q-points/s through the host C ABI, the dominant kernel's roofline, and
    accuracy on one q-point against the oracle or the FP64 form).  Sample
    sizes are stated per entry; the full q sets are the parity tests' and the
    README's business."""
    import torch
    from oracle import oracle as O
    from parphom_gb300 import api, autograd, synth
    res = {}
    # 1: N=148, FP64, 64 q on Gamma-K-M-Gamma, range A, eigenvalues only
    c = synth.tblg_cell(3)
    phi = synth.spring_force_constants(c, seed=0)
    S = O.System.from_cell(c, phi)
    with api.PhononContext.from_cell(c, phi) as ctx:
        q = synth.band_path(64)
        o = api.EigOpts(jobz="N", precision=api.PP_PREC_FP64)
        r, e = timed(lambda: ctx.solve(q, o, want_z=False), 64, c.n)
        e.update({"workload": "N=148 (3N=444), FP64, 64 q band path, range A, no vectors", "sample": "all 64 q",
                  "vs_oracle": oracle_check(S, q[5], r.w[5], None)})
        res["1_n148_fp64"] = e
    # 2: N=868, band path, vectors + analytic v_g, FP64 form and mixed form
    c = synth.tblg_cell(8)
    phi = synth.spring_force_constants(c, seed=0)
    S = O.System.from_cell(c, phi)
    with api.PhononContext.from_cell(c, phi) as ctx:
        q = synth.band_path(256)[::16]   # 16 of the 256
        ent = {"workload": "N=868 (3N=2604), band path, eigenvectors + analytic v_g",
               "sample": "16 of the 256 band-path q (every 16th)"}
        outs = {}
        for name, prec in (("fp64", api.PP_PREC_FP64), ("mixed", api.PP_PREC_MIXED)):
            o = api.EigOpts(jobz="V", vel=True, precision=prec)
            outs[name], ent[name] = timed(lambda: ctx.solve(q, o), len(q), c.n)
        ent["mixed_over_fp64"] = ent["mixed"]["value"] / ent["fp64"]["value"]
        big = np.abs(outs["fp64"].w) >= 1.0
        ent["mixed_vs_fp64"] = {
            "max_abs_dw_cm1": float(np.abs(outs["fp64"].w - outs["mixed"].w)[big].max()),
            "max_dv_rel_per_mode": max(per_mode_dv(outs["mixed"].vel[t], outs["fp64"].vel[t],
                                                   w_to_lambda(outs["fp64"].w[t]),
                                                   float(np.abs(outs["fp64"].vel).max())) for t in range(len(q)))}
        ent["vs_oracle"] = oracle_check(S, q[3], outs["mixed"].w[3], outs["mixed"].vel[3])
        res["2_n868_vectors_velocities"] = ent
    # 3: uneven cells in shared batches (pp_solve_multi), eigenvalues + velocities
    cells = [synth.tblg_cell(m) for m in (3, 5, 8)]
    ctxs = [api.PhononContext.from_cell(cc, synth.spring_force_constants(cc, seed=0)) for cc in cells]
    try:
        g = synth.uniform_grid(8)
        q = np.vstack([g, g, g])
        cell_of = np.repeat(np.arange(3), len(g))
        o = api.EigOpts(jobz="N", vel=True, precision=api.PP_PREC_MIXED)
        r, e = timed(lambda: api.solve_multi(ctxs, cell_of, q, o, want_z=False), len(q),
                     [(cc.n, len(g)) for cc in cells])
        e.update({"workload": "N=148/364/868 in shared batches, Gamma-centred grids, w + v_g, mixed",
                  "sample": "8x8 grid per cell (64 q each, 192 q) of the 32x32 grids"})
        res["3_uneven_cells"] = e
    finally:
        for cc in ctxs:
            cc.close()
    # 4: forward + backward (dL/dq, dL/dPhi) at N=1588
    c = synth.tblg_cell(11)
    phi = synth.spring_force_constants(c, seed=0)
    rng = np.random.default_rng(1)
    spec = autograd.PhononSpectrum.from_cell(c, precision=api.PP_PREC_MIXED, batch=8)
    try:
        q = torch.tensor(synth.band_path(128)[::16], device=dev, requires_grad=True)   # 8 of the 128
        pt = torch.tensor(phi, device=dev, requires_grad=True)
        target = spec.frequencies(q.detach(), pt.detach()) * torch.tensor(
            1.0 + 0.03 * rng.uniform(-1, 1, (len(q), c.n)), device=dev)
        for rep in range(2):   # the first pass tunes the launch configuration of the backward's solve
            q.grad = pt.grad = None
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            w = spec.frequencies(q, pt)
            loss = ((w - target) ** 2).sum()
            loss.backward()
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
        res["4_n1588_forward_backward"] = {
            "workload": "N=1588, loss = sum (w - w_target)^2, dL/dq and dL/dPhi (autograd.Function, device tensors)",
            "sample": "8 of the 128 q", "value": len(q) / dt, "unit": "q-pts/s (forward + backward)", "s": dt,
            "grad_phi_finite": bool(torch.isfinite(pt.grad).all()),
            "grad_phi_symmetric": bool(torch.allclose(pt.grad, pt.grad.T))}
    finally:
        spec.close()
    return res


def cusolver_context(ctx, qs, dev):
    """Context only (not on the product path): the same D(q) handed to the
    vendor library's FP64 Hermitian eigensolver (torch.linalg.eigvalsh /
    eigh on complex128, cuSOLVER heevd) on this GPU, seconds per q-point."""
    import torch
    out = {"note": "cuSOLVER heevd through torch.linalg on the library's D(q); no velocities; context for the "
                   "FP64 form, not a baseline of the metric"}
    Ds = [torch.as_tensor(ctx.dynamical_matrix(q), device=dev) for q in qs]
    for name, fn in (("eigvalsh_s_per_q", torch.linalg.eigvalsh), ("eigh_s_per_q", torch.linalg.eigh)):
        fn(Ds[0])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for D in Ds:
            fn(D)
        torch.cuda.synchronize()
        out[name] = (time.perf_counter() - t0) / len(Ds)
    del Ds
    torch.cuda.empty_cache()
    return out


def cpu_baseline(cell, phi, q_all):
    """The oracle on one q of the workload, timed; its result is kept for the
    accuracy check of the GPU path at the same q."""
    from oracle import oracle as O
    S = O.System.from_cell(cell, phi)
    t0 = time.perf_counter()
    ref = O.solve_q(S, q_all[3], vel=True, vel_method="A")
    dt = time.perf_counter() - t0
    ref["S"] = S
    return ({"value": 1.0 / dt, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
             "sample": "1 q-point of the same workload: oracle D(q) (C restatement) + LAPACK zheevx (OpenBLAS, all "
                       "host threads) + dense dD/dq velocities"}, ref)


C_W = float(np.float32(15.633302)) * float(np.float32(33.35641))


def w_to_lambda(w):
    return np.sign(w) * (np.asarray(w) / C_W) ** 2


def per_mode_dv(v, v_ref, lam_ref, vmax, gap_rel=1e-6):
    """Worst per-mode velocity difference relative to max(|v_ref|, 1e-3 vmax),
    with cluster sums inside clusters of eigenvalues closer than
    gap_rel ||D||; clamped acoustic modes (2|w| < 1e-3 cm^-1) are left out
    (their value is rounding noise over the clamp constant)."""
    lam_ref = np.asarray(lam_ref)
    norm = np.abs(lam_ref).max()
    w_ref = np.sign(lam_ref) * np.sqrt(np.abs(lam_ref)) * C_W
    floor = max(1e-3 * vmax, 1e-6)
    groups, cur = [], [0]
    for j in range(1, len(lam_ref)):
        if lam_ref[j] - lam_ref[j - 1] <= gap_rel * norm:
            cur.append(j)
        else:
            groups.append(cur)
            cur = [j]
    groups.append(cur)
    worst = 0.0
    for g in groups:
        if np.all(2.0 * np.abs(w_ref[g]) < 1e-3):
            continue
        a, b = v[g].sum(axis=0), v_ref[g].sum(axis=0)
        worst = max(worst, float((np.abs(a - b) / np.maximum(np.abs(b), floor)).max()))
    return worst


def oracle_accuracy(ctx, ref, q, dev):
    """The mixed form at the oracle's q: frequencies and per-mode velocities
    through the benchmark's own path (no eigenvector output), and the
    residual and orthogonality of its eigenvectors (a second solve with
    eigenvector output) against the oracle's D(q)."""
    import torch
    from parphom_gb300 import api
    q = np.asarray(q)[None, :]
    r = ctx.solve(q, api.EigOpts(jobz="N", vel=True, vel_method="A", precision=api.PP_PREC_MIXED), want_z=False)
    n = len(ref["w_cm"])
    big = np.abs(ref["w_cm"]) >= 1.0
    dw = float(np.abs(r.w[0, :n] - ref["w_cm"])[big].max())
    vmax = float(np.abs(ref["vel"]).max())
    dv = per_mode_dv(r.vel[0, :n], ref["vel"], ref["lam"], vmax)
    rz = ctx.solve(q, api.EigOpts(jobz="V", vel=False, precision=api.PP_PREC_MIXED))
    D = torch.as_tensor(ref["S"].dynmat(q[0]), device=dev)
    Z = torch.as_tensor(rz.z[0][:, :n], device=dev)
    lam = torch.as_tensor(w_to_lambda(rz.w[0, :n]), device=dev)
    dn = float(torch.abs(lam).max().item())
    res = float((torch.linalg.vector_norm(D @ Z - Z * lam[None, :], dim=0).max() / dn).item())
    orth = float(torch.abs(Z.conj().T @ Z - torch.eye(n, dtype=Z.dtype, device=dev)).max().item())
    del D, Z
    torch.cuda.empty_cache()
    return {"q": q[0].tolist(), "precision": "mixed", "max_abs_dw_cm1": dw, "max_dv_rel_per_mode": dv,
            "residual_rel": res, "orthogonality": orth, "n_modes_below_1cm1": int((~big).sum()),
            "oracle": "C restatement of D(q) + LAPACK zheevx (OpenBLAS) + dense dD/dq velocities",
            "gate": "|dw| < 1e-4 cm^-1, per-mode dv < 1e-6"}


if __name__ == "__main__":
    main()
