#!/usr/bin/env python
"""Benchmark of the GB300 PIC hot path (one JSON line on rank 0).

Workload (default): the explicit Buneman/Tristan Yee step on a periodic
128^3 box, electron-proton plasma (mass ratio 100), 16 particles per cell per
species (67,108,864 particles), dx = 0.1, Courant 0.45, theta_e = 0.1,
theta_p = 1e-3, B0 along x with sigma = 0.1; FP32 particles (cell index +
offset) and Yee fields, FP64 current.  A step is one full explicit step:
B half step, fused gather/push/zigzag deposit, B half step, current
assembly, E step, plus the cell sort when it is due.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Multi-GPU runs are independent replicas (one per rank, no collective on the
data path); the value is the sum over ranks of particle-steps/s computed
from the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s/GPU; implicit-solve time to 1e-8 residual, learned vs plain"
UNIT = "particle-steps/s"


def _args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--grid", type=int, nargs=3, default=[128, 128, 128])
    p.add_argument("--ppc", type=int, default=16)
    # sorting every 5 steps: 3.15 ms per step at 128^3 against 3.36, 3.20, 3.11
    # and 3.15 every 3, 4, 6 and 8 steps (6 is faster but would put 3 or 4
    # sorts into 20 timed steps depending on the phase)
    p.add_argument("--sort-every", type=int, default=5)
    p.add_argument("--e2e-steps", type=int, default=3)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--implicit-grid", type=int, nargs=3, default=[256, 256, 64])
    p.add_argument("--implicit-ppc", type=int, default=64)
    p.add_argument("--implicit-steps", type=int, default=200, help="steps of the implicit run (2 untimed)")
    p.add_argument("--implicit-sort-every", type=int, default=1, help="sort cadence of the implicit run")
    p.add_argument("--drift-steps", type=int, default=500, help="steps of the FP32-vs-FP64 explicit energy run")
    p.add_argument("--no-energy", action="store_true")
    p.add_argument("--shock-grid", type=int, nargs=3, default=[4096, 256, 4])
    p.add_argument("--shock-steps", type=int, default=20)
    p.add_argument("--shock-drift-steps", type=int, default=100)
    p.add_argument("--no-shock", action="store_true")
    p.add_argument("--only-shock", action="store_true", help="run and print only the reflecting-wall shock section")
    p.add_argument("--mixed-inner", type=int, default=12, help="most FP32 inner steps of the mixed-precision solve")
    p.add_argument("--mixed-steps", type=int, default=12, help="implicit steps timed with the mixed-precision solve")
    p.add_argument("--nn-steps", type=int, default=4000, help="training steps of the learned preconditioner")
    p.add_argument("--nn-batch", type=int, default=4, help="triples per training step (Adam, lr 1e-3)")
    p.add_argument("--nn-triples", type=int, default=2000, help="recorded plain-solve triples to train on")
    p.add_argument("--no-implicit", action="store_true")
    p.add_argument("--only-implicit", action="store_true",
                   help="run and print only the implicit section (profiling the implicit step, solver and network)")
    return p.parse_args()


def implicit_section(a):
    """The implicit counter-streaming-beams system (256x256x64, dx = dt = 0.5,
    theta = 0.5, electron-ion mass ratio 25, 64 ppc per species, beams with
    gamma = 10 along +-x, theta_e = 0.01 in the beam frame, B0 along z with
    sigma = 0.01), loaded on the device.  Times one implicit step and the
    field solve to an FP64 true relative residual of 1e-8 with plain
    GMRES(30); the learned-preconditioner solve is reported when available."""
    import math
    import torch
    import numpy as np
    import picpp_gb300 as P
    from picpp_gb300 import initstate as I
    nx, ny, nz = a.implicit_grid
    ppc = a.implicit_ppc
    box = I.Box(nx, ny, nz, 0.5, 0.5, 0.5, 0.5, theta=0.5)
    n_e = 1.0 / (4 * math.pi)
    w = I.density_weight(box, n_e, ppc)
    # pressure tensor deposited at the particle's own cells (the reference's
    # loop-index placement is the parity mode pressure_compat=1)
    # sorting every step: the deposit sums the lanes of one cell per warp
    # pass, and the beams move about a cell per step (with a sort every
    # other step the moment phase measured 362 ms instead of 141 ms)
    sim = P.GpuSimulation(box, P.IMPLICIT, particle_real=P.F32, pressure_compat=0, sort_every=a.implicit_sort_every)
    N = box.ncells
    sim.add_species(-1.0, 1.0, w, N * ppc)
    sim.add_species(1.0, 25.0, w, N * ppc)
    E = np.zeros((3, nz, ny, nx))
    B = np.zeros((3, nz, ny, nx))
    B[2] = math.sqrt(4 * math.pi * 0.01 * n_e * 26.0 * 10.0)

    def refill():
        sim.fill_species(0, ppc, 3, 0.01, 10.0, True)
        sim.fill_species(1, ppc, 4, 0.01 / 25.0, 10.0, True)
        sim.upload_fields(E, B)

    refill()
    npart = 2 * N * ppc
    opts = P.solve_opts(P.GMRES_RESTARTED, restart=30, max_iter=600, tol=1e-8)
    out = {"workload": f"implicit_beams_{nx}x{ny}x{nz}_{ppc}ppc_2species", "particles": npart, "unknowns": 3 * N}
    stream = torch.cuda.ExternalStream(sim.stream)
    # the stated run: a.implicit_steps steps from the initial state, the first
    # two untimed (warm-up), every later one bracketed by CUDA events on the
    # library stream, the phase split accumulated over the timed steps; the
    # total energy at the start and every 20 steps (outside the timed steps)
    energy = [(0, sim.updateEnergy().tolist())]
    for _ in range(2):
        sim.implicit_step(opts)
    sim.profile(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times, its, restarts = [], [], []
    for k in range(2, a.implicit_steps):
        e0.record(stream)
        info = sim.implicit_step(opts)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
        its.append(info["iterations"])
        restarts.append(info["restarts"])
        if (k + 1) % 20 == 0 or k + 1 == a.implicit_steps:
            energy.append((k + 1, sim.updateEnergy().tolist()))
    phases, launches = sim.profile(False)
    nt = len(times)
    ms = statistics.median(times)
    per = {k: v / nt for k, v in phases.items() if v > 0}
    out["steps_run"] = a.implicit_steps
    out["timed_steps"] = nt
    out["step_ms"] = {"median": ms, "mean": statistics.fmean(times), "min": min(times), "max": max(times),
                      "stdev": statistics.pstdev(times)}
    out["particle_steps_per_s"] = npart / (ms * 1e-3)
    out["phase_ms"] = per
    out["phase_note"] = "deposit (the particle deposit kernel) is part of moments"
    peak, src = _hbm_peak()
    dep_bytes = 28 * npart + 352 * N    # particles read; J-hat, mu, rho-hat, Pi FP64 read-modify-write per cell
    mov_bytes = 56 * npart + 96 * N     # particles read and written; E, B FP64 gathers per cell
    roof = {}
    for kern, ph, b, per_unit in (("k_implicit_deposit_tile<float>", "deposit", dep_bytes, "28 B/particle + 352 B/cell"),
                                  ("k_implicit_push_tile<float>", "mover", mov_bytes, "56 B/particle + 96 B/cell")):
        if per.get(ph):
            ach = b / (per[ph] * 1e-3) / 1e9
            roof[kern] = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                          "peak_source": src, "algorithmic_bytes_per_launch": b, "bytes_per_unit": per_unit,
                          "launch_ms": per[ph]}
    # GMRES(30) bytes: Arnoldi step j (j basis vectors) moves 120 + 24 (2j + 5) B per cell, plus one
    # operator apply (120 B/cell) for the residual at the start of each cycle and for the true residual
    it_med = statistics.median(its)
    gm_bytes = statistics.fmean(
        N * (sum(120 + 24 * (2 * (i % 30 + 1) + 5) for i in range(n_it)) + 240 * (n_rs + 1))
        for n_it, n_rs in zip(its, restarts))
    if per.get("solve"):
        ach = gm_bytes / (per["solve"] * 1e-3) / 1e9
        roof["gmres_solve"] = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                               "peak_source": src, "algorithmic_bytes_per_solve": gm_bytes,
                               "bytes_per_unit": "sum over iterations of 120 + 24 (2j + 5) B/cell + 240 B/cell per cycle",
                               "solve_ms": per["solve"]}
    out["roofline"] = roof
    if per.get("moments"):
        out["mass_matrix_deposits_per_s"] = npart * 8 * 9 / (per["moments"] * 1e-3)
    if per.get("deposit"):
        out["mass_matrix_deposits_per_s_kernel"] = npart * 8 * 9 / (per["deposit"] * 1e-3)
    if per.get("solve"):
        out["field_solves_per_s"] = 1.0 / (per["solve"] * 1e-3)
    out["gmres_iterations"] = {"median": it_med, "min": min(its), "max": max(its)}
    out["energy_drift"] = _drift(energy)
    out["plain"] = {"solver": "GMRES(30), classical Gram-Schmidt with selective second pass, FP64",
                    "iterations": info["iterations"], "restarts": info["restarts"],
                    "rel_residual": info["rel_residual"], "seconds": info["seconds"]}
    out["mixed_vs_plain"] = mixed_solve(a, sim, opts, refill)
    if a.nn_steps > 0:
        out["learned_vs_plain"] = learned_solve(a, sim, box, w, opts)
    sim.close()
    if a.nn_steps > 0:
        out["learned_vs_plain_stiff"] = stiff_solve(a, w)
    return out


def _hbm_peak():
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(peaks["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _drift(series):
    """Total energy (kinetic + electric + magnetic) of (step, pic_energy)
    samples: relative change from the first sample to the last, and the
    largest relative excursion."""
    w = [(k, e[0] + e[1] + e[2]) for k, e in series]
    w0 = w[0][1]
    return {"steps": w[-1][0], "samples": len(w), "total_initial": w0, "total_final": w[-1][1],
            "drift": (w[-1][1] - w0) / w0, "max_excursion": max(abs(v - w0) for _, v in w) / w0,
            "field_energy_final": series[-1][1][1] + series[-1][1][2]}


def energy_section(a, st):
    """Energy bookkeeping of two stated runs (pic_energy, the reference's
    updateEnergy): the Weibel pairs (32x32x1, 32 ppc per species, dt = 0.1,
    seed 1) for 100 implicit steps in FP64, and the explicit workload's
    state run for a.drift_steps steps with FP32 particles and fields and
    with FP64 throughout from the same initial state, energy every 10
    steps, with the FP32 run's field and energy differences from FP64."""
    import numpy as np
    import torch
    import picpp_gb300 as P
    from picpp_gb300 import initstate as I
    out = {}
    ws = I.weibel_pairs(32, 32, 1, seed=1)
    sim = P.GpuSimulation(ws.box, P.IMPLICIT, particle_real=P.F64, pressure_compat=0, sort_every=1)
    sim.upload_state(ws)
    ser = [(0, sim.updateEnergy().tolist())]
    t0 = time.perf_counter()
    for k in range(100):
        sim.implicit_step(P.solve_opts(P.GMRES_REFERENCE))
        ser.append((k + 1, sim.updateEnergy().tolist()))
    out["weibel_32x32x1_fp64"] = dict(_drift(ser), wall_s=time.perf_counter() - t0,
                                      solver="GMRES, reference stopping rule")
    sim.close()
    runs = {}
    for name, real in (("fp32", P.F32), ("fp64", P.F64)):
        sim = P.GpuSimulation(st.box, P.BUNEMAN, particle_real=real, sort_every=a.sort_every)
        sim.upload_state(st)
        ser = [(0, sim.updateEnergy().tolist())]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(0, a.drift_steps, 10):
            n = min(10, a.drift_steps - k)
            sim.buneman_step(n)
            ser.append((k + n, sim.updateEnergy().tolist()))
        wall = time.perf_counter() - t0
        E, B, _ = sim.download_fields()
        runs[name] = (ser, E, B, wall)
        sim.close()
    s32, E32, B32, w32 = runs["fp32"]
    s64, E64, B64, w64 = runs["fp64"]
    tot32 = np.array([e[0] + e[1] + e[2] for _, e in s32])
    tot64 = np.array([e[0] + e[1] + e[2] for _, e in s64])
    rel = lambda x, y: float(np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300))  # noqa: E731
    nx, ny, nz = a.grid
    out[f"buneman_{nx}x{ny}x{nz}_fp32_vs_fp64"] = {
        "steps": a.drift_steps, "fp32": dict(_drift(s32), wall_s=w32), "fp64": dict(_drift(s64), wall_s=w64),
        "energy_series_max_rel_diff": float(np.abs(tot32 - tot64).max() / np.abs(tot64).max()),
        "field_rel_l2_diff_final": {"E": rel(E32, E64), "B": rel(B32, B64),
                                    "B_minus_B0": rel(B32 - st.B, B64 - st.B)}}
    return out


def _shock_sim(P, I, nx, ny, nz, real, seed, cap_factor=1.5, dt=0.4, dx=0.5):
    """A wall box of the reflecting-wall shock setup filled on the device
    (flow along -x), with its injector; returns (sim, injector, particles)."""
    specs, E0, B0, v0 = I.shock_parameters(dx)
    box = I.Box(nx, ny, nz, dx, dx, dx, dt, theta=0.5)
    sim = P.GpuSimulation(box, P.IMPLICIT, particle_real=real, pressure_compat=0, sort_every=1,
                          boundary_x=P.BOUNDARY_WALL_OPEN, e_right=tuple(E0), b_right=tuple(B0))
    cells = (nx - 2) * ny * nz
    total = 0
    for s, (q, m, n, ppc, th) in enumerate(specs):
        sim.add_species(q, m, I.density_weight(box, n, ppc), int(cap_factor * ppc * cells) + 64 * ny * nz)
        sim.fill_species(s, ppc, seed * 10 + s, th, 1.5, -1)
        total += ppc * cells
    E, B = I.wall_fields(nx, ny, nz, E0, B0)
    sim.upload_fields(E, B)
    return sim, I.Injector(box, specs, 1.5, seed=seed), total


def shock_section(a):
    """The reflecting-wall shock: a conductor wall at x = 0 and an open
    boundary on the right through which the upstream plasma (electrons 32,
    protons of mass 64 32, He2+ of mass 256 8 particles per cell at 10% of
    the proton density, flow gamma 1.5 towards -x, theta_e = 1e-3, B0 at 60
    degrees to x with sigma = 0.04, dx = 0.5, dt = 0.4) keeps entering.
    Storage a.shock_grid (the physical domain is two cells shorter along x),
    FP32 push, FP64 GMRES(30) to a 1e-8 relative residual, a.shock_steps
    timed steps with injection; the solve of the last step's system with
    plain GMRES(30) and with FGMRES(30) + the network (trained on a periodic
    64x64x4 box of the upstream plasma); and the total energy of an FP32 and
    an FP64 run of a 512x64x4 box of the same setup for a.shock_drift_steps
    steps with the same injected particles."""
    import numpy as np
    import torch
    import picpp_gb300 as P
    from picpp_gb300 import initstate as I
    nx, ny, nz = a.shock_grid
    out = {"workload": f"shock_wall_{nx}x{ny}x{nz}_32_32_8ppc_3species",
           "physical_cells_x": nx - 2, "note": "storage nx includes the two ghost columns of the wall box"}
    opts = P.solve_opts(P.GMRES_RESTARTED, restart=30, max_iter=600, tol=1e-8)
    sim, inj, n0 = _shock_sim(P, I, nx, ny, nz, P.F32, 5)
    out["particles_initial"] = n0
    stream = torch.cuda.ExternalStream(sim.stream)

    def count():
        return sum(sim.download_particles(s, with_ids=False)["cell"].size for s in range(3))

    def inject():
        k = 0
        for s, new in enumerate(inj.step()):
            sim.append_particles(s, new)
            k += new["cell"].size
        return k

    inject()
    sim.implicit_step(opts)   # warm-up
    e0 = sim.updateEnergy().tolist()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times, its, injected, psteps = [], [], 0, 0
    sim.profile(True)
    for _ in range(a.shock_steps):
        ev0.record(stream)
        injected += inject()
        info = sim.implicit_step(opts)
        ev1.record(stream)
        ev1.synchronize()
        times.append(ev0.elapsed_time(ev1))
        its.append(info["iterations"])
    phases, _ = sim.profile(False)
    n_end = count()
    e1 = sim.updateEnergy().tolist()
    ms = statistics.median(times)
    out["timed_steps"] = a.shock_steps
    out["step_ms"] = {"median": ms, "min": min(times), "max": max(times)}
    out["particles_end"] = n_end
    out["injected_per_step"] = injected / max(a.shock_steps, 1)
    out["particle_steps_per_s"] = 0.5 * (n0 + n_end) / (ms * 1e-3)
    out["phase_ms"] = {k: v / a.shock_steps for k, v in phases.items() if v > 0}
    out["gmres_iterations"] = {"median": statistics.median(its), "max": max(its)}
    out["total_energy"] = {"after_warmup": e0[0] + e0[1] + e0[2], "end": e1[0] + e1[1] + e1[2],
                           "note": "open system: injected and escaped particles carry energy in and out"}
    if a.nn_steps > 0:
        # the network on a periodic box of the upstream plasma
        specs, E0, B0, v0 = I.shock_parameters()
        tb = I.Box(64, 64, 4, 0.5, 0.5, 0.5, 0.4, theta=0.5)
        tsim = P.GpuSimulation(tb, P.IMPLICIT, particle_real=P.F32, pressure_compat=0, sort_every=1)
        for s, (q, m, n, ppc, th) in enumerate(specs):
            tsim.add_species(q, m, I.density_weight(tb, n, ppc), ppc * tb.ncells)
            tsim.fill_species(s, ppc, 70 + s, th, 1.5, -1)
        tsim.upload_fields(*I.wall_fields(64, 64, 4, E0, B0))
        tsim.implicit_step(opts)
        tsim.updateElectroMagneticParameters()
        tsim.nn_init(1)
        tr = tsim.nn_train(steps=a.nn_steps // 2, batch=a.nn_batch, lr=1e-3, seed=5, smooth_max=2)
        params = tsim.nn_get_params()
        tsim.close()
        sim.nn_set_params(params)
        sim.updateElectroMagneticParameters()
        _, mu, _, rhs = sim.download_moments()
        plain = P.solve_opts(P.GMRES_RESTARTED, restart=30, max_iter=600, tol=1e-8)
        learned = P.solve_opts(P.FGMRES_LEARNED, restart=30, max_iter=600, tol=1e-8)
        sim.maxwell_solve(mu, rhs, plain)
        sim.maxwell_solve(mu, rhs, learned)
        _, ip = sim.maxwell_solve(mu, rhs, plain)
        _, il = sim.maxwell_solve(mu, rhs, learned)
        out["learned_vs_plain"] = {
            "plain": {k: ip[k] for k in ("iterations", "restarts", "rel_residual", "seconds")},
            "learned": {k: il[k] for k in ("iterations", "restarts", "used_fallback", "rel_residual", "seconds")},
            "speedup": ip["seconds"] / il["seconds"] if il["seconds"] > 0 else None,
            "train": {"box": [64, 64, 4], "steps": tr["steps"], "seconds": tr["seconds"],
                      "first_loss": tr["first_loss"], "last_loss": tr["last_loss"]}}
    sim.close()
    # FP32 against FP64 on a smaller box, the same injected particles
    runs = {}
    for name, real in (("fp32", P.F32), ("fp64", P.F64)):
        s2, inj2, _ = _shock_sim(P, I, 512, 64, 4, real, 6)
        ser = []
        for k in range(a.shock_drift_steps):
            for sp_id, new in enumerate(inj2.step()):
                s2.append_particles(sp_id, new)
            s2.implicit_step(opts)
            if k % 10 == 9 or k == a.shock_drift_steps - 1:
                ser.append(s2.updateEnergy())
        E2, B2, _ = s2.download_fields()
        runs[name] = (np.array(ser), E2, B2)
        s2.close()
    t32 = runs["fp32"][0][:, :3].sum(axis=1)
    t64 = runs["fp64"][0][:, :3].sum(axis=1)
    rel = lambda x, y: float(np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300))  # noqa: E731
    out["fp32_vs_fp64_512x64x4"] = {"steps": a.shock_drift_steps,
                                    "energy_series_max_rel_diff": float(np.abs(t32 - t64).max() / np.abs(t64).max()),
                                    "field_rel_l2_diff_final": {"E": rel(runs["fp32"][1], runs["fp64"][1]),
                                                                "B": rel(runs["fp32"][2], runs["fp64"][2])}}
    return out

def _beams(box, ppc, w, seeds):
    """A simulation of the implicit beam plasma on box (device fill), with
    the uniform B0 along z; particles and fields as in implicit_section."""
    import math
    import numpy as np
    import picpp_gb300 as P
    sim = P.GpuSimulation(box, P.IMPLICIT, particle_real=P.F32, pressure_compat=0, sort_every=1)
    N = box.ncells
    sim.add_species(-1.0, 1.0, w, N * ppc)
    sim.add_species(1.0, 25.0, w, N * ppc)
    sim.fill_species(0, ppc, seeds[0], 0.01, 10.0, True)
    sim.fill_species(1, ppc, seeds[1], 0.01 / 25.0, 10.0, True)
    E = np.zeros((3, box.nz, box.ny, box.nx))
    B = np.zeros((3, box.nz, box.ny, box.nx))
    B[2] = math.sqrt(4 * math.pi * 0.01 * (1.0 / (4 * math.pi)) * 26.0 * 10.0)
    sim.upload_fields(E, B)
    return sim


def stiff_solve(a, w):
    """The same plasma and grid with dt = 2 (K / dx^2 = (c' theta dt / dx)^2
    ~ 4.2 instead of 0.26): the system of the first implicit step solved to
    an FP64 relative residual of 1e-8 with plain GMRES(30) and with
    FGMRES(30) + the network trained on a 64x64x16 box of it (white-noise
    fields).  A regime where the preconditioner has work to do; the
    headline comparison is learned_vs_plain (dt = 0.5)."""
    import picpp_gb300 as P
    from picpp_gb300 import initstate as I
    nx, ny, nz = a.implicit_grid
    ppc = a.implicit_ppc
    box = I.Box(nx, ny, nz, 0.5, 0.5, 0.5, 2.0, theta=0.5)
    tb = I.Box(64, 64, 16, 0.5, 0.5, 0.5, 2.0, theta=0.5)
    tsim = _beams(tb, ppc, w, (33, 34))
    tsim.updateElectroMagneticParameters()
    tsim.nn_init(1)
    tr = tsim.nn_train(steps=a.nn_steps, batch=a.nn_batch, lr=1e-3, seed=3, smooth_max=0)
    params = tsim.nn_get_params()
    tsim.close()
    sim = _beams(box, ppc, w, (23, 24))
    sim.nn_set_params(params)
    sim.updateElectroMagneticParameters()
    _, mu, _, rhs = sim.download_moments()
    plain_opts = P.solve_opts(P.GMRES_RESTARTED, restart=30, max_iter=3000, tol=1e-8)
    learned_opts = P.solve_opts(P.FGMRES_LEARNED, restart=30, max_iter=3000, tol=1e-8)
    mixed_opts = P.solve_opts(P.FGMRES_MIXED, restart=30, max_iter=3000, tol=1e-8, inner=a.mixed_inner)
    sim.maxwell_solve(mu, rhs, plain_opts)   # warm-up of all three paths
    sim.maxwell_solve(mu, rhs, learned_opts)
    sim.maxwell_solve(mu, rhs, mixed_opts)
    _, ip = sim.maxwell_solve(mu, rhs, plain_opts)
    _, il = sim.maxwell_solve(mu, rhs, learned_opts)
    _, im = sim.maxwell_solve(mu, rhs, mixed_opts)
    sim.close()
    return {"system": f"first implicit step, {nx}x{ny}x{nz}, dt = 2 (K/dx^2 = 4.2)", "tol": 1e-8,
            "plain": {k: ip[k] for k in ("iterations", "restarts", "rel_residual", "seconds")},
            "learned": {k: il[k] for k in ("iterations", "restarts", "used_fallback", "rel_residual", "seconds")},
            "speedup": ip["seconds"] / il["seconds"] if il["seconds"] > 0 else None,
            "mixed": {"inner": a.mixed_inner, **{k: im[k] for k in ("iterations", "restarts", "used_fallback",
                                                                     "rel_residual", "seconds")},
                      "speedup": ip["seconds"] / im["seconds"] if im["seconds"] > 0 else None},
            "train": {"box": [64, 64, 16], "steps": tr["steps"], "seconds": tr["seconds"],
                      "first_loss": tr["first_loss"], "last_loss": tr["last_loss"]}}


NET_LAYERS = [(16, 16, 0), (16, 16, 0), (16, 32, 1), (32, 32, 1), (32, 64, 2), (64, 64, 2), (96, 32, 1),
              (32, 32, 1), (48, 16, 0), (16, 16, 0), (16, 16, 0)]   # (cin, cout, level) of the network


def mixed_solve(a, sim, plain_opts, refill=None):
    """The mixed-precision right preconditioner (FGMRES(30) in FP64 around an
    FP32 GMRES solve of at most `inner` Arnoldi steps) against plain GMRES(30) on the
    system of the state after the timed steps, to an FP64 true relative
    residual of 1e-8: iterations and device time for several inner lengths;
    then a.mixed_steps implicit steps with the mixed solve (inner
    a.mixed_inner) from the stated run's initial state (refill), two
    untimed, timed like the stated run."""
    import torch
    import picpp_gb300 as P
    sim.updateElectroMagneticParameters()
    _, mu, _, rhs = sim.download_moments()
    sim.maxwell_solve(mu, rhs, plain_opts)   # warm-up
    _, ip = sim.maxwell_solve(mu, rhs, plain_opts)
    rows = []
    for k in (8, 12, 16, 20, 24):
        o = P.solve_opts(P.FGMRES_MIXED, restart=30, max_iter=600, tol=1e-8, inner=k)
        sim.maxwell_solve(mu, rhs, o)   # warm-up (workspace)
        _, im = sim.maxwell_solve(mu, rhs, o)
        rows.append({"inner": k, "outer_iterations": im["iterations"], "ms": im["seconds"] * 1e3,
                     "rel_residual": im["rel_residual"], "fallback": im["used_fallback"],
                     "speedup": ip["seconds"] / im["seconds"]})
    out = {"system": "the state after the timed steps", "tol": 1e-8,
           "plain": {"iterations": ip["iterations"], "ms": ip["seconds"] * 1e3, "rel_residual": ip["rel_residual"]},
           "mixed": rows}
    if a.mixed_steps > 0 and refill is not None:
        # the same plasma from the same seeds: these steps start where the
        # stated run started
        refill()
        mo = P.solve_opts(P.FGMRES_MIXED, restart=30, max_iter=600, tol=1e-8, inner=a.mixed_inner)
        stream = torch.cuda.ExternalStream(sim.stream)
        for _ in range(2):
            sim.implicit_step(mo)
        sim.profile(True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        times, its = [], []
        for _ in range(a.mixed_steps):
            e0.record(stream)
            info = sim.implicit_step(mo)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            its.append(info["iterations"])
        phases, _ = sim.profile(False)
        out["steps"] = {"inner": a.mixed_inner, "from": "the stated run's initial state, 2 untimed steps",
                        "timed_steps": len(times), "step_ms_median": statistics.median(times),
                        "step_ms_min": min(times), "step_ms_max": max(times),
                        "outer_iterations": {"min": min(its), "max": max(its)},
                        "phase_ms": {k: v / len(times) for k, v in phases.items() if v > 0}}
    return out


def learned_solve(a, sim, box, w, opts):
    """The learned preconditioner's protocol: the first a.nn_triples
    (right-hand side, mu, FP64 solution) triples that plain GMRES(30)
    produces on runs of seeds 10-19 of the same plasma (a 64x64x16 box, 200
    steps per run; the network is convolutional, its parameters carry over
    to the full box), Adam at lr 1e-3, batch a.nn_batch: half of a.nn_steps
    on random fields of the last recorded operator (residual loss), half on
    the triples (supervised and residual losses); then, on held-out seeds
    20-24 of the
    full box, the system of the step after the first is solved to an FP64
    relative residual of 1e-8 with plain GMRES(30) and with FGMRES(30) + the
    network: iterations and device time, mean and spread over the seeds."""
    import math
    import numpy as np
    import picpp_gb300 as P
    from picpp_gb300 import initstate as I
    ppc = a.implicit_ppc
    tb = I.Box(64, 64, 16, box.dx, box.dy, box.dz, box.dt, theta=box.theta)
    tsim = _beams(tb, ppc, w, (20, 21))
    tsim.nn_record(a.nn_triples)
    runs = 0
    for seed in range(10, 20):
        if tsim.nn_record_count() >= a.nn_triples:
            break
        tsim.fill_species(0, ppc, 2 * seed, 0.01, 10.0, True)
        tsim.fill_species(1, ppc, 2 * seed + 1, 0.01 / 25.0, 10.0, True)
        E, B = I.zero_fields(tb)
        B[2] = math.sqrt(4 * math.pi * 0.01 * (1.0 / (4 * math.pi)) * 26.0 * 10.0)
        tsim.upload_fields(E, B)
        runs += 1
        for _ in range(200):
            tsim.implicit_step(opts)
            if tsim.nn_record_count() >= a.nn_triples:
                break
    triples = tsim.nn_record_count()
    # first on random fields of the last recorded operator (residual loss, rough
    # inputs like the later Krylov vectors), then on the recorded triples
    tsim.updateElectroMagneticParameters()
    tsim.nn_init(1)
    tr0 = tsim.nn_train(steps=a.nn_steps // 2, batch=a.nn_batch, lr=1e-3, seed=3, smooth_max=2, source=0)
    tr = tsim.nn_train(steps=a.nn_steps - a.nn_steps // 2, batch=a.nn_batch, lr=1e-3, seed=4, source=1,
                       supervised_weight=0.5)
    params = tsim.nn_get_params()
    tsim.close()
    sim.nn_set_params(params)
    plain_opts = P.solve_opts(P.GMRES_RESTARTED, restart=30, max_iter=600, tol=1e-8)
    learned_opts = P.solve_opts(P.FGMRES_LEARNED, restart=30, max_iter=600, tol=1e-8)
    rows = []
    for seed in range(20, 25):
        sim.fill_species(0, ppc, 2 * seed, 0.01, 10.0, True)
        sim.fill_species(1, ppc, 2 * seed + 1, 0.01 / 25.0, 10.0, True)
        E, B = I.zero_fields(box)
        B[2] = math.sqrt(4 * math.pi * 0.01 * (1.0 / (4 * math.pi)) * 26.0 * 10.0)
        sim.upload_fields(E, B)
        sim.implicit_step(opts)
        sim.updateElectroMagneticParameters()
        _, mu, _, rhs = sim.download_moments()
        if not rows:   # warm-up of both paths
            sim.maxwell_solve(mu, rhs, plain_opts)
            sim.maxwell_solve(mu, rhs, learned_opts)
        _, ip = sim.maxwell_solve(mu, rhs, plain_opts)
        _, il = sim.maxwell_solve(mu, rhs, learned_opts)
        rows.append((seed, ip, il))
    n = box.ncells
    flop = sum(2 * 27 * ci * co * n / 8 ** lv for ci, co, lv in NET_LAYERS)

    def stats(vals):
        return {"mean": statistics.fmean(vals), "min": min(vals), "max": max(vals),
                "stdev": statistics.pstdev(vals)}

    pit = [r[1]["iterations"] for r in rows]
    lit = [r[2]["iterations"] for r in rows]
    pms = [r[1]["seconds"] * 1e3 for r in rows]
    lms = [r[2]["seconds"] * 1e3 for r in rows]
    per_it = statistics.fmean(p / max(i, 1) for p, i in zip(pms, pit))
    apply_ms = statistics.fmean(max(l - i * per_it, 0.0) / max(i, 1) for l, i in zip(lms, lit))
    return {"system": "step 2 of held-out seeds 20-24 of the full box", "tol": 1e-8,
            "plain": {"iterations": stats(pit), "ms": stats(pms)},
            "learned": {"iterations": stats(lit), "ms": stats(lms),
                        "fallbacks": sum(r[2]["used_fallback"] for r in rows)},
            "speedup": statistics.fmean(pms) / statistics.fmean(lms),
            "per_seed": [{"seed": sd, "plain_iterations": ip["iterations"], "plain_ms": ip["seconds"] * 1e3,
                          "learned_iterations": il["iterations"], "learned_ms": il["seconds"] * 1e3}
                         for sd, ip, il in rows],
            "network": {"flop_per_apply": flop, "apply_ms_est": apply_ms,
                        "tflops_est": flop / (apply_ms * 1e-3) / 1e12 if apply_ms > 0 else None,
                        "train": {"box": [64, 64, 16], "triples": triples, "runs": runs, "seeds": "10-19",
                                  "batch": a.nn_batch, "lr": 1e-3,
                                  "random_fields": {"steps": tr0["steps"], "seconds": tr0["seconds"],
                                                    "first_loss": tr0["first_loss"], "last_loss": tr0["last_loss"],
                                                    "loss": "|A z - r|^2/|r|^2"},
                                  "triples": {"steps": tr["steps"], "seconds": tr["seconds"],
                                              "first_loss": tr["first_loss"], "last_loss": tr["last_loss"],
                                              "loss": "0.5 |z - x|^2/|x|^2 + 0.5 |A z - b|^2/|b|^2"}}}}

def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x, world):
    """The slowest rank's time: an all-reduce MAX over the process group
    (CUDA tensor under NCCL, CPU tensor under gloo); x itself for one rank."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(particles_per_rank, world, ms_per_step):
    """Whole-job particle-steps/s of world replicas, each with
    particles_per_rank particles, from the slowest rank's ms per step."""
    return particles_per_rank * world / (ms_per_step * 1e-3)


# ---------------------------------------------------------------- CPU side
def _oracle_worker(args):
    """One replica of the oracle on a bounded sample box (spawned process)."""
    nx, ny, nz, ppc, steps, seed = args
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    from picpp_gb300 import initstate as I
    st = I.buneman_plasma(nx, ny, nz, ppc=ppc, seed=seed)
    g = O.make_grid(st.box)
    sp = st.species
    E, B = st.E.copy(), st.B.copy()
    O.buneman_step(g, sp, E, B)   # warm-up
    t0 = time.perf_counter()
    for _ in range(steps):
        O.buneman_step(g, sp, E, B)
    dt = time.perf_counter() - t0
    return sum(len(s["cell"]) for s in sp) * steps, dt


def cpu_baseline(ppc, procs=1, target_s=10.0):
    """The oracle (plain-C restatement of the reference) on a 16^3 sample box
    with the workload's ppc and physics; procs independent replicas."""
    import multiprocessing as mp
    sample = (16, 16, 16, ppc)
    ctx = mp.get_context("spawn")
    with ctx.Pool(1) as pool:
        n, dt = pool.apply(_oracle_worker, ((*sample, 2, 11),))
    per_step = dt / 2
    steps = max(2, int(target_s / max(per_step, 1e-3)))
    with ctx.Pool(procs) as pool:
        res = pool.map(_oracle_worker, [(*sample, steps, 100 + r) for r in range(procs)])
    total = sum(r[0] for r in res)
    wall = max(r[1] for r in res)
    desc = f"{procs} replica(s) of a 16x16x16 box, {ppc} ppc x 2 species, {steps} steps each"
    return total / wall, desc, steps


def run_reference(a):
    rank, world, _ = _dist()
    if rank != 0:
        return
    procs = os.cpu_count() or 1
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    O.build()
    t0 = time.perf_counter()
    vals = []
    for _ in range(a.warmup):
        cpu_baseline(a.ppc, procs, target_s=2.0)
    for _ in range(a.steps):
        v, desc, steps = cpu_baseline(a.ppc, procs, target_s=2.0)
        vals.append(v)
    value = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": _config(a),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port", "sample": desc},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": time.perf_counter() - t0,
    }
    print(json.dumps(line), flush=True)


def _config(a):
    nx, ny, nz = a.grid
    n = nx * ny * nz * a.ppc * 2
    return {"workload": f"buneman_yee_{nx}x{ny}x{nz}_{a.ppc}ppc_2species", "grid": [nx, ny, nz],
            "ppc_per_species": a.ppc, "species": 2, "particles": n, "mass_ratio": 100,
            "dx": 0.1, "courant": 0.45, "precision": "fp32 particles and Yee fields, fp64 current",
            "sort_every": a.sort_every, "parallelism": f"replicas x{a.gpus}",
            "l2_policy": "inputs larger than L2 (particle state 1.9 GB per GPU)"}


# ---------------------------------------------------------------- clocks
class Clocks:
    def __init__(self, index):
        self.p = None
        fd, self.path = tempfile.mkstemp(prefix="picpp_clocks_", suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={q}", "--format=csv,noheader",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.p.terminate()
        self.p.wait()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for row in open(self.path):
            f = [x.strip() for x in row.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1].split()[0]))
                smax.append(float(f[2].split()[0]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        try:
            os.unlink(self.path)
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons)}


# ---------------------------------------------------------------- GPU side
def run_gb300(a):
    import numpy as np
    import torch
    import picpp_gb300 as P
    from picpp_gb300 import initstate as I

    rank, world, local = _dist()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    P.load_library()
    nx, ny, nz = a.grid
    st = I.buneman_plasma(nx, ny, nz, ppc=a.ppc, seed=2 + rank)
    npart = sum(len(s["cell"]) for s in st.species)
    sim = P.GpuSimulation(st.box, P.BUNEMAN, particle_real=P.F32, sort_every=a.sort_every)
    sim.upload_state(st)
    stream = torch.cuda.ExternalStream(sim.stream)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    sim.buneman_step(a.warmup)
    barrier()
    clocks = Clocks(local)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    sim.buneman_step(a.steps)
    e1.record(stream)
    e1.synchronize()
    barrier()
    ck = clocks.stop()
    ms = max_over_ranks(e0.elapsed_time(e1), world)
    ms_step = ms / a.steps
    value = replica_value(npart, world, ms_step)

    # phase breakdown of the same workload, a separate profiled pass
    sim.profile(True)
    sim.buneman_step(a.steps)
    phases, launches = sim.profile(False)
    launches_per_step = launches / a.steps
    push_ms = phases["push_deposit"] / a.steps
    N = nx * ny * nz
    alg_bytes = 56 * npart + 24 * N   # particles r+w (28 B each way) + E,B gather (FP32) once per cell
    peak, peak_src = _hbm_peak()
    achieved = alg_bytes / (push_ms * 1e-3) / 1e9
    # DRAM bytes of one launch from an ncu capture of the same kernel on the
    # 64^3 case (dram__bytes_read.sum + dram__bytes_write.sum = 518.8 MB),
    # scaled by the units a launch processes (particles and cells grow alike)
    units = npart / (64 ** 3 * 2 * a.ppc) if a.ppc else 0.0
    traffic = 518.8e6 * units if (nx * ny * nz) * 2 * a.ppc == npart else None
    roof = {"kernel": "k_push_deposit_tile<float,float>", "bound": "hbm", "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
            "traffic_source": "ncu dram bytes of the 64^3 launch scaled by the particles per launch",
            "peak_source": peak_src,
            "algorithmic_bytes_per_launch": alg_bytes, "launch_ms": push_ms,
            "phase_ms_per_step": {k: v / a.steps for k, v in phases.items() if v > 0}}

    # end to end through the C ABI with pinned host buffers
    def pinned(shape, dtype):
        return torch.empty(shape, dtype=dtype, pin_memory=True).numpy()

    hsp = []
    for s in st.species:
        n = len(s["cell"])
        d = {k: pinned(n, torch.float64) for k in ("ox", "oy", "oz", "px", "py", "pz")}
        d["cell"] = pinned(n, torch.int32)
        for k in d:
            d[k][:] = s[k]
        hsp.append(d)
    hE = pinned(st.E.shape, torch.float64); hE[:] = st.E
    hB = pinned(st.B.shape, torch.float64); hB[:] = st.B
    hJ = pinned(st.E.shape, torch.float64)
    h2d = sum(len(d["cell"]) * (4 + 6 * 8) for d in hsp) + 2 * hE.nbytes
    d2h = sum(len(d["cell"]) * (4 + 6 * 8) for d in hsp) + 3 * hE.nbytes
    L = sim.L
    ptr = lambda x: x.ctypes.data_as(P._dp)  # noqa: E731
    iptr = lambda x: x.ctypes.data_as(P._ip)  # noqa: E731

    def e2e_step():
        for sid, d in enumerate(hsp):
            sim._ck(L.pic_upload_particles(sim.ctx, sid, len(d["cell"]), iptr(d["cell"]), ptr(d["ox"]), ptr(d["oy"]),
                                           ptr(d["oz"]), ptr(d["px"]), ptr(d["py"]), ptr(d["pz"]), None))
        sim._ck(L.pic_upload_fields(sim.ctx, ptr(hE), ptr(hB)))
        sim._ck(L.pic_buneman_step(sim.ctx, 1))
        for sid, d in enumerate(hsp):
            sim._ck(L.pic_download_particles(sim.ctx, sid, None, iptr(d["cell"]), ptr(d["ox"]), ptr(d["oy"]),
                                             ptr(d["oz"]), ptr(d["px"]), ptr(d["py"]), ptr(d["pz"]), None))
        sim._ck(L.pic_download_fields(sim.ctx, ptr(hE), ptr(hB), ptr(hJ)))

    e2e_step()
    barrier()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(a.e2e_steps):
        e2e_step()
    f1.record(stream)
    f1.synchronize()
    barrier()
    e2e_ms = max_over_ranks(f0.elapsed_time(f1), world) / a.e2e_steps
    e2e_val = replica_value(npart, world, e2e_ms)

    sim.close()
    # the sections after the timed replicas describe one GPU and only rank 0
    # reports them: the other ranks release their GPUs here
    energy = None
    if not a.no_energy and rank == 0:
        energy = energy_section(a, st)
    del st
    imp = None
    if not a.no_implicit and rank == 0:
        imp = implicit_section(a)
    shock = None
    if not a.no_shock and rank == 0:
        shock = shock_section(a)
    if rank == 0:
        cpu = None
        if not a.no_cpu_baseline:
            v, desc, _ = cpu_baseline(a.ppc, 1, target_s=10.0)
            cpu = {"value": v, "unit": UNIT, "cores": 1, "kind": "port", "sample": desc}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Maxwell-Juttner plasma)",
            "config": _config(a), "roofline": roof, "cpu_baseline": cpu,
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": e2e_ms},
            "gpu_launches": int(round(launches_per_step * a.steps)), "clocks": ck,
            "implicit_solve": imp, "energy_drift": energy, "shock": shock,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    a = _args()
    if a.impl == "reference":
        run_reference(a)
    elif a.only_shock:
        import picpp_gb300 as P
        P.load_library()
        print(json.dumps({"shock": shock_section(a)}), flush=True)
    elif a.only_implicit:
        import picpp_gb300 as P
        P.load_library()
        print(json.dumps({"implicit_solve": implicit_section(a)}), flush=True)
    else:
        run_gb300(a)


if __name__ == "__main__":
    main()
