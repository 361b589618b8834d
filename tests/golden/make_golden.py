"""Generates the golden vectors in this directory from the PIC++ reference.

Each case builds a seeded initial state (picpp_gb300.initstate), runs the
reference -- compiled from its own sources by oracle/Makefile and driven by
oracle/ref/harness.cpp -- and stores inputs and outputs in one .npz.  The
reference tree is needed to run this script; the fixtures it writes are what
the tests read on machines without it.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pyoracle as O  # noqa: E402
from picpp_gb300 import initstate as I  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def _noise(st, amp, seed):
    rng = np.random.default_rng(seed)
    st.E = st.E + amp * rng.standard_normal(st.E.shape)
    st.B = st.B + amp * rng.standard_normal(st.B.shape)
    return st


def _save(name, solver, st, steps, out_sp, E, B, extra):
    d = dict(solver=solver, steps=steps,
             box=np.array([st.box.nx, st.box.ny, st.box.nz]),
             params=np.array([st.box.dx, st.box.dy, st.box.dz, st.box.dt, st.box.theta, st.box.eta, st.box.cfix]),
             E0=st.E, B0=st.B, E=E, B=B, nspecies=len(st.species))
    for s, (sp, o) in enumerate(zip(st.species, out_sp)):
        d[f"s{s}_qmw"] = np.array([sp["q"], sp["m"], sp["w"]])
        for k in ("cell", "ox", "oy", "oz", "px", "py", "pz"):
            d[f"s{s}_{k}"] = sp[k]
        for k in ("x", "y", "z", "px", "py", "pz"):
            d[f"s{s}_out_{k}"] = o[k]
    for k, v in extra.items():
        d[f"x_{k}"] = v
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
    print("wrote", name)


def buneman(name, nx, ny, nz, ppc, steps, seed, smoothing=(0, 0.5)):
    st = _noise(I.buneman_plasma(nx, ny, nz, ppc=ppc, seed=seed), 0.05, seed + 100)
    out_sp, E, B, extra = O.run_reference(0, st.box, st.species, st.E, st.B, steps, smoothing_count=smoothing[0],
                                          smoothing_parameter=smoothing[1])
    if smoothing[0]:
        extra["smoothing"] = np.array(smoothing, dtype=np.float64)
    _save(name, 0, st, steps, out_sp, E, B, extra)


def implicit(name, nx, ny, nz, ppc, steps, seed, beam_gamma=2.0, dt=0.2):
    st = _noise(I.beams_plasma(nx, ny, nz, ppc=ppc, beam_gamma=beam_gamma, dt=dt, seed=seed), 0.05, seed + 100)
    out_sp, E, B, extra = O.run_reference(1, st.box, st.species, st.E, st.B, steps, dump=True)
    _save(name, 1, st, steps, out_sp, E, B, extra)


def wall(name, nx, ny, nz, ppc, steps, seed, flow_gamma=3.0, theta_e=0.3):
    """The reflecting-wall setup (conductor wall at x = 0, open boundary at
    x = (nx - 2) dx with constant fields) with a third of every species
    turned towards the open boundary, so that particles both reflect and
    escape; the reference runs SUPER_CONDUCTOR_LEFT without injection."""
    st = I.shock_plasma(nx, ny, nz, ppc=ppc, flow_gamma=flow_gamma, theta_e=theta_e, seed=seed)
    rng = np.random.default_rng(seed + 100)
    for sp in st.species:
        sp["px"][::3] = -sp["px"][::3]
    st.E = st.E + 0.02 * rng.standard_normal(st.E.shape)
    out_sp, E, B, extra = O.run_reference(1, st.box, st.species, st.E, st.B, steps, dump=True, wall_x=1,
                                          e_right=st.e_right, b_right=st.b_right)
    extra["wall"] = np.concatenate([np.asarray(st.e_right), np.asarray(st.b_right)])
    _save(name, 1, st, steps, out_sp, E, B, extra)


def tristan_wall(name, nx, ny, nz, ppc, steps, seed, flow_gamma=3.0, theta_e=0.3, dx=0.5, courant=0.45):
    """The explicit path in a reflecting-wall box: the flow fills the cells
    from the reflecting wall (node 18) to the open boundary and a third of
    every species is turned towards the open boundary, so that particles
    both reflect and escape; E_right's y, z components are Simulation::E0
    on the boundary node."""
    st = I.shock_plasma(nx, ny, nz, dx=dx, dt=courant * dx, ppc=ppc, flow_gamma=flow_gamma, theta_e=theta_e,
                        seed=seed, first_cell=I.TRISTAN_WALL_NODE)
    rng = np.random.default_rng(seed + 100)
    for sp in st.species:
        sp["px"][::3] = -sp["px"][::3]
    st.E = st.E + 0.02 * rng.standard_normal(st.E.shape)
    out_sp, E, B, extra = O.run_reference(0, st.box, st.species, st.E, st.B, steps, wall_x=1,
                                          e_right=st.e_right, b_right=st.b_right)
    extra["wall"] = np.concatenate([np.asarray(st.e_right), np.asarray(st.b_right)])
    _save(name, 0, st, steps, out_sp, E, B, extra)


def density(name, nx, ny, nz, ppc, seed):
    """updateDensityParameters of a seeded state, one species per reference
    run (the harness gives every particle reference type 0)."""
    st = I.beams_plasma(nx, ny, nz, ppc=ppc, beam_gamma=2.0, dt=0.2, seed=seed)
    conc, en, vel, rho = [], [], [], 0.0
    for sp in st.species:
        _, _, _, extra = O.run_reference(1, st.box, [dict(sp)], st.E, st.B, 0, density=True)
        c, e, v, r = extra["density"]
        conc.append(c[0]); en.append(e[0]); vel.append(v[0]); rho = rho + r
    extra = dict(conc=np.array(conc), energy=np.array(en), vel=np.array(vel), rho=rho)
    _save(name, 1, st, 0, [dict(x=sp["ox"], y=sp["oy"], z=sp["oz"], px=sp["px"], py=sp["py"], pz=sp["pz"])
                           for sp in st.species], st.E, st.B, extra)


def wall_density(name, nx, ny, nz, ppc, seed):
    """updateDensityParameters in the reflecting-wall box (SUPER_CONDUCTOR_LEFT,
    one rank): particles fill every physical cell and a third move towards
    the wall, so that both ghost-column folds carry mass and momentum."""
    st = I.shock_plasma(nx, ny, nz, ppc=ppc, flow_gamma=3.0, theta_e=0.3, seed=seed)
    for sp in st.species:
        sp["px"][::3] = -sp["px"][::3]
    conc, en, vel, rho = [], [], [], 0.0
    for sp in st.species:
        _, _, _, extra = O.run_reference(1, st.box, [dict(sp)], st.E, st.B, 0, density=True, wall_x=1,
                                         e_right=st.e_right, b_right=st.b_right)
        c, e, v, r = extra["density"]
        conc.append(c[0]); en.append(e[0]); vel.append(v[0]); rho = rho + r
    extra = dict(conc=np.array(conc), energy=np.array(en), vel=np.array(vel), rho=rho,
                 wall=np.concatenate([np.asarray(st.e_right), np.asarray(st.b_right)]))
    _save(name, 1, st, 0, [dict(x=sp["ox"], y=sp["oy"], z=sp["oz"], px=sp["px"], py=sp["py"], pz=sp["pz"])
                           for sp in st.species], st.E, st.B, extra)


def main():
    if not O.reference_available():
        sys.exit("the PIC++ reference tree is not available here (set PICPP_REFERENCE_SRC)")
    only = sys.argv[1:]   # optional name prefixes: regenerate just those cases
    if only:
        global _save
        full_save = _save

        def _save(name, *a, **k):   # noqa: F811
            if any(name.startswith(p) for p in only):
                full_save(name, *a, **k)
    buneman("buneman_8x8x8_3steps", 8, 8, 8, 2, 3, 11)
    buneman("buneman_12x6x5_2steps", 12, 6, 5, 3, 2, 12)
    buneman("buneman_2d_16x8x1_3steps", 16, 8, 1, 4, 3, 13)
    implicit("implicit_6x5x7_1step", 6, 5, 7, 2, 1, 21)
    implicit("implicit_8x8x8_3steps", 8, 8, 8, 2, 3, 22)
    implicit("implicit_gamma10_6x6x6_2steps", 6, 6, 6, 2, 2, 23, beam_gamma=10.0, dt=0.5)
    buneman("buneman_smooth_8x6x5_2steps", 8, 6, 5, 3, 2, 14, smoothing=(2, 0.4))
    buneman("buneman_smooth_2d_12x8x1_2steps", 12, 8, 1, 3, 2, 15, smoothing=(1, 0.5))
    wall("wall_7x4x4_4steps", 7, 4, 4, (4, 4, 2), 4, 41)
    wall("wall_10x6x5_2steps", 10, 6, 5, (3, 3, 2), 2, 42)
    tristan_wall("tristan_wall_26x4x4_4steps", 26, 4, 4, (3, 3, 2), 4, 51)
    tristan_wall("tristan_wall_32x6x5_3steps", 32, 6, 5, (4, 3, 2), 3, 52)
    density("density_8x6x5", 8, 6, 5, 3, 31)
    density("density_2d_8x8x1", 8, 8, 1, 4, 32)
    wall_density("density_wall_12x6x5", 12, 6, 5, (3, 3, 2), 61)
    wall_density("density_wall_9x5x4", 9, 5, 4, (4, 3, 2), 62)


if __name__ == "__main__":
    main()
