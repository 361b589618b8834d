"""Seeded synthetic initial states for the workloads this library runs.

The reference seeds its particle loader with ``srand(time(NULL)+rank)`` and a
4096-level quantised ``rand()`` (PIC++/main.cpp:73, PIC++/random.cpp:16-18),
so its runs cannot be replayed.  Every comparison here instead starts from one
state produced by this module and fed identically to the CUDA path, the
oracle and the reference harness.

Units are the reference's normalised units: c = 1, electron mass 1,
elementary charge 1, and the electron plasma frequency 1, i.e. an electron
density of 1/(4 pi).  A species' macro-particle weight is its density times
the cell volume divided by the particles per cell.

Each species is a dict with float ``q``, ``m``, ``w`` and numpy arrays
``cell`` (int32, linear cell index, i fastest), ``ox``, ``oy``, ``oz``
(in-cell offsets in [0, 1)) and ``px``, ``py``, ``pz`` (momentum m*gamma*v).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

FOUR_PI = 4.0 * math.pi


@dataclass
class Box:
    nx: int
    ny: int
    nz: int
    dx: float
    dy: float
    dz: float
    dt: float
    theta: float = 0.5
    eta: float = 0.5
    cfix: float = 1.025

    @property
    def ncells(self) -> int:
        return self.nx * self.ny * self.nz


@dataclass
class State:
    box: Box
    species: list = field(default_factory=list)
    E: np.ndarray | None = None   # (3, nz, ny, nx) float64
    B: np.ndarray | None = None   # (3, nz, ny, nx) float64


def _juttner_speed_table(theta: float, n: int = 200001):
    """CDF of u = |p|/(mc) under the Maxwell-Juttner law
    f(u) ~ u^2 exp(-(gamma(u)-1)/theta), tabulated for inverse sampling."""
    umax = math.sqrt((1.0 + 40.0 * theta) ** 2 - 1.0) + 1e-12
    u = np.linspace(0.0, umax, n)
    g = np.sqrt(1.0 + u * u)
    pdf = u * u * np.exp(-(g - 1.0) / theta)
    cdf = np.concatenate([[0.0], np.cumsum(0.5 * (pdf[1:] + pdf[:-1]) * np.diff(u))])
    cdf /= cdf[-1]
    return u, cdf


def sample_juttner(rng: np.random.Generator, count: int, theta: float, mass: float,
                   drift_gamma: float = 1.0, drift_sign: np.ndarray | float = 1.0):
    """Momenta (px, py, pz) of a Maxwell-Juttner plasma of temperature theta
    (kT/mc^2), optionally drifting along x with Lorentz factor drift_gamma.
    The drift uses the flipping method (Zenitani 2015, Phys. Plasmas 22,
    042116) so that the boosted distribution carries the right Jacobian."""
    if theta <= 0.0:
        u = np.zeros((count, 3))
    else:
        ug, cdf = _juttner_speed_table(theta)
        s = np.interp(rng.random(count), cdf, ug)
        cos_t = 2.0 * rng.random(count) - 1.0
        phi = 2.0 * math.pi * rng.random(count)
        sin_t = np.sqrt(np.maximum(0.0, 1.0 - cos_t * cos_t))
        u = np.stack([s * cos_t, s * sin_t * np.cos(phi), s * sin_t * np.sin(phi)], axis=1)
    if drift_gamma > 1.0:
        beta = math.sqrt(1.0 - 1.0 / (drift_gamma * drift_gamma))
        sign = np.broadcast_to(np.asarray(drift_sign, dtype=np.float64), (count,))
        g = np.sqrt(1.0 + np.sum(u * u, axis=1))
        vx = u[:, 0] / g
        flip = (-beta * sign * vx) > rng.random(count)
        u[flip, 0] = -u[flip, 0]
        ux = drift_gamma * (u[:, 0] + sign * beta * g)
        u[:, 0] = ux
    return u[:, 0] * mass, u[:, 1] * mass, u[:, 2] * mass


def uniform_species(rng, box: Box, ppc: int, q: float, m: float, w: float, theta: float,
                    drift_gamma: float = 1.0, drift_sign=1.0) -> dict:
    """ppc particles in every cell, offsets uniform in the cell."""
    n = box.ncells * ppc
    cell = np.repeat(np.arange(box.ncells, dtype=np.int32), ppc)
    off = rng.random((3, n))
    px, py, pz = sample_juttner(rng, n, theta, m, drift_gamma, drift_sign)
    return dict(q=float(q), m=float(m), w=float(w), cell=cell,
                ox=off[0].copy(), oy=off[1].copy(), oz=off[2].copy(),
                px=px, py=py, pz=pz)


def density_weight(box: Box, density: float, ppc: int) -> float:
    return density * box.dx * box.dy * box.dz / ppc


def zero_fields(box: Box):
    shape = (3, box.nz, box.ny, box.nx)
    return np.zeros(shape), np.zeros(shape)


def buneman_plasma(nx, ny, nz, dx=0.1, courant=0.45, ppc=16, mass_ratio=100.0,
                   theta_e=0.1, theta_p=1e-3, sigma=0.1, seed=2) -> State:
    """Electron-proton plasma with a uniform B0 along x: the explicit Yee
    workload (128^3, dx = 0.1, Courant 0.45, 16 ppc per species, mass ratio
    100, theta_e = 0.1, theta_p = 1e-3, sigma = 0.1 at full size)."""
    box = Box(nx, ny, nz, dx, dx, dx, courant * dx)
    rng = np.random.default_rng(seed)
    n_e = 1.0 / FOUR_PI
    w = density_weight(box, n_e, ppc)
    el = uniform_species(rng, box, ppc, -1.0, 1.0, w, theta_e)
    pr = uniform_species(rng, box, ppc, 1.0, mass_ratio, w, theta_p)
    E, B = zero_fields(box)
    B0 = math.sqrt(FOUR_PI * sigma * n_e * (1.0 + mass_ratio))
    B[0] = B0
    return State(box, [el, pr], E, B)


def beams_plasma(nx, ny, nz, dx=0.5, dt=0.5, ppc=64, mass_ratio=25.0, beam_gamma=10.0,
                 theta_e=0.01, sigma=0.01, theta=0.5, seed=3) -> State:
    """Counter-streaming electron-ion beams (Lorentz factor beam_gamma along
    +-x, half of each species each way), uniform B0 along z: the implicit
    workload (256x256x64, dx = dt = 0.5, 64 ppc per species at full size)."""
    box = Box(nx, ny, nz, dx, dx, dx, dt, theta=theta)
    rng = np.random.default_rng(seed)
    n_e = 1.0 / FOUR_PI
    w = density_weight(box, n_e, ppc)
    species = []
    for q, m, th in ((-1.0, 1.0, theta_e), (1.0, mass_ratio, theta_e / mass_ratio)):
        n = box.ncells * ppc
        sign = np.where(np.arange(n) % 2 == 0, 1.0, -1.0)
        sp = uniform_species(rng, box, ppc, q, m, w, th, beam_gamma, sign)
        species.append(sp)
    E, B = zero_fields(box)
    B[2] = math.sqrt(FOUR_PI * sigma * n_e * (1.0 + mass_ratio) * beam_gamma)
    return State(box, species, E, B)


def weibel_pairs(nx, ny, nz, dx=0.2, dt=0.1, ppc=32, theta_t=0.01, drift_v=0.5,
                 theta=0.5, seed=1) -> State:
    """Electron-positron Weibel setup: +-0.5c drifts along x, half of each
    species each way (net current zero), zero initial fields."""
    box = Box(nx, ny, nz, dx, dx, dx, dt, theta=theta)
    rng = np.random.default_rng(seed)
    n_e = 1.0 / FOUR_PI
    w = density_weight(box, n_e, ppc)
    g = 1.0 / math.sqrt(1.0 - drift_v * drift_v)
    species = []
    for q in (-1.0, 1.0):
        n = box.ncells * ppc
        sign = np.where(np.arange(n) % 2 == 0, 1.0, -1.0)
        species.append(uniform_species(rng, box, ppc, q, 1.0, w, theta_t, g, sign))
    E, B = zero_fields(box)
    return State(box, species, E, B)


@dataclass
class FlowState(State):
    """A State of a box with a conductor wall at x = 0 and an open boundary
    at x = (nx - 2) dx (storage columns nx - 2 and nx - 1 are the ghost
    cells beyond the open boundary and left of the wall), with the
    boundary's constant fields and the upstream flow that feeds it."""
    e_right: tuple = (0.0, 0.0, 0.0)
    b_right: tuple = (0.0, 0.0, 0.0)
    flow_gamma: float = 1.0
    temperatures: tuple = ()   # theta = kT / m c^2 per species
    ppc: tuple = ()


def shock_parameters(dx=0.5, ppc=(32, 32, 8), flow_gamma=1.5, theta_e=1e-3, sigma=0.04, angle_deg=60.0,
                     mass_ratio=64.0, he_mass=256.0, he_fraction=0.1):
    """Species and fields of the reflecting-wall shock setup: a plasma of
    electrons, protons (mass_ratio) and fully ionised helium (charge 2, mass
    he_mass, number density he_fraction of the protons'), charge neutral,
    flowing towards -x with Lorentz factor flow_gamma; every species at the
    electron temperature (theta = theta_e m_e / m_s); B0 at angle_deg to x
    in the x-y plane with sigma = B0^2 / (4 pi flow_gamma sum_s n_s m_s);
    E0 = -V0 x B0 (initializeFluxFromRight, PIC++/initialization.cpp:
    5201-5207).  Electron density 1 / (4 pi) (omega_pe = 1).  Returns
    (species [(q, m, density, ppc, theta)], E0, B0, v0)."""
    n_e = 1.0 / FOUR_PI
    n_p = n_e / (1.0 + 2.0 * he_fraction)
    n_he = he_fraction * n_p
    specs = [(-1.0, 1.0, n_e, ppc[0], theta_e), (1.0, mass_ratio, n_p, ppc[1], theta_e / mass_ratio),
             (2.0, he_mass, n_he, ppc[2], theta_e / he_mass)]
    v0 = math.sqrt(1.0 - 1.0 / (flow_gamma * flow_gamma))
    rho_m = sum(n * m for _, m, n, _, _ in specs)
    b0 = math.sqrt(sigma * FOUR_PI * flow_gamma * rho_m)
    a = math.radians(angle_deg)
    B0 = np.array([b0 * math.cos(a), b0 * math.sin(a), 0.0])
    E0 = -np.cross(np.array([-v0, 0.0, 0.0]), B0)
    return specs, E0, B0, v0


def wall_fields(nx, ny, nz, E0, B0):
    """Initial fields of a wall box: E0 and B0 everywhere, Ey = Ez = 0 on
    the wall node (initializeFluxFromRight)."""
    E = np.zeros((3, nz, ny, nx))
    B = np.zeros((3, nz, ny, nx))
    for d in range(3):
        E[d] = E0[d]
        B[d] = B0[d]
    E[1, :, :, 0] = 0.0
    E[2, :, :, 0] = 0.0
    return E, B


# The explicit (Tristan) mover reflects at xgrid[reflectingWallPoint]
# (PIC++/mover.cpp:746-750, constants.h:64): node 18 of the wall box, and
# createParticles fills the box from there (initialization.cpp:8152-8155).
TRISTAN_WALL_NODE = 18


def shock_plasma(nx, ny, nz, dx=0.5, dt=0.4, ppc=(32, 32, 8), flow_gamma=1.5, theta_e=1e-3, sigma=0.04,
                 angle_deg=60.0, mass_ratio=64.0, he_mass=256.0, he_fraction=0.1, theta=0.5, seed=5,
                 first_cell=0) -> FlowState:
    """The reflecting-wall shock setup (shock_parameters) on a wall box of
    nx x ny x nz storage cells: the flow fills the physical cells
    first_cell .. nx - 3 of every x row (first_cell = TRISTAN_WALL_NODE for
    the explicit path, whose particles reflect there)."""
    box = Box(nx, ny, nz, dx, dx, dx, dt, theta=theta)
    rng = np.random.default_rng(seed)
    specs, E0, B0, v0 = shock_parameters(dx, ppc, flow_gamma, theta_e, sigma, angle_deg, mass_ratio, he_mass,
                                         he_fraction)
    phys = Box(nx - 2 - first_cell, ny, nz, dx, dx, dx, dt, theta=theta)
    species, temps = [], []
    for q, m, n, c, th in specs:
        sp = uniform_species(rng, phys, c, q, m, density_weight(box, n, c), th, flow_gamma, -1.0)
        i = sp["cell"] % phys.nx + first_cell
        rest = sp["cell"] // phys.nx
        sp["cell"] = (rest * nx + i).astype(np.int32)   # physical cells in the storage layout
        species.append(sp)
        temps.append(th)
    E, B = wall_fields(nx, ny, nz, E0, B0)
    return FlowState(box, species, E, B, tuple(E0), tuple(B0), flow_gamma, tuple(temps), tuple(ppc))


class Injector:
    """The open boundary's particle source with the bookkeeping of
    Simulation::simulate and injectNewParticles (PIC++/simulation.cpp:126,
    281-285; PIC++/mover.cpp:910-1000): per species an injection length
    that grows by |V0| dt every step; while ppc * length >= dx it shrinks by
    dx / ppc and one particle enters every (y, z) cell column at
    x = (nx - 2) dx - length.  Offsets along y and z are uniform per
    particle (the reference draws one pair per call) and momenta are the
    species' drifting Maxwell-Juttner law."""

    def __init__(self, box: Box, species, flow_gamma: float, seed: int = 0):
        self.box = box
        self.species = species          # [(q, m, density, ppc, theta)]
        self.gamma = flow_gamma
        self.v0 = math.sqrt(1.0 - 1.0 / (flow_gamma * flow_gamma))
        self.length = [box.dx / c - 1e-4 * box.dx for _, _, _, c, _ in species]
        self.rng = np.random.default_rng(seed)

    def step(self):
        """The particles of one step, one dict per species (cell, ox, oy, oz,
        px, py, pz)."""
        b = self.box
        cols = b.ny * b.nz
        out = []
        for s, (q, m, n, ppc, th) in enumerate(self.species):
            self.length[s] += abs(self.v0 * b.dt)
            lengths = []
            while self.length[s] * ppc >= b.dx:
                self.length[s] -= b.dx / ppc
                lengths.append(self.length[s])
            k = len(lengths)
            x = ((b.nx - 2) * b.dx - np.repeat(np.array(lengths, dtype=np.float64), cols)) / b.dx
            ci = np.floor(x)
            jk = np.tile(np.arange(cols), k)
            cell = ((jk // b.ny) * b.ny + jk % b.ny) * b.nx + ci.astype(np.int64)
            px, py, pz = sample_juttner(self.rng, k * cols, th, m, self.gamma, -1.0)
            out.append(dict(cell=cell.astype(np.int32), ox=x - ci, oy=self.rng.random(k * cols),
                            oz=self.rng.random(k * cols), px=px, py=py, pz=pz))
        return out

def positions(box: Box, sp: dict):
    """Physical positions in [0, L) from cell + offset (float64)."""
    c = sp["cell"].astype(np.int64)
    i = c % box.nx
    j = (c // box.nx) % box.ny
    k = c // (box.nx * box.ny)
    return ((i + sp["ox"]) * box.dx, (j + sp["oy"]) * box.dy, (k + sp["oz"]) * box.dz)


def from_positions(box: Box, x, y, z):
    """Cell index and offsets from physical positions (wrapped periodic)."""
    out = []
    for pos, d, n in ((x, box.dx, box.nx), (y, box.dy, box.ny), (z, box.dz, box.nz)):
        u = np.asarray(pos, dtype=np.float64) / d
        c = np.floor(u)
        o = u - c
        c = c.astype(np.int64)
        over = o >= 1.0
        o[over] -= 1.0
        c[over] += 1
        out.append((np.mod(c, n), o))
    (i, ox), (j, oy), (k, oz) = out
    cell = ((k * box.ny + j) * box.nx + i).astype(np.int32)
    return cell, ox, oy, oz
