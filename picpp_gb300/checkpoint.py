"""Host-side reader and writer of the binary checkpoint that
``pic_save_checkpoint`` / ``pic_load_checkpoint`` use (include/picpp_gb300.h).

The same file carries a state in both directions between this library and
any host code: a state written here from an ``initstate.State`` loads on the
GPU, and a checkpoint the GPU wrote reads back into an ``initstate.State``
that a CPU implementation of the step can continue.  It replaces the text
backup of PIC++ (``outputSimulationBackup`` / ``readBackup``,
PIC++/output.cpp:3432-3601, PIC++/input.cpp:342-624), which rounds every
value to 10 significant digits (``%15.10g``) and reads the particle type
table at ``type - 1`` (PIC++/input.cpp:608).

Layout (little endian, no padding other than noted):

* header, 120 bytes: ``char magic[8] = "PICGB300"``; int32 version (2),
  solver (0 Buneman, 1 implicit), particle_real, field_real (0 FP32,
  1 FP64), nx, ny, nz, nspecies, has_net, sorted, reserved; 4 bytes of
  padding; int64 step; float64 dx, dy, dz, dt, theta, eta, cfix;
* per species: float64 q, m, w; int64 n; int32 cell[n], id[n]; then ox, oy,
  oz, px, py, pz, n values each in the particle precision; when ``sorted``,
  int32 off[ncells + 1], the per-key offsets of the last sort;
* fields, three components of nx*ny*nz values each, component-major then
  k, j, i: Buneman runs E and B in the particle precision and the last
  current J in FP64; implicit runs E (nodes), B (cell centres) and the last
  J-hat, all FP64;
* when ``has_net``, the learned preconditioner's FP32 parameters to the end
  of the file.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np

from .initstate import Box, State

MAGIC = b"PICGB300"
VERSION = 2
HEADER = struct.Struct("<8s11i4xq7d")
PARTICLE_ARRAYS = ("ox", "oy", "oz", "px", "py", "pz")


@dataclass
class Checkpoint:
    box: Box
    solver: int
    particle_real: int
    field_real: int
    step: int = 0
    species: list = field(default_factory=list)   # dicts: q, m, w, cell, id, ox..pz, off (or None)
    E: np.ndarray | None = None                    # (3, nz, ny, nx)
    B: np.ndarray | None = None
    J: np.ndarray | None = None
    params: np.ndarray | None = None               # FP32 network parameters
    sorted: bool = False


def _rdtype(real: int):
    return np.float64 if real else np.float32


def read(path) -> Checkpoint:
    with open(path, "rb") as f:
        raw = f.read()
    if len(raw) < HEADER.size:
        raise ValueError("checkpoint truncated")
    (magic, version, solver, preal, freal, nx, ny, nz, nspecies, has_net, srt, _res, step,
     dx, dy, dz, dt, theta, eta, cfix) = HEADER.unpack_from(raw, 0)
    if magic != MAGIC or version != VERSION:
        raise ValueError("not a picpp_gb300 checkpoint")
    box = Box(nx, ny, nz, dx, dy, dz, dt, theta, eta, cfix)
    N = nx * ny * nz
    pos = HEADER.size

    def take(dtype, count):
        nonlocal pos
        nbytes = np.dtype(dtype).itemsize * count
        if pos + nbytes > len(raw):
            raise ValueError("checkpoint truncated")
        a = np.frombuffer(raw, dtype=np.dtype(dtype).newbyteorder("<"), count=count, offset=pos).copy()
        pos += nbytes
        return a

    pt = _rdtype(preal)
    species = []
    for _ in range(nspecies):
        q, m, w = take(np.float64, 3)
        (n,) = take(np.int64, 1)
        sp = dict(q=float(q), m=float(m), w=float(w))
        sp["cell"] = take(np.int32, int(n))
        sp["id"] = take(np.int32, int(n))
        for k in PARTICLE_ARRAYS:
            sp[k] = take(pt, int(n))
        sp["off"] = take(np.int32, N + 1) if srt else None
        species.append(sp)
    shape = (3, nz, ny, nx)
    ft = pt if solver == 0 else np.float64
    E = take(ft, 3 * N).reshape(shape)
    B = take(ft, 3 * N).reshape(shape)
    J = take(np.float64, 3 * N).reshape(shape)
    params = None
    if has_net:
        rest = len(raw) - pos
        if rest <= 0 or rest % 4:
            raise ValueError("checkpoint network parameters truncated")
        params = take(np.float32, rest // 4)
    if pos != len(raw):
        raise ValueError("trailing bytes in checkpoint")
    return Checkpoint(box, solver, preal, freal, int(step), species, E, B, J, params, bool(srt))


def write(path, ck: Checkpoint) -> None:
    b = ck.box
    N = b.nx * b.ny * b.nz
    pt = _rdtype(ck.particle_real)
    ft = pt if ck.solver == 0 else np.float64
    srt = bool(ck.sorted) and all(sp.get("off") is not None for sp in ck.species)
    out = [HEADER.pack(MAGIC, VERSION, ck.solver, ck.particle_real, ck.field_real, b.nx, b.ny, b.nz,
                       len(ck.species), 1 if ck.params is not None else 0, 1 if srt else 0, 0, int(ck.step),
                       b.dx, b.dy, b.dz, b.dt, b.theta, b.eta, b.cfix)]
    for sp in ck.species:
        n = len(sp["cell"])
        out.append(np.array([sp["q"], sp["m"], sp["w"]], dtype="<f8").tobytes())
        out.append(np.array([n], dtype="<i8").tobytes())
        out.append(np.ascontiguousarray(sp["cell"], dtype="<i4").tobytes())
        ids = sp.get("id")
        ids = np.arange(n, dtype=np.int32) if ids is None else ids
        out.append(np.ascontiguousarray(ids, dtype="<i4").tobytes())
        for k in PARTICLE_ARRAYS:
            out.append(np.ascontiguousarray(sp[k], dtype=pt).astype(np.dtype(pt).newbyteorder("<")).tobytes())
        if srt:
            off = np.ascontiguousarray(sp["off"], dtype="<i4")
            if off.size != N + 1:
                raise ValueError("sort offsets need ncells + 1 entries")
            out.append(off.tobytes())
    for F, t in ((ck.E, ft), (ck.B, ft), (ck.J, np.float64)):
        a = np.zeros(3 * N) if F is None else np.asarray(F).reshape(-1)
        if a.size != 3 * N:
            raise ValueError("field arrays need 3 * ncells values")
        out.append(a.astype(np.dtype(t).newbyteorder("<")).tobytes())
    if ck.params is not None:
        out.append(np.ascontiguousarray(ck.params, dtype="<f4").tobytes())
    with open(path, "wb") as f:
        f.write(b"".join(out))


def from_state(state: State, solver: int, particle_real: int, field_real: int | None = None,
               step: int = 0) -> Checkpoint:
    """A checkpoint of an initial state (particles in input order, ids
    0..n-1, no sort offsets, zero current)."""
    species = []
    for sp in state.species:
        d = {k: sp[k] for k in ("q", "m", "w", "cell")}
        d["id"] = np.arange(len(sp["cell"]), dtype=np.int32)
        for k in PARTICLE_ARRAYS:
            d[k] = np.asarray(sp[k])
        d["off"] = None
        species.append(d)
    fr = particle_real if field_real is None else field_real
    return Checkpoint(state.box, solver, particle_real, fr, step, species, np.asarray(state.E), np.asarray(state.B),
                      None, None, False)


def to_state(ck: Checkpoint, by_id: bool = True) -> State:
    """The checkpoint's particles and fields as an FP64 ``State`` (each
    species in id order when by_id, else in the stored order)."""
    species = []
    for sp in ck.species:
        order = np.argsort(sp["id"], kind="stable") if by_id else np.arange(len(sp["cell"]))
        d = dict(q=sp["q"], m=sp["m"], w=sp["w"], cell=sp["cell"][order].astype(np.int32))
        for k in PARTICLE_ARRAYS:
            d[k] = sp[k][order].astype(np.float64)
        species.append(d)
    return State(ck.box, species, ck.E.astype(np.float64), ck.B.astype(np.float64))
