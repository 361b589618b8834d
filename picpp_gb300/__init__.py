"""picpp_gb300 -- GB300 (sm_103a) implementation of PIC++'s per-timestep hot
path behind a C ABI (include/picpp_gb300.h), with a Python mirror of the
reference's ``Simulation`` call surface for tests and benchmarks.

The CUDA library is mandatory: every entry point runs on the GPU, and
loading fails loudly when ``libpicpp_gb300.so`` is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpicpp_gb300.so")

PIC_OK = 0
PIC_ERR_ARG = 1
STATUS = {0: "OK", 1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_STATE", 4: "ERR_NOMEM", 5: "ERR_NUMERIC",
          6: "ERR_NOT_CONVERGED"}
PIC_NOALLOC_MAX_SPECIES = 16
BUNEMAN, IMPLICIT = 0, 1
BOUNDARY_PERIODIC, BOUNDARY_WALL_OPEN = 0, 1
F32, F64 = 0, 1
GMRES_REFERENCE, GMRES_RESTARTED, FGMRES_LEARNED, FGMRES_MIXED = 0, 1, 2, 3

EXPORTS = [
    "pic_create", "pic_destroy", "pic_last_error", "pic_stream", "pic_add_species", "pic_upload_particles",
    "pic_append_particles",
    "pic_download_particles", "pic_upload_fields", "pic_download_fields", "pic_tristan_evaluate_b_half_step",
    "pic_move_particles", "pic_tristan_update_flux", "pic_tristan_evaluate_e", "pic_buneman_step",
    "pic_update_electromagnetic_parameters", "pic_evaluate_electric_field", "pic_evaluate_magnetic_field",
    "pic_update_fields", "pic_implicit_step", "pic_download_moments", "pic_maxwell_apply",
    "pic_maxwell_apply_transpose", "pic_maxwell_solve",
    "pic_sort_particles", "pic_download_permutation", "pic_energy", "pic_profile", "pic_energy_noalloc",
    "pic_fill_species", "pic_nn_param_count", "pic_nn_init", "pic_nn_set_params", "pic_nn_get_params",
    "pic_nn_train", "pic_nn_record", "pic_nn_record_count", "pic_nn_wait_limit", "pic_nn_forward", "pic_nn_loss_grad", "pic_update_density_parameters", "pic_download_density",
    "pic_save_checkpoint", "pic_load_checkpoint",
]
PHASES = ["sort", "fields", "push_deposit", "assemble", "moments", "solve", "mover", "deposit"]


class PicError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Config(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double), ("dt", C.c_double),
                ("theta", C.c_double), ("eta", C.c_double), ("cfix", C.c_double),
                ("solver", C.c_int), ("particle_real", C.c_int), ("field_real", C.c_int),
                ("pressure_compat", C.c_int), ("sort_every", C.c_int), ("tile", C.c_int * 3),
                ("max_species", C.c_int), ("smoothing_count", C.c_int), ("smoothing_parameter", C.c_double),
                ("boundary_x", C.c_int), ("e_right", C.c_double * 3), ("b_right", C.c_double * 3)]


class SolveOpts(C.Structure):
    _fields_ = [("method", C.c_int), ("restart", C.c_int), ("max_iter", C.c_int), ("tol", C.c_double),
                ("inner", C.c_int)]


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int), ("restarts", C.c_int), ("used_fallback", C.c_int),
                ("rel_residual", C.c_double), ("seconds", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class TrainOpts(C.Structure):
    _fields_ = [("steps", C.c_int), ("batch", C.c_int), ("lr", C.c_double), ("seed", C.c_ulonglong),
                ("smooth_max", C.c_int), ("source", C.c_int), ("supervised_weight", C.c_double)]


class TrainInfo(C.Structure):
    _fields_ = [("first_loss", C.c_double), ("last_loss", C.c_double), ("seconds", C.c_double), ("steps", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None
_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)


def library_path() -> str:
    return LIB_PATH


def load_library(path: str | None = None):
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with python -m picpp_gb300.build")
    L = C.CDLL(path)
    vp = C.c_void_p
    L.pic_create.argtypes = [C.POINTER(Config), C.POINTER(vp)]
    L.pic_destroy.argtypes = [vp]
    L.pic_last_error.argtypes = [vp]
    L.pic_last_error.restype = C.c_char_p
    L.pic_stream.argtypes = [vp]
    L.pic_stream.restype = vp
    L.pic_add_species.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_long, _ip]
    L.pic_upload_particles.argtypes = [vp, C.c_int, C.c_long, _ip, _dp, _dp, _dp, _dp, _dp, _dp, _ip]
    L.pic_append_particles.argtypes = [vp, C.c_int, C.c_long, _ip, _dp, _dp, _dp, _dp, _dp, _dp, _ip]
    L.pic_download_particles.argtypes = [vp, C.c_int, C.POINTER(C.c_long), _ip, _dp, _dp, _dp, _dp, _dp, _dp, _ip]
    L.pic_upload_fields.argtypes = [vp, _dp, _dp]
    L.pic_download_fields.argtypes = [vp, _dp, _dp, _dp]
    for name in ("pic_tristan_evaluate_b_half_step", "pic_move_particles", "pic_tristan_update_flux",
                 "pic_tristan_evaluate_e", "pic_update_electromagnetic_parameters", "pic_evaluate_magnetic_field",
                 "pic_update_fields", "pic_sort_particles"):
        getattr(L, name).argtypes = [vp]
    L.pic_buneman_step.argtypes = [vp, C.c_int]
    L.pic_evaluate_electric_field.argtypes = [vp, C.POINTER(SolveOpts), C.POINTER(SolveInfo)]
    L.pic_implicit_step.argtypes = [vp, C.POINTER(SolveOpts), C.POINTER(SolveInfo)]
    L.pic_download_moments.argtypes = [vp, _dp, _dp, _dp, _dp]
    L.pic_maxwell_apply.argtypes = [vp, _dp, _dp, _dp]
    L.pic_maxwell_apply_transpose.argtypes = [vp, _dp, _dp, _dp]
    L.pic_maxwell_solve.argtypes = [vp, _dp, _dp, _dp, C.POINTER(SolveOpts), C.POINTER(SolveInfo)]
    L.pic_download_permutation.argtypes = [vp, C.c_int, C.POINTER(C.c_long), _ip]
    L.pic_energy.argtypes = [vp, _dp]
    L.pic_profile.argtypes = [vp, C.c_int, _dp, C.POINTER(C.c_long)]
    L.pic_fill_species.argtypes = [vp, C.c_int, C.c_int, C.c_ulonglong, C.c_double, C.c_double, C.c_int]
    ptrs = C.POINTER(C.c_void_p)
    L.pic_energy_noalloc.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, vp, vp, C.c_int,
                                     C.POINTER(C.c_long), _dp, _dp, ptrs, ptrs, ptrs, vp, _dp]
    L.pic_save_checkpoint.argtypes = [vp, C.c_char_p]
    L.pic_load_checkpoint.argtypes = [vp, C.c_char_p]
    L.pic_update_density_parameters.argtypes = [vp]
    L.pic_download_density.argtypes = [vp, C.c_int, _dp, _dp, _dp, _dp]
    L.pic_nn_param_count.argtypes = []
    L.pic_nn_param_count.restype = C.c_long
    L.pic_nn_init.argtypes = [vp, C.c_ulonglong]
    L.pic_nn_set_params.argtypes = [vp, _fp]
    L.pic_nn_get_params.argtypes = [vp, _fp]
    L.pic_nn_train.argtypes = [vp, C.POINTER(TrainOpts), C.POINTER(TrainInfo)]
    L.pic_nn_record.argtypes = [vp, C.c_int]
    L.pic_nn_wait_limit.argtypes = [vp, C.c_uint]
    L.pic_nn_record_count.argtypes = [vp, C.POINTER(C.c_int)]
    L.pic_nn_forward.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, _fp, _fp]
    L.pic_nn_loss_grad.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, _fp, _fp, _dp, _fp]
    for name in EXPORTS:
        if name not in ("pic_last_error", "pic_stream", "pic_nn_param_count"):
            getattr(L, name).restype = C.c_int
    _lib = L
    return L


def _d(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def _f(a):
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(_fp)


def _i(a):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


def solve_opts(method=GMRES_REFERENCE, restart=30, max_iter=50, tol=1e-8, inner=0) -> SolveOpts:
    return SolveOpts(method, restart, max_iter, tol, inner)


class GpuSimulation:
    """The reference's ``Simulation`` hot-path methods (PIC++/simulation.h)
    on one GPU.  State goes in with ``upload_*`` and comes back with
    ``download_*``; each method mirrors the member function of that name."""

    def __init__(self, box, solver=BUNEMAN, particle_real=F32, field_real=None, pressure_compat=1,
                 sort_every=1, tile=(8, 8, 8), max_species=8, smoothing_count=0, smoothing_parameter=0.5,
                 boundary_x=BOUNDARY_PERIODIC, e_right=(0.0, 0.0, 0.0), b_right=(0.0, 0.0, 0.0)):
        """boundary_x = BOUNDARY_WALL_OPEN: conductor wall at x = 0 and open
        boundary at x = (nx - 2) dx with the constant fields e_right, b_right
        (include/picpp_gb300.h, pic_boundary_x)."""
        self.L = load_library()
        self.box = box
        cfg = Config()
        cfg.nx, cfg.ny, cfg.nz = box.nx, box.ny, box.nz
        cfg.dx, cfg.dy, cfg.dz, cfg.dt = box.dx, box.dy, box.dz, box.dt
        cfg.theta, cfg.eta, cfg.cfix = box.theta, box.eta, box.cfix
        cfg.solver = solver
        cfg.particle_real = particle_real
        cfg.field_real = particle_real if field_real is None else field_real
        cfg.pressure_compat = pressure_compat
        cfg.sort_every = sort_every
        cfg.smoothing_count = smoothing_count
        cfg.smoothing_parameter = smoothing_parameter
        cfg.tile[0], cfg.tile[1], cfg.tile[2] = tile
        cfg.max_species = max_species
        cfg.boundary_x = boundary_x
        for a in range(3):
            cfg.e_right[a] = e_right[a]
            cfg.b_right[a] = b_right[a]
        self.cfg = cfg
        self.ctx = C.c_void_p()
        st = self.L.pic_create(C.byref(cfg), C.byref(self.ctx))
        if st != PIC_OK:
            raise PicError(st, "pic_create failed")
        self.solver = solver
        self.species = []
        self.last_solve = None

    # -------------------------------------------------------------- plumbing
    def _ck(self, st):
        if st != PIC_OK:
            raise PicError(st, self.L.pic_last_error(self.ctx).decode())
        return st

    def close(self):
        if self.ctx:
            self.L.pic_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return self.L.pic_stream(self.ctx)

    @property
    def N(self):
        return self.box.nx * self.box.ny * self.box.nz

    # -------------------------------------------------------------- state
    def add_species(self, q, m, w, capacity) -> int:
        sid = C.c_int()
        self._ck(self.L.pic_add_species(self.ctx, q, m, w, int(capacity), C.byref(sid)))
        self.species.append(dict(q=q, m=m, w=w))
        return sid.value

    def upload_particles(self, sid, sp, ids=None):
        n = len(sp["cell"])
        arrs = [np.ascontiguousarray(sp[k], dtype=np.float64) for k in ("ox", "oy", "oz", "px", "py", "pz")]
        cell = np.ascontiguousarray(sp["cell"], dtype=np.int32)
        ids = None if ids is None else np.ascontiguousarray(ids, dtype=np.int32)
        self._ck(self.L.pic_upload_particles(self.ctx, sid, n, _i(cell), *[_d(a) for a in arrs], _i(ids)))

    def append_particles(self, sid, sp, ids=None):
        """Adds the particles of sp after the species' current ones
        (injection at an open boundary)."""
        n = len(sp["cell"])
        arrs = [np.ascontiguousarray(sp[k], dtype=np.float64) for k in ("ox", "oy", "oz", "px", "py", "pz")]
        cell = np.ascontiguousarray(sp["cell"], dtype=np.int32)
        ids = None if ids is None else np.ascontiguousarray(ids, dtype=np.int32)
        self._ck(self.L.pic_append_particles(self.ctx, sid, n, _i(cell), *[_d(a) for a in arrs], _i(ids)))

    def download_particles(self, sid, with_ids=True):
        n = C.c_long()
        self._ck(self.L.pic_download_particles(self.ctx, sid, C.byref(n), None, None, None, None, None, None, None,
                                               None))
        n = n.value
        out = {k: np.empty(n) for k in ("ox", "oy", "oz", "px", "py", "pz")}
        out["cell"] = np.empty(n, dtype=np.int32)
        ids = np.empty(n, dtype=np.int32) if with_ids else None
        self._ck(self.L.pic_download_particles(self.ctx, sid, C.byref(C.c_long()), _i(out["cell"]),
                                               *[_d(out[k]) for k in ("ox", "oy", "oz", "px", "py", "pz")], _i(ids)))
        if with_ids:
            out["id"] = ids
        return out

    def fill_species(self, sid, ppc, seed, theta, drift_gamma=1.0, alternate_drift=False):
        """Device-side seeded loading (pic_fill_species).  alternate_drift:
        False / 0 drift along +x, True / 1 every other particle along -x,
        -1 every particle along -x."""
        mode = int(alternate_drift) if not isinstance(alternate_drift, bool) else (1 if alternate_drift else 0)
        self._ck(self.L.pic_fill_species(self.ctx, sid, int(ppc), int(seed), float(theta), float(drift_gamma), mode))

    def upload_state(self, state):
        """Species (adding them on first use) and fields of an initstate.State."""
        for s, sp in enumerate(state.species):
            if s >= len(self.species):
                self.add_species(sp["q"], sp["m"], sp["w"], len(sp["cell"]))
            self.upload_particles(s, sp)
        self.upload_fields(state.E, state.B)

    def upload_fields(self, E, B):
        E = None if E is None else np.ascontiguousarray(E, dtype=np.float64).reshape(-1)
        B = None if B is None else np.ascontiguousarray(B, dtype=np.float64).reshape(-1)
        self._ck(self.L.pic_upload_fields(self.ctx, _d(E), _d(B)))

    def download_fields(self):
        shape = (3, self.box.nz, self.box.ny, self.box.nx)
        E, B, J = np.empty(shape), np.empty(shape), np.empty(shape)
        self._ck(self.L.pic_download_fields(self.ctx, _d(E), _d(B), _d(J)))
        return E, B, J

    # -------------------------------------------------------------- explicit phases
    def tristanEvaluateBhalfStep(self):
        self._ck(self.L.pic_tristan_evaluate_b_half_step(self.ctx))

    def moveParticles(self):
        self._ck(self.L.pic_move_particles(self.ctx))

    def tristanUpdateFlux(self):
        self._ck(self.L.pic_tristan_update_flux(self.ctx))

    def tristanEvaluateE(self):
        self._ck(self.L.pic_tristan_evaluate_e(self.ctx))

    def buneman_step(self, nsteps=1):
        self._ck(self.L.pic_buneman_step(self.ctx, nsteps))

    # -------------------------------------------------------------- implicit phases
    def updateElectroMagneticParameters(self):
        self._ck(self.L.pic_update_electromagnetic_parameters(self.ctx))

    def evaluateElectricField(self, opts=None):
        info = SolveInfo()
        opts = opts or solve_opts()
        st = self.L.pic_evaluate_electric_field(self.ctx, C.byref(opts), C.byref(info))
        self.last_solve = info.as_dict()
        self._ck(st)
        return self.last_solve

    def evaluateMagneticField(self):
        self._ck(self.L.pic_evaluate_magnetic_field(self.ctx))

    def updateFields(self):
        self._ck(self.L.pic_update_fields(self.ctx))

    def implicit_step(self, opts=None):
        info = SolveInfo()
        opts = opts or solve_opts()
        st = self.L.pic_implicit_step(self.ctx, C.byref(opts), C.byref(info))
        self.last_solve = info.as_dict()
        self._ck(st)
        return self.last_solve

    def download_moments(self):
        N = self.N
        ext = [n + 1 if n > 1 else 1 for n in (self.box.nx, self.box.ny, self.box.nz)]
        J, mu, rhs = np.empty(3 * N), np.empty(9 * N), np.empty(3 * N)
        rho = np.empty(ext[0] * ext[1] * ext[2])
        self._ck(self.L.pic_download_moments(self.ctx, _d(J), _d(mu), _d(rho), _d(rhs)))
        return J, mu, rho, rhs

    def maxwell_apply(self, mu, x):
        mu = np.ascontiguousarray(mu, dtype=np.float64)
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        self._ck(self.L.pic_maxwell_apply(self.ctx, _d(mu), _d(x), _d(y)))
        return y

    def maxwell_apply_transpose(self, mu, y):
        mu = np.ascontiguousarray(mu, dtype=np.float64)
        y = np.ascontiguousarray(y, dtype=np.float64)
        out = np.empty_like(y)
        self._ck(self.L.pic_maxwell_apply_transpose(self.ctx, _d(mu), _d(y), _d(out)))
        return out

    def maxwell_solve(self, mu, rhs, opts=None):
        mu = np.ascontiguousarray(mu, dtype=np.float64)
        rhs = np.ascontiguousarray(rhs, dtype=np.float64)
        x = np.empty_like(rhs)
        info = SolveInfo()
        opts = opts or solve_opts()
        st = self.L.pic_maxwell_solve(self.ctx, _d(mu), _d(rhs), _d(x), C.byref(opts), C.byref(info))
        self.last_solve = info.as_dict()
        self._ck(st)
        return x, self.last_solve

    # -------------------------------------------------------------- checkpoint
    def save_checkpoint(self, path):
        self._ck(self.L.pic_save_checkpoint(self.ctx, os.fsencode(path)))

    def load_checkpoint(self, path):
        self._ck(self.L.pic_load_checkpoint(self.ctx, os.fsencode(path)))

    # -------------------------------------------------------------- diagnostics
    def updateDensityParameters(self):
        self._ck(self.L.pic_update_density_parameters(self.ctx))

    def download_density(self, sid):
        """(conc[N], energy[N], vel[3][N], rho[N]) of one species (rho: all)."""
        N = self.box.ncells
        conc, en, vel, rho = np.empty(N), np.empty(N), np.empty(3 * N), np.empty(N)
        self._ck(self.L.pic_download_density(self.ctx, sid, _d(conc), _d(en), _d(vel), _d(rho)))
        return conc, en, vel.reshape(3, N), rho

    # -------------------------------------------------------------- learned preconditioner
    def nn_init(self, seed=1):
        self._ck(self.L.pic_nn_init(self.ctx, seed))

    def nn_set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.L.pic_nn_param_count()
        self._ck(self.L.pic_nn_set_params(self.ctx, _f(p)))

    def nn_get_params(self):
        p = np.empty(self.L.pic_nn_param_count(), dtype=np.float32)
        self._ck(self.L.pic_nn_get_params(self.ctx, _f(p)))
        return p

    def nn_train(self, steps=200, batch=1, lr=1e-3, seed=1, smooth_max=4, source=0, supervised_weight=0.5):
        """source 0: random fields on the current operator; 1: the recorded
        (b, mu, x) triples (nn_record), loss weight supervised_weight on
        |z - x|^2 / |x|^2 against the residual |A z - b|^2 / |b|^2."""
        info = TrainInfo()
        opts = TrainOpts(steps, batch, lr, seed, smooth_max, source, supervised_weight)
        self._ck(self.L.pic_nn_train(self.ctx, C.byref(opts), C.byref(info)))
        return info.as_dict()

    def nn_wait_limit(self, polls):
        """Bound of the convolutions' MMA-completion wait (0: built-in)."""
        self._ck(self.L.pic_nn_wait_limit(self.ctx, int(polls)))

    def nn_record(self, capacity):
        """Keep the (b, mu, x) triples of the next plain field solves, the
        first `capacity` of them (0 stops and frees them)."""
        self._ck(self.L.pic_nn_record(self.ctx, int(capacity)))

    def nn_record_count(self) -> int:
        n = C.c_int()
        self._ck(self.L.pic_nn_record_count(self.ctx, C.byref(n)))
        return n.value

    def nn_forward(self, x0):
        x0 = np.ascontiguousarray(x0, dtype=np.float32)
        n, d, h, w, c = x0.shape
        assert c == 16
        out = np.empty_like(x0)
        self._ck(self.L.pic_nn_forward(self.ctx, n, d, h, w, _f(x0), _f(out)))
        return out

    def nn_loss_grad(self, x0, target):
        x0 = np.ascontiguousarray(x0, dtype=np.float32)
        target = np.ascontiguousarray(target, dtype=np.float32)
        n, d, h, w, _ = x0.shape
        loss = np.zeros(1)
        grad = np.empty(self.L.pic_nn_param_count(), dtype=np.float32)
        self._ck(self.L.pic_nn_loss_grad(self.ctx, n, d, h, w, _f(x0), _f(target), _d(loss), _f(grad)))
        return float(loss[0]), grad

    # -------------------------------------------------------------- order, diagnostics
    def sort(self):
        self._ck(self.L.pic_sort_particles(self.ctx))

    def download_permutation(self, sid):
        n = C.c_long()
        self._ck(self.L.pic_download_permutation(self.ctx, sid, C.byref(n), None))
        perm = np.empty(n.value, dtype=np.int32)
        self._ck(self.L.pic_download_permutation(self.ctx, sid, C.byref(n), _i(perm)))
        return perm

    def updateEnergy(self):
        out = np.zeros(6)
        self._ck(self.L.pic_energy(self.ctx, _d(out)))
        return out

    def profile(self, enable: bool):
        """Starts (clearing) or stops per-phase device timing; returns the
        accumulated {phase: ms} and the number of kernels launched."""
        ms = np.zeros(len(PHASES))
        n = C.c_long()
        self._ck(self.L.pic_profile(self.ctx, 1 if enable else 0, _d(ms), C.byref(n)))
        return dict(zip(PHASES, ms.tolist())), n.value
