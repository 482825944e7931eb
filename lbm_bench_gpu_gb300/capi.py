"""ctypes bindings of liblbm_gb300.so (the C-ABI in include/lbm_gb300.h).

This is the Python face of the same entry points a C, C++ or Fortran driver
calls.  There is no fallback: if the library is missing or cannot be loaded,
``load()`` raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "liblbm_gb300.so"

LBM_OK, LBM_EINVAL, LBM_ENOMEM, LBM_ECUDA, LBM_ENAN, LBM_ETIMEOUT, LBM_EIO, LBM_ESTATE = range(8)
STORAGE = {"fp32": 0, "fp16": 1, "bf16": 2}

# Every symbol include/lbm_gb300.h declares.
EXPORTS = [
    "lbm_read_inputs", "lbm_derive", "lbm_init", "lbm_init_bubbles", "lbm_step", "lbm_stats",
    "lbm_get_dist", "lbm_set_dist", "lbm_steps_done", "lbm_stream", "lbm_sync", "lbm_destroy",
    "lbm_strerror", "lbm_last_error", "lbm_stats_noalloc", "lbm_step_adjoint",
    "lbm_objective", "lbm_stats_fields", "lbm_pressure", "lbm_device_name", "lbm_adjoint_release",
    "lbm_wait_selftest", "lbm_adjoint_forward_steps", "lbm_state_bytes", "lbm_save_state", "lbm_load_state",
    "lbm_split_z", "lbm_merge_z", "lbm_slab_step", "lbm_halo_bytes", "lbm_halo_pack", "lbm_halo_unpack",
    "lbm_slab_step_local", "lbm_stats_raw", "lbm_stats_combine", "lbm_slab_stats", "lbm_slab_maxabs",
    "lbm_slab_init_bubbles", "lbm_slab_step_interior", "lbm_slab_step_boundary",
    "lbm_adjoint_forward_steps_tiers",
]
OBJECTIVES = {"light_uz_mean": 0, "light_z_centroid": 1}


class Params(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("block_x", C.c_int), ("block_y", C.c_int),
        ("rhoL", C.c_float), ("rhoH", C.c_float),
        ("tauRho", C.c_float), ("tauPhi", C.c_float),
        ("width", C.c_float), ("sigma", C.c_float), ("Gamma", C.c_float),
        ("Eo", C.c_float), ("rc0", C.c_float),
        ("storage", C.c_int), ("device", C.c_int), ("compat", C.c_int),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class Run(C.Structure):
    _fields_ = [("max_step", C.c_int), ("relax_step", C.c_int), ("save", C.c_int), ("stat", C.c_int)]


class Derived(C.Structure):
    _fields_ = [(k, C.c_float) for k in (
        "phiStar", "phiStarSq", "invTauRho", "invTauRhoOne", "invTauRhoHalf", "eta", "eta2", "invEta2",
        "invTauPhi", "invTauPhiOne", "alpha", "alpha4", "kappa", "gravity", "grav",
        "K0", "K1", "K2", "KC0", "KC1", "KC2")]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class StatsOut(C.Structure):
    _fields_ = [("step", C.c_longlong)] + [(k, C.c_double) for k in (
        "umax", "vol", "ux_av", "uy_av", "uz_av", "ref", "p_in", "p_out", "p_dif", "p_err",
        "phi_sum", "rho_sum", "mom_x", "mom_y", "mom_z", "vol_full", "umax_full")] + [("nonfinite", C.c_longlong)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class AdjointOpts(C.Structure):
    _fields_ = [("objective", C.c_int), ("nsteps", C.c_int), ("window", C.c_int), ("grav", C.c_float),
                ("checkpoint_bytes", C.c_double), ("host_checkpoint_bytes", C.c_double)]


class AdjointOut(C.Structure):
    _fields_ = [("J", C.c_double), ("dJ_dgrav", C.c_double), ("dJ_dphi0", C.POINTER(C.c_float)),
                ("slots", C.c_int), ("forward_steps", C.c_longlong), ("adjoint_steps", C.c_longlong),
                ("seconds", C.c_double), ("checkpoint_bytes_used", C.c_double), ("host_slots", C.c_int)]


class LbmError(RuntimeError):
    def __init__(self, code: int, what: str, detail: str):
        super().__init__(f"{what}: status {code} ({detail})")
        self.code = code


_lib: C.CDLL | None = None

_F = C.POINTER(C.c_float)


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load liblbm_gb300.so (raises OSError if it is missing)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    # LBM_GB300_LIB selects another build of the library (the tests' checked build)
    p = Path(path) if path else Path(os.environ.get("LBM_GB300_LIB", LIB_PATH))
    if not p.exists():
        raise OSError(f"{p} not found: build it with `python -m lbm_bench_gpu_gb300.build`")
    lib = C.CDLL(str(p))
    lib.lbm_read_inputs.argtypes = [C.c_char_p, C.POINTER(Params), C.POINTER(Run), _F, C.c_int, C.POINTER(C.c_int)]
    lib.lbm_derive.argtypes = [C.POINTER(Params), C.POINTER(Derived)]
    lib.lbm_init.argtypes = [C.POINTER(C.c_void_p), C.POINTER(Params), _F, _F, _F, _F, _F, _F]
    lib.lbm_init_bubbles.argtypes = [C.POINTER(C.c_void_p), C.POINTER(Params), _F, C.c_int]
    lib.lbm_step.argtypes = [C.c_void_p, C.c_int, C.c_float]
    lib.lbm_stats.argtypes = [C.c_void_p, C.POINTER(StatsOut), _F, _F, _F, _F, _F]
    lib.lbm_get_dist.argtypes = [C.c_void_p, _F, _F]
    lib.lbm_set_dist.argtypes = [C.c_void_p, _F, _F]
    lib.lbm_stats_noalloc.argtypes = [C.POINTER(Params), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_void_p]
    lib.lbm_step_adjoint.argtypes = [C.c_void_p, C.POINTER(AdjointOpts), C.POINTER(AdjointOut)]
    lib.lbm_objective.argtypes = [C.c_void_p, C.POINTER(AdjointOpts), C.POINTER(C.c_double)]
    lib.lbm_adjoint_release.argtypes = [C.c_void_p]
    lib.lbm_wait_selftest.argtypes = [C.c_void_p]
    lib.lbm_adjoint_forward_steps.argtypes = [C.c_longlong, C.c_int]
    lib.lbm_adjoint_forward_steps.restype = C.c_longlong
    lib.lbm_adjoint_forward_steps_tiers.argtypes = [C.c_longlong, C.c_int, C.c_longlong]
    lib.lbm_adjoint_forward_steps_tiers.restype = C.c_longlong
    lib.lbm_state_bytes.argtypes = [C.c_void_p]
    lib.lbm_state_bytes.restype = C.c_longlong
    lib.lbm_save_state.argtypes = [C.c_void_p, C.c_void_p]
    lib.lbm_load_state.argtypes = [C.c_void_p, C.c_void_p]
    lib.lbm_stats_fields.argtypes = [C.c_void_p, C.POINTER(StatsOut), _F, _F, _F, _F, _F]
    lib.lbm_pressure.argtypes = [C.c_void_p, _F]
    lib.lbm_device_name.argtypes = [C.c_int, C.c_char_p, C.c_int, C.POINTER(C.c_double)]
    lib.lbm_steps_done.argtypes = [C.c_void_p]
    lib.lbm_steps_done.restype = C.c_longlong
    lib.lbm_stream.argtypes = [C.c_void_p]
    lib.lbm_stream.restype = C.c_void_p
    lib.lbm_sync.argtypes = [C.c_void_p]
    lib.lbm_destroy.argtypes = [C.c_void_p]
    lib.lbm_destroy.restype = None
    lib.lbm_strerror.argtypes = [C.c_int]
    lib.lbm_strerror.restype = C.c_char_p
    lib.lbm_last_error.argtypes = []
    lib.lbm_last_error.restype = C.c_char_p
    _V, _I, _D = C.POINTER(C.c_void_p), C.POINTER(C.c_int), C.POINTER(C.c_double)
    lib.lbm_split_z.argtypes = [C.c_void_p, C.c_int, _I, _I, _V]
    lib.lbm_merge_z.argtypes = [_V, C.c_int, C.c_void_p]
    lib.lbm_slab_maxabs.argtypes = [C.POINTER(Params), _F, C.c_int, C.c_int, C.c_int, _F]
    lib.lbm_slab_init_bubbles.argtypes = [C.POINTER(C.c_void_p), C.POINTER(Params), _F, C.c_int, C.c_int, C.c_int,
                                          _F]
    lib.lbm_slab_step.argtypes = [_V, C.c_int, C.c_int, C.c_float]
    lib.lbm_halo_bytes.argtypes = [C.c_void_p, C.c_int]
    lib.lbm_halo_bytes.restype = C.c_longlong
    lib.lbm_halo_pack.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    lib.lbm_halo_unpack.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    lib.lbm_slab_step_local.argtypes = [C.c_void_p, C.c_float]
    lib.lbm_slab_step_interior.argtypes = [C.c_void_p, C.c_float]
    lib.lbm_slab_step_boundary.argtypes = [C.c_void_p, C.c_float]
    lib.lbm_stats_raw.argtypes = [C.c_void_p, _D]
    lib.lbm_stats_combine.argtypes = [C.POINTER(Params), C.c_longlong, _D, C.c_int, C.POINTER(StatsOut)]
    lib.lbm_slab_stats.argtypes = [_V, C.c_int, C.POINTER(StatsOut)]
    if path is None:
        _lib = lib
    return lib


def check(code: int, what: str) -> None:
    if code != LBM_OK:
        lib = load()
        detail = lib.lbm_last_error().decode() or lib.lbm_strerror(code).decode()
        raise LbmError(code, what, detail)


def fptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(_F)


def make_params(nx: int, ny: int, nz: int, *, rhoL: float, rhoH: float, tauRho: float, tauPhi: float,
                width: float, sigma: float, Gamma: float, Eo: float = 0.0, rc0: float = 0.0,
                block_x: int = 32, block_y: int = 8, storage: str = "fp32", device: int = 0,
                compat: bool = False) -> Params:
    p = Params()
    p.nx, p.ny, p.nz = nx, ny, nz
    p.block_x, p.block_y = block_x, block_y
    p.rhoL, p.rhoH, p.tauRho, p.tauPhi = rhoL, rhoH, tauRho, tauPhi
    p.width, p.sigma, p.Gamma, p.Eo, p.rc0 = width, sigma, Gamma, Eo, rc0
    p.storage, p.device, p.compat = STORAGE[storage], device, int(compat)
    return p


def adjoint_forward_steps(nsteps: int, slots: int, host_slots: int = 0) -> int:
    """lbm_adjoint_forward_steps(_tiers): forward steps of the checkpointing
    schedule with `slots` device and `host_slots` host checkpoints (not run)."""
    lib = load()
    if host_slots:
        return int(lib.lbm_adjoint_forward_steps_tiers(int(nsteps), int(slots), int(host_slots)))
    return int(lib.lbm_adjoint_forward_steps(int(nsteps), int(slots)))


def read_inputs(directory: str | os.PathLike, max_bubbles: int = 4096):
    """Parse properties.in / discrete.in with the library's reader.

    Returns (Params, Run, bubbles (nb x 4 float32))."""
    lib = load()
    p, r = Params(), Run()
    buf = np.zeros((max_bubbles, 4), np.float32)
    nb = C.c_int(0)
    check(lib.lbm_read_inputs(str(directory).encode(), C.byref(p), C.byref(r), fptr(buf), max_bubbles,
                              C.byref(nb)), "lbm_read_inputs")
    if nb.value > max_bubbles:
        return read_inputs(directory, nb.value)
    return p, r, buf[: nb.value].copy()


def derive(p: Params) -> Derived:
    d = Derived()
    check(load().lbm_derive(C.byref(p), C.byref(d)), "lbm_derive")
    return d


LBM_HALO_PRE, LBM_HALO_POST, LBM_HALO_PHI = 0, 1, 2


def stats_combine(params: Params, steps: int, raw) -> dict:
    """lbm_stats_combine: lbm_stats_out of a whole box from per-slab raw statistics."""
    r = np.ascontiguousarray(raw, np.float64).reshape(-1, 16)
    s = StatsOut()
    check(load().lbm_stats_combine(C.byref(params), int(steps), r.ctypes.data_as(C.POINTER(C.c_double)), len(r),
                                   C.byref(s)), "lbm_stats_combine")
    return s.as_dict()


class Lattice:
    """One simulation context on one GPU (owns all its device memory)."""

    def __init__(self, handle: C.c_void_p, params: Params):
        self._h = handle
        self.params = params
        self.shape = (params.nz, params.ny, params.nx)
        self.n = params.nx * params.ny * params.nz

    @classmethod
    def from_fields(cls, params: Params, phi, rho, ux=None, uy=None, uz=None, phi_ghost=None) -> "Lattice":
        lib = load()
        h = C.c_void_p()
        arrs = [None if a is None else np.ascontiguousarray(a, np.float32) for a in (phi, rho, ux, uy, uz, phi_ghost)]
        check(lib.lbm_init(C.byref(h), C.byref(params), *[fptr(a) for a in arrs]), "lbm_init")
        return cls(h, params)

    @classmethod
    def from_bubbles(cls, params: Params, bubbles) -> "Lattice":
        lib = load()
        h = C.c_void_p()
        b = np.ascontiguousarray(bubbles, np.float32).reshape(-1, 4)
        check(lib.lbm_init_bubbles(C.byref(h), C.byref(params), fptr(b) if len(b) else None, len(b)),
              "lbm_init_bubbles")
        return cls(h, params)

    def step(self, nsteps: int, grav: float = 0.0) -> None:
        check(load().lbm_step(self._h, int(nsteps), float(grav)), "lbm_step")

    def stats(self, fields: bool = False, allow_nan: bool = False):
        """Return (stats dict, fields dict or None)."""
        s = StatsOut()
        arrs = [np.empty(self.shape, np.float32) for _ in range(5)] if fields else [None] * 5
        code = load().lbm_stats(self._h, C.byref(s), *[fptr(a) for a in arrs])
        if not (allow_nan and code == LBM_ENAN):
            check(code, "lbm_stats")
        out = dict(zip(("phi", "rho", "ux", "uy", "uz"), arrs)) if fields else None
        return s.as_dict(), out

    def fields(self) -> dict:
        arrs = [np.empty(self.shape, np.float32) for _ in range(5)]
        check(load().lbm_stats(self._h, None, *[fptr(a) for a in arrs]), "lbm_stats")
        return dict(zip(("phi", "rho", "ux", "uy", "uz"), arrs))

    def stats_of(self, phi, rho, ux, uy, uz, allow_nan: bool = False) -> dict:
        """lbm_stats_fields: the statistics of the given host fields."""
        s = StatsOut()
        arrs = [np.ascontiguousarray(a, np.float32) for a in (phi, rho, ux, uy, uz)]
        code = load().lbm_stats_fields(self._h, C.byref(s), *[fptr(a) for a in arrs])
        if not (allow_nan and code == LBM_ENAN):
            check(code, "lbm_stats_fields")
        return s.as_dict()

    def pressure(self) -> np.ndarray:
        """lbm_pressure: the pressure field of the current phi and rho."""
        p = np.empty(self.shape, np.float32)
        check(load().lbm_pressure(self._h, fptr(p)), "lbm_pressure")
        return p

    def dist(self):
        f = np.empty((7,) + self.shape, np.float32)
        g = np.empty((19,) + self.shape, np.float32)
        check(load().lbm_get_dist(self._h, fptr(f), fptr(g)), "lbm_get_dist")
        return f, g

    def set_dist(self, f, g) -> None:
        f = np.ascontiguousarray(f, np.float32)
        g = np.ascontiguousarray(g, np.float32)
        check(load().lbm_set_dist(self._h, fptr(f), fptr(g)), "lbm_set_dist")

    def adjoint(self, nsteps: int, grav: float, objective: str = "light_uz_mean", window: int = 1,
                checkpoint_bytes: float = 0.0, want_phi0: bool = True, host_checkpoint_bytes: float = 0.0) -> dict:
        """lbm_step_adjoint: J, dJ/dgrav and dJ/dphi0 over nsteps from the initial state
        (host_checkpoint_bytes > 0: a second checkpoint tier in pinned host memory)."""
        o = AdjointOpts(OBJECTIVES[objective], int(nsteps), int(window), float(grav), float(checkpoint_bytes),
                        float(host_checkpoint_bytes))
        out = AdjointOut()
        grad = np.zeros(self.shape, np.float32) if want_phi0 else None
        out.dJ_dphi0 = fptr(grad) if want_phi0 else None
        check(load().lbm_step_adjoint(self._h, C.byref(o), C.byref(out)), "lbm_step_adjoint")
        return {"J": out.J, "dJ_dgrav": out.dJ_dgrav, "dJ_dphi0": grad, "slots": out.slots,
                "forward_steps": out.forward_steps, "adjoint_steps": out.adjoint_steps, "seconds": out.seconds,
                "checkpoint_bytes_used": out.checkpoint_bytes_used, "host_slots": out.host_slots}

    def objective(self, nsteps: int, grav: float, objective: str = "light_uz_mean", window: int = 1) -> float:
        """lbm_objective: J alone over nsteps from the initial state (forward run)."""
        o = AdjointOpts(OBJECTIVES[objective], int(nsteps), int(window), float(grav), 0.0)
        J = C.c_double()
        check(load().lbm_objective(self._h, C.byref(o), C.byref(J)), "lbm_objective")
        return float(J.value)

    def save_state(self) -> np.ndarray:
        """lbm_save_state: the context's native state as a byte array (checkpoint)."""
        buf = np.empty(int(load().lbm_state_bytes(self._h)), np.uint8)
        check(load().lbm_save_state(self._h, buf.ctypes.data_as(C.c_void_p)), "lbm_save_state")
        return buf

    def load_state(self, buf: np.ndarray) -> None:
        """lbm_load_state: restore a snapshot from save_state (resume)."""
        buf = np.ascontiguousarray(buf, dtype=np.uint8)
        check(load().lbm_load_state(self._h, buf.ctypes.data_as(C.c_void_p)), "lbm_load_state")

    def wait_selftest(self) -> int:
        """lbm_wait_selftest: the status code a timed-out bounded wait reports (LBM_ETIMEOUT)."""
        return int(load().lbm_wait_selftest(self._h))

    def adjoint_release(self) -> None:
        """lbm_adjoint_release: free the adjoint workspace and checkpoint pool kept in the context."""
        check(load().lbm_adjoint_release(self._h), "lbm_adjoint_release")

    @property
    def steps(self) -> int:
        return int(load().lbm_steps_done(self._h))

    @property
    def stream(self) -> int:
        return int(load().lbm_stream(self._h) or 0)

    def sync(self) -> None:
        check(load().lbm_sync(self._h), "lbm_sync")

    def close(self) -> None:
        if self._h:
            load().lbm_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Slabs:
    """A whole box held by z-slab contexts (lbm_split_z): slab k holds
    depths[k] consecutive planes, on devices[k] (default: the whole context's
    device); lbm_slab_step steps them together with their halo exchanges."""

    def __init__(self, whole: Lattice | None, depths, devices=None):
        self.n = len(depths)
        self.depths = list(depths)
        self._h = (C.c_void_p * self.n)()
        if whole is None:   # filled by from_bubbles
            return
        self.params = whole.params
        d = (C.c_int * self.n)(*[int(v) for v in depths])
        dev = (C.c_int * self.n)(*[int(v) for v in devices]) if devices is not None else None
        check(load().lbm_split_z(whole._h, self.n, d, dev, self._h), "lbm_split_z")

    @classmethod
    def from_bubbles(cls, p: Params, bubbles, depths, devices=None) -> "Slabs":
        """Each slab built on its own from the bubble list (lbm_slab_maxabs,
        the maxima reduced here as processes would with MPI_Allreduce(MAX),
        then lbm_slab_init_bubbles): no whole box on any device."""
        b = np.ascontiguousarray(bubbles, np.float32).reshape(-1, 4)
        z0s = np.concatenate([[0], np.cumsum(depths)[:-1]]).astype(int)
        per = []
        for k, (z0, d) in enumerate(zip(z0s, depths)):
            q = Params(**{**p.as_dict(), "device": devices[k] if devices is not None else p.device})
            m = np.zeros(26, np.float32)
            check(load().lbm_slab_maxabs(C.byref(q), fptr(b), len(b), int(z0), int(d), fptr(m)), "lbm_slab_maxabs")
            per.append((q, m))
        maxabs = np.max([m for _, m in per], axis=0).astype(np.float32)
        self = cls(None, depths)
        self.params = p
        for k, (z0, d) in enumerate(zip(z0s, depths)):
            h = C.c_void_p()
            check(load().lbm_slab_init_bubbles(C.byref(h), C.byref(per[k][0]), fptr(b), len(b), int(z0), int(d),
                                               fptr(maxabs)), "lbm_slab_init_bubbles")
            self._h[k] = h.value
        return self

    def step(self, nsteps: int, grav: float = 0.0) -> None:
        check(load().lbm_slab_step(self._h, self.n, int(nsteps), float(grav)), "lbm_slab_step")

    def stats(self) -> dict:
        s = StatsOut()
        check(load().lbm_slab_stats(self._h, self.n, C.byref(s)), "lbm_slab_stats")
        return s.as_dict()

    def raw_stats(self) -> np.ndarray:
        """lbm_stats_raw of every slab (after an LBM_HALO_PHI exchange by stats())."""
        out = np.zeros((self.n, 16), np.float64)
        for k in range(self.n):
            check(load().lbm_stats_raw(self._h[k], out[k].ctypes.data_as(C.POINTER(C.c_double))), "lbm_stats_raw")
        return out

    def merge_into(self, whole: Lattice) -> None:
        check(load().lbm_merge_z(self._h, self.n, whole._h), "lbm_merge_z")

    def handle(self, k: int):
        return self._h[k]

    def close(self) -> None:
        if self._h is not None:
            for k in range(self.n):
                if self._h[k]:
                    load().lbm_destroy(self._h[k])
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
