"""ctypes front-ends of the two CPU oracles (test infrastructure only).

* ``Oracle``  -- the FP64 restatement in zsc_oracle.c.
* ``RefCPU``  -- the reference's own kernels compiled for the host CPU
  (oracle/_ref/libzsc_ref.so, see oracle/build.py).

Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline and
reference legs use this module, and only as the oracle or the timed CPU
baseline -- never as the thing measured on the GPU.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import build as _build

_D = C.POINTER(C.c_double)
_Fp = C.POINTER(C.c_float)


def _dptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_D)


def _fptr(a):
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(_Fp)


_oracle_lib = None
_ref_lib = None


def oracle_lib() -> C.CDLL:
    global _oracle_lib
    if _oracle_lib is None:
        lib = C.CDLL(str(_build.build_oracle()))
        lib.zo_create.argtypes = [C.c_int, C.c_int, C.c_int, _D]
        lib.zo_create.restype = C.c_void_p
        lib.zo_destroy.argtypes = [C.c_void_p]
        lib.zo_constants.argtypes = [C.c_void_p, _D]
        lib.zo_bubble_phi.argtypes = [C.c_void_p, _Fp, C.c_int, _D]
        lib.zo_init.argtypes = [C.c_void_p, _D, _D, _D, _D, _D, _D]
        lib.zo_step.argtypes = [C.c_void_p, C.c_int, C.c_double]
        lib.zo_moments.argtypes = [C.c_void_p, _D, _D, _D, _D, _D]
        lib.zo_dist.argtypes = [C.c_void_p, _D, _D]
        lib.zo_set_dist.argtypes = [C.c_void_p, _D, _D]
        lib.zo_compare.argtypes = [C.c_void_p, _Fp, _Fp, _Fp, _D]
        lib.zo_slab_create.argtypes = [C.c_int, C.c_int, C.c_int, _D]
        lib.zo_slab_create.restype = C.c_void_p
        for name in ("zo_slab_moments", "zo_slab_stream"):
            getattr(lib, name).argtypes = [C.c_void_p]
        lib.zo_slab_collide.argtypes = [C.c_void_p, C.c_double]
        for name in ("zo_slab_phi_plane", "zo_slab_set_phi_ghost", "zo_slab_post_plane", "zo_slab_set_post_ghost"):
            getattr(lib, name).argtypes = [C.c_void_p, C.c_int, _D]
        lib.zo_stats.argtypes = [C.c_void_p, _D]
        lib.zo_steps.argtypes = [C.c_void_p]
        lib.zo_steps.restype = C.c_long
        lib.zo_threads.restype = C.c_int
        lib.zo_adjoint_run.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_int, C.c_int, _D, _D, _D]
        lib.zo_adjoint_run.restype = C.c_double
        lib.zo_objective_run.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_int, C.c_int]
        lib.zo_objective_run.restype = C.c_double
        lib.zo_adjoint_apply.argtypes = [C.c_void_p, C.c_double, _D, _D, _D, _D, C.POINTER(C.c_double)]
        lib.zo_adjoint_apply.restype = C.c_int
        lib.zo_heavy_mask.argtypes = [C.c_void_p, C.c_int, C.c_long]
        lib.zo_heavy_mask.restype = C.c_int
        lib.zo_init_adjoint.argtypes = [C.c_void_p, _D, _D, _D, _D, _D]
        lib.zo_set_rounding.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int, C.c_double, _D]
        lib.zo_round_array.argtypes = [C.c_int, _D, _D, C.c_long]
        _oracle_lib = lib
    return _oracle_lib


CONSTANT_NAMES = ["phiStar", "phiStarSq", "invTauRho", "invTauRhoOne", "invTauRhoHalf", "eta", "eta2",
                  "invEta2", "invTauPhi", "invTauPhiOne", "alpha", "alpha4", "kappa", "gravity", "grav",
                  "K0", "K1", "K2", "KC0", "KC1", "KC2"]
STATS_NAMES = ["umax", "vol", "ux_av", "uy_av", "uz_av", "ref", "p_in", "p_out", "p_dif", "p_err",
               "phi_sum", "rho_sum", "mom_x", "mom_y", "mom_z", "vol_full", "umax_full"]


FORMATS = {"none": 0, "fp32": 1, "fp16": 2, "bf16": 3}


def round_to(fmt: str, a) -> np.ndarray:
    """a rounded (from its FP32 value, to nearest even) to a storage format, as
    the oracle's storage-rounding emulation does."""
    a = np.ascontiguousarray(a, np.float64)
    out = np.empty_like(a)
    oracle_lib().zo_round_array(FORMATS[fmt], _dptr(a), _dptr(out), a.size)
    return out


class Oracle:
    """FP64 periodic-box ZSC step; arrays are (nz, ny, nx) float64."""

    def __init__(self, nx: int, ny: int, nz: int, *, rhoL, rhoH, tauRho, tauPhi, width, sigma, Gamma,
                 Eo=0.0, rc0=0.0):
        self.lib = oracle_lib()
        # the GPU reads these as float32: promote the same float32 values
        prm = np.array([np.float32(v) for v in (rhoL, rhoH, tauRho, tauPhi, width, sigma, Gamma, Eo, rc0)],
                       np.float64)
        self.h = self.lib.zo_create(nx, ny, nz, _dptr(prm))
        if not self.h:
            raise MemoryError("zo_create failed")
        self.shape = (nz, ny, nx)
        self.nx, self.ny, self.nz = nx, ny, nz
        self.rhoL, self.rhoH = float(prm[0]), float(prm[1])

    @classmethod
    def from_params(cls, p) -> "Oracle":
        return cls(p.nx, p.ny, p.nz, rhoL=p.rhoL, rhoH=p.rhoH, tauRho=p.tauRho, tauPhi=p.tauPhi, width=p.width,
                   sigma=p.sigma, Gamma=p.Gamma, Eo=p.Eo, rc0=p.rc0)

    def constants(self) -> dict:
        out = np.zeros(len(CONSTANT_NAMES), np.float64)
        self.lib.zo_constants(self.h, _dptr(out))
        return dict(zip(CONSTANT_NAMES, out))

    def bubble_phi(self, bubbles) -> np.ndarray:
        """phi with ghost planes, shape (nz + 2, ny, nx): plane k = reference z."""
        b = np.ascontiguousarray(bubbles, np.float32).reshape(-1, 4)
        out = np.empty((self.nz + 2, self.ny, self.nx), np.float64)
        self.lib.zo_bubble_phi(self.h, _fptr(b) if len(b) else None, len(b), _dptr(out))
        return out

    def init(self, phi, rho, ux=None, uy=None, uz=None, ghost=None) -> None:
        z = np.zeros(self.shape, np.float64)
        arrs = [np.ascontiguousarray(a if a is not None else z, np.float64) for a in (phi, rho, ux, uy, uz)]
        g = None if ghost is None else np.ascontiguousarray(ghost, np.float64)
        self.lib.zo_init(self.h, *[_dptr(a) for a in arrs], _dptr(g))

    def init_bubbles(self, bubbles) -> None:
        """src/init.c + init_f/init_g: phi from bubbles (ghost planes from the
        geometry, src/init.c:41-59), rho = (rhoH + rhoL) / 2, u = 0."""
        pg = self.bubble_phi(bubbles)
        rho = np.full(self.shape, 0.5 * (self.rhoH + self.rhoL), np.float64)
        self.init(pg[1:-1], rho, ghost=np.stack([pg[0], pg[-1]]))

    def step(self, n: int, grav: float = 0.0) -> None:
        self.lib.zo_step(self.h, int(n), float(grav))

    def moments(self) -> dict:
        arrs = [np.empty(self.shape, np.float64) for _ in range(5)]
        self.lib.zo_moments(self.h, *[_dptr(a) for a in arrs])
        return dict(zip(("phi", "rho", "ux", "uy", "uz"), arrs))

    def dist(self):
        f = np.empty((7,) + self.shape, np.float64)
        g = np.empty((19,) + self.shape, np.float64)
        self.lib.zo_dist(self.h, _dptr(f), _dptr(g))
        return f, g

    FIELD_NAMES = ([f"f{i}" for i in range(7)] + [f"g{i}" for i in range(19)]
                   + ["phi", "rho", "ux", "uy", "uz"])

    def compare(self, f=None, g=None, mom=None) -> dict:
        """Node-by-node comparison of float32 arrays with the oracle's state, in C
        without copies: f (7, nz, ny, nx) and g (19, ...) streamed distributions,
        mom (5, ...) phi, rho, ux, uy, uz.  Returns {field: (max |a - b|,
        max |b|)} for the fields given."""
        out = np.zeros(62, np.float64)
        self.lib.zo_compare(self.h, _fptr(f), _fptr(g), _fptr(mom), _dptr(out))
        res = {}
        for q, name in enumerate(self.FIELD_NAMES):
            given = (f is not None) if q < 7 else (g is not None) if q < 26 else (mom is not None)
            if given:
                res[name] = (float(out[2 * q]), float(out[2 * q + 1]))
        return res

    def set_dist(self, f, g) -> None:
        self.lib.zo_set_dist(self.h, _dptr(np.ascontiguousarray(f, np.float64)),
                             _dptr(np.ascontiguousarray(g, np.float64)))

    def stats(self) -> dict:
        out = np.zeros(17, np.float64)
        self.lib.zo_stats(self.h, _dptr(out))
        return dict(zip(STATS_NAMES, out))

    @property
    def steps(self) -> int:
        return int(self.lib.zo_steps(self.h))

    # --- discrete adjoint (FP64) ---
    OBJECTIVES = {"light_uz_mean": 0, "light_z_centroid": 1}

    def adjoint(self, T: int, grav: float, objective: str = "light_uz_mean", window: int = 1):
        """J, dJ/dgrav and dJ/ds^0 (f: 7 x shape, g: 19 x shape) over T steps from
        the current state; the oracle ends at s^T."""
        dg = C.c_double(0.0)
        lf = np.zeros((7,) + self.shape, np.float64)
        lg = np.zeros((19,) + self.shape, np.float64)
        J = self.lib.zo_adjoint_run(self.h, int(T), float(grav), self.OBJECTIVES[objective], int(window),
                                    C.byref(dg), _dptr(lf), _dptr(lg))
        return J, dg.value, lf, lg

    def objective(self, T: int, grav: float, objective: str = "light_uz_mean", window: int = 1) -> float:
        return float(self.lib.zo_objective_run(self.h, int(T), float(grav), self.OBJECTIVES[objective], int(window)))

    def adjoint_apply(self, grav: float, lf, lg):
        """J^T (lf, lg) for one step at the current streamed state, and dJ/dgrav's
        term sum lambda_Fz H(phi > 0)."""
        lf = np.ascontiguousarray(lf, np.float64)
        lg = np.ascontiguousarray(lg, np.float64)
        of = np.empty_like(lf)
        og = np.empty_like(lg)
        dg = C.c_double(0.0)
        if self.lib.zo_adjoint_apply(self.h, float(grav), _dptr(lf), _dptr(lg), _dptr(of), _dptr(og), C.byref(dg)):
            raise MemoryError("zo_adjoint_apply")
        return of, og, dg.value

    def set_rounding(self, f0: str = "none", f: str = "none", f_scale: float = 1.0, g: str = "none",
                     g_scale: float = 1.0, g_shift=None) -> None:
        """Storage-rounding emulation (zo_set_rounding in zsc_oracle.c): after
        every collision round f_0 to format f0, f_1..f_6 to fmt(f_k * f_scale)
        and g_i to fmt((g_i - g_shift[i]) * g_scale), formats "none", "fp32",
        "fp16", "bf16".  All-"none" switches it off."""
        sh = np.zeros(19) if g_shift is None else np.ascontiguousarray(g_shift, np.float64)
        self.lib.zo_set_rounding(self.h, FORMATS[f0], FORMATS[f], float(f_scale), FORMATS[g], float(g_scale),
                                 _dptr(sh))

    def heavy_mask(self, mode: str, steps: int = 0) -> None:
        """Heavy-node log: "record" H(phi > 0) of the next `steps` collisions
        after init, "replay" it instead of testing phi, "off"."""
        code = {"off": 0, "record": 1, "replay": 2}[mode]
        if self.lib.zo_heavy_mask(self.h, code, int(steps)) != 0:
            raise RuntimeError(f"zo_heavy_mask({mode}) failed")

    def init_adjoint(self, phi0, lf, lg):
        """dJ/dphi0 and dJ/drho0 from dJ/ds^0 through the initial equilibrium (periodic z)."""
        lphi = np.zeros(self.shape, np.float64)
        lrho = np.zeros(self.shape, np.float64)
        self.lib.zo_init_adjoint(self.h, _dptr(np.ascontiguousarray(phi0, np.float64)),
                                 _dptr(np.ascontiguousarray(lf, np.float64)),
                                 _dptr(np.ascontiguousarray(lg, np.float64)), _dptr(lphi), _dptr(lrho))
        return lphi, lrho

    @staticmethod
    def threads() -> int:
        return int(oracle_lib().zo_threads())

    def close(self) -> None:
        if self.h:
            self.lib.zo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SlabOracle(Oracle):
    """The FP64 step on planes [z0, z0 + nz) of a periodic box whose other
    planes live elsewhere (another rank): the reference's domain split
    (src/vgrid.c:38-52) with its three halo exchanges per step, as whole
    planes (zsc_oracle.c, zo_slab_*).  One step is

        moments(); exchange phi planes; collide(grav); exchange post planes; stream()

    where an exchange sends plane(side 0) to the slab below and plane(side 1)
    to the slab above, and sets the received planes as ghosts (side 0 below,
    side 1 above)."""

    def __init__(self, nx: int, ny: int, nz: int, **kw):
        self.lib = oracle_lib()
        prm = np.array([np.float32(kw[k]) for k in ("rhoL", "rhoH", "tauRho", "tauPhi", "width", "sigma", "Gamma")]
                       + [np.float32(kw.get("Eo", 0.0)), np.float32(kw.get("rc0", 0.0))], np.float64)
        self.h = self.lib.zo_slab_create(nx, ny, nz, _dptr(prm))
        if not self.h:
            raise MemoryError("zo_slab_create failed")
        self.shape = (nz, ny, nx)
        self.nx, self.ny, self.nz = nx, ny, nz
        self.rhoL, self.rhoH = float(prm[0]), float(prm[1])

    def moments_update(self) -> None:
        self.lib.zo_slab_moments(self.h)

    def phi_plane(self, side: int) -> np.ndarray:
        out = np.empty((self.ny, self.nx), np.float64)
        self.lib.zo_slab_phi_plane(self.h, side, _dptr(out))
        return out

    def set_phi_ghost(self, side: int, plane) -> None:
        self.lib.zo_slab_set_phi_ghost(self.h, side, _dptr(np.ascontiguousarray(plane, np.float64)))

    def collide(self, grav: float) -> None:
        self.lib.zo_slab_collide(self.h, float(grav))

    def post_plane(self, side: int) -> np.ndarray:
        out = np.empty((26, self.ny, self.nx), np.float64)
        self.lib.zo_slab_post_plane(self.h, side, _dptr(out))
        return out

    def set_post_ghost(self, side: int, planes) -> None:
        self.lib.zo_slab_set_post_ghost(self.h, side, _dptr(np.ascontiguousarray(planes, np.float64)))

    def stream(self) -> None:
        self.lib.zo_slab_stream(self.h)

    def step(self, n: int, grav: float = 0.0) -> None:
        raise TypeError("a slab steps through moments_update / collide / stream with exchanges between them")


def oracle_from_inputs(p, bubbles=None) -> Oracle:
    """Oracle for library Params p, initialised from bubbles like lbm_init_bubbles."""
    o = Oracle.from_params(p)
    if bubbles is not None:
        o.init_bubbles(bubbles)
    return o


def ref_lib() -> C.CDLL | None:
    """The reference's kernels on the CPU, or None when the sources are unavailable."""
    global _ref_lib
    if _ref_lib is None:
        path = _build.build_reference()
        if path is None:
            return None
        lib = C.CDLL(str(path))
        lib.zr_init.argtypes = [C.c_char_p, _Fp]
        lib.zr_step.argtypes = [C.c_int, C.c_float]
        lib.zr_fields.argtypes = [_Fp] * 5
        lib.zr_dist.argtypes = [_Fp, _Fp]
        lib.zr_dims.argtypes = [C.POINTER(C.c_int)]
        lib.zr_consts.argtypes = [_Fp]
        lib.zr_write_stats.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int]
        lib.zr_threads.restype = C.c_int
        _ref_lib = lib
    return _ref_lib


REF_CONSTANT_NAMES = ["phiStar", "phiStarSq", "invTauRhoOne", "eta", "eta2", "invEta2", "invTauPhi",
                      "invTauPhiOne", "alpha", "alpha4", "kappa", "gravity", "grav", "K0", "K1", "K2",
                      "KC0", "KC1", "KC2"]


class RefCPU:
    """The reference's own step (FP32, its seven kernels and three halo
    exchanges) run on the CPU.  One instance at a time (the reference keeps
    its state in globals)."""

    def __init__(self, directory: str | os.PathLike, phi_override: np.ndarray | None = None):
        self.lib = ref_lib()
        if self.lib is None:
            raise FileNotFoundError("reference sources not available")
        po = None if phi_override is None else np.ascontiguousarray(phi_override, np.float32)
        rc = self.lib.zr_init(str(directory).encode(), _fptr(po))
        if rc != 0:
            raise RuntimeError(f"zr_init failed with {rc}")
        d = (C.c_int * 11)()
        self.lib.zr_dims(d)
        self.nx, self.ny, self.nz = d[0], d[1], d[2]
        self.nbubbles, self.max_step, self.relax_step = d[4], d[5], d[6]
        self.shape = (self.nz, self.ny, self.nx)

    def constants(self) -> dict:
        out = np.zeros(len(REF_CONSTANT_NAMES), np.float32)
        self.lib.zr_consts(_fptr(out))
        return dict(zip(REF_CONSTANT_NAMES, out))

    def step(self, n: int, grav: float = 0.0) -> None:
        rc = self.lib.zr_step(int(n), float(grav))
        if rc != 0:
            raise RuntimeError(f"zr_step failed with {rc}")

    def fields(self) -> dict:
        arrs = [np.empty(self.shape, np.float32) for _ in range(5)]
        self.lib.zr_fields(*[_fptr(a) for a in arrs])
        return dict(zip(("phi", "rho", "ux", "uy", "uz"), arrs))

    def dist(self):
        f = np.empty((7,) + self.shape, np.float32)
        g = np.empty((19,) + self.shape, np.float32)
        self.lib.zr_dist(_fptr(f), _fptr(g))
        return f, g

    def write_stats(self, directory, relax: int, step_no: int, with_log: bool = False) -> None:
        rc = self.lib.zr_write_stats(str(directory).encode(), relax, step_no, int(with_log))
        if rc != 0:
            raise RuntimeError(f"zr_write_stats failed with {rc}")

    @staticmethod
    def threads() -> int:
        lib = ref_lib()
        return int(lib.zr_threads()) if lib else 0
