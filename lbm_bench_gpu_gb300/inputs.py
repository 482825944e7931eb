"""Input files and the seeded synthetic workloads.

The reference reads two positional text files from its working directory
(src/paramread.c:36-75): ``properties.in`` (step counts, box, block size,
densities, relaxation times, interface width / tension / mobility, Eotvos
number) and ``discrete.in`` (bubble list: xc yc zc Rc, x and y 0-based, z
1-based).  ``write_inputs`` produces files in that format; parsing is done by
the library (``capi.read_inputs``).

Workloads (all synthetic and seeded; the reference ships no dataset):
  static_bubble   64^3, one bubble of radius 12 in the centre, no gravity
  bubbly          256^3, 64 bubbles, radii U[6, 10], surface gap >= 3
  bubbly_512      512^3, 512 bubbles, radii U[6, 12]
  adjoint_short   128^3, 8 bubbles of radius 10
Gravity g is given as a body force; the reference takes the Eotvos number
instead (src/paramread.c:160-161: grav = 0.25 Eo sigma / Rc0^2 after the
density factors cancel), so ``eo_for_gravity`` inverts that relation.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

SEED = 20261203


@dataclass
class Inputs:
    nx: int
    ny: int
    nz: int
    rhoL: float = 0.1
    rhoH: float = 1.0
    tauRho: float = 0.7
    tauPhi: float = 1.0
    width: float = 4.0
    sigma: float = 1e-3
    Gamma: float = 1.0
    Eo: float = 0.0
    max_step: int = 1000
    relax_step: int = 0
    save: int = 1_000_000
    stat: int = 1_000_000
    block_x: int = 32
    block_y: int = 8
    bubbles: np.ndarray = field(default_factory=lambda: np.zeros((0, 4), np.float32))

    @property
    def rc0(self) -> float:
        return float(self.bubbles[0, 3]) if len(self.bubbles) else 0.0


def eo_for_gravity(g: float, rc0: float, sigma: float) -> float:
    """Eotvos number that makes the reference's grav equal g."""
    return 4.0 * g * rc0 * rc0 / sigma


def write_inputs(directory: str | os.PathLike, inp: Inputs) -> Path:
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    (d / "properties.in").write_text(
        "maxStep\trelaxStep\tsave\tstat\n"
        f"{inp.max_step}\t{inp.relax_step}\t\t{inp.save}\t{inp.stat}\n\n"
        "xmax\tymax\tzmax\n"
        f"{inp.nx}\t{inp.ny}\t{inp.nz}\n\n"
        "BLOCK_SIZE_X\tBLOCK_SIZE_Y\n"
        f"{inp.block_x}\t\t{inp.block_y}\n\n"
        "rhoL\trhoH\n"
        f"{inp.rhoL:.9g}\t{inp.rhoH:.9g}\n\n"
        "tauRho\ttauPhi\n"
        f"{inp.tauRho:.9g}\t{inp.tauPhi:.9g}\n\n"
        "width\tsigma\tGamma\n"
        f"{inp.width:.9g} \t{inp.sigma:.9g}\t{inp.Gamma:.9g}\n\n"
        "Eo\n"
        f"{inp.Eo:.9g}\n"
    )
    rows = "".join(f"{b[0]:.4f}\t{b[1]:.4f}\t{b[2]:.4f}\t{b[3]:.4f}\n" for b in inp.bubbles)
    (d / "discrete.in").write_text(f"nBubbles\n{len(inp.bubbles)}\n\nxc\tyc\tzc\tRc\n{rows}")
    return d


def place_bubbles(n: int, box: tuple[int, int, int], r_range: tuple[float, float], *, gap: float = 3.0,
                  width: float = 4.0, seed: int = SEED, max_tries: int = 200_000) -> np.ndarray:
    """Seeded rejection sampling of non-overlapping bubbles (numpy PCG64).

    Radii are uniform in r_range (rounded to 1e-4 so the text file holds them
    exactly); centres are uniform with every centre at least R + width + 1
    from every face (so no interface reaches the periodic seams and the
    reference's ghost-plane initialisation equals periodic wrap) and every
    pair of surfaces at least ``gap`` apart.  Returns n x 4 float32 rows
    {xc, yc, zc, Rc} in the reference's coordinates (z 1-based)."""
    nx, ny, nz = box
    rng = np.random.Generator(np.random.PCG64(seed))
    out: list[tuple[float, float, float, float]] = []
    tries = 0
    while len(out) < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError(f"could only place {len(out)} of {n} bubbles")
        r = round(float(rng.uniform(*r_range)), 4)
        m = r + width + 1.0
        lo = np.array([m, m, 1.0 + m])
        hi = np.array([nx - 1 - m, ny - 1 - m, nz - m])
        if np.any(hi <= lo):
            continue
        c = np.round(rng.uniform(lo, hi), 4)
        if all(np.linalg.norm(c - np.array(o[:3])) >= r + o[3] + gap for o in out):
            out.append((float(c[0]), float(c[1]), float(c[2]), r))
    return np.array(out, dtype=np.float32)


def static_bubble(n: int = 64, radius: float = 12.0, steps: int = 1000) -> Inputs:
    """One bubble of radius 12 centred in an n^3 box, no gravity (Laplace check)."""
    c = n / 2.0
    return Inputs(nx=n, ny=n, nz=n, max_step=1, relax_step=steps, Eo=0.0,
                  bubbles=np.array([[c, c, c, radius]], np.float32))


def bubbly(n: int = 256, count: int = 64, r_range=(6.0, 10.0), gravity: float = -1e-6, seed: int = SEED,
           steps: int = 10_000, tauRho: float = 0.7) -> Inputs:
    """Seeded bubbly flow with a body force along z."""
    b = place_bubbles(count, (n, n, n), r_range, seed=seed)
    inp = Inputs(nx=n, ny=n, nz=n, tauRho=tauRho, max_step=steps + 1, relax_step=0, bubbles=b)
    inp.Eo = eo_for_gravity(gravity, float(b[0, 3]), inp.sigma)
    return inp


def adjoint_short(seed: int = SEED) -> Inputs:
    """128^3, 8 bubbles of radius 10 at seeded non-overlapping centres."""
    b = place_bubbles(8, (128, 128, 128), (10.0, 10.0), seed=seed)
    inp = Inputs(nx=128, ny=128, nz=128, tauRho=0.8, max_step=2001, relax_step=0, bubbles=b)
    inp.Eo = eo_for_gravity(-1e-6, 10.0, inp.sigma)
    return inp
