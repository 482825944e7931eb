"""Generate the golden fixtures in this directory from the reference itself.

Runs the reference's own kernels (compiled for the host CPU by
oracle/build.py from the reference sources) on small seeded inputs written in
the reference's input format, and stores the inputs together with the
reference's phi, rho, u arrays after the given number of steps, plus the
text its stats()/logSave() write.  The fixtures pin the FP64 oracle (and the
GPU path) on machines where the reference sources are not available.

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from lbm_bench_gpu_gb300 import inputs  # noqa: E402
from oracle.oracle import RefCPU  # noqa: E402

# name -> (Inputs, steps, grav)
CASES = {
    # one off-centre bubble, relaxation (no gravity)
    "relax32": (inputs.Inputs(nx=32, ny=32, nz=32, bubbles=np.array([[15.7, 16.2, 16.45, 8.3]], np.float32)),
                10, 0.0),
    # two overlapping bubbles (last writer wins) whose shells reach the z ghost
    # planes (ghost planes initialised from the geometry), with gravity
    "overlap_ghost32": (inputs.Inputs(nx=32, ny=32, nz=24, tauRho=0.8,
                                      bubbles=np.array([[12.0, 14.0, 3.5, 6.0], [17.0, 15.0, 5.0, 5.5]],
                                                       np.float32)),
                        6, -2e-5),
    # non-cubic box, large density ratio of the reference's sample input, gravity
    "sample_ratio": (inputs.Inputs(nx=64, ny=32, nz=16, rhoL=1.0, rhoH=1000.0, tauRho=1.0, tauPhi=0.7,
                                   width=4.0, sigma=0.01, Gamma=400.0, Eo=10.0,
                                   bubbles=np.array([[30.0, 16.0, 8.0, 5.0]], np.float32)),
                     3, None),
}


def main() -> int:
    manifest = {}
    for name, (inp, steps, grav) in CASES.items():
        with tempfile.TemporaryDirectory() as d:
            inputs.write_inputs(d, inp)
            props = (Path(d) / "properties.in").read_text()
            disc = (Path(d) / "discrete.in").read_text()
            ref = RefCPU(d)
            consts = ref.constants()
            g = float(consts["grav"]) if grav is None else grav
            init = ref.fields()
            ref.write_stats(d, relax=1, step_no=0)
            ref.step(steps, g)
            out = ref.fields()
            ref.write_stats(d, relax=1, step_no=steps, with_log=True)
            stats_txt = (Path(d) / "relax_stats.out").read_text()
            runlog_txt = (Path(d) / "runlog.out").read_text()
        np.savez_compressed(
            HERE / f"{name}.npz",
            **{f"init_{k}": v for k, v in init.items()},
            **{k: v for k, v in out.items()},
        )
        manifest[name] = {
            "steps": steps, "grav": g, "properties.in": props, "discrete.in": disc,
            "relax_stats.out": stats_txt, "runlog.out": runlog_txt,
            "ref_constants": {k: float(v) for k, v in consts.items()},
        }
        print(name, "done")
    (HERE / "golden.json").write_text(json.dumps(manifest, indent=1))
    return 0


if __name__ == "__main__":
    sys.exit(main())
