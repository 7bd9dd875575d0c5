"""Generates the golden fixtures of the oracle (tests/golden/*.npz).

The reference (komietty/metriko) cannot be built here and ships no tests or golden data, so
these fixtures pin the FP64 CPU oracle's outputs on small seeded meshes; the GPU tests check
the CUDA path against them and the CPU tests check that the oracle still reproduces them.
Run:  python tests/golden/make_golden.py [name ...]   (all fixtures when no name is given)
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from metriko_gb300 import meshgen  # noqa: E402
from oracle import metriko_oracle as O  # noqa: E402

NAMES = ["ico2_noise", "ico3_noise", "torus_32x16", "genus2_s3"]


def main(names):
    for name in names:
        V, F, ratio, rs = meshgen.workload(name)
        out = O.pipeline(V, F, ratio=ratio, round_seams=rs)
        info = out["info"]
        np.savez_compressed(
            Path(__file__).parent / f"{name}.npz",
            V=V, F=F, ratio=ratio, round_seams=rs,
            compressed=out["compressed"], singular=out["singular"], seam=np.packbits(out["seam"]),
            n_edges=len(out["seam"]), combed_matching=out["combed_matching"].astype(np.int8),
            fix_order=np.asarray(info["fix_order"], np.int32), fix_vals=np.asarray(info["fix_vals"], np.int32),
            fullx=out["fullx"], x_naive=info["x0"], cutF=out["cutF"].astype(np.int32))
        print(name, len(F), "faces", len(info["fix_order"]), "fixings")


if __name__ == "__main__":
    main(sys.argv[1:] or NAMES)
