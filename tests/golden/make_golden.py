"""Regenerates the golden fixtures of this folder from the CPU oracle.

    python tests/golden/make_golden.py

Each case is a small seeded input (hvgpu.datasets SplitMix64 points) whose
mesh the oracle computes: sorted 1-based vertex signatures, coordinates,
neighbour CSR (and lattice shifts on periodic cuboids) and VI_POLYGON volumes
and areas.  The fixtures pin the oracle across changes (tests/test_oracle.py)
and are the expected outputs of the GPU parity tests (tests/test_gpu_golden.py).
The reference itself (Julia) cannot run here, so the vectors are the oracle's.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "highvoronoi.jl_gb300"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    sys.path.insert(0, p)

import oracle as O  # noqa: E402
from hvgpu import datasets as D  # noqa: E402
from _domains import simplex, simplex_points  # noqa: E402

# name: (d, n, seed, domain) with domain "box", "simplex" or "periodic"
CASES = {
    "box2d_64": (2, 64, 101, "box"),
    "box3d_48": (3, 48, 102, "box"),
    "box4d_40": (4, 40, 103, "box"),
    "box5d_24": (5, 24, 104, "box"),
    "box6d_14": (6, 14, 105, "box"),
    "simplex3d_40": (3, 40, 106, "simplex"),
    "periodic2d_40": (2, 40, 107, "periodic"),
    "periodic3d_30": (3, 30, 108, "periodic"),
}


def case_inputs(name):
    d, n, seed, dom = CASES[name]
    if dom == "simplex":
        return simplex_points(d, n, seed), dom
    return D.uniform_points(d, n, seed), dom


def compute(name):
    d, n, seed, dom = CASES[name]
    X, _ = case_inputs(name)
    out = {"pts": X}
    if dom == "periodic":
        P = O.periodic_mesh(X, np.zeros(d), np.ones(d), [1] * d, integrate=True)
        out.update(sig=P["sig"], r=P["r"], offs=P["offs"], nbr=P["nbr"], shift=P["shift"], vol=P["vol"], area=P["area"])
        key = np.lexsort(np.concatenate([out["sig"], np.round(out["r"], 9)], axis=1).T[::-1])
        out["sig"], out["r"] = out["sig"][key], out["r"][key]
        return out
    if dom == "simplex":
        base, normal, _ = simplex(d)
        m = O.OracleMesh(X, planes=(base, normal), integrate=True)
        out.update(base=base, normal=normal)
    else:
        m = O.OracleMesh(X, integrate=True)
    out["sig"], out["r"] = m.vertices()
    out["offs"], out["nbr"] = m.neighbors()
    out["vol"], out["area"] = m.polygon()
    return out


def main():
    for name in CASES:
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **compute(name))
        print(name)


if __name__ == "__main__":
    main()
