"""Generates tests/golden/golden_small.npz from the CPU oracle.

The reference has no test vectors of its own and cannot be built here (no
Fortran compiler), so these fixtures are the oracle's outputs on small seeded
cases, committed so that the GPU path and later oracle builds are checked
against fixed numbers on every machine:

  * cluster structure of a 16 x 8 3dph mesh: lod and the leaf list;
  * 64 kernel entries each for 2dvs (n=256), 3dph (16 x 8) and 3dnt (rough
    6 x 3 km fault, 24 x 12 x 2 triangles), shear and normal; the same for
    2dph (600 elements dipping 30 degrees from the surface), 2dn (600
    elements on a seeded bent fault) and 3dht (the 3dnt fault buried 0.5 km
    in a half space);
  * derivs and one rkck step of the 2dvs system (n=256, ACA eps 1e-6, aging
    law, b tapering below 15 km) from its steady initial state.

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from oracle import oracle as O  # noqa: E402
from hbi_gb300 import configs  # noqa: E402
from gpu_cases import case, oracle_geometry  # noqa: E402


def main():
    O.build()
    out = {}
    rng = np.random.default_rng(2024)
    # structure
    prob, n, g, w, eps = case("3dph", (16, 8))
    coord = np.stack([g["xcol"], g["ycol"], g["zcol"]], 1)
    lod, leaves, _ = O.build_structure(coord)
    out["struct_coord"] = coord
    out["struct_lod"] = lod
    out["struct_leaves"] = np.array(leaves, dtype=np.int32)
    # entries
    for kind in ("2dvs", "3dph", "3dnt", "2dph", "2dn", "3dht"):
        prob, n, g, w, eps = case(kind, 256 if kind == "2dvs" else None)
        ii = rng.integers(1, n + 1, 64)
        jj = rng.integers(1, n + 1, 64)
        jj[:8] = ii[:8]  # self terms
        for v in ("s", "n"):
            if kind == "2dvs" and v == "n":
                continue
            geo = oracle_geometry(O, prob, n, g, w, v)
            out[f"entry_{kind}_{v}"] = np.array([O.entry(geo, int(i), int(j)) for i, j in zip(ii, jj)])
        out[f"entry_{kind}_ij"] = np.stack([ii, jj], 1).astype(np.int32)
    # derivs / rkck of the 2dvs system
    wl = configs.c1_2dvs(256)
    coord = np.stack([wl.geom_kw["xcol"], np.zeros(256), np.zeros(256)], 1)
    lod, lv, _ = O.build_structure(coord)
    p = O.default_params()
    p[70] = wl.eps_h
    Hm = O.HMatrix(O.Geometry(1, 256, "s", **wl.geom_kw), lod, lv, p)
    y0, pp = wl.initial_state(lod)
    R = O.RSF(256, Hm, evlaw=0, a=pp["a"], b=pp["b"], dc=pp["dc"], f0=pp["f0"], vplv=pp["vpl"])
    out["rk_y0"] = y0
    out["rk_dydx"] = R.derivs(y0)
    yo, ye = R.rkck(y0, 0.0, 1.0e6)
    out["rk_h"] = np.array([1.0e6])
    out["rk_yout"], out["rk_yerr"] = yo, ye
    path = os.path.join(ROOT, "tests", "golden", "golden_small.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
