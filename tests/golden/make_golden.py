"""Generates the committed golden fixtures under tests/golden/.

  gll.json    GLL points/weights for N=1..15 to 30 digits (sympy roots of
              (1-x^2) P_N'(x) at 50-digit precision), pinning the oracle's
              ZWGLL restatement (src/nek5_speclib.F:107-283).
  gs_ref.npz  the reference's own gather-scatter (NekCEM src/jl/gs.c,
              compiled from the reference tree by oracle/build_ref.sh) applied
              to the face ids of small box meshes with 6 fields of seeded
              data: ids, input, output.  Pins the oracle's gs_op_fields.

Run from the repo root: python tests/golden/make_golden.py
(needs sympy, gcc and the reference tree for gs_ref.npz).
"""
import ctypes as C
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def make_gll():
    import sympy as sp
    x = sp.symbols("x")
    out = {}
    for N in range(1, 16):
        P = sp.legendre(N, x)
        dP = sp.diff(P, x)
        roots = [-1] + sorted(sp.Poly(dP, x).nroots(n=50, maxsteps=200)) + [1] if N > 1 else [-1, 1]
        z = [sp.Float(r, 50) for r in roots]
        w = [sp.Float(2, 50) / (N * (N + 1) * P.subs(x, zi) ** 2) for zi in z]
        out[str(N)] = {"z": [sp.N(v, 30).__str__() for v in z], "w": [sp.N(v, 30).__str__() for v in w]}
    with open(os.path.join(HERE, "gll.json"), "w") as f:
        json.dump(out, f, indent=1)


def make_gs():
    subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    L = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libjlgs.so"))
    L.jlgs_apply.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int]
    from oracle import refcpu as R
    data = {}
    meshes = [(3, (2, 2, 2), (1, 0, 1)), (2, (3, 1, 2), (0, 1, 1)), (4, (1, 1, 1), (1, 1, 1))]
    for t, (N, nel, bc) in enumerate(meshes):
        m = R.RefBox(N, nel, (0, 0, 0), (1, 1, 1), bc)
        ids = m.l("glo_face").copy()
        n = m.nxzfl
        u = np.random.default_rng(100 + t).standard_normal(6 * n)
        out = u.copy()
        assert L.jlgs_apply(ids.ctypes.data, n, out.ctypes.data, n, 6) == 0
        data[f"m{t}_meta"] = np.array([N, *nel, *bc])
        data[f"m{t}_ids"] = ids
        data[f"m{t}_in"] = u
        data[f"m{t}_out"] = out
    np.savez_compressed(os.path.join(HERE, "gs_ref.npz"), **data)


if __name__ == "__main__":
    make_gll()
    make_gs()
    print("golden fixtures written")
