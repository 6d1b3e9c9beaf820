"""Shared test helpers: oracle <-> GPU context plumbing and error measures."""
from __future__ import annotations

import numpy as np

from oracle import refcpu as R
from nekcem_gb300 import MaxwellGPU, cases

# reference COMMON-array names (src/EMWAVE, src/GEOM) -> oracle names
ORACLE_NAMES = {
    "dxm1": "dxm1", "w3mn": "w3m1", "bmn": "bm1", "xmn": "xm1", "ymn": "ym1", "zmn": "zm1",
    "rxmn": "rxm1", "rymn": "rym1", "rzmn": "rzm1", "sxmn": "sxm1", "symn": "sym1",
    "szmn": "szm1", "txmn": "txm1", "tymn": "tym1", "tzmn": "tzm1",
    "unxm": "unx", "unym": "uny", "unzm": "unz", "aream": "area",
    "Z_0": "Z_0", "Z_1": "Z_1", "Y_0": "Y_0", "Y_1": "Y_1", "ebm1": "ebm1", "hbm1": "hbm1",
}


def oracle_arrays(ref: R.RefBox) -> dict:
    """The static arrays the Fortran driver would hand to nekgpu_init."""
    out = {k: ref.d(v).copy() for k, v in ORACLE_NAMES.items()}
    out["cemface"] = ref.i("cemface").copy()
    out["cempec"] = ref.i("cempec").copy()
    out["glo_face"] = ref.l("glo_face").copy()
    if getattr(ref, "pml", None):
        out["pmlsigma"] = ref.d("pmlsigma").copy()
        out["pmlptr"] = ref.i("pmlptr").copy()
        out["permittivity"] = ref.d("permittivity").copy()
        out["permeability"] = ref.d("permeability").copy()
    return out


def make_ref(N, nel, lo, hi, bc, eps=None, mu=None, C0=1.0, threads=0, pml=None, deform=0.0):
    if threads:
        R.set_threads(threads)
    ref = R.RefBox(N, nel, lo, hi, bc, deform=deform)
    if eps is not None or mu is not None:
        x, y, z = ref.coords()
        e = np.ones(ref.npts) if eps is None else (eps(x, y, z) if callable(eps) else eps)
        m = np.ones(ref.npts) if mu is None else (mu(x, y, z) if callable(mu) else mu)
        ref.set_materials(np.asarray(e, float), np.asarray(m, float))
    ref.set_flux(C0)
    ref.pml = pml
    if pml is not None:
        ref.set_pml(*pml)
    return ref


def gpu_from_ref(ref: R.RefBox, form: str, C0: float = 1.0) -> MaxwellGPU:
    return MaxwellGPU.from_arrays(oracle_arrays(ref), ref.n, ref.nelt, form=form, C0=C0)


def gpu_from_box(ref: R.RefBox, form: str, C0: float = 1.0) -> MaxwellGPU:
    eps = ref.d("permittivity").copy()
    mu = ref.d("permeability").copy()
    uniform = np.all(eps == 1.0) and np.all(mu == 1.0)
    return MaxwellGPU.from_box(ref.N, ref.nel, ref.lo, ref.hi, ref.bc, form=form,
                               permittivity=None if uniform else eps,
                               permeability=None if uniform else mu, C0=C0,
                               pml=getattr(ref, "pml", None))


def random_fields(npts: int, seed: int):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((3, npts)), rng.standard_normal((3, npts))


def smooth_fields(ref: R.RefBox, seed: int):
    """Smooth seeded fields (sums of a few low modes) so that contraction
    errors behave like the physical cases."""
    x, y, z = ref.coords()
    rng = np.random.default_rng(seed)
    L = np.array(ref.hi) - np.array(ref.lo)
    out = []
    for q in range(6):
        f = np.zeros_like(x)
        for _ in range(3):
            k = rng.integers(1, 3, size=3) * 2 * np.pi / L
            ph = rng.uniform(0, 2 * np.pi)
            f += rng.standard_normal() * np.cos(k[0] * x + k[1] * y + k[2] * z + ph)
        out.append(f)
    out = np.array(out)
    return out[:3].copy(), out[3:].copy()


def rel_err(a_H, a_E, b_H, b_E) -> float:
    a = np.concatenate([np.ravel(a_H), np.ravel(a_E)])
    b = np.concatenate([np.ravel(b_H), np.ravel(b_E)])
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
