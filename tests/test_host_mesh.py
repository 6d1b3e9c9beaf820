"""Host setup (no GPU): the library's box builder against the oracle's
restatement of the reference setup (genwz, genxyz, glmapm1, geodat1, area3,
cem_set_fc_ptr, setup_dgds2 pairing, pec_init, cem_maxwell_materials)."""
import ctypes as C

import numpy as np
import pytest

from oracle import refcpu as R
from nekcem_gb300 import _lib as L

BOXES = [
    dict(N=4, nel=(3, 2, 2), lo=(0, 0, 0), hi=(1, 1.5, 0.75), bc=(0, 0, 0)),
    dict(N=7, nel=(2, 3, 1), lo=(-1, 0, 2), hi=(1, 1, 3), bc=(1, 0, 1)),
    dict(N=5, nel=(1, 1, 2), lo=(0, 0, 0), hi=(2, 2, 2), bc=(1, 1, 1)),
]


def box_struct(b, eps=None, mu=None, pml=None):
    s = L.NekgpuBox()
    s.N = b["N"]; s.nelx, s.nely, s.nelz = b["nel"]
    for d in range(3):
        s.lo[d] = b["lo"][d]; s.hi[d] = b["hi"][d]; s.bc[d] = b["bc"][d]
    s.C0 = 1.0
    if pml is not None:
        s.pml_thick, s.pml_order, s.pml_referr = pml
    keep = []
    if eps is not None:
        keep.append(eps); s.permittivity = eps.ctypes.data_as(L.dp)
    if mu is not None:
        keep.append(mu); s.permeability = mu.ctypes.data_as(L.dp)
    return s, keep


def export_d(s, name):
    lib = L.load()
    n = C.c_long()
    L.check(lib.nekgpu_box_export_d(C.byref(s), name.encode(), None, C.byref(n)), name)
    out = np.empty(n.value)
    L.check(lib.nekgpu_box_export_d(C.byref(s), name.encode(), out.ctypes.data_as(L.dp), C.byref(n)), name)
    return out


def export_i(s, name):
    lib = L.load()
    n = C.c_long()
    L.check(lib.nekgpu_box_export_i(C.byref(s), name.encode(), None, C.byref(n)), name)
    out = np.empty(n.value, dtype=np.int64)
    L.check(lib.nekgpu_box_export_i(C.byref(s), name.encode(), out.ctypes.data_as(L.lp), C.byref(n)), name)
    return out


def pairing(ids):
    order = np.lexsort((np.arange(ids.size), ids))
    s = ids[order]
    groups = {}
    start = 0
    for i in range(1, s.size + 1):
        if i == s.size or s[i] != s[start]:
            groups[tuple(sorted(order[start:i]))] = True
            start = i
    return set(groups)


@pytest.mark.parametrize("b", BOXES)
def test_box_builder_matches_oracle_setup(b):
    ref = R.RefBox(b["N"], b["nel"], b["lo"], b["hi"], b["bc"])
    x, y, z = ref.coords()
    eps = 1.0 + 0.5 * np.sin(2 * x) ** 2 + 0.3 * (y > 0.5)
    mu = 1.0 + 0.2 * np.cos(3 * z) ** 2
    ref.set_materials(eps, mu)
    s, keep = box_struct(b, np.ascontiguousarray(eps), np.ascontiguousarray(mu))
    tol = dict(rtol=1e-13, atol=1e-14)
    np.testing.assert_allclose(export_d(s, "dxm1"), ref.d("dxm1"), rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(export_d(s, "w3mn"), ref.d("w3m1"), **tol)
    np.testing.assert_allclose(export_d(s, "bmn"), ref.d("bm1"), rtol=1e-12)
    for a, o in (("xmn", "xm1"), ("ymn", "ym1"), ("zmn", "zm1")):
        np.testing.assert_allclose(export_d(s, a), ref.d(o), rtol=1e-13, atol=1e-13)
    for a, o in (("rxmn", "rxm1"), ("symn", "sym1"), ("tzmn", "tzm1")):
        np.testing.assert_allclose(export_d(s, a), ref.d(o), rtol=1e-12)
    for a, o in (("unxm", "unx"), ("unym", "uny"), ("unzm", "unz")):
        np.testing.assert_allclose(export_d(s, a), ref.d(o), rtol=0, atol=1e-13)
    np.testing.assert_allclose(export_d(s, "aream"), ref.d("area"), rtol=1e-12)
    np.testing.assert_array_equal(export_i(s, "cemface"), ref.i("cemface") + 1)
    np.testing.assert_array_equal(export_i(s, "cempec"), ref.i("cempec") + 1)
    assert pairing(export_i(s, "glo_face")) == pairing(ref.l("glo_face").astype(np.int64))
    for a in ("Z_0", "Z_1", "Y_0", "Y_1"):
        np.testing.assert_allclose(export_d(s, a), ref.d(a), rtol=1e-14)
    np.testing.assert_allclose(export_d(s, "ebm1"), ref.d("ebm1"), rtol=1e-12)
    np.testing.assert_allclose(export_d(s, "hbm1"), ref.d("hbm1"), rtol=1e-12)


def test_box_builder_rejects_bad_boxes():
    lib = L.load()
    s, _ = box_struct(dict(N=0, nel=(1, 1, 1), lo=(0, 0, 0), hi=(1, 1, 1), bc=(0, 0, 0)))
    n = C.c_long()
    assert lib.nekgpu_box_export_d(C.byref(s), b"bmn", None, C.byref(n)) == -1
    s, _ = box_struct(dict(N=3, nel=(1, 1, 1), lo=(0, 0, 0), hi=(0, 1, 1), bc=(0, 0, 0)))
    assert lib.nekgpu_box_export_d(C.byref(s), b"bmn", None, C.byref(n)) == -1
    s, _ = box_struct(dict(N=3, nel=(1, 1, 1), lo=(0, 0, 0), hi=(1, 1, 1), bc=(0, 0, 0)))
    assert lib.nekgpu_box_export_d(C.byref(s), b"nope", None, C.byref(n)) == -1


PML_BOXES = [
    dict(N=4, nel=(6, 6, 6), lo=(-1, -1, -1), hi=(1, 1, 1), bc=(2, 2, 2), pml=(1, 3.0, 1e-8)),
    dict(N=3, nel=(5, 4, 6), lo=(0, 0, 0), hi=(1.25, 1, 1.5), bc=(2, 1, 2), pml=(2, 2.0, 1e-6)),
    dict(N=5, nel=(4, 3, 2), lo=(0, 0, 0), hi=(1, 1, 1), bc=(0, 2, 1), pml=(1, 4.0, 1e-4)),
]


@pytest.mark.parametrize("b", PML_BOXES)
def test_box_builder_pml_matches_oracle(b):
    """PML boxes: the layer tags, extents and graded sigma of the library's
    box builder against the oracle's restatement of the reference's face
    marching (pml_fill_faceary, march_faces, pml_extent_and_tags,
    pml_calc_sigma); PML faces join the PEC list and keep Z_1 = Y_1 = 0."""
    ref = R.RefBox(b["N"], b["nel"], b["lo"], b["hi"], b["bc"])
    x, y, z = ref.coords()
    eps = 1.0 + 0.5 * np.sin(2 * x) ** 2
    mu = 1.0 + 0.2 * np.cos(3 * z) ** 2
    ref.set_materials(eps, mu)
    ref.set_pml(*b["pml"])
    s, keep = box_struct(b, np.ascontiguousarray(eps), np.ascontiguousarray(mu), pml=b["pml"])
    np.testing.assert_array_equal(export_i(s, "pmlptr"), ref.i("pmlptr") + 1)
    np.testing.assert_allclose(export_d(s, "pmlsigma"), ref.d("pmlsigma"), rtol=1e-12, atol=1e-12)
    np.testing.assert_array_equal(export_i(s, "cempec"), ref.i("cempec") + 1)
    for a in ("Z_0", "Z_1", "Y_0", "Y_1"):
        np.testing.assert_allclose(export_d(s, a), ref.d(a), rtol=1e-14)


def test_box_builder_rejects_bad_pml():
    lib = L.load()
    n = C.c_long()
    base = dict(N=3, nel=(4, 4, 4), lo=(0, 0, 0), hi=(1, 1, 1), bc=(2, 0, 0))
    for pml in ((0, 3.0, 1e-8), (3, 3.0, 1e-8), (1, 0.5, 1e-8), (1, 3.0, 0.0), (1, 3.0, 2.0)):
        s, _ = box_struct(base, pml=pml)  # thickness 3 of 4 elements: the layers collide
        assert lib.nekgpu_box_export_d(C.byref(s), b"bmn", None, C.byref(n)) == -1, pml
