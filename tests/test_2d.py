"""2-D TE / TM forms (the reference's ldim = 2 build, param(4) = 1 TE, 2 TM).

CPU: the oracle's 2-D branches pass the reference's own known-answer tests,
tests/2dboxpec and tests/2dboxper (3x3 quadrilaterals, N=8, dt 0.005, 1000
steps, per-component L2 / Linf tolerances of their userchk), for TE and TM.
GPU: nekgpu_init2d from the oracle's arrays matches the oracle bit for bit
(PEC, periodic and mixed boxes, with and without materials) and passes the
same known answers; what 2-D does not support is refused.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import oracle_arrays
from nekcem_gb300 import MaxwellGPU, cases
from nekcem_gb300 import _lib as L
from oracle import refcpu as R

TE, TM = cases.TE, cases.TM
PEC, PER = 0, 1


def known_answer(name, mode, gpu: bool):
    cs = cases.CASES_2D[name]
    ref = R.RefBox2D(cs["N"], cs["nel"], cs["lo"], cs["hi"], cs["bc"], mode)
    x, y, z = (a.copy() for a in ref.coords())
    sol = cs["sol"](mode)
    H, E = sol(x, y, z, 0.0)
    if gpu:
        g = MaxwellGPU.from_arrays2d(oracle_arrays(ref), ref.n, ref.nelt, mode)
        g.set_state(H, E)
        t = g.run(cs["nsteps"], 0.0, cs["dt"])
        Hg, Eg = g.get_state()
        g.close()
    else:
        ref.set_state(H, E)
        ref.run(cs["nsteps"], 0.0, cs["dt"])
        t = cs["nsteps"] * cs["dt"]
        Hg, Eg = ref.hn.copy(), ref.en.copy()
    Hx, Ex = sol(x, y, z, t)
    res = []
    for a, b in [(Hg[q], Hx[q]) for q in range(3)] + [(Eg[q], Ex[q]) for q in range(3)]:
        res.append(ref.cem_error(a, b))
    ref.close()
    active = [0, 1, 5] if mode == TM else [2, 3, 4]
    for q in range(6):
        l2, li = res[q]
        if q in active:
            assert l2 <= cs["l2tol"] and li <= cs["linftol"], (name, mode, q, l2, li)
        else:
            assert l2 == 0.0 and li == 0.0, (name, mode, q, l2, li)
    return res


@pytest.mark.parametrize("name", list(cases.CASES_2D))
@pytest.mark.parametrize("mode", [TE, TM])
def test_oracle_2d_known_answers(name, mode):
    known_answer(name, mode, gpu=False)


def test_oracle_2d_geometry():
    """Affine quads: cofactors, Jacobian, normals and edge weights."""
    ref = R.RefBox2D(4, (3, 2), (0.0, -1.0), (1.5, 1.0), (PEC, PER), TE)
    hx, hy = 0.5, 1.0
    np.testing.assert_allclose(ref.d("rxm1"), hy / 2, rtol=1e-12)
    np.testing.assert_allclose(ref.d("sym1"), hx / 2, rtol=1e-12)
    np.testing.assert_allclose(ref.d("rym1"), 0, atol=1e-13)
    np.testing.assert_allclose(ref.d("jacm1"), hx * hy / 4, rtol=1e-12)
    assert ref.volvm1 == pytest.approx(1.5 * 2.0, rel=1e-12)
    n = ref.n
    unx = ref.d("unx").reshape(-1, 4, n)
    uny = ref.d("uny").reshape(-1, 4, n)
    np.testing.assert_array_equal(uny[:, 0], -1.0)  # s = -1 face
    np.testing.assert_array_equal(unx[:, 1], 1.0)   # r = +1
    np.testing.assert_array_equal(uny[:, 2], 1.0)   # s = +1
    np.testing.assert_array_equal(unx[:, 3], -1.0)  # r = -1
    w = ref.d("wxm1")
    area = ref.d("area").reshape(-1, 4, n)
    np.testing.assert_allclose(area[:, 0], np.broadcast_to(hx / 2 * w, area[:, 0].shape), rtol=1e-12)
    np.testing.assert_allclose(area[:, 1], np.broadcast_to(hy / 2 * w, area[:, 1].shape), rtol=1e-12)
    assert len(ref.i("cempec")) == 4 * n  # two faces on each x wall (y is periodic)
    ref.close()


# ---- GPU ----------------------------------------------------------------------------
MESHES_2D = {
    "pec": dict(N=5, nel=(3, 2), lo=(0.0, 0.0), hi=(1.5, 1.0), bc=(PEC, PEC)),
    "periodic": dict(N=8, nel=(2, 3), lo=(0.0, 0.0), hi=(1.0, 1.0), bc=(PER, PER)),
    "mixed": dict(N=7, nel=(4, 2), lo=(-1.0, 0.0), hi=(1.0, 0.5), bc=(PER, PEC)),
}


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(MESHES_2D))
@pytest.mark.parametrize("mode", [TE, TM])
@pytest.mark.parametrize("materials", [False, True])
def test_2d_bit_exact(name, mode, materials):
    b = MESHES_2D[name]
    ref = R.RefBox2D(b["N"], b["nel"], b["lo"], b["hi"], b["bc"], mode)
    x, y, z = ref.coords()
    if materials:
        ref.set_materials(1.0 + 0.5 * np.sin(3 * x) ** 2, 1.0 + 0.3 * np.cos(2 * y) ** 2)
    g = MaxwellGPU.from_arrays2d(oracle_arrays(ref), ref.n, ref.nelt, mode)
    rng = np.random.default_rng(mode * 10 + len(name))
    H = rng.standard_normal((3, ref.npts))
    E = rng.standard_normal((3, ref.npts))
    ref.set_state(H, E)
    g.set_state(H, E)
    dt = 0.2 * ref.dxmin()
    ref.run(5, 0.0, dt)
    g.run(5, 0.0, dt)
    Hg, Eg = g.get_state()
    np.testing.assert_array_equal(Hg, ref.hn)
    np.testing.assert_array_equal(Eg, ref.en)
    g.close(); ref.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(MESHES_2D))
@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("mode", [TE, TM])
def test_2d_source_bit_exact(name, kind, mode):
    """usersrc in the 2-D forms: a Gaussian line source on the out-of-plane
    field (E_z in TM, H_z in TE; z ignored), added after the lift and before
    the inverse mass, as the reference's 2-D cases do
    (tests/2dboxpml/2dboxpml.usr: srcez or srchz -= norm exp(..)
    sin(-omega t) bm1); Ricker (kind 0) or sin(f0 t) (kind 1) in time;
    bit-identical to the oracle over 5 steps from rest."""
    b = MESHES_2D[name]
    ref = R.RefBox2D(b["N"], b["nel"], b["lo"], b["hi"], b["bc"], mode)
    x, y, z = ref.coords()
    g = MaxwellGPU.from_arrays2d(oracle_arrays(ref), ref.n, ref.nelt, mode)
    xc = (0.5 * (b["lo"][0] + b["hi"][0]), 0.5 * (b["lo"][1] + b["hi"][1]), 0.0)
    src = dict(xc=xc, sigma=0.15, amp=2.0, f0=2.0, t0=0.05)
    for obj in (ref, g):
        obj.set_source_kind(kind)
        obj.set_source(**src)
    zero = np.zeros((3, ref.npts))
    ref.set_state(zero, zero)
    g.set_state(zero, zero)
    dt = 0.2 * ref.dxmin()
    ref.run(5, 0.0, dt)
    g.run(5, 0.0, dt)
    Hg, Eg = g.get_state()
    out_of_plane = ref.en[2] if mode == TM else ref.hn[2]
    assert np.abs(out_of_plane).max() > 1e-6  # the source drove the field
    np.testing.assert_array_equal(Hg, ref.hn)
    np.testing.assert_array_equal(Eg, ref.en)
    g.close(); ref.close()


PML2D = 2  # REF_BC_PML / NEKGPU_BC_PML


def boxpml2d(gpu: bool, mode: int):
    """The reference's maxwell-2dboxpml-te / -tm (tests/2dboxpml, param(4) =
    1 | 2): 8 x 8 elements on [-1,1]^2 (usrdat2 scales the box), N=8, 'PML'
    on all four sides (2 layers, order 3, error 1e-8: params 77-79), a
    Gaussian line current I0 delta(x) delta(y) sin(omega t) on the
    out-of-plane field (E_z in TM, H_z in TE; width 0.1, omega = 2, norm
    1/(2 pi width^2)), zero initial fields, dt = 0.1 dxmin (CFL 0.1), 4000
    steps; usersol is zero and userchk asks L2 and Linf <= 1 on the mode's
    three components (the waves must leave through the PML)."""
    ref = R.RefBox2D(8, (8, 8), (-1.0, -1.0), (1.0, 1.0), (PML2D, PML2D), mode)
    ref.set_pml(2, 3.0, 1e-8)
    ref.pml = (2, 3.0, 1e-8)
    src = dict(xc=(0.0, 0.0, 0.0), sigma=0.1, amp=1.0 / (2 * np.pi * 0.01), f0=2.0, t0=0.0)
    obj = ref
    if gpu:
        obj = MaxwellGPU.from_arrays2d(oracle_arrays(ref), ref.n, ref.nelt, mode)
    obj.set_source_kind(1)
    obj.set_source(**src)
    zero = np.zeros((3, ref.npts))
    obj.set_state(zero, zero)
    dt = 0.1 * ref.dxmin()
    obj.run(4000, 0.0, dt)
    if gpu:
        H, E = obj.get_state()
        obj.close()
    else:
        H, E = ref.hn.copy(), ref.en.copy()
    for comp in ((H[0], H[1], E[2]) if mode == TM else (E[0], E[1], H[2])):
        l2, li = ref.cem_error(comp, np.zeros_like(comp))
        assert l2 <= 1.0 and li <= 1.0, (l2, li)
        assert li > 1e-3  # the source did drive the field
    ref.close()


@pytest.mark.parametrize("mode", [TE, TM])
def test_oracle_2dboxpml_known_answer(mode):
    boxpml2d(False, mode)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [TE, TM])
def test_2dboxpml_known_answer_gpu(mode):
    boxpml2d(True, mode)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [TE, TM])
@pytest.mark.parametrize("materials", [False, True])
def test_2d_pml_bit_exact(mode, materials):
    """pml_step and the auxiliary fields' RK update in the 2-D form: state and
    pmlbn / pmldn bit-identical to the oracle over 5 steps ('PML' on x, PEC
    or periodic on y, random fields, the auxiliary fields started at mu H and
    eps E as the reference's userini sets them)."""
    bc = (PML2D, PEC if mode == TE else PER)
    ref = R.RefBox2D(5, (6, 4), (0.0, 0.0), (1.5, 1.0), bc, mode)
    x, y, z = ref.coords()
    if materials:
        ref.set_materials(1.0 + 0.5 * np.sin(3 * x) ** 2, 1.0 + 0.3 * np.cos(2 * y) ** 2)
    ref.set_pml(2, 3.0, 1e-6)
    ref.pml = (2, 3.0, 1e-6)
    g = MaxwellGPU.from_arrays2d(oracle_arrays(ref), ref.n, ref.nelt, mode)
    rng = np.random.default_rng(7 + mode)
    H = np.zeros((3, ref.npts)); E = np.zeros((3, ref.npts))
    Hact, Eact = ((0, 1), (2,)) if mode == TM else ((2,), (0, 1))
    for q in Hact: H[q] = rng.standard_normal(ref.npts)
    for q in Eact: E[q] = rng.standard_normal(ref.npts)
    eps, mu = ref.d("permittivity"), ref.d("permeability")
    ref.set_state(H, E); g.set_state(H, E)
    ref.d("pmlbn")[:] = (mu * H).ravel(); ref.d("pmldn")[:] = (eps * E).ravel()
    g.set_array("pmlbn", mu * H); g.set_array("pmldn", eps * E)
    dt = 0.2 * ref.dxmin()
    ref.run(5, 0.0, dt)
    g.run(5, 0.0, dt)
    Hg, Eg = g.get_state()
    np.testing.assert_array_equal(Hg, ref.hn)
    np.testing.assert_array_equal(Eg, ref.en)
    np.testing.assert_array_equal(g.array("pmlbn"), ref.d("pmlbn"))
    np.testing.assert_array_equal(g.array("pmldn"), ref.d("pmldn"))
    assert np.abs(ref.d("pmldn")).max() > 0
    g.close(); ref.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(cases.CASES_2D))
@pytest.mark.parametrize("mode", [TE, TM])
def test_2d_known_answers_gpu(name, mode):
    known_answer(name, mode, gpu=True)


@pytest.mark.gpu
def test_2d_refusals(tmp_path):
    ref = R.RefBox2D(3, (2, 2), (0.0, 0.0), (1.0, 1.0), (PEC, PEC), TM)
    arrays = oracle_arrays(ref)
    g = MaxwellGPU.from_arrays2d(arrays, ref.n, ref.nelt, TM)
    g.set_state(np.zeros((3, g.npts)), np.zeros((3, g.npts)))
    calls = [
        lambda: g.set_dispersive(g.DRUDE, np.ones((2, g.npts)), np.arange(3)),
        lambda: g.adjoint_gradient(1, 0.0, 0.01, np.ones(g.npts)),
        lambda: g.write_vtk(str(tmp_path / "x.vtk")),
    ]
    for call in calls:
        with pytest.raises(L.NekgpuError) as e:
            call()
        assert e.value.status == -8
    g.close()
    bad = dict(arrays)
    cf = bad["cemface"].copy()
    cf[[0, 1]] = cf[[1, 0]]  # not the reference's face numbering
    bad["cemface"] = cf
    with pytest.raises(L.NekgpuError) as e:
        MaxwellGPU.from_arrays2d(bad, ref.n, ref.nelt, TM)
    assert e.value.status == -2
    with pytest.raises(L.NekgpuError) as e:
        MaxwellGPU.from_arrays2d(arrays, ref.n, ref.nelt, 3)
    assert e.value.status == -1
    ref.close()
