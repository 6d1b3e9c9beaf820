"""Pins of the FP64 oracle (no GPU): GLL points/weights against 30-digit
values, the derivative matrix on polynomials, the reference's own
known-answer tests at its own tolerances, the face exchange against the
reference's compiled gs.c (committed golden vectors), and the impedance
semantics of cem_maxwell_materials."""
import json
import os

import numpy as np
import pytest

from oracle import refcpu as R
from nekcem_gb300 import cases

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
R.set_threads(os.cpu_count() or 1)


@pytest.mark.parametrize("N", list(range(1, 16)))
def test_zwgll_against_30_digit_values(N):
    g = json.load(open(os.path.join(GOLD, "gll.json")))[str(N)]
    z, w = R.zwgll(N + 1)
    # the Jacobi-recursion algorithm of the reference is accurate to a few ulp
    np.testing.assert_allclose(z, np.array([float(v) for v in g["z"]]), rtol=0, atol=1e-14)
    np.testing.assert_allclose(w, np.array([float(v) for v in g["w"]]), rtol=2e-14, atol=0)


@pytest.mark.parametrize("N", [2, 4, 5, 7, 8, 11])
def test_dgll_differentiates_polynomials_exactly(N):
    z, _ = R.zwgll(N + 1)
    D, _ = R.dgll(z)
    for p in range(N + 1):
        f = z ** p
        df = p * z ** (p - 1) if p > 0 else 0 * z
        np.testing.assert_allclose(D @ f, df, atol=5e-13 * max(1, N * N))


def _known_answer(name):
    c = cases.make(name)
    m = R.RefBox(c.N, c.nel, c.lo, c.hi, c.bc)
    x, y, z = m.coords()
    m.set_state(*c.exact(x, y, z, 0.0))
    t = m.run(c.nsteps, 0.0, c.dt)
    H, E = c.exact(x, y, z, t)
    errs = [m.cem_error(m.hn[q], H[q]) for q in range(3)] + [m.cem_error(m.en[q], E[q]) for q in range(3)]
    return c, np.array(errs)


def test_known_answer_3dboxpec():
    """tests/3dboxpec: 27 el, N=8, dt=0.005, 1000 steps; L2 <= 5e-8, Linf <= 5e-7
    per component (tests/3dboxpec/3dboxpec.usr:186-210)."""
    c, e = _known_answer("3dboxpec")
    assert np.all(e[:, 0] <= c.l2tol), e
    assert np.all(e[:, 1] <= c.linftol), e


def test_known_answer_3dboxper():
    """tests/3dboxper: 4x4x8 el, N=8, dt=2e-4, 50 steps; L2 <= 5e-10, Linf <= 5e-9
    (tests/3dboxper/3dboxper.usr:169-193)."""
    c, e = _known_answer("3dboxper")
    assert np.all(e[:, 0] <= c.l2tol), e
    assert np.all(e[:, 1] <= c.linftol), e


def test_gs_against_reference_gs_golden():
    g = np.load(os.path.join(GOLD, "gs_ref.npz"))
    t = 0
    while f"m{t}_meta" in g:
        meta = g[f"m{t}_meta"]
        N, nel, bc = int(meta[0]), tuple(int(v) for v in meta[1:4]), tuple(int(v) for v in meta[4:7])
        m = R.RefBox(N, nel, (0, 0, 0), (1, 1, 1), bc)
        np.testing.assert_array_equal(m.l("glo_face"), g[f"m{t}_ids"])
        u = g[f"m{t}_in"].copy()
        m.call("gs_op_fields", u.ctypes.data_as(R.C.POINTER(R.C.c_double)), m.nxzfl, 6)
        np.testing.assert_array_equal(u, g[f"m{t}_out"])
        t += 1
    assert t >= 3


def test_gs_against_reference_gs_live():
    """When the reference tree is present (oracle/build_ref.sh finds it, or
    NEKCEM_REFERENCE_ROOT names it), build its gs.c and compare live."""
    import ctypes as C
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([os.path.join(root, "oracle", "build_ref.sh")], capture_output=True)
    if r.returncode == 3:
        pytest.skip("reference tree not present")
    assert r.returncode == 0, r.stderr
    L = C.CDLL(os.path.join(root, "oracle", "_ref", "libjlgs.so"))
    L.jlgs_apply.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int]
    m = R.RefBox(5, (3, 2, 4), (0, 0, 0), (1, 2, 3), (1, 0, 1))
    ids = m.l("glo_face").copy()
    u = np.random.default_rng(9).standard_normal(6 * m.nxzfl)
    a = u.copy(); b = u.copy()
    assert L.jlgs_apply(ids.ctypes.data, m.nxzfl, a.ctypes.data, m.nxzfl, 6) == 0
    m.call("gs_op_fields", b.ctypes.data_as(C.POINTER(C.c_double)), m.nxzfl, 6)
    np.testing.assert_array_equal(a, b)


def test_materials_impedance_semantics():
    """Z_0 = (Z- + Z+)/2, Z_1 = Z+ on paired faces; Z_0 = Z_1 = Z- on PEC
    faces (src/cem_maxwell.F:262-325)."""
    m = R.RefBox(3, (2, 1, 1), (0, 0, 0), (2, 1, 1), (0, 0, 0))
    x, y, z = m.coords()
    eps = np.repeat([1.0, 4.0], m.npts // 2)  # element 0 eps=1, element 1 eps=4
    mu = np.ones(m.npts)
    m.set_materials(eps, mu)
    Z0, Z1, Y0, Y1 = m.d("Z_0"), m.d("Z_1"), m.d("Y_0"), m.d("Y_1")
    n2 = m.nxzf
    # element 0 slot 1 (r=+1) faces element 1 (Z = 0.5, Y = 2)
    sl = slice(1 * n2, 2 * n2)
    np.testing.assert_allclose(Z0[sl], 0.75); np.testing.assert_allclose(Z1[sl], 0.5)
    np.testing.assert_allclose(Y0[sl], 1.5); np.testing.assert_allclose(Y1[sl], 2.0)
    # element 0 slot 3 (r=-1) is a PEC wall
    sl = slice(3 * n2, 4 * n2)
    np.testing.assert_allclose(Z0[sl], 1.0); np.testing.assert_allclose(Z1[sl], 1.0)
    # ebm1 = 1/(eps*bm1)
    np.testing.assert_allclose(m.d("ebm1"), 1.0 / (eps * m.d("bm1")))


def test_cavity_p_convergence():
    """The oracle converges spectrally on the TM110 cavity mode."""
    errs = []
    for N in (3, 5, 7):
        c = cases.make("cavity", N=N, nel=(2, 2, 2), nsteps=40)
        m = R.RefBox(c.N, c.nel, c.lo, c.hi, c.bc)
        x, y, z = m.coords()
        dt = 0.1 * c.timestep(x, y, z)
        m.set_state(*c.exact(x, y, z, 0.0))
        t = m.run(c.nsteps, 0.0, dt)
        H, E = c.exact(x, y, z, t)
        errs.append(m.cem_error(m.en[2], E[2])[0])
    assert errs[0] > 20 * errs[1] > 20 * 20 * errs[2] * 0.05, errs


def test_dt_rule():
    """dt = 0.5 * (smallest adjacent GLL spacing); get_dxmin restated in numpy
    agrees with the oracle's get_dxmin."""
    c = cases.make("cavity")
    m = R.RefBox(c.N, c.nel, c.lo, c.hi, c.bc)
    x, y, z = m.coords()
    assert abs(cases.get_dxmin(x, y, z, c.N + 1, c.nelt) - m.dxmin()) < 1e-15
    z7, _ = R.zwgll(8)
    np.testing.assert_allclose(c.timestep(x, y, z), 0.5 * (z7[1] - z7[0]) * 0.125, rtol=1e-12)


# ---- PML (src/cem_maxwell_pml.F) -------------------------------------------------
def test_oracle_pml_layers_and_sigma():
    """6^3 box on [-1,1]^3 with 'PML' on every face, one layer: the outer
    shell of 152 elements is tagged, the extents are the layer boundaries and
    sigma grows as sigmamax ((x - inner)/(outer - inner))^order with
    sigmamax = -(order + 1) ln(referr) / (2 eta width)."""
    ref = R.RefBox(3, (6, 6, 6), (-1, -1, -1), (1, 1, 1), (2, 2, 2))
    ref.set_pml(1, 3.0, 1e-8)
    tag = ref.i("pmltag")
    assert (tag != 0).sum() == 6 ** 3 - 4 ** 3
    np.testing.assert_allclose(ref.d("pmlinner"), [-2 / 3, 2 / 3] * 3, rtol=1e-14)
    np.testing.assert_allclose(ref.d("pmlouter"), [-1, 1] * 3, rtol=1e-14)
    x = ref.coords()[0]
    sx = ref.d("pmlsigma")[:ref.npts]
    smax = -(3.0 + 1) * np.log(1e-8) / (2 * 1.0 * (1 / 3))
    right = x > 2 / 3
    np.testing.assert_allclose(sx[right], smax * ((x[right] - 2 / 3) / (1 / 3)) ** 3, rtol=1e-12,
                               atol=1e-12)
    assert np.all(sx[np.abs(x) < 2 / 3 - 1e-12] == 0)
    # PML faces are in the PEC list and are not doubled in the materials
    assert R.lib().ref_size(ref._c, b"ncempec") == 6 * 36 * 16
    assert np.all(ref.d("Z_1")[ref.i("cempec")] == 0)


def test_oracle_3dboxpml_short_run_bounded():
    """The reference's tests/3dboxpml setup (6^3 el on [-1,1]^3, all faces
    'PML', thickness 1, order 3, error 1e-8, Gaussian dipole sin(2t), zero
    initial fields, dt = 0.1 dxmin) at N=4 for 300 steps: the fields stay
    below the reference's bound 1 (L2 and Linf), and the PML elements carry
    non-zero auxiliary fields once the wave reaches them."""
    R.set_threads(os.cpu_count() or 1)
    ref = R.RefBox(4, (6, 6, 6), (-1, -1, -1), (1, 1, 1), (2, 2, 2))
    ref.set_pml(1, 3.0, 1e-8)
    ref.set_source_kind(1)
    ref.set_source((0.0, 0.0, 0.0), 0.1, 1.0, 2.0, 0.0)
    dt = 0.1 * ref.dxmin()
    ref.set_state(np.zeros((3, ref.npts)), np.zeros((3, ref.npts)))
    ref.run(300, 0.0, dt)
    for comp in list(ref.hn) + list(ref.en):
        l2, li = ref.cem_error(comp.copy(), np.zeros(ref.npts))
        assert l2 <= 1.0 and li <= 1.0
    assert np.abs(ref.d("pmldn")).max() > 0
