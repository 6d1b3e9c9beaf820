"""GPU parity: the CUDA forms against the FP64 oracle through the C ABI.

Bars (the tolerance of each assertion is written beside it):
  * plain form on the reference's own arrays: bit-identical to the oracle,
    routine by routine and over many steps;
  * fused FP64 form: <= 1e-12 relative per step (max-norm over the 6
    components, relative to the field's max), both from the reference's
    arrays (drop-in init) and from the library's own box builder;
  * mixed form: per step <= 1e-9 relative (MIXED_TOL: the exact-hi FP32
    contractions carry ~2^-34 of sum|D||u|; a contraction that lost the low
    part of a split would sit near 2^-24 ~ 6e-8 and fail), and the L2 error
    against the analytic solution within 1.5x of the FP64 one.
"""
MIXED_TOL = 1e-9
import numpy as np
import pytest

from oracle import refcpu as R
from nekcem_gb300 import MaxwellGPU, NekgpuError, cases
from tests.helpers import (gpu_from_box, gpu_from_ref, make_ref, random_fields, rel_err,
                           smooth_fields)

pytestmark = pytest.mark.gpu
PEC, PER = cases.PEC, cases.PERIODIC
R.set_threads(8)


def eps_bumpy(x, y, z):
    return 1.0 + 0.5 * np.sin(3 * x) ** 2 + 0.25 * np.cos(2 * y + z)


def mu_bumpy(x, y, z):
    return 1.0 + 0.3 * np.cos(x - 2 * z) ** 2


# small meshes covering the boundary mixes, orders and material cases
MESHES = {
    "pec_n5": dict(N=4, nel=(3, 2, 2), lo=(0, 0, 0), hi=(1, 1.5, 0.75), bc=(PEC, PEC, PEC)),
    "mixed_bc": dict(N=5, nel=(3, 2, 2), lo=(-1, 0, 0), hi=(1, 1, 2), bc=(PER, PEC, PER)),
    "periodic_n8": dict(N=7, nel=(2, 2, 2), lo=(0, 0, 0), hi=(6.3, 6.3, 6.3), bc=(PER, PER, PER)),
    "odd_n9": dict(N=8, nel=(2, 1, 2), lo=(0, 0, 0), hi=(1, 1, 1), bc=(PEC, PER, PEC)),
    "n3": dict(N=2, nel=(2, 3, 2), lo=(0, 0, 0), hi=(1, 1, 1), bc=(PEC, PEC, PER)),
    "single_periodic": dict(N=5, nel=(1, 1, 1), lo=(0, 0, 0), hi=(2, 2, 2), bc=(PER, PER, PER)),
    "single_pec": dict(N=6, nel=(1, 1, 1), lo=(0, 0, 0), hi=(1, 1, 1), bc=(PEC, PEC, PEC)),
    # N=7 with non-cubic elements and fewer elements than SMs (the mixed
    # form's two-threads-per-line kernel)
    "rect_n7": dict(N=7, nel=(2, 3, 1), lo=(0, 0, 0), hi=(1, 2, 0.5), bc=(PEC, PER, PEC)),
}


def ref_for(name, materials=False, C0=1.0):
    m = MESHES[name]
    return make_ref(m["N"], m["nel"], m["lo"], m["hi"], m["bc"],
                    eps=eps_bumpy if materials else None, mu=mu_bumpy if materials else None,
                    C0=C0)


# ---------------------------------------------------------------------------
# plain form: bit-identical, routine by routine
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("mesh", ["pec_n5", "mixed_bc", "odd_n9"])
@pytest.mark.parametrize("materials", [False, True])
def test_plain_routines_bit_exact(mesh, materials):
    ref = ref_for(mesh, materials)
    g = gpu_from_ref(ref, "plain")
    H, E = random_fields(ref.npts, 1)
    ref.set_state(H, E)
    g.set_state(H, E)
    npts, nf = ref.npts, ref.nxzfl
    # maxwell_wght_curl x2 + chsign
    ref.call("cem_maxwell"); g.call("cem_maxwell")
    np.testing.assert_array_equal(g.work("reshn"), ref.d("reshn"))
    np.testing.assert_array_equal(g.work("resen"), ref.d("resen"))
    ref.call("restrict_to_face"); g.call("restrict_to_face")
    np.testing.assert_array_equal(g.work("fhn"), ref.d("fhn"))
    np.testing.assert_array_equal(g.work("fen"), ref.d("fen"))
    ref.call("flux3d"); g.call("flux3d")
    np.testing.assert_array_equal(g.work("srflx"), ref.d("srflx"))
    ref.call("add_flux_to_res"); g.call("add_flux_to_res")
    np.testing.assert_array_equal(g.work("reshn"), ref.d("reshn"))
    np.testing.assert_array_equal(g.work("resen"), ref.d("resen"))
    ref.call("invqmass"); g.call("invqmass")
    np.testing.assert_array_equal(g.work("reshn"), ref.d("reshn"))
    np.testing.assert_array_equal(g.work("resen"), ref.d("resen"))
    # rk_maxwell_ab of stage 2 (a != 0) after seeding k
    kH, kE = random_fields(npts, 2)
    ref.d("khn")[:] = kH.ravel(); ref.d("ken")[:] = kE.ravel()
    g.set_rk_register(kH, kE)
    a, b, c = R.rk_coeffs()
    dt = 1e-3
    # rk_maxwell_ab == rk4_upd on the 6 components with (b[1], a[1], dt),
    # restated with numpy (no fused multiply-add)
    hn, en = ref.hn, ref.en
    khn = ref.d("khn").reshape(3, npts); ken = ref.d("ken").reshape(3, npts)
    resh = ref.d("reshn").reshape(3, npts); rese = ref.d("resen").reshape(3, npts)
    khn[...] = a[1] * khn + dt * resh
    hn[...] = hn + b[1] * khn
    ken[...] = a[1] * ken + dt * rese
    en[...] = en + b[1] * ken
    g.call("rk_maxwell_ab", 2, dt)
    gH, gE = g.get_state()
    gkH, gkE = g.get_rk_register()
    np.testing.assert_array_equal(gkH, khn)
    np.testing.assert_array_equal(gkE, ken)
    np.testing.assert_array_equal(gH, hn)
    np.testing.assert_array_equal(gE, en)
    g.close(); ref.close()


def test_plain_gs_op_fields_bit_exact():
    ref = ref_for("mixed_bc")
    g = gpu_from_ref(ref, "plain")
    u = np.random.default_rng(5).standard_normal(6 * ref.nxzfl)
    want = u.copy()
    ref.call("gs_op_fields", want.ctypes.data_as(R.C.POINTER(R.C.c_double)), ref.nxzfl, 6)
    got = g.gs_op_fields(u, 6)
    np.testing.assert_array_equal(got, want)
    g.close(); ref.close()


@pytest.mark.parametrize("mesh", ["pec_n5", "mixed_bc", "periodic_n8", "single_periodic"])
def test_plain_steps_bit_exact(mesh):
    ref = ref_for(mesh, materials=True)
    g = gpu_from_ref(ref, "plain")
    H, E = smooth_fields(ref, 3)
    ref.set_state(H, E); g.set_state(H, E)
    dt = 0.2 * ref.dxmin()
    t_ref = ref.run(20, 0.0, dt)
    t_gpu = g.run(20, 0.0, dt)
    assert t_ref == t_gpu
    gH, gE = g.get_state()
    np.testing.assert_array_equal(gH, ref.hn)
    np.testing.assert_array_equal(gE, ref.en)
    g.close(); ref.close()


# ---------------------------------------------------------------------------
# fused forms: 1e-12 per step (FP64), MIXED_TOL per step (mixed)
# ---------------------------------------------------------------------------
FUSED_MESHES = ["pec_n5", "mixed_bc", "periodic_n8", "odd_n9", "n3", "single_periodic",
                "single_pec"]


@pytest.mark.parametrize("init", ["arrays", "box"])
@pytest.mark.parametrize("mesh", FUSED_MESHES)
@pytest.mark.parametrize("materials", [False, True])
def test_fused64_per_step(mesh, init, materials):
    ref = ref_for(mesh, materials)
    g = (gpu_from_ref if init == "arrays" else gpu_from_box)(ref, "fused64")
    H, E = smooth_fields(ref, 7)
    dt = 0.2 * ref.dxmin()
    t = 0.0
    for step in range(4):  # one step from identical states, four times along the path
        ref.set_state(H, E); g.set_state(H, E)
        ref.op_rk(t, dt)
        g.run(1, t, dt)
        gH, gE = g.get_state()
        err = rel_err(gH, gE, ref.hn, ref.en)
        assert err <= 1e-12, f"step {step}: relative error {err:.3e} > 1e-12"
        H, E = ref.hn.copy(), ref.en.copy()
        t += dt
    g.close(); ref.close()


@pytest.mark.parametrize("mesh", list(MESHES))
@pytest.mark.parametrize("materials", [False, True])
def test_mixed_per_step(mesh, materials):
    """Four steps along the oracle's path, each from the oracle's state."""
    ref = ref_for(mesh, materials)
    g = gpu_from_box(ref, "mixed")
    H, E = smooth_fields(ref, 11)
    dt = 0.2 * ref.dxmin()
    t = 0.0
    for step in range(4):
        ref.set_state(H, E); g.set_state(H, E)
        ref.op_rk(t, dt)
        g.run(1, t, dt)
        gH, gE = g.get_state()
        err = rel_err(gH, gE, ref.hn, ref.en)
        assert err <= MIXED_TOL, f"step {step}: relative error {err:.3e} > {MIXED_TOL:g}"
        H, E = ref.hn.copy(), ref.en.copy()
        t += dt
    g.close(); ref.close()


def test_fused64_many_steps_drift():
    """100 steps of the FP64 fused form stay within 100 x 1e-12 of the oracle."""
    ref = ref_for("mixed_bc", materials=True)
    g = gpu_from_ref(ref, "fused64")
    H, E = smooth_fields(ref, 13)
    dt = 0.2 * ref.dxmin()
    ref.set_state(H, E); g.set_state(H, E)
    ref.run(100, 0.0, dt)
    g.run(100, 0.0, dt)
    gH, gE = g.get_state()
    assert rel_err(gH, gE, ref.hn, ref.en) <= 1e-10
    g.close(); ref.close()


# ---------------------------------------------------------------------------
# known answers of the reference's own tests, on every form
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("form", ["plain", "fused64", "mixed"])
@pytest.mark.parametrize("name", ["3dboxpec", "3dboxper"])
def test_reference_known_answer(name, form):
    c = cases.make(name)
    g = MaxwellGPU.from_box(c.N, c.nel, c.lo, c.hi, c.bc, form=form)
    x, y, z = g.coords()
    H, E = c.init_fields(x, y, z)
    g.set_state(H, E)
    t = g.run(c.nsteps, 0.0, c.dt)
    l2, linf = g.cem_error(*c.exact(x, y, z, t))
    # the reference's own tolerances, for the mixed form too
    assert np.all(l2 <= c.l2tol), l2
    assert np.all(linf <= c.linftol), linf
    g.close()


@pytest.mark.parametrize("name", ["cavity", "planewave"])
def test_mixed_l2_within_1p5x_of_fp64(name):
    """Full configs: 1000-step cavity (4^3, N=7) and 2000-step plane wave
    (16^3, N=7); mixed L2 error vs analytic within 1.5x of FP64's."""
    c = cases.make(name)
    res = {}
    for form in ("fused64", "mixed"):
        g = MaxwellGPU.from_box(c.N, c.nel, c.lo, c.hi, c.bc, form=form)
        x, y, z = g.coords()
        dt = c.timestep(x, y, z)
        g.set_state(*c.init_fields(x, y, z))
        t = g.run(c.nsteps, 0.0, dt)
        l2, _ = g.cem_error(*c.exact(x, y, z, t))
        res[form] = np.sqrt(np.sum(l2 ** 2))
        g.close()
    assert res["mixed"] <= 1.5 * res["fused64"], res


def test_cavity_fp64_matches_oracle_l2():
    """1000-step cavity: the FP64 fused L2 error vs analytic equals the
    oracle's to 1e-6 relative (the fields agree to ~1e-12 per step)."""
    c = cases.make("cavity")
    ref = make_ref(c.N, c.nel, c.lo, c.hi, c.bc, threads=8)
    x, y, z = ref.coords()
    dt = c.timestep(x, y, z)
    ref.set_state(*c.exact(x, y, z, 0.0))
    t = ref.run(c.nsteps, 0.0, dt)
    H, E = c.exact(x, y, z, t)
    l2_ref = np.array([ref.cem_error(ref.hn[q], H[q])[0] for q in range(3)]
                      + [ref.cem_error(ref.en[q], E[q])[0] for q in range(3)])
    g = gpu_from_ref(ref, "fused64")
    g.set_state(*c.exact(x, y, z, 0.0))
    tg = g.run(c.nsteps, 0.0, dt)
    assert tg == t
    l2_gpu, _ = g.cem_error(H, E)
    np.testing.assert_allclose(l2_gpu, l2_ref, rtol=1e-6, atol=1e-14)
    g.close(); ref.close()


# ---------------------------------------------------------------------------
# source term, host entry points, errors
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("form", ["plain", "fused64", "mixed"])
def test_source_parity(form):
    """Gaussian/Ricker E_z source from a zero state: the fields are the
    source's alone.  Plain: bit-identical over 10 steps; fused FP64: 1e-11
    after 10 steps; mixed: each of the 10 steps from the oracle's state
    within MIXED_TOL."""
    ref = make_ref(5, (3, 3, 3), (0, 0, 0), (1, 1, 1), (PEC,) * 3, eps=eps_bumpy)
    src = dict(xc=(0.3, 0.45, 0.5), sigma=0.08, amp=2.0, f0=2.0, t0=0.1)
    ref.set_source(**src)
    g = gpu_from_box(ref, form) if form == "mixed" else gpu_from_ref(ref, form)
    g.set_source(**src)
    z = np.zeros((3, ref.npts))
    ref.set_state(z, z); g.set_state(z, z)
    dt = 0.2 * ref.dxmin()
    if form == "mixed":
        t = 0.0
        for step in range(10):
            H, E = ref.hn.copy(), ref.en.copy()
            g.set_state(H, E)
            ref.op_rk(t, dt)
            g.run(1, t, dt)
            gH, gE = g.get_state()
            if step > 0:  # step 0 starts from zero: the source alone
                err = rel_err(gH, gE, ref.hn, ref.en)
                assert err <= MIXED_TOL, f"step {step}: relative error {err:.3e}"
            t += dt
        g.close(); ref.close()
        return
    ref.run(10, 0.0, dt)
    g.run(10, 0.0, dt)
    gH, gE = g.get_state()
    if form == "plain":
        np.testing.assert_array_equal(gE, ref.en)
        np.testing.assert_array_equal(gH, ref.hn)
    else:
        assert rel_err(gH, gE, ref.hn, ref.en) <= 1e-11
    g.close(); ref.close()


def test_mixed_inverse_mass_pair_isolated():
    """The mixed form's FP64-class pieces apart from its FP32 contractions:
    from a zero state the first RK stage sees only the Gaussian/Ricker source
    (the split pairs are exactly zero, so contractions and flux add nothing).
    The stage multiplies the source's float pair by the dt-scaled inverse
    mass, held as a float pair (hi = the top 24 mantissa bits, lo = the rest
    rounded to 24 bits: ~48 bits), and applies the FP64 RK update.  Against
    the oracle's FP64 stage: 1e-13 relative (an FP32 coefficient would give
    ~6e-8)."""
    ref = make_ref(5, (3, 3, 3), (0, 0, 0), (1, 1, 1), (PEC,) * 3, eps=eps_bumpy, mu=mu_bumpy)
    src = dict(xc=(0.3, 0.45, 0.5), sigma=0.08, amp=2.0, f0=2.0, t0=0.1)
    ref.set_source(**src)
    g = gpu_from_box(ref, "mixed")
    g.set_source(**src)
    z = np.zeros((3, ref.npts))
    ref.set_state(z, z); g.set_state(z, z)
    dt = 0.2 * ref.dxmin()
    ref.stage(1, 0.05, dt)
    g.stage(1, 0.05, dt)
    gH, gE = g.get_state()
    assert np.abs(ref.en[2]).max() > 0
    assert rel_err(gH, gE, ref.hn, ref.en) <= 1e-13
    g.close(); ref.close()


@pytest.mark.parametrize("form", ["plain", "fused64", "mixed"])
def test_op_rk_host_equals_device_steps(form):
    ref = ref_for("mixed_bc", materials=True)
    g1 = gpu_from_box(ref, form)
    g2 = gpu_from_box(ref, form)
    H, E = smooth_fields(ref, 17)
    dt = 0.2 * ref.dxmin()
    g1.set_state(H, E)
    g1.run(3, 0.0, dt)
    Hh, Eh = H.copy(), E.copy()
    t = 0.0
    for _ in range(3):
        g2.op_rk_host(Hh, Eh, t, dt)
        t += dt
    a_H, a_E = g1.get_state()
    np.testing.assert_array_equal(a_H, Hh)
    np.testing.assert_array_equal(a_E, Eh)
    g1.close(); g2.close(); ref.close()


@pytest.mark.parametrize("bc", [(1, 1, 1), (0, 0, 0), (1, 0, 1)], ids=["periodic", "pec", "mixed_bc"])
def test_op_rk_host_chunked_equals_device_steps(bc):
    """A mesh of a few thousand elements takes the wavefront host-field step
    of the mixed form (element chunks; stage s of a chunk waits for stage
    s-1 of the chunks holding its face partners, periodic wrap-around
    included; copies in and out overlapped with the stages): bit-identical
    to the same steps on a device-resident state, with the source term on."""
    from nekcem_gb300 import MaxwellGPU
    nel, lo, hi = (16, 12, 12), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)
    g1 = MaxwellGPU.from_box(7, nel, lo, hi, bc, form="mixed")
    g2 = MaxwellGPU.from_box(7, nel, lo, hi, bc, form="mixed")
    x, y, z = g1.coords()
    k = 2 * np.pi
    H = np.stack([np.sin(k * y) * np.cos(k * z), np.cos(k * x) * np.sin(k * z), 0.3 * np.sin(k * x)])
    E = np.stack([np.cos(k * y), np.sin(k * z) * np.cos(k * x), np.sin(k * x) * np.sin(k * y)])
    src = dict(xc=(0.4, 0.5, 0.6), sigma=0.1, amp=1.0, f0=2.0, t0=0.1)
    g1.set_source(**src); g2.set_source(**src)
    dt = 0.002
    g1.set_state(H, E)
    g1.run(4, 0.0, dt)
    Hh, Eh = H.copy(), E.copy()
    t, launches = 0.0, []
    for _ in range(4):
        g2.op_rk_host(Hh, Eh, t, dt)
        launches.append(g2.last_launches())
        t += dt
    a_H, a_E = g1.get_state()
    np.testing.assert_array_equal(a_H, Hh)
    np.testing.assert_array_equal(a_E, Eh)
    # every call runs as a wavefront of chunk launches (five per chunk)
    assert all(n >= 20 for n in launches), launches
    g1.close(); g2.close()


@pytest.mark.parametrize("bc", [(1, 1, 1), (1, 0, 1)], ids=["periodic", "mixed_bc"])
def test_op_rk_host_graph_equals_device_steps(bc):
    """Page-locked host arrays and no time-dependent source: the wavefront
    step is captured once per state parity as a CUDA graph and replayed.
    Six steps (two captures, four replays) are bit-identical to device
    steps and report the graph's kernels; after the arrays are unregistered
    the step is enqueued directly and still agrees."""
    from nekcem_gb300 import MaxwellGPU
    nel, lo, hi = (16, 12, 12), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)
    g1 = MaxwellGPU.from_box(7, nel, lo, hi, bc, form="mixed")
    g2 = MaxwellGPU.from_box(7, nel, lo, hi, bc, form="mixed")
    x, y, z = g1.coords()
    k = 2 * np.pi
    H = np.stack([np.sin(k * y) * np.cos(k * z), np.cos(k * x) * np.sin(k * z), 0.3 * np.sin(k * x)])
    E = np.stack([np.cos(k * y), np.sin(k * z) * np.cos(k * x), np.sin(k * x) * np.sin(k * y)])
    dt = 0.002
    g1.set_state(H, E)
    Hh, Eh = np.ascontiguousarray(H.copy()), np.ascontiguousarray(E.copy())
    g2.register_host(Hh); g2.register_host(Eh)
    t, launches = 0.0, []
    for _ in range(6):
        g2.op_rk_host(Hh, Eh, t, dt)
        launches.append(g2.last_launches())
        t += dt
    g1.run(6, 0.0, dt)
    a_H, a_E = g1.get_state()
    np.testing.assert_array_equal(a_H, Hh)
    np.testing.assert_array_equal(a_E, Eh)
    # the first call also scales the inverse-mass pairs for dt (one kernel)
    assert launches[0] - launches[1] in (0, 1), launches
    assert all(n == launches[1] and n >= 20 for n in launches[1:]), launches
    g2.unregister_host(Hh); g2.unregister_host(Eh)
    g2.op_rk_host(Hh, Eh, t, dt)
    g1.run(1, t, dt)
    a_H, a_E = g1.get_state()
    np.testing.assert_array_equal(a_H, Hh)
    np.testing.assert_array_equal(a_E, Eh)
    g1.close(); g2.close()


@pytest.mark.parametrize("form", ["fused64", "mixed"])
def test_deterministic(form):
    ref = ref_for("periodic_n8", materials=True)
    H, E = smooth_fields(ref, 19)
    dt = 0.2 * ref.dxmin()
    outs = []
    for _ in range(2):
        g = gpu_from_box(ref, form)
        g.set_state(H, E)
        g.run(10, 0.0, dt)
        outs.append(g.get_state())
        g.close()
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])


def test_state_leading_dimension():
    """hn(ld,3) with ld > npts (lpts1 of a SIZE file larger than the mesh)."""
    ref = ref_for("pec_n5")
    g = gpu_from_box(ref, "mixed")
    import ctypes as C
    from nekcem_gb300 import _lib as L
    ld = ref.npts + 37
    Hp = np.full((3, ld), 7.0); Ep = np.full((3, ld), -7.0)
    H, E = smooth_fields(ref, 23)
    Hp[:, :ref.npts] = H; Ep[:, :ref.npts] = E
    dp = L.dp
    L.check(L.load().nekgpu_set_state(g._h, Hp.ctypes.data_as(dp), Ep.ctypes.data_as(dp), ld), "set")
    out_H = np.full((3, ld), 3.0); out_E = np.full((3, ld), 3.0)
    L.check(L.load().nekgpu_get_state(g._h, out_H.ctypes.data_as(dp), out_E.ctypes.data_as(dp), ld), "get")
    np.testing.assert_array_equal(out_H[:, :ref.npts], H)
    np.testing.assert_array_equal(out_E[:, :ref.npts], E)
    assert np.all(out_H[:, ref.npts:] == 3.0) and np.all(out_E[:, ref.npts:] == 3.0)
    g.close(); ref.close()


def test_fused_forms_take_curvilinear_meshes_and_refuse_other_face_numbering():
    """A non-affine mesh runs in the fused forms through their curvilinear
    kernels; a face numbering other than the reference's (two cemface
    entries of one face swapped) is refused by the fused forms with
    NEKGPU_ERR_MESH and accepted by the plain form."""
    from tests.helpers import oracle_arrays
    ref = ref_for("pec_n5")
    arr = oracle_arrays(ref)
    arr["rxmn"] = arr["rxmn"] * (1.0 + 0.01 * np.sin(np.arange(ref.npts)))
    for form in ("mixed", "fused64"):
        MaxwellGPU.from_arrays(arr, ref.n, ref.nelt, form=form).close()
    arr = oracle_arrays(ref)
    cf = arr["cemface"].copy()
    cf[[0, 1]] = cf[[1, 0]]
    arr["cemface"] = cf
    for form in ("mixed", "fused64"):
        with pytest.raises(NekgpuError) as ei:
            MaxwellGPU.from_arrays(arr, ref.n, ref.nelt, form=form)
        assert ei.value.status == -2
    g = MaxwellGPU.from_arrays(arr, ref.n, ref.nelt, form="plain")
    g.close(); ref.close()


def test_errors_are_status_codes(monkeypatch):
    ref = ref_for("pec_n5")
    with pytest.raises(NekgpuError) as ei:
        MaxwellGPU.from_box(4, (2, 2, 2), (0, 0, 0), (1, 1, 1), (PEC, PEC, 7))
    assert ei.value.status == -1
    g = gpu_from_box(ref, "mixed")
    with pytest.raises(NekgpuError) as ei:
        g.stage(0, 0.0, 1e-3)  # stage index outside 1..5
    assert ei.value.status in (-1, -5)
    with pytest.raises(NekgpuError) as ei:
        g.call("cem_maxwell")  # per-routine entry points are plain-form only
    assert ei.value.status == -8
    g.close()
    # allocation failure, simulated by a device-memory budget
    monkeypatch.setenv("NEKGPU_MEM_BUDGET_MB", "1")
    with pytest.raises(NekgpuError) as ei:
        MaxwellGPU.from_box(7, (8, 8, 8), (0, 0, 0), (1, 1, 1), (PEC,) * 3, form="mixed")
    assert ei.value.status == -4
    ref.close()


def test_blowup_detection():
    ref = ref_for("pec_n5")
    g = gpu_from_box(ref, "mixed")
    H, E = smooth_fields(ref, 29)
    g.set_state(H, E)
    g.check_blowup()
    H[1, 5] = np.inf
    g.set_state(H, E)
    with pytest.raises(NekgpuError) as ei:
        g.check_blowup()
    assert ei.value.status == -6
    g.close(); ref.close()


def test_bounded_wait_runs_out_and_context_survives():
    """A device wait that nothing ends (an mbarrier no one arrives at) gives
    up after its poll budget and reports NEKGPU_ERR_TIMEOUT through the
    status word, without a fault; the same context then steps normally and
    matches a fresh one bit for bit."""
    ref = ref_for("pec_n5")
    g = gpu_from_box(ref, "mixed")
    assert g.selftest_wait(1000) == -7
    assert g.selftest_wait(1) == -7
    H, E = smooth_fields(ref, 31)
    dt = 0.2 * ref.dxmin()
    g.set_state(H, E)
    g.run(3, 0.0, dt)
    g2 = gpu_from_box(ref, "mixed")
    g2.set_state(H, E)
    g2.run(3, 0.0, dt)
    a, b = g.get_state(), g2.get_state()
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    g.close(); g2.close(); ref.close()


@pytest.mark.parametrize("form", ["fused64", "mixed"])
def test_energy_central_vs_upwind(form):
    """Central flux (C0=0) on a periodic box: the semi-discrete operator
    conserves the discrete energy, so the only loss is the RK45 integrator's,
    which must fall at least 16x when dt halves; the upwind flux (C0=1)
    dissipates more."""
    loss = {}
    for C0, dt_scale in ((0.0, 0.1), (0.0, 0.05), (1.0, 0.1)):
        ref = make_ref(5, (2, 2, 2), (0, 0, 0), (2, 2, 2), (PER,) * 3, C0=C0)
        g = gpu_from_ref(ref, form, C0=C0)
        H, E = smooth_fields(ref, 31)
        g.set_state(H, E)
        e0 = g.energy()
        dt = dt_scale * ref.dxmin()
        g.run(int(round(5.0 / dt_scale)), 0.0, dt)  # the same end time
        loss[(C0, dt_scale)] = (e0 - g.energy()) / e0
        g.close(); ref.close()
    c1, c2, up = loss[(0.0, 0.1)], loss[(0.0, 0.05)], loss[(1.0, 0.1)]
    assert 0 <= c1 < 1e-4 and abs(c2) <= c1 / 16 + 1e-13, loss
    assert up > 10 * c1, loss
