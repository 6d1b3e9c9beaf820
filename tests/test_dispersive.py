"""Dispersive media: Drude and Lorentz polarisation currents
(cem_maxwell_drude / cem_maxwell_lorentz, src/cem_maxwell.F:3095-3212, called
from usersrc as tests/drude/drude.usr:167 and tests/lorentz/lorentz.usr:174 do).

CPU: the oracle converges to the analytic plane-wave modes of a uniform Drude
or Lorentz medium (cases.DispersiveWave), the known answer that pins it.
GPU: the plain form matches the oracle bit for bit (fields and currents), the
fused FP64 form at 1e-12 per step, the mixed form at its per-step tolerance;
all three forms reach the analytic mode; currents round-trip through the
C ABI and through checkpoints; bad lists and unsupported forms are refused.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import gpu_from_box, gpu_from_ref, make_ref, rel_err, smooth_fields
from nekcem_gb300 import MaxwellGPU, cases
from nekcem_gb300 import _lib as L
from oracle import refcpu as R

DRUDE, LORENTZ = MaxwellGPU.DRUDE, MaxwellGPU.LORENTZ
TWO_PI = 2 * np.pi

WAVES = {
    "drude": ("drude", (0.0, 4.0, 0.0)),
    "drude_lossy": ("drude", (0.5, 4.0, 0.0)),
    "lorentz": ("lorentz", (0.0, 9.0, 3.0)),
    "lorentz_lossy": ("lorentz", (0.3, 9.0, 3.0)),
}


def wave_run(N, wave, T=3.0, gpu_form=None):
    """Uniform dispersive medium on the periodic box [0, 2pi]^3 (4x2x2 el):
    the analytic mode as initial data, run to T; returns the max field and
    current errors against the mode at T."""
    model, pars = WAVES[wave]
    w = cases.DispersiveWave(model, *pars)
    ref = R.RefBox(N, (4, 2, 2), (0, 0, 0), (TWO_PI,) * 3, (1, 1, 1))
    x, y, z = (a.copy() for a in ref.coords())
    n = ref.npts
    idx = np.arange(n)
    H0, E0 = w.exact(x, y, z, 0.0)
    J0 = w.currents(x, y, z, 0.0)
    dt = 0.5 * cases.CFL * cases.min_gll_spacing(x, y, z, ref.n, ref.nelt)
    nsteps = int(np.ceil(T / dt))
    dt = T / nsteps
    if gpu_form is None:
        if model == "drude":
            ref.set_drude(np.full(n, pars[0]), np.full(n, pars[1]), idx)
            ref.drude_jn[:] = J0
        else:
            ref.set_lorentz(np.full(n, pars[0]), np.full(n, pars[1]), np.full(n, pars[2]), idx)
            ref.lorentz_jn[:] = J0
        ref.set_state(H0, E0)
        ref.run(nsteps, 0.0, dt)
        H, E = ref.hn, ref.en
        J = ref.drude_jn if model == "drude" else ref.lorentz_jn
    else:
        g = gpu_from_box(ref, gpu_form)
        kind = DRUDE if model == "drude" else LORENTZ
        params = np.stack([np.full(n, p) for p in pars[: 2 if model == "drude" else 3]])
        g.set_dispersive(kind, params, idx)
        g.set_current(kind, J0)
        g.set_state(H0, E0)
        g.run(nsteps, 0.0, dt)
        H, E = g.get_state()
        J = g.get_current(kind)
        g.close()
    H1, E1 = w.exact(x, y, z, T)
    J1 = w.currents(x, y, z, T)
    err = max(np.abs(H - H1).max(), np.abs(E - E1).max())
    jerr = np.abs(J - J1).max() / max(np.abs(J1).max(), 1e-300)
    ref.close()
    return err, jerr


@pytest.mark.parametrize("wave", list(WAVES))
def test_analytic_mode_is_a_root(wave):
    model, pars = WAVES[wave]
    w = cases.DispersiveWave(model, *pars)
    assert w.residual() < 1e-12
    assert w.omega.real > 0 and w.omega.imag <= 1e-12


@pytest.mark.parametrize("wave", list(WAVES))
def test_oracle_converges_to_the_dispersive_mode(wave):
    """N=5 -> N=7 on 4x2x2 elements: the error drops at least 10x and ends
    below 4e-5 (fields, amplitude 1) and 2e-4 (currents, relative)."""
    e5, j5 = wave_run(5, wave)
    e7, j7 = wave_run(7, wave)
    assert e7 < 0.1 * e5, (e5, e7)
    assert e7 < 4e-5 and j7 < 2e-4, (e7, j7)


# ---- GPU --------------------------------------------------------------------------
MESHES = {
    "pec": dict(N=4, nel=(3, 2, 2), lo=(0, 0, 0), hi=(1.5, 1, 1), bc=(0, 0, 0)),
    "mixed_bc": dict(N=5, nel=(2, 3, 2), lo=(0, 0, 0), hi=(1, 1, 1), bc=(1, 0, 1)),
    "periodic_n7": dict(N=7, nel=(2, 2, 2), lo=(0, 0, 0), hi=(1, 1, 1), bc=(1, 1, 1)),
}
SRC = dict(xc=(0.3, 0.4, 0.5), sigma=0.2, amp=1.0, f0=2.0, t0=0.1)


def disp_problem(name, materials, seed):
    """A Drude slab (x < 0.4) and a Lorentz ball, random parameters per node,
    random initial currents, smooth fields, the Ricker source."""
    b = MESHES[name]
    eps = (lambda x, y, z: 1.0 + 0.5 * np.sin(2 * x) ** 2) if materials else None
    mu = (lambda x, y, z: 1.0 + 0.2 * np.cos(3 * z) ** 2) if materials else None
    ref = make_ref(b["N"], b["nel"], b["lo"], b["hi"], b["bc"], eps=eps, mu=mu)
    x, y, z = ref.coords()
    n = ref.npts
    rng = np.random.default_rng(seed)
    dr = np.nonzero(x < 0.4)[0]
    lz = np.nonzero(((x - 0.8) ** 2 + (y - 0.5) ** 2 + (z - 0.5) ** 2 < 0.1) & (x >= 0.4))[0]
    pd = np.stack([rng.uniform(0, 2, n), rng.uniform(1, 20, n)])
    pl = np.stack([rng.uniform(0, 2, n), rng.uniform(1, 30, n), rng.uniform(1, 10, n)])
    Jd = rng.standard_normal((3, n))
    Jl = rng.standard_normal((6, n))
    Jd[:, np.setdiff1d(np.arange(n), dr)] = 0
    Jl[:, np.setdiff1d(np.arange(n), lz)] = 0
    return ref, dict(dr=dr, lz=lz, pd=pd, pl=pl, Jd=Jd, Jl=Jl)


def start(ref, g, p, seed):
    ref.set_drude(p["pd"][0], p["pd"][1], p["dr"])
    ref.set_lorentz(p["pl"][0], p["pl"][1], p["pl"][2], p["lz"])
    ref.drude_jn[:] = p["Jd"]
    ref.lorentz_jn[:] = p["Jl"]
    g.set_dispersive(DRUDE, p["pd"], p["dr"])
    g.set_dispersive(LORENTZ, p["pl"], p["lz"])
    g.set_current(DRUDE, p["Jd"])
    g.set_current(LORENTZ, p["Jl"])
    H, E = smooth_fields(ref, seed)
    ref.set_state(H, E)
    g.set_state(H, E)
    ref.set_source(**SRC)
    g.set_source(**SRC)
    return 0.3 * ref.dxmin()


def cur_err(g, ref):
    a = np.concatenate([g.get_current(DRUDE), g.get_current(LORENTZ)])
    b = np.concatenate([ref.drude_jn, ref.lorentz_jn])
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(MESHES))
@pytest.mark.parametrize("materials", [False, True])
def test_plain_dispersive_bit_exact(name, materials):
    ref, p = disp_problem(name, materials, 7)
    g = gpu_from_ref(ref, "plain")
    dt = start(ref, g, p, 8)
    ref.run(4, 0.0, dt)
    g.run(4, 0.0, dt)
    H, E = g.get_state()
    np.testing.assert_array_equal(H, ref.hn)
    np.testing.assert_array_equal(E, ref.en)
    np.testing.assert_array_equal(g.get_current(DRUDE), ref.drude_jn)
    np.testing.assert_array_equal(g.get_current(LORENTZ), ref.lorentz_jn)
    assert np.abs(ref.lorentz_jn[3:]).max() > 0
    g.close(); ref.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(MESHES))
@pytest.mark.parametrize("materials", [False, True])
def test_fused64_dispersive(name, materials):
    ref, p = disp_problem(name, materials, 9)
    g = gpu_from_box(ref, "fused64")
    dt = start(ref, g, p, 10)
    for step in range(4):
        ref.op_rk(step * dt, dt)
        g.run(1, step * dt, dt)
        H, E = g.get_state()
        assert rel_err(H, E, ref.hn, ref.en) <= 1e-12 * (step + 1), step
    assert cur_err(g, ref) <= 1e-11
    g.close(); ref.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(MESHES))
@pytest.mark.parametrize("materials", [False, True])
def test_mixed_dispersive_per_step(name, materials):
    ref, p = disp_problem(name, materials, 11)
    g = gpu_from_box(ref, "mixed")
    dt = start(ref, g, p, 12)
    ref.op_rk(0.0, dt)
    g.run(1, 0.0, dt)
    H, E = g.get_state()
    # the mixed form's per-step bar (pair-precision contractions and flux)
    assert rel_err(H, E, ref.hn, ref.en) <= 1e-9
    assert cur_err(g, ref) <= 1e-9
    g.close(); ref.close()


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["plain", "fused64", "mixed"])
@pytest.mark.parametrize("wave", ["drude_lossy", "lorentz"])
def test_gpu_reaches_the_dispersive_mode(form, wave):
    err, jerr = wave_run(7, wave, gpu_form=form)
    ref_err, ref_jerr = wave_run(7, wave)
    assert err <= 1.5 * ref_err + 1e-9 and jerr <= 1.5 * ref_jerr + 1e-9, (err, ref_err)


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["plain", "fused64", "mixed"])
def test_dispersive_checkpoint_resume(form, tmp_path):
    ref, p = disp_problem("mixed_bc", True, 13)
    g = gpu_from_box(ref, form) if form != "plain" else gpu_from_ref(ref, form)
    dt = start(ref, g, p, 14)
    g.run(2, 0.0, dt)
    g.checkpoint_save(tmp_path / "ck.bin", 2 * dt, 2)
    g.run(3, 2 * dt, dt)
    H1, E1 = g.get_state()
    J1 = g.get_current(LORENTZ)
    g.set_dispersive(DRUDE, p["pd"], p["dr"])  # resets every current
    assert np.abs(g.get_current(LORENTZ)).max() == 0
    t, n = g.checkpoint_load(tmp_path / "ck.bin")
    assert (t, n) == (2 * dt, 2)
    g.run(3, t, dt)
    H2, E2 = g.get_state()
    np.testing.assert_array_equal(H2, H1)
    np.testing.assert_array_equal(E2, E1)
    np.testing.assert_array_equal(g.get_current(LORENTZ), J1)
    g.close(); ref.close()


@pytest.mark.gpu
def test_dispersive_lists_are_checked():
    g = MaxwellGPU.from_box(3, (2, 2, 2), (0, 0, 0), (1, 1, 1), (0, 0, 0), form="fused64")
    n = g.npts
    pd = np.ones((2, n))
    pl = np.ones((3, n))
    for bad in ([n], [-1], [3, 3]):
        with pytest.raises(L.NekgpuError) as e:
            g.set_dispersive(DRUDE, pd, np.array(bad))
        assert e.value.status == -1
    g.set_dispersive(DRUDE, pd, np.arange(10))
    with pytest.raises(L.NekgpuError):  # node 5 is already a Drude node
        g.set_dispersive(LORENTZ, pl, np.array([5, 20]))
    g.set_dispersive(LORENTZ, pl, np.array([10, 20]))
    g.set_dispersive(DRUDE, pd, np.array([], dtype=int))  # removes the Drude list
    g.set_dispersive(LORENTZ, pl, np.array([5]))
    J = np.zeros((6, n)); J[:, 5] = 1.0; J[:, 6] = 2.0
    g.set_current(LORENTZ, J)
    got = g.get_current(LORENTZ)
    assert got[:, 5].tolist() == [1.0] * 6 and np.abs(got[:, 6]).max() == 0
    g.set_state(np.zeros((3, n)), np.zeros((3, n)))
    with pytest.raises(L.NekgpuError) as e:  # no adjoint through the currents
        g.adjoint_gradient(1, 0.0, 0.01, np.ones(n))
    assert e.value.status == -8
    g.close()
    g = MaxwellGPU.from_box(3, (2, 2, 2), (0, 0, 0), (1, 1, 1), (0, 0, 0), form="mixed_naive")
    with pytest.raises(L.NekgpuError) as e:
        g.set_dispersive(DRUDE, pd, np.arange(3))
    assert e.value.status == -8
    g.close()
