"""Curvilinear (non-affine) elements: boxes with a smooth interior
deformation (per-node metrics, curved faces with per-node normals and areas).
The plain form runs them from the reference's arrays bit for bit against the
oracle; the fused FP64 form runs them through its curvilinear kernel at
1e-12 per step; the mixed form through its curvilinear kernel (exact-hi FP32
derivatives, float-pair metrics and flux, FP64 update) at 1e-9 per step,
each step from the oracle's state; the cavity mode (whose walls do not
move) keeps its accuracy on all three."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import gpu_from_ref, make_ref, rel_err, smooth_fields
from nekcem_gb300 import cases
from nekcem_gb300 import _lib as L

pytestmark = pytest.mark.gpu

CURVED = [
    dict(N=4, nel=(3, 3, 3), bc=(0, 0, 0), deform=0.05),
    dict(N=5, nel=(2, 3, 2), bc=(1, 0, 1), deform=0.08),
    dict(N=7, nel=(2, 2, 2), bc=(1, 1, 1), deform=0.04),
]


@pytest.mark.parametrize("m", CURVED, ids=["pec_n4", "mixed_bc_n5", "periodic_n7"])
@pytest.mark.parametrize("materials", [False, True])
def test_plain_curved_bit_exact(m, materials):
    eps = (lambda x, y, z: 1.0 + 0.5 * np.sin(2 * x) ** 2) if materials else None
    ref = make_ref(m["N"], m["nel"], (0, 0, 0), (1, 1, 1), m["bc"], eps=eps, deform=m["deform"])
    assert np.abs(ref.d("rym1")).max() > 1e-3  # the metrics are not diagonal
    g = gpu_from_ref(ref, "plain")
    H, E = smooth_fields(ref, 5)
    ref.set_state(H, E); g.set_state(H, E)
    dt = 0.2 * ref.dxmin()
    ref.run(5, 0.0, dt); g.run(5, 0.0, dt)
    gH, gE = g.get_state()
    np.testing.assert_array_equal(gH, ref.hn)
    np.testing.assert_array_equal(gE, ref.en)
    g.close(); ref.close()


@pytest.mark.parametrize("m", CURVED, ids=["pec_n4", "mixed_bc_n5", "periodic_n7"])
@pytest.mark.parametrize("materials", [False, True])
def test_fused64_curved_per_step(m, materials):
    """The curvilinear kernel of the fused FP64 form against the oracle, with
    the Ricker source on: 1e-12 relative per step over 4 steps."""
    eps = (lambda x, y, z: 1.0 + 0.5 * np.sin(2 * x) ** 2) if materials else None
    mu = (lambda x, y, z: 1.0 + 0.2 * np.cos(3 * z) ** 2) if materials else None
    ref = make_ref(m["N"], m["nel"], (0, 0, 0), (1, 1, 1), m["bc"], eps=eps, mu=mu,
                   deform=m["deform"])
    g = gpu_from_ref(ref, "fused64")
    H, E = smooth_fields(ref, 6)
    ref.set_state(H, E); g.set_state(H, E)
    src = dict(xc=(0.4, 0.5, 0.6), sigma=0.2, amp=1.0, f0=2.0, t0=0.1)
    ref.set_source(**src); g.set_source(**src)
    dt = 0.2 * ref.dxmin()
    for step in range(4):
        ref.op_rk(step * dt, dt)
        g.run(1, step * dt, dt)
        gH, gE = g.get_state()
        assert rel_err(gH, gE, ref.hn, ref.en) <= 1e-12 * (step + 1), step
    g.close(); ref.close()


@pytest.mark.parametrize("m", CURVED, ids=["pec_n4", "mixed_bc_n5", "periodic_n7"])
@pytest.mark.parametrize("materials", [False, True])
def test_mixed_curved_per_step(m, materials):
    """The curvilinear kernel of the mixed form against the oracle, with the
    Ricker source on: 1e-9 relative per step, four steps, each from the
    oracle's state (the affine mixed kernel's bar)."""
    eps = (lambda x, y, z: 1.0 + 0.5 * np.sin(2 * x) ** 2) if materials else None
    mu = (lambda x, y, z: 1.0 + 0.2 * np.cos(3 * z) ** 2) if materials else None
    ref = make_ref(m["N"], m["nel"], (0, 0, 0), (1, 1, 1), m["bc"], eps=eps, mu=mu,
                   deform=m["deform"])
    g = gpu_from_ref(ref, "mixed")
    H, E = smooth_fields(ref, 6)
    src = dict(xc=(0.4, 0.5, 0.6), sigma=0.2, amp=1.0, f0=2.0, t0=0.1)
    ref.set_source(**src); g.set_source(**src)
    dt = 0.2 * ref.dxmin()
    t = 0.0
    for step in range(4):
        ref.set_state(H, E); g.set_state(H, E)
        ref.op_rk(t, dt)
        g.run(1, t, dt)
        gH, gE = g.get_state()
        err = rel_err(gH, gE, ref.hn, ref.en)
        assert err <= 1e-9, f"step {step}: relative error {err:.3e} > 1e-9"
        H, E = ref.hn.copy(), ref.en.copy()
        t += dt
    g.close(); ref.close()


def test_mixed_curved_multi_step_tracks_fp64():
    """100 steps on the deformed N=7 box from a smooth state: the mixed
    run stays within 1e-8 (relative, max norm) of the fused FP64 run."""
    ref = make_ref(7, (2, 2, 2), (0, 0, 0), (1, 1, 1), (1, 1, 1), deform=0.04)
    a, b = gpu_from_ref(ref, "mixed"), gpu_from_ref(ref, "fused64")
    H, E = smooth_fields(ref, 9)
    dt = 0.2 * ref.dxmin()
    for g in (a, b):
        g.set_state(H, E)
        g.run(100, 0.0, dt)
    aH, aE = a.get_state()
    bH, bE = b.get_state()
    assert rel_err(aH, aE, bH, bE) <= 1e-8
    a.close(); b.close(); ref.close()


@pytest.mark.parametrize("form", ["plain", "fused64", "mixed"])
def test_curved_cavity_keeps_its_accuracy(form):
    """TM110 cavity on a deformed 4^3, N=7 mesh (the walls stay put, so the
    analytic mode is unchanged): after 300 steps the L2 error stays small.
    It is larger than on the affine mesh (9e-10 there): the curved geometry
    is only represented to the GLL interpolant's accuracy and the metric
    products alias (the reference's dealiased curl, maxwell_wght_dcurl,
    addresses the latter)."""
    res = {}
    for deform in (0.0, 0.04):
        ref = make_ref(7, (4, 4, 4), (0, 0, 0), (1, 1, 1), (0, 0, 0), deform=deform)
        g = gpu_from_ref(ref, form)
        x, y, z = (a.copy() for a in ref.coords())
        c = cases.make("cavity")
        dt = 0.5 * cases.min_gll_spacing(x, y, z, 8, 64) * 0.5
        g.set_state(*c.exact(x, y, z, 0.0))
        t = g.run(300, 0.0, dt)
        l2, _ = g.cem_error(*c.exact(x, y, z, t))
        res[deform] = float(np.sqrt(np.sum(l2 ** 2)))
        g.close(); ref.close()
    assert res[0.0] < 1e-8, res
    assert res[0.04] < 1e-6, res


def test_curved_refusals():
    """The curvilinear kernels have no dispersive media; the adjoint is the
    affine fused FP64 form's; the dealiased curl is the FP64 forms'."""
    ref = make_ref(4, (2, 2, 2), (0, 0, 0), (1, 1, 1), (0, 0, 0), deform=0.05)
    for form in ("fused64", "mixed"):
        g = gpu_from_ref(ref, form)
        g.set_state(np.zeros((3, g.npts)), np.zeros((3, g.npts)))
        calls = [lambda: g.set_dispersive(g.DRUDE, np.ones((2, g.npts)), np.arange(3)),
                 lambda: g.adjoint_gradient(1, 0.0, 0.01, np.ones(g.npts))]
        if form == "mixed":
            calls.append(lambda: g.set_dealias(6))
        for call in calls:
            with pytest.raises(L.NekgpuError) as e:
                call()
            assert e.value.status == -8
        g.close()
    ref.close()
