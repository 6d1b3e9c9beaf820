"""PML (src/cem_maxwell_pml.F) on the GPU against the oracle: the plain form
bit for bit (state and auxiliary fields), the fused FP64 form at 1e-12 per
step, the mixed form at its per-step tolerance; the reference's
tests/3dboxpml known answer on every form; absorption compared with PEC
walls; forms without PML support refuse it."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import gpu_from_box, gpu_from_ref, make_ref, rel_err, smooth_fields
from nekcem_gb300 import MaxwellGPU, cases
from nekcem_gb300 import _lib as L

pytestmark = pytest.mark.gpu

PML_MESHES = {
    "all6": dict(N=4, nel=(6, 6, 6), lo=(-1, -1, -1), hi=(1, 1, 1), bc=(2, 2, 2), pml=(1, 3.0, 1e-8)),
    "mixed_bc": dict(N=3, nel=(5, 4, 6), lo=(0, 0, 0), hi=(1.25, 1, 1.5), bc=(2, 1, 2),
                     pml=(2, 2.0, 1e-6)),
    "pec_y_n5": dict(N=5, nel=(4, 3, 2), lo=(0, 0, 0), hi=(1, 1, 1), bc=(0, 2, 1), pml=(1, 4.0, 1e-4)),
}
SRC = dict(xc=(0.3, 0.2, 0.1), sigma=0.2, amp=1.0, f0=2.0, t0=0.0)


def ref_for(name, materials):
    b = PML_MESHES[name]
    eps = (lambda x, y, z: 1.0 + 0.5 * np.sin(2 * x) ** 2) if materials else None
    mu = (lambda x, y, z: 1.0 + 0.2 * np.cos(3 * z) ** 2) if materials else None
    return make_ref(b["N"], b["nel"], b["lo"], b["hi"], b["bc"], eps=eps, mu=mu, pml=b["pml"])


def start(ref, g, seed):
    """Smooth fields, zero auxiliary fields, the sine dipole source on both."""
    H, E = smooth_fields(ref, seed)
    ref.set_state(H, E)
    g.set_state(H, E)
    ref.set_source_kind(1)
    ref.set_source(**SRC)
    g.set_source_kind(1)
    g.set_source(**SRC)
    return 0.3 * ref.dxmin()


def aux_err(g, ref):
    a = np.concatenate([g.array("pmlbn"), g.array("pmldn")])
    b = np.concatenate([ref.d("pmlbn"), ref.d("pmldn")])
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("name", list(PML_MESHES))
@pytest.mark.parametrize("materials", [False, True])
def test_plain_pml_bit_exact(name, materials):
    ref = ref_for(name, materials)
    g = gpu_from_ref(ref, "plain")
    dt = start(ref, g, 41)
    ref.run(4, 0.0, dt)
    g.run(4, 0.0, dt)
    H, E = g.get_state()
    np.testing.assert_array_equal(H, ref.hn)
    np.testing.assert_array_equal(E, ref.en)
    np.testing.assert_array_equal(g.array("pmlbn"), ref.d("pmlbn"))
    np.testing.assert_array_equal(g.array("pmldn"), ref.d("pmldn"))
    assert np.abs(ref.d("pmldn")).max() > 0
    g.close(); ref.close()


@pytest.mark.parametrize("name", list(PML_MESHES))
@pytest.mark.parametrize("materials", [False, True])
@pytest.mark.parametrize("path", ["arrays", "box"])
def test_fused64_pml(name, materials, path):
    ref = ref_for(name, materials)
    g = gpu_from_ref(ref, "fused64") if path == "arrays" else gpu_from_box(ref, "fused64")
    dt = start(ref, g, 42)
    for step in range(4):
        ref.op_rk(step * dt, dt)
        g.run(1, step * dt, dt)
        H, E = g.get_state()
        assert rel_err(H, E, ref.hn, ref.en) <= 1e-12 * (step + 1), step
    assert aux_err(g, ref) <= 1e-11
    g.close(); ref.close()


@pytest.mark.parametrize("name", list(PML_MESHES))
@pytest.mark.parametrize("materials", [False, True])
def test_mixed_pml_per_step(name, materials):
    ref = ref_for(name, materials)
    g = gpu_from_box(ref, "mixed")
    dt = start(ref, g, 43)
    ref.op_rk(0.0, dt)
    g.run(1, 0.0, dt)
    H, E = g.get_state()
    # the mixed form's per-step bar (pair-precision contractions and flux)
    assert rel_err(H, E, ref.hn, ref.en) <= 1e-9
    assert aux_err(g, ref) <= 1e-9
    g.close(); ref.close()


@pytest.mark.parametrize("form", ["plain", "fused64", "mixed"])
def test_3dboxpml_known_answer(form):
    """tests/3dboxpml (6^3 el, N=8, [-1,1]^3, 'PML' on all faces; params 77-79:
    thickness 1, order 3, error 1e-8; the Gaussian dipole sin(2t), width 0.1,
    at the origin; zero initial fields; dt = 0.1 dxmin; 2000 steps): every
    component's L2 and Linf stay below 1 at steps 1..10 and every 10 steps."""
    g = MaxwellGPU.from_box(8, (6, 6, 6), (-1, -1, -1), (1, 1, 1), (2, 2, 2), form=form,
                            pml=(1, 3.0, 1e-8))
    x, y, z = g.coords()
    dt = 0.1 * cases.get_dxmin(x, y, z, 9, 216)
    g.set_source_kind(1)
    g.set_source((0.0, 0.0, 0.0), 0.1, 1.0, 2.0, 0.0)
    zero = np.zeros((3, g.npts))
    g.set_state(zero, zero)
    t, step = 0.0, 0
    while step < 2000:
        n = 1 if step < 10 else 10
        t = g.run(n, t, dt)
        step += n
        l2, li = g.cem_error(zero, zero)
        assert np.all(l2 <= 1.0) and np.all(li <= 1.0), (step, l2, li)
    assert np.abs(g.array("pmldn")).max() > 0
    g.close()


def test_pml_absorbs_what_pec_reflects():
    """A pulse leaves the box through the PML but stays inside a PEC box: after the wave has crossed the boundary twice the energy left
    with PML is far below the PEC one (mixed form; dt = 0.1 dxmin as in the
    reference's PML test: the graded sigma makes the layers stiff)."""
    energies = {}
    for bc, pml in (((2, 2, 2), (2, 3.0, 1e-8)), ((0, 0, 0), None)):
        g = MaxwellGPU.from_box(5, (8, 8, 8), (-1, -1, -1), (1, 1, 1), bc, form="mixed", pml=pml)
        x, y, z = g.coords()
        # a divergence-free pulse (E = curl of psi e_z, psi Gaussian): all of
        # it propagates (a Gaussian E_z alone has a static gradient part)
        psi = np.exp(-(x * x + y * y + z * z) / (2 * 0.15 ** 2)) / 0.15 ** 2
        g.set_state(np.zeros((3, g.npts)), np.stack([y * psi, -x * psi, 0 * psi]))
        dt = 0.1 * cases.get_dxmin(x, y, z, 6, 512)
        e0 = g.energy()
        g.run(int(3.0 / dt), 0.0, dt)
        energies[bc[0]] = g.energy() / e0
        g.close()
    assert energies[2] < 0.05 * energies[0], energies


def test_pml_unsupported_forms():
    with pytest.raises(L.NekgpuError) as e:
        MaxwellGPU.from_box(3, (4, 4, 4), (0, 0, 0), (1, 1, 1), (2, 0, 0), form="mixed_naive",
                            pml=(1, 3.0, 1e-8))
    assert e.value.status == -8
    g = MaxwellGPU.from_box(3, (4, 4, 4), (0, 0, 0), (1, 1, 1), (2, 0, 0), form="fused64",
                            pml=(1, 3.0, 1e-8))
    g.set_state(np.zeros((3, g.npts)), np.zeros((3, g.npts)))
    with pytest.raises(L.NekgpuError) as e:
        g.adjoint_gradient(2, 0.0, 0.01, np.ones(g.npts))
    assert e.value.status == -8
    g.close()
