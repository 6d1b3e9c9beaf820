"""GPU-state output: the reference's VTK file byte for byte (plain form,
whose state equals the oracle's), and checkpoints that resume a run bit for
bit on every form, PML auxiliary fields included."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import gpu_from_ref, make_ref, smooth_fields
from nekcem_gb300 import MaxwellGPU, cases
from nekcem_gb300 import _lib as L
from vtk_ref import vtk_bytes

pytestmark = pytest.mark.gpu


def test_vtk_matches_the_reference_writer(tmp_path):
    ref = make_ref(4, (2, 3, 2), (0, 0, 0), (1, 1.5, 1), (0, 1, 0))
    g = gpu_from_ref(ref, "plain")
    H, E = smooth_fields(ref, 7)
    ref.set_state(H, E); g.set_state(H, E)
    dt = 0.2 * ref.dxmin()
    ref.run(3, 0.0, dt); g.run(3, 0.0, dt)
    x, y, z = ref.coords()
    sH, sE = smooth_fields(ref, 8)
    g.write_vtk(tmp_path / "a.vtk", sol=(sH, sE))
    got = (tmp_path / "a.vtk").read_bytes()
    want = vtk_bytes(x, y, z, ref.n, ref.nelt, ref.hn, ref.en, sH, sE)
    assert got == want
    g.write_vtk(tmp_path / "b.vtk")
    assert (tmp_path / "b.vtk").read_bytes() == vtk_bytes(x, y, z, ref.n, ref.nelt, ref.hn, ref.en)
    g.close(); ref.close()


@pytest.mark.parametrize("form", ["plain", "fused64", "mixed"])
@pytest.mark.parametrize("pml", [None, (1, 3.0, 1e-8)])
def test_checkpoint_resume_is_exact(tmp_path, form, pml):
    bc = (2, 2, 2) if pml else (0, 1, 0)
    kw = dict(form=form, pml=pml)
    g = MaxwellGPU.from_box(4, (4, 4, 4), (-1, -1, -1), (1, 1, 1), bc, **kw)
    x, y, z = g.coords()
    g.set_source_kind(1)
    g.set_source((0.1, 0.0, -0.1), 0.2, 1.0, 2.0, 0.0)
    g.set_state(*cases.gaussian_pulse_ez((0.0, 0.1, 0.0), 0.2)(x, y, z))
    dt = 0.1 * cases.get_dxmin(x, y, z, 5, 64)
    t = g.run(5, 0.0, dt)
    g.checkpoint_save(tmp_path / "ck.bin", t, 5)
    t = g.run(4, t, dt)
    H1, E1 = g.get_state()
    g2 = MaxwellGPU.from_box(4, (4, 4, 4), (-1, -1, -1), (1, 1, 1), bc, **kw)
    g2.set_source_kind(1)
    g2.set_source((0.1, 0.0, -0.1), 0.2, 1.0, 2.0, 0.0)
    t2, step = g2.checkpoint_load(tmp_path / "ck.bin")
    assert step == 5
    g2.run(4, t2, dt)
    H2, E2 = g2.get_state()
    np.testing.assert_array_equal(H2, H1)
    np.testing.assert_array_equal(E2, E1)
    if pml:
        np.testing.assert_array_equal(g2.array("pmldn"), g.array("pmldn"))
    # a checkpoint of another mesh or form is refused
    g3 = MaxwellGPU.from_box(4, (4, 4, 2), (-1, -1, -1), (1, 1, 1), bc, **kw)
    with pytest.raises(L.NekgpuError) as e:
        g3.checkpoint_load(tmp_path / "ck.bin")
    assert e.value.status == -2
    g.close(); g2.close(); g3.close()
