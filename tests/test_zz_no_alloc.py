"""nekgpu_norms_noalloc: the cem_error norms for callers that cannot allocate
device memory while time stepping (their device memory is all handed to a
pool at start-up, or an allocation failure or cudaFree's synchronisation is
not acceptable between steps).  It takes the exact fields already on the
device and keeps its scratch in a fixed device array of the library, so it
must agree with nekgpu_norms -- which copies the exact fields to a fresh
device buffer -- on two calls in a row (the second reuses the array the first
left behind), leave the context's device memory and the device's free
memory unchanged across a call, and refuse meshes larger than that array
allows.

This file is collected last on purpose (pytest runs files in name order).
"""
import ctypes as C

import numpy as np
import pytest

from nekcem_gb300 import MaxwellGPU, cases
from nekcem_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def _device_copy(a: np.ndarray):
    torch = pytest.importorskip("torch")
    t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to("cuda")
    torch.cuda.synchronize()
    return t


def _noalloc(g: MaxwellGPU, exact_dev_ptr: int):
    l2 = np.zeros(6)
    li = np.zeros(6)
    st = L.load().nekgpu_norms_noalloc(g._h, C.c_void_p(exact_dev_ptr), l2.ctypes.data_as(L.dp),
                                       li.ctypes.data_as(L.dp))
    return st, l2, li


@pytest.mark.parametrize("form", ["mixed", "plain"])
def test_norms_noalloc_matches_norms_twice(form):
    c = cases.make("cavity")
    g = MaxwellGPU.from_box(c.N, c.nel, c.lo, c.hi, c.bc, form=form)
    x, y, z = g.coords()
    dt = c.timestep(x, y, z)
    g.set_state(*c.exact(x, y, z, 0.0))
    t = g.run(40, 0.0, dt)
    Hx, Ex = c.exact(x, y, z, t)
    l2_ref, li_ref = g.cem_error(Hx, Ex)
    exact_dev = _device_copy(np.concatenate([Hx.ravel(), Ex.ravel()]))
    import torch
    for call in range(2):
        # the first call also loads the kernels; the second must allocate nothing
        before = (g.device_bytes(), torch.cuda.mem_get_info()[0])
        st, l2, li = _noalloc(g, exact_dev.data_ptr())
        after = (g.device_bytes(), torch.cuda.mem_get_info()[0])
        assert st == 0, L.load().nekgpu_error_string(st).decode()
        np.testing.assert_allclose(l2, l2_ref, rtol=1e-12, atol=0, err_msg=f"call {call}")
        np.testing.assert_allclose(li, li_ref, rtol=1e-12, atol=0, err_msg=f"call {call}")
        if call == 1:
            assert after == before, (before, after)
    g.close()


def test_norms_noalloc_rejects_meshes_beyond_its_scratch():
    # 26^3 elements of N=7: 8,998,912 nodes > 8,388,608
    g = MaxwellGPU.from_box(7, (26, 26, 26), (0, 0, 0), (1, 1, 1), (0, 0, 0), form="mixed")
    exact_dev = _device_copy(np.zeros(8))
    st, _, _ = _noalloc(g, exact_dev.data_ptr())
    assert st == -9  # NEKGPU_ERR_TOO_LARGE
    assert "8,388,608" in L.load().nekgpu_error_string(st).decode()
    g.close()
