"""The C ABI driven by a compiled program laid out like NekCEM's own driver
(tests/c_driver.c: COMMON-style static arrays with lpts1 > npts, the
time_advancing_pde loop of src/cem_drive.F:618-651 with `time = time + dt`
done by the caller, userchk reading fields and norms back).

CPU: the driver compiles with gcc against include/nekcem_gpu.h and links the
library.  GPU: the reference's tests/3dboxpec known answer through the
driver (final time exactly the caller's sum of dt, L2 and Linf at the
reference's tolerances), and, with the time-dependent volume source on, the
fields after 40 steps match the oracle's run at the right stage times (plain
form, device-resident and host-array paths: within 1e-10 relative, the
driver's geometry coming from the library's box builder, which agrees with
the oracle's setup to ~1e-13) and equal bit for bit the same steps driven
through the Python binding; a library that also advanced the caller's time
would drive the source at twice its rate and fail both.
"""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from nekcem_gb300 import build as libbuild
from nekcem_gb300 import cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_driver.c")
SOURCE = dict(xc=(0.2, -0.1, 0.3), sigma=0.3, amp=1.0, f0=2.0, t0=0.05)
FORMS = {"plain": 0, "fused64": 1, "mixed": 2}


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    lib = libbuild.build()
    exe = str(tmp_path_factory.mktemp("c_driver") / "c_driver")
    libdir = os.path.dirname(lib)
    cmd = ["gcc", "-std=c99", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           SRC, "-o", exe, "-L", libdir, "-lnekcem_gb300", f"-Wl,-rpath,{libdir}", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def run_driver(exe, tmp_path, form, path, nsteps, iocomm, source):
    out = str(tmp_path / f"fields_{form}_{path}_{source}.bin")
    r = subprocess.run([exe, str(FORMS[form]), path, str(nsteps), str(iocomm), str(int(source)),
                        out], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    chk, final = [], None
    for ln in r.stdout.splitlines():
        p = ln.split()
        if p[0] == "chk":
            chk.append((int(p[1]), float(p[2]), np.array([float(v) for v in p[3:9]]),
                        np.array([float(v) for v in p[9:15]])))
        elif p[0] == "final_time":
            final = float(p[1])
    u = np.fromfile(out, dtype=np.float64).reshape(6, -1)
    return chk, final, u[:3], u[3:]


def caller_time(nsteps, dt=0.005):
    t = 0.0
    for _ in range(nsteps):
        t = t + dt
    return t


def test_driver_compiles_and_reports_status_without_gpu(driver, tmp_path):
    """Without a usable GPU the first device call fails with a status the
    driver prints, and the program exits 2 (no crash)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: the GPU tests below run the driver")
    r = subprocess.run([driver, "1", "step", "1", "1", "0", str(tmp_path / "x.bin")],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 2
    assert "nekgpu_init" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["fused64", "mixed"])
def test_driver_3dboxpec_known_answer(driver, tmp_path, form):
    c = cases.make("3dboxpec")
    chk, final, H, E = run_driver(driver, tmp_path, form, "step", c.nsteps, 250, False)
    assert final == caller_time(c.nsteps)
    assert [k[0] for k in chk] == [250, 500, 750, 1000]
    for istep, t, l2, linf in chk:
        assert t == caller_time(istep)
        assert np.all(l2 <= c.l2tol), (istep, l2)
        assert np.all(linf <= c.linftol), (istep, linf)


@pytest.mark.gpu
@pytest.mark.parametrize("path", ["step", "host"])
def test_driver_source_run_matches_oracle(driver, tmp_path, path):
    from helpers import make_ref
    nsteps, dt = 40, 0.005
    chk, final, H, E = run_driver(driver, tmp_path, "plain", path, nsteps, 10, True)
    assert final == caller_time(nsteps)
    ref = make_ref(8, (3, 3, 3), (-1, -1, -1), (1, 1, 1), (0, 0, 0))
    ref.set_source(**SOURCE)
    x, y, z = ref.coords()
    ref.set_state(*cases.sol_3dboxpec(x, y, z, 0.0))
    t = ref.run(nsteps, 0.0, dt)
    assert t == final
    a = np.concatenate([H, E]); b = np.concatenate([ref.hn, ref.en])
    ref.close()
    assert np.abs(a - b).max() <= 1e-10 * np.abs(b).max()
    from nekcem_gb300 import MaxwellGPU
    g = MaxwellGPU.from_box(8, (3, 3, 3), (-1, -1, -1), (1, 1, 1), (0, 0, 0), form="plain")
    g.set_source(**SOURCE)
    g.set_state(*cases.sol_3dboxpec(*g.coords(), 0.0))
    assert g.run(nsteps, 0.0, dt) == final
    gH, gE = g.get_state()
    g.close()
    np.testing.assert_array_equal(H, gH)
    np.testing.assert_array_equal(E, gE)
