"""Discrete adjoint dJ/deps of J = sum jw |E(T)|^2 (jw = bm1 on a probe box).

CPU: the torch tape restatement (tests/tape_maxwell.py) matches the oracle's
time steps, and its tape gradient matches central differences of the oracle.
GPU: nekgpu_adjoint_gradient matches central differences of the library's
own FP64 forward (h = 1e-6, 20 seeded directions, 1e-6 relative), the tape
gradient node by node, and does not depend on the checkpoint stride or on
where its snapshots live (device or pinned host memory).  With the forward
steps in the mixed form (reverse stages FP64) it stays within 1e-8 of the
FP64 gradient and passes the same central-difference check.
"""
from __future__ import annotations

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from helpers import make_ref  # noqa: E402
from nekcem_gb300 import MaxwellGPU, cases  # noqa: E402
from nekcem_gb300 import _lib as L  # noqa: E402
from tape_maxwell import TapeMaxwell  # noqa: E402

PEC, PER = 0, 1
SOURCE = dict(xc=(0.3, 0.3, 0.3), sigma=0.1, amp=1.0, f0=2.0, t0=0.3)


def problem_data(N, nel, bc, seed):
    """Mesh on [0,1]^3, seeded random eps (smooth field + node noise), a
    Gaussian E_z pulse plus the Gaussian/Ricker source, probe (0.5,1)^3."""
    ref = make_ref(N, nel, (0, 0, 0), (1, 1, 1), bc)
    x, y, z = (a.copy() for a in ref.coords())
    rng = np.random.default_rng(seed)
    eps = cases.eps_random(x, y, z, seed=seed, length=0.3) + 0.2 * rng.random(ref.npts)
    ref.set_materials(eps, np.ones(ref.npts))
    H0, E0 = cases.gaussian_pulse_ez((0.55, 0.5, 0.45), 0.15)(x, y, z)
    bm1 = ref.d("bm1").copy()
    inside = (x > 0.5) & (y > 0.5) & (z > 0.5)
    jw = np.where(inside, bm1, 0.0)
    dt = 0.5 * cases.CFL * cases.min_gll_spacing(x, y, z, ref.n, ref.nelt)
    return ref, eps, H0, E0, jw, dt, (x, y, z)


def oracle_J(ref, eps, H0, E0, jw, nsteps, dt):
    ref.set_materials(eps, np.ones(ref.npts))
    ref.set_source(**SOURCE)
    ref.set_state(H0, E0)
    ref.run(nsteps, 0.0, dt)
    return float(np.sum(jw * ref.en ** 2))


def tape_J(tm, eps_t, H0, E0, jw, nsteps, dt):
    H, E = tm.run(torch.tensor(H0), torch.tensor(E0), eps_t, nsteps, 0.0, dt)
    return torch.sum(torch.tensor(jw) * E * E)


def make_tape(ref, xyz):
    tm = TapeMaxwell(ref)
    tm.set_source(*xyz, **SOURCE)
    return tm


# ---- CPU: the tape restatement against the oracle ------------------------------
def test_tape_forward_matches_oracle():
    ref, eps, H0, E0, jw, dt, xyz = problem_data(3, (2, 2, 2), (PEC, PER, PEC), seed=11)
    nsteps = 6
    tm = make_tape(ref, xyz)
    H, E = tm.run(torch.tensor(H0), torch.tensor(E0), torch.tensor(eps), nsteps, 0.0, dt)
    ref.set_source(**SOURCE)
    ref.set_state(H0, E0)
    ref.run(nsteps, 0.0, dt)
    scale = max(np.abs(ref.hn).max(), np.abs(ref.en).max())
    assert np.abs(H.numpy() - ref.hn).max() <= 1e-12 * scale
    assert np.abs(E.numpy() - ref.en).max() <= 1e-12 * scale


def test_tape_gradient_matches_oracle_central_differences():
    ref, eps, H0, E0, jw, dt, xyz = problem_data(3, (2, 2, 2), (PEC, PEC, PER), seed=12)
    nsteps = 6
    tm = make_tape(ref, xyz)
    eps_t = torch.tensor(eps, requires_grad=True)
    tape_J(tm, eps_t, H0, E0, jw, nsteps, dt).backward()
    grad = eps_t.grad.numpy()
    rng = np.random.default_rng(5)
    h = 1e-6
    for _ in range(4):
        d = rng.standard_normal(ref.npts)
        fd = (oracle_J(ref, eps + h * d, H0, E0, jw, nsteps, dt)
              - oracle_J(ref, eps - h * d, H0, E0, jw, nsteps, dt)) / (2 * h)
        ad = float(grad @ d)
        assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)


# ---- GPU: the library's adjoint ------------------------------------------------------
def gpu_problem(N, nel, bc, seed, nsteps, stride=0):
    from adjoint_autograd import BoxProblem
    ref, eps, H0, E0, jw, dt, xyz = problem_data(N, nel, bc, seed)
    pb = BoxProblem(N, nel, (0, 0, 0), (1, 1, 1), bc, H0, E0, jw, nsteps, dt, source=SOURCE,
                    stride=stride)
    return pb, eps, ref, xyz


MESHES = [
    pytest.param(3, (2, 2, 2), (PEC, PEC, PEC), 30, id="N3-pec"),
    pytest.param(4, (3, 2, 2), (PER, PEC, PER), 30, id="N4-mixed-bc"),
    pytest.param(7, (2, 2, 2), (PEC, PER, PEC), 20, id="N7"),
    pytest.param(6, (2, 2, 3), (PER, PER, PER), 20, id="N6-periodic"),
]


@pytest.mark.gpu
@pytest.mark.parametrize("N,nel,bc,nsteps", MESHES)
def test_adjoint_matches_central_differences(N, nel, bc, nsteps):
    pb, eps, _, _ = gpu_problem(N, nel, bc, seed=21 + N, nsteps=nsteps)
    J, grad = pb.gradient(eps)
    assert J == pytest.approx(pb.objective(eps), rel=1e-14)
    rng = np.random.default_rng(100 + N)
    h = 1e-6
    worst = 0.0
    for _ in range(20):
        d = rng.standard_normal(eps.size)
        fd = (pb.objective(eps + h * d) - pb.objective(eps - h * d)) / (2 * h)
        ad = float(grad @ d)
        worst = max(worst, abs(fd - ad) / abs(ad))
    assert worst <= 1e-6, worst


@pytest.mark.gpu
def test_adjoint_matches_tape_node_by_node():
    N, nel, bc, nsteps = 3, (2, 2, 2), (PEC, PER, PEC), 12
    pb, eps, ref, xyz = gpu_problem(N, nel, bc, seed=31, nsteps=nsteps)
    J, grad = pb.gradient(eps)
    tm = make_tape(ref, xyz)
    eps_t = torch.tensor(eps, requires_grad=True)
    Jt = tape_J(tm, eps_t, pb.H0, pb.E0, pb.jw, nsteps, pb.dt)
    Jt.backward()
    assert J == pytest.approx(Jt.item(), rel=1e-12)
    gt = eps_t.grad.numpy()
    assert np.abs(grad - gt).max() <= 1e-9 * np.abs(gt).max()


@pytest.mark.gpu
@pytest.mark.parametrize("N,nel,bc,nsteps", MESHES)
def test_mixed_forward_adjoint_matches_fp64_and_central_differences(N, nel, bc, nsteps):
    """Forward steps in the mixed form, reverse stages in FP64: J within
    1e-8 and dJ/deps within 1e-8 (of its largest entry) of the all-FP64
    gradient, and central differences of the FP64 forward (h = 1e-6, 20
    directions) within 1e-6 relative."""
    pb, eps, _, _ = gpu_problem(N, nel, bc, seed=21 + N, nsteps=nsteps)
    J0, g0 = pb.gradient(eps)
    pb.form = "mixed"
    J1, g1 = pb.gradient(eps)
    assert J1 == pytest.approx(J0, rel=1e-8)
    assert np.abs(g1 - g0).max() <= 1e-8 * np.abs(g0).max()
    rng = np.random.default_rng(200 + N)
    h = 1e-6
    worst = 0.0
    for _ in range(20):
        d = rng.standard_normal(eps.size)
        fd = (pb.objective(eps + h * d) - pb.objective(eps - h * d)) / (2 * h)
        ad = float(g1 @ d)
        worst = max(worst, abs(fd - ad) / abs(ad))
    assert worst <= 1e-6, worst


@pytest.mark.gpu
@pytest.mark.parametrize("N,nel,bc,nsteps", [MESHES[1], MESHES[2]])
def test_mixed_recompute_matches_exact_and_central_differences(N, nel, bc, nsteps):
    """Fused FP64 context, sqrt(steps) segments recomputed in mixed stages
    from the FP64 checkpoints: J is the FP64 forward's (bit for bit), dJ/deps
    within 1e-8 (of its largest entry) of the exact gradient, and central
    differences of the FP64 forward (h = 1e-6, 10 directions) within 1e-6."""
    pb, eps, _, _ = gpu_problem(N, nel, bc, seed=21 + N, nsteps=nsteps, stride=4)
    J0, g0 = pb.gradient(eps)
    pb.recompute_mixed = True
    J1, g1 = pb.gradient(eps)
    assert J1 == J0
    assert np.abs(g1 - g0).max() <= 1e-8 * np.abs(g0).max()
    rng = np.random.default_rng(300 + N)
    h = 1e-6
    worst = 0.0
    for _ in range(10):
        d = rng.standard_normal(eps.size)
        fd = (pb.objective(eps + h * d) - pb.objective(eps - h * d)) / (2 * h)
        ad = float(g1 @ d)
        worst = max(worst, abs(fd - ad) / abs(ad))
    assert worst <= 1e-6, worst


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["fused64", "mixed"])
def test_host_snapshots_give_the_same_gradient(form):
    """Four binomial snapshots split between device and pinned host memory
    (4+0, 3+1, 2+2, 1+3): the same schedule, so bit-identical gradients, and
    the final state left in the context equals a plain forward run's."""
    pb, eps, _, _ = gpu_problem(4, (2, 2, 2), (PEC, PER, PEC), seed=73, nsteps=13)
    pb.form = form
    pb.stride = -4
    J0, g0 = pb.gradient(eps)
    for dev, host in ((3, 1), (2, 2), (1, 3)):
        pb.stride, pb.host_snapshots = -dev, host
        J1, g1 = pb.gradient(eps)
        assert J1 == J0
        np.testing.assert_array_equal(g1, g0, err_msg=f"{dev} device + {host} host")
    g = pb.context(eps, form)
    g.adjoint_gradient(pb.nsteps, 0.0, pb.dt, pb.jw, -1, host_snapshots=3)
    H, E = g.get_state()
    g.close()
    g = pb.context(eps, form)
    g.run(pb.nsteps, 0.0, pb.dt)
    H2, E2 = g.get_state()
    g.close()
    np.testing.assert_array_equal(H, H2)
    np.testing.assert_array_equal(E, E2)


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["fused64", "mixed"])
def test_adjoint_gradient_does_not_depend_on_the_checkpoint_stride(form):
    pb, eps, _, _ = gpu_problem(4, (2, 2, 2), (PEC, PEC, PEC), seed=41, nsteps=17)
    pb.form = form
    grads = []
    for stride in (1, 4, 17, 0):
        pb.stride = stride
        grads.append(pb.gradient(eps)[1])
    for g in grads[1:]:
        np.testing.assert_array_equal(g, grads[0])


@pytest.mark.gpu
def test_autograd_function_backward_is_the_adjoint():
    from adjoint_autograd import FieldEnergy
    pb, eps, _, _ = gpu_problem(3, (2, 2, 2), (PEC, PEC, PEC), seed=51, nsteps=10)
    eps_t = torch.tensor(eps, requires_grad=True)
    J = FieldEnergy.apply(eps_t, pb)
    (2.0 * J).backward()
    _, grad = pb.gradient(eps)
    np.testing.assert_array_equal(eps_t.grad.numpy(), 2.0 * grad)


@pytest.mark.gpu
def test_adjoint_rejects_other_forms_and_missing_state():
    g = MaxwellGPU.from_box(3, (2, 2, 2), (0, 0, 0), (1, 1, 1), (PEC,) * 3, form="mixed_naive")
    g.set_state(np.zeros((3, g.npts)), np.zeros((3, g.npts)))
    with pytest.raises(L.NekgpuError) as e:
        g.adjoint_gradient(2, 0.0, 0.01, np.ones(g.npts))
    assert e.value.status == -8
    g.close()
    g = MaxwellGPU.from_box(3, (2, 2, 2), (0, 0, 0), (1, 1, 1), (PEC,) * 3, form="fused64")
    with pytest.raises(L.NekgpuError) as e:
        g.adjoint_gradient(2, 0.0, 0.01, np.ones(g.npts))
    assert e.value.status == -5
    g.close()


@pytest.mark.gpu
def test_adjoint_init_run_equals_gradient():
    pb, eps, _, _ = gpu_problem(3, (2, 2, 2), (PEC, PER, PEC), seed=61, nsteps=9, stride=2)
    J0, g0 = pb.gradient(eps)
    g = pb.context(eps)
    with pytest.raises(L.NekgpuError) as e:
        g.adjoint_run(pb.nsteps, 0.0, pb.dt)
    assert e.value.status == -5
    g.adjoint_init(pb.jw, 2)
    J1, g1 = g.adjoint_run(pb.nsteps, 0.0, pb.dt)
    g.close()
    assert J1 == J0
    np.testing.assert_array_equal(g1, g0)


@pytest.mark.gpu
def test_binomial_schedule_gives_the_same_gradient():
    """Snapshot schedules (1, 2, 3 and 8 snapshots) against sqrt(steps)
    segments: the same forward states and reverse stages in the same order,
    so bit-identical gradients."""
    pb, eps, _, _ = gpu_problem(4, (2, 2, 2), (PEC, PER, PEC), seed=71, nsteps=13)
    J0, g0 = pb.gradient(eps)
    for snaps in (1, 2, 3, 8):
        pb.stride = -snaps
        J1, g1 = pb.gradient(eps)
        assert J1 == J0
        np.testing.assert_array_equal(g1, g0, err_msg=f"{snaps} snapshots")


@pytest.mark.gpu
def test_memory_budget_selects_the_binomial_schedule(monkeypatch):
    """Under a device-memory budget too small for the sqrt(steps) segment
    storage the automatic schedule falls back to snapshots and gives the same
    gradient; a forced stride that does not fit is refused."""
    pb, eps, _, _ = gpu_problem(7, (4, 4, 4), (PEC, PEC, PEC), seed=81, nsteps=64)
    J0, g0 = pb.gradient(eps)  # no budget: sqrt(64) = 8-step segments
    monkeypatch.setenv("NEKGPU_MEM_BUDGET_MB", "120")  # segments need ~150-280 MB
    J1, g1 = pb.gradient(eps)
    assert J1 == J0
    np.testing.assert_array_equal(g1, g0)
    pb.stride = 8
    with pytest.raises(L.NekgpuError) as e:
        pb.gradient(eps)
    assert e.value.status == -4


@pytest.mark.gpu
def test_adjoint_workload_matches_central_differences_at_full_length():
    """The adjoint configuration at its own size and length: unit PEC box,
    8^3 elements, N=7, eps = 1 + 3 sigmoid(Gaussian random field, length
    0.15, seed 4), the Gaussian E_z source (sigma 0.05 at 0.3 (1,1,1),
    Ricker), zero initial fields, 2000 RK45 steps, J = sum bm1 |E|^2 over the
    probe cube [0.7, 0.9]^3 at the final time.  dJ/deps from the adjoint with
    sqrt(steps) checkpointing against central differences of the FP64
    forward, h = 1e-6, 20 directions v ~ N(0,1) per node from seeds
    1000..1019, 1e-6 relative."""
    from adjoint_autograd import BoxProblem
    c = cases.make("adjoint")
    g = MaxwellGPU.from_box(c.N, c.nel, c.lo, c.hi, c.bc, form="fused64")
    x, y, z = g.coords()
    bm1 = g.array("bmn")
    g.close()
    eps = c.eps(x, y, z)
    (p0, p1), (q0, q1), (r0, r1) = c.extra["probe"]
    inside = (x > p0) & (x < p1) & (y > q0) & (y < q1) & (z > r0) & (z < r1)
    jw = np.where(inside, bm1, 0.0)
    H0, E0 = c.init_fields(x, y, z)
    dt = c.timestep(x, y, z)
    pb = BoxProblem(c.N, c.nel, c.lo, c.hi, c.bc, H0, E0, jw, c.nsteps, dt, source=c.source)
    J, grad = pb.gradient(eps)
    pb.recompute_mixed = True  # the same with the segments recomputed in mixed stages
    Jm, gradm = pb.gradient(eps)
    assert c.nsteps == 2000
    assert J == pytest.approx(pb.objective(eps), rel=1e-14)
    assert Jm == J
    h = 1e-6
    worst = worst_m = 0.0
    for seed in range(1000, 1020):
        d = np.random.default_rng(seed).standard_normal(eps.size)
        fd = (pb.objective(eps + h * d) - pb.objective(eps - h * d)) / (2 * h)
        ad, adm = float(grad @ d), float(gradm @ d)
        worst = max(worst, abs(fd - ad) / abs(ad))
        worst_m = max(worst_m, abs(fd - adm) / abs(adm))
    assert worst <= 1e-6, worst
    assert worst_m <= 1e-6, worst_m
