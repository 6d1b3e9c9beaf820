"""Test and benchmark cases: what a NekCEM ``.usr`` file supplies for the
Maxwell path (userini / usersol / uservp / usersrc) plus the mesh and dt.

Cases
  3dboxpec   the reference's known-answer PEC cavity test
             (tests/3dboxpec/3dboxpec.usr:64-119; 27 el, N=8, dt=0.005)
  3dboxper   the reference's periodic known-answer test
             (tests/3dboxper/3dboxper.usr:45-86; 4x4x8 el, N=8, dt=2e-4)
  cavity     PEC cavity [0,1]^3, 4^3 el, N=7, TM(1,1,0) mode, 1000 steps
  planewave  periodic [0,2pi]^3, 16^3 el, N=7, k=(1,1,1) plane wave, 2000 steps
  dielectric PEC box [0,1]^3, 32^3 el, N=5, eps=4 in a sphere, Gaussian E_z pulse
  adjoint    PEC box [0,1]^3, 8^3 el, N=7, smooth random eps, E_z source
  large      PEC box [0,1]^3, 64^3 el, N=7, smooth random eps in [1,4]
Inputs are synthetic and seeded (numpy default_rng); the reference ships no
data sets for this path.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Callable, Optional, Sequence

import numpy as np

PEC, PERIODIC = 0, 1
TWO_PI = 2.0 * np.pi


@dataclass
class Case:
    name: str
    N: int
    nel: Sequence[int]
    lo: Sequence[float]
    hi: Sequence[float]
    bc: Sequence[int]
    nsteps: int
    dt: Optional[float] = None       # fixed dt (param(12) < 0) ...
    cfl: Optional[float] = None      # ... or dt = 0.5 * cfl * min GLL spacing
    exact: Optional[Callable] = None  # (x, y, z, t) -> (H(3,n), E(3,n))
    initial: Optional[Callable] = None
    eps: Optional[Callable] = None   # (x, y, z) -> eps per node
    source: Optional[dict] = None
    l2tol: Optional[float] = None
    linftol: Optional[float] = None
    extra: dict = field(default_factory=dict)

    @property
    def nelt(self) -> int:
        return int(np.prod(self.nel))

    @property
    def npts(self) -> int:
        return self.nelt * (self.N + 1) ** 3

    def init_fields(self, x, y, z):
        if self.initial is not None:
            return self.initial(x, y, z)
        return self.exact(x, y, z, 0.0)

    def timestep(self, x, y, z) -> float:
        if self.dt is not None:
            return self.dt
        return 0.5 * self.cfl * min_gll_spacing(x, y, z, self.N + 1, self.nelt)


def get_dxmin(x, y, z, n: int, nelt: int) -> float:
    """get_dxmin (src/nek5_courant.F:2-75): half the smallest distance between
    the two neighbours of an interior GLL node, over the three directions."""
    X = np.asarray(x).reshape(nelt, n, n, n)  # (e, k, j, i)
    Y = np.asarray(y).reshape(nelt, n, n, n)
    Z = np.asarray(z).reshape(nelt, n, n, n)
    d2m = 1.0e20
    inner = slice(1, n - 1)
    for ax in (3, 2, 1):  # i, j, k
        def span(A):
            sl_p = [slice(None), inner, inner, inner]
            sl_m = [slice(None), inner, inner, inner]
            sl_p[ax] = slice(2, n)
            sl_m[ax] = slice(0, n - 2)
            return A[tuple(sl_p)] - A[tuple(sl_m)]
        dx, dy, dz = span(X), span(Y), span(Z)
        d2m = min(d2m, float(np.min(dx * dx + dy * dy + dz * dz)))
    return float(np.sqrt(d2m) / 2.0)


def min_gll_spacing(x, y, z, n: int, nelt: int) -> float:
    """Smallest distance between adjacent GLL nodes of any element."""
    P = [np.asarray(a).reshape(nelt, n, n, n) for a in (x, y, z)]
    best = np.inf
    for ax in (3, 2, 1):
        sl_p = [slice(None)] * 4
        sl_m = [slice(None)] * 4
        sl_p[ax] = slice(1, n)
        sl_m[ax] = slice(0, n - 1)
        d2 = sum((A[tuple(sl_p)] - A[tuple(sl_m)]) ** 2 for A in P)
        best = min(best, float(np.min(d2)))
    return float(np.sqrt(best))


# ---- analytic solutions ------------------------------------------------------

def sol_3dboxpec(x, y, z, t):
    """usersol of tests/3dboxpec/3dboxpec.usr:64-119 (omega = pi*sqrt(3))."""
    ww = np.pi
    tmph = np.cos(ww * np.sqrt(3.0) * t) / np.sqrt(6.0)
    tmpe = np.sin(ww * np.sqrt(3.0) * t) / np.sqrt(2.0)
    sx, cx = np.sin(ww * x), np.cos(ww * x)
    sy, cy = np.sin(ww * y), np.cos(ww * y)
    sz, cz = np.sin(ww * z), np.cos(ww * z)
    H = np.stack([-sx * cy * cz * tmph, -cx * sy * cz * tmph, 2 * cx * cy * sz * tmph])
    E = np.stack([-cx * sy * sz * tmpe, sx * cy * sz * tmpe, 0 * x])
    return H, E


def sol_3dboxper(x, y, z, t):
    """usersol of tests/3dboxper/3dboxper.usr:45-86 (omega = sqrt(3))."""
    om = np.sqrt(3.0)
    tmph = np.sin(om * t) / om
    tmpe = np.cos(om * t)
    H = np.stack([2 * np.cos(x) * np.sin(y) * np.cos(z) * tmph,
                  -np.sin(x) * np.cos(y) * np.cos(z) * tmph,
                  np.sin(x) * np.sin(y) * np.sin(z) * tmph])
    E = np.stack([0 * x, np.cos(x) * np.sin(y) * np.sin(z) * tmpe,
                  np.cos(x) * np.cos(y) * np.cos(z) * tmpe])
    return H, E


def sol_tm110(x, y, z, t):
    """TM(1,1,0) mode of the unit PEC cavity, omega = pi*sqrt(2):
    Ez = sin(pi x) sin(pi y) cos(wt), Hx = -(pi/w) sin(pi x) cos(pi y) sin(wt),
    Hy = (pi/w) cos(pi x) sin(pi y) sin(wt)."""
    w = np.pi * np.sqrt(2.0)
    sx, cx = np.sin(np.pi * x), np.cos(np.pi * x)
    sy, cy = np.sin(np.pi * y), np.cos(np.pi * y)
    st, ct = np.sin(w * t), np.cos(w * t)
    H = np.stack([-(np.pi / w) * sx * cy * st, (np.pi / w) * cx * sy * st, 0 * x])
    E = np.stack([0 * x, 0 * x, sx * sy * ct])
    return H, E


def sol_planewave(x, y, z, t):
    """Plane wave k=(1,1,1), omega=sqrt(3), E = e cos(k.x - wt) with
    e = (1,-1,0)/sqrt(2) and H = khat x E = (1,1,-2)/sqrt(6) cos(k.x - wt)."""
    ph = np.cos(x + y + z - np.sqrt(3.0) * t)
    e = np.array([1.0, -1.0, 0.0]) / np.sqrt(2.0)
    h = np.array([1.0, 1.0, -2.0]) / np.sqrt(6.0)
    E = e[:, None] * ph[None, :]
    H = h[:, None] * ph[None, :]
    return H, E


# ---- materials and sources -----------------------------------------------------

TE, TM = 1, 2
BOTH = 3  # TE and TM superposed (3-D cases only)


def sol_2dboxpec(mode: int):
    """tests/2dboxpec/2dboxpec.usr usersol: [-1,1]^2 PEC, w = 1.5 pi,
    omega = sqrt(2); TM: Hx, Hy, Ez; TE: Hz, Ex, Ey."""
    ww, om = 1.5 * np.pi, np.sqrt(2.0)

    def sol(x, y, z, t):
        tmph = np.sin(ww * om * t) / om
        tmpe = np.cos(ww * om * t)
        zero = np.zeros_like(x)
        if mode == TM:
            H = np.stack([np.cos(ww * x) * np.sin(ww * y) * tmph,
                          -np.sin(ww * x) * np.cos(ww * y) * tmph, zero])
            E = np.stack([zero, zero, np.cos(ww * x) * np.cos(ww * y) * tmpe])
        else:
            H = np.stack([zero, zero, np.sin(ww * x) * np.sin(ww * y) * tmpe])
            E = np.stack([np.sin(ww * x) * np.cos(ww * y) * tmph,
                          -np.cos(ww * x) * np.sin(ww * y) * tmph, zero])
        return H, E
    return sol


def sol_2dboxper(mode: int):
    """tests/2dboxper/2dboxper.usr usersol: [0,2pi]^2 periodic, omega = sqrt(2)."""
    om = np.sqrt(2.0)

    def sol(x, y, z, t):
        zero = np.zeros_like(x)
        if mode == TM:
            tmph, tmpe = np.sin(om * t) / om, np.cos(om * t)
            H = np.stack([np.cos(x) * np.sin(y) * tmph, -np.sin(x) * np.cos(y) * tmph, zero])
            E = np.stack([zero, zero, np.cos(x) * np.cos(y) * tmpe])
        else:
            tmph, tmpe = np.cos(om * t), np.sin(om * t) / om
            H = np.stack([zero, zero, np.sin(x) * np.sin(y) * tmph])
            E = np.stack([np.sin(x) * np.cos(y) * tmpe, -np.cos(x) * np.sin(y) * tmpe, zero])
        return H, E
    return sol


# the reference's 2-D known-answer cases: 3x3 quadrilaterals, N=8, dt 0.005,
# 1000 steps; tolerances per active component (userchk)
CASES_2D = {
    "2dboxpec": dict(N=8, nel=(3, 3), lo=(-1.0, -1.0), hi=(1.0, 1.0), bc=(PEC, PEC), dt=0.005,
                     nsteps=1000, sol=sol_2dboxpec, l2tol=1e-6, linftol=1e-5),
    "2dboxper": dict(N=8, nel=(3, 3), lo=(0.0, 0.0), hi=(TWO_PI, TWO_PI), bc=(PERIODIC, PERIODIC),
                     dt=0.005, nsteps=1000, sol=sol_2dboxper, l2tol=5e-8, linftol=5e-7),
}


def eps_sphere(x, y, z, center=(0.5, 0.5, 0.5), radius=0.25, inside=4.0):
    r2 = (x - center[0]) ** 2 + (y - center[1]) ** 2 + (z - center[2]) ** 2
    return np.where(r2 < radius * radius, inside, 1.0)


def gaussian_random_field(x, y, z, length: float, seed: int, nfeat: int = 512):
    """Zero-mean, unit-variance smooth random field from random Fourier
    features: g = sqrt(2/F) sum_f cos(k_f . x + phi_f), k_f ~ N(0, 1/length^2).
    Evaluated in node blocks (bounded temporaries); on a CUDA device through
    torch when one is present and the mesh is large."""
    rng = np.random.default_rng(seed)
    k = rng.normal(0.0, 1.0 / length, size=(nfeat, 3))
    ph = rng.uniform(0.0, TWO_PI, size=nfeat)
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    z = np.asarray(z, dtype=np.float64)
    n = x.size
    g = np.zeros(n)
    if n > 4_000_000:
        try:
            import torch
            if torch.cuda.is_available():
                dev = torch.device("cuda")
                kt = torch.tensor(k, device=dev)
                pt = torch.tensor(ph, device=dev)
                for s0 in range(0, n, 1 << 20):
                    s1 = min(n, s0 + (1 << 20))
                    xyz = torch.tensor(np.stack([x[s0:s1], y[s0:s1], z[s0:s1]], axis=1), device=dev)
                    g[s0:s1] = torch.cos(xyz @ kt.T + pt).sum(dim=1).cpu().numpy()
                return g * np.sqrt(2.0 / nfeat)
        except ImportError:
            pass
    block, chunk = 1 << 16, 64
    for s0 in range(0, n, block):
        s1 = min(n, s0 + block)
        for f0 in range(0, nfeat, chunk):
            kk = k[f0:f0 + chunk]
            arg = (np.outer(x[s0:s1], kk[:, 0]) + np.outer(y[s0:s1], kk[:, 1])
                   + np.outer(z[s0:s1], kk[:, 2]) + ph[f0:f0 + chunk])
            g[s0:s1] += np.cos(arg).sum(axis=1)
    return g * np.sqrt(2.0 / nfeat)


def eps_random(x, y, z, seed: int, length: float = 0.15):
    g = gaussian_random_field(x, y, z, length, seed)
    return 1.0 + 3.0 / (1.0 + np.exp(-g))


def gaussian_pulse_ez(center, sigma):
    def init(x, y, z):
        r2 = (x - center[0]) ** 2 + (y - center[1]) ** 2 + (z - center[2]) ** 2
        E = np.stack([0 * x, 0 * x, np.exp(-r2 / (2 * sigma * sigma))])
        return np.zeros_like(E), E
    return init


class DispersiveWave:
    """Plane wave along x (E_y, H_z) in a uniform dispersive medium, the
    analytic mode of the Maxwell system with the reference's polarisation
    currents (cem_maxwell_drude / cem_maxwell_lorentz,
    src/cem_maxwell.F:3095-3212):

        eps dE/dt = curl H - J1,   mu dH/dt = -curl E,
        Drude:   dJ1/dt = -a J1 + b E
        Lorentz: dJ1/dt = -a J1 - b J2 + c E,   dJ2/dt = J1

    Fields are Re(X exp(i(k x - w t))) with E_y amplitude 1 and the complex
    frequency w a root of the dispersion relation (the least damped root with
    Re w > 0, the upper branch when there are two)."""

    def __init__(self, model: str, a: float, b: float, c: float = 0.0, k: float = 1.0,
                 eps: float = 1.0, mu: float = 1.0):
        self.model, self.a, self.b, self.c = model, a, b, c
        self.k, self.eps, self.mu = k, eps, mu
        k2 = k * k / mu
        if model == "drude":
            poly = [-1j * eps, a * eps, 1j * (k2 + b), -a * k2]
        elif model == "lorentz":
            poly = [-eps, -1j * a * eps, eps * b + k2 + c, 1j * a * k2, -b * k2]
        else:
            raise KeyError(model)
        roots = [w for w in np.roots(poly) if w.real > 1e-9]
        self.omega = max(roots, key=lambda w: (round(w.imag, 12), w.real))
        w = self.omega
        self.Hh = k / (mu * w)
        if model == "drude":
            self.J1 = b / (a - 1j * w)
            self.J2 = 0.0
        else:
            den = b - w * w - 1j * a * w
            self.J1 = c * (-1j * w) / den
            self.J2 = c / den

    def residual(self) -> float:
        """|-i w eps E + i k H + J1| of the E equation (0 up to rounding)"""
        w = self.omega
        return abs(-1j * w * self.eps + 1j * self.k * self.Hh + self.J1)

    def exact(self, x, y, z, t):
        ph = np.exp(1j * (self.k * np.asarray(x) - self.omega * t))
        zero = np.zeros(np.shape(x))
        H = np.stack([zero, zero, (self.Hh * ph).real])
        E = np.stack([zero, (ph).real, zero])
        return H, E

    def currents(self, x, y, z, t):
        """J1 (3, n) for Drude; J1 then J2 (6, n) for Lorentz"""
        ph = np.exp(1j * (self.k * np.asarray(x) - self.omega * t))
        zero = np.zeros(np.shape(x))
        J = [zero, (self.J1 * ph).real, zero]
        if self.model == "lorentz":
            J += [zero, (self.J2 * ph).real, zero]
        return np.stack(J)


class DrudeHalfSpace:
    """The reference's tests/drude case (a normally incident plane wave on a
    Drude half-space, tests/drude/drude.usr) restated in 3-D: x and z
    periodic, 'PML' at both y ends (6 layers, order 3, error 1e-15; the
    reference has PEC below, where the transmitted wave has decayed by
    e^-43), vacuum above y = 0, a Drude medium below (eps_inf = 1, a = 0,
    b = 100, so eps(omega = 5) = -3 and the wave is totally reflected).  The
    incident field cos(-k1 y - omega t) (H_z, eta1 E_x) enters through the
    y = 0 faces of the upper elements (userinc); above them the field is the
    reflected wave (damped inside the PML as usersol damps it), below it the
    evanescent transmitted wave with its Drude current.

    model="lorentz" restates tests/lorentz/lorentz.usr the same way: a
    Lorentz half-space with a = 0, b = 0.9 omega^2, c = b (eps = -8), its
    two currents initialised as the case's userini does; userchk's
    tolerances there are L2 5e-6 and Linf 5e-5 on H_z and E_x."""

    N, nel = 8, (2, 32, 2)
    lo, hi = (-2.5, -5.0, -2.5), (2.5, 5.0, 2.5)
    bc = (PERIODIC, 2, PERIODIC)
    pml = (6, 3.0, 1e-15)
    dt, nsteps = 0.005, 1000
    omega, a, b, c = 5.0, 0.0, 100.0, 0.0

    def __init__(self, model: str = "drude"):
        self.model = model
        w = self.omega
        if model == "lorentz":
            self.a, self.b = 0.0, 0.9 * w * w
            self.c = self.b
            self.eps2 = 1.0 + self.c / (self.b - 1j * self.a * w - w * w)
            self.l2tol, self.linftol = 5e-6, 5e-5
        else:
            self.eps2 = 1.0 - self.b / (w * (w + 1j * self.a))
            self.l2tol, self.linftol = 1e-7, 5e-6
        self.eta1 = 1.0
        eta2 = np.sqrt(1.0 / self.eps2 + 0j)
        if eta2.real == 0.0 and eta2.imag > 0.0:  # the branch drude.usr picks
            eta2 = -eta2
        self.eta2 = eta2
        self.k1 = w
        self.k2 = w * np.sqrt(self.eps2 + 0j)
        self.refl = (self.eta1 - eta2) / (self.eta1 + eta2)
        self.tran = 2 * self.eta1 / (self.eta1 + eta2)
        hy = (self.hi[1] - self.lo[1]) / self.nel[1]
        self.pml_inner = self.hi[1] - self.pml[0] * hy
        self.pml_outer = self.hi[1]

    def regions(self, y, n3):
        """per node: upper (element centre y > 0) and inside the upper PML"""
        yc = np.repeat(np.asarray(y).reshape(-1, n3).mean(axis=1), n3)
        return yc > 0.0, yc > self.pml_inner

    def exact(self, x, y, z, t, n3):
        up, inpml = self.regions(y, n3)
        d = self.pml_outer - self.pml_inner
        order, referr = self.pml[1], self.pml[2]
        smax = -(order + 1) * np.log(referr) / (2.0 * self.eta1 * d)
        fac = np.where(inpml, (smax * d / (order + 1)) * np.clip((y - self.pml_inner) / d, 0, None)
                       ** (order + 1), 0.0)
        w = self.omega
        usc_up = self.refl * np.exp(1j * (self.k1 * y - w * t) - self.eta1 * fac)
        usc_lo = self.tran * np.exp(1j * (-self.k2 * y - w * t))
        zero = np.zeros_like(y)
        Hz = np.where(up, usc_up.real, usc_lo.real)
        Ex = np.where(up, (-self.eta1 * usc_up).real, (self.eta2 * usc_lo).real)
        return np.stack([zero, zero, Hz]), np.stack([Ex, zero, zero])

    def drude(self, y, n3):
        """node indices of the dispersive medium, its parameters ((2, n)
        Drude, (3, n) Lorentz) and the initial currents ((3, n) Drude J;
        (6, n) Lorentz J1 then J2), as the cases' userini set them"""
        up, _ = self.regions(y, n3)
        idx = np.nonzero(~up)[0]
        n = np.size(y)
        w = self.omega
        efac = self.tran * self.eta2 * np.exp(1j * (-self.k2 * np.asarray(y)))
        if self.model == "lorentz":
            params = np.stack([np.full(n, self.a), np.full(n, self.b), np.full(n, self.c)])
            sig = 1j * self.c * w / (w * w + 1j * self.a * w - self.b)
            J = np.zeros((6, n))
            J[0, idx] = (sig * efac).real[idx]
            J[3, idx] = ((1j / w) * sig * efac).real[idx]
            return idx, params, J
        params = np.stack([np.full(n, self.a), np.full(n, self.b)])
        sig = self.b / (self.a - 1j * w)
        J = np.zeros((3, n))
        J[0, idx] = (sig * efac).real[idx]
        return idx, params, J

    def incident_slots(self, y, cemface, n3, nf):
        """0-based face slots of the upper elements' faces that lie on y = 0"""
        up, _ = self.regions(y, n3)
        y = np.asarray(y)
        cf = np.asarray(cemface).reshape(-1, nf)
        slots = []
        for f in range(cf.shape[0]):
            nodes = cf[f]
            if up[nodes[0]] and np.all(np.abs(y[nodes]) <= 1e-8):
                slots.extend(range(f * nf, (f + 1) * nf))
        return np.array(slots, dtype=np.int64)

    def incident(self):
        """amp (H then E), k and omega of userinc"""
        return (0.0, 0.0, 1.0, self.eta1, 0.0, 0.0), (0.0, -self.k1, 0.0), self.omega


class DielectricHalfSpace:
    """The reference's tests/2ddielectric case (twomat: a normally incident
    plane wave on a dielectric half-space eps2 = 2) restated in 3-D like
    DrudeHalfSpace: 2 x 32 x 2 elements on [-2.5,2.5] x [-5,5] x
    [-2.5,2.5], N=8, x and z periodic, 'PML' at both y ends (10 layers,
    order 3, error 1e-30, params 77-79 of 2ddielectric.rea: both the
    reflected and the transmitted wave leave
    through a PML, and usersol damps each inside its own), dt = 0.005, 1000
    steps; TE (H_z, E_x) or TM (E_z, H_x).  userchk's tolerances: L2 5e-7,
    Linf 5e-6 on the two active components; with one material (param(70) =
    0: eps2 = 1, the wave passes y = 0 unreflected) L2 5e-8, Linf 1e-6 (TE)
    or 5e-6 (TM).  mode BOTH runs TE and TM superposed (their components are
    disjoint), as tests/3ddielectric does."""

    N, nel = 8, (2, 32, 2)
    lo, hi = (-2.5, -5.0, -2.5), (2.5, 5.0, 2.5)
    bc = (PERIODIC, 2, PERIODIC)
    pml = (10, 3.0, 1e-30)
    dt, nsteps = 0.005, 1000
    omega, eps1, eps2 = 5.0, 1.0, 2.0
    l2tol, linftol = 5e-7, 5e-6

    def __init__(self, mode: int = TE, twomat: bool = True):
        self.mode = mode
        if not twomat:
            self.eps2 = 1.0
            self.l2tol, self.linftol = 5e-8, (1e-6 if mode == TE else 5e-6)
        z1, z2 = np.sqrt(1.0 / self.eps1), np.sqrt(1.0 / self.eps2)
        self.z1, self.z2 = z1, z2
        # uservp of the reference's dielectric cases
        self.reflte, self.trante = (z1 - z2) / (z1 + z2), 2 * z1 / (z1 + z2)
        self.refltm, self.trantm = (z2 - z1) / (z1 + z2), 2 * z2 / (z1 + z2)
        if mode == TM:
            self.refl, self.tran = self.refltm, self.trantm
        else:
            self.refl, self.tran = self.reflte, self.trante
        hy = (self.hi[1] - self.lo[1]) / self.nel[1]
        self.up_inner, self.up_outer = self.hi[1] - self.pml[0] * hy, self.hi[1]
        self.lo_inner, self.lo_outer = self.lo[1] + self.pml[0] * hy, self.lo[1]

    def active(self):
        """component indices (H1..H3, E1..E3 = 0..5) the wave lives in"""
        return {TE: (2, 3), TM: (0, 5)}.get(self.mode, (0, 2, 3, 5))

    def regions(self, y, n3):
        yc = np.repeat(np.asarray(y).reshape(-1, n3).mean(axis=1), n3)
        return yc > 0.0, (yc > self.up_inner) | (yc < self.lo_inner)

    def eps(self, y, n3):
        up, _ = self.regions(y, n3)
        return np.where(up, self.eps1, self.eps2)

    def exact(self, x, y, z, t, n3):
        """usersol: the reflected wave above y = 0, the transmitted one below,
        each damped inside its PML"""
        up, inpml = self.regions(y, n3)
        y = np.asarray(y)
        eps = np.where(up, self.eps1, self.eps2)
        eta, ky = np.sqrt(1.0 / eps), self.omega * np.sqrt(eps)
        order, referr = self.pml[1], self.pml[2]
        d_up = self.up_outer - self.up_inner
        d_lo = self.lo_inner - self.lo_outer
        with np.errstate(divide="ignore", invalid="ignore"):
            f_up = (-(order + 1) * np.log(referr) / (2 * eta * d_up) * d_up / (order + 1)) * \
                np.clip((y - self.up_inner) / d_up, 0, None) ** (order + 1)
            f_lo = (-(order + 1) * np.log(referr) / (2 * eta * d_lo) * d_lo / (order + 1)) * \
                np.clip((self.lo_inner - y) / d_lo, 0, None) ** (order + 1)
        fac = np.where(inpml, np.where(up, f_up, f_lo), 0.0)
        wave = np.where(up, np.exp(-eta * fac) * np.cos(ky * y - self.omega * t),
                        np.exp(-eta * fac) * np.cos(-ky * y - self.omega * t))
        zero = np.zeros_like(y)
        H = [zero, zero, zero]
        E = [zero, zero, zero]
        if self.mode in (TE, BOTH):
            uu = np.where(up, self.reflte, self.trante) * wave
            H[2] = uu
            E[0] = np.where(up, -eta * uu, eta * uu)
        if self.mode in (TM, BOTH):
            uu = np.where(up, self.refltm, self.trantm) * wave
            H[0] = np.where(up, uu / eta, -uu / eta)
            E[2] = uu
        return np.stack(H), np.stack(E)

    def incident_slots(self, y, cemface, n3, nf):
        up, _ = self.regions(y, n3)
        y = np.asarray(y)
        cf = np.asarray(cemface).reshape(-1, nf)
        out = []
        for f in range(cf.shape[0]):
            nodes = cf[f]
            if up[nodes[0]] and np.all(np.abs(y[nodes]) <= 1e-8):
                out.extend(range(f * nf, (f + 1) * nf))
        return np.array(out, dtype=np.int64)

    def incident(self):
        """userinc: amplitudes (H1..H3, E1..E3) of cos(-ky y - omega t)"""
        eta, ky = np.sqrt(1.0 / self.eps1), self.omega * np.sqrt(self.eps1)
        te = (0.0, 0.0, 1.0, eta, 0.0, 0.0)   # incfhz += u, incfex += eta u
        tm = (-1.0 / eta, 0.0, 0.0, 0.0, 0.0, 1.0)  # incfhx -= u/eta, incfez += u
        if self.mode == TE:
            amp = te
        elif self.mode == TM:
            amp = tm
        else:
            amp = tuple(a + b for a, b in zip(te, tm))
        return amp, (0.0, -ky, 0.0), self.omega


class Dielectric3D(DielectricHalfSpace):
    """The reference's tests/3ddielectric case (maxwell-3ddielectric-1mat and
    -2mat, param(70) = 0 | 1): TE and TM plane waves together, normally
    incident from y > 0 on eps2 = 1 or 2, omega = 2; 4 x 8 x 4 elements on
    [-2.5,2.5] x [-5,5] x [-2.5,2.5] (usrdat2 scales the [-1,1]^3 box), N=8
    (SIZE lxi = 8), x and z periodic, 'PML' at both y ends (2 layers, order 3,
    error 1e-10: params 77-79), dt = 0.005, 1000 steps.  userchk's
    tolerances per component H1..H3, E1..E3: L2 5e-4, 5e-14, 5e-4, 5e-4,
    5e-14, 5e-4; Linf 5e-3 on the active components and 1e-12 (2mat) or
    5e-12 (1mat) on H2 and E2."""

    nel = (4, 8, 4)
    pml = (2, 3.0, 1e-10)
    omega = 2.0

    def __init__(self, twomat: bool):
        self.eps2 = 2.0 if twomat else 1.0
        super().__init__(BOTH)
        q = 1e-12 if twomat else 5e-12
        self.l2tol = (5e-4, 5e-14, 5e-4, 5e-4, 5e-14, 5e-4)
        self.linftol = (5e-3, q, 5e-3, 5e-3, q, 5e-3)


class GrapheneSheet:
    """The reference's tests/3dgraphene case: two superimposed normally
    incident plane waves (TE: H_z, E_x; TM: E_z, H_x) from y > 0 on a
    graphene sheet at y = 0 (Drude term plus two critical points,
    cem_3d_graphene_current), vacuum on both sides, 'PML' at both y ends
    (2 layers, order 3, error 1e-10), x and z periodic; 4 x 12 x 4 elements
    on [-2.5,2.5] x [-5,5] x [-2.5,2.5], N=8, dt = 0.005, 1000 steps.  The
    exact solution is the reflected wave above and the transmitted wave
    below, each damped inside its PML as usersol damps it."""

    N, nel = 8, (4, 12, 4)
    lo, hi = (-2.5, -5.0, -2.5), (2.5, 5.0, 2.5)
    bc = (PERIODIC, 2, PERIODIC)
    pml = (2, 3.0, 1e-10)
    dt, nsteps = 0.005, 1000
    omega = 5.0
    # a_d, b_d, b_cp1, a_211, a_221, b_11, b_21, b_cp2, a_212, a_222, b_12, b_22
    params = (0.0, 1.499, -2.599e-03, 4.632e+05, 1.090e+03, -1.391, -3.125e+02,
              -1.049e-03, 4.271e+05, 2.742e+02, -7.769e-02, 4.268e+02)
    l2tol = (5e-4, 1e-14, 5e-4, 5e-4, 1e-14, 5e-4)
    linftol = (5e-3, 5e-12, 5e-3, 5e-3, 5e-12, 5e-3)

    def __init__(self):
        w, CI = self.omega, 1j
        a_d, b_d, b_cp1, a_211, a_221, b_11, b_21, b_cp2, a_212, a_222, b_12, b_22 = self.params
        s_d = b_d / (a_d - CI * w)
        s_cp1 = (CI / w) * ((a_211 * b_11 + CI * w * b_21) / (w ** 2 - a_211 + CI * w * a_221) + b_11) - b_cp1
        s_cp2 = (CI / w) * ((a_212 * b_12 + CI * w * b_22) / (w ** 2 - a_212 + CI * w * a_222) + b_12) - b_cp2
        sg = s_d + s_cp1 + s_cp2
        z1 = z2 = 1.0
        self.sigma = sg
        self.reflte = (z1 - z2 + sg * z1 * z2) / (z1 + z2 + sg * z1 * z2)
        self.trante = 2 * z1 / (z1 + z2 + sg * z1 * z2)
        self.refltm = (z2 - z1 - z1 * z2 * sg) / (z1 + z2 + z1 * z2 * sg)
        self.trantm = 2 * z2 / (z1 + z2 + z1 * z2 * sg)
        hy = (self.hi[1] - self.lo[1]) / self.nel[1]
        self.up_inner, self.up_outer = self.hi[1] - self.pml[0] * hy, self.hi[1]
        self.lo_inner, self.lo_outer = self.lo[1] + self.pml[0] * hy, self.lo[1]

    def regions(self, y, n3):
        yc = np.repeat(np.asarray(y).reshape(-1, n3).mean(axis=1), n3)
        return yc > 0.0, (yc > self.up_inner) | (yc < self.lo_inner)

    def exact(self, x, y, z, t, n3):
        up, inpml = self.regions(y, n3)
        order, referr = self.pml[1], self.pml[2]
        w, eta, ky = self.omega, 1.0, self.omega
        d_up = self.up_outer - self.up_inner
        d_lo = self.lo_inner - self.lo_outer
        smax_up = -(order + 1) * np.log(referr) / (2 * eta * d_up)
        smax_lo = -(order + 1) * np.log(referr) / (2 * eta * d_lo)
        y = np.asarray(y)
        fac = np.where(up, (smax_up * d_up / (order + 1)) * np.clip((y - self.up_inner) / d_up, 0, None)
                       ** (order + 1),
                       (smax_lo * d_lo / (order + 1)) * np.clip((self.lo_inner - y) / d_lo, 0, None)
                       ** (order + 1))
        fac = np.where(inpml, fac, 0.0)
        uu_up = np.exp(1j * (ky * y - w * t) - eta * fac)
        uu_lo = np.exp(1j * (-ky * y - w * t) - eta * fac)
        zero = np.zeros_like(y)
        Hz = np.where(up, (self.reflte * uu_up).real, (self.trante * uu_lo).real)
        Ex = np.where(up, -(self.reflte * eta * uu_up).real, (self.trante * eta * uu_lo).real)
        Ez = np.where(up, (self.refltm * uu_up).real, (self.trantm * uu_lo).real)
        Hx = np.where(up, (self.refltm * uu_up / eta).real, -(self.trantm * uu_lo / eta).real)
        return np.stack([Hx, zero, Hz]), np.stack([Ex, zero, Ez])

    def face_slots(self, y, cemface, n3, nf, upper_only):
        up, _ = self.regions(y, n3)
        y = np.asarray(y)
        cf = np.asarray(cemface).reshape(-1, nf)
        out = []
        for f in range(cf.shape[0]):
            nodes = cf[f]
            if (up[nodes[0]] or not upper_only) and np.all(np.abs(y[nodes]) <= 1e-8):
                out.extend(range(f * nf, (f + 1) * nf))
        return np.array(out, dtype=np.int64)

    def sheet(self, y, cemface, n3, nf, nxzfl):
        """graphene slots (both sides of y = 0), params (12, nxzfl) and the
        initial face currents (6, 3, nxzfl) of userini"""
        slots = self.face_slots(y, cemface, n3, nf, upper_only=False)
        params = np.zeros((12, nxzfl))
        params[:, slots] = np.asarray(self.params)[:, None]
        w, CI = self.omega, 1j
        a_d, b_d, b_cp1, a_211, a_221, b_11, b_21, b_cp2, a_212, a_222, b_12, b_22 = self.params
        enpar = np.array([0.5 * 1.0 * (1.0 - self.reflte), 0.0, 0.5 * (1.0 + self.refltm)])
        fjn = np.zeros((6, 3, nxzfl))
        f2 = b_d / (a_d - CI * w)
        f4 = (a_211 * b_11 + CI * w * b_21) / (w ** 2 - a_211 + CI * w * a_221)
        f3 = (CI / w) * (f4 + b_11)
        f6 = (a_212 * b_12 + CI * w * b_22) / (w ** 2 - a_212 + CI * w * a_222)
        f5 = (CI / w) * (f6 + b_12)
        for k, fac in ((1, f2), (3, f4), (2, f3), (5, f6), (4, f5)):
            for m in range(3):
                fjn[k, m, slots] = (fac * enpar[m]).real
        return slots, params, fjn

    def incident_slots(self, y, cemface, n3, nf):
        return self.face_slots(y, cemface, n3, nf, upper_only=True)

    def incident(self):
        """amp (H then E), k, omega: incfhz += u, incfex += eta u, incfez += u,
        incfhx -= u/eta, u = cos(-ky y - omega t)"""
        return (-1.0, 0.0, 1.0, 1.0, 0.0, 1.0), (0.0, -self.omega, 0.0), self.omega


class Graphene2D(GrapheneSheet):
    """The reference's tests/2dgraphene (maxwell-2dgraphene-te / -tm) restated
    in 3-D like the other 2-D cases: one mode, TE (H_z, E_x) or TM (E_z, H_x),
    the same sheet model as tests/3dgraphene; 4 x 32 elements on [-2.5,2.5] x
    [-5,5] (usrdat2: sx = 5, sy = 10), two periodic elements along z on
    [-2.5,2.5] (no coarser than y, so dxmin is the 2-D one), N=8, 'PML' at
    both y ends (6 layers, order 3, error 1e-15: params 77-79), dt = 0.2
    dxmin (CFL 0.2), 1000 steps.  userchk's tolerances: L2 1e-7, Linf 5e-6 on
    the mode's two components.  The 2-D case also bounds E_y (TE) or H_y (TM),
    zero in the exact solution, by its 2-D round-off (L2 1e-14, Linf 5e-13);
    the 3-D operator's round-off there is larger (Linf 6.9e-13), so all
    components that are zero get the FP64 round-off bound of the tests."""

    nel = (4, 32, 2)
    pml = (6, 3.0, 1e-15)
    cfl = 0.2

    def __init__(self, mode: int):
        super().__init__()
        self.mode = mode
        act = (2, 3) if mode == TE else (0, 5)
        self.l2tol = tuple(1e-7 if q in act else None for q in range(6))
        self.linftol = tuple(5e-6 if q in act else None for q in range(6))

    def exact(self, x, y, z, t, n3):
        H, E = super().exact(x, y, z, t, n3)
        if self.mode == TE:  # H_z, E_x
            H[0] = 0.0; E[2] = 0.0
        else:  # E_z, H_x
            H[2] = 0.0; E[0] = 0.0
        return H, E

    def sheet(self, y, cemface, n3, nf, nxzfl):
        # userini's enpar for the one mode (tests/2dgraphene/2dgraphene.usr)
        keep = self.refltm, self.reflte
        if self.mode == TE:
            self.refltm = -1.0  # 0.5 (1 + refl) = 0 on z
        else:
            self.reflte = 1.0   # 0.5 z1 (1 - refl) = 0 on x
        try:
            return super().sheet(y, cemface, n3, nf, nxzfl)
        finally:
            self.refltm, self.reflte = keep

    def incident(self):
        amp, k, om = super().incident()
        if self.mode == TE:  # incfhz += u, incfex += eta u
            amp = (0.0, 0.0, 1.0, 1.0, 0.0, 0.0)
        else:  # incfez += u, incfhx -= u/eta
            amp = (-1.0, 0.0, 0.0, 0.0, 0.0, 1.0)
        return amp, k, om


def zero_fields(x, y, z):
    return np.zeros((3, x.size)), np.zeros((3, x.size))


def pulse_center(seed: int = 3):
    u = np.random.default_rng(seed).uniform(-1.0, 1.0, size=3)
    return tuple(0.5 + 0.05 * u)


# dt = 0.5 * CFL * (smallest adjacent GLL node distance) with CFL = 1.  At N=7
# that is 0.31 * dxmin of get_dxmin; the upwind RK45 scheme blows up above
# about 0.42 * dxmin there, so "0.5 * dxmin" is not a usable reading.
CFL = 1.0


def make(name: str, **over) -> Case:
    if name == "3dboxpec":
        c = Case(name, 8, (3, 3, 3), (-1, -1, -1), (1, 1, 1), (PEC,) * 3, 1000, dt=0.005,
                 exact=sol_3dboxpec, l2tol=5e-8, linftol=5e-7)
    elif name == "3dboxper":
        c = Case(name, 8, (4, 4, 8), (0, 0, 0), (TWO_PI,) * 3, (PERIODIC,) * 3, 50, dt=2e-4,
                 exact=sol_3dboxper, l2tol=5e-10, linftol=5e-9)
    elif name == "cavity":
        c = Case(name, 7, (4, 4, 4), (0, 0, 0), (1, 1, 1), (PEC,) * 3, 1000, cfl=CFL,
                 exact=sol_tm110)
    elif name == "planewave":
        c = Case(name, 7, (16, 16, 16), (0, 0, 0), (TWO_PI,) * 3, (PERIODIC,) * 3, 2000,
                 cfl=CFL, exact=sol_planewave)
    elif name == "dielectric":
        c = Case(name, 5, (32, 32, 32), (0, 0, 0), (1, 1, 1), (PEC,) * 3, 4000, cfl=CFL,
                 initial=gaussian_pulse_ez(pulse_center(3), 0.05), eps=eps_sphere)
    elif name == "adjoint":
        c = Case(name, 7, (8, 8, 8), (0, 0, 0), (1, 1, 1), (PEC,) * 3, 2000, cfl=CFL,
                 initial=zero_fields, eps=lambda x, y, z: eps_random(x, y, z, seed=4),
                 source=dict(xc=(0.3, 0.3, 0.3), sigma=0.05, amp=1.0, f0=2.0, t0=0.6),
                 extra=dict(probe=((0.7, 0.9),) * 3))
    elif name == "large":
        c = Case(name, 7, (64, 64, 64), (0, 0, 0), (1, 1, 1), (PEC,) * 3, 1000, cfl=CFL,
                 initial=gaussian_pulse_ez((0.5, 0.5, 0.5), 0.05),
                 eps=lambda x, y, z: eps_random(x, y, z, seed=5))
    else:
        raise KeyError(name)
    for k, v in over.items():
        setattr(c, k, v)
    return c


CASES = ("3dboxpec", "3dboxper", "cavity", "planewave", "dielectric", "adjoint", "large")
