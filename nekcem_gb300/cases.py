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
