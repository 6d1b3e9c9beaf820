"""ctypes wrapper around the oracle library (refcpu.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py``.  The product library never loads
it.  ``build()`` compiles ``refcpu.c`` in place with gcc (no FMA contraction,
so x86 and Arm give the same bits).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librefcpu.so")
BC_PEC, BC_PERIODIC, BC_PML = 0, 1, 2


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "refcpu.c")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(os.path.join(HERE, "refcpu.h"))):
        return LIB_PATH
    cmd = ["gcc", "-O3", "-std=c99", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-o", LIB_PATH + ".tmp", src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        vp, ip, dp = C.c_void_p, C.c_int, C.POINTER(C.c_double)
        L.ref_create_box.restype = vp
        L.ref_create_box.argtypes = [ip, ip, ip, ip, dp, dp, C.POINTER(C.c_int)]
        L.ref_create_box_mapped.restype = vp
        L.ref_create_box_mapped.argtypes = [ip, ip, ip, ip, dp, dp, C.POINTER(C.c_int), C.c_double]
        L.ref_destroy.argtypes = [vp]
        L.ref_darray.restype = dp
        L.ref_darray.argtypes = [vp, C.c_char_p, C.POINTER(C.c_long)]
        L.ref_iarray.restype = C.POINTER(C.c_int)
        L.ref_iarray.argtypes = [vp, C.c_char_p, C.POINTER(C.c_long)]
        L.ref_larray.restype = C.POINTER(C.c_longlong)
        L.ref_larray.argtypes = [vp, C.c_char_p, C.POINTER(C.c_long)]
        L.ref_size.restype = C.c_long
        L.ref_size.argtypes = [vp, C.c_char_p]
        L.ref_volvm1.restype = C.c_double
        L.ref_volvm1.argtypes = [vp]
        L.ref_set_materials.argtypes = [vp, dp, dp]
        L.ref_set_flux.argtypes = [vp, C.c_double]
        L.ref_set_source.argtypes = [vp, ip, dp, C.c_double, C.c_double, C.c_double, C.c_double]
        L.ref_set_source_kind.argtypes = [vp, ip]
        L.ref_set_pml.argtypes = [vp, ip, C.c_double, C.c_double]
        L.ref_pml_step.argtypes = [vp]
        L.ref_set_incident.argtypes = [vp, C.POINTER(C.c_int), C.c_long, dp, dp, C.c_double]
        L.ref_set_graphene.argtypes = [vp, dp, C.POINTER(C.c_int), C.c_long]
        L.ref_set_dealias.restype = ip
        L.ref_set_dealias.argtypes = [vp, ip]
        L.ref_create_box2d.restype = vp
        L.ref_create_box2d.argtypes = [ip, ip, ip, dp, dp, C.POINTER(C.c_int), ip]
        L.ref_set_drude.argtypes = [vp, dp, C.POINTER(C.c_int), C.c_long]
        L.ref_set_lorentz.argtypes = [vp, dp, C.POINTER(C.c_int), C.c_long]
        L.ref_source_time.restype = C.c_double
        L.ref_source_time.argtypes = [C.c_double, C.c_double, C.c_double]
        for nm in ("ref_cem_maxwell", "ref_restrict_to_face", "ref_flux3d", "ref_flux_pre",
                   "ref_flux_pec", "ref_flux_upwind", "ref_add_flux_to_res", "ref_invqmass"):
            getattr(L, nm).argtypes = [vp]
        L.ref_usersrc.argtypes = [vp, C.c_double]
        L.ref_maxwell_op.argtypes = [vp, C.c_double]
        L.ref_gs_op_fields.argtypes = [vp, dp, C.c_long, ip]
        L.ref_rk_stage.argtypes = [vp, ip, C.c_double, C.c_double]
        L.ref_op_rk.argtypes = [vp, C.c_double, C.c_double]
        L.ref_run.argtypes = [vp, ip, dp, C.c_double]
        L.ref_get_dxmin.restype = C.c_double
        L.ref_get_dxmin.argtypes = [vp]
        L.ref_cem_error.argtypes = [vp, dp, dp, C.c_long, dp, dp]
        L.ref_rk_coeffs.argtypes = [dp, dp, dp]
        L.ref_zwgll.argtypes = [dp, dp, ip]
        L.ref_dgll.argtypes = [dp, dp, dp, ip]
        L.ref_set_threads.argtypes = [ip]
        L.ref_get_threads.restype = ip
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def zwgll(np_: int):
    z = np.zeros(np_); w = np.zeros(np_)
    lib().ref_zwgll(_dp(z), _dp(w), np_)
    return z, w


def dgll(z: np.ndarray):
    n = len(z)
    d = np.zeros(n * n); dt = np.zeros(n * n)
    lib().ref_dgll(_dp(d), _dp(dt), _dp(np.ascontiguousarray(z, dtype=np.float64)), n)
    return d.reshape(n, n).T.copy(), dt  # D[i, j]


def rk_coeffs():
    a = np.zeros(5); b = np.zeros(5); c = np.zeros(6)
    lib().ref_rk_coeffs(_dp(a), _dp(b), _dp(c))
    return a, b, c


def set_threads(n: int):
    lib().ref_set_threads(int(n))


class RefBox:
    """Oracle for one structured affine box mesh (reference COMMON arrays)."""

    def __init__(self, N, nel, lo, hi, bc, deform: float = 0.0):
        L = lib()
        lo_a = (C.c_double * 3)(*lo); hi_a = (C.c_double * 3)(*hi)
        bc_a = (C.c_int * 3)(*bc)
        if deform:
            self._c = L.ref_create_box_mapped(int(N), int(nel[0]), int(nel[1]), int(nel[2]),
                                              lo_a, hi_a, bc_a, float(deform))
        else:
            self._c = L.ref_create_box(int(N), int(nel[0]), int(nel[1]), int(nel[2]),
                                       lo_a, hi_a, bc_a)
        if not self._c:
            raise ValueError("ref_create_box rejected the mesh")
        self.N, self.nel, self.lo, self.hi, self.bc = N, tuple(nel), tuple(lo), tuple(hi), tuple(bc)
        self.n = N + 1
        self.nelt = int(L.ref_size(self._c, b"nelt"))
        self.npts = int(L.ref_size(self._c, b"npts"))
        self.nxzf = int(L.ref_size(self._c, b"nxzf"))
        self.nxzfl = int(L.ref_size(self._c, b"nxzfl"))

    def close(self):
        if getattr(self, "_c", None):
            lib().ref_destroy(self._c)
            self._c = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- named COMMON arrays as numpy views (they alias the C memory) ---
    def d(self, name: str) -> np.ndarray:
        n = C.c_long(0)
        p = lib().ref_darray(self._c, name.encode(), C.byref(n))
        if not p or n.value == 0:
            raise KeyError(name)
        return np.ctypeslib.as_array(p, shape=(n.value,))

    def i(self, name: str) -> np.ndarray:
        n = C.c_long(0)
        p = lib().ref_iarray(self._c, name.encode(), C.byref(n))
        if not p:
            raise KeyError(name)
        if n.value == 0:
            return np.zeros(0, dtype=np.int32)
        return np.ctypeslib.as_array(p, shape=(n.value,))

    def l(self, name: str) -> np.ndarray:
        n = C.c_long(0)
        p = lib().ref_larray(self._c, name.encode(), C.byref(n))
        if not p:
            raise KeyError(name)
        return np.ctypeslib.as_array(p, shape=(n.value,))

    @property
    def volvm1(self) -> float:
        return lib().ref_volvm1(self._c)

    def set_materials(self, eps: np.ndarray, mu: np.ndarray):
        eps = np.ascontiguousarray(eps, dtype=np.float64)
        mu = np.ascontiguousarray(mu, dtype=np.float64)
        assert eps.size == self.npts and mu.size == self.npts
        lib().ref_set_materials(self._c, _dp(eps), _dp(mu))

    def set_flux(self, C0: float):
        lib().ref_set_flux(self._c, float(C0))

    def set_pml(self, thick: int, order: float, referr: float):
        lib().ref_set_pml(self._c, int(thick), float(order), float(referr))

    def _set_dispersive(self, fn, params, index, ncol):
        params = np.ascontiguousarray(params, dtype=np.float64).reshape(-1)
        assert params.size == ncol * self.npts
        index = np.ascontiguousarray(index, dtype=np.int32)
        assert index.size == 0 or (index.min() >= 0 and index.max() < self.npts)
        fn(self._c, _dp(params), index.ctypes.data_as(C.POINTER(C.c_int)), int(index.size))

    def set_drude(self, a, b, index):
        """Drude current jn at the 0-based nodes ``index`` (cem_maxwell_drude):
        dJ/dt = -a J + b E, resE -= J bm1; a, b per node (npts each)."""
        self._set_dispersive(lib().ref_set_drude, np.stack([a, b]), index, 2)

    def set_lorentz(self, a, b, c, index):
        """Lorentz currents (cem_maxwell_lorentz): dJ1/dt = -a J1 - b J2 + c E,
        dJ2/dt = J1, resE -= J1 bm1."""
        self._set_dispersive(lib().ref_set_lorentz, np.stack([a, b, c]), index, 3)

    @property
    def drude_jn(self):
        """(3, npts) view of the Drude current"""
        return self.d("drudejn").reshape(3, self.npts)

    @property
    def lorentz_jn(self):
        """(6, npts) view of the Lorentz currents: J1 (3 rows) then J2"""
        return self.d("lorentzjn").reshape(6, self.npts)

    def set_incident(self, slots, amp, k, omega):
        """userinc plane wave amp * cos(k.x - omega t) on the 0-based face
        slots (amp: H then E, 6 values)."""
        slots = np.ascontiguousarray(slots, dtype=np.int32)
        a = (C.c_double * 6)(*amp)
        kk = (C.c_double * 3)(*k)
        lib().ref_set_incident(self._c, slots.ctypes.data_as(C.POINTER(C.c_int)), int(slots.size),
                               a, kk, float(omega))

    def set_graphene(self, params, slots):
        """graphene sheets on the 0-based face slots: params (12, nxzfl) in the
        reference's graphparams column order"""
        params = np.ascontiguousarray(params, dtype=np.float64).reshape(-1)
        assert params.size == 12 * self.nxzfl
        slots = np.ascontiguousarray(slots, dtype=np.int32)
        lib().ref_set_graphene(self._c, _dp(params), slots.ctypes.data_as(C.POINTER(C.c_int)),
                               int(slots.size))

    @property
    def fjn(self):
        """(6, 3, nxzfl) view of the face currents fjn(nxzfl,3,6)"""
        return self.d("fjn").reshape(6, 3, self.nxzfl)

    def set_dealias(self, md: int):
        """Dealiased curl on md GLL points per direction (param(18) = -1 with
        lxd = md); 0 returns to the plain weighted curl."""
        if lib().ref_set_dealias(self._c, int(md)) != 0:
            raise ValueError("ref_set_dealias rejected md")

    def set_source_kind(self, kind: int):
        lib().ref_set_source_kind(self._c, int(kind))

    def set_source(self, xc, sigma, amp, f0, t0, enabled=True):
        xa = (C.c_double * 3)(*xc)
        lib().ref_set_source(self._c, 1 if enabled else 0, xa, sigma, amp, f0, t0)

    # state (hn, en) as (3, npts) views
    @property
    def hn(self):
        return self.d("hn").reshape(3, self.npts)

    @property
    def en(self):
        return self.d("en").reshape(3, self.npts)

    def set_state(self, H: np.ndarray, E: np.ndarray, zero_k: bool = True):
        self.hn[...] = H
        self.en[...] = E
        if zero_k:
            self.d("khn")[:] = 0.0
            self.d("ken")[:] = 0.0

    def dxmin(self) -> float:
        return lib().ref_get_dxmin(self._c)

    def stage(self, rkstep: int, time: float, dt: float):
        lib().ref_rk_stage(self._c, int(rkstep), float(time), float(dt))

    def op_rk(self, time: float, dt: float):
        lib().ref_op_rk(self._c, float(time), float(dt))

    def run(self, nsteps: int, time: float, dt: float) -> float:
        t = C.c_double(time)
        lib().ref_run(self._c, int(nsteps), C.byref(t), float(dt))
        return t.value

    def maxwell_op(self, rktime: float):
        lib().ref_maxwell_op(self._c, float(rktime))

    def call(self, name: str, *args):
        return getattr(lib(), "ref_" + name)(self._c, *args)

    def cem_error(self, u: np.ndarray, exact: np.ndarray):
        u = np.ascontiguousarray(u, dtype=np.float64)
        ex = np.ascontiguousarray(exact, dtype=np.float64)
        l2 = C.c_double(); li = C.c_double()
        lib().ref_cem_error(self._c, _dp(u), _dp(ex), u.size, C.byref(l2), C.byref(li))
        return l2.value, li.value

    def coords(self):
        return self.d("xm1"), self.d("ym1"), self.d("zm1")


class RefBox2D(RefBox):
    """Oracle for a 2-D box of quadrilaterals in the TE (mode 1: E1, E2, H3) or
    TM (mode 2: H1, H2, E3) form.  Fields keep the 3-component layout (the
    inactive components stay zero); ``coords()`` gives x, y (z = 0)."""

    def __init__(self, N, nel, lo, hi, bc, mode: int):
        L = lib()
        lo_a = (C.c_double * 2)(*lo); hi_a = (C.c_double * 2)(*hi)
        bc_a = (C.c_int * 2)(*bc)
        self._c = L.ref_create_box2d(int(N), int(nel[0]), int(nel[1]), lo_a, hi_a, bc_a, int(mode))
        if not self._c:
            raise ValueError("ref_create_box2d rejected the mesh")
        self.N, self.nel, self.lo, self.hi, self.bc = N, tuple(nel), tuple(lo), tuple(hi), tuple(bc)
        self.mode = int(mode)
        self.n = N + 1
        self.nelt = int(L.ref_size(self._c, b"nelt"))
        self.npts = int(L.ref_size(self._c, b"npts"))
        self.nxzf = int(L.ref_size(self._c, b"nxzf"))
        self.nxzfl = int(L.ref_size(self._c, b"nxzfl"))

