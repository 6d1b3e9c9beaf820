"""Host-side mirror of NekCEM's Maxwell time-step interface over the C ABI.

``MaxwellGPU`` plays the part the Fortran driver plays in the reference
(src/cem_drive.F, src/cem_maxwell.F): it hands the static arrays to the
library once, sets the fields, advances them with ``op_rk`` /
``time_advancing`` and evaluates ``cem_error``.  Method names follow the
reference routines.  All arithmetic runs in the CUDA library; this module
only moves numpy arrays across the ABI.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import _lib as L


def _dp(a: np.ndarray):
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError("expected a C-contiguous float64 array")
    return a.ctypes.data_as(L.dp)


def _ip(a: np.ndarray):
    if a.dtype != np.int32 or not a.flags.c_contiguous:
        raise TypeError("expected a C-contiguous int32 array")
    return a.ctypes.data_as(L.ip)


class MaxwellGPU:
    """One GPU context: mesh, materials, fields and the stage kernels."""

    def __init__(self, handle: C.c_void_p, form: int, keep: list):
        self._h = handle
        self.form = form
        self._keep = keep  # arrays the ABI structs point into (kept alive)
        npts, nxzfl = C.c_long(), C.c_long()
        nelt, nx1 = C.c_int(), C.c_int()
        L.check(L.load().nekgpu_sizes(self._h, C.byref(npts), C.byref(nxzfl), C.byref(nelt),
                                      C.byref(nx1)), "nekgpu_sizes")
        self.npts, self.nxzfl, self.nelt, self.nx1 = npts.value, nxzfl.value, nelt.value, nx1.value

    # ---- construction -------------------------------------------------------
    @classmethod
    def from_box(cls, N: int, nel: Sequence[int], lo: Sequence[float], hi: Sequence[float],
                 bc: Sequence[int], form: str = "mixed", permittivity: Optional[np.ndarray] = None,
                 permeability: Optional[np.ndarray] = None, C0: float = 1.0,
                 pml: Optional[Sequence[float]] = None) -> "MaxwellGPU":
        """Structured affine box (genbox + geometry + uservp of the reference).
        bc per axis: 0 PEC, 1 periodic, 2 PML; pml = (thick, order, referr)."""
        lib = L.load()
        b = L.NekgpuBox()
        b.N = int(N)
        b.nelx, b.nely, b.nelz = (int(v) for v in nel)
        for d in range(3):
            b.lo[d] = float(lo[d]); b.hi[d] = float(hi[d]); b.bc[d] = int(bc[d])
        keep = []
        for name, arr in (("permittivity", permittivity), ("permeability", permeability)):
            if arr is not None:
                a = np.ascontiguousarray(arr, dtype=np.float64)
                keep.append(a)
                setattr(b, name, _dp(a))
        b.C0 = float(C0)
        if pml is not None:
            b.pml_thick, b.pml_order, b.pml_referr = int(pml[0]), float(pml[1]), float(pml[2])
        h = C.c_void_p()
        L.check(lib.nekgpu_init_box(C.byref(h), C.byref(b), L.FORMS[form]), "nekgpu_init_box")
        return cls(h, L.FORMS[form], keep)

    @classmethod
    def from_arrays(cls, arrays: dict, nx1: int, nelt: int, form: str = "plain",
                    C0: float = 1.0) -> "MaxwellGPU":
        """Drop-in init from the reference's arrays (as cem_maxwell_init leaves
        them).  ``arrays`` holds the COMMON arrays by their Fortran names;
        ``cemface``/``cempec`` are 0-based here and converted to Fortran's
        1-based convention."""
        m, keep = cls._mesh(arrays, nx1, nelt, C0)
        h = C.c_void_p()
        L.check(L.load().nekgpu_init(C.byref(h), C.byref(m), L.FORMS[form]), "nekgpu_init")
        return cls(h, L.FORMS[form], keep)

    @classmethod
    def from_arrays2d(cls, arrays: dict, nx1: int, nelt: int, mode: int,
                      C0: float = 1.0) -> "MaxwellGPU":
        """2-D TE (mode 1) or TM (mode 2) context from the reference's ldim = 2
        arrays (nekgpu_init2d); z-metric arrays are not read."""
        m, keep = cls._mesh(arrays, nx1, nelt, C0)
        h = C.c_void_p()
        L.check(L.load().nekgpu_init2d(C.byref(h), C.byref(m), int(mode)), "nekgpu_init2d")
        return cls(h, L.FORMS["fused64"], keep)

    @staticmethod
    def _mesh(arrays: dict, nx1: int, nelt: int, C0: float):
        m = L.NekgpuMesh()
        m.nx1, m.nelt = int(nx1), int(nelt)
        keep = []

        def d(name):
            a = np.ascontiguousarray(arrays[name], dtype=np.float64)
            keep.append(a)
            return _dp(a)

        m.dxm1 = d("dxm1"); m.w3mn = d("w3mn")
        for nm in ("rx", "ry", "rz", "sx", "sy", "sz", "tx", "ty", "tz"):
            setattr(m, nm + "mn", d(nm + "mn"))
        m.bmn = d("bmn")
        for nm in ("xmn", "ymn", "zmn"):
            if nm in arrays:
                setattr(m, nm, d(nm))
        m.unxm = d("unxm"); m.unym = d("unym"); m.unzm = d("unzm"); m.aream = d("aream")
        cf = np.ascontiguousarray(np.asarray(arrays["cemface"]) + 1, dtype=np.int32)
        keep.append(cf); m.cemface = _ip(cf)
        gl = np.ascontiguousarray(arrays["glo_face"], dtype=np.int64)
        keep.append(gl); m.glo_face = gl.ctypes.data_as(L.lp)
        pec = np.ascontiguousarray(np.asarray(arrays["cempec"]) + 1, dtype=np.int32)
        keep.append(pec); m.cempec = _ip(pec); m.ncempec = int(pec.size)
        m.Z_0 = d("Z_0"); m.Z_1 = d("Z_1"); m.Y_0 = d("Y_0"); m.Y_1 = d("Y_1")
        m.ebm1 = d("ebm1"); m.hbm1 = d("hbm1")
        m.C0 = float(C0)
        if arrays.get("pmlsigma") is not None:
            m.pmlsigma = d("pmlsigma")
            pp = np.ascontiguousarray(np.asarray(arrays["pmlptr"]) + 1, dtype=np.int32)
            keep.append(pp); m.pmlptr = _ip(pp); m.npml = int(pp.size)
            m.permittivity = d("permittivity"); m.permeability = d("permeability")
        return m, keep

    def close(self):
        if getattr(self, "_h", None):
            L.load().nekgpu_finalize(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- arrays ------------------------------------------------------------
    def array(self, name: str) -> np.ndarray:
        out = np.empty(3 * self.npts if name in ("pmlbn", "pmldn", "pmlsigma") else self.npts)
        L.check(L.load().nekgpu_get_array(self._h, name.encode(), _dp(out)), "nekgpu_get_array")
        return out

    def coords(self):
        return self.array("xmn"), self.array("ymn"), self.array("zmn")

    @property
    def volume(self) -> float:
        return L.load().nekgpu_volume(self._h)

    def set_source_kind(self, kind: int):
        """0: Ricker time function (default); 1: amp * sin(f0 * t)."""
        L.check(L.load().nekgpu_set_source_kind(self._h, int(kind)), "nekgpu_set_source_kind")

    def set_source(self, xc, sigma, amp, f0, t0, enabled: bool = True):
        x = (C.c_double * 3)(*xc)
        L.check(L.load().nekgpu_set_source(self._h, 1 if enabled else 0, x, sigma, amp, f0, t0),
                "nekgpu_set_source")

    # ---- incident field (userinc) and PML auxiliary fields ---------------------
    def set_incident(self, slots, amp, k, omega):
        """userinc plane wave amp * cos(k.x - omega t) on the 0-based face
        slots (amp: H then E)."""
        sl = np.ascontiguousarray(np.asarray(slots) + 1, dtype=np.int32)
        a = (C.c_double * 6)(*amp)
        kk = (C.c_double * 3)(*k)
        self._keep.append(sl)
        L.check(L.load().nekgpu_set_incident(self._h, sl.ctypes.data_as(L.ip), int(sl.size), a, kk,
                                             float(omega)), "nekgpu_set_incident")

    def set_array(self, name: str, values: np.ndarray):
        """"pmlbn" / "pmldn" (3, npts)"""
        v = np.ascontiguousarray(values, dtype=np.float64).reshape(-1)
        L.check(L.load().nekgpu_set_array(self._h, name.encode(), _dp(v)), "nekgpu_set_array")

    # ---- graphene sheets (plain form) -----------------------------------------
    def set_graphene(self, params, slots, yconduc):
        """sheets on the 0-based face slots: params (12, nxzfl), yconduc (nxzfl)"""
        p = np.ascontiguousarray(params, dtype=np.float64).reshape(-1)
        yc = np.ascontiguousarray(yconduc, dtype=np.float64).reshape(-1)
        sl = np.ascontiguousarray(np.asarray(slots) + 1, dtype=np.int32)
        self._keep.extend([p, yc, sl])
        L.check(L.load().nekgpu_set_graphene(self._h, _dp(p), sl.ctypes.data_as(L.ip), int(sl.size),
                                             _dp(yc)), "nekgpu_set_graphene")

    def set_graphene_current(self, fjn):
        """(6, 3, nxzfl) face currents"""
        f = np.ascontiguousarray(fjn, dtype=np.float64).reshape(-1)
        L.check(L.load().nekgpu_set_graphene_current(self._h, _dp(f), self.nxzfl),
                "nekgpu_set_graphene_current")

    def get_graphene_current(self) -> np.ndarray:
        f = np.empty(18 * self.nxzfl)
        L.check(L.load().nekgpu_get_graphene_current(self._h, _dp(f), self.nxzfl),
                "nekgpu_get_graphene_current")
        return f.reshape(6, 3, self.nxzfl)

    # ---- dealiased curl (plain form) ------------------------------------------
    def set_dealias(self, lxd: int, jgl=None, dxmd=None, w3md=None, metd=None):
        """maxwell_wght_dcurl on lxd points per direction with the reference's
        tables (Fortran layouts, flattened); lxd = 0 switches it off."""
        if lxd == 0:
            L.check(L.load().nekgpu_set_dealias(self._h, 0, None, None, None, None),
                    "nekgpu_set_dealias")
            return
        arrs = [np.ascontiguousarray(a, dtype=np.float64).ravel() for a in (jgl, dxmd, w3md, metd)]
        self._keep.extend(arrs)
        L.check(L.load().nekgpu_set_dealias(self._h, int(lxd), *[_dp(a) for a in arrs]),
                "nekgpu_set_dealias")

    # ---- dispersive media (cem_maxwell_drude / cem_maxwell_lorentz) ----------
    DRUDE, LORENTZ = 1, 2

    def set_dispersive(self, model: int, params, index):
        """Polarisation currents at the 0-based nodes ``index``: Drude
        (params (2, npts) = a, b) or Lorentz (params (3, npts) = a, b, c).
        Replaces the model's list and restarts all currents at zero."""
        ncol = 2 if model == self.DRUDE else 3
        index = np.ascontiguousarray(index, dtype=np.int32).reshape(-1) + 1
        n = int(index.size)
        if n:
            params = np.ascontiguousarray(params, dtype=np.float64).reshape(ncol, self.npts)
            pp, ld = _dp(params), self.npts
        else:
            pp, ld = None, self.npts
        L.check(L.load().nekgpu_set_dispersive(self._h, int(model), pp, ld,
                                               index.ctypes.data_as(L.ip), n),
                "nekgpu_set_dispersive")

    def set_current(self, model: int, J):
        nc = 3 if model == self.DRUDE else 6
        J = np.ascontiguousarray(J, dtype=np.float64).reshape(nc, self.npts)
        L.check(L.load().nekgpu_set_current(self._h, int(model), _dp(J), self.npts),
                "nekgpu_set_current")

    def get_current(self, model: int) -> np.ndarray:
        """(3, npts) Drude J or (6, npts) Lorentz J1, J2; zero off the lists"""
        nc = 3 if model == self.DRUDE else 6
        J = np.empty((nc, self.npts))
        L.check(L.load().nekgpu_get_current(self._h, int(model), _dp(J), self.npts),
                "nekgpu_get_current")
        return J

    # ---- fields (Fortran hn(npts,3), en(npts,3) as (3, npts)) --------------
    def set_state(self, H: np.ndarray, E: np.ndarray):
        H = np.ascontiguousarray(H, dtype=np.float64).reshape(3, self.npts)
        E = np.ascontiguousarray(E, dtype=np.float64).reshape(3, self.npts)
        L.check(L.load().nekgpu_set_state(self._h, _dp(H), _dp(E), self.npts), "nekgpu_set_state")

    def get_state(self):
        H = np.empty((3, self.npts)); E = np.empty((3, self.npts))
        L.check(L.load().nekgpu_get_state(self._h, _dp(H), _dp(E), self.npts), "nekgpu_get_state")
        return H, E

    def set_rk_register(self, kH: np.ndarray, kE: np.ndarray):
        kH = np.ascontiguousarray(kH, dtype=np.float64).reshape(3, self.npts)
        kE = np.ascontiguousarray(kE, dtype=np.float64).reshape(3, self.npts)
        L.check(L.load().nekgpu_set_rk_register(self._h, _dp(kH), _dp(kE), self.npts),
                "nekgpu_set_rk_register")

    def get_rk_register(self):
        kH = np.empty((3, self.npts)); kE = np.empty((3, self.npts))
        L.check(L.load().nekgpu_get_rk_register(self._h, _dp(kH), _dp(kE), self.npts),
                "nekgpu_get_rk_register")
        return kH, kE

    # ---- time stepping -------------------------------------------------------
    def stage(self, rkstep: int, time: float, dt: float):
        L.check(L.load().nekgpu_stage(self._h, int(rkstep), float(time), float(dt)), "nekgpu_stage")

    def run(self, nsteps: int, time: float, dt: float) -> float:
        """time_advancing_pde's loop: nsteps of cem_maxwell_op_rk, time += dt each."""
        t = C.c_double(time)
        L.check(L.load().nekgpu_step(self._h, int(nsteps), C.byref(t), float(dt)), "nekgpu_step")
        return t.value

    def op_rk_host(self, H: np.ndarray, E: np.ndarray, time: float, dt: float):
        """One cem_maxwell_op_rk on host fields, updated in place."""
        L.check(L.load().nekgpu_op_rk_host(self._h, _dp(H), _dp(E), self.npts, float(time),
                                           float(dt)), "nekgpu_op_rk_host")

    def time_steps(self, nsteps: int, time: float, dt: float):
        t = C.c_double(time); ms = C.c_double()
        L.check(L.load().nekgpu_time_steps(self._h, int(nsteps), C.byref(t), float(dt),
                                           C.byref(ms)), "nekgpu_time_steps")
        return t.value, ms.value

    def device_bytes(self) -> int:
        return int(L.load().nekgpu_device_bytes(self._h))

    def last_launches(self) -> int:
        return int(L.load().nekgpu_last_launches(self._h))

    def sync(self):
        L.check(L.load().nekgpu_sync(self._h), "nekgpu_sync")

    def register_host(self, arr: np.ndarray):
        L.check(L.load().nekgpu_register_host(self._h, arr.ctypes.data, arr.nbytes),
                "nekgpu_register_host")

    def unregister_host(self, arr: np.ndarray):
        L.check(L.load().nekgpu_unregister_host(self._h, arr.ctypes.data), "nekgpu_unregister_host")

    # ---- the reference routines one by one (plain form) -----------------------
    def call(self, routine: str, *args):
        fn = getattr(L.load(), "nekgpu_" + routine)
        L.check(fn(self._h, *args), "nekgpu_" + routine)

    def work(self, name: str) -> np.ndarray:
        n = {"reshn": 3 * self.npts, "resen": 3 * self.npts, "fhn": 3 * self.nxzfl,
             "fen": 3 * self.nxzfl, "srflx": 6 * self.nxzfl}[name]
        out = np.empty(n)
        L.check(L.load().nekgpu_get_work(self._h, name.encode(), _dp(out)), "nekgpu_get_work")
        return out

    def gs_op_fields(self, u: np.ndarray, nfld: int) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64).copy()
        L.check(L.load().nekgpu_gs_op_fields(self._h, _dp(u), int(nfld)), "nekgpu_gs_op_fields")
        return u

    # ---- norms -----------------------------------------------------------------
    def cem_error(self, Hex: np.ndarray, Eex: np.ndarray):
        """L2 and Linf of exact - numerical for the 6 components (cem_error)."""
        Hex = np.ascontiguousarray(Hex, dtype=np.float64).reshape(3, self.npts)
        Eex = np.ascontiguousarray(Eex, dtype=np.float64).reshape(3, self.npts)
        l2 = np.zeros(6); li = np.zeros(6)
        L.check(L.load().nekgpu_norms(self._h, _dp(Hex), _dp(Eex), self.npts, _dp(l2), _dp(li)),
                "nekgpu_norms")
        return l2, li

    def energy(self) -> float:
        e = C.c_double()
        L.check(L.load().nekgpu_energy(self._h, C.byref(e)), "nekgpu_energy")
        return e.value

    def selftest_wait(self, polls: int = 1000) -> int:
        """status of a kernel whose bounded mbarrier wait runs out on purpose
        (NEKGPU_ERR_TIMEOUT); the context stays usable"""
        return int(L.load().nekgpu_selftest_wait(self._h, int(polls)))

    def check_blowup(self):
        L.check(L.load().nekgpu_check_blowup(self._h), "nekgpu_check_blowup")

    # ---- discrete adjoint (fused FP64 and mixed forms) ----------------------------
    def adjoint_gradient(self, nsteps: int, t0: float, dt: float, jw: np.ndarray, stride: int = 0,
                         host_snapshots: Optional[int] = None,
                         recompute_mixed: Optional[bool] = None):
        """J = sum_g jw[g] |E(g)|^2 after nsteps steps from the current state and
        dJ/deps at every node, by the discrete adjoint (forward steps in the
        context's form, reverse stages in FP64).  ``stride`` > 0: checkpoints
        every stride steps; 0: every ceil(sqrt(nsteps)) steps when that fits
        in device memory, else the binomial schedule; < 0: the binomial
        schedule with -stride device snapshots.  ``host_snapshots``: pinned
        host snapshots the binomial schedule may add (kept for later calls).
        ``recompute_mixed`` (fused FP64 form): the sqrt schedule's segments
        recomputed in mixed stages (kept for later calls).  Leaves the final
        state in the context.  Returns (J, dJdeps, forward_ms, adjoint_ms)."""
        if recompute_mixed is not None:
            L.check(L.load().nekgpu_adjoint_recompute_mixed(self._h, int(bool(recompute_mixed))),
                    "nekgpu_adjoint_recompute_mixed")
        if host_snapshots is not None:
            L.check(L.load().nekgpu_adjoint_host_snapshots(self._h, int(host_snapshots)),
                    "nekgpu_adjoint_host_snapshots")
        jw = np.ascontiguousarray(jw, dtype=np.float64).reshape(self.npts)
        out = np.empty(self.npts)
        J = C.c_double(); fms = C.c_double(); ams = C.c_double()
        L.check(L.load().nekgpu_adjoint_gradient(self._h, int(nsteps), float(t0), float(dt), _dp(jw),
                                                 C.byref(J), _dp(out), int(stride), C.byref(fms),
                                                 C.byref(ams)), "nekgpu_adjoint_gradient")
        return J.value, out, fms.value, ams.value

    def adjoint_init(self, jw: np.ndarray, stride: int = 0):
        """Set the objective weights and checkpoint stride for adjoint_run."""
        jw = np.ascontiguousarray(jw, dtype=np.float64).reshape(self.npts)
        L.check(L.load().nekgpu_adjoint_init(self._h, _dp(jw), int(stride)), "nekgpu_adjoint_init")

    def adjoint_run(self, nsteps: int, t0: float, dt: float):
        """(J, dJ/deps) with the weights of adjoint_init."""
        out = np.empty(self.npts)
        J = C.c_double()
        L.check(L.load().nekgpu_adjoint_run(self._h, int(nsteps), float(t0), float(dt), C.byref(J),
                                            _dp(out)), "nekgpu_adjoint_run")
        return J.value, out

    # ---- output ----------------------------------------------------------------
    def write_vtk(self, path: str, sol: Optional[tuple] = None):
        """The reference's param(81)=3 VTK file of the current state; sol =
        (solH, solE) adds the analytic fields."""
        lib = L.load()
        if sol is None:
            L.check(lib.nekgpu_write_vtk(self._h, str(path).encode(), None, None, 0), "nekgpu_write_vtk")
            return
        sh = np.ascontiguousarray(sol[0], dtype=np.float64).reshape(3, self.npts)
        se = np.ascontiguousarray(sol[1], dtype=np.float64).reshape(3, self.npts)
        L.check(lib.nekgpu_write_vtk(self._h, str(path).encode(), _dp(sh), _dp(se), self.npts),
                "nekgpu_write_vtk")

    def checkpoint_save(self, path: str, time: float, istep: int = 0):
        L.check(L.load().nekgpu_checkpoint_save(self._h, str(path).encode(), float(time), int(istep)),
                "nekgpu_checkpoint_save")

    def checkpoint_load(self, path: str):
        """Returns (time, istep) of the checkpoint."""
        t = C.c_double(); n = C.c_long()
        L.check(L.load().nekgpu_checkpoint_load(self._h, str(path).encode(), C.byref(t), C.byref(n)),
                "nekgpu_checkpoint_load")
        return t.value, n.value
