"""Dealiased curl (param(18) = -1: maxwell_wght_dcurl,
src/cem_maxwell.F:1541-1729): the fields are interpolated to md GLL points per
direction (gen_int with Fornberg's weights, fd_weights_full), differentiated
there (gen_dgl), combined with the interpolated metrics and projected back
with the transposed interpolation (intp_rstd backward).

CPU: the oracle's tables against independent formulas (Lagrange
interpolation, the GLL derivative matrix at md points); the oracle's dealiased
curl against a numpy restatement of the same operator; md = nx1 reduces to
the plain weighted curl.  GPU: the plain form's k_dcurl matches the oracle
bit for bit on curved meshes; the fused FP64 form with the dealiased curl
matches it to 1e-12 per step; the forms on affine meshes refuse it.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import gpu_from_ref, make_ref, smooth_fields
from nekcem_gb300 import _lib as L
from oracle import refcpu as R


def lagrange_matrix(zf, zc):
    """J[i, j] = l_j(zf[i]) for the Lagrange basis on zc"""
    J = np.ones((len(zf), len(zc)))
    for j in range(len(zc)):
        for m in range(len(zc)):
            if m != j:
                J[:, j] *= (zf - zc[m]) / (zc[j] - zc[m])
    return J


@pytest.mark.parametrize("N,md", [(3, 5), (5, 9), (7, 12)])
def test_dealias_tables(N, md):
    ref = make_ref(N, (1, 1, 1), (0, 0, 0), (1, 1, 1), (0, 0, 0))
    ref.set_dealias(md)
    mx = N + 1
    zc, _ = R.zwgll(mx)
    zf, wf = R.zwgll(md)
    jgl = ref.d("jgl").reshape(mx, md).T  # Fortran jgl(md, mx)
    np.testing.assert_allclose(jgl, lagrange_matrix(zf, zc), rtol=0, atol=1e-13)
    dxmd = ref.d("dxmd").reshape(md, md).T
    np.testing.assert_allclose(dxmd, R.dgll(zf)[0], rtol=0, atol=1e-11 * md * md)
    w3 = ref.d("w3md").reshape(md, md, md)
    np.testing.assert_allclose(w3, np.einsum("k,j,i->kji", wf, wf, wf), rtol=1e-15)
    ref.close()


def numpy_dcurl(ref, md, u1, u2, u3):
    """The same operator with numpy tensor contractions (element by element)"""
    mx, ne = ref.n, ref.nelt
    J = ref.d("jgl").reshape(mx, md).T
    D = ref.d("dxmd").reshape(md, md).T
    w3 = ref.d("w3md").reshape(md, md, md)
    met = ref.d("metd").reshape(9, ne, md, md, md)
    out = [np.zeros(ref.npts) for _ in range(3)]
    fwd = lambda u: np.einsum("ai,bj,ck,kji->cba", J, J, J, u)
    bwd = lambda w: np.einsum("ai,bj,ck,cba->kji", J, J, J, w)
    for e in range(ne):
        sl = slice(e * mx ** 3, (e + 1) * mx ** 3)
        g = []
        for u in (u1, u2, u3):
            f = fwd(u[sl].reshape(mx, mx, mx))
            g.append((np.einsum("il,kjl->kji", D, f) * w3, np.einsum("jl,kli->kji", D, f) * w3,
                      np.einsum("kl,lji->kji", D, f) * w3))
        rx, ry, rz, sx, sy, sz, tx, ty, tz = met[:, e]
        (u1r, u1s, u1t), (u2r, u2s, u2t), (u3r, u3s, u3t) = g
        wd1 = u3r * ry + u3s * sy + u3t * ty - u2r * rz - u2s * sz - u2t * tz
        wd2 = u1r * rz + u1s * sz + u1t * tz - u3r * rx - u3s * sx - u3t * tx
        wd3 = u2r * rx + u2s * sx + u2t * tx - u1r * ry - u1s * sy - u1t * ty
        for q, w in enumerate((wd1, wd2, wd3)):
            out[q][sl] = bwd(w).ravel()
    return np.stack(out)


@pytest.mark.parametrize("md", [6, 9])
def test_oracle_dcurl_matches_numpy(md):
    ref = make_ref(5, (2, 1, 2), (0, 0, 0), (1, 1, 1), (0, 0, 0), deform=0.06)
    ref.set_dealias(md)
    H, E = smooth_fields(ref, 4)
    ref.set_state(H, E)
    ref.call("cem_maxwell")
    got = ref.d("resen").reshape(3, -1).copy()
    want = numpy_dcurl(ref, md, H[0], H[1], H[2])
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-11 * np.abs(want).max())
    ref.close()


def test_dealias_on_nx1_points_is_the_plain_curl():
    ref = make_ref(5, (2, 2, 2), (0, 0, 0), (1, 1, 1), (0, 0, 0), deform=0.05)
    H, E = smooth_fields(ref, 3)
    ref.set_state(H, E)
    ref.call("cem_maxwell")
    r0 = np.concatenate([ref.d("reshn"), ref.d("resen")])
    ref.set_dealias(6)
    ref.call("cem_maxwell")
    r1 = np.concatenate([ref.d("reshn"), ref.d("resen")])
    np.testing.assert_allclose(r1, r0, rtol=0, atol=1e-14 * np.abs(r0).max())
    with pytest.raises(ValueError):
        ref.set_dealias(5)  # fewer points than nx1
    ref.close()


@pytest.mark.gpu
@pytest.mark.parametrize("N,md,bc,deform", [(4, 6, (0, 0, 0), 0.05), (5, 9, (1, 0, 1), 0.08),
                                          (7, 12, (1, 1, 1), 0.04)])
def test_plain_dcurl_bit_exact(N, md, bc, deform):
    ref = make_ref(N, (2, 2, 2), (0, 0, 0), (1, 1, 1), bc, deform=deform,
                   eps=lambda x, y, z: 1.0 + 0.5 * np.sin(2 * x) ** 2)
    ref.set_dealias(md)
    g = gpu_from_ref(ref, "plain")
    g.set_dealias(md, ref.d("jgl"), ref.d("dxmd"), ref.d("w3md"), ref.d("metd"))
    H, E = smooth_fields(ref, 7)
    ref.set_state(H, E); g.set_state(H, E)
    dt = 0.2 * ref.dxmin()
    ref.run(3, 0.0, dt); g.run(3, 0.0, dt)
    gH, gE = g.get_state()
    np.testing.assert_array_equal(gH, ref.hn)
    np.testing.assert_array_equal(gE, ref.en)
    g.close(); ref.close()


@pytest.mark.gpu
@pytest.mark.parametrize("N,md,bc,deform", [(4, 6, (0, 0, 0), 0.05), (5, 9, (1, 0, 1), 0.08),
                                          (7, 12, (1, 1, 1), 0.04)])
def test_fused64_dcurl_per_step(N, md, bc, deform):
    """The fused FP64 form on curved meshes with the dealiased curl (its
    volume term from k_dcurl, then flux, lift, source, inverse mass and RK in
    the curved stage kernel): three steps, each from the oracle's state,
    within 1e-12 relative, with the Gaussian/Ricker source on."""
    ref = make_ref(N, (2, 2, 2), (0, 0, 0), (1, 1, 1), bc, deform=deform,
                   eps=lambda x, y, z: 1.0 + 0.5 * np.sin(2 * x) ** 2)
    ref.set_dealias(md)
    src = dict(xc=(0.4, 0.5, 0.55), sigma=0.2, amp=1.0, f0=2.0, t0=0.05)
    ref.set_source(**src)
    g = gpu_from_ref(ref, "fused64")
    g.set_dealias(md, ref.d("jgl"), ref.d("dxmd"), ref.d("w3md"), ref.d("metd"))
    g.set_source(**src)
    H, E = smooth_fields(ref, 9)
    dt = 0.2 * ref.dxmin()
    t = 0.0
    for step in range(3):
        ref.set_state(H, E); g.set_state(H, E)
        ref.op_rk(t, dt)
        g.run(1, t, dt)
        gH, gE = g.get_state()
        a = np.concatenate([gH, gE]); b = np.concatenate([ref.hn, ref.en])
        err = np.abs(a - b).max() / np.abs(b).max()
        assert err <= 1e-12, (step, err)
        H, E = ref.hn.copy(), ref.en.copy()
        t += dt
    g.close(); ref.close()


@pytest.mark.gpu
def test_dealias_refusals():
    ref = make_ref(4, (2, 2, 2), (0, 0, 0), (1, 1, 1), (0, 0, 0), deform=0.05)
    ref.set_dealias(6)
    tabs = (ref.d("jgl"), ref.d("dxmd"), ref.d("w3md"), ref.d("metd"))
    flat = make_ref(4, (2, 2, 2), (0, 0, 0), (1, 1, 1), (0, 0, 0))
    flat.set_dealias(6)
    ftabs = (flat.d("jgl"), flat.d("dxmd"), flat.d("w3md"), flat.d("metd"))
    for form in ("fused64", "mixed"):  # affine meshes: the compact fused kernels
        g = gpu_from_ref(flat, form)
        with pytest.raises(L.NekgpuError) as e:
            g.set_dealias(6, *ftabs)
        assert e.value.status == -8
        g.close()
    flat.close()
    g = gpu_from_ref(ref, "plain")
    with pytest.raises(L.NekgpuError) as e:
        g.set_dealias(4, *tabs)  # fewer points than nx1
    assert e.value.status == -1
    g.set_dealias(6, *tabs)
    g.set_dealias(0)  # back to the plain curl
    H, E = smooth_fields(ref, 2)
    ref.set_dealias(0)
    ref.set_state(H, E); g.set_state(H, E)
    ref.run(2, 0.0, 1e-3); g.run(2, 0.0, 1e-3)
    np.testing.assert_array_equal(g.get_state()[1], ref.en)
    g.close(); ref.close()

