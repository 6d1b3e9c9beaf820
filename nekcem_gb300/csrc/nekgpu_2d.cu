// 2-D TE / TM Maxwell DG stage (the reference's ldim = 2 build, param(4) = 1
// TE or 2 TM) as one kernel per RK stage, in the reference's arithmetic:
// weighted curl with local_grad2 (src/cem_maxwell.F:1500-1536,
// src/nek5_grad.F:21-34) and the TM / TE branches of cem_maxwell
// (src/cem_maxwell.F:584-595), restriction to faces (:616-637),
// cem_maxwell_flux2d with the gs face sum and the PEC mirror (:811-920,
// :1408-1421), the lift in face-slot order (:736-755), the inverse mass
// (:1887-1898) and rk4_upd of the three active components (:1925-1932).
// Compiled without FMA contraction, the same operations in the same order as
// the reference's loops: bit-identical to the FP64 CPU path.
//
// One block per element (at most 16^2 nodes); the partner element's face
// values are read from the stage input, which no block writes.
#include <cuda_runtime.h>

#include "nekgpu_internal.h"

namespace nekgpu {

namespace {

// -n x (the tangential field pair) at a face node: the first loop of
// cem_maxwell_flux2d for TM (E3; H1, H2) and TE (H3; E1, E2)
__device__ __forceinline__ void flux_pre(const Stage2dDev& a, long node, double nx, double ny,
                                         double& s0, double& s1, double& s2) {
  const long P = a.npts;
  if (a.imode == 2) {
    const double e3 = a.u_in[5 * P + node], h1 = a.u_in[node], h2 = a.u_in[P + node];
    s0 = -ny * e3;
    s1 = nx * e3;
    s2 = -nx * h2 + ny * h1;
  } else {
    const double h3 = a.u_in[2 * P + node], e1 = a.u_in[3 * P + node], e2 = a.u_in[4 * P + node];
    s0 = -ny * h3;
    s1 = nx * h3;
    s2 = -nx * e2 + ny * e1;
  }
}

__global__ void k_stage2d(const Stage2dDev a) {
  extern __shared__ double sm[];
  const int n = a.nx, n2 = n * n, nf = 4 * n;
  double* s_u = sm;            // 3 * n2: the active components
  double* s_D = s_u + 3 * n2;  // n2
  double* s_Dt = s_D + n2;     // n2
  double* s_f = s_Dt + n2;     // 3 * nf: face fluxes
  const long P = a.npts;
  const int e = blockIdx.x, tid = threadIdx.x;
  const bool tm = a.imode == 2;
  const int comp[3] = {tm ? 0 : 3, tm ? 1 : 4, tm ? 5 : 2};
  for (int t = tid; t < n2; t += blockDim.x) {
    s_D[t] = a.D[t];
    s_Dt[t] = a.Dt[t];
    const long g = (long)e * n2 + t;
    for (int q = 0; q < 3; ++q) s_u[q * n2 + t] = a.u_in[comp[q] * P + g];
  }
  __syncthreads();

  // ---- weighted curl ---------------------------------------------------------
  const int v = tid;
  const bool node = v < n2;
  double r[3] = {0.0, 0.0, 0.0};
  if (node) {
    const int i = v % n, j = v / n;
    double ur[3], us[3];
    for (int q = 0; q < 3; ++q) {
      const double* u = s_u + q * n2;
      double s = s_D[i] * u[n * j];  // mxm(D, n, u, n, ur, n)
      for (int l = 1; l < n; ++l) s = s + s_D[i + n * l] * u[l + n * j];
      ur[q] = s;
      double t = u[i] * s_Dt[n * j];  // mxm(u, n, Dt, n, us, n)
      for (int l = 1; l < n; ++l) t = t + u[i + n * l] * s_Dt[l + n * j];
      us[q] = t;
    }
    const long k = (long)e * n2 + v;
    const double w = a.w3[v];
    const double u1rw = ur[0] * w, u1sw = us[0] * w;
    const double u2rw = ur[1] * w, u2sw = us[1] * w;
    const double u3rw = ur[2] * w, u3sw = us[2] * w;
    const double rx = a.rx[k], sx = a.sx[k], ry = a.ry[k], sy = a.sy[k];
    const double w1 = (u3rw * ry + u3sw * sy);
    const double w2 = -(u3rw * rx + u3sw * sx);
    const double w3 = (u2rw * rx + u2sw * sx - u1rw * ry - u1sw * sy);
    if (tm) {  // chsign resHN(1,1), resHN(1,2)
      r[0] = -w1;
      r[1] = -w2;
      r[2] = w3;
    } else {  // chsign resHN(1,3)
      r[0] = w1;
      r[1] = w2;
      r[2] = -w3;
    }
  }

  // ---- face fluxes: own + partner (gs add), PEC, upwind ---------------------
  for (int t = tid; t < nf; t += blockDim.x) {
    const long js = (long)e * nf + t;
    const double nx = a.unx[js], ny = a.uny[js];
    double s0, s1, s2;
    flux_pre(a, a.cemface[js], nx, ny, s0, s1, s2);
    const int ps = a.partner[js];
    if (ps >= 0) {
      double p0, p1, p2;
      flux_pre(a, a.cemface[ps], a.unx[ps], a.uny[ps], p0, p1, p2);
      s0 = s0 + p0;
      s1 = s1 + p1;
      s2 = s2 + p2;
    }
    if (a.pec[js]) {
      if (tm) {
        s0 = 2.0 * s0;
        s1 = 2.0 * s1;
        s2 = 0.0;
      } else {
        s0 = 0.0;
        s1 = 0.0;
        s2 = 2.0 * s2;
      }
    }
    const double Y0 = a.Y0[js], Y1 = a.Y1[js], Z0 = a.Z0[js], Z1 = a.Z1[js], C0 = a.C0;
    double o0, o1, o2;
    if (tm) {
      const double fu1 = ny * s2;
      const double fu2 = -nx * s2;
      const double fw3 = nx * s1 - ny * s0;
      o0 = 0.5 / Y0 * (-Y1 * s0 - C0 * fu1);
      o1 = 0.5 / Y0 * (-Y1 * s1 - C0 * fu2);
      o2 = 0.5 / Z0 * (Z1 * s2 - C0 * fw3);
    } else {
      const double fw1 = ny * s2;
      const double fw2 = -nx * s2;
      const double fu3 = nx * s1 - ny * s0;
      o0 = 0.5 / Z0 * (Z1 * s0 - C0 * fw1);
      o1 = 0.5 / Z0 * (Z1 * s1 - C0 * fw2);
      o2 = 0.5 / Y0 * (-Y1 * s2 - C0 * fu3);
    }
    s_f[t] = o0;
    s_f[nf + t] = o1;
    s_f[2 * nf + t] = o2;
  }
  __syncthreads();

  if (!node) return;
  // ---- lift in face-slot order, inverse mass, RK ----------------------------
  const int i = v % n, j = v / n;
  auto add = [&](int f, int aa) {
    const int t = f * n + aa;
    const double ar = a.area[(long)e * nf + t];
    r[0] = r[0] + ar * s_f[t];
    r[1] = r[1] + ar * s_f[nf + t];
    r[2] = r[2] + ar * s_f[2 * nf + t];
  };
  if (j == 0) add(0, i);
  if (i == n - 1) add(1, j);
  if (j == n - 1) add(2, i);
  if (i == 0) add(3, j);
  const long g = (long)e * n2 + v;
  // pml_step after the lift (src/cem_maxwell_pml.F:508-590) on the active
  // components, in the reference's expression order: the auxiliary residual
  // res/bm1 - A aux and the PML term (-A aux + B aux - C u) bm1 added to res.
  // (A, B, C) per component: x (sy, sx, sz), y (sz, sy, sx), z (sx, sz, sy),
  // sigma/eps everywhere except C on E, which is sigma itself.
  const bool pml = a.pml_elem && a.pml_elem[e];
  double pres[3] = {0.0, 0.0, 0.0};
  if (pml) {
    const double bm = a.bm1[g];
    const double bm1inv = 1.0 / bm;
    const double sig[3] = {a.pml_sigma[g], a.pml_sigma[g + P], a.pml_sigma[g + 2 * P]};
    const double ep = a.eps[g];
    const double sp[3] = {sig[0] / ep, sig[1] / ep, sig[2] / ep};
    const double permeab = a.mu[g];
    for (int q = 0; q < 3; ++q) {
      const int c = comp[q], x = c % 3;  // x: the component's axis
      const int ia = x == 0 ? 1 : (x == 1 ? 2 : 0), ib = x, ic = x == 0 ? 2 : (x == 1 ? 0 : 1);
      const double aux = a.pml_aux[(long)c * P + g];
      pres[q] = r[q] * bm1inv - sp[ia] * aux;
      double t;
      if (c < 3)
        t = -sp[ia] * aux + sp[ib] * aux - sp[ic] * permeab * s_u[q * n2 + v];
      else
        t = -sp[ia] * aux + sp[ib] * aux - sig[ic] * s_u[q * n2 + v];
      r[q] = r[q] + t * bm;
    }
  }
  // usersrc after the lift, before the inverse mass (src/cem_maxwell.F:503):
  // the out-of-plane field (E3 in TM, H3 in TE) += bm1-weighted Gaussian x
  // time factor
  if (a.src_w) r[2] = r[2] + a.src_w[g] * a.src_ft;
  const double hb = a.hbm1[g], eb = a.ebm1[g];
  r[0] = r[0] * (tm ? hb : eb);
  r[1] = r[1] * (tm ? hb : eb);
  r[2] = r[2] * (tm ? eb : hb);
  bool active[6] = {false, false, false, false, false, false};
  for (int q = 0; q < 3; ++q) {
    const long o = comp[q] * P + g;
    const double kh = a.ca * a.k[o] + a.dt * r[q];
    a.k[o] = kh;
    a.u_out[o] = s_u[q * n2 + v] + a.cb * kh;
    active[comp[q]] = true;
  }
  for (int c = 0; c < 6; ++c)  // the inactive components carry over
    if (!active[c]) a.u_out[c * P + g] = a.u_in[c * P + g];
  if (pml)  // rk4_upd of the active auxiliary fields (src/cem_maxwell.F:1942-1955)
    for (int q = 0; q < 3; ++q) {
      const long o = comp[q] * P + g;
      const double kk = a.ca * a.pml_k[o] + a.dt * pres[q];
      a.pml_k[o] = kk;
      a.pml_aux[o] = a.pml_aux[o] + a.cb * kk;
    }
}

}  // namespace

int stage2d(Context* c, int rkstep, double time, double dt) {
  Stage2dDev a = c->s2;
  if (a.src_w) a.src_ft = source_ft(c->src, time + dt * c->rk_c[rkstep - 1]);
  a.u_in = c->d_u[c->cur];
  a.u_out = c->d_u[c->cur ^ 1];
  a.k = c->d_k;
  a.ca = c->rk_a[rkstep - 1];
  a.cb = c->rk_b[rkstep - 1];
  a.dt = dt;
  const int n2 = c->nx * c->nx;
  const int nt = ((n2 > 4 * c->nx ? n2 : 4 * c->nx) + 31) / 32 * 32;
  const size_t smem = (5 * (size_t)n2 + 12 * (size_t)c->nx) * sizeof(double);
  k_stage2d<<<c->nelt, nt, smem, c->stream>>>(a);
  c->last_launches += 1;
  int st = check_cuda(cudaGetLastError());
  if (st) return st;
  c->cur ^= 1;
  return NEKGPU_OK;
}

}  // namespace nekgpu
