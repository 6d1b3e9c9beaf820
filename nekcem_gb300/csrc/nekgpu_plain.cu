// Plain form: one all-FP64 kernel per reference routine of the Maxwell stage.
//
// This translation unit is compiled with --fmad=false: every product and sum
// is rounded separately, in the reference's order, so that on the reference's
// own arrays the results are bit-identical to an unfused CPU evaluation
// (Fortran without FMA contraction).  It works on the reference's general
// per-node metric / per-face-node arrays, i.e. any conforming hex mesh.
#include <cuda_runtime.h>

#include "nekgpu_internal.h"

namespace nekgpu {

namespace {

constexpr int kThreads = 256;

inline int blocks_for(long n, int t = kThreads) {
  long b = (n + t - 1) / t;
  return (int)(b < 1 ? 1 : b);
}

// maxwell_wght_curl (src/cem_maxwell.F:1428-1497) with local_grad3
// (src/nek5_grad.F:2-19) and the mxf summation order (src/nek5_mxm_std.F:173-191),
// applied to H (-> resE) and E (-> resH, negated as chsign does,
// src/cem_maxwell.F:580-582).  One CTA per element; field blocks in smem.
__global__ void k_curl(PlainDev a) {
  extern __shared__ double sm[];
  const int n = a.nx;
  const int n2 = n * n, n3 = n2 * n;
  double* su = sm;           // 3*n3
  double* sD = sm + 3 * n3;  // n2  D(i,l) at [i + n*l]
  double* sDt = sD + n2;     // n2  Dt(l,j) at [l + n*j]
  const int e = blockIdx.x;
  for (int t = threadIdx.x; t < n2; t += blockDim.x) {
    sD[t] = a.dxm1[t];
    sDt[t] = a.dxtm1[t];
  }
  for (int fld = 0; fld < 2; ++fld) {
    // fld 0: u = H (comps 0..2) -> resE (3..5); fld 1: u = E -> resH (0..2), negated
    const int uin = fld == 0 ? 0 : 3, wout = fld == 0 ? 3 : 0;
    __syncthreads();
    for (int t = threadIdx.x; t < 3 * n3; t += blockDim.x) {
      int q = t / n3, v = t - q * n3;
      su[t] = a.u[(long)(uin + q) * a.npts + (long)e * n3 + v];
    }
    __syncthreads();
    for (int v = threadIdx.x; v < n3; v += blockDim.x) {
      const int i = v % n, j = (v / n) % n, k = v / n2;
      double g[3][3];  // g[q][0..2] = d u_q / d(r,s,t)
      for (int q = 0; q < 3; ++q) {
        const double* u = su + q * n3;
        // ur(i,jk) = sum_l D(i,l) u(l,jk)
        double s = sD[i] * u[j * n + k * n2];
        for (int l = 1; l < n; ++l) s = s + sD[i + n * l] * u[l + j * n + k * n2];
        g[q][0] = s;
        // us(i,j,k) = sum_l u(i,l,k) Dt(l,j)
        s = u[i + k * n2] * sDt[n * j];
        for (int l = 1; l < n; ++l) s = s + u[i + n * l + k * n2] * sDt[l + n * j];
        g[q][1] = s;
        // ut(ij,k) = sum_l u(ij,l) Dt(l,k)
        s = u[i + n * j] * sDt[n * k];
        for (int l = 1; l < n; ++l) s = s + u[i + n * j + n2 * l] * sDt[l + n * k];
        g[q][2] = s;
      }
      const long gk = (long)e * n3 + v;
      const double w = a.w3[v];
      const double u1rw = g[0][0] * w, u1sw = g[0][1] * w, u1tw = g[0][2] * w;
      const double u2rw = g[1][0] * w, u2sw = g[1][1] * w, u2tw = g[1][2] * w;
      const double u3rw = g[2][0] * w, u3sw = g[2][1] * w, u3tw = g[2][2] * w;
      const double* M = a.metrics;
      const long P = a.npts;
      const double rx = M[0 * P + gk], ry = M[1 * P + gk], rz = M[2 * P + gk];
      const double sx = M[3 * P + gk], sy = M[4 * P + gk], sz = M[5 * P + gk];
      const double tx = M[6 * P + gk], ty = M[7 * P + gk], tz = M[8 * P + gk];
      double w1 = u3rw * ry + u3sw * sy + u3tw * ty - u2rw * rz - u2sw * sz - u2tw * tz;
      double w2 = u1rw * rz + u1sw * sz + u1tw * tz - u3rw * rx - u3sw * sx - u3tw * tx;
      double w3 = u2rw * rx + u2sw * sx + u2tw * tx - u1rw * ry - u1sw * sy - u1tw * ty;
      if (fld == 1) { w1 = -w1; w2 = -w2; w3 = -w3; }
      a.res[(long)(wout + 0) * P + gk] = w1;
      a.res[(long)(wout + 1) * P + gk] = w2;
      a.res[(long)(wout + 2) * P + gk] = w3;
    }
  }
}

// mxm (src/nek5_mxm_std.F:173-191) on shared-memory operands by the whole
// block: c(i,j) = sum_l a(i,l) b(l,j), l ascending, a n1 x n2, b n2 x n3
__device__ __forceinline__ void block_mxm(const double* A, int n1, const double* B, int n2,
                                          double* Cm, int n3) {
  for (int t = threadIdx.x; t < n1 * n3; t += blockDim.x) {
    const int i = t % n1, j = t / n1;
    double s = A[i] * B[n2 * j];
    for (int l = 1; l < n2; ++l) s = s + A[i + n1 * l] * B[l + n2 * j];
    Cm[t] = s;
  }
}

// maxwell_wght_dcurl (src/cem_maxwell.F:1541-1729): per element, each field
// interpolated to md^3 points (intp_rstd forward = specmpn with jgl, jgt,
// src/cem_common.F:418-460, 507-538), local_grad3 there with dxmd, the
// weighted curl with the interpolated metrics, and the projection back
// (intp_rstd backward: specmpn with jgt, jgl).  H -> resE, E -> resH
// (negated, chsign).  One CTA per element, every array in shared memory.
__global__ void k_dcurl(PlainDev a) {
  extern __shared__ double sm[];
  const int mx = a.nx, md = a.md;
  const int mx2 = mx * mx, mx3 = mx2 * mx, md2 = md * md, md3 = md2 * md;
  double* s_jgl = sm;                 // md x mx
  double* s_jgt = s_jgl + md * mx;    // mx x md
  double* s_D = s_jgt + md * mx;      // md x md
  double* s_Dt = s_D + md2;           // md x md
  double* s_w3 = s_Dt + md2;          // md^3
  double* s_ju = s_w3 + md3;          // 3 md^3
  double* s_wd = s_ju + 3 * md3;      // 3 md^3
  double* s_t1 = s_wd + 3 * md3;      // max(md mx^2, mx md^2)
  double* s_t2 = s_t1 + md2 * mx;     // max(md^2 mx, mx^2 md)
  double* s_u = s_t2 + md2 * mx;      // mx^3
  const int e = blockIdx.x;
  const long P = a.npts;
  for (int t = threadIdx.x; t < md * mx; t += blockDim.x) {
    s_jgl[t] = a.jgl[t];
    s_jgt[t] = a.jgt[t];
  }
  for (int t = threadIdx.x; t < md2; t += blockDim.x) {
    s_D[t] = a.dxmd[t];
    s_Dt[t] = a.dxtmd[t];
  }
  for (int t = threadIdx.x; t < md3; t += blockDim.x) s_w3[t] = a.w3md[t];
  for (int fld = 0; fld < 2; ++fld) {
    const int uin = fld == 0 ? 0 : 3, wout = fld == 0 ? 3 : 0;
    // ---- forward interpolation of the three components ----------------------
    for (int q = 0; q < 3; ++q) {
      __syncthreads();
      for (int t = threadIdx.x; t < mx3; t += blockDim.x)
        s_u[t] = a.u[(long)(uin + q) * P + (long)e * mx3 + t];
      __syncthreads();
      block_mxm(s_jgl, md, s_u, mx, s_t1, mx2);
      __syncthreads();
      for (int iz = 0; iz < mx; ++iz) block_mxm(s_t1 + md * mx * iz, md, s_jgt, mx, s_t2 + md2 * iz, md);
      __syncthreads();
      block_mxm(s_t2, md2, s_jgt, mx, s_ju + q * md3, md);
    }
    __syncthreads();
    // ---- derivatives and the weighted curl on the md^3 points -----------------
    for (int v = threadIdx.x; v < md3; v += blockDim.x) {
      const int i = v % md, j = (v / md) % md, k = v / md2;
      double g[3][3];
      for (int q = 0; q < 3; ++q) {
        const double* u = s_ju + q * md3;
        double s = s_D[i] * u[md * j + md2 * k];
        for (int l = 1; l < md; ++l) s = s + s_D[i + md * l] * u[l + md * j + md2 * k];
        g[q][0] = s;
        s = u[i + md2 * k] * s_Dt[md * j];
        for (int l = 1; l < md; ++l) s = s + u[i + md * l + md2 * k] * s_Dt[l + md * j];
        g[q][1] = s;
        s = u[i + md * j] * s_Dt[md * k];
        for (int l = 1; l < md; ++l) s = s + u[i + md * j + md2 * l] * s_Dt[l + md * k];
        g[q][2] = s;
      }
      const double w = s_w3[v];
      const double u1rw = g[0][0] * w, u1sw = g[0][1] * w, u1tw = g[0][2] * w;
      const double u2rw = g[1][0] * w, u2sw = g[1][1] * w, u2tw = g[1][2] * w;
      const double u3rw = g[2][0] * w, u3sw = g[2][1] * w, u3tw = g[2][2] * w;
      const long nm = (long)md3 * a.nelt, k0 = (long)e * md3 + v;
      const double* M = a.metd;
      const double rx = M[k0], ry = M[nm + k0], rz = M[2 * nm + k0];
      const double sx = M[3 * nm + k0], sy = M[4 * nm + k0], sz = M[5 * nm + k0];
      const double tx = M[6 * nm + k0], ty = M[7 * nm + k0], tz = M[8 * nm + k0];
      s_wd[v] = u3rw * ry + u3sw * sy + u3tw * ty - u2rw * rz - u2sw * sz - u2tw * tz;
      s_wd[md3 + v] = u1rw * rz + u1sw * sz + u1tw * tz - u3rw * rx - u3sw * sx - u3tw * tx;
      s_wd[2 * md3 + v] = u2rw * rx + u2sw * sx + u2tw * tx - u1rw * ry - u1sw * sy - u1tw * ty;
    }
    // ---- projection back to the nx1^3 points ------------------------------------
    for (int q = 0; q < 3; ++q) {
      __syncthreads();
      block_mxm(s_jgt, mx, s_wd + q * md3, md, s_t1, md2);
      __syncthreads();
      for (int iz = 0; iz < md; ++iz) block_mxm(s_t1 + mx * md * iz, mx, s_jgl, md, s_t2 + mx2 * iz, mx);
      __syncthreads();
      for (int t = threadIdx.x; t < mx3; t += blockDim.x) {
        const int ij = t % mx2, kk = t / mx2;
        double s = s_t2[ij] * s_jgl[md * kk];
        for (int l = 1; l < md; ++l) s = s + s_t2[ij + mx2 * l] * s_jgl[l + md * kk];
        a.res[(long)(wout + q) * P + (long)e * mx3 + t] = fld == 1 ? -s : s;
      }
    }
  }
}

// cem_maxwell_restrict_to_face (src/cem_maxwell.F:604-623)
__global__ void k_restrict(PlainDev a) {
  long j = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (j >= a.nxzfl) return;
  long i = a.cemface[j];
  for (int q = 0; q < 6; ++q) a.fface[q * a.nxzfl + j] = a.u[q * a.npts + i];
}

// first loop of cem_maxwell_flux3d (src/cem_maxwell.F:944-955): -n x E, -n x H
__global__ void k_flux_pre(PlainDev a) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long k = a.nxzfl;
  if (i >= k) return;
  const double nx = a.unx[i], ny = a.uny[i], nz = a.unz[i];
  const double* fh = a.fface;
  const double* fe = a.fface + 3 * k;
  double* s = a.srflx;
  s[0 * k + i] = -ny * fe[2 * k + i] + nz * fe[1 * k + i];
  s[1 * k + i] = -nz * fe[0 * k + i] + nx * fe[2 * k + i];
  s[2 * k + i] = -nx * fe[1 * k + i] + ny * fe[0 * k + i];
  s[3 * k + i] = -ny * fh[2 * k + i] + nz * fh[1 * k + i];
  s[4 * k + i] = -nz * fh[0 * k + i] + nx * fh[2 * k + i];
  s[5 * k + i] = -nx * fh[1 * k + i] + ny * fh[0 * k + i];
}

// gs_op_fields(gsh_face, u, stride, nfld, 1, add, 0) on single-rank face ids
// (src/jl/gs.c:2074-2099): each id group is a pair (or a singleton, left
// alone); both members receive the same sum.
__global__ void k_gs_pairs(const int* pairs, int npairs, double* u, long stride, int nfld) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npairs) return;
  const int j0 = pairs[2 * p], j1 = pairs[2 * p + 1];
  for (int q = 0; q < nfld; ++q) {
    double* v = u + q * stride;
    const double s = v[j0] + v[j1];
    v[j0] = s;
    v[j1] = s;
  }
}

// cem_maxwell_flux_pec (src/cem_maxwell.F:1368-1426)
__global__ void k_flux_pec(PlainDev a) {
  int jj = blockIdx.x * blockDim.x + threadIdx.x;
  if (jj >= a.ncempec) return;
  const long k = a.nxzfl, i = a.cempec[jj];
  double* s = a.srflx;
  s[0 * k + i] = 2.0 * s[0 * k + i];
  s[1 * k + i] = 2.0 * s[1 * k + i];
  s[2 * k + i] = 2.0 * s[2 * k + i];
  s[3 * k + i] = 0.0;
  s[4 * k + i] = 0.0;
  s[5 * k + i] = 0.0;
}

// upwind combination (src/cem_maxwell.F:969-997)
__global__ void k_flux_upwind(PlainDev a) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long k = a.nxzfl;
  if (i >= k) return;
  double* s = a.srflx;
  const double Y0 = a.Y0[i], Y1 = a.Y1[i], Z0 = a.Z0[i], Z1 = a.Z1[i];
  const double Y02 = -0.5 / Y0 * Y1;
  const double Z02 = 0.5 / Z0 * Z1;
  const double C02Y = 0.5 / Y0 * a.C0;
  const double C02Z = 0.5 / Z0 * a.C0;
  const double nx = a.unx[i], ny = a.uny[i], nz = a.unz[i];
  const double s0 = s[0 * k + i], s1 = s[1 * k + i], s2 = s[2 * k + i];
  const double s3 = s[3 * k + i], s4 = s[4 * k + i], s5 = s[5 * k + i];
  const double fu1 = ny * s5 - nz * s4;
  const double fu2 = nz * s3 - nx * s5;
  const double fu3 = nx * s4 - ny * s3;
  const double fw1 = ny * s2 - nz * s1;
  const double fw2 = nz * s0 - nx * s2;
  const double fw3 = nx * s1 - ny * s0;
  s[0 * k + i] = Y02 * s0 - C02Y * fu1;
  s[1 * k + i] = Y02 * s1 - C02Y * fu2;
  s[2 * k + i] = Y02 * s2 - C02Y * fu3;
  s[3 * k + i] = Z02 * s3 - C02Z * fw1;
  s[4 * k + i] = Z02 * s4 - C02Z * fw2;
  s[5 * k + i] = Z02 * s5 - C02Z * fw3;
}

// cem_maxwell_add_flux_to_res (src/cem_maxwell.F:725-735).  The reference's
// serial loop adds face slots in increasing order; here each volume node
// gathers its slots (CSR, ascending) so the per-node order is the same and
// no two threads write one node (the OpenACC variant's cemface_ptr idea,
// src/cem_common.F:262-275).
__global__ void k_lift(PlainDev a) {
  long v = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (v >= a.npts) return;
  const int b = a.lift_ptr[v], e = a.lift_ptr[v + 1];
  if (b == e) return;
  const long k = a.nxzfl, P = a.npts;
  double r[6];
  for (int q = 0; q < 6; ++q) r[q] = a.res[q * P + v];
  for (int t = b; t < e; ++t) {
    const long j = a.lift_slot[t];
    const double ar = a.area[j];
    for (int q = 0; q < 6; ++q) r[q] = r[q] + ar * a.srflx[q * k + j];
  }
  for (int q = 0; q < 6; ++q) a.res[q * P + v] = r[q];
}

// usersrc for the Gaussian E_z source (src/cem_maxwell.F:503)
__global__ void k_usersrc(PlainDev a, double ft) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= a.npts) return;
  double* rez = a.res + 5 * a.npts;
  rez[i] = rez[i] + a.src_w[i] * ft;
}

// cem_maxwell_invqmass (src/cem_maxwell.F:1878-1886)
__global__ void k_invqmass(PlainDev a) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= a.npts) return;
  const long P = a.npts;
  const double hb = a.hbm1[i], eb = a.ebm1[i];
  for (int q = 0; q < 3; ++q) a.res[q * P + i] = a.res[q * P + i] * hb;
  for (int q = 3; q < 6; ++q) a.res[q * P + i] = a.res[q * P + i] * eb;
}

// rk_maxwell_ab -> rk4_upd (src/cem_maxwell.F:1906-1940, src/cem_common.F:18-75)
__global__ void k_rk(PlainDev a, double ca, double cb, double dt) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= 6 * a.npts) return;
  const double kh = ca * a.k[i] + dt * a.res[i];
  a.k[i] = kh;
  a.u[i] = a.u[i] + cb * kh;
}

// pml_step (src/cem_maxwell_pml.F:508-590): one thread per node of a PML
// element; the auxiliary residuals, then their contribution to res
__global__ void k_pml_step(PlainDev a, int n3) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= (long)a.npml * n3) return;
  const long P = a.npts;
  const long j = (long)a.pmlptr[t / n3] * n3 + t % n3;
  const double* sg = a.pmlsigma;
  const double* bn = a.pmlaux;
  const double* dn = a.pmlaux + 3 * P;
  double* rb = a.pmlres;
  double* rd = a.pmlres + 3 * P;
  double* rh = a.pmlres + 6 * P;
  double* re = a.pmlres + 9 * P;
  const double* hn = a.u;
  const double* en = a.u + 3 * P;
  double* rsh = a.res;
  double* rse = a.res + 3 * P;
  const double bm1inv = 1.0 / a.bm1[j];
  const double sigx = sg[j], sigy = sg[j + P], sigz = sg[j + 2 * P];
  const double sxp = sigx / a.eps[j], syp = sigy / a.eps[j], szp = sigz / a.eps[j];
  const double permeab = a.mu[j];
  rb[j] = rsh[j] * bm1inv - syp * bn[j];
  rb[j + P] = rsh[j + P] * bm1inv - szp * bn[j + P];
  rb[j + 2 * P] = rsh[j + 2 * P] * bm1inv - sxp * bn[j + 2 * P];
  rd[j] = rse[j] * bm1inv - syp * dn[j];
  rd[j + P] = rse[j + P] * bm1inv - szp * dn[j + P];
  rd[j + 2 * P] = rse[j + 2 * P] * bm1inv - sxp * dn[j + 2 * P];
  rh[j] = -syp * bn[j] + sxp * bn[j] - szp * permeab * hn[j];
  rh[j + P] = -szp * bn[j + P] + syp * bn[j + P] - sxp * permeab * hn[j + P];
  rh[j + 2 * P] = -sxp * bn[j + 2 * P] + szp * bn[j + 2 * P] - syp * permeab * hn[j + 2 * P];
  re[j] = -syp * dn[j] + sxp * dn[j] - sigz * en[j];
  re[j + P] = -szp * dn[j + P] + syp * dn[j + P] - sigx * en[j + P];
  re[j + 2 * P] = -sxp * dn[j + 2 * P] + szp * dn[j + 2 * P] - sigy * en[j + 2 * P];
  const double b = a.bm1[j];
  rsh[j] = rsh[j] + rh[j] * b;
  rsh[j + P] = rsh[j + P] + rh[j + P] * b;
  rsh[j + 2 * P] = rsh[j + 2 * P] + rh[j + 2 * P] * b;
  rse[j] = rse[j] + re[j] * b;
  rse[j + P] = rse[j + P] + re[j + P] * b;
  rse[j + 2 * P] = rse[j + 2 * P] + re[j + 2 * P] * b;
}

// rk4_upd of the PML auxiliary fields (src/cem_maxwell.F:1942-1955)
__global__ void k_pml_rk(PlainDev a, double ca, double cb, double dt) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= 6 * a.npts) return;
  const double kh = ca * a.pmlk[i] + dt * a.pmlres[i];
  a.pmlk[i] = kh;
  a.pmlaux[i] = a.pmlaux[i] + cb * kh;
}

// cem_maxwell_drude (src/cem_maxwell.F:3095-3147) and cem_maxwell_lorentz
// (:3149-3212) at one node of an element holding listed nodes, followed by
// the rk4_upd of its currents; unlisted nodes (kind 0) are left alone, as the
// reference's rk4_upd leaves a zero current with a zero residual.
__global__ void k_dispersive(PlainDev a, int n3, double ca, double cb, double dt) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const DispDev& d = a.disp;
  if (t >= d.n) return;
  const long nn = d.n, P = a.npts;
  const int kind = (int)d.data[t];
  if (kind == 0) return;
  const long j = (long)d.elem[t / n3] * n3 + t % n3;
  const double pa = d.data[nn + t], pb = d.data[2 * nn + t], pc = d.data[3 * nn + t];
  const double bm1 = d.data[4 * nn + t];
  const double* en = a.u + 3 * P;
  double* rse = a.res + 3 * P;
  for (int q = 0; q < 3; ++q) {
    const double j1 = d.aux[q * nn + t];
    rse[j + q * P] = rse[j + q * P] - j1 * bm1;
    if (kind == 1) {
      const double r = -pa * j1 + pb * en[j + q * P];
      const double kh = ca * d.k[q * nn + t] + dt * r;
      d.k[q * nn + t] = kh;
      d.aux[q * nn + t] = j1 + cb * kh;
    } else {
      const double j2 = d.aux[(3 + q) * nn + t];
      const double r1 = -pa * j1 - pb * j2 + pc * en[j + q * P];
      const double k1 = ca * d.k[q * nn + t] + dt * r1;
      const double k2 = ca * d.k[(3 + q) * nn + t] + dt * j1;
      d.k[q * nn + t] = k1;
      d.k[(3 + q) * nn + t] = k2;
      d.aux[q * nn + t] = j1 + cb * k1;
      d.aux[(3 + q) * nn + t] = j2 + cb * k2;
    }
  }
}

// userinc (src/cem_maxwell.F:495-496): the listed slots' face values get the
// stage's incident field, H into fhn and E into fen
__global__ void k_incident(PlainDev a) {
  const long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (q >= a.ninc) return;
  const long j = a.inc_slot[q], L = a.nxzfl;
  for (int m = 0; m < 6; ++m) a.fface[m * L + j] = a.fface[m * L + j] + a.inc_val[6 * q + m];
}

// cem_3d_graphene_current (src/cem_maxwell.F:2827-2931) at one listed face
// slot: the surface current from the face fields, the residuals of its Drude
// and critical-point currents and their rk4_upd, then userfsrc's -J on the
// -n x H part of srflx (tests/3dgraphene/3dgraphene.usr:236-264)
__global__ void k_graphene(PlainDev a, double ca, double cb, double dt) {
  const long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long ng = a.ngraph;
  if (q >= ng) return;
  const long j = a.gr_slot[q], L = a.nxzfl;
  double p[12];
  for (int i = 0; i < 12; ++i) p[i] = a.gr_par[i * ng + q];
  const double a_d = p[0], b_d = p[1], b_cp1 = p[2], a_211 = p[3], a_221 = p[4], b_11 = p[5];
  const double b_21 = p[6], b_cp2 = p[7], a_212 = p[8], a_222 = p[9], b_12 = p[10], b_22 = p[11];
  const double ux = a.unx[j], uy = a.uny[j], uz = a.unz[j];
  const double* fh = a.fface;
  const double* fe = a.fface + 3 * L;
  double nH[3], nEn[3];
  nH[0] = -uy * fh[2 * L + j] + uz * fh[L + j];
  nH[1] = ux * fh[2 * L + j] - uz * fh[j];
  nH[2] = -ux * fh[L + j] + uy * fh[j];
  const double ndotE = ux * fe[j] + uy * fe[L + j] + uz * fe[2 * L + j];
  nEn[0] = fe[j] - ux * ndotE;
  nEn[1] = fe[L + j] - uy * ndotE;
  nEn[2] = fe[2 * L + j] - uz * ndotE;
  const double Yfac = 0.5 / a.Y0[j];
  const double cpfac = b_cp1 + b_cp2;
  const double jnfac = 1.0 - cpfac * Yfac;
  for (int m = 0; m < 3; ++m) {
    double F[6], R[6];
    for (int k = 1; k < 6; ++k) F[k] = a.gr_f[(3 * k + m) * ng + q];
    const double tmp = Yfac * (nH[m] + a.gr_yc[q] * nEn[m]);
    F[0] = (F[1] + F[2] + F[4] - cpfac * tmp) / jnfac;
    const double f = tmp - Yfac * F[0];
    R[1] = -a_d * F[1] + b_d * f;
    R[2] = F[3] + b_11 * f;
    R[3] = -a_211 * F[2] - a_221 * F[3] + b_21 * f;
    R[4] = F[5] + b_12 * f;
    R[5] = -a_212 * F[4] - a_222 * F[5] + b_22 * f;
    a.gr_f[m * ng + q] = F[0];
    for (int k = 1; k < 6; ++k) {
      const long o = (3 * k + m) * ng + q;
      const double kh = ca * a.gr_k[o] + dt * R[k];
      a.gr_k[o] = kh;
      a.gr_f[o] = F[k] + cb * kh;
    }
    a.srflx[(3 + m) * L + j] = a.srflx[(3 + m) * L + j] - F[0];
  }
}

int last_error() { return check_cuda(cudaGetLastError()); }

}  // namespace

int plain_incident(Context* c) {
  if (!c->pargs.ninc) return NEKGPU_OK;
  k_incident<<<blocks_for(c->pargs.ninc), kThreads, 0, c->stream>>>(c->pargs);
  c->last_launches += 1;
  return last_error();
}

int plain_dispersive(Context* c, double ca, double cb, double dt) {
  if (!c->pargs.disp.n) return NEKGPU_OK;
  const int n3 = c->nx * c->nx * c->nx;
  k_dispersive<<<blocks_for(c->pargs.disp.n), kThreads, 0, c->stream>>>(c->pargs, n3, ca, cb, dt);
  c->last_launches += 1;
  return last_error();
}

size_t dcurl_smem(int mx, int md) {
  const size_t md2 = (size_t)md * md, md3 = md2 * md;
  return (2 * (size_t)md * mx + 2 * md2 + 7 * md3 + 2 * md2 * mx + (size_t)mx * mx * mx) *
         sizeof(double);
}

int dcurl_into(Context* c, const double* u, double* res) {
  static bool dattr = false;
  if (!dattr) {
    if (check_cuda(cudaFuncSetAttribute(k_dcurl, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024)))
      return NEKGPU_ERR_CUDA;
    dattr = true;
  }
  PlainDev p = c->pargs;
  p.nx = c->nx;
  p.nelt = c->nelt;
  p.npts = c->npts;
  p.u = const_cast<double*>(u);
  p.res = res;
  k_dcurl<<<c->nelt, kThreads, dcurl_smem(c->nx, p.md), c->stream>>>(p);
  c->last_launches += 1;
  return last_error();
}

int plain_cem_maxwell(Context* c) {
  if (c->pargs.md) {
    static bool dattr = false;
    if (!dattr) {
      cudaFuncSetAttribute(k_dcurl, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
      dattr = true;
    }
    k_dcurl<<<c->nelt, kThreads, dcurl_smem(c->nx, c->pargs.md), c->stream>>>(c->pargs);
    c->last_launches += 1;
    return last_error();
  }
  const int n = c->nx, n3 = n * n * n;
  size_t smem = (3 * (size_t)n3 + 2 * n * n) * sizeof(double);
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_curl, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attr_set = true;
  }
  k_curl<<<c->nelt, kThreads, smem, c->stream>>>(c->pargs);
  c->last_launches += 1;
  return last_error();
}

int plain_restrict_to_face(Context* c) {
  k_restrict<<<blocks_for(c->nxzfl), kThreads, 0, c->stream>>>(c->pargs);
  c->last_launches += 1;
  return last_error();
}

int plain_gs(Context* c, double* d_u, int nfld) {
  if (c->pargs.npairs == 0) return NEKGPU_OK;
  k_gs_pairs<<<blocks_for(c->pargs.npairs), kThreads, 0, c->stream>>>(
      c->pargs.pairs, c->pargs.npairs, d_u, c->nxzfl, nfld);
  c->last_launches += 1;
  return last_error();
}

int plain_flux3d(Context* c, const double* rk) {
  k_flux_pre<<<blocks_for(c->nxzfl), kThreads, 0, c->stream>>>(c->pargs);
  if (rk && c->pargs.ngraph) {
    c->last_launches += 1;
    k_graphene<<<blocks_for(c->pargs.ngraph), kThreads, 0, c->stream>>>(c->pargs, rk[0], rk[1], rk[2]);
  }
  int st = plain_gs(c, c->pargs.srflx, 6);
  if (st) return st;
  c->last_launches += 1;
  if (c->pargs.ncempec > 0) {
    k_flux_pec<<<blocks_for(c->pargs.ncempec), kThreads, 0, c->stream>>>(c->pargs);
    c->last_launches += 1;
  }
  k_flux_upwind<<<blocks_for(c->nxzfl), kThreads, 0, c->stream>>>(c->pargs);
  c->last_launches += 1;
  return last_error();
}

int plain_add_flux_to_res(Context* c) {
  k_lift<<<blocks_for(c->npts), kThreads, 0, c->stream>>>(c->pargs);
  c->last_launches += 1;
  return last_error();
}

int plain_usersrc(Context* c, double ft) {
  if (!c->pargs.src_w) return NEKGPU_OK;
  k_usersrc<<<blocks_for(c->npts), kThreads, 0, c->stream>>>(c->pargs, ft);
  c->last_launches += 1;
  return last_error();
}

int plain_invqmass(Context* c) {
  k_invqmass<<<blocks_for(c->npts), kThreads, 0, c->stream>>>(c->pargs);
  c->last_launches += 1;
  return last_error();
}

int plain_pml_step(Context* c) {
  if (!c->pargs.npml) return NEKGPU_OK;
  const int n3 = c->nx * c->nx * c->nx;
  k_pml_step<<<blocks_for((long)c->pargs.npml * n3), kThreads, 0, c->stream>>>(c->pargs, n3);
  c->last_launches += 1;
  return last_error();
}

int plain_pml_rk_update(Context* c, double ca, double cb, double dt) {
  if (!c->pargs.npml) return NEKGPU_OK;
  k_pml_rk<<<blocks_for(6 * c->npts), kThreads, 0, c->stream>>>(c->pargs, ca, cb, dt);
  c->last_launches += 1;
  return last_error();
}

int plain_rk_update(Context* c, double ca, double cb, double dt) {
  k_rk<<<blocks_for(6 * c->npts), kThreads, 0, c->stream>>>(c->pargs, ca, cb, dt);
  c->last_launches += 1;
  return last_error();
}

}  // namespace nekgpu
