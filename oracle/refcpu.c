/*
 * refcpu.c -- CPU FP64 restatement of NekCEM's 3-D Maxwell DG time step.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  Only the tests, the smoke check and
 * the CPU-baseline leg of the benchmark load this file's library; the product
 * library never does.
 *
 * Each function names the reference routine it restates (path:line inside the
 * NekCEM source tree).  Layout is the reference's: a scalar field is
 * u[i + n*j + n*n*k + n^3*e] (Fortran u(i,j,k,e)), a 3-vector field is three
 * such arrays back to back (Fortran hn(npts,3)), face arrays are indexed by the
 * face slot j + n^2*(f + 6*e) with f in the reference's "pff" face order.
 * Summation orders follow the reference; build with -ffp-contract=off so no
 * fused multiply-add changes the rounding on either x86 or Arm.
 */
#include "refcpu.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 1;
void ref_set_threads(int nthreads) { g_threads = nthreads < 1 ? 1 : nthreads; }
int ref_get_threads(void) { return g_threads; }

struct ref_ctx {
  int N, n, nelt, nel[3], bc[3];
  int ndim, imode, nfaces; /* 3, 3, 6; or 2 with imode 1 (TE) / 2 (TM), 4 */
  long npts, nxzf, nxzfl, ncempec;
  double lo[3], hi[3];
  double *zgm1, *wxm1, *dxm1, *dxtm1, *w3m1;
  double *xm1, *ym1, *zm1;
  double *rxm1, *rym1, *rzm1, *sxm1, *sym1, *szm1, *txm1, *tym1, *tzm1, *jacm1, *bm1;
  double *unx, *uny, *unz, *area;
  int *cemface, *cbc, *cempec;
  long long* glo_face;
  int *gs_order, *gs_start, gs_ngroups;
  double *permittivity, *permeability, *impede, *conduc, *zimpede, *yconduc;
  double *Z_0, *Z_1, *Y_0, *Y_1, *ebm1, *hbm1;
  double *hn, *en, *khn, *ken, *reshn, *resen, *fhn, *fen, *srflx;
  double *src_w; /* bm1 * exp(-r^2/(2 sigma^2)) per node, or NULL */
  double C0, src_amp, src_f0, src_t0;
  int src_kind;
  /* PML (src/PML): tags per element, sigma (npts,3), auxiliary fields and
   * their RK registers and residuals (npts,3 each) */
  int ifpml, maxpml, *pmltag, *pmlptr;
  double *pmlsigma, *pmlbn, *pmldn, *kpmlbn, *kpmldn, *respmlbn, *respmldn, *respmlhn, *respmlen;
  double pmlinner[6], pmlouter[6];
  /* dispersive media (the /userdrude/ and /userlorentz/ blocks of
   * tests/drude/drude.usr and tests/lorentz/lorentz.usr): per node parameters
   * (npts,2) / (npts,3), 0-based index lists, currents jn(npts,3) /
   * jn(npts,3,2) with their RK registers and residuals */
  long ndrude, nlorentz;
  int *drudeindex, *lorentzindex;
  double *drudeparams, *djn, *dkjn, *dresjn;
  double *lorentzparams, *ljn, *lkjn, *lresjn;
  /* dealiased curl (ifdealias, param(18) = -1): md = lxd GLL points per
   * direction, interpolation jgl (md x mx) / jgt, derivative dxmd / dxtmd on
   * the md points, weights w3md and the metrics interpolated to md^3 nodes */
  int md;
  double *jgl, *jgt, *dxmd, *dxtmd, *w3md, *metd;
  /* graphene sheets (the /usergraph/ block of tests/3dgraphene): 12
   * parameters per face slot (nxzfl,12), the listed slots, the face currents
   * fjn(nxzfl,3,6) with registers and residuals */
  long ngraph;
  int* graphindex;
  double *graphparams, *fjn, *kfjn, *resfjn;
  /* userinc plane wave: amp (H then E) * cos(k.x - omega t) on listed slots */
  long ninc;
  int* incslot;
  double incamp[6], inck[3], incomega;
  int rkstep_now; /* stage of the op in progress (0 outside ref_rk_stage) */
  double dt_now;
  double volvm1;
};

/* ------------------------------------------------------------------------ */
/* Spectral library (src/nek5_speclib.F)                                     */
/* ------------------------------------------------------------------------ */

/* JACOBF (src/nek5_speclib.F:482-522): Jacobi polynomial of degree n at x,
 * its derivative, and the degree n-1 / n-2 values. */
static void jacobf(double* poly, double* pder, double* polym1, double* pderm1, double* polym2,
                   double* pderm2, int n, double alp, double bet, double x) {
  double apb = alp + bet;
  double p = 1.0, pd = 0.0, pl, pdl, psave = 0.0, pdsave = 0.0;
  *poly = p; *pder = pd;
  if (n == 0) return;
  pl = p; pdl = pd;
  p = (alp - bet + (apb + 2.0) * x) / 2.0;
  pd = (apb + 2.0) / 2.0;
  if (n == 1) { *poly = p; *pder = pd; return; }
  for (int k = 2; k <= n; ++k) {
    double dk = (double)k;
    double a1 = 2.0 * dk * (dk + apb) * (2.0 * dk + apb - 2.0);
    double a2 = (2.0 * dk + apb - 1.0) * (alp * alp - bet * bet);
    double b3 = (2.0 * dk + apb - 2.0);
    double a3 = b3 * (b3 + 1.0) * (b3 + 2.0);
    double a4 = 2.0 * (dk + alp - 1.0) * (dk + bet - 1.0) * (2.0 * dk + apb);
    double polyn = ((a2 + a3 * x) * p - a4 * pl) / a1;
    double pdern = ((a2 + a3 * x) * pd - a4 * pdl + a3 * p) / a1;
    psave = pl; pdsave = pdl;
    pl = p; p = polyn;
    pdl = pd; pd = pdern;
  }
  *poly = p; *pder = pd;
  *polym1 = pl; *pderm1 = pdl;
  *polym2 = psave; *pderm2 = pdsave;
}

/* GAMMAF (src/nek5_speclib.F:373-394): table of the values the GLL code uses. */
static double gammaf(double x) {
  const double pi = 4.0 * atan(1.0);
  double g = 1.0;
  if (x == -0.5) g = -2.0 * sqrt(pi);
  if (x == 0.5) g = sqrt(pi);
  if (x == 1.0) g = 1.0;
  if (x == 2.0) g = 1.0;
  if (x == 1.5) g = sqrt(pi) / 2.0;
  if (x == 2.5) g = 1.5 * sqrt(pi) / 2.0;
  if (x == 3.5) g = 0.5 * (2.5 * (1.5 * sqrt(pi)));
  if (x == 3.0) g = 2.0;
  if (x == 4.0) g = 6.0;
  if (x == 5.0) g = 24.0;
  if (x == 6.0) g = 120.0;
  return g;
}

/* PNORMJ (src/nek5_speclib.F:396-421) */
static double pnormj(int n, double alpha, double beta) {
  double dn = (double)n, cnst = alpha + beta + 1.0, prod;
  if (n <= 1) {
    prod = gammaf(dn + alpha) * gammaf(dn + beta);
    prod = prod / (gammaf(dn) * gammaf(dn + alpha + beta));
    return prod * pow(2.0, cnst) / (2.0 * dn + cnst);
  }
  prod = gammaf(alpha + 1.0) * gammaf(beta + 1.0);
  prod = prod / (2.0 * (1.0 + cnst) * gammaf(cnst + 1.0));
  prod = prod * (1.0 + alpha) * (2.0 + alpha);
  prod = prod * (1.0 + beta) * (2.0 + beta);
  for (int i = 3; i <= n; ++i) {
    double di = (double)i;
    double frac = (di + alpha) * (di + beta) / (di * (di + alpha + beta));
    prod = prod * frac;
  }
  return prod * pow(2.0, cnst) / (2.0 * dn + cnst);
}

/* JACG (src/nek5_speclib.F:423-480): Gauss-Jacobi points by Newton with
 * deflation, then sorted ascending. */
static void jacg(double* xjac, int np, double alpha, double beta) {
  const int kstop = 10;
  const double eps = 1.0e-12;
  int n = np - 1;
  double dth = 4.0 * atan(1.0) / (2.0 * (double)n + 2.0);
  double xlast = 0.0, p, pd, pm1, pdm1, pm2, pdm2;
  for (int j = 1; j <= np; ++j) {
    double x;
    if (j == 1) {
      x = cos((2.0 * ((double)j - 1.0) + 1.0) * dth);
    } else {
      double x1 = cos((2.0 * ((double)j - 1.0) + 1.0) * dth);
      x = (x1 + xlast) / 2.0;
    }
    for (int k = 1; k <= kstop; ++k) {
      jacobf(&p, &pd, &pm1, &pdm1, &pm2, &pdm2, np, alpha, beta, x);
      double recsum = 0.0;
      for (int i = 1; i <= j - 1; ++i) recsum = recsum + 1.0 / (x - xjac[np - i]);
      double delx = -p / (pd - recsum * p);
      x = x + delx;
      if (fabs(delx) < eps) break;
    }
    xjac[np - j] = x;
    xlast = x;
  }
  for (int i = 0; i < np; ++i) {
    double xmin = 2.0;
    int jmin = i;
    for (int j = i; j < np; ++j)
      if (xjac[j] < xmin) { xmin = xjac[j]; jmin = j; }
    if (jmin != i) { double s = xjac[i]; xjac[i] = xjac[jmin]; xjac[jmin] = s; }
  }
}

/* ZWGJD (src/nek5_speclib.F:156-205) */
static void zwgjd(double* z, double* w, int np, double alpha, double beta) {
  int n = np - 1;
  double apb = alpha + beta, p, pd, pm1, pdm1, pm2, pdm2;
  if (np == 1) {
    z[0] = (beta - alpha) / (apb + 2.0);
    w[0] = gammaf(alpha + 1.0) * gammaf(beta + 1.0) / gammaf(apb + 2.0) * pow(2.0, apb + 1.0);
    return;
  }
  jacg(z, np, alpha, beta);
  int np1 = n + 1, np2 = n + 2;
  double dnp1 = (double)np1, dnp2 = (double)np2;
  double fac1 = dnp1 + alpha + beta + 1.0;
  double fac2 = fac1 + dnp1;
  double fac3 = fac2 + 1.0;
  double fnorm = pnormj(np1, alpha, beta);
  double rcoef = (fnorm * fac2 * fac3) / (2.0 * fac1 * dnp2);
  for (int i = 0; i < np; ++i) {
    jacobf(&p, &pd, &pm1, &pdm1, &pm2, &pdm2, np2, alpha, beta, z[i]);
    w[i] = -rcoef / (p * pdm1);
  }
}

/* ENDW1 / ENDW2 (src/nek5_speclib.F:285-371) */
static double endw(int which, int n, double alpha, double beta) {
  double apb = alpha + beta, f1, f2, f3 = 0.0, fint1, fint2;
  if (n == 0) return 0.0;
  if (which == 1) {
    f1 = gammaf(alpha + 2.0) * gammaf(beta + 1.0) / gammaf(apb + 3.0);
  } else {
    f1 = gammaf(alpha + 1.0) * gammaf(beta + 2.0) / gammaf(apb + 3.0);
  }
  f1 = f1 * (apb + 2.0) * pow(2.0, apb + 2.0) / 2.0;
  if (n == 1) return f1;
  if (which == 1) {
    fint1 = gammaf(alpha + 2.0) * gammaf(beta + 1.0) / gammaf(apb + 3.0);
  } else {
    fint1 = gammaf(alpha + 1.0) * gammaf(beta + 2.0) / gammaf(apb + 3.0);
  }
  fint1 = fint1 * pow(2.0, apb + 2.0);
  fint2 = gammaf(alpha + 2.0) * gammaf(beta + 2.0) / gammaf(apb + 4.0);
  fint2 = fint2 * pow(2.0, apb + 3.0);
  if (which == 1)
    f2 = (-2.0 * (beta + 2.0) * fint1 + (apb + 4.0) * fint2) * (apb + 3.0) / 4.0;
  else
    f2 = (2.0 * (alpha + 2.0) * fint1 - (apb + 4.0) * fint2) * (apb + 3.0) / 4.0;
  if (n == 2) return f2;
  for (int i = 3; i <= n; ++i) {
    double di = (double)(i - 1);
    double abn = alpha + beta + di;
    double abnn = abn + di;
    double a1 = -(2.0 * (di + alpha) * (di + beta)) / (abn * abnn * (abnn + 1.0));
    double a2 = (2.0 * (alpha - beta)) / (abnn * (abnn + 2.0));
    double a3 = (2.0 * (abn + 1.0)) / ((abnn + 2.0) * (abnn + 1.0));
    f3 = -(a2 * f2 + a1 * f1) / a3;
    f1 = f2;
    f2 = f3;
  }
  return f3;
}

/* ZWGLL -> ZWGLJ -> ZWGLJD (src/nek5_speclib.F:107-121, 208-283), alpha=beta=0 */
void ref_zwgll(double* z, double* w, int np) {
  const double alpha = 0.0, beta = 0.0;
  int n = np - 1, nm1 = n - 1;
  double p, pd, pm1, pdm1, pm2, pdm2;
  if (nm1 > 0) zwgjd(z + 1, w + 1, nm1, alpha + 1.0, beta + 1.0);
  z[0] = -1.0;
  z[np - 1] = 1.0;
  for (int i = 1; i < np - 1; ++i) w[i] = w[i] / (1.0 - z[i] * z[i]);
  jacobf(&p, &pd, &pm1, &pdm1, &pm2, &pdm2, n, alpha, beta, z[0]);
  w[0] = endw(1, n, alpha, beta) / (2.0 * pd);
  jacobf(&p, &pd, &pm1, &pdm1, &pm2, &pdm2, n, alpha, beta, z[np - 1]);
  w[np - 1] = endw(2, n, alpha, beta) / (2.0 * pd);
}

/* PNLEG (src/nek5_speclib.F:882-910) */
double ref_pnleg(double z, int n) {
  if (fabs(z) < 1.0e-25) z = 0.0;
  double p1 = 1.0, p2, p3;
  if (n == 0) return p1;
  p2 = z;
  p3 = p2;
  for (int k = 1; k <= n - 1; ++k) {
    double fk = (double)k;
    p3 = ((2.0 * fk + 1.0) * z * p2 - fk * p1) / (fk + 1.0);
    p1 = p2;
    p2 = p3;
  }
  return p3;
}

/* DGLL (src/nek5_speclib.F:807-840) */
void ref_dgll(double* d, double* dt, const double* z, int nz) {
  int n = nz - 1;
  if (nz == 1) { d[0] = 0.0; dt[0] = 0.0; return; }
  double fn = (double)n;
  double d0 = fn * (fn + 1.0) / 4.0;
  for (int i = 0; i < nz; ++i)
    for (int j = 0; j < nz; ++j) {
      double v = 0.0;
      if (i != j) v = ref_pnleg(z[i], n) / (ref_pnleg(z[j], n) * (z[i] - z[j]));
      if (i == j && i == 0) v = -d0;
      if (i == j && i == nz - 1) v = d0;
      d[i + nz * j] = v;
      dt[j + nz * i] = v;
    }
}

/* ------------------------------------------------------------------------ */
/* Tensor contractions (src/nek5_grad.F:2-19, src/nek5_mxm_std.F:173-191)    */
/* ------------------------------------------------------------------------ */

/* mxm with the mxf summation order: c(i,j) = sum_l a(i,l) b(l,j), l ascending */
static void mxm(const double* a, int n1, const double* b, int n2, double* c, int n3) {
  for (int j = 0; j < n3; ++j)
    for (int i = 0; i < n1; ++i) {
      double s = a[i] * b[(size_t)n2 * j];
      for (int l = 1; l < n2; ++l) s = s + a[i + (size_t)n1 * l] * b[l + (size_t)n2 * j];
      c[i + (size_t)n1 * j] = s;
    }
}

/* local_grad3 (src/nek5_grad.F:2-19): ur = D u, us_k = u_k Dt, ut = u Dt */
void ref_local_grad3(double* ur, double* us, double* ut, const double* u, int n, const double* D,
                     const double* Dt) {
  int m2 = n * n;
  mxm(D, n, u, n, ur, m2);
  for (int k = 0; k < n; ++k) mxm(u + (size_t)m2 * k, n, Dt, n, us + (size_t)m2 * k, n);
  mxm(u, m2, Dt, n, ut, n);
}

/* ------------------------------------------------------------------------ */
/* Mesh / geometry                                                           */
/* ------------------------------------------------------------------------ */

/* Face slot f (0..5, the reference's pff order) -> reference axis (0=r,1=s,2=t)
 * and side; EFACE/SKPDAT (src/nek5_connect11.F:1067-1078, 1483-1530). */
static const int slot_axis[6] = {1, 0, 1, 0, 2, 2};
static const int slot_side[6] = {-1, +1, +1, -1, -1, +1};

/* volume index (within element) of node (a,b) of slot f; a walks fastest
 * (cem_set_fc_ptr, src/cem_common.F:214-257 with SKPDAT) */
static int face_vol_index(int f, int a, int b, int n) {
  int fixed = slot_side[f] < 0 ? 0 : n - 1;
  switch (slot_axis[f]) {
    case 0: return fixed + n * a + n * n * b;
    case 1: return a + n * fixed + n * n * b;
    default: return a + n * b + n * n * fixed;
  }
}

static double* dalloc(long n) { return (double*)calloc((size_t)(n > 0 ? n : 1), sizeof(double)); }
static int* ialloc(long n) { return (int*)calloc((size_t)(n > 0 ? n : 1), sizeof(int)); }

static long long* g_sort_keys;
static int cmp_by_key(const void* a, const void* b) {
  long long ka = g_sort_keys[*(const int*)a], kb = g_sort_keys[*(const int*)b];
  if (ka != kb) return ka < kb ? -1 : 1;
  return *(const int*)a - *(const int*)b;
}

/* gs_setup semantics (src/jl/gs.h:17-60): group face slots by global id. */
static void gs_setup_local(ref_ctx* c) {
  long m = c->nxzfl;
  c->gs_order = ialloc(m);
  c->gs_start = ialloc(m + 1);
  for (long i = 0; i < m; ++i) c->gs_order[i] = (int)i;
  g_sort_keys = c->glo_face;
  qsort(c->gs_order, (size_t)m, sizeof(int), cmp_by_key);
  g_sort_keys = NULL;
  int ng = 0;
  for (long i = 0; i < m; ++i)
    if (i == 0 || c->glo_face[c->gs_order[i]] != c->glo_face[c->gs_order[i - 1]])
      c->gs_start[ng++] = (int)i;
  c->gs_start[ng] = (int)m;
  c->gs_ngroups = ng;
}

/* genxyz for an axis-aligned hex (src/nek5_genxyz.F:562-655): trilinear map
 * of the 8 corners, accumulated in the reference's corner loop order. */
static void genxyz_box(ref_ctx* c) {
  int n = c->n;
  for (int e = 0; e < c->nelt; ++e) {
    int ex = e % c->nel[0], ey = (e / c->nel[0]) % c->nel[1], ez = e / (c->nel[0] * c->nel[1]);
    int ec[3] = {ex, ey, ez};
    double cb[3][2];
    for (int d = 0; d < 3; ++d) {
      double L = c->hi[d] - c->lo[d];
      cb[d][0] = c->lo[d] + L * (double)ec[d] / (double)c->nel[d];
      cb[d][1] = c->lo[d] + L * (double)(ec[d] + 1) / (double)c->nel[d];
    }
    double h[16][2];
    for (int i = 0; i < n; ++i) {
      h[i][0] = (1.0 - c->zgm1[i]) * 0.5;
      h[i][1] = (1.0 + c->zgm1[i]) * 0.5;
    }
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          long idx = i + (long)n * j + (long)n * n * k + (long)n * n * n * e;
          c->xm1[idx] = c->ym1[idx] = c->zm1[idx] = 0.0;
        }
    for (int izt = 0; izt < 2; ++izt)
      for (int iyt = 0; iyt < 2; ++iyt)
        for (int ixt = 0; ixt < 2; ++ixt)
          for (int k = 0; k < n; ++k)
            for (int j = 0; j < n; ++j) {
              double hh = h[j][iyt] * h[k][izt];
              for (int i = 0; i < n; ++i) {
                double hhh = h[i][ixt] * hh;
                long idx = i + (long)n * j + (long)n * n * k + (long)n * n * n * e;
                c->xm1[idx] = c->xm1[idx] + hhh * cb[0][ixt];
                c->ym1[idx] = c->ym1[idx] + hhh * cb[1][iyt];
                c->zm1[idx] = c->zm1[idx] + hhh * cb[2][izt];
              }
            }
  }
}

/* Smooth interior deformation of the box (a usrdat2-style user mapping,
 * tests/3dboxpml/3dboxpml.usr:159-194 shows the hook): every point moves by
 * amp * L_d * s * sin(2 pi xi_(d+1)), s = sin(pi xi_x) sin(pi xi_y) sin(pi xi_z),
 * xi the point's position in [0,1] per axis.  The domain boundary does not
 * move, so the face pairing and PEC/periodic faces stay as they are, while
 * the elements become curvilinear. */
static void map_box(ref_ctx* c, double amp) {
  const double pi = 4.0 * atan(1.0);
  for (long i = 0; i < c->npts; ++i) {
    double xi[3] = {(c->xm1[i] - c->lo[0]) / (c->hi[0] - c->lo[0]),
                    (c->ym1[i] - c->lo[1]) / (c->hi[1] - c->lo[1]),
                    (c->zm1[i] - c->lo[2]) / (c->hi[2] - c->lo[2])};
    double s = sin(pi * xi[0]) * sin(pi * xi[1]) * sin(pi * xi[2]);
    double dx = amp * (c->hi[0] - c->lo[0]) * s * sin(2 * pi * xi[1]);
    double dy = amp * (c->hi[1] - c->lo[1]) * s * sin(2 * pi * xi[2]);
    double dz = amp * (c->hi[2] - c->lo[2]) * s * sin(2 * pi * xi[0]);
    c->xm1[i] += dx;
    c->ym1[i] += dy;
    c->zm1[i] += dz;
  }
}

static ref_ctx* create_box(int N, int nelx, int nely, int nelz, const double lo[3],
                           const double hi[3], const int bc[3], double amp);

ref_ctx* ref_create_box(int N, int nelx, int nely, int nelz, const double lo[3],
                        const double hi[3], const int bc[3]) {
  return create_box(N, nelx, nely, nelz, lo, hi, bc, 0.0);
}

ref_ctx* ref_create_box_mapped(int N, int nelx, int nely, int nelz, const double lo[3],
                               const double hi[3], const int bc[3], double amp) {
  return create_box(N, nelx, nely, nelz, lo, hi, bc, amp);
}

static ref_ctx* create_box(int N, int nelx, int nely, int nelz, const double lo[3],
                           const double hi[3], const int bc[3], double amp) {
  if (N < 1 || N > 15 || nelx < 1 || nely < 1 || nelz < 1) return NULL;
  ref_ctx* c = (ref_ctx*)calloc(1, sizeof(ref_ctx));
  int n = N + 1;
  c->N = N; c->n = n;
  c->ndim = 3; c->imode = 3; c->nfaces = 6;
  c->nel[0] = nelx; c->nel[1] = nely; c->nel[2] = nelz;
  c->nelt = nelx * nely * nelz;
  for (int d = 0; d < 3; ++d) { c->lo[d] = lo[d]; c->hi[d] = hi[d]; c->bc[d] = bc[d]; }
  long n3 = (long)n * n * n;
  c->npts = n3 * c->nelt;
  c->nxzf = (long)n * n;
  c->nxzfl = 6 * c->nxzf * c->nelt;
  long npts = c->npts, nxzfl = c->nxzfl;

  /* GENWZ (src/nek5_coef.F:1-260) */
  c->zgm1 = dalloc(n); c->wxm1 = dalloc(n);
  c->dxm1 = dalloc(n * n); c->dxtm1 = dalloc(n * n);
  c->w3m1 = dalloc(n3);
  ref_zwgll(c->zgm1, c->wxm1, n);
  ref_dgll(c->dxm1, c->dxtm1, c->zgm1, n);
  for (int iz = 0; iz < n; ++iz)
    for (int iy = 0; iy < n; ++iy)
      for (int ix = 0; ix < n; ++ix)
        c->w3m1[ix + n * iy + n * n * iz] = c->wxm1[ix] * c->wxm1[iy] * c->wxm1[iz];

  c->xm1 = dalloc(npts); c->ym1 = dalloc(npts); c->zm1 = dalloc(npts);
  genxyz_box(c);
  if (amp != 0.0) map_box(c, amp);

  /* XYZRST (src/nek5_coef.F:877-924) + GLMAPM1 (555-635) + GEODAT1 bm1 (758) */
  double *xr = dalloc(npts), *yr = dalloc(npts), *zr = dalloc(npts);
  double *xs = dalloc(npts), *ys = dalloc(npts), *zs = dalloc(npts);
  double *xt = dalloc(npts), *yt = dalloc(npts), *zt = dalloc(npts);
  for (int e = 0; e < c->nelt; ++e) {
    long o = n3 * e;
    ref_local_grad3(xr + o, xs + o, xt + o, c->xm1 + o, n, c->dxm1, c->dxtm1);
    ref_local_grad3(yr + o, ys + o, yt + o, c->ym1 + o, n, c->dxm1, c->dxtm1);
    ref_local_grad3(zr + o, zs + o, zt + o, c->zm1 + o, n, c->dxm1, c->dxtm1);
  }
  c->rxm1 = dalloc(npts); c->rym1 = dalloc(npts); c->rzm1 = dalloc(npts);
  c->sxm1 = dalloc(npts); c->sym1 = dalloc(npts); c->szm1 = dalloc(npts);
  c->txm1 = dalloc(npts); c->tym1 = dalloc(npts); c->tzm1 = dalloc(npts);
  c->jacm1 = dalloc(npts); c->bm1 = dalloc(npts);
  for (long i = 0; i < npts; ++i) {
    double jac = 0.0;
    jac = jac + xr[i] * ys[i] * zt[i];
    jac = jac + xt[i] * yr[i] * zs[i];
    jac = jac + xs[i] * yt[i] * zr[i];
    jac = jac - xr[i] * yt[i] * zs[i];
    jac = jac - xs[i] * yr[i] * zt[i];
    jac = jac - xt[i] * ys[i] * zr[i];
    c->jacm1[i] = jac;
    c->rxm1[i] = ys[i] * zt[i] - yt[i] * zs[i];
    c->rym1[i] = xt[i] * zs[i] - xs[i] * zt[i];
    c->rzm1[i] = xs[i] * yt[i] - xt[i] * ys[i];
    c->sxm1[i] = yt[i] * zr[i] - yr[i] * zt[i];
    c->sym1[i] = xr[i] * zt[i] - xt[i] * zr[i];
    c->szm1[i] = xt[i] * yr[i] - xr[i] * yt[i];
    c->txm1[i] = yr[i] * zs[i] - ys[i] * zr[i];
    c->tym1[i] = xs[i] * zr[i] - xr[i] * zs[i];
    c->tzm1[i] = xr[i] * ys[i] - xs[i] * yr[i];
  }
  for (int e = 0; e < c->nelt; ++e)
    for (long i = 0; i < n3; ++i) c->bm1[n3 * e + i] = c->jacm1[n3 * e + i] * c->w3m1[i];
  c->volvm1 = 0.0;
  for (long i = 0; i < npts; ++i) c->volvm1 += c->bm1[i];

  /* AREA3 (src/nek5_coef.F:1150-1237): per-node cross products, then the
   * face restriction; UNITVEC (src/nek5_mat1.F:2006) normalises. */
  c->unx = dalloc(nxzfl); c->uny = dalloc(nxzfl); c->unz = dalloc(nxzfl); c->area = dalloc(nxzfl);
  for (int e = 0; e < c->nelt; ++e)
    for (int f = 0; f < 6; ++f) {
      int ax = slot_axis[f], sd = slot_side[f];
      for (int b = 0; b < n; ++b)
        for (int a = 0; a < n; ++a) {
          long v = n3 * e + face_vol_index(f, a, b, n);
          double A, B, C, wgt;
          if (ax == 0) { /* "R": xs x xt */
            A = ys[v] * zt[v] - zs[v] * yt[v];
            B = zs[v] * xt[v] - xs[v] * zt[v];
            C = xs[v] * yt[v] - ys[v] * xt[v];
          } else if (ax == 1) { /* "S": xr x xt */
            A = yr[v] * zt[v] - zr[v] * yt[v];
            B = zr[v] * xt[v] - xr[v] * zt[v];
            C = xr[v] * yt[v] - yr[v] * xt[v];
          } else { /* "T": xr x xs */
            A = yr[v] * zs[v] - zr[v] * ys[v];
            B = zr[v] * xs[v] - xr[v] * zs[v];
            C = xr[v] * ys[v] - yr[v] * xs[v];
          }
          double dot = A * A + B * B + C * C;
          wgt = c->wxm1[a] * c->wxm1[b];
          /* sign: r: +A on r=+1, -A on r=-1; s: +A on s=-1, -A on s=+1;
           * t: -A on t=-1, +A on t=+1 */
          double sg;
          if (ax == 0) sg = sd > 0 ? 1.0 : -1.0;
          else if (ax == 1) sg = sd < 0 ? 1.0 : -1.0;
          else sg = sd > 0 ? 1.0 : -1.0;
          long j = a + (long)n * b + c->nxzf * (f + 6L * e);
          c->area[j] = sqrt(dot) * wgt;
          double nx = sg * A, ny = sg * B, nz = sg * C;
          double len = sqrt(nx * nx + ny * ny + nz * nz);
          if (len != 0.0) { nx = nx / len; ny = ny / len; nz = nz / len; }
          c->unx[j] = nx; c->uny[j] = ny; c->unz[j] = nz;
        }
    }
  free(xr); free(yr); free(zr); free(xs); free(ys); free(zs); free(xt); free(yt); free(zt);

  /* cem_set_fc_ptr (src/cem_common.F:214-257); face global numbering with the
   * semantics of setup_dgds2 (src/nek5_connect11.F:2179-2233): the two
   * slots that share a face node carry the same positive id; a PEC face node
   * is a singleton.  CBC codes: 0 = 'E  ' interior, 1 = 'PEC', 2 = 'P  ',
   * 3 = 'PML'. */
  c->cemface = ialloc(nxzfl);
  c->glo_face = (long long*)calloc((size_t)nxzfl, sizeof(long long));
  c->cbc = ialloc(6L * c->nelt);
  long long nplanes_off[3];
  nplanes_off[0] = 0;
  nplanes_off[1] = (long long)(nelx + 1) * nely * nelz;
  nplanes_off[2] = nplanes_off[1] + (long long)(nely + 1) * nelx * nelz;
  /* physical axis of each reference axis for an axis-aligned box: r->x, s->y, t->z */
  for (int e = 0; e < c->nelt; ++e) {
    int ec[3] = {e % nelx, (e / nelx) % nely, e / (nelx * nely)};
    for (int f = 0; f < 6; ++f) {
      int ax = slot_axis[f], sd = slot_side[f];
      int plane = ec[ax] + (sd > 0 ? 1 : 0);
      int boundary = (plane == 0 || plane == c->nel[ax]);
      if (boundary)
        c->cbc[6 * e + f] = c->bc[ax] == REF_BC_PERIODIC ? 2 : (c->bc[ax] == REF_BC_PML ? 3 : 1);
      if (boundary && c->bc[ax] == REF_BC_PERIODIC) plane = plane % c->nel[ax];
      long long fid;
      if (ax == 0) fid = nplanes_off[0] + ((long long)plane * nely + ec[1]) * nelz + ec[2];
      else if (ax == 1) fid = nplanes_off[1] + ((long long)plane * nelx + ec[0]) * nelz + ec[2];
      else fid = nplanes_off[2] + ((long long)plane * nelx + ec[0]) * nely + ec[1];
      for (int b = 0; b < n; ++b)
        for (int a = 0; a < n; ++a) {
          long j = a + (long)n * b + c->nxzf * (f + 6L * e);
          c->cemface[j] = (int)(n3 * e + face_vol_index(f, a, b, n));
          c->glo_face[j] = fid * (long long)(n * n) + a + (long long)n * b + 1;
        }
    }
  }
  gs_setup_local(c);

  /* cem_maxwell_pec_init (src/cem_maxwell.F:1338-1366): 'PEC' and 'PML' faces */
  c->cempec = ialloc(nxzfl);
  long l = 0;
  for (int e = 0; e < c->nelt; ++e)
    for (int f = 0; f < 6; ++f)
      if (c->cbc[6 * e + f] == 1 || c->cbc[6 * e + f] == 3)
        for (long j = 0; j < c->nxzf; ++j) c->cempec[l++] = (int)(j + c->nxzf * (f + 6L * e));
  c->ncempec = l;

  /* state and work arrays (src/EMWAVE) */
  c->hn = dalloc(3 * npts); c->en = dalloc(3 * npts);
  c->khn = dalloc(3 * npts); c->ken = dalloc(3 * npts);
  c->reshn = dalloc(3 * npts); c->resen = dalloc(3 * npts);
  c->fhn = dalloc(3 * nxzfl); c->fen = dalloc(3 * nxzfl);
  c->srflx = dalloc(6 * nxzfl);
  c->permittivity = dalloc(npts); c->permeability = dalloc(npts);
  c->impede = dalloc(npts); c->conduc = dalloc(npts);
  c->zimpede = dalloc(nxzfl); c->yconduc = dalloc(nxzfl);
  c->Z_0 = dalloc(nxzfl); c->Z_1 = dalloc(nxzfl); c->Y_0 = dalloc(nxzfl); c->Y_1 = dalloc(nxzfl);
  c->ebm1 = dalloc(npts); c->hbm1 = dalloc(npts);
  c->C0 = 1.0;
  double* one = dalloc(npts);
  for (long i = 0; i < npts; ++i) one[i] = 1.0;
  ref_set_materials(c, one, one);
  free(one);
  return c;
}

void ref_destroy(ref_ctx* c) {
  if (!c) return;
  double* d[] = {c->zgm1, c->wxm1, c->dxm1, c->dxtm1, c->w3m1, c->xm1, c->ym1, c->zm1,
                 c->rxm1, c->rym1, c->rzm1, c->sxm1, c->sym1, c->szm1, c->txm1, c->tym1,
                 c->tzm1, c->jacm1, c->bm1, c->unx, c->uny, c->unz, c->area,
                 c->permittivity, c->permeability, c->impede, c->conduc, c->zimpede,
                 c->yconduc, c->Z_0, c->Z_1, c->Y_0, c->Y_1, c->ebm1, c->hbm1, c->hn, c->en,
                 c->khn, c->ken, c->reshn, c->resen, c->fhn, c->fen, c->srflx, c->src_w};
  for (size_t i = 0; i < sizeof(d) / sizeof(d[0]); ++i) free(d[i]);
  free(c->cemface); free(c->cbc); free(c->cempec); free(c->glo_face);
  double* p[] = {c->pmlsigma, c->pmlbn, c->pmldn, c->kpmlbn, c->kpmldn, c->respmlbn,
                 c->respmldn, c->respmlhn, c->respmlen};
  for (size_t i = 0; i < sizeof(p) / sizeof(p[0]); ++i) free(p[i]);
  free(c->pmltag); free(c->pmlptr);
  double* q[] = {c->drudeparams, c->djn, c->dkjn, c->dresjn,
                 c->lorentzparams, c->ljn, c->lkjn, c->lresjn};
  for (size_t i = 0; i < sizeof(q) / sizeof(q[0]); ++i) free(q[i]);
  free(c->drudeindex); free(c->lorentzindex);
  free(c->jgl); free(c->jgt); free(c->dxmd); free(c->dxtmd); free(c->w3md); free(c->metd);
  free(c->incslot);
  free(c->graphindex); free(c->graphparams); free(c->fjn); free(c->kfjn); free(c->resfjn);
  free(c->gs_order); free(c->gs_start);
  free(c);
}

double* ref_darray(ref_ctx* c, const char* name, long* len) {
  struct { const char* nm; double* p; long n; } t[] = {
      {"zgm1", c->zgm1, c->n}, {"wxm1", c->wxm1, c->n}, {"dxm1", c->dxm1, (long)c->n * c->n},
      {"dxtm1", c->dxtm1, (long)c->n * c->n}, {"w3m1", c->w3m1, (long)c->n * c->n * c->n},
      {"xm1", c->xm1, c->npts}, {"ym1", c->ym1, c->npts}, {"zm1", c->zm1, c->npts},
      {"rxm1", c->rxm1, c->npts}, {"rym1", c->rym1, c->npts}, {"rzm1", c->rzm1, c->npts},
      {"sxm1", c->sxm1, c->npts}, {"sym1", c->sym1, c->npts}, {"szm1", c->szm1, c->npts},
      {"txm1", c->txm1, c->npts}, {"tym1", c->tym1, c->npts}, {"tzm1", c->tzm1, c->npts},
      {"jacm1", c->jacm1, c->npts}, {"bm1", c->bm1, c->npts},
      {"unx", c->unx, c->nxzfl}, {"uny", c->uny, c->nxzfl}, {"unz", c->unz, c->nxzfl},
      {"area", c->area, c->nxzfl},
      {"permittivity", c->permittivity, c->npts}, {"permeability", c->permeability, c->npts},
      {"Z_0", c->Z_0, c->nxzfl}, {"Z_1", c->Z_1, c->nxzfl}, {"Y_0", c->Y_0, c->nxzfl},
      {"Y_1", c->Y_1, c->nxzfl}, {"ebm1", c->ebm1, c->npts}, {"hbm1", c->hbm1, c->npts},
      {"hn", c->hn, 3 * c->npts}, {"en", c->en, 3 * c->npts}, {"khn", c->khn, 3 * c->npts},
      {"ken", c->ken, 3 * c->npts}, {"reshn", c->reshn, 3 * c->npts},
      {"resen", c->resen, 3 * c->npts}, {"fhn", c->fhn, 3 * c->nxzfl},
      {"fen", c->fen, 3 * c->nxzfl}, {"srflx", c->srflx, 6 * c->nxzfl},
      {"src_w", c->src_w, c->src_w ? c->npts : 0},
      {"pmlsigma", c->pmlsigma, c->pmlsigma ? 3 * c->npts : 0},
      {"pmlbn", c->pmlbn, c->pmlbn ? 3 * c->npts : 0},
      {"pmldn", c->pmldn, c->pmldn ? 3 * c->npts : 0},
      {"pmlinner", c->pmlinner, c->ifpml ? 6 : 0}, {"pmlouter", c->pmlouter, c->ifpml ? 6 : 0},
      {"fjn", c->fjn, c->fjn ? 18 * c->nxzfl : 0},
      {"yconduc", c->yconduc, c->nxzfl},
      {"jgl", c->jgl, c->md ? (long)c->md * c->n : 0},
      {"dxmd", c->dxmd, c->md ? (long)c->md * c->md : 0},
      {"w3md", c->w3md, c->md ? (long)c->md * c->md * c->md : 0},
      {"metd", c->metd, c->md ? 9L * c->md * c->md * c->md * c->nelt : 0},
      {"drudejn", c->djn, c->djn ? 3 * c->npts : 0},
      {"lorentzjn", c->ljn, c->ljn ? 6 * c->npts : 0},
  };
  for (size_t i = 0; i < sizeof(t) / sizeof(t[0]); ++i)
    if (strcmp(t[i].nm, name) == 0) { if (len) *len = t[i].n; return t[i].p; }
  if (len) *len = 0;
  return NULL;
}

int* ref_iarray(ref_ctx* c, const char* name, long* len) {
  if (strcmp(name, "cemface") == 0) { if (len) *len = c->nxzfl; return c->cemface; }
  if (strcmp(name, "cbc") == 0) { if (len) *len = (long)c->nfaces * c->nelt; return c->cbc; }
  if (strcmp(name, "pmltag") == 0 && c->ifpml) { if (len) *len = c->nelt; return c->pmltag; }
  if (strcmp(name, "pmlptr") == 0 && c->ifpml) { if (len) *len = c->maxpml; return c->pmlptr; }
  if (strcmp(name, "cempec") == 0) { if (len) *len = c->ncempec; return c->cempec; }
  if (len) *len = 0;
  return NULL;
}

long long* ref_larray(ref_ctx* c, const char* name, long* len) {
  if (strcmp(name, "glo_face") == 0) { if (len) *len = c->nxzfl; return c->glo_face; }
  if (len) *len = 0;
  return NULL;
}

long ref_size(const ref_ctx* c, const char* name) {
  if (strcmp(name, "n") == 0) return c->n;
  if (strcmp(name, "nelt") == 0) return c->nelt;
  if (strcmp(name, "npts") == 0) return c->npts;
  if (strcmp(name, "nxzf") == 0) return c->nxzf;
  if (strcmp(name, "nxzfl") == 0) return c->nxzfl;
  if (strcmp(name, "ncempec") == 0) return c->ncempec;
  return -1;
}

double ref_volvm1(const ref_ctx* c) { return c->volvm1; }

/* ------------------------------------------------------------------------ */
/* Materials (src/cem_maxwell.F:262-325, 183-186)                            */
/* ------------------------------------------------------------------------ */
void ref_set_materials(ref_ctx* c, const double* permittivity, const double* permeability) {
  long npts = c->npts, nxzfl = c->nxzfl;
  memcpy(c->permittivity, permittivity, sizeof(double) * npts);
  memcpy(c->permeability, permeability, sizeof(double) * npts);
  for (long i = 0; i < npts; ++i) {
    c->impede[i] = sqrt(c->permeability[i] / c->permittivity[i]);
    c->conduc[i] = sqrt(c->permittivity[i] / c->permeability[i]);
  }
  for (long j = 0; j < nxzfl; ++j) {
    int i = c->cemface[j];
    c->zimpede[j] = c->impede[i];
    c->yconduc[j] = c->conduc[i];
  }
  memcpy(c->Z_0, c->zimpede, sizeof(double) * nxzfl);
  memcpy(c->Y_0, c->yconduc, sizeof(double) * nxzfl);
  ref_gs_op_fields(c, c->Z_0, nxzfl, 1);
  ref_gs_op_fields(c, c->Y_0, nxzfl, 1);
  int nf = c->nfaces;
  for (int e = 0; e < c->nelt; ++e)
    for (int f = 0; f < nf; ++f)
      if (c->cbc[nf * e + f] == 1)
        for (long j = 0; j < c->nxzf; ++j) {
          long i = j + c->nxzf * (f + (long)nf * e);
          c->Y_0[i] = 2.0 * c->Y_0[i];
          c->Z_0[i] = 2.0 * c->Z_0[i];
        }
  for (long j = 0; j < nxzfl; ++j) {
    c->Z_1[j] = c->Z_0[j] - c->zimpede[j];
    c->Y_1[j] = c->Y_0[j] - c->yconduc[j];
  }
  for (long j = 0; j < nxzfl; ++j) {
    c->Z_0[j] = 0.5 * c->Z_0[j];
    c->Y_0[j] = 0.5 * c->Y_0[j];
  }
  /* ebm1 = 1/(eps*bm1), hbm1 = 1/(mu*bm1): col3 then invcol1 */
  for (long i = 0; i < npts; ++i) {
    c->ebm1[i] = 1.0 / (c->permittivity[i] * c->bm1[i]);
    c->hbm1[i] = 1.0 / (c->permeability[i] * c->bm1[i]);
  }
}

void ref_set_flux(ref_ctx* c, double C0) { c->C0 = C0; }

double ref_source_time(double t, double f0, double t0) {
  const double pi = 4.0 * atan(1.0);
  double a = pi * f0 * (t - t0);
  double a2 = a * a;
  return (1.0 - 2.0 * a2) * exp(-a2);
}

void ref_set_source_kind(ref_ctx* c, int kind) { c->src_kind = kind; }

void ref_set_source(ref_ctx* c, int enabled, const double xc[3], double sigma, double amp,
                    double f0, double t0) {
  free(c->src_w);
  c->src_w = NULL;
  if (!enabled) return;
  c->src_w = dalloc(c->npts);
  double s2 = 2.0 * sigma * sigma;
  for (long i = 0; i < c->npts; ++i) {
    double dx = c->xm1[i] - xc[0], dy = c->ym1[i] - xc[1], dz = c->zm1[i] - xc[2];
    c->src_w[i] = c->bm1[i] * exp(-(dx * dx + dy * dy + dz * dz) / s2);
  }
  c->src_amp = amp; c->src_f0 = f0; c->src_t0 = t0;
}

/* ------------------------------------------------------------------------ */
/* The stage operator                                                        */
/* ------------------------------------------------------------------------ */

/* maxwell_wght_curl (src/cem_maxwell.F:1428-1497) */
void ref_wght_curl(ref_ctx* c, double* w1, double* w2, double* w3, const double* u1,
                   const double* u2, const double* u3) {
  int n = c->n;
  long n3 = (long)n * n * n;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int e = 0; e < c->nelt; ++e) {
    double buf[9 * 16 * 16 * 16];
    double *u1r = buf, *u1s = buf + n3, *u1t = buf + 2 * n3;
    double *u2r = buf + 3 * n3, *u2s = buf + 4 * n3, *u2t = buf + 5 * n3;
    double *u3r = buf + 6 * n3, *u3s = buf + 7 * n3, *u3t = buf + 8 * n3;
    long j = n3 * e;
    ref_local_grad3(u1r, u1s, u1t, u1 + j, n, c->dxm1, c->dxtm1);
    ref_local_grad3(u2r, u2s, u2t, u2 + j, n, c->dxm1, c->dxtm1);
    ref_local_grad3(u3r, u3s, u3t, u3 + j, n, c->dxm1, c->dxtm1);
    for (long i = 0; i < n3; ++i) {
      long k = i + j;
      double w = c->w3m1[i];
      double u1rw = u1r[i] * w, u1sw = u1s[i] * w, u1tw = u1t[i] * w;
      double u2rw = u2r[i] * w, u2sw = u2s[i] * w, u2tw = u2t[i] * w;
      double u3rw = u3r[i] * w, u3sw = u3s[i] * w, u3tw = u3t[i] * w;
      double rx = c->rxm1[k], sx = c->sxm1[k], tx = c->txm1[k];
      double ry = c->rym1[k], sy = c->sym1[k], ty = c->tym1[k];
      double rz = c->rzm1[k], sz = c->szm1[k], tz = c->tzm1[k];
      w1[k] = u3rw * ry + u3sw * sy + u3tw * ty - u2rw * rz - u2sw * sz - u2tw * tz;
      w2[k] = u1rw * rz + u1sw * sz + u1tw * tz - u3rw * rx - u3sw * sx - u3tw * tx;
      w3[k] = u2rw * rx + u2sw * sx + u2tw * tx - u1rw * ry - u1sw * sy - u1tw * ty;
    }
  }
}

static void cem_maxwell_2d(ref_ctx* c);
static void restrict_2d(ref_ctx* c);
static void flux2d(ref_ctx* c);
static void lift_2d(ref_ctx* c);
static void invqmass_2d(ref_ctx* c);

/* cem_maxwell 3-D branch (src/cem_maxwell.F:574-582) */
void ref_cem_maxwell(ref_ctx* c) {
  if (c->ndim == 2) { cem_maxwell_2d(c); return; }
  long np = c->npts;
  if (c->md) { /* ifdealias branch (src/cem_maxwell.F:519-530) */
    ref_wght_dcurl(c, c->resen, c->resen + np, c->resen + 2 * np, c->hn, c->hn + np, c->hn + 2 * np);
    ref_wght_dcurl(c, c->reshn, c->reshn + np, c->reshn + 2 * np, c->en, c->en + np, c->en + 2 * np);
  } else {
    ref_wght_curl(c, c->resen, c->resen + np, c->resen + 2 * np, c->hn, c->hn + np, c->hn + 2 * np);
    ref_wght_curl(c, c->reshn, c->reshn + np, c->reshn + 2 * np, c->en, c->en + np, c->en + 2 * np);
  }
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (long i = 0; i < 3 * np; ++i) c->reshn[i] = -c->reshn[i];
}

/* cem_maxwell_restrict_to_face (src/cem_maxwell.F:604-623) */
void ref_restrict_to_face(ref_ctx* c) {
  if (c->ndim == 2) { restrict_2d(c); return; }
  long np = c->npts, nf = c->nxzfl;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (long j = 0; j < nf; ++j) {
    long i = c->cemface[j];
    for (int q = 0; q < 3; ++q) {
      c->fhn[j + q * nf] = c->hn[i + q * np];
      c->fen[j + q * nf] = c->en[i + q * np];
    }
  }
}

/* first loop of cem_maxwell_flux3d (src/cem_maxwell.F:944-955) */
void ref_flux_pre(ref_ctx* c) {
  long k = c->nxzfl;
  double *s = c->srflx, *fe = c->fen, *fh = c->fhn;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (long i = 0; i < k; ++i) {
    double nx = c->unx[i], ny = c->uny[i], nz = c->unz[i];
    s[0 * k + i] = -ny * fe[2 * k + i] + nz * fe[1 * k + i];
    s[1 * k + i] = -nz * fe[0 * k + i] + nx * fe[2 * k + i];
    s[2 * k + i] = -nx * fe[1 * k + i] + ny * fe[0 * k + i];
    s[3 * k + i] = -ny * fh[2 * k + i] + nz * fh[1 * k + i];
    s[4 * k + i] = -nz * fh[0 * k + i] + nx * fh[2 * k + i];
    s[5 * k + i] = -nx * fh[1 * k + i] + ny * fh[0 * k + i];
  }
}

/* gs_op_fields(gsh_face, u, stride, nfld, dom=1, op=add, transpose=0)
 * (src/jl/gs.c:2074-2099): every entry is replaced by the sum over its id
 * group; summed in increasing slot order. */
void ref_gs_op_fields(ref_ctx* c, double* u, long stride, int nfld) {
  for (int fld = 0; fld < nfld; ++fld) {
    double* v = u + stride * fld;
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int g = 0; g < c->gs_ngroups; ++g) {
      int b = c->gs_start[g], e = c->gs_start[g + 1];
      if (e - b < 2) continue;
      double s = v[c->gs_order[b]];
      for (int q = b + 1; q < e; ++q) s = s + v[c->gs_order[q]];
      for (int q = b; q < e; ++q) v[c->gs_order[q]] = s;
    }
  }
}

/* cem_maxwell_flux_pec (src/cem_maxwell.F:1368-1426) */
void ref_flux_pec(ref_ctx* c) {
  long k = c->nxzfl;
  double* s = c->srflx;
  for (long j = 0; j < c->ncempec; ++j) {
    long i = c->cempec[j];
    s[0 * k + i] = 2.0 * s[0 * k + i];
    s[1 * k + i] = 2.0 * s[1 * k + i];
    s[2 * k + i] = 2.0 * s[2 * k + i];
    s[3 * k + i] = 0.0;
    s[4 * k + i] = 0.0;
    s[5 * k + i] = 0.0;
  }
}

/* upwind combination (src/cem_maxwell.F:969-997) */
void ref_flux_upwind(ref_ctx* c) {
  long k = c->nxzfl;
  double* s = c->srflx;
  double C0 = c->C0;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (long i = 0; i < k; ++i) {
    double Y0 = c->Y_0[i], Y1 = c->Y_1[i], Z0 = c->Z_0[i], Z1 = c->Z_1[i];
    double Y02 = -0.5 / Y0 * Y1;
    double Z02 = 0.5 / Z0 * Z1;
    double C02Y = 0.5 / Y0 * C0;
    double C02Z = 0.5 / Z0 * C0;
    double nx = c->unx[i], ny = c->uny[i], nz = c->unz[i];
    double fu1 = ny * s[5 * k + i] - nz * s[4 * k + i];
    double fu2 = nz * s[3 * k + i] - nx * s[5 * k + i];
    double fu3 = nx * s[4 * k + i] - ny * s[3 * k + i];
    double fw1 = ny * s[2 * k + i] - nz * s[1 * k + i];
    double fw2 = nz * s[0 * k + i] - nx * s[2 * k + i];
    double fw3 = nx * s[1 * k + i] - ny * s[0 * k + i];
    s[0 * k + i] = Y02 * s[0 * k + i] - C02Y * fu1;
    s[1 * k + i] = Y02 * s[1 * k + i] - C02Y * fu2;
    s[2 * k + i] = Y02 * s[2 * k + i] - C02Y * fu3;
    s[3 * k + i] = Z02 * s[3 * k + i] - C02Z * fw1;
    s[4 * k + i] = Z02 * s[4 * k + i] - C02Z * fw2;
    s[5 * k + i] = Z02 * s[5 * k + i] - C02Z * fw3;
  }
}

/* cem_maxwell_flux3d (src/cem_maxwell.F:922-1002); userfsrc carries the
 * graphene currents when sheets are set (a no-op otherwise) */
void ref_flux3d(ref_ctx* c) {
  if (c->ndim == 2) { flux2d(c); return; }
  ref_flux_pre(c);
  if (c->ngraph && c->rkstep_now > 0) ref_graphene(c, c->rkstep_now, c->dt_now);
  ref_gs_op_fields(c, c->srflx, c->nxzfl, 6);
  if (c->ncempec > 0) ref_flux_pec(c);
  ref_flux_upwind(c);
}

/* cem_maxwell_add_flux_to_res, CPU branch (src/cem_maxwell.F:725-735).  The
 * serial loop adds face slots in increasing order; the element-parallel loop
 * below keeps that order because an element's slots are contiguous and only
 * touch that element's nodes. */
void ref_add_flux_to_res(ref_ctx* c) {
  if (c->ndim == 2) { lift_2d(c); return; }
  long k = c->nxzfl, np = c->npts, per = 6 * c->nxzf;
  double* s = c->srflx;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int e = 0; e < c->nelt; ++e)
    for (long j = per * e; j < per * (e + 1); ++j) {
      long i = c->cemface[j];
      double a = c->area[j];
      c->reshn[i + 0 * np] = c->reshn[i + 0 * np] + a * s[0 * k + j];
      c->reshn[i + 1 * np] = c->reshn[i + 1 * np] + a * s[1 * k + j];
      c->reshn[i + 2 * np] = c->reshn[i + 2 * np] + a * s[2 * k + j];
      c->resen[i + 0 * np] = c->resen[i + 0 * np] + a * s[3 * k + j];
      c->resen[i + 1 * np] = c->resen[i + 1 * np] + a * s[4 * k + j];
      c->resen[i + 2 * np] = c->resen[i + 2 * np] + a * s[5 * k + j];
    }
}

/* ------------------------------------------------------------------------ */
/* Dispersive media, called from usersrc (tests/drude/drude.usr:167,        */
/* tests/lorentz/lorentz.usr:174)                                           */
/* ------------------------------------------------------------------------ */

/* Drude and Lorentz parameters at the listed nodes (0-based); the currents,
 * their RK registers and residuals restart at zero (uservp, rzero) */
void ref_set_drude(ref_ctx* c, const double* params, const int* index, long n) {
  long np = c->npts;
  free(c->drudeparams); free(c->djn); free(c->dkjn); free(c->dresjn); free(c->drudeindex);
  c->drudeparams = dalloc(2 * np);
  memcpy(c->drudeparams, params, 2 * np * sizeof(double));
  c->djn = dalloc(3 * np); c->dkjn = dalloc(3 * np); c->dresjn = dalloc(3 * np);
  c->drudeindex = ialloc(n);
  memcpy(c->drudeindex, index, (size_t)n * sizeof(int));
  c->ndrude = n;
}

void ref_set_lorentz(ref_ctx* c, const double* params, const int* index, long n) {
  long np = c->npts;
  free(c->lorentzparams); free(c->ljn); free(c->lkjn); free(c->lresjn); free(c->lorentzindex);
  c->lorentzparams = dalloc(3 * np);
  memcpy(c->lorentzparams, params, 3 * np * sizeof(double));
  c->ljn = dalloc(6 * np); c->lkjn = dalloc(6 * np); c->lresjn = dalloc(6 * np);
  c->lorentzindex = ialloc(n);
  memcpy(c->lorentzindex, index, (size_t)n * sizeof(int));
  c->nlorentz = n;
}

/* cem_maxwell_drude (src/cem_maxwell.F:3095-3147): resE -= jn bm1,
 * resjn = -a jn + b en at the listed nodes, then rk4_upd of jn on all nodes */
static void drude_step(ref_ctx* c, int rkstep, double dt) {
  long np = c->npts;
  const double* pa = c->drudeparams;
  for (long i = 0; i < c->ndrude; ++i) {
    long j = c->drudeindex[i];
    double a = pa[j], b = pa[np + j];
    for (int q = 0; q < 3; ++q) {
      c->resen[j + q * np] = c->resen[j + q * np] - c->djn[j + q * np] * c->bm1[j];
      c->dresjn[j + q * np] = -a * c->djn[j + q * np] + b * c->en[j + q * np];
    }
  }
  double ra[5], rb[5], rc[6];
  ref_rk_coeffs(ra, rb, rc);
  for (int q = 0; q < 3; ++q)
    ref_rk4_upd(c->djn + q * np, c->dkjn + q * np, c->dresjn + q * np, rb[rkstep - 1],
                ra[rkstep - 1], dt, np);
}

/* cem_maxwell_lorentz (src/cem_maxwell.F:3149-3212): resE -= jn1 bm1,
 * resjn1 = -a jn1 - b jn2 + c en, resjn2 = jn1, then rk4_upd of both */
static void lorentz_step(ref_ctx* c, int rkstep, double dt) {
  long np = c->npts;
  const double* pa = c->lorentzparams;
  double* j1 = c->ljn;
  double* j2 = c->ljn + 3 * np;
  for (long i = 0; i < c->nlorentz; ++i) {
    long j = c->lorentzindex[i];
    double a = pa[j], b = pa[np + j], cc = pa[2 * np + j];
    for (int q = 0; q < 3; ++q) {
      c->resen[j + q * np] = c->resen[j + q * np] - j1[j + q * np] * c->bm1[j];
      c->lresjn[j + q * np] = -a * j1[j + q * np] - b * j2[j + q * np] + cc * c->en[j + q * np];
      c->lresjn[j + (3 + q) * np] = j1[j + q * np];
    }
  }
  double ra[5], rb[5], rc[6];
  ref_rk_coeffs(ra, rb, rc);
  for (int q = 0; q < 6; ++q)
    ref_rk4_upd(c->ljn + q * np, c->lkjn + q * np, c->lresjn + q * np, rb[rkstep - 1],
                ra[rkstep - 1], dt, np);
}

/* the dispersive currents inside usersrc, before the volume source */
void ref_dispersive(ref_ctx* c, int rkstep, double dt) {
  if (c->djn) drude_step(c, rkstep, dt);
  if (c->ljn) lorentz_step(c, rkstep, dt);
}

/* usersrc (src/cem_maxwell.F:503): mass-weighted E_z source; in the 2-D TE
 * form the out-of-plane H_z instead (tests/2dboxpml/2dboxpml.usr:28-100:
 * srchz in TE, srcez in TM) */
void ref_usersrc(ref_ctx* c, double rktime) {
  if (!c->src_w) return;
  /* kind 1: tests/3dboxpml/3dboxpml.usr:72-82, srcez - exp(..) * sin(-omega t) * bm1 */
  double ft = c->src_kind == 1 ? -c->src_amp * sin(-c->src_f0 * rktime)
                               : c->src_amp * ref_source_time(rktime, c->src_f0, c->src_t0);
  double* rez = (c->ndim == 2 && c->imode == 1 ? c->reshn : c->resen) + 2 * c->npts;
  for (long i = 0; i < c->npts; ++i) rez[i] = rez[i] + c->src_w[i] * ft;
}

/* cem_maxwell_invqmass, CPU branch (src/cem_maxwell.F:1878-1886) */
void ref_invqmass(ref_ctx* c) {
  if (c->ndim == 2) { invqmass_2d(c); return; }
  long np = c->npts;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (long i = 0; i < np; ++i) {
    for (int q = 0; q < 3; ++q) {
      c->reshn[i + q * np] = c->reshn[i + q * np] * c->hbm1[i];
      c->resen[i + q * np] = c->resen[i + q * np] * c->ebm1[i];
    }
  }
}

/* ------------------------------------------------------------------------ */
/* PML (src/cem_maxwell_pml.F)                                              */
/* ------------------------------------------------------------------------ */

/* slots of the negative / positive face of reference axis ax (pff order) */
static const int neg_slot[3] = {3, 0, 4};
static const int pos_slot[3] = {1, 2, 5};

/* gs_op(gsh_face, u, 1, 4 = max, 0): every entry of a face-node group
 * becomes the group's maximum (singletons unchanged) */
static void gs_max(ref_ctx* c, double* v) {
  for (int g = 0; g < c->gs_ngroups; ++g) {
    int b = c->gs_start[g], e = c->gs_start[g + 1];
    if (e - b < 2) continue;
    double m = v[c->gs_order[b]];
    for (int q = b + 1; q < e; ++q) m = v[c->gs_order[q]] > m ? v[c->gs_order[q]] : m;
    for (int q = b; q < e; ++q) v[c->gs_order[q]] = m;
  }
}

/* march_faces (src/cem_maxwell_pml.F:85-137) */
static void march_faces(ref_ctx* c, double* far) {
  long n2 = c->nxzf;
  const int nfc = c->nfaces;
  for (int e = 0; e < c->nelt; ++e)
    for (int ax = 0; ax < c->ndim; ++ax) {
      double* pf = far + n2 * (pos_slot[ax] + (long)nfc * e);
      double* nf = far + n2 * (neg_slot[ax] + (long)nfc * e);
      for (long i = 0; i < n2; ++i) {
        double sum = pf[i] + nf[i];
        if (sum != 0) { pf[i] = pf[i] + 1; nf[i] = nf[i] + 1; }
      }
    }
  gs_max(c, far);
}

void ref_set_pml(ref_ctx* c, int thick, double order, double referr) {
  const int n = c->n, nd = c->ndim, nfc = c->nfaces;
  const long n2 = c->nxzf, np = c->npts;
  const long n3 = nd == 3 ? (long)n * n * n : (long)n * n;  /* nodes per element */
  /* pml_fill_faceary (:139-190): ones at the interior nodes of 'PML' faces
   * (2-D: face nodes 2..lx1-1), then `thick` marches */
  double* far = dalloc(c->nxzfl);
  for (int e = 0; e < c->nelt; ++e)
    for (int f = 0; f < nfc; ++f)
      if (c->cbc[nfc * e + f] == 3) {
        if (nd == 3) {
          for (int b = 1; b < n - 1; ++b)
            for (int a = 1; a < n - 1; ++a) far[a + (long)n * b + n2 * (f + 6L * e)] = 1;
        } else {
          for (int a = 1; a < n - 1; ++a) far[a + n2 * (f + 4L * e)] = 1;
        }
      }
  for (int i = 0; i < thick; ++i) march_faces(c, far);

  /* pml_extent_and_tags (:261-431); extents in sym order (x-, x+, y-, ...) */
  const double inf = 1e20;
  for (int ax = 0; ax < 3; ++ax) {
    c->pmlouter[2 * ax] = inf;
    c->pmlinner[2 * ax] = -inf;
    c->pmlinner[2 * ax + 1] = inf;
    c->pmlouter[2 * ax + 1] = -inf;
  }
  free(c->pmltag);
  c->pmltag = ialloc(c->nelt);
  /* a face interior point: node (1,1) of the face in 3-D, node 2 (1-based) in 2-D */
  const long ind = nd == 3 ? 1 + (long)n : 1;
  const double* coord[3] = {c->xm1, c->ym1, c->zm1};
  const double* met[3][3] = {{c->rxm1, c->sxm1, c->txm1}, {c->rym1, c->sym1, c->tym1},
                             {c->rzm1, c->szm1, c->tzm1}};
  for (int e = 0; e < c->nelt; ++e)
    for (int ax = 0; ax < nd; ++ax) {
      double here = far[ind + n2 * (neg_slot[ax] + (long)nfc * e)];
      double opp = far[ind + n2 * (pos_slot[ax] + (long)nfc * e)];
      if (here == 0 || opp == 0) continue;
      /* dir_local_to_global (:192-259) of the local -ax direction */
      double loc[3] = {0, 0, 0}, glob[3];
      loc[ax] = -1;
      long v0 = n3 * e;
      for (int d = 0; d < 3; ++d)
        glob[d] = met[d][0][v0] * loc[0] + met[d][1][v0] * loc[1] + met[d][2][v0] * loc[2];
      double big = 0;
      int amax = 0;
      for (int d = 0; d < 3; ++d)
        if (fabs(glob[d]) >= big) { big = fabs(glob[d]); amax = d; }
      int globface = 2 * amax + (glob[amax] >= 0 ? 1 : 0);
      int ga = globface / 2;
      int gsign = (globface % 2) * 2 - 1;
      double mn = coord[ga][v0], mx = coord[ga][v0];
      for (long i = 1; i < n3; ++i) {
        double x = coord[ga][v0 + i];
        mn = x < mn ? x : mn;
        mx = x > mx ? x : mx;
      }
      if (gsign * (here - opp) > 0) { /* positive side */
        int fp = 2 * ga + 1;
        c->pmlinner[fp] = c->pmlinner[fp] < mn ? c->pmlinner[fp] : mn;
        c->pmlouter[fp] = c->pmlouter[fp] > mx ? c->pmlouter[fp] : mx;
        c->pmltag[e] |= 1 << fp;
      }
      if (gsign * (here - opp) < 0) { /* negative side */
        int fm = 2 * ga;
        c->pmlinner[fm] = c->pmlinner[fm] > mx ? c->pmlinner[fm] : mx;
        c->pmlouter[fm] = c->pmlouter[fm] < mn ? c->pmlouter[fm] : mn;
        c->pmltag[e] |= 1 << fm;
      }
    }
  free(far);

  /* pml_calc_sigma (:433-506) */
  free(c->pmlptr);
  c->pmlptr = ialloc(c->nelt);
  c->maxpml = 0;
  for (int e = 0; e < c->nelt; ++e)
    if (c->pmltag[e]) c->pmlptr[c->maxpml++] = e;
  double** arr[] = {&c->pmlsigma, &c->pmlbn, &c->pmldn, &c->kpmlbn, &c->kpmldn, &c->respmlbn,
                    &c->respmldn, &c->respmlhn, &c->respmlen};
  for (size_t i = 0; i < sizeof(arr) / sizeof(arr[0]); ++i) {
    free(*arr[i]);
    *arr[i] = dalloc(3 * np);
  }
  for (int l = 0; l < c->maxpml; ++l) {
    int e = c->pmlptr[l];
    for (int face = 0; face < 2 * nd; ++face) {
      int ax = face / 2;
      double width = fabs(c->pmlouter[face] - c->pmlinner[face]);
      if (!(c->pmltag[e] & (1 << face))) continue;
      for (long i = 0; i < n3; ++i) {
        long j = i + n3 * e;
        double eta = c->permeability[j] / c->permittivity[j];
        eta = sqrt(eta);
        double sigmamax = -(order + 1) * log(referr) / (2 * eta * width);
        double z2o = (coord[ax][j] - c->pmlinner[face]) / (c->pmlouter[face] - c->pmlinner[face]);
        c->pmlsigma[j + ax * np] = sigmamax * pow(z2o, order);
      }
    }
  }
  c->ifpml = 1;
}

/* pml_step (src/cem_maxwell_pml.F:508-590) */
void ref_pml_step(ref_ctx* c) {
  const long n3 = c->ndim == 3 ? (long)c->n * c->n * c->n : (long)c->n * c->n;
  const long np = c->npts;
  double *sg = c->pmlsigma, *bn = c->pmlbn, *dn = c->pmldn;
  double *rb = c->respmlbn, *rd = c->respmldn, *rh = c->respmlhn, *re = c->respmlen;
  double *hn = c->hn, *en = c->en, *rsh = c->reshn, *rse = c->resen;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int l = 0; l < c->maxpml; ++l) {
    long e = c->pmlptr[l];
    for (long i = 0; i < n3; ++i) {
      long j = i + n3 * e;
      double bm1inv = 1.0 / c->bm1[j];
      double sigx = sg[j], sigy = sg[j + np], sigz = sg[j + 2 * np];
      double sxp = sigx / c->permittivity[j];
      double syp = sigy / c->permittivity[j];
      double szp = sigz / c->permittivity[j];
      double permeab = c->permeability[j];
      rb[j] = rsh[j] * bm1inv - syp * bn[j];
      rb[j + np] = rsh[j + np] * bm1inv - szp * bn[j + np];
      rb[j + 2 * np] = rsh[j + 2 * np] * bm1inv - sxp * bn[j + 2 * np];
      rd[j] = rse[j] * bm1inv - syp * dn[j];
      rd[j + np] = rse[j + np] * bm1inv - szp * dn[j + np];
      rd[j + 2 * np] = rse[j + 2 * np] * bm1inv - sxp * dn[j + 2 * np];
      rh[j] = -syp * bn[j] + sxp * bn[j] - szp * permeab * hn[j];
      rh[j + np] = -szp * bn[j + np] + syp * bn[j + np] - sxp * permeab * hn[j + np];
      rh[j + 2 * np] = -sxp * bn[j + 2 * np] + szp * bn[j + 2 * np] - syp * permeab * hn[j + 2 * np];
      re[j] = -syp * dn[j] + sxp * dn[j] - sigz * en[j];
      re[j + np] = -szp * dn[j + np] + syp * dn[j + np] - sigx * en[j + np];
      re[j + 2 * np] = -sxp * dn[j + 2 * np] + szp * dn[j + 2 * np] - sigy * en[j + 2 * np];
      rsh[j] = rsh[j] + rh[j] * c->bm1[j];
      rsh[j + np] = rsh[j + np] + rh[j + np] * c->bm1[j];
      rsh[j + 2 * np] = rsh[j + 2 * np] + rh[j + 2 * np] * c->bm1[j];
      rse[j] = rse[j] + re[j] * c->bm1[j];
      rse[j + np] = rse[j + np] + re[j + np] * c->bm1[j];
      rse[j + 2 * np] = rse[j + 2 * np] + re[j + 2 * np] * c->bm1[j];
    }
  }
}

/* userinc (called by cem_maxwell_op between the restriction and the flux,
 * src/cem_maxwell.F:495-496) in the plane-wave form the reference's cases
 * use (tests/drude/drude.usr:7-42, tests/3dgraphene/3dgraphene.usr:7-50):
 * the face values of the listed slots get amp * cos(k.x - omega t). */
void ref_set_incident(ref_ctx* c, const int* slots, long n, const double amp[6],
                      const double k[3], double omega) {
  free(c->incslot);
  c->incslot = ialloc(n);
  memcpy(c->incslot, slots, (size_t)n * sizeof(int));
  c->ninc = n;
  for (int m = 0; m < 6; ++m) c->incamp[m] = amp[m];
  for (int m = 0; m < 3; ++m) c->inck[m] = k[m];
  c->incomega = omega;
}

void ref_userinc(ref_ctx* c, double rktime) {
  long nf = c->nxzfl;
  for (long q = 0; q < c->ninc; ++q) {
    long j = c->incslot[q];
    long i = c->cemface[j];
    double ph = c->inck[0] * c->xm1[i] + c->inck[1] * c->ym1[i] + c->inck[2] * c->zm1[i] -
                c->incomega * rktime;
    double u = cos(ph);
    for (int m = 0; m < 3; ++m) {
      c->fhn[j + m * nf] = c->fhn[j + m * nf] + c->incamp[m] * u;
      c->fen[j + m * nf] = c->fen[j + m * nf] + c->incamp[3 + m] * u;
    }
  }
}

/* cem_maxwell_op (src/cem_maxwell.F:484-508); userfsrc is a no-op */
void ref_maxwell_op(ref_ctx* c, double rktime) {
  ref_cem_maxwell(c);
  ref_restrict_to_face(c);
  if (c->ninc) ref_userinc(c, rktime);
  ref_flux3d(c);
  ref_add_flux_to_res(c);
  if (c->ifpml) ref_pml_step(c);
  if (c->rkstep_now > 0) ref_dispersive(c, c->rkstep_now, c->dt_now);
  ref_usersrc(c, rktime);
  ref_invqmass(c);
}

/* rk4_upd (src/cem_common.F:18-75): kh = ca*kh + dt*resh; h = h + cb*kh */
void ref_rk4_upd(double* h, double* kh, const double* resh, double cb, double ca, double dt,
                 long n) {
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (long i = 0; i < n; ++i) {
    kh[i] = ca * kh[i] + dt * resh[i];
    h[i] = h[i] + cb * kh[i];
  }
}

/* rk_storage, RK45 branch (src/cem_common.F:78-104) */
void ref_rk_coeffs(double a[5], double b[5], double c[6]) {
  a[0] = 0.0;
  a[1] = -567301805773.0 / 1357537059087.0;
  a[2] = -2404267990393.0 / 2016746695238.0;
  a[3] = -3550918686646.0 / 2091501179385.0;
  a[4] = -1275806237668.0 / 842570457699.0;
  b[0] = 1432997174477.0 / 9575080441755.0;
  b[1] = 5161836677717.0 / 13612068292357.0;
  b[2] = 1720146321549.0 / 2090206949498.0;
  b[3] = 3134564353537.0 / 4481467310338.0;
  b[4] = 2277821191437.0 / 14882151754819.0;
  c[0] = 0.0;
  c[1] = 1432997174477.0 / 9575080441755.0;
  c[2] = 2526269341429.0 / 6820363962896.0;
  c[3] = 2006345519317.0 / 3224310063776.0;
  c[4] = 2802321613138.0 / 2924317926251.0;
  c[5] = 1.0;
}

/* one stage: rk_c, cem_maxwell_op, rk_maxwell_ab (src/cem_maxwell.F:336-340,
 * src/cem_common.F:2-15, src/cem_maxwell.F:1906-1940) */
void ref_rk_stage(ref_ctx* c, int rkstep, double time, double dt) {
  double a[5], b[5], cc[6];
  ref_rk_coeffs(a, b, cc);
  double rktime = time + dt * cc[rkstep - 1];
  c->rkstep_now = rkstep;
  c->dt_now = dt;
  ref_maxwell_op(c, rktime);
  c->rkstep_now = 0;
  long np = c->npts;
  if (c->ndim == 2) { /* rk_maxwell_ab TM / TE branches (src/cem_maxwell.F:1925-1932) */
    double* u[3]; double* k[3]; double* r[3];
    int tm = c->imode == 2;
    u[0] = (tm ? c->hn : c->en); k[0] = (tm ? c->khn : c->ken); r[0] = (tm ? c->reshn : c->resen);
    u[1] = u[0] + np; k[1] = k[0] + np; r[1] = r[0] + np;
    u[2] = (tm ? c->en : c->hn) + 2 * np; k[2] = (tm ? c->ken : c->khn) + 2 * np;
    r[2] = (tm ? c->resen : c->reshn) + 2 * np;
    for (int q = 0; q < 3; ++q)
      ref_rk4_upd(u[q], k[q], r[q], b[rkstep - 1], a[rkstep - 1], dt, np);
  } else {
    for (int q = 0; q < 3; ++q)
      ref_rk4_upd(c->hn + q * np, c->khn + q * np, c->reshn + q * np, b[rkstep - 1],
                  a[rkstep - 1], dt, np);
    for (int q = 0; q < 3; ++q)
      ref_rk4_upd(c->en + q * np, c->ken + q * np, c->resen + q * np, b[rkstep - 1],
                  a[rkstep - 1], dt, np);
  }
  if (c->ifpml) { /* src/cem_maxwell.F:1942-1955 */
    for (int q = 0; q < 3; ++q)
      ref_rk4_upd(c->pmlbn + q * np, c->kpmlbn + q * np, c->respmlbn + q * np, b[rkstep - 1],
                  a[rkstep - 1], dt, np);
    for (int q = 0; q < 3; ++q)
      ref_rk4_upd(c->pmldn + q * np, c->kpmldn + q * np, c->respmldn + q * np, b[rkstep - 1],
                  a[rkstep - 1], dt, np);
  }
}

/* cem_maxwell_op_rk (src/cem_maxwell.F:327-345) */
void ref_op_rk(ref_ctx* c, double time, double dt) {
  for (int s = 1; s <= 5; ++s) ref_rk_stage(c, s, time, dt);
}

/* time loop body of time_advancing_pde (src/cem_drive.F:618-651) */
void ref_run(ref_ctx* c, int nsteps, double* time, double dt) {
  for (int s = 0; s < nsteps; ++s) {
    ref_op_rk(c, *time, dt);
    *time = *time + dt;
  }
}

/* get_dxmin (src/nek5_courant.F:2-75) */
double ref_get_dxmin(const ref_ctx* c) {
  int n = c->n;
  double d2m = 1.0e20;
  const double *x = c->xm1, *y = c->ym1, *z = c->zm1;
  if (c->ndim == 2) { /* the 2D branch */
    for (int e = 0; e < c->nelt; ++e)
      for (int j = 1; j < n - 1; ++j)
        for (int i = 1; i < n - 1; ++i) {
          long o = (long)n * n * e;
          double dx = x[o + i + 1 + n * j] - x[o + i - 1 + n * j];
          double dy = y[o + i + 1 + n * j] - y[o + i - 1 + n * j];
          double d2 = dx * dx + dy * dy;
          d2m = d2 < d2m ? d2 : d2m;
          dx = x[o + i + n * (j + 1)] - x[o + i + n * (j - 1)];
          dy = y[o + i + n * (j + 1)] - y[o + i + n * (j - 1)];
          d2 = dx * dx + dy * dy;
          d2m = d2 < d2m ? d2 : d2m;
        }
    return sqrt(d2m) / 2.0;
  }
#define IDX(i, j, k, e) ((long)(i) + (long)n * (j) + (long)n * n * (k) + (long)n * n * n * (e))
  for (int e = 0; e < c->nelt; ++e)
    for (int k = 1; k < n - 1; ++k)
      for (int j = 1; j < n - 1; ++j)
        for (int i = 1; i < n - 1; ++i) {
          double dx, dy, dz, d2;
          dx = x[IDX(i + 1, j, k, e)] - x[IDX(i - 1, j, k, e)];
          dy = y[IDX(i + 1, j, k, e)] - y[IDX(i - 1, j, k, e)];
          dz = z[IDX(i + 1, j, k, e)] - z[IDX(i - 1, j, k, e)];
          d2 = dx * dx + dy * dy + dz * dz;
          d2m = d2 < d2m ? d2 : d2m;
          dx = x[IDX(i, j + 1, k, e)] - x[IDX(i, j - 1, k, e)];
          dy = y[IDX(i, j + 1, k, e)] - y[IDX(i, j - 1, k, e)];
          dz = z[IDX(i, j + 1, k, e)] - z[IDX(i, j - 1, k, e)];
          d2 = dx * dx + dy * dy + dz * dz;
          d2m = d2 < d2m ? d2 : d2m;
          dx = x[IDX(i, j, k + 1, e)] - x[IDX(i, j, k - 1, e)];
          dy = y[IDX(i, j, k + 1, e)] - y[IDX(i, j, k - 1, e)];
          dz = z[IDX(i, j, k + 1, e)] - z[IDX(i, j, k - 1, e)];
          d2 = dx * dx + dy * dy + dz * dz;
          d2m = d2 < d2m ? d2 : d2m;
        }
#undef IDX
  return sqrt(d2m) / 2.0;
}

/* cem_error (src/cem_common.F:1335-1355): L2 = sqrt(sum e*bm1*e / volvm1) */
void ref_cem_error(const ref_ctx* c, const double* u, const double* exact, long n, double* l2,
                   double* linf) {
  double s = 0.0, m = 0.0;
  for (long i = 0; i < n; ++i) {
    double err = exact[i] - u[i];
    s = s + err * c->bm1[i] * err;
    double a = fabs(err);
    m = a > m ? a : m;
  }
  s = s / c->volvm1;
  if (s > 0.0) s = sqrt(s);
  *l2 = s;
  *linf = m;
}

/* ------------------------------------------------------------------------ */
/* 2-D TE / TM forms (imode 1 / 2): the ldim=2 branches of the routines     */
/* above, on a box of quadrilaterals                                         */
/* ------------------------------------------------------------------------ */

/* face slot f (0..3, pff order: s=-1, r=+1, s=+1, r=-1) node a -> volume
 * index within the element; SKPDAT walks every 2-D face in ascending
 * coordinate order (src/nek5_connect11.F:1483-1530 with NZ = 1) */
static int face_vol_2d(int f, int a, int n) {
  switch (f) {
    case 0: return a;
    case 1: return n - 1 + n * a;
    case 2: return a + n * (n - 1);
    default: return n * a;
  }
}

/* the three active components of the mode: TM (imode 2) H1, H2, E3;
 * TE (imode 1) E1, E2, H3 */
static void mode_fields(ref_ctx* c, double* base_h, double* base_e, long ld, double* out[3]) {
  if (c->imode == 2) {
    out[0] = base_h; out[1] = base_h + ld; out[2] = base_e + 2 * ld;
  } else {
    out[0] = base_e; out[1] = base_e + ld; out[2] = base_h + 2 * ld;
  }
}

/* maxwell_wght_curl, ldim = 2 (src/cem_maxwell.F:1500-1536) with
 * local_grad2 (src/nek5_grad.F:21-34) */
static void wght_curl_2d(ref_ctx* c, double* w1, double* w2, double* w3, const double* u1,
                         const double* u2, const double* u3) {
  int n = c->n;
  long n2 = (long)n * n;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int e = 0; e < c->nelt; ++e) {
    double u1r[256], u1s[256], u2r[256], u2s[256], u3r[256], u3s[256];
    long o = n2 * e;
    mxm(c->dxm1, n, u1 + o, n, u1r, n);
    mxm(u1 + o, n, c->dxtm1, n, u1s, n);
    mxm(c->dxm1, n, u2 + o, n, u2r, n);
    mxm(u2 + o, n, c->dxtm1, n, u2s, n);
    mxm(c->dxm1, n, u3 + o, n, u3r, n);
    mxm(u3 + o, n, c->dxtm1, n, u3s, n);
    for (long i = 0; i < n2; ++i) {
      long k = i + o;
      double u1rw = u1r[i] * c->w3m1[i], u1sw = u1s[i] * c->w3m1[i];
      double u2rw = u2r[i] * c->w3m1[i], u2sw = u2s[i] * c->w3m1[i];
      double u3rw = u3r[i] * c->w3m1[i], u3sw = u3s[i] * c->w3m1[i];
      double rx = c->rxm1[k], sx = c->sxm1[k], ry = c->rym1[k], sy = c->sym1[k];
      w1[k] = (u3rw * ry + u3sw * sy);
      w2[k] = -(u3rw * rx + u3sw * sx);
      w3[k] = (u2rw * rx + u2sw * sx - u1rw * ry - u1sw * sy);
    }
  }
}

/* cem_maxwell TM / TE branches (src/cem_maxwell.F:584-595) */
static void cem_maxwell_2d(ref_ctx* c) {
  long np = c->npts;
  double *u[3], *r[3];
  mode_fields(c, c->hn, c->en, np, u);
  mode_fields(c, c->reshn, c->resen, np, r);
  wght_curl_2d(c, r[0], r[1], r[2], u[0], u[1], u[2]);
  if (c->imode == 2) { /* chsign resHN(1,1), resHN(1,2) */
    for (long i = 0; i < np; ++i) { r[0][i] = -r[0][i]; r[1][i] = -r[1][i]; }
  } else { /* chsign resHN(1,3) */
    for (long i = 0; i < np; ++i) r[2][i] = -r[2][i];
  }
}

/* cem_maxwell_restrict_to_face TM / TE branches (src/cem_maxwell.F:616-637) */
static void restrict_2d(ref_ctx* c) {
  long np = c->npts, nf = c->nxzfl;
  for (long j = 0; j < nf; ++j) {
    long i = c->cemface[j];
    for (int q = 0; q < 3; ++q) { c->fhn[j + q * nf] = 0.0; c->fen[j + q * nf] = 0.0; }
    if (c->imode == 2) {
      c->fhn[j] = c->hn[i];
      c->fhn[j + nf] = c->hn[i + np];
      c->fen[j + 2 * nf] = c->en[i + 2 * np];
    } else {
      c->fhn[j + 2 * nf] = c->hn[i + 2 * np];
      c->fen[j] = c->en[i];
      c->fen[j + nf] = c->en[i + np];
    }
  }
}

/* cem_maxwell_flux2d (src/cem_maxwell.F:811-920) with gs_op_fields over 3
 * fields and the TM / TE branches of cem_maxwell_flux_pec (:1408-1421) */
static void flux2d(ref_ctx* c) {
  long k = c->nxzfl;
  double* s = c->srflx;
  double C0 = c->C0;
  const double *fh = c->fhn, *fe = c->fen;
  for (long i = 0; i < k; ++i) {
    double nx = c->unx[i], ny = c->uny[i];
    if (c->imode == 2) {
      s[0 * k + i] = -ny * fe[2 * k + i];
      s[1 * k + i] = nx * fe[2 * k + i];
      s[2 * k + i] = -nx * fh[1 * k + i] + ny * fh[0 * k + i];
    } else {
      s[0 * k + i] = -ny * fh[2 * k + i];
      s[1 * k + i] = nx * fh[2 * k + i];
      s[2 * k + i] = -nx * fe[1 * k + i] + ny * fe[0 * k + i];
    }
  }
  ref_gs_op_fields(c, s, k, 3);
  for (long j = 0; j < c->ncempec; ++j) {
    long i = c->cempec[j];
    if (c->imode == 2) {
      s[0 * k + i] = 2.0 * s[0 * k + i];
      s[1 * k + i] = 2.0 * s[1 * k + i];
      s[2 * k + i] = 0.0;
    } else {
      s[0 * k + i] = 0.0;
      s[1 * k + i] = 0.0;
      s[2 * k + i] = 2.0 * s[2 * k + i];
    }
  }
  for (long i = 0; i < k; ++i) {
    double Y0 = c->Y_0[i], Y1 = c->Y_1[i], Z0 = c->Z_0[i], Z1 = c->Z_1[i];
    double nx = c->unx[i], ny = c->uny[i];
    if (c->imode == 2) {
      double fu1 = ny * s[2 * k + i];
      double fu2 = -nx * s[2 * k + i];
      double fw3 = nx * s[1 * k + i] - ny * s[0 * k + i];
      s[0 * k + i] = 0.5 / Y0 * (-Y1 * s[0 * k + i] - C0 * fu1);
      s[1 * k + i] = 0.5 / Y0 * (-Y1 * s[1 * k + i] - C0 * fu2);
      s[2 * k + i] = 0.5 / Z0 * (Z1 * s[2 * k + i] - C0 * fw3);
    } else {
      double fw1 = ny * s[2 * k + i];
      double fw2 = -nx * s[2 * k + i];
      double fu3 = nx * s[1 * k + i] - ny * s[0 * k + i];
      s[0 * k + i] = 0.5 / Z0 * (Z1 * s[0 * k + i] - C0 * fw1);
      s[1 * k + i] = 0.5 / Z0 * (Z1 * s[1 * k + i] - C0 * fw2);
      s[2 * k + i] = 0.5 / Y0 * (-Y1 * s[2 * k + i] - C0 * fu3);
    }
  }
}

/* cem_maxwell_add_flux_to_res TM / TE branches (src/cem_maxwell.F:736-755) */
static void lift_2d(ref_ctx* c) {
  long k = c->nxzfl, np = c->npts;
  double* s = c->srflx;
  double* r[3];
  mode_fields(c, c->reshn, c->resen, np, r);
  for (long j = 0; j < k; ++j) {
    long i = c->cemface[j];
    double a = c->area[j];
    r[0][i] = r[0][i] + a * s[0 * k + j];
    r[1][i] = r[1][i] + a * s[1 * k + j];
    r[2][i] = r[2][i] + a * s[2 * k + j];
  }
}

/* cem_maxwell_invqmass TM / TE branches (src/cem_maxwell.F:1887-1898) */
static void invqmass_2d(ref_ctx* c) {
  long np = c->npts;
  for (long i = 0; i < np; ++i) {
    if (c->imode == 2) {
      c->reshn[i] = c->reshn[i] * c->hbm1[i];
      c->reshn[i + np] = c->reshn[i + np] * c->hbm1[i];
      c->resen[i + 2 * np] = c->resen[i + 2 * np] * c->ebm1[i];
    } else {
      c->resen[i] = c->resen[i] * c->ebm1[i];
      c->resen[i + np] = c->resen[i + np] * c->ebm1[i];
      c->reshn[i + 2 * np] = c->reshn[i + 2 * np] * c->hbm1[i];
    }
  }
}

/* A box [lo,hi]^2 of nelx x nely quadrilaterals, N <= 15, for imode 1 (TE)
 * or 2 (TM): GENWZ, genxyz (bilinear corner map), XYZRST + GLMAPM1 ldim=2
 * (src/nek5_coef.F:555-613), bm1 = jac w3, AREA2 (:1020-1095) and the 2-D
 * face numbering of cem_set_fc_ptr. */
ref_ctx* ref_create_box2d(int N, int nelx, int nely, const double lo[2], const double hi[2],
                          const int bc[2], int imode) {
  if (N < 1 || N > 15 || nelx < 1 || nely < 1 || (imode != 1 && imode != 2)) return NULL;
  ref_ctx* c = (ref_ctx*)calloc(1, sizeof(ref_ctx));
  int n = N + 1;
  c->N = N; c->n = n;
  c->ndim = 2; c->imode = imode; c->nfaces = 4;
  c->nel[0] = nelx; c->nel[1] = nely; c->nel[2] = 1;
  c->nelt = nelx * nely;
  for (int d = 0; d < 2; ++d) { c->lo[d] = lo[d]; c->hi[d] = hi[d]; c->bc[d] = bc[d]; }
  c->lo[2] = 0.0; c->hi[2] = 0.0; c->bc[2] = REF_BC_PERIODIC;
  long n2 = (long)n * n;
  c->npts = n2 * c->nelt;
  c->nxzf = n;
  c->nxzfl = 4L * n * c->nelt;
  long npts = c->npts, nxzfl = c->nxzfl;

  c->zgm1 = dalloc(n); c->wxm1 = dalloc(n);
  c->dxm1 = dalloc(n * n); c->dxtm1 = dalloc(n * n);
  c->w3m1 = dalloc(n2);
  ref_zwgll(c->zgm1, c->wxm1, n);
  ref_dgll(c->dxm1, c->dxtm1, c->zgm1, n);
  for (int iy = 0; iy < n; ++iy)
    for (int ix = 0; ix < n; ++ix) c->w3m1[ix + n * iy] = c->wxm1[ix] * c->wxm1[iy];

  c->xm1 = dalloc(npts); c->ym1 = dalloc(npts); c->zm1 = dalloc(npts);
  for (int e = 0; e < c->nelt; ++e) {
    int ec[2] = {e % nelx, e / nelx};
    double cb[2][2];
    for (int d = 0; d < 2; ++d) {
      double L = c->hi[d] - c->lo[d];
      cb[d][0] = c->lo[d] + L * (double)ec[d] / (double)c->nel[d];
      cb[d][1] = c->lo[d] + L * (double)(ec[d] + 1) / (double)c->nel[d];
    }
    double h[16][2];
    for (int i = 0; i < n; ++i) {
      h[i][0] = (1.0 - c->zgm1[i]) * 0.5;
      h[i][1] = (1.0 + c->zgm1[i]) * 0.5;
    }
    for (int iyt = 0; iyt < 2; ++iyt)
      for (int ixt = 0; ixt < 2; ++ixt)
        for (int j = 0; j < n; ++j)
          for (int i = 0; i < n; ++i) {
            double hh = h[i][ixt] * h[j][iyt];
            long idx = i + (long)n * j + n2 * e;
            c->xm1[idx] = c->xm1[idx] + hh * cb[0][ixt];
            c->ym1[idx] = c->ym1[idx] + hh * cb[1][iyt];
          }
  }

  double *xr = dalloc(npts), *yr = dalloc(npts), *xs = dalloc(npts), *ys = dalloc(npts);
  for (int e = 0; e < c->nelt; ++e) {
    long o = n2 * e;
    mxm(c->dxm1, n, c->xm1 + o, n, xr + o, n);
    mxm(c->xm1 + o, n, c->dxtm1, n, xs + o, n);
    mxm(c->dxm1, n, c->ym1 + o, n, yr + o, n);
    mxm(c->ym1 + o, n, c->dxtm1, n, ys + o, n);
  }
  c->rxm1 = dalloc(npts); c->rym1 = dalloc(npts); c->rzm1 = dalloc(npts);
  c->sxm1 = dalloc(npts); c->sym1 = dalloc(npts); c->szm1 = dalloc(npts);
  c->txm1 = dalloc(npts); c->tym1 = dalloc(npts); c->tzm1 = dalloc(npts);
  c->jacm1 = dalloc(npts); c->bm1 = dalloc(npts);
  for (long i = 0; i < npts; ++i) {
    double jac = 0.0;
    jac = jac + xr[i] * ys[i];
    jac = jac - xs[i] * yr[i];
    c->jacm1[i] = jac;
    c->rxm1[i] = ys[i];
    c->rym1[i] = -xs[i];
    c->sxm1[i] = -yr[i];
    c->sym1[i] = xr[i];
    c->tzm1[i] = 1.0;
  }
  for (int e = 0; e < c->nelt; ++e)
    for (long i = 0; i < n2; ++i) c->bm1[n2 * e + i] = c->jacm1[n2 * e + i] * c->w3m1[i];
  c->volvm1 = 0.0;
  for (long i = 0; i < npts; ++i) c->volvm1 += c->bm1[i];

  /* AREA2 with SETWGTR (non-axisymmetric: the GLL weights) */
  c->unx = dalloc(nxzfl); c->uny = dalloc(nxzfl); c->unz = dalloc(nxzfl); c->area = dalloc(nxzfl);
  for (int e = 0; e < c->nelt; ++e)
    for (int f = 0; f < 4; ++f)
      for (int a = 0; a < n; ++a) {
        long v = n2 * e + face_vol_2d(f, a, n);
        long j = a + (long)n * (f + 4L * e);
        double tx, ty, len;
        if (f == 0 || f == 2) { /* "S": xr, yr */
          len = sqrt(xr[v] * xr[v] + yr[v] * yr[v]);
          tx = xr[v] / len;
          ty = yr[v] / len;
          if (f == 2) { tx = -xr[v] / len; ty = -yr[v] / len; }
        } else { /* "R": xs, ys */
          len = sqrt(xs[v] * xs[v] + ys[v] * ys[v]);
          tx = xs[v] / len;
          ty = ys[v] / len;
          if (f == 3) { tx = -xs[v] / len; ty = -ys[v] / len; }
        }
        c->unx[j] = ty;
        c->uny[j] = -tx;
        c->area[j] = len * c->wxm1[a];
      }
  free(xr); free(yr); free(xs); free(ys);

  /* cem_set_fc_ptr and the face pairing (one id per face-node position;
   * periodic axes wrap) */
  c->cemface = ialloc(nxzfl);
  c->glo_face = (long long*)calloc((size_t)nxzfl, sizeof(long long));
  c->cbc = ialloc(4L * c->nelt);
  long long yoff = (long long)(nelx + 1) * nely;
  for (int e = 0; e < c->nelt; ++e) {
    int ec[2] = {e % nelx, e / nelx};
    for (int f = 0; f < 4; ++f) {
      int ax = slot_axis[f], sd = slot_side[f];
      int plane = ec[ax] + (sd > 0 ? 1 : 0);
      int boundary = (plane == 0 || plane == c->nel[ax]);
      if (boundary)
        c->cbc[4 * e + f] = c->bc[ax] == REF_BC_PERIODIC ? 2 : (c->bc[ax] == REF_BC_PML ? 3 : 1);
      if (boundary && c->bc[ax] == REF_BC_PERIODIC) plane = plane % c->nel[ax];
      long long fid = ax == 0 ? (long long)plane * nely + ec[1]
                              : yoff + (long long)plane * nelx + ec[0];
      for (int a = 0; a < n; ++a) {
        long j = a + (long)n * (f + 4L * e);
        c->cemface[j] = (int)(n2 * e + face_vol_2d(f, a, n));
        c->glo_face[j] = fid * (long long)n + a + 1;
      }
    }
  }
  gs_setup_local(c);
  c->cempec = ialloc(nxzfl);
  long l = 0;
  for (int e = 0; e < c->nelt; ++e)  /* 'PEC' and 'PML' faces (cem_maxwell_pec_init) */
    for (int f = 0; f < 4; ++f)
      if (c->cbc[4 * e + f] == 1 || c->cbc[4 * e + f] == 3)
        for (long j = 0; j < n; ++j) c->cempec[l++] = (int)(j + (long)n * (f + 4L * e));
  c->ncempec = l;

  c->hn = dalloc(3 * npts); c->en = dalloc(3 * npts);
  c->khn = dalloc(3 * npts); c->ken = dalloc(3 * npts);
  c->reshn = dalloc(3 * npts); c->resen = dalloc(3 * npts);
  c->fhn = dalloc(3 * nxzfl); c->fen = dalloc(3 * nxzfl);
  c->srflx = dalloc(6 * nxzfl);
  c->permittivity = dalloc(npts); c->permeability = dalloc(npts);
  c->impede = dalloc(npts); c->conduc = dalloc(npts);
  c->zimpede = dalloc(nxzfl); c->yconduc = dalloc(nxzfl);
  c->Z_0 = dalloc(nxzfl); c->Z_1 = dalloc(nxzfl); c->Y_0 = dalloc(nxzfl); c->Y_1 = dalloc(nxzfl);
  c->ebm1 = dalloc(npts); c->hbm1 = dalloc(npts);
  c->C0 = 1.0;
  double* one = dalloc(npts);
  for (long i = 0; i < npts; ++i) one[i] = 1.0;
  ref_set_materials(c, one, one);
  free(one);
  return c;
}

int ref_ndim(const ref_ctx* c) { return c->ndim; }
int ref_imode(const ref_ctx* c) { return c->imode; }

/* ------------------------------------------------------------------------ */
/* Dealiased curl (maxwell_wght_dcurl, src/cem_maxwell.F:1541-1729)          */
/* ------------------------------------------------------------------------ */

/* fd_weights_full (src/nek5_coef.F:1804-1857): Fornberg's finite-difference
 * weights c(j,k) at xx for the points x(0:n), derivatives 0..m.  c holds
 * (n+1)*(m+1) values, c[j + (n+1)*k]. */
static void fd_weights(double xx, const double* x, int n, int m, double* c) {
  int np = n + 1;
  double c1 = 1.0, c4 = x[0] - xx;
  for (int k = 0; k <= m; ++k)
    for (int j = 0; j <= n; ++j) c[j + np * k] = 0.0;
  c[0] = 1.0;
  for (int i = 1; i <= n; ++i) {
    int mn = i < m ? i : m;
    double c2 = 1.0, c5 = c4;
    c4 = x[i] - xx;
    for (int j = 0; j < i; ++j) {
      double c3 = x[i] - x[j];
      c2 = c2 * c3;
      if (j == i - 1) {
        for (int k = mn; k >= 1; --k)
          c[i + np * k] = c1 * ((double)k * c[i - 1 + np * (k - 1)] - c5 * c[i - 1 + np * k]) / c2;
        c[i] = -c1 * c5 * c[i - 1] / c2;
      }
      for (int k = mn; k >= 1; --k)
        c[j + np * k] = (c4 * c[j + np * k] - (double)k * c[j + np * (k - 1)]) / c3;
      c[j] = c4 * c[j] / c3;
    }
    c1 = c2;
  }
}

/* specmpn (src/cem_common.F:418-460): tensor-product interpolation from
 * na^3 to nb^3 with ba (nb x na) and ab (na x nb) */
static void specmpn3(double* b, int nb, const double* a, int na, const double* ba,
                     const double* ab) {
  double* w1 = dalloc((long)nb * na * na);
  double* w2 = dalloc((long)nb * nb * na);
  mxm(ba, nb, a, na, w1, na * na);
  for (int iz = 0; iz < na; ++iz)
    mxm(w1 + (long)nb * na * iz, nb, ab, na, w2 + (long)nb * nb * iz, nb);
  mxm(w2, nb * nb, ab, na, b, nb);
  free(w1); free(w2);
}

/* the tables of maxwell_wght_dcurl's first call: gen_int (src/cem_common.F:
 * 584-617, GLL mx -> GLL md), gen_dgl (:619-674), w3md and the metrics
 * interpolated with intp_rstd; md = 0 switches the dealiased curl off */
int ref_set_dealias(ref_ctx* c, int md) {
  free(c->jgl); free(c->jgt); free(c->dxmd); free(c->dxtmd); free(c->w3md); free(c->metd);
  c->jgl = c->jgt = c->dxmd = c->dxtmd = c->w3md = c->metd = NULL;
  c->md = 0;
  if (md == 0) return 0;
  int mx = c->n;
  if (c->ndim != 3 || md < mx || md > 32) return -1;
  double *zx = dalloc(mx), *wx = dalloc(mx), *zd = dalloc(md), *wd = dalloc(md);
  double* cw = dalloc(2L * (md > mx ? md : mx));
  ref_zwgll(zx, wx, mx);
  ref_zwgll(zd, wd, md);
  c->jgl = dalloc((long)md * mx); c->jgt = dalloc((long)md * mx);
  for (int i = 0; i < md; ++i) {
    fd_weights(zd[i], zx, mx - 1, 0, cw);
    for (int j = 0; j < mx; ++j) c->jgl[i + (long)md * j] = cw[j];
  }
  for (int j = 0; j < mx; ++j)
    for (int i = 0; i < md; ++i) c->jgt[j + (long)mx * i] = c->jgl[i + (long)md * j];
  c->dxmd = dalloc((long)md * md); c->dxtmd = dalloc((long)md * md);
  for (int i = 0; i < md; ++i) {
    fd_weights(zd[i], zd, md - 1, 1, cw);
    for (int j = 0; j < md; ++j) c->dxmd[i + (long)md * j] = cw[md + j];
  }
  for (int j = 0; j < md; ++j)
    for (int i = 0; i < md; ++i) c->dxtmd[j + (long)md * i] = c->dxmd[i + (long)md * j];
  long md3 = (long)md * md * md, mx3 = (long)mx * mx * mx;
  c->w3md = dalloc(md3);
  for (int k = 0; k < md; ++k)
    for (int j = 0; j < md; ++j)
      for (int i = 0; i < md; ++i) c->w3md[i + md * j + (long)md * md * k] = wd[i] * wd[j] * wd[k];
  c->metd = dalloc(9 * md3 * c->nelt);
  const double* mt[9] = {c->rxm1, c->rym1, c->rzm1, c->sxm1, c->sym1, c->szm1,
                         c->txm1, c->tym1, c->tzm1};
  for (int q = 0; q < 9; ++q)
    for (int e = 0; e < c->nelt; ++e)
      specmpn3(c->metd + md3 * (c->nelt * (long)q + e), md, mt[q] + mx3 * e, mx, c->jgl, c->jgt);
  free(zx); free(wx); free(zd); free(wd); free(cw);
  c->md = md;
  return 0;
}

/* maxwell_wght_dcurl, ldim = 3: (w1,w2,w3) = B curl(u1,u2,u3) evaluated on
 * the md^3 points and projected back with the transposed interpolation */
void ref_wght_dcurl(ref_ctx* c, double* w1, double* w2, double* w3, const double* u1,
                    const double* u2, const double* u3) {
  int mx = c->n, md = c->md;
  long mx3 = (long)mx * mx * mx, md3 = (long)md * md * md, md2 = (long)md * md;
  long nm = md3 * c->nelt;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int e = 0; e < c->nelt; ++e) {
    double *ju[3], *g[9], *wdd[3];
    for (int q = 0; q < 3; ++q) { ju[q] = dalloc(md3); wdd[q] = dalloc(md3); }
    for (int q = 0; q < 9; ++q) g[q] = dalloc(md3);
    const double* u[3] = {u1 + mx3 * e, u2 + mx3 * e, u3 + mx3 * e};
    for (int q = 0; q < 3; ++q) {
      specmpn3(ju[q], md, u[q], mx, c->jgl, c->jgt);
      mxm(c->dxmd, md, ju[q], md, g[3 * q], (int)md2);
      for (int k = 0; k < md; ++k)
        mxm(ju[q] + md2 * k, md, c->dxtmd, md, g[3 * q + 1] + md2 * k, md);
      mxm(ju[q], (int)md2, c->dxtmd, md, g[3 * q + 2], md);
    }
    const double* M = c->metd;
    for (long i = 0; i < md3; ++i) {
      long k = i + md3 * e;
      double w = c->w3md[i];
      double u1rw = g[0][i] * w, u1sw = g[1][i] * w, u1tw = g[2][i] * w;
      double u2rw = g[3][i] * w, u2sw = g[4][i] * w, u2tw = g[5][i] * w;
      double u3rw = g[6][i] * w, u3sw = g[7][i] * w, u3tw = g[8][i] * w;
      double rx = M[k], ry = M[nm + k], rz = M[2 * nm + k];
      double sx = M[3 * nm + k], sy = M[4 * nm + k], sz = M[5 * nm + k];
      double tx = M[6 * nm + k], ty = M[7 * nm + k], tz = M[8 * nm + k];
      wdd[0][i] = u3rw * ry + u3sw * sy + u3tw * ty - u2rw * rz - u2sw * sz - u2tw * tz;
      wdd[1][i] = u1rw * rz + u1sw * sz + u1tw * tz - u3rw * rx - u3sw * sx - u3tw * tx;
      wdd[2][i] = u2rw * rx + u2sw * sx + u2tw * tx - u1rw * ry - u1sw * sy - u1tw * ty;
    }
    double* out[3] = {w1 + mx3 * e, w2 + mx3 * e, w3 + mx3 * e};
    for (int q = 0; q < 3; ++q) specmpn3(out[q], mx, wdd[q], md, c->jgt, c->jgl);
    for (int q = 0; q < 3; ++q) { free(ju[q]); free(wdd[q]); }
    for (int q = 0; q < 9; ++q) free(g[q]);
  }
}

/* ------------------------------------------------------------------------ */
/* Graphene sheets (cem_3d_graphene_current, src/cem_maxwell.F:2827-2931,   */
/* called through userfsrc, tests/3dgraphene/3dgraphene.usr:236-264)        */
/* ------------------------------------------------------------------------ */

void ref_set_graphene(ref_ctx* c, const double* params, const int* slots, long n) {
  long nf = c->nxzfl;
  free(c->graphindex); free(c->graphparams); free(c->fjn); free(c->kfjn); free(c->resfjn);
  c->graphindex = ialloc(n);
  memcpy(c->graphindex, slots, (size_t)n * sizeof(int));
  c->graphparams = dalloc(12 * nf);
  memcpy(c->graphparams, params, 12 * nf * sizeof(double));
  c->fjn = dalloc(18 * nf); c->kfjn = dalloc(18 * nf); c->resfjn = dalloc(18 * nf);
  c->ngraph = n;
}

/* the surface current of the listed face nodes from the face fields, the
 * residuals of its auxiliary (Drude and two critical-point) currents, their
 * rk4_upd, and userfsrc's -J on the -n x H part of srflx (before the gs sum) */
void ref_graphene(ref_ctx* c, int rkstep, double dt) {
  long nf = c->nxzfl;
#define FJ(arr, j, comp, k) arr[(j) + nf * ((comp) + 3 * (k))]
  const double *fh = c->fhn, *fe = c->fen;
  for (long q = 0; q < c->ngraph; ++q) {
    long j = c->graphindex[q];
    const double* p = c->graphparams;
    double a_d = p[j], b_d = p[nf + j], b_cp1 = p[2 * nf + j], a_211 = p[3 * nf + j];
    double a_221 = p[4 * nf + j], b_11 = p[5 * nf + j], b_21 = p[6 * nf + j];
    double b_cp2 = p[7 * nf + j], a_212 = p[8 * nf + j], a_222 = p[9 * nf + j];
    double b_12 = p[10 * nf + j], b_22 = p[11 * nf + j];
    double ux = c->unx[j], uy = c->uny[j], uz = c->unz[j];
    double nH[3], nEn[3];
    nH[0] = -uy * fh[2 * nf + j] + uz * fh[nf + j];
    nH[1] = ux * fh[2 * nf + j] - uz * fh[j];
    nH[2] = -ux * fh[nf + j] + uy * fh[j];
    double ndotE = ux * fe[j] + uy * fe[nf + j] + uz * fe[2 * nf + j];
    nEn[0] = fe[j] - ux * ndotE;
    nEn[1] = fe[nf + j] - uy * ndotE;
    nEn[2] = fe[2 * nf + j] - uz * ndotE;
    double Yfac = 0.5 / c->Y_0[j];
    double cpfac = b_cp1 + b_cp2;
    double jnfac = 1.0 - cpfac * Yfac;
    for (int m = 0; m < 3; ++m) {
      double tmp = Yfac * (nH[m] + c->yconduc[j] * nEn[m]);
      FJ(c->fjn, j, m, 0) = (FJ(c->fjn, j, m, 1) + FJ(c->fjn, j, m, 2) + FJ(c->fjn, j, m, 4) -
                             cpfac * tmp) / jnfac;
      double f = tmp - Yfac * FJ(c->fjn, j, m, 0);
      FJ(c->resfjn, j, m, 1) = -a_d * FJ(c->fjn, j, m, 1) + b_d * f;
      FJ(c->resfjn, j, m, 2) = FJ(c->fjn, j, m, 3) + b_11 * f;
      FJ(c->resfjn, j, m, 3) = -a_211 * FJ(c->fjn, j, m, 2) - a_221 * FJ(c->fjn, j, m, 3) + b_21 * f;
      FJ(c->resfjn, j, m, 4) = FJ(c->fjn, j, m, 5) + b_12 * f;
      FJ(c->resfjn, j, m, 5) = -a_212 * FJ(c->fjn, j, m, 4) - a_222 * FJ(c->fjn, j, m, 5) + b_22 * f;
    }
  }
  double ra[5], rb[5], rc[6];
  ref_rk_coeffs(ra, rb, rc);
  for (int k = 1; k < 6; ++k)
    for (int m = 0; m < 3; ++m)
      ref_rk4_upd(&FJ(c->fjn, 0, m, k), &FJ(c->kfjn, 0, m, k), &FJ(c->resfjn, 0, m, k),
                  rb[rkstep - 1], ra[rkstep - 1], dt, nf);
  double* s = c->srflx;
  for (long q = 0; q < c->ngraph; ++q) {
    long j = c->graphindex[q];
    for (int m = 0; m < 3; ++m) s[(3 + m) * nf + j] = s[(3 + m) * nf + j] - FJ(c->fjn, j, m, 0);
  }
#undef FJ
}

