/*
 * c_driver.c -- a compiled caller of the C ABI laid out like NekCEM's own
 * driver, so the boundary is exercised the way the Fortran side would use it.
 *
 *   - Static, COMMON-style arrays sized by a SIZE-like lpts1 larger than the
 *     mesh's npts (src/EMWAVE: hn(lpts1,3), en(lpts1,3)), 3-vectors stored
 *     component after component with leading dimension LPTS1.
 *   - The static geometry/material arrays that cem_maxwell_init leaves
 *     (src/cem_maxwell.F:65-191) handed to nekgpu_init through nekgpu_mesh.
 *     Here they come from the library's host-side box builder
 *     (nekgpu_box_export_*), standing in for genbox + cem_maxwell_init.
 *   - The time loop of time_advancing_pde (src/cem_drive.F:618-651): the
 *     step call, then `time = time + dt` by the caller, then userchk, which
 *     reads the fields back (nekgpu_get_state) and takes cem_error norms
 *     (nekgpu_norms) against the case's exact solution at `time`.
 *
 * The case is the reference's tests/3dboxpec (27 elements, N=8, [-1,1]^3,
 * PEC, dt = 0.005; usersol of tests/3dboxpec/3dboxpec.usr:64-119), optionally
 * with the library's Gaussian/Ricker E_z volume source, whose stage times
 * depend on the time the driver passes in.
 *
 * usage: c_driver FORM PATH NSTEPS IOCOMM SOURCE OUTFILE
 *   FORM   0 plain, 1 fused FP64, 2 mixed
 *   PATH   step (nekgpu_step on a copy of time, device-resident state)
 *          host (nekgpu_op_rk_host on the static arrays, page-locked once)
 *   SOURCE 0 | 1
 * Prints "final_time <t>" and one "chk" line per userchk with the norms;
 * writes hn(1:npts,1:3) then en(1:npts,1:3) (doubles) to OUTFILE.
 * Exit status 0, or 2 with the library's message when a call fails.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "nekcem_gpu.h"

#define LX1 9
#define LELT 32
#define LPTS1 (LX1 * LX1 * LX1 * LELT)
#define LXZFL (6 * LX1 * LX1 * LELT)

/* /maxwellv/: fields and the exact solution of userchk */
static double hn[3 * LPTS1], en[3 * LPTS1];
static double shn[3 * LPTS1], sen[3 * LPTS1];
/* /GEOM/, /EMWAVE/ static arrays */
static double dxm1[LX1 * LX1], w3mn[LX1 * LX1 * LX1];
static double xmn[LPTS1], ymn[LPTS1], zmn[LPTS1], bmn[LPTS1];
static double rxmn[LPTS1], rymn[LPTS1], rzmn[LPTS1], sxmn[LPTS1], symn[LPTS1], szmn[LPTS1],
    txmn[LPTS1], tymn[LPTS1], tzmn[LPTS1];
static double ebm1[LPTS1], hbm1[LPTS1];
static double unxm[LXZFL], unym[LXZFL], unzm[LXZFL], aream[LXZFL];
static double Z_0[LXZFL], Z_1[LXZFL], Y_0[LXZFL], Y_1[LXZFL];
static int cemface[LXZFL], cempec[LXZFL];
static long long glo_face[LXZFL], ibuf[LXZFL];

static long npts;
static nekgpu_ctx* ctx;

static void check(int st, const char* what) {
  if (st != NEKGPU_OK) {
    fprintf(stderr, "c_driver: %s: %s (%d)\n", what, nekgpu_error_string(st), st);
    if (ctx) nekgpu_finalize(ctx);
    exit(2);
  }
}

static void export_d(const nekgpu_box* b, const char* name, double* out, long want) {
  long n = 0;
  check(nekgpu_box_export_d(b, name, out, &n), name);
  if (n != want) {
    fprintf(stderr, "c_driver: %s has %ld entries, expected %ld\n", name, n, want);
    exit(2);
  }
}

static void export_i(const nekgpu_box* b, const char* name, int* out32, long long* out64,
                     long* count) {
  check(nekgpu_box_export_i(b, name, ibuf, count), name);
  for (long i = 0; i < *count; ++i) {
    if (out32) out32[i] = (int)ibuf[i];
    if (out64) out64[i] = ibuf[i];
  }
}

/* usersol of tests/3dboxpec/3dboxpec.usr:64-119 at time t */
static void usersol(double t) {
  const double ww = 3.14159265358979323846; /* pi */
  const double tmph = cos(ww * sqrt(3.0) * t) / sqrt(6.0);
  const double tmpe = sin(ww * sqrt(3.0) * t) / sqrt(2.0);
  for (long i = 0; i < npts; ++i) {
    const double sx = sin(ww * xmn[i]), cx = cos(ww * xmn[i]);
    const double sy = sin(ww * ymn[i]), cy = cos(ww * ymn[i]);
    const double sz = sin(ww * zmn[i]), cz = cos(ww * zmn[i]);
    shn[i] = -sx * cy * cz * tmph;
    shn[i + LPTS1] = -cx * sy * cz * tmph;
    shn[i + 2 * LPTS1] = 2.0 * cx * cy * sz * tmph;
    sen[i] = -cx * sy * sz * tmpe;
    sen[i + LPTS1] = sx * cy * sz * tmpe;
    sen[i + 2 * LPTS1] = 0.0;
  }
}

int main(int argc, char** argv) {
  if (argc != 7) {
    fprintf(stderr, "usage: c_driver FORM step|host NSTEPS IOCOMM SOURCE OUTFILE\n");
    return 1;
  }
  const int form = atoi(argv[1]);
  const int host_path = strcmp(argv[2], "host") == 0;
  const int nsteps = atoi(argv[3]), iocomm = atoi(argv[4]), use_source = atoi(argv[5]);

  /* genbox + cem_maxwell_init stand-in: the 3dboxpec mesh */
  nekgpu_box b;
  memset(&b, 0, sizeof b);
  b.N = LX1 - 1;
  b.nelx = b.nely = b.nelz = 3;
  for (int d = 0; d < 3; ++d) {
    b.lo[d] = -1.0;
    b.hi[d] = 1.0;
    b.bc[d] = NEKGPU_BC_PEC;
  }
  b.C0 = 1.0;
  const int nelt = b.nelx * b.nely * b.nelz;
  npts = (long)LX1 * LX1 * LX1 * nelt;
  const long nxzfl = 6L * LX1 * LX1 * nelt;
  if (nelt > LELT) return 1;
  export_d(&b, "dxm1", dxm1, LX1 * LX1);
  export_d(&b, "w3mn", w3mn, LX1 * LX1 * LX1);
  export_d(&b, "bmn", bmn, npts);
  export_d(&b, "xmn", xmn, npts);
  export_d(&b, "ymn", ymn, npts);
  export_d(&b, "zmn", zmn, npts);
  export_d(&b, "rxmn", rxmn, npts);
  export_d(&b, "symn", symn, npts);
  export_d(&b, "tzmn", tzmn, npts);
  export_d(&b, "ebm1", ebm1, npts);
  export_d(&b, "hbm1", hbm1, npts);
  export_d(&b, "unxm", unxm, nxzfl);
  export_d(&b, "unym", unym, nxzfl);
  export_d(&b, "unzm", unzm, nxzfl);
  export_d(&b, "aream", aream, nxzfl);
  export_d(&b, "Z_0", Z_0, nxzfl);
  export_d(&b, "Z_1", Z_1, nxzfl);
  export_d(&b, "Y_0", Y_0, nxzfl);
  export_d(&b, "Y_1", Y_1, nxzfl);
  long n = 0, npec = 0;
  export_i(&b, "cemface", cemface, NULL, &n);
  export_i(&b, "glo_face", NULL, glo_face, &n);
  export_i(&b, "cempec", cempec, NULL, &npec);

  nekgpu_mesh m;
  memset(&m, 0, sizeof m);
  m.nx1 = LX1;
  m.nelt = nelt;
  m.dxm1 = dxm1; m.w3mn = w3mn;
  m.rxmn = rxmn; m.rymn = rymn; m.rzmn = rzmn;
  m.sxmn = sxmn; m.symn = symn; m.szmn = szmn;
  m.txmn = txmn; m.tymn = tymn; m.tzmn = tzmn;
  m.bmn = bmn; m.xmn = xmn; m.ymn = ymn; m.zmn = zmn;
  m.unxm = unxm; m.unym = unym; m.unzm = unzm; m.aream = aream;
  m.cemface = cemface; m.glo_face = glo_face; m.cempec = cempec; m.ncempec = (int)npec;
  m.Z_0 = Z_0; m.Z_1 = Z_1; m.Y_0 = Y_0; m.Y_1 = Y_1;
  m.ebm1 = ebm1; m.hbm1 = hbm1;
  m.C0 = 1.0;
  check(nekgpu_init(&ctx, &m, form), "nekgpu_init");
  if (use_source) {
    const double xc[3] = {0.2, -0.1, 0.3};
    check(nekgpu_set_source(ctx, 1, xc, 0.3, 1.0, 2.0, 0.05), "nekgpu_set_source");
  }

  /* cem_maxwell_init_fields: userini = the exact solution at t = 0 */
  const double dt = 0.005;
  double time = 0.0;
  usersol(time);
  memcpy(hn, shn, sizeof hn);
  memcpy(en, sen, sizeof en);
  check(nekgpu_set_state(ctx, hn, en, LPTS1), "nekgpu_set_state");
  if (host_path) {
    check(nekgpu_register_host(ctx, hn, (long)sizeof hn), "nekgpu_register_host");
    check(nekgpu_register_host(ctx, en, (long)sizeof en), "nekgpu_register_host");
  }

  /* time_advancing_pde */
  for (int istep = 1; istep <= nsteps; ++istep) {
    if (host_path) {
      check(nekgpu_op_rk_host(ctx, hn, en, LPTS1, time, dt), "nekgpu_op_rk_host");
    } else {
      double tloc = time; /* the library advances its copy; the loop owns time */
      check(nekgpu_step(ctx, 1, &tloc, dt), "nekgpu_step");
    }
    time = time + dt;
    /* userchk */
    if (istep % iocomm == 0 || istep == nsteps) {
      double l2[6], linf[6];
      if (!host_path) check(nekgpu_get_state(ctx, hn, en, LPTS1), "nekgpu_get_state");
      usersol(time);
      check(nekgpu_norms(ctx, shn, sen, LPTS1, l2, linf), "nekgpu_norms");
      printf("chk %d %.17g", istep, time);
      for (int q = 0; q < 6; ++q) printf(" %.17g", l2[q]);
      for (int q = 0; q < 6; ++q) printf(" %.17g", linf[q]);
      printf("\n");
    }
  }
  printf("final_time %.17g\n", time);

  FILE* f = fopen(argv[6], "wb");
  if (!f) return 2;
  for (int q = 0; q < 3; ++q) fwrite(hn + (long)q * LPTS1, sizeof(double), (size_t)npts, f);
  for (int q = 0; q < 3; ++q) fwrite(en + (long)q * LPTS1, sizeof(double), (size_t)npts, f);
  fclose(f);
  if (host_path) {
    check(nekgpu_unregister_host(ctx, hn), "nekgpu_unregister_host");
    check(nekgpu_unregister_host(ctx, en), "nekgpu_unregister_host");
  }
  check(nekgpu_finalize(ctx), "nekgpu_finalize");
  return 0;
}
