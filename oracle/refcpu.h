/*
 * refcpu -- CPU FP64 restatement of NekCEM's 3-D Maxwell DG time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle that the CUDA path is checked
 * against (and the CPU baseline that bench.py times).  Nothing in the product
 * library links or calls it.
 *
 * Every routine restates the reference routine cited beside it, in the
 * reference's element-major Fortran layout (field(i,j,k,e), i fastest) and in
 * its summation order.  Indices are 0-based here; the reference is 1-based.
 */
#ifndef NEKCEM_REFCPU_H
#define NEKCEM_REFCPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ref_ctx ref_ctx;

/* Box boundary kind per axis (both sides of that axis): PEC walls, periodic,
 * or 'PML' faces (a PEC wall behind perfectly matched layers, set up by
 * ref_set_pml). */
enum { REF_BC_PEC = 0, REF_BC_PERIODIC = 1, REF_BC_PML = 2 };

/* GLL points/weights (src/nek5_speclib.F:107 ZWGLL -> ZWGLJD:240) */
void ref_zwgll(double* z, double* w, int np);
/* derivative matrix, column-major d[i + nz*j] = D(i,j) (src/nek5_speclib.F:807 DGLL) */
void ref_dgll(double* d, double* dt, const double* z, int nz);
/* Legendre polynomial P_n(z) (src/nek5_speclib.F:882 PNLEG) */
double ref_pnleg(double z, int n);

/*
 * Structured affine box mesh, N = polynomial order, nel{x,y,z} elements,
 * [lo,hi] per axis, bc[axis] in {REF_BC_PEC, REF_BC_PERIODIC}.
 * Performs genwz, genxyz, xyzrst, glmapm1, geodat1, area3, cem_set_fc_ptr,
 * the face global numbering (setup_dgds2 semantics) and the PEC list.
 * Materials default to eps = mu = 1; call ref_set_materials to change them.
 */
ref_ctx* ref_create_box(int N, int nelx, int nely, int nelz, const double lo[3],
                        const double hi[3], const int bc[3]);
/* the same box with a smooth interior deformation of amplitude amp (curved,
 * non-affine elements; the domain boundary stays in place) */
ref_ctx* ref_create_box_mapped(int N, int nelx, int nely, int nelz, const double lo[3],
                               const double hi[3], const int bc[3], double amp);
/* 2-D box of nelx x nely quadrilaterals for the TE (imode 1: E1, E2, H3) or
 * TM (imode 2: H1, H2, E3) form (the reference's ldim = 2 build, param(4));
 * lo/hi/bc per axis x, y.  The routines below take their 2-D branches. */
ref_ctx* ref_create_box2d(int N, int nelx, int nely, const double lo[2], const double hi[2],
                          const int bc[2], int imode);
int ref_ndim(const ref_ctx* c);
int ref_imode(const ref_ctx* c);
void ref_destroy(ref_ctx* c);

/* Named array access (the reference's COMMON arrays).  Returns NULL for an
 * unknown name; *len receives the element count. */
double* ref_darray(ref_ctx* c, const char* name, long* len);
int* ref_iarray(ref_ctx* c, const char* name, long* len);
long long* ref_larray(ref_ctx* c, const char* name, long* len);
/* integer sizes: "n", "nelt", "npts", "nxzf", "nxzfl", "ncempec" */
long ref_size(const ref_ctx* c, const char* name);
double ref_volvm1(const ref_ctx* c);

/* permittivity/permeability per node -> impedances, PEC doubling, ebm1/hbm1
 * (src/cem_maxwell.F:262-325 cem_maxwell_materials; :183-186) */
void ref_set_materials(ref_ctx* c, const double* permittivity, const double* permeability);

/* upwind C0=1 / central C0=0 (src/cem_param.F:73-74) */
void ref_set_flux(ref_ctx* c, double C0);

/* Gaussian-in-space, Ricker-in-time E_z volume source added in mass-weighted
 * form before the inverse mass (usersrc, src/cem_maxwell.F:503):
 *   resEz += bm1 * amp * exp(-|x-xc|^2/(2 sigma^2)) * ricker(t; f0, t0). */
void ref_set_source(ref_ctx* c, int enabled, const double xc[3], double sigma,
                    double amp, double f0, double t0);
double ref_source_time(double t, double f0, double t0);
/* time function of the source: 0 = Ricker (f0, t0), 1 = sin(f0 * t) (the
 * Gaussian dipole of tests/3dboxpml/3dboxpml.usr:28-85, omega = f0) */
void ref_set_source_kind(ref_ctx* c, int kind);

/* PML (src/cem_maxwell_pml.F): layers of elements marched `thick` levels in
 * from the 'PML' faces (pml_fill_faceary :139-190, march_faces :85-137 with
 * the gs max over face nodes), element tags and extents
 * (pml_extent_and_tags :261-431), the graded sigma profile
 * (pml_calc_sigma :433-506; order, reflection error referr).  The auxiliary
 * fields pmlbn, pmldn start at zero. */
void ref_set_pml(ref_ctx* c, int thick, double order, double referr);
/* pml_step (src/cem_maxwell_pml.F:508-590), after the lift and before usersrc */
void ref_pml_step(ref_ctx* c);

/* Dispersive media (cem_maxwell_drude / cem_maxwell_lorentz,
 * src/cem_maxwell.F:3095-3212, called from usersrc in tests/drude and
 * tests/lorentz).  params: Drude (npts,2) = a, b; Lorentz (npts,3) = a, b, c;
 * index: n 0-based nodes.  Inside ref_rk_stage the currents are advanced with
 * the stage (before the volume source); the currents are the darrays
 * "drudejn" (npts,3) and "lorentzjn" (npts,3,2), zero after these calls. */
void ref_set_drude(ref_ctx* c, const double* params, const int* index, long n);
void ref_set_lorentz(ref_ctx* c, const double* params, const int* index, long n);
void ref_dispersive(ref_ctx* c, int rkstep, double dt);

/* userinc as a plane wave on listed face slots (0-based): the face values
 * get amp[0..2] (H) and amp[3..5] (E) times cos(k.x - omega t) between the
 * restriction and the flux; n = 0 switches it off. */
void ref_set_incident(ref_ctx* c, const int* slots, long n, const double amp[6],
                      const double k[3], double omega);
void ref_userinc(ref_ctx* c, double rktime);

/* Graphene sheets (cem_3d_graphene_current, src/cem_maxwell.F:2827-2931,
 * through userfsrc as tests/3dgraphene does): params (nxzfl,12) per face
 * slot, n listed 0-based slots; inside ref_rk_stage the face currents are
 * computed after the flux's first loop and subtracted from -n x H before the
 * gs sum.  The currents are the darray "fjn" (nxzfl,3,6), zero after this. */
void ref_set_graphene(ref_ctx* c, const double* params, const int* slots, long n);
void ref_graphene(ref_ctx* c, int rkstep, double dt);

/* Dealiased curl (param(18) = -1: maxwell_wght_dcurl, src/cem_maxwell.F:
 * 1541-1729) on md = lxd >= nx1 GLL points per direction; md = 0 returns to
 * maxwell_wght_curl.  Returns -1 for a bad md or a 2-D mesh.  The tables
 * are the darrays "jgl" (md x mx), "dxmd" (md x md), "w3md" and "metd". */
int ref_set_dealias(ref_ctx* c, int md);
void ref_wght_dcurl(ref_ctx* c, double* w1, double* w2, double* w3, const double* u1,
                    const double* u2, const double* u3);

/* ---- the reference routines on the hot path ---- */
void ref_local_grad3(double* ur, double* us, double* ut, const double* u, int n,
                     const double* D, const double* Dt);
void ref_wght_curl(ref_ctx* c, double* w1, double* w2, double* w3, const double* u1,
                   const double* u2, const double* u3);
void ref_cem_maxwell(ref_ctx* c);            /* resE = Wcurl H, resH = -Wcurl E */
void ref_restrict_to_face(ref_ctx* c);       /* fH, fE */
void ref_flux3d(ref_ctx* c);                 /* srflx incl. gs + pec + upwind */
void ref_flux_pre(ref_ctx* c);               /* -n x E, -n x H into srflx */
void ref_gs_op_fields(ref_ctx* c, double* u, long stride, int nfld);
void ref_flux_pec(ref_ctx* c);
void ref_flux_upwind(ref_ctx* c);
void ref_add_flux_to_res(ref_ctx* c);
void ref_usersrc(ref_ctx* c, double rktime);
void ref_invqmass(ref_ctx* c);
void ref_maxwell_op(ref_ctx* c, double rktime);
void ref_rk4_upd(double* h, double* kh, const double* resh, double cb, double ca,
                 double dt, long n);
void ref_rk_coeffs(double a[5], double b[5], double c[6]);
void ref_rk_stage(ref_ctx* c, int rkstep /*1..5*/, double time, double dt);
void ref_op_rk(ref_ctx* c, double time, double dt);        /* one full time step */
void ref_run(ref_ctx* c, int nsteps, double* time, double dt); /* time += dt per step */

/* dxmin (src/nek5_courant.F:2-75), L2/Linf error (src/cem_common.F:1335-1355) */
double ref_get_dxmin(const ref_ctx* c);
void ref_cem_error(const ref_ctx* c, const double* u, const double* exact, long n,
                   double* l2, double* linf);

/* OpenMP threads used by the operator loops (1 = serial). */
void ref_set_threads(int nthreads);
int ref_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
