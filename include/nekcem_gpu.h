/*
 * nekcem_gpu.h -- C ABI of the GB300 (sm_103a) Maxwell DG time-step library.
 *
 * Drop-in boundary for NekCEM's 3-D Maxwell time step, run as `mpirun -np 1`
 * on one GPU.  The Fortran driver keeps its subroutines and its
 * element-major COMMON arrays; under a NEKGPU build, cem_maxwell_op_rk
 * (src/cem_maxwell.F:327-345) calls nekgpu_step / nekgpu_op_rk_host instead of
 * its five CPU stages, after cem_maxwell_init (src/cem_maxwell.F:65-191) has
 * handed the static arrays to nekgpu_init.  The Fortran side binds these
 * entry points with iso_c_binding interfaces (bind(c), scalars by value
 * where declared so here, arrays as assumed-size dummies).
 *
 * Conventions
 *   - Plain C types only; all arrays are caller-owned host memory in the
 *     reference's Fortran layout.  Index arrays are 1-based as in Fortran.
 *   - A 3-vector field is `hn(ld,3)`: component q of node i at hn[i + ld*q].
 *   - Face arrays are in face-slot order j + nx1^2*(f + 6*e), f in the
 *     reference's face order (src/nek5_coef.F:1182-1235).
 *   - Every call returns NEKGPU_OK (0) or a negative NEKGPU_ERR_* code;
 *     nekgpu_error_string() gives a message.  The Fortran side maps any
 *     non-zero status to exitt(1).
 *   - One host thread per context.  The context owns one CUDA stream; calls
 *     that return host data synchronise that stream, others may return before
 *     the GPU work ends.
 */
#ifndef NEKCEM_GPU_H
#define NEKCEM_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define NEKGPU_OK 0
#define NEKGPU_ERR_ARG -1         /* null pointer, bad size or index */
#define NEKGPU_ERR_MESH -2        /* mesh the chosen form cannot run */
#define NEKGPU_ERR_CUDA -3        /* CUDA runtime error */
#define NEKGPU_ERR_NOMEM -4       /* device allocation failed / over budget */
#define NEKGPU_ERR_STATE -5       /* call out of order */
#define NEKGPU_ERR_BLOWUP -6      /* non-finite or |u| > 1e20 (chk_blowup) */
#define NEKGPU_ERR_TIMEOUT -7     /* a bounded device wait ran out */
#define NEKGPU_ERR_UNSUPPORTED -8 /* feature not built for this case */
#define NEKGPU_ERR_TOO_LARGE -9   /* mesh larger than a fixed-size scratch allows */

/* Compute forms. */
#define NEKGPU_PLAIN 0   /* unfused all-FP64 kernels, one per reference routine */
#define NEKGPU_FUSED64 1 /* fused curl+flux+lift+mass+RK stage kernel, all FP64 */
#define NEKGPU_MIXED 2   /* fused stage kernel: FP32 contractions/curl/flux,
                            FP64 state, RK register, inverse mass and norms;
                            exact-hi compensated contractions on a normalised
                            residual (accuracy of the FP64 forms) */
#define NEKGPU_MIXED_NAIVE 3 /* the same fused kernel as FUSED64 computed in
                            plain FP32; kept to measure what the compensation
                            of NEKGPU_MIXED costs (its L2 error is far larger) */

/* Face boundary codes (CBC in src/cem_maxwell.F:289-300, 1338-1366). */
#define NEKGPU_BC_PEC 0
#define NEKGPU_BC_PERIODIC 1
#define NEKGPU_BC_PML 2      /* 'PML' faces: a PEC wall behind perfectly matched layers */

typedef struct nekgpu_ctx nekgpu_ctx;

/*
 * Static arrays after cem_maxwell_init (src/cem_maxwell.F:65-191), as the
 * Fortran COMMON blocks hold them (src/EMWAVE, src/GEOM).  npts = nx1^3*nelt,
 * nxzfl = 6*nx1^2*nelt.
 */
typedef struct nekgpu_mesh {
  int nx1;                 /* N+1 GLL points per direction */
  int nelt;                /* elements on this rank */
  const double* dxm1;      /* nx1*nx1, D(i,j) column-major (src/nek5_speclib.F:807) */
  const double* w3mn;      /* nx1^3 GLL tensor weights */
  const double* rxmn;      /* npts each: cofactor metrics jac*dr/dx ... */
  const double* rymn;      /*   (src/nek5_coef.F:616-624, src/cem_maxwell.F:135-162) */
  const double* rzmn;
  const double* sxmn;
  const double* symn;
  const double* szmn;
  const double* txmn;
  const double* tymn;
  const double* tzmn;
  const double* bmn;       /* npts mass jac*w3 (src/nek5_coef.F:758) */
  const double* xmn;       /* npts coordinates (used by source terms); may be NULL */
  const double* ymn;
  const double* zmn;
  const double* unxm;      /* nxzfl unit normals (src/nek5_coef.F:1150-1237) */
  const double* unym;
  const double* unzm;
  const double* aream;     /* nxzfl face area weights */
  const int* cemface;      /* nxzfl, 1-based volume index (src/cem_common.F:214-257) */
  const long long* glo_face; /* nxzfl gs ids of gsh_face (src/nek5_connect11.F:2223) */
  const int* cempec;       /* ncempec 1-based PEC face slots (src/cem_maxwell.F:1338) */
  int ncempec;
  const double* Z_0;       /* nxzfl face impedances (src/cem_maxwell.F:262-325) */
  const double* Z_1;
  const double* Y_0;
  const double* Y_1;
  const double* ebm1;      /* npts 1/(eps*bm1) (src/cem_maxwell.F:183-186) */
  const double* hbm1;      /* npts 1/(mu*bm1) */
  double C0;               /* 1 upwind, 0 central (src/cem_maxwell.F:939-940) */
  /* PML (src/cem_maxwell_pml.F; NULL / 0 without PML): */
  const double* pmlsigma;  /* 3*npts sigma x, y, z of pml_calc_sigma (:433-506) */
  const int* pmlptr;       /* npml 1-based PML elements (pmlptr of pml_calc_sigma) */
  int npml;
  const double* permittivity; /* npts per node (needed with PML) */
  const double* permeability;
} nekgpu_mesh;

/*
 * Structured affine box: what genbox + usrdat2 + uservp produce for the
 * reference's box test cases, built on the host without the Fortran side.
 * Elements are numbered x fastest, then y, then z.
 */
typedef struct nekgpu_box {
  int N;                   /* polynomial order (nx1 = N+1), 1..15 */
  int nelx, nely, nelz;
  double lo[3], hi[3];     /* domain [lo,hi] per axis */
  int bc[3];               /* NEKGPU_BC_PEC, _PERIODIC or _PML per axis */
  const double* permittivity; /* npts per node, or NULL for 1 */
  const double* permeability; /* npts per node, or NULL for 1 */
  double C0;               /* 1 upwind, 0 central */
  /* PML layers behind NEKGPU_BC_PML faces (params 77-79 of the .rea file,
   * src/cem_param.F:84-86): thickness in element layers (1..10), polynomial
   * order of the sigma grading, reflection error */
  int pml_thick;
  double pml_order, pml_referr;
} nekgpu_box;

const char* nekgpu_error_string(int status);
int nekgpu_version(void);

/* Select and check the CUDA device (default 0).  Called implicitly by init. */
int nekgpu_device_check(int device);

/* ---- setup / teardown ----------------------------------------------------- */
/* Replaces cem_maxwell_init's hand-off: uploads the static arrays once.
 * The face pairing comes from glo_face exactly as gs_setup groups it
 * (src/jl/gs.h:17-60); groups of more than two are rejected.  On affine
 * elements (per-element-constant metrics) with axis-aligned faces whose paired
 * nodes share in-face order the fused forms use their compact per-element
 * geometry; on any other conforming hex mesh with the reference's face
 * numbering and nx1 <= 8 they use their curvilinear kernels (per-node metrics,
 * per-face-node normals and areas; no PML or dispersive media there).
 * NEKGPU_PLAIN takes any conforming hex mesh. */
int nekgpu_init(nekgpu_ctx** ctx, const nekgpu_mesh* mesh, int form);
/* Builds the box case on the host (GLL points, geometry, face pairing,
 * materials) and uploads it. */
int nekgpu_init_box(nekgpu_ctx** ctx, const nekgpu_box* box, int form);
/* The 2-D forms (the reference's ldim = 2 build): imode 1 = TE (E1, E2, H3),
 * 2 = TM (H1, H2, E3), param(4).  The mesh holds the 2-D arrays: w3mn nx1^2,
 * rxmn/rymn/sxmn/symn (the 2-D cofactors of GLMAPM1), face arrays of
 * nxzfl = 4 nx1 nelt slots in the reference's 2-D face numbering; the z
 * metrics, unzm and zmn are not read.  One kernel per RK stage in the
 * reference's FP64 arithmetic (bit-identical to the CPU path); fields keep
 * the (ld,3) layout with the inactive components left as set.  PML: the
 * mesh's pmlsigma (3*npts), pmlptr and materials as in 3-D (pml_step on the
 * active components, their pmlbn/pmldn through nekgpu_set_array /
 * nekgpu_get_array).  Volume source: a line source on E_z (TM) or H_z (TE).  No
 * dispersive media, adjoint or VTK output in 2-D. */
int nekgpu_init2d(nekgpu_ctx** ctx, const nekgpu_mesh* mesh, int imode);
int nekgpu_finalize(nekgpu_ctx* ctx);

/* Host-only (no GPU needed): the box builder's reference-layout arrays, for
 * checking the host setup.  Double arrays: "dxm1" (nx1^2), "w3mn" (nx1^3),
 * "bmn","xmn","ymn","zmn","rxmn","symn","tzmn","ebm1","hbm1" (npts),
 * "unxm","unym","unzm","aream","Z_0","Z_1","Y_0","Y_1" (nxzfl), "pmlsigma"
 * (3*npts with PML, else empty).  Integer arrays: "cemface" (nxzfl, 1-based),
 * "glo_face" (nxzfl), "cempec" (1-based, *count entries), "pmlptr" (1-based
 * PML elements).  *count receives the number of entries written. */
int nekgpu_box_export_d(const nekgpu_box* box, const char* name, double* out, long* count);
int nekgpu_box_export_i(const nekgpu_box* box, const char* name, long long* out, long* count);

/* sizes: npts, nxzfl, nelt, nx1 */
int nekgpu_sizes(const nekgpu_ctx* ctx, long* npts, long* nxzfl, int* nelt, int* nx1);
/* the box builder's arrays (reference layout), for users that need
 * coordinates / mass without the Fortran side: name in
 * {"xmn","ymn","zmn","bmn","ebm1","hbm1"}; out has npts doubles.  With PML:
 * "pmlbn", "pmldn" (the auxiliary fields, 3*npts, zero outside the PML) and
 * "pmlsigma" (3*npts). */
int nekgpu_get_array(nekgpu_ctx* ctx, const char* name, double* out);
double nekgpu_volume(const nekgpu_ctx* ctx);

/* Time function of the source: 0 = Ricker (default), 1 = amp * sin(f0 * t)
 * (the Gaussian dipole of tests/3dboxpml/3dboxpml.usr:28-85, omega = f0). */
int nekgpu_set_source_kind(nekgpu_ctx* ctx, int kind);
/* Gaussian-in-space, Ricker-in-time E_z volume source in mass-weighted form,
 * added before the inverse mass like usersrc (src/cem_maxwell.F:503):
 * resEz += bm1 * amp * exp(-|x-xc|^2/(2 sigma^2)) * ricker(t; f0, t0),
 * ricker(t) = (1 - 2 a^2) exp(-a^2), a = pi f0 (t - t0).  enabled=0 clears.
 * 2-D context: a line source along z (z ignored: give xc[2] = 0) on the
 * out-of-plane field, E3 = E_z in TM and H3 = H_z in TE, as the reference's
 * 2-D cases drive it (tests/2dboxpml/2dboxpml.usr). */
int nekgpu_set_source(nekgpu_ctx* ctx, int enabled, const double xc[3], double sigma,
                      double amp, double f0, double t0);

/* ---- incident field (userinc) ------------------------------------------------ */
/* userinc between the restriction to faces and the flux
 * (src/cem_maxwell.F:495-496) in the plane-wave form of the reference's
 * cases (tests/drude/drude.usr:7-42): the face values of the n listed slots
 * (1-based incindex) get amp[0..2] * cos(k.x - omega t) on H and amp[3..5] *
 * cos(...) on E, x the face node, t the stage time.  n = 0 removes it.  All
 * three 3-D forms (not on curvilinear meshes); needs node coordinates. */
int nekgpu_set_incident(nekgpu_ctx* ctx, const int* slots, long n, const double amp[6],
                        const double kvec[3], double omega);
/* Sets "pmlbn" or "pmldn" (3*npts, the reference layout; a case's userini
 * sets pmlbn = mu H, pmldn = eps E); nodes outside the PML are ignored. */
int nekgpu_set_array(nekgpu_ctx* ctx, const char* name, const double* in);

/* ---- graphene sheets ------------------------------------------------------------ */
/* cem_3d_graphene_current (src/cem_maxwell.F:2827-2931) run through userfsrc
 * as tests/3dgraphene does: on the n listed face slots (1-based graphindex)
 * the surface current from the face fields and the 12 parameters
 * params(nxzfl,12) (a_d, b_d, b_cp1, a_211, a_221, b_11, b_21, b_cp2, a_212,
 * a_222, b_12, b_22), its auxiliary currents advanced with the RK stage, and
 * -J added to the -n x H part of the flux before the face sum.  yconduc is
 * the reference's face array (nxzfl).  The currents start at zero; n = 0
 * removes the sheets.  Plain form: any listed slot; fused FP64 and mixed
 * forms: slots on interior faces (NEKGPU_ERR_UNSUPPORTED for wall slots,
 * curvilinear and 2-D meshes). */
int nekgpu_set_graphene(nekgpu_ctx* ctx, const double* params, const int* slots, long n,
                        const double* yconduc);
/* The face currents fjn(ld,3,6), ld >= nxzfl: listed slots only. */
int nekgpu_set_graphene_current(nekgpu_ctx* ctx, const double* fjn, long ld);
int nekgpu_get_graphene_current(nekgpu_ctx* ctx, double* fjn, long ld);

/* ---- dealiased curl (NEKGPU_PLAIN; NEKGPU_FUSED64 on curvilinear meshes) ------ */
/* param(18) = -1: maxwell_wght_dcurl (src/cem_maxwell.F:1541-1729) on lxd GLL
 * points per direction instead of maxwell_wght_curl.  The tables are the
 * reference's (built on its first dcurl call): jgl(lxd,nx1) interpolation
 * (gen_int), dxmd(lxd,lxd) derivative (gen_dgl), w3md(lxd^3) weights, and
 * metd the nine metric cofactors interpolated to the lxd^3 points, ordered
 * rx, ry, rz, sx, sy, sz, tx, ty, tz, each (lxd^3, nelt).  lxd = 0 switches
 * back.  The fused FP64 form on a curvilinear mesh takes it too: each stage
 * computes the dealiased volume term first, then adds flux, lift, source,
 * inverse mass and RK update in its one stage kernel.  NEKGPU_ERR_UNSUPPORTED
 * for the other forms and for fused forms on affine meshes, 2-D meshes or an
 * lxd whose element working set does not fit in shared memory (~220 KB). */
int nekgpu_set_dealias(nekgpu_ctx* ctx, int lxd, const double* jgl, const double* dxmd,
                       const double* w3md, const double* metd);

/* ---- dispersive media ---------------------------------------------------- */
#define NEKGPU_DRUDE 1
#define NEKGPU_LORENTZ 2
/* Polarisation currents at listed nodes, advanced with every RK stage inside
 * usersrc before the volume source, as tests/drude/drude.usr:167 and
 * tests/lorentz/lorentz.usr:174 call them:
 *   NEKGPU_DRUDE (cem_maxwell_drude, src/cem_maxwell.F:3095-3147):
 *     params(ld,2) = a, b;  resE -= J bm1,  dJ/dt = -a J + b E
 *   NEKGPU_LORENTZ (cem_maxwell_lorentz, src/cem_maxwell.F:3149-3212):
 *     params(ld,3) = a, b, c;  resE -= J1 bm1,  dJ1/dt = -a J1 - b J2 + c E,
 *     dJ2/dt = J1
 * index: n 1-based node numbers (drudeindex / lorentzindex); a node may be in
 * one list once.  A call replaces that model's list (n = 0 removes it) and
 * restarts every current and its RK register at zero.  NEKGPU_PLAIN,
 * NEKGPU_FUSED64 and NEKGPU_MIXED (currents in FP64 in all three). */
int nekgpu_set_dispersive(nekgpu_ctx* ctx, int model, const double* params, long ld,
                          const int* index, long n);
/* The currents in the reference layout, jn(ld,3) (Drude) or jn(ld,3,2)
 * (Lorentz: J1 then J2); only listed nodes are read, other nodes read 0. */
int nekgpu_set_current(nekgpu_ctx* ctx, int model, const double* jn, long ld);
int nekgpu_get_current(nekgpu_ctx* ctx, int model, double* jn, long ld);

/* ---- state --------------------------------------------------------------- */
/* hn(ld,3), en(ld,3) host arrays, ld >= npts (lpts1 in the reference). */
int nekgpu_set_state(nekgpu_ctx* ctx, const double* hn, const double* en, long ld);
int nekgpu_get_state(nekgpu_ctx* ctx, double* hn, double* en, long ld);
/* RK register khn/ken (src/EMWAVE); zero after set_state unless set here. */
int nekgpu_set_rk_register(nekgpu_ctx* ctx, const double* khn, const double* ken, long ld);
int nekgpu_get_rk_register(nekgpu_ctx* ctx, double* khn, double* ken, long ld);
/* Pin caller host memory once (cudaHostRegister) so per-step copies are DMA. */
int nekgpu_register_host(nekgpu_ctx* ctx, void* ptr, long bytes);
int nekgpu_unregister_host(nekgpu_ctx* ctx, void* ptr);

/* ---- time stepping --------------------------------------------------------- */
/* One RK stage rkstep=1..5 at time `time` (rk_c + cem_maxwell_op +
 * rk_maxwell_ab; src/cem_maxwell.F:336-340). */
int nekgpu_stage(nekgpu_ctx* ctx, int rkstep, double time, double dt);
/* nsteps full steps (cem_maxwell_op_rk each) on the device-resident state,
 * step s running its stages at *time + c_i dt.  On return *time has been
 * advanced by the library: dt is added after every step, in the same
 * floating-point order as time_advancing_pde's `time = time + dt`
 * (src/cem_drive.F:639), so *time ends at the time of the new state.
 * A driver whose own loop advances time after the call (time_advancing_pde
 * does) must therefore pass a copy, `tloc = time; nekgpu_step(ctx, 1, &tloc,
 * dt);` -- passing its own time variable would advance it twice per step. */
int nekgpu_step(nekgpu_ctx* ctx, int nsteps, double* time, double dt);
/* Drop-in for one cem_maxwell_op_rk call on host arrays: copies hn/en in,
 * runs the 5 stages at time + c_i dt, copies hn/en back; returns when hn/en
 * hold the new state.  time is taken by value and not advanced: the caller's
 * loop adds dt itself, as time_advancing_pde does.  The RK register stays on the GPU.  In the mixed form on meshes of
 * several waves of blocks the copies overlap stages 1 and 5 chunk by chunk
 * (same results bit for bit); hn/en page-locked with nekgpu_register_host
 * let the copies run at the link's rate. */
int nekgpu_op_rk_host(nekgpu_ctx* ctx, double* hn, double* en, long ld, double time,
                      double dt);

/* ---- the reference routines one by one (NEKGPU_PLAIN only) ---------------- */
int nekgpu_cem_maxwell(nekgpu_ctx* ctx);            /* src/cem_maxwell.F:574-582 */
int nekgpu_restrict_to_face(nekgpu_ctx* ctx);       /* src/cem_maxwell.F:604-623 */
int nekgpu_flux3d(nekgpu_ctx* ctx);                 /* src/cem_maxwell.F:922-1002 */
int nekgpu_add_flux_to_res(nekgpu_ctx* ctx);        /* src/cem_maxwell.F:725-735 */
int nekgpu_usersrc(nekgpu_ctx* ctx, double rktime); /* src/cem_maxwell.F:503 */
int nekgpu_invqmass(nekgpu_ctx* ctx);               /* src/cem_maxwell.F:1878-1886 */
int nekgpu_rk_maxwell_ab(nekgpu_ctx* ctx, int rkstep, double dt); /* src/cem_maxwell.F:1906 */
/* gs_op_fields(gsh_face, u, nxzfl, nfld, 1, 1, 0) on host data u(nxzfl,nfld)
 * (src/jl/gs.c:2074), through the device face exchange. */
int nekgpu_gs_op_fields(nekgpu_ctx* ctx, double* u, int nfld);
/* intermediate arrays of the plain form: "reshn","resen" (npts*3),
 * "fhn","fen" (nxzfl*3), "srflx" (nxzfl*6) */
int nekgpu_get_work(nekgpu_ctx* ctx, const char* name, double* out);

/* ---- norms ----------------------------------------------------------------- */
/* cem_error (src/cem_common.F:1335-1355) for the 6 components against host
 * exact fields: l2[q] = sqrt(sum e*bm1*e / vol), linf[q] = max|e|, FP64. */
int nekgpu_norms(nekgpu_ctx* ctx, const double* exact_h, const double* exact_e, long ld,
                 double l2[6], double linf[6]);
/* No counterpart in the reference.  The same norms as nekgpu_norms for
 * callers that cannot allocate device memory while time stepping (a driver
 * that gave all free device memory to its own pool, or a loop that must not
 * risk an allocation failure or cudaFree's synchronisation between steps).
 * exact_dev: device array, 6*npts doubles, H then E, component after
 * component.  Allocates nothing: the reduction's partial sums live in a fixed
 * device array of the library (384 KB, held by every GPU that loads it until
 * exit), so at most 8,388,608 nodes (else NEKGPU_ERR_TOO_LARGE).  Calls whose
 * GPU work can overlap share that array and race.  The first call on a device
 * looks the array up (cudaGetSymbolAddress); make it before any stream
 * capture. */
int nekgpu_norms_noalloc(nekgpu_ctx* ctx, const double* exact_dev, double l2[6], double linf[6]);
/* field energy 0.5*sum bm1*(eps|E|^2 + mu|H|^2), FP64 on device */
int nekgpu_energy(nekgpu_ctx* ctx, double* energy);
/* Failure-detection self-test: one kernel polls an mbarrier that nothing
 * arrives at `polls` times (1..2^22), as the stage kernels poll for their
 * copies, and gives up; returns NEKGPU_ERR_TIMEOUT (the status word the stage
 * kernels set when a wait runs out) and leaves the context usable. */
int nekgpu_selftest_wait(nekgpu_ctx* ctx, int polls);
/* The mixed stage's join of a float pair (s, t), |t| <= ulp(s)/2, into one
 * FP64 value by integer operations, applied to n host pairs on device 0
 * (test hook): out[i] = s[i] + t[i], exact whenever the sum fits in 53 bits,
 * else truncated below one FP64 ulp. */
int nekgpu_selftest_pair_join(const float* s, const float* t, double* out, long n);
/* chk_blowup (src/cem_common.F:1150-1165): NEKGPU_ERR_BLOWUP if any state
 * value is non-finite or above 1e20 in magnitude */
int nekgpu_check_blowup(nekgpu_ctx* ctx);

/* ---- discrete adjoint (NEKGPU_FUSED64, NEKGPU_MIXED; affine meshes) -------- */
/* No routine of the reference computes gradients; this is the discrete
 * adjoint of nsteps RK45 steps of the FP64 fused stage (cem_maxwell_op_rk,
 * src/cem_maxwell.F:327-345) for J = sum_n jw[n] |E(n)|^2 at the final time.
 * The forward steps (first pass and recomputations) run in the context's
 * form: with NEKGPU_MIXED they are mixed stages, whose trajectory agrees with
 * the FP64 one to ~1e-10, and the FP64 reverse stages read those states.
 * Starts from the context's current state and leaves it at the final state.
 * Schedules: stride > 0 checkpoints the state every `stride` steps and the
 * reverse sweep recomputes one segment at a time, keeping its stage states
 * and RK registers (ceil(nsteps/stride) + 4 x (5 stride + 1) + 4 states);
 * stride = 0 does the same with stride = ceil(sqrt(nsteps)) when that fits in
 * the device memory left (under NEKGPU_MEM_BUDGET_MB: the budget less the
 * context's own memory), else falls back to the binomial schedule with the
 * snapshots that fit; stride < 0 uses the binomial schedule with -stride
 * device snapshots (15 states + snapshots; forward steps recomputed more
 * often), plus the host snapshots of nekgpu_adjoint_host_snapshots.
 * NEKGPU_ERR_NOMEM when the chosen schedule does not fit.  Returns J, dJ/deps
 * at every node (npts, host array) and the device times up to J (forward)
 * and of the rest (reverse sweep, recomputation included), in ms.
 * jw: npts host weights (e.g. bm1 on a probe region). */
int nekgpu_adjoint_gradient(nekgpu_ctx* ctx, int nsteps, double t0, double dt, const double* jw,
                            double* J, double* dJdeps, int stride, double* fwd_ms,
                            double* adj_ms);
/* The same split into the two calls of a driver that sets the objective once
 * and evaluates it for several states or step counts: nekgpu_adjoint_init
 * copies the weights jw (npts, host) and the checkpoint stride into the
 * context (it allocates nothing on the device); nekgpu_adjoint_run runs
 * nekgpu_adjoint_gradient with them.  NEKGPU_ERR_STATE if run comes first. */
int nekgpu_adjoint_init(nekgpu_ctx* ctx, const double* jw, int stride);
/* Pinned host-memory snapshots (one state each, 48 bytes per node) that the
 * binomial schedule may use beyond the device snapshots (default 0): a state
 * too large for many device snapshots reverses with fewer recomputations.
 * Each use of a host snapshot copies one state over the host link.  Gradients
 * are bit-identical whatever memory the snapshots live in. */
int nekgpu_adjoint_host_snapshots(nekgpu_ctx* ctx, int n);
/* NEKGPU_FUSED64 on affine meshes: on != 0 recomputes the segments of the
 * sqrt(steps) schedule with mixed stages (started at the FP64 checkpoints)
 * instead of FP64 ones; the first pass, J and the checkpoints stay FP64, and
 * the reverse stages read stage states within ~1e-10 per step of the FP64
 * ones (gradients within ~1e-8 of the exact discrete adjoint's).  The
 * binomial schedule is not affected.  NEKGPU_ERR_UNSUPPORTED for other forms
 * or meshes. */
int nekgpu_adjoint_recompute_mixed(nekgpu_ctx* ctx, int on);
int nekgpu_adjoint_run(nekgpu_ctx* ctx, int nsteps, double t0, double dt, double* J,
                       double* dJdeps);

/* ---- output ------------------------------------------------------------------ */
/* The reference's VTK output for param(81) = 3 (cem_out_fields3,
 * src/io.F:562-640; src/io_vtkbin.c writeheader/writenodes/write3dcells/
 * writefield; cells of vtk_dump_header_nonswap, src/io_dumpvtk.F:718-810):
 * legacy binary (big-endian), FP32 points and VECTORS "E ", "H " of the
 * current state and, when solhn/solen are given (3 x ld host arrays, the
 * analytic fields shn/sen), "solE", "solH".  Needs the node coordinates. */
int nekgpu_write_vtk(nekgpu_ctx* ctx, const char* path, const double* solhn, const double* solen,
                     long ld);
/* Checkpoints of the device state (fields, RK register, PML auxiliary fields
 * and dispersive currents with their registers, raw FP64) with the time and
 * step number; loading one into a
 * context of the same form and mesh (else NEKGPU_ERR_MESH) continues the run
 * bit for bit.  No counterpart in the reference's non-MPI build, whose
 * restart writers are empty (src/io_vtkbin.c:307-322). */
int nekgpu_checkpoint_save(nekgpu_ctx* ctx, const char* path, double time, long istep);
int nekgpu_checkpoint_load(nekgpu_ctx* ctx, const char* path, double* time, long* istep);

/* ---- timing ---------------------------------------------------------------- */
/* Runs nsteps steps between CUDA events on the context stream and returns the
 * elapsed device milliseconds (state advances; *time += nsteps*dt). */
int nekgpu_time_steps(nekgpu_ctx* ctx, int nsteps, double* time, double dt, double* ms);
/* device memory held by the context, bytes (a set_* call that replaces
 * earlier data frees the earlier device arrays) */
long nekgpu_device_bytes(const nekgpu_ctx* ctx);
/* kernel launches issued by the last nekgpu_step / nekgpu_time_steps call */
long nekgpu_last_launches(const nekgpu_ctx* ctx);
/* synchronise the context stream */
int nekgpu_sync(nekgpu_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif
