// Internal context of the GB300 Maxwell DG library (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <cmath>
#include <vector>

#include "nekcem_gpu.h"

namespace nekgpu {

constexpr int kMaxNx = 16;     // nx1 limit of the plain kernels (N <= 15)
constexpr int kMaxMixed = 10;  // nx1 limit of the parameter-resident D of the mixed form

// Compact description of an affine, axis-aligned hex mesh: what the fused
// forms consume.  Built either by the box builder or by compressing the
// reference's per-node arrays (nekgpu_init).
// PML description (src/cem_maxwell_pml.F): elements, graded sigma, materials.
struct PmlHost {
  std::vector<int> elems;       // 0-based PML elements, ascending (pmlptr order)
  std::vector<double> sigma;    // 3*npts: sigma x, y, z
  std::vector<double> eps, mu;  // npts
  bool on() const { return !elems.empty(); }
};

struct Compact {
  int nx = 0, nelt = 0;
  std::vector<double> D;        // nx*nx, D[i + nx*j] = D(i,j)
  std::vector<double> w;        // nx GLL weights (w3 = w_i w_j w_k)
  std::vector<double> w3;       // nx^3 (as given by the caller)
  std::vector<double> egeom;    // per element: rx, sy, tz, area scale per slot (6)
  std::vector<int> nbr;         // 6*nelt: partner element, -1 PEC mirror
  std::vector<double> ebm1, hbm1;   // npts
  std::vector<double> bm1;          // npts
  std::vector<double> fcoef;    // 4*nxzfl: Y02, C02Y, Z02, C02Z per face node
  bool uniform = true;          // all face coefficients equal the eps=mu=1 values
  double C0 = 1.0;
  PmlHost pml;
};

// Full reference arrays, for the plain form (one kernel per routine).
struct PlainHost {
  std::vector<double> dxm1, dxtm1, w3, metrics;  // metrics: 9*npts rx,ry,rz,sx,sy,sz,tx,ty,tz
  std::vector<double> unx, uny, unz, area, Z0, Z1, Y0, Y1, ebm1, hbm1, bm1;
  std::vector<int> cemface;      // 0-based
  std::vector<int> pairs;        // gs pairs (j0, j1), j0 < j1
  std::vector<int> cempec;       // 0-based
  std::vector<int> lift_ptr, lift_slot;  // CSR volume node -> face slots (ascending)
  double C0 = 1.0;
  PmlHost pml;
};

struct Source {
  bool enabled = false;
  int kind = 0;  // 0 Ricker(f0, t0), 1 sin(f0 t)
  double xc[3] = {0, 0, 0}, sigma = 0, amp = 0, f0 = 0, t0 = 0;
};

// amp times the source time function at t: Ricker (1 - 2a^2) exp(-a^2),
// a = pi f0 (t - t0), or -sin(-f0 t) (tests/3dboxpml/3dboxpml.usr:72-82)
inline double source_ft(const Source& s, double t) {
  if (s.kind == 1) return -s.amp * std::sin(-s.f0 * t);
  const double pi = 4.0 * std::atan(1.0);
  const double a = pi * s.f0 * (t - s.t0);
  return s.amp * ((1.0 - 2.0 * a * a) * std::exp(-a * a));
}

// Kernel argument blocks ----------------------------------------------------

// Dispersive currents (cem_maxwell_drude / cem_maxwell_lorentz), compact over
// the elements holding listed nodes (slot l holds element elem[l]); per node
// [q][l*N3 + v]: q = 0 kind (0 none, 1 Drude, 2 Lorentz), 1 a, 2 b, 3 c,
// 4 bm1, 5 bm1/(w3*rx) (a residual term t enters the mixed form's R as
// t * [5]).  aux: J1 (3 rows) then J2 (3 rows, Lorentz); k: their registers.
constexpr int kDispData = 6;
struct DispDev {
  const int* slot;  // nelt: slot of the element, -1 without listed nodes
  const int* elem;  // nslot: element of each slot
  const double* data;
  double* aux;      // 6 * n
  double* k;        // 6 * n
  long n;           // nslot * N3
};

struct PlainDev {
  int nx, nelt;
  long npts, nxzfl;
  const double* dxm1;
  const double* dxtm1;
  const double* w3;
  const double* metrics;
  const double *unx, *uny, *unz, *area, *Z0, *Z1, *Y0, *Y1, *ebm1, *hbm1;
  const int* cemface;
  const int* pairs;
  int npairs;
  const int* cempec;
  int ncempec;
  const int *lift_ptr, *lift_slot;
  double C0;
  double* u;      // 6*npts state, H then E
  double* k;      // 6*npts RK register
  double* res;    // 6*npts
  double* fface;  // 6*nxzfl restricted fields: fhn then fen
  double* srflx;  // 6*nxzfl
  const double* src_w;  // npts or null
  // PML (null / 0 without): full-size arrays in the reference layout
  const double* pmlsigma;  // 3*npts
  const double* eps;       // npts
  const double* mu;        // npts
  const double* bm1;       // npts
  const int* pmlptr;       // npml elements
  int npml;
  double* pmlaux;          // 6*npts: pmlbn then pmldn
  double* pmlk;            // 6*npts: their RK registers
  double* pmlres;          // 12*npts: respmlbn, respmldn, respmlhn, respmlen
  DispDev disp;
  // dealiased curl (md > 0): md GLL points per direction, interpolation
  // jgl (md x mx) and its transpose jgt, derivative dxmd / dxtmd on the md
  // points, weights w3md (md^3), metrics on the md^3 points (9 x md^3 x nelt)
  int md;
  const double *jgl, *jgt, *dxmd, *dxtmd, *w3md, *metd;
  // userinc: the stage's incident values (6 per listed slot) and the slots
  int ninc;
  const int* inc_slot;
  const double* inc_val;
  // graphene sheets on listed face slots, compact per listed slot q:
  // gr_par[p*ng + q] (12 parameters), gr_yc[q] (yconduc), gr_f / gr_k
  // [(3k + m)*ng + q] the face currents fjn(.,m,k) and their RK registers
  int ngraph;
  const int* gr_slot;
  const double *gr_par, *gr_yc;
  double *gr_f, *gr_k;
};

// PML data of the fused forms, compact over the PML elements (slot l holds
// element pml_elem[l]); per node of a PML element, [q][l*N3 + v]:
//   q = 0..2 sigma/eps (x, y, z), 3..5 sigma (x, y, z), 6 mu, 7 bm1, 8 1/bm1,
//   9 w3*rx/bm1 (the mixed form's normalised residual R: res/bm1 = R * [9]),
//   10 bm1/(w3*rx) (a residual term t enters R as t * [10])
constexpr int kPmlData = 11;
struct PmlDev {
  const int* slot;        // nelt: PML slot of the element, -1 outside
  const double* data;     // kPmlData * n
  double* aux;            // 6 * n: pmlbn, pmldn
  double* k;              // 6 * n: their RK registers
  long n;                 // npml * N3
};

// Graphene sheets in the fused forms: per element row (elements with a listed
// slot or the partner of one), per face node the compact index of the own
// slot and of the partner's slot when listed (-1 otherwise); per listed slot
// g the 12 parameters, Y_0, yconduc, and the face currents fjn(.,m,k) at
// [(3k+m)*ng + g], read from f_in and written to f_out (swapped every stage:
// a face node's two sides read each other's currents), RK registers in k.
struct GrapheneDev {
  const int* elem;
  const int* own;
  const int* part;
  const double *par, *y0, *yc;
  const double* f_in;
  double* f_out;
  double* k;
  long ng;
};

#ifdef __CUDACC__
// cem_3d_graphene_current (src/cem_maxwell.F:2827-2931) at listed slot g with
// unit normal n and face fields fh, fe: adds the surface current J to Jacc;
// with update, also the residuals of the auxiliary currents and their RK
// update (FP64, fused low-storage form).
__device__ inline void graphene_slot(const GrapheneDev& G, long g, const double n[3],
                                     const double fh[3], const double fe[3], bool update,
                                     bool first_stage, double ra, double rb, double dt,
                                     double Jacc[3]) {
  const long ng = G.ng;
  double p[12];
  for (int i = 0; i < 12; ++i) p[i] = G.par[i * ng + g];
  const double nH[3] = {-n[1] * fh[2] + n[2] * fh[1], n[0] * fh[2] - n[2] * fh[0],
                        -n[0] * fh[1] + n[1] * fh[0]};
  const double ndotE = n[0] * fe[0] + n[1] * fe[1] + n[2] * fe[2];
  const double Yfac = 0.5 / G.y0[g];
  const double cpfac = p[2] + p[7];
  const double jnfac = 1.0 - cpfac * Yfac;
  for (int m = 0; m < 3; ++m) {
    double F[6];
    for (int k = 1; k < 6; ++k) F[k] = G.f_in[(3 * k + m) * ng + g];
    const double tmp = Yfac * (nH[m] + G.yc[g] * (fe[m] - n[m] * ndotE));
    const double J0 = (F[1] + F[2] + F[4] - cpfac * tmp) / jnfac;
    Jacc[m] += J0;
    if (!update) continue;
    const double f = tmp - Yfac * J0;
    double R[6];
    R[1] = -p[0] * F[1] + p[1] * f;
    R[2] = F[3] + p[5] * f;
    R[3] = -p[3] * F[2] - p[4] * F[3] + p[6] * f;
    R[4] = F[5] + p[10] * f;
    R[5] = -p[8] * F[4] - p[9] * F[5] + p[11] * f;
    G.f_out[m * ng + g] = J0;
    for (int k = 1; k < 6; ++k) {
      const long o = (3 * k + m) * ng + g;
      const double kh = first_stage ? dt * R[k] : fma(ra, G.k[o], dt * R[k]);
      G.k[o] = kh;
      G.f_out[o] = fma(rb, kh, F[k]);
    }
  }
}
#endif

struct FusedDev {
  int nelt;
  long npts;
  PmlDev pml;
  DispDev disp;
  GrapheneDev gr;
  const int* inc_elem;    // nelt: row of the element in inc_val, -1 without incident faces
  const double* inc_val;  // [row][12][6*nx^2]: the stage's incident face values, H and E
                          // on the own side (0..5) and on the partner's side (6..11)
  const double* u_in;
  double* u_out;
  double* k;            // RK register read
  double* k_out;        // RK register written (== k unless stage data is being kept)
  const double* coef;   // 2*npts: dt*hbm1 then dt*ebm1
  const int* nbr;       // 6*nelt
  const double* egeom;  // 9*nelt
  const float* egeomf;  // 9*nelt, FP32 copy for the mixed form
  const void* fcoef;    // 4 per face node (T), null when uniform
  const int* src_elem;  // nelt: offset (in elements) into src_w or -1; null if no source
  const void* src_w;    // T, nx^3 per source element
  double src_ft;        // amp*ricker(rktime)
  float src_ftf;
  double a, b;          // rk4a(i), rk4b(i)
  double dt;            // for the PML auxiliary fields (coef carries dt for u)
  double C0;
  float C0f;
  int* status;
  double D[kMaxNx * kMaxNx];  // D(i,j) at [i + nx*j]
  double w[kMaxNx];
  float Df[kMaxNx * kMaxNx];  // FP32 copies (no FP64->FP32 conversion in the kernel)
  float wf[kMaxNx];
};

// Mixed form (nekgpu_mixed.cu): exact-hi FP32 contractions on a normalised
// residual; see that file for the scheme.
struct MixedDev {
  int nelt;
  long npts;
  const double* u_in;
  double* u_out;
  double* k;            // RK register read by the stage
  double* k_out;        // where the stage writes it (k itself, or a stage buffer)
  const float2* coef;   // 2*npts (hi, lo) pairs of dt*hbm1*w3*rx | dt*ebm1*w3*rx
  const int* nbr;       // 6*nelt
  const float* egm;     // 16*nelt: rho_y (hi,lo), rho_z (hi,lo), lift factor per slot (6 hi, 6 lo)
  const void* fcoef;    // per face node Y02, C02Y, Z02, C02Z: float4 hi, float4 lo; null when uniform
  const int* src_elem;  // nelt or null
  const float2* src_w;  // normalised source weights as (hi, lo) pairs, nx^3 per source element
  float2 src_ft2;       // time factor of the stage as a (hi, lo) pair
  double a, b;
  float C0f;
  int* status;
  PmlDev pml;
  DispDev disp;
  const int* inc_elem;    // as in FusedDev
  const double* inc_val;
  GrapheneDev gr;
  double dt;
  int e_begin, e_end;  // elements of this launch
};

// Reverse of one FP64 stage (nekgpu_adjoint.cu)
struct AdjointDev {
  int nelt;
  long npts;
  const double* ub_in;   // adjoint of u_i
  double* ub_out;        // adjoint of u_{i-1}
  const double* w_in;    // dt M^-1 (adjoint of k_i + b_i ub_i): the stage-i weights
  double* w_out;         // the same for stage i-1
  const double* u_prev;  // forward u_{i-1}
  const double* k_cur;   // forward k_i
  const double* k_prev;  // forward k_{i-1} (unused when a == 0)
  const double* coef;    // dt hbm1 (npts), dt ebm1 (npts)
  const double* bm1;
  double* deps;          // accumulated dJ/deps per node
  const int* nbr;
  const double* egeom;
  const double* slot;    // [16][nxzfl] static face-slot coefficients as (hi, lo) float pairs
  double a, b_next, inv_dt;
  double Dw[kMaxNx * kMaxNx];  // D(m,i) w_m at [m + NX*i]
  double w[kMaxNx];
};


// Curvilinear hexahedra in the fused FP64 form (nekgpu_curved.cu): per-node
// metrics and per-face-node geometry as the reference holds them
struct CurvedDev {
  int nelt;
  long npts, nxzfl;
  const double* u_in;
  double* u_out;
  double* k;
  const double* coef;     // 2*npts: dt*hbm1 then dt*ebm1
  const double* metrics;  // 9*npts: rx, ry, rz, sx, sy, sz, tx, ty, tz (cofactors)
  const double* w3;       // nx^3
  const double* face;     // 4*nxzfl: unx, uny, unz, area
  const double* fcoef;    // 4*nxzfl: Y02, C02Y, Z02, C02Z
  const int* partner;     // nxzfl: volume node across the face, -1 on PEC faces
  const int* src_elem;    // nelt or null
  const double* src_w;    // nx^3 per source element
  double src_ft;
  double a, b;
  const double* vres;     // 6*npts volume term from the dealiased curl, or null: the curl in-kernel
  double D[kMaxNx * kMaxNx];  // D(i,j) at [i + nx*j]
};

// 2-D TE / TM stage (nekgpu_2d.cu): the reference's ldim = 2 arrays as given
struct Stage2dDev {
  int nx, nelt, imode;  // imode 1 TE (E1, E2, H3), 2 TM (H1, H2, E3)
  long npts, nxzfl;
  const double *D, *Dt, *w3;        // nx^2 each
  const double *rx, *ry, *sx, *sy;  // npts
  const double *unx, *uny, *area, *Z0, *Z1, *Y0, *Y1;  // nxzfl
  const double *ebm1, *hbm1;        // npts
  const int* cemface;               // nxzfl, 0-based volume node
  const int* partner;               // nxzfl: the other slot of the face node, -1 if none
  const int* pec;                   // nxzfl: 1 on PEC slots
  double C0;
  const double* u_in;
  double* u_out;
  double* k;
  double ca, cb, dt;
  const double* src_w;  // npts or null: volume source on E3 (TM) or H3 (TE) (usersrc)
  double src_ft;        // its time factor at the stage time
  // PML (pml_step, the reference's full-size arrays); pml_elem null without
  const int* pml_elem;          // nelt: 1 on PML elements
  const double *pml_sigma;      // 3*npts sigma x, y, z
  const double *eps, *mu, *bm1;  // npts
  double *pml_aux, *pml_k;      // 6*npts pmlbn(3), pmldn(3) and their RK registers
};

struct Context {
  int form = NEKGPU_MIXED;
  int ndim = 3, imode = 3;  // ndim 2: TE (imode 1) or TM (imode 2) quadrilateral mesh
  Stage2dDev s2{};
  bool curved = false;      // fused FP64 form on a curvilinear mesh (nekgpu_curved.cu)
  CurvedDev cargs{};
  int device = 0;
  double* d_vres = nullptr;  // fused FP64 form with the dealiased curl: its volume term
  int nx = 0, nelt = 0;
  long npts = 0, nxzfl = 0;
  double volume = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // host-field step as a wavefront over element chunks (nekgpu_op_rk_host,
  // mixed form): copies in and out on their own streams, one stream per RK
  // stage, one event per chunk copied in and per chunk and stage finished
  cudaStream_t copy_stream = nullptr;      // host to device
  cudaStream_t copy_out_stream = nullptr;  // device to host
  cudaStream_t stage_stream[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  std::vector<cudaEvent_t> chunk_in;       // nchunk
  std::vector<cudaEvent_t> chunk_done;     // 5 * nchunk: stage s of chunk i at s*nchunk + i
  cudaEvent_t chunk_fence[2] = {nullptr, nullptr};  // stream hand-overs before / after
  std::vector<int> chunk_begin;              // nchunk + 1 element offsets
  std::vector<std::vector<int>> chunk_adj;   // per chunk: itself and the chunks of its face partners
  std::vector<int> chunk_in_order;           // order of the copies in
  std::vector<std::pair<int, int>> chunk_launch;  // (stage, chunk) launch order
  // the wavefront step captured as a CUDA graph (pinned host arrays, no
  // time-dependent source), replayed with one launch; keyed by what the
  // captured copies and kernels read: the host arrays, the state parity, dt
  // and the stage arguments (byte copy of margs)
  struct StepGraph {
    double* hn;
    double* en;
    long ld;
    int cur;
    double dt;
    unsigned char margs[sizeof(MixedDev)];
    cudaGraphExec_t exec;
    long launches;  // kernels in the graph
  };
  std::vector<StepGraph> step_graphs;

  // device memory
  double* d_u[2] = {nullptr, nullptr};  // state (plain uses d_u[0] only)
  int cur = 0;
  double* d_k = nullptr;
  double* d_bm1 = nullptr;
  double* d_eps_mu = nullptr;  // 2*npts: eps (=1/(ebm1*bm1)), mu
  double* d_red = nullptr;     // reduction scratch
  int* d_status = nullptr;
  int* h_status = nullptr;  // page-locked copy of d_status[0], read after each sync
  std::vector<void*> allocs;
  std::vector<size_t> alloc_bytes;  // size of each entry of allocs
  size_t dev_bytes = 0;  // device bytes held in allocs

  // fused form
  double* d_coef = nullptr;   // 2*npts, dt-scaled
  double* d_cbase = nullptr;  // 2*npts, the unscaled coefficients of the form
  double* d_hbm1 = nullptr;
  double* d_ebm1 = nullptr;
  double coef_dt = 0.0;
  int* d_nbr = nullptr;
  double* d_egeom = nullptr;
  float* d_egeomf = nullptr;
  void* d_fcoef = nullptr;
  int* d_src_elem = nullptr;
  void* d_src_w = nullptr;
  bool uniform = true;
  int fused_grid = 0;
  FusedDev fargs{};
  MixedDev margs{};
  float* d_egm = nullptr;
  // PML: plain form uses d_pml_sigma/d_eps/d_mu/d_pmlptr/d_pml_res (full
  // size); the fused forms d_pml_slot/d_pml_data; both d_pml_aux/d_pml_k
  // (full size for plain, compact for fused)
  int npml = 0;
  std::vector<int> pml_elems;
  double *d_pml_sigma = nullptr, *d_eps = nullptr, *d_mu = nullptr, *d_pml_res = nullptr;
  int* d_pmlptr = nullptr;
  double *d_pml_aux = nullptr, *d_pml_k = nullptr, *d_pml_data = nullptr;
  int* d_pml_slot = nullptr;
  // dispersive currents: per node model (0 none, 1 Drude, 2 Lorentz) and
  // parameters a, b, c on the host; the device side in DispDev (all forms)
  std::vector<signed char> disp_kind;
  std::vector<double> disp_par;  // 3*npts
  std::vector<int> disp_slot;    // nelt
  std::vector<int> disp_elems;
  double *d_disp_data = nullptr, *d_disp_aux = nullptr, *d_disp_k = nullptr;
  int *d_disp_slot = nullptr, *d_disp_elem = nullptr;
  long disp_n = 0;
  // userinc plane wave amp * cos(k.x - omega t) on listed face slots: the
  // slots and their nodes on the host, the values recomputed every stage
  std::vector<int> inc_slots, inc_nodes;
  std::vector<int> host_cemface;  // plain form: 0-based volume node of each face slot
  double inc_amp[6] = {0, 0, 0, 0, 0, 0}, inc_k[3] = {0, 0, 0}, inc_omega = 0;
  std::vector<int> inc_elem_rows;  // fused forms: the elements with incident faces
  std::vector<long> inc_own_pos, inc_partner_pos;  // fused forms: table positions per slot
  std::vector<int> host_nbr;       // fused forms: 6*nelt partner elements, -1 PEC mirror
  std::vector<double> inc_host;    // staging of the values
  int* d_inc_slot = nullptr;
  int* d_inc_elem = nullptr;
  double* d_inc_val = nullptr;
  // graphene sheets: listed slots on the host; the fused forms' current
  // buffers (two, swapped every stage) and the elements' rows
  std::vector<int> gr_slots;
  double* d_gr_f[2] = {nullptr, nullptr};
  int gr_cur = 0;
  GrapheneDev grdev{};
  // adjoint face-slot coefficients (built on first use, FP64 fused form)
  double* d_adj_slot = nullptr;
  std::vector<double> adj_jw;  // objective weights set by nekgpu_adjoint_init
  int adj_stride = 0;
  int adj_host_snapshots = 0;  // pinned host snapshot slots the binomial schedule may add
  bool adj_mixed_recompute = false;  // fused FP64: the sqrt schedule's segments recomputed in mixed stages
  // mixed form: the FP64 face coefficients (4 per face node, as FusedDev::fcoef)
  // for the adjoint's face-slot table; empty when uniform
  std::vector<double> host_fcoef64;

  // plain form
  PlainDev pargs{};
  double* d_src_w_plain = nullptr;

  Source src;
  std::vector<double> host_bm1, host_x, host_y, host_z;
  std::vector<double> host_w3, host_rx;  // for normalising source weights (mixed form)
  double rk_a[5], rk_b[5], rk_c[6];
  long last_launches = 0;
  bool have_state = false;
};

// host helpers (nekgpu_host.cpp)
int check_cuda(cudaError_t e);
// frees a device allocation of the context (null or foreign pointers ignored)
void release_dev(Context* c, const void* p);
void rk_coeffs(double a[5], double b[5], double c[6]);

// kernel launchers (nekgpu_plain.cu)
int plain_cem_maxwell(Context* c);
int plain_restrict_to_face(Context* c);
// rk = {ca, cb, dt} of the stage: the graphene currents run inside the flux
int plain_flux3d(Context* c, const double* rk = nullptr);
int plain_add_flux_to_res(Context* c);
int plain_usersrc(Context* c, double ft);
int plain_invqmass(Context* c);
int plain_rk_update(Context* c, double ca, double cb, double dt);
int plain_pml_step(Context* c);                                   // pml_step
int plain_pml_rk_update(Context* c, double ca, double cb, double dt);
// shared memory of the dealiased curl kernel for nx1 = mx, lxd = md
size_t dcurl_smem(int mx, int md);
// the dealiased weighted curl (k_dcurl) of state u into res (6*npts, H then E)
int dcurl_into(Context* c, const double* u, double* res);
// cem_maxwell_drude / cem_maxwell_lorentz with the currents' rk4_upd
int plain_dispersive(Context* c, double ca, double cb, double dt);
// userinc: adds the stage's incident values to the restricted face fields
int plain_incident(Context* c);
// computes the incident values of the stage time and uploads them (all forms)
int incident_upload(Context* c, double rktime);
int plain_gs(Context* c, double* d_u, int nfld);

// kernel launchers (nekgpu_fused.cu)
int fused_setup(Context* c);  // grid size / smem attributes
int fused_stage(Context* c, int rkstep, double time, double dt);
// one stage with explicit state / RK-register buffers (no ping-pong bookkeeping)
int fused_stage_buffers(Context* c, int rkstep, double time, double dt, const double* u_in,
                        double* u_out, double* k_in, double* k_out);
int scale_coef(Context* c, double dt);

// nekgpu_mixed.cu
int mixed_stage(Context* c, int rkstep, double time, double dt);
// pair_to_double on n device pairs (default stream)
int pair_join_selftest(const float* s, const float* t, double* out, long n);
// one mixed stage between given buffers (u_in -> u_out, k_in -> k_out), as
// fused_stage_buffers; the context's own state is untouched
int mixed_stage_buffers(Context* c, int rkstep, double time, double dt, const double* u_in,
                        double* u_out, double* k_in, double* k_out);
// the same with explicit stage arguments (coefficient pairs already scaled),
// e.g. those of mixed_companion
int mixed_stage_dev(Context* c, MixedDev a, int rkstep, double time, double dt, const double* u_in,
                    double* u_out, double* k_in, double* k_out);
// coef = (hi, lo) pairs of dt * base (n2 values)
int mixed_scale_pairs(Context* c, float2* coef, const double* base, long n2, double dt);
// The mixed-form stage arguments for an affine fused FP64 context (normalised
// inverse-mass pairs scaled by dt, per-element factors, face coefficient
// pairs, normalised source weight pairs; D's FP32 pieces uploaded): device
// buffers are appended to `owned` for the caller to free.
int mixed_companion(Context* c, double dt, std::vector<void*>& owned, MixedDev& m);
// launches a kernel whose bounded mbarrier wait runs out (sets the status word)
int wait_selftest(Context* c, int polls);
// one mixed stage over elements [e0, e1) of the current state, writing the
// other state buffer without switching to it
int mixed_stage_range(Context* c, int rkstep, double time, double dt, int e0, int e1,
                      bool pdl = false);
// the mixed form keeps dt-scaled coefficients as (hi, lo) float pairs in d_coef
int scale_coef_pairs(Context* c, double dt);
// D(i,j) in three FP32 pieces: Dh on a 10-bit grid per row (exact products
// with the 10-bit uh), Df = D rounded, and the remainder Dm = RN32(D - Dh),
// as float pairs (layout in nekgpu_mixed.cu); uploaded once per nx
int mixed_upload_D(int nx, const float* tab, size_t count);

// nekgpu_curved.cu: one fused FP64 stage on a curvilinear mesh
int curved_stage(Context* c, int rkstep, double time, double dt);
// mixed stage on a curvilinear mesh (curved arrays, FP64 coefficients)
int mixed_curved_stage(Context* c, int rkstep, double time, double dt);

// nekgpu_2d.cu: one 2-D TE / TM stage in the reference's arithmetic
int stage2d(Context* c, int rkstep, double time, double dt);

// nekgpu_adjoint.cu
int adjoint_stage(Context* c, const AdjointDev& a);
// w = b * coef * ub (the stage weights of the last stage of the last step)
int adjoint_seed(Context* c, double* w, const double* ub, const double* coef, double b);
// coef = dt hbm1 | dt ebm1 (2 npts), the FP64 inverse-mass scale of the
// reverse stages, for a context whose own coefficients are float pairs
int adjoint_coef64(Context* c, double* coef, double dt);

// nekgpu_noalloc.cu: cem_error norms with a fixed device scratch array
int norms_noalloc(Context* c, const double* exact_dev, double l2[6], double linf[6]);

// reductions / utilities (nekgpu_util.cu)
int util_norms(Context* c, const double* d_exact, double l2[6], double linf[6]);
int util_energy(Context* c, double* energy);
int util_blowup(Context* c, int* bad);

}  // namespace nekgpu
