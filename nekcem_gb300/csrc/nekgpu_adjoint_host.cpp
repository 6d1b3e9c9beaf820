// Driver of the discrete adjoint (nekgpu_adjoint_gradient).  J = sum jw |E|^2
// at the final time; the reverse stages are in nekgpu_adjoint.cu.  The
// forward steps (first pass and recomputations) run in the context's form:
// the fused FP64 stage, or the mixed stage (whose trajectory agrees with the
// FP64 one to ~1e-10); the reverse stages are FP64 in both.  Two schedules,
// chosen by the device memory available:
//  * sqrt(steps) checkpoints: the forward pass stores the state every S
//    steps; the reverse sweep recomputes one segment at a time, keeping every
//    stage's state and RK register of the segment, and runs its reverse
//    stages (ceil(n/S) + 2 x 2 x (5S+1) + 4 states);
//  * binomial snapshots when that does not fit: a revolve-type schedule over
//    the snapshots that fit, plus any pinned host-memory snapshots the caller
//    allows, with one step's stage storage (15 states + device snapshots);
//    more forward steps are recomputed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "nekgpu_internal.h"

using namespace nekgpu;

struct nekgpu_ctx : public Context {};

namespace {

const int kSlotAxis[6] = {1, 0, 1, 0, 2, 2};
const int kSlotSide[6] = {-1, +1, +1, -1, -1, +1};
const int kSlotOpp[6] = {2, 3, 0, 1, 5, 4};

int face_vol(int f, int a, int b, int n) {
  const int fixed = kSlotSide[f] < 0 ? 0 : n - 1;
  switch (kSlotAxis[f]) {
    case 0: return fixed + n * a + n * n * b;
    case 1: return a + n * fixed + n * n * b;
    default: return a + n * b + n * n * fixed;
  }
}

// Temporary device buffers of one call; freed on every exit path.
struct Scratch {
  std::vector<void*> ptrs;
  ~Scratch() {
    for (void* p : ptrs) cudaFree(p);
  }
  double* get(size_t count) {
    void* p = nullptr;
    if (cudaMalloc(&p, count * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    ptrs.push_back(p);
    return (double*)p;
  }
};

// Static coefficients of every face slot j (element e, slot f, node (a,b)),
// area-weighted, side-signed and stored [16][nxzfl]:
//   0 kH = -A C02Y   1 kHx = A s Z02   2 kE = -A C02Z   3 kEx = A s Y02
//   4 pH = Ap C02Y'  5 pHx = Ap s Z02' 6 pE = Ap C02Z'  7 pEx = Ap s Y02'
//   8 gA = A dC02Y/de-   9 gB = A s dY02/de-   10 gC = A s dZ02/de-  11 gD = A dC02Z/de-
//  12 hA = -Ap dC02Y'/de+  13 hB = Ap s dY02'/de+  14 hC = Ap s dZ02'/de+  15 hD = -Ap dC02Z'/de+
// (A, s: area and side of the slot; primes: the partner slot, whose side is
// -s; de-/de+: derivative with respect to eps at the slot's own node / at its
// partner node).  A PEC slot has no partner and the mirror jump (0, -2 E-):
// its kernel jump is u- itself, so kE, kEx, gB, gD carry the factor -2 and
// kH = kHx = gA = gC = p* = h* = 0.
// The coefficients are those of src/cem_maxwell.F:969-997 built from the face
// impedances of src/cem_maxwell.F:262-325: interior Y02 = -Y+/(Y- + Y+),
// C02Y = C0/(Y- + Y+), Z02 = Z+/(Z- + Z+), C02Z = C0/(Z- + Z+); PEC Y02 = -1/2,
// C02Y = C0/(2Y-), Z02 = 1/2, C02Z = C0/(2Z-); Y = sqrt(eps/mu), Z = sqrt(mu/eps)
// with eps = 1/(ebm1 bm1), mu = 1/(hbm1 bm1).
int build_adjoint_data(Context* c) {
  if (c->d_adj_slot) return NEKGPU_OK;
  const int n = c->nx;
  const long n2 = (long)n * n, n3 = n2 * n, npts = c->npts, nxzfl = c->nxzfl;
  std::vector<double> eb(npts), hb(npts), fc, eg(9 * (size_t)c->nelt);
  std::vector<int> nbr(6 * (size_t)c->nelt);
  if (check_cuda(cudaMemcpy(eb.data(), c->d_ebm1, npts * 8, cudaMemcpyDeviceToHost)) ||
      check_cuda(cudaMemcpy(hb.data(), c->d_hbm1, npts * 8, cudaMemcpyDeviceToHost)) ||
      check_cuda(cudaMemcpy(eg.data(), c->d_egeom, eg.size() * 8, cudaMemcpyDeviceToHost)) ||
      check_cuda(cudaMemcpy(nbr.data(), c->d_nbr, nbr.size() * sizeof(int), cudaMemcpyDeviceToHost)))
    return NEKGPU_ERR_CUDA;
  const double C0 = c->fargs.C0;
  if (c->form == NEKGPU_MIXED) {
    fc = c->host_fcoef64;  // the device holds float pairs
  } else if (c->d_fcoef) {
    fc.resize(4 * (size_t)nxzfl);
    if (check_cuda(cudaMemcpy(fc.data(), c->d_fcoef, fc.size() * 8, cudaMemcpyDeviceToHost)))
      return NEKGPU_ERR_CUDA;
  }
  auto coef = [&](long j, int q) {
    const double def[4] = {-0.5, 0.5 * C0, 0.5, 0.5 * C0};
    return fc.empty() ? def[q] : fc[4 * j + q];
  };
  std::vector<double> eps(npts), mu(npts);
  for (long g = 0; g < npts; ++g) {
    eps[g] = 1.0 / (eb[g] * c->host_bm1[g]);
    mu[g] = 1.0 / (hb[g] * c->host_bm1[g]);
  }
  // d(Y02, C02Y, Z02, C02Z)/d eps at the own node (dm) and at the partner (dp)
  auto derivs = [&](long g, long gp, bool pec, double dm[4], double dp[4]) {
    const double em = eps[g], Ym = std::sqrt(eps[g] / mu[g]), Zm = std::sqrt(mu[g] / eps[g]);
    if (pec) {
      dm[0] = 0.0;
      dm[1] = -C0 / (4.0 * em * Ym);
      dm[2] = 0.0;
      dm[3] = C0 / (4.0 * em * Zm);
      dp[0] = dp[1] = dp[2] = dp[3] = 0.0;
      return;
    }
    const double ep = eps[gp], Yp = std::sqrt(eps[gp] / mu[gp]), Zp = std::sqrt(mu[gp] / eps[gp]);
    const double SY2 = (Ym + Yp) * (Ym + Yp), SZ2 = (Zm + Zp) * (Zm + Zp);
    dm[0] = Yp * Ym / (2.0 * em * SY2);
    dp[0] = -Ym * Yp / (2.0 * ep * SY2);
    dm[1] = -C0 * Ym / (2.0 * em * SY2);
    dp[1] = -C0 * Yp / (2.0 * ep * SY2);
    dm[2] = Zp * Zm / (2.0 * em * SZ2);
    dp[2] = -Zm * Zp / (2.0 * ep * SZ2);
    dm[3] = C0 * Zm / (2.0 * em * SZ2);
    dp[3] = C0 * Zp / (2.0 * ep * SZ2);
  };
  const double* w = c->fargs.w;
  std::vector<double> k(16 * (size_t)nxzfl, 0.0);
  for (long e = 0; e < c->nelt; ++e)
    for (int f = 0; f < 6; ++f) {
      const int pe = nbr[6 * e + f], fp = kSlotOpp[f];
      const double s = kSlotSide[f];
      for (int b = 0; b < n; ++b)
        for (int a = 0; a < n; ++a) {
          const long j = a + (long)n * b + n2 * (f + 6 * e);
          const long g = e * n3 + face_vol(f, a, b, n);
          const double A = eg[9 * e + 3 + f] * w[a] * w[b];
          double dm[4], dp[4], dq[4], dr[4];
          auto K = [&](int m) -> double& { return k[m * nxzfl + j]; };
          if (pe < 0) {
            derivs(g, g, true, dm, dp);
            K(2) = -2.0 * A * coef(j, 3);
            K(3) = 2.0 * A * s * coef(j, 0);
            K(9) = -2.0 * A * s * dm[0];
            K(11) = -2.0 * A * dm[3];
            continue;
          }
          const long gp = (long)pe * n3 + face_vol(fp, a, b, n);
          const long jp = a + (long)n * b + n2 * (fp + 6L * pe);
          const double Ap = eg[9 * (long)pe + 3 + fp] * w[a] * w[b];
          derivs(g, gp, false, dm, dp);    // this slot: own node g, partner gp
          derivs(gp, g, false, dq, dr);    // the partner slot: own node gp, partner g
          K(0) = -A * coef(j, 1);
          K(1) = A * s * coef(j, 2);
          K(2) = -A * coef(j, 3);
          K(3) = A * s * coef(j, 0);
          K(4) = Ap * coef(jp, 1);
          K(5) = Ap * s * coef(jp, 2);
          K(6) = Ap * coef(jp, 3);
          K(7) = Ap * s * coef(jp, 0);
          K(8) = A * dm[1];
          K(9) = A * s * dm[0];
          K(10) = A * s * dm[2];
          K(11) = A * dm[3];
          K(12) = -Ap * dr[1];
          K(13) = Ap * s * dr[0];
          K(14) = Ap * s * dr[2];
          K(15) = -Ap * dr[3];
        }
    }
  void* pd = nullptr;
  if (cudaMalloc(&pd, k.size() * 8) != cudaSuccess) {
    cudaGetLastError();
    return NEKGPU_ERR_NOMEM;
  }
  c->allocs.push_back(pd);
  c->alloc_bytes.push_back(k.size() * 8);
  c->dev_bytes += k.size() * 8;
  c->d_adj_slot = (double*)pd;
  // stored as (hi, lo) float pairs (the same 8 bytes per coefficient): the
  // reverse stage works them in double-float arithmetic
  std::vector<float> kp(2 * k.size());
  for (size_t i = 0; i < k.size(); ++i) {
    kp[2 * i] = (float)k[i];
    kp[2 * i + 1] = (float)(k[i] - (double)kp[2 * i]);
  }
  if (check_cuda(cudaMemcpy(pd, kp.data(), kp.size() * sizeof(float), cudaMemcpyHostToDevice)))
    return NEKGPU_ERR_CUDA;
  return NEKGPU_OK;
}

// second stream and the events that hand buffer sets between the streams
struct StreamPair {
  cudaStream_t side = nullptr;
  cudaEvent_t done_recompute[2] = {nullptr, nullptr}, done_reverse[2] = {nullptr, nullptr};
  bool create() {
    if (cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking) != cudaSuccess) return fail();
    for (int b = 0; b < 2; ++b)
      if (cudaEventCreateWithFlags(&done_recompute[b], cudaEventDisableTiming) != cudaSuccess ||
          cudaEventCreateWithFlags(&done_reverse[b], cudaEventDisableTiming) != cudaSuccess)
        return fail();
    return true;
  }
  bool fail() {
    cudaGetLastError();
    return false;
  }
  ~StreamPair() {
    if (side) cudaStreamSynchronize(side);
    for (int b = 0; b < 2; ++b) {
      if (done_recompute[b]) cudaEventDestroy(done_recompute[b]);
      if (done_reverse[b]) cudaEventDestroy(done_reverse[b]);
    }
    if (side) cudaStreamDestroy(side);
  }
};

int copy_state(Context* c, double* dst, const double* src) {
  return check_cuda(cudaMemcpyAsync(dst, src, 6 * c->npts * sizeof(double),
                                    cudaMemcpyDeviceToDevice, c->stream));
}

// A snapshot slot of the binomial schedule: device memory, or pinned host
// memory (reached over the host link; one copy each way per use).
struct Slot {
  double* p = nullptr;
  bool host = false;
};

// state copy between a slot and a device buffer, on the context stream
int copy_slot(Context* c, double* dst, bool dst_host, const double* src, bool src_host) {
  const cudaMemcpyKind kind = src_host ? cudaMemcpyHostToDevice
                                       : (dst_host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice);
  return check_cuda(cudaMemcpyAsync(dst, src, 6 * c->npts * sizeof(double), kind, c->stream));
}

// Pinned host snapshots of one call; freed on every exit path (cudaFreeHost
// waits for the device).
struct HostSlots {
  std::vector<void*> ptrs;
  ~HostSlots() {
    for (void* p : ptrs) cudaFreeHost(p);
  }
  double* get(size_t count) {
    void* p = nullptr;
    if (cudaHostAlloc(&p, count * sizeof(double), cudaHostAllocDefault) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    ptrs.push_back(p);
    return (double*)p;
  }
};

// forward stages in the context's form
int fwd_stage(Context* c, int r, double t, double dt) {
  return c->form == NEKGPU_MIXED ? mixed_stage(c, r, t, dt) : fused_stage(c, r, t, dt);
}
int fwd_stage_buffers(Context* c, int r, double t, double dt, const double* u_in, double* u_out,
                      double* k_in, double* k_out) {
  return c->form == NEKGPU_MIXED ? mixed_stage_buffers(c, r, t, dt, u_in, u_out, k_in, k_out)
                                 : fused_stage_buffers(c, r, t, dt, u_in, u_out, k_in, k_out);
}

}  // namespace

namespace {

// Device bytes a gradient evaluation may allocate: the free device memory
// less a 1 GB margin, and under NEKGPU_MEM_BUDGET_MB what that budget leaves
// after the context's own allocations.
size_t adjoint_budget(const Context* c) {
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    cudaGetLastError();
    free_b = 0;
  }
  size_t avail = free_b > (size_t(1) << 30) ? free_b - (size_t(1) << 30) : 0;
  if (const char* b = std::getenv("NEKGPU_MEM_BUDGET_MB")) {
    const size_t budget = (size_t)std::atoll(b) << 20;
    avail = std::min(avail, budget > c->dev_bytes ? budget - c->dev_bytes : size_t(0));
  }
  return avail;
}

// beta(s, t) = C(s + t, s): steps a binomial schedule with s free snapshots
// reverses with at most t recomputations of each step
double beta(int s, int t) {
  double r = 1.0;
  for (int i = 1; i <= s; ++i) r = r * (t + i) / i;
  return r;
}

// State shared by the reverse sweeps of one gradient evaluation.
struct Sweep {
  Context* c;
  int nsteps;
  double dt;
  const double* jw;
  std::vector<double> tstep;  // time at the start of each step (time += dt, as nekgpu_step)
  double* ub[2];
  double* wb[2];
  double* deps;
  const double* coef64 = nullptr;  // dt hbm1 | dt ebm1 in FP64
  int cu = 0;
  AdjointDev a{};
  double J = 0.0;
  bool seeded = false;
  std::vector<double> final_host;  // u(T), read back by the seed

  // J and the adjoint seed from the final state: ub = (0, 2 jw E), w = b_5 dt M^-1 ub
  int seed(const double* u_final) {
    const long npts = c->npts, ns = 6 * npts;
    std::vector<double>& uf = final_host;
    std::vector<double> ubf(ns, 0.0);
    uf.resize(ns);
    if (check_cuda(cudaMemcpyAsync(uf.data(), u_final, ns * 8, cudaMemcpyDeviceToHost, c->stream)) ||
        check_cuda(cudaStreamSynchronize(c->stream)))
      return NEKGPU_ERR_CUDA;
    double Jv = 0.0;
    for (int q = 3; q < 6; ++q)
      for (long g = 0; g < npts; ++g) {
        const double e = uf[q * npts + g];
        Jv += jw[g] * e * e;
        ubf[q * npts + g] = 2.0 * jw[g] * e;
      }
    J = Jv;
    if (check_cuda(cudaMemcpyAsync(ub[0], ubf.data(), ns * 8, cudaMemcpyHostToDevice, c->stream)) ||
        check_cuda(cudaMemsetAsync(deps, 0, npts * 8, c->stream)) ||
        check_cuda(cudaStreamSynchronize(c->stream)))
      return NEKGPU_ERR_CUDA;
    cu = 0;
    seeded = true;
    return adjoint_seed(c, wb[0], ub[0], coef64, c->rk_b[4]);
  }

  // the five reverse stages of step j from its stage states (U[0..4]) and
  // RK registers (K[1..5])
  int reverse_step(double* const* U, double* const* K) {
    for (int r = 5; r >= 1; --r) {
      a.ub_in = ub[cu];
      a.ub_out = ub[cu ^ 1];
      a.w_in = wb[cu];
      a.w_out = wb[cu ^ 1];
      a.u_prev = U[r - 1];
      a.k_cur = K[r];
      a.k_prev = K[r - 1];
      a.a = c->rk_a[r - 1];
      a.b_next = c->rk_b[r == 1 ? 4 : r - 2];
      int st = adjoint_stage(c, a);
      if (st) return st;
      cu ^= 1;
    }
    return NEKGPU_OK;
  }

  void init_args() {
    a.nelt = c->nelt;
    a.npts = c->npts;
    a.coef = coef64;
    a.bm1 = c->d_bm1;
    a.deps = deps;
    a.nbr = c->d_nbr;
    a.egeom = c->d_egeom;
    a.slot = c->d_adj_slot;
    a.inv_dt = 1.0 / dt;
    const int n = c->nx;
    for (int i = 0; i < n; ++i) {
      a.w[i] = c->fargs.w[i];
      for (int m = 0; m < n; ++m) a.Dw[m + n * i] = c->fargs.D[m + n * i] * c->fargs.w[m];
    }
  }
};

// Binomial (revolve-type) schedule for meshes whose sqrt(steps) segment
// storage does not fit: snapshots of the state at chosen steps, one step's
// stage storage, and the forward steps between snapshots recomputed.
struct Binomial {
  Sweep& w;
  std::vector<Slot> free_slots;  // device slots first: the deepest levels take them
  double* SU[6];  // stage states of one step: SU[0] is the step's start state, SU[5] its end
  double* SK[6];  // RK registers; SK[0], read (never used) by stage 1, aliases SK[5]
  double* scratch;  // device: a recomputed step start, or a host snapshot brought in
  cudaEvent_t ev_seed = nullptr;
  // the slot whose state the working buffer d_u[cur] holds (the snapshot an
  // advance just wrote): a later read of that slot skips its copy back
  const double* resident = nullptr;

  int advance(Slot src, int j0, int k, Slot dst) {
    Context* c = w.c;
    int st = resident == src.p ? NEKGPU_OK : copy_slot(c, c->d_u[c->cur], false, src.p, src.host);
    for (int j = j0; j < j0 + k && !st; ++j)
      for (int r = 1; r <= 5 && !st; ++r) st = fwd_stage(c, r, w.tstep[j], w.dt);
    if (!st) st = copy_slot(c, dst.p, dst.host, c->d_u[c->cur], false);
    resident = st ? nullptr : dst.p;
    return st;
  }

  int step(int j, Slot src) {
    Context* c = w.c;
    int st = NEKGPU_OK;
    SU[0] = src.p;
    if (src.host) {
      if (resident == src.p) {  // the stages read the working buffer; it stays as it is
        SU[0] = c->d_u[c->cur];
      } else {
        if ((st = copy_slot(c, scratch, false, src.p, true))) return st;
        SU[0] = scratch;
      }
    }
    for (int r = 1; r <= 5 && !st; ++r)
      st = fwd_stage_buffers(c, r, w.tstep[j], w.dt, SU[r - 1], SU[r], SK[r - 1], SK[r]);
    if (st) return st;
    if (!w.seeded) {  // the first step reversed is the last one: its output is u(T)
      if ((st = w.seed(SU[5]))) return st;
      if (check_cuda(cudaEventRecord(ev_seed, c->stream))) return NEKGPU_ERR_CUDA;
    }
    return w.reverse_step(SU, SK);
  }

  // reverse steps b-1 .. a; the state at step a is in `sa`; s free snapshots
  int rev(int a, int b, Slot sa, int s) {
    const int n = b - a;
    if (n == 1) return step(a, sa);
    if (s == 0 || free_slots.empty()) {
      const Slot sc{scratch, false};
      for (int j = b - 1; j >= a; --j) {
        int st = j > a ? advance(sa, a, j - a, sc) : NEKGPU_OK;
        if (!st) st = step(j, j > a ? sc : sa);
        if (st) return st;
      }
      return NEKGPU_OK;
    }
    int t = 1;
    while (beta(s, t) < n) ++t;
    const int right = (int)std::min<double>(beta(s - 1, t), (double)(n - 1));
    const int m = b - right;
    const Slot sm = free_slots.back();
    free_slots.pop_back();
    int st = advance(sa, a, m - a, sm);
    if (!st) st = rev(m, b, sm, s - 1);
    free_slots.push_back(sm);
    if (!st) st = rev(a, m, sa, s);
    return st;
  }
};

}  // namespace

extern "C" int nekgpu_adjoint_gradient(nekgpu_ctx* c, int nsteps, double t0, double dt,
                                       const double* jw, double* J, double* dJdeps, int stride,
                                       double* fwd_ms, double* adj_ms) {
  if (!c || !jw || !J || !dJdeps || nsteps < 1) return NEKGPU_ERR_ARG;
  // no adjoint through PML or dispersive currents
  if ((c->form != NEKGPU_FUSED64 && c->form != NEKGPU_MIXED) || c->npml || c->disp_n ||
      c->ndim == 2 || c->curved || !c->inc_slots.empty() || c->grdev.ng)
    return NEKGPU_ERR_UNSUPPORTED;
  const bool mixed = c->form == NEKGPU_MIXED;
  if (!c->have_state) return NEKGPU_ERR_STATE;
  int st = build_adjoint_data(c);
  if (st) return st;
  const long npts = c->npts, ns = 6 * npts;
  const double state_b = (double)ns * 8;

  // ---- memory plan ----------------------------------------------------------------
  // sqrt scheme: ceil(n/S) checkpoints + sets x 2 x (5S+1) segment states +
  // 4 adjoint states; binomial scheme: 4 adjoint + 10 stage + 1 scratch
  // states + device snapshots (+ the pinned host snapshots allowed by
  // nekgpu_adjoint_host_snapshots).  Both also hold dJ/deps (npts doubles)
  // and, for the mixed form, the FP64 inverse-mass scale (2 npts doubles).
  // stride > 0: segments of `stride` steps; 0: sqrt(steps) segments if they
  // fit, else the binomial schedule with the snapshots that fit; < 0: the
  // binomial schedule with -stride device snapshots.
  // fused FP64 with mixed recomputation: the mixed stage arguments of the
  // context (coefficient pairs and their FP64 base, 32 B per face node of
  // face coefficient pairs) -- about 32 + 4.5 * 6/nx bytes per node
  const bool hybrid = !mixed && c->adj_mixed_recompute;
  const double hybrid_b = hybrid ? (32.0 + 32.0 * 6.0 / c->nx) * npts : 0.0;
  const double avail = (double)adjoint_budget(c) - (double)npts * 8 - (mixed ? 16.0 * npts : 0.0) - hybrid_b;
  const int S = stride > 0 ? stride : (int)std::ceil(std::sqrt((double)nsteps));
  const int nseg = (nsteps + S - 1) / S;
  auto sqrt_states = [&](int sets) { return (double)nseg + 4.0 + sets * 2.0 * (5.0 * S + 1.0); };
  int nsets = 0;
  if (stride >= 0) {
    if (sqrt_states(2) * state_b <= avail) nsets = 2;
    else if (sqrt_states(1) * state_b <= avail) nsets = 1;
    else if (stride > 0) return NEKGPU_ERR_NOMEM;  // the caller fixed the stride
  }
  int ndev = 0, nhost = 0;
  if (nsets == 0) {
    const double fit = std::floor(avail / state_b - 15.0);
    if (fit < 0) return NEKGPU_ERR_NOMEM;  // not even the stage storage
    ndev = (int)std::min<double>(stride < 0 ? -(double)stride : fit, (double)nsteps);
    if (ndev > fit) return NEKGPU_ERR_NOMEM;
    nhost = std::min(c->adj_host_snapshots, nsteps - ndev);
    if (ndev + nhost < 1) return NEKGPU_ERR_NOMEM;
  }

  Scratch mem;
  Sweep w{c, nsteps, dt, jw};
  w.tstep.resize(nsteps);
  {
    double t = t0;
    for (int n = 0; n < nsteps; ++n) {
      w.tstep[n] = t;
      t = t + dt;
    }
  }
  w.ub[0] = mem.get(ns);
  w.ub[1] = mem.get(ns);
  w.wb[0] = mem.get(ns);
  w.wb[1] = mem.get(ns);
  w.deps = mem.get(npts);
  if (!w.ub[0] || !w.ub[1] || !w.wb[0] || !w.wb[1] || !w.deps) return NEKGPU_ERR_NOMEM;
  if (mixed) {  // the context's coefficients are float pairs: an FP64 copy for the reverse
    double* cf = mem.get(2 * npts);
    if (!cf) return NEKGPU_ERR_NOMEM;
    if ((st = scale_coef_pairs(c, dt)) || (st = adjoint_coef64(c, cf, dt))) return st;
    w.coef64 = cf;
  } else {
    if ((st = scale_coef(c, dt))) return st;
    w.coef64 = c->d_coef;
  }
  w.init_args();
  float f_ms = 0, a_ms = 0;

  if (nsets == 0) {
    // ---- binomial schedule -------------------------------------------------------
    Binomial bs{w};
    for (int r = 1; r <= 5; ++r)
      if (!(bs.SU[r] = mem.get(ns)) || !(bs.SK[r] = mem.get(ns))) return NEKGPU_ERR_NOMEM;
    bs.SK[0] = bs.SK[5];
    if (!(bs.scratch = mem.get(ns))) return NEKGPU_ERR_NOMEM;
    HostSlots hmem;
    std::vector<Slot> slots(ndev + nhost);
    for (int q = 0; q < ndev + nhost; ++q) {
      slots[q].host = q >= ndev;
      slots[q].p = slots[q].host ? hmem.get(ns) : mem.get(ns);
      if (!slots[q].p) return NEKGPU_ERR_NOMEM;
    }
    bs.free_slots.assign(slots.begin() + 1, slots.end());
    if (check_cuda(cudaEventCreate(&bs.ev_seed))) return NEKGPU_ERR_CUDA;
    struct EvGuard {
      cudaEvent_t e;
      ~EvGuard() { cudaEventDestroy(e); }
    } guard{bs.ev_seed};
    if (check_cuda(cudaEventRecord(c->ev0, c->stream))) return NEKGPU_ERR_CUDA;
    if ((st = copy_slot(c, slots[0].p, slots[0].host, c->d_u[c->cur], false))) return st;
    bs.resident = slots[0].p;
    if ((st = bs.rev(0, nsteps, slots[0], ndev + nhost - 1))) return st;
    // u(T) back into the context (the seed read it to the host)
    if (check_cuda(cudaMemcpyAsync(c->d_u[c->cur], w.final_host.data(), ns * 8,
                                   cudaMemcpyHostToDevice, c->stream)))
      return NEKGPU_ERR_CUDA;
    if (check_cuda(cudaEventRecord(c->ev1, c->stream)) || check_cuda(cudaEventSynchronize(c->ev1)))
      return NEKGPU_ERR_CUDA;
    cudaEventElapsedTime(&f_ms, c->ev0, bs.ev_seed);
    cudaEventElapsedTime(&a_ms, bs.ev_seed, c->ev1);
  } else {
    // ---- sqrt(steps) checkpoints with segment storage ---------------------------
    std::vector<double*> ckpt(nseg);
    for (auto& p : ckpt)
      if (!(p = mem.get(ns))) return NEKGPU_ERR_NOMEM;
    // segment storage: stage states U and RK registers K of one segment; the
    // second set lets the recompute of the next segment run on a second
    // stream while the reverse stages of this one run
    std::vector<double*> U[2], K[2];
    for (int b = 0; b < nsets; ++b) {
      U[b].resize(5 * S + 1);
      K[b].resize(5 * S + 1);
      for (int i = 0; i <= 5 * S; ++i)
        if (!(U[b][i] = mem.get(ns)) || !(K[b][i] = mem.get(ns))) return NEKGPU_ERR_NOMEM;
    }
    StreamPair sp;
    if (nsets == 2 && !sp.create()) nsets = 1;
    // the recomputed segments in mixed stages (fused FP64 contexts that ask
    // for it): the first pass, J and the checkpoints stay FP64; the stage
    // states the reverse stages read come from mixed steps started at the
    // FP64 checkpoints (within ~1e-10 per step of the FP64 ones)
    MixedDev comp{};
    if (hybrid && (st = mixed_companion(c, dt, mem.ptrs, comp))) return st;

    // forward pass with checkpoints
    if (check_cuda(cudaEventRecord(c->ev0, c->stream))) return NEKGPU_ERR_CUDA;
    for (int n = 0; n < nsteps; ++n) {
      if (n % S == 0 && (st = copy_state(c, ckpt[n / S], c->d_u[c->cur]))) return st;
      for (int r = 1; r <= 5; ++r)
        if ((st = fwd_stage(c, r, w.tstep[n], dt))) return st;
    }
    if (check_cuda(cudaEventRecord(c->ev1, c->stream)) || check_cuda(cudaEventSynchronize(c->ev1)))
      return NEKGPU_ERR_CUDA;
    cudaEventElapsedTime(&f_ms, c->ev0, c->ev1);
    if ((st = w.seed(c->d_u[c->cur]))) return st;

    cudaStream_t main_stream = c->stream;
    // recompute of segment seg into buffer set b, on stream `on`
    auto recompute = [&](int seg, int b, cudaStream_t on) -> int {
      const int n0 = seg * S, nS = std::min(S, nsteps - n0);
      c->stream = on;
      int r = copy_state(c, U[b][0], ckpt[seg]);
      for (int s2 = 0; s2 < nS && !r; ++s2)
        for (int q = 1; q <= 5 && !r; ++q) {
          const int i = 5 * s2 + q;
          r = hybrid ? mixed_stage_dev(c, comp, q, w.tstep[n0 + s2], dt, U[b][i - 1], U[b][i],
                                       K[b][i - 1], K[b][i])
                     : fwd_stage_buffers(c, q, w.tstep[n0 + s2], dt, U[b][i - 1], U[b][i],
                                         K[b][i - 1], K[b][i]);
        }
      c->stream = main_stream;
      return r;
    };
    auto reverse = [&](int seg, int b) -> int {
      const int n0 = seg * S, nS = std::min(S, nsteps - n0);
      for (int s2 = nS - 1; s2 >= 0; --s2) {
        const int st2 = w.reverse_step(&U[b][5 * s2], &K[b][5 * s2]);
        if (st2) return st2;
      }
      return NEKGPU_OK;
    };
    if (check_cuda(cudaEventRecord(c->ev0, c->stream))) return NEKGPU_ERR_CUDA;
    if (nsets == 1) {
      for (int seg = nseg - 1; seg >= 0; --seg)
        if ((st = recompute(seg, 0, main_stream)) || (st = reverse(seg, 0))) return st;
    } else {
      // set b = seg & 1.  side stream: recompute(seg) after reverse(seg + 2)
      // released set b; main stream: reverse(seg) after recompute(seg).
      if (check_cuda(cudaStreamWaitEvent(sp.side, c->ev0, 0))) return NEKGPU_ERR_CUDA;
      if ((st = recompute(nseg - 1, (nseg - 1) & 1, sp.side))) return st;
      if (check_cuda(cudaEventRecord(sp.done_recompute[(nseg - 1) & 1], sp.side)))
        return NEKGPU_ERR_CUDA;
      for (int seg = nseg - 1; seg >= 0; --seg) {
        const int b = seg & 1;
        if (seg > 0) {
          const int bn = (seg - 1) & 1;
          if (seg + 1 < nseg && check_cuda(cudaStreamWaitEvent(sp.side, sp.done_reverse[bn], 0)))
            return NEKGPU_ERR_CUDA;
          if ((st = recompute(seg - 1, bn, sp.side))) return st;
          if (check_cuda(cudaEventRecord(sp.done_recompute[bn], sp.side))) return NEKGPU_ERR_CUDA;
        }
        if (check_cuda(cudaStreamWaitEvent(main_stream, sp.done_recompute[b], 0)))
          return NEKGPU_ERR_CUDA;
        if ((st = reverse(seg, b))) return st;
        if (check_cuda(cudaEventRecord(sp.done_reverse[b], main_stream))) return NEKGPU_ERR_CUDA;
      }
    }
    if (check_cuda(cudaEventRecord(c->ev1, c->stream)) || check_cuda(cudaEventSynchronize(c->ev1)))
      return NEKGPU_ERR_CUDA;
    cudaEventElapsedTime(&a_ms, c->ev0, c->ev1);
  }

  if (check_cuda(cudaMemcpyAsync(dJdeps, w.deps, npts * 8, cudaMemcpyDeviceToHost, c->stream)) ||
      check_cuda(cudaStreamSynchronize(c->stream)))
    return NEKGPU_ERR_CUDA;
  int h = 0;
  if (check_cuda(cudaMemcpy(&h, c->d_status, sizeof(int), cudaMemcpyDeviceToHost))) return NEKGPU_ERR_CUDA;
  if (h) return NEKGPU_ERR_TIMEOUT;
  *J = w.J;
  if (fwd_ms) *fwd_ms = f_ms;
  if (adj_ms) *adj_ms = a_ms;
  return NEKGPU_OK;
}

extern "C" int nekgpu_adjoint_recompute_mixed(nekgpu_ctx* c, int on) {
  if (!c) return NEKGPU_ERR_ARG;
  if (on && (c->form != NEKGPU_FUSED64 || c->curved || c->ndim != 3)) return NEKGPU_ERR_UNSUPPORTED;
  c->adj_mixed_recompute = on != 0;
  return NEKGPU_OK;
}

extern "C" int nekgpu_adjoint_host_snapshots(nekgpu_ctx* c, int n) {
  if (!c || n < 0 || n > (1 << 16)) return NEKGPU_ERR_ARG;
  c->adj_host_snapshots = n;
  return NEKGPU_OK;
}

extern "C" int nekgpu_adjoint_init(nekgpu_ctx* c, const double* jw, int stride) {
  if (!c || !jw) return NEKGPU_ERR_ARG;
  if (c->form != NEKGPU_FUSED64 && c->form != NEKGPU_MIXED) return NEKGPU_ERR_UNSUPPORTED;
  c->adj_jw.assign(jw, jw + c->npts);
  c->adj_stride = stride;
  return NEKGPU_OK;
}

extern "C" int nekgpu_adjoint_run(nekgpu_ctx* c, int nsteps, double t0, double dt, double* J,
                                  double* dJdeps) {
  if (!c || !J || !dJdeps) return NEKGPU_ERR_ARG;
  if (c->adj_jw.empty()) return NEKGPU_ERR_STATE;
  return nekgpu_adjoint_gradient(c, nsteps, t0, dt, c->adj_jw.data(), J, dJdeps, c->adj_stride,
                                 nullptr, nullptr);
}
