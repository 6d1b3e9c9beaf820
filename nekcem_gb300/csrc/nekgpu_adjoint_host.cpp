// Driver of the discrete adjoint (nekgpu_adjoint_gradient): forward pass with
// checkpoints every S steps, objective J = sum jw |E|^2, then a reverse sweep
// that recomputes one segment at a time -- keeping every stage's state and RK
// register of the segment -- and runs the reverse stages (nekgpu_adjoint.cu).
// Memory: ceil(nsteps/S) checkpoints + 2*(5S+1) stage buffers + 5 states.
#include <cuda_runtime.h>

#include <cmath>
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
  if (c->d_fcoef) {
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
  c->d_adj_slot = (double*)pd;
  if (check_cuda(cudaMemcpy(pd, k.data(), k.size() * 8, cudaMemcpyHostToDevice))) return NEKGPU_ERR_CUDA;
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

}  // namespace

extern "C" int nekgpu_adjoint_gradient(nekgpu_ctx* c, int nsteps, double t0, double dt,
                                       const double* jw, double* J, double* dJdeps, int stride,
                                       double* fwd_ms, double* adj_ms) {
  if (!c || !jw || !J || !dJdeps || nsteps < 1 || stride < 0) return NEKGPU_ERR_ARG;
  if (c->form != NEKGPU_FUSED64) return NEKGPU_ERR_UNSUPPORTED;
  if (!c->have_state) return NEKGPU_ERR_STATE;
  int st = build_adjoint_data(c);
  if (st) return st;
  const long npts = c->npts, ns = 6 * npts;
  const int S = stride > 0 ? stride : (int)std::ceil(std::sqrt((double)nsteps));
  const int nseg = (nsteps + S - 1) / S;
  Scratch mem;
  std::vector<double*> ckpt(nseg);
  for (auto& p : ckpt)
    if (!(p = mem.get(ns))) return NEKGPU_ERR_NOMEM;
  double* ub[2] = {mem.get(ns), mem.get(ns)};
  double* wb[2] = {mem.get(ns), mem.get(ns)};
  double* deps = mem.get(npts);
  if (!ub[0] || !ub[1] || !wb[0] || !wb[1] || !deps) return NEKGPU_ERR_NOMEM;
  // segment storage: stage states U and RK registers K of one segment; a
  // second set (when it fits) lets the recompute of the next segment run on a
  // second stream while the reverse stages of this one run
  std::vector<double*> U[2], K[2];
  int nsets = 0;
  for (int b = 0; b < 2; ++b) {
    U[b].resize(5 * S + 1);
    K[b].resize(5 * S + 1);
    bool ok = true;
    for (int i = 0; i <= 5 * S && ok; ++i) ok = (U[b][i] = mem.get(ns)) && (K[b][i] = mem.get(ns));
    if (!ok) break;
    ++nsets;
  }
  if (nsets == 0) return NEKGPU_ERR_NOMEM;
  StreamPair sp;
  if (nsets == 2 && !sp.create()) nsets = 1;
  if ((st = scale_coef(c, dt))) return st;

  // ---- forward pass with checkpoints ------------------------------------------
  std::vector<double> tstep(nsteps);
  double t = t0;
  if (check_cuda(cudaEventRecord(c->ev0, c->stream))) return NEKGPU_ERR_CUDA;
  for (int n = 0; n < nsteps; ++n) {
    if (n % S == 0 && (st = copy_state(c, ckpt[n / S], c->d_u[c->cur]))) return st;
    tstep[n] = t;
    for (int r = 1; r <= 5; ++r)
      if ((st = fused_stage(c, r, t, dt))) return st;
    t = t + dt;
  }
  if (check_cuda(cudaEventRecord(c->ev1, c->stream)) || check_cuda(cudaEventSynchronize(c->ev1)))
    return NEKGPU_ERR_CUDA;
  float f_ms = 0;
  cudaEventElapsedTime(&f_ms, c->ev0, c->ev1);

  // ---- objective and its gradient with respect to the final state -----------
  std::vector<double> uf(ns), ubf(ns, 0.0);
  if (check_cuda(cudaMemcpy(uf.data(), c->d_u[c->cur], ns * 8, cudaMemcpyDeviceToHost)))
    return NEKGPU_ERR_CUDA;
  double Jv = 0.0;
  for (int q = 3; q < 6; ++q)
    for (long g = 0; g < npts; ++g) {
      const double e = uf[q * npts + g];
      Jv += jw[g] * e * e;
      ubf[q * npts + g] = 2.0 * jw[g] * e;
    }
  if (check_cuda(cudaMemcpyAsync(ub[0], ubf.data(), ns * 8, cudaMemcpyHostToDevice, c->stream)) ||
      check_cuda(cudaMemsetAsync(deps, 0, npts * 8, c->stream)))
    return NEKGPU_ERR_CUDA;
  if ((st = adjoint_seed(c, wb[0], ub[0], c->rk_b[4]))) return st;

  // ---- reverse sweep ------------------------------------------------------------
  AdjointDev a{};
  a.nelt = c->nelt;
  a.npts = npts;
  a.coef = c->d_coef;
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
  int cu = 0;
  cudaStream_t main_stream = c->stream;
  // recompute of segment seg into buffer set b, on stream `on`
  auto recompute = [&](int seg, int b, cudaStream_t on) -> int {
    const int n0 = seg * S, nS = std::min(S, nsteps - n0);
    c->stream = on;
    int r = copy_state(c, U[b][0], ckpt[seg]);
    for (int s = 0; s < nS && !r; ++s)
      for (int q = 1; q <= 5 && !r; ++q) {
        const int i = 5 * s + q;
        r = fused_stage_buffers(c, q, tstep[n0 + s], dt, U[b][i - 1], U[b][i], K[b][i - 1], K[b][i]);
      }
    c->stream = main_stream;
    return r;
  };
  auto reverse = [&](int seg, int b) -> int {
    const int n0 = seg * S, nS = std::min(S, nsteps - n0);
    for (int s = nS - 1; s >= 0; --s)
      for (int r = 5; r >= 1; --r) {
        const int i = 5 * s + r;
        a.ub_in = ub[cu];
        a.ub_out = ub[cu ^ 1];
        a.w_in = wb[cu];
        a.w_out = wb[cu ^ 1];
        a.u_prev = U[b][i - 1];
        a.k_cur = K[b][i];
        a.k_prev = K[b][i - 1];
        a.a = c->rk_a[r - 1];
        a.b_next = c->rk_b[r == 1 ? 4 : r - 2];
        int st2 = adjoint_stage(c, a);
        if (st2) return st2;
        cu ^= 1;
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
    if (check_cuda(cudaEventRecord(sp.done_recompute[(nseg - 1) & 1], sp.side))) return NEKGPU_ERR_CUDA;
    for (int seg = nseg - 1; seg >= 0; --seg) {
      const int b = seg & 1;
      if (seg > 0) {
        const int bn = (seg - 1) & 1;
        if (seg + 1 < nseg && check_cuda(cudaStreamWaitEvent(sp.side, sp.done_reverse[bn], 0)))
          return NEKGPU_ERR_CUDA;
        if ((st = recompute(seg - 1, bn, sp.side))) return st;
        if (check_cuda(cudaEventRecord(sp.done_recompute[bn], sp.side))) return NEKGPU_ERR_CUDA;
      }
      if (check_cuda(cudaStreamWaitEvent(main_stream, sp.done_recompute[b], 0))) return NEKGPU_ERR_CUDA;
      if ((st = reverse(seg, b))) return st;
      if (check_cuda(cudaEventRecord(sp.done_reverse[b], main_stream))) return NEKGPU_ERR_CUDA;
    }
  }
  if (check_cuda(cudaEventRecord(c->ev1, c->stream)) || check_cuda(cudaEventSynchronize(c->ev1)))
    return NEKGPU_ERR_CUDA;
  float a_ms = 0;
  cudaEventElapsedTime(&a_ms, c->ev0, c->ev1);
  if (check_cuda(cudaMemcpyAsync(dJdeps, deps, npts * 8, cudaMemcpyDeviceToHost, c->stream)) ||
      check_cuda(cudaStreamSynchronize(c->stream)))
    return NEKGPU_ERR_CUDA;
  int h = 0;
  if (check_cuda(cudaMemcpy(&h, c->d_status, sizeof(int), cudaMemcpyDeviceToHost))) return NEKGPU_ERR_CUDA;
  if (h) return NEKGPU_ERR_TIMEOUT;
  *J = Jv;
  if (fwd_ms) *fwd_ms = f_ms;
  if (adj_ms) *adj_ms = a_ms;
  return NEKGPU_OK;
}

extern "C" int nekgpu_adjoint_init(nekgpu_ctx* c, const double* jw, int stride) {
  if (!c || !jw || stride < 0) return NEKGPU_ERR_ARG;
  if (c->form != NEKGPU_FUSED64) return NEKGPU_ERR_UNSUPPORTED;
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
