// Host runtime of the GB300 Maxwell DG library: the C ABI of nekcem_gpu.h.
//
// Responsibilities: validate and upload the reference's static arrays
// (nekgpu_init) or build a structured box case (nekgpu_init_box), own the
// device memory and the stream, and drive the stage kernels.  No arithmetic
// of the time step runs here.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "nekgpu_internal.h"

using namespace nekgpu;

struct nekgpu_ctx : public Context {};

namespace nekgpu {

static thread_local std::string g_last_cuda;

int check_cuda(cudaError_t e) {
  if (e == cudaSuccess) return NEKGPU_OK;
  g_last_cuda = cudaGetErrorString(e);
  return NEKGPU_ERR_CUDA;
}

void release_dev(Context* c, const void* p) {
  if (!p) return;
  for (size_t i = 0; i < c->allocs.size(); ++i)
    if (c->allocs[i] == p) {
      cudaFree(c->allocs[i]);  // synchronises: no launch still reads it
      c->dev_bytes -= c->alloc_bytes[i];
      c->allocs.erase(c->allocs.begin() + i);
      c->alloc_bytes.erase(c->alloc_bytes.begin() + i);
      return;
    }
}

int incident_upload(Context* c, double rktime) {
  const long n = (long)c->inc_slots.size();
  if (!n) return NEKGPU_OK;
  const long NF = 6L * c->nx * c->nx;
  const bool plain = c->form == NEKGPU_PLAIN;
  for (long q = 0; q < n; ++q) {
    const long i = c->inc_nodes[q];
    const double ph = c->inc_k[0] * c->host_x[i] + c->inc_k[1] * c->host_y[i] +
                      c->inc_k[2] * c->host_z[i] - c->inc_omega * rktime;
    const double u = std::cos(ph);
    if (plain) {
      for (int m = 0; m < 6; ++m) c->inc_host[6 * q + m] = c->inc_amp[m] * u;
    } else {
      for (int m = 0; m < 6; ++m) c->inc_host[c->inc_own_pos[q] + m * NF] = c->inc_amp[m] * u;
      if (c->inc_partner_pos[q] >= 0)
        for (int m = 0; m < 6; ++m) c->inc_host[c->inc_partner_pos[q] + m * NF] = c->inc_amp[m] * u;
    }
  }
  return check_cuda(cudaMemcpyAsync(c->d_inc_val, c->inc_host.data(),
                                    c->inc_host.size() * sizeof(double), cudaMemcpyHostToDevice,
                                    c->stream));
}

// rk_storage, RK45 branch (src/cem_common.F:78-104): Carpenter-Kennedy
// 5-stage 4th-order low-storage coefficients.
void rk_coeffs(double a[5], double b[5], double c[6]) {
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

}  // namespace nekgpu

namespace {

// face slot (reference order) -> axis (0=r,1=s,2=t), side, opposite slot
const int kSlotAxis[6] = {1, 0, 1, 0, 2, 2};
const int kSlotSide[6] = {-1, +1, +1, -1, -1, +1};
const int kSlotOpp[6] = {2, 3, 0, 1, 5, 4};

int face_vol(int f, int a, int b, int n) {
  int fixed = kSlotSide[f] < 0 ? 0 : n - 1;
  switch (kSlotAxis[f]) {
    case 0: return fixed + n * a + n * n * b;
    case 1: return a + n * fixed + n * n * b;
    default: return a + n * b + n * n * fixed;
  }
}

// ---------------------------------------------------------------------------
// GLL points, weights and derivative matrix for the box builder: interior
// points are the roots of P_N' (Newton on the Legendre recurrence, started at
// the Chebyshev-Gauss-Lobatto points), w_i = 2/(N(N+1) P_N(z_i)^2), and
// D(i,j) = P_N(z_i)/(P_N(z_j)(z_i-z_j)), D(0,0) = -N(N+1)/4,
// D(N,N) = N(N+1)/4 (the same D as DGLL, src/nek5_speclib.F:807-840).
// ---------------------------------------------------------------------------
void legendre(int N, double x, double* p, double* dp) {
  double p0 = 1.0, p1 = x;
  if (N == 0) { *p = 1.0; *dp = 0.0; return; }
  for (int k = 1; k < N; ++k) {
    double p2 = ((2.0 * k + 1.0) * x * p1 - k * p0) / (k + 1.0);
    p0 = p1;
    p1 = p2;
  }
  *p = p1;
  // P_N'(x) = N (x P_N - P_{N-1}) / (x^2 - 1), valid inside (-1,1)
  *dp = (std::fabs(x) < 1.0) ? N * (x * p1 - p0) / (x * x - 1.0) : 0.5 * N * (N + 1.0) * (x > 0 ? 1.0 : (N % 2 ? 1.0 : -1.0));
}

void gll(int N, std::vector<double>& z, std::vector<double>& w, std::vector<double>& D) {
  const int n = N + 1;
  const double pi = 4.0 * std::atan(1.0);
  z.assign(n, 0.0);
  w.assign(n, 0.0);
  z[0] = -1.0;
  z[N] = 1.0;
  for (int i = 1; i < N; ++i) {
    double x = -std::cos(pi * i / N);
    for (int it = 0; it < 100; ++it) {
      double p, dp;
      legendre(N, x, &p, &dp);
      // P_N'' from (1-x^2) P'' = 2x P' - N(N+1) P
      double d2p = (2.0 * x * dp - N * (N + 1.0) * p) / (1.0 - x * x);
      double dx = dp / d2p;
      x -= dx;
      if (std::fabs(dx) < 1e-16) break;
    }
    z[i] = x;
  }
  for (int i = 0; i < n / 2; ++i) {  // symmetrise
    double s = 0.5 * (z[N - i] - z[i]);
    z[i] = -s;
    z[N - i] = s;
  }
  if (n % 2) z[N / 2] = 0.0;
  for (int i = 0; i < n; ++i) {
    double p, dp;
    legendre(N, z[i], &p, &dp);
    w[i] = 2.0 / (N * (N + 1.0) * p * p);
  }
  D.assign((size_t)n * n, 0.0);
  std::vector<double> pn(n);
  for (int i = 0; i < n; ++i) {
    double dp;
    legendre(N, z[i], &pn[i], &dp);
  }
  const double d0 = N * (N + 1.0) / 4.0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double v = 0.0;
      if (i != j) v = pn[i] / (pn[j] * (z[i] - z[j]));
      if (i == j && i == 0) v = -d0;
      if (i == j && i == N) v = d0;
      D[i + (size_t)n * j] = v;
    }
}

// impedance combination of cem_maxwell_materials (src/cem_maxwell.F:262-325)
// for one face node: own (Zm, Ym) and partner (Zp, Yp); wall = 1 on a 'PEC'
// face (Z_0 = 2 Z-), 2 on a 'PML' face (a singleton of the gs sum, no
// doubling: Z_0 = Z-, so Z_1 = 0).
void face_impedance(double Zm, double Ym, double Zp, double Yp, int wall, double C0, double out[4]) {
  double Z0 = wall == 1 ? 2.0 * Zm : (wall == 2 ? Zm : Zm + Zp);
  double Y0 = wall == 1 ? 2.0 * Ym : (wall == 2 ? Ym : Ym + Yp);
  double Z1 = Z0 - Zm, Y1 = Y0 - Ym;
  Z0 = 0.5 * Z0;
  Y0 = 0.5 * Y0;
  out[0] = -0.5 / Y0 * Y1;  // Y02
  out[1] = 0.5 / Y0 * C0;   // C02Y
  out[2] = 0.5 / Z0 * Z1;   // Z02
  out[3] = 0.5 / Z0 * C0;   // C02Z
}

struct DevAlloc {
  Context* c;
  size_t budget, used = 0;
  explicit DevAlloc(Context* cc) : c(cc) {
    const char* b = std::getenv("NEKGPU_MEM_BUDGET_MB");
    budget = b ? (size_t)std::atoll(b) << 20 : (size_t)-1;
  }
  template <typename T>
  int get(T** p, size_t count) {
    size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
    if (used + bytes > budget) return NEKGPU_ERR_NOMEM;
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return NEKGPU_ERR_NOMEM;
    }
    used += bytes;
    c->dev_bytes += bytes;
    c->allocs.push_back(q);
    c->alloc_bytes.push_back(bytes);
    *p = (T*)q;
    return NEKGPU_OK;
  }
  template <typename T>
  int put(T** p, const std::vector<T>& h) {
    int st = get(p, h.size());
    if (st) return st;
    if (!h.empty())
      return check_cuda(cudaMemcpy(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    return NEKGPU_OK;
  }
};

void drop_step_graphs(Context* c) {
  for (auto& g : c->step_graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  c->step_graphs.clear();
}

void free_all(Context* c) {
  drop_step_graphs(c);
  if (c->h_status) cudaFreeHost(c->h_status), c->h_status = nullptr;
  for (void* p : c->allocs) cudaFree(p);
  c->allocs.clear();
  c->alloc_bytes.clear();
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  for (cudaEvent_t e : c->chunk_in)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : c->chunk_done)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t& e : c->chunk_fence)
    if (e) cudaEventDestroy(e), e = nullptr;
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  if (c->copy_out_stream) cudaStreamDestroy(c->copy_out_stream);
  for (cudaStream_t& q : c->stage_stream)
    if (q) cudaStreamDestroy(q), q = nullptr;
  if (c->stream) cudaStreamDestroy(c->stream);
  c->chunk_in.clear();
  c->chunk_done.clear();
  c->ev0 = c->ev1 = nullptr;
  c->copy_stream = c->copy_out_stream = c->stream = nullptr;
}

// ---------------------------------------------------------------------------
// Plain-form arrays from the reference's arrays (any conforming hex mesh).
// ---------------------------------------------------------------------------
int pairs_from_ids(const long long* ids, long m, std::vector<int>& pairs, std::vector<int>& single) {
  std::vector<long> ord(m);
  for (long i = 0; i < m; ++i) ord[i] = i;
  std::sort(ord.begin(), ord.end(), [&](long a, long b) {
    return ids[a] != ids[b] ? ids[a] < ids[b] : a < b;
  });
  pairs.clear();
  single.clear();
  long i = 0;
  while (i < m) {
    long j = i + 1;
    while (j < m && ids[ord[j]] == ids[ord[i]]) ++j;
    if (ids[ord[i]] <= 0) return NEKGPU_ERR_MESH;  // gs ignores id 0, flagged ids unsupported
    if (j - i == 2) {
      pairs.push_back((int)ord[i]);
      pairs.push_back((int)ord[i + 1]);
    } else if (j - i == 1) {
      single.push_back((int)ord[i]);
    } else {
      return NEKGPU_ERR_MESH;
    }
    i = j;
  }
  return NEKGPU_OK;
}

int pml_from_mesh(const nekgpu_mesh* m, PmlHost& p);

int build_plain(const nekgpu_mesh* m, PlainHost& p) {
  const int n = m->nx1;
  const long n3 = (long)n * n * n, npts = n3 * m->nelt, nxzfl = 6L * n * n * m->nelt;
  auto cp = [](const double* src, long len, std::vector<double>& dst) {
    dst.assign(src, src + len);
  };
  cp(m->dxm1, (long)n * n, p.dxm1);
  p.dxtm1.resize((size_t)n * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) p.dxtm1[j + (size_t)n * i] = m->dxm1[i + (size_t)n * j];
  cp(m->w3mn, n3, p.w3);
  p.metrics.resize(9 * (size_t)npts);
  const double* mt[9] = {m->rxmn, m->rymn, m->rzmn, m->sxmn, m->symn, m->szmn, m->txmn, m->tymn, m->tzmn};
  for (int q = 0; q < 9; ++q) std::copy(mt[q], mt[q] + npts, p.metrics.begin() + q * npts);
  cp(m->unxm, nxzfl, p.unx); cp(m->unym, nxzfl, p.uny); cp(m->unzm, nxzfl, p.unz);
  cp(m->aream, nxzfl, p.area);
  cp(m->Z_0, nxzfl, p.Z0); cp(m->Z_1, nxzfl, p.Z1); cp(m->Y_0, nxzfl, p.Y0); cp(m->Y_1, nxzfl, p.Y1);
  cp(m->ebm1, npts, p.ebm1); cp(m->hbm1, npts, p.hbm1); cp(m->bmn, npts, p.bm1);
  p.cemface.resize(nxzfl);
  for (long j = 0; j < nxzfl; ++j) {
    int v = m->cemface[j] - 1;
    if (v < 0 || v >= npts) return NEKGPU_ERR_ARG;
    p.cemface[j] = v;
  }
  std::vector<int> single;
  int st = pairs_from_ids(m->glo_face, nxzfl, p.pairs, single);
  if (st) return st;
  p.cempec.resize(m->ncempec);
  for (int j = 0; j < m->ncempec; ++j) {
    int s = m->cempec[j] - 1;
    if (s < 0 || s >= nxzfl) return NEKGPU_ERR_ARG;
    p.cempec[j] = s;
  }
  // CSR: volume node -> face slots, ascending slot order
  p.lift_ptr.assign(npts + 1, 0);
  for (long j = 0; j < nxzfl; ++j) p.lift_ptr[p.cemface[j] + 1]++;
  for (long v = 0; v < npts; ++v) p.lift_ptr[v + 1] += p.lift_ptr[v];
  p.lift_slot.assign(nxzfl, 0);
  std::vector<int> fill(p.lift_ptr.begin(), p.lift_ptr.end() - 1);
  for (long j = 0; j < nxzfl; ++j) p.lift_slot[fill[p.cemface[j]]++] = (int)j;
  p.C0 = m->C0;
  return pml_from_mesh(m, p.pml);
}

// ---------------------------------------------------------------------------
// Compact (fused-form) description from the reference's arrays: requires
// affine elements whose r,s,t axes are +x,+y,+z, canonical cemface, and
// face pairs that join opposite slots with the same in-face order.
// ---------------------------------------------------------------------------
int build_compact(const nekgpu_mesh* m, Compact& cp) {
  const int n = m->nx1, nelt = m->nelt;
  const long n2 = (long)n * n, n3 = n2 * n, npts = n3 * nelt, nxzfl = 6 * n2 * nelt;
  const double tol = 1e-9;
  cp.nx = n;
  cp.nelt = nelt;
  cp.D.assign(m->dxm1, m->dxm1 + n * n);
  cp.w3.assign(m->w3mn, m->w3mn + n3);
  cp.w.resize(n);
  const double w0 = std::cbrt(m->w3mn[0]);
  for (int i = 0; i < n; ++i) cp.w[i] = m->w3mn[i] / (w0 * w0);
  for (long v = 0; v < n3; ++v) {  // w3 must be a tensor product
    int i = v % n, j = (v / n) % n, k = v / n2;
    double t = cp.w[i] * cp.w[j] * cp.w[k];
    if (std::fabs(t - m->w3mn[v]) > 1e-12 * std::fabs(t)) return NEKGPU_ERR_MESH;
  }
  cp.egeom.assign(9 * (size_t)nelt, 0.0);
  const double* mt[9] = {m->rxmn, m->rymn, m->rzmn, m->sxmn, m->symn, m->szmn, m->txmn, m->tymn, m->tzmn};
  for (int e = 0; e < nelt; ++e) {
    const long o = n3 * e;
    double diag[3] = {0, 0, 0};
    const int di[3] = {0, 4, 8};
    for (int d = 0; d < 3; ++d) {
      double s = 0;
      for (long v = 0; v < n3; ++v) s += mt[di[d]][o + v];
      diag[d] = s / n3;
      if (!(diag[d] > 0)) return NEKGPU_ERR_MESH;
    }
    const double scale = std::max(diag[0], std::max(diag[1], diag[2]));
    for (int q = 0; q < 9; ++q) {
      const bool isdiag = (q == 0 || q == 4 || q == 8);
      const double ref = isdiag ? diag[q / 4] : 0.0;
      for (long v = 0; v < n3; ++v)
        if (std::fabs(mt[q][o + v] - ref) > tol * scale) return NEKGPU_ERR_MESH;
    }
    cp.egeom[9 * e + 0] = diag[0];
    cp.egeom[9 * e + 1] = diag[1];
    cp.egeom[9 * e + 2] = diag[2];
    for (int f = 0; f < 6; ++f) {
      const int ax = kSlotAxis[f], sd = kSlotSide[f];
      double s = 0;
      for (int b = 0; b < n; ++b)
        for (int a = 0; a < n; ++a) {
          const long j = a + (long)n * b + n2 * (f + 6L * e);
          if (m->cemface[j] - 1 != o + face_vol(f, a, b, n)) return NEKGPU_ERR_MESH;
          const double nv[3] = {m->unxm[j], m->unym[j], m->unzm[j]};
          for (int d = 0; d < 3; ++d) {
            const double want = (d == ax) ? (double)sd : 0.0;
            if (std::fabs(nv[d] - want) > tol) return NEKGPU_ERR_MESH;
          }
          s += m->aream[j] / (cp.w[a] * cp.w[b]);
        }
      s /= n2;
      for (int b = 0; b < n; ++b)
        for (int a = 0; a < n; ++a) {
          const long j = a + (long)n * b + n2 * (f + 6L * e);
          if (std::fabs(m->aream[j] / (cp.w[a] * cp.w[b]) - s) > tol * s) return NEKGPU_ERR_MESH;
        }
      cp.egeom[9 * e + 3 + f] = s;
    }
  }
  // pairing
  std::vector<int> pairs, single;
  int st = pairs_from_ids(m->glo_face, nxzfl, pairs, single);
  if (st) return st;
  std::vector<char> is_pec(nxzfl, 0);
  for (int j = 0; j < m->ncempec; ++j) {
    int s = m->cempec[j] - 1;
    if (s < 0 || s >= nxzfl) return NEKGPU_ERR_ARG;
    is_pec[s] = 1;
  }
  cp.nbr.assign(6 * (size_t)nelt, -3);  // -3: unset
  auto set_nbr = [&](int e, int f, int val) {
    int& r = cp.nbr[6 * e + f];
    if (r == -3) r = val;
    return r == val;
  };
  for (size_t p = 0; p < pairs.size(); p += 2) {
    const long j0 = pairs[p], j1 = pairs[p + 1];
    const int e0 = (int)(j0 / (6 * n2)), f0 = (int)((j0 / n2) % 6), ab0 = (int)(j0 % n2);
    const int e1 = (int)(j1 / (6 * n2)), f1 = (int)((j1 / n2) % 6), ab1 = (int)(j1 % n2);
    if (f1 != kSlotOpp[f0] || ab0 != ab1) return NEKGPU_ERR_MESH;
    if (is_pec[j0] || is_pec[j1]) return NEKGPU_ERR_MESH;
    if (!set_nbr(e0, f0, e1) || !set_nbr(e1, f1, e0)) return NEKGPU_ERR_MESH;
  }
  for (int s : single) {
    if (!is_pec[s]) return NEKGPU_ERR_MESH;  // open (non-PEC singleton) faces: plain form only
    const int e = (int)(s / (6 * n2)), f = (int)((s / n2) % 6);
    if (!set_nbr(e, f, -1)) return NEKGPU_ERR_MESH;
  }
  for (int v : cp.nbr)
    if (v == -3) return NEKGPU_ERR_MESH;
  cp.ebm1.assign(m->ebm1, m->ebm1 + npts);
  cp.hbm1.assign(m->hbm1, m->hbm1 + npts);
  cp.bm1.assign(m->bmn, m->bmn + npts);
  cp.C0 = m->C0;
  cp.fcoef.resize(4 * (size_t)nxzfl);
  cp.uniform = true;
  const double def[4] = {-0.5, 0.5 * m->C0, 0.5, 0.5 * m->C0};
  for (long j = 0; j < nxzfl; ++j) {
    const double Y0 = m->Y_0[j], Y1 = m->Y_1[j], Z0 = m->Z_0[j], Z1 = m->Z_1[j];
    double* o = &cp.fcoef[4 * j];
    o[0] = -0.5 / Y0 * Y1;
    o[1] = 0.5 / Y0 * m->C0;
    o[2] = 0.5 / Z0 * Z1;
    o[3] = 0.5 / Z0 * m->C0;
    for (int q = 0; q < 4; ++q)
      if (o[q] != def[q]) cp.uniform = false;
  }
  return pml_from_mesh(m, cp.pml);
}

// ---------------------------------------------------------------------------
// Box builder: the reference arrays of a structured affine box, produced on
// the host (genbox + genxyz + geometry + materials of the reference setup).
// ---------------------------------------------------------------------------
struct BoxArrays {
  std::vector<double> D, w3, metrics[9], bm1, x, y, z, unx, uny, unz, area, Z0, Z1, Y0, Y1, ebm1, hbm1;
  std::vector<int> cemface, cempec;
  std::vector<long long> glo;
  PmlHost pml;
  std::vector<int> pmlptr1;  // 1-based, for the mesh hand-off
  nekgpu_mesh mesh{};
};

// partner element across slot f of element ec, or -1 on a PEC wall
long box_partner(const nekgpu_box* bx, const int nel[3], const long ec[3], int f) {
  const int ax = kSlotAxis[f], sd = kSlotSide[f];
  const long plane = ec[ax] + (sd > 0 ? 1 : 0);
  if ((plane == 0 || plane == nel[ax]) && bx->bc[ax] != NEKGPU_BC_PERIODIC) return -1;
  long pc[3] = {ec[0], ec[1], ec[2]};
  pc[ax] = (pc[ax] + sd + nel[ax]) % nel[ax];
  return pc[0] + (long)nel[0] * (pc[1] + (long)nel[1] * pc[2]);
}

// impede / conduc of cem_maxwell_materials (src/cem_maxwell.F:272-275)
double node_Z(const nekgpu_box* bx, long g) {
  const double eps = bx->permittivity ? bx->permittivity[g] : 1.0;
  const double mu = bx->permeability ? bx->permeability[g] : 1.0;
  return std::sqrt(mu / eps);
}
double node_Y(const nekgpu_box* bx, long g) {
  const double eps = bx->permittivity ? bx->permittivity[g] : 1.0;
  const double mu = bx->permeability ? bx->permeability[g] : 1.0;
  return std::sqrt(eps / mu);
}

// PML of a box (src/cem_maxwell_pml.F): for an axis-aligned box the marching
// of pml_fill_faceary/march_faces (:85-190) tags exactly the elements within
// pml_thick layers of a 'PML' face, on that face's side of that axis; the
// extents inner/outer come from the tagged elements' node coordinates as in
// pml_extent_and_tags (:261-431), and sigma as in pml_calc_sigma (:433-506).
int pml_from_box(const nekgpu_box* bx, const BoxArrays& A, PmlHost& p) {
  p = PmlHost();
  bool any = false;
  for (int d = 0; d < 3; ++d) any = any || bx->bc[d] == NEKGPU_BC_PML;
  if (!any) return NEKGPU_OK;
  const int thick = bx->pml_thick;
  const double order = bx->pml_order, referr = bx->pml_referr;
  // pml_errchk (:2-30); referr = 0 would make sigma infinite
  if (thick < 1 || thick > 10 || !(order >= 1 && order <= 10) || !(referr > 0 && referr <= 1))
    return NEKGPU_ERR_ARG;
  const int n = bx->N + 1;
  const int nel[3] = {bx->nelx, bx->nely, bx->nelz};
  for (int d = 0; d < 3; ++d)
    if (bx->bc[d] == NEKGPU_BC_PML && 2 * thick > nel[d]) return NEKGPU_ERR_ARG;  // colliding layers
  const long nelt = (long)nel[0] * nel[1] * nel[2], n3 = (long)n * n * n, npts = n3 * nelt;
  const double* coord[3] = {A.x.data(), A.y.data(), A.z.data()};
  std::vector<int> tag(nelt, 0);
  double inner[6], outer[6];
  for (int d = 0; d < 3; ++d) {
    outer[2 * d] = 1e20; inner[2 * d] = -1e20;
    inner[2 * d + 1] = 1e20; outer[2 * d + 1] = -1e20;
  }
  for (long e = 0; e < nelt; ++e) {
    const long ec[3] = {e % nel[0], (e / nel[0]) % nel[1], e / ((long)nel[0] * nel[1])};
    for (int d = 0; d < 3; ++d) {
      if (bx->bc[d] != NEKGPU_BC_PML) continue;
      const bool lo_side = ec[d] < thick, hi_side = ec[d] >= nel[d] - thick;
      if (!lo_side && !hi_side) continue;
      double mn = coord[d][e * n3], mx = mn;
      for (long v = 1; v < n3; ++v) {
        mn = std::min(mn, coord[d][e * n3 + v]);
        mx = std::max(mx, coord[d][e * n3 + v]);
      }
      if (lo_side) {
        inner[2 * d] = std::max(inner[2 * d], mx);
        outer[2 * d] = std::min(outer[2 * d], mn);
        tag[e] |= 1 << (2 * d);
      }
      if (hi_side) {
        inner[2 * d + 1] = std::min(inner[2 * d + 1], mn);
        outer[2 * d + 1] = std::max(outer[2 * d + 1], mx);
        tag[e] |= 1 << (2 * d + 1);
      }
    }
  }
  p.eps.resize(npts);
  p.mu.resize(npts);
  for (long g = 0; g < npts; ++g) {
    p.eps[g] = bx->permittivity ? bx->permittivity[g] : 1.0;
    p.mu[g] = bx->permeability ? bx->permeability[g] : 1.0;
  }
  p.sigma.assign(3 * (size_t)npts, 0.0);
  for (long e = 0; e < nelt; ++e) {
    if (!tag[e]) continue;
    p.elems.push_back((int)e);
    for (int face = 0; face < 6; ++face) {
      if (!(tag[e] & (1 << face))) continue;
      const int ax = face / 2;
      const double width = std::fabs(outer[face] - inner[face]);
      for (long v = 0; v < n3; ++v) {
        const long j = e * n3 + v;
        const double eta = std::sqrt(p.mu[j] / p.eps[j]);
        const double sigmamax = -(order + 1) * std::log(referr) / (2 * eta * width);
        const double z2o = (coord[ax][j] - inner[face]) / (outer[face] - inner[face]);
        p.sigma[j + ax * npts] = sigmamax * std::pow(z2o, order);
      }
    }
  }
  return NEKGPU_OK;
}

// PML arrays handed over by the caller (nekgpu_mesh)
int pml_from_mesh(const nekgpu_mesh* m, PmlHost& p) {
  p = PmlHost();
  if (!m->pmlsigma || m->npml <= 0) return NEKGPU_OK;
  if (!m->pmlptr || !m->permittivity || !m->permeability) return NEKGPU_ERR_ARG;
  const long npts = (long)m->nx1 * m->nx1 * m->nx1 * m->nelt;
  p.sigma.assign(m->pmlsigma, m->pmlsigma + 3 * npts);
  p.eps.assign(m->permittivity, m->permittivity + npts);
  p.mu.assign(m->permeability, m->permeability + npts);
  for (int l = 0; l < m->npml; ++l) {
    const int e = m->pmlptr[l] - 1;
    if (e < 0 || e >= m->nelt || (l > 0 && e <= p.elems.back())) return NEKGPU_ERR_ARG;
    p.elems.push_back(e);
  }
  return NEKGPU_OK;
}

int build_box(const nekgpu_box* bx, BoxArrays& A, bool full) {
  const int N = bx->N, n = N + 1;
  if (N < 1 || N > 15 || bx->nelx < 1 || bx->nely < 1 || bx->nelz < 1) return NEKGPU_ERR_ARG;
  const int nel[3] = {bx->nelx, bx->nely, bx->nelz};
  const long nelt = (long)nel[0] * nel[1] * nel[2];
  const long n2 = (long)n * n, n3 = n2 * n, npts = n3 * nelt, nxzfl = 6 * n2 * nelt;
  if (npts > (1L << 31) - 1 || nxzfl > (1L << 31) - 1) return NEKGPU_ERR_ARG;
  for (int d = 0; d < 3; ++d)
    if (!(bx->hi[d] > bx->lo[d]) || (bx->bc[d] != NEKGPU_BC_PEC && bx->bc[d] != NEKGPU_BC_PERIODIC &&
                                     bx->bc[d] != NEKGPU_BC_PML))
      return NEKGPU_ERR_ARG;
  std::vector<double> z, w;
  gll(N, z, w, A.D);
  A.w3.resize(n3);
  for (long v = 0; v < n3; ++v) A.w3[v] = w[v % n] * w[(v / n) % n] * w[v / n2];
  double h[3];
  for (int d = 0; d < 3; ++d) h[d] = (bx->hi[d] - bx->lo[d]) / nel[d];
  const double xr = 0.5 * h[0], ys = 0.5 * h[1], zt = 0.5 * h[2];
  const double jac = xr * ys * zt;
  const double rx = ys * zt, sy = xr * zt, tz = xr * ys;
  A.bm1.resize(npts);
  A.x.resize(npts); A.y.resize(npts); A.z.resize(npts);
  for (long e = 0; e < nelt; ++e) {
    const long ex = e % nel[0], ey = (e / nel[0]) % nel[1], ez = e / ((long)nel[0] * nel[1]);
    for (long v = 0; v < n3; ++v) {
      const int i = v % n, j = (v / n) % n, k = v / n2;
      const long g = e * n3 + v;
      A.bm1[g] = jac * A.w3[v];
      A.x[g] = bx->lo[0] + h[0] * ex + 0.5 * (z[i] + 1.0) * h[0];
      A.y[g] = bx->lo[1] + h[1] * ey + 0.5 * (z[j] + 1.0) * h[1];
      A.z[g] = bx->lo[2] + h[2] * ez + 0.5 * (z[k] + 1.0) * h[2];
    }
  }
  // materials per node
  A.ebm1.resize(npts);
  A.hbm1.resize(npts);
  for (long g = 0; g < npts; ++g) {
    const double eps = bx->permittivity ? bx->permittivity[g] : 1.0;
    const double mu = bx->permeability ? bx->permeability[g] : 1.0;
    if (!(eps > 0) || !(mu > 0)) return NEKGPU_ERR_ARG;
    A.ebm1[g] = 1.0 / (eps * A.bm1[g]);
    A.hbm1[g] = 1.0 / (mu * A.bm1[g]);
  }
  if (full) {
    for (int q = 0; q < 9; ++q) A.metrics[q].assign(npts, 0.0);
    std::fill(A.metrics[0].begin(), A.metrics[0].end(), rx);
    std::fill(A.metrics[4].begin(), A.metrics[4].end(), sy);
    std::fill(A.metrics[8].begin(), A.metrics[8].end(), tz);
  }
  // faces: normals, areas, cemface, gs ids, PEC list, impedances (the
  // reference-layout arrays; the fused path builds its compact form instead)
  if (full) {
    A.unx.assign(nxzfl, 0.0); A.uny.assign(nxzfl, 0.0); A.unz.assign(nxzfl, 0.0);
    A.area.resize(nxzfl);
    A.cemface.resize(nxzfl);
    A.glo.resize(nxzfl);
    A.Z0.resize(nxzfl); A.Z1.resize(nxzfl); A.Y0.resize(nxzfl); A.Y1.resize(nxzfl);
    A.cempec.clear();
    const double ascale[3] = {ys * zt, xr * zt, xr * ys};  // r-, s-, t-faces
    const long long off[3] = {0, (long long)(nel[0] + 1) * nel[1] * nel[2],
                              (long long)(nel[0] + 1) * nel[1] * nel[2] + (long long)(nel[1] + 1) * nel[0] * nel[2]};
    for (long e = 0; e < nelt; ++e) {
      const long ec[3] = {e % nel[0], (e / nel[0]) % nel[1], e / ((long)nel[0] * nel[1])};
      for (int f = 0; f < 6; ++f) {
        const int ax = kSlotAxis[f], sd = kSlotSide[f];
        long plane = ec[ax] + (sd > 0 ? 1 : 0);
        const bool boundary = (plane == 0 || plane == nel[ax]);
        const int wall = !boundary ? 0 : (bx->bc[ax] == NEKGPU_BC_PEC ? 1 : (bx->bc[ax] == NEKGPU_BC_PML ? 2 : 0));
        const bool pec = wall != 0;  // PEC and PML faces: mirror flux (cem_maxwell_pec_init)
        if (boundary && !pec) plane = plane % nel[ax];
        long long fid;
        if (ax == 0) fid = off[0] + (plane * nel[1] + ec[1]) * nel[2] + ec[2];
        else if (ax == 1) fid = off[1] + (plane * nel[0] + ec[0]) * nel[2] + ec[2];
        else fid = off[2] + (plane * nel[0] + ec[0]) * nel[1] + ec[1];
        const long pe = box_partner(bx, nel, ec, f);
        for (int b = 0; b < n; ++b)
          for (int a = 0; a < n; ++a) {
            const long j = a + (long)n * b + n2 * (f + 6 * e);
            const long g = e * n3 + face_vol(f, a, b, n);
            A.cemface[j] = (int)(g + 1);
            A.glo[j] = fid * (long long)n2 + a + (long long)n * b + 1;
            if (ax == 0) A.unx[j] = sd; else if (ax == 1) A.uny[j] = sd; else A.unz[j] = sd;
            A.area[j] = ascale[ax] * w[a] * w[b];
            if (pec) A.cempec.push_back((int)(j + 1));
            const long gp = pec ? g : pe * n3 + face_vol(kSlotOpp[f], a, b, n);
            const double Zm = node_Z(bx, g), Ym = node_Y(bx, g);
            const double Zp = node_Z(bx, gp), Yp = node_Y(bx, gp);
            const double Z0 = wall == 1 ? 2.0 * Zm : (wall == 2 ? Zm : Zm + Zp);
            const double Y0 = wall == 1 ? 2.0 * Ym : (wall == 2 ? Ym : Ym + Yp);
            A.Z1[j] = Z0 - Zm;
            A.Y1[j] = Y0 - Ym;
            A.Z0[j] = 0.5 * Z0;
            A.Y0[j] = 0.5 * Y0;
          }
      }
    }
  }
  nekgpu_mesh& m = A.mesh;
  m.nx1 = n;
  m.nelt = (int)nelt;
  m.dxm1 = A.D.data();
  m.w3mn = A.w3.data();
  std::vector<double>* mt = A.metrics;
  if (!full) {  // compact path: per-node metric arrays are not needed
    for (int q = 0; q < 9; ++q) mt[q].clear();
  }
  m.rxmn = full ? mt[0].data() : nullptr; m.rymn = full ? mt[1].data() : nullptr;
  m.rzmn = full ? mt[2].data() : nullptr; m.sxmn = full ? mt[3].data() : nullptr;
  m.symn = full ? mt[4].data() : nullptr; m.szmn = full ? mt[5].data() : nullptr;
  m.txmn = full ? mt[6].data() : nullptr; m.tymn = full ? mt[7].data() : nullptr;
  m.tzmn = full ? mt[8].data() : nullptr;
  m.bmn = A.bm1.data();
  m.xmn = A.x.data(); m.ymn = A.y.data(); m.zmn = A.z.data();
  m.unxm = A.unx.data(); m.unym = A.uny.data(); m.unzm = A.unz.data(); m.aream = A.area.data();
  m.cemface = A.cemface.data();
  m.glo_face = A.glo.data();
  m.cempec = A.cempec.data();
  m.ncempec = (int)A.cempec.size();
  m.Z_0 = A.Z0.data(); m.Z_1 = A.Z1.data(); m.Y_0 = A.Y0.data(); m.Y_1 = A.Y1.data();
  m.ebm1 = A.ebm1.data(); m.hbm1 = A.hbm1.data();
  m.C0 = bx->C0;
  int st = pml_from_box(bx, A, A.pml);
  if (st) return st;
  if (A.pml.on()) {
    A.pmlptr1.resize(A.pml.elems.size());
    for (size_t l = 0; l < A.pml.elems.size(); ++l) A.pmlptr1[l] = A.pml.elems[l] + 1;
    m.pmlsigma = A.pml.sigma.data();
    m.pmlptr = A.pmlptr1.data();
    m.npml = (int)A.pmlptr1.size();
    m.permittivity = A.pml.eps.data();
    m.permeability = A.pml.mu.data();
  }
  return NEKGPU_OK;
}

// Compact description straight from the box (no per-node or per-face-node
// reference arrays).
void compact_from_box(const nekgpu_box* bx, const BoxArrays& A, Compact& cp) {
  const int n = bx->N + 1;
  const int nel[3] = {bx->nelx, bx->nely, bx->nelz};
  const long nelt = (long)nel[0] * nel[1] * nel[2];
  const long n2 = (long)n * n, n3 = n2 * n, nxzfl = 6 * n2 * nelt;
  cp.nx = n;
  cp.nelt = (int)nelt;
  cp.D = A.D;
  cp.w3 = A.w3;
  std::vector<double> z, w, D;
  gll(bx->N, z, w, D);
  cp.w = w;
  double h[3];
  for (int d = 0; d < 3; ++d) h[d] = (bx->hi[d] - bx->lo[d]) / nel[d];
  const double xr = 0.5 * h[0], ys = 0.5 * h[1], zt = 0.5 * h[2];
  const double ascale[3] = {ys * zt, xr * zt, xr * ys};
  cp.egeom.resize(9 * (size_t)nelt);
  cp.nbr.resize(6 * (size_t)nelt);
  for (long e = 0; e < nelt; ++e) {
    const long ec[3] = {e % nel[0], (e / nel[0]) % nel[1], e / ((long)nel[0] * nel[1])};
    cp.egeom[9 * e + 0] = ys * zt;
    cp.egeom[9 * e + 1] = xr * zt;
    cp.egeom[9 * e + 2] = xr * ys;
    for (int f = 0; f < 6; ++f) {
      cp.egeom[9 * e + 3 + f] = ascale[kSlotAxis[f]];
      cp.nbr[6 * e + f] = (int)box_partner(bx, nel, ec, f);
    }
  }
  cp.ebm1 = A.ebm1;
  cp.hbm1 = A.hbm1;
  cp.bm1 = A.bm1;
  cp.C0 = bx->C0;
  cp.uniform = true;
  const long npts = n3 * nelt;
  for (int d = 0; d < 3; ++d) cp.uniform = cp.uniform && bx->bc[d] != NEKGPU_BC_PML;
  cp.pml = A.pml;
  if (bx->permittivity)
    for (long g = 0; g < npts && cp.uniform; ++g) cp.uniform = bx->permittivity[g] == 1.0;
  if (bx->permeability)
    for (long g = 0; g < npts && cp.uniform; ++g) cp.uniform = bx->permeability[g] == 1.0;
  cp.fcoef.clear();
  if (!cp.uniform) {
    cp.fcoef.resize(4 * (size_t)nxzfl);
    for (long e = 0; e < nelt; ++e) {
      for (int f = 0; f < 6; ++f) {
        const int pe = cp.nbr[6 * e + f];
        for (int b = 0; b < n; ++b)
          for (int a = 0; a < n; ++a) {
            const long j = a + (long)n * b + n2 * (f + 6 * e);
            const long g = e * n3 + face_vol(f, a, b, n);
            const long gp = pe < 0 ? g : (long)pe * n3 + face_vol(kSlotOpp[f], a, b, n);
            const int wall = pe >= 0 ? 0 : (bx->bc[kSlotAxis[f]] == NEKGPU_BC_PML ? 2 : 1);
            face_impedance(node_Z(bx, g), node_Y(bx, g), node_Z(bx, gp), node_Y(bx, gp), wall,
                           bx->C0, &cp.fcoef[4 * j]);
          }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// device upload
// ---------------------------------------------------------------------------
int common_setup(Context* c, int form, int nx, int nelt) {
  int st = nekgpu_device_check(0);
  if (st) return st;
  c->form = form;
  c->nx = nx;
  c->nelt = nelt;
  c->npts = (long)nx * nx * nx * nelt;
  c->nxzfl = 6L * nx * nx * nelt;
  rk_coeffs(c->rk_a, c->rk_b, c->rk_c);
  if (check_cuda(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking))) return NEKGPU_ERR_CUDA;
  if (check_cuda(cudaEventCreate(&c->ev0)) || check_cuda(cudaEventCreate(&c->ev1))) return NEKGPU_ERR_CUDA;
  return NEKGPU_OK;
}

int upload_common(Context* c, DevAlloc& A, const std::vector<double>& bm1,
                  const std::vector<double>& ebm1, const std::vector<double>& hbm1) {
  int st;
  if ((st = A.get(&c->d_k, 6 * c->npts))) return st;
  if ((st = A.put(&c->d_bm1, bm1))) return st;
  if ((st = A.put(&c->d_ebm1, ebm1))) return st;
  if ((st = A.put(&c->d_hbm1, hbm1))) return st;
  if ((st = A.get(&c->d_red, 512 * 12))) return st;
  if ((st = A.get(&c->d_status, 4))) return st;
  if (check_cuda(cudaHostAlloc(&c->h_status, sizeof(int), cudaHostAllocDefault)))
    return NEKGPU_ERR_CUDA;
  if (check_cuda(cudaMemset(c->d_k, 0, 6 * c->npts * sizeof(double)))) return NEKGPU_ERR_CUDA;
  if (check_cuda(cudaMemset(c->d_status, 0, 4 * sizeof(int)))) return NEKGPU_ERR_CUDA;
  double vol = 0;
  for (double b : bm1) vol += b;
  c->volume = vol;
  c->host_bm1 = bm1;
  return NEKGPU_OK;
}

int upload_plain(Context* c, const PlainHost& p) {
  DevAlloc A(c);
  int st;
  c->host_cemface = p.cemface;
  if ((st = A.get(&c->d_u[0], 6 * c->npts))) return st;
  if ((st = upload_common(c, A, p.bm1, p.ebm1, p.hbm1))) return st;
  PlainDev& a = c->pargs;
  a = PlainDev{};
  a.nx = c->nx; a.nelt = c->nelt; a.npts = c->npts; a.nxzfl = c->nxzfl;
  double *d1, *d2, *d3, *d4;
  if ((st = A.put(&d1, p.dxm1)) || (st = A.put(&d2, p.dxtm1)) || (st = A.put(&d3, p.w3)) ||
      (st = A.put(&d4, p.metrics)))
    return st;
  a.dxm1 = d1; a.dxtm1 = d2; a.w3 = d3; a.metrics = d4;
  const std::vector<double>* fa[8] = {&p.unx, &p.uny, &p.unz, &p.area, &p.Z0, &p.Z1, &p.Y0, &p.Y1};
  const double** fd[8] = {&a.unx, &a.uny, &a.unz, &a.area, &a.Z0, &a.Z1, &a.Y0, &a.Y1};
  for (int q = 0; q < 8; ++q) {
    double* d;
    if ((st = A.put(&d, *fa[q]))) return st;
    *fd[q] = d;
  }
  a.ebm1 = c->d_ebm1;
  a.hbm1 = c->d_hbm1;
  int *i1, *i2, *i3, *i4, *i5;
  if ((st = A.put(&i1, p.cemface)) || (st = A.put(&i2, p.pairs)) || (st = A.put(&i3, p.cempec)) ||
      (st = A.put(&i4, p.lift_ptr)) || (st = A.put(&i5, p.lift_slot)))
    return st;
  a.cemface = i1; a.pairs = i2; a.npairs = (int)(p.pairs.size() / 2);
  a.cempec = i3; a.ncempec = (int)p.cempec.size();
  a.lift_ptr = i4; a.lift_slot = i5;
  a.C0 = p.C0;
  a.u = c->d_u[0];
  a.k = c->d_k;
  double *r, *ff, *sf;
  if ((st = A.get(&r, 6 * c->npts)) || (st = A.get(&ff, 6 * c->nxzfl)) || (st = A.get(&sf, 6 * c->nxzfl)))
    return st;
  a.res = r; a.fface = ff; a.srflx = sf;
  cudaMemset(r, 0, 6 * c->npts * sizeof(double));
  cudaMemset(ff, 0, 6 * c->nxzfl * sizeof(double));
  cudaMemset(sf, 0, 6 * c->nxzfl * sizeof(double));
  a.src_w = nullptr;
  a.bm1 = c->d_bm1;
  if (p.pml.on()) {  // the reference's full-size PML arrays (src/PML)
    c->npml = (int)p.pml.elems.size();
    c->pml_elems = p.pml.elems;
    if ((st = A.put(&c->d_pml_sigma, p.pml.sigma)) || (st = A.put(&c->d_eps, p.pml.eps)) ||
        (st = A.put(&c->d_mu, p.pml.mu)) || (st = A.put(&c->d_pmlptr, p.pml.elems)) ||
        (st = A.get(&c->d_pml_aux, 6 * c->npts)) || (st = A.get(&c->d_pml_k, 6 * c->npts)) ||
        (st = A.get(&c->d_pml_res, 12 * c->npts)))
      return st;
    if (check_cuda(cudaMemset(c->d_pml_aux, 0, 6 * c->npts * sizeof(double))) ||
        check_cuda(cudaMemset(c->d_pml_k, 0, 6 * c->npts * sizeof(double))) ||
        check_cuda(cudaMemset(c->d_pml_res, 0, 12 * c->npts * sizeof(double))))
      return NEKGPU_ERR_CUDA;
    a.pmlsigma = c->d_pml_sigma;
    a.eps = c->d_eps;
    a.mu = c->d_mu;
    a.pmlptr = c->d_pmlptr;
    a.npml = c->npml;
    a.pmlaux = c->d_pml_aux;
    a.pmlk = c->d_pml_k;
    a.pmlres = c->d_pml_res;
  }
  return NEKGPU_OK;
}

// PML data of the fused forms (layout: PmlDev), compact over the PML elements
int upload_pml_fused(Context* c, DevAlloc& A, const Compact& cp, PmlDev& out) {
  out = PmlDev{};
  if (!cp.pml.on()) return NEKGPU_OK;
  const PmlHost& p = cp.pml;
  const long n3 = (long)c->nx * c->nx * c->nx, npts = c->npts;
  const long npml = (long)p.elems.size(), nn = npml * n3;
  std::vector<int> slot(c->nelt, -1);
  std::vector<double> d((size_t)kPmlData * nn);
  for (long l = 0; l < npml; ++l) {
    const long e = p.elems[l];
    slot[e] = (int)l;
    for (long v = 0; v < n3; ++v) {
      const long j = e * n3 + v, q = l * n3 + v;
      for (int ax = 0; ax < 3; ++ax) {
        d[ax * nn + q] = p.sigma[j + ax * npts] / p.eps[j];
        d[(3 + ax) * nn + q] = p.sigma[j + ax * npts];
      }
      d[6 * nn + q] = p.mu[j];
      d[7 * nn + q] = cp.bm1[j];
      d[8 * nn + q] = 1.0 / cp.bm1[j];
      d[9 * nn + q] = cp.w3[v] * cp.egeom[9 * e] / cp.bm1[j];
      d[10 * nn + q] = cp.bm1[j] / (cp.w3[v] * cp.egeom[9 * e]);
    }
  }
  int st;
  if ((st = A.put(&c->d_pml_slot, slot)) || (st = A.put(&c->d_pml_data, d)) ||
      (st = A.get(&c->d_pml_aux, 6 * nn)) || (st = A.get(&c->d_pml_k, 6 * nn)))
    return st;
  if (check_cuda(cudaMemset(c->d_pml_aux, 0, 6 * nn * sizeof(double))) ||
      check_cuda(cudaMemset(c->d_pml_k, 0, 6 * nn * sizeof(double))))
    return NEKGPU_ERR_CUDA;
  c->npml = (int)npml;
  c->pml_elems = p.elems;
  out.slot = c->d_pml_slot;
  out.data = c->d_pml_data;
  out.aux = c->d_pml_aux;
  out.k = c->d_pml_k;
  out.n = nn;
  return NEKGPU_OK;
}

// D in the FP32 pieces of the mixed form's exact-hi contraction, as float
// pairs [0][i + n*l] = (Dh, Df) of D(i,l) and [1][j + H*l] =
// (Dm(2j,l), Dm(2j+1,l)), H = (n+1)/2: Dh on a 10-bit grid of row i (so every
// product Dh*uh with uh on a 10-bit grid has at most 21 bits and the sum over
// <= 16 terms stays exact in FP32), Df = RN32(D), Dm = RN32(D - Dh).
void split_D(const std::vector<double>& D, int n, std::vector<float>& tab) {
  const int M2 = kMaxMixed * kMaxMixed;
  tab.assign(4 * (size_t)M2, 0.0f);
  for (int i = 0; i < n; ++i) {
    double rmax = 0;
    for (int l = 0; l < n; ++l) rmax = std::max(rmax, std::fabs(D[i + (size_t)n * l]));
    int ex = 0;
    std::frexp(rmax, &ex);  // rmax < 2^ex
    const double qd = std::ldexp(1.0, ex - 10);
    for (int l = 0; l < n; ++l) {
      const size_t k = i + (size_t)n * l;
      const double h = std::nearbyint(D[k] / qd) * qd;  // at most 11 significant bits
      tab[2 * k] = (float)h;
      tab[2 * k + 1] = (float)D[k];
      const size_t kp = (size_t)(i / 2) + (size_t)((n + 1) / 2) * l;
      tab[2 * (M2 + kp) + (i & 1)] = (float)(D[k] - h);
    }
  }
}

int upload_fused(Context* c, const Compact& cp) {
  DevAlloc A(c);
  int st;
  const long n3 = (long)c->nx * c->nx * c->nx;
  if ((st = A.get(&c->d_u[0], 6 * c->npts)) || (st = A.get(&c->d_u[1], 6 * c->npts))) return st;
  if ((st = upload_common(c, A, cp.bm1, cp.ebm1, cp.hbm1))) return st;
  if ((st = A.get(&c->d_coef, 2 * c->npts))) return st;
  if ((st = A.put(&c->d_nbr, cp.nbr))) return st;
  c->host_nbr = cp.nbr;
  c->host_w3 = cp.w3;
  c->host_rx.resize(c->nelt);
  for (int e = 0; e < c->nelt; ++e) c->host_rx[e] = cp.egeom[9 * (size_t)e];
  // unscaled inverse-mass coefficients: hbm1|ebm1, or for the mixed form the
  // normalised hbm1*w3*rx | ebm1*w3*rx (the residual is res/(bm1*2/hx))
  {
    std::vector<double> base(2 * c->npts);
    for (long g = 0; g < c->npts; ++g) {
      double f = 1.0;
      if (c->form == NEKGPU_MIXED) f = cp.w3[g % n3] * cp.egeom[9 * (g / n3)];
      base[g] = cp.hbm1[g] * f;
      base[c->npts + g] = cp.ebm1[g] * f;
    }
    if ((st = A.put(&c->d_cbase, base))) return st;
  }
  c->uniform = cp.uniform;
  c->d_fcoef = nullptr;
  if (!cp.uniform) {
    if (c->form == NEKGPU_FUSED64) {
      double* d;
      if ((st = A.put(&d, cp.fcoef))) return st;
      c->d_fcoef = d;
    } else {
      std::vector<float> f(cp.fcoef.begin(), cp.fcoef.end());
      if (c->form == NEKGPU_MIXED) {
        // float pairs: per face node the hi parts (Y02, C02Y, Z02, C02Z), then
        // the lo parts
        const size_t nf = cp.fcoef.size() / 4;
        f.assign(8 * nf, 0.0f);
        for (size_t j = 0; j < nf; ++j)
          for (int q = 0; q < 4; ++q) {
            const double v = cp.fcoef[4 * j + q];
            f[8 * j + q] = (float)v;
            f[8 * j + 4 + q] = (float)(v - (double)f[8 * j + q]);
          }
      }
      float* d;
      if ((st = A.put(&d, f))) return st;
      c->d_fcoef = d;
    }
  }
  if ((st = fused_setup(c))) return st;
  c->coef_dt = std::nan("");
  if (c->form == NEKGPU_MIXED) {
    // per element (16 floats): rho_y = sy/rx and rho_z = tz/rx as float
    // pairs (1, 0 both on cubic elements), then the lift factor
    // area/(bm1*2/hx) = A_f/(w_end*rx) per slot, hi parts then lo parts
    const double wend = cp.w[0];
    std::vector<float> egm(16 * (size_t)c->nelt, 0.0f);
    for (int e = 0; e < c->nelt; ++e) {
      const double* g = &cp.egeom[9 * (size_t)e];
      const double ry = g[1] / g[0], rz = g[2] / g[0];
      float* o = &egm[16 * (size_t)e];
      o[0] = (float)ry; o[1] = (float)(ry - (double)o[0]);
      o[2] = (float)rz; o[3] = (float)(rz - (double)o[2]);
      for (int f = 0; f < 6; ++f) {
        const double lf = g[3 + f] / (wend * g[0]);
        o[4 + f] = (float)lf;
        o[10 + f] = (float)(lf - (double)o[4 + f]);
      }
    }
    if ((st = A.put(&c->d_egm, egm))) return st;
    MixedDev& m = c->margs;
    m = MixedDev{};
    m.nelt = c->nelt;
    m.npts = c->npts;
    m.k = c->d_k;
    m.k_out = c->d_k;
    m.coef = reinterpret_cast<const float2*>(c->d_coef);
    m.nbr = c->d_nbr;
    m.egm = c->d_egm;
    m.fcoef = c->d_fcoef;
    m.C0f = (float)cp.C0;
    m.status = c->d_status;
    if (c->nx > kMaxMixed) return NEKGPU_ERR_UNSUPPORTED;
    // the mixed form uses the library's own GLL D of this order (exactly
    // centro-antisymmetric, computed once per order); a caller's D must agree
    std::vector<double> z, w, D;
    gll(c->nx - 1, z, w, D);
    double dmax = 0, diff = 0;
    for (size_t k = 0; k < D.size(); ++k) {
      dmax = std::max(dmax, std::fabs(D[k]));
      diff = std::max(diff, std::fabs(D[k] - cp.D[k]));
    }
    if (diff > 1e-12 * dmax) return NEKGPU_ERR_MESH;
    std::vector<float> tab;
    split_D(D, c->nx, tab);
    if ((st = mixed_upload_D(c->nx, tab.data(), tab.size()))) return st;
    // what the FP64 reverse stages of the adjoint read: the element geometry,
    // D, the GLL weights, C0 and the FP64 face coefficients (host copy)
    if ((st = A.put(&c->d_egeom, cp.egeom))) return st;
    FusedDev& f = c->fargs;
    f = FusedDev{};
    f.nelt = c->nelt;
    f.npts = c->npts;
    f.C0 = cp.C0;
    for (int i = 0; i < c->nx * c->nx; ++i) f.D[i] = cp.D[i];
    for (int i = 0; i < c->nx; ++i) f.w[i] = cp.w[i];
    if (!cp.uniform) c->host_fcoef64 = cp.fcoef;
    return upload_pml_fused(c, A, cp, m.pml);
  }
  if ((st = A.put(&c->d_egeom, cp.egeom))) return st;
  std::vector<float> gf(cp.egeom.begin(), cp.egeom.end());
  if ((st = A.put(&c->d_egeomf, gf))) return st;
  FusedDev& a = c->fargs;
  a = FusedDev{};
  a.nelt = c->nelt;
  a.npts = c->npts;
  a.k = c->d_k;
  a.coef = c->d_coef;
  a.nbr = c->d_nbr;
  a.egeom = c->d_egeom;
  a.egeomf = c->d_egeomf;
  a.fcoef = c->d_fcoef;
  a.C0 = cp.C0;
  a.C0f = (float)cp.C0;
  a.status = c->d_status;
  for (int i = 0; i < c->nx * c->nx; ++i) {
    a.D[i] = cp.D[i];
    a.Df[i] = (float)cp.D[i];
  }
  for (int i = 0; i < c->nx; ++i) {
    a.w[i] = cp.w[i];
    a.wf[i] = (float)cp.w[i];
  }
  if (cp.pml.on() && c->form != NEKGPU_FUSED64) return NEKGPU_ERR_UNSUPPORTED;
  return upload_pml_fused(c, A, cp, a.pml);
}

// Curvilinear mesh for the fused FP64 and the mixed forms: the reference's
// per-node metrics and face arrays as given; face node partners from the gs
// ids.  The reference's face numbering is required (the lift finds a node's
// face slots from its position in the element).  The mixed form also takes
// the library's GLL D of this order in its FP32 pieces (a caller's D must
// agree with it).
int upload_curved(Context* c, const nekgpu_mesh* m) {
  const int n = m->nx1;
  const long n2 = (long)n * n, n3 = n2 * n, npts = n3 * m->nelt, nxzfl = 6 * n2 * m->nelt;
  if (n < 3 || n > 8) return NEKGPU_ERR_UNSUPPORTED;
  if (c->form == NEKGPU_MIXED) {
    std::vector<double> z, w, D;
    gll(n - 1, z, w, D);
    double dmax = 0, diff = 0;
    for (long k = 0; k < n2; ++k) {
      dmax = std::max(dmax, std::fabs(D[k]));
      diff = std::max(diff, std::fabs(D[k] - m->dxm1[k]));
    }
    if (diff > 1e-12 * dmax) return NEKGPU_ERR_MESH;
    std::vector<float> tab;
    split_D(D, n, tab);
    const int st = mixed_upload_D(n, tab.data(), tab.size());
    if (st) return st;
  }
  if (m->npml > 0) return NEKGPU_ERR_UNSUPPORTED;  // no PML on curvilinear meshes
  for (long e = 0; e < m->nelt; ++e)
    for (int f = 0; f < 6; ++f)
      for (int b = 0; b < n; ++b)
        for (int a = 0; a < n; ++a) {
          const long j = a + (long)n * b + n2 * (f + 6 * e);
          if (m->cemface[j] - 1 != e * n3 + face_vol(f, a, b, n)) return NEKGPU_ERR_MESH;
        }
  std::vector<int> pairs, single, partner(nxzfl, -2);
  int st = pairs_from_ids(m->glo_face, nxzfl, pairs, single);
  if (st) return st;
  for (size_t q = 0; q + 1 < pairs.size(); q += 2) {
    partner[pairs[q]] = m->cemface[pairs[q + 1]] - 1;
    partner[pairs[q + 1]] = m->cemface[pairs[q]] - 1;
  }
  for (int j = 0; j < m->ncempec; ++j) {
    const int sl = m->cempec[j] - 1;
    if (sl < 0 || sl >= nxzfl || partner[sl] != -2) return NEKGPU_ERR_MESH;
    partner[sl] = -1;
  }
  for (long j = 0; j < nxzfl; ++j)
    if (partner[j] == -2) return NEKGPU_ERR_MESH;  // a face node with no partner and no wall
  DevAlloc A(c);
  std::vector<double> bm1(m->bmn, m->bmn + npts), eb(m->ebm1, m->ebm1 + npts),
      hb(m->hbm1, m->hbm1 + npts);
  if ((st = A.get(&c->d_u[0], 6 * npts)) || (st = A.get(&c->d_u[1], 6 * npts))) return st;
  if ((st = upload_common(c, A, bm1, eb, hb))) return st;
  if ((st = A.get(&c->d_coef, 2 * npts))) return st;
  std::vector<double> base(2 * npts);
  for (long g = 0; g < npts; ++g) {
    base[g] = hb[g];
    base[npts + g] = eb[g];
  }
  if ((st = A.put(&c->d_cbase, base))) return st;
  c->coef_dt = std::nan("");
  const double* mt[9] = {m->rxmn, m->rymn, m->rzmn, m->sxmn, m->symn, m->szmn, m->txmn, m->tymn, m->tzmn};
  std::vector<double> metrics(9 * (size_t)npts), face(4 * (size_t)nxzfl), fcoef(4 * (size_t)nxzfl);
  for (int q = 0; q < 9; ++q) std::copy(mt[q], mt[q] + npts, metrics.begin() + q * npts);
  bool uniform = true;
  for (long j = 0; j < nxzfl; ++j) {
    face[j] = m->unxm[j];
    face[nxzfl + j] = m->unym[j];
    face[2 * nxzfl + j] = m->unzm[j];
    face[3 * nxzfl + j] = m->aream[j];
    const double Y0 = m->Y_0[j], Y1 = m->Y_1[j], Z0 = m->Z_0[j], Z1 = m->Z_1[j];
    const double o[4] = {-0.5 / Y0 * Y1, 0.5 / Y0 * m->C0, 0.5 / Z0 * Z1, 0.5 / Z0 * m->C0};
    for (int q = 0; q < 4; ++q) fcoef[q * nxzfl + j] = o[q];
    uniform = uniform && o[0] == -0.5 && o[1] == 0.5 && o[2] == 0.5 && o[3] == 0.5;
  }
  CurvedDev& a = c->cargs;
  a = CurvedDev{};
  double* d;
  int* di;
  if ((st = A.put(&d, metrics))) return st;
  a.metrics = d;
  if ((st = A.put(&d, std::vector<double>(m->w3mn, m->w3mn + n3)))) return st;
  a.w3 = d;
  if ((st = A.put(&d, face))) return st;
  a.face = d;
  if (!uniform) {
    if ((st = A.put(&d, fcoef))) return st;
    a.fcoef = d;
  }
  if ((st = A.put(&di, partner))) return st;
  a.partner = di;
  a.nelt = m->nelt;
  a.npts = npts;
  a.nxzfl = nxzfl;
  a.k = c->d_k;
  a.coef = c->d_coef;
  for (long i = 0; i < n2; ++i) a.D[i] = m->dxm1[i];
  c->host_w3.assign(m->w3mn, m->w3mn + n3);
  c->curved = true;
  // the fused arguments carry the source weights for the curved kernel too
  c->fargs = FusedDev{};
  c->fargs.nelt = m->nelt;
  c->fargs.npts = npts;
  return NEKGPU_OK;
}

int finish_init(Context* c, int st) {
  if (st) {
    free_all(c);
    return st;
  }
  return NEKGPU_OK;
}

bool valid_form(int form) {
  return form == NEKGPU_PLAIN || form == NEKGPU_FUSED64 || form == NEKGPU_MIXED ||
         form == NEKGPU_MIXED_NAIVE;
}

int sync_status(Context* c) {
  if (!c->h_status) {  // (a context without the page-locked word)
    if (check_cuda(cudaStreamSynchronize(c->stream))) return NEKGPU_ERR_CUDA;
    int h = 0;
    if (check_cuda(cudaMemcpy(&h, c->d_status, sizeof(int), cudaMemcpyDeviceToHost)))
      return NEKGPU_ERR_CUDA;
    return h ? NEKGPU_ERR_TIMEOUT : NEKGPU_OK;
  }
  // the status word follows the stream's work into page-locked memory: one
  // synchronisation, no separate copy call
  if (check_cuda(cudaMemcpyAsync(c->h_status, c->d_status, sizeof(int), cudaMemcpyDeviceToHost,
                                 c->stream)) ||
      check_cuda(cudaStreamSynchronize(c->stream)))
    return NEKGPU_ERR_CUDA;
  return *c->h_status ? NEKGPU_ERR_TIMEOUT : NEKGPU_OK;
}

double* state(Context* c) { return c->d_u[c->cur]; }

int copy_fields_in(Context* c, double* dst, const double* hn, const double* en, long ld) {
  const size_t w = c->npts * sizeof(double), pitch = ld * sizeof(double);
  if (check_cuda(cudaMemcpy2DAsync(dst, w, hn, pitch, w, 3, cudaMemcpyHostToDevice, c->stream)))
    return NEKGPU_ERR_CUDA;
  if (check_cuda(cudaMemcpy2DAsync(dst + 3 * c->npts, w, en, pitch, w, 3, cudaMemcpyHostToDevice,
                                   c->stream)))
    return NEKGPU_ERR_CUDA;
  return NEKGPU_OK;
}

int copy_fields_out(Context* c, const double* src, double* hn, double* en, long ld) {
  const size_t w = c->npts * sizeof(double), pitch = ld * sizeof(double);
  if (check_cuda(cudaMemcpy2DAsync(hn, pitch, src, w, w, 3, cudaMemcpyDeviceToHost, c->stream)))
    return NEKGPU_ERR_CUDA;
  if (check_cuda(cudaMemcpy2DAsync(en, pitch, src + 3 * c->npts, w, w, 3, cudaMemcpyDeviceToHost,
                                   c->stream)))
    return NEKGPU_ERR_CUDA;
  return NEKGPU_OK;
}


int plain_stage(Context* c, int rkstep, double time, double dt) {
  int st;
  const double rktime = time + dt * c->rk_c[rkstep - 1];
  if ((st = plain_cem_maxwell(c))) return st;
  if ((st = plain_restrict_to_face(c))) return st;
  if (c->pargs.ninc && ((st = incident_upload(c, rktime)) || (st = plain_incident(c)))) return st;
  const double rk[3] = {c->rk_a[rkstep - 1], c->rk_b[rkstep - 1], dt};
  if ((st = plain_flux3d(c, rk))) return st;
  if ((st = plain_add_flux_to_res(c))) return st;
  if ((st = plain_pml_step(c))) return st;
  if ((st = plain_dispersive(c, c->rk_a[rkstep - 1], c->rk_b[rkstep - 1], dt))) return st;
  if (c->src.enabled && (st = plain_usersrc(c, source_ft(c->src, rktime)))) return st;
  if ((st = plain_invqmass(c))) return st;
  if ((st = plain_rk_update(c, c->rk_a[rkstep - 1], c->rk_b[rkstep - 1], dt))) return st;
  return plain_pml_rk_update(c, c->rk_a[rkstep - 1], c->rk_b[rkstep - 1], dt);
}

// ---------------------------------------------------------------------------
// One RK step on host fields with the copies overlapped (mixed form), as a
// wavefront over element chunks.
// The elements are cut into up to sixteen contiguous chunks.  Stage s of a
// chunk reads the stage-(s-1) state of its own elements and of its face
// partners, and overwrites the buffer that stage s-1 read there, so it waits
// (events) only for stage s-1 of the chunks holding those partners; stage 1
// waits for their copies in.  The copies in follow a breadth-first order of
// the chunk graph from chunk 0, so every stage can start on the first chunks
// while later chunks are still arriving, and each chunk goes back as soon as
// its stage 5 is done, while other chunks still compute.  Each stage has its
// own stream and the two copy directions theirs, so copies in and out, and
// stages on different chunks, run together.  The kernels and their inputs are
// those of the plain sequence copy in, five stages, copy out: the results are
// bit-identical to it.
// ---------------------------------------------------------------------------
#ifndef NEKGPU_WAVEFRONT_CHUNKS
#define NEKGPU_WAVEFRONT_CHUNKS 16
#endif
constexpr int kWavefrontChunks = NEKGPU_WAVEFRONT_CHUNKS;  // at most, and at least 64 elements each

bool chunked_step_applies(Context* c) {
  if (c->form != NEKGPU_MIXED || c->ndim != 3 || c->curved || c->host_nbr.empty()) return false;
  const MixedDev& m = c->margs;
  if (m.pml.slot || m.disp.slot || m.inc_elem || m.gr.elem) return false;
  if (c->chunk_begin.empty()) {
    const int nch = std::min(kWavefrontChunks, c->nelt / 64);
    if (nch < 4) return false;
    c->chunk_begin.resize(nch + 1);
    for (int k = 0; k <= nch; ++k) c->chunk_begin[k] = (int)((long)c->nelt * k / nch);
    std::vector<int> owner(c->nelt);
    for (int k = 0; k < nch; ++k)
      for (int e = c->chunk_begin[k]; e < c->chunk_begin[k + 1]; ++e) owner[e] = k;
    c->chunk_adj.assign(nch, {});
    for (int k = 0; k < nch; ++k) {
      std::vector<char> mark(nch, 0);
      mark[k] = 1;
      for (int e = c->chunk_begin[k]; e < c->chunk_begin[k + 1]; ++e)
        for (int f = 0; f < 6; ++f) {
          const int p = c->host_nbr[6 * (long)e + f];
          if (p >= 0) mark[owner[p]] = 1;
        }
      for (int j = 0; j < nch; ++j)
        if (mark[j]) c->chunk_adj[k].push_back(j);
    }
    // copies in: breadth-first from chunk 0 (an arc around a periodic ring)
    std::vector<int> pos(nch, -1);
    c->chunk_in_order.clear();
    for (int root = 0; root < nch; ++root) {  // (a graph in pieces: each piece)
      if (pos[root] >= 0) continue;
      std::vector<int> queue{root};
      pos[root] = (int)c->chunk_in_order.size();
      c->chunk_in_order.push_back(root);
      for (size_t q = 0; q < queue.size(); ++q)
        for (int j : c->chunk_adj[queue[q]])
          if (pos[j] < 0) {
            pos[j] = (int)c->chunk_in_order.size();
            c->chunk_in_order.push_back(j);
            queue.push_back(j);
          }
    }
    // launches in the order their inputs become ready: the level of stage s
    // of chunk i is one more than the latest level among its dependencies
    std::vector<int> lvl(pos), nl(nch);
    std::vector<std::array<int, 3>> key;
    for (int st = 1; st <= 5; ++st) {
      for (int i = 0; i < nch; ++i) {
        int l = 0;
        for (int j : c->chunk_adj[i]) l = std::max(l, lvl[j] + 1);
        nl[i] = l;
        key.push_back({l, st, i});
      }
      lvl = nl;
    }
    std::sort(key.begin(), key.end());
    c->chunk_launch.clear();
    for (const auto& k : key) c->chunk_launch.push_back({k[1], k[2]});
    c->chunk_in.assign(nch, nullptr);
    c->chunk_done.assign(5 * (size_t)nch, nullptr);
    for (cudaEvent_t& e : c->chunk_in)
      if (check_cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming))) return false;
    for (cudaEvent_t& e : c->chunk_done)
      if (check_cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming))) return false;
    for (cudaEvent_t& e : c->chunk_fence)
      if (check_cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming))) return false;
    if (check_cuda(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking)) ||
        check_cuda(cudaStreamCreateWithFlags(&c->copy_out_stream, cudaStreamNonBlocking)))
      return false;
    for (cudaStream_t& q : c->stage_stream)
      if (check_cuda(cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking))) return false;
  }
  return c->copy_stream != nullptr;
}

int chunked_step(Context* c, double* hn, double* en, long ld, double time, double dt) {
  const int nch = (int)c->chunk_begin.size() - 1;
  const long N3 = (long)c->nx * c->nx * c->nx;
  const size_t pitch = ld * sizeof(double), w = c->npts * sizeof(double);
  int st;
  if ((st = scale_coef_pairs(c, dt))) return st;  // (once per dt, on the context stream)
  // every stream follows the earlier work on the context stream
  if (check_cuda(cudaEventRecord(c->chunk_fence[0], c->stream))) return NEKGPU_ERR_CUDA;
  for (cudaStream_t q : {c->copy_stream, c->copy_out_stream, c->stage_stream[0], c->stage_stream[1],
                         c->stage_stream[2], c->stage_stream[3], c->stage_stream[4]})
    if (check_cuda(cudaStreamWaitEvent(q, c->chunk_fence[0], 0))) return NEKGPU_ERR_CUDA;
  const int cur0 = c->cur;
  double* u = c->d_u[cur0];
  for (int k : c->chunk_in_order) {
    const long off = c->chunk_begin[k] * N3;
    const size_t bytes = (c->chunk_begin[k + 1] - c->chunk_begin[k]) * N3 * sizeof(double);
    if (check_cuda(cudaMemcpy2DAsync(u + off, w, hn + off, pitch, bytes, 3, cudaMemcpyHostToDevice,
                                     c->copy_stream)) ||
        check_cuda(cudaMemcpy2DAsync(u + 3 * c->npts + off, w, en + off, pitch, bytes, 3,
                                     cudaMemcpyHostToDevice, c->copy_stream)) ||
        check_cuda(cudaEventRecord(c->chunk_in[k], c->copy_stream)))
      return NEKGPU_ERR_CUDA;
  }
  double* out = c->d_u[cur0 ^ 1];  // stage 5's output buffer
  cudaStream_t saved = c->stream;
  for (const auto& sk : c->chunk_launch) {
    const int rk = sk.first, k = sk.second;
    cudaStream_t q = c->stage_stream[rk - 1];
    for (int j : c->chunk_adj[k]) {
      cudaEvent_t dep = rk == 1 ? c->chunk_in[j] : c->chunk_done[(size_t)(rk - 2) * nch + j];
      if (check_cuda(cudaStreamWaitEvent(q, dep, 0))) {
        c->stream = saved;
        return NEKGPU_ERR_CUDA;
      }
    }
    c->stream = q;
    c->cur = cur0 ^ ((rk - 1) & 1);
    st = mixed_stage_range(c, rk, time, dt, c->chunk_begin[k], c->chunk_begin[k + 1]);
    c->stream = saved;
    if (st) {
      c->cur = cur0;
      return st;
    }
    if (check_cuda(cudaEventRecord(c->chunk_done[(size_t)(rk - 1) * nch + k], q)))
      return NEKGPU_ERR_CUDA;
    if (rk == 5) {
      const long off = c->chunk_begin[k] * N3;
      const size_t bytes = (c->chunk_begin[k + 1] - c->chunk_begin[k]) * N3 * sizeof(double);
      if (check_cuda(cudaStreamWaitEvent(c->copy_out_stream, c->chunk_done[4 * (size_t)nch + k], 0)) ||
          check_cuda(cudaMemcpy2DAsync(hn + off, pitch, out + off, w, bytes, 3, cudaMemcpyDeviceToHost,
                                       c->copy_out_stream)) ||
          check_cuda(cudaMemcpy2DAsync(en + off, pitch, out + 3 * c->npts + off, w, bytes, 3,
                                       cudaMemcpyDeviceToHost, c->copy_out_stream)))
        return NEKGPU_ERR_CUDA;
    }
  }
  c->cur = cur0 ^ 1;
  // later work on the context stream follows the copies back (which follow
  // every stage: each stage-(s-1) launch is a dependency of some stage-s one)
  if (check_cuda(cudaEventRecord(c->chunk_fence[1], c->copy_out_stream)) ||
      check_cuda(cudaStreamWaitEvent(c->stream, c->chunk_fence[1], 0)))
    return NEKGPU_ERR_CUDA;
  return NEKGPU_OK;
}

bool pinned_host(const void* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// The wavefront step through a CUDA graph: captured on the first call with a
// given key (host arrays, state parity, dt, stage arguments) and replayed
// with one launch afterwards, so the ~80 kernels, 64 copies and their
// event dependencies cost one enqueue instead of several hundred.  Only for
// page-locked host arrays (a capture cannot hold pageable copies) and steps
// whose kernels take no time-dependent argument (no volume source); else,
// or when the capture fails, the step is enqueued directly.
int chunked_step_graph(Context* c, double* hn, double* en, long ld, double time, double dt) {
  if (c->src.enabled || !pinned_host(hn) || !pinned_host(en))
    return chunked_step(c, hn, en, ld, time, dt);
  int st = scale_coef_pairs(c, dt);  // outside the capture: the graph reads the scaled pairs
  if (st) return st;
  const int cur0 = c->cur;
  Context::StepGraph* hit = nullptr;
  for (auto& g : c->step_graphs)
    if (g.hn == hn && g.en == en && g.ld == ld && g.cur == cur0 && g.dt == dt &&
        std::memcmp(g.margs, &c->margs, sizeof(MixedDev)) == 0)
      hit = &g;
  if (!hit) {
    Context::StepGraph g{};
    g.hn = hn;
    g.en = en;
    g.ld = ld;
    g.cur = cur0;
    g.dt = dt;
    std::memcpy(g.margs, &c->margs, sizeof(MixedDev));
    const long l0 = c->last_launches;
    if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
      cudaGetLastError();
      return chunked_step(c, hn, en, ld, time, dt);
    }
    st = chunked_step(c, hn, en, ld, time, dt);
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(c->stream, &graph);
    c->cur = cur0;  // nothing ran
    g.launches = c->last_launches - l0;
    c->last_launches = l0;
    cudaError_t ei = cudaErrorUnknown;
    if (!st && ec == cudaSuccess && graph) ei = cudaGraphInstantiate(&g.exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (st || ec != cudaSuccess || ei != cudaSuccess) {
      cudaGetLastError();
      return chunked_step(c, hn, en, ld, time, dt);
    }
    if (c->step_graphs.size() >= 4) {  // (two parities x two array sets)
      cudaGraphExecDestroy(c->step_graphs.front().exec);
      c->step_graphs.erase(c->step_graphs.begin());
    }
    c->step_graphs.push_back(g);
    hit = &c->step_graphs.back();
  }
  if (check_cuda(cudaGraphLaunch(hit->exec, c->stream))) return NEKGPU_ERR_CUDA;
  c->last_launches += hit->launches;
  c->cur = cur0 ^ 1;
  return NEKGPU_OK;
}

int do_stage(Context* c, int rkstep, double time, double dt) {
  if (rkstep < 1 || rkstep > 5) return NEKGPU_ERR_ARG;
  if (c->ndim == 2) return stage2d(c, rkstep, time, dt);
  if (c->curved)
    return c->form == NEKGPU_MIXED ? mixed_curved_stage(c, rkstep, time, dt) : curved_stage(c, rkstep, time, dt);
  if (c->form == NEKGPU_PLAIN) return plain_stage(c, rkstep, time, dt);
  if (c->form == NEKGPU_MIXED) return mixed_stage(c, rkstep, time, dt);
  return fused_stage(c, rkstep, time, dt);
}

int do_steps(Context* c, int nsteps, double* time, double dt) {
  for (int s = 0; s < nsteps; ++s) {
    for (int r = 1; r <= 5; ++r) {
      int st = do_stage(c, r, *time, dt);
      if (st) return st;
    }
    *time = *time + dt;
  }
  return NEKGPU_OK;
}

}  // namespace

namespace nekgpu {

int mixed_companion(Context* c, double dt, std::vector<void*>& owned, MixedDev& m) {
  if (c->form != NEKGPU_FUSED64 || c->curved || c->ndim != 3 || c->nx < 3 || c->nx > kMaxMixed)
    return NEKGPU_ERR_UNSUPPORTED;
  if (c->npml || c->disp_n || !c->inc_slots.empty() || c->grdev.ng) return NEKGPU_ERR_UNSUPPORTED;
  const int n = c->nx;
  const long n3 = (long)n * n * n, npts = c->npts, nxzfl = c->nxzfl, nelt = c->nelt;
  auto dev = [&](size_t bytes) -> void* {
    void* p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    owned.push_back(p);
    return p;
  };
  // D in its FP32 pieces (the library's GLL D; the context's must agree)
  std::vector<double> z, w, D;
  gll(n - 1, z, w, D);
  double dmax = 0, diff = 0;
  for (size_t k = 0; k < D.size(); ++k) {
    dmax = std::max(dmax, std::fabs(D[k]));
    diff = std::max(diff, std::fabs(D[k] - c->fargs.D[k]));
  }
  if (diff > 1e-12 * dmax) return NEKGPU_ERR_MESH;
  std::vector<float> tab;
  split_D(D, n, tab);
  int st = mixed_upload_D(n, tab.data(), tab.size());
  if (st) return st;
  std::vector<double> eg(9 * (size_t)nelt), hb(npts), eb(npts);
  if (check_cuda(cudaMemcpy(eg.data(), c->d_egeom, eg.size() * 8, cudaMemcpyDeviceToHost)) ||
      check_cuda(cudaMemcpy(hb.data(), c->d_hbm1, npts * 8, cudaMemcpyDeviceToHost)) ||
      check_cuda(cudaMemcpy(eb.data(), c->d_ebm1, npts * 8, cudaMemcpyDeviceToHost)))
    return NEKGPU_ERR_CUDA;
  m = MixedDev{};
  m.nelt = c->nelt;
  m.npts = npts;
  m.k = m.k_out = c->d_k;
  m.nbr = c->d_nbr;
  m.C0f = (float)c->fargs.C0;
  m.status = c->d_status;
  // per element: rho_y, rho_z pairs and the lift factors (as upload_fused)
  {
    const double wend = c->fargs.w[0];
    std::vector<float> egm(16 * (size_t)nelt, 0.0f);
    for (long e = 0; e < nelt; ++e) {
      const double* g = &eg[9 * (size_t)e];
      const double ry = g[1] / g[0], rz = g[2] / g[0];
      float* o = &egm[16 * (size_t)e];
      o[0] = (float)ry; o[1] = (float)(ry - (double)o[0]);
      o[2] = (float)rz; o[3] = (float)(rz - (double)o[2]);
      for (int f = 0; f < 6; ++f) {
        const double lf = g[3 + f] / (wend * g[0]);
        o[4 + f] = (float)lf;
        o[10 + f] = (float)(lf - (double)o[4 + f]);
      }
    }
    float* d = (float*)dev(egm.size() * sizeof(float));
    if (!d || check_cuda(cudaMemcpy(d, egm.data(), egm.size() * sizeof(float), cudaMemcpyHostToDevice)))
      return d ? NEKGPU_ERR_CUDA : NEKGPU_ERR_NOMEM;
    m.egm = d;
  }
  // normalised inverse mass hbm1*w3*rx | ebm1*w3*rx, scaled by dt into pairs
  {
    std::vector<double> base(2 * (size_t)npts);
    for (long g = 0; g < npts; ++g) {
      const double f = c->host_w3[g % n3] * eg[9 * (g / n3)];
      base[g] = hb[g] * f;
      base[npts + g] = eb[g] * f;
    }
    double* db = (double*)dev(base.size() * 8);
    float2* cf = (float2*)dev(base.size() * sizeof(float2));
    if (!db || !cf) return NEKGPU_ERR_NOMEM;
    if (check_cuda(cudaMemcpy(db, base.data(), base.size() * 8, cudaMemcpyHostToDevice))) return NEKGPU_ERR_CUDA;
    if ((st = mixed_scale_pairs(c, cf, db, 2 * npts, dt))) return st;
    m.coef = cf;
  }
  // face coefficients as pairs (hi float4, lo float4 per face node)
  if (c->d_fcoef) {
    std::vector<double> fc(4 * (size_t)nxzfl);
    if (check_cuda(cudaMemcpy(fc.data(), c->d_fcoef, fc.size() * 8, cudaMemcpyDeviceToHost)))
      return NEKGPU_ERR_CUDA;
    std::vector<float> f(8 * (size_t)nxzfl);
    for (long j = 0; j < nxzfl; ++j)
      for (int q = 0; q < 4; ++q) {
        const double v = fc[4 * j + q];
        f[8 * j + q] = (float)v;
        f[8 * j + 4 + q] = (float)(v - (double)f[8 * j + q]);
      }
    float* d = (float*)dev(f.size() * sizeof(float));
    if (!d || check_cuda(cudaMemcpy(d, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice)))
      return d ? NEKGPU_ERR_CUDA : NEKGPU_ERR_NOMEM;
    m.fcoef = d;
  }
  // volume source: the FP64 weights normalised by w3*rx, as pairs
  if (c->src.enabled && c->fargs.src_elem) {
    std::vector<int> off(nelt);
    if (check_cuda(cudaMemcpy(off.data(), c->fargs.src_elem, nelt * sizeof(int), cudaMemcpyDeviceToHost)))
      return NEKGPU_ERR_CUDA;
    int cnt = 0;
    for (int o : off) cnt = std::max(cnt, o + 1);
    std::vector<double> wd((size_t)cnt * n3);
    if (cnt && check_cuda(cudaMemcpy(wd.data(), c->fargs.src_w, wd.size() * 8, cudaMemcpyDeviceToHost)))
      return NEKGPU_ERR_CUDA;
    std::vector<float> wf(2 * wd.size());
    for (long e = 0; e < nelt; ++e) {
      if (off[e] < 0) continue;
      for (long v = 0; v < n3; ++v) {
        const size_t i = (size_t)off[e] * n3 + v;
        const double x = wd[i] / (c->host_w3[v] * eg[9 * (size_t)e]);
        wf[2 * i] = (float)x;
        wf[2 * i + 1] = (float)(x - (double)wf[2 * i]);
      }
    }
    float* d = (float*)dev(std::max<size_t>(wf.size(), 2) * sizeof(float));
    if (!d) return NEKGPU_ERR_NOMEM;
    if (cnt && check_cuda(cudaMemcpy(d, wf.data(), wf.size() * sizeof(float), cudaMemcpyHostToDevice)))
      return NEKGPU_ERR_CUDA;
    m.src_elem = c->fargs.src_elem;
    m.src_w = reinterpret_cast<const float2*>(d);
  }
  return NEKGPU_OK;
}

}  // namespace nekgpu

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char* nekgpu_error_string(int status) {
  switch (status) {
    case NEKGPU_OK: return "ok";
    case NEKGPU_ERR_ARG: return "invalid argument";
    case NEKGPU_ERR_MESH: return "mesh not supported by this form";
    case NEKGPU_ERR_CUDA: return g_last_cuda.empty() ? "CUDA error" : g_last_cuda.c_str();
    case NEKGPU_ERR_NOMEM: return "device memory allocation failed or over budget";
    case NEKGPU_ERR_STATE: return "call out of order";
    case NEKGPU_ERR_BLOWUP: return "state blew up (non-finite or |u| > 1e20)";
    case NEKGPU_ERR_TIMEOUT: return "a bounded device wait ran out";
    case NEKGPU_ERR_UNSUPPORTED: return "not supported for this case";
    case NEKGPU_ERR_TOO_LARGE:
      return "mesh larger than the fixed scratch of the no-allocation entry point (8,388,608 nodes)";
    default: return "unknown status";
  }
}

int nekgpu_version(void) { return 1; }

int nekgpu_device_check(int device) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= device || device < 0) {
    cudaGetLastError();
    g_last_cuda = "no CUDA device available";
    return NEKGPU_ERR_CUDA;
  }
  if (check_cuda(cudaSetDevice(device))) return NEKGPU_ERR_CUDA;
  cudaDeviceProp p;
  if (check_cuda(cudaGetDeviceProperties(&p, device))) return NEKGPU_ERR_CUDA;
  if (p.major < 10) {
    g_last_cuda = "device is not Blackwell (sm_10x)";
    return NEKGPU_ERR_CUDA;
  }
  return NEKGPU_OK;
}

int nekgpu_init(nekgpu_ctx** ctx, const nekgpu_mesh* m, int form) {
  if (!ctx || !m || !valid_form(form)) return NEKGPU_ERR_ARG;
  *ctx = nullptr;
  if (m->nx1 < 2 || m->nx1 > kMaxNx || m->nelt < 1 || !m->dxm1 || !m->w3mn || !m->bmn ||
      !m->unxm || !m->unym || !m->unzm || !m->aream || !m->cemface || !m->glo_face ||
      !m->Z_0 || !m->Z_1 || !m->Y_0 || !m->Y_1 || !m->ebm1 || !m->hbm1 || !m->rxmn ||
      !m->rymn || !m->rzmn || !m->sxmn || !m->symn || !m->szmn || !m->txmn || !m->tymn ||
      !m->tzmn || m->ncempec < 0 || (m->ncempec > 0 && !m->cempec))
    return NEKGPU_ERR_ARG;
  nekgpu_ctx* c = new (std::nothrow) nekgpu_ctx();
  if (!c) return NEKGPU_ERR_NOMEM;
  int st;
  if (form == NEKGPU_PLAIN) {
    PlainHost p;
    st = build_plain(m, p);
    if (!st) st = common_setup(c, form, m->nx1, m->nelt);
    if (!st) st = upload_plain(c, p);
  } else {
    Compact cp;
    st = build_compact(m, cp);
    if (st == NEKGPU_ERR_MESH && (form == NEKGPU_FUSED64 || form == NEKGPU_MIXED)) {
      // not affine: the curvilinear variant of the fused FP64 or mixed form
      st = common_setup(c, form, m->nx1, m->nelt);
      if (!st) st = upload_curved(c, m);
    } else {
      if (!st) st = common_setup(c, form, m->nx1, m->nelt);
      if (!st) st = upload_fused(c, cp);
    }
  }
  if (!st && m->xmn && m->ymn && m->zmn) {
    c->host_x.assign(m->xmn, m->xmn + c->npts);
    c->host_y.assign(m->ymn, m->ymn + c->npts);
    c->host_z.assign(m->zmn, m->zmn + c->npts);
  }
  st = finish_init(c, st);
  if (st) {
    delete c;
    return st;
  }
  *ctx = c;
  return NEKGPU_OK;
}

int nekgpu_init2d(nekgpu_ctx** ctx, const nekgpu_mesh* m, int imode) {
  if (!ctx || !m || (imode != 1 && imode != 2)) return NEKGPU_ERR_ARG;
  *ctx = nullptr;
  if (m->nx1 < 2 || m->nx1 > kMaxNx || m->nelt < 1 || !m->dxm1 || !m->w3mn || !m->bmn ||
      !m->unxm || !m->unym || !m->aream || !m->cemface || !m->glo_face || !m->Z_0 || !m->Z_1 ||
      !m->Y_0 || !m->Y_1 || !m->ebm1 || !m->hbm1 || !m->rxmn || !m->rymn || !m->sxmn ||
      !m->symn || m->ncempec < 0 || (m->ncempec > 0 && !m->cempec))
    return NEKGPU_ERR_ARG;
  const int n = m->nx1;
  const long n2 = (long)n * n, npts = n2 * m->nelt, nxzfl = 4L * n * m->nelt;
  // the reference's 2-D face numbering: slot a + n*(f + 4e), f in pff order,
  // a ascending along the face (cem_set_fc_ptr with SKPDAT for NZ = 1)
  std::vector<int> cemface(nxzfl), partner(nxzfl, -1), pec(nxzfl, 0);
  for (long e = 0; e < m->nelt; ++e)
    for (int f = 0; f < 4; ++f)
      for (int a = 0; a < n; ++a) {
        const long js = a + (long)n * (f + 4 * e);
        const long vloc = f == 0 ? a : (f == 1 ? n - 1 + n * a : (f == 2 ? a + n * (n - 1) : n * a));
        if (m->cemface[js] - 1 != e * n2 + vloc) return NEKGPU_ERR_MESH;
        cemface[js] = (int)(e * n2 + vloc);
      }
  std::vector<int> pairs, single;
  int st = pairs_from_ids(m->glo_face, nxzfl, pairs, single);
  if (st) return st;
  for (size_t q = 0; q + 1 < pairs.size(); q += 2) {
    partner[pairs[q]] = pairs[q + 1];
    partner[pairs[q + 1]] = pairs[q];
  }
  for (int j = 0; j < m->ncempec; ++j) {
    const int sl = m->cempec[j] - 1;
    if (sl < 0 || sl >= nxzfl || partner[sl] >= 0) return NEKGPU_ERR_MESH;
    pec[sl] = 1;
  }
  nekgpu_ctx* c = new (std::nothrow) nekgpu_ctx();
  if (!c) return NEKGPU_ERR_NOMEM;
  st = common_setup(c, NEKGPU_FUSED64, n, m->nelt);
  if (!st) {
    c->ndim = 2;
    c->imode = imode;
    c->npts = npts;
    c->nxzfl = nxzfl;
    DevAlloc A(c);
    std::vector<double> bm1(m->bmn, m->bmn + npts), eb(m->ebm1, m->ebm1 + npts),
        hb(m->hbm1, m->hbm1 + npts);
    if (!st) st = A.get(&c->d_u[0], 6 * npts);
    if (!st) st = A.get(&c->d_u[1], 6 * npts);
    if (!st) st = upload_common(c, A, bm1, eb, hb);
    Stage2dDev& a = c->s2;
    a = Stage2dDev{};
    a.nx = n; a.nelt = m->nelt; a.imode = imode; a.npts = npts; a.nxzfl = nxzfl;
    a.C0 = m->C0;
    a.ebm1 = c->d_ebm1;
    a.hbm1 = c->d_hbm1;
    std::vector<double> D(m->dxm1, m->dxm1 + n2), Dt(n2);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) Dt[j + (size_t)n * i] = D[i + (size_t)n * j];
    const double* nsrc[4] = {m->rxmn, m->rymn, m->sxmn, m->symn};
    const double** ndst[4] = {&a.rx, &a.ry, &a.sx, &a.sy};
    const double* fsrc[7] = {m->unxm, m->unym, m->aream, m->Z_0, m->Z_1, m->Y_0, m->Y_1};
    const double** fdst[7] = {&a.unx, &a.uny, &a.area, &a.Z0, &a.Z1, &a.Y0, &a.Y1};
    double* d;
    if (!st && !(st = A.put(&d, D))) a.D = d;
    if (!st && !(st = A.put(&d, Dt))) a.Dt = d;
    if (!st && !(st = A.put(&d, std::vector<double>(m->w3mn, m->w3mn + n2)))) a.w3 = d;
    for (int q = 0; q < 4 && !st; ++q)
      if (!(st = A.put(&d, std::vector<double>(nsrc[q], nsrc[q] + npts)))) *ndst[q] = d;
    for (int q = 0; q < 7 && !st; ++q)
      if (!(st = A.put(&d, std::vector<double>(fsrc[q], fsrc[q] + nxzfl)))) *fdst[q] = d;
    int* di;
    if (!st && !(st = A.put(&di, cemface))) a.cemface = di;
    if (!st && !(st = A.put(&di, partner))) a.partner = di;
    if (!st && !(st = A.put(&di, pec))) a.pec = di;
    if (!st && m->pmlsigma && m->npml > 0) {
      // PML: the reference's full-size arrays, stepped by the stage kernel
      if (!m->pmlptr || !m->permittivity || !m->permeability) st = NEKGPU_ERR_ARG;
      std::vector<int> flag(m->nelt, 0);
      for (int l = 0; l < m->npml && !st; ++l) {
        const int e = m->pmlptr[l] - 1;
        if (e < 0 || e >= m->nelt || (l > 0 && e <= c->pml_elems.back())) st = NEKGPU_ERR_ARG;
        else { c->pml_elems.push_back(e); flag[e] = 1; }
      }
      if (!st) {
        c->npml = m->npml;
        int* dflag;
        if ((st = A.put(&dflag, flag)) ||
            (st = A.put(&c->d_pml_sigma, std::vector<double>(m->pmlsigma, m->pmlsigma + 3 * npts))) ||
            (st = A.put(&c->d_eps, std::vector<double>(m->permittivity, m->permittivity + npts))) ||
            (st = A.put(&c->d_mu, std::vector<double>(m->permeability, m->permeability + npts))) ||
            (st = A.get(&c->d_pml_aux, 6 * npts)) || (st = A.get(&c->d_pml_k, 6 * npts))) {
        } else if (check_cuda(cudaMemset(c->d_pml_aux, 0, 6 * npts * sizeof(double))) ||
                   check_cuda(cudaMemset(c->d_pml_k, 0, 6 * npts * sizeof(double)))) {
          st = NEKGPU_ERR_CUDA;
        } else {
          a.pml_elem = dflag;
          a.pml_sigma = c->d_pml_sigma;
          a.eps = c->d_eps;
          a.mu = c->d_mu;
          a.bm1 = c->d_bm1;
          a.pml_aux = c->d_pml_aux;
          a.pml_k = c->d_pml_k;
        }
      }
    }
    if (!st && m->xmn && m->ymn) {
      c->host_x.assign(m->xmn, m->xmn + npts);
      c->host_y.assign(m->ymn, m->ymn + npts);
      c->host_z.assign(npts, 0.0);
    }
  }
  st = finish_init(c, st);
  if (st) {
    delete c;
    return st;
  }
  *ctx = c;
  return NEKGPU_OK;
}

int nekgpu_init_box(nekgpu_ctx** ctx, const nekgpu_box* bx, int form) {
  if (!ctx || !bx || !valid_form(form)) return NEKGPU_ERR_ARG;
  *ctx = nullptr;
  BoxArrays A;
  int st = build_box(bx, A, form == NEKGPU_PLAIN);
  if (st) return st;
  if (form == NEKGPU_PLAIN) return nekgpu_init(ctx, &A.mesh, form);
  if (bx->N + 1 < 3 || bx->N + 1 > 9) return NEKGPU_ERR_UNSUPPORTED;
  nekgpu_ctx* c = new (std::nothrow) nekgpu_ctx();
  if (!c) return NEKGPU_ERR_NOMEM;
  Compact cp;
  compact_from_box(bx, A, cp);
  st = common_setup(c, form, bx->N + 1, A.mesh.nelt);
  if (!st) st = upload_fused(c, cp);
  if (!st) {
    c->host_x = std::move(A.x); c->host_y = std::move(A.y); c->host_z = std::move(A.z);
  }
  st = finish_init(c, st);
  if (st) {
    delete c;
    return st;
  }
  *ctx = c;
  return NEKGPU_OK;
}

int nekgpu_box_export_d(const nekgpu_box* bx, const char* name, double* out, long* count) {
  if (!bx || !name || !count) return NEKGPU_ERR_ARG;
  BoxArrays A;
  int st = build_box(bx, A, true);
  if (st) return st;
  std::string nm(name);
  const std::vector<double>* v = nullptr;
  if (nm == "dxm1") v = &A.D;
  else if (nm == "w3mn") v = &A.w3;
  else if (nm == "bmn") v = &A.bm1;
  else if (nm == "xmn") v = &A.x;
  else if (nm == "ymn") v = &A.y;
  else if (nm == "zmn") v = &A.z;
  else if (nm == "rxmn") v = &A.metrics[0];
  else if (nm == "symn") v = &A.metrics[4];
  else if (nm == "tzmn") v = &A.metrics[8];
  else if (nm == "ebm1") v = &A.ebm1;
  else if (nm == "hbm1") v = &A.hbm1;
  else if (nm == "unxm") v = &A.unx;
  else if (nm == "unym") v = &A.uny;
  else if (nm == "unzm") v = &A.unz;
  else if (nm == "aream") v = &A.area;
  else if (nm == "Z_0") v = &A.Z0;
  else if (nm == "Z_1") v = &A.Z1;
  else if (nm == "Y_0") v = &A.Y0;
  else if (nm == "Y_1") v = &A.Y1;
  else if (nm == "pmlsigma") v = &A.pml.sigma;
  if (!v) return NEKGPU_ERR_ARG;
  *count = (long)v->size();
  if (out) std::copy(v->begin(), v->end(), out);
  return NEKGPU_OK;
}

int nekgpu_box_export_i(const nekgpu_box* bx, const char* name, long long* out, long* count) {
  if (!bx || !name || !count) return NEKGPU_ERR_ARG;
  BoxArrays A;
  int st = build_box(bx, A, true);
  if (st) return st;
  std::string nm(name);
  if (nm == "glo_face") {
    *count = (long)A.glo.size();
    if (out) std::copy(A.glo.begin(), A.glo.end(), out);
  } else if (nm == "cemface") {
    *count = (long)A.cemface.size();
    if (out) std::copy(A.cemface.begin(), A.cemface.end(), out);
  } else if (nm == "cempec") {
    *count = (long)A.cempec.size();
    if (out) std::copy(A.cempec.begin(), A.cempec.end(), out);
  } else if (nm == "pmlptr") {
    *count = (long)A.pmlptr1.size();
    if (out) std::copy(A.pmlptr1.begin(), A.pmlptr1.end(), out);
  } else {
    return NEKGPU_ERR_ARG;
  }
  return NEKGPU_OK;
}

int nekgpu_finalize(nekgpu_ctx* c) {
  if (!c) return NEKGPU_ERR_ARG;
  if (c->stream) cudaStreamSynchronize(c->stream);
  free_all(c);
  delete c;
  return NEKGPU_OK;
}

int nekgpu_sizes(const nekgpu_ctx* c, long* npts, long* nxzfl, int* nelt, int* nx1) {
  if (!c) return NEKGPU_ERR_ARG;
  if (npts) *npts = c->npts;
  if (nxzfl) *nxzfl = c->nxzfl;
  if (nelt) *nelt = c->nelt;
  if (nx1) *nx1 = c->nx;
  return NEKGPU_OK;
}

double nekgpu_volume(const nekgpu_ctx* c) { return c ? c->volume : 0.0; }

int nekgpu_get_array(nekgpu_ctx* c, const char* name, double* out) {
  if (!c || !name || !out) return NEKGPU_ERR_ARG;
  const std::vector<double>* v = nullptr;
  std::string nm(name);
  if (nm == "xmn") v = &c->host_x;
  else if (nm == "ymn") v = &c->host_y;
  else if (nm == "zmn") v = &c->host_z;
  else if (nm == "bmn") v = &c->host_bm1;
  if (v) {
    if ((long)v->size() != c->npts) return NEKGPU_ERR_STATE;
    std::copy(v->begin(), v->end(), out);
    return NEKGPU_OK;
  }
  const double* d = nullptr;
  if (nm == "ebm1") d = c->d_ebm1;
  else if (nm == "hbm1") d = c->d_hbm1;
  if (d) return check_cuda(cudaMemcpy(out, d, c->npts * sizeof(double), cudaMemcpyDeviceToHost));
  // PML arrays, 3*npts in the reference layout (zero outside the PML)
  const bool bn = nm == "pmlbn", dn = nm == "pmldn", sg = nm == "pmlsigma";
  if (!bn && !dn && !sg) return NEKGPU_ERR_ARG;
  const long P = c->npts, n3 = (long)c->nx * c->nx * c->nx;
  std::fill(out, out + 3 * P, 0.0);
  if (!c->npml) return NEKGPU_OK;
  if (c->form == NEKGPU_PLAIN || c->ndim == 2) {  // full-size arrays
    const double* src = sg ? c->d_pml_sigma : c->d_pml_aux + (dn ? 3 * P : 0);
    return check_cuda(cudaMemcpy(out, src, 3 * P * sizeof(double), cudaMemcpyDeviceToHost));
  }
  const long nn = (long)c->npml * n3;
  std::vector<double> h(sg ? (size_t)kPmlData * nn : 6 * (size_t)nn);
  const double* src = sg ? c->d_pml_data : c->d_pml_aux;
  if (check_cuda(cudaMemcpy(h.data(), src, h.size() * sizeof(double), cudaMemcpyDeviceToHost)))
    return NEKGPU_ERR_CUDA;
  for (long l = 0; l < c->npml; ++l)
    for (long v = 0; v < n3; ++v) {
      const long q = l * n3 + v, g = (long)c->pml_elems[l] * n3 + v;
      for (int cc = 0; cc < 3; ++cc) {
        if (sg)  // sigma = (sigma/eps) * eps is not stored; sigma itself is q = 3..5
          out[cc * P + g] = h[(3 + cc) * nn + q];
        else
          out[cc * P + g] = h[((dn ? 3 : 0) + cc) * nn + q];
      }
    }
  return NEKGPU_OK;
}

long nekgpu_device_bytes(const nekgpu_ctx* c) { return c ? (long)c->dev_bytes : 0; }

int nekgpu_set_source_kind(nekgpu_ctx* c, int kind) {
  if (!c || kind < 0 || kind > 1) return NEKGPU_ERR_ARG;
  c->src.kind = kind;
  return NEKGPU_OK;
}

// userinc as a plane wave on listed face slots.  The values depend on the
// stage time; the host evaluates amp * cos(k.x - omega t) per listed slot
// each stage (the reference's arithmetic, on the CPU) and uploads them.
int nekgpu_set_incident(nekgpu_ctx* c, const int* slots, long n, const double amp[6],
                        const double kvec[3], double omega) {
  if (!c || n < 0 || (n > 0 && (!slots || !amp || !kvec))) return NEKGPU_ERR_ARG;
  if (c->ndim == 2 || c->curved || c->form == NEKGPU_MIXED_NAIVE) return NEKGPU_ERR_UNSUPPORTED;
  const long n3 = (long)c->nx * c->nx * c->nx, NF = 6L * c->nx * c->nx;
  if (n > 0 && (long)c->host_x.size() != c->npts) return NEKGPU_ERR_STATE;  // needs coordinates
  std::vector<int> sl(n), nodes(n);
  std::vector<char> seen(c->nxzfl, 0);
  for (long q = 0; q < n; ++q) {
    const long j = (long)slots[q] - 1;
    if (j < 0 || j >= c->nxzfl || seen[j]) return NEKGPU_ERR_ARG;
    seen[j] = 1;
    sl[q] = (int)j;
    if (c->form == NEKGPU_PLAIN) {
      nodes[q] = c->host_cemface.empty() ? -1 : c->host_cemface[j];
      if (nodes[q] < 0) return NEKGPU_ERR_STATE;
    } else {  // the fused forms hold the reference numbering (checked at init)
      const long e = j / NF, t = j % NF, f = t / ((long)c->nx * c->nx), ab = t % ((long)c->nx * c->nx);
      nodes[q] = (int)(e * n3 + face_vol((int)f, (int)(ab % c->nx), (int)(ab / c->nx), c->nx));
    }
  }
  for (const void* q : {(const void*)c->d_inc_slot, (const void*)c->d_inc_elem,
                        (const void*)c->d_inc_val, (const void*)c->pargs.inc_slot})
    release_dev(c, q);
  c->d_inc_slot = nullptr;
  c->d_inc_elem = nullptr;
  c->d_inc_val = nullptr;
  c->pargs.inc_slot = nullptr;
  DevAlloc A(c);
  int st;
  c->inc_slots = sl;
  c->inc_nodes = nodes;
  for (int m = 0; m < 6; ++m) c->inc_amp[m] = n ? amp[m] : 0.0;
  for (int m = 0; m < 3; ++m) c->inc_k[m] = n ? kvec[m] : 0.0;
  c->inc_omega = omega;
  c->pargs.ninc = 0;
  c->fargs.inc_elem = c->margs.inc_elem = nullptr;
  if (n == 0) return NEKGPU_OK;
  if (c->form == NEKGPU_PLAIN) {
    int* d;
    if ((st = A.put(&d, sl)) || (st = A.get(&c->d_inc_val, 6 * n))) return st;
    c->pargs.inc_slot = d;
    c->pargs.inc_val = c->d_inc_val;
    c->pargs.ninc = (int)n;
    c->inc_host.assign(6 * n, 0.0);
    return NEKGPU_OK;
  }
  // each listed slot adds to its own side and, across the face, to the value
  // its partner element sees of this side (the gs sum carries the modified
  // face value to both slots)
  std::vector<int> rows(c->nelt, -1);
  c->inc_elem_rows.clear();
  auto row_of = [&](int e) {
    if (rows[e] < 0) {
      rows[e] = (int)c->inc_elem_rows.size();
      c->inc_elem_rows.push_back(e);
    }
    return rows[e];
  };
  const long N2 = (long)c->nx * c->nx;
  c->inc_own_pos.assign(n, -1);
  c->inc_partner_pos.assign(n, -1);
  for (long q = 0; q < n; ++q) {
    const long j = sl[q], e = j / NF, t = j % NF, f = t / N2, ab = t % N2;
    c->inc_own_pos[q] = (long)row_of((int)e) * 12 * NF + t;
    const int pe = c->host_nbr[6 * e + f];
    if (pe >= 0) {
      const long fo = f < 4 ? (f + 2) & 3 : 9 - f;  // the opposite slot of the partner
      c->inc_partner_pos[q] = (long)row_of(pe) * 12 * NF + 6 * NF + fo * N2 + ab;
    }
  }
  const size_t nv = 12 * (size_t)NF * c->inc_elem_rows.size();
  if ((st = A.put(&c->d_inc_elem, rows)) || (st = A.get(&c->d_inc_val, nv))) return st;
  c->inc_host.assign(nv, 0.0);
  c->fargs.inc_elem = c->margs.inc_elem = c->d_inc_elem;
  c->fargs.inc_val = c->margs.inc_val = c->d_inc_val;
  return NEKGPU_OK;
}

// Graphene sheets in the fused FP64 and mixed forms: interior face slots of
// the affine mesh; Y_0 = (yconduc + partner's yconduc) / 2 as
// cem_maxwell_materials forms it for an interior face node.
static int set_graphene_fused(nekgpu_ctx* c, const double* params, const int* slots, long n,
                              const double* yconduc) {
  const long L = c->nxzfl, N2 = (long)c->nx * c->nx, NF = 6 * N2;
  std::vector<int> sl(n);
  std::vector<char> seen(L, 0);
  std::vector<double> par(12 * (size_t)n), y0(n), yc(n);
  std::vector<int> rows(c->nelt, -1), relem;
  auto row_of = [&](int e) {
    if (rows[e] < 0) {
      rows[e] = (int)relem.size();
      relem.push_back(e);
    }
    return rows[e];
  };
  std::vector<std::pair<long, int>> own, part;  // (row*NF + t, g)
  for (long q = 0; q < n; ++q) {
    const long j = (long)slots[q] - 1;
    if (j < 0 || j >= L || seen[j]) return NEKGPU_ERR_ARG;
    seen[j] = 1;
    sl[q] = (int)j;
    const long e = j / NF, t = j % NF, f = t / N2, ab = t % N2;
    const int pe = c->host_nbr[6 * e + f];
    if (pe < 0) return NEKGPU_ERR_UNSUPPORTED;  // sheets on interior faces only
    const long fo = f < 4 ? (f + 2) & 3 : 9 - f, tp = fo * N2 + ab;
    for (int p = 0; p < 12; ++p) par[p * n + q] = params[p * L + j];
    yc[q] = yconduc[j];
    y0[q] = 0.5 * (yconduc[j] + yconduc[(long)pe * NF + tp]);
    own.push_back({(long)row_of((int)e) * NF + t, (int)q});
    part.push_back({(long)row_of(pe) * NF + tp, (int)q});
  }
  GrapheneDev& G = c->grdev;
  for (const void* q : {(const void*)G.elem, (const void*)G.own, (const void*)G.part,
                        (const void*)G.par, (const void*)G.y0, (const void*)G.yc, (const void*)G.k,
                        (const void*)c->d_gr_f[0], (const void*)c->d_gr_f[1]})
    release_dev(c, q);
  G = GrapheneDev{};
  c->d_gr_f[0] = c->d_gr_f[1] = nullptr;
  c->gr_cur = 0;
  c->gr_slots = sl;
  c->fargs.gr = c->margs.gr = G;
  if (n == 0) return NEKGPU_OK;
  std::vector<int> vown(relem.size() * NF, -1), vpart(relem.size() * NF, -1);
  for (auto& o : own) vown[o.first] = o.second;
  for (auto& o : part) vpart[o.first] = o.second;
  DevAlloc A(c);
  int *d_elem, *d_own, *d_part;
  double *d_par, *d_y0, *d_yc, *d_k;
  int st;
  if ((st = A.put(&d_elem, rows)) || (st = A.put(&d_own, vown)) || (st = A.put(&d_part, vpart)) ||
      (st = A.put(&d_par, par)) || (st = A.put(&d_y0, y0)) || (st = A.put(&d_yc, yc)) ||
      (st = A.get(&d_k, 18 * n)) || (st = A.get(&c->d_gr_f[0], 18 * n)) ||
      (st = A.get(&c->d_gr_f[1], 18 * n)))
    return st;
  for (void* d : {(void*)d_k, (void*)c->d_gr_f[0], (void*)c->d_gr_f[1]})
    if (check_cuda(cudaMemset(d, 0, 18 * n * sizeof(double)))) return NEKGPU_ERR_CUDA;
  G.elem = d_elem; G.own = d_own; G.part = d_part;
  G.par = d_par; G.y0 = d_y0; G.yc = d_yc; G.k = d_k;
  G.ng = n;
  c->fargs.gr = c->margs.gr = G;
  return NEKGPU_OK;
}

// Graphene sheets (plain form): the reference's graphparams(nxzfl,12),
// graphindex (1-based) and yconduc(nxzfl); the face currents start at zero.
int nekgpu_set_graphene(nekgpu_ctx* c, const double* params, const int* slots, long n,
                        const double* yconduc) {
  if (!c || n < 0 || (n > 0 && (!params || !slots || !yconduc))) return NEKGPU_ERR_ARG;
  if (c->ndim == 2 || c->curved || c->form == NEKGPU_MIXED_NAIVE) return NEKGPU_ERR_UNSUPPORTED;
  if (c->form != NEKGPU_PLAIN) return set_graphene_fused(c, params, slots, n, yconduc);
  const long L = c->nxzfl;
  std::vector<int> sl(n);
  std::vector<char> seen(L, 0);
  std::vector<double> par(12 * (size_t)n), yc(n);
  for (long q = 0; q < n; ++q) {
    const long j = (long)slots[q] - 1;
    if (j < 0 || j >= L || seen[j]) return NEKGPU_ERR_ARG;
    seen[j] = 1;
    sl[q] = (int)j;
    for (int p = 0; p < 12; ++p) par[p * n + q] = params[p * L + j];
    yc[q] = yconduc[j];
  }
  PlainDev& pa = c->pargs;
  for (const void* q : {(const void*)pa.gr_slot, (const void*)pa.gr_par, (const void*)pa.gr_yc,
                        (const void*)pa.gr_f, (const void*)pa.gr_k})
    release_dev(c, q);
  pa.gr_slot = nullptr;
  pa.gr_par = pa.gr_yc = nullptr;
  pa.gr_f = pa.gr_k = nullptr;
  pa.ngraph = 0;
  c->gr_slots = sl;
  if (n == 0) return NEKGPU_OK;
  DevAlloc A(c);
  int* d_sl;
  double *d_par, *d_yc, *d_f, *d_k;
  int st;
  if ((st = A.put(&d_sl, sl)) || (st = A.put(&d_par, par)) || (st = A.put(&d_yc, yc)) ||
      (st = A.get(&d_f, 18 * n)) || (st = A.get(&d_k, 18 * n)))
    return st;
  if (check_cuda(cudaMemset(d_f, 0, 18 * n * sizeof(double))) ||
      check_cuda(cudaMemset(d_k, 0, 18 * n * sizeof(double))))
    return NEKGPU_ERR_CUDA;
  PlainDev& a = c->pargs;
  a.gr_slot = d_sl; a.gr_par = d_par; a.gr_yc = d_yc; a.gr_f = d_f; a.gr_k = d_k;
  a.ngraph = (int)n;
  return NEKGPU_OK;
}

// The graphene face currents in the reference layout fjn(ld,3,6) (only the
// listed slots are read / written; other slots read 0)
static int graphene_copy(nekgpu_ctx* c, double* fjn, long ld, bool to_device) {
  if (!c || !fjn || ld < c->nxzfl) return NEKGPU_ERR_ARG;
  const bool plain = c->form == NEKGPU_PLAIN;
  const long ng = plain ? c->pargs.ngraph : c->grdev.ng;
  double* dptr = plain ? c->pargs.gr_f : c->d_gr_f[c->gr_cur];
  std::vector<double> h(18 * (size_t)ng);
  if (ng && (check_cuda(cudaStreamSynchronize(c->stream)) ||
             check_cuda(cudaMemcpy(h.data(), dptr, h.size() * sizeof(double),
                                   cudaMemcpyDeviceToHost))))
    return NEKGPU_ERR_CUDA;
  if (!to_device) std::fill(fjn, fjn + 18 * ld, 0.0);
  for (long q = 0; q < ng; ++q)
    for (int r = 0; r < 18; ++r) {  // r = 3k + m: fjn(j, m, k)
      if (to_device)
        h[r * ng + q] = fjn[r * ld + c->gr_slots[q]];
      else
        fjn[r * ld + c->gr_slots[q]] = h[r * ng + q];
    }
  if (to_device && ng &&
      check_cuda(cudaMemcpy(dptr, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice)))
    return NEKGPU_ERR_CUDA;
  return NEKGPU_OK;
}

int nekgpu_set_graphene_current(nekgpu_ctx* c, const double* fjn, long ld) {
  return graphene_copy(c, const_cast<double*>(fjn), ld, true);
}

int nekgpu_get_graphene_current(nekgpu_ctx* c, double* fjn, long ld) {
  return graphene_copy(c, fjn, ld, false);
}

// PML auxiliary fields set from the reference layout (3*npts; the case's
// userini sets pmlbn = mu H, pmldn = eps E); nodes outside the PML ignored
int nekgpu_set_array(nekgpu_ctx* c, const char* name, const double* in) {
  if (!c || !name || !in) return NEKGPU_ERR_ARG;
  const std::string nm(name);
  const bool bn = nm == "pmlbn", dn = nm == "pmldn";
  if (!bn && !dn) return NEKGPU_ERR_ARG;
  if (!c->npml) return NEKGPU_ERR_STATE;
  const long P = c->npts, n3 = (long)c->nx * c->nx * c->nx;
  if (check_cuda(cudaStreamSynchronize(c->stream))) return NEKGPU_ERR_CUDA;
  if (c->form == NEKGPU_PLAIN || c->ndim == 2)  // full-size arrays
    return check_cuda(cudaMemcpy(c->d_pml_aux + (dn ? 3 * P : 0), in, 3 * P * sizeof(double),
                                 cudaMemcpyHostToDevice));
  const long nn = (long)c->npml * n3;
  std::vector<double> h(6 * (size_t)nn);
  if (check_cuda(cudaMemcpy(h.data(), c->d_pml_aux, h.size() * sizeof(double), cudaMemcpyDeviceToHost)))
    return NEKGPU_ERR_CUDA;
  for (long l = 0; l < c->npml; ++l)
    for (long v = 0; v < n3; ++v) {
      const long q = l * n3 + v, g = (long)c->pml_elems[l] * n3 + v;
      for (int cc = 0; cc < 3; ++cc) h[((dn ? 3 : 0) + cc) * nn + q] = in[cc * P + g];
    }
  return check_cuda(cudaMemcpy(c->d_pml_aux, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
}

// Dealiased curl (plain form, and the fused FP64 form on curvilinear
// meshes): the driver's tables as the reference builds them on the first
// maxwell_wght_dcurl call.
int nekgpu_set_dealias(nekgpu_ctx* c, int lxd, const double* jgl, const double* dxmd,
                       const double* w3md, const double* metd) {
  if (!c) return NEKGPU_ERR_ARG;
  const bool fused_curved = c->form == NEKGPU_FUSED64 && c->curved;
  if ((c->form != NEKGPU_PLAIN && !fused_curved) || c->ndim == 2) return NEKGPU_ERR_UNSUPPORTED;
  {
    PlainDev& pa = c->pargs;
    for (const void* q : {(const void*)pa.jgl, (const void*)pa.jgt, (const void*)pa.dxmd,
                          (const void*)pa.dxtmd, (const void*)pa.w3md, (const void*)pa.metd})
      release_dev(c, q);
    pa.jgl = pa.jgt = pa.dxmd = pa.dxtmd = pa.w3md = pa.metd = nullptr;
    pa.md = 0;
  }
  if (lxd == 0) return NEKGPU_OK;
  const int mx = c->nx, md = lxd;
  if (md < mx || !jgl || !dxmd || !w3md || !metd) return NEKGPU_ERR_ARG;
  int dev_smem = 0;
  cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device);
  if (dcurl_smem(mx, md) > (size_t)std::min(dev_smem, 220 * 1024)) return NEKGPU_ERR_UNSUPPORTED;
  const long md2 = (long)md * md, md3 = md2 * md;
  std::vector<double> vjgl(jgl, jgl + md * mx), vjgt((size_t)md * mx), vD(dxmd, dxmd + md2),
      vDt(md2), vw3(w3md, w3md + md3), vmet(metd, metd + 9 * md3 * c->nelt);
  for (int j = 0; j < mx; ++j)
    for (int i = 0; i < md; ++i) vjgt[j + (size_t)mx * i] = vjgl[i + (size_t)md * j];
  for (int j = 0; j < md; ++j)
    for (int i = 0; i < md; ++i) vDt[j + (size_t)md * i] = vD[i + (size_t)md * j];
  DevAlloc A(c);
  double *d1, *d2, *d3, *d4, *d5, *d6;
  int st;
  if ((st = A.put(&d1, vjgl)) || (st = A.put(&d2, vjgt)) || (st = A.put(&d3, vD)) ||
      (st = A.put(&d4, vDt)) || (st = A.put(&d5, vw3)) || (st = A.put(&d6, vmet)))
    return st;
  if (fused_curved && !c->d_vres && (st = A.get(&c->d_vres, 6 * (size_t)c->npts))) return st;
  PlainDev& a = c->pargs;
  a.jgl = d1; a.jgt = d2; a.dxmd = d3; a.dxtmd = d4; a.w3md = d5; a.metd = d6;
  a.md = md;
  return NEKGPU_OK;
}

// Dispersive media: the per-node model and parameters live on the host; each
// call rebuilds the compact per-element device arrays of all listed nodes.
int nekgpu_set_dispersive(nekgpu_ctx* c, int model, const double* params, long ld,
                          const int* index, long n) {
  if (!c || (model != NEKGPU_DRUDE && model != NEKGPU_LORENTZ) || n < 0 ||
      (n > 0 && (!params || !index || ld < c->npts)))
    return NEKGPU_ERR_ARG;
  if (c->form == NEKGPU_MIXED_NAIVE || c->ndim == 2 || c->curved) return NEKGPU_ERR_UNSUPPORTED;
  const long P = c->npts, n3 = (long)c->nx * c->nx * c->nx;
  std::vector<signed char> kind = c->disp_kind;
  std::vector<double> par = c->disp_par;
  if (kind.empty()) {
    kind.assign(P, 0);
    par.assign(3 * P, 0.0);
  }
  for (long j = 0; j < P; ++j)
    if (kind[j] == model) kind[j] = 0;
  for (long i = 0; i < n; ++i) {
    const long j = (long)index[i] - 1;
    if (j < 0 || j >= P || kind[j] != 0) return NEKGPU_ERR_ARG;  // out of range or listed twice
    kind[j] = (signed char)model;
    par[j] = params[j];
    par[P + j] = params[ld + j];
    par[2 * P + j] = model == NEKGPU_LORENTZ ? params[2 * ld + j] : 0.0;
  }
  std::vector<int> slot(c->nelt, -1), elems;
  for (int e = 0; e < c->nelt; ++e)
    for (long v = 0; v < n3; ++v)
      if (kind[e * n3 + v]) {
        slot[e] = (int)elems.size();
        elems.push_back(e);
        break;
      }
  const long nn = (long)elems.size() * n3;
  for (const void* q : {(const void*)c->d_disp_slot, (const void*)c->d_disp_elem,
                        (const void*)c->d_disp_data, (const void*)c->d_disp_aux,
                        (const void*)c->d_disp_k})
    release_dev(c, q);
  c->d_disp_slot = c->d_disp_elem = nullptr;
  c->d_disp_data = c->d_disp_aux = c->d_disp_k = nullptr;
  DispDev d{};
  if (nn) {
    std::vector<double> data((size_t)kDispData * nn, 0.0);
    for (size_t l = 0; l < elems.size(); ++l)
      for (long v = 0; v < n3; ++v) {
        const long j = elems[l] * n3 + v, q = (long)l * n3 + v;
        data[q] = kind[j];
        for (int p = 0; p < 3; ++p) data[(1 + p) * nn + q] = par[p * P + j];
        data[4 * nn + q] = c->host_bm1[j];
        if (!c->host_rx.empty())
          data[5 * nn + q] = c->host_bm1[j] / (c->host_w3[v] * c->host_rx[elems[l]]);
      }
    DevAlloc A(c);
    int* d_slot;
    int* d_elem;
    double *d_data, *d_aux, *d_k;
    int st;
    if ((st = A.put(&d_slot, slot)) || (st = A.put(&d_elem, elems)) || (st = A.put(&d_data, data)) ||
        (st = A.get(&d_aux, 6 * nn)) || (st = A.get(&d_k, 6 * nn)))
      return st;
    if (check_cuda(cudaMemset(d_aux, 0, 6 * nn * sizeof(double))) ||
        check_cuda(cudaMemset(d_k, 0, 6 * nn * sizeof(double))))
      return NEKGPU_ERR_CUDA;
    d = DispDev{d_slot, d_elem, d_data, d_aux, d_k, nn};
  }
  c->disp_kind.swap(kind);
  c->disp_par.swap(par);
  c->disp_slot.swap(slot);
  c->disp_elems.swap(elems);
  c->d_disp_slot = const_cast<int*>(d.slot);
  c->d_disp_elem = const_cast<int*>(d.elem);
  c->d_disp_data = const_cast<double*>(d.data);
  c->d_disp_aux = d.aux;
  c->d_disp_k = d.k;
  c->disp_n = nn;
  c->pargs.disp = d;
  c->fargs.disp = d;
  c->margs.disp = d;
  return NEKGPU_OK;
}

static int current_copy(nekgpu_ctx* c, int model, double* jn, long ld, bool to_device) {
  if (!c || (model != NEKGPU_DRUDE && model != NEKGPU_LORENTZ) || !jn || ld < c->npts)
    return NEKGPU_ERR_ARG;
  const long P = c->npts, n3 = (long)c->nx * c->nx * c->nx, nn = c->disp_n;
  const int nc = model == NEKGPU_DRUDE ? 3 : 6;
  std::vector<double> aux(6 * nn);
  if (nn && check_cuda(cudaStreamSynchronize(c->stream))) return NEKGPU_ERR_CUDA;
  if (nn && check_cuda(cudaMemcpy(aux.data(), c->d_disp_aux, aux.size() * sizeof(double),
                                  cudaMemcpyDeviceToHost)))
    return NEKGPU_ERR_CUDA;
  if (!to_device)
    for (int q = 0; q < nc; ++q) std::fill(jn + q * ld, jn + q * ld + P, 0.0);
  for (size_t l = 0; l < c->disp_elems.size(); ++l)
    for (long v = 0; v < n3; ++v) {
      const long j = (long)c->disp_elems[l] * n3 + v, t = (long)l * n3 + v;
      if (c->disp_kind[j] != model) continue;
      for (int q = 0; q < nc; ++q) {
        if (to_device)
          aux[q * nn + t] = jn[q * ld + j];
        else
          jn[q * ld + j] = aux[q * nn + t];
      }
    }
  if (to_device && nn &&
      check_cuda(cudaMemcpy(c->d_disp_aux, aux.data(), aux.size() * sizeof(double),
                            cudaMemcpyHostToDevice)))
    return NEKGPU_ERR_CUDA;
  return NEKGPU_OK;
}

int nekgpu_set_current(nekgpu_ctx* c, int model, const double* jn, long ld) {
  return current_copy(c, model, const_cast<double*>(jn), ld, true);
}

int nekgpu_get_current(nekgpu_ctx* c, int model, double* jn, long ld) {
  return current_copy(c, model, jn, ld, false);
}

int nekgpu_set_source(nekgpu_ctx* c, int enabled, const double xc[3], double sigma, double amp,
                      double f0, double t0) {
  if (!c) return NEKGPU_ERR_ARG;
  if (!enabled) {
    c->src.enabled = false;
    c->s2.src_w = nullptr;
    c->pargs.src_w = nullptr;
    c->fargs.src_elem = nullptr;
    c->fargs.src_w = nullptr;
    c->margs.src_elem = nullptr;
    c->margs.src_w = nullptr;
    return NEKGPU_OK;
  }
  if (!xc || !(sigma > 0)) return NEKGPU_ERR_ARG;
  // 2-D: a line source along z on the out-of-plane field, E3 = E_z in TM and
  // H3 = H_z in TE, as the reference's 2-D cases drive them
  if ((long)c->host_x.size() != c->npts) return NEKGPU_ERR_STATE;  // needs coordinates
  const double s2 = 2.0 * sigma * sigma;
  std::vector<double> g(c->npts);
  double gmax = 0;
  for (long i = 0; i < c->npts; ++i) {
    const double dx = c->host_x[i] - xc[0], dy = c->host_y[i] - xc[1], dz = c->host_z[i] - xc[2];
    g[i] = c->host_bm1[i] * std::exp(-(dx * dx + dy * dy + dz * dz) / s2);
    gmax = std::max(gmax, g[i]);
  }
  DevAlloc A(c);
  int st;
  if (c->form == NEKGPU_PLAIN || c->ndim == 2) {
    if (!c->d_src_w_plain && (st = A.get(&c->d_src_w_plain, c->npts))) return st;
    if (check_cuda(cudaMemcpy(c->d_src_w_plain, g.data(), c->npts * sizeof(double),
                              cudaMemcpyHostToDevice)))
      return NEKGPU_ERR_CUDA;
    if (c->ndim == 2)
      c->s2.src_w = c->d_src_w_plain;
    else
      c->pargs.src_w = c->d_src_w_plain;
  } else {
    release_dev(c, c->d_src_elem);  // a previous source's arrays
    release_dev(c, c->d_src_w);
    c->d_src_elem = nullptr;
    c->d_src_w = nullptr;
    // elements whose weights are all below 1e-30 of the peak carry no source
    const long n3 = (long)c->nx * c->nx * c->nx;
    std::vector<int> off(c->nelt, -1);
    std::vector<double> wd;
    int cnt = 0;
    for (int e = 0; e < c->nelt; ++e) {
      double m = 0;
      for (long v = 0; v < n3; ++v) m = std::max(m, g[e * n3 + v]);
      if (m > 1e-30 * gmax) {
        off[e] = cnt++;
        wd.insert(wd.end(), g.begin() + e * n3, g.begin() + (e + 1) * n3);
      }
    }
    int* d_off;
    if ((st = A.put(&d_off, off))) return st;
    if (c->form == NEKGPU_MIXED && !c->curved) {
      // normalised like the residual: weight / (bm1 * 2/hx) = weight / (w3 * rx),
      // as a (hi, lo) float pair (~2^-48 of the weight)
      std::vector<float> wf(2 * wd.size());
      for (int e = 0, s0 = 0; e < c->nelt; ++e) {
        if (off[e] < 0) continue;
        for (long v = 0; v < n3; ++v) {
          const size_t i = (size_t)s0 * n3 + v;
          const double w = wd[i] / (c->host_w3[v] * c->host_rx[e]);
          const float hi = (float)w;
          wf[2 * i] = hi;
          wf[2 * i + 1] = (float)(w - (double)hi);
        }
        ++s0;
      }
      float* d;
      if ((st = A.put(&d, wf))) return st;
      c->d_src_w = d;
      c->margs.src_elem = d_off;
      c->margs.src_w = reinterpret_cast<const float2*>(d);
    } else if (c->form == NEKGPU_MIXED_NAIVE) {
      std::vector<float> wf(wd.begin(), wd.end());
      float* d;
      if ((st = A.put(&d, wf))) return st;
      c->d_src_w = d;
    } else {
      double* d;
      if ((st = A.put(&d, wd))) return st;
      c->d_src_w = d;
    }
    c->d_src_elem = d_off;
    c->fargs.src_elem = d_off;
    c->fargs.src_w = c->d_src_w;
  }
  c->src.enabled = true;
  c->src.xc[0] = xc[0]; c->src.xc[1] = xc[1]; c->src.xc[2] = xc[2];
  c->src.sigma = sigma; c->src.amp = amp; c->src.f0 = f0; c->src.t0 = t0;
  return NEKGPU_OK;
}

int nekgpu_set_state(nekgpu_ctx* c, const double* hn, const double* en, long ld) {
  if (!c || !hn || !en || ld < c->npts) return NEKGPU_ERR_ARG;
  int st = copy_fields_in(c, state(c), hn, en, ld);
  if (st) return st;
  if (check_cuda(cudaMemsetAsync(c->d_k, 0, 6 * c->npts * sizeof(double), c->stream)))
    return NEKGPU_ERR_CUDA;
  c->have_state = true;
  return check_cuda(cudaStreamSynchronize(c->stream));
}

int nekgpu_get_state(nekgpu_ctx* c, double* hn, double* en, long ld) {
  if (!c || !hn || !en || ld < c->npts) return NEKGPU_ERR_ARG;
  int st = copy_fields_out(c, state(c), hn, en, ld);
  if (st) return st;
  return sync_status(c);
}

int nekgpu_set_rk_register(nekgpu_ctx* c, const double* khn, const double* ken, long ld) {
  if (!c || !khn || !ken || ld < c->npts) return NEKGPU_ERR_ARG;
  int st = copy_fields_in(c, c->d_k, khn, ken, ld);
  if (st) return st;
  return check_cuda(cudaStreamSynchronize(c->stream));
}

int nekgpu_get_rk_register(nekgpu_ctx* c, double* khn, double* ken, long ld) {
  if (!c || !khn || !ken || ld < c->npts) return NEKGPU_ERR_ARG;
  int st = copy_fields_out(c, c->d_k, khn, ken, ld);
  if (st) return st;
  return sync_status(c);
}

int nekgpu_register_host(nekgpu_ctx* c, void* ptr, long bytes) {
  if (!c || !ptr || bytes <= 0) return NEKGPU_ERR_ARG;
  return check_cuda(cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterDefault));
}

int nekgpu_unregister_host(nekgpu_ctx* c, void* ptr) {
  if (!c || !ptr) return NEKGPU_ERR_ARG;
  drop_step_graphs(c);  // their copies may read this memory
  return check_cuda(cudaHostUnregister(ptr));
}

int nekgpu_stage(nekgpu_ctx* c, int rkstep, double time, double dt) {
  if (!c) return NEKGPU_ERR_ARG;
  if (!c->have_state) return NEKGPU_ERR_STATE;
  c->last_launches = 0;
  return do_stage(c, rkstep, time, dt);
}

int nekgpu_step(nekgpu_ctx* c, int nsteps, double* time, double dt) {
  if (!c || !time || nsteps < 0) return NEKGPU_ERR_ARG;
  if (!c->have_state) return NEKGPU_ERR_STATE;
  c->last_launches = 0;
  return do_steps(c, nsteps, time, dt);
}

int nekgpu_op_rk_host(nekgpu_ctx* c, double* hn, double* en, long ld, double time, double dt) {
  if (!c || !hn || !en || ld < c->npts) return NEKGPU_ERR_ARG;
  c->last_launches = 0;
  int st = NEKGPU_OK;
  if (chunked_step_applies(c)) {
    if ((st = chunked_step_graph(c, hn, en, ld, time, dt))) return st;
    c->have_state = true;
    return sync_status(c);
  }
  st = copy_fields_in(c, state(c), hn, en, ld);
  if (st) return st;
  c->have_state = true;
  for (int r = 1; r <= 5 && !st; ++r) st = do_stage(c, r, time, dt);
  if (st) return st;
  st = copy_fields_out(c, state(c), hn, en, ld);
  if (st) return st;
  return sync_status(c);
}

static int plain_only(nekgpu_ctx* c) {
  if (!c) return NEKGPU_ERR_ARG;
  if (c->form != NEKGPU_PLAIN) return NEKGPU_ERR_UNSUPPORTED;
  c->last_launches = 0;
  return NEKGPU_OK;
}

int nekgpu_cem_maxwell(nekgpu_ctx* c) {
  int st = plain_only(c);
  return st ? st : plain_cem_maxwell(c);
}
int nekgpu_restrict_to_face(nekgpu_ctx* c) {
  int st = plain_only(c);
  return st ? st : plain_restrict_to_face(c);
}
int nekgpu_flux3d(nekgpu_ctx* c) {
  int st = plain_only(c);
  return st ? st : plain_flux3d(c);
}
int nekgpu_add_flux_to_res(nekgpu_ctx* c) {
  int st = plain_only(c);
  return st ? st : plain_add_flux_to_res(c);
}
int nekgpu_usersrc(nekgpu_ctx* c, double rktime) {
  int st = plain_only(c);
  if (st) return st;
  if (!c->src.enabled) return NEKGPU_OK;
  return plain_usersrc(c, source_ft(c->src, rktime));
}
int nekgpu_invqmass(nekgpu_ctx* c) {
  int st = plain_only(c);
  return st ? st : plain_invqmass(c);
}
int nekgpu_rk_maxwell_ab(nekgpu_ctx* c, int rkstep, double dt) {
  int st = plain_only(c);
  if (st) return st;
  if (rkstep < 1 || rkstep > 5) return NEKGPU_ERR_ARG;
  return plain_rk_update(c, c->rk_a[rkstep - 1], c->rk_b[rkstep - 1], dt);
}

int nekgpu_gs_op_fields(nekgpu_ctx* c, double* u, int nfld) {
  int st = plain_only(c);
  if (st) return st;
  if (!u || nfld < 1 || nfld > 6) return NEKGPU_ERR_ARG;
  double* d = c->pargs.srflx;  // scratch of 6*nxzfl
  const size_t bytes = (size_t)nfld * c->nxzfl * sizeof(double);
  if (check_cuda(cudaMemcpyAsync(d, u, bytes, cudaMemcpyHostToDevice, c->stream))) return NEKGPU_ERR_CUDA;
  if ((st = plain_gs(c, d, nfld))) return st;
  if (check_cuda(cudaMemcpyAsync(u, d, bytes, cudaMemcpyDeviceToHost, c->stream))) return NEKGPU_ERR_CUDA;
  return check_cuda(cudaStreamSynchronize(c->stream));
}

int nekgpu_get_work(nekgpu_ctx* c, const char* name, double* out) {
  int st = plain_only(c);
  if (st) return st;
  if (!name || !out) return NEKGPU_ERR_ARG;
  std::string nm(name);
  const double* src = nullptr;
  size_t count = 0;
  if (nm == "reshn") { src = c->pargs.res; count = 3 * c->npts; }
  else if (nm == "resen") { src = c->pargs.res + 3 * c->npts; count = 3 * c->npts; }
  else if (nm == "fhn") { src = c->pargs.fface; count = 3 * c->nxzfl; }
  else if (nm == "fen") { src = c->pargs.fface + 3 * c->nxzfl; count = 3 * c->nxzfl; }
  else if (nm == "srflx") { src = c->pargs.srflx; count = 6 * c->nxzfl; }
  else return NEKGPU_ERR_ARG;
  if (check_cuda(cudaMemcpyAsync(out, src, count * sizeof(double), cudaMemcpyDeviceToHost, c->stream)))
    return NEKGPU_ERR_CUDA;
  return check_cuda(cudaStreamSynchronize(c->stream));
}

int nekgpu_norms(nekgpu_ctx* c, const double* exact_h, const double* exact_e, long ld,
                 double l2[6], double linf[6]) {
  if (!c || !exact_h || !exact_e || !l2 || !linf || ld < c->npts) return NEKGPU_ERR_ARG;
  double* d = nullptr;
  if (check_cuda(cudaMallocAsync(&d, 6 * c->npts * sizeof(double), c->stream))) return NEKGPU_ERR_NOMEM;
  int st = copy_fields_in(c, d, exact_h, exact_e, ld);
  if (!st) st = util_norms(c, d, l2, linf);
  cudaFreeAsync(d, c->stream);
  cudaStreamSynchronize(c->stream);
  return st;
}

int nekgpu_norms_noalloc(nekgpu_ctx* c, const double* exact_dev, double l2[6], double linf[6]) {
  if (!c || !exact_dev || !l2 || !linf) return NEKGPU_ERR_ARG;
  return norms_noalloc(c, exact_dev, l2, linf);
}

int nekgpu_energy(nekgpu_ctx* c, double* energy) {
  if (!c || !energy) return NEKGPU_ERR_ARG;
  return util_energy(c, energy);
}

int nekgpu_selftest_pair_join(const float* s, const float* t, double* out, long n) {
  if (!s || !t || !out || n < 1 || n > (1L << 26)) return NEKGPU_ERR_ARG;
  int st = nekgpu_device_check(0);
  if (st) return st;
  float *ds = nullptr, *dt = nullptr;
  double* dout = nullptr;
  if (cudaMalloc(&ds, n * sizeof(float)) != cudaSuccess || cudaMalloc(&dt, n * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&dout, n * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(ds), cudaFree(dt), cudaFree(dout);
    return NEKGPU_ERR_NOMEM;
  }
  st = NEKGPU_OK;
  if (check_cuda(cudaMemcpy(ds, s, n * sizeof(float), cudaMemcpyHostToDevice)) ||
      check_cuda(cudaMemcpy(dt, t, n * sizeof(float), cudaMemcpyHostToDevice)))
    st = NEKGPU_ERR_CUDA;
  if (!st) st = pair_join_selftest(ds, dt, dout, n);
  if (!st && check_cuda(cudaMemcpy(out, dout, n * sizeof(double), cudaMemcpyDeviceToHost)))
    st = NEKGPU_ERR_CUDA;
  cudaFree(ds);
  cudaFree(dt);
  cudaFree(dout);
  return st;
}

int nekgpu_selftest_wait(nekgpu_ctx* c, int polls) {
  if (!c || polls < 1 || polls > (1 << 22)) return NEKGPU_ERR_ARG;
  c->last_launches = 0;
  if (check_cuda(cudaMemsetAsync(c->d_status, 0, sizeof(int), c->stream))) return NEKGPU_ERR_CUDA;
  int st = wait_selftest(c, polls);
  if (st) return st;
  st = sync_status(c);
  // the context stays usable: clear the word the wait set
  if (check_cuda(cudaMemset(c->d_status, 0, sizeof(int)))) return NEKGPU_ERR_CUDA;
  return st;
}

int nekgpu_check_blowup(nekgpu_ctx* c) {
  if (!c) return NEKGPU_ERR_ARG;
  int bad = 0;
  int st = util_blowup(c, &bad);
  if (st) return st;
  return bad ? NEKGPU_ERR_BLOWUP : NEKGPU_OK;
}

int nekgpu_time_steps(nekgpu_ctx* c, int nsteps, double* time, double dt, double* ms) {
  if (!c || !time || !ms || nsteps < 0) return NEKGPU_ERR_ARG;
  if (!c->have_state) return NEKGPU_ERR_STATE;
  c->last_launches = 0;
  if (c->form != NEKGPU_PLAIN) {
    // keep the one-off rescale out of the timed region
    int st = c->form == NEKGPU_MIXED && !c->curved ? scale_coef_pairs(c, dt) : scale_coef(c, dt);
    if (st) return st;
  }
  if (check_cuda(cudaEventRecord(c->ev0, c->stream))) return NEKGPU_ERR_CUDA;
  c->last_launches = 0;
  int st = do_steps(c, nsteps, time, dt);
  if (st) return st;
  if (check_cuda(cudaEventRecord(c->ev1, c->stream))) return NEKGPU_ERR_CUDA;
  if (check_cuda(cudaEventSynchronize(c->ev1))) return NEKGPU_ERR_CUDA;
  float f = 0;
  if (check_cuda(cudaEventElapsedTime(&f, c->ev0, c->ev1))) return NEKGPU_ERR_CUDA;
  *ms = f;
  return sync_status(c);
}

long nekgpu_last_launches(const nekgpu_ctx* c) { return c ? c->last_launches : -1; }

int nekgpu_sync(nekgpu_ctx* c) {
  if (!c) return NEKGPU_ERR_ARG;
  return sync_status(c);
}

}  // extern "C"
