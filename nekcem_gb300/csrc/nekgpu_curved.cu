// Fused FP64 stage on curvilinear hexahedra (NEKGPU_FUSED64 on a mesh whose
// metrics vary inside the elements): the general weighted curl with all nine
// per-node metrics (maxwell_wght_curl, src/cem_maxwell.F:1428-1497), the
// upwind flux with per-face-node normals and areas and the partner's values
// read directly (cem_maxwell_flux3d and gs_op_fields,
// src/cem_maxwell.F:922-1002, 1368-1426), the lift (:725-735), the volume
// source, the inverse mass and the low-storage RK update
// (src/cem_common.F:18-75), one kernel per stage.  With the dealiased curl
// (param(18) = -1, maxwell_wght_dcurl) its volume term comes from k_dcurl,
// launched before the stage kernel, which then adds flux, lift, source,
// inverse mass and RK update in one pass.
//
// One block of N3 threads per element at a time (thread per node); the
// element's six field components sit in shared memory for the derivative
// contractions, which take D from shared memory.  The metrics add 72 bytes
// per node and stage to the affine kernel's traffic; the face geometry
// 4 doubles and the partner index per face node.
#include <cuda_runtime.h>

#include "nekgpu_internal.h"

namespace nekgpu {

namespace {

template <int NX>
__device__ __forceinline__ int face_vol_c(int f, int a, int b) {
  // slot order s=-1, r=+1, s=+1, r=-1, t=-1, t=+1 (pff)
  switch (f) {
    case 0: return a + NX * NX * b;
    case 1: return NX - 1 + NX * a + NX * NX * b;
    case 2: return a + NX * (NX - 1) + NX * NX * b;
    case 3: return NX * a + NX * NX * b;
    case 4: return a + NX * b;
    default: return a + NX * b + NX * NX * (NX - 1);
  }
}

template <int NX>
__global__ void __launch_bounds__((NX * NX * NX + 31) / 32 * 32)
    k_curved_stage(const CurvedDev a) {
  constexpr int N2 = NX * NX, N3 = N2 * NX, NF = 6 * N2;
  constexpr int NT = (N3 + 31) / 32 * 32;
  __shared__ double s_u[6 * N3];
  __shared__ double s_D[N2];
  __shared__ double s_w3[N3];
  __shared__ double s_flux[6 * NF];
  const int tid = threadIdx.x;
  const long P = a.npts;
  const bool node = tid < N3;
  const int vi = tid % NX, vj = (tid / NX) % NX, vk = tid / N2;
  const bool first_stage = (a.a == 0.0);
  for (int t = tid; t < N2; t += NT) s_D[t] = a.D[t];
  for (int t = tid; t < N3; t += NT) s_w3[t] = a.w3[t];

  for (int e = blockIdx.x; e < a.nelt; e += gridDim.x) {
    __syncthreads();  // the previous element's shared data is consumed
    if (node) {
      const long g = (long)e * N3 + tid;
#pragma unroll
      for (int c = 0; c < 6; ++c) s_u[c * N3 + tid] = a.u_in[c * P + g];
    }
    __syncthreads();

    // ---- weighted curl with the general metrics ---------------------------
    // (or, with the dealiased curl, its volume term computed before)
    double res[6];
    if (node && a.vres) {
      const long g = (long)e * N3 + tid;
#pragma unroll
      for (int c = 0; c < 6; ++c) res[c] = a.vres[c * P + g];
    } else if (node) {
      double dr[6], ds[6], dt[6];
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const double* u = s_u + c * N3;
        double sr = s_D[vi] * u[NX * vj + N2 * vk];
        double ss = s_D[vj] * u[vi + N2 * vk];
        double st = s_D[vk] * u[vi + NX * vj];
#pragma unroll
        for (int l = 1; l < NX; ++l) {
          sr = fma(s_D[vi + NX * l], u[l + NX * vj + N2 * vk], sr);
          ss = fma(s_D[vj + NX * l], u[vi + NX * l + N2 * vk], ss);
          st = fma(s_D[vk + NX * l], u[vi + NX * vj + N2 * l], st);
        }
        const double w = s_w3[tid];
        dr[c] = sr * w;
        ds[c] = ss * w;
        dt[c] = st * w;
      }
      const long g = (long)e * N3 + tid;
      const double rx = a.metrics[g], ry = a.metrics[P + g], rz = a.metrics[2 * P + g];
      const double sx = a.metrics[3 * P + g], sy = a.metrics[4 * P + g], sz = a.metrics[5 * P + g];
      const double tx = a.metrics[6 * P + g], ty = a.metrics[7 * P + g], tz = a.metrics[8 * P + g];
      // w = curl(u1, u2, u3) with d/dx = rx d/dr + sx d/ds + tx d/dt, etc.
      auto curl = [&](int c1, int c2, int c3, double* w) {
        w[0] = (dr[c3] * ry + ds[c3] * sy + dt[c3] * ty) - (dr[c2] * rz + ds[c2] * sz + dt[c2] * tz);
        w[1] = (dr[c1] * rz + ds[c1] * sz + dt[c1] * tz) - (dr[c3] * rx + ds[c3] * sx + dt[c3] * tx);
        w[2] = (dr[c2] * rx + ds[c2] * sx + dt[c2] * tx) - (dr[c1] * ry + ds[c1] * sy + dt[c1] * ty);
      };
      double wE[3], wH[3];
      curl(0, 1, 2, wE);  // resE = W curl H
      curl(3, 4, 5, wH);  // resH = -W curl E
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        res[c] = -wH[c];
        res[3 + c] = wE[c];
      }
    }

    // ---- upwind flux per face node ----------------------------------------
    for (int t = tid; t < NF; t += NT) {
      const int f = t / N2, ab = t - f * N2;
      const int v = face_vol_c<NX>(f, ab % NX, ab / NX);
      const long js = (long)e * NF + t, L = a.nxzfl;
      const int pv = a.partner[js];
      double dH[3], dE[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const double hm = s_u[c * N3 + v], em = s_u[(c + 3) * N3 + v];
        if (pv >= 0) {
          dH[c] = a.u_in[c * P + pv] - hm;
          dE[c] = a.u_in[(c + 3) * P + pv] - em;
        } else {  // PEC mirror: H+ = H-, E+ = -E-
          dH[c] = 0.0;
          dE[c] = -2.0 * em;
        }
      }
      const double nx = a.face[js], ny = a.face[L + js], nz = a.face[2 * L + js];
      const double area = a.face[3 * L + js];
      double Y02 = -0.5, C02Y = 0.5, Z02 = 0.5, C02Z = 0.5;
      if (a.fcoef) {
        Y02 = a.fcoef[js]; C02Y = a.fcoef[L + js]; Z02 = a.fcoef[2 * L + js]; C02Z = a.fcoef[3 * L + js];
      }
      // n x [E], n x [H] (the gs sums of -n x E, -n x H), then the upwind terms
      const double nE[3] = {ny * dE[2] - nz * dE[1], nz * dE[0] - nx * dE[2], nx * dE[1] - ny * dE[0]};
      const double nH[3] = {ny * dH[2] - nz * dH[1], nz * dH[0] - nx * dH[2], nx * dH[1] - ny * dH[0]};
      const double fu[3] = {ny * nH[2] - nz * nH[1], nz * nH[0] - nx * nH[2], nx * nH[1] - ny * nH[0]};
      const double fw[3] = {ny * nE[2] - nz * nE[1], nz * nE[0] - nx * nE[2], nx * nE[1] - ny * nE[0]};
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        s_flux[c * NF + t] = area * (Y02 * nE[c] - C02Y * fu[c]);
        s_flux[(3 + c) * NF + t] = area * (Z02 * nH[c] - C02Z * fw[c]);
      }
    }
    __syncthreads();

    if (node) {
      // ---- lift in face-slot order ---------------------------------------
      auto add = [&](int f, int ab) {
#pragma unroll
        for (int c = 0; c < 6; ++c) res[c] += s_flux[c * NF + f * N2 + ab];
      };
      if (vj == 0) add(0, vi + NX * vk);
      if (vi == NX - 1) add(1, vj + NX * vk);
      if (vj == NX - 1) add(2, vi + NX * vk);
      if (vi == 0) add(3, vj + NX * vk);
      if (vk == 0) add(4, vi + NX * vj);
      if (vk == NX - 1) add(5, vi + NX * vj);
      // ---- volume source (usersrc), mass-weighted ------------------------
      if (a.src_elem) {
        const int so = a.src_elem[e];
        if (so >= 0) res[5] += a.src_w[(long)so * N3 + tid] * a.src_ft;
      }
      // ---- inverse mass + low-storage RK ---------------------------------
      const long g = (long)e * N3 + tid;
      const double ch = a.coef[g], ce = a.coef[P + g];
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const double r = res[c] * (c < 3 ? ch : ce);
        const double kn = first_stage ? r : fma(a.a, a.k[c * P + g], r);
        a.k[c * P + g] = kn;
        a.u_out[c * P + g] = fma(a.b, kn, s_u[c * N3 + tid]);
      }
    }
  }
}

template <int NX>
int launch_curved(Context* c, const CurvedDev& a) {
  constexpr int NT = (NX * NX * NX + 31) / 32 * 32;
  static int grid = 0;
  if (!grid) {
    int per_sm = 0, sms = 0;
    if (check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_curved_stage<NX>, NT, 0)))
      return NEKGPU_ERR_CUDA;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    if (per_sm < 1) return NEKGPU_ERR_UNSUPPORTED;
    grid = per_sm * sms;
  }
  const int g = c->nelt < grid ? c->nelt : grid;
  k_curved_stage<NX><<<g, NT, 0, c->stream>>>(a);
  c->last_launches += 1;
  return check_cuda(cudaGetLastError());
}

}  // namespace

int curved_stage(Context* c, int rkstep, double time, double dt) {
  int st = scale_coef(c, dt);
  if (st) return st;
  CurvedDev a = c->cargs;
  a.u_in = c->d_u[c->cur];
  a.u_out = c->d_u[c->cur ^ 1];
  a.a = c->rk_a[rkstep - 1];
  a.b = c->rk_b[rkstep - 1];
  a.src_elem = c->fargs.src_elem;
  a.src_w = reinterpret_cast<const double*>(c->fargs.src_w);
  if (c->src.enabled) a.src_ft = source_ft(c->src, time + dt * c->rk_c[rkstep - 1]);
  a.vres = nullptr;
  if (c->pargs.md > 0) {  // param(18) = -1: the dealiased curl of the stage's input
    if ((st = dcurl_into(c, a.u_in, c->d_vres))) return st;
    a.vres = c->d_vres;
  }
  switch (c->nx) {
    case 3: st = launch_curved<3>(c, a); break;
    case 4: st = launch_curved<4>(c, a); break;
    case 5: st = launch_curved<5>(c, a); break;
    case 6: st = launch_curved<6>(c, a); break;
    case 7: st = launch_curved<7>(c, a); break;
    case 8: st = launch_curved<8>(c, a); break;
    default: return NEKGPU_ERR_UNSUPPORTED;
  }
  if (st) return st;
  c->cur ^= 1;
  return NEKGPU_OK;
}

}  // namespace nekgpu
