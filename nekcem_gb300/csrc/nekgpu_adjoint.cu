// Discrete adjoint of the FP64 fused stage (nekgpu_fused.cu, T = double) with
// respect to the state and to the permittivity eps at every node.
//
// Forward stage i (src/cem_maxwell.F:484-508, src/cem_common.F:18-75):
//   r_i = M^-1(eps) (A(eps) u_{i-1} + s(t_i)),  k_i = a_i k_{i-1} + dt r_i,
//   u_i = u_{i-1} + b_i k_i,
// A = weighted curl (src/cem_maxwell.F:1428-1497) + upwind face flux with the
// partner face (src/cem_maxwell.F:922-1002) + lift; M^-1 = diag(hbm1, ebm1),
// ebm1 = 1/(eps bm1); the face impedance coefficients depend on eps at the
// node and at its partner (src/cem_maxwell.F:262-325).
//
// Reverse stage i carries (ub_i, w_i) with w_i = dt M^-1 (kb_i + b_i ub_i),
// kb_i the adjoint of k_i:
//   ub_{i-1} = ub_i + A^T w_i
//   w_{i-1}  = a_i w_i + b_{i-1} dt M^-1 ub_{i-1}      (kb_{i-1} = a_i kt_i)
//   deps    += -(bm1/dt) sum_E w_i,E (k_i - a_i k_{i-1})_E   (d ebm1/d eps)
//            + w_i^T (dA/deps) u_{i-1}                      (face impedances)
// A^T: the curl transposes to D^T contractions of w3 w; a face node's flux
// term L (u+ - u-) transposes to -L^T w at the node and +L^T w at its partner,
// and only the two tangential components of H and E enter (the normal one is
// projected out).  Every element gathers what lands on its own nodes, reading
// the partner elements' face nodes, so all writes are element-local: no
// atomics, and the adjoint state ping-pongs like the forward state.
// The D^T contractions and the face terms run in double-float FP32
// arithmetic (D w, the stage weights, the face-slot coefficients and the
// jumps as (hi, lo) float pairs, products with their FMA error terms,
// two-sum accumulation: ~2^-47 of the sum of the magnitudes, near FP64's
// 2^-53) and join the FP64 arithmetic as one FP64 value each; the updates of
// ub, w and deps are FP64.  The contractions and face terms were ~130 of the
// ~166 FP64 operations per node.
#include <cuda_runtime.h>

#include "nekgpu_internal.h"
#include "nekgpu_pair.cuh"

namespace nekgpu {

namespace {

__host__ __device__ constexpr int slot_axis(int f) { return f == 1 || f == 3 ? 0 : (f < 4 ? 1 : 2); }
__host__ __device__ constexpr int slot_side(int f) { return (f == 0 || f == 3 || f == 4) ? -1 : 1; }
__host__ __device__ constexpr int slot_opp(int f) { return f < 4 ? (f + 2) & 3 : 9 - f; }
// tangential axes in cyclic order: (e_a x x)_t1 = -x_t2, (e_a x x)_t2 = x_t1
__host__ __device__ constexpr int tan1(int a) { return a == 0 ? 1 : (a == 1 ? 2 : 0); }
__host__ __device__ constexpr int tan2(int a) { return a == 0 ? 2 : (a == 1 ? 0 : 1); }

// double-float values: (h, l) with h + l the value to ~2^-48
struct P2 {
  float h, l;
};
__device__ __forceinline__ P2 p2(double d) { return P2{d2f_hi(d), d2f_lo(d)}; }
__device__ __forceinline__ P2 p2(float2 v) { return P2{v.x, v.y}; }
__device__ __forceinline__ P2 pmul(P2 a, P2 b) {
  const float p = a.h * b.h;
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return P2{p, e};
}
__device__ __forceinline__ P2 padd(P2 a, P2 b) {
  float s, t;
  two_sum(a.h, b.h, s, t);
  return P2{s, (a.l + b.l) + t};
}
__device__ __forceinline__ P2 pneg(P2 a) { return P2{-a.h, -a.l}; }
__device__ __forceinline__ double pdbl(P2 a) {
  float s, t;
  two_sum(a.h, a.l, s, t);
  return pair_to_double(s, t);
}

template <int NX>
__device__ __forceinline__ int face_vol(int f, int a, int b) {
  const int fixed = slot_side(f) < 0 ? 0 : NX - 1;
  const int ax = slot_axis(f);
  return ax == 0 ? fixed + NX * a + NX * NX * b
                 : (ax == 1 ? a + NX * fixed + NX * NX * b : a + NX * b + NX * NX * fixed);
}

template <int NX>
struct ACfg {
  static constexpr int N2 = NX * NX, N3 = N2 * NX, NF = 6 * N2;
  static constexpr int NT = ((N3 + 31) / 32) * 32;
  static constexpr int FPT = (NF + NT - 1) / NT;
  // shared: face results (5*NF) in FP64; the stage weights w and D w as
  // float pairs (6*N3 + NX*NX)
  static constexpr size_t smem = 5 * NF * sizeof(double) + (6 * N3 + NX * NX) * sizeof(float2);
};

template <int NX>
__global__ void __launch_bounds__(ACfg<NX>::NT) k_adjoint_stage(const AdjointDev a) {
  using C = ACfg<NX>;
  constexpr int N2 = C::N2, N3 = C::N3, NT = C::NT, NF = C::NF, FPT = C::FPT;
  extern __shared__ double sm[];
  double* s_fu = sm;                // [4][NF]  tangential face contributions to ub
  double* s_fe = s_fu + 4 * NF;     // [NF]     face contributions to deps
  float2* s_wp = reinterpret_cast<float2*>(s_fe + NF);  // [6][N3] w as (hi, lo)
  float2* s_Dp = s_wp + 6 * N3;                          // D w as (hi, lo)
  const int tid = threadIdx.x;
  const long P = a.npts, PF = (long)a.nelt * NF;
  const bool node = tid < N3;
  const int vi = tid % NX, vj = (tid / NX) % NX, vk = tid / N2;
  for (int t = tid; t < NX * NX; t += NT) {
    s_Dp[t] = make_float2(d2f_hi(a.Dw[t]), d2f_lo(a.Dw[t]));
  }
  const double wi = a.w[vi], wj = a.w[vj], wk = a.w[vk];

  for (int e = blockIdx.x; e < a.nelt; e += gridDim.x) {
    const long g = (long)e * N3 + tid;
    double ub[6], wn[6], mass = 0.0;
    __syncthreads();  // s_wp / s_fu of the previous element are consumed
    if (node) {
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        ub[c] = a.ub_in[c * P + g];
        wn[c] = a.w_in[c * P + g];
        s_wp[c * N3 + tid] = make_float2(d2f_hi(wn[c]), d2f_lo(wn[c]));
      }
#pragma unroll
      for (int c = 3; c < 6; ++c) {
        const double r = a.a == 0.0 ? a.k_cur[c * P + g]
                                    : fma(-a.a, a.k_prev[c * P + g], a.k_cur[c * P + g]);
        mass = fma(wn[c], r, mass);
      }
      mass *= -a.bm1[g] * a.inv_dt;
    }
    __syncthreads();
    // ---- face slots: transposed flux and impedance derivatives --------------
#pragma unroll
    for (int q = 0; q < FPT; ++q) {
      const int t = tid + q * NT;
      if (t >= NF) continue;
      const int f = t / N2, ab = t - f * N2, fa = ab % NX, fb = ab / NX;
      const int ax = slot_axis(f), t1 = tan1(ax), t2 = tan2(ax);
      const int vl = face_vol<NX>(f, fa, fb);
      const long gn = (long)e * N3 + vl;
      const long j = (long)e * NF + t;
      // the slot's coefficients, the stage weights and the jumps as float
      // pairs; sums of products in double-float arithmetic (as the D^T
      // contractions), each result joined into one FP64 value
      const float2* kslot = reinterpret_cast<const float2*>(a.slot);
      P2 k[16];
#pragma unroll
      for (int m = 0; m < 16; ++m) {
        const float2 kv = kslot[m * PF + j];
        k[m] = P2{kv.x, kv.y};
      }
      // own stage weights (tangential) from shared memory
      const P2 nH1 = p2(s_wp[t1 * N3 + vl]), nH2 = p2(s_wp[t2 * N3 + vl]);
      const P2 nE1 = p2(s_wp[(3 + t1) * N3 + vl]), nE2 = p2(s_wp[(3 + t2) * N3 + vl]);
      P2 pH1{0.0f, 0.0f}, pH2{0.0f, 0.0f}, pE1{0.0f, 0.0f}, pE2{0.0f, 0.0f};
      // jump u+ - u- of u_{i-1} (PEC: u-, the -2 of the mirror is in the coefficients)
      const double oH1 = a.u_prev[t1 * P + gn], oH2 = a.u_prev[t2 * P + gn];
      const double oE1 = a.u_prev[(3 + t1) * P + gn], oE2 = a.u_prev[(3 + t2) * P + gn];
      P2 dH1 = p2(oH1), dH2 = p2(oH2), dE1 = p2(oE1), dE2 = p2(oE2);
      const int pe = a.nbr[6 * e + f];
      if (pe >= 0) {
        const long gp = (long)pe * N3 + face_vol<NX>(slot_opp(f), fa, fb);
        pH1 = p2(a.w_in[t1 * P + gp]);
        pH2 = p2(a.w_in[t2 * P + gp]);
        pE1 = p2(a.w_in[(3 + t1) * P + gp]);
        pE2 = p2(a.w_in[(3 + t2) * P + gp]);
        dH1 = padd(p2(a.u_prev[t1 * P + gp]), pneg(dH1));
        dH2 = padd(p2(a.u_prev[t2 * P + gp]), pneg(dH2));
        dE1 = padd(p2(a.u_prev[(3 + t1) * P + gp]), pneg(dE1));
        dE2 = padd(p2(a.u_prev[(3 + t2) * P + gp]), pneg(dE2));
      }
      // k: 0 kH 1 kHx 2 kE 3 kEx | 4 pH 5 pHx 6 pE 7 pEx | 8..11 gA..gD | 12..15 hA..hD
      s_fu[0 * NF + t] = pdbl(padd(padd(pmul(k[0], nH1), pneg(pmul(k[1], nE2))),
                                   padd(pmul(k[4], pH1), pneg(pmul(k[5], pE2)))));
      s_fu[1 * NF + t] = pdbl(padd(padd(pmul(k[0], nH2), pmul(k[1], nE1)),
                                   padd(pmul(k[4], pH2), pmul(k[5], pE1))));
      s_fu[2 * NF + t] = pdbl(padd(padd(pneg(pmul(k[3], nH2)), pmul(k[2], nE1)),
                                   padd(pneg(pmul(k[7], pH2)), pmul(k[6], pE1))));
      s_fu[3 * NF + t] = pdbl(padd(padd(pmul(k[3], nH1), pmul(k[2], nE2)),
                                   padd(pmul(k[7], pH1), pmul(k[6], pE2))));
      // fe = A.PdH + B.(e_a x dE) + C.(e_a x dH) + D.PdE with A = gA wH(n) + hA wH(p) ...
      const P2 A1 = padd(pmul(k[8], nH1), pmul(k[12], pH1)), A2 = padd(pmul(k[8], nH2), pmul(k[12], pH2));
      const P2 B1 = padd(pmul(k[9], nH1), pmul(k[13], pH1)), B2 = padd(pmul(k[9], nH2), pmul(k[13], pH2));
      const P2 C1 = padd(pmul(k[10], nE1), pmul(k[14], pE1)), C2 = padd(pmul(k[10], nE2), pmul(k[14], pE2));
      const P2 D1 = padd(pmul(k[11], nE1), pmul(k[15], pE1)), D2 = padd(pmul(k[11], nE2), pmul(k[15], pE2));
      P2 fe = pmul(A1, dH1);
      fe = padd(fe, pmul(A2, dH2));
      fe = padd(fe, pneg(pmul(B1, dE2)));
      fe = padd(fe, pmul(B2, dE1));
      fe = padd(fe, pneg(pmul(C1, dH2)));
      fe = padd(fe, pmul(C2, dH1));
      fe = padd(fe, pmul(D1, dE1));
      fe = padd(fe, pmul(D2, dE2));
      s_fe[t] = pdbl(fe);
    }
    __syncthreads();
    if (!node) continue;
    // ---- transposed weighted curl: D^T contractions of w3 w ------------------
    const double* eg = a.egeom + 9 * e;
    const double Rr = eg[0] * wj * wk, Ss = eg[1] * wi * wk, Tt = eg[2] * wi * wj;
    // sum_m D(m,row) w_m z_m over one line of the stage weights, double-float
    auto dot = [&](const float2* z, int zs, int row) -> double {
      float S = 0.0f, E = 0.0f;
#pragma unroll
      for (int m = 0; m < NX; ++m) {
        const float2 d = s_Dp[m + NX * row];
        const float2 x = z[zs * m];
        const float p = d.x * x.x;
        float e = fmaf(d.x, x.x, -p);
        e = fmaf(d.x, x.y, e);
        e = fmaf(d.y, x.x, e);
        float s, t;
        two_sum(S, p, s, t);
        S = s;
        E += e + t;
      }
      float s, t;
      two_sum(S, E, s, t);
      return pair_to_double(s, t);
    };
    auto dtr = [&](int c) { return dot(s_wp + c * N3 + NX * vj + N2 * vk, 1, vi); };
    auto dts = [&](int c) { return dot(s_wp + c * N3 + vi + N2 * vk, NX, vj); };
    auto dtt = [&](int c) { return dot(s_wp + c * N3 + vi + NX * vj, N2, vk); };
    double out[6];
    out[0] = fma(Tt, dtt(4), fma(-Ss, dts(5), ub[0]));
    out[1] = fma(Rr, dtr(5), fma(-Tt, dtt(3), ub[1]));
    out[2] = fma(Ss, dts(3), fma(-Rr, dtr(4), ub[2]));
    out[3] = fma(Ss, dts(2), fma(-Tt, dtt(1), ub[3]));
    out[4] = fma(Tt, dtt(0), fma(-Rr, dtr(2), ub[4]));
    out[5] = fma(Rr, dtr(1), fma(-Ss, dts(0), ub[5]));
    // ---- face contributions, in face-slot order ------------------------------
    double fe = 0.0;
    auto add = [&](int f, int ab) {
      const int t = f * N2 + ab, ax = slot_axis(f);
      out[tan1(ax)] += s_fu[0 * NF + t];
      out[tan2(ax)] += s_fu[1 * NF + t];
      out[3 + tan1(ax)] += s_fu[2 * NF + t];
      out[3 + tan2(ax)] += s_fu[3 * NF + t];
      fe += s_fe[t];
    };
    if (vj == 0) add(0, vi + NX * vk);
    if (vi == NX - 1) add(1, vj + NX * vk);
    if (vj == NX - 1) add(2, vi + NX * vk);
    if (vi == 0) add(3, vj + NX * vk);
    if (vk == 0) add(4, vi + NX * vj);
    if (vk == NX - 1) add(5, vi + NX * vj);
    const double cH = a.b_next * a.coef[g], cE = a.b_next * a.coef[P + g];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      a.ub_out[c * P + g] = out[c];
      a.w_out[c * P + g] = fma(a.a, wn[c], (c < 3 ? cH : cE) * out[c]);
    }
    a.deps[g] += mass + fe;
  }
}

__global__ void k_adjoint_seed(double* w, const double* ub, const double* coef, long P, double b) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= 6 * P) return;
  const long g = i % P;
  w[i] = b * coef[(i < 3 * P ? 0 : P) + g] * ub[i];
}

// dt hbm1 | dt ebm1: the same product the fused FP64 form's coefficient
// scaling forms from its unnormalised base
__global__ void k_adjoint_coef64(double* coef, const double* hbm1, const double* ebm1, long P,
                                 double dt) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= 2 * P) return;
  coef[i] = dt * (i < P ? hbm1[i] : ebm1[i - P]);
}

template <int NX>
int launch_adjoint(Context* c, const AdjointDev& a) {
  using C = ACfg<NX>;
  auto kern = k_adjoint_stage<NX>;
  static bool ready = false;
  static int grid = 0;
  if (!ready) {
    if (check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)C::smem)))
      return NEKGPU_ERR_CUDA;
    int per_sm = 0, sms = 0;
    if (check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, C::NT, C::smem)))
      return NEKGPU_ERR_CUDA;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    if (per_sm < 1) return NEKGPU_ERR_UNSUPPORTED;
    grid = per_sm * sms;
    ready = true;
  }
  const int g = c->nelt < grid ? c->nelt : grid;
  kern<<<g, C::NT, C::smem, c->stream>>>(a);
  c->last_launches += 1;
  return check_cuda(cudaGetLastError());
}

}  // namespace

int adjoint_stage(Context* c, const AdjointDev& a) {
  switch (c->nx) {
    case 3: return launch_adjoint<3>(c, a);
    case 4: return launch_adjoint<4>(c, a);
    case 5: return launch_adjoint<5>(c, a);
    case 6: return launch_adjoint<6>(c, a);
    case 7: return launch_adjoint<7>(c, a);
    case 8: return launch_adjoint<8>(c, a);
    case 9: return launch_adjoint<9>(c, a);
    default: return NEKGPU_ERR_UNSUPPORTED;
  }
}

int adjoint_seed(Context* c, double* w, const double* ub, const double* coef, double b) {
  const long n = 6 * c->npts;
  k_adjoint_seed<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(w, ub, coef, c->npts, b);
  c->last_launches += 1;
  return check_cuda(cudaGetLastError());
}

int adjoint_coef64(Context* c, double* coef, double dt) {
  const long n = c->npts;
  k_adjoint_coef64<<<(unsigned)((2 * n + 255) / 256), 256, 0, c->stream>>>(coef, c->d_hbm1,
                                                                           c->d_ebm1, n, dt);
  c->last_launches += 1;
  return check_cuda(cudaGetLastError());
}

}  // namespace nekgpu
