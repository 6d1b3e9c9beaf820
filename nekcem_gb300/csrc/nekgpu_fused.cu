// Fused Maxwell DG stage kernel for sm_103a.
//
// One CTA works on one element at a time (persistent over elements).  The
// element's FP64 state u (6 components), RK register k (6) and the two
// dt-scaled inverse-mass coefficients arrive in shared memory by 1-D TMA bulk
// copies (cp.async.bulk + mbarrier) while the threads fetch the partner
// elements' face nodes.  Then, per node: the r/s/t contractions of the GLL
// derivative matrix (src/nek5_grad.F:2-19) combined with the per-element
// affine metrics into the weighted curl (src/cem_maxwell.F:1428-1497); per
// face node: the upwind flux (src/cem_maxwell.F:922-1002, 1368-1426) from the
// in-kernel partner read that replaces gs_op_fields; the lift
// (src/cem_maxwell.F:725-735) in face-slot order; the volume source; the
// inverse mass (src/cem_maxwell.F:1878-1886) and the low-storage RK update
// (src/cem_common.F:18-75).  u is read from one buffer and written to the
// other so neighbours always see pre-stage values; k is element-local and
// updated in place.
//
// T = float: the MIXED form (contractions, curl and flux in FP32; state, k,
// inverse mass and the RK update in FP64).  On GB300 every FP64-pipe
// instruction (including F2F conversions) runs at ~0.5 T/s, so FP64<->FP32
// conversions here are done with integer bit operations and the only FP64
// arithmetic left is 3 instructions per component per stage.
// T = double: the FUSED64 form (everything FP64).
#include <cuda_runtime.h>
#include <stdint.h>

#include "nekgpu_internal.h"

namespace nekgpu {

namespace {

// ---------------------------------------------------------------------------
// FP64 <-> FP32 conversion with integer instructions only.
// d2f: rounds to nearest (ties away from zero); |d| < 2^-126 gives a signed
// zero; finite |d| >= 2^128 is not expected (the blow-up check stops a run
// long before).  f2d: exact for normal floats, zero for zero/subnormal.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float d2f_bits(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  unsigned m = __funnelshift_l(lo, hi, 3) - 0xC0000000u;  // rebias exponent 1023 -> 127
  m = ((m & 0x7FFFFFFFu) + ((lo >> 28) & 1u)) | (hi & 0x80000000u);  // round bit 28
  return __uint_as_float((hi & 0x7FF00000u) >= 0x38100000u ? m : (hi & 0x80000000u));
}

__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned mag = b & 0x7FFFFFFFu;
  unsigned hi = (b & 0x80000000u) | ((mag >> 3) + 0x38000000u);
  unsigned lo = b << 29;
  const bool tiny = (b & 0x7F800000u) == 0u;
  hi = tiny ? (b & 0x80000000u) : hi;
  lo = tiny ? 0u : lo;
  return __longlong_as_double((long long)(((unsigned long long)hi << 32) | lo));
}

template <typename T>
__device__ __forceinline__ T from_f64(double d);
template <>
__device__ __forceinline__ float from_f64<float>(double d) { return d2f_bits(d); }
template <>
__device__ __forceinline__ double from_f64<double>(double d) { return d; }

__device__ __forceinline__ double to_f64(float f) { return f2d_bits(f); }
__device__ __forceinline__ double to_f64(double d) { return d; }

// ---------------------------------------------------------------------------
// mbarrier + 1-D TMA bulk copy (PTX)
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// orders the block's generic-proxy shared-memory accesses (after a barrier)
// before later async-proxy (TMA) accesses
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, unsigned bytes,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: gives up after ~2^22 polls (far beyond any copy time), records
// the failure in *status and reports it so the CTA can leave in step.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, int* status) {
  for (int it = 0; it < (1 << 22); ++it)
    if (mbar_try_wait(bar, parity)) return true;
  atomicExch(status, 1);
  return false;
}

// face slot f (reference order) -> reference axis 0=r,1=s,2=t and side
__host__ __device__ constexpr int slot_axis(int f) { return f == 1 || f == 3 ? 0 : (f < 4 ? 1 : 2); }
__host__ __device__ constexpr int slot_side(int f) { return (f == 0 || f == 3 || f == 4) ? -1 : 1; }
__host__ __device__ constexpr int slot_opp(int f) { return f < 4 ? (f + 2) & 3 : 9 - f; }

template <int NX>
__device__ __forceinline__ int face_vol(int f, int a, int b) {
  const int fixed = slot_side(f) < 0 ? 0 : NX - 1;
  const int ax = slot_axis(f);
  return ax == 0 ? fixed + NX * a + NX * NX * b
                 : (ax == 1 ? a + NX * fixed + NX * NX * b : a + NX * b + NX * NX * fixed);
}

// launch parameters in the compute type (FP32 copies for the mixed form)
template <typename T>
struct Par;
template <>
struct Par<float> {
  static __device__ __forceinline__ float D(const FusedDev& a, int i) { return a.Df[i]; }
  static __device__ __forceinline__ float w(const FusedDev& a, int i) { return a.wf[i]; }
  static __device__ __forceinline__ const float* geom(const FusedDev& a) { return a.egeomf; }
  static __device__ __forceinline__ float C0(const FusedDev& a) { return a.C0f; }
  static __device__ __forceinline__ float ft(const FusedDev& a) { return a.src_ftf; }
};
template <>
struct Par<double> {
  static __device__ __forceinline__ double D(const FusedDev& a, int i) { return a.D[i]; }
  static __device__ __forceinline__ double w(const FusedDev& a, int i) { return a.w[i]; }
  static __device__ __forceinline__ const double* geom(const FusedDev& a) { return a.egeom; }
  static __device__ __forceinline__ double C0(const FusedDev& a) { return a.C0; }
  static __device__ __forceinline__ double ft(const FusedDev& a) { return a.src_ft; }
};

template <int NX, typename T>
struct Cfg {
  static constexpr int N2 = NX * NX, N3 = NX * NX * NX;
  static constexpr int NT = ((N3 + 31) / 32) * 32;
  static constexpr int NF = 6 * N2;               // face nodes per element
  static constexpr int FPT = (NF + NT - 1) / NT;  // face tasks per thread
  static constexpr bool kTma = (N3 % 2) == 0;     // 16-byte aligned element blocks
  static constexpr bool kMixed = sizeof(T) == 4;
  // shared memory layout (bytes)
  static constexpr size_t off_u64 = 0;
  static constexpr size_t off_k = off_u64 + 6 * N3 * 8;
  static constexpr size_t off_coef = off_k + 6 * N3 * 8;
  static constexpr size_t off_uT = off_coef + 2 * N3 * 8;
  static constexpr size_t uT_bytes = kMixed ? 6 * N3 * sizeof(T) : 0;  // FP64 form reads u64
  static constexpr size_t off_nb = (off_uT + uT_bytes + 15) / 16 * 16;
  static constexpr size_t off_flux = off_nb + 6 * NF * sizeof(T);
  static constexpr size_t off_bar = (off_flux + 6 * NF * sizeof(T) + 15) / 16 * 16;
  static constexpr size_t smem = off_bar + 16;
  static constexpr int kMinBlocks = kMixed ? (NT <= 256 ? 4 : (NT <= 512 ? 2 : 1)) : 1;
};

template <int NX, typename T, bool EXT>
__global__ void __launch_bounds__(Cfg<NX, T>::NT, Cfg<NX, T>::kMinBlocks)
    k_fused_stage(const FusedDev a) {
  using C = Cfg<NX, T>;
  constexpr int N2 = C::N2, N3 = C::N3, NT = C::NT, NF = C::NF, FPT = C::FPT;
  extern __shared__ __align__(16) unsigned char smem[];
  double* s_u64 = reinterpret_cast<double*>(smem + C::off_u64);
  double* s_k = reinterpret_cast<double*>(smem + C::off_k);
  double* s_coef = reinterpret_cast<double*>(smem + C::off_coef);
  const T* s_uT = C::kMixed ? reinterpret_cast<const T*>(smem + C::off_uT)
                            : reinterpret_cast<const T*>(smem + C::off_u64);
  T* s_uTw = reinterpret_cast<T*>(smem + C::off_uT);
  T* s_nb = reinterpret_cast<T*>(smem + C::off_nb);      // [c][NF]
  T* s_flux = reinterpret_cast<T*>(smem + C::off_flux);  // [c][NF]
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + C::off_bar);
  __shared__ int s_abort;

  const int tid = threadIdx.x;
  const long P = a.npts;
  const bool node = tid < N3;
  const int vi = tid % NX, vj = (tid / NX) % NX, vk = tid / N2;

  // derivative-matrix rows of this node: D(i,l), D(j,l), D(k,l)
  T Dr[NX], Ds[NX], Dt[NX];
#pragma unroll
  for (int l = 0; l < NX; ++l) {
    Dr[l] = Par<T>::D(a, vi + NX * l);
    Ds[l] = Par<T>::D(a, vj + NX * l);
    Dt[l] = Par<T>::D(a, vk + NX * l);
  }
  const T w3 = node ? Par<T>::w(a, vi) * Par<T>::w(a, vj) * Par<T>::w(a, vk) : T(0);
  const bool first_stage = (a.a == 0.0);  // rk4a(1) = 0: k restarts
  const T C0 = Par<T>::C0(a);

  if (tid == 0) {
    s_abort = 0;
    if (C::kTma) {
      mbar_init(bar, 1);
      fence_mbar_init();
    }
  }
  __syncthreads();

  auto issue_tma = [&](int e) {
    const unsigned bytes = N3 * 8;
    mbar_expect_tx(bar, 14u * bytes);
    for (int c = 0; c < 6; ++c) tma_load_1d(s_u64 + c * N3, a.u_in + c * P + (long)e * N3, bytes, bar);
    for (int c = 0; c < 6; ++c) tma_load_1d(s_k + c * N3, a.k + c * P + (long)e * N3, bytes, bar);
    for (int c = 0; c < 2; ++c)
      tma_load_1d(s_coef + c * N3, a.coef + c * P + (long)e * N3, bytes, bar);
  };

  unsigned parity = 0;
  if (C::kTma && tid == 0 && blockIdx.x < a.nelt) issue_tma(blockIdx.x);

  for (int e = blockIdx.x; e < a.nelt; e += gridDim.x) {
    // ---- partner face nodes (pre-stage values of the neighbours) ----------
    double nbv[FPT][6];
    const int* nbr = a.nbr + 6 * e;
#pragma unroll
    for (int q = 0; q < FPT; ++q) {
      const int t = tid + q * NT;
      if (t < NF) {
        const int f = t / N2, ab = t - f * N2;
        const int pe = nbr[f];
        if (pe >= 0) {
          const long pv = (long)pe * N3 + face_vol<NX>(slot_opp(f), ab % NX, ab / NX);
#pragma unroll
          for (int c = 0; c < 6; ++c) nbv[q][c] = __ldg(a.u_in + c * P + pv);
        }
      }
    }
    // ---- own element: staged in shared memory -----------------------------
    if (C::kTma) {
      const bool ok = mbar_wait_bounded(bar, parity, a.status);
      if (!ok) s_abort = 1;
      parity ^= 1u;
    } else if (node) {
      const long g = (long)e * N3 + tid;
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        s_u64[c * N3 + tid] = a.u_in[c * P + g];
        s_k[c * N3 + tid] = a.k[c * P + g];
      }
      s_coef[tid] = a.coef[g];
      s_coef[N3 + tid] = a.coef[P + g];
    }
    __syncthreads();
    if (s_abort) return;
    if (C::kMixed && node) {
#pragma unroll
      for (int c = 0; c < 6; ++c) s_uTw[c * N3 + tid] = from_f64<T>(s_u64[c * N3 + tid]);
    }
#pragma unroll
    for (int q = 0; q < FPT; ++q) {
      const int t = tid + q * NT;
      if (t < NF && nbr[t / N2] >= 0) {
#pragma unroll
        for (int c = 0; c < 6; ++c) s_nb[c * NF + t] = from_f64<T>(nbv[q][c]);
      }
    }
    __syncthreads();

    // ---- weighted curl: resE = W curl H, resH = -W curl E ------------------
    const T* eg = Par<T>::geom(a) + 9 * e;
    const T rx = eg[0], sy = eg[1], tz = eg[2];
    T res[6];
    if (node) {
      auto dr = [&](int c) {
        const T* u = s_uT + c * N3 + NX * vj + N2 * vk;
        T s = Dr[0] * u[0];
#pragma unroll
        for (int l = 1; l < NX; ++l) s = fma(Dr[l], u[l], s);
        return s;
      };
      auto ds = [&](int c) {
        const T* u = s_uT + c * N3 + vi + N2 * vk;
        T s = Ds[0] * u[0];
#pragma unroll
        for (int l = 1; l < NX; ++l) s = fma(Ds[l], u[NX * l], s);
        return s;
      };
      auto dt = [&](int c) {
        const T* u = s_uT + c * N3 + vi + NX * vj;
        T s = Dt[0] * u[0];
#pragma unroll
        for (int l = 1; l < NX; ++l) s = fma(Dt[l], u[N2 * l], s);
        return s;
      };
      const T cx = rx * w3, cy = sy * w3, cz = tz * w3;
      // H = comps 0..2, E = comps 3..5
      const T Hx_s = ds(0), Hx_t = dt(0), Hy_r = dr(1), Hy_t = dt(1), Hz_r = dr(2), Hz_s = ds(2);
      res[3] = fma(cy, Hz_s, -cz * Hy_t);
      res[4] = fma(cz, Hx_t, -cx * Hz_r);
      res[5] = fma(cx, Hy_r, -cy * Hx_s);
      const T Ex_s = ds(3), Ex_t = dt(3), Ey_r = dr(4), Ey_t = dt(4), Ez_r = dr(5), Ez_s = ds(5);
      res[0] = fma(cz, Ey_t, -cy * Ez_s);
      res[1] = fma(cx, Ez_r, -cz * Ex_t);
      res[2] = fma(cy, Ex_s, -cx * Ey_r);
    }

    // ---- upwind face flux, area-weighted, into s_flux ----------------------
#pragma unroll
    for (int q = 0; q < FPT; ++q) {
      const int t = tid + q * NT;
      if (t < NF) {
        const int f = t / N2, ab = t - f * N2;
        const int fa = ab % NX, fb = ab / NX;
        const int v = face_vol<NX>(f, fa, fb);
        const int pe = nbr[f];
        T dH[3], dE[3], hmv[3], emv[3], hpv[3], epv[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          T hm = s_uT[c * N3 + v], em = s_uT[(c + 3) * N3 + v];
          T hp = pe >= 0 ? s_nb[c * NF + t] : T(0), ep = pe >= 0 ? s_nb[(c + 3) * NF + t] : T(0);
          if (EXT && !C::kMixed && a.inc_elem) {
            // userinc: the incident field on the own side of a listed face
            // node, or on the partner's side when the partner's slot is listed
            const int io = a.inc_elem[e];
            if (io >= 0) {
              const double* iv = a.inc_val + (long)io * 12 * NF + t;
              hm += (T)iv[c * NF];
              em += (T)iv[(3 + c) * NF];
              hp += (T)iv[(6 + c) * NF];
              ep += (T)iv[(9 + c) * NF];
            }
          }
          hmv[c] = hm; emv[c] = em; hpv[c] = hp; epv[c] = ep;
          if (pe >= 0) {
            dH[c] = hp - hm;
            dE[c] = ep - em;
          } else {  // PEC mirror: H+ = H-, E+ = -E-
            dH[c] = T(0);
            dE[c] = T(-2) * em;
          }
        }
        if (EXT && !C::kMixed && a.gr.elem) {
          // graphene (userfsrc): the sheet's currents on both sides of the
          // face node enter as n x [H] - J, i.e. [H] + n x J
          const int gr = a.gr.elem[e];
          const int go = gr >= 0 ? a.gr.own[(long)gr * NF + t] : -1;
          const int gp = gr >= 0 ? a.gr.part[(long)gr * NF + t] : -1;
          if (go >= 0 || gp >= 0) {
            double nv[3] = {0.0, 0.0, 0.0}, nm[3];
            nv[slot_axis(f)] = (double)slot_side(f);
            for (int c = 0; c < 3; ++c) nm[c] = -nv[c];
            const double fhm[3] = {(double)hmv[0], (double)hmv[1], (double)hmv[2]};
            const double fem[3] = {(double)emv[0], (double)emv[1], (double)emv[2]};
            const double fhp[3] = {(double)hpv[0], (double)hpv[1], (double)hpv[2]};
            const double fep[3] = {(double)epv[0], (double)epv[1], (double)epv[2]};
            double J[3] = {0.0, 0.0, 0.0};
            if (go >= 0) graphene_slot(a.gr, go, nv, fhm, fem, true, first_stage, a.a, a.b, a.dt, J);
            if (gp >= 0 && pe >= 0) graphene_slot(a.gr, gp, nm, fhp, fep, false, first_stage, a.a, a.b, a.dt, J);
            if (pe >= 0) {  // a PEC face keeps its mirror flux
              dH[0] += (T)(nv[1] * J[2] - nv[2] * J[1]);
              dH[1] += (T)(nv[2] * J[0] - nv[0] * J[2]);
              dH[2] += (T)(nv[0] * J[1] - nv[1] * J[0]);
            }
          }
        }
        T Y02 = T(-0.5), C02Y = T(0.5) * C0, Z02 = T(0.5), C02Z = T(0.5) * C0;
        if (a.fcoef) {
          const T* fc = reinterpret_cast<const T*>(a.fcoef) + 4 * ((long)e * NF + t);
          Y02 = fc[0]; C02Y = fc[1]; Z02 = fc[2]; C02Z = fc[3];
        }
        const T sg = (T)slot_side(f);
        const T area = eg[3 + f] * Par<T>::w(a, fa) * Par<T>::w(a, fb);
        const T sY = sg * Y02, sZ = sg * Z02;
        T fH[3], fE[3];
        switch (slot_axis(f)) {
          case 0:  // normal +-x
            fH[0] = T(0);
            fH[1] = fma(-sY, dE[2], C02Y * dH[1]);
            fH[2] = fma(sY, dE[1], C02Y * dH[2]);
            fE[0] = T(0);
            fE[1] = fma(-sZ, dH[2], C02Z * dE[1]);
            fE[2] = fma(sZ, dH[1], C02Z * dE[2]);
            break;
          case 1:  // normal +-y
            fH[0] = fma(sY, dE[2], C02Y * dH[0]);
            fH[1] = T(0);
            fH[2] = fma(-sY, dE[0], C02Y * dH[2]);
            fE[0] = fma(sZ, dH[2], C02Z * dE[0]);
            fE[1] = T(0);
            fE[2] = fma(-sZ, dH[0], C02Z * dE[2]);
            break;
          default:  // normal +-z
            fH[0] = fma(-sY, dE[1], C02Y * dH[0]);
            fH[1] = fma(sY, dE[0], C02Y * dH[1]);
            fH[2] = T(0);
            fE[0] = fma(-sZ, dH[1], C02Z * dE[0]);
            fE[1] = fma(sZ, dH[0], C02Z * dE[1]);
            fE[2] = T(0);
            break;
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          s_flux[c * NF + t] = area * fH[c];
          s_flux[(c + 3) * NF + t] = area * fE[c];
        }
      }
    }
    __syncthreads();

    if (node) {
      // ---- lift in face-slot order (src/cem_maxwell.F:725-735) -------------
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
      // ---- PML (pml_step, src/cem_maxwell_pml.F:508-590), FP64 form only:
      // auxiliary residuals from the residual so far, their RK update
      // (src/cem_maxwell.F:1942-1955), and their contribution to res
      if (EXT && !C::kMixed && a.pml.slot) {
        const int l = a.pml.slot[e];
        if (l >= 0) {
          const long nn = a.pml.n, q = (long)l * N3 + tid;
          const double* pd = a.pml.data;
          const double sxp = pd[q], syp = pd[nn + q], szp = pd[2 * nn + q];
          const double sigx = pd[3 * nn + q], sigy = pd[4 * nn + q], sigz = pd[5 * nn + q];
          const double mu = pd[6 * nn + q], bm1 = pd[7 * nn + q], bm1inv = pd[8 * nn + q];
          double* aux = a.pml.aux;
          double* kx = a.pml.k;
          const double bn[3] = {aux[q], aux[nn + q], aux[2 * nn + q]};
          const double dn[3] = {aux[3 * nn + q], aux[4 * nn + q], aux[5 * nn + q]};
          const double* hn = s_u64;
          const double* en = s_u64 + 3 * N3;
          double rp[6];
          rp[0] = (double)res[0] * bm1inv - syp * bn[0];
          rp[1] = (double)res[1] * bm1inv - szp * bn[1];
          rp[2] = (double)res[2] * bm1inv - sxp * bn[2];
          rp[3] = (double)res[3] * bm1inv - syp * dn[0];
          rp[4] = (double)res[4] * bm1inv - szp * dn[1];
          rp[5] = (double)res[5] * bm1inv - sxp * dn[2];
          const double rh0 = -syp * bn[0] + sxp * bn[0] - szp * mu * hn[tid];
          const double rh1 = -szp * bn[1] + syp * bn[1] - sxp * mu * hn[N3 + tid];
          const double rh2 = -sxp * bn[2] + szp * bn[2] - syp * mu * hn[2 * N3 + tid];
          const double re0 = -syp * dn[0] + sxp * dn[0] - sigz * en[tid];
          const double re1 = -szp * dn[1] + syp * dn[1] - sigx * en[N3 + tid];
          const double re2 = -sxp * dn[2] + szp * dn[2] - sigy * en[2 * N3 + tid];
          res[0] = (T)((double)res[0] + rh0 * bm1);
          res[1] = (T)((double)res[1] + rh1 * bm1);
          res[2] = (T)((double)res[2] + rh2 * bm1);
          res[3] = (T)((double)res[3] + re0 * bm1);
          res[4] = (T)((double)res[4] + re1 * bm1);
          res[5] = (T)((double)res[5] + re2 * bm1);
#pragma unroll
          for (int cc = 0; cc < 6; ++cc) {
            const double kv = first_stage ? a.dt * rp[cc] : fma(a.a, kx[cc * nn + q], a.dt * rp[cc]);
            kx[cc * nn + q] = kv;
            aux[cc * nn + q] = fma(a.b, kv, cc < 3 ? bn[cc] : dn[cc - 3]);
          }
        }
      }
      // ---- dispersive currents inside usersrc (cem_maxwell_drude /
      // cem_maxwell_lorentz, src/cem_maxwell.F:3095-3212), FP64 form only:
      // resE -= J1 bm1, the currents' residuals and their RK update
      if (EXT && !C::kMixed && a.disp.slot) {
        const int l = a.disp.slot[e];
        if (l >= 0) {
          const DispDev& d = a.disp;
          const long nn = d.n, q = (long)l * N3 + tid;
          const int kind = (int)d.data[q];
          if (kind != 0) {
            const double pa = d.data[nn + q], pb = d.data[2 * nn + q], pc = d.data[3 * nn + q];
            const double bm1 = d.data[4 * nn + q];
            const double* en = s_u64 + 3 * N3;
#pragma unroll
            for (int cc = 0; cc < 3; ++cc) {
              const double j1 = d.aux[cc * nn + q], ev = en[cc * N3 + tid];
              res[3 + cc] = (T)((double)res[3 + cc] - j1 * bm1);
              double r1 = -pa * j1 + pb * ev;
              if (kind == 2) {
                const double j2 = d.aux[(3 + cc) * nn + q];
                r1 = -pa * j1 - pb * j2 + pc * ev;
                const double k2 = first_stage ? a.dt * j1 : fma(a.a, d.k[(3 + cc) * nn + q], a.dt * j1);
                d.k[(3 + cc) * nn + q] = k2;
                d.aux[(3 + cc) * nn + q] = fma(a.b, k2, j2);
              }
              const double k1 = first_stage ? a.dt * r1 : fma(a.a, d.k[cc * nn + q], a.dt * r1);
              d.k[cc * nn + q] = k1;
              d.aux[cc * nn + q] = fma(a.b, k1, j1);
            }
          }
        }
      }
      // ---- volume source (usersrc), mass-weighted -------------------------
      if (a.src_elem) {
        const int so = a.src_elem[e];
        if (so >= 0)
          res[5] += reinterpret_cast<const T*>(a.src_w)[(long)so * N3 + tid] * Par<T>::ft(a);
      }
    }
    // ---- inverse mass + low-storage RK, FP64 -------------------------------
    double kn[6], un[6];
    if (node) {
      const double ch = s_coef[tid], ce = s_coef[N3 + tid];
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const double r = to_f64(res[c]) * (c < 3 ? ch : ce);
        kn[c] = first_stage ? r : fma(a.a, s_k[c * N3 + tid], r);
        un[c] = fma(a.b, kn[c], s_u64[c * N3 + tid]);
      }
    }
    __syncthreads();  // staged blocks consumed: the next element may land
    const int en = e + gridDim.x;
    if (C::kTma && tid == 0 && en < a.nelt) {
      fence_proxy_async_smem();
      issue_tma(en);
    }
    if (node) {
      const long g = (long)e * N3 + tid;
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        a.k_out[c * P + g] = kn[c];
        a.u_out[c * P + g] = un[c];
      }
    }
  }
}

// dt-scaled inverse-mass coefficients: coef = dt * base (2*n entries)
__global__ void k_scale_coef(double* coef, const double* base, long n2, double dt) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n2) return;
  coef[i] = dt * base[i];
}

// EXT: the variant with the PML and dispersive-current branches (a separate
// instantiation, so that meshes without them keep the kernel's register budget)
template <int NX, typename T, bool EXT>
int launch(Context* c, const FusedDev& a) {
  using C = Cfg<NX, T>;
  auto kern = k_fused_stage<NX, T, EXT>;
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
  c->fused_grid = g;
  kern<<<g, C::NT, C::smem, c->stream>>>(a);
  c->last_launches += 1;
  return check_cuda(cudaGetLastError());
}

template <typename T, bool EXT>
int dispatch_nx(Context* c, const FusedDev& a) {
  switch (c->nx) {
    case 3: return launch<3, T, EXT>(c, a);
    case 4: return launch<4, T, EXT>(c, a);
    case 5: return launch<5, T, EXT>(c, a);
    case 6: return launch<6, T, EXT>(c, a);
    case 7: return launch<7, T, EXT>(c, a);
    case 8: return launch<8, T, EXT>(c, a);
    case 9: return launch<9, T, EXT>(c, a);
    default: return NEKGPU_ERR_UNSUPPORTED;
  }
}

template <typename T>
int dispatch(Context* c, const FusedDev& a) {
  return (a.pml.slot || a.disp.slot || a.inc_elem || a.gr.elem) ? dispatch_nx<T, true>(c, a)
                                                               : dispatch_nx<T, false>(c, a);
}

}  // namespace

int scale_coef(Context* c, double dt) {
  if (c->coef_dt == dt) return NEKGPU_OK;
  long n2 = 2 * c->npts;
  k_scale_coef<<<(unsigned)((n2 + 255) / 256), 256, 0, c->stream>>>(c->d_coef, c->d_cbase, n2,
                                                                      dt);
  c->last_launches += 1;
  c->coef_dt = dt;
  return check_cuda(cudaGetLastError());
}

int fused_stage_buffers(Context* c, int rkstep, double time, double dt, const double* u_in,
                        double* u_out, double* k_in, double* k_out) {
  int st = scale_coef(c, dt);
  if (st) return st;
  FusedDev a = c->fargs;
  a.u_in = u_in;
  a.u_out = u_out;
  a.k = k_in;
  a.k_out = k_out;
  a.a = c->rk_a[rkstep - 1];
  a.b = c->rk_b[rkstep - 1];
  a.dt = dt;
  if (c->src.enabled) {
    a.src_ft = source_ft(c->src, time + dt * c->rk_c[rkstep - 1]);
    a.src_ftf = (float)a.src_ft;
  }
  return c->form == NEKGPU_MIXED_NAIVE ? dispatch<float>(c, a) : dispatch<double>(c, a);
}

int fused_setup(Context* c) {
  if (c->nx < 3 || c->nx > 9) return NEKGPU_ERR_UNSUPPORTED;
  return NEKGPU_OK;
}

int fused_stage(Context* c, int rkstep, double time, double dt) {
  int st = scale_coef(c, dt);
  if (st) return st;
  FusedDev a = c->fargs;
  a.u_in = c->d_u[c->cur];
  a.u_out = c->d_u[c->cur ^ 1];
  a.k_out = a.k;
  a.a = c->rk_a[rkstep - 1];
  a.b = c->rk_b[rkstep - 1];
  a.dt = dt;
  if (c->src.enabled) {
    a.src_ft = source_ft(c->src, time + dt * c->rk_c[rkstep - 1]);
    a.src_ftf = (float)a.src_ft;
  }
  if (a.inc_elem && (st = incident_upload(c, time + dt * c->rk_c[rkstep - 1]))) return st;
  if (a.gr.elem) {
    a.gr.f_in = c->d_gr_f[c->gr_cur];
    a.gr.f_out = c->d_gr_f[c->gr_cur ^ 1];
  }
  st = c->form == NEKGPU_MIXED_NAIVE ? dispatch<float>(c, a) : dispatch<double>(c, a);
  if (st) return st;
  if (a.gr.elem) c->gr_cur ^= 1;
  c->cur ^= 1;
  return NEKGPU_OK;
}

}  // namespace nekgpu
