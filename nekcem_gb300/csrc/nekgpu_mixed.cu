// Mixed-precision Maxwell DG stage kernel for sm_103a (NEKGPU_MIXED).
//
// Same stage as nekgpu_fused.cu -- weighted curl from the GLL derivative
// contractions (src/nek5_grad.F:2-19, src/cem_maxwell.F:1428-1497), upwind
// face flux with the partner-face read that replaces gs_op_fields
// (src/cem_maxwell.F:922-1002, 1368-1426), lift (src/cem_maxwell.F:725-735),
// volume source, inverse mass (src/cem_maxwell.F:1878-1886) and the
// low-storage RK update (src/cem_common.F:18-75) -- with the contractions, curl
// and flux in FP32 and the state, RK register, inverse mass and update in
// FP64.  FP32 is used so that it does not cost accuracy:
//
//  * Exact-hi contractions.  Per element and field component, u is split into
//    uh = u rounded to a 10-bit grid q (q from the element's largest |u|) and
//    ul = u - uh; each row of D is split the same way into Dh (10 bits) plus
//    the remainder Dm = RN32(D - Dh), so D itself is represented to ~2^-34 of
//    its row (a D rounded to FP32, 2^-24, perturbs the operator enough to
//    drift the phase over thousands of steps; 2^-34 does not: the plane-wave
//    and cavity errors stay at the FP64 form's).  Every product Dh*uh is an
//    integer multiple of q*qD below 2^20 q*qD, so the FP32 sum over the <= 16
//    terms is exact.  The small remainder sum(Df*ul + Dm*uh) is summed in FP32
//    beside it.  The FP32 rounding error is ~2^-34 of sum|D||u| instead of
//    ~2^-24.
//  * Thread per line.  Each thread contracts one GLL line at a time, so every
//    D coefficient is a compile-time constant-bank operand.  The three
//    products of a term run as packed FP32x2 FMAs (sm_100 family), one and a
//    half per term: (hi_i, lo_i) += (Dh, Df)(i,l) * (uh, ul)_l for every
//    output i and (m_i, m_i+1) += (Dm(i,l), Dm(i+1,l)) * (uh, uh)_l for every
//    pair of outputs.
//  * Normalised residual.  For an affine axis-aligned element the mass
//    cancels the GLL weights and metrics: res/(bm1*2/hx) = d_s Hz - d_t Hy
//    (+ face terms flux*area/(bm1*2/hx)), etc.  All FP32 coefficients are then
//    exact (1, or a float pair for non-cubic elements); the FP64 inverse-mass
//    coefficient carries dt*(2/hx)/eps.
//  * Pair residual.  The residual stays an unevaluated FP32 pair (hi, lo); it
//    is multiplied by the FP64 coefficient as a float-float product, rounded
//    to FP64 once (DADD) and enters the FP64 RK update (2 DFMA).
//
// FP64 <-> FP32 conversions use integer instructions only: every FP64-pipe
// instruction on GB300 (including F2F) runs at 2 lanes/clock/SM.
#include <cuda_runtime.h>
#include <stdint.h>

#include "nekgpu_internal.h"
#include "nekgpu_pair.cuh"

namespace nekgpu {

namespace {


// (Rh, Rl) += w * f for float pairs w = (wh, wl), f = (fh, fl): the product's
// rounding error and cross terms go to the low part (~2^-46 of |w f|), so a
// volume source enters the residual pair at the pair's own precision
__device__ __forceinline__ void add_pair_product(float& Rh, float& Rl, float2 w, float2 f) {
  const float p = w.x * f.x;
  float e = fmaf(w.x, f.x, -p);
  e = fmaf(w.x, f.y, e);
  e = fmaf(w.y, f.x, e);
  float s, t;
  two_sum(Rh, p, s, t);
  Rh = s;
  Rl = (Rl + e) + t;
}

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
// orders this thread's (and, after a barrier, the block's) generic-proxy
// shared-memory accesses before later async-proxy (TMA) accesses
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
// bulk prefetch of a global range into L2 (a hint: no completion to wait for);
// address and size multiples of 16 bytes
// 8-byte asynchronous global -> shared copies (element blocks whose size is
// not a multiple of 16 bytes, where a bulk copy cannot start on every element)
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
// one line into L1 ahead of a load
__device__ __forceinline__ void prefetch_l1(const void* p) {
  asm volatile("prefetch.global.L1 [%0];\n" ::"l"(p));
}
__device__ __forceinline__ void prefetch_l2(const void* src, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
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
// gives up after ~2^22 polls (far beyond any copy time) and records it
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, int* status) {
  for (int it = 0; it < (1 << 22); ++it)
    if (mbar_try_wait(bar, parity)) return true;
  atomicExch(status, 1);
  return false;
}

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

// D of order nx-1 in the FP32 pieces of the exact-hi contraction, as float
// pairs indexed by nx so that every coefficient is a compile-time
// constant-bank operand: [nx][0][i + nx*l] = (Dh, Df) of D(i,l),
// [nx][1][j + H*l] = (Dm(2j,l), Dm(2j+1,l)) with H = (nx+1)/2 (zero past the
// last row).  Dh is D on a 10-bit grid of its row, Df = RN32(D),
// Dm = RN32(D - Dh).  D depends only on nx.
__constant__ float2 c_mixD[kMaxMixed + 1][2][kMaxMixed * kMaxMixed];

// A copy of the thread index the compiler cannot see through: index math
// derived from it is recomputed in each phase instead of being hoisted out of
// the element loop, where it would stay live in registers for every phase.
__device__ __forceinline__ int opaque_tid() {
  int t = threadIdx.x;
  asm volatile("" : "+r"(t));
  return t;
}

constexpr int cmax(int a, int b) { return a > b ? a : b; }
constexpr int round32(int a) { return (a + 31) / 32 * 32; }

// TPL: threads per line task (2: each computes half of a line's outputs, for
// meshes with fewer elements than SMs, where the time per stage is one
// element's latency)
template <int NX, int TPL = 1>
struct MCfg {
  static constexpr int N2 = NX * NX, N3 = N2 * NX;
  // Node layout of the FP32 pair arrays.  NX = 8: unpadded, node
  // v = i + 8j + 64k stored at v ^ ((v >> 3) & 15) (low three bits i^j, bit 3
  // j0^k0), so the 16 lanes of a half warp -- 8 lines or nodes of two
  // neighbouring rows -- hit 16 distinct 8-byte bank pairs along r-, s- and
  // t-lines, on every face and in node order.  Other NX: rows padded to NX+1.
  static constexpr bool kSwz = (NX == 8);
  static constexpr int RS = kSwz ? NX : NX + 1;
  static constexpr int SZ = RS * NX;
  static constexpr int N3P = NX * SZ;
  static constexpr int NF = 6 * N2;
  static constexpr int NTASK = 4 * N2;  // line tasks per direction
  static constexpr int NT = round32(cmax(NTASK * TPL, (N3 + 1) / 2));
  static constexpr int NW = NT / 32;
  static constexpr int NPT = (N3 + NT - 1) / NT;
  static constexpr int FPT = (NF + NT - 1) / NT;
  static constexpr int TPT = (NTASK * TPL + NT - 1) / NT;
  static constexpr bool kTma = (N3 % 2) == 0;
  // odd node counts: the next element staged by per-thread 8-byte async
  // copies where that measured faster (N=8 +3 %, N=6 +0.9 %; N=4, N=2 load
  // synchronously: -0.5 %, -1.8 % with the async copies)
  static constexpr bool kAsync = !kTma && NX >= 7;
  // L1 prefetch of the finish's loads where it measured faster: in the t-line
  // tasks that finish (N=6 +2.5 %, N=4 +0.4 %; N=5 -1.9 %: it spills there)
  // and for the next node of the node-by-node finish (N=8 +1.4 %; N=7 -2.2 %)
  static constexpr bool kPfLine = NX == 5 || NX == 7;
  static constexpr bool kPfNode = NX == 9;
  // Where the components finish (inverse mass, RK update) without the
  // extension terms: true = the t-line tasks finish H1, H2, E1, E2 on their
  // lines and H3, E3 (no t-derivative) finish beside them, with no barrier and
  // no residual round trip; false = node by node after the t-lines (NX = 8
  // and 9: the t-line tasks cannot cover the loads of eight or nine finishes;
  // the in-line finish measured 5 % slower at NX = 8 and 16 % slower at
  // NX = 9, 20 % faster at NX = 6).
  static constexpr bool kFin = !kSwz && NX != 9;
  // r = p + ee without an FP64 add (rk_finish_cf) where that measured faster:
  // N=7 -1.8 %, N=6 -1.9 %, N=4 -0.9 % per step; N=8 unchanged; N=5 +5.4 %
  static constexpr bool kIntAdd = NX == 5 || NX == 7 || NX == 8;
  // Two areas of SA bytes swap roles from one element to the next.  One holds,
  // in turn, the staged FP64 state (until the split), the partner face values
  // parked for the flux (FP64) and the residual pairs (hi, lo); the other the
  // split pairs (uh, ul), dead after the t-lines, so the next element's state
  // can land there while this one is finished.  54 KB in all at NX=8, four
  // blocks per SM.
  static constexpr size_t SA = cmax(cmax(6 * N3 * 8, 6 * N3P * 8), 6 * NF * 8);
  static constexpr size_t off_F = 2 * SA;  // float2 flux pairs [face][line slot][N2]
  static constexpr size_t off_wmax = off_F + 24 * N2 * 8;
  static constexpr size_t off_E = off_wmax + NW * 6 * 4;
  static constexpr size_t off_bar = (off_E + 8 * 4 + 15) / 16 * 16;
  static constexpr size_t smem = off_bar + 16;
};

// components contracted in each direction, the residual they feed, the sign
// and whether they start (init) or add to that residual.  Residual index
// 0..2 = H1..H3 (-curl E), 3..5 = E1..E3 (curl H); field 0..2 = H, 3..5 = E.
//   E1 = ds Hz - dt Hy   E2 = dt Hx - dr Hz   E3 = dr Hy - ds Hx
//   H1 = dt Ey - ds Ez   H2 = dr Ez - dt Ex   H3 = ds Ex - dr Ey
__constant__ const int kLineComp[3][4] = {{1, 2, 4, 5}, {0, 2, 3, 5}, {0, 1, 3, 4}};
__constant__ const int kLineRes[3][4] = {{5, 4, 2, 1}, {5, 3, 2, 0}, {4, 3, 1, 0}};
__constant__ const float kLineSign[3][4] = {{1, -1, -1, 1}, {-1, 1, 1, -1}, {1, -1, -1, 1}};
__constant__ const int kLineInit[3][4] = {{1, 1, 1, 1}, {0, 1, 0, 1}, {0, 0, 0, 0}};

template <int NX, int DIR>
__device__ __forceinline__ int line_node(int a, int b, int l) {
  constexpr int RS = MCfg<NX>::RS, SZ = MCfg<NX>::SZ;
  if constexpr (MCfg<NX>::kSwz) {
    // node (l,a,b), (a,l,b) or (a,b,l) under the NX = 8 swizzle
    if constexpr (DIR == 0) return (((a << 3) | (b << 6)) ^ ((b & 1) << 3)) | (l ^ a);
    if constexpr (DIR == 1) return (a ^ l) | ((l ^ (b & 1)) << 3) | (b << 6);
    return (a ^ b) | ((b ^ (l & 1)) << 3) | (l << 6);
  }
  return DIR == 0 ? l + RS * a + SZ * b : (DIR == 1 ? a + RS * l + SZ * b : a + RS * b + SZ * l);
}
template <int NX>
__device__ __forceinline__ int pnode(int v) {  // stored index of node v = i + NX*j + NX^2*k
  if constexpr (MCfg<NX>::kSwz) return v ^ ((v >> 3) & 15);
  return (v % NX) + MCfg<NX>::RS * ((v / NX) % NX) + MCfg<NX>::SZ * (v / (NX * NX));
}

// Inverse mass and RK update of one component c at global node g, in FP64,
// from the normalised residual pair (Rh, Rl): the pair times the dt-scaled
// FP64 coefficient as a float-float product, rounded to FP64 once (DADD),
// then k = a k + r and u = u + b k (two DFMA; one at stage 1).  The state is
// read again from global memory (an L2 hit: the element's block was copied in
// at the start of its turn), the RK register and the coefficients were
// prefetched into L2 with that copy.
// IA: r = p + ee formed by a two-sum and pair_to_double (integer and FP32
// operations) instead of an FP64 add: two FP64 operations per component
// instead of three, for the orders whose finish the FP64 pipe limits.
template <bool IA>
__device__ __forceinline__ void rk_finish_cf(const MixedDev& a, int c, long g, float Rh, float Rl,
                                             float2 cf, bool first_stage) {
  const long P = a.npts;
  const float p = cf.x * Rh;
  float ee = fmaf(cf.x, Rh, -p);
  ee = fmaf(cf.x, Rl, ee);
  ee = fmaf(cf.y, Rh, ee);
  double r;
  if constexpr (IA) {
    float s, t;
    two_sum(p, ee, s, t);
    r = pair_to_double(s, t);
  } else {
    r = f2d(p) + f2d(ee);
  }
  const double kn = first_stage ? r : fma(a.a, a.k[c * P + g], r);
  a.k_out[c * P + g] = kn;
  a.u_out[c * P + g] = fma(a.b, kn, __ldg(a.u_in + c * P + g));
}
// All six components of node g: the node's RK register and state loaded
// first (twelve loads in flight; the stores of one component would otherwise
// keep the next component's loads behind them, k_out possibly being k), then
// the six updates as in rk_finish_cf.
template <bool IA>
__device__ __forceinline__ void rk_finish_node(const MixedDev& a, long g, const float* Rh,
                                               const float* Rl, float2 cfH, float2 cfE,
                                               bool first_stage) {
  const long P = a.npts;
  double kk[6], uu[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    kk[c] = first_stage ? 0.0 : a.k[c * P + g];
    uu[c] = __ldg(a.u_in + c * P + g);
  }
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    const float2 cf = c < 3 ? cfH : cfE;
    const float p = cf.x * Rh[c];
    float ee = fmaf(cf.x, Rh[c], -p);
    ee = fmaf(cf.x, Rl[c], ee);
    ee = fmaf(cf.y, Rh[c], ee);
    double r;
    if constexpr (IA) {
      float s, t;
      two_sum(p, ee, s, t);
      r = pair_to_double(s, t);
    } else {
      r = f2d(p) + f2d(ee);
    }
    const double kn = first_stage ? r : fma(a.a, kk[c], r);
    a.k_out[c * P + g] = kn;
    a.u_out[c * P + g] = fma(a.b, kn, uu[c]);
  }
}
template <bool IA>
__device__ __forceinline__ void rk_finish(const MixedDev& a, int c, long g, float Rh, float Rl,
                                          bool first_stage) {
  rk_finish_cf<IA>(a, c, g, Rh, Rl, a.coef[(c < 3 ? 0 : a.npts) + g], first_stage);
}

// c1*J1 + c2*J2 times the lift factor lf, all float pairs, as a float pair.
// A jump J = (A, B) is an unevaluated pair (jump_pair); the coefficients are
// (hi, lo) pairs.  Absolute error ~2^-24 of |c B| and of |lf (c1 A1 + c2 A2)|
// 2^-24, i.e. ~2^-34 of the field: the flux keeps the residual pair's
// precision whatever the size of the jump.
__device__ __forceinline__ float2 flux_pair(float2 c1, float2 J1, float2 c2, float2 J2, float2 lf) {
  const float p1 = c1.x * J1.x;
  float e1 = fmaf(c1.x, J1.x, -p1);
  e1 = fmaf(c1.x, J1.y, e1);
  e1 = fmaf(c1.y, J1.x, e1);
  const float p2 = c2.x * J2.x;
  float e2 = fmaf(c2.x, J2.x, -p2);
  e2 = fmaf(c2.x, J2.y, e2);
  e2 = fmaf(c2.y, J2.x, e2);
  float s, t;
  two_sum(p1, p2, s, t);
  const float lo = (e1 + e2) + t;
  const float fh = lf.x * s;
  float fl = fmaf(lf.x, s, -fh);
  fl = fmaf(lf.x, lo, fl);
  fl = fmaf(lf.y, s, fl);
  return make_float2(fh, fl);
}

__device__ __forceinline__ float2 neg2(float2 v) { return make_float2(-v.x, -v.y); }

// J += d for an FP64 term d (incident fields, sheet currents), in pair
// arithmetic
__device__ __forceinline__ void add_jump(float2& J, double d) {
  float s, t;
  two_sum(J.x, d2f_hi(d), s, t);
  J = make_float2(s, (J.y + d2f_lo(d)) + t);
}

// Field component of the k-th parked partner value of face f: all six with
// the extension terms, else H and E along the two axes tangential to f
// (k = 0, 1: H; k = 2, 3: E; lower axis first).
template <bool EXT>
__device__ __forceinline__ int partner_comp(int f, int k) {
  if (EXT) return k;
  const int ax = slot_axis(f);
  const int tang = (k & 1) ? (ax == 2 ? 1 : 2) : (ax == 0 ? 1 : 0);
  return (k < 2 ? 0 : 3) + tang;
}

// The jump p - (uh + ul) of a partner value p (FP64) against the own split
// pair, as an unevaluated pair: the hi difference with its rounding error
// (two-sum: a jump as large as the field needs 25 bits), the lo parts beside
// it (their difference is below 2^-10 of the element's largest value).
__device__ __forceinline__ float2 jump_pair(double p, float2 own) {
  float s, t;
  two_sum(d2f_hi(p), -own.x, s, t);
  return make_float2(s, (d2f_lo(p) - own.y) + t);
}

// Outputs I0 .. I0+NXP-1 of one line task (all NX of them, or one half when
// two threads share the line): the contraction, the rho factor, the lifted
// flux at the line's ends and the accumulation into the residual pairs (or,
// FIN, the finish).
template <int NX, int DIR, bool FIN, int TPL, int I0, int NXP>
__device__ __forceinline__ void line_outputs(const float2* u, float2* R0, float2 flux_m,
                                             float2 flux_p, bool cubic, float rh, float rl,
                                             float sg, bool init, int la, int lb, int rt,
                                             const MixedDev& a, int e, bool first_stage) {
  using C = MCfg<NX, TPL>;
  // packed in float pairs:
  //   (hi_i, lo_i)   += (Dh, Df)(i,l) * (uh, ul)_l      hi exact
  //   (m_i, m_i+1)   += (Dm(i,l), Dm(i+1,l)) * (uh, uh)_l
  constexpr int H = (NX + 1) / 2, HP = (NXP + 1) / 2, J0 = I0 / 2;
  static_assert(I0 % 2 == 0, "output pairs start on an even output");
  float2 x[NXP], y[HP];
#pragma unroll
  for (int j = 0; j < NXP; ++j) x[j] = __fmul2_rn(c_mixD[NX][0][I0 + j], u[0]);
#pragma unroll
  for (int j = 0; j < HP; ++j) y[j] = __fmul2_rn(c_mixD[NX][1][J0 + j], make_float2(u[0].x, u[0].x));
#pragma unroll
  for (int l = 1; l < NX; ++l) {
    const float2 uu = make_float2(u[l].x, u[l].x);
#pragma unroll
    for (int j = 0; j < NXP; ++j) x[j] = __ffma2_rn(c_mixD[NX][0][I0 + j + NX * l], u[l], x[j]);
#pragma unroll
    for (int j = 0; j < HP; ++j) y[j] = __ffma2_rn(c_mixD[NX][1][J0 + j + H * l], uu, y[j]);
  }
#pragma unroll
  for (int j = 0; j < NXP; ++j) {
    const int i = I0 + j;
    float h = x[j].x, r = x[j].y + ((j & 1) ? y[j / 2].y : y[j / 2].x);
    if (DIR != 0 && !cubic) {  // times rho = g_dir/g_x as a float pair
      const float p = rh * h;
      float ee = fmaf(rh, h, -p);
      ee = fmaf(rh, r, ee);
      ee = fmaf(rl, h, ee);
      h = p;
      r = ee;
    }
    h *= sg;
    r *= sg;
    if (i == 0 || i == NX - 1) {  // the lifted flux pair of the end's face
      const float2 F = i == 0 ? flux_m : flux_p;
      float s, t;
      two_sum(h, F.x, s, t);
      h = s;
      r = (r + F.y) + t;
    }
    float2* Rp = R0 + line_node<NX, DIR>(la, lb, i);
    if (FIN) {
      const float2 old = *Rp;
      float sum, err;
      two_sum(old.x, h, sum, err);
      const int vol = DIR == 0 ? i + NX * la + C::N2 * lb
                               : (DIR == 1 ? la + NX * i + C::N2 * lb : la + NX * lb + C::N2 * i);
      rk_finish<C::kIntAdd>(a, rt, (long)e * C::N3 + vol, sum, (old.y + r) + err, first_stage);
    } else if (init) {
      *Rp = make_float2(h, r);
    } else {
      const float2 old = *Rp;
      float sum, err;
      two_sum(old.x, h, sum, err);
      *Rp = make_float2(sum, (old.y + r) + err);
    }
  }
}

// One direction of the contraction: tasks (component, line) accumulate the
// signed derivative pair into the residual pair arrays.  The line's two end
// nodes lie on the faces normal to DIR; the lifted flux of those faces in the
// task's residual component (s_F, stored in this direction's slot order) is
// added to their low parts.  FIN (last direction): the residual of the
// task's component is complete at the line's nodes, so the task finishes
// them (inverse mass, RK update) instead of storing the pairs.  TPL = 2: two
// threads per line, each with half of its outputs (the halves in separate
// warps, so the branch on the half is warp-uniform).
template <int NX, int DIR, bool FIN, int TPL = 1>
__device__ __forceinline__ void line_phase(const float2* s_u2, float2* s_R2, const float2* s_F,
                                           bool cubic, float rh, float rl, const MixedDev& a,
                                           int e, bool first_stage) {
  using C = MCfg<NX, TPL>;
  static_assert(TPL == 1 || (TPL == 2 && !FIN && NX % 4 == 0), "two threads per line: NX = 4k, no FIN");
  const int tid = opaque_tid();
#pragma unroll
  for (int q = 0; q < C::TPT; ++q) {
    const int task = tid + q * C::NT;
    if (task < C::NTASK * TPL) {
      const int part = TPL == 1 ? 0 : task / C::NTASK;
      const int lt = task - part * C::NTASK;
      const int slot = lt / C::N2, lam = lt - slot * C::N2;
      const int la = lam % NX, lb = lam / NX;
      const int comp = kLineComp[DIR][slot], rt = kLineRes[DIR][slot];
      const float sg = kLineSign[DIR][slot];
      const bool init = kLineInit[DIR][slot] != 0;
      const float2* pu = s_u2 + comp * C::N3P;
      if (FIN && C::kPfLine) {  // the line's RK register and state, read by its finish: into L1 now
        const long P = a.npts;
#pragma unroll
        for (int i = 0; i < NX; ++i) {
          const int vol = DIR == 0 ? i + NX * la + C::N2 * lb
                                   : (DIR == 1 ? la + NX * i + C::N2 * lb : la + NX * lb + C::N2 * i);
          const long g = (long)e * C::N3 + vol;
          if (!first_stage) prefetch_l1(a.k + rt * P + g);
          prefetch_l1(a.u_in + rt * P + g);
        }
      }
      // lifted flux at the line's ends: faces 3|1 (r), 0|2 (s), 4|5 (t)
      constexpr int FM = DIR == 0 ? 3 : (DIR == 1 ? 0 : 4);
      constexpr int FP = DIR == 0 ? 1 : (DIR == 1 ? 2 : 5);
      const float2 flux_m = s_F[(FM * 4 + slot) * C::N2 + lam];
      const float2 flux_p = s_F[(FP * 4 + slot) * C::N2 + lam];
      float2 u[NX];
#pragma unroll
      for (int l = 0; l < NX; ++l) u[l] = pu[line_node<NX, DIR>(la, lb, l)];
      float2* R0 = s_R2 + rt * C::N3P;
      if constexpr (TPL == 1) {
        line_outputs<NX, DIR, FIN, TPL, 0, NX>(u, R0, flux_m, flux_p, cubic, rh, rl, sg, init, la, lb,
                                               rt, a, e, first_stage);
      } else if (part == 0) {
        line_outputs<NX, DIR, FIN, TPL, 0, NX / 2>(u, R0, flux_m, flux_p, cubic, rh, rl, sg, init, la,
                                                   lb, rt, a, e, first_stage);
      } else {
        line_outputs<NX, DIR, FIN, TPL, NX / 2, NX / 2>(u, R0, flux_m, flux_p, cubic, rh, rl, sg, init,
                                                        la, lb, rt, a, e, first_stage);
      }
    }
  }
}

// PML (pml_step, src/cem_maxwell_pml.F:508-590) at one node of a PML element,
// in FP64: the auxiliary residuals from res/bm1 = R * (w3 rx / bm1), their RK
// update (src/cem_maxwell.F:1942-1955), and the PML terms of res added to the
// normalised residual pair R as FP32 pairs.
template <int N3>
__device__ __forceinline__ void pml_node(const MixedDev& a, int l, int v, long g, bool first_stage,
                                      float* Rh, float* Rl) {
  const long nn = a.pml.n, q = (long)l * N3 + v, P = a.npts;
  const double* pd = a.pml.data;
  const double sxp = pd[q], syp = pd[nn + q], szp = pd[2 * nn + q];
  const double sigx = pd[3 * nn + q], sigy = pd[4 * nn + q], sigz = pd[5 * nn + q];
  const double mu = pd[6 * nn + q], fac = pd[9 * nn + q], inv = pd[10 * nn + q];
  double* aux = a.pml.aux;
  double* kx = a.pml.k;
  double bn[3], dn[3], hn[3], en[3], rp[6];
  for (int c = 0; c < 3; ++c) {
    bn[c] = aux[c * nn + q];
    dn[c] = aux[(3 + c) * nn + q];
    hn[c] = __ldg(a.u_in + c * P + g);
    en[c] = __ldg(a.u_in + (3 + c) * P + g);
  }
  double rb[6];
  for (int c = 0; c < 6; ++c) rb[c] = (f2d(Rh[c]) + f2d(Rl[c])) * fac;
  rp[0] = rb[0] - syp * bn[0];
  rp[1] = rb[1] - szp * bn[1];
  rp[2] = rb[2] - sxp * bn[2];
  rp[3] = rb[3] - syp * dn[0];
  rp[4] = rb[4] - szp * dn[1];
  rp[5] = rb[5] - sxp * dn[2];
  double t[6];
  t[0] = -syp * bn[0] + sxp * bn[0] - szp * mu * hn[0];
  t[1] = -szp * bn[1] + syp * bn[1] - sxp * mu * hn[1];
  t[2] = -sxp * bn[2] + szp * bn[2] - syp * mu * hn[2];
  t[3] = -syp * dn[0] + sxp * dn[0] - sigz * en[0];
  t[4] = -szp * dn[1] + syp * dn[1] - sigx * en[1];
  t[5] = -sxp * dn[2] + szp * dn[2] - sigy * en[2];
  for (int c = 0; c < 6; ++c) {
    const double dR = t[c] * inv;  // res += t bm1  ->  R += t bm1 / (w3 rx)
    float s, e;
    two_sum(Rh[c], d2f_hi(dR), s, e);
    Rh[c] = s;
    Rl[c] = (Rl[c] + d2f_lo(dR)) + e;
    const double kv = first_stage ? a.dt * rp[c] : fma(a.a, kx[c * nn + q], a.dt * rp[c]);
    kx[c * nn + q] = kv;
    aux[c * nn + q] = fma(a.b, kv, c < 3 ? bn[c] : dn[c - 3]);
  }
}

// Dispersive currents (cem_maxwell_drude / cem_maxwell_lorentz,
// src/cem_maxwell.F:3095-3212) at one node of an element holding listed
// nodes, in FP64: resE -= J1 bm1 enters the normalised residual pair as
// -J1 * bm1/(w3 rx), and the currents take their RK update.
template <int N3>
__device__ __forceinline__ void disp_node(const MixedDev& a, int l, int v, long g, bool first_stage,
                                          float* Rh, float* Rl) {
  const DispDev& d = a.disp;
  const long nn = d.n, q = (long)l * N3 + v, P = a.npts;
  const int kind = (int)d.data[q];
  if (kind == 0) return;
  const double pa = d.data[nn + q], pb = d.data[2 * nn + q], pc = d.data[3 * nn + q];
  const double inv = d.data[5 * nn + q];
  for (int c = 0; c < 3; ++c) {
    const double j1 = d.aux[c * nn + q], ev = __ldg(a.u_in + (3 + c) * P + g);
    const double dR = -(j1 * inv);
    float s, e;
    two_sum(Rh[3 + c], d2f_hi(dR), s, e);
    Rh[3 + c] = s;
    Rl[3 + c] = (Rl[3 + c] + d2f_lo(dR)) + e;
    double r1 = -pa * j1 + pb * ev;
    if (kind == 2) {
      const double j2 = d.aux[(3 + c) * nn + q];
      r1 = -pa * j1 - pb * j2 + pc * ev;
      const double k2 = first_stage ? a.dt * j1 : fma(a.a, d.k[(3 + c) * nn + q], a.dt * j1);
      d.k[(3 + c) * nn + q] = k2;
      d.aux[(3 + c) * nn + q] = fma(a.b, k2, j2);
    }
    const double k1 = first_stage ? a.dt * r1 : fma(a.a, d.k[c * nn + q], a.dt * r1);
    d.k[c * nn + q] = k1;
    d.aux[c * nn + q] = fma(a.b, k1, j1);
  }
}

// Blocks per SM the launch is built for: three at NX = 8 (62 KB of shared
// memory with the face flux as float pairs: a fourth does not fit; up to 80
// registers), six at NX = 6 (160 threads, 32 KB, 64 registers), two at NX = 9
// (384 threads, 94 KB), three otherwise and with the extension branches.
template <int NX, bool EXT, int TPL = 1>
constexpr int mixed_min_blocks() {
  return TPL == 2 ? 1 : (NX == 9 ? 2 : (EXT ? 3 : (NX == 6 ? 6 : 3)));
}

// EXT: the variant with the PML, dispersive-current, incident-field and
// graphene branches
template <int NX, bool EXT, int TPL = 1>
__global__ void __launch_bounds__(MCfg<NX, TPL>::NT, mixed_min_blocks<NX, EXT, TPL>())
    k_mixed_stage(const MixedDev a) {
  using C = MCfg<NX, TPL>;
  constexpr int N2 = C::N2, N3 = C::N3, NT = C::NT, NF = C::NF, N3P = C::N3P;
  constexpr int NPT = C::NPT, FPT = C::FPT;
  constexpr bool FIN = !EXT && C::kFin;  // the extension terms need all six at a node
  extern __shared__ __align__(16) unsigned char smem[];
  float2* s_F = reinterpret_cast<float2*>(smem + C::off_F);
  unsigned* s_wmax = reinterpret_cast<unsigned*>(smem + C::off_wmax);
  unsigned* s_E = reinterpret_cast<unsigned*>(smem + C::off_E);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + C::off_bar);
  __shared__ int s_abort;
  // launched as a programmatic dependent of the previous stage (device-
  // resident steps): read nothing the previous stage wrote before it has
  // completed and its writes are visible (a no-op for an ordinary launch).
  // Each block lets the next stage launch when it starts its last element,
  // so the next stage's blocks take the SMs this grid leaves (triggering at
  // entry let several stages' grids pile up waiting: C1 1.5x slower)
  asm volatile("griddepcontrol.wait;\n" ::: "memory");

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int tid = threadIdx.x;
  const long P = a.npts;
  const bool first_stage = (a.a == 0.0);  // rk4a(1) = 0: k restarts

  if (tid == 0) {
    s_abort = 0;
    if (C::kTma) {
      mbar_init(bar, 1);
      fence_mbar_init();
    }
  }
  __syncthreads();
  // element e's state into area `into`
  auto issue_tma = [&](int e, int into) {
    const unsigned bytes = N3 * 8;
    double* dst = reinterpret_cast<double*>(smem + into * C::SA);
    mbar_expect_tx(bar, 6u * bytes);
    for (int c = 0; c < 6; ++c) tma_load_1d(dst + c * N3, a.u_in + c * P + (long)e * N3, bytes, bar);
    // the RK register and the coefficients are read at the end of the
    // element's turn: start bringing them into L2 now
    if (!first_stage)
      for (int c = 0; c < 6; ++c) prefetch_l2(a.k + c * P + (long)e * N3, bytes);
    for (int c = 0; c < 2; ++c) prefetch_l2(a.coef + c * P + (long)e * N3, N3 * 8u);
    // and the face impedance coefficients the flux reads (float4 per face node)
    if (a.fcoef) prefetch_l2(reinterpret_cast<const float4*>(a.fcoef) + 2L * e * NF, NF * 32u);
  };
  // the same with every thread copying its own nodes (odd node counts)
  auto issue_async = [&](int e, int into, int t) {
    double* dst = reinterpret_cast<double*>(smem + into * C::SA);
#pragma unroll
    for (int q = 0; q < NPT; ++q) {
      const int v = t + q * NT;
      if (v < N3)
#pragma unroll
        for (int c = 0; c < 6; ++c) cp_async8(dst + c * N3 + v, a.u_in + c * P + (long)e * N3 + v);
    }
    cp_async_commit();
  };
  unsigned parity = 0;
  int buf = 0;  // area of the element's staged state and residual pairs
  if (C::kTma && tid == 0 && a.e_begin + (int)blockIdx.x < a.e_end) issue_tma(a.e_begin + blockIdx.x, 0);
  if (C::kAsync && a.e_begin + (int)blockIdx.x < a.e_end) issue_async(a.e_begin + blockIdx.x, 0, tid);

  for (int e = a.e_begin + blockIdx.x; e < a.e_end; e += gridDim.x, buf ^= 1) {
    int tid = opaque_tid();
    if (e + (int)gridDim.x >= a.e_end) asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
    double* s_u64 = reinterpret_cast<double*>(smem + buf * C::SA);
    float2* s_R2 = reinterpret_cast<float2*>(smem + buf * C::SA);
    float2* s_u2 = reinterpret_cast<float2*>(smem + (buf ^ 1) * C::SA);
    const int en = e + gridDim.x;
    const int* nbr = a.nbr + 6 * e;
    const float* eg = a.egm + 16 * e;
    // ---- early loads: partner face nodes (kept in registers until the flux)
    // The flux of a face uses the components tangential to it: without the
    // extension terms only those four are loaded (H and E along the two
    // other axes); the graphene sheets need all six.
    constexpr int NPC = EXT ? 6 : 4;
    double nbv[FPT][NPC];
#pragma unroll
    for (int q = 0; q < FPT; ++q) {
      const int t = tid + q * NT;
      if (t < NF) {
        const int f = t / N2, ab = t - f * N2;
        const int pe = nbr[f];
        if (pe >= 0) {
          const long pv = (long)pe * N3 + face_vol<NX>(slot_opp(f), ab % NX, ab / NX);
#pragma unroll
          for (int k = 0; k < NPC; ++k) nbv[q][k] = __ldg(a.u_in + partner_comp<EXT>(f, k) * P + pv);
        }
      }
    }
    // ---- own element state ----------------------------------------------
    if (C::kTma) {
      if (!mbar_wait_bounded(bar, parity, a.status)) s_abort = 1;
      parity ^= 1u;
    } else if (C::kAsync) {
      cp_async_wait_all();  // this thread's copies; the barrier below: everyone's
    } else {
#pragma unroll
      for (int q = 0; q < NPT; ++q) {
        const int v = tid + q * NT;
        if (v < N3)
#pragma unroll
          for (int c = 0; c < 6; ++c) s_u64[c * N3 + v] = a.u_in[c * P + (long)e * N3 + v];
      }
    }
    __syncthreads();
    if (s_abort) return;
    // ---- per-component largest exponent of the element -> 10-bit grid ----
    {
      unsigned em[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
      for (int q = 0; q < NPT; ++q) {
        const int v = tid + q * NT;
        if (v < N3)
#pragma unroll
          for (int c = 0; c < 6; ++c) {
            const unsigned hw = (unsigned)__double2hiint(s_u64[c * N3 + v]);
            em[c] = max(em[c], (hw >> 20) & 0x7FFu);
          }
      }
#pragma unroll
      for (int c = 0; c < 6; ++c) em[c] = __reduce_max_sync(0xffffffffu, em[c]);
      if (lane == 0)
#pragma unroll
        for (int c = 0; c < 6; ++c) s_wmax[warp * 6 + c] = em[c];
    }
    __syncthreads();
    if (tid < 6) {
      unsigned m = 0;
      for (int w = 0; w < C::NW; ++w) m = max(m, s_wmax[w * 6 + tid]);
      s_E[tid] = min(max(m, 906u), 1158u);
    }
    __syncthreads();
    // ---- split: uh on the grid q = 2^(E-1032), ul = u - uh ----------------
    tid = opaque_tid();
    {
      const float M = 12582912.0f;  // 1.5 * 2^23: float rounding to integers
      unsigned Ec[6];
#pragma unroll
      for (int c = 0; c < 6; ++c) Ec[c] = s_E[c];
#pragma unroll
      for (int q = 0; q < NPT; ++q) {
        const int v = tid + q * NT;
        if (v < N3) {
          double u[6];  // loaded before any store (which they could not pass)
#pragma unroll
          for (int c = 0; c < 6; ++c) u[c] = s_u64[c * N3 + v];
          const int pv = pnode<NX>(v);
#pragma unroll
          for (int c = 0; c < 6; ++c) {
            const int E = (int)Ec[c];
            const float qv = __int_as_float((E - 905) << 23);    // 2^(E-1032)
            const float qi = __int_as_float((1159 - E) << 23);   // 2^(1032-E)
            const float uf = d2f_hi(u[c]), ulo = d2f_lo(u[c]);
            const float uh = (__fadd_rn(__fmaf_rn(uf, qi, M), -M)) * qv;
            s_u2[c * N3P + pv] = make_float2(uh, __fadd_rn(__fsub_rn(uf, uh), ulo));
          }
        }
      }
    }
    __syncthreads();
    // ---- upwind flux per face node, lifted, into s_F ------------------------
    // The partner values are parked in the dead FP64 staging area (each thread
    // reads back only what it wrote) to keep the flux's registers free.
    tid = opaque_tid();
    double* s_nbv = s_u64;
#pragma unroll
    for (int q = 0; q < FPT; ++q) {
      const int t = tid + q * NT;
      if (t < NF && nbr[t / N2] >= 0)
#pragma unroll
        for (int k = 0; k < NPC; ++k) s_nbv[k * NF + t] = nbv[q][k];
    }
#pragma unroll
    for (int q = 0; q < FPT; ++q) {
      const int t = tid + q * NT;
      if (t < NF) {
        const int f = t / N2, ab = t - f * N2;
        const int fa = ab % NX, fb = ab / NX;
        const int pv = pnode<NX>(face_vol<NX>(f, fa, fb));
        const int pe = nbr[f];
        float2 JH[3], JE[3];  // jumps partner - own as unevaluated pairs
        const int ax = slot_axis(f), ta = ax == 0 ? 1 : 0;  // the tangential axes ta < tb
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          if (!EXT && c == ax) {  // the normal component: not in the flux
            JH[c] = JE[c] = make_float2(0.0f, 0.0f);
            continue;
          }
          const float2 h = s_u2[c * N3P + pv], ev = s_u2[(c + 3) * N3P + pv];
          if (pe >= 0) {
            const int kh = EXT ? c : (c == ta ? 0 : 1), ke = EXT ? c + 3 : kh + 2;
            JH[c] = jump_pair(s_nbv[kh * NF + t], h);
            JE[c] = jump_pair(s_nbv[ke * NF + t], ev);
          } else {  // PEC mirror H+ = H-, E+ = -E-: [H] = 0, [E] = -2E exactly
            JH[c] = make_float2(0.0f, 0.0f);
            JE[c] = make_float2(-2.0f * ev.x, -2.0f * ev.y);
          }
          if (EXT && a.inc_elem) {
            // userinc: the incident field on the own side of a listed face
            // node, or on the partner's side when the partner's slot is listed
            const int io = a.inc_elem[e];
            if (io >= 0) {  // (FP64 differences: listed elements only)
              const double* iv = a.inc_val + (long)io * 12 * NF + t;
              if (pe >= 0) {
                add_jump(JH[c], iv[(6 + c) * NF] - iv[c * NF]);
                add_jump(JE[c], iv[(9 + c) * NF] - iv[(3 + c) * NF]);
              } else {
                add_jump(JE[c], -2.0 * iv[(3 + c) * NF]);
              }
            }
          }
        }
        if (EXT && a.gr.elem) {
          // graphene (userfsrc): the sheet's currents on both sides of the
          // face node enter as n x [H] - J, i.e. [H] + n x J (FP64)
          const int gr = a.gr.elem[e];
          const int go = gr >= 0 ? a.gr.own[(long)gr * NF + t] : -1;
          const int gp = gr >= 0 ? a.gr.part[(long)gr * NF + t] : -1;
          if (go >= 0 || gp >= 0) {
            double nv[3] = {0.0, 0.0, 0.0}, nm[3];
            nv[slot_axis(f)] = (double)slot_side(f);
            double fhm[3], fem[3], fhp[3], fep[3];
            const int io = a.inc_elem ? a.inc_elem[e] : -1;
            for (int c = 0; c < 3; ++c) {
              nm[c] = -nv[c];
              const float2 h = s_u2[c * N3P + pv], ev = s_u2[(c + 3) * N3P + pv];
              fhm[c] = f2d(h.x) + f2d(h.y);
              fem[c] = f2d(ev.x) + f2d(ev.y);
              fhp[c] = pe >= 0 ? s_nbv[c * NF + t] : 0.0;  // EXT: all six parked
              fep[c] = pe >= 0 ? s_nbv[(c + 3) * NF + t] : 0.0;
              if (io >= 0) {
                const double* iv = a.inc_val + (long)io * 12 * NF + t;
                fhm[c] += iv[c * NF];
                fem[c] += iv[(3 + c) * NF];
                fhp[c] += iv[(6 + c) * NF];
                fep[c] += iv[(9 + c) * NF];
              }
            }
            double J[3] = {0.0, 0.0, 0.0};
            if (go >= 0) graphene_slot(a.gr, go, nv, fhm, fem, true, first_stage, a.a, a.b, a.dt, J);
            if (gp >= 0 && pe >= 0) graphene_slot(a.gr, gp, nm, fhp, fep, false, first_stage, a.a, a.b, a.dt, J);
            if (pe >= 0) {  // a PEC face keeps its mirror flux
              add_jump(JH[0], nv[1] * J[2] - nv[2] * J[1]);
              add_jump(JH[1], nv[2] * J[0] - nv[0] * J[2]);
              add_jump(JH[2], nv[0] * J[1] - nv[1] * J[0]);
            }
          }
        }
        // coefficient pairs Y02, C02Y, Z02, C02Z (hi in the first float4 of
        // the face node, lo in the second)
        float2 Y02 = make_float2(-0.5f, 0.0f), C02Y = make_float2(0.5f * a.C0f, 0.0f);
        float2 Z02 = make_float2(0.5f, 0.0f), C02Z = C02Y;
        if (a.fcoef) {
          const float4* fc = reinterpret_cast<const float4*>(a.fcoef) + 2 * ((long)e * NF + t);
          const float4 hi = fc[0], lo = fc[1];
          Y02 = make_float2(hi.x, lo.x);
          C02Y = make_float2(hi.y, lo.y);
          Z02 = make_float2(hi.z, lo.z);
          C02Z = make_float2(hi.w, lo.w);
        }
        const float sg = (float)slot_side(f);
        const float2 sY = make_float2(sg * Y02.x, sg * Y02.y), sZ = make_float2(sg * Z02.x, sg * Z02.y);
        // lift factor area / (bm1 * 2/hx) at this face, as a pair
        const float2 lf = make_float2(eg[4 + f], eg[10 + f]);
        // the four tangential components, in the line slot order of the
        // face's direction (residuals 5,4,2,1 | 5,3,2,0 | 4,3,1,0)
        float2 F0, F1, F2, F3;
        switch (slot_axis(f)) {
          case 0:
            F0 = flux_pair(sZ, JH[1], C02Z, JE[2], lf);        // E3
            F1 = flux_pair(neg2(sZ), JH[2], C02Z, JE[1], lf);  // E2
            F2 = flux_pair(sY, JE[1], C02Y, JH[2], lf);        // H3
            F3 = flux_pair(neg2(sY), JE[2], C02Y, JH[1], lf);  // H2
            break;
          case 1:
            F0 = flux_pair(neg2(sZ), JH[0], C02Z, JE[2], lf);  // E3
            F1 = flux_pair(sZ, JH[2], C02Z, JE[0], lf);        // E1
            F2 = flux_pair(neg2(sY), JE[0], C02Y, JH[2], lf);  // H3
            F3 = flux_pair(sY, JE[2], C02Y, JH[0], lf);        // H1
            break;
          default:
            F0 = flux_pair(sZ, JH[0], C02Z, JE[1], lf);        // E2
            F1 = flux_pair(neg2(sZ), JH[1], C02Z, JE[0], lf);  // E1
            F2 = flux_pair(sY, JE[0], C02Y, JH[1], lf);        // H2
            F3 = flux_pair(neg2(sY), JE[1], C02Y, JH[0], lf);  // H1
            break;
        }
        float2* Fp = s_F + f * 4 * N2 + ab;
        Fp[0] = F0;
        Fp[N2] = F1;
        Fp[2 * N2] = F2;
        Fp[3 * N2] = F3;
      }
    }
    __syncthreads();
    // ---- contractions (and lift): r, s, t lines --------------------------------
    {
      const bool cubic = eg[0] == 1.0f && eg[1] == 0.0f && eg[2] == 1.0f && eg[3] == 0.0f;
      const float r1h = eg[0], r1l = eg[1], r2h = eg[2], r2l = eg[3];
      line_phase<NX, 0, false, TPL>(s_u2, s_R2, s_F, cubic, 0.0f, 0.0f, a, e, first_stage);
      __syncthreads();
      line_phase<NX, 1, false, TPL>(s_u2, s_R2, s_F, cubic, r1h, r1l, a, e, first_stage);
      __syncthreads();
      // without the extension terms each component can finish on its own
      // (MCfg::kFin): H3, E3 (no t-derivative) are complete since the s-lines
      line_phase<NX, 2, FIN, TPL>(s_u2, s_R2, s_F, cubic, r2h, r2l, a, e, first_stage);
    }
    if constexpr (FIN) {
      tid = opaque_tid();
      const int so = a.src_elem ? a.src_elem[e] : -1;
      constexpr int NPT2 = (2 * N3 + NT - 1) / NT;
#pragma unroll
      for (int q = 0; q < NPT2; ++q) {
        const int w = tid + q * NT;
        if (w < 2 * N3) {
          const int c = w < N3 ? 2 : 5;
          const int v = w < N3 ? w : w - N3;
          const float2 rr = s_R2[c * N3P + pnode<NX>(v)];
          float Rh = rr.x, Rl = rr.y;
          if (c == 5 && so >= 0) add_pair_product(Rh, Rl, a.src_w[(long)so * N3 + v], a.src_ft2);
          rk_finish<C::kIntAdd>(a, c, (long)e * N3 + v, Rh, Rl, first_stage);
        }
      }
      __syncthreads();  // the split pairs are consumed: the next element may land
      if (C::kTma && tid == 0 && en < a.e_end) {
        fence_proxy_async_smem();
        issue_tma(en, buf ^ 1);
      }
      if (C::kAsync && en < a.e_end) issue_async(en, buf ^ 1, tid);
    } else {
      tid = opaque_tid();
      __syncthreads();
      // the split pairs are consumed: the next element's state lands in their
      // area while this one finishes (the next element's own barriers order
      // these reads of the residual pairs before its split overwrites them)
      if (C::kTma && tid == 0 && en < a.e_end) {
        fence_proxy_async_smem();
        issue_tma(en, buf ^ 1);
      }
      if (C::kAsync && en < a.e_end) issue_async(en, buf ^ 1, tid);
      // ---- source, inverse mass, RK update ----------------------------------------
      // All six components of a node at once (the PML and dispersive terms
      // couple them to the node's auxiliary fields).
      const int so = a.src_elem ? a.src_elem[e] : -1;
      const int pml_l = (EXT && a.pml.slot) ? a.pml.slot[e] : -1;
      const int disp_l = (EXT && a.disp.slot) ? a.disp.slot[e] : -1;
#pragma unroll
      for (int q = 0; q < NPT; ++q) {
        const int v = tid + q * NT;
        if (v >= N3) continue;
        if (C::kPfNode && q + 1 < NPT && v + NT < N3) {  // the next node's loads into L1 meanwhile
          const long g2 = (long)e * N3 + v + NT;
#pragma unroll
          for (int c = 0; c < 6; ++c) {
            if (!first_stage) prefetch_l1(a.k + c * P + g2);
            prefetch_l1(a.u_in + c * P + g2);
          }
        }
        const int pv = pnode<NX>(v);
        float Rh[6], Rl[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) {
          const float2 rr = s_R2[c * N3P + pv];
          Rh[c] = rr.x;
          Rl[c] = rr.y;
        }
        if (EXT && pml_l >= 0) pml_node<N3>(a, pml_l, v, (long)e * N3 + v, first_stage, Rh, Rl);
        if (EXT && disp_l >= 0) disp_node<N3>(a, disp_l, v, (long)e * N3 + v, first_stage, Rh, Rl);
        if (so >= 0) add_pair_product(Rh[5], Rl[5], a.src_w[(long)so * N3 + v], a.src_ft2);
        // the node's two coefficient pairs, H and E, once for its six components
        const long g = (long)e * N3 + v;
        const float2 cfH = a.coef[g], cfE = a.coef[P + g];
        rk_finish_node<C::kIntAdd>(a, g, Rh, Rl, cfH, cfE, first_stage);
      }
    }
  }
}

// dt-scaled inverse-mass coefficients as float pairs: (hi, lo) of dt * base,
// hi = the top 24 mantissa bits, lo = the rest (2*n entries)
__global__ void k_scale_coef_pairs(float2* coef, const double* base, long n2, double dt) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n2) return;
  const double v = dt * base[i];
  coef[i] = make_float2(d2f_hi(v), d2f_lo(v));
}

template <int NX, bool EXT, int TPL = 1>
int launch_mixed(Context* c, const MixedDev& a, bool pdl) {
  using C = MCfg<NX, TPL>;
  auto kern = k_mixed_stage<NX, EXT, TPL>;
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
  const int n = a.e_end - a.e_begin;
  if (n <= 0) return NEKGPU_OK;
  const int g = n < grid ? n : grid;
  c->fused_grid = g;
  if (pdl) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(g);
    cfg.blockDim = dim3(C::NT);
    cfg.dynamicSmemBytes = C::smem;
    cfg.stream = c->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (check_cuda(cudaLaunchKernelEx(&cfg, kern, a))) return NEKGPU_ERR_CUDA;
  } else {
    kern<<<g, C::NT, C::smem, c->stream>>>(a);
  }
  c->last_launches += 1;
  return check_cuda(cudaGetLastError());
}

// ===========================================================================
// Mixed stage on curvilinear hexahedra (NEKGPU_MIXED on a mesh whose metrics
// vary inside the elements): the general weighted curl with the nine
// per-node metrics (maxwell_wght_curl, src/cem_maxwell.F:1428-1497), the
// upwind flux with per-face-node normals and areas (cem_maxwell_flux3d,
// src/cem_maxwell.F:922-1002) and the partner's values read directly, lift,
// volume source, inverse mass and RK update -- the arrays of the curved FP64
// form (CurvedDev), converted to float pairs on the fly by integer
// operations.  The derivatives are exact-hi FP32 contractions as in the
// affine kernel (the element's 10-bit grid per component, D in its Dh, Df,
// Dm pieces); metrics, weights, normals, areas, face coefficients, source
// weights and the inverse mass enter as float pairs in float-float
// arithmetic; the RK update is FP64.  One block of NX^3 threads per element
// (thread per node); the state of the thread's node stays in registers.
// ===========================================================================
struct PairF {
  float h, l;
};
__device__ __forceinline__ PairF pr(double d) { return PairF{d2f_hi(d), d2f_lo(d)}; }
__device__ __forceinline__ PairF pmul(PairF a, PairF b) {
  const float p = a.h * b.h;
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return PairF{p, e};
}
__device__ __forceinline__ PairF padd(PairF a, PairF b) {
  float s, t;
  two_sum(a.h, b.h, s, t);
  return PairF{s, (a.l + b.l) + t};
}
__device__ __forceinline__ PairF pneg(PairF a) { return PairF{-a.h, -a.l}; }
__device__ __forceinline__ PairF psub(PairF a, PairF b) { return padd(a, pneg(b)); }
// a x b for pair 3-vectors
__device__ __forceinline__ void pcross(const PairF* a, const PairF* b, PairF* o) {
  o[0] = psub(pmul(a[1], b[2]), pmul(a[2], b[1]));
  o[1] = psub(pmul(a[2], b[0]), pmul(a[0], b[2]));
  o[2] = psub(pmul(a[0], b[1]), pmul(a[1], b[0]));
}

template <int NX>
struct CMCfg {
  static constexpr int N2 = NX * NX, N3 = N2 * NX, NF = 6 * N2;
  static constexpr int NT = (N3 + 31) / 32 * 32, NW = NT / 32;
  static constexpr size_t off_F = 6 * (size_t)N3 * 8;            // float2 split pairs [c][v]
  static constexpr size_t off_D = off_F + 6 * (size_t)NF * 8;    // float2 flux pairs [c][face node]
  static constexpr size_t off_Dm = off_D + (size_t)N2 * 8;       // (Dh, Df) [i + NX l]
  static constexpr size_t off_wmax = off_Dm + (size_t)N2 * 4;    // Dm [i + NX l]
  static constexpr size_t off_E = off_wmax + NW * 6 * 4;
  static constexpr size_t smem = off_E + 8 * 4;
};

template <int NX>
__global__ void __launch_bounds__(CMCfg<NX>::NT, 1) k_mixed_curved(const CurvedDev a) {
  using C = CMCfg<NX>;
  constexpr int N2 = C::N2, N3 = C::N3, NF = C::NF, NT = C::NT;
  extern __shared__ __align__(16) unsigned char smem[];
  float2* s_u2 = reinterpret_cast<float2*>(smem);
  float2* s_F = reinterpret_cast<float2*>(smem + C::off_F);
  float2* s_Dhf = reinterpret_cast<float2*>(smem + C::off_D);
  float* s_Dm = reinterpret_cast<float*>(smem + C::off_Dm);
  unsigned* s_wmax = reinterpret_cast<unsigned*>(smem + C::off_wmax);
  unsigned* s_E = reinterpret_cast<unsigned*>(smem + C::off_E);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long P = a.npts;
  const bool node = tid < N3;
  const int vi = tid % NX, vj = (tid / NX) % NX, vk = tid / N2;
  const bool first_stage = (a.a == 0.0);
  constexpr int H = (NX + 1) / 2;
  for (int t = tid; t < N2; t += NT) {
    const int i = t % NX, l = t / NX;
    s_Dhf[t] = c_mixD[NX][0][t];
    const float2 m = c_mixD[NX][1][i / 2 + H * l];
    s_Dm[t] = (i & 1) ? m.y : m.x;
  }
  for (int e = blockIdx.x; e < a.nelt; e += gridDim.x) {
    __syncthreads();  // the previous element's shared data is consumed
    const long g = (long)e * N3 + tid;
    double u[6];
    unsigned em[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      u[c] = node ? a.u_in[c * P + g] : 0.0;
      em[c] = ((unsigned)__double2hiint(u[c]) >> 20) & 0x7FFu;
      em[c] = __reduce_max_sync(0xffffffffu, em[c]);
    }
    if (lane == 0)
#pragma unroll
      for (int c = 0; c < 6; ++c) s_wmax[warp * 6 + c] = em[c];
    __syncthreads();
    if (tid < 6) {
      unsigned m = 0;
      for (int w = 0; w < C::NW; ++w) m = max(m, s_wmax[w * 6 + tid]);
      s_E[tid] = min(max(m, 906u), 1158u);
    }
    __syncthreads();
    if (node) {  // split: uh on the element's 10-bit grid of the component, ul = u - uh
      const float M = 12582912.0f;
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const int E = (int)s_E[c];
        const float qv = __int_as_float((E - 905) << 23);
        const float qi = __int_as_float((1159 - E) << 23);
        const float uf = d2f_hi(u[c]), ulo = d2f_lo(u[c]);
        const float uh = (__fadd_rn(__fmaf_rn(uf, qi, M), -M)) * qv;
        s_u2[c * N3 + tid] = make_float2(uh, __fadd_rn(__fsub_rn(uf, uh), ulo));
      }
    }
    __syncthreads();
    // ---- upwind flux per face node, float pairs ---------------------------
    for (int t = tid; t < NF; t += NT) {
      const int f = t / N2, ab = t - f * N2;
      const int v = face_vol<NX>(f, ab % NX, ab / NX);
      const long js = (long)e * NF + t, L = a.nxzfl;
      const int pv = a.partner[js];
      PairF JH[3], JE[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float2 h = s_u2[c * N3 + v], ev = s_u2[(c + 3) * N3 + v];
        if (pv >= 0) {
          const float2 jh = jump_pair(a.u_in[c * P + pv], h), je = jump_pair(a.u_in[(c + 3) * P + pv], ev);
          JH[c] = PairF{jh.x, jh.y};
          JE[c] = PairF{je.x, je.y};
        } else {  // PEC mirror: [H] = 0, [E] = -2E exactly
          JH[c] = PairF{0.0f, 0.0f};
          JE[c] = PairF{-2.0f * ev.x, -2.0f * ev.y};
        }
      }
      const PairF n[3] = {pr(a.face[js]), pr(a.face[L + js]), pr(a.face[2 * L + js])};
      const PairF area = pr(a.face[3 * L + js]);
      PairF Y02{-0.5f, 0.0f}, C02Y{0.5f, 0.0f}, Z02{0.5f, 0.0f}, C02Z{0.5f, 0.0f};
      if (a.fcoef) {
        Y02 = pr(a.fcoef[js]); C02Y = pr(a.fcoef[L + js]);
        Z02 = pr(a.fcoef[2 * L + js]); C02Z = pr(a.fcoef[3 * L + js]);
      }
      // n x [E], n x [H] (the gs sums of -n x E, -n x H), then the upwind terms
      PairF nE[3], nH[3], fu[3], fw[3];
      pcross(n, JE, nE);
      pcross(n, JH, nH);
      pcross(n, nH, fu);
      pcross(n, nE, fw);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const PairF fh = pmul(area, psub(pmul(Y02, nE[c]), pmul(C02Y, fu[c])));
        const PairF fe = pmul(area, psub(pmul(Z02, nH[c]), pmul(C02Z, fw[c])));
        s_F[c * NF + t] = make_float2(fh.h, fh.l);
        s_F[(3 + c) * NF + t] = make_float2(fe.h, fe.l);
      }
    }
    __syncthreads();
    if (!node) continue;
    // ---- derivatives (exact-hi contractions) and the weighted curl -----------
    // d_dir u_c at the node as a pair: hi = sum Dh uh (exact), lo = the rest
    auto deriv = [&](int c, int dir) {
      const float2* pu = s_u2 + c * N3;
      const int row = dir == 0 ? vi : (dir == 1 ? vj : vk);
      float2 x = make_float2(0.0f, 0.0f);
      float m = 0.0f;
#pragma unroll
      for (int l = 0; l < NX; ++l) {
        const int q = dir == 0 ? l + NX * vj + N2 * vk
                               : (dir == 1 ? vi + NX * l + N2 * vk : vi + NX * vj + N2 * l);
        const float2 uu = pu[q];
        x = __ffma2_rn(s_Dhf[row + NX * l], uu, x);
        m = fmaf(s_Dm[row + NX * l], uu.x, m);
      }
      return PairF{x.x, x.y + m};
    };
    // curl_k = eps(k, ax, q) d u_q / d x_ax with d/dx_ax = sum_dir metric(dir, ax) d/d_dir,
    // accumulated direction by direction (one row of D live at a time): the
    // two axes other than q give
    //   w[(q+2)%3] -= metric(dir, (q+1)%3) du_q/d_dir,  w[(q+1)%3] += metric(dir, (q+2)%3) du_q/d_dir
    PairF w[6] = {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f},
                  {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}};  // curl H, curl E
#pragma unroll
    for (int dir = 0; dir < 3; ++dir) {
      const PairF m3[3] = {pr(a.metrics[(3 * dir) * P + g]), pr(a.metrics[(3 * dir + 1) * P + g]),
                           pr(a.metrics[(3 * dir + 2) * P + g])};  // r|s|t x, y, z
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const int q = c % 3, o = c - q;
        const PairF d = deriv(c, dir);
        w[o + (q + 2) % 3] = psub(w[o + (q + 2) % 3], pmul(d, m3[(q + 1) % 3]));
        w[o + (q + 1) % 3] = padd(w[o + (q + 1) % 3], pmul(d, m3[(q + 2) % 3]));
      }
    }
    const PairF w3 = pr(a.w3[tid]);
    PairF res[6];  // resH = -W curl E, resE = W curl H
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      res[q] = pneg(pmul(w3, w[3 + q]));
      res[3 + q] = pmul(w3, w[q]);
    }
    // ---- lift in face-slot order ---------------------------------------------
    auto add = [&](int f, int ab) {
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const float2 F = s_F[c * NF + f * N2 + ab];
        res[c] = padd(res[c], PairF{F.x, F.y});
      }
    };
    if (vj == 0) add(0, vi + NX * vk);
    if (vi == NX - 1) add(1, vj + NX * vk);
    if (vj == NX - 1) add(2, vi + NX * vk);
    if (vi == 0) add(3, vj + NX * vk);
    if (vk == 0) add(4, vi + NX * vj);
    if (vk == NX - 1) add(5, vi + NX * vj);
    // ---- volume source (usersrc), mass-weighted ----------------------------------
    if (a.src_elem) {
      const int so = a.src_elem[e];
      if (so >= 0) res[5] = padd(res[5], pmul(pr(a.src_w[(long)so * N3 + tid]), pr(a.src_ft)));
    }
    // ---- inverse mass (pair product, one DADD) and the FP64 RK update ------------
    const PairF ch = pr(a.coef[g]), ce = pr(a.coef[P + g]);
    double kk[6], uu[6];  // all twelve loads before the stores (k may be read and written)
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      kk[c] = first_stage ? 0.0 : a.k[c * P + g];
      uu[c] = a.u_in[c * P + g];
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      const PairF p = pmul(res[c], c < 3 ? ch : ce);
      const double r = f2d(p.h) + f2d(p.l);
      const double kn = first_stage ? r : fma(a.a, kk[c], r);
      a.k[c * P + g] = kn;
      a.u_out[c * P + g] = fma(a.b, kn, uu[c]);
    }
  }
}

template <int NX>
int launch_mixed_curved(Context* c, const CurvedDev& a) {
  using C = CMCfg<NX>;
  static int grid = 0;
  if (!grid) {
    if (check_cuda(cudaFuncSetAttribute(k_mixed_curved<NX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)C::smem)))
      return NEKGPU_ERR_CUDA;
    int per_sm = 0, sms = 0;
    if (check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mixed_curved<NX>, C::NT, C::smem)))
      return NEKGPU_ERR_CUDA;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    if (per_sm < 1) return NEKGPU_ERR_UNSUPPORTED;
    grid = per_sm * sms;
  }
  const int g = c->nelt < grid ? c->nelt : grid;
  k_mixed_curved<NX><<<g, C::NT, C::smem, c->stream>>>(a);
  c->last_launches += 1;
  return check_cuda(cudaGetLastError());
}

// The bounded wait run out on purpose: an mbarrier that nothing arrives at,
// polled `polls` times, then the status word is set as a stage kernel sets it
// when its copy never lands.  No fault, no trap, no endless loop.
__global__ void k_wait_selftest(int polls, int* status) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  bool done = false;
  for (int it = 0; it < polls && !done; ++it) done = mbar_try_wait(&bar, 0);
  if (!done && threadIdx.x == 0) atomicExch(status, 1);
}

// pair_to_double over arrays (self-test of the finish's integer join)
__global__ void k_pair_join(const float* s, const float* t, double* out, long n) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = pair_to_double(s[i], t[i]);
}

}  // namespace

int pair_join_selftest(const float* s, const float* t, double* out, long n) {
  k_pair_join<<<(unsigned)((n + 255) / 256), 256>>>(s, t, out, n);
  return check_cuda(cudaGetLastError());
}

int wait_selftest(Context* c, int polls) {
  k_wait_selftest<<<1, 32, 0, c->stream>>>(polls, c->d_status);
  c->last_launches += 1;
  return check_cuda(cudaGetLastError());
}

int mixed_upload_D(int nx, const float* tab, size_t count) {
  static bool done[kMaxMixed + 1] = {false};
  constexpr size_t kCount = 2 * 2 * kMaxMixed * kMaxMixed;  // floats per nx
  if (nx < 2 || nx > kMaxMixed || count != kCount) return NEKGPU_ERR_UNSUPPORTED;
  if (done[nx]) return NEKGPU_OK;
  if (check_cuda(cudaMemcpyToSymbol(c_mixD, tab, sizeof(float) * kCount, sizeof(float) * kCount * nx)))
    return NEKGPU_ERR_CUDA;
  done[nx] = true;
  return NEKGPU_OK;
}

int scale_coef_pairs(Context* c, double dt) {
  if (c->coef_dt == dt) return NEKGPU_OK;
  const long n2 = 2 * c->npts;
  k_scale_coef_pairs<<<(unsigned)((n2 + 255) / 256), 256, 0, c->stream>>>(
      reinterpret_cast<float2*>(c->d_coef), c->d_cbase, n2, dt);
  c->last_launches += 1;
  c->coef_dt = dt;
  return check_cuda(cudaGetLastError());
}

int num_sms(Context* c) {
  static int n = 0;
  if (!n) {
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess) {
      cudaGetLastError();
      n = 1;
    }
  }
  return n;
}

int mixed_stage_range(Context* c, int rkstep, double time, double dt, int e0, int e1, bool pdl) {
  int st = scale_coef_pairs(c, dt);
  if (st) return st;
  MixedDev a = c->margs;
  a.e_begin = e0;
  a.e_end = e1;
  a.u_in = c->d_u[c->cur];
  a.u_out = c->d_u[c->cur ^ 1];
  a.a = c->rk_a[rkstep - 1];
  a.b = c->rk_b[rkstep - 1];
  a.dt = dt;
  if (c->src.enabled) {
    const double ft = source_ft(c->src, time + dt * c->rk_c[rkstep - 1]);
    const float hi = (float)ft;
    a.src_ft2 = make_float2(hi, (float)(ft - (double)hi));
  }
  const bool ext = a.pml.slot || a.disp.slot || a.inc_elem || a.gr.elem;
  if (a.inc_elem && (st = incident_upload(c, time + dt * c->rk_c[rkstep - 1]))) return st;
  if (a.gr.elem) {
    a.gr.f_in = c->d_gr_f[c->gr_cur];
    a.gr.f_out = c->d_gr_f[c->gr_cur ^ 1];
  }
  switch (c->nx) {
    case 3: st = ext ? launch_mixed<3, true>(c, a, pdl) : launch_mixed<3, false>(c, a, pdl); break;
    case 4: st = ext ? launch_mixed<4, true>(c, a, pdl) : launch_mixed<4, false>(c, a, pdl); break;
    case 5: st = ext ? launch_mixed<5, true>(c, a, pdl) : launch_mixed<5, false>(c, a, pdl); break;
    case 6: st = ext ? launch_mixed<6, true>(c, a, pdl) : launch_mixed<6, false>(c, a, pdl); break;
    case 7: st = ext ? launch_mixed<7, true>(c, a, pdl) : launch_mixed<7, false>(c, a, pdl); break;
    case 8:
      // fewer elements than SMs: two threads per line (one element per SM
      // either way; the element's latency is the stage's time)
      st = ext ? launch_mixed<8, true>(c, a, pdl)
               : (e1 - e0 <= num_sms(c) ? launch_mixed<8, false, 2>(c, a, pdl)
                                         : launch_mixed<8, false>(c, a, pdl));
      break;
    case 9: st = ext ? launch_mixed<9, true>(c, a, pdl) : launch_mixed<9, false>(c, a, pdl); break;
    default: return NEKGPU_ERR_UNSUPPORTED;
  }
  return st;
}

// One mixed stage on a curvilinear mesh (the curved form's arrays, FP64
// coefficients scaled once per dt).
int mixed_curved_stage(Context* c, int rkstep, double time, double dt) {
  int st = scale_coef(c, dt);
  if (st) return st;
  CurvedDev a = c->cargs;
  a.u_in = c->d_u[c->cur];
  a.u_out = c->d_u[c->cur ^ 1];
  a.a = c->rk_a[rkstep - 1];
  a.b = c->rk_b[rkstep - 1];
  a.src_elem = c->fargs.src_elem;
  a.src_w = reinterpret_cast<const double*>(c->fargs.src_w);
  a.vres = nullptr;
  if (c->src.enabled) a.src_ft = source_ft(c->src, time + dt * c->rk_c[rkstep - 1]);
  switch (c->nx) {
    case 3: st = launch_mixed_curved<3>(c, a); break;
    case 4: st = launch_mixed_curved<4>(c, a); break;
    case 5: st = launch_mixed_curved<5>(c, a); break;
    case 6: st = launch_mixed_curved<6>(c, a); break;
    case 7: st = launch_mixed_curved<7>(c, a); break;
    case 8: st = launch_mixed_curved<8>(c, a); break;
    default: return NEKGPU_ERR_UNSUPPORTED;
  }
  if (st) return st;
  c->cur ^= 1;
  return NEKGPU_OK;
}

int mixed_scale_pairs(Context* c, float2* coef, const double* base, long n2, double dt) {
  k_scale_coef_pairs<<<(unsigned)((n2 + 255) / 256), 256, 0, c->stream>>>(coef, base, n2, dt);
  c->last_launches += 1;
  return check_cuda(cudaGetLastError());
}

int mixed_stage_buffers(Context* c, int rkstep, double time, double dt, const double* u_in,
                        double* u_out, double* k_in, double* k_out) {
  const int st = scale_coef_pairs(c, dt);
  if (st) return st;
  return mixed_stage_dev(c, c->margs, rkstep, time, dt, u_in, u_out, k_in, k_out);
}

int mixed_stage_dev(Context* c, MixedDev a, int rkstep, double time, double dt, const double* u_in,
                    double* u_out, double* k_in, double* k_out) {
  if (a.pml.slot || a.disp.slot || a.inc_elem || a.gr.elem) return NEKGPU_ERR_UNSUPPORTED;
  a.e_begin = 0;
  a.e_end = c->nelt;
  a.u_in = u_in;
  a.u_out = u_out;
  a.k = k_in;
  a.k_out = k_out;
  a.a = c->rk_a[rkstep - 1];
  a.b = c->rk_b[rkstep - 1];
  a.dt = dt;
  if (c->src.enabled) {
    const double ft = source_ft(c->src, time + dt * c->rk_c[rkstep - 1]);
    const float hi = (float)ft;
    a.src_ft2 = make_float2(hi, (float)(ft - (double)hi));
  }
  switch (c->nx) {
    case 3: return launch_mixed<3, false>(c, a, false);
    case 4: return launch_mixed<4, false>(c, a, false);
    case 5: return launch_mixed<5, false>(c, a, false);
    case 6: return launch_mixed<6, false>(c, a, false);
    case 7: return launch_mixed<7, false>(c, a, false);
    case 8: return launch_mixed<8, false>(c, a, false);
    case 9: return launch_mixed<9, false>(c, a, false);
    default: return NEKGPU_ERR_UNSUPPORTED;
  }
}

int mixed_stage(Context* c, int rkstep, double time, double dt) {
  const int st = mixed_stage_range(c, rkstep, time, dt, 0, c->nelt, true);
  if (st) return st;
  c->cur ^= 1;
  if (c->margs.gr.elem) c->gr_cur ^= 1;
  return NEKGPU_OK;
}

}  // namespace nekgpu
