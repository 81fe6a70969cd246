// od_common.cuh — device-side definitions shared by the superion step kernels.
//
// Units on the device: length lambda = r_D_e, time d_t, so a leapfrog half kick is
// v += 0.5*a and a drift is x += v. Ion state is FP32 (float4 SoA: pos, vel);
// grain charges, sums, series and averages are FP64.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/opendust_gb300.h"

#define OD_PI_D 3.14159265358979323846
#define OD_TJ 256              // source positions per shared-memory tile
#define OD_PAD 512             // ion arrays are padded to a multiple of this
#define OD_SENTINEL 1.0e4f     // padded sources sit here: exp(-r) underflows to 0
#define OD_WAIT_LIMIT (1u << 26)

// Device error word bits (reported by the host as OD_ERR_TIMEOUT / OD_ERR_STATE)
#define OD_DERR_TIMEOUT 1u
#define OD_DERR_LIST 2u
#define OD_DERR_CELL 4u            // a cell holds more ions than the in-block sort takes

// Per-simulation constants, resident in device memory.
struct od_dparams {
  int32_t N, Npad, P, dist, coll, method, sim, nwords;
  uint32_t seed_lo, seed_hi;
  int32_t force_every;               // ion–ion force interval k (1: every step)
  int32_t ion0;                      // global index of local ion 0 (a shard of a larger run; 0)
  // integer forms of u < Pmax (u < pmax_int 2^-24) and u <= p_coll (u <= pcoll_int 2^-24;
  // -1: never) for u = (w >> 8) 2^-24
  uint32_t pmax_int;
  int32_t pcoll_int;
  // FP32 hot-loop constants (lambda / d_t units)
  float A_ii, rho0, Rh, Hh, Hh_half, a_field, vT, vfl;
  float rc2, rc, rs, inv_w;          // cutoff^2, cutoff, switch start, 1/(rc-rs)
  float trapc[15];                   // -2*A_ii*alpha[k]
  float A_id;                        // ion–dust prefactor, times q_p
  double A_id_d;                     // same in FP64
  float gxh[OD_MAX_GRAINS], gxl[OD_MAX_GRAINS];  // grain centres as two-float
  float gyh[OD_MAX_GRAINS], gyl[OD_MAX_GRAINS];
  float gzh[OD_MAX_GRAINS], gzl[OD_MAX_GRAINS];
  float gr2f[OD_MAX_GRAINS];
  float Rh2f, Hz_f;
  float mfp_inv, vmax_mfp;
  float rel_s, rel_inv;              // cell side of the cell-relative positions (a power of two)
  // FP64 exact-flag constants (identical doubles in the CPU oracle)
  double gx[OD_MAX_GRAINS], gy[OD_MAX_GRAINS], gz[OD_MAX_GRAINS], gr2[OD_MAX_GRAINS];
  double Rh2, Hh_half_d;
  double p_coll, Pmax_mfp, mfp_inv_d, p_t, p_s, p_b;
  // injection tables (lambda/d_t units for v and slope)
  int32_t tn[OD_NTAB];
  float tv[OD_NTAB][OD_MAX_TABLE];
  double txi[OD_NTAB][OD_MAX_TABLE];
  float tsl[OD_NTAB][OD_MAX_TABLE];
  // FP64 tail constants (SI)
  double k, q_s, m_s, lam, dt, vunit, n_inf, T_e, T_n, k_B, m_e, e, E, v_T_si, v_fl_si;
  double alpha[15];
  double gxs[OD_MAX_GRAINS], gys[OD_MAX_GRAINS], gzs[OD_MAX_GRAINS], grs[OD_MAX_GRAINS];
  int32_t gmethod[OD_MAX_GRAINS];
  int64_t n_steps, avg_start;
  // external field of order 2 (chains/matthews.py:481-495) in acceleration units:
  // a_z = fa0 + fa1 zc + fa2 zc^2 with zc = z clamped to [fz1, fz7]
  int32_t field_order, trap_kind;
  float fa0, fa1, fa2, fz1, fz7;
  // tabulated trap (OD_TRAP_TABLE): knots th0 + j*tdh, j < ttn, on [th0, th1] (lambda);
  // tcf[k][j] = -A_ii times the natural-cubic-spline coefficients (c0..c3 in powers of h - h_j)
  // of alpha_k on [h_j, h_j+1]
  int32_t ttn;
  float th0, th1, tdh, tinv_dh;
  float tcf[5][OD_MAX_TRAP][4];
  // FP64 tail factors: field at each grain [V/m] and out-of-domain trap force per unit
  // charge [N/C] (OD_TRAP_TABLE)
  double gfield[OD_MAX_GRAINS];
  double gout[OD_MAX_GRAINS][3];
  // per-grain constants of the FP64 tail, precomputed on the host (tail_consts): the electron
  // term of the charge update is ge_pref exp(ge_arg q), the OML ion term oml_a + oml_b q; the
  // dust–dust force on grain g is q_g sum_j q_j dd[g][j] (N/C^2)
  double ge_pref[OD_MAX_GRAINS], ge_arg[OD_MAX_GRAINS], oml_a[OD_MAX_GRAINS], oml_b[OD_MAX_GRAINS];
  double dd[OD_MAX_GRAINS][OD_MAX_GRAINS][3];
};

// Per-simulation FP64 accumulators and bookkeeping, resident in device memory.
struct od_dstate {
  int64_t step;                       // next step index (series row) of the current window
  int64_t rng_base;                   // Philox step counter of series row 0 (windows)
  uint32_t err;                       // OD_DERR_* bits
  int32_t nlist;                      // flagged ions this step
  double q_param[OD_MAX_GRAINS];      // charges the ion forces use (q at the previous step)
  double dN[OD_MAX_GRAINS];           // ions collected this step
  double M[OD_MAX_GRAINS][3];         // sum of collected velocities (lambda/d_t)
  double avg[OD_MAX_GRAINS][13];      // running sums over the averaging window
  int64_t n_avg;
  int64_t n_inj_total;
  uint32_t ticket;                    // orbit blocks of K5 done this step (0 between steps)
};

// ------------------------------------------------------------------ Philox4x32-10
struct od_u4 { uint32_t x, y, z, w; };

__device__ __forceinline__ od_u4 od_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                           uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
  }
  return od_u4{c0, c1, c2, c3};
}
__device__ __forceinline__ od_u4 od_draw(const od_dparams& p, uint32_t ion, uint32_t step,
                                         uint32_t stream) {
  return od_philox(ion, step, stream, (uint32_t)p.sim, p.seed_lo, p.seed_hi);
}
__device__ __forceinline__ float od_u01(uint32_t w) { return (float)(w >> 8) * (1.0f / 16777216.0f); }
__device__ __forceinline__ float od_u01c(uint32_t w) {
  return (float)((w >> 8) + 1u) * (1.0f / 16777216.0f);
}
__device__ __forceinline__ void od_gauss2(uint32_t a, uint32_t b, float& g0, float& g1) {
  float r = sqrtf(-2.0f * logf(od_u01c(a)));
  float s, c;
  sincospif(2.0f * od_u01(b), &s, &c);
  g0 = r * c;
  g1 = r * s;
}

// ------------------------------------------------------------------ SFU approximations
__device__ __forceinline__ float od_rsqrt(float x) {
  float r; asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x)); return r;
}
__device__ __forceinline__ float od_rcp(float x) {
  float r; asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x)); return r;
}
__device__ __forceinline__ float od_ex2(float x) {
  float r; asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x)); return r;
}
#define OD_NLOG2E (-1.4426950408889634f)

// ------------------------------------------------------------------ packed f32x2 arithmetic
// Blackwell executes two FP32 lanes per instruction with the f32x2 forms of add/sub/mul/fma.
typedef unsigned long long od_u64;
__device__ __forceinline__ od_u64 p2(float lo, float hi) {
  od_u64 r; asm("mov.b64 %0, {%1,%2};" : "=l"(r) : "f"(lo), "f"(hi)); return r;
}
__device__ __forceinline__ float2 up2(od_u64 v) {
  float2 r; asm("mov.b64 {%0,%1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v)); return r;
}
__device__ __forceinline__ od_u64 fma2(od_u64 a, od_u64 b, od_u64 c) {
  od_u64 d; asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c)); return d;
}
__device__ __forceinline__ od_u64 add2(od_u64 a, od_u64 b) {
  od_u64 d; asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b)); return d;
}
__device__ __forceinline__ od_u64 sub2(od_u64 a, od_u64 b) {
  od_u64 d; asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b)); return d;
}
__device__ __forceinline__ od_u64 mul2(od_u64 a, od_u64 b) {
  od_u64 d; asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b)); return d;
}


__device__ __forceinline__ float sum2(od_u64 v) {
  const float2 f = up2(v);
  return f.x + f.y;
}

// ------------------------------------------------------------------ two-float sums
// Knuth TwoSum: hi + lo == a + b exactly.
__device__ __forceinline__ void od_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// accumulate x into (hi, lo)
__device__ __forceinline__ void od_acc2(float& hi, float& lo, float x) {
  float s, e;
  od_two_sum(hi, x, s, e);
  hi = s;
  lo = __fadd_rn(lo, e);
}

// ------------------------------------------------------------------ fixed-point sums
// The each-pair-once kernels add every (tile pair, ion) partial sum to the ion's accumulator
// with a 64-bit integer atomic: the value in units of 2^-32 (lambda units of the pair sums;
// per-ion sums are 10^0..10^5 and single terms at most ~1/r0^2 = 1e6, far inside the 2^31
// range). Integer addition is associative, so the result is the same bits for any order of
// the atomics; each partial (hi + lo) is rounded once per word, 2^-32 at most, against the
// two-float partial's own rounding of ~1e-7 of its size.
#define OD_FIX_SCALE 4294967296.0f          // 2^32
#define OD_FIX_INV 2.3283064365386963e-10   // 2^-32
#define OD_FIX_INV_F 2.3283064365386963e-10f
__device__ __forceinline__ unsigned long long od_fix(float hi, float lo) {
  return (unsigned long long)(__float2ll_rn(hi * OD_FIX_SCALE) + __float2ll_rn(lo * OD_FIX_SCALE));
}
__device__ __forceinline__ void od_fix_add(unsigned long long* a, float hi, float lo) {
  atomicAdd(a, od_fix(hi, lo));
}
// accumulator (3 words, component stride `stride`) -> two-float sums, and the words cleared for
// the next evaluation
// (FP32 only: FP64 is slow on GB300.) A word x is H + M 2^-16 + L 2^-32 with H = x >> 32
// (signed, exact in FP32 for |H| < 2^24) and M, L its two low 16-bit halves, each exact in FP32;
// the two-float sum is TwoSum(H, M 2^-16) with L 2^-32 added to the low part.
__device__ __forceinline__ void od_fix_split(unsigned long long x, float& hi, float& lo) {
  const float h = (float)(int)((long long)x >> 32);  // arithmetic shift: floor(x / 2^32)
  const float m = (float)(unsigned)((x >> 16) & 0xFFFFull) * 1.52587890625e-05f;  // 2^-16
  const float l = (float)(unsigned)(x & 0xFFFFull) * OD_FIX_INV_F;
  od_two_sum(h, m, hi, lo);
  lo += l;
}
__device__ __forceinline__ void od_fix_take(unsigned long long* a, size_t stride, float3& hi,
                                           float3& lo) {
  const unsigned long long x = a[0], y = a[stride], z = a[2 * stride];
  a[0] = 0ull; a[stride] = 0ull; a[2 * stride] = 0ull;
  od_fix_split(x, hi.x, lo.x);
  od_fix_split(y, hi.y, lo.y);
  od_fix_split(z, hi.z, lo.z);
}

// ------------------------------------------------------------------ pair kernel
// Radial factor c(r) of the Yukawa pair force: the acceleration on i from j is
// A_ii * c * (x_i - x_j), c = exp(-r) (1/s + 1/s^2) / r, s = r + rho0 (opendust.py:472).
// r2 carries +1e-30 so that the self pair (dx = 0) contributes exactly zero.
__device__ __forceinline__ float od_pair_c(float r2, float rho0) {
  float ri = od_rsqrt(r2);
  float r = r2 * ri;
  float si = od_rcp(r + rho0);
  float ex = od_ex2(r * OD_NLOG2E);
  float t = fmaf(si, si, si);
  return (ex * ri) * t;
}
// Same with OpenMM's switching polynomial on the energy and a hard cutoff (opendust.py:481-485).
__device__ __forceinline__ float od_pair_c_cut(float r2, const od_dparams& p) {
  float ri = od_rsqrt(r2);
  float r = r2 * ri;
  float si = od_rcp(r + p.rho0);
  float ex = od_ex2(r * OD_NLOG2E);
  float f = ex * fmaf(si, si, si);
  float x = fmaxf((r - p.rs) * p.inv_w, 0.0f);
  // S = 1 - 10x^3 + 15x^4 - 6x^5 = (1-x)^3 (1 + 3x + 6x^2) (no cancellation as x -> 1),
  // S' = -30 x^2 (1-x)^2 / (rc - rs)
  const float om = 1.0f - x;
  float S = om * om * om * fmaf(x, fmaf(6.0f, x, 3.0f), 1.0f);
  const float q = x * om;
  float dS = -30.0f * q * q * p.inv_w;
  float c = (f * S - ex * si * dS) * ri;
  return r2 < p.rc2 ? c : 0.0f;
}

// ------------------------------------------------------------------ external forces
// grains (opendust.py:350-352), trap (opendust.py:552-577), field (opendust.py:580-585)
__device__ __forceinline__ float3 od_ext_accel(const od_dparams& p, const float* cq, float x,
                                               float y, float z) {
  float ax = 0.f, ay = 0.f, az = p.a_field;
  if (p.field_order == 2) {  // chains/matthews.py:484-495, the field clamped outside [z1, z7]
    const float zc = fminf(fmaxf(z, p.fz1), p.fz7);
    az = fmaf(fmaf(p.fa2, zc, p.fa1), zc, p.fa0);
  }
  for (int g = 0; g < p.P; g++) {
    float dx = (x - p.gxh[g]) - p.gxl[g];
    float dy = (y - p.gyh[g]) - p.gyl[g];
    float dz = (z - p.gzh[g]) - p.gzl[g];
    float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    float ri = rsqrtf(r2);
    float c = cq[g] * ri * ri * ri;
    ax = fmaf(c, dx, ax); ay = fmaf(c, dy, ay); az = fmaf(c, dz, az);
  }
  if (p.trap_kind == OD_TRAP_TABLE) {
    // -A_ii grad [alpha_0(h) + alpha_1(h) u + .. + alpha_4(h) u^4], u = x^2 + y^2, h = z
    // (chains/matthews.py:463-478); the tabulated functions are zero outside [-H/2, H/2]
    if (z >= p.th0 && z <= p.th1) {
      const int j = min((int)((z - p.th0) * p.tinv_dh), p.ttn - 2);
      const float t = z - fmaf((float)j, p.tdh, p.th0);
      const float u = fmaf(x, x, y * y);
      float Pu = 0.f, Pz = 0.f;
#pragma unroll
      for (int k = 4; k >= 0; k--) {
        const float* c = p.tcf[k][j];
        const float a = fmaf(fmaf(fmaf(c[3], t, c[2]), t, c[1]), t, c[0]);
        const float da = fmaf(fmaf(3.f * c[3], t, 2.f * c[2]), t, c[1]);
        if (k > 0) Pu = fmaf(Pu, u, (float)k * a);
        Pz = fmaf(Pz, u, da);
      }
      ax = fmaf(2.f * x, Pu, ax);
      ay = fmaf(2.f * y, Pu, ay);
      az += Pz;
    }
    return make_float3(ax, ay, az);
  }
  if (p.trap_kind == OD_TRAP_NONE) return make_float3(ax, ay, az);
  const float* t = p.trapc;
  float u = fmaf(x, x, y * y), w = z * z;
  // P_u and P_w of the 14-term even polynomial; t[k] = -2 A_ii alpha_k
  float Pu = t[1] + w * (t[3] + w * (t[7] + w * t[12])) +
             u * (2.f * t[4] + w * (2.f * t[6] + w * 2.f * t[10]) +
                  u * (3.f * t[8] + w * 3.f * t[11] + u * 4.f * t[13]));
  float Pw = t[2] + u * (t[3] + u * (t[6] + u * t[11])) +
             w * (2.f * t[5] + u * (2.f * t[7] + u * 2.f * t[10]) +
                  w * (3.f * t[9] + u * 3.f * t[12] + w * 4.f * t[14]));
  ax = fmaf(x, Pu, ax);
  ay = fmaf(y, Pu, ay);
  az = fmaf(z, Pw, az);
  return make_float3(ax, ay, az);
}

// ------------------------------------------------------------------ exact flags
// opendust.py:894-910 on squared distances, FP64 with explicit rounding (never contracted);
// the CPU oracle performs the same operations. An FP32 test with a 1e-5 relative margin
// decides all but the ions within that margin of a surface.
__device__ __forceinline__ int od_flag_exact(const od_dparams& p, float xf, float yf, float zf) {
  double x = xf, y = yf, z = zf;
  int bits = 0;
  for (int g = 0; g < p.P; g++) {
    double dx = __dsub_rn(x, p.gx[g]), dy = __dsub_rn(y, p.gy[g]), dz = __dsub_rn(z, p.gz[g]);
    double d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
    d2 = __dadd_rn(d2, __dmul_rn(dz, dz));
    if (d2 <= p.gr2[g]) bits |= 1 << g;
  }
  double rr = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
  if (rr >= p.Rh2) bits |= 1 << 30;
  if (fabs(z) >= p.Hh_half_d) bits |= 1 << 29;
  return bits;
}
__device__ __forceinline__ int od_flag(const od_dparams& p, float x, float y, float z) {
  bool near = false;
  int bits = 0;
  for (int g = 0; g < p.P; g++) {
    float dx = (x - p.gxh[g]) - p.gxl[g];
    float dy = (y - p.gyh[g]) - p.gyl[g];
    float dz = (z - p.gzh[g]) - p.gzl[g];
    float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    if (d2 < p.gr2f[g] * 0.99999f) bits |= 1 << g;
    else if (d2 <= p.gr2f[g] * 1.00001f) near = true;
  }
  float rr = fmaf(x, x, y * y);
  if (rr > p.Rh2f * 1.00001f) bits |= 1 << 30;
  else if (rr >= p.Rh2f * 0.99999f) near = true;
  // |z| >= H/2 (double) is exactly |z| >= Hz_f, the smallest float not below H/2
  if (fabsf(z) >= p.Hz_f) bits |= 1 << 29;
  if (near) return od_flag_exact(p, x, y, z);
  return bits;
}

// ------------------------------------------------------------------ bounded mbarrier / bulk copy
__device__ __forceinline__ uint32_t od_smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void od_mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(od_smem_addr(bar)), "r"(count));
}
__device__ __forceinline__ void od_mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(od_smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void od_fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void od_mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(od_smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
// one-dimensional TMA bulk copy global -> shared, completing on an mbarrier
__device__ __forceinline__ void od_bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                           uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          od_smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(od_smem_addr(bar))
      : "memory");
}
// Programmatic dependent launch (sm_90+): a kernel launched with programmatic stream
// serialization may start while its predecessor runs; it waits here until the predecessor has
// completed and its memory is visible (a no-op for an ordinary launch). A kernel lets its
// successor launch early with od_pdl_trigger (its successors still wait for its completion).
__device__ __forceinline__ void od_pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void od_pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Impulse multiple time stepping (force interval k = p.force_every): the ion–ion force is
// evaluated at the end of steps with step % k == k - 1 and enters the half kicks at the end of
// that step and at the start of the next with weight k; weight 1 every step for k = 1.
__device__ __forceinline__ bool od_evaluates(int k, int64_t step) {
  return k <= 1 || step % k == k - 1;
}
__device__ __forceinline__ float od_first_kick_weight(int k, int64_t step) {
  return k <= 1 ? 1.f : (step % k == 0 ? (float)k : 0.f);
}

// Wait for phase `parity` of the barrier; gives up after `limit` polls and returns false.
__device__ __forceinline__ bool od_mbar_wait_n(uint64_t* bar, uint32_t parity, uint32_t limit) {
  uint32_t addr = od_smem_addr(bar);
  for (uint32_t it = 0; it < limit; it++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
// The production wait: OD_WAIT_LIMIT polls (seconds on a GB300) before it gives up.
__device__ __forceinline__ bool od_mbar_wait(uint64_t* bar, uint32_t parity) {
  return od_mbar_wait_n(bar, parity, OD_WAIT_LIMIT);
}
__device__ __forceinline__ void od_mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(od_smem_addr(bar)) : "memory");
}

// Cell-relative positions. The integration state of an ion is its cell (cx, cy, cz) on a grid
// of side s = rel_s (a power of two in lambda units, chosen per simulation so that the domain
// spans at most half of the index range) and its FP32 offset from that cell's corner; w holds
// the three cell indices, biased by 512 and packed 10 bits each (bits 30-31 stay clear, so the
// word is never a NaN pattern). The absolute FP32 position that the force, flag and injection
// kernels read is fmaf(c, s, offset): the exact sum, rounded once. An offset stays below s, so
// the drift keeps 24 bits below the cell size whatever the distance from the origin.
constexpr int OD_REL_BIAS = 512;   // cell indices in [-512, 511]
__host__ __device__ __forceinline__ int od_rel_pack(int cx, int cy, int cz) {
  return (cx + OD_REL_BIAS) | ((cy + OD_REL_BIAS) << 10) | ((cz + OD_REL_BIAS) << 20);
}
__host__ __device__ __forceinline__ int od_rel_clamp(int c) {
  return c < -OD_REL_BIAS ? -OD_REL_BIAS : (c > OD_REL_BIAS - 1 ? OD_REL_BIAS - 1 : c);
}
__device__ __forceinline__ int3 od_rel_cells(float w) {
  const int k = __float_as_int(w);
  return make_int3((k & 1023) - OD_REL_BIAS, ((k >> 10) & 1023) - OD_REL_BIAS,
                   ((k >> 20) & 1023) - OD_REL_BIAS);
}
// absolute FP32 position of a cell-relative state
__device__ __forceinline__ float4 od_rel_abs(const od_dparams& p, float4 r) {
  const int3 c = od_rel_cells(r.w);
  return make_float4(__fmaf_rn((float)c.x, p.rel_s, r.x), __fmaf_rn((float)c.y, p.rel_s, r.y),
                     __fmaf_rn((float)c.z, p.rel_s, r.z), 0.f);
}
// cell-relative state of an absolute FP32 position (offset x - c s rounded once)
__device__ __forceinline__ float od_rel_axis(float x, float s, float inv, int& c) {
  c = od_rel_clamp((int)floorf(x * inv));
  return __fmaf_rn(-(float)c, s, x);
}
__device__ __forceinline__ float4 od_rel_encode(const od_dparams& p, float x, float y, float z) {
  int cx, cy, cz;
  const float ox = od_rel_axis(x, p.rel_s, p.rel_inv, cx);
  const float oy = od_rel_axis(y, p.rel_s, p.rel_inv, cy);
  const float oz = od_rel_axis(z, p.rel_s, p.rel_inv, cz);
  return make_float4(ox, oy, oz, __int_as_float(od_rel_pack(cx, cy, cz)));
}
// offset o += d on one axis, moved to the cell it has entered
__device__ __forceinline__ float od_rel_move(float o, float d, float s, float inv, int& c) {
  o += d;
  if (!(o >= 0.f && o < s)) {
    const int cn = od_rel_clamp(c + (int)floorf(o * inv));
    o = __fmaf_rn(-(float)(cn - c), s, o);
    c = cn;
  }
  return o;
}
__device__ __forceinline__ void od_rel_drift(const od_dparams& p, float4& r, float dx, float dy,
                                             float dz) {
  int3 c = od_rel_cells(r.w);
  r.x = od_rel_move(r.x, dx, p.rel_s, p.rel_inv, c.x);
  r.y = od_rel_move(r.y, dy, p.rel_s, p.rel_inv, c.y);
  r.z = od_rel_move(r.z, dz, p.rel_s, p.rel_inv, c.z);
  r.w = __int_as_float(od_rel_pack(c.x, c.y, c.z));
}
