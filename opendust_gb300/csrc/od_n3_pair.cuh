// od_n3_pair.cuh — pair arithmetic shared by the each-pair-once kernels: the all-pairs
// tile pairs (od_n3.cu) and the cutoff tile pairs (od_cutn3.cu). Screened pair terms on packed
// f32x2 lanes, the rotating group pair, the staggered tile pair and their register budgets.
#pragma once
#include "od_internal.h"

namespace {


constexpr int kWarps = 8;

// Pair-term constants. CUT = 0: all pairs; 1: cutoff with OpenMM's switching polynomial on
// the energy (S = (1-x)^3 (1 + 3x + 6x^2), x = (r - r_s)/(r_c - r_s) clamped to [0, 1], so that
// pairs beyond r_c contribute exactly 0, opendust.py:481-485); 2: hard cutoff without switching.
struct n3_consts {
  od_u64 eps, rho, nl2e, one, three, six, invw, nrsw, p30w;
  float rc2;
  float skip2;  // cutoff forms: a pack whose pairs all lie beyond sqrt(skip2) contributes 0
  float band_lo, band_hi;  // hard cutoff: r^2 in FP32 within rounding of r_c^2
  double rcd;              // hard cutoff: r_c in FP64, as the reference decides it
};
struct n3_cut {
  float rho0, rc2, rs, inv_w;
  float in2;  // cutoff tile pairs: group pairs closer than sqrt(in2) take the CUT = 0 term
  double rcd;  // hard cutoff: r_c (lambda) in FP64
};

__device__ __forceinline__ n3_consts make_consts(const n3_cut& c) {
  n3_consts k;
  k.eps = p2(1e-30f, 1e-30f);
  k.rho = p2(c.rho0, c.rho0);
  k.nl2e = p2(OD_NLOG2E, OD_NLOG2E);
  k.one = p2(1.f, 1.f); k.three = p2(3.f, 3.f); k.six = p2(6.f, 6.f);
  k.invw = p2(c.inv_w, c.inv_w);
  k.nrsw = p2(-c.rs * c.inv_w, -c.rs * c.inv_w);
  k.p30w = p2(30.f * c.inv_w, 30.f * c.inv_w);
  k.rc2 = c.rc2;
  // (1 + 2e-5) rc^2: beyond it the clamped switching variable is 1 in FP32, so S = 0 and the
  // switched term is exactly zero (the hard cutoff is exactly zero from rc^2 on)
  k.skip2 = c.rc2 * 1.00002f;
  // the FP32 r^2 of a pair is within 4e-7 of its exact value on the same float positions
  k.band_lo = c.rc2 * (1.f - 2e-6f);
  k.band_hi = c.rc2 * (1.f + 2e-6f);
  k.rcd = c.rcd;
  return k;
}

// Is the pair of float positions t, s inside the cutoff as the FP64 reference decides it:
// sqrt((dx^2 + dy^2) + dz^2) < r_c with the differences taken exactly in FP64 and every
// operation rounded once (the oracle's pair_factor).
__device__ __noinline__ bool n3_inside_exact(float tx, float ty, float tz, float sx, float sy,
                                             float sz, double rcd) {
  const double dx = __dsub_rn((double)tx, (double)sx), dy = __dsub_rn((double)ty, (double)sy),
               dz = __dsub_rn((double)tz, (double)sz);
  const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  return __dsqrt_rn(r2) < rcd;
}

// two pair terms (target X,Y,Z broadcast in both halves; sources packed in QX,QY,QZ); COUNT
// adds the directed pairs inside the cutoff (self pairs, at r^2 = 1e-30, excluded)
template <int CUT, bool REACT, bool COUNT>
__device__ __forceinline__ void n3_pair(const n3_consts& k, od_u64 X, od_u64 Y, od_u64 Z,
                                        od_u64 QX, od_u64 QY, od_u64 QZ, od_u64& AX, od_u64& AY,
                                        od_u64& AZ, od_u64& RX, od_u64& RY, od_u64& RZ,
                                        unsigned int& cnt) {
  const od_u64 DX = sub2(X, QX), DY = sub2(Y, QY), DZ = sub2(Z, QZ);
  od_u64 R2 = fma2(DX, DX, k.eps);
  R2 = fma2(DY, DY, R2);
  R2 = fma2(DZ, DZ, R2);
  const float2 r2 = up2(R2);
  // cutoff forms: when every pair of this pack across the warp lies beyond the cutoff (group
  // pairs whose boxes come within r_c but whose ions do not), the terms are exactly zero and the
  // reciprocal, exponential and switching work is skipped (warp-uniform branch)
  if (CUT != 0 && __all_sync(0xffffffffu, fminf(r2.x, r2.y) >= k.skip2)) return;
  const od_u64 RI = p2(od_rsqrt(r2.x), od_rsqrt(r2.y));
  const od_u64 R = mul2(R2, RI);
  const float2 s = up2(add2(R, k.rho));
  const od_u64 SI = p2(od_rcp(s.x), od_rcp(s.y));
  const float2 ea = up2(mul2(R, k.nl2e));
  const od_u64 EX = p2(od_ex2(ea.x), od_ex2(ea.y));
  od_u64 C;
  if (CUT == 0) {
    C = mul2(mul2(EX, RI), fma2(SI, SI, SI));
  } else if (CUT == 1) {
    const float2 xx = up2(fma2(R, k.invw, k.nrsw));
    const od_u64 X2 = p2(fmaxf(xx.x, 0.f), fmaxf(xx.y, 0.f));
    const float2 om = up2(sub2(k.one, X2));
    const od_u64 OM = p2(fmaxf(om.x, 0.f), fmaxf(om.y, 0.f));
    const od_u64 S = mul2(mul2(OM, OM), mul2(OM, fma2(X2, fma2(k.six, X2, k.three), k.one)));
    const od_u64 Q = mul2(X2, OM);
    // e (1/s + 1/s^2) S - e (1/s) S' with S' = -30 Q^2 / (r_c - r_s):
    // = e (1/s) [(1 + 1/s) S + 30 Q^2 / (r_c - r_s)]
    const od_u64 U = fma2(mul2(Q, Q), k.p30w, fma2(SI, S, S));
    C = mul2(mul2(EX, RI), mul2(SI, U));
  } else {
    const float2 c = up2(mul2(mul2(EX, RI), fma2(SI, SI, SI)));
    bool ix = r2.x < k.rc2, iy = r2.y < k.rc2;
    // a pair within FP32 rounding of r_c is decided exactly as the FP64 reference decides it,
    // so that both include the same pairs (rare: a warp-uniform branch)
    const bool nx = r2.x > k.band_lo && r2.x < k.band_hi, ny = r2.y > k.band_lo && r2.y < k.band_hi;
    if (__any_sync(0xffffffffu, nx || ny)) {
      const float2 tx = up2(X), ty = up2(Y), tz = up2(Z), sx = up2(QX), sy = up2(QY), sz = up2(QZ);
      if (nx) ix = n3_inside_exact(tx.x, ty.x, tz.x, sx.x, sy.x, sz.x, k.rcd);
      if (ny) iy = n3_inside_exact(tx.y, ty.y, tz.y, sx.y, sy.y, sz.y, k.rcd);
    }
    C = p2(ix ? c.x : 0.f, iy ? c.y : 0.f);
    if (COUNT)
      cnt += (REACT ? 2u : 1u) * ((unsigned)(ix && r2.x > 1e-29f) + (unsigned)(iy && r2.y > 1e-29f));
  }
  if (COUNT && CUT != 2)
    cnt += (REACT ? 2u : 1u) * ((unsigned)(r2.x < k.rc2 && r2.x > 1e-29f) +
                                (unsigned)(r2.y < k.rc2 && r2.y > 1e-29f));
  AX = fma2(C, DX, AX); AY = fma2(C, DY, AY); AZ = fma2(C, DZ, AZ);
  if (REACT) { RX = fma2(C, DX, RX); RY = fma2(C, DY, RY); RZ = fma2(C, DZ, RZ); }
}

__device__ __forceinline__ od_u64 shfl64(od_u64 v, int src) {
  return __shfl_sync(0xffffffffu, v, src);
}

// One group pair: 32 lane steps of MT x MS pair terms per lane with rotating sources. Each
// source pack moves on as soon as its terms are done, so that its shuffles overlap the next
// pack's arithmetic. UNR lane steps are interleaved (0: two for the cutoff forms, one for the
// plain term).
template <int MT, int MS, int CUT, bool REACT, bool COUNT, int UNR = 0>
__device__ __forceinline__ void n3_group(const n3_consts& k, const od_u64 (&X)[MT],
                                         const od_u64 (&Y)[MT], const od_u64 (&Z)[MT],
                                         od_u64 (&QX)[MS / 2], od_u64 (&QY)[MS / 2],
                                         od_u64 (&QZ)[MS / 2], od_u64 (&AX)[MT], od_u64 (&AY)[MT],
                                         od_u64 (&AZ)[MT], od_u64 (&RX)[MS / 2],
                                         od_u64 (&RY)[MS / 2], od_u64 (&RZ)[MS / 2], int src,
                                         unsigned int& cnt) {
  // two lane steps interleaved give a 2 x 2 shape (two packs per step) more independent work
  // per warp
  constexpr int kUnroll = UNR != 0 ? UNR : (CUT != 0 ? 2 : 1);
#pragma unroll kUnroll
  for (int st = 0; st < 32; st++) {
#pragma unroll
    for (int q = 0; q < MS / 2; q++) {
#pragma unroll
      for (int kt = 0; kt < MT; kt++)
        n3_pair<CUT, REACT, COUNT>(k, X[kt], Y[kt], Z[kt], QX[q], QY[q], QZ[q], AX[kt], AY[kt],
                                   AZ[kt], RX[q], RY[q], RZ[q], cnt);
      QX[q] = shfl64(QX[q], src); QY[q] = shfl64(QY[q], src); QZ[q] = shfl64(QZ[q], src);
      if (REACT) {
        RX[q] = shfl64(RX[q], src); RY[q] = shfl64(RY[q], src); RZ[q] = shfl64(RZ[q], src);
      }
    }
  }
}

// Target-packed group pair: a lane holds its MT targets as MT/2 packs (targets k = 2p and 2p + 1
// in the low and high halves) and its MS sources as scalars, each broadcast into both halves for
// the packed arithmetic, so that a packed operation evaluates two targets against one source.
// The targets take half the registers of the source-packed form (no duplicated halves), which
// leaves room for more independent pair chains in flight. The two halves of a source's reaction
// are added before the source moves on.
template <int MT, int MS, int CUT, bool REACT, bool COUNT>
__device__ __forceinline__ void n3_group_tp(const n3_consts& k, const od_u64 (&X)[MT / 2],
                                            const od_u64 (&Y)[MT / 2], const od_u64 (&Z)[MT / 2],
                                            float (&qx)[MS], float (&qy)[MS], float (&qz)[MS],
                                            od_u64 (&AX)[MT / 2], od_u64 (&AY)[MT / 2],
                                            od_u64 (&AZ)[MT / 2], float (&rx)[MS],
                                            float (&ry)[MS], float (&rz)[MS], int src,
                                            unsigned int& cnt) {
#pragma unroll 1
  for (int st = 0; st < 32; st++) {
#pragma unroll
    for (int m = 0; m < MS; m++) {
      const od_u64 QX = p2(qx[m], qx[m]), QY = p2(qy[m], qy[m]), QZ = p2(qz[m], qz[m]);
      od_u64 RX = p2(rx[m], 0.f), RY = p2(ry[m], 0.f), RZ = p2(rz[m], 0.f);
#pragma unroll
      for (int p = 0; p < MT / 2; p++)
        n3_pair<CUT, REACT, COUNT>(k, X[p], Y[p], Z[p], QX, QY, QZ, AX[p], AY[p], AZ[p], RX, RY,
                                   RZ, cnt);
      qx[m] = __shfl_sync(0xffffffffu, qx[m], src);
      qy[m] = __shfl_sync(0xffffffffu, qy[m], src);
      qz[m] = __shfl_sync(0xffffffffu, qz[m], src);
      if (REACT) {
        rx[m] = __shfl_sync(0xffffffffu, sum2(RX), src);
        ry[m] = __shfl_sync(0xffffffffu, sum2(RY), src);
        rz[m] = __shfl_sync(0xffffffffu, sum2(RZ), src);
      }
    }
  }
}

// (hi, lo) += (h, l) on two-float pairs
__device__ __forceinline__ void acc2x2(float& hi, float& lo, float h, float l) {
  od_acc2(hi, lo, h);
  lo = __fadd_rn(lo, l);
}

// Register and shared-memory budget per instantiation (MT targets and MS sources per lane,
// PA passes). The two-float target sums live in shared memory where registers are scarce:
// 4 x 4 with tiles up to 2048 ions (80 registers, three blocks per SM) and 8 x 2 (128 registers,
// two blocks per SM). Measured on GB300 at 2^20 ions, pair terms/s: 8 x 2 with 2048-ion tiles
// 2.99e12, 4 x 4 with 2048-ion tiles 2.91e12 (two blocks per SM with the sums in registers:
// 2.73e12), 4 x 2 2.89e12, 2 x 2 2.22e12.
template <int MT, int MS, int PA>
struct n3_traits {
  static constexpr int GT = 32 * MT, GS = 32 * MS;  // target and source group sizes
  static constexpr int T = PA * kWarps * GT;        // ions per tile
  static constexpr int NBT = T / GT;                // target groups per tile
  static constexpr int NBS = T / GS;                // source groups per tile (a power of two)
  static constexpr bool HL_SMEM = (MT == 4 && T <= 2048) || MT == 8;
  static constexpr int MIN_BLOCKS = MT == 8 ? 2 : (T <= 2048 ? 3 : 2);
  static constexpr size_t SMEM = sizeof(float) * (6 * T + (HL_SMEM ? 6 * kWarps * GT : 0));
  // target-packed group pairs (n3_group_tp) for 8 targets per lane: 2^20 ions, 3.045e12 pair
  // terms/s against 2.994e12 source-packed (2^17: 2.913e12 against 2.853e12); with 4 targets
  // per lane the 80-register budget spills and the source-packed form is faster
  static constexpr bool TP = MT == 8;
};

// lane steps interleaved by the tile pairs below (source-packed form): two for 2 x 2 and 4 x 4
// (all pairs on GB300: 2 x 2 with 512-ion tiles 2.04e12 pair terms/s at 2^14 ions against 1.82e12
// with one step; 4 x 4 with 1024-ion tiles 2.93e12 at 2^16 against 2.81e12; the batched sweep's
// step 17.8 against 18.7 ms), the n3_group default otherwise
template <int MT>
constexpr int kN3Unroll = MT <= 4 ? 2 : 0;

// (union) box of n consecutive 64-ion groups starting at group g0; 6 floats min xyz, max xyz
__device__ __forceinline__ void group_box(const float* __restrict__ gbox, int g0, int n,
                                          float (&bx)[6]) {
#pragma unroll
  for (int d = 0; d < 6; d++) bx[d] = gbox[g0 * 6 + d];
  for (int q = 1; q < n; q++)
#pragma unroll
    for (int d = 0; d < 3; d++) {
      bx[d] = fminf(bx[d], gbox[(g0 + q) * 6 + d]);
      bx[3 + d] = fmaxf(bx[3 + d], gbox[(g0 + q) * 6 + 3 + d]);
    }
}

// Tile pair (a, b), a <= b, of one simulation: one block. The two-float sums of tile a's ions
// from tile b and of tile b's ions from tile a (one sum per ion when a == b) are added to the
// ions' fixed-point accumulators acc[c * stride + ion] (od_fix_add), ions below Npad only.
// sm: dynamic shared memory of n3_traits::SMEM bytes. CULL skips group pairs whose 64-ion group
// boxes (gbox) are farther apart than sqrt(cull2). Returns the directed pairs inside the cutoff
// when COUNT.
template <int MT, int MS, int PA, int CUT, bool COUNT, bool CULL = false,
          int UNR = kN3Unroll<MT>>
__device__ __forceinline__ unsigned int n3_tile_pair(const float* __restrict__ sx,
                                                     const float* __restrict__ sy,
                                                     const float* __restrict__ sz, int Npad,
                                                     unsigned long long* __restrict__ acc,
                                                     size_t stride, const n3_cut& cut,
                                                     int a, int b, float* sm,
                                                     const float* __restrict__ gbox = nullptr,
                                                     float cull2 = 0.f) {
  using TR = n3_traits<MT, MS, PA>;
  constexpr int GT = TR::GT, GS = TR::GS, T = TR::T, NBT = TR::NBT, NBS = TR::NBS;
  constexpr bool HLS = TR::HL_SMEM, TP = TR::TP;
  // sm: [6][T] hi x, y, z, lo x, y, z of tile b's ions; then (HLS) per warp [6][GT] target sums
  const bool diag = a == b;
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31, src = (lane + 1) & 31;
  const int ngt = Npad / GT, ngs = Npad / GS;
  for (int e = tid; e < 6 * T; e += kWarps * 32) sm[e] = 0.f;
  __syncthreads();
  const n3_consts k = make_consts(cut);
  unsigned int cnt = 0;
  for (int p = 0; p < PA; p++) {
    const int ga = w + kWarps * p;
    const int GA = a * NBT + ga;
    const bool ta_ok = GA < ngt;
    // source-packed form: X[kt] = (x, x) of target kt; target-packed form: X[p] = targets 2p, 2p+1
    od_u64 X[TP ? MT / 2 : MT], Y[TP ? MT / 2 : MT], Z[TP ? MT / 2 : MT];
    float tb[6];  // CULL: box of the target group
    if (CULL && ta_ok) group_box(gbox, GA * (GT / 64), GT / 64, tb);
    // two-float target sums: registers, or this warp's shared-memory slice (lane-private words)
    float hreg[HLS ? 1 : 6 * MT];
    float* const hsm = sm + 6 * T + w * 6 * GT + lane;
#define N3_H(c, kt) (HLS ? hsm[(c) * GT + 32 * (kt)] : hreg[(c) * MT + (kt)])
#pragma unroll
    for (int kt = 0; kt < MT; kt++) {
      const int i = (ta_ok ? GA : 0) * GT + lane + 32 * kt;
      const float x = sx[i], y = sy[i], z = sz[i];
      if constexpr (TP) {
        if (kt & 1) {
          X[kt / 2] = p2(up2(X[kt / 2]).x, x);
          Y[kt / 2] = p2(up2(Y[kt / 2]).x, y);
          Z[kt / 2] = p2(up2(Z[kt / 2]).x, z);
        } else {
          X[kt / 2] = p2(x, 0.f); Y[kt / 2] = p2(y, 0.f); Z[kt / 2] = p2(z, 0.f);
        }
      } else {
        X[kt] = p2(x, x); Y[kt] = p2(y, y); Z[kt] = p2(z, z);
      }
#pragma unroll
      for (int c = 0; c < 6; c++) N3_H(c, kt) = 0.f;
    }
    for (int s = 0; s < NBS; s++) {
      const int gb = (s + w * (NBS / kWarps)) & (NBS - 1);
      const int GB = b * NBS + gb;
      int mode = 0;  // 0: skip, 1: directed (sources inside the target group), 2: each pair once
      if (ta_ok && GB < ngs) {
        const int s0 = gb * GS, t0 = ga * GT;  // tile-local first ions (GS divides GT)
        mode = (!diag || s0 >= t0 + GT) ? 2 : (s0 >= t0 ? 1 : 0);
        if (CULL && mode == 2) {
          // skip group pairs whose boxes are farther apart than the cutoff
          float sb[6];
          group_box(gbox, GB * (GS / 64), GS / 64, sb);
          float d2 = 0.f;
#pragma unroll
          for (int d = 0; d < 3; d++) {
            const float gap = fmaxf(fmaxf(sb[d] - tb[3 + d], tb[d] - sb[3 + d]), 0.f);
            d2 = fmaf(gap, gap, d2);
          }
          if (!(d2 < cull2)) mode = 0;
        }
      }
      if constexpr (TP) {
        if (mode != 0) {
          float qx[MS], qy[MS], qz[MS], rx[MS], ry[MS], rz[MS];
          od_u64 AX[MT / 2], AY[MT / 2], AZ[MT / 2];
  #pragma unroll
          for (int m = 0; m < MS; m++) {
            const int j = GB * GS + lane + 32 * m;
            qx[m] = sx[j]; qy[m] = sy[j]; qz[m] = sz[j];
            rx[m] = ry[m] = rz[m] = 0.f;
          }
  #pragma unroll
          for (int q = 0; q < MT / 2; q++) AX[q] = AY[q] = AZ[q] = 0ull;
          if (mode == 2)
            n3_group_tp<MT, MS, CUT, true, COUNT>(k, X, Y, Z, qx, qy, qz, AX, AY, AZ, rx, ry, rz,
                                                  src, cnt);
          else
            n3_group_tp<MT, MS, CUT, false, COUNT>(k, X, Y, Z, qx, qy, qz, AX, AY, AZ, rx, ry, rz,
                                                   src, cnt);
  #pragma unroll
          for (int q = 0; q < MT / 2; q++) {
            const float2 ax = up2(AX[q]), ay = up2(AY[q]), az = up2(AZ[q]);
            od_acc2(N3_H(0, 2 * q), N3_H(3, 2 * q), ax.x);
            od_acc2(N3_H(1, 2 * q), N3_H(4, 2 * q), ay.x);
            od_acc2(N3_H(2, 2 * q), N3_H(5, 2 * q), az.x);
            od_acc2(N3_H(0, 2 * q + 1), N3_H(3, 2 * q + 1), ax.y);
            od_acc2(N3_H(1, 2 * q + 1), N3_H(4, 2 * q + 1), ay.y);
            od_acc2(N3_H(2, 2 * q + 1), N3_H(5, 2 * q + 1), az.y);
          }
          if (mode == 2) {
  #pragma unroll
            for (int m = 0; m < MS; m++) {
              const int e = gb * GS + lane + 32 * m;
              od_acc2(sm[e], sm[3 * T + e], -rx[m]);
              od_acc2(sm[T + e], sm[4 * T + e], -ry[m]);
              od_acc2(sm[2 * T + e], sm[5 * T + e], -rz[m]);
            }
          }
        }
      } else {
        if (mode != 0) {
          od_u64 QX[MS / 2], QY[MS / 2], QZ[MS / 2], RX[MS / 2], RY[MS / 2], RZ[MS / 2];
          od_u64 AX[MT], AY[MT], AZ[MT];
  #pragma unroll
          for (int q = 0; q < MS / 2; q++) {
            const int j = GB * GS + lane + 64 * q;
            QX[q] = p2(sx[j], sx[j + 32]);
            QY[q] = p2(sy[j], sy[j + 32]);
            QZ[q] = p2(sz[j], sz[j + 32]);
            RX[q] = RY[q] = RZ[q] = 0ull;
          }
  #pragma unroll
          for (int kt = 0; kt < MT; kt++) AX[kt] = AY[kt] = AZ[kt] = 0ull;
          if (mode == 2)
            n3_group<MT, MS, CUT, true, COUNT, UNR>(k, X, Y, Z, QX, QY, QZ, AX, AY, AZ, RX, RY,
                                                    RZ, src, cnt);
          else
            n3_group<MT, MS, CUT, false, COUNT, UNR>(k, X, Y, Z, QX, QY, QZ, AX, AY, AZ, RX, RY,
                                                     RZ, src, cnt);
  #pragma unroll
          for (int kt = 0; kt < MT; kt++) {
            od_acc2(N3_H(0, kt), N3_H(3, kt), sum2(AX[kt]));
            od_acc2(N3_H(1, kt), N3_H(4, kt), sum2(AY[kt]));
            od_acc2(N3_H(2, kt), N3_H(5, kt), sum2(AZ[kt]));
          }
          if (mode == 2) {
            // the force on the sources is minus the accumulated terms
  #pragma unroll
            for (int q = 0; q < MS / 2; q++) {
              const float2 rx = up2(RX[q]), ry = up2(RY[q]), rz = up2(RZ[q]);
              const int e0 = gb * GS + lane + 64 * q, e1 = e0 + 32;
              od_acc2(sm[e0], sm[3 * T + e0], -rx.x);
              od_acc2(sm[T + e0], sm[4 * T + e0], -ry.x);
              od_acc2(sm[2 * T + e0], sm[5 * T + e0], -rz.x);
              od_acc2(sm[e1], sm[3 * T + e1], -rx.y);
              od_acc2(sm[T + e1], sm[4 * T + e1], -ry.y);
              od_acc2(sm[2 * T + e1], sm[5 * T + e1], -rz.y);
            }
          }
        }
      }
      __syncthreads();
    }
    if (ta_ok) {
      if (diag) {
        // tile a is tile b: add the target sums to the same slice
#pragma unroll
        for (int kt = 0; kt < MT; kt++) {
          const int e = ga * GT + lane + 32 * kt;
          acc2x2(sm[e], sm[3 * T + e], N3_H(0, kt), N3_H(3, kt));
          acc2x2(sm[T + e], sm[4 * T + e], N3_H(1, kt), N3_H(4, kt));
          acc2x2(sm[2 * T + e], sm[5 * T + e], N3_H(2, kt), N3_H(5, kt));
        }
      } else {
#pragma unroll
        for (int kt = 0; kt < MT; kt++) {
          const size_t gi = (size_t)GA * GT + lane + 32 * kt;  // < Npad: ta_ok
#pragma unroll
          for (int c = 0; c < 3; c++) od_fix_add(acc + c * stride + gi, N3_H(c, kt), N3_H(3 + c, kt));
        }
      }
    }
    __syncthreads();
  }
#undef N3_H
  for (int e = tid; e < T; e += kWarps * 32) {
    const size_t gi = (size_t)b * T + e;
    if (gi < (size_t)Npad)
#pragma unroll
      for (int c = 0; c < 3; c++) od_fix_add(acc + c * stride + gi, sm[c * T + e], sm[(3 + c) * T + e]);
  }
  return cnt;
}

}  // namespace
