// od_n3.cu — all-pairs ion–ion sums with each unordered pair evaluated once (variant 7).
//
// The screened pair term is antisymmetric: for dx = x_i - x_j the contribution to ion i is
// c(r)·dx and the contribution to ion j is -c(r)·dx, with the same FP32 bits (IEEE subtraction
// is exactly antisymmetric and r^2 depends on dx^2 only). Evaluating every unordered pair once
// and applying both contributions halves the SFU and FP32 work of the directed-pair kernels
// (the reference's OpenMM CUDA nonbonded kernel also applies each pair force to both atoms).
//
// Decomposition
//   * A warp owns a target group of GT = 32·MT ions (lane l holds ions l + 32k, k < MT) and
//     visits source groups of GS = 32·MS ions. Tiles hold T = PA·8·GT ions (8 warps, PA passes).
//   * One block per tile pair (a, b), a <= b. Warp w, pass p, holds target group ga = w + 8p of
//     tile a in registers and sweeps the source groups of tile b in a staggered order (group
//     s + w·NBS/8 at step s), so that at every step the eight warps touch eight different
//     source groups and a __syncthreads() between steps makes the shared-memory updates
//     race-free.
//   * Inside a group pair the sources rotate around the warp: at each of the 32 lane steps every
//     lane evaluates its MT targets against the MS sources it holds (packed f32x2, two sources
//     per operation), then passes the sources — positions and their FP32 reaction sums — to the
//     previous lane. After 32 steps every source is back in its own lane with the sum of the
//     GT target reactions on it.
//   * Diagonal tiles (a == b) evaluate the source groups inside a warp's own target group as
//     directed pairs (no reaction; the self pair contributes exactly 0) and skip source groups
//     below it.
//   * Per target group the per-step FP32 sums are folded into two-float accumulators; reaction
//     sums are folded into a two-float shared-memory slice of tile b.
//   * Output: a dense matrix S[t][y] of two-float partial sums for the ions of tile t from the
//     ions of tile y (t < y: target side of block (t, y); t > y: reaction side of block (y, t);
//     t == y: both). A second kernel sums row t over y in a fixed order into slab 0 of the
//     partial-sum arrays (the all-pairs consumers then see one slab). Every result bit is
//     independent of scheduling.
#include "od_internal.h"
#include "od_hilbert.h"

namespace {

constexpr int kWarps = 8;

// Pair-term constants. CUT = 0: all pairs; 1: cutoff with OpenMM's switching polynomial on
// the energy (S = (1-x)^3 (1 + 3x + 6x^2), x = (r - r_s)/(r_c - r_s) clamped to [0, 1], so that
// pairs beyond r_c contribute exactly 0, opendust.py:481-485); 2: hard cutoff without switching.
struct n3_consts {
  od_u64 eps, rho, nl2e, one, three, six, invw, nrsw, p30w;
  float rc2;
};
struct n3_cut {
  float rho0, rc2, rs, inv_w;
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
  return k;
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
    C = p2(r2.x < k.rc2 ? c.x : 0.f, r2.y < k.rc2 ? c.y : 0.f);
  }
  if (COUNT)
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
// pack's arithmetic.
template <int MT, int MS, int CUT, bool REACT, bool COUNT>
__device__ __forceinline__ void n3_group(const n3_consts& k, const od_u64 (&X)[MT],
                                         const od_u64 (&Y)[MT], const od_u64 (&Z)[MT],
                                         od_u64 (&QX)[MS / 2], od_u64 (&QY)[MS / 2],
                                         od_u64 (&QZ)[MS / 2], od_u64 (&AX)[MT], od_u64 (&AY)[MT],
                                         od_u64 (&AZ)[MT], od_u64 (&RX)[MS / 2],
                                         od_u64 (&RY)[MS / 2], od_u64 (&RZ)[MS / 2], int src,
                                         unsigned int& cnt) {
#pragma unroll 1
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
};

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

// Tile pair (a, b), a <= b, of one simulation: one block. outT receives the two-float sums
// of tile a's ions from tile b, outR those of tile b's ions from tile a (the same slice when
// a == b); each [6][T]. sm: dynamic shared memory of n3_traits::SMEM bytes. CULL skips group
// pairs whose 64-ion group boxes (gbox) are farther apart than sqrt(cull2). Returns the
// directed pairs inside the cutoff when COUNT.
template <int MT, int MS, int PA, int CUT, bool COUNT, bool CULL = false>
__device__ __forceinline__ unsigned int n3_tile_pair(const float* __restrict__ sx,
                                                     const float* __restrict__ sy,
                                                     const float* __restrict__ sz, int Npad,
                                                     float* __restrict__ outT,
                                                     float* __restrict__ outR, const n3_cut& cut,
                                                     int a, int b, float* sm,
                                                     const float* __restrict__ gbox = nullptr,
                                                     float cull2 = 0.f) {
  using TR = n3_traits<MT, MS, PA>;
  constexpr int GT = TR::GT, GS = TR::GS, T = TR::T, NBT = TR::NBT, NBS = TR::NBS;
  constexpr bool HLS = TR::HL_SMEM;
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
    od_u64 X[MT], Y[MT], Z[MT];
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
      X[kt] = p2(x, x); Y[kt] = p2(y, y); Z[kt] = p2(z, z);
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
          n3_group<MT, MS, CUT, true, COUNT>(k, X, Y, Z, QX, QY, QZ, AX, AY, AZ, RX, RY, RZ, src,
                                             cnt);
        else
          n3_group<MT, MS, CUT, false, COUNT>(k, X, Y, Z, QX, QY, QZ, AX, AY, AZ, RX, RY, RZ, src,
                                              cnt);
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
        float* o = outT;
#pragma unroll
        for (int kt = 0; kt < MT; kt++) {
          const int e = ga * GT + lane + 32 * kt;
#pragma unroll
          for (int c = 0; c < 6; c++) o[c * T + e] = N3_H(c, kt);
        }
      }
    }
    __syncthreads();
  }
#undef N3_H
  for (int e = tid; e < 6 * T; e += kWarps * 32) outR[e] = sm[e];
  return cnt;
}

// (a, b) of the k-th pair of the b-major upper triangle
__device__ __forceinline__ int2 tri_pair(int kb) {
  int b = (int)((sqrtf(8.f * (float)kb + 1.f) - 1.f) * 0.5f);
  while ((b + 1) * (b + 2) / 2 <= kb) b++;
  while (b * (b + 1) / 2 > kb) b--;
  return make_int2(kb - b * (b + 1) / 2, b);
}

template <int MT, int MS, int PA>
__global__ void __launch_bounds__(kWarps * 32, (n3_traits<MT, MS, PA>::MIN_BLOCKS))
    k_pairs_n3(const float* __restrict__ sx, const float* __restrict__ sy,
               const float* __restrict__ sz, int Npad, int nT, float* __restrict__ S,
               float rho0) {
  extern __shared__ float sm[];
  const int2 ab = tri_pair(blockIdx.x);
  constexpr size_t T6 = 6 * (size_t)n3_traits<MT, MS, PA>::T;
  n3_tile_pair<MT, MS, PA, 0, false>(sx, sy, sz, Npad, S + ((size_t)ab.x * nT + ab.y) * T6,
                                     S + ((size_t)ab.y * nT + ab.x) * T6, n3_cut{rho0, 0.f, 0.f, 0.f},
                                     ab.x, ab.y, sm);
}

// Batched form: block k takes work item k = (simulation, tile a, tile b) of a table that lists
// every tile pair of every simulation using this instantiation.
template <int MT, int MS, int PA>
__global__ void __launch_bounds__(kWarps * 32, (n3_traits<MT, MS, PA>::MIN_BLOCKS))
    k_b_pairs_n3(const od_simdesc* __restrict__ sims, const int4* __restrict__ items) {
  extern __shared__ float sm[];
  const int4 w = items[blockIdx.x];
  const od_simdesc& d = sims[w.x];
  constexpr size_t T6 = 6 * (size_t)n3_traits<MT, MS, PA>::T;
  n3_tile_pair<MT, MS, PA, 0, false>(d.b.sx, d.b.sy, d.b.sz, d.Npad,
                                     d.b.n3 + ((size_t)w.y * w.w + w.z) * T6,
                                     d.b.n3 + ((size_t)w.z * w.w + w.y) * T6,
                                     n3_cut{d.rho0, 0.f, 0.f, 0.f}, w.y, w.z, sm);
}

// Row sums of S in a fixed order: slab 0 of (ph, pl) for ion i < Npad.
__device__ __forceinline__ void n3_row_sum(const float* __restrict__ S, int nT, int T, int i,
                                           float4* __restrict__ ph, float4* __restrict__ pl) {
  const int t = i / T, e = i - t * T;
  float hx = 0.f, hy = 0.f, hz = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
  const float* r = S + (size_t)t * nT * 6 * (size_t)T + e;
  const size_t step = 6 * (size_t)T;
  // loads of kB entries are issued before their (ordered) accumulation: the sum is a stream
  // of 24 bytes per entry and would otherwise wait on one load at a time
  constexpr int kB = 8;
  int y = 0;
  for (; y + kB <= nT; y += kB, r += kB * step) {
    float v[kB][6];
#pragma unroll
    for (int u = 0; u < kB; u++)
#pragma unroll
      for (int c = 0; c < 6; c++) v[u][c] = __ldcs(r + u * step + c * T);
#pragma unroll
    for (int u = 0; u < kB; u++) {
      acc2x2(hx, lx, v[u][0], v[u][3]);
      acc2x2(hy, ly, v[u][1], v[u][4]);
      acc2x2(hz, lz, v[u][2], v[u][5]);
    }
  }
  for (; y < nT; y++, r += step) {
    acc2x2(hx, lx, r[0], r[3 * T]);
    acc2x2(hy, ly, r[T], r[4 * T]);
    acc2x2(hz, lz, r[2 * T], r[5 * T]);
  }
  ph[i] = make_float4(hx, hy, hz, 0.f);
  pl[i] = make_float4(lx, ly, lz, 0.f);
}

__global__ void k_n3_reduce(const float* __restrict__ S, int nT, int T, int Npad,
                            float4* __restrict__ ph, float4* __restrict__ pl) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < Npad) n3_row_sum(S, nT, T, i, ph, pl);
}

// Batched row sums: block k covers 256 ions of the simulation in blk[k] (those using variant 7).
__global__ void k_b_n3_reduce(const od_simdesc* __restrict__ sims, const int2* __restrict__ blk) {
  const int2 e = blk[blockIdx.x];
  const od_simdesc& d = sims[e.x];
  n3_row_sum(d.b.n3, (d.Npad + d.n3_tile - 1) / d.n3_tile, d.n3_tile, e.y * 256 + threadIdx.x,
             d.b.part_hi, d.b.part_lo);
}

template <int MT, int MS, int PA>
cudaError_t launch_n3(const od_pair_io& io, int Npad, float* S, float4* ph, float4* pl,
                      float rho0, cudaStream_t s) {
  using TR = n3_traits<MT, MS, PA>;
  const int nT = (Npad + TR::T - 1) / TR::T;
  const long long nblk = (long long)nT * (nT + 1) / 2;
  k_pairs_n3<MT, MS, PA><<<(unsigned)nblk, kWarps * 32, TR::SMEM, s>>>(io.sx, io.sy, io.sz, Npad,
                                                                      nT, S, rho0);
  k_n3_reduce<<<(Npad + 255) / 256, 256, 0, s>>>(S, nT, TR::T, Npad, ph, pl);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ cutoff over tile pairs
// Cell grid of G^3 cells over the cube [lo, lo + G/inv_s)^3; a cell's key is its index along
// a Hilbert curve (od_hilbert.h), so that the ions sorted by key fill tiles and 64-ion groups
// with compact bounding boxes: at 2^19 ions in the 3 x 6 lambda cylinder the group boxes keep
// 1.73x the pairs inside a 2 lambda cutoff, against 1.94x in Morton order.
__global__ void k_mc_clear(int ncells, int32_t* __restrict__ count, int32_t* __restrict__ fill) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncells) { count[c] = 0; fill[c] = 0; }
}

__global__ void k_mc_count(int n, const float4* __restrict__ pos, float lo, float inv_s, int G,
                           int32_t* __restrict__ cell_of, int32_t* __restrict__ count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = pos[i];
  const int cx = min(max((int)floorf((p.x - lo) * inv_s), 0), G - 1);
  const int cy = min(max((int)floorf((p.y - lo) * inv_s), 0), G - 1);
  const int cz = min(max((int)floorf((p.z - lo) * inv_s), 0), G - 1);
  const int c = (int)od_hilbert3((uint32_t)cx, (uint32_t)cy, (uint32_t)cz, 31 - __clz(G));
  cell_of[i] = c;
  atomicAdd(&count[c], 1);
}

// exclusive scan of in[0..n) into out[0..n], out[n] = total (one 1024-thread block; in and out
// may be the same array: every thread reads each of its entries before writing it)
__global__ void __launch_bounds__(1024) k_scan_excl(int n, const int32_t* in, int32_t* out) {
  __shared__ int s_w[32];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int per = (n + 1023) / 1024;
  const int c0 = min(tid * per, n), c1 = min(c0 + per, n);
  int a = 0;
  for (int c = c0; c < c1; c++) a += in[c];
  int ia = a;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, ia, o);
    if (lane >= o) ia += y;
  }
  if (lane == 31) s_w[wid] = ia;
  __syncthreads();
  if (wid == 0) {
    const int v = s_w[lane];
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    s_w[lane] = x - v;
  }
  __syncthreads();
  int off = s_w[wid] + ia - a;
  for (int c = c0; c < c1; c++) {
    const int v = in[c];
    out[c] = off;
    off += v;
  }
  if (tid == 1023) out[n] = off;
}

__global__ void k_mc_scatter(int n, const int32_t* __restrict__ cell_of,
                             const int32_t* __restrict__ start, int32_t* __restrict__ fill,
                             int32_t* __restrict__ perm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = cell_of[i];
  perm[start[c] + atomicAdd(&fill[c], 1)] = i;
}

// One block per cell: sort the cell's ions by index (bitonic in shared memory; the order of
// the atomic scatter is not reproducible, the sorted order is) and write their positions.
constexpr int kCellMax = 2048;
__global__ void __launch_bounds__(128) k_mc_sort(const int32_t* __restrict__ count,
                                                 const int32_t* __restrict__ start,
                                                 const float4* __restrict__ pos,
                                                 int32_t* __restrict__ perm, float* __restrict__ xs,
                                                 float* __restrict__ ys, float* __restrict__ zs,
                                                 uint32_t* __restrict__ err) {
  __shared__ int32_t key[kCellMax];
  const int c = blockIdx.x;
  const int n0 = count[c];
  if (n0 == 0) return;
  if (n0 > kCellMax) {
    if (threadIdx.x == 0) atomicOr(err, OD_DERR_CELL);
    return;
  }
  const int s0 = start[c];
  int m = 1;
  while (m < n0) m <<= 1;
  for (int k = threadIdx.x; k < m; k += 128) key[k] = k < n0 ? perm[s0 + k] : 0x7fffffff;
  __syncthreads();
  for (int size = 2; size <= m; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int k = threadIdx.x; k < m; k += 128) {
        const int l = k ^ stride;
        if (l > k) {
          const bool up = (k & size) == 0;
          const int a = key[k], b = key[l];
          if ((a > b) == up) { key[k] = b; key[l] = a; }
        }
      }
      __syncthreads();
    }
  for (int k = threadIdx.x; k < n0; k += 128) {
    const int i = key[k];
    const float4 p = pos[i];
    perm[s0 + k] = i;
    xs[s0 + k] = p.x; ys[s0 + k] = p.y; zs[s0 + k] = p.z;
  }
}

// bounding boxes of every 64-slot group of tile t (real ions only; a group without ions gets
// an inverted box that is never within range) and of the tile itself
__global__ void __launch_bounds__(256) k_tile_box(int n, int T, const float* __restrict__ xs,
                                                  const float* __restrict__ ys,
                                                  const float* __restrict__ zs,
                                                  float* __restrict__ gbox, float* __restrict__ box) {
  __shared__ float tb[8][6];
  const int t = blockIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float um[6] = {3e38f, 3e38f, 3e38f, -3e38f, -3e38f, -3e38f};  // this warp's union
  for (int g = w; g < T / 64; g += 8) {
    float mn[3] = {3e38f, 3e38f, 3e38f}, mx[3] = {-3e38f, -3e38f, -3e38f};
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int i = t * T + g * 64 + h * 32 + lane;
      if (i < n) {
        const float v[3] = {xs[i], ys[i], zs[i]};
#pragma unroll
        for (int d = 0; d < 3; d++) { mn[d] = fminf(mn[d], v[d]); mx[d] = fmaxf(mx[d], v[d]); }
      }
    }
#pragma unroll
    for (int d = 0; d < 3; d++)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        mn[d] = fminf(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
        mx[d] = fmaxf(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
      }
    if (lane < 6) gbox[((size_t)t * (T / 64) + g) * 6 + lane] = lane < 3 ? mn[lane] : mx[lane - 3];
#pragma unroll
    for (int d = 0; d < 3; d++) { um[d] = fminf(um[d], mn[d]); um[3 + d] = fmaxf(um[3 + d], mx[d]); }
  }
  if (lane == 0)
    for (int d = 0; d < 6; d++) tb[w][d] = um[d];
  __syncthreads();
  if (threadIdx.x < 6) {
    float v = tb[0][threadIdx.x];
    for (int k = 1; k < 8; k++)
      v = threadIdx.x < 3 ? fminf(v, tb[k][threadIdx.x]) : fmaxf(v, tb[k][threadIdx.x]);
    box[t * 6 + threadIdx.x] = v;
  }
}

// row a of the tile-pair bitmap: b >= a whose box comes within the cutoff (box distance in
// FP32 with a relative margin of 1e-5, so that no pair inside r_c is dropped by rounding)
__global__ void __launch_bounds__(128) k_tile_adj(int nT, int nwords, const float* __restrict__ box,
                                                  float rc2m, uint32_t* __restrict__ adj,
                                                  int32_t* __restrict__ rowcnt) {
  __shared__ int s_cnt;
  const int a = blockIdx.x;
  uint32_t* row = adj + (size_t)a * nwords;
  for (int w = threadIdx.x; w < nwords; w += 128) row[w] = 0u;
  if (threadIdx.x == 0) s_cnt = 0;
  __syncthreads();
  const float* A = box + a * 6;
  int cnt = 0;
  for (int b = a + threadIdx.x; b < nT; b += 128) {
    const float* B = box + b * 6;
    float d2 = 0.f;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const float g = fmaxf(fmaxf(B[d] - A[3 + d], A[d] - B[3 + d]), 0.f);
      d2 = fmaf(g, g, d2);
    }
    if (d2 < rc2m) { atomicOr(&row[b >> 5], 1u << (b & 31)); cnt++; }
  }
  atomicAdd(&s_cnt, cnt);
  __syncthreads();
  if (threadIdx.x == 0) rowcnt[a] = s_cnt;
}

// listed pairs of row a in increasing b (one thread per row: at most nT bits)
__global__ void k_tile_list(int nT, int nwords, const uint32_t* __restrict__ adj,
                            const int32_t* __restrict__ rowptr, int2* __restrict__ pairs) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nT) return;
  const uint32_t* row = adj + (size_t)a * nwords;
  int k = rowptr[a];
  for (int w = a >> 5; w < nwords; w++) {
    uint32_t bits = row[w];
    while (bits) {
      const int j = __ffs(bits) - 1;
      bits &= bits - 1;
      pairs[k++] = make_int2(a, w * 32 + j);
    }
  }
}

// Balanced tile pair of the cutoff path: 512-ion tiles, NBT target groups of GT = 32·MT ions
// and NBS source groups of GS = 32·MS ions per tile (MT targets and MS sources per lane). The
// group pairs whose boxes come within the cutoff form a list in (target group, source group)
// order, and warp w takes the contiguous slice [w·n/8, (w+1)·n/8) of it, so that the warps
// evaluate the same number of group pairs (± 1) whatever the culling left and no barrier
// separates them. A warp keeps one target group while consecutive items share it and sums its
// targets into a segment slot of its own (a new segment at every change of target group and
// at every slice start: at most NBT + 7); every item stores its FP32 reaction sums in a slot of
// its own. The block then sums the slots of each ion in a fixed order — target segments in list
// order, then reactions in target-group order — so the result does not depend on which warp
// ran what, or when.
template <int MT, int MS>
struct cut_traits {
  static constexpr int GT = 32 * MT, GS = 32 * MS;    // target and source group sizes
  static constexpr int T = 512;                       // ions per tile
  static constexpr int NBT = T / GT, NBS = T / GS;    // groups per tile
  static constexpr int NI = NBT * NBS;                // group pairs per tile pair (<= 64)
  static constexpr int NSEG = NBT + kWarps;           // target segments
  static constexpr bool HS = MT > 2;                  // target sums kept in the segment slot
  static constexpr size_t RFL = (size_t)NI * 3 * GS;  // reaction slots (floats)
  static constexpr size_t TFL = (size_t)NSEG * 6 * GT;  // two-float target segment slots
  static constexpr size_t SMEM = sizeof(float) * (RFL + TFL) + 256;  // + list metadata
};

// warp that owns list entry i of n
__device__ __forceinline__ int cut_owner(int i, int n) {
  int w = 0;
  while (w < kWarps - 1 && (((w + 1) * n) >> 3) <= i) w++;
  return w;
}

// group pair (ga, gb) of a diagonal tile: 2 each pair once, 1 directed (the sources lie in the
// target group), 0 skipped (counted from the other side)
template <int GT, int GS>
__device__ __forceinline__ int cut_diag_mode(int ga, int gb) {
  const int t0 = ga * GT, s0 = gb * GS;
  return s0 >= t0 + GT ? 2 : (s0 >= t0 ? 1 : 0);
}

template <int MT, int MS, int CUT, bool COUNT>
__device__ __forceinline__ unsigned int cut_tile_pair(const float* __restrict__ sx,
                                                      const float* __restrict__ sy,
                                                      const float* __restrict__ sz,
                                                      float* __restrict__ outT,
                                                      float* __restrict__ outR,
                                                      const n3_consts& k, int a, int b, float* sm,
                                                      const float* __restrict__ gbox,
                                                      float cull2) {
  using CT = cut_traits<MT, MS>;
  constexpr int GT = CT::GT, GS = CT::GS, T = CT::T, NBT = CT::NBT, NBS = CT::NBS, NI = CT::NI;
  constexpr int MS2 = MS / 2;
  constexpr bool HS = CT::HS;
  static_assert(NI % 32 == 0 && NI <= 64 && NBT <= 8, "list of at most 64 group pairs");
  float* const R = sm;              // [NI][3][GS] reaction sums of each listed group pair
  float* const Tg = sm + CT::RFL;   // [NSEG][6][GT] two-float target sums of each segment
  unsigned char* const items = reinterpret_cast<unsigned char*>(Tg + CT::TFL);  // ga·NBS + gb
  unsigned char* const segid = items + 64;                                       // per entry
  signed char* const item_of = reinterpret_cast<signed char*>(items + 128);      // by ga·NBS+gb
  signed char* const gs0 = item_of + 64;  // first and last segment of each target group
  signed char* const gs1 = gs0 + 8;
  int* const s_n = reinterpret_cast<int*>(items + 208);
  const bool diag = a == b;
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31, src = (lane + 1) & 31;

  // 1. the list (warp 0): group pairs within range; on a diagonal tile the source groups
  // inside a target group (directed) and those above it
  if (w == 0) {
    int n = 0;
    for (int r = 0; r < NI / 32; r++) {
      const int c = r * 32 + lane, ga = c / NBS, gb = c % NBS;
      const int mode = diag ? cut_diag_mode<GT, GS>(ga, gb) : 2;
      bool keep = mode == 1;
      if (mode == 2) {
        float ta[6], tb[6];
        group_box(gbox, (a * NBT + ga) * (GT / 64), GT / 64, ta);
        group_box(gbox, (b * NBS + gb) * (GS / 64), GS / 64, tb);
        float d2 = 0.f;
#pragma unroll
        for (int d = 0; d < 3; d++) {
          const float gap = fmaxf(fmaxf(tb[d] - ta[3 + d], ta[d] - tb[3 + d]), 0.f);
          d2 = fmaf(gap, gap, d2);
        }
        keep = d2 < cull2;
      }
      const unsigned int bal = __ballot_sync(0xffffffffu, keep);
      const int pos = n + __popc(bal & ((1u << lane) - 1u));
      if (keep) items[pos] = (unsigned char)c;
      item_of[c] = keep ? (signed char)pos : (signed char)-1;
      n += __popc(bal);
    }
    __syncwarp();
    // a segment starts at every change of target group and at the start of every slice
    int nseg = 0;
    for (int r = 0; r < 2; r++) {
      const int i = r * 32 + lane;
      bool f = false;
      if (i < n)
        f = i == 0 || items[i - 1] / NBS != items[i] / NBS ||
            cut_owner(i - 1, n) != cut_owner(i, n);
      const unsigned int bal = __ballot_sync(0xffffffffu, f);
      if (i < n) segid[i] = (unsigned char)(nseg + __popc(bal & ((2u << lane) - 1u)) - 1);
      nseg += __popc(bal);
    }
    if (lane < 8) { gs0[lane] = 0; gs1[lane] = -1; }
    __syncwarp();
    for (int r = 0; r < 2; r++) {
      const int i = r * 32 + lane;
      if (i < n) {
        const int ga = items[i] / NBS;
        if (i == 0 || items[i - 1] / NBS != ga) gs0[ga] = (signed char)segid[i];
        if (i == n - 1 || items[i + 1] / NBS != ga) gs1[ga] = (signed char)segid[i];
      }
    }
    if (lane == 0) *s_n = n;
  }
  __syncthreads();

  // 2. this warp's slice of the list
  const int n = *s_n, i0 = (w * n) >> 3, i1 = ((w + 1) * n) >> 3;
  unsigned int cnt = 0;
  od_u64 X[MT], Y[MT], Z[MT];
  float hreg[HS ? 1 : 6 * MT];
  float* hs = Tg + lane;  // HS: this warp's current segment slot (lane-private words)
#define CUT_H(c, kt) (HS ? hs[(c) * GT + 32 * (kt)] : hreg[(c) * MT + (kt)])
  int cur = -1;
  for (int i = i0; i < i1; i++) {
    const int c = items[i], ga = c / NBS, gb = c % NBS;
    if (ga != cur) {
      if (!HS && cur >= 0) {
        float* t = Tg + (size_t)segid[i - 1] * 6 * GT + lane;
#pragma unroll
        for (int q = 0; q < 6 * MT; q++) t[(q / MT) * GT + 32 * (q % MT)] = hreg[q];
      }
      if (HS) hs = Tg + (size_t)segid[i] * 6 * GT + lane;
#pragma unroll
      for (int kt = 0; kt < MT; kt++) {
        const int j = (a * NBT + ga) * GT + lane + 32 * kt;
        const float x = sx[j], y = sy[j], z = sz[j];
        X[kt] = p2(x, x); Y[kt] = p2(y, y); Z[kt] = p2(z, z);
#pragma unroll
        for (int q = 0; q < 6; q++) CUT_H(q, kt) = 0.f;
      }
      cur = ga;
    }
    od_u64 QX[MS2], QY[MS2], QZ[MS2], RX[MS2], RY[MS2], RZ[MS2], AX[MT], AY[MT], AZ[MT];
#pragma unroll
    for (int q = 0; q < MS2; q++) {
      const int j = (b * NBS + gb) * GS + lane + 64 * q;
      QX[q] = p2(sx[j], sx[j + 32]);
      QY[q] = p2(sy[j], sy[j + 32]);
      QZ[q] = p2(sz[j], sz[j + 32]);
      RX[q] = RY[q] = RZ[q] = 0ull;
    }
#pragma unroll
    for (int kt = 0; kt < MT; kt++) AX[kt] = AY[kt] = AZ[kt] = 0ull;
    if (diag && cut_diag_mode<GT, GS>(ga, gb) == 1) {
      n3_group<MT, MS, CUT, false, COUNT>(k, X, Y, Z, QX, QY, QZ, AX, AY, AZ, RX, RY, RZ, src,
                                          cnt);
    } else {
      n3_group<MT, MS, CUT, true, COUNT>(k, X, Y, Z, QX, QY, QZ, AX, AY, AZ, RX, RY, RZ, src,
                                         cnt);
      // the force on the sources is minus the accumulated terms
      float* r = R + (size_t)i * 3 * GS + lane;
#pragma unroll
      for (int q = 0; q < MS2; q++) {
        const float2 rx = up2(RX[q]), ry = up2(RY[q]), rz = up2(RZ[q]);
        r[64 * q] = -rx.x; r[64 * q + 32] = -rx.y;
        r[GS + 64 * q] = -ry.x; r[GS + 64 * q + 32] = -ry.y;
        r[2 * GS + 64 * q] = -rz.x; r[2 * GS + 64 * q + 32] = -rz.y;
      }
    }
#pragma unroll
    for (int kt = 0; kt < MT; kt++) {
      od_acc2(CUT_H(0, kt), CUT_H(3, kt), sum2(AX[kt]));
      od_acc2(CUT_H(1, kt), CUT_H(4, kt), sum2(AY[kt]));
      od_acc2(CUT_H(2, kt), CUT_H(5, kt), sum2(AZ[kt]));
    }
  }
  if (!HS && cur >= 0) {
    float* t = Tg + (size_t)segid[i1 - 1] * 6 * GT + lane;
#pragma unroll
    for (int q = 0; q < 6 * MT; q++) t[(q / MT) * GT + 32 * (q % MT)] = hreg[q];
  }
#undef CUT_H
  __syncthreads();

  // 3. fixed-order sums of the slots; every ion of both tiles is written (zeros when no group
  // pair reached it)
  for (int e = tid; e < T; e += kWarps * 32) {
    const int g = e / GT, l = e % GT;
    float hx = 0.f, hy = 0.f, hz = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
    for (int s = gs0[g]; s <= gs1[g]; s++) {
      const float* t = Tg + (size_t)s * 6 * GT + l;
      acc2x2(hx, lx, t[0], t[3 * GT]);
      acc2x2(hy, ly, t[GT], t[4 * GT]);
      acc2x2(hz, lz, t[2 * GT], t[5 * GT]);
    }
    if (!diag) {
      outT[e] = hx; outT[T + e] = hy; outT[2 * T + e] = hz;
      outT[3 * T + e] = lx; outT[4 * T + e] = ly; outT[5 * T + e] = lz;
      hx = hy = hz = lx = ly = lz = 0.f;
    }
    const int gb = e / GS, l2 = e % GS;
    for (int ga = 0; ga < NBT; ga++) {
      const int it = item_of[ga * NBS + gb];
      if (it < 0 || (diag && cut_diag_mode<GT, GS>(ga, gb) == 1)) continue;
      const float* r = R + (size_t)it * 3 * GS + l2;
      od_acc2(hx, lx, r[0]);
      od_acc2(hy, ly, r[GS]);
      od_acc2(hz, lz, r[2 * GS]);
    }
    outR[e] = hx; outR[T + e] = hy; outR[2 * T + e] = hz;
    outR[3 * T + e] = lx; outR[4 * T + e] = ly; outR[5 * T + e] = lz;
  }
  __syncthreads();  // the next tile pair rewrites the list and the slots
  return cnt;
}

// every listed tile pair, each unordered ion pair once (static assignment: pair k to block
// k mod grid), group pairs beyond the cutoff skipped. BAL: the balanced list routine above
// (512-ion tiles); otherwise the staggered tile-pair routine.
template <int MT, int MS, int PA, int CUT, bool COUNT, bool BAL>
__global__ void __launch_bounds__(kWarps * 32, (n3_traits<MT, MS, PA>::MIN_BLOCKS))
    k_pairs_cutn3(const float* __restrict__ xs, const float* __restrict__ ys,
                  const float* __restrict__ zs, int nslots, int nT,
                  const int2* __restrict__ pairs, const int32_t* __restrict__ npairs,
                  float* __restrict__ S, n3_cut cut, const float* __restrict__ gbox, float cull2,
                  unsigned long long* __restrict__ pair_count) {
  extern __shared__ float sm[];
  constexpr size_t T6 = 6 * (size_t)(BAL ? cut_traits<MT, MS>::T : n3_traits<MT, MS, PA>::T);
  static_assert(!BAL || PA == 1, "balanced list: one pass");
  const int np = *npairs;
  unsigned int cnt = 0;
  if constexpr (BAL) {
    const n3_consts kc = make_consts(cut);
    for (int k = blockIdx.x; k < np; k += gridDim.x) {
      const int2 ab = pairs[k];
      cnt += cut_tile_pair<MT, MS, CUT, COUNT>(xs, ys, zs, S + ((size_t)ab.x * nT + ab.y) * T6,
                                               S + ((size_t)ab.y * nT + ab.x) * T6, kc, ab.x,
                                               ab.y, sm, gbox, cull2);
    }
  } else {
    for (int k = blockIdx.x; k < np; k += gridDim.x) {
      const int2 ab = pairs[k];
      cnt += n3_tile_pair<MT, MS, PA, CUT, COUNT, true>(xs, ys, zs, nslots,
                                                        S + ((size_t)ab.x * nT + ab.y) * T6,
                                                        S + ((size_t)ab.y * nT + ab.x) * T6, cut,
                                                        ab.x, ab.y, sm, gbox, cull2);
    }
  }
  if (COUNT) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(pair_count, (unsigned long long)cnt);
  }
}

// Row sums over the tiles that share a listed pair with tile t, in increasing tile order,
// written to the ions' entries of (ph, pl). Block (t, c) sums ions c·256 .. c·256+255 of tile t,
// one ion per thread; the matrix rows are read once (streaming loads, four neighbours in flight
// per thread), so the kernel runs at the HBM rate.
__global__ void __launch_bounds__(256) k_tile_reduce(int nT, int nwords, int T,
                                                     const uint32_t* __restrict__ adj,
                                                     const float* __restrict__ S,
                                                     const int32_t* __restrict__ perm,
                                                     float4* __restrict__ ph,
                                                     float4* __restrict__ pl) {
  extern __shared__ int32_t nb[];  // [nT] neighbour tiles, then [8] warp counts
  int32_t* wcnt = nb + nT;
  __shared__ int s_m;
  const int t = blockIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_m = 0;
  __syncthreads();
  // ordered compaction of {y : pair (min(t, y), max(t, y)) listed}, 256 candidates per round
  for (int y0 = 0; y0 < nT; y0 += 256) {
    const int y = y0 + threadIdx.x;
    bool f = false;
    if (y < nT)
      f = y < t ? (adj[(size_t)y * nwords + (t >> 5)] >> (t & 31)) & 1u
                : (adj[(size_t)t * nwords + (y >> 5)] >> (y & 31)) & 1u;
    const uint32_t bal = __ballot_sync(0xffffffffu, f);
    if (lane == 0) wcnt[w] = __popc(bal);
    __syncthreads();
    int base = s_m;
    for (int k = 0; k < w; k++) base += wcnt[k];
    if (f) nb[base + __popc(bal & ((1u << lane) - 1u))] = y;
    __syncthreads();
    if (threadIdx.x == 0) {
      int tot = 0;
      for (int k = 0; k < 8; k++) tot += wcnt[k];
      s_m += tot;
    }
    __syncthreads();
  }
  const int m = s_m;
  const int e = blockIdx.y * 256 + threadIdx.x;
  const int i = perm[t * T + e];
  if (i < 0) return;  // sentinel slot (no barrier follows)
  const float* row = S + (size_t)t * nT * 6 * (size_t)T + e;
  float hx = 0.f, hy = 0.f, hz = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
  int q = 0;
  for (; q + 4 <= m; q += 4) {
    float v[4][6];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const float* r = row + (size_t)nb[q + u] * 6 * T;
#pragma unroll
      for (int c = 0; c < 6; c++) v[u][c] = __ldcs(r + c * T);
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      acc2x2(hx, lx, v[u][0], v[u][3]);
      acc2x2(hy, ly, v[u][1], v[u][4]);
      acc2x2(hz, lz, v[u][2], v[u][5]);
    }
  }
  for (; q < m; q++) {
    const float* r = row + (size_t)nb[q] * 6 * T;
    acc2x2(hx, lx, __ldcs(r), __ldcs(r + 3 * T));
    acc2x2(hy, ly, __ldcs(r + T), __ldcs(r + 4 * T));
    acc2x2(hz, lz, __ldcs(r + 2 * T), __ldcs(r + 5 * T));
  }
  ph[i] = make_float4(hx, hy, hz, 0.f);
  pl[i] = make_float4(lx, ly, lz, 0.f);
}

template <int MT, int MS, int PA>
cudaError_t prepare_n3() {
  const int smem = (int)n3_traits<MT, MS, PA>::SMEM;
  cudaError_t e = cudaFuncSetAttribute(k_pairs_n3<MT, MS, PA>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_b_pairs_n3<MT, MS, PA>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

}  // namespace

// (plan ipt, tile) -> instantiation: ipt 2 and 4 take as many sources as targets per lane,
// ipt 8 takes 8 targets and 2 sources per lane.
#define OD_N3_CASES(CALL)                                                  \
  case 21024: return CALL(2, 2, 2); case 22048: return CALL(2, 2, 4);      \
  case 24096: return CALL(2, 2, 8); case 41024: return CALL(4, 4, 1);      \
  case 42048: return CALL(4, 4, 2); case 44096: return CALL(4, 4, 4);      \
  case 82048: return CALL(8, 2, 1); case 84096: return CALL(8, 2, 2);

bool od_n3_supported(int ipt, int tile) {
#define OD_N3_YES(a, b, c) true
  switch (ipt * 10000 + tile) { OD_N3_CASES(OD_N3_YES) }
#undef OD_N3_YES
  return false;
}

cudaError_t od_n3_prepare(const od_pair_plan& pl) {
#define OD_N3_PREP(a, b, c) prepare_n3<a, b, c>()
  switch (pl.ipt * 10000 + pl.tile) { OD_N3_CASES(OD_N3_PREP) }
#undef OD_N3_PREP
  return cudaErrorInvalidValue;
}

cudaError_t od_launch_pairs_n3(const od_pair_plan& pl, const od_pair_io& io, int Npad, float4* ph,
                               float4* plo, float rho0, cudaStream_t s) {
  if (!io.n3) return cudaErrorInvalidValue;
#define OD_N3_LAUNCH(a, b, c) launch_n3<a, b, c>(io, Npad, io.n3, ph, plo, rho0, s)
  switch (pl.ipt * 10000 + pl.tile) { OD_N3_CASES(OD_N3_LAUNCH) }
#undef OD_N3_LAUNCH
  return cudaErrorInvalidValue;
}

int od_n3_default(int Npad, size_t budget_bytes, int* ipt) {
  // 4 x 4 with 1024-ion tiles up to 2^17 ions (2.87e12 pair terms/s at 2^17 against 2.85e12
  // for 8 x 2), then 8 x 2 with 2048-ion tiles (2.94e12 at 2^18, 2.99e12 at 2^20), then 4 x 4
  // with 4096-ion tiles: the first whose tile-pair matrix fits the budget
  const int cand[3][2] = {{4, 1024}, {8, 2048}, {4, 4096}};
  for (int c = Npad <= (1 << 17) ? 0 : 1; c < 3; c++)
    if (sizeof(float) * od_n3_floats(Npad, cand[c][1]) <= budget_bytes) {
      *ipt = cand[c][0];
      return cand[c][1];
    }
  return 0;
}

size_t od_n3_floats(int Npad, int T) {
  if (T <= 0) return 0;
  const size_t nT = (size_t)((Npad + T - 1) / T);
  return nT * nT * 6 * (size_t)T;
}

cudaError_t od_launch_batch_pairs_n3(const od_batchview& v, cudaStream_t s) {
  // the two instantiations batch members use (od_n3_batch_plan)
  if (v.n3_nitems[0] > 0)
    k_b_pairs_n3<4, 4, 1><<<v.n3_nitems[0], kWarps * 32, n3_traits<4, 4, 1>::SMEM, s>>>(
        v.sims, v.n3_items[0]);
  if (v.n3_nitems[1] > 0)
    k_b_pairs_n3<8, 2, 1><<<v.n3_nitems[1], kWarps * 32, n3_traits<8, 2, 1>::SMEM, s>>>(
        v.sims, v.n3_items[1]);
  if (v.n3_nblk > 0) k_b_n3_reduce<<<v.n3_nblk, 256, 0, s>>>(v.sims, v.n3_blk);
  return cudaGetLastError();
}

int od_n3_batch_plan(int Npad, size_t budget_bytes, int* ipt) {
  // batch members: 4 x 4 with 1024-ion tiles up to 2^17 ions (also below 2^15, where the tile
  // pairs of the other members fill the GPU), 8 x 2 with 2048-ion tiles above; 0 when the
  // matrix does not fit (the member then takes the directed-pair kernel)
  const int T = Npad <= (1 << 17) ? 1024 : 2048;
  if (sizeof(float) * od_n3_floats(Npad, T) > budget_bytes) return 0;
  *ipt = T == 1024 ? 4 : 8;
  return T;
}

int od_cutn3_grid(int N) {
  // about 16 ions per cell: G the smallest power of two with G^3 >= N / 22, 8 <= G <= 128
  int G = 8;
  while (G < 128 && (double)G * G * G * 8.0 * 16.0 < (double)N * 1.4142) G <<= 1;
  return G;
}

size_t od_cutn3_bytes(int N, int T, int G) {
  const size_t nT = (size_t)((N + T - 1) / T), ns = nT * T, nc = (size_t)G * G * G;
  const size_t nw = (nT + 31) / 32;
  return sizeof(float) * nT * nT * 6 * T                      // S
         + sizeof(int2) * nT * (nT + 1) / 2                   // pairs
         + sizeof(uint32_t) * nT * nw                         // bitmap
         + sizeof(float) * (3 * ns + 6 * nT + 6 * (ns / 64))  // sorted positions, boxes
         + sizeof(int32_t) * (ns + N + 3 * nc + nT + 4);
}

// cutoff tile-pair shapes: (ipt, T) = (2, 512) the balanced list with 2 x 2 targets x sources
// per lane, (4, 1024) the staggered tile pair with 4 x 4. Measured on GB300 at 2^19 ions
// (field_chain): 45.2 ms per step with (2, 512), 48.1 with the balanced list at 4 x 2 (128-ion
// target groups: more arithmetic per shuffle, but coarser culling), 55.7 with (4, 1024).
template <int MT, int MS, bool BAL>
cudaError_t prepare_cutn3(int smem) {
  void* fn[4] = {(void*)k_pairs_cutn3<MT, MS, 1, 1, false, BAL>,
                 (void*)k_pairs_cutn3<MT, MS, 1, 1, true, BAL>,
                 (void*)k_pairs_cutn3<MT, MS, 1, 2, false, BAL>,
                 (void*)k_pairs_cutn3<MT, MS, 1, 2, true, BAL>};
  for (int q = 0; q < 4; q++) {
    const cudaError_t e =
        cudaFuncSetAttribute(fn[q], cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

bool od_cutn3_supported(int ipt, int T) {
  return (ipt == 2 && T == 512) || (ipt == 4 && T == 1024);
}

cudaError_t od_cutn3_prepare(int ipt, int T) {
  if (ipt == 2 && T == 512) return prepare_cutn3<2, 2, true>((int)cut_traits<2, 2>::SMEM);
  if (ipt == 4 && T == 1024)
    return prepare_cutn3<4, 4, false>((int)n3_traits<4, 4, 1>::SMEM);
  return cudaErrorInvalidValue;
}

cudaError_t od_launch_cutoff_n3(const od_cutn3& L, const float4* pos, int n, float4* part_hi,
                                float4* part_lo, float rho0, float rc, float rs, uint32_t* err,
                                unsigned long long* pair_count, cudaStream_t s) {
  k_mc_clear<<<(L.ncells + 255) / 256, 256, 0, s>>>(L.ncells, L.count, L.fill);
  k_mc_count<<<(n + 255) / 256, 256, 0, s>>>(n, pos, L.lo, L.inv_s, L.G, L.cell_of, L.count);
  k_scan_excl<<<1, 1024, 0, s>>>(L.ncells, L.count, L.start);
  k_mc_scatter<<<(n + 255) / 256, 256, 0, s>>>(n, L.cell_of, L.start, L.fill, L.perm);
  k_mc_sort<<<L.ncells, 128, 0, s>>>(L.count, L.start, pos, L.perm, L.xs, L.ys, L.zs, err);
  k_tile_box<<<L.nT, 256, 0, s>>>(n, L.T, L.xs, L.ys, L.zs, L.gbox, L.box);
  const float rc2m = rc * rc * 1.00001f;
  k_tile_adj<<<L.nT, 128, 0, s>>>(L.nT, L.nwords, L.box, rc2m, L.adj, L.rowptr);
  k_scan_excl<<<1, 1024, 0, s>>>(L.nT, L.rowptr, L.rowptr);
  k_tile_list<<<(L.nT + 127) / 128, 128, 0, s>>>(L.nT, L.nwords, L.adj, L.rowptr, L.pairs);
  const bool sw = rs < rc;
  const n3_cut cut{rho0, rc * rc, rs, sw ? 1.0f / (rc - rs) : 0.0f};
  const int32_t* np = L.rowptr + L.nT;
#define OD_CUTN3(MT, MS, BAL, SM)                                                             \
  do {                                                                                        \
    if (sw) {                                                                                 \
      if (pair_count) OD_CUTN3L(MT, MS, 1, true, BAL, SM);                                    \
      else OD_CUTN3L(MT, MS, 1, false, BAL, SM);                                              \
    } else {                                                                                  \
      if (pair_count) OD_CUTN3L(MT, MS, 2, true, BAL, SM);                                    \
      else OD_CUTN3L(MT, MS, 2, false, BAL, SM);                                              \
    }                                                                                         \
  } while (0)
#define OD_CUTN3L(MT, MS, CUT, CNT, BAL, SM)                                                  \
  k_pairs_cutn3<MT, MS, 1, CUT, CNT, BAL><<<L.grid, kWarps * 32, SM, s>>>(                    \
      L.xs, L.ys, L.zs, L.nslots, L.nT, L.pairs, np, L.S, cut, L.gbox, rc2m, pair_count)
  if (L.ipt == 2 && L.T == 512) OD_CUTN3(2, 2, true, (cut_traits<2, 2>::SMEM));
  else if (L.ipt == 4 && L.T == 1024) OD_CUTN3(4, 4, false, (n3_traits<4, 4, 1>::SMEM));
  else return cudaErrorInvalidValue;
#undef OD_CUTN3L
#undef OD_CUTN3
  const size_t smem = sizeof(int32_t) * (L.nT + 8);
  k_tile_reduce<<<dim3(L.nT, L.T / 256), 256, smem, s>>>(L.nT, L.nwords, L.T, L.adj, L.S, L.perm,
                                                        part_hi, part_lo);
  return cudaGetLastError();
}
