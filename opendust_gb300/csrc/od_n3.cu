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

namespace {

constexpr int kWarps = 8;

struct n3_consts {
  od_u64 eps, rho, nl2e;
};

// two pair terms (target X,Y,Z broadcast in both halves; sources packed in QX,QY,QZ)
template <bool REACT>
__device__ __forceinline__ void n3_pair(const n3_consts& k, od_u64 X, od_u64 Y, od_u64 Z,
                                        od_u64 QX, od_u64 QY, od_u64 QZ, od_u64& AX, od_u64& AY,
                                        od_u64& AZ, od_u64& RX, od_u64& RY, od_u64& RZ) {
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
  const od_u64 C = mul2(mul2(EX, RI), fma2(SI, SI, SI));
  AX = fma2(C, DX, AX); AY = fma2(C, DY, AY); AZ = fma2(C, DZ, AZ);
  if (REACT) { RX = fma2(C, DX, RX); RY = fma2(C, DY, RY); RZ = fma2(C, DZ, RZ); }
}

__device__ __forceinline__ od_u64 shfl64(od_u64 v, int src) {
  return __shfl_sync(0xffffffffu, v, src);
}

// One group pair: 32 lane steps of MT x MS pair terms per lane with rotating sources. Each
// source pack moves on as soon as its terms are done, so that its shuffles overlap the next
// pack's arithmetic.
template <int MT, int MS, bool REACT>
__device__ __forceinline__ void n3_group(const n3_consts& k, const od_u64 (&X)[MT],
                                         const od_u64 (&Y)[MT], const od_u64 (&Z)[MT],
                                         od_u64 (&QX)[MS / 2], od_u64 (&QY)[MS / 2],
                                         od_u64 (&QZ)[MS / 2], od_u64 (&AX)[MT], od_u64 (&AY)[MT],
                                         od_u64 (&AZ)[MT], od_u64 (&RX)[MS / 2],
                                         od_u64 (&RY)[MS / 2], od_u64 (&RZ)[MS / 2], int src) {
#pragma unroll 1
  for (int st = 0; st < 32; st++) {
#pragma unroll
    for (int q = 0; q < MS / 2; q++) {
#pragma unroll
      for (int kt = 0; kt < MT; kt++)
        n3_pair<REACT>(k, X[kt], Y[kt], Z[kt], QX[q], QY[q], QZ[q], AX[kt], AY[kt], AZ[kt],
                       RX[q], RY[q], RZ[q]);
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

// Tile pair (a, b), a <= b, of one simulation: one block. sm: dynamic shared memory of
// n3_traits::SMEM bytes.
template <int MT, int MS, int PA>
__device__ __forceinline__ void n3_tile_pair(const float* __restrict__ sx,
                                             const float* __restrict__ sy,
                                             const float* __restrict__ sz, int Npad, int nT,
                                             float* __restrict__ S, float rho0, int a, int b,
                                             float* sm) {
  using TR = n3_traits<MT, MS, PA>;
  constexpr int GT = TR::GT, GS = TR::GS, T = TR::T, NBT = TR::NBT, NBS = TR::NBS;
  constexpr bool HLS = TR::HL_SMEM;
  // sm: [6][T] hi x, y, z, lo x, y, z of tile b's ions; then (HLS) per warp [6][GT] target sums
  const bool diag = a == b;
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31, src = (lane + 1) & 31;
  const int ngt = Npad / GT, ngs = Npad / GS;
  for (int e = tid; e < 6 * T; e += kWarps * 32) sm[e] = 0.f;
  __syncthreads();
  n3_consts k;
  k.eps = p2(1e-30f, 1e-30f);
  k.rho = p2(rho0, rho0);
  k.nl2e = p2(OD_NLOG2E, OD_NLOG2E);
  for (int p = 0; p < PA; p++) {
    const int ga = w + kWarps * p;
    const int GA = a * NBT + ga;
    const bool ta_ok = GA < ngt;
    od_u64 X[MT], Y[MT], Z[MT];
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
          n3_group<MT, MS, true>(k, X, Y, Z, QX, QY, QZ, AX, AY, AZ, RX, RY, RZ, src);
        else
          n3_group<MT, MS, false>(k, X, Y, Z, QX, QY, QZ, AX, AY, AZ, RX, RY, RZ, src);
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
        float* o = S + ((size_t)a * nT + b) * (6 * (size_t)T);
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
  float* o = S + ((size_t)b * nT + a) * (6 * (size_t)T);
  for (int e = tid; e < 6 * T; e += kWarps * 32) o[e] = sm[e];
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
  n3_tile_pair<MT, MS, PA>(sx, sy, sz, Npad, nT, S, rho0, ab.x, ab.y, sm);
}

// Batched form: block k takes work item k = (simulation, tile a, tile b) of a table that lists
// every tile pair of every simulation using this instantiation.
template <int MT, int MS, int PA>
__global__ void __launch_bounds__(kWarps * 32, (n3_traits<MT, MS, PA>::MIN_BLOCKS))
    k_b_pairs_n3(const od_simdesc* __restrict__ sims, const int4* __restrict__ items) {
  extern __shared__ float sm[];
  const int4 w = items[blockIdx.x];
  const od_simdesc& d = sims[w.x];
  n3_tile_pair<MT, MS, PA>(d.b.sx, d.b.sy, d.b.sz, d.Npad, w.w, d.b.n3, d.rho0, w.y, w.z, sm);
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
