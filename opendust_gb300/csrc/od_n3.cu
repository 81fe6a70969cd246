// od_n3.cu — all-pairs ion–ion sums with each unordered pair evaluated once (variant 7).
//
// The screened pair term is antisymmetric: for dx = x_i - x_j the contribution to ion i is
// c(r)·dx and the contribution to ion j is -c(r)·dx, with the same FP32 bits (IEEE subtraction
// is exactly antisymmetric and r^2 depends on dx^2 only). Evaluating every unordered pair once
// and applying both contributions halves the SFU and FP32 work of the directed-pair kernels
// (the reference's OpenMM CUDA nonbonded kernel also applies each pair force to both atoms).
//
// Decomposition
//   * Ions are split into groups of G = 32·M (one warp: lane l owns the ions l + 32k, k < M)
//     and tiles of T = PA·8·G ions (8 warps, PA passes).
//   * One block per tile pair (a, b), a <= b. Warp w, pass p, holds target group
//     ga = w + 8p of tile a in registers and sweeps the source groups of tile b in a staggered
//     order (gb = (s + w·PA) mod groups-per-tile at step s), so that at every step the eight
//     warps touch eight different source groups and a __syncthreads() between steps makes the
//     shared-memory updates race-free.
//   * Inside a group pair the sources rotate around the warp: at each of the 32 lane steps every
//     lane evaluates its M targets against the M sources it holds (packed f32x2, two sources per
//     operation), then passes its sources — positions and their FP32 reaction sums — to the
//     previous lane. After 32 steps every source is back in its own lane with the sum of the
//     M·32 target reactions on it.
//   * Diagonal tiles (a == b) evaluate a group against itself as directed pairs (no reaction,
//     self pair included: it contributes exactly 0) and skip groups below the diagonal.
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

// One group pair: 32 lane steps of M x M pair terms per lane with rotating sources.
template <int M, bool REACT>
__device__ __forceinline__ void n3_group(const n3_consts& k, const od_u64 (&X)[M],
                                         const od_u64 (&Y)[M], const od_u64 (&Z)[M],
                                         od_u64 (&QX)[M / 2], od_u64 (&QY)[M / 2],
                                         od_u64 (&QZ)[M / 2], od_u64 (&AX)[M], od_u64 (&AY)[M],
                                         od_u64 (&AZ)[M], od_u64 (&RX)[M / 2],
                                         od_u64 (&RY)[M / 2], od_u64 (&RZ)[M / 2], int src) {
#pragma unroll 1
  for (int st = 0; st < 32; st++) {
    // each source pack moves on as soon as its terms are done, so that its shuffles overlap
    // the next pack's arithmetic
#pragma unroll
    for (int q = 0; q < M / 2; q++) {
#pragma unroll
      for (int kt = 0; kt < M; kt++)
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

// Register and shared-memory budget per instantiation. With 4 ions per lane the target sums
// live in shared memory for tiles up to 2048 ions, so that 80 registers per thread give three
// blocks (24 warps) per SM; the 4096-ion tile keeps them in registers (two blocks per SM, the
// shared-memory limit). Measured on GB300 at 2^20 ions: 2.91e12 pair terms/s against 2.73e12
// for the two-block form.
template <int M, int PA>
struct n3_traits {
  static constexpr int T = PA * kWarps * 32 * M;
  static constexpr bool HL_SMEM = M == 4 && T <= 2048;
  static constexpr int MIN_BLOCKS = T <= 2048 ? 3 : 2;
  static constexpr size_t SMEM = sizeof(float) * (6 * T + (HL_SMEM ? 6 * kWarps * 32 * M : 0));
};

template <int M, int PA>
__global__ void __launch_bounds__(kWarps * 32, (n3_traits<M, PA>::MIN_BLOCKS))
    k_pairs_n3(const float* __restrict__ sx, const float* __restrict__ sy,
               const float* __restrict__ sz, int ngroups, int nT, float* __restrict__ S,
               float rho0) {
  constexpr int G = 32 * M;
  constexpr int NBT = PA * kWarps;  // groups per tile (a power of two)
  constexpr int T = NBT * G;        // ions per tile
  constexpr bool HLS = n3_traits<M, PA>::HL_SMEM;
  // [6][T]: hi x, y, z, lo x, y, z of tile b's ions; then (HLS) per warp [6][G] target sums
  extern __shared__ float sm[];
  // tile pair (a, b), a <= b, from the block index (b-major upper triangle)
  const int kb = blockIdx.x;
  int b = (int)((sqrtf(8.f * (float)kb + 1.f) - 1.f) * 0.5f);
  while ((b + 1) * (b + 2) / 2 <= kb) b++;
  while (b * (b + 1) / 2 > kb) b--;
  const int a = kb - b * (b + 1) / 2;
  const bool diag = a == b;
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31, src = (lane + 1) & 31;
  for (int e = tid; e < 6 * T; e += kWarps * 32) sm[e] = 0.f;
  __syncthreads();
  n3_consts k;
  k.eps = p2(1e-30f, 1e-30f);
  k.rho = p2(rho0, rho0);
  k.nl2e = p2(OD_NLOG2E, OD_NLOG2E);
  for (int p = 0; p < PA; p++) {
    const int ga = w + kWarps * p;
    const int GA = a * NBT + ga;
    const bool ta_ok = GA < ngroups;
    od_u64 X[M], Y[M], Z[M];
    // two-float target sums: registers, or this warp's shared-memory slice (lane-private words)
    float hreg[HLS ? 1 : 6 * M];
    float* const hsm = sm + 6 * T + w * 6 * G + lane;
#define N3_H(c, kt) (HLS ? hsm[(c) * G + 32 * (kt)] : hreg[(c) * M + (kt)])
#pragma unroll
    for (int kt = 0; kt < M; kt++) {
      const int i = (ta_ok ? GA : 0) * G + lane + 32 * kt;
      const float x = sx[i], y = sy[i], z = sz[i];
      X[kt] = p2(x, x); Y[kt] = p2(y, y); Z[kt] = p2(z, z);
#pragma unroll
      for (int c = 0; c < 6; c++) N3_H(c, kt) = 0.f;
    }
    for (int s = 0; s < NBT; s++) {
      const int gb = (s + w * PA) & (NBT - 1);
      const int GB = b * NBT + gb;
      int mode = 0;  // 0: skip, 1: directed (the group against itself), 2: each pair once
      if (ta_ok && GB < ngroups) mode = (!diag || gb > ga) ? 2 : (gb == ga ? 1 : 0);
      if (mode != 0) {
        od_u64 QX[M / 2], QY[M / 2], QZ[M / 2], RX[M / 2], RY[M / 2], RZ[M / 2];
        od_u64 AX[M], AY[M], AZ[M];
#pragma unroll
        for (int q = 0; q < M / 2; q++) {
          const int j = GB * G + lane + 64 * q;
          QX[q] = p2(sx[j], sx[j + 32]);
          QY[q] = p2(sy[j], sy[j + 32]);
          QZ[q] = p2(sz[j], sz[j + 32]);
          RX[q] = RY[q] = RZ[q] = 0ull;
        }
#pragma unroll
        for (int kt = 0; kt < M; kt++) AX[kt] = AY[kt] = AZ[kt] = 0ull;
        if (mode == 2)
          n3_group<M, true>(k, X, Y, Z, QX, QY, QZ, AX, AY, AZ, RX, RY, RZ, src);
        else
          n3_group<M, false>(k, X, Y, Z, QX, QY, QZ, AX, AY, AZ, RX, RY, RZ, src);
#pragma unroll
        for (int kt = 0; kt < M; kt++) {
          od_acc2(N3_H(0, kt), N3_H(3, kt), sum2(AX[kt]));
          od_acc2(N3_H(1, kt), N3_H(4, kt), sum2(AY[kt]));
          od_acc2(N3_H(2, kt), N3_H(5, kt), sum2(AZ[kt]));
        }
        if (mode == 2) {
          // the force on the sources is minus the accumulated terms
#pragma unroll
          for (int q = 0; q < M / 2; q++) {
            const float2 rx = up2(RX[q]), ry = up2(RY[q]), rz = up2(RZ[q]);
            const int e0 = gb * G + lane + 64 * q, e1 = e0 + 32;
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
        for (int kt = 0; kt < M; kt++) {
          const int e = ga * G + lane + 32 * kt;
          acc2x2(sm[e], sm[3 * T + e], N3_H(0, kt), N3_H(3, kt));
          acc2x2(sm[T + e], sm[4 * T + e], N3_H(1, kt), N3_H(4, kt));
          acc2x2(sm[2 * T + e], sm[5 * T + e], N3_H(2, kt), N3_H(5, kt));
        }
      } else {
        float* o = S + ((size_t)a * nT + b) * (6 * (size_t)T);
#pragma unroll
        for (int kt = 0; kt < M; kt++) {
          const int e = ga * G + lane + 32 * kt;
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

// Row sums of S in a fixed order: slab 0 of (ph, pl) for every ion below Npad.
__global__ void k_n3_reduce(const float* __restrict__ S, int nT, int T, int Npad,
                            float4* __restrict__ ph, float4* __restrict__ pl) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Npad) return;
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

template <int M, int PA>
cudaError_t launch_n3(const od_pair_io& io, int Npad, float* S, float4* ph, float4* pl,
                      float rho0, cudaStream_t s) {
  constexpr int T = PA * kWarps * 32 * M;
  const int ngroups = Npad / (32 * M);
  const int nT = (Npad + T - 1) / T;
  const size_t smem = n3_traits<M, PA>::SMEM;
  const long long nblk = (long long)nT * (nT + 1) / 2;
  k_pairs_n3<M, PA><<<(unsigned)nblk, kWarps * 32, smem, s>>>(io.sx, io.sy, io.sz, ngroups, nT,
                                                              S, rho0);
  k_n3_reduce<<<(Npad + 255) / 256, 256, 0, s>>>(S, nT, T, Npad, ph, pl);
  return cudaGetLastError();
}

template <int M, int PA>
cudaError_t prepare_n3() {
  return cudaFuncSetAttribute(k_pairs_n3<M, PA>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)n3_traits<M, PA>::SMEM);
}

}  // namespace

cudaError_t od_n3_prepare(const od_pair_plan& pl) {
  const int key = pl.ipt * 10000 + pl.tile;
  switch (key) {
    case 21024: return prepare_n3<2, 2>();
    case 22048: return prepare_n3<2, 4>();
    case 24096: return prepare_n3<2, 8>();
    case 41024: return prepare_n3<4, 1>();
    case 42048: return prepare_n3<4, 2>();
    case 44096: return prepare_n3<4, 4>();
  }
  return cudaErrorInvalidValue;
}

int od_n3_tile(int Npad, size_t budget_bytes) {
  // 1024-ion tiles up to 2^17 ions (enough blocks for several waves), then 2048 (the fastest
  // measured), then 4096, whichever first keeps the tile-pair matrix within the budget
  const int first = Npad <= (1 << 17) ? 1024 : 2048;
  for (int T = first; T <= 4096; T <<= 1)
    if (sizeof(float) * od_n3_floats(Npad, T) <= budget_bytes) return T;
  return 0;
}

size_t od_n3_floats(int Npad, int T) {
  if (T <= 0) return 0;
  const size_t nT = (size_t)((Npad + T - 1) / T);
  return nT * nT * 6 * (size_t)T;
}

cudaError_t od_launch_pairs_n3(const od_pair_plan& pl, const od_pair_io& io, int Npad, float4* ph,
                               float4* plo, float rho0, cudaStream_t s) {
  if (!io.n3) return cudaErrorInvalidValue;
  // ipt selects the ions per lane (M); the tile fixes the passes per block
  if (pl.ipt == 2) {
    switch (pl.tile) {
      case 1024: return launch_n3<2, 2>(io, Npad, io.n3, ph, plo, rho0, s);
      case 2048: return launch_n3<2, 4>(io, Npad, io.n3, ph, plo, rho0, s);
      case 4096: return launch_n3<2, 8>(io, Npad, io.n3, ph, plo, rho0, s);
    }
  } else if (pl.ipt == 4) {
    switch (pl.tile) {
      case 1024: return launch_n3<4, 1>(io, Npad, io.n3, ph, plo, rho0, s);
      case 2048: return launch_n3<4, 2>(io, Npad, io.n3, ph, plo, rho0, s);
      case 4096: return launch_n3<4, 4>(io, Npad, io.n3, ph, plo, rho0, s);
    }
  }
  return cudaErrorInvalidValue;
}
