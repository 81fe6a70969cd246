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
//     lane evaluates its MT targets against the MS sources it holds, then passes the sources —
//     positions and their FP32 reaction sums — to the previous lane. After 32 steps every source
//     is back in its own lane with the sum of the GT target reactions on it. The packed f32x2
//     operations pair two sources against one target (each target duplicated in both halves)
//     or, with 8 targets per lane, two targets against one broadcast source (n3_group_tp: half
//     the target registers, more independent pair chains in flight).
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
#include "od_n3_pair.cuh"

namespace {

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
               const float* __restrict__ sz, int Npad, unsigned long long* __restrict__ acc,
               float rho0) {
  extern __shared__ float sm[];
  const int2 ab = tri_pair(blockIdx.x);
  n3_tile_pair<MT, MS, PA, 0, false>(sx, sy, sz, Npad, acc, (size_t)Npad,
                                     n3_cut{rho0, 0.f, 0.f, 0.f}, ab.x, ab.y, sm);
}

// Batched form: block k takes work item k = (simulation, tile a, tile b) of a table that lists
// every tile pair of every simulation using this instantiation.
template <int MT, int MS, int PA>
__global__ void __launch_bounds__(kWarps * 32, (n3_traits<MT, MS, PA>::MIN_BLOCKS))
    k_b_pairs_n3(const od_simdesc* __restrict__ sims, const int4* __restrict__ items) {
  extern __shared__ float sm[];
  const int4 w = items[blockIdx.x];
  const od_simdesc& d = sims[w.x];
  if (!od_evaluates(d.dp->force_every, d.ds->step)) return;  // force interval: no evaluation
  n3_tile_pair<MT, MS, PA, 0, false>(d.b.sx, d.b.sy, d.b.sz, d.Npad, d.b.n3, (size_t)d.Npad,
                                     n3_cut{d.rho0, 0.f, 0.f, 0.f}, w.y, w.z, sm);
}

// Accumulators -> slab 0 of (ph, pl) as two-float sums, and cleared for the next evaluation.
__global__ void k_n3_take(unsigned long long* __restrict__ acc, int Npad, float4* __restrict__ ph,
                          float4* __restrict__ pl) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Npad) return;
  float3 hi, lo;
  od_fix_take(acc + i, (size_t)Npad, hi, lo);
  ph[i] = make_float4(hi.x, hi.y, hi.z, 0.f);
  pl[i] = make_float4(lo.x, lo.y, lo.z, 0.f);
}

// Batched form: block k covers 256 ions of the simulation in blk[k] (those using variant 7).
__global__ void k_b_n3_take(const od_simdesc* __restrict__ sims, const int2* __restrict__ blk) {
  const int2 e = blk[blockIdx.x];
  const od_simdesc& d = sims[e.x];
  if (!od_evaluates(d.dp->force_every, d.ds->step)) return;
  const int i = e.y * 256 + threadIdx.x;
  if (i >= d.Npad) return;
  float3 hi, lo;
  od_fix_take(d.b.n3 + i, (size_t)d.Npad, hi, lo);
  d.b.part_hi[i] = make_float4(hi.x, hi.y, hi.z, 0.f);
  d.b.part_lo[i] = make_float4(lo.x, lo.y, lo.z, 0.f);
}

template <int MT, int MS, int PA>
cudaError_t launch_n3(const od_pair_io& io, int Npad, unsigned long long* acc, float4* ph,
                      float4* pl, float rho0, cudaStream_t s, bool take) {
  using TR = n3_traits<MT, MS, PA>;
  const int nT = (Npad + TR::T - 1) / TR::T;
  const long long nblk = (long long)nT * (nT + 1) / 2;
  k_pairs_n3<MT, MS, PA><<<(unsigned)nblk, kWarps * 32, TR::SMEM, s>>>(io.sx, io.sy, io.sz, Npad,
                                                                      acc, rho0);
  if (take) k_n3_take<<<(Npad + 255) / 256, 256, 0, s>>>(acc, Npad, ph, pl);
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
  case 20512: return CALL(2, 2, 1);                                        \
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
                               float4* plo, float rho0, cudaStream_t s, bool take) {
  if (!io.n3) return cudaErrorInvalidValue;
#define OD_N3_LAUNCH(a, b, c) launch_n3<a, b, c>(io, Npad, io.n3, ph, plo, rho0, s, take)
  switch (pl.ipt * 10000 + pl.tile) { OD_N3_CASES(OD_N3_LAUNCH) }
#undef OD_N3_LAUNCH
  return cudaErrorInvalidValue;
}

int od_n3_default(int Npad, size_t budget_bytes, int* ipt) {
  // 2 x 2 with 512-ion tiles up to 2^15 ions (2.04e12 pair terms/s at 2^14 against 1.77e12 for
  // the directed-pair kernel and 1.70e12 for 4 x 4 with 1024-ion tiles, which leave SMs idle:
  // 136 tile pairs; 2.50e12 at 2^15 against 2.39e12), 4 x 4 with 1024-ion tiles up to 2^16
  // (2.93e12 against 2.62e12 for 2 x 2 and 2.51e12 for 8 x 2), then 8 x 2 with 2048-ion tiles
  // (2.91e12 at 2^17, 2.99e12 at 2^18, 3.05e12 at 2^20), then 4 x 4 with 4096-ion tiles: the
  // first whose accumulators fit the budget (always: 24 bytes per ion)
  const int cand[4][2] = {{2, 512}, {4, 1024}, {8, 2048}, {4, 4096}};
  for (int c = Npad <= (1 << 15) ? 0 : (Npad <= (1 << 16) ? 1 : 2); c < 4; c++)
    if (sizeof(float) * od_n3_floats(Npad, cand[c][1]) <= budget_bytes) {
      *ipt = cand[c][0];
      return cand[c][1];
    }
  return 0;
}

size_t od_n3_floats(int Npad, int T) {
  // three 64-bit fixed-point accumulators per ion, whatever the tile
  if (T <= 0) return 0;
  return 6 * (size_t)Npad;
}

cudaError_t od_launch_batch_pairs_n3(const od_batchview& v, cudaStream_t s) {
  // the two instantiations batch members use (od_n3_batch_plan)
  if (v.n3_nitems[0] > 0)
    k_b_pairs_n3<4, 4, 1><<<v.n3_nitems[0], kWarps * 32, n3_traits<4, 4, 1>::SMEM, s>>>(
        v.sims, v.n3_items[0]);
  if (v.n3_nitems[1] > 0)
    k_b_pairs_n3<8, 2, 1><<<v.n3_nitems[1], kWarps * 32, n3_traits<8, 2, 1>::SMEM, s>>>(
        v.sims, v.n3_items[1]);
  if (v.n3_nblk > 0) k_b_n3_take<<<v.n3_nblk, 256, 0, s>>>(v.sims, v.n3_blk);
  return cudaGetLastError();
}

int od_n3_batch_plan(int Npad, size_t budget_bytes, int* ipt) {
  // batch members: 4 x 4 with 1024-ion tiles up to 2^16 ions (also below 2^15, where the tile
  // pairs of the other members fill the GPU), 8 x 2 with 2048-ion tiles above, as a member
  // stepped alone; 0 when the matrix does not fit (the member then takes the directed-pair
  // kernel)
  const int T = Npad <= (1 << 16) ? 1024 : 2048;
  if (sizeof(float) * od_n3_floats(Npad, T) > budget_bytes) return 0;
  *ipt = T == 1024 ? 4 : 8;
  return T;
}
