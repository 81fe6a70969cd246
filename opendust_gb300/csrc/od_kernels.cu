// od_kernels.cu — CUDA kernels of the superion step (sm_103a).
//
// One step of the reference program (opendust.py:839-1037 + host tail :1117-1383) runs as
//   K1 kick_drift      collisions, v += a/2 with forces at the current positions, x += v
//   K2 pairs           ion–ion sums at the drifted positions (all pairs, N^2)
//   K3 kick_flag       reduce K2 partials, v += a/2, grain/domain flags -> warp ballots
//   K4 collect_inject  ordered compaction of flagged ions, per-grain sums, re-injection
//   K5 correct_orbit   ion–ion sums moved to the re-injected positions, orbit-force sums
//   K6 tail            FP64 charge update, grain forces, result series, averages
// The reference evaluates ion–ion forces twice per step (after the drift and again after
// re-injection, because OpenMM re-evaluates forces whenever positions change). Only the few
// re-injected ions move between those two evaluations, so K5 applies their O(N*K) difference
// to K2's sums instead of a second N^2 pass; the result is the same sum.
#include <cuda_runtime.h>
#include <stdint.h>
#include "od_internal.h"

namespace {

constexpr int kBlk = 256;

// ============================================================== K2: all-pairs ion–ion sums
// Block = NT threads x IPT targets; grid.y splits the sources into chunks. Source tiles of
// OD_TJ float4 are staged in shared memory by one-dimensional TMA bulk copies (double
// buffered, completion on an mbarrier); every thread then reads each source with a
// broadcast shared-memory load (VARIANT 0) or each warp reads 32 sources and broadcasts
// them with warp shuffles (VARIANT 1). Per target the tile's pair terms are summed in FP32
// and folded into a (hi, lo) two-float accumulator once per tile.
template <int NT, int IPT, int VARIANT>
__global__ void __launch_bounds__(NT) k_pairs(const float4* __restrict__ pos, int Npad, int chunk,
                                              float4* __restrict__ part_hi,
                                              float4* __restrict__ part_lo, float rho0,
                                              uint32_t* __restrict__ err) {
  __shared__ __align__(128) float4 tile[2][OD_TJ];
  __shared__ __align__(8) uint64_t bar[2];
  const int tid = threadIdx.x;
  const int ibase = blockIdx.x * (NT * IPT) + tid;
  const int j0 = blockIdx.y * chunk;
  const int j1 = min(j0 + chunk, Npad);
  const int ntiles = (j1 - j0) / OD_TJ;

  float px[IPT], py[IPT], pz[IPT], hx[IPT], hy[IPT], hz[IPT], lx[IPT], ly[IPT], lz[IPT];
#pragma unroll
  for (int k = 0; k < IPT; k++) {
    float4 q = pos[ibase + k * NT];
    px[k] = q.x; py[k] = q.y; pz[k] = q.z;
    hx[k] = hy[k] = hz[k] = lx[k] = ly[k] = lz[k] = 0.f;
  }
  if (tid == 0) {
    od_mbar_init(&bar[0], 1);
    od_mbar_init(&bar[1], 1);
    od_fence_barrier_init();
  }
  __syncthreads();
  int issued = 0;
  if (tid == 0) {
    for (; issued < 2 && issued < ntiles; issued++) {
      od_mbar_expect_tx(&bar[issued], OD_TJ * 16);
      od_bulk_g2s(tile[issued], pos + j0 + issued * OD_TJ, OD_TJ * 16, &bar[issued]);
    }
  }
  bool ok = true;
  int t = 0;
  for (; t < ntiles; t++) {
    const int s = t & 1;
    ok = __syncthreads_and(od_mbar_wait(&bar[s], (t >> 1) & 1));
    if (!ok) break;
    float ax[IPT], ay[IPT], az[IPT];
#pragma unroll
    for (int k = 0; k < IPT; k++) ax[k] = ay[k] = az[k] = 0.f;
    if (VARIANT == 0) {
#pragma unroll 8
      for (int j = 0; j < OD_TJ; j++) {
        const float4 q = tile[s][j];
#pragma unroll
        for (int k = 0; k < IPT; k++) {
          float dx = px[k] - q.x, dy = py[k] - q.y, dz = pz[k] - q.z;
          float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, 1e-30f)));
          float c = od_pair_c(r2, rho0);
          ax[k] = fmaf(c, dx, ax[k]); ay[k] = fmaf(c, dy, ay[k]); az[k] = fmaf(c, dz, az[k]);
        }
      }
    } else {
      const int lane = tid & 31;
      for (int jj = 0; jj < OD_TJ; jj += 32) {
        const float4 mine = tile[s][jj + lane];
#pragma unroll 8
        for (int l = 0; l < 32; l++) {
          float qx = __shfl_sync(0xffffffffu, mine.x, l);
          float qy = __shfl_sync(0xffffffffu, mine.y, l);
          float qz = __shfl_sync(0xffffffffu, mine.z, l);
#pragma unroll
          for (int k = 0; k < IPT; k++) {
            float dx = px[k] - qx, dy = py[k] - qy, dz = pz[k] - qz;
            float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, 1e-30f)));
            float c = od_pair_c(r2, rho0);
            ax[k] = fmaf(c, dx, ax[k]); ay[k] = fmaf(c, dy, ay[k]); az[k] = fmaf(c, dz, az[k]);
          }
        }
      }
    }
#pragma unroll
    for (int k = 0; k < IPT; k++) {
      od_acc2(hx[k], lx[k], ax[k]);
      od_acc2(hy[k], ly[k], ay[k]);
      od_acc2(hz[k], lz[k], az[k]);
    }
    __syncthreads();  // all threads are done with stage s
    if (tid == 0 && issued < ntiles) {
      od_mbar_expect_tx(&bar[s], OD_TJ * 16);
      od_bulk_g2s(tile[s], pos + j0 + issued * OD_TJ, OD_TJ * 16, &bar[s]);
      issued++;
    }
  }
  if (!ok) {
    if (tid == 0) {
      atomicOr(err, OD_DERR_TIMEOUT);
      for (int u = t; u < issued; u++) od_mbar_wait(&bar[u & 1], (u >> 1) & 1);
    }
    return;
  }
  const size_t off = (size_t)blockIdx.y * Npad;
#pragma unroll
  for (int k = 0; k < IPT; k++) {
    const int i = ibase + k * NT;
    part_hi[off + i] = make_float4(hx[k], hy[k], hz[k], 0.f);
    part_lo[off + i] = make_float4(lx[k], ly[k], lz[k], 0.f);
  }
}

// ------------------------------------------------------------------ packed f32x2 variant
// Blackwell executes two FP32 lanes per instruction with the f32x2 forms of add/sub/mul/fma.
// Sources are staged as SoA slices (x[], y[], z[]) so that one 128-bit shared load gives two
// packed source pairs (x0,x1),(x2,x3). Each thread owns two targets; a packed operation then
// evaluates two pairs in one issue slot. The SFU (rsqrt, rcp, ex2) stays scalar per pair.
// NEWTON = 1: target 1 takes 1/s from two packed Newton steps seeded with 1/r (error
// (r0/r)^4); when any lane of the warp saw r^2 < newton_r2 in the tile, the tile is redone
// for target 1 with the SFU reciprocal.
struct od_pk {
  od_u64 eps, rho, nrho, nl2e, one;
};

// two pair terms (target vs sources a and b), SFU reciprocal
__device__ __forceinline__ void pair2_sfu(const od_pk& k, od_u64 X, od_u64 Y, od_u64 Z, od_u64 QX,
                                          od_u64 QY, od_u64 QZ, od_u64& AX, od_u64& AY, od_u64& AZ) {
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
}
// same with 1/s from Newton steps seeded with 1/r; tracks the smallest r^2 seen
__device__ __forceinline__ void pair2_newton(const od_pk& k, od_u64 X, od_u64 Y, od_u64 Z, od_u64 QX,
                                             od_u64 QY, od_u64 QZ, od_u64& AX, od_u64& AY,
                                             od_u64& AZ, float& mr2) {
  const od_u64 DX = sub2(X, QX), DY = sub2(Y, QY), DZ = sub2(Z, QZ);
  od_u64 R2 = fma2(DX, DX, k.eps);
  R2 = fma2(DY, DY, R2);
  R2 = fma2(DZ, DZ, R2);
  const float2 r2 = up2(R2);
  mr2 = fminf(mr2, fminf(r2.x, r2.y));
  const od_u64 RI = p2(od_rsqrt(r2.x), od_rsqrt(r2.y));
  const od_u64 R = mul2(R2, RI);
  const od_u64 NS = sub2(k.nrho, R);  // -(r + rho0)
  od_u64 E = fma2(NS, RI, k.one);
  od_u64 SI = fma2(RI, E, RI);
  E = fma2(NS, SI, k.one);
  SI = fma2(SI, E, SI);
  const float2 ea = up2(mul2(R, k.nl2e));
  const od_u64 EX = p2(od_ex2(ea.x), od_ex2(ea.y));
  const od_u64 C = mul2(mul2(EX, RI), fma2(SI, SI, SI));
  AX = fma2(C, DX, AX); AY = fma2(C, DY, AY); AZ = fma2(C, DZ, AZ);
}


// One block's share of the packed all-pairs sums: targets iblk*2*NT .. +2*NT, sources
// [j0, j1); partial sums written at part_*[slab_off + i]. Returns false after a wait timeout.
// Newton reciprocal with a warp-uniform fallback: when any lane of the warp has a pair closer
// than sqrt(newton_r2) (where two Newton steps from 1/r are not accurate), the SFU reciprocal
// replaces the Newton result for the whole warp.
__device__ __forceinline__ void pair2_newton_vote(const od_pk& k, od_u64 X, od_u64 Y, od_u64 Z,
                                                  od_u64 QX, od_u64 QY, od_u64 QZ, od_u64& AX,
                                                  od_u64& AY, od_u64& AZ, float newton_r2) {
  const od_u64 DX = sub2(X, QX), DY = sub2(Y, QY), DZ = sub2(Z, QZ);
  od_u64 R2 = fma2(DX, DX, k.eps);
  R2 = fma2(DY, DY, R2);
  R2 = fma2(DZ, DZ, R2);
  const float2 r2 = up2(R2);
  const od_u64 RI = p2(od_rsqrt(r2.x), od_rsqrt(r2.y));
  const od_u64 R = mul2(R2, RI);
  const od_u64 NS = sub2(k.nrho, R);  // -(r + rho0)
  od_u64 E = fma2(NS, RI, k.one);
  od_u64 SI = fma2(RI, E, RI);
  E = fma2(NS, SI, k.one);
  SI = fma2(SI, E, SI);
  if (__any_sync(0xffffffffu, fminf(r2.x, r2.y) < newton_r2)) {
    const float2 ns = up2(NS);
    SI = p2(od_rcp(-ns.x), od_rcp(-ns.y));
  }
  const float2 ea = up2(mul2(R, k.nl2e));
  const od_u64 EX = p2(od_ex2(ea.x), od_ex2(ea.y));
  const od_u64 C = mul2(mul2(EX, RI), fma2(SI, SI, SI));
  AX = fma2(C, DX, AX); AY = fma2(C, DY, AY); AZ = fma2(C, DZ, AZ);
}

template <int NT, int NEWTON, int TPT = 2>
__device__ __forceinline__ bool pairs_x2_body(const float* __restrict__ sx,
                                              const float* __restrict__ sy,
                                              const float* __restrict__ sz, int iblk, int j0,
                                              int j1, size_t slab_off,
                                              float4* __restrict__ part_hi,
                                              float4* __restrict__ part_lo, float rho0,
                                              float newton_r2, uint32_t* __restrict__ err,
                                              int tgt_off = 0,
                                              unsigned long long* __restrict__ acc = nullptr,
                                              size_t acc_stride = 0) {
  __shared__ __align__(128) float tx[2][OD_TJ];
  __shared__ __align__(128) float ty[2][OD_TJ];
  __shared__ __align__(128) float tz[2][OD_TJ];
  __shared__ __align__(8) uint64_t bar[2];
  const int tid = threadIdx.x;
  const int i0 = iblk * (TPT * NT) + tid, i1 = TPT == 2 ? i0 + NT : i0;
  const int ntiles = (j1 - j0) / OD_TJ;
  // targets: entries tgt_off + i of the source arrays (a shard's own ions within all sources)
  const int t0 = tgt_off + i0, t1 = tgt_off + i1;
  const od_u64 X0 = p2(sx[t0], sx[t0]), Y0 = p2(sy[t0], sy[t0]), Z0 = p2(sz[t0], sz[t0]);
  const od_u64 X1 = p2(sx[t1], sx[t1]), Y1 = p2(sy[t1], sy[t1]), Z1 = p2(sz[t1], sz[t1]);
  od_pk k;
  k.eps = p2(1e-30f, 1e-30f);
  k.rho = p2(rho0, rho0);
  k.nrho = p2(-rho0, -rho0);
  k.nl2e = p2(OD_NLOG2E, OD_NLOG2E);
  k.one = p2(1.0f, 1.0f);
  float h0x = 0.f, h0y = 0.f, h0z = 0.f, l0x = 0.f, l0y = 0.f, l0z = 0.f;
  float h1x = 0.f, h1y = 0.f, h1z = 0.f, l1x = 0.f, l1y = 0.f, l1z = 0.f;
  if (tid == 0) {
    od_mbar_init(&bar[0], 1);
    od_mbar_init(&bar[1], 1);
    od_fence_barrier_init();
  }
  __syncthreads();
  constexpr uint32_t kBytes = OD_TJ * 4;
  int issued = 0;
  if (tid == 0) {
    for (; issued < 2 && issued < ntiles; issued++) {
      const int jb = j0 + issued * OD_TJ;
      od_mbar_expect_tx(&bar[issued], 3 * kBytes);
      od_bulk_g2s(tx[issued], sx + jb, kBytes, &bar[issued]);
      od_bulk_g2s(ty[issued], sy + jb, kBytes, &bar[issued]);
      od_bulk_g2s(tz[issued], sz + jb, kBytes, &bar[issued]);
    }
  }
  bool ok = true;
  int t = 0;
  for (; t < ntiles; t++) {
    const int s = t & 1;
    ok = __syncthreads_and(od_mbar_wait(&bar[s], (t >> 1) & 1));
    if (!ok) break;
    od_u64 A0x = 0, A0y = 0, A0z = 0, A1x = 0, A1y = 0, A1z = 0;
    float mr2 = 3.0e38f;
#pragma unroll 2
    for (int j = 0; j < OD_TJ; j += 4) {
      const ulonglong2 qx = *reinterpret_cast<const ulonglong2*>(&tx[s][j]);
      const ulonglong2 qy = *reinterpret_cast<const ulonglong2*>(&ty[s][j]);
      const ulonglong2 qz = *reinterpret_cast<const ulonglong2*>(&tz[s][j]);
      pair2_sfu(k, X0, Y0, Z0, qx.x, qy.x, qz.x, A0x, A0y, A0z);
      if (TPT == 1) {
        // one target per thread: the second source pair of the load takes the Newton
        // reciprocal (NEWTON == 2) or the SFU one
        if (NEWTON == 2)
          pair2_newton_vote(k, X0, Y0, Z0, qx.y, qy.y, qz.y, A0x, A0y, A0z, newton_r2);
        else
          pair2_sfu(k, X0, Y0, Z0, qx.y, qy.y, qz.y, A0x, A0y, A0z);
        continue;
      }
      pair2_sfu(k, X0, Y0, Z0, qx.y, qy.y, qz.y, A0x, A0y, A0z);
      if (NEWTON == 2) {
        pair2_newton_vote(k, X1, Y1, Z1, qx.x, qy.x, qz.x, A1x, A1y, A1z, newton_r2);
        pair2_newton_vote(k, X1, Y1, Z1, qx.y, qy.y, qz.y, A1x, A1y, A1z, newton_r2);
      } else if (NEWTON == 1) {
        pair2_newton(k, X1, Y1, Z1, qx.x, qy.x, qz.x, A1x, A1y, A1z, mr2);
        pair2_newton(k, X1, Y1, Z1, qx.y, qy.y, qz.y, A1x, A1y, A1z, mr2);
      } else {
        pair2_sfu(k, X1, Y1, Z1, qx.x, qy.x, qz.x, A1x, A1y, A1z);
        pair2_sfu(k, X1, Y1, Z1, qx.y, qy.y, qz.y, A1x, A1y, A1z);
      }
    }
    if (TPT == 2 && NEWTON == 1 && __any_sync(0xffffffffu, mr2 < newton_r2)) {
      A1x = A1y = A1z = 0;
      for (int j = 0; j < OD_TJ; j += 4) {
        const ulonglong2 qx = *reinterpret_cast<const ulonglong2*>(&tx[s][j]);
        const ulonglong2 qy = *reinterpret_cast<const ulonglong2*>(&ty[s][j]);
        const ulonglong2 qz = *reinterpret_cast<const ulonglong2*>(&tz[s][j]);
        pair2_sfu(k, X1, Y1, Z1, qx.x, qy.x, qz.x, A1x, A1y, A1z);
        pair2_sfu(k, X1, Y1, Z1, qx.y, qy.y, qz.y, A1x, A1y, A1z);
      }
    }
    od_acc2(h0x, l0x, sum2(A0x)); od_acc2(h0y, l0y, sum2(A0y)); od_acc2(h0z, l0z, sum2(A0z));
    if (TPT == 2) {
      od_acc2(h1x, l1x, sum2(A1x)); od_acc2(h1y, l1y, sum2(A1y)); od_acc2(h1z, l1z, sum2(A1z));
    }
    __syncthreads();
    if (tid == 0 && issued < ntiles) {
      const int jb = j0 + issued * OD_TJ;
      od_mbar_expect_tx(&bar[s], 3 * kBytes);
      od_bulk_g2s(tx[s], sx + jb, kBytes, &bar[s]);
      od_bulk_g2s(ty[s], sy + jb, kBytes, &bar[s]);
      od_bulk_g2s(tz[s], sz + jb, kBytes, &bar[s]);
      issued++;
    }
  }
  if (!ok) {
    if (tid == 0) {
      atomicOr(err, OD_DERR_TIMEOUT);
      for (int u = t; u < issued; u++) od_mbar_wait(&bar[u & 1], (u >> 1) & 1);
    }
    return false;
  }
  if (acc) {
    // fixed-point accumulators: the source chunks of a target add up in any order
    od_fix_add(acc + i0, h0x, l0x);
    od_fix_add(acc + acc_stride + i0, h0y, l0y);
    od_fix_add(acc + 2 * acc_stride + i0, h0z, l0z);
    if (TPT == 2) {
      od_fix_add(acc + i1, h1x, l1x);
      od_fix_add(acc + acc_stride + i1, h1y, l1y);
      od_fix_add(acc + 2 * acc_stride + i1, h1z, l1z);
    }
  } else {
    const size_t off = slab_off;
    part_hi[off + i0] = make_float4(h0x, h0y, h0z, 0.f);
    part_lo[off + i0] = make_float4(l0x, l0y, l0z, 0.f);
    if (TPT == 2) {
      part_hi[off + i1] = make_float4(h1x, h1y, h1z, 0.f);
      part_lo[off + i1] = make_float4(l1x, l1y, l1z, 0.f);
    }
  }
  // release the barriers so that the next call of this body (persistent loop) can init them
  __syncthreads();
  if (tid == 0) { od_mbar_inval(&bar[0]); od_mbar_inval(&bar[1]); }
  return true;
}

template <int NT, int NEWTON, int TPT = 2>
__global__ void __launch_bounds__(NT) k_pairs_x2(const float* __restrict__ sx,
                                                 const float* __restrict__ sy,
                                                 const float* __restrict__ sz, int Npad, int chunk,
                                                 float4* __restrict__ part_hi,
                                                 float4* __restrict__ part_lo, float rho0,
                                                 float newton_r2, uint32_t* __restrict__ err,
                                                 unsigned long long* __restrict__ acc) {
  const int j0 = blockIdx.y * chunk;
  pairs_x2_body<NT, NEWTON, TPT>(sx, sy, sz, blockIdx.x, j0, min(j0 + chunk, Npad),
                                 (size_t)blockIdx.y * Npad, part_hi, part_lo, rho0, newton_r2, err,
                                 0, acc, (size_t)Npad);
}

// Fixed-point accumulators -> slab 0 of (ph, pl) as two-float sums, cleared for the next
// evaluation (the forms that read slabs: initial sums, snapshots, autotuner probes).
__global__ void k_acc_take(unsigned long long* __restrict__ acc, int Npad, float4* __restrict__ ph,
                           float4* __restrict__ pl) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Npad) return;
  float3 hi, lo;
  od_fix_take(acc + i, (size_t)Npad, hi, lo);
  ph[i] = make_float4(hi.x, hi.y, hi.z, 0.f);
  pl[i] = make_float4(lo.x, lo.y, lo.z, 0.f);
}

__global__ void k_aos_to_soa(const float4* __restrict__ pos, int Npad, float* __restrict__ sx,
                             float* __restrict__ sy, float* __restrict__ sz) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Npad) return;
  const float4 p = pos[i];
  sx[i] = p.x; sy[i] = p.y; sz[i] = p.z;
}

// sum the jsplit partial slabs of ion i into (hi, lo)
__device__ __forceinline__ void reduce_parts(const float4* __restrict__ ph,
                                             const float4* __restrict__ pl, int Npad, int jsplit,
                                             int i, float3& hi, float3& lo) {
  hi = make_float3(0.f, 0.f, 0.f);
  lo = make_float3(0.f, 0.f, 0.f);
  for (int s = 0; s < jsplit; s++) {
    float4 a = ph[(size_t)s * Npad + i], b = pl[(size_t)s * Npad + i];
    od_acc2(hi.x, lo.x, a.x); lo.x += b.x;
    od_acc2(hi.y, lo.y, a.y); lo.y += b.y;
    od_acc2(hi.z, lo.z, a.z); lo.z += b.z;
  }
}

__global__ void k_reduce(int Npad, int jsplit, const float4* __restrict__ ph,
                         const float4* __restrict__ pl, float4* __restrict__ fhi,
                         float4* __restrict__ flo) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Npad) return;
  float3 hi, lo;
  reduce_parts(ph, pl, Npad, jsplit, i, hi, lo);
  fhi[i] = make_float4(hi.x, hi.y, hi.z, 0.f);
  flo[i] = make_float4(lo.x, lo.y, lo.z, 0.f);
}

// ============================================================== K1: collisions, kick, drift
__device__ __forceinline__ void collide(const od_dparams& p, uint32_t ion, uint32_t step,
                                        float4& v) {
  if (p.coll == OD_COLL_PER_DOF) {
    // opendust.py:869-873: collision = step(p_collision - uniform) per velocity component;
    // u01 is a multiple of 2^-24, so u <= p_coll is an integer comparison (exact)
    od_u4 w = od_draw(p, ion, step, OD_RNG_COLL_TEST);
    const bool c0 = (int)(w.x >> 8) <= p.pcoll_int, c1 = (int)(w.y >> 8) <= p.pcoll_int,
               c2 = (int)(w.z >> 8) <= p.pcoll_int;
    if (c0 | c1 | c2) {
      od_u4 g = od_draw(p, ion, step, OD_RNG_COLL_GAUSS);
      float gx, gy, gz, dummy;
      od_gauss2(g.x, g.y, gx, gy);
      od_gauss2(g.z, g.w, gz, dummy);
      if (c0) v.x = p.vT * gx;
      if (c1) v.y = p.vT * gy;
      if (c2) v.z = p.vT * gz;
    }
  } else if (p.coll == OD_COLL_MFP) {
    // null collision: candidate with probability Pmax = 1 - exp(-vmax/mfp), real with
    // probability |v|/vmax; an ion faster than the majorant vmax (accelerated by a grain or the
    // field) collides with its own probability 1 - exp(-|v| d_t/mfp) instead of being capped.
    // The decisions are the oracle's FP64 ones against the FP32 majorant: FP32 decides when it
    // is 1e-5 away from the boundary (its error is ~2e-7), FP64 inside that band (the squares of
    // FP32 components are exact in FP64, so (x^2 + y^2) + z^2 rounds the same with or without
    // FMA contraction); u < Pmax is an integer comparison (u is a multiple of 2^-24).
    od_u4 w = od_draw(p, ion, step, OD_RNG_MFP_TEST);
    const float vm = p.vmax_mfp, vm2 = vm * vm;
    const float sp2f = fmaf(v.x, v.x, fmaf(v.y, v.y, v.z * v.z));
    bool slow;
    if (sp2f < vm2 * (1.f - 1e-5f)) slow = true;
    else if (sp2f > vm2 * (1.f + 1e-5f)) slow = false;
    else slow = (double)v.x * v.x + (double)v.y * v.y + (double)v.z * v.z <= (double)vm * vm;
    bool hit;
    if (slow) {
      hit = false;
      if ((w.x >> 8) < p.pmax_int) {
        const float t = od_u01(w.y) * vm, spf = sqrtf(sp2f);
        if (t < spf * (1.f - 1e-5f)) hit = true;
        else if (t > spf * (1.f + 1e-5f)) hit = false;
        else hit = (double)od_u01(w.y) * (double)vm <
                   sqrt((double)v.x * v.x + (double)v.y * v.y + (double)v.z * v.z);
      }
    } else {  // faster than the majorant (rare)
      const double sp = sqrt((double)v.x * v.x + (double)v.y * v.y + (double)v.z * v.z);
      hit = (double)od_u01(w.z) < 1.0 - exp(-sp * p.mfp_inv_d);
    }
    if (hit) {
      od_u4 g = od_draw(p, ion, step, OD_RNG_MFP_GAUSS);
      float gx, gy, gz, dummy;
      od_gauss2(g.x, g.y, gx, gy);
      od_gauss2(g.z, g.w, gz, dummy);
      v.x = p.vT * gx; v.y = p.vT * gy; v.z = p.vT * gz;
    }
  }
}

// The drift moves the cell-relative state (rel) and writes the absolute FP32 position derived
// from it to pos and to the SoA copy.
__device__ __forceinline__ void kick_drift_body(const od_dparams& p, const od_dstate* __restrict__ ds,
                                                float4* __restrict__ rel, float4* __restrict__ pos,
                                                float4* __restrict__ vel,
                                                const float4* __restrict__ fhi,
                                                const float4* __restrict__ flo,
                                                const float* __restrict__ cq,
                                                float* __restrict__ sx, float* __restrict__ sy,
                                                float* __restrict__ sz, int i) {
  if (i >= p.N) return;
  float4 r = rel[i], v = vel[i];
  if (p.coll != OD_COLL_NONE)
    collide(p, (uint32_t)(p.ion0 + i), (uint32_t)(ds->step + ds->rng_base), v);
  const float4 gh = fhi[i], gl = flo[i];
  const float4 x0 = od_rel_abs(p, r);
  float3 a = od_ext_accel(p, cq, x0.x, x0.y, x0.z);
  const float aii = p.A_ii * od_first_kick_weight(p.force_every, ds->step);
  a.x = fmaf(aii, gh.x + gl.x, a.x);
  a.y = fmaf(aii, gh.y + gl.y, a.y);
  a.z = fmaf(aii, gh.z + gl.z, a.z);
  v.x = fmaf(0.5f, a.x, v.x); v.y = fmaf(0.5f, a.y, v.y); v.z = fmaf(0.5f, a.z, v.z);
  od_rel_drift(p, r, v.x, v.y, v.z);
  const float4 x = od_rel_abs(p, r);
  rel[i] = r;
  pos[i] = x;
  vel[i] = v;
  sx[i] = x.x; sy[i] = x.y; sz[i] = x.z;
}

__global__ void __launch_bounds__(kBlk) k_kick_drift(const od_dparams* __restrict__ dp,
                                                     const od_dstate* __restrict__ ds,
                                                     float4* __restrict__ rel,
                                                     float4* __restrict__ pos,
                                                     float4* __restrict__ vel,
                                                     const float4* __restrict__ fhi,
                                                     const float4* __restrict__ flo,
                                                     const float* __restrict__ cq,
                                                     float* __restrict__ sx, float* __restrict__ sy,
                                                     float* __restrict__ sz) {
  kick_drift_body(*dp, ds, rel, pos, vel, fhi, flo, cq, sx, sy, sz,
                  blockIdx.x * blockDim.x + threadIdx.x);
}

// ============================================================== K3: kick + flags
// all 32 lanes of a warp call this (warp ballot); i covers [0, Npad)
__device__ __forceinline__ void kick_flag_body(const od_dparams& p, const od_dstate* __restrict__ ds,
                                               const float4* __restrict__ pos,
                                               float4* __restrict__ vel,
                                               const float4* __restrict__ ph,
                                               const float4* __restrict__ pl, int jsplit,
                                               float4* __restrict__ fhi, float4* __restrict__ flo,
                                               uint32_t* __restrict__ flags,
                                               const float* __restrict__ cq, int i,
                                               unsigned long long* __restrict__ acc = nullptr) {
  int flag = 0;
  if (i < p.N) {
    // a step without an ion–ion evaluation (force interval k > 1) keeps the stored sums and
    // kicks with the grain, trap and field forces only
    float3 hi = make_float3(0.f, 0.f, 0.f), lo = make_float3(0.f, 0.f, 0.f);
    float aii = 0.f;
    if (od_evaluates(p.force_every, ds->step)) {
      // from the fixed-point accumulators (and cleared), or from the partial slabs
      if (acc) od_fix_take(acc + i, (size_t)p.Npad, hi, lo);
      else reduce_parts(ph, pl, p.Npad, jsplit, i, hi, lo);
      fhi[i] = make_float4(hi.x, hi.y, hi.z, 0.f);
      flo[i] = make_float4(lo.x, lo.y, lo.z, 0.f);
      aii = p.force_every > 1 ? p.A_ii * (float)p.force_every : p.A_ii;
    }
    const float4 x = pos[i];
    float4 v = vel[i];
    float3 a = od_ext_accel(p, cq, x.x, x.y, x.z);
    a.x = fmaf(aii, hi.x + lo.x, a.x);
    a.y = fmaf(aii, hi.y + lo.y, a.y);
    a.z = fmaf(aii, hi.z + lo.z, a.z);
    v.x = fmaf(0.5f, a.x, v.x); v.y = fmaf(0.5f, a.y, v.y); v.z = fmaf(0.5f, a.z, v.z);
    vel[i] = v;
    flag = od_flag(p, x.x, x.y, x.z) != 0;
  }
  const uint32_t ballot = __ballot_sync(0xffffffffu, flag);
  if ((threadIdx.x & 31) == 0) flags[i >> 5] = ballot;
}

__global__ void __launch_bounds__(kBlk) k_kick_flag(const od_dparams* __restrict__ dp,
                                                    const od_dstate* __restrict__ ds,
                                                    const float4* __restrict__ pos,
                                                    float4* __restrict__ vel,
                                                    const float4* __restrict__ ph,
                                                    const float4* __restrict__ pl, int jsplit,
                                                    float4* __restrict__ fhi,
                                                    float4* __restrict__ flo,
                                                    uint32_t* __restrict__ flags,
                                                    const float* __restrict__ cq,
                                                    unsigned long long* __restrict__ acc) {
  od_pdl_wait();
  od_pdl_trigger();
  kick_flag_body(*dp, ds, pos, vel, ph, pl, jsplit, fhi, flo, flags, cq,
                 blockIdx.x * blockDim.x + threadIdx.x, acc);  // grid covers Npad exactly
}

__global__ void __launch_bounds__(kBlk) k_flags_only(const od_dparams* __restrict__ dp, int n,
                                                     const float4* __restrict__ pos,
                                                     uint32_t* __restrict__ flags) {
  const od_dparams& p = *dp;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int flag = 0;
  if (i < n) {
    const float4 x = pos[i];
    flag = od_flag(p, x.x, x.y, x.z) != 0;
  }
  const uint32_t ballot = __ballot_sync(0xffffffffu, flag);
  if ((threadIdx.x & 31) == 0) flags[i >> 5] = ballot;
}

// ============================================================== K4: compaction + re-injection
// Order-preserving compaction of the ballot words by one 1024-thread block: each thread owns
// a contiguous range of words, counts its bits, takes an exclusive block scan, then writes
// its indices in increasing order. Returns the total (same in every thread).
constexpr int kCT = 1024;
__device__ int build_list(const uint32_t* __restrict__ flags, int nwords, int32_t* __restrict__ list) {
  __shared__ int s_warp[32];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int per = (nwords + kCT - 1) / kCT;
  const int w0 = min(tid * per, nwords), w1 = min(w0 + per, nwords);
  int cnt = 0;
  for (int w = w0; w < w1; w++) cnt += __popc(__ldcg(flags + w));
  int incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) s_warp[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int v = s_warp[lane], iv = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, iv, o);
      if (lane >= o) iv += y;
    }
    s_warp[lane] = iv - v;  // exclusive prefix of warp totals
  }
  __syncthreads();
  int off = s_warp[wid] + incl - cnt;
  for (int w = w0; w < w1; w++) {
    uint32_t b = __ldcg(flags + w);
    while (b) {
      int bit = __ffs(b) - 1;
      list[off++] = w * 32 + bit;
      b &= b - 1;
    }
  }
  // total = exclusive prefix of last warp + its inclusive total
  __shared__ int s_total;
  if (tid == kCT - 1) s_total = off;
  __syncthreads();
  int total = s_total;
  __syncthreads();
  return total;
}

// FP64 block sum over 1024 threads in a fixed order (deterministic)
__device__ double block_sum_1024(double v) {
  __shared__ double s_red[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) s_red[wid] = v;
  __syncthreads();
  double r = 0;
  if (wid == 0) {
    r = s_red[lane];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    if (lane == 0) s_red[0] = r;
  }
  __syncthreads();
  r = s_red[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ float tab_eval(const od_dparams& p, int t, float u) {
  // the first node i in [1, n - 1) with u <= txi[i], else n - 1 (txi is a CDF: non-decreasing),
  // by bisection
  const int n = p.tn[t];
  const double ud = u;
  int lo = 1, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (ud > p.txi[t][mid]) lo = mid + 1;
    else hi = mid;
  }
  const int i = lo;
  return p.tv[t][i - 1] + (u - (float)p.txi[t][i - 1]) * p.tsl[t][i];
}

// Re-injection of one ion (opendust.py:923-975); draws keyed by (ion, step).
__device__ void inject_one(const od_dparams& p, uint32_t ion, uint32_t step, float4& x, float4& v) {
  od_u4 w = od_draw(p, ion, step, OD_RNG_FACE);
  const double uf = od_u01(w.x);
  int face;  // 0 top, 1 side, 2 bottom
  if (uf <= p.p_t) face = 0;
  else if (uf <= p.p_t + p.p_s || p.p_b == 0.0) face = 1;
  else face = 2;
  if (face != 1) {
    const bool top = face == 0;
    w = od_draw(p, ion, step, top ? OD_RNG_TOP_V : OD_RNG_BOT_V);
    float gx, gy;
    od_gauss2(w.x, w.y, gx, gy);
    const float vz = tab_eval(p, top ? OD_TAB_TOP : OD_TAB_BOTTOM, od_u01(w.z));
    v = make_float4(p.vT * gx, p.vT * gy, vz, 0.f);
    w = od_draw(p, ion, step, top ? OD_RNG_TOP_X : OD_RNG_BOT_X);
    const float rr = p.Rh * sqrtf(od_u01(w.x));
    float s, c;
    sincospif(2.0f * od_u01(w.y), &s, &c);
    x = make_float4(rr * c, rr * s, top ? -p.Hh_half : p.Hh_half, 0.f);
  } else {
    w = od_draw(p, ion, step, OD_RNG_SIDE_X);
    float s, c;
    sincospif(2.0f * od_u01(w.x), &s, &c);
    x = make_float4(p.Rh * c, p.Rh * s, od_u01(w.y) * p.Hh - p.Hh_half, 0.f);
    w = od_draw(p, ion, step, OD_RNG_SIDE_V);
    float gy, gz;
    od_gauss2(w.x, w.y, gy, gz);
    const float us = od_u01(w.z);
    const float vn = tab_eval(p, OD_TAB_SIDE, us);
    const float cx = x.x / p.Rh, cy = x.y / p.Rh;
    v.x = -vn * cx + p.vT * gy * cy;
    v.y = -vn * cy - p.vT * gy * cx;
    v.z = (p.dist == OD_DIST_MAXWELLIAN) ? gz * p.vT + p.vfl : tab_eval(p, OD_TAB_VZ, us);
    v.w = 0.f;
  }
}

// per-grain collected count and momentum (opendust.py:911-921) over list entries 0..K-1, in a
// fixed order (FP64; one block of kCT threads)
__device__ __forceinline__ void list_sums(const od_dparams& p, od_dstate* __restrict__ ds, int K,
                                          const int32_t* __restrict__ list_bits,
                                          const float4* __restrict__ list_v) {
  // one warp: lane l takes entries l, l + 32, ... in order, then a fixed shuffle tree (the list
  // is short: K is the number of ions that left or hit a grain this step)
  if (threadIdx.x >= 32) return;
  const int lane = threadIdx.x;
  for (int g = 0; g < p.P; g++) {
    double dn = 0, mx = 0, my = 0, mz = 0;
    for (int k = lane; k < K; k += 32)
      if ((list_bits[k] >> g) & 1) {
        const float4 v = list_v[k];
        dn += 1.0; mx += v.x; my += v.y; mz += v.z;
      }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      dn += __shfl_xor_sync(0xffffffffu, dn, o);
      mx += __shfl_xor_sync(0xffffffffu, mx, o);
      my += __shfl_xor_sync(0xffffffffu, my, o);
      mz += __shfl_xor_sync(0xffffffffu, mz, o);
    }
    if (lane == 0) { ds->dN[g] = dn; ds->M[g][0] = mx; ds->M[g][1] = my; ds->M[g][2] = mz; }
  }
}

__device__ __forceinline__ void collect_inject_body(
    const od_dparams& p, od_dstate* __restrict__ ds, float4* __restrict__ rel,
    float4* __restrict__ pos, float4* __restrict__ vel, const uint32_t* __restrict__ flags,
    int32_t* __restrict__ list,
    int32_t* __restrict__ list_bits, float4* __restrict__ list_old,
    float4* __restrict__ list_new, float4* __restrict__ list_v) {
  const int tid = threadIdx.x;
  const int K = build_list(flags, p.nwords, list);
  if (tid == 0) ds->nlist = K;
  for (int k = tid; k < K; k += kCT) {
    const int i = list[k];
    const float4 x = pos[i], v = __ldcg(vel + i);  // L2: K3's velocities
    list_bits[k] = od_flag_exact(p, x.x, x.y, x.z);
    list_old[k] = x;
    list_v[k] = v;
  }
  __syncthreads();
  // warp 0 sums the grains' collected counts and momenta while warps 1.. re-inject
  list_sums(p, ds, K, list_bits, list_v);
  if (tid < 32) return;
  const uint32_t step = (uint32_t)(ds->step + ds->rng_base);
  if (p.dist == OD_DIST_MATTHEWS) {
    // the fork (chains/matthews.py:653-682): ions past |z| = H/2 or inside a grain re-enter
    // through the top face; ions past the side wall keep their position and have the radial
    // velocity component reversed, with the normal taken before any re-injection
    const int grains = (1 << p.P) - 1;
    for (int k = tid - 32; k < K; k += kCT - 32) {
      const int i = list[k];
      const int bits = list_bits[k];
      const float4 xo = list_old[k];
      float4 x = xo, v = list_v[k];
      if (bits & (grains | (1 << 29))) {
        inject_one(p, (uint32_t)(p.ion0 + i), step, x, v);
        const float4 r = od_rel_encode(p, x.x, x.y, x.z);
        x = od_rel_abs(p, r);
        rel[i] = r;
      }
      if (bits & (1 << 30)) {
        const float rr = sqrtf(fmaf(xo.x, xo.x, xo.y * xo.y));
        const float nx = xo.x / rr, ny = xo.y / rr;
        const float vn = fmaf(v.x, nx, v.y * ny);          // dot(v, n)
        const float vt = fmaf(v.x, ny, -v.y * nx);         // dot(v, tau), tau = (y, -x)/rho
        v.x = fmaf(-vn, nx, vt * ny);
        v.y = fmaf(-vn, ny, -vt * nx);
      }
      pos[i] = x;
      vel[i] = v;
      list_new[k] = x;
    }
    return;
  }
  for (int k = tid - 32; k < K; k += kCT - 32) {
    const int i = list[k];
    float4 x, v;
    inject_one(p, (uint32_t)(p.ion0 + i), step, x, v);
    const float4 r = od_rel_encode(p, x.x, x.y, x.z);
    x = od_rel_abs(p, r);
    rel[i] = r;
    pos[i] = x;
    vel[i] = v;
    list_new[k] = x;
  }
}

__global__ void __launch_bounds__(kCT) k_collect_inject(
    const od_dparams* __restrict__ dp, od_dstate* __restrict__ ds, float4* __restrict__ rel,
    float4* __restrict__ pos, float4* __restrict__ vel, const uint32_t* __restrict__ flags,
    int32_t* __restrict__ list, int32_t* __restrict__ list_bits, float4* __restrict__ list_old,
    float4* __restrict__ list_new, float4* __restrict__ list_v) {
  od_pdl_wait();
  od_pdl_trigger();
  collect_inject_body(*dp, ds, rel, pos, vel, flags, list, list_bits, list_old, list_new, list_v);
}

// list + per-grain counts of a snapshot (no state change)
__global__ void __launch_bounds__(kCT) k_list_only(const od_dparams* __restrict__ dp, int nwords,
                                                   const float4* __restrict__ pos,
                                                   const uint32_t* __restrict__ flags,
                                                   int32_t* __restrict__ list,
                                                   int32_t* __restrict__ list_bits,
                                                   double* __restrict__ counts) {
  const od_dparams& p = *dp;
  const int tid = threadIdx.x;
  const int K = build_list(flags, nwords, list);
  for (int k = tid; k < K; k += kCT) {
    const float4 x = pos[list[k]];
    list_bits[k] = od_flag_exact(p, x.x, x.y, x.z);
  }
  __syncthreads();
  for (int g = 0; g < p.P; g++) {
    double dn = 0;
    for (int k = tid; k < K; k += kCT) dn += (list_bits[k] >> g) & 1;
    dn = block_sum_1024(dn);
    if (tid == 0) counts[g] = dn;
  }
  if (tid == 0) counts[OD_MAX_GRAINS] = K;
}

// ============================================================== K5: correction + orbit sums
__device__ __forceinline__ double block_sum_256(double v, double* s_red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) s_red[wid] = v;
  __syncthreads();
  double r = 0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kBlk / 32; w++) r += s_red[w];
  __syncthreads();
  return r;  // valid in thread 0
}

// block blk of nb + nrec: blocks [0, nb) correct and sum orbit terms, the rest recompute the
// re-injected ions' sums
__device__ __forceinline__ void correct_orbit_body(
    const od_dparams& p, const od_dstate* __restrict__ ds,
    const float4* __restrict__ pos, float4* __restrict__ fhi, float4* __restrict__ flo,
    const uint32_t* __restrict__ flags, const int32_t* __restrict__ list,
    const float4* __restrict__ list_old, const float4* __restrict__ list_new,
    double* __restrict__ orbit_part, int nb, int blk, int nrec,
    const float* __restrict__ ssx = nullptr, const float* __restrict__ ssy = nullptr,
    const float* __restrict__ ssz = nullptr, int nsrc = 0) {
  // ssx..ssz (a shard of a larger run): the list holds the re-injected ions of every shard by
  // global index, the re-injected ions' full sums run over the nsrc source positions ssx..ssz
  // (all shards' ions, re-injected ones at their new positions), and only this shard's own
  // entries (global index - p.ion0 in [0, p.N)) are written
  const int K = ds->nlist;
  const int tid = threadIdx.x;
  if (blk < nb) {
    const int i = blk * kBlk + tid;
    const bool live = i < p.N;
    const float4 x = live ? pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    // orbit sums (opendust.py:977-1037): exp(-r)(x_p - x)(1/r^3 + 1/r^2), lambda units; FP64
    // warp trees for every component, then the 8 warps in order
    __shared__ double s_orb[kBlk / 32][OD_MAX_GRAINS * 3];
    const int lane = tid & 31, w = tid >> 5;
    for (int g = 0; g < p.P; g++) {
      float tx = 0.f, ty = 0.f, tz = 0.f;
      if (live) {
        const float dx = (p.gxh[g] - x.x) + p.gxl[g];
        const float dy = (p.gyh[g] - x.y) + p.gyl[g];
        const float dz = (p.gzh[g] - x.z) + p.gzl[g];
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const float ri = rsqrtf(r2);
        const float r = r2 * ri;
        const float e = od_ex2(r * OD_NLOG2E);
        const float t = e * ri * ri * (ri + 1.0f);
        tx = dx * t; ty = dy * t; tz = dz * t;
      }
      double sx = tx, sy = ty, sz = tz;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        sy += __shfl_xor_sync(0xffffffffu, sy, o);
        sz += __shfl_xor_sync(0xffffffffu, sz, o);
      }
      if (lane == 0) { s_orb[w][3 * g] = sx; s_orb[w][3 * g + 1] = sy; s_orb[w][3 * g + 2] = sz; }
    }
    __syncthreads();
    if (tid < 3 * p.P) {
      double v = 0;
      for (int k = 0; k < kBlk / 32; k++) v += s_orb[k][tid];
      orbit_part[(size_t)blk * p.P * 3 + tid] = v;
    }
    // move the ion–ion sums of unflagged ions to the re-injected positions (the entries are
    // loaded kU at a time so that their loads overlap; the terms are added in list order)
    if (K > 0 && live && !((flags[i >> 5] >> (i & 31)) & 1u)) {
      float gx = 0.f, gy = 0.f, gz = 0.f;
      const bool cut = p.method == OD_FORCE_CUTOFF;
      constexpr int kU = 4;
      for (int k0 = 0; k0 < K; k0 += kU) {
        float4 qn[kU], qo[kU];
#pragma unroll
        for (int u = 0; u < kU; u++)
          if (k0 + u < K) { qn[u] = list_new[k0 + u]; qo[u] = list_old[k0 + u]; }
#pragma unroll
        for (int u = 0; u < kU; u++) {
          if (k0 + u >= K) break;
          float dx = x.x - qn[u].x, dy = x.y - qn[u].y, dz = x.z - qn[u].z;
          float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, 1e-30f)));
          float c = cut ? od_pair_c_cut(r2, p) : od_pair_c(r2, p.rho0);
          gx = fmaf(c, dx, gx); gy = fmaf(c, dy, gy); gz = fmaf(c, dz, gz);
          dx = x.x - qo[u].x; dy = x.y - qo[u].y; dz = x.z - qo[u].z;
          r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, 1e-30f)));
          c = cut ? od_pair_c_cut(r2, p) : od_pair_c(r2, p.rho0);
          gx = fmaf(-c, dx, gx); gy = fmaf(-c, dy, gy); gz = fmaf(-c, dz, gz);
        }
      }
      float4 h = fhi[i], l = flo[i];
      od_acc2(h.x, l.x, gx); od_acc2(h.y, l.y, gy); od_acc2(h.z, l.z, gz);
      fhi[i] = h;
      flo[i] = l;
    }
  } else {
    // full ion–ion sums of the re-injected ions at their new positions
    __shared__ float s_h[3][kBlk], s_l[3][kBlk];
    const bool cut = p.method == OD_FORCE_CUTOFF;
    for (int k = blk - nb; k < K; k += nrec) {
      const int i = ssx ? list[k] - p.ion0 : list[k];
      if (ssx && (i < 0 || i >= p.N)) continue;  // another shard's ion (uniform per block)
      const float4 xi = list_new[k];
      float hx = 0.f, hy = 0.f, hz = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
      float ax = 0.f, ay = 0.f, az = 0.f;
      int cnt = 0;
      const int nj = ssx ? nsrc : p.N;
      // sources j = tid, tid + kBlk, ... in that order, loaded kU at a time so that their loads
      // overlap (a load per iteration waited the full memory latency each time)
      constexpr int kU = 8;
      for (int j0 = tid; j0 < nj; j0 += kU * kBlk) {
        float4 q[kU];
#pragma unroll
        for (int u = 0; u < kU; u++) {
          const int j = j0 + u * kBlk;
          if (j < nj) q[u] = ssx ? make_float4(ssx[j], ssy[j], ssz[j], 0.f) : pos[j];
        }
#pragma unroll
        for (int u = 0; u < kU; u++) {
          if (j0 + u * kBlk >= nj) break;
          const float dx = xi.x - q[u].x, dy = xi.y - q[u].y, dz = xi.z - q[u].z;
          const float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, 1e-30f)));
          const float c = cut ? od_pair_c_cut(r2, p) : od_pair_c(r2, p.rho0);
          ax = fmaf(c, dx, ax); ay = fmaf(c, dy, ay); az = fmaf(c, dz, az);
          if (++cnt == 64) {
            od_acc2(hx, lx, ax); od_acc2(hy, ly, ay); od_acc2(hz, lz, az);
            ax = ay = az = 0.f;
            cnt = 0;
          }
        }
      }
      od_acc2(hx, lx, ax); od_acc2(hy, ly, ay); od_acc2(hz, lz, az);
      // two-float warp trees (fixed order), then the 8 warps in order
      const int lane = tid & 31, w = tid >> 5;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        float t;
        t = __shfl_xor_sync(0xffffffffu, hx, o); lx += __shfl_xor_sync(0xffffffffu, lx, o);
        od_acc2(hx, lx, t);
        t = __shfl_xor_sync(0xffffffffu, hy, o); ly += __shfl_xor_sync(0xffffffffu, ly, o);
        od_acc2(hy, ly, t);
        t = __shfl_xor_sync(0xffffffffu, hz, o); lz += __shfl_xor_sync(0xffffffffu, lz, o);
        od_acc2(hz, lz, t);
      }
      if (lane == 0) {
        s_h[0][w] = hx; s_h[1][w] = hy; s_h[2][w] = hz;
        s_l[0][w] = lx; s_l[1][w] = ly; s_l[2][w] = lz;
      }
      __syncthreads();
      if (tid < 3) {
        float h = 0.f, l = 0.f;
        for (int u = 0; u < kBlk / 32; u++) { od_acc2(h, l, s_h[tid][u]); l += s_l[tid][u]; }
        s_h[tid][0] = h;
        s_l[tid][0] = l;
      }
      __syncthreads();
      if (tid == 0) {
        fhi[i] = make_float4(s_h[0][0], s_h[1][0], s_h[2][0], 0.f);
        flo[i] = make_float4(s_l[0][0], s_l[1][0], s_l[2][0], 0.f);
      }
      __syncthreads();
    }
  }
}

__global__ void __launch_bounds__(kBlk) k_correct_orbit(
    const od_dparams* __restrict__ dp, od_dstate* __restrict__ ds,
    const float4* __restrict__ pos, float4* __restrict__ fhi, float4* __restrict__ flo,
    const uint32_t* __restrict__ flags, const int32_t* __restrict__ list,
    const float4* __restrict__ list_old, const float4* __restrict__ list_new,
    double* __restrict__ orbit_part, int nb) {
  correct_orbit_body(*dp, ds, pos, fhi, flo, flags, list, list_old, list_new, orbit_part, nb,
                     blockIdx.x, gridDim.x - nb);
}

// ============================================================== K6: FP64 host-tail on device
// opendust.py:1117-1202 (charge), :1205-1235 (dust–dust), :1237-1331 (orbit + out-of-domain),
// :1333-1365 (collect), :1367-1383 (field)
// charge of grain g after a step with dN collected ions (opendust.py:1117-1202), from the
// host-precomputed constants of tail_consts
__device__ __forceinline__ double charge_update(const od_dparams& p, int g, double q_prev,
                                                double dN) {
  const double ge = p.ge_pref[g] * exp(p.ge_arg[g] * q_prev);
  if (p.gmethod[g] == OD_CHARGE_CONSISTENT) return q_prev + (dN * p.q_s + ge);
  if (p.gmethod[g] == OD_CHARGE_OML) return q_prev + (fma(p.oml_b[g], q_prev, p.oml_a[g]) + ge);
  return q_prev;
}

// FP64 tail of one step (opendust.py:1117-1383): orbit sums over the blocks' partials in a fixed
// order (all components at once), then one thread per grain for the charge update and the
// grain forces, from the host-precomputed constants.
__device__ __forceinline__ void tail_body(const od_dparams& p, od_dstate* __restrict__ ds,
                                          const double* __restrict__ orbit_part, int nb,
                                          double* __restrict__ s_q, double* __restrict__ s_orbit,
                                          double* __restrict__ s_collect,
                                          double* __restrict__ s_dust,
                                          double* __restrict__ s_field, float* __restrict__ cq) {
  __shared__ double s_red[kBlk / 32][OD_MAX_GRAINS * 3];
  __shared__ double S[OD_MAX_GRAINS * 3];
  __shared__ double qn[OD_MAX_GRAINS];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int P = p.P, nc = P * 3;
  for (int g = 0; g < P; g++) {
    double v[3] = {0, 0, 0};
    // L2 loads: the partials may come from other blocks of the same launch (fused tail); the
    // three components of a grain are loaded together so that their latencies overlap
    for (int b = tid; b < nb; b += kBlk) {
      const double* o = orbit_part + (size_t)b * nc + 3 * g;
      const double a0 = __ldcg(o), a1 = __ldcg(o + 1), a2 = __ldcg(o + 2);
      v[0] += a0; v[1] += a1; v[2] += a2;
    }
#pragma unroll
    for (int d = 0; d < 3; d++) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[d] += __shfl_xor_sync(0xffffffffu, v[d], o);
      if (lane == 0) s_red[w][3 * g + d] = v[d];
    }
  }
  const int64_t step = ds->step;
  if (tid < P)
    qn[tid] = step > 0 ? charge_update(p, tid, ds->q_param[tid], ds->dN[tid]) : ds->q_param[tid];
  __syncthreads();
  if (tid < nc) {
    double v = 0;
    for (int k = 0; k < kBlk / 32; k++) v += s_red[k][tid];
    S[tid] = v;
  }
  __syncthreads();
  const bool avg = step >= p.avg_start;
  if (tid < P) {
    const int g = tid;
    double fd[3] = {0, 0, 0};
    for (int j = 0; j < P; j++) {
      if (j == g) continue;
      fd[0] = fma(qn[j], p.dd[g][j][0], fd[0]);
      fd[1] = fma(qn[j], p.dd[g][j][1], fd[1]);
      fd[2] = fma(qn[j], p.dd[g][j][2], fd[2]);
    }
    const double so = qn[g] * p.k * p.q_s / (p.lam * p.lam);
    const double sc = p.vunit * p.m_s / p.dt;
    double vals[13];
    vals[0] = qn[g];
    for (int d = 0; d < 3; d++) {
      vals[1 + d] = S[g * 3 + d] * so + qn[g] * p.gout[g][d];
      vals[4 + d] = ds->M[g][d] * sc;
      vals[7 + d] = qn[g] * fd[d];
      vals[10 + d] = d == 2 ? qn[g] * p.gfield[g] : 0.0;
    }
    const size_t r = (size_t)step * P + g;
    s_q[r] = vals[0];
    for (int d = 0; d < 3; d++) {
      s_orbit[r * 3 + d] = vals[1 + d];
      s_collect[r * 3 + d] = vals[4 + d];
      s_dust[r * 3 + d] = vals[7 + d];
      s_field[r * 3 + d] = vals[10 + d];
    }
    if (avg)
      for (int m = 0; m < 13; m++) ds->avg[g][m] += vals[m];
    ds->q_param[g] = qn[g];
    cq[g] = (float)(p.A_id_d * qn[g]);
  }
  __syncthreads();  // every grain has read ds->step
  if (tid == 0) {
    if (avg) ds->n_avg += 1;
    ds->n_inj_total += ds->nlist;
    ds->step = step + 1;
  }
}

__global__ void __launch_bounds__(kBlk) k_tail(const od_dparams* __restrict__ dp,
                                               od_dstate* __restrict__ ds,
                                               const double* __restrict__ orbit_part, int nb,
                                               double* __restrict__ s_q, double* __restrict__ s_orbit,
                                               double* __restrict__ s_collect,
                                               double* __restrict__ s_dust,
                                               double* __restrict__ s_field, float* __restrict__ cq) {
  tail_body(*dp, ds, orbit_part, nb, s_q, s_orbit, s_collect, s_dust, s_field, cq);
}

// K5 + K6: the last of the nb orbit blocks to finish (a ticket taken after its partials are
// fenced) runs the FP64 tail over all partials, so the tail needs no launch of its own.
__global__ void __launch_bounds__(kBlk) k_correct_orbit_tail(
    const od_dparams* __restrict__ dp, od_dstate* __restrict__ ds,
    const float4* __restrict__ pos, float4* __restrict__ fhi, float4* __restrict__ flo,
    const uint32_t* __restrict__ flags, const int32_t* __restrict__ list,
    const float4* __restrict__ list_old, const float4* __restrict__ list_new,
    double* __restrict__ orbit_part, int nb, double* __restrict__ s_q,
    double* __restrict__ s_orbit, double* __restrict__ s_collect, double* __restrict__ s_dust,
    double* __restrict__ s_field, float* __restrict__ cq) {
  od_pdl_wait();
  correct_orbit_body(*dp, ds, pos, fhi, flo, flags, list, list_old, list_new, orbit_part, nb,
                     blockIdx.x, gridDim.x - nb);
  if ((int)blockIdx.x >= nb) return;  // re-injected ions' sums: the tail does not read them
  __shared__ bool s_last;
  __syncthreads();                    // this block's partials are written
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(&ds->ticket, 1u) == (unsigned)nb - 1u;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  tail_body(*dp, ds, orbit_part, nb, s_q, s_orbit, s_collect, s_dust, s_field, cq);
  if (threadIdx.x == 0) ds->ticket = 0u;
}


__global__ void k_set_charges(const od_dparams* __restrict__ dp, const od_dstate* __restrict__ ds,
                              float* __restrict__ cq, int P) {
  const int g = threadIdx.x;
  if (g < P) cq[g] = (float)(dp->A_id_d * ds->q_param[g]);
}

// ============================================================== trap-fit potential grid
constexpr int kTrapPts = 2048;
__global__ void __launch_bounds__(kBlk) k_trap(double Rh, double Hh, int n_r, int n_h,
                                               int64_t n_points, int64_t pts_per_block,
                                               uint32_t k0, uint32_t k1,
                                               double* __restrict__ part) {
  __shared__ float4 s_pts[kTrapPts];
  const int node = blockIdx.x * kBlk + threadIdx.x;
  const int nn = n_r * n_h;
  float gr = 0.f, gh = 0.f;
  if (node < nn) {
    const int i = node / n_h, j = node % n_h;
    gr = (float)((i == n_r - 1) ? Rh : i * (Rh / (n_r - 1)));
    gh = (float)((j == n_h - 1) ? Hh / 2.0 : j * ((Hh / 2.0) / (n_h - 1)));
  }
  const int64_t p0 = blockIdx.y * pts_per_block;
  const int64_t p1 = min(p0 + pts_per_block, n_points);
  double acc = 0.0;
  for (int64_t t0 = p0; t0 < p1; t0 += kTrapPts) {
    const int cnt = (int)min((int64_t)kTrapPts, p1 - t0);
    __syncthreads();
    for (int q = threadIdx.x; q < cnt; q += kBlk) {
      od_u4 w = od_philox((uint32_t)(t0 + q), 0u, OD_RNG_TRAP, 0u, k0, k1);
      const float r = sqrtf(od_u01(w.x));
      float s, c;
      sincospif(2.0f * od_u01(w.y), &s, &c);
      s_pts[q] = make_float4((float)Rh * r * c, (float)Rh * r * s,
                             (float)Hh * od_u01(w.z) - (float)Hh * 0.5f, 0.f);
    }
    __syncthreads();
    float a = 0.f;
    for (int q = 0; q < cnt; q++) {
      const float4 pt = s_pts[q];
      const float dx = gr - pt.x, dy = pt.y, dz = gh - pt.z;
      const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
      const float ri = od_rsqrt(fmaxf(r2, 1e-30f));
      const float r = r2 * ri;
      a += od_ex2(r * OD_NLOG2E) * od_rcp(r + 0.001f);
    }
    acc += a;
  }
  if (node < nn) part[(size_t)blockIdx.y * nn + node] = acc;
}

// ============================================================== initial state on the device
// opendust.py:373-451: rejection sampling of uniform positions in the cylinder outside every
// grain, Maxwellian (or tabulated field-driven v_z) velocities; Philox streams INIT_X / INIT_V.
__global__ void __launch_bounds__(kBlk) k_init_state(const od_dparams* __restrict__ dp,
                                                     float4* __restrict__ rel,
                                                     float4* __restrict__ pos,
                                                     float4* __restrict__ vel,
                                                     const float* __restrict__ vz_v,
                                                     const double* __restrict__ vz_cdf, int vz_n,
                                                     uint32_t* __restrict__ err) {
  const od_dparams& p = *dp;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.N) return;
  float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
  bool ok = false;
  for (uint32_t a = 0; a < 256 && !ok; a++) {
    const od_u4 w = od_draw(p, (uint32_t)i, a, OD_RNG_INIT_X);
    const float r = p.Rh * sqrtf(od_u01(w.x));
    float s, c;
    sincospif(2.0f * od_u01(w.y), &s, &c);
    x = make_float4(r * c, r * s, p.Hh * od_u01(w.z) - p.Hh_half, 0.f);
    ok = true;
    for (int g = 0; g < p.P; g++) {
      const float dx = (x.x - p.gxh[g]) - p.gxl[g], dy = (x.y - p.gyh[g]) - p.gyl[g],
                  dz = (x.z - p.gzh[g]) - p.gzl[g];
      if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= p.gr2f[g]) ok = false;
    }
  }
  if (!ok) atomicOr(err, OD_DERR_LIST);
  const od_u4 w = od_draw(p, (uint32_t)i, 0u, OD_RNG_INIT_V);
  float gx, gy, gz, dummy;
  od_gauss2(w.x, w.y, gx, gy);
  od_gauss2(w.z, w.w, gz, dummy);
  float vz;
  if (vz_n >= 2) {
    const float u = od_u01(od_draw(p, (uint32_t)i, 1u, OD_RNG_INIT_V).x);
    int k = 1;
    while (k < vz_n - 1 && (double)u > vz_cdf[k]) k++;
    const float x0 = (float)vz_cdf[k - 1], x1 = (float)vz_cdf[k];
    vz = vz_v[k - 1] + (u - x0) * (vz_v[k] - vz_v[k - 1]) / fmaxf(x1 - x0, 1e-30f);
  } else {
    vz = fmaf(p.vT, gz, p.vfl);
  }
  const float4 r = od_rel_encode(p, x.x, x.y, x.z);
  rel[i] = r;
  pos[i] = od_rel_abs(p, r);
  vel[i] = make_float4(p.vT * gx, p.vT * gy, vz, 0.f);
}

}  // namespace

cudaError_t od_launch_init_state(const od_dparams* dp, int N, float4* rel, float4* pos,
                                 float4* vel, const float* vz_v, const double* vz_cdf, int vz_n,
                                 uint32_t* err, cudaStream_t s) {
  k_init_state<<<(N + kBlk - 1) / kBlk, kBlk, 0, s>>>(dp, rel, pos, vel, vz_v, vz_cdf, vz_n, err);
  return cudaGetLastError();
}

// ============================================================== launch wrappers
// launch with programmatic stream serialization (the kernel calls od_pdl_wait first)
template <typename... KArgs, typename... Args>
static cudaError_t od_launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t s,
                                 Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

int od_num_sms(int device) {
  int n = 0;
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device);
  return n;
}

// grid.x limit for timing probes of the autotuner (0 = the full grid)
static thread_local int g_gridx_limit = 0;
static inline unsigned gx_of(int full) {
  return (unsigned)((g_gridx_limit > 0 && g_gridx_limit < full) ? g_gridx_limit : full);
}

template <int NT, int IPT, int V>
static void launch_pairs_t(const od_pair_plan& pl, const float4* pos, int Npad, float4* ph,
                           float4* plo, float rho0, uint32_t* err, cudaStream_t s) {
  dim3 grid(gx_of(Npad / (NT * IPT)), pl.jsplit);
  k_pairs<NT, IPT, V><<<grid, NT, 0, s>>>(pos, Npad, pl.chunk, ph, plo, rho0, err);
}
template <int NT, int NEWTON, int TPT = 2>
static void launch_pairs_x2(const od_pair_plan& pl, const od_pair_io& io, int Npad, float4* ph,
                            float4* plo, float rho0, uint32_t* err, cudaStream_t s) {
  dim3 grid(gx_of(Npad / (NT * TPT)), pl.jsplit);
  const float nr = 64.0f * rho0;  // Newton (2 steps) keeps 1/s within 2^-24 for r > 64 r0
  k_pairs_x2<NT, NEWTON, TPT><<<grid, NT, 0, s>>>(io.sx, io.sy, io.sz, Npad, pl.chunk, ph, plo,
                                                  rho0, nr * nr, err, io.n3);
}

cudaError_t od_launch_pairs(const od_pair_plan& pl, const od_pair_io& io, int Npad, float4* ph,
                            float4* plo, float rho0, uint32_t* err, cudaStream_t s, bool take) {
  if (pl.variant == 7) return od_launch_pairs_n3(pl, io, Npad, ph, plo, rho0, s, take);
  const int key = pl.nt * 100 + pl.ipt * 10 + pl.variant;
  const float4* pos = io.pos;
  switch (key) {
    case 12810: launch_pairs_t<128, 1, 0>(pl, pos, Npad, ph, plo, rho0, err, s); break;
    case 12820: launch_pairs_t<128, 2, 0>(pl, pos, Npad, ph, plo, rho0, err, s); break;
    case 25610: launch_pairs_t<256, 1, 0>(pl, pos, Npad, ph, plo, rho0, err, s); break;
    case 25620: launch_pairs_t<256, 2, 0>(pl, pos, Npad, ph, plo, rho0, err, s); break;
    case 12811: launch_pairs_t<128, 1, 1>(pl, pos, Npad, ph, plo, rho0, err, s); break;
    case 25611: launch_pairs_t<256, 1, 1>(pl, pos, Npad, ph, plo, rho0, err, s); break;
    case 25621: launch_pairs_t<256, 2, 1>(pl, pos, Npad, ph, plo, rho0, err, s); break;
    case 12822: launch_pairs_x2<128, 0>(pl, io, Npad, ph, plo, rho0, err, s); break;
    case 25622: launch_pairs_x2<256, 0>(pl, io, Npad, ph, plo, rho0, err, s); break;
    case 12823: launch_pairs_x2<128, 1>(pl, io, Npad, ph, plo, rho0, err, s); break;
    case 25623: launch_pairs_x2<256, 1>(pl, io, Npad, ph, plo, rho0, err, s); break;
    case 12824: launch_pairs_x2<128, 2>(pl, io, Npad, ph, plo, rho0, err, s); break;
    case 25624: launch_pairs_x2<256, 2>(pl, io, Npad, ph, plo, rho0, err, s); break;
    case 12815: launch_pairs_x2<128, 0, 1>(pl, io, Npad, ph, plo, rho0, err, s); break;
    case 25615: launch_pairs_x2<256, 0, 1>(pl, io, Npad, ph, plo, rho0, err, s); break;
    case 12816: launch_pairs_x2<128, 2, 1>(pl, io, Npad, ph, plo, rho0, err, s); break;
    case 25616: launch_pairs_x2<256, 2, 1>(pl, io, Npad, ph, plo, rho0, err, s); break;
    default: return cudaErrorInvalidValue;
  }
  // variants 2-6 with accumulators (io.n3): into slab 0 unless the caller takes them itself
  if (io.n3 && pl.variant >= 2 && take)
    k_acc_take<<<(Npad + 255) / 256, 256, 0, s>>>(io.n3, Npad, ph, plo);
  return cudaGetLastError();
}

cudaError_t od_launch_pairs_probe(const od_pair_plan& pl, const od_pair_io& io, int Npad,
                                  int gridx_limit, float4* ph, float4* plo, float rho0,
                                  uint32_t* err, cudaStream_t s) {
  g_gridx_limit = gridx_limit;
  cudaError_t e = od_launch_pairs(pl, io, Npad, ph, plo, rho0, err, s);
  g_gridx_limit = 0;
  return e;
}

cudaError_t od_launch_aos_to_soa(const float4* pos, int Npad, float* sx, float* sy, float* sz,
                                 cudaStream_t s) {
  k_aos_to_soa<<<(Npad + kBlk - 1) / kBlk, kBlk, 0, s>>>(pos, Npad, sx, sy, sz);
  return cudaGetLastError();
}

cudaError_t od_launch_reduce(const od_dparams* dp, int Npad, int jsplit, const float4* ph,
                             const float4* pl, float4* fhi, float4* flo, cudaStream_t s) {
  (void)dp;
  k_reduce<<<(Npad + kBlk - 1) / kBlk, kBlk, 0, s>>>(Npad, jsplit, ph, pl, fhi, flo);
  return cudaGetLastError();
}

cudaError_t od_launch_force(const od_force_ctx& fc, const od_pair_io& io, int n, int Npad,
                            float4* part_hi, float4* part_lo, uint32_t* err, cudaStream_t s,
                            bool take) {
  if (fc.cut)
    return od_launch_cutoff(*fc.cut, io.pos, n, Npad, part_hi, part_lo, fc.rho0, fc.rc, fc.rs, err,
                            fc.pair_count, s);
  return od_launch_pairs(fc.plan, io, Npad, part_hi, part_lo, fc.rho0, err, s, take);
}

// part 0: K1 (kick/drift); part 1: K2 (ion–ion sums); part 2: K3..K6
cudaError_t od_launch_step_part(int part, const od_dparams* dp, od_dstate* ds, const od_dbufs& b,
                                int N, int Npad, int P, const od_force_ctx& fc, int nrec,
                                cudaStream_t s) {
  (void)P;
  const int nb = Npad / kBlk;
  if (part == 0) {
    k_kick_drift<<<(N + kBlk - 1) / kBlk, kBlk, 0, s>>>(dp, ds, b.rel, b.pos, b.vel, b.fhi, b.flo, b.cq,
                                                        b.sx, b.sy, b.sz);
    return cudaGetLastError();
  }
  // with accumulators (fc.acc) K3 takes the ion–ion sums from them
  if (part == 1)
    return od_launch_force(fc, od_pair_io{b.pos, b.sx, b.sy, b.sz, b.n3}, N, Npad, b.part_hi, b.part_lo,
                           &ds->err, s, fc.acc == nullptr);
  const int jsplit = fc.cut ? 1 : fc.plan.jsplit;
  // K3, K4 and K5 with programmatic dependent launch: each starts launching while its
  // predecessor runs and waits in od_pdl_wait for the predecessor's results
  cudaError_t e = od_launch_pdl(k_kick_flag, dim3(nb), dim3(kBlk), s, dp, ds, b.pos, b.vel,
                                (const float4*)b.part_hi, (const float4*)b.part_lo, jsplit, b.fhi,
                                b.flo, b.flags, (const float*)b.cq, fc.acc);
  if (e == cudaSuccess)
    e = od_launch_pdl(k_collect_inject, dim3(1), dim3(kCT), s, dp, ds, b.rel, b.pos, b.vel,
                      (const uint32_t*)b.flags, b.list, b.list_bits, b.list_old, b.list_new,
                      b.list_v);
  if (e == cudaSuccess)
    e = od_launch_pdl(k_correct_orbit_tail, dim3(nb + nrec), dim3(kBlk), s, dp, ds,
                      (const float4*)b.pos, b.fhi, b.flo, (const uint32_t*)b.flags,
                      (const int32_t*)b.list, (const float4*)b.list_old,
                      (const float4*)b.list_new, b.orbit_part, nb, b.s_q, b.s_orbit,
                      b.s_collect, b.s_dust, b.s_field, b.cq);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

cudaError_t od_launch_step(const od_dparams* dp, od_dstate* ds, const od_dbufs& b, int N, int Npad,
                           int P, const od_force_ctx& fc, int nrec, cudaStream_t s) {
  for (int part = 0; part < 3; part++) {
    cudaError_t e = od_launch_step_part(part, dp, ds, b, N, Npad, P, fc, nrec, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// FP32 FMA throughput probe: 8 independent FMA chains per thread, 8 blocks of 256 per SM.
// The body is unrolled 16 times (128 FMAs per loop trip), so the loop counter and branch cost
// about 2 % of the issue slots.
__global__ void k_ffma_probe(float* out, float a, float b, int iters) {
  float x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5,
        x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; i += 16) {
#pragma unroll
    for (int u = 0; u < 16; u++) {
      x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
      x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

cudaError_t od_run_fp32_probe(int device, double* tflops) {
  const int blocks = od_num_sms(device) * 8, threads = 256, iters = 1 << 14;
  float* out = nullptr;
  cudaError_t e = cudaMalloc(&out, sizeof(float) * blocks * threads);
  if (e != cudaSuccess) return e;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int r = 0; r < 6; r++) {
    cudaEventRecord(e0);
    k_ffma_probe<<<blocks, threads>>>(out, 0.999f, 0.001f, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms;
    cudaEventElapsedTime(&ms, e0, e1);
    if (r >= 2 && ms < best) best = ms;
  }
  e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  *tflops = 2.0 * 8.0 * (double)iters * blocks * threads / (best * 1e-3) / 1e12;
  return e;
}

cudaError_t od_launch_snapshot_flags(const od_dparams* dp, int n, int Npad, const float4* pos,
                                     uint32_t* flags, int32_t* list, int32_t* list_bits,
                                     double* counts, cudaStream_t s) {
  k_flags_only<<<Npad / kBlk, kBlk, 0, s>>>(dp, n, pos, flags);
  k_list_only<<<1, kCT, 0, s>>>(dp, Npad / 32, pos, flags, list, list_bits, counts);
  return cudaGetLastError();
}

cudaError_t od_launch_set_charges(const od_dparams* dp, od_dstate* ds, float* cq, int P,
                                  cudaStream_t s) {
  k_set_charges<<<1, 32, 0, s>>>(dp, ds, cq, P);
  return cudaGetLastError();
}

cudaError_t od_launch_trap(double Rh, double Hh, int n_r, int n_h, int64_t n_points, uint64_t seed,
                           double* part, int nchunks, cudaStream_t s) {
  const int nn = n_r * n_h;
  const int64_t per = (n_points + nchunks - 1) / nchunks;
  dim3 grid((nn + kBlk - 1) / kBlk, nchunks);
  k_trap<<<grid, kBlk, 0, s>>>(Rh, Hh, n_r, n_h, n_points, per, (uint32_t)(seed & 0xffffffffu),
                               (uint32_t)(seed >> 32), part);
  return cudaGetLastError();
}

// ============================================================== scratch-array variant
// Kernels behind od_ion_forces_static: the same packed all-pairs kernel, reading positions
// and writing partial sums in a caller-independent scratch region (see od_api.cu).
namespace {
__global__ void k_static_pack(const double* __restrict__ pos, int n, int Npad, double inv_lam,
                              float* __restrict__ sx, float* __restrict__ sy,
                              float* __restrict__ sz) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Npad) return;
  if (i < n) {
    sx[i] = (float)(pos[3 * i] * inv_lam);
    sy[i] = (float)(pos[3 * i + 1] * inv_lam);
    sz[i] = (float)(pos[3 * i + 2] * inv_lam);
  } else {
    sx[i] = OD_SENTINEL; sy[i] = OD_SENTINEL; sz[i] = OD_SENTINEL;
  }
}

__global__ void k_static_finish(const float4* __restrict__ ph, const float4* __restrict__ pl,
                                int n, int Npad, int jsplit, double scale,
                                double* __restrict__ force) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float3 hi, lo;
  reduce_parts(ph, pl, Npad, jsplit, i, hi, lo);
  force[3 * i] = scale * ((double)hi.x + (double)lo.x);
  force[3 * i + 1] = scale * ((double)hi.y + (double)lo.y);
  force[3 * i + 2] = scale * ((double)hi.z + (double)lo.z);
}
}  // namespace

cudaError_t od_launch_static_forces(const od_static_view& v, const double* pos, int n, double lam,
                                    double r0, double scale, double* force, cudaStream_t s) {
  const int Npad = ((n + OD_PAD - 1) / OD_PAD) * OD_PAD;
  int jsplit = v.max_split < Npad / OD_TJ ? v.max_split : Npad / OD_TJ;
  int chunk = (Npad + jsplit - 1) / jsplit;
  chunk = ((chunk + OD_TJ - 1) / OD_TJ) * OD_TJ;
  jsplit = (Npad + chunk - 1) / chunk;
  k_static_pack<<<(Npad + kBlk - 1) / kBlk, kBlk, 0, s>>>(pos, n, Npad, 1.0 / lam, v.sx, v.sy, v.sz);
  const float rho0 = (float)(r0 / lam);
  const float nr = 64.0f * rho0;
  dim3 grid(Npad / 512, jsplit);
  k_pairs_x2<256, 0><<<grid, 256, 0, s>>>(v.sx, v.sy, v.sz, Npad, chunk, v.part_hi, v.part_lo,
                                          rho0, nr * nr, v.err, nullptr);  // partial slabs
  k_static_finish<<<(n + kBlk - 1) / kBlk, kBlk, 0, s>>>(v.part_hi, v.part_lo, n, Npad, jsplit,
                                                        scale, force);
  return cudaGetLastError();
}

// ============================================================== batched step
// Many independent simulations advance together: every stage of the step is one launch for
// the whole batch. Blocks of the ion-parallel stages look up (simulation, local block) in a
// table; the all-pairs stage is one persistent launch whose blocks take work items
// (simulation, 256-target block, source range) from a device counter, largest items first;
// compaction/re-injection and the FP64 tail run one block per simulation. Each simulation
// keeps its own buffers, source split and partial slabs, so its results are bitwise the
// results of the same simulation stepped alone.
namespace {

__global__ void __launch_bounds__(kBlk) k_b_kick_drift(const od_simdesc* __restrict__ sims,
                                                       const int2* __restrict__ blk) {
  const int2 e = blk[blockIdx.x];
  const od_simdesc& d = sims[e.x];
  kick_drift_body(*d.dp, d.ds, d.b.rel, d.b.pos, d.b.vel, d.b.fhi, d.b.flo, d.b.cq, d.b.sx, d.b.sy, d.b.sz,
                  e.y * kBlk + threadIdx.x);
}

__global__ void __launch_bounds__(256) k_b_pairs(const od_simdesc* __restrict__ sims,
                                                 const int4* __restrict__ items, int nitems,
                                                 unsigned int* __restrict__ next,
                                                 uint32_t* __restrict__ err) {
  __shared__ int s_item;
  for (;;) {
    if (threadIdx.x == 0) s_item = (int)atomicAdd(next, 1u);
    __syncthreads();
    const int it = s_item;
    __syncthreads();
    if (it >= nitems) return;
    const int4 w = items[it];
    const od_simdesc& d = sims[w.x];
    if (!od_evaluates(d.dp->force_every, d.ds->step)) continue;
    const bool ok = pairs_x2_body<256, 0, 1>(d.b.sx, d.b.sy, d.b.sz, w.y, w.z, w.w,
                                          (size_t)(w.z / d.chunk) * d.Npad, d.b.part_hi,
                                          d.b.part_lo, d.rho0, d.newton_r2, err);
    if (!ok) return;
  }
}

__global__ void __launch_bounds__(kBlk) k_b_kick_flag(const od_simdesc* __restrict__ sims,
                                                      const int2* __restrict__ blk) {
  const int2 e = blk[blockIdx.x];
  const od_simdesc& d = sims[e.x];
  kick_flag_body(*d.dp, d.ds, d.b.pos, d.b.vel, d.b.part_hi, d.b.part_lo, d.jsplit, d.b.fhi, d.b.flo,
                 d.b.flags, d.b.cq, e.y * kBlk + threadIdx.x);
}

__global__ void __launch_bounds__(kCT) k_b_collect_inject(const od_simdesc* __restrict__ sims) {
  const od_simdesc& d = sims[blockIdx.x];
  collect_inject_body(*d.dp, d.ds, d.b.rel, d.b.pos, d.b.vel, d.b.flags, d.b.list, d.b.list_bits,
                      d.b.list_old, d.b.list_new, d.b.list_v);
}

__global__ void __launch_bounds__(kBlk) k_b_correct_orbit(const od_simdesc* __restrict__ sims,
                                                          const int2* __restrict__ blk) {
  const int2 e = blk[blockIdx.x];
  const od_simdesc& d = sims[e.x];
  correct_orbit_body(*d.dp, d.ds, d.b.pos, d.b.fhi, d.b.flo, d.b.flags, d.b.list, d.b.list_old,
                     d.b.list_new, d.b.orbit_part, d.nb, e.y, d.nrec);
}

__global__ void __launch_bounds__(kBlk) k_b_tail(const od_simdesc* __restrict__ sims) {
  const od_simdesc& d = sims[blockIdx.x];
  tail_body(*d.dp, d.ds, d.b.orbit_part, d.nb, d.b.s_q, d.b.s_orbit, d.b.s_collect, d.b.s_dust,
            d.b.s_field, d.b.cq);
}

}  // namespace

// Screened potential of the ions at grid points (the fork's trap fit, chains/matthews.py:
// 397-421): one block per point, FP64 terms in a fixed order (per-thread strided sums, then a
// fixed tree).
__global__ void __launch_bounds__(kBlk) k_grid_potential(const float4* __restrict__ pos, int N,
                                                         const double* __restrict__ pts,
                                                         double rho0, double* __restrict__ out) {
  __shared__ double red[kBlk];
  const double gx = pts[2 * blockIdx.x], gz = pts[2 * blockIdx.x + 1];
  double acc = 0.0;
  for (int i = threadIdx.x; i < N; i += kBlk) {
    const float4 x = pos[i];
    const double dx = gx - x.x, dy = -(double)x.y, dz = gz - x.z;
    const double r = sqrt(dx * dx + dy * dy + dz * dz);
    acc += exp(-r) / (r + rho0);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = kBlk / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

cudaError_t od_launch_grid_potential(const float4* pos, int N, const double* pts, int npts,
                                     double rho0, double* out, cudaStream_t s) {
  if (npts <= 0) return cudaSuccess;
  k_grid_potential<<<npts, kBlk, 0, s>>>(pos, N, pts, rho0, out);
  return cudaGetLastError();
}

cudaError_t od_launch_batch_step(const od_batchview& v, cudaStream_t s) {
  k_b_kick_drift<<<v.nblk_ion, kBlk, 0, s>>>(v.sims, v.blk_ion);
  if (v.nitems > 0) {  // members on the directed-pair kernel
    cudaError_t e = cudaMemsetAsync(v.next, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return e;
    k_b_pairs<<<v.pair_grid, 256, 0, s>>>(v.sims, v.items, v.nitems, v.next, v.err);
  }
  cudaError_t e = od_launch_batch_pairs_n3(v, s);
  if (e != cudaSuccess) return e;
  k_b_kick_flag<<<v.nblk_ion, kBlk, 0, s>>>(v.sims, v.blk_ion);
  k_b_collect_inject<<<v.nsims, kCT, 0, s>>>(v.sims);
  k_b_correct_orbit<<<v.nblk_corr, kBlk, 0, s>>>(v.sims, v.blk_corr);
  k_b_tail<<<v.nsims, kBlk, 0, s>>>(v.sims);
  return cudaGetLastError();
}

// ============================================================== shards of one simulation
// A shard owns ions [ion0, ion0 + N) of a larger simulation and keeps every shard's positions
// as sources (SoA, nsrc entries). Its step: K1 on its own ions (writing their positions into
// the sources), the ion–ion sums of its ions over all sources, K3 and its own compaction and
// re-injection (Philox keyed by the global index); then, given every shard's list (in shard
// order, which is the global index order), the grain sums over the whole list, the new
// positions in the sources, the correction and orbit sums of its own ions; then the FP64 tail
// over every shard's orbit partials. With shard boundaries on 512-ion multiples every sum is
// taken in the single-simulation order, so the shards reproduce the single simulation's bits.

// global list (K entries) -> grain sums and the sources' re-injected positions
__global__ void __launch_bounds__(kCT) k_shard_list(const od_dparams* __restrict__ dp,
                                                    od_dstate* __restrict__ ds, int K,
                                                    const int32_t* __restrict__ gidx,
                                                    const int32_t* __restrict__ gbits,
                                                    const float4* __restrict__ gnew,
                                                    const float4* __restrict__ gv,
                                                    float* __restrict__ sx, float* __restrict__ sy,
                                                    float* __restrict__ sz) {
  if (threadIdx.x == 0) ds->nlist = K;
  list_sums(*dp, ds, K, gbits, gv);
  for (int k = threadIdx.x; k < K; k += kCT) {
    const int i = gidx[k];
    const float4 x = gnew[k];
    sx[i] = x.x; sy[i] = x.y; sz[i] = x.z;
  }
}

__global__ void __launch_bounds__(kBlk) k_shard_correct_orbit(
    const od_dparams* __restrict__ dp, const od_dstate* __restrict__ ds,
    const float4* __restrict__ pos, float4* __restrict__ fhi, float4* __restrict__ flo,
    const uint32_t* __restrict__ flags, const int32_t* __restrict__ gidx,
    const float4* __restrict__ gold, const float4* __restrict__ gnew,
    double* __restrict__ orbit_part, int nb, const float* __restrict__ sx,
    const float* __restrict__ sy, const float* __restrict__ sz, int nsrc) {
  correct_orbit_body(*dp, ds, pos, fhi, flo, flags, gidx, gold, gnew, orbit_part, nb, blockIdx.x,
                     gridDim.x - nb, sx, sy, sz, nsrc);
}

// directed ion–ion sums of a shard's ions (sources tgt_off .. tgt_off + Npad_local of the
// sources) over all nsrc_pad sources, plan variants 2-6 (one target or two per thread)
template <int NT, int NEWTON, int TPT>
__global__ void __launch_bounds__(NT) k_shard_pairs(const float* __restrict__ sx,
                                                    const float* __restrict__ sy,
                                                    const float* __restrict__ sz, int nsrc_pad,
                                                    int chunk, int Npad_local, int tgt_off,
                                                    float4* __restrict__ part_hi,
                                                    float4* __restrict__ part_lo, float rho0,
                                                    float newton_r2, uint32_t* __restrict__ err,
                                                    unsigned long long* __restrict__ acc) {
  const int j0 = blockIdx.y * chunk;
  pairs_x2_body<NT, NEWTON, TPT>(sx, sy, sz, blockIdx.x, j0, min(j0 + chunk, nsrc_pad),
                                 (size_t)blockIdx.y * Npad_local, part_hi, part_lo, rho0,
                                 newton_r2, err, tgt_off, acc, (size_t)Npad_local);
}

cudaError_t od_launch_shard_pairs(const od_pair_plan& pl, const float* sx, const float* sy,
                                  const float* sz, int nsrc_pad, int Npad_local, int tgt_off,
                                  float4* ph, float4* plo, float rho0, uint32_t* err,
                                  unsigned long long* acc, bool take, cudaStream_t s) {
  const int tpt = (pl.variant == 5 || pl.variant == 6) ? 1 : 2;
  if (pl.variant < 2 || pl.variant > 6 || (pl.nt != 128 && pl.nt != 256) || pl.ipt != tpt ||
      Npad_local % (tpt * pl.nt) || pl.chunk % OD_TJ || tgt_off % OD_PAD)
    return cudaErrorInvalidValue;
  const dim3 grid(Npad_local / (tpt * pl.nt), pl.jsplit);
  const float nr = 64.0f * rho0, nr2 = nr * nr;  // as launch_pairs_x2
#define OD_SHARD_PAIRS(NT, NW, TP)                                                              \
  k_shard_pairs<NT, NW, TP><<<grid, NT, 0, s>>>(sx, sy, sz, nsrc_pad, pl.chunk, Npad_local,    \
                                                tgt_off, ph, plo, rho0, nr2, err, acc)
  switch (pl.nt * 100 + pl.variant) {
    case 12802: OD_SHARD_PAIRS(128, 0, 2); break;
    case 25602: OD_SHARD_PAIRS(256, 0, 2); break;
    case 12803: OD_SHARD_PAIRS(128, 1, 2); break;
    case 25603: OD_SHARD_PAIRS(256, 1, 2); break;
    case 12804: OD_SHARD_PAIRS(128, 2, 2); break;
    case 25604: OD_SHARD_PAIRS(256, 2, 2); break;
    case 12805: OD_SHARD_PAIRS(128, 0, 1); break;
    case 25605: OD_SHARD_PAIRS(256, 0, 1); break;
    case 12806: OD_SHARD_PAIRS(128, 2, 1); break;
    case 25606: OD_SHARD_PAIRS(256, 2, 1); break;
    default: return cudaErrorInvalidValue;
  }
#undef OD_SHARD_PAIRS
  if (take) k_acc_take<<<(Npad_local + 255) / 256, 256, 0, s>>>(acc, Npad_local, ph, plo);
  return cudaGetLastError();
}

cudaError_t od_launch_shard_list(const od_dparams* dp, od_dstate* ds, int K, const int32_t* gidx,
                                 const int32_t* gbits, const float4* gnew, const float4* gv,
                                 float* sx, float* sy, float* sz, cudaStream_t s) {
  k_shard_list<<<1, kCT, 0, s>>>(dp, ds, K, gidx, gbits, gnew, gv, sx, sy, sz);
  return cudaGetLastError();
}

cudaError_t od_launch_shard_correct(const od_dparams* dp, const od_dstate* ds, const od_dbufs& b,
                                    int Npad_local, int nrec, const int32_t* gidx,
                                    const float4* gold, const float4* gnew, const float* sx,
                                    const float* sy, const float* sz, int nsrc, cudaStream_t s) {
  const int nb = Npad_local / kBlk;
  k_shard_correct_orbit<<<nb + nrec, kBlk, 0, s>>>(dp, ds, b.pos, b.fhi, b.flo, b.flags, gidx,
                                                   gold, gnew, b.orbit_part, nb, sx, sy, sz, nsrc);
  return cudaGetLastError();
}

cudaError_t od_launch_shard_tail(const od_dparams* dp, od_dstate* ds, const od_dbufs& b,
                                 const double* orbit_all, int nb_all, cudaStream_t s) {
  k_tail<<<1, kBlk, 0, s>>>(dp, ds, orbit_all, nb_all, b.s_q, b.s_orbit, b.s_collect, b.s_dust,
                           b.s_field, b.cq);
  return cudaGetLastError();
}

// K1 of a shard (its positions also go to sources ion0 .. ion0 + N), or K3 + K4
cudaError_t od_launch_shard_part(int part, const od_dparams* dp, od_dstate* ds, const od_dbufs& b,
                                 int N, int Npad, int jsplit, float* sx, float* sy, float* sz,
                                 cudaStream_t s) {
  if (part == 0) {
    k_kick_drift<<<(N + kBlk - 1) / kBlk, kBlk, 0, s>>>(dp, ds, b.rel, b.pos, b.vel, b.fhi, b.flo, b.cq,
                                                        sx, sy, sz);
    return cudaGetLastError();
  }
  k_kick_flag<<<Npad / kBlk, kBlk, 0, s>>>(dp, ds, b.pos, b.vel, b.part_hi, b.part_lo, jsplit,
                                          b.fhi, b.flo, b.flags, b.cq, b.n3);
  k_collect_inject<<<1, kCT, 0, s>>>(dp, ds, b.rel, b.pos, b.vel, b.flags, b.list, b.list_bits,
                                     b.list_old, b.list_new, b.list_v);
  return cudaGetLastError();
}

// Bounded-wait self test. One thread arms an mbarrier that expects one arrival; with arrive = 0
// nothing ever arrives, so od_mbar_wait_n gives up after `limit` polls and the kernel records
// OD_DERR_TIMEOUT in *err and returns, the same path every production wait takes when its
// limit runs out. No copy is in flight, so nothing else has to drain before the return.
__global__ void k_wait_selftest(uint32_t* err, uint32_t limit, int arrive) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    od_mbar_init(&bar, 1);
    od_fence_barrier_init();
    if (arrive) od_mbar_arrive(&bar);
    if (!od_mbar_wait_n(&bar, 0, limit)) atomicOr(err, OD_DERR_TIMEOUT);
    od_mbar_inval(&bar);
  }
}

cudaError_t od_launch_wait_selftest(uint32_t* err, uint32_t limit, int arrive, cudaStream_t s) {
  k_wait_selftest<<<1, 32, 0, s>>>(err, limit, arrive);
  return cudaGetLastError();
}
