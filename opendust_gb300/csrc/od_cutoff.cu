// od_cutoff.cu — cutoff ion–ion force over a device-built cell list (sm_103a).
//
// The reference's cutOff=True path (opendust.py:481-485) is an OpenMM CutoffNonPeriodic
// CustomNonbondedForce with cutoff 3.2 lambda and OpenMM's switching polynomial from
// 3.0 lambda. Here, every force evaluation
//   1. bins the ions into a uniform grid of cells of side c = cutoff / k (atomic counts),
//   2. takes an exclusive scan of the cell counts padded to multiples of 8 (32-byte aligned
//      segments), and of the number of 128-target chunks per cell,
//   3. scatters ion indices into their cell segments, sorts each segment by ion index (so the
//      summation order, and therefore the result, does not depend on atomic timing) and
//      stores each source as a cell-relative FP32 offset (SoA); padding slots hold far-away
//      sentinels,
//   4. runs one block per (cell, 128-target chunk): the block walks the pruned stencil of
//      source cells whose nearest point lies within the cutoff, stages each source tile in
//      shared memory, shifts its targets into the source cell's frame once per cell and
//      accumulates masked pair terms (two-float per tile, as the all-pairs kernel).
// The sums are written in ion order into slab 0 of the partial-sum buffer, so the rest of
// the step (kick, flags, re-injection, correction) is shared with the all-pairs path.
#include <cuda_runtime.h>
#include <stdint.h>
#include "od_internal.h"

namespace {

constexpr int kBlk = 256;
constexpr int kTgt = 128;        // targets per block (one per thread)
constexpr int kSortMax = 4096;   // largest cell a block sorts in shared memory

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

__device__ __forceinline__ int cell_of_pos(const od_cellgeom& g, float x, float y, float z, int& cx,
                                           int& cy, int& cz) {
  cx = clampi((int)floorf((x - g.lox) * g.inv_c), 0, g.gx - 1);
  cy = clampi((int)floorf((y - g.loy) * g.inv_c), 0, g.gy - 1);
  cz = clampi((int)floorf((z - g.loz) * g.inv_c), 0, g.gz - 1);
  return (cz * g.gy + cy) * g.gx + cx;
}

__global__ void k_cells_clear(int ncells, int32_t* __restrict__ count, int32_t* __restrict__ fill) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncells) { count[c] = 0; fill[c] = 0; }
}

__global__ void k_cells_count(od_cellgeom g, int n, const float4* __restrict__ pos,
                              int32_t* __restrict__ cell_of, int32_t* __restrict__ count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = pos[i];
  int cx, cy, cz;
  const int c = cell_of_pos(g, p.x, p.y, p.z, cx, cy, cz);
  cell_of[i] = c;
  atomicAdd(&count[c], 1);
}

// Exclusive scans (one 1024-thread block): start[] of 8-padded segments, chunk_prefix[] of
// target chunks; start[ncells] = total slots, chunk_prefix[ncells] = total chunks. Also
// records the largest cell in err_word bit 4 if it exceeds kSortMax.
__global__ void __launch_bounds__(1024) k_cells_scan(int ncells, const int32_t* __restrict__ count,
                                                     int32_t* __restrict__ start,
                                                     int32_t* __restrict__ chunk_prefix,
                                                     uint32_t* __restrict__ err) {
  __shared__ int s_a[32], s_b[32];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int per = (ncells + 1023) / 1024;
  const int c0 = min(tid * per, ncells), c1 = min(c0 + per, ncells);
  int a = 0, b = 0;
  bool big = false;
  for (int c = c0; c < c1; c++) {
    const int n = count[c];
    a += (n + 7) & ~7;
    b += (n + kTgt - 1) / kTgt;
    big |= n > kSortMax;
  }
  if (big) atomicOr(err, OD_DERR_CELL);
  int ia = a, ib = b;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int ya = __shfl_up_sync(0xffffffffu, ia, o), yb = __shfl_up_sync(0xffffffffu, ib, o);
    if (lane >= o) { ia += ya; ib += yb; }
  }
  if (lane == 31) { s_a[wid] = ia; s_b[wid] = ib; }
  __syncthreads();
  if (wid == 0) {
    int va = s_a[lane], vb = s_b[lane], xa = va, xb = vb;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int ya = __shfl_up_sync(0xffffffffu, xa, o), yb = __shfl_up_sync(0xffffffffu, xb, o);
      if (lane >= o) { xa += ya; xb += yb; }
    }
    s_a[lane] = xa - va;
    s_b[lane] = xb - vb;
  }
  __syncthreads();
  int oa = s_a[wid] + ia - a, ob = s_b[wid] + ib - b;
  for (int c = c0; c < c1; c++) {
    const int n = count[c];
    start[c] = oa;
    chunk_prefix[c] = ob;
    oa += (n + 7) & ~7;
    ob += (n + kTgt - 1) / kTgt;
  }
  if (tid == 1023) { start[ncells] = oa; chunk_prefix[ncells] = ob; }
}

__global__ void k_cells_scatter(int n, const int32_t* __restrict__ cell_of,
                                const int32_t* __restrict__ start, int32_t* __restrict__ fill,
                                int32_t* __restrict__ perm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = cell_of[i];
  perm[start[c] + atomicAdd(&fill[c], 1)] = i;
}

// One block per cell: sort the segment by ion index (bitonic, shared memory), then write the
// cell-relative offsets of its ions and sentinels in the padding slots.
__global__ void __launch_bounds__(kBlk) k_cells_sort(od_cellgeom g, const float4* __restrict__ pos,
                                                     const int32_t* __restrict__ count,
                                                     const int32_t* __restrict__ start,
                                                     int32_t* __restrict__ perm,
                                                     float* __restrict__ ox, float* __restrict__ oy,
                                                     float* __restrict__ oz) {
  __shared__ int32_t s_key[kSortMax];
  const int c = blockIdx.x;
  const int n = min(count[c], kSortMax);
  const int s0 = start[c], s1 = start[c + 1];
  int m = 1;
  while (m < n) m <<= 1;
  for (int k = threadIdx.x; k < m; k += kBlk) s_key[k] = k < n ? perm[s0 + k] : 0x7fffffff;
  __syncthreads();
  for (int size = 2; size <= m; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int k = threadIdx.x; k < m; k += kBlk) {
        const int l = k ^ stride;
        if (l > k) {
          const bool up = (k & size) == 0;
          const int a = s_key[k], b = s_key[l];
          if ((a > b) == up) { s_key[k] = b; s_key[l] = a; }
        }
      }
      __syncthreads();
    }
  const int cx = c % g.gx, cy = (c / g.gx) % g.gy, cz = c / (g.gx * g.gy);
  const float bx = g.lox + cx * g.c, by = g.loy + cy * g.c, bz = g.loz + cz * g.c;
  for (int k = threadIdx.x; k < s1 - s0; k += kBlk) {
    if (k < n) {
      const int i = s_key[k];
      const float4 p = pos[i];
      perm[s0 + k] = i;
      ox[s0 + k] = p.x - bx; oy[s0 + k] = p.y - by; oz[s0 + k] = p.z - bz;
    } else {
      ox[s0 + k] = OD_SENTINEL; oy[s0 + k] = OD_SENTINEL; oz[s0 + k] = OD_SENTINEL;
    }
  }
}

// pair factor with a hard cutoff and (SWITCH) OpenMM's switching polynomial on the energy
template <bool SWITCH>
__device__ __forceinline__ float pair_c_cut(float r2, float rho0, float rc2, float rs, float inv_w) {
  const float ri = od_rsqrt(r2);
  const float r = r2 * ri;
  const float si = od_rcp(r + rho0);
  const float ex = od_ex2(r * OD_NLOG2E);
  float f = ex * fmaf(si, si, si);
  if (SWITCH) {
    const float x = fmaxf((r - rs) * inv_w, 0.0f);
    // 1 - 10x^3 + 15x^4 - 6x^5 in the factored form (1-x)^3 (1 + 3x + 6x^2)
    const float om = 1.0f - x;
    const float S = om * om * om * fmaf(x, fmaf(6.0f, x, 3.0f), 1.0f);
    const float q = x * om;
    const float dS = -30.0f * q * q * inv_w;
    f = fmaf(-ex * si, dS, f * S);
  }
  const float c = f * ri;
  return r2 < rc2 ? c : 0.0f;
}

template <bool SWITCH>
__global__ void __launch_bounds__(kTgt) k_pairs_cut(od_cellgeom g, const int32_t* __restrict__ count,
                                                    const int32_t* __restrict__ start,
                                                    const int32_t* __restrict__ chunk_prefix,
                                                    const int32_t* __restrict__ perm,
                                                    const float* __restrict__ ox,
                                                    const float* __restrict__ oy,
                                                    const float* __restrict__ oz,
                                                    const int4* __restrict__ stencil, int nstencil,
                                                    int Npad, float4* __restrict__ part_hi,
                                                    float4* __restrict__ part_lo, float rho0,
                                                    float rc2, float rs, float inv_w,
                                                    unsigned long long* __restrict__ pair_count) {
  __shared__ __align__(16) float tx[OD_TJ], ty[OD_TJ], tz[OD_TJ];
  const int b = blockIdx.x;
  const int total = chunk_prefix[g.ncells];
  if (b >= total) return;
  // cell of this block: largest c with chunk_prefix[c] <= b
  int lo = 0, hi = g.ncells - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (chunk_prefix[mid] <= b) lo = mid; else hi = mid - 1;
  }
  const int cell = lo;
  const int chunk = b - chunk_prefix[cell];
  const int n_cell = count[cell];
  const int t = chunk * kTgt + threadIdx.x;
  const bool live = t < n_cell;
  const int slot = start[cell] + (live ? t : 0);
  const float txo = ox[slot], tyo = oy[slot], tzo = oz[slot];
  const int cx = cell % g.gx, cy = (cell / g.gx) % g.gy, cz = cell / (g.gx * g.gy);
  float hx = 0.f, hy = 0.f, hz = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
  unsigned int inside = 0;
  for (int st = 0; st < nstencil; st++) {
    const int4 d = stencil[st];
    const int sx = cx + d.x, sy = cy + d.y, sz = cz + d.z;
    if (sx < 0 || sy < 0 || sz < 0 || sx >= g.gx || sy >= g.gy || sz >= g.gz) continue;
    const int sc = (sz * g.gy + sy) * g.gx + sx;
    const int s0 = start[sc], s1 = start[sc + 1];
    if (s1 == s0) continue;
    // target in the source cell's frame (integer multiples of the cell side)
    const float px = fmaf((float)(-d.x), g.c, txo), py = fmaf((float)(-d.y), g.c, tyo),
                pz = fmaf((float)(-d.z), g.c, tzo);
    for (int j0 = s0; j0 < s1; j0 += OD_TJ) {
      const int nt = min(OD_TJ, s1 - j0);
      __syncthreads();
      for (int k = threadIdx.x; k < nt; k += kTgt) {
        tx[k] = ox[j0 + k]; ty[k] = oy[j0 + k]; tz[k] = oz[j0 + k];
      }
      __syncthreads();
      float ax = 0.f, ay = 0.f, az = 0.f;
#pragma unroll 4
      for (int k = 0; k < nt; k++) {
        const float dx = px - tx[k], dy = py - ty[k], dz = pz - tz[k];
        const float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, 1e-30f)));
        const float c = pair_c_cut<SWITCH>(r2, rho0, rc2, rs, inv_w);
        inside += r2 < rc2;
        ax = fmaf(c, dx, ax); ay = fmaf(c, dy, ay); az = fmaf(c, dz, az);
      }
      od_acc2(hx, lx, ax); od_acc2(hy, ly, ay); od_acc2(hz, lz, az);
    }
  }
  if (live) {
    const int i = perm[slot];
    part_hi[i] = make_float4(hx, hy, hz, 0.f);
    part_lo[i] = make_float4(lx, ly, lz, 0.f);
  }
  if (pair_count) {
    // pairs inside the cutoff, self pair excluded
    unsigned int v = live ? inside - 1u : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(pair_count, (unsigned long long)v);
  }
}

// ------------------------------------------------------------------ packed variant
// Two targets per thread, two sources per packed f32x2 operation (as the all-pairs kernel).
// With switching, (1 - x) is clamped at 0, which makes S and S' vanish beyond r_c, so pairs
// outside the cutoff contribute exactly 0 without a separate mask.
constexpr int kTgt2 = 256;  // targets per block (128 threads x 2)

struct cut_pk {
  od_u64 eps, rho, nl2e, one, three, six, invw, nrsw, m30w;
  float rc2;
};

template <bool SWITCH, bool COUNT>
__device__ __forceinline__ void pair2_cut(const cut_pk& k, od_u64 X, od_u64 Y, od_u64 Z, od_u64 QX,
                                          od_u64 QY, od_u64 QZ, od_u64& AX, od_u64& AY, od_u64& AZ,
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
  od_u64 F = mul2(EX, fma2(SI, SI, SI));
  od_u64 C;
  if (SWITCH) {
    const float2 xx = up2(fma2(R, k.invw, k.nrsw));
    const od_u64 X2 = p2(fmaxf(xx.x, 0.f), fmaxf(xx.y, 0.f));
    const float2 om = up2(sub2(k.one, X2));
    const od_u64 OM = p2(fmaxf(om.x, 0.f), fmaxf(om.y, 0.f));
    const od_u64 S = mul2(mul2(OM, OM), mul2(OM, fma2(X2, fma2(k.six, X2, k.three), k.one)));
    const od_u64 Q = mul2(X2, OM);
    const od_u64 DS = mul2(mul2(Q, Q), k.m30w);
    F = sub2(mul2(F, S), mul2(mul2(EX, SI), DS));
    C = mul2(F, RI);
  } else {
    const float2 c = up2(mul2(F, RI));
    C = p2(r2.x < k.rc2 ? c.x : 0.f, r2.y < k.rc2 ? c.y : 0.f);
  }
  if (COUNT) cnt += (r2.x < k.rc2) + (r2.y < k.rc2);
  AX = fma2(C, DX, AX); AY = fma2(C, DY, AY); AZ = fma2(C, DZ, AZ);
}

template <bool SWITCH, bool COUNT>
__global__ void __launch_bounds__(128) k_pairs_cut_x2(od_cellgeom g, const int32_t* __restrict__ count,
                                                      const int32_t* __restrict__ start,
                                                      const int32_t* __restrict__ chunk_prefix,
                                                      const int32_t* __restrict__ perm,
                                                      const float* __restrict__ ox,
                                                      const float* __restrict__ oy,
                                                      const float* __restrict__ oz,
                                                      const int4* __restrict__ stencil, int nstencil,
                                                      float4* __restrict__ part_hi,
                                                      float4* __restrict__ part_lo, float rho0,
                                                      float rc2, float rs, float inv_w,
                                                      unsigned long long* __restrict__ pair_count) {
  __shared__ __align__(16) float tx[OD_TJ], ty[OD_TJ], tz[OD_TJ];
  const int b = blockIdx.x;
  const int total = chunk_prefix[g.ncells];
  if (b >= total) return;
  int lo = 0, hi = g.ncells - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (chunk_prefix[mid] <= b) lo = mid; else hi = mid - 1;
  }
  const int cell = lo;
  const int chunk = b - chunk_prefix[cell];
  const int n_cell = count[cell];
  const int t0 = chunk * kTgt2 + threadIdx.x, t1 = t0 + kTgt2 / 2;
  const bool live0 = t0 < n_cell, live1 = t1 < n_cell;
  const int slot0 = start[cell] + (live0 ? t0 : 0), slot1 = start[cell] + (live1 ? t1 : 0);
  const float ax0 = ox[slot0], ay0 = oy[slot0], az0 = oz[slot0];
  const float ax1 = ox[slot1], ay1 = oy[slot1], az1 = oz[slot1];
  const int cx = cell % g.gx, cy = (cell / g.gx) % g.gy, cz = cell / (g.gx * g.gy);
  cut_pk k;
  k.eps = p2(1e-30f, 1e-30f); k.rho = p2(rho0, rho0); k.nl2e = p2(OD_NLOG2E, OD_NLOG2E);
  k.one = p2(1.f, 1.f); k.three = p2(3.f, 3.f); k.six = p2(6.f, 6.f);
  k.invw = p2(inv_w, inv_w); k.nrsw = p2(-rs * inv_w, -rs * inv_w);
  k.m30w = p2(-30.f * inv_w, -30.f * inv_w); k.rc2 = rc2;
  float h0x = 0.f, h0y = 0.f, h0z = 0.f, l0x = 0.f, l0y = 0.f, l0z = 0.f;
  float h1x = 0.f, h1y = 0.f, h1z = 0.f, l1x = 0.f, l1y = 0.f, l1z = 0.f;
  unsigned int c0 = 0, c1 = 0;
  for (int st = 0; st < nstencil; st++) {
    const int4 d = stencil[st];
    const int sx = cx + d.x, sy = cy + d.y, sz = cz + d.z;
    if (sx < 0 || sy < 0 || sz < 0 || sx >= g.gx || sy >= g.gy || sz >= g.gz) continue;
    const int sc = (sz * g.gy + sy) * g.gx + sx;
    const int s0 = start[sc], s1 = start[sc + 1];
    if (s1 == s0) continue;
    const float fx = (float)(-d.x) * g.c, fy = (float)(-d.y) * g.c, fz = (float)(-d.z) * g.c;
    const float px0 = ax0 + fx, py0 = ay0 + fy, pz0 = az0 + fz;
    const float px1 = ax1 + fx, py1 = ay1 + fy, pz1 = az1 + fz;
    const od_u64 X0 = p2(px0, px0), Y0 = p2(py0, py0), Z0 = p2(pz0, pz0);
    const od_u64 X1 = p2(px1, px1), Y1 = p2(py1, py1), Z1 = p2(pz1, pz1);
    for (int j0 = s0; j0 < s1; j0 += OD_TJ) {
      const int nt = min(OD_TJ, s1 - j0);  // a multiple of 8 (segments are 8-padded)
      __syncthreads();
      for (int q = threadIdx.x; q < nt; q += kTgt2 / 2) {
        tx[q] = ox[j0 + q]; ty[q] = oy[j0 + q]; tz[q] = oz[j0 + q];
      }
      __syncthreads();
      od_u64 A0x = 0, A0y = 0, A0z = 0, A1x = 0, A1y = 0, A1z = 0;
#pragma unroll 2
      for (int j = 0; j < nt; j += 4) {
        const ulonglong2 qx = *reinterpret_cast<const ulonglong2*>(&tx[j]);
        const ulonglong2 qy = *reinterpret_cast<const ulonglong2*>(&ty[j]);
        const ulonglong2 qz = *reinterpret_cast<const ulonglong2*>(&tz[j]);
        pair2_cut<SWITCH, COUNT>(k, X0, Y0, Z0, qx.x, qy.x, qz.x, A0x, A0y, A0z, c0);
        pair2_cut<SWITCH, COUNT>(k, X0, Y0, Z0, qx.y, qy.y, qz.y, A0x, A0y, A0z, c0);
        pair2_cut<SWITCH, COUNT>(k, X1, Y1, Z1, qx.x, qy.x, qz.x, A1x, A1y, A1z, c1);
        pair2_cut<SWITCH, COUNT>(k, X1, Y1, Z1, qx.y, qy.y, qz.y, A1x, A1y, A1z, c1);
      }
      od_acc2(h0x, l0x, sum2(A0x)); od_acc2(h0y, l0y, sum2(A0y)); od_acc2(h0z, l0z, sum2(A0z));
      od_acc2(h1x, l1x, sum2(A1x)); od_acc2(h1y, l1y, sum2(A1y)); od_acc2(h1z, l1z, sum2(A1z));
    }
  }
  if (live0) {
    const int i = perm[slot0];
    part_hi[i] = make_float4(h0x, h0y, h0z, 0.f);
    part_lo[i] = make_float4(l0x, l0y, l0z, 0.f);
  }
  if (live1) {
    const int i = perm[slot1];
    part_hi[i] = make_float4(h1x, h1y, h1z, 0.f);
    part_lo[i] = make_float4(l1x, l1y, l1z, 0.f);
  }
  if (COUNT) {
    unsigned int v = (live0 ? c0 - 1u : 0u) + (live1 ? c1 - 1u : 0u);  // self pairs excluded
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(pair_count, (unsigned long long)v);
  }
}

__global__ void k_chunks2(int ncells, const int32_t* __restrict__ count,
                          int32_t* __restrict__ chunk_prefix2) {
  // exclusive prefix of ceil(count / kTgt2), one 1024-thread block
  __shared__ int s_w[32];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int per = (ncells + 1023) / 1024;
  const int c0 = min(tid * per, ncells), c1 = min(c0 + per, ncells);
  int a = 0;
  for (int c = c0; c < c1; c++) a += (count[c] + kTgt2 - 1) / kTgt2;
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
    chunk_prefix2[c] = off;
    off += (count[c] + kTgt2 - 1) / kTgt2;
  }
  if (tid == 1023) chunk_prefix2[ncells] = off;
}

}  // namespace

cudaError_t od_launch_cutoff(const od_cutlist& L, const float4* pos, int n, int Npad,
                             float4* part_hi, float4* part_lo, float rho0, float rc, float rs,
                             uint32_t* err, unsigned long long* pair_count, cudaStream_t s) {
  if (L.n3)
    return od_launch_cutoff_n3(*L.n3, pos, n, part_hi, part_lo, rho0, rc, rs, err, pair_count, s);
  const od_cellgeom& g = L.g;
  k_cells_clear<<<(g.ncells + kBlk - 1) / kBlk, kBlk, 0, s>>>(g.ncells, L.count, L.fill);
  k_cells_count<<<(n + kBlk - 1) / kBlk, kBlk, 0, s>>>(g, n, pos, L.cell_of, L.count);
  k_cells_scan<<<1, 1024, 0, s>>>(g.ncells, L.count, L.start, L.chunk_prefix, err);
  k_cells_scatter<<<(n + kBlk - 1) / kBlk, kBlk, 0, s>>>(n, L.cell_of, L.start, L.fill, L.perm);
  k_cells_sort<<<g.ncells, kBlk, 0, s>>>(g, pos, L.count, L.start, L.perm, L.ox, L.oy, L.oz);
  const bool sw = rs < rc;
  const float inv_w = sw ? 1.0f / (rc - rs) : 0.0f;
  if (L.packed) {
    k_chunks2<<<1, 1024, 0, s>>>(g.ncells, L.count, L.chunk_prefix2);
    const int blocks2 = (n + kTgt2 - 1) / kTgt2 + g.ncells;
#define OD_CUT2(SW, CNT)                                                                        \
  k_pairs_cut_x2<SW, CNT><<<blocks2, kTgt2 / 2, 0, s>>>(g, L.count, L.start, L.chunk_prefix2,   \
                                                         L.perm, L.ox, L.oy, L.oz, L.stencil,   \
                                                         L.nstencil, part_hi, part_lo, rho0,    \
                                                         rc * rc, rs, inv_w, pair_count)
    if (sw) { if (pair_count) OD_CUT2(true, true); else OD_CUT2(true, false); }
    else { if (pair_count) OD_CUT2(false, true); else OD_CUT2(false, false); }
#undef OD_CUT2
    return cudaGetLastError();
  }
  const int blocks = (n + kTgt - 1) / kTgt + g.ncells;
  if (sw)
    k_pairs_cut<true><<<blocks, kTgt, 0, s>>>(g, L.count, L.start, L.chunk_prefix, L.perm, L.ox, L.oy,
                                              L.oz, L.stencil, L.nstencil, Npad, part_hi, part_lo,
                                              rho0, rc * rc, rs, inv_w, pair_count);
  else
    k_pairs_cut<false><<<blocks, kTgt, 0, s>>>(g, L.count, L.start, L.chunk_prefix, L.perm, L.ox,
                                               L.oy, L.oz, L.stencil, L.nstencil, Npad, part_hi,
                                               part_lo, rho0, rc * rc, rs, inv_w, pair_count);
  return cudaGetLastError();
}
