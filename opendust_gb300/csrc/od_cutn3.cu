// od_cutn3.cu — ion–ion forces within a cutoff over tile pairs (cutoff variant 3): ions sorted
// along a Hilbert curve of a cell grid, 512- or 1024-ion tiles of consecutive sorted ions, the tile
// pairs whose bounding boxes come within the cutoff listed, each unordered pair inside the cutoff
// evaluated once (od_n3_pair.cuh) with 64-ion group pairs beyond it skipped, and the sums added
// as 64-bit fixed point with integer atomics (per-ion words in shared memory, then per-slot
// accumulators). Every result bit is independent of scheduling.
#include "od_hilbert.h"
#include "od_n3_pair.cuh"

namespace {

// ------------------------------------------------------------------ cutoff over tile pairs
// Cell grid of G^3 cells over the cube [lo, lo + G/inv_s)^3; a cell's key is its index along
// a Hilbert curve (od_hilbert.h), so that the ions sorted by key fill tiles and 64-ion groups
// with compact bounding boxes: at 2^19 ions in the 3 x 6 lambda cylinder the group boxes keep
// 1.73x the pairs inside a 2 lambda cutoff, against 1.94x in Morton order.
__global__ void k_mc_clear(int ncells, int32_t* __restrict__ count, int32_t* __restrict__ fill) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncells) { count[c] = 0; fill[c] = 0; }
}

// Cubes of G^3 cells stacked nb deep along z (nb = 1 for a compact domain); a cell's key is its
// cube's index times G^3 plus its index along the cube's Hilbert curve.
__global__ void k_mc_count(int n, const float4* __restrict__ pos, float lo, float lo_z,
                           float inv_s, int G, int nb, int32_t* __restrict__ cell_of,
                           int32_t* __restrict__ count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = pos[i];
  const int bits = 31 - __clz(G);
  const int cx = min(max((int)floorf((p.x - lo) * inv_s), 0), G - 1);
  const int cy = min(max((int)floorf((p.y - lo) * inv_s), 0), G - 1);
  const int cz = min(max((int)floorf((p.z - lo_z) * inv_s), 0), nb * G - 1);
  const int c = ((cz >> bits) << (3 * bits)) +
                (int)od_hilbert3((uint32_t)cx, (uint32_t)cy, (uint32_t)(cz & (G - 1)), bits);
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
// separates them. Every listed group pair adds its FP32 target and reaction sums, converted to
// 64-bit fixed point (od_fix), into per-ion words in shared memory with integer atomics, so
// the block's sums do not depend on which warp ran what, or when; the block then adds each
// ion's words to its global accumulators. A group pair whose farthest box distance is below the
// switching radius (hard cutoff: the cutoff) is marked inner and takes the plain screened term:
// the switching factor is exactly 1 for all its pairs.
template <int MT, int MS>
struct cut_traits {
  static constexpr int GT = 32 * MT, GS = 32 * MS;    // target and source group sizes
  static constexpr int T = 512;                       // ions per tile
  static constexpr int NBT = T / GT, NBS = T / GS;    // groups per tile
  static constexpr int NI = NBT * NBS;                // group pairs per tile pair (<= 64)
  // [3][T] fixed-point words of tile a's ions and [3][T] of tile b's, then the list
  static constexpr size_t SMEM = sizeof(unsigned long long) * 6 * T + 256;
};

// group pair (ga, gb) of a diagonal tile: 2 each pair once, 1 directed (the sources lie in the
// target group), 0 skipped (counted from the other side)
template <int GT, int GS>
__device__ __forceinline__ int cut_diag_mode(int ga, int gb) {
  const int t0 = ga * GT, s0 = gb * GS;
  return s0 >= t0 + GT ? 2 : (s0 >= t0 ? 1 : 0);
}

constexpr int kItem = 63, kInner = 128;  // list entry: group pair index | inner flag

template <int MT, int MS, int CUT, bool COUNT>
__device__ __forceinline__ unsigned int cut_tile_pair(const float* __restrict__ sx,
                                                         const float* __restrict__ sy,
                                                         const float* __restrict__ sz,
                                                         unsigned long long* __restrict__ acc,
                                                         size_t stride, const n3_consts& k, int a,
                                                         int b, float* sm,
                                                         const float* __restrict__ gbox,
                                                         float cull2, float k_in2) {
  using CT = cut_traits<MT, MS>;
  constexpr int GT = CT::GT, GS = CT::GS, T = CT::T, NBT = CT::NBT, NBS = CT::NBS, NI = CT::NI;
  constexpr int MS2 = MS / 2;
  static_assert(NI % 32 == 0 && NI <= 64, "list of at most 64 group pairs");
  // [3][T] fixed-point sums of tile a's ions, then [3][T] of tile b's (unused when a == b)
  unsigned long long* const fa = reinterpret_cast<unsigned long long*>(sm);
  unsigned long long* const fb = fa + 3 * T;
  unsigned char* const items = reinterpret_cast<unsigned char*>(fb + 3 * T);  // ga·NBS + gb
  int* const s_n = reinterpret_cast<int*>(items + 64);
  const bool diag = a == b;
  unsigned long long* const fs = diag ? fa : fb;  // where the reactions go
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31, src = (lane + 1) & 31;

  // 1. the list (warp 0): group pairs within range; on a diagonal tile the source groups
  // inside a target group (directed) and those above it
  if (w == 0) {
    int n = 0;
    for (int r = 0; r < NI / 32; r++) {
      const int c = r * 32 + lane, ga = c / NBS, gb = c % NBS;
      const int mode = diag ? cut_diag_mode<GT, GS>(ga, gb) : 2;
      bool keep = mode == 1, inner = false;
      if (mode != 0) {
        float ta[6], tb[6];
        group_box(gbox, (a * NBT + ga) * (GT / 64), GT / 64, ta);
        group_box(gbox, (b * NBS + gb) * (GS / 64), GS / 64, tb);
        float d2 = 0.f, f2 = 0.f;
#pragma unroll
        for (int d = 0; d < 3; d++) {
          const float gap = fmaxf(fmaxf(tb[d] - ta[3 + d], ta[d] - tb[3 + d]), 0.f);
          const float far = fmaxf(tb[3 + d] - ta[d], ta[3 + d] - tb[d]);
          d2 = fmaf(gap, gap, d2);
          f2 = fmaf(far, far, f2);
        }
        if (mode == 2) keep = d2 < cull2;
        inner = f2 < k_in2;
      }
      const unsigned int bal = __ballot_sync(0xffffffffu, keep);
      const int pos = n + __popc(bal & ((1u << lane) - 1u));
      if (keep) items[pos] = (unsigned char)(c | (inner ? kInner : 0));
      n += __popc(bal);
    }
    if (lane == 0) *s_n = n;
  }
  __syncthreads();

  // 2. this warp's slice of the list; sums into the shared fixed-point words
  const int n = *s_n, i0 = (w * n) >> 3, i1 = ((w + 1) * n) >> 3;
  unsigned int cnt = 0;
  od_u64 X[MT], Y[MT], Z[MT];
  int cur = -1;
  for (int i = i0; i < i1; i++) {
    const int c = items[i] & kItem, ga = c / NBS, gb = c % NBS;
    const bool inner = (items[i] & kInner) != 0;
    if (ga != cur) {
#pragma unroll
      for (int kt = 0; kt < MT; kt++) {
        const int j = (a * NBT + ga) * GT + lane + 32 * kt;
        const float x = sx[j], y = sy[j], z = sz[j];
        X[kt] = p2(x, x); Y[kt] = p2(y, y); Z[kt] = p2(z, z);
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
    const bool react = !(diag && cut_diag_mode<GT, GS>(ga, gb) == 1);
    if (!react) {
      if (inner)
        n3_group<MT, MS, 0, false, COUNT>(k, X, Y, Z, QX, QY, QZ, AX, AY, AZ, RX, RY, RZ, src,
                                          cnt);
      else
        n3_group<MT, MS, CUT, false, COUNT>(k, X, Y, Z, QX, QY, QZ, AX, AY, AZ, RX, RY, RZ, src,
                                            cnt);
    } else {
      if (inner)
        n3_group<MT, MS, 0, true, COUNT>(k, X, Y, Z, QX, QY, QZ, AX, AY, AZ, RX, RY, RZ, src,
                                         cnt);
      else
        n3_group<MT, MS, CUT, true, COUNT>(k, X, Y, Z, QX, QY, QZ, AX, AY, AZ, RX, RY, RZ, src,
                                           cnt);
      // the force on the sources is minus the accumulated terms
#pragma unroll
      for (int q = 0; q < MS2; q++) {
        const int e = gb * GS + lane + 64 * q;
        const float2 rx = up2(RX[q]), ry = up2(RY[q]), rz = up2(RZ[q]);
        atomicAdd(fs + e, od_fix(-rx.x, 0.f));
        atomicAdd(fs + e + 32, od_fix(-rx.y, 0.f));
        atomicAdd(fs + T + e, od_fix(-ry.x, 0.f));
        atomicAdd(fs + T + e + 32, od_fix(-ry.y, 0.f));
        atomicAdd(fs + 2 * T + e, od_fix(-rz.x, 0.f));
        atomicAdd(fs + 2 * T + e + 32, od_fix(-rz.y, 0.f));
      }
    }
#pragma unroll
    for (int kt = 0; kt < MT; kt++) {
      const int e = ga * GT + lane + 32 * kt;
      atomicAdd(fa + e, od_fix(sum2(AX[kt]), 0.f));
      atomicAdd(fa + T + e, od_fix(sum2(AY[kt]), 0.f));
      atomicAdd(fa + 2 * T + e, od_fix(sum2(AZ[kt]), 0.f));
    }
  }
  __syncthreads();

  // 3. the block's words into the ions' global accumulators, and cleared for the next tile pair
  for (int e = tid; e < T; e += kWarps * 32) {
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const unsigned long long va = fa[c * T + e];
      if (va) atomicAdd(acc + c * stride + (size_t)a * T + e, va);
      fa[c * T + e] = 0ull;
      if (!diag) {
        const unsigned long long vb = fb[c * T + e];
        if (vb) atomicAdd(acc + c * stride + (size_t)b * T + e, vb);
        fb[c * T + e] = 0ull;
      }
    }
  }
  __syncthreads();  // the next tile pair rewrites the list and the words
  return cnt;
}

// ions per tile of the staggered tile pair, or of the balanced list (BAL)
template <bool BAL, int MT, int MS, int PA>
struct cutn3_tile {
  static constexpr int T = n3_traits<MT, MS, PA>::T;
};
template <int MT, int MS, int PA>
struct cutn3_tile<true, MT, MS, PA> {
  static constexpr int T = cut_traits<MT, MS>::T;
};

// every listed tile pair, each unordered ion pair once (static assignment: pair k to block
// k mod grid), group pairs beyond the cutoff skipped. BAL: the balanced list routine above
// (512-ion tiles); otherwise the staggered tile-pair routine.
// blocks per SM the registers of the balanced tile pair are budgeted for. Measured on GB300 at
// 2^19 ions (field_chain), ms per step: with switching 32.9 (4 blocks of at most 64 registers),
// 34.2 (3 blocks), 35.8 with per-item slots in shared memory summed in a fixed order (74 KB per
// block, 3 blocks); hard cutoff 30.6 (3 blocks), 31.6 (4 blocks: its exact-decision branch
// spills at 64 registers), 31.9 with the slots.
template <int CUT>
struct cut_blocks {
  static constexpr int value = CUT == 2 ? 3 : 4;
};

template <int MT, int MS, int PA, int CUT, bool COUNT, bool BAL>
__global__ void __launch_bounds__(kWarps * 32, (BAL ? cut_blocks<CUT>::value
                                                                : n3_traits<MT, MS, PA>::MIN_BLOCKS))
    k_pairs_cutn3(const float* __restrict__ xs, const float* __restrict__ ys,
                  const float* __restrict__ zs, int nslots, int nT,
                  const int2* __restrict__ pairs, const int32_t* __restrict__ npairs,
                  unsigned long long* __restrict__ acc, n3_cut cut,
                  const float* __restrict__ gbox, float cull2,
                  unsigned long long* __restrict__ pair_count) {
  extern __shared__ float sm[];
  static_assert(!BAL || PA == 1, "balanced list: one pass");
  const int np = *npairs;
  unsigned int cnt = 0;
  if constexpr (BAL) {
    const n3_consts kc = make_consts(cut);
    unsigned long long* const f = reinterpret_cast<unsigned long long*>(sm);
    for (int e = threadIdx.x; e < 6 * cut_traits<MT, MS>::T; e += kWarps * 32) f[e] = 0ull;
    __syncthreads();
    for (int k = blockIdx.x; k < np; k += gridDim.x) {
      const int2 ab = pairs[k];
      cnt += cut_tile_pair<MT, MS, CUT, COUNT>(xs, ys, zs, acc, (size_t)nslots, kc, ab.x,
                                                  ab.y, sm, gbox, cull2, cut.in2);
    }
  } else {
    for (int k = blockIdx.x; k < np; k += gridDim.x) {
      const int2 ab = pairs[k];
      cnt += n3_tile_pair<MT, MS, PA, CUT, COUNT, true>(xs, ys, zs, nslots, acc, (size_t)nslots,
                                                        cut, ab.x, ab.y, sm, gbox, cull2);
    }
  }
  if (COUNT) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(pair_count, (unsigned long long)cnt);
  }
}

// Slot accumulators -> the ions' entries of (ph, pl) as two-float sums (slot s holds ion
// perm[s], -1 for the sentinels in the tail), every slot cleared for the next evaluation.
__global__ void __launch_bounds__(256) k_slot_take(int nslots, unsigned long long* __restrict__ acc,
                                                  const int32_t* __restrict__ perm,
                                                  float4* __restrict__ ph, float4* __restrict__ pl) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nslots) return;
  float3 hi, lo;
  od_fix_take(acc + e, (size_t)nslots, hi, lo);
  const int i = perm[e];
  if (i < 0) return;
  ph[i] = make_float4(hi.x, hi.y, hi.z, 0.f);
  pl[i] = make_float4(lo.x, lo.y, lo.z, 0.f);
}

}  // namespace

od_cgrid od_cutn3_grid(int N, double R, double H) {
  od_cgrid g;
  // a domain at most 1.5 times as high as wide is one cube; a taller one a column of cubes as
  // wide as the domain, so that the cells keep their size whatever the aspect ratio
  g.nb = H <= 3.0 * R ? 1 : (int)std::ceil(H / (2.0 * R));
  g.side = (g.nb == 1 ? std::max(2.0 * R, H) : 2.0 * R) * 1.02;
  // about 16 ions per cell: G the smallest power of two with G^3 >= (N / nb) / 22, 8 <= G <= 128
  const double per = (double)N / g.nb;
  g.G = 8;
  while (g.G < 128 && (double)g.G * g.G * g.G * 8.0 * 16.0 < per * 1.4142) g.G <<= 1;
  g.ncells = g.nb * g.G * g.G * g.G;
  return g;
}

size_t od_cutn3_bytes(int N, int T, int ncells) {
  const size_t nT = (size_t)((N + T - 1) / T), ns = nT * T, nc = (size_t)ncells;
  const size_t nw = (nT + 31) / 32;
  return sizeof(unsigned long long) * 3 * ns                 // accumulators
         + sizeof(int2) * nT * (nT + 1) / 2                   // pairs
         + sizeof(uint32_t) * nT * nw                         // bitmap
         + sizeof(float) * (3 * ns + 6 * nT + 6 * (ns / 64))  // sorted positions, boxes
         + sizeof(int32_t) * (ns + N + 3 * nc + nT + 4);
}

// cutoff tile-pair shapes: (ipt, T) = (2, 512) the balanced list with 2 x 2 targets x sources
// per lane, (4, 1024) the staggered tile pair with 4 x 4. Measured on GB300 at 2^19 ions
// (field_chain), ms per step: 32.9 with (2, 512); the balanced list at 4 x 2 (128-ion target
// groups: more arithmetic per shuffle, but coarser culling) 33.2 with 3 blocks per SM and 34.3
// with 4 (it spills at 64 registers); the staggered (4, 1024) 55.7 in an earlier form.
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

// dynamic shared memory of the balanced tile pair
constexpr size_t kCutBalSmem = cut_traits<2, 2>::SMEM;

// resident blocks per SM of the production pair kernel (the persistent grid is this times the
// SM count)
int od_cutn3_blocks_per_sm(int ipt, int T, bool hard) {
  int nb = 0;
  cudaError_t e = cudaErrorInvalidValue;
  if (ipt == 2 && T == 512)
    e = hard ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                   &nb, k_pairs_cutn3<2, 2, 1, 2, false, true>, kWarps * 32, kCutBalSmem)
             : cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                   &nb, k_pairs_cutn3<2, 2, 1, 1, false, true>, kWarps * 32, kCutBalSmem);
  else if (ipt == 4 && T == 1024)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_pairs_cutn3<4, 4, 1, 1, false, false>,
                                                      kWarps * 32, n3_traits<4, 4, 1>::SMEM);
  if (e != cudaSuccess) cudaGetLastError();
  return e == cudaSuccess && nb > 0 ? nb : 3;
}

cudaError_t od_cutn3_prepare(int ipt, int T) {
  if (ipt == 2 && T == 512) return prepare_cutn3<2, 2, true>((int)kCutBalSmem);
  if (ipt == 4 && T == 1024)
    return prepare_cutn3<4, 4, false>((int)n3_traits<4, 4, 1>::SMEM);
  return cudaErrorInvalidValue;
}

cudaError_t od_launch_cutoff_n3(const od_cutn3& L, const float4* pos, int n, float4* part_hi,
                                float4* part_lo, float rho0, float rc, float rs, uint32_t* err,
                                unsigned long long* pair_count, cudaStream_t s) {
  k_mc_clear<<<(L.ncells + 255) / 256, 256, 0, s>>>(L.ncells, L.count, L.fill);
  k_mc_count<<<(n + 255) / 256, 256, 0, s>>>(n, pos, L.lo, L.lo_z, L.inv_s, L.G, L.nb,
                                              L.cell_of, L.count);
  k_scan_excl<<<1, 1024, 0, s>>>(L.ncells, L.count, L.start);
  k_mc_scatter<<<(n + 255) / 256, 256, 0, s>>>(n, L.cell_of, L.start, L.fill, L.perm);
  k_mc_sort<<<L.ncells, 128, 0, s>>>(L.count, L.start, pos, L.perm, L.xs, L.ys, L.zs, err);
  k_tile_box<<<L.nT, 256, 0, s>>>(n, L.T, L.xs, L.ys, L.zs, L.gbox, L.box);
  const float rc2m = rc * rc * 1.00001f;
  k_tile_adj<<<L.nT, 128, 0, s>>>(L.nT, L.nwords, L.box, rc2m, L.adj, L.rowptr);
  k_scan_excl<<<1, 1024, 0, s>>>(L.nT, L.rowptr, L.rowptr);
  k_tile_list<<<(L.nT + 127) / 128, 128, 0, s>>>(L.nT, L.nwords, L.adj, L.rowptr, L.pairs);
  const bool sw = rs < rc;
  // group pairs whose farthest box distance is below the switching radius (hard cutoff: the
  // cutoff), with a relative margin of 1e-5 against rounding, skip the switching polynomial
  const float rin = (sw ? rs : rc) * (1.0f - 1e-5f);
  const n3_cut cut{rho0, rc * rc, rs, sw ? 1.0f / (rc - rs) : 0.0f, rin * rin, L.rc_d};
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
  k_pairs_cutn3<MT, MS, 1, CUT, CNT, BAL><<<sw ? L.grid : L.grid_hard, kWarps * 32, SM, s>>>( \
      L.xs, L.ys, L.zs, L.nslots, L.nT, L.pairs, np, L.acc, cut, L.gbox, rc2m, pair_count)
  if (L.ipt == 2 && L.T == 512) OD_CUTN3(2, 2, true, kCutBalSmem);
  else if (L.ipt == 4 && L.T == 1024) OD_CUTN3(4, 4, false, (n3_traits<4, 4, 1>::SMEM));
  else return cudaErrorInvalidValue;
#undef OD_CUTN3L
#undef OD_CUTN3
  k_slot_take<<<(L.nslots + 255) / 256, 256, 0, s>>>(L.nslots, L.acc, L.perm, part_hi, part_lo);
  return cudaGetLastError();
}
