// od_internal.h — launch wrappers shared by the kernel and ABI translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include "od_common.cuh"

// Work decomposition of the all-pairs force kernel.
struct od_pair_plan {
  int nt;      // threads per block
  int ipt;     // targets per thread
  int jsplit;  // source chunks (grid.y); partial slabs written per ion
  int chunk;   // sources per chunk (multiple of OD_TJ)
  int variant; // 0: shared-memory broadcast, 1: warp-shuffle broadcast, 2: packed f32x2 with
               // SoA tiles (ipt 2), 3: as 2 with Newton reciprocals for half of the targets,
               // 4-6: further packed forms, 7: each unordered pair once (od_n3.cu)
  int tile;    // variant 7: ions per tile (1024, 2048 or 4096); ipt = targets per lane (2, 4:
               // as many sources; 8: two sources)
};

// Position views the all-pairs kernels read: float4 AoS, and SoA slices for variants 2-3.
struct od_pair_io {
  const float4* pos;
  const float *sx, *sy, *sz;
  unsigned long long* n3 = nullptr;  // variant 7: fixed-point ion–ion accumulators [3][Npad]
};

// Device buffers of one simulation.
struct od_dbufs {
  float4 *pos, *vel, *fhi, *flo;        // absolute FP32 positions (derived from rel each
                                        // step), velocities, ion–ion sums (two-float)
  float4* rel;                          // [Npad] position state: cell-relative FP32 offsets
                                        // and packed cell indices (od_rel_* in od_common.cuh)
  float4 *part_hi, *part_lo;            // [jsplit][Npad] partial sums
  uint32_t* flags;                      // [nwords] ballot words
  int32_t* list;                        // [Npad] flagged ion indices, increasing
  int32_t* list_bits;                   // [Npad] flag bits of each entry
  float4 *list_old, *list_new, *list_v; // [Npad] pre/post re-injection positions, velocities
  double* orbit_part;                   // [nb_corr][P][3]
  double *s_q, *s_orbit, *s_collect, *s_dust, *s_field;  // result series
  float* cq;                            // [P] A_id * q_param, FP32 copy for the ion kernels
  float *sx, *sy, *sz;                  // [Npad] SoA copy of positions (all-pairs sources)
  unsigned long long* n3;               // variant 7 fixed-point accumulators [3][Npad] (or NULL)
  size_t n3_len;                        // allocation at n3, in units of 4 bytes
};

int od_num_sms(int device);

// Variant 7 (od_n3.cu): whether (ions per lane, tile) has a kernel; the default (ions per lane,
// tile) for a padded ion count (returns the tile, 0 when none fits the byte budget); the size of
// the fixed-point accumulators in 4-byte units; and the launch (pair kernel, then with take the
// accumulators into slab 0 of ph/pl).
bool od_n3_supported(int ipt, int tile);
int od_n3_default(int Npad, size_t budget_bytes, int* ipt);
size_t od_n3_floats(int Npad, int tile);
cudaError_t od_n3_prepare(const od_pair_plan& pl);  // shared-memory opt-in, current device
cudaError_t od_launch_pairs_n3(const od_pair_plan& pl, const od_pair_io& io, int Npad, float4* ph,
                               float4* pl_lo, float rho0, cudaStream_t s, bool take = true);

// One member of a batch, as the batched kernels see it.
struct od_simdesc {
  const od_dparams* dp;
  od_dstate* ds;
  od_dbufs b;
  int N, Npad, nb, jsplit, chunk, nrec;
  float rho0, newton_r2;
  int n3_tile;  // variant-7 tile of this member (its accumulators are b.n3), 0 otherwise
};
// Device tables of one batch step.
struct od_batchview {
  const od_simdesc* sims;
  int nsims;
  const int2* blk_ion;   // (member, local 256-ion block) for the ion-parallel stages
  int nblk_ion;
  const int4* items;     // (member, 256-target block, j0, j1) all-pairs work items
  int nitems;
  const int2* blk_corr;  // (member, local block in [0, nb + nrec)) for correction/orbit sums
  int nblk_corr;
  int pair_grid;         // persistent blocks of the all-pairs stage
  unsigned int* next;    // work counter of the all-pairs stage
  uint32_t* err;
  // members on variant 7: (member, tile a, tile b, tiles) per instantiation (0: 4 x 4 with
  // 1024-ion tiles, 1: 8 x 2 with 2048-ion tiles), and (member, 256-ion block) row-sum blocks
  const int4* n3_items[2];
  int n3_nitems[2];
  const int2* n3_blk;
  int n3_nblk;
};
cudaError_t od_launch_batch_step(const od_batchview& v, cudaStream_t s);
// pot[k] = sum over ions i < N of exp(-r)/(r + rho0), r = |(pts[2k], 0, pts[2k+1]) - x_i|
cudaError_t od_launch_grid_potential(const float4* pos, int N, const double* pts, int npts,
                                     double rho0, double* out, cudaStream_t s);
cudaError_t od_launch_batch_pairs_n3(const od_batchview& v, cudaStream_t s);
// Variant-7 plan of a batch member (ions per lane through ipt; returns the tile, 0: none fits).
int od_n3_batch_plan(int Npad, size_t budget_bytes, int* ipt);

// Uniform cell grid of the cutoff path (lambda units): cell (cx, cy, cz) spans
// [lo + c*cx, lo + c*(cx+1)) per axis; ions outside the grid are clamped into border cells.
struct od_cellgeom {
  int gx, gy, gz, ncells;
  float c, inv_c, lox, loy, loz;
};
// Device cell list of the cutoff path.
// Cutoff over tile pairs (cutoff variant 3, od_cutn3.cu): ions sorted along a Hilbert curve of a
// G^3 cell grid, tiles of T consecutive sorted ions, and every tile pair whose bounding boxes
// come within the cutoff evaluated with each unordered pair once (64-ion group pairs farther
// apart than the cutoff skipped).
struct od_cutn3 {
  int G, bits, nb, ncells;          // cells per cube axis (power of two), key bits per axis,
                                    // cubes along z, nb * G^3
  float lo, lo_z, inv_s;            // grid origin (x and y, z) and 1 / cell side (lambda)
  int T, ipt, nT, nslots, nwords;   // tile, targets per lane, tiles, nT*T slots, bitmap words
  int32_t *cell_of, *count, *fill, *start;  // [N], [ncells], [ncells], [ncells + 1]
  int32_t* perm;                    // [nslots] ion of each sorted slot, -1 for sentinels
  float *xs, *ys, *zs;              // [nslots] sorted positions; sentinels in the tail
  float* box;                       // [nT][6] min xyz, max xyz
  float* gbox;                      // [nslots / 64][6] boxes of 64-slot groups
  uint32_t* adj;                    // [nT][nwords] tile pairs (a, b >= a) within the cutoff
  int32_t* rowptr;                  // [nT + 1] pair counts, then their exclusive prefix
  int2* pairs;                      // [nT (nT + 1) / 2] listed pairs, row-major
  unsigned long long* acc;          // [3][nslots] fixed-point ion–ion sums per sorted slot
  double rc_d;                      // cutoff / r_D_e in FP64 (the hard cutoff's exact test)
  int grid, grid_hard;              // persistent blocks of the pair kernel (switching, hard)
};
// cell grid of the tile-pair cutoff for N ions in a cylinder of radius R and height H (any
// unit): nb cubes of side `side` (that unit) along z, G^3 cells each
struct od_cgrid { int G, nb, ncells; double side; };
od_cgrid od_cutn3_grid(int N, double R, double H);
size_t od_cutn3_bytes(int N, int T, int ncells);
bool od_cutn3_supported(int ipt, int T);
cudaError_t od_cutn3_prepare(int ipt, int T);
int od_cutn3_blocks_per_sm(int ipt, int T, bool hard);  // after od_cutn3_prepare
cudaError_t od_launch_cutoff_n3(const od_cutn3& L, const float4* pos, int n, float4* part_hi,
                                float4* part_lo, float rho0, float rc, float rs, uint32_t* err,
                                unsigned long long* pair_count, cudaStream_t s);

struct od_cutlist {
  od_cellgeom g;
  od_cutn3* n3;          // cutoff variant 3 (or NULL)
  int32_t *cell_of, *count, *fill, *start, *chunk_prefix, *perm;  // start/chunk_prefix: ncells+1
  float *ox, *oy, *oz;   // sorted cell-relative offsets, 8-padded segments
  int4* stencil;         // source-cell offsets within the cutoff of a target cell
  int nstencil, cap;
  int32_t* chunk_prefix2; // ncells+1: prefix of 256-target chunks (packed kernel)
  bool packed;           // packed f32x2 kernel (default) or the scalar one
};
cudaError_t od_launch_cutoff(const od_cutlist& L, const float4* pos, int n, int Npad,
                             float4* part_hi, float4* part_lo, float rho0, float rc, float rs,
                             uint32_t* err, unsigned long long* pair_count, cudaStream_t s);

// Pointers into the allocation-free scratch array of od_ion_forces_static.
struct od_static_view {
  uint32_t* err;
  float *sx, *sy, *sz;
  float4 *part_hi, *part_lo;
  int max_split;
};
cudaError_t od_launch_static_forces(const od_static_view& v, const double* pos, int n, double lam,
                                    double r0, double scale, double* force, cudaStream_t s);

cudaError_t od_launch_pairs(const od_pair_plan& pl, const od_pair_io& io, int Npad, float4* part_hi,
                            float4* part_lo, float rho0, uint32_t* err, cudaStream_t s,
                            bool take = true);
// the same launch restricted to the first gridx_limit target blocks (autotuner probes)
cudaError_t od_launch_pairs_probe(const od_pair_plan& pl, const od_pair_io& io, int Npad,
                                  int gridx_limit, float4* part_hi, float4* part_lo, float rho0,
                                  uint32_t* err, cudaStream_t s);
cudaError_t od_launch_init_state(const od_dparams* dp, int N, float4* rel, float4* pos, float4* vel,
                                 const float* vz_v, const double* vz_cdf, int vz_n, uint32_t* err,
                                 cudaStream_t s);
cudaError_t od_launch_aos_to_soa(const float4* pos, int Npad, float* sx, float* sy, float* sz,
                                 cudaStream_t s);
cudaError_t od_launch_reduce(const od_dparams* dp, int Npad, int jsplit, const float4* part_hi,
                             const float4* part_lo, float4* fhi, float4* flo, cudaStream_t s);
// Force-evaluation context of one simulation: the all-pairs plan, or the cell list when cut != 0.
struct od_force_ctx {
  od_pair_plan plan;
  const od_cutlist* cut;
  float rho0, rc, rs;
  unsigned long long* pair_count;  // pairs inside the cutoff (cutoff path, optional)
  unsigned long long* acc;         // fixed-point ion–ion accumulators that K3 takes (or NULL)
};
// take: leave the ion–ion sums in slab 0 of (part_hi, part_lo) (false: in the accumulators)
cudaError_t od_launch_force(const od_force_ctx& fc, const od_pair_io& io, int n, int Npad,
                            float4* part_hi, float4* part_lo, uint32_t* err, cudaStream_t s,
                            bool take = true);
cudaError_t od_launch_step(const od_dparams* dp, od_dstate* ds, const od_dbufs& b, int N, int Npad,
                           int P, const od_force_ctx& fc, int nrec, cudaStream_t s);
cudaError_t od_launch_step_part(int part, const od_dparams* dp, od_dstate* ds, const od_dbufs& b,
                                int N, int Npad, int P, const od_force_ctx& fc, int nrec,
                                cudaStream_t s);
cudaError_t od_run_fp32_probe(int device, double* tflops);
// shards of one simulation (od_kernels.cu): K1 (part 0, positions also into the sources) or
// K3 + K4 (part 1); the ion–ion sums of the shard's ions over all sources (directed variants
// 2-6); the whole run's re-injection list -> grain sums and sources; correction and orbit sums
// of the shard's ions; the tail over all shards' orbit partials
cudaError_t od_launch_shard_part(int part, const od_dparams* dp, od_dstate* ds, const od_dbufs& b,
                                 int N, int Npad, int jsplit, float* sx, float* sy, float* sz,
                                 cudaStream_t s);
cudaError_t od_launch_shard_pairs(const od_pair_plan& pl, const float* sx, const float* sy,
                                  const float* sz, int nsrc_pad, int Npad_local, int tgt_off,
                                  float4* ph, float4* plo, float rho0, uint32_t* err,
                                  unsigned long long* acc, bool take, cudaStream_t s);
cudaError_t od_launch_shard_list(const od_dparams* dp, od_dstate* ds, int K, const int32_t* gidx,
                                 const int32_t* gbits, const float4* gnew, const float4* gv,
                                 float* sx, float* sy, float* sz, cudaStream_t s);
cudaError_t od_launch_shard_correct(const od_dparams* dp, const od_dstate* ds, const od_dbufs& b,
                                    int Npad_local, int nrec, const int32_t* gidx,
                                    const float4* gold, const float4* gnew, const float* sx,
                                    const float* sy, const float* sz, int nsrc, cudaStream_t s);
cudaError_t od_launch_shard_tail(const od_dparams* dp, od_dstate* ds, const od_dbufs& b,
                                 const double* orbit_all, int nb_all, cudaStream_t s);
// one-thread mbarrier wait that gives up after `limit` polls unless `arrive` (self test)
cudaError_t od_launch_wait_selftest(uint32_t* err, uint32_t limit, int arrive, cudaStream_t s);
cudaError_t od_launch_snapshot_flags(const od_dparams* dp, int n, int Npad, const float4* pos,
                                     uint32_t* flags, int32_t* list, int32_t* list_bits,
                                     double* counts, cudaStream_t s);
cudaError_t od_launch_set_charges(const od_dparams* dp, od_dstate* ds, float* cq, int P,
                                  cudaStream_t s);
cudaError_t od_launch_trap(double Rh, double Hh, int n_r, int n_h, int64_t n_points, uint64_t seed,
                           double* part, int nchunks, cudaStream_t s);

// Record msg as the last error of calls without a handle (od_last_error(NULL)); returns st.
od_status od_fail_nohandle(od_status st, const std::string& msg);

