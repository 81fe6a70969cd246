/*
 * opendust_gb300.h — C ABI of the GB300 superion step engine.
 *
 * This is the drop-in boundary for OpenDust's per-timestep superion update.
 * In the reference (OpenDust, src/opendust/opendust.py) that update is an
 * OpenMM program: a CustomNonbondedForce for ion–ion forces (opendust.py:471-485),
 * one CustomExternalForce per grain (opendust.py:350-360, :487-495), a trap
 * CustomExternalForce (opendust.py:552-577), a field force (opendust.py:579-585),
 * a CustomIntegrator program (opendust.py:839-1037) driven by
 * integrator.step(1) (opendust.py:1061), and a per-step host tail
 * (opendust.py:1117-1383) that reads integrator globals back with
 * getGlobalVariableByName and writes grain charges with context.setParameter.
 * Every entry point below replaces one of those call sites; the citation on
 * each declaration names the one it replaces.
 *
 * Conventions
 *  - Plain C types only; the caller owns every host array, the library owns all
 *    device memory it allocates.
 *  - No exceptions cross the ABI: every call returns od_status; a message for the
 *    last failure on a handle is returned by od_last_error(handle) (or by
 *    od_last_error(NULL) for failures without a handle).
 *  - One host thread per handle. Each handle owns one CUDA stream.
 *  - All device-side waits inside the library are bounded; a wait that runs out
 *    sets a device error word that the next host call reports as OD_ERR_TIMEOUT. The step
 *    that timed out is incomplete (its ion–ion accumulators may be partly filled): destroy the
 *    handle and start again from the last good state.
 *  - Units at the boundary are SI (m, s, m/s, C, kg, N), as in the reference API.
 *
 * Random numbers (identical definition in the CUDA library and the CPU oracle)
 *  Philox4x32-10 (Salmon et al., SC'11), key = (seed & 0xffffffff, seed >> 32),
 *  counter = (ion index, step index, stream id, simulation id).
 *  uniform  u = (w >> 8) * 2^-24            in [0,1)
 *  uniform' u = ((w >> 8) + 1) * 2^-24      in (0,1]
 *  gaussian pair from words (a,b): sqrt(-2 ln u'(a)) * (cos, sin)(2 pi u(b))
 *  Stream ids are the OD_RNG_* constants below; the word use of each stream is
 *  documented beside it.
 */
#ifndef OPENDUST_GB300_H
#define OPENDUST_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OD_ABI_VERSION 3

typedef enum od_status {
  OD_OK = 0,
  OD_ERR_INVALID = 1,      /* bad argument or configuration */
  OD_ERR_CUDA = 2,         /* CUDA runtime failure (message has the CUDA error) */
  OD_ERR_OOM = 3,          /* device allocation failed or HBM budget exceeded */
  OD_ERR_STATE = 4,        /* call not valid in the handle's current state */
  OD_ERR_TIMEOUT = 5,      /* a bounded device wait ran out */
  OD_ERR_UNSUPPORTED = 6,  /* feature not compiled in / no suitable GPU */
  OD_ERR_CAPACITY = 7      /* an output buffer given by the caller is too small */
} od_status;

/* distributionType (opendust.py:261, :302): "Maxwellian" / "fieldDriven"; MATTHEWS is the
 * plasma model of the reference's chains/matthews.py fork (PlasmaParametersInSIUnitsMatthews,
 * matthews.py:50-112): shifted-Maxwellian inflow through the top face only, per-DOF
 * charge-exchange collisions, specular reflection at the side wall (matthews.py:653-682). */
enum { OD_DIST_MAXWELLIAN = 0, OD_DIST_FIELD_DRIVEN = 1, OD_DIST_MATTHEWS = 2 };
/* ion trap: the 14-term even polynomial alpha[] (opendust.py:499-577), the fork's radial
 * polynomial with height-dependent coefficients alpha_k(h) tabulated on uniform knots and
 * interpolated by natural cubic splines (OpenMM Continuous1DFunction, matthews.py:395-478), or
 * none (simulate(considerTrap=False), matthews.py:505-514). */
enum { OD_TRAP_POLY = 0, OD_TRAP_TABLE = 1, OD_TRAP_NONE = 2 };
#define OD_MAX_TRAP 128
/* chargeCalculationMethod (opendust.py:1120, :1153): "given" / "consistent" / "oml" */
enum { OD_CHARGE_GIVEN = 0, OD_CHARGE_CONSISTENT = 1, OD_CHARGE_OML = 2 };
/* ion–neutral collisions.
 *  PER_DOF: the reference's field-driven model (opendust.py:869-873): each velocity
 *           component independently replaced by v_T*gaussian with probability d_t*w_c.
 *  MFP:     charge exchange with a constant mean free path (rate |v|/mfp), sampled by the
 *           null-collision method; the whole velocity is replaced by a neutral draw. */
enum { OD_COLL_NONE = 0, OD_COLL_PER_DOF = 1, OD_COLL_MFP = 2 };
/* ion–ion force: all pairs (NoCutoff, opendust.py:472) or cutoff with the OpenMM
 * switching polynomial (CutoffNonPeriodic + switching, opendust.py:481-485) */
enum { OD_FORCE_ALLPAIRS = 0, OD_FORCE_CUTOFF = 1 };
/* injection tables: index into od_config.tab_* */
enum { OD_TAB_TOP = 0, OD_TAB_BOTTOM = 1, OD_TAB_SIDE = 2, OD_TAB_VZ = 3, OD_NTAB = 4 };

/* Philox stream ids (counter word 2) and the words each one uses. */
enum {
  OD_RNG_COLL_TEST = 1,  /* PER_DOF: w0..w2 = per-axis collision test u <= d_t*w_c */
  OD_RNG_COLL_GAUSS = 2, /* PER_DOF: gauss(w0,w1) -> (gx,gy), gauss(w2,w3).cos -> gz */
  OD_RNG_MFP_TEST = 3,   /* MFP: w0 = null-collision screen, w1 = real/null acceptance */
  OD_RNG_MFP_GAUSS = 4,  /* MFP: new velocity v_T*(gx,gy,gz) as for COLL_GAUSS */
  OD_RNG_FACE = 5,       /* w0: face choice (opendust.py:923-926) */
  OD_RNG_TOP_V = 6,      /* gauss(w0,w1) -> (gx,gy), w2 -> u for the top inverse CDF */
  OD_RNG_TOP_X = 7,      /* w0 -> radius^2 fraction, w1 -> angle fraction */
  OD_RNG_BOT_V = 8,      /* as TOP_V with the bottom table */
  OD_RNG_BOT_X = 9,      /* as TOP_X */
  OD_RNG_SIDE_X = 10,    /* w0 -> angle fraction, w1 -> axial fraction */
  OD_RNG_SIDE_V = 11,    /* gauss(w0,w1) -> (gy,gz), w2 -> u for side (and v_z) tables */
  OD_RNG_TRAP = 13,      /* trap-fit sample point p: counter (p,0,13,0); w0 radius^2, w1 angle, w2 axial */
  OD_RNG_INIT_X = 14,    /* initial position of ion i, attempt a: counter (i,a,14,sim); w0 radius^2,
                            w1 angle, w2 axial */
  OD_RNG_INIT_V = 15     /* initial velocity of ion i: counter (i,0,15,sim): gauss(w0,w1) -> (gx,gy),
                            gauss(w2,w3).cos -> gz; counter (i,1,15,sim) w0 -> u for the v_z table */
};

#define OD_MAX_GRAINS 16
#define OD_MAX_TABLE 256

/* Everything one simulation needs; SI units. Mirrors the state that the reference
 * builds in OpenDust.__init__ (opendust.py:255-360) and simulate() setup
 * (opendust.py:370-1044). Array pointers are read during od_create only. */
typedef struct od_config {
  int32_t abi_version;      /* must be OD_ABI_VERSION */
  int32_t distribution;     /* OD_DIST_* */
  int32_t collision_model;  /* OD_COLL_* */
  int32_t force_method;     /* OD_FORCE_* */
  int64_t n_ions;           /* N superions (opendust.py:280) */
  int64_t n_steps;          /* n: length of the per-step result series (opendust.py:282) */
  int64_t avg_start;        /* first step of the steady-state time average */
  int32_t n_grains;         /* P <= OD_MAX_GRAINS */
  int32_t sim_id;           /* Philox counter word 3 */
  uint64_t seed;            /* Philox key */

  /* constants as written in the reference (opendust.py:64-67) */
  double k_B, e, eps_0, m_e;
  /* plasma (opendust.py:49-77, :112-143) */
  double T_e, T_n, n_inf, m_i;
  double r_D_e;             /* electron Debye length = length unit lambda */
  double v_T, v_fl;         /* thermal and flow speed [m/s] */
  double E;                 /* external field along z [V/m] (fieldDriven) */
  double w_c;               /* ion–neutral collision frequency [1/s] (PER_DOF) */
  double mfp;               /* mean free path [m] (MFP) */
  /* simulation (opendust.py:181-200) */
  double R, H, d_t, r_0, N_s;
  /* cutoff (opendust.py:481-485): cutoff and switching distance [m]; switch_dist <= 0: none */
  double cutoff, switch_dist;
  /* trap polynomial coefficients alpha[0..14] (opendust.py:525-550); alpha[0] unused */
  double alpha[15];
  /* face probabilities (opendust.py:806-837) */
  double p_top, p_side, p_bottom;
  /* piecewise-linear inverse CDFs (opendust.py:608-787): for node i in 1..n-1 the
   * reference term is v[i-1] + (u - xi[i-1]) * slope[i] on xi[i-1] <= u <= xi[i].
   * v and slope in m/s (bottom table already negated, as opendust.py:716-717). */
  int32_t tab_n[OD_NTAB];
  const double* tab_v[OD_NTAB];
  const double* tab_xi[OD_NTAB];
  const double* tab_slope[OD_NTAB];
  /* grains (opendust.py:25-40, :314-338) */
  const double* grain_x;
  const double* grain_y;
  const double* grain_z;
  const double* grain_r;
  const double* grain_q0;
  const int32_t* grain_method; /* OD_CHARGE_* */
  /* external field order (matthews.py:481-495): 0 uniform E (fieldDriven and the fork's
   * order 0); 2: E(z) = E + field_alpha z + field_beta z^2 for field_z1 <= z <= field_z7,
   * E(field_z1) below and E(field_z7) above (the derivative of the fork's potential).
   * Units V/m, V/m^2, V/m^3, m. Applies to MATTHEWS; fieldDriven uses order 0 with E. */
  int32_t field_order;
  int32_t trap_kind;        /* OD_TRAP_* */
  double field_alpha, field_beta, field_z1, field_z7;
  /* OD_TRAP_TABLE: trap_tab[k * trap_n + j] = alpha_k at h_j = -H/2 + j H/(trap_n - 1),
   * k = 0..4 (coefficients of rho^0, rho^2, .., rho^8, rho = r/r_D_e, dimensionless as the
   * fork's fit returns them); 4 <= trap_n <= OD_MAX_TRAP. Zero outside [-H/2, H/2]. */
  int32_t trap_n;
  const double* trap_tab;
  /* per-grain factors of the host tail, or NULL: grain_field[p] is the field at grain p
   * [V/m] so that forceExternalField_z = q_p * grain_field[p] (NULL: E for fieldDriven, 0
   * otherwise); grain_out[3p..3p+2] is the out-of-domain trap force per unit grain charge
   * [N/C] for OD_TRAP_TABLE (the fork evaluates it with quartic splines of the table,
   * matthews.py:978-1007; NULL: zero). */
  const double* grain_field;
  const double* grain_out;
  /* Ion–ion force interval k (no counterpart in the reference, whose integrator evaluates the
   * ion–ion force every step, opendust.py:864-877). 0 or 1: every step, the reference's
   * integrator. k > 1: impulse multiple time stepping: the ion–ion force is evaluated at the
   * end of steps k-1, 2k-1, ... (step index s with s % k == k - 1) and applied as a half kick
   * of k times its size at the end of that step and at the start of the next; the other steps
   * move the ions under the grain, trap and field forces only. Between evaluations the stored
   * ion–ion sums still follow re-injection (removed ions' terms out, new ions' terms in). An
   * approximation that cuts pair work by k: use it where its error on the quantities of
   * interest has been measured (opendust_gb300.tuning.choose_force_interval). */
  int32_t force_every;
} od_config;

typedef struct od_handle od_handle;

/* Library identification. */
int32_t od_abi_version(void);
const char* od_version(void);
/* Number of CUDA devices visible (0 on a host without a GPU); never allocates. */
int32_t od_device_count(void);

/* Replaces mm.Context(system, integrator, Platform "CUDA", {DeviceIndex, Precision})
 * and the System/force/integrator build (opendust.py:469-604, :839-1044).
 * Allocates device state for cfg->n_ions ions and the n_steps result series. */
od_status od_create(const od_config* cfg, int32_t device, od_handle** out);

/* Replaces Context destruction. Safe on NULL. */
od_status od_destroy(od_handle* h);

/* Message for the last failure on h (or the last failure without a handle if h is NULL). */
const char* od_last_error(const od_handle* h);

/* Replaces context.setPositions / setVelocities (opendust.py:1043-1044) and the
 * restart-file read (opendust.py:452-466). pos [m], vel [m/s], both n x 3 row-major.
 * Positions are held cell-relative: per axis a cell index c on a grid of side s (in Debye
 * lengths, the smallest power of two not below 1/256 of the domain's half extent) and the FP32 offset
 * x - c s, rounded once from the FP64 input; the force, flag and injection kernels read the
 * absolute FP32 position fmaf(c, s, offset) derived from it each step. A non-finite position or
 * velocity is OD_ERR_INVALID (nothing is copied). */
od_status od_set_state(od_handle* h, const double* pos, const double* vel, int64_t n);

/* Samples the initial ion state on the device (replaces the host loops of opendust.py:373-451):
 * positions uniform in the cylinder and outside every grain (rejection, inclusive grain
 * surface as in the reference), velocities N(0, v_T) across and N(v_fl, v_T) along the axis
 * (Maxwellian), or, for field-driven plasmas, v_z from the piecewise-linear inverse CDF given by
 * nodes vz_v [m/s] / vz_cdf (vz_n >= 2; the table of opendust.py:405-448). Random numbers:
 * streams OD_RNG_INIT_X / OD_RNG_INIT_V with the configuration's seed. Then computes the
 * ion–ion sums like od_set_state. */
od_status od_init_state(od_handle* h, const double* vz_v, const double* vz_cdf, int32_t vz_n);

/* Screened potential of the current ions at grid points: pot[j * n_r + i] =
 * sum over ions of exp(-r)/(r + r_0) with r the distance from (gr[i], 0, gz[j]) in units of
 * r_D_e (FP64, fixed summation order). Replaces the CuPy loop of the fork's trap fit
 * (matthews.py:397-421), which evaluates this sum from the simulation's own ions. */
od_status od_ion_potential_grid(od_handle* h, const double* gr, const double* gz, int32_t n_r,
                                int32_t n_z, double* pot);

/* Replaces the fork's trap force setup (matthews.py:423-478: the fitted or file-read table
 * and its Continuous1DFunctions): switches the handle to OD_TRAP_TABLE with trap_tab / trap_n
 * as in od_config (n = 0: OD_TRAP_NONE) and the per-grain out-of-domain factors grain_out
 * [P][3] (N/C, may be NULL). Takes effect at the next step. */
od_status od_set_trap_table(od_handle* h, const double* trap_tab, int32_t n,
                            const double* grain_out);

/* Moves the grains and sets their charges between windows, keeping the ions resident (the
 * dust-dynamics driver of the reference, examples/DustDynamics/TwoParticles/launch.py:120-224,
 * rebuilds the OpenDust object each iteration and passes the ions through a restart file).
 * x, y, z [m], q [C] per grain; grain_field [P] and grain_out [P][3] as in od_config (NULL
 * keeps the current factors). The ion–ion sums are unchanged; the grain forces on the ions
 * follow at the next step. */
od_status od_set_grains(od_handle* h, const double* x, const double* y, const double* z,
                        const double* q, const double* grain_field, const double* grain_out);

/* Starts a new result window: the next step writes series row 0 and restarts the time
 * averages; the ion state, the grain charges and the random streams continue (the Philox
 * step counter keeps counting across windows). No counterpart in the reference: it creates
 * a new simulation per window (launch.py:120-145). */
od_status od_begin_window(od_handle* h);

/* Replaces context.getState(...).getPositions/getVelocities (opendust.py:1074-1078, :1102-1105).
 * Positions are the cell-relative state, exactly (c s + offset in FP64). */
od_status od_get_state(od_handle* h, double* pos, double* vel, int64_t n);

/* Replaces `integrator.step(1)` plus the host tail, nsteps times (opendust.py:1059-1383).
 * Each step appends one entry to the result series. Fails with OD_ERR_STATE when the
 * series (cfg->n_steps entries) is full. */
od_status od_step(od_handle* h, int64_t nsteps);

/* Device timing of od_step (no counterpart in the reference, which times simulate() with
 * time.time(), performance/NVIDIA-V100/benchmark.py:82-87). With timing enabled, od_step
 * launches kernel by kernel and records CUDA events on the handle's stream around every step
 * and every all-pairs force launch; od_get_timing returns the summed device milliseconds.
 * enable: 0 off, 1 on (the cutoff force kernels also count the pairs inside the cutoff for
 * od_get_cutoff_pairs), 2 on without counting (the kernels a step runs untimed). Enabling
 * resets the sums and the count. Without timing, od_step replays a CUDA graph of one step. */
od_status od_set_timing(od_handle* h, int32_t enable);
od_status od_get_timing(od_handle* h, double* step_ms, int64_t* steps, double* pair_ms,
                        int64_t* pair_launches);
/* Pairs inside the cutoff evaluated by the cutoff force kernel while timing was enabled
 * (0 for the all-pairs method). */
od_status od_get_cutoff_pairs(od_handle* h, int64_t* pairs);
/* Use (1, default) or bypass (0) the CUDA-graph replay of a step. */
od_status od_set_graph(od_handle* h, int32_t enable);
/* Work decomposition of the all-pairs force kernel (OpenMM picks its own nonbonded
 * kernel configuration; this exposes ours). variant 0: shared-memory broadcast of each
 * source, 1: warp-shuffle broadcast, 2: packed f32x2 pair arithmetic on SoA tiles (two
 * targets per thread), 3: as 2 with Newton reciprocals for half of the targets (tile redone on
 * the SFU when a pair is too close), 4: as 3 with a warp-vote SFU fallback per pair,
 * 5: packed with one target per thread (targets_per_thread 1), 6: as 5 with every other source
 * pair on the Newton path of variant 4, 7: each unordered pair evaluated once and applied to
 * both ions (threads 256; targets_per_thread = target ions per lane: 2 or 4 with as many source
 * ions, 8 with two; jsplit = ions per tile, 1024, 2048 or 4096 (not 1024 with 8; also 512 with
 * 2), <= 0 for the default). Variants 2-7 add their sums into 64-bit fixed-point accumulators (24
 * bytes per ion) with integer atomics, so results do not depend on the order of the GPU's
 * blocks. From 2^14 ions od_create selects variant 7.
 * jsplit <= 0 picks the source split from the SM count. Takes effect at the next step.
 * Cutoff method (force_method OD_FORCE_CUTOFF): variant 0 or 2 walks a stencil of cells per
 * target cell (scalar or packed); variant 3 (the default) sorts
 * the ions along a Hilbert curve and evaluates each pair inside the cutoff once over tile
 * pairs whose bounding boxes come within it — targets_per_thread 2 with 512-ion tiles
 * (balanced group-pair lists) or 4 with 1024-ion tiles; a positive jsplit must name that tile
 * size; 24 bytes of accumulators per ion slot. */
od_status od_set_pair_plan(od_handle* h, int32_t threads, int32_t targets_per_thread,
                           int32_t variant, int32_t jsplit);
/* Autotuner: times every supported (threads, targets_per_thread, variant) and three source
 * splits on the handle's current positions and keeps the fastest; with use_cache the result
 * cached for this (device, padded size) in the process is reused. *best_pairs_per_s receives
 * the measured rate (0 when cached). All-pairs method only. */
od_status od_autotune(od_handle* h, int32_t use_cache, double* best_pairs_per_s);
/* plan5 = {threads, targets_per_thread, variant, jsplit (variant 7: ions per tile), chunk} */
od_status od_get_pair_plan(const od_handle* h, int32_t* plan5);
/* FP32 FMA throughput of the device in TFLOP/s (2 flops per FMA), measured by a short probe
 * kernel: the denominator of the all-pairs kernel's roofline. */
od_status od_probe_fp32_peak(int32_t device, double* tflops);
/* ---- Shards of one simulation (replaces the reference's multi-GPU OpenMM context:
 * Platform property DeviceIndex "0,1,..." of opendust.py:1040-1042, timed by
 * performance/MultipleGPU/benchmark.py:83). One handle per GPU owns the ions [first,
 * first + count) of a simulation of cfg->n_ions ions (first a multiple of 512, count a multiple
 * of 512 except for the last shard); every shard keeps all positions as sources. A step is five
 * calls per shard with three all-gathers between them (the caller moves the data: MPI, NCCL,
 * torch.distributed, or plain copies; pointers may be host or device memory):
 *   od_shard_begin       kick and drift of the shard's ions; writes their positions, 3 x count
 *                        floats (x, then y, then z; units of r_D_e), to xyz_out
 *   all-gather           -> xyz_all, 3 x n_ions floats, shards in order
 *   od_shard_forces      ion–ion sums of the shard's ions over all positions, kick, flags, the
 *                        shard's ordered compaction and re-injection; *n_list = its entries
 *   od_shard_get_list    the shard's entries: global index, flag bits, position before and
 *                        after re-injection and velocity (float4 each, units of r_D_e, d_t)
 *   all-gather           -> the run's list, shards in order (= increasing global index)
 *   od_shard_set_list    grain sums over the run's list, the re-injected positions, correction
 *                        and orbit sums of the shard's ions; writes the shard's orbit partial
 *                        sums (orbit_blocks x P x 3 doubles, od_shard_info) to orbit_out
 *   all-gather           -> orbit_all, every shard's partials in order
 *   od_shard_finish      the FP64 tail (charges, forces, series); every shard holds the series
 * All ion–ion sums use the directed all-pairs plan of a single simulation of n_ions ions
 * (variant 5, the source split of jsplit chunks, 0: the default), and every sum keeps the
 * single-simulation order: the shards' results equal those of one handle with that plan, bit for
 * bit. All-pairs force, force_every <= 1, Maxwellian or field-driven ions only
 * (OD_ERR_UNSUPPORTED otherwise). Calls out of order return OD_ERR_STATE. */
od_status od_shard_create(const od_config* cfg, int64_t first, int64_t count, int32_t jsplit,
                          int32_t device, od_handle** out);
/* pos_all: n_ions x 3 positions of the whole run (m); vel_own: count x 3 velocities of the
 * shard's ions (m/s). Computes the initial ion–ion sums (as od_set_state). */
od_status od_shard_set_state(od_handle* h, const double* pos_all, const double* vel_own);
od_status od_shard_begin(od_handle* h, float* xyz_out);
od_status od_shard_forces(od_handle* h, const float* xyz_all, int64_t* n_list);
od_status od_shard_get_list(od_handle* h, int32_t* idx, int32_t* bits, float* old4, float* new4,
                            float* v4);
od_status od_shard_set_list(od_handle* h, int64_t n, const int32_t* idx, const int32_t* bits,
                            const float* old4, const float* new4, const float* v4,
                            double* orbit_out);
od_status od_shard_finish(od_handle* h, const double* orbit_all);
od_status od_shard_info(const od_handle* h, int64_t* first, int64_t* count, int64_t* n_total,
                        int64_t* orbit_blocks);

/* Self test of the bounded device waits (no counterpart in the reference, whose OpenMM waits
 * are unbounded). One thread on `device` arms an mbarrier and waits on it with the same wait
 * routine the step kernels use, but with `limit` polls (1 to 2^26) instead of 2^26. With
 * arrive = 0 nothing arrives, the wait runs out, the kernel records it in a device error word
 * and returns, and the call returns OD_ERR_TIMEOUT with the context still usable; with
 * arrive != 0 the thread arrives first and the call returns OD_OK. */
od_status od_selftest_wait(int32_t device, uint32_t limit, int32_t arrive);

/* Index of the next step (number of steps taken so far). */
int64_t od_step_index(const od_handle* h);

/* Replaces the per-step reads of dustParticles[p].q / forceIonsOrbit / forceIonsCollect /
 * forceDust / forceExternalField (opendust.py:1117-1383). Copies steps [first, first+count)
 * into row-major host arrays: q [count x P] (C), forces [count x P x 3] (N). Any output
 * pointer may be NULL. f_field is zero for Maxwellian runs. */
od_status od_get_series(od_handle* h, int64_t first, int64_t count, double* q,
                        double* f_orbit, double* f_collect, double* f_dust, double* f_field);

/* FP64 time averages over steps [avg_start, steps taken): out has P x 13 doubles per grain:
 * q, f_orbit[3], f_collect[3], f_dust[3], f_field[3]. *n_avg receives the number of steps. */
od_status od_get_averages(od_handle* h, double* out, int64_t* n_avg);

/* Ion–ion force on a given snapshot (the CustomNonbondedForce of opendust.py:471-485 evaluated
 * alone): pos [m] n x 3 -> force [N] n x 3 on each ion, with the handle's force method.
 * The positions are rounded to the device representation first; od_snapshot_positions
 * returns exactly the values the kernel consumed. */
od_status od_force_snapshot(od_handle* h, const double* pos, int64_t n, double* force);

/* The device representation of a snapshot, as doubles [m] (what od_force_snapshot and
 * od_collect_flags consume for the same input). */
od_status od_snapshot_positions(od_handle* h, const double* pos, int64_t n, double* pos_dev);

/* Collection / removal flags of opendust.py:894-910 on a given snapshot: idx_out receives, in
 * increasing order, every ion index with inside_dust_p or outside_domain set (cap entries max);
 * *count the number of such ions; grain_counts[P] the number inside each grain (delta_q_p of
 * opendust.py:911-912). Returns OD_ERR_CAPACITY if count > cap (count is still set). */
od_status od_collect_flags(od_handle* h, const double* pos, int64_t n, int64_t* idx_out,
                           int64_t cap, int64_t* count, int64_t* grain_counts);

/* Monte-Carlo background potential of the trap fit (the CuPy loop of opendust.py:499-523):
 * for an n_r x n_h grid (rows: radius linspace(0,R/lambda,n_r); columns: height
 * linspace(0,H/(2 lambda),n_h)) writes the mean of exp(-r)/(r+0.001) over n_points
 * uniform points of the cylinder (lambda units), row-major into pot[n_r*n_h].
 * Points come from Philox stream OD_RNG_TRAP with the given seed. */
od_status od_trap_potential(double R_over_lambda, double H_over_lambda, int32_t n_r, int32_t n_h,
                            int64_t n_points, uint64_t seed, int32_t device, double* pot);

/* ---- Batches: many independent simulations stepped together (no counterpart in the
 * reference, whose parameter sweeps call simulate() once per point, e.g.
 * examples/Piel2017/Figure5/launchPiel2017Figure5.py:32-106). Every stage of a batch step is
 * one launch for all members; the N^2 stage is one persistent launch over work items of all
 * members. Members are ordinary handles: read their results with od_get_series /
 * od_get_averages / od_get_state on od_batch_member(). A member's results are bitwise those of
 * the same simulation stepped alone. Members use the all-pairs force method. */
typedef struct od_batch od_batch;
od_status od_batch_create(int32_t device, od_batch** out);
/* Creates a member from cfg with initial state pos/vel (as od_create + od_set_state), or, with
 * pos = vel = NULL, a Maxwellian initial state sampled on the device (od_init_state); *slot
 * receives its slot index. May be called between steps (continuous batching). */
od_status od_batch_add(od_batch* b, const od_config* cfg, const double* pos, const double* vel,
                       int32_t* slot);
/* Each-pair-once plan of a batch member (no counterpart in the reference): (ions per lane, tile)
 * = (4, 1024) or (8, 2048), the two shapes the batched kernels run; od_batch_add gives the
 * od_batch_pair_plan rule, opendust_gb300.tuning.batch_plan_for picks by measurement per size
 * bucket. Results change by FP32 rounding only. */
od_status od_batch_set_plan(od_batch* b, int32_t slot, int32_t ions_per_lane, int32_t tile);
od_status od_batch_remove(od_batch* b, int32_t slot);
od_handle* od_batch_member(od_batch* b, int32_t slot);
int32_t od_batch_size(const od_batch* b);
/* Advances every member by nsteps (fails with OD_ERR_STATE if a member's series would overflow). */
od_status od_batch_step(od_batch* b, int64_t nsteps);
/* Device milliseconds of the last od_batch_step (CUDA events on the batch stream). */
od_status od_batch_last_step_ms(const od_batch* b, double* ms);
/* The all-pairs plan a batch member with n_ions ions steps with (plan5 as od_get_pair_plan;
 * jsplit 0 = the member's default split): variant 7 with 4 x 4 ions per lane and 1024-ion
 * tiles up to 2^16 ions, 8 x 2 and 2048-ion tiles above (od_batch_set_plan changes it). A single
 * simulation given the same plan produces bitwise the same results. No
 * counterpart in the reference (it has no batching). */
od_status od_batch_pair_plan(int64_t n_ions, int32_t* plan5);
od_status od_batch_destroy(od_batch* b);
const char* od_batch_last_error(const od_batch* b);
/* Free and total device memory (admission control of a request server). */
od_status od_device_memory(int32_t device, int64_t* free_bytes, int64_t* total_bytes);
/* Device bytes a simulation created by od_create with this configuration allocates, including
 * the fixed-point accumulators and the cutoff's sort and tile-pair list (admission control). */
od_status od_config_device_bytes(const od_config* cfg, int64_t* bytes);

/* Trajectory dumps of OpenDust.simulate() (opendust.py:1071-1098, which writes them with a Python
 * loop per ion). Host only, no device work. Positions are n x 3 doubles in nm. Numbers are
 * written as Python's "{}".format writes a float (shortest round-trip digits; fixed notation for
 * decimal exponents -4..15, else d.ddde+XX), so the files are byte-identical to the reference's.
 * od_write_xyz_frame appends "n\nframe\n" and one "Ar\tx\ty\tz\n" line per ion to path;
 * od_write_csv_frame writes the file path with the header "x,y,z,density,mass" and one row per
 * ion, "\r\n" line ends as Python's csv.writer. Failures to open or write return OD_ERR_INVALID
 * (od_last_error(NULL) names the file). od_format_double writes one number (at most 32 chars
 * and a terminating NUL) and returns its length. */
od_status od_write_xyz_frame(const char* path, const double* xyz_nm, int64_t n, int64_t frame);
od_status od_write_csv_frame(const char* path, const double* xyz_nm, int64_t n, double density,
                             double mass);
int32_t od_format_double(double v, char* buf);
/* The restart file of OpenDust.simulate() (opendust.py:1099-1115; read at :452-466): one ion per
 * line, "x\ty\tz\tvx\tvy\tvz\n" in nm and nm/ps, numbers formatted as above. od_read_restart
 * reads the first n lines (strtod, as Python's float()); a file with fewer lines or fields
 * returns OD_ERR_INVALID. */
od_status od_write_restart(const char* path, const double* pos_nm, const double* vel_nmps,
                           int64_t n);
od_status od_read_restart(const char* path, int64_t n, double* pos_nm, double* vel_nmps);

/* Ion–ion forces for callers that cannot allocate device memory (no counterpart in the
 * reference). Plug-ins that live inside another runtime's allocator, loops that forbid
 * cudaMalloc after start-up, or frameworks that own every device buffer can still evaluate
 * the screened ion–ion force of opendust.py:472: the caller passes device arrays pos_dev
 * (n x 3 doubles, metres) and force_dev (n x 3 doubles, newtons, written), the Debye length
 * r_D_e, the softening r_0 and the prefactor kq_sq_s = k q_s^2 (J m, the reference's
 * "kq_sq_s" parameter). The call allocates and frees nothing: its scratch (positions in
 * device units, partial sums, an error word) is one file-scope device array of about 8.8 MB
 * that every GPU which loads this library holds until the process exits; it limits n to
 * 2..32768 (larger n returns OD_ERR_INVALID). The call runs on the calling thread's current
 * device and on `stream` (a cudaStream_t, NULL for the default stream) and returns after the
 * stream has finished it. The first call on each device looks up the array's device address
 * (cudaGetSymbolAddress), so make that first call before any stream capture. All calls share
 * the array: calls that overlap on the GPU (other streams, other host threads) race. r_0 must
 * be at least 1e-9 r_D_e (each ion's own pair has r = 0 and would overflow FP32 below that);
 * smaller values return OD_ERR_INVALID. The device address is cached per device ordinal for
 * the primary context: only the primary context is supported, and the cache is not cleared
 * by cudaDeviceReset, so do not call this after resetting a device in the same process. */
od_status od_ion_forces_static(const double* pos_dev, int64_t n, double r_D_e, double r_0,
                               double kq_sq_s, double* force_dev, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* OPENDUST_GB300_H */
