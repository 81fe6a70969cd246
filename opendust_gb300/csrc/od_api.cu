// od_api.cu — the C ABI declared in include/opendust_gb300.h (host side).
//
// A handle owns one simulation's device state and one CUDA stream. Host arrays belong to
// the caller; every device buffer belongs to the handle. No C++ exception crosses the ABI.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <algorithm>
#include <cstddef>
#include <cstdlib>
#include <mutex>
#include <string>
#include <vector>
#include "od_internal.h"

#define OD_VERSION_STRING "opendust-gb300 0.1.0 (sm_103a)"

struct od_handle {
  int device = 0;
  cudaStream_t stream = nullptr;
  od_config cfg{};
  od_dparams hp{};
  od_dparams* dp = nullptr;
  od_dstate* ds = nullptr;
  od_dbufs b{};
  int N = 0, Npad = 0, P = 0, nb = 0, nrec = 32;
  int64_t step = 0;
  bool state_set = false;
  od_pair_plan plan{};
  // cutoff path (force_method == OD_FORCE_CUTOFF)
  bool has_cut = false;
  od_cutlist cut{};
  unsigned long long* d_pairs = nullptr;  // pairs inside the cutoff, counted in timing mode
  // snapshot scratch (allocated on first use)
  float4 *snap_pos = nullptr, *snap_hi = nullptr, *snap_lo = nullptr;
  double* snap_counts = nullptr;
  // CUDA graph of one step (production path)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  // force interval k > 1: the step graph without the ion–ion launch (steps that do not evaluate)
  cudaGraph_t graph_nf = nullptr;
  cudaGraphExec_t graph_exec_nf = nullptr;
  bool use_graph = true;
  // device timing (events on the handle's stream)
  bool timing = false;
  bool count_pairs = false;  // timing mode 1: the cutoff kernel also counts its pairs
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, int>> ev_step, ev_pair;  // indices into ev_pool
  double t_step_ms = 0, t_pair_ms = 0;
  int64_t t_steps = 0, t_pair_launches = 0;
  // shard of a larger simulation (od_shard_create): ions ion0 .. ion0 + N of n_total
  bool shard = false;
  int64_t ion0 = 0, n_total = 0;
  int Npad_total = 0, shard_phase = 0;
  float *ssx = nullptr, *ssy = nullptr, *ssz = nullptr;  // [Npad_total] every shard's positions
  int32_t *g_idx = nullptr, *g_bits = nullptr;            // [n_total] the run's list
  float4 *g_old = nullptr, *g_new = nullptr, *g_v = nullptr;
  double* g_orbit = nullptr;                              // [Npad_total / 256][P][3]
  std::string err;
};

static thread_local std::string g_err;

static od_status fail(od_handle* h, od_status st, const std::string& msg) {
  if (h) h->err = msg; else g_err = msg;
  return st;
}
od_status od_fail_nohandle(od_status st, const std::string& msg) { return fail(nullptr, st, msg); }
static od_status cuda_fail(od_handle* h, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  return fail(h, e == cudaErrorMemoryAllocation ? OD_ERR_OOM : OD_ERR_CUDA, m);
}
#define OD_CK(h, call)                                  \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, #call); \
  } while (0)

extern "C" int32_t od_abi_version(void) { return OD_ABI_VERSION; }
extern "C" const char* od_version(void) { return OD_VERSION_STRING; }
extern "C" int32_t od_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) { cudaGetLastError(); return 0; }
  return n;
}
extern "C" const char* od_last_error(const od_handle* h) {
  return h ? h->err.c_str() : g_err.c_str();
}

// smallest float not below d
static float float_ceil(double d) {
  float f = (float)d;
  if ((double)f < d) f = nextafterf(f, INFINITY);
  return f;
}
static void split2(double d, float& hi, float& lo) {
  hi = (float)d;
  lo = (float)(d - (double)hi);
}

// Plans whose ion–ion sums go to the fixed-point accumulators b.n3 (directed packed variants
// 2-6 and the each-pair-once variant 7; not the cutoff, not the scalar variants 0 and 1).
static bool uses_acc(const od_handle* h) {
  return !h->has_cut && h->b.n3 && h->plan.variant >= 2;
}

static od_force_ctx force_ctx(const od_handle* h, bool count_pairs) {
  od_force_ctx fc{};
  fc.plan = h->plan;
  fc.cut = h->has_cut ? &h->cut : nullptr;
  fc.rho0 = h->hp.rho0;
  fc.rc = h->hp.rc;
  fc.rs = h->hp.rs;
  fc.pair_count = (count_pairs && h->has_cut) ? h->d_pairs : nullptr;
  fc.acc = uses_acc(h) ? h->b.n3 : nullptr;
  return fc;
}
// slabs that hold the ion–ion sums after od_launch_force with take = true
static int force_jsplit(const od_handle* h) {
  return h->has_cut || uses_acc(h) ? 1 : h->plan.jsplit;
}

static od_status validate(const od_config* c) {
  if (!c) return fail(nullptr, OD_ERR_INVALID, "config is NULL");
  if (c->abi_version != OD_ABI_VERSION)
    return fail(nullptr, OD_ERR_INVALID, "config abi_version mismatch");
  if (c->n_ions < 2 || c->n_ions > (int64_t)1 << 30)
    return fail(nullptr, OD_ERR_INVALID, "n_ions must be in [2, 2^30]");
  if (c->n_grains < 0 || c->n_grains > OD_MAX_GRAINS)
    return fail(nullptr, OD_ERR_INVALID, "n_grains must be in [0, 16]");
  if (c->n_steps < 1) return fail(nullptr, OD_ERR_INVALID, "n_steps must be >= 1");
  if (c->distribution < OD_DIST_MAXWELLIAN || c->distribution > OD_DIST_MATTHEWS)
    return fail(nullptr, OD_ERR_INVALID, "distribution must be Maxwellian, fieldDriven or Matthews");
  if (c->field_order != 0 && c->field_order != 2)
    return fail(nullptr, OD_ERR_INVALID, "field_order must be 0 or 2");
  if (c->field_order == 2 && !(c->field_z7 >= c->field_z1))
    return fail(nullptr, OD_ERR_INVALID, "field order 2 needs field_z1 <= field_z7");
  if (c->trap_kind < OD_TRAP_POLY || c->trap_kind > OD_TRAP_NONE)
    return fail(nullptr, OD_ERR_INVALID, "unknown trap kind");
  if (c->trap_kind == OD_TRAP_TABLE &&
      (c->trap_n < 4 || c->trap_n > OD_MAX_TRAP || !c->trap_tab))
    return fail(nullptr, OD_ERR_INVALID, "a trap table needs 4..OD_MAX_TRAP knots");
  if (c->collision_model < OD_COLL_NONE || c->collision_model > OD_COLL_MFP)
    return fail(nullptr, OD_ERR_INVALID, "unknown collision model");
  if (c->collision_model == OD_COLL_MFP && !(c->mfp > 0))
    return fail(nullptr, OD_ERR_INVALID, "MFP collisions need mfp > 0");
  if (c->force_method != OD_FORCE_ALLPAIRS && c->force_method != OD_FORCE_CUTOFF)
    return fail(nullptr, OD_ERR_INVALID, "unknown force method");
  if (c->force_method == OD_FORCE_CUTOFF && !(c->cutoff > 0))
    return fail(nullptr, OD_ERR_INVALID, "cutoff method needs cutoff > 0");
  if (c->force_every < 0 || c->force_every > 1024)
    return fail(nullptr, OD_ERR_INVALID, "force_every must be in [0, 1024]");
  if (c->force_every > 1 && c->distribution == OD_DIST_MATTHEWS)
    return fail(nullptr, OD_ERR_INVALID, "force_every > 1 is not available for the fork's model");
  if (!(c->r_D_e > 0) || !(c->d_t > 0) || !(c->R > 0) || !(c->H > 0) || !(c->N_s > 0))
    return fail(nullptr, OD_ERR_INVALID, "r_D_e, d_t, R, H and N_s must be positive");
  for (int t = 0; t < OD_NTAB; t++) {
    if (c->tab_n[t] < 0 || c->tab_n[t] > OD_MAX_TABLE)
      return fail(nullptr, OD_ERR_INVALID, "injection table longer than OD_MAX_TABLE");
    if (c->tab_n[t] > 0 && (!c->tab_v[t] || !c->tab_xi[t] || !c->tab_slope[t]))
      return fail(nullptr, OD_ERR_INVALID, "injection table pointer is NULL");
  }
  if (c->tab_n[OD_TAB_TOP] < 2 && c->p_top > 0)
    return fail(nullptr, OD_ERR_INVALID, "top table needs at least 2 nodes");
  if (c->tab_n[OD_TAB_SIDE] < 2 && c->p_side > 0)
    return fail(nullptr, OD_ERR_INVALID, "side table needs at least 2 nodes");
  if (c->distribution == OD_DIST_FIELD_DRIVEN && c->tab_n[OD_TAB_VZ] < 2)
    return fail(nullptr, OD_ERR_INVALID, "fieldDriven needs the side v_z table");
  if (c->n_grains > 0 &&
      (!c->grain_x || !c->grain_y || !c->grain_z || !c->grain_r || !c->grain_q0 || !c->grain_method))
    return fail(nullptr, OD_ERR_INVALID, "grain array pointer is NULL");
  for (int g = 0; g < c->n_grains; g++)
    if (c->grain_method[g] < OD_CHARGE_GIVEN || c->grain_method[g] > OD_CHARGE_OML)
      return fail(nullptr, OD_ERR_INVALID, "unknown charge method");
  return OD_OK;
}

// Natural cubic spline through y[0..n-1] on uniform knots of spacing d (second derivative zero
// at both ends, as OpenMM's Continuous1DFunction): coef[j] = (c0, c1, c2, c3) of
// y_j + c1 t + c2 t^2 + c3 t^3 on [h_j, h_j+1], t = h - h_j. Tridiagonal solve (Thomas) in FP64.
static void natural_spline(const double* y, int n, double d, double (*coef)[4]) {
  std::vector<double> M(n, 0.0), cp(n, 0.0), dp(n, 0.0);
  // rows j = 1..n-2: M[j-1] + 4 M[j] + M[j+1] = 6 (y[j+1] - 2 y[j] + y[j-1]) / d^2
  for (int j = 1; j < n - 1; j++) {
    const double r = 6.0 * (y[j + 1] - 2.0 * y[j] + y[j - 1]) / (d * d);
    const double den = 4.0 - (j > 1 ? cp[j - 1] : 0.0);
    cp[j] = 1.0 / den;
    dp[j] = (r - (j > 1 ? dp[j - 1] : 0.0)) / den;
  }
  for (int j = n - 2; j >= 1; j--) M[j] = dp[j] - cp[j] * (j < n - 2 ? M[j + 1] : 0.0);
  for (int j = 0; j < n - 1; j++) {
    coef[j][0] = y[j];
    coef[j][1] = (y[j + 1] - y[j]) / d - d * (2.0 * M[j] + M[j + 1]) / 6.0;
    coef[j][2] = M[j] / 2.0;
    coef[j][3] = (M[j + 1] - M[j]) / (6.0 * d);
  }
}

// Tabulated trap (OD_TRAP_TABLE): knots over [-Hh/2, Hh/2] (lambda), coefficients times -A_ii.
static void fill_trap_table(od_dparams* p, const double* tab, int n, double Hh, double A_ii) {
  p->trap_kind = n > 0 ? OD_TRAP_TABLE : OD_TRAP_NONE;
  p->ttn = n;
  if (n <= 0) return;
  const double d = Hh / (n - 1);
  p->th0 = (float)(-Hh / 2.0); p->th1 = (float)(Hh / 2.0);
  p->tdh = (float)d; p->tinv_dh = (float)(1.0 / d);
  std::vector<double> c((size_t)(n - 1) * 4);
  for (int k = 0; k < 5; k++) {
    natural_spline(tab + (size_t)k * n, n, d, reinterpret_cast<double(*)[4]>(c.data()));
    for (int j = 0; j < n - 1; j++)
      for (int m = 0; m < 4; m++) p->tcf[k][j][m] = (float)(-A_ii * c[(size_t)j * 4 + m]);
  }
}

// Out-of-domain trap force on a grain per unit grain charge [N/C] (opendust.py:1258-1321: the
// gradient of the trap polynomial at the grain, times k q_s / r_D_e).
static void out_domain_per_charge(const od_dparams& p, double x, double y, double z, double* f) {
  const double* a = p.alpha;
  const double L = p.lam, L2 = L * L, L4 = L2 * L2, L6 = L4 * L2, L8 = L4 * L4;
  const double r = sqrt(x * x + y * y);
  const double r2 = r * r, r3 = r2 * r, r4 = r2 * r2, r5 = r4 * r, r6 = r4 * r2, r7 = r6 * r;
  const double z2 = z * z, z3 = z2 * z, z4 = z2 * z2, z5 = z4 * z, z6 = z4 * z2, z7 = z6 * z;
  double fR = (-2 * a[1] * r) / L2;
  fR += (-2 * a[3] * r * z2 - 4 * a[4] * r3) / L4;
  fR += (-4 * a[6] * r3 * z2 - 2 * a[7] * r * z4 - 6 * a[8] * r5) / L6;
  fR += (-4 * a[10] * r3 * z4 - 6 * a[11] * r5 * z2 - 2 * a[12] * r * z6 - 8 * a[13] * r7) / L8;
  fR *= p.k * p.q_s / L;
  double fH = (-2 * a[2] * z) / L2;
  fH += (-2 * a[3] * r2 * z - 4 * a[5] * z3) / L4;
  fH += (-2 * a[6] * r4 * z - 4 * a[7] * r2 * z3 - 6 * a[9] * z5) / L6;
  fH += (-4 * a[10] * r4 * z3 - 2 * a[11] * r6 * z - 6 * a[12] * r2 * z5 - 8 * a[14] * z7) / L8;
  fH *= p.k * p.q_s / L;
  if (r == 0) { f[0] = 0; f[1] = 0; }
  else { f[0] = fR * x / r; f[1] = fR * y / r; }
  f[2] = fH;
}

// Per-grain constants of the FP64 tail (charge update, opendust.py:1117-1202; dust–dust force,
// :1205-1235; out-of-domain force for the trap polynomial), so that the device tail evaluates one
// exponential and a few products per grain and step (FP64 is slow on GB300). Needs the tail
// constants and the grains of p; called again when grains move.
static void tail_consts(od_dparams* p) {
  const double pi = OD_PI_D;
  for (int g = 0; g < p->P; g++) {
    const double r = p->grs[g], S = r * r * 4.0 * pi;
    // gamma_e dt S e with gamma_e = n_inf sqrt(T_e k_B / pi / m_e / 2) exp(-e k q / r / T_e / k_B)
    p->ge_pref[g] = p->n_inf * sqrt(p->T_e * p->k_B / pi / p->m_e / 2.0) * p->dt * S * p->e;
    p->ge_arg[g] = -p->e * p->k / r / p->T_e / p->k_B;
    // OML: gamma_i dt S |e| with gamma_i = n_inf v_ti u/4 ((1 + 1/(2u*2) + chi/u^2) erf(u)
    // + exp(-u^2)/(u sqrt(pi))), chi = e k q / r / T_n / k_B (the reference's literal 2*u*2)
    const double u = p->v_fl_si / p->v_T_si / sqrt(2.0);
    const double v_ti = p->v_T_si * sqrt(2.0);
    const double c0 = p->n_inf * v_ti * u / 4.0 * p->dt * S * fabs(p->e);
    p->oml_a[g] = c0 * ((1.0 + 1.0 / (2.0 * u * 2)) * erf(u) + 1.0 / u / sqrt(pi) * exp(-(u * u)));
    p->oml_b[g] = c0 * erf(u) / (u * u) * (p->e * p->k / r / p->T_n / p->k_B);
    for (int j = 0; j < p->P; j++) {
      double* d = p->dd[g][j];
      if (j == g) { d[0] = d[1] = d[2] = 0.0; continue; }
      const double dx = p->gxs[g] - p->gxs[j], dy = p->gys[g] - p->gys[j], dz = p->gzs[g] - p->gzs[j];
      const double rr = sqrt(dx * dx + dy * dy + dz * dz);
      const double kk = p->k / (rr * rr * rr);
      d[0] = kk * dx; d[1] = kk * dy; d[2] = kk * dz;
    }
    if (p->trap_kind == OD_TRAP_POLY) out_domain_per_charge(*p, p->gxs[g], p->gys[g], p->gzs[g], p->gout[g]);
  }
}

static void fill_params(const od_config* c, int N, int Npad, od_dparams* p) {
  memset(p, 0, sizeof(*p));
  const double pi = OD_PI_D;
  p->N = N; p->Npad = Npad; p->P = c->n_grains; p->dist = c->distribution;
  p->coll = c->collision_model; p->method = c->force_method; p->sim = c->sim_id;
  p->nwords = Npad / 32;
  p->force_every = c->force_every > 1 ? c->force_every : 1;
  p->seed_lo = (uint32_t)(c->seed & 0xffffffffu);
  p->seed_hi = (uint32_t)(c->seed >> 32);
  const double lam = c->r_D_e, dt = c->d_t;
  const double k = 1.0 / (c->eps_0 * 4.0 * pi);
  const double q_s = fabs(c->e) * c->N_s;
  const double m_s = c->m_i * c->N_s;
  const double sc = dt * dt / (m_s * lam * lam * lam);
  const double A_ii = k * q_s * q_s * sc;
  p->A_ii = (float)A_ii;
  p->A_id_d = k * q_s * sc;
  p->A_id = (float)p->A_id_d;
  p->rho0 = (float)(c->r_0 / lam);
  const double Rh = c->R / lam, Hh = c->H / lam;
  p->Rh = (float)Rh; p->Hh = (float)Hh; p->Hh_half = (float)(Hh / 2.0);
  const double sf = q_s * dt * dt / (m_s * lam);  // field [V/m] -> acceleration (lambda/d_t^2)
  p->a_field = c->distribution != OD_DIST_MAXWELLIAN ? (float)(c->E * sf) : 0.f;
  p->field_order = c->distribution == OD_DIST_MATTHEWS ? c->field_order : 0;
  if (p->field_order == 2) {
    p->fa0 = (float)(c->E * sf);
    p->fa1 = (float)(c->field_alpha * lam * sf);
    p->fa2 = (float)(c->field_beta * lam * lam * sf);
    p->fz1 = (float)(c->field_z1 / lam);
    p->fz7 = (float)(c->field_z7 / lam);
  }
  p->trap_kind = c->trap_kind;
  if (c->trap_kind == OD_TRAP_TABLE) fill_trap_table(p, c->trap_tab, c->trap_n, Hh, A_ii);
  const double vunit = lam / dt;
  p->vT = (float)(c->v_T / vunit);
  p->vfl = (float)(c->v_fl / vunit);
  if (c->force_method == OD_FORCE_CUTOFF) {
    double rc = c->cutoff / lam, rs = c->switch_dist > 0 ? c->switch_dist / lam : rc;
    p->rc = (float)rc; p->rc2 = (float)(rc * rc); p->rs = (float)rs;
    p->inv_w = rc > rs ? (float)(1.0 / (rc - rs)) : 0.f;
  }
  for (int i = 0; i < 15; i++) {
    p->trapc[i] = (float)(-2.0 * A_ii * c->alpha[i]);
    p->alpha[i] = c->alpha[i];
  }
  for (int g = 0; g < c->n_grains; g++) {
    double gx = c->grain_x[g] / lam, gy = c->grain_y[g] / lam, gz = c->grain_z[g] / lam;
    double r = c->grain_r[g] / lam;
    p->gx[g] = gx; p->gy[g] = gy; p->gz[g] = gz; p->gr2[g] = r * r;
    split2(gx, p->gxh[g], p->gxl[g]);
    split2(gy, p->gyh[g], p->gyl[g]);
    split2(gz, p->gzh[g], p->gzl[g]);
    p->gr2f[g] = (float)(r * r);
    p->gxs[g] = c->grain_x[g]; p->gys[g] = c->grain_y[g]; p->gzs[g] = c->grain_z[g];
    p->grs[g] = c->grain_r[g];
    p->gmethod[g] = c->grain_method[g];
    p->gfield[g] = c->grain_field ? c->grain_field[g]
                                  : (c->distribution == OD_DIST_FIELD_DRIVEN ? c->E : 0.0);
    for (int d = 0; d < 3; d++) p->gout[g][d] = c->grain_out ? c->grain_out[3 * g + d] : 0.0;
  }
  p->Rh2 = Rh * Rh;
  p->Hh_half_d = Hh / 2.0;
  // cell side of the cell-relative positions: the power of two with the domain's half extent
  // at most 256 cells (of the 512 each way the 10-bit indices give)
  p->rel_s = (float)std::ldexp(1.0, (int)std::ceil(std::log2(std::max(Rh, Hh / 2.0) / 256.0)));
  p->rel_inv = 1.0f / p->rel_s;
  p->Rh2f = (float)(Rh * Rh);
  p->Hz_f = float_ceil(Hh / 2.0);
  p->p_coll = dt * c->w_c;
  // u <= p_coll with u = k 2^-24: k <= floor(p_coll 2^24) (exact in FP64); -1 below zero
  p->pcoll_int = p->p_coll < 0 ? -1
                 : (int32_t)std::min(floor(p->p_coll * 16777216.0), 16777216.0);
  if (c->collision_model == OD_COLL_MFP) {
    double mfp_h = c->mfp / lam;
    double vmax = 3.0 * fabs(c->v_fl / vunit) + 10.0 * (c->v_T / vunit);
    p->mfp_inv = (float)(1.0 / mfp_h);
    p->vmax_mfp = (float)vmax;
    p->Pmax_mfp = 1.0 - exp(-vmax / mfp_h);
    // u < Pmax with u = k 2^-24: k < ceil(Pmax 2^24)
    p->pmax_int = (uint32_t)std::min(ceil(p->Pmax_mfp * 16777216.0), 16777216.0);
    p->mfp_inv_d = 1.0 / mfp_h;
  }
  p->p_t = c->p_top; p->p_s = c->p_side; p->p_b = c->p_bottom;
  for (int t = 0; t < OD_NTAB; t++) {
    p->tn[t] = c->tab_n[t];
    for (int i = 0; i < c->tab_n[t]; i++) {
      p->tv[t][i] = (float)(c->tab_v[t][i] / vunit);
      p->txi[t][i] = c->tab_xi[t][i];
      p->tsl[t][i] = (float)(c->tab_slope[t][i] / vunit);
    }
  }
  p->k = k; p->q_s = q_s; p->m_s = m_s; p->lam = lam; p->dt = dt; p->vunit = vunit;
  p->n_inf = c->n_inf; p->T_e = c->T_e; p->T_n = c->T_n; p->k_B = c->k_B; p->m_e = c->m_e;
  p->e = c->e; p->E = c->E; p->v_T_si = c->v_T; p->v_fl_si = c->v_fl;
  p->n_steps = c->n_steps; p->avg_start = c->avg_start;
  tail_consts(p);
}

// Default all-pairs plan: packed f32x2 arithmetic on SoA tiles with one target per thread
// (variant 5, the fastest measured on GB300 from 2^16 to 2^20 ions), with enough source chunks
// for several waves on every SM.
// From 2^15 padded ions the default is variant 7 (each unordered pair once: 4 x 4 ions per lane
// with 1024-ion tiles up to 2^16 ions, then 8 x 2 with 2048-ion tiles); its sums go to 24 bytes of
// fixed-point accumulators per ion, so it always fits (the budget below only bounds the rule).
static constexpr size_t OD_N3_BUDGET = (size_t)32 << 30;
// The cutoff's tile-pair path (variant 3: 512-ion tiles with balanced group-pair lists) needs its
// sort, boxes, tile-pair list and slot accumulators (0.3 GB at 2^20 ions); the budget bounds the
// tile-pair list for very large N, beyond which 1024-ion tiles or the cell stencil take over.
static constexpr size_t OD_CUTN3_BUDGET = (size_t)64 << 30;
static bool uses_n3_default(int Npad) { return Npad >= 16384; }
static od_status set_plan_n3(od_handle* h, int ions_per_lane, int tile);

static od_pair_plan default_plan(int Npad, int sms) {
  od_pair_plan pl{};
  pl.nt = 256; pl.ipt = 1; pl.variant = 5;
  const int nbx = Npad / (pl.nt * pl.ipt);
  const int target = std::max(1, sms * 8 * 4);
  int js = std::max(1, (target + nbx - 1) / nbx);
  js = std::min(js, Npad / OD_TJ);
  int chunk = (Npad + js - 1) / js;
  chunk = ((chunk + OD_TJ - 1) / OD_TJ) * OD_TJ;
  pl.chunk = chunk;
  pl.jsplit = (Npad + chunk - 1) / chunk;
  return pl;
}

template <typename T>
static cudaError_t dalloc(T** p, size_t n) {
  return cudaMalloc((void**)p, sizeof(T) * std::max<size_t>(n, 1));
}

static void free_timing(od_handle* h) {
  for (cudaEvent_t e : h->ev_pool) cudaEventDestroy(e);
  h->ev_pool.clear();
  h->ev_step.clear();
  h->ev_pair.clear();
}

static void free_cutn3(od_handle* h);

static void free_all(od_handle* h) {
  free_cutn3(h);
  if (h->graph_exec) { cudaGraphExecDestroy(h->graph_exec); h->graph_exec = nullptr; }
  if (h->graph) { cudaGraphDestroy(h->graph); h->graph = nullptr; }
  if (h->graph_exec_nf) { cudaGraphExecDestroy(h->graph_exec_nf); h->graph_exec_nf = nullptr; }
  if (h->graph_nf) { cudaGraphDestroy(h->graph_nf); h->graph_nf = nullptr; }
  free_timing(h);
  void* ptrs[] = {h->dp, h->ds, h->b.pos, h->b.rel, h->b.vel, h->b.fhi, h->b.flo, h->b.part_hi, h->b.part_lo,
                  h->b.flags, h->b.list, h->b.list_bits, h->b.list_old, h->b.list_new, h->b.list_v,
                  h->b.orbit_part, h->b.s_q, h->b.s_orbit, h->b.s_collect, h->b.s_dust,
                  h->b.s_field, h->b.cq, h->snap_pos, h->snap_hi, h->snap_lo, h->snap_counts,
                  h->b.sx, h->b.sy, h->b.sz, h->cut.cell_of, h->cut.count, h->cut.fill,
                  h->cut.start, h->cut.chunk_prefix, h->cut.perm, h->cut.ox, h->cut.oy, h->cut.oz,
                  h->cut.stencil, h->d_pairs, h->cut.chunk_prefix2, h->b.n3, h->ssx, h->ssy,
                  h->ssz, h->g_idx, h->g_bits, h->g_old, h->g_new, h->g_v, h->g_orbit};
  for (void* p : ptrs)
    if (p) cudaFree(p);
}

static od_status alloc_scratch_for_plan(od_handle* h) {
  if (h->b.part_hi) { cudaFree(h->b.part_hi); h->b.part_hi = nullptr; }
  if (h->b.part_lo) { cudaFree(h->b.part_lo); h->b.part_lo = nullptr; }
  size_t n = (size_t)h->plan.jsplit * h->Npad;
  OD_CK(h, dalloc(&h->b.part_hi, n));
  OD_CK(h, dalloc(&h->b.part_lo, n));
  return OD_OK;
}

static od_status create_handle(const od_config* cfg, int32_t device, bool n3_default,
                               od_handle** out);
static od_status alloc_cutn3(od_handle* h, int ipt, int T);
static od_status ensure_acc(od_handle* h);

extern "C" od_status od_create(const od_config* cfg, int32_t device, od_handle** out) {
  return create_handle(cfg, device, true, out);
}

// n3_default = false: keep the directed-pair default plan (batch members, which the batched
// all-pairs kernel steps with their own plan).
static od_status create_handle(const od_config* cfg, int32_t device, bool n3_default,
                               od_handle** out) {
  if (!out) return fail(nullptr, OD_ERR_INVALID, "out is NULL");
  *out = nullptr;
  od_status st = validate(cfg);
  if (st != OD_OK) return st;
  if (od_device_count() <= device || device < 0)
    return fail(nullptr, OD_ERR_UNSUPPORTED, "no CUDA device with that index");
  od_handle* h = new (std::nothrow) od_handle();
  if (!h) return fail(nullptr, OD_ERR_OOM, "host allocation failed");
  h->device = device;
  h->cfg = *cfg;
  h->N = (int)cfg->n_ions;
  h->Npad = (int)(((cfg->n_ions + OD_PAD - 1) / OD_PAD) * OD_PAD);
  h->P = cfg->n_grains;
  h->nb = h->Npad / 256;
  auto bail = [&](od_status s) {
    g_err = h->err;
    free_all(h);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return s;
  };
#define OD_CKC(call)                                           \
  do {                                                         \
    cudaError_t e_ = (call);                                   \
    if (e_ != cudaSuccess) return bail(cuda_fail(h, e_, #call)); \
  } while (0)
  OD_CKC(cudaSetDevice(device));
  OD_CKC(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  fill_params(cfg, h->N, h->Npad, &h->hp);
  h->plan = default_plan(h->Npad, od_num_sms(device));
  const size_t Np = h->Npad, P = std::max(h->P, 1), ns = cfg->n_steps;
  OD_CKC(dalloc(&h->dp, 1));
  OD_CKC(dalloc(&h->ds, 1));
  OD_CKC(dalloc(&h->b.pos, Np));
  OD_CKC(dalloc(&h->b.rel, Np));
  OD_CKC(dalloc(&h->b.vel, Np));
  OD_CKC(dalloc(&h->b.fhi, Np));
  OD_CKC(dalloc(&h->b.flo, Np));
  OD_CKC(dalloc(&h->b.flags, Np / 32));
  OD_CKC(dalloc(&h->b.list, Np));
  OD_CKC(dalloc(&h->b.list_bits, Np));
  OD_CKC(dalloc(&h->b.list_old, Np));
  OD_CKC(dalloc(&h->b.list_new, Np));
  OD_CKC(dalloc(&h->b.list_v, Np));
  OD_CKC(dalloc(&h->b.orbit_part, (size_t)h->nb * P * 3));
  OD_CKC(dalloc(&h->b.s_q, ns * P));
  OD_CKC(dalloc(&h->b.s_orbit, ns * P * 3));
  OD_CKC(dalloc(&h->b.s_collect, ns * P * 3));
  OD_CKC(dalloc(&h->b.s_dust, ns * P * 3));
  OD_CKC(dalloc(&h->b.s_field, ns * P * 3));
  OD_CKC(dalloc(&h->b.cq, OD_MAX_GRAINS));
  OD_CKC(dalloc(&h->b.sx, Np));
  OD_CKC(dalloc(&h->b.sy, Np));
  OD_CKC(dalloc(&h->b.sz, Np));
  if (alloc_scratch_for_plan(h) != OD_OK) return bail(OD_ERR_OOM);
  if (cfg->force_method != OD_FORCE_CUTOFF && ensure_acc(h) != OD_OK) return bail(OD_ERR_OOM);
  int n3_ipt = 0, n3_tile = 0;
  if (n3_default && cfg->force_method != OD_FORCE_CUTOFF && uses_n3_default(h->Npad))
    n3_tile = od_n3_default(h->Npad, OD_N3_BUDGET, &n3_ipt);
  if (n3_tile && set_plan_n3(h, n3_ipt, n3_tile) != OD_OK) {
    // no each-pair-once shape for this size: stay on the directed-pair default
    cudaGetLastError();
    h->err.clear();
  }
  if (cfg->force_method == OD_FORCE_CUTOFF) {
    // Cells of side c = a power of two not above rc/4 (halved while the mean occupancy exceeds
    // ~800 ions), on a grid whose origin is a multiple of c: cell origins and the shifts between
    // cells are then exact in FP32, so a target moved into a neighbour cell's frame is rounded
    // once, to within half an ulp of 2c.
    const double rc = h->hp.rc, Rh = h->hp.Rh, Hh = h->hp.Hh;
    const double dens = cfg->n_ions / (OD_PI_D * Rh * Rh * Hh);
    double c = std::ldexp(1.0, (int)std::floor(std::log2(rc / 4.0)));
    while (dens * c * c * c > 800.0 && c > rc / 64.0) c *= 0.5;
    const int kk = (int)std::ceil(rc / c);
    od_cellgeom& g = h->cut.g;
    g.c = (float)c;
    g.inv_c = (float)(1.0 / c);
    const double mx = std::ceil(Rh / c + 1.0), mz = std::ceil(Hh / 2 / c + 1.0);
    g.lox = g.loy = (float)(-mx * c);
    g.loz = (float)(-mz * c);
    g.gx = g.gy = (int)(2 * mx);
    g.gz = (int)(2 * mz);
    g.ncells = g.gx * g.gy * g.gz;
    std::vector<int4> st;
    for (int dz = -kk - 1; dz <= kk + 1; dz++)
      for (int dy = -kk - 1; dy <= kk + 1; dy++)
        for (int dx = -kk - 1; dx <= kk + 1; dx++) {
          auto m = [&](int d) { double v = std::max(std::abs(d) - 1, 0) * c; return v * v; };
          if (m(dx) + m(dy) + m(dz) < rc * rc) st.push_back(make_int4(dx, dy, dz, 0));
        }
    h->cut.nstencil = (int)st.size();
    h->cut.cap = h->Npad + 8 * g.ncells;
    const size_t nc = g.ncells;
    OD_CKC(dalloc(&h->cut.cell_of, Np));
    OD_CKC(dalloc(&h->cut.count, nc));
    OD_CKC(dalloc(&h->cut.fill, nc));
    OD_CKC(dalloc(&h->cut.start, nc + 1));
    OD_CKC(dalloc(&h->cut.chunk_prefix, nc + 1));
    OD_CKC(dalloc(&h->cut.chunk_prefix2, nc + 1));
    h->cut.packed = true;
    OD_CKC(dalloc(&h->cut.perm, h->cut.cap));
    OD_CKC(dalloc(&h->cut.ox, h->cut.cap));
    OD_CKC(dalloc(&h->cut.oy, h->cut.cap));
    OD_CKC(dalloc(&h->cut.oz, h->cut.cap));
    OD_CKC(dalloc(&h->cut.stencil, st.size()));
    OD_CKC(dalloc(&h->d_pairs, 1));
    OD_CKC(cudaMemcpy(h->cut.stencil, st.data(), sizeof(int4) * st.size(), cudaMemcpyHostToDevice));
    OD_CKC(cudaMemset(h->d_pairs, 0, sizeof(unsigned long long)));
    h->has_cut = true;
    // default: tile pairs with each pair once (512-ion tiles, else 1024) when their memory
    // fits the budget; the cell-stencil kernel otherwise
    const int nc3 = od_cutn3_grid(h->N, h->hp.Rh, h->hp.Hh).ncells;
    const int cut_ipt = od_cutn3_bytes(h->N, 512, nc3) <= OD_CUTN3_BUDGET ? 2
                        : (od_cutn3_bytes(h->N, 1024, nc3) <= OD_CUTN3_BUDGET ? 4 : 0);
    if (cut_ipt && alloc_cutn3(h, cut_ipt, cut_ipt == 2 ? 512 : 1024) != OD_OK) {
      cudaGetLastError();
      h->err.clear();
    }
  }
  OD_CKC(cudaMemcpyAsync(h->dp, &h->hp, sizeof(od_dparams), cudaMemcpyHostToDevice, h->stream));
  od_dstate s0{};
  for (int g = 0; g < h->P; g++) s0.q_param[g] = cfg->grain_q0[g];
  OD_CKC(cudaMemcpyAsync(h->ds, &s0, sizeof(s0), cudaMemcpyHostToDevice, h->stream));
  // padded slots: far-away sources, zero velocity
  std::vector<float4> pad(Np, make_float4(OD_SENTINEL, OD_SENTINEL, OD_SENTINEL, 0.f));
  OD_CKC(cudaMemcpy(h->b.pos, pad.data(), sizeof(float4) * Np, cudaMemcpyHostToDevice));
  OD_CKC(cudaMemset(h->b.rel, 0, sizeof(float4) * Np));
  OD_CKC(od_launch_aos_to_soa(h->b.pos, h->Npad, h->b.sx, h->b.sy, h->b.sz, h->stream));
  OD_CKC(cudaMemset(h->b.vel, 0, sizeof(float4) * Np));
  OD_CKC(cudaMemset(h->b.fhi, 0, sizeof(float4) * Np));
  OD_CKC(cudaMemset(h->b.flo, 0, sizeof(float4) * Np));
  OD_CKC(cudaMemset(h->b.s_q, 0, sizeof(double) * ns * P));
  OD_CKC(cudaMemset(h->b.s_field, 0, sizeof(double) * ns * P * 3));
  OD_CKC(od_launch_set_charges(h->dp, h->ds, h->b.cq, h->P, h->stream));
  OD_CKC(cudaStreamSynchronize(h->stream));
#undef OD_CKC
  *out = h;
  return OD_OK;
}

extern "C" od_status od_destroy(od_handle* h) {
  if (!h) return OD_OK;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  free_all(h);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return OD_OK;
}

static void to_device_units(const od_handle* h, const double* pos, const double* vel, int64_t n,
                            std::vector<float4>& xp, std::vector<float4>* vp) {
  const double lam = h->hp.lam, vunit = h->hp.vunit;
  if (pos) {  // NULL: velocities only (the state's positions come from to_rel_state)
    xp.resize(n);
    for (int64_t i = 0; i < n; i++)
      xp[i] = make_float4((float)(pos[3 * i] / lam), (float)(pos[3 * i + 1] / lam),
                          (float)(pos[3 * i + 2] / lam), 0.f);
  }
  if (vp) {
    vp->resize(n);
    for (int64_t i = 0; i < n; i++)
      (*vp)[i] = make_float4((float)(vel[3 * i] / vunit), (float)(vel[3 * i + 1] / vunit),
                             (float)(vel[3 * i + 2] / vunit), 0.f);
  }
}

static od_status check_device_err(od_handle* h) {
  od_dstate s;
  OD_CK(h, cudaMemcpyAsync(&s, h->ds, sizeof(s), cudaMemcpyDeviceToHost, h->stream));
  OD_CK(h, cudaStreamSynchronize(h->stream));
  if (s.err & OD_DERR_TIMEOUT) return fail(h, OD_ERR_TIMEOUT, "a bounded device wait ran out");
  if (s.err & OD_DERR_CELL)
    return fail(h, OD_ERR_CAPACITY, "a cutoff cell holds more than 4096 ions (density too high)");
  if (s.err) return fail(h, OD_ERR_STATE, "device error word set");
  return OD_OK;
}

// ion–ion sums of the current positions into fhi/flo (the force the first half kick uses)
static od_status refresh_forces(od_handle* h) {
  const float rho0 = h->hp.rho0;
  OD_CK(h, od_launch_aos_to_soa(h->b.pos, h->Npad, h->b.sx, h->b.sy, h->b.sz, h->stream));
  (void)rho0;
  OD_CK(h, od_launch_force(force_ctx(h, false), od_pair_io{h->b.pos, h->b.sx, h->b.sy, h->b.sz, h->b.n3}, h->N,
                           h->Npad, h->b.part_hi, h->b.part_lo, &h->ds->err, h->stream));
  OD_CK(h, od_launch_reduce(h->dp, h->Npad, force_jsplit(h), h->b.part_hi, h->b.part_lo, h->b.fhi,
                            h->b.flo, h->stream));
  return OD_OK;
}

// Cell-relative state (od_common.cuh) of positions in metres, and the absolute FP32 positions
// that the device derives from it: per axis, c = floor(x / s) and the offset x - c s rounded
// once to FP32 (from the FP64 position, so nothing is lost to an FP32 absolute first).
static void to_rel_state(const od_handle* h, const double* pos, int64_t n,
                         std::vector<float4>& rel, std::vector<float4>& xp) {
  const double lam = h->hp.lam, s = h->hp.rel_s, inv = h->hp.rel_inv;
  rel.resize(n);
  xp.resize(n);
  for (int64_t i = 0; i < n; i++) {
    int c[3];
    float o[3], a[3];
    for (int d = 0; d < 3; d++) {
      const double v = pos[3 * i + d] / lam;
      c[d] = od_rel_clamp((int)std::max(std::min(std::floor(v * inv), 1e9), -1e9));
      o[d] = (float)(v - c[d] * s);
      if (o[d] == (float)s && c[d] < OD_REL_BIAS - 1) { c[d] += 1; o[d] = 0.f; }
      a[d] = (float)std::fma((double)c[d], s, (double)o[d]);  // exact, then rounded once
    }
    int key = od_rel_pack(c[0], c[1], c[2]);
    float w;
    memcpy(&w, &key, sizeof(w));
    rel[i] = make_float4(o[0], o[1], o[2], w);
    xp[i] = make_float4(a[0], a[1], a[2], 0.f);
  }
}

static bool all_finite(const double* a, int64_t n) {
  for (int64_t i = 0; i < n; i++)
    if (!std::isfinite(a[i])) return false;
  return true;
}

extern "C" od_status od_set_state(od_handle* h, const double* pos, const double* vel, int64_t n) {
  if (!h) return fail(nullptr, OD_ERR_INVALID, "handle is NULL");
  if (!pos || !vel) return fail(h, OD_ERR_INVALID, "pos/vel is NULL");
  if (n != h->N) return fail(h, OD_ERR_INVALID, "n must equal the configured n_ions");
  if (!all_finite(pos, 3 * n) || !all_finite(vel, 3 * n))
    return fail(h, OD_ERR_INVALID, "a position or velocity is not finite");
  OD_CK(h, cudaSetDevice(h->device));
  std::vector<float4> xp, vp, rel;
  to_device_units(h, nullptr, vel, n, xp, &vp);
  to_rel_state(h, pos, n, rel, xp);
  OD_CK(h, cudaMemcpyAsync(h->b.rel, rel.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, h->stream));
  OD_CK(h, cudaMemcpyAsync(h->b.pos, xp.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, h->stream));
  OD_CK(h, cudaMemcpyAsync(h->b.vel, vp.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, h->stream));
  od_status st = refresh_forces(h);
  if (st != OD_OK) return st;
  OD_CK(h, cudaStreamSynchronize(h->stream));
  h->state_set = true;
  return check_device_err(h);
}

extern "C" od_status od_init_state(od_handle* h, const double* vz_v, const double* vz_cdf,
                                   int32_t vz_n) {
  if (!h) return fail(nullptr, OD_ERR_INVALID, "handle is NULL");
  if (vz_n != 0 && (vz_n < 2 || !vz_v || !vz_cdf))
    return fail(h, OD_ERR_INVALID, "the v_z table needs at least 2 nodes");
  if (h->cfg.distribution == OD_DIST_FIELD_DRIVEN && vz_n < 2)
    return fail(h, OD_ERR_INVALID, "field-driven initial states need the v_z table");
  OD_CK(h, cudaSetDevice(h->device));
  float* d_v = nullptr;
  double* d_x = nullptr;
  if (vz_n >= 2) {
    std::vector<float> v(vz_n);
    for (int k = 0; k < vz_n; k++) v[k] = (float)(vz_v[k] / h->hp.vunit);
    OD_CK(h, cudaMalloc(&d_v, sizeof(float) * vz_n));
    OD_CK(h, cudaMalloc(&d_x, sizeof(double) * vz_n));
    OD_CK(h, cudaMemcpy(d_v, v.data(), sizeof(float) * vz_n, cudaMemcpyHostToDevice));
    OD_CK(h, cudaMemcpy(d_x, vz_cdf, sizeof(double) * vz_n, cudaMemcpyHostToDevice));
  }
  cudaError_t e = od_launch_init_state(h->dp, h->N, h->b.rel, h->b.pos, h->b.vel, d_v, d_x, vz_n,
                                       &h->ds->err, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (d_v) cudaFree(d_v);
  if (d_x) cudaFree(d_x);
  if (e != cudaSuccess) return cuda_fail(h, e, "od_init_state");
  od_status st = refresh_forces(h);
  if (st != OD_OK) return st;
  OD_CK(h, cudaStreamSynchronize(h->stream));
  h->state_set = true;
  st = check_device_err(h);
  if (st == OD_ERR_STATE) return fail(h, OD_ERR_STATE, "no position outside the grains was found");
  return st;
}

extern "C" od_status od_ion_potential_grid(od_handle* h, const double* gr, const double* gz,
                                           int32_t n_r, int32_t n_z, double* pot) {
  if (!h || !gr || !gz || !pot) return fail(h, OD_ERR_INVALID, "NULL argument");
  if (n_r < 1 || n_z < 1 || (int64_t)n_r * n_z > (1 << 20))
    return fail(h, OD_ERR_INVALID, "grid must have 1..2^20 points");
  if (!h->state_set) return fail(h, OD_ERR_STATE, "no ion state set");
  OD_CK(h, cudaSetDevice(h->device));
  const int npts = n_r * n_z;
  std::vector<double> pts((size_t)2 * npts);
  for (int j = 0; j < n_z; j++)
    for (int i = 0; i < n_r; i++) {
      pts[2 * ((size_t)j * n_r + i)] = gr[i];
      pts[2 * ((size_t)j * n_r + i) + 1] = gz[j];
    }
  double *d_pts = nullptr, *d_out = nullptr;
  OD_CK(h, cudaMalloc((void**)&d_pts, sizeof(double) * pts.size()));
  cudaError_t e = cudaMalloc((void**)&d_out, sizeof(double) * npts);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_pts, pts.data(), sizeof(double) * pts.size(), cudaMemcpyHostToDevice,
                        h->stream);
  if (e == cudaSuccess)
    e = od_launch_grid_potential(h->b.pos, h->N, d_pts, npts, h->cfg.r_0 / h->cfg.r_D_e, d_out,
                                 h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(pot, d_out, sizeof(double) * npts, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(d_pts);
  if (d_out) cudaFree(d_out);
  if (e != cudaSuccess) return cuda_fail(h, e, "od_ion_potential_grid");
  return OD_OK;
}

extern "C" od_status od_set_trap_table(od_handle* h, const double* trap_tab, int32_t n,
                                       const double* grain_out) {
  if (!h) return fail(nullptr, OD_ERR_INVALID, "handle is NULL");
  if (n != 0 && (n < 4 || n > OD_MAX_TRAP || !trap_tab))
    return fail(h, OD_ERR_INVALID, "a trap table needs 4..OD_MAX_TRAP knots");
  OD_CK(h, cudaSetDevice(h->device));
  const double lam = h->cfg.r_D_e, dt = h->cfg.d_t;
  const double k = 1.0 / (h->cfg.eps_0 * 4.0 * OD_PI_D);
  const double q_s = fabs(h->cfg.e) * h->cfg.N_s, m_s = h->cfg.m_i * h->cfg.N_s;
  const double A_ii = k * q_s * q_s * dt * dt / (m_s * lam * lam * lam);
  fill_trap_table(&h->hp, trap_tab, n, h->cfg.H / lam, A_ii);
  for (int g = 0; g < h->P; g++)
    for (int d = 0; d < 3; d++) h->hp.gout[g][d] = grain_out ? grain_out[3 * g + d] : 0.0;
  tail_consts(&h->hp);
  h->cfg.trap_kind = h->hp.trap_kind;
  h->cfg.trap_n = n;
  OD_CK(h, cudaMemcpyAsync(h->dp, &h->hp, sizeof(od_dparams), cudaMemcpyHostToDevice, h->stream));
  OD_CK(h, cudaStreamSynchronize(h->stream));
  return OD_OK;
}

extern "C" od_status od_set_grains(od_handle* h, const double* x, const double* y,
                                   const double* z, const double* q, const double* grain_field,
                                   const double* grain_out) {
  if (!h) return fail(nullptr, OD_ERR_INVALID, "handle is NULL");
  if (h->P > 0 && (!x || !y || !z || !q)) return fail(h, OD_ERR_INVALID, "NULL argument");
  OD_CK(h, cudaSetDevice(h->device));
  const double lam = h->cfg.r_D_e;
  od_dparams& p = h->hp;
  for (int g = 0; g < h->P; g++) {
    const double gx = x[g] / lam, gy = y[g] / lam, gz = z[g] / lam;
    p.gx[g] = gx; p.gy[g] = gy; p.gz[g] = gz;
    split2(gx, p.gxh[g], p.gxl[g]);
    split2(gy, p.gyh[g], p.gyl[g]);
    split2(gz, p.gzh[g], p.gzl[g]);
    p.gxs[g] = x[g]; p.gys[g] = y[g]; p.gzs[g] = z[g];
    if (grain_field) p.gfield[g] = grain_field[g];
    if (grain_out)
      for (int d = 0; d < 3; d++) p.gout[g][d] = grain_out[3 * g + d];
  }
  tail_consts(&p);
  OD_CK(h, cudaMemcpyAsync(h->dp, &h->hp, sizeof(od_dparams), cudaMemcpyHostToDevice, h->stream));
  OD_CK(h, cudaMemcpyAsync(reinterpret_cast<char*>(h->ds) + offsetof(od_dstate, q_param), q,
                           sizeof(double) * h->P, cudaMemcpyHostToDevice, h->stream));
  OD_CK(h, od_launch_set_charges(h->dp, h->ds, h->b.cq, h->P, h->stream));
  OD_CK(h, cudaStreamSynchronize(h->stream));
  return OD_OK;
}

extern "C" od_status od_begin_window(od_handle* h) {
  if (!h) return fail(nullptr, OD_ERR_INVALID, "handle is NULL");
  OD_CK(h, cudaSetDevice(h->device));
  od_dstate s;
  OD_CK(h, cudaMemcpyAsync(&s, h->ds, sizeof(s), cudaMemcpyDeviceToHost, h->stream));
  OD_CK(h, cudaStreamSynchronize(h->stream));
  s.rng_base += s.step;
  s.step = 0;
  memset(s.avg, 0, sizeof(s.avg));
  s.n_avg = 0;
  OD_CK(h, cudaMemcpyAsync(h->ds, &s, sizeof(s), cudaMemcpyHostToDevice, h->stream));
  OD_CK(h, cudaStreamSynchronize(h->stream));
  h->step = 0;
  return OD_OK;
}

extern "C" od_status od_get_state(od_handle* h, double* pos, double* vel, int64_t n) {
  if (!h) return fail(nullptr, OD_ERR_INVALID, "handle is NULL");
  if (n != h->N) return fail(h, OD_ERR_INVALID, "n must equal the configured n_ions");
  OD_CK(h, cudaSetDevice(h->device));
  std::vector<float4> rp(n), vp(n);
  OD_CK(h, cudaMemcpyAsync(rp.data(), h->b.rel, sizeof(float4) * n, cudaMemcpyDeviceToHost, h->stream));
  OD_CK(h, cudaMemcpyAsync(vp.data(), h->b.vel, sizeof(float4) * n, cudaMemcpyDeviceToHost, h->stream));
  OD_CK(h, cudaStreamSynchronize(h->stream));
  const double lam = h->hp.lam, vunit = h->hp.vunit, s = h->hp.rel_s;
  for (int64_t i = 0; i < n; i++) {
    if (pos) {  // the cell-relative state, exactly (c s + offset is exact in FP64)
      int key;
      memcpy(&key, &rp[i].w, sizeof(key));
      const double c[3] = {(double)((key & 1023) - OD_REL_BIAS), (double)(((key >> 10) & 1023) - OD_REL_BIAS),
                           (double)(((key >> 20) & 1023) - OD_REL_BIAS)};
      pos[3 * i] = (c[0] * s + rp[i].x) * lam;
      pos[3 * i + 1] = (c[1] * s + rp[i].y) * lam;
      pos[3 * i + 2] = (c[2] * s + rp[i].z) * lam;
    }
    if (vel) { vel[3 * i] = vp[i].x * vunit; vel[3 * i + 1] = vp[i].y * vunit; vel[3 * i + 2] = vp[i].z * vunit; }
  }
  return OD_OK;
}

// Does step `step` evaluate the ion–ion force (force interval k = cfg.force_every)?
static bool step_evaluates(const od_handle* h, int64_t step) {
  const int k = h->cfg.force_every;
  return k <= 1 || step % k == k - 1;
}

static od_status event_at(od_handle* h, size_t slot, int* idx) {
  while (h->ev_pool.size() <= slot) {
    cudaEvent_t e;
    OD_CK(h, cudaEventCreate(&e));
    h->ev_pool.push_back(e);
  }
  *idx = (int)slot;
  return OD_OK;
}

// Steps launched one kernel at a time with CUDA events around every step and every all-pairs
// launch (timing mode).
static od_status step_timed(od_handle* h, int64_t nsteps) {
  size_t slot = 0;
  const od_force_ctx fc = force_ctx(h, h->count_pairs);
  h->ev_step.clear();
  h->ev_pair.clear();
  for (int64_t s = 0; s < nsteps; s++) {
    int a, b, c, d;
    if (event_at(h, slot++, &a) || event_at(h, slot++, &b) || event_at(h, slot++, &c) ||
        event_at(h, slot++, &d))
      return OD_ERR_CUDA;
    OD_CK(h, cudaEventRecord(h->ev_pool[a], h->stream));
    const int nb = h->Npad / 256;
    const bool eval = step_evaluates(h, h->step + s);
    OD_CK(h, od_launch_step_part(0, h->dp, h->ds, h->b, h->N, h->Npad, h->P, fc, h->nrec,
                                 h->stream));
    OD_CK(h, cudaEventRecord(h->ev_pool[c], h->stream));
    if (eval)
      OD_CK(h, od_launch_step_part(1, h->dp, h->ds, h->b, h->N, h->Npad, h->P, fc, h->nrec,
                                   h->stream));
    OD_CK(h, cudaEventRecord(h->ev_pool[d], h->stream));
    OD_CK(h, od_launch_step_part(2, h->dp, h->ds, h->b, h->N, h->Npad, h->P, fc, h->nrec,
                                 h->stream));
    OD_CK(h, cudaEventRecord(h->ev_pool[b], h->stream));
    (void)nb;
    h->ev_step.push_back({a, b});
    if (eval) h->ev_pair.push_back({c, d});
  }
  OD_CK(h, cudaStreamSynchronize(h->stream));
  for (auto& p : h->ev_step) {
    float ms;
    OD_CK(h, cudaEventElapsedTime(&ms, h->ev_pool[p.first], h->ev_pool[p.second]));
    h->t_step_ms += ms;
    h->t_steps++;
  }
  for (auto& p : h->ev_pair) {
    float ms;
    OD_CK(h, cudaEventElapsedTime(&ms, h->ev_pool[p.first], h->ev_pool[p.second]));
    h->t_pair_ms += ms;
    h->t_pair_launches++;
  }
  return OD_OK;
}

// One step's launches; `with_force` false leaves out the ion–ion launch (part 1).
static cudaError_t launch_step_parts(od_handle* h, const od_force_ctx& fc, bool with_force) {
  for (int part = 0; part < 3; part++) {
    if (part == 1 && !with_force) continue;
    cudaError_t e = od_launch_step_part(part, h->dp, h->ds, h->b, h->N, h->Npad, h->P, fc, h->nrec,
                                        h->stream);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

static od_status capture_step(od_handle* h, bool with_force, cudaGraph_t* graph,
                              cudaGraphExec_t* exec) {
  if (*exec) return OD_OK;
  OD_CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = launch_step_parts(h, force_ctx(h, false), with_force);
  cudaGraph_t g = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(h->stream, &g);
  if (e != cudaSuccess) { if (g) cudaGraphDestroy(g); return cuda_fail(h, e, "step capture"); }
  if (e2 != cudaSuccess) return cuda_fail(h, e2, "cudaStreamEndCapture");
  *graph = g;
  OD_CK(h, cudaGraphInstantiate(exec, g, 0));
  return OD_OK;
}

static od_status ensure_graph(od_handle* h) {
  od_status st = capture_step(h, true, &h->graph, &h->graph_exec);
  if (st != OD_OK || h->cfg.force_every <= 1) return st;
  return capture_step(h, false, &h->graph_nf, &h->graph_exec_nf);
}

extern "C" od_status od_step(od_handle* h, int64_t nsteps) {
  if (!h) return fail(nullptr, OD_ERR_INVALID, "handle is NULL");
  if (!h->state_set) return fail(h, OD_ERR_STATE, "od_set_state has not been called");
  if (nsteps < 0) return fail(h, OD_ERR_INVALID, "nsteps < 0");
  if (h->step + nsteps > h->cfg.n_steps)
    return fail(h, OD_ERR_STATE, "the result series is full (n_steps reached)");
  OD_CK(h, cudaSetDevice(h->device));
  if (h->timing) {
    od_status st = step_timed(h, nsteps);
    if (st != OD_OK) return st;
  } else if (h->use_graph) {
    od_status st = ensure_graph(h);
    if (st != OD_OK) return st;
    for (int64_t s = 0; s < nsteps; s++)
      OD_CK(h, cudaGraphLaunch(step_evaluates(h, h->step + s) ? h->graph_exec : h->graph_exec_nf,
                               h->stream));
  } else {
    for (int64_t s = 0; s < nsteps; s++)
      OD_CK(h, launch_step_parts(h, force_ctx(h, false), step_evaluates(h, h->step + s)));
  }
  h->step += nsteps;
  return check_device_err(h);
}

extern "C" od_status od_set_timing(od_handle* h, int32_t enable) {
  if (!h) return fail(nullptr, OD_ERR_INVALID, "handle is NULL");
  if (enable < 0 || enable > 2) return fail(h, OD_ERR_INVALID, "timing mode must be 0, 1 or 2");
  h->timing = enable != 0;
  h->count_pairs = enable == 1;
  h->t_step_ms = h->t_pair_ms = 0;
  h->t_steps = h->t_pair_launches = 0;
  if (h->d_pairs) OD_CK(h, cudaMemsetAsync(h->d_pairs, 0, sizeof(unsigned long long), h->stream));
  return OD_OK;
}

extern "C" od_status od_get_cutoff_pairs(od_handle* h, int64_t* pairs) {
  if (!h || !pairs) return fail(h, OD_ERR_INVALID, "NULL argument");
  unsigned long long v = 0;
  if (h->d_pairs) {
    OD_CK(h, cudaMemcpyAsync(&v, h->d_pairs, sizeof(v), cudaMemcpyDeviceToHost, h->stream));
    OD_CK(h, cudaStreamSynchronize(h->stream));
  }
  *pairs = (int64_t)v;
  return OD_OK;
}

extern "C" od_status od_get_timing(od_handle* h, double* step_ms, int64_t* steps, double* pair_ms,
                                   int64_t* pair_launches) {
  if (!h) return fail(nullptr, OD_ERR_INVALID, "handle is NULL");
  if (step_ms) *step_ms = h->t_step_ms;
  if (steps) *steps = h->t_steps;
  if (pair_ms) *pair_ms = h->t_pair_ms;
  if (pair_launches) *pair_launches = h->t_pair_launches;
  return OD_OK;
}

extern "C" od_status od_set_graph(od_handle* h, int32_t enable) {
  if (!h) return fail(nullptr, OD_ERR_INVALID, "handle is NULL");
  h->use_graph = enable != 0;
  return OD_OK;
}

static bool plan_supported(int nt, int ipt, int variant) {
  const int key = nt * 100 + ipt * 10 + variant;
  switch (key) {
    case 12810: case 12820: case 25610: case 25620: case 12811: case 25611: case 25621:
    case 12822: case 25622: case 12823: case 25623: case 12824: case 25624:
    case 12815: case 25615: case 12816: case 25616:
    case 25627: case 25647: case 25687:  // each unordered pair once
      return true;
    default:
      return false;
  }
}

static void free_cutn3(od_handle* h) {
  od_cutn3* L = h->cut.n3;
  if (!L) return;
  void* ptrs[] = {L->cell_of, L->count, L->fill, L->start, L->perm, L->xs, L->ys, L->zs,
                  L->box, L->gbox, L->adj, L->rowptr, L->pairs, L->acc};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete L;
  h->cut.n3 = nullptr;
}

// Cutoff variant 3: Hilbert-sorted tiles of T ions (ipt 4: 1024, ipt 2: 512) and the per-slot
// fixed-point accumulators (24 bytes per slot).
static od_status alloc_cutn3(od_handle* h, int ipt, int T) {
  free_cutn3(h);
  OD_CK(h, cudaSetDevice(h->device));
  OD_CK(h, od_cutn3_prepare(ipt, T));
  od_cutn3* L = new (std::nothrow) od_cutn3();
  if (!L) return fail(h, OD_ERR_OOM, "host allocation");
  h->cut.n3 = L;
  const int N = h->N;
  const od_cgrid g = od_cutn3_grid(N, h->hp.Rh, h->hp.Hh);
  const int G = g.G;
  L->G = G;
  L->bits = 0;
  while ((1 << L->bits) < G) L->bits++;
  L->nb = g.nb;
  L->ncells = g.ncells;
  L->lo = (float)(-g.side / 2.0);
  L->lo_z = (float)(-g.side * g.nb / 2.0);
  L->inv_s = (float)(G / g.side);
  L->T = T; L->ipt = ipt;
  L->rc_d = h->cfg.cutoff / h->cfg.r_D_e;
  L->nT = (N + T - 1) / T;
  L->nslots = L->nT * T;
  L->nwords = (L->nT + 31) / 32;
  L->grid = od_num_sms(h->device) * od_cutn3_blocks_per_sm(ipt, T, false);
  L->grid_hard = od_num_sms(h->device) * od_cutn3_blocks_per_sm(ipt, T, true);
  const size_t nT = L->nT, ns = L->nslots, nc = L->ncells;
  auto al = [&](auto** p, size_t n) {
    return cudaMalloc((void**)p, sizeof(**p) * std::max<size_t>(n, 1));
  };
  cudaError_t e = al(&L->cell_of, (size_t)N);
  if (e == cudaSuccess) e = al(&L->count, nc);
  if (e == cudaSuccess) e = al(&L->fill, nc);
  if (e == cudaSuccess) e = al(&L->start, nc + 1);
  if (e == cudaSuccess) e = al(&L->perm, ns);
  if (e == cudaSuccess) e = al(&L->xs, ns);
  if (e == cudaSuccess) e = al(&L->ys, ns);
  if (e == cudaSuccess) e = al(&L->zs, ns);
  if (e == cudaSuccess) e = al(&L->box, nT * 6);
  if (e == cudaSuccess) e = al(&L->gbox, (ns / 64) * 6);
  if (e == cudaSuccess) e = al(&L->adj, nT * L->nwords);
  if (e == cudaSuccess) e = al(&L->rowptr, nT + 1);
  if (e == cudaSuccess) e = al(&L->pairs, nT * (nT + 1) / 2);
  if (e == cudaSuccess) e = al(&L->acc, 3 * ns);
  if (e == cudaSuccess) e = cudaMemset(L->acc, 0, sizeof(unsigned long long) * 3 * ns);
  if (e != cudaSuccess) {
    cudaGetLastError();
    free_cutn3(h);
    return fail(h, OD_ERR_OOM, "no device memory for the tile-pair cutoff");
  }
  // tail slots: far-away sentinels that no ion owns
  if (ns > (size_t)N) {
    std::vector<float> sent(ns - N, OD_SENTINEL);
    std::vector<int32_t> none(ns - N, -1);
    OD_CK(h, cudaMemcpy(L->xs + N, sent.data(), sizeof(float) * (ns - N), cudaMemcpyHostToDevice));
    OD_CK(h, cudaMemcpy(L->ys + N, sent.data(), sizeof(float) * (ns - N), cudaMemcpyHostToDevice));
    OD_CK(h, cudaMemcpy(L->zs + N, sent.data(), sizeof(float) * (ns - N), cudaMemcpyHostToDevice));
    OD_CK(h, cudaMemcpy(L->perm + N, none.data(), sizeof(int32_t) * (ns - N),
                        cudaMemcpyHostToDevice));
  }
  return OD_OK;
}

static void drop_graph(od_handle* h) {
  if (h->graph_exec) { cudaGraphExecDestroy(h->graph_exec); h->graph_exec = nullptr; }
  if (h->graph) { cudaGraphDestroy(h->graph); h->graph = nullptr; }
  if (h->graph_exec_nf) { cudaGraphExecDestroy(h->graph_exec_nf); h->graph_exec_nf = nullptr; }
  if (h->graph_nf) { cudaGraphDestroy(h->graph_nf); h->graph_nf = nullptr; }
}

static void free_n3(od_handle* h) {
  if (h->b.n3) { cudaFree(h->b.n3); h->b.n3 = nullptr; }
  h->b.n3_len = 0;
}

// The fixed-point ion–ion accumulators (three 64-bit words per ion, zero between evaluations).
static od_status ensure_acc(od_handle* h) {
  const size_t need = od_n3_floats(h->Npad, 1);  // in units of 4 bytes
  if (h->b.n3 && h->b.n3_len >= need) return OD_OK;
  free_n3(h);
  if (cudaMalloc((void**)&h->b.n3, sizeof(float) * need) != cudaSuccess) {
    cudaGetLastError();
    h->b.n3 = nullptr;
    return fail(h, OD_ERR_OOM, "no device memory for the ion–ion accumulators");
  }
  h->b.n3_len = need;
  OD_CK(h, cudaMemset(h->b.n3, 0, sizeof(float) * need));
  return OD_OK;
}

// Variant 7: `ions_per_lane` targets per lane (2 or 4 with as many sources, 8 with two sources),
// `tile` ions per tile (1024, 2048, 4096; <= 0: 1024 up to 2^17 ions, else 2048). The pair
// sums go to three 64-bit fixed-point accumulators per ion (24 bytes per ion: 25 MB at 2^20).
static od_status set_plan_n3(od_handle* h, int ions_per_lane, int tile) {
  if (!plan_supported(256, ions_per_lane, 7))
    return fail(h, OD_ERR_INVALID, "variant 7 takes 2, 4 or 8 targets per lane");
  if (tile <= 0) {
    for (int T = h->Npad <= (1 << 17) ? 1024 : 2048; T <= 4096 && tile <= 0; T <<= 1)
      if (od_n3_supported(ions_per_lane, T) &&
          sizeof(float) * od_n3_floats(h->Npad, T) <= OD_N3_BUDGET)
        tile = T;
    if (tile <= 0) return fail(h, OD_ERR_OOM, "variant 7 needs more than its memory budget here");
  }
  if (!od_n3_supported(ions_per_lane, tile))
    return fail(h, OD_ERR_INVALID,
                "variant 7 tiles hold 1024, 2048 or 4096 ions (2048 or 4096 with 8 per lane)");
  OD_CK(h, cudaSetDevice(h->device));
  od_pair_plan pl{};
  pl.nt = 256; pl.ipt = ions_per_lane; pl.variant = 7; pl.tile = tile;
  pl.jsplit = 1; pl.chunk = h->Npad;
  OD_CK(h, od_n3_prepare(pl));
  const size_t need = od_n3_floats(h->Npad, tile);
  if (h->b.n3_len < need) {
    free_n3(h);
    if (cudaMalloc((void**)&h->b.n3, sizeof(float) * need) != cudaSuccess) {
      cudaGetLastError();
      h->b.n3 = nullptr;
      return fail(h, OD_ERR_OOM, "no device memory for the variant-7 accumulators");
    }
    h->b.n3_len = need;
    // the accumulators start at zero; every evaluation clears them after reading them
    OD_CK(h, cudaMemset(h->b.n3, 0, sizeof(float) * need));
  }
  h->plan = pl;  // one partial slab: part_hi/part_lo always hold at least one
  drop_graph(h);
  return OD_OK;
}

extern "C" od_status od_set_pair_plan(od_handle* h, int32_t threads, int32_t targets_per_thread,
                                      int32_t variant, int32_t jsplit) {
  if (!h) return fail(nullptr, OD_ERR_INVALID, "handle is NULL");
  if (h->has_cut) {
    // cutoff method: variant 0 selects the scalar pair kernel, 2 the packed one, 3 the tile
    // pairs with each pair once (targets_per_thread 2: 512-ion tiles, 4: 1024-ion tiles; a
    // positive jsplit must name that tile size)
    if (variant != 0 && variant != 2 && variant != 3)
      return fail(h, OD_ERR_INVALID, "cutoff variants are 0, 2 and 3");
    if (variant == 3) {
      const int T = jsplit > 0 ? jsplit : (targets_per_thread == 4 ? 1024 : 512);
      if (!od_cutn3_supported(targets_per_thread, T))
        return fail(h, OD_ERR_INVALID,
                    "cutoff variant 3 takes (2, 512) or (4, 1024) as (targets per lane, tile)");
      if (!h->cut.n3 || h->cut.n3->T != T || h->cut.n3->ipt != targets_per_thread) {
        od_status st = alloc_cutn3(h, targets_per_thread, T);
        if (st != OD_OK) return st;
      }
    } else {
      free_cutn3(h);
    }
    h->cut.packed = variant == 2;
    if (h->graph_exec) { cudaGraphExecDestroy(h->graph_exec); h->graph_exec = nullptr; }
    if (h->graph) { cudaGraphDestroy(h->graph); h->graph = nullptr; }
    if (h->graph_exec_nf) { cudaGraphExecDestroy(h->graph_exec_nf); h->graph_exec_nf = nullptr; }
    if (h->graph_nf) { cudaGraphDestroy(h->graph_nf); h->graph_nf = nullptr; }
    return OD_OK;
  }
  if (!plan_supported(threads, targets_per_thread, variant))
    return fail(h, OD_ERR_INVALID, "unsupported (threads, targets_per_thread, variant)");
  if (variant == 7) return set_plan_n3(h, targets_per_thread, jsplit);
  if (h->Npad % (threads * targets_per_thread) != 0)
    return fail(h, OD_ERR_INVALID, "block does not divide the padded ion count");
  if (variant >= 2) {
    od_status st = ensure_acc(h);
    if (st != OD_OK) return st;
  }
  od_pair_plan pl{};
  pl.nt = threads; pl.ipt = targets_per_thread; pl.variant = variant;
  if (jsplit <= 0) {
    pl = default_plan(h->Npad, od_num_sms(h->device));
    pl.nt = threads; pl.ipt = targets_per_thread; pl.variant = variant;
    const int nbx = h->Npad / (threads * targets_per_thread);
    jsplit = std::max(1, (od_num_sms(h->device) * 8 * 4 + nbx - 1) / nbx);
  }
  jsplit = std::min(jsplit, h->Npad / OD_TJ);
  int chunk = (h->Npad + jsplit - 1) / jsplit;
  chunk = ((chunk + OD_TJ - 1) / OD_TJ) * OD_TJ;
  pl.chunk = chunk;
  pl.jsplit = (h->Npad + chunk - 1) / chunk;
  const bool grow = pl.jsplit > h->plan.jsplit;
  h->plan = pl;
  if (grow && alloc_scratch_for_plan(h) != OD_OK) return OD_ERR_OOM;
  if (h->graph_exec) { cudaGraphExecDestroy(h->graph_exec); h->graph_exec = nullptr; }
  if (h->graph) { cudaGraphDestroy(h->graph); h->graph = nullptr; }
  if (h->graph_exec_nf) { cudaGraphExecDestroy(h->graph_exec_nf); h->graph_exec_nf = nullptr; }
  if (h->graph_nf) { cudaGraphDestroy(h->graph_nf); h->graph_nf = nullptr; }
  return OD_OK;
}

// Autotuner: times each supported (threads, targets per thread, variant) with the default split
// and with half and twice as many source chunks, on the handle's current positions, over the
// first target blocks only (enough for several waves), and keeps the fastest plan. Results are
// cached per (device, padded ion count) for the process.
#include <map>
static std::mutex g_tune_mu;
static std::map<std::pair<int, int>, od_pair_plan> g_tuned;

extern "C" od_status od_autotune(od_handle* h, int32_t use_cache, double* best_pairs_per_s) {
  if (!h) return fail(nullptr, OD_ERR_INVALID, "handle is NULL");
  if (h->has_cut) return fail(h, OD_ERR_UNSUPPORTED, "the autotuner covers the all-pairs method");
  OD_CK(h, cudaSetDevice(h->device));
  const auto key = std::make_pair(h->device, h->Npad);
  if (use_cache) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) {
      const od_pair_plan& p = it->second;
      if (best_pairs_per_s) *best_pairs_per_s = 0;
      return od_set_pair_plan(h, p.nt, p.ipt, p.variant, p.variant == 7 ? p.tile : p.jsplit);
    }
  }
  OD_CK(h, od_launch_aos_to_soa(h->b.pos, h->Npad, h->b.sx, h->b.sy, h->b.sz, h->stream));
  const int shapes[][3] = {{256, 1, 0}, {128, 1, 0}, {256, 1, 1}, {128, 2, 2}, {256, 2, 2},
                           {128, 2, 3}, {256, 2, 3}, {128, 2, 4}, {256, 2, 4},
                           {128, 1, 5}, {256, 1, 5}, {128, 1, 6}, {256, 1, 6},
                           {256, 2, 7}, {256, 4, 7}, {256, 8, 7}};
  const int sms = od_num_sms(h->device);
  cudaEvent_t e0, e1;
  OD_CK(h, cudaEventCreate(&e0));
  OD_CK(h, cudaEventCreate(&e1));
  double best = -1;
  od_pair_plan best_plan = h->plan;
  for (const auto& sh : shapes) {
    if (sh[2] == 7) {
      // each unordered pair once: timed over a full launch with the default tile, and only
      // (the pair rate counts directed pairs, as for the others)
      if (h->Npad < 8192 || od_set_pair_plan(h, sh[0], sh[1], 7, 0) != OD_OK) {
        cudaGetLastError();
        continue;
      }
      const od_pair_io io{h->b.pos, h->b.sx, h->b.sy, h->b.sz, h->b.n3};
      OD_CK(h, od_launch_pairs(h->plan, io, h->Npad, h->b.part_hi, h->b.part_lo, h->hp.rho0,
                               &h->ds->err, h->stream));
      OD_CK(h, cudaEventRecord(e0, h->stream));
      for (int r = 0; r < 2; r++)
        OD_CK(h, od_launch_pairs(h->plan, io, h->Npad, h->b.part_hi, h->b.part_lo, h->hp.rho0,
                                 &h->ds->err, h->stream));
      OD_CK(h, cudaEventRecord(e1, h->stream));
      OD_CK(h, cudaEventSynchronize(e1));
      float ms = 0;
      OD_CK(h, cudaEventElapsedTime(&ms, e0, e1));
      const double rate = 2.0 * (double)h->Npad * h->Npad / (ms * 1e-3);
      if (rate > best) { best = rate; best_plan = h->plan; }
      continue;
    }
    const int nbx = h->Npad / (sh[0] * sh[1]);
    const int js0 = std::max(1, (sms * 8 * 4 + nbx - 1) / nbx);
    for (int mult = 0; mult < 3; mult++) {
      const int js = mult == 0 ? js0 : (mult == 1 ? std::max(1, js0 / 2) : js0 * 2);
      if (od_set_pair_plan(h, sh[0], sh[1], sh[2], js) != OD_OK) continue;
      const od_pair_plan& pl = h->plan;
      // enough target blocks for ~8 waves of the source split, at most the full grid
      const int limit = std::min(nbx, std::max(1, (sms * 32 + pl.jsplit - 1) / pl.jsplit));
      const od_pair_io io{h->b.pos, h->b.sx, h->b.sy, h->b.sz, h->b.n3};
      OD_CK(h, od_launch_pairs_probe(pl, io, h->Npad, limit, h->b.part_hi, h->b.part_lo, h->hp.rho0,
                                     &h->ds->err, h->stream));
      OD_CK(h, cudaEventRecord(e0, h->stream));
      for (int r = 0; r < 2; r++)
        OD_CK(h, od_launch_pairs_probe(pl, io, h->Npad, limit, h->b.part_hi, h->b.part_lo,
                                       h->hp.rho0, &h->ds->err, h->stream));
      OD_CK(h, cudaEventRecord(e1, h->stream));
      OD_CK(h, cudaEventSynchronize(e1));
      float ms = 0;
      OD_CK(h, cudaEventElapsedTime(&ms, e0, e1));
      const double pairs = 2.0 * limit * (double)(sh[0] * sh[1]) * h->Npad;
      const double rate = pairs / (ms * 1e-3);
      if (rate > best) { best = rate; best_plan = pl; }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  od_status st = od_set_pair_plan(h, best_plan.nt, best_plan.ipt, best_plan.variant,
                                  best_plan.variant == 7 ? best_plan.tile : best_plan.jsplit);
  if (st != OD_OK) return st;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[key] = h->plan;
  }
  if (best_pairs_per_s) *best_pairs_per_s = best;
  // the probes overwrote the partial slabs: restore the ion–ion sums of the current state
  if (h->state_set) return refresh_forces(h);
  return OD_OK;
}

extern "C" od_status od_get_pair_plan(const od_handle* h, int32_t* plan5) {
  if (!h || !plan5) return fail(nullptr, OD_ERR_INVALID, "NULL argument");
  if (h->has_cut) {  // cutoff variant: 3 (tile pairs), 2 (packed cells) or 0 (scalar cells)
    plan5[0] = 256;
    plan5[1] = h->cut.n3 ? h->cut.n3->ipt : 2;
    plan5[2] = h->cut.n3 ? 3 : (h->cut.packed ? 2 : 0);
    plan5[3] = h->cut.n3 ? h->cut.n3->T : 0;
    plan5[4] = 0;
    return OD_OK;
  }
  plan5[0] = h->plan.nt; plan5[1] = h->plan.ipt; plan5[2] = h->plan.variant;
  plan5[3] = h->plan.variant == 7 ? h->plan.tile : h->plan.jsplit; plan5[4] = h->plan.chunk;
  return OD_OK;
}

extern "C" od_status od_probe_fp32_peak(int32_t device, double* tflops) {
  if (!tflops) return fail(nullptr, OD_ERR_INVALID, "tflops is NULL");
  if (od_device_count() <= device || device < 0)
    return fail(nullptr, OD_ERR_UNSUPPORTED, "no CUDA device with that index");
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = od_run_fp32_probe(device, tflops);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "fp32 probe");
  return OD_OK;
}

extern "C" od_status od_selftest_wait(int32_t device, uint32_t limit, int32_t arrive) {
  if (od_device_count() <= device || device < 0)
    return fail(nullptr, OD_ERR_UNSUPPORTED, "no CUDA device with that index");
  if (limit < 1 || limit > OD_WAIT_LIMIT)
    return fail(nullptr, OD_ERR_INVALID, "limit must be 1 to 2^26 polls");
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaSetDevice");
  uint32_t* d_err = nullptr;
  e = cudaMalloc(&d_err, sizeof(uint32_t));
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaMalloc(error word)");
  uint32_t err = 0;
  e = cudaMemset(d_err, 0, sizeof(uint32_t));
  if (e == cudaSuccess) e = od_launch_wait_selftest(d_err, limit, arrive ? 1 : 0, nullptr);
  if (e == cudaSuccess) e = cudaMemcpy(&err, d_err, sizeof(err), cudaMemcpyDeviceToHost);
  cudaFree(d_err);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "wait self test");
  if (err & OD_DERR_TIMEOUT) return fail(nullptr, OD_ERR_TIMEOUT, "a bounded device wait ran out");
  return OD_OK;
}

extern "C" int64_t od_step_index(const od_handle* h) { return h ? h->step : -1; }

extern "C" od_status od_get_series(od_handle* h, int64_t first, int64_t count, double* q,
                                   double* f_orbit, double* f_collect, double* f_dust,
                                   double* f_field) {
  if (!h) return fail(nullptr, OD_ERR_INVALID, "handle is NULL");
  if (first < 0 || count < 0 || first + count > h->step)
    return fail(h, OD_ERR_INVALID, "requested steps have not been taken");
  if (count == 0) return OD_OK;
  OD_CK(h, cudaSetDevice(h->device));
  const size_t P = h->P;
  const size_t o1 = first * P, n1 = count * P;
  if (q) OD_CK(h, cudaMemcpyAsync(q, h->b.s_q + o1, n1 * 8, cudaMemcpyDeviceToHost, h->stream));
  if (f_orbit) OD_CK(h, cudaMemcpyAsync(f_orbit, h->b.s_orbit + 3 * o1, 3 * n1 * 8, cudaMemcpyDeviceToHost, h->stream));
  if (f_collect) OD_CK(h, cudaMemcpyAsync(f_collect, h->b.s_collect + 3 * o1, 3 * n1 * 8, cudaMemcpyDeviceToHost, h->stream));
  if (f_dust) OD_CK(h, cudaMemcpyAsync(f_dust, h->b.s_dust + 3 * o1, 3 * n1 * 8, cudaMemcpyDeviceToHost, h->stream));
  if (f_field) OD_CK(h, cudaMemcpyAsync(f_field, h->b.s_field + 3 * o1, 3 * n1 * 8, cudaMemcpyDeviceToHost, h->stream));
  OD_CK(h, cudaStreamSynchronize(h->stream));
  return OD_OK;
}

extern "C" od_status od_get_averages(od_handle* h, double* out, int64_t* n_avg) {
  if (!h || !out) return fail(h, OD_ERR_INVALID, "NULL argument");
  OD_CK(h, cudaSetDevice(h->device));
  od_dstate s;
  OD_CK(h, cudaMemcpyAsync(&s, h->ds, sizeof(s), cudaMemcpyDeviceToHost, h->stream));
  OD_CK(h, cudaStreamSynchronize(h->stream));
  const double n = s.n_avg > 0 ? (double)s.n_avg : 1.0;
  for (int g = 0; g < h->P; g++)
    for (int m = 0; m < 13; m++) out[g * 13 + m] = s.avg[g][m] / n;
  if (n_avg) *n_avg = s.n_avg;
  return OD_OK;
}

static od_status ensure_snapshot(od_handle* h) {
  if (h->snap_pos) return OD_OK;
  OD_CK(h, dalloc(&h->snap_pos, h->Npad));
  OD_CK(h, dalloc(&h->snap_hi, h->Npad));
  OD_CK(h, dalloc(&h->snap_lo, h->Npad));
  OD_CK(h, dalloc(&h->snap_counts, OD_MAX_GRAINS + 1));
  return OD_OK;
}

static od_status upload_snapshot(od_handle* h, const double* pos, int64_t n) {
  od_status st = ensure_snapshot(h);
  if (st != OD_OK) return st;
  std::vector<float4> xp;
  to_device_units(h, pos, nullptr, n, xp, nullptr);
  xp.resize(h->Npad, make_float4(OD_SENTINEL, OD_SENTINEL, OD_SENTINEL, 0.f));
  OD_CK(h, cudaMemcpyAsync(h->snap_pos, xp.data(), sizeof(float4) * h->Npad, cudaMemcpyHostToDevice, h->stream));
  OD_CK(h, cudaStreamSynchronize(h->stream));
  return OD_OK;
}

extern "C" od_status od_force_snapshot(od_handle* h, const double* pos, int64_t n, double* force) {
  if (!h) return fail(nullptr, OD_ERR_INVALID, "handle is NULL");
  if (!pos || !force) return fail(h, OD_ERR_INVALID, "NULL argument");
  if (n < 1 || n > h->N) return fail(h, OD_ERR_INVALID, "n must be in [1, n_ions]");
  OD_CK(h, cudaSetDevice(h->device));
  od_status st = upload_snapshot(h, pos, n);
  if (st != OD_OK) return st;
  // the snapshot borrows the SoA source buffers; od_step rewrites them before its next use
  OD_CK(h, od_launch_aos_to_soa(h->snap_pos, h->Npad, h->b.sx, h->b.sy, h->b.sz, h->stream));
  OD_CK(h, od_launch_force(force_ctx(h, false), od_pair_io{h->snap_pos, h->b.sx, h->b.sy, h->b.sz, h->b.n3},
                           (int)n, h->Npad, h->b.part_hi, h->b.part_lo, &h->ds->err, h->stream));
  OD_CK(h, od_launch_reduce(h->dp, h->Npad, force_jsplit(h), h->b.part_hi, h->b.part_lo, h->snap_hi,
                            h->snap_lo, h->stream));
  std::vector<float4> hi(n), lo(n);
  OD_CK(h, cudaMemcpyAsync(hi.data(), h->snap_hi, sizeof(float4) * n, cudaMemcpyDeviceToHost, h->stream));
  OD_CK(h, cudaMemcpyAsync(lo.data(), h->snap_lo, sizeof(float4) * n, cudaMemcpyDeviceToHost, h->stream));
  OD_CK(h, cudaStreamSynchronize(h->stream));
  st = check_device_err(h);
  if (st != OD_OK) return st;
  const double F = h->hp.k * h->hp.q_s * h->hp.q_s / (h->hp.lam * h->hp.lam);
  for (int64_t i = 0; i < n; i++) {
    force[3 * i] = F * ((double)hi[i].x + (double)lo[i].x);
    force[3 * i + 1] = F * ((double)hi[i].y + (double)lo[i].y);
    force[3 * i + 2] = F * ((double)hi[i].z + (double)lo[i].z);
  }
  return OD_OK;
}

extern "C" od_status od_snapshot_positions(od_handle* h, const double* pos, int64_t n, double* pos_dev) {
  if (!h || !pos || !pos_dev) return fail(h, OD_ERR_INVALID, "NULL argument");
  std::vector<float4> xp;
  to_device_units(h, pos, nullptr, n, xp, nullptr);
  for (int64_t i = 0; i < n; i++) {
    pos_dev[3 * i] = (double)xp[i].x * h->hp.lam;
    pos_dev[3 * i + 1] = (double)xp[i].y * h->hp.lam;
    pos_dev[3 * i + 2] = (double)xp[i].z * h->hp.lam;
  }
  return OD_OK;
}

extern "C" od_status od_collect_flags(od_handle* h, const double* pos, int64_t n, int64_t* idx_out,
                                      int64_t cap, int64_t* count, int64_t* grain_counts) {
  if (!h) return fail(nullptr, OD_ERR_INVALID, "handle is NULL");
  if (!pos || !count || (cap > 0 && !idx_out)) return fail(h, OD_ERR_INVALID, "NULL argument");
  if (n < 1 || n > h->N) return fail(h, OD_ERR_INVALID, "n must be in [1, n_ions]");
  OD_CK(h, cudaSetDevice(h->device));
  od_status st = upload_snapshot(h, pos, n);
  if (st != OD_OK) return st;
  OD_CK(h, od_launch_snapshot_flags(h->dp, (int)n, h->Npad, h->snap_pos, h->b.flags, h->b.list,
                                    h->b.list_bits, h->snap_counts, h->stream));
  double counts[OD_MAX_GRAINS + 1];
  OD_CK(h, cudaMemcpyAsync(counts, h->snap_counts, sizeof(counts), cudaMemcpyDeviceToHost, h->stream));
  OD_CK(h, cudaStreamSynchronize(h->stream));
  const int64_t K = (int64_t)counts[OD_MAX_GRAINS];
  *count = K;
  if (grain_counts)
    for (int g = 0; g < h->P; g++) grain_counts[g] = (int64_t)counts[g];
  const int64_t m = std::min(K, cap);
  if (m > 0) {
    std::vector<int32_t> li(m);
    OD_CK(h, cudaMemcpyAsync(li.data(), h->b.list, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, h->stream));
    OD_CK(h, cudaStreamSynchronize(h->stream));
    for (int64_t k = 0; k < m; k++) idx_out[k] = li[k];
  }
  if (K > cap) return fail(h, OD_ERR_CAPACITY, "idx_out too small");
  return OD_OK;
}

extern "C" od_status od_trap_potential(double Rh, double Hh, int32_t n_r, int32_t n_h,
                                       int64_t n_points, uint64_t seed, int32_t device, double* pot) {
  if (!pot || n_r < 2 || n_h < 2 || n_points < 1 || !(Rh > 0) || !(Hh > 0))
    return fail(nullptr, OD_ERR_INVALID, "bad trap-fit arguments");
  if (od_device_count() <= device || device < 0)
    return fail(nullptr, OD_ERR_UNSUPPORTED, "no CUDA device with that index");
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaSetDevice");
  const int nn = n_r * n_h;
  const int nchunks = std::max(1, (int)std::min<int64_t>(od_num_sms(device) * 4, (n_points + 4095) / 4096));
  double* part = nullptr;
  e = cudaMalloc(&part, sizeof(double) * nn * nchunks);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaMalloc");
  e = od_launch_trap(Rh, Hh, n_r, n_h, n_points, seed, part, nchunks, 0);
  std::vector<double> hpart((size_t)nn * nchunks);
  if (e == cudaSuccess) e = cudaMemcpy(hpart.data(), part, sizeof(double) * nn * nchunks, cudaMemcpyDeviceToHost);
  cudaFree(part);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "trap potential");
  for (int i = 0; i < nn; i++) {
    double s = 0;
    for (int c = 0; c < nchunks; c++) s += hpart[(size_t)c * nn + i];
    pot[i] = s / (double)n_points;
  }
  return OD_OK;
}

// ============================================================== allocation-free ion–ion forces
// Some callers cannot create device allocations at the moment they need forces: code that runs
// inside another runtime's memory pool or allocator callbacks, real-time loops that forbid
// cudaMalloc after start-up, or plug-ins whose host framework owns every device buffer and
// hands them only pointers. od_ion_forces_static serves them: the caller passes device
// arrays for the positions and the forces, and every scratch byte the kernels need (a padded
// SoA copy of the positions, the partial sums of the source split, and an error word) lives
// in the file-scope array below, which each GPU that loads this library holds until the
// process exits.
#define OD_STATIC_MAX_IONS 32768
#define OD_STATIC_MAX_SPLIT 8
static constexpr size_t kStaticSoA = (size_t)OD_STATIC_MAX_IONS * sizeof(float);
static constexpr size_t kStaticSlab = (size_t)OD_STATIC_MAX_SPLIT * OD_STATIC_MAX_IONS * sizeof(float4);
static constexpr size_t kStaticBytes = 256 + 3 * kStaticSoA + 2 * kStaticSlab;  // about 8.8 MB
static __device__ __align__(256) unsigned char od_static_scratch[kStaticBytes];

// Device address of od_static_scratch on each device. In host code the array's name is only a
// host-side stand-in, so its device address is looked up once per device, with that device
// current, on the first call made on it.
static std::mutex g_static_mu;
static void* g_static_addr[64];

static cudaError_t static_scratch_addr(int dev, unsigned char** out) {
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_static_mu);
  if (!g_static_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, od_static_scratch);
    if (e != cudaSuccess) return e;
    g_static_addr[dev] = p;
  }
  *out = (unsigned char*)g_static_addr[dev];
  return cudaSuccess;
}

extern "C" od_status od_ion_forces_static(const double* pos_dev, int64_t n, double r_D_e,
                                          double r_0, double kq_sq_s, double* force_dev,
                                          void* stream) {
  if (!pos_dev || !force_dev) return fail(nullptr, OD_ERR_INVALID, "pos_dev/force_dev is NULL");
  if (n < 2 || n > OD_STATIC_MAX_IONS)
    return fail(nullptr, OD_ERR_INVALID,
                "od_ion_forces_static takes 2 to 32768 ions (its scratch array is sized for "
                "32768); use od_force_snapshot for larger systems");
  // Every ion is also a source, so its own pair enters with r = 0 and 1/(r + r_0) = 1/r_0;
  // below r_0 = 1e-9 r_D_e the FP32 pair magnitude overflows there and turns the ion's force
  // into NaN. The reference's own r_0 is 1e-3 r_D_e.
  if (!(r_D_e > 0) || !(r_0 >= 1e-9 * r_D_e))
    return fail(nullptr, OD_ERR_INVALID, "r_D_e must be positive and r_0 at least 1e-9 r_D_e");
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaGetDevice");
  unsigned char* base = nullptr;
  e = static_scratch_addr(dev, &base);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaGetSymbolAddress(od_static_scratch)");
  od_static_view v{};
  v.err = (uint32_t*)base;
  v.sx = (float*)(base + 256);
  v.sy = (float*)(base + 256 + kStaticSoA);
  v.sz = (float*)(base + 256 + 2 * kStaticSoA);
  v.part_hi = (float4*)(base + 256 + 3 * kStaticSoA);
  v.part_lo = (float4*)(base + 256 + 3 * kStaticSoA + kStaticSlab);
  v.max_split = OD_STATIC_MAX_SPLIT;
  cudaStream_t s = (cudaStream_t)stream;
  // the error word keeps the previous call's value: clear it
  e = cudaMemsetAsync(v.err, 0, sizeof(uint32_t), s);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaMemsetAsync(error word)");
  const double scale = kq_sq_s / (r_D_e * r_D_e);
  e = od_launch_static_forces(v, pos_dev, (int)n, r_D_e, r_0, scale, force_dev, s);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "all-pairs launch");
  uint32_t err = 0;
  e = cudaMemcpyAsync(&err, v.err, sizeof(err), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "od_ion_forces_static");
  if (err & OD_DERR_TIMEOUT) return fail(nullptr, OD_ERR_TIMEOUT, "a bounded device wait ran out");
  return OD_OK;
}

// ============================================================== batches of simulations
// A batch owns member handles (ordinary od_handle objects) and steps all of them with one set
// of batch-wide launches per step (od_launch_batch_step), replayed from a CUDA graph that is
// rebuilt whenever members join or leave.
struct od_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<od_handle*> members;  // nullptr marks a free slot
  bool dirty = true;
  od_simdesc* d_sims = nullptr;
  int2* d_blk_ion = nullptr;
  int4* d_items = nullptr;
  int2* d_blk_corr = nullptr;
  size_t c_sims = 0, c_blk_ion = 0, c_items = 0, c_blk_corr = 0;
  int4* d_n3_items[2] = {nullptr, nullptr};
  size_t c_n3_items[2] = {0, 0};
  int2* d_n3_blk = nullptr;
  size_t c_n3_blk = 0;
  unsigned int* d_next = nullptr;
  uint32_t* d_err = nullptr;
  od_batchview view{};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0;
  std::string err;
};

static od_status bfail(od_batch* b, od_status st, const std::string& msg) {
  if (b) b->err = msg; else g_err = msg;
  return st;
}
#define OD_BCK(b, call)                                                                  \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return bfail(b, e_ == cudaErrorMemoryAllocation ? OD_ERR_OOM : OD_ERR_CUDA,        \
                   std::string(#call) + ": " + cudaGetErrorString(e_));                  \
  } while (0)

extern "C" const char* od_batch_last_error(const od_batch* b) { return b ? b->err.c_str() : g_err.c_str(); }

extern "C" od_status od_batch_create(int32_t device, od_batch** out) {
  if (!out) return bfail(nullptr, OD_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (od_device_count() <= device || device < 0)
    return bfail(nullptr, OD_ERR_UNSUPPORTED, "no CUDA device with that index");
  od_batch* b = new (std::nothrow) od_batch();
  if (!b) return bfail(nullptr, OD_ERR_OOM, "host allocation failed");
  b->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_next, sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_err, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemset(b->d_err, 0, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
  if (e != cudaSuccess) {
    g_err = std::string("od_batch_create: ") + cudaGetErrorString(e);
    if (b->d_next) cudaFree(b->d_next);
    if (b->d_err) cudaFree(b->d_err);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return OD_ERR_CUDA;
  }
  *out = b;
  return OD_OK;
}

extern "C" od_status od_batch_add(od_batch* b, const od_config* cfg, const double* pos,
                                  const double* vel, int32_t* slot) {
  if (!b || !cfg || !slot || (!pos) != (!vel)) return bfail(b, OD_ERR_INVALID, "NULL argument");
  if (cfg->force_method != OD_FORCE_ALLPAIRS)
    return bfail(b, OD_ERR_UNSUPPORTED, "batch members use the all-pairs force method");
  od_handle* h = nullptr;
  od_status st = create_handle(cfg, b->device, false, &h);
  if (st != OD_OK) return bfail(b, st, g_err);
  // each unordered pair once (od_n3_batch_plan), else the directed kernel
  int ipt = 0;
  const int tile = od_n3_batch_plan(h->Npad, OD_N3_BUDGET, &ipt);
  st = tile ? set_plan_n3(h, ipt, tile) : OD_ERR_OOM;
  if (st != OD_OK) {
    cudaGetLastError();
    st = od_set_pair_plan(h, 256, 1, 5, 0);
    if (st != OD_OK) { std::string m = h->err; od_destroy(h); return bfail(b, st, m); }
  }
  st = pos ? od_set_state(h, pos, vel, cfg->n_ions) : od_init_state(h, nullptr, nullptr, 0);
  if (st != OD_OK) { std::string m = h->err; od_destroy(h); return bfail(b, st, m); }
  int s = -1;
  for (size_t k = 0; k < b->members.size(); k++)
    if (!b->members[k]) { s = (int)k; break; }
  if (s < 0) { s = (int)b->members.size(); b->members.push_back(nullptr); }
  b->members[s] = h;
  b->dirty = true;
  *slot = s;
  return OD_OK;
}

extern "C" od_status od_batch_set_plan(od_batch* b, int32_t slot, int32_t ions_per_lane,
                                       int32_t tile) {
  if (!b || slot < 0 || slot >= (int32_t)b->members.size() || !b->members[slot])
    return bfail(b, OD_ERR_INVALID, "no batch member in that slot");
  if (!((ions_per_lane == 4 && tile == 1024) || (ions_per_lane == 8 && tile == 2048)))
    return bfail(b, OD_ERR_INVALID, "batch members take (4, 1024) or (8, 2048)");
  od_handle* h = b->members[slot];
  const od_status st = set_plan_n3(h, ions_per_lane, tile);
  if (st != OD_OK) return bfail(b, st, h->err);
  b->dirty = true;
  return OD_OK;
}

extern "C" od_status od_batch_remove(od_batch* b, int32_t slot) {
  if (!b || slot < 0 || slot >= (int32_t)b->members.size() || !b->members[slot])
    return bfail(b, OD_ERR_INVALID, "no batch member in that slot");
  od_destroy(b->members[slot]);
  b->members[slot] = nullptr;
  b->dirty = true;
  return OD_OK;
}

extern "C" od_handle* od_batch_member(od_batch* b, int32_t slot) {
  if (!b || slot < 0 || slot >= (int32_t)b->members.size()) return nullptr;
  return b->members[slot];
}

extern "C" int32_t od_batch_size(const od_batch* b) {
  if (!b) return 0;
  int32_t n = 0;
  for (od_handle* h : b->members) n += h != nullptr;
  return n;
}

template <typename T>
static od_status upload_table(od_batch* b, T** dptr, size_t* cap, const std::vector<T>& v) {
  if (v.size() > *cap) {
    if (*dptr) cudaFree(*dptr);
    *dptr = nullptr;
    *cap = 0;
    OD_BCK(b, cudaMalloc((void**)dptr, sizeof(T) * std::max<size_t>(v.size(), 1)));
    *cap = v.size();
  }
  if (!v.empty())
    OD_BCK(b, cudaMemcpyAsync(*dptr, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, b->stream));
  return OD_OK;
}

static od_status batch_rebuild(od_batch* b) {
  std::vector<od_simdesc> sims;
  std::vector<int2> blk_ion, blk_corr;
  struct item { int4 w; long long work; };
  std::vector<item> items;
  std::vector<int4> n3_items[2];
  std::vector<int2> n3_blk;
  for (od_handle* h : b->members) {
    if (!h) continue;
    const int m = (int)sims.size();
    od_simdesc d{};
    d.dp = h->dp; d.ds = h->ds; d.b = h->b;
    d.N = h->N; d.Npad = h->Npad; d.nb = h->Npad / 256;
    d.jsplit = h->plan.jsplit; d.chunk = h->plan.chunk; d.nrec = h->nrec;
    d.rho0 = h->hp.rho0;
    const float nr = 64.0f * h->hp.rho0;
    d.newton_r2 = nr * nr;
    d.n3_tile = h->plan.variant == 7 ? h->plan.tile : 0;
    sims.push_back(d);
    for (int lb = 0; lb < d.nb; lb++) blk_ion.push_back(make_int2(m, lb));
    for (int lb = 0; lb < d.nb + d.nrec; lb++) blk_corr.push_back(make_int2(m, lb));
    if (d.n3_tile) {
      // every tile pair of this member, in the table of its instantiation
      const int nT = (d.Npad + d.n3_tile - 1) / d.n3_tile;
      std::vector<int4>& t = n3_items[h->plan.ipt == 4 && d.n3_tile == 1024 ? 0 : 1];
      for (int bb = 0; bb < nT; bb++)
        for (int aa = 0; aa <= bb; aa++) t.push_back(make_int4(m, aa, bb, nT));
      for (int lb = 0; lb < d.nb; lb++) n3_blk.push_back(make_int2(m, lb));
      continue;
    }
    for (int ib = 0; ib < d.Npad / 256; ib++)
      for (int js = 0; js < d.jsplit; js++) {
        const int j0 = js * d.chunk, j1 = std::min(j0 + d.chunk, d.Npad);
        if (j1 > j0) items.push_back({make_int4(m, ib, j0, j1), (long long)(j1 - j0)});
      }
  }
  std::stable_sort(items.begin(), items.end(), [](const item& a, const item& c) { return a.work > c.work; });
  std::vector<int4> w(items.size());
  for (size_t k = 0; k < items.size(); k++) w[k] = items[k].w;
  od_status st;
  if ((st = upload_table(b, &b->d_sims, &b->c_sims, sims)) != OD_OK) return st;
  if ((st = upload_table(b, &b->d_blk_ion, &b->c_blk_ion, blk_ion)) != OD_OK) return st;
  if ((st = upload_table(b, &b->d_items, &b->c_items, w)) != OD_OK) return st;
  if ((st = upload_table(b, &b->d_blk_corr, &b->c_blk_corr, blk_corr)) != OD_OK) return st;
  for (int k = 0; k < 2; k++)
    if ((st = upload_table(b, &b->d_n3_items[k], &b->c_n3_items[k], n3_items[k])) != OD_OK)
      return st;
  if ((st = upload_table(b, &b->d_n3_blk, &b->c_n3_blk, n3_blk)) != OD_OK) return st;
  OD_BCK(b, cudaStreamSynchronize(b->stream));
  od_batchview& v = b->view;
  v.sims = b->d_sims; v.nsims = (int)sims.size();
  v.blk_ion = b->d_blk_ion; v.nblk_ion = (int)blk_ion.size();
  v.items = b->d_items; v.nitems = (int)w.size();
  v.blk_corr = b->d_blk_corr; v.nblk_corr = (int)blk_corr.size();
  v.pair_grid = od_num_sms(b->device) * 4;
  v.next = b->d_next; v.err = b->d_err;
  for (int k = 0; k < 2; k++) {
    v.n3_items[k] = b->d_n3_items[k];
    v.n3_nitems[k] = (int)n3_items[k].size();
  }
  v.n3_blk = b->d_n3_blk; v.n3_nblk = (int)n3_blk.size();
  if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
  if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
  if (v.nsims > 0) {
    OD_BCK(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = od_launch_batch_step(v, b->stream);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return bfail(b, OD_ERR_CUDA, std::string("batch step capture: ") +
                                       cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    b->graph = g;
    OD_BCK(b, cudaGraphInstantiate(&b->exec, g, 0));
  }
  b->dirty = false;
  return OD_OK;
}

extern "C" od_status od_batch_step(od_batch* b, int64_t nsteps) {
  if (!b) return bfail(nullptr, OD_ERR_INVALID, "batch is NULL");
  if (nsteps < 0) return bfail(b, OD_ERR_INVALID, "nsteps < 0");
  for (od_handle* h : b->members)
    if (h && h->step + nsteps > h->cfg.n_steps)
      return bfail(b, OD_ERR_STATE, "a member's result series would overflow (n_steps reached)");
  OD_BCK(b, cudaSetDevice(b->device));
  if (b->dirty) {
    od_status st = batch_rebuild(b);
    if (st != OD_OK) return st;
  }
  if (!b->exec || nsteps == 0) { b->last_ms = 0; return OD_OK; }
  OD_BCK(b, cudaEventRecord(b->ev0, b->stream));
  for (int64_t s = 0; s < nsteps; s++) OD_BCK(b, cudaGraphLaunch(b->exec, b->stream));
  OD_BCK(b, cudaEventRecord(b->ev1, b->stream));
  OD_BCK(b, cudaStreamSynchronize(b->stream));
  float ms = 0;
  OD_BCK(b, cudaEventElapsedTime(&ms, b->ev0, b->ev1));
  b->last_ms = ms;
  uint32_t berr = 0;
  OD_BCK(b, cudaMemcpy(&berr, b->d_err, sizeof(berr), cudaMemcpyDeviceToHost));
  for (od_handle* h : b->members) {
    if (!h) continue;
    h->step += nsteps;
    od_status st = check_device_err(h);
    if (st != OD_OK) return bfail(b, st, h->err);
  }
  if (berr & OD_DERR_TIMEOUT) return bfail(b, OD_ERR_TIMEOUT, "a bounded device wait ran out");
  return OD_OK;
}

extern "C" od_status od_batch_pair_plan(int64_t n_ions, int32_t* plan5) {
  if (!plan5 || n_ions <= 0) return bfail(nullptr, OD_ERR_INVALID, "bad argument");
  const int Npad = (int)(((n_ions + OD_PAD - 1) / OD_PAD) * OD_PAD);
  int ipt = 0;
  const int tile = od_n3_batch_plan(Npad, OD_N3_BUDGET, &ipt);
  if (tile) {
    plan5[0] = 256; plan5[1] = ipt; plan5[2] = 7; plan5[3] = tile; plan5[4] = Npad;
  } else {
    const od_pair_plan pl = default_plan(Npad, 152);
    plan5[0] = pl.nt; plan5[1] = pl.ipt; plan5[2] = pl.variant; plan5[3] = 0; plan5[4] = 0;
  }
  return OD_OK;
}

extern "C" od_status od_batch_last_step_ms(const od_batch* b, double* ms) {
  if (!b || !ms) return OD_ERR_INVALID;
  *ms = b->last_ms;
  return OD_OK;
}

extern "C" od_status od_batch_destroy(od_batch* b) {
  if (!b) return OD_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (od_handle* h : b->members)
    if (h) od_destroy(h);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  void* ptrs[] = {b->d_sims,         b->d_blk_ion,      b->d_items,  b->d_blk_corr, b->d_next,
                  b->d_err,          b->d_n3_items[0], b->d_n3_items[1], b->d_n3_blk};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return OD_OK;
}

extern "C" od_status od_config_device_bytes(const od_config* cfg, int64_t* bytes) {
  if (!cfg || !bytes) return bfail(nullptr, OD_ERR_INVALID, "NULL argument");
  od_status st = validate(cfg);
  if (st != OD_OK) return st;
  const int64_t Np = ((cfg->n_ions + OD_PAD - 1) / OD_PAD) * OD_PAD;
  const od_pair_plan pl = default_plan((int)Np, 152);
  const int64_t P = std::max(cfg->n_grains, 1);
  int64_t b = 0;
  if (cfg->force_method == OD_FORCE_CUTOFF) {  // tile-pair cutoff, as od_create chooses it
    const int nc = od_cutn3_grid((int)cfg->n_ions, cfg->R, cfg->H).ncells;
    const size_t c512 = od_cutn3_bytes((int)cfg->n_ions, 512, nc);
    const size_t c1024 = od_cutn3_bytes((int)cfg->n_ions, 1024, nc);
    if (c512 <= OD_CUTN3_BUDGET) b += (int64_t)c512;
    else if (c1024 <= OD_CUTN3_BUDGET) b += (int64_t)c1024;
  }
  if (cfg->force_method != OD_FORCE_CUTOFF && uses_n3_default((int)Np)) {
    int ipt = 0;
    const int tile = od_n3_default((int)Np, OD_N3_BUDGET, &ipt);
    if (tile) b += (int64_t)(sizeof(float) * od_n3_floats((int)Np, tile));  // tile-pair sums
  }
  b += Np * 16 * 4;                 // pos, vel, fhi, flo
  b += Np * 12;                     // SoA copy
  b += (int64_t)pl.jsplit * Np * 32;  // partial slabs
  b += Np / 32 * 4 + Np * (4 + 4 + 48);  // flags, list, list bits, list positions/velocities
  b += (Np / 256) * P * 3 * 8;      // orbit partials
  b += cfg->n_steps * P * 13 * 8;   // result series
  b += sizeof(od_dparams) + sizeof(od_dstate) + 4096;
  *bytes = b;
  return OD_OK;
}

extern "C" od_status od_device_memory(int32_t device, int64_t* free_bytes, int64_t* total_bytes) {
  if (!free_bytes || !total_bytes) return fail(nullptr, OD_ERR_INVALID, "NULL argument");
  if (od_device_count() <= device || device < 0)
    return fail(nullptr, OD_ERR_UNSUPPORTED, "no CUDA device with that index");
  int prev = 0;
  cudaGetDevice(&prev);
  cudaError_t e = cudaSetDevice(device);
  size_t f = 0, t = 0;
  if (e == cudaSuccess) e = cudaMemGetInfo(&f, &t);
  cudaSetDevice(prev);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaMemGetInfo");
  *free_bytes = (int64_t)f;
  *total_bytes = (int64_t)t;
  return OD_OK;
}

// ============================================================== shards of one simulation
// One simulation split over several handles (one per GPU), each owning a contiguous range of
// ions; the caller moves three things between the shards every step (all-gathers: positions,
// re-injection lists, orbit partial sums). Every sum keeps the single-simulation order, so the
// shards reproduce a single handle stepped with the same directed all-pairs plan bit for bit.
static od_status shard_check(od_handle* h, int phase) {
  if (!h) return fail(nullptr, OD_ERR_INVALID, "handle is NULL");
  if (!h->shard) return fail(h, OD_ERR_STATE, "not a shard handle (od_shard_create)");
  if (!h->state_set) return fail(h, OD_ERR_STATE, "od_shard_set_state has not been called");
  if (phase >= 0 && h->shard_phase != phase)
    return fail(h, OD_ERR_STATE, "shard calls out of order (begin, positions, forces, list, "
                                 "finish)");
  if (h->step >= h->cfg.n_steps) return fail(h, OD_ERR_STATE, "the result series is full");
  OD_CK(h, cudaSetDevice(h->device));
  return OD_OK;
}

extern "C" od_status od_shard_create(const od_config* cfg, int64_t first, int64_t count,
                                     int32_t jsplit, int32_t device, od_handle** out) {
  if (!cfg || !out) return fail(nullptr, OD_ERR_INVALID, "NULL argument");
  *out = nullptr;
  od_status st = validate(cfg);
  if (st != OD_OK) return st;
  const int64_t Nt = cfg->n_ions;
  if (cfg->force_method != OD_FORCE_ALLPAIRS || cfg->force_every > 1 ||
      cfg->distribution == OD_DIST_MATTHEWS)
    return fail(nullptr, OD_ERR_UNSUPPORTED,
                "shards take the all-pairs force, every step, Maxwellian or field-driven ions");
  if (first < 0 || count < 1 || first + count > Nt || first % OD_PAD ||
      (first + count < Nt && count % OD_PAD))
    return fail(nullptr, OD_ERR_INVALID,
                "a shard starts on a multiple of 512 ions and holds a multiple of 512 (the last "
                "shard: the rest)");
  od_config local = *cfg;
  local.n_ions = count;
  st = create_handle(&local, device, false, out);
  if (st != OD_OK) return st;
  od_handle* h = *out;
  h->shard = true;
  h->ion0 = first;
  h->n_total = Nt;
  h->Npad_total = (int)(((Nt + OD_PAD - 1) / OD_PAD) * OD_PAD);
  h->hp.ion0 = (int32_t)first;
  // the directed plan of a single simulation of n_total ions (variant 5, the source split over
  // all sources), or jsplit source chunks when given
  od_pair_plan pl = default_plan(h->Npad_total, od_num_sms(device));
  if (jsplit > 0) {
    int chunk = (h->Npad_total + jsplit - 1) / jsplit;
    chunk = ((chunk + OD_TJ - 1) / OD_TJ) * OD_TJ;
    pl.chunk = chunk;
    pl.jsplit = (h->Npad_total + chunk - 1) / chunk;
  }
  h->plan = pl;
  auto bad = [&](const char* what) {
    od_status r = fail(h, OD_ERR_OOM, what);
    std::string m = h->err;
    od_destroy(h);
    *out = nullptr;
    g_err = m;
    return r;
  };
  if (alloc_scratch_for_plan(h) != OD_OK) return bad("no device memory for the partial sums");
  const size_t nt = (size_t)h->Npad_total, P = std::max(h->P, 1);
  if (dalloc(&h->ssx, nt) || dalloc(&h->ssy, nt) || dalloc(&h->ssz, nt) ||
      dalloc(&h->g_idx, (size_t)Nt) || dalloc(&h->g_bits, (size_t)Nt) ||
      dalloc(&h->g_old, (size_t)Nt) || dalloc(&h->g_new, (size_t)Nt) ||
      dalloc(&h->g_v, (size_t)Nt) || dalloc(&h->g_orbit, nt / 256 * P * 3)) {
    cudaGetLastError();
    return bad("no device memory for the shard's sources");
  }
  if (nt > (size_t)Nt) {  // padding sources: far-away sentinels
    std::vector<float> sent(nt - Nt, OD_SENTINEL);
    for (float* a : {h->ssx, h->ssy, h->ssz})
      if (cudaMemcpy(a + Nt, sent.data(), sizeof(float) * (nt - Nt), cudaMemcpyHostToDevice))
        return bad("sentinel upload");
  }
  if (cudaMemcpy(h->dp, &h->hp, sizeof(od_dparams), cudaMemcpyHostToDevice) != cudaSuccess)
    return bad("parameter upload");
  return OD_OK;
}

// take: into slab 0 of the partial sums (initial state); else left in the accumulators for K3
static od_status shard_forces_now(od_handle* h, bool take) {
  OD_CK(h, od_launch_shard_pairs(h->plan, h->ssx, h->ssy, h->ssz, h->Npad_total, h->Npad,
                                 (int)h->ion0, h->b.part_hi, h->b.part_lo, h->hp.rho0, &h->ds->err,
                                 h->b.n3, take, h->stream));
  return OD_OK;
}

extern "C" od_status od_shard_set_state(od_handle* h, const double* pos_all,
                                        const double* vel_own) {
  if (!h) return fail(nullptr, OD_ERR_INVALID, "handle is NULL");
  if (!h->shard) return fail(h, OD_ERR_STATE, "not a shard handle (od_shard_create)");
  if (!pos_all || !vel_own) return fail(h, OD_ERR_INVALID, "pos_all/vel_own is NULL");
  if (!all_finite(pos_all, 3 * h->n_total) || !all_finite(vel_own, 3 * h->N))
    return fail(h, OD_ERR_INVALID, "a position or velocity is not finite");
  OD_CK(h, cudaSetDevice(h->device));
  std::vector<float4> xa, vp, xo, ra, ro;
  to_rel_state(h, pos_all, h->n_total, ra, xa);  // every shard's sources, as their owners hold them
  to_device_units(h, nullptr, vel_own, h->N, xo, &vp);
  to_rel_state(h, pos_all + 3 * h->ion0, h->N, ro, xo);
  std::vector<float> c(h->n_total);
  float* dst[3] = {h->ssx, h->ssy, h->ssz};
  for (int d = 0; d < 3; d++) {
    for (int64_t i = 0; i < h->n_total; i++) c[i] = d == 0 ? xa[i].x : (d == 1 ? xa[i].y : xa[i].z);
    OD_CK(h, cudaMemcpy(dst[d], c.data(), sizeof(float) * h->n_total, cudaMemcpyHostToDevice));
  }
  OD_CK(h, cudaMemcpy(h->b.pos, xo.data(), sizeof(float4) * h->N, cudaMemcpyHostToDevice));
  OD_CK(h, cudaMemcpy(h->b.rel, ro.data(), sizeof(float4) * h->N, cudaMemcpyHostToDevice));
  OD_CK(h, cudaMemcpy(h->b.vel, vp.data(), sizeof(float4) * h->N, cudaMemcpyHostToDevice));
  od_status st = shard_forces_now(h, true);
  if (st != OD_OK) return st;
  OD_CK(h, od_launch_reduce(h->dp, h->Npad, 1, h->b.part_hi, h->b.part_lo, h->b.fhi, h->b.flo,
                            h->stream));
  OD_CK(h, cudaStreamSynchronize(h->stream));
  h->state_set = true;
  h->shard_phase = 0;
  return check_device_err(h);
}

extern "C" od_status od_shard_begin(od_handle* h, float* xyz_out) {
  od_status st = shard_check(h, 0);
  if (st != OD_OK) return st;
  if (!xyz_out) return fail(h, OD_ERR_INVALID, "xyz_out is NULL");
  float* own[3] = {h->ssx + h->ion0, h->ssy + h->ion0, h->ssz + h->ion0};
  OD_CK(h, od_launch_shard_part(0, h->dp, h->ds, h->b, h->N, h->Npad, h->plan.jsplit, own[0],
                                own[1], own[2], h->stream));
  for (int d = 0; d < 3; d++)
    OD_CK(h, cudaMemcpyAsync(xyz_out + (size_t)d * h->N, own[d], sizeof(float) * h->N,
                             cudaMemcpyDefault, h->stream));
  OD_CK(h, cudaStreamSynchronize(h->stream));
  h->shard_phase = 1;
  return OD_OK;
}

extern "C" od_status od_shard_forces(od_handle* h, const float* xyz_all, int64_t* n_list) {
  od_status st = shard_check(h, 1);
  if (st != OD_OK) return st;
  if (!xyz_all || !n_list) return fail(h, OD_ERR_INVALID, "NULL argument");
  float* dst[3] = {h->ssx, h->ssy, h->ssz};
  for (int d = 0; d < 3; d++)
    OD_CK(h, cudaMemcpyAsync(dst[d], xyz_all + (size_t)d * h->n_total, sizeof(float) * h->n_total,
                             cudaMemcpyDefault, h->stream));
  st = shard_forces_now(h, false);
  if (st != OD_OK) return st;
  OD_CK(h, od_launch_shard_part(1, h->dp, h->ds, h->b, h->N, h->Npad, h->plan.jsplit, nullptr,
                                nullptr, nullptr, h->stream));
  int32_t K = 0;
  OD_CK(h, cudaMemcpyAsync(&K, &h->ds->nlist, sizeof(K), cudaMemcpyDeviceToHost, h->stream));
  OD_CK(h, cudaStreamSynchronize(h->stream));
  *n_list = K;
  h->shard_phase = 2;
  return check_device_err(h);
}

extern "C" od_status od_shard_get_list(od_handle* h, int32_t* idx, int32_t* bits, float* old4,
                                       float* new4, float* v4) {
  od_status st = shard_check(h, 2);
  if (st != OD_OK) return st;
  if (!idx || !bits || !old4 || !new4 || !v4) return fail(h, OD_ERR_INVALID, "NULL argument");
  int32_t K = 0;
  OD_CK(h, cudaMemcpy(&K, &h->ds->nlist, sizeof(K), cudaMemcpyDeviceToHost));
  if (K == 0) return OD_OK;
  std::vector<int32_t> li(K);
  OD_CK(h, cudaMemcpy(li.data(), h->b.list, sizeof(int32_t) * K, cudaMemcpyDeviceToHost));
  for (auto& i : li) i += (int32_t)h->ion0;  // global indices
  OD_CK(h, cudaMemcpy(idx, li.data(), sizeof(int32_t) * K, cudaMemcpyDefault));
  OD_CK(h, cudaMemcpy(bits, h->b.list_bits, sizeof(int32_t) * K, cudaMemcpyDefault));
  OD_CK(h, cudaMemcpy(old4, h->b.list_old, sizeof(float4) * K, cudaMemcpyDefault));
  OD_CK(h, cudaMemcpy(new4, h->b.list_new, sizeof(float4) * K, cudaMemcpyDefault));
  OD_CK(h, cudaMemcpy(v4, h->b.list_v, sizeof(float4) * K, cudaMemcpyDefault));
  return OD_OK;
}

extern "C" od_status od_shard_set_list(od_handle* h, int64_t n, const int32_t* idx,
                                       const int32_t* bits, const float* old4, const float* new4,
                                       const float* v4, double* orbit_out) {
  od_status st = shard_check(h, 2);
  if (st != OD_OK) return st;
  if (n < 0 || n > h->n_total) return fail(h, OD_ERR_INVALID, "list longer than the run");
  if (!orbit_out || (n > 0 && (!idx || !bits || !old4 || !new4 || !v4)))
    return fail(h, OD_ERR_INVALID, "NULL argument");
  if (n > 0) {
    OD_CK(h, cudaMemcpyAsync(h->g_idx, idx, sizeof(int32_t) * n, cudaMemcpyDefault, h->stream));
    OD_CK(h, cudaMemcpyAsync(h->g_bits, bits, sizeof(int32_t) * n, cudaMemcpyDefault, h->stream));
    OD_CK(h, cudaMemcpyAsync(h->g_old, old4, sizeof(float4) * n, cudaMemcpyDefault, h->stream));
    OD_CK(h, cudaMemcpyAsync(h->g_new, new4, sizeof(float4) * n, cudaMemcpyDefault, h->stream));
    OD_CK(h, cudaMemcpyAsync(h->g_v, v4, sizeof(float4) * n, cudaMemcpyDefault, h->stream));
  }
  OD_CK(h, od_launch_shard_list(h->dp, h->ds, (int)n, h->g_idx, h->g_bits, h->g_new, h->g_v,
                                h->ssx, h->ssy, h->ssz, h->stream));
  OD_CK(h, od_launch_shard_correct(h->dp, h->ds, h->b, h->Npad, h->nrec, h->g_idx, h->g_old,
                                   h->g_new, h->ssx, h->ssy, h->ssz, (int)h->n_total, h->stream));
  const size_t nc = (size_t)(h->Npad / 256) * std::max(h->P, 1) * 3;
  OD_CK(h, cudaMemcpyAsync(orbit_out, h->b.orbit_part, sizeof(double) * nc, cudaMemcpyDefault,
                           h->stream));
  OD_CK(h, cudaStreamSynchronize(h->stream));
  h->shard_phase = 3;
  return check_device_err(h);
}

extern "C" od_status od_shard_finish(od_handle* h, const double* orbit_all) {
  od_status st = shard_check(h, 3);
  if (st != OD_OK) return st;
  if (!orbit_all) return fail(h, OD_ERR_INVALID, "orbit_all is NULL");
  const int nb_all = h->Npad_total / 256;
  const size_t nc = (size_t)nb_all * std::max(h->P, 1) * 3;
  OD_CK(h, cudaMemcpyAsync(h->g_orbit, orbit_all, sizeof(double) * nc, cudaMemcpyDefault,
                           h->stream));
  OD_CK(h, od_launch_shard_tail(h->dp, h->ds, h->b, h->g_orbit, nb_all, h->stream));
  OD_CK(h, cudaStreamSynchronize(h->stream));
  h->step += 1;
  h->shard_phase = 0;
  return check_device_err(h);
}

extern "C" od_status od_shard_info(const od_handle* h, int64_t* first, int64_t* count,
                                   int64_t* n_total, int64_t* orbit_blocks) {
  if (!h || !h->shard) return fail(nullptr, OD_ERR_INVALID, "not a shard handle");
  if (first) *first = h->ion0;
  if (count) *count = h->N;
  if (n_total) *n_total = h->n_total;
  if (orbit_blocks) *orbit_blocks = h->Npad / 256;
  return OD_OK;
}
