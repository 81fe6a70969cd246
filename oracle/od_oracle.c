/*
 * od_oracle.c — CPU ORACLE (test infrastructure only; never part of the product path).
 *
 * A plain-C, FP64 restatement of OpenDust's per-timestep superion update
 * (src/opendust/opendust.py), used by tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py as the checker for the CUDA library.
 *
 * It follows the reference's OpenMM CustomIntegrator program literally
 * (opendust.py:839-1037): collisions -> half kick with forces at the current
 * positions -> drift -> half kick with forces recomputed at the drifted positions
 * -> grain/domain flags -> collection sums -> re-injection -> orbit sums, and then
 * the host tail (opendust.py:1117-1383). That is two full ion–ion force
 * evaluations per step, as OpenMM performs them (forces are re-evaluated whenever
 * positions changed). Lengths are in units of lambda = r_D_e and time in units of
 * d_t inside the step; grain quantities are SI.
 *
 * The third-party arithmetic of the reference's path lives in OpenMM (version
 * unpinned in conda-recipe/meta.yaml:12-16), CuPy and scipy; this file restates
 * the expressions OpenDust hands to them. Random numbers are Philox4x32-10
 * (Salmon, Moraes, Dror, Shaw, SC'11), defined in include/opendust_gb300.h; the
 * reference's own streams are unseeded, so trajectory parity with the reference
 * is statistical (see tests/golden).
 *
 * Build: oracle/Makefile (gcc -O2 -fopenmp -ffp-contract=off).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "../include/opendust_gb300.h"

#define ODO_PI 3.14159265358979323846

/* ------------------------------------------------------------------ Philox */
static void philox_round(uint32_t c[4], const uint32_t k[2]) {
  uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
  uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
  uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
  uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
  uint32_t n0 = hi1 ^ c[1] ^ k[0];
  uint32_t n2 = hi0 ^ c[3] ^ k[1];
  c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
}

void odo_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
  uint32_t k[2] = {key[0], key[1]};
  for (int r = 0; r < 10; r++) {
    if (r) { k[0] += 0x9E3779B9u; k[1] += 0xBB67AE85u; }
    philox_round(c, k);
  }
  memcpy(out, c, sizeof(c));
}

static void draw(uint64_t seed, uint32_t ion, uint32_t step, uint32_t stream, uint32_t sim,
                 uint32_t w[4]) {
  uint32_t ctr[4] = {ion, step, stream, sim};
  uint32_t key[2] = {(uint32_t)(seed & 0xffffffffu), (uint32_t)(seed >> 32)};
  odo_philox(ctr, key, w);
}
static double u01(uint32_t w) { return (double)(w >> 8) * (1.0 / 16777216.0); }
static double u01c(uint32_t w) { return (double)((w >> 8) + 1u) * (1.0 / 16777216.0); }
static void gauss2(uint32_t a, uint32_t b, double* g0, double* g1) {
  double r = sqrt(-2.0 * log(u01c(a)));
  double t = 2.0 * ODO_PI * u01(b);
  *g0 = r * cos(t);
  *g1 = r * sin(t);
}

/* ------------------------------------------------------- scaled parameters */
typedef struct {
  int dist, coll, method, P;
  int64_t N;
  uint64_t seed;
  uint32_t sim;
  double lam, dt, vunit, k, q_s, m_s;
  double A_ii, A_id, rho0, Rh, Hh, Rh2, Hh_half, a_field, vT, vfl, p_coll;
  double mfp_h, vmax_mfp, Pmax_mfp;
  double rc, rs; /* cutoff / switching in lambda units */
  double gx[OD_MAX_GRAINS], gy[OD_MAX_GRAINS], gz[OD_MAX_GRAINS], gr2[OD_MAX_GRAINS];
  int tn[OD_NTAB];
  double tv[OD_NTAB][OD_MAX_TABLE], txi[OD_NTAB][OD_MAX_TABLE], tsl[OD_NTAB][OD_MAX_TABLE];
  double p_t, p_s, p_b;
  /* chains/matthews.py fork: field of order 2 (acceleration units, z in lambda), tabulated
   * trap (natural cubic splines of alpha_k(h), h in lambda), per-grain tail factors */
  int field_order, trap_kind, ttn;
  double fa0, fa1, fa2, fz1, fz7;
  double th0, tdh;
  double tcf[5][OD_MAX_TRAP][4];
  double gfield[OD_MAX_GRAINS], gout[OD_MAX_GRAINS][3];
} odo_par;

/* Natural cubic spline (zero second derivative at both ends: OpenMM's Continuous1DFunction)
 * through y[0..n-1] on knots of spacing d. Second derivatives from the tridiagonal system
 * M[j-1] + 4 M[j] + M[j+1] = 6 (y[j+1] - 2 y[j] + y[j-1]) / d^2, solved by Gaussian elimination
 * without pivoting; coef[j] = (y_j, slope, M_j / 2, (M_j+1 - M_j) / (6 d)) in powers of h - h_j. */
static void spline_natural(const double* y, int n, double d, double (*coef)[4]) {
  double M[OD_MAX_TRAP] = {0}, diag[OD_MAX_TRAP], rhs[OD_MAX_TRAP];
  for (int j = 1; j < n - 1; j++) {
    diag[j] = 4.0;
    rhs[j] = 6.0 * (y[j + 1] - 2.0 * y[j] + y[j - 1]) / (d * d);
  }
  for (int j = 2; j < n - 1; j++) {
    double m = 1.0 / diag[j - 1];
    diag[j] -= m;
    rhs[j] -= m * rhs[j - 1];
  }
  for (int j = n - 2; j >= 1; j--) M[j] = (rhs[j] - (j < n - 2 ? M[j + 1] : 0.0)) / diag[j];
  for (int j = 0; j < n - 1; j++) {
    coef[j][0] = y[j];
    coef[j][1] = (y[j + 1] - y[j]) / d - d * (2.0 * M[j] + M[j + 1]) / 6.0;
    coef[j][2] = M[j] / 2.0;
    coef[j][3] = (M[j + 1] - M[j]) / (6.0 * d);
  }
}

static int make_par(const od_config* c, odo_par* p) {
  if (!c || c->abi_version != OD_ABI_VERSION) return 1;
  if (c->n_grains < 0 || c->n_grains > OD_MAX_GRAINS) return 1;
  memset(p, 0, sizeof(*p));
  p->dist = c->distribution; p->coll = c->collision_model; p->method = c->force_method;
  p->P = c->n_grains; p->N = c->n_ions; p->seed = c->seed; p->sim = (uint32_t)c->sim_id;
  p->lam = c->r_D_e; p->dt = c->d_t; p->vunit = c->r_D_e / c->d_t;
  p->k = 1.0 / (c->eps_0 * 4.0 * ODO_PI);                 /* opendust.py:289 */
  p->q_s = fabs(c->e) * c->N_s;                           /* opendust.py:302 */
  p->m_s = c->m_i * c->N_s;                               /* opendust.py:303-305 */
  double s = c->d_t * c->d_t / (p->m_s * c->r_D_e * c->r_D_e * c->r_D_e);
  p->A_ii = p->k * p->q_s * p->q_s * s;                   /* ion–ion and trap prefactor */
  p->A_id = p->k * p->q_s * s;                            /* times q_p: ion–dust prefactor */
  p->rho0 = c->r_0 / c->r_D_e;
  p->Rh = c->R / c->r_D_e; p->Hh = c->H / c->r_D_e;
  p->Rh2 = p->Rh * p->Rh; p->Hh_half = p->Hh / 2.0;
  double sf = p->q_s * c->d_t * c->d_t / (p->m_s * c->r_D_e); /* V/m -> lambda/d_t^2 */
  p->a_field = (c->distribution != OD_DIST_MAXWELLIAN) ? c->E * sf : 0.0;
  p->field_order = c->distribution == OD_DIST_MATTHEWS ? c->field_order : 0;
  if (p->field_order == 2) { /* chains/matthews.py:484-495 */
    p->fa0 = c->E * sf;
    p->fa1 = c->field_alpha * c->r_D_e * sf;
    p->fa2 = c->field_beta * c->r_D_e * c->r_D_e * sf;
    p->fz1 = c->field_z1 / c->r_D_e;
    p->fz7 = c->field_z7 / c->r_D_e;
  }
  p->trap_kind = c->trap_kind;
  if (c->trap_kind == OD_TRAP_TABLE) { /* chains/matthews.py:463-478 */
    if (c->trap_n < 4 || c->trap_n > OD_MAX_TRAP || !c->trap_tab) return 1;
    p->ttn = c->trap_n;
    p->th0 = -c->H / c->r_D_e / 2.0;
    p->tdh = c->H / c->r_D_e / (c->trap_n - 1);
    for (int k = 0; k < 5; k++) spline_natural(c->trap_tab + (size_t)k * c->trap_n, c->trap_n, p->tdh, p->tcf[k]);
  }
  p->vT = c->v_T / p->vunit; p->vfl = c->v_fl / p->vunit;
  p->p_coll = c->d_t * c->w_c;
  if (c->collision_model == OD_COLL_MFP) {
    p->mfp_h = c->mfp / c->r_D_e;
    p->vmax_mfp = 3.0 * fabs(p->vfl) + 10.0 * p->vT;
    p->Pmax_mfp = 1.0 - exp(-p->vmax_mfp / p->mfp_h);
  }
  p->rc = c->cutoff / c->r_D_e;
  p->rs = c->switch_dist > 0 ? c->switch_dist / c->r_D_e : p->rc;
  for (int g = 0; g < p->P; g++) {
    p->gx[g] = c->grain_x[g] / c->r_D_e;
    p->gy[g] = c->grain_y[g] / c->r_D_e;
    p->gz[g] = c->grain_z[g] / c->r_D_e;
    double r = c->grain_r[g] / c->r_D_e;
    p->gr2[g] = r * r;
    p->gfield[g] = c->grain_field ? c->grain_field[g]
                                  : (c->distribution == OD_DIST_FIELD_DRIVEN ? c->E : 0.0);
    for (int d = 0; d < 3; d++) p->gout[g][d] = c->grain_out ? c->grain_out[3 * g + d] : 0.0;
  }
  for (int t = 0; t < OD_NTAB; t++) {
    p->tn[t] = c->tab_n[t];
    if (p->tn[t] > OD_MAX_TABLE) return 1;
    for (int i = 0; i < p->tn[t]; i++) {
      p->tv[t][i] = c->tab_v[t][i] / p->vunit;
      p->txi[t][i] = c->tab_xi[t][i];
      p->tsl[t][i] = c->tab_slope[t][i] / p->vunit;
    }
  }
  p->p_t = c->p_top; p->p_s = c->p_side; p->p_b = c->p_bottom;
  return 0;
}

/* ------------------------------------------------------------- forces */
/* Ion–ion kernel of opendust.py:472: U = kq_sq_s exp(-r/r_D_e)/(r+r_0). Returns the radial
 * factor c such that the acceleration on i is A_ii * c * (x_i - x_j). With a cutoff, OpenMM's
 * switching polynomial S = 1 - 10x^3 + 15x^4 - 6x^5 multiplies the energy (opendust.py:481-485). */
static double pair_factor(const odo_par* p, double r2) {
  double r = sqrt(r2);
  if (p->method == OD_FORCE_CUTOFF && r >= p->rc) return 0.0;
  double e = exp(-r);
  double sg = r + p->rho0;
  double f = e * (1.0 / sg + 1.0 / (sg * sg));
  if (p->method == OD_FORCE_CUTOFF && r > p->rs) {
    double w = p->rc - p->rs;
    double x = (r - p->rs) / w;
    double S = 1.0 - x * x * x * (10.0 - x * (15.0 - 6.0 * x));
    double dS = -x * x * (30.0 - x * (60.0 - 30.0 * x)) / w;
    f = f * S - (e / sg) * dS;
  }
  return f / r;
}

/* Cell list for the cutoff method: bins of side >= rc/2 over the ions' bounding box (a target
 * visits the 5 x 5 x 5 bins around its own),
 * ions of a bin listed in increasing index order (stable counting sort). Only the cost of the
 * oracle changes: pair_factor is still applied to every pair of neighbouring bins and returns
 * 0 beyond rc, so the set of pairs and their terms equal the plain double loop's (the order
 * of the FP64 sum differs). */
typedef struct {
  int nc[3];
  double lo[3], inv[3];
  int64_t* start; /* nc0*nc1*nc2 + 1 */
  int64_t* list;  /* n */
} odo_cells;

static int cell_coord(const odo_cells* cl, int d, double v) {
  int c = (int)floor((v - cl->lo[d]) * cl->inv[d]);
  return c < 0 ? 0 : (c >= cl->nc[d] ? cl->nc[d] - 1 : c);
}

static int cells_build(const odo_par* p, int64_t n, const double* x, odo_cells* cl) {
  for (int d = 0; d < 3; d++) { cl->lo[d] = INFINITY; }
  double hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = 0; i < n; i++)
    for (int d = 0; d < 3; d++) {
      double v = x[3 * i + d];
      if (v < cl->lo[d]) cl->lo[d] = v;
      if (v > hi[d]) hi[d] = v;
    }
  int64_t total = 1;
  for (int d = 0; d < 3; d++) {
    double ext = hi[d] - cl->lo[d];
    int m = (int)floor(2.0 * ext / p->rc);
    if (m < 1) m = 1;
    if (m > 512) m = 512;
    cl->nc[d] = m;
    cl->inv[d] = ext > 0 ? m / ext : 0.0; /* bin side ext/m >= rc/2 */
    total *= m;
  }
  cl->start = (int64_t*)calloc((size_t)total + 1, sizeof(int64_t));
  cl->list = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
  int64_t* cid = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
  if (!cl->start || !cl->list || !cid) { free(cl->start); free(cl->list); free(cid); return 1; }
  for (int64_t i = 0; i < n; i++) {
    int cx = cell_coord(cl, 0, x[3 * i]), cy = cell_coord(cl, 1, x[3 * i + 1]);
    int cz = cell_coord(cl, 2, x[3 * i + 2]);
    cid[i] = ((int64_t)cz * cl->nc[1] + cy) * cl->nc[0] + cx;
    cl->start[cid[i] + 1]++;
  }
  for (int64_t c = 0; c < total; c++) cl->start[c + 1] += cl->start[c];
  int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)total);
  if (!fill) { free(cl->start); free(cl->list); free(cid); return 1; }
  memcpy(fill, cl->start, sizeof(int64_t) * (size_t)total);
  for (int64_t i = 0; i < n; i++) cl->list[fill[cid[i]]++] = i;
  free(fill); free(cid);
  return 0;
}

static void cells_free(odo_cells* cl) { free(cl->start); free(cl->list); }

/* G_i for one target i over the bins around it */
static void ionion_cells_one(const odo_par* p, const odo_cells* cl, const double* x, int64_t i,
                             double* g) {
  double xi = x[3 * i], yi = x[3 * i + 1], zi = x[3 * i + 2];
  int c0 = cell_coord(cl, 0, xi), c1 = cell_coord(cl, 1, yi), c2 = cell_coord(cl, 2, zi);
  /* pairs with r^2 above rc^2 (1 + 1e-12) have r > rc, where pair_factor is 0: skipped */
  const double r2max = p->rc * p->rc * (1.0 + 1e-12);
  double gx = 0, gy = 0, gz = 0;
  for (int bz = c2 - 2; bz <= c2 + 2; bz++) {
    if (bz < 0 || bz >= cl->nc[2]) continue;
    for (int by = c1 - 2; by <= c1 + 2; by++) {
      if (by < 0 || by >= cl->nc[1]) continue;
      for (int bx = c0 - 2; bx <= c0 + 2; bx++) {
        if (bx < 0 || bx >= cl->nc[0]) continue;
        int64_t c = ((int64_t)bz * cl->nc[1] + by) * cl->nc[0] + bx;
        for (int64_t k = cl->start[c]; k < cl->start[c + 1]; k++) {
          int64_t j = cl->list[k];
          if (j == i) continue;
          double dx = xi - x[3 * j], dy = yi - x[3 * j + 1], dz = zi - x[3 * j + 2];
          double r2 = dx * dx + dy * dy + dz * dz;
          if (r2 > r2max) continue;
          double cc = pair_factor(p, r2);
          gx += cc * dx; gy += cc * dy; gz += cc * dz;
        }
      }
    }
  }
  g[0] = gx; g[1] = gy; g[2] = gz;
}

/* G_i = sum_{j != i} c(r_ij) (x_i - x_j), lambda units */
static void ionion(const odo_par* p, int64_t n, const double* x, double* G) {
  odo_cells cl;
  if (p->method == OD_FORCE_CUTOFF && n > 4096 && !cells_build(p, n, x, &cl)) {
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < n; i++) ionion_cells_one(p, &cl, x, i, G + 3 * i);
    cells_free(&cl);
    return;
  }
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < n; i++) {
    double xi = x[3 * i], yi = x[3 * i + 1], zi = x[3 * i + 2];
    double gx = 0, gy = 0, gz = 0;
    for (int64_t j = 0; j < n; j++) {
      if (j == i) continue;
      double dx = xi - x[3 * j], dy = yi - x[3 * j + 1], dz = zi - x[3 * j + 2];
      double c = pair_factor(p, dx * dx + dy * dy + dz * dz);
      gx += c * dx; gy += c * dy; gz += c * dz;
    }
    G[3 * i] = gx; G[3 * i + 1] = gy; G[3 * i + 2] = gz;
  }
}

/* trap (opendust.py:552-577): U = C * sum_k alpha_k r^a h^b with r = rho/lambda, h = z/lambda.
 * In u = r^2, w = h^2 the acceleration is -A_ii * (2x P_u, 2y P_u, 2z P_w). */
static void trap_accel(const double* al, double A, double x, double y, double z, double* a) {
  double u = x * x + y * y, w = z * z;
  double Pu = al[1] + al[3] * w + 2 * al[4] * u + 2 * al[6] * u * w + al[7] * w * w +
              3 * al[8] * u * u + 2 * al[10] * u * w * w + 3 * al[11] * u * u * w +
              al[12] * w * w * w + 4 * al[13] * u * u * u;
  double Pw = al[2] + al[3] * u + 2 * al[5] * w + al[6] * u * u + 2 * al[7] * u * w +
              3 * al[9] * w * w + 2 * al[10] * u * u * w + al[11] * u * u * u +
              3 * al[12] * u * w * w + 4 * al[14] * w * w * w;
  a[0] = -A * 2 * x * Pu;
  a[1] = -A * 2 * y * Pu;
  a[2] = -A * 2 * z * Pw;
}

/* tabulated trap (chains/matthews.py:463-478): -A grad [alpha_0(h) + alpha_1(h) u + .. +
 * alpha_4(h) u^4], u = x^2 + y^2, h = z; zero outside [-H/2, H/2] */
static void trap_table_accel(const odo_par* p, double x, double y, double z, double* a) {
  a[0] = a[1] = a[2] = 0.0;
  double h1 = p->th0 + p->tdh * (p->ttn - 1);
  if (z < p->th0 || z > h1) return;
  int j = (int)floor((z - p->th0) / p->tdh);
  if (j > p->ttn - 2) j = p->ttn - 2;
  double t = z - (p->th0 + j * p->tdh), u = x * x + y * y;
  double Pu = 0.0, Pz = 0.0, un = 1.0, um = 1.0; /* dP/du = sum_k k alpha_k u^(k-1), dP/dh */
  for (int k = 0; k <= 4; k++) {
    const double* c = p->tcf[k][j];
    double al = c[0] + c[1] * t + c[2] * t * t + c[3] * t * t * t;
    double dal = c[1] + 2.0 * c[2] * t + 3.0 * c[3] * t * t;
    Pz += dal * un; /* un = u^k */
    if (k > 0) { Pu += k * al * um; um *= u; } /* um = u^(k-1) */
    un *= u;
  }
  a[0] = -p->A_ii * 2.0 * x * Pu;
  a[1] = -p->A_ii * 2.0 * y * Pu;
  a[2] = -p->A_ii * Pz;
}

/* field along z: uniform, or of order 2 with z clamped to [z1, z7] (chains/matthews.py:484-495) */
static double field_accel(const odo_par* p, double z) {
  if (p->field_order != 2) return p->a_field;
  double zc = z < p->fz1 ? p->fz1 : (z > p->fz7 ? p->fz7 : z);
  return p->fa0 + p->fa1 * zc + p->fa2 * zc * zc;
}

/* total acceleration: ion–ion + grains (opendust.py:350-352) + trap + field (opendust.py:580-585) */
static void accel_total(const odo_par* p, const double* alpha, int64_t n, const double* x,
                        const double* qp, double* a) {
  ionion(p, n, x, a);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) {
    double xi = x[3 * i], yi = x[3 * i + 1], zi = x[3 * i + 2];
    double ax = p->A_ii * a[3 * i], ay = p->A_ii * a[3 * i + 1], az = p->A_ii * a[3 * i + 2];
    for (int g = 0; g < p->P; g++) {
      double dx = xi - p->gx[g], dy = yi - p->gy[g], dz = zi - p->gz[g];
      double r2 = dx * dx + dy * dy + dz * dz;
      double c = p->A_id * qp[g] / (r2 * sqrt(r2));
      ax += c * dx; ay += c * dy; az += c * dz;
    }
    double t[3] = {0, 0, 0};
    if (p->trap_kind == OD_TRAP_POLY) trap_accel(alpha, p->A_ii, xi, yi, zi, t);
    else if (p->trap_kind == OD_TRAP_TABLE) trap_table_accel(p, xi, yi, zi, t);
    a[3 * i] = ax + t[0];
    a[3 * i + 1] = ay + t[1];
    a[3 * i + 2] = az + t[2] + field_accel(p, zi);
  }
}

/* Acceleration with a stored ion–ion sum G (lambda units) weighted by w: the force interval
 * (od_config.force_every) uses w = k on the kicks next to an evaluation and 0 otherwise. */
static void accel_mts(const odo_par* p, const double* alpha, int64_t n, const double* x,
                      const double* qp, const double* G, double w, double* a) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) {
    double xi = x[3 * i], yi = x[3 * i + 1], zi = x[3 * i + 2];
    double ax = w * p->A_ii * G[3 * i], ay = w * p->A_ii * G[3 * i + 1], az = w * p->A_ii * G[3 * i + 2];
    for (int g = 0; g < p->P; g++) {
      double dx = xi - p->gx[g], dy = yi - p->gy[g], dz = zi - p->gz[g];
      double r2 = dx * dx + dy * dy + dz * dz;
      double c = p->A_id * qp[g] / (r2 * sqrt(r2));
      ax += c * dx; ay += c * dy; az += c * dz;
    }
    double t[3] = {0, 0, 0};
    if (p->trap_kind == OD_TRAP_POLY) trap_accel(alpha, p->A_ii, xi, yi, zi, t);
    else if (p->trap_kind == OD_TRAP_TABLE) trap_table_accel(p, xi, yi, zi, t);
    a[3 * i] = ax + t[0];
    a[3 * i + 1] = ay + t[1];
    a[3 * i + 2] = az + t[2] + field_accel(p, zi);
  }
}

/* After re-injection the stored ion–ion sums follow the new ion set, as the CUDA step does
 * between evaluations: for every ion that stayed, the removed ions' terms come out and the
 * new ions' terms go in (at the ion's current position); every re-injected ion gets its full
 * sum over all current positions. inj[m] lists the m re-injected ions with their old and new
 * positions. */
static void mts_follow_injection(const odo_par* p, int64_t n, const double* x, const int* fl,
                                 const int64_t* inj, const double* xold, int64_t m, double* G) {
  if (m == 0) return;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; i++) {
    if (fl[i]) continue;
    double xi = x[3 * i], yi = x[3 * i + 1], zi = x[3 * i + 2];
    double gx = 0, gy = 0, gz = 0;
    for (int64_t k = 0; k < m; k++) {
      const double* qn = x + 3 * inj[k];
      const double* qo = xold + 3 * k;
      double dx = xi - qn[0], dy = yi - qn[1], dz = zi - qn[2];
      double c = pair_factor(p, dx * dx + dy * dy + dz * dz);
      gx += c * dx; gy += c * dy; gz += c * dz;
      dx = xi - qo[0]; dy = yi - qo[1]; dz = zi - qo[2];
      c = pair_factor(p, dx * dx + dy * dy + dz * dz);
      gx -= c * dx; gy -= c * dy; gz -= c * dz;
    }
    G[3 * i] += gx; G[3 * i + 1] += gy; G[3 * i + 2] += gz;
  }
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t k = 0; k < m; k++) {
    int64_t i = inj[k];
    double xi = x[3 * i], yi = x[3 * i + 1], zi = x[3 * i + 2];
    double gx = 0, gy = 0, gz = 0;
    for (int64_t j = 0; j < n; j++) {
      if (j == i) continue;
      double dx = xi - x[3 * j], dy = yi - x[3 * j + 1], dz = zi - x[3 * j + 2];
      double c = pair_factor(p, dx * dx + dy * dy + dz * dz);
      gx += c * dx; gy += c * dy; gz += c * dz;
    }
    G[3 * i] = gx; G[3 * i + 1] = gy; G[3 * i + 2] = gz;
  }
}

/* ------------------------------------------------------------- flags */
/* opendust.py:894-910: inside_dust_p = step(r_p - d) (inclusive), outside_domain_r =
 * step(rho - R), outside_domain_z = step(|z| - H/2). Evaluated on squared distances in FP64
 * with a fixed operation order; the CUDA library uses the same operations. */
static int flag_bits(const odo_par* p, double x, double y, double z) {
  int bits = 0;
  for (int g = 0; g < p->P; g++) {
    double dx = x - p->gx[g], dy = y - p->gy[g], dz = z - p->gz[g];
    double d2 = dx * dx + dy * dy;
    d2 = d2 + dz * dz;
    if (d2 <= p->gr2[g]) bits |= 1 << g;
  }
  double rr = x * x + y * y;
  if (rr >= p->Rh2) bits |= 1 << 30;
  if (fabs(z) >= p->Hh_half) bits |= 1 << 29;
  return bits;
}

/* ------------------------------------------------------------- injection */
static double tab_eval(const odo_par* p, int t, double u) {
  int n = p->tn[t];
  int i = 1;
  while (i < n - 1 && u > p->txi[t][i]) i++;
  return p->tv[t][i - 1] + (u - p->txi[t][i - 1]) * p->tsl[t][i];
}

/* Re-injection of one flagged ion (opendust.py:923-975). */
static void inject_one(const odo_par* p, uint32_t ion, uint32_t step, double* x, double* v) {
  uint32_t w[4];
  draw(p->seed, ion, step, OD_RNG_FACE, p->sim, w);
  double uf = u01(w[0]);
  int face; /* 0 top, 1 side, 2 bottom */
  if (uf <= p->p_t) face = 0;
  else if (uf <= p->p_t + p->p_s || p->p_b == 0.0) face = 1;
  else face = 2;
  if (face != 1) {
    int top = face == 0;
    double gx, gy;
    draw(p->seed, ion, step, top ? OD_RNG_TOP_V : OD_RNG_BOT_V, p->sim, w);
    gauss2(w[0], w[1], &gx, &gy);
    double vz = tab_eval(p, top ? OD_TAB_TOP : OD_TAB_BOTTOM, u01(w[2]));
    v[0] = p->vT * gx; v[1] = p->vT * gy; v[2] = vz;
    draw(p->seed, ion, step, top ? OD_RNG_TOP_X : OD_RNG_BOT_X, p->sim, w);
    double rr = p->Rh * sqrt(u01(w[0]));
    double th = 2.0 * ODO_PI * u01(w[1]);
    x[0] = rr * cos(th); x[1] = rr * sin(th); x[2] = top ? -p->Hh_half : p->Hh_half;
  } else {
    draw(p->seed, ion, step, OD_RNG_SIDE_X, p->sim, w);
    double th = 2.0 * ODO_PI * u01(w[0]);
    x[0] = p->Rh * cos(th); x[1] = p->Rh * sin(th); x[2] = u01(w[1]) * p->Hh - p->Hh_half;
    double gy, gz;
    draw(p->seed, ion, step, OD_RNG_SIDE_V, p->sim, w);
    gauss2(w[0], w[1], &gy, &gz);
    double us = u01(w[2]);
    double vn = tab_eval(p, OD_TAB_SIDE, us);
    double cx = x[0] / p->Rh, cy = x[1] / p->Rh;
    v[0] = -vn * cx + p->vT * gy * cy;
    v[1] = -vn * cy - p->vT * gy * cx;
    v[2] = (p->dist == OD_DIST_MAXWELLIAN) ? gz * p->vT + p->vfl : tab_eval(p, OD_TAB_VZ, us);
  }
}

static void collide(const odo_par* p, uint32_t ion, uint32_t step, double* v) {
  uint32_t w[4], g[4];
  if (p->coll == OD_COLL_PER_DOF) {
    /* opendust.py:869-873: collision = step(p_collision - uniform) per DOF */
    draw(p->seed, ion, step, OD_RNG_COLL_TEST, p->sim, w);
    int c0 = u01(w[0]) <= p->p_coll, c1 = u01(w[1]) <= p->p_coll, c2 = u01(w[2]) <= p->p_coll;
    if (c0 | c1 | c2) {
      double gx, gy, gz, dummy;
      draw(p->seed, ion, step, OD_RNG_COLL_GAUSS, p->sim, g);
      gauss2(g[0], g[1], &gx, &gy);
      gauss2(g[2], g[3], &gz, &dummy);
      if (c0) v[0] = p->vT * gx;
      if (c1) v[1] = p->vT * gy;
      if (c2) v[2] = p->vT * gz;
    }
  } else if (p->coll == OD_COLL_MFP) {
    /* null collision against the majorant speed vmax; an ion faster than vmax collides with
       its own probability 1 - exp(-|v| d_t / mfp) */
    /* the branch compares against the majorant rounded to FP32, as the CUDA path stores it */
    draw(p->seed, ion, step, OD_RNG_MFP_TEST, p->sim, w);
    double sp2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    double vm = (double)(float)p->vmax_mfp;
    double sp = sqrt(sp2);
    int hit = sp2 <= vm * vm ? (u01(w[0]) < p->Pmax_mfp && u01(w[1]) * vm < sp)
                             : u01(w[2]) < 1.0 - exp(-sp / p->mfp_h);
    if (hit) {
      double gx, gy, gz, dummy;
      draw(p->seed, ion, step, OD_RNG_MFP_GAUSS, p->sim, g);
      gauss2(g[0], g[1], &gx, &gy);
      gauss2(g[2], g[3], &gz, &dummy);
      v[0] = p->vT * gx; v[1] = p->vT * gy; v[2] = p->vT * gz;
    }
  }
}

/* ------------------------------------------------------------- host tail */
/* opendust.py:1117-1202: charge of grain g at step i from the charge at step i-1 */
static double charge_update(const od_config* c, const odo_par* p, int g, double q_prev, double dN) {
  double r = c->grain_r[g];
  double phi = p->k * q_prev / r;
  double gamma_e = c->n_inf * pow(c->T_e * c->k_B / ODO_PI / c->m_e / 2.0, 0.5) *
                   exp(-c->e * phi / c->T_e / c->k_B);
  double S = r * r * 4.0 * ODO_PI;
  if (c->grain_method[g] == OD_CHARGE_CONSISTENT) {
    double dq = dN * p->q_s + gamma_e * c->d_t * S * c->e;
    return q_prev + dq;
  }
  if (c->grain_method[g] == OD_CHARGE_OML) {
    double u = c->v_fl / c->v_T / sqrt(2.0);
    double chi = c->e * phi / c->T_n / c->k_B;
    double v_ti = c->v_T * sqrt(2.0);
    double gamma_i = c->n_inf * v_ti * u / 4.0 *
                     ((1.0 + 1.0 / (2.0 * u * 2) + chi / (u * u)) * erf(u) +
                      1.0 / u / sqrt(ODO_PI) * exp(-(u * u)));
    double dq = gamma_i * c->d_t * S * fabs(c->e) + gamma_e * c->d_t * S * c->e;
    return q_prev + dq;
  }
  return q_prev;
}

/* opendust.py:1258-1321: trap gradient at a grain (SI) */
static void out_domain_force(const od_config* c, const odo_par* p, double x, double y, double z,
                             double q, double* f) {
  const double* a = c->alpha;
  double L = c->r_D_e;
  double r = sqrt(x * x + y * y);
  double L2 = L * L, L4 = L2 * L2, L6 = L4 * L2, L8 = L4 * L4;
  double fR = (-2 * a[1] * r) / L2;
  fR += (-2 * a[3] * r * z * z - 4 * a[4] * r * r * r) / L4;
  fR += (-4 * a[6] * pow(r, 3) * z * z - 2 * a[7] * r * pow(z, 4) - 6 * a[8] * pow(r, 5)) / L6;
  fR += (-4 * a[10] * pow(r, 3) * pow(z, 4) - 6 * a[11] * pow(r, 5) * z * z -
         2 * a[12] * r * pow(z, 6) - 8 * a[13] * pow(r, 7)) / L8;
  fR *= p->k * q * p->q_s / L;
  double fH = (-2 * a[2] * z) / L2;
  fH += (-2 * a[3] * r * r * z - 4 * a[5] * pow(z, 3)) / L4;
  fH += (-2 * a[6] * pow(r, 4) * z - 4 * a[7] * r * r * pow(z, 3) - 6 * a[9] * pow(z, 5)) / L6;
  fH += (-4 * a[10] * pow(r, 4) * pow(z, 3) - 2 * a[11] * pow(r, 6) * z -
         6 * a[12] * r * r * pow(z, 5) - 8 * a[14] * pow(z, 7)) / L8;
  fH *= p->k * q * p->q_s / L;
  if (r == 0) { f[0] = 0; f[1] = 0; }
  else { f[0] = fR * x / r; f[1] = fR * y / r; }
  f[2] = fH;
}

/* ------------------------------------------------------------- public oracle API */
void odo_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
int odo_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* The device's cell-relative position state (od_set_state): per axis a cell index c on a grid
 * of side s (the smallest power of two not below 1/256 of max(R, H/2) in lambda) and the
 * offset v - c s rounded once to float; the state is c s + offset exactly. */
static double rel_side(const odo_par* p) {
  return ldexp(1.0, (int)ceil(log2(fmax(p->Rh, p->Hh / 2.0) / 256.0)));
}
static double rel_state(double v, double s) {
  double c = floor(v / s);
  c = c < -512.0 ? -512.0 : (c > 511.0 ? 511.0 : c);
  float o = (float)(v - c * s);
  if (o == (float)s && c < 511.0) { c += 1.0; o = 0.f; }
  return c * s + (double)o;
}

/* positions [m] -> lambda units. round32: 0 as given; 1 rounded to float (the snapshot calls'
 * representation); 2 the absolute float positions the device derives from its cell-relative
 * state (what its kernels read after od_set_state); 3 that state itself, exactly. */
static double hat(double v, int round32, double s) {
  if (round32 == 1) return (double)(float)v;
  if (round32 == 2) return (double)(float)rel_state(v, s);
  if (round32 == 3) return rel_state(v, s);
  return v;
}
static void to_hat(const odo_par* p, const double* pos, int64_t n, int round32, double* xh) {
  const double s = rel_side(p);
  for (int64_t i = 0; i < 3 * n; i++) xh[i] = hat(pos[i] / p->lam, round32, s);
}

/* ion–ion force [N] on each ion (the CustomNonbondedForce of opendust.py:471-485 alone) */
int odo_force_snapshot(const od_config* c, const double* pos, int64_t n, int round32, double* force) {
  odo_par* p = (odo_par*)malloc(sizeof(odo_par));
  if (!p || make_par(c, p)) { free(p); return 1; }
  double* xh = (double*)malloc(sizeof(double) * 3 * n);
  to_hat(p, pos, n, round32, xh);
  ionion(p, n, xh, force);
  double F = p->k * p->q_s * p->q_s / (p->lam * p->lam);
  for (int64_t i = 0; i < 3 * n; i++) force[i] *= F;
  free(xh); free(p);
  return 0;
}

int odo_collect_flags(const od_config* c, const double* pos, int64_t n, int round32,
                      int64_t* idx, int64_t cap, int64_t* count, int64_t* grain_counts) {
  odo_par* p = (odo_par*)malloc(sizeof(odo_par));
  if (!p || make_par(c, p)) { free(p); return 1; }
  int64_t cnt = 0;
  for (int g = 0; g < p->P; g++) grain_counts[g] = 0;
  for (int64_t i = 0; i < n; i++) {
    const double s = rel_side(p);
    double x = hat(pos[3 * i] / p->lam, round32, s), y = hat(pos[3 * i + 1] / p->lam, round32, s),
           z = hat(pos[3 * i + 2] / p->lam, round32, s);
    int b = flag_bits(p, x, y, z);
    if (b) {
      if (cnt < cap) idx[cnt] = i;
      cnt++;
      for (int g = 0; g < p->P; g++) if (b & (1 << g)) grain_counts[g]++;
    }
  }
  *count = cnt;
  free(p);
  return cnt > cap ? 7 : 0;
}

/* Trap-fit Monte-Carlo potential grid (opendust.py:499-523), lambda units. */
int odo_trap_potential(double Rh, double Hh, int n_r, int n_h, int64_t n_points, uint64_t seed,
                       double* pot) {
  double* px = (double*)malloc(sizeof(double) * 3 * n_points);
  if (!px) return 3;
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < n_points; q++) {
    uint32_t w[4];
    draw(seed, (uint32_t)q, 0, OD_RNG_TRAP, 0, w);
    double r = sqrt(u01(w[0]));
    double th = 2.0 * ODO_PI * u01(w[1]);
    px[3 * q] = Rh * r * cos(th);
    px[3 * q + 1] = Rh * r * sin(th);
    px[3 * q + 2] = Hh * u01(w[2]) - Hh / 2.0;
  }
  double dR = n_r > 1 ? Rh / (n_r - 1) : 0, dH = n_h > 1 ? (Hh / 2.0) / (n_h - 1) : 0;
#pragma omp parallel for schedule(dynamic, 1) collapse(2)
  for (int i = 0; i < n_r; i++)
    for (int j = 0; j < n_h; j++) {
      double gr = (i == n_r - 1) ? Rh : i * dR;
      double gh = (j == n_h - 1) ? Hh / 2.0 : j * dH;
      double s = 0;
      for (int64_t q = 0; q < n_points; q++) {
        double dx = gr - px[3 * q], dy = px[3 * q + 1], dz = gh - px[3 * q + 2];
        double r = sqrt(dx * dx + dy * dy + dz * dz);
        s += exp(-r) / (r + 0.001);
      }
      pot[i * n_h + j] = s / (double)n_points;
    }
  free(px);
  return 0;
}

/* One re-injection draw for tests: ion, step -> position [m] and velocity [m/s]. */
int odo_inject(const od_config* c, int64_t ion, int64_t step, double* x, double* v) {
  odo_par* p = (odo_par*)malloc(sizeof(odo_par));
  if (!p || make_par(c, p)) { free(p); return 1; }
  inject_one(p, (uint32_t)ion, (uint32_t)step, x, v);
  for (int d = 0; d < 3; d++) { x[d] *= p->lam; v[d] *= p->vunit; }
  free(p);
  return 0;
}

/* Run steps [first_step, first_step+nsteps) of the reference program from the given state.
 * pos [m] / vel [m/s] (n x 3) are updated in place; q_param[P] holds the charges the forces
 * use (q at the previous step) and is updated; per-step outputs (row i = step first_step+i):
 * q_out[P], f_orbit/f_collect/f_dust/f_field[P*3], n_inj (ions re-injected), dN[P].
 * round32: 1 rounds the initial positions and velocities to float; 2 takes the device's
 * cell-relative position state (to_hat mode 3) and float velocities.
 * rng_base: Philox step counter of step 0, for later windows whose random streams continue. */
int odo_run(const od_config* c, double* pos, double* vel, int64_t n, int round32,
            int64_t first_step, int64_t nsteps, int64_t rng_base, double* q_param, double* q_out,
            double* f_orbit, double* f_collect, double* f_dust, double* f_field,
            int64_t* n_inj, int64_t* dN_out) {
  odo_par* p = (odo_par*)malloc(sizeof(odo_par));
  if (!p || make_par(c, p)) { free(p); return 1; }
  const int P = p->P;
  double* x = (double*)malloc(sizeof(double) * 3 * n);
  double* v = (double*)malloc(sizeof(double) * 3 * n);
  double* a = (double*)malloc(sizeof(double) * 3 * n);
  int* fl = (int*)malloc(sizeof(int) * n);
  to_hat(p, pos, n, round32 == 2 ? 3 : round32, x);
  for (int64_t i = 0; i < 3 * n; i++) {
    double vv = vel[i] / p->vunit;
    v[i] = round32 ? (double)(float)vv : vv;
  }
  double q[OD_MAX_GRAINS];
  for (int g = 0; g < P; g++) q[g] = q_param[g];
  /* force interval k > 1 (od_config.force_every): stored ion–ion sums G, evaluated at the
   * start and at the end of steps with step % k == k - 1 */
  const int kf = c->force_every > 1 ? c->force_every : 1;
  double* G = NULL;
  int64_t* inj = NULL;
  double* xold = NULL;
  if (kf > 1) {
    G = (double*)malloc(sizeof(double) * 3 * n);
    inj = (int64_t*)malloc(sizeof(int64_t) * n);
    xold = (double*)malloc(sizeof(double) * 3 * n);
    ionion(p, n, x, G);
  }

  for (int64_t s = 0; s < nsteps; s++) {
    int64_t step = first_step + s;        /* step of the window: step 0 keeps the charges */
    uint32_t st = (uint32_t)(rng_base + step); /* Philox step counter (continues across windows) */
    if (p->coll != OD_COLL_NONE)
      for (int64_t i = 0; i < n; i++) collide(p, (uint32_t)i, st, v + 3 * i);
    if (kf > 1) {
      /* impulse multiple time stepping: kicks of weight k next to an evaluation */
      accel_mts(p, c->alpha, n, x, q, G, step % kf == 0 ? (double)kf : 0.0, a);
      for (int64_t i = 0; i < 3 * n; i++) { v[i] += 0.5 * a[i]; x[i] += v[i]; }
      int ev = step % kf == kf - 1;
      if (ev) ionion(p, n, x, G);
      accel_mts(p, c->alpha, n, x, q, G, ev ? (double)kf : 0.0, a);
      for (int64_t i = 0; i < 3 * n; i++) v[i] += 0.5 * a[i];
    } else {
    /* addUpdateContextState; v += 0.5 dt f/m; x += dt v; v += 0.5 dt f/m (opendust.py:864-877) */
    accel_total(p, c->alpha, n, x, q, a);
    for (int64_t i = 0; i < 3 * n; i++) { v[i] += 0.5 * a[i]; x[i] += v[i]; }
    accel_total(p, c->alpha, n, x, q, a);
    for (int64_t i = 0; i < 3 * n; i++) v[i] += 0.5 * a[i];
    }
    /* flags and collection sums (opendust.py:894-921) */
    double dN[OD_MAX_GRAINS] = {0}, M[OD_MAX_GRAINS][3];
    memset(M, 0, sizeof(M));
    int64_t ninj = 0;
    for (int64_t i = 0; i < n; i++) {
      fl[i] = flag_bits(p, x[3 * i], x[3 * i + 1], x[3 * i + 2]);
      for (int g = 0; g < P; g++)
        if (fl[i] & (1 << g)) {
          dN[g] += 1.0;
          M[g][0] += v[3 * i]; M[g][1] += v[3 * i + 1]; M[g][2] += v[3 * i + 2];
        }
    }
    /* re-injection (opendust.py:923-975) */
    if (p->dist == OD_DIST_MATTHEWS) {
      /* chains/matthews.py:653-682: past |z| = H/2 or inside a grain -> top face; past the side
       * wall -> radial velocity reversed with the normal of the position before re-injection */
      int grains = (1 << P) - 1;
      for (int64_t i = 0; i < n; i++) {
        if (!fl[i]) continue;
        double xo = x[3 * i], yo = x[3 * i + 1];
        if (fl[i] & (grains | (1 << 29))) inject_one(p, (uint32_t)i, st, x + 3 * i, v + 3 * i);
        if (fl[i] & (1 << 30)) {
          double rr = sqrt(xo * xo + yo * yo), nx = xo / rr, ny = yo / rr;
          double vx = v[3 * i], vy = v[3 * i + 1];
          double vn = vx * nx + vy * ny, vt = vx * ny - vy * nx;
          v[3 * i] = -vn * nx + vt * ny;
          v[3 * i + 1] = -vn * ny - vt * nx;
        }
        ninj++;
      }
    } else {
      for (int64_t i = 0; i < n; i++)
        if (fl[i]) {
          if (kf > 1) {
            inj[ninj] = i;
            memcpy(xold + 3 * ninj, x + 3 * i, 3 * sizeof(double));
          }
          inject_one(p, (uint32_t)i, st, x + 3 * i, v + 3 * i);
          ninj++;
        }
    }
    if (kf > 1) mts_follow_injection(p, n, x, fl, inj, xold, ninj, G);
    /* orbit sums on the re-injected positions (opendust.py:977-1037) */
    double S[OD_MAX_GRAINS][3];
    memset(S, 0, sizeof(S));
    for (int g = 0; g < P; g++) {
      double sx = 0, sy = 0, sz = 0;
#pragma omp parallel for reduction(+ : sx, sy, sz) schedule(static)
      for (int64_t i = 0; i < n; i++) {
        double dx = p->gx[g] - x[3 * i], dy = p->gy[g] - x[3 * i + 1], dz = p->gz[g] - x[3 * i + 2];
        double r = sqrt(dx * dx + dy * dy + dz * dz);
        double e = exp(-r);
        double t = e / (r * r * r) + e / (r * r);
        sx += dx * t; sy += dy * t; sz += dz * t;
      }
      S[g][0] = sx; S[g][1] = sy; S[g][2] = sz;
    }
    /* host tail (opendust.py:1117-1383) */
    double qn[OD_MAX_GRAINS];
    for (int g = 0; g < P; g++) qn[g] = step > 0 ? charge_update(c, p, g, q[g], dN[g]) : q[g];
    for (int g = 0; g < P; g++) {
      double fd[3] = {0, 0, 0};
      for (int j = 0; j < P; j++) {
        if (j == g) continue;
        double dx = c->grain_x[g] - c->grain_x[j], dy = c->grain_y[g] - c->grain_y[j],
               dz = c->grain_z[g] - c->grain_z[j];
        double r = sqrt(dx * dx + dy * dy + dz * dz);
        double kk = p->k * qn[g] * qn[j] / (r * r * r);
        fd[0] += kk * dx; fd[1] += kk * dy; fd[2] += kk * dz;
      }
      double fo[3] = {0, 0, 0};
      if (p->trap_kind == OD_TRAP_POLY)
        out_domain_force(c, p, c->grain_x[g], c->grain_y[g], c->grain_z[g], qn[g], fo);
      else if (p->trap_kind == OD_TRAP_TABLE)
        for (int d = 0; d < 3; d++) fo[d] = qn[g] * p->gout[g][d];
      double so = qn[g] * p->k * p->q_s / (p->lam * p->lam);
      double sc = p->vunit * p->m_s / c->d_t;
      if (q_out) q_out[s * P + g] = qn[g];
      for (int d = 0; d < 3; d++) {
        if (f_orbit) f_orbit[(s * P + g) * 3 + d] = S[g][d] * so + fo[d];
        if (f_collect) f_collect[(s * P + g) * 3 + d] = M[g][d] * sc;
        if (f_dust) f_dust[(s * P + g) * 3 + d] = fd[d];
        if (f_field) f_field[(s * P + g) * 3 + d] = d == 2 ? qn[g] * p->gfield[g] : 0.0;
      }
      if (dN_out) dN_out[s * P + g] = (int64_t)dN[g];
    }
    if (n_inj) n_inj[s] = ninj;
    for (int g = 0; g < P; g++) q[g] = qn[g];
  }
  for (int64_t i = 0; i < 3 * n; i++) { pos[i] = x[i] * p->lam; vel[i] = v[i] * p->vunit; }
  for (int g = 0; g < P; g++) q_param[g] = q[g];
  free(x); free(v); free(a); free(fl); free(p);
  free(G); free(inj); free(xold);
  return 0;
}

/* Total acceleration (ion–ion + grains + trap + field) on every ion, in m/s^2, with grain
 * charges q[P] [C]; the force the reference's integrator divides by m (opendust.py:864-877). */
int odo_accel(const od_config* c, const double* pos, int64_t n, int round32, const double* q,
              double* acc) {
  odo_par* p = (odo_par*)malloc(sizeof(odo_par));
  if (!p || make_par(c, p)) { free(p); return 1; }
  double* xh = (double*)malloc(sizeof(double) * 3 * n);
  to_hat(p, pos, n, round32, xh);
  accel_total(p, c->alpha, n, xh, q, acc);
  double s = p->lam / (p->dt * p->dt);
  for (int64_t i = 0; i < 3 * n; i++) acc[i] *= s;
  free(xh); free(p);
  return 0;
}

/* Ion–ion force [N] on the m target ions idx[] only (all n sources). */
int odo_force_targets(const od_config* c, const double* pos, int64_t n, int round32,
                      const int64_t* idx, int64_t m, double* force) {
  odo_par* p = (odo_par*)malloc(sizeof(odo_par));
  if (!p || make_par(c, p)) { free(p); return 1; }
  double* xh = (double*)malloc(sizeof(double) * 3 * n);
  to_hat(p, pos, n, round32, xh);
  double F = p->k * p->q_s * p->q_s / (p->lam * p->lam);
  odo_cells cl;
  if (p->method == OD_FORCE_CUTOFF && n > 4096 && !cells_build(p, n, xh, &cl)) {
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t t = 0; t < m; t++) {
      double g[3];
      ionion_cells_one(p, &cl, xh, idx[t], g);
      force[3 * t] = F * g[0]; force[3 * t + 1] = F * g[1]; force[3 * t + 2] = F * g[2];
    }
    cells_free(&cl);
    free(xh); free(p);
    return 0;
  }
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t t = 0; t < m; t++) {
    int64_t i = idx[t];
    double xi = xh[3 * i], yi = xh[3 * i + 1], zi = xh[3 * i + 2];
    double gx = 0, gy = 0, gz = 0;
    for (int64_t j = 0; j < n; j++) {
      if (j == i) continue;
      double dx = xi - xh[3 * j], dy = yi - xh[3 * j + 1], dz = zi - xh[3 * j + 2];
      double cc = pair_factor(p, dx * dx + dy * dy + dz * dz);
      gx += cc * dx; gy += cc * dy; gz += cc * dz;
    }
    force[3 * t] = F * gx; force[3 * t + 1] = F * gy; force[3 * t + 2] = F * gz;
  }
  free(xh); free(p);
  return 0;
}

/* Screened potential sum over the ions at grid points (r_i, 0, z_j) in units of r_D_e
 * (chains/matthews.py:397-421): pot[j * n_r + i] = sum_ions exp(-r)/(r + r_0). */
int odo_ion_potential_grid(const od_config* c, const double* pos, int64_t n, int round32,
                           const double* gr, const double* gz, int n_r, int n_z, double* pot) {
  odo_par* p = (odo_par*)malloc(sizeof(odo_par));
  if (!p || make_par(c, p)) { free(p); return 1; }
  double* xh = (double*)malloc(sizeof(double) * 3 * n);
  to_hat(p, pos, n, round32, xh);
#pragma omp parallel for schedule(dynamic, 1)
  for (int q = 0; q < n_r * n_z; q++) {
    double gx = gr[q % n_r], gzz = gz[q / n_r], acc = 0.0;
    for (int64_t i = 0; i < n; i++) {
      double dx = gx - xh[3 * i], dy = -xh[3 * i + 1], dz = gzz - xh[3 * i + 2];
      double r = sqrt(dx * dx + dy * dy + dz * dz);
      acc += exp(-r) / (r + p->rho0);
    }
    pot[q] = acc;
  }
  free(xh); free(p);
  return 0;
}
