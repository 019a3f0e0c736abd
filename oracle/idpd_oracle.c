/*
 * CPU oracle for the implicit_dpd short-range particle step (see
 * idpd_oracle.h). TEST INFRASTRUCTURE ONLY: tests, smoke() and the bench's
 * CPU-baseline leg call it as the checker; the product never does.
 *
 * Each function restates the reference algorithm named in its comment, in the
 * reference's FP64 operation order. Build with -ffp-contract=off.
 */
#include "idpd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* Compile-time constants of parameter.hpp:189-205. */
#define ORC_TEMPERA 1.0
#define ORC_ALL_UNIT 4u
#define ORC_BOND_LENG 0.5
#define ORC_ARC 0.9
#define ORC_REO 1.4
#define ORC_SEARCH_RAD 1.2
#define ORC_RN_C 1.2
#define ORC_CM_CORR 100u

/* ------------------------------------------------------------------ Saru */
/* saruprng.hpp:239-255 (3-seed constructor), :173-177 (LCG and Weyl
 * constants), :199-202 (one Weyl step), :322-333 (output mix). */
typedef struct {
  uint32_t lcg, weyl;
} orc_saru;

static inline uint32_t asr(uint32_t x, int s) { return (uint32_t)((int32_t)x >> s); }

static void saru_seed3(orc_saru* r, uint32_t a, uint32_t b, uint32_t c) {
  c ^= (a << 7) ^ (b >> 6);
  b += (a >> 4) ^ (c >> 15);
  a ^= (b << 9) + (c << 8);
  c ^= 0xA5366B4Du * ((b >> 11) ^ (a << 1));
  b += 0x72BE1579u * ((a << 4) ^ (c >> 16));
  a ^= 0x3F38A6EDu * ((c >> 5) ^ asr(b, 22));
  b += a * c;
  a += c ^ (b >> 2);
  b ^= asr(b, 17);
  r->lcg = 0x79dedea3u * (a ^ asr(a, 14));
  r->weyl = (r->lcg + b) ^ asr(r->lcg, 8);
  r->lcg = r->lcg + (r->weyl * (r->weyl ^ 0xdddf97f5u));
  r->weyl = 0xABCB96F7u + (r->weyl >> 1);
}

static inline uint32_t saru_next(orc_saru* r) {
  r->lcg = 0x4beb5d59u * r->lcg + 0x2600e1f7u;
  r->weyl = r->weyl + 0x8009d14bu + (asr(r->weyl, 31) & 0xda879addu);
  uint32_t v = (r->lcg ^ (r->lcg >> 26)) + r->weyl;
  return (v ^ (v >> 20)) * 0x6957f5a7u;
}

/* saruprng.hpp:427-432: (int(u >> 1) + 0.5) / 2^31 */
static inline double saru_uni_open(orc_saru* r) {
  return ((double)(int32_t)(saru_next(r) >> 1) + 0.5) * (1.0 / 2147483648.0);
}

/* saruprng.hpp:442-445. The first draw feeds the logarithm, the second the
 * cosine: the order the reference's g++ build evaluates the two operands in
 * (pinned by tests/golden/saru_*). */
static inline double saru_nrml(orc_saru* r) {
  const double u1 = saru_uni_open(r);
  const double u2 = saru_uni_open(r);
  return sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
}

void orc_saru_u32(uint32_t s1, uint32_t s2, uint32_t s3, int32_t count, uint32_t* out) {
  orc_saru r;
  saru_seed3(&r, s1, s2, s3);
  for (int32_t k = 0; k < count; k++) out[k] = saru_next(&r);
}

double orc_saru_nrml(uint32_t s1, uint32_t s2, uint32_t s3) {
  orc_saru r;
  saru_seed3(&r, s1, s2, s3);
  return saru_nrml(&r);
}

/* --------------------------------------------------------------- MT19937 */
/* Matsumoto & Nishimura (1998), mt19937ar: init_genrand, genrand_int32,
 * genrand_real1 = u / (2^32 - 1), genrand_real3 = (u + 0.5) / 2^32. */
void orc_mt_seed(orc_mt* g, uint32_t seed) {
  g->mt[0] = seed;
  for (int i = 1; i < 624; i++) g->mt[i] = 1812433253u * (g->mt[i - 1] ^ (g->mt[i - 1] >> 30)) + (uint32_t)i;
  g->mti = 624;
}

uint32_t orc_mt_u32(orc_mt* g) {
  if (g->mti >= 624) {
    for (int k = 0; k < 624; k++) {
      const uint32_t y = (g->mt[k] & 0x80000000u) | (g->mt[(k + 1) % 624] & 0x7fffffffu);
      g->mt[k] = g->mt[(k + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    g->mti = 0;
  }
  uint32_t y = g->mt[g->mti++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

double orc_mt_real1(orc_mt* g) { return orc_mt_u32(g) * (1.0 / 4294967295.0); }
double orc_mt_real3(orc_mt* g) { return (((double)orc_mt_u32(g)) + 0.5) * (1.0 / 4294967296.0); }

void orc_mt_draws(uint32_t seed, int32_t n, uint32_t* out) {
  orc_mt g;
  orc_mt_seed(&g, seed);
  for (int32_t i = 0; i < n; i++) out[i] = orc_mt_u32(&g);
}

/* ------------------------------------------------------- CalcInterCoef */
/* parameter.hpp:29-38 (FillUpperTri), :138-186 (CalcInterCoef), :139-144
 * (harmonic-mean gamma when cf_r < 0). */
int orc_derive_params(const idpd_run_param* rp, idpd_params* out) {
  memset(out, 0, sizeof(*out));
  double cf_c[3][3], cf_g[3][3], cf_r[3][3], cf_m[3][3][3];
  const double kappa = rp->kappa, rho_co = rp->rho_co, chi = rp->chi;
  cf_c[1][1] = -2.0 * (kappa + 3.0) / rho_co;
  cf_c[0][0] = cf_c[2][2] = rp->vbb;
  cf_c[0][1] = cf_c[1][0] = chi / (rho_co) + 0.5 * (cf_c[0][0] + cf_c[1][1]);
  cf_c[2][1] = cf_c[1][2] = cf_c[0][1];
  cf_c[2][0] = cf_c[0][2] = cf_c[0][0];
  const double m0 = 1.5 * (kappa + 2.0) / (rho_co * rho_co);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      for (int k = 0; k < 3; k++) cf_m[i][j][k] = m0;
  cf_m[0][0][0] = 0.0;
  cf_m[2][2][2] = 0.0;
  int cnt = 0;
  for (int i = 0; i < 3; i++)
    for (int j = i; j < 3; j++) cf_r[i][j] = rp->cf_r_upper[cnt++];
  for (int i = 0; i < 3; i++)
    for (int j = i + 1; j < 3; j++) cf_r[j][i] = cf_r[i][j];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) cf_g[i][j] = 0.5 * cf_r[i][j] * cf_r[i][j] / ORC_TEMPERA;
  for (int i = 0; i < 3; i++)
    for (int j = i + 1; j < 3; j++)
      if (cf_r[i][j] < 0.0) {
        cf_g[i][j] = cf_g[j][i] = 2.0 / ((1.0 / cf_g[i][i]) + (1.0 / cf_g[j][j]));
        cf_r[i][j] = cf_r[j][i] = sqrt(2.0 * cf_g[i][j] * ORC_TEMPERA);
      }
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) cf_r[i][j] /= sqrt(rp->dt);
  const double reo3 = ORC_REO * ORC_REO * ORC_REO;
  const double mol_energy = reo3 / (double)(ORC_ALL_UNIT * ORC_ALL_UNIT);
  const double arc = ORC_ARC;
  const double arc5 = arc * arc * arc * arc * arc;
  const double w2 = -45.0 / ((arc5 * (2.0 * arc - 3.0) + (3.0 * arc - 2.0)) * M_PI);
  const double w3 = 15.0 / M_PI;
  const double dens_unit = ((ORC_REO * ORC_REO * ORC_REO * 15.0) / (2.0 * M_PI * (double)ORC_ALL_UNIT));
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) cf_c[i][j] *= mol_energy * w2;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      for (int k = 0; k < 3; k++) cf_m[i][j][k] *= mol_energy * (2.0 / 3.0) * w3 * dens_unit;
  memcpy(out->cf_c, cf_c, sizeof(cf_c));
  memcpy(out->cf_g, cf_g, sizeof(cf_g));
  memcpy(out->cf_r, cf_r, sizeof(cf_r));
  memcpy(out->cf_m, cf_m, sizeof(cf_m));
  out->cf_s = rp->cf_s;
  out->cf_b = rp->cf_b;
  out->cf_b_rigid = rp->cf_b_rigid;
  for (int d = 0; d < 3; d++) out->box[d] = rp->box[d];
  out->dt = rp->dt;
  return 0;
}

/* ----------------------------------------------------------------- cells */
int32_t orc_cells(int32_t n, const double* pos, const double* box, double r_cell, int32_t* nc,
                  int32_t* cell_of, int32_t* start, int32_t* members) {
  double inv[3];
  for (int d = 0; d < 3; d++) {
    nc[d] = (int32_t)(box[d] / r_cell);
    if (nc[d] < 3) return -1;
    inv[d] = nc[d] / box[d];
  }
  const int32_t ncell = nc[0] * nc[1] * nc[2];
  memset(start, 0, sizeof(int32_t) * (ncell + 1));
  for (int32_t i = 0; i < n; i++) {
    int32_t c[3];
    for (int d = 0; d < 3; d++) {
      c[d] = (int32_t)(pos[3 * i + d] * inv[d]);
      if (c[d] < 0) c[d] = 0;
      if (c[d] >= nc[d]) c[d] = nc[d] - 1;
    }
    cell_of[i] = (c[2] * nc[1] + c[1]) * nc[0] + c[0];
    start[cell_of[i] + 1]++;
  }
  for (int32_t c = 0; c < ncell; c++) start[c + 1] += start[c];
  int32_t* fill = (int32_t*)malloc(sizeof(int32_t) * (ncell > 0 ? ncell : 1));
  memcpy(fill, start, sizeof(int32_t) * ncell);
  for (int32_t i = 0; i < n; i++) members[fill[cell_of[i]]++] = i;
  free(fill);
  return ncell;
}

typedef struct {
  int32_t nc[3];
  int32_t ncell;
  int32_t *cell_of, *start, *members;
} orc_grid;

static int grid_build(orc_grid* g, int32_t n, const double* pos, const double* box) {
  int32_t nc[3];
  for (int d = 0; d < 3; d++) nc[d] = (int32_t)(box[d] / ORC_SEARCH_RAD);
  if (nc[0] < 3 || nc[1] < 3 || nc[2] < 3) return -1;
  g->ncell = nc[0] * nc[1] * nc[2];
  g->cell_of = (int32_t*)malloc(sizeof(int32_t) * (n > 0 ? n : 1));
  g->start = (int32_t*)malloc(sizeof(int32_t) * (g->ncell + 1));
  g->members = (int32_t*)malloc(sizeof(int32_t) * (n > 0 ? n : 1));
  orc_cells(n, pos, box, ORC_SEARCH_RAD, g->nc, g->cell_of, g->start, g->members);
  return 0;
}

static void grid_free(orc_grid* g) {
  free(g->cell_of);
  free(g->start);
  free(g->members);
}

/* Neighbour cell (cx+dx, ...) wrapped, and the periodic image shift n*L that
 * takes its particles next to cell (cx, cy, cz). */
static inline int32_t nbr_cell(const orc_grid* g, const double* box, int cx, int cy, int cz, int dx,
                               int dy, int dz, double* sh) {
  const int q[3] = {cx + dx, cy + dy, cz + dz};
  int w[3];
  for (int d = 0; d < 3; d++) {
    const int s = q[d] < 0 ? -1 : (q[d] >= g->nc[d] ? 1 : 0);
    w[d] = q[d] - s * g->nc[d];
    sh[d] = (double)s * box[d];
  }
  return (w[2] * g->nc[1] + w[1]) * g->nc[0] + w[0];
}

/* --------------------------------------------------------------- pass 1 */
/* CalcDensity::operator() (nbdf_calculator.hpp:11-60) and
 * FPDPD::copyFromForce(RESULT::Density) (ptcl_class.hpp:53-57). */
int orc_density(const idpd_params* p, int32_t n, const double* pos, const uint32_t* prop,
                double* dens, double* nei_cm, uint32_t* nei_cnt, int32_t nthreads) {
  orc_grid g;
  if (grid_build(&g, n, pos, p->box) != 0) return -1;
  const double rn_c2 = ORC_RN_C * ORC_RN_C;
  const int warren = p->form == IDPD_FORM_WARREN;
  const double rd = p->warren_rd;
  const double rd2 = rd * rd;
  const double wn = 15.0 / (2.0 * M_PI * rd * rd * rd);
  const double dcut2 = warren ? rd2 : 1.0;
  (void)nthreads;
#pragma omp parallel for schedule(dynamic, 8) num_threads(nthreads > 0 ? nthreads : 1)
  for (int32_t c = 0; c < g.ncell; c++) {
    const int cx = c % g.nc[0], cy = (c / g.nc[0]) % g.nc[1], cz = c / (g.nc[0] * g.nc[1]);
    for (int32_t m = g.start[c]; m < g.start[c + 1]; m++) {
      const int32_t i = g.members[m];
      const double rix = pos[3 * i], riy = pos[3 * i + 1], riz = pos[3 * i + 2];
      double d_sum[3] = {0.0, 0.0, 0.0};
      double hb[3] = {0.0, 0.0, 0.0}, hl[3] = {rix, riy, riz};
      uint32_t cb = 0, cl = 1;
      for (int dz = -1; dz <= 1; dz++)
        for (int dy = -1; dy <= 1; dy++)
          for (int dx = -1; dx <= 1; dx++) {
            double sh[3];
            const int32_t cj = nbr_cell(&g, p->box, cx, cy, cz, dx, dy, dz, sh);
            for (int32_t mj = g.start[cj]; mj < g.start[cj + 1]; mj++) {
              const int32_t j = g.members[mj];
              const double pjx = pos[3 * j] + sh[0], pjy = pos[3 * j + 1] + sh[1],
                           pjz = pos[3 * j + 2] + sh[2];
              const double ddx = rix - pjx, ddy = riy - pjy, ddz = riz - pjz;
              const double dr2 = ddx * ddx + ddy * ddy + ddz * ddz;
              if (dr2 < rn_c2 && dr2 != 0.0) {
                const uint32_t pj = prop[j];
                if (pj == IDPD_HYPHOB) {
                  hb[0] += pjx;
                  hb[1] += pjy;
                  hb[2] += pjz;
                  cb++;
                }
                if (dr2 < 1.0) {
                  const double dr = sqrt(dr2);
                  if (!warren) {
                    d_sum[pj] += (1.0 - dr) * (1.0 - dr);
                  } else if (dr2 < dcut2) {
                    const double t = 1.0 - dr / rd;
                    d_sum[pj] += wn * (t * t);
                  }
                  if (pj == IDPD_HYPHIL) {
                    hl[0] += pjx;
                    hl[1] += pjy;
                    hl[2] += pjz;
                    cl++;
                  }
                }
              }
            }
          }
      for (int k = 0; k < 3; k++) dens[3 * i + k] = 0.0 + d_sum[k];
      if (nei_cm) {
        for (int d = 0; d < 3; d++) {
          nei_cm[6 * i + d] = (0.0 + hl[d]) / (double)cl;
          nei_cm[6 * i + 3 + d] = (0.0 + hb[d]) / (double)cb;
        }
      }
      if (nei_cnt) {
        nei_cnt[2 * i] = cl;
        nei_cnt[2 * i + 1] = cb;
      }
    }
  }
  grid_free(&g);
  return 0;
}

/* Ordered pairs within the cutoff (r < 1, i != j): the pair set of
 * CalcForceEpEpDPD (nbdf_calculator.hpp:84-88) counted over the image-shifted
 * cells, for the pairs-per-particle figure of the CPU baseline. */
int64_t orc_pair_count(const idpd_params* p, int32_t n, const double* pos, int32_t nthreads) {
  orc_grid g;
  if (grid_build(&g, n, pos, p->box) != 0) return -1;
  int64_t total = 0;
  (void)nthreads;
#pragma omp parallel for schedule(dynamic, 8) reduction(+ : total) num_threads(nthreads > 0 ? nthreads : 1)
  for (int32_t c = 0; c < g.ncell; c++) {
    const int cx = c % g.nc[0], cy = (c / g.nc[0]) % g.nc[1], cz = c / (g.nc[0] * g.nc[1]);
    for (int32_t m = g.start[c]; m < g.start[c + 1]; m++) {
      const int32_t i = g.members[m];
      for (int dz = -1; dz <= 1; dz++)
        for (int dy = -1; dy <= 1; dy++)
          for (int dx = -1; dx <= 1; dx++) {
            double sh[3];
            const int32_t cj = nbr_cell(&g, p->box, cx, cy, cz, dx, dy, dz, sh);
            for (int32_t mj = g.start[cj]; mj < g.start[cj + 1]; mj++) {
              const int32_t j = g.members[mj];
              if (j == i) continue;
              const double ddx = pos[3 * i] - (pos[3 * j] + sh[0]),
                           ddy = pos[3 * i + 1] - (pos[3 * j + 1] + sh[1]),
                           ddz = pos[3 * i + 2] - (pos[3 * j + 2] + sh[2]);
              total += (ddx * ddx + ddy * ddy + ddz * ddz) < 1.0;
            }
          }
    }
  }
  grid_free(&g);
  return total;
}

/* ------------------------------------------------- precursor conversion */
/* Saru 3-seed constructor and u32 (saruprng.hpp:239-255, 322-333) keyed on
 * (id, time, seed); the pair test of pass 1 (nbdf_calculator.hpp:27-29). */
int64_t orc_precursor(const idpd_params* p, int32_t n, const double* pos, const uint32_t* id,
                      uint32_t* prop, uint32_t time, uint32_t from, uint32_t near, uint32_t to,
                      uint32_t threshold, uint32_t seed, int32_t nthreads) {
  orc_grid g;
  if (grid_build(&g, n, pos, p->box) != 0) return -1;
  uint8_t* conv = (uint8_t*)calloc(n > 0 ? n : 1, 1);
  (void)nthreads;
#pragma omp parallel for schedule(dynamic, 8) num_threads(nthreads > 0 ? nthreads : 1)
  for (int32_t c = 0; c < g.ncell; c++) {
    const int cx = c % g.nc[0], cy = (c / g.nc[0]) % g.nc[1], cz = c / (g.nc[0] * g.nc[1]);
    for (int32_t m = g.start[c]; m < g.start[c + 1]; m++) {
      const int32_t i = g.members[m];
      if (prop[i] != from) continue;
      const double rix = pos[3 * i], riy = pos[3 * i + 1], riz = pos[3 * i + 2];
      int found = 0;
      for (int dz = -1; dz <= 1 && !found; dz++)
        for (int dy = -1; dy <= 1 && !found; dy++)
          for (int dx = -1; dx <= 1 && !found; dx++) {
            double sh[3];
            const int32_t cj = nbr_cell(&g, p->box, cx, cy, cz, dx, dy, dz, sh);
            for (int32_t mj = g.start[cj]; mj < g.start[cj + 1]; mj++) {
              const int32_t j = g.members[mj];
              if (j == i || prop[j] != near) continue;
              const double ddx = rix - (pos[3 * j] + sh[0]), ddy = riy - (pos[3 * j + 1] + sh[1]),
                           ddz = riz - (pos[3 * j + 2] + sh[2]);
              if (ddx * ddx + ddy * ddy + ddz * ddz < 1.0) {
                found = 1;
                break;
              }
            }
          }
      if (found) {
        orc_saru r;
        saru_seed3(&r, id[i], time, seed);
        conv[i] = saru_next(&r) < threshold;
      }
    }
  }
  int64_t count = 0;
  for (int32_t i = 0; i < n; i++)
    if (conv[i]) {
      prop[i] = to;
      count++;
    }
  free(conv);
  grid_free(&g);
  return count;
}

/* --------------------------------------------------------------- pass 2 */
/* CalcForceEpEpDPD::operator() (nbdf_calculator.hpp:63-145) and
 * FPDPD::copyFromForce(RESULT::ForceDPD) (ptcl_class.hpp:48-51). */
int orc_force(const idpd_params* p, int32_t n, const double* pos, const double* vel,
              const uint32_t* id, const uint32_t* prop, const double* dens, double* acc,
              double* press, int32_t nthreads) {
  orc_grid g;
  if (grid_build(&g, n, pos, p->box) != 0) return -1;
  const uint32_t seed = p->seed + p->time;
  const int form = p->form;
  const double rd = p->warren_rd;
  (void)nthreads;
#pragma omp parallel for schedule(dynamic, 8) num_threads(nthreads > 0 ? nthreads : 1)
  for (int32_t c = 0; c < g.ncell; c++) {
    const int cx = c % g.nc[0], cy = (c / g.nc[0]) % g.nc[1], cz = c / (g.nc[0] * g.nc[1]);
    for (int32_t m = g.start[c]; m < g.start[c + 1]; m++) {
      const int32_t i = g.members[m];
      const double rix = pos[3 * i], riy = pos[3 * i + 1], riz = pos[3 * i + 2];
      const double vix = vel[3 * i], viy = vel[3 * i + 1], viz = vel[3 * i + 2];
      const uint32_t idi = id[i], pi = prop[i];
      const double* densi = dens + 3 * i;
      double fs[3] = {0.0, 0.0, 0.0}, ps[3] = {0.0, 0.0, 0.0};
      for (int dz = -1; dz <= 1; dz++)
        for (int dy = -1; dy <= 1; dy++)
          for (int dx = -1; dx <= 1; dx++) {
            double sh[3];
            const int32_t cj = nbr_cell(&g, p->box, cx, cy, cz, dx, dy, dz, sh);
            for (int32_t mj = g.start[cj]; mj < g.start[cj + 1]; mj++) {
              const int32_t j = g.members[mj];
              if (idi == id[j]) continue;
              const double ddx = rix - (pos[3 * j] + sh[0]);
              const double ddy = riy - (pos[3 * j + 1] + sh[1]);
              const double ddz = riz - (pos[3 * j + 2] + sh[2]);
              const double dr2 = ddx * ddx + ddy * ddy + ddz * ddz;
              if (dr2 < 1.0) {
                const double dvx = vix - vel[3 * j], dvy = viy - vel[3 * j + 1],
                             dvz = viz - vel[3 * j + 2];
                const uint32_t idj = id[j];
                double densij[3];
                for (int k = 0; k < 3; k++) densij[k] = densi[k] + dens[3 * j + k];
                uint32_t mi = idi, mj2 = idj;
                if (idi > idj) {
                  mi = idj;
                  mj2 = idi;
                }
                orc_saru s;
                saru_seed3(&s, mi, mj2, seed);
                const double rnd = saru_nrml(&s);
                const double dr = sqrt(dr2);
                const double inv_dr = 1.0 / dr;
                const uint32_t pj = prop[j];
                const double rc_m_dr = 1.0 - dr;
                double cons;
                if (form == IDPD_FORM_PAIRWISE) {
                  const double cf_pair = 25.0, cf_mbd = 0.0;
                  cons = (cf_pair + cf_mbd) * rc_m_dr;
                } else if (form == IDPD_FORM_WARREN) {
                  const double rho = densij[0] + densij[1] + densij[2];
                  const double wb = (dr < rd) ? (1.0 - dr / rd) : 0.0;
                  cons = p->warren_a * rc_m_dr + p->warren_b * rho * wb;
                } else {
                  const double cf_pair = p->cf_c[pi][pj] * (dr - ORC_ARC) * (double)(dr >= ORC_ARC);
                  double cf_mbd = 0.0;
                  for (int k = 0; k < 3; k++) cf_mbd += p->cf_m[pi][pj][k] * densij[k];
                  cons = (cf_pair + cf_mbd) * rc_m_dr;
                }
                const double wrij = rc_m_dr;
                const double sq_wrij = sqrt(wrij);
                const double drij_dvij = ddx * dvx + ddy * dvy + ddz * dvz;
                const double all_cf = (cons + p->cf_r[pi][pj] * sq_wrij * rnd -
                                       p->cf_g[pi][pj] * wrij * drij_dvij * inv_dr) *
                                      inv_dr;
                const double dfx = all_cf * ddx, dfy = all_cf * ddy, dfz = all_cf * ddz;
                fs[0] += dfx;
                fs[1] += dfy;
                fs[2] += dfz;
                ps[0] += dfx * ddx;
                ps[1] += dfy * ddy;
                ps[2] += dfz * ddz;
              }
            }
          }
      for (int d = 0; d < 3; d++) {
        acc[3 * i + d] = 0.0 + fs[d];
        if (press) press[3 * i + d] = 0.0 + ps[d];
      }
    }
  }
  grid_free(&g);
  return 0;
}

/* --------------------------------------------------------------- bonded */
/* ForceBonded::MakeGlobalBondedList (bdf_calculator.hpp:61-88). */
int orc_build_topology(int32_t n, const uint32_t* amp_id, const uint32_t* unit, int32_t n_amp,
                       int32_t n_core, const uint32_t* core_amp_id, double cf_b, double cf_b_rigid,
                       uint32_t* topol, double* cf_bend) {
  int64_t cnt = 0;
  for (int32_t i = 0; i < n; i++) {
    if (amp_id[i] != 0xffffffffu && unit[i] != 0xffffffffu) {
      const uint64_t slot = (uint64_t)amp_id[i] * ORC_ALL_UNIT + unit[i];
      if (slot >= (uint64_t)n_amp * ORC_ALL_UNIT || unit[i] >= ORC_ALL_UNIT) return -1;
      topol[slot] = (uint32_t)i;
      cnt++;
    }
  }
  for (int32_t a = 0; a < n_amp; a++) {
    cf_bend[a] = cf_b;
    for (int32_t k = 0; k < n_core; k++)
      if ((uint32_t)a == core_amp_id[k]) cf_bend[a] = cf_b_rigid;
  }
  return cnt == (int64_t)n_amp * ORC_ALL_UNIT ? 0 : -1;
}

/* ForceBonded::MinImage (bdf_calculator.hpp:55-59). */
static inline void min_image(double* d, const double* box, const double* ibox) {
  for (int k = 0; k < 3; k++) d[k] -= box[k] * round(d[k] * ibox[k]);
}

/* StoreBondForceWithARLaw (bdf_calculator.hpp:95-115); cf_spring<true>
 * (parameter.hpp:713-716). */
static inline void bond_force(const double* dr, double inv_dr, double cf_s, double* vir, double* F0,
                              double* F1) {
  const double cf_bond = cf_s * (inv_dr - 1.0 / ORC_BOND_LENG);
  double fb[3];
  for (int k = 0; k < 3; k++) fb[k] = cf_bond * dr[k];
  for (int k = 0; k < 3; k++) vir[k] += 2.0 * dr[k] * fb[k];
  for (int k = 0; k < 3; k++) {
    F0[k] -= fb[k];
    F1[k] += fb[k];
  }
}

/* StoreBendForceWithARLaw (bdf_calculator.hpp:117-150). */
static inline void bend_force(const double* dr0, const double* dr1, double inv0, double inv1,
                              double cf_b, double* vir, double* F0, double* F1, double* F2) {
  const double inv_dr_prod = inv0 * inv1;
  const double inv_dist0 = inv0 * inv0, inv_dist1 = inv1 * inv1;
  const double in_prod = dr0[0] * dr1[0] + dr0[1] * dr1[1] + dr0[2] * dr1[2];
  const double cf_bd = cf_b * inv_dr_prod;
  const double crs0 = in_prod * inv_dist0, crs1 = in_prod * inv_dist1;
  double t0[3], t1[3];
  for (int k = 0; k < 3; k++) {
    t0[k] = cf_bd * (dr1[k] - crs0 * dr0[k]);
    t1[k] = cf_bd * (dr0[k] - crs1 * dr1[k]);
  }
  for (int k = 0; k < 3; k++) vir[k] += 2.0 * (dr0[k] * t0[k] + dr1[k] * t1[k]);
  for (int k = 0; k < 3; k++) {
    F0[k] -= t0[k];
    F1[k] += t0[k] - t1[k];
    F2[k] += t1[k];
  }
}

/* CalcBondBendGlobalCell<4> (bdf_calculator.hpp:153-189) over all molecules
 * in order (the non-OpenMP branch of CalcListedForce, :211-217). */
void orc_bonded(const idpd_params* p, int32_t n_amp, const uint32_t* topol, const double* cf_bend,
                const double* pos, double* acc, double* vir) {
  double ibox[3];
  for (int k = 0; k < 3; k++) ibox[k] = 1.0 / p->box[k];
  double v[3] = {0.0, 0.0, 0.0};
  for (int32_t a = 0; a < n_amp; a++) {
    const uint32_t* l = topol + ORC_ALL_UNIT * a;
    double F[4][3] = {{0}};
    double dr[3][3], inv[3];
    for (int u = 1; u < 4; u++) {
      for (int k = 0; k < 3; k++) dr[u - 1][k] = pos[3 * l[u] + k] - pos[3 * l[u - 1] + k];
      min_image(dr[u - 1], p->box, ibox);
      const double d2 = dr[u - 1][0] * dr[u - 1][0] + dr[u - 1][1] * dr[u - 1][1] +
                        dr[u - 1][2] * dr[u - 1][2];
      inv[u - 1] = 1.0 / sqrt(d2);
      bond_force(dr[u - 1], inv[u - 1], p->cf_s, v, F[u - 1], F[u]);
      if (u >= 2) bend_force(dr[u - 2], dr[u - 1], inv[u - 2], inv[u - 1], cf_bend[a], v, F[u - 2],
                             F[u - 1], F[u]);
    }
    for (int u = 0; u < 4; u++)
      for (int k = 0; k < 3; k++) acc[3 * l[u] + k] += F[u][k];
  }
  if (vir)
    for (int k = 0; k < 3; k++) vir[k] = v[k];
}

/* ----------------------------------------------------------- integrator */
/* drift_and_predict (driftkick.hpp:6-27). */
void orc_drift(const idpd_params* p, int32_t n, double* pos, double* vel, double* vel_buf,
               const double* acc, double* dsr) {
  const double dt = p->dt;
  double ib[3];
  for (int k = 0; k < 3; k++) ib[k] = 1.0 / p->box[k];
  for (int32_t i = 0; i < n; i++) {
    double dr[3];
    for (int k = 0; k < 3; k++) dr[k] = dt * (vel[3 * i + k] + 0.5 * dt * acc[3 * i + k]);
    for (int k = 0; k < 3; k++) {
      const double t = pos[3 * i + k] + dr[k];
      if (dsr) dsr[3 * i + k] += dr[k];
      pos[3 * i + k] = t - floor(t * ib[k]) * p->box[k];
    }
    const double h = 0.5 * dt;
    for (int k = 0; k < 3; k++) {
      const double v = vel[3 * i + k] + h * acc[3 * i + k];
      if (vel_buf) vel_buf[3 * i + k] = v;
      vel[3 * i + k] = v;
    }
  }
}

/* kick (driftkick.hpp:33-40). */
void orc_kick(double dt, int32_t n, double* vel, const double* vel_buf, const double* acc) {
  const double h = dt * 0.5;
  for (int32_t i = 0; i < n; i++)
    for (int k = 0; k < 3; k++) vel[3 * i + k] = vel_buf[3 * i + k] + h * acc[3 * i + k];
}

/* remove_cmdrift_global (driftkick.hpp:43-54). */
void orc_remove_cmdrift(int32_t n, double* vel) {
  double s[3] = {0.0, 0.0, 0.0};
  for (int32_t i = 0; i < n; i++)
    for (int k = 0; k < 3; k++) s[k] += vel[3 * i + k];
  for (int k = 0; k < 3; k++) s[k] = s[k] / (double)n;
  for (int32_t i = 0; i < n; i++)
    for (int k = 0; k < 3; k++) vel[3 * i + k] -= s[k];
}

/* Main loop body, src/main.cpp:167-184 (single process, no chemistry). */
int orc_md_step(idpd_params* p, int32_t n, double* pos, double* vel, double* vel_buf, double* acc,
                double* dsr, const uint32_t* id, const uint32_t* prop, int32_t n_amp,
                const uint32_t* topol, const double* cf_bend, double* dens, double* press,
                double* bonded_vir, int32_t nthreads) {
  orc_drift(p, n, pos, vel, vel_buf, acc, dsr);
  if (orc_density(p, n, pos, prop, dens, NULL, NULL, nthreads) != 0) return -1;
  if (orc_force(p, n, pos, vel, id, prop, dens, acc, press, nthreads) != 0) return -1;
  double v[3] = {0.0, 0.0, 0.0};
  if (n_amp > 0) orc_bonded(p, n_amp, topol, cf_bend, pos, acc, v);
  if (bonded_vir)
    for (int k = 0; k < 3; k++) bonded_vir[k] = v[k];
  orc_kick(p->dt, n, vel, vel_buf, acc);
  if (p->time % ORC_CM_CORR == 0) orc_remove_cmdrift(n, vel);
  p->time++;
  return 0;
}

/* ------------------------------------------------------------ chemistry */
static inline void normalize3(double* v) {
  const double s = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  for (int k = 0; k < 3; k++) v[k] /= s;
}

/* ChemManager::ApplyPBC (chemmanager.hpp:22-26). */
static inline void apply_pbc(double* x, const double* box, const double* ibox) {
  for (int k = 0; k < 3; k++) x[k] -= floor(x[k] * ibox[k]) * box[k];
}

/* GenThermalVeloc (chemmanager.hpp:18-20); first draw feeds the logarithm. */
static inline double thermal_veloc(orc_mt* g) {
  const double r1 = orc_mt_real3(g);
  const double r2 = orc_mt_real3(g);
  return sqrt(-2.0 * ORC_TEMPERA * log(r1)) * cos(2.0 * M_PI * r2);
}

/* RandomChemEvent, single-node version (chemmanager.hpp:244-281) with
 * DetermineTargetIdWithCorePos (:115-162), GetCorePos (:84-113),
 * GetMembraneTangRandomVec (:164-172) and CreateAmpPart (:35-67). */
int orc_chem_event(const idpd_params* p, const idpd_chem_params* cp, orc_mt* g, int32_t* n_io,
                   int32_t n_cap, double* pos, double* vel, double* vel_buf, double* acc,
                   double* dsr, uint32_t* id, uint32_t* prop, uint32_t* amp_id, uint32_t* unit,
                   const double* nei_cm, const uint32_t* topol, int32_t n_core,
                   const uint32_t* core_ptcl_id, uint32_t* amp_num_out, uint32_t* targets_out,
                   int32_t* n_targets_out) {
  const int32_t glb_num = *n_io;
  double ibox[3];
  for (int k = 0; k < 3; k++) ibox[k] = 1.0 / p->box[k];
  int32_t nt = 0, tcap = 1 << 20;
  uint32_t* tgt = (uint32_t*)malloc(sizeof(uint32_t) * 2 * tcap);
  for (int32_t c = 0; c < n_core; c++) {
    double h[3] = {-1.0, -1.0, -1.0}, t[3] = {-1.0, -1.0, -1.0}, cm[3] = {-1.0, -1.0, -1.0};
    for (int32_t i = 0; i < glb_num; i++)
      if (id[i] == core_ptcl_id[c]) {
        for (int k = 0; k < 3; k++) {
          h[k] = pos[3 * i + k];
          t[k] = nei_cm[6 * i + 3 + k];
          cm[k] = nei_cm[6 * i + k];
        }
        break;
      }
    double h2t[3], c2cm[3];
    for (int k = 0; k < 3; k++) h2t[k] = t[k] - h[k];
    min_image(h2t, p->box, ibox);
    normalize3(h2t);
    for (int k = 0; k < 3; k++) c2cm[k] = cm[k] - h[k];
    min_image(c2cm, p->box, ibox);
    const double prj = c2cm[0] * h2t[0] + c2cm[1] * h2t[1] + c2cm[2] * h2t[2];
    for (int k = 0; k < 3; k++) h[k] += prj * h2t[k];
    apply_pbc(h, p->box, ibox);
    for (uint32_t j = 0; j < cp->amp_num; j++) {
      const uint32_t head = topol[ORC_ALL_UNIT * j];
      if (head < (uint32_t)glb_num) {
        double rnd = 2.0;
        double c2p[3];
        for (int k = 0; k < 3; k++) c2p[k] = pos[3 * head + k] - h[k];
        min_image(c2p, p->box, ibox);
        const double depth = h2t[0] * c2p[0] + h2t[1] * c2p[1] + h2t[2] * c2p[2];
        double tang[3];
        for (int k = 0; k < 3; k++) tang[k] = c2p[k] - depth * h2t[k];
        const double rad = sqrt(tang[0] * tang[0] + tang[1] * tang[1] + tang[2] * tang[2]);
        const double rad_th = cp->influ_grd * depth + cp->influ_rad;
        if ((rad <= rad_th) && (depth >= -cp->influ_hei) && (depth <= cp->influ_dep))
          rnd = orc_mt_real1(g);
        if (rnd <= cp->p_thresld) {
          if (nt >= tcap) {
            free(tgt);
            return -1;
          }
          tgt[2 * nt] = head;
          tgt[2 * nt + 1] = topol[ORC_ALL_UNIT * j + 2];
          nt++;
        }
      }
    }
  }
  if ((int64_t)glb_num + (int64_t)nt * ORC_ALL_UNIT > n_cap) {
    free(tgt);
    return -1;
  }
  uint32_t new_id = (uint32_t)glb_num;
  int32_t row = glb_num;
  for (int32_t i = 0; i < nt; i++) {
    const uint32_t hd = tgt[2 * i], tl = tgt[2 * i + 1];
    double h2e[3];
    for (int k = 0; k < 3; k++) h2e[k] = pos[3 * tl + k] - pos[3 * hd + k];
    min_image(h2e, p->box, ibox);
    normalize3(h2e);
    const double theta = 2.0 * M_PI * orc_mt_real1(g);
    const double base[3] = {cos(theta), sin(theta), 0.0};
    const double bdot = base[0] * h2e[0] + base[1] * h2e[1] + base[2] * h2e[2];
    double tang[3];
    for (int k = 0; k < 3; k++) tang[k] = base[k] - h2e[k] * bdot;
    normalize3(tang);
    for (int k = 0; k < 3; k++) tang[k] = tang[k] * cp->eps;
    for (int k = 0; k < 3; k++) h2e[k] *= ORC_BOND_LENG;
    double copied[3];
    for (int k = 0; k < 3; k++) copied[k] = tang[k] + pos[3 * hd + k];
    const uint32_t new_amp = cp->amp_num + (uint32_t)i;
    for (uint32_t u = 0; u < ORC_ALL_UNIT; u++) {
      double x[3];
      for (int k = 0; k < 3; k++) x[k] = copied[k] + h2e[k] * (double)u;
      apply_pbc(x, p->box, ibox);
      id[row] = new_id++;
      prop[row] = (u == 0) ? IDPD_HYPHIL : IDPD_HYPHOB;
      amp_id[row] = new_amp;
      unit[row] = u;
      for (int k = 0; k < 3; k++) {
        pos[3 * row + k] = x[k];
        if (dsr) dsr[3 * row + k] = 0.0;
        if (vel_buf) vel_buf[3 * row + k] = 0.0;
        acc[3 * row + k] = 0.0;
      }
      vel[3 * row] = thermal_veloc(g);
      vel[3 * row + 1] = thermal_veloc(g);
      vel[3 * row + 2] = thermal_veloc(g);
      row++;
    }
  }
  if (targets_out)
    for (int32_t i = 0; i < 2 * nt; i++) targets_out[i] = tgt[i];
  if (n_targets_out) *n_targets_out = nt;
  free(tgt);
  *n_io = row;
  const uint32_t amp_new = cp->amp_num + (uint32_t)nt;
  *amp_num_out = amp_new;
  return amp_new >= cp->max_amp_num ? 0 : 1;
}

/* ------------------------------------------------------ naive pair list */
/* make_nlist_naive (test/nearlist/near_list.cpp:69-92). */
int64_t orc_pairs_naive(int32_t n, const double* pos, const double* box, double rc, uint32_t* pi,
                        uint32_t* pj, int64_t cap) {
  const double rc2 = rc * rc;
  int64_t cnt = 0;
  for (int32_t i = 0; i < n; i++)
    for (int32_t j = 0; j < n; j++) {
      if (i == j) continue;
      double d[3];
      for (int k = 0; k < 3; k++) {
        d[k] = pos[3 * i + k] - pos[3 * j + k];
        d[k] -= box[k] * round(d[k] / box[k]);
      }
      const double dr2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
      if (dr2 < rc2) {
        if (cnt < cap) {
          pi[cnt] = (uint32_t)i;
          pj[cnt] = (uint32_t)j;
        }
        cnt++;
      }
    }
  return cnt;
}
