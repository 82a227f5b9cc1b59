/* md_oracle.c -- TEST INFRASTRUCTURE ONLY.  CPU restatement (FP64, one thread
 * per context unless orc_set_threads asks for more) of the reference's LLG +
 * Brownian-dynamics time step.  See
 * md_oracle.h.  Each function names the reference lines it restates
 * (paths relative to the MD_Sim_Wolfschwenger repository).  The loop order
 * and the arithmetic order of the reference are kept so that the two agree
 * to a few ulps; the product's CUDA path is checked against this file.
 */
#define _POSIX_C_SOURCE 199309L
#include "md_oracle.h"

#include <math.h>
#include <stdint.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

struct orc_ctx {
  orc_cfg cfg;
  int64_t n;
  /* particle properties (PartProps_S, src/typedefs.h:21-34) */
  double *rMag, *rHydr, *volMag, *magMom, *zetaRot, *zetaTrans, *velEa1, *velEa2;
  /* coordinates, column-major N x 3 */
  double *pos, *mm, *ea, *truePos, *posRef;
  double *demag, *force, *tTorque, *tField, *tForce, *mom, momSum[3];
  double *tcos, *tsin; /* [(j*N + i)*3 + axis], j = 0..nc */
  /* pair list (IntLists_S, src/typedefs.h:120-127) */
  int64_t pairs, cap;
  double *pvec, *plen;
  int32_t* pidx;
  unsigned char* psr;
  double *jac; /* Jacobi overlap displacement, N x 3 */
  /* Heun work arrays (IntCoefficient_S) */
  double *k1m, *k1e, *k2m, *k2e, *c2m, *c2e, *beff, *b2, *b3, *dot;
  /* adaptive solvers: stage slopes k_s (m, n) and stage coordinates */
  double *skm[7], *ske[7], *scm, *sce, *ebuf;
  /* Ewald constants (InitEwaldConst, interaction.cpp:353-374) */
  double nc2, w, cFluxDens, cForce, cSurf, cSelf, alpha2, alpha4, volBox;
  double Pxy, Pxz, Pyz;
  double t, last_seconds;
  int64_t step;
  /* threads of the pair list and the Ewald sums (orc_set_threads): private
   * accumulators per thread, [T][6 N] (B then F), pressure [T][3] */
  int nthreads;
  double *tacc, *tP;
};

#define AX(a, i, c, n) (a)[(int64_t)(c) * (n) + (i)]

static double* zalloc(int64_t k) { return (double*)calloc((size_t)(k > 0 ? k : 1), sizeof(double)); }

/* InitEwaldConst (interaction.cpp:353-374): constants for both Ewald sums. */
static void ewald_consts(orc_ctx* c) {
  const orc_cfg* g = &c->cfg;
  double L = g->lBox, pi = g->my_pi;
  c->nc2 = (double)g->nc * (double)g->nc;
  c->w = pow(pi / (L * g->alpha), 2.0);
  c->cFluxDens = 4.0 * pi * g->facEwald / pow(L, 3.0);
  c->cForce = 8.0 * pi * pi * g->facEwald / pow(L, 4.0);
  c->cSurf = g->facEwald * 4.0 * pi / (3 * pow(L, 3.0));
  c->cSelf = g->facEwald * 4.0 * pow(g->alpha, 3.0) / (3.0 * sqrt(pi));
  c->alpha2 = g->alpha * g->alpha;
  c->alpha4 = c->alpha2 * c->alpha2;
  c->volBox = pow(L, 3.0);
}

orc_ctx* orc_create(const orc_cfg* cfg) {
  orc_ctx* c = (orc_ctx*)calloc(1, sizeof(orc_ctx));
  int64_t n = cfg->n, n3 = 3 * cfg->n, nt = (cfg->nc + 1) * n3;
  c->cfg = *cfg;
  c->n = n;
  double** arrs1[] = {&c->rMag, &c->rHydr, &c->volMag, &c->magMom, &c->zetaRot, &c->zetaTrans,
                      &c->velEa1, &c->velEa2, &c->dot};
  for (size_t k = 0; k < sizeof arrs1 / sizeof *arrs1; k++) *arrs1[k] = zalloc(n);
  double** arrs3[] = {&c->pos, &c->mm, &c->ea, &c->truePos, &c->posRef, &c->demag, &c->force,
                      &c->tTorque, &c->tField, &c->tForce, &c->mom, &c->jac, &c->k1m, &c->k1e,
                      &c->k2m, &c->k2e, &c->c2m, &c->c2e, &c->beff, &c->b2, &c->b3};
  for (size_t k = 0; k < sizeof arrs3 / sizeof *arrs3; k++) *arrs3[k] = zalloc(n3);
  c->tcos = zalloc(nt);
  c->tsin = zalloc(nt);
  for (int q = 0; q < 7; q++) {
    c->skm[q] = zalloc(n3);
    c->ske[q] = zalloc(n3);
  }
  c->scm = zalloc(n3);
  c->sce = zalloc(n3);
  c->ebuf = zalloc(n3);
  ewald_consts(c);
  return c;
}

void orc_destroy(orc_ctx* c) {
  if (!c) return;
  double* all[] = {c->rMag, c->rHydr, c->volMag, c->magMom, c->zetaRot, c->zetaTrans, c->velEa1,
                   c->velEa2, c->dot, c->pos, c->mm, c->ea, c->truePos, c->posRef, c->demag,
                   c->force, c->tTorque, c->tField, c->tForce, c->mom, c->jac, c->k1m, c->k1e,
                   c->k2m, c->k2e, c->c2m, c->c2e, c->beff, c->b2, c->b3, c->tcos, c->tsin,
                   c->pvec, c->plen};
  for (size_t k = 0; k < sizeof all / sizeof *all; k++) free(all[k]);
  for (int q = 0; q < 7; q++) {
    free(c->skm[q]);
    free(c->ske[q]);
  }
  free(c->scm);
  free(c->sce);
  free(c->ebuf);
  free(c->pidx);
  free(c->psr);
  free(c->tacc);
  free(c->tP);
  free(c);
}

/* Threads for the pair list and the Ewald sums (the bench's CPU arm on all
 * host cores).  t > 1 needs the Jacobi overlap push (overlap_mode 1): the
 * sequential push of the reference depends on the loop order.  Results
 * equal the one-thread ones up to the order of the final additions. */
int orc_set_threads(orc_ctx* c, int t) {
  if (t < 1 || t > 256) return 1;
  if (t > 1 && c->cfg.overlap_mode != 1) return 2;
  free(c->tacc);
  free(c->tP);
  c->tacc = c->tP = NULL;
  c->nthreads = t;
  if (t > 1) {
    c->tacc = zalloc((int64_t)t * 6 * c->n);
    c->tP = zalloc(3 * (int64_t)t);
  }
  return 0;
}

typedef struct {
  orc_ctx* c;
  int t;
  int64_t a, b;   /* range of rows, pairs or k vectors */
  double *B, *F;  /* private accumulators (N x 3 each) */
  int field_only;
  /* pair list: private list */
  int64_t np, cap;
  double *pvec, *plen, *jac;
  int32_t* pidx;
  unsigned char* psr;
} orc_job;

static void run_jobs(orc_job* jobs, int T, void* (*fn)(void*)) {
  pthread_t th[256];
  int started[256] = {0};
  for (int t = 1; t < T; t++) started[t] = pthread_create(&th[t], NULL, fn, &jobs[t]) == 0;
  fn(&jobs[0]);
  for (int t = 1; t < T; t++) {
    if (started[t])
      pthread_join(th[t], NULL);
    else
      fn(&jobs[t]);  /* no thread: run it here */
  }
}

/* InitParticleProps derived quantities (simulation.cpp:204-210). */
void orc_set_props(orc_ctx* c, const double* rMag, const double* rHydr, double vis) {
  const orc_cfg* g = &c->cfg;
  double pi = g->my_pi;
  for (int64_t i = 0; i < c->n; i++) {
    c->rMag[i] = rMag[i];
    c->rHydr[i] = rHydr[i];
    c->volMag[i] = 4.0 / 3.0 * pi * pow(rMag[i], 3.0);
    double volHydr = 4.0 / 3.0 * pi * pow(rHydr[i], 3.0);
    (void)volHydr;
    c->magMom[i] = g->satMag * c->volMag[i];
    c->zetaRot[i] = 8.0 * pi * vis * pow(rHydr[i], 3.0);
    c->zetaTrans[i] = 6.0 * pi * vis * rHydr[i];
    c->velEa1[i] = 2.0 * g->anisEn * (c->volMag[i] / c->zetaRot[i]);
    c->velEa2[i] = 1.0 / c->zetaRot[i];
  }
}

void orc_set_state(orc_ctx* c, const double* pos, const double* mm, const double* ea, double t) {
  int64_t n3 = 3 * c->n;
  memcpy(c->pos, pos, (size_t)n3 * sizeof(double));
  memcpy(c->mm, mm, (size_t)n3 * sizeof(double));
  memcpy(c->ea, ea, (size_t)n3 * sizeof(double));
  c->t = t;
}

void orc_get_state(const orc_ctx* c, double* pos, double* mm, double* ea, double* t) {
  int64_t n3 = 3 * c->n;
  if (pos) memcpy(pos, c->pos, (size_t)n3 * sizeof(double));
  if (mm) memcpy(mm, c->mm, (size_t)n3 * sizeof(double));
  if (ea) memcpy(ea, c->ea, (size_t)n3 * sizeof(double));
  if (t) *t = c->t;
}

/* InitSimulation (simulation.cpp:108-109): MSD reference = current positions. */
void orc_reset_observables(orc_ctx* c) {
  int64_t n3 = 3 * c->n;
  memcpy(c->posRef, c->pos, (size_t)n3 * sizeof(double));
  memcpy(c->truePos, c->pos, (size_t)n3 * sizeof(double));
}

/* ------------------------------------------------------------------ noise */

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): 10 rounds of two 32x32
 * multiplies with the published multipliers and Weyl key increments. */
static void philox4x32_10(uint32_t ctr[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * ctr[0];
    uint64_t p1 = (uint64_t)0xCD9E8D57u * ctr[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ ctr[1] ^ k0, n2 = hi0 ^ ctr[3] ^ k1;
    ctr[0] = n0;
    ctr[1] = lo1;
    ctr[2] = n2;
    ctr[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

/* 9 standard normals for particle i at step s: counter {i, block, s_lo, s_hi},
 * key {seed_lo, seed_hi}; uniforms (x + 0.5) 2^-32; Box-Muller pairs. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
  philox4x32_10(c, key[0], key[1]);
  for (int q = 0; q < 4; q++) out[q] = c[q];
}

void orc_philox_normals(uint64_t seed, uint64_t step, int64_t n, double* xi) {
  const double twopi = 6.283185307179586476925286766559;
  for (int64_t i = 0; i < n; i++) {
    double z[12];
    for (uint32_t b = 0; b < 3; b++) {
      uint32_t ctr[4] = {(uint32_t)i, b, (uint32_t)step, (uint32_t)(step >> 32)};
      philox4x32_10(ctr, (uint32_t)seed, (uint32_t)(seed >> 32));
      for (int h = 0; h < 2; h++) {
        double u1 = ((double)ctr[2 * h] + 0.5) * 2.3283064365386963e-10;
        double u2 = ((double)ctr[2 * h + 1] + 0.5) * 2.3283064365386963e-10;
        double r = sqrt(-2.0 * log(u1));
        z[4 * b + 2 * h] = r * cos(twopi * u2);
        z[4 * b + 2 * h + 1] = r * sin(twopi * u2);
      }
    }
    for (int k = 0; k < 9; k++) xi[(int64_t)(k / 3) * 3 * n + (int64_t)(k % 3) * n + i] = z[k];
  }
}

/* DefThermFluct (simulation.cpp:563-603). */
void orc_thermal(orc_ctx* c, double dt, int noise_mode, const double* xi, uint64_t seed,
                 double* torque, double* field, double* force) {
  const orc_cfg* g = &c->cfg;
  int64_t n = c->n, n3 = 3 * n;
  double* gen = NULL;
  const double* src = xi;
  if (noise_mode == ORC_NOISE_PHILOX) {
    gen = zalloc(3 * n3);
    orc_philox_normals(seed, (uint64_t)c->step, n, gen);
    src = gen;
  }
  for (int64_t i = 0; i < n; i++) {
    double sT = sqrt((2.0 * g->kB * g->temp / dt) * c->zetaRot[i]);
    double sB = sqrt(2.0 * g->kB * g->temp * g->magDamp / (g->gyroMr * g->satMag * dt) *
                     (1.0 / c->volMag[i]));
    double sF = sqrt((2.0 * g->kB * g->temp / dt) * c->zetaTrans[i]);
    for (int a = 0; a < 3; a++) {
      int on = noise_mode != ORC_NOISE_OFF;
      AX(torque, i, a, n) = (on && g->enable_therm_torque) ? AX(src, i, a, n) * sT : 0.0;
      AX(field, i, a, n) = (on && g->enable_therm_field) ? AX(src + n3, i, a, n) * sB : 0.0;
      AX(force, i, a, n) = (on && g->enable_therm_force) ? AX(src + 2 * n3, i, a, n) * sF : 0.0;
    }
  }
  free(gen);
}

/* --------------------------------------------------------- interactions */

/* EvalSinCos (interaction.cpp:521-548): Chebyshev recurrence per axis. */
static void eval_sincos(orc_ctx* c) {
  int64_t n = c->n, nc = c->cfg.nc;
  double t = 2 * c->cfg.my_pi / c->cfg.lBox;
  for (int64_t i = 0; i < n; i++) {
    for (int a = 0; a < 3; a++) {
      double tt = t * AX(c->pos, i, a, n);
#define TC(j) c->tcos[((int64_t)(j) * n + i) * 3 + a]
#define TS(j) c->tsin[((int64_t)(j) * n + i) * 3 + a]
      TC(0) = 1;
      TS(0) = 0;
      TC(1) = cos(tt);
      TS(1) = sin(tt);
      double u = 2.0 * TC(1);
      if (nc >= 2) {
        TC(2) = u * TC(1);
        TS(2) = u * TS(1);
        TC(2) -= 1.0;
      }
      for (int64_t j = 3; j <= nc; j++) {
        double w = u * TC(j - 1);
        TC(j) = w - TC(j - 2);
        w = u * TS(j - 1);
        TS(j) = w - TS(j - 2);
      }
#undef TC
#undef TS
    }
  }
}

static void list_push(orc_ctx* c, double r, const double v[3], int32_t i1, int32_t i2, int sr) {
  if (c->pairs == c->cap) {
    int64_t nc = c->cap ? 2 * c->cap : 1024;
    c->pvec = (double*)realloc(c->pvec, (size_t)nc * 3 * sizeof(double));
    c->plen = (double*)realloc(c->plen, (size_t)nc * sizeof(double));
    c->pidx = (int32_t*)realloc(c->pidx, (size_t)nc * 2 * sizeof(int32_t));
    c->psr = (unsigned char*)realloc(c->psr, (size_t)nc);
    c->cap = nc;
  }
  int64_t p = c->pairs++;
  c->plen[p] = r;
  for (int a = 0; a < 3; a++) c->pvec[3 * p + a] = v[a] / r;
  c->pidx[2 * p] = i1;
  c->pidx[2 * p + 1] = i2;
  c->psr[p] = (unsigned char)sr;
}

static void pair_list_threads(orc_ctx* c);

/* CompInteractVecs + ApplyBoundaryCondVec (interaction.cpp:88-155): all pairs,
 * minimum image, list of pairs with r < rCutLR, and the overlap push of the
 * cores (in place and sequential for overlap_mode 0, Jacobi for 1). */
static void pair_list(orc_ctx* c) {
  if (c->nthreads > 1) {
    pair_list_threads(c);
    return;
  }
  int64_t n = c->n;
  double L = c->cfg.lBox, h = L / 2, rc = c->cfg.rCutLR, rsr = c->cfg.rCutSR;
  int jac = c->cfg.overlap_mode == 1;
  c->pairs = 0;
  if (jac) memset(c->jac, 0, (size_t)(3 * n) * sizeof(double));
  for (int64_t i1 = 0; i1 < n - 1; i1++) {
    for (int64_t i2 = i1 + 1; i2 < n; i2++) {
      double v[3];
      for (int a = 0; a < 3; a++) {
        double d = AX(c->pos, i2, a, n) - AX(c->pos, i1, a, n);
        d -= L * (double)(d > h);
        d += L * (double)(d < -h);
        v[a] = d;
      }
      double r = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
      if (r < rc) {
        list_push(c, r, v, (int32_t)i1, (int32_t)i2, r < rsr);
        int64_t p = c->pairs - 1;
        double dCont = c->rMag[i1] + c->rMag[i2] + 1e-10;
        if (r < dCont) {
          double d = dCont - r;
          for (int a = 0; a < 3; a++) {
            double u = c->pvec[3 * p + a];
            if (jac) {
              AX(c->jac, i1, a, n) -= 0.5 * d * u;
              AX(c->jac, i2, a, n) += 0.5 * d * u;
            } else {
              AX(c->pos, i1, a, n) -= 0.5 * d * u;
              AX(c->pos, i2, a, n) += 0.5 * d * u;
            }
          }
          c->plen[p] = dCont;
        }
      }
    }
  }
  if (jac)
    for (int64_t k = 0; k < 3 * n; k++) c->pos[k] += c->jac[k];
}

/* The pair list over rows [a, b) of the all-pairs loop into a private list
 * (Jacobi overlap push into a private displacement array). */
static void* pair_rows(void* arg) {
  orc_job* j = (orc_job*)arg;
  orc_ctx* c = j->c;
  int64_t n = c->n;
  double L = c->cfg.lBox, h = L / 2, rc = c->cfg.rCutLR, rsr = c->cfg.rCutSR;
  for (int64_t i1 = j->a; i1 < j->b; i1++) {
    for (int64_t i2 = i1 + 1; i2 < n; i2++) {
      double v[3];
      for (int a = 0; a < 3; a++) {
        double d = AX(c->pos, i2, a, n) - AX(c->pos, i1, a, n);
        d -= L * (double)(d > h);
        d += L * (double)(d < -h);
        v[a] = d;
      }
      double r = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
      if (r < rc) {
        if (j->np == j->cap) {
          int64_t nc = j->cap ? 2 * j->cap : 4096;
          j->pvec = (double*)realloc(j->pvec, (size_t)nc * 3 * sizeof(double));
          j->plen = (double*)realloc(j->plen, (size_t)nc * sizeof(double));
          j->pidx = (int32_t*)realloc(j->pidx, (size_t)nc * 2 * sizeof(int32_t));
          j->psr = (unsigned char*)realloc(j->psr, (size_t)nc);
          j->cap = nc;
        }
        int64_t p = j->np++;
        j->plen[p] = r;
        for (int a = 0; a < 3; a++) j->pvec[3 * p + a] = v[a] / r;
        j->pidx[2 * p] = (int32_t)i1;
        j->pidx[2 * p + 1] = (int32_t)i2;
        j->psr[p] = (unsigned char)(r < rsr);
        double dCont = c->rMag[i1] + c->rMag[i2] + 1e-10;
        if (r < dCont) {
          double d = dCont - r;
          for (int a = 0; a < 3; a++) {
            double u = j->pvec[3 * p + a];
            AX(j->jac, i1, a, n) -= 0.5 * d * u;
            AX(j->jac, i2, a, n) += 0.5 * d * u;
          }
          j->plen[p] = dCont;
        }
      }
    }
  }
  return NULL;
}

/* pair_list on T threads: rows split into ranges of equal candidate counts,
 * the private lists concatenated in row order (the one-thread list order). */
static void pair_list_threads(orc_ctx* c) {
  int T = c->nthreads;
  int64_t n = c->n;
  orc_job jobs[256];
  memset(jobs, 0, sizeof jobs);
  double total = 0.5 * (double)n * (double)(n - 1);
  int64_t row = 0;
  for (int t = 0; t < T; t++) {
    jobs[t].c = c;
    jobs[t].t = t;
    jobs[t].a = row;
    double target = total * (double)(t + 1) / T;
    while (row < n && (double)(row + 1) * (double)(n - 1) - 0.5 * (double)(row + 1) * (double)row < target) row++;
    if (t == T - 1) row = n;
    jobs[t].b = row;
    jobs[t].jac = c->tacc + (int64_t)t * 6 * n;
    memset(jobs[t].jac, 0, (size_t)(3 * n) * sizeof(double));
  }
  run_jobs(jobs, T, pair_rows);
  int64_t total_pairs = 0;
  for (int t = 0; t < T; t++) total_pairs += jobs[t].np;
  if (total_pairs > c->cap) {
    c->pvec = (double*)realloc(c->pvec, (size_t)total_pairs * 3 * sizeof(double));
    c->plen = (double*)realloc(c->plen, (size_t)total_pairs * sizeof(double));
    c->pidx = (int32_t*)realloc(c->pidx, (size_t)total_pairs * 2 * sizeof(int32_t));
    c->psr = (unsigned char*)realloc(c->psr, (size_t)total_pairs);
    c->cap = total_pairs;
  }
  c->pairs = 0;
  for (int t = 0; t < T; t++) {
    const int64_t m = jobs[t].np, o = c->pairs;
    if (m) {
      memcpy(c->pvec + 3 * o, jobs[t].pvec, (size_t)m * 3 * sizeof(double));
      memcpy(c->plen + o, jobs[t].plen, (size_t)m * sizeof(double));
      memcpy(c->pidx + 2 * o, jobs[t].pidx, (size_t)m * 2 * sizeof(int32_t));
      memcpy(c->psr + o, jobs[t].psr, (size_t)m);
    }
    c->pairs += m;
    free(jobs[t].pvec);
    free(jobs[t].plen);
    free(jobs[t].pidx);
    free(jobs[t].psr);
  }
  for (int t = 0; t < T; t++)
    for (int64_t k = 0; k < 3 * n; k++) c->pos[k] += jobs[t].jac[k];
}

static inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* CompDipInteractEwaldR + EvalPressTensLR (interaction.cpp:383-422,
 * postprocessing.cpp:195-200); field only when F == NULL
 * (CompDipFieldEwaldR, interaction.cpp:555-582). */
static void ewald_real_range(orc_ctx* c, double* B, double* F, int64_t p0, int64_t p1, double* P) {
  int64_t n = c->n;
  double al = c->cfg.alpha, al2 = c->alpha2, al4 = c->alpha4, fe = c->cfg.facEwald;
  for (int64_t p = p0; p < p1; p++) {
    int64_t i1 = c->pidx[2 * p], i2 = c->pidx[2 * p + 1];
    double r = c->plen[p], r2 = r * r;
    double t = 2.0 * al * exp(-al2 * r2) * c->cfg.irPi / r2;
    double a1 = erfc(al * r) / (r2 * r) + t;
    double a2 = 3.0 * a1 / r2 + 2.0 * al2 * t;
    double a3 = 5.0 * a2 / r2 + 4.0 * al4 * t;
    const double* u = &c->pvec[3 * p];
    double m1[3], m2[3];
    for (int a = 0; a < 3; a++) {
      m1[a] = AX(c->mom, i1, a, n);
      m2[a] = AX(c->mom, i2, a, n);
    }
    double dot1 = dot3(m1, u), dot2 = dot3(m2, u);
    if (F) {
      double m12 = dot3(m1, m2), v1[3];
      for (int a = 0; a < 3; a++)
        v1[a] = fe * ((a2 * m12 - a3 * dot1 * dot2 * r2) * u[a] * r + a2 * r * (dot2 * m1[a] + dot1 * m2[a]));
      for (int a = 0; a < 3; a++) {
        AX(B, i1, a, n) += fe * (a2 * dot2 * u[a] * r2 - a1 * m2[a]);
        AX(B, i2, a, n) += fe * (a2 * dot1 * u[a] * r2 - a1 * m1[a]);
        AX(F, i1, a, n) -= v1[a];
        AX(F, i2, a, n) += v1[a];
      }
      P[0] += r * u[0] * v1[1];
      P[1] += r * u[0] * v1[2];
      P[2] += r * u[1] * v1[2];
    } else {
      for (int a = 0; a < 3; a++) {
        AX(B, i1, a, n) += fe * (a2 * dot2 * u[a] * r2 - a1 * m2[a]);
        AX(B, i2, a, n) += fe * (a2 * dot1 * u[a] * r2 - a1 * m1[a]);
      }
    }
  }
}

static void* real_job(void* arg) {
  orc_job* j = (orc_job*)arg;
  double* P = j->c->tP + 3 * j->t;
  P[0] = P[1] = P[2] = 0;
  ewald_real_range(j->c, j->B, j->F, j->a, j->b, P);
  return NULL;
}

/* Adds the private accumulators of T jobs in thread order. */
static void reduce_jobs(orc_ctx* c, orc_job* jobs, int T, double* B, double* F) {
  int64_t n3 = 3 * c->n;
  for (int t = 0; t < T; t++)
    for (int64_t k = 0; k < n3; k++) {
      B[k] += jobs[t].B[k];
      if (F) F[k] += jobs[t].F[k];
    }
}

static void ewald_real(orc_ctx* c, double* B, double* F) {
  if (c->nthreads <= 1) {
    double P[3] = {c->Pxy, c->Pxz, c->Pyz};
    ewald_real_range(c, B, F, 0, c->pairs, P);
    c->Pxy = P[0];
    c->Pxz = P[1];
    c->Pyz = P[2];
    return;
  }
  int T = c->nthreads;
  int64_t n = c->n;
  orc_job jobs[256];
  memset(jobs, 0, sizeof jobs);
  for (int t = 0; t < T; t++) {
    jobs[t].c = c;
    jobs[t].t = t;
    jobs[t].a = c->pairs * t / T;
    jobs[t].b = c->pairs * (t + 1) / T;
    jobs[t].B = c->tacc + (int64_t)t * 6 * n;
    jobs[t].F = F ? jobs[t].B + 3 * n : NULL;
    memset(jobs[t].B, 0, (size_t)(6 * n) * sizeof(double));
  }
  run_jobs(jobs, T, real_job);
  reduce_jobs(c, jobs, T, B, F);
  for (int t = 0; t < T; t++) {
    c->Pxy += c->tP[3 * t];
    c->Pxz += c->tP[3 * t + 1];
    c->Pyz += c->tP[3 * t + 2];
  }
}

/* CompDipInteractEwaldF (interaction.cpp:429-514); field only when F == NULL
 * (CompDipFieldEwaldF, interaction.cpp:588-672).  Includes self and surface terms. */
static void ewald_kspace_range(orc_ctx* c, double* B, double* F, int64_t k0, int64_t k1) {
  int64_t n = c->n, nc = c->cfg.nc, kidx = -1;
  for (int64_t nz = 0; nz <= nc; nz++)
    for (int64_t ny = -nc; ny <= nc; ny++)
      for (int64_t nx = -nc; nx <= nc; nx++) {
        double kv[3] = {(double)nx, (double)ny, (double)nz};
        double lenSqr = dot3(kv, kv);
        if (lenSqr == 0 || lenSqr > c->nc2) continue;
        kidx++;
        if (kidx < k0 || kidx >= k1) continue;
        double e = 2.0 * exp(-c->w * lenSqr) / lenSqr;
        if (nz == 0) e *= 0.5;
        double sumC = 0, sumS = 0;
        int64_t ax = nx < 0 ? -nx : nx, ay = ny < 0 ? -ny : ny, az = nz;
        for (int pass = 0; pass < 2; pass++) {
          for (int64_t i = 0; i < n; i++) {
            double vcx = c->tcos[(ax * n + i) * 3 + 0], vcy = c->tcos[(ay * n + i) * 3 + 1],
                   vcz = c->tcos[(az * n + i) * 3 + 2];
            double vsx = c->tsin[(ax * n + i) * 3 + 0], vsy = c->tsin[(ay * n + i) * 3 + 1],
                   vsz = c->tsin[(az * n + i) * 3 + 2];
            if (nx < 0) vsx = -vsx;
            if (ny < 0) vsy = -vsy;
            double pc = vcx * vcy * vcz - vcx * vsy * vsz - vsx * vcy * vsz - vsx * vsy * vcz;
            double ps = vsx * vcy * vcz + vcx * vsy * vcz + vcx * vcy * vsz - vsx * vsy * vsz;
            double mi[3] = {AX(c->mom, i, 0, n), AX(c->mom, i, 1, n), AX(c->mom, i, 2, n)};
            double preFac = dot3(kv, mi);
            if (pass == 0) {
              sumC += preFac * pc;
              sumS += preFac * ps;
            } else {
              if (F) {
                double s = c->cForce * e * preFac * (sumC * ps - sumS * pc);
                for (int a = 0; a < 3; a++) AX(F, i, a, n) += s * kv[a];
              }
              double s = c->cFluxDens * e * (sumC * pc + sumS * ps);
              for (int a = 0; a < 3; a++) AX(B, i, a, n) -= s * kv[a];
            }
          }
        }
      }
}

static void* kspace_job(void* arg) {
  orc_job* j = (orc_job*)arg;
  ewald_kspace_range(j->c, j->B, j->F, j->a, j->b);
  return NULL;
}

static void ewald_kspace(orc_ctx* c, double* B, double* F) {
  int64_t n = c->n;
  if (c->nthreads <= 1) {
    ewald_kspace_range(c, B, F, 0, INT64_MAX);
  } else {
    int64_t nk = 0, nc = c->cfg.nc;
    for (int64_t nz = 0; nz <= nc; nz++)
      for (int64_t ny = -nc; ny <= nc; ny++)
        for (int64_t nx = -nc; nx <= nc; nx++) {
          double l = (double)(nx * nx + ny * ny + nz * nz);
          if (l > 0 && l <= c->nc2) nk++;
        }
    int T = c->nthreads;
    orc_job jobs[256];
    memset(jobs, 0, sizeof jobs);
    for (int t = 0; t < T; t++) {
      jobs[t].c = c;
      jobs[t].t = t;
      jobs[t].a = nk * t / T;
      jobs[t].b = nk * (t + 1) / T;
      jobs[t].B = c->tacc + (int64_t)t * 6 * n;
      jobs[t].F = F ? jobs[t].B + 3 * n : NULL;
      memset(jobs[t].B, 0, (size_t)(6 * n) * sizeof(double));
    }
    run_jobs(jobs, T, kspace_job);
    reduce_jobs(c, jobs, T, B, F);
  }
  for (int64_t i = 0; i < n; i++)
    for (int a = 0; a < 3; a++)
      AX(B, i, a, n) += c->cSelf * AX(c->mom, i, a, n) - c->cSurf * c->momSum[a];
}

/* Coating potentials over the pair list (simulation.cpp:648-676 with
 * CompSterRep, CompElectrostatRep, CompForceVdW interaction.cpp:766-832 and
 * EvalPressTensSR postprocessing.cpp:208-213).  The short-range flag is the
 * intended cutoff r < rCutSR of the current step. */
static void coating_forces(orc_ctx* c, double* F) {
  const orc_cfg* g = &c->cfg;
  int64_t n = c->n;
  for (int64_t p = 0; p < c->pairs; p++) {
    if (!c->psr[p]) continue;
    int64_t i1 = c->pidx[2 * p], i2 = c->pidx[2 * p + 1];
    double r1 = c->rMag[i1], r2m = c->rMag[i2], r = c->plen[p];
    const double* u = &c->pvec[3 * p];
    double v2[3] = {0, 0, 0}, s;
    double dDelta = 2 * (r1 + g->effLenSurfMol);
    s = r <= dDelta ? (2 * r2m / (r1 + r2m)) * g->sterRepFac * r1 * r1 * log(dDelta / r) : 0.0;
    for (int a = 0; a < 3; a++) { double v = s * u[a]; AX(F, i1, a, n) -= v; AX(F, i2, a, n) += v; v2[a] += v; }
    s = (r1 * r2m / (r1 + r2m)) * g->electrostatRepFac * exp(-g->kappa * (r - r1 - r2m));
    for (int a = 0; a < 3; a++) { double v = s * u[a]; AX(F, i1, a, n) -= v; AX(F, i2, a, n) += v; v2[a] += v; }
    s = -g->hamaker * r * pow(4 * r1 * r2m, 3.0) /
        (6 * pow((r - r1 - r2m) * (r + r1 + r2m), 2.0) * pow(r * r - pow(r1 - r2m, 2.0), 2.0));
    for (int a = 0; a < 3; a++) { double v = s * u[a]; AX(F, i1, a, n) -= v; AX(F, i2, a, n) += v; v2[a] += v; }
    c->Pxy += r * u[0] * v2[1];
    c->Pxz += r * u[0] * v2[2];
    c->Pyz += r * u[1] * v2[2];
  }
}

static void moments(orc_ctx* c, const double* mm) {
  int64_t n = c->n;
  for (int a = 0; a < 3; a++) {
    double s = 0;
    for (int64_t i = 0; i < n; i++) {
      AX(c->mom, i, a, n) = AX(mm, i, a, n) * c->magMom[i];
      s += AX(c->mom, i, a, n);
    }
    c->momSum[a] = s;
  }
}

/* EvalSinCos + CompInteractions (simulation.cpp:475-476, 628-680). */
void orc_compute_interactions(orc_ctx* c, double* B, double* F, double* P3) {
  int64_t n3 = 3 * c->n;
  eval_sincos(c);
  memset(c->force, 0, (size_t)n3 * sizeof(double));
  memset(c->demag, 0, (size_t)n3 * sizeof(double));
  c->Pxy = c->Pxz = c->Pyz = 0;
  moments(c, c->mm);
  pair_list(c);
  ewald_real(c, c->demag, c->force);
  ewald_kspace(c, c->demag, c->force);
  if (c->cfg.enable_coating) coating_forces(c, c->force);
  for (int64_t k = 0; k < n3; k++) c->force[k] += c->tForce[k];
  if (B) memcpy(B, c->demag, (size_t)n3 * sizeof(double));
  if (F) memcpy(F, c->force, (size_t)n3 * sizeof(double));
  if (P3) { P3[0] = c->Pxy; P3[1] = c->Pxz; P3[2] = c->Pyz; }
}

/* CompDemagField (simulation.cpp:688-697). */
void orc_compute_field(orc_ctx* c, const double* mm, double* B) {
  int64_t n3 = 3 * c->n;
  memset(c->demag, 0, (size_t)n3 * sizeof(double));
  moments(c, mm);
  ewald_real(c, c->demag, NULL);
  ewald_kspace(c, c->demag, NULL);
  if (B) memcpy(B, c->demag, (size_t)n3 * sizeof(double));
}

/* -------------------------------------------------------------- integrator */

static void cross_rows(const double* a, const double* b, double* r, int64_t n) {
  for (int64_t i = 0; i < n; i++) {
    AX(r, i, 0, n) = AX(a, i, 1, n) * AX(b, i, 2, n) - AX(a, i, 2, n) * AX(b, i, 1, n);
    AX(r, i, 1, n) = AX(a, i, 2, n) * AX(b, i, 0, n) - AX(a, i, 0, n) * AX(b, i, 2, n);
    AX(r, i, 2, n) = AX(a, i, 0, n) * AX(b, i, 1, n) - AX(a, i, 1, n) * AX(b, i, 0, n);
  }
}

/* RKCoeffs (simulation.cpp:876-902). */
static void rk_coeffs(orc_ctx* c, const double* mm, const double* ea, const double* ext,
                      double* kM, double* kE) {
  const orc_cfg* g = &c->cfg;
  int64_t n = c->n;
  for (int64_t i = 0; i < n; i++)
    c->dot[i] = AX(mm, i, 0, n) * AX(ea, i, 0, n) + AX(mm, i, 1, n) * AX(ea, i, 1, n) +
                AX(mm, i, 2, n) * AX(ea, i, 2, n);
  for (int a = 0; a < 3; a++)
    for (int64_t i = 0; i < n; i++)
      AX(c->beff, i, a, n) = ext[a] + AX(c->demag, i, a, n) + g->anisConst * (AX(ea, i, a, n) * c->dot[i]) +
                             AX(c->tField, i, a, n);
  if (g->enable_mobilization) {
    cross_rows(c->tTorque, ea, c->b2, n);
    for (int a = 0; a < 3; a++)
      for (int64_t i = 0; i < n; i++)
        AX(kE, i, a, n) = (AX(mm, i, a, n) - AX(ea, i, a, n) * c->dot[i]) * (c->velEa1[i] * c->dot[i]) +
                          AX(c->b2, i, a, n) * c->velEa2[i];
  } else {
    memset(kE, 0, (size_t)(3 * n) * sizeof(double));
  }
  cross_rows(mm, c->beff, c->b2, n);
  cross_rows(mm, c->b2, c->b3, n);
  for (int64_t k = 0; k < 3 * n; k++) kM[k] = -g->velMmConst * (c->b2[k] + g->magDamp * c->b3[k]);
}

/* DefExtField (simulation.cpp:546-556); field_kind 1 is an extension. */
static void ext_field(const orc_ctx* c, double t, double ext[3]) {
  ext[0] = ext[1] = 0;
  if (c->cfg.field_kind == 1)
    ext[2] = c->cfg.field_amp * sin(2.0 * 3.141592653589793238 * c->cfg.field_freq * t);
  else
    ext[2] = t < c->cfg.tMag ? c->cfg.magFluxDens : 0.0;
}

void orc_step(orc_ctx* c, double dt, int noise_mode, const double* xi, uint64_t seed,
              double* B1, double* F1, double* B2, double* obs) {
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  int64_t n = c->n, n3 = 3 * n;
  double ext[3];
  ext_field(c, c->t, ext);
  orc_thermal(c, dt, noise_mode, xi, seed, c->tTorque, c->tField, c->tForce);
  orc_compute_interactions(c, B1, F1, NULL);
  /* IntegrationRot, HEUN_EULER branch with a fixed step (simulation.cpp:721-749, 866-867). */
  rk_coeffs(c, c->mm, c->ea, ext, c->k1m, c->k1e);
  for (int64_t k = 0; k < n3; k++) {
    c->c2e[k] = c->ea[k] + dt * c->k1e[k];
    c->c2m[k] = c->mm[k] + dt * c->k1m[k];
  }
  orc_compute_field(c, c->c2m, B2);
  rk_coeffs(c, c->c2m, c->c2e, ext, c->k2m, c->k2e);
  for (int64_t k = 0; k < n3; k++) {
    c->ea[k] += dt * (0.5 * c->k1e[k] + 0.5 * c->k2e[k]);
    c->mm[k] += dt * (0.5 * c->k1m[k] + 0.5 * c->k2m[k]);
  }
  for (int64_t i = 0; i < n; i++) {
    double nm = sqrt(AX(c->mm, i, 0, n) * AX(c->mm, i, 0, n) + AX(c->mm, i, 1, n) * AX(c->mm, i, 1, n) +
                     AX(c->mm, i, 2, n) * AX(c->mm, i, 2, n));
    double ne = sqrt(AX(c->ea, i, 0, n) * AX(c->ea, i, 0, n) + AX(c->ea, i, 1, n) * AX(c->ea, i, 1, n) +
                     AX(c->ea, i, 2, n) * AX(c->ea, i, 2, n));
    for (int a = 0; a < 3; a++) {
      AX(c->mm, i, a, n) /= nm;
      AX(c->ea, i, a, n) /= ne;
    }
  }
  /* IntegrationTrans + ApplyBoundaryCondArr (simulation.cpp:959-962, 610-620). */
  double L = c->cfg.lBox, h = L / 2;
  for (int a = 0; a < 3; a++)
    for (int64_t i = 0; i < n; i++) {
      double x = AX(c->pos, i, a, n) + dt * (AX(c->force, i, a, n) / c->zetaTrans[i]);
      x -= L * (double)(x > h);
      x += L * (double)(x < -h);
      AX(c->pos, i, a, n) = x;
    }
  clock_gettime(CLOCK_MONOTONIC, &t1);
  c->last_seconds = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
  /* EvalTransCoeffs (postprocessing.cpp:167-187) and mz (simulation.cpp:514-515). */
  double msd[3] = {0, 0, 0}, mz = 0;
  for (int a = 0; a < 3; a++)
    for (int64_t i = 0; i < n; i++) {
      double x = AX(c->pos, i, a, n);
      double tp = x + round((AX(c->truePos, i, a, n) - x) / L) * L;
      AX(c->truePos, i, a, n) = tp;
      double d = tp - AX(c->posRef, i, a, n);
      msd[a] += d * d;
    }
  for (int64_t i = 0; i < n; i++) mz += AX(c->mm, i, 2, n);
  if (obs) {
    obs[0] = c->t;
    obs[1] = mz / (double)n;
    for (int a = 0; a < 3; a++) obs[2 + a] = msd[a] / (double)n;
    obs[5] = c->Pxy / c->volBox;
    obs[6] = c->Pxz / c->volBox;
    obs[7] = c->Pyz / c->volBox;
  }
  c->t += dt;
  c->step++;
}

/* ------------------------------------------------------- adaptive solvers */

/* Normalises the rows of mm and ea (simulation.cpp:869-870) and moves the
 * particles with the step-start force for deltaTused (IntegrationTrans +
 * ApplyBoundaryCondArr, simulation.cpp:959-962, 610-620), then the records
 * (EvalTransCoeffs, postprocessing.cpp:167-187; mz, simulation.cpp:514-515). */
static void finish_step(orc_ctx* c, double used, double* obs) {
  int64_t n = c->n;
  for (int64_t i = 0; i < n; i++) {
    double nm = sqrt(AX(c->mm, i, 0, n) * AX(c->mm, i, 0, n) + AX(c->mm, i, 1, n) * AX(c->mm, i, 1, n) +
                     AX(c->mm, i, 2, n) * AX(c->mm, i, 2, n));
    double ne = sqrt(AX(c->ea, i, 0, n) * AX(c->ea, i, 0, n) + AX(c->ea, i, 1, n) * AX(c->ea, i, 1, n) +
                     AX(c->ea, i, 2, n) * AX(c->ea, i, 2, n));
    for (int a = 0; a < 3; a++) {
      AX(c->mm, i, a, n) /= nm;
      AX(c->ea, i, a, n) /= ne;
    }
  }
  double L = c->cfg.lBox, h = L / 2;
  for (int a = 0; a < 3; a++)
    for (int64_t i = 0; i < n; i++) {
      double x = AX(c->pos, i, a, n) + used * (AX(c->force, i, a, n) / c->zetaTrans[i]);
      x -= L * (double)(x > h);
      x += L * (double)(x < -h);
      AX(c->pos, i, a, n) = x;
    }
  double msd[3] = {0, 0, 0}, mz = 0;
  for (int a = 0; a < 3; a++)
    for (int64_t i = 0; i < n; i++) {
      double x = AX(c->pos, i, a, n);
      double tp = x + round((AX(c->truePos, i, a, n) - x) / L) * L;
      AX(c->truePos, i, a, n) = tp;
      double d = tp - AX(c->posRef, i, a, n);
      msd[a] += d * d;
    }
  for (int64_t i = 0; i < n; i++) mz += AX(c->mm, i, 2, n);
  if (obs) {
    obs[0] = c->t;
    obs[1] = mz / (double)n;
    for (int a = 0; a < 3; a++) obs[2 + a] = msd[a] / (double)n;
    obs[5] = c->Pxy / c->volBox;
    obs[6] = c->Pxz / c->volBox;
    obs[7] = c->Pyz / c->volBox;
  }
  c->t += used;
  c->step++;
}

/* row-wise Euclidean norm, maximum over rows (`rowwise().norm().maxCoeff()`) */
static double max_row_norm(const double* v, int64_t n) {
  double m = 0;
  for (int64_t i = 0; i < n; i++) {
    double s = AX(v, i, 0, n) * AX(v, i, 0, n) + AX(v, i, 1, n) * AX(v, i, 1, n) + AX(v, i, 2, n) * AX(v, i, 2, n);
    s = sqrt(s);
    if (s > m) m = s;
  }
  return m;
}

/* AdjustTimeStep (simulation.cpp:912-951), including its clamp: the
 * min(., deltaTmax) result is overwritten by max(., deltaTmin), so deltaTmax
 * is never applied.  On a rejection the thermal field, torque and force are
 * rescaled by sqrt(new / old). */
static void adjust_time_step(orc_ctx* c, const orc_adapt* ad, double error, double power, double* dt, int* cond,
                             int* noFailed) {
  double tnew;
  if (error > ad->absTol) {
    if (*noFailed) {
      *noFailed = 0;
      double q = 0.9 * pow(ad->absTol / error, power);
      tnew = fmax(ad->dtMin, (*dt) * fmax(0.1, q));
    } else {
      tnew = fmax(ad->dtMin, (*dt) * 0.5);
    }
    double f = sqrt(tnew / (*dt));
    for (int64_t k = 0; k < 3 * c->n; k++) {
      c->tField[k] *= f;
      c->tTorque[k] *= f;
      c->tForce[k] *= f;
    }
  } else {
    if (*noFailed)
      tnew = (*dt) * fmin(fmax(0.9 * pow(ad->absTol / error, power), 0.2), 5.0);
    else
      tnew = *dt;
    *cond = 0;
  }
  *dt = fmin(tnew, ad->dtMax);
  *dt = fmax(tnew, ad->dtMin);
}

/* stage coordinates y0 + dt * sum_j a_j k_j, written to (scm, sce) */
static void stage_coords(orc_ctx* c, double dt, int ns, const double* a) {
  int64_t n3 = 3 * c->n;
  for (int64_t k = 0; k < n3; k++) {
    double sm = 0, se = 0;
    for (int j = 0; j < ns; j++) {
      if (a[j] == 0.0) continue;
      sm += a[j] * c->skm[j][k];
      se += a[j] * c->ske[j][k];
    }
    c->sce[k] = c->ea[k] + dt * se;
    c->scm[k] = c->mm[k] + dt * sm;
  }
}

void orc_step_adaptive(orc_ctx* c, const orc_adapt* ad, double* deltaT, int noise_mode, const double* xi,
                       uint64_t seed, double* obs, double* used_out, int* attempts_out) {
  int64_t n = c->n, n3 = 3 * n;
  double ext[3];
  ext_field(c, c->t, ext);
  orc_thermal(c, *deltaT, noise_mode, xi, seed, c->tTorque, c->tField, c->tForce);
  orc_compute_interactions(c, NULL, NULL, NULL);
  /* IntegrationRot (simulation.cpp:707-871).  The slopes of stage 1 use the
   * demagnetising field currently held: the step-start field on the first
   * attempt, the last stage's field after a rejection (as the reference). */
  static const double A_he[2][1] = {{0}, {1.0}};
  static const double A_bs[4][3] = {{0, 0, 0}, {1.0 / 2.0, 0, 0}, {0, 3.0 / 4.0, 0}, {2.0 / 9.0, 1.0 / 3.0, 4.0 / 9.0}};
  static const double A_dp[7][6] = {
      {0, 0, 0, 0, 0, 0},
      {1.0 / 5.0, 0, 0, 0, 0, 0},
      {3.0 / 40.0, 9.0 / 40.0, 0, 0, 0, 0},
      {44.0 / 45.0, -56.0 / 15.0, 32.0 / 9.0, 0, 0, 0},
      {19372.0 / 6561.0, -25360.0 / 2187.0, 64448.0 / 6561.0, -212.0 / 729.0, 0, 0},
      {9017.0 / 3168.0, -355.0 / 33.0, 46732.0 / 5247.0, 49.0 / 176.0, -5103.0 / 18656.0, 0},
      {35.0 / 384.0, 0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0}};
  static const double E_he[2] = {0.5, -0.5};
  static const double E_bs[4] = {-5.0 / 72.0, 1.0 / 12.0, 1.0 / 9.0, -1.0 / 8.0};
  static const double E_dp[7] = {71.0 / 57600.0, 0, -71.0 / 16695.0, 71.0 / 1920.0, -17253.0 / 339200.0, 22.0 / 525.0,
                                 -1.0 / 40.0};
  int S;
  double power;
  const double* E;
  if (ad->solver == 1) {
    S = 4;
    power = 1.0 / 3.0;
    E = E_bs;
  } else if (ad->solver == 2) {
    S = 7;
    power = 1.0 / 5.0;
    E = E_dp;
  } else {
    S = 2;
    power = 1.0 / 2.0;
    E = E_he;
  }
  int cond = 1, noFailed = 1, attempts = 0;
  double used = *deltaT;
  while (cond) {
    const double dt = *deltaT;
    attempts++;
    rk_coeffs(c, c->mm, c->ea, ext, c->skm[0], c->ske[0]);
    for (int s = 1; s < S; s++) {
      const double* a = ad->solver == 1 ? A_bs[s] : (ad->solver == 2 ? A_dp[s] : A_he[s]);
      stage_coords(c, dt, s, a);
      orc_compute_field(c, c->scm, NULL);
      rk_coeffs(c, c->scm, c->sce, ext, c->skm[s], c->ske[s]);
    }
    for (int64_t k = 0; k < n3; k++) {
      double e = 0;
      for (int j = 0; j < S; j++)
        if (E[j] != 0.0) e += E[j] * c->skm[j][k];
      c->ebuf[k] = e;
    }
    double err = dt * max_row_norm(c->ebuf, n);
    used = dt;
    adjust_time_step(c, ad, err, power, deltaT, &cond, &noFailed);
  }
  if (ad->solver == 1) {
    /* the third-order solution: the last stage's coordinates */
    memcpy(c->mm, c->scm, (size_t)n3 * sizeof(double));
    memcpy(c->ea, c->sce, (size_t)n3 * sizeof(double));
  } else {
    const double* b = ad->solver == 2 ? A_dp[6] : NULL;
    for (int64_t k = 0; k < n3; k++) {
      double sm, se;
      if (ad->solver == 2) {
        sm = se = 0;
        for (int j = 0; j < 6; j++) {
          if (b[j] == 0.0) continue;
          sm += b[j] * c->skm[j][k];
          se += b[j] * c->ske[j][k];
        }
      } else {
        sm = 0.5 * c->skm[0][k] + 0.5 * c->skm[1][k];
        se = 0.5 * c->ske[0][k] + 0.5 * c->ske[1][k];
      }
      c->ea[k] += used * se;
      c->mm[k] += used * sm;
    }
  }
  finish_step(c, used, obs);
  if (used_out) *used_out = used;
  if (attempts_out) *attempts_out = attempts;
}

/* ------------------------------------------------------------ error model */

/* FunRealError (interaction.cpp:330-338). */
double orc_fun_real_error(double x, double M, double fAl, double lBox, double rc, double n,
                          double facEwald, double errTol) {
  double a = x * rc;
  double b = M / sqrt(pow(lBox, 3.0) * pow(rc, 9.0) * n * pow(x, 4.0));
  double cc = 4.0 * pow(a, 4.0) + 6.0 * pow(a, 2.0) + 3.0;
  double d = 8.0 * pow(a, 6.0) + 20.0 * pow(a, 4.0) + 30.0 * pow(a, 2.0) + 15.0;
  return facEwald * b * sqrt(13.0 / 6.0 * cc * cc + 2.0 / 15.0 * d * d - 13.0 / 15.0 * cc * d) * exp(-a * a) / fAl -
         errTol / sqrt(2.0);
}

/* FunRezError (interaction.cpp:344-347). */
double orc_fun_rez_error(double x, double M, double fAl, double lBox, double alpha, double n,
                         double facEwald, double my_pi, double errTol) {
  return facEwald * 8.0 * M * my_pi / pow(lBox, 3.0) * alpha *
             sqrt(2.0 * my_pi * x * x * x / (15.0 * n)) * exp(-pow(my_pi * x / (alpha * lBox), 2.0)) / fAl -
         errTol / sqrt(2.0);
}

/* The alpha and kc search of CompEwaldParams for one rc (interaction.cpp:190-257). */
int orc_ewald_for_rc(double rc, double M, double fAl, double lBox, double n, double facEwald,
                     double my_pi, double errTol, double* alpha, double* kc) {
  const int steps = 10000;
  int i1 = 0, i2 = 0, rcfail = 0;
  double x0 = 0, v0 = 0, x1 = 0, v1 = 0;
  for (int i = 0; i < steps; i++) {
    double x = 2e8 * (double)i / (steps - 1);
    double v = orc_fun_real_error(x, M, fAl, lBox, rc, n, facEwald, errTol);
    if (v < 0) { i2 = i; i1 = i - 1; x1 = x; v1 = v; break; }
    x0 = x; v0 = v;
  }
  if (i1 == 0 || i2 == 0) rcfail = 1;
  double a = -v0 / (v1 - v0) * (x1 - x0) + x0;
  *alpha = a;
  int maxIdx = 0;
  double maxVal = -1e300;
  double* vals = (double*)malloc(sizeof(double) * steps);
  for (int i = 0; i < steps; i++) {
    double x = 30.0 * (double)i / (steps - 1);
    vals[i] = orc_fun_rez_error(x, M, fAl, lBox, a, n, facEwald, my_pi, errTol);
    if (vals[i] > maxVal) { maxVal = vals[i]; maxIdx = i; }
  }
  if (maxVal < 0) { free(vals); return 2; }
  double k = 0;
  int found = 0;
  for (int i = maxIdx; i < steps; i++)
    if (vals[i] < 0) {
      double xa = 30.0 * (double)(i - 1) / (steps - 1), xb = 30.0 * (double)i / (steps - 1);
      k = -vals[i - 1] / (vals[i] - vals[i - 1]) * (xb - xa) + xa;
      found = 1;
      break;
    }
  free(vals);
  if (!found) return 3;
  if (k < 2.0) k = 2.0;
  *kc = k;
  return rcfail;
}

int64_t orc_pairs(const orc_ctx* c) { return c->pairs; }
double orc_last_seconds(const orc_ctx* c) { return c->last_seconds; }

/* InitCoordsFromSketch's random sequential addition (simulation.cpp:241-264)
 * in index order: candidate uniform in [-(L/2 - rHydr_i), L/2 - rHydr_i]^3,
 * rejected if it overlaps a placed hydrodynamic sphere (periodic distances),
 * with a seeded splitmix64 generator instead of EigenRand's.  pos: N x 3
 * column-major.  Returns 0, or 1 if a particle found no place. */
static uint64_t sm64(uint64_t* x) {
  uint64_t z = (*x += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static double sm64_unit(uint64_t* x) { return (double)(sm64(x) >> 11) * (1.0 / 9007199254740992.0); }

/* Placement by random sequential addition with a stream per particle (the
 * restatement the GPU placement md_place_rsa is checked against bit for bit):
 * the particles in `order` (NULL: index order, as the reference) each take
 * the first attempt t = 0, 1, ... whose position overlaps no particle placed
 * before it -- distance below the sum of the hydrodynamic radii, plain
 * distance inside the box as in the reference's InitCoordsFromSketch
 * (src/simulation.cpp:241-264).  Attempt t of particle i: Philox4x32-10 with
 * key {seed_lo, seed_hi} and counters {i, t_lo, t_hi, 0xA5A5A5A5},
 * {i, t_lo, t_hi, 0x5A5A5A5A}; uniforms u = ((w_a << 21) ^ (w_b >> 11)) 2^-53
 * from the word pairs (0,1), (2,3) of the first and (0,1) of the second;
 * coordinate (2u - 1)(L/2 - r_i), the reference's box-interior draw.  The
 * build turns floating-point contraction off, so the distance test rounds
 * like the GPU's.  tries (optional) gets each particle's accepted attempt. */
static void rsa_cand(uint64_t seed, int64_t i, int64_t t, double ext, double x[3]) {
  uint32_t a[4] = {(uint32_t)i, (uint32_t)t, (uint32_t)((uint64_t)t >> 32), 0xA5A5A5A5u};
  uint32_t b[4] = {(uint32_t)i, (uint32_t)t, (uint32_t)((uint64_t)t >> 32), 0x5A5A5A5Au};
  philox4x32_10(a, (uint32_t)seed, (uint32_t)(seed >> 32));
  philox4x32_10(b, (uint32_t)seed, (uint32_t)(seed >> 32));
  const uint32_t w[6] = {a[0], a[1], a[2], a[3], b[0], b[1]};
  for (int c = 0; c < 3; c++) {
    const uint64_t m = ((uint64_t)w[2 * c] << 21) ^ (uint64_t)(w[2 * c + 1] >> 11);
    const double u = (double)m * 1.1102230246251565e-16; /* 2^-53 */
    x[c] = (2.0 * u - 1.0) * ext;
  }
}

int orc_rsa_philox(int64_t n, double lBox, const double* rHydr, uint64_t seed, const int64_t* order,
                   int64_t max_tries, double* pos, int64_t* tries) {
  for (int64_t q = 0; q < n; q++) {
    const int64_t i = order ? order[q] : q;
    const double ri = rHydr[i], ext = 0.5 * lBox - ri;
    int placed = 0;
    for (int64_t t = 0; t < max_tries && !placed; t++) {
      double x[3];
      rsa_cand(seed, i, t, ext, x);
      placed = 1;
      for (int64_t p = 0; p < q && placed; p++) {
        const int64_t j = order ? order[p] : p;
        const double dx = AX(pos, j, 0, n) - x[0], dy = AX(pos, j, 1, n) - x[1], dz = AX(pos, j, 2, n) - x[2];
        const double s = ri + rHydr[j];
        const double r2 = dx * dx + dy * dy + dz * dz;
        if (r2 < s * s) placed = 0;
      }
      if (placed) {
        for (int c = 0; c < 3; c++) AX(pos, i, c, n) = x[c];
        if (tries) tries[i] = t;
      }
    }
    if (!placed) return 1;
  }
  return 0;
}

int orc_rsa(int64_t n, double lBox, const double* rHydr, uint64_t seed, int64_t max_tries, double* pos) {
  uint64_t st = seed;
  double L = lBox;
  for (int64_t i = 0; i < n; i++) {
    int placed = 0;
    for (int64_t t = 0; t < max_tries && !placed; t++) {
      double x[3];
      for (int a = 0; a < 3; a++) x[a] = (2.0 * sm64_unit(&st) - 1.0) * (L / 2.0 - rHydr[i]);
      placed = 1;
      const double h = L / 2.0;
      for (int64_t j = 0; j < i && placed; j++) {
        const double s = rHydr[i] + rHydr[j];
        double r2 = 0;
        int far = 0;
        for (int a = 0; a < 3 && !far; a++) {
          double d = AX(pos, j, a, n) - x[a];
          d -= L * (double)(d > h);
          d += L * (double)(d < -h);
          far = d > s || d < -s;
          r2 += d * d;
        }
        if (!far && r2 < s * s) placed = 0;
      }
      if (placed)
        for (int a = 0; a < 3; a++) AX(pos, i, a, n) = x[a];
    }
    if (!placed) return 1;
  }
  return 0;
}
