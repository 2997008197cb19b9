/*
 * moc_oracle.c -- CPU oracle (test infrastructure only; see moc_oracle.h).
 *
 * Plain C99 restatement of the SimpleMOC solver arithmetic.  Every float
 * expression keeps the reference's operand order and its float/double
 * promotions, so that a build with -O2 -ffp-contract=off rounds exactly as the
 * reference's serial build (src/Makefile with OPTIMIZE=no fast-math) does.
 * File:line citations are relative to the reference project root.
 */
#include "moc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------------ */
/* exponential table: src/utils.c:48-78                                      */
/* ------------------------------------------------------------------------ */
int32_t oracle_exp_table_size(float precision, float maxval)
{
  /* utils.c:54 -- float operands promoted to double */
  return (int32_t)(maxval * sqrt(1.0 / (8.0 * precision * 0.01)));
}

void oracle_build_exp_table(float precision, float maxval, float *values,
                            float *dx_out, float *maxval_out, int32_t *n_out)
{
  int32_t N = oracle_exp_table_size(precision, maxval);
  float dx = maxval / (float)N;                         /* utils.c:57 */
  for (int32_t n = 0; n < N; n++) {                     /* utils.c:63-69 */
    float e = (float)exp(-n * dx);                      /* (-n) * dx in float */
    values[2 * n] = -e;
    values[2 * n + 1] = 1 + (n * dx - 1) * e;
  }
  *dx_out = dx;
  *maxval_out = maxval - dx;                            /* utils.c:74 */
  *n_out = N;
}

/* src/solver.c:1441-1464 */
float oracle_interpolate(const float *values, float dx, float maxval, float x)
{
  if (x > maxval)
    return 1.0f;
  int interval = (int)(x / dx + 0.5f * dx);
  float slope = values[2 * interval];
  float intercept = values[2 * interval + 1];
  return slope * x + intercept;
}

/* src/utils.c:29-45 */
float oracle_pairwise_sum(const float *v, int64_t n)
{
  float sum = 0;
  if (n <= 16) {
    for (int64_t i = 0; i < n; i++)
      sum += v[i];
  } else {
    sum = oracle_pairwise_sum(v, n / 2) + oracle_pairwise_sum(v + n / 2, n - n / 2);
  }
  return sum;
}

static double pairwise64(const double *v, int64_t n)
{
  double sum = 0;
  if (n <= 16) {
    for (int64_t i = 0; i < n; i++)
      sum += v[i];
  } else {
    sum = pairwise64(v, n / 2) + pairwise64(v + n / 2, n - n / 2);
  }
  return sum;
}

/* ------------------------------------------------------------------------ */
/* traversal quantities                                                      */
/* ------------------------------------------------------------------------ */
float oracle_mu(float polar_angle)
{
  return (float)cos(polar_angle);                       /* solver.c:373 */
}

float oracle_ds(float len, float polar_angle)
{
  return (float)(len / sin(polar_angle));               /* solver.c:382-383 */
}

/* Explicit-track height rule: z <- z + ds*mu wrapped into [0, H). */
float oracle_advance_z(float z, float ds, float mu, float domain_height)
{
  float dzt = ds * mu;
  z = z + dzt;
  while (z >= domain_height)
    z -= domain_height;
  while (z < 0.0f)
    z += domain_height;
  return z;
}

static float fine_dz(const oracle_problem *P)
{
  /* solver.c:38: float / int */
  return P->height / (P->F * P->decomp_ax * P->cai);
}

/* ------------------------------------------------------------------------ */
/* one segment: attenuate_fluxes (solver.c:14-280) / attenuate_FSR_fluxes    */
/* (solver.c:1040-1138)                                                      */
/* ------------------------------------------------------------------------ */
/* Computes the tally vector of one segment into tally[G], updates psi, and
 * returns the fine axial interval the tally belongs to. */
static int attenuate_core(const oracle_problem *P, float z, float ds, float mu,
                          float weight, const float *q, const float *sigt_row,
                          float *psi, float *tally_out)
{
  const int G = P->G, F = P->F;
  float dz = fine_dz(P);
  float zin = z - dz * ((int)(z / dz) + 0.5f);          /* solver.c:41-42 */
  int fine_id = (int)(z / dz) % F;                      /* solver.c:45 */

  if (P->axial_exp == 0) {
    /* attenuate_FSR_fluxes: solver.c:1064-1131 */
    float w = weight * mu;
    const float *qf = q + (int64_t)fine_id * G;
    for (int g = 0; g < G; g++) {
      float sigT = sigt_row[g];
      float tau = sigT * ds;
      float e = oracle_interpolate(P->table, P->table_dx, P->table_maxval, tau);
      float qq = qf[g] / sigT;
      float delta_psi = (psi[g] - qq) * e;
      tally_out[g] = w * delta_psi;
      psi[g] -= delta_psi;
    }
    return fine_id;
  }

  float mu2 = mu * mu;                                  /* solver.c:50 */
  int r0;
  if (fine_id == 0) {                                   /* solver.c:55-83 */
    zin -= dz;
    r0 = fine_id;
  } else if (fine_id == F - 1) {                        /* solver.c:84-112 */
    zin += dz;
    r0 = fine_id - 2;
  } else {                                              /* solver.c:113-138 */
    r0 = fine_id - 1;
  }
  const float *row1 = q + (int64_t)r0 * G;
  const float *row2 = row1 + G;
  const float *row3 = row2 + G;

  for (int g = 0; g < G; g++) {
    float y1 = row1[g], y2 = row2[g], y3 = row3[g];
    float c0 = y2;                                      /* solver.c:74-81 */
    float c1 = (y1 - y3) / (2.f * dz);
    float c2 = (y1 - 2.f * y2 + y3) / (2.f * dz * dz);
    float q0 = c0 + c1 * zin + c2 * zin * zin;
    float q1 = c1 + 2.f * c2 * zin;
    float q2 = c2;

    float sigT = sigt_row[g];                           /* solver.c:149-153 */
    float tau = sigT * ds;
    float sigT2 = sigT * sigT;
    float e = oracle_interpolate(P->table, P->table_dx, P->table_maxval, tau);
    /* solver.c:175-176: the precedence is the reference's (reuse) */
    float reuse = tau * (tau - 2.f) + 2.f * e / (sigT * sigT2);
    float p = psi[g];
    /* solver.c:195-198 */
    float fi = (q0 * tau + (sigT * p - q0) * e) / sigT2 + q1 * mu * reuse
             + q2 * mu2 * (tau * (tau * (tau - 3.f) + 6.f) - 6.f * e)
               / (3.f * sigT2 * sigT2);
    tally_out[g] = weight * fi;                         /* solver.c:209 */
    float t1 = q0 * e / sigT;                           /* solver.c:238-268 */
    float t2 = q1 * mu * (tau - e) / sigT2;
    float t3 = q2 * mu2 * reuse;
    float t4 = p * (1.f - e);
    psi[g] = t1 + t2 + t3 + t4;                         /* solver.c:278 */
  }
  return fine_id;
}

void oracle_attenuate(const oracle_problem *P, float z, float ds, float mu,
                      float weight, const float *q, float *phi,
                      const float *sigt_row, float *psi)
{
  float tally[4096];
  float *t = P->G <= 4096 ? tally : (float *)malloc(sizeof(float) * (size_t)P->G);
  int fine_id = attenuate_core(P, z, ds, mu, weight, q, sigt_row, psi, t);
  float *flux = phi + (int64_t)fine_id * P->G;
  for (int g = 0; g < P->G; g++)                        /* solver.c:221-224 */
    flux[g] += t[g];
  if (t != tally)
    free(t);
}

/* ------------------------------------------------------------------------ */
/* sweeps                                                                    */
/* ------------------------------------------------------------------------ */
static void sweep_one_track(const oracle_problem *P, const float *fine_source,
                            float *fine_flux, int64_t t, float *psi)
{
  const int64_t G = P->G, F = P->F, S = P->S;
  const int64_t PZ = (int64_t)P->P * P->Z;
  int64_t i = t / PZ;
  int j = (int)((t / P->Z) % P->P);
  float theta = P->polar_angles[j];
  float mu = oracle_mu(theta);
  float Hd = P->height / P->decomp_ax;
  float weight = P->p_weight[t] * P->az_weight[i];      /* solver.c:49 */
  float z = P->z0[t];
  for (int64_t n = 0; n < S; n++) {
    float ds = oracle_ds(P->seg_len[i * S + n], theta);
    int64_t s = P->seg_src[t * S + n];
    oracle_attenuate(P, z, ds, mu, weight, fine_source + s * F * G,
                     fine_flux + s * F * G, P->sigt + (int64_t)P->src_sigt[s] * G, psi);
    z = oracle_advance_z(z, ds, mu, Hd);
  }
}

int64_t oracle_sweep(const oracle_problem *P, const float *fine_source,
                     float *fine_flux, float *psi_f)
{
  const int64_t N3D = P->N2D * P->P * P->Z;
  for (int64_t t = 0; t < N3D; t++)
    sweep_one_track(P, fine_source, fine_flux, t, psi_f + t * P->G);
  return N3D * P->S;
}

void oracle_sweep_tracks(const oracle_problem *P, const float *fine_source,
                         const int64_t *tracks, int64_t n, const float *psi_in,
                         float *psi_out, float *fine_flux)
{
  const int64_t G = P->G;
  float *scratch = NULL;
  if (!fine_flux) {
    scratch = (float *)calloc((size_t)(P->NS * P->F * G), sizeof(float));
    fine_flux = scratch;
  }
  for (int64_t m = 0; m < n; m++) {
    int64_t t = tracks[m];
    memcpy(psi_out + m * G, psi_in + t * G, (size_t)G * sizeof(float));
    sweep_one_track(P, fine_source, fine_flux, t, psi_out + m * G);
  }
  free(scratch);
}

int oracle_omp_max_threads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 0;
#endif
}

#ifdef _OPENMP
/* One segment with the tally added under the fine region's lock, as the
 * reference's OpenMP build does (solver.c:212-228). */
static void attenuate_locked(const oracle_problem *P, float z, float ds, float mu,
                             float weight, const float *q, float *phi,
                             const float *sigt_row, float *psi, float *tally,
                             omp_lock_t *locks)
{
  int fine_id = attenuate_core(P, z, ds, mu, weight, q, sigt_row, psi, tally);
  float *flux = phi + (int64_t)fine_id * P->G;
  omp_set_lock(locks + fine_id);
  for (int g = 0; g < P->G; g++)
    flux[g] += tally[g];
  omp_unset_lock(locks + fine_id);
}
#endif

int64_t oracle_sweep_omp(const oracle_problem *P, const float *fine_source,
                         float *fine_flux, float *psi_f, int nthreads)
{
#ifdef _OPENMP
  const int64_t G = P->G, F = P->F, S = P->S;
  const int64_t N3D = P->N2D * P->P * P->Z;
  const int64_t PZ = (int64_t)P->P * P->Z;
  int64_t nlocks = P->NS * F;
  omp_lock_t *locks = (omp_lock_t *)malloc(sizeof(omp_lock_t) * (size_t)nlocks);
  for (int64_t l = 0; l < nlocks; l++)
    omp_init_lock(&locks[l]);
  if (nthreads <= 0)
    nthreads = omp_get_max_threads();
  float Hd = P->height / P->decomp_ax;
#pragma omp parallel num_threads(nthreads)
  {
    float *buf = (float *)malloc(sizeof(float) * (size_t)G);
#pragma omp for schedule(dynamic, 64)
    for (int64_t t = 0; t < N3D; t++) {
      int64_t i = t / PZ;
      int j = (int)((t / P->Z) % P->P);
      float theta = P->polar_angles[j];
      float mu = oracle_mu(theta);
      float weight = P->p_weight[t] * P->az_weight[i];
      float z = P->z0[t];
      float *psi = psi_f + t * G;
      for (int64_t n = 0; n < S; n++) {
        float ds = oracle_ds(P->seg_len[i * S + n], theta);
        int64_t s = P->seg_src[t * S + n];
        attenuate_locked(P, z, ds, mu, weight, fine_source + s * F * G,
                         fine_flux + s * F * G, P->sigt + (int64_t)P->src_sigt[s] * G,
                         psi, buf, locks + s * F);
        z = oracle_advance_z(z, ds, mu, Hd);
      }
    }
    free(buf);
  }
  for (int64_t l = 0; l < nlocks; l++)
    omp_destroy_lock(&locks[l]);
  free(locks);
  return N3D * S;
#else
  (void)nthreads;
  return oracle_sweep(P, fine_source, fine_flux, psi_f);
#endif
}

/* ------------------------------------------------------------------------ */
/* the reference traversal, src/solver.c:283-552 (serial build)              */
/* ------------------------------------------------------------------------ */
/* src/solver.c:895-907: float z, float dz */
static int pos_interval(float z, float dz) { return (int)(z / dz); }
static int neg_interval(float z, float dz) { return ceil(z / dz); }

int64_t oracle_ref_sweep(const oracle_problem *P, const oracle_refgeo *R,
                         const float *fine_source, float *fine_flux, float *psi_f,
                         float *z_height, const int32_t *ids)
{
  const int64_t G = P->G, F = P->F, NS = P->NS;
  /* solver.c:288-289: float height / int -> float, held in double */
  double node_delta_z = P->height / P->decomp_ax;
  double fine_delta_z = node_delta_z / (P->cai * P->F);
  int64_t seq = 0;
  for (int64_t i = 0; i < R->N2D; i++) {                       /* solver.c:348 */
    int pos_z_dir = 1;
    const int64_t nseg = R->seg_off[i + 1] - R->seg_off[i];
    const float *len = R->seg_len + R->seg_off[i];
    for (int j = 0; j < P->P; j++) {                           /* solver.c:368 */
      if (j == P->P / 2)
        pos_z_dir = 0;
      float p_angle = P->polar_angles[j];
      float mu = cos(p_angle);
      int begin_stacked = 0;
      int end_stacked = P->Z;
      for (int64_t n = 0; n < nseg; n++) {                     /* solver.c:379 */
        float s_full = len[n] / sin(p_angle);
        float ds = 0;
        for (int k = begin_stacked; k < end_stacked; k++) {    /* solver.c:389 */
          float s = s_full;
          const int64_t t = ((int64_t)i * P->P + j) * P->Z + k;
          int seg_complete = 0;
          int curr_interval = pos_z_dir ? pos_interval(z_height[t], fine_delta_z)
                                        : neg_interval(z_height[t], fine_delta_z);
          while (!seg_complete) {                              /* solver.c:409 */
            int reset = 0;
            float z = z_height[t] + s * cos(p_angle);
            int new_interval = pos_z_dir ? pos_interval(z, fine_delta_z)
                                         : neg_interval(z, fine_delta_z);
            if (new_interval == curr_interval) {
              seg_complete = 1;
              ds = s;
            } else {
              if (pos_z_dir) {
                curr_interval++;
                z = fine_delta_z * (float)curr_interval;
              } else {
                curr_interval--;
                z = fine_delta_z * (float)curr_interval;
              }
              ds = (z - z_height[t]) / cos(p_angle);
              s -= ds;
              if (s <= 0)
                seg_complete = 1;
              if (z <= 0 || z >= node_delta_z) {               /* solver.c:460-473 */
                seg_complete = 1;
                if (pos_z_dir)
                  end_stacked--;
                else
                  begin_stacked++;
                reset = 1;
              }
            }
            int64_t qsr = ids ? ids[seq] : (int64_t)(rand() % NS);   /* solver.c:481 */
            seq++;
            float weight = R->p_weight[t] * R->az_weight[i];
            oracle_attenuate(P, z_height[t], ds, mu, weight, fine_source + qsr * F * G,
                             fine_flux + qsr * F * G, P->sigt + (int64_t)P->src_sigt[qsr] * G,
                             psi_f + t * G);
            if (n == nseg - 1 || reset) {                      /* solver.c:514-523 */
              if (pos_z_dir)
                z_height[t] = R->axial_z_sep * k;
              else
                z_height[t] = R->axial_z_sep * (k + 1);
            } else {
              z_height[t] = z;
            }
          }
        }
      }
    }
  }
  return seq;
}

/* ------------------------------------------------------------------------ */
/* post-sweep steps, serial build semantics                                  */
/* ------------------------------------------------------------------------ */
void oracle_renormalize(const oracle_problem *P, float *fine_flux,
                        float *psi_f, float *psi_b)
{
  const int64_t G = P->G, F = P->F, NS = P->NS;
  float *fission_rates = (float *)malloc(sizeof(float) * (size_t)NS);
  float *fine_rates = (float *)malloc(sizeof(float) * (size_t)F);
  float *g_rates = (float *)malloc(sizeof(float) * (size_t)G);
  for (int64_t i = 0; i < NS; i++) {                    /* solver.c:1161-1173 */
    const float *x = P->xs + (int64_t)P->src_xs[i] * G * 3;
    for (int64_t j = 0; j < F; j++) {
      const float *phi = fine_flux + (i * F + j) * G;
      for (int64_t g = 0; g < G; g++)
        g_rates[g] = phi[g] * P->vol[i] * x[g * 3 + 0];
      fine_rates[j] = oracle_pairwise_sum(g_rates, G);
    }
    fission_rates[i] = oracle_pairwise_sum(fine_rates, F);
  }
  float total = oracle_pairwise_sum(fission_rates, NS);   /* solver.c:1174 */
  float norm_factor = 1.0 / total;                        /* solver.c:1203 */
  for (int64_t i = 0; i < NS; i++) {                      /* solver.c:1207-1214 */
    float adjust = norm_factor * 4 * M_PI * F / P->vol[i];
    float *phi = fine_flux + i * F * G;
    for (int64_t k = 0; k < F * G; k++)
      phi[k] *= adjust;
  }
  const int64_t n = P->N2D * P->P * P->Z * G;             /* solver.c:1219-1226 */
  for (int64_t k = 0; k < n; k++) {
    psi_f[k] *= norm_factor;
    psi_b[k] *= norm_factor;
  }
  free(fission_rates);
  free(fine_rates);
  free(g_rates);
}

float oracle_update_sources(const oracle_problem *P, const float *fine_flux,
                            float *fine_source, float keff)
{
  const int64_t G = P->G, F = P->F, NS = P->NS;
  float inverse_k = 1.0 / keff;                           /* solver.c:1241 */
  float *group_res = (float *)malloc(sizeof(float) * (size_t)G);
  float *fine_res = (float *)malloc(sizeof(float) * (size_t)F);
  float *residuals = (float *)malloc(sizeof(float) * (size_t)NS);
  float *fission_rates = (float *)malloc(sizeof(float) * (size_t)G);
  float *scatter_rates = (float *)malloc(sizeof(float) * (size_t)G);
  for (int64_t i = 0; i < NS; i++) {
    const float *x = P->xs + (int64_t)P->src_xs[i] * G * 3;
    const float *S = P->scatter + (int64_t)P->src_xs[i] * G * G;
    for (int64_t j = 0; j < F; j++) {
      const float *phi = fine_flux + (i * F + j) * G;
      float *q = fine_source + (i * F + j) * G;
      for (int64_t g = 0; g < G; g++)                     /* solver.c:1266-1271 */
        fission_rates[g] = phi[g] * x[g * 3 + 0];
      float fission_source = oracle_pairwise_sum(fission_rates, G);
      fission_source *= inverse_k;
      for (int64_t g = 0; g < G; g++) {                   /* solver.c:1274-1300 */
        for (int64_t g2 = 0; g2 < G; g2++)
          scatter_rates[g2] = S[g * G + g2] * phi[g2];
        float scatter_source = oracle_pairwise_sum(scatter_rates, G);
        float chi = x[g * 3 + 2];
        float newSrc = (fission_source * chi + scatter_source) / (4.0 * M_PI);
        float oldSrc = q[g];
        group_res[g] = (newSrc - oldSrc) * (newSrc - oldSrc) / (oldSrc * oldSrc);
        q[g] = newSrc;
      }
      fine_res[j] = oracle_pairwise_sum(group_res, G);
    }
    residuals[i] = oracle_pairwise_sum(fine_res, F);
  }
  float residual = oracle_pairwise_sum(residuals, NS);    /* solver.c:1307 */
  free(group_res);
  free(fine_res);
  free(residuals);
  free(fission_rates);
  free(scatter_rates);
  return residual;
}

static float rate_sum(const oracle_problem *P, const float *fine_flux, int which)
{
  const int64_t G = P->G, F = P->F, NS = P->NS;
  float *sigma = (float *)malloc(sizeof(float) * (size_t)G);
  float *group_rates = (float *)malloc(sizeof(float) * (size_t)G);
  float *fine_rates = (float *)malloc(sizeof(float) * (size_t)F);
  float *qsr_rates = (float *)malloc(sizeof(float) * (size_t)NS);
  for (int64_t i = 0; i < NS; i++) {
    const float *x = P->xs + (int64_t)P->src_xs[i] * G * 3;
    for (int64_t g = 0; g < G; g++)
      sigma[g] = x[g * 3 + which];
    for (int64_t j = 0; j < F; j++) {
      const float *phi = fine_flux + (i * F + j) * G;
      for (int64_t g = 0; g < G; g++)
        group_rates[g] = sigma[g] * phi[g];
      fine_rates[j] = oracle_pairwise_sum(group_rates, G);
    }
    qsr_rates[i] = oracle_pairwise_sum(fine_rates, F);
  }
  float r = oracle_pairwise_sum(qsr_rates, NS);
  free(sigma);
  free(group_rates);
  free(fine_rates);
  free(qsr_rates);
  return r;
}

float oracle_compute_keff(const oracle_problem *P, const float *fine_flux,
                          float leakage)
{
  float node_abs = rate_sum(P, fine_flux, 1);             /* solver.c:1335-1356 */
  float node_fission = rate_sum(P, fine_flux, 0);         /* solver.c:1361-1382 */
  return node_fission / (node_abs + leakage);             /* solver.c:1425 */
}

/* ------------------------------------------------------------------------ */
/* FP64 yardstick                                                            */
/* ------------------------------------------------------------------------ */
static void attenuate64(const oracle_problem *P, float z, float ds_f, float mu_f,
                        double weight, const double *q, double *phi,
                        const float *sigt_row, double *psi)
{
  const int G = P->G, F = P->F;
  float dz_f = fine_dz(P);
  int idx = (int)(z / dz_f);                  /* same fine interval as FP32 */
  int fine_id = idx % F;
  double dz = dz_f, ds = ds_f, mu = mu_f;
  double zin = (double)z - dz * (idx + 0.5);
  double *flux = phi + (int64_t)fine_id * G;
  if (P->axial_exp == 0) {
    double w = weight * mu;
    const double *qf = q + (int64_t)fine_id * G;
    for (int g = 0; g < G; g++) {
      double sigT = sigt_row[g];
      double tau = sigT * ds;
      double e = -expm1(-tau);
      double delta_psi = (psi[g] - qf[g] / sigT) * e;
      psi[g] -= delta_psi;
      flux[g] += w * delta_psi;
    }
    return;
  }
  double mu2 = mu * mu;
  int r0;
  if (fine_id == 0) {
    zin -= dz;
    r0 = 0;
  } else if (fine_id == F - 1) {
    zin += dz;
    r0 = fine_id - 2;
  } else {
    r0 = fine_id - 1;
  }
  const double *row1 = q + (int64_t)r0 * G, *row2 = row1 + G, *row3 = row2 + G;
  for (int g = 0; g < G; g++) {
    double y1 = row1[g], y2 = row2[g], y3 = row3[g];
    double c1 = (y1 - y3) / (2.0 * dz);
    double c2 = (y1 - 2.0 * y2 + y3) / (2.0 * dz * dz);
    double q0 = y2 + c1 * zin + c2 * zin * zin;
    double q1 = c1 + 2.0 * c2 * zin;
    double q2 = c2;
    double sigT = sigt_row[g];
    double tau = sigT * ds;
    double sigT2 = sigT * sigT;
    double e = -expm1(-tau);
    double reuse = tau * (tau - 2.0) + 2.0 * e / (sigT * sigT2);
    double p = psi[g];
    double fi = (q0 * tau + (sigT * p - q0) * e) / sigT2 + q1 * mu * reuse
              + q2 * mu2 * (tau * (tau * (tau - 3.0) + 6.0) - 6.0 * e)
                / (3.0 * sigT2 * sigT2);
    flux[g] += weight * fi;
    psi[g] = q0 * e / sigT + q1 * mu * (tau - e) / sigT2 + q2 * mu2 * reuse
           + p * (1.0 - e);
  }
}

int64_t oracle_sweep64(const oracle_problem *P, const double *fine_source,
                       double *fine_flux, double *psi_f)
{
  const int64_t G = P->G, F = P->F, S = P->S;
  const int64_t PZ = (int64_t)P->P * P->Z;
  const int64_t N3D = P->N2D * PZ;
  float Hd = P->height / P->decomp_ax;
  for (int64_t t = 0; t < N3D; t++) {
    int64_t i = t / PZ;
    int j = (int)((t / P->Z) % P->P);
    float theta = P->polar_angles[j];
    float mu = oracle_mu(theta);
    /* the track weight is an input quantity: the reference's float product */
    double weight = (double)(P->p_weight[t] * P->az_weight[i]);
    float z = P->z0[t];
    double *psi = psi_f + t * G;
    for (int64_t n = 0; n < S; n++) {
      float ds = oracle_ds(P->seg_len[i * S + n], theta);
      int64_t s = P->seg_src[t * S + n];
      attenuate64(P, z, ds, mu, weight, fine_source + s * F * G,
                  fine_flux + s * F * G, P->sigt + (int64_t)P->src_sigt[s] * G, psi);
      z = oracle_advance_z(z, ds, mu, Hd);
    }
  }
  return N3D * S;
}

void oracle_renormalize64(const oracle_problem *P, double *fine_flux,
                          double *psi_f, double *psi_b)
{
  const int64_t G = P->G, F = P->F, NS = P->NS;
  double *rates = (double *)malloc(sizeof(double) * (size_t)NS);
  for (int64_t i = 0; i < NS; i++) {
    const float *x = P->xs + (int64_t)P->src_xs[i] * G * 3;
    double r = 0;
    for (int64_t k = 0; k < F * G; k++)
      r += fine_flux[i * F * G + k] * (double)P->vol[i] * x[(k % G) * 3 + 0];
    rates[i] = r;
  }
  double norm = 1.0 / pairwise64(rates, NS);
  for (int64_t i = 0; i < NS; i++) {
    double adjust = norm * 4.0 * M_PI * F / P->vol[i];
    for (int64_t k = 0; k < F * G; k++)
      fine_flux[i * F * G + k] *= adjust;
  }
  const int64_t n = P->N2D * P->P * P->Z * G;
  for (int64_t k = 0; k < n; k++) {
    psi_f[k] *= norm;
    psi_b[k] *= norm;
  }
  free(rates);
}

double oracle_update_sources64(const oracle_problem *P, const double *fine_flux,
                               double *fine_source, double keff)
{
  const int64_t G = P->G, F = P->F, NS = P->NS;
  double residual = 0;
  for (int64_t i = 0; i < NS; i++) {
    const float *x = P->xs + (int64_t)P->src_xs[i] * G * 3;
    const float *S = P->scatter + (int64_t)P->src_xs[i] * G * G;
    for (int64_t j = 0; j < F; j++) {
      const double *phi = fine_flux + (i * F + j) * G;
      double *q = fine_source + (i * F + j) * G;
      double fission = 0;
      for (int64_t g = 0; g < G; g++)
        fission += phi[g] * x[g * 3 + 0];
      fission /= keff;
      for (int64_t g = 0; g < G; g++) {
        double sc = 0;
        for (int64_t g2 = 0; g2 < G; g2++)
          sc += (double)S[g * G + g2] * phi[g2];
        double nw = (fission * x[g * 3 + 2] + sc) / (4.0 * M_PI);
        double old = q[g];
        residual += (nw - old) * (nw - old) / (old * old);
        q[g] = nw;
      }
    }
  }
  return residual;
}

double oracle_compute_keff64(const oracle_problem *P, const double *fine_flux,
                             double leakage)
{
  const int64_t G = P->G, F = P->F, NS = P->NS;
  double ab = 0, fi = 0;
  for (int64_t i = 0; i < NS; i++) {
    const float *x = P->xs + (int64_t)P->src_xs[i] * G * 3;
    for (int64_t k = 0; k < F * G; k++) {
      double phi = fine_flux[i * F * G + k];
      ab += x[(k % G) * 3 + 1] * phi;
      fi += x[(k % G) * 3 + 0] * phi;
    }
  }
  return fi / (ab + leakage);
}

/* ------------------------------------------------------------------------ */
/* FP64 adjoint: reverse mode of attenuate64 over every track                */
/* ------------------------------------------------------------------------ */
typedef struct seg64 {
  int64_t qrow, frow;   /* first fitted row and tally row (row index, not x G) */
  int64_t srow;         /* sigma_t row */
  double zin, ds;
} seg64;

static seg64 geometry64(const oracle_problem *P, float z, float ds_f, int64_t s)
{
  seg64 g;
  const int F = P->F;
  float dz_f = fine_dz(P);
  int idx = (int)(z / dz_f);
  int fine_id = idx % F;
  double dz = dz_f;
  g.zin = (double)z - dz * (idx + 0.5);
  int r0 = fine_id;
  if (P->axial_exp == 2) {
    if (fine_id == 0) { g.zin -= dz; r0 = 0; }
    else if (fine_id == F - 1) { g.zin += dz; r0 = fine_id - 2; }
    else r0 = fine_id - 1;
  }
  g.qrow = s * F + r0;
  g.frow = s * F + fine_id;
  g.srow = P->src_sigt[s];
  g.ds = ds_f;
  return g;
}

void oracle_adjoint64(const oracle_problem *P, const double *fine_source,
                      const double *psi_in, const double *dphi, double *dq,
                      double *dsigt, double *dpsi_in)
{
  const int64_t G = P->G, S = P->S;
  const int64_t PZ = (int64_t)P->P * P->Z;
  const int64_t N3D = P->N2D * PZ;
  const int64_t NR = P->NS * P->F;
  const double dz = fine_dz(P);
  const double rd1 = 1.0 / (2.0 * dz), rd2 = 1.0 / (2.0 * dz * dz);
  float Hd = P->height / P->decomp_ax;
  memset(dq, 0, sizeof(double) * (size_t)(NR * G));
  double *hist = (double *)malloc(sizeof(double) * (size_t)((S + 1) * G));
  seg64 *segs = (seg64 *)malloc(sizeof(seg64) * (size_t)S);
  for (int64_t t = 0; t < N3D; t++) {
    int64_t i = t / PZ;
    int j = (int)((t / P->Z) % P->P);
    float theta = P->polar_angles[j];
    float mu_f = oracle_mu(theta);
    const double mu = mu_f, mu2 = mu * mu;
    const double w = (double)(P->p_weight[t] * P->az_weight[i]);
    float z = P->z0[t];
    for (int64_t g = 0; g < G; g++)
      hist[g] = psi_in ? psi_in[t * G + g] : 0.0;
    /* forward: psi entering every segment */
    for (int64_t n = 0; n < S; n++) {
      float ds = oracle_ds(P->seg_len[i * S + n], theta);
      segs[n] = geometry64(P, z, ds, P->seg_src[t * S + n]);
      const seg64 *sg = &segs[n];
      for (int64_t g = 0; g < G; g++) {
        const double sig = P->sigt[sg->srow * G + g], tau = sig * sg->ds;
        const double e = -expm1(-tau), p = hist[n * G + g];
        double pn;
        if (P->axial_exp == 2) {
          const double *qr = fine_source + sg->qrow * G;
          const double y1 = qr[g], y2 = qr[G + g], y3 = qr[2 * G + g];
          const double c1 = (y1 - y3) * rd1, c2 = (y1 - 2.0 * y2 + y3) * rd2;
          const double q0 = y2 + c1 * sg->zin + c2 * sg->zin * sg->zin;
          const double q1 = c1 + 2.0 * c2 * sg->zin, sig2 = sig * sig;
          const double reuse = tau * (tau - 2.0) + 2.0 * e / (sig * sig2);
          pn = q0 * e / sig + q1 * mu * (tau - e) / sig2 + c2 * mu2 * reuse + p * (1.0 - e);
        } else {
          pn = p - (p - fine_source[sg->qrow * G + g] / sig) * e;
        }
        hist[(n + 1) * G + g] = pn;
      }
      z = oracle_advance_z(z, ds, mu_f, Hd);
    }
    /* reverse */
    for (int64_t g = 0; g < G; g++) {
      double pbar = 0.0;
      for (int64_t n = S - 1; n >= 0; n--) {
        const seg64 *sg = &segs[n];
        const double sig = P->sigt[sg->srow * G + g], ds = sg->ds, tau = sig * ds;
        const double e = -expm1(-tau), eps = 1.0 - e, psi = hist[n * G + g];
        const double r1 = 1.0 / sig, r2 = r1 * r1, r3 = r2 * r1;
        const double lam = dphi[sg->frow * G + g];
        if (P->axial_exp == 2) {
          const double abar = lam * w;
          const double r4 = r2 * r2 / 3.0;
          const double *qr = fine_source + sg->qrow * G;
          const double y1 = qr[g], y2 = qr[G + g], y3 = qr[2 * G + g];
          const double zin = sg->zin;
          const double c1 = (y1 - y3) * rd1, c2 = (y1 - 2.0 * y2 + y3) * rd2;
          const double q0 = y2 + c1 * zin + c2 * zin * zin, q1 = c1 + 2.0 * c2 * zin, q2 = c2;
          const double R = tau * (tau - 2.0) + 2.0 * e * r3;
          const double Cc = tau * (tau * (tau - 3.0) + 6.0) - 6.0 * e;
          const double tme = tau - e;
          const double q0b = abar * tme * r2 + pbar * e * r1;
          const double q1b = mu * (abar * R + pbar * tme * r2);
          const double q2b = mu2 * (abar * Cc * r4 + pbar * R);
          const double c1b = q0b * zin + q1b;
          const double c2b = q0b * zin * zin + 2.0 * q1b * zin + q2b;
          dq[sg->qrow * G + g] += c1b * rd1 + c2b * rd2;
          dq[(sg->qrow + 1) * G + g] += q0b - 2.0 * c2b * rd2;
          dq[(sg->qrow + 2) * G + g] += c2b * rd2 - c1b * rd1;
          const double A = (q0 * tau + (sig * psi - q0) * e) * r2;
          const double dA = (q0 * ds + psi * e + (sig * psi - q0) * eps * ds) * r2 - 2.0 * A * r1;
          const double dR = (2.0 * tau - 2.0) * ds + 2.0 * eps * ds * r3 - 6.0 * e * r3 * r1;
          const double dC = ((3.0 * tau - 6.0) * tau + 6.0) * ds - 6.0 * eps * ds;
          const double dfi = dA + q1 * mu * dR + q2 * mu2 * (dC * r4 - 4.0 * Cc * r4 * r1);
          const double dpn = q0 * (eps * ds * r1 - e * r2) + q1 * mu * (e * ds * r2 - 2.0 * tme * r3)
                           + q2 * mu2 * dR - psi * eps * ds;
          dsigt[sg->srow * G + g] += abar * dfi + pbar * dpn;
          pbar = pbar * eps + abar * e * r1;
        } else {
          const double abar = lam * w * mu;
          const double y = fine_source[sg->qrow * G + g];
          const double dbar = abar - pbar;
          dq[sg->qrow * G + g] += -dbar * e * r1;
          dsigt[sg->srow * G + g] += dbar * (y * r2 * e + (psi - y * r1) * eps * ds);
          pbar = pbar + dbar * e;
        }
      }
      if (dpsi_in)
        dpsi_in[t * G + g] = pbar;
    }
  }
  free(hist);
  free(segs);
}
