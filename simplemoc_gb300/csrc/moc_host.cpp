// moc_host.cpp -- host-side pieces of the library: the exponential table
// (src/utils.c:48-78), the seeded synthetic problem generator (the random
// construction of src/tracks.c and src/source.c made reproducible), and the
// derived per-segment / per-material arrays that the kernels read.
//
// Compiled with -ffp-contract=off so that every float expression here rounds
// exactly as the reference's does.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "moc_host.h"
#include "simplemoc_gb300.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

extern "C" int32_t moc_exp_table_size(float precision, float maxval) {
  if (!(precision > 0.0f) || !(maxval > 0.0f)) return 0;
  return (int32_t)(maxval * sqrt(1.0 / (8.0 * precision * 0.01)));   // src/utils.c:54
}

extern "C" int moc_build_exp_table(float precision, float maxval, float *values, int32_t n,
                                   float *dx_out, float *maxval_out) {
  int32_t N = moc_exp_table_size(precision, maxval);
  if (N < 1 || n != N || !values || !dx_out || !maxval_out) return MOC_ERR_ARG;
  float dx = maxval / (float)N;                                        // src/utils.c:57
  for (int32_t k = 0; k < N; k++) {                                    // src/utils.c:63-69
    float e = (float)exp((double)(-k * dx));              // C promotes to double
    values[2 * k] = -e;
    values[2 * k + 1] = 1 + (k * dx - 1) * e;
  }
  *dx_out = dx;
  *maxval_out = maxval - dx;                                           // src/utils.c:74
  return MOC_OK;
}

// ---------------------------------------------------------------------------
// Counter-based generator: every value is a pure function of
// (seed, array stream, element index), so any thread count gives the same
// problem.  mix64 is the SplitMix64 output function (Steele, Lea, Flood,
// OOPSLA 2014); the i-th draw of a stream is mix64(key + i * golden gamma).
// ---------------------------------------------------------------------------
namespace {

inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
constexpr uint64_t GAMMA = 0x9E3779B97F4A7C15ull;

struct Stream {
  uint64_t key;
  Stream(uint64_t seed, uint64_t id) : key(mix64(seed * GAMMA + id * 0xD1B54A32D192ED03ull)) {}
  inline uint64_t bits(uint64_t i) const { return mix64(key + (i + 1) * GAMMA); }
  // uniform in [0, 1) with 24 random bits
  inline float u(uint64_t i) const { return (float)(bits(i) >> 40) * (1.0f / 16777216.0f); }
  // uniform integer in [0, n)
  inline int32_t below(uint64_t i, uint32_t n) const {
    return (int32_t)(((bits(i) >> 32) * (uint64_t)n) >> 32);
  }
};

enum : uint64_t {
  ST_SEG_LEN = 1, ST_SEG_SRC, ST_AZ_W, ST_P_W, ST_SRC_MAT, ST_VOL, ST_SIGT, ST_SCAT, ST_NUSF,
  ST_CHI, ST_QINIT
};

}  // namespace

extern "C" int moc_generate(const moc_dims *d, const moc_gen_params *gp, float *seg_len,
                            int32_t *seg_src, float *az_weight, float *p_weight, float *z0,
                            float *polar_angles, int32_t *src_sigt, int32_t *src_xs, float *vol,
                            float *sigt, float *xs, float *scatter, float *fine_source) {
  if (!d || !gp) return MOC_ERR_ARG;
  const int64_t G = d->n_groups, F = d->fai, NS = d->n_sources, N2D = d->n_tracks_2d;
  const int64_t P = d->n_polar, Z = d->z_stacked, S = d->n_seg;
  const int64_t NM = gp->n_materials;
  if (G < 1 || F < 1 || NS < 1 || N2D < 1 || P < 1 || Z < 1 || S < 1 || NM < 1) return MOC_ERR_ARG;
  if (d->n_sigt != NM || d->n_xs != NM) return MOC_ERR_ARG;
  if (NS > INT32_MAX) return MOC_ERR_ARG;
  const int64_t N3D = N2D * P * Z;
  const uint64_t seed = gp->seed;

  if (seg_len) {
    Stream st(seed, ST_SEG_LEN);
    const float lo = gp->len_lo, span = gp->len_hi - gp->len_lo;
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < N2D * S; k++) seg_len[k] = lo + span * st.u((uint64_t)k);
  }
  if (seg_src) {
    Stream st(seed, ST_SEG_SRC);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < N3D * S; k++) seg_src[k] = st.below((uint64_t)k, (uint32_t)NS);
  }
  if (az_weight) {
    Stream st(seed, ST_AZ_W);                     // src/tracks.c:12
    for (int64_t i = 0; i < N2D; i++) az_weight[i] = st.u((uint64_t)i);
  }
  if (p_weight) {
    Stream st(seed, ST_P_W);                      // src/tracks.c:132
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < N3D; t++) p_weight[t] = st.u((uint64_t)t);
  }
  if (polar_angles) {
    for (int64_t j = 0; j < P; j++)               // src/tracks.c:165
      polar_angles[j] = (float)(M_PI * (j + 0.5) / P);
  }
  if (z0) {
    // src/tracks.c:126-129: upward tracks start at sep*k, downward at sep*(k+1)
    const float sep = gp->axial_z_sep > 0.0f ? gp->axial_z_sep : d->height / (float)Z;
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < N3D; t++) {
      const int64_t k = t % Z;
      const int64_t j = (t / Z) % P;
      z0[t] = (j < P / 2) ? sep * (int)k : sep * (int)(k + 1);
    }
  }
  if (src_sigt || src_xs) {
    Stream st(seed, ST_SRC_MAT);
    for (int64_t s = 0; s < NS; s++) {
      int32_t m = st.below((uint64_t)s, (uint32_t)NM);
      if (src_sigt) src_sigt[s] = m;
      if (src_xs) src_xs[s] = m;
    }
  }
  if (vol) {
    Stream st(seed, ST_VOL);
    const float lo = gp->vol_lo, span = gp->vol_hi - gp->vol_lo;
    for (int64_t s = 0; s < NS; s++) vol[s] = lo + span * st.u((uint64_t)s);
  }
  std::vector<float> sig_tmp;
  if (sigt || xs) {
    Stream st(seed, ST_SIGT);
    const float lo = gp->sigt_lo, span = gp->sigt_hi - gp->sigt_lo;
    sig_tmp.resize((size_t)(NM * G));
    for (int64_t k = 0; k < NM * G; k++) sig_tmp[k] = lo + span * st.u((uint64_t)k);
    if (sigt) memcpy(sigt, sig_tmp.data(), sizeof(float) * (size_t)(NM * G));
  }
  if (scatter) {
    Stream st(seed, ST_SCAT);
    for (int64_t r = 0; r < NM * G; r++) {        // row r = (material, destination group)
      double sum = 0.0;
      for (int64_t g2 = 0; g2 < G; g2++) {
        float v = st.u((uint64_t)(r * G + g2));
        scatter[r * G + g2] = v;
        sum += v;
      }
      const float scale = (float)(gp->scatter_ratio / (sum > 0.0 ? sum : 1.0));
      for (int64_t g2 = 0; g2 < G; g2++) scatter[r * G + g2] *= scale;
    }
  }
  if (xs) {
    Stream sn(seed, ST_NUSF), sc(seed, ST_CHI);
    for (int64_t m = 0; m < NM; m++) {
      double csum = 0.0;
      std::vector<float> chi((size_t)G);
      for (int64_t g = 0; g < G; g++) {
        chi[g] = sc.u((uint64_t)(m * G + g));
        csum += chi[g];
      }
      for (int64_t g = 0; g < G; g++) {
        float *x = xs + (m * G + g) * 3;
        x[0] = (m < gp->n_fuel) ? gp->nusf_hi * sn.u((uint64_t)(m * G + g)) : 0.0f;
        x[1] = gp->siga_ratio * sig_tmp[m * G + g];
        x[2] = (float)(chi[g] / (csum > 0.0 ? csum : 1.0));
      }
    }
  }
  if (fine_source) {
    Stream st(seed, ST_QINIT);                    // src/source.c:157-160
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < NS * F * G; k++) fine_source[k] = st.u((uint64_t)k);
  }
  return MOC_OK;
}

// ---------------------------------------------------------------------------
// Derived arrays
// ---------------------------------------------------------------------------
int moc_host_derive(const moc_dims *d, const moc_host *h, int32_t ldg, float *seg_ds, float *mu,
                    float *weight, float *coef, float *scatter_t, float *max_abs_dz) {
  const int64_t G = d->n_groups, P = d->n_polar, Z = d->z_stacked, S = d->n_seg;
  const int64_t N2D = d->n_tracks_2d;
  float worst = 0.0f;
  int nonfinite = 0;
  for (int64_t j = 0; j < P; j++) mu[j] = (float)cos((double)h->polar_angles[j]);   // src/solver.c:373
#pragma omp parallel for schedule(static) reduction(max : worst) reduction(| : nonfinite)
  for (int64_t i = 0; i < N2D; i++) {
    for (int64_t j = 0; j < P; j++) {
      const float a = h->polar_angles[j];
      const float muj = (float)cos((double)a);
      const double sin_a = sin((double)a);
      for (int64_t n = 0; n < S; n++) {
        const float ds = (float)(h->seg_len[i * S + n] / sin_a);           // src/solver.c:382
        seg_ds[(i * P + j) * S + n] = ds;
        const float step = fabsf(ds * muj);
        nonfinite |= !isfinite(step);
        worst = step > worst ? step : worst;
      }
    }
  }
  *max_abs_dz = nonfinite ? INFINITY : worst;
  const int64_t PZ = P * Z;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < N2D; i++) {
    const float az = h->az_weight[i];
    for (int64_t t = i * PZ; t < (i + 1) * PZ; t++)
      weight[t] = h->p_weight[t] * az;                                     // src/solver.c:49
  }
  moc_host_coef(d, h->sigt, ldg, coef);
  for (int64_t m = 0; m < d->n_xs; m++)
    for (int64_t g = 0; g < G; g++)
      for (int64_t g2 = 0; g2 < G; g2++)
        scatter_t[(m * G + g2) * G + g] = h->scatter[(m * G + g) * G + g2];
  return MOC_OK;
}

void moc_host_coef(const moc_dims *d, const float *sigt, int32_t ldg, float *coef) {
  const int64_t G = d->n_groups;
  for (int64_t m = 0; m < d->n_sigt; m++) {
    float *row = coef + m * MOC_COEF_PLANES * (int64_t)ldg;
    for (int64_t g = 0; g < ldg; g++) {
      const float sig = g < G ? sigt[m * G + g] : 1.0f;
      const float sig2 = sig * sig;                                        // src/solver.c:153
      const float sig3 = sig * sig2;                                       // src/solver.c:176
      const float sig4 = 3.f * sig2 * sig2;                                // src/solver.c:198
      float *c = row + (g / 4) * 4 * MOC_COEF_PLANES + g % 4;
      c[0] = sig;
      c[4] = 1.0f / sig;
      c[8] = 1.0f / sig2;
      c[12] = 1.0f / sig3;
      c[16] = 1.0f / sig4;
      c[20] = 2.0f * (1.0f / sig3);
    }
  }
}

int moc_host_validate_ids(const moc_dims *d, const int32_t *seg_src, int64_t first, int64_t end) {
  const int64_t NS = d->n_sources;
  const uint32_t *ids = reinterpret_cast<const uint32_t *>(seg_src);
  uint32_t mx = 0;                       // a negative id is a huge unsigned one
  // One contiguous block per thread, eight independent maxima per step (two
  // 4-lane vector maxima): the scan runs at memory speed rather than at the
  // latency of one dependent max per id.
  constexpr int W = 8;
  const int64_t n = end > first ? end - first : 0;
#pragma omp parallel reduction(max : mx)
  {
    int nt = 1, t = 0;
#ifdef _OPENMP
    nt = omp_get_num_threads();
    t = omp_get_thread_num();
#endif
    const int64_t a = first + n * t / nt, b = first + n * (t + 1) / nt;
    uint32_t m[W] = {0};
    int64_t k = a;
    for (; k + W <= b; k += W)
      for (int j = 0; j < W; ++j) m[j] = ids[k + j] > m[j] ? ids[k + j] : m[j];
    for (; k < b; ++k) m[0] = ids[k] > m[0] ? ids[k] : m[0];
    for (int j = 0; j < W; ++j) mx = m[j] > mx ? m[j] : mx;
  }
  return n > 0 && (int64_t)mx >= NS ? MOC_ERR_ARG : MOC_OK;
}

int moc_host_validate(const moc_dims *d, const moc_host *h) {
  int rc = moc_host_validate_except_ids(d, h);
  if (rc != MOC_OK) return rc;
  return moc_host_validate_ids(d, h->seg_src, 0,
                               d->n_tracks_2d * d->n_polar * d->z_stacked * (int64_t)d->n_seg);
}

int moc_host_validate_except_ids(const moc_dims *d, const moc_host *h) {
  const int64_t G = d->n_groups, NS = d->n_sources;
  const int64_t S = d->n_seg;
  if (G < 1 || d->fai < 1 || d->cai < 1 || d->decomp_ax < 1 || NS < 1 || d->n_sigt < 1 ||
      d->n_xs < 1 || d->n_tracks_2d < 1 || d->n_polar < 1 || d->n_polar > 64 ||
      d->z_stacked < 1 || S < 1)
    return MOC_ERR_ARG;
  // Every array size must fit in 64-bit element and byte counts: products
  // beyond 2^50 elements are rejected before any of them is formed in integers.
  {
    const double lim = 1125899906842624.0;   // 2^50
    const double n2d = (double)d->n_tracks_2d, n3d = n2d * d->n_polar * d->z_stacked;
    const double ldg = (double)G + 3.0;
    if (n2d * d->n_polar * S > lim || n3d * S > lim || n3d * ldg > lim ||
        (double)NS * d->fai * ldg > lim || (double)d->n_xs * G * G > lim ||
        (double)d->n_sigt * ldg * 8 > lim || (double)d->table_n * 2 > lim)
      return MOC_ERR_ARG;
  }
  const int64_t N3D = d->n_tracks_2d * d->n_polar * d->z_stacked;
  if (!(d->height > 0.0f) || NS > INT32_MAX) return MOC_ERR_ARG;
  if (d->axial_exp != 0 && d->axial_exp != 2) return MOC_ERR_ARG;   // src/solver.c:506-511
  if (d->axial_exp == 2 && d->fai < 3) return MOC_ERR_ARG;          // three rows are fitted
  if (d->table_n < 1 || !(d->table_dx > 0.0f)) return MOC_ERR_ARG;
  if (!h->seg_len || !h->seg_src || !h->az_weight || !h->p_weight || !h->z0 ||
      !h->polar_angles || !h->src_sigt || !h->src_xs || !h->vol || !h->sigt || !h->xs ||
      !h->scatter || !h->fine_source || !h->table)
    return MOC_ERR_ARG;
  for (int64_t j = 0; j < d->n_polar; j++) {
    const float a = h->polar_angles[j];
    if (!(a > 0.0f && a < 3.14159265f)) return MOC_ERR_ARG;
  }
  for (int64_t s = 0; s < NS; s++) {
    if (h->src_sigt[s] < 0 || h->src_sigt[s] >= d->n_sigt) return MOC_ERR_ARG;
    if (h->src_xs[s] < 0 || h->src_xs[s] >= d->n_xs) return MOC_ERR_ARG;
    if (!(h->vol[s] > 0.0f)) return MOC_ERR_ARG;
  }
  for (int64_t k = 0; k < (int64_t)d->n_sigt * G; k++)
    if (!(h->sigt[k] > 0.0f) || isinf(h->sigt[k])) return MOC_ERR_ARG;
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int64_t k = 0; k < d->n_tracks_2d * S; k++)
    bad |= !(h->seg_len[k] >= 0.0f) || isinf(h->seg_len[k]);
  if (bad) return MOC_ERR_ARG;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int64_t t = 0; t < N3D; t++) bad |= !(h->z0[t] >= 0.0f) || isinf(h->z0[t]);
  if (bad) return MOC_ERR_ARG;
  return MOC_OK;
}
