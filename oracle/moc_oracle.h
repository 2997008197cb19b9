/*
 * moc_oracle.h -- CPU oracle for the SimpleMOC transport-sweep path.
 *
 * TEST INFRASTRUCTURE ONLY.  The GPU library's results are compared against
 * it; nothing in the product links, loads or calls it.  Only
 * tests/, __graft_entry__.smoke() and the CPU-baseline legs of bench.py use it.
 *
 * It restates, in plain C99, the arithmetic of the reference solver
 * (src/solver.c, src/utils.c) over the flat storage described in
 * include/simplemoc_gb300.h.  Each function cites the reference lines it
 * follows.  Compiled with -O2 -ffp-contract=off and no fast-math so that every
 * float operation rounds exactly as the reference's serial build does.
 * The restatement is pinned against the reference's own compiled objects by
 * oracle/ref_harness.c and the fixtures in tests/golden/.
 */
#ifndef MOC_ORACLE_H
#define MOC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_problem {
  int32_t G, F, cai, decomp_ax;
  float   height;
  int32_t axial_exp;
  int64_t NS;
  int64_t N2D;
  int32_t P, Z, S;
  const float   *seg_len;      /* [N2D*S]  */
  const int32_t *seg_src;      /* [N3D*S]  */
  const float   *az_weight;    /* [N2D]    */
  const float   *p_weight;     /* [N3D]    */
  const float   *z0;           /* [N3D]    */
  const float   *polar_angles; /* [P]      */
  const int32_t *src_sigt;     /* [NS]     */
  const int32_t *src_xs;       /* [NS]     */
  const float   *vol;          /* [NS]     */
  const float   *sigt;         /* [n_sigt*G] */
  const float   *xs;           /* [n_xs*G*3] */
  const float   *scatter;      /* [n_xs*G*G] */
  const float   *table;        /* [2*table_n] */
  int32_t table_n;
  float   table_dx;
  float   table_maxval;
} oracle_problem;

/* src/utils.c:48-78 */
int32_t oracle_exp_table_size(float precision, float maxval);
void    oracle_build_exp_table(float precision, float maxval, float *values,
                               float *dx, float *maxval_out, int32_t *n);
/* src/solver.c:1441-1464 */
float   oracle_interpolate(const float *values, float dx, float maxval, float x);
/* src/utils.c:29-45 */
float   oracle_pairwise_sum(const float *v, int64_t n);

/* Per 3D track quantities of the explicit-track traversal. */
float   oracle_mu(float polar_angle);                /* solver.c:373 */
float   oracle_ds(float len, float polar_angle);     /* solver.c:382 */
float   oracle_advance_z(float z, float ds, float mu, float domain_height);

/* One segment of attenuate_fluxes (solver.c:14-280, axial_exp 2) or
 * attenuate_FSR_fluxes (solver.c:1040-1138, axial_exp 0).  `q` and `phi` are
 * the F*G rows of the segment's source region; psi is updated in place. */
void oracle_attenuate(const oracle_problem *P, float z, float ds, float mu,
                      float weight, const float *q, float *phi,
                      const float *sigt_row, float *psi);

/* Serial sweep over all 3D tracks in index order (solver.c:283-552 restated
 * over explicit segment streams).  Returns segments processed. */
int64_t oracle_sweep(const oracle_problem *P, const float *fine_source,
                     float *fine_flux, float *psi_f);
/* The same arithmetic for a list of tracks only; psi rows of those tracks are
 * read from psi_in and written to psi_out[n*G]; tallies go to fine_flux
 * (may be NULL to drop them). */
void oracle_sweep_tracks(const oracle_problem *P, const float *fine_source,
                         const int64_t *tracks, int64_t n, const float *psi_in,
                         float *psi_out, float *fine_flux);
/* OpenMP sweep with one lock per fine source region, as the reference's
 * OpenMP build (solver.c:212-228, init.c:229-240).  Used for CPU timing. */
int64_t oracle_sweep_omp(const oracle_problem *P, const float *fine_source,
                         float *fine_flux, float *psi_f, int nthreads);
/* Threads OpenMP will use (0 when built without OpenMP). */
int     oracle_omp_max_threads(void);

/* The reference's own traversal (src/solver.c:347-523, serial build): 2D
 * tracks with their own segment counts, the z-stacked rays of each polar
 * angle, axial splitting at fine-interval boundaries, the begin/end retirement
 * of stacked rays at the domain bounds, and the stacked-ray height state kept
 * between sweeps.  The source region of each 3D sub-segment is ids[seq] for the
 * seq-th sub-segment in traversal order, or rand() % NS (libc, exactly as the
 * serial reference) when ids is NULL. */
typedef struct oracle_refgeo {
  int64_t N2D;
  const int64_t *seg_off;      /* [N2D+1] first segment of each 2D track */
  const float *seg_len;        /* [seg_off[N2D]] 2D segment lengths */
  const float *az_weight;      /* [N2D] */
  const float *p_weight;       /* [N3D] */
  float axial_z_sep;           /* Input.axial_z_sep */
} oracle_refgeo;

int64_t oracle_ref_sweep(const oracle_problem *P, const oracle_refgeo *R,
                         const float *fine_source, float *fine_flux, float *psi_f,
                         float *z_height, const int32_t *ids);

/* src/solver.c:1143-1230, serial build semantics. */
void  oracle_renormalize(const oracle_problem *P, float *fine_flux,
                         float *psi_f, float *psi_b);
/* src/solver.c:1235-1320 */
float oracle_update_sources(const oracle_problem *P, const float *fine_flux,
                            float *fine_source, float keff);
/* src/solver.c:1324-1437 (serial: keff = fission / (abs + leakage)). */
float oracle_compute_keff(const oracle_problem *P, const float *fine_flux,
                          float leakage);

/* FP64 yardstick: the same formulas in double with exact 1-exp(-tau),
 * applied to the FP32 geometry (heights, lengths, cosines, fine interval of
 * each segment).  State arrays are double. */
int64_t oracle_sweep64(const oracle_problem *P, const double *fine_source,
                       double *fine_flux, double *psi_f);
void   oracle_renormalize64(const oracle_problem *P, double *fine_flux,
                            double *psi_f, double *psi_b);
double oracle_update_sources64(const oracle_problem *P, const double *fine_flux,
                               double *fine_source, double keff);
double oracle_compute_keff64(const oracle_problem *P, const double *fine_flux,
                             double leakage);

/* FP64 adjoint of one sweep (oracle_sweep64's arithmetic): given dL/dphi,
 * writes dL/dq [NS*F*G], adds dL/dsigma_t into dsigt [n_sigt*G], and writes
 * dL/dpsi entering each track [N3D*G] (may be NULL).  psi_in is the angular
 * flux entering the tracks (NULL = zero). */
void oracle_adjoint64(const oracle_problem *P, const double *fine_source,
                      const double *psi_in, const double *dphi, double *dq,
                      double *dsigt, double *dpsi_in);

#ifdef __cplusplus
}
#endif
#endif
