/*
 * simplemoc_refabi.h -- the reference's own solver entry points, served by
 * libsimplemoc_gb300.so on the GPU.
 *
 * SimpleMOC's driver (src/main.c:61,75,81,87) calls four functions declared in
 * src/SimpleMOC_header.h:225,235-237.  The library exports the same four
 * symbols with the same C signatures, so main.c, io.c, init.c, tracks.c,
 * source.c and utils.c of the reference link against the library in place of
 * solver.o, unchanged:
 *
 *     gcc main.c io.c init.c tracks.c source.c utils.c \
 *         -L<dir> -lsimplemoc_gb300 -lm -o SimpleMOC_gpu
 *
 * The structs below are declared only so that this library can read the
 * reference's objects: they repeat the field order and types of
 * src/SimpleMOC_header.h:28-158 for the reference's serial build (no MPI, no
 * PAPI; define SIMPLEMOC_REF_OPENMP for the OpenMP build's Source, which has
 * one more pointer).  Callers keep using the reference's own header.
 *
 * Semantics:
 *  * transport_sweep (src/solver.c:283-552) runs the reference's traversal on
 *    the device: 2D tracks with their own segment counts, z-stacked rays,
 *    axial splitting at fine-interval boundaries, the begin/end retirement of
 *    stacked rays, and the stacked-ray heights kept between sweeps.  Each 3D
 *    sub-segment's source region is rand() % n_source_regions_per_node drawn
 *    in the reference's traversal order (the serial build's sequence for the
 *    caller's srand seed), or a counter hash (moc_ref_set_rng).
 *    attenuate_fluxes / attenuate_FSR_fluxes are the PLAIN arithmetic.
 *  * The first call uploads the problem; from then on the device copy of the
 *    fluxes, sources, angular fluxes and stacked-ray heights is the live state.
 *    moc_ref_sync_to_host copies it back into the reference's arrays.
 *  * renormalize_flux / update_sources / compute_keff (src/solver.c:1143-1437)
 *    act on the device state; sums are FP64.
 *  * Errors never exit: the functions leave their outputs untouched (keff and
 *    the residual become NaN), and moc_ref_status() returns the status.
 */
#ifndef SIMPLEMOC_REFABI_H
#define SIMPLEMOC_REFABI_H

#include <stdbool.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* src/SimpleMOC_header.h:28-76 (serial build: no PAPI fields) */
typedef struct moc_ref_input {
  int x_assemblies;
  int y_assemblies;
  int cai;
  int fai;
  int axial_exp;
  float radial_ray_sep;
  float axial_z_sep;
  int n_azimuthal;
  int n_polar_angles;
  int n_egroups;
  bool decompose;
  int decomp_assemblies_ax;
  long segments_per_track;
  float assembly_width;
  float height;
  float domain_height;
  float precision;
  long mype;
  long ntracks_2D;
  int z_stacked;
  long ntracks;
  int nthreads;
  int papi_event_set;
  long n_2D_source_regions_per_assembly;
  long n_source_regions_per_node;
  bool load_tracks;
  char *track_file;
  long segments_processed;
} moc_ref_input;

/* src/SimpleMOC_header.h:86-89 */
typedef struct moc_ref_segment {
  float length;
  long source_id;
} moc_ref_segment;

/* src/SimpleMOC_header.h:92-97 */
typedef struct moc_ref_track2d {
  float az_weight;
  long n_segments;
  moc_ref_segment *segments;
  int n_3D_segments;
} moc_ref_track2d;

/* src/SimpleMOC_header.h:100-107 */
typedef struct moc_ref_track {
  float p_weight;
  float z_height;
  long rank_in;
  long rank_out;
  float *f_psi;
  float *b_psi;
} moc_ref_track;

/* src/SimpleMOC_header.h:110-120 */
typedef struct moc_ref_source {
  float **fine_flux;
  float **fine_source;
  float vol;
  float *sigT;
  float **XS;
  float **scattering_matrix;
#ifdef SIMPLEMOC_REF_OPENMP
  void *locks;
#endif
} moc_ref_source;

/* src/SimpleMOC_header.h:123-128 */
typedef struct moc_ref_table {
  float *values;
  float dx;
  float maxVal;
  int N;
} moc_ref_table;

/* src/SimpleMOC_header.h:131-138 */
typedef struct moc_ref_params {
  moc_ref_track2d *tracks_2D;
  moc_ref_track ***tracks;
  moc_ref_source *sources;
  float *polar_angles;
  float *leakage;
  moc_ref_table expTable;
} moc_ref_params;

/* src/SimpleMOC_header.h:141-158 (serial build: no MPI communicator) */
typedef struct moc_ref_commgrid {
  int x_pos_src, x_pos_dest, x_neg_src, x_neg_dest;
  int y_pos_src, y_pos_dest, y_neg_src, y_neg_dest;
  int z_pos_src, z_pos_dest, z_neg_src, z_neg_dest;
} moc_ref_commgrid;

/* ---- the reference entry points (src/SimpleMOC_header.h:225,235-237) ---- */
void transport_sweep(moc_ref_params *params, moc_ref_input *I);
void renormalize_flux(moc_ref_params params, moc_ref_input I, moc_ref_commgrid grid);
float update_sources(moc_ref_params params, moc_ref_input I, float keff);
float compute_keff(moc_ref_params params, moc_ref_input I, moc_ref_commgrid grid);

/* ---- additions for the device-resident state --------------------------- */
#define MOC_REF_RNG_LIBC 0   /* rand() in traversal order (default) */
#define MOC_REF_RNG_HASH 1   /* counter hash of (seed, sweep, sub-segment) */
int moc_ref_set_rng(int mode, uint64_t seed);
/* Copies fine_flux, fine_source, f_psi, b_psi and the stacked-ray heights back
 * into the reference's arrays. */
int moc_ref_sync_to_host(moc_ref_params *params, const moc_ref_input *I);
/* Drops the device state; the next call uploads the problem again. */
void moc_ref_finalize(void);
/* Status of the last reference-ABI call (MOC_OK == 0). */
int moc_ref_status(void);
/* Sub-segments of the last sweep (Input.segments_processed). */
int64_t moc_ref_last_segments(void);
/* Host milliseconds the last sweep spent drawing its rand() values
 * (MOC_REF_RNG_LIBC: one libc rand() value per sub-segment on the calling
 * thread, the serial reference's sequence; 0 in the hash mode). */
double moc_ref_last_rng_ms(void);
/* The draws of MOC_REF_RNG_LIBC: the next n values of the process's rand()
 * sequence into out, libc's state left as n rand() calls leave it.  With
 * glibc's additive generator states (the default one included) they are
 * produced in bulk from the generator's state (*bulk = 1, after a one-time
 * check against rand() itself); otherwise by n rand() calls (*bulk = 0).  No
 * other thread may call rand() meanwhile, as in the serial reference.
 * MOC_ERR_ARG for n < 0 or a NULL out with n > 0; bulk may be NULL. */
int moc_ref_libc_draws(int32_t *out, int64_t n, int *bulk);

#ifdef __cplusplus
}
#endif
#endif
