/*
 * ref_harness.c -- drives the reference's own compiled solver on explicit
 * segment streams (test infrastructure only).
 *
 * Built by oracle/Makefile against the UNMODIFIED reference sources
 * (src/solver.c, src/utils.c, src/io.c of the mounted SimpleMOC tree, with the
 * reference's own SimpleMOC_header.h), serial, -O2, no fast-math.  Nothing of
 * the reference is copied here: this file only fills the reference's
 * Input / Params / Source / Track structs with pointers into the flat arrays
 * of an oracle_problem and calls
 *   attenuate_fluxes / attenuate_FSR_fluxes  (src/solver.c:14, :1040)
 *   renormalize_flux                         (src/solver.c:1143)
 *   update_sources                           (src/solver.c:1235)
 *   compute_keff                             (src/solver.c:1324)
 *   buildExponentialTable                    (src/utils.c:48)
 *   load_OpenMOC_tracks                      (src/tracks.c:170)
 * The only restated part is the traversal: the reference draws the source
 * region of each 3D segment from a time-seeded rand_r (src/solver.c:476-483)
 * and splits 2D segments axially; here every 3D track walks its explicit
 * stream of S segments (length seg_len, source seg_src) and advances
 * z <- wrap(z + ds*mu, [0, H)), with ds and mu formed as src/solver.c:373,382.
 */
#include "SimpleMOC_header.h"
#include "moc_oracle.h"

static Input I;
static Params Pr;
static const oracle_problem *PP;
static Source *src;
static Track *track_data;
static Track **track_rows;
static Track ***tracks;
static float **fs_rows, **ff_rows, **xs_rows, **sc_rows;
static AttenuateVars A;
static float *A_buf;
static float leak;

static Track2D *tracks2d;
static Segment *segs2d;

void refh_teardown(void)
{
  free(tracks2d); free(segs2d);
  tracks2d = NULL; segs2d = NULL;
  free(src); free(track_data); free(track_rows); free(tracks);
  free(fs_rows); free(ff_rows); free(xs_rows); free(sc_rows); free(A_buf);
  if (Pr.expTable.values) free(Pr.expTable.values);
  src = NULL; track_data = NULL; track_rows = NULL; tracks = NULL;
  fs_rows = ff_rows = xs_rows = sc_rows = NULL; A_buf = NULL;
  Pr.expTable.values = NULL;
}

/* The reference's own exponential table (src/utils.c:48-78). */
int refh_table(float precision, float *values, int cap, float *dx, float *maxval)
{
  Table t = buildExponentialTable(precision, 10.0);
  if (t.N > cap) { free(t.values); return -t.N; }
  memcpy(values, t.values, sizeof(float) * 2 * (size_t)t.N);
  *dx = t.dx;
  *maxval = t.maxVal;
  int n = t.N;
  free(t.values);
  return n;
}

int refh_setup(const oracle_problem *P, float precision, float *fine_source,
               float *fine_flux, float *psi_f, float *psi_b)
{
  refh_teardown();
  PP = P;
  memset(&I, 0, sizeof I);
  I.n_egroups = P->G;
  I.fai = P->F;
  I.cai = P->cai;
  I.decomp_assemblies_ax = P->decomp_ax;
  I.height = P->height;
  I.axial_exp = P->axial_exp;
  I.n_source_regions_per_node = P->NS;
  I.ntracks_2D = P->N2D;
  I.n_polar_angles = P->P;
  I.z_stacked = P->Z;
  I.ntracks = P->N2D * P->P * P->Z;
  I.precision = precision;
  I.mype = 1;                       /* keeps the reference's progress prints quiet */

  const long G = P->G, F = P->F, NS = P->NS;
  long n_sigt_rows = 0, n_xs_rows = 0;
  for (long s = 0; s < NS; s++) {
    if (P->src_sigt[s] + 1 > n_sigt_rows) n_sigt_rows = P->src_sigt[s] + 1;
    if (P->src_xs[s] + 1 > n_xs_rows) n_xs_rows = P->src_xs[s] + 1;
  }
  src = calloc(NS, sizeof(Source));
  fs_rows = malloc(sizeof(float *) * NS * F);
  ff_rows = malloc(sizeof(float *) * NS * F);
  xs_rows = malloc(sizeof(float *) * n_xs_rows * G);
  sc_rows = malloc(sizeof(float *) * n_xs_rows * G);
  for (long m = 0; m < n_xs_rows; m++)
    for (long g = 0; g < G; g++) {
      xs_rows[m * G + g] = (float *)&P->xs[(m * G + g) * 3];
      sc_rows[m * G + g] = (float *)&P->scatter[(m * G + g) * G];
    }
  for (long s = 0; s < NS; s++) {
    for (long f = 0; f < F; f++) {
      fs_rows[s * F + f] = &fine_source[(s * F + f) * G];
      ff_rows[s * F + f] = &fine_flux[(s * F + f) * G];
    }
    src[s].fine_source = &fs_rows[s * F];
    src[s].fine_flux = &ff_rows[s * F];
    src[s].vol = P->vol[s];
    src[s].sigT = (float *)&P->sigt[(long)P->src_sigt[s] * G];
    src[s].XS = &xs_rows[(long)P->src_xs[s] * G];
    src[s].scattering_matrix = &sc_rows[(long)P->src_xs[s] * G];
  }
  const long N3D = I.ntracks;
  track_data = calloc(N3D, sizeof(Track));
  track_rows = malloc(sizeof(Track *) * P->N2D * P->P);
  tracks = malloc(sizeof(Track **) * P->N2D);
  for (long i = 0; i < P->N2D; i++) {
    tracks[i] = &track_rows[i * P->P];
    for (int j = 0; j < P->P; j++)
      tracks[i][j] = &track_data[(i * P->P + j) * P->Z];
  }
  for (long t = 0; t < N3D; t++) {
    track_data[t].p_weight = P->p_weight[t];
    track_data[t].z_height = P->z0[t];
    track_data[t].f_psi = &psi_f[t * G];
    track_data[t].b_psi = &psi_b[t * G];
  }
  Pr.tracks_2D = NULL;
  Pr.tracks = tracks;
  Pr.sources = src;
  Pr.polar_angles = (float *)P->polar_angles;
  leak = 0;
  Pr.leakage = &leak;
  Pr.expTable = buildExponentialTable(precision, 10.0);   /* src/init.c:156 */

  A_buf = malloc(sizeof(float) * 14 * G);                  /* src/solver.c:317-345 */
  float *p = A_buf;
  A.q0 = p; p += G; A.q1 = p; p += G; A.q2 = p; p += G; A.sigT = p; p += G;
  A.tau = p; p += G; A.sigT2 = p; p += G; A.expVal = p; p += G; A.reuse = p; p += G;
  A.flux_integral = p; p += G; A.tally = p; p += G; A.t1 = p; p += G;
  A.t2 = p; p += G; A.t3 = p; p += G; A.t4 = p;
  return 0;
}

long refh_sweep(void)
{
  const oracle_problem *P = PP;
  const long S = P->S, PZ = (long)P->P * P->Z, N3D = P->N2D * PZ;
  float Hd = I.height / I.decomp_assemblies_ax;
  long segments = 0;
  for (long t = 0; t < N3D; t++) {
    long i = t / PZ;
    int j = (int)((t / P->Z) % P->P);
    float p_angle = Pr.polar_angles[j];
    float mu = cos(p_angle);                               /* src/solver.c:373 */
    Track *track = &track_data[t];
    float z = P->z0[t];
    for (long n = 0; n < S; n++) {
      float ds = P->seg_len[i * S + n] / sin(p_angle);     /* src/solver.c:382 */
      long qsr = P->seg_src[t * S + n];
      track->z_height = z;
      if (I.axial_exp == 2)
        attenuate_fluxes(track, true, &src[qsr], &I, &Pr, ds, mu, P->az_weight[i], &A);
      else
        attenuate_FSR_fluxes(track, true, &src[qsr], &I, &Pr, ds, mu, P->az_weight[i], &A);
      segments++;
      float dzt = ds * mu;
      z = z + dzt;
      while (z >= Hd) z -= Hd;
      while (z < 0.0f) z += Hd;
    }
    track->z_height = P->z0[t];                            /* src/solver.c:514-521 */
  }
  I.segments_processed = segments;
  return segments;
}

/* ---- the reference's own transport_sweep over a reference-style geometry --- */

/* Fills Params.tracks_2D (2D tracks with their own segment counts) and the
 * stacked-ray heights, on top of a refh_setup() problem. */
int refh_setup_ref(const oracle_refgeo *R, const float *z_height, float axial_z_sep)
{
  free(tracks2d); free(segs2d);
  const long N2D = R->N2D;
  tracks2d = calloc(N2D, sizeof(Track2D));
  segs2d = calloc(R->seg_off[N2D] > 0 ? R->seg_off[N2D] : 1, sizeof(Segment));
  for (long i = 0; i < N2D; i++) {
    tracks2d[i].az_weight = R->az_weight[i];
    tracks2d[i].n_segments = R->seg_off[i + 1] - R->seg_off[i];
    tracks2d[i].segments = &segs2d[R->seg_off[i]];
    for (long n = 0; n < tracks2d[i].n_segments; n++)
      tracks2d[i].segments[n].length = R->seg_len[R->seg_off[i] + n];
  }
  Pr.tracks_2D = tracks2d;
  I.axial_z_sep = axial_z_sep;
  for (long t = 0; t < I.ntracks; t++) {
    track_data[t].z_height = z_height[t];
    track_data[t].p_weight = R->p_weight[t];
  }
  return 0;
}

/* The reference's transport_sweep (src/solver.c:283-552, serial build: the
 * source regions come from libc rand(), seeded by the caller's srand). */
long refh_transport_sweep(float *z_height_out)
{
  transport_sweep(&Pr, &I);
  for (long t = 0; t < I.ntracks; t++)
    z_height_out[t] = track_data[t].z_height;
  return I.segments_processed;
}

void refh_renormalize(void)
{
  CommGrid grid;
  memset(&grid, 0, sizeof grid);
  renormalize_flux(Pr, I, grid);
}

float refh_update_sources(float keff)
{
  return update_sources(Pr, I, keff);
}

float refh_compute_keff(void)
{
  CommGrid grid;
  memset(&grid, 0, sizeof grid);
  return compute_keff(Pr, I, grid);
}

/* The reference's own OpenMOC track-file reader (src/tracks.c:170-323):
 * loads `path` and copies out what the traversal uses (per 2D track its
 * segment count, per segment its float length and region id), with the
 * reader's metadata.  Returns the number of 2D tracks, or -1 when the caller's
 * arrays (cap_tracks, cap_segs) are too small. */
long refh_load_openmoc(const char *path, int cmfd, long cap_tracks, long cap_segs,
                       int *n_azimuthal, float *ray_sep, long *segments_per_track,
                       long *n_segments, float *lengths, long *source_ids)
{
  Input in;
  memset(&in, 0, sizeof in);
  in.n_polar_angles = 1;
  in.z_stacked = 1;
  size_t nbytes = 0;
  Track2D *t = load_OpenMOC_tracks((char *)path, cmfd != 0, &in, &nbytes);
  long n = in.ntracks_2D, k = 0;
  if (n > cap_tracks) n = -1;
  for (long i = 0; n >= 0 && i < n; i++) {
    n_segments[i] = t[i].n_segments;
    for (long s = 0; s < t[i].n_segments; s++, k++) {
      if (k >= cap_segs) { n = -1; break; }
      lengths[k] = t[i].segments[s].length;
      source_ids[k] = t[i].segments[s].source_id;
    }
  }
  *n_azimuthal = in.n_azimuthal;
  *ray_sep = in.radial_ray_sep;
  *segments_per_track = in.segments_per_track;
  if (in.ntracks_2D > 0) free(t[0].segments);      /* the loader's contiguous block */
  free(t);
  return n;
}
