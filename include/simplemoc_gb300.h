/*
 * simplemoc_gb300.h -- C ABI of the GB300 transport-sweep library
 * (libsimplemoc_gb300.so).
 *
 * The library replaces the solver layer of SimpleMOC (src/solver.c) and the
 * track / source storage it reads (src/tracks.c, src/source.c) with device
 * resident storage and hand-written sm_103a kernels.  Every entry point takes
 * plain pointers and sizes and returns an int status (MOC_OK == 0); the
 * library never calls exit().  One problem handle is driven from one host
 * thread on one CUDA stream, like the reference's single-threaded driver.
 *
 * Storage model (flat, row-major, group index fastest):
 *   2D tracks      N2D, each with S segments          seg_len[N2D*S]
 *   3D tracks      N3D = N2D*P*Z, index (i*P + j)*Z + k (src/tracks.c:100-101)
 *   3D segments    seg_src[N3D*S]: source region of segment n of track t
 *   sources        NS regions, F fine axial intervals each; an FSR is (s, f)
 *   fine_source    [NS*F*G]  (src/source.c:137 row stride G)
 *   fine_flux      [NS*F*G]  (src/source.c:146)
 *   sigma_t table  [n_sigt*G], row src_sigt[s] for source s
 *   xs table       [n_xs*G*3] = (nu*SigmaF, SigmaA, chi)  (src/source.c:53-55)
 *   scatter table  [n_xs*G*G], row g = destination group  (src/solver.c:1279)
 *   psi_f, psi_b   [N3D*G] angular flux at the track ends (src/tracks.c:135-138)
 */
#ifndef SIMPLEMOC_GB300_H
#define SIMPLEMOC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define MOC_OK               0
#define MOC_ERR_ARG          1  /* invalid argument or inconsistent sizes      */
#define MOC_ERR_CUDA         2  /* a CUDA runtime call failed                  */
#define MOC_ERR_OOM          3  /* device allocation failed                    */
#define MOC_ERR_STATE        4  /* call out of order / handle not usable       */
#define MOC_ERR_TIMEOUT      5  /* a bounded device wait gave up               */
#define MOC_ERR_UNSUPPORTED  6  /* mode or size not supported by the library  */
#define MOC_ERR_NO_DEVICE    7  /* no CUDA device visible                      */

/* ---- sweep arithmetic modes (moc_set_mode) ----------------------------- */
/* PLAIN: the reference arithmetic of attenuate_fluxes (src/solver.c:14-280)
 * and attenuate_FSR_fluxes (src/solver.c:1040-1138) operation by operation in
 * FP32 with the reference interpolation table (src/solver.c:1441-1464); the
 * angular flux of every track is bit-identical to the reference's. */
#define MOC_MODE_PLAIN   0
/* MIXED: FP32 attenuation with fused multiply-adds, precomputed reciprocals
 * and an accurate 1-exp(-tau) (SFU exponential plus a series below a cut-off);
 * FP64 reductions.  Errors are stated against the FP64 mode. */
#define MOC_MODE_MIXED   1
/* FP64: the same formulas in double precision with exact 1-exp(-tau); the
 * high-precision yardstick for MIXED at sizes a CPU cannot sweep. */
#define MOC_MODE_FP64    2

/* mode flags */
#define MOC_FLAG_COMPENSATED 0x1  /* MIXED: compensated (hi/lo) FSR tallies  */
/* MIXED runs update_sources' scatter/fission contraction on the tensor cores
 * (split TF32, FP32 accumulation; up to 104 groups); this flag keeps it on the
 * CUDA cores instead. */
#define MOC_FLAG_SIMT_UPDATE 0x2
/* PLAIN or MIXED: deterministic-order tallies.  The sweep records every
 * segment's contribution instead of adding it; the contributions of each FSR
 * are then added to the scalar flux in the serial order of the tracks and
 * their segments (track t before t + 1, segment n before n + 1), the order of
 * the reference's serial sweep over the same tracks (its tally
 * fine_flux[g] += ..., src/solver.c:212-228).  The flux is then the same in
 * every run, and in PLAIN equal bit for bit to the serial reference's.  The
 * records take up to ~2 GiB of device memory, in chunks of whole 2D tracks;
 * the sweep takes a few times longer.  Explicit segment streams, up to 256
 * groups, not with MOC_FLAG_COMPENSATED (MOC_ERR_UNSUPPORTED). */
#define MOC_FLAG_DETERMINISTIC 0x4
/* FP64 only: FP64 arithmetic on state stored as FP32 values.  The scalar
 * flux and angular flux are rounded to FP32 after each sweep and
 * renormalisation, the fine source after each update, as an FP32-state solver
 * stores them.  Its distance from the plain FP64 mode is the error floor that
 * FP32 storage of the state alone sets (a yardstick for MIXED, which stores its
 * state in FP32). */
#define MOC_FLAG_FP32_STATE 0x8

/* ---- problem description ---------------------------------------------- */
typedef struct moc_dims {
  int32_t n_groups;      /* G   Input.n_egroups                              */
  int32_t fai;           /* F   fine axial intervals per coarse interval     */
  int32_t cai;           /*     coarse axial intervals                        */
  int32_t decomp_ax;     /*     Input.decomp_assemblies_ax                    */
  float   height;        /*     Input.height                                  */
  int32_t axial_exp;     /*     2 = quadratic source, 0 = flat source         */
  int64_t n_sources;     /* NS  Input.n_source_regions_per_node              */
  int32_t n_sigt;        /*     rows of the sigma_t table                     */
  int32_t n_xs;          /*     rows of the xs / scatter tables               */
  int64_t n_tracks_2d;   /* N2D Input.ntracks_2D                              */
  int32_t n_polar;       /* P   Input.n_polar_angles                          */
  int32_t z_stacked;     /* Z   Input.z_stacked                               */
  int32_t n_seg;         /* S   segments per 3D track                         */
  int32_t table_n;       /*     exponential table intervals (Table.N)         */
  float   table_dx;      /*     Table.dx                                      */
  float   table_maxval;  /*     Table.maxVal (already reduced by dx)          */
} moc_dims;

typedef struct moc_host {
  const float   *seg_len;      /* [N2D*S]    2D segment lengths               */
  const int32_t *seg_src;      /* [N3D*S]    source region of each 3D segment */
  const float   *az_weight;    /* [N2D]      Track2D.az_weight                */
  const float   *p_weight;     /* [N3D]      Track.p_weight                   */
  const float   *z0;           /* [N3D]      Track.z_height at sweep start    */
  const float   *polar_angles; /* [P]        Params.polar_angles              */
  const int32_t *src_sigt;     /* [NS]       sigma_t row of each source       */
  const int32_t *src_xs;       /* [NS]       xs / scatter row of each source  */
  const float   *vol;          /* [NS]       Source.vol                       */
  const float   *sigt;         /* [n_sigt*G]                                  */
  const float   *xs;           /* [n_xs*G*3]                                  */
  const float   *scatter;      /* [n_xs*G*G]                                  */
  const float   *fine_source;  /* [NS*F*G]                                    */
  const float   *fine_flux;    /* [NS*F*G]   NULL = zeros                     */
  const float   *psi_f;        /* [N3D*G]    NULL = zeros                     */
  const float   *psi_b;        /* [N3D*G]    NULL = zeros                     */
  const float   *table;        /* [2*table_n] (slope, intercept) pairs        */
} moc_host;

typedef struct moc_problem moc_problem;   /* opaque device-side problem */

/* ---- exponential table (host) ------------------------------------------ */
/* Number of intervals buildExponentialTable uses (src/utils.c:54). */
int32_t moc_exp_table_size(float precision, float maxval);
/* Fills values[2*N] exactly as buildExponentialTable (src/utils.c:48-78),
 * and the derived dx and reduced maxVal. */
int moc_build_exp_table(float precision, float maxval, float *values,
                        int32_t n, float *dx_out, float *maxval_out);

/* ---- synthetic problem generator (host, seeded, counter-based) ---------- */
typedef struct moc_gen_params {
  uint64_t seed;
  int32_t  n_materials;     /* rows of every cross-section table (8)          */
  int32_t  n_fuel;          /* materials < n_fuel carry nu*SigmaF (4)          */
  float    len_lo, len_hi;  /* 2D segment length range (0.05, 1.5) cm         */
  float    sigt_lo, sigt_hi;/* sigma_t range (0.1, 2.0) /cm                   */
  float    scatter_ratio;   /* scatter row sum (0.7)                           */
  float    nusf_hi;         /* nu*SigmaF ~ U(0, nusf_hi) in fuel (0.05)        */
  float    siga_ratio;      /* SigmaA = siga_ratio * sigma_t (0.3)             */
  float    vol_lo, vol_hi;  /* source volume range (0.5, 1.5)                 */
  float    axial_z_sep;     /* stacked-ray spacing; 0 = height / Z            */
} moc_gen_params;

/* Fills every array of `out` (caller-allocated with the sizes given by
 * `dims`; psi and fine_flux may be NULL and are then left alone).  Values
 * depend only on (seed, array, index), never on the thread count. */
int moc_generate(const moc_dims *dims, const moc_gen_params *gp,
                 float *seg_len, int32_t *seg_src, float *az_weight,
                 float *p_weight, float *z0, float *polar_angles,
                 int32_t *src_sigt, int32_t *src_xs, float *vol, float *sigt,
                 float *xs, float *scatter, float *fine_source);

/* ---- device problem lifecycle ------------------------------------------ */
/* Replaces the one-time setup of build_tracks (src/init.c:106-159) on the
 * device: allocates device storage for `dims` and uploads `host`. */
int moc_create(const moc_dims *dims, const moc_host *host, int device,
               moc_problem **out);
int moc_destroy(moc_problem *p);
/* Re-uploads every input array of `host` into the existing storage (same
 * dims).  The per-track arrays (seg_src, psi_f, psi_b) are copied on a second
 * stream in up to 8 chunks of whole 2D tracks (the first 1/256 of them, each
 * next chunk 4x the one before) and the call returns with them in flight: the
 * next moc_transport_sweep / moc_power_iteration sweeps each chunk as soon as
 * it lands, and every other call waits for the copies first.  The host arrays
 * must stay unchanged until a call that waits for the device (moc_synchronize,
 * moc_download, moc_power_iteration with outputs, ...) has returned.
 * Invalid input is MOC_ERR_ARG: from this call for everything but the
 * per-segment source ids, which the sweep checks as it reads them (an id out
 * of range is swept as source 0); the first call after that sweep that waits
 * for the device returns MOC_ERR_ARG.  Either way every other call then
 * returns MOC_ERR_STATE until an upload succeeds (the device state is partly
 * overwritten); the handle itself stays usable for that upload.
 * The scalar flux of a streamed upload goes to a side buffer (one more
 * fine_flux-sized array, allocated by the first streamed upload when the
 * handle's device budget allows, else the flux is copied into place) and is
 * added to the sweep's tallies once it has landed, so the first sweep waits
 * for the fine source only. */
int moc_upload(moc_problem *p, const moc_host *host);
/* Copies results back (any pointer may be NULL to skip that array). */
int moc_download(moc_problem *p, float *fine_flux, float *fine_source,
                 float *psi_f, float *psi_b);
/* FP64 state (valid after moc_set_mode(MOC_MODE_FP64)); NULL skips. */
int moc_download64(moc_problem *p, double *fine_flux, double *fine_source,
                   double *psi_f, double *psi_b);
/* Sticky error status of the handle (first failure since create). */
int moc_status(const moc_problem *p);
const char *moc_status_string(int status);
/* Device bytes held by the handle. */
int64_t moc_device_bytes(const moc_problem *p);

/* ---- modes and launch shape -------------------------------------------- */
int moc_set_mode(moc_problem *p, int mode, int flags);
/* Threads per track (4, 8, 16 or 32) and 4-group chunks per thread (1, 2, 4)
 * for the sweep kernel, or 10 threads x 5 two-group chunks (up to 100 groups,
 * three tracks a warp), or 10 threads x 1 four-group chunk (up to 40 groups,
 * three tracks a warp); 0, 0 = pick automatically (autotuner choice). */
int moc_set_launch(moc_problem *p, int threads_per_track, int chunks_per_thread);
int moc_get_launch(const moc_problem *p, int *threads_per_track,
                   int *chunks_per_thread);
/* The sweep's pipeline: 0 prefetches the next segment's fine-source rows into
 * registers; 4 copies them into a 4-stage shared-memory ring per track with
 * the bulk-copy engine, 3 segments ahead (MIXED and PLAIN, explicit streams);
 * -1 = automatic (moc_autotune times both). */
int moc_set_pipeline(moc_problem *p, int stages);
int moc_get_pipeline(const moc_problem *p, int *stages);

/* Autotuner: times every launch shape of the current mode on the first
 * n_tracks tracks (0 = up to 262144), with scratch tally and angular-flux
 * buffers so that the problem's state is unchanged, and selects the fastest.
 * Choices are cached per (segments per track, groups, polar angles, mode,
 * source order, compensation); with ms_best == NULL a cached choice is reused
 * without timing. */
int moc_autotune(moc_problem *p, int64_t n_tracks, int *threads_per_track,
                 int *chunks_per_thread, double *ms_best);

/* ---- the hot path (replaces src/solver.c) ------------------------------- */
/* transport_sweep (src/solver.c:283-552) over the explicit 3D tracks:
 * attenuates every segment, tallies fine_flux, updates psi_f in place.
 * *segments_processed = N3D*S (Input.segments_processed, solver.c:549). */
int moc_transport_sweep(moc_problem *p, int64_t *segments_processed);
/* renormalize_flux (src/solver.c:1143-1230), FP64 fission-rate sum. */
int moc_renormalize_flux(moc_problem *p);
/* update_sources (src/solver.c:1235-1320); returns the source residual. */
int moc_update_sources(moc_problem *p, double keff, double *residual);
/* compute_keff (src/solver.c:1324-1437); leakage as Params.leakage. */
int moc_compute_keff(moc_problem *p, double leakage, double *keff);
/* One power iteration of src/main.c:57-92 (sweep, renormalize, update with
 * keff_in, compute keff). */
int moc_power_iteration(moc_problem *p, double keff_in, double *keff_out,
                        double *residual);
/* Waits for the handle's stream. */
int moc_synchronize(moc_problem *p);

/* ---- timing helpers (CUDA events on the handle's stream) --------------- */
/* Runs `iters` sweeps and returns the mean device time of one sweep kernel
 * launch in milliseconds, measured with events on the launching stream. */
int moc_time_sweep(moc_problem *p, int iters, double *ms_per_sweep);
/* Runs `iters` power iterations back to back with k_eff kept on the device
 * (update_sources of iteration i uses the k_eff of iteration i-1, starting
 * from the last value computed or given).  Reports the device time of the
 * whole sequence and of the sweep kernels alone (both from events on the
 * launching stream) and the final k_eff and residual. */
int moc_time_power_iterations(moc_problem *p, int iters, double *ms_total,
                              double *ms_sweeps, double *keff, double *residual);
/* Per-phase device times of `iters` power iterations, under the phases of the
 * reference's results summary (src/main.c:103-113): phase_ms[MOC_N_PHASES],
 * milliseconds summed over the iterations, from events on the launching
 * stream.  The exchange phase is 0 on one device (the track-partitioned
 * sweep's all-reduce runs outside the handle).  update_sources and
 * compute_keff run as the reference's two calls, k_eff chained on the device
 * (moc_power_iteration fuses their passes over the flux). */
#define MOC_PHASE_SWEEP       0   /* Transport Sweep Time         */
#define MOC_PHASE_EXCHANGE    1   /* Domain Flux Exchange Time    */
#define MOC_PHASE_RENORMALIZE 2   /* Flux Renormalization Time    */
#define MOC_PHASE_UPDATE      3   /* Update Source Time           */
#define MOC_PHASE_KEFF        4   /* K-Effective Calc Time        */
#define MOC_N_PHASES          5
int moc_time_phases(moc_problem *p, int iters, double *phase_ms, double *keff,
                    double *residual);
/* Number of kernels the library has launched on this handle so far. */
int64_t moc_launch_count(const moc_problem *p);

/* ---- state on device pointers (row stride n_groups) --------------------- */
int moc_set_fine_source_device(moc_problem *p, const float *q);
int moc_set_fine_source64_device(moc_problem *p, const double *q);  /* FP64 mode */
/* Replaces the sigma_t table (host array [n_sigt*G]) and its coefficients. */
int moc_set_sigma_t(moc_problem *p, const float *sigt);
/* Zeroes the scalar flux (a fixed-source sweep tallies from zero) and/or the
 * angular flux, in every precision held. */
int moc_zero_state(moc_problem *p, int flux, int psi);
int moc_get_fine_flux_device(moc_problem *p, float *phi);
int moc_get_fine_flux64_device(moc_problem *p, double *phi);   /* FP64 mode */
/* The handle's own scalar-flux storage (FP32, or FP64 in the FP64 mode):
 * [NS*F][ldg] with ldg = G rounded up to a multiple of 4; the padding columns
 * stay zero.  For a collective on the flux in place (the track-partitioned
 * sweep sums the ranks' tallies with an all-reduce, the MPI_Allreduce of
 * src/solver.c:1189-1196 widened from the fission rate to the flux): the
 * caller orders its own access after moc_synchronize and finishes it before
 * the handle's next call.  Any pending streamed upload is joined first. */
int moc_fine_flux_storage(moc_problem *p, void **ptr, int64_t *n_elems, int32_t *ldg,
                          int32_t *elem_bytes);

/* ---- failure handling ---------------------------------------------------
 * Every call returns a status; after a CUDA failure, or after a kernel found an
 * invalid input or a bounded device wait ran out (reported by the next call
 * that waits for the device: MOC_ERR_ARG / MOC_ERR_TIMEOUT), the handle's status
 * is sticky and later calls return MOC_ERR_STATE.  Other handles and the CUDA
 * context stay usable: no kernel of the library traps.
 *
 * moc_set_memory_limit caps the device bytes one handle may allocate (0: no
 * cap; allocations beyond it are MOC_ERR_OOM, e.g. to keep several handles
 * inside a budget or to test out-of-memory handling).
 * moc_inject_fault marks a handle as a failing call would (host side, for
 * tests of a caller's error handling):
 *   MOC_FAULT_CUDA            a failed CUDA call (status MOC_ERR_CUDA, sticky)
 *   MOC_FAULT_DEVICE_INPUT    a kernel's input check (next wait: MOC_ERR_ARG)
 *   MOC_FAULT_DEVICE_TIMEOUT  a bounded device wait (next wait: MOC_ERR_TIMEOUT)
 * moc_selftest_wait runs a kernel whose wait nothing completes, bounded by
 * `cycles` SM clocks (1 .. 2^32): it returns MOC_ERR_TIMEOUT. */
#define MOC_FAULT_CUDA           0
#define MOC_FAULT_DEVICE_INPUT   1
#define MOC_FAULT_DEVICE_TIMEOUT 2
int moc_set_memory_limit(int64_t bytes);
int moc_inject_fault(moc_problem *p, int kind);
int moc_selftest_wait(moc_problem *p, int64_t cycles);

/* ---- OpenMOC track files (src/tracks.c:170-323, the reference's -d input) --
 * moc_openmoc_probe reads the sizes of a track file; moc_openmoc_read fills
 * caller arrays sized from them (any output may be NULL):
 *   num_tracks, num_x, num_y, azim_weights  [n_azimuthal]
 *   track_geometry [N2D][5] (x0, y0, x1, y1, phi), azim_index [N2D]
 *   seg_off [N2D+1], seg_len / material_id / region_id [n_segments]
 * Lengths are converted to float as the reference does.  cmfd != 0: the
 * segments carry the two CMFD mesh-surface ids.  A missing, short or
 * inconsistent file is MOC_ERR_ARG (the reference does not check). */
int moc_openmoc_probe(const char *path, int cmfd, int32_t *n_azimuthal, double *spacing,
                      int64_t *n_tracks_2d, int64_t *n_segments);
int moc_openmoc_read(const char *path, int cmfd, int64_t n_tracks_2d, int64_t n_segments,
                     int32_t *num_tracks, int32_t *num_x, int32_t *num_y,
                     double *azim_weights, double *track_geometry, int32_t *azim_index,
                     int64_t *seg_off, float *seg_len, int32_t *material_id,
                     int32_t *region_id);

/* ---- adjoint sweep (no counterpart in the reference) ------------------- */
/* Reverse-mode derivative of one transport sweep in the MIXED arithmetic
 * (the PLAIN table is piecewise linear with jumps, not differentiable).
 * moc_adjoint_forward runs the sweep (tallies added to the scalar flux, psi_f
 * updated) and checkpoints the angular flux every k_ckpt (1..8) segments.
 * moc_adjoint_backward takes dL/dphi for any loss L of the scalar flux (device
 * array [NS*F*G]) and writes, on device arrays (NULL skips):
 *   dq     [NS*F*G]       dL/d fine_source (the q0/q1/q2 fit rows)
 *   dsigt  [n_sigt*G]     dL/d sigma_t, FP64
 *   dpsi_in [N3D*G]       dL/d angular flux entering each track
 * psi is recomputed from the checkpoints, not stored per segment. */
int moc_adjoint_forward(moc_problem *p, int k_ckpt);
int moc_adjoint_backward(moc_problem *p, const float *dphi, float *dq, double *dsigt,
                         float *dpsi_in);
/* The same, with the fine-source gradient also given per quadratic fit
 * (src/solver.c:69-81): the segments that fit fine rows w, w+1, w+2 of a source
 * use q(z) = c0 + c1 z + c2 z^2 with c0 = y2, c1 = (y1 - y3)/(2dz),
 * c2 = (y1 - 2 y2 + y3)/(2dz^2), and
 *   dfit [NS][F-2][3][G]   dL/dc0, dL/dc1, dL/dc2 of window w of each source,
 * summed over those segments.  Quadratic source only (MOC_ERR_UNSUPPORTED). */
int moc_adjoint_backward_fit(moc_problem *p, const float *dphi, float *dq, double *dsigt,
                             float *dpsi_in, float *dfit);
/* Reverse mode of update_sources (src/solver.c:1235-1300) for the adjoint
 * workload, whose source is one update step from a scalar flux phi0:
 *   q[r][g] = (chi[m][g] * sum_h nuSigmaF[m][h] phi0[r][h] / k
 *              + sum_h S[m][g][h] phi0[r][h]) / (4 pi)
 * for each fine region r of a source of material m.  Given dL/dq it writes
 * (device arrays; NULL skips):
 *   dscatter [n_xs*G*G]  dL/dS, FP64 (row g = destination group)
 *   dnusf    [n_xs*G]    dL/dnuSigmaF through the fission source, FP64
 *   dphi0    [NS*F*G]    dL/dphi0
 * phi0 and dq are [NS*F*G] (row stride G).  Up to 256 groups. */
int moc_update_sources_adjoint(moc_problem *p, const float *phi0, const float *dq, double keff,
                               double *dscatter, double *dnusf, float *dphi0);
/* Replaces the cross-section tables (host arrays [n_xs*G*3] and [n_xs*G*G],
 * the layout of moc_host) and everything derived from them. */
int moc_set_cross_sections(moc_problem *p, const float *xs, const float *scatter);
/* The scalar flux from / the fine source to device arrays (row stride G). */
int moc_set_fine_flux_device(moc_problem *p, const float *phi);
int moc_get_fine_source_device(moc_problem *p, float *q);
/* Device time (events on the handle's stream) of one moc_adjoint_forward(k_ckpt)
 * and of the reverse sweep that follows it for dL/dphi (device [NS*F*G]), in
 * milliseconds; the gradients stay in the handle's work arrays. */
int moc_time_adjoint(moc_problem *p, int k_ckpt, const float *dphi, double *ms_forward,
                     double *ms_reverse);
/* Lanes per track (1..32, any width) and 4-group chunks per lane (1 or 2) of
 * the reverse sweep; 0, 0 = automatic (ceil(G/4) lanes of one chunk up to 128
 * groups).  MOC_ERR_ARG when lanes x chunks x 4 < G. */
int moc_set_adjoint_width(moc_problem *p, int lanes_per_track, int chunks_per_lane);

/* ---- batched sweep of independent problems ------------------------------ */
/* Many independent problems ("cores", e.g. small reactor cores of different
 * sizes and group counts) on one device, swept by ONE persistent launch: warps
 * take (core, tracks) tasks from a work counter, the largest first, each core
 * with its own threads per track.  The batch references the problems (they
 * stay owned by the caller and keep their own state); all must share the
 * device, mode (PLAIN or MIXED), source order and exponential table, and have
 * at most 256 groups. */
typedef struct moc_batch moc_batch;
int moc_batch_create(int n, moc_problem *const *problems, moc_batch **out);
int moc_batch_destroy(moc_batch *b);
/* Autotuner of the batch: per distinct (segments per track, groups, polar
 * angles, mode) the threads per track of the fastest measured launch. */
int moc_batch_autotune(moc_batch *b);
int moc_batch_set_width(moc_batch *b, int core, int threads_per_track);
int moc_batch_widths(const moc_batch *b, int *threads_per_track);
/* One batched transport sweep (waits for it). */
int moc_batch_sweep(moc_batch *b);
/* `iters` power iterations of every core (batched sweep, then each core's
 * renormalize_flux / update_sources / compute_keff with k_eff kept on the
 * device); use_graph captures one iteration as a CUDA graph and replays it.
 * Every call makes exactly `iters` iterations: before it captures (its first
 * call, and the first after an upload or a mode flag change of a core) it runs
 * the first of them without the graph and replays the rest.  *ms_total =
 * device time of the `iters` iterations (events on the batch stream; a call
 * that captures also counts the time the device waits for the capture).  Each
 * call first waits for the cores' own streams and refreshes their sweep
 * arguments. */
int moc_batch_power_iterations(moc_batch *b, int iters, int use_graph,
                               double *ms_total);
/* Per-core k_eff and source residual of the last iteration. */
int moc_batch_results(moc_batch *b, double *keff, double *residual);
int64_t moc_batch_launch_count(const moc_batch *b);

/* ---- renormalize_flux without device allocation ------------------------ */
/* No counterpart in the reference.  For callers that cannot let the library
 * call cudaMalloc (a framework or pool allocator that accounts for every
 * device byte, a real-time loop that allocates nothing after start-up,
 * buffers mapped from another process): the same computation as
 * moc_renormalize_flux on device buffers the caller owns, in the reference
 * layout (row stride n_groups):
 *   fine_flux [n_sources*fai*n_groups]  in/out   psi_f, psi_b [n_tracks_3d*n_groups] in/out
 *     (psi_f and psi_b may be NULL when n_tracks_3d == 0)
 *   vol [n_sources], src_xs [n_sources], xs [n_xs*n_groups*3]  in
 *   norm_out: NULL or a device double[2] receiving (total fission rate, norm)
 * Launches on `stream` (a cudaStream_t; NULL = the legacy default stream) and
 * returns without waiting.  Its scratch is a static device array of
 * MOC_NOALLOC_SCRATCH_BYTES reserved on every GPU that loads the library until
 * the process exits; n_sources above MOC_NOALLOC_MAX_SOURCES, or element
 * counts above 2^50, are rejected with MOC_ERR_ARG.  The first call on a
 * device looks up the array's device address (make it before any stream
 * capture); a call that finds another context current on the device (after a
 * cudaDeviceReset) looks it up again.  All calls share the one array: calls
 * whose kernels overlap on the GPU race. */
#define MOC_NOALLOC_MAX_SOURCES (1 << 20)
#define MOC_NOALLOC_SCRATCH_BYTES (8 * 1032 + 4 * MOC_NOALLOC_MAX_SOURCES)
int moc_renormalize_flux_noalloc(float *fine_flux, float *psi_f, float *psi_b,
                                 const float *vol, const int32_t *src_xs,
                                 const float *xs, int64_t n_sources, int32_t fai,
                                 int32_t n_groups, int64_t n_tracks_3d,
                                 double *norm_out, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* SIMPLEMOC_GB300_H */
