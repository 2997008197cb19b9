// moc_internal.h -- device-side problem state shared by the library's
// translation units (not part of the public ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstring>

#include "simplemoc_gb300.h"

#include "moc_host.h"

#include <nvtx3/nvToolsExt.h>

// NVTX range over one entry point (header-only NVTX 3: a no-op unless a
// profiler injects itself), so that a timeline shows the library's calls under
// the reference's names.
struct MocNvtxRange {
  explicit MocNvtxRange(const char *name) { nvtxRangePushA(name); }
  ~MocNvtxRange() { nvtxRangePop(); }
  MocNvtxRange(const MocNvtxRange &) = delete;
  MocNvtxRange &operator=(const MocNvtxRange &) = delete;
};
#define MOC_NVTX_CAT2(a, b) a##b
#define MOC_NVTX_CAT(a, b) MOC_NVTX_CAT2(a, b)
#define MOC_NVTX_RANGE(name) MocNvtxRange MOC_NVTX_CAT(moc_nvtx_range_, __LINE__)(name)

// Coefficients per (sigma_t row, group): the interleaved planes of moc_host.h.
enum { COEF_PLANES = MOC_COEF_PLANES };

struct SweepArgs {
  const float *seg_ds;      // [N2D*P*S] 3D segment length per (2D track, polar, seg)
  const int32_t *seg_src;   // [N3D*S]
  const float *weight;      // [N3D]  p_weight * az_weight (float, reference order)
  const float *z0;          // [N3D]
  const float *mu;          // [P]
  const int32_t *src_sigt;  // [NS]
  const float *coef;        // [n_sigt][8][ldg]
  const float2 *table;      // [N] (slope, intercept)
  const float *q;           // [NS*F*ldg]
  float *phi;               // [NS*F*ldg]
  float *phi_lo;            // [NS*F*ldg] compensation words (MIXED + flag) or null
  float *psi;               // [N3D*ldg]  forward angular flux, in place
  float *rec;               // [N3D*S*ldg] recorded tallies (deterministic mode) or null
  int32_t *rec_row;         // [N3D*S]     their FSR rows
  const float *psi_scale;   // pending renormalisation factor of psi, or null
  const double *q64;        // FP64 mode state
  double *phi64;
  double *psi64;
  int64_t n3d;
  int64_t ns;               // source regions (bound of seg_src)
  int32_t G, ldg, nchunk;   // groups, padded stride, ldg/4
  int32_t F, P, Z, S;
  int32_t axial_exp;
  int32_t table_n;
  float table_dx, table_rdx, table_halfdx, table_maxval;
  float dz, rdz;            // fine interval height and its reciprocal
  float d1, rd1, d2, rd2;   // 2 dz and 2 dz dz, and reciprocals
  float hd;                 // domain height
  // 1, -1 and -0 as values the compiler cannot see: the PLAIN pair arithmetic
  // multiplies and adds through FMAs with them, which it can neither simplify
  // nor contract (the reference rounds every product and sum on its own)
  float rt_one, rt_m1, rt_nz;
  uint32_t fmagic;          // zi % F == zi - F*umulhi(zi, fmagic) for reachable zi; 0 = use %
  int32_t *err;             // device error word (0 = ok)
  // psi checkpoints of the adjoint's forward sweep: every ck_k segments,
  // ck_n per track ([N3D][ck_n][ldg] and [N3D][ck_n] heights)
  float *ck_psi;
  float *ck_z;
  int32_t ck_k, ck_n;
  // variable-length sub-segment streams (reference traversal), else null
  const int64_t *csr_off;   // [N3D+1]
  const float *csr_ds;      // [M] sub-segment lengths
  const float *csr_z;       // [M] start heights
  const int32_t *csr_src;   // [M] source regions
};

// The next n values of the process's libc rand() sequence, libc's state
// advanced as by n calls (moc_libc_rand.cpp).  Returns 1 if they were drawn in
// bulk from libc's generator state, 0 if by n rand() calls.
int moc_libc_draws(int32_t *out, int64_t n);

struct MocDet;   // deterministic-order tally buffers (moc_determ.cu)

struct moc_problem {
  moc_dims d;
  int device = 0;
  cudaStream_t stream = nullptr;
  int status = MOC_OK;
  int mode = MOC_MODE_PLAIN;
  int flags = 0;
  int tpw = 0, cpl = 0;          // 0 = automatic
  int stages = -1;               // sweep pipeline: 0 register prefetch, N > 0 an N-stage
                                 // shared-memory ring; -1 = automatic (0 until tuned)
  int adj_tpw = 0, adj_cpl = 0;  // reverse sweep lanes per track, chunks per lane; 0 = automatic
  int64_t launches = 0;
  int64_t n3d = 0, nfsr = 0;
  int32_t ldg = 0;
  uint32_t fmagic = 0;
  int64_t bytes = 0;
  // inputs
  float *seg_ds = nullptr;
  int32_t *seg_src = nullptr;
  float *weight = nullptr, *z0 = nullptr, *mu = nullptr;
  int32_t *src_sigt = nullptr, *src_xs = nullptr;
  float *vol = nullptr, *coef = nullptr, *xs = nullptr, *scatter_t = nullptr;
  float *table = nullptr;
  // state
  float *q = nullptr, *phi = nullptr, *phi_lo = nullptr, *psi_f = nullptr, *psi_b = nullptr;
  double *q64 = nullptr, *phi64 = nullptr, *psi_f64 = nullptr, *psi_b64 = nullptr;
  // update_sources work list: sources ordered by xs row, and items
  // (xs row, first, end) of at most 128 sources each, over that order
  int32_t *xs_order = nullptr;
  int32_t *upd_items = nullptr;
  int32_t n_upd_items = 0;
  // lazy psi renormalisation (FP32 modes): psi_f holds values still to be
  // multiplied by *psi_scale while psi_pending; psi_b is scaled only when the
  // device flag psi_b_nonzero is set
  float *psi_scale = nullptr;
  int32_t *psi_b_nonzero = nullptr;
  // tensor-core update_sources (MIXED): per material the split operand
  // [hi, lo][tc_np x tc_kp] in the canonical layout, and tiles of <= 128 / F
  // sources of one material (material, first, end) in xs_order
  float *adj_dfit = nullptr;            // [NS][F-2][3][ldg] fit-coefficient adjoints
  float *tc_b = nullptr;
  int32_t *tc_items = nullptr;
  int32_t n_tc_items = 0;
  int tc_kp = 0, tc_np = 0;             // 0: groups beyond the tensor-core path
  bool psi_pending = false;
  // adjoint: psi checkpoints of the last moc_adjoint_forward and work arrays
  float *ck_psi = nullptr, *ck_z = nullptr;
  int32_t ck_k = 0, ck_n = 0;
  float *adj_dphi = nullptr, *adj_dq = nullptr;
  double *adj_dsig = nullptr;
  // reductions / scalars
  double *partials = nullptr;    // [3 * RED_BLOCKS]
  double *scalars = nullptr;     // see post kernels
  int32_t *err = nullptr;        // device error word, MOC_DEV_ERR_* bits
  int32_t red_blocks = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // Upload of the per-track arrays (segment sources, psi_f, psi_b) on a copy
  // stream in chunks of whole 2D tracks, so that the next sweep starts on the
  // first chunk while the rest are still copied.  n_chunks > 0 while an upload
  // is in flight; every other entry point first joins it (moc_join_upload).
  static constexpr int MAX_UPLOAD_CHUNKS = 8;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t main_ev = nullptr, copy_done = nullptr;
  cudaEvent_t chunk_ev[MAX_UPLOAD_CHUNKS] = {};
  int64_t chunk_end[MAX_UPLOAD_CHUNKS] = {};     // one past the chunk's last 2D track
  int n_chunks = 0;
  bool detect_pending = false;                   // psi_b's nonzero flag still to be set
  // A streamed upload copies the scalar flux into phi_in on the copy stream
  // and zeroes phi, so that the first sweep need not wait for it: the sweep
  // tallies into phi, and the join adds phi_in (the same sum in another order).
  float *phi_in = nullptr;
  bool phi_fold_pending = false;
  bool stale = false;                            // rejected input: device state undefined
  int64_t uploads = 0;                           // moc_upload calls that issued copies
  void *h_stage = nullptr;                       // pinned host staging of derived arrays
  cudaEvent_t stage_ev = nullptr;                // after the last copy from h_stage
  bool stage_pending = false;
  // deterministic-order tally mode: record / sort / ordered-add buffers
  MocDet *det = nullptr;
  // host copies needed for re-upload and derived arrays
  float polar[64];
};

// Bits of the device error word.  A source id out of range comes from the
// input of the last upload (a streamed upload leaves the ids to the sweep,
// which reads each one through a bounds check that substitutes source 0): the
// handle then refuses work until the next valid upload, where the other bits
// are failures of the handle.
constexpr int32_t MOC_DEV_ERR_ARG = 1;        // an argument error found by a kernel
constexpr int32_t MOC_DEV_ERR_TIMEOUT = 2;    // a bounded device wait gave up
constexpr int32_t MOC_DEV_ERR_SOURCE = 4;     // a segment source id out of range

// Groups one track covers with a launch shape: TPW x CPL chunks of 4 groups,
// or of 2 groups when TPW is not a power of two (10 x 5: 100 groups).
int moc_shape_groups(int tpw, int cpl);

// Launchers implemented in moc_sweep.cu / moc_post.cu.
int moc_launch_sweep(moc_problem *p);
// The sweep of 2D tracks [i2_begin, i2_end) with all their 3D tracks.
int moc_launch_sweep_range(moc_problem *p, int64_t i2_begin, int64_t i2_end);
// The sweep of 2D tracks [i2_begin, i2_end) with recorded tallies (no flux
// update): contribution of segment n of the range's track t at
// rec[(t * S + n) * ldg], its FSR row at rec_row[t * S + n].
int moc_launch_sweep_record(moc_problem *p, int64_t i2_begin, int64_t i2_end, float *rec,
                            int32_t *rec_row);
// Deterministic-order sweep (moc_determ.cu): the tallies of every FSR added in
// the serial order of the tracks and their segments.
int moc_det_sweep(moc_problem *p);
void moc_det_release(moc_problem *p);
// Device allocation counted against the handle's budget (moc_set_memory_limit).
int moc_dev_alloc(moc_problem *p, void **ptr, int64_t bytes);
void moc_dev_free(moc_problem *p, void *ptr, int64_t bytes);
// Makes the stream wait for an upload in flight (no-op when there is none).
int moc_join_upload(moc_problem *p);
// Waits for the handle's stream and folds its device error word into the
// status: MOC_ERR_ARG with the handle stale for a source id out of range (the
// input of the last upload), a failure of the handle otherwise.
int moc_sync_check(moc_problem *p);

// Tensor-core update_sources.  The second operand of tile GEMM for material m
// is B[n][k] (n < G: scatter S[m][n][k]; n = G: nuSigmaF[m][k]; n = G + 1:
// SigmaA[m][k]; zero elsewhere), K-major in 8-row x 16-byte core matrices:
// element (n, k) at float offset (k / 4) * np * 4 + n * 4 + k % 4.
constexpr int MOC_TC_MAX_NP = 112;
inline bool moc_tc_dims(int G, int F, int *kp, int *np) {
  const int k = (G + 7) / 8 * 8, n = (G + 2 + 15) / 16 * 16;
  if (G < 1 || k > 104 || n > MOC_TC_MAX_NP || F < 1 || F > 128) return false;
  *kp = k;
  *np = n;
  return true;
}
// x rounded to TF32 (10-bit significand), to nearest with ties away from zero,
// as cvt.rna.tf32.f32 does on the device.
inline float moc_tf32_rna(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  if ((u & 0x7F800000u) == 0x7F800000u) return x;     // inf, nan
  u = (u + 0x1000u) & 0xFFFFE000u;
  float r;
  std::memcpy(&r, &u, 4);
  return r;
}
inline int64_t moc_tc_b_offset(int n, int k, int np) {
  return (int64_t)(k / 4) * np * 4 + (int64_t)n * 4 + k % 4;
}
int moc_launch_update_tc(moc_problem *p);
int moc_launch_sweep_csr(moc_problem *p, const int64_t *off, const float *ds, const float *z,
                         const int32_t *src);
SweepArgs moc_sweep_args(moc_problem *p);
int moc_launch_sweep_batch(int device, cudaStream_t st, int mode, bool quad, const SweepArgs *args,
                           const int2 *tasks, int64_t n_tasks, const int *tpw,
                           unsigned long long *counter, const float2 *table, int table_n);
int moc_reset_psi_scale(moc_problem *p);
int moc_launch_sweep_ckpt(moc_problem *p, float *ck_psi, float *ck_z, int k, int nck);
int moc_launch_adjoint(moc_problem *p, const float *ck_psi, const float *ck_z, int k, int nck,
                       const float *dphi, float *dq, double *dsig, float *dpsi_in, float *dfit);
int moc_sweep_launch_shape(const moc_problem *p, int *tpw, int *cpl);
int moc_sweep_autotune(moc_problem *p, int64_t n_sub, int *tpw, int *cpl, int *stages,
                       double *ms);
int moc_launch_renormalize(moc_problem *p);
int moc_launch_update(moc_problem *p, double keff, bool keff_on_device, bool with_keff);
int moc_set_leakage(moc_problem *p, double leakage);
int moc_launch_keff(moc_problem *p, double leakage);
int moc_post_scratch_blocks();
int moc_psi_materialize(moc_problem *p);
// Adjoint of update_sources (moc_update_adj.cu): device arrays, row stride G.
int moc_launch_update_adjoint(moc_problem *p, const float *phi0, const float *dq, double keff,
                              double *dscatter, double *dnusf, float *dphi0);
// FP64 mode with MOC_FLAG_FP32_STATE: rounds the chosen state arrays to FP32
// values (no-op otherwise).
int moc_round_state_fp32(moc_problem *p, bool flux, bool psi, bool source);
int moc_detect_psi_b(moc_problem *p);

// Scalars slots in p->scalars (double):
enum {
  SC_TOTAL_FISSION = 0,   // renormalize: total fission rate
  SC_NORM = 1,            // renormalize: norm factor (as applied)
  SC_RESIDUAL = 2,        // update_sources residual
  SC_ABS = 3,             // compute_keff absorption
  SC_FISSION = 4,         // compute_keff fission
  SC_KEFF = 5,            // compute_keff result
  SC_KEFF_IN = 6,         // keff used by update_sources
  SC_LEAKAGE = 7,
  SC_COUNT = 8
};

#define MOC_CUDA_TRY(expr)                                                     \
  do {                                                                         \
    cudaError_t e_ = (expr);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      return (e_ == cudaErrorMemoryAllocation) ? MOC_ERR_OOM : MOC_ERR_CUDA;   \
    }                                                                          \
  } while (0)
