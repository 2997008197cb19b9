// moc_api.cu -- the C ABI of libsimplemoc_gb300.so: problem lifecycle,
// uploads and downloads, modes, and the four solver entry points of
// src/solver.c (transport_sweep, renormalize_flux, update_sources,
// compute_keff) over device-resident storage.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <atomic>
#include <cmath>
#include <new>
#include <vector>

#include "moc_host.h"

#include "moc_internal.h"

namespace {

__global__ void widen_kernel(const float *__restrict__ src, double *__restrict__ dst, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (double)src[i];
}

// phi += phi_in, four floats at a time (n a multiple of 4).
__global__ void add_kernel(float *__restrict__ phi, const float *__restrict__ phi_in, int64_t n) {
  float4 *a = reinterpret_cast<float4 *>(phi);
  const float4 *b = reinterpret_cast<const float4 *>(phi_in);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n / 4;
       i += (int64_t)gridDim.x * blockDim.x) {
    float4 x = a[i];
    const float4 y = b[i];
    x.x = __fadd_rn(x.x, y.x);
    x.y = __fadd_rn(x.y, y.y);
    x.z = __fadd_rn(x.z, y.z);
    x.w = __fadd_rn(x.w, y.w);
    a[i] = x;
  }
}

__global__ void fold_kernel(float *__restrict__ hi, float *__restrict__ lo, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    hi[i] = hi[i] + lo[i];
    lo[i] = 0.0f;
  }
}

// Device bytes one handle may allocate (0: no limit); moc_set_memory_limit.
std::atomic<int64_t> g_memory_limit{0};

template <typename T>
int dalloc(moc_problem *p, T **ptr, int64_t count) {
  if (count <= 0) count = 1;
  const int64_t limit = g_memory_limit.load();
  if (limit > 0 && p->bytes + (int64_t)sizeof(T) * count > limit) return MOC_ERR_OOM;
  void *d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(T) * (size_t)count);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? MOC_ERR_OOM : MOC_ERR_CUDA;
  }
  *ptr = static_cast<T *>(d);
  p->bytes += (int64_t)sizeof(T) * count;
  return MOC_OK;
}

}  // namespace

int moc_dev_alloc(moc_problem *p, void **ptr, int64_t bytes) {
  unsigned char *d = nullptr;
  const int rc = dalloc(p, &d, bytes);
  *ptr = d;
  return rc;
}

void moc_dev_free(moc_problem *p, void *ptr, int64_t bytes) {
  if (!ptr) return;
  cudaFree(ptr);
  p->bytes -= bytes > 0 ? bytes : 1;
}

namespace {

template <typename T>
void dfree(T *&ptr) {
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
}

// Copies a [rows x G] host matrix into a [rows x ldg] device matrix.
int put_rows(moc_problem *p, float *dst, const float *src, int64_t rows,
             cudaStream_t st = nullptr) {
  const int64_t G = p->d.n_groups, L = p->ldg;
  if (!st) st = p->stream;
  if (!src) {
    MOC_CUDA_TRY(cudaMemsetAsync(dst, 0, sizeof(float) * (size_t)(rows * L), st));
    return MOC_OK;
  }
  if (L == G) {
    MOC_CUDA_TRY(cudaMemcpyAsync(dst, src, sizeof(float) * (size_t)(rows * G),
                                 cudaMemcpyHostToDevice, st));
  } else {
    MOC_CUDA_TRY(cudaMemsetAsync(dst, 0, sizeof(float) * (size_t)(rows * L), st));
    MOC_CUDA_TRY(cudaMemcpy2DAsync(dst, sizeof(float) * L, src, sizeof(float) * G,
                                   sizeof(float) * G, (size_t)rows, cudaMemcpyHostToDevice, st));
  }
  return MOC_OK;
}

template <typename T>
int get_rows(moc_problem *p, T *dst, const T *src, int64_t rows) {
  const int64_t G = p->d.n_groups, L = p->ldg;
  if (L == G) {
    MOC_CUDA_TRY(cudaMemcpyAsync(dst, src, sizeof(T) * (size_t)(rows * G), cudaMemcpyDeviceToHost,
                                 p->stream));
  } else {
    MOC_CUDA_TRY(cudaMemcpy2DAsync(dst, sizeof(T) * G, src, sizeof(T) * L, sizeof(T) * G,
                                   (size_t)rows, cudaMemcpyDeviceToHost, p->stream));
  }
  return MOC_OK;
}

template <typename T>
int put(moc_problem *p, T *dst, const T *src, int64_t count, cudaStream_t st = nullptr) {
  MOC_CUDA_TRY(cudaMemcpyAsync(dst, src, sizeof(T) * (size_t)count, cudaMemcpyHostToDevice,
                               st ? st : p->stream));
  return MOC_OK;
}

#define TRY(x)                      \
  do {                              \
    int rc_ = (x);                  \
    if (rc_ != MOC_OK) return rc_;  \
  } while (0)

// Per material the tensor-core update's second operand: rows n < G the
// scatter rows S[m][n][.], n = G nuSigmaF, n = G + 1 SigmaA, split into TF32
// hi and lo planes in the canonical K-major layout.
void build_tc_b(const moc_problem *p, const float *xs, const float *scatter, float *tc_b) {
  const moc_dims &d = p->d;
  const int64_t G = d.n_groups;
  const int np = p->tc_np;
  const int64_t plane = (int64_t)np * p->tc_kp;
  std::memset(tc_b, 0, sizeof(float) * (size_t)(d.n_xs * 2 * plane));
  for (int64_t m = 0; m < d.n_xs; ++m)
    for (int n = 0; n < G + 2; ++n)
      for (int k = 0; k < G; ++k) {
        const float v = n < G ? scatter[(m * G + n) * G + k]            // S[m][to n][from k]
                              : xs[(m * G + k) * 3 + (n - G)];          // nuSigmaF, SigmaA
        const float hi = moc_tf32_rna(v);
        const int64_t o = m * 2 * plane + moc_tc_b_offset(n, k, np);
        tc_b[(size_t)o] = hi;
        tc_b[(size_t)(o + plane)] = moc_tf32_rna(v - hi);
      }
}

// Host staging of the arrays the upload derives: one pinned block per handle,
// allocated on the first upload, so that their copies are asynchronous (a copy
// from pageable memory first waits for everything queued on its stream, here
// the 2 GB of fine source and flux).  An event recorded after the last copy
// from the block guards its reuse by the next upload.
struct Staging {
  float *seg_ds, *weight, *mu, *coef, *st, *tc_b;
  int32_t *order, *items, *tc_items;
};

int staging(moc_problem *p, Staging *out) {
  const moc_dims &d = p->d;
  const int64_t G = d.n_groups, NS = d.n_sources;
  const int64_t n[9] = {
      (int64_t)d.n_tracks_2d * d.n_polar * d.n_seg,                 // seg_ds
      p->n3d,                                                       // weight
      d.n_polar,                                                    // mu
      (int64_t)d.n_sigt * COEF_PLANES * p->ldg,                     // coef
      (int64_t)d.n_xs * G * G,                                      // st
      p->tc_b ? (int64_t)d.n_xs * 2 * p->tc_np * p->tc_kp : 0,      // tc_b
      NS,                                                           // order
      3 * ((int64_t)d.n_xs + NS / 128 + 1),                         // items
      p->tc_b ? 3 * ((int64_t)d.n_xs + NS / (128 / d.fai) + 1) : 0  // tc_items
  };
  size_t off[10] = {0};
  for (int i = 0; i < 9; ++i) off[i + 1] = off[i] + ((size_t)n[i] * 4 + 63) / 64 * 64;
  if (!p->h_stage) {
    if (cudaMallocHost(&p->h_stage, off[9]) != cudaSuccess) {
      cudaGetLastError();
      p->h_stage = nullptr;
      return MOC_ERR_OOM;
    }
    MOC_CUDA_TRY(cudaEventCreateWithFlags(&p->stage_ev, cudaEventDisableTiming));
  } else if (p->stage_pending) {
    MOC_CUDA_TRY(cudaEventSynchronize(p->stage_ev));
  }
  p->stage_pending = false;
  unsigned char *b = static_cast<unsigned char *>(p->h_stage);
  out->seg_ds = reinterpret_cast<float *>(b + off[0]);
  out->weight = reinterpret_cast<float *>(b + off[1]);
  out->mu = reinterpret_cast<float *>(b + off[2]);
  out->coef = reinterpret_cast<float *>(b + off[3]);
  out->st = reinterpret_cast<float *>(b + off[4]);
  out->tc_b = reinterpret_cast<float *>(b + off[5]);
  out->order = reinterpret_cast<int32_t *>(b + off[6]);
  out->items = reinterpret_cast<int32_t *>(b + off[7]);
  out->tc_items = reinterpret_cast<int32_t *>(b + off[8]);
  return MOC_OK;
}

// Uploads every input and state array of `h` (validated) into the storage.
// With stream_tracks the per-track arrays go on the copy stream in chunks of
// whole 2D tracks (events chunk_ev[k]) and the call returns with the upload in
// flight; the next sweep starts on each chunk as it lands.
int upload_all(moc_problem *p, const moc_host *h, bool stream_tracks) {
  const moc_dims &d = p->d;
  const int64_t N2D = d.n_tracks_2d, P = d.n_polar, S = d.n_seg, G = d.n_groups;
  const int64_t NS = d.n_sources;
  if (stream_tracks) {
    // Fine source and flux (2 GB on the default problem) go first, so that the
    // host's validation and derivation below run while they are in flight; the
    // per-track arrays follow on the copy stream at the end.  The arrays copied
    // before the validation must at least exist.  The per-segment source ids
    // (2.6 GB) are not scanned on the host: the sweep reads every id through a
    // bounds check (MOC_DEV_ERR_SOURCE), so the upload returns in a few ms and
    // the first sweep starts as soon as the first chunk has landed.
    if (!h->fine_source || !h->seg_src) return MOC_ERR_ARG;
    TRY(put_rows(p, p->q, h->fine_source, p->nfsr));
    // The scalar flux goes to phi_in on the copy stream, after the chunks, and
    // phi starts at zero: the first range sweep waits for the fine source only
    // (1 GB, not 2).  Without room for phi_in it is copied into phi here.
    if (!p->phi_in && dalloc(p, &p->phi_in, p->nfsr * p->ldg) != MOC_OK) p->phi_in = nullptr;
    p->phi_fold_pending = false;
    if (p->phi_in)
      MOC_CUDA_TRY(cudaMemsetAsync(p->phi, 0, sizeof(float) * (size_t)(p->nfsr * p->ldg),
                                   p->stream));
    else
      TRY(put_rows(p, p->phi, h->fine_flux, p->nfsr));
    TRY(moc_host_validate_except_ids(&d, h));
  }
  Staging sg;
  TRY(staging(p, &sg));
  float max_step = 0.0f;
  TRY(moc_host_derive(&d, h, p->ldg, sg.seg_ds, sg.mu, sg.weight, sg.coef, sg.st, &max_step));
  // one wrap per segment keeps the height rule exact (checked, not assumed)
  const float hd = d.height / (float)d.decomp_ax;
  if (!(max_step < hd)) return MOC_ERR_ARG;
  // zi % F as zi - F * umulhi(zi, m): verified for every fine-interval index
  // the heights can reach (start heights and one wrap of [0, hd)).
  {
    float zmax = hd;
    const int64_t n3d = p->n3d;
#pragma omp parallel for schedule(static) reduction(max : zmax)
    for (int64_t t = 0; t < n3d; ++t) zmax = h->z0[t] > zmax ? h->z0[t] : zmax;
    const float dz = d.height / (float)(d.fai * d.decomp_ax * d.cai);
    const double lim = (double)zmax / (double)dz + 4.0;
    uint32_t m = (uint32_t)(0x100000000ull / (uint64_t)d.fai + 1ull);
    if (lim > (double)(1u << 24)) m = 0;
    for (uint32_t zi = 0; m && zi <= (uint32_t)lim; ++zi) {
      const uint32_t q = (uint32_t)(((uint64_t)zi * m) >> 32);
      if (zi - q * (uint32_t)d.fai != zi % (uint32_t)d.fai) m = 0;
    }
    p->fmagic = m;
  }
  TRY(put(p, p->seg_ds, sg.seg_ds, N2D * P * S));
  if (!stream_tracks) TRY(put(p, p->seg_src, h->seg_src, p->n3d * S));
  TRY(put(p, p->weight, sg.weight, p->n3d));
  TRY(put(p, p->z0, h->z0, p->n3d));
  TRY(put(p, p->mu, sg.mu, P));
  TRY(put(p, p->src_sigt, h->src_sigt, NS));
  TRY(put(p, p->src_xs, h->src_xs, NS));
  TRY(put(p, p->vol, h->vol, NS));
  TRY(put(p, p->coef, sg.coef, (int64_t)d.n_sigt * COEF_PLANES * p->ldg));
  TRY(put(p, p->xs, h->xs, (int64_t)d.n_xs * G * 3));
  TRY(put(p, p->scatter_t, sg.st, (int64_t)d.n_xs * G * G));
  TRY(put(p, p->table, h->table, 2 * (int64_t)d.table_n));
  // update_sources work list: sources grouped by xs row, items of <= 128 sources
  {
    std::vector<int64_t> start((size_t)d.n_xs + 1, 0);
    for (int64_t s = 0; s < NS; ++s) start[(size_t)h->src_xs[s] + 1]++;
    for (int32_t m = 0; m < d.n_xs; ++m) start[(size_t)m + 1] += start[(size_t)m];
    int32_t *order = sg.order, *items = sg.items;
    int64_t n_items = 0;
    std::vector<int64_t> fill(start.begin(), start.end() - 1);
    for (int64_t s = 0; s < NS; ++s) order[(size_t)fill[(size_t)h->src_xs[s]]++] = (int32_t)s;
    for (int32_t m = 0; m < d.n_xs; ++m)
      for (int64_t a = start[(size_t)m]; a < start[(size_t)m + 1]; a += 128) {
        const int64_t b = a + 128 < start[(size_t)m + 1] ? a + 128 : start[(size_t)m + 1];
        items[n_items++] = m;
        items[n_items++] = (int32_t)a;
        items[n_items++] = (int32_t)b;
      }
    p->n_upd_items = (int32_t)(n_items / 3);
    TRY(put(p, p->xs_order, order, NS));
    TRY(put(p, p->upd_items, items, n_items));
    // tensor-core tiles: <= 128 fine regions (128 / F sources) of one material,
    // and per material the split second operand (scatter rows, nuSigmaF, SigmaA)
    if (p->tc_b) {
      const int64_t per = 128 / d.fai;
      int32_t *tc_items = sg.tc_items;
      int64_t n_tc = 0;
      for (int32_t m = 0; m < d.n_xs; ++m)
        for (int64_t a = start[(size_t)m]; a < start[(size_t)m + 1]; a += per) {
          const int64_t b = a + per < start[(size_t)m + 1] ? a + per : start[(size_t)m + 1];
          tc_items[n_tc++] = m;
          tc_items[n_tc++] = (int32_t)a;
          tc_items[n_tc++] = (int32_t)b;
        }
      const int64_t plane = (int64_t)p->tc_np * p->tc_kp;
      build_tc_b(p, h->xs, h->scatter, sg.tc_b);
      p->n_tc_items = (int32_t)(n_tc / 3);
      TRY(put(p, p->tc_items, tc_items, n_tc));
      TRY(put(p, p->tc_b, sg.tc_b, d.n_xs * 2 * plane));
    }
    // the staged sources are reused by the next upload once these copies ran
    MOC_CUDA_TRY(cudaEventRecord(p->stage_ev, p->stream));
    p->stage_pending = true;
  }
  if (!stream_tracks) {
    TRY(put_rows(p, p->q, h->fine_source, p->nfsr));
    TRY(put_rows(p, p->phi, h->fine_flux, p->nfsr));
    TRY(put(p, p->seg_src, h->seg_src, p->n3d * S));
    TRY(put_rows(p, p->psi_f, h->psi_f, p->n3d));
    TRY(put_rows(p, p->psi_b, h->psi_b, p->n3d));
  } else {
    // the per-track arrays last, after everything queued on the stream: copies
    // on two streams share the copy engines, and the fine source, flux and
    // derived arrays above are what the first chunk's sweep waits for (this also
    // orders the chunks after any sweep still reading the arrays they overwrite)
    MOC_CUDA_TRY(cudaEventRecord(p->main_ev, p->stream));
    MOC_CUDA_TRY(cudaStreamWaitEvent(p->copy_stream, p->main_ev, 0));
    const int64_t PZ = P * d.z_stacked;
    int n = 0;
    int64_t len = N2D / 256 > 0 ? N2D / 256 : 1;
    for (int64_t i1 = 0; i1 < N2D; ++n, len *= 4) {
      const int64_t i0 = i1;
      i1 = (n == moc_problem::MAX_UPLOAD_CHUNKS - 1 || N2D - i0 <= len) ? N2D : i0 + len;
      const int64_t t0 = i0 * PZ, nt = (i1 - i0) * PZ;
      TRY(put(p, p->seg_src + t0 * S, h->seg_src + t0 * S, nt * S, p->copy_stream));
      TRY(put_rows(p, p->psi_f + t0 * p->ldg, h->psi_f ? h->psi_f + t0 * G : nullptr, nt,
                   p->copy_stream));
      MOC_CUDA_TRY(cudaEventRecord(p->chunk_ev[n], p->copy_stream));
      p->chunk_end[n] = i1;
    }
    if (p->phi_in) {
      TRY(put_rows(p, p->phi_in, h->fine_flux, p->nfsr, p->copy_stream));
      p->phi_fold_pending = true;
    }
    TRY(put_rows(p, p->psi_b, h->psi_b, p->n3d, p->copy_stream));
    MOC_CUDA_TRY(cudaEventRecord(p->copy_done, p->copy_stream));
    p->n_chunks = n;
  }
  if (p->phi_lo)
    MOC_CUDA_TRY(cudaMemsetAsync(p->phi_lo, 0, sizeof(float) * (size_t)(p->nfsr * p->ldg), p->stream));
  // fresh FP64 state follows the uploaded FP32 state
  if (p->q64) {
    widen_kernel<<<1024, 256, 0, p->stream>>>(p->q, p->q64, p->nfsr * p->ldg);
    widen_kernel<<<1024, 256, 0, p->stream>>>(p->phi, p->phi64, p->nfsr * p->ldg);
    widen_kernel<<<1024, 256, 0, p->stream>>>(p->psi_f, p->psi_f64, p->n3d * p->ldg);
    widen_kernel<<<1024, 256, 0, p->stream>>>(p->psi_b, p->psi_b64, p->n3d * p->ldg);
    p->launches += 4;
  }
  p->psi_pending = false;
  TRY(moc_reset_psi_scale(p));
  if (!h->psi_b) {
    // zeros by definition: no scan of the (cleared) array needed
    p->detect_pending = false;
    MOC_CUDA_TRY(cudaMemsetAsync(p->psi_b_nonzero, 0, sizeof(int32_t), p->stream));
  } else if (stream_tracks) {
    p->detect_pending = true;          // psi_b is still being copied
  } else {
    TRY(moc_detect_psi_b(p));
  }
  MOC_CUDA_TRY(cudaMemsetAsync(p->err, 0, sizeof(int32_t), p->stream));
  return MOC_OK;
}

void release(moc_problem *p) {
  moc_det_release(p);
  dfree(p->seg_ds); dfree(p->seg_src); dfree(p->weight); dfree(p->z0); dfree(p->mu);
  dfree(p->src_sigt); dfree(p->src_xs); dfree(p->vol); dfree(p->coef); dfree(p->xs);
  dfree(p->scatter_t); dfree(p->table); dfree(p->q); dfree(p->phi); dfree(p->phi_lo);
  dfree(p->phi_in);
  dfree(p->psi_f); dfree(p->psi_b); dfree(p->q64); dfree(p->phi64); dfree(p->psi_f64);
  dfree(p->psi_b64); dfree(p->partials); dfree(p->scalars); dfree(p->err);
  dfree(p->xs_order); dfree(p->upd_items); dfree(p->psi_scale); dfree(p->psi_b_nonzero);
  dfree(p->ck_psi); dfree(p->ck_z); dfree(p->adj_dphi); dfree(p->adj_dq); dfree(p->adj_dsig);
  dfree(p->tc_b); dfree(p->tc_items); dfree(p->adj_dfit);
  if (p->stage_ev) cudaEventSynchronize(p->stage_ev);
  if (p->h_stage) cudaFreeHost(p->h_stage);
  if (p->stage_ev) cudaEventDestroy(p->stage_ev);
  p->h_stage = nullptr;
  p->stage_ev = nullptr;
  if (p->ev0) cudaEventDestroy(p->ev0);
  if (p->ev1) cudaEventDestroy(p->ev1);
  if (p->copy_stream) cudaStreamSynchronize(p->copy_stream);
  for (cudaEvent_t &e : p->chunk_ev)
    if (e) cudaEventDestroy(e);
  if (p->main_ev) cudaEventDestroy(p->main_ev);
  if (p->copy_done) cudaEventDestroy(p->copy_done);
  if (p->copy_stream) cudaStreamDestroy(p->copy_stream);
  if (p->stream) cudaStreamDestroy(p->stream);
  p->ev0 = p->ev1 = p->main_ev = p->copy_done = nullptr;
  p->copy_stream = p->stream = nullptr;
  p->n_chunks = 0;
}

// Records a failure on the handle; later calls report MOC_ERR_STATE.
int fail(moc_problem *p, int rc) {
  if (rc != MOC_OK && p->status == MOC_OK) p->status = rc;
  return rc;
}

int usable(const moc_problem *p) {
  if (!p) return MOC_ERR_ARG;
  if (p->status != MOC_OK) return MOC_ERR_STATE;
  if (p->stale) return MOC_ERR_STATE;      // a rejected upload: upload again
  return MOC_OK;
}

// Entry-point guard: a usable handle whose stream has joined any upload in
// flight.
int ready(moc_problem *p) {
  int rc = usable(p);
  if (rc != MOC_OK) return rc;
  rc = moc_join_upload(p);
  return rc == MOC_OK ? MOC_OK : fail(p, rc);
}

}  // namespace

// Waits for the stream and folds the device error word into the status.
int moc_sync_check(moc_problem *p) {
  cudaError_t e = cudaStreamSynchronize(p->stream);
  if (e != cudaSuccess) return fail(p, MOC_ERR_CUDA);
  int32_t err = 0;
  e = cudaMemcpy(&err, p->err, sizeof(int32_t), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail(p, MOC_ERR_CUDA);
  if (err & MOC_DEV_ERR_TIMEOUT) return fail(p, MOC_ERR_TIMEOUT);
  if (err == MOC_DEV_ERR_SOURCE) {   // input of the last upload: refuse work until the next
    p->stale = true;
    return MOC_ERR_ARG;
  }
  if (err != 0) return fail(p, MOC_ERR_ARG);
  return MOC_OK;
}

namespace {

int sync_check(moc_problem *p) { return moc_sync_check(p); }

int read_scalars(moc_problem *p, double *out) {
  int rc = sync_check(p);
  if (rc != MOC_OK) return rc;
  if (cudaMemcpy(out, p->scalars, sizeof(double) * SC_COUNT, cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(p, MOC_ERR_CUDA);
  return MOC_OK;
}

int sweep_impl(moc_problem *p) {
  const bool had_pending = p->psi_pending && p->mode != MOC_MODE_FP64;
  int rc = MOC_OK;
  if (p->flags & MOC_FLAG_DETERMINISTIC) {
    // the uploaded flux lands first: the tallies are added on top of it in order
    rc = moc_join_upload(p);
    if (rc == MOC_OK) rc = moc_det_sweep(p);
  } else if (p->n_chunks > 0 && p->mode != MOC_MODE_FP64) {
    // sweep each chunk of 2D tracks once its copy has landed
    int64_t i0 = 0;
    for (int k = 0; k < p->n_chunks && rc == MOC_OK; ++k) {
      if (cudaStreamWaitEvent(p->stream, p->chunk_ev[k], 0) != cudaSuccess) return fail(p, MOC_ERR_CUDA);
      rc = moc_launch_sweep_range(p, i0, p->chunk_end[k]);
      i0 = p->chunk_end[k];
    }
    if (rc == MOC_OK) rc = moc_join_upload(p);
  } else {
    rc = moc_join_upload(p);
    if (rc == MOC_OK) rc = moc_launch_sweep(p);
  }
  if (rc != MOC_OK) return fail(p, rc);
  if (had_pending) {                   // the sweep applied it
    p->psi_pending = false;
    rc = moc_reset_psi_scale(p);
    if (rc != MOC_OK) return fail(p, rc);
  }
  if (p->mode == MOC_MODE_FP64) {
    rc = moc_round_state_fp32(p, true, true, false);
    if (rc != MOC_OK) return fail(p, rc);
  }
  if (p->mode == MOC_MODE_MIXED && (p->flags & MOC_FLAG_COMPENSATED) && p->phi_lo) {
    fold_kernel<<<1024, 256, 0, p->stream>>>(p->phi, p->phi_lo, p->nfsr * p->ldg);
    p->launches++;
    if (cudaGetLastError() != cudaSuccess) return fail(p, MOC_ERR_CUDA);
  }
  return MOC_OK;
}

}  // namespace

// A device wait that nothing completes: an mbarrier expecting one arrival
// that never comes, polled with the same clock-bounded loop as every device
// wait of the library; on expiry it sets the timeout bit and returns.
__global__ void selftest_wait_kernel(int32_t *err, long long cycles) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  const uint32_t addr = (uint32_t)__cvta_generic_to_shared(&bar);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(addr), "r"(1) : "memory");
  const long long t0 = clock64();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred P1;\n\tmbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, P1;\n\t}\n"
        : "=r"(done)
        : "r"(addr), "r"(0)
        : "memory");
    if (done) return;
    if (clock64() - t0 > cycles) {
      atomicOr(err, MOC_DEV_ERR_TIMEOUT);
      return;
    }
  }
}

int moc_join_upload(moc_problem *p) {
  if (p->n_chunks == 0) return MOC_OK;
  p->n_chunks = 0;
  MOC_CUDA_TRY(cudaStreamWaitEvent(p->stream, p->copy_done, 0));
  if (p->phi_fold_pending) {         // the uploaded scalar flux under the tallies
    p->phi_fold_pending = false;
    add_kernel<<<1024, 256, 0, p->stream>>>(p->phi, p->phi_in, p->nfsr * p->ldg);
    MOC_CUDA_TRY(cudaGetLastError());
    p->launches++;
  }
  if (p->detect_pending) {
    p->detect_pending = false;
    return moc_detect_psi_b(p);
  }
  return MOC_OK;
}

extern "C" {

int moc_selftest_wait(moc_problem *p, int64_t cycles) {
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  if (cycles < 1 || cycles > (int64_t)1 << 32) return MOC_ERR_ARG;   // at most ~2 s
  cudaSetDevice(p->device);
  selftest_wait_kernel<<<1, 32, 0, p->stream>>>(p->err, (long long)cycles);
  if (cudaGetLastError() != cudaSuccess) return fail(p, MOC_ERR_CUDA);
  p->launches++;
  return sync_check(p);
}

int moc_set_memory_limit(int64_t bytes) {
  if (bytes < 0) return MOC_ERR_ARG;
  g_memory_limit.store(bytes);
  return MOC_OK;
}

int moc_inject_fault(moc_problem *p, int kind) {
  if (!p) return MOC_ERR_ARG;
  cudaSetDevice(p->device);
  switch (kind) {
    case MOC_FAULT_CUDA:                  // as if a CUDA call of the handle had failed
      fail(p, MOC_ERR_CUDA);
      return MOC_OK;
    case MOC_FAULT_DEVICE_INPUT:          // a kernel found an invalid source id
    case MOC_FAULT_DEVICE_TIMEOUT: {      // a bounded device wait ran out
      const int32_t bit = kind == MOC_FAULT_DEVICE_INPUT ? 1 : 2;
      MOC_CUDA_TRY(cudaMemcpyAsync(p->err, &bit, sizeof bit, cudaMemcpyHostToDevice, p->stream));
      MOC_CUDA_TRY(cudaStreamSynchronize(p->stream));
      return MOC_OK;
    }
    default:
      return MOC_ERR_ARG;
  }
}

const char *moc_status_string(int status) {
  switch (status) {
    case MOC_OK: return "ok";
    case MOC_ERR_ARG: return "invalid argument";
    case MOC_ERR_CUDA: return "CUDA runtime error";
    case MOC_ERR_OOM: return "device out of memory";
    case MOC_ERR_STATE: return "handle unusable after an earlier error";
    case MOC_ERR_TIMEOUT: return "bounded device wait gave up";
    case MOC_ERR_UNSUPPORTED: return "unsupported mode or size";
    case MOC_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
  }
}

int moc_create(const moc_dims *dims, const moc_host *host, int device, moc_problem **out) {
  if (!dims || !host || !out) return MOC_ERR_ARG;
  *out = nullptr;
  int rc = moc_host_validate(dims, host);
  if (rc != MOC_OK) return rc;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return MOC_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= ndev) return MOC_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return MOC_ERR_CUDA;
  moc_problem *p = new (std::nothrow) moc_problem();
  if (!p) return MOC_ERR_OOM;
  p->d = *dims;
  p->device = device;
  p->ldg = (dims->n_groups + 3) / 4 * 4;
  p->n3d = dims->n_tracks_2d * dims->n_polar * dims->z_stacked;
  p->nfsr = dims->n_sources * dims->fai;
  const int64_t N2D = dims->n_tracks_2d, P = dims->n_polar, S = dims->n_seg;
  const int64_t G = dims->n_groups, NS = dims->n_sources;
  rc = MOC_OK;
  bool ev_ok = true;
  for (cudaEvent_t &e : p->chunk_ev)
    ev_ok = ev_ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
  if (!ev_ok || cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&p->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&p->main_ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&p->copy_done, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreate(&p->ev0) != cudaSuccess || cudaEventCreate(&p->ev1) != cudaSuccess)
    rc = MOC_ERR_CUDA;
  if (rc == MOC_OK) rc = dalloc(p, &p->seg_ds, N2D * P * S);
  if (rc == MOC_OK) rc = dalloc(p, &p->seg_src, p->n3d * S);
  if (rc == MOC_OK) rc = dalloc(p, &p->weight, p->n3d);
  if (rc == MOC_OK) rc = dalloc(p, &p->z0, p->n3d);
  if (rc == MOC_OK) rc = dalloc(p, &p->mu, P);
  if (rc == MOC_OK) rc = dalloc(p, &p->src_sigt, NS);
  if (rc == MOC_OK) rc = dalloc(p, &p->src_xs, NS);
  if (rc == MOC_OK) rc = dalloc(p, &p->vol, NS);
  if (rc == MOC_OK) rc = dalloc(p, &p->coef, (int64_t)dims->n_sigt * COEF_PLANES * p->ldg);
  if (rc == MOC_OK) rc = dalloc(p, &p->xs, (int64_t)dims->n_xs * G * 3);
  if (rc == MOC_OK) rc = dalloc(p, &p->scatter_t, (int64_t)dims->n_xs * G * G);
  if (rc == MOC_OK) rc = dalloc(p, &p->table, 2 * (int64_t)dims->table_n);
  if (rc == MOC_OK) rc = dalloc(p, &p->xs_order, NS);
  if (rc == MOC_OK) rc = dalloc(p, &p->psi_scale, 1);
  if (rc == MOC_OK) rc = dalloc(p, &p->psi_b_nonzero, 1);
  if (rc == MOC_OK) rc = dalloc(p, &p->upd_items, 3 * ((int64_t)dims->n_xs + NS / 128 + 1));
  if (rc == MOC_OK && moc_tc_dims(dims->n_groups, dims->fai, &p->tc_kp, &p->tc_np)) {
    const int64_t per = 128 / dims->fai;
    rc = dalloc(p, &p->tc_items, 3 * ((int64_t)dims->n_xs + NS / per + 1));
    if (rc == MOC_OK) rc = dalloc(p, &p->tc_b, (int64_t)dims->n_xs * 2 * p->tc_np * p->tc_kp);
  }
  if (rc == MOC_OK) rc = dalloc(p, &p->q, p->nfsr * p->ldg);
  if (rc == MOC_OK) rc = dalloc(p, &p->phi, p->nfsr * p->ldg);
  if (rc == MOC_OK) rc = dalloc(p, &p->psi_f, p->n3d * p->ldg);
  if (rc == MOC_OK) rc = dalloc(p, &p->psi_b, p->n3d * p->ldg);
  if (rc == MOC_OK) rc = dalloc(p, &p->partials, 3 * (int64_t)moc_post_scratch_blocks() + NS);
  if (rc == MOC_OK) rc = dalloc(p, &p->scalars, (int64_t)SC_COUNT);
  if (rc == MOC_OK) rc = dalloc(p, &p->err, 1);
  if (rc == MOC_OK) {
    double init[SC_COUNT] = {0};
    init[SC_KEFF_IN] = 1.0;
    init[SC_KEFF] = 1.0;
    if (cudaMemcpy(p->scalars, init, sizeof init, cudaMemcpyHostToDevice) != cudaSuccess)
      rc = MOC_ERR_CUDA;
  }
  if (rc == MOC_OK) rc = upload_all(p, host, false);
  if (rc == MOC_OK && cudaStreamSynchronize(p->stream) != cudaSuccess) rc = MOC_ERR_CUDA;
  if (rc != MOC_OK) {
    release(p);
    delete p;
    return rc;
  }
  *out = p;
  return MOC_OK;
}

int moc_destroy(moc_problem *p) {
  if (!p) return MOC_ERR_ARG;
  cudaSetDevice(p->device);
  if (p->copy_stream) cudaStreamSynchronize(p->copy_stream);
  if (p->stream) cudaStreamSynchronize(p->stream);
  release(p);
  delete p;
  return MOC_OK;
}

int moc_upload(moc_problem *p, const moc_host *host) {
  MOC_NVTX_RANGE("moc_upload");
  if (!p) return MOC_ERR_ARG;
  if (p->status != MOC_OK) return MOC_ERR_STATE;
  if (!host) return MOC_ERR_ARG;
  cudaSetDevice(p->device);
  int rc = moc_join_upload(p);
  if (rc != MOC_OK) return fail(p, rc);
  // FP64 state is widened from the uploaded FP32 state at once: no streaming.
  // Streamed uploads validate all but the per-segment source ids while their
  // copies are in flight; the sweep checks the ids (MOC_DEV_ERR_SOURCE).
  const bool streamed = p->q64 == nullptr;
  if (!streamed) {
    rc = moc_host_validate(&p->d, host);
    if (rc != MOC_OK) return rc;
  }
  p->uploads++;
  rc = upload_all(p, host, streamed);
  if (rc == MOC_OK) {
    p->stale = false;
    return MOC_OK;
  }
  // a rejected input after copies were issued: let them finish (the caller
  // may free its buffers) and refuse work until a valid upload
  cudaStreamSynchronize(p->copy_stream);
  cudaStreamSynchronize(p->stream);
  p->n_chunks = 0;
  p->detect_pending = false;
  p->phi_fold_pending = false;
  p->stale = true;
  return rc == MOC_ERR_ARG ? rc : fail(p, rc);
}

int moc_download(moc_problem *p, float *fine_flux, float *fine_source, float *psi_f, float *psi_b) {
  MOC_NVTX_RANGE("moc_download");
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  if (psi_f && p->psi_pending) {
    rc = moc_psi_materialize(p);
    if (rc != MOC_OK) return fail(p, rc);
  }
  rc = sync_check(p);
  if (rc != MOC_OK) return rc;
  if (fine_flux) rc = get_rows(p, fine_flux, p->phi, p->nfsr);
  if (rc == MOC_OK && fine_source) rc = get_rows(p, fine_source, p->q, p->nfsr);
  if (rc == MOC_OK && psi_f) rc = get_rows(p, psi_f, p->psi_f, p->n3d);
  if (rc == MOC_OK && psi_b) rc = get_rows(p, psi_b, p->psi_b, p->n3d);
  if (rc != MOC_OK) return fail(p, rc);
  return sync_check(p);
}

int moc_download64(moc_problem *p, double *fine_flux, double *fine_source, double *psi_f,
                   double *psi_b) {
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  if (!p->q64) return MOC_ERR_STATE;
  rc = sync_check(p);
  if (rc != MOC_OK) return rc;
  if (fine_flux) rc = get_rows(p, fine_flux, p->phi64, p->nfsr);
  if (rc == MOC_OK && fine_source) rc = get_rows(p, fine_source, p->q64, p->nfsr);
  if (rc == MOC_OK && psi_f) rc = get_rows(p, psi_f, p->psi_f64, p->n3d);
  if (rc == MOC_OK && psi_b) rc = get_rows(p, psi_b, p->psi_b64, p->n3d);
  if (rc != MOC_OK) return fail(p, rc);
  return sync_check(p);
}

int moc_status(const moc_problem *p) { return p ? p->status : MOC_ERR_ARG; }

int64_t moc_device_bytes(const moc_problem *p) { return p ? p->bytes : 0; }

int64_t moc_launch_count(const moc_problem *p) { return p ? p->launches : 0; }

int moc_set_mode(moc_problem *p, int mode, int flags) {
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  if (mode != MOC_MODE_PLAIN && mode != MOC_MODE_MIXED && mode != MOC_MODE_FP64) return MOC_ERR_ARG;
  if (flags & ~(MOC_FLAG_COMPENSATED | MOC_FLAG_SIMT_UPDATE | MOC_FLAG_DETERMINISTIC |
                MOC_FLAG_FP32_STATE))
    return MOC_ERR_ARG;
  if ((flags & MOC_FLAG_FP32_STATE) && mode != MOC_MODE_FP64) return MOC_ERR_UNSUPPORTED;
  if ((flags & MOC_FLAG_DETERMINISTIC) &&
      (mode == MOC_MODE_FP64 || (flags & MOC_FLAG_COMPENSATED) || p->ldg > 256))
    return MOC_ERR_UNSUPPORTED;
  if (p->psi_pending) {
    rc = moc_psi_materialize(p);
    if (rc != MOC_OK) return fail(p, rc);
  }
  if (mode == MOC_MODE_FP64 && !p->q64) {
    // the FP64 state starts from the current FP32 state
    rc = dalloc(p, &p->q64, p->nfsr * p->ldg);
    if (rc == MOC_OK) rc = dalloc(p, &p->phi64, p->nfsr * p->ldg);
    if (rc == MOC_OK) rc = dalloc(p, &p->psi_f64, p->n3d * p->ldg);
    if (rc == MOC_OK) rc = dalloc(p, &p->psi_b64, p->n3d * p->ldg);
    if (rc != MOC_OK) {
      dfree(p->q64); dfree(p->phi64); dfree(p->psi_f64); dfree(p->psi_b64);
      return rc;
    }
    widen_kernel<<<1024, 256, 0, p->stream>>>(p->q, p->q64, p->nfsr * p->ldg);
    widen_kernel<<<1024, 256, 0, p->stream>>>(p->phi, p->phi64, p->nfsr * p->ldg);
    widen_kernel<<<1024, 256, 0, p->stream>>>(p->psi_f, p->psi_f64, p->n3d * p->ldg);
    widen_kernel<<<1024, 256, 0, p->stream>>>(p->psi_b, p->psi_b64, p->n3d * p->ldg);
    p->launches += 4;
    if (cudaGetLastError() != cudaSuccess) return fail(p, MOC_ERR_CUDA);
  }
  if (mode == MOC_MODE_MIXED && (flags & MOC_FLAG_COMPENSATED) && !p->phi_lo) {
    rc = dalloc(p, &p->phi_lo, p->nfsr * p->ldg);
    if (rc != MOC_OK) return rc;
    if (cudaMemsetAsync(p->phi_lo, 0, sizeof(float) * (size_t)(p->nfsr * p->ldg), p->stream) !=
        cudaSuccess)
      return fail(p, MOC_ERR_CUDA);
  }
  p->mode = mode;
  p->flags = flags;
  return MOC_OK;
}

int moc_set_launch(moc_problem *p, int threads_per_track, int chunks_per_thread) {
  if (!p) return MOC_ERR_ARG;
  if (threads_per_track == 0 && chunks_per_thread == 0) {
    p->tpw = p->cpl = 0;
    return MOC_OK;
  }
  static const int ok[][2] = {{32, 1}, {32, 2}, {32, 4}, {16, 1}, {16, 2}, {8, 1}, {8, 4}, {4, 2},
                              {10, 5}, {10, 1}};
  for (auto &s : ok) {
    if (s[0] == threads_per_track && s[1] == chunks_per_thread) {
      if (moc_shape_groups(threads_per_track, chunks_per_thread) < p->ldg) return MOC_ERR_ARG;
      p->tpw = threads_per_track;
      p->cpl = chunks_per_thread;
      return MOC_OK;
    }
  }
  return MOC_ERR_UNSUPPORTED;
}

int moc_set_pipeline(moc_problem *p, int stages) {
  if (!p) return MOC_ERR_ARG;
  if (stages != -1 && stages != 0 && stages != 4) return MOC_ERR_UNSUPPORTED;
  p->stages = stages;
  return MOC_OK;
}

int moc_get_pipeline(const moc_problem *p, int *stages) {
  if (!p || !stages) return MOC_ERR_ARG;
  *stages = p->stages > 0 ? p->stages : 0;
  return MOC_OK;
}

int moc_set_adjoint_width(moc_problem *p, int lanes_per_track, int chunks_per_lane) {
  if (!p) return MOC_ERR_ARG;
  if (lanes_per_track == 0 && chunks_per_lane == 0) {
    p->adj_tpw = p->adj_cpl = 0;
    return MOC_OK;
  }
  if (lanes_per_track < 1 || lanes_per_track > 32 || chunks_per_lane < 1 || chunks_per_lane > 2)
    return MOC_ERR_UNSUPPORTED;
  if ((int64_t)lanes_per_track * chunks_per_lane * 4 < p->ldg) return MOC_ERR_ARG;
  p->adj_tpw = lanes_per_track;
  p->adj_cpl = chunks_per_lane;
  return MOC_OK;
}

int moc_get_launch(const moc_problem *p, int *threads_per_track, int *chunks_per_thread) {
  if (!p || !threads_per_track || !chunks_per_thread) return MOC_ERR_ARG;
  return moc_sweep_launch_shape(p, threads_per_track, chunks_per_thread);
}

int moc_autotune(moc_problem *p, int64_t n_tracks, int *threads_per_track,
                 int *chunks_per_thread, double *ms_best) {
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  cudaSetDevice(p->device);
  int tpw = 0, cpl = 0, stages = 0;
  rc = moc_sweep_autotune(p, n_tracks, &tpw, &cpl, &stages, ms_best);
  if (rc != MOC_OK) return rc;
  p->tpw = tpw;
  p->cpl = cpl;
  p->stages = stages;
  if (threads_per_track) *threads_per_track = tpw;
  if (chunks_per_thread) *chunks_per_thread = cpl;
  return MOC_OK;
}

int moc_transport_sweep(moc_problem *p, int64_t *segments_processed) {
  MOC_NVTX_RANGE("transport_sweep");
  int rc = usable(p);
  if (rc != MOC_OK) return rc;
  cudaSetDevice(p->device);
  rc = sweep_impl(p);
  if (rc != MOC_OK) return rc;
  if (segments_processed) *segments_processed = p->n3d * p->d.n_seg;   // src/solver.c:549
  return MOC_OK;
}

int moc_renormalize_flux(moc_problem *p) {
  MOC_NVTX_RANGE("renormalize_flux");
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  cudaSetDevice(p->device);
  rc = moc_launch_renormalize(p);
  return rc == MOC_OK ? MOC_OK : fail(p, rc);
}

int moc_update_sources(moc_problem *p, double keff, double *residual) {
  MOC_NVTX_RANGE("update_sources");
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  if (!(keff != 0.0)) return MOC_ERR_ARG;
  cudaSetDevice(p->device);
  rc = moc_launch_update(p, keff, false, false);
  if (rc != MOC_OK) return fail(p, rc);
  if (residual) {
    double sc[SC_COUNT];
    rc = read_scalars(p, sc);
    if (rc != MOC_OK) return rc;
    *residual = sc[SC_RESIDUAL];
  }
  return MOC_OK;
}

int moc_compute_keff(moc_problem *p, double leakage, double *keff) {
  MOC_NVTX_RANGE("compute_keff");
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  cudaSetDevice(p->device);
  rc = moc_launch_keff(p, leakage);
  if (rc != MOC_OK) return fail(p, rc);
  double sc[SC_COUNT];
  rc = read_scalars(p, sc);
  if (rc != MOC_OK) return rc;
  if (keff) *keff = sc[SC_KEFF];
  return MOC_OK;
}

int moc_power_iteration(moc_problem *p, double keff_in, double *keff_out, double *residual) {
  MOC_NVTX_RANGE("power_iteration");
  int rc = usable(p);
  if (rc != MOC_OK) return rc;
  if (!(keff_in != 0.0)) return MOC_ERR_ARG;
  cudaSetDevice(p->device);
  rc = sweep_impl(p);
  if (rc != MOC_OK) return rc;
  rc = moc_launch_renormalize(p);
  if (rc != MOC_OK) return fail(p, rc);
  rc = moc_launch_update(p, keff_in, false, true);
  if (rc != MOC_OK) return fail(p, rc);
  if (keff_out || residual) {
    double sc[SC_COUNT];
    rc = read_scalars(p, sc);
    if (rc != MOC_OK) return rc;
    if (keff_out) *keff_out = sc[SC_KEFF];
    if (residual) *residual = sc[SC_RESIDUAL];
  }
  return MOC_OK;
}

int moc_synchronize(moc_problem *p) {
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  return sync_check(p);
}

int moc_time_sweep(moc_problem *p, int iters, double *ms_per_sweep) {
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  if (iters < 1 || !ms_per_sweep) return MOC_ERR_ARG;
  cudaSetDevice(p->device);
  double total = 0.0;
  for (int i = 0; i < iters; ++i) {
    const bool had_pending = p->psi_pending && p->mode != MOC_MODE_FP64;
    if (cudaEventRecord(p->ev0, p->stream) != cudaSuccess) return fail(p, MOC_ERR_CUDA);
    rc = moc_launch_sweep(p);
    if (rc != MOC_OK) return fail(p, rc);
    if (cudaEventRecord(p->ev1, p->stream) != cudaSuccess) return fail(p, MOC_ERR_CUDA);
    if (had_pending) {                 // the sweep applied the pending factor
      p->psi_pending = false;
      rc = moc_reset_psi_scale(p);
      if (rc != MOC_OK) return fail(p, rc);
    }
    if (cudaEventSynchronize(p->ev1) != cudaSuccess) return fail(p, MOC_ERR_CUDA);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p->ev0, p->ev1);
    total += ms;
  }
  *ms_per_sweep = total / iters;
  return sync_check(p);
}

int moc_time_power_iterations(moc_problem *p, int iters, double *ms_total, double *ms_sweeps,
                              double *keff, double *residual) {
  MOC_NVTX_RANGE("moc_time_power_iterations");
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  if (iters < 1) return MOC_ERR_ARG;
  cudaSetDevice(p->device);
  std::vector<cudaEvent_t> ev((size_t)(2 * iters + 2), nullptr);
  for (auto &e : ev)
    if (cudaEventCreate(&e) != cudaSuccess) {
      for (auto &x : ev)
        if (x) cudaEventDestroy(x);
      return fail(p, MOC_ERR_CUDA);
    }
  rc = MOC_OK;
  cudaEventRecord(ev[0], p->stream);
  for (int i = 0; i < iters && rc == MOC_OK; ++i) {
    cudaEventRecord(ev[2 + 2 * i], p->stream);
    rc = sweep_impl(p);
    cudaEventRecord(ev[3 + 2 * i], p->stream);
    if (rc == MOC_OK) rc = moc_launch_renormalize(p);
    if (rc == MOC_OK) rc = moc_launch_update(p, 0.0, true, true);
  }
  cudaEventRecord(ev[1], p->stream);
  if (rc == MOC_OK && cudaEventSynchronize(ev[1]) != cudaSuccess) rc = MOC_ERR_CUDA;
  double sweeps = 0.0;
  float tot = 0.f;
  if (rc == MOC_OK) {
    cudaEventElapsedTime(&tot, ev[0], ev[1]);
    for (int i = 0; i < iters; ++i) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev[2 + 2 * i], ev[3 + 2 * i]);
      sweeps += ms;
    }
  }
  for (auto &e : ev) cudaEventDestroy(e);
  if (rc != MOC_OK) return fail(p, rc);
  if (ms_total) *ms_total = tot;
  if (ms_sweeps) *ms_sweeps = sweeps;
  double sc[SC_COUNT];
  rc = read_scalars(p, sc);
  if (rc != MOC_OK) return rc;
  if (keff) *keff = sc[SC_KEFF];
  if (residual) *residual = sc[SC_RESIDUAL];
  return MOC_OK;
}

int moc_time_phases(moc_problem *p, int iters, double *phase_ms, double *keff,
                    double *residual) {
  MOC_NVTX_RANGE("moc_time_phases");
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  if (iters < 1 || !phase_ms) return MOC_ERR_ARG;
  cudaSetDevice(p->device);
  // per iteration: start, after the sweep, after renormalize, after update, after keff
  constexpr int EV = 5;
  std::vector<cudaEvent_t> ev((size_t)(EV * iters), nullptr);
  for (auto &e : ev)
    if (cudaEventCreate(&e) != cudaSuccess) {
      for (auto &x : ev)
        if (x) cudaEventDestroy(x);
      return fail(p, MOC_ERR_CUDA);
    }
  for (int i = 0; i < iters && rc == MOC_OK; ++i) {
    cudaEvent_t *e = ev.data() + (size_t)EV * i;
    cudaEventRecord(e[0], p->stream);
    rc = sweep_impl(p);
    cudaEventRecord(e[1], p->stream);
    if (rc == MOC_OK) rc = moc_launch_renormalize(p);
    cudaEventRecord(e[2], p->stream);
    // the reference's two calls, k_eff chained on the device (src/main.c:81,87)
    if (rc == MOC_OK) rc = moc_launch_update(p, 0.0, true, false);
    cudaEventRecord(e[3], p->stream);
    if (rc == MOC_OK) rc = moc_launch_keff(p, 0.0);
    cudaEventRecord(e[4], p->stream);
  }
  if (rc == MOC_OK && cudaEventSynchronize(ev.back()) != cudaSuccess) rc = MOC_ERR_CUDA;
  double acc[MOC_N_PHASES] = {0.0, 0.0, 0.0, 0.0, 0.0};
  if (rc == MOC_OK) {
    for (int i = 0; i < iters; ++i) {
      const cudaEvent_t *e = ev.data() + (size_t)EV * i;
      const int slot[4] = {MOC_PHASE_SWEEP, MOC_PHASE_RENORMALIZE, MOC_PHASE_UPDATE,
                           MOC_PHASE_KEFF};
      for (int k = 0; k < 4; ++k) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e[k], e[k + 1]);
        acc[slot[k]] += ms;
      }
    }
  }
  for (auto &e : ev) cudaEventDestroy(e);
  if (rc != MOC_OK) return fail(p, rc);
  for (int k = 0; k < MOC_N_PHASES; ++k) phase_ms[k] = acc[k];   // no exchange on one device
  double sc[SC_COUNT];
  rc = read_scalars(p, sc);
  if (rc != MOC_OK) return rc;
  if (keff) *keff = sc[SC_KEFF];
  if (residual) *residual = sc[SC_RESIDUAL];
  return MOC_OK;
}

}  // extern "C"

// ---- state access on device pointers (the torch binding) -----------------
namespace {
template <typename T>
int copy_rows_dd(moc_problem *p, T *dst, int64_t dpitch, const T *src, int64_t spitch,
                 int64_t rows, int64_t width) {
  MOC_CUDA_TRY(cudaMemcpy2DAsync(dst, sizeof(T) * dpitch, src, sizeof(T) * spitch,
                                 sizeof(T) * width, (size_t)rows, cudaMemcpyDeviceToDevice,
                                 p->stream));
  return MOC_OK;
}
}  // namespace

extern "C" {

int moc_set_fine_source_device(moc_problem *p, const float *q) {
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  if (!q) return MOC_ERR_ARG;
  cudaSetDevice(p->device);
  const int64_t G = p->d.n_groups;
  rc = copy_rows_dd(p, p->q, p->ldg, q, G, p->nfsr, G);
  if (rc == MOC_OK && p->q64) {
    widen_kernel<<<1024, 256, 0, p->stream>>>(p->q, p->q64, p->nfsr * p->ldg);
    p->launches++;
  }
  return rc == MOC_OK ? MOC_OK : fail(p, rc);
}

int moc_set_fine_source64_device(moc_problem *p, const double *q) {
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  if (!q || !p->q64) return !q ? MOC_ERR_ARG : MOC_ERR_STATE;
  cudaSetDevice(p->device);
  rc = copy_rows_dd(p, p->q64, p->ldg, q, (int64_t)p->d.n_groups, p->nfsr, p->d.n_groups);
  return rc == MOC_OK ? MOC_OK : fail(p, rc);
}

int moc_set_sigma_t(moc_problem *p, const float *sigt) {
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  if (!sigt) return MOC_ERR_ARG;
  for (int64_t k = 0; k < (int64_t)p->d.n_sigt * p->d.n_groups; ++k)
    if (!(sigt[k] > 0.0f) || isinf(sigt[k])) return MOC_ERR_ARG;
  cudaSetDevice(p->device);
  std::vector<float> coef((size_t)p->d.n_sigt * COEF_PLANES * p->ldg);
  moc_host_coef(&p->d, sigt, p->ldg, coef.data());
  rc = put(p, p->coef, coef.data(), (int64_t)coef.size());
  if (rc == MOC_OK && cudaStreamSynchronize(p->stream) != cudaSuccess) rc = MOC_ERR_CUDA;
  return rc == MOC_OK ? MOC_OK : fail(p, rc);
}

int moc_set_cross_sections(moc_problem *p, const float *xs, const float *scatter) {
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  if (!xs || !scatter) return MOC_ERR_ARG;
  const moc_dims &d = p->d;
  const int64_t G = d.n_groups, nx = d.n_xs;
  for (int64_t k = 0; k < nx * G * 3; ++k)
    if (!std::isfinite(xs[k])) return MOC_ERR_ARG;
  for (int64_t k = 0; k < nx * G * G; ++k)
    if (!std::isfinite(scatter[k])) return MOC_ERR_ARG;
  cudaSetDevice(p->device);
  // the update kernel reads the scatter matrix transposed: St[m][from][to]
  std::vector<float> st((size_t)(nx * G * G));
  for (int64_t m = 0; m < nx; ++m)
    for (int64_t g = 0; g < G; ++g)
      for (int64_t h = 0; h < G; ++h) st[(size_t)((m * G + h) * G + g)] = scatter[(m * G + g) * G + h];
  rc = put(p, p->xs, xs, nx * G * 3);
  if (rc == MOC_OK) rc = put(p, p->scatter_t, st.data(), nx * G * G);
  std::vector<float> tcb;
  if (rc == MOC_OK && p->tc_b) {
    tcb.resize((size_t)(nx * 2 * p->tc_np * p->tc_kp));
    build_tc_b(p, xs, scatter, tcb.data());
    rc = put(p, p->tc_b, tcb.data(), (int64_t)tcb.size());
  }
  if (rc == MOC_OK && cudaStreamSynchronize(p->stream) != cudaSuccess) rc = MOC_ERR_CUDA;
  return rc == MOC_OK ? MOC_OK : fail(p, rc);
}

int moc_set_fine_flux_device(moc_problem *p, const float *phi) {
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  if (!phi) return MOC_ERR_ARG;
  cudaSetDevice(p->device);
  const int64_t G = p->d.n_groups;
  rc = copy_rows_dd(p, p->phi, p->ldg, phi, G, p->nfsr, G);
  if (rc == MOC_OK && p->phi_lo)
    rc = cudaMemsetAsync(p->phi_lo, 0, sizeof(float) * (size_t)(p->nfsr * p->ldg), p->stream) ==
                 cudaSuccess ? MOC_OK : MOC_ERR_CUDA;
  if (rc == MOC_OK && p->phi64) {
    widen_kernel<<<1024, 256, 0, p->stream>>>(p->phi, p->phi64, p->nfsr * p->ldg);
    p->launches++;
  }
  return rc == MOC_OK ? MOC_OK : fail(p, rc);
}

int moc_get_fine_source_device(moc_problem *p, float *q) {
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  if (!q) return MOC_ERR_ARG;
  cudaSetDevice(p->device);
  rc = copy_rows_dd(p, q, (int64_t)p->d.n_groups, p->q, p->ldg, p->nfsr, p->d.n_groups);
  return rc == MOC_OK ? MOC_OK : fail(p, rc);
}

int moc_update_sources_adjoint(moc_problem *p, const float *phi0, const float *dq, double keff,
                               double *dscatter, double *dnusf, float *dphi0) {
  MOC_NVTX_RANGE("update_sources_adjoint");
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  if (!phi0 || !dq || !(keff != 0.0)) return MOC_ERR_ARG;
  if (p->d.n_groups > 256) return MOC_ERR_UNSUPPORTED;
  cudaSetDevice(p->device);
  rc = moc_launch_update_adjoint(p, phi0, dq, keff, dscatter, dnusf, dphi0);
  return rc == MOC_OK ? MOC_OK : fail(p, rc);
}

int moc_zero_state(moc_problem *p, int flux, int psi) {
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  cudaSetDevice(p->device);
  const size_t fb = sizeof(float) * (size_t)(p->nfsr * p->ldg);
  const size_t pb = sizeof(float) * (size_t)(p->n3d * p->ldg);
  if (flux) {
    MOC_CUDA_TRY(cudaMemsetAsync(p->phi, 0, fb, p->stream));
    if (p->phi_lo) MOC_CUDA_TRY(cudaMemsetAsync(p->phi_lo, 0, fb, p->stream));
    if (p->phi64) MOC_CUDA_TRY(cudaMemsetAsync(p->phi64, 0, 2 * fb, p->stream));
  }
  if (psi) {
    MOC_CUDA_TRY(cudaMemsetAsync(p->psi_f, 0, pb, p->stream));
    MOC_CUDA_TRY(cudaMemsetAsync(p->psi_b, 0, pb, p->stream));
    if (p->psi_f64) MOC_CUDA_TRY(cudaMemsetAsync(p->psi_f64, 0, 2 * pb, p->stream));
    if (p->psi_b64) MOC_CUDA_TRY(cudaMemsetAsync(p->psi_b64, 0, 2 * pb, p->stream));
    if (p->psi_pending) {
      p->psi_pending = false;
      rc = moc_reset_psi_scale(p);
      if (rc != MOC_OK) return fail(p, rc);
    }
    rc = moc_detect_psi_b(p);
    if (rc != MOC_OK) return fail(p, rc);
  }
  return MOC_OK;
}

int moc_get_fine_flux_device(moc_problem *p, float *phi) {
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  if (!phi) return MOC_ERR_ARG;
  cudaSetDevice(p->device);
  rc = copy_rows_dd(p, phi, (int64_t)p->d.n_groups, p->phi, p->ldg, p->nfsr, p->d.n_groups);
  return rc == MOC_OK ? MOC_OK : fail(p, rc);
}

int moc_get_fine_flux64_device(moc_problem *p, double *phi) {
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  if (!phi || !p->phi64) return !phi ? MOC_ERR_ARG : MOC_ERR_STATE;
  cudaSetDevice(p->device);
  rc = copy_rows_dd(p, phi, (int64_t)p->d.n_groups, p->phi64, p->ldg, p->nfsr, p->d.n_groups);
  return rc == MOC_OK ? MOC_OK : fail(p, rc);
}

int moc_fine_flux_storage(moc_problem *p, void **ptr, int64_t *n_elems, int32_t *ldg,
                          int32_t *elem_bytes) {
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  if (!ptr) return MOC_ERR_ARG;
  const bool fp64 = p->mode == MOC_MODE_FP64;
  if (fp64 && !p->phi64) return MOC_ERR_STATE;
  *ptr = fp64 ? static_cast<void *>(p->phi64) : static_cast<void *>(p->phi);
  if (n_elems) *n_elems = p->nfsr * p->ldg;
  if (ldg) *ldg = p->ldg;
  if (elem_bytes) *elem_bytes = fp64 ? 8 : 4;
  return MOC_OK;
}

// ---- adjoint ---------------------------------------------------------------

int moc_adjoint_forward(moc_problem *p, int k_ckpt) {
  MOC_NVTX_RANGE("moc_adjoint_forward");
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  if (k_ckpt < 1 || k_ckpt > 8) return MOC_ERR_ARG;
  if (p->d.n_groups > 256) return MOC_ERR_UNSUPPORTED;
  cudaSetDevice(p->device);
  const int nck = (p->d.n_seg + k_ckpt - 1) / k_ckpt;
  if (!p->ck_psi || p->ck_n != nck) {
    dfree(p->ck_psi);
    dfree(p->ck_z);
    rc = dalloc(p, &p->ck_psi, p->n3d * nck * p->ldg);
    if (rc == MOC_OK) rc = dalloc(p, &p->ck_z, p->n3d * nck);
    if (rc != MOC_OK) return rc;
  }
  p->ck_k = k_ckpt;
  p->ck_n = nck;
  const bool had_pending = p->psi_pending;
  rc = moc_launch_sweep_ckpt(p, p->ck_psi, p->ck_z, k_ckpt, nck);
  if (rc != MOC_OK) return fail(p, rc);
  if (had_pending) {
    p->psi_pending = false;
    rc = moc_reset_psi_scale(p);
    if (rc != MOC_OK) return fail(p, rc);
  }
  return MOC_OK;
}

int moc_adjoint_backward_fit(moc_problem *p, const float *dphi, float *dq, double *dsigt,
                             float *dpsi_in, float *dfit) {
  MOC_NVTX_RANGE("moc_adjoint_backward");
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  if (!dphi || !p->ck_psi) return !dphi ? MOC_ERR_ARG : MOC_ERR_STATE;
  if (dfit && p->d.axial_exp != 2) return MOC_ERR_UNSUPPORTED;   // no fit for a flat source
  cudaSetDevice(p->device);
  const int64_t G = p->d.n_groups;
  if (!p->adj_dphi) {
    rc = dalloc(p, &p->adj_dphi, p->nfsr * p->ldg);
    if (rc == MOC_OK) rc = dalloc(p, &p->adj_dq, p->nfsr * p->ldg);
    if (rc == MOC_OK) rc = dalloc(p, &p->adj_dsig, (int64_t)p->d.n_sigt * p->ldg);
    if (rc != MOC_OK) return rc;
  }
  const int64_t fit_rows = p->d.n_sources * (int64_t)(p->d.fai - 2) * 3;
  if (dfit && !p->adj_dfit) {
    rc = dalloc(p, &p->adj_dfit, fit_rows * p->ldg);
    if (rc != MOC_OK) return rc;
  }
  const size_t fb = sizeof(float) * (size_t)(p->nfsr * p->ldg);
  MOC_CUDA_TRY(cudaMemsetAsync(p->adj_dphi, 0, fb, p->stream));
  MOC_CUDA_TRY(cudaMemsetAsync(p->adj_dq, 0, fb, p->stream));
  MOC_CUDA_TRY(cudaMemsetAsync(p->adj_dsig, 0, sizeof(double) * (size_t)p->d.n_sigt * p->ldg,
                               p->stream));
  if (dfit)
    MOC_CUDA_TRY(cudaMemsetAsync(p->adj_dfit, 0, sizeof(float) * (size_t)(fit_rows * p->ldg),
                                 p->stream));
  rc = copy_rows_dd(p, p->adj_dphi, p->ldg, dphi, G, p->nfsr, G);
  if (rc == MOC_OK)
    rc = moc_launch_adjoint(p, p->ck_psi, p->ck_z, p->ck_k, p->ck_n, p->adj_dphi, p->adj_dq,
                            p->adj_dsig, dpsi_in, dfit ? p->adj_dfit : nullptr);
  if (rc == MOC_OK && dq) rc = copy_rows_dd(p, dq, G, p->adj_dq, p->ldg, p->nfsr, G);
  if (rc == MOC_OK && dsigt)
    rc = copy_rows_dd(p, dsigt, G, p->adj_dsig, p->ldg, (int64_t)p->d.n_sigt, G);
  if (rc == MOC_OK && dfit) rc = copy_rows_dd(p, dfit, G, p->adj_dfit, p->ldg, fit_rows, G);
  if (rc != MOC_OK) return fail(p, rc);
  return MOC_OK;
}

int moc_adjoint_backward(moc_problem *p, const float *dphi, float *dq, double *dsigt,
                         float *dpsi_in) {
  return moc_adjoint_backward_fit(p, dphi, dq, dsigt, dpsi_in, nullptr);
}

int moc_time_adjoint(moc_problem *p, int k_ckpt, const float *dphi, double *ms_forward,
                     double *ms_reverse) {
  int rc = ready(p);
  if (rc != MOC_OK) return rc;
  if (!dphi || !ms_forward || !ms_reverse) return MOC_ERR_ARG;
  cudaSetDevice(p->device);
  cudaEvent_t mid = nullptr;
  if (cudaEventCreate(&mid) != cudaSuccess) return fail(p, MOC_ERR_CUDA);
  if (cudaEventRecord(p->ev0, p->stream) != cudaSuccess) rc = MOC_ERR_CUDA;
  if (rc == MOC_OK) rc = moc_adjoint_forward(p, k_ckpt);
  if (rc == MOC_OK && cudaEventRecord(mid, p->stream) != cudaSuccess) rc = MOC_ERR_CUDA;
  if (rc == MOC_OK) rc = moc_adjoint_backward_fit(p, dphi, nullptr, nullptr, nullptr, nullptr);
  if (rc == MOC_OK && cudaEventRecord(p->ev1, p->stream) != cudaSuccess) rc = MOC_ERR_CUDA;
  if (rc == MOC_OK && cudaEventSynchronize(p->ev1) != cudaSuccess) rc = MOC_ERR_CUDA;
  float f = 0.f, r = 0.f;
  if (rc == MOC_OK) {
    cudaEventElapsedTime(&f, p->ev0, mid);
    cudaEventElapsedTime(&r, mid, p->ev1);
  }
  cudaEventDestroy(mid);
  if (rc != MOC_OK) return rc == MOC_ERR_CUDA ? fail(p, rc) : rc;
  *ms_forward = f;
  *ms_reverse = r;
  return sync_check(p);
}

}  // extern "C"
