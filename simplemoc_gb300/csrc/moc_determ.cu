// moc_determ.cu -- deterministic-order tallies (MOC_FLAG_DETERMINISTIC).
//
// The reference's serial sweep adds the contributions to each FSR in the order
// it visits the segments: track by track, segment by segment, one FP32 addition
// each (fine_flux[g] += ..., src/solver.c:212-228).  The regular sweep adds
// them with unordered reductions, so its FSR fluxes differ from the serial ones
// in the last bits and from run to run.  This mode reproduces the serial order:
//
//   for each chunk of whole 2D tracks, in track order:
//     1. sweep the chunk with its tallies recorded: segment n of track t writes
//        its contribution vector and FSR row to slot t*S + n (the serial order);
//     2. sort the chunk's slots by FSR row, stably (LSD radix sort), so that
//        each row's slots stay in serial order;
//     3. one warp per row adds the row's contributions to the flux in that
//        order, one FP32 addition per contribution and group.
//
// Chunks run in track order and each row's additions within a chunk in slot
// order, so every FSR flux sees the serial sequence of additions.  With the
// PLAIN arithmetic (contributions bit-identical to the reference's) the flux
// equals the serial reference's bit for bit.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cub/cub.cuh>

#include "moc_internal.h"

struct MocDet {
  int64_t chunk_2d = 0;        // 2D tracks per chunk
  int64_t cap = 0;             // segments per chunk
  int32_t ldg = 0;
  float *rec = nullptr;        // [cap][ldg]
  uint32_t *row = nullptr;     // [cap] FSR row of each slot (sort keys)
  uint32_t *row_s = nullptr;   // sorted keys
  uint32_t *idx = nullptr;     // [cap] slot numbers (sort values)
  uint32_t *idx_s = nullptr;   // sorted slots
  uint32_t *starts = nullptr;  // [cap] first sorted position of each row's run
  uint32_t *n_runs = nullptr;
  void *temp = nullptr;
  size_t temp_bytes = 0;
  int64_t bytes[8] = {};
};

namespace {

constexpr int64_t DET_BUDGET = int64_t(2) << 30;   // bytes of records and sort buffers

__global__ void iota_kernel(uint32_t *v, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    v[i] = (uint32_t)i;
}

// First sorted position of every run of equal rows (in no particular order).
__global__ void run_starts_kernel(const uint32_t *__restrict__ keys, int64_t n,
                                  uint32_t *__restrict__ starts, uint32_t *__restrict__ n_runs) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    if (i == 0 || keys[i] != keys[i - 1]) starts[atomicAdd(n_runs, 1u)] = (uint32_t)i;
}

// One warp per run: the row's contributions added to its flux in sorted (=
// serial) order, lanes over the groups.
__global__ void ordered_add_kernel(const uint32_t *__restrict__ keys,
                                   const uint32_t *__restrict__ slots, int64_t n,
                                   const uint32_t *__restrict__ starts,
                                   const uint32_t *__restrict__ n_runs,
                                   const float *__restrict__ rec, float *__restrict__ phi,
                                   int ldg) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t runs = *n_runs;
  for (int64_t r = warp; r < runs; r += n_warps) {
    const int64_t start = starts[r];
    const uint32_t row = keys[start];
    // the run ends where the key changes (32 keys a step, by ballot)
    int64_t end = start + 1;
    for (int64_t b = start + 1; b < n; b += 32) {
      const int64_t i = b + lane;
      const bool other = i >= n || keys[i] != row;
      const unsigned m = __ballot_sync(0xffffffffu, other);
      if (m) {
        end = b + __ffs(m) - 1;
        break;
      }
      end = b + 32;
    }
    float *dst = phi + (int64_t)row * ldg;
    for (int g = lane; g < ldg; g += 32) {
      float acc = dst[g];
      int64_t j = start;
      // four loads in flight, the additions in order
      for (; j + 4 <= end; j += 4) {
        const float c0 = rec[(int64_t)slots[j] * ldg + g];
        const float c1 = rec[(int64_t)slots[j + 1] * ldg + g];
        const float c2 = rec[(int64_t)slots[j + 2] * ldg + g];
        const float c3 = rec[(int64_t)slots[j + 3] * ldg + g];
        acc = __fadd_rn(acc, c0);
        acc = __fadd_rn(acc, c1);
        acc = __fadd_rn(acc, c2);
        acc = __fadd_rn(acc, c3);
      }
      for (; j < end; ++j) acc = __fadd_rn(acc, rec[(int64_t)slots[j] * ldg + g]);
      dst[g] = acc;
    }
  }
}

int end_bit_for(int64_t nfsr) {
  int b = 1;
  while (b < 32 && ((int64_t)1 << b) < nfsr) ++b;
  return b;
}

int det_alloc(moc_problem *p);

// The buffers, allocated on the first deterministic sweep (all or none).
int det_setup(moc_problem *p) {
  if (p->det && p->det->ldg == p->ldg) return MOC_OK;
  const int rc = det_alloc(p);
  if (rc != MOC_OK) moc_det_release(p);
  return rc;
}

int det_alloc(moc_problem *p) {
  const int64_t PZS = (int64_t)p->d.n_polar * p->d.z_stacked * p->d.n_seg;
  moc_det_release(p);
  MocDet *d = new MocDet();
  p->det = d;
  d->ldg = p->ldg;
  // records (ldg floats) + keys, sorted keys, slots, sorted slots, run starts
  const int64_t per_seg = 4 * (int64_t)p->ldg + 5 * 4;
  int64_t chunk = DET_BUDGET / (per_seg * PZS);
  if (chunk < 1) chunk = 1;
  if (chunk > p->d.n_tracks_2d) chunk = p->d.n_tracks_2d;
  while (chunk > 1 && chunk * PZS > (int64_t)INT32_MAX) chunk /= 2;
  if (chunk * PZS > (int64_t)INT32_MAX) return MOC_ERR_UNSUPPORTED;
  d->chunk_2d = chunk;
  d->cap = chunk * PZS;
  const int64_t sizes[7] = {4 * d->cap * p->ldg, 4 * d->cap, 4 * d->cap, 4 * d->cap,
                            4 * d->cap, 4 * d->cap, 4};
  void **ptrs[7] = {reinterpret_cast<void **>(&d->rec), reinterpret_cast<void **>(&d->row),
                    reinterpret_cast<void **>(&d->row_s), reinterpret_cast<void **>(&d->idx),
                    reinterpret_cast<void **>(&d->idx_s), reinterpret_cast<void **>(&d->starts),
                    reinterpret_cast<void **>(&d->n_runs)};
  for (int k = 0; k < 7; ++k) {
    const int rc = moc_dev_alloc(p, ptrs[k], sizes[k]);
    if (rc != MOC_OK) return rc;
    d->bytes[k] = sizes[k];
  }
  size_t tb = 0;
  if (cub::DeviceRadixSort::SortPairs(nullptr, tb, d->row, d->row_s, d->idx, d->idx_s,
                                      (int)d->cap, 0, end_bit_for(p->nfsr), p->stream) !=
      cudaSuccess)
    return MOC_ERR_CUDA;
  const int rc = moc_dev_alloc(p, &d->temp, (int64_t)tb);
  if (rc != MOC_OK) return rc;
  d->temp_bytes = tb;
  d->bytes[7] = (int64_t)tb;
  return MOC_OK;
}

}  // namespace

void moc_det_release(moc_problem *p) {
  MocDet *d = p->det;
  if (!d) return;
  void *ptrs[8] = {d->rec, d->row, d->row_s, d->idx, d->idx_s, d->starts, d->n_runs, d->temp};
  for (int k = 0; k < 8; ++k) moc_dev_free(p, ptrs[k], d->bytes[k]);
  delete d;
  p->det = nullptr;
}

int moc_det_sweep(moc_problem *p) {
  int rc = det_setup(p);
  if (rc != MOC_OK) return rc;
  MocDet *d = p->det;
  const int64_t PZS = (int64_t)p->d.n_polar * p->d.z_stacked * p->d.n_seg;
  const int end_bit = end_bit_for(p->nfsr);
  int sms = 0;
  MOC_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device));
  for (int64_t i0 = 0; i0 < p->d.n_tracks_2d; i0 += d->chunk_2d) {
    const int64_t i1 = i0 + d->chunk_2d < p->d.n_tracks_2d ? i0 + d->chunk_2d : p->d.n_tracks_2d;
    const int64_t n = (i1 - i0) * PZS;
    rc = moc_launch_sweep_record(p, i0, i1, d->rec, reinterpret_cast<int32_t *>(d->row));
    if (rc != MOC_OK) return rc;
    iota_kernel<<<(unsigned)(sms * 4), 256, 0, p->stream>>>(d->idx, n);
    size_t tb = d->temp_bytes;
    MOC_CUDA_TRY(cub::DeviceRadixSort::SortPairs(d->temp, tb, d->row, d->row_s, d->idx, d->idx_s,
                                                 (int)n, 0, end_bit, p->stream));
    MOC_CUDA_TRY(cudaMemsetAsync(d->n_runs, 0, sizeof(uint32_t), p->stream));
    run_starts_kernel<<<(unsigned)(sms * 4), 256, 0, p->stream>>>(d->row_s, n, d->starts,
                                                                  d->n_runs);
    ordered_add_kernel<<<(unsigned)(sms * 8), 256, 0, p->stream>>>(
        d->row_s, d->idx_s, n, d->starts, d->n_runs, d->rec, p->phi, p->ldg);
    MOC_CUDA_TRY(cudaGetLastError());
    p->launches += 3;   // iota, run starts, ordered add (the sweep counts itself)
  }
  return MOC_OK;
}
