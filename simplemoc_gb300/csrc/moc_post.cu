// moc_post.cu -- the post-sweep steps of one power iteration on the device:
//   renormalize_flux  (src/solver.c:1143-1230)
//   update_sources    (src/solver.c:1235-1320)
//   compute_keff      (src/solver.c:1324-1437)
// All global sums are FP64 and deterministic: each reduction kernel runs a
// fixed number of blocks, writes one partial per block, and a one-block
// finalize kernel adds the partials in index order.  Scalars (norm factor,
// keff, residual) stay on the device so that a whole power iteration can be
// captured in a CUDA graph.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <mutex>

#include "moc_internal.h"

namespace {

constexpr int RBLOCKS = 1024;      // partials per reduction (fixed: deterministic sums)
constexpr int RTHREADS = 256;
constexpr double PI = 3.14159265358979323846;

__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }

__device__ __forceinline__ double block_sum(double v, double *sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r += sh[i];
  __syncthreads();
  return r;   // valid in thread 0
}

// ---- renormalize_flux, step 1: fission-rate partials, sum of phi*vol*nuSigF
// (src/solver.c:1160-1175; the float products keep the reference order).
template <typename T>
__global__ void __launch_bounds__(RTHREADS) renorm_partials(const T *__restrict__ phi,
                                                            const float *__restrict__ vol,
                                                            const int32_t *__restrict__ src_xs,
                                                            const float *__restrict__ xs,
                                                            int64_t nfsr, int F, int G, int ldg,
                                                            double *__restrict__ partials) {
  __shared__ double sh[RTHREADS / 32];
  double acc = 0.0;
  const int64_t n = nfsr * (int64_t)G;
  for (int64_t e = (int64_t)blockIdx.x * RTHREADS + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * RTHREADS) {
    const int64_t row = e / G;
    const int g = (int)(e - row * G);
    const int64_t s = row / F;
    const float nusf = xs[((int64_t)src_xs[s] * G + g) * 3 + 0];
    if (sizeof(T) == 4) {
      float v = __fmul_rn(__fmul_rn((float)phi[row * ldg + g], vol[s]), nusf);
      acc += (double)v;
    } else {
      acc += (double)phi[row * ldg + g] * (double)vol[s] * (double)nusf;
    }
  }
  double b = block_sum(acc, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = b;
}

// step 2: total, norm factor (src/solver.c:1203: float norm_factor = 1.0 / total)
template <typename T>
__global__ void renorm_finalize(const double *__restrict__ partials, int nparts,
                                double *__restrict__ scalars) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double total = 0.0;
  for (int i = 0; i < nparts; ++i) total += partials[i];
  scalars[SC_TOTAL_FISSION] = total;
  if (sizeof(T) == 4)
    scalars[SC_NORM] = (double)(float)(1.0 / total);
  else
    scalars[SC_NORM] = 1.0 / total;
}

// step 3: per-source adjust = norm * 4 * pi * F / vol (src/solver.c:1210)
template <typename T>
__global__ void renorm_adjust(const float *__restrict__ vol, int64_t ns, int F,
                              const double *__restrict__ scalars, T *__restrict__ adjust) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= ns) return;
  if (sizeof(T) == 4) {
    const float norm = (float)scalars[SC_NORM];
    // float*int -> float, then double arithmetic, rounded to float
    adjust[s] = (T)((double)__fmul_rn(norm, 4.0f) * PI * (double)F / (double)vol[s]);
  } else {
    adjust[s] = (T)(scalars[SC_NORM] * 4.0 * PI * (double)F / (double)vol[s]);
  }
}

// step 4: phi *= adjust(source); psi_f, psi_b *= norm (src/solver.c:1207-1226)
template <typename T>
__global__ void __launch_bounds__(RTHREADS) renorm_scale(T *__restrict__ phi,
                                                         const T *__restrict__ adjust,
                                                         int64_t nphi, int64_t row_elems,
                                                         T *__restrict__ psi_f,
                                                         T *__restrict__ psi_b, int64_t npsi,
                                                         const double *__restrict__ scalars) {
  const T norm = (T)scalars[SC_NORM];
  const int64_t stride = (int64_t)gridDim.x * RTHREADS;
  for (int64_t e = (int64_t)blockIdx.x * RTHREADS + threadIdx.x; e < nphi; e += stride)
    phi[e] = phi[e] * adjust[e / row_elems];
  for (int64_t e = (int64_t)blockIdx.x * RTHREADS + threadIdx.x; e < npsi; e += stride) {
    psi_f[e] = psi_f[e] * norm;
    psi_b[e] = psi_b[e] * norm;
  }
}

// ---- update_sources (+ optional compute_keff sums), one warp per fine region.
// The scatter table is stored transposed, St[m][g2][g] = S[m][g][g2], so that
// the lanes of a warp read consecutive destination groups.
template <typename T, bool WITH_KEFF>
__global__ void __launch_bounds__(RTHREADS) update_kernel(
    const T *__restrict__ phi, T *__restrict__ q, const int32_t *__restrict__ src_xs,
    const float *__restrict__ xs, const float *__restrict__ st, int64_t nfsr, int F, int G,
    int ldg, double *__restrict__ scalars, double *__restrict__ partials) {
  extern __shared__ unsigned char smem_raw[];
  T *sphi = reinterpret_cast<T *>(smem_raw);           // [warps][ldg]
  __shared__ double sh[RTHREADS / 32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int warps = RTHREADS / 32;
  T *myphi = sphi + (int64_t)warp * ldg;
  double res_acc = 0.0, abs_acc = 0.0, fis_acc = 0.0;
  const double keff = scalars[SC_KEFF_IN];
  const float inverse_k_f = (float)(1.0 / keff);        // src/solver.c:1241
  for (int64_t row = (int64_t)blockIdx.x * warps + warp; row < nfsr;
       row += (int64_t)gridDim.x * warps) {
    const int64_t s = row / F;
    const int64_t m = src_xs[s];
    const float *x = xs + m * G * 3;
    const float *S = st + m * (int64_t)G * G;
    const T *ph = phi + row * ldg;
    T *qr = q + row * ldg;
    // fission source of the region (src/solver.c:1266-1271)
    T fis = 0;
    double ab64 = 0.0, fi64 = 0.0;
    // explicit roundings: the fused (WITH_KEFF) and plain instances must
    // produce identical sources whatever the compiler's contraction choices
    for (int g = lane; g < G; g += 32) {
      const T v = ph[g];
      myphi[g] = v;
      const T fprod = mul_rn(v, (T)x[g * 3 + 0]);
      fis = add_rn(fis, fprod);
      if (WITH_KEFF) {
        ab64 += (double)mul_rn((T)x[g * 3 + 1], v);
        fi64 += (double)fprod;
      }
    }
    for (int o = 16; o > 0; o >>= 1) fis += __shfl_xor_sync(0xffffffffu, fis, o);
    __syncwarp();
    if (sizeof(T) == 4)
      fis = mul_rn(fis, (T)inverse_k_f);
    else
      fis = fis / (T)keff;
    if (WITH_KEFF) {
      abs_acc += ab64;
      fis_acc += fi64;
    }
    // scatter source and new source per group (src/solver.c:1274-1300)
    for (int g = lane; g < G; g += 32) {
      T sc = 0;
      for (int g2 = 0; g2 < G; ++g2) sc = add_rn(sc, mul_rn((T)S[(int64_t)g2 * G + g], myphi[g2]));
      const T chi = (T)x[g * 3 + 2];
      T nw;
      if (sizeof(T) == 4)
        nw = (T)((double)__fadd_rn(__fmul_rn((float)fis, (float)chi), (float)sc) / (4.0 * PI));
      else
        nw = (fis * chi + sc) / (T)(4.0 * PI);
      const T old = qr[g];
      const T d = add_rn(nw, -old);
      res_acc += (double)div_rn(mul_rn(d, d), mul_rn(old, old));
      qr[g] = nw;
    }
    __syncwarp();
  }
  double r = block_sum(res_acc, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = r;
  if (WITH_KEFF) {
    double a = block_sum(abs_acc, sh);
    if (threadIdx.x == 0) partials[RBLOCKS + blockIdx.x] = a;
    double f = block_sum(fis_acc, sh);
    if (threadIdx.x == 0) partials[2 * RBLOCKS + blockIdx.x] = f;
  }
}

// compute_keff sums alone (src/solver.c:1335-1382)
template <typename T>
__global__ void __launch_bounds__(RTHREADS) keff_partials(const T *__restrict__ phi,
                                                          const int32_t *__restrict__ src_xs,
                                                          const float *__restrict__ xs,
                                                          int64_t nfsr, int F, int G, int ldg,
                                                          double *__restrict__ partials) {
  __shared__ double sh[RTHREADS / 32];
  double ab = 0.0, fi = 0.0;
  const int64_t n = nfsr * (int64_t)G;
  for (int64_t e = (int64_t)blockIdx.x * RTHREADS + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * RTHREADS) {
    const int64_t row = e / G;
    const int g = (int)(e - row * G);
    const float *x = xs + ((int64_t)src_xs[row / F] * G + g) * 3;
    const T v = phi[row * ldg + g];
    ab += (double)((T)x[1] * v);
    fi += (double)((T)x[0] * v);
  }
  double a = block_sum(ab, sh);
  if (threadIdx.x == 0) partials[RBLOCKS + blockIdx.x] = a;
  double f = block_sum(fi, sh);
  if (threadIdx.x == 0) partials[2 * RBLOCKS + blockIdx.x] = f;
}

__global__ void update_finalize(const double *__restrict__ partials, double *__restrict__ scalars,
                                int with_residual, int with_keff) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (with_residual) {
    double r = 0.0;
    for (int i = 0; i < RBLOCKS; ++i) r += partials[i];
    scalars[SC_RESIDUAL] = r;
  }
  if (with_keff) {
    double a = 0.0, f = 0.0;
    for (int i = 0; i < RBLOCKS; ++i) {
      a += partials[RBLOCKS + i];
      f += partials[2 * RBLOCKS + i];
    }
    scalars[SC_ABS] = a;
    scalars[SC_FISSION] = f;
    const double k = f / (a + scalars[SC_LEAKAGE]);
    scalars[SC_KEFF] = k;
    scalars[SC_KEFF_IN] = k;     // the next update_sources uses it (src/main.c:81,87)
  }
}

__global__ void set_scalar(double *scalars, int slot, double v) {
  if (threadIdx.x == 0 && blockIdx.x == 0) scalars[slot] = v;
}

template <typename T>
int renorm_t(moc_problem *p, T *phi, T *psi_f, T *psi_b, T *adjust) {
  const moc_dims &d = p->d;
  renorm_partials<T><<<RBLOCKS, RTHREADS, 0, p->stream>>>(phi, p->vol, p->src_xs, p->xs,
                                                          p->nfsr, d.fai, d.n_groups, p->ldg,
                                                          p->partials);
  renorm_finalize<T><<<1, 32, 0, p->stream>>>(p->partials, RBLOCKS, p->scalars);
  const int64_t ns = d.n_sources;
  renorm_adjust<T><<<(unsigned)((ns + 255) / 256), 256, 0, p->stream>>>(p->vol, ns, d.fai,
                                                                       p->scalars, adjust);
  int sms = 0;
  MOC_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device));
  renorm_scale<T><<<(unsigned)(sms * 8), RTHREADS, 0, p->stream>>>(
      phi, adjust, p->nfsr * p->ldg, (int64_t)d.fai * p->ldg, psi_f, psi_b, p->n3d * p->ldg,
      p->scalars);
  MOC_CUDA_TRY(cudaGetLastError());
  p->launches += 4;
  return MOC_OK;
}

template <typename T>
int update_t(moc_problem *p, const T *phi, T *q, bool with_keff) {
  const moc_dims &d = p->d;
  size_t smem = sizeof(T) * (size_t)p->ldg * (RTHREADS / 32);
  if (with_keff)
    update_kernel<T, true><<<RBLOCKS, RTHREADS, smem, p->stream>>>(
        phi, q, p->src_xs, p->xs, p->scatter_t, p->nfsr, d.fai, d.n_groups, p->ldg, p->scalars,
        p->partials);
  else
    update_kernel<T, false><<<RBLOCKS, RTHREADS, smem, p->stream>>>(
        phi, q, p->src_xs, p->xs, p->scatter_t, p->nfsr, d.fai, d.n_groups, p->ldg, p->scalars,
        p->partials);
  update_finalize<<<1, 32, 0, p->stream>>>(p->partials, p->scalars, 1, with_keff ? 1 : 0);
  MOC_CUDA_TRY(cudaGetLastError());
  p->launches += 2;
  return MOC_OK;
}

template <typename T>
int keff_t(moc_problem *p, const T *phi) {
  const moc_dims &d = p->d;
  keff_partials<T><<<RBLOCKS, RTHREADS, 0, p->stream>>>(phi, p->src_xs, p->xs, p->nfsr, d.fai,
                                                        d.n_groups, p->ldg, p->partials);
  update_finalize<<<1, 32, 0, p->stream>>>(p->partials, p->scalars, 0, 1);
  MOC_CUDA_TRY(cudaGetLastError());
  p->launches += 2;
  return MOC_OK;
}

}  // namespace

int moc_post_scratch_blocks() { return RBLOCKS; }

int moc_launch_renormalize(moc_problem *p) {
  if (p->mode == MOC_MODE_FP64)
    return renorm_t<double>(p, p->phi64, p->psi_f64, p->psi_b64,
                            reinterpret_cast<double *>(p->partials + 3 * RBLOCKS));
  return renorm_t<float>(p, p->phi, p->psi_f, p->psi_b,
                         reinterpret_cast<float *>(p->partials + 3 * RBLOCKS));
}

int moc_launch_update(moc_problem *p, double keff, bool keff_on_device, bool with_keff) {
  if (!keff_on_device) {
    set_scalar<<<1, 1, 0, p->stream>>>(p->scalars, SC_KEFF_IN, keff);
    p->launches++;
  }
  if (p->mode == MOC_MODE_FP64) return update_t<double>(p, p->phi64, p->q64, with_keff);
  return update_t<float>(p, p->phi, p->q, with_keff);
}

int moc_launch_keff(moc_problem *p, double leakage) {
  set_scalar<<<1, 1, 0, p->stream>>>(p->scalars, SC_LEAKAGE, leakage);
  p->launches++;
  if (p->mode == MOC_MODE_FP64) return keff_t<double>(p, p->phi64);
  return keff_t<float>(p, p->phi);
}

int moc_set_leakage(moc_problem *p, double leakage) {
  set_scalar<<<1, 1, 0, p->stream>>>(p->scalars, SC_LEAKAGE, leakage);
  p->launches++;
  MOC_CUDA_TRY(cudaGetLastError());
  return MOC_OK;
}

// ---------------------------------------------------------------------------
// renormalize_flux without device allocation.
//
// Some callers cannot let a library call cudaMalloc: a framework or memory
// pool that must account for every device byte it hands out, a real-time loop
// that forbids allocation once it has started, or a process whose buffers are
// mapped from another process over IPC.  This entry point runs the same four
// kernels as moc_renormalize_flux on buffers the caller owns, with its scratch
// (per-block partial sums, the two scalars, one float per source region) in a
// file-scope device array instead of an allocation.  The array is reserved on
// every GPU that loads the library and stays there until the process exits.
//
// Host code must not pass g_renorm_scratch itself to a kernel: on the host the
// name is only a stand-in for the device object.  Its device address is looked
// up once per device with cudaGetSymbolAddress, below, while that device is
// current; the first call on a device does this set-up, so make that first
// call before any stream capture.
// ---------------------------------------------------------------------------
namespace {

constexpr int64_t NOALLOC_FLOATS = MOC_NOALLOC_MAX_SOURCES;                 // adjust[]
constexpr int64_t NOALLOC_DOUBLES = RBLOCKS + SC_COUNT + NOALLOC_FLOATS / 2;

static __device__ __align__(256) double g_renorm_scratch[NOALLOC_DOUBLES];
static_assert(sizeof(g_renorm_scratch) == MOC_NOALLOC_SCRATCH_BYTES,
              "scratch size must match the size stated in the header");

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_scratch_mu;
double *g_scratch_dev[NOALLOC_MAX_DEVICES] = {};

// Device address of g_renorm_scratch on the current device (set-up once).
int scratch_address(int device, double **out) {
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_dev[device]) {
    void *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_renorm_scratch);
    if (e != cudaSuccess || ptr == nullptr) {
      cudaGetLastError();
      return MOC_ERR_CUDA;
    }
    g_scratch_dev[device] = static_cast<double *>(ptr);
  }
  *out = g_scratch_dev[device];
  return MOC_OK;
}

}  // namespace

extern "C" int moc_renormalize_flux_noalloc(float *fine_flux, float *psi_f, float *psi_b,
                                            const float *vol, const int32_t *src_xs,
                                            const float *xs, int64_t n_sources, int32_t fai,
                                            int32_t n_groups, int64_t n_tracks_3d,
                                            double *norm_out, void *stream) {
  if (!fine_flux || !psi_f || !psi_b || !vol || !src_xs || !xs) return MOC_ERR_ARG;
  if (n_sources < 1 || fai < 1 || n_groups < 1 || n_tracks_3d < 0) return MOC_ERR_ARG;
  if (n_sources > MOC_NOALLOC_MAX_SOURCES) return MOC_ERR_ARG;   // scratch holds one float per source
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) {
    cudaGetLastError();
    return MOC_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= NOALLOC_MAX_DEVICES) return MOC_ERR_UNSUPPORTED;
  double *scratch = nullptr;
  int rc = scratch_address(device, &scratch);
  if (rc != MOC_OK) return rc;
  double *partials = scratch;
  double *scalars = scratch + RBLOCKS;
  float *adjust = reinterpret_cast<float *>(scratch + RBLOCKS + SC_COUNT);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t nfsr = n_sources * fai;
  int sms = 0;
  MOC_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  // Every scratch slot read below is written earlier in the same call (all
  // RBLOCKS partials, both scalars, adjust[0..n_sources)), so nothing has to be
  // cleared between calls.  Two calls whose kernels overlap on the GPU (other
  // streams, other host threads) share the one array and race.
  renorm_partials<float><<<RBLOCKS, RTHREADS, 0, s>>>(fine_flux, vol, src_xs, xs, nfsr, fai,
                                                      n_groups, n_groups, partials);
  renorm_finalize<float><<<1, 32, 0, s>>>(partials, RBLOCKS, scalars);
  renorm_adjust<float><<<(unsigned)((n_sources + 255) / 256), 256, 0, s>>>(vol, n_sources, fai,
                                                                           scalars, adjust);
  renorm_scale<float><<<(unsigned)(sms * 8), RTHREADS, 0, s>>>(
      fine_flux, adjust, nfsr * n_groups, (int64_t)fai * n_groups, psi_f, psi_b,
      n_tracks_3d * n_groups, scalars);
  MOC_CUDA_TRY(cudaGetLastError());
  if (norm_out)
    MOC_CUDA_TRY(cudaMemcpyAsync(norm_out, scalars + SC_TOTAL_FISSION, 2 * sizeof(double),
                                 cudaMemcpyDeviceToDevice, s));
  return MOC_OK;
}
