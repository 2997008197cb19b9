// moc_post.cu -- the post-sweep steps of one power iteration on the device:
//   renormalize_flux  (src/solver.c:1143-1230)
//   update_sources    (src/solver.c:1235-1320)
//   compute_keff      (src/solver.c:1324-1437)
// All global sums are FP64 and deterministic: each reduction kernel runs a
// fixed number of blocks, writes one partial per block, and a one-block
// finalize kernel adds the partials in index order.  Scalars (norm factor,
// keff, residual) stay on the device so that a whole power iteration can be
// captured in a CUDA graph.
#include <cuda.h>
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
// (src/solver.c:1160-1175; the float products keep the reference order).  One
// warp per source: its F fine regions are contiguous rows, and the material's
// nuSigmaF of the lane's groups is loaded once for all of them (up to 128
// groups in registers).  Each lane adds its groups of a region in FP32 and
// folds the result into its FP64 accumulator once per region (FP64 arithmetic
// is a small fraction of FP32 throughput on this part, so it is kept per
// region, not per element).
template <typename T>
__global__ void __launch_bounds__(RTHREADS) renorm_partials(const T *__restrict__ phi,
                                                           const float *__restrict__ vol,
                                                           const int32_t *__restrict__ src_xs,
                                                           const float *__restrict__ xs,
                                                           int64_t ns, int F, int G, int ldg,
                                                           double *__restrict__ partials) {
  __shared__ double sh[RTHREADS / 32];
  double acc = 0.0;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int64_t s = (int64_t)blockIdx.x * (RTHREADS / 32) + warp; s < ns;
       s += (int64_t)gridDim.x * (RTHREADS / 32)) {
    const float v_s = vol[s];
    const float *x = xs + (int64_t)src_xs[s] * G * 3;
    const T *ph = phi + s * F * ldg;
    if (G <= 128) {
      float nsf[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) nsf[i] = lane + 32 * i < G ? __ldg(x + (lane + 32 * i) * 3) : 0.f;
#pragma unroll 4
      for (int f = 0; f < F; ++f) {
        const T *row = ph + (int64_t)f * ldg;
        if (sizeof(T) == 4) {
          float r = 0.f;
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int g = lane + 32 * i;
            if (g < G) r = __fadd_rn(r, __fmul_rn(__fmul_rn((float)__ldg(row + g), v_s), nsf[i]));
          }
          acc += (double)r;
        } else {
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int g = lane + 32 * i;
            if (g < G) acc += (double)__ldg(row + g) * (double)v_s * (double)nsf[i];
          }
        }
      }
    } else {
      for (int f = 0; f < F; ++f) {
        const T *row = ph + (int64_t)f * ldg;
        if (sizeof(T) == 4) {
          float r = 0.f;
          for (int g = lane; g < G; g += 32)
            r = __fadd_rn(r, __fmul_rn(__fmul_rn((float)row[g], v_s), x[g * 3 + 0]));
          acc += (double)r;
        } else {
          for (int g = lane; g < G; g += 32) acc += (double)row[g] * (double)v_s * (double)x[g * 3];
        }
      }
    }
  }
  double b = block_sum(acc, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = b;
}

// The sum of n partials by one warp, in a fixed order: lane l adds partials
// l, l + 32, l + 64, ... into four accumulators in turn, and the lanes' sums
// meet in a fixed shuffle tree.  The order never depends on timing, so every
// run gives the same bits; a single thread adding 1024 partials one after the
// other took ~60-160 us a call, which the batched iteration pays once per core.
// Returns the sum in lane 0.
__device__ __forceinline__ double warp_fixed_sum(const double *__restrict__ x, int n) {
  const int lane = threadIdx.x & 31;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  int i = lane;
  for (; i + 96 < n; i += 128) {
    s0 += x[i];
    s1 += x[i + 32];
    s2 += x[i + 64];
    s3 += x[i + 96];
  }
  for (; i < n; i += 32) s0 += x[i];
  double s = (s0 + s1) + (s2 + s3);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  return s;
}

// step 2: total, norm factor (src/solver.c:1203: float norm_factor = 1.0 / total).
// One warp (launched with 32 threads).
template <typename T>
__global__ void renorm_finalize(const double *__restrict__ partials, int nparts,
                                double *__restrict__ scalars) {
  if (blockIdx.x != 0 || threadIdx.x >= 32) return;
  const double total = warp_fixed_sum(partials, nparts);
  if (threadIdx.x != 0) return;
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

// compute_keff sums alone (src/solver.c:1335-1382): one warp per fine region,
// FP32 within the region's groups, FP64 across regions.
template <typename T>
__global__ void __launch_bounds__(RTHREADS) keff_partials(const T *__restrict__ phi,
                                                          const int32_t *__restrict__ src_xs,
                                                          const float *__restrict__ xs,
                                                          int64_t nfsr, int F, int G, int ldg,
                                                          double *__restrict__ partials) {
  __shared__ double sh[RTHREADS / 32];
  double ab = 0.0, fi = 0.0;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int64_t row = (int64_t)blockIdx.x * (RTHREADS / 32) + warp; row < nfsr;
       row += (int64_t)gridDim.x * (RTHREADS / 32)) {
    const float *x = xs + (int64_t)src_xs[row / F] * G * 3;
    const T *ph = phi + row * ldg;
    T ra = 0, rf = 0;
    for (int g = lane; g < G; g += 32) {
      const T v = ph[g];
      ra = add_rn(ra, mul_rn((T)x[g * 3 + 1], v));
      rf = add_rn(rf, mul_rn((T)x[g * 3 + 0], v));
    }
    ab += (double)ra;
    fi += (double)rf;
  }
  double a = block_sum(ab, sh);
  if (threadIdx.x == 0) partials[RBLOCKS + blockIdx.x] = a;
  double f = block_sum(fi, sh);
  if (threadIdx.x == 0) partials[2 * RBLOCKS + blockIdx.x] = f;
}

// One warp (launched with 32 threads).
__global__ void update_finalize(const double *__restrict__ partials, double *__restrict__ scalars,
                                int with_residual, int with_keff) {
  if (blockIdx.x != 0 || threadIdx.x >= 32) return;
  const double r = with_residual ? warp_fixed_sum(partials, RBLOCKS) : 0.0;
  const double a = with_keff ? warp_fixed_sum(partials + RBLOCKS, RBLOCKS) : 0.0;
  const double f = with_keff ? warp_fixed_sum(partials + 2 * RBLOCKS, RBLOCKS) : 0.0;
  if (threadIdx.x != 0) return;
  if (with_residual) scalars[SC_RESIDUAL] = r;
  if (with_keff) {
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

// Lazy angular-flux scaling (FP32 state).  renormalize_flux multiplies psi_f
// and psi_b by norm (src/solver.c:1219-1226).  Here phi is scaled as before,
// psi_f records a pending factor that the next sweep applies as it loads psi
// (the same single float multiply, so PLAIN stays bit-identical), and psi_b,
// which is never swept (src/solver.c:489), is scaled only if it holds a
// non-zero value (a device flag set at upload).
__global__ void __launch_bounds__(RTHREADS) renorm_scale_lazy(
    float *__restrict__ phi, const float *__restrict__ adjust, int64_t nphi, int64_t row_elems,
    float *__restrict__ psi_b, int64_t npsi, const int32_t *__restrict__ psi_b_nonzero,
    const double *__restrict__ scalars, float *__restrict__ psi_scale) {
  const float norm = (float)scalars[SC_NORM];
  const int64_t stride = (int64_t)gridDim.x * RTHREADS;
  const int64_t t0 = (int64_t)blockIdx.x * RTHREADS + threadIdx.x;
  if (t0 == 0) *psi_scale = norm;
  for (int64_t e = t0; e < nphi; e += stride) phi[e] = phi[e] * adjust[e / row_elems];
  if (*psi_b_nonzero)
    for (int64_t e = t0; e < npsi; e += stride) psi_b[e] = psi_b[e] * norm;
}

__global__ void psi_materialize(float *__restrict__ psi, int64_t n, const float *__restrict__ scale) {
  const float s = *scale;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    psi[e] = psi[e] * s;
}

__global__ void detect_nonzero(const float *__restrict__ v, int64_t n, int32_t *__restrict__ flag) {
  bool nz = false;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    nz |= (v[e] != 0.0f);
  if (__syncthreads_or(nz) && threadIdx.x == 0) *flag = 1;
}

template <typename T>
int renorm_t(moc_problem *p, T *phi, T *psi_f, T *psi_b, T *adjust) {
  const moc_dims &d = p->d;
  renorm_partials<T><<<RBLOCKS, RTHREADS, 0, p->stream>>>(phi, p->vol, p->src_xs, p->xs,
                                                          d.n_sources, d.fai, d.n_groups,
                                                          p->ldg, p->partials);
  renorm_finalize<T><<<1, 32, 0, p->stream>>>(p->partials, RBLOCKS, p->scalars);
  const int64_t ns = d.n_sources;
  renorm_adjust<T><<<(unsigned)((ns + 255) / 256), 256, 0, p->stream>>>(p->vol, ns, d.fai,
                                                                       p->scalars, adjust);
  int sms = 0;
  MOC_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device));
  if (sizeof(T) == 4 && p->psi_scale) {
    // a second renormalize before any sweep: apply the pending factor first so
    // that psi sees the reference's sequence of roundings
    if (p->psi_pending) {
      psi_materialize<<<(unsigned)(sms * 8), RTHREADS, 0, p->stream>>>(
          reinterpret_cast<float *>(psi_f), p->n3d * p->ldg, p->psi_scale);
      p->launches++;
    }
    renorm_scale_lazy<<<(unsigned)(sms * 8), RTHREADS, 0, p->stream>>>(
        reinterpret_cast<float *>(phi), reinterpret_cast<const float *>(adjust),
        p->nfsr * p->ldg, (int64_t)d.fai * p->ldg, reinterpret_cast<float *>(psi_b),
        p->n3d * p->ldg, p->psi_b_nonzero, p->scalars, p->psi_scale);
    p->psi_pending = true;
  } else {
    renorm_scale<T><<<(unsigned)(sms * 8), RTHREADS, 0, p->stream>>>(
        phi, adjust, p->nfsr * p->ldg, (int64_t)d.fai * p->ldg, psi_f, psi_b, p->n3d * p->ldg,
        p->scalars);
  }
  MOC_CUDA_TRY(cudaGetLastError());
  p->launches += 4;
  return MOC_OK;
}

// ---- update_sources as a material-grouped, register-tiled contraction (FP32).
// Work item = (material m, a range of its sources).  The block stages the
// transposed scatter matrix St_m[g2][g] of the item in shared memory; each warp
// takes UT_ROWS fine regions at a time, stages their fluxes as [g2][row] (read
// back as broadcasts), and every lane accumulates 4 destination groups x
// UT_ROWS regions: acc[r][g] += St_m[g2][g] * phi_r[g2], 100 FMAs per 3 shared
// loads.  The same pass forms the fission source and the k_eff sums; sums are
// FP64 per block, added in block order by the finalize kernel.
constexpr int UT_ROWS = 8;
constexpr int UT_WARPS = RTHREADS / 32;

__global__ void __launch_bounds__(RTHREADS) update_tiled_kernel(
    const float *__restrict__ phi, float *__restrict__ q, const int32_t *__restrict__ xs_order,
    const int32_t *__restrict__ items, int n_items, const float *__restrict__ xs,
    const float *__restrict__ st, int F, int G, int ldg, const double *__restrict__ scalars,
    double *__restrict__ partials) {
  extern __shared__ float smem_f[];
  float *sS = smem_f;                                   // [G][ldg]
  float *sP = smem_f + (int64_t)G * ldg;                // [UT_WARPS][G][UT_ROWS]
  __shared__ double sh[RTHREADS / 32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *myP = sP + (int64_t)warp * G * UT_ROWS;
  const int nchunk = ldg / 4;
  const float inverse_k = (float)(1.0 / scalars[SC_KEFF_IN]);     // src/solver.c:1241
  // src/solver.c:1289-1290 divides by 4*pi in double; here the float quotient
  // by fl(4 pi), correctly rounded (Markstein correction), within 1 ulp of it
  const float four_pi = (float)(4.0 * PI);
  const float r_four_pi = 1.0f / four_pi;
  double res_acc = 0.0, abs_acc = 0.0, fis_acc = 0.0;
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const int m = items[3 * it], s0 = items[3 * it + 1], s1 = items[3 * it + 2];
    const float *Sm = st + (int64_t)m * G * G;
    const float *x = xs + (int64_t)m * G * 3;
    __syncthreads();
    for (int e = threadIdx.x; e < G * ldg; e += RTHREADS) {
      const int g2 = e / ldg, g = e - g2 * ldg;
      sS[e] = g < G ? Sm[(int64_t)g2 * G + g] : 0.f;
    }
    __syncthreads();
    const int n_rows = (s1 - s0) * F;
    for (int base = warp * UT_ROWS; base < n_rows; base += UT_WARPS * UT_ROWS) {
      int64_t grow[UT_ROWS];
      float fis[UT_ROWS];
      float pa_lane = 0.f, pf_lane = 0.f;
#pragma unroll
      for (int r = 0; r < UT_ROWS; ++r) {
        const int lr = base + r;
        grow[r] = -1;
        if (lr < n_rows) grow[r] = (int64_t)xs_order[s0 + lr / F] * F + (lr % F);
      }
#pragma unroll
      for (int r = 0; r < UT_ROWS; ++r) {
        fis[r] = 0.f;
        for (int g = lane; g < G; g += 32) {
          const float v = grow[r] >= 0 ? phi[grow[r] * ldg + g] : 0.f;
          myP[g * UT_ROWS + r] = v;
          const float fprod = __fmul_rn(v, x[g * 3 + 0]);
          fis[r] = __fadd_rn(fis[r], fprod);
          pa_lane = __fadd_rn(pa_lane, __fmul_rn(x[g * 3 + 1], v));
        }
        pf_lane = __fadd_rn(pf_lane, fis[r]);
      }
      abs_acc += (double)pa_lane;
      fis_acc += (double)pf_lane;
#pragma unroll
      for (int r = 0; r < UT_ROWS; ++r)
        for (int o = 16; o > 0; o >>= 1) fis[r] = __fadd_rn(fis[r], __shfl_xor_sync(0xffffffffu, fis[r], o));
      __syncwarp();
      if (lane < nchunk) {
        float acc[UT_ROWS][4];
#pragma unroll
        for (int r = 0; r < UT_ROWS; ++r) acc[r][0] = acc[r][1] = acc[r][2] = acc[r][3] = 0.f;
        const float *col = sS + 4 * lane;
#pragma unroll 4
        for (int g2 = 0; g2 < G; ++g2) {
          const float4 s4 = *reinterpret_cast<const float4 *>(col + (int64_t)g2 * ldg);
          const float4 pa = *reinterpret_cast<const float4 *>(myP + g2 * UT_ROWS);
          const float4 pb = *reinterpret_cast<const float4 *>(myP + g2 * UT_ROWS + 4);
          const float pr[UT_ROWS] = {pa.x, pa.y, pa.z, pa.w, pb.x, pb.y, pb.z, pb.w};
#pragma unroll
          for (int r = 0; r < UT_ROWS; ++r) {
            acc[r][0] = fmaf(s4.x, pr[r], acc[r][0]);
            acc[r][1] = fmaf(s4.y, pr[r], acc[r][1]);
            acc[r][2] = fmaf(s4.z, pr[r], acc[r][2]);
            acc[r][3] = fmaf(s4.w, pr[r], acc[r][3]);
          }
        }
        float res_lane = 0.f;
#pragma unroll
        for (int r = 0; r < UT_ROWS; ++r) {
          if (grow[r] < 0) continue;
          const float fk = __fmul_rn(fis[r], inverse_k);
          float *qr = q + grow[r] * ldg + 4 * lane;
          float4 old = *reinterpret_cast<const float4 *>(qr);
          float4 nw;
          float *po = &old.x, *pn = &nw.x;
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const int g = 4 * lane + e;
            if (g < G) {
              const float chi = x[g * 3 + 2];
              // src/solver.c:1289-1295
              const float num = __fadd_rn(__fmul_rn(fk, chi), acc[r][e]);
              float qq = __fmul_rn(num, r_four_pi);
              qq = __fmaf_rn(__fmaf_rn(-qq, four_pi, num), r_four_pi, qq);
              pn[e] = qq;
              const float d = __fsub_rn(pn[e], po[e]);
              res_lane = __fadd_rn(res_lane, __fdiv_rn(__fmul_rn(d, d), __fmul_rn(po[e], po[e])));
            } else {
              pn[e] = po[e];
            }
          }
          *reinterpret_cast<float4 *>(qr) = nw;
        }
        res_acc += (double)res_lane;
      }
      __syncwarp();
    }
  }
  double r = block_sum(res_acc, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = r;
  double a = block_sum(abs_acc, sh);
  if (threadIdx.x == 0) partials[RBLOCKS + blockIdx.x] = a;
  double f = block_sum(fis_acc, sh);
  if (threadIdx.x == 0) partials[2 * RBLOCKS + blockIdx.x] = f;
}

template <typename T>
int update_t(moc_problem *p, const T *phi, T *q, bool with_keff) {
  const moc_dims &d = p->d;
  if (sizeof(T) == 4 && p->mode == MOC_MODE_MIXED && !(p->flags & MOC_FLAG_SIMT_UPDATE) &&
      p->tc_b && (const void *)phi == (const void *)p->phi && (const void *)q == (const void *)p->q) {
    const int rc = moc_launch_update_tc(p);
    if (rc != MOC_OK) return rc;
    update_finalize<<<1, 32, 0, p->stream>>>(p->partials, p->scalars, 1, with_keff ? 1 : 0);
    MOC_CUDA_TRY(cudaGetLastError());
    p->launches++;
    return MOC_OK;
  }
  if (sizeof(T) == 4 && p->upd_items && p->ldg <= 128) {
    const size_t smem = sizeof(float) * ((size_t)d.n_groups * p->ldg +
                                         (size_t)UT_WARPS * d.n_groups * UT_ROWS);
    // the attribute is set outside any stream capture: the first call of a
    // process raises it to the largest size the kernel can take
    static bool attr_set = false;
    if (!attr_set) {
      MOC_CUDA_TRY(cudaFuncSetAttribute(update_tiled_kernel,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)(sizeof(float) * (128 * 128 + UT_WARPS * 128 * UT_ROWS))));
      attr_set = true;
    }
    update_tiled_kernel<<<RBLOCKS, RTHREADS, smem, p->stream>>>(
        reinterpret_cast<const float *>(phi), reinterpret_cast<float *>(q), p->xs_order,
        p->upd_items, p->n_upd_items, p->xs, p->scatter_t, d.fai, d.n_groups, p->ldg,
        p->scalars, p->partials);
    update_finalize<<<1, 32, 0, p->stream>>>(p->partials, p->scalars, 1, with_keff ? 1 : 0);
    MOC_CUDA_TRY(cudaGetLastError());
    p->launches += 2;
    return MOC_OK;
  }
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

__global__ void set_float(float *dst, float v) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *dst = v;
}

// The device factor is 1 whenever no renormalisation is pending, so that a
// kernel may apply it unconditionally (the batched sweep does).
int moc_reset_psi_scale(moc_problem *p) {
  set_float<<<1, 32, 0, p->stream>>>(p->psi_scale, 1.0f);
  MOC_CUDA_TRY(cudaGetLastError());
  p->launches++;
  return MOC_OK;
}

int moc_psi_materialize(moc_problem *p) {
  if (!p->psi_pending) return MOC_OK;
  int sms = 0;
  MOC_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device));
  psi_materialize<<<(unsigned)(sms * 8), RTHREADS, 0, p->stream>>>(p->psi_f, p->n3d * p->ldg,
                                                                   p->psi_scale);
  MOC_CUDA_TRY(cudaGetLastError());
  p->launches++;
  p->psi_pending = false;
  return moc_reset_psi_scale(p);
}

int moc_detect_psi_b(moc_problem *p) {
  MOC_CUDA_TRY(cudaMemsetAsync(p->psi_b_nonzero, 0, sizeof(int32_t), p->stream));
  int sms = 0;
  MOC_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device));
  detect_nonzero<<<(unsigned)(sms * 8), RTHREADS, 0, p->stream>>>(p->psi_b, p->n3d * p->ldg,
                                                                  p->psi_b_nonzero);
  MOC_CUDA_TRY(cudaGetLastError());
  p->launches++;
  return MOC_OK;
}

__global__ void round_to_float_kernel(double *__restrict__ x, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = (double)(float)x[i];
}

// MOC_FLAG_FP32_STATE: the FP64 state arrays rounded to FP32 values in place.
int moc_round_state_fp32(moc_problem *p, bool flux, bool psi, bool source) {
  if (p->mode != MOC_MODE_FP64 || !(p->flags & MOC_FLAG_FP32_STATE)) return MOC_OK;
  int sms = 0;
  MOC_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device));
  const unsigned grid = (unsigned)(sms * 8);
  if (flux) round_to_float_kernel<<<grid, 256, 0, p->stream>>>(p->phi64, p->nfsr * p->ldg);
  if (source) round_to_float_kernel<<<grid, 256, 0, p->stream>>>(p->q64, p->nfsr * p->ldg);
  if (psi) {
    round_to_float_kernel<<<grid, 256, 0, p->stream>>>(p->psi_f64, p->n3d * p->ldg);
    round_to_float_kernel<<<grid, 256, 0, p->stream>>>(p->psi_b64, p->n3d * p->ldg);
  }
  MOC_CUDA_TRY(cudaGetLastError());
  p->launches += (flux ? 1 : 0) + (source ? 1 : 0) + (psi ? 2 : 0);
  return MOC_OK;
}

int moc_launch_renormalize(moc_problem *p) {
  if (p->mode == MOC_MODE_FP64) {
    const int rc = renorm_t<double>(p, p->phi64, p->psi_f64, p->psi_b64,
                                    reinterpret_cast<double *>(p->partials + 3 * RBLOCKS));
    return rc == MOC_OK ? moc_round_state_fp32(p, true, true, false) : rc;
  }
  return renorm_t<float>(p, p->phi, p->psi_f, p->psi_b,
                         reinterpret_cast<float *>(p->partials + 3 * RBLOCKS));
}

int moc_launch_update(moc_problem *p, double keff, bool keff_on_device, bool with_keff) {
  if (!keff_on_device) {
    set_scalar<<<1, 1, 0, p->stream>>>(p->scalars, SC_KEFF_IN, keff);
    p->launches++;
  }
  if (p->mode == MOC_MODE_FP64) {
    const int rc = update_t<double>(p, p->phi64, p->q64, with_keff);
    return rc == MOC_OK ? moc_round_state_fp32(p, false, false, true) : rc;
  }
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
// call before any stream capture.  The address belongs to the device's
// context: the set-up records that context's unique id (cuCtxGetId) and is
// repeated when a later call finds another context current (after a
// cudaDeviceReset the module is loaded again, possibly at another address).
// ---------------------------------------------------------------------------
namespace {

constexpr int64_t NOALLOC_FLOATS = MOC_NOALLOC_MAX_SOURCES;                 // adjust[]
constexpr int64_t NOALLOC_DOUBLES = RBLOCKS + SC_COUNT + NOALLOC_FLOATS / 2;

static __device__ __align__(256) double g_renorm_scratch[NOALLOC_DOUBLES];
static_assert(sizeof(g_renorm_scratch) == MOC_NOALLOC_SCRATCH_BYTES,
              "scratch size must match the size stated in the header");

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_scratch_mu;
struct ScratchSlot {
  unsigned long long ctx_id;   // context the address was looked up in
  double *addr;
};
ScratchSlot g_scratch_dev[NOALLOC_MAX_DEVICES] = {};

// The two driver calls that identify the current context, resolved through
// the runtime (the library does not link the driver library itself).
using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

// Unique id of the current context, 0 when none is current yet.
int current_context_id(unsigned long long *id) {
  *id = 0;
  if (!g_ctx_get_current || !g_ctx_get_id) {
    void *f1 = nullptr, *f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault,
                                         &q1) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) !=
            cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2) {
      cudaGetLastError();
      return MOC_ERR_CUDA;
    }
    g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
    g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
  }
  CUcontext ctx = nullptr;
  if (g_ctx_get_current(&ctx) != CUDA_SUCCESS) return MOC_ERR_CUDA;
  if (ctx && g_ctx_get_id(ctx, id) != CUDA_SUCCESS) return MOC_ERR_CUDA;
  return MOC_OK;
}

// Device address of g_renorm_scratch on the current device: looked up once per
// device, and again only if the device's context has changed since.
int scratch_address(int device, double **out) {
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  unsigned long long id = 0;
  int rc = current_context_id(&id);
  if (rc != MOC_OK) return rc;
  ScratchSlot &slot = g_scratch_dev[device];
  if (!slot.addr || id == 0 || slot.ctx_id != id) {
    void *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_renorm_scratch);
    if (e != cudaSuccess || ptr == nullptr) {
      cudaGetLastError();
      return MOC_ERR_CUDA;
    }
    // the look-up makes the device's primary context current if none was
    rc = current_context_id(&id);
    if (rc != MOC_OK) return rc;
    slot.addr = static_cast<double *>(ptr);
    slot.ctx_id = id;
  }
  *out = slot.addr;
  return MOC_OK;
}

}  // namespace

extern "C" int moc_renormalize_flux_noalloc(float *fine_flux, float *psi_f, float *psi_b,
                                            const float *vol, const int32_t *src_xs,
                                            const float *xs, int64_t n_sources, int32_t fai,
                                            int32_t n_groups, int64_t n_tracks_3d,
                                            double *norm_out, void *stream) {
  if (!fine_flux || !vol || !src_xs || !xs) return MOC_ERR_ARG;
  if (n_sources < 1 || fai < 1 || n_groups < 1 || n_tracks_3d < 0) return MOC_ERR_ARG;
  if (n_tracks_3d > 0 && (!psi_f || !psi_b)) return MOC_ERR_ARG;  // no tracks: psi may be NULL
  if (n_sources > MOC_NOALLOC_MAX_SOURCES) return MOC_ERR_ARG;   // scratch holds one float per source
  {
    // element counts must fit 64-bit integers: products beyond 2^50 are
    // rejected before they are formed (the bound of the handle's validation)
    const double lim = 1125899906842624.0;   // 2^50
    if ((double)n_sources * fai * n_groups > lim || (double)n_tracks_3d * n_groups > lim)
      return MOC_ERR_ARG;
  }
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
  renorm_partials<float><<<RBLOCKS, RTHREADS, 0, s>>>(fine_flux, vol, src_xs, xs, n_sources,
                                                      fai, n_groups, n_groups, partials);
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
