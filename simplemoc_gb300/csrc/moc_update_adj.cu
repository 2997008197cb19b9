// moc_update_adj.cu -- reverse mode of update_sources (src/solver.c:1235-1300).
//
// The forward step maps the scalar flux phi0 of every fine region r of a
// source of material m to its new source
//     q[r][g] = (chi[m][g] * F_r / k + sum_h S[m][g][h] * phi0[r][h]) / (4 pi),
//     F_r     = sum_h nuSigmaF[m][h] * phi0[r][h].
// Given dL/dq it accumulates, per material,
//     dL/dS[m][g][h]      = sum_{r in m} dq[r][g] * phi0[r][h] / (4 pi)
//     dL/dnuSigmaF[m][h]  = sum_{r in m} a_r * phi0[r][h] / (4 pi k),  a_r = sum_g dq[r][g] chi[m][g]
// and per fine region
//     dL/dphi0[r][h]      = (sum_g dq[r][g] S[m][g][h] + a_r nuSigmaF[m][h] / k) / (4 pi).
// Sources come grouped by material in the update work items (material, first,
// end of xs_order); one block takes an item, so each material's sums build up
// in registers or shared memory and reach global memory (FP64) once a block.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "moc_internal.h"

namespace {

constexpr int ADJ_THREADS = 256;
constexpr int TILE = 32;            // dL/dS tile: 32 destination x 32 source groups
constexpr int CHUNK = 32;           // fine regions staged at a time
constexpr double FOUR_PI = 12.566370614359172953850573533118;

// dL/dS of one item and one 32 x 32 tile (blockIdx.y): each thread holds four
// FP64 accumulators (one destination group, four source groups).
__global__ void __launch_bounds__(ADJ_THREADS) scatter_adjoint_kernel(
    const float *__restrict__ phi0, const float *__restrict__ dq, const int32_t *__restrict__ items,
    const int32_t *__restrict__ order, int F, int G, double *__restrict__ dscatter) {
  __shared__ float s_dq[CHUNK][TILE + 1];
  __shared__ float s_ph[CHUNK][TILE + 1];
  const int m = items[3 * blockIdx.x], a = items[3 * blockIdx.x + 1], b = items[3 * blockIdx.x + 2];
  const int tiles = (G + TILE - 1) / TILE;
  const int g0 = (blockIdx.y / tiles) * TILE, h0 = (blockIdx.y % tiles) * TILE;
  const int tg = threadIdx.x >> 3, th = (threadIdx.x & 7) * 4;    // entry (tg, th .. th + 3)
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const int rows = (b - a) * F;
  for (int c0 = 0; c0 < rows; c0 += CHUNK) {
    // stage CHUNK regions' dq over the tile's destination groups and phi0 over
    // its source groups
    for (int i = threadIdx.x; i < CHUNK * TILE; i += ADJ_THREADS) {
      const int rr = i / TILE, col = i % TILE;
      const int ri = c0 + rr;
      float vq = 0.f, vp = 0.f;
      if (ri < rows) {
        const int64_t row = (int64_t)order[a + ri / F] * F + ri % F;
        if (g0 + col < G) vq = dq[row * G + g0 + col];
        if (h0 + col < G) vp = phi0[row * G + h0 + col];
      }
      s_dq[rr][col] = vq;
      s_ph[rr][col] = vp;
    }
    __syncthreads();
    const int n = rows - c0 < CHUNK ? rows - c0 : CHUNK;
    for (int rr = 0; rr < n; ++rr) {
      const double x = s_dq[rr][tg];
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[e] = fma(x, (double)s_ph[rr][th + e], acc[e]);
    }
    __syncthreads();
  }
  const int g = g0 + tg;
  if (g < G) {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int h = h0 + th + e;
      if (h < G) atomicAdd(dscatter + ((int64_t)m * G + g) * G + h, acc[e] / FOUR_PI);
    }
  }
}

// dL/dnuSigmaF of one item (accumulated in shared memory) and dL/dphi0 of its
// fine regions: one warp per region, lanes over groups.
__global__ void __launch_bounds__(ADJ_THREADS) fission_adjoint_kernel(
    const float *__restrict__ phi0, const float *__restrict__ dq, const int32_t *__restrict__ items,
    const int32_t *__restrict__ order, const float *__restrict__ xs, const float *__restrict__ st,
    int F, int G, double keff, double *__restrict__ dnusf, float *__restrict__ dphi0) {
  extern __shared__ unsigned char s_raw[];
  double *s_nusf = reinterpret_cast<double *>(s_raw);                     // [G]
  float *s_row = reinterpret_cast<float *>(s_raw + sizeof(double) * G);    // [warps][G]
  const int m = items[3 * blockIdx.x], a = items[3 * blockIdx.x + 1], b = items[3 * blockIdx.x + 2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int WARPS = ADJ_THREADS / 32;
  for (int h = threadIdx.x; h < G; h += ADJ_THREADS) s_nusf[h] = 0.0;
  __syncthreads();
  float *myrow = s_row + (int64_t)warp * G;
  const float *xm = xs + (int64_t)m * G * 3;
  const float *stm = st + (int64_t)m * G * G;          // St[h][g] = S[g][h]
  const int rows = (b - a) * F;
  for (int ri = warp; ri < rows; ri += WARPS) {
    const int64_t row = (int64_t)order[a + ri / F] * F + ri % F;
    double part = 0.0;
    for (int g = lane; g < G; g += 32) {
      const float v = dq[row * G + g];
      myrow[g] = v;
      part = fma((double)v, (double)xm[3 * g + 2], part);               // dq . chi
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    __syncwarp();
    const double ar = part;
    for (int h = lane; h < G; h += 32) {
      if (dnusf) atomicAdd(s_nusf + h, ar * (double)phi0[row * G + h]);
      if (dphi0) {
        double sdot = 0.0;
        const float *sh = stm + (int64_t)h * G;
        for (int g = 0; g < G; ++g) sdot = fma((double)myrow[g], (double)sh[g], sdot);
        dphi0[row * G + h] = (float)((sdot + ar * (double)xm[3 * h] / keff) / FOUR_PI);
      }
    }
    __syncwarp();
  }
  __syncthreads();
  if (dnusf)
    for (int h = threadIdx.x; h < G; h += ADJ_THREADS)
      atomicAdd(dnusf + (int64_t)m * G + h, s_nusf[h] / (FOUR_PI * keff));
}

}  // namespace

int moc_launch_update_adjoint(moc_problem *p, const float *phi0, const float *dq, double keff,
                              double *dscatter, double *dnusf, float *dphi0) {
  const int G = p->d.n_groups, F = p->d.fai, items = p->n_upd_items;
  if (items < 1) return MOC_OK;
  if (dscatter) {
    MOC_CUDA_TRY(cudaMemsetAsync(dscatter, 0, sizeof(double) * (size_t)p->d.n_xs * G * G,
                                 p->stream));
    const int tiles = (G + TILE - 1) / TILE;
    scatter_adjoint_kernel<<<dim3((unsigned)items, (unsigned)(tiles * tiles)), ADJ_THREADS, 0,
                             p->stream>>>(phi0, dq, p->upd_items, p->xs_order, F, G, dscatter);
    MOC_CUDA_TRY(cudaGetLastError());
    p->launches++;
  }
  if (dnusf || dphi0) {
    if (dnusf)
      MOC_CUDA_TRY(cudaMemsetAsync(dnusf, 0, sizeof(double) * (size_t)p->d.n_xs * G, p->stream));
    const size_t smem = sizeof(double) * G + sizeof(float) * (size_t)(ADJ_THREADS / 32) * G;
    fission_adjoint_kernel<<<(unsigned)items, ADJ_THREADS, smem, p->stream>>>(
        phi0, dq, p->upd_items, p->xs_order, p->xs, p->scatter_t, F, G, keff, dnusf, dphi0);
    MOC_CUDA_TRY(cudaGetLastError());
    p->launches++;
  }
  return MOC_OK;
}
