// update_sources (src/solver.c:1235-1320) of the MIXED mode on the tensor
// cores: per tile of 128 fine regions of one material, one GEMM
//
//     D[r][n] = sum_k phi[r][k] * B[n][k],   B = [ S[m] ; nuSigmaF[m] ; SigmaA[m] ]
//
// on tcgen05 (kind::tf32, FP32 accumulation in tensor memory), so the scatter
// source of every group, the fission rate and the absorption rate of a region
// come out of the same product.  FP32 accuracy from TF32 operands by the
// split-precision product x = hi + lo, hi = tf32(x):
//     A.B ~ Ahi.Bhi + Ahi.Blo + Alo.Bhi         (three MMAs per K step)
// whose dropped term Alo.Blo is ~2^-22 relative.  The tensor core rounds its
// FP32 accumulation towards zero at each K step relative to the running sum, so
// the main product Ahi.Bhi is accumulated in up to three K ranges, each in its
// own tensor-memory accumulator, and the two correction products in a fourth;
// the epilogue adds the four with FP32 round-to-nearest (the accumulation bias
// drops from ~1.4e-6 to the level of the CUDA-core kernel).  Four threads per
// region row read its accumulator columns into shared memory; the epilogue,
// coalesced along the rows, forms the new source
//     q = (nuSigmaF.phi / k * chi + S phi) / (4 pi)
// with the residual and the k_eff partial sums, as update_tiled_kernel does.
//
// Shared-memory operands use the canonical K-major layout without swizzle:
// 8-row x 16-byte core matrices, rows 16 bytes apart, core matrices along M/N
// 128 bytes apart (the descriptor's stride offset) and along K `rows x 16`
// bytes apart (its leading offset).  B is split and laid out once per upload on
// the host; A is split while it is staged.
#include <cstring>
#include <vector>

#include "moc_internal.h"

namespace {

constexpr int TC_M = 128;          // fine regions per tile = tensor-memory lanes
constexpr int TC_THREADS = 512;    // four threads per region row
constexpr int TC_MAX_KG = 26;      // K groups of 4 (groups <= 104)
constexpr double TC_PI = 3.14159265358979323846;
// ~1 s at 2 GHz: an MMA tile takes microseconds, so only a fault of the
// tensor pipe runs this out
constexpr long long TC_WAIT_CYCLES = 1LL << 31;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: start address, leading (K) and stride
// (M/N) byte offsets, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t mma_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

__device__ __forceinline__ float to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ float4 ld_nc4(const float *p) {
  float4 v;
  asm("ld.global.nc.L1::no_allocate.v4.f32 {%0,%1,%2,%3}, [%4];"
      : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
      : "l"(p));
  return v;
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// Waits for the barrier phase with a cycle limit; false when it ran out.
__device__ __forceinline__ bool wait_phase(uint64_t *bar, uint32_t phase) {
  const long long t0 = clock64();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred P1;\n\tmbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, P1;\n\t}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(phase)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > TC_WAIT_CYCLES) return false;
  }
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// 16 columns of the product: the main-product accumulators in K order, then
// the corrections (at 3 * stride), added in FP32 round-to-nearest as
// ((K0 + K1) + K2) + corrections.
__device__ __forceinline__ void tmem_ld16_nowait(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

__device__ __forceinline__ void acc_ld16(uint32_t taddr, uint32_t stride, int n_chain,
                                         float (&v)[16]) {
  uint32_t r[16];
  tmem_ld16_nowait(taddr, r);                       // K range 0
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
  // K ranges 1 and 2, then the corrections, in that order
  for (int c = 1; c <= 3; ++c) {
    if (c < 3 && c >= n_chain) continue;
    tmem_ld16_nowait(taddr + (uint32_t)c * stride, r);
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __fadd_rn(v[i], __uint_as_float(r[i]));
  }
}

__device__ __forceinline__ double block_sum_tc(double v, double *sh) {
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

struct TcArgs {
  const float *phi;
  float *q;
  const int32_t *xs_order;
  const int32_t *items;        // (material, first, end) in xs_order, <= 128 / F sources
  int n_items;
  const float *bmat;           // [n_xs][hi, lo][np * kp] in the canonical layout
  const float *xs;             // [n_xs][G][3] (nuSigmaF, SigmaA, chi)
  const double *scalars;
  double *partials;
  int32_t *err;
  int n_partials;
  int F, G, ldg, kp, np;
  uint32_t acc_stride;         // tensor-memory columns per accumulator (power of 2 >= np)
  uint32_t tmem_cols;          // 4 * acc_stride
};

// Shared memory of the kernel (floats unless noted):
//   region 0: A hi and lo, [kgroups][TC_A_LBO bytes] each (K groups padded by
//             16 bytes: the coalesced staging stores are conflict-free); after
//             the products the same space holds the accumulator rows
//             D[128][np + 4] (a row stride of an odd number of 16-byte units)
//   region 1: B hi and lo of the current material, then chi[G]
//   region 2: the global row of each tile row, two buffers of 128 int64
constexpr int TC_A_LBO = TC_M * 16 + 16;      // bytes between K groups of A

__host__ __device__ constexpr int tc_region0_bytes(int kp, int np) {
  return (2 * (kp / 4) * TC_A_LBO > TC_M * (np + 4) * 4 ? 2 * (kp / 4) * TC_A_LBO
                                                         : TC_M * (np + 4) * 4);
}
__host__ __device__ constexpr int tc_smem_bytes(int kp, int np, int G) {
  return tc_region0_bytes(kp, np) + (2 * np * kp + (G + 3) / 4 * 4) * 4 + 2 * TC_M * 8;
}

// The global row (fine region) of tile row `row`, -1 beyond the tile.
__device__ __forceinline__ int64_t tile_grow(const TcArgs &x, int it, int row) {
  if (it >= x.n_items) return -1;
  const int s0 = x.items[3 * it + 1], s1 = x.items[3 * it + 2];
  if (row >= (s1 - s0) * x.F) return -1;
  return (int64_t)x.xs_order[s0 + row / x.F] * x.F + row % x.F;
}

// Each warp moves 8 rows of a tile as (row, K group) pairs, lane-consecutive
// along the row: element e = lane + 32 t of warp w is row 8 w + e / kgroups,
// K group e % kgroups.  rk[t] packs (row << 8) | kgroup, -1 past the warp's rows.
constexpr int TC_ROWS_PER_WARP = TC_M / (TC_THREADS / 32);            // 8
constexpr int TC_PER_LANE = (TC_ROWS_PER_WARP * TC_MAX_KG + 31) / 32;   // 7

__global__ void __launch_bounds__(TC_THREADS, 1) update_tc_kernel(TcArgs x) {
  extern __shared__ __align__(128) unsigned char tc_smem[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  __shared__ double sh[TC_THREADS / 32];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row = tid & (TC_M - 1);            // = (warp % 4) * 32 + lane: its TMEM lane
  const int part = tid >> 7;                   // which quarter of the accumulator columns
  const int KP = x.kp, NP = x.np, G = x.G, ldg = x.ldg;
  const int kgroups = KP / 4;
  const int DS = NP + 4;                       // accumulator row stride in shared memory
  unsigned char *a_hi = tc_smem;
  unsigned char *a_lo = a_hi + kgroups * TC_A_LBO;
  float *d_s = reinterpret_cast<float *>(tc_smem);                  // after the products
  float *b_hi = reinterpret_cast<float *>(tc_smem + tc_region0_bytes(KP, NP));
  float *b_lo = b_hi + NP * KP;
  float *chi_s = b_lo + NP * KP;
  int64_t *grow_s = reinterpret_cast<int64_t *>(chi_s + (G + 3) / 4 * 4);   // [2][128]

  int rk[TC_PER_LANE];
#pragma unroll
  for (int t = 0; t < TC_PER_LANE; ++t) {
    const int e = lane + 32 * t;
    rk[t] = e < TC_ROWS_PER_WARP * kgroups
                ? ((TC_ROWS_PER_WARP * warp + e / kgroups) << 8) | (e % kgroups)
                : -1;
  }

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(x.tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&bar)), "r"(1)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
  }
  int it = blockIdx.x;
  int cur_buf = 0;
  if (tid < TC_M) grow_s[tid] = tile_grow(x, it, tid);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;
  const uint32_t taddr = tmem + ((uint32_t)((warp & 3) * 32) << 16);
  const int ksteps = KP / 8;
  const int n_chain = ksteps < 3 ? ksteps : 3;     // accumulators of the main product
  const uint32_t AS = x.acc_stride;
  // kind::tf32: F32 accumulator, TF32 A and B, both K-major, N = np, M = 128
  const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NP >> 3) << 17) |
                         ((uint32_t)(TC_M >> 4) << 24);
  const float inverse_k = (float)(1.0 / x.scalars[SC_KEFF_IN]);   // src/solver.c:1241
  const float four_pi = (float)(4.0 * TC_PI);
  const float r_four_pi = 1.0f / four_pi;
  double res_acc = 0.0, abs_acc = 0.0, fis_acc = 0.0;
  uint32_t phase = 0;
  int cur_m = -1;
  const int nch = (NP + 15) / 16;               // 16-column chunks of the product
  const int c0 = part * nch / 4, c1 = (part + 1) * nch / 4;

  // this tile's fluxes, coalesced: row-consecutive 16-byte pieces per lane
  float4 buf[TC_PER_LANE];
  auto load_fluxes = [&](const int64_t *gs) {
#pragma unroll
    for (int t = 0; t < TC_PER_LANE; ++t) {
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (rk[t] >= 0) {
        const int64_t gr = gs[rk[t] >> 8];
        const int k = 4 * (rk[t] & 255);
        if (gr >= 0 && k < ldg) v = ld_nc4(x.phi + gr * ldg + k);
        if (k + 0 >= G) v.x = 0.f;
        if (k + 1 >= G) v.y = 0.f;
        if (k + 2 >= G) v.z = 0.f;
        if (k + 3 >= G) v.w = 0.f;
      }
      buf[t] = v;
    }
  };
  load_fluxes(grow_s);

  while (it < x.n_items) {
    const int m = x.items[3 * it];
    const int64_t *gcur = grow_s + cur_buf * TC_M;
    int64_t *gnext = grow_s + (cur_buf ^ 1) * TC_M;
    if (m != cur_m) {                          // the same on every thread
      const uint4 *src = reinterpret_cast<const uint4 *>(x.bmat + (int64_t)m * 2 * NP * KP);
      uint4 *dst = reinterpret_cast<uint4 *>(b_hi);
      for (int i = tid; i < 2 * NP * KP / 4; i += TC_THREADS) dst[i] = __ldg(src + i);
      for (int i = tid; i < G; i += TC_THREADS) chi_s[i] = __ldg(x.xs + ((int64_t)m * G + i) * 3 + 2);
      cur_m = m;
    }
    // ---- A: the fluxes split into TF32 hi and lo (lo rounded as well: the
    // tensor core would otherwise drop its low 13 bits, a bias to zero)
#pragma unroll
    for (int t = 0; t < TC_PER_LANE; ++t) {
      if (rk[t] < 0) continue;
      const float4 v = buf[t];
      const float4 hi = make_float4(to_tf32(v.x), to_tf32(v.y), to_tf32(v.z), to_tf32(v.w));
      const float4 lo = make_float4(to_tf32(v.x - hi.x), to_tf32(v.y - hi.y),
                                    to_tf32(v.z - hi.z), to_tf32(v.w - hi.w));
      const int off = (rk[t] & 255) * TC_A_LBO + (rk[t] >> 8) * 16;
      *reinterpret_cast<float4 *>(a_hi + off) = hi;
      *reinterpret_cast<float4 *>(a_lo + off) = lo;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    // ---- the products, K steps of 8, issued by one thread
    if (tid == 0) {
      tc_fence_after();
      const uint32_t lbo_b = (uint32_t)NP * 16;
      const uint32_t ah = smem_u32(a_hi), al = smem_u32(a_lo);
      const uint32_t bh = smem_u32(b_hi), bl = smem_u32(b_lo);
      for (int kk = 0; kk < ksteps; ++kk) {
        const uint64_t dah = mma_desc(ah + kk * 2 * TC_A_LBO, TC_A_LBO, 128);
        const uint64_t dal = mma_desc(al + kk * 2 * TC_A_LBO, TC_A_LBO, 128);
        const uint64_t dbh = mma_desc(bh + kk * 2 * lbo_b, lbo_b, 128);
        const uint64_t dbl = mma_desc(bl + kk * 2 * lbo_b, lbo_b, 128);
        const int chain = kk * n_chain / ksteps;
        const bool first = kk == 0 || (kk - 1) * n_chain / ksteps != chain;
        mma_tf32(tmem + (uint32_t)chain * AS, dah, dbh, idesc, first ? 0u : 1u);
        mma_tf32(tmem + 3 * AS, dah, dbl, idesc, kk > 0 ? 1u : 0u);
        mma_tf32(tmem + 3 * AS, dal, dbh, idesc, 1u);
      }
      mma_commit(&bar);
    }
    // ---- meanwhile: the next tile's rows and fluxes, this tile's old sources
    const int nx = it + (int)gridDim.x;
    if (tid < TC_M) gnext[tid] = tile_grow(x, nx, tid);
    __syncthreads();
    load_fluxes(gnext);
    float4 qold[TC_PER_LANE];
#pragma unroll
    for (int t = 0; t < TC_PER_LANE; ++t) {
      qold[t] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (rk[t] < 0) continue;
      const int64_t gr = gcur[rk[t] >> 8];
      const int k = 4 * (rk[t] & 255);
      if (gr >= 0 && k < ldg) qold[t] = *reinterpret_cast<const float4 *>(x.q + gr * ldg + k);
    }
    if (tid == 0) {
      if (!wait_phase(&bar, phase)) {
        abort_flag = 1;
        atomicOr(x.err, 2);
      }
      tc_fence_before();
    }
    __syncthreads();
    if (abort_flag) break;
    phase ^= 1u;
    tc_fence_after();
    // ---- the accumulator rows to shared memory (A is consumed), one thread
    // per row and a quarter of its 16-column chunks
#pragma unroll
    for (int cc = 0; cc < (MOC_TC_MAX_NP / 16 + 3) / 4; ++cc) {
      const int c = c0 + cc;
      if (c >= c1) break;                      // the same on every lane of a warp
      float v[16];
      acc_ld16(taddr + (uint32_t)(16 * c), AS, n_chain, v);
      float4 *dr = reinterpret_cast<float4 *>(d_s + row * DS + 16 * c);
      dr[0] = make_float4(v[0], v[1], v[2], v[3]);
      dr[1] = make_float4(v[4], v[5], v[6], v[7]);
      dr[2] = make_float4(v[8], v[9], v[10], v[11]);
      dr[3] = make_float4(v[12], v[13], v[14], v[15]);
    }
    tc_fence_before();
    __syncthreads();
    if (tid < TC_M && gcur[tid] >= 0) {        // the k_eff sums: columns G and G + 1
      fis_acc += (double)d_s[tid * DS + G];
      abs_acc += (double)d_s[tid * DS + G + 1];
    }
    // ---- the new sources, coalesced along the rows
    float res = 0.f;
#pragma unroll
    for (int t = 0; t < TC_PER_LANE; ++t) {
      if (rk[t] < 0) continue;
      const int r = rk[t] >> 8, g = 4 * (rk[t] & 255);
      const int64_t gr = gcur[r];
      if (gr < 0 || g >= ldg) continue;
      const float4 d4 = *reinterpret_cast<const float4 *>(d_s + r * DS + g);
      const float fk = __fmul_rn(d_s[r * DS + G], inverse_k);
      const float *pd = &d4.x;
      const float4 chi4 = *reinterpret_cast<const float4 *>(chi_s + g);   // one conflict-free read
      const float *pc = &chi4.x;
      const float4 old = qold[t];
      float4 nw = old;
      const float *po = &old.x;
      float *pn = &nw.x;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        if (g + e >= G) continue;
        // src/solver.c:1289-1295
        const float num = __fadd_rn(__fmul_rn(fk, pc[e]), pd[e]);
        float qq = __fmul_rn(num, r_four_pi);
        qq = __fmaf_rn(__fmaf_rn(-qq, four_pi, num), r_four_pi, qq);
        pn[e] = qq;
        const float dd = qq - po[e];
        res += __fdividef(dd * dd, po[e] * po[e]);   // a diagnostic: fast quotient
      }
      *reinterpret_cast<float4 *>(x.q + gr * ldg + g) = nw;
    }
    res_acc += (double)res;
    __syncthreads();                           // the shared rows are read: next tile
    it = nx;
    cur_buf ^= 1;
  }
  // ---- teardown: with the products drained, free the tensor memory
  if (abort_flag && tid == 0) wait_phase(&bar, phase);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(x.tmem_cols)
                 : "memory");
  const double r = block_sum_tc(res_acc, sh);
  if (tid == 0) x.partials[blockIdx.x] = r;
  const double a = block_sum_tc(abs_acc, sh);
  if (tid == 0) x.partials[x.n_partials + blockIdx.x] = a;
  const double f = block_sum_tc(fis_acc, sh);
  if (tid == 0) x.partials[2 * x.n_partials + blockIdx.x] = f;
  if (blockIdx.x == 0)
    for (int i = (int)gridDim.x + tid; i < x.n_partials; i += TC_THREADS)
      x.partials[i] = x.partials[x.n_partials + i] = x.partials[2 * x.n_partials + i] = 0.0;
}

}  // namespace

// Launches the tensor-core update (partials only; update_finalize follows).
int moc_launch_update_tc(moc_problem *p) {
  const int kp = p->tc_kp, np = p->tc_np;
  if (!p->tc_b || kp == 0 || p->n_tc_items < 1) return MOC_ERR_UNSUPPORTED;
  const size_t smem = (size_t)tc_smem_bytes(kp, np, p->d.n_groups);
  // set outside any stream capture by the first call (the largest operands)
  static bool attr_set = false;
  if (!attr_set) {
    const size_t max_smem = (size_t)tc_smem_bytes(4 * TC_MAX_KG, MOC_TC_MAX_NP, 4 * TC_MAX_KG);
    MOC_CUDA_TRY(cudaFuncSetAttribute(update_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)max_smem));
    attr_set = true;
  }
  int sms = 0;
  MOC_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device));
  TcArgs x{};
  x.phi = p->phi;
  x.q = p->q;
  x.xs_order = p->xs_order;
  x.items = p->tc_items;
  x.n_items = p->n_tc_items;
  x.bmat = p->tc_b;
  x.xs = p->xs;
  x.scalars = p->scalars;
  x.partials = p->partials;
  x.err = p->err;
  x.n_partials = moc_post_scratch_blocks();
  x.F = p->d.fai;
  x.G = p->d.n_groups;
  x.ldg = p->ldg;
  x.kp = kp;
  x.np = np;
  x.acc_stride = 32;
  while ((int)x.acc_stride < np) x.acc_stride <<= 1;
  x.tmem_cols = 4 * x.acc_stride;                       // <= 512 (np <= 112)
  int grid = sms < p->n_tc_items ? sms : p->n_tc_items;
  if (grid > x.n_partials) grid = x.n_partials;
  update_tc_kernel<<<grid, TC_THREADS, smem, p->stream>>>(x);
  MOC_CUDA_TRY(cudaGetLastError());
  p->launches++;
  return MOC_OK;
}
