// moc_sweep.cu -- the transport-sweep kernel (replaces transport_sweep and
// attenuate_fluxes / attenuate_FSR_fluxes, src/solver.c:14-552).
//
// Mapping: a group of TPW threads owns one 3D track; thread `li` of the group
// owns the 4-group chunks li, li+TPW, ... (CPL of them) and keeps their angular
// flux in registers for the whole track.  The segment streams (3D length and
// source region) are read TPW entries at a time, one per thread, and broadcast
// with warp shuffles.  Per segment every thread gathers its chunks of the three
// neighbouring fine-source rows (one 16-byte load per row, not allocated in
// L1), forms the quadratic source, attenuates, and adds its tally chunk with a
// single vector reduction (red.global.add.v4.f32).  The grid is persistent:
// one wave of resident blocks walks all tracks.
//
// Modes:
//  PLAIN  every float operation of src/solver.c:38-279 in the reference order,
//         with no contraction; divisions by per-material or per-problem
//         constants use a correctly rounded quotient built from the precomputed
//         reciprocal (one FMA correction, Markstein), and the exponential comes
//         from the reference table (src/solver.c:1441-1464).  psi is
//         bit-identical to the reference's.
//  MIXED  contracted FP32 with reciprocals and an accurate 1-exp(-tau).
//  FP64   double state and arithmetic, exact 1-exp(-tau) (expm1).
#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <mutex>
#include <tuple>
#include <utility>

#include "moc_internal.h"

namespace {

constexpr int MODE_PLAIN = MOC_MODE_PLAIN;
constexpr int MODE_MIXED = MOC_MODE_MIXED;
constexpr int BLOCK = 256;
constexpr unsigned FULL = 0xffffffffu;

// a / b correctly rounded, given rb = RN(1/b): q = a*rb, r = a - b*q (exact),
// q + r*rb (P. Markstein, IBM J. Res. Dev. 34(1), 1990).
__device__ __forceinline__ float div_cr(float a, float b, float rb) {
  float q = __fmul_rn(a, rb);
  float r = __fmaf_rn(-q, b, a);
  return __fmaf_rn(r, rb, q);
}

__device__ __forceinline__ float4 ld_stream(const float *p) {
  float4 v;
  asm("ld.global.nc.L1::no_allocate.v4.f32 {%0,%1,%2,%3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "l"(p));
  return v;
}

__device__ __forceinline__ void red_add_v4(float *p, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1,%2,%3,%4};" ::"l"(p), "f"(a), "f"(b),
               "f"(c), "f"(d));
}

// L2 residency of the tallies.  Every tally is a read-modify-write of a
// scalar-flux line in L2, and one that finds its line resident saves both the
// DRAM read and the later write-back, while the fine-source rows (1 GB against
// a 129 MB L2) are read once per segment with no reuse to speak of.  MIXED
// therefore marks its tallies evict-last, which leaves the L2 to the scalar
// flux (233.7 against 239.3 ms on the 13.1 M-track default problem).  PLAIN,
// which issues more arithmetic per byte, measured 0.7 % slower with the hint
// and goes without it; an evict-first hint on the rows was slower in both.
__device__ __forceinline__ uint64_t l2_evict_last_policy() {
  uint64_t p;
  asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}

__device__ __forceinline__ void red_add_v4_last(float *p, float4 t, uint64_t pol) {
  asm volatile("red.global.add.L2::cache_hint.v4.f32 [%0], {%1,%2,%3,%4}, %5;" ::"l"(p),
               "f"(t.x), "f"(t.y), "f"(t.z), "f"(t.w), "l"(pol));
}
__device__ __forceinline__ void red_add_vec_last(float *p, float4 t, uint64_t pol) {
  red_add_v4_last(p, t, pol);
}
__device__ __forceinline__ void red_add_vec_last(float *p, float2 t, uint64_t pol) {
  asm volatile("red.global.add.L2::cache_hint.v2.f32 [%0], {%1,%2}, %3;" ::"l"(p), "f"(t.x),
               "f"(t.y), "l"(pol));
}
__device__ __forceinline__ void red_add_vec(float *p, float4 t) {
  red_add_v4(p, t.x, t.y, t.z, t.w);
}
__device__ __forceinline__ void red_add_vec(float *p, float2 t) {
  asm volatile("red.global.add.v2.f32 [%0], {%1,%2};" ::"l"(p), "f"(t.x), "f"(t.y));
}

__device__ __forceinline__ float get(const float4 &v, int e) {
  return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w;
}
__device__ __forceinline__ void set(float4 &v, int e, float x) {
  if (e == 0) v.x = x;
  else if (e == 1) v.y = x;
  else if (e == 2) v.z = x;
  else v.w = x;
}
__device__ __forceinline__ float get(const float2 &v, int e) { return e == 0 ? v.x : v.y; }
__device__ __forceinline__ void set(float2 &v, int e, float x) {
  if (e == 0) v.x = x;
  else v.y = x;
}

// A chunk of the group axis: VW = 4 consecutive groups (float4) or 2 (float2).
// Two-group chunks let a track of G groups fill lane counts that are not a
// power of two (100 groups: 10 lanes x 5 chunks, three tracks a warp).
template <int VW>
struct VecOf;
template <>
struct VecOf<4> {
  using T = float4;
};
template <>
struct VecOf<2> {
  using T = float2;
};

__device__ __forceinline__ void vzero(float4 &v) { v = make_float4(0.f, 0.f, 0.f, 0.f); }
__device__ __forceinline__ void vzero(float2 &v) { v = make_float2(0.f, 0.f); }

// Fine-source row loads.  L1A: allocate in L1, so that the loads of one row by
// several instructions (a row is 400 bytes at 100 groups, split across lanes
// and chunks at boundaries that need not fall on a 32-byte sector) meet in L1
// instead of each fetching the shared sectors.  Measured on the default
// problem: MIXED 234.6 -> 227.1 ms at 16 x 2 and 254 -> 226.7 ms at 10 x 5,
// PLAIN 311.5 -> 303.5 ms at 10 x 5; PLAIN at 16 x 2 was 1 % slower with it
// and goes without.
template <bool L1A>
__device__ __forceinline__ void ld_row_vec(const float *p, float4 &v) {
  if (L1A)
    asm("ld.global.nc.v4.f32 {%0,%1,%2,%3}, [%4];"
        : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
        : "l"(p));
  else
    v = ld_stream(p);
}
template <bool L1A>
__device__ __forceinline__ void ld_row_vec(const float *p, float2 &v) {
  if (L1A)
    asm("ld.global.nc.v2.f32 {%0,%1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p));
  else
    asm("ld.global.nc.L1::no_allocate.v2.f32 {%0,%1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p));
}
__device__ __forceinline__ void ldg_vec(const float *p, float4 &v) {
  v = __ldg(reinterpret_cast<const float4 *>(p));
}
__device__ __forceinline__ void ldg_vec(const float *p, float2 &v) {
  v = __ldg(reinterpret_cast<const float2 *>(p));
}

// 1 - exp(-tau) to ~1e-7 relative: Taylor series below 0.5, SFU exponential above.
__device__ __forceinline__ float one_minus_exp(float t) {
  // (1 - e^-t) / t = sum_k (-t)^k / (k+1)!, to degree 7: the first omitted
  // term is t^8 / 9! <= 1.1e-8 below t = 0.5
  float s = fmaf(t, 1.0f / 40320.0f, -1.0f / 5040.0f);
  s = fmaf(t, s, 1.0f / 720.0f);
  s = fmaf(t, s, -1.0f / 120.0f);
  s = fmaf(t, s, 1.0f / 24.0f);
  s = fmaf(t, s, -1.0f / 6.0f);
  s = fmaf(t, s, 0.5f);
  s = fmaf(t, -s, 1.0f);
  float small = t * s;
  float big = 1.0f - __expf(-t);
  return t < 0.5f ? small : big;
}

struct Seg {
  float zin;      // height within the fitted interval (after edge shift)
  int mat;        // sigma_t row of the source region
  int64_t qrow;   // first of the three fine-source rows (quadratic) or the row (flat)
  int64_t frow;   // tally row
  int64_t crow;   // coefficient block
};

// FMA_ZIN (MIXED and the adjoint): the height within the fitted interval in one
// rounding, zin = RN(z - dz (centre)), with the edge shift folded into the
// centre.  The reference's float expression (PLAIN) rounds the product
// dz (zi + 1/2) of a height of up to the domain's (hundreds of cm) and then the
// difference and the shift: an absolute error of ~1e-5 cm in a zin of a few cm,
// which reaches the quadratic fit's q0 and q1 at ~1e-6 relative and was the
// largest error of the MIXED sweep against FP64.
template <bool FMA_ZIN = false>
__device__ __forceinline__ Seg segment_geometry(const SweepArgs &a, float z, int s) {
  Seg g;
  // src/solver.c:38-45 (z / dz once: both uses are the same expression)
  int zi = __float2int_rz(div_cr(z, a.dz, a.rdz));
  const float centre = __fadd_rn(__int2float_rn(zi), 0.5f);      // exact below 2^23
  float zin = FMA_ZIN ? 0.f : __fsub_rn(z, __fmul_rn(a.dz, centre));
  // zi % F by a multiply-high; the host verified the magic over every reachable zi
  int fine = a.fmagic ? zi - a.F * (int)__umulhi((unsigned)zi, a.fmagic) : zi % a.F;
  int r0 = fine;
  float shift = 0.f;
  if (a.axial_exp == 2) {
    if (fine == 0) {                     // src/solver.c:55-58
      if (!FMA_ZIN) zin = __fsub_rn(zin, a.dz);
      shift = 1.f;
      r0 = 0;
    } else if (fine == a.F - 1) {        // src/solver.c:84-87
      if (!FMA_ZIN) zin = __fadd_rn(zin, a.dz);
      shift = -1.f;
      r0 = fine - 2;
    } else {
      r0 = fine - 1;
    }
  }
  if (FMA_ZIN) zin = __fmaf_rn(-a.dz, __fadd_rn(centre, shift), z);
  g.zin = zin;
  int64_t base = (int64_t)s * a.F;
  g.qrow = (base + r0) * a.ldg;
  g.frow = (base + fine) * a.ldg;
  g.mat = __ldg(a.src_sigt + s);
  g.crow = (int64_t)g.mat * COEF_PLANES * a.ldg;
  return g;
}

__device__ __forceinline__ float advance_z(const SweepArgs &a, float z, float ds, float mu) {
  z = __fadd_rn(z, __fmul_rn(ds, mu));
  // |ds*mu| < domain height is checked at upload, so one pass of each suffices;
  // the bound keeps the loop finite whatever the input.
#pragma unroll 1
  for (int it = 0; it < 4 && z >= a.hd; ++it) z = __fsub_rn(z, a.hd);
#pragma unroll 1
  for (int it = 0; it < 4 && z < 0.0f; ++it) z = __fadd_rn(z, a.hd);
  return z;
}

// ---- MIXED arithmetic, quadratic source
// The fit q(z) = q0 + q1 (z - zin) + q2 (z - zin)^2 of the three fine sources
// y1, y2, y3 (src/solver.c:69-81) with d1 = y1 - y3, d2 = y1 - 2 y2 + y3:
//   q0 = y2 + d1 zin/(2dz) + d2 zin^2/(2dz^2),
//   q1 mu = d1 mu/(2dz) + d2 (2 mu zin)/(2dz^2),   q2 mu^2 = d2 mu^2/(2dz^2).
// The factors that depend only on the track (mu) and the segment (zin) are
// formed once per segment (MixedFit), not once per group.
struct MixedFit {
  float a1, a0;        // zin/(2dz), zin^2/(2dz^2)
  float b1, b2;        // mu/(2dz), 2 mu zin/(2dz^2)
  float c2m;           // mu^2/(2dz^2)
};

__device__ __forceinline__ MixedFit mixed_fit(const SweepArgs &a, float zin, float mu,
                                              float mu2) {
  MixedFit f;
  f.a1 = a.rd1 * zin;
  f.a0 = a.rd2 * zin * zin;
  f.b1 = mu * a.rd1;
  f.b2 = 2.f * mu * a.rd2 * zin;
  f.c2m = mu2 * a.rd2;
  return f;
}

// The flux integral fi and the outgoing psi (src/solver.c:195-278) are both
// linear in (q0, q1 mu, q2 mu^2, psi) with weights that depend on tau only:
//   fi = q0 T + psi U + q1mu R + q2mu2 C/(3 sig^4)
//   pn = q0 U + q1mu T + q2mu2 R + psi (1 - E)
// with E = 1 - e^-tau, T = (tau - E)/sig^2, U = E/sig and the reference's
// reuse term R = tau (tau - 2) + 2E/sig^3 (its precedence kept, as PLAIN).
// r1, r2, r3x2, r4 are the coefficient planes 1/sig, 1/sig^2, 2/sig^3,
// 1/(3 sig^4).
__device__ __forceinline__ float mixed_quad_e(float y1, float y2, float y3, const MixedFit &f,
                                              float sig, float r1, float r2, float r3x2,
                                              float r4, float ds, float w, float &p, float &Eo) {
  const float d1 = y1 - y3;
  const float d2 = fmaf(-2.f, y2, y1) + y3;
  const float q0 = fmaf(d2, f.a0, fmaf(d1, f.a1, y2));
  const float q1mu = fmaf(d2, f.b2, d1 * f.b1);
  const float q2mu2 = d2 * f.c2m;
  const float tau = sig * ds;
  const float E = one_minus_exp(tau);
  const float T = (tau - E) * r2;
  const float U = E * r1;
  const float R = fmaf(E, r3x2, tau * (tau - 2.f));
  const float Cr = fmaf(tau, fmaf(tau, tau - 3.f, 6.f), -6.f * E) * r4;
  const float fi = fmaf(q0, T, fmaf(p, U, fmaf(q1mu, R, q2mu2 * Cr)));
  p = fmaf(q0, U, fmaf(q1mu, T, fmaf(q2mu2, R, p * (1.f - E))));
  Eo = E;
  return w * fi;
}


__device__ __forceinline__ float mixed_flat(float y, float sig, float r1, float ds, float w_mu,
                                            float &p) {
  float e = one_minus_exp(sig * ds);
  float dpsi = (p - y * r1) * e;
  p -= dpsi;
  return w_mu * dpsi;
}

// ---- packed pairs of groups.  sm_100 and later issue one FP32 FMA, multiply
// or add on two lanes at once (__ffma2_rn, __fmul2_rn, __fadd2_rn), each lane
// rounded as __fmaf_rn / __fmul_rn / __fadd_rn (a - b is written fma(b, -1, a):
// one rounding of the same difference).  Pairs halve the instructions but also
// the independent chains a thread has in flight, so they pay only where issue
// slots, not latency, bound a loop (the adjoint's reverse pass).
__device__ __forceinline__ float2 bc2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 lo2(const float4 &v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(const float4 &v) { return make_float2(v.z, v.w); }
__device__ __forceinline__ float4 cat4(float2 l, float2 h) { return make_float4(l.x, l.y, h.x, h.y); }

// MixedFit with every factor on both lanes
struct MixedFit2 {
  float2 a1, a0, b1, b2, c2m;
};
__device__ __forceinline__ MixedFit2 pair_fit(const MixedFit &f) {
  return MixedFit2{bc2(f.a1), bc2(f.a0), bc2(f.b1), bc2(f.b2), bc2(f.c2m)};
}

// ---- PLAIN: the reference's float arithmetic, operation for operation, on
// two groups at once.  Each of its operations is one rounding, and the packed
// pair FMA rounds each lane as __fmaf_rn, so every product, sum and difference
// is an FMA with a runtime 1, -1 or -0 (RN(a b + -0) = RN(a b), RN(a 1 + b) =
// RN(a + b), RN(b (-1) + a) = RN(a - b), signed zeros included).  Plain pair
// multiplies and adds would be legal for the compiler to contract into one
// FMA, which the reference never does.  A divisor enters div_cr only as -b in
// fma(-q, b, a) = fma(q, -b, a), so the pair forms carry the negated divisors
// (-sig, -sig^2, -sig^3, -3 sig^4, formed with the reference's roundings:
// RN(-x) = -RN(x)).
struct Exact2 {
  float2 one, m1, nz;
};
__device__ __forceinline__ Exact2 exact2(const SweepArgs &a) {
  return Exact2{bc2(a.rt_one), bc2(a.rt_m1), bc2(a.rt_nz)};
}
__device__ __forceinline__ float2 xmul(const Exact2 &k, float2 a, float2 b) { return fma2(a, b, k.nz); }
__device__ __forceinline__ float2 xadd(const Exact2 &k, float2 a, float2 b) { return fma2(a, k.one, b); }
__device__ __forceinline__ float2 xsub(const Exact2 &k, float2 a, float2 b) { return fma2(b, k.m1, a); }
// div_cr on two lanes
__device__ __forceinline__ float2 xdiv(const Exact2 &k, float2 a, float2 nb, float2 rb) {
  const float2 q = xmul(k, a, rb);
  return fma2(fma2(q, nb, a), rb, q);
}

// The reference's interpolation table (src/solver.c:1441-1464) on two lanes.
__device__ __forceinline__ float2 table_lookup2(const SweepArgs &a, const Exact2 &k,
                                                const float2 *tab, float2 x) {
  const float2 f = xadd(k, xdiv(k, x, bc2(-a.table_dx), bc2(a.table_rdx)), bc2(a.table_halfdx));
  const int i0 = max(0, min(__float2int_rz(f.x), a.table_n - 1));
  const int i1 = max(0, min(__float2int_rz(f.y), a.table_n - 1));
  const float2 s0 = tab[i0], s1 = tab[i1];
  const float2 v = xadd(k, xmul(k, make_float2(s0.x, s1.x), x), make_float2(s0.y, s1.y));
  return make_float2(x.x > a.table_maxval ? 1.0f : v.x, x.y > a.table_maxval ? 1.0f : v.y);
}

// quadratic source, src/solver.c:74-278
__device__ __forceinline__ float2 plain_quad_v(const SweepArgs &a, const float2 *tab, float2 y1,
                                               float2 y2, float2 y3, float2 sig, float2 r1,
                                               float2 r2, float2 r3, float2 r4, float2 zin,
                                               float2 ds, float2 mu, float2 mu2, float2 w,
                                               float2 &p) {
  const Exact2 k = exact2(a);
  const float2 two = bc2(2.f);
  // the reference's divisors (solver.c:153, 176, 198), negated
  const float2 nsg = xmul(k, sig, k.m1);
  const float2 nsg2 = xmul(k, nsg, sig);
  const float2 nsg3 = xmul(k, sig, nsg2);
  const float2 nsg4 = xmul(k, xmul(k, bc2(-3.f), nsg2), nsg2);
  const float2 c0 = y2;
  const float2 c1 = xdiv(k, xsub(k, y1, y3), bc2(-a.d1), bc2(a.rd1));
  const float2 c2 =
      xdiv(k, xadd(k, xsub(k, y1, xmul(k, two, y2)), y3), bc2(-a.d2), bc2(a.rd2));
  const float2 q0 = xadd(k, xadd(k, c0, xmul(k, c1, zin)), xmul(k, xmul(k, c2, zin), zin));
  const float2 q1 = xadd(k, c1, xmul(k, xmul(k, two, c2), zin));
  const float2 q2 = c2;
  const float2 tau = xmul(k, sig, ds);
  const float2 e = table_lookup2(a, k, tab, tau);
  const float2 reuse =
      xadd(k, xmul(k, tau, xsub(k, tau, two)), xdiv(k, xmul(k, two, e), nsg3, r3));
  const float2 A = xdiv(
      k, xadd(k, xmul(k, q0, tau), xmul(k, xsub(k, xmul(k, sig, p), q0), e)), nsg2, r2);
  const float2 q1mu = xmul(k, q1, mu);
  const float2 B = xmul(k, q1mu, reuse);
  const float2 cub = xsub(k, xmul(k, tau, xadd(k, xmul(k, tau, xsub(k, tau, bc2(3.f))), bc2(6.f))),
                          xmul(k, bc2(6.f), e));
  const float2 q2mu2 = xmul(k, q2, mu2);
  const float2 C = xdiv(k, xmul(k, q2mu2, cub), nsg4, r4);
  const float2 fi = xadd(k, xadd(k, A, B), C);
  const float2 t1 = xdiv(k, xmul(k, q0, e), nsg, r1);
  const float2 t2 = xdiv(k, xmul(k, q1mu, xsub(k, tau, e)), nsg2, r2);
  const float2 t3 = xmul(k, q2mu2, reuse);
  const float2 t4 = xmul(k, p, xsub(k, k.one, e));
  p = xadd(k, xadd(k, xadd(k, t1, t2), t3), t4);
  return xmul(k, w, fi);
}
__device__ __forceinline__ float4 plain_quad_v(const SweepArgs &a, const float2 *tab, float4 y1,
                                               float4 y2, float4 y3, float4 sig, float4 r1,
                                               float4 r2, float4 r3, float4 r4, float2 zin,
                                               float2 ds, float2 mu, float2 mu2, float2 w,
                                               float4 &p) {
  float2 pl = lo2(p), ph = hi2(p);
  const float2 tl = plain_quad_v(a, tab, lo2(y1), lo2(y2), lo2(y3), lo2(sig), lo2(r1), lo2(r2),
                                 lo2(r3), lo2(r4), zin, ds, mu, mu2, w, pl);
  const float2 th = plain_quad_v(a, tab, hi2(y1), hi2(y2), hi2(y3), hi2(sig), hi2(r1), hi2(r2),
                                 hi2(r3), hi2(r4), zin, ds, mu, mu2, w, ph);
  p = cat4(pl, ph);
  return cat4(tl, th);
}

// flat source, src/solver.c:1075-1115
__device__ __forceinline__ float2 plain_flat_v(const SweepArgs &a, const float2 *tab, float2 y,
                                               float2 sig, float2 r1, float2 ds, float2 w_mu,
                                               float2 &p) {
  const Exact2 k = exact2(a);
  const float2 e = table_lookup2(a, k, tab, xmul(k, sig, ds));
  const float2 qq = xdiv(k, y, xmul(k, sig, k.m1), r1);
  const float2 dpsi = xmul(k, xsub(k, p, qq), e);
  p = xsub(k, p, dpsi);
  return xmul(k, w_mu, dpsi);
}
__device__ __forceinline__ float4 plain_flat_v(const SweepArgs &a, const float2 *tab, float4 y,
                                               float4 sig, float4 r1, float2 ds, float2 w_mu,
                                               float4 &p) {
  float2 pl = lo2(p), ph = hi2(p);
  const float2 tl = plain_flat_v(a, tab, lo2(y), lo2(sig), lo2(r1), ds, w_mu, pl);
  const float2 th = plain_flat_v(a, tab, hi2(y), hi2(sig), hi2(r1), ds, w_mu, ph);
  p = cat4(pl, ph);
  return cat4(tl, th);
}

// one_minus_exp on two lanes
__device__ __forceinline__ float2 one_minus_exp2(float2 t) {
  float2 s = fma2(t, bc2(1.0f / 40320.0f), bc2(-1.0f / 5040.0f));
  s = fma2(t, s, bc2(1.0f / 720.0f));
  s = fma2(t, s, bc2(-1.0f / 120.0f));
  s = fma2(t, s, bc2(1.0f / 24.0f));
  s = fma2(t, s, bc2(-1.0f / 6.0f));
  s = fma2(t, s, bc2(0.5f));
  const float2 nt = mul2(t, bc2(-1.0f));
  s = fma2(nt, s, bc2(1.0f));                 // 1 - t s
  const float2 small = mul2(t, s);
  return make_float2(t.x < 0.5f ? small.x : 1.0f - __expf(nt.x),
                     t.y < 0.5f ? small.y : 1.0f - __expf(nt.y));
}

// mixed_quad_e's tally and psi on two groups, operation for operation: the
// same bits (the sweeps run this; the adjoint's recomputation, which also
// keeps E, runs mixed_quad_e)
__device__ __forceinline__ float2 mixed_quad_v(float2 y1, float2 y2, float2 y3,
                                               const MixedFit2 &f, float2 sig, float2 r1,
                                               float2 r2, float2 r3x2, float2 r4, float2 ds,
                                               float2 w, float2 &p) {
  const float2 m1 = bc2(-1.f);
  const float2 d1 = fma2(y3, m1, y1);
  const float2 d2 = add2(fma2(bc2(-2.f), y2, y1), y3);
  const float2 q0 = fma2(d2, f.a0, fma2(d1, f.a1, y2));
  const float2 q1mu = fma2(d2, f.b2, mul2(d1, f.b1));
  const float2 q2mu2 = mul2(d2, f.c2m);
  const float2 tau = mul2(sig, ds);
  const float2 E = one_minus_exp2(tau);
  const float2 T = mul2(fma2(E, m1, tau), r2);
  const float2 U = mul2(E, r1);
  const float2 R = fma2(E, r3x2, mul2(tau, add2(tau, bc2(-2.f))));
  const float2 Cr =
      mul2(fma2(tau, fma2(tau, add2(tau, bc2(-3.f)), bc2(6.f)), mul2(bc2(-6.f), E)), r4);
  const float2 fi = fma2(q0, T, fma2(p, U, fma2(q1mu, R, mul2(q2mu2, Cr))));
  p = fma2(q0, U, fma2(q1mu, T, fma2(q2mu2, R, mul2(p, fma2(E, m1, bc2(1.f))))));
  return mul2(w, fi);
}
// four groups as two pairs
__device__ __forceinline__ float4 mixed_quad_v(float4 y1, float4 y2, float4 y3,
                                               const MixedFit2 &f, float4 sig, float4 r1,
                                               float4 r2, float4 r3x2, float4 r4, float2 ds,
                                               float2 w, float4 &p) {
  float2 pl = lo2(p), ph = hi2(p);
  const float2 tl = mixed_quad_v(lo2(y1), lo2(y2), lo2(y3), f, lo2(sig), lo2(r1), lo2(r2),
                                 lo2(r3x2), lo2(r4), ds, w, pl);
  const float2 th = mixed_quad_v(hi2(y1), hi2(y2), hi2(y3), f, hi2(sig), hi2(r1), hi2(r2),
                                 hi2(r3x2), hi2(r4), ds, w, ph);
  p = cat4(pl, ph);
  return cat4(tl, th);
}

// The rounding error of old + x (TwoSum, Knuth): exact in round-to-nearest.
__device__ __forceinline__ float two_sum_err(float old, float x) {
  const float s = __fadd_rn(old, x);
  const float bp = __fsub_rn(s, old);
  return __fadd_rn(__fsub_rn(old, __fsub_rn(s, bp)), __fsub_rn(x, bp));
}

// A chunk of compensated tallies: one vector atomic that returns the old hi
// words (atom.global.v4/.v2.f32, sm_90 and later), the TwoSum errors of the
// chunk's additions, and one vector reduction of them into the lo words.  The
// hi additions are the same single-rounding additions as the plain tallies;
// the lo words collect what each of them rounded away.
__device__ __forceinline__ void comp_add_vec(float *hi, float *lo, float4 t) {
  float4 o;
  asm volatile("atom.global.v4.f32.add {%0,%1,%2,%3}, [%4], {%5,%6,%7,%8};"
               : "=f"(o.x), "=f"(o.y), "=f"(o.z), "=f"(o.w)
               : "l"(hi), "f"(t.x), "f"(t.y), "f"(t.z), "f"(t.w)
               : "memory");
  red_add_v4(lo, two_sum_err(o.x, t.x), two_sum_err(o.y, t.y), two_sum_err(o.z, t.z),
             two_sum_err(o.w, t.w));
}
__device__ __forceinline__ void comp_add_vec(float *hi, float *lo, float2 t) {
  float2 o;
  asm volatile("atom.global.v2.f32.add {%0,%1}, [%2], {%3,%4};"
               : "=f"(o.x), "=f"(o.y)
               : "l"(hi), "f"(t.x), "f"(t.y)
               : "memory");
  asm volatile("red.global.add.v2.f32 [%0], {%1,%2};" ::"l"(lo), "f"(two_sum_err(o.x, t.x)),
               "f"(two_sum_err(o.y, t.y)));
}

// The returning vector atomic of a compensated chunk: the old hi words.
__device__ __forceinline__ float4 atom_add_vec(float *hi, float4 t) {
  float4 o;
  asm volatile("atom.global.v4.f32.add {%0,%1,%2,%3}, [%4], {%5,%6,%7,%8};"
               : "=f"(o.x), "=f"(o.y), "=f"(o.z), "=f"(o.w)
               : "l"(hi), "f"(t.x), "f"(t.y), "f"(t.z), "f"(t.w)
               : "memory");
  return o;
}
__device__ __forceinline__ float2 atom_add_vec(float *hi, float2 t) {
  float2 o;
  asm volatile("atom.global.v2.f32.add {%0,%1}, [%2], {%3,%4};"
               : "=f"(o.x), "=f"(o.y)
               : "l"(hi), "f"(t.x), "f"(t.y)
               : "memory");
  return o;
}
__device__ __forceinline__ float4 two_sum_err(float4 o, float4 t) {
  return make_float4(two_sum_err(o.x, t.x), two_sum_err(o.y, t.y), two_sum_err(o.z, t.z),
                     two_sum_err(o.w, t.w));
}
__device__ __forceinline__ float2 two_sum_err(float2 o, float2 t) {
  return make_float2(two_sum_err(o.x, t.x), two_sum_err(o.y, t.y));
}

// Loads of one segment that are issued one segment ahead (software pipeline):
// the three fine-source rows (one row for the flat source) of every chunk.
template <int CPL, bool QUAD, int VW = 4>
struct Rows {
  typename VecOf<VW>::T v[CPL][QUAD ? 3 : 1];
};

// nch = chunks of VW groups in a row (ldg / VW).
template <int CPL, bool QUAD, int VW, bool L1A>
__device__ __forceinline__ void load_rows(const SweepArgs &a, const Seg &g, int li, int TPW,
                                          Rows<CPL, QUAD, VW> &r, int nch) {
#pragma unroll
  for (int k = 0; k < CPL; ++k) {
    const int c = li + TPW * k;
    if (c < nch) {
      const float *qr = a.q + g.qrow + VW * c;
      ld_row_vec<L1A>(qr, r.v[k][0]);
      if (QUAD) {
        ld_row_vec<L1A>(qr + a.ldg, r.v[k][QUAD ? 1 : 0]);
        ld_row_vec<L1A>(qr + 2 * a.ldg, r.v[k][QUAD ? 2 : 0]);
      }
    }
  }
}

__device__ __forceinline__ int checked_source(const SweepArgs &a, int s, int li) {
  if ((uint32_t)s >= (uint64_t)a.ns) {   // the ids of a streamed upload are checked here
    if (li == 0) atomicOr(a.err, MOC_DEV_ERR_SOURCE);
    return 0;
  }
  return s;
}

// CSR: the tracks' segment streams are variable-length (the reference
// traversal's sub-segments, csr_off/csr_ds/csr_z/csr_src) with the start height
// of every sub-segment given; otherwise every track has S segments and its
// height advances by ds*mu.  With several CSR tracks in a warp the warp runs
// to its longest track: the stream shuffles and the geometry stay warp-uniform,
// and a track past its end skips the arithmetic and the tallies.
// One 3D track (or one group of TPW lanes' track) of the sweep.  TPW_CT is
// the threads per track when known at compile time; 0 takes tpw_rt (the
// batched kernel, where each core has its own width).
template <int TPW_CT, int CPL, int MODE, bool QUAD, bool CSR, bool CKPT = false, int VW = 4,
          bool REC = false, bool COMP = false>
__device__ __forceinline__ void sweep_track(const SweepArgs &a, int64_t track, int lane,
                                            int tpw_rt, const float2 *s_table) {
  const int TPW = TPW_CT ? TPW_CT : tpw_rt;
  const int li = lane % TPW;
  const int gb = lane - li;              // the track's first lane
  // lane k of the track: a width-TPW shuffle for power-of-two widths, the
  // absolute lane gb + k otherwise
  constexpr bool POW2 = TPW_CT > 0 && (TPW_CT & (TPW_CT - 1)) == 0;
  auto tshfl = [&](auto v, int k) {
    return (POW2 || TPW_CT == 0) ? __shfl_sync(FULL, v, k, TPW) : __shfl_sync(FULL, v, gb + k);
  };
  using V = typename VecOf<VW>::T;
  constexpr bool L1A = MODE == MODE_MIXED || VW == 2;   // row loads allocate in L1
  const int nch = VW == 4 ? a.nchunk : a.ldg / VW;   // chunks of VW groups in a row
  const int64_t PZ = (int64_t)a.P * a.Z;
  const bool valid = track < a.n3d;
  const int64_t tr = valid ? track : a.n3d - 1;
  const int64_t i2 = tr / PZ;
  const int j = (int)((tr / a.Z) % a.P);
  const float mu = a.mu[j];
  const float mu2 = __fmul_rn(mu, mu);
  const float w = a.weight[tr];
  const float w_mu = __fmul_rn(w, mu);
  float z;
  int S;
  const float *dsb;
  const int32_t *srcb;
  const float *zb = nullptr;
  if (CSR) {
    const int64_t o0 = a.csr_off[tr];
    S = (int)(a.csr_off[tr + 1] - o0);
    dsb = a.csr_ds + o0;
    srcb = a.csr_src + o0;
    zb = a.csr_z + o0;
    z = 0.f;
  } else {
    S = a.S;
    z = a.z0[tr];
    dsb = a.seg_ds + (i2 * a.P + j) * S;
    srcb = a.seg_src + tr * S;
  }

  V psi[CPL];
#pragma unroll
  for (int k = 0; k < CPL; ++k) {
    const int c = li + TPW * k;
    vzero(psi[k]);
    if (c < nch) psi[k] = *reinterpret_cast<const V *>(a.psi + tr * a.ldg + VW * c);
    if (a.psi_scale) {                    // renormalisation still to apply (src/solver.c:1224)
      const float sc = *a.psi_scale;
#pragma unroll
      for (int e = 0; e < VW; ++e) set(psi[k], e, __fmul_rn(get(psi[k], e), sc));
    }
  }

  // segment streams: the current chunk of TPW entries and the next one
  float ds_c = li < S ? __ldg(dsb + li) : 0.f;
  int src_c = li < S ? __ldg(srcb + li) : 0;
  float ds_n = TPW + li < S ? __ldg(dsb + TPW + li) : 0.f;
  int src_n = TPW + li < S ? __ldg(srcb + TPW + li) : 0;
  float z_c = 0.f, z_n = 0.f;
  if (CSR) {
    z_c = li < S ? __ldg(zb + li) : 0.f;
    z_n = TPW + li < S ? __ldg(zb + TPW + li) : 0.f;
    z = tshfl(z_c, 0);
  }

  float ds = tshfl(ds_c, 0);
  Seg g = segment_geometry<MODE == MODE_MIXED>(a, z, checked_source(a, tshfl(src_c, 0), li));
  int S_loop = S;                        // the warp's longest track (CSR, several a warp)
  if (CSR && TPW < 32) S_loop = (int)__reduce_max_sync(FULL, (unsigned)S);
  const uint64_t tally_pol = MODE == MODE_MIXED ? l2_evict_last_policy() : 0;
  Rows<CPL, QUAD, VW> rows;
  if (S_loop > 0) load_rows<CPL, QUAD, VW, L1A>(a, g, li, TPW, rows, nch);

  // COMP: the compensation of each chunk's tallies waits one segment, so that
  // the returning atomic's old values arrive under the next segment's work
  V pend_o[COMP ? CPL : 1], pend_t[COMP ? CPL : 1];
  int64_t pend_off[COMP ? CPL : 1];
#pragma unroll
  for (int k = 0; k < (COMP ? CPL : 1); ++k) pend_off[k] = -1;
  int ck_left = 0;                       // segments to the next checkpoint
  int64_t ck_slot = CKPT ? tr * a.ck_n : 0;
  for (int n = 0; n < S_loop; ++n) {
    const bool live = n < S;             // false only past a CSR track's end
    if (CKPT && ck_left-- == 0) {
      // angular flux and height entering segment n (n a multiple of ck_k),
      // for the reverse sweep
      ck_left = a.ck_k - 1;
      if (valid) {
#pragma unroll
        for (int k = 0; k < CPL; ++k) {
          const int c = li + TPW * k;
          if (c < nch) *reinterpret_cast<V *>(a.ck_psi + ck_slot * a.ldg + VW * c) = psi[k];
        }
        if (li == 0) a.ck_z[ck_slot] = z;
      }
      ++ck_slot;
    }
    float z_next = CSR ? 0.f : advance_z(a, z, ds, mu);
    // ---- issue the loads of segment n+1 before the arithmetic of segment n
    float ds1 = 0.f;
    Seg g1 = g;
    Rows<CPL, QUAD, VW> rows1 = rows;
    const int m = n + 1;
    if (m < S_loop) {
      const int k = (POW2 || TPW_CT == 0) ? (m & (TPW - 1)) : m % TPW;
      if (k == 0) {
        ds_c = ds_n;
        src_c = src_n;
        const int nl = m + TPW + li;
        ds_n = nl < S ? __ldg(dsb + nl) : 0.f;
        src_n = nl < S ? __ldg(srcb + nl) : 0;
        if (CSR) {
          z_c = z_n;
          z_n = nl < S ? __ldg(zb + nl) : 0.f;
        }
      }
      if (CSR) z_next = tshfl(z_c, k);
      ds1 = tshfl(ds_c, k);
      g1 = segment_geometry<MODE == MODE_MIXED>(a, z_next, checked_source(a, tshfl(src_c, k), li));
      load_rows<CPL, QUAD, VW, L1A>(a, g1, li, TPW, rows1, nch);
    }
    // ---- segment n
    const MixedFit fit = (MODE == MODE_MIXED && QUAD) ? mixed_fit(a, g.zin, mu, mu2) : MixedFit{};
    const MixedFit2 fit2 = pair_fit(fit);
#pragma unroll
    for (int k = 0; k < CPL; ++k) {
      const int c = li + TPW * k;
      if (c >= nch || !live) continue;
      const int g4 = VW * c;                                      // first group of the chunk
      // this chunk's planes: the 4-group block holding it, offset within the block
      const float *cf = VW == 4 ? a.coef + g.crow + 4 * COEF_PLANES * c
                                : a.coef + g.crow + 4 * COEF_PLANES * (c >> 1) + 2 * (c & 1);
      V sig, r1;
      ldg_vec(cf, sig);
      ldg_vec(cf + 4, r1);
      V t;
      if (QUAD) {
        const V y1 = rows.v[k][0];
        const V y2 = rows.v[k][QUAD ? 1 : 0];
        const V y3 = rows.v[k][QUAD ? 2 : 0];
        if (MODE == MODE_PLAIN) {
          V r2, r3, r4;
          ldg_vec(cf + 8, r2);
          ldg_vec(cf + 12, r3);
          ldg_vec(cf + 16, r4);
          // groups in packed pairs, the reference's roundings
          t = plain_quad_v(a, s_table, y1, y2, y3, sig, r1, r2, r3, r4, bc2(g.zin), bc2(ds),
                           bc2(mu), bc2(mu2), bc2(w), psi[k]);
        } else {
          V r2, r4, r3x2;
          ldg_vec(cf + 8, r2);
          ldg_vec(cf + 16, r4);
          ldg_vec(cf + 20, r3x2);
          // groups in packed pairs: mixed_quad_e's bits
          t = mixed_quad_v(y1, y2, y3, fit2, sig, r1, r2, r3x2, r4, bc2(ds), bc2(w), psi[k]);
        }
      } else {
        const V y = rows.v[k][0];
        if (MODE == MODE_PLAIN) {
          t = plain_flat_v(a, s_table, y, sig, r1, bc2(ds), bc2(w_mu), psi[k]);
        } else {
#pragma unroll
          for (int e = 0; e < VW; ++e) {
            float p = get(psi[k], e);
            set(t, e, mixed_flat(get(y, e), get(sig, e), get(r1, e), ds, w_mu, p));
            set(psi[k], e, p);
          }
        }
      }
      if (REC) {
        // deterministic-order tallies: the contribution goes to the track's
        // record slot (segment n of track tr), its FSR row beside it; an ordered
        // reduction adds the records to the flux later
        if (valid) {
          const int64_t slot = tr * a.S + n;
          *reinterpret_cast<V *>(a.rec + slot * a.ldg + g4) = t;
          if (c == 0) a.rec_row[slot] = (int32_t)(g.frow / a.ldg);
        }
      } else if (COMP) {
        if (valid) {
          const int64_t off = g.frow + g4;
          const V o = atom_add_vec(a.phi + off, t);
          if (pend_off[k] >= 0) red_add_vec(a.phi_lo + pend_off[k], two_sum_err(pend_o[k], pend_t[k]));
          pend_o[k] = o;
          pend_t[k] = t;
          pend_off[k] = off;
        }
      } else if (valid) {
        float *dst = a.phi + g.frow + g4;
        if (MODE == MODE_MIXED) {
          red_add_vec_last(dst, t, tally_pol);
        } else {
          red_add_vec(dst, t);
        }
      }
    }
    z = z_next;
    ds = ds1;
    g = g1;
    rows = rows1;
  }
  if (COMP) {
#pragma unroll
    for (int k = 0; k < (COMP ? CPL : 1); ++k)
      if (pend_off[k] >= 0) red_add_vec(a.phi_lo + pend_off[k], two_sum_err(pend_o[k], pend_t[k]));
  }
  if (valid) {
#pragma unroll
    for (int k = 0; k < CPL; ++k) {
      const int c = li + TPW * k;
      if (c < nch) *reinterpret_cast<V *>(a.psi + tr * a.ldg + VW * c) = psi[k];
    }
  }
}

// With TPW not dividing 32 the last 32 % TPW lanes own no track: they run the
// loop on an out-of-range track (loads clamped to a real one, no stores) so that
// the warp's shuffles stay converged.
template <int TPW, int CPL, int MODE, bool QUAD, bool CSR, bool CKPT, int VW, bool REC = false,
          bool COMP = false>
__device__ __forceinline__ void sweep_body(const SweepArgs &a, float2 *s_table) {
  if (MODE == MODE_PLAIN) {
    for (int i = threadIdx.x; i < a.table_n; i += BLOCK) s_table[i] = a.table[i];
    __syncthreads();
  }
  constexpr int GPW = 32 / TPW;
  const int lane = threadIdx.x & 31;
  const int gw = lane / TPW;
  const int64_t warp_id = ((int64_t)blockIdx.x * BLOCK + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * BLOCK) >> 5;
  for (int64_t base = warp_id * GPW; base < a.n3d; base += n_warps * GPW)
    sweep_track<TPW, CPL, MODE, QUAD, CSR, CKPT, VW, REC, COMP>(a, gw < GPW ? base + gw : a.n3d, lane,
                                                          TPW, s_table);
}

template <int TPW, int CPL, int MODE, bool QUAD, bool CSR = false, bool CKPT = false>
__global__ void __launch_bounds__(BLOCK) sweep_kernel(SweepArgs a) {
  extern __shared__ float2 s_table[];
  sweep_body<TPW, CPL, MODE, QUAD, CSR, CKPT, 4>(a, s_table);
}

// The sweep with recorded tallies (deterministic-order mode): every segment's
// contribution is stored, not added.
template <int TPW, int CPL, int MODE, bool QUAD>
__global__ void __launch_bounds__(BLOCK) sweep_record_kernel(SweepArgs a) {
  extern __shared__ float2 s_table[];
  sweep_body<TPW, CPL, MODE, QUAD, false, false, 4, true>(a, s_table);
}

// MIXED with compensated tallies (MOC_FLAG_COMPENSATED): the hi words by a
// returning vector atomic, their rounding errors one segment later into the lo
// words (four-group chunks).
template <int TPW, int CPL, bool QUAD>
__global__ void __launch_bounds__(BLOCK) sweep_comp_kernel(SweepArgs a) {
  extern __shared__ float2 s_table[];
  sweep_body<TPW, CPL, MODE_MIXED, QUAD, false, false, 4, false, true>(a, s_table);
}

// Two-group chunks: held to two blocks an SM (the MIXED quadratic variant
// would otherwise take 139 registers and run one).
template <int TPW, int CPL, int MODE, bool QUAD, bool CSR = false, bool CKPT = false>
__global__ void __launch_bounds__(BLOCK, 2) sweep_kernel_v2(SweepArgs a) {
  extern __shared__ float2 s_table[];
  sweep_body<TPW, CPL, MODE, QUAD, CSR, CKPT, 2>(a, s_table);
}

// ---- Staged sweep.  The fine-source rows of each segment (the three fit rows
// are one contiguous block, 16-byte aligned) are copied into a ring of NST
// shared-memory stages per track by the bulk-copy engine (cp.async.bulk with
// mbarrier::complete_tx), NST-1 segments ahead of the arithmetic, so the bytes
// in flight cost no registers.  The track's lanes run the geometry ahead (the
// height chain runs NST-1 segments ahead of the arithmetic); lane 0 stores it
// beside the stage and issues the copy.  The lanes wait on the stage's barrier
// (bounded), read the rows from shared memory and do the arithmetic and the
// tallies of sweep_track.  Every wait has a cycle limit; on expiry the kernel
// sets error bit 2, lets its copies in flight land (bounded) and returns.
constexpr long long STAGE_WAIT_CYCLES = 1LL << 31;     // ~1 s at 2 GHz

struct StageGeo {              // 32 bytes, beside each stage
  float zin, ds;
  int mat, pad;
  int64_t frow, crow;
};

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ bool stage_wait(uint64_t *bar, uint32_t phase) {
  const long long t0 = clock64();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred P1;\n\tmbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, P1;\n\t}\n"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(phase)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > STAGE_WAIT_CYCLES) return false;
  }
}

__device__ __forceinline__ void stage_issue(uint64_t *bar, void *dst, const void *src,
                                            uint32_t bytes) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// Per-track state of the copy side or the arithmetic side: the track, its
// polar cosine, and the segment cursor.
struct StageCursor {
  int64_t base;          // the warp's current track base (tracks base + gw)
  int64_t tr;            // this group's track (clamped), valid if < n3d
  bool valid;
  int seg;               // next segment
  float mu;
};

__device__ __forceinline__ void cursor_track(const SweepArgs &a, StageCursor &c, int gw) {
  const int64_t track = c.base + gw;
  c.valid = track < a.n3d;
  c.tr = c.valid ? track : a.n3d - 1;
  c.mu = a.mu[(int)((c.tr / a.Z) % a.P)];
  c.seg = 0;
}

template <int TPW, int CPL, int MODE, bool QUAD, int NST>
__global__ void __launch_bounds__(BLOCK) sweep_staged_kernel(SweepArgs a, int rowbytes) {
  extern __shared__ __align__(128) unsigned char s_dyn[];
  constexpr int GPW = 32 / TPW;
  constexpr int GROUPS = BLOCK / TPW;
  // [table (PLAIN)] [barriers] [geometry] [rows], each region 128-byte aligned
  const int tab_bytes = MODE == MODE_PLAIN ? ((int)sizeof(float2) * a.table_n + 127) / 128 * 128 : 0;
  float2 *s_table = reinterpret_cast<float2 *>(s_dyn);
  uint64_t *s_bar = reinterpret_cast<uint64_t *>(s_dyn + tab_bytes);
  StageGeo *s_geo = reinterpret_cast<StageGeo *>(s_dyn + tab_bytes + ((GROUPS * NST * 8 + 127) / 128) * 128);
  unsigned char *s_rows = reinterpret_cast<unsigned char *>(s_geo) +
                          ((GROUPS * NST * (int)sizeof(StageGeo) + 127) / 128) * 128;
  const int lane = threadIdx.x & 31;
  const int li = lane % TPW;
  const int gw = lane / TPW;
  const int grp = (threadIdx.x >> 5) * GPW + gw;
  uint64_t *bar = s_bar + grp * NST;
  StageGeo *geo = s_geo + grp * NST;
  unsigned char *rows = s_rows + (size_t)grp * NST * rowbytes;
  if (MODE == MODE_PLAIN)
    for (int i = threadIdx.x; i < a.table_n; i += BLOCK) s_table[i] = a.table[i];
  if (li == 0)
    for (int k = 0; k < NST; ++k)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar + k)), "r"(1)
                   : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  __syncthreads();

  const int64_t warp_id = ((int64_t)blockIdx.x * BLOCK + threadIdx.x) >> 5;
  const int64_t stride = (((int64_t)gridDim.x * BLOCK) >> 5) * GPW;
  const int S = a.S;
  const int64_t PZ = (int64_t)a.P * a.Z;

  // ---- copy side: cursor, height chain and segment-stream chunks
  StageCursor pc;
  pc.base = warp_id * GPW;
  cursor_track(a, pc, gw);
  float pz = a.z0[pc.tr];
  const float *p_dsb = a.seg_ds + (pc.tr / PZ * a.P + (int)((pc.tr / a.Z) % a.P)) * S;
  const int32_t *p_srcb = a.seg_src + pc.tr * S;
  float ds_c = li < S ? __ldg(p_dsb + li) : 0.f;
  int src_c = li < S ? __ldg(p_srcb + li) : 0;
  float ds_n = TPW + li < S ? __ldg(p_dsb + TPW + li) : 0.f;
  int src_n = TPW + li < S ? __ldg(p_srcb + TPW + li) : 0;
  uint32_t issued = 0, consumed = 0;
  bool abort = false;

  // issues the copy of the copy cursor's segment; all lanes of the warp call it
  auto issue = [&]() {
    const int k = pc.seg % TPW;
    if (k == 0 && pc.seg > 0) {
      ds_c = ds_n;
      src_c = src_n;
      const int nl = pc.seg + TPW + li;
      ds_n = nl < S ? __ldg(p_dsb + nl) : 0.f;
      src_n = nl < S ? __ldg(p_srcb + nl) : 0;
    }
    const float ds = __shfl_sync(FULL, ds_c, k, TPW);
    const int src = __shfl_sync(FULL, src_c, k, TPW);
    const Seg g = segment_geometry<MODE == MODE_MIXED>(a, pz, checked_source(a, src, li));
    const int slot = (int)(issued % NST);
    if (li == 0) {
      StageGeo sg;
      sg.zin = g.zin;
      sg.ds = ds;
      sg.mat = g.mat;
      sg.pad = 0;
      sg.frow = g.frow;
      sg.crow = g.crow;
      geo[slot] = sg;
      stage_issue(bar + slot, rows + (size_t)slot * rowbytes, a.q + g.qrow, (uint32_t)rowbytes);
    }
    ++issued;
    pz = advance_z(a, pz, ds, pc.mu);
    if (++pc.seg == S) {                       // the next track of this group
      pc.base += stride;
      cursor_track(a, pc, gw);
      pz = a.z0[pc.tr];
      p_dsb = a.seg_ds + (pc.tr / PZ * a.P + (int)((pc.tr / a.Z) % a.P)) * S;
      p_srcb = a.seg_src + pc.tr * S;
      ds_c = li < S ? __ldg(p_dsb + li) : 0.f;
      src_c = li < S ? __ldg(p_srcb + li) : 0;
      ds_n = TPW + li < S ? __ldg(p_dsb + TPW + li) : 0.f;
      src_n = TPW + li < S ? __ldg(p_srcb + TPW + li) : 0;
    }
  };

  for (int k = 0; k < NST && pc.base < a.n3d; ++k) issue();

  // ---- arithmetic side: one track after the other
  for (int64_t base = warp_id * GPW; base < a.n3d && !abort; base += stride) {
    const int64_t track = base + gw;
    const bool valid = track < a.n3d;
    const int64_t tr = valid ? track : a.n3d - 1;
    const float mu = a.mu[(int)((tr / a.Z) % a.P)];
    const float mu2 = __fmul_rn(mu, mu);          // as sweep_track: the same psi
    const float w = a.weight[tr];
    const float w_mu = __fmul_rn(w, mu);
    float4 psi[CPL];
#pragma unroll
    for (int k = 0; k < CPL; ++k) {
      const int c = li + TPW * k;
      psi[k] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (c < a.nchunk) psi[k] = *reinterpret_cast<const float4 *>(a.psi + tr * a.ldg + 4 * c);
      if (a.psi_scale) {
        const float sc = *a.psi_scale;
        psi[k].x = __fmul_rn(psi[k].x, sc);
        psi[k].y = __fmul_rn(psi[k].y, sc);
        psi[k].z = __fmul_rn(psi[k].z, sc);
        psi[k].w = __fmul_rn(psi[k].w, sc);
      }
    }
    for (int n = 0; n < S; ++n) {
      const int slot = (int)(consumed % NST);
      const bool ok = stage_wait(bar + slot, (consumed / NST) & 1u);
      if (__any_sync(FULL, !ok)) {
        if (lane == 0) atomicOr(a.err, 2);
        abort = true;
        break;
      }
      const StageGeo sg = geo[slot];
      const float ds = sg.ds;
      const float *rq = reinterpret_cast<const float *>(rows + (size_t)slot * rowbytes);
      const MixedFit fit = (MODE == MODE_MIXED && QUAD) ? mixed_fit(a, sg.zin, mu, mu2) : MixedFit{};
#pragma unroll
      for (int k = 0; k < CPL; ++k) {
        const int c = li + TPW * k;
        if (c >= a.nchunk) continue;
        const int g4 = 4 * c;
        const float *cf = a.coef + sg.crow + 4 * COEF_PLANES * c;
        const float4 sig = __ldg(reinterpret_cast<const float4 *>(cf));
        const float4 r1 = __ldg(reinterpret_cast<const float4 *>(cf + 4));
        float4 t;
        const float4 y1 = *reinterpret_cast<const float4 *>(rq + g4);
        if (QUAD) {
          const float4 y2 = *reinterpret_cast<const float4 *>(rq + a.ldg + g4);
          const float4 y3 = *reinterpret_cast<const float4 *>(rq + 2 * a.ldg + g4);
          if (MODE == MODE_PLAIN) {
            const float4 r2 = __ldg(reinterpret_cast<const float4 *>(cf + 8));
            const float4 r3 = __ldg(reinterpret_cast<const float4 *>(cf + 12));
            const float4 r4 = __ldg(reinterpret_cast<const float4 *>(cf + 16));
            t = plain_quad_v(a, s_table, y1, y2, y3, sig, r1, r2, r3, r4, bc2(sg.zin), bc2(ds),
                             bc2(mu), bc2(mu2), bc2(w), psi[k]);
          } else {
            const float4 r2 = __ldg(reinterpret_cast<const float4 *>(cf + 8));
            const float4 r4 = __ldg(reinterpret_cast<const float4 *>(cf + 16));
            const float4 r3x2 = __ldg(reinterpret_cast<const float4 *>(cf + 20));
            t = mixed_quad_v(y1, y2, y3, pair_fit(fit), sig, r1, r2, r3x2, r4, bc2(ds), bc2(w),
                             psi[k]);
          }
        } else {
          if (MODE == MODE_PLAIN) {
            t = plain_flat_v(a, s_table, y1, sig, r1, bc2(ds), bc2(w_mu), psi[k]);
          } else {
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              float p = get(psi[k], e);
              set(t, e, mixed_flat(get(y1, e), get(sig, e), get(r1, e), ds, w_mu, p));
              set(psi[k], e, p);
            }
          }
        }
        if (valid) {
          float *dst = a.phi + sg.frow + g4;
          if (MODE == MODE_MIXED && a.phi_lo != nullptr) {
            comp_add_vec(dst, a.phi_lo + sg.frow + g4, t);
          } else {
            red_add_v4(dst, t.x, t.y, t.z, t.w);
          }
        }
      }
      ++consumed;
      __syncwarp();                            // the stage is read: it may be refilled
      if (pc.base < a.n3d) issue();
    }
    if (abort) break;
    if (valid) {
#pragma unroll
      for (int k = 0; k < CPL; ++k) {
        const int c = li + TPW * k;
        if (c < a.nchunk) *reinterpret_cast<float4 *>(a.psi + tr * a.ldg + 4 * c) = psi[k];
      }
    }
  }
  // copies still in flight (only after an expired wait) land before the block exits
  for (; consumed < issued; ++consumed)
    stage_wait(bar + consumed % NST, (consumed / NST) & 1u);
}

// Chunks of 4 groups per thread in the batched kernel: with threads per track
// from 4 to 32 this covers 8 to 256 groups.
constexpr int BATCH_CPL = 2;

// Batched sweep of many independent problems ("cores") in one persistent
// launch.  Work = tasks (core, first track) of 32/tpw tracks each, ordered by
// cost; every warp takes the next task from a global counter until none is
// left (a work queue, not a wait).  Each core runs with its own threads per
// track (tpw), so small group counts pack several tracks into a warp.
template <int MODE, bool QUAD>
__global__ void __launch_bounds__(BLOCK, 2) sweep_batch_kernel(const SweepArgs *__restrict__ cores,
                                                            const int2 *__restrict__ tasks,
                                                            int64_t n_tasks,
                                                            const int *__restrict__ core_tpw,
                                                            unsigned long long *__restrict__ counter,
                                                            const float2 *__restrict__ table,
                                                            int table_n) {
  extern __shared__ float2 s_table[];
  if (MODE == MODE_PLAIN) {
    for (int i = threadIdx.x; i < table_n; i += BLOCK) s_table[i] = table[i];
    __syncthreads();
  }
  // the task's core arguments, one slot per warp: the sweep reads its fields
  // from shared memory instead of holding the whole struct in registers
  __shared__ SweepArgs s_args[BLOCK / 32];
  const int lane = threadIdx.x & 31;
  SweepArgs &a = s_args[threadIdx.x >> 5];
  for (;;) {
    unsigned long long t = 0;
    if (lane == 0) t = atomicAdd(counter, 1ull);
    t = __shfl_sync(FULL, t, 0);
    if (t >= (unsigned long long)n_tasks) break;
    const int2 task = tasks[t];
    static_assert(sizeof(SweepArgs) % 4 == 0, "the arguments copy as 4-byte words");
    const uint32_t *src = reinterpret_cast<const uint32_t *>(cores + task.x);
    uint32_t *dst = reinterpret_cast<uint32_t *>(&a);
    for (int i = lane; i < (int)(sizeof(SweepArgs) / 4); i += 32) dst[i] = __ldg(src + i);
    __syncwarp();
    const int tpw = core_tpw[task.x];
    sweep_track<0, BATCH_CPL, MODE, QUAD, false>(a, (int64_t)task.y + lane / tpw, lane, tpw,
                                                 s_table);
    __syncwarp();                             // every lane is done with the slot
  }
}

// ---- FP64 yardstick: same traversal, double state, exact 1-exp(-tau).
template <int TPW, bool QUAD>
__global__ void __launch_bounds__(BLOCK) sweep64_kernel(SweepArgs a) {
  const int lane = threadIdx.x & 31;
  const int li = lane % TPW;
  const int gw = lane / TPW;
  constexpr int GPW = 32 / TPW;
  const int64_t warp_id = ((int64_t)blockIdx.x * BLOCK + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * BLOCK) >> 5;
  const int64_t PZ = (int64_t)a.P * a.Z;
  for (int64_t base = warp_id * GPW; base < a.n3d; base += n_warps * GPW) {
    const int64_t track = base + gw;
    const bool valid = track < a.n3d;
    const int64_t tr = valid ? track : a.n3d - 1;
    const int64_t i2 = tr / PZ;
    const int j = (int)((tr / a.Z) % a.P);
    const float muf = a.mu[j];
    const double mu = muf, mu2 = mu * mu;
    const double w = a.weight[tr];     // reference weight, promoted
    float z = a.z0[tr];
    const float *dsb = a.seg_ds + (i2 * a.P + j) * a.S;
    const int32_t *srcb = a.seg_src + tr * a.S;
    for (int n = 0; n < a.S; ++n) {
      const float dsf = __ldg(dsb + n);
      int s = __ldg(srcb + n);
      if ((uint32_t)s >= (uint64_t)a.ns) {
        if (li == 0) atomicOr(a.err, MOC_DEV_ERR_SOURCE);
        s = 0;
      }
      const double ds = dsf;
      const int zi = __float2int_rz(div_cr(z, a.dz, a.rdz));
      const int fine = zi % a.F;
      const double dz = a.dz;
      double zin = (double)z - dz * (zi + 0.5);
      int r0 = fine;
      if (QUAD) {
        if (fine == 0) { zin -= dz; r0 = 0; }
        else if (fine == a.F - 1) { zin += dz; r0 = fine - 2; }
        else r0 = fine - 1;
      }
      const int64_t sb = (int64_t)s * a.F;
      const double *qr = a.q64 + (sb + r0) * a.ldg;
      double *fr = a.phi64 + (sb + fine) * a.ldg;
      const float *sigr = a.coef + (int64_t)__ldg(a.src_sigt + s) * COEF_PLANES * a.ldg;
      // one FP64 division per (segment, group): the divisors of src/solver.c
      // (sigma^k, 2dz, 2dz^2) become products with reciprocals, a change of a
      // few units in the 16th digit (the FP64 pipe is the yardstick's bound)
      const double r2dz = 1.0 / (2.0 * dz), r2dz2 = 1.0 / (2.0 * dz * dz);
      for (int g = li; g < a.G; g += TPW) {
        const double sig = sigr[(g >> 2) * 4 * COEF_PLANES + (g & 3)];
        const double rs = 1.0 / sig;
        const double tau = sig * ds;
        const double e = -expm1(-tau);
        double p = a.psi64[tr * a.ldg + g];
        double tally;
        if (QUAD) {
          const double y1 = qr[g], y2 = qr[a.ldg + g], y3 = qr[2 * a.ldg + g];
          const double c1 = (y1 - y3) * r2dz;
          const double c2 = (y1 - 2.0 * y2 + y3) * r2dz2;
          const double q0 = y2 + c1 * zin + c2 * zin * zin;
          const double q1 = c1 + 2.0 * c2 * zin;
          const double rs2 = rs * rs;
          const double reuse = tau * (tau - 2.0) + 2.0 * e * (rs * rs2);
          const double fi = (q0 * tau + (sig * p - q0) * e) * rs2 + q1 * mu * reuse +
                            c2 * mu2 * (tau * (tau * (tau - 3.0) + 6.0) - 6.0 * e) *
                                (rs2 * rs2 * (1.0 / 3.0));
          tally = w * fi;
          p = q0 * e * rs + q1 * mu * (tau - e) * rs2 + c2 * mu2 * reuse + p * (1.0 - e);
        } else {
          const double dpsi = (p - qr[g] * rs) * e;
          p -= dpsi;
          tally = w * mu * dpsi;
        }
        if (valid) {
          a.psi64[tr * a.ldg + g] = p;
          atomicAdd(fr + g, tally);
        }
      }
      z = advance_z(a, z, dsf, muf);
    }
  }
}

template <int TPW, int CPL, int MODE, bool QUAD, bool CSR = false, bool CKPT = false,
          int VW = 4, bool REC = false, bool COMP = false>
int launch_t(moc_problem *p, const SweepArgs &a) {
  void (*kern)(SweepArgs);
  if constexpr (COMP)
    kern = sweep_comp_kernel<TPW, CPL, QUAD>;
  else if constexpr (REC)
    kern = sweep_record_kernel<TPW, CPL, MODE, QUAD>;
  else if constexpr (VW == 4)
    kern = sweep_kernel<TPW, CPL, MODE, QUAD, CSR, CKPT>;
  else
    kern = sweep_kernel_v2<TPW, CPL, MODE, QUAD, CSR, CKPT>;
  size_t smem = (MODE == MODE_PLAIN) ? sizeof(float2) * (size_t)a.table_n : 0;
  if (smem > 48 * 1024) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return MOC_ERR_UNSUPPORTED;
  }
  int per_sm = 0, sms = 0;
  MOC_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BLOCK, smem));
  MOC_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device));
  if (per_sm < 1) return MOC_ERR_UNSUPPORTED;
  int64_t groups = (a.n3d + (32 / TPW) - 1) / (32 / TPW);         // warps of work
  int64_t blocks_needed = (groups + (BLOCK / 32) - 1) / (BLOCK / 32);
  int64_t grid = (int64_t)per_sm * sms;
  if (grid > blocks_needed) grid = blocks_needed;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, BLOCK, smem, p->stream>>>(a);
  MOC_CUDA_TRY(cudaGetLastError());
  p->launches++;
  return MOC_OK;
}

template <int TPW, bool QUAD>
int launch64_t(moc_problem *p, const SweepArgs &a) {
  auto kern = sweep64_kernel<TPW, QUAD>;
  int per_sm = 0, sms = 0;
  MOC_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BLOCK, 0));
  MOC_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device));
  int64_t warps = (a.n3d + (32 / TPW) - 1) / (32 / TPW);
  int64_t grid = (int64_t)per_sm * sms;
  int64_t need = (warps + 7) / 8;
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, BLOCK, 0, p->stream>>>(a);
  MOC_CUDA_TRY(cudaGetLastError());
  p->launches++;
  return MOC_OK;
}

template <int MODE, bool QUAD>
int dispatch_shape(moc_problem *p, const SweepArgs &a, int tpw, int cpl) {
  if (tpw == 32 && cpl == 1) return launch_t<32, 1, MODE, QUAD>(p, a);
  if (tpw == 32 && cpl == 2) return launch_t<32, 2, MODE, QUAD>(p, a);
  if (tpw == 32 && cpl == 4) return launch_t<32, 4, MODE, QUAD>(p, a);
  if (tpw == 16 && cpl == 1) return launch_t<16, 1, MODE, QUAD>(p, a);
  if (tpw == 16 && cpl == 2) return launch_t<16, 2, MODE, QUAD>(p, a);
  if (tpw == 8 && cpl == 1) return launch_t<8, 1, MODE, QUAD>(p, a);
  if (tpw == 8 && cpl == 4) return launch_t<8, 4, MODE, QUAD>(p, a);
  if (tpw == 4 && cpl == 2) return launch_t<4, 2, MODE, QUAD>(p, a);
  if (tpw == 10 && cpl == 5) return launch_t<10, 5, MODE, QUAD, false, false, 2>(p, a);
  // 10 lanes x one 4-group chunk: up to 40 groups, three tracks a warp
  if (tpw == 10 && cpl == 1) return launch_t<10, 1, MODE, QUAD>(p, a);
  return MOC_ERR_UNSUPPORTED;
}

// The compensated MIXED sweep: power-of-two shapes of four-group chunks; any
// other shape falls back to the narrowest of them that covers the groups.
template <bool QUAD>
int dispatch_comp(moc_problem *p, const SweepArgs &a, int tpw, int cpl) {
  constexpr int M = MODE_MIXED;
  if (tpw == 32 && cpl == 1) return launch_t<32, 1, M, QUAD, false, false, 4, false, true>(p, a);
  if (tpw == 32 && cpl == 2) return launch_t<32, 2, M, QUAD, false, false, 4, false, true>(p, a);
  if (tpw == 32 && cpl == 4) return launch_t<32, 4, M, QUAD, false, false, 4, false, true>(p, a);
  if (tpw == 16 && cpl == 1) return launch_t<16, 1, M, QUAD, false, false, 4, false, true>(p, a);
  if (tpw == 16 && cpl == 2) return launch_t<16, 2, M, QUAD, false, false, 4, false, true>(p, a);
  if (tpw == 8 && cpl == 1) return launch_t<8, 1, M, QUAD, false, false, 4, false, true>(p, a);
  if (tpw == 8 && cpl == 4) return launch_t<8, 4, M, QUAD, false, false, 4, false, true>(p, a);
  if (tpw == 4 && cpl == 2) return launch_t<4, 2, M, QUAD, false, false, 4, false, true>(p, a);
  const int nchunk = p->ldg / 4;
  if (nchunk <= 8) return dispatch_comp<QUAD>(p, a, 8, 1);
  if (nchunk <= 16) return dispatch_comp<QUAD>(p, a, 16, 1);
  if (nchunk <= 32) return dispatch_comp<QUAD>(p, a, 16, 2);
  if (nchunk <= 64) return dispatch_comp<QUAD>(p, a, 32, 2);
  if (nchunk <= 128) return dispatch_comp<QUAD>(p, a, 32, 4);
  return MOC_ERR_UNSUPPORTED;
}

// Shared memory of the staged kernel: table, barriers, stage geometry, rows.
size_t staged_smem(const SweepArgs &a, int mode, bool quad, int tpw, int nst) {
  const size_t groups = BLOCK / tpw;
  const size_t tab = mode == MODE_PLAIN ? (sizeof(float2) * a.table_n + 127) / 128 * 128 : 0;
  const size_t rowbytes = (quad ? 3 : 1) * (size_t)a.ldg * 4;
  return tab + (groups * nst * 8 + 127) / 128 * 128 +
         (groups * nst * sizeof(StageGeo) + 127) / 128 * 128 + groups * nst * rowbytes;
}

template <int TPW, int CPL, int MODE, bool QUAD, int NST>
int launch_staged_t(moc_problem *p, const SweepArgs &a) {
  auto kern = sweep_staged_kernel<TPW, CPL, MODE, QUAD, NST>;
  const size_t smem = staged_smem(a, MODE, QUAD, TPW, NST);
  if (smem > 227 * 1024) return MOC_ERR_UNSUPPORTED;
  MOC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0, sms = 0;
  MOC_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BLOCK, smem));
  MOC_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device));
  if (per_sm < 1) return MOC_ERR_UNSUPPORTED;
  const int64_t warps = (a.n3d + (32 / TPW) - 1) / (32 / TPW);
  const int64_t need = (warps + (BLOCK / 32) - 1) / (BLOCK / 32);
  int64_t grid = (int64_t)per_sm * sms;
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  const int rowbytes = (QUAD ? 3 : 1) * a.ldg * 4;
  kern<<<(unsigned)grid, BLOCK, smem, p->stream>>>(a, rowbytes);
  MOC_CUDA_TRY(cudaGetLastError());
  p->launches++;
  return MOC_OK;
}

template <int MODE, bool QUAD>
int dispatch_staged(moc_problem *p, const SweepArgs &a, int tpw, int cpl, int stages) {
  if (stages != 4) return MOC_ERR_UNSUPPORTED;
  if (tpw == 32 && cpl == 1) return launch_staged_t<32, 1, MODE, QUAD, 4>(p, a);
  if (tpw == 32 && cpl == 2) return launch_staged_t<32, 2, MODE, QUAD, 4>(p, a);
  if (tpw == 16 && cpl == 1) return launch_staged_t<16, 1, MODE, QUAD, 4>(p, a);
  if (tpw == 16 && cpl == 2) return launch_staged_t<16, 2, MODE, QUAD, 4>(p, a);
  if (tpw == 8 && cpl == 1) return launch_staged_t<8, 1, MODE, QUAD, 4>(p, a);
  return MOC_ERR_UNSUPPORTED;
}

}  // namespace

// Default threads-per-track and chunks-per-thread for a group count, from the
// launch-shape measurements on GB300 (two tracks per warp with two chunks per
// thread was fastest for 100 groups in both modes); moc_autotune measures.
int moc_shape_groups(int tpw, int cpl) {
  return tpw * cpl * ((tpw == 10 && cpl == 5) ? 2 : 4);
}

int moc_sweep_launch_shape(const moc_problem *p, int *tpw, int *cpl) {
  const int nchunk = p->ldg / 4;
  if (p->tpw > 0) {
    *tpw = p->tpw;
    *cpl = p->cpl;
    if (moc_shape_groups(p->tpw, p->cpl) < p->ldg) return MOC_ERR_ARG;
    return MOC_OK;
  }
  if (nchunk <= 8) { *tpw = 8; *cpl = 1; }
  else if (nchunk <= 16) { *tpw = 16; *cpl = 1; }
  else if (nchunk <= 32) { *tpw = 16; *cpl = 2; }
  else if (nchunk <= 64) { *tpw = 32; *cpl = 2; }
  else if (nchunk <= 128) { *tpw = 32; *cpl = 4; }
  else return MOC_ERR_UNSUPPORTED;
  return MOC_OK;
}

namespace {

SweepArgs build_args(moc_problem *p) {
  const moc_dims &d = p->d;
  SweepArgs a{};
  a.seg_ds = p->seg_ds;
  a.seg_src = p->seg_src;
  a.weight = p->weight;
  a.z0 = p->z0;
  a.mu = p->mu;
  a.src_sigt = p->src_sigt;
  a.coef = p->coef;
  a.table = reinterpret_cast<const float2 *>(p->table);
  a.q = p->q;
  a.phi = p->phi;
  a.phi_lo = (p->mode == MOC_MODE_MIXED && (p->flags & MOC_FLAG_COMPENSATED)) ? p->phi_lo : nullptr;
  a.psi = p->psi_f;
  a.psi_scale = (p->psi_pending && p->mode != MOC_MODE_FP64) ? p->psi_scale : nullptr;
  a.q64 = p->q64;
  a.phi64 = p->phi64;
  a.psi64 = p->psi_f64;
  a.n3d = p->n3d;
  a.ns = d.n_sources;
  a.G = d.n_groups;
  a.ldg = p->ldg;
  a.nchunk = p->ldg / 4;
  a.F = d.fai;
  a.P = d.n_polar;
  a.Z = d.z_stacked;
  a.S = d.n_seg;
  a.axial_exp = d.axial_exp;
  a.table_n = d.table_n;
  a.table_dx = d.table_dx;
  a.table_rdx = 1.0f / d.table_dx;
  a.table_halfdx = 0.5f * d.table_dx;
  a.table_maxval = d.table_maxval;
  a.rt_one = 1.0f;
  a.rt_m1 = -1.0f;
  a.rt_nz = -0.0f;
  // src/solver.c:38 -- float height over the int product
  a.dz = d.height / (float)(d.fai * d.decomp_ax * d.cai);
  a.rdz = 1.0f / a.dz;
  a.d1 = 2.f * a.dz;                      // src/solver.c:75
  a.rd1 = 1.0f / a.d1;
  a.d2 = 2.f * a.dz * a.dz;               // src/solver.c:76
  a.rd2 = 1.0f / a.d2;
  a.hd = d.height / (float)d.decomp_ax;
  a.fmagic = p->fmagic;
  a.err = p->err;
  return a;
}

int launch_args(moc_problem *p, const SweepArgs &a, int tpw, int cpl, int stages) {
  const bool quad = p->d.axial_exp == 2;
  if (p->mode == MOC_MODE_FP64) {
    if (!p->q64) return MOC_ERR_STATE;
    return quad ? launch64_t<32, true>(p, a) : launch64_t<32, false>(p, a);
  }
  if (stages > 0) {
    if (p->mode == MOC_MODE_PLAIN)
      return quad ? dispatch_staged<MODE_PLAIN, true>(p, a, tpw, cpl, stages)
                  : dispatch_staged<MODE_PLAIN, false>(p, a, tpw, cpl, stages);
    return quad ? dispatch_staged<MODE_MIXED, true>(p, a, tpw, cpl, stages)
                : dispatch_staged<MODE_MIXED, false>(p, a, tpw, cpl, stages);
  }
  if (p->mode == MOC_MODE_PLAIN)
    return quad ? dispatch_shape<MODE_PLAIN, true>(p, a, tpw, cpl)
                : dispatch_shape<MODE_PLAIN, false>(p, a, tpw, cpl);
  if (a.phi_lo)
    return quad ? dispatch_comp<true>(p, a, tpw, cpl) : dispatch_comp<false>(p, a, tpw, cpl);
  return quad ? dispatch_shape<MODE_MIXED, true>(p, a, tpw, cpl)
              : dispatch_shape<MODE_MIXED, false>(p, a, tpw, cpl);
}

struct TuneKey {
  int S, G, P, mode, axial, comp;
  bool operator<(const TuneKey &o) const {
    return std::tie(S, G, P, mode, axial, comp) < std::tie(o.S, o.G, o.P, o.mode, o.axial, o.comp);
  }
};
std::mutex g_tune_mu;
struct TuneChoice {
  int tpw, cpl, stages;
};
std::map<TuneKey, TuneChoice> g_tune_cache;

}  // namespace

int moc_launch_sweep(moc_problem *p) {
  int tpw = 0, cpl = 0;
  int st = moc_sweep_launch_shape(p, &tpw, &cpl);
  if (st != MOC_OK) return st;
  return launch_args(p, build_args(p), tpw, cpl, p->stages > 0 ? p->stages : 0);
}

// A range of whole 2D tracks is a contiguous range of 3D tracks (the track
// index is (i2 * P + polar) * Z + stack), so the sweep of the range is the
// sweep kernel over per-track arrays offset to its first track.
int moc_launch_sweep_range(moc_problem *p, int64_t i2_begin, int64_t i2_end) {
  const int64_t P = p->d.n_polar, Z = p->d.z_stacked, S = p->d.n_seg;
  if (i2_begin < 0 || i2_end > p->d.n_tracks_2d || i2_begin >= i2_end) return MOC_ERR_ARG;
  if (p->mode == MOC_MODE_FP64) return MOC_ERR_UNSUPPORTED;
  int tpw = 0, cpl = 0;
  int st = moc_sweep_launch_shape(p, &tpw, &cpl);
  if (st != MOC_OK) return st;
  SweepArgs a = build_args(p);
  const int64_t t0 = i2_begin * P * Z;
  a.seg_ds += i2_begin * P * S;
  a.seg_src += t0 * S;
  a.weight += t0;
  a.z0 += t0;
  a.psi += t0 * p->ldg;
  a.n3d = (i2_end - i2_begin) * P * Z;
  return launch_args(p, a, tpw, cpl, p->stages > 0 ? p->stages : 0);
}

namespace {
template <int MODE, bool QUAD>
int dispatch_record(moc_problem *p, const SweepArgs &a) {
  if (p->ldg <= 128) return launch_t<16, 2, MODE, QUAD, false, false, 4, true>(p, a);
  if (p->ldg <= 256) return launch_t<32, 2, MODE, QUAD, false, false, 4, true>(p, a);
  return MOC_ERR_UNSUPPORTED;
}
}  // namespace

// The sweep of 2D tracks [i2_begin, i2_end) with its tallies recorded: the
// contribution of segment n of the range's track t (counted from the range's
// first track) goes to rec[(t * S + n) * ldg ...], its FSR row to
// rec_row[t * S + n].
int moc_launch_sweep_record(moc_problem *p, int64_t i2_begin, int64_t i2_end, float *rec,
                            int32_t *rec_row) {
  const int64_t P = p->d.n_polar, Z = p->d.z_stacked, S = p->d.n_seg;
  if (i2_begin < 0 || i2_end > p->d.n_tracks_2d || i2_begin >= i2_end) return MOC_ERR_ARG;
  if (p->mode == MOC_MODE_FP64) return MOC_ERR_UNSUPPORTED;
  SweepArgs a = build_args(p);
  const int64_t t0 = i2_begin * P * Z;
  a.seg_ds += i2_begin * P * S;
  a.seg_src += t0 * S;
  a.weight += t0;
  a.z0 += t0;
  a.psi += t0 * p->ldg;
  a.n3d = (i2_end - i2_begin) * P * Z;
  a.phi_lo = nullptr;
  a.rec = rec;
  a.rec_row = rec_row;
  const bool quad = p->d.axial_exp == 2;
  if (p->mode == MOC_MODE_PLAIN)
    return quad ? dispatch_record<MODE_PLAIN, true>(p, a) : dispatch_record<MODE_PLAIN, false>(p, a);
  return quad ? dispatch_record<MODE_MIXED, true>(p, a) : dispatch_record<MODE_MIXED, false>(p, a);
}

// Times every launch shape that covers the groups on the first n_sub tracks.
// Tallies go to a scratch copy of the flux array and the tracks' angular flux
// to a scratch copy, so the problem's state is not changed.
int moc_sweep_autotune(moc_problem *p, int64_t n_sub, int *tpw_out, int *cpl_out,
                       int *stages_out, double *ms_out) {
  if (p->mode == MOC_MODE_FP64) {
    *tpw_out = 32;
    *cpl_out = 1;
    *stages_out = 0;
    if (ms_out) *ms_out = 0.0;
    return MOC_OK;
  }
  const TuneKey key{p->d.n_seg, p->d.n_groups, p->d.n_polar, p->mode, p->d.axial_exp,
                    (p->flags & MOC_FLAG_COMPENSATED) ? 1 : 0};
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end() && ms_out == nullptr) {
      *tpw_out = it->second.tpw;
      *cpl_out = it->second.cpl;
      *stages_out = it->second.stages;
      return MOC_OK;
    }
  }
  if (n_sub <= 0) n_sub = p->n3d < 262144 ? p->n3d : 262144;
  if (n_sub > p->n3d) n_sub = p->n3d;
  float *phi_s = nullptr, *psi_s = nullptr, *lo_s = nullptr;
  const size_t phi_bytes = sizeof(float) * (size_t)(p->nfsr * p->ldg);
  const size_t psi_bytes = sizeof(float) * (size_t)(n_sub * p->ldg);
  MOC_CUDA_TRY(cudaMalloc(&phi_s, phi_bytes));
  if (cudaMalloc(&psi_s, psi_bytes) != cudaSuccess ||
      (p->phi_lo && cudaMalloc(&lo_s, phi_bytes) != cudaSuccess)) {
    cudaGetLastError();
    cudaFree(phi_s);
    cudaFree(psi_s);
    return MOC_ERR_OOM;
  }
  SweepArgs a = build_args(p);
  a.n3d = n_sub;
  a.phi = phi_s;
  a.psi = psi_s;
  if (a.phi_lo) a.phi_lo = lo_s;
  int rc = MOC_OK;
  if (cudaMemsetAsync(phi_s, 0, phi_bytes, p->stream) != cudaSuccess ||
      (lo_s && cudaMemsetAsync(lo_s, 0, phi_bytes, p->stream) != cudaSuccess) ||
      cudaMemcpyAsync(psi_s, p->psi_f, psi_bytes, cudaMemcpyDeviceToDevice, p->stream) !=
          cudaSuccess)
    rc = MOC_ERR_CUDA;
  // register-prefetch shapes, then the staged kernel (4-stage ring) shapes
  static const int shapes[][3] = {{32, 1, 0}, {32, 2, 0}, {32, 4, 0}, {16, 1, 0}, {16, 2, 0},
                                  {8, 1, 0},  {8, 4, 0},  {4, 2, 0},  {10, 5, 0}, {10, 1, 0},
                                  {32, 1, 4},
                                  {32, 2, 4}, {16, 1, 4}, {16, 2, 4}, {8, 1, 4}};
  double best = 1e30;
  int bt = 0, bc = 0, bs = 0;
  for (auto &sh : shapes) {
    if (rc != MOC_OK) break;
    const int covered = moc_shape_groups(sh[0], sh[1]);
    if (covered < p->ldg) continue;
    if (a.phi_lo && sh[0] == 10) continue;       // no compensated ten-lane variant
    if (covered >= 4 * p->ldg && sh[1] > 1) continue;                  // mostly idle lanes
    if (sh[2] > 0 && staged_smem(a, p->mode == MOC_MODE_PLAIN ? MODE_PLAIN : MODE_MIXED,
                                 p->d.axial_exp == 2, sh[0], sh[2]) > 227 * 1024)
      continue;
    rc = launch_args(p, a, sh[0], sh[1], sh[2]);             // warm-up
    double tot = 0.0;
    for (int r = 0; r < 2 && rc == MOC_OK; ++r) {
      cudaEventRecord(p->ev0, p->stream);
      rc = launch_args(p, a, sh[0], sh[1], sh[2]);
      cudaEventRecord(p->ev1, p->stream);
      if (rc == MOC_OK && cudaEventSynchronize(p->ev1) != cudaSuccess) rc = MOC_ERR_CUDA;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, p->ev0, p->ev1);
      tot += ms;
    }
    if (rc == MOC_OK && tot / 2 < best) {
      best = tot / 2;
      bt = sh[0];
      bc = sh[1];
      bs = sh[2];
    }
  }
  cudaStreamSynchronize(p->stream);
  cudaFree(phi_s);
  cudaFree(psi_s);
  if (lo_s) cudaFree(lo_s);
  if (rc != MOC_OK) return rc;
  if (bt == 0) return MOC_ERR_UNSUPPORTED;
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune_cache[key] = {bt, bc, bs};
  }
  *tpw_out = bt;
  *cpl_out = bc;
  *stages_out = bs;
  if (ms_out) *ms_out = best;
  return MOC_OK;
}

// Sweep over variable-length sub-segment streams (the reference traversal).
int moc_launch_sweep_csr(moc_problem *p, const int64_t *off, const float *ds, const float *z,
                         const int32_t *src) {
  SweepArgs a = build_args(p);
  a.csr_off = off;
  a.csr_ds = ds;
  a.csr_z = z;
  a.csr_src = src;
  const bool quad = p->d.axial_exp == 2;
  const int nchunk = p->ldg / 4;
  if (p->mode == MOC_MODE_FP64) return MOC_ERR_UNSUPPORTED;
  const bool plain = p->mode == MOC_MODE_PLAIN;
  if (nchunk <= 32)                      // two stacked rays a warp, two chunks a lane
    return plain ? (quad ? launch_t<16, 2, MODE_PLAIN, true, true>(p, a)
                         : launch_t<16, 2, MODE_PLAIN, false, true>(p, a))
                 : (quad ? launch_t<16, 2, MODE_MIXED, true, true>(p, a)
                         : launch_t<16, 2, MODE_MIXED, false, true>(p, a));
  if (nchunk <= 64)
    return plain ? (quad ? launch_t<32, 2, MODE_PLAIN, true, true>(p, a)
                         : launch_t<32, 2, MODE_PLAIN, false, true>(p, a))
                 : (quad ? launch_t<32, 2, MODE_MIXED, true, true>(p, a)
                         : launch_t<32, 2, MODE_MIXED, false, true>(p, a));
  if (nchunk <= 128)
    return plain ? (quad ? launch_t<32, 4, MODE_PLAIN, true, true>(p, a)
                         : launch_t<32, 4, MODE_PLAIN, false, true>(p, a))
                 : (quad ? launch_t<32, 4, MODE_MIXED, true, true>(p, a)
                         : launch_t<32, 4, MODE_MIXED, false, true>(p, a));
  return MOC_ERR_UNSUPPORTED;
}

// One persistent launch over the tasks of many problems (see sweep_batch_kernel).
int moc_launch_sweep_batch(int device, cudaStream_t st, int mode, bool quad, const SweepArgs *args,
                           const int2 *tasks, int64_t n_tasks, const int *tpw,
                           unsigned long long *counter, const float2 *table, int table_n) {
  if (mode == MOC_MODE_FP64) return MOC_ERR_UNSUPPORTED;
  const bool plain = mode == MOC_MODE_PLAIN;
  auto kern = plain ? (quad ? sweep_batch_kernel<MODE_PLAIN, true> : sweep_batch_kernel<MODE_PLAIN, false>)
                    : (quad ? sweep_batch_kernel<MODE_MIXED, true> : sweep_batch_kernel<MODE_MIXED, false>);
  const size_t smem = plain ? sizeof(float2) * (size_t)table_n : 0;
  if (smem > 48 * 1024)
    MOC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0, sms = 0;
  MOC_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BLOCK, smem));
  MOC_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  if (per_sm < 1) return MOC_ERR_UNSUPPORTED;
  int64_t grid = (int64_t)per_sm * sms;
  const int64_t need = (n_tasks + (BLOCK / 32) - 1) / (BLOCK / 32);
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  MOC_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st));
  kern<<<(unsigned)grid, BLOCK, smem, st>>>(args, tasks, n_tasks, tpw, counter, table, table_n);
  MOC_CUDA_TRY(cudaGetLastError());
  return MOC_OK;
}

SweepArgs moc_sweep_args(moc_problem *p) { return build_args(p); }

// ===========================================================================
// Adjoint (reverse-mode) sweep of the MIXED arithmetic.
//
// The loss is any function of the scalar fluxes; the caller gives its gradient
// dL/dphi.  Each segment adds tally = w * fi(psi, q, sigma) to one fine region
// and maps psi to pn(psi, q, sigma) (per group, groups independent), so per
// track and group the reverse sweep is a scalar recurrence
//     psibar_n = psibar_{n+1} * dpn/dpsi + (w dL/dphi) * dfi/dpsi,
// with the parameter adjoints accumulated from the same two partials.  psi_n
// is recomputed forward from the checkpoint that the forward sweep stored
// every ck_k (<= 8) segments, held in registers for the block, and consumed
// backwards.  dL/dq goes to the three fine-source rows of every segment with
// vector reductions; dL/dsigma_t is summed per sub-warp in shared memory and
// added to an FP64 array once per block.
// ===========================================================================
namespace {

constexpr int ADJ_KMAX = 8;

struct AdjArgs {
  SweepArgs a;
  const float *dphi;      // [NS*F*ldg] dL/dphi
  float *dq;              // [NS*F*ldg] dL/dq, added to
  double *dsig;           // [n_sigt*ldg] dL/dsigma_t, added to
  float *dpsi_in;         // [N3D*G] dL/dpsi entering each track, or null
  float *dfit;            // [NS][F-2][3][ldg] dL/d(c0, c1, c2) per fit window, or null
  int n_sigt;
  int slices;             // 1: shared-memory accumulators per sub-warp
  int tpw;                // lanes per track (any width 1..32)
  int nsub;               // tracks per block: (BLOCK / 32) * (32 / tpw)
};

struct AdjOut {
  float pbar, y1b, y2b, y3b, sbar;
  float q0b, q1mub, q2mu2b;   // quadratic source: dL/d q0, d(q1 mu), d(q2 mu^2)
};

// Reverse of mixed_quad_e for one group.  With the per-segment fit factors f
// (mixed_fit), E = 1 - e^-tau and the weights
//   T = (tau - E)/sig^2, U = E/sig, R = tau (tau - 2) + 2E/sig^3 (the reference's
//   reuse term), C = (tau^3 - 3 tau^2 + 6 tau - 6E)/(3 sig^4),
// the forward is fi = q0 T + psi U + q1mu R + q2mu2 C and
// pn = q0 U + q1mu T + q2mu2 R + psi (1 - E).  Given abar = dL/dfi (w dL/dphi) and
// pbar = dL/dpn it returns dL/dpsi, dL/d of the three fit rows and of q0, q1 mu,
// q2 mu^2, and dL/dsigma through the sigma-derivatives of the weights
// (tau = sig ds, E' = ds (1 - E)):
//   U' = (E' - U)/sig, T' = ds E/sig^2 - 2T/sig, R' = (2tau - 2) ds + 2/sig^3 (E' - 3U),
//   C' = ((3tau^2 - 6tau + 6) ds - 6E')/(3 sig^4) - 4C/sig.
// Two groups at once, on packed FP32 pairs.
struct AdjOut2 {
  float2 pbar, y1b, y2b, y3b, sbar, q0b, q1mub, q2mu2b;
};
__device__ __forceinline__ AdjOut2 adj_quad2(float2 y1, float2 y2, float2 y3, const MixedFit2 &f,
                                             float2 sig, float2 r1, float2 ds, float2 E,
                                             float2 psi, float2 pbar, float2 abar) {
  const float2 m1 = bc2(-1.f), two = bc2(2.f);
  const float2 r2 = mul2(r1, r1), r3 = mul2(r1, r2);
  const float2 r4 = mul2(mul2(r2, r2), bc2(1.0f / 3.0f));
  const float2 d1 = fma2(y3, m1, y1);
  const float2 d2 = add2(fma2(bc2(-2.f), y2, y1), y3);
  const float2 q0 = fma2(d2, f.a0, fma2(d1, f.a1, y2));
  const float2 q1mu = fma2(d2, f.b2, mul2(d1, f.b1));
  const float2 q2mu2 = mul2(d2, f.c2m);
  const float2 tau = mul2(sig, ds);
  const float2 eps = fma2(E, m1, bc2(1.f));
  const float2 T = mul2(fma2(E, m1, tau), r2);
  const float2 U = mul2(E, r1);
  const float2 R = fma2(mul2(two, E), r3, mul2(tau, add2(tau, bc2(-2.f))));
  const float2 C =
      mul2(fma2(tau, fma2(tau, add2(tau, bc2(-3.f)), bc2(6.f)), mul2(bc2(-6.f), E)), r4);
  AdjOut2 o;
  o.pbar = fma2(pbar, eps, mul2(abar, U));
  o.q0b = fma2(abar, T, mul2(pbar, U));
  o.q1mub = fma2(abar, R, mul2(pbar, T));
  o.q2mu2b = fma2(abar, C, mul2(pbar, R));
  const float2 d1b = fma2(o.q0b, f.a1, mul2(o.q1mub, f.b1));
  const float2 d2b = fma2(o.q0b, f.a0, fma2(o.q1mub, f.b2, mul2(o.q2mu2b, f.c2m)));
  o.y1b = add2(d1b, d2b);
  o.y2b = fma2(bc2(-2.f), d2b, o.q0b);
  o.y3b = fma2(d1b, m1, d2b);
  const float2 Ep = mul2(ds, eps);
  const float2 Up = mul2(fma2(U, m1, Ep), r1);
  const float2 Tp = fma2(mul2(ds, E), r2, mul2(mul2(bc2(-2.f), T), r1));
  const float2 Rp = fma2(fma2(two, tau, bc2(-2.f)), ds, mul2(mul2(two, r3), fma2(bc2(-3.f), U, Ep)));
  const float2 Cp = fma2(fma2(fma2(fma2(bc2(3.f), tau, bc2(-6.f)), tau, bc2(6.f)), ds,
                              mul2(bc2(-6.f), Ep)),
                         r4, mul2(mul2(bc2(-4.f), C), r1));
  const float2 dfi = fma2(q0, Tp, fma2(psi, Up, fma2(q1mu, Rp, mul2(q2mu2, Cp))));
  const float2 dpn = fma2(q0, Up, fma2(q1mu, Tp, fma2(q2mu2, Rp, mul2(mul2(psi, m1), Ep))));
  o.sbar = fma2(abar, dfi, mul2(pbar, dpn));
  return o;
}

__device__ __forceinline__ AdjOut adj_flat(float y, float sig, float r1, float ds, float psi,
                                           float pbar, float abar) {
  const float e = one_minus_exp(sig * ds);
  const float eps = 1.f - e;
  const float dbar = abar - pbar;                     // dL/d(delta psi)
  AdjOut o;
  o.pbar = pbar + dbar * e;
  o.y1b = -dbar * e * r1;
  o.y2b = o.y3b = 0.f;
  o.q0b = o.q1mub = o.q2mu2b = 0.f;
  o.sbar = dbar * (y * r1 * r1 * e + (psi - y * r1) * eps * ds);
  return o;
}

// The per-segment operands of one thread's chunks.  The recomputation needs the
// forward's coefficient planes and the fit rows; the reverse pass sigma_t,
// 1/sigma_t, the fit rows and dL/dphi of the tally row.
template <int CPL, bool QUAD>
struct AdjFwdRows {
  float4 sig[CPL], r1[CPL], r2[CPL], r3x2[CPL], r4[CPL], y[CPL][QUAD ? 3 : 1];
};
template <int CPL, bool QUAD>
struct AdjRevRows {
  float4 sig[CPL], r1[CPL], y[CPL][QUAD ? 3 : 1], lam[CPL];
};

// the fit rows of one chunk, allocating in L1: the reverse pass reads the rows
// the recomputation read a few segments before
template <bool QUAD>
__device__ __forceinline__ void adj_rows(const SweepArgs &a, const Seg &g, int c, float4 *y) {
  const float *qr = a.q + g.qrow + 4 * c;
  ld_row_vec<true>(qr, y[0]);
  if (QUAD) {
    ld_row_vec<true>(qr + a.ldg, y[QUAD ? 1 : 0]);
    ld_row_vec<true>(qr + 2 * a.ldg, y[QUAD ? 2 : 0]);
  }
}

template <int CPL, bool QUAD>
__device__ __forceinline__ void adj_load_fwd(const SweepArgs &a, const Seg &g, int li, int TPW,
                                             AdjFwdRows<CPL, QUAD> &r) {
#pragma unroll
  for (int k = 0; k < CPL; ++k) {
    const int c = li + TPW * k;
    if (c >= a.nchunk) continue;
    const float *cf = a.coef + g.crow + 4 * COEF_PLANES * c;
    r.sig[k] = __ldg(reinterpret_cast<const float4 *>(cf));
    r.r1[k] = __ldg(reinterpret_cast<const float4 *>(cf + 4));
    if (QUAD) {
      r.r2[k] = __ldg(reinterpret_cast<const float4 *>(cf + 8));
      r.r4[k] = __ldg(reinterpret_cast<const float4 *>(cf + 16));
      r.r3x2[k] = __ldg(reinterpret_cast<const float4 *>(cf + 20));
    }
    adj_rows<QUAD>(a, g, c, r.y[k]);
  }
}

template <int CPL, bool QUAD>
__device__ __forceinline__ void adj_load_rev(const SweepArgs &a, const AdjArgs &x, const Seg &g,
                                             int li, int TPW, AdjRevRows<CPL, QUAD> &r) {
#pragma unroll
  for (int k = 0; k < CPL; ++k) {
    const int c = li + TPW * k;
    if (c >= a.nchunk) continue;
    const float *cf = a.coef + g.crow + 4 * COEF_PLANES * c;
    r.sig[k] = __ldg(reinterpret_cast<const float4 *>(cf));
    r.r1[k] = __ldg(reinterpret_cast<const float4 *>(cf + 4));
    adj_rows<QUAD>(a, g, c, r.y[k]);
    r.lam[k] = __ldg(reinterpret_cast<const float4 *>(x.dphi + g.frow + 4 * c));
  }
}

// Shared memory of the reverse sweep: the recomputed angular flux of the
// current checkpoint block (ADJ_KMAX x CPL float4 per thread), then the
// per-sub-warp dL/dsigma_t accumulators when they fit.
// Two planes per thread and block segment: psi entering it and (quadratic
// source) E = 1 - e^-tau of its groups, both from the recomputation.
template <int CPL>
constexpr size_t adj_hist_bytes() {
  return 2 * sizeof(float4) * (size_t)BLOCK * ADJ_KMAX * CPL;
}

// Lanes per track are a runtime width: the kernel has no shuffles, so a track
// of nchunk float4 chunks takes exactly ceil(nchunk / CPL) lanes and a warp
// holds floor(32 / width) tracks (G = 40: 10 lanes, three tracks a warp).  The
// lanes left over run the loops with no chunk so that the warp stays converged.
// FIT: dL/d of the quadratic fits' coefficients too (x.dfit).
template <int CPL, bool QUAD, bool FIT = false>
__global__ void __launch_bounds__(BLOCK, 2) adjoint_kernel(AdjArgs x) {
  extern __shared__ float4 s_adj[];
  const SweepArgs &a = x.a;
  const int TPW = x.tpw;
  const int GPW = 32 / TPW;
  const int lane = threadIdx.x & 31;
  const bool idle = lane >= GPW * TPW;
  const int li = idle ? (1 << 20) : lane % TPW;    // idle lanes own no chunk
  const int gw = idle ? 0 : lane / TPW;
  const int sub = (threadIdx.x >> 5) * GPW + gw;
  // this thread's history slots: hist(jj, k) at s_adj[(jj * CPL + k) * BLOCK + threadIdx.x]
  float4 *hist_base = s_adj + threadIdx.x;
  float4 *ehist_base = hist_base + (size_t)BLOCK * ADJ_KMAX * CPL;
  // the block's segment geometry and lengths, one copy per track (written by
  // its lane 0)
  Seg *s_geo_all = reinterpret_cast<Seg *>(s_adj + (size_t)2 * BLOCK * ADJ_KMAX * CPL);
  Seg *s_geo = s_geo_all + (size_t)sub * ADJ_KMAX;
  float *s_ds_all = reinterpret_cast<float *>(s_geo_all + (size_t)x.nsub * ADJ_KMAX);
  float *s_ds = s_ds_all + (size_t)sub * ADJ_KMAX;
  float *s_acc = s_ds_all + (size_t)x.nsub * ADJ_KMAX;
  const int64_t per_slice = (int64_t)x.n_sigt * a.ldg;
  float *acc = x.slices ? s_acc + sub * per_slice : nullptr;
  if (x.slices) {
    for (int64_t i = threadIdx.x; i < per_slice * x.nsub; i += BLOCK) s_acc[i] = 0.f;
    __syncthreads();
  }
  const int64_t warp_id = ((int64_t)blockIdx.x * BLOCK + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * BLOCK) >> 5;
  const int64_t PZ = (int64_t)a.P * a.Z;
  const int S = a.S, K = a.ck_k, NCK = a.ck_n;
  for (int64_t base = warp_id * GPW; base < a.n3d; base += n_warps * GPW) {
    const int64_t track = base + gw;
    const bool valid = !idle && track < a.n3d;
    const int64_t tr = track < a.n3d ? track : a.n3d - 1;
    const int64_t i2 = tr / PZ;
    const int j = (int)((tr / a.Z) % a.P);
    const float mu = a.mu[j];
    const float mu2 = mu * mu;
    const float w = a.weight[tr];
    const float w_mu = w * mu;
    const float *dsb = a.seg_ds + (i2 * a.P + j) * S;
    const int32_t *srcb = a.seg_src + tr * S;
    float4 pbar[CPL];
#pragma unroll
    for (int k = 0; k < CPL; ++k) pbar[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int b = NCK - 1; b >= 0; --b) {
      const int n0 = b * K;
      const int cnt = min(K, S - n0);
      float4 psi[CPL];
#pragma unroll
      for (int k = 0; k < CPL; ++k) {
        const int c = li + TPW * k;
        psi[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (c < a.nchunk)
          psi[k] = *reinterpret_cast<const float4 *>(a.ck_psi + (tr * NCK + b) * a.ldg + 4 * c);
      }
      // ---- recompute psi entering each segment of the block.  The loops over
      // the block stay rolled (unrolled, the derivative code outgrows the
      // instruction cache); each iteration issues the next segment's loads
      // before its own arithmetic (software pipeline, as the forward sweep).
      float z = a.ck_z[tr * NCK + b];
      float ds = __ldg(dsb + n0);
      Seg g = segment_geometry<true>(a, z, checked_source(a, __ldg(srcb + n0), li));
      // (one chunk a lane; with two the second set of operands would spill)
      constexpr bool PF = CPL == 1;
      {
        AdjFwdRows<CPL, QUAD> cur;
        if (PF) adj_load_fwd<CPL, QUAD>(a, g, li, TPW, cur);
#pragma unroll 1
        for (int jj = 0; jj < cnt; ++jj) {
          if (li == 0) {
            s_geo[jj] = g;
            s_ds[jj] = ds;
          }
          if (!PF) adj_load_fwd<CPL, QUAD>(a, g, li, TPW, cur);
          float ds1 = ds;
          Seg g1 = g;
          AdjFwdRows<CPL, QUAD> nxt = cur;
          if (jj + 1 < cnt) {
            z = advance_z(a, z, ds, mu);
            ds1 = __ldg(dsb + n0 + jj + 1);
            g1 = segment_geometry<true>(a, z, checked_source(a, __ldg(srcb + n0 + jj + 1), li));
            if (PF) adj_load_fwd<CPL, QUAD>(a, g1, li, TPW, nxt);
          }
          const MixedFit fit = QUAD ? mixed_fit(a, g.zin, mu, mu2) : MixedFit{};
#pragma unroll
          for (int k = 0; k < CPL; ++k) {
            hist_base[(jj * CPL + k) * BLOCK] = psi[k];
            const int c = li + TPW * k;
            if (c >= a.nchunk) continue;
            float4 ev;
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              float p = get(psi[k], e);
              float Ee = 0.f;
              if (QUAD)
                mixed_quad_e(get(cur.y[k][0], e), get(cur.y[k][QUAD ? 1 : 0], e),
                             get(cur.y[k][QUAD ? 2 : 0], e), fit, get(cur.sig[k], e),
                             get(cur.r1[k], e), get(cur.r2[k], e), get(cur.r3x2[k], e),
                             get(cur.r4[k], e), ds, w, p, Ee);
              else
                mixed_flat(get(cur.y[k][0], e), get(cur.sig[k], e), get(cur.r1[k], e), ds, w_mu,
                           p);
              set(psi[k], e, p);
              set(ev, e, Ee);
            }
            if (QUAD) ehist_base[(jj * CPL + k) * BLOCK] = ev;
          }
          g = g1;
          ds = ds1;
          if (PF) cur = nxt;
        }
      }
      __syncwarp();
      // ---- reverse through the block, the previous segment's loads issued
      // before this one's arithmetic
      {
        Seg gc = s_geo[cnt - 1];
        float dsc = s_ds[cnt - 1];
        AdjRevRows<CPL, QUAD> cur;
        if (PF) adj_load_rev<CPL, QUAD>(a, x, gc, li, TPW, cur);
#pragma unroll 1
        for (int jj = cnt - 1; jj >= 0; --jj) {
          if (!PF) adj_load_rev<CPL, QUAD>(a, x, gc, li, TPW, cur);
          Seg gn = gc;
          float dsn = dsc;
          AdjRevRows<CPL, QUAD> nxt = cur;
          if (jj > 0) {
            gn = s_geo[jj - 1];
            dsn = s_ds[jj - 1];
            if (PF) adj_load_rev<CPL, QUAD>(a, x, gn, li, TPW, nxt);
          }
          const int mat = gc.mat;
          const MixedFit2 fit2 = pair_fit(QUAD ? mixed_fit(a, gc.zin, mu, mu2) : MixedFit{});
          const float2 ds2 = bc2(dsc);
#pragma unroll
          for (int k = 0; k < CPL; ++k) {
            const int c = li + TPW * k;
            if (c >= a.nchunk) continue;
            const int g4 = 4 * c;
            const float4 ph = hist_base[(jj * CPL + k) * BLOCK];
            const float4 eh = QUAD ? ehist_base[(jj * CPL + k) * BLOCK] : ph;
            float4 b1, b2, b3, sb, f0, f1, f2;
            vzero(f0);
            vzero(f1);
            vzero(f2);
            if (QUAD) {
              // groups in pairs
              float2 pb[2], y1b[2], y2b[2], y3b[2], sbr[2], c0b[2], c1b[2], c2b[2];
#pragma unroll
              for (int h = 0; h < 2; ++h) {
                auto half = [h](const float4 &v) { return h ? hi2(v) : lo2(v); };
                const AdjOut2 o =
                    adj_quad2(half(cur.y[k][0]), half(cur.y[k][QUAD ? 1 : 0]),
                              half(cur.y[k][QUAD ? 2 : 0]), fit2, half(cur.sig[k]),
                              half(cur.r1[k]), ds2, half(eh), half(ph), half(pbar[k]),
                              mul2(half(cur.lam[k]), bc2(w)));
                pb[h] = o.pbar;
                y1b[h] = o.y1b;
                y2b[h] = o.y2b;
                y3b[h] = o.y3b;
                sbr[h] = o.sbar;
                if (FIT) {
                  // dL/d of the fit's c0, c1, c2 (q0 = c0 + c1 zin + c2 zin^2,
                  // q1 = c1 + 2 c2 zin, q2 = c2)
                  const float2 zin = bc2(gc.zin);
                  const float2 q1b = mul2(bc2(mu), o.q1mub), q2b = mul2(bc2(mu2), o.q2mu2b);
                  c0b[h] = o.q0b;
                  c1b[h] = fma2(o.q0b, zin, q1b);
                  c2b[h] = fma2(fma2(o.q0b, zin, mul2(bc2(2.f), q1b)), zin, q2b);
                }
              }
              pbar[k] = cat4(pb[0], pb[1]);
              b1 = cat4(y1b[0], y1b[1]);
              b2 = cat4(y2b[0], y2b[1]);
              b3 = cat4(y3b[0], y3b[1]);
              sb = cat4(sbr[0], sbr[1]);
              if (FIT) {
                f0 = cat4(c0b[0], c0b[1]);
                f1 = cat4(c1b[0], c1b[1]);
                f2 = cat4(c2b[0], c2b[1]);
              }
#pragma unroll
              for (int e = 0; e < 4; ++e)
                if (g4 + e >= a.G) set(sb, e, 0.f);
            } else {
#pragma unroll
              for (int e = 0; e < 4; ++e) {
                const AdjOut o = adj_flat(get(cur.y[k][0], e), get(cur.sig[k], e),
                                          get(cur.r1[k], e), dsc, get(ph, e), get(pbar[k], e),
                                          get(cur.lam[k], e) * w_mu);
                set(pbar[k], e, o.pbar);
                set(b1, e, o.y1b);
                set(b2, e, o.y2b);
                set(b3, e, o.y3b);
                set(sb, e, g4 + e < a.G ? o.sbar : 0.f);
              }
            }
            if (valid) {
              if (acc) {
                // one 16-byte read-modify-write per lane: the lanes of a
                // sub-warp own distinct chunks of the row, sub-warps own slices
                float4 *t = reinterpret_cast<float4 *>(acc + (int64_t)mat * a.ldg + g4);
                float4 v = *t;
                v.x += sb.x;
                v.y += sb.y;
                v.z += sb.z;
                v.w += sb.w;
                *t = v;
              } else {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                  if (g4 + e < a.G)
                    atomicAdd(x.dsig + (int64_t)mat * a.ldg + g4 + e, (double)get(sb, e));
              }
              float *dq = x.dq + gc.qrow + g4;
              red_add_v4(dq, b1.x, b1.y, b1.z, b1.w);
              if (QUAD) {
                red_add_v4(dq + a.ldg, b2.x, b2.y, b2.z, b2.w);
                red_add_v4(dq + 2 * a.ldg, b3.x, b3.y, b3.z, b3.w);
                if (FIT) {
                  // the fit window: its first row r0 of source s (rows s F + r0 ..)
                  const int64_t wrow = gc.qrow / a.ldg;
                  const int64_t src = wrow / a.F, r0 = wrow - src * a.F;
                  float *df = x.dfit + ((src * (a.F - 2) + r0) * 3) * a.ldg + g4;
                  red_add_v4(df, f0.x, f0.y, f0.z, f0.w);
                  red_add_v4(df + a.ldg, f1.x, f1.y, f1.z, f1.w);
                  red_add_v4(df + 2 * a.ldg, f2.x, f2.y, f2.z, f2.w);
                }
              }
            }
          }
          gc = gn;
          dsc = dsn;
          if (PF) cur = nxt;
        }
      }
      __syncwarp();
    }
    if (valid && x.dpsi_in) {
#pragma unroll
      for (int k = 0; k < CPL; ++k) {
        const int c = li + TPW * k;
        for (int e = 0; e < 4; ++e)
          if (c < a.nchunk && 4 * c + e < a.G) x.dpsi_in[tr * a.G + 4 * c + e] = get(pbar[k], e);
      }
    }
  }
  if (x.slices) {
    __syncthreads();
    for (int64_t i = threadIdx.x; i < per_slice; i += BLOCK) {
      double v = 0.0;
      for (int sl = 0; sl < x.nsub; ++sl) v += (double)s_acc[sl * per_slice + i];
      if (v != 0.0) atomicAdd(x.dsig + i, v);
    }
  }
}


template <int CPL, bool QUAD>
int launch_adj_t(moc_problem *p, const AdjArgs &x, int tpw) {
  auto kern = x.dfit ? adjoint_kernel<CPL, QUAD, true> : adjoint_kernel<CPL, QUAD, false>;
  AdjArgs y = x;
  y.tpw = tpw;
  y.nsub = (BLOCK / 32) * (32 / tpw);
  const size_t slice_bytes = sizeof(float) * (size_t)x.n_sigt * x.a.ldg * y.nsub;
  const size_t fixed = adj_hist_bytes<CPL>() + (sizeof(Seg) + sizeof(float)) * y.nsub * ADJ_KMAX;
  // per-track dL/dsigma_t accumulators in shared memory while two blocks still
  // fit an SM (227 KB each at most, 228 KB an SM with 1 KB reserved a block);
  // otherwise FP64 atomics straight to global memory
  y.slices = fixed + slice_bytes <= 113 * 1024 ? 1 : 0;
  const size_t smem = fixed + (y.slices ? slice_bytes : 0);
  if (smem > 48 * 1024)
    MOC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0, sms = 0;
  MOC_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BLOCK, smem));
  MOC_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device));
  if (per_sm < 1) return MOC_ERR_UNSUPPORTED;
  const int gpw = 32 / tpw;
  const int64_t warps = (x.a.n3d + gpw - 1) / gpw;
  int64_t grid = (int64_t)per_sm * sms;
  const int64_t need = (warps + 7) / 8;
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, BLOCK, smem, p->stream>>>(y);
  MOC_CUDA_TRY(cudaGetLastError());
  p->launches++;
  return MOC_OK;
}

// Lanes per track of the reverse sweep: every lane holds one float4 chunk up
// to 32 chunks (128 groups), two beyond (256 groups); p->adj_tpw/adj_cpl
// override.
template <bool QUAD>
int dispatch_adj(moc_problem *p, const AdjArgs &x) {
  const int nchunk = p->ldg / 4;
  int cpl = nchunk <= 32 ? 1 : 2;
  if (p->adj_cpl > 0) cpl = p->adj_cpl;
  int tpw = p->adj_tpw > 0 ? p->adj_tpw : (nchunk + cpl - 1) / cpl;
  if (tpw < 1 || tpw > 32 || (int64_t)tpw * cpl < nchunk) return MOC_ERR_UNSUPPORTED;
  if (cpl == 1) return launch_adj_t<1, QUAD>(p, x, tpw);
  if (cpl == 2) return launch_adj_t<2, QUAD>(p, x, tpw);
  return MOC_ERR_UNSUPPORTED;
}

template <bool QUAD>
int dispatch_ckpt(moc_problem *p, const SweepArgs &a) {
  const int nchunk = p->ldg / 4;
  if (nchunk <= 8) return launch_t<8, 1, MODE_MIXED, QUAD, false, true>(p, a);
  // 33 to 40 groups: 10 lanes of one 4-group chunk, three tracks a warp
  if (p->ldg <= 40) return launch_t<10, 1, MODE_MIXED, QUAD, false, true>(p, a);
  // 33 to 100 groups: two-group chunks, three tracks a warp (the forward sweep's
  // 10 x 5 shape; 16 lanes of float4 chunks would leave most of them idle)
  if (p->ldg <= 100) return launch_t<10, 5, MODE_MIXED, QUAD, false, true, 2>(p, a);
  if (nchunk <= 16) return launch_t<16, 1, MODE_MIXED, QUAD, false, true>(p, a);
  if (nchunk <= 32) return launch_t<32, 1, MODE_MIXED, QUAD, false, true>(p, a);
  if (nchunk <= 64) return launch_t<32, 2, MODE_MIXED, QUAD, false, true>(p, a);
  return MOC_ERR_UNSUPPORTED;
}

}  // namespace

// Forward sweep (MIXED) storing psi and the height every k segments.
int moc_launch_sweep_ckpt(moc_problem *p, float *ck_psi, float *ck_z, int k, int nck) {
  SweepArgs a = build_args(p);
  a.phi_lo = nullptr;
  a.ck_psi = ck_psi;
  a.ck_z = ck_z;
  a.ck_k = k;
  a.ck_n = nck;
  return p->d.axial_exp == 2 ? dispatch_ckpt<true>(p, a) : dispatch_ckpt<false>(p, a);
}

int moc_launch_adjoint(moc_problem *p, const float *ck_psi, const float *ck_z, int k, int nck,
                       const float *dphi, float *dq, double *dsig, float *dpsi_in, float *dfit) {
  if (k < 1 || k > ADJ_KMAX) return MOC_ERR_ARG;
  AdjArgs x{};
  x.a = build_args(p);
  x.a.psi_scale = nullptr;
  x.a.ck_psi = const_cast<float *>(ck_psi);
  x.a.ck_z = const_cast<float *>(ck_z);
  x.a.ck_k = k;
  x.a.ck_n = nck;
  x.dphi = dphi;
  x.dq = dq;
  x.dsig = dsig;
  x.dpsi_in = dpsi_in;
  x.dfit = dfit;
  x.n_sigt = p->d.n_sigt;
  return p->d.axial_exp == 2 ? dispatch_adj<true>(p, x) : dispatch_adj<false>(p, x);
}
