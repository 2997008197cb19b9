// moc_refabi.cu -- the reference's four solver entry points (transport_sweep,
// renormalize_flux, update_sources, compute_keff; src/SimpleMOC_header.h:225,
// 235-237) served on the GPU, with the reference's own structs as arguments.
//
// transport_sweep reproduces the reference traversal (src/solver.c:347-523)
// on the device in two passes of a geometry kernel, one warp per (2D track,
// polar angle) and lanes over the stacked rays:
//   pass 0 counts the axial sub-segments of every 3D track and of every
//          (2D track, polar angle) pair;
//   pass 1 lays the sub-segments of each 3D track out contiguously (length,
//          start height, source region) and updates the stacked-ray heights;
// then the sweep kernel attenuates those variable-length streams.  The
// reference processes the stacked rays of a segment in order and retires one
// ray per boundary hit (end_stacked-- / begin_stacked++, src/solver.c:460-473),
// which couples the rays; the warp evaluates every ray's hit speculatively and
// finds the processed prefix with ballots, which is exactly the sequential
// rule.  Source regions are rand() % NS drawn on the host in traversal order
// (the sequence of the reference's serial build for the caller's srand seed) or
// a counter hash.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "moc_internal.h"
#include "simplemoc_refabi.h"

namespace {

constexpr unsigned FULL = 0xffffffffu;
// Splits allowed for one 3D track across one 2D segment; a valid geometry needs
// at most (segment height / fine interval + 2).  The bound only keeps a
// malformed input from looping; reaching it is reported as an argument error.
constexpr int MAX_SPLITS = 1 << 16;

inline uint64_t mix64_host(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct RefArgs {
  int64_t n2d;
  int P, Z;
  const int64_t *seg_off;   // [N2D+1]
  const float *seg_len;     // [M2D]
  const double *cos_d;      // [P] cos(polar angle) in double
  const double *sin_d;      // [P]
  float fine_dz_f;          // (float)fine_delta_z, the dz of get_pos/neg_interval
  double fine_dz;           // fine_delta_z
  double node_dz;           // node_delta_z
  float sep;                // Input.axial_z_sep
  int64_t ns;
  uint64_t ns_m;            // floor((2^64 - 1) / ns), for mod_barrett
  float *z;                 // [N3D] stacked-ray heights (pass 0: a scratch copy)
  int32_t *cnt;             // [N3D] pass 0: sub-segments; pass 1: emitted so far
  int64_t *ij_tot;          // [N2D*P]
  const int64_t *ij_base;   // [N2D*P]
  int64_t *off;             // [N3D+1]
  float *sds, *sz;          // [M]
  int32_t *ssrc;            // [M]
  const int32_t *rng;       // [M] rand() values in traversal order, or null
  uint64_t hash_key;
  int32_t *err;             // device error word of the core problem
};

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// x mod d for d >= 1 by Barrett reduction, given m = floor((2^64 - 1) / d):
// q = umulhi(x, m) is floor(x / d) or one less (x m / 2^64 lies in
// (x/d - 1, x/d]), so x - q d is the remainder or the remainder + d.  Exact
// for every 64-bit x, at a fraction of the cost of a 64-bit division.
__device__ __forceinline__ uint64_t mod_barrett(uint64_t x, uint64_t d, uint64_t m) {
  const uint64_t q = __umul64hi(x, m);
  uint64_t r = x - q * d;
  if (r >= d) r -= d;
  return r;
}

// The source region of the sub-segment drawn q-th in traversal order
// (src/solver.c:476-483): the reference's rand() value (never negative) modulo
// the region count, or the counter hash modulo the region count.
__device__ __forceinline__ int32_t sub_segment_source(const RefArgs &r, int64_t q) {
  if (r.rng) {
    const int32_t v = r.rng[q];
    return v >= 0 ? (int32_t)mod_barrett((uint64_t)v, (uint64_t)r.ns, r.ns_m)
                  : (int32_t)((int64_t)v % r.ns);
  }
  return (int32_t)mod_barrett(mix64(r.hash_key + (uint64_t)q * 0x9E3779B97F4A7C15ull),
                              (uint64_t)r.ns, r.ns_m);
}

// Staged stores of the emitting pass.  Each lane writes the sub-segments of a
// different stacked ray, so direct 4-byte stores scatter over as many sectors
// as lanes; partly written sectors then cost a read and a write each in DRAM.
// Instead each ray's entries collect in a STAGE_N-entry group in shared memory
// (ds, z, source: 3 STAGE_N words) and leave as whole 16-byte pieces of each
// stream once the group is full; the two pieces of a 32-byte sector meet in L2.
// A ray's first and last groups are shared with the neighbouring rays' streams
// and go out entry by entry.
constexpr int STAGE_N = 4;
constexpr int STAGE_W = 3 * STAGE_N;     // words per ray

// Writes the entries [max(g0, first), end) of the group that ends at `end`
// (g0 = the group's first slot, a multiple of STAGE_N).
__device__ __forceinline__ void stage_flush(const RefArgs &r, const float *buf, int64_t first,
                                            int64_t end) {
  const int64_t g0 = (end - 1) & ~int64_t(STAGE_N - 1);
  const int32_t *bsrc = reinterpret_cast<const int32_t *>(buf + 2 * STAGE_N);
  if (g0 >= first && end - g0 == STAGE_N) {
    // whole group: the streams are 256-byte aligned, so slot g0 starts a 16-byte piece
    float4 *ds4 = reinterpret_cast<float4 *>(r.sds + g0);
    float4 *z4 = reinterpret_cast<float4 *>(r.sz + g0);
    int4 *s4 = reinterpret_cast<int4 *>(r.ssrc + g0);
#pragma unroll
    for (int v = 0; v < STAGE_N / 4; ++v) {
      ds4[v] = make_float4(buf[4 * v], buf[4 * v + 1], buf[4 * v + 2], buf[4 * v + 3]);
      z4[v] = make_float4(buf[STAGE_N + 4 * v], buf[STAGE_N + 4 * v + 1],
                          buf[STAGE_N + 4 * v + 2], buf[STAGE_N + 4 * v + 3]);
      s4[v] = make_int4(bsrc[4 * v], bsrc[4 * v + 1], bsrc[4 * v + 2], bsrc[4 * v + 3]);
    }
    return;
  }
  for (int64_t x = g0 > first ? g0 : first; x < end; ++x) {
    const int e = (int)(x - g0);
    r.sds[x] = buf[e];
    r.sz[x] = buf[STAGE_N + e];
    r.ssrc[x] = bsrc[e];
  }
}

// One entry of a ray's stream at slot x: into its group, which goes out when
// its last entry arrives.
__device__ __forceinline__ void stage_put(const RefArgs &r, float *buf, int64_t first, int64_t x,
                                          float ds, float zh, int32_t src) {
  const int e = (int)(x & (STAGE_N - 1));
  buf[e] = ds;
  buf[STAGE_N + e] = zh;
  reinterpret_cast<int32_t *>(buf + 2 * STAGE_N)[e] = src;
  if (e == STAGE_N - 1) stage_flush(r, buf, first, x + 1);
}

// One 3D track over one 2D segment: the while loop of src/solver.c:409-524.
// Returns the number of sub-segments; *hit = the track reached a domain bound
// (and was reset); zh is updated by the reference's rule (src/solver.c:514-523).
// EMIT: the sub-segments go to slots slot, slot + 1, ... of the streams, through
// the ray's staging group `stg` (the ray's stream starts at slot `first`) or,
// with stg null, directly.
// KEEP (counting call of the emitting pass): the first KEEP sub-segments'
// (ds, height) also go to keep[], so that the emitting call can be skipped.
template <bool EMIT, int KEEP = 0>
__device__ int track_segment(const RefArgs &r, bool pos, double cos_d, float s_full, float &zh,
                             bool last_seg, int k, bool *hit, int64_t slot, int64_t seq,
                             float *stg = nullptr, int64_t first = 0,
                             float2 *keep = nullptr) {
  float s = s_full;
  // get_pos_interval / get_neg_interval (src/solver.c:895-907): float z / dz
  int curr = pos ? __float2int_rz(__fdiv_rn(zh, r.fine_dz_f))
                 : (int)ceilf(__fdiv_rn(zh, r.fine_dz_f));
  bool complete = false;
  int count = 0;
  *hit = false;
  while (!complete) {
    if (count >= MAX_SPLITS) {
      atomicOr(r.err, 1);
      break;
    }
    bool reset = false;
    // float z = z_height + s * cos(p_angle): double arithmetic, rounded to float
    float z = __double2float_rn(__dadd_rn((double)zh, __dmul_rn((double)s, cos_d)));
    const int nw = pos ? __float2int_rz(__fdiv_rn(z, r.fine_dz_f))
                       : (int)ceilf(__fdiv_rn(z, r.fine_dz_f));
    float ds;
    if (nw == curr) {
      complete = true;
      ds = s;
    } else {
      curr += pos ? 1 : -1;
      z = __double2float_rn(__dmul_rn(r.fine_dz, (double)__int2float_rn(curr)));
      ds = __double2float_rn(__ddiv_rn((double)__fsub_rn(z, zh), cos_d));
      s = __fsub_rn(s, ds);
      if (s <= 0.f) complete = true;
      if (z <= 0.f || (double)z >= r.node_dz) {
        complete = true;
        reset = true;
        *hit = true;
      }
    }
    if (KEEP > 0 && count < KEEP) keep[count] = make_float2(ds, zh);
    if (EMIT) {
      const int32_t src = sub_segment_source(r, seq + count);
      if (stg) {
        stage_put(r, stg, first, slot + count, ds, zh, src);
      } else {
        r.sds[slot + count] = ds;
        r.sz[slot + count] = zh;
        r.ssrc[slot + count] = src;
      }
    }
    ++count;
    if (last_seg || reset)
      zh = pos ? __fmul_rn(r.sep, (float)k) : __fmul_rn(r.sep, (float)(k + 1));
    else
      zh = z;
  }
  return count;
}

__device__ __forceinline__ int warp_incl_scan(int v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(FULL, v, o);
    if (lane >= o) v += u;
  }
  return v;
}

// Sub-segments of one ray over one 2D segment that the emitting pass keeps from
// its counting call (about one on average; more are evaluated again).
constexpr int REF_KEEP = 4;

// STAGED (pass 1): the warp's stacked rays keep their staging groups in
// dynamic shared memory, STAGE_W words per ray, Z rays per warp.
template <int PASS, bool STAGED = false>
__global__ void __launch_bounds__(128) ref_expand(RefArgs r) {
  extern __shared__ float s_stage[];
  const int lane = threadIdx.x & 31;
  float *wstage = STAGED ? s_stage + (size_t)(threadIdx.x >> 5) * r.Z * STAGE_W : nullptr;
  const int64_t ij = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (ij >= r.n2d * r.P) return;        // uniform per warp
  const int64_t i = ij / r.P;
  const int j = (int)(ij % r.P);
  const bool pos = j < r.P / 2;          // src/solver.c:367-371
  const double cos_d = r.cos_d[j], sin_d = r.sin_d[j];
  const int64_t s0 = r.seg_off[i], nseg = r.seg_off[i + 1] - s0;
  float *zst = r.z + ij * r.Z;
  int32_t *cst = r.cnt + ij * r.Z;
  if (PASS == 1) {
    // this pair's streams occupy [ij_base, ij_base + total) in both the
    // traversal order and the per-track layout
    int64_t run = r.ij_base[ij];
    for (int kc = 0; kc < r.Z; kc += 32) {
      const int k = kc + lane;
      const int c = k < r.Z ? cst[k] : 0;
      const int incl = warp_incl_scan(c, lane);
      if (k < r.Z) {
        r.off[ij * r.Z + k] = run + incl - c;
        cst[k] = 0;
      }
      run += __shfl_sync(FULL, incl, 31);
    }
    __syncwarp();
  }
  int begin = 0, end = r.Z;
  int64_t local = 0;
  for (int64_t n = 0; n < nseg; ++n) {
    const float s_full = __double2float_rn(__ddiv_rn((double)r.seg_len[s0 + n], sin_d));
    const bool last_seg = n == nseg - 1;
    int e_cur = end, hits = 0;
    for (int kc = begin; kc < (pos ? e_cur : end); kc += 32) {
      const int k = kc + lane;
      const bool active = k < (pos ? e_cur : end);
      bool hit = false;
      int c = 0;
      float zh = 0.f;
      // pass 1: the sub-segments of this call, emitted below without a second
      // evaluation of the double-precision split when they all fit
      float2 keep[PASS == 1 ? REF_KEEP : 1];
      if (active) {
        zh = zst[k];
        c = track_segment<false, PASS == 1 ? REF_KEEP : 0>(r, pos, cos_d, s_full, zh, last_seg,
                                                           k, &hit, 0, 0, nullptr, 0, keep);
      }
      const unsigned amask = __ballot_sync(FULL, active);
      const unsigned H = __ballot_sync(FULL, active && hit);
      unsigned proc = amask;
      bool cut = false;
      if (pos) {
        // ray k runs iff k < end_stacked at its turn: hits of the rays before it
        // in this chunk have already lowered end_stacked (src/solver.c:466-467)
        const unsigned lt = (1u << lane) - 1u;
        const bool cond = active && (k < e_cur - __popc(H & lt));
        const unsigned C = __ballot_sync(FULL, cond);
        const unsigned fail = amask & ~C;
        if (fail) {
          proc = C & ((1u << (__ffs(fail) - 1)) - 1u);
          cut = true;
        }
      }
      const bool mine = (proc >> lane) & 1u;
      const int cm = mine ? c : 0;
      const int incl = warp_incl_scan(cm, lane);
      if (mine) {
        if (PASS == 0) {
          zst[k] = zh;
          cst[k] += c;
        } else {
          const int64_t t = ij * r.Z + k;
          const int64_t first = r.off[t], slot = first + cst[k];
          const int64_t seq = r.ij_base[ij] + local + (incl - cm);
          float *stg = STAGED ? wstage + (size_t)k * STAGE_W : nullptr;
          if (c <= REF_KEEP) {
            for (int q = 0; q < c; ++q) {
              const int32_t src = sub_segment_source(r, seq + q);
              if (stg) {
                stage_put(r, stg, first, slot + q, keep[q].x, keep[q].y, src);
              } else {
                r.sds[slot + q] = keep[q].x;
                r.sz[slot + q] = keep[q].y;
                r.ssrc[slot + q] = src;
              }
            }
            zst[k] = zh;
          } else {
            float zz = zst[k];
            bool h2;
            track_segment<true>(r, pos, cos_d, s_full, zz, last_seg, k, &h2, slot, seq, stg,
                                first);
            zst[k] = zz;
          }
          cst[k] += c;
        }
      }
      local += __shfl_sync(FULL, incl, 31);
      if (pos) {
        e_cur -= __popc(H & proc);
        if (cut) break;
      } else {
        hits += __popc(H);
      }
    }
    if (pos)
      end = e_cur;
    else
      begin += hits;                     // src/solver.c:468-469
  }
  if (PASS == 0 && lane == 0) r.ij_tot[ij] = local;
  if (PASS == 1 && STAGED) {
    // the last, partly filled group of every ray
    __syncwarp();
    for (int k = lane; k < r.Z; k += 32) {
      const int64_t first = r.off[ij * r.Z + k], end = first + cst[k];
      if (end > first && (end & (STAGE_N - 1)) != 0)
        stage_flush(r, wstage + (size_t)k * STAGE_W, first, end);
    }
  }
}

// ---------------------------------------------------------------------------
// device state of the reference entry points
// ---------------------------------------------------------------------------
struct RefState {
  moc_problem *p = nullptr;
  const void *k_sources = nullptr, *k_tracks = nullptr, *k_tracks2d = nullptr;
  int64_t n2d = 0, n3d = 0, ns = 0;
  int P = 0, Z = 0, G = 0, F = 0;
  float sep = 0.f;
  double fine_dz = 0.0, node_dz = 0.0;
  int64_t *d_seg_off = nullptr;
  float *d_seg_len = nullptr;
  double *d_cos = nullptr, *d_sin = nullptr;
  float *d_z = nullptr, *d_zc = nullptr;
  int32_t *d_cnt = nullptr;
  int64_t *d_ij_tot = nullptr, *d_ij_base = nullptr, *d_off = nullptr;
  float *d_sds = nullptr, *d_sz = nullptr;
  int32_t *d_ssrc = nullptr, *d_rng = nullptr;
  int32_t *h_rng = nullptr;       // pinned staging of the rand() draws
  int64_t cap = 0, h_rng_cap = 0;
  int64_t sweeps = 0;
  int64_t last_segments = 0;
  double last_rng_ms = 0.0;
};

std::mutex g_mu;
RefState g_ref;
int g_status = MOC_OK;
int g_rng_mode = MOC_REF_RNG_LIBC;
uint64_t g_rng_seed = 0;

template <typename T>
void dfree(T *&ptr) {
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
}

void release_ref() {
  RefState &r = g_ref;
  if (r.p) moc_destroy(r.p);
  dfree(r.d_seg_off); dfree(r.d_seg_len); dfree(r.d_cos); dfree(r.d_sin); dfree(r.d_z);
  dfree(r.d_zc); dfree(r.d_cnt); dfree(r.d_ij_tot); dfree(r.d_ij_base); dfree(r.d_off);
  dfree(r.d_sds); dfree(r.d_sz); dfree(r.d_ssrc); dfree(r.d_rng);
  if (r.h_rng) cudaFreeHost(r.h_rng);
  r = RefState();
}

template <typename T>
int dmalloc(T **ptr, int64_t count) {
  if (count < 1) count = 1;
  if (cudaMalloc(ptr, sizeof(T) * (size_t)count) != cudaSuccess) {
    cudaGetLastError();
    return MOC_ERR_OOM;
  }
  return MOC_OK;
}

#define RTRY(x)                     \
  do {                              \
    int rc_ = (x);                  \
    if (rc_ != MOC_OK) return rc_;  \
  } while (0)

int device_from_env() {
  const char *e = getenv("SIMPLEMOC_GB300_DEVICE");
  return e ? atoi(e) : 0;
}

// Flattens the reference's Params (pointer-per-row storage of src/source.c and
// src/tracks.c) into the library's layout and uploads it.
int upload_ref(const moc_ref_params *prm, const moc_ref_input *I) {
  release_ref();
  RefState &r = g_ref;
  const int64_t G = I->n_egroups, F = I->fai, NS = I->n_source_regions_per_node;
  const int64_t N2D = I->ntracks_2D, P = I->n_polar_angles, Z = I->z_stacked;
  if (G < 1 || F < 1 || NS < 1 || N2D < 1 || P < 1 || Z < 1 || !prm->sources || !prm->tracks ||
      !prm->tracks_2D || !prm->polar_angles || !prm->expTable.values || prm->expTable.N < 1)
    return MOC_ERR_ARG;
  const int64_t N3D = N2D * P * Z;
  // sources; cross-section sets are identified by their row pointers (the
  // reference shares them between sources, src/source.c:189-192)
  std::vector<float> q((size_t)(NS * F * G)), phi((size_t)(NS * F * G)), sigt((size_t)(NS * G));
  std::vector<float> vol((size_t)NS), xs, scat;
  std::vector<int32_t> src_sigt((size_t)NS), src_xs((size_t)NS);
  std::map<std::pair<const void *, const void *>, int32_t> xs_id;
  for (int64_t s = 0; s < NS; ++s) {
    const moc_ref_source &S = prm->sources[s];
    for (int64_t f = 0; f < F; ++f) {
      memcpy(&q[(size_t)((s * F + f) * G)], S.fine_source[f], sizeof(float) * (size_t)G);
      memcpy(&phi[(size_t)((s * F + f) * G)], S.fine_flux[f], sizeof(float) * (size_t)G);
    }
    memcpy(&sigt[(size_t)(s * G)], S.sigT, sizeof(float) * (size_t)G);
    src_sigt[(size_t)s] = (int32_t)s;
    vol[(size_t)s] = S.vol;
    auto key = std::make_pair((const void *)S.XS, (const void *)S.scattering_matrix);
    auto it = xs_id.find(key);
    if (it == xs_id.end()) {
      const int32_t m = (int32_t)xs_id.size();
      it = xs_id.emplace(key, m).first;
      for (int64_t g = 0; g < G; ++g)
        for (int c = 0; c < 3; ++c) xs.push_back(S.XS[g][c]);
      for (int64_t g = 0; g < G; ++g)
        for (int64_t g2 = 0; g2 < G; ++g2) scat.push_back(S.scattering_matrix[g][g2]);
    }
    src_xs[(size_t)s] = it->second;
  }
  // tracks
  std::vector<int64_t> seg_off((size_t)N2D + 1, 0);
  for (int64_t i = 0; i < N2D; ++i) seg_off[(size_t)i + 1] = seg_off[(size_t)i] + prm->tracks_2D[i].n_segments;
  std::vector<float> seg_len((size_t)seg_off[(size_t)N2D]), az((size_t)N2D);
  for (int64_t i = 0; i < N2D; ++i) {
    az[(size_t)i] = prm->tracks_2D[i].az_weight;
    for (int64_t n = 0; n < prm->tracks_2D[i].n_segments; ++n)
      seg_len[(size_t)(seg_off[(size_t)i] + n)] = prm->tracks_2D[i].segments[n].length;
  }
  std::vector<float> pw((size_t)N3D), z((size_t)N3D), psi_f((size_t)(N3D * G)), psi_b((size_t)(N3D * G));
  for (int64_t i = 0; i < N2D; ++i)
    for (int64_t j = 0; j < P; ++j)
      for (int64_t k = 0; k < Z; ++k) {
        const moc_ref_track &T = prm->tracks[i][j][k];
        const int64_t t = (i * P + j) * Z + k;
        pw[(size_t)t] = T.p_weight;
        z[(size_t)t] = T.z_height;
        memcpy(&psi_f[(size_t)(t * G)], T.f_psi, sizeof(float) * (size_t)G);
        memcpy(&psi_b[(size_t)(t * G)], T.b_psi, sizeof(float) * (size_t)G);
      }
  // the core problem: one dummy explicit segment per 3D track (the sweep uses
  // the variable-length streams instead)
  std::vector<float> dummy_len((size_t)N2D, 0.f);
  std::vector<int32_t> dummy_src((size_t)N3D, 0);
  moc_dims d{};
  d.n_groups = (int32_t)G;
  d.fai = (int32_t)F;
  d.cai = I->cai;
  d.decomp_ax = I->decomp_assemblies_ax;
  d.height = I->height;
  d.axial_exp = I->axial_exp;
  d.n_sources = NS;
  d.n_sigt = (int32_t)NS;
  d.n_xs = (int32_t)xs_id.size();
  d.n_tracks_2d = N2D;
  d.n_polar = (int32_t)P;
  d.z_stacked = (int32_t)Z;
  d.n_seg = 1;
  d.table_n = prm->expTable.N;
  d.table_dx = prm->expTable.dx;
  d.table_maxval = prm->expTable.maxVal;
  moc_host h{};
  h.seg_len = dummy_len.data();
  h.seg_src = dummy_src.data();
  h.az_weight = az.data();
  h.p_weight = pw.data();
  h.z0 = z.data();
  h.polar_angles = prm->polar_angles;
  h.src_sigt = src_sigt.data();
  h.src_xs = src_xs.data();
  h.vol = vol.data();
  h.sigt = sigt.data();
  h.xs = xs.data();
  h.scatter = scat.data();
  h.fine_source = q.data();
  h.fine_flux = phi.data();
  h.psi_f = psi_f.data();
  h.psi_b = psi_b.data();
  h.table = prm->expTable.values;
  RTRY(moc_create(&d, &h, device_from_env(), &r.p));
  r.k_sources = prm->sources;
  r.k_tracks = prm->tracks;
  r.k_tracks2d = prm->tracks_2D;
  r.n2d = N2D;
  r.n3d = N3D;
  r.ns = NS;
  r.P = (int)P;
  r.Z = (int)Z;
  r.G = (int)G;
  r.F = (int)F;
  r.sep = I->axial_z_sep;
  r.node_dz = I->height / I->decomp_assemblies_ax;          // src/solver.c:288
  r.fine_dz = r.node_dz / (I->cai * I->fai);                // src/solver.c:289
  std::vector<double> cd((size_t)P), sd((size_t)P);
  for (int64_t j = 0; j < P; ++j) {
    cd[(size_t)j] = cos((double)prm->polar_angles[j]);
    sd[(size_t)j] = sin((double)prm->polar_angles[j]);
  }
  RTRY(dmalloc(&r.d_seg_off, N2D + 1));
  RTRY(dmalloc(&r.d_seg_len, (int64_t)seg_len.size()));
  RTRY(dmalloc(&r.d_cos, P));
  RTRY(dmalloc(&r.d_sin, P));
  RTRY(dmalloc(&r.d_z, N3D));
  RTRY(dmalloc(&r.d_zc, N3D));
  RTRY(dmalloc(&r.d_cnt, N3D));
  RTRY(dmalloc(&r.d_ij_tot, N2D * P));
  RTRY(dmalloc(&r.d_ij_base, N2D * P));
  RTRY(dmalloc(&r.d_off, N3D + 1));
  cudaStream_t st = r.p->stream;
  MOC_CUDA_TRY(cudaMemcpyAsync(r.d_seg_off, seg_off.data(), sizeof(int64_t) * seg_off.size(),
                               cudaMemcpyHostToDevice, st));
  MOC_CUDA_TRY(cudaMemcpyAsync(r.d_seg_len, seg_len.data(), sizeof(float) * seg_len.size(),
                               cudaMemcpyHostToDevice, st));
  MOC_CUDA_TRY(cudaMemcpyAsync(r.d_cos, cd.data(), sizeof(double) * cd.size(), cudaMemcpyHostToDevice, st));
  MOC_CUDA_TRY(cudaMemcpyAsync(r.d_sin, sd.data(), sizeof(double) * sd.size(), cudaMemcpyHostToDevice, st));
  MOC_CUDA_TRY(cudaMemcpyAsync(r.d_z, z.data(), sizeof(float) * z.size(), cudaMemcpyHostToDevice, st));
  MOC_CUDA_TRY(cudaStreamSynchronize(st));
  return MOC_OK;
}

int ensure_state(const moc_ref_params *prm, const moc_ref_input *I) {
  const RefState &r = g_ref;
  if (r.p && r.k_sources == prm->sources && r.k_tracks == prm->tracks &&
      r.k_tracks2d == prm->tracks_2D && r.ns == I->n_source_regions_per_node &&
      r.G == I->n_egroups && r.n2d == I->ntracks_2D && r.P == I->n_polar_angles &&
      r.Z == I->z_stacked)
    return moc_status(r.p) == MOC_OK ? MOC_OK : MOC_ERR_STATE;
  return upload_ref(prm, I);
}

RefArgs make_args(RefState &r, float *z) {
  RefArgs a{};
  a.n2d = r.n2d;
  a.P = r.P;
  a.Z = r.Z;
  a.seg_off = r.d_seg_off;
  a.seg_len = r.d_seg_len;
  a.cos_d = r.d_cos;
  a.sin_d = r.d_sin;
  a.fine_dz_f = (float)r.fine_dz;
  a.fine_dz = r.fine_dz;
  a.node_dz = r.node_dz;
  a.sep = r.sep;
  a.ns = r.ns;
  a.ns_m = ~0ull / (uint64_t)r.ns;
  a.z = z;
  a.cnt = r.d_cnt;
  a.ij_tot = r.d_ij_tot;
  a.ij_base = r.d_ij_base;
  a.off = r.d_off;
  a.sds = r.d_sds;
  a.sz = r.d_sz;
  a.ssrc = r.d_ssrc;
  a.rng = g_rng_mode == MOC_REF_RNG_LIBC ? r.d_rng : nullptr;
  a.hash_key = mix64_host(g_rng_seed * 0x9E3779B97F4A7C15ull + (uint64_t)r.sweeps);
  a.err = r.p->err;
  return a;
}

int sweep_ref(int64_t *segments) {
  RefState &r = g_ref;
  cudaStream_t st = r.p->stream;
  const int64_t pairs = r.n2d * r.P;
  const unsigned grid = (unsigned)((pairs * 32 + 127) / 128);
  // pass 0 on a copy of the heights: counts only
  MOC_CUDA_TRY(cudaMemcpyAsync(r.d_zc, r.d_z, sizeof(float) * (size_t)r.n3d,
                               cudaMemcpyDeviceToDevice, st));
  MOC_CUDA_TRY(cudaMemsetAsync(r.d_cnt, 0, sizeof(int32_t) * (size_t)r.n3d, st));
  ref_expand<0><<<grid, 128, 0, st>>>(make_args(r, r.d_zc));
  MOC_CUDA_TRY(cudaGetLastError());
  std::vector<int64_t> tot((size_t)pairs), base((size_t)pairs);
  MOC_CUDA_TRY(cudaMemcpyAsync(tot.data(), r.d_ij_tot, sizeof(int64_t) * (size_t)pairs,
                               cudaMemcpyDeviceToHost, st));
  MOC_CUDA_TRY(cudaStreamSynchronize(st));
  int64_t M = 0;
  for (int64_t k = 0; k < pairs; ++k) {
    base[(size_t)k] = M;
    M += tot[(size_t)k];
  }
  if (M > r.cap) {
    dfree(r.d_sds); dfree(r.d_sz); dfree(r.d_ssrc); dfree(r.d_rng);
    const int64_t cap = M + M / 8 + 1024;
    RTRY(dmalloc(&r.d_sds, cap));
    RTRY(dmalloc(&r.d_sz, cap));
    RTRY(dmalloc(&r.d_ssrc, cap));
    RTRY(dmalloc(&r.d_rng, cap));
    r.cap = cap;
  }
  r.last_rng_ms = 0.0;
  if (g_rng_mode == MOC_REF_RNG_LIBC && M > 0) {
    // the serial reference draws rand() once per sub-segment in traversal
    // order (src/solver.c:481); the same draws, from the process's libc state,
    // in bulk where libc's generator allows it (moc_libc_rand.cpp)
    if (M > r.h_rng_cap) {
      if (r.h_rng) cudaFreeHost(r.h_rng);
      r.h_rng = nullptr;
      r.h_rng_cap = 0;
      const int64_t cap = M + M / 8 + 1024;
      MOC_CUDA_TRY(cudaMallocHost(&r.h_rng, sizeof(int32_t) * (size_t)cap));
      r.h_rng_cap = cap;
    }
    const auto t0 = std::chrono::steady_clock::now();
    moc_libc_draws(r.h_rng, M);
    r.last_rng_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    MOC_CUDA_TRY(cudaMemcpyAsync(r.d_rng, r.h_rng, sizeof(int32_t) * (size_t)M,
                                 cudaMemcpyHostToDevice, st));
    MOC_CUDA_TRY(cudaStreamSynchronize(st));
  }
  MOC_CUDA_TRY(cudaMemcpyAsync(r.d_ij_base, base.data(), sizeof(int64_t) * (size_t)pairs,
                               cudaMemcpyHostToDevice, st));
  MOC_CUDA_TRY(cudaMemcpyAsync(r.d_off + r.n3d, &M, sizeof(int64_t), cudaMemcpyHostToDevice, st));
  // pass 1 with staged stores: one warp a block, STAGE_W words of groups per ray
  const size_t stage_bytes = sizeof(float) * STAGE_W * (size_t)r.Z;
  if (stage_bytes <= (size_t)200 * 1024) {
    if (stage_bytes > 48 * 1024)
      MOC_CUDA_TRY(cudaFuncSetAttribute(ref_expand<1, true>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)stage_bytes));
    ref_expand<1, true><<<(unsigned)pairs, 32, stage_bytes, st>>>(make_args(r, r.d_z));
  } else {
    ref_expand<1><<<grid, 128, 0, st>>>(make_args(r, r.d_z));
  }
  MOC_CUDA_TRY(cudaGetLastError());
  const bool had_pending = r.p->psi_pending;
  RTRY(moc_launch_sweep_csr(r.p, r.d_off, r.d_sds, r.d_sz, r.d_ssrc));
  if (had_pending) {          // the sweep applied the pending renormalisation
    r.p->psi_pending = false;
    RTRY(moc_reset_psi_scale(r.p));
  }
  MOC_CUDA_TRY(cudaStreamSynchronize(st));
  r.p->launches += 2;
  r.sweeps++;
  r.last_segments = M;
  *segments = M;
  return moc_synchronize(r.p);
}

}  // namespace

extern "C" {

void transport_sweep(moc_ref_params *params, moc_ref_input *I) {
  MOC_NVTX_RANGE("transport_sweep");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!params || !I) {
    g_status = MOC_ERR_ARG;
    return;
  }
  if (I->axial_exp != 0 && I->axial_exp != 2) {
    // the reference prints and exits here (src/solver.c:506-511); the library
    // reports instead
    fprintf(stderr, "Error: invalid axial expansion order\n Please input 0 or 2\n");
    g_status = MOC_ERR_ARG;
    return;
  }
  int rc = ensure_state(params, I);
  int64_t segs = 0;
  if (rc == MOC_OK) rc = sweep_ref(&segs);
  g_status = rc;
  if (rc == MOC_OK) I->segments_processed = segs;            // src/solver.c:549
}

void renormalize_flux(moc_ref_params params, moc_ref_input I, moc_ref_commgrid grid) {
  MOC_NVTX_RANGE("renormalize_flux");
  (void)grid;
  std::lock_guard<std::mutex> lock(g_mu);
  int rc = ensure_state(&params, &I);
  if (rc == MOC_OK) rc = moc_renormalize_flux(g_ref.p);
  if (rc == MOC_OK) rc = moc_synchronize(g_ref.p);
  g_status = rc;
}

float update_sources(moc_ref_params params, moc_ref_input I, float keff) {
  MOC_NVTX_RANGE("update_sources");
  std::lock_guard<std::mutex> lock(g_mu);
  int rc = ensure_state(&params, &I);
  double res = NAN;
  if (rc == MOC_OK) rc = moc_update_sources(g_ref.p, keff, &res);
  g_status = rc;
  return rc == MOC_OK ? (float)res : NAN;
}

float compute_keff(moc_ref_params params, moc_ref_input I, moc_ref_commgrid grid) {
  MOC_NVTX_RANGE("compute_keff");
  (void)grid;
  std::lock_guard<std::mutex> lock(g_mu);
  int rc = ensure_state(&params, &I);
  double k = NAN;
  if (rc == MOC_OK) rc = moc_compute_keff(g_ref.p, params.leakage ? *params.leakage : 0.0, &k);
  g_status = rc;
  return rc == MOC_OK ? (float)k : NAN;
}

int moc_ref_set_rng(int mode, uint64_t seed) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (mode != MOC_REF_RNG_LIBC && mode != MOC_REF_RNG_HASH) return MOC_ERR_ARG;
  g_rng_mode = mode;
  g_rng_seed = seed;
  return MOC_OK;
}

int moc_ref_sync_to_host(moc_ref_params *prm, const moc_ref_input *I) {
  std::lock_guard<std::mutex> lock(g_mu);
  RefState &r = g_ref;
  if (!prm || !I) return MOC_ERR_ARG;
  if (!r.p || r.k_sources != prm->sources || r.k_tracks != prm->tracks) return MOC_ERR_STATE;
  const int64_t G = r.G, F = r.F;
  std::vector<float> phi((size_t)(r.ns * F * G)), q((size_t)(r.ns * F * G));
  std::vector<float> pf((size_t)(r.n3d * G)), pb((size_t)(r.n3d * G)), z((size_t)r.n3d);
  int rc = moc_download(r.p, phi.data(), q.data(), pf.data(), pb.data());
  if (rc != MOC_OK) return rc;
  if (cudaMemcpy(z.data(), r.d_z, sizeof(float) * z.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
    return MOC_ERR_CUDA;
  for (int64_t s = 0; s < r.ns; ++s)
    for (int64_t f = 0; f < F; ++f) {
      memcpy(prm->sources[s].fine_flux[f], &phi[(size_t)((s * F + f) * G)], sizeof(float) * (size_t)G);
      memcpy(prm->sources[s].fine_source[f], &q[(size_t)((s * F + f) * G)], sizeof(float) * (size_t)G);
    }
  for (int64_t i = 0; i < r.n2d; ++i)
    for (int64_t j = 0; j < r.P; ++j)
      for (int64_t k = 0; k < r.Z; ++k) {
        moc_ref_track &T = prm->tracks[i][j][k];
        const int64_t t = (i * r.P + j) * r.Z + k;
        memcpy(T.f_psi, &pf[(size_t)(t * G)], sizeof(float) * (size_t)G);
        memcpy(T.b_psi, &pb[(size_t)(t * G)], sizeof(float) * (size_t)G);
        T.z_height = z[(size_t)t];
      }
  return MOC_OK;
}

void moc_ref_finalize(void) {
  std::lock_guard<std::mutex> lock(g_mu);
  release_ref();
  g_status = MOC_OK;
}

int moc_ref_status(void) { return g_status; }

int64_t moc_ref_last_segments(void) { return g_ref.last_segments; }

double moc_ref_last_rng_ms(void) { return g_ref.last_rng_ms; }

int moc_ref_libc_draws(int32_t *out, int64_t n, int *bulk) {
  if (n < 0 || (n > 0 && !out)) return MOC_ERR_ARG;
  const int b = moc_libc_draws(out, n);
  if (bulk) *bulk = b;
  return MOC_OK;
}

}  // extern "C"
