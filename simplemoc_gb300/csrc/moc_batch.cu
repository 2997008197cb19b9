// moc_batch.cu -- many independent problems ("cores") swept by one persistent
// launch, and their power iteration replayed as a CUDA graph.
//
// Each core keeps its own storage and post-sweep scalars (a moc_problem).  The
// batch owns the task list of the persistent sweep: (core, first track) pairs of
// 32/tpw tracks each, with the cores of the largest work per task first, and
// one threads-per-track width per core, measured by moc_batch_autotune for
// every distinct (segments per track, groups, polar angles, mode) key.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <numeric>
#include <tuple>
#include <vector>

#include "moc_internal.h"

struct moc_batch {
  std::vector<moc_problem *> cores;
  int device = 0;
  int mode = MOC_MODE_PLAIN;
  bool quad = true;
  cudaStream_t stream = nullptr;
  SweepArgs *d_args = nullptr;
  int2 *d_tasks = nullptr;
  int *d_tpw = nullptr;
  unsigned long long *d_counter = nullptr;
  int64_t n_tasks = 0;
  std::vector<int> tpw;
  const float2 *table = nullptr;
  int table_n = 0;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  std::vector<int64_t> graph_key;       // per core (uploads, flags) when captured
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int64_t launches = 0;
};

namespace {

struct WidthKey {
  int S, G, P, mode, axial;
  bool operator<(const WidthKey &o) const {
    return std::tie(S, G, P, mode, axial) < std::tie(o.S, o.G, o.P, o.mode, o.axial);
  }
};
std::mutex g_width_mu;
std::map<WidthKey, int> g_width_cache;

// Two 4-group chunks per thread (the batched kernel's shape): the narrowest
// power-of-two width that covers the groups.
constexpr int BATCH_CPL = 2;

int default_width(const moc_problem *p) {
  const int nchunk = p->ldg / 4;
  int w = 4;
  while (w * BATCH_CPL < nchunk) w <<= 1;
  return w;
}

// Copies every core's sweep arguments to the device.  The batched kernel and a
// captured graph read them there at run time, so they follow the cores' state
// (an upload recomputes the fine-interval divisor check from the start heights).
int upload_args(moc_batch *b) {
  const int n = (int)b->cores.size();
  std::vector<SweepArgs> args((size_t)n);
  for (int c = 0; c < n; ++c) {
    moc_problem *p = b->cores[(size_t)c];
    args[(size_t)c] = moc_sweep_args(p);
    // the factor is 1 whenever no renormalisation is pending (see moc_reset_psi_scale)
    args[(size_t)c].psi_scale = p->psi_scale;
  }
  MOC_CUDA_TRY(cudaMemcpy(b->d_args, args.data(), sizeof(SweepArgs) * (size_t)n, cudaMemcpyHostToDevice));
  return MOC_OK;
}

// The captured iteration bakes in each core's work lists (rebuilt by an
// upload) and update kernel (chosen by the mode flags).
std::vector<int64_t> graph_key(const moc_batch *b) {
  std::vector<int64_t> k;
  for (const moc_problem *p : b->cores) {
    k.push_back(p->uploads);
    k.push_back(p->flags);
  }
  return k;
}

void drop_graph(moc_batch *b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

// Builds the per-core sweep arguments and the cost-ordered task list.
int rebuild_tasks(moc_batch *b) {
  const int n = (int)b->cores.size();
  std::vector<int> order((size_t)n);
  std::iota(order.begin(), order.end(), 0);
  auto cost = [&](int c) {
    const moc_problem *p = b->cores[(size_t)c];
    return (double)(32 / b->tpw[(size_t)c]) * p->d.n_seg * p->ldg;
  };
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost(x) > cost(y); });
  std::vector<int2> tasks;
  for (int c : order) {
    const int gpw = 32 / b->tpw[(size_t)c];
    for (int64_t t = 0; t < b->cores[(size_t)c]->n3d; t += gpw) tasks.push_back(make_int2(c, (int)t));
  }
  if (b->d_tasks) cudaFree(b->d_tasks);
  b->d_tasks = nullptr;
  b->n_tasks = (int64_t)tasks.size();
  MOC_CUDA_TRY(cudaMalloc(&b->d_tasks, sizeof(int2) * (tasks.empty() ? 1 : tasks.size())));
  MOC_CUDA_TRY(cudaMemcpy(b->d_tasks, tasks.data(), sizeof(int2) * tasks.size(), cudaMemcpyHostToDevice));
  const int rc = upload_args(b);
  if (rc != MOC_OK) return rc;
  MOC_CUDA_TRY(cudaMemcpy(b->d_tpw, b->tpw.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice));
  drop_graph(b);
  return MOC_OK;
}

// One batched sweep on b->stream (no host synchronisation).
int batch_sweep(moc_batch *b) {
  int rc = moc_launch_sweep_batch(b->device, b->stream, b->mode, b->quad, b->d_args, b->d_tasks,
                                  b->n_tasks, b->d_tpw, b->d_counter, b->table, b->table_n);
  if (rc != MOC_OK) return rc;
  b->launches += 2;
  for (moc_problem *p : b->cores) {
    cudaStream_t own = p->stream;
    p->stream = b->stream;
    rc = moc_reset_psi_scale(p);
    p->stream = own;
    p->psi_pending = false;
    if (rc != MOC_OK) return rc;
  }
  return MOC_OK;
}

// renormalize + update_sources + keff of every core on b->stream, k_eff chained
// on the device.
int batch_post(moc_batch *b) {
  for (moc_problem *p : b->cores) {
    cudaStream_t own = p->stream;
    p->stream = b->stream;
    int rc = moc_launch_renormalize(p);
    if (rc == MOC_OK) rc = moc_launch_update(p, 0.0, true, true);
    p->stream = own;
    if (rc != MOC_OK) return rc;
  }
  return MOC_OK;
}

// Before the batch stream reads the cores' arrays: each core's copies have
// landed and its own stream has drained (work issued on a core since the batch
// last ran), and the sweep arguments follow the cores' current state.  A core
// that failed, whose last upload was rejected, or whose mode no longer matches
// the batch is refused.
int join_cores(moc_batch *b) {
  MOC_CUDA_TRY(cudaStreamSynchronize(b->stream));   // no batch kernel reads the arguments
  for (moc_problem *p : b->cores) {
    if (p->status != MOC_OK || p->stale) return MOC_ERR_STATE;
    if (p->mode != b->mode || (p->mode == MOC_MODE_MIXED && (p->flags & MOC_FLAG_COMPENSATED)))
      return MOC_ERR_STATE;
    int rc = moc_join_upload(p);
    if (rc != MOC_OK) return rc;
    MOC_CUDA_TRY(cudaStreamSynchronize(p->stream));
  }
  if (b->exec && graph_key(b) != b->graph_key) drop_graph(b);
  return upload_args(b);
}

// After the batch stream has drained: every core's device error word, as a
// call on that core would report it (a source id out of range from a streamed
// upload leaves that core stale).  The first error, MOC_OK if none.
int check_cores(moc_batch *b) {
  int first = MOC_OK;
  for (moc_problem *p : b->cores) {
    const int rc = moc_sync_check(p);
    if (first == MOC_OK) first = rc;
  }
  return first;
}

}  // namespace

extern "C" {

int moc_batch_create(int n, moc_problem *const *problems, moc_batch **out) {
  if (n < 1 || !problems || !out) return MOC_ERR_ARG;
  *out = nullptr;
  moc_batch *b = new moc_batch();
  b->cores.assign(problems, problems + n);
  const moc_problem *p0 = problems[0];
  if (!p0) {
    delete b;
    return MOC_ERR_ARG;
  }
  b->device = p0->device;
  b->mode = p0->mode;
  b->quad = p0->d.axial_exp == 2;
  for (moc_problem *p : b->cores) {
    // one launch: same device, mode, source order and (PLAIN) exponential table
    if (!p || p->status != MOC_OK || p->stale || p->device != b->device || p->mode != b->mode ||
        (p->d.axial_exp == 2) != b->quad || p->ldg > 256 || p->n3d > INT32_MAX ||
        p->mode == MOC_MODE_FP64 ||
        (p->mode == MOC_MODE_MIXED && (p->flags & MOC_FLAG_COMPENSATED)) ||
        p->d.table_n != p0->d.table_n || p->d.table_dx != p0->d.table_dx ||
        p->d.table_maxval != p0->d.table_maxval) {
      delete b;
      return MOC_ERR_ARG;
    }
  }
  cudaSetDevice(b->device);
  b->table = reinterpret_cast<const float2 *>(p0->table);
  b->table_n = p0->d.table_n;
  for (moc_problem *p : b->cores) b->tpw.push_back(default_width(p));
  int rc = MOC_OK;
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess ||
      cudaMalloc(&b->d_args, sizeof(SweepArgs) * (size_t)n) != cudaSuccess ||
      cudaMalloc(&b->d_tpw, sizeof(int) * (size_t)n) != cudaSuccess ||
      cudaMalloc(&b->d_counter, sizeof(unsigned long long)) != cudaSuccess)
    rc = MOC_ERR_CUDA;
  // make every core's previous work visible to the batch stream
  for (moc_problem *p : b->cores) {
    if (rc == MOC_OK) rc = moc_join_upload(p);
    if (rc == MOC_OK && cudaStreamSynchronize(p->stream) != cudaSuccess) rc = MOC_ERR_CUDA;
  }
  if (rc == MOC_OK) rc = rebuild_tasks(b);
  if (rc != MOC_OK) {
    moc_batch_destroy(b);
    return rc;
  }
  *out = b;
  return MOC_OK;
}

int moc_batch_destroy(moc_batch *b) {
  if (!b) return MOC_ERR_ARG;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->d_args) cudaFree(b->d_args);
  if (b->d_tasks) cudaFree(b->d_tasks);
  if (b->d_tpw) cudaFree(b->d_tpw);
  if (b->d_counter) cudaFree(b->d_counter);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return MOC_OK;
}

int moc_batch_set_width(moc_batch *b, int core, int threads_per_track) {
  if (!b || core < 0 || core >= (int)b->cores.size()) return MOC_ERR_ARG;
  const int w = threads_per_track;
  if (w != 4 && w != 8 && w != 16 && w != 32) return MOC_ERR_ARG;
  if (w * 4 * BATCH_CPL < b->cores[(size_t)core]->ldg) return MOC_ERR_ARG;
  b->tpw[(size_t)core] = w;
  cudaSetDevice(b->device);
  return rebuild_tasks(b);
}

int moc_batch_widths(const moc_batch *b, int *threads_per_track) {
  if (!b || !threads_per_track) return MOC_ERR_ARG;
  std::copy(b->tpw.begin(), b->tpw.end(), threads_per_track);
  return MOC_OK;
}

// Autotuner of the batch: for every distinct key, times the persistent kernel on
// up to 65536 tracks of one core of that key for each width that covers its
// groups, with scratch tallies and angular fluxes (the state is untouched).
int moc_batch_autotune(moc_batch *b) {
  if (!b) return MOC_ERR_ARG;
  cudaSetDevice(b->device);
  const int rc0 = join_cores(b);
  if (rc0 != MOC_OK) return rc0;
  const int n = (int)b->cores.size();
  std::map<WidthKey, int> chosen;
  for (int c = 0; c < n; ++c) {
    moc_problem *p = b->cores[(size_t)c];
    const WidthKey key{p->d.n_seg, p->d.n_groups, p->d.n_polar, p->mode, p->d.axial_exp};
    {
      std::lock_guard<std::mutex> lock(g_width_mu);
      auto it = g_width_cache.find(key);
      if (it != g_width_cache.end()) {
        b->tpw[(size_t)c] = it->second;
        continue;
      }
    }
    if (chosen.count(key)) {
      b->tpw[(size_t)c] = chosen[key];
      continue;
    }
    const int64_t nsub = p->n3d < 65536 ? p->n3d : 65536;
    float *phi_s = nullptr, *psi_s = nullptr;
    SweepArgs *d_a = nullptr;
    int2 *d_t = nullptr;
    int *d_w = nullptr;
    const size_t phi_bytes = sizeof(float) * (size_t)(p->nfsr * p->ldg);
    const size_t psi_bytes = sizeof(float) * (size_t)(nsub * p->ldg);
    int rc = MOC_OK;
    if (cudaMalloc(&phi_s, phi_bytes) != cudaSuccess || cudaMalloc(&psi_s, psi_bytes) != cudaSuccess ||
        cudaMalloc(&d_a, sizeof(SweepArgs)) != cudaSuccess ||
        cudaMalloc(&d_t, sizeof(int2) * (size_t)nsub) != cudaSuccess ||
        cudaMalloc(&d_w, sizeof(int)) != cudaSuccess)
      rc = MOC_ERR_OOM;
    SweepArgs a = moc_sweep_args(p);
    a.n3d = nsub;
    a.phi = phi_s;
    a.psi = psi_s;
    a.psi_scale = nullptr;
    if (rc == MOC_OK &&
        (cudaMemset(phi_s, 0, phi_bytes) != cudaSuccess ||
         cudaMemcpy(psi_s, p->psi_f, psi_bytes, cudaMemcpyDeviceToDevice) != cudaSuccess ||
         cudaMemcpy(d_a, &a, sizeof a, cudaMemcpyHostToDevice) != cudaSuccess))
      rc = MOC_ERR_CUDA;
    double best = 1e30;
    int bw = default_width(p);
    for (int w = 4; w <= 32 && rc == MOC_OK; w <<= 1) {
      if (w * 4 * BATCH_CPL < p->ldg) continue;
      const int gpw = 32 / w;
      std::vector<int2> t;
      for (int64_t k = 0; k < nsub; k += gpw) t.push_back(make_int2(0, (int)k));
      if (cudaMemcpy(d_t, t.data(), sizeof(int2) * t.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
          cudaMemcpy(d_w, &w, sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) {
        rc = MOC_ERR_CUDA;
        break;
      }
      double tot = 0.0;
      for (int r = 0; r < 3 && rc == MOC_OK; ++r) {
        cudaEventRecord(b->ev0, b->stream);
        rc = moc_launch_sweep_batch(b->device, b->stream, b->mode, b->quad, d_a, d_t,
                                    (int64_t)t.size(), d_w, b->d_counter, b->table, b->table_n);
        cudaEventRecord(b->ev1, b->stream);
        if (rc == MOC_OK && cudaEventSynchronize(b->ev1) != cudaSuccess) rc = MOC_ERR_CUDA;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, b->ev0, b->ev1);
        if (r > 0) tot += ms;                      // first run is the warm-up
      }
      if (rc == MOC_OK && tot < best) {
        best = tot;
        bw = w;
      }
    }
    cudaFree(phi_s);
    cudaFree(psi_s);
    cudaFree(d_a);
    cudaFree(d_t);
    cudaFree(d_w);
    if (rc != MOC_OK) return rc;
    chosen[key] = bw;
    b->tpw[(size_t)c] = bw;
    std::lock_guard<std::mutex> lock(g_width_mu);
    g_width_cache[key] = bw;
  }
  return rebuild_tasks(b);
}

int moc_batch_sweep(moc_batch *b) {
  MOC_NVTX_RANGE("moc_batch_sweep");
  if (!b) return MOC_ERR_ARG;
  cudaSetDevice(b->device);
  int rc = join_cores(b);
  if (rc == MOC_OK) rc = batch_sweep(b);
  if (rc != MOC_OK) return rc;
  MOC_CUDA_TRY(cudaStreamSynchronize(b->stream));
  return check_cores(b);
}

// `iters` power iterations of every core: the batched sweep, then each core's
// renormalize / update_sources / compute_keff, k_eff chained on the device.
// With use_graph the iteration is captured once as a CUDA graph and replayed.
// The call makes exactly `iters` iterations: before its first capture it runs
// one of them eagerly (kernel attributes get set and every core reaches the
// pending renormalisation that the graph replays) and replays the rest.
int moc_batch_power_iterations(moc_batch *b, int iters, int use_graph, double *ms_total) {
  MOC_NVTX_RANGE("moc_batch_power_iterations");
  if (!b || iters < 1) return MOC_ERR_ARG;
  cudaSetDevice(b->device);
  int rc = join_cores(b);
  if (rc != MOC_OK) return rc;
  int done = 0;
  cudaEventRecord(b->ev0, b->stream);
  if (use_graph && !b->exec) {
    rc = batch_sweep(b);
    if (rc == MOC_OK) rc = batch_post(b);
    if (rc != MOC_OK) return rc;
    done = 1;
    // capture records without executing; the eager iteration above runs on
    if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
      return MOC_ERR_CUDA;
    rc = batch_sweep(b);
    if (rc == MOC_OK) rc = batch_post(b);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (rc != MOC_OK || e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return rc != MOC_OK ? rc : MOC_ERR_CUDA;
    }
    b->graph = g;
    if (cudaGraphInstantiate(&b->exec, g, 0) != cudaSuccess) {
      drop_graph(b);
      return MOC_ERR_CUDA;
    }
    b->graph_key = graph_key(b);
  }
  for (int i = done; i < iters && rc == MOC_OK; ++i) {
    if (use_graph) {
      if (cudaGraphLaunch(b->exec, b->stream) != cudaSuccess) rc = MOC_ERR_CUDA;
      b->launches++;
    } else {
      rc = batch_sweep(b);
      if (rc == MOC_OK) rc = batch_post(b);
    }
  }
  cudaEventRecord(b->ev1, b->stream);
  if (rc != MOC_OK) return rc;
  MOC_CUDA_TRY(cudaEventSynchronize(b->ev1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, b->ev0, b->ev1);
  if (ms_total) *ms_total = ms;
  for (moc_problem *p : b->cores) p->psi_pending = true;   // the last step renormalised
  return check_cores(b);
}

int moc_batch_results(moc_batch *b, double *keff, double *residual) {
  if (!b) return MOC_ERR_ARG;
  cudaSetDevice(b->device);
  MOC_CUDA_TRY(cudaStreamSynchronize(b->stream));
  const int rc = check_cores(b);
  if (rc != MOC_OK) return rc;
  for (size_t c = 0; c < b->cores.size(); ++c) {
    double sc[SC_COUNT];
    MOC_CUDA_TRY(cudaMemcpy(sc, b->cores[c]->scalars, sizeof sc, cudaMemcpyDeviceToHost));
    if (keff) keff[c] = sc[SC_KEFF];
    if (residual) residual[c] = sc[SC_RESIDUAL];
  }
  return MOC_OK;
}

int64_t moc_batch_launch_count(const moc_batch *b) { return b ? b->launches : 0; }

}  // extern "C"
