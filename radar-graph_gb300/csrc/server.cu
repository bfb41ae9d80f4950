// Serving: a request loop over graphs kept resident on the device.
//
// Queries (BFS depth, BC dependencies, Radii) on any resident graph are
// submitted from any thread and complete asynchronously.  Worker threads --
// each with its own CUDA stream and scratch, so their work overlaps on the
// device -- take queries in arrival order:
//  * BFS queries waiting for the same graph are coalesced, up to 64, into one
//    bitmask multi-source traversal (rg_bfs_multi); a query that arrives while
//    others are on the GPU joins the next batch (continuous batching);
//  * a Radii query (64 seeded sample vertices) is one 64-source traversal
//    whose per-vertex maximum depth is exactly Radii.C's radius (a vertex's
//    mask last changes in the round of its farthest sample);
//  * a BC query (one source) runs BC-manyiter-v2's forward/backward phases.
// A batch is admitted only when its estimated device memory fits the free
// HBM budget taken at start-up; otherwise it waits for running batches to
// release theirs (or runs alone if nothing else is running).
// Every result equals the same query run alone through the single-query
// entry points.

#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "app_common.cuh"

namespace rg {
rg_status bfs_multi_run(rg_graph* g, const uint32_t* src_orig, int k, int32_t* h_depths, int64_t* rounds_out,
                        int32_t* d_depths_out);
rg_status bc_run(rg_graph* g, int variant, const uint32_t* src_orig, int nsrc, double* h_deps, int64_t* levels_out,
                 uint32_t hub_h);
}  // namespace rg

namespace {

using Clock = std::chrono::steady_clock;

double now_ms() {
  return std::chrono::duration<double, std::milli>(Clock::now().time_since_epoch()).count();
}

struct Query {
  uint64_t ticket;
  int graph;
  int kind;
  uint32_t source;
  double t_submit;
};

struct Result {
  std::vector<char> data;
  double latency_ms = 0;
  rg_status status = RG_OK;
  bool done = false;
};

}  // namespace

struct rg_server {
  std::vector<rg_graph*> graphs;
  int device = 0;
  int max_batch = 64;
  size_t hbm_budget = 0, hbm_in_use = 0;
  int running = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_mem;
  std::deque<Query> pending;
  std::unordered_map<uint64_t, Result> results;
  std::vector<std::thread> workers;
  bool stop = false;
  uint64_t next_ticket = 1;
  // statistics since the last reset
  std::vector<double> latencies;
  double t_first = 0, t_last = 0;
  int64_t completed = 0, launches = 0, batched = 0;
};

namespace {

using rg::fail;

// Radii sample vertices of a query: hashInt(seed*64 + i) % n, i < min(n, 64)
// (Radii.C:162-169 draws hashInt(i) % n; the seed selects a different set).
int radii_seeds(uint64_t seed, int64_t n, uint32_t* out) {
  const int k = (int)std::min<int64_t>(n, 64);
  for (int i = 0; i < k; i++) out[i] = (uint32_t)(rg::hash_u64(seed * 64 + (uint64_t)i) % (uint64_t)n);
  return k;
}

size_t estimate_bytes(const rg_graph* g, int kind, int k) {
  const size_t n = (size_t)g->n;
  if (kind == RG_QUERY_BC) return 64 * n;
  // masks, depths (k rows) and their original-order copy, two frontiers
  return (size_t)(8 * k + 40) * n;
}

void worker_main(rg_server* S) {
  cudaSetDevice(S->device);
  std::vector<int32_t> depths;
  std::vector<uint32_t> src;
  for (;;) {
    std::vector<Query> batch;
    size_t need = 0;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_work.wait(lk, [&] { return S->stop || !S->pending.empty(); });
      if (S->stop && S->pending.empty()) return;
      const Query q0 = S->pending.front();
      S->pending.pop_front();
      batch.push_back(q0);
      if (q0.kind == RG_QUERY_BFS) {  // coalesce waiting BFS queries on the same graph
        for (auto it = S->pending.begin(); it != S->pending.end() && (int)batch.size() < S->max_batch;) {
          if (it->kind == RG_QUERY_BFS && it->graph == q0.graph) {
            batch.push_back(*it);
            it = S->pending.erase(it);
          } else {
            ++it;
          }
        }
      }
      rg_graph* g = S->graphs[q0.graph];
      need = estimate_bytes(g, q0.kind, q0.kind == RG_QUERY_BFS ? (int)batch.size() : 64);
      // admission by free HBM: wait while the budget is taken by running work
      S->cv_mem.wait(lk, [&] { return S->running == 0 || S->hbm_in_use + need <= S->hbm_budget; });
      S->hbm_in_use += need;
      S->running++;
    }
    rg_graph* g = S->graphs[batch[0].graph];
    const int64_t n = g->n;
    const int kind = batch[0].kind;
    std::vector<std::vector<char>> out(batch.size());
    rg_status st = RG_OK;
    if (kind == RG_QUERY_BFS) {
      const int k = (int)batch.size();
      src.resize(k);
      for (int i = 0; i < k; i++) src[i] = batch[i].source;
      depths.resize((size_t)k * n);
      st = rg::bfs_multi_run(g, src.data(), k, depths.data(), nullptr, nullptr);
      for (int i = 0; i < k && st == RG_OK; i++) {
        out[i].resize(4 * n);
        memcpy(out[i].data(), depths.data() + (size_t)i * n, 4 * n);
      }
    } else if (kind == RG_QUERY_RADII) {
      src.resize(64);
      const int k = radii_seeds(batch[0].source, n, src.data());
      depths.resize((size_t)k * n);
      st = rg::bfs_multi_run(g, src.data(), k, depths.data(), nullptr, nullptr);
      if (st == RG_OK) {
        out[0].resize(4 * n);
        int32_t* r = reinterpret_cast<int32_t*>(out[0].data());
        for (int64_t v = 0; v < n; v++) {
          int32_t m = -1;
          for (int q = 0; q < k; q++) m = std::max(m, depths[(size_t)q * n + v]);
          r[v] = m;
        }
      }
    } else {
      out[0].resize(8 * n);
      const uint32_t s = batch[0].source;
      st = rg::bc_run(g, g->sorted ? RG_DEGSORT : RG_PUSH, &s, 1, reinterpret_cast<double*>(out[0].data()), nullptr,
                      0);
    }
    const double t_done = now_ms();
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->hbm_in_use -= need;
      S->running--;
      S->launches++;
      if (batch.size() > 1) S->batched += (int64_t)batch.size();
      for (size_t i = 0; i < batch.size(); i++) {
        Result& r = S->results[batch[i].ticket];
        r.status = st;
        r.data = std::move(out[i]);
        r.latency_ms = t_done - batch[i].t_submit;
        r.done = true;
        S->latencies.push_back(r.latency_ms);
        S->completed++;
        if (S->t_first == 0 || batch[i].t_submit < S->t_first) S->t_first = batch[i].t_submit;
      }
      S->t_last = std::max(S->t_last, t_done);
    }
    S->cv_done.notify_all();
    S->cv_mem.notify_all();
  }
}

}  // namespace

using namespace rg;

extern "C" {

rg_status rg_server_create(rg_graph* const* graphs, int ngraphs, int nworkers, int max_batch, double hbm_fraction,
                           rg_server** out) {
  if (!graphs || ngraphs < 1 || nworkers < 1 || nworkers > 64 || max_batch < 1 || max_batch > 64 ||
      hbm_fraction <= 0 || hbm_fraction > 1 || !out) {
    return fail(RG_EINVAL, "rg_server_create: bad arguments");
  }
  for (int i = 0; i < ngraphs; i++) {
    if (!graphs[i]) return fail(RG_EINVAL, "rg_server_create: null graph %d", i);
  }
  rg_server* S = new (std::nothrow) rg_server();
  if (!S) return fail(RG_ENOMEM, "host allocation failed");
  S->graphs.assign(graphs, graphs + ngraphs);
  S->max_batch = max_batch;
  RG_CUDA(cudaGetDevice(&S->device));
  size_t free_b = 0, total_b = 0;
  RG_CUDA(cudaMemGetInfo(&free_b, &total_b));
  S->hbm_budget = (size_t)(hbm_fraction * (double)free_b);
  for (int i = 0; i < nworkers; i++) S->workers.emplace_back(worker_main, S);
  *out = S;
  return RG_OK;
}

rg_status rg_server_submit(rg_server* S, int graph, rg_query_kind kind, uint32_t source, uint64_t* ticket) {
  if (!S || !ticket || graph < 0 || graph >= (int)S->graphs.size() || kind < RG_QUERY_BFS || kind > RG_QUERY_RADII) {
    return fail(RG_EINVAL, "rg_server_submit: bad arguments");
  }
  if (kind != RG_QUERY_RADII && source >= (uint64_t)S->graphs[graph]->n) {
    return fail(RG_EINVAL, "rg_server_submit: source %u >= n", source);
  }
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) return fail(RG_EINVAL, "server is stopping");
    const uint64_t t = S->next_ticket++;
    S->pending.push_back(Query{t, graph, (int)kind, source, now_ms()});
    S->results[t];
    *ticket = t;
  }
  S->cv_work.notify_one();
  return RG_OK;
}

rg_status rg_server_wait(rg_server* S, uint64_t ticket, void* h_result, size_t bytes, double* latency_ms) {
  if (!S) return fail(RG_EINVAL, "null server");
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->results.find(ticket);
  if (it == S->results.end()) return fail(RG_EINVAL, "unknown ticket %llu", (unsigned long long)ticket);
  S->cv_done.wait(lk, [&] { return S->results[ticket].done; });
  Result r = std::move(S->results[ticket]);
  S->results.erase(ticket);
  lk.unlock();
  if (r.status != RG_OK) return r.status;
  if (h_result) {
    if (bytes < r.data.size()) return fail(RG_EINVAL, "result buffer too small: need %zu bytes", r.data.size());
    memcpy(h_result, r.data.data(), r.data.size());
  }
  if (latency_ms) *latency_ms = r.latency_ms;
  return RG_OK;
}

rg_status rg_server_get_stats(rg_server* S, rg_server_stats* out) {
  if (!S || !out) return fail(RG_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  memset(out, 0, sizeof *out);
  out->completed = S->completed;
  out->launches = S->launches;
  out->batched = S->batched;
  if (!S->latencies.empty()) {
    std::vector<double> l(S->latencies);
    std::sort(l.begin(), l.end());
    auto pct = [&](double p) { return l[std::min(l.size() - 1, (size_t)(p * (double)(l.size() - 1) + 0.5))]; };
    out->p50_ms = pct(0.50);
    out->p99_ms = pct(0.99);
    const double span = S->t_last - S->t_first;
    out->qps = span > 0 ? 1000.0 * (double)S->completed / span : 0;
  }
  return RG_OK;
}

rg_status rg_server_reset_stats(rg_server* S) {
  if (!S) return fail(RG_EINVAL, "null server");
  std::lock_guard<std::mutex> lk(S->mu);
  S->latencies.clear();
  S->completed = S->launches = S->batched = 0;
  S->t_first = S->t_last = 0;
  return RG_OK;
}

rg_status rg_server_free(rg_server* S) {
  if (!S) return RG_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv_work.notify_all();
  for (auto& t : S->workers) t.join();
  delete S;
  return RG_OK;
}

}  // extern "C"
