// Serving: a request loop over graphs kept resident on the device.
//
// Queries (BFS depth, BC dependencies, Radii) on any resident graph are
// submitted from any thread and complete asynchronously.  Worker threads --
// each with its own CUDA stream and scratch, so their work overlaps on the
// device -- take queries in arrival order:
//  * BFS queries waiting for the same graph are coalesced, up to 64, into one
//    bitmask multi-source traversal (rg_bfs_multi); a query that arrives while
//    others are on the GPU joins the next batch (continuous batching).  A batch
//    smaller than the graph's break-even size -- measured when the server
//    starts: the 64-source traversal's time over one single-source BFS's --
//    runs as single-source traversals instead, so light load costs no more
//    than one query per launch;
//  * a Radii query (64 seeded sample vertices) is one 64-bit mask traversal
//    (Radii.C), the same run as rg_radii_seeds; up to 8 waiting on the same
//    graph run as one traversal with one mask word per query
//    (rg_radii_multi);
//  * BC queries waiting for the same graph are coalesced the same way into one
//    multi-source BC (rg_bc_multi: levels from one bitmask BFS, path counts
//    and dependencies for every source per level); below the graph's BC
//    break-even size (measured at start-up from two batch sizes against one
//    single-source BC) each runs BC-manyiter-v2's single-source pass.
// Results stay in device memory (stream-ordered allocations) until the client
// fetches them with rg_server_wait, which copies one query's array straight
// into the client's buffer.  A batch is admitted only when its working set
// and results fit the HBM budget taken at start-up beside what running
// batches and unfetched results hold; otherwise it waits for running batches
// to finish, and runs once none is running (unfetched results alone never
// hold a batch back, whatever order the clients fetch in).  Every result equals the same query run alone
// through the single-query entry points.

#include <cuda_runtime.h>
#include <string.h>

#include <math.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "app_common.cuh"

namespace {

using Clock = std::chrono::steady_clock;

// Radii queries per shared traversal: one 8-byte mask word per query and
// vertex, up to rg_radii_multi's 16.  The dense rounds gather whole W-word
// rows, so the cost per query falls as the batch grows even where the masks
// stream from DRAM (RMAT s24: 3.32 ms per query in batches of 4, 2.92 in 8,
// 2.80 in 16; s22: 1.17, 0.91, 0.81); HBM admission bounds the memory.
constexpr int kRadiiBatch = 16;
int radii_batch(const rg_graph*) { return kRadiiBatch; }

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

// A device allocation holding the results of one batch; freed (and its bytes
// returned to the admission budget) when its last result has been fetched.
struct Block {
  void* p = nullptr;
  size_t bytes = 0;
  int refs = 0;
};

struct Result {
  std::shared_ptr<Block> block;
  size_t offset = 0, bytes = 0;
  double latency_ms = 0;
  rg_status status = RG_OK;
  bool done = false;
  bool cancelled = false;  // rg_server_cancel while it ran: its result is dropped at completion
};

}  // namespace

struct rg_server {
  std::vector<rg_graph*> graphs;
  std::vector<int> bfs_breakeven;  // per graph: smallest batch worth a multi-source traversal
  std::vector<int> bc_breakeven;   // the same for BC
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
  bool paused = false;  // rg_server_pause: workers take no new queries
  uint64_t next_ticket = 1;
  // statistics since the last reset
  std::vector<double> latencies;
  double t_first = 0, t_last = 0;
  int64_t completed = 0, launches = 0, batched = 0;
  int64_t admission_waits = 0, cancelled = 0;
  int peak_running = 0;
};

namespace {

using rg::cuda_fail;
using rg::fail;

// Radii sample vertices of a query: hashInt(seed*64 + i) % n, i < min(n, 64)
// (Radii.C:162-169 draws hashInt(i) % n; the seed selects a different set).
int radii_seeds(uint64_t seed, int64_t n, uint32_t* out) {
  const int k = (int)std::min<int64_t>(n, 64);
  for (int i = 0; i < k; i++) out[i] = (uint32_t)(rg::hash_u64(seed * 64 + (uint64_t)i) % (uint64_t)n);
  return k;
}

size_t result_bytes(const rg_graph* g, int kind, int k) {
  const size_t n = (size_t)g->n;
  return kind == RG_QUERY_BC ? 8 * n * k : 4 * n * k;
}

// Break-even batch size for one graph: time one single-source BFS and one
// 64-source traversal (each after a warm-up run) on the calling thread.
rg_status calibrate_bfs(rg_graph* g, int* breakeven) {
  using namespace rg;
  const int64_t n = g->n;
  const int k = (int)std::min<int64_t>(n, 64);
  std::vector<uint32_t> src(k);
  for (int i = 0; i < k; i++) src[i] = (uint32_t)(hash_u64((uint64_t)i + 7) % (uint64_t)n);
  DevBuf out;
  RG_TRY(out.reserve(4 * (size_t)n * (size_t)k));
  const int variant = g->sorted ? RG_DEGSORT : RG_PUSH;
  double t1 = 0, tk = 0;
  for (int rep = 0; rep < 2; rep++) {
    auto a = Clock::now();
    RG_TRY(bfs_run(g, variant, src[0], nullptr, nullptr, nullptr, nullptr, 0, out.as<int32_t>()));
    auto b = Clock::now();
    RG_TRY(bfs_multi_run(g, src.data(), k, nullptr, nullptr, out.as<int32_t>()));
    auto c = Clock::now();
    t1 = std::chrono::duration<double>(b - a).count();
    tk = std::chrono::duration<double>(c - b).count();
  }
  *breakeven = (int)std::min<double>(65.0, std::max(2.0, std::ceil(tk / std::max(t1, 1e-9))));
  return RG_OK;
}

// BC break-even: one single-source pass against multi-source passes of 2 and
// 16 sources (cost ~ a + b k); the smallest k with a + b k < k * single.
rg_status calibrate_bc(rg_graph* g, int* breakeven) {
  using namespace rg;
  const int64_t n = g->n;
  std::vector<uint32_t> src(16);
  RG_TRY(bc_pick(g, 16, src.data()));
  DevBuf out;
  RG_TRY(out.reserve(8 * (size_t)n * 16));
  const int variant = g->sorted ? RG_DEGSORT : RG_PUSH;
  double t1 = 0, t2 = 0, t16 = 0;
  for (int rep = 0; rep < 2; rep++) {
    auto a = Clock::now();
    RG_TRY(bc_run(g, variant, src.data(), 1, nullptr, nullptr, 0, out.as<double>()));
    RG_CUDA(cudaStreamSynchronize(ctx().stream));
    auto b = Clock::now();
    RG_TRY(bc_multi_run(g, src.data(), 2, nullptr, out.as<double>(), nullptr));
    auto c = Clock::now();
    RG_TRY(bc_multi_run(g, src.data(), 16, nullptr, out.as<double>(), nullptr));
    auto d = Clock::now();
    t1 = std::chrono::duration<double>(b - a).count();
    t2 = std::chrono::duration<double>(c - b).count();
    t16 = std::chrono::duration<double>(d - c).count();
  }
  const double per = std::max(0.0, (t16 - t2) / 14.0), fixed = std::max(0.0, t2 - 2 * per);
  *breakeven = t1 > per ? (int)std::min(65.0, std::max(2.0, std::floor(fixed / (t1 - per)) + 1)) : 65;
  return RG_OK;
}

size_t working_bytes(const rg_graph* g, int kind, int k) {
  const size_t n = (size_t)g->n;
  // multi-source BC: two rows of ceil4(k) columns, the level store, masks and frontiers
  if (kind == RG_QUERY_BC) return k > 1 ? (size_t)(16 * ((k + 3) & ~3) + 112) * n : 72 * n;
  if (kind == RG_QUERY_RADII) {  // two mask rows of W words, radii rows and their copy, two frontiers
    int W = 1;
    while (W < k) W *= 2;
    return (size_t)(16 * W + 8 * k + 40) * n;
  }
  return (size_t)(8 * k + 40) * n;  // masks, depth rows and their original-order copy, two frontiers
}

void worker_main(rg_server* S) {
  cudaSetDevice(S->device);
  rg::Ctx* cx = nullptr;
  rg::get_ctx(&cx);
  std::vector<uint32_t> src;
  for (;;) {
    std::vector<Query> batch;
    size_t work = 0, res = 0;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_work.wait(lk, [&] { return S->stop || (!S->paused && !S->pending.empty()); });
      if (S->stop && (S->paused || S->pending.empty())) return;
      const Query q0 = S->pending.front();
      S->pending.pop_front();
      batch.push_back(q0);
      {  // coalesce waiting queries of the same kind on the same graph
        const int cap = q0.kind == RG_QUERY_RADII ? std::min(S->max_batch, radii_batch(S->graphs[q0.graph]))
                                                  : S->max_batch;
        for (auto it = S->pending.begin(); it != S->pending.end() && (int)batch.size() < cap;) {
          if (it->kind == q0.kind && it->graph == q0.graph) {
            batch.push_back(*it);
            it = S->pending.erase(it);
          } else {
            ++it;
          }
        }
      }
      const rg_graph* g = S->graphs[q0.graph];
      const int k = (int)batch.size();
      work = working_bytes(g, q0.kind, k);
      res = result_bytes(g, q0.kind, k);
      // admission by free HBM: wait while running batches and unfetched
      // results hold the budget -- but never for unfetched results alone: a
      // client may fetch in any order, and one waiting for this batch while
      // holding the results of an earlier one would otherwise wait forever.
      // With nothing running the batch is admitted (then only the client's
      // unfetched results exceed the budget).
      auto fits = [&] { return S->running == 0 || S->hbm_in_use + work + res <= S->hbm_budget; };
      if (!fits()) {
        S->admission_waits++;
        S->cv_mem.wait(lk, [&] { return S->stop || fits(); });
      }
      S->hbm_in_use += work + res;
      S->running++;
      S->peak_running = std::max(S->peak_running, S->running);
    }
    rg_graph* g = S->graphs[batch[0].graph];
    const int64_t n = g->n;
    const int kind = batch[0].kind;
    cudaStream_t st = cx ? cx->stream : nullptr;
    auto block = std::make_shared<Block>();
    block->bytes = res;
    rg_status status = cx ? RG_OK : RG_ENODEV;
    // BFS and BC batches below the graph's break-even size run query by query
    const bool multi = (kind == RG_QUERY_BFS && (int)batch.size() >= S->bfs_breakeven[batch[0].graph]) ||
                       (kind == RG_QUERY_BC && (int)batch.size() >= S->bc_breakeven[batch[0].graph]) ||
                       (kind == RG_QUERY_RADII && batch.size() >= 2);
    if (status == RG_OK && cudaMallocAsync(&block->p, res, st) != cudaSuccess) {
      cudaGetLastError();
      status = fail(RG_ENOMEM, "server: result allocation of %zu bytes failed", res);
    }
    if (status == RG_OK) {
      if (kind == RG_QUERY_BFS) {
        const int k = (int)batch.size();
        if (!multi) {
          for (int i = 0; i < k && status == RG_OK; i++) {
            status = rg::bfs_run(g, g->sorted ? RG_DEGSORT : RG_PUSH, batch[i].source, nullptr, nullptr, nullptr,
                                 nullptr, 0, static_cast<int32_t*>(block->p) + (size_t)i * (size_t)n);
          }
        } else {
          src.resize(k);
          for (int i = 0; i < k; i++) src[i] = batch[i].source;
          status = rg::bfs_multi_run(g, src.data(), k, nullptr, nullptr, static_cast<int32_t*>(block->p));
        }
      } else if (kind == RG_QUERY_RADII) {
        const int nq = (int)batch.size();
        const int k = (int)std::min<int64_t>(n, 64);  // samples per query
        src.resize((size_t)k * nq);
        for (int i = 0; i < nq; i++) radii_seeds(batch[i].source, n, src.data() + (size_t)i * k);
        if (multi) {
          status = rg::radii_multi_run(g, src.data(), k, nq, nullptr, static_cast<int32_t*>(block->p), nullptr);
        } else {
          status = rg::radii_run(g, g->sorted ? RG_DEGSORT : RG_PUSH, src.data(), k, nullptr, nullptr, 0,
                                 static_cast<int32_t*>(block->p));
        }
      } else {
        const int k = (int)batch.size();
        src.resize(k);
        for (int i = 0; i < k; i++) src[i] = batch[i].source;
        if (multi) {
          status = rg::bc_multi_run(g, src.data(), k, nullptr, static_cast<double*>(block->p), nullptr);
        } else {
          for (int i = 0; i < k && status == RG_OK; i++) {
            status = rg::bc_run(g, g->sorted ? RG_DEGSORT : RG_PUSH, &src[i], 1, nullptr, nullptr, 0,
                                static_cast<double*>(block->p) + (size_t)i * (size_t)n);
          }
        }
      }
      // the result is complete before any client (on another stream) copies it
      if (status == RG_OK) {
        const cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) status = cuda_fail(e, "server batch", __FILE__, __LINE__);
      }
    }
    const double t_done = now_ms();
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->hbm_in_use -= work;
      if (status != RG_OK) S->hbm_in_use -= res;
      S->running--;
      if (!multi) {
        S->launches += (int64_t)batch.size();
      } else {
        S->launches++;
      }
      if (multi) S->batched += (int64_t)batch.size();
      const size_t row = kind == RG_QUERY_BC ? 8 * n : 4 * n;
      block->refs = 0;
      for (size_t i = 0; i < batch.size(); i++) {
        Result& r = S->results[batch[i].ticket];
        r.status = r.cancelled ? RG_ECANCELED : status;
        if (status == RG_OK && !r.cancelled) {
          r.block = block;
          r.offset = i * row;
          r.bytes = row;
          block->refs++;
        }
        r.latency_ms = t_done - batch[i].t_submit;
        r.done = true;
        S->latencies.push_back(r.latency_ms);
        S->completed++;
        if (S->t_first == 0 || batch[i].t_submit < S->t_first) S->t_first = batch[i].t_submit;
      }
      S->t_last = std::max(S->t_last, t_done);
      if (block->refs == 0) S->hbm_in_use -= status == RG_OK ? res : 0;  // every query of the batch was cancelled
    }
    if (block->refs == 0 && block->p) cudaFreeAsync(block->p, st);
    S->cv_done.notify_all();
    S->cv_mem.notify_all();
  }
}

// One fetched (or dropped) result of a batch: the batch's block is freed and
// its bytes returned to the admission budget when its last result goes.
void release_result(rg_server* S, const std::shared_ptr<Block>& block, cudaStream_t st) {
  bool last = false;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    last = --block->refs == 0;
    if (last) S->hbm_in_use -= block->bytes;
  }
  if (last) {
    cudaFreeAsync(block->p, st);
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
  S->bfs_breakeven.assign(ngraphs, 1);
  S->bc_breakeven.assign(ngraphs, 2);
  for (int i = 0; i < ngraphs; i++) {
    rg_status cs = calibrate_bfs(S->graphs[i], &S->bfs_breakeven[i]);
    if (cs == RG_OK && S->graphs[i]->m > 0) cs = calibrate_bc(S->graphs[i], &S->bc_breakeven[i]);
    if (cs != RG_OK) {
      delete S;
      return cs;
    }
  }
  // freed result blocks stay in the stream-ordered pool (the library keeps
  // the device pool's freed memory mapped for reuse)
  cudaGetLastError();
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

rg_status rg_server_wait_for(rg_server* S, uint64_t ticket, void* h_result, size_t bytes, double* latency_ms,
                             double timeout_ms) {
  if (!S) return fail(RG_EINVAL, "null server");
  Ctx* cx = nullptr;
  RG_TRY(get_ctx(&cx));
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->results.find(ticket);
  if (it == S->results.end()) return fail(RG_EINVAL, "unknown ticket %llu", (unsigned long long)ticket);
  auto ready = [&] { return S->results[ticket].done; };
  if (timeout_ms < 0) {
    S->cv_done.wait(lk, ready);
  } else if (!S->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), ready)) {
    // the ticket stays valid: wait again later, or cancel it
    return fail(RG_ETIMEOUT, "ticket %llu not done after %.3f ms", (unsigned long long)ticket, timeout_ms);
  }
  Result r = std::move(S->results[ticket]);
  S->results.erase(ticket);
  lk.unlock();
  rg_status st = r.status;
  if (st == RG_ECANCELED) return fail(RG_ECANCELED, "ticket %llu was cancelled", (unsigned long long)ticket);
  if (st == RG_OK && h_result && bytes < r.bytes) {
    st = fail(RG_EINVAL, "result buffer too small: need %zu bytes", r.bytes);
  }
  if (st == RG_OK && h_result) {
    const cudaError_t e =
        cudaMemcpyAsync(h_result, static_cast<char*>(r.block->p) + r.offset, r.bytes, cudaMemcpyDeviceToHost,
                        cx->stream);
    if (e != cudaSuccess || cudaStreamSynchronize(cx->stream) != cudaSuccess) {
      st = cuda_fail(e != cudaSuccess ? e : cudaErrorUnknown, "server result copy", __FILE__, __LINE__);
    }
  }
  if (r.block) release_result(S, r.block, cx->stream);
  if (st == RG_OK && latency_ms) *latency_ms = r.latency_ms;
  return st;
}

rg_status rg_server_wait(rg_server* S, uint64_t ticket, void* h_result, size_t bytes, double* latency_ms) {
  return rg_server_wait_for(S, ticket, h_result, bytes, latency_ms, -1.0);
}

rg_status rg_server_cancel(rg_server* S, uint64_t ticket) {
  if (!S) return fail(RG_EINVAL, "null server");
  std::shared_ptr<Block> drop;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->results.find(ticket);
    if (it == S->results.end()) return fail(RG_EINVAL, "unknown ticket %llu", (unsigned long long)ticket);
    Result& r = it->second;
    if (r.cancelled || r.status == RG_ECANCELED) return RG_OK;
    auto q = std::find_if(S->pending.begin(), S->pending.end(), [&](const Query& x) { return x.ticket == ticket; });
    if (q != S->pending.end()) {  // not started: it never runs
      S->pending.erase(q);
      r.status = RG_ECANCELED;
      r.done = true;
    } else if (!r.done) {  // running: the worker drops its result
      r.cancelled = true;
    } else {  // finished and not fetched: release the result now
      drop = std::move(r.block);
      r.block.reset();
      if (r.status == RG_OK) r.status = RG_ECANCELED;
    }
    S->cancelled++;
  }
  if (drop) {
    Ctx* cx = nullptr;
    RG_TRY(get_ctx(&cx));
    release_result(S, drop, cx->stream);
  }
  S->cv_done.notify_all();
  return RG_OK;
}

rg_status rg_server_pause(rg_server* S, int paused) {
  if (!S) return fail(RG_EINVAL, "null server");
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->paused = paused != 0;
  }
  S->cv_work.notify_all();
  return RG_OK;
}

rg_status rg_server_get_stats(rg_server* S, rg_server_stats* out) {
  if (!S || !out) return fail(RG_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  memset(out, 0, sizeof *out);
  out->completed = S->completed;
  out->launches = S->launches;
  out->batched = S->batched;
  out->admission_waits = S->admission_waits;
  out->cancelled = S->cancelled;
  out->peak_running = S->peak_running;
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
  S->completed = S->launches = S->batched = S->admission_waits = S->cancelled = 0;
  S->peak_running = S->running;
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
  S->cv_mem.notify_all();
  for (auto& t : S->workers) t.join();
  // results never fetched: release their blocks
  for (auto& kv : S->results) {
    if (kv.second.block && kv.second.block->p && --kv.second.block->refs == 0) cudaFree(kv.second.block->p);
  }
  delete S;
  return RG_OK;
}

rg_status rg_pinned_alloc(size_t bytes, void** h_ptr) {
  if (!h_ptr || bytes == 0) return fail(RG_EINVAL, "rg_pinned_alloc: bad arguments");
  RG_CUDA(cudaHostAlloc(h_ptr, bytes, cudaHostAllocDefault));
  return RG_OK;
}

rg_status rg_pinned_free(void* h_ptr) {
  if (h_ptr) RG_CUDA(cudaFreeHost(h_ptr));
  return RG_OK;
}

}  // extern "C"
