// Autotuner: for one graph and variant, times candidate schedules of each
// app (push/pull direction, the dense threshold m/x of ligra.h:283, hub
// copies on/off and their shared-memory budget, PageRank's sweep shape) and
// keeps the fastest per app
// in the graph.  Later app calls on that graph use the choice.  No schedule
// changes any result, so tuning is safe to run on live graphs.

#include <cuda_runtime.h>

#include <vector>

#include "app_common.cuh"

using namespace rg;

namespace {

std::vector<Options> candidates(int app, bool hubs, const Options& base) {
  std::vector<Options> out;
  auto add = [&](int64_t dir, int64_t div, int64_t kb, int64_t fwd_hubs = 1) {
    Options o = base;
    o.direction = dir;
    o.dense_div = div;
    o.hub_smem_kb = kb;
    o.bc_fwd_hubs = fwd_hubs;
    out.push_back(o);
  };
  // hub budgets: 4 KiB (the 512 hottest ids) keeps the push at full
  // occupancy and already absorbs the hot-spot reductions into the top hubs
  // (BC at RMAT s24: 9.2 -> 7.8 ms); 16 and 48 KiB cover more hubs at fewer
  // resident CTAs
  const std::vector<int64_t> kbs = hubs ? std::vector<int64_t>{0, 4, 16, 48} : std::vector<int64_t>{0};
  switch (app) {
    case kAppPagerank:  // push (with or without hub copies) against pull (with or without cached
                        // hubs, 8 or 16 edges per lane: fewer warp scans per edge against more registers)
      for (int64_t kb : kbs) add(0, 20, kb);
      for (int64_t shape : {81, 161}) {
        add(1, 20, 0);
        out.back().sweep_shape = shape;
        if (hubs) {
          add(1, 20, 48);
          out.back().sweep_shape = shape;
        }
      }
      break;
    case kAppBfs:
      for (int64_t div : {10, 20, 40, 80}) add(1, div, 0);
      for (int64_t kb : kbs) add(0, 20, kb);
      break;
    case kAppRadii:  // push (hub budget x dense threshold) against pulled dense rounds
      for (int64_t kb : kbs)
        for (int64_t div : {20, 80}) add(0, div, kb);
      for (int64_t div : {2, 5, 20}) add(1, div, 0);
      break;
    default:  // BC pushes (its pull scans every unvisited vertex: measured slower),
              // with hub copies in both phases or in the backward phase only
      for (int64_t kb : kbs)
        for (int64_t div : {20, 80}) {
          add(0, div, kb);
          if (kb > 0) add(0, div, kb, 0);
        }
      break;
  }
  return out;
}

}  // namespace

extern "C" rg_status rg_autotune(rg_graph* g, rg_variant variant, double* best_ms) {
  if (!g || variant < 0 || variant > 4) return fail(RG_EINVAL, "rg_autotune: bad arguments");
  if (g->m == 0) return fail(RG_EINVAL, "rg_autotune: graph has no edges");
  uint32_t root = 0;
  RG_TRY(bc_pick(g, 1, &root));
  const int k = (int)std::min<int64_t>(g->n, 64);
  std::vector<uint32_t> seeds(k);
  for (int i = 0; i < k; i++) seeds[i] = (uint32_t)(hash_u64((uint64_t)i) % (uint64_t)g->n);
  const bool hubs = variant == RG_RADAR || variant == RG_HUBDUP;
  const bool kt = g_kernel_timing;
  g_kernel_timing = false;
  for (int app = 0; app < 4; app++) {
    double best = 1e30;
    Options choice = g_opts;
    for (const Options& o : candidates(app, hubs, g_opts)) {
      g->tuned[app] = true;
      g->topt[app] = o;
      double t = 0;
      for (int rep = 0; rep < 2; rep++) {  // the first run warms caches and allocations
        rg_status s;
        switch (app) {
          case kAppPagerank: s = pagerank_run(g, variant, 5, nullptr, nullptr, nullptr, 0); break;
          case kAppBfs: s = bfs_run(g, variant, root, nullptr, nullptr, nullptr, nullptr, 0); break;
          case kAppBc: s = bc_run(g, variant, &root, 1, nullptr, nullptr, 0); break;
          default: s = radii_run(g, variant, seeds.data(), k, nullptr, nullptr, 0); break;
        }
        if (s != RG_OK) {
          g->tuned[app] = false;
          g_kernel_timing = kt;
          return s;
        }
        t = g_timing.total_ms;
      }
      if (t < best) {
        best = t;
        choice = o;
      }
    }
    g->topt[app] = choice;
    g->tuned[app] = true;
    if (best_ms) best_ms[app] = best;
  }
  g_kernel_timing = kt;
  return RG_OK;
}

extern "C" rg_status rg_graph_tuned_option(const rg_graph* g, int app, rg_option opt, int64_t* value) {
  if (!g || app < 0 || app > 3 || !value) return fail(RG_EINVAL, "bad arguments");
  if (!g->tuned[app]) {
    *value = -1;
    return RG_OK;
  }
  const Options& o = g->topt[app];
  switch (opt) {
    case RG_OPT_DIRECTION: *value = o.direction; return RG_OK;
    case RG_OPT_HUB_SLOTS: *value = o.hub_slots; return RG_OK;
    case RG_OPT_HUB_SMEM_KB: *value = o.hub_smem_kb; return RG_OK;
    case RG_OPT_DENSE_DIV: *value = o.dense_div; return RG_OK;
    case RG_OPT_SWEEP_SHAPE: *value = o.sweep_shape; return RG_OK;
    case RG_OPT_BC_FWD_HUBS: *value = o.bc_fwd_hubs; return RG_OK;
    case RG_OPT_ASYNC_RESULTS: return fail(RG_EINVAL, "async_results is a thread option, not a schedule");
  }
  return fail(RG_EINVAL, "unknown option %d", (int)opt);
}

extern "C" rg_status rg_graph_set_tuned_option(rg_graph* g, int app, rg_option opt, int64_t value) {
  if (!g || app < 0 || app > 3) return fail(RG_EINVAL, "bad arguments");
  if (!g->tuned[app]) {
    g->topt[app] = g_opts;
    g->tuned[app] = true;
  }
  Options& o = g->topt[app];
  switch (opt) {
    case RG_OPT_DIRECTION: o.direction = value; return RG_OK;
    case RG_OPT_HUB_SLOTS: o.hub_slots = value; return RG_OK;
    case RG_OPT_HUB_SMEM_KB: o.hub_smem_kb = value; return RG_OK;
    case RG_OPT_DENSE_DIV: o.dense_div = value; return RG_OK;
    case RG_OPT_SWEEP_SHAPE: o.sweep_shape = value; return RG_OK;
    case RG_OPT_BC_FWD_HUBS: o.bc_fwd_hubs = value; return RG_OK;
    case RG_OPT_ASYNC_RESULTS: return fail(RG_EINVAL, "async_results is a thread option, not a schedule");
  }
  return fail(RG_EINVAL, "unknown option %d", (int)opt);
}

extern "C" rg_status rg_graph_clear_tuning(rg_graph* g) {
  if (!g) return fail(RG_EINVAL, "null graph");
  for (int a = 0; a < 4; a++) g->tuned[a] = false;
  return RG_OK;
}
