// Batched independent reconstructions (mmh_batch_run): host worker threads,
// each with its own stream and contexts, pull problems from a shared queue.
// Small grids leave most of the GPU idle and spend their time in launch
// latency and host synchronisation; several workers keep several problems in
// flight at once.  Host-only code.
#include <algorithm>
#include <atomic>
#include <map>
#include <numeric>
#include <thread>
#include <vector>

#include "../../include/mmh.h"

namespace {

int run_one(mmh_ctx* ctx, mmh_problem& p) {
  int st = mmh_load_f64(ctx, nullptr, p.rho, 1);
  mmh_diag d{};
  if (st == MMH_OK) st = mmh_iterate(ctx, p.niter, &d);
  p.vcycles = d.vcycles;
  if (st != MMH_OK && st != MMH_ERR_DIVERGED) return st;
  int st2 = MMH_OK;
  if (p.grad || p.delta) st2 = mmh_outputs_f64(ctx, p.grad, p.delta);
  if (st2 == MMH_OK && p.def) st2 = mmh_store_f64(ctx, p.def, nullptr, 1);
  return st2 != MMH_OK ? st2 : st;
}

}  // namespace

extern "C" int mmh_batch_run(const mmh_config* cfg, mmh_problem* probs, int count, int workers) {
  if (!cfg || (count > 0 && !probs) || count < 0 || workers < 1) return MMH_ERR_ARG;
  for (int i = 0; i < count; ++i) {
    if (!probs[i].rho || probs[i].niter < 0) return MMH_ERR_ARG;
    probs[i].status = MMH_OK;
    probs[i].vcycles = 0;
  }
  // largest grids first, so the long problems do not end up last
  std::vector<int> order(count);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return probs[a].n > probs[b].n; });
  std::atomic<int> next{0};
  workers = std::min(workers, std::max(count, 1));
  auto work = [&]() {
    std::map<int, mmh_ctx*> ctxs;
    for (int i; (i = next.fetch_add(1)) < count;) {
      mmh_problem& p = probs[order[i]];
      mmh_ctx*& ctx = ctxs[p.n];
      if (!ctx) {
        mmh_config c = *cfg;
        c.n = p.n;
        c.stream = nullptr;  // each context makes its own stream
        int st = mmh_create(&ctx, &c);
        if (st != MMH_OK) {
          ctx = nullptr;
          p.status = st;
          continue;
        }
      }
      p.status = run_one(ctx, p);
    }
    for (auto& kv : ctxs)
      if (kv.second) mmh_destroy(kv.second);
  };
  std::vector<std::thread> pool;
  for (int w = 1; w < workers; ++w) pool.emplace_back(work);
  work();
  for (std::thread& t : pool) t.join();
  for (int i = 0; i < count; ++i)
    if (probs[i].status != MMH_OK && probs[i].status != MMH_ERR_DIVERGED) return probs[i].status;
  for (int i = 0; i < count; ++i)
    if (probs[i].status != MMH_OK) return probs[i].status;
  return MMH_OK;
}
