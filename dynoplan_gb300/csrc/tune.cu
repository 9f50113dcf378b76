// tune.cu -- dpg_autotune (include/dpg_tune.h): times the launch choices of
// the expansion on the caller's batch and keeps the fastest, cached per
// workload key.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.h"
#include "dpg.h"
#include "dpg_tune.h"

namespace {

std::string workload_key(const dpg_ctx *c, int64_t N) {
  const int P = c->P;
  int max_len = 1;
  for (int p = 0; p < P; p++) max_len = std::max(max_len, c->h_len[p]);
  int hist[8] = {};
  for (int p = 0; p < P; p++) hist[std::min(7, (int)((int64_t)c->h_len[p] * 8 / (max_len + 1)))]++;
  std::string k = "k" + std::to_string(c->robot.kind) + "_P" + std::to_string(P) + "_Lmax" + std::to_string(max_len) +
                  "_h";
  for (int i = 0; i < 8; i++) {
    k += std::to_string((int)std::lround(16.0 * hist[i] / std::max(P, 1)));
    if (i < 7) k += "-";
  }
  int lg = 0;
  while (((int64_t)1 << (lg + 1)) <= std::max<int64_t>(N, 1)) lg++;
  if (N > ((int64_t)1 << lg) + ((int64_t)1 << lg) / 2) lg++;  // nearest power of two
  k += "_O" + std::to_string(c->n_obs) + "_N2^" + std::to_string(lg);
  return k;
}

bool cache_lookup(const char *path, const std::string &key, dpg_tuning *t, double *ms) {
  if (!path) return false;
  FILE *f = std::fopen(path, "r");
  if (!f) return false;
  char k[256];
  dpg_tuning v{};
  double m = 0;
  bool found = false;
  while (std::fscanf(f, "%255s %d %d %d %d %d %lf", k, &v.check_variant, &v.check_blocks_per_sm,
                     &v.grid_min_nodes, &v.pipe_launches, &v.host_output, &m) == 7) {
    if (key == k) {  // the last line of a key wins
      *t = v;
      *ms = m;
      found = true;
    }
  }
  std::fclose(f);
  return found;
}

void cache_store(const char *path, const std::string &key, const dpg_tuning &t, double ms) {
  if (!path) return;
  FILE *f = std::fopen(path, "a");
  if (!f) return;
  std::fprintf(f, "%s %d %d %d %d %d %.6f\n", key.c_str(), t.check_variant, t.check_blocks_per_sm,
               t.grid_min_nodes, t.pipe_launches, t.host_output, ms);
  std::fclose(f);
}

}  // namespace

extern "C" int dpg_tune_key(const dpg_ctx *c, int64_t N, char *key, int32_t size) {
  if (!c || !key || size <= 0 || N < 0) return DPG_ERR_ARG;
  if (!c->have_prims || !c->have_env) return DPG_ERR_STATE;
  const std::string k = workload_key(c, N);
  std::snprintf(key, (size_t)size, "%s", k.c_str());
  return DPG_OK;
}

extern "C" int dpg_autotune(dpg_ctx *c, const dpg_expand_opts *opts, int64_t N, const double *x_dev, int32_t reps,
                            const char *cache_path, dpg_tune_report *rep) {
  if (!c || !opts || N <= 0 || !x_dev || reps < 1 || reps > 100) return DPG_ERR_ARG;
  if (!c->have_prims || !c->have_env) return DPG_ERR_STATE;
  dpg_tune_report r{};
  r.initial = c->tune;
  const std::string key = workload_key(c, N);
  std::snprintf(r.key, sizeof(r.key), "%s", key.c_str());
  dpg_tuning cached{};
  double cms = 0;
  if (cache_lookup(cache_path, key, &cached, &cms) && dpg_set_tuning(c, &cached) == DPG_OK) {
    r.chosen = cached;
    r.ms_chosen = cms;
    r.from_cache = 1;
    if (rep) *rep = r;
    return DPG_OK;
  }
  const auto t0 = std::chrono::steady_clock::now();
  if (cudaSetDevice(c->device) != cudaSuccess) return DPG_ERR_CUDA;
  dpg_expand_opts o = *opts;
  o.x_on_device = 1;
  o.out_on_device = 1;
  o.mode = 0;
  // output rows: one probe call with no capacity
  dpg_expand_out out{};
  int rc = dpg_expand(c, &o, N, x_dev, &out);
  if (rc != DPG_ERR_CAPACITY && rc != DPG_OK) return rc;
  const int64_t cap = std::max<int64_t>(out.n_pairs, 1);
  const size_t es = o.precision == DPG_FP32 ? sizeof(float) : sizeof(double);
  const size_t row = 4 + 4 + 1 + 2 + es * c->robot.nx + 4 + 1;
  void *buf = nullptr;
  if (cudaMalloc(&buf, row * (size_t)cap + 64 * 8) != cudaSuccess) return DPG_ERR_OOM;
  char *b = static_cast<char *>(buf);
  auto carve = [&](size_t bytes) {
    char *p = b;
    b += (bytes + 255) / 256 * 256;
    return p;
  };
  out = dpg_expand_out{};
  out.capacity = cap;
  out.node = (uint32_t *)carve(4 * cap);
  out.prim = (uint32_t *)carve(4 * cap);
  out.verdict = (uint8_t *)carve(cap);
  out.first_invalid = (int16_t *)carve(2 * cap);
  out.end_state = carve(es * c->robot.nx * cap);
  out.min_gap = (float *)carve(4 * cap);
  out.flags = (uint8_t *)carve(cap);
  (void)b;

  // candidates: narrow-phase variant x resident blocks x key-grid threshold
  std::vector<dpg_tuning> cand;
  const bool grid_choice = N >= 2048 && c->kg.n0 > 0;
  for (int v : {DPG_CHECK_SLOTS, DPG_CHECK_LOCKSTEP})
    for (int bl : {0, 3, 2})
      for (int g : {2048, INT_MAX}) {
        if (!grid_choice && g != 2048) continue;
        cand.push_back(dpg_tuning{v, bl, g, r.initial.pipe_launches, r.initial.host_output});
      }
  auto time_choice = [&](const dpg_tuning &t, double *ms) -> int {
    int e = dpg_set_tuning(c, &t);
    if (e) return e;
    std::vector<double> v;
    for (int i = 0; i <= reps; i++) {
      dpg_expand_out w = out;
      if ((e = dpg_expand(c, &o, N, x_dev, &w))) return e;
      double tm[4];
      dpg_last_timings(c, tm, 4);
      if (i > 0) v.push_back(tm[0] + tm[1]);  // ball scan + check, device time
    }
    std::sort(v.begin(), v.end());
    *ms = v[v.size() / 2];
    return DPG_OK;
  };
  rc = time_choice(r.initial, &r.ms_initial);
  dpg_tuning best = r.initial;
  double best_ms = r.ms_initial;
  for (size_t i = 0; i < cand.size() && rc == DPG_OK; i++) {
    double ms = 0;
    rc = time_choice(cand[i], &ms);
    r.candidates++;
    if (rc == DPG_OK && ms < best_ms * 0.99) {  // a clear win over the incumbent
      best = cand[i];
      best_ms = ms;
    }
  }
  cudaFree(buf);
  if (rc != DPG_OK) {
    dpg_set_tuning(c, &r.initial);
    return rc;
  }
  dpg_set_tuning(c, &best);
  r.chosen = best;
  r.ms_chosen = best_ms;
  r.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  cache_store(cache_path, key, best, best_ms);
  if (rep) *rep = r;
  return DPG_OK;
}
