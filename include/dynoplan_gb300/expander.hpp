// expander.hpp -- C++17 host layer over the C ABI (dpg.h) with the
// reference's interface for the expansion step.
//
// Mirrors, with the same names and argument meaning:
//   Motion                 include/dynoplan/ompl/robots.h:206-235
//   LazyTraj               include/dynoplan/dbastar/dbastar.hpp:160-230
//   Expander               include/dynoplan/dbastar/dbastar.hpp:233-313
//     (delta = the radius, set to alpha * delta by the caller as at
//      src/dbastar/dbastar.cpp:585-586; seed(); random shuffle with
//      std::mt19937 + std::shuffle; max_k cap)
//   check_lazy_trajectory  include/dynoplan/dbastar/dbastar.hpp:334-339,
//                          src/dbastar/dbastar.cpp:391-490
//   Time_benchmark         include/dynoplan/dbastar/options.hpp:16-96 (subset)
// Error behaviour follows the reference: failures throw (the reference's
// CHECK / ERROR_WITH_INFO throw std::runtime_error).
//
// The GPU checks every (node, motion) pair of a batch in one launch, so
// expand_lazy_batch() is the fast entry; expand_lazy() on one state runs a
// batch of one.  check_lazy_trajectory() then returns the verdict the batch
// computed and fills the transformed end state.
//
// Neighbour order before the shuffle: ascending Motion::idx (the order of
// nigh's KD-tree result is an implementation detail of nigh).
#pragma once

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <limits>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "dpg.h"

namespace dynoplan_gb300 {

struct Trajectory {
  std::vector<std::vector<double>> states;
  std::vector<std::vector<double>> actions;
  double cost = 1e8;
};

struct Motion {
  Trajectory traj;
  double cost = 1e8;
  size_t idx = 0;
  bool disabled = false;
  double get_cost() const { return cost; }
  const std::vector<double> &getStateEig() const { return traj.states.front(); }
  const std::vector<double> &getLastStateEig() const { return traj.states.back(); }
};

struct Time_benchmark {
  double time_lazy_expand = 0;      // ms, batch expand (ball scan + checks)
  double time_nearestMotion = 0;    // ms, device ball scan
  double time_collisions = 0;       // ms, device exact check + FP64 re-check
  double time_transform_primitive = 0;
  double check_bounds = 0;
  int expands = 0;
  int num_nn_motions = 0;
  int num_col_motions = 0;
};

// One (node, motion) candidate with the verdict the batch computed.
struct LazyTraj {
  const std::vector<double> *offset = nullptr;  // the node state the motion is applied to
  const Motion *motion = nullptr;
  int verdict = DPG_VALID;
  int first_invalid = 0;
  std::vector<double> end_state;
  float min_gap = 0;
  bool rechecked_fp64 = false;
};

class Robot {
 public:
  dpg_robot_desc desc{};
  dpg_ctx *ctx = nullptr;

  explicit Robot(int32_t kind, int device = 0) {
    check(dpg_robot_default(kind, &desc));
    check(dpg_create(&ctx, device, &desc));
  }
  Robot(const dpg_robot_desc &d, int device = 0) : desc(d) { check(dpg_create(&ctx, device, &desc)); }
  ~Robot() { dpg_destroy(ctx); }
  Robot(const Robot &) = delete;
  Robot &operator=(const Robot &) = delete;

  // load_env (src/dbastar/dbastar.cpp:535): position bounds + boxes
  void load_env(const std::vector<double> &lo, const std::vector<double> &hi,
                const std::vector<std::vector<double>> &obs_lo, const std::vector<std::vector<double>> &obs_hi) {
    const int dim = (int)lo.size();
    std::vector<double> a, b;
    for (size_t i = 0; i < obs_lo.size(); i++) {
      a.insert(a.end(), obs_lo[i].begin(), obs_lo[i].end());
      b.insert(b.end(), obs_hi[i].begin(), obs_hi[i].end());
    }
    check(dpg_upload_env(ctx, dim, lo.data(), hi.data(), (int32_t)obs_lo.size(), a.empty() ? nullptr : a.data(),
                         b.empty() ? nullptr : b.data()));
  }

  void check(int rc) const {
    if (rc != DPG_OK) {
      std::string msg = std::string("dpg: ") + dpg_errstr(rc);
      if (ctx) msg += std::string(": ") + dpg_last_error(ctx);
      throw std::runtime_error(msg);
    }
  }
};

class Expander {
 public:
  Robot *robot;
  const std::vector<Motion> *motions;
  double delta = -1;  // ball radius (alpha * delta of the search)
  bool random = true;
  size_t max_k = std::numeric_limits<size_t>::max();
  int precision = DPG_FP32;
  std::mt19937 g;
  double time_in_nn = 0;

  Expander(Robot *robot, const std::vector<Motion> *motions, double delta)
      : robot(robot), motions(motions), delta(delta) {
    std::random_device rd;
    g = std::mt19937{rd()};
    std::vector<int32_t> len;
    std::vector<double> st, ac;
    for (const Motion &m : *motions) {
      len.push_back((int32_t)m.traj.states.size());
      for (auto &s : m.traj.states) st.insert(st.end(), s.begin(), s.end());
      for (auto &u : m.traj.actions) ac.insert(ac.end(), u.begin(), u.end());
    }
    if (ac.empty()) ac.assign(robot->desc.nu, 0.0);
    robot->check(dpg_upload_primitives(robot->ctx, (int32_t)len.size(), len.data(), st.data(), ac.data()));
  }

  void seed(int s) { g.seed(s); }

  // Batched expand_lazy: out[i] holds the candidates of xs[i], already checked.
  void expand_lazy_batch(const std::vector<std::vector<double>> &xs, std::vector<std::vector<LazyTraj>> &out,
                         Time_benchmark *tb = nullptr) {
    const int nx = robot->desc.nx;
    std::vector<double> flat;
    flat.reserve(xs.size() * nx);
    for (auto &x : xs) {
      if ((int)x.size() != nx) throw std::runtime_error("expand_lazy: state size != nx");
      flat.insert(flat.end(), x.begin(), x.end());
    }
    dpg_expand_opts o{};
    o.radius = delta;
    o.precision = precision;
    o.contact_band = 1e-4;
    o.ball_band = 1e-5;
    int64_t cap = std::max<int64_t>(1024, (int64_t)xs.size() * 64);
    dpg_expand_out r{};
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
      node_.resize(cap); prim_.resize(cap); verdict_.resize(cap); fi_.resize(cap); gap_.resize(cap); flags_.resize(cap);
      es32_.resize(precision == DPG_FP32 ? cap * nx : 0);
      es64_.resize(precision != DPG_FP32 ? cap * nx : 0);
      r = dpg_expand_out{};
      r.capacity = cap;
      r.node = node_.data(); r.prim = prim_.data(); r.verdict = verdict_.data(); r.first_invalid = fi_.data();
      r.end_state = precision == DPG_FP32 ? (void *)es32_.data() : (void *)es64_.data();
      r.min_gap = gap_.data(); r.flags = flags_.data();
      const int rc = dpg_expand(robot->ctx, &o, (int64_t)xs.size(), flat.data(), &r);
      if (rc == DPG_ERR_CAPACITY) { cap = r.n_pairs; continue; }
      robot->check(rc);
      break;
    }
    if (tb) {
      double t[4];
      dpg_last_timings(robot->ctx, t, 4);
      tb->time_nearestMotion += t[0];
      tb->time_collisions += t[1] + t[2];
      tb->time_lazy_expand +=
          std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      tb->num_nn_motions += (int)xs.size();
    }
    // group by node, motions ascending, then shuffle and cap per node
    std::vector<int64_t> count(xs.size() + 1, 0);
    for (int64_t i = 0; i < r.n_pairs; i++) count[node_[i] + 1]++;
    for (size_t n = 0; n < xs.size(); n++) count[n + 1] += count[n];
    std::vector<int64_t> rows(r.n_pairs), fill(count.begin(), count.end() - 1);
    for (int64_t i = 0; i < r.n_pairs; i++) rows[fill[node_[i]]++] = i;
    out.assign(xs.size(), {});
    for (size_t n = 0; n < xs.size(); n++) {
      auto b = rows.begin() + count[n], e = rows.begin() + count[n + 1];
      std::sort(b, e, [&](int64_t a, int64_t c) { return prim_[a] < prim_[c]; });
      if (random) std::shuffle(b, e, g);
      const size_t k = std::min<size_t>(e - b, max_k);
      out[n].reserve(k);
      for (size_t j = 0; j < k; j++) {
        const int64_t i = *(b + j);
        LazyTraj lt;
        lt.offset = &xs[n];
        lt.motion = &(*motions)[prim_[i]];
        lt.verdict = verdict_[i];
        lt.first_invalid = fi_[i];
        lt.min_gap = gap_[i];
        lt.rechecked_fp64 = flags_[i] & DPG_FLAG_CONTACT_RECHECK;
        lt.end_state.resize(nx);
        for (int c = 0; c < nx; c++)
          lt.end_state[c] = precision == DPG_FP32 ? (double)es32_[i * nx + c] : es64_[i * nx + c];
        out[n].push_back(std::move(lt));
      }
    }
  }

  // Expander::expand_lazy (dbastar.hpp:270-312) for one state.
  void expand_lazy(const std::vector<double> &x, std::vector<LazyTraj> &lazy_trajs) {
    if (!lazy_trajs.empty()) throw std::runtime_error("expand_lazy: lazy_trajs must be empty");
    std::vector<std::vector<LazyTraj>> out;
    one_[0] = x;
    expand_lazy_batch(one_, out);
    lazy_trajs = std::move(out[0]);
  }

 private:
  std::vector<std::vector<double>> one_ = std::vector<std::vector<double>>(1);
  std::vector<uint32_t> node_, prim_;
  std::vector<uint8_t> verdict_, flags_;
  std::vector<int16_t> fi_;
  std::vector<float> gap_, es32_;
  std::vector<double> es64_;
};

// check_lazy_trajectory (dbastar.cpp:391-490): true iff the transformed
// motion stays in bounds and collision-free.  aux_last_state receives the
// transformed last state; num_valid_states the number of states before the
// first out-of-bounds one (the bounded rollout's count).
inline bool check_lazy_trajectory(LazyTraj &lazy_traj, Time_benchmark &time_bench,
                                  std::vector<double> &aux_last_state, int *num_valid_states = nullptr) {
  if (!lazy_traj.motion) throw std::runtime_error("check_lazy_trajectory: no motion");
  aux_last_state = lazy_traj.end_state;
  if (num_valid_states)
    *num_valid_states = lazy_traj.verdict == DPG_OUT_OF_BOUNDS ? lazy_traj.first_invalid
                                                               : (int)lazy_traj.motion->traj.states.size();
  if (lazy_traj.verdict != DPG_OUT_OF_BOUNDS) time_bench.num_col_motions++;
  return lazy_traj.verdict == DPG_VALID;
}

}  // namespace dynoplan_gb300
