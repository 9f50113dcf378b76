// C++ check of the reference-shaped interface (include/dynoplan_gb300/expander.hpp)
// over the C ABI.  Usage: test_expander <input.bin> <output.bin>
//
// input  (little endian): int32 kind, int32 P, int32 len[P], f64 states[sum L][nx],
//        f64 actions[sum(L-1)][nu], int32 dim, f64 lo[dim], f64 hi[dim], int32 O,
//        f64 obs_lo[O][dim], f64 obs_hi[O][dim], int64 N, f64 x[N][nx], f64 radius
// output: int64 rows, then rows of (int32 node, int32 idx, int32 verdict,
//        int32 first_invalid, f64 end_state[nx]); node-major, idx ascending.
// It also checks, and reports on stderr, the interface contract: expand_lazy
// on one state == the batch row, seeded shuffles repeat, max_k caps.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>

#include "dynoplan_gb300/expander.hpp"

using namespace dynoplan_gb300;

template <class T> static T rd(std::ifstream &f) {
  T v;
  f.read(reinterpret_cast<char *>(&v), sizeof(T));
  return v;
}

#define EXPECT(c)                                                  \
  do {                                                             \
    if (!(c)) {                                                    \
      std::cerr << "FAILED: " #c " at line " << __LINE__ << "\n"; \
      return 1;                                                    \
    }                                                              \
  } while (0)

int main(int argc, char **argv) {
  if (argc != 3) return 2;
  std::ifstream f(argv[1], std::ios::binary);
  const int kind = rd<int32_t>(f);
  Robot robot(kind);
  const int nx = robot.desc.nx, nu = robot.desc.nu;
  const int P = rd<int32_t>(f);
  std::vector<int32_t> len(P);
  for (auto &l : len) l = rd<int32_t>(f);
  std::vector<Motion> motions(P);
  for (int p = 0; p < P; p++) {
    motions[p].idx = p;
    motions[p].traj.states.assign(len[p], std::vector<double>(nx));
    for (auto &s : motions[p].traj.states)
      for (auto &v : s) v = rd<double>(f);
  }
  for (int p = 0; p < P; p++) {
    motions[p].traj.actions.assign(len[p] - 1, std::vector<double>(nu));
    for (auto &u : motions[p].traj.actions)
      for (auto &v : u) v = rd<double>(f);
  }
  const int dim = rd<int32_t>(f);
  std::vector<double> lo(dim), hi(dim);
  for (auto &v : lo) v = rd<double>(f);
  for (auto &v : hi) v = rd<double>(f);
  const int O = rd<int32_t>(f);
  std::vector<std::vector<double>> olo(O, std::vector<double>(dim)), ohi(O, std::vector<double>(dim));
  for (auto &o : olo)
    for (auto &v : o) v = rd<double>(f);
  for (auto &o : ohi)
    for (auto &v : o) v = rd<double>(f);
  const int64_t N = rd<int64_t>(f);
  std::vector<std::vector<double>> xs(N, std::vector<double>(nx));
  for (auto &x : xs)
    for (auto &v : x) v = rd<double>(f);
  const double radius = rd<double>(f);
  robot.load_env(lo, hi, olo, ohi);

  Expander expander(&robot, &motions, radius);
  expander.random = false;
  std::vector<std::vector<LazyTraj>> out;
  Time_benchmark tb;
  expander.expand_lazy_batch(xs, out, &tb);

  // interface contract
  {
    std::vector<LazyTraj> one;
    expander.expand_lazy(xs[0], one);
    EXPECT(one.size() == out[0].size());
    for (size_t j = 0; j < one.size(); j++) {
      EXPECT(one[j].motion->idx == out[0][j].motion->idx);
      EXPECT(one[j].verdict == out[0][j].verdict);
    }
    bool threw = false;
    if (one.empty()) one.push_back(LazyTraj{});
    try {
      expander.expand_lazy(xs[0], one);  // the reference asserts an empty list
    } catch (const std::runtime_error &) {
      threw = true;
    }
    EXPECT(threw);
    Expander sh(&robot, &motions, radius);
    std::vector<LazyTraj> a, b;
    sh.seed(0);
    sh.expand_lazy(xs[0], a);
    sh.seed(0);
    sh.expand_lazy(xs[0], b);
    EXPECT(a.size() == b.size());
    for (size_t j = 0; j < a.size(); j++) EXPECT(a[j].motion == b[j].motion);
    sh.max_k = 3;
    std::vector<LazyTraj> c;
    sh.expand_lazy(xs[0], c);
    EXPECT(c.size() == std::min<size_t>(3, a.size()));
    int valid = 0;
    for (auto &lt : out[0]) {
      std::vector<double> aux;
      int nv = -1;
      const bool ok = check_lazy_trajectory(lt, tb, aux, &nv);
      EXPECT(ok == (lt.verdict == DPG_VALID));
      EXPECT((int)aux.size() == nx);
      valid += ok;
    }
    std::cerr << "node 0: " << out[0].size() << " candidates, " << valid << " valid\n";
  }

  FILE *o = std::fopen(argv[2], "wb");
  int64_t rows = 0;
  for (auto &v : out) rows += (int64_t)v.size();
  std::fwrite(&rows, 8, 1, o);
  for (int64_t n = 0; n < N; n++)
    for (auto &lt : out[n]) {
      int32_t rec[4] = {(int32_t)n, (int32_t)lt.motion->idx, lt.verdict, lt.first_invalid};
      std::fwrite(rec, 4, 4, o);
      std::fwrite(lt.end_state.data(), 8, nx, o);
    }
  std::fclose(o);
  std::cerr << "rows " << rows << " lazy_expand_ms " << tb.time_lazy_expand << "\n";
  return 0;
}
