// ctx.h -- the context behind the opaque dpg_ctx handle of include/dpg.h
// (shared by the translation units of the library; not part of the ABI).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "dpg.h"
#include "expand_kernels.cuh"

struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
};

struct dpg_ctx {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  dpg_robot_desc robot{};
  dpg::RobotParams rp{};
  std::string err;

  // primitives
  bool have_prims = false;
  int P = 0;
  int64_t S = 0, A = 0;
  std::vector<int32_t> h_len, h_order;
  std::vector<int64_t> h_soff, h_aoff, h_coff;
  DevBuf len, soff, aoff, order, key32, kconst32, st64, st32, act64, pose32, pose64, pbox, pbox32;
  DevBuf coff, cbox32, tbox32;
  // reverse ball (tdb-A*'s reverse search): keys of each primitive's last state
  DevBuf rkey32, rkconst32, rkrow;
  // key-space grid of the primitives (robots with one or two key components)
  DevBuf kg_start, kg_tab;
  dpg::KeyGrid kg{};  // n0 = 0: no grid

  // environment
  bool have_env = false;
  int dim = 0;
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  int n_obs = 0;
  DevBuf obs32, obs64;

  // per-call arena
  DevBuf x64, nkey32, noff32, mask, cnt, tot, pbase, ord_pbase, ord_ibase;
  DevBuf item_pos;  // work item -> its primitive's position in length order
  DevBuf p_node, p_prim, p_verdict, p_fi, p_end, p_gap, p_flags;
  DevBuf q_node, q_prim, q_sorted, q_idx, q_fill;  // dpg_check_pairs
  DevBuf ord_cell, ord_perm, ord_cnt, ord_start, ord_rank, ord_tiles, x64s;  // spatial order of a batch
  dpg::DevCounters *d_ctr = nullptr;
  dpg::DevCounters *h_ctr = nullptr;  // pinned, 2 entries: after the ball scan, at the end
  // host-buffer expands: result copies overlap the check (copy stream, one
  // event per check launch, pinned mirrors of the item / pair bases)
  cudaStream_t cstream = nullptr;
  cudaStream_t xstream = nullptr;  // every other check launch, so one drains while the next fills
  cudaEvent_t ev_ball = nullptr;
  cudaEvent_t ev_sub[dpg::kMaxSub] = {};
  cudaEvent_t ev_tot = nullptr;
  cudaEvent_t ev_cl[2] = {};  // around the last copy range of a host-buffer expand
  double pipe_decay = 0.75;   // each copy range this fraction of the one before (adapted per call)
  unsigned long long *h_bases = nullptr;  // [2][h_bases_n]: ord_ibase, ord_pbase
  size_t h_bases_n = 0;
  // dpg_lazy_check: candidates by node, ranks, cursors, round lists, counters
  DevBuf lz_off, lz_cnt, lz_cur, lz_next, lz_valid, lz_rank, lz_lnode, lz_ldest, lz_ctr, lz_table;
  void *h_lz = nullptr;  // pinned mirror of the lazy counters
  int *h_rflag = nullptr;  // mapped pinned: copy-range flags of DPG_HOST_OUT_PROGRESS
  int *d_rflag = nullptr;
  int *h_abort = nullptr;             // mapped pinned
  int *d_abort = nullptr;
  // launch choices (dpg_set_tuning): check variant, blocks per SM, the batch
  // size from which the ball scan uses the key grid, pipelined check launches
  dpg_tuning tune{DPG_CHECK_SLOTS, 0, 2048, 8, DPG_HOST_OUT_PROGRESS};
  cudaEvent_t ev[6] = {};
  double timings[4] = {0, 0, 0, 0};
};

