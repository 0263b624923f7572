// Autotuner of the chain's launch shape.  Mixed form: the thread-block
// cluster size, which fixes the k-vectors each CTA holds (the k-chunk) and
// the CTAs that work on one molecule move, times the threads that tile one
// real-space unit (an atom position against a neighbour cell's slots).
// FP64 form: the CTAs of the cooperative grid (the threads on one move and
// the k-chunk per CTA) times whether the CTAs that write the next move's
// context also hold k-vectors (the k-chunk at a fixed grid) times one or
// two moves in flight.  Each candidate
// is timed on the box's own system: the box's state is checkpointed, the
// candidate runs a short trial segment, the state is restored; the best
// candidate is kept.  No counterpart in the reference (its GPU kernels use
// fixed launch shapes, src/GPU/CalculateEwaldCUDAKernel.cu:29-243).
#include "gomc_gb300.h"
#include "gb_box.h"
#include "gb_mc.h"

#include <cstring>
#include <vector>

namespace gb {

int mc_autotune(Box &b, int objective, int trial_moves, gb_mc_shape *chosen,
                gb_mc_shape *tried, int cap, int *n_tried) {
  if (!b.mc)
    return b.Fail(ERR_STATE, "gb_mc_init has not been called");
  if (objective != 0 && objective != 1)
    return b.Fail(ERR_ARG, "objective must be 0 (latency) or 1 (throughput)");
  if (trial_moves <= 0)
    trial_moves = 200;
  const bool mixed = b.cfg.precision == GB_MIXED;
  gb_mc_params p = b.mc->params;
  int64_t step = b.mc->next_step;
  int rc;
  int64_t bytes;
  checkpoint_size(b, &bytes);
  std::vector<unsigned char> saved((size_t)bytes);
  if ((rc = checkpoint_save(b, saved.data(), bytes)))
    return rc;
  // the candidate shapes, in the order tried
  std::vector<gb_mc_shape> cands;
  if (mixed) {
    for (int c : {2, 4, 8, 16})
      for (int lanes : {32, 64, 128, 256})
        cands.push_back({c, lanes, 0, 0, 0, 0.0});
  } else {
    const int sms = b.sm_count;
    int prev = 0;
    for (int num : {4, 3, 2, 1}) {
      const int g = sms * num / 4;
      if (g < 2 || g == prev)
        continue;
      prev = g;
      for (int wk : {0, 1})
        for (int fl : {1, 2})
          cands.push_back({g, 0, wk, fl, 1, 0.0});
    }
  }
  double best = -1.0;
  gb_mc_shape best_s{};
  int n = 0;
  for (gb_mc_shape &cs : cands) {
    gb_mc_params q = p;
    q.recompute_freq = 0;  // trials measure the chain alone
    if (mixed) {
      q.cluster_size = cs.ctas;
      q.unit_lanes = cs.unit_lanes;
    } else {
      q.grid_ctas = cs.ctas;
      q.writer_kchunk = cs.writer_kchunk;
      q.moves_in_flight = cs.moves_in_flight;
    }
    if (mc_init(b, q) == OK) {
      if ((rc = checkpoint_load(b, saved.data(), bytes)))
        return rc;
      if (mixed)
        cs.max_concurrent = max_active_clusters(b.mc->cluster, b.mc->mixed_smem);
      mc_timing(b, 1, nullptr, nullptr, nullptr, nullptr, nullptr);
      // one warm-up segment, then the timed one
      if ((rc = mc_run(b, step, trial_moves / 4 + 1, nullptr, nullptr,
                       nullptr, nullptr)) ||
          (rc = mc_timing(b, 1, nullptr, nullptr, nullptr, nullptr, nullptr)))
        return rc;
      int64_t t0 = step + trial_moves / 4 + 1;
      double ms = 0.0;
      if ((rc = mc_run(b, t0, trial_moves, nullptr, nullptr, nullptr,
                       nullptr)) ||
          (rc = mc_timing(b, 1, &ms, nullptr, nullptr, nullptr, nullptr)))
        return rc;
      cs.us_per_move = ms * 1e3 / trial_moves;
      double score = objective == 0 ? 1.0 / cs.us_per_move
                                    : (double)cs.max_concurrent / cs.us_per_move;
      if (score > best) {
        best = score;
        best_s = cs;
      }
    }
    // shapes that do not fit the box are reported with zero time
    if (tried && n < cap)
      tried[n] = cs;
    ++n;
  }
  if (n_tried)
    *n_tried = n < cap || !tried ? n : cap;
  if (best < 0.0)
    return b.Fail(ERR_UNSUPPORTED, "no launch shape fits this box");
  // the chosen shape, the saved state
  gb_mc_params q = p;
  if (mixed) {
    q.cluster_size = best_s.ctas;
    q.unit_lanes = best_s.unit_lanes;
  } else {
    q.grid_ctas = best_s.ctas;
    q.writer_kchunk = best_s.writer_kchunk;
    q.moves_in_flight = best_s.moves_in_flight;
  }
  if ((rc = mc_init(b, q)) || (rc = checkpoint_load(b, saved.data(), bytes)))
    return rc;
  if (chosen)
    *chosen = best_s;
  return OK;
}

}  // namespace gb
