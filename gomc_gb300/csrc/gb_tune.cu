// Autotuner of the mixed-form chain geometry: the thread-block cluster size,
// which fixes the k-vectors each CTA holds (the k-chunk), the threads that
// work on one molecule move (cluster size x 256) and whether the cold
// k-chunk arrays fit in shared memory.  Each candidate is timed on the
// box's own system: the box's state is checkpointed, the candidate runs a
// short trial segment, the state is restored; the best candidate is kept.
// No counterpart in the reference (its GPU kernels use fixed launch shapes,
// src/GPU/CalculateEwaldCUDAKernel.cu:29-243).
#include "gomc_gb300.h"
#include "gb_box.h"
#include "gb_mc.h"

#include <cstring>
#include <vector>

namespace gb {

int mc_autotune(Box &b, int objective, int trial_moves, int *chosen,
                double *us_per_move4) {
  if (!b.mc)
    return b.Fail(ERR_STATE, "gb_mc_init has not been called");
  if (b.cfg.precision != GB_MIXED)
    return b.Fail(ERR_UNSUPPORTED, "the FP64 chain has one launch shape");
  if (objective != 0 && objective != 1)
    return b.Fail(ERR_ARG, "objective must be 0 (latency) or 1 (throughput)");
  if (trial_moves <= 0)
    trial_moves = 200;
  gb_mc_params p = b.mc->params;
  int64_t step = b.mc->next_step;
  int rc;
  int64_t bytes;
  checkpoint_size(b, &bytes);
  std::vector<unsigned char> saved((size_t)bytes);
  if ((rc = checkpoint_save(b, saved.data(), bytes)))
    return rc;
  const int cands[4] = {2, 4, 8, 16};
  double best = -1.0;
  int best_c = 0;
  for (int i = 0; i < 4; ++i) {
    if (us_per_move4)
      us_per_move4[i] = 0.0;
    gb_mc_params q = p;
    q.cluster_size = cands[i];
    q.recompute_freq = 0;  // trials measure the chain alone
    if (mc_init(b, q) != OK)
      continue;  // this shape does not fit the box
    if ((rc = checkpoint_load(b, saved.data(), bytes)))
      return rc;
    int conc = max_active_clusters(b.mc->cluster, b.mc->mixed_smem);
    mc_timing(b, 1, nullptr, nullptr, nullptr, nullptr, nullptr);
    // one warm-up segment, then the timed one
    if ((rc = mc_run(b, step, trial_moves / 4 + 1, nullptr, nullptr, nullptr,
                     nullptr)) ||
        (rc = mc_timing(b, 1, nullptr, nullptr, nullptr, nullptr, nullptr)))
      return rc;
    int64_t t0 = step + trial_moves / 4 + 1;
    double ms = 0.0;
    if ((rc = mc_run(b, t0, trial_moves, nullptr, nullptr, nullptr,
                     nullptr)) ||
        (rc = mc_timing(b, 1, &ms, nullptr, nullptr, nullptr, nullptr)))
      return rc;
    double us = ms * 1e3 / trial_moves;
    if (us_per_move4)
      us_per_move4[i] = us;
    double score = objective == 0 ? 1.0 / us : (double)conc / us;
    if (score > best) {
      best = score;
      best_c = cands[i];
    }
  }
  if (!best_c)
    return b.Fail(ERR_UNSUPPORTED, "no cluster shape fits this box");
  // the chosen shape, the saved state
  gb_mc_params q = p;
  q.cluster_size = best_c;
  if ((rc = mc_init(b, q)) || (rc = checkpoint_load(b, saved.data(), bytes)))
    return rc;
  if (chosen)
    *chosen = best_c;
  return OK;
}

}  // namespace gb
