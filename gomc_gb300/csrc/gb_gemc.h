// Gibbs ensemble (GEMC NVT) of single-site LJ particles in two boxes, run
// on the device as one persistent thread-block cluster (gb_gemc.cu).
#pragma once

#include "gomc_gb300.h"
#include "gb_internal.h"

#include <string>
#include <vector>

namespace gb {

constexpr int GEMC_KINDS = 14;    // move kinds of the reference's GEMC build
constexpr int GEMC_DISPLACE = 0;  // src/MoveConst.h
constexpr int GEMC_ROTATE = 1;
constexpr int GEMC_TRANSFER = 10;
constexpr int GEMC_VOLUME = 13;
constexpr int GEMC_NTMAX = 16;    // CBMC first-atom trials per build
constexpr int GEMC_THREADS = 256;

// The dynamic state of a Gibbs-ensemble run: box geometry, running energies,
// move settings (src/MoveSettings.h) and the MT19937 position.  Kept in
// global memory between launches and in every CTA's shared memory during
// one.  Counters: [box][0 displacement, 1 transfer, 2 volume].
struct GemcCtl {
  double ax[2][3], half[2][3], vol[2], volInv[2], minVol[2];
  double e[2];
  double scale[2][3];  // displacement, rotation, volume exchange
  long long tries[2][3], acc[2][3], ttries[2][3], tacc[2][3];
  int start1;          // molecules in box 0 (the lookup's box boundary)
  int err;             // 1: a volume exchange would shrink a box below 2 Rcut
  int mt_left, mt_next;
  unsigned mt[624];
};

// Constants of a run and the device pointers the kernel works on.
struct GemcParams {
  int n, nt, adj, cluster;
  double perc[GEMC_KINDS];
  double cum[GEMC_KINDS];     // cumulative weights of PickArbDist's walk
  double boxdiv[GEMC_KINDS];  // movPerc / 2 (PRNG::PickBox)
  double sigmaSq, eps_cn, nexp, rcut, rcutSq, rcutLowSq, beta;
  float sigmaSq_f, eps_cn_f, rcutSq_f, rcutLowSq_f;
  double *x, *y, *z, *cx, *cy, *cz;  // positions and centres (FP64 masters)
  int *lookup;                        // molecule lookup, box 0 then box 1
  GemcCtl *ctl;
  long long first;
  int nsteps;
  int *tr_i;     // per step: kind, box, molecule, accepted, molecules in box 0
  double *tr_d;  // per step: four move values, energies, volumes
  // phase clocks of CTA 0 (NULL: not collected): [kind slot 0 displacement,
  // 1 transfer, 2 volume][phase: draw, energies, exchange, decision,
  // commit], then the moves of each kind slot
  long long *prof;
};

struct Gemc {
  int device = 0, precision = 0, cluster = 16;
  cudaStream_t stream = nullptr;
  GemcParams p{};
  GemcCtl h_ctl{};
  std::vector<void *> allocs;
  size_t smem = 0;
  std::string last_error;
  int64_t next_step = 0;
  int *d_tr_i = nullptr;
  double *d_tr_d = nullptr;
  size_t trace_cap = 0;
  double *d_tot = nullptr;  // recompute output
  float last_ms = 0.0f;     // device time of the last run
  long long *d_prof = nullptr;  // phase clocks (gb_gemc_profile)
  bool profile = false;
  int Fail(int code, const std::string &msg) {
    last_error = msg;
    return code;
  }
  int CudaCheck(cudaError_t e, const char *what) {
    if (e == cudaSuccess)
      return OK;
    last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? ERR_NOMEM : ERR_CUDA;
  }
};

size_t gemc_smem(int n, int mixed);
int gemc_launch(Gemc &g, int nsteps, cudaEvent_t e0, cudaEvent_t e1);
int gemc_recompute(Gemc &g, double *e2);

}  // namespace gb
