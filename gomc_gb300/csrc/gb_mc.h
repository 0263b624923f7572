// Device-resident Monte Carlo loop: MT19937 move stream on the host,
// persistent chain kernels on the device, MultiParticle as a kernel sequence.
#pragma once

#include "gomc_gb300.h"
#include "gb_box.h"

#include <cstdint>
#include <vector>

namespace gb {

// One pre-drawn move (everything that does not depend on accept history).
struct MoveRec {
  int32_t kind;   // 0 displacement, 1 rotation, 2 multiparticle
  int32_t mol;    // molecule (kinds 0/1) or MultiParticle type (kind 2)
  double u[3];    // displacement: three rand() draws; rotation: u[0] = angle draw
  double ax[3];   // rotation axis (PRNG::PickOnUnitSphere, src/PRNG.h:143-151)
  double pacc;    // Metropolis uniform (Translate::Accept, src/moves/Translate.h:101)
  double lpacc;   // log(pacc), for the mixed form's log-domain comparison
};

// MoveSettings state (src/MoveSettings.h:28-160) for one box, one kind.
struct Settings {
  double scale[2];          // DISPLACE, ROTATE
  double mp_t_max, mp_r_max;
  long long tries[3], accepted[3], tempTries[3], tempAccepted[3];
  long long mp_tries[2], mp_acc[2], mp_itries[2], mp_iacc[2];
  int singleMoveAccepted;
  int adj;
  double amin;              // smallest box edge
};

// MT19937 (Matsumoto & Nishimura 1998) seeded as MTRand(uint32)
// (src/MersenneTwister.h:194-230) and the PRNG wrappers the moves draw from
// (src/PRNG.h:48-170).
class MT19937 {
 public:
  explicit MT19937(uint32_t seed);
  uint32_t u32();
  double rand01() { return (double)u32() * (1.0 / 4294967295.0); }
  double randExc01() { return (double)u32() * (1.0 / 4294967296.0); }
  uint32_t randInt(uint32_t n);
  // the generator's full state (checkpoints)
  void Save(uint32_t st[624], int32_t *left, int32_t *next) const;
  void Load(const uint32_t st[624], int32_t left, int32_t next);

 private:
  void reload();
  uint32_t st_[624];
  int left_ = 0, next_ = 0;
};

// Host generator of the move stream of one box (System::PickMove,
// MolTransformBase::GetBoxAndMol, Coordinates::TranslateRand / RotateRand,
// MultiParticle::Prep, the Accept draw).
class MoveStream {
 public:
  MoveStream(uint32_t seed, const double frac[3], int n_mol,
             const std::vector<int> &mol_len);
  void Next(MoveRec *r);
  MT19937 &mt() { return mt_; }

 private:
  MT19937 mt_;
  double perc_[9];
  int n_mol_;
  std::vector<int> mol_len_;
  bool all_single_;
};

struct MixedChain;

struct McState {
  gb_mc_params params{};
  // mixed form: cluster size, descriptor ring, drift records
  int cluster = 0;
  size_t mixed_smem = 0;
  unsigned char *d_cold = nullptr;  // cold per-k arrays when not in smem
  MixedChain *d_desc = nullptr;   // [desc_cap]
  MixedChain *h_desc = nullptr;   // pinned
  int desc_cap = 0, desc_next = 0;
  int ulog = 7;  // log2 of the threads per real-space unit
  double drift_max[4] = {0, 0, 0, 0};  // inter, real, recip, total (relative)
  double drift_last[4] = {0, 0, 0, 0};
  int64_t recomputes = 0;
  MoveStream *stream = nullptr;
  int64_t next_step = 0;     // step the stream is positioned at
  // moves drawn ahead of next_step (batched runs look ahead for the next
  // MultiParticle move, where a box's chain segment has to end), and a copy
  // of the stream from before the first of them (checkpoints save the
  // generator's position at next_step)
  std::vector<MoveRec> ahead;
  size_t ahead_pos = 0;
  MoveStream *ahead_from = nullptr;
  Settings *d_set = nullptr; // device copy of Settings
  MoveRec *d_moves = nullptr;
  MoveRec *h_moves = nullptr;  // pinned
  size_t move_cap = 0;
  double *d_prop = nullptr;  // per-move proposal (matrix or shift)
  int *d_trace_i = nullptr;  // kind, mol, acc per step
  double *d_trace_d = nullptr;
  size_t trace_cap = 0;
  double *d_part = nullptr;  // per-CTA partials
  unsigned *d_seq = nullptr; // FP64 chain decision and per-CTA flags
  int na_max = 1;            // atoms of the largest molecule
  unsigned *d_bar = nullptr; // grid barrier words
  double *d_ctx = nullptr;   // per-move context (positions, tables)
  int grid = 0, kchunk = 0;
  bool pipe = false;  // FP64 chain: two moves in flight (k_chain_fp64_pipe)
  // MultiParticle buffers (new state)
  double *d_xn = nullptr, *d_yn = nullptr, *d_zn = nullptr;
  double *d_cxn = nullptr, *d_cyn = nullptr, *d_czn = nullptr;
  double *d_aFn = nullptr, *d_mFn = nullptr, *d_aRn = nullptr,
         *d_mRn = nullptr, *d_tqn = nullptr, *d_tk = nullptr;
  int *d_inrange = nullptr;
  double *d_mp = nullptr;    // MultiParticle scalars
  DevBox cells_new{};        // cell grid of the trial state
  std::vector<void *> allocs;
  size_t bytes = 0;          // device memory of the Monte Carlo state
  // device-time accounting (CUDA events on the box stream)
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> chain_ev, mp_ev;
  std::vector<int> chain_ev_moves;
  double chain_ms = 0.0, mp_ms = 0.0;
  int64_t chain_launches = 0, chain_moves = 0, mp_moves = 0;
  long long *d_prof = nullptr;  // FP64 chain phase clocks (gb_mc_profile)
  unsigned spin_limit = 1u << 22;  // polls of a device wait (gb_mc_set_wait_limit)
  bool profile = false;
};

int mc_timing(Box &b, int reset, double *chain_ms, int64_t *chain_launches,
              int64_t *chain_moves, double *mp_ms, int64_t *mp_moves);
int mc_profile(Box &b, int enable, double *us13, int64_t *moves2);
int mc_set_wait_limit(Box &b, int64_t polls);

// One chain of the mixed-precision chain kernel (gb_mixed.cu).
struct MixedChain {
  DevBox b;
  const FF *ff;
  Settings *set;
  const MoveRec *moves;
  double *prop;
  int64_t first;
  int n;
  int ulog;  // log2 of the threads per real-space unit (5, 6 or 7)
  int *tr_i;
  double *tr_d;
  unsigned char *cold;  // cold per-k arrays in global memory (NULL: in smem)
};
// Dynamic shared memory of one CTA, with or without the cold arrays.
size_t mixed_smem(int K, int kmax, int csize, bool cold_smem);
// Bytes of the global buffer that holds the cold arrays of one chain.
size_t mixed_cold_buffer(int K, int csize);
int launch_chain_mixed(cudaStream_t st, const MixedChain *d_chains, int nchains,
                       int csize, size_t smem);
int max_active_clusters(int csize, size_t smem);

int mc_init(Box &b, const gb_mc_params &p);
int mc_run(Box &b, int64_t first_step, int64_t nsteps, int32_t *kind,
           int32_t *mol, int32_t *acc, double *de);
int mc_state(Box &b, double *scales4, int64_t *counts6);
int mc_run_batch(const std::vector<Box *> &boxes, int64_t first_step,
                 int64_t nsteps);

// Largest dynamic shared memory the mixed chain kernel asks for per CTA.
constexpr size_t MIXED_SMEM_MAX = 214 * 1024;  // plus ~11 KB static: under 227 KB
// Batched segments of mixed boxes (gb_mc.cu): mixed_launch uploads the next
// n[i] moves of box i and launches one kernel per cluster size on the stream
// of that group's first box (`leaders`); mixed_complete waits for them and
// runs the periodic FP64 recomputes that fall due, or, given `due`, marks
// them there for the caller to run (mc_recompute).  mixed_segment_limit is
// the longest segment (at most cap) that ends at or before the box's next
// recompute boundary.
int mixed_launch(const std::vector<Box *> &boxes,
                 const std::vector<int64_t> &n, std::vector<Box *> *leaders);
int mixed_complete(const std::vector<Box *> &boxes,
                   const std::vector<int64_t> &n,
                   const std::vector<Box *> &leaders,
                   std::vector<char> *due = nullptr);
int mc_recompute(Box &b);
int64_t mixed_segment_limit(Box &b, int64_t cap);
// The next move record of box b's stream (drawn-ahead records first).
void draw_next(McState &s, MoveRec *r);
// The MT19937 state of the stream positioned at next_step.
void stream_state_at_next(McState &s, uint32_t st[624], int32_t *left,
                          int32_t *next);
void mc_destroy(Box &b);

// Timed choice of the chain's launch shape (gb_tune.cu)
int mc_autotune(Box &b, int objective, int trial_moves, gb_mc_shape *chosen,
                gb_mc_shape *tried, int cap, int *n_tried);

// The reference's checkpoint file (gb_gomc_chk.cu)
int gomc_chk_read(const void *buf, int64_t bytes, gb_gomc_chk *out);
int gomc_chk_write(const void *tmpl, int64_t tbytes, const gb_gomc_chk *in,
                   void *out, int64_t cap, int64_t *out_bytes);
int mc_get_gomc_state(Box &b, gb_gomc_chk *c);
int mc_set_gomc_state(Box &b, const gb_gomc_chk *c);

// Checkpoints of a box's dynamic state (gb_ckpt.cu)
int checkpoint_size(Box &b, int64_t *bytes);
int checkpoint_save(Box &b, void *buf, int64_t bytes);
int checkpoint_load(Box &b, const void *buf, int64_t bytes);

}  // namespace gb
