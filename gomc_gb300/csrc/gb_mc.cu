// Device-resident Monte Carlo loop (FP64 plain form).
//
// Host: an MT19937 stream (the reference's PRNG, src/PRNG.h,
// src/MersenneTwister.h) pre-draws every number that does not depend on the
// accept history -- move kind, molecule, displacement and angle draws, the
// rotation axis and the Metropolis uniform -- into MoveRec records.
//
// Device: a persistent cooperative "chain" kernel runs a segment of
// displacement / rotation moves on one CTA per SM.  Every CTA owns a fixed
// chunk of k-vectors, whose Ref and New structure factors live in its shared
// memory for the whole segment, and a strided share of the atoms, whose
// positions, charges and fixed-point turns live there too.  Per move:
//   phase A  all CTAs: the moved atoms (old and new positions) against the
//            own atoms (every G-th atom) (FP32 pre-test, FP64 pair terms of the pairs inside
//            the cutoff) and the k-chunk's structure-factor change ->
//            partial slots in global memory
//   phase B  the last CTA adds the partials in one fixed order, takes the
//            Metropolis decision, commits the coordinates and publishes the
//            decision in one word; every CTA then commits its own k-chunk
//            and own atoms.  Meanwhile designated CTAs build the next
//            move's context (header and phase tables) in global memory.
// The cell grid is rebuilt from the coordinates after each segment
// (CellList::GridAll).
// Move-size adjustment (MoveSettings::AdjustMoves) is replayed identically in
// every CTA.  Barriers spin a bounded number of times and then raise an error
// flag that the host turns into GB_ERR_TIMEOUT.
//
// MultiParticle moves run as a kernel sequence between chain segments
// (src/moves/MultiParticle.h:164-544), with Philox4x64-10 keyed
// (step, seed) as in Random123Wrapper (src/Random123Wrapper.cpp:16-84).
#include "gb_mc.h"
#include "gb_cells.cuh"
#include "gb_moves.cuh"
#include "gb_pair.cuh"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <system_error>
#include <thread>

namespace gb {

// ===========================================================================
// Host: MT19937 and the move stream
// ===========================================================================
MT19937::MT19937(uint32_t seed) {
  st_[0] = seed;
  for (int i = 1; i < 624; ++i)
    st_[i] = 1812433253u * (st_[i - 1] ^ (st_[i - 1] >> 30)) + (uint32_t)i;
  reload();
}

void MT19937::reload() {
  for (int i = 0; i < 624; ++i) {
    uint32_t nx = st_[(i + 1) % 624];
    uint32_t y = (st_[i] & 0x80000000u) | (nx & 0x7fffffffu);
    st_[i] = st_[(i + 397) % 624] ^ (y >> 1) ^ ((nx & 1u) ? 0x9908b0dfu : 0u);
  }
  left_ = 624;
  next_ = 0;
}

uint32_t MT19937::u32() {
  if (left_ == 0)
    reload();
  --left_;
  uint32_t y = st_[next_++];
  y ^= (y >> 11);
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  return y ^ (y >> 18);
}

void MT19937::Save(uint32_t st[624], int32_t *left, int32_t *next) const {
  for (int i = 0; i < 624; ++i)
    st[i] = st_[i];
  *left = left_;
  *next = next_;
}

void MT19937::Load(const uint32_t st[624], int32_t left, int32_t next) {
  for (int i = 0; i < 624; ++i)
    st_[i] = st[i];
  left_ = left;
  next_ = next;
}

uint32_t MT19937::randInt(uint32_t n) {
  uint32_t used = n;
  used |= used >> 1;
  used |= used >> 2;
  used |= used >> 4;
  used |= used >> 8;
  used |= used >> 16;
  uint32_t i;
  do
    i = u32() & used;
  while (i > n);
  return i;
}

MoveStream::MoveStream(uint32_t seed, const double frac[3], int n_mol,
                       const std::vector<int> &mol_len)
    : mt_(seed), n_mol_(n_mol), mol_len_(mol_len) {
  // StaticVals normalises movePerc over the nine NVT move kinds
  // (src/StaticVals.cpp:37-96, src/MoveConst.h:22-33).
  double tot = 0.0;
  double raw[9] = {frac[0], frac[1], frac[2], 0, 0, 0, 0, 0, 0};
  for (int i = 0; i < 9; ++i)
    tot += raw[i];
  for (int i = 0; i < 9; ++i)
    perc_[i] = raw[i] / tot;
  all_single_ = true;
  for (int l : mol_len)
    if (l != 1)
      all_single_ = false;
}

void MoveStream::Next(MoveRec *r) {
  std::memset(r, 0, sizeof(MoveRec));
  // PRNG::PickArbDist (src/PRNG.h:153-163) with Wt = 1
  double sum = 0.0, draw = mt_.rand01() * 1.0;
  int pick;
  for (pick = 0; pick < 9 && sum < draw; ++pick)
    sum += perc_[pick];
  if (pick != 0)
    --pick;
  if (pick > 2 || perc_[pick] == 0.0) {
    // only reachable by rounding at draw ~ 1: the last kind with weight
    pick = perc_[2] > 0 ? 2 : (perc_[1] > 0 ? 1 : 0);
  }
  if (pick == 2) {
    // MultiParticle::Prep: randIntExc(MPTOTALTYPES) unless all molecules
    // are single sites (src/moves/MultiParticle.h:178-183)
    r->kind = 2;
    r->mol = all_single_ ? 0 : (int)mt_.randInt(1);
    return;
  }
  // PRNG::PickMolAndBox, one box and one movable kind: randIntExc(count)
  uint32_t m = mt_.randInt((uint32_t)(n_mol_ - 1));
  r->mol = (int)m;
  if (pick == 1 && mol_len_[m] <= 1)
    pick = 0;  // ROTATE_ON_SINGLE_ATOM -> displacement (src/System.cpp:291-297)
  r->kind = pick;
  if (pick == 0) {
    // Coordinates::TranslateRand -> PRNG::SymXYZ (src/PRNG.h:69-75)
    r->u[0] = mt_.rand01();
    r->u[1] = mt_.rand01();
    r->u[2] = mt_.rand01();
  } else {
    // Coordinates::RotateRand: Sym(max), then PickOnUnitSphere
    r->u[0] = mt_.rand01();
    double u = mt_.rand01() * 2.0 - 1.0;
    double theta = mt_.randExc01() * (2.0 * M_PI);
    double rootTerm = std::sqrt(1.0 - u * u);
    r->ax[0] = rootTerm * std::cos(theta);
    r->ax[1] = rootTerm * std::sin(theta);
    r->ax[2] = u;
  }
  r->pacc = mt_.rand01();  // Translate/Rotate::Accept prng()
  r->lpacc = std::log(r->pacc);
}

// ===========================================================================
// Device helpers
// ===========================================================================
__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

constexpr unsigned SPIN_LIMIT = 1u << 22;  // default polls of a device wait

// Grid-wide barrier with a bounded wait.  bar[0] counts arrivals, bar[1] is
// the generation.  Returns false (and sets DERR_BARRIER_TIMEOUT) when the
// wait gives up or another CTA reported an error.
__device__ bool grid_sync(unsigned *bar, unsigned nblocks, unsigned &gen,
                          int *err, int *s_flag, unsigned limit) {
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    unsigned g = gen;
    __threadfence();
    unsigned prev = atomicAdd(&bar[0], 1u);
    if (prev == nblocks - 1) {
      bar[0] = 0;
      __threadfence();
      atomicExch(&bar[1], g + 1);
    } else {
      unsigned it = 0;
      while (ld_acquire(&bar[1]) == g) {
        if (++it > limit) {
          atomicOr(err, DERR_BARRIER_TIMEOUT);
          ok = 0;
          break;
        }
        if ((it & 255u) == 0 && *(volatile int *)err) {
          ok = 0;
          break;
        }
      }
    }
    __threadfence();
    gen = g + 1;
    *s_flag = ok && (*(volatile int *)err == 0);
  }
  __syncthreads();
  return *s_flag != 0;
}

// Wait (one thread) until *p >= target; bounded like grid_sync.  Returns
// false when the wait gives up (DERR_BARRIER_TIMEOUT) or another CTA has
// reported an error.
__device__ bool wait_geq(const unsigned *p, unsigned target, int *err,
                         unsigned limit, bool backoff = false) {
  unsigned it = 0;
  while ((int)(ld_acquire(p) - target) < 0) {
    if (backoff)
      __nanosleep(64);
    if (++it > limit) {
      atomicOr(err, DERR_BARRIER_TIMEOUT);
      return false;
    }
    if ((it & 255u) == 0 && *(volatile int *)err)
      return false;
  }
  // the acquire load that saw the target orders this thread's later
  // reads (and, through the CTA barrier after it, the other threads')
  return *(volatile int *)err == 0;
}

__global__ void k_fill_u64(unsigned long long *p, int n, unsigned long long v) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
    p[i] = v;
}

// Wait (one warp) until flags[c] >= target for every c < n: each lane
// loads its flags together, then the warp votes, so a round of checks costs
// one memory round trip.  Bounded like grid_sync.
__device__ bool warp_wait_all(const unsigned *flags, int n, unsigned target,
                              int *err, unsigned limit) {
  const int lane = threadIdx.x & 31;
  unsigned it = 0;
  for (;;) {
    bool mine = true;
#pragma unroll 4
    for (int c = lane; c < n; c += 32)
      mine &= (int)(ld_acquire(flags + c) - target) >= 0;
    if (__all_sync(0xffffffffu, mine))
      break;
    int bad = 0;
    if (lane == 0) {
      if (++it > limit) {
        atomicOr(err, DERR_BARRIER_TIMEOUT);
        bad = 1;
      } else if ((it & 255u) == 0 && *(volatile int *)err) {
        bad = 1;
      }
    }
    if (__shfl_sync(0xffffffffu, bad, 0))
      return false;
  }
  return true;
}

__device__ __forceinline__ void st_release(unsigned *p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Apply a stored proposal to the atoms of molecule m.
// kind 0: shift (Coordinates::TranslateRand, src/Coordinates.cpp:83-100)
// kind 1: rotation about the molecule centre (RotateRand, :103-128)
__device__ __forceinline__ void apply_proposal(const DevBox &b, int kind,
                                               const double *prop, int na,
                                               const double (*oldp)[3],
                                               const double *com,
                                               double (*newp)[3],
                                               double *newcom) {
  if (kind == 0) {
    for (int a = 0; a < na; ++a)
      for (int d = 0; d < 3; ++d)
        newp[a][d] = wrap1(__dadd_rn(oldp[a][d], prop[d]), b.L[d]);
    for (int d = 0; d < 3; ++d)
      newcom[d] = wrap1(__dadd_rn(com[d], prop[d]), b.L[d]);
  } else {
    for (int a = 0; a < na; ++a) {
      double v[3];
      for (int d = 0; d < 3; ++d) {
        v[d] = unwrap1(oldp[a][d], com[d], b.L[d], b.half[d]);
        v[d] = __dadd_rn(v[d], -com[d]);
      }
      for (int i = 0; i < 3; ++i) {
        double w = __dadd_rn(__dadd_rn(__dmul_rn(prop[3 * i], v[0]),
                                       __dmul_rn(prop[3 * i + 1], v[1])),
                             __dmul_rn(prop[3 * i + 2], v[2]));
        newp[a][i] = wrap1(__dadd_rn(w, com[i]), b.L[i]);
      }
    }
    for (int d = 0; d < 3; ++d)
      newcom[d] = com[d];
  }
}

// exp(2 pi i phase / 2^64) in FP64 for a phase given as an exact 64-bit
// fraction of a turn: the reduction to |x| <= pi/4 is integer arithmetic,
// sin and cos of the remainder are their Taylor series to x^19 / x^20
// (truncation below 1e-19 there).
__device__ __forceinline__ double2 cis_turns64(uint64_t phase) {
  int64_t s = (int64_t)phase;                       // [-1/2, 1/2) turn
  int64_t q = (s + (1LL << 61)) >> 62;              // nearest quarter turn
  int64_t r = s - (int64_t)((uint64_t)q << 62);     // |r| <= 2^61
  double x = (double)r * 3.4061215800865545e-19;    // 2 pi / 2^64
  double x2 = x * x;
  double ps = -1.0 / 121645100408832000.0;          // -1/19!
  ps = fma(x2, ps, 1.0 / 355687428096000.0);        //  1/17!
  ps = fma(x2, ps, -1.0 / 1307674368000.0);         // -1/15!
  ps = fma(x2, ps, 1.0 / 6227020800.0);             //  1/13!
  ps = fma(x2, ps, -1.0 / 39916800.0);              // -1/11!
  ps = fma(x2, ps, 1.0 / 362880.0);                 //  1/9!
  ps = fma(x2, ps, -1.0 / 5040.0);                  // -1/7!
  ps = fma(x2, ps, 1.0 / 120.0);                    //  1/5!
  ps = fma(x2, ps, -1.0 / 6.0);                     // -1/3!
  double sn = fma(x * x2, ps, x);
  double pc = 1.0 / 2432902008176640000.0;          //  1/20!
  pc = fma(x2, pc, -1.0 / 6402373705728000.0);      // -1/18!
  pc = fma(x2, pc, 1.0 / 20922789888000.0);         //  1/16!
  pc = fma(x2, pc, -1.0 / 87178291200.0);           // -1/14!
  pc = fma(x2, pc, 1.0 / 479001600.0);              //  1/12!
  pc = fma(x2, pc, -1.0 / 3628800.0);               // -1/10!
  pc = fma(x2, pc, 1.0 / 40320.0);                  //  1/8!
  pc = fma(x2, pc, -1.0 / 720.0);                   // -1/6!
  pc = fma(x2, pc, 1.0 / 24.0);                     //  1/4!
  pc = fma(x2, pc, -0.5);
  double cs = fma(x2, pc, 1.0);
  switch ((int)(q & 3)) {
    case 0: return make_double2(cs, sn);
    case 1: return make_double2(-sn, cs);
    case 2: return make_double2(-cs, -sn);
    default: return make_double2(sn, -cs);
  }
}

// Neighbour nn of a cell (offsets dx, dy, dz in -1..1, dz fastest, each
// axis wrapped): the entry of the 27-neighbour table Box::Init builds
// (CellList::RebuildNeighbors order), computed instead of loaded.
__device__ __forceinline__ int nbr_cell(const int *e, int cell, int nn) {
  int z = cell % e[2], xy = cell / e[2];
  int y = xy % e[1], x = xy / e[1];
  x += nn / 9 - 1;
  y += (nn / 3) % 3 - 1;
  z += nn % 3 - 1;
  x += x < 0 ? e[0] : (x >= e[0] ? -e[0] : 0);
  y += y < 0 ? e[1] : (y >= e[1] ? -e[1] : 0);
  z += z < 0 ? e[2] : (z >= e[2] ? -e[2] : 0);
  return (x * e[1] + y) * e[2] + z;
}

__device__ __forceinline__ double2 cmul2(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 tab_at(const double2 *row, int n) {
  double2 v = row[n < 0 ? -n : n];
  // exp(-i x) = conj(exp(i x)): the sign bit of the imaginary part flipped
  // by an integer operation (the same value as a negation)
  v.y = __longlong_as_double(
      (long long)((unsigned long long)__double_as_longlong(v.y) ^
                  ((unsigned long long)(n < 0) << 63)));
  return v;
}

// ===========================================================================
// The FP64 chain kernel
// ===========================================================================
constexpr int CT = 256;
constexpr int HDR = 128;  // doubles in the move-context header
constexpr int ICL_MAX = 256;  // in-cutoff pairs a CTA lists per move
// Words of the chain's flag array: [0] the decision word, alone on its
// 128-byte line; from SEQ_CTX, one word per CTA: its part of a move's
// context written (grid <= PART_MAX_GRID).
constexpr int SEQ_CTX = 32;
// A CTA's partial slots hold this NaN pattern until written: the leader
// polls the values themselves (each 8-byte store is single-copy atomic), so
// no separate arrival flag, fence or atomic is needed
constexpr unsigned long long PART_EMPTY = 0x7FF4C0DE7FF4C0DEULL;
constexpr int PART_MAX_GRID = 256;  // partial slots the leader holds per lane: 8
constexpr int NPAIR_CAP = 64; // (n_x, n_y) columns a CTA's k-chunk may span
                              // for the shared x-y phase products

// CTAs of the chain grid without a k-chunk: the context writers 0 ..
// nrows_max - 1 when they are at most half the grid, else none; none when
// the writers are asked to hold k-vectors too (writer_k).
inline int chain_kless(int nrows_max, int grid, bool writer_k) {
  return !writer_k && nrows_max > 0 && 2 * nrows_max <= grid ? nrows_max : 0;
}

// doubles of one move context: the header and 2 MAX_MOL_ATOMS x 3 phase
// rows of kmax + 1 double2 entries
__host__ __device__ constexpr size_t chain_ctx_len(int stride) {
  return HDR + 2 * (size_t)(2 * MAX_MOL_ATOMS * 3) * stride;
}

// Context header layout (doubles):
//  0 m, 1 kind, 2 na, 3 pacc, 4..6 newcom, 8..15 cell old, 16..23 cell new,
//  24..47 old positions [8][3], 48..71 new positions [8][3], 72..79 charges,
//  80 log(pacc), 81 log(pacc) + 1e-9, 82 log(pacc) - 1e-9,
//  84..107 fixed-point turns of the positions as uint32 [side][atom][3]
struct ChainArgs {
  DevBox b;
  const FF *ff;
  Settings *set;
  const MoveRec *moves;
  double *prop;   // [n][12]
  int64_t first;
  int n;
  double *part;   // [2][grid][4], by move parity
  unsigned *bar;  // [0..1] grid barrier
  unsigned *seq;  // [0] decision published (2 (t + 1) + accept); from
                  // SEQ_CTX: per CTA, its part of the context of move t
                  // written (t)
  double *ctx;    // [nctx][ctx_len], by move modulo nctx: HDR + tables
  size_t ctx_len;
  int nctx;       // context buffers: 2 (one move in flight) or 3 (two)
  int nrows_max;  // phase rows of the largest molecule (6 x its atoms)
  int nkless;     // CTAs 0 .. nkless - 1 hold no k-vectors (context writers)
  // permutation of the atom index for the pipelined chain's atom ownership
  // (p = a * perm_m mod n_atoms, a = p * perm_minv mod n_atoms)
  unsigned long long perm_m, perm_minv;
  unsigned long long perm_r;  // floor((2^64 - 1) / n_atoms), for x mod n_atoms
  int *tr_i;      // [n][3] or null
  double *tr_d;   // [n][3] or null
  // phase clocks (NULL: not collected): [0 CTA 0, 1 the leader][phase:
  // context load, real-space listing, pair terms and k-vectors to the
  // partials, decision wait, commit and next context], then moves; then,
  // from the end of phase A, the leader's last partial, its last context
  // flag, and CTA 0's part of the next context written
  long long *prof;
  unsigned spin;  // polls after which a device wait gives up
};

struct ChainShared {
  Settings set;
  double e_run[5];
  double hdr[HDR];
  double red[CT / 32];
  double red3[3][CT / 32];
  int ovl_any;
  double tot[4];
  int accept, flag, ok, bok;
  unsigned gen, word;
  // the last decided move: its molecule, outcome and new positions and
  // centre (the leader writes them to global memory after it publishes)
  int last_m, last_acc;
  double last_newp[MAX_MOL_ATOMS][3], last_newcom[3];
  long long pclk[3];  // phase-clock marks of other warps (gb_mc_profile)
  // inputs and new positions of the context being built
  double b_oldp[MAX_MOL_ATOMS][3], b_newp[MAX_MOL_ATOMS][3];
  double b_com[3], b_newcom[3], b_prop[12], b_q[MAX_MOL_ATOMS];
  double b_pacc, b_lpacc;
  int b_m, b_a0, b_na, b_kind, b_writer, b_ka[MAX_MOL_ATOMS];
};

// Synchronise the threads [first, first + count) of the CTA: the whole CTA
// through __syncthreads, a group of whole warps through named barrier 1.
__device__ __forceinline__ void group_sync(int count) {
  if (count == (int)blockDim.x)
    __syncthreads();
  else
    asm volatile("bar.sync 1, %0;" ::"r"(count) : "memory");
}

// Is this CTA one of the writers of a move's context: CTA 0 (header) and
// one CTA per phase row.
__device__ __forceinline__ bool ctx_writer(const ChainArgs &A, int na) {
  int nrows = A.b.K > 0 ? 2 * na * 3 : 0;
  return blockIdx.x == 0 || (int)blockIdx.x < nrows;
}

// Second half of building move t's context from the inputs in S.b_*
// (threads tid = 0..count-1 of the CTA, count >= 128; the tasks sit on
// different warps so that they overlap): the proposal applied
// (Coordinates::TranslateRand / RotateRand arithmetic, see apply_proposal),
// the header (CTA 0) and this CTA's phase row.  Used where a context is
// built behind a grid barrier (the first move, and a move that follows one
// of the same molecule or a settings adjustment).
__device__ void build_ctx_rest(const ChainArgs &A, ChainShared &S, int t,
                               int tid, int count) {
  const DevBox &b = A.b;
  const int m = S.b_m, na = S.b_na, kind = S.b_kind;
  const int G = gridDim.x;
  const int stride = b.kmax + 1;
  const int nrows = b.K > 0 ? 2 * na * 3 : 0;
  const double *prop = S.b_prop;
  if (tid < na) {
    int a = tid;
    double v[3], w[3];
    if (kind == 0) {
      for (int d = 0; d < 3; ++d)
        w[d] = wrap1(__dadd_rn(S.b_oldp[a][d], prop[d]), b.L[d]);
    } else {
      for (int d = 0; d < 3; ++d) {
        v[d] = unwrap1(S.b_oldp[a][d], S.b_com[d], b.L[d], b.half[d]);
        v[d] = __dadd_rn(v[d], -S.b_com[d]);
      }
      for (int i = 0; i < 3; ++i) {
        double u = __dadd_rn(__dadd_rn(__dmul_rn(prop[3 * i], v[0]),
                                       __dmul_rn(prop[3 * i + 1], v[1])),
                             __dmul_rn(prop[3 * i + 2], v[2]));
        w[i] = wrap1(__dadd_rn(u, S.b_com[i]), b.L[i]);
      }
    }
    for (int d = 0; d < 3; ++d)
      S.b_newp[a][d] = w[d];
  } else if (tid >= 32 && tid < 35) {
    int d = tid - 32;
    S.b_newcom[d] = kind == 0 ? wrap1(__dadd_rn(S.b_com[d], prop[d]), b.L[d])
                              : S.b_com[d];
  }
  group_sync(count);
  double *const ctx = A.ctx + (size_t)(t % A.nctx) * A.ctx_len;
  if (blockIdx.x == 0) {
    double *h = ctx;
    if (tid == 64) {
      h[0] = m;
      h[1] = kind;
      h[2] = na;
      h[3] = S.b_pacc;
      h[80] = S.b_lpacc;
      h[81] = S.b_lpacc + 1e-9;  // the decision's margins, precomputed
      h[82] = S.b_lpacc - 1e-9;
      for (int d = 0; d < 3; ++d)
        h[4 + d] = S.b_newcom[d];
    } else if (tid >= 96 && tid < 96 + 2 * na) {
      int i = tid - 96, a = i % na, side = i / na;
      const double *p = side ? S.b_newp[a] : S.b_oldp[a];
      h[(side ? 16 : 8) + a] = position_to_cell_fast(b, p[0], p[1], p[2]);
      for (int d = 0; d < 3; ++d)
        h[(side ? 48 : 24) + 3 * a + d] = p[d];
      if (side == 0) {
        double q = S.b_q[a];
        h[72 + a] = fabs(q) < 0.000000001 ? 0.0 : q;
        h[108 + a] = q;  // the charge and kind of the real-space terms
        ((int *)(h + 116))[a] = S.b_ka[a];
      }
    } else if (tid >= 128 && tid < 128 + 6 * na) {
      int i = tid - 128, pa = i / 3, d = i % 3;  // pa = side * na + atom
      const double *p = pa < na ? S.b_oldp[pa] : S.b_newp[pa - na];
      ((uint32_t *)(h + 84))[i] = to_turns(p[d], b.invL[d]);
    }
  }
  // phase rows exp(i n 2 pi r_d / L_d), n = 0..kmax, one entry per thread:
  // the coordinate as a 64-bit fraction of the box edge, n times it exact
  // modulo one turn; in CTA 0 on the threads the header leaves free
  double2 *tab = (double2 *)(ctx + HDR);
  const int rfirst = blockIdx.x == 0 ? 160 : 0;
  if (tid >= rfirst) {
    for (int rr = blockIdx.x; rr < nrows; rr += G) {
      int p = rr / 3, d = rr % 3;
      double coord = p < na ? S.b_oldp[p][d] : S.b_newp[p - na][d];
      double tt = coord * b.invL[d];
      if (tt >= 1.0)
        tt -= 1.0;
      uint64_t u = __double2ull_rn(tt * 18446744073709551616.0);  // 2^64
      for (int n = tid - rfirst; n < stride; n += count - rfirst)
        tab[(size_t)rr * stride + n] = cis_turns64((uint64_t)n * u);
    }
  }
}

// Move t's context from the inputs in S.b_* by one warp, then this CTA's
// flag for the leader: the same tasks as build_ctx_rest, in sequence.
__device__ void build_ctx_warp(const ChainArgs &A, ChainShared &S, int t) {
  const DevBox &b = A.b;
  const int lane = threadIdx.x & 31;
  const int m = S.b_m, na = S.b_na, kind = S.b_kind;
  const int G = gridDim.x;
  const int stride = b.kmax + 1;
  const int nrows = b.K > 0 ? 2 * na * 3 : 0;
  const double *prop = S.b_prop;
  if (lane < na) {
    const int a = lane;
    double v[3], w[3];
    if (kind == 0) {
      for (int d = 0; d < 3; ++d)
        w[d] = wrap1(__dadd_rn(S.b_oldp[a][d], prop[d]), b.L[d]);
    } else {
      for (int d = 0; d < 3; ++d) {
        v[d] = unwrap1(S.b_oldp[a][d], S.b_com[d], b.L[d], b.half[d]);
        v[d] = __dadd_rn(v[d], -S.b_com[d]);
      }
      for (int i = 0; i < 3; ++i) {
        double u = __dadd_rn(__dadd_rn(__dmul_rn(prop[3 * i], v[0]),
                                       __dmul_rn(prop[3 * i + 1], v[1])),
                             __dmul_rn(prop[3 * i + 2], v[2]));
        w[i] = wrap1(__dadd_rn(u, S.b_com[i]), b.L[i]);
      }
    }
    for (int d = 0; d < 3; ++d)
      S.b_newp[a][d] = w[d];
  } else if (lane >= 8 && lane < 11) {
    const int d = lane - 8;
    S.b_newcom[d] = kind == 0 ? wrap1(__dadd_rn(S.b_com[d], prop[d]), b.L[d])
                              : S.b_com[d];
  }
  __syncwarp();
  double *const ctx = A.ctx + (size_t)(t % A.nctx) * A.ctx_len;
  if (blockIdx.x == 0) {
    double *h = ctx;
    if (lane == 0) {
      h[0] = m;
      h[1] = kind;
      h[2] = na;
      h[3] = S.b_pacc;
      h[80] = S.b_lpacc;
      h[81] = S.b_lpacc + 1e-9;  // the decision's margins, precomputed
      h[82] = S.b_lpacc - 1e-9;
      for (int d = 0; d < 3; ++d)
        h[4 + d] = S.b_newcom[d];
    }
    if (lane >= 16 && lane < 16 + 2 * na) {
      const int i = lane - 16, a = i % na, side = i / na;
      const double *p = side ? S.b_newp[a] : S.b_oldp[a];
      h[(side ? 16 : 8) + a] = position_to_cell_fast(b, p[0], p[1], p[2]);
      for (int d = 0; d < 3; ++d)
        h[(side ? 48 : 24) + 3 * a + d] = p[d];
      if (side == 0) {
        double q = S.b_q[a];
        h[72 + a] = fabs(q) < 0.000000001 ? 0.0 : q;
        h[108 + a] = q;  // the charge and kind of the real-space terms
        ((int *)(h + 116))[a] = S.b_ka[a];
      }
    }
    for (int i = lane; i < 6 * na; i += 32) {
      const int pa = i / 3, d = i % 3;  // pa = side * na + atom
      const double *p = pa < na ? S.b_oldp[pa] : S.b_newp[pa - na];
      ((uint32_t *)(h + 84))[i] = to_turns(p[d], b.invL[d]);
    }
  }
  // phase rows exp(i n 2 pi r_d / L_d), n = 0..kmax (as build_ctx_rest)
  double2 *tab = (double2 *)(ctx + HDR);
  for (int rr = blockIdx.x; rr < nrows; rr += G) {
    const int p = rr / 3, d = rr % 3;
    const double coord = p < na ? S.b_oldp[p][d] : S.b_newp[p - na][d];
    double tt = coord * b.invL[d];
    if (tt >= 1.0)
      tt -= 1.0;
    const uint64_t u = __double2ull_rn(tt * 18446744073709551616.0);  // 2^64
    for (int n = lane; n < stride; n += 32)
      tab[(size_t)rr * stride + n] = cis_turns64((uint64_t)n * u);
  }
  __syncwarp();
  if (lane == 0)  // a release store: it orders the warp's writes before it
    st_release(A.seq + SEQ_CTX + blockIdx.x, (unsigned)t);
}

// Build move t's context with threads [first, first + count) of the CTA,
// count >= 192 (all of them after a decision; prev_hdr / prev_acc: the
// previous move's header and outcome, whose new positions are the current
// ones when the same molecule moves again).
__device__ void build_ctx(const ChainArgs &A, ChainShared &S, int t,
                          const double *prev_hdr, int prev_acc, int first,
                          int count) {
  const int tid = (int)threadIdx.x - first;
  const DevBox &b = A.b;
  const MoveRec &r = A.moves[t];
  int m = r.mol;
  int a0 = b.mstart[m], na = b.mstart[m + 1] - a0;
  if (!ctx_writer(A, na))
    return;
  bool same = prev_acc && prev_hdr && (int)prev_hdr[0] == m;
  if (tid == 0) {
    S.b_m = m;
    S.b_a0 = a0;
    S.b_na = na;
    S.b_kind = r.kind;
    S.b_pacc = r.pacc;
    S.b_lpacc = r.lpacc;
  }
  for (int i = tid; i < 12; i += count)
    S.b_prop[i] = A.prop[(size_t)t * 12 + i];
  for (int d = tid; d < 3; d += count) {
    double *cs[3] = {b.cx, b.cy, b.cz};
    S.b_com[d] = (same && (int)prev_hdr[1] == 0) ? prev_hdr[4 + d]
                                                 : __ldcg(cs[d] + m);
  }
  for (int i = tid; i < 3 * na; i += count) {
    int a = i / 3, d = i % 3;
    double *xs[3] = {b.x, b.y, b.z};
    S.b_oldp[a][d] = same ? prev_hdr[48 + 3 * a + d] : __ldcg(xs[d] + a0 + a);
  }
  for (int a = tid; a < na; a += count) {
    S.b_q[a] = b.q[a0 + a];
    S.b_ka[a] = b.kind[a0 + a];
  }
  group_sync(count);
  build_ctx_rest(A, S, t, tid, count);
}

// Inputs of move t's context gathered by one warp in registers, in two
// steps so that each load has a stretch of other work to arrive in: step 1
// the move record and the molecule's atom range, step 2 the proposal
// (lanes 0..11), the centre (12..14), the old coordinates (lanes < 3 na)
// and the charges (lanes < na).
struct CtxPre {
  int m, a0, na, kind, ka;
  double pacc, lpacc;
  double v0, v1, q;
  bool writer;
};
// The static inputs of a move's context, gathered two moves ahead in two
// steps so that no load is waited for: the move record first, a move later
// the molecule's atom range (whose address needs the record's molecule).
__device__ __forceinline__ void ctx_pre_record(const ChainArgs &A, int t,
                                               CtxPre &c) {
  c.m = -1;
  if (t < A.n) {
    const MoveRec &r = A.moves[t];
    c.m = r.mol;
    c.kind = r.kind;
    c.pacc = r.pacc;
    c.lpacc = r.lpacc;
  }
}
__device__ __forceinline__ void ctx_pre_range(const ChainArgs &A, CtxPre &c,
                                              int &a1) {
  c.a0 = a1 = 0;
  if (c.m >= 0) {
    c.a0 = A.b.mstart[c.m];
    a1 = A.b.mstart[c.m + 1];
  }
}
__device__ __forceinline__ void ctx_pre2(const ChainArgs &A,
                                         const ChainShared &S, int t,
                                         CtxPre &c) {
  const DevBox &b = A.b;
  const int lane = threadIdx.x & 31;
  c.writer = ctx_writer(A, c.na);
  c.v0 = c.v1 = c.q = 0.0;
  c.ka = 0;
  if (!c.writer)
    return;
  // the molecule of the move decided last has its new positions here (the
  // leader writes them to global memory only after it publishes)
  const bool last = c.m == S.last_m && S.last_acc;
  if (lane < 12)
    c.v0 = A.prop[(size_t)t * 12 + lane];
  else if (lane < 15)
    c.v0 = last ? S.last_newcom[lane - 12]
                : __ldcg((lane == 12 ? b.cx : lane == 13 ? b.cy : b.cz) + c.m);
  if (lane < 3 * c.na) {
    int a = lane / 3, d = lane % 3;
    c.v1 = last ? S.last_newp[a][d]
                : __ldcg((d == 0 ? b.x : d == 1 ? b.y : b.z) + c.a0 + a);
  }
  if (lane < c.na) {
    c.q = b.q[c.a0 + lane];
    c.ka = b.kind[c.a0 + lane];
  }
}
// Stage the gathered inputs in shared memory (by the loading warp).
__device__ __forceinline__ void ctx_pre_store(ChainShared &S, const CtxPre &c) {
  const int lane = threadIdx.x & 31;
  if (lane == 0) {
    S.b_m = c.m;
    S.b_a0 = c.a0;
    S.b_na = c.na;
    S.b_kind = c.kind;
    S.b_pacc = c.pacc;
    S.b_lpacc = c.lpacc;
  }
  if (lane < 12)
    S.b_prop[lane] = c.v0;
  else if (lane < 15)
    S.b_com[lane - 12] = c.v0;
  if (lane < 3 * c.na)
    S.b_oldp[lane / 3][lane % 3] = c.v1;
  if (lane < c.na) {
    S.b_q[lane] = c.q;
    S.b_ka[lane] = c.ka;
  }
}


// FP64 term of one candidate pair of the chain: unit u (atom, old/new side,
// neighbour cell) against cell slot s: the exact minimum-image distance and
// cutoff test, the overlap flag for new positions, and the LJ and
// erfc-screened Coulomb terms, old positions subtracted.
// The neighbour's position and charge (p: x, y, z, q) and meta word come
// from the caller's loads; the moved atom's from the move header.
__device__ __forceinline__ void pair_term(const ChainArgs &A,
                                          const ChainShared &S, int u,
                                          double2 pxy, double2 pzq, int mj,
                                          double &lj, double &re,
                                          double &ovl) {
  const DevBox &b = A.b;
  const FF &ff = *A.ff;
  int a = u / (2 * NB27), side = (u / NB27) % 2;
  const double *pp = S.hdr + (side ? 48 : 24) + 3 * a;
  double dx = min_image(pp[0] - pxy.x, b.L[0], b.half[0]);
  double dy = min_image(pp[1] - pxy.y, b.L[1], b.half[1]);
  double dz = min_image(pp[2] - pzq.x, b.L[2], b.half[2]);
  double d2 = dsq3(dx, dy, dz);
  if (!(ff.rcutSq > d2))
    return;
  if (side && d2 < ff.rcutLowSq)
    ovl = 1.0;
  double qa = S.hdr[108 + a];
  int ka = ((const int *)(S.hdr + 116))[a];
  double e = 0.0;
  if (ff.electrostatic) {
    double qq = qa * pzq.y * QQ_FACT;
    if (qq != 0.0)
      e = coulomb_energy(ff, d2, qq);
  }
  double l = lj_energy(ff, d2, ka + meta_kind(mj) * ff.n_kinds);
  if (side) {
    re += e;
    lj += l;
  } else {
    re += -e;
    lj += -l;
  }
}

// The (n_x, n_y) columns a k-chunk spans (its k-vectors run x outer, y, z
// inner): pair_n[c] the columns in order and pidx[i] the column of
// k-vector i; returns their number, or -1 when there are more than
// NPAIR_CAP (the products are then formed per k-vector).  One thread.
__device__ inline int chunk_columns(const char4 *kn, int kc, char2 *pair_n,
                                    unsigned short *pidx) {
  int np = 0;
  for (int i = 0; i < kc; ++i) {
    char4 n = kn[i];
    if (np == 0 || pair_n[np - 1].x != n.x || pair_n[np - 1].y != n.y) {
      if (np == NPAIR_CAP)
        return -1;
      pair_n[np++] = make_char2(n.x, n.y);
    }
    pidx[i] = (unsigned short)(np - 1);
  }
  return np;
}

// The charge-weighted x-y products of a move for each column of the chunk
// and each old / new atom position, entries e = e0, e0 + step, ... of
// npair x 2 na (exy[column * 2 na + side * na + atom]).
__device__ __forceinline__ void xy_products(int e0, int step, int npair,
                                            const char2 *pair_n,
                                            const double2 *tab, int stride,
                                            int na, const double *q,
                                            double2 *exy) {
  for (int e = e0; e < npair * 2 * na; e += step) {
    int p = e / (2 * na), r = e - p * 2 * na;
    const double2 *rx = tab + (size_t)(r * 3) * stride;
    double qa = q[r < na ? r : r - na];
    double2 v = cmul2(rx[pair_n[p].x], tab_at(rx + stride, pair_n[p].y));
    exy[e] = make_double2(qa * v.x, qa * v.y);
  }
}

// The change of the structure factor at k-vector n from a move context:
// the sum over the moved atoms of q (e^{i k.r_new} - e^{i k.r_old}), four
// FMAs per atom and side.  col: the move's charge-weighted x-y products of
// this k-vector's (n_x, n_y) column (old atoms, then new), or NULL to form
// them from the phase rows `tab` (stride entries per row, rows atom-major
// old then new, x, y, z); q: the charges (hdr + 72).  A zero charge gives
// exact zeros (the products carry the charge), so it is not tested.
__device__ __forceinline__ void kvec_delta(char4 n, const double2 *col,
                                           const double2 *tab, int stride,
                                           int na, const double *q,
                                           double &dR, double &dI) {
  dR = 0.0;
  dI = 0.0;
  for (int a = 0; a < na; ++a) {
    const double2 *ro = tab + (size_t)(a * 3) * stride;
    const double2 *rn = tab + (size_t)((na + a) * 3) * stride;
    double2 xo, xn;
    if (col) {
      xo = col[a];
      xn = col[na + a];
    } else {
      double2 vo = cmul2(ro[n.x], tab_at(ro + stride, n.y));
      double2 vn = cmul2(rn[n.x], tab_at(rn + stride, n.y));
      xo = make_double2(q[a] * vo.x, q[a] * vo.y);
      xn = make_double2(q[a] * vn.x, q[a] * vn.y);
    }
    double2 zo = tab_at(ro + 2 * stride, n.z);
    double2 zn = tab_at(rn + 2 * stride, n.z);
    dR = fma(xn.x, zn.x, dR);
    dR = fma(-xn.y, zn.y, dR);
    dR = fma(-xo.x, zo.x, dR);
    dR = fma(xo.y, zo.y, dR);
    dI = fma(xn.x, zn.y, dI);
    dI = fma(xn.y, zn.x, dI);
    dI = fma(-xo.x, zo.y, dI);
    dI = fma(-xo.y, zo.x, dI);
  }
}

__global__ void __launch_bounds__(CT, 1) k_chain_fp64(ChainArgs A) {
  extern __shared__ double dyn[];
  __shared__ ChainShared S;
  const DevBox &b = A.b;
  const FF &ff = *A.ff;
  int G = gridDim.x, cta = blockIdx.x;
  // The context writers (CTAs below nrows_max) build the next move's
  // context during phase A; they take no k-vectors, so that its FP64 chain
  // does not queue behind the k-vector warps' (the others' chunks grow by a
  // few lanes of the same warp passes).
  const int nkb = A.nkless;
  const int kG = G - nkb;
  int kc_max = (b.K + kG - 1) / kG;
  int kbeg = cta < nkb ? b.K : min(b.K, (cta - nkb) * kc_max);
  int kc = cta < nkb ? 0 : min(kc_max, b.K - kbeg);
  const bool kless = cta < nkb;
  const int pw = kless ? 0 : 3;  // the warp that evaluates the pair terms
  double *sR = dyn, *sI = sR + kc_max, *nR = sI + kc_max, *nI = nR + kc_max,
         *pf = nI + kc_max;
  char4 *kn = (char4 *)(pf + kc_max);
  int stride = b.kmax + 1;
  double2 *tab = (double2 *)(dyn + ((5 * kc_max + (kc_max + 1) / 2 + 1) & ~1));
  // The k-chunk lists k-vectors x outer, y, z inner, so it spans a few
  // (n_x, n_y) columns; per move the products exp(i n_x t_x) exp(i n_y t_y)
  // are formed once per column and atom, and each k-vector multiplies in
  // its exp(i n_z t_z) -- the same products, in the same order, as forming
  // all three per k-vector.
  double2 *exy = tab + (size_t)(2 * MAX_MOL_ATOMS * 3) * (b.kmax + 1);
  unsigned short *pidx = (unsigned short *)(exy + NPAIR_CAP * 2 * MAX_MOL_ATOMS);
  // this CTA's own atoms, resident for the whole launch: atoms cta,
  // cta + G, cta + 2G, ... (strided, so that the atoms near any molecule,
  // and with them the pair terms of its moves, spread over all CTAs);
  // x, y | z, q | fixed-point turns and the meta word
  const int own_per = (b.n_atoms + G - 1) / G;
  const int on = cta < b.n_atoms ? (b.n_atoms - cta + G - 1) / G : 0;
  double2 *oxy = (double2 *)(((uintptr_t)(pidx + kc_max) + 15) & ~(uintptr_t)15);
  double2 *ozq = oxy + own_per;
  uint4 *ot = (uint4 *)(ozq + own_per);
  __shared__ char2 pair_n[NPAIR_CAP];
  __shared__ int npair;
  for (int i = threadIdx.x; i < kc; i += CT) {
    int k = kbeg + i;
    sR[i] = b.sumRref[k];
    sI[i] = b.sumIref[k];
    pf[i] = b.prefact[k];
    kn[i] = b.kn[k];
  }
  for (int i = threadIdx.x; i < on; i += CT) {
    const int a = cta + G * i;
    const double x = b.x[a], y = b.y[a], z = b.z[a];
    oxy[i] = make_double2(x, y);
    ozq[i] = make_double2(z, b.q[a]);
    ot[i] = make_uint4(to_turns(x, b.invL[0]), to_turns(y, b.invL[1]),
                       to_turns(z, b.invL[2]),
                       (unsigned)pack_meta(b.mol[a], b.kind[a]));
  }
  if (threadIdx.x == 0) {
    S.pclk[0] = S.pclk[1] = S.pclk[2] = 0;
    S.last_m = -1;
    S.last_acc = 0;
    S.set = *A.set;
    for (int i = 0; i < 5; ++i)
      S.e_run[i] = b.energy[i];
    S.gen = ld_acquire(&A.bar[1]);
  }
  __syncthreads();
  if (threadIdx.x == 0)
    npair = chunk_columns(kn, kc, pair_n, pidx);
  __syncthreads();

  const int total_threads = G * CT;
  const int gtid = cta * CT + threadIdx.x;
  // FP32 candidate pre-test: turn lengths and a cutoff padded by 1e-4 of
  // Rcut^2 (FP32 and fixed-point rounding stay below 1e-6 of it)
  const float turn_f[3] = {(float)(b.L[0] * 2.3283064365386963e-10),
                           (float)(b.L[1] * 2.3283064365386963e-10),
                           (float)(b.L[2] * 2.3283064365386963e-10)};
  const float cut_f = (float)(ff.rcutSq * 1.0001);
  // proposals from move t to the next adjustment boundary
  auto make_props = [&](int t0) {
    int t1 = t0;
    while (t1 < A.n) {
      long long step = A.first + t1;
      if (t1 > t0 && (step + 1) % S.set.adj == 0)
        break;
      ++t1;
    }
    for (int t = t0 + gtid; t < t1; t += total_threads)
      make_proposal(A.moves[t], S.set, A.prop + (size_t)t * 12);
  };

  // prologue
  if (threadIdx.x == 0)
    settings_adjust(S.set, A.first);
  __syncthreads();
  make_props(0);
  if (!grid_sync(A.bar, G, S.gen, b.err, &S.flag, A.spin))
    return;
  build_ctx(A, S, 0, nullptr, 0, 0, CT);
  if (!grid_sync(A.bar, G, S.gen, b.err, &S.flag, A.spin))
    return;

  const int pslot = cta == 0 ? 0 : cta == G - 1 ? 1 : -1;
  const bool prof = A.prof && threadIdx.x == 0 && pslot >= 0;
  long long pacc[5] = {0, 0, 0, 0, 0}, poff[3] = {0, 0, 0}, tb = 0;
  long long tclk = prof ? clock64() : 0;
  auto mark = [&](int ph) {
    if (prof) {
      long long now = clock64();
      pacc[ph] += now - tclk;
      tclk = now;
    }
  };
  // the molecule of the move after the current one, loaded a move ahead;
  // warps 7 (context inputs) and 4 (the leader's count of context writers)
  // carry the next moves' records and atom ranges through a two-stage
  // pipeline: at move t the record of move t + 3 is requested, the atom
  // range of move t + 2, and move t + 1's are complete
  int nmol = A.n > 1 ? A.moves[1].mol : -1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool piper = warp == 7 || warp == 4;
  CtxPre pipe_a, pipe_b;  // record of t + 2 (a), record and range of t + 1 (b)
  int pipe_b1 = 0;
  pipe_a.writer = pipe_b.writer = false;
  pipe_a.m = pipe_b.m = -1;
  if (piper) {
    ctx_pre_record(A, 1, pipe_b);
    ctx_pre_range(A, pipe_b, pipe_b1);
    ctx_pre_record(A, 2, pipe_a);
  }
  for (int t = 0; t < A.n; ++t) {
    const int mol_next = nmol;
    nmol = t + 2 < A.n ? A.moves[t + 2].mol : -1;
    CtxPre pre = pipe_b;
    pre.na = pipe_b1 - pipe_b.a0;
    if (piper) {
      pipe_b = pipe_a;
      ctx_pre_range(A, pipe_b, pipe_b1);
      ctx_pre_record(A, t + 3, pipe_a);
    }
    // ---------------- phase A ----------------
    // the header and the rows of the largest molecule in one round trip
    const double *ctx_t = A.ctx + (size_t)(t % A.nctx) * A.ctx_len;
    for (int i = threadIdx.x; i < HDR; i += CT)
      S.hdr[i] = __ldcg(ctx_t + i);
    for (int i = threadIdx.x; i < A.nrows_max * stride; i += CT)
      tab[i] = __ldcg((const double2 *)(ctx_t + HDR) + i);
    __syncthreads();
    mark(0);
    int m = (int)S.hdr[0];
    int na = (int)S.hdr[2];
    // The next move's context does not depend on this move's outcome unless
    // the next move touches the same molecule or follows a settings
    // adjustment; then it is built after the decision, behind a grid
    // barrier.  Otherwise warp 7 of each context writer gathers its inputs
    // during this phase (the loads overlap it) and the writer builds it
    // right after its partials are out.
    const bool spec = t + 1 < A.n && mol_next != m &&
                      (A.first + t + 2) % S.set.adj != 0;
    pre.writer = false;
    const bool wload = spec && warp == 7;
    // the next context's writers, counted by the leader's warp 4 from the
    // next move's atom count its pipeline holds
    const int nbuild = max(1, min(G, b.K > 0 ? 2 * pre.na * 3 : 0));
    double lj = 0.0, re = 0.0, ovl = 0.0, er = 0.0;
    // first atom of the moved molecule, for the commit to the own atoms
    const int a0m = __ldg(b.mstart + m);
    // x-y column products times the atom's charge, one per (column,
    // old/new atom)
    xy_products(threadIdx.x, CT, npair, pair_n, tab, stride, na, S.hdr + 72,
                exy);
    if (wload)
      ctx_pre2(A, S, t + 1, pre);
    // (1) Real space: this CTA's own atoms against the old and new
    //     positions of the moved atoms.  An FP32 pre-test on the
    //     fixed-point turns (the wrapped integer difference is the minimum
    //     image; the exact FP64 test is made where the listed pairs are
    //     evaluated), and the pairs inside it compacted, in (own atom,
    //     position) order, into a shared list (a warp scan and a scan over
    //     the warps, so the order and every sum stay fixed).  Every pair
    //     within the cutoff is found, as the 27 neighbour cells of the
    //     cell list find it, and the moved molecule's own atoms are left out
    //     as CellList::RemoveMol leaves them out.
    __shared__ double2 icl_pos[ICL_MAX][2];  // neighbour x, y | z, q
    __shared__ int icl_meta[ICL_MAX];
    __shared__ short icl_unit[ICL_MAX];
    __shared__ int icl_warp[CT / 32 + 1];
    const int npos = 2 * na;
    const uint32_t *pturn = (const uint32_t *)(S.hdr + 84);
    int icl_n = 0;
    for (int base = 0; base < on; base += CT) {
      const int i = base + threadIdx.x;
      unsigned hit = 0;  // bit p: position p = side * na + atom passed
      uint4 f = make_uint4(0, 0, 0, 0);
      if (i < on) {
        f = ot[i];
        if (meta_mol((int)f.w) != m) {
          for (int pp = 0; pp < npos; ++pp) {
            float dx = (float)(int)(pturn[3 * pp] - f.x) * turn_f[0];
            float dy = (float)(int)(pturn[3 * pp + 1] - f.y) * turn_f[1];
            float dz = (float)(int)(pturn[3 * pp + 2] - f.z) * turn_f[2];
            if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) < cut_f)
              hit |= 1u << pp;
          }
        }
      }
      const int cnt = __popc(hit);
      int incl = cnt;
      for (int o = 1; o < 32; o <<= 1) {
        int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o)
          incl += v;
      }
      if (lane == 31)
        icl_warp[warp] = incl;
      __syncthreads();
      if (threadIdx.x == 0) {
        int run = icl_n;
        for (int w = 0; w < CT / 32; ++w) {
          int c = icl_warp[w];
          icl_warp[w] = run;
          run += c;
        }
        icl_warp[CT / 32] = run;
      }
      __syncthreads();
      if (hit) {
        const double2 pxy = oxy[i], pzq = ozq[i];
        int pos = icl_warp[warp] + incl - cnt;
        for (unsigned h = hit; h; h &= h - 1) {
          const int pp = __ffs(h) - 1;
          const int side = pp >= na ? 1 : 0, a = pp - side * na;
          const int u = (a * 2 + side) * NB27;
          if (pos < ICL_MAX) {
            icl_pos[pos][0] = pxy;
            icl_pos[pos][1] = pzq;
            icl_meta[pos] = (int)f.w;
            icl_unit[pos] = (short)u;
          } else {
            // past the list (not met at liquid densities): evaluated here
            pair_term(A, S, u, pxy, pzq, (int)f.w, lj, re, ovl);
          }
          ++pos;
        }
      }
      icl_n = icl_warp[CT / 32];
      __syncthreads();
    }
    __syncthreads();  // the x-y products (a CTA may own no atoms)
    mark(1);
    // (2) Warp 3 evaluates the listed pairs (the FP64-heavy LJ and
    //     erfc-screened Coulomb terms) while warps 0, 1, 2, 4, 5, 6 take the
    //     k-vectors: with warps issued to the SM's four sub-partitions by
    //     warp index modulo 4, the pair terms run beside the k-vectors
    //     instead of after them.  In a context writer without k-vectors
    //     warp 0 takes the pairs and warps 1..7 build the next context.
    const int n_eval = min(icl_n, ICL_MAX);
    if (warp == pw) {
      for (int i = lane; i < n_eval; i += 32)
        pair_term(A, S, icl_unit[i], icl_pos[i][0], icl_pos[i][1],
                  icl_meta[i], lj, re, ovl);
    }
    if (kless) {
      // A context writer without k-vectors: warps 1..7 build its part of
      // the next move's context now, from the inputs warp 7 gathered at the
      // start of this phase, so that the context is complete by the time
      // the other CTAs' partials are in.
      if (spec && warp >= 1) {
        if (warp == 7) {
          if (pre.writer)
            ctx_pre_store(S, pre);
          if (lane == 0)
            S.b_writer = pre.writer;
        }
        group_sync(CT - 32);
        if (S.b_writer) {
          build_ctx_rest(A, S, t + 1, (int)threadIdx.x - 32, CT - 32);
          group_sync(CT - 32);
          if (threadIdx.x == 32) {
            // a release store: it orders the writes of the warps that met
            // at the barrier before it
            st_release(A.seq + SEQ_CTX + blockIdx.x, (unsigned)(t + 1));
            if (A.prof)
              S.pclk[2] = clock64();
          }
        }
      }
    } else if (wload && pre.writer) {
      // warp 7 of a context writer with k-vectors (a grid too small for
      // k-less writers) builds its part beside the k-vector warps
      ctx_pre_store(S, pre);
      __syncwarp();
      build_ctx_warp(A, S, t + 1);
      if (A.prof && lane == 0)
        S.pclk[2] = clock64();
    }
    if (!kless && warp != 3 && warp != 7) {
      const int kw = warp < 3 ? warp : warp - 1;  // 0..5
      for (int i = kw * 32 + lane; i < kc; i += 6 * 32) {
        double dR, dI;
        kvec_delta(kn[i], npair > 0 ? exy + (size_t)pidx[i] * 2 * na : nullptr,
                   tab, stride, na, S.hdr + 72, dR, dI);
        double srn = sR[i] + dR;
        double sin_ = sI[i] + dI;
        nR[i] = srn;
        nI[i] = sin_;
        er += (srn * srn + sin_ * sin_) * pf[i];
      }
    }
    // CTA partials in a fixed order: the pair terms are warp 3's (all
    // warps' when the list overflowed and other threads evaluated pairs),
    // the reciprocal energy is the k-vector warps'; only those warps reduce
    // (warp shuffles, then lanes 0..2 of warp 0 add over the warps); the
    // overlap flag by vote
    {
      const bool all_pairs = icl_n > ICL_MAX;
      double v0 = lj, v1 = re, v2 = er;
      if (warp == pw || all_pairs) {
        for (int o = 16; o > 0; o >>= 1) {
          v0 += __shfl_down_sync(0xffffffffu, v0, o);
          v1 += __shfl_down_sync(0xffffffffu, v1, o);
        }
      }
      if (!kless && warp != 3 && warp != 7) {
        for (int o = 16; o > 0; o >>= 1)
          v2 += __shfl_down_sync(0xffffffffu, v2, o);
      }
      int any = __syncthreads_or(ovl > 0.0);
      if (lane == 0) {
        S.red3[0][warp] = v0;
        S.red3[1][warp] = v1;
        S.red3[2][warp] = v2;
      }
      __syncthreads();
      double *part_t = A.part + (size_t)(t & 1) * G * 4;
      if (threadIdx.x < 3) {
        double r = 0.0;
        if (threadIdx.x < 2 && !all_pairs) {
          r = S.red3[threadIdx.x][pw];
        } else if (threadIdx.x < 2 || !kless) {
          for (int w = 0; w < CT / 32; ++w)
            if (threadIdx.x < 2 || (w != 3 && w != 7))
              r += S.red3[threadIdx.x][w];
        }
        __stcg(part_t + (size_t)cta * 4 + threadIdx.x, r);
        if (threadIdx.x == 0)
          __stcg(part_t + (size_t)cta * 4 + 3, any ? 1.0 : 0.0);
      }
    }
    mark(2);
    tb = tclk;  // phase B starts
    // ---------------- phase B ----------------
    // The last CTA (the leader) waits for every CTA's partials, reduces them
    // in a fixed order, decides, commits an accepted move (coordinates,
    // centre, cell slots) and publishes the decision; the other CTAs wait
    // for that one word.  Meanwhile warps 1..7 of the context-building CTAs
    // build the next move's context (into the other parity buffer): it does
    // not depend on this decision unless the next move touches the same
    // molecule or follows a settings adjustment (then it is built after the
    // decision, behind a grid barrier, as in the prologue).  The leader
    // publishes only after those builds are counted in, so one published
    // word orders the decision, the commit and the next context before
    // every CTA's next phase A.
    const bool leader = cta == G - 1;
    if ((int)threadIdx.x >= 128) {
      if (leader && warp == 4) {
        // the writers' flags of the next context, polled from the start of
        // phase B beside the partials; warp 0 reads the outcome at barrier
        // 3 before it publishes
        int bok = spec ? warp_wait_all(A.seq + SEQ_CTX, nbuild,
                                       (unsigned)(t + 1), b.err, A.spin)
                       : 1;
        if (lane == 0) {
          S.bok = bok;
          if (A.prof)
            S.pclk[1] = clock64();
        }
        asm volatile("bar.sync 3, 64;" ::: "memory");
      }
    } else if (leader) {
      // Warps 0..3 of the leader each gather one quantity over all CTAs
      // (LJ, real space, reciprocal energy, overlap), polling the values
      // until every CTA's is present, so the FP64 additions run on four
      // SM sub-partitions at once.  Lane l adds CTAs l, l + 32, ... in
      // order, then the warp tree: a fixed order.
      const int q = warp;
      double *part_t = A.part + (size_t)(t & 1) * G * 4;
      constexpr int PF = PART_MAX_GRID / 32;
      // three polls in flight, staggered, so that a check comes about
      // every third of a memory round trip
      constexpr int NPOLL = 3;
      double pp[NPOLL][PF];
      auto issue = [&](double *dst) {
#pragma unroll
        for (int i = 0; i < PF; ++i) {
          int c = lane + 32 * i;
          dst[i] = c < G ? __ldcg(part_t + (size_t)c * 4 + q) : 0.0;
        }
      };
      auto present = [&](const double *src) {
        bool mine = true;
#pragma unroll
        for (int i = 0; i < PF; ++i)
          mine &= __double_as_longlong(src[i]) != (long long)PART_EMPTY;
        return __all_sync(0xffffffffu, mine);
      };
#pragma unroll
      for (int j = 0; j < NPOLL; ++j) {
        if (j)
          __nanosleep(150);
        issue(pp[j]);
      }
      int ok = 1, got = -1;
      unsigned it = 0;
      for (;;) {
#pragma unroll
        for (int j = 0; j < NPOLL; ++j) {
          if (got < 0) {
            if (present(pp[j]))
              got = j;  // warp-uniform
            else
              issue(pp[j]);
          }
        }
        if (got >= 0)
          break;
        int bad = 0;
        if (lane == 0) {
          if (++it > A.spin) {
            atomicOr(b.err, DERR_BARRIER_TIMEOUT);
            bad = 1;
          } else if ((it & 255u) == 0 && *(volatile int *)b.err) {
            bad = 1;
          }
        }
        if (__shfl_sync(0xffffffffu, bad, 0)) {
          ok = 0;
          break;
        }
      }
      if (A.prof && lane == 0 && q == 0)
        S.pclk[0] = clock64();
      double pv[PF];
#pragma unroll
      for (int i = 0; i < PF; ++i)
        pv[i] = got == 0 ? pp[0][i] : got == 1 ? pp[1][i] : pp[2][i];
      // read: this quantity's slots are marked empty for move t + 2 after
      // the decision word is out (before the next word, which every writer
      // of move t + 2 waits for)
      auto reset_slots = [&]() {
#pragma unroll
        for (int i = 0; i < PF; ++i) {
          int c = lane + 32 * i;
          if (c < G)
            __stcg(part_t + (size_t)c * 4 + q, __longlong_as_double(PART_EMPTY));
        }
      };
      if (ok) {
        if (q < 3) {
          double v = 0.0;
#pragma unroll
          for (int i = 0; i < PF; ++i)
            v += pv[i];
          for (int o = 16; o > 0; o >>= 1)
            v += __shfl_down_sync(0xffffffffu, v, o);
          if (lane == 0)
            S.tot[q] = v;
        } else {
          bool any = false;
#pragma unroll
          for (int i = 0; i < PF; ++i)
            any |= __double_as_longlong(pv[i]) != 0;
          any = __any_sync(0xffffffffu, any);
          if (lane == 0)
            S.tot[3] = any ? 1.0 : 0.0;
        }
      }
      if (lane == 0)
        S.red3[0][q] = ok;  // per-warp status
      asm volatile("bar.sync 2, 128;" ::: "memory");
      ok = S.red3[0][0] != 0.0 && S.red3[0][1] != 0.0 && S.red3[0][2] != 0.0 &&
           S.red3[0][3] != 0.0;
      if (warp != 0 && ok)
        reset_slots();  // not ordered before warp 0's release below
      int acc = 0;
      if (warp == 0 && ok) {
        double dLJ = 0.0, dRe = 0.0, dRc = 0.0;
        if (lane == 0) {
          bool over = S.tot[3] > 0;
          dLJ = S.tot[0];
          dRe = S.tot[1];
          dRc = (!over && b.K > 0) ? S.tot[2] - S.e_run[2] : 0.0;
          double ex = __dmul_rn(-ff.beta, __dadd_rn(__dadd_rn(dLJ, dRe), dRc));
          // pacc < exp(ex), decided on logarithms unless the two sides are
          // within 1e-9 (or pacc is 0): the outcome of the exp comparison
          // without its FP64 exp on the critical path
          int res;
          if (S.hdr[3] > 0.0 && ex > S.hdr[81])
            res = 1;
          else if (S.hdr[3] > 0.0 && ex < S.hdr[82])
            res = 0;
          else
            res = S.hdr[3] < exp(ex);
          acc = res && !over;
        }
        acc = __shfl_sync(0xffffffffu, acc, 0);
        // the next context must be complete before the word goes out
        asm volatile("bar.sync 3, 64;" ::: "memory");
        ok = S.bok != 0;
        // release: it orders the next context (through warp 4's acquire
        // and barrier 3); no store of this move precedes it, so it does
        // not wait for one
        if (lane == 0 && ok)
          st_release(A.seq, 2u * (unsigned)(t + 1) + (unsigned)acc);
        if (ok)
          reset_slots();
        if (acc) {
          // the new coordinates and centre, after the word: the next
          // context reads them from the last move's copy in shared memory,
          // later ones after the next word (the cell grid is rebuilt from
          // the coordinates after the launch)
          if (lane < na) {
            const double *np = S.hdr + 48 + 3 * lane;
            b.x[a0m + lane] = np[0];
            b.y[a0m + lane] = np[1];
            b.z[a0m + lane] = np[2];
          }
          if (lane == 0 && (int)S.hdr[1] == 0) {
            b.cx[m] = S.hdr[4];
            b.cy[m] = S.hdr[5];
            b.cz[m] = S.hdr[6];
          }
          __syncwarp();
        }
        if (lane == 0) {
          // off the critical path: running energies and the trace
          if (acc) {
            S.e_run[0] += dLJ;
            S.e_run[1] += dRe;
            S.e_run[2] += dRc;
          }
          if (A.tr_i) {
            A.tr_i[3 * (size_t)t] = (int)S.hdr[1];
            A.tr_i[3 * (size_t)t + 1] = m;
            A.tr_i[3 * (size_t)t + 2] = acc;
            A.tr_d[3 * (size_t)t] = dLJ;
            A.tr_d[3 * (size_t)t + 1] = dRe;
            A.tr_d[3 * (size_t)t + 2] = dRc;
          }
          S.accept = acc;
          S.ok = ok;
        }
      } else if (warp == 0) {
        asm volatile("bar.sync 3, 64;" ::: "memory");  // warp 4 is there
        if (lane == 0) {
          S.accept = 0;
          S.ok = 0;
        }
      }
    } else {
      if (threadIdx.x == 0) {
        int ok = wait_geq(A.seq, 2u * (unsigned)(t + 1), b.err, A.spin);
        S.accept = ok ? (int)(ld_acquire(A.seq) & 1u) : 0;
        S.ok = ok;
      }
    }
    __syncthreads();
    if (!S.ok)
      return;
    mark(3);
    if (prof) {
      // when, after this CTA's phase A, the leader had every partial and
      // every context flag, and this CTA (a context writer) had written
      // its part of the next context
      for (int k = 0; k < 3; ++k)
        if (S.pclk[k])
          poff[k] += S.pclk[k] - tb;
      S.pclk[0] = S.pclk[1] = S.pclk[2] = 0;
    }
    const int acc = S.accept;
    if (threadIdx.x == 0) {
      settings_update(S.set, (int)S.hdr[1], acc);
      S.last_m = m;
      S.last_acc = acc;
    }
    if (acc) {
      for (int i = threadIdx.x; i < kc; i += CT) {
        sR[i] = nR[i];
        sI[i] = nI[i];
      }
      for (int i = threadIdx.x; i < 3 * na + 3; i += CT) {
        if (i < 3 * na)
          S.last_newp[i / 3][i % 3] = S.hdr[48 + i];
        else
          S.last_newcom[i - 3 * na] = S.hdr[4 + i - 3 * na];
      }
      // the moved atoms this CTA owns take their new positions
      for (int a = threadIdx.x; a < na; a += CT) {
        const int ga = a0m + a, i = ga / G;
        if (ga - i * G == cta) {
          const double *np = S.hdr + 48 + 3 * a;
          const uint32_t *pt = (const uint32_t *)(S.hdr + 84) + (na + a) * 3;
          oxy[i] = make_double2(np[0], np[1]);
          ozq[i].x = np[2];
          ot[i] = make_uint4(pt[0], pt[1], pt[2], ot[i].w);
        }
      }
      __syncthreads();  // before the next context overwrites the header
    }
    if (t + 1 < A.n) {
      long long step = A.first + t + 1;
      if ((step + 1) % S.set.adj == 0) {
        __syncthreads();
        if (threadIdx.x == 0)
          settings_adjust(S.set, step);
        __syncthreads();
        make_props(t + 1);
        if (!grid_sync(A.bar, G, S.gen, b.err, &S.flag, A.spin))
          return;
      }
      if (!spec) {
        build_ctx(A, S, t + 1, S.hdr, acc, 0, CT);
        if (!grid_sync(A.bar, G, S.gen, b.err, &S.flag, A.spin))
          return;
      }
    }
    mark(4);
  }
  if (prof) {
    for (int ph = 0; ph < 5; ++ph)
      A.prof[5 * pslot + ph] += pacc[ph];
    A.prof[10 + pslot] += A.n;
    if (pslot == 1) {
      A.prof[12] += poff[0];
      A.prof[13] += poff[1];
    } else {
      A.prof[14] += poff[2];
    }
  }
  // write back this CTA's structure factors; the leader the settings and
  // the running energies
  for (int i = threadIdx.x; i < kc; i += CT) {
    b.sumRref[kbeg + i] = sR[i];
    b.sumIref[kbeg + i] = sI[i];
  }
  if (cta == G - 1 && threadIdx.x == 0) {
    *A.set = S.set;
    for (int i = 0; i < 5; ++i)
      b.energy[i] = S.e_run[i];
  }
}

#include "gb_chain_pipe.cuh"

// ===========================================================================
// MultiParticle kernels (src/moves/MultiParticle.h)
// ===========================================================================
__device__ __forceinline__ void philox4x64(uint64_t c0, uint64_t c1,
                                           uint64_t c2, uint64_t c3,
                                           uint64_t k0, uint64_t k1,
                                           uint64_t *o) {
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k0 += 0x9E3779B97F4A7C15ULL;
      k1 += 0xBB67AE8584CAA73BULL;
    }
    uint64_t lo0 = 0xD2E7470EE14C6C93ULL * c0;
    uint64_t hi0 = __umul64hi(0xD2E7470EE14C6C93ULL, c0);
    uint64_t lo1 = 0xCA5A826395121157ULL * c2;
    uint64_t hi1 = __umul64hi(0xCA5A826395121157ULL, c2);
    uint64_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  o[0] = c0;
  o[1] = c1;
  o[2] = c2;
  o[3] = c3;
}
// r123::u01<double> and uneg11<double> of a 64-bit word
__device__ __forceinline__ double u01_64(uint64_t v) {
  const double f = 1.0 / 18446744073709551616.0;
  return __dadd_rn(__dmul_rn(__ull2double_rn(v), f), 0.5 * f);
}
__device__ __forceinline__ double uneg11_64(uint64_t v) {
  const double f = 1.0 / 9223372036854775808.0;
  return __dadd_rn(__dmul_rn(__ll2double_rn((long long)v), f), 0.5 * f);
}

struct MpArgs {
  DevBox b;
  Settings *set;
  int type;        // 0 displacement, 1 rotation
  uint64_t step, seed;
  double beta;
  const double *mF, *mR, *tq;  // reference forces / torque
  double *xn, *yn, *zn, *cxn, *cyn, *czn, *tk;
  int *inrange;
  int *fail;
};

// CalculateTrialDistRot + Translate/RotateForceBiased/Random
// (src/moves/MultiParticle.h:546-714), one thread per molecule.
__global__ void k_mp_transform(MpArgs P) {
  const DevBox &b = P.b;
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= b.n_mol)
    return;
  const Settings &s = *P.set;
  const double lambda = 0.5;
  double lb[3];
  for (int d = 0; d < 3; ++d) {
    double v = P.type == 1 ? P.tq[3 * (size_t)m + d]
                           : __dadd_rn(P.mF[3 * (size_t)m + d],
                                       P.mR[3 * (size_t)m + d]);
    lb[d] = __dmul_rn(__dmul_rn(v, lambda), P.beta);
  }
  double mx = P.type == 1 ? s.mp_r_max : s.mp_t_max;
  double lbmax[3];
  bool fir = true;
  for (int d = 0; d < 3; ++d) {
    lbmax[d] = __dmul_rn(lb[d], mx);
    double a = fabs(lbmax[d]);
    fir = fir && a > 1E-12 && a < 30;
  }
  uint64_t r[4];
  philox4x64((uint64_t)m, 0, 0, 0, P.step, P.seed, r);
  double val[3] = {0.0, 0.0, 0.0};
  if (fir)
    for (int d = 0; d < 3; ++d)
      val[d] = log(__dadd_rn(exp(-1.0 * lbmax[d]),
                             __dmul_rn(__dmul_rn(2.0, u01_64(r[d])),
                                       sinh(lbmax[d])))) /
               lb[d];
  P.inrange[m] = fir;
  for (int d = 0; d < 3; ++d)
    P.tk[3 * (size_t)m + d] = val[d];
  // MultiParticle::Transform checks (src/moves/MultiParticle.h:366-409)
  double len = sqrt(val[0] * val[0] + val[1] * val[1] + val[2] * val[2]);
  if (!isfinite(len) ||
      (P.type == 0 && (val[0] > b.half[0] || val[1] > b.half[1] ||
                       val[2] > b.half[2])))
    atomicOr(P.fail, 1);
  int a0 = b.mstart[m], na = b.mstart[m + 1] - a0;
  double com[3] = {b.cx[m], b.cy[m], b.cz[m]};
  if (P.type == 1) {
    double rm[9];
    if (fir) {
      double rotLen = sqrt(val[0] * val[0] + val[1] * val[1] + val[2] * val[2]);
      double inv = 1.0 / rotLen;
      double ax[3] = {val[0] * inv, val[1] * inv, val[2] * inv};
      axis_angle_matrix(rotLen, ax, rm);
    } else {
      double symRand = __dmul_rn(s.mp_r_max, uneg11_64(r[0]));
      double u = uneg11_64(r[1]);
      double theta = __dmul_rn(2.0 * M_PI, u01_64(r[2]));
      double rootTerm = sqrt(__dadd_rn(1.0, -__dmul_rn(u, u)));
      double ax[3] = {rootTerm * cos(theta), rootTerm * sin(theta), u};
      axis_angle_matrix(symRand, ax, rm);
    }
    for (int p = 0; p < na; ++p) {
      int a = a0 + p;
      double v[3] = {b.x[a], b.y[a], b.z[a]};
      for (int d = 0; d < 3; ++d) {
        v[d] = unwrap1(v[d], com[d], b.L[d], b.half[d]);
        v[d] = __dadd_rn(v[d], -com[d]);
      }
      double w[3];
      for (int i = 0; i < 3; ++i)
        w[i] = __dadd_rn(__dadd_rn(__dmul_rn(rm[3 * i], v[0]),
                                   __dmul_rn(rm[3 * i + 1], v[1])),
                         __dmul_rn(rm[3 * i + 2], v[2]));
      P.xn[a] = wrap1(__dadd_rn(w[0], com[0]), b.L[0]);
      P.yn[a] = wrap1(__dadd_rn(w[1], com[1]), b.L[1]);
      P.zn[a] = wrap1(__dadd_rn(w[2], com[2]), b.L[2]);
    }
    P.cxn[m] = com[0];
    P.cyn[m] = com[1];
    P.czn[m] = com[2];
  } else {
    double sh[3];
    for (int d = 0; d < 3; ++d)
      sh[d] = fir ? val[d] : __dmul_rn(s.mp_t_max, uneg11_64(r[d]));
    for (int p = 0; p < na; ++p) {
      int a = a0 + p;
      P.xn[a] = wrap1(__dadd_rn(b.x[a], sh[0]), b.L[0]);
      P.yn[a] = wrap1(__dadd_rn(b.y[a], sh[1]), b.L[1]);
      P.zn[a] = wrap1(__dadd_rn(b.z[a], sh[2]), b.L[2]);
    }
    P.cxn[m] = wrap1(__dadd_rn(com[0], sh[0]), b.L[0]);
    P.cyn[m] = wrap1(__dadd_rn(com[1], sh[1]), b.L[1]);
    P.czn[m] = wrap1(__dadd_rn(com[2], sh[2]), b.L[2]);
  }
}

struct MpAcceptArgs {
  DevBox b;
  Settings *set;
  int type;
  uint64_t step, seed;
  double beta;
  const double *mF, *mR, *tq, *mFn, *mRn, *tqn, *tk;
  const int *inrange, *fail;
  const double *newE;  // [0] recip, [1] inter, [2] real
  double *out;         // [0] accept flag
  int *tr_i;
  double *tr_d;
};

// MultiParticle::GetCoeff + Accept (src/moves/MultiParticle.h:447-544)
__global__ void k_mp_accept(MpAcceptArgs P) {
  const DevBox &b = P.b;
  Settings &s = *P.set;
  const double lBeta = 0.5 * P.beta;
  double mx = P.type == 1 ? s.mp_r_max : s.mp_t_max;
  double w = 1.0;
  for (int m = threadIdx.x; m < b.n_mol; m += blockDim.x) {
    if (!P.inrange[m])
      continue;
    double wr = 1.0;
    for (int d = 0; d < 3; ++d) {
      size_t i = 3 * (size_t)m + d;
      double lo, ln;
      if (P.type == 1) {
        lo = P.tq[i] * lBeta;
        ln = P.tqn[i] * lBeta;
      } else {
        lo = (P.mF[i] + P.mR[i]) * lBeta;
        ln = (P.mFn[i] + P.mRn[i]) * lBeta;
      }
      double k = P.tk[i];
      wr *= ln * exp(-ln * k) / (2.0 * sinh(ln * mx));
      wr /= lo * exp(lo * k) / (2.0 * sinh(lo * mx));
    }
    w *= wr;
  }
  __shared__ double sh[1024];
  sh[threadIdx.x] = w;
  __syncthreads();
  if (threadIdx.x == 0) {
    double W = 1.0;
    for (int i = 0; i < (int)blockDim.x; ++i)
      W *= sh[i];
    if (!isfinite(W))
      W = 0.0;
    double *e = b.energy;
    double newRecip = P.newE[0], newInter = P.newE[1], newReal = P.newE[2];
    double totNew = 0.0 + 0.0 + newInter + 0.0 + newReal + newRecip + e[3] + e[4];
    double totOld = 0.0 + 0.0 + e[0] + 0.0 + e[1] + e[2] + e[3] + e[4];
    double uBoltz = exp(-P.beta * (totNew - totOld));
    double accept = W * uBoltz;
    uint64_t r[4];
    philox4x64((uint64_t)b.n_mol, 0, 0, 0, P.step, P.seed, r);
    double pr = u01_64(r[0]);
    int result = (*P.fail == 0) && pr < accept;
    if (result) {
      e[0] = newInter;
      e[1] = newReal;
      e[2] = newRecip;
    }
    s.mp_itries[P.type]++;
    if (result)
      s.mp_iacc[P.type]++;
    settings_update(s, 2, result);
    P.out[0] = result;
    if (P.tr_i) {
      P.tr_i[0] = 2;
      P.tr_i[1] = P.type;
      P.tr_i[2] = result;
      P.tr_d[0] = newInter;
      P.tr_d[1] = newReal;
      P.tr_d[2] = newRecip;
    }
  }
}

// Commit the trial state when accepted (the swaps of MultiParticle::Accept).
struct MpCommitArgs {
  DevBox b, bn;
  const double *flag;
  int K;
  double *aF, *mF, *aR, *mR, *tq;
  const double *aFn, *mFn, *aRn, *mRn, *tqn;
};
__global__ void k_mp_commit(MpCommitArgs P) {
  if (P.flag[0] == 0.0)
    return;
  const DevBox &b = P.b, &n = P.bn;
  size_t tid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = tid; i < (size_t)b.n_atoms; i += stride) {
    b.x[i] = n.x[i];
    b.y[i] = n.y[i];
    b.z[i] = n.z[i];
    b.atom_cell[i] = n.atom_cell[i];
    b.atom_slot[i] = n.atom_slot[i];
    for (int d = 0; d < 3; ++d) {
      P.aF[3 * i + d] = P.aFn[3 * i + d];
      P.aR[3 * i + d] = P.aRn[3 * i + d];
    }
  }
  for (size_t i = tid; i < (size_t)b.n_mol; i += stride) {
    b.cx[i] = n.cx[i];
    b.cy[i] = n.cy[i];
    b.cz[i] = n.cz[i];
    for (int d = 0; d < 3; ++d) {
      P.mF[3 * i + d] = P.mFn[3 * i + d];
      P.mR[3 * i + d] = P.mRn[3 * i + d];
      P.tq[3 * i + d] = P.tqn[3 * i + d];
    }
  }
  for (size_t i = tid; i < (size_t)P.K; i += stride) {
    b.sumRref[i] = b.sumRnew[i];
    b.sumIref[i] = b.sumInew[i];
  }
  size_t nc = (size_t)b.ncell * b.cap;
  for (size_t i = tid; i < nc; i += stride) {
    b.cell_atom[i] = n.cell_atom[i];
    b.cell_pos[i] = n.cell_pos[i];
    b.cell_meta[i] = n.cell_meta[i];
    b.cell_fix[i] = n.cell_fix[i];
    b.cell_qlo[i] = n.cell_qlo[i];
  }
  for (size_t i = tid; i < (size_t)b.ncell; i += stride)
    b.cell_count[i] = n.cell_count[i];
}

__global__ void k_settings_adjust(Settings *s, long long step) {
  settings_adjust(*s, step);
}
__global__ void k_set_energy2(double *energy, const double *v) {
  energy[0] = v[0];
  energy[1] = v[1];
}

// ===========================================================================
// Host orchestration
// ===========================================================================
template <class T>
static int mc_alloc(Box &b, McState &s, T **p, size_t n) {
  void *q = nullptr;
  cudaError_t e = cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T));
  if (e != cudaSuccess)
    return b.CudaCheck(e, "cudaMalloc (Monte Carlo state)");
  s.allocs.push_back(q);
  s.bytes += std::max<size_t>(n, 1) * sizeof(T);
  *p = (T *)q;
  return OK;
}

static void harvest(McState &s);

void mc_destroy(Box &b) {
  if (!b.mc)
    return;
  McState &s = *b.mc;
  if (b.stream)
    cudaStreamSynchronize(b.stream);
  harvest(s);
  for (void *p : s.allocs)
    cudaFree(p);
  if (s.h_moves)
    cudaFreeHost(s.h_moves);
  if (s.h_desc)
    cudaFreeHost(s.h_desc);
  delete s.stream;
  delete s.ahead_from;
  delete b.mc;
  b.mc = nullptr;
}

// A multiplier near 0.618 n coprime with n and its inverse modulo n: the
// permutation a -> a m mod n spreads runs of nearby indices over the range
// (multiplicative hashing with the golden ratio).
static void chain_perm(int n, unsigned long long *m, unsigned long long *minv) {
  if (n <= 2) {
    *m = *minv = 1;
    return;
  }
  long long c = (long long)(0.6180339887498949 * n);
  auto gcd = [](long long x, long long y) {
    while (y) {
      long long r = x % y;
      x = y;
      y = r;
    }
    return x;
  };
  while (gcd(c, n) != 1)
    ++c;
  // extended Euclid: c * u = 1 mod n
  long long r0 = n, r1 = c % n, u0 = 0, u1 = 1;
  while (r1) {
    long long q = r0 / r1, t = r0 - q * r1;
    r0 = r1;
    r1 = t;
    t = u0 - q * u1;
    u0 = u1;
    u1 = t;
  }
  if (u0 < 0)
    u0 += n;
  *m = (unsigned long long)(c % n);
  *minv = (unsigned long long)u0;
}

static size_t chain_smem(const Box &b, int grid, int nrows_max,
                         bool writer_k, bool pipe) {
  // the pipelined chain spreads atoms and k-vectors over all CTAs but the
  // deciding one, and holds four k-chunk buffers instead of two
  const int work = pipe ? grid - 1 : grid;
  const int kG = work - chain_kless(nrows_max, work, writer_k);
  int kc_max = (b.dev.K + kG - 1) / kG;
  // (the pipelined chain's atoms are owned by the CTAs with a k-chunk)
  const int owners = pipe ? kG : grid;
  size_t own_per = ((size_t)b.dev.n_atoms + owners - 1) / owners;
  const size_t kvec =
      pipe ? chain_pipe_kvec_doubles(kc_max)
           : ((5 * (size_t)kc_max + (kc_max + 1) / 2 + 1) & ~(size_t)1);
  return sizeof(double) * kvec +
         (pipe ? 2 : 1) * sizeof(double2) * (size_t)(2 * MAX_MOL_ATOMS * 3) *
             (b.dev.kmax + 1) +
         sizeof(double2) * (size_t)NPAIR_CAP * 2 * MAX_MOL_ATOMS +
         sizeof(unsigned short) * (size_t)kc_max + 64 +
         own_per * (2 * sizeof(double2) + sizeof(uint4)) +
         // (the pipelined chain's copy of the erfc(alpha r)/r segments)
         (pipe && b.ff.erfc_tab ? sizeof(double) * (size_t)b.ff.etab_nseg *
                                      (ETAB_DEG + 1)
                                : 0);
}

int mc_init(Box &b, const gb_mc_params &p) {
  mc_destroy(b);
  if (p.adj_steps <= 0)
    return b.Fail(ERR_ARG, "AdjSteps must be positive");
  if (!(p.frac[0] >= 0 && p.frac[1] >= 0 && p.frac[2] >= 0) ||
      p.frac[0] + p.frac[1] + p.frac[2] <= 0)
    return b.Fail(ERR_ARG, "move frequencies must be non-negative, not all 0");
  const HostSystem &h = b.host;
  std::vector<int> len(h.n_mol);
  int na_max = 1;
  for (int m = 0; m < h.n_mol; ++m) {
    len[m] = h.mstart[m + 1] - h.mstart[m];
    na_max = std::max(na_max, len[m]);
    if (len[m] > MAX_MOL_ATOMS)
      return b.Fail(ERR_UNSUPPORTED, "molecules above 8 atoms in the move loop");
  }
  b.mc = new McState();
  McState &s = *b.mc;
  s.params = p;
  s.na_max = na_max;
  s.stream = new MoveStream(p.seed, p.frac, h.n_mol, len);
  s.next_step = 0;
  int rc;
  if ((rc = mc_alloc(b, s, &s.d_set, 1)))
    return rc;
  Settings st{};
  // MoveSettings::Init reads the box axis before BoxDimensions::Init sets it
  // (src/System.cpp:72-81), so a fresh start has displacement scale 0.
  st.scale[0] = 0.0;
  st.scale[1] = M_PI_4;
  st.mp_r_max = 0.01 * M_PI;
  st.mp_t_max = 0.02;
  if (p.use_scales) {
    st.scale[0] = p.scales[0];
    st.scale[1] = p.scales[1];
    st.mp_t_max = p.scales[2];
    st.mp_r_max = p.scales[3];
  }
  st.singleMoveAccepted = 1;
  st.adj = p.adj_steps;
  st.amin = std::min(h.L[0], std::min(h.L[1], h.L[2]));
  if ((rc = b.CudaCheck(cudaMemcpyAsync(s.d_set, &st, sizeof(Settings),
                                        cudaMemcpyHostToDevice, b.stream),
                        "upload")))
    return rc;
  // chain-kernel geometry: at most one CTA per SM (cooperative residency
  // checked), one CTA per SM unless asked for fewer; one CTA at least per
  // phase row of the largest molecule (each writes one row of a context)
  if (p.writer_kchunk != 0 && p.writer_kchunk != 1)
    return b.Fail(ERR_ARG, "writer_kchunk must be 0 or 1");
  if (p.moves_in_flight < 0 || p.moves_in_flight > 2)
    return b.Fail(ERR_ARG, "moves_in_flight must be 0, 1 or 2");
  // two moves in flight unless asked for one or the grid leaves no CTA to
  // decide (the writers' rows and the deciding CTA need nrows + 1 CTAs)
  s.pipe = p.moves_in_flight == 2 ||
           (p.moves_in_flight == 0 &&
            (p.grid_ctas ? p.grid_ctas : b.sm_count) >=
                std::max(3, (b.dev.K > 0 ? 6 * na_max : 0) + 1));
  if (p.grid_ctas < 0 || p.grid_ctas > b.sm_count)
    return b.Fail(ERR_ARG, "grid_ctas must be 0 or 2 .. the SM count");
  s.grid = p.grid_ctas ? p.grid_ctas : b.sm_count;
  const int nrows_max = b.dev.K > 0 ? 6 * na_max : 0;
  // (and, with two moves in flight, one more CTA that only decides)
  if (s.grid < 3 || s.grid < nrows_max + (s.pipe ? 1 : 0))
    return b.Fail(ERR_ARG,
                  "the chain grid needs 3 CTAs and one per phase row of the "
                  "largest molecule (6 x its atoms), plus the deciding CTA "
                  "with two moves in flight");
  int per_sm = 0;
  const void *kfn = s.pipe ? (const void *)k_chain_fp64_pipe
                           : (const void *)k_chain_fp64;
  size_t sm = chain_smem(b, s.grid, nrows_max, p.writer_kchunk != 0, s.pipe);
  raise_smem_limit(kfn, sm);
  if ((rc = b.CudaCheck(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                            &per_sm, kfn, CT, sm),
                        "occupancy")))
    return rc;
  if (per_sm < 1)
    return b.Fail(ERR_UNSUPPORTED, "chain kernel does not fit on an SM");
  if (s.grid > PART_MAX_GRID)
    return b.Fail(ERR_UNSUPPORTED, "the chain needs 2 to 256 SMs");
  if (p.move_buffer < 0)
    return b.Fail(ERR_ARG, "move_buffer must be >= 0");
  s.move_cap = p.move_buffer > 0 ? (size_t)p.move_buffer : (size_t)1 << 16;
  int stride = b.dev.kmax + 1;
  if ((rc = mc_alloc(b, s, &s.d_moves, s.move_cap)) ||
      (rc = mc_alloc(b, s, &s.d_prop, s.move_cap * 12)) ||
      (rc = mc_alloc(b, s, &s.d_part, 3 * (size_t)s.grid * 8)) ||
      (rc = mc_alloc(b, s, &s.d_bar, 8)) ||
      (rc = mc_alloc(b, s, &s.d_seq, SEQ_CTX + PART_MAX_GRID)) ||
      (rc = mc_alloc(b, s, &s.d_ctx, 3 * chain_ctx_len(stride))) ||
      (rc = mc_alloc(b, s, &s.d_mp, 16)))
    return rc;
  if ((rc = b.CudaCheck(cudaMallocHost(&s.h_moves, s.move_cap * sizeof(MoveRec)),
                        "pinned")))
    return rc;
  if ((rc = b.CudaCheck(cudaMemsetAsync(s.d_bar, 0, 32, b.stream), "memset")))
    return rc;
  // a new loop starts without the error of an earlier one (a wait that gave
  // up left the box's state as it was before that call)
  if ((rc = b.CudaCheck(cudaMemsetAsync(b.dev.err, 0, 16, b.stream), "memset")))
    return rc;
  if (b.cfg.precision == GB_MIXED) {
    // FP32 pair terms assume the 12-6 form
    for (int i = 0; i < b.ff.n_kinds * b.ff.n_kinds; ++i)
      if (b.ff.eps_cn[i] != 0.0 && b.ff.nexp[i] != 12.0)
        return b.Fail(ERR_UNSUPPORTED, "mixed form supports Mie n = 12 only");
    int want = p.cluster_size;
    if (want != 0 && want != 2 && want != 4 && want != 8 && want != 16)
      return b.Fail(ERR_ARG, "cluster_size must be 0, 2, 4, 8 or 16");
    // Largest cluster first (shortest move latency); per cluster size the
    // k-chunk arrays all in shared memory if they fit, else the cold half of
    // them in a global buffer.
    int cands[4] = {16, 8, 4, 2};
    s.cluster = 0;
    bool cold_global = false;
    for (int c : cands) {
      if (want && c != want)
        continue;
      for (int cold_smem = 1; cold_smem >= 0 && !s.cluster; --cold_smem) {
        size_t sm = mixed_smem(b.dev.K, b.dev.kmax, c, cold_smem != 0);
        if (sm > MIXED_SMEM_MAX || max_active_clusters(c, sm) < 1)
          continue;
        s.cluster = c;
        s.mixed_smem = sm;
        cold_global = !cold_smem;
      }
      if (s.cluster)
        break;
    }
    if (!s.cluster)
      return b.Fail(ERR_UNSUPPORTED, "no cluster shape fits this box");
    if (cold_global &&
        (rc = mc_alloc(b, s, &s.d_cold, mixed_cold_buffer(b.dev.K, s.cluster))))
      return rc;
    // threads per real-space unit: as asked, else the smallest of 32, 64,
    // 128 that covers a cell's mean occupancy in one pass, 128 above that
    // (timed on SPC/E water at Rcut 9-10 A: 64 lanes at 56 atoms per cell,
    // 128 at 94 and 111; 256 was slower at each)
    int lanes = p.unit_lanes;
    if (lanes == 0) {
      const double cells = (double)b.dev.edge[0] * b.dev.edge[1] * b.dev.edge[2];
      const double occ = cells > 0 ? b.dev.n_atoms / cells : 0.0;
      lanes = occ <= 32 ? 32 : occ <= 64 ? 64 : 128;
    }
    if (lanes != 32 && lanes != 64 && lanes != 128 && lanes != 256)
      return b.Fail(ERR_ARG, "unit_lanes must be 0, 32, 64, 128 or 256");
    s.ulog = lanes == 32 ? 5 : lanes == 64 ? 6 : lanes == 128 ? 7 : 8;
    s.desc_cap = 256;
    if ((rc = mc_alloc(b, s, &s.d_desc, s.desc_cap)))
      return rc;
    if ((rc = b.CudaCheck(cudaMallocHost(&s.h_desc,
                                         s.desc_cap * sizeof(MixedChain)),
                          "pinned")))
      return rc;
  }
  // MultiParticle trial-state buffers
  int N = b.dev.n_atoms, M = b.dev.n_mol;
  if ((rc = mc_alloc(b, s, &s.d_xn, N)) || (rc = mc_alloc(b, s, &s.d_yn, N)) ||
      (rc = mc_alloc(b, s, &s.d_zn, N)) || (rc = mc_alloc(b, s, &s.d_cxn, M)) ||
      (rc = mc_alloc(b, s, &s.d_cyn, M)) || (rc = mc_alloc(b, s, &s.d_czn, M)) ||
      (rc = mc_alloc(b, s, &s.d_aFn, 3 * (size_t)N)) ||
      (rc = mc_alloc(b, s, &s.d_mFn, 3 * (size_t)M)) ||
      (rc = mc_alloc(b, s, &s.d_aRn, 3 * (size_t)N)) ||
      (rc = mc_alloc(b, s, &s.d_mRn, 3 * (size_t)M)) ||
      (rc = mc_alloc(b, s, &s.d_tqn, 3 * (size_t)M)) ||
      (rc = mc_alloc(b, s, &s.d_tk, 3 * (size_t)M)) ||
      (rc = mc_alloc(b, s, &s.d_inrange, M)))
    return rc;
  DevBox &n = s.cells_new;
  n = b.dev;
  n.x = s.d_xn;
  n.y = s.d_yn;
  n.z = s.d_zn;
  n.cx = s.d_cxn;
  n.cy = s.d_cyn;
  n.cz = s.d_czn;
  size_t NC = (size_t)b.dev.ncell * b.dev.cap;
  if ((rc = mc_alloc(b, s, &n.cell_count, b.dev.ncell)) ||
      (rc = mc_alloc(b, s, &n.cell_atom, NC)) ||
      (rc = mc_alloc(b, s, &n.cell_pos, NC)) ||
      (rc = mc_alloc(b, s, &n.cell_meta, NC)) ||
      (rc = mc_alloc(b, s, &n.cell_fix, NC)) ||
      (rc = mc_alloc(b, s, &n.cell_qlo, NC)) ||
      (rc = mc_alloc(b, s, &n.atom_cell, N)) ||
      (rc = mc_alloc(b, s, &n.atom_slot, N)))
    return rc;
  return b.Sync();
}

// Draw moves up to `step` without running them (restart at a later step).
void draw_next(McState &s, MoveRec *r) {
  if (s.ahead_pos < s.ahead.size()) {
    *r = s.ahead[s.ahead_pos++];
    if (s.ahead_pos == s.ahead.size()) {
      s.ahead.clear();
      s.ahead_pos = 0;
    }
    return;
  }
  s.stream->Next(r);
}

// Single-molecule moves before box s's next MultiParticle move, at most
// cap; the records it draws to see that wait in s.ahead.
static int64_t singles_ahead(McState &s, int64_t cap) {
  if (s.params.frac[2] <= 0)
    return cap;
  int64_t k = 0;
  for (; k < cap; ++k) {
    size_t idx = s.ahead_pos + (size_t)k;
    if (idx >= s.ahead.size()) {
      if (s.ahead.size() == s.ahead_pos) {
        // the first record drawn ahead: keep the stream's position
        if (!s.ahead_from)
          s.ahead_from = new MoveStream(*s.stream);
        else
          *s.ahead_from = *s.stream;
        s.ahead.clear();
        s.ahead_pos = 0;
        idx = 0;
      }
      MoveRec r;
      s.stream->Next(&r);
      s.ahead.push_back(r);
    }
    if (s.ahead[idx].kind == 2)
      break;
  }
  return k;
}

void stream_state_at_next(McState &s, uint32_t st[624], int32_t *left,
                          int32_t *next) {
  if (s.ahead_pos >= s.ahead.size()) {
    s.stream->mt().Save(st, left, next);
    return;
  }
  MoveStream tmp(*s.ahead_from);
  MoveRec r;
  for (size_t i = 0; i < s.ahead_pos; ++i)
    tmp.Next(&r);
  tmp.mt().Save(st, left, next);
}

static void skip_to(McState &s, int64_t step) {
  MoveRec r;
  while (s.next_step < step) {
    draw_next(s, &r);
    s.next_step++;
  }
}

static std::pair<cudaEvent_t, cudaEvent_t> ev_pair() {
  cudaEvent_t a = nullptr, z = nullptr;
  cudaEventCreate(&a);
  cudaEventCreate(&z);
  return {a, z};
}

// Fold finished event pairs into the accumulated device times.
static void harvest(McState &s) {
  for (size_t i = 0; i < s.chain_ev.size(); ++i) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, s.chain_ev[i].first, s.chain_ev[i].second) ==
        cudaSuccess)
      s.chain_ms += ms;
    s.chain_launches++;
    s.chain_moves += s.chain_ev_moves[i];
    cudaEventDestroy(s.chain_ev[i].first);
    cudaEventDestroy(s.chain_ev[i].second);
  }
  for (auto &e : s.mp_ev) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, e.first, e.second) == cudaSuccess)
      s.mp_ms += ms;
    s.mp_moves++;
    cudaEventDestroy(e.first);
    cudaEventDestroy(e.second);
  }
  s.chain_ev.clear();
  s.chain_ev_moves.clear();
  s.mp_ev.clear();
}

int mc_set_wait_limit(Box &b, int64_t polls) {
  if (!b.mc)
    return b.Fail(ERR_STATE, "gb_mc_init has not been called");
  if (polls < 0 || polls > 0xffffffffLL)
    return b.Fail(ERR_ARG, "the wait limit must be 0 (default) to 2^32 - 1");
  b.mc->spin_limit = polls == 0 ? SPIN_LIMIT : (unsigned)polls;
  return OK;
}

int mc_profile(Box &b, int enable, double *us13, int64_t *moves2) {
  if (!b.mc)
    return b.Fail(ERR_STATE, "gb_mc_init has not been called");
  McState &s = *b.mc;
  int rc;
  if (!s.d_prof) {
    if ((rc = mc_alloc(b, s, &s.d_prof, 15)) ||
        (rc = b.CudaCheck(cudaMemsetAsync(s.d_prof, 0, 15 * sizeof(long long),
                                          b.stream),
                          "memset")))
      return rc;
  }
  long long hp[15];
  if ((rc = b.CudaCheck(cudaMemcpyAsync(hp, s.d_prof, sizeof hp,
                                        cudaMemcpyDeviceToHost, b.stream),
                        "download")) ||
      (rc = b.CudaCheck(cudaMemsetAsync(s.d_prof, 0, sizeof hp, b.stream),
                        "memset")) ||
      (rc = b.Sync()))
    return rc;
  int khz = 0;
  cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, b.cfg.device);
  for (int k = 0; k < 13; ++k)
    if (us13)
      us13[k] = khz > 0 ? (double)hp[k < 10 ? k : k + 2] / (khz * 1e-3) : 0.0;
  for (int k = 0; k < 2; ++k)
    if (moves2)
      moves2[k] = hp[10 + k];
  s.profile = enable != 0;
  return OK;
}

int mc_timing(Box &b, int reset, double *chain_ms, int64_t *chain_launches,
              int64_t *chain_moves, double *mp_ms, int64_t *mp_moves) {
  if (!b.mc)
    return b.Fail(ERR_STATE, "gb_mc_init has not been called");
  int rc = b.Sync();
  if (rc)
    return rc;
  McState &s = *b.mc;
  harvest(s);
  if (chain_ms)
    *chain_ms = s.chain_ms;
  if (chain_launches)
    *chain_launches = s.chain_launches;
  if (chain_moves)
    *chain_moves = s.chain_moves;
  if (mp_ms)
    *mp_ms = s.mp_ms;
  if (mp_moves)
    *mp_moves = s.mp_moves;
  if (reset) {
    s.chain_ms = s.mp_ms = 0.0;
    s.chain_launches = s.chain_moves = s.mp_moves = 0;
  }
  return OK;
}

static int run_chain(Box &b, McState &s, const MoveRec *moves, int64_t first,
                     int n, int *tr_i, double *tr_d) {
  ChainArgs A;
  A.b = b.dev;
  A.ff = b.d_ff;
  A.set = s.d_set;
  A.moves = moves;
  A.prop = s.d_prop;
  A.first = first;
  A.n = n;
  A.part = s.d_part;
  A.bar = s.d_bar;
  A.seq = s.d_seq;
  A.ctx = s.d_ctx;
  A.ctx_len = chain_ctx_len(b.dev.kmax + 1);
  A.nrows_max = b.dev.K > 0 ? 6 * s.na_max : 0;
  A.nkless = chain_kless(A.nrows_max, s.pipe ? s.grid - 1 : s.grid,
                         s.params.writer_kchunk != 0);
  A.nctx = s.pipe ? 3 : 2;
  chain_perm(b.dev.n_atoms, &A.perm_m, &A.perm_minv);
  A.perm_r = ~0ULL / (unsigned long long)std::max(b.dev.n_atoms, 1);
  A.tr_i = tr_i;
  A.tr_d = tr_d;
  A.prof = s.profile ? s.d_prof : nullptr;
  A.spin = s.spin_limit;
  void *args[] = {&A};
  size_t sm = chain_smem(b, s.grid, A.nrows_max, s.params.writer_kchunk != 0,
                         s.pipe);
  // the per-launch counters of the decision protocol and the grid barrier
  // start from zero
  int rc = b.CudaCheck(cudaMemsetAsync(s.d_seq, 0,
                                       (SEQ_CTX + PART_MAX_GRID) *
                                           sizeof(unsigned),
                                       b.stream),
                       "memset");
  if (!rc)
    rc = b.CudaCheck(cudaMemsetAsync(s.d_bar, 0, 8 * sizeof(unsigned),
                                     b.stream),
                     "memset");
  if (rc)
    return rc;
  k_fill_u64<<<(3 * s.grid * 8 + 255) / 256, 256, 0, b.stream>>>(
      (unsigned long long *)s.d_part, 3 * s.grid * 8, PART_EMPTY);
  auto ev = ev_pair();
  cudaEventRecord(ev.first, b.stream);
  rc = b.CudaCheck(cudaLaunchCooperativeKernel(
                       s.pipe ? (void *)k_chain_fp64_pipe : (void *)k_chain_fp64,
                       dim3(s.grid), dim3(CT), args, sm, b.stream),
                   "chain kernel");
  // the chain keeps positions, not cell slots: CellList::GridAll of the new
  // coordinates brings the grid up to date
  if (!rc)
    rc = launch_grid_all(b, b.dev);
  cudaEventRecord(ev.second, b.stream);
  s.chain_ev.push_back(ev);
  s.chain_ev_moves.push_back(n);
  return rc;
}

static MixedChain fill_mixed(Box &b, McState &s, const MoveRec *moves,
                             int64_t first, int n, int *tr_i, double *tr_d) {
  MixedChain c;
  c.b = b.dev;
  c.ff = b.d_ff;
  c.set = s.d_set;
  c.moves = moves;
  c.prop = s.d_prop;
  c.first = first;
  c.n = n;
  c.ulog = s.ulog;
  c.tr_i = tr_i;
  c.tr_d = tr_d;
  c.cold = s.d_cold;
  return c;
}

static int next_desc(Box &b, McState &s) {
  if (s.desc_next >= s.desc_cap) {
    int rc = b.Sync();  // every staged descriptor has been copied
    if (rc)
      return -1;
    s.desc_next = 0;
  }
  return s.desc_next++;
}

static int run_chain_mixed(Box &b, McState &s, const MoveRec *moves,
                           int64_t first, int n, int *tr_i, double *tr_d) {
  int slot = next_desc(b, s);
  if (slot < 0)
    return ERR_CUDA;
  s.h_desc[slot] = fill_mixed(b, s, moves, first, n, tr_i, tr_d);
  int rc = b.CudaCheck(cudaMemcpyAsync(s.d_desc + slot, s.h_desc + slot,
                                       sizeof(MixedChain),
                                       cudaMemcpyHostToDevice, b.stream),
                       "descriptor upload");
  if (rc)
    return rc;
  auto ev = ev_pair();
  cudaEventRecord(ev.first, b.stream);
  rc = launch_chain_mixed(b.stream, s.d_desc + slot, 1, s.cluster, s.mixed_smem);
  cudaEventRecord(ev.second, b.stream);
  s.chain_ev.push_back(ev);
  s.chain_ev_moves.push_back(n);
  if (rc)
    return b.CudaCheck(cudaGetLastError(), "mixed chain kernel");
  return OK;
}

// Periodic full FP64 recompute of the mixed form: record how far the running
// energies drifted, then restart from the FP64 values (the reference's
// UpdateVectorsAndRecipTerms + SystemTotal, src/Simulation.cpp:170-223).
static int recompute_fp64(Box &b, McState &s) {
  double run[5], tot[9];
  int rc;
  if ((rc = b.GetEnergy(run)) || (rc = b.SystemTotal(tot)))
    return rc;
  double rt = run[0] + run[1] + run[2] + run[3] + run[4];
  double ft = tot[0] + tot[1] + tot[2] + tot[3] + tot[4];
  double d[4] = {std::fabs(run[0] - tot[0]) / std::max(std::fabs(tot[0]), 1e-300),
                 std::fabs(run[1] - tot[1]) / std::max(std::fabs(tot[1]), 1e-300),
                 std::fabs(run[2] - tot[2]) / std::max(std::fabs(tot[2]), 1e-300),
                 std::fabs(rt - ft) / std::max(std::fabs(ft), 1e-300)};
  for (int i = 0; i < 4; ++i) {
    s.drift_last[i] = d[i];
    s.drift_max[i] = std::max(s.drift_max[i], d[i]);
  }
  s.recomputes++;
  return OK;
}

static int run_mp(Box &b, McState &s, int64_t step, int type, int *tr_i,
                  double *tr_d) {
  int rc;
  auto ev = ev_pair();
  cudaEventRecord(ev.first, b.stream);
  s.mp_ev.push_back(ev);
  k_settings_adjust<<<1, 1, 0, b.stream>>>(s.d_set, (long long)step);
  Settings host_set;
  if ((rc = b.CudaCheck(cudaMemcpyAsync(&host_set, s.d_set, sizeof(Settings),
                                        cudaMemcpyDeviceToHost, b.stream),
                        "download")) ||
      (rc = b.Sync()))
    return rc;
  DevBox &d = b.dev;
  if (host_set.singleMoveAccepted) {
    // forces of the current state (MultiParticle::Prep, :208-227)
    if ((rc = b.CopyRecip()) ||
        (rc = launch_force_recip(b, d, d.sumRnew, d.sumInew, b.d_aR, b.d_mR)) ||
        (rc = launch_box_force(b, d, b.d_aF, b.d_mF, s.d_mp + 8)))
      return rc;
    k_set_energy2<<<1, 1, 0, b.stream>>>(d.energy, s.d_mp + 8);
    if ((rc = launch_torque(b, d, b.d_aF, b.d_aR, b.d_tq)))
      return rc;
  }
  if ((rc = b.CudaCheck(cudaMemsetAsync(s.d_mp, 0, 16 * sizeof(double),
                                        b.stream),
                        "memset")))
    return rc;
  MpArgs P;
  P.b = d;
  P.set = s.d_set;
  P.type = type;
  P.step = (uint64_t)step;
  P.seed = s.params.seed;
  P.beta = b.ff.beta;
  P.mF = b.d_mF;
  P.mR = b.d_mR;
  P.tq = b.d_tq;
  P.xn = s.d_xn;
  P.yn = s.d_yn;
  P.zn = s.d_zn;
  P.cxn = s.d_cxn;
  P.cyn = s.d_cyn;
  P.czn = s.d_czn;
  P.tk = s.d_tk;
  P.inrange = s.d_inrange;
  P.fail = (int *)(s.d_mp + 12);
  k_mp_transform<<<(d.n_mol + 127) / 128, 128, 0, b.stream>>>(P);
  // trial state: grid, structure factors, forces, torque
  DevBox n = s.cells_new;
  n.sumRnew = d.sumRnew;
  n.sumInew = d.sumInew;
  n.sumRref = d.sumRref;
  n.sumIref = d.sumIref;
  n.energy = d.energy;
  n.err = d.err;
  if ((rc = launch_grid_all(b, n)) ||
      (rc = launch_recip_sums(b, n.x, n.y, n.z, d.sumRnew, d.sumInew)) ||
      (rc = launch_recip_energy(b, d.sumRnew, d.sumInew, s.d_mp)) ||
      (rc = launch_box_force(b, n, s.d_aFn, s.d_mFn, s.d_mp + 1)) ||
      (rc = launch_force_recip(b, n, d.sumRnew, d.sumInew, s.d_aRn, s.d_mRn)) ||
      (rc = launch_torque(b, n, s.d_aFn, s.d_aRn, s.d_tqn)))
    return rc;
  if (!b.cfg.ewald)
    cudaMemsetAsync(s.d_mp, 0, sizeof(double), b.stream);
  MpAcceptArgs Q;
  Q.b = d;
  Q.set = s.d_set;
  Q.type = type;
  Q.step = (uint64_t)step;
  Q.seed = s.params.seed;
  Q.beta = b.ff.beta;
  Q.mF = b.d_mF;
  Q.mR = b.d_mR;
  Q.tq = b.d_tq;
  Q.mFn = s.d_mFn;
  Q.mRn = s.d_mRn;
  Q.tqn = s.d_tqn;
  Q.tk = s.d_tk;
  Q.inrange = s.d_inrange;
  Q.fail = (const int *)(s.d_mp + 12);
  Q.newE = s.d_mp;
  Q.out = s.d_mp + 4;
  Q.tr_i = tr_i;
  Q.tr_d = tr_d;
  k_mp_accept<<<1, 256, 0, b.stream>>>(Q);
  MpCommitArgs C;
  C.b = d;
  C.bn = n;
  C.flag = s.d_mp + 4;
  C.K = b.cfg.ewald ? d.K : 0;
  C.aF = b.d_aF;
  C.mF = b.d_mF;
  C.aR = b.d_aR;
  C.mR = b.d_mR;
  C.tq = b.d_tq;
  C.aFn = s.d_aFn;
  C.mFn = s.d_mFn;
  C.aRn = s.d_aRn;
  C.mRn = s.d_mRn;
  C.tqn = s.d_tqn;
  k_mp_commit<<<2 * b.sm_count, 256, 0, b.stream>>>(C);
  cudaEventRecord(ev.second, b.stream);
  return b.CudaCheck(cudaGetLastError(), "multiparticle");
}

int mc_run(Box &b, int64_t first, int64_t nsteps, int32_t *kind, int32_t *mol,
           int32_t *acc, double *de) {
  if (!b.mc)
    return b.Fail(ERR_STATE, "gb_mc_init has not been called");
  McState &s = *b.mc;
  if (first < s.next_step)
    return b.Fail(ERR_STATE, "steps must be run in increasing order");
  if (nsteps < 0)
    return b.Fail(ERR_ARG, "negative step count");
  skip_to(s, first);
  bool trace = kind || mol || acc || de;
  int rc;
  if (trace && (size_t)nsteps > s.trace_cap) {
    if ((rc = mc_alloc(b, s, &s.d_trace_i, 3 * (size_t)nsteps)) ||
        (rc = mc_alloc(b, s, &s.d_trace_d, 3 * (size_t)nsteps)))
      return rc;
    s.trace_cap = nsteps;
  }
  int64_t done = 0;
  while (done < nsteps) {
    // fill a chunk of move records
    int64_t chunk = std::min<int64_t>(nsteps - done, (int64_t)s.move_cap);
    if ((rc = b.Sync()))  // the previous chunk may still read h_moves
      return rc;
    for (int64_t i = 0; i < chunk; ++i)
      draw_next(s, &s.h_moves[i]);
    s.next_step += chunk;
    if ((rc = b.CudaCheck(cudaMemcpyAsync(s.d_moves, s.h_moves,
                                          chunk * sizeof(MoveRec),
                                          cudaMemcpyHostToDevice, b.stream),
                          "upload moves")))
      return rc;
    // split into chain segments, MultiParticle moves and (mixed form)
    // periodic FP64 recomputes
    const bool mixed = b.cfg.precision == GB_MIXED;
    const int64_t R = mixed ? s.params.recompute_freq : 0;
    int64_t i = 0;
    while (i < chunk) {
      int64_t step = first + done + i;
      int *ti = trace ? s.d_trace_i + 3 * (done + i) : nullptr;
      double *td = trace ? s.d_trace_d + 3 * (done + i) : nullptr;
      if (s.h_moves[i].kind == 2) {
        if ((rc = run_mp(b, s, step, s.h_moves[i].mol, ti, td)))
          return rc;
        ++i;
        if (R > 0 && (step + 1) % R == 0 && (rc = recompute_fp64(b, s)))
          return rc;
        continue;
      }
      int64_t j = i;
      while (j < chunk && s.h_moves[j].kind != 2) {
        ++j;
        if (R > 0 && (first + done + j) % R == 0)
          break;
      }
      rc = mixed ? run_chain_mixed(b, s, s.d_moves + i, step, (int)(j - i), ti, td)
                 : run_chain(b, s, s.d_moves + i, step, (int)(j - i), ti, td);
      if (rc)
        return rc;
      if (R > 0 && (first + done + j) % R == 0 && (rc = recompute_fp64(b, s)))
        return rc;
      i = j;
    }
    done += chunk;
  }
  if ((rc = b.Sync()) || (rc = b.CheckError()))
    return rc;
  harvest(s);
  if (trace) {
    std::vector<int> ti(3 * (size_t)nsteps);
    std::vector<double> td(3 * (size_t)nsteps);
    if ((rc = b.CudaCheck(cudaMemcpy(ti.data(), s.d_trace_i, ti.size() * 4,
                                     cudaMemcpyDeviceToHost),
                          "trace")) ||
        (rc = b.CudaCheck(cudaMemcpy(td.data(), s.d_trace_d, td.size() * 8,
                                     cudaMemcpyDeviceToHost),
                          "trace")))
      return rc;
    for (int64_t t = 0; t < nsteps; ++t) {
      if (kind)
        kind[t] = ti[3 * t];
      if (mol)
        mol[t] = ti[3 * t + 1];
      if (acc)
        acc[t] = ti[3 * t + 2];
      if (de)
        for (int d = 0; d < 3; ++d)
          de[3 * t + d] = td[3 * t + d];
    }
  }
  return OK;
}

int mc_state(Box &b, double *scales4, int64_t *counts6) {
  if (!b.mc)
    return b.Fail(ERR_STATE, "gb_mc_init has not been called");
  Settings st;
  int rc;
  if ((rc = b.CudaCheck(cudaMemcpyAsync(&st, b.mc->d_set, sizeof(Settings),
                                        cudaMemcpyDeviceToHost, b.stream),
                        "download")) ||
      (rc = b.Sync()))
    return rc;
  if (scales4) {
    scales4[0] = st.scale[0];
    scales4[1] = st.scale[1];
    scales4[2] = st.mp_t_max;
    scales4[3] = st.mp_r_max;
  }
  if (counts6)
    for (int k = 0; k < 3; ++k) {
      counts6[2 * k] = st.tries[k];
      counts6[2 * k + 1] = st.accepted[k];
    }
  return OK;
}

// Launch one segment of several mixed boxes: box i runs n[i] moves (0: not
// in this launch) from its own next step.  Boxes are grouped by cluster size;
// each group is one launch on the stream of its first box, and the groups
// overlap on the device.  Each n[i] must end at or before the box's next
// recompute boundary and fit its move buffer.  `leaders` receives the box
// whose stream carries each launch.
int mixed_launch(const std::vector<Box *> &boxes,
                 const std::vector<int64_t> &n, std::vector<Box *> *leaders) {
  leaders->clear();
  std::vector<int> sizes;
  for (size_t i = 0; i < boxes.size(); ++i)
    if (n[i] > 0 &&
        std::find(sizes.begin(), sizes.end(), boxes[i]->mc->cluster) == sizes.end())
      sizes.push_back(boxes[i]->mc->cluster);
  int rc;
  for (int csize : sizes) {
    std::vector<size_t> g;
    size_t smem = 0;
    for (size_t i = 0; i < boxes.size(); ++i)
      if (n[i] > 0 && boxes[i]->mc->cluster == csize) {
        g.push_back(i);
        smem = std::max(smem, boxes[i]->mc->mixed_smem);
      }
    Box &L = *boxes[g[0]];
    McState &sl = *L.mc;
    int nb = (int)g.size();
    if ((rc = L.Sync()))  // the descriptor staging area is free
      return rc;
    if (sl.desc_cap < nb) {
      sl.desc_cap = std::max(nb, 256);
      if ((rc = mc_alloc(L, sl, &sl.d_desc, sl.desc_cap)))
        return rc;
      if (sl.h_desc)
        cudaFreeHost(sl.h_desc);
      sl.h_desc = nullptr;
      if ((rc = L.CudaCheck(cudaMallocHost(&sl.h_desc,
                                           sl.desc_cap * sizeof(MixedChain)),
                            "pinned")))
        return rc;
    }
    sl.desc_next = sl.desc_cap;  // a single-box run re-syncs before reuse
    int64_t total = 0;
    for (int k = 0; k < nb; ++k) {
      Box &b = *boxes[g[k]];
      McState &s = *b.mc;
      int64_t m = n[g[k]];
      if (m > (int64_t)s.move_cap)
        return b.Fail(ERR_ARG, "segment longer than the move buffer");
      if ((rc = b.Sync()))  // h_moves is free
        return rc;
      for (int64_t t = 0; t < m; ++t)
        draw_next(s, &s.h_moves[t]);
      if ((rc = b.CudaCheck(cudaMemcpyAsync(s.d_moves, s.h_moves,
                                            m * sizeof(MoveRec),
                                            cudaMemcpyHostToDevice, L.stream),
                            "upload moves")))
        return rc;
      sl.h_desc[k] = fill_mixed(b, s, s.d_moves, s.next_step, (int)m, nullptr,
                                nullptr);
      s.next_step += m;
      total += m;
    }
    if ((rc = L.CudaCheck(cudaMemcpyAsync(sl.d_desc, sl.h_desc,
                                          nb * sizeof(MixedChain),
                                          cudaMemcpyHostToDevice, L.stream),
                          "descriptor upload")))
      return rc;
    auto ev = ev_pair();
    cudaEventRecord(ev.first, L.stream);
    if ((rc = launch_chain_mixed(L.stream, sl.d_desc, nb, csize, smem)))
      return L.CudaCheck(cudaGetLastError(), "batched mixed chain kernel");
    cudaEventRecord(ev.second, L.stream);
    sl.chain_ev.push_back(ev);
    sl.chain_ev_moves.push_back((int)total);
    leaders->push_back(&L);
  }
  return OK;
}

// Wait for the launches of mixed_launch, then run the periodic FP64
// recompute of every box whose step count reached a multiple of its
// recompute frequency.
int mixed_complete(const std::vector<Box *> &boxes,
                   const std::vector<int64_t> &n,
                   const std::vector<Box *> &leaders,
                   std::vector<char> *due) {
  int rc;
  for (Box *L : leaders) {
    if ((rc = L->Sync()))
      return rc;
    harvest(*L->mc);  // the launch's events folded into its device time
  }
  if (due)
    due->assign(boxes.size(), 0);
  std::vector<Box *> rec;
  for (size_t i = 0; i < boxes.size(); ++i) {
    if (n[i] <= 0)
      continue;
    Box &b = *boxes[i];
    McState &s = *b.mc;
    if ((rc = b.CheckError()))
      return rc;
    int64_t R = s.params.recompute_freq;
    if (R > 0 && s.next_step % R == 0) {
      if (due)
        (*due)[i] = 1;
      else
        rec.push_back(&b);
    }
  }
  // The due recomputes, several boxes at once: each runs on its own box's
  // stream and waits on that stream only, so one box's kernels fill the
  // tails and host gaps of another's.  Boxes are independent; the order
  // changes no result.
  if (rec.size() == 1)
    return recompute_fp64(*rec[0], *rec[0]->mc);
  if (!rec.empty()) {
    const int dev = rec[0]->cfg.device;
    const int nt = (int)std::min<size_t>(rec.size(), 4);
    std::vector<int> rcs(rec.size(), OK);
    std::atomic<size_t> next{0};
    auto worker = [&] {
      cudaError_t e = cudaSetDevice(dev);
      for (size_t i; (i = next++) < rec.size();)
        rcs[i] = e != cudaSuccess ? rec[i]->CudaCheck(e, "cudaSetDevice")
                                  : recompute_fp64(*rec[i], *rec[i]->mc);
    };
    std::vector<std::thread> th;
    for (int k = 0; k < nt; ++k) {
      // a thread that cannot be started leaves its share to the others and,
      // with none started, to this thread
      try {
        th.emplace_back(worker);
      } catch (const std::system_error &) {
        break;
      }
    }
    if (th.empty())
      worker();
    for (auto &x : th)
      x.join();
    for (int r : rcs)
      if (r)
        return r;
  }
  return OK;
}

int mc_recompute(Box &b) {
  if (!b.mc)
    return b.Fail(ERR_STATE, "gb_mc_init has not been called");
  return recompute_fp64(b, *b.mc);
}

// Moves box i can run before its next recompute boundary (at most cap).
int64_t mixed_segment_limit(Box &b, int64_t cap) {
  McState &s = *b.mc;
  int64_t m = std::min<int64_t>(cap, (int64_t)s.move_cap);
  int64_t R = s.params.recompute_freq;
  if (R > 0)
    m = std::min(m, R - s.next_step % R);
  // a chain segment ends before the box's next MultiParticle move
  return singles_ahead(s, m);
}

// Run fn(i) for every listed box on up to four helper threads (each box's
// work waits on its own stream only); the first error is returned.
template <class F>
static int for_boxes_concurrently(const std::vector<Box *> &boxes,
                                  const std::vector<size_t> &idx, F fn) {
  if (idx.empty())
    return OK;
  if (idx.size() == 1)
    return fn(idx[0]);
  const int dev = boxes[idx[0]]->cfg.device;
  const int nt = (int)std::min<size_t>(idx.size(), 4);
  std::vector<int> rcs(idx.size(), OK);
  std::atomic<size_t> next{0};
  auto worker = [&] {
    cudaError_t e = cudaSetDevice(dev);
    for (size_t k; (k = next++) < idx.size();)
      rcs[k] = e != cudaSuccess ? boxes[idx[k]]->CudaCheck(e, "cudaSetDevice")
                                : fn(idx[k]);
  };
  std::vector<std::thread> th;
  for (int k = 0; k < nt; ++k) {
    try {
      th.emplace_back(worker);
    } catch (const std::system_error &) {
      break;
    }
  }
  if (th.empty())
    worker();
  for (auto &x : th)
    x.join();
  for (int r : rcs)
    if (r)
      return r;
  return OK;
}

int mc_run_batch(const std::vector<Box *> &boxes, int64_t first,
                 int64_t nsteps) {
  // FP64 boxes, boxes on several devices or a single box run one after
  // another through mc_run.
  bool all_mixed = boxes.size() > 1;
  for (Box *b : boxes) {
    if (!b->mc)
      return b->Fail(ERR_STATE, "gb_mc_init has not been called");
    if (b->cfg.precision != GB_MIXED)
      all_mixed = false;
    if (b->cfg.device != boxes[0]->cfg.device)
      all_mixed = false;
  }
  if (!all_mixed) {
    for (Box *b : boxes) {
      int rc = mc_run(*b, first, nsteps, nullptr, nullptr, nullptr, nullptr);
      if (rc)
        return rc;
    }
    return OK;
  }
  int rc;
  for (Box *b : boxes) {
    if (first < b->mc->next_step)
      return b->Fail(ERR_STATE, "steps must be run in increasing order");
    skip_to(*b->mc, first);
  }
  std::vector<int64_t> left(boxes.size(), nsteps), n(boxes.size());
  std::vector<Box *> leaders;
  for (;;) {
    bool any = false, more = false;
    for (size_t i = 0; i < boxes.size(); ++i) {
      n[i] = left[i] > 0 ? mixed_segment_limit(*boxes[i], left[i]) : 0;
      any = any || n[i] > 0;
      more = more || left[i] > 0;
    }
    if (!more)
      break;
    if (any) {
      if ((rc = mixed_launch(boxes, n, &leaders)) ||
          (rc = mixed_complete(boxes, n, leaders)))
        return rc;
      for (size_t i = 0; i < boxes.size(); ++i)
        left[i] -= n[i];
    }
    // boxes whose next move is a MultiParticle move run it now, several at
    // once (each a kernel sequence on its own stream), with the periodic
    // FP64 recompute that falls due after it
    std::vector<size_t> mp;
    for (size_t i = 0; i < boxes.size(); ++i)
      if (left[i] > 0 && singles_ahead(*boxes[i]->mc, 1) == 0)
        mp.push_back(i);
    rc = for_boxes_concurrently(boxes, mp, [&](size_t i) {
      Box &b = *boxes[i];
      McState &s = *b.mc;
      MoveRec r;
      draw_next(s, &r);
      const int64_t step = s.next_step++;
      int e = run_mp(b, s, step, r.mol, nullptr, nullptr);
      const int64_t R = s.params.recompute_freq;
      if (!e && R > 0 && (step + 1) % R == 0)
        e = recompute_fp64(b, s);
      return e;
    });
    if (rc)
      return rc;
    for (size_t i : mp)
      left[i] -= 1;
  }
  return OK;
}

}  // namespace gb
