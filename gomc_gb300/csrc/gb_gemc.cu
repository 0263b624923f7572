// Gibbs ensemble (GEMC NVT) of single-site LJ particles: both boxes in one
// persistent launch of one thread-block cluster.
//
// The move loop follows the reference's System::PickMove / RunMove
// (src/System.cpp:262-302) with Translate (src/moves/Translate.h:52-138),
// MoleculeTransfer building its trial sets through DCLinear / DCSingle
// (src/moves/MoleculeTransfer.h:71-245, src/cbmc/DCLinear.cpp:44-55,
// src/cbmc/DCSingle.cpp:23-90) and VolumeTransfer for GEMC-NVT
// (src/moves/VolumeTransfer.h:71-318), the picks of src/PRNG.h:48-470, the
// box arithmetic of BoxDimensions::ExchangeVolume / SetVolume
// (src/BoxDimensions.cpp:124-227) and Coordinates::TranslateRand /
// TranslateOneBox (src/Coordinates.cpp:83-180), the lookup reordering of
// MoleculeLookup::Shift (src/MoleculeLookup.cpp:178-200) and the move-size
// adjustment of MoveSettings (src/MoveSettings.cpp:94-238).
//
// Every CTA of the cluster holds the whole two-box system in shared memory
// (positions in FP64 with FP32 copies, or 32-bit fixed-point turns in the
// mixed form, and the molecule lookup) and runs its own copy of the
// reference's MT19937 stream: warp 0 draws a move's random numbers (their
// count depends on the state -- molecule counts of the boxes, rejection
// loops -- so they are drawn on the device), every CTA takes a slice of the
// move's pair energies, the partials are exchanged through distributed
// shared memory, and every CTA adds them in rank order, decides and commits
// the same way: one cluster barrier per move (two for a volume exchange).
// The molecule centres live in global memory and are kept by CTA 0 alone;
// the positions go back to global memory at the end of the launch.
//
// Pair sums cover each box's particles in lookup order (all pairs inside the
// cutoff; the reference's cell lists enumerate the same pairs).  Plain form:
// an FP32 distance pre-filter queues each warp's candidate pairs in order and
// full warps evaluate the queue in FP64.  Mixed form: FP32 pair energies on
// exact fixed-point separations, float-float sums per thread and warp, FP64
// across warps and CTAs.
#include "gb_gemc.h"
#include "gb_pair.cuh"

#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

namespace cg = cooperative_groups;

namespace gb {

namespace {

constexpr int PMAX = 3 * GEMC_NTMAX;  // partial values per CTA
constexpr int NW = GEMC_THREADS / 32;
constexpr double SMALL_WEIGHT = 1.0e-38;  // lib/NumLib.h:19
constexpr double TARGET = 0.5;            // MoveSettings::TARGET_ACCEPT_FRACT
constexpr double TINY = 1.0e-7;           // MoveSettings::TINY_AMOUNT
constexpr double TURN = 4294967296.0;

constexpr int WQ = 96;  // per-warp queue of FP64 pair candidates

// One move as warp 0 drew it, with what every warp needs of it in the
// number formats its pair loop uses.
struct Move {
  int kind, b, b1, m, ok;
  double u_acc;            // acceptance uniform (displacement, volume)
  unsigned pick_word;      // raw word of PickWeighted (transfer)
  double np[3], sh[3];     // displacement: new position; shift
  float nf[3];             // its FP32 copy
  unsigned nt[3];          // its fixed-point turns (mixed form)
  double tr[2 * GEMC_NTMAX][3];     // transfer: new trials, then old trials
  float trf[2 * GEMC_NTMAX][3];
  unsigned trt[2 * GEMC_NTMAX][3];
  double nax[2][3], nhalf[2][3], nvol[2], nvolInv[2], sc[2][3];  // volume
  float vcut[2];           // volume: FP32 pre-filter of the old distances
  float nlt[2][3];         // volume: FP32 turn lengths at the new edges
  double d[4];             // values reported in the trace
  double tot[PMAX];        // cluster sums of the partials
  unsigned words[6 * GEMC_NTMAX + 2];  // raw words of a transfer's build
  double wts[2 * GEMC_NTMAX];      // trial weights
};

struct GemcShared {
  GemcCtl c;
  Move mv;
  float axf[2][3], halff[2][3], ltf[2][3];  // FP32 edges, half edges, turns
  float pcut[2];  // FP32 distance pre-filter (FP64 form): Rcut with room
                  // for the FP32 copies' rounding, L 2^-24 per coordinate
  double part[2][PMAX];       // this CTA's partials, by move parity
  double wred[NW][2];         // per-warp sums (displacement, volume)
  int2 wq[NW][WQ];            // per-warp FP64 candidate queues
  int accept;
  int slot;                   // a transferred molecule's slot in the lookup
};

__device__ __forceinline__ double wrapd(double v, double ax) {
  if (v >= ax)
    v -= ax;
  else if (v < 0)
    v += ax;
  return v;
}
__device__ __forceinline__ double unwrapd(double v, double ref, double ax,
                                          double half) {
  if (fabs(ref - v) > half) {
    if (ref < half)
      v -= ax;
    else
      v += ax;
  }
  return v;
}
__device__ __forceinline__ double mimg(double raw, double ax, double half) {
  if (raw > half)
    raw -= ax;
  else if (raw < -half)
    raw += ax;
  return raw;
}
__device__ __forceinline__ float mimgf(float raw, float ax, float half) {
  if (raw > half)
    raw -= ax;
  else if (raw < -half)
    raw += ax;
  return raw;
}
// FFParticle::CalcEn, lambda = 1 (src/FFParticle.cpp:295-325), inside Rcut
__device__ __forceinline__ double lj64(const GemcParams &p, double d2) {
  double rRat2 = p.sigmaSq / d2;
  double rRat4 = rRat2 * rRat2;
  double attract = rRat4 * rRat2;
  double repulse = p.nexp == 12.0 ? attract * attract
                                  : pow(rRat2, p.nexp * 0.5);
  return p.eps_cn * (repulse - attract);
}
__device__ __forceinline__ float lj32(const GemcParams &p, float d2) {
  float s = __fdividef(p.sigmaSq_f, d2);
  float s3 = s * s * s;
  float rep = p.nexp == 12.0 ? s3 * s3 : __powf(s, (float)(p.nexp * 0.5));
  return p.eps_cn_f * (rep - s3);
}
__device__ __forceinline__ unsigned turns(double v, double invL) {
  double t = v * invL;
  t -= floor(t);
  double s = t * TURN;
  unsigned long long u = (unsigned long long)(s + 0.5);
  return (unsigned)(u & 0xffffffffULL);
}

// ---------------------------------------------------------------------------
// MT19937 (Matsumoto & Nishimura 1998) with the output of MTRand
// (src/MersenneTwister.h:320-372), run by the 32 lanes of warp 0: every lane
// holds the same cursor; a block of 624 words is regenerated in four
// dependency phases (the recurrence reads word i + 1 and word i + 397 mod
// 624, which are already new past the first 227 words).
// ---------------------------------------------------------------------------
__device__ void mt_phase(unsigned *st, int lo, int hi) {
  const int lane = threadIdx.x & 31;
  unsigned v[8];
  int c = 0;
  for (int i = lo + lane; i < hi; i += 32) {
    unsigned a = st[i], b = st[(i + 1) % 624], m = st[(i + 397) % 624];
    unsigned y = (a & 0x80000000u) | (b & 0x7fffffffu);
    v[c++] = m ^ (y >> 1) ^ ((b & 1u) ? 0x9908b0dfu : 0u);
  }
  __syncwarp();
  c = 0;
  for (int i = lo + lane; i < hi; i += 32)
    st[i] = v[c++];
  __syncwarp();
}
struct MtCursor {
  unsigned *st;
  int left, next;
  __device__ void reload() {
    mt_phase(st, 0, 227);
    mt_phase(st, 227, 454);
    mt_phase(st, 454, 623);
    mt_phase(st, 623, 624);
    left = 624;
    next = 0;
  }
  __device__ static unsigned temper(unsigned y) {
    y ^= (y >> 11);
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    return y ^ (y >> 18);
  }
  __device__ unsigned u32() {
    if (left == 0)
      reload();
    --left;
    return temper(st[next++]);
  }
  // The next `count` words of the stream into dst (shared memory), the lanes
  // of the warp tempering one word each -- the same words, in the same
  // order, as `count` calls of u32(); every lane calls it.
  __device__ void bulk(unsigned *dst, int count, int lane) {
    int done = 0;
    while (done < count) {
      if (left == 0)
        reload();
      const int take = min(left, count - done);
      for (int i = lane; i < take; i += 32)
        dst[done + i] = temper(st[next + i]);
      next += take;
      left -= take;
      done += take;
    }
    __syncwarp();
  }
  __device__ double rand01() { return (double)u32() * (1.0 / 4294967295.0); }
  __device__ double randExc01() {
    return (double)u32() * (1.0 / 4294967296.0);
  }
  __device__ unsigned randInt(unsigned n) {
    unsigned used = n;
    used |= used >> 1;
    used |= used >> 2;
    used |= used >> 4;
    used |= used >> 8;
    used |= used >> 16;
    unsigned i;
    do
      i = u32() & used;
    while (i > n);
    return i;
  }
};

__device__ __forceinline__ int first_of(const GemcCtl &c, int b) {
  return b == 0 ? 0 : c.start1;
}
__device__ __forceinline__ int count_of(const GemcCtl &c, int n, int b) {
  return b == 0 ? c.start1 : n - c.start1;
}

// MoveSettings::Update (src/MoveSettings.cpp:94-137), counter slot k
__device__ void settings_update(GemcCtl &c, int k, int acc, int b) {
  c.tries[b][k]++;
  c.ttries[b][k]++;
  if (acc) {
    c.tacc[b][k]++;
    c.acc[b][k]++;
  }
}

// MoveSettings::AdjustMoves / Adjust (src/MoveSettings.cpp:147-238)
__device__ void settings_adjust(GemcCtl &c, long long step, int adj) {
  if ((step + 1) % adj != 0)
    return;
  for (int b = 0; b < 2; ++b)
    for (int k = 0; k < 3; ++k) {
      // slots: displacement (counter 0), rotation (no tries), volume (2)
      int cnt = k == 0 ? 0 : k == 2 ? 2 : -1;
      if (cnt >= 0 && c.ttries[b][cnt] > 0) {
        double currentAccept =
            (double)(c.tacc[b][cnt]) / (double)(c.ttries[b][cnt]);
        double f = currentAccept / TARGET;
        if (f > 0.0)
          c.scale[b][k] *= f;
        else
          c.scale[b][k] *= 0.5;
      }
      double lo, hi;
      if (k == 0) {
        double mn = c.ax[b][0];
        if (mn > c.ax[b][1])
          mn = c.ax[b][1];
        if (mn > c.ax[b][2])
          mn = c.ax[b][2];
        lo = 1.0e-10;
        hi = (mn * 0.5) - TINY;
      } else if (k == 1) {
        lo = 1.0e-6;
        hi = M_PI - TINY;
      } else {
        lo = 0.001;
        hi = 0.34 * (c.vol[b] - c.minVol[b]);
      }
      if (c.scale[b][k] < lo)
        c.scale[b][k] = lo;
      if (c.scale[b][k] > hi)
        c.scale[b][k] = hi;
    }
  for (int b = 0; b < 2; ++b)
    for (int k = 0; k < 3; ++k)
      c.ttries[b][k] = c.tacc[b][k] = 0;
}

// Shared-memory arrays after GemcShared: lookup [n]; positions px, py, pz
// and trial positions qx, qy, qz (FP64); the plain form adds FP32 copies
// fx, fy, fz of the positions, the mixed form fixed-point turns tx, ty, tz
// of the positions and ux, uy, uz of the trial positions (uint32).
template <bool MIXED>
struct Arrays {
  int *lookup;
  double *px, *py, *pz, *qx, *qy, *qz;
  float *fx, *fy, *fz;
  unsigned *tx, *ty, *tz, *ux, *uy, *uz;
  __device__ Arrays(unsigned char *base, int n) {
    lookup = (int *)base;
    size_t off = ((size_t)n * 4 + 15) / 16 * 16;
    px = (double *)(base + off);
    py = px + n;
    pz = py + n;
    qx = pz + n;
    qy = qx + n;
    qz = qy + n;
    if (!MIXED) {
      fx = (float *)(qz + n);
      fy = fx + n;
      fz = fy + n;
    } else {
      tx = (unsigned *)(qz + n);
      ty = tx + n;
      tz = ty + n;
      ux = tz + n;
      uy = ux + n;
      uz = uy + n;
    }
  }
};

// FP32 copies of the box edges for the pair loops (after every change).
__device__ void box_consts(GemcShared &S, double rcut) {
  for (int b = 0; b < 2; ++b) {
    for (int d = 0; d < 3; ++d) {
      S.axf[b][d] = (float)S.c.ax[b][d];
      S.halff[b][d] = (float)S.c.half[b][d];
      S.ltf[b][d] = (float)(S.c.ax[b][d] / TURN);
    }
    const double lmax =
        fmax(S.c.ax[b][0], fmax(S.c.ax[b][1], S.c.ax[b][2]));
    const double r = rcut + 1e-5 * lmax + 1e-4;
    S.pcut[b] = (float)(r * r);
  }
}

// Error-free FP32 accumulation: (hi, lo) += v.
__device__ __forceinline__ void two_sum_add(float &hi, float &lo, float v) {
  float s = hi + v;
  float bp = s - hi;
  float err = (hi - (s - bp)) + (v - bp);
  hi = s;
  lo += err;
}
// Warp sum of a float-float pair, to lane 0.
__device__ __forceinline__ void warp_two_sum(float &hi, float &lo) {
  for (int o = 16; o > 0; o >>= 1) {
    float h2 = __shfl_down_sync(0xffffffffu, hi, o);
    float l2 = __shfl_down_sync(0xffffffffu, lo, o);
    two_sum_add(hi, lo, h2);
    lo += l2;
  }
}
__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1)
    v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ int warp_sum_i(int v) {
  for (int o = 16; o > 0; o >>= 1)
    v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float r2_turns(unsigned ax, unsigned ay,
                                          unsigned az, unsigned bx,
                                          unsigned by, unsigned bz,
                                          const float *lt) {
  float dx = (float)(int)(ax - bx) * lt[0];
  float dy = (float)(int)(ay - by) * lt[1];
  float dz = (float)(int)(az - bz) * lt[2];
  return fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}
__device__ __forceinline__ float r2_f32(float ax, float ay, float az,
                                        float bx, float by, float bz,
                                        const float *L, const float *H) {
  float dx = mimgf(ax - bx, L[0], H[0]);
  float dy = mimgf(ay - by, L[1], H[1]);
  float dz = mimgf(az - bz, L[2], H[2]);
  return fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}
__device__ __forceinline__ double r2_f64(double ax, double ay, double az,
                                         double bx, double by, double bz,
                                         const double *L, const double *H) {
  double ex = mimg(ax - bx, L[0], H[0]);
  double ey = mimg(ay - by, L[1], H[1]);
  double ez = mimg(az - bz, L[2], H[2]);
  return ex * ex + ey * ey + ez * ez;
}

// Evaluates a warp's queued candidates 32 at a time, in queue order (all:
// also the last partial group), and moves the rest to the queue's front.
// Between flushes a warp adds at most 64 entries to fewer than 32, so the
// queue never holds more than 95.
template <class F>
__device__ __forceinline__ void qflush(int2 *q, int &qn, bool all, int lane,
                                       F &eval) {
  while (qn >= 32 || (all && qn > 0)) {
    __syncwarp();
    if (lane < qn)
      eval(q[lane]);
    const int rest = qn > 32 ? qn - 32 : 0;
    int2 a = make_int2(0, 0), a2 = make_int2(0, 0);
    if (lane < rest)
      a = q[32 + lane];
    if (lane + 32 < rest)
      a2 = q[64 + lane];
    __syncwarp();
    if (lane < rest)
      q[lane] = a;
    if (lane + 32 < rest)
      q[lane + 32] = a2;
    __syncwarp();
    qn = rest;
  }
}

__device__ __forceinline__ void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
  asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// The Gibbs-ensemble loop (src/moves/*.h of the GEMC build; the move
// sequence of System::RunningCheck / ChooseAndRunMove): warp 0 of every CTA
// draws the move from its copy of the MT19937 state, every CTA evaluates
// its slice of the pair terms, the partials meet over distributed shared
// memory, and every CTA takes the same decision.
//   FP64 form: an FP32 distance pre-filter queues the candidate pairs of
//   each warp in order; the queue is evaluated in FP64 on full warps.
//   Mixed form: FP32 pair energies on exact fixed-point separations, summed
//   error-free in float-float, one FP64 value per warp.
template <bool MIXED>
__global__ void __launch_bounds__(GEMC_THREADS)
    k_gemc(const GemcParams p) {
  extern __shared__ __align__(16) unsigned char dyn[];
  GemcShared &S = *(GemcShared *)dyn;
  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const unsigned lt_mask = (1u << lane) - 1u;
  const int n = p.n, nt = p.nt;
  Arrays<MIXED> A(dyn + (sizeof(GemcShared) + 15) / 16 * 16, n);
  GemcCtl &c = S.c;

  // ---- load the state ----
  {
    const unsigned *src = (const unsigned *)p.ctl;
    unsigned *dst = (unsigned *)&S.c;
    for (int i = tid; i < (int)(sizeof(GemcCtl) / 4); i += GEMC_THREADS)
      dst[i] = src[i];
  }
  __syncthreads();
  if (tid == 0)
    box_consts(S, p.rcut);
  for (int i = tid; i < n; i += GEMC_THREADS)
    A.lookup[i] = p.lookup[i];
  __syncthreads();
  for (int i = tid; i < n; i += GEMC_THREADS) {
    int j = A.lookup[i];
    int b = i < c.start1 ? 0 : 1;
    A.px[j] = p.x[j];
    A.py[j] = p.y[j];
    A.pz[j] = p.z[j];
    if (!MIXED) {
      A.fx[j] = (float)p.x[j];
      A.fy[j] = (float)p.y[j];
      A.fz[j] = (float)p.z[j];
    } else {
      A.tx[j] = turns(p.x[j], 1.0 / c.ax[b][0]);
      A.ty[j] = turns(p.y[j], 1.0 / c.ax[b][1]);
      A.tz[j] = turns(p.z[j], 1.0 / c.ax[b][2]);
    }
  }
  __syncthreads();
  cluster.sync();

  const bool prof = p.prof && rank == 0 && tid == 0;
  long long pacc[3][5] = {}, pcnt[3] = {0, 0, 0};
  long long tclk = prof ? clock64() : 0;
  auto mark = [&](int slot, int ph) {
    if (prof && slot >= 0) {
      long long now = clock64();
      pacc[slot][ph] += now - tclk;
      tclk = now;
    }
  };
  Move &M = S.mv;

  double cpend = 0.0;  // CTA 0, warp 0, lanes 0-2: a displaced centre
  for (int t = 0; t < p.nsteps; ++t) {
    const long long step = p.first + t;
    const int par = t & 1;
    // ---------------- draw the move (warp 0) ----------------
    if (warp == 0) {
      if (lane == 0)
        settings_adjust(c, step, p.adj);
      __syncwarp();
      MtCursor R{c.mt, c.mt_left, c.mt_next};
      // System::PickMove: PRNG::PickArbDist (Wt = 1) walks the running sums
      // of the weights and takes the first kind whose sum reaches the draw
      const double draw = R.rand01() * 1.0;
      const bool ge = lane < GEMC_KINDS && p.cum[lane] >= draw;
      const unsigned bal = __ballot_sync(0xffffffffu, ge);
      const int kind = bal ? __ffs(bal) - 1 : GEMC_KINDS - 1;
      const double prevSum = kind > 0 ? p.cum[kind - 1] : 0.0;
      const double subDraw = draw - prevSum;
      int b = -1, b1 = -1, m = -1, ok = 0;
      unsigned pick_word = 0;
      if (kind == GEMC_DISPLACE || kind == GEMC_TRANSFER ||
          kind == GEMC_VOLUME) {
        // PRNG::PickBox: (uint)(subDraw / boxDiv) of two boxes, boxDiv =
        // movPerc / 2; the rounded quotient reaches 1 exactly when subDraw
        // reaches boxDiv
        b = subDraw >= p.boxdiv[kind] ? 1 : 0;
        b1 = 1 - b;
      }
      if (kind == GEMC_DISPLACE || kind == GEMC_TRANSFER) {
        // PRNG::PickMol / PickMol2: a molecule of the (single) kind
        int nb = count_of(c, n, b);
        if (nb > 0) {
          unsigned off = R.randInt((unsigned)nb - 1u);
          m = A.lookup[first_of(c, b) + off];
          ok = 1;
        }
      } else if (kind == GEMC_VOLUME) {
        ok = 1;
      }
      if (kind == GEMC_DISPLACE && ok) {
        // Coordinates::TranslateRand with PRNG::SymXYZ (three words), then
        // the acceptance word; lane d takes axis d
        const unsigned w0 = R.u32(), w1 = R.u32(), w2 = R.u32(),
                       w3 = R.u32();
        if (lane < 3) {
          const unsigned w = lane == 0 ? w0 : lane == 1 ? w1 : w2;
          const double bound = c.scale[b][0], bound2 = 2.0 * bound;
          const double sh = (double)w * (1.0 / 4294967295.0) * bound2 - bound;
          const double pv = lane == 0 ? A.px[m] : lane == 1 ? A.py[m] : A.pz[m];
          const double nv = wrapd(pv + sh, c.ax[b][lane]);
          M.np[lane] = nv;
          M.sh[lane] = sh;
          M.nf[lane] = (float)nv;
          if (MIXED)
            M.nt[lane] = turns(nv, 1.0 / c.ax[b][lane]);
          if (rank == 0)  // the centres are CTA 0's (global memory): the
                          // load is consumed at the commit
            cpend = lane == 0 ? p.cx[m] : lane == 1 ? p.cy[m] : p.cz[m];
        } else if (lane == 3) {
          M.u_acc = (double)w3 * (1.0 / 4294967295.0);
        }
      } else if (kind == GEMC_TRANSFER && ok) {
        // DCLinear::Build: direction, DCSingle::BuildNew (trials in the
        // destination box, PickWeighted), DCSingle::BuildOld (trials in the
        // source box, trial 0 at the molecule): the raw words in order, then
        // each lane scales its own coordinates
        // randInt(1) draws one word (a 1-bit mask never rejects), then
        // 3 nt words, the PickWeighted word, 3 nt words: 6 nt + 2 words
        unsigned *wbuf = M.words;
        R.bulk(wbuf, 6 * nt + 2, lane);
        pick_word = wbuf[1 + 3 * nt];
        wbuf += 1;  // the trial words: [0, 3 nt) new, [3 nt + 1, ...) old
        for (int q = lane; q < 6 * nt; q += 32) {
          const int k = q / 3, d = q - 3 * k;
          const int bb = k < nt ? b1 : b;
          const unsigned w = wbuf[q < 3 * nt ? q : q + 1];
          double v = (double)w * (1.0 / 4294967296.0) * c.ax[bb][d];
          if (k == nt)
            v = wrapd(d == 0 ? A.px[m] : d == 1 ? A.py[m] : A.pz[m],
                      c.ax[b][d]);
          M.tr[k][d] = v;
          M.trf[k][d] = (float)v;
          if (MIXED)
            M.trt[k][d] = turns(v, 1.0 / c.ax[bb][d]);
        }
      } else if (kind == GEMC_VOLUME) {
        // Coordinates::VolumeTransferTranslate: PRNG::Sym, then
        // BoxDimensions::ExchangeVolume
        double max = c.scale[b][2];
        if (c.scale[b1][2] < max)
          max = c.scale[b1][2];
        double transfer = R.rand01() * (2.0 * max) - max;
        if (lane == 0) {
          for (int bb = 0; bb < 2; ++bb) {
            for (int d = 0; d < 3; ++d) {
              M.nax[bb][d] = c.ax[bb][d];
              M.nhalf[bb][d] = c.half[bb][d];
            }
            M.nvol[bb] = c.vol[bb];
            M.nvolInv[bb] = c.volInv[bb];
          }
          const int bp[2] = {b, b1};
          double vTot = (c.vol[bp[0]] + c.vol[bp[1]]);
          for (int i = 0; i < 2; ++i) {
            int bb = bp[i];
            double v = i == 0 ? c.vol[bp[0]] + transfer : vTot - M.nvol[bp[0]];
            double ratio = cbrt(v / M.nvol[bb]);
            for (int d = 0; d < 3; ++d) {
              M.nax[bb][d] *= ratio;
              M.nhalf[bb][d] *= ratio;
            }
            M.nvol[bb] = v;
            M.nvolInv[bb] = 1.0 / v;
          }
          for (int i = 0; i < 2; ++i) {
            int bb = bp[i];
            double smin = 1e300;
            for (int d = 0; d < 3; ++d) {
              M.sc[bb][d] = M.nax[bb][d] / c.ax[bb][d];
              smin = fmin(smin, M.sc[bb][d]);
              M.nlt[bb][d] = (float)(M.nax[bb][d] / TURN);
            }
            // a new separation is the old one scaled by sc per axis: the
            // FP32 pre-filter on the old distances, with room for rounding
            double lmax = fmax(c.ax[bb][0], fmax(c.ax[bb][1], c.ax[bb][2]));
            double rr = (p.rcut + 1e-5 * lmax + 1e-4) / smin;
            M.vcut[bb] = (float)(rr * rr);
            if (M.nhalf[bb][0] < p.rcut || M.nhalf[bb][1] < p.rcut ||
                M.nhalf[bb][2] < p.rcut || M.nvol[bb] < c.minVol[bb])
              c.err = 1;
          }
        }
        __syncwarp();
        if (!c.err) {
          double u = R.rand01();
          if (lane == 0)
            M.u_acc = u;
        }
      }
      if (lane == 0) {
        M.kind = kind;
        M.b = b;
        M.b1 = b1;
        M.m = m;
        M.ok = ok;
        M.pick_word = pick_word;
        c.mt_left = R.left;
        c.mt_next = R.next;
      }
    }
    __syncthreads();
    if (c.err)
      break;  // every CTA drew the same volume change
    const int kind = M.kind, b = M.b, b1 = M.b1, m = M.m;
    const int pslot = kind == GEMC_DISPLACE ? 0 : kind == GEMC_TRANSFER ? 1
                      : kind == GEMC_VOLUME ? 2 : -1;
    mark(pslot, 0);
    int nval = 0;
    int2 *q = S.wq[warp];
    // ---------------- energy phase (all CTAs) ----------------
    if (kind == GEMC_DISPLACE && M.ok) {
      // Translate::CalcEn -> MoleculeInter (the molecule out of the cell
      // list): this CTA's slice of the box's molecules
      nval = 2;
      const int a0 = first_of(c, b), nb = count_of(c, n, b);
      const int lo = (int)((long long)nb * rank / C);
      const int hi = (int)((long long)nb * (rank + 1) / C);
      if (!MIXED) {
        const float *L = S.axf[b], *H = S.halff[b];
        const float ofx = A.fx[m], ofy = A.fy[m], ofz = A.fz[m];
        const float nfx = M.nf[0], nfy = M.nf[1], nfz = M.nf[2];
        const double opx = A.px[m], opy = A.py[m], opz = A.pz[m];
        const double npx = M.np[0], npy = M.np[1], npz = M.np[2];
        double acc = 0.0;
        int ovl = 0, qn = 0;
        const float pc = S.pcut[b];
        auto eval = [&](int2 e) {  // e = (molecule, 1: new position)
          const bool nw = e.y != 0;
          double d2 = r2_f64(nw ? npx : opx, nw ? npy : opy, nw ? npz : opz,
                             A.px[e.x], A.py[e.x], A.pz[e.x], c.ax[b],
                             c.half[b]);
          if (d2 < p.rcutSq) {
            double en = lj64(p, d2);
            acc += nw ? en : -en;
            if (nw && d2 < p.rcutLowSq)
              ++ovl;
          }
        };
        for (int i0 = lo + warp * 32; i0 < hi; i0 += GEMC_THREADS) {
          const int i = i0 + lane;
          int j = i < hi ? A.lookup[a0 + i] : -1;
          bool co = false, cn = false;
          if (j >= 0 && j != m) {
            const float jx = A.fx[j], jy = A.fy[j], jz = A.fz[j];
            co = r2_f32(ofx, ofy, ofz, jx, jy, jz, L, H) < pc;
            cn = r2_f32(nfx, nfy, nfz, jx, jy, jz, L, H) < pc;
          }
          const unsigned bo = __ballot_sync(0xffffffffu, co);
          if (co)
            q[qn + __popc(bo & lt_mask)] = make_int2(j, 0);
          qn += __popc(bo);
          const unsigned bn = __ballot_sync(0xffffffffu, cn);
          if (cn)
            q[qn + __popc(bn & lt_mask)] = make_int2(j, 1);
          qn += __popc(bn);
          qflush(q, qn, false, lane, eval);
        }
        qflush(q, qn, true, lane, eval);
        acc = warp_sum(acc);
        ovl = warp_sum_i(ovl);
        if (lane == 0) {
          S.wred[warp][0] = acc;
          S.wred[warp][1] = (double)ovl;
        }
      } else {
        const float *lt = S.ltf[b];
        const unsigned otx = A.tx[m], oty = A.ty[m], otz = A.tz[m];
        const unsigned ntx = M.nt[0], nty = M.nt[1], ntz = M.nt[2];
        float sh = 0.0f, sl = 0.0f;
        int ovl = 0;
        for (int i = lo + tid; i < hi; i += GEMC_THREADS) {
          const int j = A.lookup[a0 + i];
          if (j == m)
            continue;
          const unsigned jx = A.tx[j], jy = A.ty[j], jz = A.tz[j];
          const float ro = r2_turns(otx, oty, otz, jx, jy, jz, lt);
          const float rn = r2_turns(ntx, nty, ntz, jx, jy, jz, lt);
          const float eo = ro < p.rcutSq_f ? lj32(p, ro) : 0.0f;
          float en = 0.0f;
          if (rn < p.rcutSq_f) {
            en = lj32(p, rn);
            if (rn < p.rcutLowSq_f)
              ++ovl;
          }
          two_sum_add(sh, sl, en);
          two_sum_add(sh, sl, -eo);
        }
        warp_two_sum(sh, sl);
        ovl = warp_sum_i(ovl);
        if (lane == 0) {
          S.wred[warp][0] = (double)sh + (double)sl;
          S.wred[warp][1] = (double)ovl;
        }
      }
    } else if (kind == GEMC_TRANSFER && M.ok) {
      // CalculateEnergy::ParticleInter of each trial (the molecule is out of
      // its box's cell list): new trials in the destination box, old trials
      // in the source box; warp w takes trials w, w + 8, ... over this
      // CTA's slice of the trial's box
      nval = 3 * nt;
      if (!MIXED) {
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        int ov[4] = {0, 0, 0, 0};
        int qn = 0;
        auto eval = [&](int2 e) {  // e = (molecule, trial of this warp)
          const int k = warp + NW * e.y;
          const int bb = k < nt ? b1 : b;
          double d2 = r2_f64(M.tr[k][0], M.tr[k][1], M.tr[k][2], A.px[e.x],
                             A.py[e.x], A.pz[e.x], c.ax[bb], c.half[bb]);
          if (d2 < p.rcutSq) {
            double en = lj64(p, d2);
            bool lowr = d2 < p.rcutLowSq;
#pragma unroll
            for (int u = 0; u < 4; ++u)
              if (u == e.y) {
                acc[u] += en;
                ov[u] += lowr ? 1 : 0;
              }
          }
        };
        for (int kl = 0; warp + NW * kl < 2 * nt; ++kl) {
          const int k = warp + NW * kl;
          const int bb = k < nt ? b1 : b;
          const int a0 = first_of(c, bb), nb = count_of(c, n, bb);
          const int lo = (int)((long long)nb * rank / C);
          const int hi = (int)((long long)nb * (rank + 1) / C);
          const float sx = M.trf[k][0], sy = M.trf[k][1], sz = M.trf[k][2];
          const float *L = S.axf[bb], *H = S.halff[bb];
          const float pc = S.pcut[bb];
          for (int i0 = lo; i0 < hi; i0 += 32) {
            const int i = i0 + lane;
            int j = i < hi ? A.lookup[a0 + i] : -1;
            bool cd = j >= 0 && j != m &&
                      r2_f32(sx, sy, sz, A.fx[j], A.fy[j], A.fz[j], L, H) < pc;
            const unsigned bc = __ballot_sync(0xffffffffu, cd);
            if (cd)
              q[qn + __popc(bc & lt_mask)] = make_int2(j, kl);
            qn += __popc(bc);
            qflush(q, qn, false, lane, eval);
          }
        }
        qflush(q, qn, true, lane, eval);
        for (int kl = 0; warp + NW * kl < 2 * nt; ++kl) {
          const int k = warp + NW * kl;
          double a = 0.0;
          int o = 0;
#pragma unroll
          for (int u = 0; u < 4; ++u)
            if (u == kl) {
              a = acc[u];
              o = ov[u];
            }
          a = warp_sum(a);
          o = warp_sum_i(o);
          if (lane == 0) {
            S.part[par][k] = a;
            if (k < nt)
              S.part[par][2 * nt + k] = (double)o;
          }
        }
      } else {
        for (int k = warp; k < 2 * nt; k += NW) {
          const int bb = k < nt ? b1 : b;
          const int a0 = first_of(c, bb), nb = count_of(c, n, bb);
          const int lo = (int)((long long)nb * rank / C);
          const int hi = (int)((long long)nb * (rank + 1) / C);
          const unsigned ux = M.trt[k][0], uy = M.trt[k][1], uz = M.trt[k][2];
          const float *lt = S.ltf[bb];
          float sh = 0.0f, sl = 0.0f;
          int ovl = 0;
          for (int i = lo + lane; i < hi; i += 32) {
            const int j = A.lookup[a0 + i];
            if (j == m)
              continue;
            const float r2 =
                r2_turns(ux, uy, uz, A.tx[j], A.ty[j], A.tz[j], lt);
            if (r2 < p.rcutSq_f) {
              two_sum_add(sh, sl, lj32(p, r2));
              if (r2 < p.rcutLowSq_f)
                ++ovl;
            }
          }
          warp_two_sum(sh, sl);
          ovl = warp_sum_i(ovl);
          if (lane == 0) {
            S.part[par][k] = (double)sh + (double)sl;
            if (k < nt)
              S.part[par][2 * nt + k] = (double)ovl;
          }
        }
      }
    } else if (kind == GEMC_VOLUME) {
      // Coordinates::TranslateOneBox of both boxes into the trial arrays,
      // then BoxInter of both boxes at the new axes.  The centres are CTA
      // 0's (global memory): a cluster barrier first makes its latest
      // writes visible; every CTA moves its slice of the molecules, and a
      // second barrier lets each copy the other slices.
      nval = 2;
      cluster_barrier();
      {
        const int lo = (int)((long long)n * rank / C);
        const int hi = (int)((long long)n * (rank + 1) / C);
        for (int i = lo + tid; i < hi; i += GEMC_THREADS) {
          int j = A.lookup[i];
          int bb = i < c.start1 ? 0 : 1;
          double ocx = p.cx[j], ocy = p.cy[j], ocz = p.cz[j];
          double ncx = ocx * M.sc[bb][0], ncy = ocy * M.sc[bb][1],
                 ncz = ocz * M.sc[bb][2];
          double ux = unwrapd(A.px[j], ocx, c.ax[bb][0], c.half[bb][0]);
          double uy = unwrapd(A.py[j], ocy, c.ax[bb][1], c.half[bb][1]);
          double uz = unwrapd(A.pz[j], ocz, c.ax[bb][2], c.half[bb][2]);
          double nx = wrapd(ux + (ncx - ocx), M.nax[bb][0]);
          double ny = wrapd(uy + (ncy - ocy), M.nax[bb][1]);
          double nz = wrapd(uz + (ncz - ocz), M.nax[bb][2]);
          A.qx[j] = nx;
          A.qy[j] = ny;
          A.qz[j] = nz;
          if (MIXED) {
            A.ux[j] = turns(nx, 1.0 / M.nax[bb][0]);
            A.uy[j] = turns(ny, 1.0 / M.nax[bb][1]);
            A.uz[j] = turns(nz, 1.0 / M.nax[bb][2]);
          }
        }
      }
      cluster_barrier();
      for (int r = 0; r < C; ++r) {
        if (r == rank)
          continue;
        const int lo = (int)((long long)n * r / C);
        const int hi = (int)((long long)n * (r + 1) / C);
        const double *rqx = cluster.map_shared_rank(A.qx, (unsigned)r);
        const double *rqy = cluster.map_shared_rank(A.qy, (unsigned)r);
        const double *rqz = cluster.map_shared_rank(A.qz, (unsigned)r);
        for (int i = lo + tid; i < hi; i += GEMC_THREADS) {
          int j = A.lookup[i];
          A.qx[j] = rqx[j];
          A.qy[j] = rqy[j];
          A.qz[j] = rqz[j];
          if (MIXED) {
            A.ux[j] = cluster.map_shared_rank(A.ux, (unsigned)r)[j];
            A.uy[j] = cluster.map_shared_rank(A.uy, (unsigned)r)[j];
            A.uz[j] = cluster.map_shared_rank(A.uz, (unsigned)r)[j];
          }
        }
      }
      __syncthreads();
      // pair tiles of 32 x 32 (block row <= block column) dealt to the
      // cluster's warps; lane l takes row l of its tile
      const int gw = rank * NW + warp, GW = C * NW;
      double ebox[2] = {0.0, 0.0};
      for (int bb = 0; bb < 2; ++bb) {
        const int a0 = first_of(c, bb), nb = count_of(c, n, bb);
        const int nbt = (nb + 31) / 32;
        const int ntile = nbt * (nbt + 1) / 2;
        double acc = 0.0;
        float sh = 0.0f, sl = 0.0f;
        int qn = 0;
        const float *L = S.axf[bb], *H = S.halff[bb];
        const float vcut = M.vcut[bb];
        const float *nlt = M.nlt[bb];
        auto eval = [&](int2 e) {  // e = (molecule, molecule)
          double d2 = r2_f64(A.qx[e.x], A.qy[e.x], A.qz[e.x], A.qx[e.y],
                             A.qy[e.y], A.qz[e.y], M.nax[bb], M.nhalf[bb]);
          if (d2 < p.rcutSq)
            acc += lj64(p, d2);
        };
        for (int tl = gw; tl < ntile; tl += GW) {
          int ib = 0, rem = tl;
          while (rem >= nbt - ib) {
            rem -= nbt - ib;
            ++ib;
          }
          const int jb = ib + rem;
          const int i = ib * 32 + lane;
          const bool act = i < nb;
          const int pi = act ? A.lookup[a0 + i] : 0;
          float fxi = 0, fyi = 0, fzi = 0;
          unsigned txi = 0, tyi = 0, tzi = 0;
          if (act) {
            if (!MIXED) {
              fxi = A.fx[pi];
              fyi = A.fy[pi];
              fzi = A.fz[pi];
            } else {
              txi = A.ux[pi];
              tyi = A.uy[pi];
              tzi = A.uz[pi];
            }
          }
          const int j0 = jb * 32, j1 = min(nb, j0 + 32);
          for (int jj = j0; jj < j1; ++jj) {
            const int pj = A.lookup[a0 + jj];
            const bool valid = act && jj > i;
            if (!MIXED) {
              bool cd = valid && r2_f32(fxi, fyi, fzi, A.fx[pj], A.fy[pj],
                                        A.fz[pj], L, H) < vcut;
              const unsigned bc = __ballot_sync(0xffffffffu, cd);
              if (cd)
                q[qn + __popc(bc & lt_mask)] = make_int2(pi, pj);
              qn += __popc(bc);
              qflush(q, qn, false, lane, eval);
            } else if (valid) {
              const float r2 = r2_turns(txi, tyi, tzi, A.ux[pj], A.uy[pj],
                                        A.uz[pj], nlt);
              if (r2 < p.rcutSq_f)
                two_sum_add(sh, sl, lj32(p, r2));
            }
          }
        }
        if (!MIXED) {
          qflush(q, qn, true, lane, eval);
          ebox[bb] = warp_sum(acc);
        } else {
          warp_two_sum(sh, sl);
          ebox[bb] = (double)sh + (double)sl;
        }
      }
      if (lane == 0) {
        S.wred[warp][0] = ebox[0];
        S.wred[warp][1] = ebox[1];
      }
    }
    __syncthreads();
    mark(pslot, 1);
    // this CTA's partials, warps in order (a transfer's trials went straight
    // to their slots)
    if (tid < nval && kind != GEMC_TRANSFER) {
      double v = 0.0;
      for (int w = 0; w < NW; ++w)
        v += S.wred[w][tid];
      S.part[par][tid] = v;
    }
    // ---------------- exchange: one cluster barrier ----------------
    cluster_barrier();
    if (tid < nval) {
      // the ranks' partials loaded together, added in rank order
      double pr[16];
#pragma unroll
      for (int r = 0; r < 16; ++r)
        pr[r] = r < C ? cluster.map_shared_rank(&S.part[par][0],
                                                (unsigned)r)[tid]
                      : 0.0;
      double v = 0.0;
      for (int r = 0; r < C; ++r)
        v += pr[r];
      M.tot[tid] = v;
    }
    __syncthreads();
    mark(pslot, 2);
    // ---------------- decision (identical in every CTA) ----------------
    if (warp == 0) {
      MtCursor R{c.mt, c.mt_left, c.mt_next};
      int acc = 0;
      if (kind == GEMC_DISPLACE) {
        if (M.ok) {
          double dLJ = M.tot[0];
          bool ovl = M.tot[1] > 0.0;
          int res = M.u_acc < exp(-p.beta * (dLJ + 0.0 + 0.0));
          acc = res && !ovl;
          if (lane == 0) {
            if (acc)
              c.e[b] += dLJ;
            M.d[0] = dLJ;
            M.d[1] = ovl ? 1.0 : 0.0;
            M.d[2] = M.d[3] = 0.0;
            settings_update(c, 0, acc, b);
          }
        } else if (lane == 0) {
          settings_update(c, 0, 0, b);
          M.d[0] = M.d[1] = M.d[2] = M.d[3] = 0.0;
        }
      } else if (kind == GEMC_TRANSFER) {
        if (M.ok) {
          // the Boltzmann weights of all trials, one lane each, then added
          // in trial order
          double *wv = M.wts;
          for (int k = lane; k < 2 * nt; k += 32)
            wv[k] = exp(-1 * p.beta * ((0.0 + M.tot[k]) + 0.0));
          __syncwarp();
          double stepWeight = 0.0;
          for (int k = 0; k < nt; ++k)
            stepWeight += wv[k];
          // PRNG::PickWeighted (src/PRNG.h:167-200)
          double draw = ((double)M.pick_word * (1.0 / 4294967295.0)) *
                        stepWeight;
          double s = 0.0;
          int winner = -1;
          for (int k = 0; k < nt; ++k) {
            s += wv[k];
            if (s >= draw) {
              winner = k;
              break;
            }
          }
          if (winner < 0) {
            int lastZero = nt;
            for (int k = nt - 1; k > 0 && wv[k] == 0.0; --k)
              lastZero = k;
            winner = lastZero - 1;  // |draw - total| < 0.001 in practice
          }
          bool overlap = M.tot[2 * nt + winner] > 0.0;
          double Wn = 1.0 * (stepWeight / nt);
          double sumOld = 0.0;
          for (int k = 0; k < nt; ++k)
            sumOld += wv[nt + k];
          double Wo = 1.0 * (sumOld / nt);
          double eNew = 0.0 + M.tot[winner], eOld = 0.0 + M.tot[nt];
          int nsrc = count_of(c, n, b), ndest = count_of(c, n, b1);
          double coeff = (double)(nsrc) / (double)(ndest + 1) * c.vol[b1] *
                         c.volInv[b];
          double Wrat = Wn / Wo * 1.0 * 1.0;
          if (Wn > SMALL_WEIGHT && !overlap)
            acc = R.rand01() < coeff * Wrat;
          if (lane == 0) {
            M.d[0] = Wn;
            M.d[1] = Wo;
            M.d[2] = eNew;
            M.d[3] = eOld;
            if (acc) {
              c.e[b] -= eOld;
              c.e[b1] += eNew;
              for (int d = 0; d < 3; ++d) {
                M.np[d] = M.tr[winner][d];
                M.nf[d] = M.trf[winner][d];
                M.nt[d] = M.trt[winner][d];
              }
            }
            settings_update(c, 1, acc, b1);
          }
        } else if (lane == 0) {
          settings_update(c, 1, 0, b1);
          M.d[0] = M.d[1] = M.d[2] = M.d[3] = 0.0;
        }
      } else if (kind == GEMC_VOLUME) {
        double en0 = M.tot[0], en1 = M.tot[1];
        double coeff = 1.0;
        const int bp[2] = {b, b1};
        for (int i = 0; i < 2; ++i) {
          int bb = bp[i];
          coeff *= pow(M.nvol[bb] / c.vol[bb], (double)count_of(c, n, bb));
        }
        double tNew = (0.0 + en0) + en1;
        double tRef = (0.0 + c.e[0]) + c.e[1];
        double uBoltz = exp(-p.beta * (tNew - tRef));
        acc = M.u_acc < coeff * uBoltz;
        if (lane == 0) {
          M.d[0] = en0;
          M.d[1] = en1;
          M.d[2] = M.d[3] = 0.0;
          settings_update(c, 2, acc, b);
          settings_update(c, 2, acc, b1);
        }
      }
      if (lane == 0) {
        S.accept = acc;
        c.mt_left = R.left;
        c.mt_next = R.next;
      }
    }
    __syncthreads();
    mark(pslot, 3);
    // ---------------- commit ----------------
    const int acc = S.accept;
    if (acc && kind == GEMC_TRANSFER) {
      // MoleculeLookup::Shift needs the molecule's slot in its box's
      // section of the lookup: the threads scan it together (the molecule
      // appears once)
      const int a0 = first_of(c, b), nb = count_of(c, n, b);
      for (int i = tid; i < nb; i += GEMC_THREADS)
        if (A.lookup[a0 + i] == m)
          S.slot = a0 + i;
      __syncthreads();
    }
    if (acc && (kind == GEMC_DISPLACE || kind == GEMC_TRANSFER)) {
      if (tid == 0) {
        A.px[m] = M.np[0];
        A.py[m] = M.np[1];
        A.pz[m] = M.np[2];
        if (!MIXED) {
          A.fx[m] = M.nf[0];
          A.fy[m] = M.nf[1];
          A.fz[m] = M.nf[2];
        } else {
          A.tx[m] = M.nt[0];
          A.ty[m] = M.nt[1];
          A.tz[m] = M.nt[2];
        }
        if (kind == GEMC_DISPLACE) {
          // the centre: below, by the lanes that loaded it
        } else {
          // COM::SetNew of one atom; MoleculeLookup::Shift
          if (rank == 0) {
            p.cx[m] = wrapd(M.np[0] * (1.0 / 1.0), c.ax[b1][0]);
            p.cy[m] = wrapd(M.np[1] * (1.0 / 1.0), c.ax[b1][1]);
            p.cz[m] = wrapd(M.np[2] * (1.0 / 1.0), c.ax[b1][2]);
          }
          const int idx = S.slot;
          int ni = b == 0 ? --c.start1 : c.start1++;
          int tmp = A.lookup[idx];
          A.lookup[idx] = A.lookup[ni];
          A.lookup[ni] = tmp;
          int left = count_of(c, n, b);
          if (left == 0 || left == 1)
            c.e[b] = 0.0;
        }
      }
    }
    if (acc && kind == GEMC_DISPLACE && rank == 0 && warp == 0 && lane < 3) {
      double *cc = lane == 0 ? p.cx : lane == 1 ? p.cy : p.cz;
      cc[m] = wrapd(cpend + M.sh[lane], c.ax[b][lane]);
    }
    if (acc && kind == GEMC_VOLUME) {
      // new positions, centres and axes
      for (int i = tid; i < n; i += GEMC_THREADS) {
        int j = A.lookup[i];
        int bb = i < c.start1 ? 0 : 1;
        A.px[j] = A.qx[j];
        A.py[j] = A.qy[j];
        A.pz[j] = A.qz[j];
        if (!MIXED) {
          A.fx[j] = (float)A.qx[j];
          A.fy[j] = (float)A.qy[j];
          A.fz[j] = (float)A.qz[j];
        } else {
          A.tx[j] = A.ux[j];
          A.ty[j] = A.uy[j];
          A.tz[j] = A.uz[j];
        }
        if (rank == 0) {
          p.cx[j] = p.cx[j] * M.sc[bb][0];
          p.cy[j] = p.cy[j] * M.sc[bb][1];
          p.cz[j] = p.cz[j] * M.sc[bb][2];
        }
      }
      __syncthreads();
      if (tid == 0) {
        c.e[0] = M.tot[0];
        c.e[1] = M.tot[1];
        for (int bb = 0; bb < 2; ++bb) {
          for (int d = 0; d < 3; ++d) {
            c.ax[bb][d] = M.nax[bb][d];
            c.half[bb][d] = M.nhalf[bb][d];
          }
          c.vol[bb] = M.nvol[bb];
          c.volInv[bb] = M.nvolInv[bb];
        }
        box_consts(S, p.rcut);
      }
    }
    if (rank == 0 && tid == 0 && p.tr_i) {
      int *ti = p.tr_i + 5 * (size_t)t;
      double *td = p.tr_d + 8 * (size_t)t;
      ti[0] = kind;
      ti[1] = b;
      ti[2] = kind == GEMC_VOLUME ? -1 : m;
      ti[3] = acc;
      ti[4] = c.start1;
      for (int k = 0; k < 4; ++k)
        td[k] = M.d[k];
      td[4] = c.e[0];
      td[5] = c.e[1];
      td[6] = c.vol[0];
      td[7] = c.vol[1];
    }
    __syncthreads();
    mark(pslot, 4);
    if (prof && pslot >= 0)
      pcnt[pslot]++;
  }
  if (prof) {
    for (int k = 0; k < 3; ++k) {
      for (int ph = 0; ph < 5; ++ph)
        p.prof[5 * k + ph] += pacc[k][ph];
      p.prof[15 + k] += pcnt[k];
    }
  }
  // ---- write the state back (CTA 0) ----
  __syncthreads();
  if (rank == 0) {
    for (int i = tid; i < n; i += GEMC_THREADS) {
      p.x[i] = A.px[i];
      p.y[i] = A.py[i];
      p.z[i] = A.pz[i];
    }
    for (int i = tid; i < n; i += GEMC_THREADS)
      p.lookup[i] = A.lookup[i];
    const unsigned *src = (const unsigned *)&S.c;
    unsigned *dst = (unsigned *)p.ctl;
    for (int i = tid; i < (int)(sizeof(GemcCtl) / 4); i += GEMC_THREADS)
      dst[i] = src[i];
  }
  cluster.sync();  // no CTA leaves while another may read its shared memory
}

// BoxInter of both boxes from the FP64 masters (the periodic check of the
// running energies): one CTA per pair tile row block, partials in order.
__global__ void __launch_bounds__(256)
    k_gemc_box_energy(const GemcParams p, double *part) {
  const GemcCtl &c = *p.ctl;
  int bb = blockIdx.y;
  int a0 = bb == 0 ? 0 : c.start1;
  int nb = bb == 0 ? c.start1 : p.n - c.start1;
  double acc = 0.0;
  for (int i = blockIdx.x; i < nb; i += gridDim.x) {
    int pi = p.lookup[a0 + i];
    for (int jj = i + 1 + threadIdx.x; jj < nb; jj += blockDim.x) {
      int pj = p.lookup[a0 + jj];
      double ex = mimg(p.x[pi] - p.x[pj], c.ax[bb][0], c.half[bb][0]);
      double ey = mimg(p.y[pi] - p.y[pj], c.ax[bb][1], c.half[bb][1]);
      double ez = mimg(p.z[pi] - p.z[pj], c.ax[bb][2], c.half[bb][2]);
      double d2 = ex * ex + ey * ey + ez * ez;
      if (d2 < p.rcutSq)
        acc += lj64(p, d2);
    }
  }
  __shared__ double red[8];
  double s = block_sum<256>(acc, red);
  if (threadIdx.x == 0)
    part[bb * gridDim.x + blockIdx.x] = s;
}

__global__ void k_gemc_sum(const double *part, int nblk, double *out) {
  int bb = threadIdx.x;
  if (bb < 2) {
    double s = 0.0;
    for (int i = 0; i < nblk; ++i)
      s += part[bb * nblk + i];
    out[bb] = s;
  }
}

template <bool MIXED>
void gemc_attrs(size_t smem) {
  static std::mutex mu;
  static size_t set = 0;
  std::lock_guard<std::mutex> g(mu);
  if (smem > set) {
    cudaFuncSetAttribute(k_gemc<MIXED>,
                         cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (cudaFuncSetAttribute(k_gemc<MIXED>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) == cudaSuccess)
      set = smem;
    cudaGetLastError();
  }
}

}  // namespace

size_t gemc_smem(int n, int mixed) {
  size_t head = (sizeof(GemcShared) + 15) / 16 * 16;
  size_t lk = ((size_t)n * 4 + 15) / 16 * 16;
  size_t per = 6 * sizeof(double) +
               (mixed ? 6 * sizeof(unsigned) : 3 * sizeof(float));
  return head + lk + per * (size_t)n;
}

int gemc_launch(Gemc &g, int nsteps, cudaEvent_t e0, cudaEvent_t e1) {
  g.p.nsteps = nsteps;
  const bool mixed = g.precision == GB_MIXED;
  if (mixed)
    gemc_attrs<true>(g.smem);
  else
    gemc_attrs<false>(g.smem);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(g.cluster);
  cfg.blockDim = dim3(GEMC_THREADS);
  cfg.dynamicSmemBytes = g.smem;
  cfg.stream = g.stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = g.cluster;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if (e0)
    cudaEventRecord(e0, g.stream);
  cudaError_t e = mixed ? cudaLaunchKernelEx(&cfg, k_gemc<true>, g.p)
                        : cudaLaunchKernelEx(&cfg, k_gemc<false>, g.p);
  if (e1)
    cudaEventRecord(e1, g.stream);
  return g.CudaCheck(e, "GEMC chain launch");
}

int gemc_recompute(Gemc &g, double *e2) {
  const int nblk = 304;
  int rc = OK;
  if (!g.d_tot) {
    void *q = nullptr;
    if ((rc = g.CudaCheck(cudaMalloc(&q, (2 * nblk + 2) * sizeof(double)),
                          "cudaMalloc")))
      return rc;
    g.allocs.push_back(q);
    g.d_tot = (double *)q;
  }
  k_gemc_box_energy<<<dim3(nblk, 2), 256, 0, g.stream>>>(g.p, g.d_tot);
  k_gemc_sum<<<1, 32, 0, g.stream>>>(g.d_tot, nblk, g.d_tot + 2 * nblk);
  if ((rc = g.CudaCheck(cudaGetLastError(), "GEMC recompute")) ||
      (rc = g.CudaCheck(cudaMemcpyAsync(e2, g.d_tot + 2 * nblk,
                                        2 * sizeof(double),
                                        cudaMemcpyDeviceToHost, g.stream),
                        "download")) ||
      (rc = g.CudaCheck(cudaStreamSynchronize(g.stream), "sync")))
    return rc;
  return OK;
}

}  // namespace gb

// ===========================================================================
// Host side and C ABI
// ===========================================================================
#include "gb_mc.h"  // MT19937

struct gb_gemc {
  gb::Gemc g;
};

namespace {
thread_local std::string g_gemc_create_error;

int gemc_fail_create(int code, const char *msg) {
  g_gemc_create_error = msg;
  return code;
}

template <class T>
int gemc_alloc(gb::Gemc &g, T **p, size_t n) {
  void *q = nullptr;
  cudaError_t e = cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T));
  if (e != cudaSuccess)
    return g.CudaCheck(e, "cudaMalloc");
  g.allocs.push_back(q);
  *p = (T *)q;
  return gb::OK;
}

void gemc_free(gb::Gemc &g) {
  if (g.stream)
    cudaStreamSynchronize(g.stream);
  for (void *p : g.allocs)
    cudaFree(p);
  g.allocs.clear();
  if (g.stream)
    cudaStreamDestroy(g.stream);
  g.stream = nullptr;
}

inline double host_wrap(double v, double ax) {
  if (v >= ax)
    v -= ax;
  else if (v < 0)
    v += ax;
  return v;
}
}  // namespace

extern "C" {

int gb_gemc_create(const gb_gemc_desc *d, const gb_gemc_config *cfg,
                   gb_gemc **out) {
  using namespace gb;
  if (!d || !cfg || !out || (d->n0 > 0 && !d->pos0) ||
      (d->n1 > 0 && !d->pos1))
    return gemc_fail_create(ERR_ARG, "null argument");
  const int n = d->n0 + d->n1;
  if (d->n0 < 0 || d->n1 < 0 || n <= 0)
    return gemc_fail_create(ERR_ARG, "molecule counts out of range");
  for (int k = 0; k < 3; ++k)
    if (!(d->box0[k] > 0) || !(d->box1[k] > 0))
      return gemc_fail_create(ERR_ARG, "box edges must be positive");
  if (!(cfg->rcut > 0) || !(cfg->temperature > 0) || !(d->sigma > 0) ||
      !(d->epsilon >= 0) || !(d->n_mie > 6))
    return gemc_fail_create(ERR_ARG,
                            "Rcut, Temperature and the Mie parameters must "
                            "be positive (exponent above 6)");
  if (cfg->cbmc_first < 1 || cfg->cbmc_first > GEMC_NTMAX)
    return gemc_fail_create(ERR_UNSUPPORTED,
                            "CBMC_First must lie in 1..16 on this engine");
  if (cfg->adj_steps < 1)
    return gemc_fail_create(ERR_ARG, "AdjSteps must be positive");
  double ftot = cfg->frac[0] + cfg->frac[1] + cfg->frac[2];
  if (!(cfg->frac[0] >= 0 && cfg->frac[1] >= 0 && cfg->frac[2] >= 0 &&
        ftot > 0))
    return gemc_fail_create(ERR_ARG, "move frequencies must not be negative");
  int csize = cfg->cluster_size ? cfg->cluster_size : 16;
  if (csize != 1 && csize != 2 && csize != 4 && csize != 8 && csize != 16)
    return gemc_fail_create(ERR_ARG, "cluster size must be 1, 2, 4, 8 or 16");
  if (cfg->precision != GB_FP64 && cfg->precision != GB_MIXED)
    return gemc_fail_create(ERR_ARG, "precision must be GB_FP64 or GB_MIXED");

  gb_gemc *h = new gb_gemc();
  Gemc &g = h->g;
  g.device = cfg->device;
  g.precision = cfg->precision;
  g.cluster = csize;
  int rc;
  auto fail = [&](int code) {
    g_gemc_create_error = g.last_error;
    gemc_free(g);
    delete h;
    return code;
  };
  if ((rc = g.CudaCheck(cudaSetDevice(g.device), "cudaSetDevice")))
    return fail(rc);
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin,
                         g.device);
  g.smem = gemc_smem(n, g.precision == GB_MIXED);
  if ((int)g.smem > optin) {
    g.last_error = "both boxes do not fit one CTA's shared memory (" +
                   std::to_string(g.smem) + " bytes)";
    return fail(ERR_UNSUPPORTED);
  }
  if ((rc = g.CudaCheck(cudaStreamCreateWithFlags(&g.stream,
                                                  cudaStreamNonBlocking),
                        "stream")))
    return fail(rc);

  // System::Init for two boxes: coordinates wrapped, centres of one-atom
  // molecules, the molecule lookup of box 0 then box 1
  std::vector<double> x(n), y(n), z(n), cx(n), cy(n), cz(n);
  std::vector<int> lookup(n);
  GemcCtl &c = g.h_ctl;
  std::memset(&c, 0, sizeof c);
  for (int k = 0; k < 3; ++k) {
    c.ax[0][k] = d->box0[k];
    c.ax[1][k] = d->box1[k];
    c.half[0][k] = d->box0[k] * 0.5;
    c.half[1][k] = d->box1[k] * 0.5;
  }
  for (int b = 0; b < 2; ++b) {
    c.vol[b] = c.ax[b][0] * c.ax[b][1] * c.ax[b][2];
    c.volInv[b] = 1.0 / c.vol[b];
    c.minVol[b] = 8.0 * (cfg->rcut * cfg->rcut) * cfg->rcut + 0.001;
  }
  for (int i = 0; i < n; ++i) {
    const double *q = i < d->n0 ? d->pos0 + 3 * i : d->pos1 + 3 * (i - d->n0);
    int b = i < d->n0 ? 0 : 1;
    x[i] = host_wrap(q[0], c.ax[b][0]);
    y[i] = host_wrap(q[1], c.ax[b][1]);
    z[i] = host_wrap(q[2], c.ax[b][2]);
    if (!(x[i] >= 0 && x[i] <= c.ax[b][0] && y[i] >= 0 &&
          y[i] <= c.ax[b][1] && z[i] >= 0 && z[i] <= c.ax[b][2])) {
      g.last_error = "a particle lies outside its box after wrapping";
      return fail(ERR_ARG);
    }
    cx[i] = host_wrap(x[i] * (1.0 / 1.0), c.ax[b][0]);
    cy[i] = host_wrap(y[i] * (1.0 / 1.0), c.ax[b][1]);
    cz[i] = host_wrap(z[i] * (1.0 / 1.0), c.ax[b][2]);
    lookup[i] = i;
  }
  c.start1 = d->n0;
  // MoveSettings::Init: the displacement scale reads the axes before they
  // are set (0), rotation pi/4, volume exchange 500 A^3
  for (int b = 0; b < 2; ++b) {
    c.scale[b][0] = 0.0 * 0.25;
    c.scale[b][1] = M_PI_4;
    c.scale[b][2] = 500;
  }
  MT19937 mt(cfg->seed);
  int32_t left = 0, next = 0;
  mt.Save(c.mt, &left, &next);
  c.mt_left = left;
  c.mt_next = next;

  GemcParams &p = g.p;
  p.n = n;
  p.nt = cfg->cbmc_first;
  p.adj = cfg->adj_steps;
  p.cluster = csize;
  // StaticVals::InitMovePercents over the GEMC move kinds
  double raw[GEMC_KINDS] = {0};
  raw[GEMC_DISPLACE] = cfg->frac[0];
  raw[GEMC_VOLUME] = cfg->frac[1];
  raw[GEMC_TRANSFER] = cfg->frac[2];
  double tot = 0.0;
  for (int k = 0; k < GEMC_KINDS; ++k)
    tot += raw[k];
  for (int k = 0; k < GEMC_KINDS; ++k)
    p.perc[k] = raw[k] / tot;
  // the running sums PRNG::PickArbDist forms (src/PRNG.h:153-163), in its
  // order of additions
  {
    double sum = 0.0;
    for (int k = 0; k < GEMC_KINDS; ++k) {
      sum += p.perc[k];
      p.cum[k] = sum;
      p.boxdiv[k] = p.perc[k] / 2;
    }
  }
  // FFParticle::Blend for one kind
  const double nm = d->n_mie;
  const double cn = nm / (nm - 6.0) * std::pow(nm / 6.0, (6.0 / (nm - 6.0)));
  p.nexp = nm;
  p.sigmaSq = d->sigma * d->sigma;
  p.eps_cn = cn * std::sqrt(d->epsilon * d->epsilon);
  p.rcut = cfg->rcut;
  p.rcutSq = cfg->rcut * cfg->rcut;
  p.rcutLowSq = cfg->rcut_low * cfg->rcut_low;
  p.beta = 1 / cfg->temperature;
  p.sigmaSq_f = (float)p.sigmaSq;
  p.rcutLowSq_f = (float)p.rcutLowSq;
  p.eps_cn_f = (float)p.eps_cn;
  // the FP32 distance pre-filter of the plain form passes every pair within
  // Rcut: FP32 copies of positions lie within L 2^-24 of the FP64 ones
  double lmax = std::max(std::max(c.ax[0][0], c.ax[0][1]),
                         std::max(c.ax[1][0], c.ax[1][2]));
  double rpad = cfg->rcut + 1e-5 * lmax + 1e-4;
  p.rcutSq_f = g.precision == GB_MIXED ? (float)p.rcutSq
                                       : (float)(rpad * rpad);
  if ((rc = gemc_alloc(g, &p.x, n)) || (rc = gemc_alloc(g, &p.y, n)) ||
      (rc = gemc_alloc(g, &p.z, n)) || (rc = gemc_alloc(g, &p.cx, n)) ||
      (rc = gemc_alloc(g, &p.cy, n)) || (rc = gemc_alloc(g, &p.cz, n)) ||
      (rc = gemc_alloc(g, &p.lookup, n)) || (rc = gemc_alloc(g, &p.ctl, 1)))
    return fail(rc);
  auto up = [&](void *dst, const void *src, size_t bytes) {
    return g.CudaCheck(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice,
                                       g.stream),
                       "upload");
  };
  if ((rc = up(p.x, x.data(), n * 8)) || (rc = up(p.y, y.data(), n * 8)) ||
      (rc = up(p.z, z.data(), n * 8)) || (rc = up(p.cx, cx.data(), n * 8)) ||
      (rc = up(p.cy, cy.data(), n * 8)) || (rc = up(p.cz, cz.data(), n * 8)) ||
      (rc = up(p.lookup, lookup.data(), n * 4)) ||
      (rc = up(p.ctl, &c, sizeof c)))
    return fail(rc);
  // initial energies (System::Init -> SystemTotal), FP64
  double e2[2];
  if ((rc = gemc_recompute(g, e2)))
    return fail(rc);
  c.e[0] = e2[0];
  c.e[1] = e2[1];
  if ((rc = up(p.ctl, &c, sizeof c)) ||
      (rc = g.CudaCheck(cudaStreamSynchronize(g.stream), "sync")))
    return fail(rc);
  *out = h;
  return OK;
}

void gb_gemc_destroy(gb_gemc *h) {
  if (!h)
    return;
  gemc_free(h->g);
  delete h;
}

const char *gb_gemc_error(const gb_gemc *h) {
  if (!h)
    return g_gemc_create_error.c_str();
  return h->g.last_error.c_str();
}

int gb_gemc_run(gb_gemc *h, int64_t first_step, int64_t nsteps,
                int32_t *trace_i5, double *trace_d8) {
  using namespace gb;
  if (!h)
    return ERR_ARG;
  Gemc &g = h->g;
  if (nsteps < 0 || nsteps > (int64_t)1 << 30)
    return g.Fail(ERR_ARG, "step count out of range");
  if (first_step != g.next_step)
    return g.Fail(ERR_STATE, "steps must continue from the last one run");
  if (g.h_ctl.err)
    return g.Fail(ERR_STATE, "an earlier run stopped on an invalid volume");
  if (nsteps == 0)
    return OK;
  int rc;
  cudaSetDevice(g.device);
  const bool trace = trace_i5 || trace_d8;
  if (trace && (size_t)nsteps > g.trace_cap) {
    if ((rc = gemc_alloc(g, &g.d_tr_i, 5 * (size_t)nsteps)) ||
        (rc = gemc_alloc(g, &g.d_tr_d, 8 * (size_t)nsteps)))
      return rc;
    g.trace_cap = (size_t)nsteps;
  }
  g.p.tr_i = trace ? g.d_tr_i : nullptr;
  g.p.tr_d = trace ? g.d_tr_d : nullptr;
  g.p.prof = g.profile ? g.d_prof : nullptr;
  g.p.first = first_step;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  rc = gemc_launch(g, (int)nsteps, e0, e1);
  if (!rc)
    rc = g.CudaCheck(cudaMemcpyAsync(&g.h_ctl, g.p.ctl, sizeof(GemcCtl),
                                     cudaMemcpyDeviceToHost, g.stream),
                     "download");
  if (!rc && trace_i5)
    rc = g.CudaCheck(cudaMemcpyAsync(trace_i5, g.d_tr_i,
                                     5 * sizeof(int32_t) * (size_t)nsteps,
                                     cudaMemcpyDeviceToHost, g.stream),
                     "download");
  if (!rc && trace_d8)
    rc = g.CudaCheck(cudaMemcpyAsync(trace_d8, g.d_tr_d,
                                     8 * sizeof(double) * (size_t)nsteps,
                                     cudaMemcpyDeviceToHost, g.stream),
                     "download");
  if (!rc)
    rc = g.CudaCheck(cudaStreamSynchronize(g.stream), "GEMC run");
  if (!rc)
    cudaEventElapsedTime(&g.last_ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc)
    return rc;
  if (g.h_ctl.err)
    return g.Fail(ERR_STATE,
                  "a volume exchange would shrink a box below 2 Rcut (the "
                  "reference stops its run there)");
  g.next_step += nsteps;
  return OK;
}

int gb_gemc_state(gb_gemc *h, double *energy2, double *edges6,
                  int32_t *n_box0, double *scales4, int64_t *counts12,
                  double *last_ms) {
  if (!h)
    return gb::ERR_ARG;
  const gb::GemcCtl &c = h->g.h_ctl;
  for (int b = 0; b < 2; ++b) {
    if (energy2)
      energy2[b] = c.e[b];
    if (edges6)
      for (int d = 0; d < 3; ++d)
        edges6[3 * b + d] = c.ax[b][d];
    if (scales4) {
      scales4[2 * b] = c.scale[b][0];
      scales4[2 * b + 1] = c.scale[b][2];
    }
    if (counts12)
      for (int k = 0; k < 3; ++k) {
        counts12[6 * b + 2 * k] = c.tries[b][k];
        counts12[6 * b + 2 * k + 1] = c.acc[b][k];
      }
  }
  if (n_box0)
    *n_box0 = c.start1;
  if (last_ms)
    *last_ms = h->g.last_ms;
  return gb::OK;
}

int gb_gemc_coords(gb_gemc *h, double *xyz, double *com, int32_t *lookup) {
  if (!h)
    return gb::ERR_ARG;
  gb::Gemc &g = h->g;
  const int n = g.p.n;
  std::vector<double> t(6 * (size_t)n);
  double *src[6] = {g.p.x, g.p.y, g.p.z, g.p.cx, g.p.cy, g.p.cz};
  int rc;
  for (int k = 0; k < 6; ++k)
    if ((rc = g.CudaCheck(cudaMemcpyAsync(t.data() + (size_t)k * n, src[k],
                                          (size_t)n * 8,
                                          cudaMemcpyDeviceToHost, g.stream),
                          "download")))
      return rc;
  if (lookup && (rc = g.CudaCheck(cudaMemcpyAsync(lookup, g.p.lookup,
                                                  (size_t)n * 4,
                                                  cudaMemcpyDeviceToHost,
                                                  g.stream),
                                  "download")))
    return rc;
  if ((rc = g.CudaCheck(cudaStreamSynchronize(g.stream), "sync")))
    return rc;
  for (int i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d) {
      if (xyz)
        xyz[3 * i + d] = t[(size_t)d * n + i];
      if (com)
        com[3 * i + d] = t[(size_t)(3 + d) * n + i];
    }
  return gb::OK;
}

int gb_gemc_profile(gb_gemc *h, int32_t enable, double *us15,
                    int64_t *moves3) {
  using namespace gb;
  if (!h)
    return ERR_ARG;
  Gemc &g = h->g;
  int rc;
  cudaSetDevice(g.device);
  if (!g.d_prof) {
    if ((rc = gemc_alloc(g, &g.d_prof, 18)) ||
        (rc = g.CudaCheck(cudaMemsetAsync(g.d_prof, 0, 18 * sizeof(long long),
                                          g.stream),
                          "memset")))
      return rc;
  }
  long long hp[18];
  if ((rc = g.CudaCheck(cudaMemcpyAsync(hp, g.d_prof, sizeof hp,
                                        cudaMemcpyDeviceToHost, g.stream),
                        "download")) ||
      (rc = g.CudaCheck(cudaMemsetAsync(g.d_prof, 0, sizeof hp, g.stream),
                        "memset")) ||
      (rc = g.CudaCheck(cudaStreamSynchronize(g.stream), "sync")))
    return rc;
  int khz = 0;
  cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, g.device);
  for (int k = 0; k < 15; ++k)
    if (us15)
      us15[k] = khz > 0 ? (double)hp[k] / (khz * 1e-3) : 0.0;
  for (int k = 0; k < 3; ++k)
    if (moves3)
      moves3[k] = hp[15 + k];
  g.profile = enable != 0;
  return OK;
}

int gb_gemc_system_total(gb_gemc *h, double *energy2) {
  if (!h || !energy2)
    return gb::ERR_ARG;
  cudaSetDevice(h->g.device);
  return gb::gemc_recompute(h->g, energy2);
}

}  // extern "C"
