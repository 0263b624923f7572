// Mixed-precision chain kernel: one thread-block cluster runs one Markov
// chain, many chains per launch.
//
// Per move, every CTA of the cluster:
//   * builds the move header (FP64 old/new positions, exact cell indices,
//     32-bit fixed-point turns, the midpoint p = (r + r')/2 and the half step
//     h = (r' - r)/2 of every atom) and per-axis phase rows exp(2 pi i n p/L)
//     from the exact fixed-point phase;
//   * evaluates its share of the real-space (atom, old/new, neighbour cell)
//     units in FP32 from fixed-point coordinates -- the minimum image is the
//     wrapped 32-bit difference -- with an exact FP64 decision for pairs whose
//     r^2 lies within 1e-5 of the cutoff;
//   * evaluates its chunk of k-vectors with
//       exp(i k.r') - exp(i k.r) = 2i sin(k.h) exp(i k.p),
//     which keeps the structure-factor change accurate relative to itself,
//     and dE_k = prefact (2 S.dS + |dS|^2) against its resident accumulators;
//   * exchanges its partial sums through distributed shared memory; after a
//     cluster barrier every CTA adds the partials in one order, takes the
//     same Metropolis decision (FP64 exponent against log u) and, on accept,
//     folds dS into its accumulators.
// Structure factors are float-float accumulators (an FP32 value and its
// FP32 remainder, about 48 bits) in shared memory, updated by an error-free
// sum on every accepted move; they are read from and written back to the
// box's FP64 arrays at launch boundaries.  Running energies are FP64.
#include "gb_cells.cuh"
#include "gb_f32math.cuh"
#include "gb_mc.h"
#include "gb_moves.cuh"
#include "gb_pair.cuh"

#include <cooperative_groups.h>
#include <mutex>

namespace cg = cooperative_groups;

namespace gb {

constexpr int MT_THREADS = 256;  // threads per CTA
constexpr int MAXA = MAX_MOL_ATOMS;

struct MHdr {
  int m, kind, na, a0;
  double lpacc;
  double oldp[MAXA][3], newp[MAXA][3], newcom[3];
  int cell_old[MAXA], cell_new[MAXA];
  uint32_t uo[MAXA][3], un[MAXA][3], P[MAXA][3];
  float hf[MAXA][3];
  float qf[MAXA], qflo[MAXA];  // charge (structure factors) and remainder
  float qs[MAXA], qslo[MAXA];  // q * SQRT_QQ_FACT: FP32 value and remainder
  int ka[MAXA];
};

// Inputs of the next move's header that warp 7 loaded during the current
// move (its record, atom range, proposal, centre, positions, charges).
struct MPre {
  int m, kind, a0, na;
  double lpacc;
  double prop[12], com[3], oldp[MAXA][3], q[MAXA];
  int ka[MAXA];
};

struct MShared {
  MHdr hh[2];  // this move's header and the next one's, by move parity
  MPre pre;
  Settings set;
  double e_run[5];
  double part[4];        // this CTA's partial: LJ, real, recip, overlap
  double tot[4];
  double wred[MT_THREADS / 32][4];
  double prop[12];
  int accept;
};

// Byte offsets of the per-CTA k-chunk arrays.  The structure factor of each
// k-vector is held in float-float: s32 (its FP32 value, read by every move)
// plus lo (the remainder), updated on every accepted move by an error-free
// sum and renormalised, so it carries about 48 bits without FP64 storage.
// The arrays read by every move (s32R/I, this move's changes dR/dI,
// prefactors pf, integer k) always live in dynamic shared memory, 24 B per
// k-vector; the remainders loR/I (8 B, touched on accept) follow them when
// the chunk fits, else they sit in a per-chain global buffer with the same
// offsets.  Every array starts on a 16-byte boundary whatever the chunk
// length.
struct MixedLayout {
  size_t kcs;   // padded chunk length (multiple of 4)
  size_t cold;  // offset of the remainders (in shared memory or the buffer)
  size_t tab;   // offset of the phase rows in shared memory
};
__host__ __device__ __forceinline__ MixedLayout mixed_layout(int kc_max,
                                                             bool cold_smem) {
  MixedLayout L;
  L.kcs = ((size_t)kc_max + 3) & ~(size_t)3;
  L.cold = 24 * L.kcs;
  L.tab = cold_smem ? L.cold + 8 * L.kcs : L.cold;
  return L;
}
__host__ __device__ __forceinline__ size_t mixed_cold_bytes(int kc_max) {
  return 8 * (((size_t)kc_max + 3) & ~(size_t)3);
}

// Whether cells c1 and c2 are in one another's 27-cell neighbourhood (every
// axis has at least 3 cells, src/CellList.cpp:138-161).
__device__ __forceinline__ bool cells_adjacent(const DevBox &b, int c1, int c2) {
  const int e1 = b.edge[1], e2 = b.edge[2];
  int d[3] = {c2 / (e1 * e2) - c1 / (e1 * e2), (c2 / e2) % e1 - (c1 / e2) % e1,
              c2 % e2 - c1 % e2};
  bool ok = true;
  for (int i = 0; i < 3; ++i) {
    int v = d[i] < 0 ? -d[i] : d[i];
    ok = ok && (v <= 1 || v == b.edge[i] - 1);
  }
  return ok;
}

// Ewald bracket erfc(a r')/r' - erfc(a r)/r of a far pair (alpha r >= 2 at
// both positions) from the FP32 distances: the FP32 erfc form with the
// first-order corrections for the FP32 turn length and alpha_f (coul_da;
// the charge factor carries the 1 / (1 + eta) part).  Cheaper than
// far_coulomb; at these distances its amplified argument rounding is below
// the error of the near-cutoff terms.
__device__ __forceinline__ float fp32_bracket(float r2o, float r2n, float dr2,
                                              float alpha, float coul_da) {
  float ro = sqrtf(r2o), rn = sqrtf(r2n);
  float inv_o = 1.0f / ro, inv_n = 1.0f / rn, sum_r = ro + rn;
  float dinv = -dr2 * inv_o * inv_n / sum_r;  // 1/rn - 1/ro
  float tlo = alpha * ro, thi = alpha * rn;
  float dt = alpha * dr2 / sum_r;             // thi - tlo
  float derfc, dal;
  if (fabsf(dt) < 0.25f) {
    // 3-point Gauss-Legendre of (2/sqrt pi) exp(-t^2) over [tlo, thi], the
    // weights times 2/sqrt(pi) as FP32 hi + lo pairs
    float tm = 0.5f * (tlo + thi), hw = 0.5f * dt;
    float t1 = fmaf(-0.774596669f, hw, tm), t3 = fmaf(0.774596669f, hw, tm);
    float em = expf(-tm * tm), e13 = expf(-t1 * t1) + expf(-t3 * t3);
    float g = fmaf(1.00300372f, em, 0.626877308f * e13) +
              fmaf(-1.23839108e-8f, em, 7.16121695e-9f * e13);
    derfc = -hw * g;
    // exp(-tn^2) - exp(-to^2) = -2 tm dt exp(-tm^2) + O(dt^3)
    dal = 2.0f * coul_da * tm * dt * em;
  } else {
    derfc = erfc_f32(thi) - erfc_f32(tlo);
    dal = -coul_da * (expf(-thi * thi) - expf(-tlo * tlo));
  }
  return fmaf(erfc_f32(thi), dinv, derfc * inv_o) + dal;
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 tabf(const float2 *row, int n) {
  float2 v = row[n < 0 ? -n : n];
  if (n < 0)
    v.y = -v.y;
  return v;
}

// Header of move t into h (all threads of the CTA call it); prev is the
// previous move's header, whose new positions are the current ones when
// that move was accepted and touched the same molecule.
// With `pre`, the inputs come from warp 7's loads (S.pre) instead of
// global memory.
__device__ void mixed_header(const MixedChain &C, MShared &S, int t,
                             bool prev_acc, int prev_m, int prev_kind,
                             const MHdr &prev, MHdr &h, bool pre = false) {
  const DevBox &b = C.b;
  const MoveRec &r = C.moves[t];
  const MPre &P = S.pre;
  int m = pre ? P.m : r.mol;
  int a0 = pre ? P.a0 : b.mstart[m];
  int na = pre ? P.na : b.mstart[m + 1] - a0;
  const int rkind = pre ? P.kind : r.kind;
  const double rlpacc = pre ? P.lpacc : r.lpacc;
  bool same = prev_acc && prev_m == m;
  // the previous header still holds that move's new positions
  __shared__ double oldp[MAXA][3], com[3];
  if (threadIdx.x < 12)
    S.prop[threadIdx.x] = pre ? P.prop[threadIdx.x]
                              : C.prop[(size_t)t * 12 + threadIdx.x];
  if (threadIdx.x < 3) {
    int d = threadIdx.x;
    const double *cs[3] = {b.cx, b.cy, b.cz};
    com[d] = (same && prev_kind == 0) ? prev.newcom[d]
             : pre                    ? P.com[d]
                                      : __ldcg(cs[d] + m);
  }
  if (threadIdx.x >= 32 && threadIdx.x < 32 + 3 * na) {
    int i = threadIdx.x - 32, a = i / 3, d = i % 3;
    const double *xs[3] = {b.x, b.y, b.z};
    oldp[a][d] = same ? prev.newp[a][d]
                 : pre ? P.oldp[a][d]
                       : __ldcg(xs[d] + a0 + a);
  }
  __syncthreads();
  if (threadIdx.x < na) {
    int a = threadIdx.x;
    double w[3];
    if (rkind == 0) {
      for (int d = 0; d < 3; ++d)
        w[d] = wrap1(__dadd_rn(oldp[a][d], S.prop[d]), b.L[d]);
    } else {
      double v[3];
      for (int d = 0; d < 3; ++d) {
        v[d] = unwrap1(oldp[a][d], com[d], b.L[d], b.half[d]);
        v[d] = __dadd_rn(v[d], -com[d]);
      }
      for (int i = 0; i < 3; ++i) {
        double u = __dadd_rn(__dadd_rn(__dmul_rn(S.prop[3 * i], v[0]),
                                       __dmul_rn(S.prop[3 * i + 1], v[1])),
                             __dmul_rn(S.prop[3 * i + 2], v[2]));
        w[i] = wrap1(__dadd_rn(u, com[i]), b.L[i]);
      }
    }
    for (int d = 0; d < 3; ++d) {
      h.oldp[a][d] = oldp[a][d];
      h.newp[a][d] = w[d];
      uint32_t uo = to_turns(oldp[a][d], b.invL[d]);
      uint32_t un = to_turns(w[d], b.invL[d]);
      int32_t D = (int32_t)(un - uo);
      h.uo[a][d] = uo;
      h.un[a][d] = un;
      h.P[a][d] = uo + (uint32_t)(D >> 1);
      float Df = (float)D;  // pi / 2^32 as FP32 hi + lo
      h.hf[a][d] = fmaf(Df, -2.03547013e-17f, Df * 7.31459060e-10f);
    }
    h.cell_old[a] = position_to_cell_fast(b, oldp[a][0], oldp[a][1], oldp[a][2]);
    h.cell_new[a] = position_to_cell_fast(b, w[0], w[1], w[2]);
    double q = pre ? P.q[a] : b.q[a0 + a];
    bool q0 = fabs(q) < 0.000000001;
    h.qf[a] = q0 ? 0.0f : (float)q;
    h.qflo[a] = q0 ? 0.0f : (float)(q - (double)(float)q);
    double qs = q * SQRT_QQ_FACT;
    h.qs[a] = q0 ? 0.0f : (float)qs;
    h.qslo[a] = q0 ? 0.0f : (float)(qs - (double)(float)qs);
    h.ka[a] = pre ? P.ka[a] : b.kind[a0 + a];
  }
  if (threadIdx.x == 64) {
    h.m = m;
    h.kind = rkind;
    h.na = na;
    h.a0 = a0;
    h.lpacc = rlpacc;
    for (int d = 0; d < 3; ++d)
      h.newcom[d] = rkind == 0 ? wrap1(__dadd_rn(com[d], S.prop[d]), b.L[d])
                               : com[d];
  }
  __syncthreads();
}

// Phase rows exp(2 pi i n P / 2^32), n = 0..kmax, for every atom and axis.
__device__ __forceinline__ void mixed_tables(const MixedChain &C,
                                             const MHdr &h, float2 *tab) {
  int stride = C.b.kmax + 1;
  int rows = 3 * h.na;
  for (int i = threadIdx.x; i < rows * stride; i += MT_THREADS) {
    int row = i / stride, n = i % stride;
    uint32_t P = h.P[row / 3][row % 3];
    tab[i] = cis_turns((uint32_t)n * P);
  }
}

__global__ void __launch_bounds__(MT_THREADS)
    k_chain_mixed(const MixedChain *__restrict__ chains) {
  cg::cluster_group cluster = cg::this_cluster();
  const int csize = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  const int chain_id = blockIdx.x / csize;
  const MixedChain &C = chains[chain_id];
  const DevBox &b = C.b;
  const FF &ff = *C.ff;
  __shared__ MShared S;
  extern __shared__ __align__(16) unsigned char dyn[];
  const int K = b.K;
  const int kc_max = (K + csize - 1) / csize;
  const int kbeg = min(K, rank * kc_max);
  const int kc = min(kc_max, K - kbeg);
  const bool cold_smem = C.cold == nullptr;
  MixedLayout L = mixed_layout(kc_max, cold_smem);
  float *s32R = (float *)dyn, *s32I = s32R + L.kcs, *dR = s32I + L.kcs,
        *dI = dR + L.kcs, *pf = dI + L.kcs;
  char4 *kn = (char4 *)(pf + L.kcs);
  unsigned char *cb = cold_smem ? dyn + L.cold
                                : C.cold + (size_t)rank * mixed_cold_bytes(kc_max);
  float *loR = (float *)cb, *loI = loR + L.kcs;
  // phase rows of this move and the next, by move parity
  float2 *const tabs = (float2 *)(dyn + L.tab);
  const size_t tab_len = (size_t)3 * MAXA * (b.kmax + 1);
  const int stride = b.kmax + 1;

  for (int i = threadIdx.x; i < kc; i += MT_THREADS) {
    int k = kbeg + i;
    double r = b.sumRref[k], im = b.sumIref[k];
    s32R[i] = (float)r;
    s32I[i] = (float)im;
    loR[i] = (float)(r - (double)s32R[i]);
    loI[i] = (float)(im - (double)s32I[i]);
    pf[i] = b.prefact_f[k];
    kn[i] = b.kn[k];
  }
  if (threadIdx.x == 0) {
    S.set = *C.set;
    for (int i = 0; i < 5; ++i)
      S.e_run[i] = b.energy[i];
  }
  __syncthreads();
  const int tpc = MT_THREADS * csize;
  const int gt = rank * MT_THREADS + threadIdx.x;
  auto make_props = [&](int t0) {
    int t1 = t0;
    while (t1 < C.n) {
      long long step = C.first + t1;
      if (t1 > t0 && (step + 1) % S.set.adj == 0)
        break;
      ++t1;
    }
    for (int t = t0 + gt; t < t1; t += tpc)
      make_proposal(C.moves[t], S.set, C.prop + (size_t)t * 12);
  };

  if (C.n > 0) {
    if (threadIdx.x == 0)
      settings_adjust(S.set, C.first);
    __syncthreads();
    make_props(0);
    cluster.sync();
    mixed_header(C, S, 0, false, -1, 0, S.hh[1], S.hh[0]);
    mixed_tables(C, S.hh[0], tabs);
    __syncthreads();
  }
  const float rc2 = (float)ff.rcutSq;
  const float rcc2 = (float)ff.rcutCoulSq;
  const float rl2 = (float)ff.rcutLowSq;
  const float alpha = ff.alpha_f;
  const float sx = (float)(b.L[0] * 2.3283064365386963e-10);  // L / 2^32
  const float sy = (float)(b.L[1] * 2.3283064365386963e-10);
  const float sz = (float)(b.L[2] * 2.3283064365386963e-10);
  const bool coul_cut = ff.rcutCoulSq < ff.rcutSq;
  const bool narrow = b.cellSize[0] * b.cellSize[0] < ff.rcutSq ||
                      b.cellSize[1] * b.cellSize[1] < ff.rcutSq ||
                      b.cellSize[2] * b.cellSize[2] < ff.rcutSq;

  // Warp 7 gathers the next move's header inputs one move ahead: the move
  // record two moves ahead, its atom range a move later, and at the start
  // of a move the proposal, centre, positions and charges of the next one,
  // so that the next header is built from registers inside the cluster
  // barrier.
  const int wid = threadIdx.x >> 5, lid = threadIdx.x & 31;
  int pa_m = -1, pa_kind = 0, pb_m = -1, pb_kind = 0, pb_a0 = 0, pb_a1 = 0;
  double pa_lp = 0.0, pb_lp = 0.0;
  auto pipe_record = [&](int t) {
    pa_m = -1;
    if (t < C.n) {
      pa_m = C.moves[t].mol;
      pa_kind = C.moves[t].kind;
      pa_lp = C.moves[t].lpacc;
    }
  };
  auto pipe_range = [&]() {
    pb_m = pa_m;
    pb_kind = pa_kind;
    pb_lp = pa_lp;
    if (pb_m >= 0) {
      pb_a0 = b.mstart[pb_m];
      pb_a1 = b.mstart[pb_m + 1];
    }
  };
  if (wid == 7) {
    pipe_record(1);
    pipe_range();
    pipe_record(2);
  }
  for (int t = 0; t < C.n; ++t) {
    const MHdr &h = S.hh[t & 1];
    // warp 7: the next move's inputs (their record and range loaded before)
    int n_m = -1, n_kind = 0, n_a0 = 0, n_na = 0;
    double n_lp = 0.0, v_prop = 0.0, v_com = 0.0, v_pos = 0.0, v_q = 0.0;
    int v_k = 0;
    if (wid == 7) {
      n_m = pb_m;
      n_kind = pb_kind;
      n_lp = pb_lp;
      n_a0 = pb_a0;
      n_na = pb_a1 - pb_a0;
      if (n_m >= 0) {
        if (lid < 12)
          v_prop = C.prop[(size_t)(t + 1) * 12 + lid];
        if (lid < 3)
          v_com = __ldcg((lid == 0 ? b.cx : lid == 1 ? b.cy : b.cz) + n_m);
        if (lid < 3 * n_na) {
          const int a = lid / 3, d = lid % 3;
          v_pos = __ldcg((d == 0 ? b.x : d == 1 ? b.y : b.z) + n_a0 + a);
        }
        if (lid < n_na) {
          v_q = b.q[n_a0 + lid];
          v_k = b.kind[n_a0 + lid];
        }
      }
      pipe_range();
      pipe_record(t + 3);
    }
    const float2 *const tab = tabs + (t & 1) * tab_len;
    const int m = h.m, na = h.na;
    // The next header does not depend on this move's outcome unless the
    // next move touches the same molecule or follows a settings adjustment:
    // then it is built during the cluster barrier before the decision.
    const bool spec = t + 1 < C.n && C.moves[t + 1].mol != m &&
                      (C.first + t + 2) % S.set.adj != 0;
    // the moved atoms' current cells and slots, for the commit of rank 0
    // (loaded now, used after the decision)
    int cur_cell = -1, cur_slot = -1;
    if (rank == 0 && threadIdx.x < na) {
      cur_cell = __ldcg(b.atom_cell + h.a0 + threadIdx.x);
      cur_slot = __ldcg(b.atom_slot + h.a0 + threadIdx.x);
    }
    // ---------------- real space ----------------
    // Each neighbour j is taken once: from the new position's cells when it
    // is inside the cutoff there (then as the difference u(r') - u(r) if it
    // was also inside before), from the old position's cells when it was
    // inside only before.  Differences use r'^2 - r^2 = delta . (d + d').
    float lj_h = 0.f, lj_l = 0.f, re_h = 0.f, re_l = 0.f, ovl = 0.f;
    const int units = na * 2 * NB27;
    // a unit's neighbour-cell slots are tiled over ul threads: slot lu,
    // lu + ul, ... of unit usub of this CTA's upc units per pass
    const int ul = 1 << C.ulog, upc = MT_THREADS >> C.ulog;
    const int lu = threadIdx.x & (ul - 1), usub = threadIdx.x >> C.ulog;
    // the units' neighbour cells and slot counts, all at once
    __shared__ int mu_c2[2 * MAXA * NB27], mu_n2[2 * MAXA * NB27];
    for (int u = threadIdx.x; u < units; u += MT_THREADS) {
      int a = u / (2 * NB27), side = (u / NB27) % 2, nn = u % NB27;
      int cell = side ? h.cell_new[a] : h.cell_old[a];
      int c2 = b.nbr[cell * NB27 + nn];
      mu_c2[u] = c2;
      mu_n2[u] = __ldcg(b.cell_count + c2);
    }
    __syncthreads();
    // one candidate: unit u against cell slot s (meta mj, fixed-point slot f)
    auto pair = [&](int u, size_t s, int mj, uint4 f) {
      if (meta_mol(mj) == m)
        return;
      const int a = u / (2 * NB27), side = (u / NB27) % 2;
      const int c2 = mu_c2[u];
      const uint32_t *uo = h.uo[a], *un = h.un[a];
      const float ddx = (float)(int32_t)(un[0] - uo[0]) * sx;
      const float ddy = (float)(int32_t)(un[1] - uo[1]) * sy;
      const float ddz = (float)(int32_t)(un[2] - uo[2]) * sz;
      const float qa = h.qs[a], qa_lo = h.qslo[a];
      const int ka = h.ka[a];
      int32_t ox = (int32_t)(uo[0] - f.x), oy = (int32_t)(uo[1] - f.y),
              oz = (int32_t)(uo[2] - f.z);
      int32_t nx_ = (int32_t)(un[0] - f.x), ny_ = (int32_t)(un[1] - f.y),
              nz_ = (int32_t)(un[2] - f.z);
      float dox = (float)ox * sx, doy = (float)oy * sy, doz = (float)oz * sz;
      float dnx = (float)nx_ * sx, dny = (float)ny_ * sy, dnz = (float)nz_ * sz;
      float r2o = fmaf(dox, dox, fmaf(doy, doy, doz * doz));
      float r2n = fmaf(dnx, dnx, fmaf(dny, dny, dnz * dnz));
      // inside-cutoff decisions, exact in FP64 within 1e-5 of the cutoff
      bool in_o = r2o < rc2, in_n = r2n < rc2;
      bool amb_o = fabsf(r2o - rc2) <= rc2 * 1e-5f;
      bool amb_n = fabsf(r2n - rc2) <= rc2 * 1e-5f;
      bool amb_l = side && r2n < rl2 * 1.00001f;
      if (side ? (!in_n && !amb_n) : (!in_o && !amb_o))
        return;
      if (amb_o || amb_n || amb_l) {
        const double *pp = (const double *)(b.cell_pos + s);
        double px = __ldcg(pp), py = __ldcg(pp + 1), pz = __ldcg(pp + 2);
        if (amb_o) {
          const double *mp = h.oldp[a];
          double d2 = dsq3(min_image(mp[0] - px, b.L[0], b.half[0]),
                           min_image(mp[1] - py, b.L[1], b.half[1]),
                           min_image(mp[2] - pz, b.L[2], b.half[2]));
          in_o = ff.rcutSq > d2;
        }
        if (amb_n || amb_l) {
          const double *mp = h.newp[a];
          double d2 = dsq3(min_image(mp[0] - px, b.L[0], b.half[0]),
                           min_image(mp[1] - py, b.L[1], b.half[1]),
                           min_image(mp[2] - pz, b.L[2], b.half[2]));
          in_n = ff.rcutSq > d2;
          if (side && in_n && d2 < ff.rcutLowSq)
            ovl = 1.f;
        }
      }
      // With cells narrower than the cutoff a pair inside it may lie
      // outside the other position's neighbourhood, where it is not summed.
      if (narrow && in_o && in_n &&
          !cells_adjacent(b, c2, side ? h.cell_old[a] : h.cell_new[a])) {
        if (side)
          in_o = false;
        else
          in_n = false;
      }
      int kj = meta_kind(mj);
      int idx = ka + kj * ff.n_kinds;
      // q_i q_j QQ_FACT / (1 + eta) = qq + qc up to FP32 rounding of the
      // remainder qc: the pair's charge product carries no systematic FP32
      // bias, and qc also takes up the FP32 turn length (FF::coul_qfac_f)
      float qb = __uint_as_float(f.w);
      float qq = qa * qb;
      bool coul = ff.electrostatic && qq != 0.f;
      float qres = 0.f, qc = 0.f;
      if (coul) {
        qres = fmaf(qa, qb, -qq) + fmaf(qa, __ldcg(b.cell_qlo + s), qa_lo * qb);
        qc = fmaf(qq, ff.coul_qfac_f, qres);
      }
      // Coulomb cutoff: the pair cutoff decision when it is the larger one
      bool cin_o = coul_cut ? r2o <= rcc2 : true;
      bool cin_n = coul_cut ? r2n <= rcc2 : true;
      float sg2 = ff.sigmaSq_f[idx], ecn = ff.eps_cn_f[idx];
      float k6 = ff.lj_k6_f[idx], k3 = ff.lj_k3_f[idx];
      if (side) {
        if (!in_n)
          return;
        if (in_o) {
          const int32_t o3[3] = {ox, oy, oz}, n3[3] = {nx_, ny_, nz_};
          if (r2o < ff.close_r2_f && r2n < ff.close_r2_f) {
            // close pair: both differences in float-float from the exact
            // squared distances, added with their rounding residuals
            ClosePair cp = close_pair(o3, n3, ff.turn2_hi, ff.turn2_lo);
            if (ecn != 0.0f) {
              ff2 du = close_lj(cp, {sg2, ff.sigmaSq_lo_f[idx]},
                                {ecn, ff.eps_cn_lo_f[idx]});
              two_sum_add(lj_h, lj_l, du.hi);
              lj_l += du.lo;
            }
            if (coul && cin_n && cin_o) {
              ff2 X = close_coulomb(cp, ff.ewald, ff.alpha2_f,
                                    {ff.alpha3_hi, ff.alpha3_lo});
              float pr = qq * X.hi;
              two_sum_add(re_h, re_l, pr);
              re_l += fmaf(qq, X.hi, -pr) + fmaf(qres, X.hi, qq * X.lo);
            }
            return;
          }
          // difference of the pair terms between r and r'
          // (d + d') in FP32: the integer sum can leave the int32 range
          float dr2 = fmaf(ddx, dox + dnx, fmaf(ddy, doy + dny, ddz * (doz + dnz)));
          float so = sg2 / r2o, sn = sg2 / r2n;
          float ds = -sg2 * dr2 / (r2o * r2n);
          float so3 = so * so * so, sn3 = sn * sn * sn;
          float d3 = ds * fmaf(sn, sn, fmaf(sn, so, so * so));
          float s33 = sn3 + so3;
          two_sum_add(lj_h, lj_l,
                      ecn * d3 * ((s33 - 1.0f) + fmaf(s33, k6, -k3)));
          if (coul && cin_n && cin_o) {
            if (ff.ewald && r2o >= ff.far_r2_f && r2n >= ff.far_r2_f) {
              float X = fp32_bracket(r2o, r2n, dr2, alpha, ff.coul_da_f);
              two_sum_add(re_h, re_l, fmaf(qq, X, qc * X));
            } else {
              // the erfc form on the exact distances (float-float r,
              // alpha r and their differences)
              ClosePair cp = close_pair(o3, n3, ff.turn2_hi, ff.turn2_lo);
              float X = ff.ewald
                            ? far_coulomb(cp, {ff.alpha_f, ff.alpha_lo_f})
                            : close_coulomb(cp, false, 0.0f, {0.0f, 0.0f}).hi;
              two_sum_add(re_h, re_l, fmaf(qq, X, qres * X));
            }
          } else if (coul) {
            if (cin_n) {
              float rr = sqrtf(r2n);
              float X = ff.ewald ? erfc_f32(alpha * rr) / rr : 1.0f / rr;
              two_sum_add(re_h, re_l, fmaf(qq, X, qc * X));
            }
            if (cin_o) {
              float rr = sqrtf(r2o);
              float X = ff.ewald ? erfc_f32(alpha * rr) / rr : 1.0f / rr;
              two_sum_add(re_h, re_l, -fmaf(qq, X, qc * X));
            }
          }
        } else {
          float rr2 = sg2 / r2n, r6 = rr2 * rr2 * rr2, r12 = r6 * r6;
          two_sum_add(lj_h, lj_l,
                      ecn * ((r12 - r6) + fmaf(r12, k6, -r6 * k3)));
          if (coul && cin_n) {
            float rr = sqrtf(r2n);
            float X = ff.ewald ? erfc_f32(alpha * rr) / rr : 1.0f / rr;
            two_sum_add(re_h, re_l, fmaf(qq, X, qc * X));
          }
        }
      } else {
        if (!in_o || in_n)
          return;  // counted from the new position's cells
        float rr2 = sg2 / r2o, r6 = rr2 * rr2 * rr2, r12 = r6 * r6;
        two_sum_add(lj_h, lj_l,
                    -ecn * ((r12 - r6) + fmaf(r12, k6, -r6 * k3)));
        if (coul && cin_o) {
          float rr = sqrtf(r2o);
          float X = ff.ewald ? erfc_f32(alpha * rr) / rr : 1.0f / rr;
          two_sum_add(re_h, re_l, -fmaf(qq, X, qc * X));
        }
      }
    };
    // This CTA takes units rank upc + usub, stepping upc csize; a thread
    // takes slot lu of its unit (and lu + ul, ... in fuller cells).  The
    // next unit's slot data are loaded while this one is evaluated.
    const int ustep = upc * csize;
    int pu = -1, pmj = 0;
    size_t ps = 0;
    uint4 pfix = make_uint4(0, 0, 0, 0);
    auto fetch = [&](int ub) {
      int u = ub + usub;
      pu = -1;
      if (u < units && lu < mu_n2[u]) {
        ps = (size_t)mu_c2[u] * b.cap + lu;
        pmj = __ldcg(b.cell_meta + ps);
        pfix = __ldcg(b.cell_fix + ps);
        pu = u;
      }
    };
    fetch(rank * upc);
    for (int ub = rank * upc; ub < units; ub += ustep) {
      const int u = pu, mj = pmj;
      const size_t s = ps;
      const uint4 f = pfix;
      if (ub + ustep < units)
        fetch(ub + ustep);
      if (u >= 0)
        pair(u, s, mj, f);
      const int uu = ub + usub;
      if (uu < units)
        for (int j = lu + ul; j < mu_n2[uu]; j += ul) {
          size_t s2 = (size_t)mu_c2[uu] * b.cap + j;
          pair(uu, s2, __ldcg(b.cell_meta + s2), __ldcg(b.cell_fix + s2));
        }
    }
    // ---------------- reciprocal space ----------------
    float de_h = 0.f, de_l = 0.f;
    for (int i = threadIdx.x; i < kc; i += MT_THREADS) {
      char4 n = kn[i];
      float fx = (float)n.x, fy = (float)n.y, fz = (float)n.z;
      float ddR = 0.f, ddI = 0.f;
      for (int a = 0; a < na; ++a) {
        float q = h.qf[a];
        if (q == 0.f)
          continue;
        float arg = fmaf(fx, h.hf[a][0], fmaf(fy, h.hf[a][1], fz * h.hf[a][2]));
        float sa = sin_f32(arg);
        float w = 2.0f * fmaf(h.qflo[a], sa, q * sa);
        const float2 *rx = tab + (size_t)(3 * a) * stride;
        float2 e = cmulf(cmulf(rx[n.x], tabf(rx + stride, n.y)),
                         tabf(rx + 2 * stride, n.z));
        ddR = fmaf(-w, e.y, ddR);
        ddI = fmaf(w, e.x, ddI);
      }
      dR[i] = ddR;
      dI[i] = ddI;
      float sr = s32R[i], si = s32I[i];
      two_sum_add(de_h, de_l, pf[i] * fmaf(2.0f * sr + ddR, ddR, (2.0f * si + ddI) * ddI));
    }
    // ---------------- reduce: warp (FP32), CTA (FP64) ----------------
    // compensated warp reduction, then FP64 across warps
    float vh[3] = {lj_h, re_h, de_h}, vl[3] = {lj_l, re_l, de_l}, v3 = ovl;
    for (int o = 16; o > 0; o >>= 1) {
      for (int c = 0; c < 3; ++c) {
        float oh = __shfl_down_sync(0xffffffffu, vh[c], o);
        float ol = __shfl_down_sync(0xffffffffu, vl[c], o);
        two_sum_add(vh[c], vl[c], oh);
        vl[c] += ol;
      }
      v3 = fmaxf(v3, __shfl_down_sync(0xffffffffu, v3, o));
    }
    int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
      for (int c = 0; c < 3; ++c)
        S.wred[w][c] = (double)vh[c] + (double)vl[c];
      S.wred[w][3] = v3;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
      int c = threadIdx.x;
      double acc = 0.0;
      for (int i = 0; i < MT_THREADS / 32; ++i)
        acc = c == 3 ? fmax(acc, S.wred[i][3]) : acc + S.wred[i][c];
      S.part[c] = acc;
    }
    // split cluster barrier: arrive with this CTA's partial, build the next
    // header meanwhile, wait before reading the other CTAs' partials
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
    if (spec) {
      if (wid == 7) {
        MPre &P = S.pre;
        if (lid == 0) {
          P.m = n_m;
          P.kind = n_kind;
          P.a0 = n_a0;
          P.na = n_na;
          P.lpacc = n_lp;
        }
        if (lid < 12)
          P.prop[lid] = v_prop;
        if (lid < 3)
          P.com[lid] = v_com;
        if (lid < 3 * n_na)
          P.oldp[lid / 3][lid % 3] = v_pos;
        if (lid < n_na) {
          P.q[lid] = v_q;
          P.ka[lid] = v_k;
        }
      }
      __syncthreads();
      mixed_header(C, S, t + 1, false, -1, 0, h, S.hh[(t + 1) & 1], true);
      mixed_tables(C, S.hh[(t + 1) & 1], tabs + ((t + 1) & 1) * tab_len);
    }
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
    // ---------------- decision (identical in every CTA) ----------------
    if (threadIdx.x < 32) {
      double p[4] = {0, 0, 0, 0};
      if ((int)threadIdx.x < csize) {
        const double *rp = cluster.map_shared_rank(S.part, (unsigned)threadIdx.x);
        for (int c = 0; c < 4; ++c)
          p[c] = rp[c];
      }
      for (int o = 16; o > 0; o >>= 1) {
        p[0] += __shfl_down_sync(0xffffffffu, p[0], o);
        p[1] += __shfl_down_sync(0xffffffffu, p[1], o);
        p[2] += __shfl_down_sync(0xffffffffu, p[2], o);
        p[3] = fmax(p[3], __shfl_down_sync(0xffffffffu, p[3], o));
      }
      if (threadIdx.x == 0) {
        bool over = p[3] > 0;
        double dLJ = p[0], dRe = p[1], dRc = over ? 0.0 : p[2];
        double ex = -ff.beta * ((dLJ + dRe) + dRc);
        int acc = !over && (ex > h.lpacc);
        if (acc) {
          S.e_run[0] += dLJ;
          S.e_run[1] += dRe;
          S.e_run[2] += dRc;
        }
        settings_update(S.set, h.kind, acc);
        S.accept = acc;
        if (rank == 0 && C.tr_i) {
          C.tr_i[3 * (size_t)t] = h.kind;
          C.tr_i[3 * (size_t)t + 1] = m;
          C.tr_i[3 * (size_t)t + 2] = acc;
          C.tr_d[3 * (size_t)t] = dLJ;
          C.tr_d[3 * (size_t)t + 1] = dRe;
          C.tr_d[3 * (size_t)t + 2] = dRc;
        }
      }
    }
    __syncthreads();
    const int acc = S.accept;
    const int prev_m = m, prev_kind = h.kind;
    if (acc) {
      for (int i = threadIdx.x; i < kc; i += MT_THREADS) {
        // (s32 + lo) += d, error-free sum then renormalised
        ff2 r = ff_two_sum(s32R[i], dR[i]);
        ff2 im = ff_two_sum(s32I[i], dI[i]);
        r = ff_quick(r.hi, r.lo + loR[i]);
        im = ff_quick(im.hi, im.lo + loI[i]);
        s32R[i] = r.hi;
        loR[i] = r.lo;
        s32I[i] = im.hi;
        loI[i] = im.lo;
      }
      if (rank == 0 && threadIdx.x < 32) {
        // Atoms that stay in their cell are rewritten in place by one lane
        // each; then the atoms that change cell are relinked one after
        // another, in atom order -- the slot layout that relinking every
        // atom in order would give.
        const int a = threadIdx.x;
        bool stay = false;
        if (a < na) {
          const double *np = h.newp[a];
          const int at = h.a0 + a;
          b.x[at] = np[0];
          b.y[at] = np[1];
          b.z[at] = np[2];
          stay = cur_cell == h.cell_new[a];
          if (stay)
            cell_write_slot(b, cur_cell, cur_slot, at, np[0], np[1], np[2],
                            h.un[a]);
        }
        const unsigned moving = __ballot_sync(0xffffffffu, a < na && !stay);
        __syncwarp();
        if (a == 0) {
          for (int i = 0; i < na; ++i)
            if (moving & (1u << i)) {
              const double *np = h.newp[i];
              cell_move_atom(b, h.a0 + i, np[0], np[1], np[2], h.cell_new[i],
                             h.un[i]);
            }
          if (h.kind == 0) {
            b.cx[m] = h.newcom[0];
            b.cy[m] = h.newcom[1];
            b.cz[m] = h.newcom[2];
          }
        }
      }
    }
    if (t + 1 < C.n) {
      long long step = C.first + t + 1;
      if ((step + 1) % S.set.adj == 0) {
        __syncthreads();
        if (threadIdx.x == 0)
          settings_adjust(S.set, step);
        __syncthreads();
        make_props(t + 1);
        cluster.sync();
      }
      if (!spec) {
        __syncthreads();
        mixed_header(C, S, t + 1, acc, prev_m, prev_kind, h,
                     S.hh[(t + 1) & 1]);
        mixed_tables(C, S.hh[(t + 1) & 1], tabs + ((t + 1) & 1) * tab_len);
      }
    }
    cluster.sync();  // the cell grid committed by rank 0 is visible
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kc; i += MT_THREADS) {
    b.sumRref[kbeg + i] = (double)s32R[i] + (double)loR[i];
    b.sumIref[kbeg + i] = (double)s32I[i] + (double)loI[i];
  }
  if (rank == 0 && threadIdx.x == 0) {
    *C.set = S.set;
    for (int i = 0; i < 5; ++i)
      b.energy[i] = S.e_run[i];
  }
}

size_t mixed_smem(int K, int kmax, int csize, bool cold_smem) {
  int kc_max = (K + csize - 1) / csize;
  MixedLayout L = mixed_layout(kc_max, cold_smem);
  return L.tab + 2 * sizeof(float2) * (size_t)3 * MAXA * (kmax + 1) + 16;
}

size_t mixed_cold_buffer(int K, int csize) {
  return (size_t)csize * mixed_cold_bytes((K + csize - 1) / csize);
}

// The kernel's attributes are set once, to the largest shared memory it ever
// asks for: launches and occupancy queries may then come from several host
// threads (the job server's round and set-up threads) without one changing
// the limit under another's launch.
static void mixed_attrs() {
  static std::once_flag once;
  std::call_once(once, [] {
    cudaFuncSetAttribute(k_chain_mixed,
                         cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaFuncSetAttribute(k_chain_mixed,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)MIXED_SMEM_MAX);
    // a refused attribute must not surface later as another call's error;
    // the launch itself then reports the problem
    cudaGetLastError();
  });
}

int launch_chain_mixed(cudaStream_t st, const MixedChain *d_chains, int nchains,
                       int csize, size_t smem) {
  if (smem > MIXED_SMEM_MAX)
    return ERR_UNSUPPORTED;
  mixed_attrs();
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nchains * csize);
  cfg.blockDim = dim3(MT_THREADS);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = csize;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaError_t e = cudaLaunchKernelEx(&cfg, k_chain_mixed, d_chains);
  return e == cudaSuccess ? OK : ERR_CUDA;
}

int max_active_clusters(int csize, size_t smem) {
  if (smem > MIXED_SMEM_MAX)
    return 0;
  mixed_attrs();
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(csize);
  cfg.blockDim = dim3(MT_THREADS);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = csize;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, k_chain_mixed, &cfg) != cudaSuccess)
    return 0;
  return n;
}

}  // namespace gb
