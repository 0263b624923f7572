// FP64 move chain with two moves in flight (included by gb_mc.cu, after
// k_chain_fp64, whose helpers and layout it shares).
//
// The chain of k_chain_fp64 spends about half of a move waiting: the last
// partial reaches the deciding CTA, the sums, the decision, its release
// store and its way back to every CTA take about as long as the CTAs' own
// phase A.  Here one CTA (the last) does nothing but decide, and the other
// G - 1 CTAs ("work CTAs") start move t + 1 as soon as their partials of
// move t are out, while move t is being decided.  Move t + 1's energy
// depends on move t's outcome in two places only, and a work CTA evaluates
// both outcomes:
//   * reciprocal space: the new sums of move t + 1 on the committed
//     structure factors (t rejected) and on move t's new sums (t
//     accepted), both kept, one of them chosen at the commit -- the same
//     additions, in the same order, as the chain that waits;
//   * real space: the atoms of move t's molecule that the CTA owns, at
//     their old and at their new positions, against move t + 1's molecule
//     (all other own atoms are the same on both outcomes).
// Each work CTA stores two sets of partials (one per outcome of the
// previous move); the decider reads the set its own previous decision
// names.  Move t + 1 does not run ahead of move t's decision when it moves
// the same molecule as move t or as move t - 1 while that one is still
// undecided, or follows a settings adjustment: then move t's decision is
// waited for, committed, and move t + 1's context is built behind a grid
// barrier (as in k_chain_fp64).
//
// Ordering (acquire/release on the decision word and the context flags):
//   * work CTA at move t: phase A(t) -> partials(t) -> decision(t - 1)
//     and the flags of context(t + 1), in one poll -> commit(t - 1) ->
//     phase A(t + 1);
//   * decider at move t: CTA 0's flag of context(t) -> header -> every
//     work CTA's partials(t) -> decision -> release of the word -> partial
//     slots reset, coordinates written.
// Contexts rotate over three buffers and partials over three slot sets: a
// writer overwrites context t - 1's buffer while building context t + 2,
// after it has seen decision t, which the decider gave only after every
// work CTA had read context t - 1 and stored partials(t); a work CTA stores
// partials(t + 3) after it has seen decision t + 1, behind which the
// decider reset slot set t.  The decider can run at most one move past a
// work CTA's read of the word.
// No counterpart in the reference (its moves are sequential,
// src/moves/Translate.h:97-138, src/moves/Rotation.h:89-130).

// The decision word of move t: ((t + 1) << 4) | the outcomes of moves t,
// t - 1, t - 2, t - 3 in bits 0..3, so that one load of it gives a work
// CTA the outcome of a move the decider has already passed.
__device__ __forceinline__ unsigned dec_word(int t, unsigned hist) {
  return ((unsigned)(t + 1) << 4) | (hist & 15u);
}
__device__ __forceinline__ unsigned ld_relaxed(const unsigned *p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
// the outcome of move tt from a word at or past it (at most three moves)
__device__ __forceinline__ int dec_outcome(unsigned w, int tt) {
  return (int)((w >> ((int)(w >> 4) - (tt + 1))) & 1u);
}

// Dynamic shared memory of one CTA of k_chain_fp64_pipe (the layout of
// k_chain_fp64 with four k-chunk buffers and the atoms spread over the
// work CTAs).
__host__ __device__ inline size_t chain_pipe_kvec_doubles(int kc_max) {
  return ((9 * (size_t)kc_max + (kc_max + 1) / 2 + 1) & ~(size_t)1);
}

// The pair list of a k-chunk CTA: one segment of PSEG entries per warp
// (its own atoms' pairs, found by a warp-level scan) and one for the
// previous move's atoms, so that the list needs one CTA barrier and no
// CTA-wide prefix sum.
constexpr int PSEG = 64;
constexpr int PNSEG = CT / 32 + 1;
constexpr int ICL_CAP = PSEG * PNSEG;

// Minimum-image wrap of one axis decided on fixed-point turns when a pair
// is listed: 1 for -L, 2 for +L (2 bits per axis).  Only a pair near half a
// box edge apart -- far outside the cutoff -- could be decided otherwise
// than by the FP64 test of BoxDimensions::MinImage.
__device__ __forceinline__ unsigned turn_wrap(const uint32_t *tp, uint4 f) {
  const uint32_t tf[3] = {f.x, f.y, f.z};
  unsigned w = 0;
  for (int d = 0; d < 3; ++d) {
    const long long dt = (long long)tp[d] - (long long)tf[d];
    if (dt > 2147483648LL)
      w |= 1u << (2 * d);
    else if (dt < -2147483648LL)
      w |= 2u << (2 * d);
  }
  return w;
}

// pair_term of the chain with two moves in flight, with fewer FP64
// instructions (a warp's FP64 instruction holds its SM sub-partition's FP64
// unit for about 64 cycles on GB300, so their count sets the time of a
// pass over the pair list): the minimum image from the listed wrap bits
// (the same FP64 differences: x - L is x + (-L)), the neighbour's charge
// stored times QQ_FACT, and -- where every kind pair has the 12-6 form --
// 1 / r^2 by two Newton-Raphson steps from the FP32 reciprocal (relative
// error below 2^-90 before the final rounding) with sigma^2 / r^2 as a
// product; the Coulomb cutoff is tested only where it is shorter than the
// pair cutoff.
// The force field's pair tables held in shared memory by the chain with two
// moves in flight: the erfc(alpha r)/r segments (NULL: read from global
// memory) and the LJ sigma^2 and epsilon C_n of every kind pair.
struct PairTabs {
  const double *etab;
  const double *sig2, *eps;
};

// erfc(alpha r) / r as erfc_over_r: the same segment polynomial, its
// coefficients read from shared memory
__device__ __forceinline__ double erfc_over_r_tab(const FF &ff,
                                                  const double *tab, double s) {
  const long long bits = __double_as_longlong(s);
  const int seg = (int)(bits >> 46) - ff.etab_key0;
  if (tab == nullptr || (unsigned)seg >= (unsigned)ff.etab_nseg)
    return erfc_over_r(ff, s);
  const double a = __longlong_as_double(bits & ~((1LL << 46) - 1));
  const double scale = __longlong_as_double((2053LL - (bits >> 52)) << 52);
  const double u = fma(s - a, scale, -1.0);
  const double *c = tab + (size_t)seg * (ETAB_DEG + 1);
  double p = c[ETAB_DEG];
#pragma unroll
  for (int m = ETAB_DEG - 1; m >= 0; --m)
    p = fma(p, u, c[m]);
  return p;
}

// One pair's terms, signed for the side (new position +, old -): false
// outside the cutoff.  pzq: the neighbour's z and the pair's charge
// product q_i q_j QQ_FACT (formed when the pair was listed).
__device__ __forceinline__ bool pair_energy_pipe(const ChainArgs &A,
                                                 const double *hdr, int u,
                                                 double2 pxy, double2 pzq,
                                                 int mj, unsigned wrap,
                                                 bool lj12, bool coul_cut,
                                                 const PairTabs &pt, double &e,
                                                 double &l, bool &ov) {
  const DevBox &b = A.b;
  const FF &ff = *A.ff;
  const int a = u / (2 * NB27), side = (u / NB27) % 2;
  const double *pp = hdr + (side ? 48 : 24) + 3 * a;
  double dx = pp[0] - pxy.x, dy = pp[1] - pxy.y, dz = pp[2] - pzq.x;
  dx += (wrap & 1u) ? -b.L[0] : (wrap & 2u) ? b.L[0] : 0.0;
  dy += (wrap & 4u) ? -b.L[1] : (wrap & 8u) ? b.L[1] : 0.0;
  dz += (wrap & 16u) ? -b.L[2] : (wrap & 32u) ? b.L[2] : 0.0;
  const double d2 = dsq3(dx, dy, dz);
  if (!(ff.rcutSq > d2))
    return false;
  ov = side && d2 < ff.rcutLowSq;
  e = 0.0;
  if (ff.electrostatic && !(coul_cut && ff.rcutCoulSq < d2))
    e = ff.ewald ? pzq.y * erfc_over_r_tab(ff, pt.etab, d2) : pzq.y / sqrt(d2);
  const int idx = ((const int *)(hdr + 116))[a] + meta_kind(mj) * ff.n_kinds;
  if (lj12) {
    double y = (double)__frcp_rn((float)d2);
    double r = fma(-d2, y, 1.0);
    y = fma(y, r, y);
    r = fma(-d2, y, 1.0);
    y = fma(y, r, y);
    const double rRat2 = pt.sig2[idx] * y;
    const double attract = rRat2 * rRat2 * rRat2;
    l = pt.eps[idx] * (attract * attract - attract);
  } else {
    l = lj_energy(ff, d2, idx);
  }
  // the old position's terms subtracted: the sign bit flipped (exact)
  const unsigned long long neg = side ? 0ull : 0x8000000000000000ull;
  e = __longlong_as_double((long long)((unsigned long long)__double_as_longlong(e) ^ neg));
  l = __longlong_as_double((long long)((unsigned long long)__double_as_longlong(l) ^ neg));
  return true;
}

// pair_energy_pipe added to one set of sums
__device__ __forceinline__ void pair_term_pipe(const ChainArgs &A,
                                               const double *hdr, int u,
                                               double2 pxy, double2 pzq,
                                               int mj, unsigned wrap,
                                               bool lj12, bool coul_cut,
                                               const PairTabs &pt,
                                               double &lj, double &re,
                                               double &ovl) {
  double e, l;
  bool ov;
  if (pair_energy_pipe(A, hdr, u, pxy, pzq, mj, wrap, lj12, coul_cut, pt, e, l,
                       ov)) {
    re += e;
    lj += l;
    if (ov)
      ovl = 1.0;
  }
}

__global__ void __launch_bounds__(CT, 1) k_chain_fp64_pipe(ChainArgs A) {
  extern __shared__ double dyn[];
  __shared__ ChainShared S;
  __shared__ double red6[6][CT / 32];     // warp sums, both outcomes
  const DevBox &b = A.b;
  const FF &ff = *A.ff;
  const int G = gridDim.x, cta = blockIdx.x;
  const int W = G - 1;  // work CTAs 0 .. W - 1; CTA W decides
  const bool leader = cta == W;
  const int nkb = A.nkless;
  const int kG = W - nkb;
  const int kc_max = (b.K + kG - 1) / kG;
  const bool kless = cta < nkb;
  const int kbeg = (kless || leader) ? b.K : min(b.K, (cta - nkb) * kc_max);
  const int kc = (kless || leader) ? 0 : min(kc_max, b.K - kbeg);
  const int pw = kless ? 0 : 3;  // the warp that evaluates the pair terms
  // k-chunk buffers [4][re, im][kc_max]: the committed structure factors,
  // the previous move's new sums while it is undecided, and this move's new
  // sums on either outcome of the previous one (the roles rotate)
  double *const kbuf = dyn;
  auto KR = [&](int i) { return kbuf + (size_t)(2 * i) * kc_max; };
  auto KI = [&](int i) { return kbuf + (size_t)(2 * i + 1) * kc_max; };
  double *const pf = dyn + 8 * (size_t)kc_max;
  char4 *const kn = (char4 *)(pf + kc_max);
  const int stride = b.kmax + 1;
  // phase rows of this move and, prefetched, of the next (the roles swap)
  double2 *const tab0 = (double2 *)(dyn + chain_pipe_kvec_doubles(kc_max));
  double2 *const tab1 = tab0 + (size_t)(2 * MAX_MOL_ATOMS * 3) * stride;
  double2 *tab = tab0;
  double2 *const exy = tab1 + (size_t)(2 * MAX_MOL_ATOMS * 3) * stride;
  unsigned short *const pidx =
      (unsigned short *)(exy + NPAIR_CAP * 2 * MAX_MOL_ATOMS);
  // The atoms are owned by the work CTAs with a k-chunk (the context
  // writers without one build the next context instead), through a
  // multiplicative permutation of the atom index (p = a * perm_m mod
  // n_atoms): atom a by CTA nkb + p % OWN, at index p / OWN of its share.
  // Atom indices follow the build order of the system (a lattice, at
  // first), so without the permutation the atoms near a molecule can crowd
  // onto a few CTAs and lengthen their pair lists.
  const int OWN = W - nkb;
  // x mod n_atoms by Barrett reduction (perm_r = floor((2^64 - 1) / n)):
  // integer multiplies only, no 64-bit division
  auto mod_n = [&](unsigned long long x) {
    const unsigned long long n = (unsigned long long)b.n_atoms;
    unsigned long long r = x - __umul64hi(x, A.perm_r) * n;
    return (int)(r >= n ? r - n : r);
  };
  auto perm = [&](int a) { return mod_n((unsigned long long)a * A.perm_m); };
  const int orank = cta - nkb;  // this CTA's rank among the owners
  const int own_per = (b.n_atoms + OWN - 1) / OWN;
  const int on = (!leader && orank >= 0 && orank < b.n_atoms)
                     ? (b.n_atoms - orank + OWN - 1) / OWN
                     : 0;
  double2 *const oxy =
      (double2 *)(((uintptr_t)(pidx + kc_max) + 15) & ~(uintptr_t)15);
  double2 *const ozq = oxy + own_per;
  uint4 *const ot = (uint4 *)(ozq + own_per);
  // the erfc(alpha r)/r segments after them (k-chunk CTAs, Ewald on)
  double *const etab_s = (double *)(ot + own_per);
  __shared__ double lj_sig2_s[MAX_KINDS * MAX_KINDS];
  __shared__ double lj_eps_s[MAX_KINDS * MAX_KINDS];
  __shared__ char2 pair_n[NPAIR_CAP];
  __shared__ int npair;
  int bS = 0, bP = -1;  // committed and pending k-chunk buffers
  for (int i = threadIdx.x; i < kc; i += CT) {
    int k = kbeg + i;
    KR(0)[i] = b.sumRref[k];
    KI(0)[i] = b.sumIref[k];
    pf[i] = b.prefact[k];
    kn[i] = b.kn[k];
  }
  for (int i = threadIdx.x; i < on; i += CT) {
    const int a = mod_n((unsigned long long)(orank + OWN * i) * A.perm_minv);
    const double x = b.x[a], y = b.y[a], z = b.z[a];
    oxy[i] = make_double2(x, y);
    ozq[i] = make_double2(z, b.q[a] * QQ_FACT);  // the charge times QQ_FACT
    ot[i] = make_uint4(to_turns(x, b.invL[0]), to_turns(y, b.invL[1]),
                       to_turns(z, b.invL[2]),
                       (unsigned)pack_meta(b.mol[a], b.kind[a]));
  }
  const bool own_tab = !leader && !kless && ff.erfc_tab != nullptr;
  if (own_tab)
    for (int i = threadIdx.x; i < ff.etab_nseg * (ETAB_DEG + 1); i += CT)
      etab_s[i] = ff.erfc_tab[i];
  for (int i = threadIdx.x; i < ff.n_kinds * ff.n_kinds; i += CT) {
    lj_sig2_s[i] = ff.sigmaSq[i];
    lj_eps_s[i] = ff.eps_cn[i];
  }
  const PairTabs ptab{own_tab ? etab_s : nullptr, lj_sig2_s, lj_eps_s};
  __shared__ int lj12_sh;
  if (threadIdx.x == 0) {
    int all12 = 1;
    for (int i = 0; i < ff.n_kinds * ff.n_kinds; ++i)
      all12 &= ff.eps_cn[i] == 0.0 || ff.nexp[i] == 12.0;
    lj12_sh = all12;
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
  const bool lj12 = lj12_sh != 0;
  const bool coul_cut = ff.rcutCoulSq < ff.rcutSq;
  const float turn_f[3] = {(float)(b.L[0] * 2.3283064365386963e-10),
                           (float)(b.L[1] * 2.3283064365386963e-10),
                           (float)(b.L[2] * 2.3283064365386963e-10)};
  const float cut_f = (float)(ff.rcutSq * 1.0001);
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

  // prologue: the first block's proposals and context 0
  if (threadIdx.x == 0)
    settings_adjust(S.set, A.first);
  __syncthreads();
  make_props(0);
  if (!grid_sync(A.bar, G, S.gen, b.err, &S.flag, A.spin))
    return;
  build_ctx(A, S, 0, nullptr, 0, 0, CT);
  if (!grid_sync(A.bar, G, S.gen, b.err, &S.flag, A.spin))
    return;

  // the profiled work CTA: the first with a k-chunk (the context writers
  // before it only build contexts)
  const int pslot = cta == nkb ? 0 : leader ? 1 : -1;
  const bool prof = A.prof && threadIdx.x == 0 && pslot >= 0;
  long long pacc[5] = {0, 0, 0, 0, 0};
  long long tclk = prof ? clock64() : 0;
  auto mark = [&](int ph) {
    if (prof) {
      long long now = clock64();
      pacc[ph] += now - tclk;
      tclk = now;
    }
  };
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // the settings adjustment before a move (the next move's proposals are
  // made after it), behind a grid barrier; false when a wait gave up
  auto adjust_before = [&](int t1, bool bnd) -> bool {
    long long step = A.first + t1;
    if (!bnd)
      return true;
    __syncthreads();
    if (threadIdx.x == 0)
      settings_adjust(S.set, step);
    __syncthreads();
    make_props(t1);
    return grid_sync(A.bar, G, S.gen, b.err, &S.flag, A.spin);
  };
  int nmol = A.n > 1 ? A.moves[1].mol : -1;
  // (first + t + 2) mod AdjSteps, carried from move to move (no 64-bit
  // division per move): zero where a settings adjustment precedes move
  // t + 1
  int adj_r = (int)((A.first + 2) % S.set.adj);

  if (leader) {
    // ---------------- the deciding CTA ----------------
    bool pend = false;
    int m_prev = -1, acc_prev = 0;
    unsigned hist = 0;  // outcomes of the last moves, newest in bit 0
    for (int t = 0; t < A.n; ++t) {
      const int mol_next = nmol;
      nmol = t + 2 < A.n ? A.moves[t + 2].mol : -1;
      const bool bnd = adj_r == 0;
      adj_r = adj_r + 1 == S.set.adj ? 0 : adj_r + 1;
      // this move's header: complete once CTA 0 has flagged the context
      // when it was built during the previous move's phase A, and behind
      // the last grid barrier otherwise
      if (threadIdx.x == 0)
        S.ok = pend ? wait_geq(A.seq + SEQ_CTX, (unsigned)t, b.err, A.spin)
                    : 1;
      __syncthreads();
      if (!S.ok)
        return;
      const double *ctx_t = A.ctx + (size_t)(t % A.nctx) * A.ctx_len;
      for (int i = threadIdx.x; i < HDR; i += CT)
        S.hdr[i] = __ldcg(ctx_t + i);
      __syncthreads();
      mark(0);
      const int m = (int)S.hdr[0];
      const int na = (int)S.hdr[2];
      const int a0m = __ldg(b.mstart + m);
      const bool nspec = t + 1 < A.n && mol_next != m && !bnd &&
                         !(pend && mol_next == m_prev);
      const int var = pend ? acc_prev : 0;  // the partials' outcome set
      double *part_t = A.part + (size_t)(t % 3) * G * 8;
      constexpr int PF = PART_MAX_GRID / 32;
      if (warp < 4) {
        // warps 0..3 each gather one quantity over the work CTAs (LJ, real
        // space, reciprocal energy, overlap), polling until every CTA's is
        // present; lane l adds CTAs l, l + 32, ... in order, then the warp
        // tree: a fixed order
        const int q = warp;
        constexpr int NPOLL = 3;
        double pp[NPOLL][PF];
        auto issue = [&](double *dst) {
#pragma unroll
          for (int i = 0; i < PF; ++i) {
            int c = lane + 32 * i;
            dst[i] = c < W ? __ldcg(part_t + (size_t)c * 8 + 4 * var + q) : 0.0;
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
        if (prof)
          mark(2);
        double pv[PF];
#pragma unroll
        for (int i = 0; i < PF; ++i)
          pv[i] = got == 0 ? pp[0][i] : got == 1 ? pp[1][i] : pp[2][i];
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
          S.red3[0][q] = ok;
        asm volatile("bar.sync 2, 128;" ::: "memory");
        ok = S.red3[0][0] != 0.0 && S.red3[0][1] != 0.0 &&
             S.red3[0][2] != 0.0 && S.red3[0][3] != 0.0;
        int acc = 0;
        if (warp == 0 && ok) {
          double dLJ = 0.0, dRe = 0.0, dRc = 0.0;
          if (lane == 0) {
            bool over = S.tot[3] > 0;
            dLJ = S.tot[0];
            dRe = S.tot[1];
            dRc = (!over && b.K > 0) ? S.tot[2] - S.e_run[2] : 0.0;
            double ex = __dmul_rn(-ff.beta, __dadd_rn(__dadd_rn(dLJ, dRe), dRc));
            // pacc < exp(ex), decided on logarithms unless the two sides
            // are within 1e-9 (or pacc is 0)
            int res;
            if (S.hdr[3] > 0.0 && ex > S.hdr[81])
              res = 1;
            else if (S.hdr[3] > 0.0 && ex < S.hdr[82])
              res = 0;
            else
              res = S.hdr[3] < exp(ex);
            acc = res && !over;
            hist = (hist << 1) | (unsigned)acc;
            st_release(A.seq, dec_word(t, hist));
          }
          acc = __shfl_sync(0xffffffffu, acc, 0);
          if (prof)
            mark(3);
          if (acc) {
            // the new coordinates and centre, after the word (a context
            // built before the next word reads them from its builders'
            // copies of this move)
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
          }
          if (lane == 0) {
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
          }
        }
        if (warp == 0 && lane == 0)
          S.ok = ok;
        // slot set t % 3 of every work CTA, both outcomes, marked empty
        // for move t + 3 (ordered before the next word by the barrier
        // below and that word's release)
        if (ok) {
#pragma unroll
          for (int i = 0; i < PF; ++i) {
            int c = lane + 32 * i;
            if (c < W) {
              __stcg(part_t + (size_t)c * 8 + q, __longlong_as_double(PART_EMPTY));
              __stcg(part_t + (size_t)c * 8 + 4 + q,
                     __longlong_as_double(PART_EMPTY));
            }
          }
        }
      }
      __syncthreads();
      if (!S.ok)
        return;
      const int acc = S.accept;
      if (threadIdx.x == 0)
        settings_update(S.set, (int)S.hdr[1], acc);
      if (!nspec && t + 1 < A.n) {
        if (!adjust_before(t + 1, bnd))
          return;
        // the next context is built by the work CTAs behind this barrier
        if (!grid_sync(A.bar, G, S.gen, b.err, &S.flag, A.spin))
          return;
      }
      mark(4);
      pend = nspec;
      acc_prev = acc;
      m_prev = m;
    }
  } else {
    // ---------------- work CTAs ----------------
    // warp 7 gathers the next context's inputs, warp 0 counts its writers
    const bool piper = warp == 7 || warp == 0;
    CtxPre pipe_a, pipe_b;  // record of t + 2 (a), record and range of t + 1 (b)
    int pipe_b1 = 0;
    pipe_a.writer = pipe_b.writer = false;
    pipe_a.m = pipe_b.m = -1;
    if (piper) {
      ctx_pre_record(A, 1, pipe_b);
      ctx_pre_range(A, pipe_b, pipe_b1);
      ctx_pre_record(A, 2, pipe_a);
    }
    bool pend = false;  // this move runs before the previous one's decision
    int m_prev = -1, na_prev = 0, a0_prev = 0;
    int mol_cur = A.n > 0 ? A.moves[0].mol : -1;
    bool have_next = false;  // this move's context prefetched into smem
    // three header buffers in turn: this move's (hc), the previous move's
    // while it is undecided (hq), the next move's, prefetched (hn)
    __shared__ double hbuf[3][HDR];
    int hc = 0, hq = 1, hn = 2;
    for (int t = 0; t < A.n; ++t) {
      const int mol_next = nmol;
      nmol = t + 2 < A.n ? A.moves[t + 2].mol : -1;
      const bool bnd = adj_r == 0;
      adj_r = adj_r + 1 == S.set.adj ? 0 : adj_r + 1;
      CtxPre pre = pipe_b;
      pre.na = pipe_b1 - pipe_b.a0;
      if (piper) {
        pipe_b = pipe_a;
        ctx_pre_range(A, pipe_b, pipe_b1);
        ctx_pre_record(A, t + 3, pipe_a);
      }
      // ---------------- phase A ----------------
      const double *ctx_t = A.ctx + (size_t)(t % A.nctx) * A.ctx_len;
      const int m = mol_cur;
      // this move's atom range, from the record pipeline of warp 0 (stored
      // during the previous move) but for the first move
      __shared__ int nx_a0, nx_na;
      const int a0m = t == 0 ? __ldg(b.mstart + m) : nx_a0;
      const int na = t == 0 ? __ldg(b.mstart + m + 1) - a0m : nx_na;
      // may move t + 1 run before this move's decision
      const bool nspec = t + 1 < A.n && mol_next != m && !bnd &&
                         !(pend && mol_next == m_prev);
      pre.writer = false;
      const bool wload = nspec && warp == 7;
      const int nbuild = max(1, min(W, b.K > 0 ? 2 * pre.na * 3 : 0));
      double lj = 0.0, re = 0.0, ovl = 0.0, er = 0.0, er2 = 0.0;
      // pair terms of the previous move's atoms this CTA owns, at their
      // old positions (that move rejected) and new ones (accepted)
      double ljR = 0.0, reR = 0.0, ovR = 0.0, ljA = 0.0, reA = 0.0, ovA = 0.0;
      // this move's new sums on either outcome of the previous move
      int fr[3], nfr = 0;
      for (int i = 0; i < 4; ++i)
        if (i != bS && i != bP && nfr < 3)
          fr[nfr++] = i;
      const int bR = fr[0], bA = fr[1];
      // Real space, as in k_chain_fp64: own atoms against the old and new
      // positions of the moved atoms, FP32 pre-test on fixed-point turns,
      // the pairs compacted in order into a shared list.  While the previous
      // move is undecided, its atoms are left out of the pre-test and listed
      // after the others on both of its outcomes, so that one warp pass
      // takes them all.
      __shared__ double2 icl_pos[ICL_CAP][2];
      __shared__ int icl_meta[ICL_CAP];
      __shared__ short icl_unit[ICL_CAP];
      // entry class: 0 an own atom that both outcomes of the previous move
      // share, 1 / 2 an atom of the previous move's molecule at its old
      // position (that move rejected) / its new one (accepted)
      __shared__ unsigned char icl_cls[ICL_CAP];
      __shared__ unsigned char icl_wrap[ICL_CAP];  // turn_wrap of the pair
      __shared__ int seg_cnt[PNSEG];  // entries found per segment
      const int npos = 2 * na;
      double *const hd = hbuf[hc];        // this move's header
      const double *const hdrp = hbuf[hq];  // the previous move's
      const uint32_t *pturn = (const uint32_t *)(hd + 84);
      int n_prev = 0;  // own atoms of the previous molecule (usually 0 or 1)
      if (pend)
        for (int ap = 0; ap < na_prev; ++ap)
          n_prev += perm(a0_prev + ap) % OWN == orank;
      const int ncomb = n_prev * 2 * npos;
      double *const part_c = A.part + (size_t)(t % 3) * G * 8 + (size_t)cta * 8;
      // own atom i against this move's positions: bit p set where position
      // p passes the FP32 pre-test
      auto pretest = [&](int i, uint4 &f) -> unsigned {
        unsigned hit = 0;
        f = ot[i];
        const int mj = meta_mol((int)f.w);
        if (mj != m && !(pend && mj == m_prev)) {
          for (int pp = 0; pp < npos; ++pp) {
            float dx = (float)(int)(pturn[3 * pp] - f.x) * turn_f[0];
            float dy = (float)(int)(pturn[3 * pp + 1] - f.y) * turn_f[1];
            float dz = (float)(int)(pturn[3 * pp + 2] - f.z) * turn_f[2];
            if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) < cut_f)
              hit |= 1u << pp;
          }
        }
        return hit;
      };
      // list own atom i's passing positions from slot pos on, below slot
      // lim (past it: evaluated here, not met at liquid densities)
      auto list_hits = [&](int i, unsigned hit, uint4 f, int pos, int lim) {
        const double2 pxy = oxy[i], oq = ozq[i];
        for (unsigned h = hit; h; h &= h - 1) {
          const int pp = __ffs(h) - 1;
          const int side = pp >= na ? 1 : 0, a = pp - side * na;
          const int u = (a * 2 + side) * NB27;
          const double2 pzq = make_double2(oq.x, hd[108 + a] * oq.y);
          const unsigned wr = turn_wrap(pturn + 3 * pp, f);
          if (pos < lim) {
            icl_pos[pos][0] = pxy;
            icl_pos[pos][1] = pzq;
            icl_meta[pos] = (int)f.w;
            icl_unit[pos] = (short)u;
            icl_cls[pos] = 0;
            icl_wrap[pos] = (unsigned char)wr;
          } else {
            pair_term_pipe(A, hd, u, pxy, pzq, (int)f.w, wr, lj12, coul_cut, ptab,
                           lj, re, ovl);
          }
          ++pos;
        }
      };
      // The previous move's atoms this CTA owns on both outcomes (entries
      // c = (atom, outcome, position)), pre-tested like the others and
      // appended in order from slot n0 by one warp, below slot lim; those
      // past it are evaluated here.  Returns the end of the entries.
      auto list_prev = [&](int n0, int lim) -> int {
        int n = n0;
        const int nc = na_prev * 2 * npos;
        for (int base = 0; base < nc; base += 32) {
          const int c = base + lane;
          bool hit = false;
          int i = 0, vr = 0, ap = 0, pp = 0;
          uint4 f = make_uint4(0, 0, 0, 0);
          if (c < nc) {
            ap = c / (2 * npos);
            const int r = c - ap * 2 * npos;
            vr = r / npos;
            pp = r - vr * npos;
            const int ga = a0_prev + ap;
            const int pg = perm(ga);
            if (pg % OWN == orank) {
              i = pg / OWN;
              f = ot[i];
              if (vr) {
                const uint32_t *nt = (const uint32_t *)(hdrp + 84) + (na_prev + ap) * 3;
                f.x = nt[0];
                f.y = nt[1];
                f.z = nt[2];
              }
              float dx = (float)(int)(pturn[3 * pp] - f.x) * turn_f[0];
              float dy = (float)(int)(pturn[3 * pp + 1] - f.y) * turn_f[1];
              float dz = (float)(int)(pturn[3 * pp + 2] - f.z) * turn_f[2];
              hit = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) < cut_f;
            }
          }
          const unsigned mask = __ballot_sync(0xffffffffu, hit);
          if (hit) {
            const int pos = n + __popc(mask & ((1u << lane) - 1));
            const int side = pp >= na ? 1 : 0, a = pp - side * na;
            const int u = (a * 2 + side) * NB27;
            double2 pxy = oxy[i], pzq = ozq[i];
            if (vr) {
              const double *np = hdrp + 48 + 3 * ap;
              pxy = make_double2(np[0], np[1]);
              pzq.x = np[2];
            }
            pzq.y *= hd[108 + a];  // q_i q_j QQ_FACT
            const unsigned wr = turn_wrap(pturn + 3 * pp, f);
            if (pos < lim) {
              icl_pos[pos][0] = pxy;
              icl_pos[pos][1] = pzq;
              icl_meta[pos] = (int)f.w;
              icl_unit[pos] = (short)u;
              icl_cls[pos] = (unsigned char)(1 + vr);
              icl_wrap[pos] = (unsigned char)wr;
            } else if (vr) {
              pair_term_pipe(A, hd, u, pxy, pzq, (int)f.w, wr, lj12, coul_cut,
                             ptab, ljA, reA, ovA);
            } else {
              pair_term_pipe(A, hd, u, pxy, pzq, (int)f.w, wr, lj12, coul_cut,
                             ptab, ljR, reR, ovR);
            }
          }
          n += __popc(mask);
        }
        return n;
      };
      // the listed pairs, by the lanes of one warp, each added to its
      // class's sums; the previous move's pairs past a full list directly
      // (entries first * 32 + lane, stepping step * 32: the passes of 32
      // entries split between two warps when the list is longer than one)
      // (entry v of the list: slot v, or with segments the v-th listed
      // entry counting through the segments in order)
      auto eval_pairs = [&](int n_eval, int first, int step, bool segs) {
        for (int v = first * 32 + lane; v < n_eval; v += step * 32) {
          int i = v;
          if (segs) {
            int r = v;
            for (int sg = 0; sg < PNSEG; ++sg) {
              const int c = min(seg_cnt[sg], PSEG);
              if (r < c) {
                i = sg * PSEG + r;
                break;
              }
              r -= c;
            }
          }
          double e, l;
          bool o;
          if (!pair_energy_pipe(A, hd, icl_unit[i], icl_pos[i][0],
                                icl_pos[i][1], icl_meta[i], icl_wrap[i], lj12,
                                coul_cut, ptab, e, l, o))
            continue;
          const int c = icl_cls[i];
          if (c == 0) {
            lj += l;
            re += e;
            if (o)
              ovl = 1.0;
          } else if (c == 1) {
            ljR += l;
            reR += e;
            if (o)
              ovR = 1.0;
          } else {
            ljA += l;
            reA += e;
            if (o)
              ovA = 1.0;
          }
        }
      };
      // the pair partials of the warp that evaluated this CTA's pairs (with
      // the second pair warp's sums from shared memory, when the passes were
      // split): warp sums (both outcomes), stored by lane 0
      __shared__ double pair2[4];
      __shared__ int pair2_ov[2];
      auto store_pairs_warp = [&](bool split) {
        double v[4] = {lj + ljR, re + reR, lj + ljA, re + reA};
        if (ncomb > 0 || split) {  // (the outcomes may differ)
          for (int o = 16; o > 0; o >>= 1)
            for (int j = 0; j < 4; ++j)
              v[j] += __shfl_down_sync(0xffffffffu, v[j], o);
        } else {
          // both outcomes share every pair of this CTA
          for (int o = 16; o > 0; o >>= 1)
            for (int j = 0; j < 2; ++j)
              v[j] += __shfl_down_sync(0xffffffffu, v[j], o);
          v[2] = v[0];
          v[3] = v[1];
        }
        bool any0 = __any_sync(0xffffffffu, ovl > 0.0 || ovR > 0.0);
        bool any1 = __any_sync(0xffffffffu, ovl > 0.0 || ovA > 0.0);
        if (split) {
          // the second pair warp's sums (named barrier 5: the two warps)
          asm volatile("bar.sync 5, 64;" ::: "memory");
          for (int j = 0; j < 4; ++j)
            v[j] += pair2[j];
          any0 = any0 || pair2_ov[0];
          any1 = any1 || pair2_ov[1];
        }
        if (lane == 0) {
          __stcg(part_c + 0, v[0]);
          __stcg(part_c + 1, v[1]);
          __stcg(part_c + 3, any0 ? 1.0 : 0.0);
          __stcg(part_c + 4, v[2]);
          __stcg(part_c + 5, v[3]);
          __stcg(part_c + 7, any1 ? 1.0 : 0.0);
        }
      };

      // What this CTA waits for before its next phase A, polled by one warp
      // that is otherwise idle (its loads' round trips hidden behind the
      // phase): the previous move's decision and the flags of the next
      // context's writers when the next move runs ahead, else this move's
      // decision.  The decision word (lane 0) until it has passed move
      // `want`; S.ok false when a wait gave up.
      const int want = nspec ? (pend ? t - 1 : -1) : t;
      auto poll_warp = [&]() {
        unsigned it = 0, w = 0;
        int ok = 1;
        // relaxed loads while polling (an acquire load may invalidate the
        // SM's L1, which the pair terms beside this warp read their tables
        // through), one acquire fence once everything is seen
        for (;;) {
          bool mine = true;
          if (nspec)
            for (int c = lane; c < nbuild; c += 32)
              mine &= (int)(ld_relaxed(A.seq + SEQ_CTX + c) - (unsigned)(t + 1)) >= 0;
          if (lane == 0 && want >= 0) {
            w = ld_relaxed(A.seq);
            mine &= (int)(w >> 4) >= want + 1;
          }
          if (__all_sync(0xffffffffu, mine)) {
            asm volatile("fence.acq_rel.gpu;" ::: "memory");
            break;
          }
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
          __nanosleep(32);
        }
        if (lane == 0) {
          S.ok = ok && *(volatile int *)b.err == 0;
          S.word = w;
        }
        if (ok && nspec && !kless) {
          // the next context is complete (its writers' flags were seen):
          // its header and phase rows into shared memory now, off the
          // next phase A's path
          const double *ctx_n = A.ctx + (size_t)((t + 1) % A.nctx) * A.ctx_len;
          double2 *tabn = tab == tab0 ? tab1 : tab0;
          for (int i = lane; i < HDR; i += 32)
            hbuf[hn][i] = __ldcg(ctx_n + i);
          for (int i = lane; i < A.nrows_max * stride; i += 32)
            tabn[i] = __ldcg((const double2 *)(ctx_n + HDR) + i);
        }
      };

      if (kless) {
        // A context writer without k-vectors.  Warp 0 takes this move's
        // header, lists its own atoms (a warp-level scan), evaluates the
        // pairs and stores the partials; warps 1..7 build their part of the
        // next move's context meanwhile, from the start of the phase (it
        // does not depend on this move's header).
        if (warp == 0) {
          for (int i = lane; i < HDR; i += 32)
            hd[i] = __ldcg(ctx_t + i);
          __syncwarp();
          mark(0);
          int icl_n = 0;
          for (int base = 0; base < on; base += 32) {
            const int i = base + lane;
            uint4 f = make_uint4(0, 0, 0, 0);
            const unsigned hit = i < on ? pretest(i, f) : 0u;
            const int cnt = __popc(hit);
            int incl = cnt;
            for (int o = 1; o < 32; o <<= 1) {
              int v = __shfl_up_sync(0xffffffffu, incl, o);
              if (lane >= o)
                incl += v;
            }
            if (hit)
              list_hits(i, hit, f, icl_n + incl - cnt, ICL_CAP);
            icl_n += __shfl_sync(0xffffffffu, incl, 31);
          }
          __syncwarp();
          if (ncomb > 0)
            icl_n = list_prev(icl_n, ICL_CAP);
          __syncwarp();
          mark(1);
          eval_pairs(min(icl_n, ICL_CAP), 0, 1, false);
          store_pairs_warp(false);
          if (lane == 0) {
            __stcg(part_c + 2, 0.0);
            __stcg(part_c + 6, 0.0);
          }
          poll_warp();
        } else if (nspec) {
          if (warp == 7) {
            ctx_pre2(A, S, t + 1, pre);
            if (pre.writer)
              ctx_pre_store(S, pre);
            if (lane == 0)
              S.b_writer = pre.writer;
          }
          group_sync(CT - 32);
          if (S.b_writer) {
            build_ctx_rest(A, S, t + 1, (int)threadIdx.x - 32, CT - 32);
            group_sync(CT - 32);
            if (threadIdx.x == 32)
              st_release(A.seq + SEQ_CTX + blockIdx.x, (unsigned)(t + 1));
          }
        }
        __syncthreads();
        mark(2);
      } else {
        // A CTA with a k-chunk.  Warp 3 evaluates the listed pairs beside
        // the k-vectors of warps 0, 1, 2, 4, 5, 6 (warps issue to the SM's
        // sub-partitions by index modulo 4); each stores its partials as
        // soon as they are summed.  Warp 7 of a context writer with
        // k-vectors builds its part of the next context.
        if (have_next) {
          // header and rows prefetched by the polling warp during the
          // previous phase A (behind that phase's closing barriers)
          tab = tab == tab0 ? tab1 : tab0;
        } else {
          for (int i = threadIdx.x; i < HDR; i += CT)
            hd[i] = __ldcg(ctx_t + i);
          for (int i = threadIdx.x; i < A.nrows_max * stride; i += CT)
            tab[i] = __ldcg((const double2 *)(ctx_t + HDR) + i);
          __syncthreads();
        }
        mark(0);
        if (wload)
          ctx_pre2(A, S, t + 1, pre);
        // each warp lists its atoms' pairs into its own segment; warp 0
        // the previous move's atoms into the last
        int n_w = 0;
        for (int base = 0; base < on; base += CT) {
          const int i = base + threadIdx.x;
          uint4 f = make_uint4(0, 0, 0, 0);
          const unsigned hit = i < on ? pretest(i, f) : 0u;
          const int cnt = __popc(hit);
          int incl = cnt;
          for (int o = 1; o < 32; o <<= 1) {
            int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o)
              incl += v;
          }
          if (hit)
            list_hits(i, hit, f, warp * PSEG + n_w + incl - cnt,
                      (warp + 1) * PSEG);
          n_w += __shfl_sync(0xffffffffu, incl, 31);
        }
        if (lane == 0)
          seg_cnt[warp] = n_w;
        if (warp == 0) {
          const int b0 = (PNSEG - 1) * PSEG;
          const int n = ncomb > 0 ? list_prev(b0, ICL_CAP) - b0 : 0;
          if (lane == 0)
            seg_cnt[PNSEG - 1] = n;
        }
        __syncthreads();  // the listed pairs
        mark(1);
        // pairs past a full segment were evaluated where they were found
        // (not met at liquid densities): then the pair sums are the CTA's
        int n_eval = 0;
        bool all_pairs = false;
        for (int sg = 0; sg < PNSEG; ++sg) {
          n_eval += min(seg_cnt[sg], PSEG);
          all_pairs |= seg_cnt[sg] > PSEG;
        }
        // A list longer than one warp pass: warp 4 (another sub-partition)
        // takes every second pass after its k-vectors, instead of warp 3
        // taking them all in sequence.
        const bool split = n_eval > 32 && !all_pairs;
        if (warp == pw) {
          eval_pairs(n_eval, 0, split ? 2 : 1, true);
          if (!all_pairs)
            store_pairs_warp(split);
        } else if (warp == 7) {
          if (wload && pre.writer) {
            ctx_pre_store(S, pre);
            __syncwarp();
            build_ctx_warp(A, S, t + 1);
          }
          if (!all_pairs)
            poll_warp();
        } else {
          const int kw = warp < 3 ? warp : warp - 1;  // 0..5
          // the x-y column products first (named barrier 4: the six warps)
          xy_products(kw * 32 + lane, 6 * 32, npair, pair_n, tab, stride, na,
                      hd + 72, exy);
          asm volatile("bar.sync 4, 192;" ::: "memory");
          const double *sR = KR(bS), *sI = KI(bS);
          const double *pR = pend ? KR(bP) : nullptr;
          const double *pI = pend ? KI(bP) : nullptr;
          double *rR = KR(bR), *rI = KI(bR), *aR = KR(bA), *aI = KI(bA);
          for (int i = kw * 32 + lane; i < kc; i += 6 * 32) {
            double dR, dI;
            kvec_delta(kn[i],
                       npair > 0 ? exy + (size_t)pidx[i] * 2 * na : nullptr,
                       tab, stride, na, hd + 72, dR, dI);
            double srn = sR[i] + dR, sin_ = sI[i] + dI;
            rR[i] = srn;
            rI[i] = sin_;
            er += (srn * srn + sin_ * sin_) * pf[i];
            if (pend) {
              double arn = pR[i] + dR, ain = pI[i] + dI;
              aR[i] = arn;
              aI[i] = ain;
              er2 += (arn * arn + ain * ain) * pf[i];
            }
          }
          // the reciprocal energy of the chunk on both outcomes: warp sums,
          // then the six warps in order (named barrier 4)
          for (int o = 16; o > 0; o >>= 1) {
            er += __shfl_down_sync(0xffffffffu, er, o);
            er2 += __shfl_down_sync(0xffffffffu, er2, o);
          }
          if (lane == 0) {
            red6[2][warp] = er;
            red6[5][warp] = er2;
          }
          asm volatile("bar.sync 4, 192;" ::: "memory");
          if (threadIdx.x == 0) {
            double r0 = 0.0, r1 = 0.0;
            for (int w = 0; w < CT / 32; ++w)
              if (w != 3 && w != 7) {
                r0 += red6[2][w];
                r1 += red6[5][w];
              }
            __stcg(part_c + 2, r0);
            __stcg(part_c + 6, pend ? r1 : r0);
          }
          if (split && warp == 4) {
            // the second pair warp: its passes, summed, to warp 3
            lj = re = ovl = ljR = reR = ovR = ljA = reA = ovA = 0.0;
            eval_pairs(n_eval, 1, 2, true);
            double v[4] = {lj + ljR, re + reR, lj + ljA, re + reA};
            for (int o = 16; o > 0; o >>= 1)
              for (int j = 0; j < 4; ++j)
                v[j] += __shfl_down_sync(0xffffffffu, v[j], o);
            const bool any0 = __any_sync(0xffffffffu, ovl > 0.0 || ovR > 0.0);
            const bool any1 = __any_sync(0xffffffffu, ovl > 0.0 || ovA > 0.0);
            if (lane == 0) {
              for (int j = 0; j < 4; ++j)
                pair2[j] = v[j];
              pair2_ov[0] = any0;
              pair2_ov[1] = any1;
            }
            asm volatile("bar.sync 5, 64;" ::: "memory");
          }
        }
        if (all_pairs) {
          // pairs past the list were evaluated by every warp: the CTA's
          // pair sums over all warps, in warp order
          double v[4] = {lj + ljR, re + reR, lj + ljA, re + reA};
          for (int o = 16; o > 0; o >>= 1)
            for (int j = 0; j < 4; ++j)
              v[j] += __shfl_down_sync(0xffffffffu, v[j], o);
          const int any0 = __syncthreads_or(ovl > 0.0 || ovR > 0.0);
          const int any1 = __syncthreads_or(ovl > 0.0 || ovA > 0.0);
          if (lane == 0) {
            red6[0][warp] = v[0];
            red6[1][warp] = v[1];
            red6[3][warp] = v[2];
            red6[4][warp] = v[3];
          }
          __syncthreads();
          if (threadIdx.x < 4) {
            const int j = threadIdx.x < 2 ? threadIdx.x : threadIdx.x + 1;
            double r = 0.0;
            for (int w = 0; w < CT / 32; ++w)
              r += red6[j][w];
            __stcg(part_c + (threadIdx.x < 2 ? threadIdx.x : threadIdx.x + 2), r);
          } else if (threadIdx.x == 4) {
            __stcg(part_c + 3, any0 ? 1.0 : 0.0);
            __stcg(part_c + 7, any1 ? 1.0 : 0.0);
          }
          // the poll after the CTA-wide sums (warp 7 took part in them)
          if (warp == 7)
            poll_warp();
        }
        __syncthreads();
        mark(2);
      }
      // ---------------- phase B ----------------
      // an accepted move (hd: its header): its new positions for the next
      // contexts, and the moved atoms this CTA owns take them
      auto commit_atoms = [&](const double *hd, int nn, int a0) {
        for (int i = threadIdx.x; i < 3 * nn + 3; i += CT) {
          if (i < 3 * nn)
            S.last_newp[i / 3][i % 3] = hd[48 + i];
          else
            S.last_newcom[i - 3 * nn] = hd[4 + i - 3 * nn];
        }
        for (int a = threadIdx.x; a < nn; a += CT) {
          const int pg = perm(a0 + a), i = pg / OWN;
          if (pg - i * OWN == orank) {
            const double *np = hd + 48 + 3 * a;
            const uint32_t *pt = (const uint32_t *)(hd + 84) + (nn + a) * 3;
            oxy[i] = make_double2(np[0], np[1]);
            ozq[i].x = np[2];
            ot[i] = make_uint4(pt[0], pt[1], pt[2], ot[i].w);
          }
        }
      };
      if (!S.ok)
        return;
      const unsigned word = S.word;
      if (threadIdx.x == 0) {  // the next move's range (read after a barrier)
        nx_a0 = pre.a0;
        nx_na = pre.na;
      }
      if (pend) {
        const int acc_p = dec_outcome(word, t - 1);
        if (threadIdx.x == 0) {
          settings_update(S.set, (int)hdrp[1], acc_p);
          S.last_m = m_prev;
          S.last_acc = acc_p;
        }
        if (acc_p) {
          commit_atoms(hdrp, na_prev, a0_prev);
          bS = bP;  // the previous move's new sums are committed
          bP = bA;  // and this move's new sums on that outcome pend
        } else {
          bP = bR;
        }
        __syncthreads();  // the previous header is read before it is replaced
      } else {
        bP = bR;
      }
      mark(3);
      if (nspec) {
        m_prev = m;
        na_prev = na;
        a0_prev = a0m;
        pend = true;
        have_next = !kless;
        __syncthreads();
      } else {
        // this move's decision and commit, then the next context behind a
        // grid barrier
        const int acc = dec_outcome(word, t);
        __syncthreads();
        if (threadIdx.x == 0) {
          settings_update(S.set, (int)hd[1], acc);
          S.last_m = m;
          S.last_acc = acc;
        }
        if (acc) {
          commit_atoms(hd, na, a0m);
          bS = bP;
        }
        bP = -1;
        have_next = false;
        __syncthreads();
        if (t + 1 < A.n) {
          if (!adjust_before(t + 1, bnd))
            return;
          build_ctx(A, S, t + 1, hd, acc, 0, CT);
          if (!grid_sync(A.bar, G, S.gen, b.err, &S.flag, A.spin))
            return;
        }
        pend = false;
      }
      mark(4);
      mol_cur = mol_next;
      // the headers' roles: this move's becomes the previous one's, the
      // prefetched one (or a free buffer) this move's
      const int hfree = hq;
      hq = hc;
      hc = hn;
      hn = hfree;
    }
  }
  if (prof) {
    for (int ph = 0; ph < 5; ++ph)
      A.prof[5 * pslot + ph] += pacc[ph];
    A.prof[10 + pslot] += A.n;
  }
  // write back this CTA's structure factors; the decider the settings and
  // the running energies
  for (int i = threadIdx.x; i < kc; i += CT) {
    b.sumRref[kbeg + i] = KR(bS)[i];
    b.sumIref[kbeg + i] = KI(bS)[i];
  }
  if (leader && threadIdx.x == 0) {
    *A.set = S.set;
    for (int i = 0; i < 5; ++i)
      b.energy[i] = S.e_run[i];
  }
}
