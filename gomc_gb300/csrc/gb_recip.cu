// Ewald reciprocal-space kernels (FP64 plain form).
//
//   structure factor  sumR/I[k] = sum_j q_j {cos, sin}(k . r_j)
//                     (Ewald::BoxReciprocalSetup/Sums, src/Ewald.cpp:193-361)
//   energy            sum_k prefact_k (sumR^2 + sumI^2)
//                     (Ewald::BoxReciprocal, src/Ewald.cpp:375-406)
//   molecule delta    sumNew = sumRef + new - old, energy difference
//                     (Ewald::MolReciprocal, src/Ewald.cpp:409-473) and the
//                     insert / delete deltas (SwapDestRecip / SwapSourceRecip,
//                     src/Ewald.cpp:478-531, 657-710)
//   reciprocal force  (Ewald::BoxForceReciprocal, src/Ewald.cpp:1496-1596)
//
// The full-box kernels evaluate exp(i k.r) as a product of per-axis phase
// factors exp(i n_x t_x) exp(i n_y t_y) exp(i n_z t_z), t = 2 pi r / L, held
// per atom in shared memory; each CTA owns a chunk of k-vectors (the
// structure factor: runs of consecutive n_x) and one chunk of atoms, and
// chunk partials are added in a fixed order.
#include "gb_box.h"
#include "gb_f32math.cuh"
#include "gb_pair.cuh"

namespace gb {

constexpr int KT = 256;     // threads per reciprocal CTA
constexpr int TA = 16;      // atoms per shared-memory tile
constexpr int NCH_MAX = 64; // atom chunks

struct Phase {
  double2 *e;  // [atoms][3][kmax + 1]
  int stride;  // kmax + 1
};

// exp(i n t) for n = 0..kmax by recurrence from exp(i t).
__device__ __forceinline__ void phase_row(double2 *row, double t, int kmax) {
  double s, c;
  sincos(t, &s, &c);
  double2 e = make_double2(1.0, 0.0);
  row[0] = e;
  for (int n = 1; n <= kmax; ++n) {
    double re = e.x * c - e.y * s;
    double im = e.x * s + e.y * c;
    e = make_double2(re, im);
    row[n] = e;
  }
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 pick(const double2 *row, int n) {
  double2 v = row[n < 0 ? -n : n];
  if (n < 0)
    v.y = -v.y;
  return v;
}

// One thread per run of up to KRUN k-vectors sharing (n_y, n_z) with
// consecutive n_x: per atom, exp(i(n_y t_y + n_z t_z)) is formed once and
// exp(i n_x t_x) advances along the run by multiplying with exp(i t_x).
__global__ void __launch_bounds__(KT) k_recip_sums(DevBox b, const double *__restrict__ X,
                                                   const double *__restrict__ Y,
                                                   const double *__restrict__ Z,
                                                   int nch, double *part) {
  extern __shared__ double2 tab[];
  __shared__ double qs[TA];
  int stride = b.kmax + 1;
  int run = blockIdx.x * KT + threadIdx.x;
  int ch = blockIdx.y;
  int a_begin = (int)((long long)b.n_atoms * ch / nch);
  int a_end = (int)((long long)b.n_atoms * (ch + 1) / nch);
  int4 rn = run < b.nrun ? b.krun[run] : make_int4(0, 0, 0, 0);
  // members of this warp's longest run (runs are sorted longest first)
  const int wlen = __reduce_max_sync(0xffffffffu, rn.w);
  double sR[KRUN], sI[KRUN];
#pragma unroll
  for (int g = 0; g < KRUN; ++g) {
    sR[g] = 0.0;
    sI[g] = 0.0;
  }
  double cv[3];
  for (int d = 0; d < 3; ++d) {
    cv[d] = 1.0 / b.L[d];
    cv[d] *= 2.0 * M_PI;
  }
  for (int a0 = a_begin; a0 < a_end; a0 += TA) {
    int na = min(TA, a_end - a0);
    __syncthreads();
    if (threadIdx.x < na * 3) {
      int a = threadIdx.x / 3, d = threadIdx.x % 3;
      int atom = a0 + a;
      double coord = d == 0 ? X[atom] : d == 1 ? Y[atom] : Z[atom];
      phase_row(tab + (a * 3 + d) * stride, cv[d] * coord, b.kmax);
    }
    if (threadIdx.x < na) {
      double q = b.q[a0 + threadIdx.x];
      qs[threadIdx.x] = fabs(q) < 0.000000001 ? 0.0 : q;
    }
    __syncthreads();
    for (int a = 0; a < na; ++a) {
      double q = qs[a];
      if (q == 0.0)
        continue;
      const double2 *ex = tab + (a * 3 + 0) * stride;
      const double2 *ey = tab + (a * 3 + 1) * stride;
      const double2 *ez = tab + (a * 3 + 2) * stride;
      double2 step = ex[1];
      double2 e = cmul(ex[rn.z], cmul(pick(ey, rn.x), pick(ez, rn.y)));
#pragma unroll
      for (int g = 0; g < KRUN; ++g) {
        if (g < wlen) {
          sR[g] += q * e.x;
          sI[g] += q * e.y;
          e = cmul(e, step);
        }
      }
    }
  }
  if (run < b.nrun) {
#pragma unroll
    for (int g = 0; g < KRUN; ++g) {
      if (g < rn.w) {
        int k = b.krun_k[(size_t)run * KRUN + g];
        part[((size_t)ch * b.K + k) * 2] = sR[g];
        part[((size_t)ch * b.K + k) * 2 + 1] = sI[g];
      }
    }
  }
}

__global__ void k_recip_chunk_sum(int K, int nch, const double *__restrict__ part,
                                  double *sumR, double *sumI) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K)
    return;
  double r = 0.0, i = 0.0;
  for (int c = 0; c < nch; ++c) {
    r += part[((size_t)c * K + k) * 2];
    i += part[((size_t)c * K + k) * 2 + 1];
  }
  sumR[k] = r;
  sumI[k] = i;
}

// Structure factor in float-float arithmetic, the set-up and periodic
// recompute of the mixed form.  Positions enter as exact 64-bit fractions of
// a turn (u = r / L 2^64), so every phase n u is exact integer arithmetic;
// each CTA tile builds the rows exp(2 pi i n u / 2^64), n = 0..kmax, of its
// atoms directly from the phase (no recurrence), the x row scaled by the
// atom's charge, and a thread's run of k-vectors takes
// q exp(i n_x t_x) * (exp(i n_y t_y) exp(i n_z t_z)) per member, summed in
// float-float.  Each term carries a relative error of a few 2^-48, about
// 1e-14, against 1e-16 for the FP64 kernel above, at the FP32 rate.
constexpr int TAF = 16;  // atoms per tile

__global__ void __launch_bounds__(KT) k_recip_sums_ff(DevBox b,
                                                      const double *__restrict__ X,
                                                      const double *__restrict__ Y,
                                                      const double *__restrict__ Z,
                                                      int nch, double *part) {
  extern __shared__ float4 rows[];  // [TAF][3][kmax + 1]
  __shared__ float4 ctab[256];
  __shared__ unsigned long long tu[TAF * 3];
  __shared__ float2 qs[TAF];
  const int stride = b.kmax + 1;
  for (int i = threadIdx.x; i < 256; i += KT)
    ctab[i] = b.cis256[i];
  const int run = blockIdx.x * KT + threadIdx.x;
  const int ch = blockIdx.y;
  const int a_begin = (int)((long long)b.n_atoms * ch / nch);
  const int a_end = (int)((long long)b.n_atoms * (ch + 1) / nch);
  const int4 rn = run < b.nrun ? b.krun[run] : make_int4(0, 0, 0, 0);
  // members of this warp's longest run (runs are sorted longest first)
  const int wlen = __reduce_max_sync(0xffffffffu, rn.w);
  float rh[KRUN], rl[KRUN], ih[KRUN], il[KRUN];
#pragma unroll
  for (int g = 0; g < KRUN; ++g) {
    rh[g] = 0.0f;
    rl[g] = 0.0f;
    ih[g] = 0.0f;
    il[g] = 0.0f;
  }
  const int per_atom = 3 * stride;
  for (int a0 = a_begin; a0 < a_end; a0 += TAF) {
    const int na = min(TAF, a_end - a0);
    __syncthreads();
    if (threadIdx.x < na * 3) {
      int a = threadIdx.x / 3, d = threadIdx.x % 3;
      int atom = a0 + a;
      double coord = d == 0 ? X[atom] : d == 1 ? Y[atom] : Z[atom];
      double t = coord * b.invL[d];
      t -= floor(t);
      tu[threadIdx.x] = __double2ull_rn(t * 18446744073709551616.0);  // 2^64
    }
    if (threadIdx.x < na) {
      double q = b.q[a0 + threadIdx.x];
      if (fabs(q) < 0.000000001)
        q = 0.0;
      float hi = (float)q;
      qs[threadIdx.x] = make_float2(hi, (float)(q - (double)hi));
    }
    __syncthreads();
    for (int e = threadIdx.x; e < na * per_atom; e += KT) {
      int a = e / per_atom;
      int r = e - a * per_atom;
      int d = r / stride;
      int n = r - d * stride;
      float4 v = cis_turns64_ff(tu[a * 3 + d] * (unsigned long long)n, ctab);
      if (d == 0) {
        float2 q = qs[a];
        ff2 re = ff_mul({v.x, v.y}, {q.x, q.y});
        ff2 im = ff_mul({v.z, v.w}, {q.x, q.y});
        v = make_float4(re.hi, re.lo, im.hi, im.lo);
      }
      rows[e] = v;
    }
    __syncthreads();
    for (int a = 0; a < na; ++a) {
      if (qs[a].x == 0.0f)
        continue;
      const float4 *ex = rows + a * per_atom;
      const float4 *ey = ex + stride;
      const float4 *ez = ey + stride;
      float4 eyz = ffc_mul(ffc_conj_if(ey[abs(rn.x)], rn.x < 0),
                           ffc_conj_if(ez[abs(rn.y)], rn.y < 0));
#pragma unroll
      for (int g = 0; g < KRUN; ++g) {
        if (g < wlen) {
          // (hi, lo) += v without renormalising: the error-free sum's
          // remainder and v's low part collect in lo, which the end of
          // the tile folds back (lo stays within a few ulp of hi)
          float4 v = ffc_mul(ex[min(rn.z + g, b.kmax)], eyz);
          ff2 sr = ff_two_sum(rh[g], v.x);
          ff2 si = ff_two_sum(ih[g], v.z);
          rh[g] = sr.hi;
          rl[g] += sr.lo + v.y;
          ih[g] = si.hi;
          il[g] += si.lo + v.w;
        }
      }
    }
#pragma unroll
    for (int g = 0; g < KRUN; ++g) {
      ff2 r = ff_quick(rh[g], rl[g]);
      ff2 i = ff_quick(ih[g], il[g]);
      rh[g] = r.hi;
      rl[g] = r.lo;
      ih[g] = i.hi;
      il[g] = i.lo;
    }
  }
  if (run < b.nrun) {
#pragma unroll
    for (int g = 0; g < KRUN; ++g) {
      if (g < rn.w) {
        int k = b.krun_k[(size_t)run * KRUN + g];
        part[((size_t)ch * b.K + k) * 2] = (double)rh[g] + (double)rl[g];
        part[((size_t)ch * b.K + k) * 2 + 1] = (double)ih[g] + (double)il[g];
      }
    }
  }
}

static int recip_chunks(const Box &bx, const DevBox &b) {
  int kb = (b.nrun + KT - 1) / KT;
  int want = (4 * bx.sm_count + kb - 1) / kb;
  int nch = std::max(1, std::min(NCH_MAX, want));
  int maxch = std::max(1, b.n_atoms / TA);
  return std::min(nch, maxch);
}

int launch_recip_sums(Box &bx, const double *x, const double *y,
                      const double *z, double *sumR, double *sumI) {
  return launch_recip_sums_view(bx, bx.dev, x, y, z, sumR, sumI);
}

// The structure factor on a view: its k-vector set, its edges (the phases
// are 2 pi n x / L) and the given coordinates.
int launch_recip_sums_view(Box &bx, const DevBox &b, const double *x,
                           const double *y, const double *z, double *sumR,
                           double *sumI) {
  int nch = recip_chunks(bx, b);
  int rc = bx.EnsureScratch((size_t)nch * b.K * 2);
  if (rc)
    return rc;
  int kb = (b.nrun + KT - 1) / KT;
  size_t sh = (size_t)TA * 3 * (b.kmax + 1) * sizeof(double2) + 16;
  raise_smem_limit((const void *)k_recip_sums, sh);
  k_recip_sums<<<dim3(kb, nch), KT, sh, bx.stream>>>(b, x, y, z, nch,
                                                     bx.d_scratch);
  k_recip_chunk_sum<<<(b.K + 255) / 256, 256, 0, bx.stream>>>(
      b.K, nch, bx.d_scratch, sumR, sumI);
  return bx.CudaCheck(cudaGetLastError(), "recip sums");
}

int launch_recip_sums_ff(Box &bx, const double *x, const double *y,
                         const double *z, double *sumR, double *sumI) {
  DevBox &b = bx.dev;
  int kb = (b.nrun + KT - 1) / KT;
  size_t sh = (size_t)TAF * 3 * (b.kmax + 1) * sizeof(float4);
  raise_smem_limit((const void *)k_recip_sums_ff, sh);
  // atom chunks: as many CTAs as the GPU holds at once (whole waves, no
  // tail), each chunk at least one atom tile
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_recip_sums_ff,
                                                    KT, sh) != cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  int nch = std::max(1, bx.sm_count * per_sm / kb);
  nch = std::min(nch, NCH_MAX);
  nch = std::min(nch, std::max(1, b.n_atoms / TAF));
  int rc = bx.EnsureScratch((size_t)nch * b.K * 2);
  if (rc)
    return rc;
  k_recip_sums_ff<<<dim3(kb, nch), KT, sh, bx.stream>>>(b, x, y, z, nch,
                                                        bx.d_scratch);
  k_recip_chunk_sum<<<(b.K + 255) / 256, 256, 0, bx.stream>>>(
      b.K, nch, bx.d_scratch, sumR, sumI);
  return bx.CudaCheck(cudaGetLastError(), "recip sums (float-float)");
}

// ---------------------------------------------------------------------------
// Energy of a set of structure factors
// ---------------------------------------------------------------------------
constexpr int ET = 256;
__global__ void k_recip_energy(DevBox b, const double *__restrict__ sR,
                               const double *__restrict__ sI, double *part) {
  int k = blockIdx.x * ET + threadIdx.x;
  double e = 0.0;
  if (k < b.K)
    e = ((sR[k] * sR[k] + sI[k] * sI[k]) * b.prefact[k]);
  __shared__ double red[ET / 32];
  double s = block_sum<ET>(e, red);
  if (threadIdx.x == 0)
    part[blockIdx.x] = s;
}

__global__ void k_sum_in_order(const double *__restrict__ part, int n,
                               const double *sub, double *out) {
  __shared__ double red[ET / 32];
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += ET)
    v += part[i];
  double s = block_sum<ET>(v, red);
  if (threadIdx.x == 0)
    out[0] = sub ? s - sub[0] : s;
}

int launch_recip_energy(Box &bx, const double *sumR, const double *sumI,
                        double *d_out) {
  return launch_recip_energy_view(bx, bx.dev, sumR, sumI, d_out);
}

// The energy of sums with the prefactors and k count of a view (the New
// k-vector set for a trial volume).
int launch_recip_energy_view(Box &bx, const DevBox &b, const double *sumR,
                             const double *sumI, double *d_out) {
  int nb = (b.K + ET - 1) / ET;
  int rc = bx.EnsureScratch(nb);
  if (rc)
    return rc;
  k_recip_energy<<<nb, ET, 0, bx.stream>>>(b, sumR, sumI, bx.d_scratch);
  k_sum_in_order<<<1, ET, 0, bx.stream>>>(bx.d_scratch, nb, nullptr, d_out);
  return bx.CudaCheck(cudaGetLastError(), "recip energy");
}

// ---------------------------------------------------------------------------
// One-molecule delta.  mode 0: displacement/rotation (new - old),
// 1: insertion (+ new), 2: deletion (- given positions).  One thread per k,
// with the reference's dot-product phases.
// ---------------------------------------------------------------------------
__global__ void k_mol_recip(DevBox b, int m, const double *__restrict__ newpos,
                            int mode, double *part) {
  int k = blockIdx.x * ET + threadIdx.x;
  double e = 0.0;
  if (k < b.K) {
    int a0 = b.mstart[m], n = b.mstart[m + 1] - a0;
    double kx = b.kx[k], ky = b.ky[k], kz = b.kz[k];
    double rN = 0, iN = 0, rO = 0, iO = 0;
    for (int p = 0; p < n; ++p) {
      int a = a0 + p;
      double q = b.q[a];
      if (fabs(q) < 0.000000001)
        continue;
      double dn = (newpos[3 * p] * kx + newpos[3 * p + 1] * ky +
                   newpos[3 * p + 2] * kz);
      double s, c;
      sincos(dn, &s, &c);
      rN += q * c;
      iN += q * s;
      if (mode == 0) {
        double dold = (b.x[a] * kx + b.y[a] * ky + b.z[a] * kz);
        sincos(dold, &s, &c);
        rO += q * c;
        iO += q * s;
      }
    }
    double sr, si;
    if (mode == 0) {
      sr = b.sumRref[k] + 1.0 * (rN - rO);
      si = b.sumIref[k] + 1.0 * (iN - iO);
    } else if (mode == 1) {
      sr = b.sumRref[k] + rN;
      si = b.sumIref[k] + iN;
    } else {
      sr = b.sumRref[k] - rN;
      si = b.sumIref[k] - iN;
    }
    b.sumRnew[k] = sr;
    b.sumInew[k] = si;
    e = (sr * sr + si * si) * b.prefact[k];
  }
  __shared__ double red[ET / 32];
  double s = block_sum<ET>(e, red);
  if (threadIdx.x == 0)
    part[blockIdx.x] = s;
}

int launch_mol_recip(Box &bx, int m, const double *d_newpos, int mode,
                     double *d_out) {
  DevBox &b = bx.dev;
  int nb = (b.K + ET - 1) / ET;
  int rc = bx.EnsureScratch(nb);
  if (rc)
    return rc;
  k_mol_recip<<<nb, ET, 0, bx.stream>>>(b, m, d_newpos, mode, bx.d_scratch);
  // energyRecipNew - sysPotRef.boxEnergy[box].recip
  k_sum_in_order<<<1, ET, 0, bx.stream>>>(bx.d_scratch, nb, b.energy + 2, d_out);
  return bx.CudaCheck(cudaGetLastError(), "mol recip");
}

// ---------------------------------------------------------------------------
// Reciprocal force on every atom, with the intramolecular erf correction.
// CTA = 64 atoms x one quarter of the k-vectors; thread = atom.
// ---------------------------------------------------------------------------
constexpr int FA = 64;      // atoms per CTA
constexpr int FK = 128;     // k-vectors staged per step
constexpr int FKS = 4;      // k splits
__global__ void __launch_bounds__(FA) k_force_recip(DevBox b, const FF *__restrict__ pff,
                                                    const double *__restrict__ sR,
                                                    const double *__restrict__ sI,
                                                    int intra, double *fpart) {
  extern __shared__ double2 tab[];
  const FF &ff = *pff;
  int stride = b.kmax + 1;
  int pad = 3 * stride + 1;  // per-atom table stride (odd) against conflicts
  double2 *ktab = tab + (size_t)FA * pad;
  double *kxs = (double *)ktab;
  // per k-vector: the components of k and the prefactor times the
  // structure factor, prefact * (sumR, sumI)
  double *kys = kxs + FK, *kzs = kys + FK, *pas = kzs + FK, *pbs = pas + FK;
  char4 *kns = (char4 *)(pbs + FK);
  int a = blockIdx.x * FA + threadIdx.x;
  bool own = a < b.n_atoms;
  double cv[3];
  for (int d = 0; d < 3; ++d) {
    cv[d] = 1.0 / b.L[d];
    cv[d] *= 2.0 * M_PI;
  }
  double q = 0.0, FX = 0.0, FY = 0.0, FZ = 0.0;
  double2 *my = tab + (size_t)threadIdx.x * pad;
  if (own) {
    q = b.q[a];
    phase_row(my, cv[0] * b.x[a], b.kmax);
    phase_row(my + stride, cv[1] * b.y[a], b.kmax);
    phase_row(my + 2 * stride, cv[2] * b.z[a], b.kmax);
    if (intra && blockIdx.y == 0 && fabs(q) >= 0.000000001 && ff.ewald) {
      // intramolecular correction (src/Ewald.cpp:1556-1575)
      double constValue = ff.alpha * M_2_SQRTPI;
      int m = b.mol[a];
      for (int j = b.mstart[m]; j < b.mstart[m + 1]; j++) {
        if (j == a)
          continue;
        double dx = min_image(b.x[a] - b.x[j], b.L[0], b.half[0]);
        double dy = min_image(b.y[a] - b.y[j], b.L[1], b.half[1]);
        double dz = min_image(b.z[a] - b.z[j], b.L[2], b.half[2]);
        double distSq = dsq3(dx, dy, dz);
        double dist = sqrt(distSq);
        double expConstValue = exp(-1.0 * ff.alphaSq * distSq);
        double qiqj = q * b.q[j] * QQ_FACT;
        double intraForce = qiqj * 1.0 * 1.0 / distSq;
        intraForce *= ((erf(ff.alpha * dist) / dist) - constValue * expConstValue);
        FX -= intraForce * dx;
        FY -= intraForce * dy;
        FZ -= intraForce * dz;
      }
    }
  }
  bool charged = own && fabs(q) >= 0.000000001 && ff.ewald;
  int kper = (b.K + FKS - 1) / FKS;
  int kbeg = blockIdx.y * kper, kend = min(b.K, kbeg + kper);
  double fx = 0.0, fy = 0.0, fz = 0.0;
  for (int k0 = kbeg; k0 < kend; k0 += FK) {
    int nk = min(FK, kend - k0);
    __syncthreads();
    for (int i = threadIdx.x; i < nk; i += FA) {
      int k = k0 + i;
      kxs[i] = b.kx[k];
      kys[i] = b.ky[k];
      kzs[i] = b.kz[k];
      const double pf = b.prefact[k];
      pas[i] = pf * sR[k];
      pbs[i] = pf * sI[k];
      kns[i] = b.kn[k];
    }
    __syncthreads();
    if (!charged)
      continue;
    // Ewald::BoxForceReciprocal: factor_k = 2 q prefact_k (sin(k.r) sumR -
    // cos(k.r) sumI), F += factor_k k.  The common 2 q is applied once per
    // atom; the k-vectors run x outer, y, z inner, so the x-y phase product
    // is formed once per (n_x, n_y) column.
    int px = -1000, py = -1000;
    double2 exy = make_double2(0.0, 0.0);
    for (int i = 0; i < nk; ++i) {
      const char4 n = kns[i];
      if (n.x != px || n.y != py) {
        exy = cmul(my[n.x], pick(my + stride, n.y));
        px = n.x;
        py = n.y;
      }
      const double2 e = cmul(exy, pick(my + 2 * stride, n.z));
      const double t = e.y * pas[i] - e.x * pbs[i];
      fx += t * kxs[i];
      fy += t * kys[i];
      fz += t * kzs[i];
    }
  }
  if (own) {
    const double q2 = 2.0 * q;
    double *f = fpart + ((size_t)blockIdx.y * b.n_atoms + a) * 3;
    f[0] = q2 * fx + (blockIdx.y == 0 ? FX : 0.0);
    f[1] = q2 * fy + (blockIdx.y == 0 ? FY : 0.0);
    f[2] = q2 * fz + (blockIdx.y == 0 ? FZ : 0.0);
  }
}

__global__ void k_force_recip_gather(DevBox b, const double *__restrict__ fpart,
                                     double *aR, double *mR) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= b.n_mol)
    return;
  double mx = 0, my = 0, mz = 0;
  for (int a = b.mstart[m]; a < b.mstart[m + 1]; ++a) {
    double f[3] = {0, 0, 0};
    for (int s = 0; s < FKS; ++s)
      for (int d = 0; d < 3; ++d)
        f[d] += fpart[((size_t)s * b.n_atoms + a) * 3 + d];
    for (int d = 0; d < 3; ++d)
      aR[3 * (size_t)a + d] = f[d];
    mx += f[0];
    my += f[1];
    mz += f[2];
  }
  mR[3 * (size_t)m] = mx;
  mR[3 * (size_t)m + 1] = my;
  mR[3 * (size_t)m + 2] = mz;
}

int launch_force_recip(Box &bx, const DevBox &b, const double *sumR,
                       const double *sumI, double *aR, double *mR) {
  if (!bx.cfg.ewald) {
    cudaMemsetAsync(aR, 0, (size_t)b.n_atoms * 24, bx.stream);
    cudaMemsetAsync(mR, 0, (size_t)b.n_mol * 24, bx.stream);
    return bx.CudaCheck(cudaGetLastError(), "force recip");
  }
  int rc = bx.EnsureScratch((size_t)FKS * b.n_atoms * 3);
  if (rc)
    return rc;
  int pad = 3 * (b.kmax + 1) + 1;
  size_t sh = (size_t)FA * pad * sizeof(double2) + (size_t)FK * (6 * 8 + 4);
  raise_smem_limit((const void *)k_force_recip, sh);
  dim3 grid((b.n_atoms + FA - 1) / FA, FKS);
  k_force_recip<<<grid, FA, sh, bx.stream>>>(b, bx.d_ff, sumR, sumI, 1,
                                             bx.d_scratch);
  k_force_recip_gather<<<(b.n_mol + 127) / 128, 128, 0, bx.stream>>>(
      b, bx.d_scratch, aR, mR);
  return bx.CudaCheck(cudaGetLastError(), "force recip");
}

}  // namespace gb

namespace gb {

// ---------------------------------------------------------------------------
// Reciprocal virial (Ewald::VirialReciprocal, src/Ewald.cpp:1168-1305) from
// the Ref structure factors: the k-space sum, one thread per k-vector,
//   w_d += prefact |S|^2 (1 - 2 (1/(4 alpha^2) + 1/k^2) k_d^2),
// and the intramolecular part, one thread per atom,
//   w_d += -F_d (r_d - com_d),
// F the reciprocal force of the atom without the intramolecular correction
// (k_force_recip with intra = 0): sum_k 2 q prefact (S_I cos - S_R sin) k_d
// is -F_d.  Partials per CTA, three per row.
// ---------------------------------------------------------------------------
constexpr int VT = 256;
__global__ void k_virial_k(DevBox b, const FF *__restrict__ pff,
                           double *part) {
  const FF &ff = *pff;
  int k = blockIdx.x * VT + threadIdx.x;
  double w[3] = {0.0, 0.0, 0.0};
  if (k < b.K) {
    double constVal = 1.0 / (4.0 * ff.alphaSq);
    double factor = b.prefact[k] * (b.sumRref[k] * b.sumRref[k] +
                                    b.sumIref[k] * b.sumIref[k]);
    double c = 2.0 * (constVal + 1.0 / b.hsqr[k]);
    double kv[3] = {b.kx[k], b.ky[k], b.kz[k]};
    for (int d = 0; d < 3; ++d)
      w[d] = factor * (1.0 - c * kv[d] * kv[d]);
  }
  __shared__ double red[VT / 32];
  for (int d = 0; d < 3; ++d) {
    double r = block_sum<VT>(w[d], red);
    if (threadIdx.x == 0)
      part[3 * blockIdx.x + d] = r;
  }
}

__global__ void k_virial_intra(DevBox b, const double *__restrict__ fpart,
                               int nchunk, double *part) {
  int a = blockIdx.x * VT + threadIdx.x;
  double w[3] = {0.0, 0.0, 0.0};
  if (a < b.n_atoms && fabs(b.q[a]) >= 0.000000001) {
    int m = b.mol[a];
    double com[3] = {b.cx[m], b.cy[m], b.cz[m]};
    double pos[3] = {b.x[a], b.y[a], b.z[a]};
    for (int d = 0; d < 3; ++d) {
      double F = 0.0;
      for (int c = 0; c < nchunk; ++c)
        F += fpart[((size_t)c * b.n_atoms + a) * 3 + d];
      double diff = unwrap1(pos[d], com[d], b.L[d], b.half[d]) - com[d];
      w[d] = -F * diff;
    }
  }
  __shared__ double red[VT / 32];
  for (int d = 0; d < 3; ++d) {
    double r = block_sum<VT>(w[d], red);
    if (threadIdx.x == 0)
      part[3 * blockIdx.x + d] = r;
  }
}

__global__ void k_sum3(const double *__restrict__ part, int n, double *out) {
  __shared__ double red[VT / 32];
  for (int d = 0; d < 3; ++d) {
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += VT)
      v += part[3 * i + d];
    double r = block_sum<VT>(v, red);
    if (threadIdx.x == 0)
      out[d] = r;
  }
}

// d_out6: k-space sum (xx, yy, zz), then the intramolecular part
int launch_virial_recip(Box &bx, double *d_out6) {
  DevBox &b = bx.dev;
  int nkb = (b.K + VT - 1) / VT, nab = (b.n_atoms + VT - 1) / VT;
  size_t fp = (size_t)FKS * b.n_atoms * 3;
  int rc = bx.EnsureScratch(fp + 3 * (size_t)(nkb + nab));
  if (rc)
    return rc;
  double *kpart = bx.d_scratch + fp, *ipart = kpart + 3 * (size_t)nkb;
  int pad = 3 * (b.kmax + 1) + 1;
  size_t sh = (size_t)FA * pad * sizeof(double2) + (size_t)FK * (6 * 8 + 4);
  raise_smem_limit((const void *)k_force_recip, sh);
  dim3 grid((b.n_atoms + FA - 1) / FA, FKS);
  k_force_recip<<<grid, FA, sh, bx.stream>>>(b, bx.d_ff, b.sumRref, b.sumIref,
                                             0, bx.d_scratch);
  k_virial_k<<<nkb, VT, 0, bx.stream>>>(b, bx.d_ff, kpart);
  k_virial_intra<<<nab, VT, 0, bx.stream>>>(b, bx.d_scratch, FKS, ipart);
  k_sum3<<<1, VT, 0, bx.stream>>>(kpart, nkb, d_out6);
  k_sum3<<<1, VT, 0, bx.stream>>>(ipart, nab, d_out6 + 3);
  return bx.CudaCheck(cudaGetLastError(), "virial recip");
}

}  // namespace gb
