// Real-space kernels (FP64 plain form):
//   BoxInter        one CTA per (cell, neighbour) tile, i < j pairs
//                   (src/CalculateEnergy.cpp:157-266)
//   MoleculeInter   one CTA per (atom, old/new, neighbour cell)
//                   (src/CalculateEnergy.cpp:581-686)
//   ParticleInter   one CTA per (trial, neighbour cell)
//                   (src/CalculateEnergy.cpp:727-785)
//   BoxForce        one CTA per (cell, third of the neighbour shell); each
//                   thread gathers the force on one atom, so no atomics
//                   (src/CalculateEnergy.cpp:268-406)
//   MolCorrection   per molecule (src/Ewald.cpp:1056-1085)
//   CalculateTorque per molecule (src/CalculateEnergy.cpp:1365-1406)
// Partial sums land in per-CTA slots and a final single-CTA kernel adds them
// in a fixed order, so every result is reproducible run to run.
#include "gb_box.h"
#include "gb_cells.cuh"
#include "gb_pair.cuh"

namespace gb {

constexpr int RT = 128;  // threads per real-space CTA

// Sum `n` partials of width `w` (stride w) into out[0..w), fixed order.
__global__ void k_reduce_partials(const double *__restrict__ part, int n, int w,
                                  double *out, int max_mode) {
  __shared__ double sh[RT / 32];
  for (int c = 0; c < w; ++c) {
    double v = 0.0;
    if (max_mode && c == w - 1) {
      for (int i = threadIdx.x; i < n; i += RT)
        v = fmax(v, part[(size_t)i * w + c]);
      for (int o = 16; o > 0; o >>= 1)
        v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
      if ((threadIdx.x & 31) == 0)
        sh[threadIdx.x >> 5] = v;
      __syncthreads();
      if (threadIdx.x == 0) {
        double r = 0;
        for (int i = 0; i < RT / 32; ++i)
          r = fmax(r, sh[i]);
        out[c] = r;
      }
      __syncthreads();
      continue;
    }
    for (int i = threadIdx.x; i < n; i += RT)
      v += part[(size_t)i * w + c];
    double r = block_sum<RT>(v, sh);
    if (threadIdx.x == 0)
      out[c] = r;
  }
}

// ---------------------------------------------------------------------------
// BoxInter
// ---------------------------------------------------------------------------
// A warp scans its 32 atoms of cell c against the neighbour cell with an
// FP32 distance pre-filter (its radius padded beyond FP32 position
// rounding) and queues the candidate pairs (i < j atom ids, other molecule)
// in shared memory; every 32 queued pairs are evaluated in FP64 by the full
// warp, with the exact FP64 cutoff test.  The FP64 energy work then scales
// with the pairs inside the cutoff, not with the pairs scanned.
constexpr int QW = 64;  // queue slots per warp

// Bulk asynchronous copies (the TMA engine's untiled form) from global to
// this CTA's shared memory, completed on an mbarrier: the copy engine moves
// a cell's slots while no thread issues a load.  Addresses and sizes are
// multiples of 16 bytes (cell slot arrays are padded to multiples of 32).
__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src,
                                         unsigned bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait on phase 0 of the barrier; false (and the box's error word
// set) when it gives up, after a second bounded wait for the copies.
__device__ bool mbar_wait_bounded(uint64_t *bar, int *err) {
  constexpr unsigned LIMIT = 1u << 22;
  for (unsigned it = 0; it < LIMIT; ++it)
    if (mbar_try_wait(bar, 0))
      return true;
  atomicOr(err, DERR_BARRIER_TIMEOUT);
  for (unsigned it = 0; it < LIMIT; ++it)
    if (mbar_try_wait(bar, 0))
      break;
  return false;
}

// One CTA per (cell c, neighbour cell c2) tile.  Thread 0 starts bulk copies
// of both cells' slots (positions and charges, meta words, atom ids) into
// shared memory; then every warp scans 32 atoms of c against c2.
__global__ void __launch_bounds__(RT) k_box_inter(DevBox b, const FF *__restrict__ pff,
                                                  double *part) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ int2 queue[RT / 32][QW];
  __shared__ __align__(8) uint64_t bar;
  const FF &ff = *pff;
  int tile = blockIdx.x;
  int c = tile / NB27, n = tile % NB27;
  int c2 = b.nbr[c * NB27 + n];
  int n1 = b.cell_count[c], n2 = b.cell_count[c2];
  if (n1 == 0 || n2 == 0) {  // no pair in this tile
    if (threadIdx.x == 0) {
      part[2 * tile] = 0.0;
      part[2 * tile + 1] = 0.0;
    }
    return;
  }
  const int cap = b.cap;
  double4_32a *sp = (double4_32a *)smem;  // neighbour cell c2
  float4 *sf = (float4 *)(sp + cap);
  int *sm = (int *)(sf + cap);
  int *sa = sm + cap;
  double4_32a *cp = (double4_32a *)(sa + cap);  // cell c
  int *cm = (int *)(cp + cap);
  int *ca = cm + cap;
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar))
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    const unsigned p1 = (unsigned)n1 * 32, p2 = (unsigned)n2 * 32;
    const unsigned w1 = (unsigned)((n1 + 3) & ~3) * 4;
    const unsigned w2 = (unsigned)((n2 + 3) & ~3) * 4;
    asm volatile(
        "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
            smem_u32(&bar)),
        "r"(p1 + p2 + 2 * (w1 + w2))
        : "memory");
    const size_t o1 = (size_t)c * cap, o2 = (size_t)c2 * cap;
    bulk_g2s(sp, b.cell_pos + o2, p2, &bar);
    bulk_g2s(sm, b.cell_meta + o2, w2, &bar);
    bulk_g2s(sa, b.cell_atom + o2, w2, &bar);
    bulk_g2s(cp, b.cell_pos + o1, p1, &bar);
    bulk_g2s(cm, b.cell_meta + o1, w1, &bar);
    bulk_g2s(ca, b.cell_atom + o1, w1, &bar);
  }
  __syncthreads();  // the barrier is initialised before anyone waits on it
  const bool ok = mbar_wait_bounded(&bar, b.err);
  if (!ok)
    return;  // the error word reports it; no partial is read
  for (int j = threadIdx.x; j < n2; j += RT) {
    const double4_32a p = sp[j];
    sf[j] = make_float4((float)p.x, (float)p.y, (float)p.z, 0.0f);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const float Lf[3] = {(float)b.L[0], (float)b.L[1], (float)b.L[2]};
  const float Hf[3] = {(float)b.half[0], (float)b.half[1], (float)b.half[2]};
  // FP32 positions are within L 2^-24 of the FP64 ones; the pre-filter
  // radius covers twice that per axis plus 1e-4 of Rcut^2
  const double lmax = fmax(b.L[0], fmax(b.L[1], b.L[2]));
  const double rpad = ff.rcut + 1e-6 * lmax;
  const float cut_f = (float)(rpad * rpad * 1.0001);
  int2 *q = queue[warp];
  double lj = 0.0, re = 0.0;
  // FP64 energy of queued pair e (slot of cell c, slot of the neighbour cell)
  auto eval = [&](int2 e) {
    double4_32a pi = cp[e.x];
    double4_32a pj = sp[e.y];
    double dx = min_image(pi.x - pj.x, b.L[0], b.half[0]);
    double dy = min_image(pi.y - pj.y, b.L[1], b.half[1]);
    double dz = min_image(pi.z - pj.z, b.L[2], b.half[2]);
    double distSq = dsq3(dx, dy, dz);
    if (ff.rcutSq > distSq) {
      int ki = meta_kind(cm[e.x]);
      int kj = meta_kind(sm[e.y]);
      if (ff.electrostatic) {
        double qq = pi.w * pj.w * QQ_FACT;
        if (qq != 0.0)
          re += coulomb_energy(ff, distSq, qq);
      }
      lj += lj_energy(ff, distSq, ki + kj * ff.n_kinds);
    }
  };
  int qn = 0;  // warp-uniform queue fill
  for (int i0 = warp * 32; i0 < n1; i0 += RT) {
    int i = i0 + lane;
    bool act = i < n1;
    int ai = -1, moli = -1;
    float px = 0.0f, py = 0.0f, pz = 0.0f;
    if (act) {
      double4_32a p = cp[i];
      px = (float)p.x;
      py = (float)p.y;
      pz = (float)p.z;
      ai = ca[i];
      moli = meta_mol(cm[i]);
    }
    for (int j = 0; j < n2; ++j) {
      bool in = false;
      if (act && ai < sa[j] && moli != meta_mol(sm[j])) {
        float4 pj = sf[j];
        float dx = px - pj.x, dy = py - pj.y, dz = pz - pj.z;
        dx = dx > Hf[0] ? dx - Lf[0] : dx < -Hf[0] ? dx + Lf[0] : dx;
        dy = dy > Hf[1] ? dy - Lf[1] : dy < -Hf[1] ? dy + Lf[1] : dy;
        dz = dz > Hf[2] ? dz - Lf[2] : dz < -Hf[2] ? dz + Lf[2] : dz;
        in = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) < cut_f;
      }
      unsigned m = __ballot_sync(0xffffffffu, in);
      if (in)
        q[qn + __popc(m & lt)] = make_int2(i, j);
      qn += __popc(m);
      if (qn >= 32) {
        __syncwarp();
        eval(q[lane]);
        int rest = qn - 32;
        int2 mv = lane < rest ? q[32 + lane] : make_int2(0, 0);
        __syncwarp();
        if (lane < rest)
          q[lane] = mv;
        __syncwarp();
        qn = rest;
      }
    }
  }
  __syncwarp();
  if (lane < qn)
    eval(q[lane]);
  __shared__ double red[RT / 32];
  double a = block_sum<RT>(lj, red);
  double r = block_sum<RT>(re, red);
  if (threadIdx.x == 0) {
    part[2 * tile] = a;
    part[2 * tile + 1] = r;
  }
}

// ---------------------------------------------------------------------------
// Pair virial (CalculateEnergy::VirialCalc CPU branch,
// src/CalculateEnergy.cpp:458-519): the BoxInter tiles, each pair's force
// factor times the product of its atom separation and the molecule-centre
// separation, diagonal components; partials = LJ xx, yy, zz, then the
// Coulomb factor (q_i q_j, without qqFact) xx, yy, zz.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(RT) k_box_virial(DevBox b, const FF *__restrict__ pff,
                                                   double *part) {
  extern __shared__ __align__(32) unsigned char smem[];
  const FF &ff = *pff;
  int tile = blockIdx.x;
  int c = tile / NB27, n = tile % NB27;
  int c2 = b.nbr[c * NB27 + n];
  int n1 = b.cell_count[c], n2 = b.cell_count[c2];
  double4_32a *sp = (double4_32a *)smem;
  int *sm = (int *)(sp + b.cap);
  int *sa = sm + b.cap;
  for (int j = threadIdx.x; j < n2; j += RT) {
    size_t s = (size_t)c2 * b.cap + j;
    sp[j] = b.cell_pos[s];
    sm[j] = b.cell_meta[s];
    sa[j] = b.cell_atom[s];
  }
  __syncthreads();
  double v[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < n1; i += RT) {
    size_t si = (size_t)c * b.cap + i;
    double4_32a pi = b.cell_pos[si];
    int mi = b.cell_meta[si], ai = b.cell_atom[si];
    int moli = meta_mol(mi), ki = meta_kind(mi);
    for (int j = 0; j < n2; ++j) {
      int aj = sa[j];
      int mj = sm[j];
      int molj = meta_mol(mj);
      if (!(ai < aj && moli != molj))
        continue;
      double4_32a pj = sp[j];
      double vc[3] = {min_image(pi.x - pj.x, b.L[0], b.half[0]),
                      min_image(pi.y - pj.y, b.L[1], b.half[1]),
                      min_image(pi.z - pj.z, b.L[2], b.half[2])};
      double distSq = dsq3(vc[0], vc[1], vc[2]);
      if (!(ff.rcutSq > distSq))
        continue;
      double cc[3] = {min_image(b.cx[moli] - b.cx[molj], b.L[0], b.half[0]),
                      min_image(b.cy[moli] - b.cy[molj], b.L[1], b.half[1]),
                      min_image(b.cz[moli] - b.cz[molj], b.L[2], b.half[2])};
      if (ff.electrostatic) {
        double qi_qj = pi.w * pj.w;
        if (qi_qj != 0.0) {
          double pRF = coulomb_virial(ff, distSq, qi_qj);
          for (int d = 0; d < 3; ++d)
            v[3 + d] += pRF * (vc[d] * cc[d]);
        }
      }
      double pVF = lj_virial(ff, distSq, ki + meta_kind(mj) * ff.n_kinds);
      for (int d = 0; d < 3; ++d)
        v[d] += pVF * (vc[d] * cc[d]);
    }
  }
  __shared__ double red[RT / 32];
  for (int d = 0; d < 6; ++d) {
    double r = block_sum<RT>(v[d], red);
    if (threadIdx.x == 0)
      part[6 * tile + d] = r;
  }
}

int launch_box_virial(Box &bx, double *d_out6) {
  DevBox &b = bx.dev;
  int tiles = b.ncell * NB27;
  int rc = bx.EnsureScratch((size_t)tiles * 6);
  if (rc)
    return rc;
  size_t sh = (size_t)b.cap * (sizeof(double4_32a) + 2 * sizeof(int));
  raise_smem_limit((const void *)k_box_virial, sh);
  k_box_virial<<<tiles, RT, sh, bx.stream>>>(b, bx.d_ff, bx.d_scratch);
  k_reduce_partials<<<1, RT, 0, bx.stream>>>(bx.d_scratch, tiles, 6, d_out6, 0);
  return bx.CudaCheck(cudaGetLastError(), "box virial");
}

int launch_box_inter(Box &bx, double *d_out2) {
  return launch_box_inter_view(bx, bx.dev, d_out2);
}

// BoxInter on a view (its coordinates, cell grid and edges).
int launch_box_inter_view(Box &bx, const DevBox &b, double *d_out2) {
  int tiles = b.ncell * NB27;
  int rc = bx.EnsureScratch((size_t)tiles * 2);
  if (rc)
    return rc;
  // neighbour cell: positions, FP32 copies, meta, atom ids; cell c:
  // positions, meta, atom ids
  size_t sh = (size_t)b.cap * (2 * sizeof(double4_32a) + sizeof(float4) +
                                4 * sizeof(int));
  raise_smem_limit((const void *)k_box_inter, sh);
  k_box_inter<<<tiles, RT, sh, bx.stream>>>(b, bx.d_ff, bx.d_scratch);
  k_reduce_partials<<<1, RT, 0, bx.stream>>>(bx.d_scratch, tiles, 2, d_out2, 0);
  return bx.CudaCheck(cudaGetLastError(), "box inter");
}

// ---------------------------------------------------------------------------
// MoleculeInter: unit u = ((atom * 2 + side) * 27 + neighbour)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(RT) k_mol_inter(DevBox b, const FF *__restrict__ pff,
                                                  int m, const double *__restrict__ newpos,
                                                  double *part) {
  const FF &ff = *pff;
  int u = blockIdx.x;
  int a = u / (2 * NB27), side = (u / NB27) % 2, n = u % NB27;
  int atom = b.mstart[m] + a;
  double px, py, pz;
  if (side == 0) {
    px = b.x[atom];
    py = b.y[atom];
    pz = b.z[atom];
  } else {
    px = newpos[3 * a];
    py = newpos[3 * a + 1];
    pz = newpos[3 * a + 2];
  }
  int cell = position_to_cell_fast(b, px, py, pz);
  int c2 = b.nbr[cell * NB27 + n];
  int n2 = b.cell_count[c2];
  double qa = b.q[atom];
  int ka = b.kind[atom];
  double lj = 0.0, re = 0.0, ovl = 0.0;
  for (int j = threadIdx.x; j < n2; j += RT) {
    size_t s = (size_t)c2 * b.cap + j;
    int mj = b.cell_meta[s];
    if (meta_mol(mj) == m)
      continue;  // the moving molecule is out of the cell list
    double4_32a pj = b.cell_pos[s];
    double dx = min_image(px - pj.x, b.L[0], b.half[0]);
    double dy = min_image(py - pj.y, b.L[1], b.half[1]);
    double dz = min_image(pz - pj.z, b.L[2], b.half[2]);
    double distSq = dsq3(dx, dy, dz);
    if (ff.rcutSq > distSq) {
      if (side == 1 && distSq < ff.rcutLowSq)
        ovl = 1.0;
      double e = 0.0;
      if (ff.electrostatic) {
        double qq = qa * pj.w * QQ_FACT;
        if (qq != 0.0)
          e = coulomb_energy(ff, distSq, qq);
      }
      double l = lj_energy(ff, distSq, ka + meta_kind(mj) * ff.n_kinds);
      if (side == 0) {
        re += -e;
        lj += -l;
      } else {
        re += e;
        lj += l;
      }
    }
  }
  __shared__ double red[RT / 32];
  double A = block_sum<RT>(lj, red);
  double R = block_sum<RT>(re, red);
  double O = block_sum<RT>(ovl, red);
  if (threadIdx.x == 0) {
    part[3 * u] = A;
    part[3 * u + 1] = R;
    part[3 * u + 2] = O > 0 ? 1.0 : 0.0;
  }
}

int launch_mol_inter(Box &bx, int m, const double *d_newpos, double *d_out3) {
  int na = bx.host.mstart[m + 1] - bx.host.mstart[m];
  int units = na * 2 * NB27;
  int rc = bx.EnsureScratch((size_t)units * 3);
  if (rc)
    return rc;
  k_mol_inter<<<units, RT, 0, bx.stream>>>(bx.dev, bx.d_ff, m, d_newpos,
                                           bx.d_scratch);
  k_reduce_partials<<<1, RT, 0, bx.stream>>>(bx.d_scratch, units, 3, d_out3, 1);
  return bx.CudaCheck(cudaGetLastError(), "molecule inter");
}

// ---------------------------------------------------------------------------
// SingleMoleculeInter: unit u = atom * 27 + neighbour cell of the atom's
// current cell; the molecule stays in the cell list and its own atoms are
// skipped (src/CalculateEnergy.cpp:1494-1556).  lam = old VDW, new VDW, old
// Coulomb, new Coulomb; partials = old LJ, old real, new LJ, new real.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(RT) k_single_mol_inter(
    DevBox b, const FF *__restrict__ pff, int m,
    const double *__restrict__ lam, double *part) {
  const FF &ff = *pff;
  int u = blockIdx.x;
  int a = u / NB27, n = u % NB27;
  int atom = b.mstart[m] + a;
  double px = b.x[atom], py = b.y[atom], pz = b.z[atom];
  int cell = position_to_cell_fast(b, px, py, pz);
  int c2 = b.nbr[cell * NB27 + n];
  int n2 = b.cell_count[c2];
  double qa = b.q[atom];
  int ka = b.kind[atom];
  double lov = lam[0], lnv = lam[1], loc = lam[2], lnc = lam[3];
  double ljo = 0.0, reo = 0.0, ljn = 0.0, ren = 0.0;
  for (int j = threadIdx.x; j < n2; j += RT) {
    size_t s = (size_t)c2 * b.cap + j;
    int mj = b.cell_meta[s];
    if (meta_mol(mj) == m)
      continue;
    double4_32a pj = b.cell_pos[s];
    double dx = min_image(px - pj.x, b.L[0], b.half[0]);
    double dy = min_image(py - pj.y, b.L[1], b.half[1]);
    double dz = min_image(pz - pj.z, b.L[2], b.half[2]);
    double distSq = dsq3(dx, dy, dz);
    if (!(ff.rcutSq > distSq))
      continue;
    int idx = ka + meta_kind(mj) * ff.n_kinds;
    if (ff.electrostatic) {
      double qq = qa * pj.w * QQ_FACT;
      if (qq != 0.0) {
        ren += coulomb_energy_lambda(ff, distSq, idx, qq, lnc);
        reo += coulomb_energy_lambda(ff, distSq, idx, qq, loc);
      }
    }
    ljn += lj_energy_lambda(ff, distSq, idx, lnv);
    ljo += lj_energy_lambda(ff, distSq, idx, lov);
  }
  __shared__ double red[RT / 32];
  double v[4] = {ljo, reo, ljn, ren};
  for (int c = 0; c < 4; ++c) {
    double r = block_sum<RT>(v[c], red);
    if (threadIdx.x == 0)
      part[4 * u + c] = r;
  }
}

int launch_single_mol_inter(Box &bx, int m, const double *d_lam4,
                            double *d_out4) {
  int na = bx.host.mstart[m + 1] - bx.host.mstart[m];
  int units = na * NB27;
  int rc = bx.EnsureScratch((size_t)units * 4);
  if (rc)
    return rc;
  k_single_mol_inter<<<units, RT, 0, bx.stream>>>(bx.dev, bx.d_ff, m, d_lam4,
                                                  bx.d_scratch);
  k_reduce_partials<<<1, RT, 0, bx.stream>>>(bx.d_scratch, units, 4, d_out4, 0);
  return bx.CudaCheck(cudaGetLastError(), "single molecule inter");
}

// ---------------------------------------------------------------------------
// ParticleInter: unit u = trial * 27 + neighbour, against every atom the
// cell grid holds (a molecule being grown by CBMC is taken out of the grid
// first, as in the reference).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(RT) k_particle_inter(DevBox b, const FF *__restrict__ pff,
                                                       int ka, double qa,
                                                       const double *__restrict__ trials,
                                                       double *part) {
  const FF &ff = *pff;
  int u = blockIdx.x;
  int t = u / NB27, n = u % NB27;
  double px = trials[3 * t], py = trials[3 * t + 1], pz = trials[3 * t + 2];
  int cell = position_to_cell_fast(b, px, py, pz);
  int c2 = b.nbr[cell * NB27 + n];
  int n2 = b.cell_count[c2];
  double lj = 0.0, re = 0.0, ovl = 0.0;
  for (int j = threadIdx.x; j < n2; j += RT) {
    size_t s = (size_t)c2 * b.cap + j;
    int mj = b.cell_meta[s];
    double4_32a pj = b.cell_pos[s];
    double dx = min_image(px - pj.x, b.L[0], b.half[0]);
    double dy = min_image(py - pj.y, b.L[1], b.half[1]);
    double dz = min_image(pz - pj.z, b.L[2], b.half[2]);
    double distSq = dsq3(dx, dy, dz);
    if (ff.rcutSq > distSq) {
      if (distSq < ff.rcutLowSq)
        ovl = 1.0;
      lj += lj_energy(ff, distSq, ka + meta_kind(mj) * ff.n_kinds);
      if (ff.electrostatic) {
        double qq = pj.w * qa * QQ_FACT;
        if (qq != 0.0)
          re += coulomb_energy(ff, distSq, qq);
      }
    }
  }
  __shared__ double red[RT / 32];
  double A = block_sum<RT>(lj, red);
  double R = block_sum<RT>(re, red);
  double O = block_sum<RT>(ovl, red);
  if (threadIdx.x == 0) {
    part[3 * u] = A;
    part[3 * u + 1] = R;
    part[3 * u + 2] = O > 0 ? 1.0 : 0.0;
  }
}

__global__ void k_reduce_trials(const double *__restrict__ part, int ntrials,
                                double *out) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntrials)
    return;
  double a = 0, r = 0, o = 0;
  for (int n = 0; n < NB27; ++n) {
    const double *p = part + 3 * ((size_t)t * NB27 + n);
    a += p[0];
    r += p[1];
    o = fmax(o, p[2]);
  }
  out[3 * t] = a;
  out[3 * t + 1] = r;
  out[3 * t + 2] = o;
}

int launch_particle_inter(Box &bx, int kind, double charge,
                          const double *d_trials, int ntrials, double *d_out) {
  int units = ntrials * NB27;
  int rc = bx.EnsureScratch((size_t)units * 3);
  if (rc)
    return rc;
  k_particle_inter<<<units, RT, 0, bx.stream>>>(bx.dev, bx.d_ff, kind, charge,
                                                d_trials, bx.d_scratch);
  k_reduce_trials<<<(ntrials + 127) / 128, 128, 0, bx.stream>>>(bx.d_scratch,
                                                               ntrials, d_out);
  return bx.CudaCheck(cudaGetLastError(), "particle inter");
}

// ---------------------------------------------------------------------------
// Ewald intramolecular correction, one thread per molecule
// ---------------------------------------------------------------------------
__global__ void k_correction(DevBox b, const FF *__restrict__ pff, double *part) {
  const FF &ff = *pff;
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  double corr = 0.0;
  if (m < b.n_mol) {
    int a0 = b.mstart[m], n = b.mstart[m + 1] - a0;
    for (int i = 0; i < n; i++) {
      if (fabs(b.q[a0 + i]) < 0.000000001)
        continue;
      for (int j = i + 1; j < n; j++) {
        int p = a0 + i, q = a0 + j;
        double dx = min_image(b.x[p] - b.x[q], b.L[0], b.half[0]);
        double dy = min_image(b.y[p] - b.y[q], b.L[1], b.half[1]);
        double dz = min_image(b.z[p] - b.z[q], b.L[2], b.half[2]);
        double distSq = dsq3(dx, dy, dz);
        double dist = sqrt(distSq);
        corr += (b.q[p] * b.q[q] * erf(ff.alpha * dist) / dist);
      }
    }
    corr = -1.0 * QQ_FACT * corr;
  }
  __shared__ double red[RT / 32];
  double s = block_sum<RT>(corr, red);
  if (threadIdx.x == 0)
    part[blockIdx.x] = s;
}

int launch_correction(Box &bx, double *d_out) {
  int nb = (bx.dev.n_mol + RT - 1) / RT;
  int rc = bx.EnsureScratch(nb);
  if (rc)
    return rc;
  k_correction<<<nb, RT, 0, bx.stream>>>(bx.dev, bx.d_ff, bx.d_scratch);
  k_reduce_partials<<<1, RT, 0, bx.stream>>>(bx.d_scratch, nb, 1, d_out, 0);
  return bx.CudaCheck(cudaGetLastError(), "correction");
}

// ---------------------------------------------------------------------------
// BoxForce: CTA (cell c, group g of 9 neighbour cells); thread = atom of c.
// Energies count each pair once (i < j); forces gather every pair.
// ---------------------------------------------------------------------------
constexpr int FG = 3;  // neighbour-shell groups
// Each thread owns one atom of cell c per pass and gathers the force on it
// from the CTA's third of the neighbour shell.  Per neighbour cell (staged in
// shared memory with FP32 copies of the positions) a thread first marks the
// neighbours that pass an FP32 distance pre-filter in a bit mask, then the
// warp walks the masks together: in each round every thread evaluates its
// next marked pair in FP64 (exact cutoff test, forces, and the energy of
// pairs with i < j).  The FP64 work then follows the pairs inside the
// cutoff, and each atom's sum runs over its pairs in neighbour order.
constexpr int FMW = 8;  // 64-bit mask words per neighbour-cell chunk (512)
__global__ void __launch_bounds__(RT) k_box_force(DevBox b, const FF *__restrict__ pff,
                                                  double *fpart, double *epart) {
  extern __shared__ __align__(32) unsigned char smem[];
  const FF &ff = *pff;
  int c = blockIdx.x, g = blockIdx.y;
  int n1 = b.cell_count[c];
  double4_32a *sp = (double4_32a *)smem;
  float4 *sf = (float4 *)(sp + b.cap);
  int *sm = (int *)(sf + b.cap);
  int *sa = sm + b.cap;
  const float Lf[3] = {(float)b.L[0], (float)b.L[1], (float)b.L[2]};
  const float Hf[3] = {(float)b.half[0], (float)b.half[1], (float)b.half[2]};
  // FP32 positions are within L 2^-24 of the FP64 ones; the pre-filter
  // radius covers twice that per axis plus 1e-4 of Rcut^2
  const double lmax = fmax(b.L[0], fmax(b.L[1], b.L[2]));
  const double rpad = ff.rcut + 1e-6 * lmax;
  const float cut_f = (float)(rpad * rpad * 1.0001);
  double lj = 0.0, re = 0.0;
  for (int base = 0; base < n1; base += RT) {
    int i = base + threadIdx.x;
    bool own = i < n1;
    double4_32a pi = make_double4_32a(0, 0, 0, 0);
    int mi = 0, ai = -1;
    if (own) {
      size_t si = (size_t)c * b.cap + i;
      pi = b.cell_pos[si];
      mi = b.cell_meta[si];
      ai = b.cell_atom[si];
    }
    const float pxf = (float)pi.x, pyf = (float)pi.y, pzf = (float)pi.z;
    const int moli = meta_mol(mi), ki = meta_kind(mi);
    double fx = 0, fy = 0, fz = 0;
    for (int nn = g * (NB27 / FG); nn < (g + 1) * (NB27 / FG); ++nn) {
      int c2 = b.nbr[c * NB27 + nn];
      int n2 = b.cell_count[c2];
      __syncthreads();
      for (int j = threadIdx.x; j < n2; j += RT) {
        size_t s2 = (size_t)c2 * b.cap + j;
        const double4_32a p = b.cell_pos[s2];
        sp[j] = p;
        sf[j] = make_float4((float)p.x, (float)p.y, (float)p.z, 0.0f);
        sm[j] = b.cell_meta[s2];
        sa[j] = b.cell_atom[s2];
      }
      __syncthreads();
      for (int jb = 0; jb < n2; jb += 64 * FMW) {
        // candidates of this thread's atom among neighbours jb .. jb + 511
        unsigned long long mk[FMW];
#pragma unroll
        for (int w = 0; w < FMW; ++w) {
          unsigned long long m = 0;
          const int j0 = jb + 64 * w;
          if (own)
            for (int k = 0; k < 64 && j0 + k < n2; ++k) {
              const int j = j0 + k;
              const float4 q = sf[j];
              float dx = pxf - q.x, dy = pyf - q.y, dz = pzf - q.z;
              dx = dx > Hf[0] ? dx - Lf[0] : dx < -Hf[0] ? dx + Lf[0] : dx;
              dy = dy > Hf[1] ? dy - Lf[1] : dy < -Hf[1] ? dy + Lf[1] : dy;
              dz = dz > Hf[2] ? dz - Lf[2] : dz < -Hf[2] ? dz + Lf[2] : dz;
              if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) < cut_f &&
                  moli != meta_mol(sm[j]))
                m |= 1ull << k;
            }
          mk[w] = m;
        }
        // rounds: every thread takes its next marked neighbour
        for (;;) {
          int j = -1;
#pragma unroll
          for (int w = 0; w < FMW; ++w)
            if (j < 0 && mk[w]) {
              const int k = __ffsll((long long)mk[w]) - 1;
              mk[w] &= mk[w] - 1;
              j = jb + 64 * w + k;
            }
          if (!__any_sync(0xffffffffu, j >= 0))
            break;
          if (j < 0)
            continue;
          const int mj = sm[j];
          const double4_32a pj = sp[j];
          double dx = min_image(pi.x - pj.x, b.L[0], b.half[0]);
          double dy = min_image(pi.y - pj.y, b.L[1], b.half[1]);
          double dz = min_image(pi.z - pj.z, b.L[2], b.half[2]);
          double distSq = dsq3(dx, dy, dz);
          if (ff.rcutSq > distSq) {
            int idx = ki + meta_kind(mj) * ff.n_kinds;
            double fR = 0.0;
            bool hasR = false;
            const bool first = ai < sa[j];
            if (ff.electrostatic) {
              double qq = pi.w * pj.w * QQ_FACT;
              if (qq != 0.0) {
                if (first)
                  re += coulomb_energy(ff, distSq, qq);
                fR = coulomb_virial(ff, distSq, qq);
                hasR = true;
              }
            }
            if (first)
              lj += lj_energy(ff, distSq, idx);
            double fL = lj_virial(ff, distSq, idx);
            fx += dx * fL + (hasR ? dx * fR : 0.0);
            fy += dy * fL + (hasR ? dy * fR : 0.0);
            fz += dz * fL + (hasR ? dz * fR : 0.0);
          }
        }
      }
    }
    if (own) {
      double *f = fpart + ((size_t)g * b.n_atoms + ai) * 3;
      f[0] = fx;
      f[1] = fy;
      f[2] = fz;
    }
  }
  __shared__ double red[RT / 32];
  double A = block_sum<RT>(lj, red);
  double R = block_sum<RT>(re, red);
  if (threadIdx.x == 0) {
    size_t t = (size_t)c * FG + g;
    epart[2 * t] = A;
    epart[2 * t + 1] = R;
  }
}

__global__ void k_force_gather(DevBox b, const double *__restrict__ fpart,
                               double *aF, double *mF) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= b.n_mol)
    return;
  double mx = 0, my = 0, mz = 0;
  for (int a = b.mstart[m]; a < b.mstart[m + 1]; ++a) {
    double f[3] = {0, 0, 0};
    for (int g = 0; g < FG; ++g)
      for (int d = 0; d < 3; ++d)
        f[d] += fpart[((size_t)g * b.n_atoms + a) * 3 + d];
    for (int d = 0; d < 3; ++d)
      aF[3 * (size_t)a + d] = f[d];
    mx += f[0];
    my += f[1];
    mz += f[2];
  }
  mF[3 * (size_t)m] = mx;
  mF[3 * (size_t)m + 1] = my;
  mF[3 * (size_t)m + 2] = mz;
}

int launch_box_force(Box &bx, const DevBox &b, double *aF, double *mF,
                     double *d_out2) {
  size_t need = (size_t)FG * b.n_atoms * 3 + (size_t)b.ncell * FG * 2;
  int rc = bx.EnsureScratch(need);
  if (rc)
    return rc;
  double *fpart = bx.d_scratch;
  double *epart = fpart + (size_t)FG * b.n_atoms * 3;
  size_t sh = (size_t)b.cap * (sizeof(double4_32a) + sizeof(float4) +
                                2 * sizeof(int));
  raise_smem_limit((const void *)k_box_force, sh);
  k_box_force<<<dim3(b.ncell, FG), RT, sh, bx.stream>>>(b, bx.d_ff, fpart, epart);
  k_force_gather<<<(b.n_mol + 127) / 128, 128, 0, bx.stream>>>(b, fpart, aF,
                                                              mF);
  k_reduce_partials<<<1, RT, 0, bx.stream>>>(epart, b.ncell * FG, 2, d_out2, 0);
  return bx.CudaCheck(cudaGetLastError(), "box force");
}

// ---------------------------------------------------------------------------
// CalculateTorque: molecule torque from atom forces (real + reciprocal)
// ---------------------------------------------------------------------------
__global__ void k_torque(DevBox b, const double *__restrict__ aF,
                         const double *__restrict__ aR, double *tq) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= b.n_mol)
    return;
  double tx = 0, ty = 0, tz = 0;
  for (int p = b.mstart[m]; p < b.mstart[m + 1]; ++p) {
    double d0 = min_image(b.x[p] - b.cx[m], b.L[0], b.half[0]);
    double d1 = min_image(b.y[p] - b.cy[m], b.L[1], b.half[1]);
    double d2 = min_image(b.z[p] - b.cz[m], b.L[2], b.half[2]);
    double f0 = aF[3 * (size_t)p] + aR[3 * (size_t)p];
    double f1 = aF[3 * (size_t)p + 1] + aR[3 * (size_t)p + 1];
    double f2 = aF[3 * (size_t)p + 2] + aR[3 * (size_t)p + 2];
    tx += d1 * f2 - d2 * f1;
    ty += d2 * f0 - d0 * f2;
    tz += d0 * f1 - d1 * f0;
  }
  tq[3 * (size_t)m] = tx;
  tq[3 * (size_t)m + 1] = ty;
  tq[3 * (size_t)m + 2] = tz;
}

int launch_torque(Box &bx, const DevBox &d, const double *aF,
                  const double *aR, double *tq) {
  k_torque<<<(d.n_mol + 127) / 128, 128, 0, bx.stream>>>(d, aF, aR, tq);
  return bx.CudaCheck(cudaGetLastError(), "torque");
}

}  // namespace gb
