// Internal definitions of the GB300 Monte Carlo energy engine.
//
// One gb_box holds one orthogonal periodic box resident in HBM: FP64 master
// coordinates, per-atom charge / kind / molecule, a padded cell grid in
// cell-ordered SoA form, the Ewald k-vector tables and structure factors, and
// the running box energies.  All kernels of the engine see it through the
// plain-pointer view DevBox.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

namespace gb {

constexpr double QQ_FACT = 167103.208067979;  // lib/NumLib.h:22
// sqrt(QQ_FACT): the mixed form stores charges scaled by it, so that the
// product of two scaled charges is q_i q_j QQ_FACT
constexpr double SQRT_QQ_FACT = 408.7825926675193;
constexpr int NB27 = 27;
constexpr int MAX_KINDS = 8;
constexpr int ETAB_DEG = 8;  // degree of the erfc(alpha r)/r segments
constexpr int MAX_MOL_ATOMS = 8;   // rigid molecules handled by the move loop
constexpr int END_CELL = -1;
constexpr int KRUN = 8;  // k-vectors per run of the structure-factor kernel

// Status codes of the C ABI (include/gomc_gb300.h).
enum Status : int {
  OK = 0,
  ERR_ARG = 1,
  ERR_CUDA = 2,
  ERR_NOMEM = 3,
  ERR_CAPACITY = 4,
  ERR_TIMEOUT = 5,
  ERR_STATE = 6,
  ERR_UNSUPPORTED = 7,
};

// Device error word bits (DevBox::err).
enum DevErr : int {
  DERR_CELL_OVERFLOW = 1,
  DERR_BARRIER_TIMEOUT = 2,
  DERR_BAD_INPUT = 4,
};

// Force-field constants, FlatIndex(i, j) = i + j * n_kinds
// (src/FFParticle.h:116) and Forcefield::InitBasicVals
// (src/Forcefield.cpp:37-83).
struct FF {
  int n_kinds;
  int ewald, electrostatic;
  double rcut, rcutSq, rcutLowSq, rcutCoulSq;
  double alpha, alphaSq, recip_rcut, recip_rcutSq, beta;
  double sigmaSq[MAX_KINDS * MAX_KINDS];
  double eps_cn[MAX_KINDS * MAX_KINDS];
  double nexp[MAX_KINDS * MAX_KINDS];
  double eps_cn_6[MAX_KINDS * MAX_KINDS];
  double nOver6[MAX_KINDS * MAX_KINDS];
  // erfc(alpha r) / r as piecewise degree-8 polynomials in r^2 (Ewald
  // only): 64 segments per binade of r^2 from 0.5 A^2, 9 coefficients each;
  // segment of r^2 = (its IEEE exponent and top 6 mantissa bits) - key0
  const double *erfc_tab;
  // (erfc(alpha r) / r + 2 alpha / sqrt(pi) exp(-alpha^2 r^2)) / r^2, the
  // Coulomb force factor of FFParticle::CalcCoulombVir, on the same segments
  const double *vir_tab;
  int etab_key0, etab_nseg;
  // soft-core settings at lambda < 1 (Forcefield::sc_*,
  // src/Forcefield.cpp:59-75)
  double sc_alpha, sc_sigma_6;
  int sc_power, sc_coul;
  // FP32 copies for the mixed form
  float sigmaSq_f[MAX_KINDS * MAX_KINDS];
  float eps_cn_f[MAX_KINDS * MAX_KINDS];
  // Rounding a constant to FP32 scales every pair of one kind by the same
  // factor, a bias that adds up over many moves.  The same holds for the
  // FP32 length of one fixed-point turn, L 2^-32 rounded to FP32: distances
  // from it are r_f = r / (1 + eta), eta = (L 2^-32) / fl(L 2^-32) - 1 (the
  // mean over the axes; exact for a cubic box).  With s = sigmaSq_f / r_f^2
  // the exact 12-6 energy is
  //   eps_cn_f * [(s^6 - s^3) + (k6 s^6 - k3 s^3)],
  //   k6 = (eps_cn / eps_cn_f) (sigmaSq / sigmaSq_f / (1 + eta)^2)^6 - 1,
  // k3 likewise with the third power.
  float lj_k6_f[MAX_KINDS * MAX_KINDS];
  float lj_k3_f[MAX_KINDS * MAX_KINDS];
  // Coulomb of a single position (and FP32 pair brackets): erfc(alpha r)/r =
  // (1 + coul_qfac) erfc(alpha_f r_f) / r_f to first order in eta, with
  // coul_qfac = 1 / (1 + eta) - 1 (alpha_lo_f = alpha - alpha_f is below
  // what those near-cutoff terms can show).  Pair differences use exact
  // distances and alpha as alpha_f + alpha_lo_f.
  float alpha_f, alpha_lo_f, coul_qfac_f;
  // pairs with both alpha r >= 2 (r^2 >= far_r2) take the FP32 bracket on
  // FP32 distances, with first-order corrections for the turn length (eta)
  // and alpha_f: coul_da = (alpha (1 + eta) - alpha_f) 2 / sqrt(pi)
  float far_r2_f, coul_da_f;
  // close pairs (both distances below sqrt(close_r2), alpha r < 1.3): exact squared
  // distances from the turn counts, turn2 = (L_d 2^-32)^2 as hi + lo,
  // alpha^2 and alpha^3 (hi + lo) for close_coulomb (gb_f32math.cuh)
  float turn2_hi[3], turn2_lo[3];
  float sigmaSq_lo_f[MAX_KINDS * MAX_KINDS];  // sigmaSq - sigmaSq_f
  float eps_cn_lo_f[MAX_KINDS * MAX_KINDS];   // eps_cn - eps_cn_f
  float alpha2_f, alpha3_hi, alpha3_lo, close_r2_f;
};

// Plain-pointer view of one box, passed by value to kernels.
struct DevBox {
  double L[3], half[3];
  double volume;
  int n_atoms, n_mol;
  // atoms, indexed by atom id
  double *x, *y, *z;
  double *cx, *cy, *cz;  // molecule centres (COM::CalcCOM)
  double *q;
  int *kind, *mol, *mstart;
  // cell grid: `cap` padded slots per cell, SoA by slot
  int edge[3];
  double cellSize[3];
  double invCell[3];  // 1 / cellSize
  double invL[3];     // 1 / L
  int ncell, cap;
  int *nbr;          // [ncell * 27], src/CellList.cpp:191-218 order
  int *cell_count;   // [ncell]
  int *cell_atom;    // [ncell * cap]
  double4_32a *cell_pos; // [ncell * cap] x, y, z, q
  int *cell_meta;    // [ncell * cap] (mol << 4) | kind
  uint4 *cell_fix;   // [ncell * cap] fixed-point turns x, y, z; and
                     // q * SQRT_QQ_FACT rounded to FP32, as float bits
  float *cell_qlo;   // [ncell * cap] q * SQRT_QQ_FACT minus that FP32 value
  int *atom_cell, *atom_slot;  // [n_atoms]
  // Ewald
  int K, kmax;
  double *kx, *ky, *kz, *prefact, *hsqr;  // [K]
  char4 *kn;                              // [K] integer k indices
  // runs of up to KRUN k-vectors with one (n_y, n_z) and consecutive n_x,
  // for the full structure factor: (n_y, n_z, first n_x, length) and the
  // k index of each member (-1 past the length)
  int nrun;
  int4 *krun;   // [nrun]
  int *krun_k;  // [nrun * KRUN]
  float *prefact_f;                       // [K]
  float4 *cis256;  // [256] exp(2 pi i j / 256) as float-float (re, im)
  double *sumRref, *sumIref, *sumRnew, *sumInew;  // [K]
  // running energies: inter, real, recip, self, correction
  double *energy;
  int *err;
};

// ---------------------------------------------------------------------------
// Host-side description of a box (owned by gb_box).
// ---------------------------------------------------------------------------
struct HostSystem {
  int n_atoms = 0, n_mol = 0, n_kinds = 0;
  std::vector<double> x, y, z, cx, cy, cz, q;
  std::vector<int> kind, mol, mstart;
  std::vector<double> eps, sigma, nexp;
  double L[3] = {0, 0, 0};
};

// ---------------------------------------------------------------------------
// Device math shared by the kernels
// ---------------------------------------------------------------------------
#ifdef __CUDACC__
#define GB_HD __host__ __device__ __forceinline__
#else
#define GB_HD inline
#endif

// BoxDimensions::MinImageSigned, src/BoxDimensions.h:169-175
GB_HD double min_image(double raw, double ax, double half) {
  if (raw > half)
    raw -= ax;
  else if (raw < -half)
    raw += ax;
  return raw;
}
// BoxDimensions::WrapPBC(double&, double), src/BoxDimensions.cpp:283-313
GB_HD double wrap1(double v, double ax) {
  if (v >= ax)
    v -= ax;
  else if (v < 0)
    v += ax;
  return v;
}
// BoxDimensions::UnwrapPBC(double&, ...), src/BoxDimensions.cpp:315-339
GB_HD double unwrap1(double v, double ref, double ax, double half) {
  if (fabs(ref - v) > half) {
    if (ref < half)
      v -= ax;
    else
      v += ax;
  }
  return v;
}

#ifdef __CUDACC__
// Products and sums without contraction so that FP64 distances round the way
// the reference's host build rounds them.
__device__ __forceinline__ double dsq3(double dx, double dy, double dz) {
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)),
                   __dmul_rn(dz, dz));
}
#endif

// CellList::PositionToCell, src/CellList.h:88-101
GB_HD int position_to_cell(const DevBox &b, double px, double py, double pz) {
  int x = (int)(px / b.cellSize[0]);
  int y = (int)(py / b.cellSize[1]);
  int z = (int)(pz / b.cellSize[2]);
  x -= (x == b.edge[0] ? 1 : 0);
  y -= (y == b.edge[1] ? 1 : 0);
  z -= (z == b.edge[2] ? 1 : 0);
  return x * b.edge[1] * b.edge[2] + y * b.edge[2] + z;
}

// The same cell index with one multiply per axis: trunc(x * (1/cellSize))
// equals trunc(x / cellSize) whenever the product is more than 1e-9 away
// from an integer (its error is a few ulp); otherwise the exact division
// decides.  Bit-identical membership at a fraction of the FP64 latency.
GB_HD int cell_axis(double x, double cs, double inv, int edge) {
  double y = x * inv;
  double t = trunc(y);
  double fr = y - t;
  int c = (fr > 1e-9 && fr < 1.0 - 1e-9) ? (int)t : (int)(x / cs);
  return c - (c == edge ? 1 : 0);
}
GB_HD int position_to_cell_fast(const DevBox &b, double px, double py,
                                double pz) {
  int x = cell_axis(px, b.cellSize[0], b.invCell[0], b.edge[0]);
  int y = cell_axis(py, b.cellSize[1], b.invCell[1], b.edge[1]);
  int z = cell_axis(pz, b.cellSize[2], b.invCell[2], b.edge[2]);
  return x * b.edge[1] * b.edge[2] + y * b.edge[2] + z;
}

// Fixed-point fraction of the box edge: round(v / L * 2^32) mod 2^32.
GB_HD uint32_t to_turns(double v, double invL) {
  double t = v * invL;
  t -= floor(t);
  double s = t * 4294967296.0;
  unsigned long long u = (unsigned long long)(s + 0.5);
  return (uint32_t)(u & 0xffffffffULL);
}

}  // namespace gb

// The opaque handle of the C ABI.
struct gb_box;
