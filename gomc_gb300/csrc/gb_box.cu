// Box set-up, resident state and the host side of the energy-path calls.
#include "gb_box.h"

#include <cmath>
#include <cstring>
#include <algorithm>
#include <map>
#include <mutex>

namespace gb {

void raise_smem_limit(const void *func, size_t bytes) {
  // The opt-in is needed whenever static plus dynamic shared memory passes
  // 48 KiB, so it is set for every size (once per device, kernel and size).
  static std::mutex mu;
  static std::map<std::pair<int, const void *>, size_t> limit;
  int dev = 0;
  cudaGetDevice(&dev);  // the attribute belongs to the current device
  std::lock_guard<std::mutex> g(mu);
  size_t &cur = limit[{dev, func}];
  if (bytes > cur) {
    // a refused size must not surface later as another call's error; the
    // launch that needs it reports the problem
    if (cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)bytes) == cudaSuccess)
      cur = bytes;
    else
      cudaGetLastError();
  }
}

// ---------------------------------------------------------------------------
// Force field: FFSetup::Particle::Read zeroing (src/FFSetup.cpp:246-255),
// FFParticle::Blend (src/FFParticle.cpp:200-242) and
// Forcefield::InitBasicVals (src/Forcefield.cpp:37-83).
// ---------------------------------------------------------------------------
void build_ff(const HostSystem &s, const BoxConfig &c, FF *ff) {
  std::memset(ff, 0, sizeof(FF));
  int nk = s.n_kinds;
  // FP32 turn length of the mixed form: fl(L 2^-32) = (L 2^-32) / (1 + eta)
  double eta = 0.0;
  for (int d = 0; d < 3; ++d) {
    double exact = s.L[d] * 2.3283064365386963e-10;
    eta += exact / (double)(float)exact - 1.0;
  }
  eta /= 3.0;
  const double len2 = (1.0 + eta) * (1.0 + eta);
  ff->n_kinds = nk;
  for (int i = 0; i < nk; ++i)
    for (int j = 0; j < nk; ++j) {
      int idx = i + j * nk;
      double ei = std::fabs(s.eps[i]) < 1.0e-20 ? 0.0 : s.eps[i];
      double ej = std::fabs(s.eps[j]) < 1.0e-20 ? 0.0 : s.eps[j];
      double ni = std::fabs(s.eps[i]) < 1.0e-20 ? 12.0 : s.nexp[i];
      double nj = std::fabs(s.eps[j]) < 1.0e-20 ? 12.0 : s.nexp[j];
      double n = (ni + nj) * 0.5;
      double cn = n / (n - 6.0) * std::pow(n / 6.0, (6.0 / (n - 6.0)));
      double sg = (s.sigma[i] + s.sigma[j]) * 0.5;
      ff->nexp[idx] = n;
      ff->sigmaSq[idx] = sg * sg;
      double e = std::sqrt(ei * ej);
      ff->eps_cn[idx] = cn * e;
      ff->eps_cn_6[idx] = ff->eps_cn[idx] * 6;
      ff->nOver6[idx] = n / 6;
      ff->sigmaSq_f[idx] = (float)ff->sigmaSq[idx];
      ff->eps_cn_f[idx] = (float)ff->eps_cn[idx];
      double rs = ff->sigmaSq_f[idx] != 0.0f
                      ? ff->sigmaSq[idx] / (double)ff->sigmaSq_f[idx] / len2
                      : 1.0;
      double re = ff->eps_cn_f[idx] != 0.0f
                      ? ff->eps_cn[idx] / (double)ff->eps_cn_f[idx] : 1.0;
      ff->sigmaSq_lo_f[idx] =
          (float)(ff->sigmaSq[idx] - (double)ff->sigmaSq_f[idx]);
      ff->eps_cn_lo_f[idx] = (float)(ff->eps_cn[idx] - (double)ff->eps_cn_f[idx]);
      ff->lj_k6_f[idx] = (float)(re * std::pow(rs, 6) - 1.0);
      ff->lj_k3_f[idx] = (float)(re * std::pow(rs, 3) - 1.0);
    }
  ff->rcut = c.rcut;
  ff->rcutSq = c.rcut * c.rcut;
  ff->rcutLowSq = c.rcut_low * c.rcut_low;
  ff->rcutCoulSq = c.rcut_coulomb * c.rcut_coulomb;
  ff->ewald = c.ewald;
  ff->electrostatic = c.electrostatic;
  if (c.ewald) {
    ff->alpha = std::sqrt(-std::log(c.tolerance)) / c.rcut_coulomb;
    ff->alphaSq = ff->alpha * ff->alpha;
    ff->alpha_f = (float)ff->alpha;
    ff->alpha_lo_f = (float)(ff->alpha - (double)ff->alpha_f);
    ff->coul_da_f =
        (float)((ff->alpha * (1.0 + eta) - (double)ff->alpha_f) * M_2_SQRTPI);
    ff->far_r2_f = (float)(4.0 / ff->alphaSq);
    ff->recip_rcut = -2.0 * std::log(c.tolerance) / c.rcut_coulomb;
    ff->recip_rcutSq = ff->recip_rcut * ff->recip_rcut;
  }
  ff->coul_qfac_f = (float)(1.0 / (1.0 + eta) - 1.0);
  for (int d = 0; d < 3; ++d) {
    double t = s.L[d] * 2.3283064365386963e-10;
    double t2 = t * t;
    ff->turn2_hi[d] = (float)t2;
    ff->turn2_lo[d] = (float)(t2 - (double)ff->turn2_hi[d]);
  }
  double a3 = ff->alpha * ff->alpha * ff->alpha;
  ff->alpha2_f = (float)ff->alphaSq;
  ff->alpha3_hi = (float)a3;
  ff->alpha3_lo = (float)(a3 - (double)ff->alpha3_hi);
  // the split 1/r - erf(a r)/r while alpha r < 1.3: beyond it erf(a r)/r
  // nearly equals 1/r, their difference (erfc) loses the digits the split
  // gains, and the erfc form on exact distances is the more accurate one;
  // r < 4 A without Ewald
  ff->close_r2_f = (float)(c.ewald ? 1.3 * 1.3 / ff->alphaSq : 16.0);
  ff->beta = 1 / c.temperature;
  ff->sc_alpha = c.sc_alpha;
  ff->sc_sigma_6 = std::pow(c.sc_sigma, 6.0);
  ff->sc_power = c.sc_power;
  ff->sc_coul = c.sc_coul;
}

// ---------------------------------------------------------------------------
// Table of erfc(alpha r) / r (with `force`: the force factor
// (erfc(alpha r) / r + 2 alpha / sqrt(pi) exp(-alpha^2 r^2)) / r^2) over r^2
// in [0.5, 2^e1) A^2, 2^e1 > s_max: per
// segment (64 per binade) the degree-8 Chebyshev interpolant at 9 first-kind
// Chebyshev nodes, computed in long double and stored as monomial
// coefficients in u = 2 (s - a) / h - 1.  Interpolation error below 1.1e-16
// relative on [0.5, 100] for alpha = 0.339 (degree 6 reached only 2e-14 in
// the widest segments, where exp(-alpha^2 r^2) bends most per segment).
// ---------------------------------------------------------------------------
static void erfc_table(double alpha, double s_max, std::vector<double> &tab,
                       int *key0, int *nseg, bool force = false) {
  constexpr int D = ETAB_DEG, NC = ETAB_DEG + 1;
  const int E0 = -1;
  int e1 = E0;
  while (std::ldexp(1.0, e1) <= s_max)
    ++e1;
  *nseg = (e1 - E0) * 64;
  *key0 = (1023 + E0) << 6;
  tab.assign((size_t)*nseg * NC, 0.0);
  const long double al = alpha;
  const long double pi = 3.14159265358979323846264338327950288L;
  long double node[NC], tk[NC][NC];  // nodes; T_k(node_i)
  for (int i = 0; i < NC; ++i) {
    node[i] = cosl(pi * (i + 0.5L) / NC);
    for (int k = 0; k < NC; ++k)
      tk[k][i] = cosl(pi * k * (i + 0.5L) / NC);
  }
  // power-basis coefficients of T_0..T_D
  long double mono[NC][NC] = {};
  mono[0][0] = 1.0L;
  mono[1][1] = 1.0L;
  for (int k = 1; k < D; ++k)
    for (int m = 0; m < NC; ++m)
      mono[k + 1][m] = (m > 0 ? 2.0L * mono[k][m - 1] : 0.0L) - mono[k - 1][m];
  for (int seg = 0; seg < *nseg; ++seg) {
    int bin = seg / 64, j = seg % 64;
    long double w = ldexpl(1.0L, E0 + bin);
    long double a = w * (1.0L + j / 64.0L), h = w / 64.0L;
    long double f[NC], c[NC];
    for (int i = 0; i < NC; ++i) {
      long double sv = a + h * (node[i] + 1.0L) * 0.5L;
      long double r = sqrtl(sv);
      f[i] = erfcl(al * r) / r;
      if (force)  // the force factor (src/FFParticle.cpp:401-446)
        f[i] = (f[i] + al * 2.0L / sqrtl(pi) * expl(-al * al * sv)) / sv;
    }
    for (int k = 0; k < NC; ++k) {
      long double acc = 0.0L;
      for (int i = 0; i < NC; ++i)
        acc += f[i] * tk[k][i];
      c[k] = acc * (2.0L / NC) * (k == 0 ? 0.5L : 1.0L);
    }
    for (int m = 0; m < NC; ++m) {
      long double p = 0.0L;
      for (int k = 0; k < NC; ++k)
        p += c[k] * mono[k][m];
      tab[(size_t)seg * NC + m] = (double)p;
    }
  }
}

// ---------------------------------------------------------------------------
// k-vectors of an orthogonal box, in the reference's order: x outer (x >= 0),
// y, z inner, |k|^2 < k_c^2 (Ewald::RecipInitOrth, src/Ewald.cpp:847-903).
// ---------------------------------------------------------------------------
void recip_vectors(const double L[3], double volume, double alphaSq,
                   double recip_rcutSq, double recip_rcut,
                   std::vector<double> &kx, std::vector<double> &ky,
                   std::vector<double> &kz, std::vector<double> &hsqr,
                   std::vector<double> &prefact, std::vector<char4> &kn,
                   int *kmax) {
  double alpsqr4 = 1.0 / (4.0 * alphaSq);
  double cv[3];
  for (int d = 0; d < 3; ++d) {
    cv[d] = 1.0 / L[d];
    cv[d] *= 2.0 * M_PI;
  }
  double vol = volume / (4.0 * M_PI);
  int nkx = (int)(recip_rcut * L[0] / (2.0 * M_PI)) + 1;
  int nky = (int)(recip_rcut * L[1] / (2.0 * M_PI)) + 1;
  int nkz = (int)(recip_rcut * L[2] / (2.0 * M_PI)) + 1;
  *kmax = std::max(std::max(nkx, nky), std::max(nky, nkz));
  kx.clear(); ky.clear(); kz.clear(); hsqr.clear(); prefact.clear(); kn.clear();
  for (int x = 0; x <= nkx; x++) {
    int nky_min = (x == 0) ? 0 : -nky;
    for (int y = nky_min; y <= nky; y++) {
      int nkz_min = (x == 0 && y == 0) ? 1 : -nkz;
      for (int z = nkz_min; z <= nkz; z++) {
        double kX = cv[0] * x;
        double kY = cv[1] * y;
        double kZ = cv[2] * z;
        double ksqr = kX * kX + kY * kY + kZ * kZ;
        if (ksqr < recip_rcutSq) {
          kx.push_back(kX);
          ky.push_back(kY);
          kz.push_back(kZ);
          hsqr.push_back(ksqr);
          prefact.push_back(QQ_FACT * std::exp(-ksqr * alpsqr4) /
                            (ksqr * vol));
          kn.push_back(make_char4((signed char)x, (signed char)y,
                                  (signed char)z, 0));
        }
      }
    }
  }
}

// COM::CalcCOM (src/COM.h:47-68), including its unwrap / re-wrap of the
// atom coordinates: each molecule is unwrapped against its first atom,
// averaged, and its atoms and centre wrapped back into the box.
static void calc_com(HostSystem &s) {
  const int M = s.n_mol;
  double half[3] = {s.L[0] * 0.5, s.L[1] * 0.5, s.L[2] * 0.5};
  s.cx.assign(M, 0);
  s.cy.assign(M, 0);
  s.cz.assign(M, 0);
  for (int m = 0; m < M; ++m) {
    int a0 = s.mstart[m], a1 = s.mstart[m + 1];
    double rx = s.x[a0], ry = s.y[a0], rz = s.z[a0];
    for (int p = a0; p < a1; ++p) {
      s.x[p] = unwrap1(s.x[p], rx, s.L[0], half[0]);
      s.y[p] = unwrap1(s.y[p], ry, s.L[1], half[1]);
      s.z[p] = unwrap1(s.z[p], rz, s.L[2], half[2]);
    }
    double cx = 0, cy = 0, cz = 0;
    for (int p = a0; p < a1; ++p) {
      cx += s.x[p];
      cy += s.y[p];
      cz += s.z[p];
    }
    for (int p = a0; p < a1; ++p) {
      s.x[p] = wrap1(s.x[p], s.L[0]);
      s.y[p] = wrap1(s.y[p], s.L[1]);
      s.z[p] = wrap1(s.z[p], s.L[2]);
    }
    double inv = 1.0 / (double)(a1 - a0);
    cx *= inv;
    cy *= inv;
    cz *= inv;
    s.cx[m] = wrap1(cx, s.L[0]);
    s.cy[m] = wrap1(cy, s.L[1]);
    s.cz[m] = wrap1(cz, s.L[2]);
  }
}

// ---------------------------------------------------------------------------
Box::~Box() { FreeAll(); }

int Box::Fail(int code, const std::string &msg) {
  last_error = msg;
  return code;
}

int Box::CudaCheck(cudaError_t e, const char *what) {
  if (e == cudaSuccess)
    return OK;
  last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? ERR_NOMEM : ERR_CUDA;
}

template <class T>
int Box::Alloc(T **p, size_t n) {
  void *q = nullptr;
  cudaError_t e = cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T));
  if (e != cudaSuccess)
    return CudaCheck(e, "cudaMalloc");
  allocs_.push_back(q);
  dev_bytes += std::max<size_t>(n, 1) * sizeof(T);
  *p = (T *)q;
  return OK;
}

void Box::FreeAll() {
  if (stream)
    cudaStreamSynchronize(stream);
  for (void *p : allocs_)
    cudaFree(p);
  allocs_.clear();
  for (void *p : trial.allocs)
    cudaFree(p);
  trial.allocs.clear();
  if (h_pinned)
    cudaFreeHost(h_pinned);
  h_pinned = nullptr;
  if (own_stream && stream)
    cudaStreamDestroy(stream);
  stream = nullptr;
}


// (Re)allocate *p to hold `bytes`, dropping its old contents; the pointer is
// owned by `allocs`.
static int regrow(Box &b, void **p, size_t bytes, std::vector<void *> &allocs) {
  if (*p) {
    cudaFree(*p);
    allocs.erase(std::remove(allocs.begin(), allocs.end(), *p), allocs.end());
    *p = nullptr;
  }
  void *q = nullptr;
  cudaError_t e = cudaMalloc(&q, std::max<size_t>(bytes, 1));
  if (e != cudaSuccess)
    return b.CudaCheck(e, "cudaMalloc");
  allocs.push_back(q);
  b.dev_bytes += bytes;
  *p = q;
  return OK;
}

// CellList::ResizeGrid / RebuildNeighbors (src/CellList.cpp:138-218) for
// edges L: cells per axis max(floor(L / Rcut), 3), the 27-neighbour table in
// the reference's order, and the slot capacity (three times the fullest cell
// of the given coordinates, at least 32, a multiple of 32).  The cell arrays
// grow when the grid needs more slots than they hold.
int Box::GridGeometry(const double L[3], const double *x, const double *y,
                      const double *z, DevBox &d, size_t *cell_cap,
                      size_t *nbr_cap, std::vector<void *> &allocs) {
  for (int k = 0; k < 3; ++k) {
    d.L[k] = L[k];
    d.half[k] = L[k] * 0.5;
    d.edge[k] = std::max((int)std::floor(L[k] / cfg.rcut), 3);
    d.cellSize[k] = L[k] / d.edge[k];
    d.invCell[k] = 1.0 / d.cellSize[k];
    d.invL[k] = 1.0 / L[k];
  }
  d.volume = L[0] * L[1] * L[2];
  d.ncell = d.edge[0] * d.edge[1] * d.edge[2];
  std::vector<int> nbr((size_t)d.ncell * NB27);
  {
    int *e = d.edge;
    for (int x = 0; x < e[0]; ++x)
      for (int y = 0; y < e[1]; ++y)
        for (int z = 0; z < e[2]; ++z) {
          int cell = x * e[2] * e[1] + y * e[2] + z;
          int n = 0;
          for (int dx = -1; dx <= 1; ++dx)
            for (int dy = -1; dy <= 1; ++dy)
              for (int dz = -1; dz <= 1; ++dz)
                nbr[(size_t)cell * NB27 + n++] =
                    ((x + dx + e[0]) % e[0]) * e[2] * e[1] +
                    ((y + dy + e[1]) % e[1]) * e[2] + ((z + dz + e[2]) % e[2]);
        }
  }
  {
    std::vector<int> cnt(d.ncell, 0);
    int mx = 0;
    for (int i = 0; i < d.n_atoms; ++i) {
      int cc = position_to_cell(d, x[i], y[i], z[i]);
      if (cc < 0 || cc >= d.ncell)
        return Fail(ERR_ARG, "coordinates must lie inside the box");
      mx = std::max(mx, ++cnt[cc]);
    }
    int cap = std::max(3 * mx, 32);
    d.cap = (cap + 31) / 32 * 32;
  }
  int rc;
  size_t NC = (size_t)d.ncell * d.cap;
  if (NC > *cell_cap) {
    if ((rc = regrow(*this, (void **)&d.cell_atom, NC * 4, allocs)) ||
        (rc = regrow(*this, (void **)&d.cell_pos, NC * sizeof(double4_32a),
                     allocs)) ||
        (rc = regrow(*this, (void **)&d.cell_meta, NC * 4, allocs)) ||
        (rc = regrow(*this, (void **)&d.cell_fix, NC * sizeof(uint4),
                     allocs)) ||
        (rc = regrow(*this, (void **)&d.cell_qlo, NC * 4, allocs)))
      return rc;
    *cell_cap = NC;
  }
  if ((size_t)d.ncell * NB27 > *nbr_cap) {
    if ((rc = regrow(*this, (void **)&d.nbr, nbr.size() * 4, allocs)) ||
        (rc = regrow(*this, (void **)&d.cell_count, (size_t)d.ncell * 4,
                     allocs)))
      return rc;
    *nbr_cap = (size_t)d.ncell * NB27;
  }
  return CudaCheck(cudaMemcpyAsync(d.nbr, nbr.data(), nbr.size() * 4,
                                   cudaMemcpyHostToDevice, stream),
                   "upload");
}

// Ewald::RecipInit (src/Ewald.cpp:835-903) for edges L into `ks`: the
// k-vectors with their prefactors, the integer indices, and runs of up to
// KRUN consecutive n_x per (n_y, n_z) column for the structure-factor
// kernels (longest runs first).
int Box::BuildKSet(const double L[3], KSet &ks) {
  std::vector<double> kx, ky, kz, hs, pf;
  std::vector<char4> kn;
  int kmax = 0;
  recip_vectors(L, L[0] * L[1] * L[2], ff.alphaSq, ff.recip_rcutSq,
                ff.recip_rcut, kx, ky, kz, hs, pf, kn, &kmax);
  if (kmax > 127)
    return Fail(ERR_UNSUPPORTED, "k-vector index above 127");
  const int K = (int)kx.size();
  std::vector<float> pff(pf.begin(), pf.end());
  std::map<std::pair<int, int>, std::vector<std::pair<int, int>>> cols;
  for (int k = 0; k < K; ++k)
    cols[{kn[k].y, kn[k].z}].push_back({kn[k].x, k});
  std::vector<int4> runs;
  std::vector<int> run_k;
  for (auto &c : cols) {
    auto &v = c.second;  // n_x ascending (k vectors are listed x outer)
    size_t i = 0;
    while (i < v.size()) {
      size_t j = i + 1;
      while (j < v.size() && j - i < (size_t)KRUN &&
             v[j].first == v[j - 1].first + 1)
        ++j;
      runs.push_back(make_int4(c.first.first, c.first.second, v[i].first,
                               (int)(j - i)));
      for (int g = 0; g < KRUN; ++g)
        run_k.push_back(i + g < j ? v[i + g].second : -1);
      i = j;
    }
  }
  // longest runs first: neighbouring threads then take runs of equal
  // length, and a warp skips the members none of its runs has (each run's
  // sums do not depend on which thread takes it)
  {
    std::vector<int> order(runs.size());
    for (size_t r = 0; r < runs.size(); ++r)
      order[r] = (int)r;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
      return runs[x].w > runs[y].w;
    });
    std::vector<int4> r2(runs.size());
    std::vector<int> k2(run_k.size());
    for (size_t r = 0; r < runs.size(); ++r) {
      r2[r] = runs[order[r]];
      for (int g = 0; g < KRUN; ++g)
        k2[r * KRUN + g] = run_k[(size_t)order[r] * KRUN + g];
    }
    runs.swap(r2);
    run_k.swap(k2);
  }
  int rc;
  if ((size_t)K > ks.cap) {
    if ((rc = regrow(*this, (void **)&ks.kx, (size_t)K * 8, allocs_)) ||
        (rc = regrow(*this, (void **)&ks.ky, (size_t)K * 8, allocs_)) ||
        (rc = regrow(*this, (void **)&ks.kz, (size_t)K * 8, allocs_)) ||
        (rc = regrow(*this, (void **)&ks.prefact, (size_t)K * 8, allocs_)) ||
        (rc = regrow(*this, (void **)&ks.hsqr, (size_t)K * 8, allocs_)) ||
        (rc = regrow(*this, (void **)&ks.kn, (size_t)K * 4, allocs_)) ||
        (rc = regrow(*this, (void **)&ks.prefact_f, (size_t)K * 4, allocs_)))
      return rc;
    ks.cap = K;
  }
  if (runs.size() > ks.run_cap) {
    if ((rc = regrow(*this, (void **)&ks.krun, runs.size() * sizeof(int4),
                     allocs_)) ||
        (rc = regrow(*this, (void **)&ks.krun_k, run_k.size() * sizeof(int),
                     allocs_)))
      return rc;
    ks.run_cap = runs.size();
  }
  auto up = [&](void *dst, const void *src, size_t bytes) {
    return CudaCheck(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice,
                                     stream),
                     "upload");
  };
  if ((rc = up(ks.kx, kx.data(), (size_t)K * 8)) ||
      (rc = up(ks.ky, ky.data(), (size_t)K * 8)) ||
      (rc = up(ks.kz, kz.data(), (size_t)K * 8)) ||
      (rc = up(ks.prefact, pf.data(), (size_t)K * 8)) ||
      (rc = up(ks.hsqr, hs.data(), (size_t)K * 8)) ||
      (rc = up(ks.kn, kn.data(), (size_t)K * 4)) ||
      (rc = up(ks.krun, runs.data(), runs.size() * sizeof(int4))) ||
      (rc = up(ks.krun_k, run_k.data(), run_k.size() * sizeof(int))) ||
      (rc = up(ks.prefact_f, pff.data(), (size_t)K * 4)))
    return rc;
  // the host vectors go out of scope: wait for the copies
  if ((rc = Sync()))
    return rc;
  ks.K = K;
  ks.kmax = kmax;
  ks.nrun = (int)runs.size();
  for (int d = 0; d < 3; ++d)
    ks.L[d] = L[d];
  return OK;
}

// The four structure-factor arrays hold at least K entries; growing them
// keeps the Ref sums (their first entries).
int Box::EnsureSums(size_t K) {
  if (K <= sums_cap)
    return OK;
  double **arr[4] = {&dev.sumRref, &dev.sumIref, &dev.sumRnew, &dev.sumInew};
  for (int i = 0; i < 4; ++i) {
    double *old = *arr[i];
    double *q = nullptr;
    int rc = Alloc(&q, K);
    if (rc)
      return rc;
    if (old && sums_cap) {
      if ((rc = CudaCheck(cudaMemcpyAsync(q, old, sums_cap * 8,
                                          cudaMemcpyDeviceToDevice, stream),
                          "copy")) ||
          (rc = Sync()))
        return rc;
      cudaFree(old);
      allocs_.erase(std::remove(allocs_.begin(), allocs_.end(), (void *)old),
                    allocs_.end());
    }
    *arr[i] = q;
  }
  sums_cap = K;
  return OK;
}

void Box::MirrorKRef() {
  dev.K = kref.K;
  dev.kmax = kref.kmax;
  dev.nrun = kref.nrun;
  dev.kx = kref.kx;
  dev.ky = kref.ky;
  dev.kz = kref.kz;
  dev.prefact = kref.prefact;
  dev.hsqr = kref.hsqr;
  dev.kn = kref.kn;
  dev.prefact_f = kref.prefact_f;
  dev.krun = kref.krun;
  dev.krun_k = kref.krun_k;
}

int Box::EnsureScratch(size_t n) {
  if (n <= scratch_len)
    return OK;
  int rc = Alloc(&d_scratch, n);
  if (rc)
    return rc;
  scratch_len = n;
  return OK;
}

int Box::Sync() {
  return CudaCheck(cudaStreamSynchronize(stream), "stream synchronize");
}

int Box::Create(const HostSystem &sys, const BoxConfig &cfg, Box **out,
                std::string *err) {
  Box *b = new Box();
  int rc = b->Init(sys, cfg);
  if (rc) {
    if (err)
      *err = b->last_error;
    delete b;
    return rc;
  }
  *out = b;
  return OK;
}

int Box::Init(const HostSystem &s0, const BoxConfig &c) {
  cfg = c;
  if (s0.n_atoms <= 0 || s0.n_mol <= 0 || s0.n_kinds <= 0 ||
      s0.n_kinds > MAX_KINDS)
    return Fail(ERR_ARG, "atom, molecule or kind count out of range");
  for (int d = 0; d < 3; ++d)
    if (!(s0.L[d] > 0))
      return Fail(ERR_ARG, "box edge must be positive");
  if (!(c.rcut > 0) || !(c.temperature > 0))
    return Fail(ERR_ARG, "Rcut and Temperature must be positive");
  if (c.ewald && !(c.tolerance > 0 && c.tolerance < 1))
    return Fail(ERR_ARG, "Ewald tolerance must be in (0, 1)");
  if ((int)s0.mstart.size() != s0.n_mol + 1 || s0.mstart[0] != 0 ||
      s0.mstart[s0.n_mol] != s0.n_atoms)
    return Fail(ERR_ARG, "molecule start offsets are inconsistent");
  for (int m = 0; m < s0.n_mol; ++m)
    if (s0.mstart[m + 1] <= s0.mstart[m])
      return Fail(ERR_ARG, "empty molecule");
  for (int i = 0; i < s0.n_atoms; ++i)
    if (s0.kind[i] < 0 || s0.kind[i] >= s0.n_kinds)
      return Fail(ERR_ARG, "atom kind out of range");

  int rc = CudaCheck(cudaSetDevice(c.device), "cudaSetDevice");
  if (rc)
    return rc;
  cudaDeviceProp prop;
  rc = CudaCheck(cudaGetDeviceProperties(&prop, c.device), "device props");
  if (rc)
    return rc;
  sm_count = prop.multiProcessorCount;
  rc = CudaCheck(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking),
                 "stream");
  if (rc)
    return rc;
  own_stream = true;

  host = s0;
  HostSystem &s = host;
  int N = s.n_atoms, M = s.n_mol;
  s.mol.assign(N, 0);
  for (int m = 0; m < M; ++m)
    for (int a = s.mstart[m]; a < s.mstart[m + 1]; ++a)
      s.mol[a] = m;
  // Coordinates::WrapCoordinate (src/Coordinates.cpp:24-73)
  for (int i = 0; i < N; ++i) {
    s.x[i] = wrap1(s.x[i], s.L[0]);
    s.y[i] = wrap1(s.y[i], s.L[1]);
    s.z[i] = wrap1(s.z[i], s.L[2]);
    if (!(s.x[i] >= 0 && s.x[i] <= s.L[0] && s.y[i] >= 0 && s.y[i] <= s.L[1] &&
          s.z[i] >= 0 && s.z[i] <= s.L[2]))
      return Fail(ERR_ARG, "an atom lies outside the box after wrapping");
  }
  double half[3] = {s.L[0] * 0.5, s.L[1] * 0.5, s.L[2] * 0.5};
  calc_com(s);
  build_ff(s, c, &ff);
  DevBox &d = dev;
  for (int k = 0; k < 3; ++k) {
    d.L[k] = s.L[k];
    d.half[k] = half[k];
  }
  d.volume = s.L[0] * s.L[1] * s.L[2];
  d.n_atoms = N;
  d.n_mol = M;

  // device allocations; the cell grid (CellList::ResizeGrid /
  // RebuildNeighbors, src/CellList.cpp:138-218) and its arrays
  if ((rc = Alloc(&d.x, N)) || (rc = Alloc(&d.y, N)) || (rc = Alloc(&d.z, N)) ||
      (rc = Alloc(&d.cx, M)) || (rc = Alloc(&d.cy, M)) ||
      (rc = Alloc(&d.cz, M)) || (rc = Alloc(&d.q, N)) ||
      (rc = Alloc(&d.kind, N)) || (rc = Alloc(&d.mol, N)) ||
      (rc = Alloc(&d.mstart, M + 1)) ||
      (rc = Alloc(&d.atom_cell, N)) ||
      (rc = Alloc(&d.atom_slot, N)) || (rc = Alloc(&d.energy, 8)) ||
      (rc = Alloc(&d.err, 4)) || (rc = Alloc(&d_ff, 1)) ||
      (rc = Alloc(&d_small, 4096)) || (rc = Alloc(&d_aF, 3 * (size_t)N)) ||
      (rc = Alloc(&d_mF, 3 * (size_t)M)) || (rc = Alloc(&d_aR, 3 * (size_t)N)) ||
      (rc = Alloc(&d_mR, 3 * (size_t)M)) || (rc = Alloc(&d_tq, 3 * (size_t)M)))
    return rc;
  if ((rc = GridGeometry(s.L, s.x.data(), s.y.data(), s.z.data(), d,
                         &grid_cell_cap_, &grid_nbr_cap_, allocs_)))
    return rc;
  rc = CudaCheck(cudaMallocHost(&h_pinned, 4096 * sizeof(double)), "pinned");
  if (rc)
    return rc;

  auto up = [&](void *dst, const void *src, size_t bytes) {
    return CudaCheck(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice,
                                     stream),
                     "upload");
  };
  if ((rc = up(d.x, s.x.data(), N * 8)) || (rc = up(d.y, s.y.data(), N * 8)) ||
      (rc = up(d.z, s.z.data(), N * 8)) ||
      (rc = up(d.cx, s.cx.data(), M * 8)) ||
      (rc = up(d.cy, s.cy.data(), M * 8)) ||
      (rc = up(d.cz, s.cz.data(), M * 8)) ||
      (rc = up(d.q, s.q.data(), N * 8)) ||
      (rc = up(d.kind, s.kind.data(), N * 4)) ||
      (rc = up(d.mol, s.mol.data(), N * 4)) ||
      (rc = up(d.mstart, s.mstart.data(), (M + 1) * 4)))
    return rc;
  ff.erfc_tab = nullptr;
  ff.vir_tab = nullptr;
  ff.etab_key0 = ff.etab_nseg = 0;
  if (c.ewald) {
    std::vector<double> et, vt;
    double *d_et = nullptr, *d_vt = nullptr;
    erfc_table(ff.alpha, ff.rcutCoulSq, et, &ff.etab_key0, &ff.etab_nseg);
    erfc_table(ff.alpha, ff.rcutCoulSq, vt, &ff.etab_key0, &ff.etab_nseg,
               true);
    if ((rc = Alloc(&d_et, et.size())) ||
        (rc = up(d_et, et.data(), et.size() * sizeof(double))) ||
        (rc = Alloc(&d_vt, vt.size())) ||
        (rc = up(d_vt, vt.data(), vt.size() * sizeof(double))))
      return rc;
    ff.erfc_tab = d_et;
    ff.vir_tab = d_vt;
  }
  if ((rc = up(d_ff, &ff, sizeof(FF))))
    return rc;
  if ((rc = CudaCheck(cudaMemsetAsync(d.err, 0, 16, stream), "memset")) ||
      (rc = CudaCheck(cudaMemsetAsync(d.energy, 0, 64, stream), "memset")))
    return rc;

  // Ewald tables: the k-vector set of the box edges and its structure
  // factors; exp(2 pi i j / 256) (float-float) for the mixed form's phases
  if (c.ewald) {
    if ((rc = BuildKSet(s.L, kref)) || (rc = EnsureSums(kref.K)))
      return rc;
    MirrorKRef();
    if ((rc = Alloc(&d.cis256, 256)))
      return rc;
    // exp(2 pi i j / 256) from the first octant by symmetry, each value
    // split into FP32 hi + lo
    std::vector<float4> cis(256);
    for (int j = 0; j < 256; ++j) {
      int o = j & 63;  // angle within its quarter turn, in 1/256 turns
      bool flip = o > 32;
      long double a = (flip ? 64 - o : o) * (3.14159265358979323846264338327950L / 128.0L);
      double c = (double)cosl(a), sn = (double)sinl(a);
      if (flip)
        std::swap(c, sn);
      double re, im;
      switch (j >> 6) {
        case 0: re = c; im = sn; break;
        case 1: re = -sn; im = c; break;
        case 2: re = -c; im = -sn; break;
        default: re = sn; im = -c; break;
      }
      float rh = (float)re, ih = (float)im;
      cis[j] = make_float4(rh, (float)(re - (double)rh), ih,
                           (float)(im - (double)ih));
    }
    if ((rc = up(d.cis256, cis.data(), 256 * sizeof(float4))))
      return rc;
  }
  if ((rc = GridAll()))
    return rc;
  // initial energies (System::Init -> SystemTotal)
  double tot[9];
  if ((rc = SystemTotal(tot)))
    return rc;
  return OK;
}

int Box::CheckError() {
  int herr[4] = {0, 0, 0, 0};
  int rc = CudaCheck(cudaMemcpyAsync(herr, dev.err, 16, cudaMemcpyDeviceToHost,
                                     stream),
                     "error read");
  if (rc)
    return rc;
  if ((rc = Sync()))
    return rc;
  if (herr[0] & DERR_CELL_OVERFLOW)
    return Fail(ERR_CAPACITY, "a cell exceeded its slot capacity");
  if (herr[0] & DERR_BARRIER_TIMEOUT)
    return Fail(ERR_TIMEOUT, "a device-side wait ran out of iterations");
  if (herr[0] & DERR_BAD_INPUT)
    return Fail(ERR_ARG, "invalid input detected on the device");
  return OK;
}

int Box::GridAll() {
  int rc = launch_grid_all(*this, dev);
  if (rc)
    return rc;
  cell_out.assign(dev.n_mol, 0);
  n_cell_out = 0;
  return OK;
}

int Box::CellRemoveMol(int m) {
  if (m < 0 || m >= dev.n_mol)
    return Fail(ERR_ARG, "molecule index out of range");
  if (cell_out[m])
    return Fail(ERR_STATE, "molecule is not in the cell list");
  int rc = launch_cell_remove_mol(*this, m);
  if (rc)
    return rc;
  cell_out[m] = 1;
  ++n_cell_out;
  return OK;
}

int Box::CellAddMol(int m) {
  if (m < 0 || m >= dev.n_mol)
    return Fail(ERR_ARG, "molecule index out of range");
  if (!cell_out[m])
    return Fail(ERR_STATE, "molecule is already in the cell list");
  int rc = launch_cell_add_mol(*this, m);
  if (rc || (rc = CheckError()))
    return rc;
  cell_out[m] = 0;
  --n_cell_out;
  return OK;
}

int Box::BoxInter(double *inter, double *real) {
  int rc = launch_box_inter(*this, d_small);
  if (rc)
    return rc;
  rc = CudaCheck(cudaMemcpyAsync(h_pinned, d_small, 16, cudaMemcpyDeviceToHost,
                                 stream),
                 "download");
  if (rc || (rc = Sync()))
    return rc;
  *inter = h_pinned[0];
  *real = h_pinned[1];
  return CheckError();
}

int Box::RecipSums(const double *x, const double *y, const double *z) {
  if (!cfg.ewald)
    return OK;
  if (cfg.precision == 1)  // mixed form: float-float structure factor
    return launch_recip_sums_ff(*this, x, y, z, dev.sumRnew, dev.sumInew);
  return launch_recip_sums(*this, x, y, z, dev.sumRnew, dev.sumInew);
}

int Box::RecipSetup() {
  if (!cfg.ewald)
    return OK;
  int rc = RecipSums(dev.x, dev.y, dev.z);
  if (rc)
    return rc;
  // SetRecipRef: Ref <- New
  size_t bytes = (size_t)dev.K * 8;
  if ((rc = CudaCheck(cudaMemcpyAsync(dev.sumRref, dev.sumRnew, bytes,
                                      cudaMemcpyDeviceToDevice, stream),
                      "copy")) ||
      (rc = CudaCheck(cudaMemcpyAsync(dev.sumIref, dev.sumInew, bytes,
                                      cudaMemcpyDeviceToDevice, stream),
                      "copy")))
    return rc;
  return OK;
}

int Box::RecipEnergy(double *e, bool ref_sums) {
  if (!cfg.ewald) {
    *e = 0;
    return OK;
  }
  int rc = launch_recip_energy(*this, ref_sums ? dev.sumRref : dev.sumRnew,
                               ref_sums ? dev.sumIref : dev.sumInew, d_small);
  if (rc)
    return rc;
  if ((rc = CudaCheck(cudaMemcpyAsync(h_pinned, d_small, 8,
                                      cudaMemcpyDeviceToHost, stream),
                      "download")) ||
      (rc = Sync()))
    return rc;
  *e = h_pinned[0];
  return OK;
}

int Box::BoxSelf(double *e) {
  // Ewald::BoxSelf (src/Ewald.cpp:1125-1163): per molecule kind, the sum of
  // squared charges of one molecule times the molecule count.  Molecules are
  // grouped by identical (kind, charge) lists in first-seen order.
  if (!cfg.ewald) {
    *e = 0;
    return OK;
  }
  const HostSystem &s = host;
  std::vector<int> seen(s.n_mol, 0);
  double self = 0.0;
  for (int m = 0; m < s.n_mol; ++m) {
    if (seen[m])
      continue;
    int len = s.mstart[m + 1] - s.mstart[m];
    long count = 0;
    for (int m2 = m; m2 < s.n_mol; ++m2) {
      if (seen[m2] || s.mstart[m2 + 1] - s.mstart[m2] != len)
        continue;
      bool same = true;
      for (int a = 0; a < len && same; ++a)
        same = s.q[s.mstart[m2] + a] == s.q[s.mstart[m] + a] &&
               s.kind[s.mstart[m2] + a] == s.kind[s.mstart[m] + a];
      if (same) {
        seen[m2] = 1;
        count++;
      }
    }
    double molSelf = 0.0;
    for (int a = 0; a < len; ++a)
      molSelf += (s.q[s.mstart[m] + a] * s.q[s.mstart[m] + a]);
    self += (molSelf * count);
  }
  self *= -1.0 * ff.alpha * QQ_FACT * M_2_SQRTPI * 0.5;
  *e = self;
  return OK;
}

int Box::BoxCorrection(double *e) {
  if (!cfg.ewald) {
    *e = 0;
    return OK;
  }
  int rc = launch_correction(*this, d_small);
  if (rc)
    return rc;
  if ((rc = CudaCheck(cudaMemcpyAsync(h_pinned, d_small, 8,
                                      cudaMemcpyDeviceToHost, stream),
                      "download")) ||
      (rc = Sync()))
    return rc;
  *e = h_pinned[0];
  return OK;
}

int Box::MolCorrection(int m, double *e) {
  // Ewald::MolCorrection (src/Ewald.cpp:1056-1085), on the host copy of the
  // molecule's current coordinates.
  if (m < 0 || m >= dev.n_mol)
    return Fail(ERR_ARG, "molecule index out of range");
  if (!cfg.ewald) {
    *e = 0;
    return OK;
  }
  int a0 = host.mstart[m], n = host.mstart[m + 1] - a0;
  std::vector<double> xyz(3 * n);
  for (int d = 0; d < 3; ++d) {
    double *src = d == 0 ? dev.x : d == 1 ? dev.y : dev.z;
    int rc = CudaCheck(cudaMemcpyAsync(h_pinned + d * n, src + a0, n * 8,
                                       cudaMemcpyDeviceToHost, stream),
                       "download");
    if (rc)
      return rc;
  }
  int rc = Sync();
  if (rc)
    return rc;
  double corr = 0.0;
  for (int i = 0; i < n; ++i) {
    if (std::fabs(host.q[a0 + i]) < 0.000000001)
      continue;
    for (int j = i + 1; j < n; ++j) {
      double dx = min_image(h_pinned[i] - h_pinned[j], dev.L[0], dev.half[0]);
      double dy = min_image(h_pinned[n + i] - h_pinned[n + j], dev.L[1],
                            dev.half[1]);
      double dz = min_image(h_pinned[2 * n + i] - h_pinned[2 * n + j],
                            dev.L[2], dev.half[2]);
      double distSq = dx * dx + dy * dy + dz * dz;
      double dist = std::sqrt(distSq);
      corr += (host.q[a0 + i] * host.q[a0 + j] * std::erf(ff.alpha * dist) /
               dist);
    }
  }
  *e = -1.0 * QQ_FACT * corr * 1.0 * 1.0;
  return OK;
}

int Box::SystemTotal(double out[9]) {
  // CalculateEnergy::SystemTotal (src/CalculateEnergy.cpp:83-138) after
  // Ewald::UpdateVectorsAndRecipTerms: real space, reciprocal sums of the
  // current coordinates (Ref <- New), self and correction terms.
  double inter, real;
  int rc = BoxInter(&inter, &real);
  if (rc)
    return rc;
  double recip = 0.0, self = 0.0, corr = 0.0;
  if (cfg.ewald) {
    if ((rc = RecipSetup()) || (rc = RecipEnergy(&recip, true)) ||
        (rc = BoxCorrection(&corr)) || (rc = BoxSelf(&self)))
      return rc;
  }
  out[0] = inter;
  out[1] = real;
  out[2] = recip;
  out[3] = self;
  out[4] = corr;
  out[5] = 0.0;
  out[6] = 0.0;
  out[7] = 0.0;
  out[8] = 0.0 + 0.0 + inter + 0.0 + real + recip + self + corr;
  double e5[5] = {inter, real, recip, self, corr};
  return SetEnergy(e5);
}

int Box::GetEnergy(double e5[5]) {
  int rc = CudaCheck(cudaMemcpyAsync(h_pinned, dev.energy, 40,
                                     cudaMemcpyDeviceToHost, stream),
                     "download");
  if (rc || (rc = Sync()))
    return rc;
  for (int i = 0; i < 5; ++i)
    e5[i] = h_pinned[i];
  return OK;
}

int Box::SetEnergy(const double e5[5]) {
  for (int i = 0; i < 5; ++i)
    h_pinned[i] = e5[i];
  int rc = CudaCheck(cudaMemcpyAsync(dev.energy, h_pinned, 40,
                                     cudaMemcpyHostToDevice, stream),
                     "upload");
  if (rc)
    return rc;
  return Sync();
}

static int check_newpos(const Box &b, int m, const double *p, int n) {
  for (int a = 0; a < n; ++a)
    for (int d = 0; d < 3; ++d) {
      double v = p[3 * a + d];
      if (!(v >= 0.0 && v <= b.dev.L[d]))
        return ERR_ARG;
    }
  return OK;
}

int Box::MoleculeInter(int m, const double *new_pos, double *lj, double *real,
                       int *overlap) {
  if (m < 0 || m >= dev.n_mol)
    return Fail(ERR_ARG, "molecule index out of range");
  int n = host.mstart[m + 1] - host.mstart[m];
  if (n > 64)
    return Fail(ERR_UNSUPPORTED, "molecule larger than 64 atoms");
  if (check_newpos(*this, m, new_pos, n))
    return Fail(ERR_ARG, "trial coordinates must lie inside the box");
  std::memcpy(h_pinned, new_pos, 3 * n * sizeof(double));
  int rc = CudaCheck(cudaMemcpyAsync(d_small + 1024, h_pinned, 3 * n * 8,
                                     cudaMemcpyHostToDevice, stream),
                     "upload");
  if (rc || (rc = launch_mol_inter(*this, m, d_small + 1024, d_small)))
    return rc;
  if ((rc = CudaCheck(cudaMemcpyAsync(h_pinned, d_small, 24,
                                      cudaMemcpyDeviceToHost, stream),
                      "download")) ||
      (rc = Sync()))
    return rc;
  *lj = h_pinned[0];
  *real = h_pinned[1];
  *overlap = h_pinned[2] != 0.0;
  return CheckError();
}

// CalculateEnergy::VirialCalc (src/CalculateEnergy.cpp:411-579, LRC off)
// with Ewald::VirialReciprocal (src/Ewald.cpp:1168-1305): inter, real,
// recip, total, then the diagonals of interTens, realTens, recipTens,
// totalTens (the reference computes no off-diagonal components).
int Box::VirialCalc(double out[16]) {
  int rc;
  if ((rc = launch_box_virial(*this, d_small)))
    return rc;
  if (cfg.ewald && (rc = launch_virial_recip(*this, d_small + 8)))
    return rc;
  if ((rc = CudaCheck(cudaMemcpyAsync(h_pinned, d_small, 14 * 8,
                                      cudaMemcpyDeviceToHost, stream),
                      "download")) ||
      (rc = Sync()))
    return rc;
  double vt[3], rt[3], wt[3];
  for (int d = 0; d < 3; ++d) {
    vt[d] = h_pinned[d];
    rt[d] = cfg.electrostatic ? h_pinned[3 + d] * QQ_FACT : 0.0;
    wt[d] = cfg.ewald ? h_pinned[8 + d] + h_pinned[11 + d] : 0.0;
  }
  out[0] = vt[0] + vt[1] + vt[2];
  out[1] = cfg.electrostatic
               ? (h_pinned[3] + h_pinned[4] + h_pinned[5]) * QQ_FACT
               : 0.0;
  out[2] = wt[0] + wt[1] + wt[2];
  out[3] = out[0] + out[1] + out[2];
  for (int d = 0; d < 3; ++d) {
    out[4 + d] = vt[d];
    out[7 + d] = rt[d];
    out[10 + d] = wt[d];
    out[13 + d] = vt[d] + rt[d] + wt[d];
  }
  return CheckError();
}

// CalculateEnergy::SingleMoleculeInter (src/CalculateEnergy.cpp:1494-1556)
int Box::SingleMoleculeInter(int m, const double lam[4], double out[4]) {
  if (m < 0 || m >= dev.n_mol)
    return Fail(ERR_ARG, "molecule index out of range");
  for (int i = 0; i < 4; ++i)
    if (!(lam[i] >= 0.0 && lam[i] <= 1.0))
      return Fail(ERR_ARG, "lambda outside [0, 1]");
  std::memcpy(h_pinned, lam, 4 * sizeof(double));
  int rc = CudaCheck(cudaMemcpyAsync(d_small + 1024, h_pinned, 32,
                                     cudaMemcpyHostToDevice, stream),
                     "upload");
  if (rc || (rc = launch_single_mol_inter(*this, m, d_small + 1024, d_small)))
    return rc;
  if ((rc = CudaCheck(cudaMemcpyAsync(h_pinned, d_small, 32,
                                      cudaMemcpyDeviceToHost, stream),
                      "download")) ||
      (rc = Sync()))
    return rc;
  for (int i = 0; i < 4; ++i)
    out[i] = h_pinned[i];
  return CheckError();
}

// CalculateEnergy::ParticleInter (src/CalculateEnergy.cpp:727-785): atom
// `part` of molecule m (its kind and charge) at each trial position, against
// the atoms in the cell grid.
int Box::ParticleInter(int m, int part, const double *trials, int ntrials,
                       double *en, double *real, int *overlap) {
  if (m < 0 || m >= dev.n_mol || part < 0 ||
      part >= host.mstart[m + 1] - host.mstart[m] || ntrials <= 0 ||
      ntrials > 256)
    return Fail(ERR_ARG, "ParticleInter arguments out of range");
  const int kind = host.kind[host.mstart[m] + part];
  const double charge = host.q[host.mstart[m] + part];
  if (check_newpos(*this, m, trials, ntrials))
    return Fail(ERR_ARG, "trial coordinates must lie inside the box");
  std::memcpy(h_pinned, trials, 3 * ntrials * sizeof(double));
  int rc = CudaCheck(cudaMemcpyAsync(d_small + 1024, h_pinned, 3 * ntrials * 8,
                                     cudaMemcpyHostToDevice, stream),
                     "upload");
  if (rc || (rc = launch_particle_inter(*this, kind, charge, d_small + 1024,
                                        ntrials, d_small)))
    return rc;
  if ((rc = CudaCheck(cudaMemcpyAsync(h_pinned, d_small, 3 * ntrials * 8,
                                      cudaMemcpyDeviceToHost, stream),
                      "download")) ||
      (rc = Sync()))
    return rc;
  for (int t = 0; t < ntrials; ++t) {
    en[t] = h_pinned[3 * t];
    real[t] = h_pinned[3 * t + 1];
    overlap[t] = h_pinned[3 * t + 2] != 0.0;
  }
  return CheckError();
}

int Box::MolReciprocal(int m, const double *new_pos, double *de) {
  if (m < 0 || m >= dev.n_mol)
    return Fail(ERR_ARG, "molecule index out of range");
  if (!cfg.ewald) {
    *de = 0;
    return OK;
  }
  int n = host.mstart[m + 1] - host.mstart[m];
  if (n > 64)
    return Fail(ERR_UNSUPPORTED, "molecule larger than 64 atoms");
  std::memcpy(h_pinned, new_pos, 3 * n * sizeof(double));
  int rc = CudaCheck(cudaMemcpyAsync(d_small + 1024, h_pinned, 3 * n * 8,
                                     cudaMemcpyHostToDevice, stream),
                     "upload");
  if (rc || (rc = launch_mol_recip(*this, m, d_small + 1024, 0, d_small)))
    return rc;
  if ((rc = CudaCheck(cudaMemcpyAsync(h_pinned, d_small, 8,
                                      cudaMemcpyDeviceToHost, stream),
                      "download")) ||
      (rc = Sync()))
    return rc;
  *de = h_pinned[0];
  return OK;
}

int Box::SwapRecip(int m, const double *pos, bool insert, double *de) {
  if (m < 0 || m >= dev.n_mol)
    return Fail(ERR_ARG, "molecule index out of range");
  if (!cfg.ewald) {
    *de = 0;
    return OK;
  }
  int n = host.mstart[m + 1] - host.mstart[m];
  if (n > 64)
    return Fail(ERR_UNSUPPORTED, "molecule larger than 64 atoms");
  std::memcpy(h_pinned, pos, 3 * n * sizeof(double));
  int rc = CudaCheck(cudaMemcpyAsync(d_small + 1024, h_pinned, 3 * n * 8,
                                     cudaMemcpyHostToDevice, stream),
                     "upload");
  if (rc || (rc = launch_mol_recip(*this, m, d_small + 1024, insert ? 1 : 2,
                                   d_small)))
    return rc;
  if ((rc = CudaCheck(cudaMemcpyAsync(h_pinned, d_small, 8,
                                      cudaMemcpyDeviceToHost, stream),
                      "download")) ||
      (rc = Sync()))
    return rc;
  *de = h_pinned[0];
  return OK;
}

int Box::UpdateRecip() {
  // Ewald::UpdateRecip (src/Ewald.cpp:1420-1434): swap New and Ref
  std::swap(dev.sumRnew, dev.sumRref);
  std::swap(dev.sumInew, dev.sumIref);
  return OK;
}

int Box::CopyRecip() {
  if (!cfg.ewald)
    return OK;
  size_t bytes = (size_t)dev.K * 8;
  int rc;
  if ((rc = CudaCheck(cudaMemcpyAsync(dev.sumRnew, dev.sumRref, bytes,
                                      cudaMemcpyDeviceToDevice, stream),
                      "copy")) ||
      (rc = CudaCheck(cudaMemcpyAsync(dev.sumInew, dev.sumIref, bytes,
                                      cudaMemcpyDeviceToDevice, stream),
                      "copy")))
    return rc;
  return OK;
}

int Box::BoxForce(double *inter, double *real, double *h_aF, double *h_mF) {
  int rc = launch_box_force(*this, dev, d_aF, d_mF, d_small);
  if (rc)
    return rc;
  return ForceDownload(inter, real, h_aF, h_mF);
}

int Box::ForceDownload(double *inter, double *real, double *h_aF,
                       double *h_mF) {
  int rc;
  if ((rc = CudaCheck(cudaMemcpyAsync(h_pinned, d_small, 16,
                                      cudaMemcpyDeviceToHost, stream),
                      "download")))
    return rc;
  if (h_aF && (rc = CudaCheck(cudaMemcpyAsync(h_aF, d_aF,
                                              (size_t)dev.n_atoms * 24,
                                              cudaMemcpyDeviceToHost, stream),
                              "download")))
    return rc;
  if (h_mF && (rc = CudaCheck(cudaMemcpyAsync(h_mF, d_mF,
                                              (size_t)dev.n_mol * 24,
                                              cudaMemcpyDeviceToHost, stream),
                              "download")))
    return rc;
  if ((rc = Sync()))
    return rc;
  *inter = h_pinned[0];
  *real = h_pinned[1];
  return CheckError();
}

int Box::BoxForceRecip(double *h_aR, double *h_mR) {
  int rc = launch_force_recip(*this, dev, dev.sumRnew, dev.sumInew, d_aR, d_mR);
  if (rc)
    return rc;
  if (h_aR && (rc = CudaCheck(cudaMemcpyAsync(h_aR, d_aR,
                                              (size_t)dev.n_atoms * 24,
                                              cudaMemcpyDeviceToHost, stream),
                              "download")))
    return rc;
  if (h_mR && (rc = CudaCheck(cudaMemcpyAsync(h_mR, d_mR,
                                              (size_t)dev.n_mol * 24,
                                              cudaMemcpyDeviceToHost, stream),
                              "download")))
    return rc;
  return Sync();
}

int Box::Torque(double *h_tq) {
  int rc = launch_torque(*this, dev, d_aF, d_aR, d_tq);
  if (rc)
    return rc;
  if (h_tq && (rc = CudaCheck(cudaMemcpyAsync(h_tq, d_tq,
                                              (size_t)dev.n_mol * 24,
                                              cudaMemcpyDeviceToHost, stream),
                              "download")))
    return rc;
  return Sync();
}

int Box::GetCoords(double *xyz, double *com) {
  int N = dev.n_atoms, M = dev.n_mol;
  std::vector<double> t(3 * (size_t)std::max(N, M));
  double *src[3] = {dev.x, dev.y, dev.z};
  double *csrc[3] = {dev.cx, dev.cy, dev.cz};
  int rc;
  if (xyz) {
    for (int d = 0; d < 3; ++d)
      if ((rc = CudaCheck(cudaMemcpyAsync(t.data() + (size_t)d * N, src[d],
                                          (size_t)N * 8, cudaMemcpyDeviceToHost,
                                          stream),
                          "download")))
        return rc;
    if ((rc = Sync()))
      return rc;
    for (int i = 0; i < N; ++i)
      for (int d = 0; d < 3; ++d)
        xyz[3 * i + d] = t[(size_t)d * N + i];
  }
  if (com) {
    for (int d = 0; d < 3; ++d)
      if ((rc = CudaCheck(cudaMemcpyAsync(t.data() + (size_t)d * M, csrc[d],
                                          (size_t)M * 8, cudaMemcpyDeviceToHost,
                                          stream),
                          "download")))
        return rc;
    if ((rc = Sync()))
      return rc;
    for (int i = 0; i < M; ++i)
      for (int d = 0; d < 3; ++d)
        com[3 * i + d] = t[(size_t)d * M + i];
  }
  return OK;
}

// Replace the coordinates (and molecule centres) and bring every derived
// quantity in line, as System::Init does after reading coordinates
// (src/System.cpp:67-100): CellList::GridAll, the Ewald structure factors
// (BoxReciprocalSetup + SetRecipRef) and the running energies
// (CalculateEnergy::SystemTotal).  Without `com` the centres are computed
// the way COM::CalcCOM does (which also re-wraps the atoms).
int Box::SetCoords(const double *xyz, const double *com) {
  int N = dev.n_atoms, M = dev.n_mol;
  for (int i = 0; i < N; ++i)
    for (int d = 0; d < 3; ++d) {
      double v = xyz[3 * i + d];
      if (!(v >= 0.0 && v <= dev.L[d]))
        return Fail(ERR_ARG, "coordinates must lie inside the box");
    }
  HostSystem s = host;
  for (int i = 0; i < N; ++i) {
    s.x[i] = xyz[3 * i];
    s.y[i] = xyz[3 * i + 1];
    s.z[i] = xyz[3 * i + 2];
  }
  if (com) {
    for (int m = 0; m < M; ++m) {
      s.cx[m] = com[3 * m];
      s.cy[m] = com[3 * m + 1];
      s.cz[m] = com[3 * m + 2];
    }
  } else {
    calc_com(s);
  }
  const double *src[6] = {s.x.data(), s.y.data(), s.z.data(),
                          s.cx.data(), s.cy.data(), s.cz.data()};
  double *dst[6] = {dev.x, dev.y, dev.z, dev.cx, dev.cy, dev.cz};
  int rc;
  for (int d = 0; d < 6; ++d)
    if ((rc = CudaCheck(cudaMemcpyAsync(dst[d], src[d],
                                        (size_t)(d < 3 ? N : M) * 8,
                                        cudaMemcpyHostToDevice, stream),
                        "upload")))
      return rc;
  if ((rc = Sync()) || (rc = GridAll()))
    return rc;
  double tot[9];
  return SystemTotal(tot);
}


// ---------------------------------------------------------------------------
// Box edges that change (VolumeTransfer, src/moves/VolumeTransfer.h:143-190)
// ---------------------------------------------------------------------------
static bool inside(const double *xyz, int n, const double L[3]) {
  for (int i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d) {
      double v = xyz[3 * i + d];
      if (!(v >= 0.0 && v <= L[d]))
        return false;
    }
  return true;
}

// Trial coordinates [N * 3] at edges L in the trial state's own buffers
// (atom back-pointers included, so the box's grid is untouched); with
// `grid`, also the trial cell grid.
int Box::TrialCoords(const double L[3], const double *xyz, bool grid) {
  const int N = dev.n_atoms, M = dev.n_mol;
  if (!inside(xyz, N, L))
    return Fail(ERR_ARG, "coordinates must lie inside the box edges");
  DevBox &v = trial.v;
  int rc;
  if (!trial.v.x) {
    v = dev;
    v.x = v.y = v.z = v.cx = v.cy = v.cz = nullptr;
    v.atom_cell = v.atom_slot = nullptr;
    v.nbr = v.cell_count = v.cell_atom = v.cell_meta = nullptr;
    v.cell_pos = nullptr;
    v.cell_fix = nullptr;
    v.cell_qlo = nullptr;
    if ((rc = regrow(*this, (void **)&v.x, (size_t)N * 8, trial.allocs)) ||
        (rc = regrow(*this, (void **)&v.y, (size_t)N * 8, trial.allocs)) ||
        (rc = regrow(*this, (void **)&v.z, (size_t)N * 8, trial.allocs)) ||
        (rc = regrow(*this, (void **)&v.cx, (size_t)M * 8, trial.allocs)) ||
        (rc = regrow(*this, (void **)&v.cy, (size_t)M * 8, trial.allocs)) ||
        (rc = regrow(*this, (void **)&v.cz, (size_t)M * 8, trial.allocs)) ||
        (rc = regrow(*this, (void **)&v.atom_cell, (size_t)N * 4,
                     trial.allocs)) ||
        (rc = regrow(*this, (void **)&v.atom_slot, (size_t)N * 4,
                     trial.allocs)))
      return rc;
  }
  std::vector<double> t(3 * (size_t)N);
  for (int i = 0; i < N; ++i)
    for (int d = 0; d < 3; ++d)
      t[(size_t)d * N + i] = xyz[3 * i + d];
  double *dst[3] = {v.x, v.y, v.z};
  for (int d = 0; d < 3; ++d)
    if ((rc = CudaCheck(cudaMemcpyAsync(dst[d], t.data() + (size_t)d * N,
                                        (size_t)N * 8, cudaMemcpyHostToDevice,
                                        stream),
                        "upload")))
      return rc;
  if (grid) {
    if ((rc = GridGeometry(L, t.data(), t.data() + N, t.data() + 2 * (size_t)N,
                           v, &trial.cell_cap, &trial.nbr_cap, trial.allocs)) ||
        (rc = launch_grid_all(*this, v)))
      return rc;
  } else {
    for (int d = 0; d < 3; ++d) {
      v.L[d] = L[d];
      v.half[d] = L[d] * 0.5;
      v.invL[d] = 1.0 / L[d];
    }
    v.volume = L[0] * L[1] * L[2];
  }
  return Sync();  // `t` goes out of scope
}

int Box::BoxInterAt(const double L[3], const double *xyz, double *inter,
                    double *real) {
  int rc = TrialCoords(L, xyz, true);
  if (rc || (rc = launch_box_inter_view(*this, trial.v, d_small)))
    return rc;
  if ((rc = CudaCheck(cudaMemcpyAsync(h_pinned, d_small, 16,
                                      cudaMemcpyDeviceToHost, stream),
                      "download")) ||
      (rc = Sync()))
    return rc;
  *inter = h_pinned[0];
  *real = h_pinned[1];
  return CheckError();
}

int Box::BoxForceAt(const double *xyz, double *inter, double *real,
                    double *h_aF, double *h_mF) {
  int rc = TrialCoords(dev.L, xyz, true);
  if (rc || (rc = launch_box_force(*this, trial.v, d_aF, d_mF, d_small)))
    return rc;
  return ForceDownload(inter, real, h_aF, h_mF);
}

int Box::RecipInit(const double L[3]) {
  if (!cfg.ewald)
    return OK;
  for (int d = 0; d < 3; ++d)
    if (!(L[d] > 0))
      return Fail(ERR_ARG, "box edge must be positive");
  int rc = BuildKSet(L, knew);
  if (rc || (rc = EnsureSums(knew.K)))
    return rc;
  return OK;
}

int Box::UpdateRecipVec() {
  if (!cfg.ewald)
    return OK;
  if (mc)
    return Fail(ERR_STATE,
                "the Monte Carlo loop of this box runs at fixed box edges");
  if (!knew.K)
    return Fail(ERR_STATE, "no k-vector set from gb_recip_init to swap in");
  std::swap(kref, knew);
  MirrorKRef();
  return OK;
}

bool Box::KSetMatchesEdges() const {
  if (!cfg.ewald)
    return true;
  for (int d = 0; d < 3; ++d)
    if (kref.L[d] != dev.L[d])
      return false;
  return true;
}

int Box::RecipSumsCoords(const double *xyz, bool new_set) {
  if (!cfg.ewald)
    return OK;
  const KSet &ks = new_set ? knew : kref;
  if (new_set && !knew.K)
    return Fail(ERR_STATE, "gb_recip_init has not built a k-vector set");
  int rc = TrialCoords(ks.L, xyz, false);
  if (rc)
    return rc;
  DevBox v = trial.v;
  v.K = ks.K;
  v.kmax = ks.kmax;
  v.nrun = ks.nrun;
  v.kx = ks.kx;
  v.ky = ks.ky;
  v.kz = ks.kz;
  v.prefact = ks.prefact;
  v.hsqr = ks.hsqr;
  v.kn = ks.kn;
  v.prefact_f = ks.prefact_f;
  v.krun = ks.krun;
  v.krun_k = ks.krun_k;
  if ((rc = launch_recip_sums_view(*this, v, v.x, v.y, v.z, dev.sumRnew,
                                   dev.sumInew)))
    return rc;
  new_sums_set_ = new_set ? 1 : 0;
  return Sync();
}

int Box::RecipEnergyNew(double *e, bool new_volume) {
  if (!cfg.ewald) {
    *e = 0;
    return OK;
  }
  const KSet &ks = new_volume ? knew : kref;
  if (new_volume && !knew.K)
    return Fail(ERR_STATE, "gb_recip_init has not built a k-vector set");
  DevBox v = dev;
  v.K = ks.K;
  v.prefact = ks.prefact;
  int rc = launch_recip_energy_view(*this, v, dev.sumRnew, dev.sumInew,
                                    d_small);
  if (rc)
    return rc;
  if ((rc = CudaCheck(cudaMemcpyAsync(h_pinned, d_small, 8,
                                      cudaMemcpyDeviceToHost, stream),
                      "download")) ||
      (rc = Sync()))
    return rc;
  *e = h_pinned[0];
  return OK;
}

// New box edges with coordinates and centres: what VolumeTransfer::Accept
// leaves (src/moves/VolumeTransfer.h:241-270: the new coordinates, box
// dimensions, UpdateRecip and UpdateRecipVec), here with every derived
// quantity recomputed as System::Init does: the cell grid of the new edges,
// the k-vector set of the new edges (the one gb_recip_init built for them, or
// a new one), the structure factors and the running energies.
int Box::SetBox(const double L[3], const double *xyz, const double *com) {
  if (mc)
    return Fail(ERR_STATE,
                "the Monte Carlo loop of this box runs at fixed box edges");
  for (int d = 0; d < 3; ++d)
    if (!(L[d] > 0))
      return Fail(ERR_ARG, "box edge must be positive");
  const int N = dev.n_atoms, M = dev.n_mol;
  if (!inside(xyz, N, L))
    return Fail(ERR_ARG, "coordinates must lie inside the box edges");
  HostSystem s = host;
  for (int d = 0; d < 3; ++d)
    s.L[d] = L[d];
  for (int i = 0; i < N; ++i) {
    s.x[i] = xyz[3 * i];
    s.y[i] = xyz[3 * i + 1];
    s.z[i] = xyz[3 * i + 2];
  }
  if (com) {
    for (int m = 0; m < M; ++m) {
      s.cx[m] = com[3 * m];
      s.cy[m] = com[3 * m + 1];
      s.cz[m] = com[3 * m + 2];
    }
  } else {
    calc_com(s);
  }
  int rc;
  if ((rc = Sync()) ||
      (rc = GridGeometry(L, s.x.data(), s.y.data(), s.z.data(), dev,
                         &grid_cell_cap_, &grid_nbr_cap_, allocs_)))
    return rc;
  // force-field constants that depend on the edges (the mixed form's FP32
  // turn length); the erfc table does not
  const double *etab = ff.erfc_tab, *vtab = ff.vir_tab;
  int key0 = ff.etab_key0, nseg = ff.etab_nseg;
  build_ff(s, cfg, &ff);
  ff.erfc_tab = etab;
  ff.vir_tab = vtab;
  ff.etab_key0 = key0;
  ff.etab_nseg = nseg;
  if ((rc = CudaCheck(cudaMemcpyAsync(d_ff, &ff, sizeof(FF),
                                      cudaMemcpyHostToDevice, stream),
                      "upload")))
    return rc;
  if (cfg.ewald && !KSetMatchesEdges()) {
    bool built = knew.K > 0;
    for (int d = 0; d < 3 && built; ++d)
      built = knew.L[d] == L[d];
    if (built)
      std::swap(kref, knew);
    else if ((rc = BuildKSet(L, kref)))
      return rc;
    if ((rc = EnsureSums(kref.K)))
      return rc;
    MirrorKRef();
  }
  const double *src[6] = {s.x.data(), s.y.data(), s.z.data(),
                          s.cx.data(), s.cy.data(), s.cz.data()};
  double *dst[6] = {dev.x, dev.y, dev.z, dev.cx, dev.cy, dev.cz};
  for (int d = 0; d < 6; ++d)
    if ((rc = CudaCheck(cudaMemcpyAsync(dst[d], src[d],
                                        (size_t)(d < 3 ? N : M) * 8,
                                        cudaMemcpyHostToDevice, stream),
                        "upload")))
      return rc;
  host.L[0] = L[0];
  host.L[1] = L[1];
  host.L[2] = L[2];
  if ((rc = Sync()) || (rc = GridAll()))
    return rc;
  double tot[9];
  return SystemTotal(tot);
}

// Ewald::SwapSelf (src/Ewald.cpp:1375-1391): self energy of molecule m.
int Box::SwapSelf(int m, double *e) {
  if (m < 0 || m >= dev.n_mol)
    return Fail(ERR_ARG, "molecule index out of range");
  if (!cfg.ewald) {
    *e = 0;
    return OK;
  }
  double en_self = 0.0;
  for (int a = host.mstart[m]; a < host.mstart[m + 1]; ++a)
    en_self -= (host.q[a] * host.q[a]);
  *e = (en_self * ff.alpha * QQ_FACT * M_2_SQRTPI * 0.5);
  return OK;
}

// Ewald::SwapCorrection (src/Ewald.cpp:1311-1333): intramolecular
// correction of molecule m at positions pos [n_atoms_of_m * 3] in this box.
int Box::SwapCorrection(int m, const double *pos, double *e) {
  if (m < 0 || m >= dev.n_mol)
    return Fail(ERR_ARG, "molecule index out of range");
  if (!cfg.ewald) {
    *e = 0;
    return OK;
  }
  int a0 = host.mstart[m], n = host.mstart[m + 1] - a0;
  double correction = 0.0;
  for (int i = 0; i < n; i++)
    for (int j = i + 1; j < n; j++) {
      double dx = min_image(pos[3 * i] - pos[3 * j], dev.L[0], dev.half[0]);
      double dy = min_image(pos[3 * i + 1] - pos[3 * j + 1], dev.L[1],
                            dev.half[1]);
      double dz = min_image(pos[3 * i + 2] - pos[3 * j + 2], dev.L[2],
                            dev.half[2]);
      double distSq = dx * dx + dy * dy + dz * dz;
      double dist = std::sqrt(distSq);
      correction -= (host.q[a0 + i] * host.q[a0 + j] *
                     std::erf(ff.alpha * dist) / dist);
    }
  *e = QQ_FACT * correction;
  return OK;
}

int Box::GetCells(int *cell_of_atom, int edge[3]) {
  int rc = CudaCheck(cudaMemcpyAsync(cell_of_atom, dev.atom_cell,
                                     (size_t)dev.n_atoms * 4,
                                     cudaMemcpyDeviceToHost, stream),
                     "download");
  if (rc || (rc = Sync()))
    return rc;
  for (int k = 0; k < 3; ++k)
    edge[k] = dev.edge[k];
  return OK;
}

int Box::GetKVectors(double *o) {
  if (!cfg.ewald)
    return OK;
  size_t K = dev.K;
  double *src[7] = {dev.kx, dev.ky, dev.kz, dev.prefact, dev.hsqr,
                    dev.sumRref, dev.sumIref};
  for (int i = 0; i < 7; ++i) {
    int rc = CudaCheck(cudaMemcpyAsync(o + i * K, src[i], K * 8,
                                       cudaMemcpyDeviceToHost, stream),
                       "download");
    if (rc)
      return rc;
  }
  return Sync();
}

int Box::GetSumNew(double *sr, double *si) {
  if (!cfg.ewald)
    return OK;
  size_t K = dev.K;
  int rc;
  if ((rc = CudaCheck(cudaMemcpyAsync(sr, dev.sumRnew, K * 8,
                                      cudaMemcpyDeviceToHost, stream),
                      "download")) ||
      (rc = CudaCheck(cudaMemcpyAsync(si, dev.sumInew, K * 8,
                                      cudaMemcpyDeviceToHost, stream),
                      "download")))
    return rc;
  return Sync();
}

}  // namespace gb
