/* CPU oracle for the GOMC Monte Carlo energy path -- TEST INFRASTRUCTURE.
 *
 * Restates, in plain C, the reference's FP64 algorithms for one orthogonal
 * NVT box.  Each function names the reference lines it follows; floating-point
 * expressions keep the reference's evaluation order (the library is built with
 * -ffp-contract=off so that no multiply-add is fused on any host).
 * Used only as the checker by tests, the smoke check and the CPU baseline of
 * the benchmark.
 */
#define _GNU_SOURCE
#include "gomc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define QQ_FACT 167103.208067979 /* lib/NumLib.h:22 */
#define NB27 27
#define END_CELL (-1)

static int g_threads = 1;
void ora_set_threads(int n) { g_threads = n > 0 ? n : 1; }

struct ora_sys {
  int n_atoms, n_mol, n_kinds;
  double box[3], half[3], volume;
  double *x, *y, *z;           /* current coordinates */
  double *cx, *cy, *cz;        /* molecule centres (COM) */
  int *kind, *mol;
  double *q;
  int *no_charge;
  int *mstart;                 /* n_mol + 1 */
  /* force field tables, FlatIndex(i, j) = i + j * n_kinds
   * (src/FFParticle.h:116, src/FFParticle.cpp:200-242) */
  double *sigmaSq, *eps_cn, *nexp, *eps_cn_6, *nOver6;
  double rcut, rcutSq, rcutLowSq, rcutCoulSq, alpha, alphaSq, recip_rcut,
      recip_rcut_Sq, beta;
  int ewald, electrostatic;
  /* cell list (src/CellList.h:56-86) */
  int edge[3];
  double cellSize[3];
  int ncell;
  int *head, *list, *nbr; /* nbr[ncell * 27] */
  /* Ewald reference-state tables (src/Ewald.h:196-211) */
  int K, kmax;
  double *kx, *ky, *kz, *hsqr, *prefact;
  double *sumRnew, *sumInew, *sumRref, *sumIref;
  /* running energies */
  double e_inter, e_real, e_recip, e_self, e_corr;
};

/* ------------------------------------------------------------------------ */
/* Geometry: BoxDimensions (src/BoxDimensions.h:169-175, .cpp:229-353)      */
/* ------------------------------------------------------------------------ */
static inline double min_image(double raw, double ax, double half) {
  if (raw > half)
    raw -= ax;
  else if (raw < -half)
    raw += ax;
  return raw;
}
static inline double wrap1(double v, double ax) {
  if (v >= ax)
    v -= ax;
  else if (v < 0)
    v += ax;
  return v;
}
static inline double unwrap1(double v, double ref, double ax, double half) {
  if (fabs(ref - v) > half) {
    if (ref < half)
      v -= ax;
    else
      v += ax;
  }
  return v;
}
/* InRcut: dist = MinImage(a - b), distSq = dx*dx + dy*dy + dz*dz */
static inline double dist_sq(const ora_sys *s, double ax, double ay, double az,
                             double bx, double by, double bz, double *d) {
  double dx = min_image(ax - bx, s->box[0], s->half[0]);
  double dy = min_image(ay - by, s->box[1], s->half[1]);
  double dz = min_image(az - bz, s->box[2], s->half[2]);
  if (d) {
    d[0] = dx;
    d[1] = dy;
    d[2] = dz;
  }
  return dx * dx + dy * dy + dz * dz;
}

/* ------------------------------------------------------------------------ */
/* Pair potentials: FFParticle (src/FFParticle.cpp:295-446)                 */
/* ------------------------------------------------------------------------ */
static inline double calc_en(const ora_sys *s, double distSq, int k1, int k2) {
  if (s->rcutSq < distSq)
    return 0.0;
  int idx = k1 + k2 * s->n_kinds;
  double rRat2 = s->sigmaSq[idx] / distSq;
  double rRat4 = rRat2 * rRat2;
  double attract = rRat4 * rRat2;
  double repulse = pow(rRat2, (s->nexp[idx] * 0.5));
  return (s->eps_cn[idx] * (repulse - attract));
}
static inline double calc_vir(const ora_sys *s, double distSq, int k1, int k2) {
  if (s->rcutSq < distSq)
    return 0.0;
  int idx = k1 + k2 * s->n_kinds;
  double rNeg2 = 1.0 / distSq;
  double rRat2 = rNeg2 * s->sigmaSq[idx];
  double rRat4 = rRat2 * rRat2;
  double attract = rRat4 * rRat2;
  double repulse = pow(rRat2, (s->nexp[idx] * 0.5));
  return s->eps_cn_6[idx] * (s->nOver6[idx] * repulse - attract) * rNeg2;
}
static inline double calc_coulomb(const ora_sys *s, double distSq, double qq) {
  if (s->rcutCoulSq < distSq)
    return 0.0;
  if (s->ewald) {
    double dist = sqrt(distSq);
    double val = s->alpha * dist;
    return qq * erfc(val) / dist;
  } else {
    double dist = sqrt(distSq);
    return qq / dist;
  }
}
static inline double calc_coulomb_vir(const ora_sys *s, double distSq,
                                      double qq) {
  if (s->rcutCoulSq < distSq)
    return 0.0;
  if (s->ewald) {
    double dist = sqrt(distSq);
    double constValue = s->alpha * M_2_SQRTPI;
    double expConstValue = exp(-1.0 * s->alphaSq * distSq);
    double temp = 1.0 - erf(s->alpha * dist);
    return qq * (temp / dist + constValue * expConstValue) / distSq;
  } else {
    double dist = sqrt(distSq);
    return qq / (distSq * dist);
  }
}

/* ------------------------------------------------------------------------ */
/* Cell list: src/CellList.cpp:81-252, src/CellList.h:88-101                */
/* ------------------------------------------------------------------------ */
static inline int position_to_cell(const ora_sys *s, double px, double py,
                                   double pz) {
  int x = (int)(px / s->cellSize[0]);
  int y = (int)(py / s->cellSize[1]);
  int z = (int)(pz / s->cellSize[2]);
  x -= (x == s->edge[0] ? 1 : 0);
  y -= (y == s->edge[1] ? 1 : 0);
  z -= (z == s->edge[2] ? 1 : 0);
  return x * s->edge[1] * s->edge[2] + y * s->edge[2] + z;
}
static void resize_grid(ora_sys *s) {
  for (int d = 0; d < 3; ++d) {
    int e = (int)floor(s->box[d] / s->rcut);
    s->edge[d] = e > 3 ? e : 3;
    s->cellSize[d] = s->box[d] / s->edge[d];
  }
  int n = s->edge[0] * s->edge[1] * s->edge[2];
  if (n != s->ncell) {
    free(s->head);
    free(s->nbr);
    s->ncell = n;
    s->head = (int *)malloc(sizeof(int) * n);
    s->nbr = (int *)malloc(sizeof(int) * n * NB27);
  }
  int *e = s->edge;
  for (int x = 0; x < e[0]; ++x)
    for (int y = 0; y < e[1]; ++y)
      for (int z = 0; z < e[2]; ++z) {
        int cell = x * e[2] * e[1] + y * e[2] + z;
        int c = 0;
        for (int dx = -1; dx <= 1; ++dx)
          for (int dy = -1; dy <= 1; ++dy)
            for (int dz = -1; dz <= 1; ++dz)
              s->nbr[cell * NB27 + c++] =
                  ((x + dx + e[0]) % e[0]) * e[2] * e[1] +
                  ((y + dy + e[1]) % e[1]) * e[2] + ((z + dz + e[2]) % e[2]);
      }
}
static void add_mol(ora_sys *s, int m) {
  for (int p = s->mstart[m]; p < s->mstart[m + 1]; ++p) {
    int cell = position_to_cell(s, s->x[p], s->y[p], s->z[p]);
    s->list[p] = s->head[cell];
    s->head[cell] = p;
  }
}
static void remove_mol(ora_sys *s, int m) {
  for (int p = s->mstart[m]; p < s->mstart[m + 1]; ++p) {
    int cell = position_to_cell(s, s->x[p], s->y[p], s->z[p]);
    int at = s->head[cell];
    if (at == p) {
      s->head[cell] = s->list[p];
    } else {
      while (at != END_CELL) {
        if (s->list[at] == p) {
          s->list[at] = s->list[p];
          break;
        }
        at = s->list[at];
      }
    }
  }
}
void ora_grid_all(ora_sys *s) {
  resize_grid(s);
  for (int c = 0; c < s->ncell; ++c)
    s->head[c] = END_CELL;
  for (int m = 0; m < s->n_mol; ++m)
    add_mol(s, m);
}
/* Neighbour enumeration order of CellList::Neighbors (src/CellList.h:196-225):
 * the 27 cells in table order, each cell's linked list from its head. */
static int gather_neighbors(const ora_sys *s, int cell, int *out) {
  int n = 0;
  for (int c = 0; c < NB27; ++c)
    for (int at = s->head[s->nbr[cell * NB27 + c]]; at != END_CELL;
         at = s->list[at])
      out[n++] = at;
  return n;
}

/* ------------------------------------------------------------------------ */
/* Ewald: src/Ewald.cpp                                                     */
/* ------------------------------------------------------------------------ */
/* RecipInitOrth, src/Ewald.cpp:847-903 */
static void recip_init(ora_sys *s) {
  double alpsqr4 = 1.0 / (4.0 * s->alphaSq);
  double cv[3];
  for (int d = 0; d < 3; ++d) {
    cv[d] = 1.0 / s->box[d];
    cv[d] *= 2.0 * M_PI;
  }
  double vol = s->volume / (4.0 * M_PI);
  int nkx_max = (int)(s->recip_rcut * s->box[0] / (2.0 * M_PI)) + 1;
  int nky_max = (int)(s->recip_rcut * s->box[1] / (2.0 * M_PI)) + 1;
  int nkz_max = (int)(s->recip_rcut * s->box[2] / (2.0 * M_PI)) + 1;
  int km = nkx_max > nky_max ? nkx_max : nky_max;
  int kmz = nky_max > nkz_max ? nky_max : nkz_max;
  s->kmax = km > kmz ? km : kmz;
  /* count, then fill */
  for (int pass = 0; pass < 2; ++pass) {
    int counter = 0;
    for (int x = 0; x <= nkx_max; x++) {
      int nky_min = (x == 0) ? 0 : -nky_max;
      for (int y = nky_min; y <= nky_max; y++) {
        int nkz_min = (x == 0 && y == 0) ? 1 : -nkz_max;
        for (int z = nkz_min; z <= nkz_max; z++) {
          double kX = cv[0] * x;
          double kY = cv[1] * y;
          double kZ = cv[2] * z;
          double ksqr = kX * kX + kY * kY + kZ * kZ;
          if (ksqr < s->recip_rcut_Sq) {
            if (pass == 1) {
              s->kx[counter] = kX;
              s->ky[counter] = kY;
              s->kz[counter] = kZ;
              s->hsqr[counter] = ksqr;
              s->prefact[counter] =
                  QQ_FACT * exp(-ksqr * alpsqr4) / (ksqr * vol);
            }
            counter++;
          }
        }
      }
    }
    if (pass == 0) {
      s->K = counter;
      size_t b = sizeof(double) * (counter > 0 ? counter : 1);
      s->kx = (double *)realloc(s->kx, b);
      s->ky = (double *)realloc(s->ky, b);
      s->kz = (double *)realloc(s->kz, b);
      s->hsqr = (double *)realloc(s->hsqr, b);
      s->prefact = (double *)realloc(s->prefact, b);
      s->sumRnew = (double *)realloc(s->sumRnew, b);
      s->sumInew = (double *)realloc(s->sumInew, b);
      s->sumRref = (double *)realloc(s->sumRref, b);
      s->sumIref = (double *)realloc(s->sumIref, b);
    }
  }
}

/* BoxReciprocalSetup/Sums, src/Ewald.cpp:193-361 (CPU branch) */
static void box_recip_sums(ora_sys *s, const double *X, const double *Y,
                           const double *Z) {
  memset(s->sumRnew, 0, sizeof(double) * s->K);
  memset(s->sumInew, 0, sizeof(double) * s->K);
  for (int m = 0; m < s->n_mol; ++m) {
    int start = s->mstart[m], len = s->mstart[m + 1] - start;
#pragma omp parallel for num_threads(g_threads)
    for (int i = 0; i < s->K; i++) {
      double sumReal = 0.0, sumImaginary = 0.0;
      for (int j = 0; j < len; j++) {
        int a = start + j;
        if (s->no_charge[a])
          continue;
        double dot = (X[a] * s->kx[i] + Y[a] * s->ky[i] + Z[a] * s->kz[i]);
        sumReal += (s->q[a] * cos(dot));
        sumImaginary += (s->q[a] * sin(dot));
      }
      s->sumRnew[i] += (1.0 * sumReal);
      s->sumInew[i] += (1.0 * sumImaginary);
    }
  }
}
/* BoxReciprocal, src/Ewald.cpp:375-406 (sums "new", prefactRef) */
static double box_recip_energy(const ora_sys *s) {
  double e = 0.0;
  for (int i = 0; i < s->K; i++)
    e += ((s->sumRnew[i] * s->sumRnew[i] + s->sumInew[i] * s->sumInew[i]) *
          s->prefact[i]);
  return e;
}
/* SetRecipRef, src/Ewald.cpp:1021-1053 */
static void set_recip_ref(ora_sys *s) {
  memcpy(s->sumRref, s->sumRnew, sizeof(double) * s->K);
  memcpy(s->sumIref, s->sumInew, sizeof(double) * s->K);
}
double ora_box_reciprocal_sums(ora_sys *s, const double *coords) {
  if (!s->ewald)
    return 0.0;
  if (coords) {
    int n = s->n_atoms;
    double *X = (double *)malloc(sizeof(double) * 3 * n);
    for (int i = 0; i < n; ++i) {
      X[i] = coords[3 * i];
      X[n + i] = coords[3 * i + 1];
      X[2 * n + i] = coords[3 * i + 2];
    }
    box_recip_sums(s, X, X + n, X + 2 * n);
    free(X);
  } else {
    box_recip_sums(s, s->x, s->y, s->z);
  }
  return box_recip_energy(s);
}
/* BoxSelf, src/Ewald.cpp:1125-1163 (no fractional molecules) */
double ora_box_self(const ora_sys *s) {
  if (!s->ewald)
    return 0.0;
  /* per molecule kind: sum of q^2 times molecule count; molecules of one
   * kind share the charge list, so summing per molecule in kind order with
   * the same charges gives the same per-kind partial. */
  double self = 0.0;
  /* group molecules by identical charge lists in first-seen order */
  int *seen = (int *)calloc(s->n_mol, sizeof(int));
  for (int m = 0; m < s->n_mol; ++m) {
    if (seen[m])
      continue;
    int len = s->mstart[m + 1] - s->mstart[m];
    int count = 0;
    for (int m2 = m; m2 < s->n_mol; ++m2) {
      if (seen[m2] || s->mstart[m2 + 1] - s->mstart[m2] != len)
        continue;
      int same = 1;
      for (int a = 0; a < len; ++a)
        if (s->q[s->mstart[m2] + a] != s->q[s->mstart[m] + a] ||
            s->kind[s->mstart[m2] + a] != s->kind[s->mstart[m] + a])
          same = 0;
      if (same) {
        seen[m2] = 1;
        count++;
      }
    }
    double molSelf = 0.0;
    for (int a = 0; a < len; ++a)
      molSelf += (s->q[s->mstart[m] + a] * s->q[s->mstart[m] + a]);
    self += (molSelf * count);
  }
  free(seen);
  self *= -1.0 * s->alpha * QQ_FACT * M_2_SQRTPI * 0.5;
  return self;
}
/* MolCorrection, src/Ewald.cpp:1056-1085 */
double ora_mol_correction(const ora_sys *s, int m) {
  if (!s->ewald)
    return 0.0;
  int start = s->mstart[m], n = s->mstart[m + 1] - start;
  double correction = 0.0;
  for (int i = 0; i < n; i++) {
    if (s->no_charge[start + i])
      continue;
    for (int j = i + 1; j < n; j++) {
      int a = start + i, b = start + j;
      double distSq =
          dist_sq(s, s->x[a], s->y[a], s->z[a], s->x[b], s->y[b], s->z[b], 0);
      double dist = sqrt(distSq);
      correction += (s->q[a] * s->q[b] * erf(s->alpha * dist) / dist);
    }
  }
  return -1.0 * QQ_FACT * correction * 1.0 * 1.0;
}

/* ------------------------------------------------------------------------ */
/* Real space: BoxInter / MoleculeInter / ParticleInter / BoxForce          */
/* ------------------------------------------------------------------------ */
/* GetCellListNeighbor (src/CellList.cpp:258-285): cell-sorted atom vector */
static void cell_vectors(const ora_sys *s, int *cellVector, int *cellStart,
                         int *mapP) {
  int vi = 0;
  for (int cell = 0; cell < s->ncell; cell++) {
    cellStart[cell] = vi;
    for (int p = s->head[cell]; p != END_CELL; p = s->list[p]) {
      cellVector[vi++] = p;
      mapP[p] = cell;
    }
    /* sort the cell's particles ascending (insertion sort, small cells) */
    for (int i = cellStart[cell] + 1; i < vi; ++i) {
      int v = cellVector[i], j = i - 1;
      while (j >= cellStart[cell] && cellVector[j] > v) {
        cellVector[j + 1] = cellVector[j];
        --j;
      }
      cellVector[j + 1] = v;
    }
  }
  cellStart[s->ncell] = vi;
}

/* BoxInter CPU branch, src/CalculateEnergy.cpp:198-247, or BoxForce CPU
 * branch, :325-394, over coordinates X/Y/Z with the current cell grid. */
static void box_pairs(ora_sys *s, const double *X, const double *Y,
                      const double *Z, double *aF, double *mF, double *outLJ,
                      double *outReal) {
  int n = s->n_atoms;
  int *cv = (int *)malloc(sizeof(int) * n);
  int *cs = (int *)malloc(sizeof(int) * (s->ncell + 1));
  int *mp = (int *)malloc(sizeof(int) * n);
  cell_vectors(s, cv, cs, mp);
  double tempREn = 0.0, tempLJEn = 0.0;
  int nv = cs[s->ncell];
  for (int ci = 0; ci < nv; ci++) {
    int cur = cv[ci];
    int cell = mp[cur];
    for (int nc = 0; nc < NB27; nc++) {
      int ncell = s->nbr[cell * NB27 + nc];
      for (int ni = cs[ncell]; ni < cs[ncell + 1]; ni++) {
        int np = cv[ni];
        if (cur < np && s->mol[cur] != s->mol[np]) {
          double d[3];
          double distSq = dist_sq(s, X[cur], Y[cur], Z[cur], X[np], Y[np],
                                  Z[np], d);
          if (s->rcutSq > distSq) {
            double fR = 0.0;
            int hasR = 0;
            if (s->electrostatic) {
              double qq = s->q[cur] * s->q[np] * QQ_FACT;
              if (qq != 0.0) {
                tempREn += calc_coulomb(s, distSq, qq);
                if (aF) {
                  fR = calc_coulomb_vir(s, distSq, qq);
                  hasR = 1;
                }
              }
            }
            tempLJEn += calc_en(s, distSq, s->kind[cur], s->kind[np]);
            if (aF) {
              double fL = calc_vir(s, distSq, s->kind[cur], s->kind[np]);
              double f[3];
              for (int k = 0; k < 3; ++k) {
                double fl = d[k] * fL;
                double fr = hasR ? d[k] * fR : 0.0;
                f[k] = fl + fr;
              }
              for (int k = 0; k < 3; ++k) {
                aF[3 * cur + k] += f[k];
                aF[3 * np + k] += -f[k];
                mF[3 * s->mol[cur] + k] += f[k];
                mF[3 * s->mol[np] + k] += -f[k];
              }
            }
          }
        }
      }
    }
  }
  free(cv);
  free(cs);
  free(mp);
  *outLJ = tempLJEn;
  *outReal = tempREn;
}

/* CalculateEnergy::VirialCalc, src/CalculateEnergy.cpp:411-579 (CPU
 * branch :458-519; LRC off) with Ewald::VirialReciprocal,
 * src/Ewald.cpp:1168-1305 (CPU branch :1228-1283).  out16 = inter, real,
 * recip, total, then the diagonals (xx, yy, zz) of interTens, realTens,
 * recipTens, totalTens; the reference leaves the off-diagonals at zero. */
void ora_virial(ora_sys *s, double *out) {
  int n = s->n_atoms;
  int *cv = (int *)malloc(sizeof(int) * n);
  int *cs = (int *)malloc(sizeof(int) * (s->ncell + 1));
  int *mp = (int *)malloc(sizeof(int) * n);
  cell_vectors(s, cv, cs, mp);
  double vT11 = 0.0, vT22 = 0.0, vT33 = 0.0;
  double rT11 = 0.0, rT22 = 0.0, rT33 = 0.0;
  int nv = cs[s->ncell];
  for (int ci = 0; ci < nv; ci++) {
    int cur = cv[ci];
    int cell = mp[cur];
    for (int nc = 0; nc < NB27; nc++) {
      int ncell = s->nbr[cell * NB27 + nc];
      for (int ni = cs[ncell]; ni < cs[ncell + 1]; ni++) {
        int np = cv[ni];
        if (!(cur < np && s->mol[cur] != s->mol[np]))
          continue;
        double virC[3];
        double distSq = dist_sq(s, s->x[cur], s->y[cur], s->z[cur], s->x[np],
                                s->y[np], s->z[np], virC);
        if (!(s->rcutSq > distSq))
          continue;
        int mc = s->mol[cur], mn = s->mol[np];
        double comC[3] = {min_image(s->cx[mc] - s->cx[mn], s->box[0], s->half[0]),
                          min_image(s->cy[mc] - s->cy[mn], s->box[1], s->half[1]),
                          min_image(s->cz[mc] - s->cz[mn], s->box[2], s->half[2])};
        if (s->electrostatic) {
          double qi_qj = s->q[cur] * s->q[np];
          if (qi_qj != 0.0) {
            double pRF = calc_coulomb_vir(s, distSq, qi_qj);
            rT11 += pRF * (virC[0] * comC[0]);
            rT22 += pRF * (virC[1] * comC[1]);
            rT33 += pRF * (virC[2] * comC[2]);
          }
        }
        double pVF = calc_vir(s, distSq, s->kind[cur], s->kind[np]);
        vT11 += pVF * (virC[0] * comC[0]);
        vT22 += pVF * (virC[1] * comC[1]);
        vT33 += pVF * (virC[2] * comC[2]);
      }
    }
  }
  free(cv);
  free(cs);
  free(mp);
  double wT11 = 0.0, wT22 = 0.0, wT33 = 0.0;
  if (s->ewald) {
    double constVal = 1.0 / (4.0 * s->alphaSq);
    for (int i = 0; i < s->K; i++) {
      double factor = s->prefact[i] * (s->sumRref[i] * s->sumRref[i] +
                                       s->sumIref[i] * s->sumIref[i]);
      wT11 += factor * (1.0 - 2.0 * (constVal + 1.0 / s->hsqr[i]) * s->kx[i] *
                                  s->kx[i]);
      wT22 += factor * (1.0 - 2.0 * (constVal + 1.0 / s->hsqr[i]) * s->ky[i] *
                                  s->ky[i]);
      wT33 += factor * (1.0 - 2.0 * (constVal + 1.0 / s->hsqr[i]) * s->kz[i] *
                                  s->kz[i]);
    }
    for (int m = 0; m < s->n_mol; ++m) {
      for (int atom = s->mstart[m]; atom < s->mstart[m + 1]; ++atom) {
        if (s->no_charge[atom])
          continue;
        double ac[3] = {unwrap1(s->x[atom], s->cx[m], s->box[0], s->half[0]),
                        unwrap1(s->y[atom], s->cy[m], s->box[1], s->half[1]),
                        unwrap1(s->z[atom], s->cz[m], s->box[2], s->half[2])};
        double diffC[3] = {ac[0] - s->cx[m], ac[1] - s->cy[m], ac[2] - s->cz[m]};
        double charge = s->q[atom] * 1.0;
        for (int i = 0; i < s->K; i++) {
          double arg = s->x[atom] * s->kx[i] + s->y[atom] * s->ky[i] +
                       s->z[atom] * s->kz[i];
          double factor = s->prefact[i] * 2.0 *
                          (s->sumIref[i] * cos(arg) - s->sumRref[i] * sin(arg)) *
                          charge;
          wT11 += factor * (s->kx[i] * diffC[0]);
          wT22 += factor * (s->ky[i] * diffC[1]);
          wT33 += factor * (s->kz[i] * diffC[2]);
        }
      }
    }
  }
  double inter = vT11 + vT22 + vT33;
  double real = s->electrostatic ? (rT11 + rT22 + rT33) * QQ_FACT : 0.0;
  double rt[3] = {0, 0, 0};
  if (s->electrostatic) {
    rt[0] = rT11 * QQ_FACT;
    rt[1] = rT22 * QQ_FACT;
    rt[2] = rT33 * QQ_FACT;
  }
  double recip = wT11 + wT22 + wT33;
  double vt[3] = {vT11, vT22, vT33}, wt[3] = {wT11, wT22, wT33};
  out[0] = inter;
  out[1] = real;
  out[2] = recip;
  out[3] = inter + 0.0 + real + recip + 0.0 + 0.0;
  for (int d = 0; d < 3; ++d) {
    out[4 + d] = vt[d];
    out[7 + d] = rt[d];
    out[10 + d] = wt[d];
    out[13 + d] = vt[d] + rt[d] + wt[d] + 0.0;
  }
}

void ora_box_force(ora_sys *s, const double *coords, double *aF, double *mF,
                   double *inter, double *real) {
  memset(aF, 0, sizeof(double) * 3 * s->n_atoms);
  memset(mF, 0, sizeof(double) * 3 * s->n_mol);
  if (coords) {
    int n = s->n_atoms;
    double *X = (double *)malloc(sizeof(double) * 3 * n);
    for (int i = 0; i < n; ++i) {
      X[i] = coords[3 * i];
      X[n + i] = coords[3 * i + 1];
      X[2 * n + i] = coords[3 * i + 2];
    }
    box_pairs(s, X, X + n, X + 2 * n, aF, mF, inter, real);
    free(X);
  } else {
    box_pairs(s, s->x, s->y, s->z, aF, mF, inter, real);
  }
}

/* MoleculeInter, src/CalculateEnergy.cpp:581-686; the caller's RemoveMol /
 * AddMol (src/moves/Translate.h:84,131) bracket it here. */
int ora_molecule_inter(ora_sys *s, int m, const double *newpos, double *dlj,
                       double *dreal) {
  double tempREn = 0.0, tempLJEn = 0.0;
  int overlap = 0;
  remove_mol(s, m);
  int *nb = (int *)malloc(sizeof(int) * (s->n_atoms + 1));
  int start = s->mstart[m], len = s->mstart[m + 1] - start;
  for (int p = 0; p < len; ++p) {
    int atom = start + p;
    int cell = position_to_cell(s, s->x[atom], s->y[atom], s->z[atom]);
    int nn = gather_neighbors(s, cell, nb);
    for (int i = 0; i < nn; i++) {
      int j = nb[i];
      double distSq = dist_sq(s, s->x[atom], s->y[atom], s->z[atom], s->x[j],
                              s->y[j], s->z[j], 0);
      if (s->rcutSq > distSq) {
        if (s->electrostatic) {
          double qq = s->q[atom] * s->q[j] * QQ_FACT;
          if (qq != 0.0)
            tempREn += -calc_coulomb(s, distSq, qq);
        }
        tempLJEn += -calc_en(s, distSq, s->kind[atom], s->kind[j]);
      }
    }
    const double *np = newpos + 3 * p;
    cell = position_to_cell(s, np[0], np[1], np[2]);
    nn = gather_neighbors(s, cell, nb);
    for (int i = 0; i < nn; i++) {
      int j = nb[i];
      double distSq =
          dist_sq(s, np[0], np[1], np[2], s->x[j], s->y[j], s->z[j], 0);
      if (s->rcutSq > distSq) {
        if (distSq < s->rcutLowSq)
          overlap |= 1;
        if (s->electrostatic) {
          double qq = s->q[atom] * s->q[j] * QQ_FACT;
          if (qq != 0.0)
            tempREn += calc_coulomb(s, distSq, qq);
        }
        tempLJEn += calc_en(s, distSq, s->kind[atom], s->kind[j]);
      }
    }
  }
  free(nb);
  add_mol(s, m);
  *dlj = tempLJEn;
  *dreal = tempREn;
  return overlap;
}

/* FFParticle::CalcEn / CalcCoulomb at a coupling lambda with the soft-core
 * distance (src/FFParticle.cpp:295-316, 361-387): below lambda 0.999999 the
 * pair is evaluated at r_sc^2 = cbrt(sc_alpha (1 - lambda)^sc_power
 * max(sigma^6, sc_sigma^6) + r^6) and scaled by lambda; Coulomb takes the
 * soft-core distance only when sc_coul is set. */
static double soft_rsq(const ora_sys *s, double distSq, int idx,
                       const ora_softcore *sc, double lambda) {
  double sigma6 = s->sigmaSq[idx] * s->sigmaSq[idx] * s->sigmaSq[idx];
  sigma6 = sigma6 > sc->sigma6 ? sigma6 : sc->sigma6;
  double dist6 = distSq * distSq * distSq;
  double lambdaCoef = sc->alpha * pow((1.0 - lambda), (double)sc->power);
  double softDist6 = lambdaCoef * sigma6 + dist6;
  return cbrt(softDist6);
}
static double calc_en_lambda(const ora_sys *s, double distSq, int k1, int k2,
                             const ora_softcore *sc, double lambda) {
  if (s->rcutSq < distSq)
    return 0.0;
  if (lambda >= 0.999999)
    return calc_en(s, distSq, k1, k2);
  int idx = k1 + k2 * s->n_kinds;
  double softRsq = soft_rsq(s, distSq, idx, sc, lambda);
  /* FFParticle::CalcEn(distSq, index) has no cutoff test */
  double rRat2 = s->sigmaSq[idx] / softRsq;
  double rRat4 = rRat2 * rRat2;
  double attract = rRat4 * rRat2;
  double repulse = pow(rRat2, (s->nexp[idx] * 0.5));
  return lambda * (s->eps_cn[idx] * (repulse - attract));
}
static double coulomb_plain(const ora_sys *s, double distSq, double qq) {
  double dist = sqrt(distSq);
  if (s->ewald)
    return qq * erfc(s->alpha * dist) / dist;
  return qq / dist;
}
static double calc_coulomb_lambda(const ora_sys *s, double distSq, int k1,
                                  int k2, double qq, const ora_softcore *sc,
                                  double lambda) {
  if (s->rcutCoulSq < distSq)
    return 0.0;
  if (lambda >= 0.999999)
    return coulomb_plain(s, distSq, qq);
  if (sc->coul) {
    int idx = k1 + k2 * s->n_kinds;
    return lambda * coulomb_plain(s, soft_rsq(s, distSq, idx, sc, lambda), qq);
  }
  return lambda * coulomb_plain(s, distSq, qq);
}

/* SingleMoleculeInter, src/CalculateEnergy.cpp:1494-1556: the real-space
 * energy of molecule m at its current position, with every other atom of its
 * 27-cell neighbourhood, at the old and the new lambda pair.
 * lam = {old VDW, new VDW, old Coulomb, new Coulomb};
 * out = {old inter, old real, new inter, new real}. */
void ora_single_molecule_inter(const ora_sys *s, int m, const double *lam,
                               const ora_softcore *sc, double *out) {
  double tempREnOld = 0.0, tempLJEnOld = 0.0;
  double tempREnNew = 0.0, tempLJEnNew = 0.0;
  int *nb = (int *)malloc(sizeof(int) * (s->n_atoms + 1));
  int start = s->mstart[m], len = s->mstart[m + 1] - start;
  for (int p = 0; p < len; ++p) {
    int atom = start + p;
    int cell = position_to_cell(s, s->x[atom], s->y[atom], s->z[atom]);
    int nn = gather_neighbors(s, cell, nb);
    for (int i = 0; i < nn; i++) {
      int j = nb[i];
      if (s->mol[j] == m)
        continue;
      double distSq = dist_sq(s, s->x[atom], s->y[atom], s->z[atom], s->x[j],
                              s->y[j], s->z[j], 0);
      if (!(s->rcutSq > distSq))
        continue;
      if (s->electrostatic) {
        double qq = s->q[atom] * s->q[j] * QQ_FACT;
        if (qq != 0.0) {
          tempREnNew += calc_coulomb_lambda(s, distSq, s->kind[atom],
                                            s->kind[j], qq, sc, lam[3]);
          tempREnOld += calc_coulomb_lambda(s, distSq, s->kind[atom],
                                            s->kind[j], qq, sc, lam[2]);
        }
      }
      tempLJEnNew +=
          calc_en_lambda(s, distSq, s->kind[atom], s->kind[j], sc, lam[1]);
      tempLJEnOld +=
          calc_en_lambda(s, distSq, s->kind[atom], s->kind[j], sc, lam[0]);
    }
  }
  free(nb);
  out[0] = tempLJEnOld;
  out[1] = tempREnOld;
  out[2] = tempLJEnNew;
  out[3] = tempREnNew;
}

/* ParticleInter, src/CalculateEnergy.cpp:727-785, one trial: atom `part` of
 * molecule m (its kind and charge) at position t against every atom the cell
 * list holds.  Like the reference it excludes nothing: callers that build a
 * molecule by CBMC take it out of the cell list first (ora_cell_remove_mol,
 * as MoleculeTransfer::Transform does, src/moves/MoleculeTransfer.h:100-106). */
int ora_particle_inter(const ora_sys *s, int m, int part, const double *t,
                       double *en, double *real) {
  int overlap = 0;
  int a = s->mstart[m] + part;
  int kindI = s->kind[a];
  double qI = s->q[a];
  int *nb = (int *)malloc(sizeof(int) * (s->n_atoms + 1));
  int cell = position_to_cell(s, t[0], t[1], t[2]);
  int nn = gather_neighbors(s, cell, nb);
  double tempLJ = 0.0, tempReal = 0.0;
  for (int i = 0; i < nn; i++) {
    int j = nb[i];
    double distSq = dist_sq(s, t[0], t[1], t[2], s->x[j], s->y[j], s->z[j], 0);
    if (s->rcutSq > distSq) {
      if (distSq < s->rcutLowSq)
        overlap = 1;
      tempLJ += calc_en(s, distSq, kindI, s->kind[j]);
      if (s->electrostatic) {
        double qq = s->q[j] * qI * QQ_FACT;
        if (qq != 0.0)
          tempReal += calc_coulomb(s, distSq, qq);
      }
    }
  }
  free(nb);
  *en = 0.0 + tempLJ;
  *real = 0.0 + tempReal;
  return overlap;
}

/* CellList::RemoveMol / AddMol, src/CellList.cpp:81-135 */
void ora_cell_remove_mol(ora_sys *s, int m) { remove_mol(s, m); }
void ora_cell_add_mol(ora_sys *s, int m) { add_mol(s, m); }

/* MolReciprocal, src/Ewald.cpp:409-473 (CPU branch) */
double ora_mol_reciprocal(ora_sys *s, const double *newpos, int m) {
  if (!s->ewald)
    return 0.0;
  int start = s->mstart[m], len = s->mstart[m + 1] - start;
  double energyRecipNew = 0.0;
#pragma omp parallel for num_threads(g_threads) reduction(+ : energyRecipNew)
  for (int i = 0; i < s->K; i++) {
    double sRN = 0.0, sIN = 0.0, sRO = 0.0, sIO = 0.0;
    for (int p = 0; p < len; ++p) {
      int a = start + p;
      if (s->no_charge[a])
        continue;
      double dotNew = (newpos[3 * p] * s->kx[i] + newpos[3 * p + 1] * s->ky[i] +
                       newpos[3 * p + 2] * s->kz[i]);
      double dotOld = (s->x[a] * s->kx[i] + s->y[a] * s->ky[i] +
                       s->z[a] * s->kz[i]);
      sRN += (s->q[a] * cos(dotNew));
      sIN += (s->q[a] * sin(dotNew));
      sRO += (s->q[a] * cos(dotOld));
      sIO += (s->q[a] * sin(dotOld));
    }
    s->sumRnew[i] = s->sumRref[i] + 1.0 * (sRN - sRO);
    s->sumInew[i] = s->sumIref[i] + 1.0 * (sIN - sIO);
    energyRecipNew += (s->sumRnew[i] * s->sumRnew[i] +
                       s->sumInew[i] * s->sumInew[i]) *
                      s->prefact[i];
  }
  return energyRecipNew - s->e_recip;
}

/* SwapDestRecip / SwapSourceRecip, src/Ewald.cpp:478-531, 657-710 */
static double swap_recip(ora_sys *s, const double *pos, int m, double sign) {
  if (!s->ewald)
    return 0.0;
  int start = s->mstart[m], len = s->mstart[m + 1] - start;
  double energyRecipNew = 0.0;
#pragma omp parallel for num_threads(g_threads) reduction(+ : energyRecipNew)
  for (int i = 0; i < s->K; i++) {
    double sRN = 0.0, sIN = 0.0;
    for (int p = 0; p < len; ++p) {
      if (s->no_charge[start + p])
        continue;
      double dot = (pos[3 * p] * s->kx[i] + pos[3 * p + 1] * s->ky[i] +
                    pos[3 * p + 2] * s->kz[i]);
      sRN += (s->q[start + p] * cos(dot));
      sIN += (s->q[start + p] * sin(dot));
    }
    if (sign > 0) {
      s->sumRnew[i] = s->sumRref[i] + sRN;
      s->sumInew[i] = s->sumIref[i] + sIN;
    } else {
      s->sumRnew[i] = s->sumRref[i] - sRN;
      s->sumInew[i] = s->sumIref[i] - sIN;
    }
    energyRecipNew += (s->sumRnew[i] * s->sumRnew[i] +
                       s->sumInew[i] * s->sumInew[i]) *
                      s->prefact[i];
  }
  return energyRecipNew - s->e_recip;
}
double ora_swap_dest_recip(ora_sys *s, const double *p, int m) {
  return swap_recip(s, p, m, 1.0);
}
double ora_swap_source_recip(ora_sys *s, const double *p, int m) {
  return swap_recip(s, p, m, -1.0);
}
/* UpdateRecip (pointer swap), src/Ewald.cpp:1420-1434 */
void ora_update_recip(ora_sys *s) {
  double *t = s->sumRnew;
  s->sumRnew = s->sumRref;
  s->sumRref = t;
  t = s->sumInew;
  s->sumInew = s->sumIref;
  s->sumIref = t;
}
/* CopyRecip, src/Ewald.cpp:1441-1460 */
void ora_copy_recip(ora_sys *s) {
  memcpy(s->sumRnew, s->sumRref, sizeof(double) * s->K);
  memcpy(s->sumInew, s->sumIref, sizeof(double) * s->K);
}

/* BoxForceReciprocal CPU branch, src/Ewald.cpp:1538-1595 */
void ora_box_force_recip(ora_sys *s, const double *coords, double *aR,
                         double *mR) {
  int n = s->n_atoms;
  double *X = (double *)malloc(sizeof(double) * 3 * n);
  for (int i = 0; i < n; ++i) {
    X[i] = coords ? coords[3 * i] : s->x[i];
    X[n + i] = coords ? coords[3 * i + 1] : s->y[i];
    X[2 * n + i] = coords ? coords[3 * i + 2] : s->z[i];
  }
  double *Y = X + n, *Z = X + 2 * n;
  double constValue = s->alpha * M_2_SQRTPI;
  for (int m = 0; m < s->n_mol; ++m) {
    mR[3 * m] = mR[3 * m + 1] = mR[3 * m + 2] = 0.0;
    int start = s->mstart[m], len = s->mstart[m + 1] - start;
    for (int p = start; p < start + len; p++) {
      double FX = 0.0, FY = 0.0, FZ = 0.0;
      if (!s->no_charge[p] && s->ewald) {
        for (int j = start; j < start + len; j++) {
          if (p != j) {
            double dv[3];
            double distSq = dist_sq(s, X[p], Y[p], Z[p], X[j], Y[j], Z[j], dv);
            double dist = sqrt(distSq);
            double expConstValue = exp(-1.0 * s->alphaSq * distSq);
            double qiqj = s->q[p] * s->q[j] * QQ_FACT;
            double intraForce = qiqj * 1.0 * 1.0 / distSq;
            intraForce *= ((erf(s->alpha * dist) / dist) -
                           constValue * expConstValue);
            FX -= intraForce * dv[0];
            FY -= intraForce * dv[1];
            FZ -= intraForce * dv[2];
          }
        }
        if (g_threads <= 1) {
          /* reference order: X starts from the correction term and
           * accumulates k by k */
          for (int i = 0; i < s->K; i++) {
            double dot = (X[p] * s->kx[i] + Y[p] * s->ky[i] + Z[p] * s->kz[i]);
            double factor = 2.0 * s->q[p] * s->prefact[i] * 1.0 *
                            (sin(dot) * s->sumRnew[i] - cos(dot) * s->sumInew[i]);
            FX += factor * s->kx[i];
            FY += factor * s->ky[i];
            FZ += factor * s->kz[i];
          }
        } else {
          double sx = 0.0, sy = 0.0, sz = 0.0;
#pragma omp parallel for num_threads(g_threads) reduction(+ : sx, sy, sz)
          for (int i = 0; i < s->K; i++) {
            double dot = (X[p] * s->kx[i] + Y[p] * s->ky[i] + Z[p] * s->kz[i]);
            double factor = 2.0 * s->q[p] * s->prefact[i] * 1.0 *
                            (sin(dot) * s->sumRnew[i] - cos(dot) * s->sumInew[i]);
            sx += factor * s->kx[i];
            sy += factor * s->ky[i];
            sz += factor * s->kz[i];
          }
          FX += sx;
          FY += sy;
          FZ += sz;
        }
      }
      aR[3 * p] = FX;
      aR[3 * p + 1] = FY;
      aR[3 * p + 2] = FZ;
      mR[3 * m] += FX;
      mR[3 * m + 1] += FY;
      mR[3 * m + 2] += FZ;
    }
  }
  free(X);
}

/* CalculateTorque, src/CalculateEnergy.cpp:1365-1406 */
void ora_torque(const ora_sys *s, const double *coords, const double *com,
                const double *aF, const double *aR, double *tq) {
  for (int m = 0; m < s->n_mol; ++m) {
    double tx = 0.0, ty = 0.0, tz = 0.0;
    for (int p = s->mstart[m]; p < s->mstart[m + 1]; p++) {
      double d[3];
      d[0] = min_image(coords[3 * p] - com[3 * m], s->box[0], s->half[0]);
      d[1] = min_image(coords[3 * p + 1] - com[3 * m + 1], s->box[1], s->half[1]);
      d[2] = min_image(coords[3 * p + 2] - com[3 * m + 2], s->box[2], s->half[2]);
      double f0 = aF[3 * p] + aR[3 * p];
      double f1 = aF[3 * p + 1] + aR[3 * p + 1];
      double f2 = aF[3 * p + 2] + aR[3 * p + 2];
      tx += d[1] * f2 - d[2] * f1;
      ty += d[2] * f0 - d[0] * f2;
      tz += d[0] * f1 - d[1] * f0;
    }
    tq[3 * m] = tx;
    tq[3 * m + 1] = ty;
    tq[3 * m + 2] = tz;
  }
}

/* ------------------------------------------------------------------------ */
/* System set-up and totals                                                 */
/* ------------------------------------------------------------------------ */
/* COM::CalcCOM, src/COM.h:47-68 (mutates coordinates by unwrap + wrap) */
static void calc_com(ora_sys *s) {
  for (int m = 0; m < s->n_mol; ++m) {
    int a0 = s->mstart[m], a1 = s->mstart[m + 1];
    double rx = s->x[a0], ry = s->y[a0], rz = s->z[a0];
    for (int p = a0; p < a1; ++p) {
      s->x[p] = unwrap1(s->x[p], rx, s->box[0], s->half[0]);
      s->y[p] = unwrap1(s->y[p], ry, s->box[1], s->half[1]);
      s->z[p] = unwrap1(s->z[p], rz, s->box[2], s->half[2]);
    }
    double cx = 0, cy = 0, cz = 0;
    for (int p = a0; p < a1; ++p) {
      cx += s->x[p];
      cy += s->y[p];
      cz += s->z[p];
    }
    for (int p = a0; p < a1; ++p) {
      s->x[p] = wrap1(s->x[p], s->box[0]);
      s->y[p] = wrap1(s->y[p], s->box[1]);
      s->z[p] = wrap1(s->z[p], s->box[2]);
    }
    double inv = 1.0 / (double)(a1 - a0);
    cx *= inv;
    cy *= inv;
    cz *= inv;
    s->cx[m] = wrap1(cx, s->box[0]);
    s->cy[m] = wrap1(cy, s->box[1]);
    s->cz[m] = wrap1(cz, s->box[2]);
  }
}

static void recompute(ora_sys *s) {
  double lj, re;
  box_pairs(s, s->x, s->y, s->z, NULL, NULL, &lj, &re);
  s->e_inter = lj;
  s->e_real = re;
  if (s->ewald) {
    recip_init(s);
    box_recip_sums(s, s->x, s->y, s->z);
    set_recip_ref(s);
    s->e_recip = box_recip_energy(s);
  } else {
    s->e_recip = 0.0;
  }
  double corr = 0.0;
  for (int m = 0; m < s->n_mol; ++m)
    corr += ora_mol_correction(s, m);
  s->e_corr = corr;
  s->e_self = ora_box_self(s);
}

ora_sys *ora_create(int n_atoms, int n_mol, const double *pos,
                    const int *kind, const double *charge,
                    const int *mol_start, int n_kinds, const double *eps,
                    const double *sigma, const double *nexp,
                    const double *box, double rcut, double rcut_low,
                    double rcut_coul, double tolerance, int ewald,
                    int electrostatic, double temperature) {
  ora_sys *s = (ora_sys *)calloc(1, sizeof(ora_sys));
  s->n_atoms = n_atoms;
  s->n_mol = n_mol;
  s->n_kinds = n_kinds;
  for (int d = 0; d < 3; ++d) {
    s->box[d] = box[d];
    s->half[d] = box[d] * 0.5;
  }
  s->volume = box[0] * box[1] * box[2];
  s->x = (double *)malloc(sizeof(double) * n_atoms);
  s->y = (double *)malloc(sizeof(double) * n_atoms);
  s->z = (double *)malloc(sizeof(double) * n_atoms);
  s->cx = (double *)malloc(sizeof(double) * n_mol);
  s->cy = (double *)malloc(sizeof(double) * n_mol);
  s->cz = (double *)malloc(sizeof(double) * n_mol);
  s->kind = (int *)malloc(sizeof(int) * n_atoms);
  s->mol = (int *)malloc(sizeof(int) * n_atoms);
  s->q = (double *)malloc(sizeof(double) * n_atoms);
  s->no_charge = (int *)malloc(sizeof(int) * n_atoms);
  s->list = (int *)malloc(sizeof(int) * n_atoms);
  s->mstart = (int *)malloc(sizeof(int) * (n_mol + 1));
  memcpy(s->mstart, mol_start, sizeof(int) * (n_mol + 1));
  for (int m = 0; m < n_mol; ++m)
    for (int a = mol_start[m]; a < mol_start[m + 1]; ++a)
      s->mol[a] = m;
  for (int i = 0; i < n_atoms; ++i) {
    /* Coordinates::WrapCoordinate, src/Coordinates.cpp:24-73 */
    s->x[i] = wrap1(pos[3 * i], box[0]);
    s->y[i] = wrap1(pos[3 * i + 1], box[1]);
    s->z[i] = wrap1(pos[3 * i + 2], box[2]);
    s->kind[i] = kind[i];
    s->q[i] = charge[i];
    s->no_charge[i] = fabs(charge[i]) < 0.000000001; /* Ewald.cpp:104 */
  }
  /* FFParticle::Blend, src/FFParticle.cpp:200-242 */
  int nk2 = n_kinds * n_kinds;
  s->sigmaSq = (double *)malloc(sizeof(double) * nk2);
  s->eps_cn = (double *)malloc(sizeof(double) * nk2);
  s->nexp = (double *)malloc(sizeof(double) * nk2);
  s->eps_cn_6 = (double *)malloc(sizeof(double) * nk2);
  s->nOver6 = (double *)malloc(sizeof(double) * nk2);
  for (int i = 0; i < n_kinds; ++i)
    for (int j = 0; j < n_kinds; ++j) {
      int idx = i + j * n_kinds;
      /* FFSetup::Particle::Read zeroes eps below 1e-20 and sets n = 12 */
      double ei = fabs(eps[i]) < 1.0e-20 ? 0.0 : eps[i];
      double ej = fabs(eps[j]) < 1.0e-20 ? 0.0 : eps[j];
      double ni = fabs(eps[i]) < 1.0e-20 ? 12.0 : nexp[i];
      double nj = fabs(eps[j]) < 1.0e-20 ? 12.0 : nexp[j];
      double n = (ni + nj) * 0.5;
      double cn = n / (n - 6.0) * pow(n / 6.0, (6.0 / (n - 6.0)));
      double sg = (sigma[i] + sigma[j]) * 0.5;
      s->nexp[idx] = n;
      s->sigmaSq[idx] = sg * sg;
      double e = sqrt(ei * ej);
      s->eps_cn[idx] = cn * e;
      s->eps_cn_6[idx] = s->eps_cn[idx] * 6;
      s->nOver6[idx] = n / 6;
    }
  /* Forcefield::InitBasicVals, src/Forcefield.cpp:37-83 */
  s->rcut = rcut;
  s->rcutSq = rcut * rcut;
  s->rcutLowSq = rcut_low * rcut_low;
  s->rcutCoulSq = rcut_coul * rcut_coul;
  s->alpha = sqrt(-log(tolerance)) / rcut_coul;
  s->alphaSq = s->alpha * s->alpha;
  s->recip_rcut = -2.0 * log(tolerance) / rcut_coul;
  s->recip_rcut_Sq = s->recip_rcut * s->recip_rcut;
  s->beta = 1 / temperature;
  s->ewald = ewald;
  s->electrostatic = electrostatic;
  calc_com(s);
  ora_grid_all(s);
  recompute(s);
  return s;
}

void ora_destroy(ora_sys *s) {
  if (!s)
    return;
  free(s->x); free(s->y); free(s->z); free(s->cx); free(s->cy); free(s->cz);
  free(s->kind); free(s->mol); free(s->q); free(s->no_charge); free(s->list);
  free(s->mstart); free(s->sigmaSq); free(s->eps_cn); free(s->nexp);
  free(s->eps_cn_6); free(s->nOver6); free(s->head); free(s->nbr);
  free(s->kx); free(s->ky); free(s->kz); free(s->hsqr); free(s->prefact);
  free(s->sumRnew); free(s->sumInew); free(s->sumRref); free(s->sumIref);
  free(s);
}

int ora_num_k(const ora_sys *s) { return s->K; }
int ora_num_cells(const ora_sys *s) { return s->ncell; }
void ora_get_coords(const ora_sys *s, double *o) {
  for (int i = 0; i < s->n_atoms; ++i) {
    o[3 * i] = s->x[i];
    o[3 * i + 1] = s->y[i];
    o[3 * i + 2] = s->z[i];
  }
}
void ora_get_com(const ora_sys *s, double *o) {
  for (int i = 0; i < s->n_mol; ++i) {
    o[3 * i] = s->cx[i];
    o[3 * i + 1] = s->cy[i];
    o[3 * i + 2] = s->cz[i];
  }
}
void ora_set_coords(ora_sys *s, const double *xyz, const double *com) {
  for (int i = 0; i < s->n_atoms; ++i) {
    s->x[i] = xyz[3 * i];
    s->y[i] = xyz[3 * i + 1];
    s->z[i] = xyz[3 * i + 2];
  }
  if (com)
    for (int i = 0; i < s->n_mol; ++i) {
      s->cx[i] = com[3 * i];
      s->cy[i] = com[3 * i + 1];
      s->cz[i] = com[3 * i + 2];
    }
  ora_grid_all(s);
}
void ora_get_kvec(const ora_sys *s, double *o) {
  int K = s->K;
  memcpy(o, s->kx, sizeof(double) * K);
  memcpy(o + K, s->ky, sizeof(double) * K);
  memcpy(o + 2 * K, s->kz, sizeof(double) * K);
  memcpy(o + 3 * K, s->prefact, sizeof(double) * K);
  memcpy(o + 4 * K, s->hsqr, sizeof(double) * K);
  memcpy(o + 5 * K, s->sumRref, sizeof(double) * K);
  memcpy(o + 6 * K, s->sumIref, sizeof(double) * K);
}
void ora_get_sum_new(const ora_sys *s, double *sr, double *si) {
  memcpy(sr, s->sumRnew, sizeof(double) * s->K);
  memcpy(si, s->sumInew, sizeof(double) * s->K);
}
void ora_get_cells(const ora_sys *s, int *cell_of_atom, int *edge3) {
  for (int c = 0; c < s->ncell; ++c)
    for (int p = s->head[c]; p != END_CELL; p = s->list[p])
      cell_of_atom[p] = c;
  edge3[0] = s->edge[0];
  edge3[1] = s->edge[1];
  edge3[2] = s->edge[2];
}
void ora_get_energy(const ora_sys *s, double *e) {
  e[0] = s->e_inter;
  e[1] = s->e_real;
  e[2] = s->e_recip;
  e[3] = s->e_self;
  e[4] = s->e_corr;
}
void ora_set_energy(ora_sys *s, const double *e) {
  s->e_inter = e[0];
  s->e_real = e[1];
  s->e_recip = e[2];
  s->e_self = e[3];
  s->e_corr = e[4];
}
void ora_system_total(ora_sys *s, double *o) {
  recompute(s);
  o[0] = s->e_inter;
  o[1] = s->e_real;
  o[2] = s->e_recip;
  o[3] = s->e_self;
  o[4] = s->e_corr;
  o[5] = 0.0;
  o[6] = 0.0;
  o[7] = 0.0;
  /* Energy::Total order, src/EnergyTypes.h:98-102 */
  o[8] = 0.0 + 0.0 + s->e_inter + 0.0 + s->e_real + s->e_recip + s->e_self +
         s->e_corr;
}

/* ------------------------------------------------------------------------ */
/* Random streams                                                           */
/* ------------------------------------------------------------------------ */
/* MT19937 (Matsumoto & Nishimura 1998), as seeded by MTRand(uint32)
 * (src/MersenneTwister.h:194-230, 320-363). */
#define MT_N 624
#define MT_M 397
struct ora_mt {
  uint32_t st[MT_N];
  int left;
  int next;
};
static void mt_reload(ora_mt *g) {
  uint32_t *p = g->st;
  for (int i = 0; i < MT_N; ++i) {
    uint32_t y = (p[i] & 0x80000000u) | (p[(i + 1) % MT_N] & 0x7fffffffu);
    uint32_t v = p[(i + MT_M) % MT_N] ^ (y >> 1) ^ ((p[(i + 1) % MT_N] & 1u) ? 0x9908b0dfu : 0u);
    p[i] = v;
  }
  g->left = MT_N;
  g->next = 0;
}
ora_mt *ora_mt_create(uint32_t seed) {
  ora_mt *g = (ora_mt *)calloc(1, sizeof(ora_mt));
  g->st[0] = seed;
  for (int i = 1; i < MT_N; ++i)
    g->st[i] = 1812433253u * (g->st[i - 1] ^ (g->st[i - 1] >> 30)) + (uint32_t)i;
  mt_reload(g);
  return g;
}
void ora_mt_destroy(ora_mt *g) { free(g); }
uint32_t ora_mt_u32(ora_mt *g) {
  if (g->left == 0)
    mt_reload(g);
  --g->left;
  uint32_t y = g->st[g->next++];
  y ^= (y >> 11);
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  return y ^ (y >> 18);
}
static double mt_rand(ora_mt *g) { /* [0,1] */
  return (double)ora_mt_u32(g) * (1.0 / 4294967295.0);
}
static double mt_randExc(ora_mt *g) { /* [0,1) */
  return (double)ora_mt_u32(g) * (1.0 / 4294967296.0);
}
static uint32_t mt_randInt(ora_mt *g, uint32_t n) { /* [0,n] */
  uint32_t used = n;
  used |= used >> 1;
  used |= used >> 2;
  used |= used >> 4;
  used |= used >> 8;
  used |= used >> 16;
  uint32_t i;
  do
    i = ora_mt_u32(g) & used;
  while (i > n);
  return i;
}

/* Philox4x64-10 (Salmon, Moraes, Dror, Shaw, SC'11), the generator behind
 * Random123Wrapper (src/Random123Wrapper.cpp:16-24). */
static inline void mulhilo64(uint64_t a, uint64_t b, uint64_t *hi,
                             uint64_t *lo) {
  unsigned __int128 p = (unsigned __int128)a * b;
  *hi = (uint64_t)(p >> 64);
  *lo = (uint64_t)p;
}
void ora_philox4x64(uint64_t c0, uint64_t c1, uint64_t c2, uint64_t c3,
                    uint64_t k0, uint64_t k1, uint64_t *out) {
  uint64_t c[4] = {c0, c1, c2, c3};
  uint64_t k[2] = {k0, k1};
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k[0] += 0x9E3779B97F4A7C15ULL;
      k[1] += 0xBB67AE8584CAA73BULL;
    }
    uint64_t hi0, lo0, hi1, lo1;
    mulhilo64(0xD2E7470EE14C6C93ULL, c[0], &hi0, &lo0);
    mulhilo64(0xCA5A826395121157ULL, c[2], &hi1, &lo1);
    uint64_t n0 = hi1 ^ c[1] ^ k[0];
    uint64_t n1 = lo1;
    uint64_t n2 = hi0 ^ c[3] ^ k[1];
    uint64_t n3 = lo0;
    c[0] = n0;
    c[1] = n1;
    c[2] = n2;
    c[3] = n3;
  }
  out[0] = c[0];
  out[1] = c[1];
  out[2] = c[2];
  out[3] = c[3];
}
/* r123::u01<double>(uint64) and uneg11<double>(uint64) */
double ora_u01_64(uint64_t v) {
  const double factor = 1.0 / (18446744073709551615.0 + 1.0);
  const double half = 0.5 * factor;
  return (double)v * factor + half;
}
double ora_uneg11_64(uint64_t v) {
  const double factor = 1.0 / (9223372036854775807.0 + 1.0);
  const double half = 0.5 * factor;
  return (double)(int64_t)v * factor + half;
}

/* ------------------------------------------------------------------------ */
/* Monte Carlo NVT loop                                                     */
/* ------------------------------------------------------------------------ */
struct ora_mc {
  ora_sys *s;
  ora_mt *mt;
  double movePerc[3]; /* displace, rotate, multiparticle (normalised) */
  int adj;
  double scale[2];     /* MoveSettings scale for DISPLACE, ROTATE */
  long tries[3], accepted[3], tempTries[3], tempAccepted[3];
  double mp_t_max, mp_r_max;
  long mp_tries[2], mp_acc[2], mp_itries[2], mp_iacc[2];
  int singleMoveAccepted;
  uint64_t seed;
  /* MultiParticle state */
  double *aF, *mF, *aR, *mR, *tq; /* reference forces / torque */
};

ora_mc *ora_mc_create(ora_sys *s, uint32_t seed, const double *frac,
                      int adj_steps) {
  ora_mc *mc = (ora_mc *)calloc(1, sizeof(ora_mc));
  mc->s = s;
  mc->mt = ora_mt_create(seed);
  mc->seed = seed;
  double tot = frac[0] + frac[1] + frac[2];
  for (int i = 0; i < 3; ++i)
    mc->movePerc[i] = frac[i] / tot;
  mc->adj = adj_steps;
  /* MoveSettings::Init runs before BoxDimensions::Init (src/System.cpp:72-81)
   * and reads a zero-filled axis: the initial displacement scale is 0. */
  mc->scale[0] = 0.0 * 0.25;
  mc->scale[1] = M_PI_4;
  /* multiparticle limits, src/MoveSettings.cpp:78-84 */
  mc->mp_r_max = 0.01 * M_PI;
  mc->mp_t_max = 0.02;
  mc->singleMoveAccepted = 1;
  int N = s->n_atoms, M = s->n_mol;
  mc->aF = (double *)calloc(3 * N, sizeof(double));
  mc->aR = (double *)calloc(3 * N, sizeof(double));
  mc->mF = (double *)calloc(3 * M, sizeof(double));
  mc->mR = (double *)calloc(3 * M, sizeof(double));
  mc->tq = (double *)calloc(3 * M, sizeof(double));
  return mc;
}
void ora_mc_destroy(ora_mc *mc) {
  if (!mc)
    return;
  ora_mt_destroy(mc->mt);
  free(mc->aF); free(mc->aR); free(mc->mF); free(mc->mR); free(mc->tq);
  free(mc);
}
void ora_mc_state(const ora_mc *mc, double *sc, long *cnt) {
  sc[0] = mc->scale[0];
  sc[1] = mc->scale[1];
  sc[2] = mc->mp_t_max;
  sc[3] = mc->mp_r_max;
  for (int k = 0; k < 3; ++k) {
    cnt[2 * k] = mc->tries[k];
    cnt[2 * k + 1] = mc->accepted[k];
  }
}
void ora_mc_set_scales(ora_mc *mc, const double *sc) {
  mc->scale[0] = sc[0];
  mc->scale[1] = sc[1];
  mc->mp_t_max = sc[2];
  mc->mp_r_max = sc[3];
}

static inline double bound(double v, double lo, double hi) {
  return v < lo ? lo : (v > hi ? hi : v);
}
/* MoveSettings::AdjustMoves / Adjust / AdjustMultiParticle,
 * src/MoveSettings.cpp:157-265 */
static void adjust_moves(ora_mc *mc, long step) {
  if ((step + 1) % mc->adj != 0)
    return;
  ora_sys *s = mc->s;
  double amin = s->box[0];
  if (amin > s->box[1]) amin = s->box[1];
  if (amin > s->box[2]) amin = s->box[2];
  for (int mv = 0; mv < 3; ++mv) {
    if (mv < 2) {
      if (mc->tempTries[mv] > 0) {
        double currentAccept =
            (double)mc->tempAccepted[mv] / (double)mc->tempTries[mv];
        double fract = currentAccept / 0.5;
        if (fract > 0.0)
          mc->scale[mv] *= fract;
        else
          mc->scale[mv] *= 0.5;
      }
      if (mv == 0)
        mc->scale[0] = bound(mc->scale[0], 1.0e-10, (amin * 0.5) - 1.0e-7);
      else
        mc->scale[1] = bound(mc->scale[1], 1.0e-6, M_PI - 1.0e-7);
    }
    mc->tempTries[mv] = 0;
    mc->tempAccepted[mv] = 0;
  }
  for (int t = 0; t < 2; ++t) {
    if (mc->mp_itries[t] > 0) {
      mc->mp_tries[t] += mc->mp_itries[t];
      mc->mp_acc[t] += mc->mp_iacc[t];
      double fTot = ((double)mc->mp_acc[t] / (double)mc->mp_tries[t]) / 0.3;
      double fInt = ((double)mc->mp_iacc[t] / (double)mc->mp_itries[t]) / 0.3;
      double *mx = (t == 0) ? &mc->mp_t_max : &mc->mp_r_max;
      if (fInt == 0.0) {
        *mx *= 0.5;
      } else if (fabs(fInt - 0.3) > 0.1) {
        *mx *= ((1.0 - 0.2) * fTot + 0.2 * fInt);
      }
      if (t == 0)
        *mx = bound(*mx, 0.001, (amin * 0.5) - 0.001);
      else
        *mx = bound(*mx, 0.001, M_PI - 0.001);
      mc->mp_iacc[t] = 0;
      mc->mp_itries[t] = 0;
    }
  }
}
static void update_settings(ora_mc *mc, int mv, int accepted) {
  mc->tries[mv]++;
  mc->tempTries[mv]++;
  if (accepted) {
    mc->tempAccepted[mv]++;
    mc->accepted[mv]++;
    mc->singleMoveAccepted = 1;
  }
  if (mv == 2)
    mc->singleMoveAccepted = 0;
}

/* RotationMatrix::FromAxisAngle, src/TransformMatrix.h:165-214 */
static void axis_angle(double theta, const double *u, double r[3][3]) {
  double c = cos(theta);
  double sn = sin(theta);
  double cross[3][3] = {{0.0, -(u[2]), u[1]}, {u[2], 0.0, -(u[0])},
                        {-(u[1]), (u[0]), 0.0}};
  double tens[3][3];
  for (int i = 0; i < 3; ++i) {
    tens[0][i] = u[0];
    tens[1][i] = u[1];
    tens[2][i] = u[2];
  }
  for (int i = 0; i < 3; ++i) {
    tens[i][0] *= u[0];
    tens[i][1] *= u[1];
    tens[i][2] *= u[2];
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      r[i][j] = (i == j) ? c : 0.0;
      r[i][j] += sn * cross[i][j] + (1 - c) * tens[i][j];
    }
}
/* rotate the atoms of m about centre (unwrap, rotate, wrap):
 * Coordinates::RotateRand, src/Coordinates.cpp:103-128 */
static void rotate_mol(const ora_sys *s, int m, const double *src_xyz_or_null,
                       const double *center, double r[3][3], double *out) {
  int a0 = s->mstart[m], len = s->mstart[m + 1] - a0;
  for (int p = 0; p < len; ++p) {
    int a = a0 + p;
    double v[3];
    if (src_xyz_or_null) {
      v[0] = src_xyz_or_null[3 * a];
      v[1] = src_xyz_or_null[3 * a + 1];
      v[2] = src_xyz_or_null[3 * a + 2];
    } else {
      v[0] = s->x[a];
      v[1] = s->y[a];
      v[2] = s->z[a];
    }
    for (int d = 0; d < 3; ++d)
      v[d] = unwrap1(v[d], center[d], s->box[d], s->half[d]);
    for (int d = 0; d < 3; ++d)
      v[d] += -center[d];
    double w[3];
    w[0] = r[0][0] * v[0] + r[0][1] * v[1] + r[0][2] * v[2];
    w[1] = r[1][0] * v[0] + r[1][1] * v[1] + r[1][2] * v[2];
    w[2] = r[2][0] * v[0] + r[2][1] * v[1] + r[2][2] * v[2];
    for (int d = 0; d < 3; ++d)
      out[3 * p + d] = wrap1(w[d] + center[d], s->box[d]);
  }
}

/* one MultiParticle move, src/moves/MultiParticle.h:164-544 (CPU branch) */
static void mp_move(ora_mc *mc, long step, int *o_type, int *o_acc,
                    double *de3) {
  ora_sys *s = mc->s;
  int N = s->n_atoms, M = s->n_mol;
  int allTranslate = 1;
  for (int m = 0; m < M; ++m)
    if (s->mstart[m + 1] - s->mstart[m] != 1)
      allTranslate = 0;
  /* MultiParticle::Prep draws randIntExc(MPTOTALTYPES) only when some
   * molecule has more than one atom (src/moves/MultiParticle.h:178-183) */
  int moveType = allTranslate ? 0 : (int)mt_randInt(mc->mt, 1);
  double *cur = (double *)malloc(sizeof(double) * 3 * N);
  double *com = (double *)malloc(sizeof(double) * 3 * M);
  ora_get_coords(s, cur);
  ora_get_com(s, com);
  if (mc->singleMoveAccepted) {
    ora_copy_recip(s);
    ora_box_force_recip(s, NULL, mc->aR, mc->mR);
    double lj, re;
    ora_box_force(s, NULL, mc->aF, mc->mF, &lj, &re);
    s->e_inter = lj;
    s->e_real = re;
    ora_torque(s, cur, com, mc->aF, mc->aR, mc->tq);
  }
  double *npos = (double *)malloc(sizeof(double) * 3 * N);
  double *ncom = (double *)malloc(sizeof(double) * 3 * M);
  double *tk = (double *)calloc(3 * M, sizeof(double));
  int *inRange = (int *)calloc(M, sizeof(int));
  memcpy(npos, cur, sizeof(double) * 3 * N);
  memcpy(ncom, com, sizeof(double) * 3 * M);
  const double lambda = 0.5;
  double BETA = s->beta;
  uint64_t key0 = (uint64_t)step, key1 = mc->seed;
  for (int m = 0; m < M; ++m) {
    double lb[3];
    double mx = moveType == 1 ? mc->mp_r_max : mc->mp_t_max;
    if (moveType == 1) {
      for (int d = 0; d < 3; ++d)
        lb[d] = mc->tq[3 * m + d] * lambda * BETA;
    } else {
      for (int d = 0; d < 3; ++d)
        lb[d] = (mc->mF[3 * m + d] + mc->mR[3 * m + d]) * lambda * BETA;
    }
    double lbmax[3] = {lb[0] * mx, lb[1] * mx, lb[2] * mx};
    int fir = fabs(lbmax[0]) > 1e-12 && fabs(lbmax[0]) < 30 &&
              fabs(lbmax[1]) > 1e-12 && fabs(lbmax[1]) < 30 &&
              fabs(lbmax[2]) > 1e-12 && fabs(lbmax[2]) < 30;
    inRange[m] = fir;
    uint64_t r[4];
    ora_philox4x64((uint64_t)m, 0, 0, 0, key0, key1, r);
    double val[3] = {0.0, 0.0, 0.0};
    if (fir) {
      for (int d = 0; d < 3; ++d)
        val[d] = log(exp(-1.0 * lbmax[d]) +
                     2.0 * ora_u01_64(r[d]) * sinh(lbmax[d])) /
                 lb[d];
    }
    for (int d = 0; d < 3; ++d)
      tk[3 * m + d] = val[d];
    int a0 = s->mstart[m], len = s->mstart[m + 1] - a0;
    if (moveType == 1) {
      double rm[3][3];
      if (fir) {
        double rotLen = sqrt(val[0] * val[0] + val[1] * val[1] + val[2] * val[2]);
        double ax[3] = {val[0] * (1.0 / rotLen), val[1] * (1.0 / rotLen),
                        val[2] * (1.0 / rotLen)};
        axis_angle(rotLen, ax, rm);
      } else {
        double symRand = mc->mp_r_max * ora_uneg11_64(r[0]);
        double u = ora_uneg11_64(r[1]);
        double theta = 2.0 * M_PI * ora_u01_64(r[2]);
        double rootTerm = sqrt(1.0 - u * u);
        double ax[3] = {rootTerm * cos(theta), rootTerm * sin(theta), u};
        axis_angle(symRand, ax, rm);
      }
      rotate_mol(s, m, cur, com + 3 * m, rm, npos + 3 * a0);
    } else {
      double sh[3];
      if (fir) {
        for (int d = 0; d < 3; ++d)
          sh[d] = val[d];
      } else {
        for (int d = 0; d < 3; ++d)
          sh[d] = mc->mp_t_max * ora_uneg11_64(r[d]);
      }
      for (int p = 0; p < len; ++p)
        for (int d = 0; d < 3; ++d)
          npos[3 * (a0 + p) + d] = wrap1(cur[3 * (a0 + p) + d] + sh[d], s->box[d]);
      for (int d = 0; d < 3; ++d)
        ncom[3 * m + d] = wrap1(com[3 * m + d] + sh[d], s->box[d]);
    }
  }
  /* CalcEn: grid on new positions, sums, forces, torque */
  double *save = (double *)malloc(sizeof(double) * 3 * N);
  memcpy(save, cur, sizeof(double) * 3 * N);
  ora_set_coords(s, npos, NULL); /* GridAll(newMolsPos) */
  double newRecip = ora_box_reciprocal_sums(s, NULL);
  double *aFn = (double *)malloc(sizeof(double) * 3 * N);
  double *mFn = (double *)malloc(sizeof(double) * 3 * M);
  double *aRn = (double *)malloc(sizeof(double) * 3 * N);
  double *mRn = (double *)malloc(sizeof(double) * 3 * M);
  double *tqn = (double *)malloc(sizeof(double) * 3 * M);
  double ljn, ren;
  ora_box_force(s, NULL, aFn, mFn, &ljn, &ren);
  if (!s->ewald)
    newRecip = 0.0;
  ora_box_force_recip(s, NULL, aRn, mRn);
  ora_torque(s, npos, ncom, aFn, aRn, tqn);
  /* GetCoeff, src/moves/MultiParticle.h:472-512 */
  double w = 1.0;
  double lBeta = lambda * BETA;
  for (int m = 0; m < M; ++m) {
    if (!inRange[m])
      continue;
    double lo[3], ln[3], mx;
    for (int d = 0; d < 3; ++d) {
      if (moveType == 1) {
        lo[d] = mc->tq[3 * m + d] * lBeta;
        ln[d] = tqn[3 * m + d] * lBeta;
      } else {
        lo[d] = (mc->mF[3 * m + d] + mc->mR[3 * m + d]) * lBeta;
        ln[d] = (mFn[3 * m + d] + mRn[3 * m + d]) * lBeta;
      }
    }
    mx = moveType == 1 ? mc->mp_r_max : mc->mp_t_max;
    double wr = 1.0;
    for (int d = 0; d < 3; ++d) {
      double k = tk[3 * m + d];
      wr *= ln[d] * exp(-ln[d] * k) / (2.0 * sinh(ln[d] * mx));
      wr /= lo[d] * exp(lo[d] * k) / (2.0 * sinh(lo[d] * mx));
    }
    w *= wr;
  }
  if (!isfinite(w))
    w = 0.0;
  double totNew = 0.0 + 0.0 + ljn + 0.0 + ren + newRecip + s->e_self + s->e_corr;
  double totOld = 0.0 + 0.0 + s->e_inter + 0.0 + s->e_real + s->e_recip +
                  s->e_self + s->e_corr;
  double uBoltz = exp(-BETA * (totNew - totOld));
  double accept = w * uBoltz;
  uint64_t r[4];
  ora_philox4x64((uint64_t)M, 0, 0, 0, key0, key1, r);
  double pr = ora_u01_64(r[0]);
  int result = pr < accept;
  de3[0] = ljn;
  de3[1] = ren;
  de3[2] = newRecip;
  if (result) {
    s->e_inter = ljn;
    s->e_real = ren;
    s->e_recip = newRecip;
    memcpy(mc->aF, aFn, sizeof(double) * 3 * N);
    memcpy(mc->mF, mFn, sizeof(double) * 3 * M);
    memcpy(mc->aR, aRn, sizeof(double) * 3 * N);
    memcpy(mc->mR, mRn, sizeof(double) * 3 * M);
    memcpy(mc->tq, tqn, sizeof(double) * 3 * M);
    for (int m = 0; m < M; ++m) {
      s->cx[m] = ncom[3 * m];
      s->cy[m] = ncom[3 * m + 1];
      s->cz[m] = ncom[3 * m + 2];
    }
    ora_update_recip(s);
  } else {
    ora_set_coords(s, save, NULL); /* GridAll(coordCurrRef) */
  }
  mc->mp_itries[moveType]++;
  if (result)
    mc->mp_iacc[moveType]++;
  update_settings(mc, 2, result);
  *o_type = moveType;
  *o_acc = result;
  free(cur); free(com); free(npos); free(ncom); free(tk); free(inRange);
  free(save); free(aFn); free(mFn); free(aRn); free(mRn); free(tqn);
}

void ora_mc_run(ora_mc *mc, long first, long nsteps, int *o_kind, int *o_mol,
                int *o_acc, int *o_ovl, double *o_de) {
  ora_sys *s = mc->s;
  double *np = (double *)malloc(sizeof(double) * 3 * 64);
  for (long t = 0; t < nsteps; ++t) {
    long step = first + t;
    adjust_moves(mc, step);
    /* PickArbDist, src/PRNG.h:153-163 (Wt = 1 after normalisation) */
    double sum = 0.0, prevSum = 0.0, draw = mt_rand(mc->mt) * 1.0;
    int pick;
    for (pick = 0; pick < 3 && sum < draw; ++pick) {
      prevSum = sum;
      sum += mc->movePerc[pick];
    }
    if (pick != 0)
      --pick;
    /* moves with zero frequency are never picked by the reference's full
     * table (src/MoveConst.h: DISPLACE=0, ROTATE=1, MULTIPARTICLE=2) */
    double de[3] = {0, 0, 0};
    int acc = 0, ovl = 0, mol = -1;
    if (pick == 2) {
      mp_move(mc, step, &mol, &acc, de);
    } else {
      /* PickMolAndBox with one box and one movable kind: the molecule is
       * randIntExc(count) (src/PRNG.h:239-272) */
      uint32_t m = mt_randInt(mc->mt, (uint32_t)(s->n_mol - 1));
      mol = (int)m;
      int a0 = s->mstart[m], len = s->mstart[m + 1] - a0;
      double newcom[3];
      if (pick == 0) {
        /* TranslateRand, src/Coordinates.cpp:83-100 */
        double bound2 = 2.0 * mc->scale[0];
        double sh[3];
        sh[0] = mt_rand(mc->mt) * bound2 - mc->scale[0];
        sh[1] = mt_rand(mc->mt) * bound2 - mc->scale[0];
        sh[2] = mt_rand(mc->mt) * bound2 - mc->scale[0];
        for (int p = 0; p < len; ++p) {
          np[3 * p] = wrap1(s->x[a0 + p] + sh[0], s->box[0]);
          np[3 * p + 1] = wrap1(s->y[a0 + p] + sh[1], s->box[1]);
          np[3 * p + 2] = wrap1(s->z[a0 + p] + sh[2], s->box[2]);
        }
        newcom[0] = wrap1(s->cx[m] + sh[0], s->box[0]);
        newcom[1] = wrap1(s->cy[m] + sh[1], s->box[1]);
        newcom[2] = wrap1(s->cz[m] + sh[2], s->box[2]);
      } else {
        /* RotateRand, src/Coordinates.cpp:103-128 */
        double theta = mt_rand(mc->mt) * (2.0 * mc->scale[1]) - mc->scale[1];
        double u = mt_rand(mc->mt) * (2.0 * 1.0) - 1.0;
        double phi = mt_randExc(mc->mt) * (2.0 * M_PI);
        double rootTerm = sqrt(1.0 - u * u);
        double ax[3] = {rootTerm * cos(phi), rootTerm * sin(phi), u};
        double rm[3][3];
        axis_angle(theta, ax, rm);
        double c[3] = {s->cx[m], s->cy[m], s->cz[m]};
        rotate_mol(s, m, NULL, c, rm, np);
        newcom[0] = s->cx[m];
        newcom[1] = s->cy[m];
        newcom[2] = s->cz[m];
      }
      double dlj, dre, drc = 0.0;
      ovl = ora_molecule_inter(s, (int)m, np, &dlj, &dre);
      if (!ovl)
        drc = ora_mol_reciprocal(s, np, (int)m);
      /* Translate::Accept, src/moves/Translate.h:97-138 */
      double pr = mt_rand(mc->mt);
      int res = pr < exp(-s->beta * (dlj + dre + drc));
      acc = res && !ovl;
      if (acc) {
        s->e_inter += dlj;
        s->e_real += dre;
        s->e_recip += drc;
        remove_mol(s, (int)m);
        for (int p = 0; p < len; ++p) {
          s->x[a0 + p] = np[3 * p];
          s->y[a0 + p] = np[3 * p + 1];
          s->z[a0 + p] = np[3 * p + 2];
        }
        s->cx[m] = newcom[0];
        s->cy[m] = newcom[1];
        s->cz[m] = newcom[2];
        ora_update_recip(s);
        add_mol(s, (int)m);
      } else {
        /* RemoveMol at CalcEn, AddMol at Accept: the molecule goes back to
         * the head of its cells' lists */
        remove_mol(s, (int)m);
        add_mol(s, (int)m);
      }
      de[0] = dlj;
      de[1] = dre;
      de[2] = drc;
      update_settings(mc, pick, acc);
    }
    if (o_kind) o_kind[t] = pick;
    if (o_mol) o_mol[t] = mol;
    if (o_acc) o_acc[t] = acc;
    if (o_ovl) o_ovl[t] = ovl;
    if (o_de) {
      o_de[3 * t] = de[0];
      o_de[3 * t + 1] = de[1];
      o_de[3 * t + 2] = de[2];
    }
  }
  free(np);
}

/* ======================================================================== */
/* Gibbs ensemble, NVT (GEMC): two boxes of single-site LJ particles with    */
/* displacement, molecule-transfer (CBMC) and volume-exchange moves.         */
/* Restates System::PickMove / RunMove (src/System.cpp:262-302) with         */
/* Translate (src/moves/Translate.h:52-138), MoleculeTransfer                */
/* (src/moves/MoleculeTransfer.h:71-245) building through DCLinear /         */
/* DCSingle (src/cbmc/DCLinear.cpp:44-55, src/cbmc/DCSingle.cpp:23-90),      */
/* VolumeTransfer (src/moves/VolumeTransfer.h:71-318), the PRNG picks        */
/* (src/PRNG.h:48-470), BoxDimensions::ExchangeVolume / SetVolume            */
/* (src/BoxDimensions.cpp:124-227), Coordinates::TranslateRand /             */
/* TranslateOneBox (src/Coordinates.cpp:83-180), MoleculeLookup::Shift       */
/* (src/MoleculeLookup.cpp:165-200) and MoveSettings (src/MoveSettings.cpp:  */
/* 19-265).  Pair sums run over each box's particles in lookup order (the    */
/* reference sums in cell-list order: the same pairs, another rounding).     */
/* ======================================================================== */
#define G_KINDS 14
#define G_DISPLACE 0
#define G_ROTATE 1
#define G_MOL_TRANSFER 10
#define G_VOL_TRANSFER 13
#define G_TARGET 0.5    /* MoveSettings::TARGET_ACCEPT_FRACT */
#define G_TINY 1.0e-7   /* MoveSettings::TINY_AMOUNT */
#define G_SMALL_WEIGHT 1.0e-38

struct ora_gemc {
  int n;
  double ax[2][3], half[2][3], vol[2], volInv[2], minVol[2];
  double *x, *y, *z, *cx, *cy, *cz;
  int *lookup, start1; /* box 0: lookup[0, start1), box 1: [start1, n) */
  double e[2];         /* running inter energies */
  double sigmaSq, eps_cn, nexp, rcut, rcutSq, rcutLowSq, beta;
  int ntrials;
  double perc[G_KINDS];
  double scale[2][G_KINDS];
  long tries[2][G_KINDS], acc[2][G_KINDS], ttries[2][G_KINDS],
      tacc[2][G_KINDS];
  int adj;
  int err; /* 1: a volume change would shrink a box below 2 Rcut */
  ora_mt *mt;
};

static inline int g_first(const ora_gemc *g, int b) {
  return b == 0 ? 0 : g->start1;
}
static inline int g_count(const ora_gemc *g, int b) {
  return b == 0 ? g->start1 : g->n - g->start1;
}
static inline double g_min_image(double raw, double ax, double half) {
  if (raw > half)
    raw -= ax;
  else if (raw < -half)
    raw += ax;
  return raw;
}
static inline double g_dist_sq(const double ax[3], const double half[3],
                               double x1, double y1, double z1, double x2,
                               double y2, double z2) {
  double dx = g_min_image(x1 - x2, ax[0], half[0]);
  double dy = g_min_image(y1 - y2, ax[1], half[1]);
  double dz = g_min_image(z1 - z2, ax[2], half[2]);
  return dx * dx + dy * dy + dz * dz;
}
/* FFParticle::CalcEn (src/FFParticle.cpp:295-325), lambda = 1 */
static inline double g_calc_en(const ora_gemc *g, double distSq) {
  if (g->rcutSq < distSq)
    return 0.0;
  double rRat2 = g->sigmaSq / distSq;
  double rRat4 = rRat2 * rRat2;
  double attract = rRat4 * rRat2;
  double repulse = pow(rRat2, (g->nexp * 0.5));
  return (g->eps_cn * (repulse - attract));
}
/* LJ energy of a particle at (px, py, pz) in box b against the box's
 * particles other than `skip` (CalculateEnergy::ParticleInter /
 * MoleculeInter's sums, src/CalculateEnergy.cpp:581-785); *ovl set when a
 * pair is closer than RcutLow */
static void g_accum(const ora_gemc *g, int b, double px, double py,
                    double pz, int skip, double sign, double *acc, int *ovl) {
  int a0 = g_first(g, b), n = g_count(g, b);
  for (int i = 0; i < n; ++i) {
    int j = g->lookup[a0 + i];
    if (j == skip)
      continue;
    double d2 = g_dist_sq(g->ax[b], g->half[b], px, py, pz, g->x[j], g->y[j],
                          g->z[j]);
    if (d2 < g->rcutSq) {
      if (ovl && d2 < g->rcutLowSq)
        *ovl = 1;
      *acc += sign * g_calc_en(g, d2);
    }
  }
}
static double g_particle(const ora_gemc *g, int b, double px, double py,
                         double pz, int skip, int *ovl) {
  double e = 0.0;
  g_accum(g, b, px, py, pz, skip, 1.0, &e, ovl);
  return e;
}
/* CalculateEnergy::BoxInter (src/CalculateEnergy.cpp:157-266) of box b for
 * coordinates X, Y, Z at edges ax / half */
static double g_box_inter(const ora_gemc *g, int b, const double *X,
                          const double *Y, const double *Z,
                          const double ax[3], const double half[3]) {
  double e = 0.0;
  int a0 = g_first(g, b), n = g_count(g, b);
  for (int i = 0; i < n; ++i) {
    int p = g->lookup[a0 + i];
    for (int k = i + 1; k < n; ++k) {
      int q = g->lookup[a0 + k];
      double d2 = g_dist_sq(ax, half, X[p], Y[p], Z[p], X[q], Y[q], Z[q]);
      if (d2 < g->rcutSq)
        e += g_calc_en(g, d2);
    }
  }
  return e;
}
static inline double g_wrap(double v, double ax) {
  if (v >= ax)
    v -= ax;
  else if (v < 0)
    v += ax;
  return v;
}
static inline double g_unwrap(double v, double ref, double ax, double half) {
  if (fabs(ref - v) > half) {
    if (ref < half)
      v -= ax;
    else
      v += ax;
  }
  return v;
}

ora_gemc *ora_gemc_create(int n0, const double *pos0, int n1,
                          const double *pos1, const double *L0,
                          const double *L1, double eps, double sigma,
                          double nmie, double temperature, double rcut,
                          double rcut_low, uint32_t seed,
                          const double *frac3, int adj_steps, int ntrials) {
  ora_gemc *g = (ora_gemc *)calloc(1, sizeof(ora_gemc));
  int n = n0 + n1;
  g->n = n;
  g->x = (double *)malloc(sizeof(double) * n);
  g->y = (double *)malloc(sizeof(double) * n);
  g->z = (double *)malloc(sizeof(double) * n);
  g->cx = (double *)malloc(sizeof(double) * n);
  g->cy = (double *)malloc(sizeof(double) * n);
  g->cz = (double *)malloc(sizeof(double) * n);
  g->lookup = (int *)malloc(sizeof(int) * n);
  g->start1 = n0;
  for (int d = 0; d < 3; ++d) {
    g->ax[0][d] = L0[d];
    g->ax[1][d] = L1[d];
    g->half[0][d] = L0[d] * 0.5;
    g->half[1][d] = L1[d] * 0.5;
  }
  for (int b = 0; b < 2; ++b) {
    g->vol[b] = g->ax[b][0] * g->ax[b][1] * g->ax[b][2];
    g->volInv[b] = 1.0 / g->vol[b];
    /* BoxDimensions::Init (src/BoxDimensions.cpp:19) */
    g->minVol[b] = 8.0 * (rcut * rcut) * rcut + 0.001;
  }
  /* molecules of box 0 then box 1, as the two PDBs are read; coordinates
   * wrapped (Coordinates::WrapCoordinate) and centres from COM::CalcCOM
   * (one atom: the wrapped position) */
  for (int i = 0; i < n; ++i) {
    const double *p = i < n0 ? pos0 + 3 * i : pos1 + 3 * (i - n0);
    int b = i < n0 ? 0 : 1;
    g->x[i] = g_wrap(p[0], g->ax[b][0]);
    g->y[i] = g_wrap(p[1], g->ax[b][1]);
    g->z[i] = g_wrap(p[2], g->ax[b][2]);
    g->cx[i] = g_wrap(g->x[i] * (1.0 / 1.0), g->ax[b][0]);
    g->cy[i] = g_wrap(g->y[i] * (1.0 / 1.0), g->ax[b][1]);
    g->cz[i] = g_wrap(g->z[i] * (1.0 / 1.0), g->ax[b][2]);
    g->lookup[i] = i;
  }
  /* FFParticle::Blend for one kind (src/FFParticle.cpp:200-242) */
  double cn = nmie / (nmie - 6.0) * pow(nmie / 6.0, (6.0 / (nmie - 6.0)));
  g->nexp = nmie;
  g->sigmaSq = sigma * sigma;
  g->eps_cn = cn * sqrt(eps * eps);
  g->rcut = rcut;
  g->rcutSq = rcut * rcut;
  g->rcutLowSq = rcut_low * rcut_low;
  g->beta = 1 / temperature;
  g->ntrials = ntrials;
  /* StaticVals::InitMovePercents (src/StaticVals.cpp:35-94) */
  double raw[G_KINDS] = {0};
  raw[G_DISPLACE] = frac3[0];
  raw[G_VOL_TRANSFER] = frac3[1];
  raw[G_MOL_TRANSFER] = frac3[2];
  double tot = 0.0;
  for (int m = 0; m < G_KINDS; ++m)
    tot += raw[m];
  for (int m = 0; m < G_KINDS; ++m)
    g->perc[m] = raw[m] / tot;
  /* MoveSettings::Init (src/MoveSettings.cpp:19-90) runs before
   * BoxDimensions::Init (src/System.cpp:72-81) and reads a zero-filled axis:
   * the initial displacement scale is 0 */
  for (int b = 0; b < 2; ++b) {
    g->scale[b][G_DISPLACE] = 0.0 * 0.25;
    g->scale[b][G_ROTATE] = M_PI_4;
    g->scale[b][G_VOL_TRANSFER] = 500;
  }
  g->adj = adj_steps;
  g->mt = ora_mt_create(seed);
  for (int b = 0; b < 2; ++b)
    g->e[b] = g_box_inter(g, b, g->x, g->y, g->z, g->ax[b], g->half[b]);
  return g;
}

void ora_gemc_destroy(ora_gemc *g) {
  if (!g)
    return;
  free(g->x); free(g->y); free(g->z);
  free(g->cx); free(g->cy); free(g->cz);
  free(g->lookup);
  ora_mt_destroy(g->mt);
  free(g);
}

/* MoveSettings::Update (src/MoveSettings.cpp:94-137), one kind */
static void g_update(ora_gemc *g, int move, int accepted, int b) {
  g->tries[b][move]++;
  g->ttries[b][move]++;
  if (accepted) {
    g->tacc[b][move]++;
    g->acc[b][move]++;
  }
}
/* MoveSettings::AdjustMoves / Adjust (src/MoveSettings.cpp:147-238) */
static void g_adjust(ora_gemc *g, long step) {
  if ((step + 1) % g->adj != 0)
    return;
  for (int b = 0; b < 2; ++b)
    for (int m = 0; m < G_KINDS; ++m) {
      if (m == G_DISPLACE || m == G_ROTATE || m == G_VOL_TRANSFER) {
        if (g->ttries[b][m] > 0) {
          double currentAccept =
              (double)(g->tacc[b][m]) / (double)(g->ttries[b][m]);
          double fractOfTargetAccept = currentAccept / G_TARGET;
          if (fractOfTargetAccept > 0.0)
            g->scale[b][m] *= fractOfTargetAccept;
          else
            g->scale[b][m] *= 0.5;
        }
        double lo, hi;
        if (m == G_DISPLACE) {
          double mn = g->ax[b][0];
          if (mn > g->ax[b][1])
            mn = g->ax[b][1];
          if (mn > g->ax[b][2])
            mn = g->ax[b][2];
          lo = 1.0e-10;
          hi = (mn * 0.5) - G_TINY;
        } else if (m == G_ROTATE) {
          lo = 1.0e-6;
          hi = M_PI - G_TINY;
        } else {
          double maxVolExchange = g->vol[b] - g->minVol[b];
          lo = 0.001;
          hi = 0.34 * maxVolExchange;
        }
        if (g->scale[b][m] < lo)
          g->scale[b][m] = lo;
        if (g->scale[b][m] > hi)
          g->scale[b][m] = hi;
      }
      g->tacc[b][m] = 0;
      g->ttries[b][m] = 0;
    }
}
/* PRNG::PickBox with the sub-draw remainder (src/PRNG.h:215-230) */
static int g_pick_box(double *subDraw, double *boxDiv, double movPerc) {
  *boxDiv = movPerc / 2;
  int b = (int)(unsigned)(*subDraw / *boxDiv);
  if (b >= 2)
    b--;
  *subDraw -= b * *boxDiv;
  return b;
}
/* PRNG::PickMol / PickMol2 with one molecule kind (src/PRNG.h:267-300,
 * 336-365): -1 when the box is empty */
static int g_pick_mol(ora_gemc *g, int b) {
  int nb = g_count(g, b);
  if (nb == 0)
    return -1;
  uint32_t off = mt_randInt(g->mt, (uint32_t)nb - 1u);
  return g->lookup[g_first(g, b) + off];
}
/* MoleculeLookup::Shift (src/MoleculeLookup.cpp:178-200), one kind */
static void g_shift(ora_gemc *g, int m, int from) {
  int a0 = g_first(g, from), n = g_count(g, from), idx = -1;
  for (int i = 0; i < n; ++i)
    if (g->lookup[a0 + i] == m) {
      idx = a0 + i;
      break;
    }
  int t;
  if (from == 0) { /* into box 1: the boundary moves down */
    int ni = --g->start1;
    t = g->lookup[idx];
    g->lookup[idx] = g->lookup[ni];
    g->lookup[ni] = t;
  } else { /* into box 0: the boundary moves up */
    int ni = g->start1++;
    t = g->lookup[idx];
    g->lookup[idx] = g->lookup[ni];
    g->lookup[ni] = t;
  }
}

static void g_displace(ora_gemc *g, double subDraw, double movPerc, int *o_b,
                       int *o_m, int *o_acc, double *o_d) {
  double boxDiv;
  int b = g_pick_box(&subDraw, &boxDiv, movPerc);
  /* PickMol: kind chunk from subDraw (one kind) */
  int m = g_pick_mol(g, b);
  *o_b = b;
  *o_m = m;
  if (m < 0) {
    g_update(g, G_DISPLACE, 0, b);
    return;
  }
  /* Coordinates::TranslateRand, PRNG::SymXYZ */
  double bound = g->scale[b][G_DISPLACE], bound2 = 2.0 * bound;
  double sx = mt_rand(g->mt) * bound2 - bound;
  double sy = mt_rand(g->mt) * bound2 - bound;
  double sz = mt_rand(g->mt) * bound2 - bound;
  double nx = g_wrap(g->x[m] + sx, g->ax[b][0]);
  double ny = g_wrap(g->y[m] + sy, g->ax[b][1]);
  double nz = g_wrap(g->z[m] + sz, g->ax[b][2]);
  double ncx = g_wrap(g->cx[m] + sx, g->ax[b][0]);
  double ncy = g_wrap(g->cy[m] + sy, g->ax[b][1]);
  double ncz = g_wrap(g->cz[m] + sz, g->ax[b][2]);
  /* MoleculeInter: old pairs subtracted, new pairs added */
  int ovl = 0;
  double tempLJ = 0.0;
  g_accum(g, b, g->x[m], g->y[m], g->z[m], m, -1.0, &tempLJ, NULL);
  g_accum(g, b, nx, ny, nz, m, 1.0, &tempLJ, &ovl);
  double pr = mt_rand(g->mt);
  int res = pr < exp(-g->beta * (tempLJ + 0.0 + 0.0));
  int result = res && !ovl;
  if (result) {
    g->e[b] += tempLJ;
    g->x[m] = nx; g->y[m] = ny; g->z[m] = nz;
    g->cx[m] = ncx; g->cy[m] = ncy; g->cz[m] = ncz;
  }
  g_update(g, G_DISPLACE, result, b);
  *o_acc = result;
  o_d[0] = tempLJ;
  o_d[1] = ovl;
}

/* PRNG::PickWeighted (src/PRNG.h:167-200) */
static int g_pick_weighted(ora_gemc *g, const double *w, int n, double tot,
                           int *err) {
  double draw = mt_rand(g->mt) * tot;
  double sum = 0.0;
  for (int i = 0; i < n; ++i) {
    sum += w[i];
    if (sum >= draw)
      return i;
  }
  int lastZero = n;
  for (int i = n - 1; i > 0 && w[i] == 0.0; --i)
    lastZero = i;
  lastZero--;
  if (fabs(draw - tot) < 0.001)
    return lastZero;
  *err = 2;
  return 0;
}

static void g_transfer(ora_gemc *g, double subDraw, double movPerc, int *o_b,
                       int *o_m, int *o_acc, double *o_d) {
  double boxDiv;
  int src = g_pick_box(&subDraw, &boxDiv, movPerc);
  int dest = src == 0 ? 1 : 0;
  int m = g_pick_mol(g, src);
  *o_b = src;
  *o_m = m;
  if (m < 0) {
    g_update(g, G_MOL_TRANSFER, 0, dest);
    return;
  }
  const int nt = g->ntrials;
  double tx[64], ty[64], tz[64], en[64], w[64];
  int ov[64];
  /* DCLinear::Build: direction draw, then BuildNew and BuildOld */
  (void)mt_randInt(g->mt, 1);
  /* DCSingle::BuildNew in the destination box */
  for (int t = 0; t < nt; ++t) {
    tx[t] = mt_randExc(g->mt) * g->ax[dest][0];
    ty[t] = mt_randExc(g->mt) * g->ax[dest][1];
    tz[t] = mt_randExc(g->mt) * g->ax[dest][2];
  }
  double stepWeight = 0;
  for (int t = 0; t < nt; ++t) {
    ov[t] = 0;
    en[t] = 0.0 + g_particle(g, dest, tx[t], ty[t], tz[t], m, &ov[t]);
    w[t] = exp(-1 * g->beta * (en[t] + 0.0));
    stepWeight += w[t];
  }
  int winner = g_pick_weighted(g, w, nt, stepWeight, &g->err);
  int overlap = ov[winner];
  double Wn = 1.0 * (stepWeight / nt);
  double e_new = en[winner];
  double nx = tx[winner], ny = ty[winner], nz = tz[winner];
  /* DCSingle::BuildOld in the source box, trial 0 at the particle */
  for (int t = 0; t < nt; ++t) {
    tx[t] = mt_randExc(g->mt) * g->ax[src][0];
    ty[t] = mt_randExc(g->mt) * g->ax[src][1];
    tz[t] = mt_randExc(g->mt) * g->ax[src][2];
  }
  tx[0] = g_wrap(g->x[m], g->ax[src][0]);
  ty[0] = g_wrap(g->y[m], g->ax[src][1]);
  tz[0] = g_wrap(g->z[m], g->ax[src][2]);
  double stepWeightOld = 0;
  for (int t = 0; t < nt; ++t) {
    ov[t] = 0;
    en[t] = 0.0 + g_particle(g, src, tx[t], ty[t], tz[t], m, &ov[t]);
    stepWeightOld += exp(-1 * g->beta * (en[t] + 0.0));
  }
  double Wo = 1.0 * (stepWeightOld / nt);
  double e_old = en[0];
  /* MoleculeTransfer::GetCoeff / Accept (GEMC) */
  int nsrc = g_count(g, src), ndest = g_count(g, dest);
  double coeff = (double)(nsrc) / (double)(ndest + 1) * g->vol[dest] *
                 g->volInv[src];
  double Wrat = Wn / Wo * 1.0 * 1.0;
  int result = 0;
  if (Wn > G_SMALL_WEIGHT && !overlap)
    result = mt_rand(g->mt) < coeff * Wrat;
  if (result) {
    g->e[src] -= e_old;
    g->e[dest] += e_new;
    g->x[m] = nx; g->y[m] = ny; g->z[m] = nz;
    /* COM::SetNew of one atom: its wrapped position */
    g->cx[m] = g_wrap(nx * (1.0 / 1.0), g->ax[dest][0]);
    g->cy[m] = g_wrap(ny * (1.0 / 1.0), g->ax[dest][1]);
    g->cz[m] = g_wrap(nz * (1.0 / 1.0), g->ax[dest][2]);
    g_shift(g, m, src);
    if (g_count(g, src) == 0 || g_count(g, src) == 1)
      g->e[src] = 0.0;
  }
  g_update(g, G_MOL_TRANSFER, result, dest);
  *o_acc = result;
  o_d[0] = Wn;
  o_d[1] = Wo;
  o_d[2] = e_new;
  o_d[3] = e_old;
}

/* BoxDimensions::SetVolume, cubic scaling (src/BoxDimensions.cpp:215-227) */
static void g_set_volume(double ax[3], double half[3], double *vol,
                         double *volInv, double v) {
  double ratio = cbrt(v / *vol);
  for (int d = 0; d < 3; ++d) {
    ax[d] *= ratio;
    half[d] *= ratio;
  }
  *vol = v;
  *volInv = 1.0 / v;
}

static void g_volume(ora_gemc *g, double subDraw, double movPerc, int *o_b,
                     int *o_acc, double *o_d) {
  double boxDiv = movPerc / 2;
  int b0 = (int)(unsigned)(subDraw / boxDiv);
  if (b0 >= 2)
    b0--;
  int b1 = b0 == 0 ? 1 : 0;
  *o_b = b0;
  int bp[2] = {b0, b1};
  double max = g->scale[b0][G_VOL_TRANSFER];
  if (g->scale[b1][G_VOL_TRANSFER] < max)
    max = g->scale[b1][G_VOL_TRANSFER];
  double transfer = mt_rand(g->mt) * (2.0 * max) - max;
  /* BoxDimensions::ExchangeVolume */
  double nax[2][3], nhalf[2][3], nvol[2], nvolInv[2], sc[2][3];
  for (int b = 0; b < 2; ++b) {
    for (int d = 0; d < 3; ++d) {
      nax[b][d] = g->ax[b][d];
      nhalf[b][d] = g->half[b][d];
    }
    nvol[b] = g->vol[b];
    nvolInv[b] = g->volInv[b];
  }
  double vTot = (g->vol[bp[0]] + g->vol[bp[1]]);
  g_set_volume(nax[bp[0]], nhalf[bp[0]], &nvol[bp[0]], &nvolInv[bp[0]],
               g->vol[bp[0]] + transfer);
  g_set_volume(nax[bp[1]], nhalf[bp[1]], &nvol[bp[1]], &nvolInv[bp[1]],
               vTot - nvol[bp[0]]);
  for (int i = 0; i < 2; ++i) {
    int b = bp[i];
    for (int d = 0; d < 3; ++d)
      sc[b][d] = nax[b][d] / g->ax[b][d];
    if (nhalf[b][0] < g->rcut || nhalf[b][1] < g->rcut ||
        nhalf[b][2] < g->rcut || nvol[b] < g->minVol[b]) {
      g->err = 1; /* the reference exits here */
      return;
    }
  }
  /* Coordinates::TranslateOneBox for both boxes */
  int n = g->n;
  double *X = (double *)malloc(sizeof(double) * 6 * n);
  double *Y = X + n, *Z = X + 2 * n, *CX = X + 3 * n, *CY = X + 4 * n,
         *CZ = X + 5 * n;
  for (int i = 0; i < n; ++i) {
    X[i] = g->x[i]; Y[i] = g->y[i]; Z[i] = g->z[i];
    CX[i] = g->cx[i]; CY[i] = g->cy[i]; CZ[i] = g->cz[i];
  }
  for (int b = 0; b < 2; ++b) {
    int a0 = g_first(g, b), nb = g_count(g, b);
    for (int i = 0; i < nb; ++i) {
      int m = g->lookup[a0 + i];
      double ux = CX[m] * sc[b][0], uy = CY[m] * sc[b][1],
             uz = CZ[m] * sc[b][2];
      CX[m] = ux; CY[m] = uy; CZ[m] = uz;
      double shx = CX[m] - g->cx[m], shy = CY[m] - g->cy[m],
             shz = CZ[m] - g->cz[m];
      double px = g_unwrap(X[m], g->cx[m], g->ax[b][0], g->half[b][0]);
      double py = g_unwrap(Y[m], g->cy[m], g->ax[b][1], g->half[b][1]);
      double pz = g_unwrap(Z[m], g->cz[m], g->ax[b][2], g->half[b][2]);
      X[m] = g_wrap(px + shx, nax[b][0]);
      Y[m] = g_wrap(py + shy, nax[b][1]);
      Z[m] = g_wrap(pz + shz, nax[b][2]);
    }
  }
  /* VolumeTransfer::CalcEn: BoxInter of both boxes at the new axes */
  double en[2];
  en[0] = g->e[0];
  en[1] = g->e[1];
  for (int i = 0; i < 2; ++i) {
    int b = bp[i];
    en[b] = g_box_inter(g, b, X, Y, Z, nax[b], nhalf[b]);
  }
  /* VolumeTransfer::GetCoeff / Accept */
  double coeff = 1.0;
  for (int i = 0; i < 2; ++i) {
    int b = bp[i];
    coeff *= pow(nvol[b] / g->vol[b], (double)g_count(g, b));
  }
  double tNew = (0.0 + en[0]) + en[1];
  double tRef = (0.0 + g->e[0]) + g->e[1];
  double uBoltz = exp(-g->beta * (tNew - tRef));
  double accept = coeff * uBoltz;
  int result = mt_rand(g->mt) < accept;
  if (result) {
    g->e[0] = en[0];
    g->e[1] = en[1];
    for (int i = 0; i < n; ++i) {
      g->x[i] = X[i]; g->y[i] = Y[i]; g->z[i] = Z[i];
      g->cx[i] = CX[i]; g->cy[i] = CY[i]; g->cz[i] = CZ[i];
    }
    for (int b = 0; b < 2; ++b) {
      for (int d = 0; d < 3; ++d) {
        g->ax[b][d] = nax[b][d];
        g->half[b][d] = nhalf[b][d];
      }
      g->vol[b] = nvol[b];
      g->volInv[b] = nvolInv[b];
    }
  }
  free(X);
  g_update(g, G_VOL_TRANSFER, result, bp[0]);
  g_update(g, G_VOL_TRANSFER, result, bp[1]);
  *o_acc = result;
  o_d[0] = en[0];
  o_d[1] = en[1];
}

/* Run steps [first, first + nsteps).  Per step: kind, box, molecule,
 * accepted, and four move values (as the reference probe's trace). */
int ora_gemc_run(ora_gemc *g, long first, long nsteps, int *o_kind, int *o_box,
                 int *o_mol, int *o_acc, double *o_d4, double *o_state5) {
  for (long t = 0; t < nsteps; ++t) {
    long step = first + t;
    g_adjust(g, step);
    /* System::PickMove: PRNG::PickArbDist over the GEMC move kinds */
    double sum = 0.0, prevSum = 0.0, draw = mt_rand(g->mt) * 1.0;
    int pick;
    for (pick = 0; pick < G_KINDS && sum < draw; ++pick) {
      prevSum = sum;
      sum += g->perc[pick];
    }
    if (pick != 0)
      --pick;
    double subDraw = draw - prevSum;
    int b = -1, m = -1, acc = 0;
    double d[4] = {0, 0, 0, 0};
    if (pick == G_DISPLACE)
      g_displace(g, subDraw, g->perc[pick], &b, &m, &acc, d);
    else if (pick == G_MOL_TRANSFER)
      g_transfer(g, subDraw, g->perc[pick], &b, &m, &acc, d);
    else if (pick == G_VOL_TRANSFER)
      g_volume(g, subDraw, g->perc[pick], &b, &acc, d);
    if (g->err)
      return g->err;
    if (o_kind) o_kind[t] = pick;
    if (o_box) o_box[t] = b;
    if (o_mol) o_mol[t] = m;
    if (o_acc) o_acc[t] = acc;
    if (o_d4)
      for (int k = 0; k < 4; ++k)
        o_d4[4 * t + k] = d[k];
    if (o_state5) {
      o_state5[5 * t] = g->e[0];
      o_state5[5 * t + 1] = g->e[1];
      o_state5[5 * t + 2] = g->vol[0];
      o_state5[5 * t + 3] = g->vol[1];
      o_state5[5 * t + 4] = g->start1;
    }
  }
  return 0;
}

/* coordinates [n * 3], centres [n * 3], lookup [n], molecules in box 0,
 * running energies [2], axes [2 * 3] */
void ora_gemc_get(const ora_gemc *g, double *xyz, double *com, int *lookup,
                  int *n0, double *e2, double *axes6) {
  for (int i = 0; i < g->n; ++i) {
    if (xyz) {
      xyz[3 * i] = g->x[i]; xyz[3 * i + 1] = g->y[i]; xyz[3 * i + 2] = g->z[i];
    }
    if (com) {
      com[3 * i] = g->cx[i]; com[3 * i + 1] = g->cy[i];
      com[3 * i + 2] = g->cz[i];
    }
    if (lookup)
      lookup[i] = g->lookup[i];
  }
  if (n0)
    *n0 = g->start1;
  if (e2) {
    e2[0] = g->e[0];
    e2[1] = g->e[1];
  }
  if (axes6)
    for (int b = 0; b < 2; ++b)
      for (int d = 0; d < 3; ++d)
        axes6[3 * b + d] = g->ax[b][d];
}
/* full recompute of both boxes' inter energies */
void ora_gemc_system_total(const ora_gemc *g, double *e2) {
  for (int b = 0; b < 2; ++b)
    e2[b] = g_box_inter(g, b, g->x, g->y, g->z, g->ax[b], g->half[b]);
}
/* scales: displacement and volume per box; counts: tries and accepted of
 * displacement, transfer, volume per box */
void ora_gemc_settings(const ora_gemc *g, double *scale4, long *counts12) {
  for (int b = 0; b < 2; ++b) {
    scale4[2 * b] = g->scale[b][G_DISPLACE];
    scale4[2 * b + 1] = g->scale[b][G_VOL_TRANSFER];
    const int mv[3] = {G_DISPLACE, G_MOL_TRANSFER, G_VOL_TRANSFER};
    for (int k = 0; k < 3; ++k) {
      counts12[6 * b + 2 * k] = g->tries[b][mv[k]];
      counts12[6 * b + 2 * k + 1] = g->acc[b][mv[k]];
    }
  }
}
