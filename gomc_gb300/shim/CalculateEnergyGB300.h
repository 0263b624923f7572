// CalculateEnergyGB300.h -- the reference-side calls for the non-virtual
// CalculateEnergy and CellList methods (src/CalculateEnergy.h:52-179,
// src/CellList.h:24-64).  Each function takes the reference's own argument
// types, calls the C ABI of gomc_gb300.h on the box's resident gb_box and
// returns what the reference method returns; a maintainer calls it from an
// `#ifdef GOMC_GB300` branch at the top of the method, beside the existing
// `#ifdef GOMC_CUDA` branches (e.g. src/CalculateEnergy.cpp:175-197).
// A non-zero status ends the run through GOMC's fatal path.
#ifndef GOMC_GB300_CALCULATE_ENERGY_SHIM_H
#define GOMC_GB300_CALCULATE_ENERGY_SHIM_H

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "BoxDimensions.h"
#include "EnergyTypes.h"
#include "XYZArray.h"
#include "gomc_gb300.h"

namespace gb300 {

inline void Check(int rc, gb_box *box) {
  if (rc) {
    std::fprintf(stderr, "gomc_gb300: %s\n", gb_last_error(box));
    std::exit(EXIT_FAILURE);
  }
}

inline std::vector<double> Flatten(XYZArray const &c) {
  std::vector<double> v(3 * (size_t)c.Count());
  for (uint i = 0; i < c.Count(); ++i) {
    v[3 * i] = c.x[i];
    v[3 * i + 1] = c.y[i];
    v[3 * i + 2] = c.z[i];
  }
  return v;
}

// CalculateEnergy::MoleculeInter (src/CalculateEnergy.cpp:581-686)
inline bool MoleculeInter(gb_box *box, Intermolecular &inter_LJ,
                          Intermolecular &inter_coulomb,
                          XYZArray const &molCoords, const uint molIndex) {
  std::vector<double> xyz = Flatten(molCoords);
  double lj = 0.0, real = 0.0;
  int32_t overlap = 0;
  Check(gb_molecule_inter(box, (int32_t)molIndex, xyz.data(), &lj, &real,
                          &overlap),
        box);
  inter_LJ.energy += lj;
  inter_coulomb.energy += real;
  return overlap != 0;
}

// CalculateEnergy::BoxInter (src/CalculateEnergy.cpp:157-266) of given
// coordinates at given axes (the box's own state is untouched)
inline SystemPotential BoxInter(gb_box *box, SystemPotential potential,
                                XYZArray const &coords,
                                BoxDimensions const &boxAxes, const uint b) {
  std::vector<double> xyz = Flatten(coords);
  XYZ ax = boxAxes.GetAxis(b);
  double edges[3] = {ax.x, ax.y, ax.z};
  double lj = 0.0, real = 0.0;
  Check(gb_box_inter_coords(box, edges, xyz.data(), &lj, &real), box);
  potential.boxEnergy[b].inter = lj;
  potential.boxEnergy[b].real = real;
  potential.Total();
  return potential;
}

// CalculateEnergy::BoxForce (src/CalculateEnergy.cpp:268-406)
inline SystemPotential BoxForce(gb_box *box, SystemPotential potential,
                                XYZArray const &coords, XYZArray &atomForce,
                                XYZArray &molForce, const uint b) {
  std::vector<double> xyz = Flatten(coords);
  std::vector<double> a(3 * (size_t)atomForce.Count());
  std::vector<double> m(3 * (size_t)molForce.Count());
  double lj = 0.0, real = 0.0;
  Check(gb_box_force_coords(box, xyz.data(), &lj, &real, a.data(), m.data()),
        box);
  for (uint i = 0; i < atomForce.Count(); ++i)
    atomForce.Set(i, a[3 * i], a[3 * i + 1], a[3 * i + 2]);
  for (uint i = 0; i < molForce.Count(); ++i)
    molForce.Set(i, m[3 * i], m[3 * i + 1], m[3 * i + 2]);
  potential.boxEnergy[b].inter = lj;
  potential.boxEnergy[b].real = real;
  potential.Total();
  return potential;
}

// CalculateEnergy::ParticleInter (src/CalculateEnergy.cpp:727-785): adds to
// en[] / real[] and ORs overlap[] like the reference
inline void ParticleInter(gb_box *box, double *en, double *real,
                          XYZArray const &trialPos, bool *overlap,
                          const uint partIndex, const uint molIndex,
                          const uint trials) {
  std::vector<double> xyz = Flatten(trialPos);
  std::vector<double> e(trials), r(trials);
  std::vector<int32_t> ov(trials);
  Check(gb_particle_inter(box, (int32_t)molIndex, (int32_t)partIndex,
                          xyz.data(), (int32_t)trials, e.data(), r.data(),
                          ov.data()),
        box);
  for (uint t = 0; t < trials; ++t) {
    en[t] += e[t];
    real[t] += r[t];
    overlap[t] |= ov[t] != 0;
  }
}

// CalculateEnergy::SingleMoleculeInter (src/CalculateEnergy.cpp:1494-1556)
inline void SingleMoleculeInter(gb_box *box, Energy &interEnOld,
                                Energy &interEnNew, const double lambdaOldVDW,
                                const double lambdaNewVDW,
                                const double lambdaOldCoulomb,
                                const double lambdaNewCoulomb,
                                const uint molIndex) {
  double lam[4] = {lambdaOldVDW, lambdaNewVDW, lambdaOldCoulomb,
                   lambdaNewCoulomb};
  double out[4];
  Check(gb_single_molecule_inter(box, (int32_t)molIndex, lam, out), box);
  interEnOld.inter = out[0];
  interEnOld.real = out[1];
  interEnNew.inter = out[2];
  interEnNew.real = out[3];
}

// CellList::RemoveMol / AddMol (src/CellList.cpp:81-135) on the device copy
inline void RemoveMol(gb_box *box, const int molIndex) {
  Check(gb_cell_remove_mol(box, molIndex), box);
}
inline void AddMol(gb_box *box, const int molIndex) {
  Check(gb_cell_add_mol(box, molIndex), box);
}

}  // namespace gb300

#endif  // GOMC_GB300_CALCULATE_ENERGY_SHIM_H
