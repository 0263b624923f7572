// EwaldGB300.h -- the reference-side shim: an Ewald subclass whose energy
// calls run on the GB300 library through the C ABI of gomc_gb300.h.
//
// A maintainer adds this header to the GOMC source tree and selects the class
// where System::Init picks Ewald / EwaldCached / NoEwald
// (src/System.cpp:132-148), with one gb_box per simulation box created from
// the same Coordinates / Forcefield / Molecules (gb_box_create).  Ewald's
// methods are virtual (src/Ewald.h:49-179), so callers stay unchanged; every
// override below keeps the reference signature (checked by `override`) and
// turns a non-zero status into GOMC's own fatal path (print, exit), as
// checkLastErrorCUDA does (src/GPU/VariablesCUDA.cuh:20-39).
//
// Molecule indices are those of the reference (one gb_box holds every
// molecule of its box in the reference's order, as in an NVT run).
// Methods not overridden here (VirialReciprocal, ChangeLambdaRecip,
// MolExchangeReciprocal, the free-energy Change* calls) keep the reference's
// host implementation.
#ifndef GOMC_GB300_EWALD_SHIM_H
#define GOMC_GB300_EWALD_SHIM_H

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "BoxDimensions.h"
#include "Ewald.h"
#include "TrialMol.h"
#include "XYZArray.h"
#include "gomc_gb300.h"

class EwaldGB300 : public Ewald {
public:
  // boxes[b] is the resident GB300 machine of simulation box b
  EwaldGB300(StaticVals &stat, System &sys, gb_box *const *boxes, uint nbox)
      : Ewald(stat, sys), boxes_(boxes, boxes + nbox) {}

  // Ewald::RecipInit (src/Ewald.cpp:835-903): k-vectors of trial axes
  void RecipInit(uint box, BoxDimensions const &boxAxes) override {
    XYZ ax = boxAxes.GetAxis(box);
    double edges[3] = {ax.x, ax.y, ax.z};
    int32_t k = 0;
    Check(gb_recip_init(Box(box), edges, &k), box);
  }
  // Ewald::BoxReciprocalSetup (src/Ewald.cpp:193-274)
  void BoxReciprocalSetup(uint box, XYZArray const &molCoords) override {
    std::vector<double> xyz = Flatten(molCoords);
    Check(gb_box_reciprocal_setup_coords(Box(box), xyz.data()), box);
  }
  // Ewald::BoxReciprocalSums (src/Ewald.cpp:281-361)
  void BoxReciprocalSums(uint box, XYZArray const &molCoords) override {
    std::vector<double> xyz = Flatten(molCoords);
    Check(gb_box_reciprocal_sums_coords(Box(box), xyz.data()), box);
  }
  // Ewald::BoxReciprocal (src/Ewald.cpp:375-406)
  double BoxReciprocal(uint box, bool isNewVolume) const override {
    double e = 0.0;
    Check(gb_box_reciprocal(Box(box), isNewVolume ? 1 : 0, &e), box);
    return e;
  }
  // Ewald::BoxSelf (src/Ewald.cpp:1125-1163)
  double BoxSelf(uint box) const override {
    double e = 0.0;
    Check(gb_box_self(Box(box), &e), box);
    return e;
  }
  // Ewald::MolReciprocal (src/Ewald.cpp:409-473)
  double MolReciprocal(XYZArray const &molCoords, const uint molIndex,
                       const uint box) override {
    std::vector<double> xyz = Flatten(molCoords);
    double d = 0.0;
    Check(gb_mol_reciprocal(Box(box), (int32_t)molIndex, xyz.data(), &d), box);
    return d;
  }
  // Ewald::MolCorrection (src/Ewald.cpp:1056-1085)
  double MolCorrection(uint molIndex, uint box) const override {
    double e = 0.0;
    Check(gb_mol_correction(Box(box), (int32_t)molIndex, &e), box);
    return e;
  }
  // Ewald::SwapDestRecip / SwapSourceRecip (src/Ewald.cpp:478-531, 657-710)
  double SwapDestRecip(const cbmc::TrialMol &newMol, const uint box,
                       const int molIndex) override {
    std::vector<double> xyz = Flatten(newMol.GetCoords());
    double d = 0.0;
    Check(gb_swap_dest_recip(Box(box), molIndex, xyz.data(), &d), box);
    return d;
  }
  double SwapSourceRecip(const cbmc::TrialMol &oldMol, const uint box,
                         const int molIndex) override {
    std::vector<double> xyz = Flatten(oldMol.GetCoords());
    double d = 0.0;
    Check(gb_swap_source_recip(Box(box), molIndex, xyz.data(), &d), box);
    return d;
  }
  // Ewald::SwapCorrection / SwapSelf (src/Ewald.cpp:1311-1391); the trial
  // molecule's kind gives the charges, which the library takes from the
  // molecule `mol` of that kind (index 0 here: every molecule of a kind has
  // the same charges)
  double SwapCorrection(const cbmc::TrialMol &trialMol) const override {
    std::vector<double> xyz = Flatten(trialMol.GetCoords());
    double e = 0.0;
    Check(gb_swap_correction(Box(trialMol.GetBox()), KindMol(trialMol),
                             xyz.data(), &e),
          trialMol.GetBox());
    return e;
  }
  double SwapSelf(const cbmc::TrialMol &trialMol) const override {
    double e = 0.0;
    Check(gb_swap_self(Box(trialMol.GetBox()), KindMol(trialMol), &e),
          trialMol.GetBox());
    return e;
  }
  // Ewald::UpdateRecip / CopyRecip / UpdateRecipVec (src/Ewald.cpp:1420-1487)
  void UpdateRecip(uint box) override { Check(gb_update_recip(Box(box)), box); }
  void CopyRecip(uint box) override { Check(gb_copy_recip(Box(box)), box); }
  void UpdateRecipVec(uint box) override {
    Check(gb_update_recip_vec(Box(box)), box);
  }
  // Ewald::SetRecipRef (src/Ewald.cpp:1021-1053): the library keeps New and
  // Ref in step through gb_box_reciprocal_setup / gb_update_recip
  void SetRecipRef(uint box) override { Check(gb_copy_recip(Box(box)), box); }
  // Ewald::BoxForceReciprocal (src/Ewald.cpp:1496-1596) of the New sums
  void BoxForceReciprocal(XYZArray const &molCoords, XYZArray &atomForceRec,
                          XYZArray &molForceRec, uint box) override {
    (void)molCoords;  // the box holds the coordinates of the New sums
    std::vector<double> a(3 * (size_t)atomForceRec.Count());
    std::vector<double> m(3 * (size_t)molForceRec.Count());
    Check(gb_box_force_reciprocal(Box(box), a.data(), m.data()), box);
    Unflatten(a, atomForceRec);
    Unflatten(m, molForceRec);
  }

private:
  gb_box *Box(uint b) const { return boxes_.at(b); }
  int32_t KindMol(const cbmc::TrialMol &t) const {
    // the first molecule of the trial molecule's kind (MoleculeKind is
    // shared by all of its molecules)
    const uint k = t.GetKind().kindIndex;
    for (uint m = 0; m < mols.count; ++m)
      if (mols.GetMolKind(m) == k)
        return (int32_t)m;
    return -1;  // no molecule of the kind: the library reports GB_ERR_ARG
  }
  static std::vector<double> Flatten(XYZArray const &c) {
    std::vector<double> v(3 * (size_t)c.Count());
    for (uint i = 0; i < c.Count(); ++i) {
      v[3 * i] = c.x[i];
      v[3 * i + 1] = c.y[i];
      v[3 * i + 2] = c.z[i];
    }
    return v;
  }
  static void Unflatten(const std::vector<double> &v, XYZArray &c) {
    for (uint i = 0; i < c.Count(); ++i)
      c.Set(i, v[3 * i], v[3 * i + 1], v[3 * i + 2]);
  }
  void Check(int rc, uint box) const {
    if (rc) {
      std::fprintf(stderr, "gomc_gb300 (box %u): %s\n", box,
                   gb_last_error(boxes_.at(box)));
      std::exit(EXIT_FAILURE);
    }
  }
  std::vector<gb_box *> boxes_;
};

#endif  // GOMC_GB300_EWALD_SHIM_H
