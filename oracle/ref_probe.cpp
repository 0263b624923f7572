// Probe program linked against the reference GOMC objects (built by
// oracle/ref.mk).  It loads a generated fixture through the reference's own
// Simulation constructor and dumps, at full FP64 precision, the numbers that
// pin the oracle and the GPU path:
//   - per-term initial energies (CalculateEnergy::SystemTotal,
//     src/CalculateEnergy.cpp:83-138) and the k-vector tables / structure
//     factors (Ewald::RecipInitOrth + BoxReciprocalSetup, src/Ewald.cpp:193-274,
//     847-903),
//   - cell-list membership (CellList::GetCellListNeighbor,
//     src/CellList.cpp:258-285),
//   - MoleculeInter / MolReciprocal / SwapDestRecip / SwapSourceRecip deltas for
//     a list of proposals read from a file (src/CalculateEnergy.cpp:581-686,
//     src/Ewald.cpp:409-531,657-710),
//   - BoxForce / BoxForceReciprocal / CalculateTorque outputs when the
//     fixture enables the MultiParticle move,
//   - ParticleInter trial energies (src/CalculateEnergy.cpp:727-785) with
//     and without the molecule in the cell list,
//   - trial-volume energies (VolumeTransfer's energy calls: RecipInit,
//     BoxReciprocalSetup, BoxInter at new axes) and the state after one
//     accepted volume change,
//   - a per-step trace of the reference Monte Carlo loop
//     (src/Simulation.cpp:94-96 without output, src/System.cpp:262-302),
//   - with GOMC_PROBE_CHK_STEP=N, the reference's own checkpoint file
//     (CheckpointOutput::saveCheckpointFile, src/CheckpointOutput.cpp:55-90)
//     after N steps of that loop, with the coordinates and the loop state it
//     holds; `ref_probe --read-chk file outdir` reads a checkpoint back with
//     the reference's deserializer (src/CheckpointSetup.cpp:45-82) and dumps
//     the same state.
// It is test infrastructure: it runs only in the build container.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <string>
#include <vector>
#include <algorithm>
#include <cmath>
#include <sstream>
#include <memory>
#include <functional>
#include <iomanip>
#include <set>
#include <list>
#include <unordered_map>
#include <array>
#include <limits>
#include <cassert>
#include <random>

// Access the reference's non-public state from this probe only.
#define private public
#define protected public
#include "Simulation.h"
#include "System.h"
#include "StaticVals.h"
#include "CalculateEnergy.h"
#include "Ewald.h"
#include "CellList.h"
#include "MoveBase.h"
#include "Translate.h"
#include "Rotation.h"
#include "MultiParticle.h"
#include "TrialMol.h"
#if ENSEMBLE == GEMC
#include "MoleculeTransfer.h"
#include "VolumeTransfer.h"
#include "Checkpoint.h"
#include "CheckpointOutput.h"
#endif
#undef private
#undef protected

static FILE *open_out(const std::string &dir, const char *name) {
  std::string p = dir + "/" + name;
  FILE *f = fopen(p.c_str(), "w");
  if (!f) {
    fprintf(stderr, "cannot write %s\n", p.c_str());
    exit(2);
  }
  return f;
}

static void dump_energy(FILE *f, const char *tag, const Energy &e) {
  fprintf(f, "%s inter %.17g\n", tag, e.inter);
  fprintf(f, "%s real %.17g\n", tag, e.real);
  fprintf(f, "%s recip %.17g\n", tag, e.recip);
  fprintf(f, "%s self %.17g\n", tag, e.self);
  fprintf(f, "%s correction %.17g\n", tag, e.correction);
  fprintf(f, "%s tailCorrection %.17g\n", tag, e.tailCorrection);
  fprintf(f, "%s intraBond %.17g\n", tag, e.intraBond);
  fprintf(f, "%s intraNonbond %.17g\n", tag, e.intraNonbond);
  fprintf(f, "%s total %.17g\n", tag, e.total);
}

static void dump_coords(const std::string &dir, const char *name,
                        const XYZArray &c) {
  FILE *f = open_out(dir, name);
  for (uint i = 0; i < c.Count(); ++i)
    fprintf(f, "%.17g %.17g %.17g\n", c.x[i], c.y[i], c.z[i]);
  fclose(f);
}

// Known-answer vectors of the reference's random streams: MTRand(seed)
// (src/MersenneTwister.h) and Random123Wrapper's Philox4x64-10
// (src/Random123Wrapper.cpp:16-84).
// The Monte Carlo state a checkpoint holds (step, MT19937, move settings of
// box 0 for molecule kind 0), one value per line.
static void dump_chk_state(const std::string &dir, const Checkpoint &c) {
  FILE *f = open_out(dir, "chk_state.txt");
  fprintf(f, "%llu %llu\n", (unsigned long long)c.stepNumber,
          (unsigned long long)c.trueStepNumber);
  for (int i = 0; i < N_array_size + 1; ++i)
    fprintf(f, "%u\n", c.saveArray[i]);
  fprintf(f, "%u %u %u\n", c.seedLocation, c.seedLeft, c.seedValue);
  const uint nm = c.scaleVec[0].size();
  fprintf(f, "%u\n", nm);
  for (uint m = 0; m < nm; ++m)
    fprintf(f, "%.17g %.17g %u %u %u %u\n", c.scaleVec[0][m][0],
            c.acceptPercentVec[0][m][0], c.acceptedVec[0][m][0],
            c.triesVec[0][m][0], c.tempAcceptedVec[0][m][0],
            c.tempTriesVec[0][m][0]);
  for (uint t = 0; t < c.mp_triesVec[0].size(); ++t)
    fprintf(f, "%u %u %u %u\n", c.mp_triesVec[0][t], c.mp_acceptedVec[0][t],
            c.mp_interval_triesVec[0][t], c.mp_interval_acceptedVec[0][t]);
  fprintf(f, "%.17g %.17g %d\n", c.mp_t_maxVec[0], c.mp_r_maxVec[0],
          (int)c.isSingleMoveAcceptedVec[0]);
  fclose(f);
}

// A checkpoint file read back as CheckpointSetup::loadCheckpointFile reads
// it: the Checkpoint object, then the molecule lookup's arrays.
static int read_chk(const char *file, const std::string &dir) {
  std::ifstream ifs(file, std::ios::binary);
  if (!ifs.is_open())
    return 1;
  Checkpoint c;
  cereal::BinaryInputArchive ia(ifs);
  ia >> c;
  MoleculeLookup &ml = c.originalMoleculeLookup;
  std::vector<uint32_t> a(ml.molLookupCount), b(ml.boxAndKindStartLength),
      sw(ml.boxAndKindSwappableLength);
  std::vector<int32_t> mi(ml.atomCount), ai(ml.atomCount), mk(ml.atomCount),
      ak(ml.atomCount);
  std::vector<double> q(ml.atomCount);
  ia(cereal::binary_data(a.data(), 4 * a.size()));
  ia(cereal::binary_data(b.data(), 4 * b.size()));
  ia(cereal::binary_data(sw.data(), 4 * sw.size()));
  ia(cereal::binary_data(mi.data(), 4 * mi.size()));
  ia(cereal::binary_data(ai.data(), 4 * ai.size()));
  ia(cereal::binary_data(mk.data(), 4 * mk.size()));
  ia(cereal::binary_data(ak.data(), 4 * ak.size()));
  ia(cereal::binary_data(q.data(), 8 * q.size()));
  dump_chk_state(dir, c);
  FILE *f = open_out(dir, "chk_lookup.txt");
  for (uint32_t v : a)
    fprintf(f, "%u\n", v);
  fclose(f);
  return 0;
}

static int dump_kat(const std::string &dir) {
  FILE *f = open_out(dir, "kat_mt.txt");
  const unsigned seeds[3] = {1234u, 4321u, 4294967295u};
  for (unsigned s : seeds) {
    MTRand g(s);
    for (int i = 0; i < 1500; ++i) fprintf(f, "%u %u\n", s, g.randInt());
  }
  fclose(f);
  f = open_out(dir, "kat_philox.txt");
  const unsigned long steps[3] = {0ul, 1ul, 123456ul};
  const unsigned long pseeds[3] = {0ul, 4321ul, 4294967295ul};
  const unsigned ctrs[4] = {0u, 1u, 255u, 8000u};
  for (unsigned long st : steps)
    for (unsigned long sd : pseeds)
      for (unsigned c : ctrs) {
        Random123Wrapper w;
        w.SetStep(st);
        w.SetRandomSeed(sd);
        RNG::ctr_type r = w.getRNG(c);
        XYZ rc = w.GetRandomCoords(c);
        XYZ sc = w.GetSymRandomCoords(c, 1.0);
        fprintf(f, "%lu %lu %u %llu %llu %llu %llu %.17g %.17g %.17g %.17g %.17g %.17g\n",
                st, sd, c, (unsigned long long)r[0], (unsigned long long)r[1],
                (unsigned long long)r[2], (unsigned long long)r[3], rc.x, rc.y,
                rc.z, sc.x, sc.y, sc.z);
      }
  fclose(f);
  return 0;
}

int main(int argc, char **argv) {
  if (argc == 3 && std::string(argv[1]) == "--kat")
    return dump_kat(argv[2]);
  if (argc == 4 && std::string(argv[1]) == "--read-chk")
    return read_chk(argv[2], argv[3]);
  if (argc < 4) {
    fprintf(stderr,
            "usage: ref_probe in.conf outdir nsteps [proposals.txt|-] "
            "[lambdas.txt|-] [particles.txt|-] [volumes.txt]\n");
    return 1;
  }
  std::string outdir = argv[2];
  long nsteps = atol(argv[3]);
  const char *propFile =
      argc > 4 && std::string(argv[4]) != "-" ? argv[4] : nullptr;
  const char *lamFile =
      argc > 5 && std::string(argv[5]) != "-" ? argv[5] : nullptr;
  const char *partFile =
      argc > 6 && std::string(argv[6]) != "-" ? argv[6] : nullptr;
  const char *volFile = argc > 7 ? argv[7] : nullptr;

  Simulation sim(argv[1]);
  System &sys = *sim.system;
  StaticVals &stat = *sim.staticValues;
  Ewald *ew = sys.calcEwald;
  const uint box = 0;

  // ---- initial state -------------------------------------------------------
  {
    FILE *f = open_out(outdir, "energies_init.txt");
    sys.potential.Total();
    dump_energy(f, "box0", sys.potential.boxEnergy[0]);
#if ENSEMBLE == GEMC || ENSEMBLE == GCMC
    dump_energy(f, "box1", sys.potential.boxEnergy[1]);
#endif
    fprintf(f, "alpha %.17g\n", stat.forcefield.alpha[0]);
    fprintf(f, "recip_rcut %.17g\n", stat.forcefield.recip_rcut[0]);
    fprintf(f, "beta %.17g\n", stat.forcefield.beta);
    if (stat.forcefield.ewald) {
      fprintf(f, "imageSize %u\n", ew->imageSizeRef[0]);
      fprintf(f, "kmax %u\n", ew->kmax[0]);
      fprintf(f, "imageTotal %u\n", ew->imageTotal);
    }
    fprintf(f, "edgeCells %d %d %d\n", sys.cellList.edgeCells[0][0],
            sys.cellList.edgeCells[0][1], sys.cellList.edgeCells[0][2]);
    fclose(f);
  }
  dump_coords(outdir, "coords_init.txt", sys.coordinates);
  dump_coords(outdir, "com_init.txt", sys.com);

  // CalculateEnergy::VirialCalc on the initial state
  // (src/CalculateEnergy.cpp:411-579): scalars and tensor diagonals
  {
    Virial v = sys.calcEnergy.VirialCalc(box);
    FILE *f = open_out(outdir, "virial.txt");
    fprintf(f, "%.17g %.17g %.17g %.17g\n", v.inter, v.real, v.recip,
            v.total);
    for (int d = 0; d < 3; ++d)
      fprintf(f, "%.17g %.17g %.17g %.17g\n", v.interTens[d][d],
              v.realTens[d][d], v.recipTens[d][d], v.totalTens[d][d]);
    fclose(f);
  }

  if (stat.forcefield.ewald) {
    FILE *f = open_out(outdir, "kvec.txt");
    for (uint i = 0; i < ew->imageSizeRef[box]; ++i)
      fprintf(f, "%.17g %.17g %.17g %.17g %.17g %.17g %.17g\n", ew->kxRef[box][i],
              ew->kyRef[box][i], ew->kzRef[box][i], ew->prefactRef[box][i],
              ew->sumRref[box][i], ew->sumIref[box][i], ew->hsqrRef[box][i]);
    fclose(f);
  }

  for (uint b = 0; b < BOX_TOTAL; ++b) {
    std::vector<int> cellVector, cellStart, mapP;
    sys.cellList.GetCellListNeighbor(b, sys.coordinates.Count(), cellVector,
                                     cellStart, mapP);
    char name[64];
    snprintf(name, sizeof name, "cells_box%u.txt", b);
    FILE *f = open_out(outdir, name);
    fprintf(f, "%d %d %d\n", sys.cellList.edgeCells[b][0],
            sys.cellList.edgeCells[b][1], sys.cellList.edgeCells[b][2]);
    // membership of every particle that sits in box b
    for (int c = 0; c + 1 < (int)cellStart.size(); ++c)
      for (int i = cellStart[c]; i < cellStart[c + 1]; ++i)
        fprintf(f, "%d %d\n", cellVector[i], c);
    fclose(f);
  }

  // ---- forces (only when the MultiParticle move is enabled) ---------------
  if (stat.multiParticleEnabled) {
    uint nAtoms = sys.coordinates.Count();
    uint nMol = sys.com.Count();
    XYZArray aF(nAtoms), mF(nMol), aR(nAtoms), mR(nMol), tq(nMol);
    SystemPotential p = sys.potential;
    p = sys.calcEnergy.BoxForce(p, sys.coordinates, aF, mF, sys.boxDimRef, box);
    ew->CopyRecip(box);
    ew->BoxForceReciprocal(sys.coordinates, aR, mR, box);
    std::vector<uint> molIdx(nMol);
    for (uint m = 0; m < nMol; ++m) molIdx[m] = m;
    sys.calcEnergy.CalculateTorque(molIdx, sys.coordinates, sys.com, aF, aR, tq,
                                   box);
    FILE *f = open_out(outdir, "forces_atom.txt");
    for (uint i = 0; i < nAtoms; ++i)
      fprintf(f, "%.17g %.17g %.17g %.17g %.17g %.17g\n", aF.x[i], aF.y[i],
              aF.z[i], aR.x[i], aR.y[i], aR.z[i]);
    fclose(f);
    f = open_out(outdir, "forces_mol.txt");
    for (uint m = 0; m < nMol; ++m)
      fprintf(f, "%.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n",
              mF.x[m], mF.y[m], mF.z[m], mR.x[m], mR.y[m], mR.z[m], tq.x[m],
              tq.y[m], tq.z[m]);
    fclose(f);
    f = open_out(outdir, "force_energy.txt");
    fprintf(f, "inter %.17g\nreal %.17g\n", p.boxEnergy[box].inter,
            p.boxEnergy[box].real);
    fclose(f);
  }

  // ---- per-proposal deltas on the initial state ---------------------------
  if (propFile) {
    std::ifstream in(propFile);
    int nprop = 0;
    in >> nprop;
    FILE *f = open_out(outdir, "proposals_out.txt");
    for (int i = 0; i < nprop; ++i) {
      uint m, na;
      in >> m >> na;
      XYZArray pos(na);
      for (uint a = 0; a < na; ++a) in >> pos.x[a] >> pos.y[a] >> pos.z[a];
      Intermolecular lj, coul;
      sys.cellList.RemoveMol(m, box, sys.coordinates);
      bool overlap =
          sys.calcEnergy.MoleculeInter(lj, coul, pos, m, box);
      sys.cellList.AddMol(m, box, sys.coordinates);
      double recip = 0.0, dest = 0.0, src = 0.0;
      if (stat.forcefield.ewald) {
        recip = ew->MolReciprocal(pos, m, box);
        // insertion of the proposed copy and deletion of the current one
        const MoleculeKind &kind = stat.mol.GetKind(m);
        cbmc::TrialMol tNew(kind, sys.boxDimRef, box);
        tNew.SetCoords(pos, 0);
        dest = ew->SwapDestRecip(tNew, box, m);
        cbmc::TrialMol tOld(kind, sys.boxDimRef, box);
        XYZArray cur(na);
        for (uint a = 0; a < na; ++a)
          cur.Set(a, sys.coordinates[stat.mol.MolStart(m) + a]);
        tOld.SetCoords(cur, 0);
        src = ew->SwapSourceRecip(tOld, box, m);
      }
      fprintf(f, "%u %d %.17g %.17g %.17g %.17g %.17g\n", m, (int)overlap,
              lj.energy, coul.energy, recip, dest, src);
    }
    fclose(f);
  }

  // ---- SingleMoleculeInter at two lambda values ---------------------------
  // lambdas.txt: "sc_alpha sc_sigma sc_power", n, then n lines
  // "mol lambdaOldVDW lambdaNewVDW lambdaOldCoulomb lambdaNewCoulomb sc_coul";
  // the soft-core settings are set on the reference's own Forcefield
  // (src/Forcefield.cpp:59-75) before each call.
  if (lamFile) {
    std::ifstream in(lamFile);
    double scA, scS;
    uint scP;
    int n = 0;
    in >> scA >> scS >> scP >> n;
    Forcefield &ffd = stat.forcefield;
    ffd.sc_alpha = scA;
    ffd.sc_sigma = scS;
    ffd.sc_sigma_6 = pow(scS, 6.0);
    ffd.sc_power = scP;
    FILE *f = open_out(outdir, "single_mol_out.txt");
    for (int i = 0; i < n; ++i) {
      uint m;
      int scc;
      double lov, lnv, loc, lnc;
      in >> m >> lov >> lnv >> loc >> lnc >> scc;
      ffd.sc_coul = scc != 0;
      Energy eo, en;
      sys.calcEnergy.SingleMoleculeInter(eo, en, lov, lnv, loc, lnc, m, box);
      fprintf(f, "%u %.17g %.17g %.17g %.17g %d %.17g %.17g %.17g %.17g\n", m,
              lov, lnv, loc, lnc, scc, eo.inter, eo.real, en.inter, en.real);
    }
    fclose(f);
  }

  // ---- ParticleInter, the CBMC first-atom trial energies ------------------
  // particles.txt: n, then n lines "mol part remove ntrials x y z ...".
  // With remove = 1 the molecule leaves the cell list around the call, as
  // MoleculeTransfer::Transform does before DCSingle::BuildOld/BuildNew
  // (src/moves/MoleculeTransfer.h:100-106, src/cbmc/DCSingle.cpp:23-90);
  // with remove = 0 the call sees the cell list as it stands.
  if (partFile) {
    std::ifstream in(partFile);
    int n = 0;
    in >> n;
    FILE *f = open_out(outdir, "particles_out.txt");
    for (int i = 0; i < n; ++i) {
      uint m, part, nt;
      int remove;
      in >> m >> part >> remove >> nt;
      XYZArray pos(nt);
      for (uint t = 0; t < nt; ++t) in >> pos.x[t] >> pos.y[t] >> pos.z[t];
      std::vector<double> en(nt, 0.0), re(nt, 0.0);
      std::unique_ptr<bool[]> ov(new bool[nt]);
      for (uint t = 0; t < nt; ++t) ov[t] = false;
      if (remove) sys.cellList.RemoveMol(m, box, sys.coordinates);
      sys.calcEnergy.ParticleInter(en.data(), re.data(), pos, ov.get(), part,
                                   m, box, nt);
      if (remove) sys.cellList.AddMol(m, box, sys.coordinates);
      fprintf(f, "%u %u %d %u", m, part, remove, nt);
      for (uint t = 0; t < nt; ++t)
        fprintf(f, " %.17g %.17g %d", en[t], re[t], (int)ov[t]);
      fprintf(f, "\n");
    }
    fclose(f);
  }

  // ---- trial volumes (the NPT branch of VolumeTransfer) -------------------
  // volumes.txt: n, then n volume changes (A^3).  Each is evaluated from the
  // initial state as VolumeTransfer::Transform / CalcEn do
  // (src/moves/VolumeTransfer.h:96-190): ShiftVolume, TranslateOneBox,
  // GridAll on the new axes, RecipInit + BoxReciprocalSetup on the new
  // coordinates, BoxInter and BoxReciprocal(box, true).  The last one is
  // then accepted (new coordinates, centres and axes, UpdateRecip,
  // UpdateRecipVec) and the state recomputed as System::Init does
  // (GridAll, UpdateVectorsAndRecipTerms, SystemTotal).
  if (volFile) {
    std::ifstream in(volFile);
    int n = 0;
    in >> n;
    FILE *f = open_out(outdir, "volume_out.txt");
    const uint N = sys.coordinates.Count();
    XYZArray scratch(N);
    COM newCOM(sys.boxDimRef, scratch, sys.molLookupRef, stat.mol);
    newCOM.Init(stat.mol.count);
    Coordinates newPos(sys.boxDimRef, newCOM, sys.molLookupRef, sys.prng,
                       stat.mol);
    newPos.Init(N);
    BoxDimensions newDim;
    for (int i = 0; i < n; ++i) {
      double delta;
      in >> delta;
      newDim = sys.boxDimRef;
      sys.coordinates.CopyRange(newPos, 0, 0, N);
      sys.com.CopyRange(newCOM, 0, 0, sys.com.Count());
      XYZ scale;
      sys.boxDimRef.ShiftVolume(newDim, scale, box, delta);
      sys.coordinates.TranslateOneBox(newPos, newCOM, sys.com, newDim, box,
                                      scale);
      sys.cellList.GridAll(newDim, newPos, sys.molLookupRef);
      SystemPotential pNew = sys.potential;
      double recip = 0.0;
      uint knew = 0;
      if (stat.forcefield.ewald) {
        ew->RecipInit(box, newDim);
        ew->BoxReciprocalSetup(box, newPos);
      }
      pNew = sys.calcEnergy.BoxInter(pNew, newPos, newDim, box);
      if (stat.forcefield.ewald) {
        recip = ew->BoxReciprocal(box, true);
        knew = ew->imageSize[box];
      }
      XYZ ax = newDim.GetAxis(box);
      fprintf(f, "%.17g %.17g %.17g %.17g %u %.17g %.17g %.17g\n", delta,
              ax.x, ax.y, ax.z, knew, pNew.boxEnergy[box].inter,
              pNew.boxEnergy[box].real, recip);
      char name[64];
      snprintf(name, sizeof name, "volume_pos_%d.txt", i);
      dump_coords(outdir, name, newPos);
      snprintf(name, sizeof name, "volume_com_%d.txt", i);
      dump_coords(outdir, name, newCOM);
    }
    fclose(f);
    if (n > 0) {
      // accept the last trial volume
      newPos.CopyRange(sys.coordinates, 0, 0, N);
      newCOM.CopyRange(sys.com, 0, 0, sys.com.Count());
      sys.boxDimRef = newDim;
      if (stat.forcefield.ewald) {
        ew->UpdateRecip(box);
        ew->UpdateRecipVec(box);
      }
      sys.cellList.GridAll(sys.boxDimRef, sys.coordinates, sys.molLookupRef);
      if (stat.forcefield.ewald)
        ew->UpdateVectorsAndRecipTerms(false);
      SystemPotential pot = sys.calcEnergy.SystemTotal();
      f = open_out(outdir, "volume_accept.txt");
      dump_energy(f, "box0", pot.boxEnergy[box]);
      if (stat.forcefield.ewald)
        fprintf(f, "imageSize %u\n", ew->imageSizeRef[box]);
      fclose(f);
    }
  }

#if ENSEMBLE == GEMC
  // ---- GEMC Monte Carlo trace ----------------------------------------------
  // One line per step: step, move kind, box (displacement: its box; swap:
  // source box; volume: first box of the pair), molecule (-1 when none was
  // picked or for a volume move), accepted, the running inter energies and
  // volumes of both boxes, molecules in box 0, then four move values:
  // displacement: dLJ, overlap, 0, 0; swap: new and old Rosenbluth weights,
  // new and old trial energies; volume: the trial inter energies of both
  // boxes, 0, 0.
  if (nsteps > 0) {
    FILE *f = open_out(outdir, "trace.txt");
    MoveSettings &ms = sys.moveSettings;
    MoleculeLookup &ml = sys.molLookupRef;
    for (long step = 0; step < nsteps; ++step) {
      ms.AdjustMoves(step);
      sys.r123wrapper.SetStep(step);
      double draw = 0;
      uint kind = 0;
      sys.PickMove(kind, draw);
      uint acc0 = 0, acc1 = 0;
      for (uint b = 0; b < BOX_TOTAL; ++b)
        for (uint k = 0; k < mv::MOVE_KINDS_TOTAL; ++k)
          acc0 += ms.GetAcceptTot(b, k);
      uint n_before[2] = {ml.NumInBox(0), ml.NumInBox(1)};
      sys.RunMove(kind, draw, step);
      for (uint b = 0; b < BOX_TOTAL; ++b)
        for (uint k = 0; k < mv::MOVE_KINDS_TOTAL; ++k)
          acc1 += ms.GetAcceptTot(b, k);
      int accepted = acc1 > acc0;
      long bx = -1, m = -1;
      double d[4] = {0, 0, 0, 0};
      if (kind == mv::DISPLACE) {
        Translate *t = static_cast<Translate *>(sys.moves[kind]);
        bx = t->b;
        if (n_before[bx] > 0) {
          m = t->m;
          d[0] = t->inter_LJ.energy;
          d[1] = t->overlap;
        }
      } else if (kind == mv::MOL_TRANSFER) {
        MoleculeTransfer *t = static_cast<MoleculeTransfer *>(sys.moves[kind]);
        bx = t->sourceBox;
        if (n_before[bx] > 0) {
          m = t->molIndex;
          d[0] = t->newMol.GetWeight();
          d[1] = t->oldMol.GetWeight();
          d[2] = t->newMol.GetEnergy().inter;
          d[3] = t->oldMol.GetEnergy().inter;
        }
      } else if (kind == mv::VOL_TRANSFER) {
        VolumeTransfer *v = static_cast<VolumeTransfer *>(sys.moves[kind]);
        bx = v->bPick[0];
        d[0] = v->sysPotNew.boxEnergy[0].inter;
        d[1] = v->sysPotNew.boxEnergy[1].inter;
      }
      fprintf(f,
              "%ld %u %ld %ld %d %.17g %.17g %.17g %.17g %u %.17g %.17g "
              "%.17g %.17g\n",
              step, kind, bx, m, accepted, sys.potential.boxEnergy[0].inter,
              sys.potential.boxEnergy[1].inter, sys.boxDimRef.volume[0],
              sys.boxDimRef.volume[1], ml.NumInBox(0), d[0], d[1], d[2], d[3]);
    }
    fclose(f);
    f = open_out(outdir, "energies_final.txt");
    sys.potential.Total();
    dump_energy(f, "running0", sys.potential.boxEnergy[0]);
    dump_energy(f, "running1", sys.potential.boxEnergy[1]);
    SystemPotential pot = sys.calcEnergy.SystemTotal();
    dump_energy(f, "recalc0", pot.boxEnergy[0]);
    dump_energy(f, "recalc1", pot.boxEnergy[1]);
    for (uint b = 0; b < BOX_TOTAL; ++b) {
      XYZ ax = sys.boxDimRef.GetAxis(b);
      fprintf(f, "axis %u %.17g %.17g %.17g\n", b, ax.x, ax.y, ax.z);
      const uint kinds[3] = {mv::DISPLACE, mv::MOL_TRANSFER, mv::VOL_TRANSFER};
      for (uint k : kinds)
        fprintf(f, "settings %u %u %u %u %.17g\n", b, k,
                ms.GetTrialTot(b, k), ms.GetAcceptTot(b, k),
                ms.GetScaleTot(b, k));
    }
    fclose(f);
    dump_coords(outdir, "coords_final.txt", sys.coordinates);
    dump_coords(outdir, "com_final.txt", sys.com);
    f = open_out(outdir, "lookup_final.txt");
    fprintf(f, "%u %u\n", ml.NumInBox(0), ml.NumInBox(1));
    for (uint i = 0; i < ml.NumInBox(0) + ml.NumInBox(1); ++i)
      fprintf(f, "%u\n", ml.molLookup[i]);
    fclose(f);
  }
  return 0;
#endif

  // ---- Monte Carlo trace ---------------------------------------------------
  if (nsteps > 0) {
    FILE *f = open_out(outdir, "trace.txt");
    MoveSettings &ms = sys.moveSettings;
    const char *chk_env = getenv("GOMC_PROBE_CHK_STEP");
    const long chk_step = chk_env ? atol(chk_env) : -1;
    for (long step = 0; step < nsteps; ++step) {
      if (step == chk_step) {
        // the checkpoint the reference writes after step chk_step - 1
        // (DoOutputRestart: the next run starts at chk_step)
        CheckpointOutput co(sys, stat, sim.set);
        co.filename = outdir + "/restart.chk";
        co.restartFromCheckpoint = false;  // a first run: true step = step
        co.startStep = 0;
        co.saveCheckpointFile(chk_step, ms, sys.prng, stat.mol,
                              sys.molLookupRef);
        Checkpoint c(chk_step, chk_step, ms, sys.prng, stat.mol,
                     sys.molLookupRef, sim.set.mol, sim.set.pdb.atoms);
        dump_chk_state(outdir, c);
        dump_coords(outdir, "coords_chk.txt", sys.coordinates);
        dump_coords(outdir, "com_chk.txt", sys.com);
      }
      ms.AdjustMoves(step);
      sys.r123wrapper.SetStep(step);
      double draw = 0;
      uint kind = 0;
      sys.PickMove(kind, draw);
      uint acc0 = 0, acc1 = 0;
      for (uint k = 0; k < mv::MOVE_KINDS_TOTAL; ++k)
        acc0 += ms.GetAcceptTot(box, k);
      sys.RunMove(kind, draw, step);
      for (uint k = 0; k < mv::MOVE_KINDS_TOTAL; ++k)
        acc1 += ms.GetAcceptTot(box, k);
      int accepted = acc1 > acc0;
      long m = -1;
      int overlap = 0;
      double dLJ = 0, dReal = 0, dRecip = 0;
      if (kind == mv::DISPLACE) {
        Translate *t = static_cast<Translate *>(sys.moves[kind]);
        m = t->m;
        overlap = t->overlap;
        dLJ = t->inter_LJ.energy;
        dReal = t->inter_Real.energy;
        dRecip = t->recip.energy;
      } else if (kind == mv::ROTATE) {
        Rotate *r = static_cast<Rotate *>(sys.moves[kind]);
        m = r->m;
        overlap = r->overlap;
        dLJ = r->inter_LJ.energy;
        dReal = r->inter_Real.energy;
        dRecip = r->recip.energy;
      } else if (kind == mv::MULTIPARTICLE) {
        MultiParticle *mp = static_cast<MultiParticle *>(sys.moves[kind]);
        m = mp->moveType;
        dLJ = mp->sysPotNew.boxEnergy[box].inter;
        dReal = mp->sysPotNew.boxEnergy[box].real;
        dRecip = mp->sysPotNew.boxEnergy[box].recip;
      }
      Energy &e = sys.potential.boxEnergy[box];
      fprintf(f, "%ld %u %ld %d %d %.17g %.17g %.17g %.17g %.17g %.17g\n", step,
              kind, m, accepted, overlap, dLJ, dReal, dRecip, e.inter, e.real,
              e.recip);
    }
    fclose(f);
    f = open_out(outdir, "energies_final.txt");
    sys.potential.Total();
    dump_energy(f, "running", sys.potential.boxEnergy[0]);
    ew->UpdateVectorsAndRecipTerms(false);
    SystemPotential pot = sys.calcEnergy.SystemTotal();
    dump_energy(f, "recalc", pot.boxEnergy[0]);
    for (uint k = 0; k < mv::MOVE_KINDS_TOTAL; ++k)
      if (ms.GetTrialTot(box, k) > 0)
        fprintf(f, "move %u tries %u accepted %u scale %.17g\n", k,
                ms.GetTrialTot(box, k), ms.GetAcceptTot(box, k),
                ms.GetScaleTot(box, k));
    fprintf(f, "mp_t_max %.17g\nmp_r_max %.17g\n", ms.GetTMAX(box),
            ms.GetRMAX(box));
    fclose(f);
    dump_coords(outdir, "coords_final.txt", sys.coordinates);
    dump_coords(outdir, "com_final.txt", sys.com);
  }
  return 0;
}
