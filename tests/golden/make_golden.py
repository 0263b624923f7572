"""Generate the golden vectors that pin the oracle and the GPU path.

Run in a container that has the reference sources (read-only), given by
``--ref`` or the ``GOMC_REFERENCE`` environment variable::

    GOMC_REFERENCE=/root/reference python tests/golden/make_golden.py [names]

It builds the reference CPU path from its own sources with ``oracle/ref.mk``
(outputs in ``oracle/_ref/``), writes seeded fixtures in the reference's input
formats, runs ``oracle/_ref/ref_probe_ens1`` on each and stores the probe's
full-precision outputs as compressed ``.npz`` files beside this script.  The
GPU machine never needs the reference: tests read only the ``.npz`` files.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from gomc_gb300.config import SimConfig  # noqa: E402
from gomc_gb300.systems import (lj_sphere_box, spce_water_box,  # noqa: E402
                                water_box_length, write_gemc_inputs,
                                write_reference_inputs)

# name -> (system builder, config, MC steps, number of proposals)
FIXTURES = {
    # 256 SPC/E waters, 19.7 A box, Rcut 9, Ewald tolerance 1e-5, T = 298 K
    "c0_water": (lambda: spce_water_box(256, 19.7, seed=7),
                 SimConfig(temperature=298.0, rcut=9.0, tolerance=1e-5,
                           run_steps=2000, eq_steps=1000, adj_steps=10,
                           dis_freq=0.5, rot_freq=0.5, random_seed=1234),
                 2000, 64),
    # same geometry family with the MultiParticle move in the mix
    "c0_water_mp": (lambda: spce_water_box(256, 19.7, seed=11),
                    SimConfig(temperature=298.0, rcut=9.0, tolerance=1e-5,
                              run_steps=600, eq_steps=300, adj_steps=10,
                              dis_freq=0.45, rot_freq=0.45,
                              multi_particle_freq=0.1, random_seed=4321),
                    600, 16),
    # 1728 waters (12^3 lattice) at 1 g/cm3: 4x4x4 cells, K ~ 8.6k
    "w1728": (lambda: spce_water_box(1728, round(water_box_length(1728), 3),
                                     seed=5),
              SimConfig(temperature=298.0, rcut=9.0, tolerance=1e-5,
                        run_steps=400, eq_steps=200, adj_steps=10,
                        dis_freq=0.5, rot_freq=0.5, random_seed=99),
              400, 32),
    # single-site LJ spheres, no charges, no Ewald (GEMC-style particles)
    "lj500": (lambda: lj_sphere_box(500, 30.0, seed=3, epsilon=148.0,
                                    sigma=3.73, min_sep=3.0, name="LJ"),
              SimConfig(temperature=150.0, rcut=12.0, ewald=False,
                        electrostatic=False, run_steps=1500, eq_steps=1000,
                        adj_steps=10, dis_freq=1.0, rot_freq=0.0,
                        random_seed=777),
              1500, 32),
    # the two boxes of the GEMC configuration, each as its own NVT box: the
    # energy calls its moves make (BoxInter, GridAll, ParticleInter, single
    # particle displacements).  Liquid: 2,400 spheres in 40 A (3 cells per
    # axis); vapour: 300 in 90 A (7 cells per axis).  Random placement at
    # the liquid's density needs a closest approach below sigma.
    "c3_liquid": (lambda: lj_sphere_box(2400, 40.0, seed=31, epsilon=148.0,
                                        sigma=3.73, min_sep=2.4, name="LJ"),
                  SimConfig(temperature=150.0, rcut=12.0, ewald=False,
                            electrostatic=False, run_steps=1000, eq_steps=500,
                            adj_steps=10, dis_freq=1.0, rot_freq=0.0,
                            random_seed=3131),
                  1000, 32),
    "c3_vapour": (lambda: lj_sphere_box(300, 90.0, seed=32, epsilon=148.0,
                                        sigma=3.73, min_sep=3.5, name="LJ"),
                  SimConfig(temperature=150.0, rcut=12.0, ewald=False,
                            electrostatic=False, run_steps=1500, eq_steps=1000,
                            adj_steps=10, dis_freq=1.0, rot_freq=0.0,
                            random_seed=3232),
                  1500, 32),
    # the 8,000-water system the benchmark runs (same generator seed): 62.1 A,
    # Rcut 10, Ewald tolerance 1e-5 (K = 24,658), 6 cells per axis; moves
    # adjusted every 1,000 steps like the benchmark's chain
    "c1_water": (lambda: spce_water_box(8000, 62.1, seed=20260),
                 SimConfig(temperature=298.0, rcut=10.0, tolerance=1e-5,
                           run_steps=2000, eq_steps=1000, adj_steps=1000,
                           dis_freq=0.5, rot_freq=0.5, random_seed=20260),
                 2000, 64),
    # the same system with the MultiParticle move in the mix (BoxForce,
    # BoxForceReciprocal and the full structure factor at 8,000 waters)
    "c1_water_mp": (lambda: spce_water_box(8000, 62.1, seed=20261),
                    SimConfig(temperature=298.0, rcut=10.0, tolerance=1e-5,
                              run_steps=60, eq_steps=30, adj_steps=10,
                              dis_freq=0.45, rot_freq=0.45,
                              multi_particle_freq=0.1, random_seed=20261),
                    60, 8),
}


def build_reference(ref: str) -> str:
    subprocess.check_call(["make", "-s", "-f", os.path.join(ROOT, "oracle",
                                                             "ref.mk"),
                           "REF=" + ref, "OUT=" + os.path.join(ROOT, "oracle",
                                                               "_ref"),
                           "-j8"], cwd=ROOT)
    return os.path.join(ROOT, "oracle", "_ref", "ref_probe_ens1")


def _energies(path):
    out = {}
    for line in open(path):
        t = line.split()
        if len(t) == 3 and t[0] in ("box0", "running", "recalc"):
            out[t[0] + "_" + t[1]] = float(t[2])
        elif len(t) == 2:
            try:
                out[t[0]] = float(t[1])
            except ValueError:
                pass
        elif len(t) == 4 and t[0] == "edgeCells":
            out["edgeCells"] = [int(v) for v in t[1:]]
        elif t and t[0] == "move":
            out["move%s" % t[1]] = [float(t[3]), float(t[5]), float(t[7])]
    return out


def make_one(probe: str, name: str) -> None:
    builder, cfg, nsteps, nprop = FIXTURES[name]
    sysm = builder()
    rng = np.random.default_rng(1000 + len(name))
    with tempfile.TemporaryDirectory() as d:
        write_reference_inputs(d, sysm, cfg)
        # proposals: random rigid shifts of random molecules, wrapped
        props_m = rng.integers(0, sysm.n_mol, size=nprop)
        na = int(sysm.mol_start[1] - sysm.mol_start[0])
        shifts = rng.uniform(-0.6, 0.6, size=(nprop, 3))
        # proposal coordinates are taken relative to the coordinates the
        # reference holds after its set-up wrap; the probe dumps those first,
        # so run it once without proposals, then build them.
        out0 = os.path.join(d, "out0")
        os.makedirs(out0)
        subprocess.check_call([probe, "in.conf", out0, "0"], cwd=d,
                              stdout=subprocess.DEVNULL)
        c0 = np.loadtxt(os.path.join(out0, "coords_init.txt")).reshape(-1, 3)
        props = np.empty((nprop, na, 3))
        for i, m in enumerate(props_m):
            a0 = int(sysm.mol_start[m])
            props[i] = np.mod(c0[a0:a0 + na] + shifts[i], sysm.box)
        with open(os.path.join(d, "props.txt"), "w") as f:
            f.write("%d\n" % nprop)
            for m, p in zip(props_m, props):
                f.write("%d %d %s\n" % (m, na, " ".join("%.17g" % v
                                                        for v in p.ravel())))
        # proposals and the Monte Carlo trace run in separate processes: the
        # proposal calls relink the cell lists, which would change the
        # summation order the trace starts from.
        outp = os.path.join(d, "outp")
        os.makedirs(outp)
        subprocess.check_call([probe, "in.conf", outp, "0", "props.txt"],
                              cwd=d, stdout=subprocess.DEVNULL)
        out = os.path.join(d, "out")
        os.makedirs(out)
        subprocess.check_call([probe, "in.conf", out, str(nsteps)], cwd=d,
                              stdout=subprocess.DEVNULL)

        def load(fn, **kw):
            p = os.path.join(out, fn)
            if not os.path.exists(p):
                p = os.path.join(outp, fn)
            return np.loadtxt(p, **kw) if os.path.exists(p) else None

        arrays = dict(
            pos=sysm.pos, box=sysm.box, atom_kind=sysm.atom_kind,
            atom_charge=sysm.atom_charge, mol_start=sysm.mol_start,
            kind_eps=np.array([k.epsilon for k in sysm.kinds]),
            kind_sigma=np.array([k.sigma for k in sysm.kinds]),
            kind_n=np.array([k.n for k in sysm.kinds]),
            coords_init=load("coords_init.txt"),
            com_init=load("com_init.txt"),
            cells=load("cells_box0.txt", skiprows=1, dtype=np.int64),
            prop_mol=props_m, prop_pos=props,
            prop_out=load("proposals_out.txt"),
            trace=load("trace.txt"),
            coords_final=load("coords_final.txt"),
            com_final=load("com_final.txt"),
        )
        kv = load("kvec.txt")
        if kv is not None:
            arrays["kvec"] = kv
        fa = load("forces_atom.txt")
        if fa is not None:
            arrays["forces_atom"] = fa
            arrays["forces_mol"] = load("forces_mol.txt")
        meta = dict(
            name=name,
            config=dict(temperature=cfg.temperature, rcut=cfg.rcut,
                        rcut_low=cfg.rcut_low, tolerance=cfg.tolerance,
                        ewald=cfg.ewald, electrostatic=cfg.electrostatic,
                        adj_steps=cfg.adj_steps, dis_freq=cfg.dis_freq,
                        rot_freq=cfg.rot_freq,
                        multi_particle_freq=cfg.multi_particle_freq,
                        random_seed=cfg.random_seed, nsteps=nsteps),
            kinds=[k.name for k in sysm.kinds],
            init=_energies(os.path.join(out, "energies_init.txt")),
            final=_energies(os.path.join(out, "energies_final.txt")),
        )
        if os.path.exists(os.path.join(out, "force_energy.txt")):
            meta["force_energy"] = _energies(os.path.join(out,
                                                          "force_energy.txt"))
        arrays["meta_json"] = np.frombuffer(json.dumps(meta).encode(),
                                            dtype=np.uint8)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **{
            k: v for k, v in arrays.items() if v is not None})
        print("wrote", name)


# soft-core settings of the SingleMoleculeInter vectors: ScaleAlpha,
# ScaleSigma, ScalePower (GOMC's defaults for free-energy runs)
SOFT_CORE = (0.5, 3.0, 2)


def make_single_mol(probe: str, name: str, n: int = 48) -> None:
    """SingleMoleculeInter (src/CalculateEnergy.cpp:1494-1556) of random
    molecules at random old/new lambda pairs, with and without soft-core
    Coulomb, on the fixture's initial state -> smi_<name>.npz."""
    builder, cfg, _, _ = FIXTURES[name]
    sysm = builder()
    rng = np.random.default_rng(2000 + len(name))
    mols = rng.integers(0, sysm.n_mol, size=n)
    lam = rng.uniform(0.0, 1.0, size=(n, 4))
    lam[::6] = 1.0                       # the lambda = 1 shortcut
    lam[1::6, :2] = 0.0                  # fully decoupled LJ
    lam[2::6, 1] = 0.9999995             # just inside the shortcut
    scc = (np.arange(n) % 2).astype(int)
    with tempfile.TemporaryDirectory() as d:
        write_reference_inputs(d, sysm, cfg)
        with open(os.path.join(d, "lam.txt"), "w") as f:
            f.write("%.17g %.17g %d\n%d\n" % (SOFT_CORE + (n,)))
            for m, l, c in zip(mols, lam, scc):
                f.write("%d %s %d\n" % (m, " ".join("%.17g" % v for v in l),
                                          c))
        out = os.path.join(d, "out")
        os.makedirs(out)
        subprocess.check_call([probe, "in.conf", out, "0", "-", "lam.txt"],
                              cwd=d, stdout=subprocess.DEVNULL)
        r = np.loadtxt(os.path.join(out, "single_mol_out.txt")).reshape(n, -1)
    np.savez_compressed(os.path.join(HERE, "smi_" + name + ".npz"),
                        mol=r[:, 0].astype(np.int64), lam=r[:, 1:5],
                        sc_coul=r[:, 5].astype(np.int64), out=r[:, 6:10],
                        soft_core=np.array(SOFT_CORE, dtype=np.float64))
    print("wrote smi_" + name)


def make_virial(probe: str, name: str) -> None:
    """CalculateEnergy::VirialCalc (src/CalculateEnergy.cpp:411-579) of the
    fixture's initial state -> vir_<name>.npz: out16 = inter, real, recip,
    total, then the xx/yy/zz diagonals of interTens, realTens, recipTens,
    totalTens."""
    builder, cfg, _, _ = FIXTURES[name]
    sysm = builder()
    with tempfile.TemporaryDirectory() as d:
        write_reference_inputs(d, sysm, cfg)
        out = os.path.join(d, "out")
        os.makedirs(out)
        subprocess.check_call([probe, "in.conf", out, "0"], cwd=d,
                              stdout=subprocess.DEVNULL)
        v = np.loadtxt(os.path.join(out, "virial.txt"))
    out16 = np.concatenate([v[0], v[1:, 0], v[1:, 1], v[1:, 2], v[1:, 3]])
    np.savez_compressed(os.path.join(HERE, "vir_" + name + ".npz"),
                        out16=out16)
    print("wrote vir_" + name)


def make_particles(probe: str, name: str, ncase: int = 24,
                   ntrials: int = 10) -> None:
    """CalculateEnergy::ParticleInter (src/CalculateEnergy.cpp:727-785), the
    CBMC first-atom trial energies, on the fixture's initial state ->
    pi_<name>.npz.  Two thirds of the cases take the molecule out of the cell
    list around the call, as MoleculeTransfer does before DCSingle builds the
    old and new trial sets (src/moves/MoleculeTransfer.h:100-106,
    src/cbmc/DCSingle.cpp:23-90), with trial 0 at the atom's own position
    (DCSingle::BuildOld); the rest call it on the full cell list at random
    positions.  Cases run in order in one process, so each removal and
    re-insertion relinks the molecule as the reference does."""
    builder, cfg, _, _ = FIXTURES[name]
    sysm = builder()
    z = np.load(os.path.join(HERE, name + ".npz"))
    c0 = z["coords_init"].reshape(-1, 3)
    rng = np.random.default_rng(3000 + len(name))
    ms = sysm.mol_start
    rows = []
    for i in range(ncase):
        m = int(rng.integers(0, sysm.n_mol))
        na = int(ms[m + 1] - ms[m])
        part = int(rng.integers(0, na))
        remove = int(i % 3 != 2)
        t = rng.uniform(0.0, 1.0, size=(ntrials, 3)) * sysm.box
        if remove:
            t[0] = c0[ms[m] + part]
        rows.append((m, part, remove, t))
    with tempfile.TemporaryDirectory() as d:
        write_reference_inputs(d, sysm, cfg)
        with open(os.path.join(d, "part.txt"), "w") as f:
            f.write("%d\n" % ncase)
            for m, part, remove, t in rows:
                f.write("%d %d %d %d %s\n" % (m, part, remove, ntrials,
                                             " ".join("%.17g" % v
                                                      for v in t.ravel())))
        out = os.path.join(d, "out")
        os.makedirs(out)
        subprocess.check_call([probe, "in.conf", out, "0", "-", "-",
                               "part.txt"], cwd=d, stdout=subprocess.DEVNULL)
        r = np.loadtxt(os.path.join(out, "particles_out.txt")).reshape(ncase,
                                                                       -1)
    res = r[:, 4:].reshape(ncase, ntrials, 3)
    np.savez_compressed(os.path.join(HERE, "pi_" + name + ".npz"),
                        mol=r[:, 0].astype(np.int64),
                        part=r[:, 1].astype(np.int64),
                        remove=r[:, 2].astype(np.int64),
                        trials=np.stack([t for _, _, _, t in rows]),
                        en=res[:, :, 0], real=res[:, :, 1],
                        overlap=res[:, :, 2].astype(np.int64))
    print("wrote pi_" + name)


PI_NAMES = ("c0_water", "w1728", "lj500", "c3_liquid", "c3_vapour",
            "c1_water")

# trial volume changes as fractions of the volume.  The reference's NVT
# build sizes its k-vector arrays for the initial box (no spare capacity), so
# the Ewald fixtures only shrink; ShiftVolume refuses edges below 2 Rcut.
VOLUME_FRACS = {"c0_water": (-0.004, -0.012), "w1728": (-0.01, -0.003),
                "lj500": (0.03, -0.025), "c3_liquid": (0.02, -0.015),
                "c3_vapour": (-0.05, 0.04)}


def make_volumes(probe: str, name: str) -> None:
    """The energy calls of a volume move (VolumeTransfer::Transform / CalcEn,
    src/moves/VolumeTransfer.h:96-190, NPT branch) on the fixture's initial
    state for each trial volume change, and the state after accepting the
    last one -> vol_<name>.npz: volume change, new edges, New k-vector count,
    BoxInter (LJ, real) and BoxReciprocal(box, true) of the trial, its
    coordinates and centres; then the accepted state's energies (inter,
    real, recip, self, correction, total) and k-vector count."""
    builder, cfg, _, _ = FIXTURES[name]
    sysm = builder()
    vol = float(np.prod(sysm.box))
    deltas = [f * vol for f in VOLUME_FRACS[name]]
    with tempfile.TemporaryDirectory() as d:
        write_reference_inputs(d, sysm, cfg)
        with open(os.path.join(d, "vol.txt"), "w") as f:
            f.write("%d\n%s\n" % (len(deltas),
                                   " ".join("%.17g" % v for v in deltas)))
        out = os.path.join(d, "out")
        os.makedirs(out)
        subprocess.check_call([probe, "in.conf", out, "0", "-", "-", "-",
                               "vol.txt"], cwd=d, stdout=subprocess.DEVNULL)
        r = np.loadtxt(os.path.join(out, "volume_out.txt")).reshape(
            len(deltas), -1)
        pos = np.stack([np.loadtxt(os.path.join(out, "volume_pos_%d.txt" % i))
                        for i in range(len(deltas))])
        com = np.stack([np.loadtxt(os.path.join(out, "volume_com_%d.txt" % i))
                        .reshape(-1, 3) for i in range(len(deltas))])
        acc = _energies(os.path.join(out, "volume_accept.txt"))
    np.savez_compressed(
        os.path.join(HERE, "vol_" + name + ".npz"), delta=r[:, 0],
        edges=r[:, 1:4], k_new=r[:, 4].astype(np.int64), inter=r[:, 5],
        real=r[:, 6], recip=r[:, 7], pos=pos, com=com,
        accepted=np.array([acc["box0_" + t] for t in
                           ("inter", "real", "recip", "self", "correction",
                            "total")]),
        accepted_k=np.int64(acc.get("imageSize", 0)))
    print("wrote vol_" + name)


# The Gibbs-ensemble configuration: LJ spheres (eps/kB 148 K, sigma 3.73 A,
# Rcut 12 A) at 150 K, the liquid box of c3_liquid (2,400 in 40 A) and the
# vapour box of c3_vapour (300 in 90 A), displacement / volume exchange /
# molecule swap 0.8 / 0.01 / 0.19, 10 CBMC trials
GEMC = dict(temperature=150.0, rcut=12.0, random_seed=3333, dis_freq=0.8,
            vol_freq=0.01, swap_freq=0.19, adj_steps=100, cbmc_first=10)
GEMC_STEPS = 6000


def make_gemc(ref: str, name: str = "c3_gemc") -> None:
    """A reference GEMC NVT trace (probe built with ENSEMBLE=GEMC) ->
    c3_gemc.npz: the two boxes as generated, the initial energies, the
    per-step trace, and the final coordinates, centres, molecule lookup,
    energies and move settings."""
    subprocess.check_call(["make", "-s", "-f", os.path.join(ROOT, "oracle",
                                                             "ref.mk"),
                           "REF=" + ref, "OUT=" + os.path.join(ROOT, "oracle",
                                                               "_ref"),
                           "ENSEMBLE=2", "-j8"], cwd=ROOT)
    probe = os.path.join(ROOT, "oracle", "_ref", "ref_probe_ens2")
    s0 = FIXTURES["c3_liquid"][0]()
    s1 = FIXTURES["c3_vapour"][0]()
    with tempfile.TemporaryDirectory() as d:
        write_gemc_inputs(d, s0, s1, run_steps=GEMC_STEPS,
                          eq_steps=GEMC_STEPS // 2, **GEMC)
        out = os.path.join(d, "out")
        os.makedirs(out)
        subprocess.check_call([probe, "in.conf", out, str(GEMC_STEPS)],
                              cwd=d, stdout=subprocess.DEVNULL)

        def ld(fn, **kw):
            return np.loadtxt(os.path.join(out, fn), **kw)
        init, fin = {}, {}
        for line in open(os.path.join(out, "energies_init.txt")):
            t = line.split()
            if len(t) == 3:
                init[t[0] + "_" + t[1]] = float(t[2])
        settings, axes = [], []
        for line in open(os.path.join(out, "energies_final.txt")):
            t = line.split()
            if len(t) == 3:
                fin[t[0] + "_" + t[1]] = float(t[2])
            elif t and t[0] == "axis":
                axes.append([float(v) for v in t[2:5]])
            elif t and t[0] == "settings":
                settings.append([float(v) for v in t[1:]])
        with open(os.path.join(out, "lookup_final.txt")) as fh:
            lk = [np.array(line.split(), dtype=np.int64) for line in fh]
        lk = [lk[0], np.concatenate(lk[1:])]
        arrays = dict(
            pos0=s0.pos, pos1=s1.pos, box0=s0.box, box1=s1.box,
            kind_eps=np.array([s0.kinds[0].epsilon]),
            kind_sigma=np.array([s0.kinds[0].sigma]),
            kind_n=np.array([s0.kinds[0].n]),
            coords_init=ld("coords_init.txt"), trace=ld("trace.txt"),
            coords_final=ld("coords_final.txt"),
            com_final=ld("com_final.txt"),
            lookup_counts=lk[0], lookup_final=lk[1],
            axes_final=np.array(axes), settings_final=np.array(settings))
        meta = dict(name=name, gemc=GEMC, steps=GEMC_STEPS,
                    init=init, final=fin)
        arrays["meta_json"] = np.frombuffer(json.dumps(meta).encode(),
                                            dtype=np.uint8)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
        print("wrote", name)


# checkpoint fixture: the reference's own checkpoint file after CHK_STEP of
# CHK_TOTAL steps of c0_water's Monte Carlo loop, with the state it holds
CHK_STEP, CHK_TOTAL = 600, 1000


def _chk_state(path):
    """chk_state.txt of the probe: steps, MT19937 save array and seeds,
    per-move settings of box 0 / kind 0, MultiParticle counters."""
    with open(path) as f:
        lines = [ln.split() for ln in f]
    steps = np.array([int(v) for v in lines[0]], dtype=np.uint64)
    mt = np.array([int(lines[1 + i][0]) for i in range(625)], dtype=np.uint64)
    seeds = np.array([int(v) for v in lines[626]], dtype=np.uint64)
    nm = int(lines[627][0])
    moves = np.array([[float(v) for v in lines[628 + m]] for m in range(nm)])
    mp = np.array([[int(v) for v in ln] for ln in lines[628 + nm:630 + nm]],
                  dtype=np.uint64)
    mpmax = np.array([float(v) for v in lines[630 + nm]])
    return dict(chk_steps=steps, chk_mt=mt, chk_seeds=seeds, chk_moves=moves,
                chk_mp=mp, chk_mpmax=mpmax)


def make_checkpoint(probe: str, name: str = "c0_water") -> None:
    """The reference's checkpoint file (CheckpointOutput) after CHK_STEP
    steps, the coordinates and loop state it belongs to, and the trace of
    the whole CHK_TOTAL-step run, so that a box handed that state continues
    the reference's run."""
    builder, cfg, _, _ = FIXTURES[name]
    sysm = builder()
    with tempfile.TemporaryDirectory() as d:
        write_reference_inputs(d, sysm, cfg)
        out = os.path.join(d, "out")
        os.makedirs(out)
        env = dict(os.environ, GOMC_PROBE_CHK_STEP=str(CHK_STEP))
        subprocess.check_call([probe, "in.conf", out, str(CHK_TOTAL)], cwd=d,
                              env=env, stdout=subprocess.DEVNULL)
        with open(os.path.join(out, "restart.chk"), "rb") as f:
            chk = np.frombuffer(f.read(), dtype=np.uint8)
        arrays = dict(chk=chk,
                      coords_chk=np.loadtxt(os.path.join(out, "coords_chk.txt")),
                      com_chk=np.loadtxt(os.path.join(out, "com_chk.txt")),
                      trace=np.loadtxt(os.path.join(out, "trace.txt")),
                      coords_final=np.loadtxt(os.path.join(out,
                                                           "coords_final.txt")),
                      **_chk_state(os.path.join(out, "chk_state.txt")))
        meta = dict(name=name, chk_step=CHK_STEP, total=CHK_TOTAL,
                    final=_energies(os.path.join(out, "energies_final.txt")))
        arrays["meta_json"] = np.frombuffer(json.dumps(meta).encode(),
                                            dtype=np.uint8)
        np.savez_compressed(os.path.join(HERE, "chk_" + name + ".npz"),
                            **arrays)
        print("wrote chk_" + name)


def make_kat(probe: str) -> None:
    """Known-answer vectors of the reference's MT19937 and Philox4x64-10."""
    with tempfile.TemporaryDirectory() as d:
        subprocess.check_call([probe, "--kat", d], stdout=subprocess.DEVNULL)
        mt = np.loadtxt(os.path.join(d, "kat_mt.txt"), dtype=np.uint64)
        ph = np.loadtxt(os.path.join(d, "kat_philox.txt"), dtype=np.float64,
                        usecols=range(7, 13))
        phi = np.loadtxt(os.path.join(d, "kat_philox.txt"), dtype=np.uint64,
                         usecols=range(0, 7))
        np.savez_compressed(os.path.join(HERE, "kat_rng.npz"), mt=mt,
                            philox_int=phi, philox_real=ph)
        print("wrote kat_rng")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("GOMC_REFERENCE"))
    ap.add_argument("--only", choices=("particles", "volumes", "gemc",
                                       "checkpoint"),
                    default=None,
                    help="only the ParticleInter, volume-move or GEMC vectors")
    ap.add_argument("names", nargs="*")
    a = ap.parse_args()
    if not a.ref or not os.path.isdir(os.path.join(a.ref, "src")):
        ap.error("give the reference source tree with --ref or GOMC_REFERENCE")
    probe = build_reference(a.ref)
    if a.only == "particles":
        for n in (a.names or PI_NAMES):
            make_particles(probe, n)
        return
    if a.only == "gemc":
        make_gemc(a.ref)
        return
    if a.only == "checkpoint":
        make_checkpoint(probe)
        return
    if a.only == "volumes":
        for n in (a.names or list(VOLUME_FRACS)):
            make_volumes(probe, n)
        return
    if not a.names:
        make_kat(probe)
    for n in (a.names or list(FIXTURES)):
        make_one(probe, n)
    for n in ("c0_water", "w1728", "lj500"):
        if not a.names or n in a.names:
            make_single_mol(probe, n)
    for n in (a.names or list(FIXTURES)):
        make_virial(probe, n)
    for n in PI_NAMES:
        if not a.names or n in a.names:
            make_particles(probe, n)
    for n in VOLUME_FRACS:
        if not a.names or n in a.names:
            make_volumes(probe, n)
    if not a.names or "c3_gemc" in a.names:
        make_gemc(a.ref)
    if not a.names:
        make_checkpoint(probe)


if __name__ == "__main__":
    main()
