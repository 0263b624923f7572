"""Loading the committed golden vectors (tests/golden/*.npz)."""
import json
import os

import numpy as np

from gomc_gb300.config import SimConfig
from gomc_gb300.systems import AtomKind, MoleculeType, MolSystem

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = ["c0_water", "c0_water_mp", "w1728", "lj500", "c3_liquid", "c3_vapour",
         "c1_water", "c1_water_mp"]
# fixtures of the 8,000-water system: the oracle takes tens of seconds per
# full structure factor on one core, so its CPU tests cover them in part
LARGE = ("c1_water", "c1_water_mp")


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(bytes(z["meta_json"]).decode())
    return z, meta


def system_of(z, meta):
    kinds = [AtomKind(n, float(e), float(s), float(x)) for n, e, s, x in
             zip(meta["kinds"], z["kind_eps"], z["kind_sigma"], z["kind_n"])]
    ms = z["mol_start"].astype(np.int32)
    n_mol = len(ms) - 1
    na = int(ms[1] - ms[0])
    mt = MoleculeType("MOL", ["A%d" % i for i in range(na)],
                      list(z["atom_kind"][:na]), list(z["atom_charge"][:na]))
    atom_mol = np.repeat(np.arange(n_mol, dtype=np.int32), np.diff(ms))
    return MolSystem(box=z["box"].astype(np.float64), kinds=kinds,
                     mol_types=[mt], pos=z["pos"].astype(np.float64),
                     atom_kind=z["atom_kind"].astype(np.int32),
                     atom_charge=z["atom_charge"].astype(np.float64),
                     atom_mol=atom_mol, mol_start=ms,
                     mol_type=np.zeros(n_mol, np.int32))


def config_of(meta):
    c = meta["config"]
    return SimConfig(temperature=c["temperature"], rcut=c["rcut"],
                     rcut_low=c["rcut_low"], tolerance=c["tolerance"],
                     ewald=c["ewald"], electrostatic=c["electrostatic"],
                     adj_steps=c["adj_steps"], eq_steps=max(c["adj_steps"], 1),
                     dis_freq=c["dis_freq"], rot_freq=c["rot_freq"],
                     multi_particle_freq=c["multi_particle_freq"],
                     random_seed=c["random_seed"])


def move_fractions(meta):
    c = meta["config"]
    return [c["dis_freq"], c["rot_freq"], c["multi_particle_freq"]]


SMI_NAMES = ["c0_water", "w1728", "lj500"]


def load_smi(name):
    """SingleMoleculeInter vectors of fixture `name` (the reference's
    CalculateEnergy::SingleMoleculeInter on the fixture's initial state):
    molecule, lambdas (old VDW, new VDW, old Coulomb, new Coulomb), sc_coul,
    outputs (old inter, old real, new inter, new real) and the soft-core
    settings (ScaleAlpha, ScaleSigma, ScalePower)."""
    return np.load(os.path.join(GOLDEN, "smi_" + name + ".npz"))


def load_virial(name):
    """The reference's CalculateEnergy::VirialCalc of fixture `name`'s
    initial state: inter, real, recip, total, then the xx/yy/zz diagonals of
    interTens, realTens, recipTens, totalTens."""
    return np.load(os.path.join(GOLDEN, "vir_" + name + ".npz"))["out16"]


PI_NAMES = ["c0_water", "w1728", "lj500", "c3_liquid", "c3_vapour", "c1_water"]


def load_pi(name):
    """ParticleInter vectors of fixture `name` (the reference's
    CalculateEnergy::ParticleInter on the fixture's initial state, cases in
    order): molecule, atom within it, whether the molecule was taken out of
    the cell list around the call, trial positions [case, trial, 3], and the
    outputs en, real, overlap [case, trial]."""
    return np.load(os.path.join(GOLDEN, "pi_" + name + ".npz"))


def load_gemc(name="c3_gemc"):
    """The reference's GEMC NVT run of the LJ-sphere configuration: both
    boxes as generated (pos0/pos1, box0/box1), the Mie parameters, the
    per-step trace (step, move kind, box, molecule, accepted, running inter
    energies of both boxes, volumes of both boxes, molecules in box 0, four
    move values) and the final coordinates, centres, molecule lookup, axes
    and move settings; meta holds the configuration and energies."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(bytes(z["meta_json"]).decode())
    return z, meta
