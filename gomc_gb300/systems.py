"""Molecular systems for the Monte Carlo energy path.

A :class:`MolSystem` holds what the reference keeps in ``Molecules``,
``MoleculeKind``, ``Coordinates`` and ``FFParticle`` for one box
(src/Molecules.h, src/MoleculeKind.h, src/FFParticle.cpp:56-200): atom
positions, per-atom kind / charge / molecule, molecule start offsets, the Mie
parameters of every atom kind, and the box edge lengths.

Generators build the seeded synthetic systems used for testing and measuring:

* :func:`spce_water_box` -- rigid 3-site SPC/E-geometry water (O q=-0.8476e,
  H q=+0.4238e, O-H 1.0 A, H-O-H 109.47 deg, LJ on O only with
  eps/kB = 78.2 K and sigma = 3.166 A), O on a cubic lattice, uniformly random
  orientations.
* :func:`lj_sphere_box` -- single-site LJ particles at seeded random
  positions with a minimum pair separation.

Writers emit the reference's input formats (PDB, PSF, Mie-style parameter
file and ``in.conf``) so that the reference program can load the same system;
coordinates are rounded to the PDB's three decimals before either side sees
them, so both read bit-identical doubles.
"""
from __future__ import annotations

import dataclasses
import math
import os
from typing import List, Optional, Sequence, Tuple

import numpy as np

# Energy units are Kelvin throughout, as in the reference (src/FFSetup.cpp:25).
QQ_FACT = 167103.208067979  # K*A/e^2, lib/NumLib.h:22


@dataclasses.dataclass
class AtomKind:
    """One NONBONDED_MIE entry: name, eps (K), sigma (A), repulsion exponent."""

    name: str
    epsilon: float
    sigma: float
    n: float = 12.0
    mass: float = 1.0


@dataclasses.dataclass
class MoleculeType:
    """A rigid molecule kind: residue name, atoms, bonds and angles (PSF)."""

    name: str
    atom_names: List[str]
    atom_kinds: List[int]
    charges: List[float]
    bonds: List[Tuple[int, int]] = dataclasses.field(default_factory=list)
    angles: List[Tuple[int, int, int]] = dataclasses.field(default_factory=list)
    bond_lengths: List[float] = dataclasses.field(default_factory=list)
    angle_degrees: List[float] = dataclasses.field(default_factory=list)


@dataclasses.dataclass
class MolSystem:
    """One periodic orthogonal box of rigid molecules."""

    box: np.ndarray                 # (3,) edge lengths, A
    kinds: List[AtomKind]
    mol_types: List[MoleculeType]
    pos: np.ndarray                 # (N, 3) float64
    atom_kind: np.ndarray           # (N,) int32
    atom_charge: np.ndarray         # (N,) float64
    atom_mol: np.ndarray            # (N,) int32
    mol_start: np.ndarray           # (M + 1,) int32
    mol_type: np.ndarray            # (M,) int32

    @property
    def n_atoms(self) -> int:
        return int(self.pos.shape[0])

    @property
    def n_mol(self) -> int:
        return int(self.mol_type.shape[0])

    @property
    def volume(self) -> float:
        return float(self.box[0] * self.box[1] * self.box[2])

    def copy(self) -> "MolSystem":
        return dataclasses.replace(
            self,
            box=self.box.copy(),
            pos=self.pos.copy(),
            atom_kind=self.atom_kind.copy(),
            atom_charge=self.atom_charge.copy(),
            atom_mol=self.atom_mol.copy(),
            mol_start=self.mol_start.copy(),
            mol_type=self.mol_type.copy(),
        )


def _round3(a: np.ndarray) -> np.ndarray:
    """Round to the PDB's %8.3f text and read it back (correctly rounded)."""
    flat = [float("%.3f" % v) for v in np.asarray(a, dtype=np.float64).ravel()]
    return np.array(flat, dtype=np.float64).reshape(np.shape(a))


def _random_rotations(rng: np.random.Generator, n: int) -> np.ndarray:
    """Uniform random rotation matrices from uniform unit quaternions."""
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    r = np.empty((n, 3, 3))
    r[:, 0, 0] = 1 - 2 * (y * y + z * z)
    r[:, 0, 1] = 2 * (x * y - z * w)
    r[:, 0, 2] = 2 * (x * z + y * w)
    r[:, 1, 0] = 2 * (x * y + z * w)
    r[:, 1, 1] = 1 - 2 * (x * x + z * z)
    r[:, 1, 2] = 2 * (y * z - x * w)
    r[:, 2, 0] = 2 * (x * z - y * w)
    r[:, 2, 1] = 2 * (y * z + x * w)
    r[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return r


SPCE_KINDS = [AtomKind("OW", 78.2, 3.166, 12.0, 15.9994),
              AtomKind("HW", 0.0, 0.0, 12.0, 1.008)]
SPCE_TYPE = MoleculeType(
    name="SPC",
    atom_names=["O", "H1", "H2"],
    atom_kinds=[0, 1, 1],
    charges=[-0.8476, 0.4238, 0.4238],
    bonds=[(0, 1), (0, 2)],
    angles=[(1, 0, 2)],
    bond_lengths=[1.0],
    angle_degrees=[109.47],
)


def water_box_length(n_mol: int, density_g_cm3: float = 1.0) -> float:
    """Cubic edge (A) holding n_mol waters at the given mass density."""
    mass_g = n_mol * 18.01528 / 6.02214076e23
    vol_a3 = mass_g / density_g_cm3 * 1e24
    return vol_a3 ** (1.0 / 3.0)


def spce_water_box(n_mol: int, box_len: float, seed: int,
                   lattice: Optional[int] = None) -> MolSystem:
    """SPC/E-geometry waters with O on a seeded cubic lattice.

    O sits at lattice site centres ``(i + 0.5) * L / n`` (x outer, z inner,
    first ``n_mol`` sites of an ``n^3`` lattice); each molecule gets a
    uniformly random orientation.  Positions are wrapped into ``[0, L)`` and
    rounded to three decimals.
    """
    n = lattice or int(math.ceil(n_mol ** (1.0 / 3.0) - 1e-9))
    if n ** 3 < n_mol:
        raise ValueError("lattice too small for %d molecules" % n_mol)
    rng = np.random.default_rng(seed)
    spacing = box_len / n
    idx = np.arange(n_mol)
    ix, iy, iz = idx // (n * n), (idx // n) % n, idx % n
    o = np.stack([(ix + 0.5) * spacing, (iy + 0.5) * spacing,
                  (iz + 0.5) * spacing], axis=1)
    half = math.radians(109.47) / 2.0
    local = np.array([[0.0, 0.0, 0.0],
                      [math.sin(half), math.cos(half), 0.0],
                      [-math.sin(half), math.cos(half), 0.0]])
    rot = _random_rotations(rng, n_mol)
    pos = o[:, None, :] + np.einsum("mij,aj->mai", rot, local)
    pos = pos.reshape(-1, 3)
    pos = np.mod(pos, box_len)
    pos = _round3(pos)
    pos[pos >= box_len] -= box_len  # a value that rounded up to L
    n_atoms = 3 * n_mol
    return MolSystem(
        box=np.array([box_len] * 3, dtype=np.float64),
        kinds=list(SPCE_KINDS),
        mol_types=[SPCE_TYPE],
        pos=pos,
        atom_kind=np.tile(np.array(SPCE_TYPE.atom_kinds, np.int32), n_mol),
        atom_charge=np.tile(np.array(SPCE_TYPE.charges, np.float64), n_mol),
        atom_mol=np.repeat(np.arange(n_mol, dtype=np.int32), 3),
        mol_start=np.arange(0, n_atoms + 1, 3, dtype=np.int32),
        mol_type=np.zeros(n_mol, dtype=np.int32),
    )


def lj_sphere_box(n: int, box_len: float, seed: int, epsilon: float,
                  sigma: float, min_sep: float, name: str = "LJ",
                  mass: float = 39.948) -> MolSystem:
    """Single-site LJ particles at seeded random positions, no pair closer
    than ``min_sep`` (A) under the minimum image."""
    rng = np.random.default_rng(seed)
    pts: List[np.ndarray] = []
    tries = 0
    arr = np.empty((0, 3))
    while len(pts) < n:
        tries += 1
        if tries > 200 * n + 10000:
            raise RuntimeError("could not place %d particles" % n)
        p = _round3(rng.random(3) * box_len)
        p[p >= box_len] -= box_len
        if arr.shape[0]:
            d = arr - p
            d -= box_len * np.round(d / box_len)
            if np.min(np.einsum("ij,ij->i", d, d)) < min_sep * min_sep:
                continue
        pts.append(p)
        arr = np.asarray(pts)
    mt = MoleculeType(name=name[:3].upper(), atom_names=[name[:2].upper()],
                      atom_kinds=[0], charges=[0.0])
    return MolSystem(
        box=np.array([box_len] * 3, dtype=np.float64),
        kinds=[AtomKind(name[:2].upper(), epsilon, sigma, 12.0, mass)],
        mol_types=[mt],
        pos=arr.astype(np.float64),
        atom_kind=np.zeros(n, np.int32),
        atom_charge=np.zeros(n, np.float64),
        atom_mol=np.arange(n, dtype=np.int32),
        mol_start=np.arange(n + 1, dtype=np.int32),
        mol_type=np.zeros(n, np.int32),
    )


# ---------------------------------------------------------------------------
# Writers for the reference's input formats
# ---------------------------------------------------------------------------

def write_pdb(path: str, sysm: MolSystem) -> None:
    with open(path, "w") as f:
        f.write("REMARK generated seeded system\n")
        f.write("CRYST1%9.3f%9.3f%9.3f  90.00  90.00  90.00 P 1           1\n"
                % tuple(sysm.box))
        a = 0
        for m in range(sysm.n_mol):
            mt = sysm.mol_types[int(sysm.mol_type[m])]
            for j, nm in enumerate(mt.atom_names):
                x, y, z = sysm.pos[a]
                f.write("ATOM  %5d %-4s %-4s%1s%4d    %8.3f%8.3f%8.3f%6.2f%6.2f"
                        "      %-4s%2s\n" % ((a + 1) % 100000, nm, mt.name, "A",
                                             (m + 1) % 10000, x, y, z, 0.0, 0.0,
                                             mt.name, nm[0]))
                a += 1
        f.write("END\n")


def write_psf(path: str, sysm: MolSystem) -> None:
    lines = ["PSF", "", "       1 !NTITLE", " REMARKS generated seeded system",
             ""]
    lines.append("%8d !NATOM" % sysm.n_atoms)
    a = 0
    bonds: List[Tuple[int, int]] = []
    angles: List[Tuple[int, int, int]] = []
    for m in range(sysm.n_mol):
        mt = sysm.mol_types[int(sysm.mol_type[m])]
        base = a
        for j, nm in enumerate(mt.atom_names):
            kind = sysm.kinds[mt.atom_kinds[j]]
            lines.append("%8d %-4s %-4d %-4s %-4s %-4s %10.6f %13.4f %11d" % (
                a + 1, "A", m + 1, mt.name, nm, kind.name, mt.charges[j],
                kind.mass, 0))
            a += 1
        bonds += [(base + i + 1, base + j + 1) for i, j in mt.bonds]
        angles += [(base + i + 1, base + j + 1, base + k + 1)
                   for i, j, k in mt.angles]
    lines.append("")
    lines.append("%8d !NBOND: bonds" % len(bonds))
    row = ""
    for i, (p, q) in enumerate(bonds):
        row += "%8d%8d" % (p, q)
        if i % 4 == 3:
            lines.append(row)
            row = ""
    if row:
        lines.append(row)
    lines.append("")
    lines.append("%8d !NTHETA: angles" % len(angles))
    row = ""
    for i, (p, q, r) in enumerate(angles):
        row += "%8d%8d%8d" % (p, q, r)
        if i % 3 == 2:
            lines.append(row)
            row = ""
    if row:
        lines.append(row)
    lines.append("")
    for tag in ("!NPHI: dihedrals", "!NIMPHI: impropers", "!NDON: donors",
                "!NACC: acceptors"):
        lines += ["%8d %s" % (0, tag), "", ""]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_mie_par(path: str, sysm: MolSystem) -> None:
    """Mie-style (EXOTIC) parameter file; bonds and angles are FIXED."""
    lines = ["* generated parameters", "", "BONDS"]
    seen = set()
    for mt in sysm.mol_types:
        for (i, j), b0 in zip(mt.bonds, mt.bond_lengths * len(mt.bonds)):
            key = tuple(sorted((sysm.kinds[mt.atom_kinds[i]].name,
                                sysm.kinds[mt.atom_kinds[j]].name)))
            if key not in seen:
                seen.add(key)
                lines.append("%-6s %-6s 999999999999 %8.4f" % (key[0], key[1], b0))
    lines += ["", "ANGLES"]
    seen = set()
    for mt in sysm.mol_types:
        for (i, j, k), th in zip(mt.angles, mt.angle_degrees * len(mt.angles)):
            names = (sysm.kinds[mt.atom_kinds[i]].name,
                     sysm.kinds[mt.atom_kinds[j]].name,
                     sysm.kinds[mt.atom_kinds[k]].name)
            if names not in seen:
                seen.add(names)
                lines.append("%-6s %-6s %-6s 999999999999 %8.3f" % (names + (th,)))
    lines += ["", "DIHEDRALS", "", "NONBONDED_MIE"]
    for k in sysm.kinds:
        lines.append("%-6s %10.4f %10.4f %6.1f" % (k.name, k.epsilon, k.sigma, k.n))
    lines += ["", "END"]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_inconf(path: str, sysm: MolSystem, cfg, names: Tuple[str, str, str]) -> None:
    """``in.conf`` for the reference NVT program from a :class:`SimConfig`."""
    pdb, psf, par = names
    L = sysm.box
    rows = [
        ("Restart", "false"), ("ExpertMode", "true"), ("PRNG", "INTSEED"),
        ("Random_Seed", str(cfg.random_seed)), ("ParaTypeCHARMM", "off"),
        ("ParaTypeEXOTIC", "on"), ("Parameters", par),
        ("Coordinates 0", pdb), ("Structure 0", psf),
        ("Temperature", repr(cfg.temperature)), ("Potential", "VDW"),
        ("LRC", "true" if cfg.lrc else "false"), ("Rcut", repr(cfg.rcut)),
        ("RcutLow", repr(cfg.rcut_low)), ("Exclude", "1-4"),
        ("Ewald", "true" if cfg.ewald else "false"),
        ("ElectroStatic", "true" if cfg.electrostatic else "false"),
    ]
    if cfg.ewald:
        rows.append(("Tolerance", repr(cfg.tolerance)))
    rows += [
        ("CachedFourier", "false"),
        ("RunSteps", str(cfg.run_steps)), ("EqSteps", str(cfg.eq_steps)),
        ("AdjSteps", str(cfg.adj_steps)),
        ("DisFreq", repr(cfg.dis_freq)), ("RotFreq", repr(cfg.rot_freq)),
        ("CBMC_First", "10"), ("CBMC_Nth", "4"), ("CBMC_Ang", "50"),
        ("CBMC_Dih", "20"),
    ]
    if cfg.multi_particle_freq > 0:
        rows.append(("MultiParticleFreq", repr(cfg.multi_particle_freq)))
    rows += [
        ("CellBasisVector1 0", "%r 0.00 0.00" % float(L[0])),
        ("CellBasisVector2 0", "0.00 %r 0.00" % float(L[1])),
        ("CellBasisVector3 0", "0.00 0.00 %r" % float(L[2])),
        ("OutputName", "out"), ("CoordinatesFreq", "false 1000000"),
        ("RestartFreq", "false 1000000"), ("CheckpointFreq", "false 1000000"),
        ("ConsoleFreq", "true 1000000"), ("BlockAverageFreq", "false 1000000"),
        ("DCDFreq", "false 1000000"),
        ("OutEnergy", "true true"), ("OutPressure", "false false"),
        ("OutMolNum", "false false"), ("OutDensity", "false false"),
        ("PressureCalc", "false"),
    ]
    with open(path, "w") as f:
        for k, v in rows:
            f.write("%-20s %s\n" % (k, v))


def write_reference_inputs(dirpath: str, sysm: MolSystem, cfg) -> str:
    """Write PDB/PSF/parameter/in.conf into ``dirpath``; return in.conf path."""
    os.makedirs(dirpath, exist_ok=True)
    names = ("system.pdb", "system.psf", "system.par")
    write_pdb(os.path.join(dirpath, names[0]), sysm)
    write_psf(os.path.join(dirpath, names[1]), sysm)
    write_mie_par(os.path.join(dirpath, names[2]), sysm)
    conf = os.path.join(dirpath, "in.conf")
    write_inconf(conf, sysm, cfg, names)
    return conf


def write_gemc_inputs(dirpath: str, box0: MolSystem, box1: MolSystem, *,
                      temperature: float, rcut: float, random_seed: int,
                      dis_freq: float, vol_freq: float, swap_freq: float,
                      run_steps: int, eq_steps: int, adj_steps: int,
                      cbmc_first: int = 10, rcut_low: float = 0.0) -> str:
    """Inputs of a two-box NVT Gibbs-ensemble run of the reference (GEMC
    NVT: one PDB / PSF per box, ``Coordinates 0/1``, ``Structure 0/1``,
    ``CellBasisVector*`` of both boxes, ``DisFreq`` / ``VolFreq`` /
    ``SwapFreq``), LJ particles without charges; returns the in.conf path.
    The two systems share one molecule and atom kind."""
    os.makedirs(dirpath, exist_ok=True)
    for b, s in enumerate((box0, box1)):
        write_pdb(os.path.join(dirpath, "box%d.pdb" % b), s)
        write_psf(os.path.join(dirpath, "box%d.psf" % b), s)
    write_mie_par(os.path.join(dirpath, "system.par"), box0)
    rows = [
        ("Restart", "false"), ("ExpertMode", "true"), ("PRNG", "INTSEED"),
        ("Random_Seed", str(random_seed)), ("ParaTypeCHARMM", "off"),
        ("ParaTypeEXOTIC", "on"), ("Parameters", "system.par"),
        ("Coordinates 0", "box0.pdb"), ("Coordinates 1", "box1.pdb"),
        ("Structure 0", "box0.psf"), ("Structure 1", "box1.psf"),
        ("GEMC", "NVT"), ("Temperature", repr(temperature)),
        ("Potential", "VDW"), ("LRC", "false"), ("Rcut", repr(rcut)),
        ("RcutLow", repr(rcut_low)), ("Exclude", "1-4"), ("Ewald", "false"),
        ("ElectroStatic", "false"), ("CachedFourier", "false"),
        ("RunSteps", str(run_steps)), ("EqSteps", str(eq_steps)),
        ("AdjSteps", str(adj_steps)), ("DisFreq", repr(dis_freq)),
        ("VolFreq", repr(vol_freq)), ("SwapFreq", repr(swap_freq)),
        ("CBMC_First", str(cbmc_first)), ("CBMC_Nth", "4"),
        ("CBMC_Ang", "50"), ("CBMC_Dih", "20"),
    ]
    for b, s in enumerate((box0, box1)):
        L = s.box
        rows += [("CellBasisVector1 %d" % b, "%r 0.00 0.00" % float(L[0])),
                 ("CellBasisVector2 %d" % b, "0.00 %r 0.00" % float(L[1])),
                 ("CellBasisVector3 %d" % b, "0.00 0.00 %r" % float(L[2]))]
    rows += [
        ("OutputName", "out"), ("CoordinatesFreq", "false 1000000"),
        ("RestartFreq", "false 1000000"), ("CheckpointFreq", "false 1000000"),
        ("ConsoleFreq", "true 1000000"), ("BlockAverageFreq", "false 1000000"),
        ("DCDFreq", "false 1000000"), ("OutEnergy", "true true"),
        ("OutPressure", "false false"), ("OutMolNum", "false false"),
        ("OutDensity", "false false"), ("PressureCalc", "false"),
    ]
    conf = os.path.join(dirpath, "in.conf")
    with open(conf, "w") as f:
        for k, v in rows:
            f.write("%-20s %s\n" % (k, v))
    return conf
