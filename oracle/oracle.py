"""ctypes wrapper of the C oracle (gomc_oracle.c) -- TEST INFRASTRUCTURE.

Only tests, the smoke check and the CPU-baseline leg of the benchmark import
this module, as the checker.  ``build()`` compiles the C restatement with
``-ffp-contract=off`` so that x86-64 and aarch64 hosts evaluate the same
expressions in the same IEEE order.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_lib = None


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "gomc_oracle.c")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src)):
        return LIB_PATH
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    tmp = LIB_PATH + ".%d.tmp" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC",
                           "-shared", "-fopenmp", src, "-o", tmp, "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P, I, D, U32, U64 = C.c_void_p, C.c_int, C.c_double, C.c_uint32, C.c_uint64
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        lp = C.POINTER(C.c_long)
        sig = {
            "ora_create": (P, [I, I, dp, ip, dp, ip, I, dp, dp, dp, dp, D, D, D,
                               D, I, I, D]),
            "ora_destroy": (None, [P]),
            "ora_set_threads": (None, [I]),
            "ora_num_k": (I, [P]),
            "ora_num_cells": (I, [P]),
            "ora_get_coords": (None, [P, dp]),
            "ora_get_com": (None, [P, dp]),
            "ora_set_coords": (None, [P, dp, dp]),
            "ora_get_kvec": (None, [P, dp]),
            "ora_get_sum_new": (None, [P, dp, dp]),
            "ora_get_cells": (None, [P, ip, ip]),
            "ora_get_energy": (None, [P, dp]),
            "ora_set_energy": (None, [P, dp]),
            "ora_system_total": (None, [P, dp]),
            "ora_grid_all": (None, [P]),
            "ora_molecule_inter": (I, [P, I, dp, dp, dp]),
            "ora_virial": (None, [P, dp]),
            "ora_single_molecule_inter": (None, [P, I, dp,
                                                 C.POINTER(SoftCore), dp]),
            "ora_particle_inter": (I, [P, I, I, dp, dp, dp]),
            "ora_cell_remove_mol": (None, [P, I]),
            "ora_cell_add_mol": (None, [P, I]),
            "ora_mol_reciprocal": (D, [P, dp, I]),
            "ora_swap_dest_recip": (D, [P, dp, I]),
            "ora_swap_source_recip": (D, [P, dp, I]),
            "ora_update_recip": (None, [P]),
            "ora_copy_recip": (None, [P]),
            "ora_box_self": (D, [P]),
            "ora_mol_correction": (D, [P, I]),
            "ora_box_force": (None, [P, dp, dp, dp, dp, dp]),
            "ora_box_reciprocal_sums": (D, [P, dp]),
            "ora_box_force_recip": (None, [P, dp, dp, dp]),
            "ora_torque": (None, [P, dp, dp, dp, dp, dp]),
            "ora_gemc_create": (P, [I, dp, I, dp, dp, dp, D, D, D, D, D, D,
                                    U32, dp, I, I]),
            "ora_gemc_destroy": (None, [P]),
            "ora_gemc_run": (I, [P, C.c_long, C.c_long, ip, ip, ip, ip, dp,
                                 dp]),
            "ora_gemc_get": (None, [P, dp, dp, ip, ip, dp, dp]),
            "ora_gemc_system_total": (None, [P, dp]),
            "ora_gemc_settings": (None, [P, dp, lp]),
            "ora_mt_create": (P, [U32]),
            "ora_mt_destroy": (None, [P]),
            "ora_mt_u32": (U32, [P]),
            "ora_philox4x64": (None, [U64, U64, U64, U64, U64, U64,
                                      C.POINTER(C.c_uint64)]),
            "ora_u01_64": (D, [U64]),
            "ora_uneg11_64": (D, [U64]),
            "ora_mc_create": (P, [P, U32, dp, I]),
            "ora_mc_destroy": (None, [P]),
            "ora_mc_run": (None, [P, C.c_long, C.c_long, ip, ip, ip, ip, dp]),
            "ora_mc_state": (None, [P, dp, lp]),
            "ora_mc_set_scales": (None, [P, dp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class SoftCore(C.Structure):
    """ora_softcore: sc_alpha, sc_sigma^6, sc_power, sc_coul."""
    _fields_ = [("alpha", C.c_double), ("sigma6", C.c_double),
                ("power", C.c_int), ("coul", C.c_int)]


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def set_threads(n: int) -> None:
    lib().ora_set_threads(int(n))


class OracleBox:
    """One NVT box in the oracle (mirrors System/CalculateEnergy/Ewald)."""

    def __init__(self, sysm, cfg):
        L = lib()
        self.sysm = sysm
        self.n_atoms = sysm.n_atoms
        self.n_mol = sysm.n_mol
        pos = np.ascontiguousarray(sysm.pos, dtype=np.float64)
        kind = np.ascontiguousarray(sysm.atom_kind, dtype=np.int32)
        q = np.ascontiguousarray(sysm.atom_charge, dtype=np.float64)
        ms = np.ascontiguousarray(sysm.mol_start, dtype=np.int32)
        eps = np.array([k.epsilon for k in sysm.kinds], dtype=np.float64)
        sig = np.array([k.sigma for k in sysm.kinds], dtype=np.float64)
        nex = np.array([k.n for k in sysm.kinds], dtype=np.float64)
        box = np.ascontiguousarray(sysm.box, dtype=np.float64)
        self._keep = (pos, kind, q, ms, eps, sig, nex, box)
        self.h = L.ora_create(self.n_atoms, self.n_mol, _dp(pos), _ip(kind),
                              _dp(q), _ip(ms), len(sysm.kinds), _dp(eps),
                              _dp(sig), _dp(nex), _dp(box), cfg.rcut,
                              cfg.rcut_low, cfg.rcut_coulomb_value,
                              cfg.tolerance, int(cfg.ewald),
                              int(cfg.electrostatic), cfg.temperature)
        self.cfg = cfg
        self._mc = None

    def __del__(self):
        try:
            L = lib()
            if self._mc:
                L.ora_mc_destroy(self._mc)
            if self.h:
                L.ora_destroy(self.h)
        except Exception:
            pass

    # --- state ------------------------------------------------------------
    @property
    def num_k(self) -> int:
        return lib().ora_num_k(self.h)

    def coords(self) -> np.ndarray:
        o = np.empty((self.n_atoms, 3))
        lib().ora_get_coords(self.h, _dp(o))
        return o

    def com(self) -> np.ndarray:
        o = np.empty((self.n_mol, 3))
        lib().ora_get_com(self.h, _dp(o))
        return o

    def set_coords(self, xyz: np.ndarray, com: Optional[np.ndarray] = None):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        c = None if com is None else np.ascontiguousarray(com, dtype=np.float64)
        lib().ora_set_coords(self.h, _dp(xyz),
                             None if c is None else _dp(c))

    def kvec(self):
        K = self.num_k
        o = np.empty(7 * K)
        lib().ora_get_kvec(self.h, _dp(o))
        o = o.reshape(7, K)
        return dict(kx=o[0], ky=o[1], kz=o[2], prefact=o[3], hsqr=o[4],
                    sumRref=o[5], sumIref=o[6])

    def sum_new(self):
        K = self.num_k
        a, b = np.empty(K), np.empty(K)
        lib().ora_get_sum_new(self.h, _dp(a), _dp(b))
        return a, b

    def cells(self):
        c = np.empty(self.n_atoms, dtype=np.int32)
        e = np.empty(3, dtype=np.int32)
        lib().ora_get_cells(self.h, _ip(c), _ip(e))
        return c, tuple(int(v) for v in e)

    def energy(self) -> np.ndarray:
        o = np.empty(5)
        lib().ora_get_energy(self.h, _dp(o))
        return o

    def set_energy(self, e5) -> None:
        a = np.ascontiguousarray(e5, dtype=np.float64)
        lib().ora_set_energy(self.h, _dp(a))

    def system_total(self) -> dict:
        o = np.empty(9)
        lib().ora_system_total(self.h, _dp(o))
        names = ["inter", "real", "recip", "self", "correction",
                 "tailCorrection", "intraBond", "intraNonbond", "total"]
        return dict(zip(names, o.tolist()))

    # --- calls --------------------------------------------------------------
    def molecule_inter(self, m: int, newpos: np.ndarray):
        p = np.ascontiguousarray(newpos, dtype=np.float64)
        a, b = C.c_double(), C.c_double()
        ov = lib().ora_molecule_inter(self.h, int(m), _dp(p), C.byref(a),
                                      C.byref(b))
        return bool(ov), a.value, b.value

    def virial(self) -> np.ndarray:
        """VirialCalc: inter, real, recip, total, then the xx/yy/zz diagonals
        of interTens, realTens, recipTens, totalTens."""
        out = np.empty(16)
        lib().ora_virial(self.h, _dp(out))
        return out

    def single_molecule_inter(self, m: int, lambdas, sc_alpha: float,
                              sc_sigma: float, sc_power: int, sc_coul: bool):
        """(old inter, old real, new inter, new real) at lambdas = (old VDW,
        new VDW, old Coulomb, new Coulomb)."""
        lam = np.ascontiguousarray(lambdas, dtype=np.float64)
        sc = SoftCore(float(sc_alpha), float(sc_sigma) ** 6, int(sc_power),
                      int(bool(sc_coul)))
        out = np.empty(4)
        lib().ora_single_molecule_inter(self.h, int(m), _dp(lam), C.byref(sc),
                                        _dp(out))
        return out

    def particle_inter(self, m: int, part: int, trial):
        """ParticleInter of atom `part` of molecule m at one trial position
        against the atoms in the cell list: (overlap, LJ, real)."""
        t = np.ascontiguousarray(trial, dtype=np.float64)
        a, b = C.c_double(), C.c_double()
        ov = lib().ora_particle_inter(self.h, int(m), int(part), _dp(t),
                                      C.byref(a), C.byref(b))
        return bool(ov), a.value, b.value

    def cell_remove_mol(self, m: int) -> None:
        lib().ora_cell_remove_mol(self.h, int(m))

    def cell_add_mol(self, m: int) -> None:
        lib().ora_cell_add_mol(self.h, int(m))

    def mol_reciprocal(self, m: int, newpos) -> float:
        p = np.ascontiguousarray(newpos, dtype=np.float64)
        return lib().ora_mol_reciprocal(self.h, _dp(p), int(m))

    def swap_dest_recip(self, m: int, pos) -> float:
        p = np.ascontiguousarray(pos, dtype=np.float64)
        return lib().ora_swap_dest_recip(self.h, _dp(p), int(m))

    def swap_source_recip(self, m: int, pos) -> float:
        p = np.ascontiguousarray(pos, dtype=np.float64)
        return lib().ora_swap_source_recip(self.h, _dp(p), int(m))

    def update_recip(self) -> None:
        lib().ora_update_recip(self.h)

    def copy_recip(self) -> None:
        lib().ora_copy_recip(self.h)

    def box_self(self) -> float:
        return lib().ora_box_self(self.h)

    def mol_correction(self, m: int) -> float:
        return lib().ora_mol_correction(self.h, int(m))

    def box_force(self, coords=None):
        aF = np.empty((self.n_atoms, 3))
        mF = np.empty((self.n_mol, 3))
        a, b = C.c_double(), C.c_double()
        c = None if coords is None else np.ascontiguousarray(coords, np.float64)
        lib().ora_box_force(self.h, None if c is None else _dp(c), _dp(aF),
                            _dp(mF), C.byref(a), C.byref(b))
        return aF, mF, a.value, b.value

    def box_reciprocal_sums(self, coords=None) -> float:
        c = None if coords is None else np.ascontiguousarray(coords, np.float64)
        return lib().ora_box_reciprocal_sums(self.h, None if c is None else _dp(c))

    def box_force_recip(self, coords=None):
        aR = np.empty((self.n_atoms, 3))
        mR = np.empty((self.n_mol, 3))
        c = None if coords is None else np.ascontiguousarray(coords, np.float64)
        lib().ora_box_force_recip(self.h, None if c is None else _dp(c),
                                  _dp(aR), _dp(mR))
        return aR, mR

    def torque(self, coords, com, aF, aR):
        tq = np.empty((self.n_mol, 3))
        args = [np.ascontiguousarray(v, np.float64) for v in (coords, com, aF, aR)]
        lib().ora_torque(self.h, *[_dp(v) for v in args], _dp(tq))
        return tq

    # --- Monte Carlo ----------------------------------------------------------
    def mc_init(self, seed: int, move_frac: Sequence[float], adj_steps: int):
        fr = np.ascontiguousarray(move_frac, dtype=np.float64)
        if self._mc:
            lib().ora_mc_destroy(self._mc)
        self._mc = lib().ora_mc_create(self.h, int(seed), _dp(fr), int(adj_steps))

    def mc_run(self, first_step: int, nsteps: int):
        k = np.empty(nsteps, np.int32)
        m = np.empty(nsteps, np.int32)
        a = np.empty(nsteps, np.int32)
        o = np.empty(nsteps, np.int32)
        de = np.empty((nsteps, 3))
        lib().ora_mc_run(self._mc, int(first_step), int(nsteps), _ip(k), _ip(m),
                         _ip(a), _ip(o), _dp(de))
        return dict(kind=k, mol=m, accepted=a, overlap=o, de=de)

    def mc_state(self):
        sc = np.empty(4)
        cnt = np.empty(6, dtype=np.int64)
        lib().ora_mc_state(self._mc, _dp(sc),
                           cnt.ctypes.data_as(C.POINTER(C.c_long)))
        return sc, cnt

    def mc_set_scales(self, scales4) -> None:
        a = np.ascontiguousarray(scales4, dtype=np.float64)
        lib().ora_mc_set_scales(self._mc, _dp(a))


class MT19937:
    def __init__(self, seed: int):
        self.h = lib().ora_mt_create(int(seed) & 0xFFFFFFFF)

    def __del__(self):
        try:
            lib().ora_mt_destroy(self.h)
        except Exception:
            pass

    def u32(self) -> int:
        return int(lib().ora_mt_u32(self.h))


def philox4x64(ctr, key):
    out = (C.c_uint64 * 4)()
    lib().ora_philox4x64(*(int(v) for v in ctr), *(int(v) for v in key), out)
    return [int(v) for v in out]


def u01_64(v: int) -> float:
    return lib().ora_u01_64(int(v))


def uneg11_64(v: int) -> float:
    return lib().ora_uneg11_64(int(v))


class OracleGemc:
    """Gibbs-ensemble NVT Monte Carlo of single-site LJ particles in two
    boxes (displacement, CBMC molecule transfer, volume exchange), restating
    the reference's moves on the host (test infrastructure)."""

    def __init__(self, pos0, pos1, box0, box1, eps, sigma, nmie, temperature,
                 rcut, seed, frac3, adj_steps, ntrials=10, rcut_low=0.0):
        p0 = np.ascontiguousarray(pos0, dtype=np.float64)
        p1 = np.ascontiguousarray(pos1, dtype=np.float64)
        L0 = np.ascontiguousarray(box0, dtype=np.float64)
        L1 = np.ascontiguousarray(box1, dtype=np.float64)
        fr = np.ascontiguousarray(frac3, dtype=np.float64)
        self.n = len(p0) + len(p1)
        self.h = lib().ora_gemc_create(len(p0), _dp(p0), len(p1), _dp(p1),
                                       _dp(L0), _dp(L1), float(eps),
                                       float(sigma), float(nmie),
                                       float(temperature), float(rcut),
                                       float(rcut_low), int(seed), _dp(fr),
                                       int(adj_steps), int(ntrials))

    def __del__(self):
        if getattr(self, "h", None):
            lib().ora_gemc_destroy(self.h)
            self.h = None

    def run(self, first: int, n: int) -> dict:
        kind, box, mol, acc = (np.empty(n, np.int32) for _ in range(4))
        d4 = np.empty((n, 4))
        st = np.empty((n, 5))
        ip = C.POINTER(C.c_int)
        rc = lib().ora_gemc_run(self.h, int(first), int(n),
                                kind.ctypes.data_as(ip),
                                box.ctypes.data_as(ip),
                                mol.ctypes.data_as(ip),
                                acc.ctypes.data_as(ip), _dp(d4), _dp(st))
        if rc:
            raise RuntimeError("oracle GEMC stopped (code %d)" % rc)
        return dict(kind=kind, box=box, mol=mol, accepted=acc, d=d4,
                    energy=st[:, :2], volume=st[:, 2:4],
                    n0=st[:, 4].astype(int))

    def state(self) -> dict:
        xyz = np.empty((self.n, 3))
        com = np.empty((self.n, 3))
        lk = np.empty(self.n, np.int32)
        n0 = C.c_int()
        e = np.empty(2)
        ax = np.empty((2, 3))
        lib().ora_gemc_get(self.h, _dp(xyz), _dp(com),
                           lk.ctypes.data_as(C.POINTER(C.c_int)),
                           C.byref(n0), _dp(e), _dp(ax))
        sc = np.empty(4)
        cnt = np.empty(12, dtype=np.int64)
        lib().ora_gemc_settings(self.h, _dp(sc),
                                cnt.ctypes.data_as(C.POINTER(C.c_long)))
        tot = np.empty(2)
        lib().ora_gemc_system_total(self.h, _dp(tot))
        return dict(xyz=xyz, com=com, lookup=lk, n0=n0.value, energy=e,
                    axes=ax, scales=sc.reshape(2, 2),
                    counts=cnt.reshape(2, 3, 2), recompute=tot)
