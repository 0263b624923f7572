"""Python host layer over the C ABI.

:class:`Box` owns one resident GB300 machine.  :class:`CalculateEnergy`,
:class:`Ewald` and :class:`CellList` expose the same method names and
argument meaning as the reference classes (src/CalculateEnergy.h:48-293,
src/Ewald.h:46-228, src/CellList.h:22-86) on top of a Box, so code written
against the reference's interfaces reads the same here.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import GB_FP64, GB_MIXED, check, lib

ENERGY_TERMS = ["inter", "real", "recip", "self", "correction",
                "tailCorrection", "intraBond", "intraNonbond", "total"]


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def system_desc(sysm):
    """gb_system_desc of a System, and the arrays it points into (keep them
    alive while the descriptor is used)."""
    keep = [np.ascontiguousarray(sysm.pos, dtype=np.float64),
            np.ascontiguousarray(sysm.atom_kind, dtype=np.int32),
            np.ascontiguousarray(sysm.atom_charge, dtype=np.float64),
            np.ascontiguousarray(sysm.mol_start, dtype=np.int32),
            np.array([k.epsilon for k in sysm.kinds], np.float64),
            np.array([k.sigma for k in sysm.kinds], np.float64),
            np.array([k.n for k in sysm.kinds], np.float64)]
    pos, kind, q, ms, eps, sig, nex = keep
    d = _lib.SystemDesc()
    d.n_atoms, d.n_mol, d.n_kinds = sysm.n_atoms, sysm.n_mol, len(sysm.kinds)
    d.pos, d.atom_kind, d.atom_charge, d.mol_start = _dp(pos), _ip(kind), \
        _dp(q), _ip(ms)
    d.kind_epsilon, d.kind_sigma, d.kind_n = _dp(eps), _dp(sig), _dp(nex)
    for i in range(3):
        d.box[i] = float(sysm.box[i])
    return d, keep


def config_struct(cfg, precision: int, device: int):
    """gb_config of a SimConfig (the in.conf keys of the energy path)."""
    c = _lib.Config()
    c.temperature = cfg.temperature
    c.rcut = cfg.rcut
    c.rcut_low = cfg.rcut_low
    c.rcut_coulomb = cfg.rcut_coulomb_value
    c.tolerance = cfg.tolerance
    c.ewald = int(cfg.ewald)
    c.electrostatic = int(cfg.electrostatic)
    c.precision = precision
    c.device = device
    c.sc_alpha = float(getattr(cfg, "sc_alpha", 0.0))
    c.sc_sigma = float(getattr(cfg, "sc_sigma", 0.0))
    c.sc_power = int(getattr(cfg, "sc_power", 0))
    c.sc_coul = int(bool(getattr(cfg, "sc_coul", False)))
    return c


def mc_params(seed: int, move_frac: Sequence[float], adj_steps: int,
              scales: Optional[Sequence[float]] = None,
              recompute_freq: int = 0, cluster_size: int = 0,
              flush_every: int = 0, move_buffer: int = 0,
              unit_lanes: int = 0, grid_ctas: int = 0,
              writer_kchunk: int = 0, moves_in_flight: int = 0):
    """gb_mc_params (Random_Seed, DisFreq / RotFreq / MultiParticleFreq,
    AdjSteps and the launch shape: the mixed form's cluster size and
    threads per real-space unit, the FP64 form's grid CTAs and whether its
    context writers hold k-vectors and its moves in flight)."""
    p = _lib.McParams()
    p.seed = int(seed) & 0xFFFFFFFF
    for i in range(3):
        p.frac[i] = float(move_frac[i])
    p.adj_steps = int(adj_steps)
    p.use_scales = 0 if scales is None else 1
    if scales is not None:
        for i in range(4):
            p.scales[i] = float(scales[i])
    p.recompute_freq = int(recompute_freq)
    p.cluster_size = int(cluster_size)
    p.flush_every = int(flush_every)
    p.move_buffer = int(move_buffer)
    p.unit_lanes = int(unit_lanes)
    p.grid_ctas = int(grid_ctas)
    p.writer_kchunk = int(writer_kchunk)
    p.moves_in_flight = int(moves_in_flight)
    return p


class Box:
    """One orthogonal periodic box resident on one GPU."""

    def __init__(self, sysm, cfg, device: int = 0,
                 precision: Optional[int] = None):
        L = lib()
        self.sysm = sysm
        self.cfg = cfg
        self.n_atoms = sysm.n_atoms
        self.n_mol = sysm.n_mol
        self.mol_start = np.ascontiguousarray(sysm.mol_start, dtype=np.int32)
        d, self._keep = system_desc(sysm)
        if precision is None:
            precision = GB_MIXED if getattr(cfg, "precision", "fp64") == "mixed" \
                else GB_FP64
        c = config_struct(cfg, precision, device)
        h = C.c_void_p()
        rc = L.gb_box_create(C.byref(d), C.byref(c), C.byref(h))
        if rc != 0:
            raise _lib.GbError(rc, (L.gb_last_error(None) or b"").decode())
        self.h = h
        self.precision = precision

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().gb_box_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _chk(self, rc: int) -> None:
        check(rc, self.h)

    def mol_atoms(self, m: int) -> int:
        return int(self.mol_start[m + 1] - self.mol_start[m])

    # ---- energies ---------------------------------------------------------
    def system_total(self) -> dict:
        o = np.empty(9)
        self._chk(lib().gb_system_total(self.h, _dp(o)))
        return dict(zip(ENERGY_TERMS, o.tolist()))

    def box_inter(self):
        a, b = C.c_double(), C.c_double()
        self._chk(lib().gb_box_inter(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def molecule_inter(self, m: int, new_pos):
        p = np.ascontiguousarray(new_pos, dtype=np.float64).reshape(-1, 3)
        if p.shape[0] != self.mol_atoms(m):
            raise ValueError("new_pos must hold every atom of the molecule")
        a, b, o = C.c_double(), C.c_double(), C.c_int32()
        self._chk(lib().gb_molecule_inter(self.h, int(m), _dp(p), C.byref(a),
                                          C.byref(b), C.byref(o)))
        return bool(o.value), a.value, b.value

    def virial(self) -> np.ndarray:
        """VirialCalc: inter, real, recip, total (K), then the xx/yy/zz
        diagonals of interTens, realTens, recipTens, totalTens."""
        out = np.empty(16)
        self._chk(lib().gb_virial(self.h, _dp(out)))
        return out

    def pressure(self) -> float:
        """Pressure in bar from the virial and the ideal-gas term
        (OutputVars::CalcAndConvert, src/OutputVars.cpp:129-180)."""
        v = self.virial()
        vol = float(np.prod(self.sysm.box))
        return 138.0649 * (self.n_mol * self.cfg.temperature +
                           v[3] / 3.0) / vol

    def single_molecule_inter(self, m: int, lambdas):
        """(old inter, old real, new inter, new real) of molecule m at
        lambdas = (old VDW, new VDW, old Coulomb, new Coulomb)."""
        lam = np.ascontiguousarray(lambdas, dtype=np.float64).reshape(4)
        out = np.empty(4)
        self._chk(lib().gb_single_molecule_inter(self.h, int(m), _dp(lam),
                                                 _dp(out)))
        return out

    def particle_inter(self, m: int, part: int, trials):
        """ParticleInter of atom `part` of molecule m at each trial position
        against the atoms in the cell list: (overlap, LJ, real) arrays."""
        t = np.ascontiguousarray(trials, dtype=np.float64).reshape(-1, 3)
        n = t.shape[0]
        en, re = np.empty(n), np.empty(n)
        ov = np.empty(n, dtype=np.int32)
        self._chk(lib().gb_particle_inter(self.h, int(m), int(part), _dp(t),
                                          n, _dp(en), _dp(re), _ip(ov)))
        return ov.astype(bool), en, re

    def cell_remove_mol(self, m: int) -> None:
        """CellList::RemoveMol: take molecule m out of the cell list."""
        self._chk(lib().gb_cell_remove_mol(self.h, int(m)))

    def cell_add_mol(self, m: int) -> None:
        """CellList::AddMol: put molecule m back at its coordinates."""
        self._chk(lib().gb_cell_add_mol(self.h, int(m)))

    def box_force(self):
        a, b = C.c_double(), C.c_double()
        aF = np.empty((self.n_atoms, 3))
        mF = np.empty((self.n_mol, 3))
        self._chk(lib().gb_box_force(self.h, C.byref(a), C.byref(b), _dp(aF),
                                     _dp(mF)))
        return aF, mF, a.value, b.value

    def calculate_torque(self):
        tq = np.empty((self.n_mol, 3))
        self._chk(lib().gb_calculate_torque(self.h, _dp(tq)))
        return tq

    # ---- Ewald --------------------------------------------------------------
    def num_kvectors(self):
        k, m = C.c_int32(), C.c_int32()
        self._chk(lib().gb_num_kvectors(self.h, C.byref(k), C.byref(m)))
        return k.value, m.value

    def kvectors(self) -> dict:
        K, _ = self.num_kvectors()
        o = np.empty(7 * max(K, 1))
        self._chk(lib().gb_get_kvectors(self.h, _dp(o)))
        o = o[:7 * K].reshape(7, K)
        return dict(kx=o[0], ky=o[1], kz=o[2], prefact=o[3], hsqr=o[4],
                    sumRref=o[5], sumIref=o[6])

    def sums_new(self):
        K, _ = self.num_kvectors()
        a, b = np.empty(max(K, 1)), np.empty(max(K, 1))
        self._chk(lib().gb_get_sums_new(self.h, _dp(a), _dp(b)))
        return a[:K], b[:K]

    def box_reciprocal_setup(self) -> None:
        self._chk(lib().gb_box_reciprocal_setup(self.h))

    def box_reciprocal_sums(self, coords=None) -> None:
        """BoxReciprocalSums: New sums of the box's coordinates or of
        `coords` [n_atoms, 3], with the current k-vector set."""
        if coords is None:
            self._chk(lib().gb_box_reciprocal_sums(self.h))
            return
        x = np.ascontiguousarray(coords, dtype=np.float64).reshape(-1, 3)
        self._chk(lib().gb_box_reciprocal_sums_coords(self.h, _dp(x)))

    def box_reciprocal(self, is_new_volume: bool = False) -> float:
        """BoxReciprocal: energy of the New sums with the New k-vector set's
        prefactors (is_new_volume) or the current set's."""
        e = C.c_double()
        self._chk(lib().gb_box_reciprocal(self.h, int(is_new_volume),
                                          C.byref(e)))
        return e.value

    def recip_init(self, edges) -> int:
        """RecipInit for trial edges: builds the New k-vector set; returns
        its size."""
        L = np.ascontiguousarray(edges, dtype=np.float64).reshape(3)
        k = C.c_int32()
        self._chk(lib().gb_recip_init(self.h, _dp(L), C.byref(k)))
        return k.value

    def box_reciprocal_setup_coords(self, coords) -> None:
        """BoxReciprocalSetup(box, molCoords): New sums of `coords` with the
        New k-vector set."""
        x = np.ascontiguousarray(coords, dtype=np.float64).reshape(-1, 3)
        self._chk(lib().gb_box_reciprocal_setup_coords(self.h, _dp(x)))

    def update_recip_vec(self) -> None:
        self._chk(lib().gb_update_recip_vec(self.h))

    def edges(self) -> np.ndarray:
        L = np.empty(3)
        self._chk(lib().gb_box_edges(self.h, _dp(L)))
        return L

    def set_box(self, edges, coords, com=None) -> None:
        """New box edges with coordinates (and centres): grid, k-vectors,
        structure factors and running energies follow."""
        L = np.ascontiguousarray(edges, dtype=np.float64).reshape(3)
        x = np.ascontiguousarray(coords, dtype=np.float64).reshape(-1, 3)
        c = None if com is None else np.ascontiguousarray(com, np.float64)
        self._chk(lib().gb_set_box(self.h, _dp(L), _dp(x),
                                   None if c is None else _dp(c)))

    def box_inter_coords(self, edges, coords):
        """BoxInter of `coords` at `edges`: (LJ, real)."""
        L = np.ascontiguousarray(edges, dtype=np.float64).reshape(3)
        x = np.ascontiguousarray(coords, dtype=np.float64).reshape(-1, 3)
        a, b = C.c_double(), C.c_double()
        self._chk(lib().gb_box_inter_coords(self.h, _dp(L), _dp(x),
                                            C.byref(a), C.byref(b)))
        return a.value, b.value

    def box_force_coords(self, coords):
        """BoxForce of `coords` at the box's edges: (atom forces, molecule
        forces, LJ, real)."""
        x = np.ascontiguousarray(coords, dtype=np.float64).reshape(-1, 3)
        a, b = C.c_double(), C.c_double()
        aF = np.empty((self.n_atoms, 3))
        mF = np.empty((self.n_mol, 3))
        self._chk(lib().gb_box_force_coords(self.h, _dp(x), C.byref(a),
                                            C.byref(b), _dp(aF), _dp(mF)))
        return aF, mF, a.value, b.value

    def swap_self(self, m: int) -> float:
        e = C.c_double()
        self._chk(lib().gb_swap_self(self.h, int(m), C.byref(e)))
        return e.value

    def swap_correction(self, m: int, pos) -> float:
        p = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        e = C.c_double()
        self._chk(lib().gb_swap_correction(self.h, int(m), _dp(p),
                                           C.byref(e)))
        return e.value

    def mol_reciprocal(self, m: int, new_pos) -> float:
        p = np.ascontiguousarray(new_pos, dtype=np.float64).reshape(-1, 3)
        e = C.c_double()
        self._chk(lib().gb_mol_reciprocal(self.h, int(m), _dp(p), C.byref(e)))
        return e.value

    def swap_dest_recip(self, m: int, pos) -> float:
        p = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        e = C.c_double()
        self._chk(lib().gb_swap_dest_recip(self.h, int(m), _dp(p), C.byref(e)))
        return e.value

    def swap_source_recip(self, m: int, pos) -> float:
        p = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        e = C.c_double()
        self._chk(lib().gb_swap_source_recip(self.h, int(m), _dp(p),
                                             C.byref(e)))
        return e.value

    def update_recip(self) -> None:
        self._chk(lib().gb_update_recip(self.h))

    def copy_recip(self) -> None:
        self._chk(lib().gb_copy_recip(self.h))

    def box_self(self) -> float:
        e = C.c_double()
        self._chk(lib().gb_box_self(self.h, C.byref(e)))
        return e.value

    def mol_correction(self, m: int) -> float:
        e = C.c_double()
        self._chk(lib().gb_mol_correction(self.h, int(m), C.byref(e)))
        return e.value

    def box_force_reciprocal(self):
        aR = np.empty((self.n_atoms, 3))
        mR = np.empty((self.n_mol, 3))
        self._chk(lib().gb_box_force_reciprocal(self.h, _dp(aR), _dp(mR)))
        return aR, mR

    # ---- cell list ----------------------------------------------------------
    def grid_all(self) -> None:
        self._chk(lib().gb_grid_all(self.h))

    def cell_membership(self):
        c = np.empty(self.n_atoms, dtype=np.int32)
        e = np.empty(3, dtype=np.int32)
        self._chk(lib().gb_cell_membership(self.h, _ip(c), _ip(e)))
        return c, tuple(int(v) for v in e)

    # ---- state --------------------------------------------------------------
    def coords(self):
        xyz = np.empty((self.n_atoms, 3))
        self._chk(lib().gb_get_coords(self.h, _dp(xyz), None))
        return xyz

    def com(self):
        c = np.empty((self.n_mol, 3))
        self._chk(lib().gb_get_coords(self.h, None, _dp(c)))
        return c

    def set_coords(self, xyz, com=None) -> None:
        x = np.ascontiguousarray(xyz, dtype=np.float64)
        c = None if com is None else np.ascontiguousarray(com, np.float64)
        self._chk(lib().gb_set_coords(self.h, _dp(x),
                                      None if c is None else _dp(c)))

    def energy(self) -> np.ndarray:
        e = np.empty(5)
        self._chk(lib().gb_get_energy(self.h, _dp(e)))
        return e

    def set_energy(self, e5) -> None:
        e = np.ascontiguousarray(e5, dtype=np.float64)
        self._chk(lib().gb_set_energy(self.h, _dp(e)))

    # ---- Monte Carlo ----------------------------------------------------------
    def mc_init(self, seed: int, move_frac: Sequence[float], adj_steps: int,
                scales: Optional[Sequence[float]] = None,
                recompute_freq: int = 0, cluster_size: int = 0,
                flush_every: int = 0, move_buffer: int = 0,
                unit_lanes: int = 0, grid_ctas: int = 0,
                writer_kchunk: int = 0, moves_in_flight: int = 0) -> None:
        p = mc_params(seed, move_frac, adj_steps, scales, recompute_freq,
                      cluster_size, flush_every, move_buffer, unit_lanes,
                      grid_ctas, writer_kchunk, moves_in_flight)
        self._chk(lib().gb_mc_init(self.h, C.byref(p)))
        # in.conf GB300Autotune: the chain's launch shape timed on this machine
        # (latency objective), unless the call named one
        shape_given = (cluster_size or unit_lanes or grid_ctas or writer_kchunk
                       or moves_in_flight)
        if getattr(self.cfg, "autotune", False) and not shape_given:
            self.mc_autotune("latency")

    def checkpoint(self) -> bytes:
        """The box's dynamic state (and its Monte Carlo state after
        mc_init) as bytes; see gb_checkpoint_save."""
        n = C.c_int64()
        self._chk(lib().gb_checkpoint_size(self.h, C.byref(n)))
        buf = C.create_string_buffer(n.value)
        self._chk(lib().gb_checkpoint_save(self.h, buf, n.value))
        return buf.raw

    def restore(self, blob: bytes) -> None:
        """Load a checkpoint written by a box of the same system and
        configuration (call mc_init first when it holds Monte Carlo
        state)."""
        buf = C.create_string_buffer(blob, len(blob))
        self._chk(lib().gb_checkpoint_load(self.h, buf, len(blob)))

    def mc_drift(self):
        mx, last = np.empty(4), np.empty(4)
        n = C.c_int64()
        self._chk(lib().gb_mc_drift(self.h, _dp(mx), _dp(last), C.byref(n)))
        names = ["inter", "real", "recip", "total"]
        return dict(max=dict(zip(names, mx.tolist())),
                    last=dict(zip(names, last.tolist())), recomputes=n.value)

    def mc_run(self, first_step: int, nsteps: int, trace: bool = False):
        if not trace:
            self._chk(lib().gb_mc_run(self.h, int(first_step), int(nsteps),
                                      None, None, None, None))
            return None
        k = np.empty(nsteps, np.int32)
        m = np.empty(nsteps, np.int32)
        a = np.empty(nsteps, np.int32)
        de = np.empty((nsteps, 3))
        self._chk(lib().gb_mc_run(self.h, int(first_step), int(nsteps), _ip(k),
                                  _ip(m), _ip(a), _dp(de)))
        return dict(kind=k, mol=m, accepted=a, de=de)

    def mc_timing(self, reset: bool = False) -> dict:
        cm, mm = C.c_double(), C.c_double()
        cl, cn, mn = C.c_int64(), C.c_int64(), C.c_int64()
        self._chk(lib().gb_mc_timing(self.h, int(reset), C.byref(cm),
                                     C.byref(cl), C.byref(cn), C.byref(mm),
                                     C.byref(mn)))
        return dict(chain_ms=cm.value, chain_launches=cl.value,
                    chain_moves=cn.value, mp_ms=mm.value, mp_moves=mn.value)

    def mc_get_gomc_state(self) -> "_lib.GomcChk":
        """The loop state as a GOMC checkpoint holds it
        (gb_mc_get_gomc_state)."""
        c = _lib.GomcChk()
        self._chk(lib().gb_mc_get_gomc_state(self.h, C.byref(c)))
        return c

    def mc_set_gomc_state(self, chk: "_lib.GomcChk") -> None:
        """Continue from a GOMC checkpoint's loop state
        (gb_mc_set_gomc_state); the next mc_run starts at chk.step."""
        self._chk(lib().gb_mc_set_gomc_state(self.h, C.byref(chk)))

    def mc_set_wait_limit(self, polls: int = 0) -> None:
        """Polls after which the FP64 chain's device waits give up
        (gb_mc_set_wait_limit; 0: the default)."""
        self._chk(lib().gb_mc_set_wait_limit(self.h, int(polls)))

    def mc_profile(self, enable: bool = True) -> dict:
        """FP64 chain phase clocks since the last call (gb_mc_profile): per
        move phase, microseconds of CTA 0 and of the deciding CTA."""
        us = np.zeros(13)
        mv = np.zeros(2, np.int64)
        self._chk(lib().gb_mc_profile(self.h, int(enable), _dp(us),
                                      mv.ctypes.data_as(C.POINTER(C.c_int64))))
        names = ["context", "listing", "partials", "decision_wait",
                 "commit_next"]
        return dict(cta0=dict(zip(names, us[:5].tolist())),
                    leader=dict(zip(names, us[5:10].tolist()),
                                last_partial_after_phase_a=us[10],
                                last_context_flag_after_phase_a=us[11]),
                    cta0_context_written_after_phase_a=us[12],
                    moves=mv.tolist())

    def mc_layout(self) -> dict:
        c, n = C.c_int32(), C.c_int32()
        sm = C.c_int64()
        self._chk(lib().gb_mc_layout(self.h, C.byref(c), C.byref(n),
                                     C.byref(sm)))
        return dict(ctas_per_chain=c.value, max_concurrent=n.value,
                    smem_bytes=sm.value)

    def mc_shape(self) -> dict:
        """The chain's launch shape (gb_mc_shape_get)."""
        sh = _lib.McShape()
        self._chk(lib().gb_mc_shape_get(self.h, C.byref(sh)))
        return dict(ctas=sh.ctas, unit_lanes=sh.unit_lanes,
                    writer_kchunk=sh.writer_kchunk,
                    moves_in_flight=sh.moves_in_flight,
                    max_concurrent=sh.max_concurrent)

    def mc_autotune(self, objective: str = "latency",
                    trial_moves: int = 0) -> dict:
        """Time each launch shape that fits on this machine's own state and keep
        the best ('latency': one chain; 'throughput': as many chains as the
        GPU holds).  Mixed form: cluster size x threads per real-space unit;
        FP64 form: grid CTAs x whether the context writers hold k-vectors x
        one or two moves in flight.
        The Monte Carlo state is unchanged.  Returns the chosen shape and
        every shape tried with its trial microseconds per move (0: it does
        not fit)."""
        best = _lib.McShape()
        tried = (_lib.McShape * 32)()
        n = C.c_int32()
        self._chk(lib().gb_mc_autotune(
            self.h, 0 if objective == "latency" else 1, int(trial_moves),
            C.byref(best), tried, 32, C.byref(n)))

        def shape(s):
            return dict(ctas=s.ctas, unit_lanes=s.unit_lanes,
                        writer_kchunk=s.writer_kchunk,
                        moves_in_flight=s.moves_in_flight,
                        max_concurrent=s.max_concurrent,
                        us_per_move=s.us_per_move)
        return dict(chosen=shape(best),
                    tried=[shape(tried[i]) for i in range(n.value)])

    def stream_ptr(self) -> int:
        p = C.c_void_p()
        self._chk(lib().gb_box_stream(self.h, C.byref(p)))
        return int(p.value or 0)

    def mc_state(self):
        sc = np.empty(4)
        cnt = np.empty(6, dtype=np.int64)
        self._chk(lib().gb_mc_state(self.h, _dp(sc),
                                    cnt.ctypes.data_as(C.POINTER(C.c_int64))))
        return sc, cnt


class Gemc:
    """Gibbs-ensemble NVT run of single-site LJ particles in two boxes
    (gb_gemc_*): displacement, CBMC molecule transfer and volume exchange,
    the whole move loop in one persistent launch on the device."""

    def __init__(self, pos0, pos1, box0, box1, epsilon: float, sigma: float,
                 n_mie: float, temperature: float, rcut: float, seed: int,
                 frac3: Sequence[float], adj_steps: int, cbmc_first: int = 10,
                 rcut_low: float = 0.0, precision: int = GB_FP64,
                 device: int = 0, cluster_size: int = 0):
        L = lib()
        self.h = None
        self._p0 = np.ascontiguousarray(pos0, dtype=np.float64).reshape(-1, 3)
        self._p1 = np.ascontiguousarray(pos1, dtype=np.float64).reshape(-1, 3)
        self.n = len(self._p0) + len(self._p1)
        d = _lib.GemcDesc()
        d.n0, d.n1 = len(self._p0), len(self._p1)
        d.pos0, d.pos1 = _dp(self._p0), _dp(self._p1)
        for k in range(3):
            d.box0[k] = float(box0[k])
            d.box1[k] = float(box1[k])
        d.epsilon, d.sigma, d.n_mie = float(epsilon), float(sigma), float(n_mie)
        c = _lib.GemcConfig()
        c.temperature, c.rcut, c.rcut_low = (float(temperature), float(rcut),
                                             float(rcut_low))
        for k in range(3):
            c.frac[k] = float(frac3[k])
        c.adj_steps, c.cbmc_first = int(adj_steps), int(cbmc_first)
        c.precision, c.device = int(precision), int(device)
        c.cluster_size, c.seed = int(cluster_size), int(seed)
        h = C.c_void_p()
        rc = L.gb_gemc_create(C.byref(d), C.byref(c), C.byref(h))
        if rc:
            raise _lib.GbError(rc, (L.gb_gemc_error(None) or b"").decode())
        self.h = h.value
        self.next_step = 0

    def close(self) -> None:
        if self.h:
            lib().gb_gemc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc: int) -> None:
        if rc:
            raise _lib.GbError(rc, (lib().gb_gemc_error(self.h) or b"")
                               .decode())

    def run(self, nsteps: int, trace: bool = False):
        """Run the next nsteps steps; with trace, per-step arrays."""
        ti = td = None
        if trace:
            ti = np.empty((nsteps, 5), np.int32)
            td = np.empty((nsteps, 8))
        self._chk(lib().gb_gemc_run(self.h, self.next_step, int(nsteps),
                                    None if ti is None else _ip(ti),
                                    None if td is None else _dp(td)))
        self.next_step += int(nsteps)
        if not trace:
            return None
        return dict(kind=ti[:, 0], box=ti[:, 1], mol=ti[:, 2],
                    accepted=ti[:, 3], n0=ti[:, 4], d=td[:, :4],
                    energy=td[:, 4:6], volume=td[:, 6:8])

    def state(self) -> dict:
        e, ax, sc = np.empty(2), np.empty((2, 3)), np.empty((2, 2))
        cnt = np.empty((2, 3, 2), np.int64)
        n0 = C.c_int32()
        ms = C.c_double()
        self._chk(lib().gb_gemc_state(self.h, _dp(e), _dp(ax), C.byref(n0),
                                      _dp(sc), cnt.ctypes.data_as(
                                          C.POINTER(C.c_int64)),
                                      C.byref(ms)))
        return dict(energy=e, axes=ax, n0=n0.value, scales=sc, counts=cnt,
                    last_ms=ms.value)

    def coords(self):
        xyz, com = np.empty((self.n, 3)), np.empty((self.n, 3))
        lk = np.empty(self.n, np.int32)
        self._chk(lib().gb_gemc_coords(self.h, _dp(xyz), _dp(com), _ip(lk)))
        return xyz, com, lk

    def system_total(self) -> np.ndarray:
        e = np.empty(2)
        self._chk(lib().gb_gemc_system_total(self.h, _dp(e)))
        return e

    def profile(self, enable: bool = True) -> dict:
        """Phase clocks since the last call (us per kind and phase) and the
        moves of each kind; switches collection on or off."""
        us = np.empty((3, 5))
        mv = np.empty(3, np.int64)
        self._chk(lib().gb_gemc_profile(self.h, int(enable), _dp(us),
                                        mv.ctypes.data_as(
                                            C.POINTER(C.c_int64))))
        kinds = ("displacement", "transfer", "volume")
        phases = ("draw", "energies", "exchange", "decision", "commit")
        return {k: dict(moves=int(mv[i]),
                        us_per_move={ph: float(us[i, j] / max(mv[i], 1))
                                     for j, ph in enumerate(phases)})
                for i, k in enumerate(kinds)}


def mc_run_batch(boxes: Sequence[Box], first_step: int, nsteps: int) -> None:
    arr = (C.c_void_p * len(boxes))(*[b.h for b in boxes])
    rc = lib().gb_mc_run_batch(arr, len(boxes), int(first_step), int(nsteps))
    if rc:
        check(rc, boxes[0].h)


# ---------------------------------------------------------------------------
# Reference-shaped facades
# ---------------------------------------------------------------------------
class CalculateEnergy:
    """src/CalculateEnergy.h:48-293 on a resident Box."""

    def __init__(self, box: Box):
        self.box = box

    def SystemTotal(self) -> dict:
        return self.box.system_total()

    def BoxInter(self):
        return self.box.box_inter()

    def MoleculeInter(self, molCoords, molIndex: int):
        """Returns (overlap, inter_LJ, inter_coulomb)."""
        return self.box.molecule_inter(molIndex, molCoords)

    def SingleMoleculeInter(self, lambdaOldVDW: float, lambdaNewVDW: float,
                            lambdaOldCoulomb: float, lambdaNewCoulomb: float,
                            molIndex: int):
        """Returns (interEnOld, interEnNew) as {inter, real} dicts."""
        o = self.box.single_molecule_inter(
            molIndex, [lambdaOldVDW, lambdaNewVDW, lambdaOldCoulomb,
                       lambdaNewCoulomb])
        return (dict(inter=o[0], real=o[1]), dict(inter=o[2], real=o[3]))

    def ParticleInter(self, trialPos, partIndex: int, molIndex: int):
        """Returns (overlap, en, real) per trial position."""
        return self.box.particle_inter(molIndex, partIndex, trialPos)

    def BoxForce(self):
        return self.box.box_force()

    def VirialCalc(self):
        return self.box.virial()

    def CalculateTorque(self):
        return self.box.calculate_torque()


class Ewald:
    """src/Ewald.h:46-228 on a resident Box."""

    def __init__(self, box: Box):
        self.box = box

    def BoxReciprocalSetup(self):
        self.box.box_reciprocal_setup()

    def BoxReciprocalSums(self, molCoords=None):
        self.box.box_reciprocal_sums(molCoords)

    def BoxReciprocal(self, isNewVolume: bool = False) -> float:
        return self.box.box_reciprocal(is_new_volume=isNewVolume)

    def RecipInit(self, boxAxes) -> int:
        return self.box.recip_init(boxAxes)

    def UpdateRecipVec(self):
        self.box.update_recip_vec()

    def SwapSelf(self, molIndex: int) -> float:
        return self.box.swap_self(molIndex)

    def SwapCorrection(self, molCoords, molIndex: int) -> float:
        return self.box.swap_correction(molIndex, molCoords)

    def MolReciprocal(self, molCoords, molIndex: int) -> float:
        return self.box.mol_reciprocal(molIndex, molCoords)

    def SwapDestRecip(self, newMolCoords, molIndex: int) -> float:
        return self.box.swap_dest_recip(molIndex, newMolCoords)

    def SwapSourceRecip(self, oldMolCoords, molIndex: int) -> float:
        return self.box.swap_source_recip(molIndex, oldMolCoords)

    def UpdateRecip(self):
        self.box.update_recip()

    def CopyRecip(self):
        self.box.copy_recip()

    def BoxSelf(self) -> float:
        return self.box.box_self()

    def MolCorrection(self, molIndex: int) -> float:
        return self.box.mol_correction(molIndex)

    def BoxForceReciprocal(self):
        return self.box.box_force_reciprocal()


class CellList:
    """src/CellList.h:22-86 on a resident Box."""

    def __init__(self, box: Box):
        self.box = box

    def GridAll(self):
        self.box.grid_all()

    def RemoveMol(self, molIndex: int):
        self.box.cell_remove_mol(molIndex)

    def AddMol(self, molIndex: int):
        self.box.cell_add_mol(molIndex)

    def CellMembership(self):
        return self.box.cell_membership()


def gomc_checkpoint_read(data: bytes) -> "_lib.GomcChk":
    """The loop state of a GOMC checkpoint file's bytes
    (gb_gomc_checkpoint_read; CheckpointSetup's reading of it)."""
    c = _lib.GomcChk()
    buf = C.create_string_buffer(bytes(data), len(data))
    check(lib().gb_gomc_checkpoint_read(buf, len(data), C.byref(c)))
    return c


def gomc_checkpoint_write(template: bytes, chk: "_lib.GomcChk") -> bytes:
    """A GOMC checkpoint file: `template` (a GOMC checkpoint of the same
    system) with the loop state of `chk` (gb_gomc_checkpoint_write)."""
    t = C.create_string_buffer(bytes(template), len(template))
    n = C.c_int64()
    check(lib().gb_gomc_checkpoint_write(t, len(template), C.byref(chk),
                                         None, 0, C.byref(n)))
    out = C.create_string_buffer(n.value)
    check(lib().gb_gomc_checkpoint_write(t, len(template), C.byref(chk),
                                         out, n.value, C.byref(n)))
    return out.raw[:n.value]
