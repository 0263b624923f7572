"""``in.conf`` keys of the energy path.

:class:`SimConfig` carries the keys the reference reads for the hot path
(src/ConfigSetup.cpp:222-1409): ``Temperature``, ``Potential``, ``LRC``,
``Rcut``, ``RcutLow``, ``Exclude``, ``Ewald``, ``ElectroStatic``,
``Tolerance``, ``RcutCoulomb``, ``CachedFourier``, ``1-4scaling``,
``Dielectric``, ``RunSteps``, ``EqSteps``, ``AdjSteps``, ``DisFreq``,
``RotFreq``, ``MultiParticleFreq``, ``PRNG``, ``Random_Seed`` and the cell
basis vectors.  Keys that only this implementation reads carry a ``GB300``
prefix, which the reference skips with an "Unknown input" warning:

* ``GB300Precision``  ``fp64`` (plain form, default) or ``mixed``
* ``GB300RecomputeFreq``  full FP64 recompute interval of the mixed form
* ``GB300Autotune``  ``true``: ``Box.mc_init`` times the chain's launch
  shapes on the box's own state (``gb_mc_autotune``, latency objective)
  and keeps the fastest, unless the call names a shape
"""
from __future__ import annotations

import dataclasses
from typing import Dict, Optional


@dataclasses.dataclass
class SimConfig:
    temperature: float = 298.0
    rcut: float = 9.0
    rcut_low: float = 0.0
    rcut_coulomb: Optional[float] = None   # defaults to Rcut (ConfigSetup.cpp:1689-1696)
    lrc: bool = False
    ewald: bool = True
    electrostatic: bool = True
    tolerance: float = 1e-5
    cached_fourier: bool = False
    scaling_14: float = 0.0
    dielectric: float = 1.0
    run_steps: int = 10000
    eq_steps: int = 5000
    adj_steps: int = 1000
    dis_freq: float = 0.5
    rot_freq: float = 0.5
    multi_particle_freq: float = 0.0
    random_seed: int = 1234
    # build-only keys
    # soft-core pair terms at lambda < 1 (ScaleAlpha, ScaleSigma, ScalePower,
    # ScaleCoulomb; 0 when free-energy and NeMTMC moves are off)
    sc_alpha: float = 0.0
    sc_sigma: float = 0.0
    sc_power: int = 0
    sc_coul: bool = False
    precision: str = "fp64"
    recompute_freq: int = 10000
    autotune: bool = False

    @property
    def rcut_coulomb_value(self) -> float:
        return self.rcut if self.rcut_coulomb is None else self.rcut_coulomb

    def move_fractions(self):
        """Normalised (displace, rotate, multiparticle) fractions, the way
        StaticVals normalises movePerc (src/StaticVals.cpp:37-96)."""
        tot = self.dis_freq + self.rot_freq + self.multi_particle_freq
        if tot <= 0:
            raise ValueError("no move frequency set")
        return (self.dis_freq / tot, self.rot_freq / tot,
                self.multi_particle_freq / tot)


_BOOL = {"true": True, "on": True, "yes": True, "1": True,
         "false": False, "off": False, "no": False, "0": False}


def parse_inconf(text: str) -> SimConfig:
    """Parse the hot-path keys of an ``in.conf`` body into a SimConfig."""
    cfg = SimConfig()
    for raw in text.splitlines():
        line = raw.split("#", 1)[0].strip()
        if not line:
            continue
        tok = line.split()
        key = tok[0]
        args = tok[1:]
        k = key.lower()
        if k == "temperature":
            cfg.temperature = float(args[0])
        elif k == "rcut":
            cfg.rcut = float(args[0])
        elif k == "rcutlow":
            cfg.rcut_low = float(args[0])
        elif k == "rcutcoulomb":
            cfg.rcut_coulomb = float(args[-1])
        elif k == "lrc":
            cfg.lrc = _BOOL[args[0].lower()]
        elif k == "ewald":
            cfg.ewald = _BOOL[args[0].lower()]
        elif k == "electrostatic":
            cfg.electrostatic = _BOOL[args[0].lower()]
        elif k == "tolerance":
            cfg.tolerance = float(args[0])
        elif k == "cachedfourier":
            cfg.cached_fourier = _BOOL[args[0].lower()]
        elif k == "1-4scaling":
            cfg.scaling_14 = float(args[0])
        elif k == "dielectric":
            cfg.dielectric = float(args[0])
        elif k == "runsteps":
            cfg.run_steps = int(args[0])
        elif k == "eqsteps":
            cfg.eq_steps = int(args[0])
        elif k == "adjsteps":
            cfg.adj_steps = int(args[0])
        elif k == "disfreq":
            cfg.dis_freq = float(args[0])
        elif k == "rotfreq":
            cfg.rot_freq = float(args[0])
        elif k == "multiparticlefreq":
            cfg.multi_particle_freq = float(args[0])
        elif k == "random_seed":
            cfg.random_seed = int(args[0])
        elif k == "gb300precision":
            if args[0].lower() not in ("fp64", "mixed"):
                raise ValueError("GB300Precision must be fp64 or mixed")
            cfg.precision = args[0].lower()
        elif k == "gb300recomputefreq":
            cfg.recompute_freq = int(args[0])
        elif k == "gb300autotune":
            cfg.autotune = _BOOL[args[0].lower()]
    if cfg.adj_steps > cfg.eq_steps:
        # Same rule the reference enforces (src/ConfigSetup.cpp:1957-1962).
        raise ValueError("AdjSteps cannot be larger than EqSteps")
    return cfg


def config_keys(cfg: SimConfig) -> Dict[str, str]:
    """The in.conf rows for a config (reference keys plus GB300 keys)."""
    return {
        "Temperature": repr(cfg.temperature), "Rcut": repr(cfg.rcut),
        "RcutLow": repr(cfg.rcut_low), "LRC": str(cfg.lrc).lower(),
        "Ewald": str(cfg.ewald).lower(),
        "ElectroStatic": str(cfg.electrostatic).lower(),
        "Tolerance": repr(cfg.tolerance), "AdjSteps": str(cfg.adj_steps),
        "DisFreq": repr(cfg.dis_freq), "RotFreq": repr(cfg.rot_freq),
        "MultiParticleFreq": repr(cfg.multi_particle_freq),
        "Random_Seed": str(cfg.random_seed),
        "GB300Precision": cfg.precision,
        "GB300RecomputeFreq": str(cfg.recompute_freq),
        "GB300Autotune": str(cfg.autotune).lower(),
    }
