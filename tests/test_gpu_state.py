"""Host-side state changes through the C ABI (FP64 form) against the oracle.

gb_set_coords replaces the coordinates and must leave the box as System::Init
would (cell list, Ewald structure factors, running energies), so a Monte
Carlo run that follows scores its moves against the new state.
"""
import numpy as np
import pytest

from tests.golden_util import config_of, load, move_fractions, system_of

pytestmark = pytest.mark.gpu

REL = 1e-10


@pytest.fixture(scope="module")
def gb():
    from gomc_gb300 import engine
    engine.lib(build_if_missing=True)
    return engine


@pytest.mark.parametrize("name", ["c0_water", "lj500"])
def test_set_coords_then_moves_match_oracle(gb, name):
    """Upload coordinates the box did not produce (the reference's final
    coordinates of the fixture's trace), then run 500 moves: the running
    energies right after the upload equal a full recompute, and the moves'
    decisions and final energies equal the oracle's fed the same
    coordinates."""
    from oracle import oracle as O
    O.set_threads(1)
    z, meta = load(name)
    sysm, cfg = system_of(z, meta), config_of(meta)
    xyz = z["coords_final"]
    com = z["com_final"].reshape(-1, 3)
    box = gb.Box(sysm, cfg)
    before = box.energy()
    box.set_coords(xyz, com)
    np.testing.assert_array_equal(box.coords(), xyz)
    np.testing.assert_array_equal(box.com(), com)
    ob = O.OracleBox(sysm, cfg)
    ob.set_coords(xyz, com)
    so = ob.system_total()
    e = box.energy()
    assert not np.array_equal(e[:3], before[:3])
    for i, term in enumerate(("inter", "real", "recip", "self", "correction")):
        assert abs(e[i] - so[term]) <= REL * max(abs(so[term]), 1.0), term
    cells, _ = box.cell_membership()
    ocells, _ = ob.cells()
    np.testing.assert_array_equal(cells, ocells)
    seed = 777
    box.mc_init(seed, move_fractions(meta), 100)
    ob.mc_init(seed, move_fractions(meta), 100)
    r = box.mc_run(0, 500, trace=True)
    r2 = ob.mc_run(0, 500)
    np.testing.assert_array_equal(r["mol"], r2["mol"])
    np.testing.assert_array_equal(r["accepted"], r2["accepted"])
    e, e2 = box.energy(), ob.energy()
    for i in range(3):
        assert abs(e[i] - e2[i]) <= REL * max(abs(e2[i]), 1.0), i
    box.close()


def test_set_coords_computes_centres(gb):
    """Without centres, gb_set_coords computes them as COM::CalcCOM does."""
    z, meta = load("c0_water")
    box = gb.Box(system_of(z, meta), config_of(meta))
    box.set_coords(z["coords_final"])
    np.testing.assert_allclose(box.com(), z["com_final"].reshape(-1, 3),
                               rtol=0, atol=1e-9)
    st = box.system_total()
    e = box.energy()
    for i, term in enumerate(("inter", "real", "recip")):
        assert abs(e[i] - st[term]) <= REL * abs(st[term]), term
    box.close()


def test_chain_profile_accounts_for_the_chain(gb):
    """gb_mc_profile: the FP64 chain's phase clocks of CTA 0 and of the
    deciding CTA cover the moves run with collection on, add up to about
    the chain's device time, and collection off adds nothing."""
    z, meta = load("c0_water")
    box = gb.Box(system_of(z, meta), config_of(meta))
    box.mc_init(meta["config"]["random_seed"], move_fractions(meta),
                meta["config"]["adj_steps"])
    box.mc_run(0, 100)
    box.mc_profile(enable=True)
    box.mc_timing(reset=True)
    box.mc_run(100, 400)
    t = box.mc_timing(reset=True)
    pr = box.mc_profile(enable=False)
    assert pr["moves"] == [400, 400]
    for who in ("cta0", "leader"):
        phases = pr[who]
        keys = ("context", "listing", "partials", "decision_wait",
                "commit_next")
        assert all(phases[k] >= 0.0 for k in keys)
        total_us = sum(phases[k] for k in keys)
        # the clocks run inside the kernel; the events also hold the launch,
        # the prologue and the grid rebuild
        assert 0.5 * t["chain_ms"] * 1e3 <= total_us <= 1.05 * t["chain_ms"] * 1e3
    box.mc_run(500, 100)
    again = box.mc_profile(enable=False)
    assert again["moves"] == [0, 0]
    box.close()
