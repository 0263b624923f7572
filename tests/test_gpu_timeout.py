"""Bounded device-side waits of the FP64 chain (gb_mc_set_wait_limit).

A wait that gives up must not fault or hang the GPU: with the limit cut to
one poll, the chain's waits (grid barrier, partials, the next context, the
decision word) run out long before the other CTAs arrive, gb_mc_run returns
GB_ERR_TIMEOUT, the box's coordinates and running energies are those before
the call, and after gb_mc_init the same box runs the reference's move
sequence exactly as a fresh box does.
"""
import numpy as np
import pytest

from tests.golden_util import config_of, load, move_fractions, system_of

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gb():
    from gomc_gb300 import engine
    engine.lib(build_if_missing=True)
    return engine


def test_wait_limit_times_out_and_box_recovers(gb):
    from gomc_gb300._lib import GbError
    z, meta = load("c0_water")
    sysm, cfg = system_of(z, meta), config_of(meta)
    seed = meta["config"]["random_seed"]
    frac = move_fractions(meta)
    adj = meta["config"]["adj_steps"]
    box = gb.Box(sysm, cfg)
    x0, e0 = box.coords(), box.energy()
    box.mc_init(seed, frac, adj)
    box.mc_set_wait_limit(1)
    with pytest.raises(GbError) as err:
        box.mc_run(0, 200)
    assert err.value.code == 5  # GB_ERR_TIMEOUT
    np.testing.assert_array_equal(box.coords(), x0)
    np.testing.assert_array_equal(box.energy(), e0)

    box.mc_init(seed, frac, adj)  # the default limit, the error cleared
    r = box.mc_run(0, 200, trace=True)
    fresh = gb.Box(sysm, cfg)
    fresh.mc_init(seed, frac, adj)
    rf = fresh.mc_run(0, 200, trace=True)
    for key in ("kind", "mol", "accepted"):
        np.testing.assert_array_equal(r[key], rf[key])
    np.testing.assert_array_equal(r["de"], rf["de"])
    np.testing.assert_array_equal(box.coords(), fresh.coords())
    np.testing.assert_array_equal(box.energy(), fresh.energy())
    box.close()
    fresh.close()


def test_wait_limit_rejects_out_of_range(gb):
    from gomc_gb300._lib import GbError
    z, meta = load("c0_water")
    box = gb.Box(system_of(z, meta), config_of(meta))
    with pytest.raises(GbError):
        box.mc_set_wait_limit(10)  # no loop yet: GB_ERR_STATE
    box.mc_init(meta["config"]["random_seed"], move_fractions(meta),
                meta["config"]["adj_steps"])
    with pytest.raises(GbError):
        box.mc_set_wait_limit(-1)
    box.mc_set_wait_limit(0)
    box.close()
