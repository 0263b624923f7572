"""Calls whose coordinates or box edges differ from the box's own (FP64 form).

* The energy calls of a volume move (VolumeTransfer::CalcEn,
  src/moves/VolumeTransfer.h:143-190): BoxInter of trial coordinates at trial
  edges, RecipInit + BoxReciprocalSetup + BoxReciprocal(box, true) with the
  New k-vector set, against the reference's own values
  (tests/golden/vol_*.npz); then the accepted state (gb_set_box) against the
  reference's recomputed energies.
* The coordinate-taking forms MultiParticle uses (BoxForce and
  BoxReciprocalSums of trial coordinates) against the oracle.
* SwapSelf / SwapCorrection against BoxSelf / MolCorrection.

Bar: 1e-10 relative per energy term (of max(|value|, 1 K)); k-vector counts
exact.
"""
import os

import numpy as np
import pytest

from tests.golden_util import GOLDEN, config_of, load, system_of

pytestmark = pytest.mark.gpu

REL = 1e-10
VOL_NAMES = ["c0_water", "w1728", "lj500", "c3_liquid", "c3_vapour"]


@pytest.fixture(scope="module")
def gb():
    from gomc_gb300 import engine
    engine.lib(build_if_missing=True)
    return engine


def close(a, b, rel=REL):
    return abs(a - b) <= rel * max(abs(b), 1.0)


@pytest.mark.parametrize("name", VOL_NAMES)
def test_volume_move_energies(gb, name):
    z, meta = load(name)
    v = np.load(os.path.join(GOLDEN, "vol_" + name + ".npz"))
    box = gb.Box(system_of(z, meta), config_of(meta))
    ewald = meta["config"]["ewald"]
    e0 = box.energy()
    for i in range(len(v["delta"])):
        L, pos = v["edges"][i], v["pos"][i]
        lj, re = box.box_inter_coords(L, pos)
        assert close(lj, v["inter"][i]), (i, lj, v["inter"][i])
        assert close(re, v["real"][i]), (i, re, v["real"][i])
        if ewald:
            assert box.recip_init(L) == v["k_new"][i]
            box.box_reciprocal_setup_coords(pos)
            e = box.box_reciprocal(is_new_volume=True)
            assert close(e, v["recip"][i]), (i, e, v["recip"][i])
    # the trials left the box's own state alone
    np.testing.assert_array_equal(box.energy(), e0)
    np.testing.assert_array_equal(box.edges(), z["box"])
    # accept the last trial: new edges, coordinates and centres
    box.set_box(v["edges"][-1], v["pos"][-1], v["com"][-1])
    np.testing.assert_array_equal(box.edges(), v["edges"][-1])
    np.testing.assert_array_equal(box.coords(), v["pos"][-1])
    e = box.energy()
    acc = v["accepted"]
    for j in range(5):
        assert close(e[j], acc[j]), (j, e[j], acc[j])
    if ewald:
        assert box.num_kvectors()[0] == int(v["accepted_k"])
    st = box.system_total()
    assert close(st["total"], acc[5])
    box.close()


def test_update_recip_vec_then_set_box(gb):
    """UpdateRecipVec swaps in the k-vector set of trial edges; calls on the
    box's coordinates are refused until gb_set_box gives it those edges."""
    from gomc_gb300._lib import GbError
    z, meta = load("c0_water")
    v = np.load(os.path.join(GOLDEN, "vol_c0_water.npz"))
    box = gb.Box(system_of(z, meta), config_of(meta))
    L, pos = v["edges"][-1], v["pos"][-1]
    k = box.recip_init(L)
    box.box_reciprocal_setup_coords(pos)
    box.update_recip_vec()
    with pytest.raises(GbError):
        box.box_inter()
    box.set_box(L, pos, v["com"][-1])
    assert box.num_kvectors()[0] == k
    e = box.energy()
    for j in range(5):
        assert close(e[j], v["accepted"][j]), j
    box.close()


def test_coordinate_forms_against_oracle(gb):
    """BoxForce and BoxReciprocalSums of coordinates the box does not hold
    (the reference's final coordinates of the fixture's trace), as
    MultiParticle::CalcEn calls them, against the oracle fed the same
    coordinates; the box's own state stays as it was."""
    from oracle import oracle as O
    O.set_threads(1)
    z, meta = load("c0_water_mp")
    sysm, cfg = system_of(z, meta), config_of(meta)
    xyz = z["coords_final"]
    box = gb.Box(sysm, cfg)
    c0, e0 = box.coords(), box.energy()
    aF, mF, lj, re = box.box_force_coords(xyz)
    box.box_reciprocal_sums(xyz)
    er = box.box_reciprocal(is_new_volume=False)
    ob = O.OracleBox(sysm, cfg)
    ob.set_coords(xyz)
    oaF, omF, olj, ore = ob.box_force(xyz)
    oer = ob.box_reciprocal_sums(xyz)
    for got, ref in ((aF, oaF), (mF, omF)):
        np.testing.assert_allclose(got, ref, rtol=0,
                                   atol=REL * np.abs(ref).max())
    assert close(lj, olj) and close(re, ore) and close(er, oer)
    np.testing.assert_array_equal(box.coords(), c0)
    np.testing.assert_array_equal(box.energy(), e0)
    box.close()


def test_swap_self_and_correction(gb):
    z, meta = load("c0_water")
    box = gb.Box(system_of(z, meta), config_of(meta))
    n_mol = len(z["mol_start"]) - 1
    ms = z["mol_start"]
    xyz = box.coords()
    for m in (0, 17, n_mol - 1):
        assert abs(box.swap_self(m) * n_mol - box.box_self()) <= (
            1e-12 * abs(box.box_self()))
        sc = box.swap_correction(m, xyz[ms[m]:ms[m + 1]])
        assert abs(sc - box.mol_correction(m)) <= 1e-12 * abs(sc)
    box.close()
