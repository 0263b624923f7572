"""Checkpoint and resume (gb_checkpoint_*): a run that stops, saves, and
continues in a fresh box from the saved state ends bit-identical to a run
that never stopped -- coordinates, molecule centres, running energies and
move statistics -- for the FP64 form (with MultiParticle moves) and the
mixed form.  The reference's restart tests pin the same property for its
own checkpoint format (test/src/CheckpointTest.cpp)."""
import numpy as np
import pytest

from gomc_gb300.config import SimConfig
from gomc_gb300.systems import spce_water_box
from tests.golden_util import config_of, load, move_fractions, system_of

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gb():
    from gomc_gb300 import engine
    engine.lib(build_if_missing=True)
    return engine


def _state(box):
    sc, cnt = box.mc_state()
    return box.coords(), box.com(), box.energy(), sc, cnt


def _resume_equals_straight(gb, make, init, first, more):
    straight = make()
    init(straight)
    straight.mc_run(0, first)
    blob = straight.checkpoint()
    straight.mc_run(first, more)
    want = _state(straight)
    straight.close()
    resumed = make()
    init(resumed)
    resumed.restore(blob)
    resumed.mc_run(first, more)
    got = _state(resumed)
    resumed.close()
    for a, b in zip(got, want):
        np.testing.assert_array_equal(a, b)


def test_fp64_with_multiparticle(gb):
    z, meta = load("c0_water_mp")
    seed = meta["config"]["random_seed"]

    def make():
        return gb.Box(system_of(z, meta), config_of(meta))

    def init(b):
        b.mc_init(seed, move_fractions(meta), meta["config"]["adj_steps"])
    _resume_equals_straight(gb, make, init, 150, 200)


def test_mixed(gb):
    def make():
        return gb.Box(spce_water_box(2000, 39.1, seed=21),
                      SimConfig(temperature=298.0, rcut=10.0, tolerance=1e-5),
                      precision=gb.GB_MIXED)

    def init(b):
        b.mc_init(77, [0.5, 0.5, 0.0], 300, scales=[0.3, 0.3, 0.02, 0.03],
                  recompute_freq=500)
    _resume_equals_straight(gb, make, init, 700, 900)


def test_rejects_other_system(gb):
    from gomc_gb300._lib import GbError
    cfg = SimConfig(temperature=298.0, rcut=9.0, tolerance=1e-5)
    a = gb.Box(spce_water_box(256, 19.7, seed=1), cfg)
    blob = a.checkpoint()
    a.close()
    b = gb.Box(spce_water_box(300, 20.8, seed=1), cfg)
    with pytest.raises(GbError):
        b.restore(blob)
    with pytest.raises(GbError):
        b.restore(b"not a checkpoint at all, just some bytes")
    b.close()


def test_rejected_load_leaves_box_unchanged(gb):
    """A checkpoint whose random-stream position or cell slots are out of
    range is refused before anything reaches the device: the box keeps its
    coordinates, energies and move stream (the next moves equal those of a
    box that never saw the bad checkpoint)."""
    from gomc_gb300._lib import GbError
    import struct
    z, meta = load("c0_water")
    seed = meta["config"]["random_seed"]

    def make():
        b = gb.Box(system_of(z, meta), config_of(meta))
        b.mc_init(seed, move_fractions(meta), meta["config"]["adj_steps"])
        return b
    src = make()
    src.mc_run(0, 300)
    good = bytearray(src.checkpoint())
    src.close()
    n_atoms, n_mol = len(z["pos"]), len(z["mol_start"]) - 1
    hdr = 48  # magic, eight int32 fields, int64 step
    K, ncell, cap = struct.unpack_from("<iii", good, 8 + 12)
    body = 8 * (3 * n_atoms + 3 * n_mol + 5 + 2 * K)
    counts = hdr + body
    slots = counts + 4 * ncell
    mc = slots + 4 * ncell * cap
    bad_mt = bytearray(good)
    struct.pack_into("<i", bad_mt, mc + 4 * 624, 700)       # mt_left
    bad_slot = bytearray(good)
    struct.pack_into("<i", bad_slot, slots, n_atoms + 5)    # slot 0 of cell 0
    dup_slot = bytearray(good)
    first, second = struct.unpack_from("<ii", good, slots)
    struct.pack_into("<i", dup_slot, slots + 4, first)      # an atom twice
    ref = make()
    ref.mc_run(0, 200)
    want = _state(ref)
    ref.close()
    box = make()
    before = (box.coords(), box.energy())
    for blob in (bad_mt, bad_slot, dup_slot):
        with pytest.raises(GbError):
            box.restore(bytes(blob))
        np.testing.assert_array_equal(box.coords(), before[0])
        np.testing.assert_array_equal(box.energy(), before[1])
    box.mc_run(0, 200)
    for a, b in zip(_state(box), want):
        np.testing.assert_array_equal(a, b)
    box.close()


def test_continues_reference_run_from_its_checkpoint(gb):
    """Hand-off from a stock GOMC run: the reference's own checkpoint after
    600 steps of c0_water (tests/golden/chk_c0_water.npz) and the
    coordinates it belongs to go into a fresh box (gb_set_coords,
    gb_mc_set_gomc_state); the box's next 400 moves are the reference's
    steps 600-999 -- same molecules, kinds and decisions, energy changes to
    1e-10 -- and its loop state at step 1,000, written back as a GOMC
    checkpoint over the reference's file, reads back with the reference's
    move counts and scales at that step."""
    import json
    import os
    from tests.golden_util import GOLDEN
    z, meta = load("c0_water")
    zc = np.load(os.path.join(GOLDEN, "chk_c0_water.npz"))
    mc = json.loads(bytes(zc["meta_json"]).decode())
    first, total = mc["chk_step"], mc["total"]
    box = gb.Box(system_of(z, meta), config_of(meta))
    box.mc_init(meta["config"]["random_seed"], move_fractions(meta),
                meta["config"]["adj_steps"])
    box.set_coords(zc["coords_chk"], zc["com_chk"].reshape(-1, 3))
    chk = gb.gomc_checkpoint_read(bytes(zc["chk"]))
    box.mc_set_gomc_state(chk)
    r = box.mc_run(first, total - first, trace=True)
    tr = zc["trace"][first:total]
    np.testing.assert_array_equal(r["kind"], tr[:, 1].astype(int))
    np.testing.assert_array_equal(r["mol"], tr[:, 2].astype(int))
    np.testing.assert_array_equal(r["accepted"], tr[:, 3].astype(int))
    scale = np.maximum(np.abs(tr[-1, 8:11]), 1.0)
    for j in range(3):
        bound = 1e-10 * np.maximum(scale[j], np.abs(tr[:, 5 + j]))
        assert (np.abs(r["de"][:, j] - tr[:, 5 + j]) <= bound).all(), j
    np.testing.assert_allclose(box.coords(), zc["coords_final"], rtol=0,
                               atol=1e-9)
    out = gb.gomc_checkpoint_write(bytes(zc["chk"]), box.mc_get_gomc_state())
    back = gb.gomc_checkpoint_read(out)
    assert back.step == total
    for k in (0, 1):
        tries, acc, scl = mc["final"]["move%d" % k]
        assert back.tries[0][k] == tries and back.accepted[0][k] == acc
        assert abs(back.scale[0][k] - scl) <= 1e-12 * scl
    box.close()
