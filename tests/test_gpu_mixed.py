"""Mixed-precision form against the FP64 form on the same move streams.

Bars: every running energy term within 1e-6 relative of a full FP64
recompute; per-move energy changes within 1e-2 K (3.4e-5 kT at 298 K) or
1e-4 of the FP64 change, whichever is larger (FP32 rounding of single pair
changes of a few thousand K, e.g. hydrogen-bonded O-H pairs, leaves a few
1e-3 K); the same accept/reject sequence as the FP64
chain over the compared moves; total-energy drift at most 1e-8 relative
between full FP64 recomputes every 10,000 moves; the mixed box's own
recompute (float-float structure factor) within 1e-11 of the FP64 box's on
the same coordinates; a box run inside a batched
launch gives bit-identical state to the same box run alone over the same
call boundaries (each call ends by folding the FP32 window of accepted
structure-factor changes into the FP64 accumulators).
"""
import numpy as np
import pytest

from gomc_gb300.config import SimConfig
from gomc_gb300.systems import spce_water_box

pytestmark = pytest.mark.gpu

TERM_REL = 1e-6      # running energy term vs FP64 recompute
DE_ABS = 1e-2        # per-move dE, K
DE_REL = 1e-4
DRIFT_REL = 1e-8     # total energy between recomputes
RECOMP_REL = 1e-11   # mixed-box recompute vs FP64 recompute, reciprocal term
SCALES = [0.3, 0.3, 0.02, 0.03]

# (molecules, box edge A, cutoff A): the 256-water box has cells narrower
# than the cutoff (3 per axis, 6.57 A); the larger ones have wide cells.
SYSTEMS = [(256, 19.7, 9.0), (2000, 39.1, 10.0), (8000, 62.1, 10.0)]


@pytest.fixture(scope="module")
def gb():
    from gomc_gb300 import engine
    engine.lib(build_if_missing=True)
    return engine


def make(gb, nmol, L, rc, precision, seed=7):
    s = spce_water_box(nmol, L, seed=seed)
    return gb.Box(s, SimConfig(temperature=298.0, rcut=rc, tolerance=1e-5),
                  precision=precision)


@pytest.mark.parametrize("nmol,L,rc", SYSTEMS)
def test_mixed_follows_fp64(gb, nmol, L, rc):
    n = 600
    bf = make(gb, nmol, L, rc, gb.GB_FP64)
    bm = make(gb, nmol, L, rc, gb.GB_MIXED)
    for b in (bf, bm):
        b.mc_init(1234, [0.5, 0.5, 0.0], 200, scales=SCALES)
    rf = bf.mc_run(0, n, trace=True)
    rm = bm.mc_run(0, n, trace=True)
    np.testing.assert_array_equal(rm["mol"], rf["mol"])
    np.testing.assert_array_equal(rm["kind"], rf["kind"])
    np.testing.assert_array_equal(rm["accepted"], rf["accepted"])
    err = np.abs(rm["de"] - rf["de"])
    bound = np.maximum(DE_ABS, DE_REL * np.abs(rf["de"]))
    ok = err <= bound
    assert ok.all(), (np.argwhere(~ok)[:5], err.max(axis=0))
    run = bm.energy()
    st = bm.system_total()
    for i, term in enumerate(["inter", "real", "recip"]):
        rel = abs(run[i] - st[term]) / abs(st[term])
        assert rel <= TERM_REL, (term, rel)
    # the mixed box's recompute (float-float structure factor from exact
    # 64-bit phases) against the FP64 box's on the same coordinates
    sf = bf.system_total()
    for term, tol in (("inter", 1e-13), ("real", 1e-13), ("recip", RECOMP_REL)):
        rel = abs(st[term] - sf[term]) / abs(sf[term])
        assert rel <= tol, (term, rel)
    # both chains moved the same molecules to the same places (to FP64
    # rounding of the shared proposal arithmetic, which is identical)
    np.testing.assert_array_equal(bm.coords(), bf.coords())
    bf.close()
    bm.close()


def test_mixed_drift_between_recomputes(gb):
    b = make(gb, 8000, 62.1, 10.0, gb.GB_MIXED)
    b.mc_init(99, [0.5, 0.5, 0.0], 1000, scales=SCALES, recompute_freq=10000)
    b.mc_run(0, 50000)
    d = b.mc_drift()
    assert d["recomputes"] == 5
    assert d["max"]["total"] <= DRIFT_REL, d
    for term in ("inter", "real", "recip"):
        assert d["max"][term] <= TERM_REL, d
    b.close()


@pytest.mark.parametrize("frac", [[0.5, 0.5, 0.0], [0.47, 0.47, 0.06]])
def test_batch_matches_alone(gb, frac):
    """Boxes of uneven size batched in one launch per segment end where each
    runs alone; with MultiParticle moves in the mix, a box's segment ends
    before its next MultiParticle move, which runs beside the other boxes'
    (each on its own stream)."""
    sizes = [(256, 19.7, 9.0), (2000, 39.1, 10.0), (1000, 31.0, 10.0)]

    def boxes(seed0):
        out = []
        for i, (n, L, rc) in enumerate(sizes):
            b = make(gb, n, L, rc, gb.GB_MIXED, seed=seed0 + i)
            # an FP64 recompute every 200 moves: the batched run makes
            # several boxes' recomputes at once
            b.mc_init(500 + i, frac, 300, scales=SCALES,
                      cluster_size=8, recompute_freq=200)
            out.append(b)
        return out

    alone = boxes(11)
    for b in alone:
        b.mc_run(0, 400)
        b.mc_run(400, 300)
    mixed = boxes(11)
    gb.mc_run_batch(mixed, 0, 400)
    gb.mc_run_batch(mixed, 400, 300)
    for a, m in zip(alone, mixed):
        np.testing.assert_array_equal(m.coords(), a.coords())
        np.testing.assert_array_equal(m.energy(), a.energy())
        sa, ca = a.mc_state()
        sm, cm = m.mc_state()
        np.testing.assert_array_equal(sm, sa)
        np.testing.assert_array_equal(cm, ca)
        if frac[2] > 0:
            assert cm[4] > 0  # MultiParticle moves ran
        dm, da = m.mc_drift(), a.mc_drift()
        assert dm == da and dm["recomputes"] == 3
    # a checkpoint taken between batched runs (records drawn ahead pending)
    # resumes the box's own stream where it stands
    blob = mixed[0].checkpoint()
    gb.mc_run_batch(mixed, 700, 150)
    want = (mixed[0].coords(), mixed[0].energy())
    mixed[0].restore(blob)
    mixed[0].mc_run(700, 150)
    np.testing.assert_array_equal(mixed[0].coords(), want[0])
    np.testing.assert_array_equal(mixed[0].energy(), want[1])
    for b in alone + mixed:
        b.close()


def test_autotune_keeps_state_and_matches_fixed_shape(gb):
    """The autotuner restores the state it found, and a box it tuned runs
    exactly as a box initialised with the chosen cluster size and threads
    per real-space unit."""
    params = dict(scales=SCALES, recompute_freq=0)
    tuned = make(gb, 2000, 39.1, 10.0, gb.GB_MIXED, seed=31)
    tuned.mc_init(41, [0.5, 0.5, 0.0], 300, **params)
    tuned.mc_run(0, 300)
    before = (tuned.coords(), tuned.energy(), tuned.mc_state())
    res = tuned.mc_autotune("throughput", 120)
    c, lanes = res["chosen"]["ctas"], res["chosen"]["unit_lanes"]
    assert c in (2, 4, 8, 16) and lanes in (32, 64, 128, 256)
    assert len(res["tried"]) == 16
    assert res["chosen"]["us_per_move"] > 0
    assert tuned.mc_layout()["ctas_per_chain"] == c
    after = (tuned.coords(), tuned.energy(), tuned.mc_state())
    np.testing.assert_array_equal(before[0], after[0])
    np.testing.assert_array_equal(before[1], after[1])
    for x, y in zip(before[2], after[2]):
        np.testing.assert_array_equal(x, y)
    # the same first 300 moves, then the chosen shape from the same state
    fixed = make(gb, 2000, 39.1, 10.0, gb.GB_MIXED, seed=31)
    fixed.mc_init(41, [0.5, 0.5, 0.0], 300, **params)
    fixed.mc_run(0, 300)
    blob = fixed.checkpoint()
    fixed.mc_init(41, [0.5, 0.5, 0.0], 300, cluster_size=c, unit_lanes=lanes,
                  **params)
    fixed.restore(blob)
    tuned.mc_run(300, 400)
    fixed.mc_run(300, 400)
    np.testing.assert_array_equal(tuned.coords(), fixed.coords())
    np.testing.assert_array_equal(tuned.energy(), fixed.energy())
    tuned.close()
    fixed.close()
