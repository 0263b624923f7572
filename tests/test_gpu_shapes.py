"""Every launch shape the autotuner can choose runs the same Markov chain.

FP64 form: the cooperative grid at fewer CTAs than SMs, and with or without
k-vectors on the CTAs that write the next move's context -- the same
decisions as the reference's own trace of the seeded run, every move's
energy change within 1e-10.  Mixed form: every cluster size x threads per
real-space unit takes the reference's decisions, with running energies
within 1e-6 of a full FP64 recompute.  The autotuner leaves the state as it
found it, and the shape it keeps continues the chain exactly as a box
initialised with that shape.
"""
import numpy as np
import pytest

from tests.golden_util import (NAMES, config_of, load, move_fractions,
                               system_of)

pytestmark = pytest.mark.gpu

REL = 1e-10


@pytest.fixture(scope="module")
def gb():
    from gomc_gb300 import engine
    engine.lib(build_if_missing=True)
    return engine


def sm_count(gb, z, meta):
    box = gb.Box(system_of(z, meta), config_of(meta))
    box.mc_init(1, move_fractions(meta), meta["config"]["adj_steps"])
    n = box.mc_layout()["ctas_per_chain"]
    box.close()
    return n


def check_trace(r, z, rel):
    tr = z["trace"]
    np.testing.assert_array_equal(r["kind"], tr[:, 1].astype(int))
    np.testing.assert_array_equal(r["mol"], tr[:, 2].astype(int))
    np.testing.assert_array_equal(r["accepted"], tr[:, 3].astype(int))
    scale = np.maximum(np.abs(tr[-1, 8:11]), 1.0)
    for j in range(3):
        bound = rel * np.maximum(scale[j], np.abs(tr[:, 5 + j]))
        err = np.abs(r["de"][:, j] - tr[:, 5 + j])
        assert (err <= bound).all(), (j, err.max())


@pytest.mark.parametrize("name", ["c0_water", "w1728", "c1_water"])
@pytest.mark.parametrize("quarters,writer_k", [(4, 1), (3, 0), (2, 0), (2, 1),
                                               (1, 0)])
def test_fp64_grid_shapes_match_reference(gb, name, quarters, writer_k):
    z, meta = load(name)
    grid = sm_count(gb, z, meta) * quarters // 4
    box = gb.Box(system_of(z, meta), config_of(meta))
    box.mc_init(meta["config"]["random_seed"], move_fractions(meta),
                meta["config"]["adj_steps"], grid_ctas=grid,
                writer_kchunk=writer_k, moves_in_flight=1)
    assert box.mc_layout()["ctas_per_chain"] == grid
    r = box.mc_run(0, z["trace"].shape[0], trace=True)
    check_trace(r, z, REL)
    np.testing.assert_allclose(box.coords(), z["coords_final"], rtol=0,
                               atol=1e-9)
    box.close()


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("flight", [1, 2])
def test_fp64_moves_in_flight_match_reference(gb, name, flight):
    """The chain that decides each move before the next one starts, and the
    chain that runs each move while the previous one is decided, both take
    the reference's decisions, every energy change within 1e-10."""
    z, meta = load(name)
    box = gb.Box(system_of(z, meta), config_of(meta))
    box.mc_init(meta["config"]["random_seed"], move_fractions(meta),
                meta["config"]["adj_steps"], moves_in_flight=flight)
    r = box.mc_run(0, z["trace"].shape[0], trace=True)
    tr = z["trace"]
    np.testing.assert_array_equal(r["kind"], tr[:, 1].astype(int))
    np.testing.assert_array_equal(r["mol"], tr[:, 2].astype(int))
    np.testing.assert_array_equal(r["accepted"], tr[:, 3].astype(int))
    scale = np.maximum(np.abs(tr[-1, 8:11]), 1.0)
    single = tr[:, 1] < 2
    for j in range(3):
        ref = tr[single, 5 + j]
        bound = REL * np.maximum(scale[j], np.abs(ref))
        err = np.abs(r["de"][single, j] - ref)
        assert (err <= bound).all(), (j, err.max())
    e = box.energy()
    for j in range(3):
        assert abs(e[j] - tr[-1, 8 + j]) <= REL * max(scale[j], 1.0)
    np.testing.assert_allclose(box.coords(), z["coords_final"], rtol=0,
                               atol=1e-9)
    # and a fresh recompute agrees with the running totals
    st = box.system_total()
    for j, term in enumerate(("inter", "real", "recip")):
        assert abs(e[j] - st[term]) <= REL * scale[j], term
    box.close()


@pytest.mark.parametrize("quarters,writer_k", [(2, 0), (1, 1)])
def test_fp64_two_moves_in_flight_other_grids(gb, quarters, writer_k):
    """Two moves in flight at fewer grid CTAs, with and without k-vectors on
    the context writers."""
    z, meta = load("c1_water")
    grid = sm_count(gb, z, meta) * quarters // 4
    box = gb.Box(system_of(z, meta), config_of(meta))
    box.mc_init(meta["config"]["random_seed"], move_fractions(meta),
                meta["config"]["adj_steps"], grid_ctas=grid,
                writer_kchunk=writer_k, moves_in_flight=2)
    r = box.mc_run(0, z["trace"].shape[0], trace=True)
    check_trace(r, z, REL)
    box.close()


def test_fp64_grid_rejects_too_few_ctas(gb):
    from gomc_gb300._lib import GbError
    z, meta = load("c0_water")
    box = gb.Box(system_of(z, meta), config_of(meta))
    # one CTA per phase row of a water (6 x 3 atoms) at least
    with pytest.raises(GbError):
        box.mc_init(1, move_fractions(meta), meta["config"]["adj_steps"],
                    grid_ctas=12)
    with pytest.raises(GbError):
        box.mc_init(1, move_fractions(meta), meta["config"]["adj_steps"],
                    writer_kchunk=2)
    box.close()


@pytest.mark.parametrize("lanes", [32, 64, 128, 256])
@pytest.mark.parametrize("cluster", [2, 4, 8, 16])
def test_mixed_unit_lanes_take_reference_decisions(gb, cluster, lanes):
    z, meta = load("w1728")
    box = gb.Box(system_of(z, meta), config_of(meta), precision=gb.GB_MIXED)
    box.mc_init(meta["config"]["random_seed"], move_fractions(meta),
                meta["config"]["adj_steps"], cluster_size=cluster,
                unit_lanes=lanes)
    assert box.mc_layout()["ctas_per_chain"] == cluster
    tr = z["trace"]
    r = box.mc_run(0, tr.shape[0], trace=True)
    np.testing.assert_array_equal(r["accepted"], tr[:, 3].astype(int))
    run = box.energy()
    st = box.system_total()
    for i, term in enumerate(("inter", "real", "recip")):
        assert abs(run[i] - st[term]) <= 1e-6 * abs(st[term]), term
    box.close()


def test_fp64_autotune_keeps_state_and_matches_fixed_shape(gb):
    z, meta = load("w1728")
    seed, frac = meta["config"]["random_seed"], move_fractions(meta)
    adj = meta["config"]["adj_steps"]
    tuned = gb.Box(system_of(z, meta), config_of(meta))
    tuned.mc_init(seed, frac, adj)
    tuned.mc_run(0, 300)
    before = (tuned.coords(), tuned.energy(), tuned.mc_state())
    res = tuned.mc_autotune("latency", 100)
    tried = res["tried"]
    assert len(tried) == 16  # 4 grids x writers' k-vectors x moves in flight
    assert all(t["us_per_move"] > 0 for t in tried)
    best = res["chosen"]
    assert best["us_per_move"] == min(t["us_per_move"] for t in tried)
    assert tuned.mc_layout()["ctas_per_chain"] == best["ctas"]
    after = (tuned.coords(), tuned.energy(), tuned.mc_state())
    np.testing.assert_array_equal(before[0], after[0])
    np.testing.assert_array_equal(before[1], after[1])
    for x, y in zip(before[2], after[2]):
        np.testing.assert_array_equal(x, y)
    fixed = gb.Box(system_of(z, meta), config_of(meta))
    fixed.mc_init(seed, frac, adj)
    fixed.mc_run(0, 300)
    blob = fixed.checkpoint()
    fixed.mc_init(seed, frac, adj, grid_ctas=best["ctas"],
                  writer_kchunk=best["writer_kchunk"],
                  moves_in_flight=best["moves_in_flight"])
    fixed.restore(blob)
    n = z["trace"].shape[0] - 300
    a = tuned.mc_run(300, n, trace=True)
    b = fixed.mc_run(300, n, trace=True)
    np.testing.assert_array_equal(a["accepted"], b["accepted"])
    np.testing.assert_array_equal(a["de"], b["de"])
    np.testing.assert_array_equal(tuned.coords(), fixed.coords())
    np.testing.assert_array_equal(tuned.energy(), fixed.energy())
    # and the reference's decisions over the whole run
    np.testing.assert_array_equal(a["accepted"],
                                  z["trace"][300:, 3].astype(int))
    tuned.close()
    fixed.close()


def test_inconf_autotune_keeps_reference_decisions(gb):
    """GB300Autotune true: mc_init times the launch shapes on the box and
    keeps one; the chain still takes the reference's decisions."""
    z, meta = load("w1728")
    cfg = config_of(meta)
    cfg.autotune = True
    box = gb.Box(system_of(z, meta), cfg)
    box.mc_init(meta["config"]["random_seed"], move_fractions(meta),
                meta["config"]["adj_steps"])
    shape = box.mc_shape()
    assert shape["moves_in_flight"] in (1, 2) and shape["ctas"] >= 2
    r = box.mc_run(0, z["trace"].shape[0], trace=True)
    check_trace(r, z, REL)
    box.close()


def _eight_site_box(n_mol, box_len, seed):
    """Rigid 8-site molecules (a 1 A cube of alternating +-0.25 e sites, LJ
    on every site) on a lattice with random orientations: the largest
    molecule the move loop takes (48 phase rows of a move context)."""
    import math
    from gomc_gb300.systems import AtomKind, MolSystem, MoleculeType
    rng = np.random.default_rng(seed)
    n = int(math.ceil(n_mol ** (1.0 / 3.0) - 1e-9))
    sp = box_len / n
    idx = np.arange(n_mol)
    c = np.stack([(idx // (n * n) + 0.5) * sp, ((idx // n) % n + 0.5) * sp,
                  (idx % n + 0.5) * sp], axis=1)
    local = 0.5 * np.array([[x, y, z] for x in (-1, 1) for y in (-1, 1)
                            for z in (-1, 1)], dtype=np.float64)
    q = rng.normal(size=(n_mol, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    rot = np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w),
                    2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w),
                    2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
                   axis=1).reshape(n_mol, 3, 3)
    pos = (c[:, None, :] + np.einsum("mij,aj->mai", rot, local)).reshape(-1, 3)
    pos = np.round(np.mod(pos, box_len), 3)
    pos[pos >= box_len] -= box_len
    charges = [0.25, -0.25, -0.25, 0.25, -0.25, 0.25, 0.25, -0.25]
    mt = MoleculeType(name="CUB", atom_names=["C%d" % i for i in range(8)],
                      atom_kinds=[0] * 8, charges=charges)
    return MolSystem(box=np.array([box_len] * 3), kinds=[AtomKind("CS", 40.0, 2.5)],
                     mol_types=[mt], pos=pos,
                     atom_kind=np.zeros(8 * n_mol, np.int32),
                     atom_charge=np.tile(np.array(charges), n_mol),
                     atom_mol=np.repeat(np.arange(n_mol, dtype=np.int32), 8),
                     mol_start=np.arange(0, 8 * n_mol + 1, 8, dtype=np.int32),
                     mol_type=np.zeros(n_mol, np.int32))


@pytest.mark.parametrize("flight", [1, 2])
def test_eight_site_molecules_match_oracle(gb, flight):
    """Both FP64 chains on molecules of eight sites (context writers for
    48 phase rows) take the oracle's decisions, every move's energy change
    within 1e-10 of the oracle's."""
    from gomc_gb300.config import SimConfig
    from oracle import oracle as O
    sysm = _eight_site_box(343, 36.0, seed=11)
    cfg = SimConfig(temperature=300.0, rcut=9.0, tolerance=1e-5)
    seed, frac, adj, n = 77, [0.5, 0.5, 0.0], 100, 300
    box = gb.Box(sysm, cfg)
    box.mc_init(seed, frac, adj, moves_in_flight=flight)
    assert box.mc_shape()["moves_in_flight"] == flight
    r = box.mc_run(0, n, trace=True)
    O.set_threads(4)
    ob = O.OracleBox(sysm, cfg)
    ob.mc_init(seed, frac, adj)
    r2 = ob.mc_run(0, n)
    np.testing.assert_array_equal(r["mol"], r2["mol"])
    np.testing.assert_array_equal(r["accepted"], r2["accepted"])
    e = np.abs(np.asarray(box.energy())[:3])
    for j in range(3):
        bound = REL * np.maximum(max(e[j], 1.0), np.abs(r2["de"][:, j]))
        assert (np.abs(r["de"][:, j] - r2["de"][:, j]) <= bound).all(), j
    box.close()


@pytest.mark.parametrize("flight", [1, 2])
def test_eight_site_long_lists_match_oracle(gb, flight):
    """A grid of 50 CTAs (no context writer without k-vectors) and a 12 A
    cutoff: about 140 listed pairs per CTA, more than a warp's segment
    holds in the chain with two moves in flight (the pairs past it are
    evaluated where they are found); still the oracle's decisions."""
    from gomc_gb300.config import SimConfig
    from oracle import oracle as O
    sysm = _eight_site_box(343, 36.0, seed=12)
    cfg = SimConfig(temperature=300.0, rcut=12.0, tolerance=1e-5)
    seed, frac, adj, n = 78, [0.5, 0.5, 0.0], 100, 200
    box = gb.Box(sysm, cfg)
    box.mc_init(seed, frac, adj, grid_ctas=50, moves_in_flight=flight)
    assert box.mc_shape()["ctas"] == 50
    r = box.mc_run(0, n, trace=True)
    O.set_threads(4)
    ob = O.OracleBox(sysm, cfg)
    ob.mc_init(seed, frac, adj)
    r2 = ob.mc_run(0, n)
    np.testing.assert_array_equal(r["mol"], r2["mol"])
    np.testing.assert_array_equal(r["accepted"], r2["accepted"])
    e = np.abs(np.asarray(box.energy())[:3])
    for j in range(3):
        bound = REL * np.maximum(max(e[j], 1.0), np.abs(r2["de"][:, j]))
        assert (np.abs(r["de"][:, j] - r2["de"][:, j]) <= bound).all(), j
    box.close()
