"""The oracle against the reference's own outputs (golden vectors).

The golden files were produced by running the reference GOMC CPU code on
seeded fixtures (tests/golden/make_golden.py).  The oracle restates the same
FP64 algorithms in C, so on one thread it must agree bit for bit on
coordinates, k-vectors, structure factors, cell membership, accept decisions
and, up to summation order, on energies (1e-12 relative here; the product
contract is 1e-10).
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.golden_util import (LARGE, NAMES, PI_NAMES, SMI_NAMES, config_of,
                               load, load_gemc, load_pi, load_smi, load_virial,
                               move_fractions, system_of)

REL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _single_thread():
    O.set_threads(1)


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


# The 8,000-water MultiParticle fixture pins the GPU path; the oracle's
# MultiParticle moves at that size take tens of seconds each on the host, and
# the oracle is pinned on the same system by c1_water and on MultiParticle by
# c0_water_mp.
ORACLE_NAMES = [n for n in NAMES if n != "c1_water_mp"]


def oracle_box(name, z, meta):
    """OracleBox of a fixture.  The set-up's structure factor is summed per
    k-vector in atom order whatever the thread count, so the large fixtures
    build it on several threads; everything after runs on one thread."""
    if name in LARGE:
        O.set_threads(8)
    try:
        return O.OracleBox(system_of(z, meta), config_of(meta))
    finally:
        O.set_threads(1)


@pytest.mark.parametrize("name", ORACLE_NAMES)
def test_initial_state(name):
    z, meta = load(name)
    box = oracle_box(name, z, meta)
    # the recompute sums the structure factor per k-vector (any thread
    # count gives the same bits) and the energies on one thread
    if name in LARGE:
        O.set_threads(8)
    try:
        st = box.system_total()
    finally:
        O.set_threads(1)
    for term in ("inter", "real", "recip", "self", "correction", "total"):
        ref = meta["init"]["box0_" + term]
        assert rel(st[term], ref) <= REL or abs(st[term] - ref) < 1e-9, term
    np.testing.assert_array_equal(box.coords(), z["coords_init"])
    np.testing.assert_array_equal(box.com(), z["com_init"].reshape(-1, 3))
    cells, edge = box.cells()
    assert list(edge) == meta["init"]["edgeCells"]
    ref_cells = np.full(box.n_atoms, -1)
    ref_cells[z["cells"][:, 0]] = z["cells"][:, 1]
    np.testing.assert_array_equal(cells, ref_cells)
    if "kvec" in z:
        kv = box.kvec()
        assert box.num_k == int(meta["init"]["imageSize"])
        for i, key in enumerate(["kx", "ky", "kz", "prefact", "sumRref",
                                 "sumIref", "hsqr"]):
            np.testing.assert_array_equal(kv[key], z["kvec"][:, i])


@pytest.mark.parametrize("name", ORACLE_NAMES)
def test_proposal_deltas(name):
    z, meta = load(name)
    box = oracle_box(name, z, meta)
    cur = box.coords()
    ms = z["mol_start"]
    for i, m in enumerate(z["prop_mol"]):
        ref = z["prop_out"][i]
        ov, lj, re = box.molecule_inter(int(m), z["prop_pos"][i])
        assert int(ref[0]) == m and int(ref[1]) == int(ov)
        assert lj == ref[2] and re == ref[3]
        if meta["config"]["ewald"]:
            assert box.mol_reciprocal(int(m), z["prop_pos"][i]) == ref[4]
            assert box.swap_dest_recip(int(m), z["prop_pos"][i]) == ref[5]
            old = cur[ms[m]:ms[m + 1]]
            assert box.swap_source_recip(int(m), old) == ref[6]


@pytest.mark.parametrize("name", ORACLE_NAMES)
def test_mc_trace(name):
    z, meta = load(name)
    box = oracle_box(name, z, meta)
    box.mc_init(meta["config"]["random_seed"], move_fractions(meta),
                meta["config"]["adj_steps"])
    tr = z["trace"]
    n = tr.shape[0]
    r = box.mc_run(0, n)
    np.testing.assert_array_equal(r["kind"], tr[:, 1].astype(int))
    np.testing.assert_array_equal(r["mol"], tr[:, 2].astype(int))
    np.testing.assert_array_equal(r["accepted"], tr[:, 3].astype(int))
    # per-move deltas: bit-exact for single-molecule moves; MultiParticle rows
    # hold new box energies
    single = tr[:, 1] < 2
    np.testing.assert_array_equal(r["de"][single], tr[single, 5:8])
    mp = ~single
    if mp.any():
        np.testing.assert_allclose(r["de"][mp], tr[mp, 5:8], rtol=1e-12,
                                   atol=1e-9)
    e = box.energy()
    np.testing.assert_allclose(e[:3], tr[-1, 8:11], rtol=REL, atol=1e-9)
    np.testing.assert_array_equal(box.coords(), z["coords_final"])
    sc, cnt = box.mc_state()
    for k in range(3):
        key = "move%d" % k
        if key in meta["final"]:
            tries, acc, scale = meta["final"][key]
            assert cnt[2 * k] == tries and cnt[2 * k + 1] == acc
            if k < 2:
                assert sc[k] == scale


def test_forces_against_reference():
    z, meta = load("c0_water_mp")
    box = O.OracleBox(system_of(z, meta), config_of(meta))
    aF, mF, lj, re = box.box_force()
    box.copy_recip()
    aR, mR = box.box_force_recip()
    tq = box.torque(box.coords(), box.com(), aF, aR)
    fa, fm = z["forces_atom"], z["forces_mol"]
    np.testing.assert_array_equal(aF, fa[:, 0:3])
    np.testing.assert_array_equal(aR, fa[:, 3:6])
    np.testing.assert_array_equal(mF, fm[:, 0:3])
    np.testing.assert_array_equal(mR, fm[:, 3:6])
    np.testing.assert_array_equal(tq, fm[:, 6:9])
    assert lj == meta["force_energy"]["inter"]
    assert re == meta["force_energy"]["real"]


def test_rng_known_answers():
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "kat_rng.npz"))
    mt = z["mt"]
    for seed in np.unique(mt[:, 0]):
        g = O.MT19937(int(seed))
        ref = mt[mt[:, 0] == seed, 1]
        got = np.array([g.u32() for _ in range(len(ref))], dtype=np.uint64)
        np.testing.assert_array_equal(got, ref)
    for row_i, row_r in zip(z["philox_int"], z["philox_real"]):
        step, seed, ctr = (int(v) for v in row_i[:3])
        r = O.philox4x64((ctr, 0, 0, 0), (step, seed))
        assert r == [int(v) for v in row_i[3:7]]
        for d in range(3):
            assert O.u01_64(r[d]) == row_r[d]
            assert 1.0 * O.uneg11_64(r[d]) == row_r[3 + d]


@pytest.mark.parametrize("name", SMI_NAMES)
def test_single_molecule_inter(name):
    """CalculateEnergy::SingleMoleculeInter at two lambda pairs, soft-core
    LJ and (every other row) soft-core Coulomb: bit-exact."""
    z, meta = load(name)
    ob = O.OracleBox(system_of(z, meta), config_of(meta))
    g = load_smi(name)
    a, s, p = g["soft_core"]
    for m, lam, c, ref in zip(g["mol"], g["lam"], g["sc_coul"], g["out"]):
        got = ob.single_molecule_inter(int(m), lam, a, s, int(p), bool(c))
        np.testing.assert_array_equal(got, ref)
    del ob


@pytest.mark.parametrize("name", ORACLE_NAMES)
def test_virial(name):
    """VirialCalc + VirialReciprocal of the initial state: bit-exact."""
    z, meta = load(name)
    ob = oracle_box(name, z, meta)
    np.testing.assert_array_equal(ob.virial(), load_virial(name))
    del ob


@pytest.mark.parametrize("name", PI_NAMES)
def test_particle_inter(name):
    """ParticleInter against the reference's vectors, bit-exact: the same
    cases in the same order, the molecule taken out of the cell list around
    the call where the reference took it out (each removal and re-insertion
    relinks the molecule at the head of its cells, as in the reference, so
    later cases sum in the reference's order too)."""
    z, meta = load(name)
    g = load_pi(name)
    ob = oracle_box(name, z, meta)
    for c in range(len(g["mol"])):
        m, part, rm = int(g["mol"][c]), int(g["part"][c]), int(g["remove"][c])
        if rm:
            ob.cell_remove_mol(m)
        for t in range(g["trials"].shape[1]):
            ov, en, re = ob.particle_inter(m, part, g["trials"][c, t])
            assert int(ov) == g["overlap"][c, t]
            assert en == g["en"][c, t] and re == g["real"][c, t], (c, t)
        if rm:
            ob.cell_add_mol(m)
    del ob


def test_gemc_trace():
    """The Gibbs-ensemble restatement against the reference's own GEMC NVT
    run (6,000 steps: displacement, CBMC molecule transfer, volume exchange):
    every move kind, box, molecule and decision identical; volumes, final
    coordinates, centres, molecule lookup order, move scales and counts
    bit-identical; running energies within 1e-12 (the sums run in another
    order than the reference's cell lists)."""
    z, meta = load_gemc()
    g = meta["gemc"]
    ob = O.OracleGemc(z["pos0"], z["pos1"], z["box0"], z["box1"],
                      z["kind_eps"][0], z["kind_sigma"][0], z["kind_n"][0],
                      g["temperature"], g["rcut"], g["random_seed"],
                      [g["dis_freq"], g["vol_freq"], g["swap_freq"]],
                      g["adj_steps"], g["cbmc_first"])
    tr = z["trace"]
    r = ob.run(0, len(tr))
    np.testing.assert_array_equal(r["kind"], tr[:, 1].astype(int))
    np.testing.assert_array_equal(r["box"], tr[:, 2].astype(int))
    vol = r["kind"] == 13
    np.testing.assert_array_equal(r["mol"][~vol], tr[~vol, 3].astype(int))
    np.testing.assert_array_equal(r["accepted"], tr[:, 4].astype(int))
    np.testing.assert_array_equal(r["volume"], tr[:, 7:9])
    np.testing.assert_array_equal(r["n0"], tr[:, 9].astype(int))
    ref = tr[:, 5:7]
    assert (np.abs(r["energy"] - ref) <= 1e-12 * np.maximum(np.abs(ref), 1.0)
            ).all()
    st = ob.state()
    np.testing.assert_array_equal(st["xyz"], z["coords_final"])
    np.testing.assert_array_equal(st["com"], z["com_final"])
    np.testing.assert_array_equal(st["lookup"], z["lookup_final"])
    assert st["n0"] == int(z["lookup_counts"][0])
    np.testing.assert_array_equal(st["axes"], z["axes_final"])
    sf = z["settings_final"]  # box, move, tries, accepted, scale
    for row in sf:
        b, mv = int(row[0]), int(row[1])
        k = {0: 0, 10: 1, 13: 2}[mv]
        assert st["counts"][b, k, 0] == row[2] and st["counts"][b, k, 1] == row[3]
        if mv == 0:
            assert st["scales"][b, 0] == row[4]
        elif mv == 13:
            assert st["scales"][b, 1] == row[4]
    fin = meta["final"]
    for b in range(2):
        assert abs(st["recompute"][b] - fin["recalc%d_inter" % b]) <= (
            1e-12 * abs(fin["recalc%d_inter" % b]))
