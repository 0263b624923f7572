"""The Gibbs-ensemble engine (gb_gemc_*) against the reference's own GEMC NVT
run of the LJ-sphere configuration (tests/golden/c3_gemc.npz: 2,400 spheres
in 40 A and 300 in 90 A, 6,000 steps of displacement / CBMC molecule
transfer / volume exchange at 0.8 / 0.19 / 0.01).

FP64 form: every move kind, box, molecule and decision identical to the
reference's; volumes and molecule counts exact; running energies within
1e-10 relative; final coordinates, centres, lookup order, move scales and
counts as the reference's (coordinates to 1e-9 A: the device's cube root
and exponential may differ from the host library's in the last bit).
Mixed form (FP32 pair energies on exact fixed-point separations, FP64
sums): the same first 2,000 decisions and running energies within 1e-6 of
an FP64 recompute after the full run.
"""
import numpy as np
import pytest

from tests.golden_util import load_gemc

pytestmark = pytest.mark.gpu

REL = 1e-10


@pytest.fixture(scope="module")
def gb():
    from gomc_gb300 import engine
    engine.lib(build_if_missing=True)
    return engine


def make(gb, z, meta, precision, cluster=0):
    g = meta["gemc"]
    return gb.Gemc(z["pos0"], z["pos1"], z["box0"], z["box1"],
                   z["kind_eps"][0], z["kind_sigma"][0], z["kind_n"][0],
                   g["temperature"], g["rcut"], g["random_seed"],
                   [g["dis_freq"], g["vol_freq"], g["swap_freq"]],
                   g["adj_steps"], g["cbmc_first"], precision=precision,
                   cluster_size=cluster)


@pytest.mark.parametrize("cluster", [16, 4])
def test_gemc_fp64_matches_reference(gb, cluster):
    z, meta = load_gemc()
    gm = make(gb, z, meta, gb.GB_FP64, cluster)
    e0 = gm.state()["energy"]
    for b in range(2):
        ref = meta["init"]["box%d_inter" % b]
        assert abs(e0[b] - ref) <= REL * abs(ref), (b, e0[b], ref)
    tr = z["trace"]
    r = gm.run(len(tr), trace=True)
    np.testing.assert_array_equal(r["kind"], tr[:, 1].astype(int))
    np.testing.assert_array_equal(r["box"], tr[:, 2].astype(int))
    vol = r["kind"] == 13
    np.testing.assert_array_equal(r["mol"][~vol], tr[~vol, 3].astype(int))
    np.testing.assert_array_equal(r["accepted"], tr[:, 4].astype(int))
    np.testing.assert_array_equal(r["n0"], tr[:, 9].astype(int))
    np.testing.assert_array_equal(r["volume"], tr[:, 7:9])
    ref = tr[:, 5:7]
    err = np.abs(r["energy"] - ref)
    assert (err <= REL * np.maximum(np.abs(ref), 1.0)).all(), err.max()
    st = gm.state()
    xyz, com, lk = gm.coords()
    np.testing.assert_array_equal(lk, z["lookup_final"])
    assert st["n0"] == int(z["lookup_counts"][0])
    np.testing.assert_allclose(xyz, z["coords_final"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(com, z["com_final"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(st["axes"], z["axes_final"], rtol=1e-14,
                               atol=0)
    for row in z["settings_final"]:  # box, move, tries, accepted, scale
        b, mv = int(row[0]), int(row[1])
        k = {0: 0, 10: 1, 13: 2}[mv]
        assert st["counts"][b, k, 0] == row[2]
        assert st["counts"][b, k, 1] == row[3]
        if mv == 0:
            assert abs(st["scales"][b, 0] - row[4]) <= 1e-12 * row[4]
        elif mv == 13:
            assert abs(st["scales"][b, 1] - row[4]) <= 1e-12 * row[4]
    tot = gm.system_total()
    for b in range(2):
        ref = meta["final"]["recalc%d_inter" % b]
        assert abs(tot[b] - ref) <= REL * abs(ref), (b, tot[b], ref)
        assert abs(st["energy"][b] - tot[b]) <= REL * abs(tot[b])
    gm.close()


def test_gemc_mixed_against_fp64(gb):
    z, meta = load_gemc()
    n = len(z["trace"])
    gf = make(gb, z, meta, gb.GB_FP64)
    gm = make(gb, z, meta, gb.GB_MIXED)
    rf = gf.run(n, trace=True)
    rm = gm.run(n, trace=True)
    k = 2000
    np.testing.assert_array_equal(rm["kind"][:k], rf["kind"][:k])
    np.testing.assert_array_equal(rm["accepted"][:k], rf["accepted"][:k])
    st = gm.state()
    tot = gm.system_total()
    for b in range(2):
        assert abs(st["energy"][b] - tot[b]) <= 1e-6 * abs(tot[b]), (
            b, st["energy"][b], tot[b])
    gf.close()
    gm.close()


def test_gemc_continues_across_launches(gb):
    """Two launches of 3,000 steps give the run of one launch of 6,000."""
    z, meta = load_gemc()
    a = make(gb, z, meta, gb.GB_FP64)
    b = make(gb, z, meta, gb.GB_FP64)
    ra = a.run(6000, trace=True)
    r1 = b.run(3000, trace=True)
    r2 = b.run(3000, trace=True)
    for key in ("kind", "mol", "accepted"):
        np.testing.assert_array_equal(ra[key],
                                      np.concatenate([r1[key], r2[key]]))
    xa, ca, la = a.coords()
    xb, cb, lb = b.coords()
    np.testing.assert_array_equal(xa, xb)
    np.testing.assert_array_equal(la, lb)
    np.testing.assert_array_equal(a.state()["energy"], b.state()["energy"])
    a.close()
    b.close()
