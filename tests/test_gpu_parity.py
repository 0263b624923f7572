"""GPU energy path (FP64 plain form) against the reference's golden vectors.

Bars (FP64 plain form): every energy term within 1e-10 relative; cell
membership, k-vector tables and initial coordinates bit-exact; per-move
accept/reject sequence identical to the reference's over the golden traces.
"""
import numpy as np
import pytest

from tests.golden_util import (NAMES, PI_NAMES, SMI_NAMES, config_of, load,
                               load_pi, load_smi, load_virial,
                               move_fractions, system_of)

pytestmark = pytest.mark.gpu

REL = 1e-10


@pytest.fixture(scope="module")
def gb():
    from gomc_gb300 import engine
    engine.lib(build_if_missing=True)
    return engine


def close(a, b, rel=REL, scale=None):
    s = abs(b) if scale is None else scale
    return abs(a - b) <= rel * max(s, 1e-300)


@pytest.mark.parametrize("name", NAMES)
def test_initial_state(gb, name):
    z, meta = load(name)
    box = gb.Box(system_of(z, meta), config_of(meta))
    st = box.system_total()
    for term in ("inter", "real", "recip", "self", "correction", "total"):
        ref = meta["init"]["box0_" + term]
        assert close(st[term], ref, scale=max(abs(ref), 1.0)), (term, st[term], ref)
    np.testing.assert_array_equal(box.coords(), z["coords_init"])
    np.testing.assert_array_equal(box.com(), z["com_init"].reshape(-1, 3))
    cells, edge = box.cell_membership()
    assert list(edge) == meta["init"]["edgeCells"]
    ref_cells = np.full(box.n_atoms, -1)
    ref_cells[z["cells"][:, 0]] = z["cells"][:, 1]
    np.testing.assert_array_equal(cells, ref_cells)
    if "kvec" in z:
        kv = box.kvectors()
        K, _ = box.num_kvectors()
        assert K == int(meta["init"]["imageSize"])
        for i, key in enumerate(["kx", "ky", "kz"]):
            np.testing.assert_array_equal(kv[key], z["kvec"][:, i])
        np.testing.assert_array_equal(kv["hsqr"], z["kvec"][:, 6])
        # prefactors go through the host libm's exp(): equal to a few ulp
        # across x86-64 and aarch64 C libraries
        np.testing.assert_allclose(kv["prefact"], z["kvec"][:, 3], rtol=1e-14,
                                   atol=0)
        smax = np.abs(z["kvec"][:, 4:6]).max()
        np.testing.assert_allclose(kv["sumRref"], z["kvec"][:, 4], rtol=0,
                                   atol=REL * smax)
        np.testing.assert_allclose(kv["sumIref"], z["kvec"][:, 5], rtol=0,
                                   atol=REL * smax)
    box.close()


@pytest.mark.parametrize("name", NAMES)
def test_proposal_deltas(gb, name):
    z, meta = load(name)
    box = gb.Box(system_of(z, meta), config_of(meta))
    st = box.system_total()
    cur = box.coords()
    ms = z["mol_start"]
    ewald = meta["config"]["ewald"]
    # scale for differences: the box-term magnitude
    s_lj = abs(meta["init"]["box0_inter"])
    s_re = abs(meta["init"]["box0_real"]) if ewald else 1.0
    s_rc = abs(meta["init"]["box0_recip"]) if ewald else 1.0
    for i, m in enumerate(z["prop_mol"]):
        ref = z["prop_out"][i]
        ov, lj, re = box.molecule_inter(int(m), z["prop_pos"][i])
        assert int(ov) == int(ref[1])
        assert close(lj, ref[2], scale=s_lj), (i, lj, ref[2])
        assert close(re, ref[3], scale=s_re), (i, re, ref[3])
        if ewald:
            assert close(box.mol_reciprocal(int(m), z["prop_pos"][i]), ref[4],
                         scale=s_rc)
            assert close(box.swap_dest_recip(int(m), z["prop_pos"][i]), ref[5],
                         scale=s_rc)
            old = cur[ms[m]:ms[m + 1]]
            assert close(box.swap_source_recip(int(m), old), ref[6], scale=s_rc)
    box.close()


def test_forces(gb):
    z, meta = load("c0_water_mp")
    box = gb.Box(system_of(z, meta), config_of(meta))
    aF, mF, lj, re = box.box_force()
    box.copy_recip()
    aR, mR = box.box_force_reciprocal()
    tq = box.calculate_torque()
    fa, fm = z["forces_atom"], z["forces_mol"]
    for got, ref in ((aF, fa[:, 0:3]), (aR, fa[:, 3:6]), (mF, fm[:, 0:3]),
                     (mR, fm[:, 3:6]), (tq, fm[:, 6:9])):
        np.testing.assert_allclose(got, ref, rtol=0,
                                   atol=REL * np.abs(ref).max())
    assert close(lj, meta["force_energy"]["inter"])
    assert close(re, meta["force_energy"]["real"])
    box.close()


@pytest.mark.parametrize("name", NAMES)
def test_mc_trace_matches_reference(gb, name):
    z, meta = load(name)
    box = gb.Box(system_of(z, meta), config_of(meta))
    box.mc_init(meta["config"]["random_seed"], move_fractions(meta),
                meta["config"]["adj_steps"])
    tr = z["trace"]
    n = tr.shape[0]
    r = box.mc_run(0, n, trace=True)
    np.testing.assert_array_equal(r["kind"], tr[:, 1].astype(int))
    np.testing.assert_array_equal(r["mol"], tr[:, 2].astype(int))
    np.testing.assert_array_equal(r["accepted"], tr[:, 3].astype(int))
    scale = np.maximum(np.abs(tr[-1, 8:11]), 1.0)
    single = tr[:, 1] < 2
    # 1e-10 of the box energy, or of the move's own change where that is
    # larger (near-overlap proposals of the sparse LJ box change the energy
    # by up to 1e11 K)
    for j in range(3):
        ref = tr[single, 5 + j]
        bound = REL * np.maximum(scale[j], np.abs(ref))
        err = np.abs(r["de"][single, j] - ref)
        assert (err <= bound).all(), (j, np.argwhere(err > bound)[:5].ravel(),
                                      err.max())
    mp = ~single
    if mp.any():
        for j in range(3):
            np.testing.assert_allclose(r["de"][mp, j], tr[mp, 5 + j], rtol=0,
                                       atol=REL * scale[j])
    e = box.energy()
    for j in range(3):
        assert close(e[j], tr[-1, 8 + j], scale=scale[j])
    np.testing.assert_allclose(box.coords(), z["coords_final"], rtol=0,
                               atol=1e-9)
    sc, cnt = box.mc_state()
    for k in range(3):
        key = "move%d" % k
        if key in meta["final"]:
            tries, acc, scl = meta["final"][key]
            assert cnt[2 * k] == tries and cnt[2 * k + 1] == acc
            if k < 2:
                assert close(sc[k], scl, rel=1e-12)
    # running totals agree with a fresh recompute
    st = box.system_total()
    for j, term in enumerate(("inter", "real", "recip")):
        assert close(e[j], st[term], scale=scale[j])
    box.close()


@pytest.mark.parametrize("name", PI_NAMES)
def test_particle_inter(gb, name):
    """ParticleInter (the CBMC first-atom trial energies) against the
    reference's vectors, cases in the reference's order: with the molecule
    taken out of the cell list around the call (as MoleculeTransfer does) or
    left in.  Each energy within 1e-10 of max(|value|, 1 K); overlap flags
    equal."""
    z, meta = load(name)
    g = load_pi(name)
    box = gb.Box(system_of(z, meta), config_of(meta))
    for c in range(len(g["mol"])):
        m, part, rm = int(g["mol"][c]), int(g["part"][c]), int(g["remove"][c])
        if rm:
            box.cell_remove_mol(m)
        ov, en, re = box.particle_inter(m, part, g["trials"][c])
        if rm:
            box.cell_add_mol(m)
        np.testing.assert_array_equal(ov.astype(int), g["overlap"][c])
        for got, ref in ((en, g["en"][c]), (re, g["real"][c])):
            err = np.abs(got - ref)
            assert (err <= REL * np.maximum(np.abs(ref), 1.0)).all(), (
                c, got, ref)
    # a molecule out of the cell list blocks the Monte Carlo loop until it
    # is back
    box.cell_remove_mol(0)
    box.mc_init(1, [0.5, 0.5, 0.0], 1000)
    with pytest.raises(RuntimeError):
        box.mc_run(0, 10)
    box.cell_add_mol(0)
    box.mc_run(0, 10)
    box.close()


@pytest.mark.parametrize("name", SMI_NAMES)
def test_single_molecule_inter(gb, name):
    """SingleMoleculeInter on the GPU against the reference's vectors: every
    output within 1e-10 relative (1e-10 K absolute for values near 0)."""
    import dataclasses
    z, meta = load(name)
    g = load_smi(name)
    a, s, p = g["soft_core"]
    boxes = {}
    for c in (0, 1):
        cfg = dataclasses.replace(config_of(meta), sc_alpha=float(a),
                                  sc_sigma=float(s), sc_power=int(p),
                                  sc_coul=bool(c))
        boxes[c] = gb.Box(system_of(z, meta), cfg)
    for m, lam, c, ref in zip(g["mol"], g["lam"], g["sc_coul"], g["out"]):
        got = boxes[int(c)].single_molecule_inter(int(m), lam)
        for x, y in zip(got, ref):
            assert abs(x - y) <= REL * max(abs(y), 1.0), (m, lam, c, got, ref)
    for b in boxes.values():
        b.close()


@pytest.mark.parametrize("name", NAMES)
def test_virial(gb, name):
    """VirialCalc on the GPU against the reference: every scalar and tensor
    component within 1e-10 of the largest virial term (the components are
    sums of cancelling terms, so each is held to the scale of the whole)."""
    z, meta = load(name)
    box = gb.Box(system_of(z, meta), config_of(meta))
    got, ref = box.virial(), load_virial(name)
    scale = np.abs(ref[:4]).max()
    for i, (x, y) in enumerate(zip(got, ref)):
        assert abs(x - y) <= REL * scale, (i, x, y)
    p = box.pressure()
    assert np.isfinite(p)
    box.close()
