"""The reference's checkpoint file (src/Checkpoint.h:27-169) through the C
ABI, on the host (no GPU).

`tests/golden/chk_c0_water.npz` holds the checkpoint the reference itself
wrote (CheckpointOutput::saveCheckpointFile) after 600 steps of c0_water's
Monte Carlo loop, with the loop state the reference held then.
gb_gomc_checkpoint_read returns that state; gb_gomc_checkpoint_write
reproduces the file byte for byte from its own reading, and a changed state
reads back changed with every later byte (lookup, molecule setup, atoms)
kept; where the reference is built in this container (oracle/_ref), the
reference's own deserializer reads the written file back.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from tests.golden_util import GOLDEN

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PROBE = os.path.join(ROOT, "oracle", "_ref", "ref_probe_ens1")


@pytest.fixture(scope="module")
def gb():
    from gomc_gb300 import engine
    engine.lib(build_if_missing=True)
    return engine


@pytest.fixture(scope="module")
def fx():
    z = np.load(os.path.join(GOLDEN, "chk_c0_water.npz"))
    meta = json.loads(bytes(z["meta_json"]).decode())
    return z, meta


def check_state(c, steps, mt, seeds, moves, mp, mpmax):
    assert (c.step, c.true_step) == tuple(int(v) for v in steps)
    np.testing.assert_array_equal(np.array(c.mt_state[:]), mt[:624])
    assert c.mt_left == int(mt[624])
    assert (c.seed_location, c.seed_left, c.seed_value) == tuple(
        int(v) for v in seeds)
    assert c.n_box == 1 and c.n_move == len(moves) and c.n_kind == 1
    for m, row in enumerate(moves):
        assert c.scale[0][m] == row[0] and c.accept_percent[0][m] == row[1]
        assert (c.accepted[0][m], c.tries[0][m], c.temp_accepted[0][m],
                c.temp_tries[0][m]) == tuple(int(v) for v in row[2:])
    for t in range(2):
        assert (c.mp_tries[0][t], c.mp_accepted[0][t],
                c.mp_interval_tries[0][t], c.mp_interval_accepted[0][t]) == \
            tuple(int(v) for v in mp[t])
    assert c.mp_t_max[0] == mpmax[0] and c.mp_r_max[0] == mpmax[1]
    assert c.single_move_accepted[0] == int(mpmax[2])


def test_read_returns_reference_state(gb, fx):
    z, meta = fx
    c = gb.gomc_checkpoint_read(bytes(z["chk"]))
    check_state(c, z["chk_steps"], z["chk_mt"], z["chk_seeds"],
                z["chk_moves"], z["chk_mp"], z["chk_mpmax"])
    assert c.step == meta["chk_step"]


def test_write_round_trip_and_changed_state(gb, fx):
    z, _ = fx
    data = bytes(z["chk"])
    c = gb.gomc_checkpoint_read(data)
    assert gb.gomc_checkpoint_write(data, c) == data
    c.step, c.true_step = 1234, 1234
    c.scale[0][0], c.scale[0][1] = 0.5, 0.25
    c.tries[0][0] += 7
    c.mp_t_max[0] = 0.03
    mt = np.array(c.mt_state[:], dtype=np.uint32)[::-1].copy()
    c.mt_state[:] = mt.tolist()
    c.seed_location, c.seed_left, c.mt_left = 100, 524, 524
    w = gb.gomc_checkpoint_write(data, c)
    c2 = gb.gomc_checkpoint_read(w)
    assert (c2.step, c2.true_step) == (1234, 1234)
    assert (c2.scale[0][0], c2.scale[0][1]) == (0.5, 0.25)
    assert c2.tries[0][0] == c.tries[0][0] and c2.mp_t_max[0] == 0.03
    np.testing.assert_array_equal(np.array(c2.mt_state[:]), mt)
    assert (c2.seed_location, c2.seed_left, c2.mt_left) == (100, 524, 524)
    # the records after the loop state are the template's
    assert w[c2.records_offset:] == data[c.records_offset:]


@pytest.mark.skipif(not os.path.exists(PROBE),
                    reason="the reference is not built in this container")
def test_reference_reads_written_file(gb, fx, tmp_path):
    z, _ = fx
    data = bytes(z["chk"])
    c = gb.gomc_checkpoint_read(data)
    c.step, c.true_step = 777, 778
    c.scale[0][0] = 0.125
    c.accepted[0][1] += 3
    path = tmp_path / "written.chk"
    path.write_bytes(gb.gomc_checkpoint_write(data, c))
    subprocess.check_call([PROBE, "--read-chk", str(path), str(tmp_path)],
                          stdout=subprocess.DEVNULL)
    lines = (tmp_path / "chk_state.txt").read_text().split("\n")
    assert lines[0].split() == ["777", "778"]
    moves = [ln.split() for ln in lines[628:630]]
    assert float(moves[0][0]) == 0.125
    assert int(moves[1][2]) == c.accepted[0][1]
    np.testing.assert_array_equal(
        np.array([int(v) for v in lines[1:625]], dtype=np.uint64),
        z["chk_mt"][:624])


def test_rejects_malformed(gb, fx):
    from gomc_gb300._lib import GbError
    z, _ = fx
    data = bytes(z["chk"])
    for bad in (data[:100], data[:3000], b"\x00" * 16,
                data[:2553] + b"\xff" * 8 + data[2561:]):
        with pytest.raises(GbError):
            gb.gomc_checkpoint_read(bad)
