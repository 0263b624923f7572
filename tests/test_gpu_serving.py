"""Continuous-batching job server (gb_server_*) on the GPU.

* alone vs in the mix: jobs of different sizes, submitted at different
  rounds and sharing rounds with each other, end in the same coordinates and
  energies, bit for bit, as each job run by itself;
* the served result is physical: the job's running energies agree with a
  full FP64 recompute of its final coordinates to 1e-6 relative per term
  (the mixed form's bar);
* admission by device memory: with a budget for about two jobs, no more than
  two are resident at once and every job still finishes;
* the worker thread: jobs submitted while others run are admitted and
  finish; the statistics count every move.
"""
import numpy as np
import pytest

from gomc_gb300.config import SimConfig
from gomc_gb300.systems import spce_water_box, water_box_length

pytestmark = pytest.mark.gpu

TERM_REL = 1e-6
SCALES = [0.3, 0.3, 0.02, 0.03]
CFG = SimConfig(temperature=298.0, rcut=9.0, tolerance=1e-5)
# (molecules, seed, moves): cluster sizes 2, 4 and 8 by k-vector count
JOBS = [(300, 1, 1500), (700, 2, 2500), (2000, 3, 1200), (500, 4, 900)]


@pytest.fixture(scope="module")
def srv_mod():
    from gomc_gb300 import engine, serving
    engine.lib(build_if_missing=True)
    return serving


def system(n, seed):
    return spce_water_box(n, water_box_length(n), seed=seed)


def submit(srv, n, seed, moves):
    return srv.submit(system(n, seed), CFG, seed=100 + seed, nsteps=moves,
                      scales=SCALES, adj_steps=500, recompute_freq=1000)


def test_alone_equals_mixed(srv_mod):
    mixed = srv_mod.Server(quantum=400)
    ids = [submit(mixed, *JOBS[0]), submit(mixed, *JOBS[1])]
    mixed.step()
    mixed.step()
    ids += [submit(mixed, *JOBS[2])]
    mixed.step()
    ids += [submit(mixed, *JOBS[3])]
    mixed.run_until_idle()
    st = mixed.stats()
    assert st["jobs_done"] == len(JOBS)
    assert st["moves"] == sum(j[2] for j in JOBS)
    assert st["mean_resident"] > 1.0  # the jobs did share rounds
    # occupancy statistics: fractions in [0, 1], counts non-negative
    assert st["mean_admitted"] > 0.0 and st["mean_in_round"] > 0.0
    assert 0.0 < st["cta_slot_frac"] <= 1.0
    assert 0.0 < st["smem_frac"] <= 1.0
    assert 0.0 < st["launch_balance"] <= 1.0 + 1e-9
    assert min(st["stops_mem"], st["stops_smem"], st["stops_ctas"],
               st["round_gap_s"], st["mean_queued"]) >= 0.0
    res_mixed = [mixed.result(i) for i in ids]
    mixed.close()
    for job, rm in zip(JOBS, res_mixed):
        alone = srv_mod.Server(quantum=400)
        i = submit(alone, *job)
        alone.run_until_idle()
        ra = alone.result(i)
        alone.close()
        np.testing.assert_array_equal(rm["xyz"], ra["xyz"])
        np.testing.assert_array_equal(rm["com"], ra["com"])
        np.testing.assert_array_equal(rm["energy"], ra["energy"])


def test_served_energies_match_fp64(srv_mod):
    from gomc_gb300 import engine
    srv = srv_mod.Server(quantum=500)
    n, seed, moves = JOBS[1]
    i = submit(srv, n, seed, moves)
    srv.run_until_idle()
    r = srv.result(i)
    srv.close()
    s = system(n, seed)
    s.pos = r["xyz"].copy()
    box = engine.Box(s, CFG, precision=engine.GB_FP64)
    tot = box.system_total()
    for k, term in enumerate(["inter", "real", "recip"]):
        rel = abs(r["energy"][k] - tot[term]) / abs(tot[term])
        assert rel <= TERM_REL, (term, rel)
    box.close()


def test_memory_admission(srv_mod):
    probe = srv_mod.Server(quantum=300)
    est = probe.estimate(system(700, 10), CFG)["bytes"]
    probe.close()
    # a budget with room for two 700-water jobs by the admission estimate
    srv = srv_mod.Server(quantum=300, mem_budget=int(2.5 * est))
    ids = [submit(srv, 700, s, 900) for s in range(10, 15)]
    peak = 0
    while True:
        left = srv.step()
        running = sum(srv.job(j)["status"] == "running" for j in ids)
        peak = max(peak, running)
        if not left:
            break
    assert all(srv.job(j)["status"] == "done" for j in ids)
    assert peak == 2, peak
    srv.close()


def test_worker_thread(srv_mod):
    import time
    srv = srv_mod.Server(quantum=500)
    srv.start()
    ids = []
    for n, seed, moves in JOBS:
        ids.append(submit(srv, n, seed, moves))
        time.sleep(0.05)
    srv.drain(timeout_s=300)
    st = srv.stats()
    assert st["jobs_done"] == len(JOBS)
    assert st["moves"] == sum(j[2] for j in JOBS)
    assert 0 < st["sweep_p50_ms"] <= st["sweep_p99_ms"]
    for j in ids:
        info = srv.job(j)
        assert info["status"] == "done"
        assert info["t_submit"] <= info["t_admit"] <= info["t_done"]
    srv.close()
