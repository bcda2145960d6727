"""The serving loop (include/eqserve.h) on the GPU: continuous batching, admission by
device-memory footprint, and every result the same alone and in the mix."""
import time

import numpy as np
import pytest

from eq_gb300 import field as F
from eq_gb300 import serve as S
from eq_gb300 import workloads as wl
from oracle import hsld

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / max(np.linalg.norm(b), 1e-300))


def small_traps(n, seed=5):
    """Uneven traps of the batched workload's physics (h = 0.25 um, D = 490) at a
    smaller size range, for test time; all share the multigrid depth."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        nx, ny = int(rng.integers(16, 129)), int(rng.integers(8, 65))
        W, H = 0.25 * nx, 0.25 * ny
        m = max(4, nx * ny // 50)
        xy = np.stack([rng.uniform(0.1, W - 0.1, m), rng.uniform(0.1, H - 0.1, m)], axis=1)
        out.append(wl.Trap(W=W, H=H, nx=nx, ny=ny, D=[490.0], g=[0.01], dt=0.1, steps=10,
                           cell_xy=xy, cell_s=rng.lognormal(0.0, 0.5, m)))
    return out


def params1(t):
    return [F.trap_params(t.W, t.H, t.nx, t.ny, t.D[0], t.dt, t.g[0], t.walls)]


def params2(t):
    return [F.trap_params(t.W, t.H, t.nx, t.ny, t.D[k], t.dt, t.g[k], t.walls, adv_u=t.adv_u,
                          adv_len=t.adv_len) for k in range(2)]


def submit(srv, t, steps, two=False):
    if two:
        return srv.submit(params2(t), t.cell_xy, t.cell_s, steps, sender=t.cell_kind)
    return srv.submit(params1(t), t.cell_xy, t.cell_s, steps)


def run_alone(t, steps, two=False):
    with S.Server(S.default_config(min_batch=1)) as srv:
        rid = submit(srv, t, steps, two)
        srv.drain()
        r = srv.result(rid)
        assert r.status == 0
        return r.cells


def test_results_alone_and_in_the_mix(lib):
    traps = small_traps(12)
    steps = [3 + (7 * i) % 11 for i in range(len(traps))]
    pair = wl.scaled(wl.two_species(2), 64, 32, n_cells=120)
    alone = [run_alone(t, k) for t, k in zip(traps, steps)]
    alone_pair = run_alone(pair, 6, two=True)
    cfg = S.default_config(min_batch=4, max_wait_ms=1.0, max_cohort_traps=8)
    with S.Server(cfg) as srv:
        ids = []
        for i, (t, k) in enumerate(zip(traps, steps)):
            ids.append(submit(srv, t, k))
            if i == 5:
                pid = submit(srv, pair, 6, two=True)
            srv.progress()
        srv.drain()
        st = srv.stats()
        res = [srv.result(i) for i in ids]
        rp = srv.result(pid)
    assert st["completed"] == len(traps) + 1 and st["failed"] == 0
    assert st["cohorts"] >= 2
    for r, a in zip(res, alone):
        assert r.status == 0
        # class-pure cohorts: the same bits alone and in the mix
        assert np.array_equal(r.cells, a)
    assert np.array_equal(rp.cells, alone_pair)
    assert rp.cohort not in {r.cohort for r in res}  # another class, its own cohort


def test_served_result_against_the_oracle(lib):
    t = small_traps(3)[1]
    ref = hsld.run_trap(t, steps=9)
    with S.Server(S.default_config(min_batch=1)) as srv:
        rid = srv.submit(params1(t), t.cell_xy, t.cell_s, 9, want_nodal=True)
        srv.drain()
        r = srv.result(rid)
    assert r.status == 0
    assert rel(r.nodal[0], ref["u"][0]) <= 1e-6
    assert rel(r.cells[0], ref["cells"][0]) <= 1e-6


def test_admission_respects_the_memory_budget(lib):
    traps = small_traps(8)
    opts = F.default_opts(F.FP32_IR)
    need = [F.footprint_estimate(params1(t), opts, t.n_cells) for t in traps]
    budget = int(2.5 * max(need))
    cfg = S.default_config(min_batch=1, max_wait_ms=0.0, hbm_budget=budget)
    with S.Server(cfg) as srv:
        ids = [submit(srv, t, 5) for t in traps]
        srv.drain()
        st = srv.stats()
        for i in ids:
            assert srv.result(i).status == 0
    assert sum(need) > budget  # not everything fits at once ...
    assert st["cohorts"] >= 2  # ... so the requests ran in several cohorts
    assert st["bytes_peak"] <= budget


def test_request_larger_than_the_budget_is_refused(lib):
    t = small_traps(1)[0]
    with S.Server(S.default_config(hbm_budget=1 << 16)) as srv:
        with pytest.raises(F.EqfError) as e:
            submit(srv, t, 3)
        assert e.value.code == -6


def test_arrivals_join_while_others_run(lib):
    big = wl.scaled(wl.single_large(1), 512, 256, n_cells=500)
    small = small_traps(2)[0]
    cfg = S.default_config(min_batch=1, max_wait_ms=0.0)
    with S.Server(cfg) as srv:
        a = submit(srv, big, 40)
        srv.progress()
        time.sleep(0.05)
        srv.progress()
        b = submit(srv, small, 2)
        srv.drain()
        ra, rb = srv.result(a), srv.result(b)
    assert ra.status == 0 and rb.status == 0
    assert rb.cohort != ra.cohort
    # b was admitted and finished while a was still running
    assert rb.t_admit < ra.t_done and rb.t_done < ra.t_done


def test_requests_reuse_the_slots_of_finished_ones(lib):
    """One resident cohort of four slots: the later, smaller requests run in the slots
    of the finished ones (eqf_replace_traps), with the bits they give alone."""
    rng = np.random.default_rng(11)
    big = []  # slot capacities: 128 x 64, the largest grid small_traps makes
    for _ in range(4):
        m = 160
        xy = np.stack([rng.uniform(0.1, 31.9, m), rng.uniform(0.1, 15.9, m)], axis=1)
        big.append(wl.Trap(W=32.0, H=16.0, nx=128, ny=64, D=[490.0], g=[0.01], dt=0.1,
                           steps=10, cell_xy=xy, cell_s=rng.lognormal(0.0, 0.5, m)))
    later = []  # grids that fit a 128 x 64 slot at every level (eqf_slot_fits)
    for nx, ny in ((85, 22), (87, 52), (41, 16), (96, 10), (120, 60), (64, 32)):
        m = max(4, nx * ny // 50)
        W, H = 0.25 * nx, 0.25 * ny
        xy = np.stack([rng.uniform(0.1, W - 0.1, m), rng.uniform(0.1, H - 0.1, m)], axis=1)
        later.append(wl.Trap(W=W, H=H, nx=nx, ny=ny, D=[490.0], g=[0.01], dt=0.1, steps=10,
                             cell_xy=xy, cell_s=rng.lognormal(0.0, 0.5, m)))
    steps_big = [2, 3, 4, 9]
    steps_later = [3, 5, 2, 4, 6, 3]
    alone_big = [run_alone(t, k) for t, k in zip(big, steps_big)]
    alone_later = [run_alone(t, k) for t, k in zip(later, steps_later)]
    cfg = S.default_config(min_batch=4, max_wait_ms=1e6, max_cohorts=1, max_cohort_traps=4)
    with S.Server(cfg) as srv:
        ids = [submit(srv, t, k) for t, k in zip(big, steps_big)]
        srv.progress()  # the cohort forms with the four large requests
        ids += [submit(srv, t, k) for t, k in zip(later, steps_later)]
        srv.drain()
        st = srv.stats()
        err = srv.last_error()
        res = [srv.result(i) for i in ids]
    assert st["completed"] == 10 and st["failed"] == 0
    assert st["cohorts"] == 1 and st["slot_admitted"] == 6, (st, err, [r.cohort for r in res])
    for r, a in zip(res, alone_big + alone_later):
        assert r.status == 0
        assert np.array_equal(r.cells, a)


def test_without_slot_reuse_every_admission_is_a_new_cohort(lib):
    """reuse_slots = 0: finished requests' slots stay frozen until their cohort ends,
    new requests form new cohorts; the results are the same bits."""
    traps = small_traps(6, seed=21)
    steps = [2, 5, 3, 4, 6, 2]
    alone = [run_alone(t, k) for t, k in zip(traps, steps)]
    cfg = S.default_config(min_batch=2, max_wait_ms=1e6, max_cohorts=1, max_cohort_traps=2,
                           reuse_slots=0)
    with S.Server(cfg) as srv:
        ids = [submit(srv, t, k) for t, k in zip(traps, steps)]
        srv.drain()
        st = srv.stats()
        res = [srv.result(i) for i in ids]
    assert st["completed"] == 6 and st["slot_admitted"] == 0 and st["cohorts"] == 3
    for r, a in zip(res, alone):
        assert r.status == 0 and np.array_equal(r.cells, a)
