"""Serving: continuous batching of solve requests.  Every request's result in
the mix must equal the same request solved alone (objective within 1e-6
relative, same support; SVM objective within 1e-5), requests that arrive while
others run are admitted between rounds, the memory budget queues requests, a
request larger than the budget is refused, and a malformed request fails
without disturbing the others."""
import numpy as np
import pytest

import acdc

pytestmark = pytest.mark.gpu


def requests(seed, count):
    out = []
    for i in range(count):
        if i % 3 == 2:
            out.append(acdc.gen_svm(400 + 50 * i, 3000, nnz_median=40, w_star_nnz=200,
                                    lam=2e-3, seed=seed + i))
        else:
            m, n = acdc.mix_sizes(seed, i, m_lo=300, m_hi=2000, n_lo=500, n_hi=4000)
            out.append(acdc.gen_lasso(m, n, nnz_mode=acdc.NNZ_UNIFORM, nnz_min=5, nnz_max=20,
                                      n_star=min(20, n // 10), lambda_frac=0.2, seed=seed + i))
    return out


def alone(ctx, inst):
    """The same request through the plain single-problem path."""
    p = acdc.Problem(ctx, inst)
    res, xs = acdc.batch_solve_path(ctx, [p], np.array([[inst.lam]]), gap_target=1e-6,
                                    max_epochs=2000, refresh_every=1, autotune=1, plain=1,
                                    want_x=True)
    p.close()
    return res[0][0], xs[0]


def drain(server, tickets, max_steps=20000):
    for _ in range(max_steps):
        if server.step() == 0:
            break
    return [server.poll(t, want_x=True) for t in tickets]


def check_same(r_mix, x_mix, r_alone, x_alone, inst):
    tol = 1e-5 if inst.loss == acdc.LOSS_SVM_DUAL else 1e-6
    assert r_mix.converged and r_alone.converged
    assert abs(r_mix.eval.primal - r_alone.eval.primal) <= tol * abs(r_alone.eval.primal)
    if inst.loss == acdc.LOSS_L1_SQUARE:
        assert set(np.nonzero(x_mix)[0]) == set(np.nonzero(x_alone)[0])


def test_each_result_is_the_same_alone_and_in_the_mix(ctx):
    insts = requests(100, 9)
    server = acdc.Server(ctx, memory_budget_bytes=8 << 30, max_slots=64, quantum_rounds=2)
    tickets = [server.submit(inst) for inst in insts[:5]]
    server.step()  # the first five start running
    tickets += [server.submit(inst) for inst in insts[5:]]  # arrive while others run
    results = drain(server, tickets)
    for inst, (res, x) in zip(insts, results):
        assert acdc.Server.STATES[res.state] == "done", res.status
        assert res.submit_time <= res.start_time <= res.finish_time
        r_alone, x_alone = alone(ctx, inst)
        check_same(res, x, r_alone, x_alone, inst)
    st = server.stats()
    assert st["admitted"] == st["retired"] == len(insts)
    assert st["steps"] >= 2 and st["builds"] >= 2 and st["rounds"] >= st["builds"]
    assert min(st["admit_s"], st["build_s"], st["rounds_s"], st["retire_s"]) > 0
    for t in tickets:
        server.release(t)
    server.close()


def test_cancel_leaves_the_others_as_they_would_be(ctx):
    """A running and a queued request cancelled between steps end failed with
    ACDC_ECANCELED and give their memory back; the rest finish as they would
    alone; cancelling a finished request changes nothing."""
    insts = requests(300, 6)
    server = acdc.Server(ctx, memory_budget_bytes=8 << 30, max_slots=3, quantum_rounds=2)
    tickets = [server.submit(inst) for inst in insts]  # three run, three wait
    server.step()
    states = [server.poll(t)[0].state for t in tickets]
    assert states[1] == 1 and states[4] == 0  # running (tables built), still queued
    server.cancel(tickets[1])  # running
    server.cancel(tickets[4])  # queued
    results = drain(server, tickets)
    for i, (inst, (res, x)) in enumerate(zip(insts, results)):
        if i in (1, 4):
            assert res.state == 3 and res.status == acdc.ECANCELED
            continue
        assert acdc.Server.STATES[res.state] == "done", res.status
        r_alone, x_alone = alone(ctx, inst)
        check_same(res, x, r_alone, x_alone, inst)
    server.cancel(tickets[0])  # finished: no change
    assert server.poll(tickets[0])[0].state == 2
    st = server.stats()
    assert st["admitted"] == 5 and st["retired"] == 4
    for t in tickets:
        server.release(t)
    server.close()


def test_memory_budget_queues_and_refuses(ctx):
    insts = requests(200, 4)
    lasso = [inst for inst in insts if inst.loss == acdc.LOSS_L1_SQUARE]

    def footprint(inst):  # the server's admission estimate (batch.cu footprint_of)
        return 20 * inst.nnz + 136 * inst.n + 32 * inst.m + (1 << 20)

    # largest first, with a budget that holds only that one
    lasso.sort(key=footprint, reverse=True)
    server = acdc.Server(ctx, memory_budget_bytes=footprint(lasso[0]) + (1 << 20), max_slots=8,
                         quantum_rounds=2)
    tickets = [server.submit(inst) for inst in lasso]
    server.step()
    states = [acdc.Server.STATES[server.poll(t)[0].state] for t in tickets]
    assert states.count("queued") >= 1  # the budget made some wait
    results = drain(server, tickets)
    assert all(acdc.Server.STATES[r.state] == "done" for r, _ in results)
    huge = acdc.gen_lasso(200000, 400000, nnz_per_col=20, n_star=10, seed=3)
    with pytest.raises(acdc.AcdcError) as e:
        server.submit(huge)
    assert e.value.code == acdc.EBUSY
    server.close()


def test_malformed_request_fails_alone(ctx):
    insts = requests(300, 3)
    bad = insts[0]
    bad_idx = bad.row_idx.copy()
    bad_idx[3] = bad.m + 5  # caught by the layout kernel's bounds check
    broken = acdc.Instance(bad.loss, bad.m, bad.n, bad.col_ptr, bad_idx, bad.vals, bad.rhs, bad.lam)
    server = acdc.Server(ctx, memory_budget_bytes=4 << 30, max_slots=8, quantum_rounds=2)
    tickets = [server.submit(broken)] + [server.submit(inst) for inst in insts[1:]]
    results = drain(server, tickets)
    assert acdc.Server.STATES[results[0][0].state] == "failed"
    assert results[0][0].status == acdc.EDEVICE
    for inst, (res, x) in zip(insts[1:], results[1:]):
        assert acdc.Server.STATES[res.state] == "done"
        r_alone, x_alone = alone(ctx, inst)
        check_same(res, x, r_alone, x_alone, inst)
    server.close()
