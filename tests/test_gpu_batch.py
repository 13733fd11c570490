"""Batched and served solves on the device.

Every problem of a batch, and every request of a served trace, must produce
exactly what the same problem produces when solved alone with the same tile
size: the batched kernels run the single-problem bodies per work item."""
import numpy as np
import pytest

from hsrq3in_gb300 import generators as G

pytestmark = pytest.mark.gpu


def _mixed(count, seed, nlo, nhi):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(round(np.exp(rng.uniform(np.log(nlo), np.log(nhi)))))
        H, lam = G.real_spectrum(n, seed * 1000 + i)
        wr = G.shift_subset(G.perturbed_shifts(lam, seed * 1000 + i + 1), rng, 0.25, 1.0)
        out.append((H, wr))
    return out


def _dev_problem(torch, H, wr, dev):
    n = H.shape[0]
    ld = n + (n & 1)
    dH = torch.zeros((n, ld), dtype=torch.float64, device=dev)
    dH[:, :n] = torch.from_numpy(np.ascontiguousarray(H.T)).to(dev)
    dwr = torch.from_numpy(np.ascontiguousarray(wr)).to(dev)
    dvr = torch.full((len(wr), ld), float("nan"), dtype=torch.float64, device=dev)
    return dH, dwr, dvr


@pytest.mark.parametrize("tlsz", [32, 64])
def test_batched_equals_alone(gpu_lib, tlsz):
    import torch
    import hsrq3in_gb300 as hsr
    dev = torch.device("cuda", 0)
    probs = _mixed(40, 3, 12, 300)
    tens = [_dev_problem(torch, H, wr, dev) for H, wr in probs]
    plan = hsr.BatchPlan(tens, tlsz=tlsz)
    for rep in range(2):                       # the graph replays identically
        for _, _, dvr in tens:
            dvr.fill_(float("nan"))
        plan.execute()
        torch.cuda.synchronize()
        for (H, wr), (dH, dwr, dvr) in zip(probs, tens):
            n = H.shape[0]
            alone = hsr.inverse_iteration(H, wr, tlsz, 16)
            assert np.array_equal(dwr.cpu().numpy(), alone["wr"])
            assert np.array_equal(dvr[:, :n].cpu().numpy().T, alone["vr"]), (rep, n)
    info = plan.info()
    # A problem of T tiles takes max(1, T-1) ticks: its setup tick also
    # solves the last diagonal tile, and each tick solves the next one ahead.
    assert info["tlsz"] == tlsz
    assert info["ticks"] == max(max(1, (H.shape[0] + tlsz - 1) // tlsz - 1) for H, _ in probs)


def _requests(probs, sel, arrivals):
    out = []
    for j, i in enumerate(sel):
        H, wr = probs[i]
        n = H.shape[0]
        out.append(dict(H=np.asfortranarray(H), wr=wr.copy(), vr=np.zeros((n, len(wr)), order="F"),
                        arrival_s=float(arrivals[j])))
    return out


def test_served_same_alone_and_in_the_mix(gpu_lib):
    import hsrq3in_gb300 as hsr
    probs = _mixed(24, 5, 20, 400)
    srv = hsr.Server(hbm_budget_bytes=2e9, tlsz=32)
    mix = _requests(probs, range(24), np.linspace(0.0, 0.03, 24))
    lat, st, stats = srv.replay(mix)
    assert all(s == 0 for s in st)
    assert all(x >= 0 for x in lat)
    assert stats["max_active"] > 1            # requests were on the device together
    for i in (0, 7, 23):
        alone = _requests(probs, [i], [0.0])
        srv.replay(alone)
        assert np.array_equal(alone[0]["vr"], mix[i]["vr"])
        ref = hsr.inverse_iteration(probs[i][0], probs[i][1], 32, 16)
        assert np.array_equal(mix[i]["vr"], ref["vr"])


def test_served_admission_respects_budget(gpu_lib):
    import hsrq3in_gb300 as hsr
    probs = _mixed(12, 7, 150, 200)
    budget = 3 * 8 * 220 * 220 * 8.0         # room for about three requests at a time
    srv = hsr.Server(hbm_budget_bytes=budget, tlsz=32)
    reqs = _requests(probs, range(12), np.zeros(12))
    lat, st, stats = srv.replay(reqs)
    assert all(s == 0 for s in st)
    assert stats["peak_bytes"] <= budget
    assert stats["max_active"] < 12
    for i in (0, 11):
        ref = hsr.inverse_iteration(probs[i][0], probs[i][1], 32, 16)
        assert np.array_equal(reqs[i]["vr"], ref["vr"])


def test_autotune_picks_a_candidate(gpu_lib):
    import torch
    import hsrq3in_gb300 as hsr
    from hsrq3in_gb300 import _lib
    dev = torch.device("cuda", 0)
    probs = _mixed(16, 9, 40, 200)
    tens = [_dev_problem(torch, H, wr, dev) for H, wr in probs]
    best, ms = hsr.autotune_batch(tens, candidates=(32, 64))
    assert best in (32, 64) and all(0 < t < 1e299 for t in ms)
    nlo = min(H.shape[0] for H, _ in probs)
    nhi = max(H.shape[0] for H, _ in probs)
    assert _lib.load().hsr_autotune_tlsz(nlo, nhi) == best


def test_served_pinned_host_buffers(gpu_lib):
    """Page-locked request buffers move by SM loads and stores through their
    mapped pointers, pageable ones by copy engine: both replays give the same
    results bit for bit, including padded leading dimensions, whose padding
    rows the output copy must leave untouched."""
    import torch
    import hsrq3in_gb300 as hsr
    probs = _mixed(10, 11, 30, 300)

    def make(pinned):
        reqs = []
        for i, (H, wr) in enumerate(probs):
            n, m = H.shape[0], len(wr)
            ldh, ldv = n + 3, n + 5
            if pinned:
                Hb = torch.zeros(ldh * n, dtype=torch.float64).pin_memory().numpy()
                Vb = torch.full((ldv * m,), -7.0, dtype=torch.float64).pin_memory().numpy()
                Wb = torch.zeros(m, dtype=torch.float64).pin_memory().numpy()
            else:
                Hb = np.zeros(ldh * n)
                Vb = np.full(ldv * m, -7.0)
                Wb = np.zeros(m)
            Hv = Hb.reshape((ldh, n), order="F")
            Hv[:n, :] = H
            Wb[:] = wr
            reqs.append(dict(H=Hv[:n, :], wr=Wb, vr=Vb.reshape((ldv, m), order="F")[:n, :],
                             vr_full=Vb.reshape((ldv, m), order="F"), arrival_s=0.002 * i))
        return reqs

    srv = hsr.Server(hbm_budget_bytes=2e9, tlsz=32)
    a, b = make(True), make(False)
    _, st_a, _ = srv.replay(a)
    _, st_b, _ = srv.replay(b)
    assert all(s == 0 for s in st_a) and all(s == 0 for s in st_b)
    for ra, rb, (H, wr) in zip(a, b, probs):
        n = H.shape[0]
        assert np.array_equal(ra["vr"], rb["vr"])
        assert np.array_equal(ra["wr"], rb["wr"])
        assert np.all(ra["vr_full"][n:, :] == -7.0) and np.all(rb["vr_full"][n:, :] == -7.0)
        ref = hsr.inverse_iteration(H, wr, 32, 16)
        assert np.array_equal(ra["vr"], ref["vr"])


@pytest.mark.parametrize("tlsz", [32, 64])
def test_queue_engine_equals_ticks_and_alone(gpu_lib, tlsz):
    """The persistent work-queue engine gives every problem exactly what the
    tick graph and a lone solve give, on two executes in a row."""
    import torch
    import hsrq3in_gb300 as hsr
    dev = torch.device("cuda", 0)
    probs = _mixed(40, 21, 12, 330)
    tens = [_dev_problem(torch, H, wr, dev) for H, wr in probs]
    plan = hsr.BatchPlan(tens, tlsz=tlsz, engine="queue")
    qi = plan.queue_info()
    assert qi["engine"] == "queue" and qi["items"] > 0 and qi["grid"] > 0 and qi["diag_warps"] >= 1
    for rep in range(2):
        for _, _, dvr in tens:
            dvr.fill_(float("nan"))
        plan.execute()
        torch.cuda.synchronize()
        for (H, wr), (dH, dwr, dvr) in zip(probs, tens):
            n = H.shape[0]
            alone = hsr.inverse_iteration(H, wr, tlsz, 16)
            assert np.array_equal(dwr.cpu().numpy(), alone["wr"])
            assert np.array_equal(dvr[:, :n].cpu().numpy().T, alone["vr"]), (rep, n)
    plan.set_engine("ticks")
    for _, _, dvr in tens:
        dvr.fill_(float("nan"))
    plan.execute()
    torch.cuda.synchronize()
    H, wr = probs[5]
    assert np.array_equal(tens[5][2][:, :H.shape[0]].cpu().numpy().T, hsr.inverse_iteration(H, wr, tlsz, 16)["vr"])
