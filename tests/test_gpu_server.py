"""The continuous-batching server: every result is the same alone and in the
mix (against a single-matrix reduction and the oracle), requests admitted
while others run, a too-large request rejected, a regrow under a tight arena."""
import threading
import time

import numpy as np
import pytest

import oracle
from openph_gb300 import complexes as cx
from openph_gb300.api import Context, OphError, OPH_ERR_OOM, Server

pytestmark = pytest.mark.gpu


def mixed_requests():
    reqs = [cx.rips_cube(n, seed=100 + n) for n in (8, 15, 22, 30)]
    reqs += [cx.rips_mixed(n, seed=200 + n) for n in (12, 19, 26)]
    reqs += [cx.lower_star_image(s, s, seed=300 + s, sigma=2.0) for s in (9, 24, 40)]
    reqs += [cx.rips_torus(60, t, seed=400 + t // 1000) for t in (3000, 12000)]
    return reqs


def test_results_same_alone_and_in_the_mix(cuda_lib):
    reqs = mixed_requests()
    with Context(0) as c:
        alone = [c.reduce(bm, "pms")[:2] for bm in reqs]
    with Server(0, budget_bytes=2 << 30, max_active=64) as srv:
        tickets = [srv.submit(bm) for bm in reqs]
        mixed = [srv.wait(t)[:2] for t in tickets]
        st = srv.stats()
    assert st["completed"] == len(reqs)
    for bm, (la, ea), (lm, em) in zip(reqs, alone, mixed):
        want, want_ess, _ = oracle.twist(bm)
        np.testing.assert_array_equal(lm, la)
        np.testing.assert_array_equal(em, ea)
        np.testing.assert_array_equal(lm, want)
        np.testing.assert_array_equal(em, want_ess)


@pytest.mark.parametrize("cap", ["1", "3", "0"])
def test_chain_cap(cuda_lib, monkeypatch, cap):
    """Bitmap-tier chains cut after every `cap` additions (0: never) and taken
    up again in later sweeps: the same results, on requests whose long
    columns go through the bitmap tiers (a torus through its anti-transpose,
    a lower-star image and a 3-D volume on D)."""
    from cases import lower_star_volume
    monkeypatch.setenv("OPH_SERVE_CHAIN_CAP", cap)
    reqs = [cx.rips_torus(400, 150_000, seed=61), cx.lower_star_image(120, 120, seed=62, sigma=6.0),
            lower_star_volume(12, 63), cx.rips_cube(40, seed=64)]
    with Server(0, budget_bytes=4 << 30, max_active=8) as srv:
        tickets = [srv.submit(bm) for bm in reqs]
        res = [srv.wait(t) for t in tickets]
    for bm, (low, ess, info) in zip(reqs, res):
        want, want_ess, _ = oracle.twist(bm)
        np.testing.assert_array_equal(low, want)
        np.testing.assert_array_equal(ess, want_ess)


def test_arrivals_while_running(cuda_lib):
    """Requests submitted from another thread while earlier ones are on the
    device are folded into the running batch."""
    reqs = mixed_requests() * 3
    out = {}
    with Server(0, budget_bytes=2 << 30, max_active=8) as srv:
        def producer():
            for k, bm in enumerate(reqs):
                out[k] = srv.submit(bm)
                time.sleep(0.001)
        th = threading.Thread(target=producer)
        th.start()
        th.join()
        res = {k: srv.wait(t) for k, t in out.items()}
    for k, bm in enumerate(reqs):
        want, _, _ = oracle.twist(bm)
        np.testing.assert_array_equal(res[k][0], want)
        assert res[k][2]["latency_ms"] >= res[k][2]["queue_ms"] >= 0


def test_request_larger_than_arena_is_rejected(cuda_lib):
    with Server(0, budget_bytes=64 << 20, max_active=4) as srv:
        with pytest.raises(OphError) as e:
            srv.submit(cx.rips_torus(400, 2_000_000, seed=1))
        assert e.value.status == OPH_ERR_OOM
        bm = cx.rips_cube(10, seed=3)
        low, _, _ = srv.wait(srv.submit(bm))
        np.testing.assert_array_equal(low, oracle.twist(bm)[0])


def test_tight_arena_regrows(cuda_lib):
    """A lower-star image whose columns grow past their pool region."""
    bm = cx.lower_star_image(96, 96, seed=8, sigma=4.0)
    with Server(0, budget_bytes=256 << 20, max_active=4) as srv:
        low, ess, info = srv.wait(srv.submit(bm))
        st = srv.stats()
    want, want_ess, _ = oracle.twist(bm)
    np.testing.assert_array_equal(low, want)
    np.testing.assert_array_equal(ess, want_ess)


def test_device_submissions_mixed_with_host(cuda_lib):
    """Matrices built on the GPU and submitted from device memory run in the
    same batch as host submissions; each result equals the oracle's, and the
    device buffers may be freed as soon as submission returns."""
    import torch
    host = [cx.rips_cube(14, seed=5), cx.lower_star_image(20, 20, seed=6, sigma=2.0)]
    pts = cx.points_torus(200, 3)
    thr = cx.rips_threshold(pts, 40_000)
    img = cx.image_smoothed(48, 40, 7)
    with Server(0, budget_bytes=1 << 30, max_active=16) as srv:
        dev = [cx.rips_device(pts, thr), cx.lower_star_device(img), cx.rips_device(cx.points_cube(9, 2))]
        want_dev = [cx.rips(pts, thr), cx.lower_star(img), cx.rips(cx.points_cube(9, 2))]
        tickets = []
        for k in range(3):
            tickets.append(("d", k, srv.submit_device(dev[k])))
            if k < len(host):
                tickets.append(("h", k, srv.submit(host[k])))
        del dev
        torch.cuda.empty_cache()
        res = {(kind, k): srv.wait(t) for kind, k, t in tickets}
        assert srv.stats()["completed"] == len(tickets)
    for k, bm in enumerate(want_dev):
        low, ess, _ = res[("d", k)]
        want, want_ess, _ = oracle.twist(bm)
        np.testing.assert_array_equal(low, want)
        np.testing.assert_array_equal(ess, want_ess)
    for k, bm in enumerate(host):
        want, want_ess, _ = oracle.twist(bm)
        np.testing.assert_array_equal(res[("h", k)][0], want)
        np.testing.assert_array_equal(res[("h", k)][1], want_ess)


def test_device_submission_rejects_malformed(cuda_lib):
    """A device colptr that decreases, or a row index out of range, is
    refused at submission with BAD_INPUT; the server keeps working."""
    import torch
    from openph_gb300.api import OPH_ERR_BAD_INPUT
    from openph_gb300.complexes import DeviceMatrix
    bm = cx.rips_cube(6, seed=1)
    with Server(0, budget_bytes=256 << 20, max_active=4) as srv:
        cp = torch.as_tensor(bm.colptr, device="cuda")
        rows = torch.as_tensor(bm.rows, device="cuda").clone()
        last = int(bm.colptr[-1]) - 1
        rows[last] = bm.m  # a row past the last column
        with pytest.raises(OphError) as e:
            srv.submit_device(DeviceMatrix(cp, rows, None))
        assert e.value.status == OPH_ERR_BAD_INPUT
        cp_bad = cp.clone()
        cp_bad[2] = cp_bad[3] + 1
        with pytest.raises(OphError) as e:
            srv.submit_device(DeviceMatrix(cp_bad, torch.as_tensor(bm.rows, device="cuda"), None))
        assert e.value.status == OPH_ERR_BAD_INPUT
        good = DeviceMatrix(cp, torch.as_tensor(bm.rows, device="cuda"), None)
        low, _, _ = srv.wait(srv.submit_device(good))
    np.testing.assert_array_equal(low, oracle.twist(bm)[0])


@pytest.fixture(scope="module")
def dual_mix():
    """Requests of at least 2^17 columns whose top dimension dwarfs the
    bottom one (reduced through their anti-transpose, as a single-matrix
    reduction would), a lower-star image of the same size (split by block:
    its D' part, then its D part) and small complexes, with the oracle's
    answers."""
    reqs = [cx.rips_torus(400, 150_000, seed=41), cx.rips_cube(95, seed=42), cx.lower_star_image(160, 160, seed=43),
            cx.rips_cube(20, seed=44), cx.rips_torus(60, 8000, seed=45), cx.rips_torus(400, 140_000, seed=46)]
    return reqs, [oracle.twist(bm)[:2] for bm in reqs]


def test_anti_transpose_requests_in_the_mix(cuda_lib, dual_mix):
    reqs, want = dual_mix
    with Context(0) as c:
        alone = [c.reduce(bm, "pms") for bm in reqs]
    with Server(0, budget_bytes=8 << 30, max_active=16) as srv:
        tickets = [srv.submit(bm) for bm in reqs]
        mixed = [srv.wait(t)[:2] for t in tickets]
        st = srv.stats()
    assert [info["dual"] for _, _, info in alone] == [1, 1, 2, 0, 0, 1]
    assert st["dual_admitted"] == 4  # requests with a part on the anti-transpose
    for (wl, we), (lm, em), (la, ea, _) in zip(want, mixed, alone):
        np.testing.assert_array_equal(lm, wl)
        np.testing.assert_array_equal(em, we)
        np.testing.assert_array_equal(lm, la)


def test_anti_transpose_requests_arriving_while_running(cuda_lib, dual_mix):
    """The same requests, twice over, submitted from another thread while
    earlier ones are on the device; small arenas of columns force retired
    column ranges to be handed out again."""
    reqs, want = dual_mix
    order = [0, 3, 1, 4, 2, 5] * 2
    out = {}
    with Server(0, budget_bytes=4 << 30, max_active=4) as srv:
        def producer():
            for k, i in enumerate(order):
                out[k] = srv.submit(reqs[i])
                time.sleep(0.002)
        th = threading.Thread(target=producer)
        th.start()
        th.join()
        res = {k: srv.wait(t) for k, t in out.items()}
        st = srv.stats()
    assert st["dual_admitted"] == 8
    for k, i in enumerate(order):
        np.testing.assert_array_equal(res[k][0], want[i][0])
        np.testing.assert_array_equal(res[k][1], want[i][1])


def test_anti_transpose_device_submission(cuda_lib, dual_mix):
    torch = pytest.importorskip("torch")
    reqs, want = dual_mix

    class Dev:
        def __init__(self, bm):
            self.colptr = torch.from_numpy(bm.colptr).cuda()
            self.rows = torch.from_numpy(bm.rows).cuda()

    with Server(0, budget_bytes=8 << 30, max_active=8) as srv:
        tickets = [srv.submit_device(Dev(reqs[0])), srv.submit(reqs[2]), srv.submit_device(Dev(reqs[1]))]
        res = [srv.wait(t) for t in tickets]
        assert srv.stats()["dual_admitted"] == 3
    for (low, ess, _), i in zip(res, (0, 2, 1)):
        np.testing.assert_array_equal(low, want[i][0])
        np.testing.assert_array_equal(ess, want[i][1])
