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
