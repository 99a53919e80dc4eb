"""Serving loop (trans_gb300.serving): requests admitted while others run retire with the same
iteration count and bit-identical fields as when each is served alone (tolerance: 0), and the
report carries latency percentiles and throughput."""
import copy

import pytest

from helpers import SMALL_CASCADE, bit_equal_fraction, interior

pytestmark = pytest.mark.gpu


def _requests():
    from trans_gb300.serving import Request
    g = dict(SMALL_CASCADE)
    return [Request(0, 0.0, "medium", 0.85, 0.6, grid=g), Request(1, 0.0, "medium", 0.90, 0.55, grid=g),
            Request(2, 0.15, "medium", 0.82, 0.65, grid=dict(g, nk=6))]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_served_alone_equals_served_in_mix(gpu_lib, precision):
    from trans_gb300 import abi
    from trans_gb300.serving import serve
    prec = abi.TRANS_MIXED if precision == "mixed" else abi.TRANS_FP64
    mix = serve(_requests(), precision=prec, drop=0.05, max_iters=400, keep_fields=True)
    assert mix["completed"] == 3 and mix["converged"] == 3
    assert mix["latency_p50_s"] > 0 and mix["latency_p99_s"] >= mix["latency_p50_s"]
    assert mix["throughput_mcell_iter_s"] > 0
    by_id = {r.rid: r for r in mix["records"]}
    for req in _requests():
        alone = serve([copy.deepcopy(req)], precision=prec, drop=0.05, max_iters=400, keep_fields=True)
        ra, rm = alone["records"][0], by_id[req.rid]
        assert ra.iterations == rm.iterations
        from trans_gb300.serving import build_case
        c = build_case(req, prec)[0]
        for ib, b in enumerate(c.blocks):
            for f in ("V", "PP", "T", "RMIU"):
                assert bit_equal_fraction(ra.result[ib][f], rm.result[ib][f], interior(b.dims)) == 1.0, (req.rid, ib, f)


def test_budget_queues_requests(gpu_lib):
    """With room for one request at a time, the others wait in the queue and still finish."""
    from trans_gb300 import abi
    from trans_gb300.serving import build_case, serve
    from trans_gb300.solver import Batch
    reqs = _requests()[:2]
    c, conns, geo, st = build_case(reqs[0], abi.TRANS_FP64)
    probe = Batch()
    need = probe.case_bytes(c, conns)
    probe.close()
    rep = serve(reqs, precision=abi.TRANS_FP64, budget_bytes=int(need * 1.5), drop=0.05, max_iters=400)
    assert rep["converged"] == 2
    first, second = sorted(rep["records"], key=lambda r: r.admitted)
    assert second.admitted >= first.retired    # the second waited for the first to leave
