"""Run-time control of pt_integrate (needs a GB300): cancellation through the
host-mapped flag (the reference's `quit`, include/globals.h:33), launch and
wall-time budgets.  Failures are made on the host (a flag set from another
thread, a budget that runs out); nothing here faults or hangs the GPU."""
import threading
import time

import numpy as np
import pytest

from pentrack_gb300 import _abi as A

pytestmark = pytest.mark.gpu


def _long_run(n=20000, simtime=200.0):
    from pentrack_gb300 import workloads
    sc, params, parts = workloads.field_storage(n=n, simtime=simtime)
    params.mode = A.MODE_BATCHED
    return sc, params, parts


def test_cancel_returns_partial_results(built):
    from pentrack_gb300 import Engine
    sc, params, parts = _long_run()
    e = Engine(sc)
    timer = threading.Timer(0.5, e.cancel)
    t0 = time.perf_counter()
    timer.start()
    out, st = e.integrate(params, parts)
    dt = time.perf_counter() - t0
    timer.cancel()
    assert e.last_status == A.PT_ERR_CANCELLED
    assert dt < 30.0
    assert st["active"] > 0                        # stopped early
    assert np.all(out.t >= parts.t)                # partial states are consistent
    assert np.all(np.isfinite(out.y))
    # the flag is consumed: the next call runs to completion
    sc2, p2, parts2 = _long_run(n=256, simtime=0.5)
    out2, st2 = e.integrate(p2, parts2)
    assert e.last_status == A.PT_OK and st2["active"] == 0


def test_launch_budget_reports_timeout(built):
    from pentrack_gb300 import Engine
    from pentrack_gb300.engine import EngineError
    sc, params, parts = _long_run(n=2000)
    params.max_launches = 4
    e = Engine(sc)
    with pytest.raises(EngineError) as ex:
        e.integrate(params, parts)
    assert ex.value.status == A.PT_ERR_TIMEOUT


def test_wall_time_budget_reports_timeout(built):
    from pentrack_gb300 import Engine
    from pentrack_gb300.engine import EngineError
    sc, params, parts = _long_run(n=20000)
    params.timeout_s = 0.3
    e = Engine(sc)
    t0 = time.perf_counter()
    with pytest.raises(EngineError) as ex:
        e.integrate(params, parts)
    assert ex.value.status == A.PT_ERR_TIMEOUT
    assert time.perf_counter() - t0 < 30.0
