"""Serving: requests solved in a mix of concurrent requests give the same bits as each request solved alone."""
import numpy as np
import pytest

import nunatak_gb300 as nk
from nunatak_gb300 import workloads
from nunatak_gb300.server import Server

pytestmark = pytest.mark.gpu


def requests():
    out = []
    for k, (nx, ny) in enumerate([(64, 32), (128, 64), (64, 32), (128, 64), (64, 32), (96, 48)]):
        out.append(workloads.marine_sheet(nx, ny, seed=1, seed_friction=100 + k, precision="mixed",
                                          minimum_coarse_size=8))
    return out


def alone(case):
    P = case.problem(nk.Problem)
    st = P.picard_solve()
    return P.get("u"), P.get("v"), st


def test_requests_in_a_mix_equal_solves_alone():
    cases = requests()
    ref = [alone(c) for c in cases]
    S = Server(max_in_flight=4)
    tickets = [S.submit(c) for c in cases]
    got = [S.wait(t) for t in tickets]
    info = S.info()
    S.close()
    for (u, v, st, times), (ur, vr, sr) in zip(got, ref):
        assert st.status == 0 and st.picard_iterations == sr.picard_iterations
        assert np.array_equal(u, ur) and np.array_equal(v, vr)
        assert times[0] <= times[1] <= times[2]
    assert info["peak_in_flight"] > 1
    assert info["resident"] >= 3


def test_memory_cap_admits_one_problem_at_a_time():
    cases = requests()[:3]
    ref = [alone(c) for c in cases]
    probe = Server(max_in_flight=1)
    probe.wait(probe.submit(cases[1]))
    one = probe.info()["device_bytes"]
    probe.close()
    S = Server(max_in_flight=4, memory_cap_bytes=one + 1)   # room for the largest problem only
    tickets = [S.submit(c) for c in cases]
    got = [S.wait(t) for t in tickets]
    info = S.info()
    S.close()
    for (u, v, st, _), (ur, vr, _) in zip(got, ref):
        assert np.array_equal(u, ur) and np.array_equal(v, vr)
    assert info["peak_in_flight"] == 1 and info["device_bytes"] <= one + 1


def test_admission_thread_runs_requests_without_the_caller():
    """NK_SERVER_ADMISSION_THREAD: requests are admitted and retired by the library's own thread while the caller
    only sleeps and reads the pending count; the results are those of each request solved alone."""
    import time
    cases = requests()
    ref = [alone(c) for c in cases]
    S = Server(max_in_flight=3, admission_thread=True)
    tickets = [S.submit(c) for c in cases]
    t0 = time.time()
    while S.progress() > 0:       # a query in this mode: the thread does the work
        assert time.time() - t0 < 120, "requests did not finish"
        time.sleep(0.01)
    got = [S.wait(t) for t in tickets]
    info = S.info()
    S.close()
    for (u, v, st, times), (ur, vr, sr) in zip(got, ref):
        assert st.status == 0 and st.picard_iterations == sr.picard_iterations
        assert np.array_equal(u, ur) and np.array_equal(v, vr)
        assert times[0] <= times[1] <= times[2]
    assert info["peak_in_flight"] > 1


def test_admission_thread_wait_blocks_until_done():
    cases = requests()[:2]
    ref = [alone(c) for c in cases]
    S = Server(max_in_flight=2, admission_thread=True)
    tickets = [S.submit(c) for c in cases]
    S.wait_all()
    got = [S.wait(t) for t in tickets]
    S.close()
    for (u, v, st, _), (ur, vr, sr) in zip(got, ref):
        assert np.array_equal(u, ur) and np.array_equal(v, vr)


@pytest.mark.parametrize("threaded", [False, True])
def test_batched_server_equals_solves_alone(threaded):
    """batch_slots > 1: queued requests of one shape share one batched solve (nk_batch); every result is still the
    request solved alone, and a later wave reuses the resident batches."""
    cases = requests() + requests()[:4]
    ref = [alone(c) for c in cases]
    S = Server(max_in_flight=6, batch_slots=3, admission_thread=threaded)
    tickets = [S.submit(c) for c in cases]
    got = [S.wait(t) for t in tickets]
    again = [S.wait(S.submit(c)) for c in cases[:3]]
    info = S.info()
    S.close()
    for (u, v, st, times), (ur, vr, sr) in zip(got + again, ref + ref[:3]):
        assert st.status == 0 and st.picard_iterations == sr.picard_iterations
        assert st.linear_iterations_total == sr.linear_iterations_total
        assert np.array_equal(u, ur) and np.array_equal(v, vr)
        assert times[0] <= times[1] <= times[2]
    assert info["resident"] >= 3   # a batch per shape (three shapes), more where a shape's batch was busy


def test_batch_slots_out_of_range_is_refused():
    with pytest.raises(ValueError):
        Server(max_in_flight=2, batch_slots=-1)
