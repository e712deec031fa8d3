"""bench.py's stream roofline model: the algorithmic bytes of a request are its cells times (Picard iterations x
the coefficient update's bytes + CG iterations x (the FP64 CG iteration's + the FP32 V-cycle's bytes))."""
import importlib.util
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_per_cell_figures():
    b = _bench()
    assert b.CG_BYTES_PER_CELL == 65 + 104 + 32 + 48      # operator, update, dots, xpby
    assert b.VCYCLE_BYTES_PER_CELL == 331                 # 62 words x 4/3 levels x 4 B
    assert b.COEF_BYTES_PER_CELL == 120                   # 15 FP64 words


def test_stream_bytes_sum_over_requests():
    b = _bench()
    per_iter = b.CG_BYTES_PER_CELL + b.VCYCLE_BYTES_PER_CELL
    got = b.stream_algorithmic_bytes([8192, 524288], [39, 39], [1120, 1985])
    want = 8192 * (39 * 120 + 1120 * per_iter) + 524288 * (39 * 120 + 1985 * per_iter)
    assert got == want
    assert b.stream_algorithmic_bytes([], [], []) == 0.0
