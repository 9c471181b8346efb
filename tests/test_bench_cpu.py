"""Host-side helpers of bench.py that need no GPU."""
import importlib.util
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_cpu_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_batch_tile_pins_parse():
    b = _bench()
    assert b.parse_batch_tiles("0:32x16/2,1:32x16/2,2:32x8/1") == {
        0: (32, 16, 2), 1: (32, 16, 2), 2: (32, 8, 1)}
    assert b.parse_batch_tiles("2:16x16") == {2: (16, 16, 1)}  # one cell per thread
    assert b.parse_batch_tiles("") == {}
