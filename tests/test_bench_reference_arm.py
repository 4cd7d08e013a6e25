"""bench.py's reference arm runs the oracle alone: scenes packed by the
oracle's packScene, scene generators seeded through the oracle's Rng, and the
CUDA library never mapped into the process (a fresh interpreter is checked
through /proc/self/maps by the arm itself)."""
import json
import pathlib
import subprocess
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent


@pytest.mark.parametrize("workload", ["cornell", "traversal", "caustic", "display"])
def test_reference_arm_loads_no_product_library(workload, oracle):
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", workload,
                          "--small", "--steps", "1", "--warmup", "0", "--cpu-seconds", "0.4"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["product_library_loaded"] is False
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0


def test_oracle_stream_draws_the_library_stream(native_lib, oracle):
    """caustic.rng.set_stream with the oracle's Rng gives the same draws as the library's ct_rng_stream."""
    import numpy as np

    import caustic as ct

    want = ct.Rng(2024).draw(5000, "range", -0.5, 0.5)
    prev = ct.rng.set_stream(oracle.rng_stream_state)
    try:
        r = ct.Rng(2024)
        got = r.draw(5000, "range", -0.5, 0.5)
        tail = r.draw(7)
    finally:
        ct.rng.set_stream(prev)
    r2 = ct.Rng(2024)
    r2.draw(5000, "range", -0.5, 0.5)
    assert np.array_equal(got, want) and np.array_equal(tail, r2.draw(7))
