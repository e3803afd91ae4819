"""Host-side logic of bench.py (no GPU): the algorithmic-byte arithmetic the
roofline is computed from, the clock-sample window, and the JSON line of the
reference arm (the CPU restatement timed on this host)."""
import importlib.util
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_algorithmic_bytes_per_contact():
    b = load_bench()
    # E+G+H per contact: positions + ids + weight in, gradient + Hessian values + CSR columns out
    assert b.BYTES_PER_CONTACT == {2: 504, 3: 1104, 4: 1944}
    # one contact of each type, ndof 12: the EE one adds eps_x + dtype, the CSR adds row pointers
    assert b.algorithmic_bytes([1, 1, 1, 1], 12) == 504 + 1104 + 2 * 1944 + 9 + 8 * 13
    # the PSD pass reads and writes each 3n x 3n slab once
    assert b.psd_bytes([1, 1, 1, 1]) == 2 * 8 * (36 + 81 + 2 * 144)


def row(sm, hw="Not Active", power_cap="Not Active"):
    return ["0", str(sm), "2070", "900", "0x0", hw, "Not Active", "Not Active", power_cap]


def test_clock_samples_inside_the_timed_window():
    b = load_bench()
    c = b.ClockSampler()
    c.rows = [(0.90, row(1200)), (1.05, row(2070)), (1.10, row(2060, power_cap="Active")), (2.0, row(900))]
    c.mark(1.0, 1.12)
    out = c.stop()
    assert out["samples"] == 2
    assert out["sm_mhz"] == 2065.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"]


def test_clock_sample_after_a_short_window():
    b = load_bench()
    c = b.ClockSampler()
    # the timed region ended before the next sample: the first one after its start is used
    c.rows = [(0.90, row(1200)), (1.30, row(2070, hw="Active")), (1.35, row(2000))]
    c.mark(1.0, 1.01)
    out = c.stop()
    assert out["samples"] == 1 and out["sm_mhz"] == 2070.0
    assert out["reasons"] == ["hw_slowdown"]


def test_clock_sampler_without_rows():
    b = load_bench()
    out = b.ClockSampler().stop()
    assert out["samples"] == 0 and out["reasons"] == ["unavailable"]


@pytest.mark.timeout(600)
def test_reference_arm_json_line():
    # the reference arm runs the CPU restatement only; it needs no GPU
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == "barrier E+grad+Hess contacts/s" and line["unit"] == "contacts/s"
    assert line["steps"] == 1 and line["warmup"] == 1 and line["higher_is_better"] is True
    assert line["value"] > 0 and line["cpu_baseline"]["value"] == line["value"]
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "contacts/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    # the same config dict as the GPU arm: the 256-scene batch
    assert line["config"] == load_bench().batch_config()
    assert line["config"]["contacts"] == 76_649_164
    assert "of the 256-scene batch" in line["cpu_baseline"]["sample"]


def test_ccd_candidate_count_marshalling():
    # No device here: the library answers with an error status (raised by the
    # mirror as ValueError / RuntimeError), not a ctypes argument error.
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "ipc-toolkit_gb300"))
    import ipctk_gb300 as ipctk
    b = load_bench()

    class NoMesh:
        _h = None

    V = np.zeros((4, 3))
    with pytest.raises((ValueError, RuntimeError)):
        b.ccd_candidate_count(ipctk, NoMesh(), V, V, strict=True)
    assert b.ccd_candidate_count(ipctk, NoMesh(), V, V) is None
