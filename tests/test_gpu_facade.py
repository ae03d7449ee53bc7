"""The C++ facade (reference-named classes over the C ABI) drives a sphere
drop the way FlipDriver::RunOneStep sequences the stages; staged and fused
runs of the same steps must agree, and the binary particle frame must use the
reference's particles_%08d layout (common/particles.cc:185-198)."""
import re
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
DEMO = ROOT / "fluid-sim-lb_gb300" / "lib" / "fsim_demo"


def _run(tmp_path, mode):
    out = tmp_path / mode
    r = subprocess.run([str(DEMO), "32", "3", str(out), mode], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    steps = [dict(re.findall(r"(\w+(?:\(\d+,\d+,\d+\))?) ([-\d.e+]+)", l))
             for l in r.stdout.splitlines() if l.startswith("step")]
    return out, steps


def test_facade_staged_matches_fused(tmp_path):
    if not DEMO.exists():
        pytest.skip("fsim_demo not built")
    out_s, st_s = _run(tmp_path, "staged")
    out_f, st_f = _run(tmp_path, "fused")
    assert len(st_s) == 3 and len(st_f) == 3
    for a, b in zip(st_s, st_f):
        assert a["dt"] == b["dt"]
        assert a["particles"] == b["particles"]
        assert a["fluid_cells"] == b["fluid_cells"]
        assert abs(int(a["pcg_iterations"]) - int(b["pcg_iterations"])) <= 2
    frame = Path(str(out_s) + "_0") / "particles_00000000"
    data = frame.read_bytes()
    hdr = struct.unpack("7i", data[:28])
    assert hdr[:6] == (0, 0, 0, 31, 31, 31)
    n = hdr[6]
    assert n == int(st_s[-1]["particles"]) and len(data) == 28 + n * 28
    rec = np.frombuffer(data[28:], dtype=np.dtype([("id", "<i4"), ("p", "<f4", 3),
                                                   ("v", "<f4", 3)]))
    assert np.array_equal(rec["id"], np.arange(n))
    assert rec["p"].min() >= 0 and rec["p"].max() <= 32
