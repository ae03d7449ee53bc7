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


def _vdb_key(c):
    """OpenVDB Tree3<T,3,3> iteration rank of a coordinate."""
    i, j, k = c
    return ((i >> 6, j >> 6, k >> 6), ((i >> 3) & 7, (j >> 3) & 7, (k >> 3) & 7),
            (i & 7, j & 7, k & 7))


def test_debug_dumps_use_the_reference_text_format(tmp_path):
    """SaveDebugDataToFile writes grid dumps as ScalarGrid/VectorGrid::Write
    do (common/scalar_grid.cc:135-160, vector_grid.cc:132-160): the box start
    and end, then 'i j k : values' for active voxels in OpenVDB order."""
    if not DEMO.exists():
        pytest.skip("fsim_demo not built")
    out = tmp_path / "dbg"
    r = subprocess.run([str(DEMO), "16", "2", str(out), "fused", "debug"], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    d = Path(str(out) + "_0") / "debug"  # output_dir of partition 0
    for name, nval, top in (("grid_velocity_00000000.txt", 3, 16), ("grid_phi_00000000.txt", 1, 15)):
        lines = (d / name).read_text().splitlines()
        assert lines[0] == "0 0 0" and lines[1] == "15 15 15"
        coords = []
        for ln in lines[2:]:
            ijk, vals = ln.split(" : ")
            c = tuple(int(x) for x in ijk.split())
            v = [float(x) for x in vals.split()]
            assert len(v) == nval and all(np.isfinite(v))
            assert all(0 <= x <= top for x in c)
            coords.append(c)
        assert len(coords) > 0
        assert coords == sorted(coords, key=_vdb_key)
    # the particle text dump: header, then "id : p p p, v v v"
    lines = (d / "particles_00000000").read_text().splitlines()
    n = int(lines[2])
    assert len(lines) == 3 + n and lines[3].startswith("0 : ")
