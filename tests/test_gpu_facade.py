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


def test_written_values_match_the_state(tmp_path):
    """The writers' values, not only their layout: the demo's fused run of a
    32^3 sphere drop (3 steps, the reference's default solver) is repeated
    through the C ABI in this process (the step is bitwise reproducible), and
    the binary frame (common/particles.cc:185-198) must hold the downloaded
    positions and velocities bit for bit, in order; the text dumps
    (Particles / VectorGrid / ScalarGrid::Write, "%f") must hold them to the
    printed precision, on exactly the active voxels."""
    import fsim

    if not DEMO.exists():
        pytest.skip("fsim_demo not built")
    n, steps = 32, 3
    out = tmp_path / "w"
    r = subprocess.run([str(DEMO), str(n), str(steps), str(out), "fused", "debug"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    g, f = fsim.physical_gravity(n)
    sim = fsim.Simulation((n, n, n), fsim.BOUNDARY_BOX, g, f, 0.95, 8)
    sim.seed(fsim.scene_passes("sphere_drop", n), seed=0)
    prm = sim.default_pcg_params()
    frame_step = float(np.float32(1.0) / np.float32(30.0))
    inv, t = sim.cfl(), 0.0
    for _ in range(steps):
        dt, t = fsim.compute_dt(inv, 1, frame_step, t)
        if np.float32(t) + np.float32(1e-5) >= np.float32(frame_step):
            t = 0.0
        inv = sim.step(dt, prm).next_inv_speed
    pos, vel, _ = sim.download_particles()
    u, ua = sim.field(fsim.FIELD_VELOCITY)
    p, pa = sim.field(fsim.FIELD_PRESSURE)
    sim.close()
    part = Path(str(out) + "_0")
    data = (part / "particles_00000000").read_bytes()
    cnt = struct.unpack("7i", data[:28])[6]
    assert cnt == pos.shape[0]
    rec = np.frombuffer(data[28:], dtype=np.dtype([("id", "<i4"), ("p", "<f4", 3),
                                                   ("v", "<f4", 3)]))
    assert np.array_equal(rec["p"], pos) and np.array_equal(rec["v"], vel)
    half_ulp = 5.0e-7 + 1e-12  # "%f" prints six decimals
    lines = (part / "debug" / "particles_00000000").read_text().splitlines()
    txt = np.array([[float(x) for x in re.split(r"[ ,:]+", ln.strip())[1:]] for ln in lines[3:]])
    assert txt.shape == (cnt, 6)
    assert np.abs(txt[:, :3] - pos).max() <= half_ulp
    assert np.abs(txt[:, 3:] - vel).max() <= half_ulp
    # the velocity dump covers the faces of [0, N]^3, the pressure dump the cells of [0, N)^3
    for name, field, act, nval, hi in (("grid_velocity_00000000.txt", u, ua, 3, n),
                                       ("grid_phi_00000000.txt", p, pa, 1, n - 1)):
        rows = (part / "debug" / name).read_text().splitlines()[2:]
        got = {}
        for ln in rows:
            ijk, vals = ln.split(" : ")
            got[tuple(int(x) for x in ijk.split())] = [float(x) for x in vals.split()]
        active = {tuple(int(x) - 1 for x in c) for c in np.argwhere(act)}
        assert len(got) > 0
        assert set(got) == {c for c in active if all(0 <= x <= hi for x in c)}, name
        for c, vals in got.items():
            ref = np.atleast_1d(field[c[0] + 1, c[1] + 1, c[2] + 1]).astype(np.float64)
            assert len(vals) == nval
            assert np.abs(np.array(vals) - ref).max() <= half_ulp, (name, c)
