"""bench.py's roofline arithmetic on synthetic timings (no GPU).

The PCG pair is reported as one iteration: algorithmic bytes are the two
kernels' bytes per unknown times the unknowns, and the time is the loop
device time the library reports per timed step (fsim_pcg_stats.loop_ms).
"""
import pytest

import bench


def _res(kt, loop_ms):
    iters, rows = [700, 800], [4_000_000, 4_100_000]
    return dict(kt=kt, piters=[750], prows=[4_050_000], prof_ms=40.0, iters=iters, rows=rows,
                loop_ms=loop_ms, ms=60.0)


def test_pcg_pair_is_one_iteration():
    kt = {"pcg_spmv": (16.0, 750), "pcg_update": (15.0, 750), "p2g_fused": (1.5, 1)}
    res = _res(kt, [24.0, 28.0])
    r = bench.roofline(res)
    assert r["kernel"].startswith("pcg_iteration (pcg_spmv + pcg_update")
    per = bench.ALG_BYTES["pcg_spmv"] + bench.ALG_BYTES["pcg_update"]
    assert r["alg_bytes_per_unknown"] == per == 34
    tot = per * (4_000_000 * 700 + 4_100_000 * 800)
    achieved = tot / (52.0e-3) / 1e9
    assert r["achieved"] == pytest.approx(achieved)
    assert r["frac"] == pytest.approx(achieved / r["peak"])
    assert r["us_per_iteration"] == pytest.approx(52.0e3 / 1500)
    assert r["share_of_step"] == pytest.approx(52.0 / 60.0)
    traffic = (bench.NCU_TRAFFIC_PER_UNKNOWN["pcg_spmv"]
               + bench.NCU_TRAFFIC_PER_UNKNOWN["pcg_update"]) * 4_050_000
    assert r["traffic"] == pytest.approx(traffic)
    assert set(r["per_kernel_profiled"]) == {"pcg_spmv", "pcg_update"}
    assert r["unfused_alg_bytes_per_unknown"] == 50
    assert r["unfused_frac"] == pytest.approx(r["frac"] * 50 / 34)


def test_mixed_pair_and_other_kernels():
    kt = {"pcg_spmv_mixed": (18.0, 750), "pcg_update_mixed": (17.0, 750)}
    r = bench.roofline(_res(kt, [30.0, 31.0]))
    assert "pcg_spmv_mixed + pcg_update_mixed" in r["kernel"]
    per = bench.NCU_TRAFFIC_PER_UNKNOWN["pcg_spmv_mixed"] + bench.NCU_TRAFFIC_PER_UNKNOWN["pcg_update_mixed"]
    assert r["traffic"] == pytest.approx(per * 4_050_000)
    assert "1024^3" in r["traffic_source"]
    # a non-PCG top kernel is reported alone, from the profiled events
    kt = {"p2g_fused": (5.0, 3), "g2p": (1.0, 3)}
    r = bench.roofline(_res(kt, [0.0, 0.0]))
    assert r["kernel"] == "p2g_fused" and r["frac"] is None


def test_resident_loop_is_one_iteration():
    """The resident loop is one launch per solve; its iteration is counted in
    the pair's 34 B per unknown, and its traffic is the measured DRAM bytes
    per iteration, with a note that frac above 1 is expected."""
    kt = {"pcg_resident": (25.0, 1), "p2g_fused": (1.5, 1)}
    r = bench.roofline(_res(kt, [12.0, 13.0]))
    assert r["kernel"] == "pcg_iteration (pcg_resident, one cooperative launch per solve)"
    assert r["alg_bytes_per_unknown"] == 34
    tot = 34 * (4_000_000 * 700 + 4_100_000 * 800)
    assert r["achieved"] == pytest.approx(tot / 25.0e-3 / 1e9)
    assert r["us_per_iteration"] == pytest.approx(25.0e3 / 1500)
    assert r["traffic"] == pytest.approx(bench.NCU_TRAFFIC_PER_UNKNOWN["pcg_resident"] * 4_050_000)
    assert r["traffic"] < 1e-3 * r["alg_bytes_per_launch"]  # on chip: almost no DRAM traffic
    assert "on chip" in r["note"]
    assert set(r["per_kernel_profiled"]) == {"pcg_resident"}


def test_whole_job_rate_counts_every_replica():
    assert bench.whole_job_rate(4, 20, 1000.0) == pytest.approx(80.0)


def test_e2e_floor():
    # 386 MB arrays at 211 / 193 GB/s, a 29.9 ms step of which 1.13 ms overlaps the uploads
    up, down = 386e6 / 211e9 * 1e3, 386e6 / 193e9 * 1e3
    f = bench.e2e_floor_ms(up, down, 29.9, 1.13)
    assert f == pytest.approx(3 * up + 28.77 + 2 * down)
    assert bench.e2e_floor_ms(1.0, 1.0, 0.5, 2.0) == pytest.approx(5.0)
