"""The oracle's host threads change nothing but its speed.

bench.py's reference arm runs the oracle with every host thread on the loops
whose iterations are independent (per particle, per leaf, per matrix row or
vector entry), on the chunk sums of the PCG dots and on the lane sums of
p.Ap; the orders the results depend on (chunk and lane totals, the P2G leaf
write-back, the stable radix passes) stay fixed.  Three steps of a 40^3 dam break (15 K
unknowns, 123 K particles: every parallel path is taken) must give the same
bits on one thread and on four.
"""
import numpy as np

import fsim
from oracle import oracle as O


def _run(threads):
    O.set_threads(threads)
    try:
        n = 40
        g, f = fsim.physical_gravity(n)
        orc = O.OracleSim((n, n, n), fsim.BOUNDARY_BOX, g, f, 0.95, 8)
        orc.seed(fsim.scene_passes("dam_break", n), seed=0)
        iters = []
        for k in range(3):
            st = orc.step(0.004 + 0.003 * k, mode=1, precision=0, max_iterations=500, tol=1e-5)
            iters.append(st.iterations)
        out = dict(zip(("pos", "vel", "gvel"), orc.particles()))
        out["keys"] = orc.keys()
        out["pressure"] = orc.field(fsim.FIELD_PRESSURE)[0]
        out["velocity"] = orc.field(fsim.FIELD_VELOCITY)[0]
        out["iters"] = np.array(iters)
        orc.close()
        return out
    finally:
        O.set_threads(1)


def test_results_do_not_depend_on_thread_count():
    a, b = _run(1), _run(4)
    assert a["pos"].shape[0] > 100_000 and a["iters"].min() > 50
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert O.get_threads() == 1
