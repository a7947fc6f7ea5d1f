"""Host-side helpers of bench.py, checked on the CPU: the treecode's
interaction count (the numerator of its FP32 roofline) equals the count the
oracle's walk makes, query for query in total."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def test_tree_interaction_count_matches_oracle_walk(oracle_lib):
    import bench
    from vortegrid_gb300 import workloads
    pos, w, s = workloads.rings(8192, count=8, seed=2, box=2.0)
    g = oracle_lib.step_geometry(pos, float(s[0]) * 0.5)
    gp = workloads.grid_points(list(g.mn), list(g.cell), g.points)
    q = np.concatenate([gp, pos, pos + np.float32(0.013)]).astype(np.float32)
    assert bench.tree_interactions(g.points, list(g.mn), list(g.ext), q) == oracle_lib.tree_interactions(g, q)
    # an anisotropic box (decimation 1 on an axis that ran out of cells)
    g2 = oracle_lib.define_shape(3000, [-1.0, -0.5, -0.1], [1.0, 0.5, 0.1])
    q2 = workloads.grid_points(list(g2.mn), list(g2.cell), g2.points)
    assert bench.tree_interactions(g2.points, list(g2.mn), list(g2.ext), q2) == oracle_lib.tree_interactions(g2, q2)


def test_measured_peaks_fallback_is_stated():
    import bench
    p = bench.measured_peaks()
    assert p["basis"] in ("measured", "fallback") and p["hbm_gbs"] > 1000
