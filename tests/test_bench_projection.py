"""The projection bench.py reports for the plain FP64 arm of the 722-angle
monostatic sweep (CPU only).  The batched arm is measured over all 722
angles; the sequential FP64 sweep would take over an hour, so its first
angles are sampled and projected: the cold start is counted once, later
angles as the sampled warm ones, sample time split by iteration count.
"""
import numpy as np

import bench


def test_sequential_projection_counts_the_cold_start_once():
    # 3 sampled angles: cold 1000 iterations, then 500 and 500; 20 s in all
    t = bench.project_sequential(20.0, [1000, 500, 500], nang=10)
    per_it = 20.0 / 2000
    assert np.isclose(t, per_it * (1000 + 9 * 500))
    # the per-RHS average of the sample would count the cold start once per 3 angles
    assert t < 10 * 20.0 / 3
