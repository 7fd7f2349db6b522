"""The sweep projections bench.py reports (CPU only).

Both arms of the 722-angle monostatic sweep are sampled and projected with the
same rule: steps that happen once (cold starts) are counted once, later steps
as sampled, and sample time is split by iteration count.
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


def test_batched_projection_splits_blocks_by_slowest_column():
    # 4 columns x 4 steps of their runs: block k's slowest column decides its time
    it = np.array([[900, 400, 300, 280],
                   [1000, 420, 310, 300],
                   [950, 410, 305, 290],
                   [980, 405, 290, 285]])
    t = bench.project_batched_warm(30.0, it.ravel(), block=4, nrun_sample=4, nang=40, steady_from=2)
    per_block = it.max(axis=0).astype(float)
    t_blk = 30.0 * per_block / per_block.sum()
    nrun = 10
    assert np.isclose(t, t_blk[0] + t_blk[1] + (nrun - 2) * t_blk[2:].mean())


def test_batched_projection_of_a_sample_that_is_the_whole_sweep():
    # when the sample covers every block, the projection is the sample's own time
    it = np.arange(1, 13).reshape(3, 4)   # 3 columns x 4 steps
    t = bench.project_batched_warm(12.0, it.ravel(), block=3, nrun_sample=4, nang=12, steady_from=2)
    assert np.isclose(t, 12.0)
