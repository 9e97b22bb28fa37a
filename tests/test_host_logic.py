"""Host-side logic that needs no GPU: the progressive-growing schedule of
scripts/train.py:90-123, the pooled-grid shapes (against torch's avg_pool3d), and the
batched form's tile and brick-size rules."""
import types

import pytest
import torch

from plenoxels_gb300 import train
from plenoxels_gb300.batch import BatchedTrainStep
from plenoxels_gb300.grid_functions import pool_shape


def test_receptive_field_schedule_follows_train_py():
    # scripts/train.py:90-91, :106: odd fields 93..3, five steps each, then 0
    ref = [i for i in range(93, 2, -2) if i % 2 != 0]
    assert train.DEFAULT_FIELDS == ref and train.STEPS_PER_FIELD == 5
    stub = types.SimpleNamespace(fields=train.DEFAULT_FIELDS, steps_per_field=5)
    for i in range(0, 5 * len(ref) + 20):
        want = ref[i // 5] if i // 5 < len(ref) else 0
        assert train.Trainer.field(stub, i) == want


@pytest.mark.parametrize("side,r", [(64, 93), (64, 33), (128, 21), (256, 9), (32, 3), (31, 5)])
def test_pooled_shapes_match_avg_pool3d(side, r):
    stride = max(1, r // 4)  # scripts/train.py:110
    if r > side:
        return
    ref = torch.nn.functional.avg_pool3d(torch.zeros(1, 4, side, side, side), r, stride=stride).shape[2:]
    od, scratch = pool_shape((side, side, side, 4), r, stride)
    assert tuple(od) == tuple(ref)
    assert scratch > 0


def test_batched_tiles_cover_the_longest_ray():
    for S, fits in [(512, {1, 2, 4, 8}), (1024, {1, 2, 4, 8}), (1025, {2, 4, 8}), (2500, {4, 8}),
                    (8192, {8})]:
        stub = types.SimpleNamespace(max_samples=S)
        got = {k for k in (1, 2, 4, 8) if BatchedTrainStep._tile_fits(stub, (k, 256))}
        assert got == fits, (S, got)


def test_bench_zeroes_multi_rank_gradients_densely():
    """Marked zeroing clears only the cells a rank's own steps wrote; an in-place
    all-reduce over ranks writes others, so multi-rank bench runs use the dense fill."""
    import importlib.util
    import os
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "bench.py")
    spec = importlib.util.spec_from_file_location("bench_module", path)
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    assert bench.zeroing_for(1) == bench.ZEROING
    assert all(bench.zeroing_for(n) == "fill" for n in (2, 4, 8))
