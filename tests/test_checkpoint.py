"""The reference's checkpoint format (scripts/train.py:197-210) round-trips on CPU."""
import torch

from plenoxels_gb300.inference import PARAM_KEYS, load_checkpoint, save_checkpoint


def test_checkpoint_round_trip(tmp_path):
    grid = torch.rand(6, 5, 4, 4)
    grad = torch.rand(6, 5, 4, 4)
    param = dict(device="cuda:0", number_of_rays=128, num_samples=600, delta_step=0.0125,
                 even_spread=False, camera_ray=False, points_distance=0.0125, gridsize=[6, 5, 4])
    path = tmp_path / "grid.pth"
    save_checkpoint(path, grid, grad, param)
    raw = torch.load(path, weights_only=False)  # the reference reads it with torch.load
    assert set(raw) == {"grid", "grid_grad", "param"} and set(raw["param"]) == set(PARAM_KEYS)
    back = load_checkpoint(path, device="cpu")
    assert torch.equal(back["grid"], grid) and torch.equal(back["grid_grad"], grad)
    assert back["param"] == param
