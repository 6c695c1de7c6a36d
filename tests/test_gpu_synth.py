"""The GPU ray caster of the synthetic scenes against the CPU one (same scene
model, FP32 instead of FP64 arithmetic)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_gpu_render_matches_cpu_render(gpu):
    from slam_gb300 import synth
    from slam_gb300.warmstart import render_views
    cam = synth.Camera().scaled(320, 240)
    rng = np.random.default_rng(4)
    tapered = synth.make_corridor(5, 0)
    tapered.wall_taper = 0.05
    scenes = [synth.make_room(11, 20), synth.make_corridor(3), tapered]
    poses = [synth.room_camera(rng), synth.corridor_camera(rng), synth.corridor_camera(rng)]
    seeds = [17, 29, 31]
    g = render_views(scenes, [0, 1, 2], poses, seeds, cam, depth=True, rgba=True, model=True)
    for i in range(3):
        c = synth.render(scenes[i], poses[i], cam, noise_seed=seeds[i], depth=True, rgba=True, model=True)
        gv, gn = g["vert"][i].cpu().numpy(), g["norm"][i].cpu().numpy()
        hit = (c["vert"][..., 3] > 0) & (gv[..., 3] > 0)
        assert hit.mean() > 0.99 * (c["vert"][..., 3] > 0).mean()
        assert np.abs(gv[hit, :3] - c["vert"][hit, :3]).max() < 1e-3
        assert np.percentile(np.abs(gn[hit, :3] - c["norm"][hit, :3]).max(axis=1), 99) < 1e-3
        drgb = np.abs(g["rgba"][i].cpu().numpy().astype(int) - c["rgba"].astype(int))
        assert (drgb[..., :3].max(axis=-1) <= 1).mean() > 0.99
        import torch
        gd = g["depth"][i].view(torch.int16).cpu().numpy().view(np.uint16).astype(int)
        cd = c["depth"].astype(int)
        assert (np.abs(gd - cd) <= 1).mean() > 0.99
