"""Host-side part of the Ferns relocalisation check (photometric_check,
src/lc/Ferns.cpp:309-356) on small synthetic images, and the parameter sets
of the two verification callers (no GPU)."""
import numpy as np


def _scene(cam):
    from slam_gb300 import synth
    T = synth.room_camera(np.random.default_rng(1))
    m = synth.render(synth.make_room(1), T, cam, depth=False, rgba=True, model=True)
    return T, m["vert"], m["rgba"][..., :3].copy()


def test_photometric_error_grows_with_the_pose_error_and_empty_is_nan():
    """The same view scores low (not zero: the reference truncates the
    projected coordinates, so a pixel centre can land one pixel left/up);
    a wrong pose scores much higher."""
    from slam_gb300 import synth, verify
    cam = synth.Camera().scaled(80, 60)
    T, vert, rgb = _scene(cam)
    pts = np.array([(x, y) for y in range(2, 58, 5) for x in range(2, 78, 5)])
    same = verify.photometric_check(vert, rgb, T, T, rgb, pts, cam, 5000)
    off = T @ synth.pose(synth.rotvec_to_R([0.0, 0.15, 0.0]), np.array([0.1, 0.0, 0.0]))
    wrong = verify.photometric_check(vert, rgb, off, T, rgb, pts, cam, 5000)
    assert wrong > 3 * same
    # every sample beyond the depth cut: no comparison, NaN (the reference's 0 / 0)
    assert np.isnan(verify.photometric_check(vert, rgb, T, T, rgb, pts, cam, 10))


def test_parameter_sets_follow_the_reference_callers():
    from slam_gb300 import verify
    f = verify.ferns_params()
    assert (f["icpWeight"], f["so3"], f["max_icp_error"], f["min_icp_count"]) == (100.0, False, 3e-4, 2400.0)
    assert verify.ferns_params(lost=True)["min_icp_count"] == 1400.0
    m = verify.model_to_model_params()
    assert (m["icpWeight"], m["so3"], m["max_icp_error"], m["min_icp_count"], m["max_covariance"]) == \
        (10.0, False, 5e-5, 40000.0, 1e-5)
