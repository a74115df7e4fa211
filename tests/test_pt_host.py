"""Path-tracer host logic that needs no GPU: the camera frame the C ABI
derives (MRay's CameraPinhole constructor) equals the oracle's, bit for bit;
the oracle's estimator is unbiased across its three sample modes."""
import numpy as np

import oracle
from mray_gb300 import scenes
from mray_gb300.pt import PathTracer


def test_camera_frame_matches_oracle(cuda_lib, built_libs):
    cam = scenes.box_camera()
    p = PathTracer.params(256, 256, 1, cam)
    frame = PathTracer.camera_frame(p)
    op = oracle.PtScene.params(256, 256, 1, cam)
    ref = np.array(list(op.camPos) + list(op.camBottomLeft) + list(op.camRight) + list(op.camUp) +
                   list(op.planeSize) + [op.nearT, op.farT], np.float32)
    assert np.array_equal(frame.view(np.uint32), ref.view(np.uint32))


def test_oracle_sample_modes_agree(built_libs):
    """Pure, NEE and NEE+MIS estimate the same image (relMSE of 16x16 tiles)."""
    S = oracle.PtScene(scenes.box_scene(0))
    cam = scenes.box_camera()
    imgs = []
    for mode in (oracle.PT_PURE, oracle.PT_NEE, oracle.PT_NEE_MIS):
        img = S.render(S.params(32, 32, 256, cam, sample_mode=mode, seed=mode))
        v = img[..., :3] / img[..., 3:]
        imgs.append(v.reshape(4, 8, 4, 8, 3).mean(axis=(1, 3)))
    ref = imgs[2]
    for v in imgs[:2]:
        rel = np.mean((v - ref) ** 2 / (ref ** 2 + 1e-3))
        assert rel < 0.01, rel
