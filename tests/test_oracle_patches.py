"""The oracle's patch entry (render_patch_u8 / accumulate_patch_f32 for a list
of patches, renderer.rs:306-362) agrees with its whole-frame patch order."""

import numpy as np

from convector_gb300 import scenes


def _room(cvx, orc):
    text, mats = scenes.room_sphere()
    bvh = cvx.Bvh.from_meshes([cvx.Mesh.parse(text, mats)])
    cam = scenes.default_camera(cvx.Camera())
    return orc.OracleScene.from_bvh(bvh), cam.as_array()


def test_patch_list_equals_frame_patch_order(cvx, orc):
    osc, cam = _room(cvx, orc)
    w, h = 96, 64
    rgba, gbuf, _, rays = osc.render(cam, w, h, 42, rng_order=0, traversal=0)
    origins = [(x, y) for x in range(0, w, 32) for y in range(0, h, 32)]
    prgba = np.zeros((h, w), np.uint32)
    pgbuf = np.zeros((h, w), np.uint32)
    prays = osc.render_patches(cam, w, h, 42, 32, origins, rgba=prgba, gbuf=pgbuf)
    assert (prgba == rgba).all() and (pgbuf == gbuf).all() and prays == rays


def test_patch_list_leaves_other_pixels(cvx, orc):
    osc, cam = _room(cvx, orc)
    w, h = 96, 64
    rgba = np.full((h, w), 0xDEADBEEF, np.uint32)
    osc.render_patches(cam, w, h, 3, 16, [(16, 4), (64, 48)], rgba=rgba)
    touched = np.zeros((h, w), bool)
    touched[4:20, 16:32] = True
    touched[48:64, 64:80] = True
    assert (rgba[~touched] == 0xDEADBEEF).all()
    assert (rgba[touched] != 0xDEADBEEF).all()
