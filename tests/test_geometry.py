"""Geometry helpers (automs_gb300/geometry.py) against the reference's own
functions (go.py:248-512, 1309-1338) run on the same seeded inputs
(tests/golden/geometry_ref.npz, made by tests/golden/make_golden.py)."""
import os

import numpy as np

from automs_gb300 import geometry as G
from make_golden import DOOR_ANGLES, geometry_inputs, write_scene_text_files

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "geometry_ref.npz")


def close(a, b, tol=2e-6):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    assert np.max(np.abs(a - b)) <= tol * max(1.0, np.max(np.abs(b))), np.max(np.abs(a - b))


def test_geometry_helpers_match_reference():
    g = np.load(GOLD)
    inp = geometry_inputs()
    cpu = dict(device="cpu")
    for n, (th, ph, up, pol, u) in enumerate(inp["dirs"]):
        close(G.gen_direction_from_angle(th, ph, up, pol, unit=u, **cpu), g[f"dir{n}"])
    for n, (c, k, i, size, sp) in enumerate(inp["mats"]):
        close(G.gen_pos_matrix(c, k, i, size, sp, **cpu), g[f"mat{n}"])
    for n, (c, k, i, size, sp, th) in enumerate(inp["mss"]):
        pos, bh, kd = G.gen_ms(c, k, i, size, sp, th, **cpu)
        close(pos, g[f"ms{n}_pos"])
        close(np.asarray(bh, np.float32), g[f"ms{n}_bh"])
        close(kd, g[f"ms{n}_k"])
    for n, (w, ij) in enumerate(inp["walls"]):
        v, kd, idir = G.gen_sth_from_wall(w, ij, **cpu)
        close(np.stack([np.asarray(v), np.asarray(kd), np.asarray(idir)]), g[f"wall{n}"])
    for n, (x, y, z) in enumerate(inp["ends"]):
        close(G.gen_pos_from_endpoint(x, y, z, **cpu), g[f"end{n}"])
    for n, (c, xl, yl, zl) in enumerate(inp["boxes"]):
        close(np.asarray(G.create_vertex_buffer(c, xl, yl, zl), np.float32), g[f"box{n}"])


def test_scene_text_files_match_reference(tmp_path):
    g = np.load(GOLD)
    write_scene_text_files(str(tmp_path))
    c, k = G.get_ap(str(tmp_path))
    assert np.array_equal(np.asarray([c, k], np.float64), g["ap"])
    for n, ang in enumerate(DOOR_ANGLES):
        assert np.array_equal(np.asarray(G.get_doors(str(tmp_path), ang), np.float64), g[f"doors{n}"])
    assert np.array_equal(np.asarray(G.get_walls(str(tmp_path)), np.float64), g["walls"])
