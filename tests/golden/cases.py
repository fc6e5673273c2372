"""Seeded input cases shared by the fixture generator and the tests.

Every case is rebuilt from a name; the fixtures store a sha256 of the inputs
so that a change in a generator is caught instead of silently comparing
different inputs.
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
from automs_gb300 import scenes  # noqa: E402

STAT_KEYS = ("rx_paths", "rx_fail", "fwd_records", "unique_records", "unique_paths", "rounds")

CHANNEL_CASES = ("tiny", "small", "pen_l3", "allpen_l4", "ms_to_rx", "ap_to_ms",
                 "bp3_door", "spl2_cap", "l0", "l5", "ms3_ap_rx", "ms3_ap_ms", "ms3_ms_rx",
                 "farfield", "empty_scene", "one_tri", "one_rx", "reserve1", "ragged",
                 "rx_row")

# edge cases on the tiny room: no triangles (free space), a single triangle
# (the hierarchy is one leaf), a single Rx, the smallest record cap with four
# samples per launch (the cap binds), an Rx grid that the grid cell size
# divides in neither direction, and a one-row Rx grid
_EDGE = ("empty_scene", "one_tri", "one_rx", "reserve1", "ragged", "rx_row")

# the three traces of the small one-metasurface channel set
_MS3 = {"ms3_ap_rx": "src_to_dst", "ms3_ap_ms": "src_to_ms{0}", "ms3_ms_rx": "ms{0}_to_dst"}


def _ms_array(n0, n1, center, normal, up, spacing):
    normal = np.asarray(normal, np.float64)
    up = np.asarray(up, np.float64)
    side = np.cross(normal, up)
    i = np.arange(n0) - (n0 - 1) / 2
    j = np.arange(n1) - (n1 - 1) / 2
    g = (np.asarray(center, np.float64)[None, None, :]
         - i[:, None, None] * spacing * up[None, None, :]
         + j[None, :, None] * spacing * side[None, None, :])
    return g.astype(np.float32)


def channel_case(name):
    lam = scenes.WAVE_LEN_60GHZ
    if name in _MS3:
        m = scenes.channel_ms_config("ms-small")
        t = m["traces"][_MS3[name]]
        tris, mat, mp = m["tris"], m["mat"], m["mat_prop"]
        if t["blackhole"]:
            tris, mat, mp = scenes.with_blackholes(tris, mat, mp, [m["blackhole"]])
        return dict(tris=tris, mat=mat, mat_prop=mp, src=t["src"], dst=t["dst"],
                    params=dict(t["params"]))
    if name in ("tiny", "pen_l3", "allpen_l4", "ms_to_rx", "bp3_door", "spl2_cap", "l0", "l5",
                "farfield") + _EDGE:
        c = scenes.coverage_config("coverage-tiny")
    elif name in ("small", "ap_to_ms"):
        c = scenes.coverage_config("coverage-small")
    else:
        raise ValueError(name)
    p = c["params"]
    if name == "pen_l3":
        c["mat_prop"][3:] *= -1
        p["max_reflection"] = 3
    elif name == "allpen_l4":
        c["mat_prop"][:] *= -1
        p["max_reflection"] = 4
        p["launch_x"] = p["launch_y"] = 32
    elif name == "ms_to_rx":
        c["src"] = _ms_array(4, 4, (4.0, 8.0 - 1e-3, 2.0), (0, -1, 0), (0, 0, 1), lam / 2)
        p["src_bptype"] = 1
        p["src_dir"] = [0.0, -1.0, 0.0]
    elif name == "ap_to_ms":
        c["dst"] = _ms_array(7, 6, (4.0, 8.0 - 1e-3, 2.0), (0, -1, 0), (0, 0, 1), 0.2)
        p["dst_bptype"] = 1
        p["dst_dir"] = [0.0, -1.0, 0.0]
        p["dst_r"] = 0.1
    elif name == "bp3_door":
        door = np.array([[[3.0, 4.0, 0.0], [5.0, 4.0, 0.0], [5.0, 4.0, 2.2]],
                         [[3.0, 4.0, 0.0], [5.0, 4.0, 2.2], [3.0, 4.0, 2.2]]], np.float32)
        c["tris"] = np.concatenate([c["tris"], door], 0)
        c["mat"] = np.concatenate([c["mat"], np.full(2, c["mat_prop"].shape[0], np.int32)])
        c["mat_prop"] = np.concatenate([c["mat_prop"], np.full((1, 19), -0.7, np.float32)], 0)
        p["src_bptype"] = 3
    elif name == "spl2_cap":
        p["samples_per_launch"] = 2
        p["reserve_size"] = 3
    elif name == "l0":
        p["max_reflection"] = 0
    elif name == "farfield":
        # A 20 m wavelength puts second reflections in the far field of the
        # first reflecting triangle (segment > 2 maxedge^2 / lambda,
        # optixPathTracer.cu:369-389), which 60 GHz never does on this mesh
        # of metre-sized triangles: the FSPL then splits at that hit.
        p["wave_len"] = 20.0
        p["max_reflection"] = 3
    elif name == "empty_scene":
        c["tris"] = np.zeros((0, 3, 3), np.float32)
        c["mat"] = np.zeros(0, np.int32)
    elif name == "one_tri":
        c["tris"] = np.ascontiguousarray(c["tris"].reshape(-1, 3, 3)[:1])
        c["mat"] = np.ascontiguousarray(c["mat"][:1])
    elif name == "one_rx":
        c["dst"] = np.ascontiguousarray(c["dst"][3:4, 5:6])
        p["launch_x"] = p["launch_y"] = 300
    elif name == "reserve1":
        p["reserve_size"] = 1
        p["samples_per_launch"] = 4
        p["launch_x"] = p["launch_y"] = 32
    elif name == "ragged":
        c["dst"] = np.ascontiguousarray(c["dst"][:7, :13])
    elif name == "rx_row":
        c["dst"] = np.ascontiguousarray(c["dst"][:1])
    elif name == "l5":
        c["mat_prop"][3:] *= -1
        p["max_reflection"] = 5
        p["launch_x"] = p["launch_y"] = 16
    return c


OBJECTIVE_CASES = ("c1", "c30", "noms", "two_ms")


def _cn(rng, shape, lam=scenes.WAVE_LEN_60GHZ):
    d = rng.uniform(2.0, 15.0, size=shape)
    g = (rng.normal(size=shape) + 1j * rng.normal(size=shape)) / np.sqrt(2)
    return (g * lam / (4 * np.pi * d)).astype(np.complex64)


def objective_case(name):
    """Channels in the reference orientation (go.py:107-157):
    src_to_dst [S,R], src_to_ms{i} [S,M_i], ms{i}_to_dst [M_i,R],
    ms{i}_to_ms{j} [M_i,M_j] (i<j)."""
    spec = {
        "c1": dict(S=16, Ms=[64], R=256, C=1, w=1.0 / 256, reflex=1, max_phase=360.0, seed=1),
        "c30": dict(S=36, Ms=[96], R=200, C=30, w=0.5, reflex=1, max_phase=300.0, seed=2),
        "noms": dict(S=36, Ms=[], R=200, C=8, w=0.5, reflex=0, max_phase=300.0, seed=3),
        "two_ms": dict(S=8, Ms=[32, 24], R=100, C=4, w=1.0, reflex=2, max_phase=270.0, seed=4),
    }[name]
    rng = np.random.Generator(np.random.PCG64(100 + spec["seed"]))
    S, R, Ms = spec["S"], spec["R"], spec["Ms"]
    ch = {"src_to_dst": _cn(rng, (S, R))}
    for i, M in enumerate(Ms):
        ch["src_to_ms{%d}" % i] = _cn(rng, (S, M))
        ch["ms{%d}_to_dst" % i] = _cn(rng, (M, R))
    for i in range(len(Ms)):
        for j in range(i + 1, len(Ms)):
            ch["ms{%d}_to_ms{%d}" % (i, j)] = _cn(rng, (Ms[i], Ms[j]))
    theta = rng.uniform(0, 2 * np.pi, size=(spec["C"], S)).astype(np.float32)
    phi = [rng.uniform(0, 2 * np.pi, size=M).astype(np.float32) for M in Ms]
    return dict(channels=ch, theta=theta, phi=phi, n_ms=len(Ms), max_ms_reflex=spec["reflex"],
                code_num=spec["C"], w=spec["w"], max_phase_deg=spec["max_phase"],
                seed=spec["seed"])


# ------------------------------------------------- the reference's scene
# A reduced channel set on the reference's own scene folder (stl/4321 of the
# reference tree), placed as its single trial places AP, Rx and metasurface
# (physical_exp_nni_model.py:26-87) but smaller: 2x2 AP, 20x18 Rx at one
# height, two metasurfaces (6x8 on wall 1 at the trial's ms_j, and a 4x6
# relay 1 m in front of it facing it, so that the ms0 -> ms1 trace finds
# paths with the reference's 100 x 100 launch), a door and a reflector
# quad, 3 reflections.
REF_SCENE = "stl/4321"
REF_SCENE_L = 3
REF_SCENE_FLOOR = -1.4161


def reference_scene_setup(go, folder, lam):
    """Inputs of the reduced reference-scene channel set, made with the
    reference's geometry helpers (module `go`)."""
    walls = go.get_walls(folder)
    center_a, k_a, _ = go.gen_sth_from_wall(walls[0], (0.5, 0.5))
    center_a[2] = REF_SCENE_FLOOR + 2.5
    ap_dir = go.gen_direction_from_angle(0, 23.4352 - 90, [0, 0, 1], [0, 1, 0])
    src = go.gen_pos_matrix(center_a + k_a * 0.3, ap_dir, [0, 0, -1], (2, 2), lam * 0.58)
    dst = go.gen_pos_from_endpoint([-6, 2.4, 20], [-1, 6.5, 18], REF_SCENE_FLOOR + 0.9)
    c, k, i = go.gen_sth_from_wall(walls[1], (0.5, 0.11939808933765397))
    c[2] = REF_SCENE_FLOOR + 2.0
    pos, bh, n = go.gen_ms(c.clone(), k, i, (6, 8), lam / 2)
    ms_list = [go.Metasurface(pos, (6, 8), n, n, bh, 300)]
    pos, bh, n = go.gen_ms(c + k * 1.0, -k, i, (4, 6), lam / 2)
    ms_list.append(go.Metasurface(pos, (4, 6), n, n, bh, 300))
    z0, z1 = REF_SCENE_FLOOR, REF_SCENE_FLOOR + 2.1
    door = [[[-3.0, 0.5, z1], [-3.0, 1.5, z1], [-3.0, 0.5, z0]],
            [[-3.0, 0.5, z0], [-3.0, 1.5, z0], [-3.0, 1.5, z1]]]
    r0, r1 = REF_SCENE_FLOOR + 0.9, REF_SCENE_FLOOR + 1.9
    reflector = [[[-0.5, 1.0, r1], [-0.5, 2.0, r1], [-0.5, 1.0, r0]],
                 [[-0.5, 1.0, r0], [-0.5, 2.0, r0], [-0.5, 2.0, r1]]]
    return dict(src=src, dst=dst, ap_dir=ap_dir, ms_list=ms_list, door=[door],
                reflector=[reflector])
