"""Helpers for the tests on the reference's own scene folder (stl/4321 of
the reference tree), rebuilt from tests/golden/ref_scene_4321.npz: the
fixture holds the folder's STL triangles, mat.txt and wall.txt, the inputs
of a reduced channel set, and what the reference's build_channels
(go.py:1135-1247, with its ingest go.py:679-737) produced for it."""
import os
import re
import struct

import numpy as np

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
LAM = 3e8 / 60e9


def load():
    return np.load(os.path.join(GOLD, "ref_scene_4321.npz"))


def blocks(fx):
    """{file name: triangles [n, 3, 3] float32} of the scene folder."""
    out, o = {}, 0
    for name, n in zip(fx["stl_names"], fx["stl_counts"]):
        out[str(name)] = fx["stl_tris"][o:o + int(n)]
        o += int(n)
    return out


def write_folder(fx, path):
    """Write the scene folder (binary STL files, mat.txt, wall.txt)."""
    for name, tris in blocks(fx).items():
        with open(os.path.join(path, name), "wb") as f:
            f.write(b"\0" * 80 + struct.pack("<I", len(tris)))
            for t in tris:
                f.write(struct.pack("<12fH", 0.0, 0.0, 0.0, *[float(x) for x in t.reshape(-1)], 0))
    with open(os.path.join(path, "mat.txt"), "w") as f:
        f.write(str(fx["mat_txt"]))
    with open(os.path.join(path, "wall.txt"), "w") as f:
        f.write(str(fx["wall_txt"]))


def expected_ingest(fx, order, blackhole=(), reflector=(), door=()):
    """The scene arrays go.py:679-737 builds when os.listdir gives `order`:
    STL files in that order with the material named by the file-name suffix,
    then blackhole (0), reflector (1) and door (-0.7) quads, each with its
    own material row appended after mat.txt's rows."""
    names, props = [], []
    for line in str(fx["mat_txt"]).splitlines():
        v = line.split()
        if v:
            names.append(v[0])
            props.append([float(x) for x in v[1:]])
    bl = blocks(fx)
    tris, mats = [], []
    for fn in order:
        if not fn.endswith(".stl"):
            continue
        mid = names.index(fn.split("_")[-1].split(".stl")[0])
        tris.append(bl[fn])
        mats.append(np.full(len(bl[fn]), mid, np.int32))
    for buf, val in ((blackhole, 0.0), (reflector, 1.0), (door, -0.7)):
        if len(buf):
            props.append([val] * 19)
            t = np.asarray(buf, np.float32).reshape(-1, 3, 3)
            tris.append(t)
            mats.append(np.full(len(t), len(names), np.int32))
            names.append("pseudo")
    return (np.concatenate(tris).astype(np.float32), np.concatenate(mats),
            np.asarray(props, np.float32))


def trace_buffers(fx, key):
    """Blackhole, reflector and door quads of one trace of the channel set
    (the other metasurfaces are blackholes, go.py:1173-1245)."""
    n = sum(1 for k in fx.files if k.startswith("ms") and k.endswith("_pos"))
    skip = {int(i) for i in re.findall(r"\{(\d+)\}", key)}  # the metasurfaces traced
    bh = [fx[f"ms{i}_blackhole"] for i in range(n) if i not in skip]
    return bh, list(fx["reflector"]), list(fx["door"])
