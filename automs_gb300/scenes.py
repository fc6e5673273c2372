"""Seeded synthetic scenes and the binary-STL scene reader.

The generators stand in for the reference's own scene (stl/4321 of the
reference tree): shoebox rooms with axis-aligned box obstacles, uniform
linear Tx arrays and planar Rx grids, all float32, seeded with
numpy.random.Generator(PCG64(seed)).

Scene arrays follow the reference op's layout (go.py:679-737):
  tris      float32 [N_tri, 3, 3]   (scene_buffer reshaped)
  mat       int32   [N_tri]
  mat_prop  float32 [n_mat, 19]     (negative = penetrable)
"""
import os
import struct

import numpy as np

WAVE_LEN_60GHZ = 3e8 / 60e9  # go.py:1343


def _quad_grid(p0, u, v, nu, nv):
    """Triangles of a planar quad p0 + s*u + t*v, s,t in [0,1], split into
    nu x nv cells of two triangles each."""
    tris = []
    for i in range(nu):
        for j in range(nv):
            a = p0 + u * (i / nu) + v * (j / nv)
            b = p0 + u * ((i + 1) / nu) + v * (j / nv)
            c = p0 + u * ((i + 1) / nu) + v * ((j + 1) / nv)
            d = p0 + u * (i / nu) + v * ((j + 1) / nv)
            tris.append([a, b, c])
            tris.append([a, c, d])
    return tris


def box_tris(lo, hi, n=1):
    """12 n^2 triangles of an axis-aligned box; n may be a pair (nu, nv) of
    quads per face side."""
    nu, nv = (n, n) if np.isscalar(n) else n
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    ex = np.array([hi[0] - lo[0], 0, 0])
    ey = np.array([0, hi[1] - lo[1], 0])
    ez = np.array([0, 0, hi[2] - lo[2]])
    tris = []
    tris += _quad_grid(lo, ex, ey, nu, nv)            # bottom
    tris += _quad_grid(lo + ez, ex, ey, nu, nv)       # top
    tris += _quad_grid(lo, ex, ez, nu, nv)            # y = lo
    tris += _quad_grid(lo + ey, ex, ez, nu, nv)       # y = hi
    tris += _quad_grid(lo, ey, ez, nu, nv)            # x = lo
    tris += _quad_grid(lo + ex, ey, ez, nu, nv)       # x = hi
    return tris


def shoebox_scene(n_boxes=20, room=(12.0, 8.0, 3.0), box_tess=3, room_tess=1,
                  seed=0, keep_clear=()):
    """Shoebox room [0,X]x[0,Y]x[0,Z] with n_boxes floor-standing boxes.

    Box footprints U[0.2,1.5]^2, heights U[0.3,2.0], centres uniform in the
    room and clipped to it; boxes that would contain a point of keep_clear
    (e.g. the Tx position) are redrawn.  Materials: floor, ceiling, walls and
    one per box, each with a reflection coefficient U[0.3,0.7] over all 19
    angle bins (non-penetrable)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    X, Y, Z = room
    tris, mats = [], []
    props = [rng.uniform(0.3, 0.7) for _ in range(3)]
    origin = np.zeros(3)
    ex, ey, ez = np.array([X, 0, 0.0]), np.array([0, Y, 0.0]), np.array([0, 0, Z])
    floor = _quad_grid(origin, ex, ey, room_tess, room_tess)
    ceil = _quad_grid(origin + ez, ex, ey, room_tess, room_tess)
    walls = (_quad_grid(origin, ex, ez, room_tess, room_tess)
             + _quad_grid(origin + ey, ex, ez, room_tess, room_tess)
             + _quad_grid(origin, ey, ez, room_tess, room_tess)
             + _quad_grid(origin + ex, ey, ez, room_tess, room_tess))
    for group, m in ((floor, 0), (ceil, 1), (walls, 2)):
        tris += group
        mats += [m] * len(group)
    clear = [np.asarray(p, np.float64) for p in keep_clear]
    for b in range(n_boxes):
        while True:
            sx, sy = rng.uniform(0.2, 1.5, size=2)
            h = rng.uniform(0.3, 2.0)
            cx, cy = rng.uniform(0, X), rng.uniform(0, Y)
            lo = np.array([max(cx - sx / 2, 0.0), max(cy - sy / 2, 0.0), 0.0])
            hi = np.array([min(cx + sx / 2, X), min(cy + sy / 2, Y), min(h, Z)])
            if all(not (np.all(p >= lo - 0.05) and np.all(p <= hi + 0.05)) for p in clear):
                break
        bt = box_tris(lo, hi, box_tess)
        tris += bt
        mats += [3 + b] * len(bt)
        props.append(rng.uniform(0.3, 0.7))
    tris = np.asarray(tris, np.float32)
    mat = np.asarray(mats, np.int32)
    mat_prop = np.repeat(np.asarray(props, np.float32)[:, None], 19, axis=1)
    return tris, mat, mat_prop


def ula(center, axis, n, spacing):
    """Uniform linear array as [1, n, 3] float32 (go.py stores arrays 2-D)."""
    center = np.asarray(center, np.float64)
    axis = np.asarray(axis, np.float64)
    axis = axis / np.linalg.norm(axis)
    k = np.arange(n) - (n - 1) / 2
    return (center[None, :] + k[:, None] * spacing * axis[None, :]).astype(np.float32)[None]


def rx_grid(x0, x1, nx, y0, y1, ny, z):
    """Planar Rx grid [nx, ny, 3] float32 like gen_pos_from_endpoint."""
    xs = np.linspace(x0, x1, nx, dtype=np.float32)
    ys = np.linspace(y0, y1, ny, dtype=np.float32)
    g = np.stack(np.meshgrid(xs, ys, indexing="ij"), axis=-1)
    zz = np.full(g.shape[:2] + (1,), z, np.float32)
    return np.concatenate([g, zz], axis=-1).astype(np.float32)


def coverage_config(name="coverage-128", seed=0):
    """Named coverage workloads.

    coverage-128: 12x8x3 m room, 20 boxes (2172 triangles), 16-element ULA at
      (6, 0.5, 2.5) facing +y, 128x128 Rx grid at z=1.5, 1000x1000 launch,
      2 reflections.
    coverage-small: the same room with 4 boxes, 4 Tx, 24x24 Rx, 96x96 launch
      (sized for the oracle).
    """
    lam = WAVE_LEN_60GHZ
    tx_pos = (6.0, 0.5, 2.5)
    if name == "coverage-128":
        tris, mat, mat_prop = shoebox_scene(20, seed=seed, keep_clear=[tx_pos])
        src = ula(tx_pos, (1, 0, 0), 16, lam / 2)
        dst = rx_grid(0.25, 11.75, 128, 0.25, 7.75, 128, 1.5)
        lx = ly = 1000
        L = 2
    elif name == "coverage-small":
        tris, mat, mat_prop = shoebox_scene(4, box_tess=1, seed=seed, keep_clear=[tx_pos])
        src = ula(tx_pos, (1, 0, 0), 4, lam / 2)
        dst = rx_grid(0.25, 11.75, 24, 0.25, 7.75, 24, 1.5)
        lx = ly = 96
        L = 2
    elif name == "coverage-tiny":
        tris, mat, mat_prop = shoebox_scene(2, box_tess=1, seed=seed, keep_clear=[tx_pos])
        src = ula(tx_pos, (1, 0, 0), 2, lam / 2)
        dst = rx_grid(0.25, 11.75, 12, 0.25, 7.75, 12, 1.5)
        lx = ly = 48
        L = 2
    else:
        raise ValueError(name)
    params = dict(samples_per_launch=1, launch_x=lx, launch_y=ly, wave_len=lam,
                  max_reflection=L, reserve_size=100, src_bptype=2, dst_bptype=0,
                  dst_gridsize=5, src_r=0.5e-5, dst_r=0.06,
                  src_dir=[0.0, 1.0, 0.0], dst_dir=[0.0, 0.0, 0.0])
    return dict(tris=tris, mat=mat, mat_prop=mat_prop, src=src, dst=dst, params=params)


def metasurface(center, normal, down, n, spacing, thickness=1e-3):
    """Element positions [n, n, 3], blackhole quad [2, 3, 3] and unit normal of
    an n x n metasurface (gen_ms, go.py:388-443), in numpy float32."""
    k = np.asarray(normal, np.float64)
    k = k / np.linalg.norm(k)
    i = np.asarray(down, np.float64)
    j = np.cross(k, i)
    i = i / np.linalg.norm(i)
    j = j / np.linalg.norm(j)
    c = np.asarray(center, np.float64) + k * thickness
    u = np.linspace(-(n - 1) / 2, (n - 1) / 2, n)
    pos = c + (u[:, None, None] * i + u[None, :, None] * j) * spacing
    io, jo = i * n / 2 * spacing, j * n / 2 * spacing
    ul, dr, ur, dl = c - io - jo, c + io + jo, c + io - jo, c - io + jo
    quad = np.array([[ul, ur, dl], [dl, dr, ur]], np.float32)
    return pos.astype(np.float32), quad, k.astype(np.float32)


def with_blackholes(tris, mat, mat_prop, quads):
    """Append blackhole quads (an all-zero material row, go.py:708-716)."""
    if len(quads) == 0:
        return tris, mat, mat_prop
    q = np.asarray(quads, np.float32).reshape(-1, 3, 3)
    return (np.concatenate([tris, q], 0),
            np.concatenate([mat, np.full(q.shape[0], mat_prop.shape[0], np.int32)]),
            np.concatenate([mat_prop, np.zeros((1, 19), np.float32)], 0))


def channel_ms_config(name="ms-256", seed=0):
    """Channel set with one metasurface: AP->Rx (the metasurface a
    blackhole), AP->MS and MS->Rx traces (build_channels, go.py:1135-1247).

    ms-256: 12x8x3 m room with 200 boxes, 5x4 quads per box face and 13x13
      per room face (50,028 triangles); 16-element ULA at (6, 0.5, 2.5)
      facing +y; 32x32 metasurface at lambda/2 on the y=8 wall centred at
      (6, 8, 2), normal -y; 256x256 Rx grid at z=1.5; 1000x1000 launch;
      3 reflections.
    ms-small: 12 boxes with 1 quad per face, 6x6 metasurface, 20x20 Rx,
      128x128 launch, 3 reflections (sized for the oracle).
    """
    lam = WAVE_LEN_60GHZ
    tx_pos = (6.0, 0.5, 2.5)
    ms_c = (6.0, 8.0 - 1e-3, 2.0)
    if name == "ms-256":
        tris, mat, mat_prop = shoebox_scene(200, box_tess=(5, 4), room_tess=13, seed=seed,
                                            keep_clear=[tx_pos, ms_c])
        n_src, n_ms, n_rx, launch = 16, 32, 256, 1000
    elif name == "ms-small":
        tris, mat, mat_prop = shoebox_scene(12, box_tess=1, seed=seed, keep_clear=[tx_pos, ms_c])
        n_src, n_ms, n_rx, launch = 4, 6, 20, 128
    else:
        raise ValueError(name)
    L = 3
    src = ula(tx_pos, (1, 0, 0), n_src, lam / 2)
    dst = rx_grid(0.25, 11.75, n_rx, 0.25, 7.75, n_rx, 1.5)
    pos, quad, k = metasurface(ms_c, (0, -1, 0), (0, 0, -1), n_ms, lam / 2)

    def prm(sbp, dbp, sdir, ddir):
        return dict(samples_per_launch=1, launch_x=launch, launch_y=launch, wave_len=lam,
                    max_reflection=L, reserve_size=100, src_bptype=sbp, dst_bptype=dbp,
                    dst_gridsize=5, src_r=0.5e-5, dst_r=0.06, src_dir=list(map(float, sdir)),
                    dst_dir=list(map(float, ddir)))

    ap_dir, none = (0.0, 1.0, 0.0), (0.0, 0.0, 0.0)
    return dict(tris=tris, mat=mat, mat_prop=mat_prop, src=src, dst=dst, ms=pos,
                blackhole=quad, normal=k,
                traces={
                    "src_to_dst": dict(src=src, dst=dst, blackhole=True,
                                       params=prm(2, 0, ap_dir, none)),
                    "src_to_ms{0}": dict(src=src, dst=pos, blackhole=False,
                                         params=prm(2, 1, ap_dir, k)),
                    "ms{0}_to_dst": dict(src=pos, dst=dst, blackhole=False,
                                         params=prm(1, 0, k, none)),
                })


def multiroom_scene(target_tris=200_000, rooms=(3, 3), seed=0, height=3.0):
    """Seeded building of rooms x rooms rooms, each side U[6, 15] m, 3 m tall.

    Outer shell (floor, ceiling, four walls) and interior walls on the room
    boundaries, each wall segment with a 1 m wide, 2.1 m tall door gap;
    floor-standing boxes (footprint U[0.2, 1.5]^2, height U[0.3, 2.0]) with
    5x4 quads per face are added room by room until the scene has about
    target_tris triangles.  Materials: floor, ceiling, walls, then one per
    box, reflection coefficients U[0.3, 0.7] over all 19 bins.
    Returns tris, mat, mat_prop, and the room grid edges (xs, ys)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    xs = np.concatenate([[0.0], np.cumsum(rng.uniform(6.0, 15.0, rooms[0]))])
    ys = np.concatenate([[0.0], np.cumsum(rng.uniform(6.0, 15.0, rooms[1]))])
    X, Y, Z = xs[-1], ys[-1], height
    tris, mats = [], []
    props = [rng.uniform(0.3, 0.7) for _ in range(3)]
    ez = np.array([0.0, 0.0, Z])
    floor = _quad_grid(np.zeros(3), np.array([X, 0, 0.0]), np.array([0, Y, 0.0]), 8, 8)
    ceil = _quad_grid(ez, np.array([X, 0, 0.0]), np.array([0, Y, 0.0]), 8, 8)
    tris += floor + ceil
    mats += [0] * len(floor) + [1] * len(ceil)

    def wall(p0, p1, door):
        """Vertical wall from p0 to p1 (floor points); door: gap centre
        fraction or None."""
        p0, p1 = np.asarray(p0, float), np.asarray(p1, float)
        L = np.linalg.norm(p1 - p0)
        u = (p1 - p0) / L
        out = []
        if door is None:
            out += _quad_grid(p0, p1 - p0, ez, 4, 2)
        else:
            c = door * L
            a, b = max(c - 0.5, 0.0), min(c + 0.5, L)
            if a > 0:
                out += _quad_grid(p0, u * a, ez, 2, 2)
            if b < L:
                out += _quad_grid(p0 + u * b, u * (L - b), ez, 2, 2)
            out += _quad_grid(p0 + u * a + np.array([0, 0, 2.1]), u * (b - a),
                              np.array([0, 0, Z - 2.1]), 1, 1)
        return out
    w = []
    w += wall((0, 0, 0), (X, 0, 0), None) + wall((0, Y, 0), (X, Y, 0), None)
    w += wall((0, 0, 0), (0, Y, 0), None) + wall((X, 0, 0), (X, Y, 0), None)
    for i in range(1, len(xs) - 1):          # interior walls x = xs[i]
        for j in range(len(ys) - 1):
            w += wall((xs[i], ys[j], 0), (xs[i], ys[j + 1], 0), rng.uniform(0.2, 0.8))
    for j in range(1, len(ys) - 1):          # interior walls y = ys[j]
        for i in range(len(xs) - 1):
            w += wall((xs[i], ys[j], 0), (xs[i + 1], ys[j], 0), rng.uniform(0.2, 0.8))
    tris += w
    mats += [2] * len(w)
    per_box = 12 * 5 * 4
    n_boxes = max(0, (target_tris - len(tris)) // per_box)
    nr = (len(xs) - 1) * (len(ys) - 1)
    for bidx in range(n_boxes):
        r = bidx % nr
        i, j = r % (len(xs) - 1), r // (len(xs) - 1)
        sx, sy = rng.uniform(0.2, 1.5, size=2)
        h = rng.uniform(0.3, 2.0)
        cx = rng.uniform(xs[i] + 0.3, xs[i + 1] - 0.3)
        cy = rng.uniform(ys[j] + 0.3, ys[j + 1] - 0.3)
        lo = np.array([max(cx - sx / 2, xs[i] + 0.05), max(cy - sy / 2, ys[j] + 0.05), 0.0])
        hi = np.array([min(cx + sx / 2, xs[i + 1] - 0.05), min(cy + sy / 2, ys[j + 1] - 0.05), h])
        bt = box_tris(lo, hi, (5, 4))
        tris += bt
        mats += [3 + bidx] * len(bt)
        props.append(rng.uniform(0.3, 0.7))
    tris = np.asarray(tris, np.float32)
    mat = np.asarray(mats, np.int32)
    mat_prop = np.repeat(np.asarray(props, np.float32)[:, None], 19, axis=1)
    return tris, mat, mat_prop, xs, ys


def tworoom_scene(seed=0, height=3.0):
    """Seeded two-room floor for the placement study: room A = [0, a] and
    room B = [a, a + b] along x, both [0, d] along y, with a, b, d U[6, 10] m;
    the wall between them has a 1.2 m wide, 2.1 m tall door gap centred at
    y_door U[1.5, d - 1.5]; 4 to 10 floor-standing boxes per room (footprint
    U[0.2, 1.5]^2, height U[0.3, 2.0], one quad per face), kept clear of the
    door.  Materials as shoebox_scene.  Returns tris, mat, mat_prop and a
    dict of the geometry (a, b, d, y_door, box bounds)."""
    rng = np.random.Generator(np.random.PCG64(5000 + seed))
    a, b, d = (float(x) for x in rng.uniform(6.0, 10.0, 3))
    y_door = float(rng.uniform(1.5, d - 1.5))
    X, Z = a + b, height
    tris, mats = [], []
    props = [rng.uniform(0.3, 0.7) for _ in range(3)]
    ex, ey, ez = np.array([X, 0, 0.0]), np.array([0, d, 0.0]), np.array([0, 0, Z])
    floor = _quad_grid(np.zeros(3), ex, ey, 2, 2)
    ceil = _quad_grid(ez, ex, ey, 2, 2)
    walls = (_quad_grid(np.zeros(3), ex, ez, 2, 1) + _quad_grid(ey, ex, ez, 2, 1)
             + _quad_grid(np.zeros(3), ey, ez, 1, 1) + _quad_grid(ex, ey, ez, 1, 1))
    # the wall between the rooms, with the door gap
    y0, y1 = y_door - 0.6, y_door + 0.6
    p = np.array([a, 0.0, 0.0])
    walls += _quad_grid(p, np.array([0, y0, 0.0]), ez, 1, 1)
    walls += _quad_grid(p + np.array([0, y1, 0.0]), np.array([0, d - y1, 0.0]), ez, 1, 1)
    walls += _quad_grid(p + np.array([0, y0, 2.1]), np.array([0, y1 - y0, 0.0]),
                        np.array([0, 0, Z - 2.1]), 1, 1)
    for group, m in ((floor, 0), (ceil, 1), (walls, 2)):
        tris += group
        mats += [m] * len(group)
    boxes = []
    for x0, x1 in ((0.0, a), (a, X)):
        for _ in range(int(rng.integers(4, 11))):
            while True:
                sx, sy = rng.uniform(0.2, 1.5, size=2)
                h = rng.uniform(0.3, 2.0)
                cx, cy = rng.uniform(x0 + 0.3, x1 - 0.3), rng.uniform(0.3, d - 0.3)
                lo = np.array([max(cx - sx / 2, x0 + 0.05), max(cy - sy / 2, 0.05), 0.0])
                hi = np.array([min(cx + sx / 2, x1 - 0.05), min(cy + sy / 2, d - 0.05), h])
                near_door = (abs(cx - a) < 2.0 and abs(cy - y_door) < 2.0)
                if not near_door:
                    break
            bt = box_tris(lo, hi, 1)
            tris += bt
            mats += [len(props)] * len(bt)
            props.append(rng.uniform(0.3, 0.7))
            boxes.append((lo, hi))
    tris = np.asarray(tris, np.float32)
    mat = np.asarray(mats, np.int32)
    mat_prop = np.repeat(np.asarray(props, np.float32)[:, None], 19, axis=1)
    return tris, mat, mat_prop, dict(a=a, b=b, d=d, y_door=y_door, door_half=0.6, boxes=boxes)


def batch_config(n_place=64, seed=0, target_tris=200_000, n_rx=256, launch=1000):
    """Batched hyper-configs: a multi-room building (multiroom_scene), a
    16-element AP in the middle room at 2.5 m facing +y, an n_rx x n_rx Rx
    grid over the footprint at 1.5 m, and n_place metasurfaces of n x n
    elements (n uniform over 16, 24, ..., 64) at lambda/2 on seeded positions
    of the four walls of the AP's room, facing into the room 1 mm off the
    wall (where the AP illuminates them, as the reference's trial places its
    metasurface on a wall the AP sees, physical_exp_nni_model.py:29-73)."""
    rng = np.random.Generator(np.random.PCG64(1000 + seed))
    tris, mat, mat_prop, xs, ys = multiroom_scene(target_tris, seed=seed)
    X, Y = xs[-1], ys[-1]
    lam = WAVE_LEN_60GHZ
    ci, cj = (len(xs) - 1) // 2, (len(ys) - 1) // 2
    ap = ((xs[ci] + xs[ci + 1]) / 2, (ys[cj] + ys[cj + 1]) / 2, 2.5)
    src = ula(ap, (1, 0, 0), 16, lam / 2)
    dst = rx_grid(0.25, X - 0.25, n_rx, 0.25, Y - 0.25, n_rx, 1.5)
    x0, x1, y0, y1 = xs[ci], xs[ci + 1], ys[cj], ys[cj + 1]
    walls = [((x0, y0), (1.0, 0.0), (0.0, 1.0), x1 - x0),    # y = y0, normal +y
             ((x0, y1), (1.0, 0.0), (0.0, -1.0), x1 - x0),   # y = y1, normal -y
             ((x0, y0), (0.0, 1.0), (1.0, 0.0), y1 - y0),    # x = x0, normal +x
             ((x1, y0), (0.0, 1.0), (-1.0, 0.0), y1 - y0)]   # x = x1, normal -x
    place = []
    for _ in range(n_place):
        w = int(rng.integers(0, 4))
        (ox, oy), (ux, uy), (nx, ny), L = walls[w]
        n = int(rng.choice(np.arange(16, 65, 8)))
        t = float(rng.uniform(1.0, L - 1.0))
        z = float(rng.uniform(1.0, 2.0))
        c = (ox + ux * t + nx * 1e-3, oy + uy * t + ny * 1e-3, z)
        pos, quad, k = metasurface(c, (nx, ny, 0.0), (0.0, 0.0, -1.0), n, lam / 2)
        place.append(dict(wall=w, size=n, pos=pos, blackhole=quad, normal=k))

    def prm(sbp, dbp, sdir, ddir):
        return dict(samples_per_launch=1, launch_x=launch, launch_y=launch, wave_len=lam,
                    max_reflection=2, reserve_size=100, src_bptype=sbp, dst_bptype=dbp,
                    dst_gridsize=5, src_r=0.5e-5, dst_r=0.06, src_dir=list(map(float, sdir)),
                    dst_dir=list(map(float, ddir)))
    return dict(tris=tris, mat=mat, mat_prop=mat_prop, src=src, dst=dst, placements=place,
                prm=prm, ap_dir=(0.0, 1.0, 0.0))


# ----------------------------------------------------------- STL scenes
def read_stl(path):
    """Binary STL triangles as float32 [N, 3, 3] (what numpy-stl's
    mesh.vectors gives, go.py:700-705)."""
    with open(path, "rb") as f:
        data = f.read()
    if len(data) < 84:
        raise ValueError(f"{path}: too short for binary STL")
    (n,) = struct.unpack_from("<I", data, 80)
    if 84 + 50 * n != len(data):
        raise ValueError(f"{path}: size does not match {n} triangles")
    rec = np.frombuffer(data, dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)),
                                              ("a", "<u2")]), count=n, offset=84)
    return np.ascontiguousarray(rec["v"], dtype=np.float32)


def read_mat(path):
    names, props = [], []
    with open(path) as f:
        for line in f:
            vals = line.split()
            if not vals:
                continue
            names.append(vals[0])
            props.append([float(x) for x in vals[1:]])
    return names, np.asarray(props, np.float32)


def load_scene_folder(folder, blackhole_buffer=(), reflector_buffer=(), door_buffer=()):
    """Scene ingest of build_channel (go.py:679-737): every *.stl in the
    folder (material from the file-name suffix), then pseudo-materials
    blackhole (0), reflector (1) and door (-0.7) for the extra quads."""
    names, props = read_mat(os.path.join(folder, "mat.txt"))
    props = [list(p) for p in props]
    tris, mats = [], []
    for fn in os.listdir(folder):  # os.listdir order, as the reference
        if not fn.endswith(".stl"):
            continue
        v = read_stl(os.path.join(folder, fn))
        mat_name = fn.split("_")[-1].split(".stl")[0]
        mid = names.index(mat_name)
        tris.append(v)
        mats.append(np.full(v.shape[0], mid, np.int32))
    for buf, val, label in ((blackhole_buffer, 0.0, "blackhole"),
                            (reflector_buffer, 1.0, "reflector"),
                            (door_buffer, -0.7, "door")):
        if len(buf) > 0:
            props.append([val] * 19)
            t = np.asarray([tri for quad in buf for tri in quad], np.float32).reshape(-1, 3, 3)
            tris.append(t)
            mats.append(np.full(t.shape[0], len(names), np.int32))
            names.append(label)
    tris = np.concatenate(tris, 0) if tris else np.zeros((0, 3, 3), np.float32)
    mat = np.concatenate(mats, 0) if mats else np.zeros((0,), np.int32)
    return tris.astype(np.float32), mat, np.asarray(props, np.float32)
