"""Array and placement geometry with the signatures of the reference's
go.py helpers (go.py:17-24, 248-293, 339-511, 533-620, 1309-1338).

The reference creates its tensors on "cuda" unconditionally; these take a
`device` keyword (default "cuda") and otherwise compute the same values.
"""
import copy
import math
import os
from typing import Literal, Tuple

import torch
import torch.nn.functional as F


class Metasurface:
    """go.py:17-24; max_phase is given in degrees and stored in radians."""

    def __init__(self, pos, size, send_dir, recv_dir, blackhole, max_phase):
        self.pos = pos
        self.size = size
        self.send_dir = send_dir
        self.recv_dir = recv_dir
        self.blackhole = blackhole
        self.max_phase = max_phase / 180 * math.pi


def _t(x, device):
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=torch.float32)
    return torch.tensor(x, dtype=torch.float32, device=device)


def gen_direction_from_angle(theta: float, phi: float, up, polar_axis,
                             unit: Literal["deg", "rad"] = "deg", device="cuda") -> torch.Tensor:
    """go.py:248-293"""
    if unit == "deg":
        theta = theta / 180 * math.pi
        phi = phi / 180 * math.pi
    up = _t(up, device)
    polar_axis = _t(polar_axis, device)
    i_dir = F.normalize(polar_axis, dim=-1)
    j_dir = F.normalize(torch.cross(up, i_dir, dim=-1), dim=-1)
    k_dir = torch.cross(i_dir, j_dir, dim=-1)
    ijk = torch.tensor([math.cos(theta) * math.cos(phi), math.cos(theta) * math.sin(phi),
                        math.sin(theta)], dtype=torch.float32, device=device)
    return ijk @ torch.stack([i_dir, j_dir, k_dir], dim=0)


def gen_pos_matrix(center, k_direction, i_direction, size: Tuple[int, int], spacing: float,
                   device="cuda") -> torch.Tensor:
    """go.py:339-385: element positions [size_i, size_j, 3]."""
    size_i, size_j = size
    center = _t(center, device)
    i_direction = _t(i_direction, device)
    k_direction = _t(k_direction, device)
    j_direction = torch.cross(k_direction, i_direction, dim=-1)
    i_direction = F.normalize(i_direction, dim=-1)
    j_direction = F.normalize(j_direction, dim=-1)
    k_direction = F.normalize(k_direction, dim=-1)
    pos_i = torch.linspace(-(size_i - 1) / 2, (size_i - 1) / 2, size_i, device=device)
    pos_j = torch.linspace(-(size_j - 1) / 2, (size_j - 1) / 2, size_j, device=device)
    pos_i, pos_j = torch.meshgrid([pos_i, pos_j], indexing="ij")
    pos_ijk = torch.stack([pos_i.flatten(), pos_j.flatten(),
                           torch.zeros(size_i * size_j, dtype=torch.float32, device=device)], -1)
    transform = torch.stack([i_direction, j_direction, k_direction], dim=0)
    pos = ((pos_ijk * spacing) @ transform) + center
    return pos.reshape(tuple(size) + (3,))


def gen_ms(center, k_direction, i_direction, size: Tuple[int, int], spacing: float,
           thickness: float = 0.001, device="cuda"):
    """go.py:388-443: positions, blackhole quad (2 triangles), normal."""
    size_i, size_j = size
    center = _t(center, device).clone()
    i_direction = _t(i_direction, device)
    k_direction = _t(k_direction, device)
    j_direction = torch.cross(k_direction, i_direction, dim=-1)
    i_direction = F.normalize(i_direction, dim=-1)
    j_direction = F.normalize(j_direction, dim=-1)
    k_direction = F.normalize(k_direction, dim=-1)
    center += k_direction * thickness
    pos = gen_pos_matrix(center, k_direction, i_direction, size, spacing, device=device)
    i_off = i_direction * size_i / 2 * spacing
    j_off = j_direction * size_j / 2 * spacing
    ul = (center - i_off - j_off).tolist()
    dr = (center + i_off + j_off).tolist()
    ur = (center + i_off - j_off).tolist()
    dl = (center - i_off + j_off).tolist()
    blackhole = [[ul, ur, dl], [dl, dr, ur]]
    return pos, blackhole, k_direction


def gen_sth_from_wall(wall, ij: Tuple[float, float], device="cuda"):
    """go.py:446-477: centre, normal and down direction on a wall."""
    up, left = ij
    v_ul, v_dl, v_dr = (_t(v, device) for v in wall)
    v_ur = v_ul + v_dr - v_dl
    v_up = (1 - left) * v_ul + left * v_ur
    v_down = (1 - left) * v_dl + left * v_dr
    v = up * v_down + (1 - up) * v_up
    i_dir = F.normalize(v_dl - v_ul, dim=-1)
    j_dir = F.normalize(v_dr - v_dl, dim=-1)
    k_dir = torch.cross(i_dir, j_dir, dim=-1)
    return v, k_dir, i_dir


def gen_pos_from_endpoint(x, y, z, device="cuda") -> torch.Tensor:
    """go.py:480-511: grid from [start, end, num] per axis (scalars fixed)."""
    pos_list, num_list = [], []
    for arg in (x, y, z):
        if not isinstance(arg, list):
            arg = [arg, arg, 1]
        start, end, num = arg
        num_list.append(num)
        pos_list.append(torch.linspace(start, end, num, dtype=torch.float32, device=device))
    num_list.remove(1)
    num_list += [-1]
    res = torch.meshgrid(pos_list, indexing="ij")
    return torch.stack(res, dim=-1).reshape(num_list)


def get_ap(scene_folder: str):
    """go.py:533-551"""
    with open(os.path.join(scene_folder, "ap.txt")) as f:
        lines = f.readlines()
    return [float(v) for v in lines[0].split()], [float(v) for v in lines[1].split()]


def get_doors(scene_folder: str, angle: float):
    """go.py:554-594: door quads rotated by `angle` (rad)."""
    doors = []
    with open(os.path.join(scene_folder, "door.txt")) as f:
        lines = f.readlines()
    for i in range(len(lines) // 4):
        tri = [[float(v) for v in lines[4 * i + j].split()] for j in range(3)]
        theta0 = math.atan2(tri[2][1] - tri[1][1], tri[2][0] - tri[1][0])
        theta = theta0 + angle * (1 - 2 * int(lines[4 * i + 3]))
        tri[2][0] = tri[1][0] + math.cos(theta)
        tri[2][1] = tri[1][1] + math.sin(theta)
        tri2 = copy.deepcopy(tri)
        tri2[1][2] = tri2[0][2]
        tri2[1][0] = tri2[2][0]
        tri2[1][1] = tri2[2][1]
        doors.append([tri, tri2])
    return doors


def get_walls(scene_folder: str):
    """go.py:597-620: candidate walls, 3 vertices each."""
    walls = []
    with open(os.path.join(scene_folder, "wall.txt")) as f:
        lines = f.readlines()
    for i in range(len(lines) // 4):
        walls.append([[float(v) for v in lines[4 * i + 1 + j].split()] for j in range(3)])
    return walls


def create_vertex_buffer(center, xlen: float = 0.2, ylen: float = 0.2, zlen: float = 1.5):
    """go.py:1309-1338: axis-aligned box as 12 triangles (nested lists)."""
    off = torch.tensor([
        [[-1, -1, 1], [1, -1, 1], [1, 1, 1]], [[-1, -1, 1], [-1, 1, 1], [1, 1, 1]],
        [[-1, -1, -1], [1, -1, -1], [1, 1, -1]], [[-1, -1, -1], [-1, 1, -1], [1, 1, -1]],
        [[-1, -1, -1], [-1, -1, 1], [-1, 1, 1]], [[-1, -1, -1], [-1, 1, -1], [-1, 1, 1]],
        [[1, -1, -1], [1, -1, 1], [1, 1, 1]], [[1, -1, -1], [1, 1, -1], [1, 1, 1]],
        [[-1, 1, -1], [1, 1, -1], [1, 1, 1]], [[-1, 1, -1], [-1, 1, 1], [1, 1, 1]],
        [[-1, -1, -1], [1, -1, -1], [1, -1, 1]], [[-1, -1, -1], [-1, -1, 1], [1, -1, 1]],
    ], dtype=torch.float32) / 2 * torch.tensor([xlen, ylen, zlen], dtype=torch.float32)
    return (off + torch.tensor(center, dtype=torch.float32)).numpy().tolist()
