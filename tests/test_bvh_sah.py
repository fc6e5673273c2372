"""Binned-SAH scene hierarchy (automs_gb300/csrc/bvh_sah.cpp), checked on the
host: tree structure, widened boxes containing their subtrees, depth within
the kernels' traversal stack, and closest hits equal to brute force over
random and axis-parallel rays (tests/bvh_sah_check.cpp, built with g++)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from automs_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "automs_gb300", "csrc")
CUDA_INC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    if shutil.which("g++") is None or not os.path.isdir(CUDA_INC):
        pytest.skip("g++ or the CUDA headers are missing")
    out = str(tmp_path_factory.mktemp("sah") / "bvh_sah_check")
    cmd = ["g++", "-O2", "-std=c++17", "-I", CSRC, "-I", CUDA_INC,
           os.path.join(ROOT, "tests", "bvh_sah_check.cpp"), os.path.join(CSRC, "bvh_sah.cpp"),
           "-o", out, "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def run(checker, tmp_path, tris, n_rays=2000, seed=1):
    p = tmp_path / "tris.bin"
    np.ascontiguousarray(tris, dtype=np.float32).tofile(p)
    r = subprocess.run([checker, str(p), str(n_rays), str(seed)], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
    return [int(x) for x in r.stdout.split()[1:]]


def test_room_with_obstacles(checker, tmp_path):
    c = scenes.channel_ms_config("ms-256")
    nodes, depth = run(checker, tmp_path, c["tris"], n_rays=3000)
    assert nodes == c["tris"].shape[0] - 1 and depth <= 62


def test_multiroom_building(checker, tmp_path):
    tris, *_ = scenes.multiroom_scene(40_000, seed=3)
    nodes, depth = run(checker, tmp_path, tris, n_rays=1500, seed=2)
    assert nodes == tris.shape[0] - 1 and depth <= 62


def test_degenerate_inputs(checker, tmp_path):
    rng = np.random.Generator(np.random.PCG64(0))
    one = rng.uniform(0, 1, size=(1, 9))
    run(checker, tmp_path, one, n_rays=50)
    two = rng.uniform(0, 1, size=(2, 9))
    run(checker, tmp_path, two, n_rays=50)
    # identical triangles: every centroid equal, splits fall back to index order
    same = np.repeat(rng.uniform(0, 1, size=(1, 9)), 3000, axis=0)
    nodes, depth = run(checker, tmp_path, same, n_rays=50)
    assert nodes == 2999 and depth <= 62
    # a thin sheet of coplanar triangles (zero extent on one axis)
    g = np.stack(np.meshgrid(np.arange(60.0), np.arange(60.0), indexing="ij"), -1).reshape(-1, 2)
    sheet = np.concatenate([g, np.zeros((len(g), 1)), g + [1, 0], np.zeros((len(g), 1)),
                            g + [0, 1], np.zeros((len(g), 1))], axis=1)
    run(checker, tmp_path, sheet, n_rays=500)
