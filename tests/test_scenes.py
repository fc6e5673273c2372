"""Workload generators: sizes, materials and placements (CPU only)."""
import numpy as np

from automs_gb300 import scenes


def test_multiroom_scene_size_and_materials():
    tris, mat, mat_prop, xs, ys = scenes.multiroom_scene(200_000, seed=0)
    assert abs(tris.shape[0] - 200_000) < 300
    assert tris.dtype == np.float32 and mat.dtype == np.int32
    assert mat.min() >= 0 and mat.max() < mat_prop.shape[0]
    assert np.all((mat_prop > 0.29) & (mat_prop < 0.71))
    assert len(xs) == 4 and len(ys) == 4 and np.all(np.diff(xs) >= 6) and np.all(np.diff(xs) <= 15)
    lo, hi = tris.reshape(-1, 3).min(0), tris.reshape(-1, 3).max(0)
    assert np.allclose(lo, 0, atol=1e-4) and abs(hi[2] - 3.0) < 1e-4


def test_batch_config_placements():
    c = scenes.batch_config(n_place=64, target_tris=20_000)
    sizes = [p["size"] for p in c["placements"]]
    assert len(sizes) == 64 and set(sizes) <= set(range(16, 65, 8))
    for p in c["placements"][:8]:
        n = p["size"]
        assert p["pos"].shape == (n, n, 3)
        assert abs(np.linalg.norm(p["normal"]) - 1) < 1e-6
        assert p["blackhole"].shape == (2, 3, 3)
    assert c["dst"].shape == (256, 256, 3) and c["src"].shape == (1, 16, 3)


def test_channel_ms_config_sizes():
    c = scenes.channel_ms_config("ms-256")
    assert c["tris"].shape[0] == 50_028
    assert c["ms"].shape == (32, 32, 3) and c["dst"].shape == (256, 256, 3)
    assert set(c["traces"]) == {"src_to_dst", "src_to_ms{0}", "ms{0}_to_dst"}


def _stl_bytes(tris, count=None):
    import struct
    tris = np.asarray(tris, np.float32).reshape(-1, 3, 3)
    out = bytearray(b"synthetic".ljust(80, b" "))
    out += struct.pack("<I", len(tris) if count is None else count)
    for t in tris:
        out += struct.pack("<3f", 0.0, 0.0, 1.0) + t.tobytes() + struct.pack("<H", 0)
    return bytes(out)


def test_read_stl_valid_and_corrupted(tmp_path):
    import pytest
    rng = np.random.Generator(np.random.PCG64(0))
    tris = rng.uniform(-1, 1, size=(5, 3, 3)).astype(np.float32)
    p = tmp_path / "ok.stl"
    p.write_bytes(_stl_bytes(tris))
    assert np.array_equal(scenes.read_stl(str(p)), tris)
    p.write_bytes(_stl_bytes(np.zeros((0, 3, 3))))
    assert scenes.read_stl(str(p)).shape == (0, 3, 3)
    for name, data in (("empty", b""), ("short_header", b"x" * 50),
                       ("truncated", _stl_bytes(tris)[:-7]),
                       ("count_mismatch", _stl_bytes(tris, count=9))):
        q = tmp_path / f"{name}.stl"
        q.write_bytes(data)
        with pytest.raises(ValueError):
            scenes.read_stl(str(q))
