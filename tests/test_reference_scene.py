"""Scene ingest of build_channel on the reference's own scene folder
(stl/4321): the package's reader against what the reference's ingest
(go.py:679-737, numpy-stl replaced by a struct reader) built for every
trace of a channel set."""
import hashlib
import os

import numpy as np
import pytest

import refscene


@pytest.fixture(scope="module")
def fx():
    return refscene.load()


def _sha(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def test_restated_ingest_matches_reference_ingest(fx):
    """The restatement used below equals the reference's ingest byte for byte
    on every trace of the channel set (file order of the fixture)."""
    order = [str(n) for n in fx["stl_names"]]
    t, m, p = refscene.expected_ingest(fx, order, *refscene.trace_buffers(fx, "src_to_dst"))
    assert np.array_equal(t.reshape(-1, 3), fx["scene0_buffer"])
    assert np.array_equal(m, fx["scene0_mat"]) and np.array_equal(p, fx["scene0_mat_prop"])
    for key in fx["keys"]:
        tag = str(key).replace("{", "").replace("}", "")
        t, m, p = refscene.expected_ingest(fx, order, *refscene.trace_buffers(fx, str(key)))
        assert _sha(t.reshape(-1, 3), m, p) == str(fx[f"{tag}_ingest_sha"]), key
        assert len(t) == int(fx[f"{tag}_n_tri"])


def test_load_scene_folder_on_reference_scene(fx, tmp_path):
    """scenes.load_scene_folder on the rebuilt folder gives the reference's
    ingest for the folder's own listdir order, for every trace."""
    from automs_gb300 import scenes
    refscene.write_folder(fx, str(tmp_path))
    order = os.listdir(str(tmp_path))
    for key in fx["keys"]:
        bufs = refscene.trace_buffers(fx, str(key))
        t, m, p = scenes.load_scene_folder(str(tmp_path), *bufs)
        te, me, pe = refscene.expected_ingest(fx, order, *bufs)
        assert t.dtype == np.float32 and m.dtype == np.int32 and p.dtype == np.float32
        assert np.array_equal(t, te) and np.array_equal(m, me) and np.array_equal(p, pe), key


def test_walls_of_reference_scene(fx, tmp_path):
    """get_walls on the rebuilt folder reads the reference's wall.txt."""
    from automs_gb300 import geometry
    refscene.write_folder(fx, str(tmp_path))
    walls = geometry.get_walls(str(tmp_path))
    assert len(walls) == 3 and all(len(w) == 3 for w in walls)
