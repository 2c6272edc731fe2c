"""The host kd-tree builder emits the reference's tree word for word."""
import hashlib
from pathlib import Path

import numpy as np
import pytest

import turner_gb300 as tg

GOLD = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def kd():
    return dict(np.load(GOLD / "ref_kdtree_tests.npz"))


@pytest.fixture(scope="module")
def scenes():
    return dict(np.load(GOLD / "ref_scenes.npz"))


FIXTURES = ["four", "cube", "overlap"] + [f"coplanar{a}" for a in range(3)] + [f"stacked{a}" for a in range(3)]


@pytest.mark.parametrize("name", FIXTURES)
def test_reference_test_trees(kd, name):
    """Trees of the reference's own kd-tree tests (tests/test_kdtree.cpp), exact."""
    t = tg.KDTree(kd[f"{name}_vertices"])
    nodes, tris, box = t.export()
    assert np.array_equal(nodes, kd[f"{name}_nodes"])
    assert np.array_equal(tris.view(np.uint32), kd[f"{name}_tris"].view(np.uint32))
    assert np.array_equal(box, kd[f"{name}_box"])
    if f"{name}_height" in kd:
        assert t.height() == int(kd[f"{name}_height"])


SCENES = {"room": dict(kind=tg.SCENE_ROOM), "sphere3": dict(kind=tg.SCENE_SPHERE_ROOM, detail=3),
          "soup2000": dict(kind=tg.SCENE_SOUP, count=2000, seed=7),
          "baffle8": dict(kind=tg.SCENE_BAFFLE_ROOM, detail=8), "mirror": dict(kind=tg.SCENE_MIRROR_ROOM)}


@pytest.mark.parametrize("name", list(SCENES))
@pytest.mark.parametrize("threads", [1, 0])
def test_scene_trees(scenes, name, threads):
    t = tg.KDTree.from_mesh(tg.make_scene(**SCENES[name]), threads=threads)
    nodes, tris, box = t.export()
    assert hashlib.sha256(nodes.tobytes()).hexdigest() == str(scenes[f"{name}_nodes_sha"])
    assert hashlib.sha256(tris.tobytes()).hexdigest() == str(scenes[f"{name}_tris_sha"])
    assert np.array_equal(box, scenes[f"{name}_box"])
    assert t.height() == int(scenes[f"{name}_height"])


@pytest.mark.slow
def test_full_size_sphere_tree(scenes):
    """327,692 triangles (icosphere level 7 in the room): 1,486,468 nodes,
    identical to the reference's tree."""
    t = tg.KDTree.from_mesh(tg.make_scene(tg.SCENE_SPHERE_ROOM, detail=7, aspect=16 / 9))
    nodes, tris, box = t.export()
    assert nodes.size == int(scenes["sphere7_num_nodes"])
    assert hashlib.sha256(nodes.tobytes()).hexdigest() == str(scenes["sphere7_nodes_sha"])
    assert hashlib.sha256(tris.tobytes()).hexdigest() == str(scenes["sphere7_tris_sha"])
    assert t.height() == int(scenes["sphere7_height"])


def test_validate_nodes_accepts_built_trees():
    t = tg.KDTree.from_mesh(tg.make_scene(tg.SCENE_SPHERE_ROOM, detail=4))
    nodes, tris, _ = t.export()
    st, depth = tg.validate_nodes(nodes, tris.shape[0])
    assert st == tg.OK and 0 < depth <= t.height()


def test_validate_nodes_rejects_corruption():
    """Corrupt node arrays are rejected on the host, before any device work."""
    t = tg.KDTree.from_mesh(tg.make_scene(tg.SCENE_SPHERE_ROOM, detail=3))
    nodes, tris, _ = t.export()
    n_tris = tris.shape[0]
    inner = np.nonzero((nodes & np.uint64(3)) != np.uint64(3))[0]
    leaves = np.nonzero((nodes & np.uint64(3)) == np.uint64(3))[0]
    bad = nodes.copy()
    bad[inner[0]] = (bad[inner[0]] & np.uint64(0xFFFFFFFF00000003)) | np.uint64((nodes.size + 5) << 2)  # right out of range
    assert tg.validate_nodes(bad, n_tris)[0] == tg.ERR_BAD_SCENE
    bad = nodes.copy()
    bad[inner[0]] = (bad[inner[0]] & np.uint64(0xFFFFFFFF00000003)) | np.uint64(0 << 2)  # backward link
    assert tg.validate_nodes(bad, n_tris)[0] == tg.ERR_BAD_SCENE
    bad = nodes.copy()
    bad[leaves[0]] = (np.uint64(n_tris + 7) << np.uint64(32)) | (bad[leaves[0]] & np.uint64(0xFFFFFFFF))  # bad id
    assert tg.validate_nodes(bad, n_tris)[0] == tg.ERR_BAD_SCENE
    # a full leaf as the last word: the leaf run would read past the array
    assert tg.validate_nodes(np.array([(np.uint64(0) << np.uint64(32)) | np.uint64((1 << 2) | 3)], np.uint64), 2)[0] \
        == tg.ERR_BAD_SCENE
    assert tg.validate_nodes(nodes[:1], n_tris)[0] == tg.ERR_BAD_SCENE


def test_builder_rejects_bad_input():
    with pytest.raises(tg.TurnerError):
        tg.KDTree(np.zeros((0, 9), np.float32))
