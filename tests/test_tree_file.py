"""Content-keyed tree files (the replacement for the reference's fixed-name
./kdtree.cache, main.cpp:142-167): round trips, zero-copy mapping, and every
way a stale or damaged file is refused."""
import numpy as np
import pytest

import turner_gb300 as tg


@pytest.fixture(scope="module")
def mesh():
    return tg.make_scene(tg.SCENE_SPHERE_ROOM, detail=3)


def export(tree):
    return tree.export()


def same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


def test_save_load_round_trip(mesh, tmp_path):
    t = tg.KDTree.from_mesh(mesh)
    key = tg.mesh_key(mesh.vertices, mesh.normals, mesh.diffuse)
    t.save(tmp_path / "a.tkd", key)
    u = tg.KDTree.load(tmp_path / "a.tkd", key)
    assert same(export(t), export(u))
    assert u.height() == t.height()
    assert same(export(t), export(tg.KDTree.load(tmp_path / "a.tkd")))   # key 0: any


def test_cache_dir_builds_then_loads(mesh, tmp_path):
    a = tg.KDTree.from_mesh(mesh, cache_dir=tmp_path / "cache")
    b = tg.KDTree.from_mesh(mesh, cache_dir=tmp_path / "cache")
    assert not a.from_cache and b.from_cache
    assert same(export(a), export(b))
    files = list((tmp_path / "cache").iterdir())
    key = tg.mesh_key(mesh.vertices, mesh.normals, mesh.diffuse)
    assert [f.name for f in files] == [f"{key:016x}.tkd"]


def test_key_follows_content(mesh):
    k = tg.mesh_key(mesh.vertices, mesh.normals, mesh.diffuse)
    v = mesh.vertices.copy()
    v[5, 1] = np.nextafter(v[5, 1], np.float32(10))
    assert tg.mesh_key(v, mesh.normals, mesh.diffuse) != k
    d = mesh.diffuse.copy()
    d[0, 0] += 0.5
    assert tg.mesh_key(mesh.vertices, mesh.normals, d) != k
    assert tg.mesh_key(mesh.vertices, None, mesh.diffuse) != k
    assert tg.mesh_key(mesh.vertices, mesh.normals, mesh.diffuse) == k


def test_stale_cache_is_rebuilt(mesh, tmp_path):
    """A file of another scene under this scene's name is refused (key check)
    and replaced: the reference's fixed-name cache would render the old scene."""
    other = tg.make_scene(tg.SCENE_ROOM)
    key = tg.mesh_key(mesh.vertices, mesh.normals, mesh.diffuse)
    (tmp_path / "c").mkdir()
    tg.KDTree.from_mesh(other).save(tmp_path / "c" / f"{key:016x}.tkd",
                                    tg.mesh_key(other.vertices, other.normals, other.diffuse))
    t = tg.KDTree.from_mesh(mesh, cache_dir=tmp_path / "c")
    assert not t.from_cache
    assert same(export(t), export(tg.KDTree.from_mesh(mesh)))
    assert tg.KDTree.from_mesh(mesh, cache_dir=tmp_path / "c").from_cache


def test_mapped_file_is_zero_copy_and_equal(mesh, tmp_path):
    t = tg.KDTree.from_mesh(mesh)
    key = tg.mesh_key(mesh.vertices, mesh.normals, mesh.diffuse)
    t.save(tmp_path / "m.tkd", key)
    f = tg.TreeFile(tmp_path / "m.tkd", key)
    nodes, tris, box = export(t)
    assert f.key == key
    assert np.array_equal(f.nodes, nodes) and np.array_equal(f.triangles.view(np.uint32), tris.view(np.uint32))
    assert np.array_equal(f.box, box)
    assert not f.nodes.flags.owndata
    st, depth = tg.validate_nodes(f.nodes, f.triangles.shape[0])
    assert st == 0 and depth >= t.height()
    f.close()


@pytest.mark.parametrize("damage", ["truncate", "magic", "payload", "key", "missing"])
def test_damaged_files_are_refused(mesh, tmp_path, damage):
    t = tg.KDTree.from_mesh(mesh)
    key = tg.mesh_key(mesh.vertices, mesh.normals, mesh.diffuse)
    p = tmp_path / "d.tkd"
    t.save(p, key)
    raw = bytearray(p.read_bytes())
    want_key = key
    if damage == "truncate":
        raw = raw[:-7]
    elif damage == "magic":
        raw[0] ^= 0xFF
    elif damage == "payload":
        raw[128 + 8 * 3 + 2] ^= 0x10
    elif damage == "key":
        want_key = key ^ 1
    if damage == "missing":
        p = tmp_path / "nothing.tkd"
    else:
        p.write_bytes(bytes(raw))
    with pytest.raises(tg.TurnerError) as e:
        tg.KDTree.load(p, want_key)
    assert e.value.status in (tg.ERR_BAD_SCENE, tg.ERR_INVALID_ARG)
    if damage == "payload":   # mapping without verification still opens it
        f = tg.TreeFile(p, key, verify=False)
        f.close()
