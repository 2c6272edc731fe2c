"""The branching estimator (-m M > 1, pathtracer.cpp:72-88) on the oracle.

Children of a hit draw from per-branch streams (a stream per ray, derived
from its parent's state), where the reference draws them depth-first from one
generator. So the contract is statistical against the reference: the same
expectation. Tested as a paired z-test over pixels: the mean per-pixel
difference of two independent renders, in units of its standard error."""
import numpy as np
import pytest

import turner_gb300 as tg
from oracle import oracle as orc


def zscore(a, b):
    d = (a[..., :3] - b[..., :3]).astype(np.float64).reshape(-1)
    return abs(d.mean()) / (d.std(ddof=1) / np.sqrt(d.size))


@pytest.fixture(scope="module")
def room():
    m = tg.make_scene(tg.SCENE_ROOM)
    nodes, tris, box = tg.KDTree.from_mesh(m).export()
    return m, orc.Scene(nodes, tris, box)


def render(m, sc, mc, seed, spp=48, depth=2, sampling=0):
    img, st = sc.render(m.camera, m.light, 24, 24, spp, depth, mc=mc, seed=seed, tone_map=False, sampling=sampling)
    return img, st


def test_branching_matches_single_branch_expectation(room):
    m, sc = room
    a, sa = render(m, sc, 2, 11)
    b, sb = render(m, sc, 1, 12, spp=96)
    assert zscore(a, b) < 4.0
    # a path of depth 2 has up to 1 + 2 + 4 traced rays
    assert int(sa[0]) > 1.5 * int(sb[0]) / 2


def test_branch_streams_are_independent_of_order(room):
    """Same seed, same image: every child's stream is a function of its
    parent's, not of the order rays are traced in."""
    m, sc = room
    a, _ = render(m, sc, 3, 5, spp=4)
    b, _ = render(m, sc, 3, 5, spp=4)
    assert np.array_equal(a, b)
    c, _ = render(m, sc, 3, 6, spp=4)
    assert not np.array_equal(a, c)


@pytest.mark.skipif(not orc.ref_available(), reason="reference sources not present")
def test_branching_matches_the_reference_statistically(room):
    m, sc = room
    ref_tree = orc.RefTree(m.vertices, m.normals, m.diffuse)
    cam = m.camera
    rimg, _ = ref_tree.render(list(cam.position), list(cam.trafo), m.hfov, cam.aspect, m.light, 24, 24, 48, 2,
                              mc=2, seed=21, exposure=1.0, gamma=False)
    img, _ = sc.render(m.camera, m.light, 24, 24, 48, 2, mc=2, seed=22, gamma=False)
    assert zscore(img, rimg) < 4.0
