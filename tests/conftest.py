import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU")
    config.addinivalue_line("markers", "slow: takes more than a few seconds on the CPU")


@pytest.fixture(scope="session", autouse=True)
def _native_build():
    """Builds the native libraries once per session if they are missing."""
    from turner_gb300 import LIB_PATH

    from oracle import oracle as orc

    if not LIB_PATH.exists() or not orc.ORACLE_SO.exists():
        from turner_gb300 import build

        build.build()
    yield


def pytest_collection_modifyitems(config, items):
    # GPU tests are skipped cleanly when no CUDA device is visible
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def sphere_room_327k():
    """The large-mesh workload's scene: the 327,692-triangle displaced sphere
    room (icosphere subdivided 7 times), its host kd-tree (the reference
    builder's node words) and the oracle on that tree. Built once per session."""
    import turner_gb300 as tg

    from oracle import oracle as orc

    mesh = tg.make_scene(tg.SCENE_SPHERE_ROOM, detail=7, aspect=16 / 9)
    nodes, tris, box = tg.KDTree.from_mesh(mesh).export()
    return mesh, nodes, tris, box, orc.Scene(nodes, tris, box)
