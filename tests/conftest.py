import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(REPO, "msc-project_gb300"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def built():
    """Builds (or reuses) the CUDA library and the CPU oracle."""
    import __graft_entry__ as g
    g.build()
    import mscgpu
    from oracle import oracle
    return mscgpu, oracle


@pytest.fixture(scope="session")
def scene_dir(tmp_path_factory):
    return tmp_path_factory.mktemp("scenes")


@pytest.fixture(scope="session")
def tiny_scene(built, scene_dir):
    mscgpu, _ = built
    return mscgpu.generate_scene(100, 1234, str(scene_dir / "tiny"))


@pytest.fixture(scope="session")
def box_scene(built, scene_dir):
    """The Cornell-style box at a reduced resolution (64x64, 16 spp)."""
    mscgpu, _ = built
    return mscgpu.generate_scene(0, 20261203, str(scene_dir / "box64"), scale=0.25)
