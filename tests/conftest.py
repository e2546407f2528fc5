"""Shared pytest configuration: the ``gpu`` marker and helpers."""

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


def raw_blocks(golden, name):
    """The raw U[0,1) blocks the reference consumed for case ``name``, in order."""
    flat = golden[f"{name}/raw"]
    shapes = golden[f"{name}/raw_shapes"]
    out, pos = [], 0
    for shp in shapes:
        n = int(np.prod(shp))
        out.append(flat[pos:pos + n].reshape(tuple(int(s) for s in shp)))
        pos += n
    return out


def replay_source(blocks, affine):
    """A uniform source handing out the recorded blocks in order (post-affine)."""
    it = iter(blocks)

    def source(n, n_dim):
        blk = next(it)
        assert blk.shape == (n, n_dim), (blk.shape, n, n_dim)
        return affine(blk)

    return source
