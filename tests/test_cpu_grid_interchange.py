"""Grid checkpoints move between the reference and this project (vflow.py:271-347).

``tests/golden/reference_grid.json`` was written by the reference's own
``save_grid`` (its 4-D grid after the ``vegas4`` run of the golden fixtures);
``tests/golden/repo_grid.json`` was written by this project's ``save_grid`` and
read by the reference's ``load_grid`` when the fixtures were generated, which
stored the grid it loaded.  Both directions must be exact."""

import json
import os

import numpy as np

from vegasflow_gb300 import VegasFlow

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_load_grid_written_by_the_reference(golden):
    inst = VegasFlow(4, 1000, verbose=False, device="cpu")
    inst.load_grid(file_name=os.path.join(HERE, "reference_grid.json"))
    np.testing.assert_array_equal(inst.divisions.numpy(), golden["vegas4/grids"][-1])


def test_reference_loads_a_grid_written_here(golden, tmp_path):
    want = golden["interchange/repo_grid"]
    np.testing.assert_array_equal(golden["interchange/ref_loaded_repo_grid"], want)
    # this project still writes that file the same way
    inst = VegasFlow(3, 1000, verbose=False, device="cpu")
    inst.load_grid(numpy_grid=want)
    out = tmp_path / "grid.json"
    inst.save_grid(str(out))
    with open(out) as fh, open(os.path.join(HERE, "repo_grid.json")) as ref:
        assert json.load(fh) == json.load(ref)


def test_reference_file_keys_and_shape():
    with open(os.path.join(HERE, "reference_grid.json")) as fh:
        d = json.load(fh)
    assert set(d) == {"dimensions", "ALPHA", "BINS", "integrand", "grid"}
    assert d["dimensions"] == 4 and d["BINS"] == 51 and d["ALPHA"] == 1.5
    assert np.array(d["grid"]).shape == (4, 51)
