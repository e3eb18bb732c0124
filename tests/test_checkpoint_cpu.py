"""Checkpoint loading as the reference's train_utils.load_checkpoint does it: weights-only, then weights-only with
numpy's reconstruction types allowed, and a full unpickle only with a warning."""
import warnings

import numpy as np
import pytest
import torch

from ffnoml_gb300.runtime import load_checkpoint


class _Custom:
    def __init__(self, v):
        self.v = v


def test_plain_tensor_checkpoint_loads_weights_only(tmp_path):
    p = tmp_path / "a.pt"
    torch.save({"model_state": {"w": torch.arange(4.0)}}, p)
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        ck = load_checkpoint(p)
    assert torch.equal(ck["model_state"]["w"], torch.arange(4.0))


def test_numpy_statistics_load_without_a_full_unpickle(tmp_path):
    p = tmp_path / "b.pt"
    stats = {"mean_X": np.arange(6, dtype=np.float32), "std_X": np.float64(2.5)}
    torch.save({"model_state": {}, "normalization_stats": stats}, p)
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        ck = load_checkpoint(p)
    assert np.array_equal(ck["normalization_stats"]["mean_X"], stats["mean_X"])
    assert float(ck["normalization_stats"]["std_X"]) == 2.5


def test_arbitrary_objects_need_a_full_unpickle_and_warn(tmp_path):
    p = tmp_path / "c.pt"
    torch.save({"model_state": {}, "extra": _Custom(3)}, p)
    with pytest.warns(RuntimeWarning, match="trusted"):
        ck = load_checkpoint(p)
    assert ck["extra"].v == 3
