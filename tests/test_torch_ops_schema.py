"""The PyTorch form registers its operators without a GPU (their schemas are plain tensors)."""
import importlib

import torch


def test_ops_are_registered():
    ops = importlib.import_module("2dense_gb300.torch_ops")
    for name in ("steps", "rhs", "stage", "batched_steps"):
        assert hasattr(torch.ops.dense2d, name)
    dense = importlib.import_module("2dense_gb300")
    c = dense.default_config(ni=40, nj=32)
    t = ops.config_tensor(c)
    assert t.dtype == torch.uint8 and t.numel() == 232
    assert ops._config(t).ni == 40 and ops._config(t).nj == 32
