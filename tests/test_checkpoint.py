"""Trainer checkpoints on the CPU: atomic replacement (a failed save leaves the previous checkpoint
intact), round trip of the saved state, and the SIGTERM flag the training loop polls to save and
return (scripts/train_scatter_field.py:132-134, :165-168)."""
import os
import signal

import numpy as np
import pytest
import torch

from augur_gb300 import learned


def test_checkpoint_round_trip_and_atomic_replace(tmp_path):
    path = str(tmp_path / "run.ckpt")
    assert learned.load_checkpoint(path) is None
    rng = np.random.default_rng(3)
    rng.random(5)
    state = {"net": {"params": torch.arange(6.0), "step": 7}, "rng": rng.bit_generator.state, "hist": [{"step": 1}],
             "skipped": 0, "it": 7}
    learned.save_checkpoint(path, state)
    assert not os.path.exists(path + ".tmp")
    back = learned.load_checkpoint(path)
    assert torch.equal(back["net"]["params"], state["net"]["params"]) and back["it"] == 7
    r2 = np.random.default_rng(0)
    r2.bit_generator.state = back["rng"]
    assert np.array_equal(r2.random(4), rng.random(4))  # the batch sampler resumes where it was

    real_save = torch.save

    def failing_save(obj, f):
        with open(f, "wb") as fh:
            fh.write(b"partial")
        raise OSError("disk full")

    torch.save = failing_save
    try:
        with pytest.raises(OSError):
            learned.save_checkpoint(path, {"it": 8})
    finally:
        torch.save = real_save
    assert learned.load_checkpoint(path)["it"] == 7


def test_sigterm_sets_the_stop_flag_and_restores_the_handler():
    before = signal.getsignal(signal.SIGTERM)
    with learned._StopFlag() as stop:
        assert not stop.set
        os.kill(os.getpid(), signal.SIGTERM)
        assert stop.set
    assert signal.getsignal(signal.SIGTERM) == before
