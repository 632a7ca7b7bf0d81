"""A checkpoint records the seed and a digest of the action list and
genetics; resuming it with other settings is refused before any device work
(the draws are keyed by the seed and the actions' windows, so the run would
otherwise continue differently from the one that was saved)."""
import numpy as np
import pytest

from qhg4_gb300 import checkpoint
from qhg4_gb300.spec import Genetics, config1_actions, spec_digest
from qhg4_gb300.workload import uniform_grid


def _fake_checkpoint(path, seed, acts, gen=Genetics()):
    z = np.zeros(1)
    np.savez(path, id=z.astype(np.int64), cell=z.astype(np.int32), birth=z.astype(np.float32),
             age=z.astype(np.float32), lastb=z.astype(np.float32), gender=z.astype(np.uint8),
             state=np.ones(1, np.uint8), step=np.array([3], np.int64), next_id=np.array([1], np.int64),
             seed=np.array([seed], np.uint64), spec=np.array(spec_digest(acts, gen)))


def test_resume_refuses_another_seed(tmp_path):
    path = str(tmp_path / "ck.npz")
    _fake_checkpoint(path, 7, config1_actions())
    with pytest.raises(ValueError, match="seed"):
        checkpoint.resume(uniform_grid(2, 30.0), config1_actions(), 8, path)


@pytest.mark.parametrize("change", ["parameter", "genetics"])
def test_resume_refuses_other_actions(tmp_path, change):
    path = str(tmp_path / "ck.npz")
    _fake_checkpoint(path, 7, config1_actions())
    acts, gen = config1_actions(), Genetics()
    if change == "parameter":
        acts = config1_actions(b0=0.21)
    else:
        gen = Genetics(64, 1, 1e-3)
    with pytest.raises(ValueError, match="other actions"):
        checkpoint.resume(uniform_grid(2, 30.0), acts, 7, path, gen)


def test_digest_follows_execution_order_not_list_order():
    acts = config1_actions()
    assert spec_digest(acts) == spec_digest(list(reversed(acts)))
    assert spec_digest(acts) != spec_digest(config1_actions(move_p=0.2))
