"""Launch autotuner of the batched form on a simulated batch (CPU): the
search keeps the fastest launch although the batch's cost per agent-step
drifts while it is tuned."""
from qhg4_gb300.batch import Autotuner


class DriftingBatch:
    """Stands in for GpuBatch: the time of a step depends on the launch
    (best at ``fast``) and on a cost that rises with every step taken, as
    a shrinking ensemble's cost per agent-step does."""

    def __init__(self, fast, drift=0.02):
        self.fast = fast
        self.drift = drift
        self.launch = (4, 4, 0, 0)
        self.steps = 0
        self.graphs_dropped = 0

    def shape(self):
        return (4, 4, 4, 4)

    def table_info(self):
        return 1_000_000, 20_000

    def set_launch(self, a, s, items=0, dense=0):
        self.launch = (a, s, items, dense)
        self.graphs_dropped += 1

    def step(self, n=1):
        self.steps += n

    def step_timed(self, n):
        t = 0.0
        for _ in range(n):
            base = 1.0 + self.drift * self.steps
            penalty = sum(0.05 * abs(x - y) for x, y in zip(self.launch, self.fast))
            t += base * (1.0 + penalty)
            self.steps += 1
        return t


def test_drift_correction_is_linear():
    c = Autotuner.drift_corrected([1.0, 3.0, 2.0, 2.0])
    assert abs(c[0] - 1.0) < 1e-12 and abs(c[-1] - 1.0) < 1e-12
    assert abs(c[1] - (3.0 - 1.0 / 3)) < 1e-12
    assert Autotuner.drift_corrected([5.0]) == [5.0]


def test_tuner_finds_the_fastest_launch_under_drift():
    # the fastest launch is found although every later trial runs on a
    # costlier batch (without the correction, the first trials would win)
    for fast in [(3, 3, 2, 48), (4, 3, 1, 12), (2, 4, 0, 24)]:
        b = DriftingBatch(fast)
        t = Autotuner(trial_steps=2, span=3)
        got = t.tune(b)
        want_dense = fast[3] if fast[3] in t.dense_choices else 24
        assert got[:3] == fast[:3] and (got[3] or 24) == want_dense, (fast, got, t.trials)
        assert b.launch == got
        # a known bucket is only set again
        steps = b.steps
        assert t.tune(b) == got and b.steps == steps


def test_incumbent_timed_in_every_stage():
    b = DriftingBatch((4, 4, 0, 0), drift=0.0)
    t = Autotuner(trial_steps=1, span=2)
    got = t.tune(b)
    assert got[:3] == (4, 4, 0)
    tried = [c for c, _ in t.trials[Autotuner.bucket(*b.table_info())]]
    # the scan stage compared its candidates with the default width (0)
    assert (4, 4, 0, 0) in tried and (4, 4, 1, 0) in tried and (4, 4, 2, 0) in tried
