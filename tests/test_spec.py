"""Execution order and draw windows of an action set."""
from qhg4_gb300.spec import (ACT_GETOLD, ACT_OLDAGEDEATH, ACT_RANDOMMOVE, ACT_RANDOMPAIR, ACT_VERHULST,
                             ACT_WEIGHTEDMOVE, Action, config1_actions, draw_windows, execution_order)


def test_priority_then_name():
    acts = [Action(ACT_RANDOMMOVE, 5), Action(ACT_GETOLD, 5), Action(ACT_RANDOMPAIR, 1)]
    assert [a.type for a in execution_order(acts)] == [ACT_RANDOMPAIR, ACT_GETOLD, ACT_RANDOMMOVE]


def test_windows():
    order = execution_order(config1_actions())
    assert draw_windows(order) == [0, 0, 0, 2, 4]
    acts = [Action(ACT_OLDAGEDEATH, 1), Action(ACT_VERHULST, 2), Action(ACT_WEIGHTEDMOVE, 3)]
    assert draw_windows(execution_order(acts)) == [0, 1, 3]
