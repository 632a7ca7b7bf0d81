"""Action set of a population, in the reference's vocabulary.

A population's step runs its actions in priority order (lower value first),
ties broken alphabetically by the action's name, which is how
``SPopulation::setPrioList`` fills the ``Prioritizer`` from a
``std::map<std::string,int>`` (core/SPopulation.cpp:251-261,
core/Prioritizer.h:20-78).  The action type codes and parameter slots are the
ones ``include/qhg_gpu.h`` declares.

Each action that draws random numbers owns a window of consecutive draws in
the per-agent Philox stream of a step: windows are handed out in execution
order, Verhulst/VerhulstVarK 2 draws (LinearBirth then LinearDeath,
actions/Verhulst.cpp:101-115), RandomMove 2 (actions/RandomMove.cpp:73-84),
WeightedMove 2 (actions/WeightedMove.cpp:57-71), OldAgeDeath 1
(actions/OldAgeDeath.cpp:57), ATanDeath 1 (actions/ATanDeath.cpp:66).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Sequence

ACT_GETOLD = 0
ACT_FERTILITY = 1
ACT_RANDOMPAIR = 2
ACT_VERHULST = 3
ACT_VERHULSTVARK = 4
ACT_OLDAGEDEATH = 5
ACT_RANDOMMOVE = 6
ACT_WEIGHTEDMOVE = 7
ACT_ATANDEATH = 8

#: reference class names (actions/*.h ATTR_*_NAME); Verhulst with a constant K
#: runs through VerhulstVarK in the reference oracle build, and no action name
#: sorts between the two, so tie-breaking is unaffected.
ACTION_NAMES = {
    ACT_GETOLD: "GetOld",
    ACT_FERTILITY: "Fertility",
    ACT_RANDOMPAIR: "RandomPair",
    ACT_VERHULST: "Verhulst",
    ACT_VERHULSTVARK: "VerhulstVarK",
    ACT_OLDAGEDEATH: "OldAgeDeath",
    ACT_RANDOMMOVE: "RandomMove",
    ACT_WEIGHTEDMOVE: "WeightedMove",
    ACT_ATANDEATH: "ATanDeath",
}

#: draws per agent per step an action may take
ACTION_DRAWS = {
    ACT_VERHULST: 2,
    ACT_VERHULSTVARK: 2,
    ACT_RANDOMMOVE: 2,
    ACT_WEIGHTEDMOVE: 2,
    ACT_OLDAGEDEATH: 1,
    ACT_ATANDEATH: 1,
}

#: number of crossovers per parent drawn from Poisson(1) (an extension; the
#: reference's Genetics_num_crossover is a fixed count)
CROSSOVER_POISSON1 = -100

MAX_ACTIONS = 16


@dataclass
class Action:
    """One action of a population with its parameters (4 slots).

    Parameter slots, by type:
      Fertility      (min_age, max_age, interbirth)
      Verhulst       (b0, d0, theta, K)
      VerhulstVarK   (b0, d0, theta)           K per cell from the grid
      OldAgeDeath    (max_age, uncertainty)
      ATanDeath      (max_age, range, slope)
      RandomMove     (prob)
      WeightedMove   (prob)                    weights from the grid's K
    """

    type: int
    prio: int
    p: Sequence[float] = field(default_factory=lambda: (0.0, 0.0, 0.0, 0.0))

    def params4(self) -> List[float]:
        v = list(self.p) + [0.0] * 4
        return [float(x) for x in v[:4]]


@dataclass
class Genetics:
    """Genetics of a population: loci per strand, crossovers per parent
    (fixed count > 0, 0 = none, CROSSOVER_POISSON1 = Poisson(1)) and the
    per-locus mutation rate (actions/Genetics.h ATTR_GENETICS_*)."""

    genome_size: int = 0
    num_crossover: int = 0
    mutation_rate: float = 0.0

    @property
    def num_blocks(self) -> int:
        return (self.genome_size + 63) // 64 if self.genome_size > 0 else 0


def execution_order(actions: Sequence[Action]) -> List[Action]:
    """Actions in the order a step executes them."""
    return sorted(actions, key=lambda a: (int(a.prio), ACTION_NAMES[a.type]))


def spec_digest(actions: Sequence[Action], genetics: Genetics = Genetics()) -> str:
    """A digest of what a run's draws and decisions depend on besides its
    seed: the actions in execution order with their parameters, and the
    genetics.  Checkpoints carry it, so that a resume with other settings is
    refused instead of silently diverging."""
    import hashlib
    parts = [f"{a.type}:{ACTION_NAMES[a.type]}:" + ",".join(repr(x) for x in a.params4())
             for a in execution_order(actions)]
    parts.append(f"genetics:{genetics.genome_size}:{genetics.num_crossover}:{genetics.mutation_rate!r}")
    return hashlib.sha256(";".join(parts).encode()).hexdigest()


def draw_windows(ordered: Sequence[Action]) -> List[int]:
    """First draw index of each action's window in the per-agent stream."""
    out, w = [], 0
    for a in ordered:
        out.append(w)
        w += ACTION_DRAWS.get(a.type, 0)
    return out


def config1_actions(b0=0.2, d0=0.05, theta=0.01, K=30.0, move_p=0.1,
                    fert_min=15.0, fert_max=45.0, interbirth=2.0) -> List[Action]:
    """The action set of the plain method: GetOld, Fertility, RandomPair,
    Verhulst and RandomMove, with the priorities of the tutorial population
    (tutorial_data/xmldat/tut_Sexual.xml: Fertility 2, RandomPair 3,
    Verhulst 6, RandomMove 7, GetOld 8)."""
    return [
        Action(ACT_FERTILITY, 2, (fert_min, fert_max, interbirth)),
        Action(ACT_RANDOMPAIR, 3),
        Action(ACT_VERHULST, 6, (b0, d0, theta, K)),
        Action(ACT_RANDOMMOVE, 7, (move_p,)),
        Action(ACT_GETOLD, 8),
    ]


def config2_actions(b0=0.5, d0=0.02, theta=0.01, move_p=0.2, max_age=64.0,
                    uncertainty=5.0 / 64.0, fert_min=15.0, fert_max=45.0,
                    interbirth=2.0) -> List[Action]:
    """Single large run: GetOld, Fertility, RandomPair, VerhulstVarK (per-cell
    K), OldAgeDeath (onset uniform in [60,70): max age 64, uncertainty 5/64)
    and WeightedMove.  The run's Verhulst rates are not fixed by its
    description; b0=0.5, d0=0.02, theta=0.01 keep a 20M population placed in
    proportion to K near its equilibrium (the plain method's b0=0.2, d0=0.05
    let it decay to a quarter within ~100 steps, because only paired fertile
    females give birth)."""
    return [
        Action(ACT_FERTILITY, 2, (fert_min, fert_max, interbirth)),
        Action(ACT_RANDOMPAIR, 3),
        Action(ACT_VERHULSTVARK, 6, (b0, d0, theta)),
        Action(ACT_WEIGHTEDMOVE, 7, (move_p,)),
        Action(ACT_GETOLD, 8),
        Action(ACT_OLDAGEDEATH, 10, (max_age, uncertainty)),
    ]


def config3_actions(b0=0.2, d0=0.05, theta=0.01, K=40.0, move_p=0.1,
                    fert_min=15.0, fert_max=45.0, interbirth=2.0) -> List[Action]:
    """Genetics run: the plain action set with K=40."""
    return config1_actions(b0=b0, d0=d0, theta=theta, K=K, move_p=move_p,
                           fert_min=fert_min, fert_max=fert_max, interbirth=interbirth)
