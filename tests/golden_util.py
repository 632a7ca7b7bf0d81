"""Loading of the golden fixtures (tests/golden/*.npz, made by
tests/golden/make_golden.py from the reference's own action code)."""
import glob
import os

import numpy as np

from qhg4_gb300.spec import Action, Genetics
from qhg4_gb300.workload import Agents, Grid

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_names():
    """Bit-exact fixtures (the ks_*.npz files hold KS-test samples instead)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz"))
                  if not os.path.basename(p).startswith("ks_"))


class Golden:
    def __init__(self, name: str):
        d = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
        self.name = name
        self.grid = Grid(0, d["nbr"], d["nnbr"], np.zeros((len(d["nnbr"]), 3)), d["K"])
        g = d["genetics"]
        self.genetics = Genetics(int(g[0]), int(g[1]), float(d["mutation_rate"][0]))
        self.agents = Agents(d["in_id"], d["in_cell"], d["in_birth"], d["in_age"], d["in_lastb"],
                             d["in_gender"], d["in_state"], d["in_genome"] if "in_genome" in d else None)
        self.actions = [Action(int(t), int(p), tuple(float(x) for x in prm))
                        for t, p, prm in zip(d["act_type"], d["act_prio"], d["act_param"])]
        self.steps = int(d["steps"][0])
        self.seed = int(d["seed"][0])
        self.expected = Agents(d["out_id"], d["out_cell"], d["out_birth"], d["out_age"], d["out_lastb"],
                               d["out_gender"], d["out_state"], d["out_genome"] if "out_genome" in d else None)
        self.stats = d["stats"]
        self.births = d["births"]
