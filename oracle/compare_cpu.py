"""Speed of the C port oracle (oracle/qhg_oracle.c) against the reference's
own OpenMP code built from its sources (oracle/_ref/qhg_ref_well:
SPopulation, the action classes, WELL512, LBController free lists), on the
same inputs and the same number of host threads.

TEST / MEASUREMENT INFRASTRUCTURE ONLY.  bench.py's CPU legs time the port,
because the reference sources (and so qhg_ref_well) exist only where the
reference tree is; this script measures how the two compare there.  Both
time the step loop only (the reference harness times PopLooper's span,
the port its qo_step calls).

  python oracle/compare_cpu.py [--threads N] [--out FILE]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import port  # noqa: E402
from oracle.refsim_io import ref_program, run_reference  # noqa: E402
from qhg4_gb300 import configs  # noqa: E402


def cases():
    return [
        ("plain method (n=32, 100k agents), 100 steps", configs.plain_method(), 100),
        ("large run's actions, n=128 altitude grid, 2M agents, 10 steps",
         configs.single_large_run(agents=2_000_000, n=128), 10),
        ("genetics run's actions, n=64, K=40, 400k agents with 2x4096-locus genomes, 5 steps",
         configs.genetics_run(agents=400_000, n=64), 5),
    ]


def time_port(w, steps, threads):
    port.set_threads(threads)
    o = port.OracleRun(w.grid, w.actions, w.seed, w.genetics, log_births=False)
    o.load(w.agents)
    t0 = time.perf_counter()
    st = o.step(steps)
    dt = time.perf_counter() - t0
    agent_steps = len(w.agents) + int(st[:-1, 0].sum())
    o.close()
    return agent_steps / dt, agent_steps, dt


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--out", default="")
    args = ap.parse_args()
    if not os.path.exists(ref_program("well")):
        sys.exit("the reference build oracle/_ref/qhg_ref_well is not present (make -C oracle/ref)")
    rows = []
    with tempfile.TemporaryDirectory() as tmp:
        for name, w, steps in cases():
            ref = run_reference("well", tmp, w.grid, w.agents, w.actions, steps, w.seed, w.genetics,
                                threads=args.threads)
            ref_v = ref.agent_steps / ref.seconds
            port_v, as_p, dt_p = time_port(w, steps, args.threads)
            rows.append({"case": name, "threads": args.threads, "reference_agent_steps_per_s": ref_v,
                         "reference_s": ref.seconds, "port_agent_steps_per_s": port_v, "port_s": dt_p,
                         "port_over_reference": port_v / ref_v})
            print(json.dumps(rows[-1]), flush=True)
    if args.out:
        with open(args.out, "w") as f:
            json.dump(rows, f, indent=1)


if __name__ == "__main__":
    main()
