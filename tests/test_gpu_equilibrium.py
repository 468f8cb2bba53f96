"""Noise on: equilibrium averages against the oracle.  24 independent runs of
the 76-bead chain (T 0.6, the reference's integrator and neighbor-list
cadence) on the engine, batched, and 24 on the oracle, each side with its own
noise streams (different seeds).  After 2,000 steps, 20 samples 100 steps
apart give each run's mean total energy (rna_etot), Rg^2 and native-contact
fraction Q; the run means are the independent samples.  For each quantity
the engine's and the oracle's averages agree within two standard errors of
their difference."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from sop_gb300 import systems as S
from sop_gb300.engine import Engine, make_params

pytestmark = pytest.mark.gpu

RUNS, EQUIL, SAMPLES, GAP = 24, 2000, 20, 100
SCRIPT = [("set", "zeta", "50"), ("set", "t_step", "0.05"), ("set", "temp", "0.6"),
          ("set", "nstep", "1000"), ("set", "nup", "1000"), ("set", "cutofftype", "neighborlist"),
          ("set", "nnlup", "10"), ("set", "boxl", "500"), ("set", "ncell", "62.5"), ("set", "run", "1")]
NAMES = ("total energy", "Rg^2", "Q")


def engine_means(system):
    out = np.zeros((RUNS, SAMPLES, 3))
    with Engine(0, max_beads=1 << 14, max_replicas=RUNS + 4, max_list_entries=1 << 21) as e:
        ids = [e.add(system, make_params(SCRIPT, seed=9100 + k)) for k in range(RUNS)]
        e.run(EQUIL)
        for s in range(SAMPLES):
            e.run(GAP)
            for k, r in enumerate(ids):
                out[k, s] = (e.energy(r)[5], e.observables(r)[2], e.observables(r)[0])
        assert all(e.status(r)[0] == 0 for r in ids)
    return out.mean(1)


def oracle_means(system):
    ports = []
    for k in range(RUNS):
        p = O.Port()
        p.set_system(system)
        for _, key, v in SCRIPT:
            p.command(key, v)
        p.set_param("seed", 5100 + k)
        p.set_force_terms(1, 1, 1, 1)
        p.setup(True)
        ports.append(p)
    threads = os.cpu_count() or 1
    O.run_many(ports, EQUIL, threads)
    out = np.zeros((RUNS, SAMPLES, 3))
    for s in range(SAMPLES):
        O.run_many(ports, GAP, threads)
        for k, p in enumerate(ports):
            p.energy_eval()
            p.observables()
            out[k, s] = (p.energy("rna_etot"), p.energy("rgsq"), p.energy("Q"))
    return out.mean(1)


def test_equilibrium_energy_rg_q_match_oracle():
    system = S.synth_chain(3076, 76)
    g = engine_means(system)
    c = oracle_means(system)
    for q, name in enumerate(NAMES):
        diff = g[:, q].mean() - c[:, q].mean()
        se = np.sqrt(g[:, q].var(ddof=1) / RUNS + c[:, q].var(ddof=1) / RUNS)
        print("%s: engine %.6g, oracle %.6g, difference %.3g, standard error %.3g"
              % (name, g[:, q].mean(), c[:, q].mean(), diff, se))
        assert se > 0, name  # the runs are independent, so they differ
        assert abs(diff) < 2.0 * se, (name, g[:, q].mean(), c[:, q].mean(), se)
