"""List rows in bands (sop_engine_config.row_bands).

The list build stores each row's far entries last: entries farther than the
pair cutoff plus a band width (half the skin; 0.35 sigma for the reference's
cadence lists) at the build.  While no bead of the replica has moved half the
band width since that build, such a pair cannot come within the pair cutoff,
so the step kernel leaves those entries out (their pair-list bits stay 0);
once some bead has, it scans whole rows until the next build.  Pair filtering
stays exact either way, so trajectories, exported pair lists, forces and
energies must be bit-identical with the bands on and off -- here over noisy
1,200-step runs in every list mode, with bead types 1/2 and left-out
candidates, and with a replica in minimum-image mode.
"""
import numpy as np
import pytest

from sop_gb300 import _lib as L
from sop_gb300 import systems as S
from sop_gb300.engine import Engine, make_params

pytestmark = pytest.mark.gpu


def script(mode="neighborlist", boxl="500", ncell="62.5"):
    return [("set", "zeta", "50"), ("set", "t_step", "0.05"), ("set", "temp", "0.8"),
            ("set", "nstep", "1000"), ("set", "nup", "1000"), ("set", "cutofftype", mode),
            ("set", "nnlup", "10"), ("set", "boxl", boxl), ("set", "ncell", ncell), ("set", "run", "1")]


def pairset(ii, jj):
    a = np.stack([np.minimum(ii, jj), np.maximum(ii, jj)], 1)
    return a[np.lexsort((a[:, 1], a[:, 0]))]


def cases():
    xyz = L.synth_chain(7601, 500)
    types = np.where(np.random.default_rng(7602).random(500) < 0.4, 2, 1).astype(np.int32)
    typed = S.with_exclusions(S.system_from_xyz(xyz, bead_type=types), 0.25, 7603)
    img = S.synth_chain(7604, 300)
    boxl = 1.1 * float((img.xyz.max(0) - img.xyz.min(0)).max())
    iscr = script(boxl="%.3f" % boxl, ncell="%.6f" % (boxl / 8.0))
    return [
        (S.synth_chain(7605, 1200), make_params(script(), seed=1)),
        (S.synth_chain(7606, 700), make_params(script("celllist"), seed=2)),
        (S.synth_chain(7607, 2600), make_params(script(), seed=3, list_mode="skin", skin=2.0)),
        (S.synth_chain(7608, 90), make_params(script(), seed=4, list_mode="skin", skin=4.0)),
        (typed, make_params(script(), seed=5, list_mode="skin", skin=3.0)),
        (img, make_params(iscr, seed=6)),
    ]


def test_bands_on_and_off_bit_identical():
    kw = dict(max_beads=1 << 15, max_replicas=16, max_list_entries=1 << 24)
    with Engine(0, **kw) as on, Engine(0, row_bands=-1, **kw) as off:
        runs = [(on.add(s, p), off.add(s, p)) for s, p in cases()]
        for _ in range(4):
            on.run(300)
            off.run(300)
            for a, b in runs:
                np.testing.assert_array_equal(on.state(a)[1], off.state(b)[1])
                for k in (1, 3):
                    np.testing.assert_array_equal(pairset(*on.pairs(a, k)), pairset(*off.pairs(b, k)))
                assert on.status(a)[0] == 0 and off.status(b)[0] == 0
        for a, b in runs:
            np.testing.assert_array_equal(on.force(a), off.force(b))
            np.testing.assert_array_equal(on.energy(a), off.energy(b))
