"""FP64 precision mode (sop_params.precision = SOP_PREC_FP64): the step in
double precision with the reference's force formulas, as the drift and
force-error reference for the mixed-precision path.

Tolerances: against the CPU oracle (FP64 restatement of the reference)
forces and energies within 1e-10 relative and a 1,000-step noise-off
trajectory within 1e-8 A RMSD (the remaining differences are the 2^-40
fixed-point rounding of each contribution and the summation order); pair
lists bit-exact; an FP64 replica inside a mixed batch is bit-identical to
the same replica alone."""
import numpy as np
import pytest

from oracle import oracle as O
from sop_gb300 import _lib as L
from sop_gb300 import systems as S
from sop_gb300.engine import Engine, make_params

pytestmark = pytest.mark.gpu

DET = L.TERM_FENE | L.TERM_ANGLE | L.TERM_VDW
F64_TOL, E64_TOL, RMSD64_TOL = 1e-10, 1e-10, 1e-8


def script(mode="neighborlist"):
    return [("set", "zeta", "50"), ("set", "t_step", "0.05"), ("set", "temp", "0.6"),
            ("set", "nstep", "1000"), ("set", "nup", "1000"), ("set", "cutofftype", mode),
            ("set", "nnlup", "10"), ("set", "boxl", "500"), ("set", "ncell", "62.5"),
            ("set", "run", "1")]


def port_for(system, scr):
    p = O.Port()
    p.set_system(system)
    for _, k, v in scr:
        p.command(k, v)
    p.set_force_terms(0, 1, 1, 1)
    return p


def pairset(ii, jj):
    a = np.stack([np.minimum(ii, jj), np.maximum(ii, jj)], 1)
    return a[np.lexsort((a[:, 1], a[:, 0]))]


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def rmsd(a, b):
    return float(np.sqrt(((np.asarray(a) - np.asarray(b)) ** 2).sum(1).mean()))


@pytest.fixture(scope="module")
def eng():
    e = Engine(0, max_beads=1 << 16, max_replicas=32, max_list_entries=1 << 23)
    yield e
    e.close()


@pytest.mark.parametrize("n", [76, 300, 1500])
def test_fp64_forces_energies(eng, n):
    system = S.synth_chain(9100 + n, n)
    r = eng.add(system, make_params(script(), force_terms=DET, precision=L.PREC_FP64))
    m = eng.add(system, make_params(script(), force_terms=DET))
    try:
        port = port_for(system, script())
        port.setup(True)
        f64 = eng.force(r)
        assert rel(f64, port.coords(3)) < F64_TOL
        # the mixed-precision force against the FP64 one, same positions
        assert rel(eng.force(m), f64) < 1e-5
        e = eng.energy(r)
        for k, name in enumerate(O.ENERGY_NAMES):
            want = port.energy(name)
            assert abs(e[k] - want) <= E64_TOL * max(abs(want), 1e-3), (name, e[k], want)
    finally:
        eng.remove(r)
        eng.remove(m)


@pytest.mark.parametrize("n,mode", [(300, "neighborlist"), (600, "celllist")])
def test_fp64_noise_off_trajectory(eng, n, mode):
    system = S.synth_chain(9200 + n, n)
    r = eng.add(system, make_params(script(mode), force_terms=DET, precision=L.PREC_FP64))
    try:
        port = port_for(system, script(mode))
        port.setup(True)
        eng.run_plain(r, 1000)
        port.run(1000)
        _, x, v = eng.state(r)
        assert rmsd(x, port.coords(1)) < RMSD64_TOL
        assert rel(v, port.coords(2)) < 1e-7
        for k in range(4):
            np.testing.assert_array_equal(pairset(*eng.pairs(r, k)), pairset(*port.pairs(k)))
    finally:
        eng.remove(r)


def test_fp64_replica_in_mixed_batch(eng):
    sizes = [50, 700, 1500, 120]
    systems = [S.synth_chain(9300 + k, n) for k, n in enumerate(sizes)]
    params = [make_params(script(), seed=930 + k, list_mode="skin" if k % 2 else "neighborlist",
                          precision=L.PREC_FP64 if k in (1, 3) else L.PREC_MIXED)
              for k in range(len(sizes))]
    alone = []
    for s, p in zip(systems, params):
        r = eng.add(s, p)
        eng.run(150)
        alone.append(eng.state(r)[1])
        eng.remove(r)
    ids = [eng.add(s, p) for s, p in zip(systems, params)]
    eng.run(150)
    for k, r in enumerate(ids):
        np.testing.assert_array_equal(eng.state(r)[1], alone[k])
        assert eng.status(r)[0] == 0
    for r in ids:
        eng.remove(r)


def typed_chain(seed, n, frac):
    xyz = L.synth_chain(seed, n)
    types = np.where(np.random.default_rng(seed + 1).random(n) < 0.4, 2, 1).astype(np.int32)
    return S.with_exclusions(S.system_from_xyz(xyz, bead_type=types), frac, seed + 2)


@pytest.mark.parametrize("n", [150, 600])
def test_fp64_typed_partial_candidates(eng, n):
    """Bead types 1/2 and a vdw file that leaves out a quarter of the
    non-native candidates, FP64 mode: forces and energies within 1e-10, a
    1,000-step noise-off trajectory within 1e-8 A, with the pulling term on."""
    system = typed_chain(9400 + n, n, 0.25)
    kw = dict(pull_force=0.2, pull_i=0, pull_j=-1)
    r = eng.add(system, make_params(script(), force_terms=DET, precision=L.PREC_FP64, **kw))
    try:
        port = port_for(system, script())
        for k, v in kw.items():
            port.set_param(k, v)
        port.setup(True)
        assert rel(eng.force(r), port.coords(3)) < F64_TOL
        e = eng.energy(r)
        for k, name in enumerate(O.ENERGY_NAMES):
            want = port.energy(name)
            assert abs(e[k] - want) <= E64_TOL * max(abs(want), 1e-3), (name, e[k], want)
        eng.run_plain(r, 1000)
        port.run(1000)
        assert rmsd(eng.state(r)[1], port.coords(1)) < RMSD64_TOL
        for k in range(4):
            np.testing.assert_array_equal(pairset(*eng.pairs(r, k)), pairset(*port.pairs(k)))
    finally:
        eng.remove(r)
