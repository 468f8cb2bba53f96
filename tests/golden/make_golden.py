"""Generate the golden vectors in tests/golden/ from the SOP-CPU reference.

Runs the unmodified reference, built by oracle/Makefile into oracle/_ref
(libsopref.so for in-process calls through oracle/ref_harness.cpp, and sop.x
for end-to-end runs of its own driver), on seeded synthetic chains written in
the reference's file formats, and stores inputs and outputs as .npz files:

  system      xyz, bonds, angles, natives (what the vdw/bonds/angles/init files hold)
  params      integrator constants after the script's set commands
  nl_*, pl_*  neighbor and pair lists (1-based pairs, reference order) at set-up
  f_*         forces at set-up per term (random term off) and all terms
  e0          energies at set-up (e_bnd, e_ang_ss, e_vdw_rr, att, rep, rna_etot)
  traj_*      state, energies, observables after 100 noise-free iterations
  cell_*      cell-list mode lists at set-up
  sd_update   sop.x update.out rows of a T=0 (steepest-descent) run
  sd_unc      its final unccoord.out coordinates
  sd_traj*    its traj.bin / traj_uncorrected.bin frames (initial + every nup)

sop_golden_N*.npz hold type-1 chains whose vdw file lists every candidate.
sop_golden_types_N*.npz hold a chain with a seeded mix of bead types 1 and 2
(sigma 3.8 / 5.4 / 7.0, rcut_nat 8 / 11 / 14 A, the type-dependent native
coefficients: global.cpp:60-92) whose vdw file leaves out a seeded quarter of
the non-native candidates (those pairs never interact, params.cpp:186-232);
they add bead_type and the left-out pairs (ie, je, 0-based).

    make -C oracle ref && python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "sop-cpu_gb300"))

from oracle.oracle import REF_EXE, Ref  # noqa: E402
from sop_gb300 import systems as S  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
SIZES = [(1030, 30), (1076, 76), (1150, 150)]
TYPED = [(1250, 150)]
NSTEPS = 100


def typed_system(seed, n):
    """A chain with a seeded mix of bead types (about 40% type 2) whose vdw
    file leaves out a seeded quarter of the non-native candidates."""
    xyz = S._lib.synth_chain(seed, n)
    types = np.where(np.random.default_rng(seed + 1).random(n) < 0.4, 2, 1).astype(np.int32)
    return S.with_exclusions(S.system_from_xyz(xyz, bead_type=types), 0.25, seed + 2)


def script(mode="neighborlist", temp="0.6", nstep=NSTEPS, nup=50):
    return [("set", "zeta", "50"), ("set", "t_step", "0.05"), ("set", "temp", temp),
            ("set", "nstep", str(nstep)), ("set", "nup", str(nup)),
            ("set", "cutofftype", mode), ("set", "nnlup", "10"), ("set", "boxl", "500"),
            ("set", "ncell", "62.5"), ("set", "run", "1")]


def lists(ref):
    out = {}
    for k, name in enumerate(("nl_att", "nl_rep", "pl_att", "pl_rep")):
        ii, jj = ref.pairs(k)
        out[name] = np.stack([ii, jj], 1).astype(np.int32)
    return out


def one(seed, n, typed=False):
    system = typed_system(seed, n) if typed else S.synth_chain(seed, n)
    rec = dict(xyz=system.xyz, ib=system.bonds[0], jb=system.bonds[1], r0=system.bonds[2],
               ia=system.angles[0], ja=system.angles[1], ka=system.angles[2], a0=system.angles[3],
               in_=system.natives[0], jn=system.natives[1], rn=system.natives[2])
    if typed:
        rec.update(bead_type=system.bead_type, ie=system.exclusions[0], je=system.exclusions[1])
    ref = Ref()
    with tempfile.TemporaryDirectory() as d:
        path = S.write_reference_files(system, d, script(), run=False)
        cwd = os.getcwd()
        os.chdir(d)
        try:
            ref.load_script(path)
            rec["params"] = np.array([ref.param(k) for k in ("T", "zeta", "h", "a1", "a2", "a3", "a4")])
            ref.set_force_terms(0, 1, 1, 1)
            ref.setup(True)
            rec.update(lists(ref))
            rec["e0"] = ref.energies()
            rec["f_all"] = ref.coords(3)
            for name, terms in (("f_fene", (0, 1, 0, 0)), ("f_ang", (0, 0, 1, 0)), ("f_vdw", (0, 0, 0, 1))):
                ref.set_force_terms(*terms)
                ref.force_eval()
                rec[name] = ref.coords(3)
            ref.set_force_terms(0, 1, 1, 1)
            ref.force_eval()
            ref.run(NSTEPS)
            ref.energy_eval()
            ref.observables()
            rec["traj_unc"] = ref.coords(1)
            rec["traj_vel"] = ref.coords(2)
            rec["traj_e"] = ref.energies()
            rec["traj_obs"] = np.array([ref.energy("Q"), ref.count("contct_nat"), ref.energy("rgsq"),
                                        ref.energy("kinT")])
            for k, v in lists(ref).items():
                rec["traj_" + k] = v
            # cell-list mode (cell_list.cpp) at the initial positions
            ref.load_script(S.write_reference_files(system, d, script("celllist"), run=False))
            ref.setup(False)
            for k, v in lists(ref).items():
                rec["cell_" + k] = v
        finally:
            os.chdir(cwd)
        # the reference program itself, T = 0 steepest descent (sop.cpp:316)
        sd = S.write_reference_files(system, d, script(temp="0.0", nstep=100, nup=50), run=True)
        subprocess.run([REF_EXE, sd], cwd=d, check=True, capture_output=True)
        rows = [list(map(float, l.split())) for l in open(os.path.join(d, "update.out"))]
        rec["sd_update"] = np.array(rows)
        rec["sd_unc"] = np.loadtxt(os.path.join(d, "unccoord.out"))[:, 1:]
        # record_traj's text frames (io.cpp:280-303): the start, then one per nup
        rec["sd_traj"] = np.loadtxt(os.path.join(d, "traj.bin"))
        rec["sd_traj_unc"] = np.loadtxt(os.path.join(d, "traj_uncorrected.bin"))
    name = ("sop_golden_types_N%d.npz" if typed else "sop_golden_N%d.npz") % n
    np.savez_compressed(os.path.join(OUT, name), **rec)
    print("wrote", name)


if __name__ == "__main__":
    for seed, n in SIZES:
        one(seed, n)
    for seed, n in TYPED:
        one(seed, n, typed=True)
