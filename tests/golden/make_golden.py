"""Regenerates tests/golden/*.npz from the reference nbots library.

Run where the nbots sources are (NBOTS_SRC in the environment, --nbots-src,
or oracle/Makefile.ref's default location):

    python tests/golden/make_golden.py [--nbots-src DIR]

It builds the unmodified reference library and the harness with
oracle/Makefile.ref (outputs under oracle/_ref/), writes each problem as a
problem file, runs ``ref_harness`` on it and stores the problem bytes plus
every dumped intermediate in one compressed npz per case.  The two T3 cases
come from nbots' own FEM unit-test flow (tessellated model files shipped
with the reference tests), so they carry the reference's known answers:
beam cantilever max |u| = 1.00701e-1 +- 1e-6, plate with a hole mean
von-Mises error < 9.7e-3.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)

from nbots_gb300 import problem_io as P  # noqa: E402
from nbots_gb300 import workloads as W  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")


def small_cases():
    cases = {}
    cases["c1_q4_64x32"] = W.config_c1()
    p = W.cantilever_q4(32, 16, top_traction=0.01, name="q4_lognormal_32x16")
    p.E = W.lognormal_E(p.n_elems, 0.5, seed=22)
    cases[p.name] = p

    # every bc form nbots has, self weight and disabled elements
    p = W.cantilever_q4(16, 8, jitter=0.15, seed=7, name="q4_allbc_16x8", E=3.0, nu=0.25,
                        thickness=0.5, top_traction=0.2)
    p.density = 1.5
    p.self_weight = True
    p.gravity = (0.3, -9.81)
    en = np.ones(p.n_elems, bool)
    en[[5, 17, 40, 41, 99]] = False
    p.enabled = en
    bottom = p.sgm[0]
    xs = p.nod[bottom, 0]
    p.bcs += [
        # function-valued Neumann on the bottom segment (values at its nodes)
        W.BC(W.NEUMANN, W.ON_SEGMENT, 0, (1, 1), (0.0, 0.0),
             node_vals=np.stack([0.1 * np.sin(xs), -0.05 * xs * xs], 1)),
        # function-valued Neumann on a vertex: nbots reads it at (0,0)
        W.BC(W.NEUMANN, W.ON_POINT, 3, (1, 0), (0.0, 0.0), node_vals=np.array([[0.125, 9.0]])),
        # prescribed, non-zero displacement at the top-right vertex
        W.BC(W.DIRICHLET, W.ON_POINT, 3, (0, 1), (0.0, -0.01)),
        # the bottom-left corner again (it is also on the clamped segment)
        W.BC(W.DIRICHLET, W.ON_POINT, 0, (1, 1), (0.0, 0.0)),
    ]
    cases[p.name] = p

    # the smallest cantilever: two elements, six nodes
    cases["q4_tiny_1x2"] = W.cantilever_q4(1, 2, name="q4_tiny_1x2")

    # a distorted element (detJ < 0): assembly must fail with status 1
    p = W.cantilever_q4(8, 4, name="q4_distorted_8x4")
    nid = 2 * 9 + 3
    p.nod[nid] = p.nod[nid + 9 + 1] + np.array([0.05, 0.02])
    cases[p.name] = p
    return cases


# nbots' damage solve (static_damage2D.c:239-470): name -> (problem source,
# ft, gf, N_steps, N_max_iter, N_max_iter_without_enhance, residual tol)
DAMAGE_CASES = {
    # converges in every step; no Gauss-Seidel fallback
    "dmg_q4_16x8": ("q4", 6.0, 10.0, 4, 40, 6, 1e-7),
    # every conjugate-gradient solve fails and falls back to Gauss-Seidel,
    # which fails too (the absolute tolerance 1e-8 is out of reach)
    "dmg_t3_beam150": ("beam150", 1e4, 10.0, 2, 30, 5, 1e-6),
    # edge settings: no iteration allowed, a cap of three iterations with a
    # break at the first residual that is not a new best, and no load step
    "dmg_q4_16x8_noiter": ("q4", 6.0, 10.0, 2, 0, 6, 1e-7),
    "dmg_q4_16x8_cap": ("q4", 6.0, 10.0, 3, 3, 1, 1e-7),
    "dmg_q4_16x8_nosteps": ("q4", 6.0, 10.0, 0, 5, 5, 1e-7),
    # self weight, function-valued loads, a prescribed displacement (the
    # q4_allbc_16x8 problem), below the damage threshold
    "dmg_q4_allbc": ("allbc", 100.0, 50.0, 3, 30, 5, 1e-7),
}


def damage_problem(src, tmp, a):
    if src == "allbc":
        path = os.path.join(tmp, "dmg_allbc.bin")
        P.write_problem(small_cases()["q4_allbc_16x8"], path)
        return path
    if src == "q4":
        p = W.cantilever_q4(16, 8, point_load=-0.5, name="dmg_q4_16x8")
        path = os.path.join(tmp, "dmg_q4.bin")
        P.write_problem(p, path)
        return path
    inputs = os.path.join(a.nbots_src, "utest/sources/nb/pde_bot/static_elasticity2D_inputs")
    path = os.path.join(tmp, "beam150.bin")
    run([HARNESS, "utest", os.path.join(inputs, "beam_cantilever.txt"), "150", path,
         os.path.join(tmp, "beam150.fem")])
    return path


def run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise SystemExit(f"{cmd} failed: {r.stderr}")


def save(name, prob_path, dump):
    with open(prob_path, "rb") as f:
        pb = np.frombuffer(f.read(), np.uint8)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), problem_bin=pb, **dump)
    print(name, {k: v.shape for k, v in dump.items()})


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--nbots-src", default=os.environ.get("NBOTS_SRC"),
                    help="nbots source tree (default: $NBOTS_SRC, else the build recipe's)")
    ap.add_argument("--only", nargs="*", help="regenerate these cases only")
    a = ap.parse_args()
    want = (lambda name: True) if not a.only else (lambda name: name in a.only)
    run(["make", "-s", "-C", ROOT, "-f", "oracle/Makefile.ref"] +
        ([f"NBOTS_SRC={a.nbots_src}"] if a.nbots_src else []) + ["-j8", "harness"])
    tmp = tempfile.mkdtemp()
    for name, p in small_cases().items():
        if not want(name):
            continue
        pb = os.path.join(tmp, name + ".bin")
        ob = os.path.join(tmp, name + ".out")
        P.write_problem(p, pb)
        run([HARNESS, "problem", pb, ob, "1"])
        save(name, pb, P.read_dump(ob))
    inputs = os.path.join(a.nbots_src, "utest/sources/nb/pde_bot/static_elasticity2D_inputs")
    for name, txt, extra in [("t3_beam_cantilever", "beam_cantilever.txt", []),
                             ("t3_plate_with_hole", "plate_with_hole.txt", ["pwh"])]:
        if not want(name):
            continue
        mb = os.path.join(tmp, name + ".bin")
        ob = os.path.join(tmp, name + ".fem")
        run([HARNESS, "utest", os.path.join(inputs, txt), "1000", mb, ob] + extra)
        fem = P.read_dump(ob)
        # then the staged dump of the same tessellated mesh
        ob2 = os.path.join(tmp, name + ".out")
        run([HARNESS, "problem", mb, ob2, "1"])
        d = P.read_dump(ob2)
        d.update({k: v for k, v in fem.items()})
        save(name, mb, d)
    for name, (src, ft, gf, steps, mi, mne, rtol) in DAMAGE_CASES.items():
        if not want(name):
            continue
        pb = damage_problem(src, tmp, a)
        ob = os.path.join(tmp, name + ".out")
        run([HARNESS, "damage", pb, ob, repr(ft), repr(gf), str(steps), str(mi), str(mne),
             repr(rtol)])
        d = P.read_dump(ob)
        d["damage_params"] = np.array([ft, gf, steps, mi, mne, rtol], np.float64)
        save(name, pb, d)


if __name__ == "__main__":
    main()
