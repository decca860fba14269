"""Generate the committed golden fixtures under tests/golden/.

1. reference_kats.json — the known-answer tests that the reference's own test
   suite holds for the paths built here, read as TEXT from the reference sources:
     * test/stiffness_test.cpp: the four TEST(stiffness, ...) lines
       (lattice side, U, beta, f-configuration, expected Drude stiffness,
       tolerance 1e-3 absolute from the obs_err line);
     * test/fast_update_test.cpp: the logZ identity case (L, U, T, seed,
       relative tolerance 1e-15) and the Chebyshev evaluator's moment_f
       checks with their tolerances;
     * test/binning_test.cpp: the data series, the expected binning
       statistics of depths 0..3 and correlation lengths (tolerance 1e-5);
     * test/jackknife_test.cpp: the two data series and the expected
       jackknife statistics, in the order the test checks them.
2. oracle_cases.json — small calc_ed and Metropolis-chain outputs of the CPU
   oracle (oracle/fk_oracle.cpp), used as fixed vectors by the GPU parity tests
   so they also compare against committed numbers, not only a live oracle.

Run from the repository root:  python tests/golden/make_golden.py <reference_root>
where <reference_root> is the root of the fk_mc reference sources (the
directory that holds test/stiffness_test.cpp); the argument is required.
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def reference_kats(ref_root):
    src = open(os.path.join(ref_root, "test", "stiffness_test.cpp")).read()
    pat = re.compile(r"TEST\(stiffness,\s*(\w+)\)\s*\{\s*test_stiffness\(([-\d.eE+]+),\s*([-\d.eE+]+),\s*\{([\d,\s]+)\},\s*([-\d.eE+]+)\)")
    tol = float(re.search(r"obs_err\s*=\s*([-\d.eE+]+)", src).group(1))
    t = float(re.search(r"double t\s*=\s*([-\d.eE+]+)", src).group(1))
    cases = []
    for name, U, beta, fs, val in pat.findall(src):
        f = [int(x) for x in fs.replace(" ", "").split(",") if x]
        L = int(round(len(f) ** 0.5))
        cases.append({"name": name, "L": L, "t": t, "U": float(U), "beta": float(beta), "f": f,
                      "stiffness": float(val), "tol": tol})
    fu = open(os.path.join(ref_root, "test", "fast_update_test.cpp")).read()
    g = lambda name: re.search(r"%s\s*=\s*([-\d.eE+]+);" % name, fu).group(1)
    logz = {"L": int(g(r"size_t L")), "U": float(g(r"double U")), "T": float(g(r"double T")),
            "seed": int(re.search(r"RNG\((\d+)\)", fu).group(1)),
            "rel_tol": float(re.search(r"/ logZ\) > ([-\d.eE+]+)\), false\);\s*\}", fu).group(1))}
    return {"source": "aeantipov/fk_mc test/stiffness_test.cpp, test/fast_update_test.cpp, "
                      "test/binning_test.cpp, test/jackknife_test.cpp",
            "stiffness": cases, "logz_identity": logz, "chebyshev": chebyshev_kats(fu),
            "binning": binning_kats(ref_root), "jackknife": jackknife_kats(ref_root)}


NUM = r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?"


def _vector(src, name):
    body = re.search(r"std::vector<double>\s+%s\s*=\s*\{([^}]*)\}" % name, src).group(1)
    return [float(x) for x in re.findall(NUM, body)]


def _tuples(src):
    return [[float(x) for x in re.findall(NUM, t)] for t in re.findall(r"std::make_tuple\(([^)]*)\)", src)]


def chebyshev_kats(fu):
    # ASSERT_NEAR(ch.moment_f([](double x){return <expr>;}, <order>), <value>, <tol>);
    pat = re.compile(r"ASSERT_NEAR\(ch\.moment_f\(\[\]\(double x\)\{return ([^;]*);\},(\d+)\),\s*(%s),\s*(%s)\)"
                     % (NUM, NUM))
    L = int(re.search(r"size_t L\s*=\s*(\d+);", fu).group(1))
    checks = [{"f": f.strip(), "order": int(o), "value": float(v), "tol": float(t)} for f, o, v, t in pat.findall(fu)]
    # cheb_size = int(log(msize))*2 (+ parity), grid points = cheb_size (fast_update_test.cpp:52-56)
    return {"L": L, "msize": L * L, "checks": checks}


def binning_kats(ref_root):
    src = open(os.path.join(ref_root, "test", "binning_test.cpp")).read()
    a = _vector(src, "a")
    stats = _tuples(src)
    cor = [float(x) for x in re.findall(NUM, re.search(r"correct_cor_lens\(\{([^}]*)\}\)", src).group(1))]
    return {"a": a, "max_depth": len(stats) - 1, "stats": stats, "cor_lens": cor, "tol": 1e-5}


def jackknife_kats(ref_root):
    src = open(os.path.join(ref_root, "test", "jackknife_test.cpp")).read()
    a, b = _vector(src, "a"), _vector(src, "b")
    t = _tuples(src)
    # the order of the checks in the test: the identity function of a at
    # depths 0, 1, 2; e2 - de2 - e^2 of (a, a^2, b) at depths 0, 1, 2; the
    # identity at depth 3 of accumulate_jackknife
    what = [("mean", 0), ("mean", 1), ("mean", 2), ("cv_unit", 0), ("cv_unit", 1), ("cv_unit", 2), ("mean", 3)]
    return {"a": a, "b": b, "tol": 1e-5,
            "cases": [{"func": f, "depth": d, "stats": st} for (f, d), st in zip(what, t)]}


def oracle_cases():
    from oracle import oracle as O
    rng = np.random.default_rng(34788)
    cases = []
    for kind, L, U, beta in [("cubic2d", 4, 1.0, 1.0), ("cubic2d", 8, 1.0, 1.0), ("triangular", 6, 2.0, 5.0),
                             ("cubic3d", 3, 2.0, 5.0), ("cubic1d", 12, 4.0, 10.0)]:
        n = L ** (3 if kind == "cubic3d" else 1 if kind == "cubic1d" else 2)
        f = rng.integers(0, 2, n).astype(np.int32)
        r = O.calc_ed(kind, L, f, beta, U, U / 2)
        cases.append({"kind": kind, "L": L, "U": U, "mu_c": U / 2, "beta": beta, "t": 1.0, "f": f.tolist(),
                      "spectrum": r["spectrum"].tolist(), "logZ": r["logZ"]})
    mc = O.mc_run("cubic2d", 8, beta=1.0, U=1.0, mu_c=0.5, mu_f=0.5, seed=34788, nsweeps=20, sweep_len=64)
    chain = {"kind": "cubic2d", "L": 8, "beta": 1.0, "U": 1.0, "mu_c": 0.5, "mu_f": 0.5, "seed": 34788,
             "nsweeps": 20, "sweep_len": 64, "ntherm_sweeps": 0, "mc_add_remove": 1.0,
             "site": mc["site"].tolist(), "accepted": mc["accepted"].tolist(), "weight": mc["weight"].tolist(),
             "energy": mc["energy"].tolist(), "f_final": mc["f_final"].tolist()}
    return {"generator": "oracle/fk_oracle.cpp via tests/golden/make_golden.py", "calc_ed": cases,
            "chain": chain}


if __name__ == "__main__":
    # usage: python tests/golden/make_golden.py <root of the fk_mc reference sources>
    if len(sys.argv) != 2 or not os.path.isdir(sys.argv[1]):
        sys.exit("usage: make_golden.py <root of the fk_mc reference sources (holds test/stiffness_test.cpp)>")
    with open(os.path.join(HERE, "reference_kats.json"), "w") as fh:
        json.dump(reference_kats(sys.argv[1]), fh, indent=1)
    with open(os.path.join(HERE, "oracle_cases.json"), "w") as fh:
        json.dump(oracle_cases(), fh)
    print("ok")
