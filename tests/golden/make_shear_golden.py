"""Generate tests/golden/shear_golden.npz from the reference's own shear estimator.

The reference's shear.py (shear.py:1-148) is a Python 2 script that reads ellipticity tables
written by data_processing (columns flux | e1 | m_e1 | err1 | e2 | m_e2 | err2 | 1D var | SNR | l | m
with a header line), rejects bad measurements together with their opposite-orientation partner
(:58-89), estimates the shape noise (:91-113) and the shear as a weighted mean with an
astropy.stats bootstrap (:115-145).  This script runs it unmodified in its logic on fixed seeded
tables, in a temporary directory: its `print` statements are turned into calls and its integer
division `len(me1)/norient` into `//` (the only Python 3 incompatibilities), and astropy.stats
(not installed) is replaced by a bootstrap that returns the original sample bootnum times, so
that the printed bootstrap mean is the full-sample weighted mean and deterministic.  Stored: the
tables and the printed outputs (selected galaxies, bad count, shape noise, shear).

Usage:  python tests/golden/make_shear_golden.py [reference checkout, default $RLF_REFERENCE_DIR]
"""
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

STUB = '''import numpy as np
def bootstrap(data, bootnum=100, samples=None, bootfunc=None):
    return np.stack([np.asarray(data)] * bootnum)
'''


def table(seed, n_pairs, bad_rows, last_odd_bad=False):
    rng = np.random.default_rng(seed)
    n = 2 * n_pairs
    e = rng.uniform(0.05, 0.6, n_pairs)
    phi = rng.uniform(0, 2 * np.pi, n_pairs)
    e1 = np.repeat(e * np.cos(phi), 2) * np.tile([1, -1], n_pairs) + 0.02 + rng.normal(0, 0.05, n)
    e2 = np.repeat(e * np.sin(phi), 2) * np.tile([1, -1], n_pairs) - 0.01 + rng.normal(0, 0.05, n)
    err1 = rng.uniform(0.01, 0.2, n)
    err2 = rng.uniform(0.01, 0.2, n)
    var = rng.uniform(2e-5, 0.04, n)
    snr = rng.uniform(10.5, 200.0, n)
    flux = rng.uniform(10, 200, n)
    for r, kind in bad_rows:
        if kind == "var":
            var[r] = 5e-6
        elif kind == "err":
            err2[r] = 5e-4
        else:
            snr[r] = 7.0
    if last_odd_bad:
        snr[n - 1] = 3.0
    t = np.stack([flux, e1 + 0.0, e1, err1, e2 + 0.0, e2, err2, var, snr, rng.uniform(-1800, 1800, n),
                  rng.uniform(-1800, 1800, n)], 1)
    return np.round(t, 12)  # the values the %.12f table holds


def write(path, t):
    with open(path, "w") as f:
        f.write("flux | e1 | m_e1 | err1 | e2 | m_e2 | err2 | 1D var | SNR | l | m\n")
        for row in t:
            f.write(" | ".join("%.12f" % x for x in row) + " \n")


def run_reference(ref_dir, t):
    src = open(os.path.join(ref_dir, "shear.py")).read()
    src = re.sub(r"^(\s*)print (.*)$", r"\1print(\2)", src, flags=re.M)
    src = src.replace("ngal = len(me1)/norient", "ngal = len(me1)//norient")
    with tempfile.TemporaryDirectory() as d:
        os.makedirs(os.path.join(d, "astropy"))
        open(os.path.join(d, "astropy", "__init__.py"), "w").close()
        open(os.path.join(d, "astropy", "stats.py"), "w").write(STUB)
        open(os.path.join(d, "shear_py3.py"), "w").write(src)
        write(os.path.join(d, "ellipticities0.txt"), t)
        r = subprocess.run([sys.executable, "shear_py3.py", "-nf", "1"], cwd=d, capture_output=True, text=True,
                           check=True)
    out = r.stdout
    num = r"([-+0-9.eE]+)"
    g = lambda pat: [float(x) for x in re.search(pat, out).groups()]
    ngal, bad = g(r"ngal:\s+" + num + r"\s+bad:\s+" + num)
    sigma = g(r"shape noise:\s+" + num)[0]
    g1, s1 = g(r"e1_shear: mean =\s+" + num + r"\s+std =\s+" + num)
    g2, s2 = g(r"e2_shear: mean =\s+" + num + r"\s+std =\s+" + num)
    assert "ERROR" not in out, out
    return np.array([ngal, bad, sigma, g1, g2, s1, s2])


CASES = {
    "clean": dict(seed=1, n_pairs=200, bad_rows=[]),
    "bad_even_and_odd": dict(seed=2, n_pairs=200, bad_rows=[(0, "var"), (5, "err"), (10, "snr"), (11, "snr"),
                                                            (101, "var"), (222, "err"), (399, "snr")]),
    "last_odd_bad": dict(seed=3, n_pairs=150, bad_rows=[(7, "var"), (42, "snr")], last_odd_bad=True),
}


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("RLF_REFERENCE_DIR", "")
    if not os.path.isfile(os.path.join(ref, "shear.py")):
        raise SystemExit("give the reference checkout (argument or RLF_REFERENCE_DIR)")
    out = {}
    for name, kw in CASES.items():
        t = table(**kw)
        out[name + "_table"] = t
        out[name + "_out"] = run_reference(ref, t)
        print(name, out[name + "_out"])
    np.savez(os.path.join(HERE, "shear_golden.npz"), **out)


if __name__ == "__main__":
    main()
