"""Golden vectors for the time-series statistics of ccp-analyze (the
reference's Program/src/sostat.cu): seeded series are fed to
oracle/_ref/sostat_driver (built from the reference sources by
oracle/ref/build_sostat.sh, host code only) and its printed lines are
stored with the inputs in tests/golden/sostat.json.

Series: an exponential relaxation (thermalisation) followed by AR(1)
noise, lengths 8 .. 1200, one to five simulations per case.
Usage: python tests/golden/make_sostat_golden.py
"""
import json
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DRIVER = os.path.join(HERE, "..", "..", "oracle", "_ref", "sostat_driver")


def series(rng, n):
    x = np.empty(n)
    a = rng.uniform(0.0, 0.95)
    x[0] = rng.normal()
    for i in range(1, n):
        x[i] = a * x[i - 1] + rng.normal()
    tau = rng.uniform(1.0, 0.3 * n)
    drift = rng.uniform(-5, 5) * np.exp(-np.arange(n) / tau)
    return (rng.uniform(-2, 10) + rng.uniform(0.01, 3) * x + drift).astype(np.float32)


def main():
    rng = np.random.default_rng(20251203)
    cases = []
    for k in range(30):
        n_sims = int(rng.integers(1, 6))
        sims = [series(rng, int(rng.integers(8, 1200))) for _ in range(n_sims)]
        text = "%d\n" % n_sims + "".join(
            "%d %s\n" % (len(s), " ".join("%.9g" % v for v in s)) for s in sims)
        out = subprocess.run([DRIVER], input=text, capture_output=True, text=True, check=True).stdout
        cases.append({"series": [[float("%.9g" % v) for v in s] for s in sims], "lines": out.splitlines()})
    with open(os.path.join(HERE, "sostat.json"), "w") as f:
        json.dump(cases, f)
    print("wrote %d cases" % len(cases))


if __name__ == "__main__":
    main()
