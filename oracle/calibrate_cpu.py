"""Test infrastructure: calibrate the CPU baseline (the oracle restatement) against the
reference's own OpenMP path on this host.

The GPU machine has no reference sources, so the bench's CPU arm there is the oracle
(oracle/gsph_oracle.cpp, OpenMP).  Where the reference sources are present, this script
ties that arm to the reference itself: it copies the sources to a scratch directory,
applies the recipe that lets GCC >= 9 compile their OpenMP clauses (`default(none)` ->
`default(shared)`, which leaves the semantics unchanged), builds the reference harness
with -fopenmp through oracle/Makefile.ref, and times the same KDK main-loop steps of the
same rotating cloud with both, on the same number of threads.

  python oracle/calibrate_cpu.py [n] [steps]      # defaults 131072 10
"""
from __future__ import annotations

import json
import os
import re
import shutil
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

REF = os.environ.get("GANDALF_SRC", "/root/reference")
SCRATCH = "/tmp/gandalf_openmp_src"
OUT = os.path.join(HERE, "_ref", "openmp")


def build() -> str:
    if not os.path.isdir(SCRATCH):
        shutil.copytree(REF, SCRATCH, ignore=shutil.ignore_patterns(".git"))
        for dirpath, _, files in os.walk(os.path.join(SCRATCH, "src")):
            for f in files:
                if f.endswith((".cpp", ".h", ".hpp")):
                    p = os.path.join(dirpath, f)
                    with open(p, errors="surrogateescape") as fh:
                        text = fh.read()
                    new = re.sub(r"default\(none\)", "default(shared)", text)
                    if new != text:
                        with open(p, "w", errors="surrogateescape") as fh:
                            fh.write(new)
    subprocess.run(["make", "-s", "-f", os.path.join(HERE, "Makefile.ref"), f"REF={SCRATCH}", f"OUT={OUT}",
                    "OMPFLAGS=-fopenmp", f"-j{os.cpu_count() or 4}"], check=True)
    return os.path.join(OUT, "gsph_ref_harness")


def main():
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 131072
    steps = int(sys.argv[2]) if len(sys.argv) > 2 else 10
    harness = build()
    from gandalf_gb300 import ics as ics_mod
    from oracle import oracle, refio
    c = ics_mod.rotating_cloud(n, seed=31)
    params = c.pop("params")
    kdk = c.pop("kdk")
    threads = os.cpu_count() or 1
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    work = "/tmp/gandalf_openmp_run"
    os.makedirs(work, exist_ok=True)
    inp = os.path.join(work, "input.bin")
    refio.write_input(inp, c, params, dict(kdk, nsteps=steps))
    t0 = time.perf_counter()
    subprocess.run([harness, inp, work], check=True, env=env, cwd=work, stdout=subprocess.DEVNULL)
    wall_ref = time.perf_counter() - t0
    timing = {}
    with open(os.path.join(work, "timing.txt")) as f:
        for line in f:
            k, v = line.split()
            timing[k] = float(v)
    r = oracle.kdk(c, params, kdk, steps, nthreads=threads)
    # the same discrete state: both ran the same main loop
    kb = refio._blocks(os.path.join(work, "kdk.bin"), "<f8")[0].reshape(n, len(refio.KDK_FIELDS))
    lv_ref = kb[:, refio.KDK_FIELDS.index("level")]
    same_levels = float(np.mean(lv_ref == r["state"]["level"]))
    out = {"n": n, "steps": steps, "threads": threads, "host": os.uname().machine,
           "reference_openmp": {"setup_s": timing["setup"], "steps_s": timing["kdk_steps"], "wall_s": wall_ref},
           "oracle": {"setup_s": r["setup_s"], "steps_s": r["steps_s"]},
           "steps_time_ratio_oracle_over_reference": r["steps_s"] / timing["kdk_steps"],
           "fraction_of_identical_levels": same_levels}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
