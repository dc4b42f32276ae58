"""The benchmark's reference arm runs the reference's CPU path (the oracle)
on inputs from the numpy generators, without loading the CUDA library, and
those generators reproduce the library's own, value for value."""
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_loads_no_cuda_library(tmp_path):
    code = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--n', '17', '--steps', '2', "
            "'--warmup', '1']; runpy.run_path('bench.py', run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); print('LIBAGB' if 'libagb' in maps else 'NO_LIBAGB'); "
            "print('LIBORACLE' if 'liboracle' in maps else 'NO_LIBORACLE')")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = r.stdout.strip().splitlines()
    line = json.loads(lines[-3])
    assert lines[-2] == "NO_LIBAGB" and lines[-1] == "LIBORACLE"
    # whole solves within the arm's time budget: at least one, at most --steps
    assert line["impl"] == "reference" and 1 <= line["steps"] <= 2 and line["warmup"] == 1
    assert line["steps"] == len(line["cpu_baseline"]["solves"])
    assert line["config"]["nodes"] == 17 ** 3
    assert all(s["f_cycles"] >= 1 for s in line["cpu_baseline"]["solves"])


def test_numpy_generators_match_the_library(agb):
    from alamo_gb300 import synth
    from alamo_gb300 import workloads as W
    C1, dx1, g1 = synth.voronoi_cubic(21, 64, seed=1, with_grain=True)
    C2, dx2, g2 = W.voronoi_cubic(21, 64, seed=1, with_grain=True)
    assert dx1 == dx2 and np.array_equal(g1, g2) and np.array_equal(C1, C2)
    a, b = synth.inclusion_iso(17), W.inclusion_iso(17)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    a, b = synth.spheres_diffuse(33, 200, seed=3), W.spheres_diffuse(33, 200, seed=3)
    assert a[3] == b[3]
    assert np.abs(a[0] - b[0]).max() <= 1e-13 and np.abs(a[1] - b[1]).max() <= 1e-15
    r = W.Rng(11)
    assert np.array_equal(synth.uniform(11, (50,)), [r.uniform(-1.0, 1.0) for _ in range(50)])
