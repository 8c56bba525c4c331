"""The CP2K surface takes the precision of a new task list from the
environment (GRID_GB300_PRECISION, GRID_GB300_MIXED_THRESHOLD), so that an
unmodified CP2K can run the mixed mode; bad values stop the process with a
message."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CODE = (
    "from cp2k_gb300 import grid as G, workload as W\n"
    "inp = W.config('c1_64atoms', scale=0.1, seed=2)\n"
    "tl = G.GridTaskList(inp, precision=None, schedule=None, api='cp2k')\n"
    "print('PREC', G.lib().grid_gb300_get_precision(tl.impl), flush=True)\n"
    "print('SPLIT', *tl.mixed_split(), flush=True)\n"
    "tl.close()\n")


def _run(env_extra):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, "-c", CODE], cwd=ROOT, env=env, capture_output=True,
                          text=True, timeout=300)


def test_default_is_fp64():
    env = {k: v for k, v in os.environ.items() if not k.startswith("GRID_GB300_")}
    r = subprocess.run([sys.executable, "-c", CODE], cwd=ROOT, env=env, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "PREC 0" in r.stdout


@pytest.mark.parametrize("value,expect", [("mixed", 1), ("fp32", 2), ("FP64", 0)])
def test_precision_from_environment(value, expect):
    r = _run({"GRID_GB300_PRECISION": value})
    assert r.returncode == 0, r.stderr
    assert f"PREC {expect}" in r.stdout


def test_threshold_from_environment():
    lo = _run({"GRID_GB300_PRECISION": "mixed", "GRID_GB300_MIXED_THRESHOLD": "0"})
    hi = _run({"GRID_GB300_PRECISION": "mixed", "GRID_GB300_MIXED_THRESHOLD": "1e30"})
    assert lo.returncode == 0 and hi.returncode == 0
    f_lo = float(lo.stdout.split("SPLIT")[1].split()[0])
    f_hi = float(hi.stdout.split("SPLIT")[1].split()[0])
    assert f_lo == 0.0 and f_hi == 1.0


@pytest.mark.parametrize("key,value", [("GRID_GB300_PRECISION", "fp16"),
                                       ("GRID_GB300_MIXED_THRESHOLD", "-1")])
def test_bad_values_stop_the_process(key, value):
    r = _run({"GRID_GB300_PRECISION": "mixed", key: value} if key != "GRID_GB300_PRECISION"
             else {key: value})
    assert r.returncode != 0
    assert key in r.stderr
