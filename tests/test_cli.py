"""The drop-in CLIs convstencil_{1d,2d,3d}: command line, prompts, output lines."""
import os
import re
import subprocess

import pytest

import convstencil_gb300 as cs

BIN = os.path.join(os.path.dirname(cs.LIB_PATH))


@pytest.fixture(scope="module", autouse=True)
def built():
    cs.build()


def run(name, *args, stdin=None):
    return subprocess.run([os.path.join(BIN, name), *args], input=stdin, capture_output=True,
                          text=True, timeout=300)


@pytest.mark.parametrize("name,args", [("convstencil_1d", ["1d1r", "64"]),
                                       ("convstencil_2d", ["box2d3r", "64", "64"]),
                                       ("convstencil_3d", ["box3d1r", "8", "8", "8"])])
def test_usage_and_bad_arguments(name, args):
    r = run(name, *args)              # too few arguments -> help, exit 1
    assert r.returncode == 1 and "Usage:" in r.stdout
    r = run(name, "nosuchshape", *args, "3")
    assert r.returncode == 1 and "Usage:" in r.stdout
    r = run(name, *(args[:1] + ["x"] + args[2:]), "3")
    assert r.returncode == 1 and "cannot convert" in r.stderr


GPU_CASES = [
    ("convstencil_1d", ["1d1r", "4096", "3"], None, r"INFO: shape = 1d1r,  n = 4096, times = 3"),
    ("convstencil_1d", ["1d2r", "4096", "3", "--custom"], "0.1 0.2 0.4 0.2 0.1\n",
     r"Please enter 5 parameters:"),
    ("convstencil_2d", ["star2d1r", "96", "128", "4", "--custom"], "0.2 0.2 0.2 0.2 0.2\n",
     r"INFO: shape = star_2d1r, m = 96, n = 128, times = 4"),
    ("convstencil_2d", ["box2d3r", "100", "130", "2"], None, r"INFO: shape = box_2d3r, m = 100, n = 130"),
    ("convstencil_2d", ["star2d3r", "64", "64", "2", "--custom"], " ".join(["0.07"] * 13) + "\n",
     r"Please enter 13 parameters:"),
    ("convstencil_3d", ["box3d1r", "16", "16", "32", "2"], None, r"INFO: shape = box_3d1r, h = 16"),
    ("convstencil_3d", ["star3d1r", "16", "16", "32", "2", "--custom"], "0.1 0.1 0.1 0.4 0.1 0.1 0.1\n",
     r"INFO: shape = star_3d1r"),
]


@pytest.mark.gpu
@pytest.mark.parametrize("name,args,stdin,pattern", GPU_CASES)
def test_cli_runs(name, args, stdin, pattern):
    r = run(name, *args, stdin=stdin)
    assert r.returncode == 0, r.stdout + r.stderr
    assert re.search(pattern, r.stdout), r.stdout
    assert re.search(r"Time = \d+\[ms\]", r.stdout)
    g = float(re.search(r"GStencil/s = ([0-9.eE+-]+)", r.stdout).group(1))
    assert g > 0
