"""The batch autotuner's search without a GPU (host logic of pf_tune.cu):
coordinate descent over the three shape axes from the default shape, two
passes, on a synthetic cost; it ends at the axis-wise optimum after a bounded
number of measurements, then answers the class from its table; finished
classes are written to PFGPU_TUNE_CACHE and read back by a fresh process."""
import ctypes as C
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
AXES = ((1, 2, 4, 8, 16, 32, 64), (2, 4, 8, 16, 32, 64), (32, 64, 128, 256))


@pytest.fixture(scope="module")
def lib():
    from platelet_fiber_gpu_gb300 import build, gpu
    build.build()
    L = gpu.lib()
    L.pfgpu_tune_next_.argtypes = [C.c_char_p, C.POINTER(C.c_int)]
    L.pfgpu_tune_record_.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.c_float]
    return L


def cost(s):
    """Separable bowl with its minimum at (16, 4, 64)."""
    import math
    return 1.0 + (math.log2(s[0]) - 4) ** 2 + 0.5 * (math.log2(s[1]) - 2) ** 2 + 0.25 * (math.log2(s[2]) - 6) ** 2


def search(L, key, f):
    sh = (C.c_int * 3)()
    seen = []
    while L.pfgpu_tune_next_(key, sh):
        s = tuple(sh)
        assert s[0] in AXES[0] and s[1] in AXES[1] and s[2] in AXES[2]
        seen.append(s)
        L.pfgpu_tune_record_(key, sh, f(s))
        assert len(seen) < 100
    return tuple(sh), seen


def test_coordinate_descent_finds_the_bowl(lib):
    best, seen = search(lib, b"test.bowl", cost)
    assert best == (16, 4, 64)
    assert len(seen) == len(set(seen))          # nothing measured twice
    assert len(seen) <= sum(len(a) for a in AXES) * 2
    assert seen[0] == (1, 8, 128)               # first axis swept from the default
    # the class is answered from the table from now on
    best2, seen2 = search(lib, b"test.bowl", cost)
    assert best2 == best and not seen2


def test_failed_measurements_never_win(lib):
    bad = lambda s: float("nan") if s == (2, 8, 128) else cost(s)  # noqa: E731
    best, _ = search(lib, b"test.nan", bad)
    assert best == (16, 4, 64)


def test_cache_file_round_trip(tmp_path):
    cache = tmp_path / "tune.txt"
    code = (
        "import ctypes as C, sys\n"
        "sys.path.insert(0, %r)\n"
        "from platelet_fiber_gpu_gb300 import gpu\n"
        "L = gpu.lib()\n"
        "sh = (C.c_int * 3)()\n"
        "n = 0\n"
        "while L.pfgpu_tune_next_(b'test.cache', sh):\n"
        "    s = tuple(sh)\n"
        "    L.pfgpu_tune_record_(b'test.cache', sh, C.c_float(1.0 + abs(s[0] - 4) + abs(s[1] - 16) + abs(s[2] - 256) / 64))\n"
        "    n += 1\n"
        "print(list(sh), n)\n" % str(ROOT))
    env = dict(os.environ, PFGPU_TUNE_CACHE=str(cache))
    first = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, check=True)
    shape, n = first.stdout.split("]")
    assert json.loads(shape + "]") == [4, 16, 256] and int(n) > 0
    assert cache.read_text().split()[:4] == ["test.cache", "4", "16", "256"]
    again = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, check=True)
    assert again.stdout.split() == ["[4,", "16,", "256]", "0"]
