"""The generator's restated random streams (csrc/gen_rng.h) against the C++
library's own std::mt19937, uniform_int_distribution,
uniform_real_distribution<float> and std::shuffle on this toolchain (GCC 13),
value for value, including the cases graph generation rarely meets: ranges
of 1, 2 and near 2^32 (where the bounded draw's rejection loop runs), draws
that round to 1.0 as floats, and shuffles on both sides of the paired-draw
threshold."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "dist_mem_gapbs_gb300", "csrc")


@pytest.fixture(scope="module")
def results(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    exe = str(tmp_path_factory.mktemp("rng") / "gen_rng_driver")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC,
                    os.path.join(ROOT, "tests", "gen_rng_driver.cc"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    return dict(line.split() for line in out.splitlines())


@pytest.mark.parametrize("check", ["raw", "bounded", "float", "shuffle", "float_clamped"])
def test_stream_matches_the_library(results, check):
    assert results[check] == "1"


def test_float_rounding_to_one_was_exercised(results):
    # one draw in 2^25 is one of the 128 values that round up to 2^32
    assert int(results["float_top_at"]) >= 0
