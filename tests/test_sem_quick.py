"""The adaptive stop test's FP32 screen (cpd_model.h, sem_quick) decides like the exact
128-bit test (sem_test) wherever it decides: tests/semtest_check.cpp compiled here with
g++ over simulated Welford states and states built at the test's boundary. Exact
agreement is required (the stop round is a decision, like a bin)."""
import os
import subprocess

from conftest import PKG_DIR, ROOT


def test_sem_quick_agrees_with_exact_test(tmp_path):
    exe = tmp_path / "semtest_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-I",
                    os.path.join(PKG_DIR, "csrc"), "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "semtest_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), "40000"], capture_output=True, text=True, check=True).stdout.split()
    r = dict(zip(out[0::2], map(int, out[1::2])))
    assert r["disagreements"] == 0, r
    assert r["boundary_cases"] > 10000, r
    assert r["decided"] > 0.4 * r["cases"], r  # the screen settles most states
