"""The integer forms of the R^k store (csrc/bs2e_dmul.h) equal the FP64
operations they replace, bit for bit: compiled for the host with g++, the
product is checked against the IEEE 754 multiply on 40 million products
(random significands over the whole normal exponent range, few-bit
significands whose products fall exactly halfway between two doubles, and
the inputs that fall back to the FP64 multiply), and the FP32-pair split of
the mixed store against its FP64 conversions on 30 million values (random,
few-bit and far below the scale, where the low word leaves the normal float
range)."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_dmul_int_equals_ieee_multiply(tmp_path):
    exe = tmp_path / "dmul_check"
    src = os.path.join(ROOT, "tests", "native", "dmul_check.cpp")
    r = subprocess.run([os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-ffp-contract=off",
                        src, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), "20000000"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 mismatches" in r.stdout
