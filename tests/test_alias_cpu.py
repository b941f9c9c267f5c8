"""Math::AliasMethod of the C++ API (Math/AliasMethod.h:26-105), under the reference's
own test (TestPetrichor/Math/TestAliasMethod.cpp:16-94): 1000 random 10-bin
distributions, 1M samples each from the reference's xor128 streams; the reference's
statistic must stay under its bound 2.09, and the count-based chi-square (9 degrees of
freedom) under 45 (p < 1e-6 for any one distribution)."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_alias_method_chi_square(tmp_path):
    exe = str(tmp_path / "alias_client")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "alias_client.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe, "1000", "1000000"], capture_output=True, text=True, check=True,
                         timeout=300).stdout.split()
    stat, chi2 = float(out[0]), float(out[1])
    assert stat <= 2.09
    assert chi2 < 45.0
